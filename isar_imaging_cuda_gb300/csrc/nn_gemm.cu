// BF16 GEMM on the 5th-generation tensor cores (tcgen05, TMEM accumulators):
//   C[Mr][Nc] (+)= A[Mr][K] * B[Nc][K]^T,  A, B bf16 row-major (K contiguous),
//   C fp32 row-major.
// The dense layers of the learned autofocus warm start (forward, data and
// weight gradients) are all of this form.
//
// One CTA of 128 threads computes a 128 x BN tile over a K range (split-K:
// blockIdx.z; partial tiles are added into C with atomics).  The operands
// stream through a ring of kStages shared-memory stages: per 64-wide K block
// the tensor memory accelerator copies A (128 x 64) and B (BN x 64) with the
// 128-byte swizzle (cp.async.bulk.tensor, rows and columns outside the
// matrices read as zero) and signals the stage's "full" mbarrier with the
// byte count; one elected thread waits on it, issues four tcgen05.mma
// (M = 128, N = BN, K = 16) into the TMEM accumulator and commits them to
// the stage's "empty" mbarrier, and refills the stage used one block earlier
// once its MMAs are done, so copies run kStages - 1 blocks ahead of the tensor
// pipe.  A final commit signals the epilogue, which reads the accumulator with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows).  Every wait is
// bounded: a timeout sets *err; the CTA then waits (bounded) for its copies
// and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "isar_kernels.h"
#include "nn.h"

namespace isar {
namespace nn {

constexpr int BM = 128;
constexpr int BK = 64;         // bf16 per swizzled row: 128 bytes
constexpr int kStages = 4;

template <int BN>
struct GemmSmem {
    static constexpr int kA = BM * BK * 2;   // A tile bytes (16 KB)
    static constexpr int kB = BN * BK * 2;   // B tile bytes
    static constexpr int kStage = kA + kB;
    // stages are 1024-byte aligned (the swizzle pattern's period); slack for
    // aligning the dynamic shared-memory base
    static constexpr size_t kBytes = 1024 + (size_t)kStages * kStage;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major tile written by the tensor
// memory accelerator with the 128-byte swizzle: start address (bytes >> 4),
// leading offset 16 B (unused for swizzled K-major tiles), stride 1024 B
// between 8-row groups, version 1 (bits 46-47), base offset 0 (the tile is
// 1024-byte aligned), layout SWIZZLE_128B (2 at bits 61-63).  A K step of 16
// elements inside the 128-byte row advances the start address by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46) | (2ull << 61);
}

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (unsigned i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void mbar_init(uint32_t bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
}

// One arrival that also expects `bytes` of copies on the barrier.
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Tiled 2-D copy of the box at (x = K element, y = row) into shared memory,
// completing `bar`'s transaction bytes.  x is a multiple of BK (128 bytes).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Tiled 3-D copy of the box at (x, y, z); y may lie partly outside the
// tensor (rows there read as zero).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
k_gemm_tn(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
          float* __restrict__ Cm, int ldc, int Mr, int Nc, int K, int klen, int atomic_out, int* err,
          const float* __restrict__ bias, __nv_bfloat16* __restrict__ out_bf16, int ld_bf16, int bias_cols,
          int conv_M, int conv_pad)
{
    static_assert(BN == 16 || BN == 32 || BN == 64, "tile N");
    using S = GemmSmem<BN>;
    constexpr int TCOLS = BN < 32 ? 32 : BN;
    extern __shared__ uint8_t gemm_smem[];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ __align__(8) uint64_t empty[kStages];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
    const int k_beg = blockIdx.z * klen;
    const int k_end = min(K, k_beg + klen);
    const int nblk = (k_end - k_beg + BK - 1) / BK;
    const uint32_t base = (smem_u32(gemm_smem) + 1023u) & ~1023u;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "n"(TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(smem_u32(&full[s]));
            mbar_init(smem_u32(&empty[s]));
        }
        mbar_init(smem_u32(&done));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
        s_fail = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = idesc_bf16(BM, BN);

    if (tid == 0) {
        auto load = [&](int b) {
            const int s = b % kStages;
            const uint32_t fb = smem_u32(&full[s]);
            const uint32_t sa = base + (uint32_t)(s * S::kStage);
            mbar_expect_tx(fb, (uint32_t)S::kStage);
            if (conv_M) {
                // implicit convolution: K block = tap, rows shifted by
                // tap - pad within the frame of this row block
                const int f = row0 / conv_M, m0 = row0 - f * conv_M;
                const int tap = k_beg / BK + b;
                tma_load_3d(sa, &map_a, 0, m0 + tap - conv_pad, f, fb);
            } else {
                tma_load_2d(sa, &map_a, k_beg + b * BK, row0, fb);
            }
            tma_load_2d(sa + S::kA, &map_b, k_beg + b * BK, col0, fb);
        };
        const int pre = min(kStages - 1, nblk);
        for (int b = 0; b < pre; ++b) load(b);
        int issued = pre, consumed = 0;
        bool ok = true;
        for (int kb = 0; kb < nblk; ++kb) {
            const int s = kb % kStages;
            if (!mbar_wait(smem_u32(&full[s]), (uint32_t)((kb / kStages) & 1))) {
                ok = false;
                break;
            }
            consumed = kb + 1;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = base + (uint32_t)(s * S::kStage);
#pragma unroll
            for (int j = 0; j < BK / 16; ++j) {
                const uint64_t ad = smem_desc_sw128(sa + 32 * j);
                const uint64_t bd = smem_desc_sw128(sa + S::kA + 32 * j);
                const uint32_t acc = (kb > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            umma_commit(smem_u32(&empty[s]));
            // refill the stage of block kb - 1 (its MMAs were issued a block
            // earlier, so the tensor pipe still holds block kb's)
            const int nb = kb + kStages - 1;
            if (nb < nblk) {
                if (nb >= kStages &&
                    !mbar_wait(smem_u32(&empty[nb % kStages]), (uint32_t)((nb / kStages - 1) & 1))) {
                    ok = false;
                    break;
                }
                load(nb);
                issued = nb + 1;
            }
        }
        if (!ok) {
            atomicExch(err, 1);
            s_fail = 1;
            // the copies in flight land before the stages are released
            for (int b = consumed; b < issued; ++b)
                (void)mbar_wait(smem_u32(&full[b % kStages]), (uint32_t)((b / kStages) & 1));
        }
        // arrives once every MMA issued above has completed
        umma_commit(smem_u32(&done));
    }
    __syncthreads();
    if (!mbar_wait(smem_u32(&done), 0u)) {
        atomicExch(err, 1);
        s_fail = 1;
    }
    __syncthreads();

    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (!s_fail && nblk > 0) {
        const int r = row0 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (r < Mr && out_bf16) {
                // bf16(max(C + bias, 0)): a hidden layer's activation
                const int cb = col0 + c0;
                if (cb + 16 <= Nc) {
                    uint32_t pk[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const float a0 = __uint_as_float(v[2 * j]) + __ldg(&bias[cb + 2 * j]);
                        const float a1 = __uint_as_float(v[2 * j + 1]) + __ldg(&bias[cb + 2 * j + 1]);
                        const __nv_bfloat162 h = __floats2bfloat162_rn(a0 > 0.0f ? a0 : 0.0f, a1 > 0.0f ? a1 : 0.0f);
                        pk[j] = *reinterpret_cast<const uint32_t*>(&h);
                    }
                    uint4* dst = reinterpret_cast<uint4*>(out_bf16 + (size_t)r * ld_bf16 + cb);
                    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int c = cb + j;
                        if (c < Nc) {
                            const float a = __uint_as_float(v[j]) + __ldg(&bias[c]);
                            out_bf16[(size_t)r * ld_bf16 + c] = __float2bfloat16_rn(a > 0.0f ? a : 0.0f);
                        }
                    }
                }
            } else if (r < Mr) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = col0 + c0 + j;
                    if (c < Nc) {
                        float x = __uint_as_float(v[j]);
                        if (c < bias_cols) x += __ldg(&bias[c]);
                        if (atomic_out) atomicAdd(&Cm[(size_t)r * ldc + c], x);
                        else Cm[(size_t)r * ldc + c] = x;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(TCOLS) : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when the driver does not provide it.
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Tensor map of a row-major bf16 matrix [rows][k] with leading dimension ld
// (elements), boxes of box_rows x BK with the 128-byte swizzle; elements
// outside [rows) x [k) read as zero.
static cudaError_t operand_map(CUtensorMap* m, const __nv_bfloat16* p, int rows, int k, int ld, int box_rows)
{
    const PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(__nv_bfloat16)};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(p), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Tensor map of act [frames][M][64] bf16 in boxes of 64 x 128 x 1 with the
// 128-byte swizzle (the implicit convolution's A operand).
static cudaError_t conv_map(CUtensorMap* m, const __nv_bfloat16* act, int frames, int M)
{
    const PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[3] = {(cuuint64_t)BK, (cuuint64_t)M, (cuuint64_t)frames};
    const cuuint64_t strides[2] = {(cuuint64_t)BK * sizeof(__nv_bfloat16),
                                   (cuuint64_t)M * BK * sizeof(__nv_bfloat16)};
    const cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)BM, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(act), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int BN>
static cudaError_t launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, dim3 grid, float* C, int ldc, int Mr,
                               int Nc, int K, int klen, int atomic_out, int* err, cudaStream_t st,
                               const GemmEpilogue& ep, const GemmConvA& conv)
{
    static PerDevice attr;   // the stage ring's dynamic shared-memory limit, once per device
    const int a = attr.get([] {
        return cudaFuncSetAttribute(k_gemm_tn<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)GemmSmem<BN>::kBytes) == cudaSuccess
                   ? 1
                   : -1;
    });
    if (a < 0) return cudaErrorInvalidConfiguration;
    k_gemm_tn<BN><<<grid, 128, GemmSmem<BN>::kBytes, st>>>(ma, mb, C, ldc, Mr, Nc, K, klen, atomic_out, err, ep.bias,
                                                          ep.out_bf16, ep.ld_bf16, ep.bias ? ep.bias_cols : 0,
                                                          conv.act ? conv.M : 0, conv.pad);
    return cudaSuccess;
}

cudaError_t gemm_tn(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int Mr,
                    int Nc, int K, int splits, int* err, cudaStream_t st, const GemmEpilogue& ep,
                    const GemmConvA& conv)
{
    if (conv.act) {
        // row blocks stay inside one frame; the taps are whole K blocks
        if (conv.M <= 0 || (conv.M % BM) || conv.frames <= 0 || (long)conv.frames * conv.M != Mr || (K % BK) ||
            conv.pad < 0 || splits != 1 || (reinterpret_cast<uintptr_t>(conv.act) & 15))
            return cudaErrorInvalidValue;
        A = conv.act;   // alignment checks below; the map is 3-D
        lda = K;
    }
    if (Mr <= 0 || Nc <= 0 || K <= 0 || (K % 8) || (lda % 8) || (ldb % 8) || lda < K || ldb < K || splits < 1)
        return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return cudaErrorMisalignedAddress;
    // the epilogues need whole sums (no split-K); the bf16 output is stored
    // 16 bytes at a time, C is not written
    if ((ep.out_bf16 || ep.bias) && splits != 1) return cudaErrorInvalidValue;
    if (ep.out_bf16 && (!ep.bias || ep.ld_bf16 < Nc || (ep.ld_bf16 % 8) ||
                        (reinterpret_cast<uintptr_t>(ep.out_bf16) & 15)))
        return cudaErrorInvalidValue;
    if (!ep.out_bf16 && !C) return cudaErrorInvalidValue;
    // split boundaries are multiples of BK, so every copy starts at a K
    // offset of a multiple of 128 bytes and no block crosses into the next
    // split's range (only the last split's last block reaches past K: zeros)
    int klen = (K + splits - 1) / splits;
    klen = (klen + BK - 1) / BK * BK;
    const int kz = (K + klen - 1) / klen;
    const int atomic_out = kz > 1 ? 1 : 0;
    const int bn = Nc <= 16 ? 16 : Nc <= 32 ? 32 : 64;
    CUtensorMap ma, mb;
    cudaError_t e;
    if (conv.act) {
        if ((e = conv_map(&ma, conv.act, conv.frames, conv.M))) return e;
    } else if ((e = operand_map(&ma, A, Mr, K, lda, BM))) {
        return e;
    }
    if ((e = operand_map(&mb, B, Nc, K, ldb, bn))) return e;
    dim3 grid((Mr + BM - 1) / BM, (Nc + bn - 1) / bn, kz);
    switch (bn) {
    case 16: e = launch_gemm<16>(ma, mb, grid, C, ldc, Mr, Nc, K, klen, atomic_out, err, st, ep, conv); break;
    case 32: e = launch_gemm<32>(ma, mb, grid, C, ldc, Mr, Nc, K, klen, atomic_out, err, st, ep, conv); break;
    default: e = launch_gemm<64>(ma, mb, grid, C, ldc, Mr, Nc, K, klen, atomic_out, err, st, ep, conv); break;
    }
    if (e) return e;
    ISAR_COUNT(1);
    return cudaGetLastError();
}

}  // namespace nn
}  // namespace isar
