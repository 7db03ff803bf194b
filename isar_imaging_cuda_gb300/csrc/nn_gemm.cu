// BF16 GEMM on the 5th-generation tensor cores (tcgen05, TMEM accumulators):
//   C[Mr][Nc] (+)= A[Mr][K] * B[Nc][K]^T,  A, B bf16 row-major (K contiguous),
//   C fp32 row-major.
// The dense layers of the learned autofocus warm start (forward, data and
// weight gradients) are all of this form.
//
// One CTA of 128 threads computes a 128 x BN tile over a K range (split-K:
// blockIdx.z; partial tiles are added into C with atomics).  Per 64-wide K
// block the CTA stages A (128 x 64) and B (BN x 64) in shared memory in the
// canonical K-major, no-swizzle layout (8 x 16-byte core matrices: LBO =
// 128 B between K-adjacent core matrices, SBO = 1024 B between 8-row groups),
// one elected thread issues four tcgen05.mma (M = 128, N = BN, K = 16) into a
// TMEM accumulator and commits them to an mbarrier; the CTA waits on the
// mbarrier (bounded) before it overwrites the stage.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows).
// Every wait is bounded: a timeout sets *err, and the CTA frees its TMEM and
// returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "isar_kernels.h"

namespace isar {
namespace nn {

constexpr int BM = 128;
constexpr int BK = 64;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, LBO, SBO (bytes, >> 4), version 1
// (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
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

template <int BN>
__global__ void __launch_bounds__(128, 1)
k_gemm_tn(const __nv_bfloat16* __restrict__ A, int lda, const __nv_bfloat16* __restrict__ B, int ldb,
          float* __restrict__ Cm, int ldc, int Mr, int Nc, int K, int klen, int atomic_out, int* err)
{
    static_assert(BN == 16 || BN == 32 || BN == 64 || BN == 128, "tile N");
    constexpr int TCOLS = BN < 32 ? 32 : BN;
    __shared__ __align__(1024) uint8_t sa[BM * BK * 2];
    __shared__ __align__(1024) uint8_t sb[BN * BK * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
    const int k_beg = blockIdx.z * klen;
    const int k_end = min(K, k_beg + klen);
    const uint32_t bar_a = smem_u32(&bar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "n"(TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_fail = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = idesc_bf16(BM, BN);

    uint32_t phase = 0;
    int nblk = 0;
    for (int k0 = k_beg; k0 < k_end; k0 += BK, ++nblk) {
        // stage A: 128 rows x 8 chunks of 8 bf16; chunk (r, c) -> core matrix
        // (r / 8, c) at ((r / 8) * 8 + c) * 128 + (r % 8) * 16 bytes
        for (int i = tid; i < BM * 8; i += 128) {
            const int r = i >> 3, c = i & 7;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            const int gr = row0 + r, gk = k0 + c * 8;
            if (gr < Mr && gk < k_end) v = *reinterpret_cast<const uint4*>(A + (size_t)gr * lda + gk);
            *reinterpret_cast<uint4*>(sa + (((r >> 3) * 8 + c) << 7) + ((r & 7) << 4)) = v;
        }
        for (int i = tid; i < BN * 8; i += 128) {
            const int r = i >> 3, c = i & 7;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            const int gr = col0 + r, gk = k0 + c * 8;
            if (gr < Nc && gk < k_end) v = *reinterpret_cast<const uint4*>(B + (size_t)gr * ldb + gk);
            *reinterpret_cast<uint4*>(sb + (((r >> 3) * 8 + c) << 7) + ((r & 7) << 4)) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int s = 0; s < BK / 16; ++s) {
                const uint64_t ad = smem_desc(smem_u32(sa) + s * 256, 128, 1024);
                const uint64_t bd = smem_desc(smem_u32(sb) + s * 256, 128, 1024);
                const uint32_t acc = (nblk > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar_a)
                         : "memory");
        }
        if (!mbar_wait(bar_a, phase)) {
            atomicExch(err, 1);
            s_fail = 1;
        }
        phase ^= 1u;
        __syncthreads();
        if (s_fail) break;
    }

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
            if (r < Mr) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = col0 + c0 + j;
                    if (c < Nc) {
                        const float x = __uint_as_float(v[j]);
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

cudaError_t gemm_tn(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int Mr,
                    int Nc, int K, int splits, int* err, cudaStream_t st)
{
    if (Mr <= 0 || Nc <= 0 || K <= 0 || (K % 8) || (lda % 8) || (ldb % 8) || splits < 1) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return cudaErrorMisalignedAddress;
    int klen = (K + splits - 1) / splits;
    klen = (klen + BK - 1) / BK * BK;
    const int kz = (K + klen - 1) / klen;
    const int atomic_out = kz > 1 ? 1 : 0;
    const int bn = Nc <= 16 ? 16 : Nc <= 32 ? 32 : 64;
    dim3 grid((Mr + BM - 1) / BM, (Nc + bn - 1) / bn, kz);
    switch (bn) {
    case 16: k_gemm_tn<16><<<grid, 128, 0, st>>>(A, lda, B, ldb, C, ldc, Mr, Nc, K, klen, atomic_out, err); break;
    case 32: k_gemm_tn<32><<<grid, 128, 0, st>>>(A, lda, B, ldb, C, ldc, Mr, Nc, K, klen, atomic_out, err); break;
    default: k_gemm_tn<64><<<grid, 128, 0, st>>>(A, lda, B, ldb, C, ldc, Mr, Nc, K, klen, atomic_out, err); break;
    }
    ISAR_COUNT(1);
    return cudaGetLastError();
}

}  // namespace nn
}  // namespace isar
