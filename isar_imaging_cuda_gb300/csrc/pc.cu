// IFDS ingest: per-pulse matched-filter pulse compression, one CTA per pulse.
// Reference: pulseCompression::pulseCompressionbyFFT (common.cu:635-746) as
// multiThreadIFDS drives it (common.cu:583-604), then cutRangeProfile with a
// single row (common.cu:494-509).  The reference runs it pulse by pulse from 8
// host threads: per pulse a host->device copy, two memsets, two small kernels
// and a device synchronisation for the reference chirp, three cuFFT calls, an
// elementwise kernel, a cuBLAS scale, a cuBLAS Icamax with a device->host read
// and a gather kernel.  Here one launch compresses a whole batch of pulses:
// every CTA runs the three transforms of its pulse in shared memory (the
// echo's spectrum parked in a global scratch row between the first and the
// second transform), forms the chirp on the fly, finds the maximum and writes
// its 4096-cell cut.
#include <cuda_runtime.h>

#include "fft.cuh"
#include "isar_kernels.h"

namespace isar {

namespace {

// Chirp sample i < S of genRefPulseCompression / genTkPulseCompression /
// genHammingVec (common.cu:260-266, 620-660), the float expressions as the
// reference writes them, rounded operation by operation (no contraction):
//   tk = (1 - v2) (Tp/-2 + i Tp/(S-1)),  ph = (c1 + c2 tk) tk,
//   ref = hamming_S[i] (cos ph, sin ph).
__device__ __forceinline__ float2 pc_ref(int i, int S, float v2c, float c1, float c2, float tpf)
{
    const float ham =
        __fsub_rn(0.54f, __fmul_rn(0.46f, cosf(__fdiv_rn(__fmul_rn(__fmul_rn(2.0f, kPiF), (float)i), (float)(S - 1)))));
    const float tk = __fmul_rn(v2c, __fadd_rn(__fdiv_rn(tpf, -2.0f), __fdiv_rn(__fmul_rn((float)i, tpf),
                                                                               __fsub_rn((float)S, 1.0f))));
    const float ph = __fmul_rn(__fadd_rn(c1, __fmul_rn(c2, tk)), tk);
    float s, c;
    sincosf(ph, &s, &c);
    return make_float2(__fmul_rn(ham, c), __fmul_rn(ham, s));
}

}  // namespace

template <int NF>
__global__ void __launch_bounds__(NF / 16)
k_pulse_compress(PCArgs a)
{
    using F = FFTShape<NF>;
    extern __shared__ float4 dyn_smem[];
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    float2* twt = sm + F::SMEM;
    __shared__ float red_v[32];
    __shared__ int red_i[32];
    __shared__ int s_off;
    const int p = blockIdx.x, lt = threadIdx.x;
    TwShared<NF>::fill(twt, a.tw, lt, F::T);
    __syncthreads();
    const TwShared<NF> tws{twt};
    const int16_t* ad = a.ad + (size_t)p * a.ad_stride;
    float2* sp = a.spec + (size_t)p * NF;
    const int L = a.iq_len;

    // X = FFT(x): the int16 I/Q samples, zero-padded to NF
    team_fft<NF, false>(
        [&](int i) {
            if (i >= L) return make_float2(0.0f, 0.0f);
            const short2 q = reinterpret_cast<const short2*>(ad)[i];
            return make_float2((float)q.x, (float)q.y);
        },
        [&](int k, float2 v, int) { sp[k] = v; }, sm, lt, tws);

    // REF = FFT(ref); Y = conj(REF) .* X into the scratch (same thread wrote
    // sp[k] in the first transform: the output mapping of a size is fixed)
    const float v2 = __fdiv_rn(__fmul_rn(2.0f, (float)a.vel[p]), 300000000.0f);   // LIGHT_SPEED
    const float v2c = __fsub_rn(1.0f, v2);
    const float c1 = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(-2.0f, kPiF), a.fc_f), v2), v2c);
    team_fft<NF, false>(
        [&](int i) { return i < a.S ? pc_ref(i, a.S, v2c, c1, a.c2, a.tp_f) : make_float2(0.0f, 0.0f); },
        [&](int k, float2 r, int) { sm[fpad(k)] = cmulc(r, sp[k]); }, sm, lt, tws);

    // y = IFFT(Y) / NF, kept in the scratch; Icamax (|Re| + |Im|, first max)
    const float inv = 1.0f / (float)NF;
    float bv = -1.0f;
    int bi = 0x7fffffff;
    team_fft<NF, true>([&](int i) { return sm[fpad(i)]; },
                       [&](int i, float2 v, int) {
                           const float2 y = make_float2(v.x * inv, v.y * inv);
                           sm[fpad(i)] = y;
                           const float m = fabsf(y.x) + fabsf(y.y);
                           if (m > bv || (m == bv && i < bi)) {
                               bv = m;
                               bi = i;
                           }
                       },
                       sm, lt, tws);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) {
            bv = ov;
            bi = oi;
        }
    }
    if ((lt & 31) == 0) {
        red_v[lt >> 5] = bv;
        red_i[lt >> 5] = bi;
    }
    __syncthreads();
    if (lt == 0) {
        float v = red_v[0];
        int ii = red_i[0];
        for (int w = 1; w < F::T / 32; ++w)
            if (red_v[w] > v || (red_v[w] == v && red_i[w] < ii)) {
                v = red_v[w];
                ii = red_i[w];
            }
        int off = ii - kRangeNumIfdsPc / 2;
        if (off < 0) off = 0;
        if (off > NF - kRangeNumIfdsPc) off = NF - kRangeNumIfdsPc;
        s_off = off;
        if (a.offsets) a.offsets[p] = off;
    }
    __syncthreads();
    const int off = s_off;
    float2* o = a.out + (size_t)p * a.out_stride;
    for (int t = lt; t < kRangeNumIfdsPc; t += F::T) o[t] = sm[fpad(off + t)];
}

namespace {

template <int NF>
size_t pc_smem()
{
    return ((size_t)FFTShape<NF>::SMEM + TwShared<NF>::kEntries) * sizeof(float2);
}

template <int NF>
cudaError_t pc_launch(const PCArgs& a, cudaStream_t st)
{
    static PerDevice attr;   // shared-memory limit, set once per device
    const int ar = attr.get([]() -> int {
        return -(int)cudaFuncSetAttribute(k_pulse_compress<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)pc_smem<NF>());
    });
    if (ar < 0) return (cudaError_t)(-ar);
    k_pulse_compress<NF><<<a.pulses, NF / 16, pc_smem<NF>(), st>>>(a);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

}  // namespace

int pc_nfft(int iq_len)
{
    // nextPow2 (common.cu:521-529): 2^(floor(log2 n) + 1)
    int n = iq_len, r = 1;
    while (n >> 1) {
        r <<= 1;
        n >>= 1;
    }
    return r << 1;
}

cudaError_t pulse_compress(const PCArgs& a, cudaStream_t st)
{
    if (a.pulses <= 0) return cudaSuccess;
    switch (a.nfft) {
    case 4096: return pc_launch<4096>(a, st);
    case 8192: return pc_launch<8192>(a, st);
    case 16384: return pc_launch<16384>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace isar
