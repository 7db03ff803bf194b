// Range alignment (with fused high-speed compensation), HRRP centering and
// range cut.  Reference: range_alignment.cu:4-78 (rangeAlignmentParallel),
// high_speed_compensation.cu:4-54, range_alignment.cu:371-465 (HRRPCenter),
// common.cu:494-518 (cutRangeProfile).
//
// Formulation.  The reference keeps the data x[m,n] (range spectra) in HBM and,
// at every level of its binary merge, IFFTs all M rows, forms group RMS
// envelopes, correlates neighbouring groups and multiplies the second group
// by a linear phase ramp.  Here x is never rewritten: every row carries a
// cumulative shift S_m (cells) and a high-speed-compensation coefficient, and
// each load applies window * exp(j*2*pi*(alpha_m*n^2 - S_m*n/N)) on the fly
// (64-bit fixed-point phase, exact modulo one cycle).  Two ways to form the
// group envelopes (isar_tuning.ra_rows_each_level):
//  - spectral merge (default): every group carries the 2N-point spectrum of
//    its half-cell power envelope, which a shift multiplies by a phase ramp
//    and a merge adds (k_ra_spec0, k_ra_spec): 4M + 3 (M/2 - 1) + M
//    transforms of N points per frame;
//  - carried envelopes: rows of the first half of a group are unchanged
//    since the previous level, so their envelope is carried over ("left"
//    vector) and only the rows shifted by the previous level are transformed
//    again (k_ra_pair, k_ra_accum, k_ra_corr): (log2 M - 1) * M/2 + 2M row
//    transforms plus 2 (M - 1) correlation transforms.
// The reference transforms all rows at every level: (log2 M + 1) * M row
// transforms plus 3 (M - 1) correlation transforms.
#include <cuda_runtime.h>

#include <type_traits>

#include "fft.cuh"
#include "isar_kernels.h"

namespace isar {

__device__ __forceinline__ int64_t frac_to_fixed(double f)
{
    f -= floor(f + 0.5);   // [-0.5, 0.5)
    return (int64_t)llrint(ldexp(f, 64));
}

__device__ __forceinline__ float2 row_phase(int64_t hq, int64_t sq, int n)
{
    const uint64_t nn = (uint64_t)n;
    const uint64_t ph = (uint64_t)hq * (nn * nn) - (uint64_t)sq * nn;
    return cis_frac64(ph);
}

// Row phase exp(j 2 pi (hq n^2 - sq n) / 2^64) of the 16 first-pass elements
// n = lt + r N/16 of one thread, requested for r = 0..15 in order.  With
// D = N/16 the fixed-point phase is exactly ph0 + r A + r^2 B
// (A = 2 hq lt D - sq D, B = hq D^2), so consecutive elements differ by the
// rotor cis(A + (2r+1) B), which itself turns by cis(2B).  Values are exact
// (sincospif of the fixed-point phase) at r = 0 and r = 8 and advanced by
// two complex multiplies in between: 5 sincospif per 16 elements instead of
// 16, with at most 7 rotor steps (~1e-6 relative) of accumulated rounding.
template <int N>
struct RowPhase {
    float2 C, S, Q;
    uint64_t ph0, A, B;
    __device__ __forceinline__ void init(int64_t hq, int64_t sq, int lt)
    {
        constexpr uint64_t D = N / 16;
        const uint64_t j = (uint64_t)lt;
        ph0 = (uint64_t)hq * (j * j) - (uint64_t)sq * j;
        A = 2ull * (uint64_t)hq * j * D - (uint64_t)sq * D;
        B = (uint64_t)hq * (D * D);
        Q = cis_frac64(2ull * B);
    }
    __device__ __forceinline__ float2 at(int r)
    {
        if (r == 0 || r == 8) {
            const uint64_t rr = (uint64_t)r;
            C = cis_frac64(ph0 + rr * A + rr * rr * B);
            S = cis_frac64(A + (2ull * rr + 1ull) * B);
        } else {
            C = cmul(C, S);
            S = cmul(S, Q);
        }
        return C;
    }
};

// Linear row phase exp(-j 2 pi sq n / 2^64) of the same 16 elements: exact
// at r = 0 and r = 8, one rotor step cis(-sq D) in between.
template <int N>
struct LinPhase {
    float2 C, R;
    uint64_t p0, d;
    __device__ __forceinline__ void init(int64_t sq, int lt)
    {
        constexpr uint64_t D = N / 16;
        p0 = 0ull - (uint64_t)sq * (uint64_t)lt;
        d = 0ull - (uint64_t)sq * D;
        R = cis_frac64(d);
    }
    __device__ __forceinline__ float2 at(int r)
    {
        if (r == 0 || r == 8) C = cis_frac64(p0 + (uint64_t)r * d);
        else C = cmul(C, R);
        return C;
    }
};

// One-row staging buffer in shared memory, filled by bulk asynchronous copies
// (cp.async.bulk, completion counted on an mbarrier).  The row kernels issue
// the copy of their next row as soon as every thread has read the current
// one (team_fft's hook), so the HBM read of row r+1 overlaps the transform
// of row r.  Waits are bounded: a wait that runs out sets *err and the CTA
// carries on (its rows are then invalid and the host reports the failure).
constexpr unsigned kRowWaitLimit = 1u << 22;

struct RowStage {
    float2* buf;      // N float2, 16-byte aligned
    uint64_t* bar;    // mbarrier
    unsigned* err;    // timeout flag (global)
    uint32_t parity;

    __device__ __forceinline__ static uint32_t saddr(const void* p)
    {
        return (uint32_t)__cvta_generic_to_shared(p);
    }
    // thread 0, before the CTA's first barrier
    __device__ __forceinline__ void init() const
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // thread 0: copy `bytes` from global src into buf
    __device__ __forceinline__ void issue(const void* src, uint32_t bytes) const
    {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(bar)), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                saddr(buf)),
            "l"(src), "r"(bytes), "r"(saddr(bar))
            : "memory");
    }
    __device__ __forceinline__ bool try_wait_once() const
    {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(saddr(bar)), "r"(parity)
            : "memory");
        return done != 0;
    }
    // every thread: wait for the copy in flight
    __device__ __forceinline__ void wait()
    {
        bool ok = false;
        for (unsigned i = 0; i < kRowWaitLimit && !ok; ++i) {
            ok = try_wait_once();
            if (!ok && i > 64) __nanosleep(64);
        }
        if (!ok) {
            atomicOr(err, 1u);
            for (unsigned i = 0; i < kRowWaitLimit && !try_wait_once(); ++i) __nanosleep(256);
        }
        parity ^= 1u;
    }
};

// Twiddle table of the range-alignment kernels: the two-level shared table
// above 2048 points (1.5 KB at N = 8192, filled by every CTA).  Measured
// alternatives were slower: a full N-entry table (read with 32-word strides
// by the radix-16 passes: many-way bank conflicts) and one exact table per
// pass (69 KB per CTA: the fill costs more than the saved multiplies).
template <int N>
using RaTw = RowTw<N>;

// HPC coefficient per pulse: alpha_m = coef * v_m / Fs^2 in cycles per n^2,
// coef = -4*pi*(B/Tp)/c (high_speed_compensation.cu:17-18).
__global__ void k_hpc_coef(const double* __restrict__ vel, int M, double coef_over_fs2, int64_t* __restrict__ hq)
{
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) {
        double cyc = coef_over_fs2 * vel[m] / 6.283185307179586476925;
        hq[m] = frac_to_fixed(cyc);
    }
}

// S[m] = 0 and its fixed-point phase slope SQ[m] = 0.
__global__ void k_zero_shift(double* __restrict__ S, int64_t* __restrict__ SQ, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        S[i] = 0.0;
        SQ[i] = 0;
    }
}

// S[row] += sh and SQ[row] = S[row] / N as a 64-bit fixed-point fraction,
// once per row (one thread), so that the row transforms read SQ directly.
__device__ __forceinline__ void add_shift(double* S, int64_t* SQ, size_t row, float sh, int N)
{
    const double v = S[row] + (double)sh;
    S[row] = v;
    SQ[row] = frac_to_fixed(v / (double)N);
}

// Standalone HPC (stage test entry): x *= exp(j*2*pi*alpha_m*n^2).
__global__ void k_hpc_apply(float2* __restrict__ x, const int64_t* __restrict__ hq, int N)
{
    const int m = blockIdx.y;
    const int64_t h = hq[m];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float2 v = x[(size_t)m * N + n];
        x[(size_t)m * N + n] = cmul(v, row_phase(h, 0, n));
    }
}

// Block-wide argmax (ArgKey order) over one value per thread slot.
template <int T>
__device__ __forceinline__ ArgKey block_argmax(ArgKey k, ArgKey* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ArgKey y;
        y.a = __shfl_xor_sync(0xffffffffu, k.a, o);
        y.i = __shfl_xor_sync(0xffffffffu, k.i, o);
        if (argkey_better(y, k)) k = y;
    }
    constexpr int W = T / 32;
    if constexpr (W > 1) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        if (lane == 0) red[w] = k;
        __syncthreads();
        if (w == 0) {
            k = (lane < W) ? red[lane] : red[0];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ArgKey y;
                y.a = __shfl_xor_sync(0xffffffffu, k.a, o);
                y.i = __shfl_xor_sync(0xffffffffu, k.i, o);
                if (argkey_better(y, k)) k = y;
            }
            if (lane == 0) red[0] = k;
        }
        __syncthreads();
        k = red[0];
        __syncthreads();
    }
    return k;
}

// Error-free float accumulation (TwoSum) of the exact product a*b (TwoProd via
// FMA) into the pair (hi, lo).
__device__ __forceinline__ void acc_prod(float a, float b, float& hi, float& lo)
{
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float t = hi + p;
    const float z = t - hi;
    lo += (hi - (t - z)) + (p - z) + e;
    hi = t;
}

// (h, l) += (h2, l2) for compensated float pairs (TwoSum on the high parts).
__device__ __forceinline__ void pair_add(float& h, float& l, float h2, float l2)
{
    const float t = h + h2;
    const float z = t - h;
    l += l2 + ((h - (t - z)) + (h2 - z));
    h = t;
}

// Block total of compensated float pairs as a double; valid in thread 0.
// Float arithmetic throughout (FP64 issues slowly on this part) with the
// precision of a double sum.
template <int T>
__device__ __forceinline__ double block_sum_pair0(float h, float l, float2* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        pair_add(h, l, __shfl_xor_sync(0xffffffffu, h, o), __shfl_xor_sync(0xffffffffu, l, o));
    double r = (double)h + (double)l;
    constexpr int W = T / 32;
    if constexpr (W > 1) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        if (lane == 0) red[w] = make_float2(h, l);
        __syncthreads();
        if (threadIdx.x == 0) {
            float H = red[0].x, L = red[0].y;
            for (int i = 1; i < W; ++i) pair_add(H, L, red[i].x, red[i].y);
            r = (double)H + (double)L;
        }
        __syncthreads();
    }
    return r;
}

// float(hi + lo + x) for a compensated pair (|lo| <= ulp(hi)), rounded once
// except in rare double-rounding ties.
__device__ __forceinline__ float csum3(float hi, float lo, float x)
{
    const float s = hi + lo;
    float e = lo - (s - hi);
    const float t = s + x;
    const float z = t - s;
    e += (s - (t - z)) + (x - z);
    return t + e;
}

// Correlates the RMS envelopes a = sqrt(ea), b = sqrt(eb) as the reference
// does, C2R(R2C(a) .* conj(R2C(b))) -> ifftshift -> argmax|.| -> parabolic
// fix (range_alignment.cu:50-66, :121-168), and returns the shift (all
// threads).  The FFT locates the peak; the three samples of the parabola are
// then evaluated directly, sum_n a[n] b[n - tau] with error-free float
// accumulation, because the second difference of a broad correlation peak
// magnifies FFT rounding into ~1e-4-cell shift errors.  A(n), B(n) return
// the amplitudes a[n], b[n] (shared-memory reads, n in [0, N)); sm_f is the
// FFT scratch.
template <int N, class AmpA, class AmpB, class Tw>
__device__ float ra_correlate_f(AmpA A, AmpB B, float* sm_f, int lt, const Tw& tw)
{
    using F = FFTShape<N>;
    constexpr int T = F::T;
    float2* sm = reinterpret_cast<float2*>(sm_f);
    __shared__ ArgKey red[32];
    __shared__ float2 redp[32];
    __shared__ float s_res;
    __shared__ int s_pos;
    // z = a + i b, forward FFT, spectrum kept in the scratch (padded slots)
    team_fft<N, false>([&](int i) { return make_float2(A(i), B(i)); },
                       [&](int i, float2 v, int) { sm[fpad(i)] = v; }, sm, lt, tw);
    // C[k] = A[k] * conj(B[k]) with A, B split from Z; corr = Re IFFT(C);
    // argmax over the ifftshifted index (i + N/2) mod N tracked per thread
    ArgKey best;
    best.a = -1.0f;
    best.i = 0x7fffffff;
    auto csrc = [&](int k) {
        const float2 zk = sm[fpad(k)];
        const float2 zn = sm[fpad((N - k) & (N - 1))];
        const float2 a = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
        const float2 d = make_float2(zk.x - zn.x, zk.y + zn.y);
        const float2 bc = make_float2(0.5f * d.y, 0.5f * d.x);   // conj(B), B = -i d / 2
        return cmul(a, bc);
    };
    auto cdst = [&](int i, float2 v, int) {
        ArgKey k;
        k.a = fabsf(v.x);
        k.i = (i + N / 2) & (N - 1);
        if (argkey_better(k, best)) best = k;
    };
    if constexpr (N == 8192 && std::is_same<Tw, RowTw<8192>>::value)
        row_fft<N, true, true>(csrc, cdst, sm, lt, tw, NoHook{});   // output order is irrelevant to an argmax
    else
        team_fft<N, true>(csrc, cdst, sm, lt, tw);
    best = block_argmax<T>(best, red);
    if (lt == 0) s_pos = best.i;
    __syncthreads();
    const int pos = s_pos;
    const int tau = (pos + N / 2) & (N - 1);
    // f_j = sum_n a[n] b[n - (tau + j)], j = -1, 0, 1
    float h[3] = {0.0f, 0.0f, 0.0f}, l[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll 4
    for (int t = 0; t < N / T; ++t) {
        const int n = lt + t * T;
        const float a = A(n);
#pragma unroll
        for (int j = 0; j < 3; ++j) acc_prod(a, B((n - tau - (j - 1)) & (N - 1)), h[j], l[j]);
    }
    double f[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) f[j] = block_sum_pair0<T>(h[j], l[j], redp);
    if (lt == 0) {
        // the reference keeps the correlation in a float buffer and fits the
        // parabola in float (binomialFixDevice, range_alignment.cu:121-131)
        const float f1 = (float)f[0], f2 = (float)f[1], f3 = (float)f[2];
        const float fa = __fdiv_rn(__fsub_rn(__fadd_rn(f1, f3), __fmul_rn(2.0f, f2)), 2.0f);
        const float fb = __fdiv_rn(__fsub_rn(f3, f1), 2.0f);
        const float delta = __fdiv_rn(-fb, __fmul_rn(2.0f, fa));
        s_res = __fsub_rn(__fadd_rn((float)pos, delta), (float)N / 2);
    }
    __syncthreads();
    const float r = s_res;
    __syncthreads();
    return r;
}

// ra_correlate_f on squared envelopes: ea, eb are adjacent N-float shared
// arrays, replaced in place by the amplitudes a = sqrt(ea), b = sqrt(eb).
template <int N, class Tw>
__device__ float ra_correlate(float* ea, float* sm_f, int lt, const Tw& tw)
{
    float* eb = ea + N;
    for (int i = lt; i < 2 * N; i += FFTShape<N>::T) ea[i] = sqrtf(ea[i]);
    __syncthreads();
    return ra_correlate_f<N>([&](int n) { return ea[n]; }, [&](int n) { return eb[n]; }, sm_f, lt, tw);
}

// s + x accumulated error-free into (s, c) (TwoSum).
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x)
{
    const float t = s + x;
    const float z = t - s;
    c += (s - (t - z)) + (x - z);
    s = t;
}

// The rows enter every transform pre-multiplied: level 0 reads the spectra
// x and stores u = x * win * exp(j 2 pi alpha n^2) / N (the window, the
// high-speed-compensation chirp and the IFFT's 1/N, which is exact) into the
// row buffer xw; later levels and the final transform read u and apply only
// the alignment ramp exp(-j 2 pi S n / N).  IFFT(u * ramp) is then the range
// profile itself, with no per-element window, chirp or scaling work.

// One row: IFFT(u * ramp), |.|^2 accumulated into acc/accl (register slots
// of this thread; compensated with COMP, else a plain float sum in acc).
// sr: the row in the staging buffer.  Level 0 (raw): sr holds x, u is formed
// and stored to ur (global); otherwise sr holds u.  hook: see team_fft.
// WARP: see row_fft.
template <int N, bool RAW, bool WARP, bool IQ16 = false, bool COMP = true, class Tw, class Hook>
__device__ __forceinline__ void ra_row_power(const float2* sr, float2* ur, const float* __restrict__ win, int64_t h,
                                             int64_t sq, float* acc, float* accl, float2* sm, int lt, const Tw& tw,
                                             Hook hook)
{
    auto sink = [&](int, float2 v, int slot) {
        const float p = v.x * v.x + v.y * v.y;
        if constexpr (COMP)
            two_sum_acc(acc[slot], accl[slot], p);
        else
            acc[slot] += p;
    };
    if constexpr (RAW) {
        const float invN = 1.0f / (float)N;
        RowPhase<N> rp;
        rp.init(h, sq, lt);
        row_fft<N, true, WARP>(
            [&](int i) {   // i = lt + r N/16, r = 0..15 in order
                float2 xv;
                if constexpr (IQ16) {
                    const short2 q = reinterpret_cast<const short2*>(sr)[i];
                    xv = make_float2((float)q.x, (float)q.y);
                } else {
                    xv = sr[i];
                }
                const float2 u = cscale(cmul(xv, rp.at((i - lt) / (N / 16))), __ldg(&win[i]) * invN);
                ur[i] = u;   // sq = 0 at level 0: the phase is the chirp alone
                return u;
            },
            sink, sm, lt, tw, hook);
    } else {
        LinPhase<N> lp;
        lp.init(sq, lt);
        row_fft<N, true, WARP>([&](int i) { return cmul(sr[i], lp.at((i - lt) / (N / 16))); }, sink, sm, lt, tw,
                               hook);
    }
}

// Level kernel, one CTA per pair j of groups (G_2j, G_2j+1) of size s=2^level.
// Level 0 (RAW) transforms both rows from x and stores their pre-multiplied
// rows into xw; level >= 1 transforms the second halves R_k of both groups
// from xw and adds the carried envelopes left_prev[k] of the first halves.
// Writes the pair shift, adds it to S of the rows of G_2j+1 and stores
// env^2(G_2j) as left_next[j].
template <int N, bool RAW, bool IQ16 = false>
__global__ void __launch_bounds__(N / 16)
k_ra_pair(const float2* __restrict__ x, float2* xw, const float* __restrict__ win, const int64_t* __restrict__ hq,
          double* __restrict__ S, int64_t* __restrict__ SQ, int level, const float* __restrict__ left_prev,
          int lstride, float* __restrict__ left_next, float* shift_out, int given, const float2* __restrict__ tw,
          unsigned* err)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(8) uint64_t bar;
    float* sm_f = reinterpret_cast<float*>(dyn_smem);
    float* ea = sm_f + 2 * F::SMEM;
    float* eb = ea + N;
    const int lt = threadIdx.x;
    const int s = 1 << level;
    const int j = blockIdx.x;
    float2* sm = reinterpret_cast<float2*>(sm_f);
    float2* twt = reinterpret_cast<float2*>(eb + N);
    // rows of this CTA in order: R_2j then R_2j+1 (one row each at level 0)
    const int nr = (level == 0) ? 1 : s / 2;
    auto row_of = [&](int t) {
        const int k = 2 * j + t / nr;
        return ((level == 0) ? k : k * s + s / 2) + t % nr;
    };
    // row r of the source: complex64 rows, or int16 I/Q rows at level 0
    constexpr uint32_t kRowBytes = IQ16 ? N * 2 * sizeof(int16_t) : N * sizeof(float2);
    const char* src = reinterpret_cast<const char*>(RAW ? x : xw);
    RowStage st{twt + RaTw<N>::kEntries, &bar, err, 0u};
    if (lt == 0) {
        st.init();
        st.issue(src + (size_t)row_of(0) * kRowBytes, kRowBytes);
    }
    RaTw<N>::fill(twt, tw, lt, F::T);
    __syncthreads();
    const RaTw<N> tws{twt};
#pragma unroll 1
    for (int g = 0; g < 2; ++g) {
        const int k = 2 * j + g;
        float acc[16], accl[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = accl[q] = 0.0f;
#pragma unroll 1
        for (int rr = 0; rr < nr; ++rr) {
            const int t = g * nr + rr;
            const int row = row_of(t);
            const int64_t h = hq ? hq[row] : 0;
            st.wait();
            auto next = [&]() {
                if (lt == 0 && t + 1 < 2 * nr) st.issue(src + (size_t)row_of(t + 1) * kRowBytes, kRowBytes);
            };
            ra_row_power<N, RAW, false, IQ16>(st.buf, xw + (size_t)row * N, win, h, SQ[row], acc, accl, sm, lt, tws,
                                              next);
        }
        float* e = g ? eb : ea;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int i = row_out_index<N, false>(lt, q);
            const float lp = (level > 0) ? left_prev[(size_t)k * lstride * N + i] : 0.0f;
            e[i] = csum3(acc[q], accl[q], lp);
        }
    }
    __syncthreads();
    if (left_next)
        for (int i = lt; i < N; i += F::T) left_next[(size_t)j * N + i] = ea[i];
    __syncthreads();
    const float shc = ra_correlate<N>(ea, sm_f, lt, tws);
    const float sh = given ? shift_out[j] : shc;   // given: shifts injected by the caller (test hook)
    if (lt == 0 && !given) shift_out[j] = sh;
    for (int m = lt; m < s; m += F::T) add_shift(S, SQ, (size_t)(2 * j + 1) * s + m, sh, N);
}

// Level >= 1, many rows per group: CTA b transforms rpc rows of R_k
// (k = b / nch, chunk q = b % nch) and writes their summed |p|^2.  The sum
// over a CTA's rows (at most 64) is a plain float sum, relative error below
// 4e-6; k_ra_reduce adds the partials with compensation.
template <int N>
__global__ void __launch_bounds__(N / 16)
k_ra_accum(const float2* __restrict__ xw, const int64_t* __restrict__ SQ, int level, int rpc,
           float* __restrict__ part, const float2* __restrict__ tw, unsigned* err)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(8) uint64_t bar;
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    const int lt = threadIdx.x;
    const int s = 1 << level;
    const int nch = (s / 2) / rpc;
    const int k = blockIdx.x / nch, q = blockIdx.x % nch;
    const int r0 = k * s + s / 2 + q * rpc;
    float2* twt = sm + F::SMEM;
    RowStage st{twt + RaTw<N>::kEntries, &bar, err, 0u};
    if (lt == 0) {
        st.init();
        st.issue(xw + (size_t)r0 * N, N * sizeof(float2));
    }
    RaTw<N>::fill(twt, tw, lt, F::T);
    __syncthreads();
    const RaTw<N> tws{twt};
    float acc[16], accl[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = accl[t] = 0.0f;
#pragma unroll 1
    for (int rr = 0; rr < rpc; ++rr) {
        const int row = r0 + rr;
        st.wait();
        auto next = [&]() {
            if (lt == 0 && rr + 1 < rpc) st.issue(xw + (size_t)(row + 1) * N, N * sizeof(float2));
        };
        ra_row_power<N, false, true, false, false>(st.buf, nullptr, nullptr, 0, SQ[row], acc, accl, sm, lt, tws, next);
    }
    // The warp transform leaves a lane's outputs 16 elements apart: reorder
    // the partial sums through the scratch (one pad word every 32) so that
    // the global stores coalesce.
    __syncthreads();   // every warp is done with the last row's tile
    float* pf = reinterpret_cast<float*>(sm);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        const int i = row_out_index<N, true>(lt, t);
        pf[i + (i >> 5)] = acc[t] + accl[t];
    }
    __syncthreads();
    for (int i = lt; i < N; i += F::T) part[(size_t)blockIdx.x * N + i] = pf[i + (i >> 5)];
}

// E[k] = left_prev[k * lstride] + sum of the nch partials of R_k
// (compensated float sum).
__global__ void k_ra_reduce(const float* __restrict__ left_prev, int lstride, const float* __restrict__ part,
                            int nch, int N, float* __restrict__ E)
{
    const int k = blockIdx.y;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float h = left_prev[(size_t)k * lstride * N + n], l = 0.0f;
        for (int q = 0; q < nch; ++q) two_sum_acc(h, l, part[((size_t)k * nch + q) * N + n]);
        E[(size_t)k * N + n] = h + l;
    }
}

// Pair correlation on materialised envelopes E[2j], E[2j+1].
template <int N>
__global__ void __launch_bounds__(N / 16)
k_ra_corr(const float* __restrict__ E, double* __restrict__ S, int64_t* __restrict__ SQ, int level,
          float* shift_out, int given, const float2* __restrict__ tw)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    float* sm_f = reinterpret_cast<float*>(dyn_smem);
    float* ea = sm_f + 2 * F::SMEM;
    const int lt = threadIdx.x;
    const int j = blockIdx.x;
    const int s = 1 << level;
    float2* twt = reinterpret_cast<float2*>(ea + 2 * N);
    RaTw<N>::fill(twt, tw, lt, F::T);
    for (int i = lt; i < 2 * N; i += F::T) ea[i] = E[(size_t)2 * j * N + i];
    __syncthreads();
    const float shc = ra_correlate<N>(ea, sm_f, lt, RaTw<N>{twt});
    const float sh = given ? shift_out[j] : shc;
    if (lt == 0 && !given) shift_out[j] = sh;
    for (int m = lt; m < s; m += F::T) add_shift(S, SQ, (size_t)(2 * j + 1) * s + m, sh, N);
}

// ---------------------------------------------------------------------------
// Spectral envelope merge.  A row's power at half-cell spacing, w[2n] =
// |p(n)|^2 and w[2n+1] = |p(n + 1/2)|^2, samples a trigonometric polynomial
// whose lags lie in (-N, N) (p carries the N frequencies 0..N-1), so the
// 2N-point spectrum W of w represents it exactly: shifting the row by s cells
// (the reference's ramp exp(-j 2 pi k s / N) on its spectrum) multiplies W[d]
// by exp(-j 2 pi d s / N), d the signed lag, and the power envelope of a
// group, sum_m |p_m(n - S_m)|^2, is the even-sample inverse transform of the
// sum of its rows' shifted spectra.  Level 0 computes each row's w (two
// IFFTs: even and odd samples), correlates the pair and stores the merged
// group spectrum W_a + ramp(s) W_b; every later level recovers both groups'
// envelopes with one packed IFFT, correlates them and merges their spectra
// with one more ramp.  Per pair that is 3 transforms instead of transforming
// every shifted row of the group again.  w is real, so W is Hermitian and
// only d in [0, N) is kept; W[N] is zero (p has no lag of N).

// Linear phase slopes sq of exp(-j 2 pi sq n / 2^64) (LinPhase, RowPhase
// without chirp): exp(+j pi n / N) (the odd samples p(n + 1/2)) and
// exp(-j pi n / N) (the odd half of W).
template <int N>
constexpr int64_t kHalfCellUp = (int64_t)(0ull - ((1ull << 63) / (uint64_t)N));
template <int N>
constexpr int64_t kHalfCellDown = (int64_t)((1ull << 63) / (uint64_t)N);

// W[d] = E[d] + exp(-j pi d / N) O[d] from Z = FFT(w_even + j w_odd):
// E = (Z[d] + conj Z[-d]) / 2, O = (Z[d] - conj Z[-d]) / 2j.
__device__ __forceinline__ float2 spec_half(float2 z, float2 zm, float2 h)
{
    const float2 e = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
    const float2 o = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
    const float2 ho = cmul(h, o);
    return make_float2(e.x + ho.x, e.y + ho.y);
}

// Level 0, one CTA per pair j of rows (2j, 2j+1): forms u = x * win * chirp
// / N and stores it into xw (x may equal xw), computes both rows' half-cell
// powers, correlates the pair, adds the shift to S of row 2j+1 and, when
// wout is set, stores the merged spectrum W_2j + ramp(s) W_2j+1 as wout[j].
// IQ16: x holds int16 I/Q pairs.  Both rows are copied into the CTA's row
// buffers by bulk asynchronous copies at the start (bounded waits set *err).
template <int N, bool IQ16>
__global__ void __launch_bounds__(N / 16)
k_ra_spec0(const float2* x, float2* xw, const float* __restrict__ win, const int64_t* __restrict__ hq,
           double* __restrict__ S, int64_t* __restrict__ SQ, float2* __restrict__ wout, float* shift_out, int given,
           const float2* __restrict__ tw, unsigned* err)
{
    using F = FFTShape<N>;
    constexpr int D = N / 16;
    constexpr uint32_t kRowBytes = IQ16 ? N * 2 * sizeof(int16_t) : N * sizeof(float2);
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(8) uint64_t bars[2];
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    // Row buffers: the staged row (contiguous), then c[n] at pc(n).  At
    // N = 8192 the row transforms run on fft8192, whose outputs arrive 16
    // apart across lanes: one pad slot per 16 keeps those stores apart in
    // the shared-memory banks.
    constexpr bool kWarp = (N == 8192);
    constexpr int CS = kWarp ? N + N / 16 : N;
    auto pc = [](int i) { return kWarp ? i + (i >> 4) : i; };
    float2* ca = sm + F::SMEM;   // row 2j: x, then (sqrt w[2n], w[2n+1]), then FFT(w_even + j w_odd)
    float2* cb = ca + CS;        // row 2j+1
    float2* twt = cb + CS;
    const int lt = threadIdx.x, j = blockIdx.x;
    RowStage sa{ca, &bars[0], err, 0u}, sb{cb, &bars[1], err, 0u};
    if (lt == 0) {
        const char* src = reinterpret_cast<const char*>(x);
        sa.init();
        sb.init();
        sa.issue(src + (size_t)(2 * j) * kRowBytes, kRowBytes);
        sb.issue(src + (size_t)(2 * j + 1) * kRowBytes, kRowBytes);
    }
    RaTw<N>::fill(twt, tw, lt, F::T);
    __syncthreads();
    const RaTw<N> tws{twt};
    const float invN = 1.0f / (float)N;
    // Four row transforms, k = 2t + odd (one instantiation): t selects the
    // row, odd = 0 the samples p(n) = IFFT(u), u formed from the staged row
    // and stored to xw (the staged copy makes x == xw safe), odd = 1 the
    // samples p(n + 1/2) = IFFT(u * exp(j pi k / N)), u read back by the
    // thread that stored it.  c[n] = (|p(n)|, |p(n + 1/2)|^2): the amplitude
    // feeds the correlation, its square the spectrum.
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int t = k >> 1, odd = k & 1;
        const int row = 2 * j + t;
        float2* c = t ? cb : ca;
        float* cf = reinterpret_cast<float*>(c) + odd;
        float2* ur = xw + (size_t)row * N;
        RowPhase<N> rp;   // the chirp (even) or the half-cell ramp (odd, no chirp)
        if (odd) rp.init(0, kHalfCellUp<N>, lt);
        else rp.init(hq ? hq[row] : 0, 0, lt);
        if (k == 0) sa.wait();
        else if (k == 2) sb.wait();
        row_fft<N, true, kWarp>(
            [&](int i) {
                const float2 ph = rp.at((i - lt) / D);
                if (odd) return cmul(ur[i], ph);
                float2 xv;
                if constexpr (IQ16) {
                    const short2 q = reinterpret_cast<const short2*>(c)[i];
                    xv = make_float2((float)q.x, (float)q.y);
                } else {
                    xv = c[i];
                }
                const float2 u = cscale(cmul(xv, ph), __ldg(&win[i]) * invN);
                ur[i] = u;
                return u;
            },
            [&](int n, float2 v, int) {
                const float w = v.x * v.x + v.y * v.y;
                cf[2 * pc(n)] = odd ? w : sqrtf(w);
            },
            sm, lt, tws, NoHook{});
    }
    __syncthreads();
    const float shc = ra_correlate_f<N>([&](int n) { return ca[pc(n)].x; }, [&](int n) { return cb[pc(n)].x; },
                                        reinterpret_cast<float*>(sm), lt, tws);
    const float sh = given ? shift_out[j] : shc;   // given: shifts injected by the caller (test hook)
    if (lt == 0) {
        if (!given) shift_out[j] = sh;
        add_shift(S, SQ, (size_t)2 * j + 1, sh, N);
    }
    if (wout == nullptr) return;
    // Z = FFT(w_even + j w_odd) in place (both transforms read all their
    // inputs before their first barrier and write their outputs after the
    // last)
#pragma unroll 1
    for (int t = 0; t < 2; ++t) {
        float2* c = t ? cb : ca;
        row_fft<N, false, kWarp>(
            [&](int i) {
                const float2 v = c[pc(i)];
                return make_float2(v.x * v.x, v.y);
            },
            [&](int k, float2 v, int) { c[pc(k)] = v; }, sm, lt, tws, NoHook{});
    }
    __syncthreads();
    LinPhase<N> h, r;
    h.init(kHalfCellDown<N>, lt);
    r.init(frac_to_fixed((double)sh / (double)N), lt);
    float2* w = wout + (size_t)j * N;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int d = lt + q * D;
        const int dm = (N - d) & (N - 1);
        const float2 hd = h.at(q), rd = r.at(q);
        const float2 wa = spec_half(ca[pc(d)], ca[pc(dm)], hd);
        const float2 wb = cmul(rd, spec_half(cb[pc(d)], cb[pc(dm)], hd));
        w[d] = make_float2(wa.x + wb.x, wa.y + wb.y);
    }
}

// Level >= 1, one CTA per pair j of groups (G_2j, G_2j+1) with merged
// spectra wprev[2j], wprev[2j+1]: envelopes
// env_a + j env_b = IFFT(X_a + j X_b) / (2N), X[d] = W[d] + conj W[N - d],
// correlation, the shift added to S of the rows of G_2j+1 and, when wout is
// set, the merged spectrum W_2j + ramp(s) W_2j+1 stored as wout[j].
template <int N>
__global__ void __launch_bounds__(N / 16)
k_ra_spec(const float2* __restrict__ wprev, float2* __restrict__ wout, double* __restrict__ S,
          int64_t* __restrict__ SQ, int level, float* shift_out, int given, const float2* __restrict__ tw)
{
    using F = FFTShape<N>;
    constexpr int D = N / 16;
    extern __shared__ float4 dyn_smem[];
    float* sm_f = reinterpret_cast<float*>(dyn_smem);
    float* ea = sm_f + 2 * F::SMEM;
    float* eb = ea + N;
    float2* twt = reinterpret_cast<float2*>(eb + N);
    float2* sm = reinterpret_cast<float2*>(sm_f);
    const int lt = threadIdx.x, j = blockIdx.x;
    const int s = 1 << level;
    RaTw<N>::fill(twt, tw, lt, F::T);
    __syncthreads();
    const RaTw<N> tws{twt};
    const float2* wa = wprev + (size_t)2 * j * N;
    const float2* wb = wa + N;
    const float inv2N = 0.5f / (float)N;
    team_fft<N, true>(
        [&](int d) {
            float2 xa = __ldg(&wa[d]), xb = __ldg(&wb[d]);
            if (d) {
                const float2 am = __ldg(&wa[N - d]), bm = __ldg(&wb[N - d]);
                xa = make_float2(xa.x + am.x, xa.y - am.y);
                xb = make_float2(xb.x + bm.x, xb.y - bm.y);
            }
            return make_float2(xa.x - xb.y, xa.y + xb.x);
        },
        [&](int n, float2 v, int) {
            ea[n] = sqrtf(fmaxf(v.x * inv2N, 0.0f));
            eb[n] = sqrtf(fmaxf(v.y * inv2N, 0.0f));
        },
        sm, lt, tws);
    __syncthreads();
    const float shc = ra_correlate_f<N>([&](int n) { return ea[n]; }, [&](int n) { return eb[n]; }, sm_f, lt, tws);
    const float sh = given ? shift_out[j] : shc;
    if (lt == 0 && !given) shift_out[j] = sh;
    for (int m = lt; m < s; m += F::T) add_shift(S, SQ, (size_t)(2 * j + 1) * s + m, sh, N);
    if (wout == nullptr) return;
    LinPhase<N> r;
    r.init(frac_to_fixed((double)sh / (double)N), lt);
    float2* w = wout + (size_t)j * N;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int d = lt + q * D;
        const float2 rb = cmul(r.at(q), __ldg(&wb[d]));
        const float2 a = __ldg(&wa[d]);
        w[d] = make_float2(a.x + rb.x, a.y + rb.y);
    }
}

// Final transform of all rows: y = IFFT(u * ramp) from the pre-multiplied
// rows xw (written in place when y == xw), or with RAW (a single pulse, no
// level ran) y = IFFT(x * win * chirp) / N from the spectra.
// Epilogue: column sums of |y| over rows < min(M,256) per CTA (ARP partials)
// and the global max |y| (HRRPCenter normalisation, range_alignment.cu:380-399).
template <int N, bool RAW>
__global__ void __launch_bounds__(N / 16)
k_ra_final(const float2* x, float2* yout, const float* __restrict__ win, const int64_t* __restrict__ hq,
           const int64_t* __restrict__ SQ, int rpc, int arp_rows, float* __restrict__ arp_part,
           unsigned* __restrict__ hmax, const float2* __restrict__ tw, unsigned* err)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    __shared__ __align__(8) uint64_t bar;
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    __shared__ float s_red[32];
    const int lt = threadIdx.x;
    const int r0 = blockIdx.x * rpc;
    float2* twt = sm + F::SMEM;
    RowStage st{twt + RaTw<N>::kEntries, &bar, err, 0u};
    if (lt == 0) {
        st.init();
        st.issue(x + (size_t)r0 * N, N * sizeof(float2));
    }
    RaTw<N>::fill(twt, tw, lt, F::T);
    __syncthreads();
    const RaTw<N> tws{twt};
    float acc[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = 0.0f;
    float mx = 0.0f;
#pragma unroll 1
    for (int rr = 0; rr < rpc; ++rr) {
        const int row = r0 + rr;
        const int64_t sq = SQ[row];
        const float2* xr = st.buf;
        float2* yr = yout + (size_t)row * N;
        st.wait();
        auto next = [&]() {
            if (lt == 0 && rr + 1 < rpc) st.issue(x + (size_t)(row + 1) * N, N * sizeof(float2));
        };
        const bool arp = row < arp_rows;
        auto sink = [&](int i, float2 y, int slot) {
            yr[i] = y;
            const float a = sqrtf(y.x * y.x + y.y * y.y);
            mx = fmaxf(mx, a);
            if (arp) acc[slot] += a;
        };
        if constexpr (RAW) {
            const float invN = 1.0f / (float)N;
            RowPhase<N> rp;
            rp.init(hq ? hq[row] : 0, sq, lt);
            row_fft<N, true, false>(
                [&](int i) { return cscale(cmul(xr[i], rp.at((i - lt) / (N / 16))), __ldg(&win[i]) * invN); },
                sink, sm, lt, tws, next);
        } else {
            LinPhase<N> lp;
            lp.init(sq, lt);
            row_fft<N, true, false>([&](int i) { return cmul(xr[i], lp.at((i - lt) / (N / 16))); }, sink, sm, lt, tws,
                                    next);
        }
    }
    if (r0 < arp_rows) {
#pragma unroll
        for (int t = 0; t < 16; ++t) arp_part[(size_t)blockIdx.x * N + row_out_index<N, false>(lt, t)] = acc[t];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((lt & 31) == 0) s_red[lt >> 5] = mx;
    __syncthreads();
    if (lt == 0) {
        float m = 0.0f;
        for (int w = 0; w < (F::T + 31) / 32; ++w) m = fmaxf(m, s_red[w]);
        atomicMax(hmax, __float_as_uint(m));
    }
}

// ARP[n] = (sum_p part[p][n]) * (1/hmax) * (1/M)   (range_alignment.cu:388-399)
__global__ void k_arp_reduce(const float* __restrict__ part, int nparts, int N, int M,
                             const unsigned* __restrict__ hmax, float* __restrict__ arp)
{
    // an all-zero frame (max 0) gives a zero profile rather than 0/0
    const float hm = __uint_as_float(*hmax);
    const float inv = hm > 0.0f ? 1.0f / hm : 0.0f;
    const float invM = 1.0f / (float)M;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int p = 0; p < nparts; ++p) s += part[(size_t)p * N + n];
        arp[n] = (s * inv) * invM;
    }
}

// Standalone ARP inputs from materialised profiles y (stage entry point).
__global__ void k_ymax(const float2* __restrict__ y, long n, unsigned* __restrict__ hmax)
{
    float mx = 0.0f;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 v = y[i];
        mx = fmaxf(mx, sqrtf(v.x * v.x + v.y * v.y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(hmax, __float_as_uint(mx));
}

__global__ void k_ycolsum(const float2* __restrict__ y, int N, int rows, float* __restrict__ colsum)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int m = 0; m < rows; ++m) {
            const float2 v = y[(size_t)m * N + n];
            s += sqrtf(v.x * v.x + v.y * v.y);
        }
        colsum[n] = s;
    }
}

// getARPMean (range_alignment.cu:524-550) for one index, float as written.
__device__ __forceinline__ float arp_mean(const float* arp, int idx, int WL, int N)
{
    float s = 0.0f;
    if (idx - WL / 2 >= 0 && idx + WL / 2 <= N - 1) {
        for (int i = idx - WL / 2; i <= idx + WL / 2; ++i) s += arp[i];
        s /= (float)(WL + 1);
    } else if (idx - WL / 2 < 0) {
        for (int i = 0; i <= idx + WL / 2; ++i) s += arp[i];
        s /= ((float)WL / 2 + idx + 1);
    } else if (idx + WL / 2 > N - 1) {
        for (int i = idx - WL / 2; i < N; ++i) s += arp[i];
        s /= ((float)N - idx - ((float)WL / 2) - 1);
    }
    return s;
}

template <class T>
__device__ __forceinline__ T block_sum_1024(T v, T* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : (T)0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[0] = v;
    }
    __syncthreads();
    v = red[0];
    __syncthreads();
    return v;
}

// Ascending sort of the n non-negative floats in s (their bit patterns order
// as unsigned integers), one CTA of 1024 threads: an LSD radix sort, four
// passes of 8-bit digits.  Threads t < n / 8 (whole warps, n >= 256) hold 8
// keys each; slot e of lane l of warp w is element 256 w + 32 e + l of the
// current order, which every pass keeps stable: within a warp a key's rank
// among equal digits comes from __match_any_sync and a running count per
// (digit, warp) over the slots, across warps from an exclusive scan of the
// counts in digit-major order.  cnt: 256 * (n / 256 + 1) ints (one pad
// column against bank conflicts); red: 32 ints.
__device__ void block_radix_sort(float* s, int n, int* cnt, int* red)
{
    const int T = n / 8, W = T / 32, WP = W + 1;
    const int lw = 31 - __clz(W);   // W = n / 256 is a power of two
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const bool act = tid < T;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned k[8];
    int off[8];
#pragma unroll 1
    for (int shift = 0; shift < 32; shift += 8) {
        for (int i = tid; i < 256 * WP; i += blockDim.x) cnt[i] = 0;
        if (act) {
#pragma unroll
            for (int e = 0; e < 8; ++e) k[e] = __float_as_uint(s[256 * w + 32 * e + lane]);
        }
        __syncthreads();   // keys loaded, counters cleared
        if (act) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int d = (int)((k[e] >> shift) & 255u);
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                const int rank = __popc(peers & lt_mask);
                const int base = cnt[d * WP + w];
                off[e] = base + rank;
                __syncwarp();
                if (rank == 0) cnt[d * WP + w] = base + __popc(peers);
                __syncwarp();
            }
        }
        __syncthreads();
        // exclusive scan of cnt over f = d * W + w: q consecutive entries per
        // thread, then the threads' totals across the block
        const int total = 256 * W;
        const int q = (total + (int)blockDim.x - 1) / (int)blockDim.x;   // <= 8
        const int f0 = tid * q;
        int loc[8];
        int sum = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            loc[j] = sum;
            const int f = f0 + j;
            if (j < q && f < total) sum += cnt[(f >> lw) * WP + (f & (W - 1))];
        }
        int x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) red[w] = x;
        __syncthreads();
        if (w == 0) {
            const int v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0;
            int z = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            red[lane] = z - v;
        }
        __syncthreads();
        const int excl = red[w] + x - sum;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int f = f0 + j;
            if (j < q && f < total) cnt[(f >> lw) * WP + (f & (W - 1))] = excl + loc[j];
        }
        __syncthreads();   // cnt holds each (digit, warp) start
        if (act) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int d = (int)((k[e] >> shift) & 255u);
                s[cnt[d * WP + w] + off[e]] = __uint_as_float(k[e]);
            }
        }
        __syncthreads();
    }
}

// HRRPCenter decisions + cutRangeProfile offset, one CTA of 1024 threads.
// dec: [0] applied, [1] shift_num, [2] cut offset, [3] |idx_1|, [4] |idx_2|,
//      [5] threshold (float bits).
__global__ void __launch_bounds__(1024)
k_center(const float* __restrict__ arp_g, const float2* __restrict__ y, int N, int inter_length,
         int* __restrict__ dec)
{
    extern __shared__ float4 dyn_smem[];
    float* arp = reinterpret_cast<float*>(dyn_smem);
    float* srt = arp + N;
    __shared__ long long red_ll[32];
    __shared__ int red_i[32];
    __shared__ float red_f[32];
    __shared__ int red_j[32];
    __shared__ int sort_cnt[256 * (kMaxN / 256 + 1)];
    const int tid = threadIdx.x;
    for (int i = tid; i < N; i += blockDim.x) {
        const float v = arp_g[i];
        arp[i] = v;
        srt[i] = v;
    }
    __syncthreads();
    // ascending sort (thrust::stable_sort of arp1, :404; values only, so
    // stability does not show)
    block_radix_sort(srt, N, sort_cnt, red_i);
    // extra = inter_length * max(arp1) / N ; diff argmin (first index) (:406-420)
    const float arp1_max = srt[N - 1];
    const float extra = (float)inter_length * arp1_max / (float)N;
    const int dl = N - inter_length;
    float bv = 3.4e38f;
    int bi = 0x7fffffff;
    for (int i = tid; i < dl; i += blockDim.x) {
        const float d = fabsf(srt[i + inter_length] - srt[i] - extra);
        if (d < bv || (d == bv && i < bi)) {
            bv = d;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov < bv || (ov == bv && oi < bi)) {
            bv = ov;
            bi = oi;
        }
    }
    if ((tid & 31) == 0) {
        red_f[tid >> 5] = bv;
        red_j[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
        float v = red_f[0];
        int ii = red_j[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (red_f[w] < v || (red_f[w] == v && red_j[w] < ii)) {
                v = red_f[w];
                ii = red_j[w];
            }
        red_j[0] = ii;
    }
    __syncthreads();
    // a profile without a finite minimum (NaN everywhere) keeps index 0
    const int dmin = red_j[0] < dl ? red_j[0] : 0;
    __syncthreads();
    const float thr = srt[dmin + inter_length / 2];
    // idx_1 = find(arp > thr); drop those whose 9-tap mean < thr (:426-449)
    int n1 = 0, n2 = 0;
    long long sum = 0;
    for (int n = tid; n < N; n += blockDim.x) {
        if (arp[n] > thr) {
            ++n1;
            if (arp_mean(arp, n, 8, N) < thr) ++n2;
            else sum += n;
        }
    }
    n1 = block_sum_1024<int>(n1, red_i);
    n2 = block_sum_1024<int>(n2, red_i);
    sum = block_sum_1024<long long>(sum, red_ll);
    int applied = 0, shift = 0;
    if (n2 != n1) {
        const int mean_idx = (int)(sum / (long long)(n1 - n2));
        shift = -(mean_idx - N / 2);
        applied = 1;
    }
    // cutRangeProfile: Icamax (|Re|+|Im|, first max) of centred row 0
    float cv = -1.0f;
    int ci = 0x7fffffff;
    for (int n = tid; n < N; n += blockDim.x) {
        const float2 v = y[(n - shift) & (N - 1)];
        const float a = fabsf(v.x) + fabsf(v.y);
        if (a > cv) {
            cv = a;
            ci = n;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, cv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, ci, o);
        if (ov > cv || (ov == cv && oi < ci)) {
            cv = ov;
            ci = oi;
        }
    }
    if ((tid & 31) == 0) {
        red_f[tid >> 5] = cv;
        red_j[tid >> 5] = ci;
    }
    __syncthreads();
    if (tid == 0) {
        float v = red_f[0];
        int ii = red_j[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (red_f[w] > v || (red_f[w] == v && red_j[w] < ii)) {
                v = red_f[w];
                ii = red_j[w];
            }
        int off = ii - kRangeCut / 2;
        if (off < 0) off = 0;
        if (off > N - kRangeCut) off = N - kRangeCut;
        dec[0] = applied;
        dec[1] = shift;
        dec[2] = off;
        dec[3] = n1;
        dec[4] = n2;
        dec[5] = __float_as_int(thr);
    }
}

// cut[m][c] = centred y[m][off + c] = y[m][(off + c - shift) mod N]
__global__ void k_cut(const float2* __restrict__ y, int N, const int* __restrict__ dec, float2* __restrict__ cut)
{
    const int m = blockIdx.x;
    const int shift = dec[1], off = dec[2];
    for (int c = threadIdx.x; c < kRangeCut; c += blockDim.x)
        cut[(size_t)m * kRangeCut + c] = y[(size_t)m * N + ((off + c - shift) & (N - 1))];
}

// IFDS pre-step (isar_main.cu:15-27): ifftshift, IFFT/N, ifftshift per row.
template <int N>
__global__ void __launch_bounds__(N / 16) k_ifds_pre(float2* x, const float2* __restrict__ tw)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    float2* xr = x + (size_t)blockIdx.x * N;
    const float invN = 1.0f / (float)N;
    team_fft<N, true>([&](int i) { return xr[(i + N / 2) & (N - 1)]; },
                      [&](int i, float2 v, int) { xr[(i + N / 2) & (N - 1)] = cscale(v, invN); },
                      sm, threadIdx.x, tw);
}

// Test entry: batched row FFTs of length N (unnormalised).
template <int N, bool INV>
__global__ void __launch_bounds__(N / 16) k_fft_rows(float2* x, const float2* __restrict__ tw)
{
    using F = FFTShape<N>;
    extern __shared__ float4 dyn_smem[];
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    float2* xr = x + (size_t)blockIdx.x * N;
    team_fft<N, INV>([&](int i) { return xr[i]; }, [&](int i, float2 v, int) { xr[i] = v; }, sm, threadIdx.x, tw);
}

// getHRRP (common.cu:541-580), one CTA per row (out may equal x): STRETCH
// rows are FFT(x * hamming) with the halves swapped (ifftshiftRows); IFDS
// rows are swapped, transformed and swapped again.  Both swaps are folded
// into the transform's load and store indices.
template <int N>
__global__ void __launch_bounds__(N / 16)
k_hrrp(const float2* x, float2* out, const float* __restrict__ ham, int ifds, const float2* __restrict__ tw)
{
    extern __shared__ float4 dyn_smem[];
    float2* sm = reinterpret_cast<float2*>(dyn_smem);
    const float2* xr = x + (size_t)blockIdx.x * N;
    float2* o = out + (size_t)blockIdx.x * N;
    team_fft<N, false>(
        [&](int i) { return ifds ? xr[(i + N / 2) & (N - 1)] : cscale(xr[i], __ldg(&ham[i])); },
        [&](int i, float2 v, int) { o[(i + N / 2) & (N - 1)] = v; }, sm, threadIdx.x, tw);
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
// pair correlation: FFT scratch + twiddle table + two envelopes
template <int N>
static size_t corr_smem()
{
    return ((size_t)FFTShape<N>::SMEM + RaTw<N>::kEntries) * sizeof(float2) + 2 * N * sizeof(float);
}
// fused pair kernel: as corr_smem plus the row staging buffer
template <int N>
static size_t pair_smem() { return corr_smem<N>() + N * sizeof(float2); }
// spectral level 0: FFT scratch + two rows of half-cell powers + twiddle table
template <int N>
static size_t spec0_smem()
{
    constexpr size_t CS = (N == 8192) ? N + N / 16 : N;
    return ((size_t)FFTShape<N>::SMEM + 2 * CS + RaTw<N>::kEntries) * sizeof(float2);
}
// range-alignment row kernels: FFT scratch + twiddle table + row staging buffer
template <int N>
static size_t ra_fft_smem() { return ((size_t)FFTShape<N>::SMEM + RaTw<N>::kEntries + N) * sizeof(float2); }
// kernels on the global twiddle table: FFT scratch only
template <int N>
static size_t fft_smem() { return (size_t)FFTShape<N>::SMEM * sizeof(float2); }

template <int N>
static cudaError_t set_attrs_now()
{
    cudaError_t e;
    const int big = (int)pair_smem<N>();
    if ((e = cudaFuncSetAttribute(k_ra_pair<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_pair<N, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big)))
        return e;
    if ((e = cudaFuncSetAttribute(k_ra_pair<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_corr<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)corr_smem<N>())))
        return e;
    const int sp0 = (int)spec0_smem<N>();
    if ((e = cudaFuncSetAttribute(k_ra_spec0<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sp0))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_spec0<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sp0))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_spec<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)corr_smem<N>())))
        return e;
    const int r = (int)ra_fft_smem<N>();
    if ((e = cudaFuncSetAttribute(k_ra_accum<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, r))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_final<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, r))) return e;
    if ((e = cudaFuncSetAttribute(k_ra_final<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, r))) return e;
    const int f = (int)fft_smem<N>();
    if ((e = cudaFuncSetAttribute(k_ifds_pre<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, f))) return e;
    if ((e = cudaFuncSetAttribute(k_fft_rows<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, f))) return e;
    if ((e = cudaFuncSetAttribute(k_fft_rows<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, f))) return e;
    if ((e = cudaFuncSetAttribute(k_hrrp<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, f))) return e;
    return cudaSuccess;
}

// Shared-memory limits of the row kernels for N cells, set once per device.
template <int N>
static cudaError_t set_attrs()
{
    static PerDevice done;
    const int r = done.get([]() -> int { return -(int)set_attrs_now<N>(); });
    return r < 0 ? (cudaError_t)(-r) : cudaSuccess;
}

template <int N>
static cudaError_t ra_run_n(const RAArgs& a, cudaStream_t st)
{
    cudaError_t e = set_attrs<N>();
    if (e) return e;
    const int M = a.M;
    const int T = N / 16;
    int L = 0;
    while ((1 << L) < M) ++L;
    k_zero_shift<<<(M + 255) / 256, 256, 0, st>>>(a.S, a.SQ, M);
    ISAR_COUNT(1);
    // spectral envelope merge: merged group spectra ping-pong between env_a
    // (M/2 x N complex) and part (M/4 x N complex)
    const bool spectral = !a.rows_each_level && L >= 1;
    if (spectral) {
        float2* wb[2] = {reinterpret_cast<float2*>(a.env_a), reinterpret_cast<float2*>(a.part)};
        float2* w0 = L > 1 ? wb[0] : nullptr;
        if (a.x_iq16)
            k_ra_spec0<N, true><<<M / 2, T, spec0_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.S, a.SQ, w0, a.shifts,
                                                                   a.given_shifts, a.tw, a.err);
        else
            k_ra_spec0<N, false><<<M / 2, T, spec0_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.S, a.SQ, w0, a.shifts,
                                                                    a.given_shifts, a.tw, a.err);
        ISAR_COUNT(1);
        int off = M / 2;
        for (int lv = 1; lv < L; ++lv) {
            const int pairs = M >> (lv + 1);
            k_ra_spec<N><<<pairs, T, corr_smem<N>(), st>>>(wb[(lv - 1) & 1], lv == L - 1 ? nullptr : wb[lv & 1], a.S,
                                                          a.SQ, lv, a.shifts + off, a.given_shifts, a.tw);
            ISAR_COUNT(1);
            off += pairs;
        }
        if ((e = cudaGetLastError())) return e;
    }
    const float* left = nullptr;
    int lstride = 1;
    float* bufs[2] = {a.env_a, a.env_b};
    int cur = 0;
    int shift_off = 0;
    for (int lv = 0; lv < L && !spectral; ++lv) {
        const int s = 1 << lv;
        const int pairs = M / (2 * s);
        const bool last = (lv == L - 1);
        const bool use_pair = (lv == 0) || pairs >= a.pair_min || (s / 2) <= 1;
        if (use_pair) {
            float* ln = last ? nullptr : bufs[cur];
            if (lv == 0 && a.x_iq16)
                k_ra_pair<N, true, true><<<pairs, T, pair_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.S, a.SQ, lv, left,
                                                                          lstride, ln, a.shifts + shift_off,
                                                                          a.given_shifts, a.tw, a.err);
            else if (lv == 0)
                k_ra_pair<N, true><<<pairs, T, pair_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.S, a.SQ, lv, left,
                                                                    lstride, ln, a.shifts + shift_off,
                                                                    a.given_shifts, a.tw, a.err);
            else
                k_ra_pair<N, false><<<pairs, T, pair_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.S, a.SQ, lv, left,
                                                                     lstride, ln, a.shifts + shift_off,
                                                                     a.given_shifts, a.tw, a.err);
            ISAR_COUNT(1);
            left = ln;
            lstride = 1;
        } else {
            int rpc = a.rpc;
            if (rpc > s / 2) rpc = s / 2;
            const int nch = (s / 2) / rpc;
            const int groups = M / s;
            k_ra_accum<N><<<groups * nch, T, ra_fft_smem<N>(), st>>>(a.y, a.SQ, lv, rpc, a.part, a.tw, a.err);
            ISAR_COUNT(1);
            float* E = bufs[cur];
            dim3 g((N + 255) / 256, groups);
            k_ra_reduce<<<g, 256, 0, st>>>(left, lstride, a.part, nch, N, E);
            ISAR_COUNT(1);
            k_ra_corr<N><<<pairs, T, corr_smem<N>(), st>>>(E, a.S, a.SQ, lv, a.shifts + shift_off, a.given_shifts,
                                                          a.tw);
            ISAR_COUNT(1);
            left = E;
            lstride = 2;
        }
        cur ^= 1;
        shift_off += pairs;
        if ((e = cudaGetLastError())) return e;
    }
    // final IFFT + ARP partials + hmax
    cudaMemsetAsync(a.hmax, 0, sizeof(unsigned), st);
    const int arp_rows = M < 256 ? M : 256;
    int rpcf = a.rpc_final;
    while (rpcf > 1 && (M % rpcf)) rpcf >>= 1;
    if (L == 0 && a.x_iq16) return cudaErrorInvalidValue;   // a single pulse: no level reads x
    if (L == 0)
        k_ra_final<N, true><<<M / rpcf, T, ra_fft_smem<N>(), st>>>(a.x, a.y, a.win, a.hq, a.SQ, rpcf, arp_rows, a.part,
                                                                  a.hmax, a.tw, a.err);
    else
        k_ra_final<N, false><<<M / rpcf, T, ra_fft_smem<N>(), st>>>(a.y, a.y, a.win, a.hq, a.SQ, rpcf, arp_rows,
                                                                   a.part, a.hmax, a.tw, a.err);
    ISAR_COUNT(1);
    const int nparts = (arp_rows + rpcf - 1) / rpcf;
    k_arp_reduce<<<(N + 255) / 256, 256, 0, st>>>(a.part, nparts, N, M, a.hmax, a.arp);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t ra_run(const RAArgs& a, cudaStream_t st)
{
    switch (a.N) {
    case 512: return ra_run_n<512>(a, st);
    case 1024: return ra_run_n<1024>(a, st);
    case 2048: return ra_run_n<2048>(a, st);
    case 4096: return ra_run_n<4096>(a, st);
    case 8192: return ra_run_n<8192>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t arp_from_y(const float2* y, int M, int N, float* tmp, unsigned* hmax, float* arp, cudaStream_t st)
{
    cudaMemsetAsync(hmax, 0, sizeof(unsigned), st);
    k_ymax<<<1024, 256, 0, st>>>(y, (long)M * N, hmax);
    ISAR_COUNT(1);
    k_ycolsum<<<(N + 255) / 256, 256, 0, st>>>(y, N, M < 256 ? M : 256, tmp);
    ISAR_COUNT(1);
    k_arp_reduce<<<(N + 255) / 256, 256, 0, st>>>(tmp, 1, N, M, hmax, arp);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t hpc_coef(const double* vel, int M, double coef_over_fs2, int64_t* hq, cudaStream_t st)
{
    k_hpc_coef<<<(M + 255) / 256, 256, 0, st>>>(vel, M, coef_over_fs2, hq);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t hpc_apply(float2* x, const int64_t* hq, int M, int N, cudaStream_t st)
{
    dim3 g((N + 255) / 256, M);
    k_hpc_apply<<<g, 256, 0, st>>>(x, hq, N);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t center_cut(const float* arp, const float2* y, int M, int N, int* dec, float2* cut, cudaStream_t st)
{
    static PerDevice attr;   // k_center's shared-memory limit, set once per device
    const int ar = attr.get([]() -> int { return -(int)center_prepare_current_device(); });
    if (ar < 0) return (cudaError_t)(-ar);
    k_center<<<1, 1024, 2 * N * sizeof(float), st>>>(arp, y, N, 30, dec);
    ISAR_COUNT(1);
    k_cut<<<M, 256, 0, st>>>(y, N, dec, cut);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t center_prepare_current_device()
{
    return cudaFuncSetAttribute(k_center, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kMaxN * (int)sizeof(float));
}

template <int N>
static cudaError_t ifds_n(float2* x, int M, const float2* tw, cudaStream_t st)
{
    cudaError_t e = set_attrs<N>();
    if (e) return e;
    k_ifds_pre<N><<<M, N / 16, fft_smem<N>(), st>>>(x, tw);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t ifds_pre(float2* x, int M, int N, const float2* tw, cudaStream_t st)
{
    switch (N) {
    case 512: return ifds_n<512>(x, M, tw, st);
    case 1024: return ifds_n<1024>(x, M, tw, st);
    case 2048: return ifds_n<2048>(x, M, tw, st);
    case 4096: return ifds_n<4096>(x, M, tw, st);
    case 8192: return ifds_n<8192>(x, M, tw, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int N>
static cudaError_t fftrows_n(float2* x, int rows, int inverse, const float2* tw, cudaStream_t st)
{
    cudaError_t e = set_attrs<N>();
    if (e) return e;
    if (inverse) k_fft_rows<N, true><<<rows, N / 16, fft_smem<N>(), st>>>(x, tw);
    else k_fft_rows<N, false><<<rows, N / 16, fft_smem<N>(), st>>>(x, tw);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

template <int N>
static cudaError_t hrrp_n(const float2* x, float2* out, int rows, const float* ham, int ifds, const float2* tw,
                          cudaStream_t st)
{
    cudaError_t e = set_attrs<N>();
    if (e) return e;
    k_hrrp<N><<<rows, N / 16, fft_smem<N>(), st>>>(x, out, ham, ifds, tw);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t hrrp(const float2* x, float2* out, int rows, int n, const float* ham, int ifds, const float2* tw,
                 cudaStream_t st)
{
    switch (n) {
    case 512: return hrrp_n<512>(x, out, rows, ham, ifds, tw, st);
    case 1024: return hrrp_n<1024>(x, out, rows, ham, ifds, tw, st);
    case 2048: return hrrp_n<2048>(x, out, rows, ham, ifds, tw, st);
    case 4096: return hrrp_n<4096>(x, out, rows, ham, ifds, tw, st);
    case 8192: return hrrp_n<8192>(x, out, rows, ham, ifds, tw, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t fft_rows(float2* x, int rows, int n, int inverse, const float2* tw, cudaStream_t st)
{
    switch (n) {
    case 512: return fftrows_n<512>(x, rows, inverse, tw, st);
    case 1024: return fftrows_n<1024>(x, rows, inverse, tw, st);
    case 2048: return fftrows_n<2048>(x, rows, inverse, tw, st);
    case 4096: return fftrows_n<4096>(x, rows, inverse, tw, st);
    case 8192: return fftrows_n<8192>(x, rows, inverse, tw, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace isar
