// Doppler tracking and fast minimum-entropy autofocus on the M x 512 cut.
// Reference: phase_adjustment.cu:4-41 (dopplerTracking), :167-332
// (fastEntropy), common.cu:341-391 (maxCols/sumCols), :436-462 (sumRows).
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include "fft.cuh"
#include "isar_kernels.h"
#include "nn.h"

namespace isar {

constexpr int C = kRangeCut;

// The cluster engines' entropy of the selected bins (stop criterion, choice
// of start, trace) sums p log2 p with the hardware base-2 logarithm
// (__log2f, ~2^-22 relative error, a few instructions instead of ~20 for
// logf) and converts once: H = ln S1 - ln 2 * S2 / S1.
constexpr float kLn2 = 0.693147180559945309f;

// The stop criterion compares the entropy every kStopEvery iterations: stop
// at iteration it (a multiple of kStopEvery, it > 0, before its update) once
// |E(it) - E(it - kStopEvery)| <= kStopEvery * tol * |E(it)|, i.e. once the
// entropy changes by at most tol * |E| per iteration on average.  Iterations
// in between skip the entropy terms and its cluster reduction.
constexpr int kStopEvery = 4;

// Column max of |cut| over rows [0, min(M,256)) per CTA of R rows, and the
// Doppler sums s[m] = sum_c conj(x[m,c]) x[m+1,c] (one warp per row).
__global__ void __launch_bounds__(256)
k_fe_stats(const float2* __restrict__ cut, int M, int rows_max, int R, float* __restrict__ cmax_part,
           float2* __restrict__ dsum)
{
    const int r0 = blockIdx.x * R;
    const int tid = threadIdx.x;
    if (cmax_part != nullptr && r0 < rows_max) {
        const int r1 = min(r0 + R, rows_max);
        for (int c = tid; c < C; c += blockDim.x) {
            float mx = 0.0f;
            for (int r = r0; r < r1; ++r) {
                const float2 v = cut[(size_t)r * C + c];
                mx = fmaxf(mx, sqrtf(v.x * v.x + v.y * v.y));
            }
            cmax_part[(size_t)blockIdx.x * C + c] = mx;
        }
    }
    const int w = tid >> 5, lane = tid & 31;
    for (int m = r0 + w; m < min(r0 + R, M - 1); m += blockDim.x >> 5) {
        float2 s = make_float2(0.0f, 0.0f);
        for (int c = lane; c < C; c += 32) {
            const float2 a = cut[(size_t)m * C + c];
            const float2 b = cut[(size_t)(m + 1) * C + c];
            const float2 p = cmulc(a, b);
            s.x += p.x;
            s.y += p.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) dsum[m] = s;
    }
}

// Same Doppler sums on the U gathered bins: s[m] = sum_u conj(g[m,u]) g[m+1,u].
__global__ void __launch_bounds__(256)
k_af_doppler(const float2* __restrict__ cut, const int* __restrict__ bins, const int* __restrict__ fdec,
             int M, float2* __restrict__ dsum)
{
    const int U = fdec[1];
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int m = w;
    if (m >= M - 1) return;
    float2 s = make_float2(0.0f, 0.0f);
    for (int u = lane; u < U; u += 32) {
        const int b = bins[u];
        const float2 p = cmulc(cut[(size_t)m * C + b], cut[(size_t)(m + 1) * C + b]);
        s.x += p.x;
        s.y += p.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) dsum[m] = s;
}

// One CTA (1024 threads).  Optional target count (phase_adjustment.cu:180-194):
// colmax, mean with an int accumulator (Q3), threshold 1.48*mean.  Then the
// Doppler phase: psi = arg(s), Phi = inclusive scan, phase[0] = 0,
// phase[m+1] = exp(-j*Phi[m]) (phase_adjustment.cu:17-31).
// fdec: [0] tgt_num, [1] U.
__global__ void __launch_bounds__(1024)
k_fe_phase(const float* __restrict__ cmax_part, int nparts, const float2* __restrict__ dsum, int M,
           float2* __restrict__ phase, int* __restrict__ fdec)
{
    __shared__ double sc[1024];
    __shared__ int s_cnt[32];
    __shared__ long long s_sum[32];
    const int tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5;
    if (nparts > 0) {
        float mx = 0.0f;
        int iv = 0;
        if (tid < C) {
            for (int p = 0; p < nparts; ++p) mx = fmaxf(mx, cmax_part[(size_t)p * C + tid]);
            iv = (int)mx;
        }
        long long sum = iv;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) s_sum[w] = sum;
        __syncthreads();
        if (tid == 0) {
            long long t = 0;
            for (int i = 0; i < 32; ++i) t += s_sum[i];
            s_sum[0] = t;
        }
        __syncthreads();
        const float mean_val = (float)(int)s_sum[0] / (float)C;
        const float thr = 1.48f * mean_val;
        int cnt = (tid < C && mx > thr) ? 1 : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0) s_cnt[w] = cnt;
        __syncthreads();
        if (tid == 0) {
            int t = 0;
            for (int i = 0; i < 32; ++i) t += s_cnt[i];
            // U = nextPow2(tgt_num / 2) (common.cu:521-529)
            int n = t / 2, u = 1;
            while (n >> 1) {
                u <<= 1;
                n >>= 1;
            }
            fdec[0] = t;
            fdec[1] = u << 1;
        }
    }
    // inclusive scan of arg(s) in double
    double v = 0.0;
    if (tid < M - 1) {
        const float2 s = dsum[tid];
        v = (double)atan2f(s.y, s.x);
    }
    sc[tid] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        double add = (tid >= o) ? sc[tid - o] : 0.0;
        __syncthreads();
        sc[tid] += add;
        __syncthreads();
    }
    if (tid == 0) phase[0] = make_float2(0.0f, 0.0f);
    if (tid < M - 1) {
        double sn, cs;
        sincos(sc[tid], &sn, &cs);
        phase[tid + 1] = make_float2((float)cs, (float)-sn);
    }
}

// team reduction (sum) of a double over the T threads of a team.
template <int T>
__device__ __forceinline__ double team_sum(double v, int lt, double* red /* per-team, >= T/32 */)
{
    if constexpr (T >= 32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        constexpr int W = T / 32;
        if constexpr (W > 1) {
            if ((lt & 31) == 0) red[lt >> 5] = v;
            __syncthreads();
            double t = 0.0;
#pragma unroll
            for (int i = 0; i < W; ++i) t += red[i];
            __syncthreads();
            return t;
        }
        return v;
    } else {
#pragma unroll
        for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, T);
        return v;
    }
}

// Per column: FFT over pulses of phase[m]*cut[m,c], energy E = sum |X|^2 and
// entropy H = -sum p ln p, p = |X|^2/E (phase_adjustment.cu:215-246).
// CB columns per CTA, one team of M/16 threads per column.
template <int M, int CB>
__global__ void __launch_bounds__(CB * M / 16)
k_fe_colfft(const float2* __restrict__ cut, const float2* __restrict__ phase, double* __restrict__ E,
            double* __restrict__ H, const float2* __restrict__ tw)
{
    using F = FFTShape<M>;
    extern __shared__ float4 dyn_smem[];
    float2* smb = reinterpret_cast<float2*>(dyn_smem);
    __shared__ double red[CB][(F::T + 31) / 32];
    const int tid = threadIdx.x;
    const int team = tid / F::T, lt = tid % F::T;
    const int c0 = blockIdx.x * CB;
    float2* twt = smb + CB * F::SMEM;
    TwShared<M>::fill(twt, tw, tid, blockDim.x);
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int m = i / CB, cc = i % CB;
        smb[cc * F::SMEM + fpad(m)] = cmul(phase[m], cut[(size_t)m * C + c0 + cc]);
    }
    __syncthreads();
    float2* sm = smb + team * F::SMEM;
    float p[16];
    team_fft<M, false>([&](int i) { return sm[fpad(i)]; },
                       [&](int, float2 v, int slot) { p[slot] = v.x * v.x + v.y * v.y; }, sm, lt,
                       TwShared<M>{twt});
    // per-thread partials in float (16 terms), team sums in double
    float ep = 0.0f;
#pragma unroll
    for (int q = 0; q < 16; ++q) ep += p[q];
    const double e = team_sum<F::T>((double)ep, lt, red[team]);
    const float ef = (float)e;
    float hp = 0.0f;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const float x = p[q] / ef;
        hp += -(x * logf(x));
    }
    const double h = team_sum<F::T>((double)hp, lt, red[team]);
    if (lt == 0) {
        E[c0 + team] = e;
        H[c0 + team] = h;
    }
}

// One element per thread of a 512-thread CTA, sorted so that thread i ends
// with the i-th element in the strict order `before`: strides below 32 are
// exchanged by warp shuffles, larger ones through shared memory (10 of the
// 45 stages).  `before` must be a strict order; equal elements are
// interchangeable (they end in either of their places).
struct SelKey {
    double key;
    int tie;   // tie-break (smaller first)
    int val;   // payload
};
__device__ __forceinline__ SelKey shfl_xor_key(const SelKey& v, int j)
{
    SelKey w;
    w.key = __shfl_xor_sync(0xffffffffu, v.key, j);
    w.tie = __shfl_xor_sync(0xffffffffu, v.tie, j);
    w.val = __shfl_xor_sync(0xffffffffu, v.val, j);
    return w;
}
template <class Before>
__device__ __forceinline__ void sort512(SelKey& v, SelKey* sm, Before before)
{
    const int i = threadIdx.x;
    for (int k = 2; k <= C; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            SelKey w;
            if (j >= 32) {
                sm[i] = v;
                __syncthreads();
                w = sm[i ^ j];
                __syncthreads();
            } else {
                w = shfl_xor_key(v, j);
            }
            const bool up = (i & k) == 0;      // this region ascends in `before` order
            const bool lower = (i & j) == 0;   // i is the lower index of its pair
            const bool v_first = before(v, w);
            if (!((lower == up) ? v_first : !v_first)) v = w;
        }
}

// Bin selection (phase_adjustment.cu:248-264), one CTA of 512 threads, one
// column per thread: stable sort by energy (descending), keep tgt_num, stable
// sort by entropy (ascending), keep U (indices beyond tgt_num are 0, as
// device_vector::resize pads), sort the kept indices.  NaN keys sort last.
// The stable sorts are strict orders with the position as tie-break.
__global__ void __launch_bounds__(C)
k_fe_select(const double* __restrict__ E, const double* __restrict__ H, int* __restrict__ fdec,
            int* __restrict__ bins)
{
    __shared__ SelKey sm[C];
    const int tid = threadIdx.x;
    const int tgt = fdec[0], U = fdec[1];
    SelKey v;
    {
        const double e = E[tid];
        v.key = isnan(e) ? -CUDART_INF : e;
        v.tie = tid;
        v.val = tid;
    }
    sort512(v, sm, [](const SelKey& a, const SelKey& b) {
        return a.key > b.key || (a.key == b.key && a.tie < b.tie);
    });
    // second key: entropy of the first tgt entries; the rest are sentinels
    {
        double h = (tid < tgt) ? H[v.val] : CUDART_INF;
        if (isnan(h)) h = CUDART_INF;
        v.key = h;
        v.tie = (tid < tgt) ? tid : (C + tid);
    }
    sort512(v, sm, [](const SelKey& a, const SelKey& b) {
        return a.key < b.key || (a.key == b.key && a.tie < b.tie);
    });
    // keep U, pad with 0, sort ascending
    {
        int b = 0x7fffffff;
        if (tid < U) b = (tid < tgt) ? v.val : 0;
        v.key = 0.0;
        v.tie = 0;
        v.val = b;
    }
    sort512(v, sm, [](const SelKey& a, const SelKey& b) { return a.val < b.val; });
    if (tid < U) bins[tid] = v.val;
}

// Grid-wide barrier for cooperative launches (all CTAs co-resident): arrive
// on a monotonic counter and wait, with at most `limit` polls (kSpinLimit,
// about a second), until it reaches `target`.  A timeout sets *err and makes
// every later barrier fail fast, so that all CTAs leave the kernel.  Returns
// false on failure.
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned target, int* err, unsigned long long limit)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        int ok = 1;
        unsigned long long spins = 0;
        for (;;) {
            if (*(volatile unsigned*)count >= target) break;
            if (*(volatile int*)err) {
                ok = 0;
                break;
            }
            if (++spins > limit) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(40);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// All minimum-entropy iterations (phase_adjustment.cu:302-322) in one
// cooperative launch of G CTAs.  CTA b owns up to 4 of the U selected bins
// (one team of M/16 threads per bin), keeps them in shared memory, and per
// iteration computes t = phase .* g, T = FFT(t), T .* |T|, h = IFFT(T)/M,
// q = conj(g) .* h and writes its partial row sums to P[m][b].  After a grid
// barrier CTA b sums the rows m = b, b+G, ... over all partials and writes
// phase[m] = sigma / |sigma|; a second barrier publishes the new phase.
// phase: in the Doppler-tracking start, out the final phase.
template <int M>
__global__ void __launch_bounds__(4 * (M / 16))
k_af_persist(const float2* __restrict__ cut, const int* __restrict__ bins, const int* __restrict__ fdec,
             float2* phase, float2* P, unsigned* bar, int* err, int iters, const float2* __restrict__ tw,
             BarrierTest bt)
{
    using F = FFTShape<M>;
    constexpr int TEAMS = 4;
    extern __shared__ float4 dyn_smem[];
    float2* gs = reinterpret_cast<float2*>(dyn_smem);   // [TEAMS][M]
    float2* smb = gs + TEAMS * M;                        // [TEAMS][SMEM]
    float2* ph = smb + TEAMS * F::SMEM;                  // [M]
    float2* twt = ph + M;                                // twiddle table
    TwShared<M>::fill(twt, tw, threadIdx.x, blockDim.x);
    const TwShared<M> tws{twt};
    const int G = gridDim.x;
    const int U = fdec[1];
    const int cpc = (U + G - 1) / G;
    const int nact = (U + cpc - 1) / cpc;                 // CTAs that own bins
    const int tid = threadIdx.x;
    const int team = tid / F::T, lt = tid % F::T;
    const int u = blockIdx.x * cpc + team;
    const bool valid = team < cpc && u < U;
    float2* g = gs + team * M;
    float2* sm = smb + team * F::SMEM;
    {
        const int b = valid ? bins[u] : 0;
        for (int m = lt; m < M; m += F::T) g[m] = valid ? cut[(size_t)m * C + b] : make_float2(0.0f, 0.0f);
    }
    const float invM = 1.0f / (float)M;
    const int lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
#pragma unroll 1
    for (int it = 0; it < iters; ++it) {
        for (int m = tid; m < M; m += blockDim.x) ph[m] = __ldcg(&phase[m]);
        __syncthreads();
        if (blockIdx.x < nact) {
            team_fft<M, false>([&](int i) { return cmul(ph[i], g[i]); },
                               [&](int i, float2 v, int) { sm[fpad(i)] = cscale(v, sqrtf(v.x * v.x + v.y * v.y)); },
                               sm, lt, tws, valid);
            team_fft<M, true>([&](int i) { return sm[fpad(i)]; },
                              [&](int i, float2 v, int) { sm[fpad(i)] = cmulc(g[i], cscale(v, invM)); }, sm, lt,
                              tws, valid);
            __syncthreads();
            const int nt = min(cpc, U - (int)blockIdx.x * cpc);   // bins of this CTA
            for (int m = tid; m < M; m += blockDim.x) {
                float2 s = make_float2(0.0f, 0.0f);
                for (int t = 0; t < nt; ++t) {
                    const float2 q = smb[t * F::SMEM + fpad(m)];
                    s.x += q.x;
                    s.y += q.y;
                }
                __stcg(&P[(size_t)m * G + blockIdx.x], s);
            }
        }
        if (!grid_barrier(bar, (unsigned)(2 * it + 1) * G + bt.extra, err, bt.limit)) return;
        for (int m = blockIdx.x + warp * G; m < M; m += nwarp * G) {
            float2 s = make_float2(0.0f, 0.0f);
            for (int b = lane; b < nact; b += 32) {
                const float2 q = __ldcg(&P[(size_t)m * G + b]);
                s.x += q.x;
                s.y += q.y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
                s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
            }
            if (lane == 0) {
                const float a = sqrtf(s.x * s.x + s.y * s.y);
                __stcg(&phase[m], make_float2(s.x / a, s.y / a));
            }
        }
        if (!grid_barrier(bar, (unsigned)(2 * it + 2) * G + bt.extra, err, bt.limit)) return;
    }
}

// ---------------------------------------------------------------------------
// Cluster-resident autofocus: the same iteration as k_af_persist, with all
// state of one frame held in the shared memory of one thread-block cluster.
//
// CTA r of a cluster of CL owns bins [r*bpc, r*bpc + nb), bpc = ceil(U/CL),
// processed TEAMS at a time (one team of M/16 threads per bin).  Two chunk
// slots of TEAMS columns are cached in shared memory; a CTA owning more
// chunks reloads the ones past the first slot from the cut every iteration.
// Per iteration: each CTA accumulates P[m] = sum over its bins of
// conj(g) .* IFFT(T .* |T|)/M, T = FFT(phase .* g); cluster barrier; CTA r
// reduces rows [r*M/CL, (r+1)*M/CL) over the CL partials (distributed shared
// memory, fixed rank order), normalises and stores the new phase into every
// CTA's copy; cluster barrier.  The entropy of the selected bins,
// E = ln S1 - ln 2 * S2/S1 with S1 = sum |T|^2, S2 = sum |T|^2 log2 |T|^2, comes out of
// the same epilogue and drives the optional stop criterion.
// Only hardware cluster barriers: no spin-waits.
// ---------------------------------------------------------------------------
template <int M>
struct AFC {
    static constexpr int T = M / 16;
    static constexpr int TEAMS = 4096 / M;     // 256 threads per CTA
    static constexpr int THREADS = TEAMS * T;  // (two fused FFTs need ~255 registers: one CTA per SM)
    static constexpr int NSLOT = 4;            // cached columns per CTA: 16384 / M
    using Tw = TwShared<M, false, true>;       // two-level twiddles (80 entries at M = 1024)
    // phase copy + FFT scratch (also holds P and the reduction buffer between
    // sweeps) + column cache + twiddles: ~171 KB at M = 1024
    static constexpr size_t SMEM_F2 =
        (size_t)M + (size_t)TEAMS * FFTShape<M>::SMEM + (size_t)NSLOT * TEAMS * M + Tw::kEntries;
    static constexpr size_t SMEM = SMEM_F2 * sizeof(float2) + 64 * sizeof(double);
    static constexpr int PR = (M + THREADS - 1) / THREADS;   // partial-sum rows per thread
};

struct AFFrame {
    const float2* cut;     // [M][512]
    const int* bins;       // [U]
    const int* fdec;       // [1] = U
    float2* phase;         // [M] in: Doppler-tracking start phase, out: final phase
    int* stat;             // [0] iterations applied (both legs), [1] entropy bits of the
                           // selected bins at the last evaluated phase, [2] learned leg
                           // kept (set by the image judge), [3], [4] those entropy bits
                           // of the plain and the learned leg, [5], [6] their
                           // iterations; may be null
    float2* alt;           // [M] learned start phase in, the learned leg's final phase
                           // out (warm start), or null
    float2* gcol;          // [U][M] scratch: contiguous copy of the bin columns
};

// With a learned start (AFFrame::alt), both cluster engines run two legs: the
// autofocus from the learned start until the stop criterion (`tol`), then the
// plain autofocus, the reference's algorithm (Doppler-tracking start, `iters`
// updates, no stop criterion).  Both final phases are returned (alt, phase);
// the judge downstream images both and keeps the lower final image entropy,
// so a frame on which the learned start ends worse reverts to the plain
// result.  (The entropy of the selected bins cannot judge: it ignores a
// linear phase, a Doppler shift of the image, which MTRC does not.)

template <int M>
__global__ void __launch_bounds__(AFC<M>::THREADS, 1)
k_af_cluster(AFFrame f, int iters, float tol, const float2* __restrict__ tw)
{
    namespace cg = cooperative_groups;
    using A = AFC<M>;
    using F = FFTShape<M>;
    using TwA = typename A::Tw;
    cg::cluster_group cl = cg::this_cluster();
    const int CL = (int)cl.num_blocks();
    const int r = (int)cl.block_rank();
    extern __shared__ float4 dyn_smem[];
    float2* ph = reinterpret_cast<float2*>(dyn_smem);   // [M]
    float2* smb = ph + M;                                // [TEAMS][SMEM]; between sweeps: P [M], buf
    float2* P = smb;
    float2* cache = smb + A::TEAMS * F::SMEM;            // [NSLOT][TEAMS][M]
    float2* twt = cache + (size_t)A::NSLOT * A::TEAMS * M;   // twiddle table
    double* red = reinterpret_cast<double*>(twt + TwA::kEntries);   // [64]
    const TwA tws{twt};
    const int tid = threadIdx.x;
    TwA::fill(twt, tw, tid, A::THREADS);
    const int team = tid / F::T, lt = tid % F::T;
    const int lane = tid & 31, warp = tid >> 5;
    const int U = f.fdec[1];
    const int bpc = (U + CL - 1) / CL;
    const int b0 = r * bpc;
    const int nb = max(0, min(bpc, U - b0));
    const int nch = (nb + A::TEAMS - 1) / A::TEAMS;
    const bool reload = nch > A::NSLOT;
    float2* sm = smb + team * F::SMEM;

    auto load_chunk = [&](int j, int slot) {
        const int t = j * A::TEAMS + team;
        float2* g = cache + ((size_t)slot * A::TEAMS + team) * M;
        if (t < nb) {
            const int b = f.bins[b0 + t];
            for (int m = lt; m < M; m += F::T) g[m] = f.cut[(size_t)m * C + b];
        }
    };
    for (int m = tid; m < M; m += A::THREADS) ph[m] = f.phase[m];
    for (int j = 0; j < min(nch, A::NSLOT); ++j) load_chunk(j, j);
    __syncthreads();

    const float invM = 1.0f / (float)M;
    const int rows = M / CL;

    // One sweep over this CTA's bins with the phase in ph: entropy sums
    // (s1, s2, only when `ent`) and, when `full`, the partial row sums of the
    // update, accumulated in registers and left in P (the start of the FFT
    // scratch) for the cluster reduction.
    auto sweep = [&](bool full, bool ent, float& s1, float& s2) {
        float2 pacc[A::PR];
#pragma unroll
        for (int k = 0; k < A::PR; ++k) pacc[k] = make_float2(0.0f, 0.0f);
#pragma unroll 1
        for (int j = 0; j < nch; ++j) {
            const int slot = j < A::NSLOT ? j : A::NSLOT - 1;
            if (reload && j >= A::NSLOT - 1) {
                __syncthreads();
                load_chunk(j, slot);
            }
            __syncthreads();
            const float2* g = cache + ((size_t)slot * A::TEAMS + team) * M;
            const bool valid = j * A::TEAMS + team < nb;
            team_fft<M, false>([&](int i) { return cmul(ph[i], g[i]); },
                               [&](int i, float2 v, int) {
                                   const float p = v.x * v.x + v.y * v.y;
                                   if (ent) {
                                       s1 += p;
                                       if (p > 0.0f) s2 += p * __log2f(p);
                                   }
                                   sm[fpad(i)] = cscale(v, sqrtf(p));
                               },
                               sm, lt, tws, valid);
            if (!full) continue;
            team_fft<M, true>([&](int i) { return sm[fpad(i)]; },
                              [&](int i, float2 v, int) { sm[fpad(i)] = cmulc(g[i], cscale(v, invM)); }, sm, lt,
                              tws, valid);
            const int nt = min(A::TEAMS, nb - j * A::TEAMS);
#pragma unroll
            for (int k = 0; k < A::PR; ++k) {
                const int m = tid + k * A::THREADS;
                if (m < M)
                    for (int t = 0; t < nt; ++t) {
                        const float2 q = smb[t * F::SMEM + fpad(m)];
                        pacc[k].x += q.x;
                        pacc[k].y += q.y;
                    }
            }
        }
        if (full) {
            __syncthreads();   // every team is done with the scratch
#pragma unroll
            for (int k = 0; k < A::PR; ++k) {
                const int m = tid + k * A::THREADS;
                if (m < M) P[m] = pacc[k];
            }
        }
    };

    // Entropy of the selected bins from the per-thread sums of one sweep:
    // float per warp, double per CTA (red[32..33]) and per cluster, by thread
    // 0 of every CTA in the same order (FP64 is slow on this part).  The
    // cluster barrier inside publishes red[32..33]; the caller's next cluster
    // barrier must come before they are rewritten.  Returns the value in
    // thread 0.
    auto entropy_sums = [&](float s1, float s2) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            red[warp] = s1;
            red[16 + warp] = s2;
        }
        __syncthreads();
        if (tid == 0) {
            double a1 = 0.0, a2 = 0.0;
            for (int w = 0; w < A::THREADS / 32; ++w) {
                a1 += red[w];
                a2 += red[16 + w];
            }
            red[32] = a1;
            red[33] = a2;
        }
        cl.sync();
        float E = 0.0f;
        if (tid == 0) {
            double S1 = 0.0, S2 = 0.0;
            for (int q = 0; q < CL; ++q) {
                const double* rr = cl.map_shared_rank(red, q);
                S1 += rr[32];
                S2 += rr[33];
            }
            E = logf((float)S1) - kLn2 * (float)S2 / (float)S1;
        }
        return E;
    };

    // One autofocus run from the phase in ph: up to `iters` updates, fewer
    // when the stop criterion ends it.  Returns (in thread 0) the entropy at
    // the last evaluated phase or, with want_final, of the final phase (one
    // more entropy sweep when all `iters` updates were applied).
    auto leg = [&](bool want_final, float ltol, int& used) -> float {
        float e_prev = 0.0f, e_last = 0.0f;   // meaningful in thread 0
        bool stopped = false;
        used = iters;
#pragma unroll 1
        for (int it = 0; it < iters; ++it) {
            // the entropy is needed by the stop criterion, and for the trace at
            // the last iteration; elsewhere its logarithms are skipped
            const bool check = ltol > 0.0f && it % kStopEvery == 0;
            const bool need_e = check || it == iters - 1;
            float s1 = 0.0f, s2 = 0.0f;
            sweep(true, need_e, s1, s2);
            const float E = entropy_sums(s1, s2);
            if (tid == 0) {
                bool stop = false;
                if (need_e) {
                    if (check) {
                        stop = it > 0 && fabsf(E - e_prev) <= (float)kStopEvery * ltol * fabsf(E);
                        e_prev = E;
                    }
                    e_last = E;
                }
                red[40] = stop ? 1.0 : 0.0;
            }
            // This CTA's rows [r*rows, (r+1)*rows) of every CTA's partial sums,
            // gathered with independent remote loads into buf[q][row] (behind P).
            float2* buf = smb + M;
            for (int idx = tid; idx < CL * rows; idx += A::THREADS) {
                const int q = idx / rows, ml = idx - q * rows;
                buf[idx] = cl.map_shared_rank(P, q)[r * rows + ml];
            }
            __syncthreads();
            const bool stop = red[40] != 0.0;
            if (!stop) {
                for (int ml = tid; ml < rows; ml += A::THREADS) {
                    float2 s = make_float2(0.0f, 0.0f);
                    for (int q = 0; q < CL; ++q) {
                        const float2 v = buf[q * rows + ml];
                        s.x += v.x;
                        s.y += v.y;
                    }
                    const float a = sqrtf(s.x * s.x + s.y * s.y);
                    buf[CL * rows + ml] = make_float2(s.x / a, s.y / a);
                }
                __syncthreads();
                for (int idx = tid; idx < CL * rows; idx += A::THREADS) {
                    const int q = idx / rows, ml = idx - q * rows;
                    cl.map_shared_rank(ph, q)[r * rows + ml] = buf[CL * rows + ml];
                }
            }
            cl.sync();
            if (stop) {
                used = it;
                stopped = true;
                break;
            }
        }
        if (want_final && !stopped) {
            float s1 = 0.0f, s2 = 0.0f;
            sweep(false, true, s1, s2);
            const float E = entropy_sums(s1, s2);
            if (tid == 0) e_last = E;
            cl.sync();   // red[32..33] are read remotely before a later sweep rewrites them
        }
        return e_last;
    };

    if (!f.alt) {
        int used;
        const float e = leg(false, tol, used);
        for (int m = r * rows + tid; m < (r + 1) * rows; m += A::THREADS) f.phase[m] = ph[m];
        if (r == 0 && tid == 0 && f.stat) {
            f.stat[0] = used;
            f.stat[1] = __float_as_int(e);
        }
        return;
    }
    // the learned leg, then the plain leg (see AFFrame)
    __syncthreads();
    for (int m = tid; m < M; m += A::THREADS) ph[m] = f.alt[m];
    __syncthreads();
    int used_l, used_d;
    const float e_l = leg(false, tol, used_l);
    for (int m = r * rows + tid; m < (r + 1) * rows; m += A::THREADS) f.alt[m] = ph[m];
    __syncthreads();
    for (int m = tid; m < M; m += A::THREADS) ph[m] = f.phase[m];
    __syncthreads();
    const float e_d = leg(false, 0.0f, used_d);
    for (int m = r * rows + tid; m < (r + 1) * rows; m += A::THREADS) f.phase[m] = ph[m];
    if (r == 0 && tid == 0 && f.stat) {
        f.stat[0] = used_l + used_d;
        f.stat[1] = __float_as_int(e_d);
        f.stat[2] = 0;
        f.stat[3] = __float_as_int(e_d);
        f.stat[4] = __float_as_int(e_l);
        f.stat[5] = used_d;
        f.stat[6] = used_l;
    }
}

// ---------------------------------------------------------------------------
// k_af_cluster for M = 1024 on warp-level FFTs (warp_fft1024): one warp per
// bin, 8 bins per round per CTA.  Element m of a bin lives in lane m % 32,
// register m / 32 through the forward transform, the T |T| epilogue and the
// inverse transform (conj-forward-conj); the transposes go through the
// warp's own tile, so no block barrier sits inside a sweep.  Per-warp partial
// row sums accumulate in registers across rounds and are reduced over the
// CTA's warps in fixed order; the cluster reduction, stop criterion and the
// choice of start are those of k_af_cluster.
// ---------------------------------------------------------------------------
struct AFW {
    static constexpr int M = 1024;
    static constexpr int WARPS = 8;
    static constexpr int THREADS = WARPS * 32;
    static constexpr int TILE = 32 * 33;       // per-warp transpose tile (float2)
    static constexpr int NSLOT = 2;            // cached rounds: 16 bins per CTA
    static constexpr size_t SMEM_F2 = (size_t)M + (size_t)WARPS * TILE + (size_t)NSLOT * WARPS * M + M;
    static constexpr size_t SMEM = SMEM_F2 * sizeof(float2) + 64 * sizeof(double);
};

// Each warp keeps NSLOT of its bins in shared memory; when the CTA has more,
// the others are read from gcol, a contiguous copy of the
// gathered columns ([U][M], written by the loading warp itself on entry), and
// successive sweeps alternate direction so that the NSLOT rounds left in
// shared memory by one sweep are the first of the next.
__global__ void __launch_bounds__(AFW::THREADS, 1)
k_af_cluster_w1024(AFFrame f, int iters, float tol, const float2* __restrict__ tw)
{
    namespace cg = cooperative_groups;
    constexpr int M = AFW::M;
    cg::cluster_group cl = cg::this_cluster();
    const int CL = (int)cl.num_blocks();
    const int r = (int)cl.block_rank();
    extern __shared__ float4 dyn_smem[];
    float2* ph = reinterpret_cast<float2*>(dyn_smem);          // [M]
    float2* tiles = ph + M;                                     // [WARPS][TILE]; between sweeps P, buf
    float2* cache = tiles + AFW::WARPS * AFW::TILE;             // [NSLOT][WARPS][M]
    float2* TWL = cache + (size_t)AFW::NSLOT * AFW::WARPS * M;  // [32][32] W^(lane k)
    double* red = reinterpret_cast<double*>(TWL + M);           // [64]
    float2* P = tiles;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < M; i += AFW::THREADS) TWL[i] = tw[(i >> 5) * (i & 31) * (kTwN / M)];
    float2* tile = tiles + warp * AFW::TILE;
    const int U = f.fdec[1];
    const int bpc = (U + CL - 1) / CL;
    const int b0 = r * bpc;
    const int nb = max(0, min(bpc, U - b0));
    const int nrd = (nb + AFW::WARPS - 1) / AFW::WARPS;
    const bool reload = nrd > AFW::NSLOT;
    float2* gw = f.gcol + (size_t)(b0 + warp) * M;   // this warp's bin of round 0

    for (int m = tid; m < M; m += AFW::THREADS) ph[m] = f.phase[m];
    // every bin of this warp: cached rounds into their slot, all rounds into
    // gcol when some must be re-read
    for (int j = 0; j < nrd; ++j) {
        const int t = j * AFW::WARPS + warp;
        if (t >= nb || (j >= AFW::NSLOT && !reload)) continue;
        const int b = f.bins[b0 + t];
        float2* g = cache + ((size_t)(j % AFW::NSLOT) * AFW::WARPS + warp) * M;
        float2* gg = gw + (size_t)j * AFW::WARPS * M;
        for (int m = lane; m < M; m += 32) {
            const float2 x = f.cut[(size_t)m * C + b];
            if (j < AFW::NSLOT) g[m] = x;
            if (reload) gg[m] = x;
        }
    }
    __syncthreads();

    const float invM = 1.0f / (float)M;
    const int rows = M / CL;
    int nsweep = 0;

    // One sweep with the phase in ph; see k_af_cluster.
    auto sweep = [&](bool full, bool ent, float& s1, float& s2) {
        float2 pacc[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) pacc[k] = make_float2(0.0f, 0.0f);
        const bool back = (nsweep++ & 1) != 0;
#pragma unroll 1
        for (int jj = 0; jj < nrd; ++jj) {
            const int j = back ? nrd - 1 - jj : jj;
            if (j * AFW::WARPS + warp >= nb) continue;   // warp-uniform; no block barrier inside
            float2* g = cache + ((size_t)(j % AFW::NSLOT) * AFW::WARPS + warp) * M;
            if (jj >= AFW::NSLOT) {   // only when reload: read the copy in gcol
                const float4* src = reinterpret_cast<const float4*>(gw + (size_t)j * AFW::WARPS * M);
                float4* dst = reinterpret_cast<float4*>(g);
#pragma unroll 4
                for (int i = lane; i < M / 2; i += 32) dst[i] = src[i];
                __syncwarp();
            }
            float2 v[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k] = cmul(ph[lane + 32 * k], g[lane + 32 * k]);
            // pass 0: T = FFT(phase * g); pass 1: conj(IFFT(T |T|)) * M as the
            // forward FFT of conj(T |T|).  One copy of the transform's code
            // (a loop, not unrolled) keeps the kernel within the instruction
            // cache.
#pragma unroll 1
            for (int pass = 0; pass < (full ? 2 : 1); ++pass) {
                warp_fft1024(v, lane, tile, TWL);
                if (pass == 0) {
#pragma unroll
                    for (int k = 0; k < 32; ++k) {
                        const float p = v[k].x * v[k].x + v[k].y * v[k].y;
                        if (ent) {
                            s1 += p;
                            if (p > 0.0f) s2 += p * __log2f(p);
                        }
                        const float a = p > 0.0f ? p * rsqrtf(p) : 0.0f;
                        v[k] = make_float2(v[k].x * a, -v[k].y * a);   // conj(T |T|)
                    }
                } else {
                    // conj(g) conj(v) / M = conj(g v) / M: g v accumulates
                    // here, the conjugate and 1/M are applied once per sweep
#pragma unroll
                    for (int k = 0; k < 32; ++k) {
                        const float2 q = g[lane + 32 * k];
                        pacc[k].x = fmaf(q.x, v[k].x, fmaf(-q.y, v[k].y, pacc[k].x));
                        pacc[k].y = fmaf(q.x, v[k].y, fmaf(q.y, v[k].x, pacc[k].y));
                    }
                }
            }
            __syncwarp();   // slot reuse by a later reload
        }
        if (full) {
            __syncthreads();   // every warp is done with its tile
#pragma unroll
            for (int k = 0; k < 32; ++k) tile[lane + 32 * k] = make_float2(pacc[k].x * invM, -pacc[k].y * invM);
            __syncthreads();
            for (int m = tid; m < M; m += AFW::THREADS) {
                float2 s = tiles[m];
#pragma unroll
                for (int w = 1; w < AFW::WARPS; ++w) {
                    const float2 q = tiles[w * AFW::TILE + m];
                    s.x += q.x;
                    s.y += q.y;
                }
                P[m] = s;
            }
        }
    };

    // Entropy of the selected bins, in two halves around a cluster barrier:
    // this CTA's sums (s1 = sum p, s2 = sum p log2 p) into red[32..33], then
    // after the barrier warp 0 adds the CL CTAs' sums (one remote read per
    // lane, a fixed-order tree: every CTA gets the same value) and returns
    // ln S1 - ln 2 * S2 / S1 in lane 0 of warp 0.
    auto entropy_part = [&](float s1, float s2) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            red[warp] = s1;
            red[16 + warp] = s2;
        }
        __syncthreads();
        if (tid == 0) {
            double a1 = 0.0, a2 = 0.0;
            for (int w = 0; w < AFW::WARPS; ++w) {
                a1 += red[w];
                a2 += red[16 + w];
            }
            red[32] = a1;
            red[33] = a2;
        }
    };
    auto entropy_total = [&]() {   // warp 0, after the cluster barrier
        double S1 = 0.0, S2 = 0.0;
        if (lane < CL) {
            const double* rr = cl.map_shared_rank(red, lane);
            S1 = rr[32];
            S2 = rr[33];
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            S1 += __shfl_xor_sync(0xffffffffu, S1, o);
            S2 += __shfl_xor_sync(0xffffffffu, S2, o);
        }
        return logf((float)S1) - kLn2 * (float)S2 / (float)S1;
    };

    // One autofocus run from the phase in ph (see k_af_cluster): returns, in
    // warp 0, the entropy at the last evaluated phase or, with want_final, of
    // the final phase.
    float2* buf = tiles + AFW::TILE;   // behind P (tile 0 holds P)
    auto leg = [&](bool want_final, float ltol, int& used) -> float {
        float e_prev = 0.0f, e_last = 0.0f;   // meaningful in warp 0
        bool stopped = false;
        used = iters;
        int lg_rows = 0;
        while ((1 << lg_rows) < rows) ++lg_rows;
#pragma unroll 1
        for (int it = 0; it < iters; ++it) {
            // the entropy is needed by the stop criterion or for the last trace
            const bool check = ltol > 0.0f && it % kStopEvery == 0;
            const bool need_e = check || it == iters - 1;
            float s1 = 0.0f, s2 = 0.0f;
            sweep(true, need_e, s1, s2);
            if (need_e) entropy_part(s1, s2);
            cl.sync();   // P and red[32..33] of every CTA are complete
            if (warp == 0) {
                bool stop = false;
                if (need_e) {
                    const float E = entropy_total();
                    if (check) {
                        stop = it > 0 && fabsf(E - e_prev) <= (float)kStopEvery * ltol * fabsf(E);
                        e_prev = E;
                    }
                    e_last = E;
                }
                if (lane == 0) red[40] = stop ? 1.0 : 0.0;
            }
            // this CTA's rows of the cluster sum: slice r of every CTA's P
#pragma unroll
            for (int i = 0; i < M / AFW::THREADS; ++i) {
                const int idx = tid + i * AFW::THREADS;
                const int q = idx >> lg_rows, ml = idx & (rows - 1);
                buf[idx] = cl.map_shared_rank(P, q)[r * rows + ml];
            }
            __syncthreads();
            const bool stop = red[40] != 0.0;
            if (!stop) {
                for (int ml = tid; ml < rows; ml += AFW::THREADS) {
                    float2 s = make_float2(0.0f, 0.0f);
                    for (int q = 0; q < CL; ++q) {
                        const float2 v = buf[q * rows + ml];
                        s.x += v.x;
                        s.y += v.y;
                    }
                    const float a = sqrtf(s.x * s.x + s.y * s.y);
                    buf[M + ml] = make_float2(s.x / a, s.y / a);
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < M / AFW::THREADS; ++i) {
                    const int idx = tid + i * AFW::THREADS;
                    const int q = idx >> lg_rows, ml = idx & (rows - 1);
                    cl.map_shared_rank(ph, q)[r * rows + ml] = buf[M + ml];
                }
            }
            cl.sync();
            if (stop) {
                used = it;
                stopped = true;
                break;
            }
        }
        if (want_final && !stopped) {
            float s1 = 0.0f, s2 = 0.0f;
            sweep(false, true, s1, s2);
            entropy_part(s1, s2);
            cl.sync();
            if (warp == 0) e_last = entropy_total();
            cl.sync();   // red[32..33] are read remotely before a later sweep rewrites them
        }
        return e_last;
    };

    if (!f.alt) {
        int used;
        const float e = leg(false, tol, used);
        for (int m = r * rows + tid; m < (r + 1) * rows; m += AFW::THREADS) f.phase[m] = ph[m];
        if (r == 0 && tid == 0 && f.stat) {
            f.stat[0] = used;
            f.stat[1] = __float_as_int(e);
        }
        return;
    }
    // the learned leg, then the plain leg (see AFFrame)
    __syncthreads();
    for (int m = tid; m < M; m += AFW::THREADS) ph[m] = f.alt[m];
    __syncthreads();
    int used_l, used_d;
    const float e_l = leg(false, tol, used_l);
    for (int m = r * rows + tid; m < (r + 1) * rows; m += AFW::THREADS) f.alt[m] = ph[m];
    __syncthreads();
    for (int m = tid; m < M; m += AFW::THREADS) ph[m] = f.phase[m];
    __syncthreads();
    const float e_d = leg(false, 0.0f, used_d);
    for (int m = r * rows + tid; m < (r + 1) * rows; m += AFW::THREADS) f.phase[m] = ph[m];
    if (r == 0 && tid == 0 && f.stat) {
        f.stat[0] = used_l + used_d;
        f.stat[1] = __float_as_int(e_d);
        f.stat[2] = 0;
        f.stat[3] = __float_as_int(e_d);
        f.stat[4] = __float_as_int(e_l);
        f.stat[5] = used_d;
        f.stat[6] = used_l;
    }
}

// cut[m][c] *= phase[m]  (phase_adjustment.cu:324)
__global__ void k_af_apply(float2* __restrict__ cut, const float2* __restrict__ phase, int M)
{
    const int m = blockIdx.x;
    const float2 p = phase[m];
    for (int c = threadIdx.x; c < C; c += blockDim.x) cut[(size_t)m * C + c] = cmul(p, cut[(size_t)m * C + c]);
}

// Both legs of a warm-started frame in one pass: cut2 = diag(phase_l) cut
// (the learned leg), then cut = diag(phase) cut in place (the plain leg).
__global__ void k_af_apply2(float2* __restrict__ cut, const float2* __restrict__ phase,
                            const float2* __restrict__ phase_l, float2* __restrict__ cut2, int M)
{
    const int m = blockIdx.x;
    const float2 p = phase[m], pl = phase_l[m];
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        const float2 x = cut[(size_t)m * C + c];
        cut2[(size_t)m * C + c] = cmul(pl, x);
        cut[(size_t)m * C + c] = cmul(p, x);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int M>
static constexpr int af_cb() { return M >= 512 ? 8 : (M >= 256 ? 16 : 32); }

// The cluster engine's kernel for M pulses: warp-level FFTs at M = 1024,
// team FFTs otherwise.
template <int M>
struct AfEngine {
    static constexpr bool kWarp = M == 1024;
    static constexpr int THREADS = kWarp ? AFW::THREADS : AFC<M>::THREADS;
    static constexpr size_t SMEM = kWarp ? AFW::SMEM : AFC<M>::SMEM;
    using Fn = void (*)(AFFrame, int, float, const float2*);
    static Fn kernel()
    {
        if constexpr (kWarp) return k_af_cluster_w1024;
        else return k_af_cluster<M>;
    }
};

// Cluster engine set-up (once per device): shared-memory limit, non-portable
// cluster sizes, and the largest of 16/8/4 CTAs per cluster that can be
// resident.  Returns that size, 0 if none, or a negative cudaError_t.
template <int M>
static int af_cluster_probe()
{
    using A = AfEngine<M>;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(A::kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)A::SMEM)))
        return -(int)e;
    if ((e = cudaFuncSetAttribute(A::kernel(), cudaFuncAttributeNonPortableClusterSizeAllowed, 1))) {
        (void)cudaGetLastError();
    }
    int best = 0;
    for (int cl = 16; cl >= 4 && best == 0; cl >>= 1) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(cl);
        cfg.blockDim = dim3(A::THREADS);
        cfg.dynamicSmemBytes = A::SMEM;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, A::kernel(), &cfg) == cudaSuccess && n > 0) best = cl;
        (void)cudaGetLastError();
    }
    return best;
}

template <int M>
static int af_cluster_setup()
{
    static PerDevice max_cl;
    return max_cl.get(af_cluster_probe<M>);
}

template <int M>
static cudaError_t af_cluster_launch(const FEArgs& a, cudaStream_t st)
{
    using A = AfEngine<M>;
    const int mx = af_cluster_setup<M>();
    if (mx < 0) return (cudaError_t)(-mx);
    const int cl = a.af_cluster;
    if (cl != 4 && cl != 8 && cl != 16) return cudaErrorInvalidValue;
    if (cl > mx) return cudaErrorInvalidClusterSize;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cl);
    cfg.blockDim = dim3(A::THREADS);
    cfg.dynamicSmemBytes = A::SMEM;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    AFFrame fr{a.cut, a.bins, a.fdec, a.phase, a.af_stat, a.ws_w ? a.ws_phase : nullptr, a.gcol};
    cudaError_t e = cudaLaunchKernelEx(&cfg, A::kernel(), fr, a.iters, a.tol, a.tw);
    if (e == cudaSuccess) ISAR_COUNT(1);
    return e;
}

int af_cluster_max(int M)
{
    int r = 0;
    switch (M) {
    case 128: r = af_cluster_setup<128>(); break;
    case 256: r = af_cluster_setup<256>(); break;
    case 512: r = af_cluster_setup<512>(); break;
    case 1024: r = af_cluster_setup<1024>(); break;
    default: return 0;
    }
    return r < 0 ? 0 : r;
}

template <int M>
static cudaError_t fe_run_m(const FEArgs& a, cudaStream_t st)
{
    constexpr int CB = af_cb<M>();
    using F = FFTShape<M>;
    const size_t smem = ((size_t)CB * F::SMEM + TwShared<M>::kEntries) * sizeof(float2);
    const size_t smem_p = (size_t)4 * M * sizeof(float2) + (size_t)4 * F::SMEM * sizeof(float2) + M * sizeof(float2) +
                          TwShared<M>::kEntries * sizeof(float2);
    // per device: shared-memory limits, and whether the cooperative grid of
    // 128 CTAs (at most 4 of the <= 512 bins each) can be co-resident
    static PerDevice setup;
    const int su = setup.get([smem, smem_p]() -> int {
        cudaError_t e;
        if ((e = cudaFuncSetAttribute(k_fe_colfft<M, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
            return -(int)e;
        if ((e = cudaFuncSetAttribute(k_af_persist<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p)))
            return -(int)e;
        int dev = 0, sms = 0, per_sm = 0;
        if ((e = cudaGetDevice(&dev))) return -(int)e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return -(int)e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_af_persist<M>, 4 * F::T, smem_p)))
            return -(int)e;
        return per_sm * sms;
    });
    if (su < 0) return (cudaError_t)(-su);
    constexpr int grid_p = 128;
    if (su < grid_p) return cudaErrorCooperativeLaunchTooLarge;
    const int rows_max = M < 256 ? M : 256;
    const int R = 8;
    const int nparts = (rows_max + R - 1) / R;
    k_fe_stats<<<(M + R - 1) / R, 256, 0, st>>>(a.cut, M, rows_max, R, a.cmax_part, a.dsum);
    ISAR_COUNT(1);
    k_fe_phase<<<1, 1024, 0, st>>>(a.cmax_part, nparts, a.dsum, M, a.phase, a.fdec);
    ISAR_COUNT(1);
    k_fe_colfft<M, CB><<<C / CB, CB * F::T, smem, st>>>(a.cut, a.phase, a.E, a.H, a.tw);
    ISAR_COUNT(1);
    k_fe_select<<<1, C, 0, st>>>(a.E, a.H, a.fdec, a.bins);
    ISAR_COUNT(1);
    k_af_doppler<<<(M * 32 + 255) / 256, 256, 0, st>>>(a.cut, a.bins, a.fdec, M, a.dsum);
    ISAR_COUNT(1);
    k_fe_phase<<<1, 1024, 0, st>>>(nullptr, 0, a.dsum, M, a.phase, a.fdec);
    ISAR_COUNT(1);
    if (a.pre_only) return cudaGetLastError();
    if (a.ws_w && (a.af_cluster == 0 || a.iters == 0)) return cudaErrorInvalidValue;
    if (a.ws_w) {
        // learned warm start: features -> network -> second start phase
        cudaError_t e;
        if ((e = nn::features(a.cut, a.E, a.dsum, M, a.ws_a->act[0], a.ws_psi, st))) return e;
        if ((e = nn::forward(*a.ws_w, *a.ws_a, 1, M, a.ws_err, st))) return e;
        if ((e = nn::ws_phase(a.ws_psi, a.ws_a->out, M, a.ws_phase, st))) return e;
    }
    if (a.iters > 0 && a.af_cluster > 0) {
        cudaError_t e = af_cluster_launch<M>(a, st);
        if (e) return e;
    } else if (a.iters > 0) {
        cudaError_t e;
        if ((e = cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned), st))) return e;
        const float2* cut = a.cut;
        const int* bins = a.bins;
        const int* fdec = a.fdec;
        float2* phase = a.phase;
        float2* P = a.sig_part;
        unsigned* bar = a.bar;
        int* err = reinterpret_cast<int*>(a.bar + 1);
        int iters = a.iters;
        const float2* tw = a.tw;
        BarrierTest bt = a.bar_test;
        void* args[] = {(void*)&cut, (void*)&bins, (void*)&fdec, (void*)&phase, (void*)&P,
                        (void*)&bar, (void*)&err, (void*)&iters, (void*)&tw, (void*)&bt};
        if ((e = cudaLaunchCooperativeKernel((const void*)k_af_persist<M>, dim3(grid_p), dim3(4 * F::T), args, smem_p,
                                             st)))
            return e;
        ISAR_COUNT(1);
    }
    if (a.defer_apply) return cudaGetLastError();   // the imaging applies the phase(s)
    if (a.ws_w && a.iters > 0 && a.af_cluster > 0)
        k_af_apply2<<<M, 256, 0, st>>>(a.cut, a.phase, a.ws_phase, a.cut2, M);
    else
        k_af_apply<<<M, 256, 0, st>>>(a.cut, a.phase, M);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t fe_run(const FEArgs& a, cudaStream_t st)
{
    switch (a.M) {
    case 128: return fe_run_m<128>(a, st);
    case 256: return fe_run_m<256>(a, st);
    case 512: return fe_run_m<512>(a, st);
    case 1024: return fe_run_m<1024>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace isar
