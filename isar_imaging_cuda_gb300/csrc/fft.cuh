// Block-level FFT engine: power-of-two complex64 FFTs held in shared memory
// and registers.  A "team" of N/16 threads owns one transform; a CTA may run
// several teams side by side (each with its own shared-memory slice), all in
// lockstep.
//
// Algorithm: Stockham auto-sort, radix-16 passes followed by one radix-2/4/8
// pass when log2(N) is not a multiple of 4.  Pass p with radix R and
// Ns = product of the earlier radices maps j in [0, N/R), k = j mod Ns:
//   a[r]  = in[j + r*N/R]
//   a[r] *= W_{Ns*R}^{r*k}                                  (twiddle table)
//   a     = DFT_R(a)                                        (registers)
//   out[(j/Ns)*Ns*R + k + r*Ns] = a[r]
// The first pass reads through a caller functor (fused pre-multiply), the last
// pass hands each output (index, value, register slot) to a caller functor
// (fused epilogue).  Shared-memory slots are padded by one element every 16
// to keep the stride-16 writes of the first pass conflict free.
//
// Conventions as cuFFT: forward = exp(-i), inverse = exp(+i), unnormalised.
#pragma once

#include "isar_common.cuh"

namespace isar {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }

template <int N>
struct FFTShape {
    static constexpr int T = N / 16;                 // threads per team
    static constexpr int LOG = ilog2c(N);
    static constexpr int NP16 = LOG / 4;             // radix-16 passes
    static constexpr int REM = LOG % 4;
    static constexpr int NPASS = NP16 + (REM ? 1 : 0);
    static constexpr int SMEM = N + N / 16;          // float2 slots per team
};

// d * exp(-+2*pi*i*j/R) with j, R compile-time after unrolling (R <= 16).
template <bool INV>
__device__ __forceinline__ float2 twc_mul(float2 d, int j, int R)
{
    const int k16 = j * (16 / R);   // angle = 2*pi*k16/16, k16 in [0, 8)
    const float c1 = 0.92387953251128674f, c2 = 0.70710678118654752f, c3 = 0.38268343236508977f;
    float c, s;
    switch (k16) {
    case 0: return d;
    case 4: return INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
    case 1: c = c1; s = c3; break;
    case 2: c = c2; s = c2; break;
    case 3: c = c3; s = c1; break;
    case 5: c = -c3; s = c1; break;
    case 6: c = -c2; s = c2; break;
    default: c = -c1; s = c3; break;   // 7
    }
    // forward: (c - i s), inverse: (c + i s)
    if (INV) return make_float2(d.x * c - d.y * s, d.x * s + d.y * c);
    return make_float2(d.x * c + d.y * s, d.y * c - d.x * s);
}

// In-register DFT of length R (2..16): radix-2 decimation in frequency, then
// the bit-reversal permutation (register renaming after unrolling).
template <int R, bool INV>
__device__ __forceinline__ void dft_reg(float2* a)
{
#pragma unroll
    for (int len = R; len >= 2; len >>= 1) {
        const int half = len >> 1;
#pragma unroll
        for (int s = 0; s < R; s += len) {
#pragma unroll
            for (int k = 0; k < half; ++k) {
                float2 u = a[s + k], v = a[s + k + half];
                a[s + k] = cadd(u, v);
                a[s + k + half] = twc_mul<INV>(csub(u, v), k * (R / len), R);
            }
        }
    }
    float2 b[R];
#pragma unroll
    for (int i = 0; i < R; ++i) b[i] = a[i];
    constexpr int L = ilog2c(R);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        int r = 0;
#pragma unroll
        for (int q = 0; q < L; ++q) r |= ((i >> q) & 1) << (L - 1 - q);
        a[i] = b[r];
    }
}

// Twiddle sources: tw(e, N) = exp(-2 pi i e / N), 0 <= e < N.
// TwGlobal reads the global kTwN-entry table through the read-only cache.
struct TwGlobal {
    const float2* __restrict__ p;
    __device__ __forceinline__ float2 operator()(int e, int n) const { return __ldg(&p[e * (kTwN / n)]); }
};

// TwShared<N>: a per-CTA shared-memory table.  For N <= 2048 (or FULL) it
// holds all N twiddles; above that (or with TWO) a two-level table
// hi[e >> 6] * lo[e & 63] (N/64 + 64 entries, one extra complex multiply,
// ~1 ulp more rounding).
template <int N, bool FULL = false, bool TWO = false>
struct TwShared {
    static constexpr bool kTwoLevel = TWO || (!FULL && N > 2048);
    static constexpr int kEntries = kTwoLevel ? N / 64 + 64 : N;
    const float2* p;
    __device__ __forceinline__ float2 operator()(int e, int) const
    {
        if constexpr (kTwoLevel) {
            const float2 h = p[e >> 6], l = p[N / 64 + (e & 63)];
            return make_float2(h.x * l.x - h.y * l.y, h.x * l.y + h.y * l.x);
        } else {
            return p[e];
        }
    }
    // Fills the table from the global kTwN table; all threads of the CTA call
    // it, followed by a __syncthreads() before first use.
    __device__ __forceinline__ static void fill(float2* t, const float2* __restrict__ g, int tid, int nthreads)
    {
        if constexpr (kTwoLevel) {
            for (int i = tid; i < N / 64; i += nthreads) t[i] = g[(i * 64) * (kTwN / N)];
            for (int i = tid; i < 64; i += nthreads) t[N / 64 + i] = g[i * (kTwN / N)];
        } else {
            for (int i = tid; i < N; i += nthreads) t[i] = g[i * (kTwN / N)];
        }
    }
};

template <class Tw>
struct TwTwoLevel {
    static constexpr bool value = false;
};
template <int N, bool F, bool T>
struct TwTwoLevel<TwShared<N, F, T>> {
    static constexpr bool value = TwShared<N, F, T>::kTwoLevel;
};

// No-op hook of team_fft.
struct NoHook {
    __device__ __forceinline__ void operator()() const {}
};

template <int N, int R, int NS, bool INV, bool FIRST, bool LAST, class Src, class Dst, class Tw, class Hook>
__device__ __forceinline__ void fft_pass(Src& src, Dst& dst, float2* sm, int lt, const Tw& tw, bool active,
                                         Hook& hook)
{
    constexpr int T = N / 16;
    constexpr int B = 16 / R;
    float2 v[16];
    if (active) {
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int j = lt + b * T;
            // fpad(j + r*K) = fpad(j) + r*K*17/16 when K is a multiple of 16
            const int pj = fpad(j);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int idx = j + r * (N / R);
                if constexpr (FIRST) v[b * R + r] = src(idx);
                else if constexpr ((N / R) % 16 == 0) v[b * R + r] = sm[pj + r * ((N / R) + (N / R) / 16)];
                else v[b * R + r] = sm[fpad(idx)];
            }
        }
    }
    // Both barriers of a pass are executed by every thread: teams narrower than
    // a warp share warps, so a barrier inside `if (active)` would diverge.
    __syncthreads();
    if constexpr (FIRST) hook();   // every src() read of the CTA is done
    if (active) {
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int j = lt + b * T;
            const int k = j & (NS - 1);
            if constexpr (NS > 1 && R == 16 && TwTwoLevel<Tw>::value) {
                // two-level table: look up W^k, W^2k, W^4k, W^8k and form the
                // others as products (depth <= 3): 8 shared loads instead of 30
                constexpr int s = N / (NS * R);
                float2 w[16];
                w[1] = tw(k * s, N);
                w[2] = tw(2 * k * s, N);
                w[4] = tw(4 * k * s, N);
                w[8] = tw(8 * k * s, N);
                w[3] = cmul(w[2], w[1]);
                w[5] = cmul(w[4], w[1]);
                w[6] = cmul(w[4], w[2]);
                w[7] = cmul(w[4], w[3]);
#pragma unroll
                for (int r = 9; r < 16; ++r) w[r] = cmul(w[8], w[r - 8]);
#pragma unroll
                for (int r = 1; r < 16; ++r) {
                    float2 x = w[r];
                    if (INV) x.y = -x.y;
                    v[b * R + r] = cmul(v[b * R + r], x);
                }
            } else if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = tw((r * k) * (N / (NS * R)), N);
                    if (INV) w.y = -w.y;
                    v[b * R + r] = cmul(v[b * R + r], w);
                }
            }
            dft_reg<R, INV>(&v[b * R]);
            const int base = (j / NS) * NS * R + k;
            const int pb = fpad(base);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int idx = base + r * NS;
                if constexpr (LAST) dst(idx, v[b * R + r], b * R + r);
                else if constexpr (NS % 16 == 0) sm[pb + r * (NS + NS / 16)] = v[b * R + r];
                else if constexpr (NS == 1 && R == 16) sm[pb + r] = v[b * R + r];   // base = 16 j
                else sm[fpad(idx)] = v[b * R + r];
            }
        }
    }
    __syncthreads();
}

template <int N, bool INV, int PASS, int NS, class Src, class Dst, class Tw, class Hook>
__device__ __forceinline__ void fft_passes(Src& src, Dst& dst, float2* sm, int lt, const Tw& tw, bool active,
                                           Hook& hook)
{
    using S = FFTShape<N>;
    constexpr int R = (PASS < S::NP16) ? 16 : (1 << S::REM);
    fft_pass<N, R, NS, INV, PASS == 0, PASS == S::NPASS - 1>(src, dst, sm, lt, tw, active, hook);
    if constexpr (PASS + 1 < S::NPASS) fft_passes<N, INV, PASS + 1, NS * R>(src, dst, sm, lt, tw, active, hook);
}

// One team transform.  src(i) -> float2 for i in [0,N) (first pass, may read
// global memory); dst(i, v, slot) receives output i (slot in [0,16) is the
// register slot, fixed per thread and output index).  sm: this team's slice
// of FFTShape<N>::SMEM float2.  lt: thread index within the team.
// A team with active == false does no work but keeps the barriers.
// Contains __syncthreads(): every thread of the CTA must call it.
// tw: the global kTwN table (TwGlobal) or a TwShared<N> accessor.
// hook() runs in every thread once all src() reads of the CTA are done
// (after the first pass's load barrier), e.g. to refill the source buffer.
template <int N, bool INV, class Src, class Dst, class Tw, class Hook = NoHook>
__device__ __forceinline__ void team_fft(Src src, Dst dst, float2* sm, int lt, const Tw& tw, bool active = true,
                                         Hook hook = Hook{})
{
    static_assert(N >= 32 && (N & (N - 1)) == 0 && N <= kTwN, "FFT size");
    fft_passes<N, INV, 0, 1>(src, dst, sm, lt, tw, active, hook);
}

template <int N, bool INV, class Src, class Dst>
__device__ __forceinline__ void team_fft(Src src, Dst dst, float2* sm, int lt, const float2* __restrict__ tw,
                                         bool active = true)
{
    team_fft<N, INV>(src, dst, sm, lt, TwGlobal{tw}, active);
}

// ---------------------------------------------------------------------------
// Row transforms of the range alignment.  At N = 8192 a CTA of 512 threads
// runs the transform as 16 x 512: one radix-16 pass over the whole CTA
// (thread t takes x[t + 512 r], r < 16, and multiplies by W_8192^(t k0)),
// one exchange through shared memory, then sixteen independent 512-point
// transforms, one per warp (warp k0 takes row k0): a 16-point DFT in
// registers over m1 (t = m0 + 32 m1, m0 = lane), the twiddles W_512^(m0 k1),
// a transpose through the warp's own part of the scratch (__syncwarp only),
// a 16-point DFT over b (m0 = 2 b + a) and a radix-2 step between lanes
// l and l ^ 16 (shuffles).  Two block barriers per transform instead of the
// eight of the four-pass Stockham transform.
// Output X[k0 + 16 k1 + 256 q + 4096 a] lands in register slot q of lane
// k1 + 16 a of warp k0.
// ---------------------------------------------------------------------------

// Twiddles of row_fft<N>: the two-level table of TwShared<N>, followed at
// N = 8192 by the step twiddles W_512^(m k) of the warp transforms at
// [32 k + m] (k < 16, m < 32).
template <int N>
struct RowTw {
    using Two = TwShared<N>;
    static constexpr int kStep = N == 8192 ? 512 : 0;
    static constexpr int kEntries = Two::kEntries + kStep;
    const float2* p;
    __device__ __forceinline__ float2 operator()(int e, int n) const { return Two{p}(e, n); }
    __device__ __forceinline__ float2 step(int k, int m) const { return p[Two::kEntries + 32 * k + m]; }
    __device__ __forceinline__ static void fill(float2* t, const float2* __restrict__ g, int tid, int nthreads)
    {
        Two::fill(t, g, tid, nthreads);
        if constexpr (kStep > 0)
            for (int i = tid; i < kStep; i += nthreads)
                t[Two::kEntries + i] = g[(((i >> 5) * (i & 31) * 16) & (N - 1)) * (kTwN / N)];
    }
};
template <int N>
struct TwTwoLevel<RowTw<N>> {
    static constexpr bool value = TwShared<N>::kTwoLevel;
};

// 8192-point transform, one CTA of 512 threads (see above).  sm: 16 x 544
// float2 (FFTShape<8192>::SMEM).  src(i) is called for i = lt + 512 r in
// order r = 0..15 and must not read sm; dst(i, v, slot) must not write sm.
// Contains __syncthreads(): every thread of the CTA must call it.
template <bool INV, class Src, class Dst, class Hook>
__device__ __forceinline__ void fft8192(Src& src, Dst& dst, float2* sm, int lt, const RowTw<8192>& tw, Hook& hook)
{
    constexpr int N = 8192;
    constexpr int RS = 544;   // scratch row stride (float2)
    const int lane = lt & 31, w = lt >> 5;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = src(lt + 512 * r);
    __syncthreads();   // the previous transform's warps are done with the scratch
    hook();
    dft_reg<16, INV>(v);
    {
        // W_8192^(lt k0): look up k0 = 1, 2, 4, 8, form the others as products
        float2 t[16];
        t[1] = tw(lt, N);
        t[2] = tw(2 * lt, N);
        t[4] = tw(4 * lt, N);
        t[8] = tw(8 * lt, N);
        t[3] = cmul(t[2], t[1]);
        t[5] = cmul(t[4], t[1]);
        t[6] = cmul(t[4], t[2]);
        t[7] = cmul(t[4], t[3]);
#pragma unroll
        for (int k = 9; k < 16; ++k) t[k] = cmul(t[8], t[k - 8]);
#pragma unroll
        for (int k = 1; k < 16; ++k) {
            float2 x = t[k];
            if (INV) x.y = -x.y;
            v[k] = cmul(v[k], x);
        }
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) sm[k * RS + lt] = v[k];
    __syncthreads();
    float2* row = sm + w * RS;
#pragma unroll
    for (int m1 = 0; m1 < 16; ++m1) v[m1] = row[lane + 32 * m1];
    dft_reg<16, INV>(v);
#pragma unroll
    for (int k = 1; k < 16; ++k) {
        float2 x = tw.step(k, lane);
        if (INV) x.y = -x.y;
        v[k] = cmul(v[k], x);
    }
    __syncwarp();   // the row is read: the tile may overwrite it
#pragma unroll
    for (int k = 0; k < 16; ++k) row[lane * 17 + k] = v[k];
    __syncwarp();
    const int k1 = lane & 15, a = lane >> 4;
#pragma unroll
    for (int b = 0; b < 16; ++b) v[b] = row[(2 * b + a) * 17 + k1];
    dft_reg<16, INV>(v);
    const float c[16] = {1.000000000f,  0.980785280f,  0.923879533f,  0.831469612f, 0.707106781f,  0.555570233f,
                         0.382683432f,  0.195090322f,  0.000000000f,  -0.195090322f, -0.382683432f, -0.555570233f,
                         -0.707106781f, -0.831469612f, -0.923879533f, -0.980785280f};
    const float s[16] = {0.000000000f, 0.195090322f, 0.382683432f, 0.555570233f, 0.707106781f, 0.831469612f,
                         0.923879533f, 0.980785280f, 1.000000000f, 0.980785280f, 0.923879533f, 0.831469612f,
                         0.707106781f, 0.555570233f, 0.382683432f, 0.195090322f};
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        float2 o;
        o.x = __shfl_xor_sync(0xffffffffu, v[q].x, 16);
        o.y = __shfl_xor_sync(0xffffffffu, v[q].y, 16);
        const float2 d0 = a ? o : v[q], d1 = a ? v[q] : o;
        const float sn = INV ? s[q] : -s[q];   // W_32^q (forward), conj for the inverse
        const float2 t = make_float2(d1.x * c[q] - d1.y * sn, d1.x * sn + d1.y * c[q]);
        const float2 y = a ? csub(d0, t) : cadd(d0, t);
        dst(w + 16 * k1 + 256 * q + 4096 * a, y, q);
    }
}

// Row transform used by the range alignment: with WARP, fft8192 at
// N = 8192; otherwise the Stockham team transform (same src / dst / hook
// contract).  fft8192 hands the outputs of a warp to dst with a stride of 16
// elements across lanes, so kernels that store the transformed rows keep the
// team transform (its outputs are lane-contiguous, stores coalesce).
template <int N, bool INV, bool WARP, class Src, class Dst, class Hook>
__device__ __forceinline__ void row_fft(Src src, Dst dst, float2* sm, int lt, const RowTw<N>& tw, Hook hook)
{
    if constexpr (WARP && N == 8192) fft8192<INV>(src, dst, sm, lt, tw, hook);
    else team_fft<N, INV>(src, dst, sm, lt, tw, true, hook);
}

// Output index of register slot `slot` of thread lt for row_fft<N, *, WARP>.
template <int N, bool WARP>
__device__ __forceinline__ int row_out_index(int lt, int slot);

// Output index of register slot `slot` for thread lt (the LAST pass mapping),
// so that callers can revisit their outputs after the transform.
template <int N>
__device__ __forceinline__ int fft_out_index(int lt, int slot)
{
    using S = FFTShape<N>;
    constexpr int R = (S::NPASS - 1 < S::NP16) ? 16 : (1 << S::REM);
    const int b = slot / R, r = slot % R;
    return lt + b * S::T + r * (N / R);
}

template <int N, bool WARP>
__device__ __forceinline__ int row_out_index(int lt, int slot)
{
    if constexpr (WARP && N == 8192) {
        const int lane = lt & 31;
        return (lt >> 5) + 16 * (lane & 15) + 256 * slot + 4096 * (lane >> 4);
    } else {
        return fft_out_index<N>(lt, slot);
    }
}

// ---------------------------------------------------------------------------
// Warp-level 1024-point FFT (forward, unnormalised).  Lane l holds element
// l + 32 r in register r (r = 0..31), before and after the transform.
// Four-step: a 32-point DFT over the registers, the twiddles W_1024^(l k),
// a transpose of the warp's 32 x 32 block through a shared tile (row stride
// 33, __syncwarp only), and a second 32-point DFT over the registers.  No
// block barrier, so the warps of a CTA run their transforms independently.
// ---------------------------------------------------------------------------

// In-register 32-point forward DFT, natural order in and out:
// X[k] = E[k] + W32^k O[k], X[k + 16] = E[k] - W32^k O[k] with E, O the
// 16-point DFTs of the even and odd elements.
__device__ __forceinline__ void dft32_reg(float2* a)
{
    const float c[16] = {1.000000000f,  0.980785280f,  0.923879533f,  0.831469612f, 0.707106781f,  0.555570233f,
                         0.382683432f,  0.195090322f,  0.000000000f,  -0.195090322f, -0.382683432f, -0.555570233f,
                         -0.707106781f, -0.831469612f, -0.923879533f, -0.980785280f};
    const float s[16] = {0.000000000f, 0.195090322f, 0.382683432f, 0.555570233f, 0.707106781f, 0.831469612f,
                         0.923879533f, 0.980785280f, 1.000000000f, 0.980785280f, 0.923879533f, 0.831469612f,
                         0.707106781f, 0.555570233f, 0.382683432f, 0.195090322f};
    float2 e[16], o[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        e[i] = a[2 * i];
        o[i] = a[2 * i + 1];
    }
    dft_reg<16, false>(e);
    dft_reg<16, false>(o);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        // o[k] * exp(-j 2 pi k / 32)
        const float2 t = make_float2(o[k].x * c[k] + o[k].y * s[k], o[k].y * c[k] - o[k].x * s[k]);
        a[k] = cadd(e[k], t);
        a[k + 16] = csub(e[k], t);
    }
}

// TWL: W_1024^(l k) at TWL[32 k + l] (l, k < 32) in shared memory, read
// lane-contiguous (conflict-free); tile: this warp's 32 x 33 float2.
// v[k] holds x[lane + 32 k] on entry and X[lane + 32 k] on return.
__device__ __forceinline__ void warp_fft1024(float2* v, int lane, float2* tile, const float2* TWL)
{
    // two 32-point DFT steps sharing one copy of the code
#pragma unroll 1
    for (int step = 0; step < 2; ++step) {
        dft32_reg(v);
        if (step == 1) break;
#pragma unroll
        for (int k = 1; k < 32; ++k) v[k] = cmul(v[k], TWL[32 * k + lane]);
#pragma unroll
        for (int k = 0; k < 32; ++k) tile[lane * 33 + k] = v[k];
        __syncwarp();
#pragma unroll
        for (int n = 0; n < 32; ++n) v[n] = tile[n * 33 + lane];
        __syncwarp();
    }
}

}  // namespace isar
