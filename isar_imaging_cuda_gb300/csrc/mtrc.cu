// CZT-based MTRC correction and image formation on the M x 512 cut.
// Reference: mtrc.cu:4-76 (mtrc), :125-172 (cztRange, Bluestein),
// isar_main.cu:191-211 (post-processing).
#include <cuda_runtime.h>

#include "fft.cuh"
#include "isar_kernels.h"

namespace isar {

constexpr int C = kRangeCut;

// Rows: ifftshift then IFFT/512 (STRETCH) or FFT (IFDS) (mtrc.cu:18-40).
template <bool INV>
__global__ void __launch_bounds__(256) k_mtrc_rows(const float2* __restrict__ cut, float2* __restrict__ st,
                                                   const float2* __restrict__ tw)
{
    using F = FFTShape<C>;
    __shared__ float2 smb[8 * F::SMEM];
    const int team = threadIdx.x / F::T, lt = threadIdx.x % F::T;
    const int m = blockIdx.x * 8 + team;
    const float2* xr = cut + (size_t)m * C;
    float2* o = st + (size_t)m * C;
    const float sc = INV ? 1.0f / (float)C : 1.0f;
    team_fft<C, INV>([&](int i) { return xr[(i + C / 2) & (C - 1)]; },
                     [&](int i, float2 v, int) { o[i] = cscale(v, sc); }, smb + team * F::SMEM, lt, tw);
}

// Bluestein CZT along pulses for CB range bins (mtrc.cu:125-172):
// y = pre .* x (zero padded to L), Y = FFT_L(y) .* V, y = IFFT_L(Y)/L,
// out[k] = y[M-1+k] * post[k].
// COLMEAN (M >= 512): the rest of the reference's chain up to the image's
// magnitude is, per column a of the CZT output, ifftshift / IFFT / M /
// fftshift (mtrc.cu:53-61), a row FFT (:63-66), the column fftshift (:69),
// the window on row 0 (isar_main.cu:192; hamming[c / M] = hamming[0] for
// every column c < 512 when M >= 512) and FFT / fftshift over pulses
// (isar_main.cu:193-201).  The row FFT commutes with the column operations,
// and the column operations collapse to a - (1 - hamming[0]) * mean(a):
// FFT(IFFT(z)/M with element 0 scaled by h) = z + (h - 1) mean(z), and the
// shifts cancel.  So this kernel writes a - (1 - hamming[0]) mean(a)
// (flipped up-down for IFDS, isar_main.cu:201-204) and the row transform
// k_mtrc_rowfft_abs forms the image.  (With M < 512 the window's factor
// differs between columns and the full chain runs.)
// phase (may be null): the autofocus phase of pulse k, applied here instead
// of to the cut (the rows' transform before this kernel is linear per row).
template <int M, int CB, bool COLMEAN = false>
__global__ void __launch_bounds__(CB * (2 * M) / 16)
k_czt(const float2* __restrict__ st, const float2* __restrict__ pre, const float2* __restrict__ post,
      const float2* __restrict__ V, float2* __restrict__ out, const float2* __restrict__ tw,
      const float* __restrict__ hamM = nullptr, int flipud = 0, const float2* __restrict__ phase = nullptr)
{
    constexpr int L = 2 * M;
    using F = FFTShape<L>;
    extern __shared__ float4 dyn_smem[];
    float2* smb = reinterpret_cast<float2*>(dyn_smem);
    float2* tile = smb + CB * F::SMEM;   // [M][CB]
    const int tid = threadIdx.x;
    const int team = tid / F::T, lt = tid % F::T;
    const int c0 = blockIdx.x * CB;
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int k = i / CB, cc = i % CB;
        const size_t g = (size_t)k * C + c0 + cc;
        const float2 v = cmul(pre[g], st[g]);
        tile[i] = phase ? cmul(v, phase[k]) : v;
    }
    __syncthreads();
    float2* sm = smb + team * F::SMEM;
    const int c = c0 + team;
    const float2* Vc = V + (size_t)c * L;
    const float invL = 1.0f / (float)L;
    team_fft<L, false>([&](int i) { return i < M ? tile[i * CB + team] : make_float2(0.0f, 0.0f); },
                       [&](int i, float2 v, int) { sm[fpad(i)] = cmul(v, Vc[i]); }, sm, lt, tw);
    team_fft<L, true>([&](int i) { return sm[fpad(i)]; },
                      [&](int i, float2 v, int) {
                          const int k = i - (M - 1);
                          if (k >= 0 && k < M) tile[k * CB + team] = cscale(v, invL);
                      },
                      sm, lt, tw);
    __syncthreads();
    if constexpr (!COLMEAN) {
        for (int i = tid; i < M * CB; i += blockDim.x) {
            const int k = i / CB, cc = i % CB;
            const size_t g = (size_t)k * C + c0 + cc;
            out[g] = cmul(tile[i], post[g]);
        }
    } else {
        static_assert((CB * (2 * M) / 16) % CB == 0 && CB <= 32, "a thread keeps one column");
        __shared__ double2 red[CB * (2 * M) / 16 / 32][CB];
        __shared__ float2 sub[CB];
        // a = y * post in place; this thread's column is tid % CB
        double sx = 0.0, sy = 0.0;
        for (int i = tid; i < M * CB; i += blockDim.x) {
            const int k = i / CB, cc = i % CB;
            const float2 v = cmul(tile[i], post[(size_t)k * C + c0 + cc]);
            tile[i] = v;
            sx += v.x;
            sy += v.y;
        }
#pragma unroll
        for (int o = 16; o >= CB; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
        }
        const int lane = tid & 31, w = tid >> 5;
        if (lane < CB) red[w][lane] = make_double2(sx, sy);
        __syncthreads();
        if (tid < CB) {
            double ax = 0.0, ay = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
                ax += red[q][tid].x;
                ay += red[q][tid].y;
            }
            const double f = (1.0 - (double)__ldg(&hamM[0])) / (double)M;
            sub[tid] = make_float2((float)(ax * f), (float)(ay * f));
        }
        __syncthreads();
        for (int i = tid; i < M * CB; i += blockDim.x) {
            const int k = i / CB, cc = i % CB;
            const int r = flipud ? M - 1 - k : k;
            const float2 v = tile[i], d = sub[cc];
            out[(size_t)r * C + c0 + cc] = make_float2(v.x - d.x, v.y - d.y);
        }
    }
}

// Columns: ifftshift, IFFT/M, ifftshift (mtrc.cu:53-61).
template <int M, int CB>
__global__ void __launch_bounds__(CB * M / 16)
k_mtrc_cols(const float2* __restrict__ in, float2* __restrict__ out, const float2* __restrict__ tw)
{
    using F = FFTShape<M>;
    extern __shared__ float4 dyn_smem[];
    float2* smb = reinterpret_cast<float2*>(dyn_smem);
    const int tid = threadIdx.x;
    const int team = tid / F::T, lt = tid % F::T;
    const int c0 = blockIdx.x * CB;
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int m = i / CB, cc = i % CB;
        smb[cc * F::SMEM + fpad(m)] = in[(size_t)((m + M / 2) & (M - 1)) * C + c0 + cc];
    }
    __syncthreads();
    float2* sm = smb + team * F::SMEM;
    const float invM = 1.0f / (float)M;
    team_fft<M, true>([&](int i) { return sm[fpad(i)]; },
                      [&](int i, float2 v, int) { sm[fpad((i + M / 2) & (M - 1))] = cscale(v, invM); }, sm, lt,
                      tw);
    __syncthreads();
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int m = i / CB, cc = i % CB;
        out[(size_t)m * C + c0 + cc] = smb[cc * F::SMEM + fpad(m)];
    }
}

// Rows: FFT(512), fftshift (mtrc.cu:63-66); IFDS adds fliplr (:72-75).
__global__ void __launch_bounds__(256) k_mtrc_rowfft(const float2* __restrict__ in, float2* __restrict__ out,
                                                     int fliplr, const float2* __restrict__ tw)
{
    using F = FFTShape<C>;
    __shared__ float2 smb[8 * F::SMEM];
    const int team = threadIdx.x / F::T, lt = threadIdx.x % F::T;
    const int m = blockIdx.x * 8 + team;
    const float2* xr = in + (size_t)m * C;
    float2* o = out + (size_t)m * C;
    team_fft<C, false>([&](int i) { return xr[i]; },
                       [&](int i, float2 v, int) {
                           int d = (i + C / 2) & (C - 1);
                           if (fliplr) d = C - 1 - d;
                           o[d] = v;
                       },
                       smb + team * F::SMEM, lt, tw);
}

// The image from the column-corrected MTRC rows (see k_czt, COLMEAN):
// |fftshift(FFT(row))| per row, IFDS flipped left-right (mtrc.cu:63-75).
__global__ void __launch_bounds__(256) k_mtrc_rowfft_abs(const float2* __restrict__ in, float* __restrict__ img,
                                                         int fliplr, const float2* __restrict__ tw)
{
    using F = FFTShape<C>;
    __shared__ float2 smb[8 * F::SMEM];
    const int team = threadIdx.x / F::T, lt = threadIdx.x % F::T;
    const int m = blockIdx.x * 8 + team;
    const float2* xr = in + (size_t)m * C;
    float* o = img + (size_t)m * C;
    team_fft<C, false>([&](int i) { return xr[i]; },
                       [&](int i, float2 v, int) {
                           int d = (i + C / 2) & (C - 1);
                           if (fliplr) d = C - 1 - d;
                           o[d] = sqrtf(v.x * v.x + v.y * v.y);
                       },
                       smb + team * F::SMEM, lt, tw);
}

// Post-processing per column: (optional column fftshift of the input),
// Hamming over pulses, FFT over pulses, fftshift, (IFDS: flipud), |.|.
// The reference's window launch (isar_main.cu:192) hands diagMulMat
// cols = echo_num, len = range_num_cut, so only element i < 512 (row 0) is
// scaled, by hamming[i / echo_num]; the other rows stay unwindowed.
template <int M, int CB>
__global__ void __launch_bounds__(CB * M / 16)
k_post(const float2* __restrict__ cut, int src_shift, const float* __restrict__ hamM, int flipud,
       float* __restrict__ img, const float2* __restrict__ tw)
{
    using F = FFTShape<M>;
    extern __shared__ float4 dyn_smem[];
    float2* smb = reinterpret_cast<float2*>(dyn_smem);
    float* tile = reinterpret_cast<float*>(smb + CB * F::SMEM);   // [M][CB]
    const int tid = threadIdx.x;
    const int team = tid / F::T, lt = tid % F::T;
    const int c0 = blockIdx.x * CB;
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int m = i / CB, cc = i % CB;
        const float2 v = cut[(size_t)((m + src_shift) & (M - 1)) * C + c0 + cc];
        smb[cc * F::SMEM + fpad(m)] = (m == 0) ? cscale(v, hamM[(c0 + cc) / M]) : v;
    }
    __syncthreads();
    float2* sm = smb + team * F::SMEM;
    team_fft<M, false>([&](int i) { return sm[fpad(i)]; },
                       [&](int i, float2 v, int) {
                           int r = (i + M / 2) & (M - 1);
                           if (flipud) r = M - 1 - r;
                           tile[r * CB + team] = sqrtf(v.x * v.x + v.y * v.y);
                       },
                       sm, lt, tw);
    __syncthreads();
    for (int i = tid; i < M * CB; i += blockDim.x) {
        const int m = i / CB, cc = i % CB;
        img[(size_t)m * C + c0 + cc] = tile[i];
    }
}

template <int M>
static constexpr int col_cb() { return M >= 512 ? 8 : (M >= 256 ? 16 : 32); }
template <int M>
static constexpr int czt_cb() { return M >= 512 ? 4 : (M >= 256 ? 8 : 16); }

template <int M>
static cudaError_t post_run_m(const PostArgs& a, cudaStream_t st)
{
    constexpr int CB = col_cb<M>();
    constexpr int CZ = czt_cb<M>();
    using F = FFTShape<M>;
    using FL = FFTShape<2 * M>;
    const size_t smem_post = (size_t)CB * F::SMEM * sizeof(float2) + (size_t)M * CB * sizeof(float);
    const size_t smem_cols = (size_t)CB * F::SMEM * sizeof(float2);
    const size_t smem_czt = (size_t)CZ * FL::SMEM * sizeof(float2) + (size_t)M * CZ * sizeof(float2);
    static PerDevice attr;   // shared-memory limits, set once per device
    const int ar = attr.get([smem_post, smem_cols, smem_czt]() -> int {
        cudaError_t e;
        if ((e = cudaFuncSetAttribute(k_post<M, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_post)))
            return -(int)e;
        if ((e = cudaFuncSetAttribute(k_mtrc_cols<M, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem_cols)))
            return -(int)e;
        if ((e = cudaFuncSetAttribute(k_czt<M, CZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_czt)))
            return -(int)e;
        if constexpr (M >= 512)
            if ((e = cudaFuncSetAttribute(k_czt<M, CZ, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem_czt)))
                return -(int)e;
        return 0;
    });
    if (ar < 0) return (cudaError_t)(-ar);
    int src_shift = 0;
    const float2* src = a.cut;
    if ((a.phase || a.rows_ready) && !(a.mtrc && M >= 512)) return cudaErrorInvalidValue;
    if (a.mtrc) {
        if (!a.rows_ready) {
            if (a.data_type == 1) k_mtrc_rows<false><<<M / 8, 256, 0, st>>>(a.cut, a.st, a.tw);
            else k_mtrc_rows<true><<<M / 8, 256, 0, st>>>(a.cut, a.st, a.tw);
            ISAR_COUNT(1);
        }
        if constexpr (M >= 512) {
            // the column IFFT, window and column FFT as one column correction
            // (see k_czt, COLMEAN), then the rows form the image; st is only
            // read from here on, so a second leg reuses it (rows_ready)
            k_czt<M, CZ, true><<<C / CZ, CZ * FL::T, smem_czt, st>>>(a.st, a.pre, a.post, a.V, a.st2, a.tw,
                                                                      a.hamM, a.data_type == 1, a.phase);
            ISAR_COUNT(1);
            k_mtrc_rowfft_abs<<<M / 8, 256, 0, st>>>(a.st2, a.img, a.data_type == 1, a.tw);
            ISAR_COUNT(1);
            return cudaGetLastError();
        }
        k_czt<M, CZ><<<C / CZ, CZ * FL::T, smem_czt, st>>>(a.st, a.pre, a.post, a.V, a.st2, a.tw);
        ISAR_COUNT(1);
        k_mtrc_cols<M, CB><<<C / CB, CB * F::T, smem_cols, st>>>(a.st2, a.st, a.tw);
        ISAR_COUNT(1);
        k_mtrc_rowfft<<<M / 8, 256, 0, st>>>(a.st, a.st2, a.data_type == 1, a.tw);
        ISAR_COUNT(1);
        src = a.st2;
        src_shift = M / 2;   // final column fftshift of mtrc (mtrc.cu:69)
    }
    k_post<M, CB><<<C / CB, CB * F::T, smem_post, st>>>(src, src_shift, a.hamM, a.data_type == 1, a.img, a.tw);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t post_run(const PostArgs& a, cudaStream_t st)
{
    switch (a.M) {
    case 128: return post_run_m<128>(a, st);
    case 256: return post_run_m<256>(a, st);
    case 512: return post_run_m<512>(a, st);
    case 1024: return post_run_m<1024>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------
// Judge of a warm-started frame.  Final image entropy (the project's
// definition, as the bench measures it): E = -sum p ln p with p = I^2 / S,
// S = sum I^2, i.e. E = ln S - ln 2 * T / S with T = sum I^2 log2 I^2 (the
// hardware base-2 logarithm).  Float sums per thread, double across warps
// and CTAs; CTA b of image i (blockIdx.y) writes its (S, T) partials to
// part[(i * kJudgeParts + b) * 2].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_img_entropy_part(const float* __restrict__ img, const float* __restrict__ img_l,
                                                          int n, double* __restrict__ part)
{
    __shared__ double red[2][8];
    const float* x = blockIdx.y ? img_l : img;
    float s = 0.0f, t = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = x[i];
        const float p = v * v;
        s += p;
        if (p > 0.0f) t += p * __log2f(p);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][w] = s;
        red[1][w] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, T = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {   // fixed order
            S += red[0][i];
            T += red[1][i];
        }
        double* q = part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 2;
        q[0] = S;
        q[1] = T;
    }
}

// Every CTA forms both entropies from the partials in the same order (warp 0:
// a lane per partial slice, then a fixed xor tree, so every CTA takes the
// same decision) and copies its slice of img_l over img when the learned
// leg's entropy is lower; NaN keeps the plain leg.
__global__ void __launch_bounds__(256) k_img_select(float* __restrict__ img, const float* __restrict__ img_l, int n,
                                                    const double* __restrict__ part, int* stat)
{
    __shared__ int s_keep;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double v[4] = {0.0, 0.0, 0.0, 0.0};   // S, T of the plain leg, S, T of the learned leg
        for (int b = lane; b < kJudgeParts; b += 32)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                v[2 * i] += part[(i * kJudgeParts + b) * 2];
                v[2 * i + 1] += part[(i * kJudgeParts + b) * 2 + 1];
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        if (lane == 0) {
            const float ln2 = 0.693147180559945309f;
            const float e = logf((float)v[0]) - ln2 * (float)(v[1] / v[0]);
            const float el = logf((float)v[2]) - ln2 * (float)(v[3] / v[2]);
            s_keep = el < e ? 1 : 0;
            if (blockIdx.x == 0 && stat) {
                stat[2] = s_keep;
                if (s_keep) stat[1] = stat[4];
            }
        }
    }
    __syncthreads();
    if (!s_keep) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) img[i] = img_l[i];
}

cudaError_t img_judge(float* img, const float* img_l, int n, double* part, int* stat, cudaStream_t st)
{
    k_img_entropy_part<<<dim3(kJudgeParts, 2), 256, 0, st>>>(img, img_l, n, part);
    ISAR_COUNT(1);
    k_img_select<<<kJudgeCopy, 256, 0, st>>>(img, img_l, n, part, stat);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

}  // namespace isar
