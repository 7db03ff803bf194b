// Learned autofocus warm start: features, network forward/backward, Adam.
// The dense layers are tcgen05 bf16 GEMMs (nn_gemm.cu); the kernels here
// stage their operands (im2col, transposes), apply bias/ReLU, reduce bias
// gradients and evaluate the loss.  See nn.h for the network.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>

#include "isar_common.cuh"
#include "isar_kernels.h"
#include "nn.h"

namespace isar {
namespace nn {

namespace {

__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }

// w[l] [rows_pad][K] and wt[l] [K][rows_pad] from the fp32 master.
__global__ void k_refresh(const float* __restrict__ master, int off, int rows, int rows_pad, int K,
                          __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt)
{
    const int n = rows_pad * K;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int o = i / K, k = i - o * K;
        const float v = o < rows ? master[off + o * K + k] : 0.0f;
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        w[i] = b;
        wt[(size_t)k * rows_pad + o] = b;
    }
}

// col[p][k*64 + c] = act[b][m + k - 2][c] (0 outside [0, M)), p = b*M + m;
// one thread per 8 channels.
__global__ void k_im2col(const __nv_bfloat16* __restrict__ act, int frames, int M, __nv_bfloat16* __restrict__ col)
{
    const long n = (long)frames * M * kTaps * (kCh / 8);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % (kCh / 8));
        const long t = i / (kCh / 8);
        const int k = (int)(t % kTaps);
        const long p = t / kTaps;
        const int m = (int)(p % M);
        const long b = p / M;
        const int ms = m + k - kTaps / 2;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (ms >= 0 && ms < M) v = *reinterpret_cast<const uint4*>(act + ((b * M + ms) * kCh + c8 * 8));
        *reinterpret_cast<uint4*>(col + (p * kColK + k * kCh + c8 * 8)) = v;
    }
}

// Per frame: delta_m = atan2(s, c) - r_m (m < M-1), z = mean exp(j delta),
// loss = 1 - |z|; d loss / d r_hat_m = Im(conj(z) exp(j delta_m)) / ((M-1) |z|)
// / frames, chained through r_hat = atan2(s, c) into dout (bf16 [rows][16]).
__global__ void __launch_bounds__(256)
k_loss(const float* __restrict__ out, const float* __restrict__ target, int M, int frames, float* __restrict__ loss,
       __nv_bfloat16* __restrict__ dout)
{
    const int b = blockIdx.x;
    const int tid = threadIdx.x;
    __shared__ float red[2][8];
    __shared__ float s_z[2];
    float zx = 0.0f, zy = 0.0f;
    for (int m = tid; m < M - 1; m += blockDim.x) {
        const long p = (long)b * M + m;
        const float d = atan2f(out[p * kOutPad + 1], out[p * kOutPad]) - target[p];
        float sd, cd;
        sincosf(d, &sd, &cd);
        zx += cd;
        zy += sd;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        zx += __shfl_xor_sync(0xffffffffu, zx, o);
        zy += __shfl_xor_sync(0xffffffffu, zy, o);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = zx;
        red[1][tid >> 5] = zy;
    }
    __syncthreads();
    if (tid == 0) {
        float a = 0.0f, c = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += red[0][w];
            c += red[1][w];
        }
        s_z[0] = a / (float)(M - 1);
        s_z[1] = c / (float)(M - 1);
        loss[b] = 1.0f - sqrtf(s_z[0] * s_z[0] + s_z[1] * s_z[1]);
    }
    __syncthreads();
    const float Zx = s_z[0], Zy = s_z[1];
    const float az = fmaxf(sqrtf(Zx * Zx + Zy * Zy), 1e-20f);
    const float scale = 1.0f / ((float)(M - 1) * az * (float)frames);
    for (int m = tid; m < M; m += blockDim.x) {
        const long p = (long)b * M + m;
        float dc = 0.0f, ds = 0.0f;
        if (m < M - 1) {
            const float c = out[p * kOutPad], s = out[p * kOutPad + 1];
            const float d = atan2f(s, c) - target[p];
            float sd, cd;
            sincosf(d, &sd, &cd);
            const float g = (Zx * sd - Zy * cd) * scale;   // Im(conj(z) e^{j d}) * scale
            const float r2 = fmaxf(c * c + s * s, 1e-30f);
            dc = -g * s / r2;
            ds = g * c / r2;
        }
        dout[p * kOutPad] = __float2bfloat16_rn(dc);
        dout[p * kOutPad + 1] = __float2bfloat16_rn(ds);
#pragma unroll
        for (int q = 2; q < kOutPad; ++q) dout[p * kOutPad + q] = __float2bfloat16_rn(0.0f);
    }
}

// dz[p][c] = bf16(dact[p][c] * (act[p][c] > 0)).
__global__ void k_relu_grad(const float* __restrict__ dact, const __nv_bfloat16* __restrict__ act, long n,
                            __nv_bfloat16* __restrict__ dz)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dz[i] = __float2bfloat16_rn(bf(act[i]) > 0.0f ? dact[i] : 0.0f);
}

// dst[c][r] = src[r][c], bf16, 32 x 32 tiles.
__global__ void k_transpose(const __nv_bfloat16* __restrict__ src, int R, int Cc, __nv_bfloat16* __restrict__ dst)
{
    __shared__ __nv_bfloat16 t[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        t[j][threadIdx.x] = (r < R && c < Cc) ? src[(size_t)r * Cc + c] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < Cc && r < R) dst[(size_t)c * R + r] = t[threadIdx.x][j];
    }
}

// g[c] += sum_p x[p][c] for c < ncols (bias gradients), ld = row stride.
__global__ void k_colsum(const __nv_bfloat16* __restrict__ x, long rows, int ld, int ncols, float* __restrict__ g)
{
    const int c = threadIdx.x;   // blockDim.x == ld (<= 64)
    float s = 0.0f;
    for (long p = blockIdx.x; p < rows; p += gridDim.x) s += bf(x[p * ld + c]);
    if (c < ncols) atomicAdd(&g[c], s);
}

// dact[b][m][c] = sum_k dcol[b][m - k + 2][k*64 + c].
__global__ void k_col2im(const float* __restrict__ dcol, int frames, int M, float* __restrict__ dact)
{
    const long n = (long)frames * M * kCh;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % kCh);
        const long p = i / kCh;
        const int m = (int)(p % M);
        const long b = p / M;
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < kTaps; ++k) {
            const int ms = m - k + kTaps / 2;
            if (ms >= 0 && ms < M) s += dcol[(b * M + ms) * kColK + k * kCh + c];
        }
        dact[i] = s;
    }
}

// g[off + o*K + k] = gwT[k][o] for o < rows (weight gradient from its transpose).
__global__ void k_scatter_gw(const float* __restrict__ gwT, int rows, int ld, int K, float* __restrict__ g, int off)
{
    const int n = rows * K;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int o = i / K, k = i - o * K;
        g[off + i] = gwT[(size_t)k * ld + o];
    }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float c1, float c2)
{
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.0f - b1) * gi;
        const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        w[i] -= lr * (a * c1) / (sqrtf(v * c2) + eps);
    }
}

// Features, one CTA (256 threads) per frame.  Channels at pulse m:
//   2q, 2q+1: unit phasor of p = conj(x[m,b_q]) x[m+1,b_q], q < 16 strongest bins
//   32 + q:   |p| / mean_m |p| of bin q
//   48, 49:   cos, sin of psi_m = arg(dsum[m]) (Doppler tracking increment)
//   50:       |dsum[m]| / mean_m |dsum|
//   51..63:   0;  pulse M-1 (no successor): all 0.
__global__ void __launch_bounds__(256)
k_features(const float2* __restrict__ cut, const double* __restrict__ E, const float2* __restrict__ dsum, int M,
           __nv_bfloat16* __restrict__ x0, float* __restrict__ psi)
{
    constexpr int C = kRangeCut;
    __shared__ int s_bins[kFeatBins];
    __shared__ float s_key[C];
    __shared__ float s_sum[kFeatBins + 1];
    __shared__ float rk[8];
    __shared__ int ri[8];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int i = tid; i < C; i += blockDim.x) {
        const double e = E[i];
        s_key[i] = isnan(e) ? -CUDART_INF_F : (float)e;
    }
    if (tid <= kFeatBins) s_sum[tid] = 0.0f;
    __syncthreads();
    for (int q = 0; q < kFeatBins; ++q) {   // q-th strongest bin (lowest index on ties)
        float bk = -CUDART_INF_F;
        int bi = 0x7fffffff;
        for (int i = tid; i < C; i += blockDim.x)
            if (s_key[i] > bk || (s_key[i] == bk && i < bi)) {
                bk = s_key[i];
                bi = i;
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float k2 = __shfl_xor_sync(0xffffffffu, bk, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
            if (k2 > bk || (k2 == bk && i2 < bi)) {
                bk = k2;
                bi = i2;
            }
        }
        if (lane == 0) {
            rk[w] = bk;
            ri[w] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            for (int j = 1; j < (int)(blockDim.x >> 5); ++j)
                if (rk[j] > rk[0] || (rk[j] == rk[0] && ri[j] < ri[0])) {
                    rk[0] = rk[j];
                    ri[0] = ri[j];
                }
            const int b = ri[0] < C ? ri[0] : 0;
            s_bins[q] = b;
            s_key[b] = -CUDART_INF_F;   // taken
        }
        __syncthreads();
    }
    // per-bin mean magnitudes of the pulse-pair products: per-thread sums in
    // registers, then a fixed-order block reduction (deterministic, no
    // shared-memory atomics)
    float acc[kFeatBins + 1];
#pragma unroll
    for (int q = 0; q <= kFeatBins; ++q) acc[q] = 0.0f;
    for (int m = tid; m < M - 1; m += blockDim.x) {
#pragma unroll
        for (int q = 0; q < kFeatBins; ++q) {
            const int b = s_bins[q];
            const float2 p = cmulc(cut[(size_t)m * C + b], cut[(size_t)(m + 1) * C + b]);
            acc[q] += sqrtf(p.x * p.x + p.y * p.y);
        }
        const float2 d = dsum[m];
        acc[kFeatBins] += sqrtf(d.x * d.x + d.y * d.y);
    }
    __shared__ float s_part[kFeatBins + 1][8];
#pragma unroll
    for (int q = 0; q <= kFeatBins; ++q) {
        float v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) s_part[q][w] = v;
    }
    __syncthreads();
    if (tid <= kFeatBins) {
        float v = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v += s_part[tid][i];
        s_sum[tid] = v;
    }
    __syncthreads();
    for (int m = tid; m < M; m += blockDim.x) {
        __nv_bfloat16* xr = x0 + (size_t)m * kCh;
        float f[kCh];
#pragma unroll
        for (int c = 0; c < kCh; ++c) f[c] = 0.0f;
        float ps = 0.0f;
        if (m < M - 1) {
#pragma unroll
            for (int q = 0; q < kFeatBins; ++q) {
                const int b = s_bins[q];
                const float2 p = cmulc(cut[(size_t)m * C + b], cut[(size_t)(m + 1) * C + b]);
                const float a = sqrtf(p.x * p.x + p.y * p.y);
                if (a > 0.0f) {
                    f[2 * q] = p.x / a;
                    f[2 * q + 1] = p.y / a;
                }
                const float mean = s_sum[q] / (float)(M - 1);
                f[32 + q] = mean > 0.0f ? a / mean : 0.0f;
            }
            const float2 d = dsum[m];
            ps = atan2f(d.y, d.x);
            float sn, cs;
            sincosf(ps, &sn, &cs);
            f[48] = cs;
            f[49] = sn;
            const float mean = s_sum[kFeatBins] / (float)(M - 1);
            f[50] = mean > 0.0f ? sqrtf(d.x * d.x + d.y * d.y) / mean : 0.0f;
        }
#pragma unroll
        for (int c = 0; c < kCh; ++c) xr[c] = __float2bfloat16_rn(f[c]);
        psi[m] = ps;
    }
}

// phase[0] = 1, phase[m+1] = exp(-j * cumsum_{i<=m} wrap(psi_i - atan2(s_i, c_i))); one CTA of 1024.
__global__ void __launch_bounds__(1024)
k_ws_phase(const float* __restrict__ psi, const float* __restrict__ out, int M, float2* __restrict__ phase)
{
    __shared__ float sc[1024];
    const int tid = threadIdx.x;
    float a = 0.0f;
    if (tid < M - 1) {
        a = psi[tid] - atan2f(out[(size_t)tid * kOutPad + 1], out[(size_t)tid * kOutPad]);
        a -= 2.0f * CUDART_PI_F * rintf(a * (0.5f / CUDART_PI_F));
    }
    sc[tid] = a;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const float add = tid >= o ? sc[tid - o] : 0.0f;
        __syncthreads();
        sc[tid] += add;
        __syncthreads();
    }
    if (tid == 0) phase[0] = make_float2(1.0f, 0.0f);
    if (tid < M - 1) {
        float sn, cs;
        sincosf(sc[tid], &sn, &cs);
        phase[tid + 1] = make_float2(cs, -sn);
    }
}

int grid_for(long n, int threads) { return (int)std::min<long>((n + threads - 1) / threads, 152L * 16); }

}  // namespace

cudaError_t refresh_bf16(const Weights& w, cudaStream_t st)
{
    for (int l = 0; l < kConv + 2; ++l) {
        const int rows = w_rows(l), rp = l == kConv + 1 ? kOutPad : rows, K = w_cols(l);
        k_refresh<<<grid_for((long)rp * K, 256), 256, 0, st>>>(w.master, w_off(l), rows, rp, K, w.w[l], w.wt[l]);
        ISAR_COUNT(1);
    }
    return cudaGetLastError();
}

cudaError_t forward(const Weights& w, Acts& a, int frames, int M, int* err, cudaStream_t st)
{
    const long rows = (long)frames * M;
    if (rows > a.rows) return cudaErrorInvalidValue;
    cudaError_t e;
    // every hidden layer: bias and ReLU in the GEMM's epilogue, bf16 out
    auto hidden = [&](int l) {
        GemmEpilogue ep;
        ep.bias = w.master + b_off(l);
        ep.out_bf16 = a.act[l + 1];
        ep.ld_bf16 = kCh;
        return ep;
    };
    for (int l = 0; l < kConv; ++l) {
        if (!a.cols[l] && M % 128 == 0) {
            // inference: the conv's im2col operand read tap by tap from the
            // activations by the GEMM itself (training keeps the columns for
            // the weight gradients)
            GemmConvA cv;
            cv.act = a.act[l];
            cv.frames = frames;
            cv.M = M;
            cv.pad = kTaps / 2;
            if ((e = gemm_tn(nullptr, kColK, w.w[l], kColK, nullptr, kCh, (int)rows, kCh, kColK, 1, err, st,
                             hidden(l), cv)))
                return e;
            continue;
        }
        __nv_bfloat16* col = a.cols[l] ? a.cols[l] : a.col;
        k_im2col<<<grid_for(rows * kTaps * (kCh / 8), 256), 256, 0, st>>>(a.act[l], frames, M, col);
        ISAR_COUNT(1);
        if ((e = gemm_tn(col, kColK, w.w[l], kColK, nullptr, kCh, (int)rows, kCh, kColK, 1, err, st, hidden(l))))
            return e;
    }
    if ((e = gemm_tn(a.act[kConv], kCh, w.w[kConv], kCh, nullptr, kCh, (int)rows, kCh, kCh, 1, err, st,
                     hidden(kConv))))
        return e;
    // output layer: bias on the two used columns (c, s)
    GemmEpilogue eo;
    eo.bias = w.master + b_off(kConv + 1);
    eo.bias_cols = 2;
    if ((e = gemm_tn(a.act[kConv + 1], kCh, w.w[kConv + 1], kCh, a.out, kOutPad, (int)rows, kOutPad, kCh, 1, err,
                     st, eo)))
        return e;
    return cudaGetLastError();
}

// Weight gradient of layer l: dW^T [K][rows_out] = X^T [K][rows] * dZ^T [rows_out][rows]^T,
// split over the rows, then scattered into g (canonical [rows_out][K]).
static cudaError_t weight_grad(const __nv_bfloat16* X, int K, const __nv_bfloat16* dz, int ldz, int nout, long rows,
                               Grads& g, int off, int* err, cudaStream_t st)
{
    cudaError_t e;
    dim3 tb(32, 8);
    k_transpose<<<dim3((K + 31) / 32, (unsigned)((rows + 31) / 32)), tb, 0, st>>>(X, (int)rows, K, g.colT);
    ISAR_COUNT(1);
    k_transpose<<<dim3((ldz + 31) / 32, (unsigned)((rows + 31) / 32)), tb, 0, st>>>(dz, (int)rows, ldz, g.dzT);
    ISAR_COUNT(1);
    if ((e = cudaMemsetAsync(g.gwT, 0, (size_t)kColK * kCh * sizeof(float), st))) return e;
    int splits = (int)std::min<long>(std::max<long>(rows / 1024, 1), 128);
    if ((e = gemm_tn(g.colT, (int)rows, g.dzT, (int)rows, g.gwT, ldz, K, ldz, (int)rows, splits, err, st))) return e;
    k_scatter_gw<<<grid_for((long)nout * K, 256), 256, 0, st>>>(g.gwT, nout, ldz, K, g.g, off);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t backward(const Weights& w, Acts& a, Grads& g, const float* target, int frames, int M, int* err,
                     cudaStream_t st)
{
    const long rows = (long)frames * M;
    cudaError_t e;
    if ((e = cudaMemsetAsync(g.g, 0, (size_t)kParams * sizeof(float), st))) return e;
    // output layer: dout (bf16 [rows][16]) into g.dz
    k_loss<<<frames, 256, 0, st>>>(a.out, target, M, frames, g.loss, g.dz);
    ISAR_COUNT(1);
    const int cs_grid = (int)std::min<long>(rows, 1024);
    k_colsum<<<cs_grid, kOutPad, 0, st>>>(g.dz, rows, kOutPad, 2, g.g + b_off(kConv + 1));
    ISAR_COUNT(1);
    if ((e = weight_grad(a.act[kConv + 1], kCh, g.dz, kOutPad, 2, rows, g, w_off(kConv + 1), err, st))) return e;
    if ((e = gemm_tn(g.dz, kOutPad, w.wt[kConv + 1], kOutPad, g.dact, kCh, (int)rows, kCh, kOutPad, 1, err, st)))
        return e;
    // 1x1 hidden layer
    k_relu_grad<<<grid_for(rows * kCh, 256), 256, 0, st>>>(g.dact, a.act[kConv + 1], rows * kCh, g.dz);
    ISAR_COUNT(1);
    k_colsum<<<cs_grid, kCh, 0, st>>>(g.dz, rows, kCh, kCh, g.g + b_off(kConv));
    ISAR_COUNT(1);
    if ((e = weight_grad(a.act[kConv], kCh, g.dz, kCh, kCh, rows, g, w_off(kConv), err, st))) return e;
    if ((e = gemm_tn(g.dz, kCh, w.wt[kConv], kCh, g.dact, kCh, (int)rows, kCh, kCh, 1, err, st))) return e;
    // conv layers
    for (int l = kConv - 1; l >= 0; --l) {
        k_relu_grad<<<grid_for(rows * kCh, 256), 256, 0, st>>>(g.dact, a.act[l + 1], rows * kCh, g.dz);
        ISAR_COUNT(1);
        k_colsum<<<cs_grid, kCh, 0, st>>>(g.dz, rows, kCh, kCh, g.g + b_off(l));
        ISAR_COUNT(1);
        if ((e = weight_grad(a.cols[l], kColK, g.dz, kCh, kCh, rows, g, w_off(l), err, st))) return e;
        if (l > 0) {
            if ((e = gemm_tn(g.dz, kCh, w.wt[l], kCh, g.dcol, kColK, (int)rows, kColK, kCh, 1, err, st))) return e;
            k_col2im<<<grid_for(rows * kCh, 256), 256, 0, st>>>(g.dcol, frames, M, g.dact);
            ISAR_COUNT(1);
        }
    }
    return cudaGetLastError();
}

cudaError_t adam_step(Weights& w, Grads& g, float lr, int t, cudaStream_t st)
{
    const float c1 = 1.0f / (1.0f - powf(0.9f, (float)t));
    const float c2 = 1.0f / (1.0f - powf(0.999f, (float)t));
    k_adam<<<grid_for(kParams, 256), 256, 0, st>>>(w.master, g.g, g.m1, g.m2, kParams, lr, c1, c2);
    ISAR_COUNT(1);
    return refresh_bf16(w, st);
}

cudaError_t features(const float2* cut, const double* E, const float2* dsum, int M, __nv_bfloat16* x0, float* psi,
                     cudaStream_t st)
{
    k_features<<<1, 256, 0, st>>>(cut, E, dsum, M, x0, psi);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

cudaError_t ws_phase(const float* psi, const float* out, int M, float2* phase, cudaStream_t st)
{
    if (M > 1024) return cudaErrorInvalidValue;
    k_ws_phase<<<1, 1024, 0, st>>>(psi, out, M, phase);
    ISAR_COUNT(1);
    return cudaGetLastError();
}

}  // namespace nn
}  // namespace isar
