// Learned autofocus warm start: internal interface.
//
// Network (per frame, along the pulse axis m = 0..M-1, channels last):
//   X0 [M][64] bf16 features  ->  6 x (1-D conv k = 5, 64 -> 64, bias, ReLU)
//   -> 1x1 64 -> 64 + ReLU -> 1x1 64 -> 2 (c_m, s_m), fp32.
// r_m = atan2(s_m, c_m) is the predicted residual of the Doppler-tracking
// phase increment: warm-start increments alpha_m = psi_m - r_m.
// All dense layers run as bf16 GEMMs on tcgen05 with fp32 accumulation
// (nn_gemm.cu); everything else is elementwise or reduction kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace isar {
namespace nn {

constexpr int kCh = 64;            // channels of every hidden layer and of X0
constexpr int kTaps = 5;           // conv kernel width
constexpr int kConv = 6;           // conv layers
constexpr int kColK = kCh * kTaps; // 320, im2col width
constexpr int kOutPad = 16;        // output layer rows (2 used)
constexpr int kFeatBins = 16;      // strongest bins used by the features

// Canonical parameter order (host fp32 vector):
//   for l in 0..5: W_l [64][320] (row o, column k*64 + c), b_l [64]
//   W6 [64][64], b6 [64], W7 [2][64], b7 [2]
constexpr int kParams = kConv * (kCh * kColK + kCh) + kCh * kCh + kCh + 2 * kCh + 2;

// Device weights: fp32 master (canonical order) + bf16 GEMM copies.
struct Weights {
    float* master = nullptr;                  // [kParams]
    __nv_bfloat16* w[kConv + 2] = {};         // [Nout][K]: conv [64][320], W6 [64][64], W7 [16][64] (rows >= 2 zero)
    __nv_bfloat16* wt[kConv + 2] = {};        // transposed [K][Nout] (data-gradient GEMMs)
    const float* bias[kConv + 2] = {};        // views into master
};

// Offsets into the canonical vector.
__host__ __device__ inline int w_off(int l) { return l < kConv ? l * (kCh * kColK + kCh) : kConv * (kCh * kColK + kCh) + (l == kConv ? 0 : kCh * kCh + kCh); }
__host__ __device__ inline int w_rows(int l) { return l <= kConv ? kCh : 2; }
__host__ __device__ inline int w_cols(int l) { return l < kConv ? kColK : kCh; }
__host__ __device__ inline int b_off(int l) { return w_off(l) + w_rows(l) * w_cols(l); }

// Inference / training activations for up to `rows` = frames * M positions.
struct Acts {
    int rows = 0;
    __nv_bfloat16* act[kConv + 2] = {};       // act[0] = X0 (caller-filled), act[l+1] = layer l output [rows][64]
    __nv_bfloat16* col = nullptr;             // [rows][320] im2col scratch (inference) or
    __nv_bfloat16* cols[kConv] = {};          // per conv layer (training keeps them for the weight gradients)
    float* out = nullptr;                     // [rows][16] network output (c, s, 14 pad)
};

// Optional epilogue of gemm_tn (no split-K): with out_bf16, the tile is
// written as bf16(max(C + bias[c], 0)) to out_bf16 [Mr][ld_bf16] (16-byte
// aligned rows) instead of C; otherwise, with bias, columns c < bias_cols of
// C get bias[c] added.
struct GemmEpilogue {
    const float* bias = nullptr;
    __nv_bfloat16* out_bf16 = nullptr;
    int ld_bf16 = 0;
    int bias_cols = 0;
};

// Optional implicit-convolution A operand of gemm_tn: with act set, A is the
// im2col matrix of act ([frames][M][64] bf16, M a multiple of 128), i.e.
// A[b*M + m][k*64 + c] = act[b][m + k - pad][c] (0 outside the frame), read
// tap by tap straight from act; A and lda are ignored and K = taps * 64.
struct GemmConvA {
    const __nv_bfloat16* act = nullptr;
    int frames = 0;
    int M = 0;
    int pad = 0;
};

cudaError_t gemm_tn(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int Mr,
                    int Nc, int K, int splits, int* err, cudaStream_t st, const GemmEpilogue& ep = GemmEpilogue{},
                    const GemmConvA& conv = GemmConvA{});

// Refreshes the bf16 copies (and transposes) from the fp32 master.
cudaError_t refresh_bf16(const Weights& w, cudaStream_t st);

// Forward over frames x M positions; act[0] must hold X0.  Keeps every
// layer's im2col when a.cols[] are set (training).
cudaError_t forward(const Weights& w, Acts& a, int frames, int M, int* err, cudaStream_t st);

// Training buffers for the backward pass.
struct Grads {
    float* g = nullptr;                       // [kParams] fp32 gradients (canonical order)
    float* m1 = nullptr;                      // Adam first moment
    float* m2 = nullptr;                      // Adam second moment
    float* dact = nullptr;                    // [rows][64] fp32
    __nv_bfloat16* dz = nullptr;              // [rows][64] bf16 (pre-activation gradient)
    __nv_bfloat16* dzT = nullptr;             // [64][rows] bf16 transposed
    __nv_bfloat16* colT = nullptr;            // [320][rows] bf16 transposed im2col
    float* dcol = nullptr;                    // [rows][320] fp32
    float* loss = nullptr;                    // [frames] per-frame loss
    float* gwT = nullptr;                     // [320][64] fp32 transposed weight-gradient scratch
};

// Loss 1 - |mean_m exp(j (r_hat_m - r_m))| per frame over m in [0, M-1), its
// gradient, and the backward pass into g.g (overwritten).
cudaError_t backward(const Weights& w, Acts& a, Grads& g, const float* target, int frames, int M, int* err,
                     cudaStream_t st);

cudaError_t adam_step(Weights& w, Grads& g, float lr, int t, cudaStream_t st);

// Features of one frame from its cut [M][512], the selected bins, the
// energies E[512] (for the strongest bins) and the Doppler sums dsum[M-1]
// over the selected bins: X0 [M][64] bf16 and psi [M] (float, psi[M-1] = 0).
cudaError_t features(const float2* cut, const double* E, const float2* dsum, int M, __nv_bfloat16* x0, float* psi,
                     cudaStream_t st);

// Warm-start phase from psi and the network output: phase[0] = 1,
// phase[m+1] = exp(-j sum_{i<=m} (psi_i - atan2(s_i, c_i))).
cudaError_t ws_phase(const float* psi, const float* out, int M, float2* phase, cudaStream_t st);

}  // namespace nn
}  // namespace isar
