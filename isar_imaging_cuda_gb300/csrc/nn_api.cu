// C ABI of the learned autofocus warm-start network (no counterpart in the
// reference): parameters, forward, loss + backward, Adam, and a bf16 GEMM
// test entry.  Training runs entirely on the GPU through these calls.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <memory>
#include <vector>

#include "../../include/isar_gb300.h"
#include "isar_kernels.h"
#include "nn.h"

using namespace isar::nn;

namespace {

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return isar::record_error(code, buf);
}

#define CU(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return fail(ISAR_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

struct isar_wsnet {
    int dev = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    int max_rows = 0;
    bool training = false;
    int step = 0;
    Weights w;
    Acts a;
    Grads g;
    int* d_err = nullptr;
    std::vector<void*> allocs;
};

namespace {

template <class T>
int nalloc(isar_wsnet* n, T** p, size_t count)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 256);
    if (e != cudaSuccess) return fail(ISAR_ENOMEM, "cudaMalloc(%zu) failed: %s", count * sizeof(T), cudaGetErrorString(e));
    n->allocs.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return ISAR_OK;
}

#define TRY(x)                          \
    do {                                \
        const int rc_ = (x);            \
        if (rc_ != ISAR_OK) return rc_; \
    } while (0)

int check_err(isar_wsnet* n)
{
    int h = 0;
    CU(cudaMemcpyAsync(&h, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, n->st));
    CU(cudaStreamSynchronize(n->st));
    if (h) {
        cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
        return fail(ISAR_ECUDA, "tensor-core GEMM wait timed out");
    }
    return ISAR_OK;
}

}  // namespace

const Weights* isar_wsnet_weights(const isar_wsnet* n) { return n ? &n->w : nullptr; }

extern "C" {

ISAR_API int isar_wsnet_param_count(void) { return kParams; }

ISAR_API int isar_wsnet_create(isar_wsnet** out, int max_rows, int training, int device, void* stream)
{
    if (!out || max_rows <= 0 || (max_rows % 8)) return fail(ISAR_EINVAL, "max_rows must be a positive multiple of 8");
    std::unique_ptr<isar_wsnet> n(new isar_wsnet());
    n->dev = device;
    CU(cudaSetDevice(device));
    if (stream) {
        n->st = static_cast<cudaStream_t>(stream);
    } else {
        CU(cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking));
        n->own_stream = true;
    }
    n->max_rows = max_rows;
    n->training = training != 0;
    const size_t R = (size_t)max_rows;
    int rc = ISAR_OK;
    auto fin = [&](int r) {
        if (r != ISAR_OK) {
            for (void* p : n->allocs) cudaFree(p);
            if (n->own_stream) cudaStreamDestroy(n->st);
        }
        return r;
    };
    if ((rc = nalloc(n.get(), &n->w.master, kParams)) != ISAR_OK) return fin(rc);
    for (int l = 0; l < kConv + 2; ++l) {
        const size_t sz = (size_t)(l == kConv + 1 ? kOutPad : w_rows(l)) * w_cols(l);
        if ((rc = nalloc(n.get(), &n->w.w[l], sz)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->w.wt[l], sz)) != ISAR_OK) return fin(rc);
        n->w.bias[l] = n->w.master + b_off(l);
    }
    n->a.rows = max_rows;
    for (int l = 1; l < kConv + 2; ++l)
        if ((rc = nalloc(n.get(), &n->a.act[l], R * kCh)) != ISAR_OK) return fin(rc);
    if ((rc = nalloc(n.get(), &n->a.out, R * kOutPad)) != ISAR_OK) return fin(rc);
    if (n->training) {
        for (int l = 0; l < kConv; ++l)
            if ((rc = nalloc(n.get(), &n->a.cols[l], R * kColK)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.g, kParams)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.m1, kParams)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.m2, kParams)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.dact, R * kCh)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.dz, R * kCh)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.dzT, R * kCh)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.colT, R * kColK)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.dcol, R * kColK)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.loss, R)) != ISAR_OK) return fin(rc);
        if ((rc = nalloc(n.get(), &n->g.gwT, (size_t)kColK * kCh)) != ISAR_OK) return fin(rc);
        cudaMemsetAsync(n->g.m1, 0, kParams * sizeof(float), n->st);
        cudaMemsetAsync(n->g.m2, 0, kParams * sizeof(float), n->st);
    } else {
        if ((rc = nalloc(n.get(), &n->a.col, R * kColK)) != ISAR_OK) return fin(rc);
    }
    if ((rc = nalloc(n.get(), &n->d_err, 1)) != ISAR_OK) return fin(rc);
    cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
    cudaMemsetAsync(n->w.master, 0, kParams * sizeof(float), n->st);
    if (cudaError_t e = refresh_bf16(n->w, n->st)) return fin(fail(ISAR_ECUDA, "refresh: %s", cudaGetErrorString(e)));
    *out = n.release();
    return ISAR_OK;
}

ISAR_API int isar_wsnet_destroy(isar_wsnet* n)
{
    if (!n) return ISAR_OK;
    cudaSetDevice(n->dev);
    cudaStreamSynchronize(n->st);
    for (void* p : n->allocs) cudaFree(p);
    if (n->own_stream) cudaStreamDestroy(n->st);
    delete n;
    return ISAR_OK;
}

ISAR_API void* isar_wsnet_stream(isar_wsnet* n) { return n ? n->st : nullptr; }

ISAR_API int isar_wsnet_set_params(isar_wsnet* n, const float* h)
{
    if (!n || !h) return fail(ISAR_EINVAL, "null argument");
    CU(cudaMemcpyAsync(n->w.master, h, kParams * sizeof(float), cudaMemcpyHostToDevice, n->st));
    CU(refresh_bf16(n->w, n->st));
    if (n->training) {
        CU(cudaMemsetAsync(n->g.m1, 0, kParams * sizeof(float), n->st));
        CU(cudaMemsetAsync(n->g.m2, 0, kParams * sizeof(float), n->st));
        n->step = 0;
    }
    CU(cudaStreamSynchronize(n->st));
    return ISAR_OK;
}

ISAR_API int isar_wsnet_get_params(isar_wsnet* n, float* h)
{
    if (!n || !h) return fail(ISAR_EINVAL, "null argument");
    CU(cudaMemcpyAsync(h, n->w.master, kParams * sizeof(float), cudaMemcpyDeviceToHost, n->st));
    CU(cudaStreamSynchronize(n->st));
    return ISAR_OK;
}

/* d_x0: bf16 [frames*M][64] features; d_out: fp32 [frames*M][2] or NULL. */
ISAR_API int isar_wsnet_forward(isar_wsnet* n, const void* d_x0, int frames, int M, float* d_out)
{
    if (!n || !d_x0 || frames <= 0 || M < 8 || (M % 8)) return fail(ISAR_EINVAL, "bad forward arguments");
    if ((long)frames * M > n->max_rows) return fail(ISAR_EINVAL, "frames * M exceeds max_rows");
    n->a.act[0] = const_cast<__nv_bfloat16*>(static_cast<const __nv_bfloat16*>(d_x0));
    CU(forward(n->w, n->a, frames, M, n->d_err, n->st));
    if (d_out)
        CU(cudaMemcpy2DAsync(d_out, 2 * sizeof(float), n->a.out, kOutPad * sizeof(float), 2 * sizeof(float),
                             (size_t)frames * M, cudaMemcpyDeviceToDevice, n->st));
    return check_err(n);
}

/* Loss and gradients of the last forward against d_target (fp32 [frames*M],
 * the residual r_m; r_{M-1} unused).  *h_loss = mean loss over frames. */
ISAR_API int isar_wsnet_backward(isar_wsnet* n, const float* d_target, int frames, int M, float* h_loss)
{
    if (!n || !n->training || !d_target) return fail(ISAR_EINVAL, "backward needs a training network and targets");
    if ((long)frames * M > n->max_rows) return fail(ISAR_EINVAL, "frames * M exceeds max_rows");
    CU(backward(n->w, n->a, n->g, d_target, frames, M, n->d_err, n->st));
    if (h_loss) {
        std::vector<float> l(frames);
        CU(cudaMemcpyAsync(l.data(), n->g.loss, frames * sizeof(float), cudaMemcpyDeviceToHost, n->st));
        CU(cudaStreamSynchronize(n->st));
        double s = 0.0;
        for (float x : l) s += x;
        *h_loss = (float)(s / frames);
    }
    return check_err(n);
}

ISAR_API int isar_wsnet_get_grads(isar_wsnet* n, float* h)
{
    if (!n || !n->training || !h) return fail(ISAR_EINVAL, "null argument or not a training network");
    CU(cudaMemcpyAsync(h, n->g.g, kParams * sizeof(float), cudaMemcpyDeviceToHost, n->st));
    CU(cudaStreamSynchronize(n->st));
    return ISAR_OK;
}

ISAR_API int isar_wsnet_adam(isar_wsnet* n, float lr)
{
    if (!n || !n->training || !(lr > 0.0f)) return fail(ISAR_EINVAL, "bad Adam arguments");
    CU(adam_step(n->w, n->g, lr, ++n->step, n->st));
    return ISAR_OK;
}

/* Test entry: C[M][N] = A[M][K] * B[N][K]^T on the tensor cores (bf16 in,
 * fp32 out; C zeroed first when splits > 1).  Blocking. */
ISAR_API int isar_nn_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, int M, int N, int K,
                               int splits, void* stream)
{
    if (!A || !B || !C) return fail(ISAR_EINVAL, "null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* err = nullptr;
    CU(cudaMalloc(&err, sizeof(int)));
    cudaMemsetAsync(err, 0, sizeof(int), st);
    if (splits > 1) cudaMemsetAsync(C, 0, (size_t)M * ldc * sizeof(float), st);
    cudaError_t e = gemm_tn(static_cast<const __nv_bfloat16*>(A), lda, static_cast<const __nv_bfloat16*>(B), ldb, C,
                            ldc, M, N, K, splits, err, st);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(err);
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "gemm: %s", cudaGetErrorString(e));
    if (h) return fail(ISAR_ECUDA, "tensor-core GEMM wait timed out");
    return ISAR_OK;
}

}  // extern "C"
