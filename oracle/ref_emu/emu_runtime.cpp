// CPU emulation runtime for the reference's CUDA sources (TEST INFRASTRUCTURE
// ONLY): host implementations of the CUDA runtime calls the reference makes,
// grid execution with fiber-based __syncthreads, the shared-memory arrays of
// its kernels, and the cuFFT / cuBLAS subsets it calls.
//
// Device memory is host memory.  Allocations are zero-filled and padded, so
// the reference's reads of never-written memory (Q1: cublasDger into a fresh
// allocation, high_speed_compensation.cu:30-32; Q4: the tail of d_ww_,
// mtrc.cu:150-156) see zeros, and its unguarded tail writes (Q5: getARPMean,
// range_alignment.cu:439/524-549) land in the padding.
#include <ucontext.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cuda_runtime.h"
#include "include/cublas_api.h"
#include "include/cufft.h"
#include "include/emu_launch.h"

// ---------------------------------------------------------------------------
// built-in variables (device_launch_parameters.h declares them extern)
extern "C" {
uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;
int warpSize = 32;
}

// Shared-memory arrays of the reference kernels (extern __shared__ in
// common.cu:350,377,419,448,477 and range_alignment.cu:88,151).  Blocks run
// one after another, so one array per name is the block's shared memory.
float sdata_getAveProfileParallel_flt[1 << 14];
int sdata_maxRowsIdxABS_int[1 << 14];
int sdata_max_cols_int[1 << 14];
float sdata_sum_cols_flt[1 << 14];
int sdata_max_rows_int[1 << 14];
cuComplex sdata_sum_rows_com_flt[1 << 14];
float sdata_sum_rows_flt[1 << 14];

namespace emu {

namespace {
const char* const kSyncKernels[] = {"getAveProfileParallel", "maxRowsIdxABS", "maxCols", "sumCols",
                                    "sumRows", "maxRowsIdx"};

bool kernel_syncs(const char* name)
{
    for (const char* k : kSyncKernels)
        if (std::strcmp(name, k) == 0) return true;
    return false;
}

struct Fiber {
    ucontext_t uc;
    std::vector<char> stack;
    bool done = false;
    uint3 tid;
};

ucontext_t g_sched;
Fiber* g_cur = nullptr;
void (*g_thunk)(void*) = nullptr;
void* g_ctx = nullptr;
std::vector<Fiber> g_pool;
constexpr size_t kStack = 64 * 1024;

void fiber_main()
{
    g_thunk(g_ctx);
    g_cur->done = true;
    swapcontext(&g_cur->uc, &g_sched);
}
}  // namespace

void syncthreads()
{
    if (g_cur) swapcontext(&g_cur->uc, &g_sched);
}

void run_grid(const char* name, dim3 grid, dim3 block, void (*thunk)(void*), void* ctx)
{
    const bool sync = kernel_syncs(name);
    gridDim = grid;
    blockDim = block;
    const unsigned nt = block.x * block.y * block.z;
    if (sync && g_pool.size() < nt) {
        g_pool.resize(nt);
        for (auto& f : g_pool)
            if (f.stack.empty()) f.stack.resize(kStack);
    }
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = make_uint3(bx, by, bz);
                if (!sync) {
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                threadIdx = make_uint3(tx, ty, tz);
                                thunk(ctx);
                            }
                    continue;
                }
                g_thunk = thunk;
                g_ctx = ctx;
                unsigned i = 0;
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx, ++i) {
                            Fiber& f = g_pool[i];
                            f.done = false;
                            f.tid = make_uint3(tx, ty, tz);
                            getcontext(&f.uc);
                            f.uc.uc_stack.ss_sp = f.stack.data();
                            f.uc.uc_stack.ss_size = f.stack.size();
                            f.uc.uc_link = nullptr;
                            makecontext(&f.uc, fiber_main, 0);
                        }
                bool pending = true;
                while (pending) {
                    pending = false;
                    for (unsigned t = 0; t < nt; ++t) {
                        Fiber& f = g_pool[t];
                        if (f.done) continue;
                        g_cur = &f;
                        threadIdx = f.tid;
                        swapcontext(&g_sched, &f.uc);
                        if (!f.done) pending = true;
                    }
                }
                g_cur = nullptr;
            }
}

}  // namespace emu

// ---------------------------------------------------------------------------
// CUDA runtime subset
namespace {
constexpr size_t kPad = 1 << 16;
}

extern "C" {

cudaError_t cudaMalloc(void** p, size_t size)
{
    *p = std::calloc(1, size + kPad);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p)
{
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind)
{
    if (n) std::memmove(dst, src, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t n, cudaMemcpyKind, cudaStream_t)
{
    if (n) std::memmove(dst, src, n);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* p, int v, size_t n)
{
    std::memset(p, v, n);
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaPeekAtLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "emulated error"; }
const char* cudaGetErrorName(cudaError_t e) { return e == cudaSuccess ? "cudaSuccess" : "cudaErrorEmulated"; }
cudaError_t cudaGetDeviceCount(int* n)
{
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDevice(int* d)
{
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr a, int)
{
    switch (a) {
    case cudaDevAttrComputeMode: *v = cudaComputeModeDefault; break;
    case cudaDevAttrComputeCapabilityMajor: *v = 10; break;
    case cudaDevAttrComputeCapabilityMinor: *v = 3; break;
    case cudaDevAttrMultiProcessorCount: *v = 1; break;
    case cudaDevAttrClockRate: *v = 1000000; break;
    default: *v = 0; break;
    }
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties_v2(cudaDeviceProp* p, int)
{
    std::memset(p, 0, sizeof(*p));
    std::strcpy(p->name, "cpu-emulation");
    p->major = 10;
    p->minor = 3;
    p->multiProcessorCount = 1;
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int d) { return cudaGetDeviceProperties_v2(p, d); }
cudaError_t cudaDriverGetVersion(int* v)
{
    *v = 13000;
    return cudaSuccess;
}
cudaError_t cudaRuntimeGetVersion(int* v)
{
    *v = 13000;
    return cudaSuccess;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FFT (double precision, radix 2, same conventions as cuFFT)
namespace {
using cd = std::complex<double>;

void fft_d(std::vector<cd>& x, bool inverse)
{
    const int n = (int)x.size();
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    const double sgn = inverse ? 1.0 : -1.0;
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            const double ang = sgn * 2.0 * M_PI * (double)k / (double)len;
            const cd w(std::cos(ang), std::sin(ang));
            for (int s = 0; s < n; s += len) {
                const cd t = x[s + k + half] * w;
                x[s + k + half] = x[s + k] - t;
                x[s + k] = x[s + k] + t;
            }
        }
    }
}

// Single-precision variant, selected by ISAR_EMU_FFT=float: the same radix-2
// transform with every butterfly in float and twiddles rounded to float.  It
// stands in for cuFFT's own FP32 arithmetic, so that the distance between the
// reference run this way and the FP64 restatement measures how far a float
// FFT alone moves the reference's results (its noise floor).
using cf32 = std::complex<float>;

void fft_f(std::vector<cd>& x, bool inverse)
{
    const int n = (int)x.size();
    std::vector<cf32> y(n);
    for (int i = 0; i < n; ++i) y[i] = cf32((float)x[i].real(), (float)x[i].imag());
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(y[i], y[j]);
    }
    const double sgn = inverse ? 1.0 : -1.0;
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            const double ang = sgn * 2.0 * M_PI * (double)k / (double)len;
            const float wr = (float)std::cos(ang), wi = (float)std::sin(ang);
            for (int s = 0; s < n; s += len) {
                const cf32 a = y[s + k], b = y[s + k + half];
                const float tr = __builtin_fmaf(b.real(), wr, -(b.imag() * wi));
                const float ti = __builtin_fmaf(b.real(), wi, b.imag() * wr);
                y[s + k + half] = cf32(a.real() - tr, a.imag() - ti);
                y[s + k] = cf32(a.real() + tr, a.imag() + ti);
            }
        }
    }
    for (int i = 0; i < n; ++i) x[i] = cd(y[i].real(), y[i].imag());
}

bool fft_single()
{
    static const bool f = [] {
        const char* e = std::getenv("ISAR_EMU_FFT");
        return e != nullptr && std::string(e) == "float";
    }();
    return f;
}

void fft_any(std::vector<cd>& x, bool inverse)
{
    if (fft_single())
        fft_f(x, inverse);
    else
        fft_d(x, inverse);
}

struct Plan {
    int n = 0, batch = 0, istride = 1, idist = 0, ostride = 1, odist = 0;
    cufftType type = CUFFT_C2C;
};
std::map<int, Plan> g_plans;
int g_next_plan = 1;
}  // namespace

cufftResult cufftPlan1d(cufftHandle* plan, int nx, cufftType type, int batch)
{
    Plan p;
    p.n = nx;
    p.batch = batch;
    p.type = type;
    p.idist = (type == CUFFT_C2R) ? nx / 2 + 1 : nx;
    p.odist = (type == CUFFT_R2C) ? nx / 2 + 1 : nx;
    *plan = g_next_plan++;
    g_plans[*plan] = p;
    return CUFFT_SUCCESS;
}

cufftResult cufftPlanMany(cufftHandle* plan, int rank, int* n, int*, int istride, int idist, int*, int ostride,
                          int odist, cufftType type, int batch)
{
    if (rank != 1) return CUFFT_INVALID_VALUE;
    Plan p;
    p.n = n[0];
    p.batch = batch;
    p.type = type;
    p.istride = istride;
    p.idist = idist;
    p.ostride = ostride;
    p.odist = odist;
    *plan = g_next_plan++;
    g_plans[*plan] = p;
    return CUFFT_SUCCESS;
}

cufftResult cufftDestroy(cufftHandle plan)
{
    g_plans.erase(plan);
    return CUFFT_SUCCESS;
}

cufftResult cufftExecC2C(cufftHandle plan, cufftComplex* in, cufftComplex* out, int direction)
{
    const Plan& p = g_plans.at(plan);
    std::vector<cd> v(p.n);
    for (int b = 0; b < p.batch; ++b) {
        for (int i = 0; i < p.n; ++i) {
            const cufftComplex c = in[(size_t)b * p.idist + (size_t)i * p.istride];
            v[i] = cd(c.x, c.y);
        }
        fft_any(v, direction == CUFFT_INVERSE);
        for (int i = 0; i < p.n; ++i)
            out[(size_t)b * p.odist + (size_t)i * p.ostride] = make_cuComplex((float)v[i].real(), (float)v[i].imag());
    }
    return CUFFT_SUCCESS;
}

cufftResult cufftExecR2C(cufftHandle plan, cufftReal* in, cufftComplex* out)
{
    const Plan& p = g_plans.at(plan);
    std::vector<cd> v(p.n);
    for (int b = 0; b < p.batch; ++b) {
        for (int i = 0; i < p.n; ++i) v[i] = cd(in[(size_t)b * p.idist + (size_t)i * p.istride], 0.0);
        fft_any(v, false);
        for (int i = 0; i <= p.n / 2; ++i)
            out[(size_t)b * p.odist + (size_t)i * p.ostride] = make_cuComplex((float)v[i].real(), (float)v[i].imag());
    }
    return CUFFT_SUCCESS;
}

cufftResult cufftExecC2R(cufftHandle plan, cufftComplex* in, cufftReal* out)
{
    const Plan& p = g_plans.at(plan);
    std::vector<cd> v(p.n);
    for (int b = 0; b < p.batch; ++b) {
        for (int i = 0; i <= p.n / 2; ++i) {
            const cufftComplex c = in[(size_t)b * p.idist + (size_t)i * p.istride];
            v[i] = cd(c.x, c.y);
        }
        v[0] = cd(v[0].real(), 0.0);
        v[p.n / 2] = cd(v[p.n / 2].real(), 0.0);
        for (int i = 1; i < p.n / 2; ++i) v[p.n - i] = std::conj(v[i]);
        fft_any(v, true);
        for (int i = 0; i < p.n; ++i) out[(size_t)b * p.odist + (size_t)i * p.ostride] = (float)v[i].real();
    }
    return CUFFT_SUCCESS;
}

// ---------------------------------------------------------------------------
// cuBLAS subset (host pointer mode)
struct cublasContext {
    int unused;
};

cublasStatus_t cublasCreate_v2(cublasHandle_t* h)
{
    *h = new cublasContext{0};
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDestroy_v2(cublasHandle_t h)
{
    delete h;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasIsamax_v2(cublasHandle_t, int n, const float* x, int incx, int* result)
{
    int best = 0;
    float bv = -1.0f;
    for (int i = 0; i < n; ++i) {
        const float v = std::fabs(x[(size_t)i * incx]);
        if (v > bv) {
            bv = v;
            best = i;
        }
    }
    *result = n > 0 ? best + 1 : 0;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasIsamin_v2(cublasHandle_t, int n, const float* x, int incx, int* result)
{
    int best = 0;
    float bv = 0.0f;
    for (int i = 0; i < n; ++i) {
        const float v = std::fabs(x[(size_t)i * incx]);
        if (i == 0 || v < bv) {
            bv = v;
            best = i;
        }
    }
    *result = n > 0 ? best + 1 : 0;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasIcamax_v2(cublasHandle_t, int n, const cuComplex* x, int incx, int* result)
{
    int best = 0;
    float bv = -1.0f;
    for (int i = 0; i < n; ++i) {
        const cuComplex c = x[(size_t)i * incx];
        const float v = std::fabs(c.x) + std::fabs(c.y);
        if (v > bv) {
            bv = v;
            best = i;
        }
    }
    *result = n > 0 ? best + 1 : 0;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasSscal_v2(cublasHandle_t, int n, const float* alpha, float* x, int incx)
{
    for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= *alpha;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasCsscal_v2(cublasHandle_t, int n, const float* alpha, cuComplex* x, int incx)
{
    for (int i = 0; i < n; ++i) {
        cuComplex& c = x[(size_t)i * incx];
        c.x *= *alpha;
        c.y *= *alpha;
    }
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDger_v2(cublasHandle_t, int m, int n, const double* alpha, const double* x, int incx,
                             const double* y, int incy, double* A, int lda)
{
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) A[i + (size_t)j * lda] += *alpha * x[(size_t)i * incx] * y[(size_t)j * incy];
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasSger_v2(cublasHandle_t, int m, int n, const float* alpha, const float* x, int incx,
                             const float* y, int incy, float* A, int lda)
{
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) A[i + (size_t)j * lda] += *alpha * x[(size_t)i * incx] * y[(size_t)j * incy];
    return CUBLAS_STATUS_SUCCESS;
}
