// cuBLAS interface subset for the CPU emulation of the reference
// (TEST INFRASTRUCTURE ONLY): BLAS semantics (1-based i?amax/i?amin returning
// the first extremum, |Re|+|Im| for complex).
#ifndef CUBLAS_API_H_
#define CUBLAS_API_H_

#include <cuComplex.h>

typedef struct cublasContext* cublasHandle_t;

typedef enum {
    CUBLAS_STATUS_SUCCESS = 0,
    CUBLAS_STATUS_NOT_INITIALIZED = 1,
    CUBLAS_STATUS_ALLOC_FAILED = 3,
    CUBLAS_STATUS_INVALID_VALUE = 7,
    CUBLAS_STATUS_ARCH_MISMATCH = 8,
    CUBLAS_STATUS_MAPPING_ERROR = 11,
    CUBLAS_STATUS_EXECUTION_FAILED = 13,
    CUBLAS_STATUS_INTERNAL_ERROR = 14,
    CUBLAS_STATUS_NOT_SUPPORTED = 15,
    CUBLAS_STATUS_LICENSE_ERROR = 16
} cublasStatus_t;

cublasStatus_t cublasCreate_v2(cublasHandle_t* handle);
cublasStatus_t cublasDestroy_v2(cublasHandle_t handle);
cublasStatus_t cublasIsamax_v2(cublasHandle_t h, int n, const float* x, int incx, int* result);
cublasStatus_t cublasIsamin_v2(cublasHandle_t h, int n, const float* x, int incx, int* result);
cublasStatus_t cublasIcamax_v2(cublasHandle_t h, int n, const cuComplex* x, int incx, int* result);
cublasStatus_t cublasSscal_v2(cublasHandle_t h, int n, const float* alpha, float* x, int incx);
cublasStatus_t cublasCsscal_v2(cublasHandle_t h, int n, const float* alpha, cuComplex* x, int incx);
cublasStatus_t cublasDger_v2(cublasHandle_t h, int m, int n, const double* alpha, const double* x, int incx,
                             const double* y, int incy, double* A, int lda);
cublasStatus_t cublasSger_v2(cublasHandle_t h, int m, int n, const float* alpha, const float* x, int incx,
                             const float* y, int incy, float* A, int lda);

#define cublasCreate cublasCreate_v2
#define cublasDestroy cublasDestroy_v2
#define cublasIsamax cublasIsamax_v2
#define cublasIsamin cublasIsamin_v2
#define cublasIcamax cublasIcamax_v2
#define cublasSscal cublasSscal_v2
#define cublasCsscal cublasCsscal_v2
#define cublasDger cublasDger_v2
#define cublasSger cublasSger_v2

#endif
