/* Host stand-in for the cuBLAS v2 calls the reference makes (oocquark.cpp:27,57,130,176,
 * 222; oocdag.cpp:279-282).  TEST INFRASTRUCTURE ONLY.  "Device" memory is host memory
 * (see cuda_runtime.h here); the level-3 calls run the host BLAS with the same
 * arguments (Fortran BLAS definitions of dtrsm, dsyrk and dgemm), so the reference's own
 * task bodies produce their results on the CPU.  Enumerator values are this shim's own. */
#ifndef OOC_REF_SHIM_CUBLAS_V2_H
#define OOC_REF_SHIM_CUBLAS_V2_H

#include "cuda_runtime.h"

typedef struct ooc_shim_cublas* cublasHandle_t;
typedef enum {
  CUBLAS_STATUS_SUCCESS = 0,
  CUBLAS_STATUS_NOT_INITIALIZED,
  CUBLAS_STATUS_ALLOC_FAILED,
  CUBLAS_STATUS_INVALID_VALUE,
  CUBLAS_STATUS_MAPPING_ERROR,
  CUBLAS_STATUS_EXECUTION_FAILED,
  CUBLAS_STATUS_INTERNAL_ERROR
} cublasStatus_t;
typedef enum { CUBLAS_FILL_MODE_LOWER = 0, CUBLAS_FILL_MODE_UPPER } cublasFillMode_t;
typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T, CUBLAS_OP_C } cublasOperation_t;
typedef enum { CUBLAS_SIDE_LEFT = 0, CUBLAS_SIDE_RIGHT } cublasSideMode_t;
typedef enum { CUBLAS_DIAG_NON_UNIT = 0, CUBLAS_DIAG_UNIT } cublasDiagType_t;

#ifdef __cplusplus
extern "C" {
#endif
cublasStatus_t cublasCreate(cublasHandle_t* h);
cublasStatus_t cublasDestroy(cublasHandle_t h);
cublasStatus_t cublasSetMatrix(int rows, int cols, int elemSize, const void* A, int lda, void* B, int ldb);
cublasStatus_t cublasGetMatrix(int rows, int cols, int elemSize, const void* A, int lda, void* B, int ldb);
cublasStatus_t cublasDtrsm_v2(cublasHandle_t h, cublasSideMode_t side, cublasFillMode_t uplo,
                              cublasOperation_t trans, cublasDiagType_t diag, int m, int n,
                              const double* alpha, const double* A, int lda, double* B, int ldb);
cublasStatus_t cublasDsyrk_v2(cublasHandle_t h, cublasFillMode_t uplo, cublasOperation_t trans, int n, int k,
                              const double* alpha, const double* A, int lda, const double* beta, double* C,
                              int ldc);
cublasStatus_t cublasDgemm_v2(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                              const double* alpha, const double* A, int lda, const double* B, int ldb,
                              const double* beta, double* C, int ldc);
#ifdef __cplusplus
}
#endif

#endif
