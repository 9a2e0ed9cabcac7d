/*
 * ooc_offload.h -- the reference's tile-offload interface (efdazedo/oocdag ooc_offload.h:28-64),
 * same names and argument lists, executed on a GB300 instead of a Xeon Phi.
 *
 * The reference compiled these only for its MIC build (ooc_offload.cpp:1, USE_MIC) and ran
 * MKL inside Intel offload regions through 32 MB per-thread bounce buffers
 * (ooc_offload.cpp:3-11).  Here:
 *   - device pointers come from offload_Alloc (device memory of the GPU chosen by
 *     offload_init: rank % number of devices, as ooc_offload.cpp:13-19);
 *   - `r` (the QUARK worker rank, ooc_offload.cpp:99) selects a per-worker CUDA stream;
 *     every call returns when its work on that stream has finished, as the reference's
 *     offload regions did;
 *   - the BLAS/LAPACK calls run the library's own sm_103a kernels (FP64 DMMA contraction,
 *     device potrf, blocked column solve); no cuBLAS/cuSOLVER.
 * MKL_INT is the LP64 int.  All functions have C linkage (the reference's were C++ except
 * offload_init_/offload_destroy_).  Errors: the BLAS-style calls return void as in the
 * reference; ooc_offload_last_error() reports the last failure (0 = none).
 */
#ifndef OOC_OFFLOAD_H
#define OOC_OFFLOAD_H

#include <stddef.h>
#include <stdint.h>

#ifndef MKL_INT
#define MKL_INT int
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ooc_offload.h:28-31 */
void offload_init(int *myrank, int *mydevice);
void offload_init_(int *myrank, int *mydevice);
void offload_destroy(void);
void offload_destroy_(void);

/* memory management, ooc_offload.h:34-36 */
intptr_t offload_Alloc(size_t size, int r);
void offload_touch(void *p, size_t size, int r);
void offload_Free(void *p, int r);

/* host <-> device copies, ooc_offload.h:39-44 (x / A on the host, y / B on the device for
 * Set*, the reverse for Get*) */
void offload_dSetVector(int n, double *x, int incx, double *y, int incy, int r);
void offload_dGetVector(int n, double *x, int incx, double *y, int incy, int r);
void offload_dSetMatrix(int rows, int cols, double *A, int lda, double *B, int ldb, int r);
void offload_dGetMatrix(int rows, int cols, double *A, int lda, double *B, int ldb, int r);
void offload_dtrSetMatrix(char uplo, int rows, int cols, double *A, int lda, double *B, int ldb, int r);
void offload_dtrGetMatrix(char uplo, int rows, int cols, double *A, int lda, double *B, int ldb, int r);

/* level 1, ooc_offload.h:47 (device x, y) */
void offload_dcopy(int n, const double *x, int incx, double *y, int incy, int r);

/* level 3, ooc_offload.h:50-60 (device a, b, c) */
void offload_dgemm(const char *transa, const char *transb, const MKL_INT *m, const MKL_INT *n, const MKL_INT *k,
                   const double *alpha, const double *a, const MKL_INT *lda, const double *b, const MKL_INT *ldb,
                   const double *beta, double *c, const MKL_INT *ldc, int r);
void offload_dsyrk(const char *uplo, const char *trans, const MKL_INT *n, const MKL_INT *k, const double *alpha,
                   const double *a, const MKL_INT *lda, const double *beta, double *c, const MKL_INT *ldc, int r);
void offload_dtrsm(const char *side, const char *uplo, const char *transa, const char *diag, const MKL_INT *m,
                   const MKL_INT *n, const double *alpha, const double *a, const MKL_INT *lda, double *b,
                   const MKL_INT *ldb, int r);

/* factorization, ooc_offload.h:63-64 (device a; *info as LAPACK dpotrf) */
void offload_dpotrf(const char *uplo, const MKL_INT *n, double *a, const MKL_INT *lda, MKL_INT *info, int r);

/* Last error of the offload layer on this thread: 0, a negative argument position, or an
 * OOC_ERR_* code (oocdag_gb300.h).  No reference counterpart (the reference asserted). */
int ooc_offload_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* OOC_OFFLOAD_H */
