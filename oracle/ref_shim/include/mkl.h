/* Host stand-in for the Intel MKL (composer_xe_2015.0.090) LAPACK routine on the
 * reference's factorization path: dpotrf_ (oocquark.cpp:87, under USE_HOST_DPOTRF).
 * TEST INFRASTRUCTURE ONLY: forwarded to the host LAPACK (same Fortran definition). */
#ifndef OOC_REF_SHIM_MKL_H
#define OOC_REF_SHIM_MKL_H
#ifdef __cplusplus
extern "C" {
#endif
void dpotrf_(const char* uplo, const int* n, double* A, const int* lda, int* info);
#ifdef __cplusplus
}
#endif
#endif
