/* Host stand-in for the one MPI call on the reference's factorization path: MPI_Wtime
 * (oocdag.cpp:51,90).  TEST INFRASTRUCTURE ONLY. */
#ifndef OOC_REF_SHIM_MPI_H
#define OOC_REF_SHIM_MPI_H
#ifdef __cplusplus
extern "C" {
#endif
double MPI_Wtime(void);
#ifdef __cplusplus
}
#endif
#endif
