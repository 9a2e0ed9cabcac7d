/* Host stand-in for the BLACS grid calls of the reference's main (oocdag.cpp:258-262,
 * 470-471): a 1 x 1 process grid.  TEST INFRASTRUCTURE ONLY; main itself is compiled
 * but never run by the recipe. */
#ifndef OOC_REF_SHIM_MKL_BLACS_H
#define OOC_REF_SHIM_MKL_BLACS_H
#ifdef __cplusplus
extern "C" {
#endif
void blacs_pinfo_(int* iam, int* nprocs);
void blacs_get_(const int* ctxt, const int* what, int* val);
void blacs_gridinit_(int* ctxt, const char* order, const int* nprow, const int* npcol);
void blacs_gridinfo_(const int* ctxt, int* nprow, int* npcol, int* myrow, int* mycol);
void blacs_gridexit_(const int* ctxt);
void blacs_exit_(const int* cont);
#ifdef __cplusplus
}
#endif
#endif
