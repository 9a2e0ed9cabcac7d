// Controls of the host stand-ins (shim.cpp) used by the compiled-reference harness.
// TEST INFRASTRUCTURE ONLY.
#ifndef OOC_REF_SHIM_H
#define OOC_REF_SHIM_H

#include "quark.h"

#ifdef __cplusplus
extern "C" {
#endif
// Load the host BLAS/LAPACK (symbols `<prefix>dgemm_` etc.).  0 on success.
int ooc_shim_init_blas(const char* path, const char* prefix);
// 1: tasks are counted but not run, and cudaMalloc returns untouchable address space.
void ooc_shim_set_dry(int dry);
// Tasks inserted so far whose body is `fn`.
long long ooc_shim_task_count(void (*fn)(Quark*));
// LAPACK info of the first dpotrf_ call that failed (0 if none did).
int ooc_shim_first_potrf_failure(void);
#ifdef __cplusplus
}
#endif

#endif
