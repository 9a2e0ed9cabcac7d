/* Host stand-in for the two CUDA runtime calls the reference driver makes
 * (oocdag.cpp:41-43 cudaMalloc, :96-98 cudaFree).  TEST INFRASTRUCTURE ONLY: "device"
 * memory is page-aligned host memory; in the shim's dry-run mode it is an inaccessible
 * address range that is never touched (only addresses are formed from it). */
#ifndef OOC_REF_SHIM_CUDA_RUNTIME_H
#define OOC_REF_SHIM_CUDA_RUNTIME_H

#include <stddef.h>

typedef enum { cudaSuccess = 0, cudaErrorMemoryAllocation } cudaError_t;

#ifdef __cplusplus
extern "C" {
#endif
cudaError_t cudaMalloc(void** p, size_t bytes);
cudaError_t cudaFree(void* p);
#ifdef __cplusplus
}
#endif

#endif
