/*
 * ref_budget.h — force-included (nvcc -include) when compiling the Subway
 * reference's shared/subgraph.cu for the reference arm of the benchmark.
 *
 * The reference sizes its device edge buffer from
 * cudaDeviceProp::totalGlobalMem (shared/subgraph.cu:16,24) and has no budget
 * flag.  This header wraps the property query so that, when the environment
 * variable SUBWAY_BUDGET_BYTES is set, totalGlobalMem reads as that many
 * bytes.  No reference source line changes.
 */
#ifndef SGW_REF_BUDGET_H
#define SGW_REF_BUDGET_H
#include <cuda_runtime.h>
#include <stdlib.h>

static inline cudaError_t sgw_ref_device_properties(struct cudaDeviceProp *prop, int device) {
  cudaError_t e = cudaGetDeviceProperties(prop, device);
  const char *b = getenv("SUBWAY_BUDGET_BYTES");
  if (e == cudaSuccess && b) {
    unsigned long long v = strtoull(b, 0, 10);
    if (v > 0 && v < prop->totalGlobalMem) prop->totalGlobalMem = (size_t)v;
  }
  return e;
}
#define cudaGetDeviceProperties sgw_ref_device_properties
#endif
