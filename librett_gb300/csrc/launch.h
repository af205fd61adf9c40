// Host-side launch interface of the kernels (kernels.cuh holds the device
// code and is only included by the .cu translation units).
#pragma once

#include <cuda_runtime.h>

#include "plan.h"

namespace lt {

// Launch whatever the plan describes on stream s.  Uses the 16-byte unit
// variant when both pointers allow it, else the element-size one.  *grid
// receives the number of CTAs launched.
cudaError_t launchPlan(const PlanDesc& pd, const void* in, void* out, cudaStream_t s, int numSMs,
                       int* grid);

// CTAs per SM of a kernel at a given dynamic smem size (cached per device);
// raises the kernel's dynamic-smem limit when smem exceeds 48 KB.
int cachedOccupancy(const void* func, int threads, int smem);

}  // namespace lt
