// Host-side launch interface of the kernels (kernels.cuh holds the device
// code and is only included by the .cu translation units).
#pragma once

#include <cuda_runtime.h>

#include "plan.h"

namespace lt {

// Offset tables of a flat-pipeline tile plan, in device memory.
struct DeviceTables {
  const int* ldOff = nullptr;
  const int* stOff = nullptr;
  const unsigned short* stSm = nullptr;
  // Status word after the tables, zero when written; a bulk-copy launch
  // whose wait for its copies ran out of time sets bit 0 (see
  // tileKernelBulk) and skips its stores.
  unsigned* status = nullptr;
};

// Allocates the plan's tables (from the library's per-device table arena,
// stream-ordered reuse) and writes them with a kernel on s.  Plans of other
// pipelines need none: *alloc = nullptr.
cudaError_t createDeviceTables(const PlanDesc& pd, cudaStream_t s, void** alloc, DeviceTables* dt);

// Releases them in stream order: reusable at once by plans on s, by plans on
// other streams once s has passed this point.
void destroyDeviceTables(void* alloc, cudaStream_t s);

// Device-table layout of a tile: total bytes; ldOff at 0, stOff at
// *stOffset, stSm at *smOffset (16-byte aligned), then a 16-byte status
// block.
size_t deviceTableBytes(const TileParams& tp, size_t* stOffset, size_t* smOffset);
size_t statusOffset(const TileParams& tp, size_t smOffset);

// Launches a kernel on s that writes the tables of tp at base (which must
// hold deviceTableBytes), and points *dt at them.
cudaError_t writeDeviceTables(const TileParams& tp, unsigned char* base, cudaStream_t s,
                              DeviceTables* dt);

// Launch whatever the plan describes on stream s.  Uses the 16-byte unit
// variant when both pointers allow it, else the element-size one.  *grid
// receives the number of CTAs launched.  dt: the plan's device tables (flat
// pipeline only).
cudaError_t launchPlan(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                       cudaStream_t s, int numSMs, int* grid);

// CTAs per SM of a kernel at a given dynamic smem size (cached per device);
// raises the kernel's dynamic-smem limit when smem exceeds 48 KB.
int cachedOccupancy(const void* func, int threads, int smem);

}  // namespace lt
