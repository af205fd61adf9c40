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
  // Bulk-copy plans: the plan's status word (bulkStatusWord), to which a
  // launch whose wait for its copies ran out of time writes the plan's
  // status tag (see tileKernelBulk) before skipping its stores.
  unsigned* status = nullptr;
};

// Tag for a new bulk-copy plan's status word: nonzero, never repeated
// within 2^32 plans.
uint32_t nextStatusTag();

// The status word of tag on the current device: one of BULK_STATUS_SLOTS
// words of a zero-initialised device array (no allocation, no launch), at
// tag mod BULK_STATUS_SLOTS.  A launch that times out writes its tag there,
// so the word equals a plan's tag exactly when a launch of that plan timed
// out and no plan sharing the word timed out after it.
constexpr uint32_t BULK_STATUS_SLOTS = 1u << 16;
cudaError_t bulkStatusWord(uint32_t tag, unsigned** word);

// Tables of a tile plan whose kernels read offset tables (flat and bulk-copy
// pipelines with more than ARITH_MAX_NTR tile ranks): allocated from the
// library's per-device table arena (stream-ordered reuse) and written by a
// kernel on s.  Other plans need none (*alloc = nullptr): no allocation and
// no launch; a bulk-copy plan gets its status word (pd.tile.statusTag).
cudaError_t createDeviceTables(const PlanDesc& pd, cudaStream_t s, void** alloc, DeviceTables* dt);

// Whether createDeviceTables allocates and writes tables for pd.
inline bool needsDeviceTables(const PlanDesc& pd) {
  return pd.kernel == K_TILE && flatTables(pd.pipe) && arithRanks(pd.tile) == 0;
}

// Releases them in stream order: reusable at once by plans on s, by plans on
// other streams once s has passed this point.
void destroyDeviceTables(void* alloc, cudaStream_t s);

// Device-table layout of a tile: total bytes; ldOff at 0, stOff at
// *stOffset, stSm at *smOffset (16-byte aligned).
size_t deviceTableBytes(const TileParams& tp, size_t* stOffset, size_t* smOffset);

// Launches a kernel on s that writes the tables of tp at base (which must
// hold deviceTableBytes), and points *dt's table pointers at them.
cudaError_t writeDeviceTables(const TileParams& tp, unsigned char* base, cudaStream_t s,
                              DeviceTables* dt);

// Launch whatever the plan describes on stream s.  Uses the 16-byte unit
// variant when both pointers allow it, else the element-size one.  *grid
// receives the number of CTAs launched.  dt: the plan's device tables and
// status word (flat and bulk-copy pipelines).
cudaError_t launchPlan(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                       cudaStream_t s, int numSMs, int* grid);

// Flat and bulk-copy tile launches per element size and tile rank count
// (A: 0..2 ranks, 0 = offset tables; B: 3..4; C: 5..6), defined in
// k_flat<ES>_<a|b|c>.cu.
#define LT_DECLARE_FLAT(NAME)                                                              \
  cudaError_t NAME(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out, \
                   cudaStream_t s, int* grid);
LT_DECLARE_FLAT(launchFlat4A)
LT_DECLARE_FLAT(launchFlat4B)
LT_DECLARE_FLAT(launchFlat4C)
LT_DECLARE_FLAT(launchFlat8A)
LT_DECLARE_FLAT(launchFlat8B)
LT_DECLARE_FLAT(launchFlat8C)
LT_DECLARE_FLAT(launchFlat16A)
LT_DECLARE_FLAT(launchFlat16B)
LT_DECLARE_FLAT(launchFlat16C)
#undef LT_DECLARE_FLAT

// CTAs per SM of a kernel at a given dynamic smem size (cached per device);
// raises the kernel's dynamic-smem limit when smem exceeds 48 KB.
int cachedOccupancy(const void* func, int threads, int smem);

}  // namespace lt
