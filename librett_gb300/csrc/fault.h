// Host-side fault injection and allocation counters (test hooks).
//
// LibreTT exits the process on any CUDA error (src/GpuUtils.h:47-56); this
// library returns LIBRETT_INTERNAL_ERROR instead and stays usable.  To test
// those paths without making a GPU fail, a site can be armed to report a
// CUDA error on the host, before the real call is made: after `after`
// further calls at that site pass, the next one returns the site's error
// (cudaErrorMemoryAllocation for allocations, cudaErrorLaunchFailure for
// launches) and the site disarms itself.  Nothing is sent to the device.
#pragma once

namespace lt {

enum FaultSite {
  FAULT_TABLE_ALLOC = 0,  // plan-table arena allocation (librettPlan / PlanMeasure)
  FAULT_GROUP_ALLOC = 1,  // device image of a group (librettGroupCreate)
  FAULT_LAUNCH = 2,       // any transpose launch (execute, group, no-allocation path)
  FAULT_SITES = 3
};

// True when an armed failure at `site` fires on this call (one-shot).
bool injectFault(int site);

// Arms site (after >= 0) or disarms it (after < 0).  False for a bad site.
bool armFault(int site, long long after);

// Device-memory requests the table arena made: slab bytes obtained with
// cudaMalloc, blocks handed out, and bytes from the stream-ordered pool.
void tableArenaStats(long long* slabBytes, long long* blocks, long long* poolBytes);

}  // namespace lt
