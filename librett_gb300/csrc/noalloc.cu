// One-shot transpose that allocates no device memory.
//
// Who needs it: callers that may not allocate device memory once they are
// running, for example a serving process whose device memory is entirely
// reserved up front by its own caching allocator, or a latency-critical loop
// where cudaMalloc / cudaMallocAsync (and the implicit synchronisation or
// pool growth they can cause) is forbidden.  librettPlan allocates the
// offset tables of flat-pipeline plans, so such callers use this entry
// point instead.
//
// How: flat and bulk-copy tiles of at most ARITH_MAX_NTR ranks compute
// their addresses and need no tables; a bulk-copy plan's status word is a
// slot of a static device array (bulkStatusWord).  Larger tiles read offset
// tables from global memory; here those tables live in a fixed file-scope
// device array (every GPU that loads the library holds it until the process
// exits).  A small kernel (writeDeviceTables) writes the tables of the
// current problem into it, then the transpose runs on them, both on the
// caller's stream.  Host code cannot use the array's name as a device
// address; its address is obtained per device with cudaGetSymbolAddress on
// the first call made with that device current.
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>
#include <vector>

#include "kernels.cuh"
#include "launch.h"
#include "librett.h"
#include "librett_c.h"
#include "plan.h"
#include "plans.h"
#include "select.h"

namespace lt {
namespace {

// Capacity of the shared scratch array.  Offset tables take at most
// 10 bytes per tile element (4096 elements for the largest tile), rounded
// for alignment, so every tile the planner produces fits.
constexpr size_t kScratchBytes = 64 * 1024;

__device__ __align__(256) unsigned char gTableScratch[kScratchBytes];

std::mutex gScratchMu;
std::unordered_map<int, unsigned char*> gScratch;

// Per-device set-up, done by the first call with that device current:
// resolve the array's device address (the host-side symbol is only a
// stand-in).  The address is kept for the life of the process, keyed by
// device ordinal; after a cudaDeviceReset of a device already used here it
// is stale, so this entry point (like the library's plan-table arena) is
// not supported across a device reset.
cudaError_t scratchFor(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(gScratchMu);
  auto it = gScratch.find(dev);
  if (it != gScratch.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  void* p = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&p, gTableScratch);
  if (err != cudaSuccess) return err;
  gScratch[dev] = static_cast<unsigned char*>(p);
  *out = static_cast<unsigned char*>(p);
  return cudaSuccess;
}

}  // namespace
}  // namespace lt

extern "C" int librett_c_transpose_noalloc(int rank, const int* dim, const int* permutation,
                                           size_t sizeofType, void* stream, const void* idata,
                                           void* odata) {
  using namespace lt;
  if (checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  if (idata == nullptr || odata == nullptr || idata == odata) return LIBRETT_INVALID_PARAMETER;
  const size_t a = sizeofType < 16 ? sizeofType : 16;
  if ((uintptr_t)idata % a != 0 || (uintptr_t)odata % a != 0) return LIBRETT_INVALID_PARAMETER;
  // the device, its SM count and name as librettPlan sees them, so both
  // paths rank candidates with the same (device-keyed) selector
  int dev = 0, sms = 0;
  const char* devName = nullptr;
  if (!currentDevice(dev, sms, &devName)) return LIBRETT_INTERNAL_ERROR;
  unsigned char* scratch = nullptr;
  if (scratchFor(dev, &scratch) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  cudaStream_t s = (cudaStream_t)stream;

  Fused f;
  fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  std::vector<PlanDesc> cands = enumerateCandidates(f, sms, true);
  if (cands.empty()) return LIBRETT_INTERNAL_ERROR;
  int pick = choosePlan(cands, sms, devName, nullptr);
  // Tile problems run the flat pipeline, whose tables go to the scratch.
  if (cands[pick].kernel == K_TILE && !flatTables(cands[pick].pipe)) {
    int flat = -1;
    for (size_t c = 0; c < cands.size(); ++c)
      if (cands[c].kernel == K_TILE && cands[c].pipe == PIPE_FLAT &&
          (flat < 0 || cands[c].cost < cands[flat].cost))
        flat = (int)c;
    if (flat >= 0) pick = flat;
  }
  if (!refineCandidate(cands[pick], sms) || !finalizePlan(cands[pick]))
    return LIBRETT_INTERNAL_ERROR;
  PlanDesc& pd = cands[pick];
  DeviceTables dt;
  const bool vecOk = ((uintptr_t)idata % 16 == 0 && (uintptr_t)odata % 16 == 0) ||
                     (pd.tile.lv == 1 && pd.tile.sv == 1);
  if (pd.kernel == K_TILE && pd.pipe == PIPE_BULK && vecOk) {
    // the status word of a one-shot call has no reader; it only keeps the
    // timed-out path of the kernel well defined
    pd.tile.statusTag = nextStatusTag();
    if (bulkStatusWord(pd.tile.statusTag, &dt.status) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  }
  if (needsDeviceTables(pd) && vecOk) {
    size_t stOffset, smOffset;
    if (deviceTableBytes(pd.tile, &stOffset, &smOffset) > kScratchBytes)
      return LIBRETT_INVALID_PARAMETER;  // tables exceed the scratch
    if (writeDeviceTables(pd.tile, scratch, s, &dt) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  }
  int grid = 0;
  if (launchPlan(pd, &dt, idata, odata, s, sms, &grid) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  return LIBRETT_SUCCESS;
}
