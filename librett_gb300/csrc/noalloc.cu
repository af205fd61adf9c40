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
// How: the flat tile kernel reads its offset tables from global memory.
// Here those tables live in a fixed file-scope device array (every GPU that
// loads the library holds it until the process exits).  A small kernel
// (writeDeviceTables) writes the tables of the current problem into it, then
// the transpose runs on them, both on the caller's stream.  Host code cannot use the array's
// name as a device address; its address is obtained per device with
// cudaGetSymbolAddress on the first call made with that device current.
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>
#include <vector>

#include "kernels.cuh"
#include "launch.h"
#include "librett.h"
#include "librett_c.h"
#include "plan.h"
#include "select.h"

namespace lt {
namespace {

// Capacity of the shared scratch array.  Offset tables take at most
// 10 bytes per tile element (4096 elements for the largest tile), rounded
// for alignment, so every tile the planner produces fits.
constexpr size_t kScratchBytes = 64 * 1024;

__device__ __align__(256) unsigned char gTableScratch[kScratchBytes];

struct DeviceScratch {
  unsigned char* ptr = nullptr;
  int numSMs = 0;
};

std::mutex gScratchMu;
std::unordered_map<int, DeviceScratch> gScratch;

// Per-device set-up, done by the first call with that device current:
// resolve the array's device address (the host-side symbol is only a
// stand-in) and the SM count.
cudaError_t scratchFor(int dev, DeviceScratch& out) {
  std::lock_guard<std::mutex> lk(gScratchMu);
  auto it = gScratch.find(dev);
  if (it != gScratch.end()) {
    out = it->second;
    return cudaSuccess;
  }
  DeviceScratch ds;
  void* p = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&p, gTableScratch);
  if (err != cudaSuccess) return err;
  err = cudaDeviceGetAttribute(&ds.numSMs, cudaDevAttrMultiProcessorCount, dev);
  if (err != cudaSuccess) return err;
  ds.ptr = static_cast<unsigned char*>(p);
  gScratch[dev] = ds;
  out = ds;
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
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  DeviceScratch ds;
  if (scratchFor(dev, ds) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  cudaStream_t s = (cudaStream_t)stream;

  Fused f;
  fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  std::vector<PlanDesc> cands = enumerateCandidates(f, ds.numSMs, true);
  if (cands.empty()) return LIBRETT_INTERNAL_ERROR;
  int pick = choosePlan(cands, ds.numSMs, nullptr, nullptr);
  // Tile problems run the flat pipeline, whose tables go to the scratch.
  if (cands[pick].kernel == K_TILE && cands[pick].pipe != PIPE_FLAT) {
    int flat = -1;
    for (size_t c = 0; c < cands.size(); ++c)
      if (cands[c].kernel == K_TILE && cands[c].pipe == PIPE_FLAT &&
          (flat < 0 || cands[c].cost < cands[flat].cost))
        flat = (int)c;
    if (flat >= 0) pick = flat;
  }
  if (!refineCandidate(cands[pick], ds.numSMs) || !finalizePlan(cands[pick]))
    return LIBRETT_INTERNAL_ERROR;
  const PlanDesc& pd = cands[pick];
  DeviceTables dt;
  const bool vecOk = ((uintptr_t)idata % 16 == 0 && (uintptr_t)odata % 16 == 0) ||
                     (pd.tile.lv == 1 && pd.tile.sv == 1);
  if (pd.kernel == K_TILE && pd.pipe == PIPE_FLAT && vecOk) {
    size_t stOffset, smOffset;
    if (deviceTableBytes(pd.tile, &stOffset, &smOffset) > kScratchBytes)
      return LIBRETT_INVALID_PARAMETER;  // tables exceed the scratch
    if (writeDeviceTables(pd.tile, ds.ptr, s, &dt) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  }
  int grid = 0;
  if (launchPlan(pd, &dt, idata, odata, s, ds.numSMs, &grid) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  return LIBRETT_SUCCESS;
}
