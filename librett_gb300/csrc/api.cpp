// Public interface: the librett.h C++ functions (same signatures and mangled
// names as LibreTT's src/librett.h) and the librett_c.h extern "C" wrappers.
//
// LibreTT counterparts: src/librett.cpp:45-49 (handle table), :57-83
// (getDeviceProp), :85-108 (input check), :110-222 (librettPlan), :224-343
// (librettPlanMeasure), :351-370 (librettDestroy), :372-385 (librettExecute).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "fault.h"
#include "launch.h"
#include "librett.h"
#include "librett_c.h"
#include "plan.h"
#include "plans.h"
#include "select.h"

namespace lt {
extern std::atomic<unsigned long long> gLaunchCount;
}

namespace {

using lt::PlanObj;

// Plans are held by shared_ptr so that an execute that has looked a plan up
// keeps it alive while a concurrent destroy removes it from the table.  The
// table lock is not held during the launch (LibreTT holds its mutex across
// the launch, src/librett.cpp:375).
std::shared_mutex gPlanMu;
std::unordered_map<librettHandle, std::shared_ptr<PlanObj>> gPlans;
std::atomic<librettHandle> gNextHandle{0};

struct DevInfo {
  int sms = 0;
  std::string name;
};
std::mutex gDevMu;
std::unordered_map<int, DevInfo> gDevs;

}  // namespace

bool lt::currentDevice(int& dev, int& sms, const char** name) {
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(gDevMu);
  auto it = gDevs.find(dev);
  if (it == gDevs.end()) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return false;
    DevInfo di;
    di.sms = prop.multiProcessorCount;
    di.name = prop.name;
    it = gDevs.emplace(dev, di).first;
  }
  sms = it->second.sms;
  // entries are never erased and map nodes do not move: the name stays valid
  if (name) *name = it->second.name.c_str();
  return true;
}

bool lt::currentDevice(int& dev, int& sms, std::string* name) {
  const char* n = nullptr;
  if (!currentDevice(dev, sms, &n)) return false;
  if (name) *name = n;
  return true;
}

namespace {

using lt::currentDevice;

bool aligned(const void* p, size_t esize) {
  size_t a = esize < 16 ? esize : 16;
  return ((uintptr_t)p % a) == 0;
}

librettHandle storePlan(std::shared_ptr<PlanObj> obj) {
  librettHandle h = gNextHandle.fetch_add(1);
  std::unique_lock<std::shared_mutex> lk(gPlanMu);
  gPlans[h] = std::move(obj);
  return h;
}

}  // namespace

namespace lt {

std::shared_ptr<PlanObj> findPlan(librettHandle h) {
  std::shared_lock<std::shared_mutex> lk(gPlanMu);
  auto it = gPlans.find(h);
  if (it == gPlans.end()) return nullptr;
  return it->second;
}

}  // namespace lt

namespace {

using lt::findPlan;

void fillInfo(const lt::PlanDesc& pd, int grid, librett_plan_info* info) {
  std::memset(info, 0, sizeof(*info));
  info->method = pd.method;
  info->element_bytes = pd.f.esize;
  info->fused_rank = pd.f.rank;
  for (int r = 0; r < pd.f.rank; ++r) {
    info->fused_dim[r] = pd.f.dim[r];
    info->fused_perm[r] = pd.f.perm[r];
    info->tile_extent[r] = pd.extent[r];
  }
  info->volume = pd.f.vol;
  info->num_tiles = pd.numWork;
  info->threads = pd.threads;
  info->slots = pd.slots;
  info->smem_bytes = pd.smemBytes;
  info->pad_shift = pd.padShift;
  info->pipeline = pd.pipe;
  info->unit_in_bytes = pd.unitBytes;
  info->unit_out_bytes = pd.kernel == lt::K_TILE ? pd.unitOutBytes : pd.unitBytes;
  info->run_in_bytes = pd.runInBytes;
  info->run_out_bytes = pd.runOutBytes;
  info->grid = grid;
  info->candidate = pd.candidate;
  info->num_candidates = pd.numCandidates;
  info->model_cost = pd.cost;
  if (lt::needsDeviceTables(pd)) {
    size_t st, sm;
    info->table_bytes = (int)lt::deviceTableBytes(pd.tile, &st, &sm);
  }
}

void fillInfo(const PlanObj& obj, librett_plan_info* info) {
  fillInfo(obj.pd, obj.lastGrid, info);
  info->selected_by = obj.selectedBy;
}

// Creates the plan object (device tables included) and stores it.
librettResult activate(librettHandle* handle, const lt::PlanDesc& pd, cudaStream_t stream, int dev,
                       int sms, int selectedBy) {
  auto obj = std::make_shared<PlanObj>();
  obj->pd = pd;
  if (pd.pipe == lt::PIPE_BULK) obj->pd.tile.statusTag = lt::nextStatusTag();
  obj->selectedBy = selectedBy;
  obj->stream = stream;
  obj->device = dev;
  obj->numSMs = sms;
  if (lt::createDeviceTables(obj->pd, stream, &obj->tablesAlloc, &obj->tables) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  *handle = storePlan(std::move(obj));
  return LIBRETT_SUCCESS;
}

// Shared by librettPlan and librett_c_plan_candidate: plan with the given
// candidate (or the heuristic's choice when candidate < 0).
// Plan cache: the planner's choice per (device, fused problem), so that a
// repeated shape skips candidate enumeration and selection (LibreTT re-plans
// every call; its launch-configuration LRU, src/kernel.cpp:671-691, caches
// only occupancy).  Least recently used entries are evicted beyond the
// capacity (LIBRETT_PLAN_CACHE entries, default 4096; 0 disables).  Cleared
// whenever the selector, its model or the candidate set changes.
struct CachedPlan {
  lt::PlanDesc pd;
  int selectedBy;
};
std::mutex gCacheMu;
std::list<std::pair<std::string, CachedPlan>> gCacheLru;  // most recent first
std::unordered_map<std::string, std::list<std::pair<std::string, CachedPlan>>::iterator> gCache;
int gCacheCap = -1;
long long gCacheHits = 0, gCacheMisses = 0;

int cacheCapacityLocked() {
  if (gCacheCap < 0) {
    const char* e = std::getenv("LIBRETT_PLAN_CACHE");
    gCacheCap = e != nullptr && *e ? std::max(0, std::atoi(e)) : 4096;
  }
  return gCacheCap;
}

void cacheClear() {
  std::lock_guard<std::mutex> lk(gCacheMu);
  gCache.clear();
  gCacheLru.clear();
}

std::string cacheKey(const lt::Fused& f, int dev, int sms) {
  std::string k;
  auto put = [&](long long v) { k.append(reinterpret_cast<const char*>(&v), sizeof(v)); };
  put(dev);
  put(sms);
  put(f.rank);
  put(f.esize);
  for (int r = 0; r < f.rank; ++r) {
    put(f.dim[r]);
    put(f.perm[r]);
  }
  return k;
}

librettResult planImpl(librettHandle* handle, int rank, const int* dim, const int* perm,
                       size_t sizeofType, cudaStream_t stream, int candidate) {
  if (handle == nullptr) return LIBRETT_INVALID_PARAMETER;
  if (lt::checkInput(rank, dim, perm, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  int dev = 0, sms = 0;
  const char* devName = nullptr;
  if (!currentDevice(dev, sms, &devName)) return LIBRETT_INTERNAL_ERROR;
  lt::Fused f;
  lt::fuseRanks(rank, dim, perm, (int)sizeofType, f);
  std::string key;
  bool cached = false;  // the cache is on (no key is built when it is off)
  if (candidate < 0) {
    {
      std::lock_guard<std::mutex> lk(gCacheMu);
      cached = cacheCapacityLocked() > 0;
    }
    if (cached) {
      key = cacheKey(f, dev, sms);
      std::unique_lock<std::mutex> lk(gCacheMu);
      auto it = gCache.find(key);
      if (it != gCache.end()) {
        gCacheLru.splice(gCacheLru.begin(), gCacheLru, it->second);
        ++gCacheHits;
        const CachedPlan hit = it->second->second;
        lk.unlock();
        return activate(handle, hit.pd, stream, dev, sms, hit.selectedBy);
      }
      ++gCacheMisses;
    }
  }
  // rank the screened candidates, then complete the chosen one
  std::vector<lt::PlanDesc> cands = lt::enumerateCandidates(f, sms, true);
  if (cands.empty()) return LIBRETT_INTERNAL_ERROR;
  bool learned = false;
  int pick = candidate < 0 ? lt::choosePlan(cands, sms, devName, &learned) : candidate;
  if (pick >= (int)cands.size()) return LIBRETT_INVALID_PARAMETER;
  if (!lt::refineCandidate(cands[pick], sms)) return LIBRETT_INTERNAL_ERROR;
  const int selectedBy = candidate >= 0 ? 3 : (learned ? 1 : 0);
  if (cached) {
    std::lock_guard<std::mutex> lk(gCacheMu);
    const int cap = cacheCapacityLocked();
    if (cap > 0 && gCache.find(key) == gCache.end()) {
      gCacheLru.emplace_front(key, CachedPlan{cands[pick], selectedBy});
      gCache[key] = gCacheLru.begin();
      while ((int)gCacheLru.size() > cap) {
        gCache.erase(gCacheLru.back().first);
        gCacheLru.pop_back();
      }
    }
  }
  return activate(handle, cands[pick], stream, dev, sms, selectedBy);
}

}  // namespace

// ---------------------------------------------------------------------------
// librett.h
// ---------------------------------------------------------------------------

void librettInitialize() {}

void librettFinalize() {}

librettResult librettPlan(librettHandle* handle, int rank, int* dim, int* permutation,
                          size_t sizeofType, librett_gpuStream_t& stream) {
  return planImpl(handle, rank, dim, permutation, sizeofType, stream, -1);
}

librettResult librettPlanMeasure(librettHandle* handle, int rank, int* dim, int* permutation,
                                 size_t sizeofType, librett_gpuStream_t& stream, void* idata,
                                 void* odata) {
  if (handle == nullptr) return LIBRETT_INVALID_PARAMETER;
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  if (idata == odata || idata == nullptr || odata == nullptr) return LIBRETT_INVALID_PARAMETER;
  if (!aligned(idata, sizeofType) || !aligned(odata, sizeofType)) return LIBRETT_INVALID_PARAMETER;
  int dev = 0, sms = 0;
  if (!currentDevice(dev, sms)) return LIBRETT_INTERNAL_ERROR;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  std::vector<lt::PlanDesc> cands = lt::enumerateCandidates(f, sms);
  if (cands.empty()) return LIBRETT_INTERNAL_ERROR;
  const size_t bytes = (size_t)f.vol * sizeofType;
  cudaEvent_t ev[2];
  if (cudaEventCreate(&ev[0]) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return LIBRETT_INTERNAL_ERROR;
  }
  // Each candidate: clear the output (as LibreTT does, src/librett.cpp:292),
  // one untimed warm-up launch, then the best of three timed launches.
  // LibreTT times a single cold launch per candidate.
  int best = -1;
  float bestMs = 0.f;
  librettResult res = LIBRETT_SUCCESS;
  for (size_t c = 0; c < cands.size() && res == LIBRETT_SUCCESS; ++c) {
    int grid = 0;
    void* alloc = nullptr;
    lt::DeviceTables dt;
    if (cands[c].pipe == lt::PIPE_BULK) cands[c].tile.statusTag = lt::nextStatusTag();
    if (!lt::finalizePlan(cands[c]) ||
        lt::createDeviceTables(cands[c], stream, &alloc, &dt) != cudaSuccess) {
      res = LIBRETT_INTERNAL_ERROR;
      break;
    }
    if (cudaMemsetAsync(odata, 0xff, bytes, stream) != cudaSuccess ||
        lt::launchPlan(cands[c], &dt, idata, odata, stream, sms, &grid) != cudaSuccess) {
      lt::destroyDeviceTables(alloc, stream);
      res = LIBRETT_INTERNAL_ERROR;
      break;
    }
    float candMs = -1.f;
    for (int rep = 0; rep < 3; ++rep) {
      if (cudaEventRecord(ev[0], stream) != cudaSuccess ||
          lt::launchPlan(cands[c], &dt, idata, odata, stream, sms, &grid) != cudaSuccess ||
          cudaEventRecord(ev[1], stream) != cudaSuccess || cudaEventSynchronize(ev[1]) != cudaSuccess) {
        res = LIBRETT_INTERNAL_ERROR;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[0], ev[1]);
      if (candMs < 0.f || ms < candMs) candMs = ms;
    }
    lt::destroyDeviceTables(alloc, stream);
    if (res == LIBRETT_SUCCESS && (best < 0 || candMs < bestMs)) {
      best = (int)c;
      bestMs = candMs;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (res != LIBRETT_SUCCESS) return res;
  return activate(handle, cands[best], stream, dev, sms, 2);
}

librettResult librettDestroy(librettHandle handle) {
  std::unique_lock<std::shared_mutex> lk(gPlanMu);
  auto it = gPlans.find(handle);
  if (it == gPlans.end()) return LIBRETT_INVALID_PLAN;
  gPlans.erase(it);
  return LIBRETT_SUCCESS;
}

librettResult librettExecute(librettHandle handle, void* idata, void* odata) {
  std::shared_ptr<PlanObj> obj = findPlan(handle);
  if (!obj) return LIBRETT_INVALID_PLAN;
  if (idata == odata || idata == nullptr || odata == nullptr) return LIBRETT_INVALID_PARAMETER;
  if (!aligned(idata, obj->pd.f.esize) || !aligned(odata, obj->pd.f.esize))
    return LIBRETT_INVALID_PARAMETER;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  if (dev != obj->device) return LIBRETT_INVALID_DEVICE;
  if (obj->needsScalar(idata, odata) && !obj->ensureScalar()) return LIBRETT_INTERNAL_ERROR;
  int grid = 0;
  if (lt::launchPlan(obj->pd, &obj->tables, idata, odata, obj->stream, obj->numSMs, &grid) !=
      cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  obj->lastGrid = grid;
  return LIBRETT_SUCCESS;
}

// ---------------------------------------------------------------------------
// librett_c.h
// ---------------------------------------------------------------------------

extern "C" {

void librett_c_initialize(void) { librettInitialize(); }

void librett_c_finalize(void) { librettFinalize(); }

int librett_c_plan(librettHandle* handle, int rank, const int* dim, const int* permutation,
                   size_t sizeofType, void* stream) {
  return planImpl(handle, rank, dim, permutation, sizeofType, (cudaStream_t)stream, -1);
}

int librett_c_plan_candidate(librettHandle* handle, int rank, const int* dim,
                             const int* permutation, size_t sizeofType, void* stream,
                             int candidate) {
  if (candidate < 0) return LIBRETT_INVALID_PARAMETER;
  return planImpl(handle, rank, dim, permutation, sizeofType, (cudaStream_t)stream, candidate);
}

int librett_c_plan_measure(librettHandle* handle, int rank, const int* dim,
                           const int* permutation, size_t sizeofType, void* stream,
                           const void* idata, void* odata) {
  if (dim == nullptr || permutation == nullptr) return LIBRETT_INVALID_PARAMETER;
  cudaStream_t s = (cudaStream_t)stream;
  return librettPlanMeasure(handle, rank, const_cast<int*>(dim), const_cast<int*>(permutation),
                            sizeofType, s, const_cast<void*>(idata), odata);
}

int librett_c_execute(librettHandle handle, const void* idata, void* odata) {
  return librettExecute(handle, const_cast<void*>(idata), odata);
}

int librett_c_destroy(librettHandle handle) { return librettDestroy(handle); }

int librett_c_plan_batch(int count, const int* ranks, const int* dims, const int* perms,
                         const size_t* sizes, void* stream, int synchronize,
                         librettHandle* handles, double* call_us) {
  if (count < 0 || (count > 0 && (ranks == nullptr || dims == nullptr || perms == nullptr ||
                                  sizes == nullptr || handles == nullptr)))
    return LIBRETT_INVALID_PARAMETER;
  cudaStream_t s = (cudaStream_t)stream;
  size_t off = 0;
  for (int k = 0; k < count; ++k) {
    const auto t0 = std::chrono::steady_clock::now();
    int rc = librett_c_plan(&handles[k], ranks[k], dims + off, perms + off, sizes[k], stream);
    const bool planned = rc == LIBRETT_SUCCESS;
    if (planned && synchronize && cudaStreamSynchronize(s) != cudaSuccess)
      rc = LIBRETT_INTERNAL_ERROR;
    const auto t1 = std::chrono::steady_clock::now();
    if (rc != LIBRETT_SUCCESS) {
      for (int j = 0; j < k + (planned ? 1 : 0); ++j) librettDestroy(handles[j]);
      return rc;
    }
    if (call_us != nullptr) call_us[k] = std::chrono::duration<double, std::micro>(t1 - t0).count();
    off += (size_t)(ranks[k] > 0 ? ranks[k] : 0);
  }
  return LIBRETT_SUCCESS;
}

int librett_c_plan_info(librettHandle handle, librett_plan_info* info) {
  if (info == nullptr) return LIBRETT_INVALID_PARAMETER;
  std::shared_ptr<PlanObj> obj = findPlan(handle);
  if (!obj) return LIBRETT_INVALID_PLAN;
  fillInfo(*obj, info);
  return LIBRETT_SUCCESS;
}

int librett_c_describe(int rank, const int* dim, const int* permutation, size_t sizeofType,
                       int num_sms, int candidate, librett_plan_info* info) {
  if (info == nullptr) return LIBRETT_INVALID_PARAMETER;
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  const int sms = num_sms > 0 ? num_sms : 152;
  std::vector<lt::PlanDesc> cands = lt::enumerateCandidates(f, sms, true);
  if (cands.empty()) return LIBRETT_INTERNAL_ERROR;
  bool learned = false;
  int pick = candidate < 0 ? lt::choosePlan(cands, sms, nullptr, &learned) : candidate;
  if (pick >= (int)cands.size()) return LIBRETT_INVALID_PARAMETER;
  if (!lt::refineCandidate(cands[pick], sms)) return LIBRETT_INTERNAL_ERROR;
  fillInfo(cands[pick], 0, info);
  info->selected_by = candidate >= 0 ? 3 : (learned ? 1 : 0);
  return LIBRETT_SUCCESS;
}

int librett_c_bulk_check(int rank, const int* dim, const int* permutation, size_t sizeofType,
                         int num_sms, int candidate) {
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  const int sms = num_sms > 0 ? num_sms : 152;
  std::vector<lt::PlanDesc> cands = lt::enumerateCandidates(f, sms, true);
  if (candidate < 0 || candidate >= (int)cands.size()) return LIBRETT_INVALID_PARAMETER;
  lt::PlanDesc pd = cands[candidate];
  if (!lt::refineCandidate(pd, sms)) return LIBRETT_INTERNAL_ERROR;
  if (pd.kernel != lt::K_TILE || pd.pipe != lt::PIPE_BULK) return LIBRETT_INVALID_DEVICE;
  const lt::TileParams& tp = pd.tile;
  const int L = tp.segLen, es = (int)sizeofType;
  if (L <= 0 || L % tp.lv || tp.tileVol % L || tp.lv * es != 16 || (L * es) % 16)
    return LIBRETT_INTERNAL_ERROR;
  std::vector<int> ldOff(tp.nIn), stOff(tp.nOut);
  std::vector<unsigned short> stSm(tp.tileVol);
  lt::tileTablesHost(tp, ldOff.data(), stOff.data(), stSm.data());
  auto pad = [&](int j) { return j + ((j >> tp.padShift) << tp.padLog); };
  // every segment is one contiguous piece of global memory and of shared
  // memory, starts 16-byte aligned in both, and the segments tile the tile
  for (int j0 = 0; j0 < tp.tileVol; j0 += L) {
    const int u0 = j0 / tp.lv;
    if (((long long)ldOff[u0] * es) % 16 || ((long long)pad(j0) * es) % 16)
      return LIBRETT_INTERNAL_ERROR;
    for (int j = j0; j < j0 + L; j += tp.lv) {
      if (ldOff[j / tp.lv] != ldOff[u0] + (j - j0)) return LIBRETT_INTERNAL_ERROR;
      if (pad(j) != pad(j0) + (j - j0)) return LIBRETT_INTERNAL_ERROR;
    }
  }
  if (pad(tp.tileVol - 1) >= tp.smStride) return LIBRETT_INTERNAL_ERROR;
  return LIBRETT_SUCCESS;
}

int librett_c_group_run_check(int rank, const int* dim, const int* permutation, size_t sizeofType,
                              int num_sms, int candidate, int element_units) {
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  std::vector<lt::PlanDesc> cands = lt::flatTileCandidates(f, num_sms > 0 ? num_sms : 152);
  if (candidate < 0 || candidate >= (int)cands.size()) return LIBRETT_INVALID_PARAMETER;
  lt::PlanDesc pd = cands[candidate];
  if (element_units) {
    if (!lt::finalizePlan(pd)) return LIBRETT_INTERNAL_ERROR;
    pd.tile = pd.tileScalar;
  }
  const lt::TileParams& tp = pd.tile;
  const lt::GroupRunSplit rs = lt::groupRunSplit(tp);
  if (rs.inRun < 1 || rs.outRun < 1 || tp.tileVol % rs.inRun || tp.tileVol % rs.outRun)
    return LIBRETT_UNDEFINED_ERROR;
  if (rs.inRun % tp.lv || rs.outRun % tp.sv) return LIBRETT_INVALID_DEVICE;  // not applicable
  std::vector<int> ldOff(tp.nIn), stOff(tp.nOut);
  std::vector<unsigned short> stSm(tp.tileVol);
  lt::tileTablesHost(tp, ldOff.data(), stOff.data(), stSm.data());
  std::vector<int> ldRow(tp.tileVol / rs.inRun), stRow(tp.tileVol / rs.outRun),
      smRow(tp.tileVol / rs.outRun), smRun(rs.outRun);
  lt::groupRunTablesHost(tp, rs, ldRow.data(), stRow.data(), smRow.data(), smRun.data());
  const lt::RunDiv inRun = lt::makeRunDiv((uint32_t)rs.inRun);
  const lt::RunDiv outRun = lt::makeRunDiv((uint32_t)rs.outRun);
  auto pad = [&](int j) { return j + ((j >> tp.padShift) << tp.padLog); };
  // evenly spaced input runs must match the table they replace
  const int ldStep = lt::groupLoadStep(tp, rs, (int)sizeofType);
  if (ldStep >= 0)
    for (size_t r = 0; r < ldRow.size(); ++r)
      if (ldRow[r] != (long long)r * ldStep) return LIBRETT_INTERNAL_ERROR;
  const lt::GroupStoreSteps st = lt::groupStoreSteps(tp, rs, (int)sizeofType);
  if (st.outStep >= 0)
    for (size_t r = 0; r < stRow.size(); ++r)
      if (stRow[r] != (long long)r * st.outStep || smRow[r] != (long long)r * st.rowSmStep)
        return LIBRETT_INTERNAL_ERROR;
  if (st.smStep >= 0)
    for (size_t a = 0; a < smRun.size(); ++a)
      if (smRun[a] != (long long)a * st.smStep) return LIBRETT_INTERNAL_ERROR;
  if (tp.tileVol >= 65536) return LIBRETT_INTERNAL_ERROR;  // run division needs indices < 2^16
  // the kernel's index arithmetic, unit by unit
  for (int u = 0; u < tp.nIn; ++u) {
    const int j = u * tp.lv;
    const uint32_t r = lt::runDivHost((uint32_t)j + 1, inRun);
    const int a = j - (int)(r * inRun.d);
    if (r >= ldRow.size() || a + ldRow[r] != ldOff[u]) return LIBRETT_INTERNAL_ERROR;
  }
  for (int w = 0; w < tp.nOut; ++w) {
    const int q = w * tp.sv;
    const uint32_t r = lt::runDivHost((uint32_t)q + 1, outRun);
    const int a = q - (int)(r * outRun.d);
    if (r >= stRow.size() || a + tp.sv > rs.outRun || a + stRow[r] != stOff[w])
      return LIBRETT_INTERNAL_ERROR;
    for (int i = 0; i < tp.sv; ++i)
      if (pad(smRow[r] + smRun[a + i]) != stSm[q + i]) return LIBRETT_INTERNAL_ERROR;
  }
  return LIBRETT_SUCCESS;
}

int librett_c_candidate_features(int rank, const int* dim, const int* permutation,
                                 size_t sizeofType, int num_sms, int candidate, float* features,
                                 int nfeatures) {
  if (features == nullptr || nfeatures < lt::NFEAT) return LIBRETT_INVALID_PARAMETER;
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0) return LIBRETT_INVALID_PARAMETER;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  const int sms = num_sms > 0 ? num_sms : 152;
  // the features the selectors see: of the screened candidate
  std::vector<lt::PlanDesc> cands = lt::enumerateCandidates(f, sms, true);
  if (candidate < 0 || candidate >= (int)cands.size()) return LIBRETT_INVALID_PARAMETER;
  lt::planFeatures(cands[candidate], sms, features);
  return LIBRETT_SUCCESS;
}

int librett_c_set_candidate_set(int all) {
  const int prev = lt::allPipelines() ? 1 : 0;
  lt::setAllPipelines(all != 0);
  cacheClear();
  return prev;
}

int librett_c_set_plan_selector(int mode) {
  if (mode < 0 || mode > 2) return -1;
  const int prev = lt::selectorMode();
  lt::setSelectorMode(mode);
  cacheClear();
  return prev;
}

int librett_c_load_plan_model(const char* path) {
  std::string why;
  const bool ok = lt::loadSelectorModel(path, &why);
  cacheClear();
  return ok ? LIBRETT_SUCCESS : LIBRETT_INVALID_PARAMETER;
}

int librett_c_set_plan_cache(int capacity) {
  std::lock_guard<std::mutex> lk(gCacheMu);
  const int prev = cacheCapacityLocked();
  gCacheCap = std::max(0, capacity);
  while ((int)gCacheLru.size() > gCacheCap) {
    gCache.erase(gCacheLru.back().first);
    gCacheLru.pop_back();
  }
  return prev;
}

int librett_c_plan_cache_stats(long long* hits, long long* misses, int* entries) {
  std::lock_guard<std::mutex> lk(gCacheMu);
  if (hits) *hits = gCacheHits;
  if (misses) *misses = gCacheMisses;
  if (entries) *entries = (int)gCacheLru.size();
  return LIBRETT_SUCCESS;
}

int librett_c_mlp_predict_host(const float* params, const float* x, int n, float* out) {
  if (params == nullptr || x == nullptr || out == nullptr || n < 0) return LIBRETT_INVALID_PARAMETER;
  // the planner's batched path, with an identity standardisation
  lt::MlpModel m;
  m.params.assign(params, params + lt::mlpParamCount());
  m.prepare();
  if (n > 0) lt::mlpForwardBatch(m, x, n, out);
  return LIBRETT_SUCCESS;
}

unsigned long long librett_c_launch_count(void) {
  return lt::gLaunchCount.load(std::memory_order_relaxed);
}

const char* librett_c_result_string(int result) {
  switch (result) {
    case LIBRETT_SUCCESS: return "LIBRETT_SUCCESS";
    case LIBRETT_INVALID_PLAN: return "LIBRETT_INVALID_PLAN";
    case LIBRETT_INVALID_PARAMETER: return "LIBRETT_INVALID_PARAMETER";
    case LIBRETT_INVALID_DEVICE: return "LIBRETT_INVALID_DEVICE";
    case LIBRETT_INTERNAL_ERROR: return "LIBRETT_INTERNAL_ERROR";
    case LIBRETT_UNDEFINED_ERROR: return "LIBRETT_UNDEFINED_ERROR";
    default: return "unknown";
  }
}

}  // extern "C"

int librett_c_inject_fault(int site, long long after) {
  return lt::armFault(site, after) ? LIBRETT_SUCCESS : LIBRETT_INVALID_PARAMETER;
}

int librett_c_table_arena_stats(long long* slab_bytes, long long* blocks, long long* pool_bytes) {
  lt::tableArenaStats(slab_bytes, blocks, pool_bytes);
  return LIBRETT_SUCCESS;
}

int librett_c_plan_status(librettHandle handle, unsigned* status) {
  if (status == nullptr) return LIBRETT_INVALID_PARAMETER;
  std::shared_ptr<PlanObj> obj = lt::findPlan(handle);
  if (!obj) return LIBRETT_INVALID_PLAN;
  *status = 0;
  if (obj->tables.status == nullptr) return LIBRETT_SUCCESS;
  unsigned word = 0;
  if (cudaMemcpyAsync(&word, obj->tables.status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                      obj->stream) != cudaSuccess ||
      cudaStreamSynchronize(obj->stream) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  *status = word == obj->pd.tile.statusTag ? 1u : 0u;
  return LIBRETT_SUCCESS;
}

int librett_c_bulk_wait_test(librettHandle handle, const void* idata, void* odata,
                             unsigned extra_bytes, unsigned* status) {
  if (status == nullptr || extra_bytes == 0 || extra_bytes > 4096) return LIBRETT_INVALID_PARAMETER;
  std::shared_ptr<PlanObj> obj = lt::findPlan(handle);
  if (!obj) return LIBRETT_INVALID_PLAN;
  if (obj->pd.kernel != lt::K_TILE || obj->pd.pipe != lt::PIPE_BULK ||
      obj->tables.status == nullptr || obj->needsScalar(idata, odata))
    return LIBRETT_INVALID_PARAMETER;
  lt::PlanDesc pd = obj->pd;
  pd.tile.testExtraTx = (int)extra_bytes;
  int grid = 0;
  *status = 0;
  unsigned word = 0;
  if (lt::launchPlan(pd, &obj->tables, idata, odata, obj->stream, obj->numSMs, &grid) !=
          cudaSuccess ||
      cudaMemcpyAsync(&word, obj->tables.status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                      obj->stream) != cudaSuccess ||
      cudaStreamSynchronize(obj->stream) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  *status = word == pd.tile.statusTag ? 1u : 0u;
  // clear the plan's word again (stream-ordered after the launch)
  if (*status != 0 &&
      (cudaMemsetAsync(obj->tables.status, 0, sizeof(unsigned), obj->stream) != cudaSuccess ||
       cudaStreamSynchronize(obj->stream) != cudaSuccess))
    return LIBRETT_INTERNAL_ERROR;
  return LIBRETT_SUCCESS;
}
