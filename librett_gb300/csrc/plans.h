// Registry of live plans, shared by the API layer (api.cpp) and grouped
// execution (group.cu).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>

#include "launch.h"
#include "librett.h"
#include "plan.h"

namespace lt {

struct PlanObj {
  PlanDesc pd;
  int selectedBy = 0;  // librett_plan_info.selected_by
  cudaStream_t stream = nullptr;
  int device = 0;
  int numSMs = 0;
  int lastGrid = 0;
  void* tablesAlloc = nullptr;  // device tables of flat-pipeline plans
  DeviceTables tables;
  // The element-unit geometry (pd.tileScalar), built on the first launch
  // with pointers that are not 16-byte aligned.
  std::once_flag scalarOnce;
  bool scalarOk = false;
  bool ensureScalar() {
    std::call_once(scalarOnce, [this] { scalarOk = finalizePlan(pd); });
    return scalarOk;
  }
  // Whether a launch with these pointers uses the element-unit geometry.
  bool needsScalar(const void* in, const void* out) const {
    return pd.kernel == K_TILE && (pd.tile.lv > 1 || pd.tile.sv > 1) &&
           (((uintptr_t)in | (uintptr_t)out) % 16) != 0;
  }
  PlanObj() = default;
  PlanObj(const PlanObj&) = delete;
  PlanObj& operator=(const PlanObj&) = delete;
  // Stream-ordered release: launches already enqueued on the plan's stream
  // finish before the tables are freed (LibreTT's plan destructor calls
  // cudaFree, which synchronises the device, src/plan.cpp:1696-1703).
  ~PlanObj() { destroyDeviceTables(tablesAlloc, stream); }
};


// The live plan behind a handle (kept alive by the returned pointer), or
// nullptr.
std::shared_ptr<PlanObj> findPlan(librettHandle h);

// Current device, its SM count and (optionally) name, cached per device.
bool currentDevice(int& dev, int& sms, std::string* name = nullptr);
bool currentDevice(int& dev, int& sms, const char** name);

}  // namespace lt
