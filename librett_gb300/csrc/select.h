// Learned plan selection: candidate features, the MLP weight file, host
// inference, and the choice between the learned and the analytic model.
//
// Role in LibreTT's terms: the MLP replaces the analytic GpuModel
// (countCycles / cyclesPacked / cyclesTiled, LibreTT src/plan.cpp:1073-1643,
// src/GpuModel.cpp:762-911) as the function that ranks candidate plans; the
// analytic model (modelTile) remains the fallback and one of the inputs.
#pragma once

#include <string>
#include <vector>

#include "plan.h"

namespace lt {

constexpr int NFEAT = 33;      // features per candidate
constexpr int MLP_HIDDEN = 128;
constexpr int MLP_LAYERS = 4;  // 3 hidden layers + output

// Parameter count of the NFEAT -> 128 -> 128 -> 128 -> 1 network
// (W1, b1, W2, b2, W3, b3, W4, b4, weights row-major [out][in]).
constexpr int mlpParamCount() {
  return MLP_HIDDEN * NFEAT + MLP_HIDDEN + 2 * (MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN) +
         MLP_HIDDEN + 1;
}

// Feature vector of one candidate (scaled to O(1); the model file carries
// the standardisation fitted at training time).
void planFeatures(const PlanDesc& pd, int numSMs, float* out);

struct MlpModel {
  int sms = 0;
  std::string device;
  std::vector<float> mean, stdv;  // feature standardisation
  float ymean = 0.f, ystd = 1.f;  // target de-standardisation
  std::vector<float> params;      // mlpParamCount() floats
  // hidden-layer weights transposed to [in][out] for the batched forward
  std::vector<float> wt1, wt2, wt3;
  void prepare();                 // fills wt1..wt3 from params
};

// Batched forward of n standardised feature rows (the planner's hot path):
// out[r] = network output.  Inner loops run over contiguous outputs, so the
// compiler vectorises them without reassociating sums.
void mlpForwardBatch(const MlpModel& m, const float* x, int n, float* out);

// Reads a weight file; false (with a reason) if the magic, version, sizes,
// checksum or any value (NaN / Inf) is wrong.
bool loadMlpModel(const std::string& path, MlpModel& m, std::string* why);

// Network output for one standardised feature vector.
float mlpForward(const float* params, const float* x);

// Predicted log-time of a candidate (feature standardisation applied).
float mlpPredict(const MlpModel& m, const float* feat);

// Which model ranks candidates: 0 = learned when a model for this device
// is loaded, else analytic; 1 = analytic; 2 = learned (falls back to the
// analytic model when none is loaded).
void setSelectorMode(int mode);
int selectorMode();

// Explicit model path (nullptr: reset to the default search).  Returns
// false if the file does not load.
bool loadSelectorModel(const char* path, std::string* why);

// The candidate to use: the learned model's argmin of predicted time when
// it applies to a device with numSMs SMs (and, when known, this device
// name), else chooseHeuristic.  *usedLearned tells which one decided.  The
// bank counts it simulates for screened short-listed candidates are kept in
// them (simulateBanks), so refining the pick does not repeat its count.
int choosePlan(std::vector<PlanDesc>& cands, int numSMs, const char* deviceName,
               bool* usedLearned);

}  // namespace lt
