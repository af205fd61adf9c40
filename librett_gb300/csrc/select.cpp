// Learned plan selection (see select.h).
#include "select.h"

#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>

namespace lt {

namespace {

float lg2(double x) { return (float)std::log2(std::max(x, 1.0)); }

}  // namespace

namespace {

// The features that depend only on the fused problem (the same for all its
// candidates).
void problemFeatures(const Fused& f, float* out) {
  const double vol = (double)f.vol;
  out[0] = lg2(vol) / 32.f;
  out[1] = f.esize / 16.f;
  out[2] = f.rank / 8.f;
  out[3] = lg2((double)f.dim[0]) / 24.f;
  out[4] = lg2((double)f.dim[f.perm[0]]) / 24.f;
  out[5] = f.perm[0] == 0 ? 1.f : 0.f;
  out[31] = lg2(vol * f.esize) / 36.f;
}

// The rest; `out` holds the problem features already, `bank` is the
// candidate's bankPerUnitOf.
void candidateFeatures(const PlanDesc& pd, int numSMs, double bank, float* out) {
  const Fused& f = pd.f;
  out[6] = pd.kernel == K_COPY;
  out[7] = pd.kernel == K_ROW;
  out[8] = pd.kernel == K_TILE;
  out[14] = lg2((double)pd.runInBytes) / 20.f;
  out[15] = lg2((double)pd.runOutBytes) / 20.f;
  out[16] = pd.unitBytes / 16.f;
  out[17] = (pd.kernel == K_TILE ? pd.unitOutBytes : pd.unitBytes) / 16.f;
  out[18] = lg2((double)pd.numWork) / 24.f;
  out[30] = (float)std::log2(std::max(pd.cost, 1e-7) * 1e6) / 16.f;
  if (pd.kernel != K_TILE) return;
  const TileParams& tp = pd.tile;
  out[9] = pd.pipe == PIPE_REG;
  out[10] = pd.pipe == PIPE_ASYNC;
  out[11] = flatTables(pd.pipe);
  out[32] = pd.pipe == PIPE_BULK;
  out[12] = lg2((double)tp.tileVol) / 12.f;
  out[13] = lg2((double)tp.tileVol * f.esize) / 16.f;
  out[19] = pd.slots / 16.f;
  out[20] = pd.smemBytes / (228.f * 1024.f);
  out[21] = pd.ctasPerSM / 8.f;
  const double conc = (double)std::max(1, numSMs) * std::max(1, pd.ctasPerSM);
  out[22] = (float)std::log2(std::max(tp.numTiles / conc, 1e-3) * 8.0) / 16.f;
  out[23] = tp.nTR / 8.f;
  out[24] = tp.nGR / 8.f;
  out[25] = tp.nRagged / 4.f;
  out[26] = (float)(pd.overlap - 1.0);
  out[27] = (float)pd.effIn;
  out[28] = (float)pd.effOut;
  out[29] = (float)(bank / 8.0);
}

}  // namespace

void planFeatures(const PlanDesc& pd, int numSMs, float* out) {
  for (int i = 0; i < NFEAT; ++i) out[i] = 0.f;
  problemFeatures(pd.f, out);
  candidateFeatures(pd, numSMs, bankPerUnitOf(pd), out);
}

// ---------------------------------------------------------------------------
// Weight file
//
//   char     magic[8]      "LTMLPv01"
//   uint32   nfeat, hidden, layers, paramCount
//   int32    sms
//   char     device[64]    NUL-padded device name
//   float    mean[nfeat], std[nfeat], ymean, ystd
//   float    params[paramCount]
//   uint32   FNV-1a of all preceding bytes
// ---------------------------------------------------------------------------
namespace {

constexpr char kMagic[8] = {'L', 'T', 'M', 'L', 'P', 'v', '0', '1'};

uint32_t fnv1a(const unsigned char* p, size_t n) {
  uint32_t h = 2166136261u;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 16777619u;
  }
  return h;
}

}  // namespace

bool loadMlpModel(const std::string& path, MlpModel& m, std::string* why) {
  auto fail = [&](const char* w) {
    if (why) *why = w;
    return false;
  };
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail("cannot open the model file");
  std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)),
                                 std::istreambuf_iterator<char>());
  const size_t head = 8 + 4 * 4 + 4 + 64;
  if (buf.size() < head + 4) return fail("model file too short");
  if (std::memcmp(buf.data(), kMagic, 8) != 0) return fail("bad magic");
  uint32_t u[4];
  std::memcpy(u, buf.data() + 8, 16);
  if (u[0] != (uint32_t)NFEAT || u[1] != (uint32_t)MLP_HIDDEN || u[2] != (uint32_t)MLP_LAYERS ||
      u[3] != (uint32_t)mlpParamCount())
    return fail("architecture mismatch");
  const size_t nfloat = 2 * NFEAT + 2 + mlpParamCount();
  if (buf.size() != head + 4 * nfloat + 4) return fail("size mismatch");
  uint32_t sum;
  std::memcpy(&sum, buf.data() + buf.size() - 4, 4);
  if (sum != fnv1a(buf.data(), buf.size() - 4)) return fail("checksum mismatch");
  int32_t sms;
  std::memcpy(&sms, buf.data() + 24, 4);
  char dev[65] = {};
  std::memcpy(dev, buf.data() + 28, 64);
  std::vector<float> vals(nfloat);
  std::memcpy(vals.data(), buf.data() + head, 4 * nfloat);
  for (float v : vals)
    if (!std::isfinite(v)) return fail("non-finite value");
  m.sms = sms;
  m.device = dev;
  m.mean.assign(vals.begin(), vals.begin() + NFEAT);
  m.stdv.assign(vals.begin() + NFEAT, vals.begin() + 2 * NFEAT);
  for (float s : m.stdv)
    if (!(s > 0.f)) return fail("non-positive feature scale");
  m.ymean = vals[2 * NFEAT];
  m.ystd = vals[2 * NFEAT + 1];
  if (!(m.ystd > 0.f)) return fail("non-positive target scale");
  m.params.assign(vals.begin() + 2 * NFEAT + 2, vals.end());
  m.prepare();
  return true;
}

float mlpForward(const float* params, const float* x) {
  float a[MLP_HIDDEN], b[MLP_HIDDEN];
  const float* w = params;
  // layer 1: NFEAT -> HIDDEN
  for (int o = 0; o < MLP_HIDDEN; ++o) {
    float s = w[MLP_HIDDEN * NFEAT + o];
    const float* row = w + o * NFEAT;
    for (int i = 0; i < NFEAT; ++i) s += row[i] * x[i];
    a[o] = s > 0.f ? s : 0.f;
  }
  w += MLP_HIDDEN * NFEAT + MLP_HIDDEN;
  // layers 2, 3: HIDDEN -> HIDDEN
  for (int l = 0; l < 2; ++l) {
    float* src = l == 0 ? a : b;
    float* dst = l == 0 ? b : a;
    for (int o = 0; o < MLP_HIDDEN; ++o) {
      float s = w[MLP_HIDDEN * MLP_HIDDEN + o];
      const float* row = w + o * MLP_HIDDEN;
      for (int i = 0; i < MLP_HIDDEN; ++i) s += row[i] * src[i];
      dst[o] = s > 0.f ? s : 0.f;
    }
    w += MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN;
  }
  // output: HIDDEN -> 1 (input is `a` after two swaps)
  float s = w[MLP_HIDDEN];
  for (int i = 0; i < MLP_HIDDEN; ++i) s += w[i] * a[i];
  return s;
}

void MlpModel::prepare() {
  auto transpose = [](const float* w, int out, int in, std::vector<float>& t) {
    t.resize((size_t)out * in);
    for (int o = 0; o < out; ++o)
      for (int i = 0; i < in; ++i) t[(size_t)i * out + o] = w[(size_t)o * in + i];
  };
  const float* w = params.data();
  transpose(w, MLP_HIDDEN, NFEAT, wt1);
  w += MLP_HIDDEN * NFEAT + MLP_HIDDEN;
  transpose(w, MLP_HIDDEN, MLP_HIDDEN, wt2);
  w += MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN;
  transpose(w, MLP_HIDDEN, MLP_HIDDEN, wt3);
}

namespace {

// y[r][o] = relu(b[o] + sum_i x[r][i] * wt[i][o]) for r < n.  The input
// index is the outer loop so each weight row is read once for all rows
// (the weights do not fit in L1; the n output rows do).
// Four-lane float vector (GCC/Clang vector extension: SSE on x86-64, NEON on
// AArch64); element-wise arithmetic only, so results match scalar code.
typedef float F4 __attribute__((vector_size(16)));

inline F4 load4(const float* p) {
  F4 v;
  std::memcpy(&v, p, sizeof(v));
  return v;
}

// y[r] = relu(b + x[r] . wt) for n rows, wt stored input-major (wt[i][o]).
// Register-blocked: RB rows by OB outputs accumulate in registers over the
// inputs (each weight vector loaded once per RB rows); each output's sum
// runs in input order starting from the bias.
// SKIP_ZERO (inputs that are ReLU outputs, in <= MLP_HIDDEN): an input that
// is zero in every row of the block is left out.  Its terms are products
// with zero, so leaving them out can change only the sign of an exactly zero
// sum, which the ReLU maps to +0 either way: the outputs are bit-identical.
// Candidates of one problem share most zero inputs (about 33 % of the second
// layer's inputs and 46 % of the third's are zero in a whole block).
template <int RB, int OB, bool SKIP_ZERO>
void denseReluBlocked(const float* x, int n, int in, const float* wt, const float* b, float* y) {
  constexpr int NV = OB / 4;
  const F4 zero = {0.f, 0.f, 0.f, 0.f};
  int active[MLP_HIDDEN];
  for (int r0 = 0; r0 < n; r0 += RB) {
    const float* xr[RB];
    for (int k = 0; k < RB; ++k) xr[k] = x + (size_t)std::min(r0 + k, n - 1) * in;
    int na = in;
    if (SKIP_ZERO) {
      na = 0;
      for (int i = 0; i < in; ++i) {
        bool any = false;
        for (int k = 0; k < RB; ++k) any |= xr[k][i] != 0.f;
        active[na] = i;
        na += any;
      }
    }
    for (int o0 = 0; o0 < MLP_HIDDEN; o0 += OB) {
      F4 acc[RB][NV];
      for (int k = 0; k < RB; ++k)
        for (int v = 0; v < NV; ++v) acc[k][v] = load4(b + o0 + 4 * v);
      for (int j = 0; j < na; ++j) {
        const int i = SKIP_ZERO ? active[j] : j;
        const float* w = wt + (size_t)i * MLP_HIDDEN + o0;
        F4 wv[NV];
        for (int v = 0; v < NV; ++v) wv[v] = load4(w + 4 * v);
        for (int k = 0; k < RB; ++k) {
          const F4 a = {xr[k][i], xr[k][i], xr[k][i], xr[k][i]};
          for (int v = 0; v < NV; ++v) acc[k][v] += a * wv[v];
        }
      }
      for (int k = 0; k < RB && r0 + k < n; ++k)
        for (int v = 0; v < NV; ++v) {
          const F4 t = acc[k][v] > zero ? acc[k][v] : zero;
          std::memcpy(y + (size_t)(r0 + k) * MLP_HIDDEN + o0 + 4 * v, &t, sizeof(t));
        }
    }
  }
}

// Row blocks sized for the host's vector registers.  AArch64 (32 vector
// registers): blocks of exactly the remaining rows up to 5 (1-2 rows by 32
// outputs, 3-5 rows by 16), 4-row blocks before a remainder of at most 5,
// so no row is computed twice; measured on Neoverse V2 against one block of
// 6-8 rows: n = 6: 7.3 vs 8.6 us, n = 7: 8.2 vs 8.8, n = 8: 9.1 vs 9.9.
// Elsewhere 4 rows by 16 outputs.  Every block sums each output in the
// same order, so the result does not depend on the split.
template <bool SKIP_ZERO>
void denseRelu(const float* x, int n, int in, const float* wt, const float* b, float* y) {
#if defined(__aarch64__)
  while (n > 5) {
    denseReluBlocked<4, 16, SKIP_ZERO>(x, 4, in, wt, b, y);
    x += (size_t)4 * in;
    y += (size_t)4 * MLP_HIDDEN;
    n -= 4;
  }
  switch (n) {
    case 1: denseReluBlocked<1, 32, SKIP_ZERO>(x, n, in, wt, b, y); return;
    case 2: denseReluBlocked<2, 32, SKIP_ZERO>(x, n, in, wt, b, y); return;
    case 3: denseReluBlocked<3, 16, SKIP_ZERO>(x, n, in, wt, b, y); return;
    case 4: denseReluBlocked<4, 16, SKIP_ZERO>(x, n, in, wt, b, y); return;
    default: denseReluBlocked<5, 16, SKIP_ZERO>(x, n, in, wt, b, y); return;
  }
#else
  denseReluBlocked<4, 16, SKIP_ZERO>(x, n, in, wt, b, y);
#endif
}

}  // namespace

void mlpForwardBatch(const MlpModel& m, const float* x, int n, float* out) {
  // activations of the layers, reused by the calling thread
  thread_local std::vector<float> a, b;
  if (a.size() < (size_t)n * MLP_HIDDEN) {
    a.resize((size_t)n * MLP_HIDDEN);
    b.resize((size_t)n * MLP_HIDDEN);
  }
  const float* p = m.params.data();
  const float* b1 = p + MLP_HIDDEN * NFEAT;
  const float* b2 = b1 + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN;
  const float* b3 = b2 + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN;
  const float* w4 = b3 + MLP_HIDDEN;
  const float b4 = w4[MLP_HIDDEN];
  denseRelu<false>(x, n, NFEAT, m.wt1.data(), b1, a.data());
  denseRelu<true>(a.data(), n, MLP_HIDDEN, m.wt2.data(), b2, b.data());
  denseRelu<true>(b.data(), n, MLP_HIDDEN, m.wt3.data(), b3, a.data());
  for (int r = 0; r < n; ++r) {
    const float* ar = a.data() + (size_t)r * MLP_HIDDEN;
    float s = 0.f;
    for (int i = 0; i < MLP_HIDDEN; ++i) s += w4[i] * ar[i];
    out[r] = s + b4;
  }
}

float mlpPredict(const MlpModel& m, const float* feat) {
  float x[NFEAT];
  for (int i = 0; i < NFEAT; ++i) x[i] = (feat[i] - m.mean[i]) / m.stdv[i];
  return mlpForward(m.params.data(), x) * m.ystd + m.ymean;
}

// ---------------------------------------------------------------------------
// Selector state
// ---------------------------------------------------------------------------
namespace {

std::mutex gSelMu;
bool gTried = false;
bool gLoaded = false;
MlpModel gModel;
std::atomic<int> gMode{-1};

int envMode() {
  const char* e = std::getenv("LIBRETT_PLAN_SELECTOR");
  if (e == nullptr) return 0;
  if (std::strcmp(e, "analytic") == 0) return 1;
  if (std::strcmp(e, "learned") == 0) return 2;
  return 0;
}

std::string defaultModelPath() {
  const char* e = std::getenv("LIBRETT_PLAN_MODEL");
  if (e != nullptr && *e) return e;
  Dl_info info;
  if (dladdr((void*)&defaultModelPath, &info) != 0 && info.dli_fname != nullptr) {
    std::string so = info.dli_fname;
    size_t slash = so.rfind('/');
    std::string dir = slash == std::string::npos ? "." : so.substr(0, slash);
    return dir + "/models/plan_mlp.bin";
  }
  return "models/plan_mlp.bin";
}

// Caller holds gSelMu.
void ensureLoaded() {
  if (gTried) return;
  gTried = true;
  MlpModel m;
  if (loadMlpModel(defaultModelPath(), m, nullptr)) {
    gModel = std::move(m);
    gLoaded = true;
  }
}

}  // namespace

void setSelectorMode(int mode) { gMode.store(mode); }

int selectorMode() {
  int m = gMode.load();
  if (m < 0) {
    m = envMode();
    gMode.store(m);
  }
  return m;
}

bool loadSelectorModel(const char* path, std::string* why) {
  std::lock_guard<std::mutex> lk(gSelMu);
  if (path == nullptr) {
    gTried = false;
    gLoaded = false;
    ensureLoaded();
    if (!gLoaded && why) *why = "no model at the default path";
    return gLoaded;
  }
  MlpModel m;
  if (!loadMlpModel(path, m, why)) return false;
  gModel = std::move(m);
  gLoaded = true;
  gTried = true;
  return true;
}

// Tiles whose candidates the learned model ranks: the analytic model's
// cheapest few.  A short list of 4 tiles cost no measurable throughput
// against ranking every candidate (random-shape suite geomean 6399.5 vs
// 6399.0 GB/s on one GB300, held-out regret 1.53% vs 1.43%), while the
// network runs on about half of them; 3 cost 0.5% on the suite.
int shortlistSize() {
  static const int k = [] {
    const char* e = std::getenv("LIBRETT_SELECTOR_SHORTLIST");
    const int v = e != nullptr && *e ? std::atoi(e) : 4;
    return v > 0 ? v : 1 << 30;  // 0: every candidate
  }();
  return k;
}

// Of the short-listed tiles, the cheapest SHORTLIST_TWINS also bring their
// bulk-copy twin.  Held out (1,000 problems): twins of all 4 tiles 2.02 %
// regret over 6.2 candidates, of the first 2 tiles 2.14 % over 5.0, of
// none 2.66 % over 3.7; on the random-shape suite (1 GiB problems) twins of
// only 2 tiles cost 0.4 % of throughput on one GB300, so all 4 keep them.
constexpr int SHORTLIST_TWINS = 4;
// A twin joins only when the tile's input runs hold at least this many bytes:
// in the timings, bulk copies of shorter runs rarely beat their per-unit
// twin (128-255 bytes: 18 of 3528 tiles, 16 % slower at the median; 256-511:
// 183 of 5613).  With the model trained on every candidate, the held-out
// regret is 2.16 % over 4.62 candidates against 2.09 % over 6.20 without
// the rule and 2.13 % over 4.99 with 1 KiB (1,800 problems of 2^28 bytes
// and more: 1.03 % against 0.99 %).  On one GB300 machine, 2 KiB against 1 KiB:
// librettPlan 16.2-16.3 against 16.6-16.7 us, the random-shape suite
// 0.02-0.03 % slower.
constexpr int SHORTLIST_TWIN_MIN_RUN = 2048;

int choosePlan(std::vector<PlanDesc>& cands, int numSMs, const char* deviceName,
               bool* usedLearned) {
  if (usedLearned) *usedLearned = false;
  const int mode = selectorMode();
  if (cands.size() <= 1 || mode == 1) return chooseHeuristic(cands);
  std::lock_guard<std::mutex> lk(gSelMu);
  ensureLoaded();
  if (!gLoaded || gModel.sms != numSMs ||
      (deviceName != nullptr && !gModel.device.empty() && gModel.device != deviceName))
    return chooseHeuristic(cands);
  // the short list: the candidates of the analytic model's cheapest few
  // tiles, in increasing analytic cost (ties by index); a tile's per-unit
  // and bulk-copy variants (same extents, same modelled cost) count once,
  // and only the cheapest SHORTLIST_TWINS tiles keep their bulk-copy twin,
  // when their input runs hold at least SHORTLIST_TWIN_MIN_RUN bytes
  std::vector<int> order(cands.size());
  for (size_t c = 0; c < order.size(); ++c) order[c] = (int)c;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cands[a].cost < cands[b].cost; });
  auto sameTile = [&](int a, int b) {
    const PlanDesc& x = cands[a];
    const PlanDesc& y = cands[b];
    if (x.kernel != K_TILE || y.kernel != K_TILE) return false;
    for (int r = 0; r < x.f.rank; ++r)
      if (x.extent[r] != y.extent[r]) return false;
    return true;
  };
  std::vector<int> tileFirst;  // first candidate of each short-listed tile
  int n = 0;                   // short list: order[0 .. n)
  for (size_t c = 0; c < order.size(); ++c) {
    int ti = 0;
    while (ti < (int)tileFirst.size() && !sameTile(tileFirst[ti], order[c])) ++ti;
    if (ti == (int)tileFirst.size()) {
      if (ti == shortlistSize()) break;
      tileFirst.push_back(order[c]);
    }
    const PlanDesc& pc = cands[order[c]];
    if (pc.pipe == PIPE_BULK && (ti >= SHORTLIST_TWINS || pc.runInBytes < SHORTLIST_TWIN_MIN_RUN))
      continue;
    order[n++] = order[c];
  }
  if (n == 1) return order[0];
  std::vector<float> x((size_t)n * NFEAT), y(n);
  float prob[NFEAT] = {};  // the problem's features, computed once
  problemFeatures(cands[order[0]].f, prob);
  for (int c = 0; c < n; ++c) {
    float* xc = x.data() + (size_t)c * NFEAT;
    std::memcpy(xc, prob, sizeof(prob));
    // screened variants of one tile share its unpadded geometry and so its
    // bank count: simulate it once per tile and keep it in the candidates
    PlanDesc& pc = cands[order[c]];
    if (pc.kernel == K_TILE && pc.bankPerUnit < 0.0) {
      for (int j = 0; j < c; ++j) {
        const PlanDesc& pj = cands[order[j]];
        if (pj.screened && pj.tile.bankWavefronts >= 0 && sameTile(order[j], order[c]) &&
            pj.tile.padShift == pc.tile.padShift) {
          pc.tile.bankWavefronts = pj.tile.bankWavefronts;
          pc.bankPerUnit = pj.bankPerUnit;
          break;
        }
      }
      simulateBanks(pc);
    }
    candidateFeatures(pc, numSMs, pc.bankPerUnit, xc);
    for (int i = 0; i < NFEAT; ++i) xc[i] = (xc[i] - gModel.mean[i]) / gModel.stdv[i];
  }
  mlpForwardBatch(gModel, x.data(), n, y.data());
  int best = 0;
  for (int c = 0; c < n; ++c) {
    if (!std::isfinite(y[c])) return chooseHeuristic(cands);
    if (y[c] < y[best]) best = c;
  }
  if (usedLearned) *usedLearned = true;
  return order[best];
}

}  // namespace lt
