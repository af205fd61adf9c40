// Host planner: input check, rank fusion, candidate enumeration, analytic
// cost model.  Pure host code (no CUDA runtime calls), so it also runs on
// machines without a GPU through librett_c_describe.
//
// LibreTT counterparts: librettPlanCheckInput (src/librett.cpp:85-108),
// reduceRanks (src/plan.cpp:64-127), createPlans and the create*Plans family
// (src/plan.cpp:493-719), countCycles + GpuModel (src/plan.cpp:1073-1643,
// src/GpuModel.cpp:39-911) and choosePlanHeuristic (src/plan.cpp:778-789).
// The candidate set and the model are this engine's own: the kernels differ,
// so the model counts the DRAM sectors and shared-memory wavefronts of this
// engine's kernels rather than LibreTT's transaction counts.
#include "plan.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <unordered_set>

namespace lt {

int checkInput(int rank, const int* dim, const int* perm, size_t sizeofType) {
  const int INVALID = 2;  // LIBRETT_INVALID_PARAMETER
  if (sizeofType != 4 && sizeofType != 8 && sizeofType != 16) return INVALID;
  if (rank < 1 || rank > MAXR) return INVALID;
  if (dim == nullptr || perm == nullptr) return INVALID;
  const int64_t volLimit = int64_t(1) << 40;
  int64_t vol = 1;
  for (int i = 0; i < rank; ++i) {
    if (dim[i] < 1) return INVALID;
    if (vol > volLimit / dim[i]) return INVALID;
    vol *= dim[i];
  }
  bool seen[MAXR] = {};
  for (int i = 0; i < rank; ++i) {
    int p = perm[i];
    if (p < 0 || p >= rank || seen[p]) return INVALID;
    seen[p] = true;
  }
  return 0;
}

static void computeStrides(Fused& f) {
  int64_t s = 1;
  for (int r = 0; r < f.rank; ++r) {
    f.sin[r] = s;
    s *= f.dim[r];
  }
  f.vol = s;
  s = 1;
  for (int i = 0; i < f.rank; ++i) {
    f.sout[f.perm[i]] = s;
    s *= f.dim[f.perm[i]];
  }
}

void fuseRanks(int rank, const int* dim, const int* perm, int esize, Fused& f) {
  std::memset(&f, 0, sizeof(f));
  f.esize = esize;
  // 1. Unit dims do not change the layout: drop them.
  int newIdx[MAXR];
  int64_t d1[MAXR];
  int r1 = 0;
  for (int r = 0; r < rank; ++r) {
    if (dim[r] > 1) {
      newIdx[r] = r1;
      d1[r1++] = dim[r];
    } else {
      newIdx[r] = -1;
    }
  }
  if (r1 == 0) {
    f.rank = 1;
    f.dim[0] = 1;
    f.perm[0] = 0;
    computeStrides(f);
    return;
  }
  int p1[MAXR] = {};  // r1 entries: perm is a bijection (checked by checkInput)
  int m = 0;
  for (int i = 0; i < rank; ++i)
    if (newIdx[perm[i]] >= 0) p1[m++] = newIdx[perm[i]];
  // 2. Walking the output order, an input rank that directly follows the
  //    previous one in the input joins its group (it stays adjacent).
  int gStart[MAXR];
  int64_t gDim[MAXR];
  int ng = 0;
  for (int i = 0; i < r1; ++i) {
    if (i > 0 && p1[i] == p1[i - 1] + 1) {
      gDim[ng - 1] *= d1[p1[i]];
    } else {
      gStart[ng] = p1[i];
      gDim[ng] = d1[p1[i]];
      ++ng;
    }
  }
  // 3. Number the groups by their position in the input.
  int order[MAXR];
  for (int g = 0; g < ng; ++g) order[g] = g;
  std::sort(order, order + ng, [&](int a, int b) { return gStart[a] < gStart[b]; });
  int inRank[MAXR];
  for (int k = 0; k < ng; ++k) inRank[order[k]] = k;
  f.rank = ng;
  for (int g = 0; g < ng; ++g) {
    f.dim[inRank[g]] = gDim[g];
    f.perm[g] = inRank[g];
  }
  computeStrides(f);
}

// ---------------------------------------------------------------------------
// Tile choice
// ---------------------------------------------------------------------------

namespace {

struct RunInfo {
  int64_t run;   // contiguous elements
  int frontier;  // first rank (in that order) not fully inside the tile, -1 if none
};

RunInfo runOf(const Fused& f, const int64_t* e, bool outputSide) {
  RunInfo ri{1, -1};
  for (int i = 0; i < f.rank; ++i) {
    int r = outputSide ? f.perm[i] : i;
    ri.run *= e[r];
    if (e[r] < f.dim[r]) {
      ri.frontier = r;
      return ri;
    }
  }
  return ri;
}

int64_t ceilDiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Relative offsets inside a tile must fit in int32.
bool offsetsFit(const Fused& f, const int64_t* e) {
  int64_t si = 0, so = 0;
  for (int r = 0; r < f.rank; ++r) {
    si += (e[r] - 1) * f.sin[r];
    so += (e[r] - 1) * f.sout[r];
  }
  return si < (int64_t(1) << 31) && so < (int64_t(1) << 31);
}

// Extent for a rank of dim d cut into chunks, at most `want` and more than
// `cur`: prefer a divisor of d (no ragged last chunk) that is a multiple of
// the 16-byte unit V when d is, among the 96 values below `want` and within
// 60% of it; else equal chunks.
// Results of pickExtent for one fused problem (its callers in one
// enumeration repeat arguments often): a small direct-mapped memo.
struct ExtentMemo {
  static constexpr int N = 32;
  int64_t d[N], want[N], cur[N], e[N];
  bool used[N] = {};
};

int64_t pickExtentUncached(int64_t d, int64_t want, int64_t cur, int V);

int64_t pickExtent(int64_t d, int64_t want, int64_t cur, int V, ExtentMemo* memo) {
  if (memo == nullptr) return pickExtentUncached(d, want, cur, V);
  const int h = (int)((uint64_t)(d * 31 + want * 7 + cur) % ExtentMemo::N);
  if (memo->used[h] && memo->d[h] == d && memo->want[h] == want && memo->cur[h] == cur)
    return memo->e[h];
  const int64_t e = pickExtentUncached(d, want, cur, V);
  memo->used[h] = true;
  memo->d[h] = d;
  memo->want[h] = want;
  memo->cur[h] = cur;
  memo->e[h] = e;
  return e;
}

int64_t pickExtentUncached(int64_t d, int64_t want, int64_t cur, int V) {
  int64_t lo = std::max(std::max(cur + 1, (want * 3 + 4) / 5), want - 95);
  // one descending scan: the first divisor that is a multiple of V (when
  // that is preferred), else the first divisor
  const bool preferV = V > 1 && d % V == 0;
  int64_t firstDiv = 0;
  auto scan = [&](auto dd) -> int64_t {
    using U = decltype(dd);
    for (int64_t c = want; c >= lo; --c) {
      if (dd % (U)c != 0) continue;
      if (!preferV || c % V == 0) return c;
      if (firstDiv == 0) firstDiv = c;
    }
    return 0;
  };
  const int64_t hit = d <= 0xffffffffLL ? scan((uint32_t)d) : scan((uint64_t)d);
  if (hit != 0) return hit;
  if (firstDiv != 0) return firstDiv;
  int64_t nch = ceilDiv(d, want);
  int64_t e = ceilDiv(d, nch);
  if (V > 1 && d % V == 0 && e % V != 0) {
    int64_t up = (e + V - 1) / V * V;
    if (up <= want) e = up;
  }
  return e;
}

// Greedy growth of the tile until both the input-contiguous and the
// output-contiguous runs reach `targetElems`, or the tile reaches `maxVol`.
// The side with the shorter run grows first; a rank that cannot be covered
// whole is cut into equal chunks so the last chunk is not a sliver.
void chooseExtents(const Fused& f, int64_t targetElems, int64_t maxVol, int64_t fillVol,
                   int64_t* e, ExtentMemo* memo = nullptr) {
  for (int r = 0; r < MAXR; ++r) e[r] = 1;
  int64_t vol = 1;
  bool blocked[2] = {false, false};
  bool filling = false;
  for (int iter = 0; iter < 8 * MAXR + 16; ++iter) {
    RunInfo ri = runOf(f, e, false), ro = runOf(f, e, true);
    bool needIn = ri.run < targetElems && ri.frontier >= 0 && !blocked[0];
    bool needOut = ro.run < targetElems && ro.frontier >= 0 && !blocked[1];
    if (!needIn && !needOut && !filling && vol < fillVol) {
      // Both runs are long enough but the tile is small: keep growing the
      // shorter side (by doubling) until the tile reaches fillVol.
      filling = true;
      blocked[0] = blocked[1] = false;
    }
    if (filling) {
      if (vol >= fillVol) break;
      needIn = ri.frontier >= 0 && !blocked[0];
      needOut = ro.frontier >= 0 && !blocked[1];
      targetElems = std::max(ri.run, ro.run) * 2;
    }
    if (!needIn && !needOut) break;
    int side = (needIn && (!needOut || ri.run <= ro.run)) ? 0 : 1;
    const RunInfo& rs = side == 0 ? ri : ro;
    int fr = rs.frontier;
    int64_t base = rs.run / e[fr];
    int64_t want = std::max(e[fr] + 1, ceilDiv(targetElems, base));
    int64_t enew = std::min<int64_t>(f.dim[fr], want);
    int64_t cap = (filling ? std::min(maxVol, fillVol * 2 - 1) : maxVol) / (vol / e[fr]);
    if (enew > cap) enew = cap;
    if (enew < f.dim[fr] && enew > e[fr])
      enew = pickExtent(f.dim[fr], enew, e[fr], 16 / f.esize, memo);
    if (enew <= e[fr]) {
      blocked[side] = true;
      continue;
    }
    int64_t old = e[fr];
    e[fr] = enew;
    if (!offsetsFit(f, e)) {
      e[fr] = old;
      blocked[side] = true;
      continue;
    }
    vol = vol / old * enew;
  }
}

}  // namespace

void tileTablesHost(const TileParams& tp, int* ldOff, int* stOff, unsigned short* stSm) {
  for (int u = 0; u < tp.nIn; ++u) {
    int rem = u * tp.lv, off = 0;
    for (int t = 0; t < tp.nTR; ++t) {
      const int c = rem % tp.trE[t];
      rem /= tp.trE[t];
      off += c * tp.trSin[t];
    }
    ldOff[u] = off;
  }
  for (int q = 0; q < tp.tileVol; ++q) {
    int rem = q, off = 0, jj = 0;
    for (int i = 0; i < tp.nTR; ++i) {
      const int t = tp.trOut[i];
      const int c = rem % tp.trE[t];
      rem /= tp.trE[t];
      off += c * tp.trSout[t];
      jj += c * tp.trInTile[t];
    }
    stSm[q] = (unsigned short)(jj + ((jj >> tp.padShift) << tp.padLog));
    if (q % tp.sv == 0) stOff[q / tp.sv] = off;
  }
}

GroupRunSplit groupRunSplit(const TileParams& tp) {
  GroupRunSplit rs;
  int k = 0;
  long long run = 1;
  while (k < tp.nTR && tp.trSin[k] == run) run *= tp.trE[k++];
  rs.inRun = (int)run;
  rs.kIn = k;
  k = 0;
  run = 1;
  while (k < tp.nTR && tp.trSout[tp.trOut[k]] == run) run *= tp.trE[tp.trOut[k++]];
  rs.outRun = (int)run;
  rs.kOut = k;
  return rs;
}

int bulkSegment(const TileParams& tp, int padShift) {
  const int inRun = groupRunSplit(tp).inRun;
  if (padShift >= PAD_NONE) return inRun;
  const int block = 1 << padShift;  // elements between two padding gaps
  if (block % inRun == 0) return inRun;
  if (inRun % block == 0) return block;
  return 0;
}

int groupLoadStep(const TileParams& tp, const GroupRunSplit& rs, int esize) {
  long long step = 0;
  int prev = -1;
  for (int t = rs.kIn; t < tp.nTR; ++t) {
    if (tp.trE[t] <= 1) continue;
    if (prev < 0)
      step = tp.trSin[t];
    else if ((long long)tp.trSin[t] != (long long)tp.trE[prev] * tp.trSin[prev])
      return -1;
    prev = t;
  }
  if (step * esize > 0x7fffffffLL) return -1;
  return (int)step;
}

GroupStoreSteps groupStoreSteps(const TileParams& tp, const GroupRunSplit& rs, int esize) {
  GroupStoreSteps st;
  long long so = 0, si = 0;
  int prev = -1;
  bool ok = true;
  for (int i = rs.kOut; i < tp.nTR && ok; ++i) {
    const int t = tp.trOut[i];
    if (tp.trE[t] <= 1) continue;
    if (prev < 0) {
      so = tp.trSout[t];
      si = tp.trInTile[t];
    } else {
      ok = (long long)tp.trSout[t] == (long long)tp.trE[prev] * tp.trSout[prev] &&
           (long long)tp.trInTile[t] == (long long)tp.trE[prev] * tp.trInTile[prev];
    }
    prev = t;
  }
  if (ok && so * esize <= 0x7fffffffLL) {
    st.outStep = (int)so;
    st.rowSmStep = (int)si;
  }
  si = 0;
  prev = -1;
  ok = true;
  for (int i = 0; i < rs.kOut && ok; ++i) {
    const int t = tp.trOut[i];
    if (tp.trE[t] <= 1) continue;
    if (prev < 0)
      si = tp.trInTile[t];
    else
      ok = (long long)tp.trInTile[t] == (long long)tp.trE[prev] * tp.trInTile[prev];
    prev = t;
  }
  if (ok) st.smStep = (int)si;
  return st;
}

void groupRunTablesHost(const TileParams& tp, const GroupRunSplit& rs, int* ldRow, int* stRow,
                        int* smRow, int* smRun) {
  for (int r = 0; r < tp.tileVol / rs.inRun; ++r) {
    int rem = r, off = 0;
    for (int t = rs.kIn; t < tp.nTR; ++t) {
      off += (rem % tp.trE[t]) * tp.trSin[t];
      rem /= tp.trE[t];
    }
    ldRow[r] = off;
  }
  for (int r = 0; r < tp.tileVol / rs.outRun; ++r) {
    int rem = r, off = 0, jj = 0;
    for (int i = rs.kOut; i < tp.nTR; ++i) {
      const int t = tp.trOut[i];
      const int c = rem % tp.trE[t];
      rem /= tp.trE[t];
      off += c * tp.trSout[t];
      jj += c * tp.trInTile[t];
    }
    stRow[r] = off;
    smRow[r] = jj;
  }
  for (int a = 0; a < rs.outRun; ++a) {
    int rem = a, jj = 0;
    for (int i = 0; i < rs.kOut; ++i) {
      const int t = tp.trOut[i];
      jj += (rem % tp.trE[t]) * tp.trInTile[t];
      rem /= tp.trE[t];
    }
    smRun[a] = jj;
  }
}

namespace {

// Wavefronts of 32-lane accesses: phases of 128 bytes; per phase the largest
// number of distinct 4-byte words any bank is asked for (a lane touches
// wordsPerLane consecutive words, so it never hits one bank twice).
// Addresses within one access are distinct (every lane touches its own
// elements, and the padding map is injective), so a phase costs the largest
// number of words that fall into one bank.
long long phaseCost(const int* addr, const bool* act, int wordsPerLane) {
  long long cost = 0;
  const int lanesPerPhase = std::max(1, 32 / wordsPerLane);
  for (int ph = 0; ph < 32; ph += lanesPerPhase) {
    // Closed form for an arithmetic progression of start words over the
    // phase's active lanes (all of them, or a prefix), stride s: lanes l and
    // l' share a start bank iff (l - l') * s == 0 mod 32, i.e. iff
    // P = 32 / g divides l - l' (g = gcd(s, 32), a power of two); distinct
    // start banks are at least g apart, so with wordsPerLane <= g no two
    // lanes' word ranges overlap across start banks, and the busiest bank
    // holds ceil(L / P) words of the L lanes.
    int L = 0;
    while (L < lanesPerPhase && act[ph + L]) ++L;
    bool prefix = true;
    for (int l = ph + L; l < ph + lanesPerPhase && prefix; ++l) prefix = !act[l];
    if (prefix && L <= 1) {
      cost += L;
      continue;
    }
    if (prefix) {
      const int s = addr[ph + 1] - addr[ph];
      bool ap = true;
      for (int l = ph + 2; l < ph + L && ap; ++l) ap = addr[l] - addr[l - 1] == s;
      if (ap) {
        const int sm = s & 31;
        const int g = sm == 0 ? 32 : (sm & -sm);  // gcd(s, 32)
        if (wordsPerLane <= g) {
          const int P = 32 / g;
          cost += (L + P - 1) / P;
          continue;
        }
      }
    }
    // Lanes whose start word is a multiple of wordsPerLane (a power of two;
    // always so for the engine's aligned units) each touch one aligned group
    // of wordsPerLane banks: the busiest bank's count is then the largest
    // number of lanes in one group, one increment per lane.  Otherwise every
    // word is counted.
    unsigned char cnt[32] = {};
    int maxPerBank = 0;
    const int groups = 32 / wordsPerLane;
    bool aligned = true;
    for (int l = ph; l < ph + lanesPerPhase; ++l) {
      if (!act[l]) continue;
      if (addr[l] & (wordsPerLane - 1)) {
        aligned = false;
        break;
      }
      const int c = ++cnt[(addr[l] / wordsPerLane) & (groups - 1)];
      maxPerBank = c > maxPerBank ? c : maxPerBank;
    }
    if (!aligned) {
      std::memset(cnt, 0, sizeof(cnt));
      maxPerBank = 0;
      for (int l = ph; l < ph + lanesPerPhase; ++l) {
        if (!act[l]) continue;
        for (int q = 0; q < wordsPerLane; ++q) {
          const int c = ++cnt[(addr[l] + q) & 31];
          maxPerBank = c > maxPerBank ? c : maxPerBank;
        }
      }
    }
    cost += maxPerBank;
  }
  return cost;
}

// Input-order index of the first n = min(nOut, sampleUnits) store units'
// elements (element m of unit w at j[m * n + w], n * sv entries); independent
// of the padding.  Returns n.
int storeSample(const TileParams& tp, int sampleUnits, int* j) {
  const int n = std::min(tp.nOut, sampleUnits);
  // output-order elements q = w * sv + m in sequence: a mixed-radix counter
  // over the tile ranks in output order carries the input-order index
  int digit[MAXR] = {};
  int jj = 0;
  for (int w = 0; w < n; ++w)
    for (int m = 0; m < tp.sv; ++m) {
      j[(size_t)m * n + w] = jj;
      for (int i = 0; i < tp.nTR; ++i) {
        const int t = tp.trOut[i];
        jj += tp.trInTile[t];
        if (++digit[i] < tp.trE[t]) break;
        jj -= tp.trE[t] * tp.trInTile[t];
        digit[i] = 0;
      }
    }
  return n;
}

// Simulated wavefronts of the sampled load and store units at a padding.
// The count stops once it reaches `limit` (the result is then >= limit):
// the padding search only asks whether a padding beats the best so far.
long long wavefronts(const TileParams& tp, int esize, int padShift, int sampleUnits,
                     const int* jStore, int nStore, long long limit = LLONG_MAX) {
  const int words = esize / 4;
  auto smIdx = [&](int j) { return j + ((j >> padShift) << tp.padLog); };
  int addr[32];
  bool act[32];
  long long total = 0;
  const int nIn = std::min(tp.nIn, sampleUnits);
  for (int base = 0; base < nIn; base += 32) {
    for (int l = 0; l < 32; ++l) {
      const int u = base + l;
      act[l] = u < nIn;
      addr[l] = act[l] ? smIdx(u * tp.lv) * words : 0;
    }
    total += phaseCost(addr, act, words * tp.lv);
    if (total >= limit) return total;
  }
  for (int base = 0; base < nStore; base += 32) {
    for (int m = 0; m < tp.sv; ++m) {
      for (int l = 0; l < 32; ++l) {
        const int w = base + l;
        act[l] = w < nStore;
        addr[l] = act[l] ? smIdx(jStore[(size_t)m * nStore + w]) * words : 0;
      }
      total += phaseCost(addr, act, words);
      if (total >= limit) return total;
    }
  }
  return total;
}

}  // namespace

long long smemWavefronts(const TileParams& tp, int esize, int padShift, int sampleUnits) {
  std::vector<int> j((size_t)std::min(tp.nOut, std::max(sampleUnits, 0)) * tp.sv);
  const int n = storeSample(tp, sampleUnits, j.data());
  return wavefronts(tp, esize, padShift, sampleUnits, j.data(), n);
}

namespace {

int nextPow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

int log2i(int x) {
  int l = 0;
  while ((1 << l) < x) ++l;
  return l;
}

// V (elements, V * esize <= 16 bytes) when units of V elements never
// straddle a run boundary and stay V-element aligned for one side (input or
// output order), including the shifted last chunks of ragged ranks; else 1.
int unitFor(const Fused& f, const int64_t* e, bool outputSide, int V) {
  if (V <= 1) return 1;
  RunInfo ri = runOf(f, e, outputSide);
  if (ri.run % V != 0) return 1;
  if (ri.frontier >= 0) {
    int64_t prefix = 1;
    for (int i = 0; i < f.rank; ++i) {
      int r = outputSide ? f.perm[i] : i;
      prefix *= f.dim[r];
      if (r == ri.frontier) break;
    }
    if (prefix % V != 0) return 1;
  }
  for (int r = 0; r < f.rank; ++r) {
    if (f.dim[r] % e[r] == 0) continue;
    int64_t s = outputSide ? f.sout[r] : f.sin[r];
    if (((f.dim[r] - e[r]) * s) % V != 0) return 1;
  }
  return V;
}

// Tile geometry for extents e with the requested units (reduced to element
// units where the layout does not allow them): tile and grid ranks, units,
// and the padding that minimises shared-memory bank wavefronts.  Shared by
// the three pipelines.  Returns false when the tile does not fit the
// kernels' limits.
bool buildTileGeometry(const Fused& f, const int64_t* e, int lv, int sv, TileParams& tp,
                       bool padSearch = true, long long noneWavefronts = -1,
                       int bulkMinElems = 0, int maxVol = TILE_MAX_VOL) {
  std::memset(&tp, 0, sizeof(tp));
  int trOfRank[MAXR];
  int nTR = 0;
  int64_t vol = 1;
  for (int r = 0; r < f.rank; ++r) {
    vol *= e[r];
    if (e[r] > 1) {
      trOfRank[r] = nTR;
      tp.trE[nTR] = (int)e[r];
      tp.trSin[nTR] = (int)f.sin[r];
      tp.trSout[nTR] = (int)f.sout[r];
      ++nTR;
    } else {
      trOfRank[r] = -1;
    }
  }
  if (vol > maxVol || vol < 1) return false;
  tp.nTR = nTR;
  tp.tileVol = (int)vol;
  int s = 1;
  for (int t = 0; t < nTR; ++t) {
    tp.trInTile[t] = s;
    s *= tp.trE[t];
  }
  int k = 0;
  for (int i = 0; i < f.rank; ++i)
    if (trOfRank[f.perm[i]] >= 0) tp.trOut[k++] = trOfRank[f.perm[i]];
  for (int t = 0; t < nTR; ++t) {
    tp.trMul[t] = (uint32_t)(((uint64_t(1) << 32) + tp.trE[t] - 1) / tp.trE[t]);
    const int o = tp.trOut[t];
    tp.toE[t] = tp.trE[o];
    tp.toSout[t] = tp.trSout[o];
    tp.toInTile[t] = tp.trInTile[o];
  }
  for (int t = 0; t < nTR; ++t) tp.toMul[t] = tp.trMul[tp.trOut[t]];
  // Grid ranks, decoded in output order so that consecutive tiles write
  // neighbouring output; except that the first input grid rank goes first
  // when it has at most kInputFirstChunks chunks (and fewer than the first
  // output grid rank): then the few tiles that share a band of input run
  // back to back, and output neighbours are only that many tiles apart, so
  // both sides' partly shared 64-byte DRAM atoms meet in L2.  On the
  // random-shape suite this took 17 problems from 0.91-0.95 of their best
  // to par (up to 14 % faster each), and larger counts measured slower.
  constexpr int64_t kInputFirstChunks = 16;
  int order[MAXR];
  for (int i = 0; i < f.rank; ++i) order[i] = f.perm[i];
  {
    int a = -1, b = -1;
    for (int i = 0; i < f.rank && a < 0; ++i)
      if (ceilDiv(f.dim[f.perm[i]], e[f.perm[i]]) > 1) a = i;
    for (int r = 0; r < f.rank && b < 0; ++r)
      if (ceilDiv(f.dim[r], e[r]) > 1) b = r;
    if (a >= 0 && b >= 0 && f.perm[a] != b) {
      const int64_t nb = ceilDiv(f.dim[b], e[b]);
      if (nb <= kInputFirstChunks && nb < ceilDiv(f.dim[f.perm[a]], e[f.perm[a]])) {
        int pos = a;
        while (order[pos] != b) ++pos;
        for (int i = pos; i > a; --i) order[i] = order[i - 1];
        order[a] = b;
      }
    }
  }
  int nGR = 0;
  int64_t numTiles = 1;
  for (int i = 0; i < f.rank; ++i) {
    int r = order[i];
    int64_t nch = ceilDiv(f.dim[r], e[r]);
    if (nch <= 1) continue;
    if (nch >= (int64_t(1) << 31)) return false;
    tp.grDiv[nGR] = makeFastDiv((uint32_t)nch);
    tp.grSin[nGR] = e[r] * f.sin[r];
    tp.grSout[nGR] = e[r] * f.sout[r];
    tp.grLastIn[nGR] = (f.dim[r] - e[r]) * f.sin[r];
    tp.grLastOut[nGR] = (f.dim[r] - e[r]) * f.sout[r];
    if (f.dim[r] % e[r] != 0) ++tp.nRagged;
    numTiles *= nch;
    if (numTiles >= (int64_t(1) << 31)) return false;
    ++nGR;
  }
  tp.nGR = nGR;
  tp.numTiles = (uint32_t)numTiles;
  if (lv > 1 && unitFor(f, e, false, lv) < lv) lv = 1;
  if (sv > 1 && unitFor(f, e, true, sv) < sv) sv = 1;
  tp.lv = lv;
  tp.sv = sv;
  tp.storeStraddle = nTR > 0 && tp.toE[0] % sv != 0;
  tp.padLog = log2i(lv);
  tp.nIn = tp.tileVol / lv;
  tp.nOut = tp.tileVol / sv;
  long long best = -1;
  int bestShift = PAD_NONE;
  // conflict-free lower bound: one wavefront per 128-byte phase
  const int words = f.esize / 4;
  const int sIn = std::min(tp.nIn, 64), sOut = std::min(tp.nOut, 64);
  const long long bound = ((sIn + 31) / 32) * std::max(1, words * lv) +
                          ((sOut + 31) / 32) * sv * std::max(1, words);
  if (!padSearch) {
    // Screening skips the padding search unless some padding could push
    // the tile past the shared-index or shared-memory limits; then the
    // search decides feasibility exactly as a full enumeration would.
    const int worst = tp.tileVol + ((tp.tileVol >> 2) << tp.padLog) + 16;
    const int tableBytes = ((2 * tp.tileVol + 15) / 16) * 16 + ((4 * (tp.nIn + tp.nOut) + 15) / 16) * 16;
    if (worst > 65535 || tableBytes + TILE_STAGES * worst * f.esize > 227 * 1024) padSearch = true;
  }
  tp.screened = padSearch ? 0 : 1;
  int jStore[64 * 4];  // 64 store units of at most 4 elements
  // a screened tile stays unpadded; its bank count is simulated only when a
  // selector asks for it (bankPerUnitOf)
  const int nStore = padSearch ? storeSample(tp, 64, jStore) : 0;
  const int shifts[] = {PAD_NONE, 8, 7, 6, 5, 4, 3, 2};
  for (int sh : shifts) {
    if (!padSearch) break;
    if (sh < tp.padLog || (!padSearch && sh != PAD_NONE)) continue;
    // a bulk-copy tile keeps its input segments whole between padding gaps
    if (bulkMinElems > 0 && sh != PAD_NONE && bulkSegment(tp, sh) < bulkMinElems) continue;
    // the unpadded tile's count may be known from screening
    // a padding that cannot beat the best so far stops counting early
    long long w = sh == PAD_NONE && noneWavefronts >= 0
                      ? noneWavefronts
                      : wavefronts(tp, f.esize, sh, 64, jStore, nStore,
                                   best < 0 ? LLONG_MAX : best);
    if (best < 0 || w < best) {
      best = w;
      bestShift = sh;
    }
    if (best <= bound) break;
  }
  tp.padShift = bestShift;
  tp.bankWavefronts = (int)best;
  tp.smStride = tp.tileVol + ((tp.tileVol >> bestShift) << tp.padLog);
  int perVec = 16 / f.esize;
  if (perVec > 1) tp.smStride = (tp.smStride + perVec - 1) / perVec * perVec;
  if (tp.smStride + 16 > 65535) return false;  // shared indices are 16-bit
  return true;
}

// Dynamic shared memory of a tile plan for one pipeline.
int tileSmemBytes(const TileParams& tp, int esize, int pipe) {
  if (flatTables(pipe)) return tp.smStride * esize;  // tables live in device memory
  const int tableBytes = ((2 * tp.tileVol + 15) / 16) * 16 + ((4 * (tp.nIn + tp.nOut) + 15) / 16) * 16;
  return tableBytes + (pipe == PIPE_ASYNC ? TILE_STAGES : 2) * tp.smStride * esize;
}

// Smallest bulk copy the bulk pipeline issues: shorter segments move as
// 16-byte cp.async units in the flat pipeline instead.
constexpr int BULK_MIN_BYTES = 128;

// PlanDesc of a tile candidate from its geometry and pipeline.
bool buildTile(const Fused& f, const int64_t* e, int pipe, const TileParams& geom, PlanDesc& pd) {
  if ((pipe == PIPE_ASYNC || pipe == PIPE_BULK) && geom.lv * f.esize != 16) return false;
  int seg = 0;
  if (pipe == PIPE_BULK) {
    seg = bulkSegment(geom, geom.padShift);
    if (seg * f.esize < BULK_MIN_BYTES || geom.tileVol % seg != 0) return false;
  }
  const int smem = tileSmemBytes(geom, f.esize, pipe);
  if (smem > 227 * 1024) return false;
  pd.pipe = pipe;
  pd.tile = geom;
  pd.tile.segLen = seg;
  for (int r = 0; r < f.rank; ++r) pd.extent[r] = e[r];
  pd.kernel = K_TILE;
  pd.threads = TILE_THREADS;
  pd.slots = nextPow2((geom.nIn + TILE_THREADS - 1) / TILE_THREADS);
  pd.ragged = geom.nRagged > 0;
  pd.smemBytes = smem;
  pd.padShift = geom.padShift;
  pd.unitBytes = geom.lv * f.esize;
  pd.unitOutBytes = geom.sv * f.esize;
  pd.numWork = geom.numTiles;
  RunInfo ri = runOf(f, e, false), ro = runOf(f, e, true);
  pd.runInBytes = (int)std::min<int64_t>(ri.run * f.esize, 1 << 30);
  pd.runOutBytes = (int)std::min<int64_t>(ro.run * f.esize, 1 << 30);
  // Method label in LibreTT's terms.
  int p0 = f.perm[0];
  bool partial = false;
  for (int r = 0; r < f.rank; ++r)
    if (e[r] > 1 && e[r] < f.dim[r]) partial = true;
  if (geom.nTR == 2 && p0 != 0 && e[0] > 1 && e[p0] > 1)
    pd.method = Tiled;
  else if (partial)
    pd.method = PackedSplit;
  else
    pd.method = Packed;
  return true;
}

bool buildRows(const Fused& f, int unit, RowParams& rp) {
  std::memset(&rp, 0, sizeof(rp));
  int64_t rowBytes = f.dim[0] * f.esize;
  if (rowBytes % unit != 0) return false;
  int64_t rowUnits = rowBytes / unit;
  if (rowUnits >= (int64_t(1) << 31)) return false;
  rp.rowUnits = (int)rowUnits;
  int64_t numRows = 1;
  int n = 0;
  for (int i = 1; i < f.rank; ++i) {
    int r = f.perm[i];
    rp.rDiv[n] = makeFastDiv((uint32_t)f.dim[r]);
    rp.rSin[n] = f.sin[r] * f.esize / unit;
    rp.rSout[n] = f.sout[r] * f.esize / unit;
    numRows *= f.dim[r];
    if (numRows >= (int64_t(1) << 31)) return false;
    ++n;
  }
  rp.nR = n;
  rp.numRows = (uint32_t)numRows;
  int64_t chunks = (rowUnits + 31) / 32;
  if (numRows * chunks >= (int64_t(1) << 31)) return false;
  rp.chunkDiv = makeFastDiv((uint32_t)chunks);
  rp.numItems = (uint32_t)(numRows * chunks);
  return true;
}

// ---------------------------------------------------------------------------
// Analytic model: DRAM sectors touched (sampled over a few tiles), partial
// sector writes, parallelism and bytes in flight.
// ---------------------------------------------------------------------------

constexpr double kBandwidth = 6.8e12;   // bytes/s, measured copy ceiling class
constexpr double kLatency = 1.2e-6;     // s, one load round trip under load
constexpr double kLaunch = 2.5e-6;      // s, launch + tail
constexpr int kSmemPerSM = 228 * 1024;

int tileCtasPerSM(const PlanDesc& pd) {
  int bySmem = kSmemPerSM / (pd.smemBytes + 1024);
  int regsPerThread = 32 + (pd.pipe == PIPE_ASYNC ? 0 : pd.slots * pd.unitBytes / 4);
  int byRegs = 65536 / (TILE_THREADS * std::min(regsPerThread, 255));
  return std::max(1, std::min(std::min(bySmem, byRegs), 2048 / TILE_THREADS));
}

void decodeTileHost(const TileParams& tp, uint32_t tile, int64_t& bin, int64_t& bout) {
  bin = bout = 0;
  uint32_t rem = tile;
  for (int g = 0; g < tp.nGR; ++g) {
    uint32_t q = fastDivHost(rem, tp.grDiv[g]);
    uint32_t c = rem - q * tp.grDiv[g].d;
    rem = q;
    const bool last = c + 1 == tp.grDiv[g].d;
    bin += last ? tp.grLastIn[g] : (int64_t)c * tp.grSin[g];
    bout += last ? tp.grLastOut[g] : (int64_t)c * tp.grSout[g];
  }
}

// In-tile offset of element x numbered in input order (outputSide false)
// or output order (true), input or output strides.
int64_t inTileOffset(const TileParams& tp, int x, bool outputSide) {
  // digits by multiply-high (trMul), exact for in-tile indices below 2^16
  uint32_t rem = (uint32_t)x;
  int64_t off = 0;
  for (int i = 0; i < tp.nTR; ++i) {
    const int t = outputSide ? tp.trOut[i] : i;
    const uint32_t q = (uint32_t)(((uint64_t)rem * tp.trMul[t]) >> 32);
    const int c = (int)(rem - q * (uint32_t)tp.trE[t]);
    rem = q;
    off += (int64_t)c * (outputSide ? tp.trSout[t] : tp.trSin[t]);
  }
  return off;
}

// Model of a tile candidate.  DRAM traffic: a tile is tileVol/run runs per
// side; each run of L bytes starting at byte b touches ((b mod 32) + L + 31)/32
// sectors, averaged over runs sampled from a few tiles; output runs that
// start or end inside a sector are partial writes.  Shifted last chunks add
// their overlap.  Time = the largest of DRAM time, latency-bound time for
// the bytes in flight, and instruction issue time, plus launch overhead.
void modelTile(PlanDesc& pd, int numSMs) {
  const Fused& f = pd.f;
  const TileParams& tp = pd.tile;
  const int es = f.esize;
  const RunInfo ri = runOf(f, pd.extent, false), ro = runOf(f, pd.extent, true);
  const int64_t runIn = ri.run, runOut = ro.run;
  const int64_t nRunsIn = tp.tileVol / runIn, nRunsOut = tp.tileVol / runOut;
  const int tilesSampled = (int)std::min<uint32_t>(2, tp.numTiles);
  double secIn = 0, secOut = 0, partial = 0;
  int samples = 0;
  for (int s = 0; s < tilesSampled; ++s) {
    const uint32_t tile = (uint32_t)((int64_t)s * tp.numTiles / tilesSampled);
    int64_t bin, bout;
    decodeTileHost(tp, tile, bin, bout);
    const int64_t kIn = std::min<int64_t>(nRunsIn, 8), kOut = std::min<int64_t>(nRunsOut, 8);
    double si = 0, so = 0, pp = 0;
    for (int64_t k = 0; k < kIn; ++k) {
      const int64_t b = (bin + inTileOffset(tp, (int)(k * nRunsIn / kIn * runIn), false)) * es;
      si += (double)(((b & 31) + runIn * es + 31) >> 5);
    }
    for (int64_t k = 0; k < kOut; ++k) {
      const int64_t b = (bout + inTileOffset(tp, (int)(k * nRunsOut / kOut * runOut), true)) * es;
      const int64_t end = b + runOut * es;
      so += (double)(((b & 31) + runOut * es + 31) >> 5);
      pp += ((b & 31) != 0) + ((end & 31) != 0);
    }
    secIn += si / kIn * nRunsIn;
    secOut += so / kOut * nRunsOut;
    partial += pp / kOut * nRunsOut;
    ++samples;
  }
  secIn /= samples;
  secOut /= samples;
  partial /= samples;
  const double useful = (double)tp.tileVol * es;
  pd.effIn = useful / (secIn * 32.0);
  pd.effOut = useful / (secOut * 32.0);
  double overlap = 1.0;
  for (int r = 0; r < f.rank; ++r) {
    const int64_t nch = ceilDiv(f.dim[r], pd.extent[r]);
    overlap *= (double)(nch * pd.extent[r]) / (double)f.dim[r];
  }
  pd.overlap = overlap;
  const double dram = (secIn + secOut + partial) * 32.0 * tp.numTiles;
  const double tDram = dram / kBandwidth;
  const int occ = tileCtasPerSM(pd);
  pd.ctasPerSM = occ;
  const double conc = (double)numSMs * occ;
  const double active = std::min<double>(conc, tp.numTiles);
  const int ahead = pd.pipe == PIPE_ASYNC ? TILE_STAGES - 1 : 1;
  const double inflight = active * ahead * useful;  // loads in flight
  const double tFlight = (double)f.vol * es * overlap / std::max(1.0, inflight) * kLatency;
  const double waves = std::ceil((double)tp.numTiles / conc);
  const double tWaves = waves * 2 * kLatency;
  const double util = (double)tp.nIn / (pd.slots * TILE_THREADS);
  // instructions per element: ~8 per load unit and ~6 + 2 per element of a
  // store unit, over 4 schedulers x 32 lanes per SM
  const double instPerElem = 8.0 / tp.lv / util + 6.0 / tp.sv + 2.0;
  const double tIssue = (double)f.vol * overlap * instPerElem / (numSMs * 128.0 * 1.9e9);
  // shared wavefronts per 32 sampled accesses, or -1 when the tile's bank
  // count has not been simulated (screened candidates: bankPerUnitOf)
  const long long wf = tp.bankWavefronts;
  const int sampled = std::min(tp.nIn, 64) + std::min(tp.nOut, 64) * tp.sv;
  pd.bankPerUnit = wf < 0 ? -1.0 : sampled > 0 ? (double)wf * 32.0 / sampled : 0.0;
  pd.cost = std::max(std::max(tDram, tFlight), std::max(tWaves, tIssue)) + kLaunch;
  // Measured on the random-shape suite: one-tile-per-CTA launches beat the
  // persistent pipelines for most shapes at equal modelled traffic.
  if (flatTables(pd.pipe)) pd.cost *= 0.9;
}

void modelRows(PlanDesc& pd, int numSMs) {
  const Fused& f = pd.f;
  int64_t rowBytes = f.dim[0] * f.esize;
  // Sectors per row averaged over the row start alignments that occur.
  int64_t rows = f.vol / f.dim[0];
  int64_t sampleRows = std::min<int64_t>(rows, 64);
  double secIn = 0, secOut = 0;
  const RowParams& rp = pd.row;
  for (int64_t s = 0; s < sampleRows; ++s) {
    uint32_t row = (uint32_t)(s * rows / sampleRows);
    int64_t bi = 0, bo = 0;
    uint32_t rem = row;
    for (int g = 0; g < rp.nR; ++g) {
      uint32_t q = fastDivHost(rem, rp.rDiv[g]);
      uint32_t c = rem - q * rp.rDiv[g].d;
      rem = q;
      bi += (int64_t)c * rp.rSin[g];
      bo += (int64_t)c * rp.rSout[g];
    }
    int64_t ai = bi * pd.unitBytes, ao = bo * pd.unitBytes;
    secIn += (double)((ai + rowBytes - 1) / 32 - ai / 32 + 1);
    secOut += (double)((ao + rowBytes - 1) / 32 - ao / 32 + 1);
  }
  double scale = (double)rows / sampleRows;
  double tDram = (secIn + secOut) * 32.0 * scale / kBandwidth;
  double inflight = (double)numSMs * 64 * std::min<int64_t>(rowBytes, 4 * 32 * pd.unitBytes);
  double tFlight = (double)f.vol * f.esize / inflight * kLatency;
  pd.cost = std::max(tDram, tFlight) + kLaunch;
}

}  // namespace

// Tile candidates: (target contiguous run bytes, maximum tile bytes,
// minimum tile bytes), each in every pipeline of the set `pipes` that can run
// it (bulk copies need 16-byte load units and whole segments of 128 bytes or
// more).
void appendTileCandidates(const Fused& f, int numSMs, int pipes, std::vector<PlanDesc>& out,
                          bool screen) {
  const int knobs[][3] = {{512, 16384, 8192},  {256, 8192, 4096},   {128, 4096, 2048},
                          {1024, 32768, 16384}, {512, 32768, 16384}, {256, 4096, 0},
                          {2048, 65536, 32768}, {64, 2048, 0},       {256, 16384, 16384}};
  constexpr int NKNOBS = sizeof(knobs) / sizeof(knobs[0]);
  int64_t seen[NKNOBS][MAXR];  // extents already enumerated
  int nSeen = 0;
  ExtentMemo memo;  // the element size is fixed for the problem (V)
  const int V = 16 / f.esize;
  for (auto& kb : knobs) {
    int64_t target = std::max<int64_t>(1, kb[0] / f.esize);
    int64_t maxVol = std::min<int64_t>(TILE_MAX_VOL, std::max<int64_t>(1, kb[1] / f.esize));
    int64_t fillVol = std::min<int64_t>(maxVol, kb[2] / f.esize);
    int64_t* e = seen[nSeen];
    chooseExtents(f, target, maxVol, fillVol, e, &memo);
    bool dup = false;
    for (int k = 0; k < nSeen && !dup; ++k)
      dup = std::equal(e, e + f.rank, seen[k]);
    if (dup) continue;
    ++nSeen;
    TileParams geom;
    if (!buildTileGeometry(f, e, V, V, geom, !screen)) continue;
    int flatIdx = -1;  // this tile's flat candidate in `out`
    for (int pipe : {PIPE_REG, PIPE_ASYNC, PIPE_FLAT, PIPE_BULK}) {
      if (!(pipes & (1 << pipe))) continue;
      if (pipe == PIPE_BULK && flatIdx >= 0 && geom.lv * f.esize == 16) {
        const int seg = bulkSegment(geom, geom.padShift);
        if (seg * f.esize >= BULK_MIN_BYTES && geom.tileVol % seg == 0) {
          // the same tile, geometry and modelled cost as its flat twin
          out.push_back(out[flatIdx]);
          out.back().pipe = PIPE_BULK;
          out.back().tile.segLen = seg;
          continue;
        }
      }
      out.emplace_back();  // built in place (a candidate is ~4 KB)
      PlanDesc& pd = out.back();
      pd.f = f;
      pd.targetRunBytes = kb[0];
      pd.maxTileBytes = kb[1];
      pd.screened = geom.screened != 0;
      TileParams g2;
      const TileParams* use = &geom;
      if (pipe == PIPE_BULK && !screen && geom.padShift != PAD_NONE &&
          bulkSegment(geom, geom.padShift) * f.esize < BULK_MIN_BYTES) {
        // the padding chosen for the other pipelines splits the segments:
        // search again among the paddings that keep them whole
        const int bulkMin = (BULK_MIN_BYTES + f.esize - 1) / f.esize;
        if (!buildTileGeometry(f, e, V, V, g2, true, -1, bulkMin)) {
          out.pop_back();
          continue;
        }
        use = &g2;
      }
      if (!buildTile(f, e, pipe, *use, pd)) {
        out.pop_back();
        continue;
      }
      modelTile(pd, numSMs);
      if (pipe == PIPE_FLAT) flatIdx = (int)out.size() - 1;
    }
  }
}

std::vector<PlanDesc> flatTileCandidates(const Fused& f, int numSMs, bool screen) {
  std::vector<PlanDesc> out;
  out.reserve(12);
  appendTileCandidates(f, numSMs < 1 ? 1 : numSMs, PIPES_FLAT, out, screen);
  for (size_t i = 0; i < out.size(); ++i) {
    out[i].candidate = (int)i;
    out[i].numCandidates = (int)out.size();
  }
  return out;
}

namespace {
std::atomic<int> gAllPipelines{-1};
}

void setAllPipelines(bool all) { gAllPipelines.store(all ? 1 : 0); }

bool allPipelines() {
  int v = gAllPipelines.load();
  if (v < 0) {
    const char* e = std::getenv("LIBRETT_ALL_PIPELINES");
    v = (e != nullptr && e[0] == '1') ? 1 : 0;
    gAllPipelines.store(v);
  }
  return v == 1;
}

std::vector<PlanDesc> enumerateCandidates(const Fused& f, int numSMs, bool screen) {
  std::vector<PlanDesc> out;
  out.reserve(allPipelines() ? 40 : 24);  // candidates are ~4 KB: no regrowth
  if (numSMs < 1) numSMs = 1;
  if (f.rank == 1) {
    PlanDesc pd;
    pd.method = Trivial;
    pd.kernel = K_COPY;
    pd.f = f;
    pd.extent[0] = f.dim[0];
    pd.threads = COPY_THREADS;
    int64_t bytes = f.vol * f.esize;
    pd.unitBytes = (bytes % 16 == 0) ? 16 : f.esize;
    pd.copy.numUnits = bytes / pd.unitBytes;
    pd.numWork = pd.copy.numUnits;
    pd.runInBytes = pd.runOutBytes = (int)std::min<int64_t>(bytes, 1 << 30);
    pd.cost = 2.0 * bytes / kBandwidth + kLaunch;
    out.push_back(pd);
  } else {
    if (f.perm[0] == 0 && f.dim[0] * f.esize >= 128) {
      PlanDesc pd;
      pd.method = TiledCopy;
      pd.kernel = K_ROW;
      pd.f = f;
      pd.threads = ROW_THREADS;
      int64_t rowBytes = f.dim[0] * f.esize;
      pd.unitBytes = (rowBytes % 16 == 0) ? 16 : f.esize;
      pd.extent[0] = f.dim[0];
      for (int r = 1; r < f.rank; ++r) pd.extent[r] = 1;
      if (buildRows(f, pd.unitBytes, pd.row) && buildRows(f, f.esize, pd.rowScalar)) {
        pd.numWork = pd.row.numRows;
        pd.runInBytes = pd.runOutBytes = (int)std::min<int64_t>(rowBytes, 1 << 30);
        modelRows(pd, numSMs);
        out.push_back(pd);
      }
    }
    appendTileCandidates(f, numSMs, allPipelines() ? PIPES_ALL : PIPES_DEFAULT, out, screen);
  }
  for (size_t i = 0; i < out.size(); ++i) {
    out[i].candidate = (int)i;
    out[i].numCandidates = (int)out.size();
  }
  return out;
}

bool widenUnits8(PlanDesc& pd, bool aligned16) {
  if (pd.kernel != K_TILE || pd.f.esize != 4) return false;
  const TileParams& cur = pd.tile;
  // 16-byte sides stay (when the pointers allow them); 4-byte sides try 8
  const int lv = cur.lv == 4 && aligned16 ? 4 : 2;
  const int sv = cur.sv == 4 && aligned16 ? 4 : 2;
  TileParams geom;
  if (!buildTileGeometry(pd.f, pd.extent, lv, sv, geom)) return false;
  if (geom.lv <= cur.lv && geom.sv <= cur.sv) return false;
  PlanDesc w;
  w.f = pd.f;
  w.targetRunBytes = pd.targetRunBytes;
  w.maxTileBytes = pd.maxTileBytes;
  if (!buildTile(pd.f, pd.extent, PIPE_FLAT, geom, w)) return false;
  w.candidate = pd.candidate;
  w.numCandidates = pd.numCandidates;
  pd = w;
  return true;
}

namespace {

// Units (elements per load and per store unit) the grouped kernel uses for
// the tile with extents e: 16-byte units where the layout allows them, and
// for 4-byte elements with 8-byte aligned pointers (eight) 8-byte units on
// the other sides; element units on both sides when a side's units would
// cross a run of the tile.  False when the tile does not fit the kernels.
bool groupUnitsFor(const Fused& f, const int64_t* e, bool eight, int& lv, int& sv) {
  const int V = 16 / f.esize;
  TileParams g;
  if (!buildTileGeometry(f, e, V, V, g, false)) return false;
  lv = g.lv;
  sv = g.sv;
  GroupRunSplit rs = groupRunSplit(g);
  if (rs.inRun % lv != 0 || rs.outRun % sv != 0) lv = sv = 1;
  if (f.esize == 4 && eight && (lv < 4 || sv < 4) &&
      buildTileGeometry(f, e, lv == 4 ? 4 : 2, sv == 4 ? 4 : 2, g, false)) {
    rs = groupRunSplit(g);
    if (rs.inRun % g.lv == 0 && rs.outRun % g.sv == 0 && (g.lv > lv || g.sv > sv)) {
      lv = g.lv;
      sv = g.sv;
    }
  }
  return true;
}

// Rank of a unit pair, from the grouped kernel's measured bucket rates: the
// narrower side first (16 + 16 > 8 + 8 ~ 16 + 8 > 16 + 4 > 8 + 4 > 4 + 4
// bytes for 4-byte elements), then the sum.
int unitScore(int lv, int sv) { return 16 * std::min(lv, sv) + lv + sv; }

}  // namespace

bool widenUnitsByExtents(PlanDesc& pd, int numSMs, bool eight) {
  if (pd.kernel != K_TILE) return false;
  const Fused& f = pd.f;
  const int V = 16 / f.esize;
  if (V <= 1) return false;
  int lv0, sv0;
  if (!groupUnitsFor(f, pd.extent, eight, lv0, sv0)) return false;
  const int score0 = unitScore(lv0, sv0);
  if (score0 >= unitScore(V, V)) return false;
  const int64_t vol0 = pd.tile.tileVol;
  int bestScore = score0;
  int64_t bestVol = 0;
  int64_t best[MAXR], e[MAXR];
  for (int r = 0; r < f.rank; ++r) {
    if (pd.extent[r] <= 1) continue;
    for (int m = V; m >= 2; m /= 2) {
      const int64_t lo = pd.extent[r] / m * m;
      for (int64_t er : {lo, lo + m}) {
        if (er < 1 || er > f.dim[r] || er == pd.extent[r]) continue;
        for (int q = 0; q < f.rank; ++q) e[q] = pd.extent[q];
        e[r] = er;
        int64_t vol = 1;
        for (int q = 0; q < f.rank; ++q) vol *= e[q];
        // 3/4 to 5/4 of the volume the policy picked
        if (4 * vol < 3 * vol0 || 4 * vol > 5 * vol0) continue;
        int lv, sv;
        if (!groupUnitsFor(f, e, eight, lv, sv)) continue;
        const int sc = unitScore(lv, sv);
        if (sc < bestScore || (sc == bestScore && vol <= bestVol)) continue;
        bestScore = sc;
        bestVol = vol;
        std::copy(e, e + f.rank, best);
      }
    }
  }
  if (bestScore == score0) return false;
  TileParams geom;
  if (!buildTileGeometry(f, best, V, V, geom)) return false;
  PlanDesc c;
  c.f = f;
  c.targetRunBytes = pd.targetRunBytes;
  c.maxTileBytes = pd.maxTileBytes;
  if (!buildTile(f, best, pd.pipe, geom, c)) return false;
  modelTile(c, numSMs < 1 ? 1 : numSMs);
  c.candidate = pd.candidate;
  c.numCandidates = pd.numCandidates;
  pd = c;
  return true;
}

bool groupDoubleTile(PlanDesc& pd, int numSMs) {
  if (pd.kernel != K_TILE) return false;
  const Fused& f = pd.f;
  const TileParams& cur = pd.tile;
  const int lv = cur.lv, sv = cur.sv;
  // load units per thread stay within the kernel's 16 slots
  if (lv < 2 || GROUP_MAX_VOL / lv > TILE_THREADS * TILE_MAX_SLOTS) return false;
  const GroupRunSplit rs0 = groupRunSplit(cur);
  if (rs0.inRun % lv != 0 || rs0.outRun % sv != 0) return false;
  const double eff0 = std::min(pd.effIn, pd.effOut);
  PlanDesc best;
  bool found = false;
  int64_t e[MAXR];
  for (int r = 0; r < f.rank; ++r) {
    if (pd.extent[r] >= f.dim[r]) continue;
    for (int q = 0; q < f.rank; ++q) e[q] = pd.extent[q];
    e[r] = std::min<int64_t>(2 * pd.extent[r], f.dim[r]);
    TileParams geom;
    if (!buildTileGeometry(f, e, lv, sv, geom, true, -1, 0, GROUP_MAX_VOL)) continue;
    if (2 * geom.tileVol < 3 * cur.tileVol || geom.lv != lv || geom.sv != sv) continue;
    const GroupRunSplit rs = groupRunSplit(geom);
    if (rs.inRun % lv != 0 || rs.outRun % sv != 0) continue;
    PlanDesc c;
    c.f = f;
    c.targetRunBytes = pd.targetRunBytes;
    c.maxTileBytes = pd.maxTileBytes;
    if (!buildTile(f, e, pd.pipe, geom, c)) continue;
    modelTile(c, numSMs < 1 ? 1 : numSMs);
    const double eff = std::min(c.effIn, c.effOut);
    if (eff < 0.95 * eff0) continue;
    if (!found || eff > std::min(best.effIn, best.effOut) ||
        (eff == std::min(best.effIn, best.effOut) && c.tile.tileVol > best.tile.tileVol)) {
      best = c;
      found = true;
    }
  }
  if (!found) return false;
  best.candidate = pd.candidate;
  best.numCandidates = pd.numCandidates;
  pd = best;
  return true;
}

namespace {

// The screened (unpadded) tile's bank count, as a full build simulates it,
// and the feature it gives.
long long screenedWavefronts(const PlanDesc& pd) {
  const TileParams& tp = pd.tile;
  int jStore[64 * 4];
  const int nStore = storeSample(tp, 64, jStore);
  return wavefronts(tp, pd.f.esize, tp.padShift, 64, jStore, nStore);
}

double bankFeature(const TileParams& tp, long long wf) {
  const int sampled = std::min(tp.nIn, 64) + std::min(tp.nOut, 64) * tp.sv;
  return sampled > 0 ? (double)wf * 32.0 / sampled : 0.0;
}

}  // namespace

double bankPerUnitOf(const PlanDesc& pd) {
  if (pd.kernel != K_TILE || pd.bankPerUnit >= 0.0) return pd.bankPerUnit;
  return bankFeature(pd.tile, screenedWavefronts(pd));
}

void simulateBanks(PlanDesc& pd) {
  if (pd.kernel != K_TILE || pd.bankPerUnit >= 0.0) return;
  const long long wf = screenedWavefronts(pd);
  pd.tile.bankWavefronts = (int)wf;
  pd.bankPerUnit = bankFeature(pd.tile, wf);
}

bool refineCandidate(PlanDesc& pd, int numSMs) {
  if (pd.kernel != K_TILE || !pd.screened) return true;
  const int V = 16 / pd.f.esize;
  TileParams geom;
  // screening simulated the unpadded tile (the same geometry and units);
  // a bulk-copy tile only takes paddings that keep its segments whole
  const int bulkMin = pd.pipe == PIPE_BULK ? (BULK_MIN_BYTES + pd.f.esize - 1) / pd.f.esize : 0;
  if (!buildTileGeometry(pd.f, pd.extent, V, V, geom, true, pd.tile.bankWavefronts, bulkMin))
    return false;
  PlanDesc full;
  full.f = pd.f;
  full.targetRunBytes = pd.targetRunBytes;
  full.maxTileBytes = pd.maxTileBytes;
  if (!buildTile(pd.f, pd.extent, pd.pipe, geom, full)) return false;
  modelTile(full, numSMs < 1 ? 1 : numSMs);
  full.candidate = pd.candidate;
  full.numCandidates = pd.numCandidates;
  pd = full;
  return true;
}

bool finalizePlan(PlanDesc& pd) {
  if (pd.kernel != K_TILE) return true;
  // element-size units for misaligned pointers, run by the register-staged
  // pipeline (which builds its own tables)
  TileParams scalar;
  if (!buildTileGeometry(pd.f, pd.extent, 1, 1, scalar)) return false;
  const int smem = tileSmemBytes(scalar, pd.f.esize, PIPE_REG);
  if (smem > 227 * 1024) return false;
  pd.tileScalar = scalar;
  pd.smemBytesScalar = smem;
  pd.slotsScalar = nextPow2((scalar.nIn + TILE_THREADS - 1) / TILE_THREADS);
  return true;
}

int chooseHeuristic(const std::vector<PlanDesc>& cands) {
  int best = 0;
  for (size_t i = 1; i < cands.size(); ++i)
    if (cands[i].cost < cands[best].cost) best = (int)i;
  return best;
}

}  // namespace lt
