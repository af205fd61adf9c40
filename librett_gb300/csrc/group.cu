// Grouped execution (see group.h): member tile choice, bucketing, the CUDA
// graph, the tile-policy autotuner, and the public librettGroup* /
// librettExecuteGrouped entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "fault.h"
#include "group.h"
#include "kernels.cuh"
#include "launch.h"
#include "librett.h"
#include "librett_c.h"
#include "plans.h"
#include "select.h"

namespace lt {
extern std::atomic<unsigned long long> gLaunchCount;
namespace {

// Writes every member's run tables; CTA b handles member b.
__global__ void __launch_bounds__(256) writeGroupTablesKernel(const GroupTableJob* __restrict__ jobs) {
  const GroupTableJob& jb = jobs[blockIdx.x];
  const TileParams& p = jb.tp;
  const GroupRunSplit rs = jb.rs;
  const int nL = p.tileVol / rs.inRun, nS = p.tileVol / rs.outRun;
  for (int r = threadIdx.x; r < nL; r += blockDim.x) {
    int rem = r, off = 0;
    for (int t = rs.kIn; t < p.nTR; ++t) {
      const int e = p.trE[t];
      const int q = rem / e;
      off += (rem - q * e) * p.trSin[t];
      rem = q;
    }
    jb.ldRow[r] = off;
  }
  for (int r = threadIdx.x; r < nS; r += blockDim.x) {
    int rem = r, off = 0, jj = 0;
    for (int i = rs.kOut; i < p.nTR; ++i) {
      const int t = p.trOut[i];
      const int e = p.trE[t];
      const int q = rem / e;
      const int c = rem - q * e;
      rem = q;
      off += c * p.trSout[t];
      jj += c * p.trInTile[t];
    }
    jb.outRows[r] = make_int2(off, jj);
  }
  for (int a = threadIdx.x; a < rs.outRun; a += blockDim.x) {
    int rem = a, jj = 0;
    for (int i = 0; i < rs.kOut; ++i) {
      const int t = p.trOut[i];
      const int e = p.trE[t];
      const int q = rem / e;
      jj += (rem - q * e) * p.trInTile[t];
      rem = q;
    }
    jb.smRun[a] = jj;
  }
  // the member's tiles: corner offsets from the grid-rank decode (same
  // arithmetic as the single-plan kernels' decodeTile), with the descriptor
  // index in the top bits of the input offset
  for (uint32_t x = threadIdx.x; x < p.numTiles; x += blockDim.x) {
    uint32_t rem = x;
    long long bin = 0, bout = 0;
    for (int g = 0; g < p.nGR; ++g) {
      const uint32_t q = fdiv(rem, p.grDiv[g]);
      const uint32_t c = rem - q * p.grDiv[g].d;
      rem = q;
      const bool last = c + 1 == p.grDiv[g].d;
      bin += last ? p.grLastIn[g] : (long long)c * p.grSin[g];
      bout += last ? p.grLastOut[g] : (long long)c * p.grSout[g];
    }
    jb.tiles[x].inAndTensor = bin | (jb.tensor << GROUP_TILE_SHIFT);
    jb.tiles[x].out = bout;
  }
}

size_t align16(size_t x) { return (x + 15) / 16 * 16; }

// Bytes of a member's run tables; sub-table offsets (16-byte aligned):
// ldRow at off[0], outRows at off[1], smRun at off[2].
size_t runTableBytes(const TileParams& tp, const GroupRunSplit& rs, size_t off[3]) {
  const size_t nL = tp.tileVol / rs.inRun, nS = tp.tileVol / rs.outRun;
  off[0] = 0;
  off[1] = align16(4 * nL);
  off[2] = off[1] + align16(8 * nS);
  return off[2] + align16(4 * (size_t)rs.outRun);
}

// Policies: policy % GP_TILES picks a member's flat tile from its
// candidates; policy / GP_TILES picks the bucket's loads (0 registers,
// 1 cp.async, one tile per CTA; 2 cp.async with persistent CTAs).
enum GroupPolicy {
  GP_SELECTOR = 0,  // the plan selector's choice for the tensor on its own
  GP_WIDE = 1,      // the largest tile within 10% of the best sector efficiency
  GP_WIDEST = 2,    // the largest tile
  GP_FILL = 3,      // the analytic model with the device assumed full of other work
  GP_TILES = 4,
  GP_COUNT = 3 * GP_TILES
};
// Buckets share a kernel shape and the CTAs per SM that their shared memory
// allows (228 KB per SM, 1 KB reserved per CTA), capped at the 8 that the
// grouped kernels' 32 registers per thread allow: a bucket's launch uses its
// largest member's shared memory, which costs its other members no
// occupancy.  On the 10k batch: 37 buckets instead of 92 with 4 KB
// shared-memory classes, 10.445 -> 10.383 ms (three interleaved runs each).
int occClass(int smem) { return std::min(8, (228 * 1024) / (smem + 1024)); }
constexpr int STAGE_MAX = 8192;   // largest store-side table set staged in shared memory

// Bytes of a member's store-side run tables (outRows, smRun) when they are
// staged in shared memory, else 0.
int stagedTableBytes(const TileParams& tp, int esize) {
  const GroupRunSplit rs = groupRunSplit(tp);
  const GroupStoreSteps st = groupStoreSteps(tp, rs, esize);
  if (st.outStep >= 0 && st.smStep >= 0) return 0;  // the kernel reads no store table
  size_t off[3];
  const size_t total = runTableBytes(tp, rs, off);
  const size_t bytes = total - off[1];
  return bytes <= (size_t)STAGE_MAX ? (int)bytes : 0;
}

// Member class: size class (bytes of one tensor < 64 KiB, < 1 MiB, < 16 MiB,
// larger) + 4 * element-size index (4, 8, 16 bytes).
int memberClass(long long bytes, int esize) {
  const int sc = bytes < (1LL << 16) ? 0 : bytes < (1LL << 20) ? 1 : bytes < (1LL << 24) ? 2 : 3;
  return sc + 4 * (esize == 4 ? 0 : esize == 8 ? 1 : 2);
}

using Policy = std::array<int, GROUP_CLASSES>;

struct Member {
  std::shared_ptr<PlanObj> plan;  // the caller's plan (kept alive by the group)
  const unsigned char* in;
  unsigned char* out;
  int cls;
  bool aligned16;
  bool aligned8;
  int picked = -1;   // policy pd was chosen with (-1: none yet)
  bool separate = false;  // runs its plan's own launch
  PlanDesc pd;       // flat tile plan inside a bucket
};

struct BucketSummary {
  int es, lv, sv, nl, loads, members, smem;
  long long tiles, bytes;
};

struct Build {
  void* alloc = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int buckets = 0, separate = 0;
  long long tiles = 0;
  std::vector<BucketSummary> summary;  // in launch order
};

void releaseBuild(Build& b, cudaStream_t s) {
  // an executable graph still in flight is released when it completes
  if (b.exec) cudaGraphExecDestroy(b.exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  // stream-ordered: after every launch of this build on s
  if (b.alloc) cudaFreeAsync(b.alloc, s);
  b = Build();
}

struct GroupObj {
  cudaStream_t stream = nullptr;
  int device = 0;
  int numSMs = 0;
  std::string devName;
  std::vector<Member> members;
  Policy policy{};
  bool tuned = false;
  uint64_t signature = 0;
  long long bytes = 0;
  Build built;
  // Serialises execution against tuning (which rebuilds the graph) and the
  // introspection calls; creation builds before the group is published.
  std::mutex mu;
  GroupObj() = default;
  GroupObj(const GroupObj&) = delete;
  GroupObj& operator=(const GroupObj&) = delete;
  ~GroupObj() {
    releaseBuild(built, stream);
    // A separately launched member's plan frees its tables on the plan's own
    // stream once the last reference goes: order that after this group.
    cudaEvent_t done = nullptr;
    for (const Member& m : members) {
      if (!m.separate || m.plan->stream == stream) continue;
      if (done == nullptr && cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess)
        cudaEventRecord(done, stream);
      if (done) cudaStreamWaitEvent(m.plan->stream, done, 0);
    }
    if (done) cudaEventDestroy(done);
  }
};

std::mutex gGroupMu;
std::unordered_map<librettGroupHandle, std::shared_ptr<GroupObj>> gGroups;
std::atomic<librettGroupHandle> gNextGroup{0};

// Tuned policies by batch signature (members' shapes, alignment, device).
std::mutex gTuneMu;
std::unordered_map<uint64_t, Policy> gTuneCache;

uint64_t fnv(uint64_t h, uint64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (v >> (8 * i)) & 0xff;
    h *= 1099511628211ULL;
  }
  return h;
}

cudaError_t launchGroupBucket(int es, int lv, int sv, int nl, int loads, const GroupTensor* tens,
                              const GroupTile* map, uint32_t tiles, int smem, cudaStream_t s,
                              int numSMs) {
  switch (es) {
    case 4: return launchGroupTile4(lv, sv, nl, loads, tens, map, tiles, smem, s, numSMs);
    case 8: return launchGroupTile8(lv, sv, nl, loads, tens, map, tiles, smem, s, numSMs);
    case 16: return launchGroupTile16(lv, sv, nl, loads, tens, map, tiles, smem, s, numSMs);
    default: return cudaErrorInvalidValue;
  }
}

// Flat tile plan of member m under a policy; false when the member must run
// its plan's own launch.
bool pickTile(const Member& m, int policy, int sms, const std::string& dev, PlanDesc& out) {
  policy %= GP_TILES;
  const PlanDesc& own = m.plan->pd;
  if (policy == GP_SELECTOR && own.kernel == K_TILE && flatTables(own.pipe)) {
    out = own;  // the group uses the tile geometry only
  } else {
    // the selector ranks screened candidates (as for librettPlan)
    std::vector<PlanDesc> c =
        flatTileCandidates(own.f, policy == GP_FILL ? sms * 64 : sms, policy == GP_SELECTOR);
    if (c.empty()) return false;
    int k = 0;
    auto eff = [](const PlanDesc& p) { return std::min(p.effIn, p.effOut); };
    switch (policy) {
      case GP_SELECTOR:
        k = choosePlan(c, sms, dev.c_str(), nullptr);
        break;
      case GP_FILL:
        k = chooseHeuristic(c);
        break;
      case GP_WIDE: {
        double best = 0.0;
        for (const PlanDesc& p : c) best = std::max(best, eff(p));
        k = -1;
        for (int i = 0; i < (int)c.size(); ++i) {
          if (eff(c[i]) < 0.9 * best) continue;
          if (k < 0 || c[i].tile.tileVol > c[k].tile.tileVol ||
              (c[i].tile.tileVol == c[k].tile.tileVol && c[i].cost < c[k].cost))
            k = i;
        }
        break;
      }
      default:  // GP_WIDEST
        for (int i = 1; i < (int)c.size(); ++i)
          if (c[i].tile.tileVol > c[k].tile.tileVol ||
              (c[i].tile.tileVol == c[k].tile.tileVol && eff(c[i]) > eff(c[k])))
            k = i;
        break;
    }
    out = c[k];
    if (!refineCandidate(out, sms)) return false;
  }
  // narrower units than the element size allows: one rank's extent rounded
  // to a multiple of 2 .. 16 / esize elements may give the runs wider units
  if (m.aligned16 && out.kernel == K_TILE) {
    PlanDesc w = out;
    if (widenUnitsByExtents(w, sms, m.aligned8)) out = w;
  }
  const GroupRunSplit rs = groupRunSplit(out.tile);
  const bool unitsFit = rs.inRun % out.tile.lv == 0 && rs.outRun % out.tile.sv == 0;
  if ((!m.aligned16 || !unitsFit) && (out.tile.lv > 1 || out.tile.sv > 1)) {
    // pointers not 16-byte aligned, or vector units that would cross a run:
    // the same tile in element units
    if (!finalizePlan(out)) return false;
    out.tile = out.tileScalar;
    out.slots = out.slotsScalar;
    out.smemBytes = out.tile.smStride * out.f.esize;
  }
  if (out.f.esize == 4 && (out.tile.lv < 4 || out.tile.sv < 4) && m.aligned8) {
    // 4-byte elements: 8-byte units on the sides that cannot take 16-byte
    // ones, when the widened units still fit the member's runs
    PlanDesc w = out;
    if (widenUnits8(w, m.aligned16)) {
      const GroupRunSplit wrs = groupRunSplit(w.tile);
      if (wrs.inRun % w.tile.lv == 0 && wrs.outRun % w.tile.sv == 0) out = w;
    }
  }
  if (out.f.esize == 4 && out.tile.lv == 4 && out.tile.sv == 4) {
    // 4-byte elements in 16-byte units: a tile of up to twice the volume
    // (16 KB -> 32 KB, as 8-byte elements' tiles), more bytes per CTA.  The
    // 10k batch: 10.40 -> 10.35 ms; doubling every 4-byte-element tile with
    // 8- or 16-byte loads as well measured 10.38 ms (more, slower buckets).
    PlanDesc w = out;
    if (groupDoubleTile(w, sms)) out = w;
  }
  // the kernel's run division needs in-tile indices below 2^16 (RunDiv)
  if (out.tile.tileVol >= 65536) return false;
  // the tile data plus the staged store-side tables
  out.smemBytes = out.tile.smStride * out.f.esize + stagedTableBytes(out.tile, out.f.esize);
  return true;
}

struct Bucket {
  int es, lv, sv, nl, loads;
  int smem = 0;
  uint32_t tiles = 0;
  long long bytes = 0;
  std::vector<int> members;  // indices into GroupObj::members
  size_t tensOff = 0, mapOff = 0;
};

// (Re)builds the device image and the graph for a policy.  Synchronises the
// group's stream.
librettResult build(GroupObj& g, const Policy& pol) {
  for (Member& m : g.members) {
    const int p = pol[m.cls] % GP_TILES;
    if (m.picked == p) continue;
    m.separate = !pickTile(m, p, g.numSMs, g.devName, m.pd);
    m.picked = p;
  }
  if (cudaStreamSynchronize(g.stream) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  releaseBuild(g.built, g.stream);
  g.policy = pol;
  Build& B = g.built;

  // buckets by kernel shape
  std::map<std::tuple<int, int, int, int, int, int>, int> key2b;
  std::vector<Bucket> buckets;
  for (int i = 0; i < (int)g.members.size(); ++i) {
    const Member& m = g.members[i];
    if (m.separate) {
      if (m.plan->needsScalar(m.in, m.out) && !m.plan->ensureScalar())
        return LIBRETT_INTERNAL_ERROR;
      ++B.separate;
      continue;
    }
    const PlanDesc& pd = m.pd;
    const int loads = pol[m.cls] / GP_TILES;
    auto key = std::make_tuple(pd.f.esize, pd.tile.lv, pd.tile.sv, pd.slots, loads,
                               occClass(pd.smemBytes));
    auto it = key2b.find(key);
    if (it == key2b.end()) {
      Bucket b;
      b.es = pd.f.esize;
      b.lv = pd.tile.lv;
      b.sv = pd.tile.sv;
      b.nl = pd.slots;
      b.loads = loads;
      it = key2b.emplace(key, (int)buckets.size()).first;
      buckets.push_back(b);
    }
    Bucket& b = buckets[it->second];
    b.members.push_back(i);
    if ((uint64_t)b.tiles + pd.tile.numTiles >= (uint64_t(1) << 31)) return LIBRETT_INVALID_PARAMETER;
    b.tiles += pd.tile.numTiles;
    b.bytes += 2 * pd.f.vol * (long long)pd.f.esize;
    b.smem = std::max(b.smem, pd.smemBytes);
  }
  B.buckets = (int)buckets.size();
  // a tile packs its descriptor index above a 40-bit offset
  for (const Bucket& b : buckets)
    if (b.members.size() >= (size_t(1) << (63 - GROUP_TILE_SHIFT))) return LIBRETT_INVALID_PARAMETER;

  // one allocation: descriptors and table jobs (written from the host),
  // tile lists and the members' run tables (written by a kernel)
  size_t off = 0;
  for (Bucket& b : buckets) {
    b.tensOff = off;
    off = align16(off + b.members.size() * sizeof(GroupTensor));
  }
  for (Bucket& b : buckets) {
    b.mapOff = off;
    off = align16(off + (size_t)b.tiles * sizeof(GroupTile));
    B.tiles += b.tiles;
  }
  std::vector<int> jobOf(g.members.size(), -1);
  int nJobs = 0;
  for (const Bucket& b : buckets)
    for (int i : b.members) jobOf[i] = nJobs++;
  const size_t jobsOff = off;
  off = align16(off + (size_t)nJobs * sizeof(GroupTableJob));
  const size_t imageBytes = off;
  std::vector<size_t> tabOff(g.members.size(), 0);
  for (const Bucket& b : buckets)
    for (int i : b.members) {
      size_t sub[3];
      const TileParams& tp = g.members[i].pd.tile;
      tabOff[i] = off;
      off = align16(off + runTableBytes(tp, groupRunSplit(tp), sub));
    }
  const size_t total = std::max<size_t>(off, 16);
  if (injectFault(FAULT_GROUP_ALLOC) || cudaMallocAsync(&B.alloc, total, g.stream) != cudaSuccess) {
    B.alloc = nullptr;
    return LIBRETT_INTERNAL_ERROR;
  }
  unsigned char* base = static_cast<unsigned char*>(B.alloc);
  std::vector<unsigned char> host(std::max<size_t>(imageBytes, 16), 0);
  GroupTableJob* jobs = reinterpret_cast<GroupTableJob*>(host.data() + jobsOff);
  for (Bucket& b : buckets) {
    GroupTensor* tens = reinterpret_cast<GroupTensor*>(host.data() + b.tensOff);
    GroupTile* map = reinterpret_cast<GroupTile*>(base + b.mapOff);  // device
    uint32_t first = 0;
    for (size_t k = 0; k < b.members.size(); ++k) {
      const int i = b.members[k];
      const Member& m = g.members[i];
      const TileParams& tp = m.pd.tile;
      const GroupRunSplit rs = groupRunSplit(tp);
      size_t sub[3];
      runTableBytes(tp, rs, sub);
      unsigned char* tb = base + tabOff[i];
      GroupTensor& t = tens[k];
      std::memset(&t, 0, sizeof(t));
      t.in = m.in;
      t.out = m.out;
      t.ldRow = reinterpret_cast<const int*>(tb + sub[0]);
      t.outRows = reinterpret_cast<const int2*>(tb + sub[1]);
      t.smRun = reinterpret_cast<const int*>(tb + sub[2]);
      t.nIn = tp.nIn;
      t.nOut = tp.nOut;
      t.inRun = makeRunDiv((uint32_t)rs.inRun);
      t.outRun = makeRunDiv((uint32_t)rs.outRun);
      t.tabBytes = stagedTableBytes(tp, m.pd.f.esize);
      t.smRunOff = (int)((sub[2] - sub[1]) / 4);
      t.padShift = tp.padShift;
      t.padLog = tp.padLog;
      const int step = groupLoadStep(tp, rs, m.pd.f.esize);
      t.ldStepBytes = step < 0 ? -1 : step * m.pd.f.esize;
      const GroupStoreSteps st = groupStoreSteps(tp, rs, m.pd.f.esize);
      t.outStepBytes = st.outStep < 0 ? -1 : st.outStep * m.pd.f.esize;
      t.rowSmStep = st.rowSmStep;
      t.smStep = st.smStep;
      GroupTableJob jb;
      std::memset(&jb, 0, sizeof(jb));
      jb.tp = tp;
      jb.rs = rs;
      jb.ldRow = reinterpret_cast<int*>(tb + sub[0]);
      jb.outRows = reinterpret_cast<int2*>(tb + sub[1]);
      jb.smRun = reinterpret_cast<int*>(tb + sub[2]);
      jb.tiles = map + first;
      jb.tensor = (long long)k;
      first += tp.numTiles;
      std::memcpy(jobs + jobOf[i], &jb, sizeof(jb));
    }
  }
  // (a pageable source is consumed before cudaMemcpyAsync returns)
  cudaError_t err = cudaMemcpyAsync(base, host.data(), imageBytes, cudaMemcpyHostToDevice, g.stream);
  if (err == cudaSuccess && nJobs > 0)
    writeGroupTablesKernel<<<(unsigned)nJobs, 256, 0, g.stream>>>(
        reinterpret_cast<const GroupTableJob*>(base + jobsOff));
  if (err == cudaSuccess) err = cudaGetLastError();
  // a separately launched member's tables were written on its plan's stream
  for (const Member& m : g.members)
    if (err == cudaSuccess && m.separate && m.plan->stream != g.stream)
      err = cudaStreamSynchronize(m.plan->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(g.stream);
  if (err != cudaSuccess) return LIBRETT_INTERNAL_ERROR;

  // The graph: one node per bucket plus one per separate member, spread over
  // parallel branches, largest work first onto the least-loaded branch.
  struct Node {
    long long bytes;
    int bucket;  // >= 0: bucket index; < 0: separate member -bucket-1
  };
  std::vector<Node> nodes;
  for (int b = 0; b < (int)buckets.size(); ++b) nodes.push_back({buckets[b].bytes, b});
  for (int i = 0; i < (int)g.members.size(); ++i)
    if (g.members[i].separate)
      nodes.push_back({2 * g.members[i].pd.f.vol * (long long)g.members[i].pd.f.esize, -i - 1});
  std::stable_sort(nodes.begin(), nodes.end(),
                   [](const Node& a, const Node& b) { return a.bytes > b.bytes; });
  const int branches = std::max(1, std::min((int)nodes.size(), 8));
  std::vector<long long> load(branches, 0);
  cudaStream_t cap = nullptr;
  std::vector<cudaStream_t> side(branches, nullptr);
  std::vector<cudaEvent_t> ev(branches + 1, nullptr);
  bool ok = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess;
  for (int b = 0; ok && b < branches; ++b)
    ok = cudaStreamCreateWithFlags(&side[b], cudaStreamNonBlocking) == cudaSuccess;
  for (int b = 0; ok && b <= branches; ++b)
    ok = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) == cudaSuccess;
  if (ok) ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed) == cudaSuccess;
  if (ok) {
    bool launched = cudaEventRecord(ev[branches], cap) == cudaSuccess;
    for (int b = 0; launched && b < branches; ++b)
      launched = cudaStreamWaitEvent(side[b], ev[branches], 0) == cudaSuccess;
    for (const Node& nd : nodes) {
      if (!launched) break;
      const int br = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[br] += nd.bytes;
      if (nd.bucket >= 0) {
        const Bucket& b = buckets[nd.bucket];
        B.summary.push_back({b.es, b.lv, b.sv, b.nl, b.loads, (int)b.members.size(), b.smem,
                             (long long)b.tiles, b.bytes});
        launched = launchGroupBucket(b.es, b.lv, b.sv, b.nl, b.loads,
                                     reinterpret_cast<const GroupTensor*>(base + b.tensOff),
                                     reinterpret_cast<const GroupTile*>(base + b.mapOff), b.tiles,
                                     b.smem, side[br], g.numSMs) == cudaSuccess;
      } else {
        const Member& m = g.members[-nd.bucket - 1];
        int grid = 0;
        launched = launchPlan(m.plan->pd, &m.plan->tables, m.in, m.out, side[br], g.numSMs,
                              &grid) == cudaSuccess;
      }
    }
    for (int b = 0; b < branches; ++b) {
      cudaEventRecord(ev[b], side[b]);
      cudaStreamWaitEvent(cap, ev[b], 0);
    }
    cudaGraph_t graph = nullptr;
    const bool ended = cudaStreamEndCapture(cap, &graph) == cudaSuccess;
    ok = launched && ended && graph != nullptr;
    B.graph = graph;
    if (ok) ok = cudaGraphInstantiate(&B.exec, graph, 0) == cudaSuccess;
  }
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t s : side)
    if (s) cudaStreamDestroy(s);
  if (cap) cudaStreamDestroy(cap);
  if (!ok) {
    cudaGetLastError();
    return LIBRETT_INTERNAL_ERROR;
  }
  return LIBRETT_SUCCESS;
}

uint64_t batchSignature(const GroupObj& g) {
  uint64_t h = 1469598103934665603ULL;
  h = fnv(h, (uint64_t)g.numSMs);
  h = fnv(h, g.members.size());
  for (const Member& m : g.members) {
    const Fused& f = m.plan->pd.f;
    h = fnv(h, ((uint64_t)f.rank << 8) | ((uint64_t)f.esize << 2) | (m.aligned8 ? 2 : 0) |
                   (m.aligned16 ? 1 : 0));
    for (int r = 0; r < f.rank; ++r) h = fnv(h, ((uint64_t)f.dim[r] << 5) | (uint64_t)f.perm[r]);
  }
  return h;
}

// Members run concurrently (one bucket launch holds many; buckets run on
// parallel graph branches), so no member's output may overlap any member's
// input or output.  Sweep over the byte ranges sorted by start: a range
// overlaps an earlier one iff the largest end seen so far exceeds its
// start; inputs may overlap inputs.
bool independentBuffers(const GroupObj& g) {
  struct Range {
    uintptr_t lo, hi;
    bool out;
  };
  std::vector<Range> r;
  r.reserve(2 * g.members.size());
  for (const Member& m : g.members) {
    const uintptr_t n = (uintptr_t)(m.plan->pd.f.vol * m.plan->pd.f.esize);
    r.push_back({(uintptr_t)m.in, (uintptr_t)m.in + n, false});
    r.push_back({(uintptr_t)m.out, (uintptr_t)m.out + n, true});
  }
  std::sort(r.begin(), r.end(), [](const Range& a, const Range& b) { return a.lo < b.lo; });
  uintptr_t endAny = 0, endOut = 0;
  for (const Range& x : r) {
    if (x.out ? endAny > x.lo : endOut > x.lo) return false;
    endAny = std::max(endAny, x.hi);
    if (x.out) endOut = std::max(endOut, x.hi);
  }
  return true;
}

librettResult create(librettGroupHandle* handle, int count, const librettHandle* plans,
                     void* const* idata, void* const* odata, cudaStream_t stream,
                     const int* policy) {
  if (handle == nullptr || count < 1 || plans == nullptr || idata == nullptr || odata == nullptr)
    return LIBRETT_INVALID_PARAMETER;
  if (policy != nullptr)
    for (int c = 0; c < GROUP_CLASSES; ++c)
      if (policy[c] < 0 || policy[c] >= GP_COUNT) return LIBRETT_INVALID_PARAMETER;
  int dev = 0, sms = 0;
  auto g = std::make_shared<GroupObj>();
  if (!currentDevice(dev, sms, &g->devName)) return LIBRETT_INTERNAL_ERROR;
  g->stream = stream;
  g->device = dev;
  g->numSMs = sms;
  g->members.resize(count);
  for (int i = 0; i < count; ++i) {
    Member& m = g->members[i];
    m.plan = findPlan(plans[i]);
    if (!m.plan) return LIBRETT_INVALID_PLAN;
    if (m.plan->device != dev) return LIBRETT_INVALID_DEVICE;
    m.in = static_cast<const unsigned char*>(idata[i]);
    m.out = static_cast<unsigned char*>(odata[i]);
    const Fused& f = m.plan->pd.f;
    const uintptr_t a = f.esize < 16 ? f.esize : 16;
    if (m.in == nullptr || m.out == nullptr || (const void*)m.in == (const void*)m.out ||
        (uintptr_t)m.in % a || (uintptr_t)m.out % a)
      return LIBRETT_INVALID_PARAMETER;
    const long long bytes = f.vol * (long long)f.esize;
    g->bytes += 2 * bytes;
    m.cls = memberClass(bytes, f.esize);
    m.aligned16 = (uintptr_t)m.in % 16 == 0 && (uintptr_t)m.out % 16 == 0;
    m.aligned8 = (uintptr_t)m.in % 8 == 0 && (uintptr_t)m.out % 8 == 0;
  }
  if (!independentBuffers(*g)) return LIBRETT_INVALID_PARAMETER;
  g->signature = batchSignature(*g);
  // Untuned default: the largest tiles, loaded by cp.async (the fastest
  // uniform policy on the 10,000-tensor batch of rank 2..6, 2^10..2^22
  // elements, f32/f64).
  Policy pol;
  pol.fill(GP_WIDEST + GP_TILES);
  if (policy != nullptr) {
    std::copy(policy, policy + GROUP_CLASSES, pol.begin());
  } else {
    std::lock_guard<std::mutex> lk(gTuneMu);
    auto it = gTuneCache.find(g->signature);
    if (it != gTuneCache.end()) {
      pol = it->second;
      g->tuned = true;
    }
  }
  librettResult r = build(*g, pol);
  if (r != LIBRETT_SUCCESS) return r;
  librettGroupHandle h = gNextGroup.fetch_add(1);
  {
    std::lock_guard<std::mutex> lk(gGroupMu);
    gGroups[h] = g;
  }
  *handle = h;
  return LIBRETT_SUCCESS;
}

std::shared_ptr<GroupObj> findGroup(librettGroupHandle h) {
  std::lock_guard<std::mutex> lk(gGroupMu);
  auto it = gGroups.find(h);
  return it == gGroups.end() ? nullptr : it->second;
}

librettResult launch(GroupObj& g) {
  if (g.built.exec == nullptr || injectFault(FAULT_LAUNCH) ||
      cudaGraphLaunch(g.built.exec, g.stream) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  gLaunchCount.fetch_add((unsigned long long)g.built.buckets + g.built.separate,
                         std::memory_order_relaxed);
  return LIBRETT_SUCCESS;
}

librettResult execute(librettGroupHandle h) {
  std::shared_ptr<GroupObj> g = findGroup(h);
  if (!g) return LIBRETT_INVALID_PLAN;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  if (dev != g->device) return LIBRETT_INVALID_DEVICE;
  std::lock_guard<std::mutex> lk(g->mu);
  return launch(*g);
}

// Best of three timed executions after one untimed one (milliseconds).
bool timeBuild(GroupObj& g, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
  if (launch(g) != LIBRETT_SUCCESS) return false;
  float best = -1.f;
  for (int rep = 0; rep < 3; ++rep) {
    if (cudaEventRecord(e0, g.stream) != cudaSuccess || launch(g) != LIBRETT_SUCCESS ||
        cudaEventRecord(e1, g.stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
      return false;
    float t = 0.f;
    if (cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) return false;
    if (best < 0.f || t < best) best = t;
  }
  *ms = best;
  return true;
}

// Autotuner.  Phase 1 times every policy applied to all classes and keeps
// the fastest; phase 2 walks the classes that hold at least 2% of the
// group's bytes (most bytes first) and tries, for one class at a time,
// the other tile choices with the same loads and the other loads with the
// same tile, keeping a change that is at least 2% faster.  Times on the
// group's own buffers (reads the inputs, overwrites the outputs); the result
// is cached by batch signature.
librettResult tune(librettGroupHandle h) {
  std::shared_ptr<GroupObj> gp = findGroup(h);
  if (!gp) return LIBRETT_INVALID_PLAN;
  GroupObj& g = *gp;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  if (dev != g.device) return LIBRETT_INVALID_DEVICE;
  std::lock_guard<std::mutex> lk(g.mu);
  long long classBytes[GROUP_CLASSES] = {};
  for (const Member& m : g.members)
    classBytes[m.cls] += 2 * m.plan->pd.f.vol * (long long)m.plan->pd.f.esize;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return LIBRETT_INTERNAL_ERROR;
  }
  librettResult r = LIBRETT_SUCCESS;
  Policy cur = g.policy;
  float best = -1.f;
  auto trial = [&](const Policy& pol) {
    float t = 0.f;
    r = build(g, pol);
    if (r == LIBRETT_SUCCESS && !timeBuild(g, e0, e1, &t)) r = LIBRETT_INTERNAL_ERROR;
    return r == LIBRETT_SUCCESS ? t : -1.f;
  };
  for (int p = 0; p < GP_COUNT && r == LIBRETT_SUCCESS; ++p) {
    Policy pol;
    pol.fill(p);
    const float t = trial(pol);
    if (r == LIBRETT_SUCCESS && (best < 0.f || t < best)) {
      best = t;
      cur = pol;
    }
  }
  int order[GROUP_CLASSES];
  for (int c = 0; c < GROUP_CLASSES; ++c) order[c] = c;
  std::stable_sort(order, order + GROUP_CLASSES,
                   [&](int a, int b) { return classBytes[a] > classBytes[b]; });
  for (int oc = 0; oc < GROUP_CLASSES && r == LIBRETT_SUCCESS; ++oc) {
    const int c = order[oc];
    if (classBytes[c] * 50 < g.bytes) continue;
    const int tile = cur[c] % GP_TILES, loads = cur[c] / GP_TILES;
    std::vector<int> alts;
    for (int t = 0; t < GP_TILES; ++t)
      if (t != tile) alts.push_back(t + GP_TILES * loads);
    for (int l = 0; l < GP_COUNT / GP_TILES; ++l)
      if (l != loads) alts.push_back(tile + GP_TILES * l);
    for (int p : alts) {
      Policy pol = cur;
      pol[c] = p;
      const float t = trial(pol);
      if (r != LIBRETT_SUCCESS) break;
      if (t < 0.98f * best) {
        best = t;
        cur = pol;
      }
    }
  }
  if (r == LIBRETT_SUCCESS && g.policy != cur) r = build(g, cur);
  if (r != LIBRETT_SUCCESS && build(g, cur) != LIBRETT_SUCCESS) g.built = Build();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r != LIBRETT_SUCCESS) return r;
  g.tuned = true;
  std::lock_guard<std::mutex> tk(gTuneMu);
  gTuneCache[g.signature] = cur;
  return LIBRETT_SUCCESS;
}

librettResult destroy(librettGroupHandle h) {
  std::lock_guard<std::mutex> lk(gGroupMu);
  auto it = gGroups.find(h);
  if (it == gGroups.end()) return LIBRETT_INVALID_PLAN;
  gGroups.erase(it);
  return LIBRETT_SUCCESS;
}

}  // namespace
}  // namespace lt

librettResult librettGroupCreate(librettGroupHandle* group, int count, const librettHandle* plans,
                                 void* const* idata, void* const* odata,
                                 librett_gpuStream_t& stream) {
  return lt::create(group, count, plans, idata, odata, stream, nullptr);
}

librettResult librettGroupTune(librettGroupHandle group) { return lt::tune(group); }

librettResult librettGroupExecute(librettGroupHandle group) { return lt::execute(group); }

librettResult librettGroupDestroy(librettGroupHandle group) { return lt::destroy(group); }

librettResult librettExecuteGrouped(int count, const librettHandle* plans, void* const* idata,
                                    void* const* odata) {
  if (count < 1 || plans == nullptr) return LIBRETT_INVALID_PARAMETER;
  std::shared_ptr<lt::PlanObj> first = lt::findPlan(plans[0]);
  if (!first) return LIBRETT_INVALID_PLAN;
  librettGroupHandle g = 0;
  librettResult r = lt::create(&g, count, plans, idata, odata, first->stream, nullptr);
  if (r != LIBRETT_SUCCESS) return r;
  r = lt::execute(g);
  lt::destroy(g);
  return r;
}

extern "C" {

int librett_c_group_create(librettGroupHandle* group, int count, const librettHandle* plans,
                           void* const* idata, void* const* odata, void* stream) {
  return lt::create(group, count, plans, idata, odata, (cudaStream_t)stream, nullptr);
}

int librett_c_group_create_policy(librettGroupHandle* group, int count,
                                  const librettHandle* plans, void* const* idata,
                                  void* const* odata, void* stream, const int* policy) {
  if (policy == nullptr) return LIBRETT_INVALID_PARAMETER;
  return lt::create(group, count, plans, idata, odata, (cudaStream_t)stream, policy);
}

int librett_c_group_tune(librettGroupHandle group) { return librettGroupTune(group); }

int librett_c_group_execute(librettGroupHandle group) { return librettGroupExecute(group); }

int librett_c_group_destroy(librettGroupHandle group) { return librettGroupDestroy(group); }

int librett_c_execute_grouped(int count, const librettHandle* plans, void* const* idata,
                              void* const* odata) {
  return librettExecuteGrouped(count, plans, idata, odata);
}

int librett_c_execute_batch(int count, const librettHandle* plans, void* const* idata,
                            void* const* odata) {
  if (count < 0 || (count > 0 && (plans == nullptr || idata == nullptr || odata == nullptr)))
    return LIBRETT_INVALID_PARAMETER;
  for (int i = 0; i < count; ++i) {
    const librettResult r = librettExecute(plans[i], idata[i], odata[i]);
    if (r != LIBRETT_SUCCESS) return r;
  }
  return LIBRETT_SUCCESS;
}

int librett_c_group_info(librettGroupHandle group, int* members, int* buckets, int* separate,
                         long long* tiles, long long* bytes) {
  std::shared_ptr<lt::GroupObj> g = lt::findGroup(group);
  if (!g) return LIBRETT_INVALID_PLAN;
  std::lock_guard<std::mutex> lk(g->mu);
  if (members) *members = (int)g->members.size();
  if (buckets) *buckets = g->built.buckets;
  if (separate) *separate = g->built.separate;
  if (tiles) *tiles = g->built.tiles;
  if (bytes) *bytes = g->bytes;
  return LIBRETT_SUCCESS;
}

int librett_c_group_bucket(librettGroupHandle group, int index, int* shape, int* members,
                           long long* tiles, long long* bytes) {
  std::shared_ptr<lt::GroupObj> g = lt::findGroup(group);
  if (!g) return LIBRETT_INVALID_PLAN;
  std::lock_guard<std::mutex> lk(g->mu);
  if (index < 0 || index >= (int)g->built.summary.size()) return LIBRETT_INVALID_PARAMETER;
  const lt::BucketSummary& b = g->built.summary[index];
  if (shape) {
    shape[0] = b.es;
    shape[1] = b.lv;
    shape[2] = b.sv;
    shape[3] = b.nl;
    shape[4] = b.smem;
    shape[5] = b.loads;
  }
  if (members) *members = b.members;
  if (tiles) *tiles = b.tiles;
  if (bytes) *bytes = b.bytes;
  return LIBRETT_SUCCESS;
}

int librett_c_group_policy(librettGroupHandle group, int* policy, int* tuned) {
  std::shared_ptr<lt::GroupObj> g = lt::findGroup(group);
  if (!g) return LIBRETT_INVALID_PLAN;
  std::lock_guard<std::mutex> lk(g->mu);
  if (policy)
    for (int c = 0; c < lt::GROUP_CLASSES; ++c) policy[c] = g->policy[c];
  if (tuned) *tuned = g->tuned ? 1 : 0;
  return LIBRETT_SUCCESS;
}

}  // extern "C"
