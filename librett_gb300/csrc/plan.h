// Planner data structures shared by the host planner (plan.cpp), the kernels
// (kernels.cu) and the API layer (api.cpp).
//
// Vocabulary follows LibreTT (src/plan.h:53-118): Mm = ranks contiguous in the
// input, Mk = ranks contiguous in the output, Mbar = the remaining ranks that
// the kernels loop over.  Here a plan is described by one "tile": an extent
// e[r] per fused rank.  Ranks with e[r] > 1 are tile ranks (the Mm u Mk
// sub-volume one CTA moves through shared memory); ranks with more than one
// chunk are grid ranks (LibreTT's Mbar, plus the split rank of PackedSplit).
#pragma once

#include <cstdint>
#include <vector>

namespace lt {

constexpr int MAXR = 16;            // maximum (fused) rank
constexpr int TILE_THREADS = 256;   // threads per CTA of the tile kernel
constexpr int TILE_MAX_SLOTS = 16;  // elements per thread per tile (max)
constexpr int TILE_MAX_VOL = TILE_THREADS * TILE_MAX_SLOTS;
constexpr int ROW_THREADS = 256;
constexpr int COPY_THREADS = 256;
constexpr int PAD_NONE = 31;
constexpr int TILE_STAGES = 3;     // cp.async pipeline depth of the tile kernel

// Tile pipelines: register-staged loads (2 shared buffers) or cp.async
// straight into a TILE_STAGES-deep ring of shared buffers.
enum Pipe { PIPE_REG = 0, PIPE_ASYNC = 1, PIPE_FLAT = 2, PIPE_BULK = 3 };
// PIPE_FLAT: one tile per CTA (no persistent loop); the offset tables are
// built at plan time and read from device memory.
// PIPE_BULK: the flat pipeline with its loads as bulk copies: each
// contiguous segment of the tile's input (an input run, or the part of it
// between two padding gaps) is one cp.async.bulk into shared memory, all
// completing on one mbarrier; 16-byte load units only.
inline bool flatTables(int pipe) { return pipe == PIPE_FLAT || pipe == PIPE_BULK; }

// Transpose methods, numbered as LibreTT's enum (src/plan.h:54-56).
enum Method { Unknown = 0, Trivial = 1, Packed = 2, PackedSplit = 3, Tiled = 4, TiledCopy = 5 };

// Kernel families.
enum Kernel { K_NONE = 0, K_COPY = 1, K_ROW = 2, K_TILE = 3 };

// Division by an invariant 32-bit divisor for numerators n < 2^31, by the
// round-up multiply-and-shift method of Granlund and Montgomery ("Division by
// invariant integers using multiplication", PLDI 1994, Thm 4.2):
//   l = ceil(log2 d), m = floor(2^(31+l) / d) + 1, q = (n * m) >> (31 + l).
// Then 2^(31+l) < m*d <= 2^(31+l) + 2^l, which makes q exact for n < 2^31,
// and m < 2^32 for every 1 <= d <= 2^31.
struct FastDiv {
  uint32_t d;
  uint32_t mul;
  uint32_t shift;
};

inline FastDiv makeFastDiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  uint64_t m = ((1ull << (31 + l)) / d) + 1;
  f.mul = (uint32_t)m;
  f.shift = 31 + l;
  return f;
}

inline uint32_t fastDivHost(uint32_t n, const FastDiv& f) {
  return (uint32_t)(((uint64_t)n * f.mul) >> f.shift);
}

// Division of in-tile indices (n < 2^16) by run lengths (1 <= d < 2^16)
// with one multiply-high and no shift: mul = floor((2^32 - 1) / d) and
// n / d == umulhi(n + 1, mul).  Proof: r = 2^32 - mul * d lies in [1, d], so
// (n + 1) * mul / 2^32 = (n + 1) / d - (n + 1) * r / (d * 2^32); with
// n = q * d + t the second term is positive and at most 1 / d whenever
// (n + 1) * d <= 2^32, so the floor is q for every t in [0, d).  Kernels
// carry n + 1 instead of n, which folds the increment into the multiply-add
// that forms the index.
struct RunDiv {
  uint32_t d;
  uint32_t mul;
};

inline RunDiv makeRunDiv(uint32_t d) { return RunDiv{d, 0xFFFFFFFFu / d}; }

// n / d for n + 1 = n1; exact while n1 * d <= 2^32.
inline uint32_t runDivHost(uint32_t n1, const RunDiv& f) {
  return (uint32_t)(((uint64_t)n1 * f.mul) >> 32);
}

// Problem after dropping unit dims and fusing ranks that stay adjacent under
// the permutation (the role of LibreTT's reduceRanks, src/plan.cpp:64-127).
struct Fused {
  int rank;           // fused rank (>= 1)
  int esize;          // element bytes (4, 8, 16)
  int64_t vol;        // elements
  int64_t dim[MAXR];  // input order
  int perm[MAXR];     // output rank i is input rank perm[i]
  int64_t sin[MAXR];  // input stride of input rank r (elements)
  int64_t sout[MAXR]; // output stride of input rank r (elements)
};

// Tiles of at most this many ranks address their units arithmetically in
// the flat and bulk-copy kernels (no offset tables).
constexpr int ARITH_MAX_NTR = 6;

struct TileParams;
inline int arithRanks(const TileParams& tp);

// Tile-kernel parameters (passed by value as a __grid_constant__ argument).
struct TileParams {
  uint32_t numTiles;
  int tileVol;          // elements in a full tile
  int lv;               // elements per load unit (16-byte units when > 1)
  int sv;               // elements per store unit
  int padLog;           // log2(lv): padding comes in whole load units
  int nIn;              // load units per tile (tileVol / lv)
  int nOut;             // store units per tile (tileVol / sv)
  int nTR;              // tile ranks (extent > 1), input order
  int nGR;              // grid ranks (more than one chunk), decode order
  int padShift;         // smem index = j + ((j >> padShift) << padLog); PAD_NONE = none
  int smStride;         // elements per smem buffer including padding
  int nRagged;          // grid ranks whose dim is not a multiple of the extent
  int bankWavefronts;   // planner only: simulated wavefronts at padShift
  int screened;         // planner only: built without the padding search
  int segLen;           // PIPE_BULK: elements per bulk copy (a multiple of lv)
  int testExtraTx;      // PIPE_BULK, test hook only: bytes armed on the mbarrier beyond
                        // the tile's (0; nonzero makes the bounded wait run out)
  uint32_t statusTag;   // PIPE_BULK: nonzero tag of the plan, written to its status
                        // word by a launch whose copies did not arrive in time
  int trE[MAXR];        // extent of tile rank t
  int trInTile[MAXR];   // in-tile input-order stride of tile rank t
  int trSin[MAXR];      // global input stride of tile rank t (elements)
  int trSout[MAXR];     // global output stride of tile rank t (elements)
  int trOut[MAXR];      // tile ranks in output order (indices into tr*)
  // Table-free addressing (tiles of at most ARITH_MAX_NTR ranks): digit t of
  // an in-tile index x (< 2^16) is __umulhi(x, trMul[t]) with trMul[t] =
  // ceil(2^32 / trE[t]) (extents are at least 2); to* are the same fields
  // for the tile ranks in output order (to*[i] = tr*[trOut[i]]).
  uint32_t trMul[MAXR];
  int toE[MAXR];
  uint32_t toMul[MAXR];
  int toSout[MAXR];
  int toInTile[MAXR];
  int storeStraddle;    // a store unit's elements may cross output tile rank 0
  // Grid rank g has grDiv[g].d chunks; chunk c starts at c * extent, except
  // that the last chunk starts at dim - extent, so that every tile is full
  // (a ragged last chunk overlaps its neighbour; the overlap is written
  // twice with identical bits).
  FastDiv grDiv[MAXR];    // number of chunks of grid rank g
  long long grSin[MAXR];  // input step of one chunk of grid rank g
  long long grSout[MAXR]; // output step of one chunk of grid rank g
  long long grLastIn[MAXR];   // input offset of the last chunk
  long long grLastOut[MAXR];  // output offset of the last chunk
};

// Rank count the flat and bulk-copy kernels address arithmetically (the
// template argument NTR), 0 when the tile needs its offset tables.
inline int arithRanks(const TileParams& tp) {
  return tp.nTR >= 1 && tp.nTR <= ARITH_MAX_NTR ? tp.nTR : 0;
}

// Row-copy parameters (TiledCopy: input rank 0 is also output rank 0).
struct RowParams {
  uint32_t numRows;
  uint32_t numItems;    // numRows * chunks of 32 units (< 2^31)
  FastDiv chunkDiv;     // chunks of 32 units per row
  int rowUnits;         // units per row
  int nR;               // row ranks, decode order (output order)
  FastDiv rDiv[MAXR];
  long long rSin[MAXR]; // input stride per row-rank step (units)
  long long rSout[MAXR];
};

struct CopyParams {
  long long numUnits;
};

// A complete plan: what to launch and with what parameters.
struct PlanDesc {
  int method = Unknown;
  int kernel = K_NONE;
  Fused f{};
  int64_t extent[MAXR]{};  // tile extent per fused rank (input order)
  int threads = 0;
  int slots = 0;           // tile: load units per thread per tile (template NL)
  int ragged = 0;          // tile: has ragged ranks
  int smemBytes = 0;       // dynamic smem per CTA
  int unitBytes = 0;       // row/copy: preferred unit (16 when the layout allows)
  int runInBytes = 0, runOutBytes = 0;
  int padShift = PAD_NONE;
  int pipe = PIPE_REG;     // tile: Pipe
  long long numWork = 0;   // tiles / rows / units
  double cost = 0.0;       // analytic estimate, seconds at nominal bandwidth
  int candidate = 0;
  int numCandidates = 0;
  int targetRunBytes = 0, maxTileBytes = 0;  // knobs that produced the tile
  bool screened = false;   // tile built without the padding search (refineCandidate)
  // model statistics (also features of the learned selector)
  double effIn = 1.0, effOut = 1.0;  // useful bytes / DRAM sector bytes per side
  double overlap = 1.0;              // elements moved / volume (shifted chunks)
  double bankPerUnit = 0.0;          // shared wavefronts per 32 sampled accesses
                                     // (-1: not simulated yet, bankPerUnitOf)
  int ctasPerSM = 0;                 // modelled occupancy
  TileParams tile{};
  TileParams tileScalar{}; // element-size units (misaligned pointers)
  int slotsScalar = 0, smemBytesScalar = 0;
  int unitOutBytes = 0;    // tile: store unit bytes
  RowParams row{};         // with unitBytes units
  RowParams rowScalar{};   // with esize units (misaligned pointers)
  CopyParams copy{};
};

// Input validation with LibreTT's rules (src/librett.cpp:85-108) plus the
// engine's limits (rank <= MAXR, volume <= 2^40).  Returns 0 or 2
// (LIBRETT_INVALID_PARAMETER).
int checkInput(int rank, const int* dim, const int* perm, size_t sizeofType);

// Drop unit dims, fuse adjacent ranks, compute strides.
void fuseRanks(int rank, const int* dim, const int* perm, int esize, Fused& f);

// Candidate plans for a fused problem on a device with numSMs SMs.  The
// first entry is never empty.  Each candidate's `cost` is filled in.  By
// default tile candidates use the one-tile-per-CTA pipeline, with per-unit
// (PIPE_FLAT) and bulk-copy (PIPE_BULK) loads; setAllPipelines(true) or
// LIBRETT_ALL_PIPELINES=1 adds the persistent register-staged and cp.async
// variants.
//
// screen: build tile candidates without the shared-memory padding search
// (padding off, bank wavefronts of the unpadded tile), the form the plan
// selectors rank; refineCandidate() then completes the chosen one, giving
// exactly the candidate a full enumeration would have built.
std::vector<PlanDesc> enumerateCandidates(const Fused& f, int numSMs, bool screen = false);
bool refineCandidate(PlanDesc& pd, int numSMs);

// Shared-memory wavefronts per 32 sampled accesses of a candidate's tile
// (pd.bankPerUnit, a selector feature): screened candidates leave the bank
// simulation out (bankPerUnit -1) until a selector asks for it here.
double bankPerUnitOf(const PlanDesc& pd);
// The same, stored in pd (pd.bankPerUnit, pd.tile.bankWavefronts).
void simulateBanks(PlanDesc& pd);

// Grouped execution, 4-byte elements: rebuilds the tile of pd (same
// extents, flat pipeline) with 8-byte units on the sides whose layout does
// not allow 16-byte units (or both sides when the pointers are 8- but not
// 16-byte aligned: aligned16 false).  False, pd unchanged, when no side
// gains.  The grouped kernel is instantiated for 4-, 8- and 16-byte units of
// 4-byte elements; single plans use 4- or 16-byte units only.
bool widenUnits8(PlanDesc& pd, bool aligned16);
// Grouped execution: a tile whose runs take wider units than pd's, made by
// rounding one rank's extent down or up to a multiple of 2 .. 16 / esize
// elements (the last tile of a rank is shifted back to end at its dim, so
// an extent need not divide it), with 3/4 to 5/4 of pd's volume.  Units are
// the grouped kernel's (with 8-byte units for 4-byte elements when eight),
// ranked by the narrower side, then the sum, then the volume.  False, pd
// unchanged, when no rounding gives wider units.
bool widenUnitsByExtents(PlanDesc& pd, int numSMs, bool eight);
// Largest tile of grouped execution (elements): 32 KB of 4-byte elements.
constexpr int GROUP_MAX_VOL = 2 * TILE_MAX_VOL;
// Grouped execution: for a tile whose load units hold at least 2 elements, a
// tile with one rank's extent doubled (at most its dim), up to GROUP_MAX_VOL
// elements and 16 load units per thread, that keeps pd's units and at least
// 95 % of its sector efficiency; the best efficiency, then the largest
// volume.  False, pd unchanged, when none.
bool groupDoubleTile(PlanDesc& pd, int numSMs);
void setAllPipelines(bool all);
bool allPipelines();

// Tile candidates in the one-tile-per-CTA pipeline only, for any fused
// problem (a fused rank-1 copy becomes a one-rank tile); used where every
// member of a batch must run in that pipeline (grouped execution).
std::vector<PlanDesc> flatTileCandidates(const Fused& f, int numSMs, bool screen = false);

// Pipelines a tile enumeration builds candidates for (bits 1 << Pipe): the
// default set is the one-tile-per-CTA pipeline with per-unit and bulk-copy
// loads; grouped execution uses the first only.
enum PipeSet {
  PIPES_FLAT = 1 << PIPE_FLAT,
  PIPES_DEFAULT = (1 << PIPE_FLAT) | (1 << PIPE_BULK),
  PIPES_ALL = (1 << PIPE_REG) | (1 << PIPE_ASYNC) | (1 << PIPE_FLAT) | (1 << PIPE_BULK)
};
void appendTileCandidates(const Fused& f, int numSMs, int pipes, std::vector<PlanDesc>& out,
                          bool screen = false);

// Index of the candidate the analytic model prefers.
int chooseHeuristic(const std::vector<PlanDesc>& cands);

// Completes a chosen candidate for activation (the element-unit twin of a
// tile plan, used when pointers are not 16-byte aligned).  False if the
// twin does not fit.
bool finalizePlan(PlanDesc& pd);

// Offset tables of a tile (the layout the tile kernels use, see
// tile_kernel.cuh): ldOff[nIn], stOff[nOut], stSm[tileVol].
void tileTablesHost(const TileParams& tp, int* ldOff, int* stOff, unsigned short* stSm);

// Run split of a tile (grouped execution).  The tile's elements in input
// order form contiguous input runs of inRun elements (the leading tile ranks
// whose input strides continue the previous ranks' extents), and in output
// order contiguous output runs of outRun elements; a unit's offsets are then
// a per-run table entry plus its position inside the run.
struct GroupRunSplit {
  int inRun, outRun;  // elements per input / output run
  int kIn, kOut;      // tile ranks (input / output order) inside one run
};
GroupRunSplit groupRunSplit(const TileParams& tp);

// Step s with ldRow[r] == r * s for every input run r of the tile (the tile
// ranks after the run chain: each non-unit rank's input stride is the
// previous one's extent times its stride), so a kernel can form the run's
// offset without the table; -1 when the runs are not evenly spaced or
// s * esize does not fit an int.
int groupLoadStep(const TileParams& tp, const GroupRunSplit& rs, int esize);

// Elements per bulk copy of a tile in the bulk-copy pipeline at a given
// padding: the input run when a padding block holds whole runs (or there is
// no padding), the padding block when a run holds whole blocks, else 0.
int bulkSegment(const TileParams& tp, int padShift);

// Steps of the store-side run tables where their entries are evenly spaced
// (the same chain rule over the tile ranks in output order): output run r
// starts r * outStep elements from the tile's output corner, at in-tile
// index r * rowSmStep; position a of an output run holds in-tile index
// a * smStep.  outStep = -1 (rows) or smStep = -1 (positions) where the
// table is not evenly spaced, or outStep * esize does not fit an int.
struct GroupStoreSteps {
  int outStep = -1, rowSmStep = 0, smStep = -1;
};
GroupStoreSteps groupStoreSteps(const TileParams& tp, const GroupRunSplit& rs, int esize);

// Host copy of the run tables: ldRow[tileVol / inRun] input offset of each
// input run; stRow / smRow[tileVol / outRun] output offset and in-tile
// (input-order) index of each output run's first element; smRun[outRun]
// in-tile index of each element of an output run relative to its first.
void groupRunTablesHost(const TileParams& tp, const GroupRunSplit& rs, int* ldRow, int* stRow,
                        int* smRow, int* smRun);

// Shared-memory bank wavefronts of the first sampleUnits load and store
// units of a tile for a given padding.
long long smemWavefronts(const TileParams& tp, int esize, int padShift, int sampleUnits);

}  // namespace lt
