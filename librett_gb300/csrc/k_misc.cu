// Copy and row-copy launches, occupancy cache, and the launch dispatcher
// (the role of LibreTT's librettKernel switch, src/kernel.cpp:1008-1215).
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "fault.h"
#include "kernels.cuh"

namespace lt {

std::atomic<unsigned long long> gLaunchCount{0};

namespace {
std::atomic<long long> gFaultAfter[FAULT_SITES] = {{-1}, {-1}, {-1}};
std::atomic<long long> gArenaSlabBytes{0}, gArenaBlocks{0}, gArenaPoolBytes{0};
}  // namespace

bool injectFault(int site) {
  std::atomic<long long>& a = gFaultAfter[site];
  long long v = a.load(std::memory_order_relaxed);
  while (v >= 0) {
    if (a.compare_exchange_weak(v, v - 1, std::memory_order_relaxed)) return v == 0;
  }
  return false;
}

bool armFault(int site, long long after) {
  if (site < 0 || site >= FAULT_SITES) return false;
  gFaultAfter[site].store(after < 0 ? -1 : after, std::memory_order_relaxed);
  return true;
}

void tableArenaStats(long long* slabBytes, long long* blocks, long long* poolBytes) {
  if (slabBytes) *slabBytes = gArenaSlabBytes.load();
  if (blocks) *blocks = gArenaBlocks.load();
  if (poolBytes) *poolBytes = gArenaPoolBytes.load();
}

int cachedOccupancy(const void* func, int threads, int smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  auto key = std::make_tuple(dev, func, smem);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  if (smem > 48 * 1024) {
    // the opt-in limit covers static and dynamic shared memory together
    // (the bulk-copy kernel holds its mbarrier in static shared memory)
    int maxOptin = 0;
    cudaDeviceGetAttribute(&maxOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, func) != cudaSuccess) return 0;
    const int maxDynamic = maxOptin - (int)fa.sharedSizeBytes;
    if (smem > maxDynamic) return 0;
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, maxDynamic) !=
        cudaSuccess)
      return 0;
  }
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, func, threads, smem) != cudaSuccess)
    return 0;
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = occ;
  return occ;
}

namespace {

template <int US>
cudaError_t launchCopy(const void* in, void* out, long long n, cudaStream_t s, int* grid) {
  using T = typename Word<US>::T;
  const long long per = (long long)COPY_THREADS * COPY_UNROLL;
  const long long g = (n + per - 1) / per;
  if (g < 1 || g > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  *grid = (int)g;
  copyKernel<US><<<(unsigned)g, COPY_THREADS, 0, s>>>((const T*)in, (T*)out, n);
  return cudaGetLastError();
}

template <int US>
cudaError_t launchRows(const RowParams& rp, const void* in, void* out, cudaStream_t s, int* grid) {
  using T = typename Word<US>::T;
  const long long g = ((long long)rp.numItems + ROW_ITEMS_PER_CTA - 1) / ROW_ITEMS_PER_CTA;
  if (g < 1) return cudaErrorInvalidConfiguration;
  *grid = (int)g;
  rowCopyKernel<US><<<(unsigned)g, ROW_THREADS, 0, s>>>(rp, (const T*)in, (T*)out);
  return cudaGetLastError();
}

cudaError_t launchCopyUnit(int unit, const void* in, void* out, long long n, cudaStream_t s,
                           int* grid) {
  switch (unit) {
    case 4: return launchCopy<4>(in, out, n, s, grid);
    case 8: return launchCopy<8>(in, out, n, s, grid);
    case 16: return launchCopy<16>(in, out, n, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launchRowsUnit(int unit, const RowParams& rp, const void* in, void* out,
                           cudaStream_t s, int* grid) {
  switch (unit) {
    case 4: return launchRows<4>(rp, in, out, s, grid);
    case 8: return launchRows<8>(rp, in, out, s, grid);
    case 16: return launchRows<16>(rp, in, out, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// The tile fields the table writer needs (about a third of TileParams, so
// the launch carries a small parameter block).
struct TableParams {
  int tileVol, lv, sv, nIn, nTR, padShift, padLog;
  int trE[MAXR], trInTile[MAXR], trSin[MAXR], trSout[MAXR], trOut[MAXR];
};

__global__ void __launch_bounds__(256)
writeTileTablesKernel(const __grid_constant__ TableParams p, int* ldOff, int* stOff,
                      unsigned short* stSm) {
  const int stride = gridDim.x * blockDim.x;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < p.nIn; u += stride) {
    int rem = u * p.lv, off = 0;
    for (int t = 0; t < p.nTR; ++t) {
      const int e = p.trE[t];
      const int q = rem / e;
      off += (rem - q * e) * p.trSin[t];
      rem = q;
    }
    ldOff[u] = off;
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.tileVol; q += stride) {
    int rem = q, off = 0, jj = 0;
    for (int i = 0; i < p.nTR; ++i) {
      const int t = p.trOut[i];
      const int e = p.trE[t];
      const int d = rem / e;
      const int c = rem - d * e;
      rem = d;
      off += c * p.trSout[t];
      jj += c * p.trInTile[t];
    }
    stSm[q] = (unsigned short)(jj + ((jj >> p.padShift) << p.padLog));
    if (q % p.sv == 0) stOff[q / p.sv] = off;
  }
}

size_t deviceTableBytes(const TileParams& tp, size_t* stOffset, size_t* smOffset) {
  // stSm is read 4 or 8 bytes at a time by the store gathers: keep it
  // 16-byte aligned
  *stOffset = 4 * (size_t)tp.nIn;
  *smOffset = ((4 * (size_t)(tp.nIn + tp.nOut) + 15) / 16) * 16;
  return ((*smOffset + 2 * (size_t)tp.tileVol + 15) / 16) * 16;
}

cudaError_t writeDeviceTables(const TileParams& tp, unsigned char* base, cudaStream_t s,
                              DeviceTables* dt) {
  size_t stOffset, smOffset;
  deviceTableBytes(tp, &stOffset, &smOffset);
  int* ld = reinterpret_cast<int*>(base);
  int* st = reinterpret_cast<int*>(base + stOffset);
  unsigned short* sm = reinterpret_cast<unsigned short*>(base + smOffset);
  TableParams p;
  p.tileVol = tp.tileVol;
  p.lv = tp.lv;
  p.sv = tp.sv;
  p.nIn = tp.nIn;
  p.nTR = tp.nTR;
  p.padShift = tp.padShift;
  p.padLog = tp.padLog;
  for (int t = 0; t < MAXR; ++t) {
    p.trE[t] = tp.trE[t];
    p.trInTile[t] = tp.trInTile[t];
    p.trSin[t] = tp.trSin[t];
    p.trSout[t] = tp.trSout[t];
    p.trOut[t] = tp.trOut[t];
  }
  writeTileTablesKernel<<<(tp.tileVol + 255) / 256, 256, 0, s>>>(p, ld, st, sm);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  dt->ldOff = ld;
  dt->stOff = st;
  dt->stSm = sm;
  return cudaSuccess;
}

namespace {

// Status words of bulk-copy plans (zero at module load; only launches that
// time out write to them, each with its plan's tag).
__device__ unsigned gBulkStatus[BULK_STATUS_SLOTS];

constexpr int kMaxDevices = 64;
std::atomic<unsigned*> gBulkStatusBase[kMaxDevices];
std::atomic<uint32_t> gStatusTag{0};

}  // namespace

uint32_t nextStatusTag() {
  uint32_t t;
  do {
    t = gStatusTag.fetch_add(1, std::memory_order_relaxed) + 1;
  } while (t == 0);
  return t;
}

// The array's device address is resolved once per device (the host-side
// symbol is only a stand-in) and kept for the life of the process; like the
// table arena it is not supported across a cudaDeviceReset.
cudaError_t bulkStatusWord(uint32_t tag, unsigned** word) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  unsigned* base = gBulkStatusBase[dev].load(std::memory_order_acquire);
  if (base == nullptr) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, gBulkStatus);
    if (err != cudaSuccess) return err;
    base = static_cast<unsigned*>(p);
    gBulkStatusBase[dev].store(base, std::memory_order_release);
  }
  *word = base + (tag % BULK_STATUS_SLOTS);
  return cudaSuccess;
}

// Plan tables come from a memory pool of the library's own per device, which
// keeps up to TABLE_POOL_KEEP bytes of freed blocks for reuse instead of
// returning them to the device at every synchronisation (what the default
// pool does), so creating a plan does not map fresh memory each time.  The
// pools live until the process exits.
constexpr uint64_t TABLE_POOL_KEEP = 256ull << 20;

cudaError_t tablePool(cudaMemPool_t* pool) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) {
    *pool = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t p = nullptr;
  err = cudaMemPoolCreate(&p, &props);
  if (err != cudaSuccess) return err;
  uint64_t keep = TABLE_POOL_KEEP;
  err = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
  if (err != cudaSuccess) {
    cudaMemPoolDestroy(p);
    return err;
  }
  pools[dev] = p;
  *pool = p;
  return cudaSuccess;
}

// Plan tables come from a host-side suballocator, so that planning makes no
// device allocation call (a stream-ordered pool allocation costs about as
// much as the table-writing launch itself).  Per device, blocks of
// 4 KiB << c bytes (c < TABLE_CLASSES) are carved from 8 MiB slabs
// (cudaMalloc, kept until the process exits); larger tables come from the
// pool above.  Reuse is stream-ordered, as with cudaFreeAsync: a free
// records the block's event on the plan's stream; a plan on the same stream
// takes the block as it is (stream order puts its table writes after every
// kernel that read the old tables), a plan on another stream makes its
// stream wait for that event first.  Blocks freed on the requesting stream
// are preferred, then unused slab space, so the wait is only paid when there
// are neither.  A block freed while its stream is being captured leaves
// circulation; a stream being captured takes no other stream's block.
constexpr int TABLE_CLASSES = 9;  // 4 KiB .. 1 MiB
constexpr size_t TABLE_SLAB = 8u << 20;

struct TableBlock {
  void* p = nullptr;
  int device = 0;
  int cls = -1;                   // -1: from the pool
  cudaStream_t stream = nullptr;  // while free: the stream it was freed on
  cudaEvent_t freed = nullptr;    // recorded there at the free
};

struct TableArena {
  std::mutex mu;
  std::unordered_map<void*, TableBlock*> blocks;  // handed out or free
  struct Dev {
    std::vector<TableBlock*> freeBlocks[TABLE_CLASSES];
    char* cur = nullptr;
    size_t left = 0;
  };
  std::map<int, Dev> devs;
};

TableArena& tableArena() {
  static TableArena* a = new TableArena();  // lives until the process exits
  return *a;
}

cudaError_t tableAlloc(size_t bytes, cudaStream_t s, void** out) {
  *out = nullptr;
  if (injectFault(FAULT_TABLE_ALLOC)) return cudaErrorMemoryAllocation;
  gArenaBlocks.fetch_add(1, std::memory_order_relaxed);
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  int c = 0;
  while (c < TABLE_CLASSES && (size_t(4096) << c) < bytes) ++c;
  TableArena& A = tableArena();
  if (c == TABLE_CLASSES) {
    cudaMemPool_t pool = nullptr;
    err = tablePool(&pool);
    if (err == cudaSuccess) err = cudaMallocFromPoolAsync(out, bytes, pool, s);
    if (err != cudaSuccess) return err;
    gArenaPoolBytes.fetch_add((long long)bytes, std::memory_order_relaxed);
    TableBlock* b = new TableBlock();
    b->p = *out;
    b->device = dev;
    std::lock_guard<std::mutex> lk(A.mu);
    A.blocks[b->p] = b;
    return cudaSuccess;
  }
  const size_t size = size_t(4096) << c;
  // a captured stream cannot wait on an event recorded outside the capture
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const bool canWait =
      cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone;
  for (;;) {
    TableBlock* other = nullptr;
    {
      std::lock_guard<std::mutex> lk(A.mu);
      TableArena::Dev& D = A.devs[dev];
      std::vector<TableBlock*>& fl = D.freeBlocks[c];
      for (size_t i = fl.size(); i-- > 0;) {
        if (fl[i]->stream != s) continue;
        TableBlock* b = fl[i];
        fl.erase(fl.begin() + (std::ptrdiff_t)i);
        *out = b->p;
        return cudaSuccess;
      }
      if (D.left >= size) {
        TableBlock* b = new TableBlock();
        b->p = D.cur;
        b->device = dev;
        b->cls = c;
        D.cur += size;
        D.left -= size;
        A.blocks[b->p] = b;
        *out = b->p;
        return cudaSuccess;
      }
      if (canWait && !fl.empty()) {
        other = fl.front();  // the longest-freed block of another stream
        fl.erase(fl.begin());
      }
    }
    if (other != nullptr) {
      err = cudaStreamWaitEvent(s, other->freed, 0);
      if (err == cudaSuccess) {
        *out = other->p;
        return cudaSuccess;
      }
      std::lock_guard<std::mutex> lk(A.mu);  // not usable from s: back to the list
      A.devs[dev].freeBlocks[c].push_back(other);
      return err;
    }
    // a new slab (outside the lock: cudaMalloc may wait for the device)
    void* slab = nullptr;
    err = cudaMalloc(&slab, TABLE_SLAB);
    if (err != cudaSuccess) return err;
    gArenaSlabBytes.fetch_add((long long)TABLE_SLAB, std::memory_order_relaxed);
    std::lock_guard<std::mutex> lk(A.mu);
    TableArena::Dev& D = A.devs[dev];
    D.cur = static_cast<char*>(slab);
    D.left = TABLE_SLAB;
  }
}

void tableFree(void* p, cudaStream_t s) {
  if (p == nullptr) return;
  TableArena& A = tableArena();
  TableBlock* b = nullptr;
  {
    std::lock_guard<std::mutex> lk(A.mu);
    auto it = A.blocks.find(p);
    if (it == A.blocks.end()) return;
    b = it->second;
    if (b->cls < 0) A.blocks.erase(it);
  }
  if (b->cls < 0) {
    delete b;
    cudaFreeAsync(p, s);
    return;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone ||
      (b->freed == nullptr &&
       cudaEventCreateWithFlags(&b->freed, cudaEventDisableTiming) != cudaSuccess) ||
      cudaEventRecord(b->freed, s) != cudaSuccess) {
    std::lock_guard<std::mutex> lk(A.mu);
    A.blocks.erase(p);  // leaves circulation
    return;
  }
  b->stream = s;
  std::lock_guard<std::mutex> lk(A.mu);
  A.devs[b->device].freeBlocks[b->cls].push_back(b);
}

cudaError_t createDeviceTables(const PlanDesc& pd, cudaStream_t s, void** alloc, DeviceTables* dt) {
  *alloc = nullptr;
  *dt = DeviceTables();
  if (pd.kernel != K_TILE || !flatTables(pd.pipe)) return cudaSuccess;
  if (pd.pipe == PIPE_BULK) {
    if (pd.tile.statusTag == 0) return cudaErrorInvalidValue;
    cudaError_t err = bulkStatusWord(pd.tile.statusTag, &dt->status);
    if (err != cudaSuccess) return err;
  }
  if (!needsDeviceTables(pd)) return cudaSuccess;  // table-free addressing
  size_t stOffset, smOffset;
  const size_t total = deviceTableBytes(pd.tile, &stOffset, &smOffset);
  void* d = nullptr;
  cudaError_t err = tableAlloc(total, s, &d);
  if (err != cudaSuccess) return err;
  // the tables are computed on the device, in stream order before any use
  err = writeDeviceTables(pd.tile, static_cast<unsigned char*>(d), s, dt);
  if (err != cudaSuccess) {
    tableFree(d, s);
    *dt = DeviceTables();
    return err;
  }
  *alloc = d;
  return cudaSuccess;
}

void destroyDeviceTables(void* alloc, cudaStream_t s) { tableFree(alloc, s); }

cudaError_t launchPlan(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                       cudaStream_t s, int numSMs, int* grid) {
  if (injectFault(FAULT_LAUNCH)) return cudaErrorLaunchFailure;
  const uintptr_t align = (uintptr_t)in | (uintptr_t)out;
  int g = 0;
  cudaError_t err = cudaErrorInvalidValue;
  switch (pd.kernel) {
    case K_COPY: {
      int unit = (align % pd.unitBytes == 0) ? pd.unitBytes : pd.f.esize;
      long long n = pd.f.vol * pd.f.esize / unit;
      err = launchCopyUnit(unit, in, out, n, s, &g);
      break;
    }
    case K_ROW: {
      bool vec = align % pd.unitBytes == 0;
      err = launchRowsUnit(vec ? pd.unitBytes : pd.f.esize, vec ? pd.row : pd.rowScalar, in, out,
                           s, &g);
      break;
    }
    case K_TILE: {
      const PlanDesc* use = &pd;
      PlanDesc scalar;
      if ((pd.tile.lv > 1 || pd.tile.sv > 1) && align % 16 != 0) {
        // 16-byte units need 16-byte aligned tensors; fall back to element
        // units and the persistent pipeline, which builds its own tables
        if (pd.tileScalar.tileVol == 0) return cudaErrorInvalidValue;  // not finalized
        scalar = pd;
        scalar.tile = pd.tileScalar;
        scalar.slots = pd.slotsScalar;
        scalar.smemBytes = pd.smemBytesScalar;
        scalar.pipe = PIPE_REG;
        use = &scalar;
      }
      switch (pd.f.esize) {
        case 4: err = launchTile4(*use, dt, in, out, s, numSMs, &g); break;
        case 8: err = launchTile8(*use, dt, in, out, s, numSMs, &g); break;
        case 16: err = launchTile16(*use, dt, in, out, s, numSMs, &g); break;
        default: err = cudaErrorInvalidValue;
      }
      break;
    }
    default:
      err = cudaErrorInvalidValue;
  }
  if (err == cudaSuccess) gLaunchCount.fetch_add(1, std::memory_order_relaxed);
  if (grid) *grid = g;
  return err;
}

}  // namespace lt
