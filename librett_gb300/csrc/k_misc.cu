// Copy and row-copy launches, occupancy cache, and the launch dispatcher
// (the role of LibreTT's librettKernel switch, src/kernel.cpp:1008-1215).
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "kernels.cuh"

namespace lt {

std::atomic<unsigned long long> gLaunchCount{0};

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
    int maxOptin = 0;
    cudaDeviceGetAttribute(&maxOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > maxOptin) return 0;
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, maxOptin) !=
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
  return *smOffset + 2 * (size_t)tp.tileVol;
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

cudaError_t createDeviceTables(const PlanDesc& pd, cudaStream_t s, void** alloc, DeviceTables* dt) {
  *alloc = nullptr;
  *dt = DeviceTables();
  if (pd.kernel != K_TILE || pd.pipe != PIPE_FLAT) return cudaSuccess;
  size_t stOffset, smOffset;
  const size_t total = deviceTableBytes(pd.tile, &stOffset, &smOffset);
  void* d = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaError_t err = tablePool(&pool);
  if (err != cudaSuccess) return err;
  err = cudaMallocFromPoolAsync(&d, total, pool, s);
  if (err != cudaSuccess) return err;
  // the tables are computed on the device, in stream order before any use
  err = writeDeviceTables(pd.tile, static_cast<unsigned char*>(d), s, dt);
  if (err != cudaSuccess) {
    cudaFreeAsync(d, s);
    *dt = DeviceTables();
    return err;
  }
  *alloc = d;
  return cudaSuccess;
}

void destroyDeviceTables(void* alloc, cudaStream_t s) {
  if (alloc != nullptr) cudaFreeAsync(alloc, s);
}

cudaError_t launchPlan(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                       cudaStream_t s, int numSMs, int* grid) {
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
