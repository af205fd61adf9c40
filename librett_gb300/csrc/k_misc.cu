// Copy and row-copy launches, occupancy cache, and the launch dispatcher
// (the role of LibreTT's librettKernel switch, src/kernel.cpp:1008-1215).
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

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
cudaError_t launchCopy(const void* in, void* out, long long n, cudaStream_t s, int numSMs,
                       int* grid) {
  using T = typename Word<US>::T;
  auto fn = copyKernel<US>;
  int occ = cachedOccupancy((const void*)fn, COPY_THREADS, 0);
  if (occ < 1) return cudaErrorInvalidConfiguration;
  long long want = (n + COPY_THREADS * 4 - 1) / (COPY_THREADS * 4);
  long long g = std::min<long long>(want, (long long)numSMs * occ);
  if (g < 1) g = 1;
  *grid = (int)g;
  fn<<<(unsigned)g, COPY_THREADS, 0, s>>>((const T*)in, (T*)out, n);
  return cudaGetLastError();
}

template <int US>
cudaError_t launchRows(const RowParams& rp, const void* in, void* out, cudaStream_t s,
                       int numSMs, int* grid) {
  using T = typename Word<US>::T;
  auto fn = rowCopyKernel<US>;
  int occ = cachedOccupancy((const void*)fn, ROW_THREADS, 0);
  if (occ < 1) return cudaErrorInvalidConfiguration;
  long long warpsPerCta = ROW_THREADS / 32;
  long long want = ((long long)rp.numItems + warpsPerCta * 4 - 1) / (warpsPerCta * 4);
  long long g = std::min<long long>(want, (long long)numSMs * occ);
  if (g < 1) g = 1;
  *grid = (int)g;
  fn<<<(unsigned)g, ROW_THREADS, 0, s>>>(rp, (const T*)in, (T*)out);
  return cudaGetLastError();
}

cudaError_t launchCopyUnit(int unit, const void* in, void* out, long long n, cudaStream_t s,
                           int numSMs, int* grid) {
  switch (unit) {
    case 4: return launchCopy<4>(in, out, n, s, numSMs, grid);
    case 8: return launchCopy<8>(in, out, n, s, numSMs, grid);
    case 16: return launchCopy<16>(in, out, n, s, numSMs, grid);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launchRowsUnit(int unit, const RowParams& rp, const void* in, void* out,
                           cudaStream_t s, int numSMs, int* grid) {
  switch (unit) {
    case 4: return launchRows<4>(rp, in, out, s, numSMs, grid);
    case 8: return launchRows<8>(rp, in, out, s, numSMs, grid);
    case 16: return launchRows<16>(rp, in, out, s, numSMs, grid);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launchPlan(const PlanDesc& pd, const void* in, void* out, cudaStream_t s, int numSMs,
                       int* grid) {
  const uintptr_t align = (uintptr_t)in | (uintptr_t)out;
  int g = 0;
  cudaError_t err = cudaErrorInvalidValue;
  switch (pd.kernel) {
    case K_COPY: {
      int unit = (align % pd.unitBytes == 0) ? pd.unitBytes : pd.f.esize;
      long long n = pd.f.vol * pd.f.esize / unit;
      err = launchCopyUnit(unit, in, out, n, s, numSMs, &g);
      break;
    }
    case K_ROW: {
      bool vec = align % pd.unitBytes == 0;
      err = launchRowsUnit(vec ? pd.unitBytes : pd.f.esize, vec ? pd.row : pd.rowScalar, in, out,
                           s, numSMs, &g);
      break;
    }
    case K_TILE: {
      const PlanDesc* use = &pd;
      PlanDesc scalar;
      if ((pd.tile.lv > 1 || pd.tile.sv > 1) && align % 16 != 0) {
        // 16-byte units need 16-byte aligned tensors; fall back to elements
        scalar = pd;
        scalar.tile = pd.tileScalar;
        scalar.slots = pd.slotsScalar;
        scalar.smemBytes = pd.smemBytesScalar;
        scalar.pipe = PIPE_REG;
        use = &scalar;
      }
      switch (pd.f.esize) {
        case 4: err = launchTile4(*use, in, out, s, numSMs, &g); break;
        case 8: err = launchTile8(*use, in, out, s, numSMs, &g); break;
        case 16: err = launchTile16(*use, in, out, s, numSMs, &g); break;
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
