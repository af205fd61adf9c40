// Device kernels of the transpose engine (sm_103a).
//
// LibreTT counterparts (src/kernel.cpp): transposeTiled (:48-170),
// transposePacked (:175-296), transposePackedSplit (:304-444) and
// transposeTiledCopy (:453-545), plus the cudaMemcpyAsync used for Trivial
// (:1014-1026).  Here one persistent tile kernel covers Tiled, Packed and
// PackedSplit: the planner's tile (an extent per fused rank) decides which of
// them a launch behaves like.  All data moves as raw 4/8/16-byte words.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "launch.h"
#include "plan.h"

namespace lt {

template <int ES> struct Word;
template <> struct Word<4> { using T = unsigned int; };
template <> struct Word<8> { using T = uint2; };
template <> struct Word<16> { using T = uint4; };

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return (uint32_t)(((unsigned long long)n * f.mul) >> f.shift);
}

// ---------------------------------------------------------------------------
// Trivial: contiguous copy in units of US bytes, four independent loads in
// flight per thread.
// ---------------------------------------------------------------------------
template <int US>
__global__ void __launch_bounds__(COPY_THREADS)
copyKernel(const typename Word<US>::T* __restrict__ in, typename Word<US>::T* __restrict__ out,
           long long n) {
  using T = typename Word<US>::T;
  const long long stride = (long long)gridDim.x * COPY_THREADS;
  long long i = (long long)blockIdx.x * COPY_THREADS + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    T a = in[i];
    T b = in[i + stride];
    T c = in[i + 2 * stride];
    T d = in[i + 3 * stride];
    out[i] = a;
    out[i + stride] = b;
    out[i + 2 * stride] = c;
    out[i + 3 * stride] = d;
  }
  for (; i < n; i += stride) out[i] = in[i];
}

// ---------------------------------------------------------------------------
// TiledCopy: input rank 0 is also output rank 0, so the tensor is a set of
// contiguous rows (dim[0] elements) that move to new row positions.  Work
// item = 32 units of one row; each warp takes four items per step so four
// loads per lane are in flight before the stores.
// ---------------------------------------------------------------------------
template <int US>
__global__ void __launch_bounds__(ROW_THREADS)
rowCopyKernel(const __grid_constant__ RowParams p, const typename Word<US>::T* __restrict__ in,
              typename Word<US>::T* __restrict__ out) {
  using T = typename Word<US>::T;
  const int lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * ROW_THREADS) >> 5;
  uint32_t it = (blockIdx.x * ROW_THREADS + threadIdx.x) >> 5;
  for (; it < p.numItems; it += 4 * nw) {
    T v[4];
    long long dst[4];
    bool ok[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t item = it + u * nw;
      ok[u] = false;
      if (item < p.numItems) {
        const uint32_t row = fdiv(item, p.chunkDiv);
        const int col = (int)(item - row * p.chunkDiv.d) * 32 + lane;
        uint32_t rem = row;
        long long bi = 0, bo = 0;
        for (int g = 0; g < p.nR; ++g) {
          const uint32_t q = fdiv(rem, p.rDiv[g]);
          const uint32_t c = rem - q * p.rDiv[g].d;
          rem = q;
          bi += (long long)c * p.rSin[g];
          bo += (long long)c * p.rSout[g];
        }
        if (col < p.rowUnits) {
          ok[u] = true;
          v[u] = in[bi + col];
          dst[u] = bo + col;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (ok[u]) out[dst[u]] = v[u];
  }
}

// ---------------------------------------------------------------------------
// Tile kernel (Tiled / Packed / PackedSplit).
//
// A tile is the sub-tensor with extent trE[t] along each tile rank.  In-tile
// element j (input order) is loaded by thread j % 256 into slot j / 256 and
// written to shared memory at j + (j >> padShift).  For the store, in-tile
// element q in output order is read back from shared memory and written to
// the output.  Per-slot offsets are computed once per CTA; per tile only the
// two 64-bit base offsets change.  Shared memory is double-buffered so one
// barrier per tile suffices, and the next tile's loads are issued before the
// current tile's stores.
// ---------------------------------------------------------------------------
template <bool RAGGED>
__device__ __forceinline__ void decodeTile(const TileParams& p, uint32_t tile, long long& bin,
                                           long long& bout, unsigned& lim0, unsigned& lim1) {
  bin = 0;
  bout = 0;
  lim0 = 1;
  lim1 = 1;
  uint32_t rem = tile;
  for (int g = 0; g < p.nGR; ++g) {
    uint32_t q = fdiv(rem, p.grDiv[g]);
    uint32_t c = rem - q * p.grDiv[g].d;
    rem = q;
    bin += (long long)c * p.grSin[g];
    bout += (long long)c * p.grSout[g];
    if (RAGGED) {
      int s = p.grRg[g];
      if (s >= 0) {
        long long left = p.rgDim[s] - (long long)c * p.rgE[s];
        unsigned lim = (unsigned)(left < p.rgE[s] ? left : p.rgE[s]);
        if (s == 0) lim0 = lim; else lim1 = lim;
      }
    }
  }
}

template <int ES, int NREG, bool RAGGED>
__global__ void __launch_bounds__(TILE_THREADS)
tileKernel(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
           typename Word<ES>::T* __restrict__ out) {
  using T = typename Word<ES>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int tid = threadIdx.x;
  const int vol = p.tileVol;
  const int pad = p.padShift;

  int ldOff[NREG];
  int stOff[NREG];
  int stSm[NREG];
  unsigned ldRg[NREG];
  unsigned stRg[NREG];
#pragma unroll
  for (int k = 0; k < NREG; ++k) {
    const int j = tid + k * TILE_THREADS;
    ldOff[k] = 0;
    stOff[k] = 0;
    stSm[k] = 0;
    ldRg[k] = 0xffffffffu;
    stRg[k] = 0xffffffffu;
    if (j < vol) {
      int rem = j, off = 0;
      unsigned rg = 0;
      for (int t = 0; t < p.nTR; ++t) {
        const int e = p.trE[t];
        const int q = rem / e;
        const int c = rem - q * e;
        rem = q;
        off += c * p.trSin[t];
        if (RAGGED) {
          if (t == p.rgTR[0]) rg |= (unsigned)c;
          if (t == p.rgTR[1]) rg |= (unsigned)c << 16;
        }
      }
      ldOff[k] = off;
      ldRg[k] = rg;
      rem = j;
      off = 0;
      rg = 0;
      int jj = 0;
      for (int i = 0; i < p.nTR; ++i) {
        const int t = p.trOut[i];
        const int e = p.trE[t];
        const int q = rem / e;
        const int c = rem - q * e;
        rem = q;
        off += c * p.trSout[t];
        jj += c * p.trInTile[t];
        if (RAGGED) {
          if (t == p.rgTR[0]) rg |= (unsigned)c;
          if (t == p.rgTR[1]) rg |= (unsigned)c << 16;
        }
      }
      stOff[k] = off;
      stSm[k] = jj + (jj >> pad);
      stRg[k] = rg;
    }
  }

  uint32_t tile = blockIdx.x;
  if (tile >= p.numTiles) return;
  long long bin, bout;
  unsigned lim0, lim1;
  decodeTile<RAGGED>(p, tile, bin, bout, lim0, lim1);

  T v[NREG];
#pragma unroll
  for (int k = 0; k < NREG; ++k) {
    const int j = tid + k * TILE_THREADS;
    bool ok = RAGGED ? ((ldRg[k] & 0xffffu) < lim0 && (ldRg[k] >> 16) < lim1) : (j < vol);
    if (ok) v[k] = in[bin + ldOff[k]];
  }

  int buf = 0;
  for (;;) {
    T* s = sm + buf * p.smStride;
#pragma unroll
    for (int k = 0; k < NREG; ++k) {
      const int j = tid + k * TILE_THREADS;
      bool ok = RAGGED ? ((ldRg[k] & 0xffffu) < lim0 && (ldRg[k] >> 16) < lim1) : (j < vol);
      if (ok) s[j + (j >> pad)] = v[k];
    }
    __syncthreads();
    const uint32_t next = tile + gridDim.x;
    const bool more = next < p.numTiles;
    long long nbin = 0, nbout = 0;
    unsigned nl0 = 1, nl1 = 1;
    if (more) {
      decodeTile<RAGGED>(p, next, nbin, nbout, nl0, nl1);
#pragma unroll
      for (int k = 0; k < NREG; ++k) {
        const int j = tid + k * TILE_THREADS;
        bool ok = RAGGED ? ((ldRg[k] & 0xffffu) < nl0 && (ldRg[k] >> 16) < nl1) : (j < vol);
        if (ok) v[k] = in[nbin + ldOff[k]];
      }
    }
#pragma unroll
    for (int k = 0; k < NREG; ++k) {
      const int j = tid + k * TILE_THREADS;
      bool ok = RAGGED ? ((stRg[k] & 0xffffu) < lim0 && (stRg[k] >> 16) < lim1) : (j < vol);
      if (ok) out[bout + stOff[k]] = s[stSm[k]];
    }
    if (!more) break;
    tile = next;
    bin = nbin;
    bout = nbout;
    lim0 = nl0;
    lim1 = nl1;
    buf ^= 1;
  }
}

// Launch helpers (defined in the per-element-size translation units).
cudaError_t launchTile4(const PlanDesc& pd, const void* in, void* out, cudaStream_t s, int numSMs,
                        int* grid);
cudaError_t launchTile8(const PlanDesc& pd, const void* in, void* out, cudaStream_t s, int numSMs,
                        int* grid);
cudaError_t launchTile16(const PlanDesc& pd, const void* in, void* out, cudaStream_t s, int numSMs,
                         int* grid);

}  // namespace lt
