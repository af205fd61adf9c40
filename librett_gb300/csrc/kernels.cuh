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
// element j (input order) is copied by thread j % 256 (slot j / 256) from
// global memory straight into shared memory at j + (j >> padShift) with
// cp.async; in-tile element q in output order is then read back from shared
// memory and stored to global memory.  Each CTA walks its tiles (blockIdx.x,
// blockIdx.x + gridDim.x, ...) through a TILE_STAGES-deep ring of shared
// buffers, so TILE_STAGES - 1 tiles of loads are in flight while one tile is
// stored.  Per-slot offsets are computed once per CTA; per tile only two
// 64-bit bases change.  Tiles cut by a ragged rank (dim not a multiple of the
// extent) take a checked path that recovers the slot's coordinate along each
// ragged rank with two invariant divisions, so no per-slot coordinates are
// kept in registers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void decodeTile(const TileParams& p, uint32_t tile, long long& bin,
                                           long long& bout, unsigned& lim0, unsigned& lim1) {
  bin = 0;
  bout = 0;
  lim0 = 0xffffu;
  lim1 = 0xffffu;
  uint32_t rem = tile;
  for (int g = 0; g < p.nGR; ++g) {
    const uint32_t q = fdiv(rem, p.grDiv[g]);
    const uint32_t c = rem - q * p.grDiv[g].d;
    rem = q;
    bin += (long long)c * p.grSin[g];
    bout += (long long)c * p.grSout[g];
    const int s = p.grRg[g];
    if (s >= 0) {
      // only the last chunk of a ragged rank is partial
      const long long left = p.rgDim[s] - (long long)c * p.rgE[s];
      if (left < p.rgE[s]) {
        if (s == 0) lim0 = (unsigned)left; else lim1 = (unsigned)left;
      }
    }
  }
}

// Coordinate along ragged slot s of in-tile index x, given the divisor of
// the rank's in-tile stride (input or output order).
__device__ __forceinline__ unsigned raggedCoord(uint32_t x, const FastDiv& strideDiv,
                                                const FastDiv& extDiv) {
  const uint32_t a = fdiv(x, strideDiv);
  return a - fdiv(a, extDiv) * extDiv.d;
}

template <int BYTES>
__device__ __forceinline__ void cpAsync(uint32_t dst, const void* src) {
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES)
                 : "memory");
  }
}

__device__ __forceinline__ void cpAsyncCommit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int NREG>
struct TileLaunchBounds {
  static constexpr int minBlocks = NREG <= 8 ? 4 : 2;
};

template <int ES, int NREG>
__global__ void __launch_bounds__(TILE_THREADS, TileLaunchBounds<NREG>::minBlocks)
tileKernelAsync(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
           typename Word<ES>::T* __restrict__ out) {
  using T = typename Word<ES>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const uint32_t smBase = (uint32_t)__cvta_generic_to_shared(smraw);
  const int tid = threadIdx.x;
  const int vol = p.tileVol;
  const int pad = p.padShift;

  // Per-slot offsets (same for every tile).
  int ldOff[NREG];
  int stOff[NREG];
  int stSm[NREG];
#pragma unroll
  for (int k = 0; k < NREG; ++k) {
    const int j = tid + k * TILE_THREADS;
    ldOff[k] = 0;
    stOff[k] = 0;
    stSm[k] = 0;
    if (j < vol) {
      int rem = j, off = 0;
      for (int t = 0; t < p.nTR; ++t) {
        const int e = p.trE[t];
        const int q = rem / e;
        off += (rem - q * e) * p.trSin[t];
        rem = q;
      }
      ldOff[k] = off;
      rem = j;
      off = 0;
      int jj = 0;
      for (int i = 0; i < p.nTR; ++i) {
        const int t = p.trOut[i];
        const int e = p.trE[t];
        const int q = rem / e;
        const int c = rem - q * e;
        rem = q;
        off += c * p.trSout[t];
        jj += c * p.trInTile[t];
      }
      stOff[k] = off;
      stSm[k] = jj + (jj >> pad);
    }
  }

  const uint32_t first = blockIdx.x;
  if (first >= p.numTiles) return;
  const uint32_t G = gridDim.x;
  const uint32_t nMine = (p.numTiles - first + G - 1) / G;

  // Issue the loads of my i-th tile into stage i % TILE_STAGES.
  auto issue = [&](uint32_t i) {
    const uint32_t tile = first + i * G;
    long long bin, bout;
    unsigned lim0, lim1;
    decodeTile(p, tile, bin, bout, lim0, lim1);
    const T* src = in + bin;
    const uint32_t dst = smBase + (uint32_t)((i % TILE_STAGES) * p.smStride) * ES;
    const bool full = lim0 == 0xffffu && lim1 == 0xffffu;
#pragma unroll
    for (int k = 0; k < NREG; ++k) {
      const int j = tid + k * TILE_THREADS;
      bool ok = j < vol;
      if (!full && ok) {
        if (p.nRagged > 0) ok = raggedCoord(j, p.rgInDiv[0], p.rgEDiv[0]) < lim0;
        if (p.nRagged > 1 && ok) ok = raggedCoord(j, p.rgInDiv[1], p.rgEDiv[1]) < lim1;
      }
      if (ok) cpAsync<ES>(dst + (uint32_t)(j + (j >> pad)) * ES, src + ldOff[k]);
    }
  };

#pragma unroll
  for (int s = 0; s < TILE_STAGES - 1; ++s) {
    if ((uint32_t)s < nMine) issue(s);
    cpAsyncCommit();
  }
  for (uint32_t i = 0; i < nMine; ++i) {
    cpAsyncWait<TILE_STAGES - 2>();
    __syncthreads();
    // The stage refilled here was last read in iteration i - 1, which every
    // thread has finished (barrier above).
    if (i + TILE_STAGES - 1 < nMine) issue(i + TILE_STAGES - 1);
    cpAsyncCommit();
    const uint32_t tile = first + i * G;
    long long bin, bout;
    unsigned lim0, lim1;
    decodeTile(p, tile, bin, bout, lim0, lim1);
    const T* s = sm + (i % TILE_STAGES) * p.smStride;
    T* dstp = out + bout;
    const bool full = lim0 == 0xffffu && lim1 == 0xffffu;
#pragma unroll
    for (int k = 0; k < NREG; ++k) {
      const int q = tid + k * TILE_THREADS;
      bool ok = q < vol;
      if (!full && ok) {
        if (p.nRagged > 0) ok = raggedCoord(q, p.rgOutDiv[0], p.rgEDiv[0]) < lim0;
        if (p.nRagged > 1 && ok) ok = raggedCoord(q, p.rgOutDiv[1], p.rgEDiv[1]) < lim1;
      }
      if (ok) dstp[stOff[k]] = s[stSm[k]];
    }
  }
  cpAsyncWait<0>();
}

// Register-staged variant: the same tile walk, but each slot's element is
// loaded into a register (plain global load), written to shared memory, and
// the next tile's loads are issued before the current tile's stores.  Two
// shared buffers, one barrier per tile.  Preferred for 4- and 8-byte
// elements, where per-element cp.async has the lower throughput.
template <int ES, int NREG>
__global__ void __launch_bounds__(TILE_THREADS, TileLaunchBounds<NREG>::minBlocks)
tileKernelReg(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
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
#pragma unroll
  for (int k = 0; k < NREG; ++k) {
    const int j = tid + k * TILE_THREADS;
    ldOff[k] = 0;
    stOff[k] = 0;
    stSm[k] = 0;
    if (j < vol) {
      int rem = j, off = 0;
      for (int t = 0; t < p.nTR; ++t) {
        const int e = p.trE[t];
        const int q = rem / e;
        off += (rem - q * e) * p.trSin[t];
        rem = q;
      }
      ldOff[k] = off;
      rem = j;
      off = 0;
      int jj = 0;
      for (int i = 0; i < p.nTR; ++i) {
        const int t = p.trOut[i];
        const int e = p.trE[t];
        const int q = rem / e;
        const int c = rem - q * e;
        rem = q;
        off += c * p.trSout[t];
        jj += c * p.trInTile[t];
      }
      stOff[k] = off;
      stSm[k] = jj + (jj >> pad);
    }
  }

  uint32_t tile = blockIdx.x;
  if (tile >= p.numTiles) return;
  long long bin, bout;
  unsigned lim0, lim1;
  decodeTile(p, tile, bin, bout, lim0, lim1);

  T v[NREG];
  auto load = [&](long long base, unsigned l0, unsigned l1) {
    const T* src = in + base;
    const bool full = l0 == 0xffffu && l1 == 0xffffu;
#pragma unroll
    for (int k = 0; k < NREG; ++k) {
      const int j = tid + k * TILE_THREADS;
      bool ok = j < vol;
      if (!full && ok) {
        if (p.nRagged > 0) ok = raggedCoord(j, p.rgInDiv[0], p.rgEDiv[0]) < l0;
        if (p.nRagged > 1 && ok) ok = raggedCoord(j, p.rgInDiv[1], p.rgEDiv[1]) < l1;
      }
      if (ok) v[k] = src[ldOff[k]];
    }
  };
  load(bin, lim0, lim1);

  int buf = 0;
  for (;;) {
    T* s = sm + buf * p.smStride;
    {
      const bool full = lim0 == 0xffffu && lim1 == 0xffffu;
#pragma unroll
      for (int k = 0; k < NREG; ++k) {
        const int j = tid + k * TILE_THREADS;
        bool ok = j < vol;
        if (!full && ok) {
          if (p.nRagged > 0) ok = raggedCoord(j, p.rgInDiv[0], p.rgEDiv[0]) < lim0;
          if (p.nRagged > 1 && ok) ok = raggedCoord(j, p.rgInDiv[1], p.rgEDiv[1]) < lim1;
        }
        if (ok) s[j + (j >> pad)] = v[k];
      }
    }
    __syncthreads();
    const uint32_t next = tile + gridDim.x;
    const bool more = next < p.numTiles;
    long long nbin = 0, nbout = 0;
    unsigned nl0 = 0xffffu, nl1 = 0xffffu;
    if (more) {
      decodeTile(p, next, nbin, nbout, nl0, nl1);
      load(nbin, nl0, nl1);
    }
    {
      T* dstp = out + bout;
      const bool full = lim0 == 0xffffu && lim1 == 0xffffu;
#pragma unroll
      for (int k = 0; k < NREG; ++k) {
        const int q = tid + k * TILE_THREADS;
        bool ok = q < vol;
        if (!full && ok) {
          if (p.nRagged > 0) ok = raggedCoord(q, p.rgOutDiv[0], p.rgEDiv[0]) < lim0;
          if (p.nRagged > 1 && ok) ok = raggedCoord(q, p.rgOutDiv[1], p.rgEDiv[1]) < lim1;
        }
        if (ok) dstp[stOff[k]] = s[stSm[k]];
      }
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
