// Tile kernel of the transpose engine (sm_103a): covers LibreTT's Tiled,
// Packed and PackedSplit methods (src/kernel.cpp:48-170, :175-296, :304-444).
//
// A tile is the sub-tensor with extent trE[t] along each tile rank.  Its
// elements are numbered j in input order and q in output order.  One CTA
// walks its tiles (blockIdx.x, blockIdx.x + gridDim.x, ...):
//   load  : load unit u (LV consecutive j, one 16-byte access when LV > 1)
//           goes from global memory to shared memory at smemIndex(u * LV);
//   store : store unit w (SV consecutive q) gathers its SV elements from
//           shared memory and leaves as one global store.
// Units never straddle a run boundary and are 16-byte aligned in global
// memory; the planner only picks LV/SV > 1 when the layout guarantees this.
//
// Offsets of units relative to the tile base are the same for every tile, so
// each CTA computes them once into shared-memory tables; only two 64-bit
// bases change per tile.  Tiles cut by a ragged rank (dim not a multiple of
// the extent) recover the coordinate along that rank with two invariant
// divisions and skip units outside the tensor.
#pragma once

#include "kernels.cuh"

namespace lt {

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

// Coordinate along a ragged rank of in-tile index x, given the divisor of
// that rank's in-tile stride (input or output order) and of its extent.
__device__ __forceinline__ unsigned raggedCoord(uint32_t x, const FastDiv& strideDiv,
                                                const FastDiv& extDiv) {
  const uint32_t a = fdiv(x, strideDiv);
  return a - fdiv(a, extDiv) * extDiv.d;
}

// A unit whose packed ragged coordinates are rg (coordinate along ragged
// rank 0 in the low 16 bits, rank 1 in the high 16 bits) lies inside a tile
// whose valid extents along those ranks are lim0 / lim1.
__device__ __forceinline__ bool insideTile(unsigned rg, unsigned lim0, unsigned lim1) {
  return (rg & 0xffffu) < lim0 && (rg >> 16) < lim1;
}

__device__ __forceinline__ bool fullTile(unsigned lim0, unsigned lim1) {
  return (lim0 & lim1) == 0xffffu;
}

// Returns x unchanged, but the compiler cannot see through it: values derived
// from it are recomputed where used instead of being hoisted out of the tile
// loop and kept live in registers for every slot.
__device__ __forceinline__ int opaque(int x) {
  asm volatile("" : "+r"(x));
  return x;
}

__device__ __forceinline__ int smemIndex(const TileParams& p, int j) {
  return j + ((j >> p.padShift) << p.padLog);
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

// Shared-memory tables, built once per CTA:
//   ldOff[u]  global input offset (elements) of load unit u,
//   stOff[w]  global output offset (elements) of store unit w,
//   stSm[q]   shared-memory data index of output-order element q,
//   rgIn[u], rgOut[w]  packed coordinates along the ragged ranks (only when
//             the tile has ragged ranks).
struct TileTables {
  int* ldOff;
  int* stOff;
  unsigned short* stSm;
  unsigned* rgIn;
  unsigned* rgOut;
  unsigned char* data;  // data buffers follow the tables (16-byte aligned)
};

// Layout: stSm (2 bytes per element, padded to 16 bytes); ldOff, stOff and,
// with ragged ranks, rgIn, rgOut (4 bytes per unit), padded to 16 bytes;
// then the data buffers.
__host__ __device__ inline int tileSmIndexBytes(int vol) { return ((2 * vol + 15) / 16) * 16; }

__host__ __device__ inline int tileTableBytes(int vol, int lv, int sv, int ragged) {
  const int units = vol / lv + vol / sv;
  return tileSmIndexBytes(vol) + ((4 * units * (ragged ? 2 : 1) + 15) / 16) * 16;
}

__device__ __forceinline__ TileTables buildTileTables(const TileParams& p, unsigned char* smraw) {
  TileTables tt;
  const bool ragged = p.nRagged > 0;
  tt.stSm = reinterpret_cast<unsigned short*>(smraw);
  tt.ldOff = reinterpret_cast<int*>(smraw + tileSmIndexBytes(p.tileVol));
  tt.stOff = tt.ldOff + p.nIn;
  tt.rgIn = reinterpret_cast<unsigned*>(tt.stOff + p.nOut);
  tt.rgOut = tt.rgIn + p.nIn;
  tt.data = smraw + tileTableBytes(p.tileVol, p.lv, p.sv, ragged);
  for (int u = threadIdx.x; u < p.nIn; u += blockDim.x) {
    int rem = u * p.lv, off = 0;
    unsigned rg = 0;
    for (int t = 0; t < p.nTR; ++t) {
      const int e = p.trE[t];
      const int q = rem / e;
      const int c = rem - q * e;
      off += c * p.trSin[t];
      rem = q;
      if (t == p.rgTR[0]) rg |= (unsigned)c;
      if (t == p.rgTR[1]) rg |= (unsigned)c << 16;
    }
    tt.ldOff[u] = off;
    if (ragged) tt.rgIn[u] = rg;
  }
  for (int q = threadIdx.x; q < p.tileVol; q += blockDim.x) {
    int rem = q, off = 0, jj = 0;
    unsigned rg = 0;
    for (int i = 0; i < p.nTR; ++i) {
      const int t = p.trOut[i];
      const int e = p.trE[t];
      const int d = rem / e;
      const int c = rem - d * e;
      rem = d;
      off += c * p.trSout[t];
      jj += c * p.trInTile[t];
      if (t == p.rgTR[0]) rg |= (unsigned)c;
      if (t == p.rgTR[1]) rg |= (unsigned)c << 16;
    }
    tt.stSm[q] = (unsigned short)smemIndex(p, jj);
    if (q % p.sv == 0) {
      tt.stOff[q / p.sv] = off;
      if (ragged) tt.rgOut[q / p.sv] = rg;
    }
  }
  __syncthreads();
  return tt;
}

// Store phase shared by both pipelines: gather SV elements per store unit
// from shared memory and write them as one access.
template <int ES, int SV>
__device__ __forceinline__ void storeTile(const TileParams& p, const TileTables& tt,
                                          const typename Word<ES>::T* s, void* outBase,
                                          unsigned lim0, unsigned lim1) {
  using T = typename Word<ES>::T;
  using ST = typename Word<ES * SV>::T;
  const int tv = opaque(threadIdx.x);
  const bool full = fullTile(lim0, lim1);
#pragma unroll 4
  for (int w = tv; w < p.nOut; w += TILE_THREADS) {
    if (!full && !insideTile(tt.rgOut[w], lim0, lim1)) continue;
    const int off = tt.stOff[w];
    if constexpr (SV == 1) {
      *reinterpret_cast<T*>(reinterpret_cast<T*>(outBase) + off) = s[tt.stSm[w]];
    } else {
      T e[SV];
      if constexpr (SV == 2) {
        const unsigned idx = *reinterpret_cast<const unsigned*>(tt.stSm + 2 * w);
        e[0] = s[idx & 0xffffu];
        e[1] = s[idx >> 16];
      } else {
        const uint2 idx = *reinterpret_cast<const uint2*>(tt.stSm + 4 * w);
        e[0] = s[idx.x & 0xffffu];
        e[1] = s[idx.x >> 16];
        e[2] = s[idx.y & 0xffffu];
        e[3] = s[idx.y >> 16];
      }
      ST v;
      static_assert(sizeof(ST) == SV * sizeof(T), "unit size");
      __builtin_memcpy(&v, e, sizeof(ST));
      *reinterpret_cast<ST*>(reinterpret_cast<T*>(outBase) + off) = v;
    }
  }
}

// Register-staged pipeline: load units go global -> registers -> shared
// memory; the next tile's loads are issued before the current tile's
// stores.  Two shared data buffers, one barrier per tile.
template <int ES, int LV, int SV, int NL>
__global__ void __launch_bounds__(TILE_THREADS)
tileKernelReg(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
              typename Word<ES>::T* __restrict__ out) {
  using T = typename Word<ES>::T;
  using LT = typename Word<ES * LV>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const TileTables tt = buildTileTables(p, smraw);
  T* sm = reinterpret_cast<T*>(tt.data);

  uint32_t tile = blockIdx.x;
  if (tile >= p.numTiles) return;
  long long bin, bout;
  unsigned lim0, lim1;
  decodeTile(p, tile, bin, bout, lim0, lim1);

  LT v[NL];
  auto load = [&](long long base, unsigned l0, unsigned l1) {
    const int tv = opaque(threadIdx.x);
    const bool full = fullTile(l0, l1);
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int u = tv + k * TILE_THREADS;
      if (u < p.nIn && (full || insideTile(tt.rgIn[u], l0, l1)))
        v[k] = *reinterpret_cast<const LT*>(in + base + tt.ldOff[u]);
    }
  };
  load(bin, lim0, lim1);

  int buf = 0;
  for (;;) {
    T* s = sm + buf * p.smStride;
    {
      const int tv = opaque(threadIdx.x);
      const bool full = fullTile(lim0, lim1);
#pragma unroll
      for (int k = 0; k < NL; ++k) {
        const int u = tv + k * TILE_THREADS;
        if (u < p.nIn && (full || insideTile(tt.rgIn[u], lim0, lim1)))
          *reinterpret_cast<LT*>(s + smemIndex(p, u * LV)) = v[k];
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
    storeTile<ES, SV>(p, tt, s, out + bout, lim0, lim1);
    if (!more) break;
    tile = next;
    bin = nbin;
    bout = nbout;
    lim0 = nl0;
    lim1 = nl1;
    buf ^= 1;
  }
}

// cp.async pipeline (16-byte load units only): load units are copied from
// global straight into a TILE_STAGES-deep ring of shared buffers, so
// TILE_STAGES - 1 tiles of loads are in flight while one tile is stored.
template <int ES, int LV, int SV>
__global__ void __launch_bounds__(TILE_THREADS)
tileKernelAsync(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
                typename Word<ES>::T* __restrict__ out) {
  static_assert(ES * LV == 16, "cp.async pipeline moves 16-byte units");
  using T = typename Word<ES>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const TileTables tt = buildTileTables(p, smraw);
  T* sm = reinterpret_cast<T*>(tt.data);
  const uint32_t smBase = (uint32_t)__cvta_generic_to_shared(tt.data);

  const uint32_t first = blockIdx.x;
  if (first >= p.numTiles) return;
  const uint32_t G = gridDim.x;
  const uint32_t nMine = (p.numTiles - first + G - 1) / G;

  auto issue = [&](uint32_t i) {
    const uint32_t tile = first + i * G;
    long long bin, bout;
    unsigned lim0, lim1;
    decodeTile(p, tile, bin, bout, lim0, lim1);
    const T* src = in + bin;
    const uint32_t dst = smBase + (uint32_t)((i % TILE_STAGES) * p.smStride) * ES;
    const int tv = opaque(threadIdx.x);
    const bool full = fullTile(lim0, lim1);
#pragma unroll 4
    for (int u = tv; u < p.nIn; u += TILE_THREADS) {
      if (full || insideTile(tt.rgIn[u], lim0, lim1))
        cpAsync<16>(dst + (uint32_t)smemIndex(p, u * LV) * ES, src + tt.ldOff[u]);
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
    long long bin, bout;
    unsigned lim0, lim1;
    decodeTile(p, first + i * G, bin, bout, lim0, lim1);
    storeTile<ES, SV>(p, tt, sm + (i % TILE_STAGES) * p.smStride, out + bout, lim0, lim1);
  }
  cpAsyncWait<0>();
}

}  // namespace lt
