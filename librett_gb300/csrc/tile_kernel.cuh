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
// Every tile is full: along a rank whose dim is not a multiple of the
// extent, the last chunk starts at dim - extent and overlaps its neighbour
// (the overlap is loaded and stored twice with identical bits).  So no tile
// needs bounds checks.  Offsets of units relative to the tile base are the
// same for every tile; each CTA computes them once into shared-memory tables
// and only two 64-bit bases change per tile.
#pragma once

#include <type_traits>

#include "group.h"
#include "kernels.cuh"

namespace lt {

__device__ __forceinline__ void decodeTile(const TileParams& p, uint32_t tile, long long& bin,
                                           long long& bout) {
  bin = 0;
  bout = 0;
  uint32_t rem = tile;
  for (int g = 0; g < p.nGR; ++g) {
    const uint32_t q = fdiv(rem, p.grDiv[g]);
    const uint32_t c = rem - q * p.grDiv[g].d;
    rem = q;
    const bool last = c + 1 == p.grDiv[g].d;
    bin += last ? p.grLastIn[g] : (long long)c * p.grSin[g];
    bout += last ? p.grLastOut[g] : (long long)c * p.grSout[g];
  }
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

// Table-free addressing for tiles of NTR ranks (1 <= NTR <= ARITH_MAX_NTR):
// the global input offset of input-order element j of a tile, and the global
// output offset and the input-order index of output-order element q, from
// their mixed-radix digits.  In-tile indices are below 2^16 and extents at
// least 2, so the digit __umulhi(x, ceil(2^32 / extent)) is exact
// (ceil(2^32 / e) * x / 2^32 exceeds x / e by less than x / 2^32 < 1 / e).
template <int NTR>
__device__ __forceinline__ int arithInOffset(const TileParams& p, uint32_t j) {
  int off = 0;
#pragma unroll
  for (int t = 0; t + 1 < NTR; ++t) {
    const uint32_t q = __umulhi(j, p.trMul[t]);
    off += (int)(j - q * (uint32_t)p.trE[t]) * p.trSin[t];
    j = q;
  }
  return off + (int)j * p.trSin[NTR - 1];
}

template <int NTR>
__device__ __forceinline__ void arithOut(const TileParams& p, uint32_t q, int& off, int& jj) {
  off = 0;
  jj = 0;
#pragma unroll
  for (int i = 0; i + 1 < NTR; ++i) {
    const uint32_t d = __umulhi(q, p.toMul[i]);
    const int c = (int)(q - d * (uint32_t)p.toE[i]);
    off += c * p.toSout[i];
    jj += c * p.toInTile[i];
    q = d;
  }
  off += (int)q * p.toSout[NTR - 1];
  jj += (int)q * p.toInTile[NTR - 1];
}

__device__ __forceinline__ void cpAsync16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}

// cp.async of one 4-, 8- or 16-byte unit (16 bytes bypass L1); PF: L2
// prefetch size in bytes (0 none, 128 or 256: the .L2::128B / .L2::256B
// qualifier).
template <int BYTES, int PF = 0>
__device__ __forceinline__ void cpAsyncUnit(uint32_t dst, const void* src) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async unit");
  static_assert(PF == 0 || PF == 128 || PF == 256, "L2 prefetch size");
  if constexpr (BYTES == 16 && PF == 256)
    asm volatile("cp.async.cg.shared.global.L2::256B [%0], [%1], 16;\n" ::"r"(dst), "l"(src)
                 : "memory");
  else if constexpr (BYTES == 16 && PF == 128)
    asm volatile("cp.async.cg.shared.global.L2::128B [%0], [%1], 16;\n" ::"r"(dst), "l"(src)
                 : "memory");
  else if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  else if constexpr (PF == 256)
    asm volatile("cp.async.ca.shared.global.L2::256B [%0], [%1], %2;\n" ::"r"(dst), "l"(src),
                 "n"(BYTES)
                 : "memory");
  else if constexpr (PF == 128)
    asm volatile("cp.async.ca.shared.global.L2::128B [%0], [%1], %2;\n" ::"r"(dst), "l"(src),
                 "n"(BYTES)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES)
                 : "memory");
}

// L2 prefetch size of the single-plan flat kernel's cp.async loads: none.
// On the 200-problem float64 suite (three interleaved runs each, one box)
// 256 bytes measured 0.2 % slower and 128 bytes the same as none.
#ifndef LT_FLAT_L2_PREFETCH
#define LT_FLAT_L2_PREFETCH 0
#endif

// L2 prefetch size of the grouped kernel's data copies: 0 (none), 128 or 256
// bytes (the .L2::128B / .L2::256B qualifier of cp.async).  256: the
// 10,000-member batch 0.3 % faster than none (two interleaved runs each, one
// box); 128 made no difference.
#ifndef LT_GROUP_L2_PREFETCH
#define LT_GROUP_L2_PREFETCH 256
#endif

// Flat tile kernels with at least this many load units per thread load
// through cp.async rather than registers: 8 (measured best on the float64
// suite: 4 is 0.1 % and register loads throughout 0.7 % slower), but 4 for
// 4-byte elements (the float32 small-leading-dim case 1.1 % faster).
#ifndef LT_FLAT_ASYNC_MIN_NL
#define LT_FLAT_ASYNC_MIN_NL 8
#endif

template <int ES>
__host__ __device__ constexpr int flatAsyncMinNL() {
  return ES == 4 && LT_FLAT_ASYNC_MIN_NL > 4 ? 4 : LT_FLAT_ASYNC_MIN_NL;
}

__device__ __forceinline__ void cpAsyncWaitAll() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
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
//   stSm[q]   shared-memory data index of output-order element q.
struct TileTables {
  int* ldOff;
  int* stOff;
  unsigned short* stSm;
  unsigned char* data;  // data buffers follow the tables (16-byte aligned)
};

// Layout: stSm (2 bytes per element, padded to 16 bytes); ldOff and stOff
// (4 bytes per unit), padded to 16 bytes; then the data buffers.
__host__ __device__ inline int tileSmIndexBytes(int vol) { return ((2 * vol + 15) / 16) * 16; }

__host__ __device__ inline int tileTableBytes(int vol, int lv, int sv) {
  return tileSmIndexBytes(vol) + ((4 * (vol / lv + vol / sv) + 15) / 16) * 16;
}

__device__ __forceinline__ TileTables buildTileTables(const TileParams& p, unsigned char* smraw) {
  TileTables tt;
  tt.stSm = reinterpret_cast<unsigned short*>(smraw);
  tt.ldOff = reinterpret_cast<int*>(smraw + tileSmIndexBytes(p.tileVol));
  tt.stOff = tt.ldOff + p.nIn;
  tt.data = smraw + tileTableBytes(p.tileVol, p.lv, p.sv);
  for (int u = threadIdx.x; u < p.nIn; u += blockDim.x) {
    int rem = u * p.lv, off = 0;
    for (int t = 0; t < p.nTR; ++t) {
      const int e = p.trE[t];
      const int q = rem / e;
      off += (rem - q * e) * p.trSin[t];
      rem = q;
    }
    tt.ldOff[u] = off;
  }
  for (int q = threadIdx.x; q < p.tileVol; q += blockDim.x) {
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
    tt.stSm[q] = (unsigned short)smemIndex(p, jj);
    if (q % p.sv == 0) tt.stOff[q / p.sv] = off;
  }
  __syncthreads();
  return tt;
}

// Store phase shared by all pipelines: gather SV elements per store unit
// from shared memory and write them as one access.  stOff / stSm point to
// the offset tables (shared memory or device memory).
template <int ES, int SV>
__device__ __forceinline__ void storeTile(const TileParams& p, const int* __restrict__ stOff,
                                          const unsigned short* __restrict__ stSm,
                                          const typename Word<ES>::T* s,
                                          typename Word<ES>::T* outBase) {
  using T = typename Word<ES>::T;
  using ST = typename Word<ES * SV>::T;
  static_assert(sizeof(ST) == SV * sizeof(T), "unit size");
  const int tv = opaque(threadIdx.x);
#pragma unroll 4
  for (int w = tv; w < p.nOut; w += TILE_THREADS) {
    T* dst = outBase + stOff[w];
    if constexpr (SV == 1) {
      *dst = s[stSm[w]];
    } else {
      T e[SV];
      if constexpr (SV == 2) {
        const unsigned idx = *reinterpret_cast<const unsigned*>(stSm + 2 * w);
        e[0] = s[idx & 0xffffu];
        e[1] = s[idx >> 16];
      } else {
        const uint2 idx = *reinterpret_cast<const uint2*>(stSm + 4 * w);
        e[0] = s[idx.x & 0xffffu];
        e[1] = s[idx.x >> 16];
        e[2] = s[idx.y & 0xffffu];
        e[3] = s[idx.y >> 16];
      }
      ST v;
      __builtin_memcpy(&v, e, sizeof(ST));
      *reinterpret_cast<ST*>(dst) = v;
    }
  }
}

// Shared indices of store unit w's SV elements (stSm entries) in one word.
template <int SV> struct SmIdx;
template <> struct SmIdx<1> { using T = unsigned short; };
template <> struct SmIdx<2> { using T = unsigned; };
template <> struct SmIdx<4> { using T = uint2; };

template <int SV>
__device__ __forceinline__ typename SmIdx<SV>::T loadSmIdx(const unsigned short* __restrict__ stSm,
                                                           int w) {
  return __ldg(reinterpret_cast<const typename SmIdx<SV>::T*>(stSm + SV * w));
}

// Store unit w: gathers its SV elements at shared indices idx and writes
// them as one access at dst.
template <int ES, int SV>
__device__ __forceinline__ void storeUnit(const typename Word<ES>::T* s,
                                          typename SmIdx<SV>::T idx, typename Word<ES>::T* dst) {
  using T = typename Word<ES>::T;
  using ST = typename Word<ES * SV>::T;
  if constexpr (SV == 1) {
    *dst = s[idx];
  } else {
    T e[SV];
    if constexpr (SV == 2) {
      e[0] = s[idx & 0xffffu];
      e[1] = s[idx >> 16];
    } else {
      e[0] = s[idx.x & 0xffffu];
      e[1] = s[idx.x >> 16];
      e[2] = s[idx.y & 0xffffu];
      e[3] = s[idx.y >> 16];
    }
    ST v;
    __builtin_memcpy(&v, e, sizeof(ST));
    *reinterpret_cast<ST*>(dst) = v;
  }
}

// Table entries of a thread's first store units, fetched while the tile's
// data loads are in flight so that the stores can start as soon as the
// barrier opens: the tables are a dependent device-memory read otherwise.
template <int SV, int PF>
struct StorePrefetch {
  int off[PF > 0 ? PF : 1];
  typename SmIdx<SV>::T idx[PF > 0 ? PF : 1];

  __device__ __forceinline__ void load(const TileParams& p, const int* __restrict__ stOff,
                                       const unsigned short* __restrict__ stSm) {
#pragma unroll
    for (int i = 0; i < PF; ++i) {
      const int w = threadIdx.x + i * TILE_THREADS;
      if (w < p.nOut) {
        off[i] = __ldg(stOff + w);
        idx[i] = loadSmIdx<SV>(stSm, w);
      }
    }
  }
};

// Store phase of the flat pipeline: the prefetched units first, then the
// rest as in storeTile.
template <int ES, int SV, int PF>
__device__ __forceinline__ void storeTileFlat(const TileParams& p, const int* __restrict__ stOff,
                                              const unsigned short* __restrict__ stSm,
                                              const StorePrefetch<SV, PF>& pf,
                                              const typename Word<ES>::T* s,
                                              typename Word<ES>::T* outBase) {
#pragma unroll
  for (int i = 0; i < PF; ++i) {
    const int w = threadIdx.x + i * TILE_THREADS;
    if (w < p.nOut) storeUnit<ES, SV>(s, pf.idx[i], outBase + pf.off[i]);
  }
  const int tv = opaque(threadIdx.x);
#pragma unroll 4
  for (int w = tv + PF * TILE_THREADS; w < p.nOut; w += TILE_THREADS)
    storeUnit<ES, SV>(s, loadSmIdx<SV>(stSm, w), outBase + stOff[w]);
}

// Store unit at output-order element q (SV consecutive elements), global
// offset off and first input-order index jj, addressed arithmetically: the
// unit's elements step along output tile rank 0 unless the unit crosses it
// (p.storeStraddle), then each element is decoded.
template <int ES, int SV, int NTR>
__device__ __forceinline__ void storeUnitArith(const TileParams& p,
                                               const typename Word<ES>::T* s, uint32_t q,
                                               int off, int jj, typename Word<ES>::T* outBase) {
  using T = typename Word<ES>::T;
  using ST = typename Word<ES * SV>::T;
  if constexpr (SV == 1) {
    outBase[off] = s[smemIndex(p, jj)];
  } else {
    T e[SV];
    e[0] = s[smemIndex(p, jj)];
    if (!p.storeStraddle) {
#pragma unroll
      for (int m = 1; m < SV; ++m) e[m] = s[smemIndex(p, jj + m * p.toInTile[0])];
    } else {
#pragma unroll
      for (int m = 1; m < SV; ++m) {
        int o2, j2;
        arithOut<NTR>(p, q + m, o2, j2);
        e[m] = s[smemIndex(p, j2)];
      }
    }
    ST v;
    __builtin_memcpy(&v, e, sizeof(ST));
    *reinterpret_cast<ST*>(outBase + off) = v;
  }
}

// Addresses of a thread's first PF store units (table-free addressing),
// computed while the tile's loads are in flight.
template <int NTR, int PF>
struct ArithPrefetch {
  int off[PF > 0 ? PF : 1];
  int jj[PF > 0 ? PF : 1];

  template <int SV>
  __device__ __forceinline__ void load(const TileParams& p) {
#pragma unroll
    for (int i = 0; i < PF; ++i) {
      const int w = threadIdx.x + i * TILE_THREADS;
      if (w < p.nOut) arithOut<NTR>(p, (uint32_t)(w * SV), off[i], jj[i]);
    }
  }
};

// Store phase of the flat and bulk-copy pipelines with table-free
// addressing: the prefetched units first, then the rest.
template <int ES, int SV, int NTR, int PF>
__device__ __forceinline__ void storeTileArith(const TileParams& p,
                                               const ArithPrefetch<NTR, PF>& pf,
                                               const typename Word<ES>::T* s,
                                               typename Word<ES>::T* outBase) {
#pragma unroll
  for (int i = 0; i < PF; ++i) {
    const int w = threadIdx.x + i * TILE_THREADS;
    if (w < p.nOut) storeUnitArith<ES, SV, NTR>(p, s, (uint32_t)(w * SV), pf.off[i], pf.jj[i], outBase);
  }
  const int tv = opaque(threadIdx.x);
#pragma unroll 4
  for (int w = tv + PF * TILE_THREADS; w < p.nOut; w += TILE_THREADS) {
    int off, jj;
    arithOut<NTR>(p, (uint32_t)(w * SV), off, jj);
    storeUnitArith<ES, SV, NTR>(p, s, (uint32_t)(w * SV), off, jj, outBase);
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
  decodeTile(p, tile, bin, bout);

  LT v[NL];
  auto load = [&](long long base) {
    const int tv = opaque(threadIdx.x);
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int u = tv + k * TILE_THREADS;
      if (u < p.nIn) v[k] = *reinterpret_cast<const LT*>(in + base + tt.ldOff[u]);
    }
  };
  load(bin);

  int buf = 0;
  for (;;) {
    T* s = sm + buf * p.smStride;
    {
      const int tv = opaque(threadIdx.x);
#pragma unroll
      for (int k = 0; k < NL; ++k) {
        const int u = tv + k * TILE_THREADS;
        if (u < p.nIn) *reinterpret_cast<LT*>(s + smemIndex(p, u * LV)) = v[k];
      }
    }
    __syncthreads();
    const uint32_t next = tile + gridDim.x;
    const bool more = next < p.numTiles;
    long long nbin = 0, nbout = 0;
    if (more) {
      decodeTile(p, next, nbin, nbout);
      load(nbin);
    }
    storeTile<ES, SV>(p, tt.stOff, tt.stSm, s, out + bout);
    if (!more) break;
    tile = next;
    bin = nbin;
    bout = nbout;
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
    long long bin, bout;
    decodeTile(p, first + i * G, bin, bout);
    const T* src = in + bin;
    const uint32_t dst = smBase + (uint32_t)((i % TILE_STAGES) * p.smStride) * ES;
    const int tv = opaque(threadIdx.x);
#pragma unroll 4
    for (int u = tv; u < p.nIn; u += TILE_THREADS)
      cpAsync16(dst + (uint32_t)smemIndex(p, u * LV) * ES, src + tt.ldOff[u]);
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
    decodeTile(p, first + i * G, bin, bout);
    storeTile<ES, SV>(p, tt.stOff, tt.stSm, sm + (i % TILE_STAGES) * p.smStride, out + bout);
  }
  cpAsyncWait<0>();
}

// Flat pipeline: one tile per CTA and no persistent loop, so the hardware
// block scheduler streams tiles through the SMs in order.  With NTR = 0 the
// offset tables were written at plan time and are read from device memory
// (L1/L2-resident: every CTA of the launch reads the same few kilobytes);
// with NTR = 1..ARITH_MAX_NTR (the tile's rank count) every unit's offsets
// are computed from its index instead and the table pointers are unused.
template <int ES, int LV, int SV, int NL, int NTR>
__global__ void __launch_bounds__(TILE_THREADS)
tileKernelFlat(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
               typename Word<ES>::T* __restrict__ out, const int* __restrict__ ldOff,
               const int* __restrict__ stOff, const unsigned short* __restrict__ stSm) {
  using T = typename Word<ES>::T;
  using LT = typename Word<ES * LV>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* s = reinterpret_cast<T*>(smraw);
  long long bin, bout;
  decodeTile(p, blockIdx.x, bin, bout);
  auto ldOffset = [&](int u) -> int {
    if constexpr (NTR > 0)
      return arithInOffset<NTR>(p, (uint32_t)(u * LV));
    else
      return __ldg(ldOff + u);
  };
  // store units per thread: nOut <= NL * TILE_THREADS * LV / SV; up to two
  // are prefetched, except where the register pipeline already holds
  // NL >= 4 data words (measured slower there: C3b 2 % down)
  constexpr int NS = (NL * LV + SV - 1) / SV;
  constexpr int PF_MAX = (NL >= flatAsyncMinNL<ES>() || NL < 4) ? 2 : 0;
  constexpr int PF = NS < PF_MAX ? NS : PF_MAX;
  StorePrefetch<SV, (NTR == 0 ? PF : 0)> pf;
  ArithPrefetch<NTR, (NTR > 0 ? PF : 0)> apf;
  auto prefetch = [&] {
    if constexpr (NTR > 0)
      apf.template load<SV>(p);
    else
      pf.load(p, stOff, stSm);
  };
  if constexpr (NL >= flatAsyncMinNL<ES>()) {
    // many load units per thread: cp.async straight into shared memory
    // instead of NL data registers per thread
    const uint32_t sBase = (uint32_t)__cvta_generic_to_shared(s);
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int u = threadIdx.x + k * TILE_THREADS;
      if (u < p.nIn)
        cpAsyncUnit<ES * LV, LT_FLAT_L2_PREFETCH>(sBase + (uint32_t)smemIndex(p, u * LV) * ES,
                                                 in + bin + ldOffset(u));
    }
    prefetch();
    cpAsyncWaitAll();
  } else {
    LT v[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int u = threadIdx.x + k * TILE_THREADS;
      if (u < p.nIn) v[k] = *reinterpret_cast<const LT*>(in + bin + ldOffset(u));
    }
    prefetch();
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int u = threadIdx.x + k * TILE_THREADS;
      if (u < p.nIn) *reinterpret_cast<LT*>(s + smemIndex(p, u * LV)) = v[k];
    }
  }
  __syncthreads();
  if constexpr (NTR > 0)
    storeTileArith<ES, SV>(p, apf, s, out + bout);
  else
    storeTileFlat<ES, SV>(p, stOff, stSm, pf, s, out + bout);
}

// mbarrier and bulk-copy primitives (PTX ISA: mbarrier, cp.async.bulk).
__device__ __forceinline__ void mbarInit(uint32_t mb, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mb), "r"(count) : "memory");
}

// Makes an initialised mbarrier visible to the asynchronous proxy (the bulk
// copies that complete on it).
__device__ __forceinline__ void mbarInitFence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbarArriveExpectTx(uint32_t mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint32_t mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mb), "r"(parity)
      : "memory");
  return ok != 0;
}

// One bulk copy global -> shared (16-byte aligned addresses, size a
// multiple of 16) that completes `bytes` transactions on mbarrier mb.
__device__ __forceinline__ void bulkLoad(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t mb) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(mb)
      : "memory");
}

__device__ __forceinline__ unsigned long long globalTimerNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// Waits for phase `parity` of mbarrier mb for at most limitNs nanoseconds.
__device__ __forceinline__ bool mbarWaitBounded(uint32_t mb, uint32_t parity,
                                                unsigned long long limitNs) {
  if (mbarTryWait(mb, parity)) return true;
  const unsigned long long t0 = globalTimerNs();
  for (;;) {
    if (mbarTryWait(mb, parity)) return true;
    if (globalTimerNs() - t0 > limitNs) return false;
  }
}

constexpr unsigned long long BULK_WAIT_NS = 1000000000ull;  // 1 s

// Bulk-copy pipeline: the flat kernel with its load phase as bulk copies.
// The tile's input-order elements form segments of p.segLen elements, each
// contiguous in global memory (inside one input run) and in shared memory
// (between two padding gaps); segment k starts at tile element k * segLen,
// whose global offset is the load-unit table entry of that element.  The
// CTA's threads issue one cp.async.bulk per segment (no per-unit
// instruction, no data registers), all completing on one mbarrier that
// thread 0 arms with the tile's byte count; every thread then waits on it
// and the stores run as in the flat pipeline.  The wait is bounded: after
// BULK_WAIT_NS without completion the CTA writes the plan's tag p.statusTag
// to *status, waits once more (bounded) for its copies in flight, and
// returns without storing.
template <int ES, int LV, int SV, int NL, int NTR>
__global__ void __launch_bounds__(TILE_THREADS)
tileKernelBulk(const __grid_constant__ TileParams p, const typename Word<ES>::T* __restrict__ in,
               typename Word<ES>::T* __restrict__ out, const int* __restrict__ ldOff,
               const int* __restrict__ stOff, const unsigned short* __restrict__ stSm,
               unsigned* status) {
  static_assert(ES * LV == 16, "bulk copies need 16-byte load units");
  using T = typename Word<ES>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) unsigned long long bar;
  T* s = reinterpret_cast<T*>(smraw);
  long long bin, bout;
  decodeTile(p, blockIdx.x, bin, bout);
  const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&bar);
  const uint32_t sBase = (uint32_t)__cvta_generic_to_shared(s);
  if (threadIdx.x == 0) {
    mbarInit(mb, 1);
    mbarInitFence();
  }
  __syncthreads();
  const int L = p.segLen;
  const int nSeg = p.tileVol / L;
  const uint32_t segBytes = (uint32_t)(L * ES);
  const T* src = in + bin;
  for (int k = threadIdx.x; k < nSeg; k += TILE_THREADS) {
    const int j0 = k * L;
    int off;
    if constexpr (NTR > 0)
      off = arithInOffset<NTR>(p, (uint32_t)j0);
    else
      off = __ldg(ldOff + j0 / LV);
    bulkLoad(sBase + (uint32_t)smemIndex(p, j0) * ES, src + off, segBytes, mb);
  }
  if (threadIdx.x == 0) mbarArriveExpectTx(mb, (uint32_t)nSeg * segBytes + (uint32_t)p.testExtraTx);
  constexpr int NS = (NL * LV + SV - 1) / SV;
  constexpr int PF = NS < 2 ? NS : 2;
  StorePrefetch<SV, (NTR == 0 ? PF : 0)> pf;
  ArithPrefetch<NTR, (NTR > 0 ? PF : 0)> apf;
  if constexpr (NTR > 0)
    apf.template load<SV>(p);
  else
    pf.load(p, stOff, stSm);
  if (!mbarWaitBounded(mb, 0, BULK_WAIT_NS)) {
    if (threadIdx.x == 0) atomicExch(status, p.statusTag);
    mbarWaitBounded(mb, 0, BULK_WAIT_NS);  // copies in flight write this CTA's shared memory
    return;
  }
  if constexpr (NTR > 0)
    storeTileArith<ES, SV>(p, apf, s, out + bout);
  else
    storeTileFlat<ES, SV>(p, stOff, stSm, pf, s, out + bout);
}

// p + i * scale bytes.  With a scale the compiler cannot see (opaque), the
// offset is one wide integer multiply-add on the FMA pipe instead of a
// sign extension and a shift-add pair on the ALU pipe, which the grouped
// kernel's narrow units would otherwise saturate.
template <typename P>
__device__ __forceinline__ P* offsetBytes(P* p, int i, int scale) {
  using B = typename std::conditional<std::is_const<P>::value, const unsigned char,
                                      unsigned char>::type;
  return reinterpret_cast<P*>(reinterpret_cast<B*>(p) + (long long)i * scale);
}

// cp.async of one unit, issued only where live: the guard is a predicate on
// the instruction rather than a branch around it (the compiler cannot
// if-convert inline assembly, so a guarded asm costs a branch per slot).
template <int BYTES>
__device__ __forceinline__ void cpAsyncUnitIf(bool live, uint32_t dst, const void* src) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async unit");
#if LT_GROUP_L2_PREFETCH == 256
#define LT_GROUP_PF ".L2::256B"
#elif LT_GROUP_L2_PREFETCH == 128
#define LT_GROUP_PF ".L2::128B"
#else
#define LT_GROUP_PF ""
#endif
  if constexpr (BYTES == 16)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %2, 0;\n"
        " @p cp.async.cg.shared.global" LT_GROUP_PF " [%0], [%1], 16;\n}\n" ::"r"(dst),
        "l"(src), "r"((int)live)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %3, 0;\n"
        " @p cp.async.ca.shared.global" LT_GROUP_PF " [%0], [%1], %2;\n}\n" ::"r"(dst),
        "l"(src), "n"(BYTES), "r"((int)live)
        : "memory");
#undef LT_GROUP_PF
}

// Shared load where live (predicated as above); the result is undefined
// where not live.
template <int BYTES>
__device__ __forceinline__ typename Word<BYTES>::T ldSharedIf(bool live, uint32_t addr) {
  typename Word<BYTES>::T v;
  if constexpr (BYTES == 4) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %2, 0;\n @p ld.shared.b32 %0, [%1];\n}\n"
                 : "=r"(v)
                 : "r"(addr), "r"((int)live));
  } else if constexpr (BYTES == 8) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %3, 0;\n @p ld.shared.v2.b32 {%0, %1}, [%2];\n}\n"
        : "=r"(v.x), "=r"(v.y)
        : "r"(addr), "r"((int)live));
  } else {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
        " @p ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n}\n"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "r"(addr), "r"((int)live));
  }
  return v;
}

template <int BYTES>
__device__ __forceinline__ typename Word<BYTES>::T ldShared(uint32_t addr) {
  typename Word<BYTES>::T v;
  if constexpr (BYTES == 4) {
    asm volatile("ld.shared.b32 %0, [%1];\n" : "=r"(v) : "r"(addr));
  } else if constexpr (BYTES == 8) {
    asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];\n" : "=r"(v.x), "=r"(v.y) : "r"(addr));
  } else {
    asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(addr));
  }
  return v;
}

template <int BYTES>
__device__ __forceinline__ void stShared(uint32_t addr, const typename Word<BYTES>::T& v) {
  if constexpr (BYTES == 4) {
    asm volatile("st.shared.b32 [%0], %1;\n" ::"r"(addr), "r"(v) : "memory");
  } else if constexpr (BYTES == 8) {
    asm volatile("st.shared.v2.b32 [%0], {%1, %2};\n" ::"r"(addr), "r"(v.x), "r"(v.y) : "memory");
  } else {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(addr), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w)
                 : "memory");
  }
}

// Grouped flat kernel: CTA b moves one tile of tensor tileTensor[b] of a
// bucket; the tile list gives the tensor and the tile's corner offsets, the
// tensor's descriptor its pointers and run tables.  Unit
// offsets come from the run split (GroupTensor): a small table entry per
// run plus the position inside the run, so the tables stay in L1 even when
// consecutive CTAs belong to different tensors; when they are small enough
// the store-side tables are copied into shared memory with the data.  LOADS:
// 0 stages the load units in registers; 1 copies them with cp.async straight
// into shared memory (no data registers, so more CTAs fit an SM).  Every
// access stays inside the member's input and output tensors.
//
// Index arithmetic is kept off the ALU pipe where it can be: with element-
// size units the kernel does little else, and integer adds, shifts and
// compares issue at half the rate of multiply-adds.  Load slot k of a thread
// starts at tile element jT + k * B (B = TILE_THREADS * LV).  Padding puts
// 2^padLog elements after every 2^padShift, with padShift <= 8 <= log2(B) or
// padShift = 31 (none), so slot k's padded index is padT + k * padStep: one
// multiply-add per slot.  Byte offsets are multiply-adds by a scale the
// compiler cannot fold into shifts.
template <int ES, int LV, int SV, int NL, int LOADS>
__device__ __forceinline__ void groupTileBody(const GroupTensor* __restrict__ tens,
                                              const GroupTile* __restrict__ tiles,
                                              uint32_t tileIndex) {
  using T = typename Word<ES>::T;
  using LT = typename Word<ES * LV>::T;
  using ST = typename Word<ES * SV>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const longlong2 tile = __ldg(reinterpret_cast<const longlong2*>(tiles) + tileIndex);
  const GroupTensor* g = tens + (int)(tile.x >> GROUP_TILE_SHIFT);
  const long long bin = tile.x & ((1LL << GROUP_TILE_SHIFT) - 1), bout = tile.y;
  // shared memory: [store-side run tables, when staged][tile data]
  const int tabBytes = g->tabBytes;
  T* s = reinterpret_cast<T*>(smraw + tabBytes);
  const T* in = reinterpret_cast<const T*>(g->in) + bin;
  T* out = reinterpret_cast<T*>(g->out) + bout;
  const int* ldRow = g->ldRow;
  const RunDiv inRun = g->inRun;
  const int nIn = g->nIn, nOut = g->nOut, padShift = g->padShift, padLog = g->padLog;
  const uint32_t sBase = (uint32_t)__cvta_generic_to_shared(s);
  const int esR = opaque(ES);
  const int padMul = 1 << padLog;
  {
    constexpr int B = TILE_THREADS * LV;
    const int jT = threadIdx.x * LV;
    const int bR = opaque(B);
    const uint32_t dst0 = sBase + (uint32_t)((jT + (jT >> padShift) * padMul) * esR);
    const int stepBytes = (B + (B >> padShift) * padMul) * esR;
    const int uMax = nIn - threadIdx.x;  // slot k is live while k * TILE_THREADS < uMax
    const int inD = (int)inRun.d;
    const int four = opaque(4);
    const int jT1 = jT + 1;
    const T* inM1 = in - 1;  // indexed by a + 1
    const int ldStepB = g->ldStepBytes;
    // STEP: input runs evenly spaced (no table read on the load path)
    auto loadAll = [&](auto step) {
      constexpr bool STEP = decltype(step)::value;
      auto unitSrc = [&](int k) {
        // j + 1 = k * B + jT + 1; run r = j / inRun, a + 1 = j + 1 - r * inRun
        const int j1 = k * bR + jT1;
        const uint32_t r = __umulhi((uint32_t)j1, inRun.mul);
        const int a1 = j1 - (int)r * inD;
        const T* runBase;
        if constexpr (STEP)
          runBase = offsetBytes(inM1, (int)r, ldStepB);
        else
          runBase = offsetBytes(inM1, __ldg(offsetBytes(ldRow, (int)r, four)), esR);
        return reinterpret_cast<const LT*>(offsetBytes(runBase, a1, esR));
      };
      if constexpr (LOADS >= 1) {
#pragma unroll
        for (int k = 0; k < NL; ++k)
          if constexpr (STEP)  // the source is arithmetic only: predicate the copy
            cpAsyncUnitIf<ES * LV>(k * TILE_THREADS < uMax, dst0 + (uint32_t)(k * stepBytes),
                                   unitSrc(k));
          else if (k * TILE_THREADS < uMax)  // a dead slot's run would index past ldRow
            cpAsyncUnit<ES * LV>(dst0 + (uint32_t)(k * stepBytes), unitSrc(k));
        cpAsyncWaitAll();
      } else {
        LT v[NL];
#pragma unroll
        for (int k = 0; k < NL; ++k)
          if (k * TILE_THREADS < uMax) v[k] = *unitSrc(k);
#pragma unroll
        for (int k = 0; k < NL; ++k)
          if (k * TILE_THREADS < uMax) stShared<ES * LV>(dst0 + (uint32_t)(k * stepBytes), v[k]);
      }
    };
    if (ldStepB >= 0)
      loadAll(std::true_type{});
    else
      loadAll(std::false_type{});
  }
  if (tabBytes > 0) {
    // the store-side tables (outRows and smRun are contiguous, 16-byte
    // aligned) into shared memory, in flight with the data loads
    const uint32_t tBase = (uint32_t)__cvta_generic_to_shared(smraw);
    const unsigned char* src = reinterpret_cast<const unsigned char*>(g->outRows);
    for (int c = threadIdx.x; c < (tabBytes >> 4); c += TILE_THREADS)
      cpAsyncUnit<16>(tBase + 16u * c, src + 16 * c);
    cpAsyncWaitAll();
  }
  __syncthreads();
  const RunDiv outRun = g->outRun;
  const int outD = (int)outRun.d;
  const int qT1 = threadIdx.x * SV + 1;
  T* outM1 = out - 1;  // indexed by a + 1
  const int bQ = opaque(TILE_THREADS * SV);
  const int wMax = nOut - threadIdx.x;  // store slot i is live while i * TILE_THREADS < wMax
  const int padBytes = padMul * esR;
  // shared address of (unpadded) tile element x
  auto smAddr = [&](int x) { return sBase + (uint32_t)(x * esR + (x >> padShift) * padBytes); };
  // nOut <= NL * TILE_THREADS * LV / SV
  constexpr int NS = (NL * LV + SV - 1) / SV;
  constexpr int UNROLL = NS <= 16 ? NS : 8;
  // ROWS: output runs evenly spaced (no outRows read); POS: positions of a
  // run evenly spaced in the tile (no smRun read)
  const int outStepB = g->outStepBytes, rowSmStep = g->rowSmStep, smStep = g->smStep;
  auto storeAll = [&](auto rowsStepped, auto posStepped, const int2* outRows, const int* smRun) {
    constexpr bool ROWS = decltype(rowsStepped)::value;
    constexpr bool POS = decltype(posStepped)::value;
#pragma unroll UNROLL
    for (int i = 0; i < NS; ++i) {
      if (i * TILE_THREADS < wMax) {
        const int q1 = i * bQ + qT1;  // q + 1
        const uint32_t r = __umulhi((uint32_t)q1, outRun.mul);
        const int a1 = q1 - (int)r * outD;  // a + 1
        const int a = a1 - 1;
        ST* dst;
        int jb;
        if constexpr (ROWS) {
          dst = reinterpret_cast<ST*>(offsetBytes(offsetBytes(outM1, a1, esR), (int)r, outStepB));
          jb = (int)r * rowSmStep;
        } else {
          const int2 row = outRows[r];
          dst = reinterpret_cast<ST*>(offsetBytes(offsetBytes(outM1, a1, esR), row.x, esR));
          jb = row.y;
        }
        if constexpr (SV == 1) {
          if constexpr (POS)
            *dst = ldShared<ES>(smAddr(a * smStep + jb));
          else
            *dst = ldShared<ES>(smAddr(jb + smRun[a]));
        } else {
          T e[SV];
          if constexpr (POS) {
            const int x0 = a * smStep + jb;
#pragma unroll
            for (int c = 0; c < SV; ++c) e[c] = ldShared<ES>(smAddr(x0 + c * smStep));
          } else if constexpr (SV == 2) {
            const int2 jr = *reinterpret_cast<const int2*>(smRun + a);
            e[0] = ldShared<ES>(smAddr(jb + jr.x));
            e[1] = ldShared<ES>(smAddr(jb + jr.y));
          } else {
            const int4 jr = *reinterpret_cast<const int4*>(smRun + a);
            e[0] = ldShared<ES>(smAddr(jb + jr.x));
            e[1] = ldShared<ES>(smAddr(jb + jr.y));
            e[2] = ldShared<ES>(smAddr(jb + jr.z));
            e[3] = ldShared<ES>(smAddr(jb + jr.w));
          }
          ST val;
          __builtin_memcpy(&val, e, sizeof(ST));
          *dst = val;
        }
      }
    }
  };
  // tables that are read come from shared memory when staged, else from
  // device memory (two instantiations, so shared reads stay shared loads)
  auto withTables = [&](auto rowsStepped, auto posStepped) {
    if (tabBytes > 0) {
      const int* t = reinterpret_cast<const int*>(smraw);
      storeAll(rowsStepped, posStepped, reinterpret_cast<const int2*>(smraw), t + g->smRunOff);
    } else {
      storeAll(rowsStepped, posStepped, g->outRows, g->smRun);
    }
  };
  using Yes = std::true_type;
  using No = std::false_type;
  if (outStepB >= 0) {
    if (smStep >= 0)
      storeAll(Yes{}, Yes{}, nullptr, nullptr);
    else
      withTables(Yes{}, No{});
  } else {
    if (smStep >= 0)
      withTables(No{}, Yes{});
    else
      withTables(No{}, No{});
  }
}

// One tile of a group bucket per CTA (LOADS 0: loads through registers,
// 1: cp.async), or, with LOADS 2, persistent CTAs (grid = SMs x occupancy)
// that walk the bucket's tile list with a grid stride, cp.async loads.
template <int ES, int LV, int SV, int NL, int LOADS>
__global__ void __launch_bounds__(TILE_THREADS)
groupTileKernel(const GroupTensor* __restrict__ tens, const GroupTile* __restrict__ tiles,
                uint32_t numTiles) {
  if constexpr (LOADS == 2) {
    for (uint32_t t = blockIdx.x; t < numTiles; t += gridDim.x) {
      groupTileBody<ES, LV, SV, NL, 1>(tens, tiles, t);
      __syncthreads();  // the next tile reuses the shared buffers
    }
  } else {
    groupTileBody<ES, LV, SV, NL, LOADS>(tens, tiles, blockIdx.x);
  }
}

}  // namespace lt
