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
// Trivial: contiguous copy in units of US bytes.  Each CTA copies one block
// of COPY_THREADS * COPY_UNROLL units (four independent loads per thread,
// issued before the stores) and exits; no grid-stride loop, so the block
// scheduler streams blocks through the SMs in address order.
// ---------------------------------------------------------------------------
constexpr int COPY_UNROLL = 4;

template <int US>
__global__ void __launch_bounds__(COPY_THREADS)
copyKernel(const typename Word<US>::T* __restrict__ in, typename Word<US>::T* __restrict__ out,
           long long n) {
  using T = typename Word<US>::T;
  const long long base = (long long)blockIdx.x * (COPY_THREADS * COPY_UNROLL) + threadIdx.x;
  T v[COPY_UNROLL];
#pragma unroll
  for (int u = 0; u < COPY_UNROLL; ++u)
    if (base + u * COPY_THREADS < n) v[u] = in[base + u * COPY_THREADS];
#pragma unroll
  for (int u = 0; u < COPY_UNROLL; ++u)
    if (base + u * COPY_THREADS < n) out[base + u * COPY_THREADS] = v[u];
}

// ---------------------------------------------------------------------------
// TiledCopy: input rank 0 is also output rank 0, so the tensor is a set of
// contiguous rows (dim[0] elements) that move to new row positions.  Work
// item = 32 units of one row.  Each CTA takes ROW_ITEMS_PER_CTA consecutive
// items (four per warp, loads issued before stores) and exits.
// ---------------------------------------------------------------------------
constexpr int ROW_ITEMS_PER_WARP = 4;
constexpr int ROW_ITEMS_PER_CTA = (ROW_THREADS / 32) * ROW_ITEMS_PER_WARP;

template <int US>
__global__ void __launch_bounds__(ROW_THREADS)
rowCopyKernel(const __grid_constant__ RowParams p, const typename Word<US>::T* __restrict__ in,
              typename Word<US>::T* __restrict__ out) {
  using T = typename Word<US>::T;
  const int lane = threadIdx.x & 31;
  const uint32_t first =
      blockIdx.x * ROW_ITEMS_PER_CTA + (threadIdx.x >> 5) * ROW_ITEMS_PER_WARP;
  T v[ROW_ITEMS_PER_WARP];
  long long dst[ROW_ITEMS_PER_WARP];
  bool ok[ROW_ITEMS_PER_WARP];
#pragma unroll
  for (int u = 0; u < ROW_ITEMS_PER_WARP; ++u) {
    const uint32_t item = first + u;
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
  for (int u = 0; u < ROW_ITEMS_PER_WARP; ++u)
    if (ok[u]) out[dst[u]] = v[u];
}

// Launch helpers (defined in the per-element-size translation units).
cudaError_t launchTile4(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                        cudaStream_t s, int numSMs, int* grid);
cudaError_t launchTile8(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                        cudaStream_t s, int numSMs, int* grid);
cudaError_t launchTile16(const PlanDesc& pd, const DeviceTables* dt, const void* in, void* out,
                         cudaStream_t s, int numSMs, int* grid);

}  // namespace lt
