// Grouped execution: many transposes of uneven shapes, permutations and
// element sizes in one CUDA graph (no LibreTT counterpart; LibreTT runs one
// kernel per librettExecute call, src/librett.cpp:372-385).
//
// Every member runs as a flat tile plan.  Members are bucketed by kernel
// shape (element size, load unit, store unit, load units per thread); each
// bucket is one launch over a device-resident descriptor table in which CTA
// b reads its tile (tensor index and corner offsets) and that tensor's
// descriptor (pointers, run tables).
//
// Which flat tile a member gets, and whether its bucket loads through
// registers or cp.async, is a policy per member class (size and element
// size); an autotuner
// (librettGroupTune) times the policies on the group's own buffers and keeps
// the fastest combination, cached by the batch's signature.  Buckets are
// also split by shared-memory size (4 KiB classes), so that a CTA reserves
// little more than its own tile needs.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace lt {

// Member classes of the tile-policy autotuner: 4 size classes (bytes of one
// tensor < 64 KiB, < 1 MiB, < 16 MiB, larger) x 3 element sizes (4, 8, 16);
// class = size class + 4 * log2(element bytes / 4).
constexpr int GROUP_CLASSES = 12;

struct GroupTensor {
  const unsigned char* in;
  unsigned char* out;
  const int* ldRow;  // [tileVol / inRun]  input offset of each input run
  // [tileVol / outRun] per output run: output offset, in-tile index of its
  // first element
  const int2* outRows;
  const int* smRun;  // [outRun] in-tile index of each element of an output run, from the first
  int nIn, nOut;       // load / store units of a tile
  RunDiv inRun, outRun;  // run lengths (in-tile indices are < 2^16)
  // Store-side tables staged in shared memory: their bytes (0 = read from
  // device memory) and the int offset of smRun inside them (outRows first).
  int tabBytes, smRunOff;
  int padShift, padLog;
  // input run r starts at r * ldStepBytes bytes from the tile corner when
  // >= 0 (evenly spaced runs; ldRow is then not read), else at ldRow[r]
  int ldStepBytes;
  // evenly spaced store-side tables (outRows / smRun then not read):
  // output run r at r * outStepBytes bytes and in-tile index r * rowSmStep
  // when outStepBytes >= 0; run position a at in-tile index a * smStep when
  // smStep >= 0
  int outStepBytes, rowSmStep, smStep;
};

// One tile of a bucket, written on the device at group creation: the
// element offset of its input corner with its tensor's descriptor index in
// the top 24 bits (offsets are < 2^40 elements), and the element offset of
// its output corner.  A CTA reads its tile with one 16-byte load instead of
// decoding the grid ranks.
struct GroupTile {
  long long inAndTensor;
  long long out;
};
constexpr int GROUP_TILE_SHIFT = 40;

// Run-table job for one member (written once, at group creation).
struct GroupTableJob {
  TileParams tp;
  GroupRunSplit rs;
  int* ldRow;
  int2* outRows;
  int* smRun;
  GroupTile* tiles;  // this member's tiles in its bucket's tile list
  long long tensor;  // descriptor index in the bucket
};

// Launch of one bucket's kernel (defined per element size in k_tile*.cu);
// loads: 0 registers, 1 cp.async (one tile per CTA), 2 cp.async with
// persistent CTAs (grid = numSMs x occupancy, a grid stride over the tiles).
cudaError_t launchGroupTile4(int lv, int sv, int nl, int loads, const GroupTensor* tens,
                             const GroupTile* tiles, uint32_t numTiles, int smem,
                             cudaStream_t s, int numSMs);
cudaError_t launchGroupTile8(int lv, int sv, int nl, int loads, const GroupTensor* tens,
                             const GroupTile* tiles, uint32_t numTiles, int smem,
                             cudaStream_t s, int numSMs);
cudaError_t launchGroupTile4Half(int lv, int sv, int nl, int loads, const GroupTensor* tens,
                                 const GroupTile* tiles, uint32_t numTiles, int smem,
                                 cudaStream_t s, int numSMs);
cudaError_t launchGroupTile16(int lv, int sv, int nl, int loads, const GroupTensor* tens,
                              const GroupTile* tiles, uint32_t numTiles, int smem,
                              cudaStream_t s, int numSMs);

}  // namespace lt
