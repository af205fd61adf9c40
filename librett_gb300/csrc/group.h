// Grouped execution: many transposes of uneven shapes, permutations and
// element sizes in one CUDA graph (no LibreTT counterpart; LibreTT runs one
// kernel per librettExecute call, src/librett.cpp:372-385).
//
// Every member runs as a flat tile plan.  Members are bucketed by kernel
// shape (element size, load unit, store unit, load units per thread); each
// bucket is one launch over a device-resident descriptor table in which CTA
// b looks up its tensor (tileTensor[b]) and that tensor's descriptor
// (pointers, offset tables, grid-rank decode).  Members that do not fit the
// compact descriptor run with their own launch inside the same graph.
//
// Which flat tile a member gets is a policy per member size class; an
// autotuner (librettGroupTune) times the policies on the group's own buffers
// and keeps the fastest combination, cached by the batch's signature.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace lt {

constexpr int GROUP_MAXG = 8;     // grid ranks a compact descriptor holds
constexpr int GROUP_CLASSES = 4;  // member size classes of the tile-policy autotuner

struct GroupTensor {
  const unsigned char* in;
  unsigned char* out;
  const int* ldOff;
  const int* stOff;
  const unsigned short* stSm;
  uint32_t firstTile;  // index of this tensor's first tile in the bucket
  int nIn, nOut;
  int padShift, padLog;
  int nGR;
  FastDiv grDiv[GROUP_MAXG];
  long long grSin[GROUP_MAXG], grSout[GROUP_MAXG];
  long long grLastIn[GROUP_MAXG], grLastOut[GROUP_MAXG];
};

// Offset-table job for one member (written once, at group creation).
struct GroupTableJob {
  TileParams tp;
  int* ldOff;
  int* stOff;
  unsigned short* stSm;
};

// Launch of one bucket's kernel (defined per element size in k_tile*.cu).
cudaError_t launchGroupTile4(int lv, int sv, int nl, const GroupTensor* tens,
                             const int* tileTensor, uint32_t numTiles, int smem, cudaStream_t s);
cudaError_t launchGroupTile8(int lv, int sv, int nl, const GroupTensor* tens,
                             const int* tileTensor, uint32_t numTiles, int smem, cudaStream_t s);
cudaError_t launchGroupTile16(int lv, int sv, int nl, const GroupTensor* tens,
                              const int* tileTensor, uint32_t numTiles, int smem, cudaStream_t s);

}  // namespace lt
