// Tile kernel instantiations for 4-byte elements: grouped execution with
// 8-byte load or store units.
#include "tile_kernel.cuh"
#define LT_ES 4
#define LT_GROUP_HALF_NAME launchGroupTile4Half
#include "tile_launch.inc"
