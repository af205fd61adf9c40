// Tile kernel instantiations for 8-byte elements: grouped execution.
#include "tile_kernel.cuh"
#define LT_ES 8
#define LT_GROUP_NAME launchGroupTile8
#include "tile_launch.inc"
