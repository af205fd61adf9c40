// Tile kernel instantiations for 16-byte elements: grouped execution.
#include "tile_kernel.cuh"
#define LT_ES 16
#define LT_GROUP_NAME launchGroupTile16
#include "tile_launch.inc"
