// Tile kernel instantiations for 4-byte elements: grouped execution.
#include "tile_kernel.cuh"
#define LT_ES 4
#define LT_GROUP_NAME launchGroupTile4
#include "tile_launch.inc"
