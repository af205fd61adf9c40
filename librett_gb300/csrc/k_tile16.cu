// Tile kernel instantiations for 16-byte elements.
#include "tile_kernel.cuh"
#define LT_ES 16
#define LT_LAUNCH_NAME launchTile16
#define LT_GROUP_NAME launchGroupTile16
#include "tile_launch.inc"
