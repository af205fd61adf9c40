// Tile kernel instantiations for 8-byte elements: single plans.
#include "tile_kernel.cuh"
#define LT_ES 8
#define LT_LAUNCH_NAME launchTile8
#define LT_FLAT_A launchFlat8A
#define LT_FLAT_B launchFlat8B
#define LT_FLAT_C launchFlat8C
#include "tile_launch.inc"
