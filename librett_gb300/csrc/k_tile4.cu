// Tile kernel instantiations for 4-byte elements: single plans.
#include "tile_kernel.cuh"
#define LT_ES 4
#define LT_LAUNCH_NAME launchTile4
#define LT_FLAT_A launchFlat4A
#define LT_FLAT_B launchFlat4B
#define LT_FLAT_C launchFlat4C
#include "tile_launch.inc"
