// Tile kernel instantiations for 16-byte elements: single plans.
#include "tile_kernel.cuh"
#define LT_ES 16
#define LT_LAUNCH_NAME launchTile16
#define LT_FLAT_A launchFlat16A
#define LT_FLAT_B launchFlat16B
#define LT_FLAT_C launchFlat16C
#include "tile_launch.inc"
