// Flat and bulk-copy tile kernels for 8-byte elements, tiles of 3..4 ranks.
#define LT_ES 8
#define LT_NTR_LO 3
#define LT_NTR_HI 4
#define LT_FLAT_NAME launchFlat8B
#include "tile_flat.inc"
