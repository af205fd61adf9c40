// Flat and bulk-copy tile kernels for 8-byte elements, tiles of 5..6 ranks.
#define LT_ES 8
#define LT_NTR_LO 5
#define LT_NTR_HI 6
#define LT_FLAT_NAME launchFlat8C
#include "tile_flat.inc"
