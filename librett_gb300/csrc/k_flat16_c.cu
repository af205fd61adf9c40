// Flat and bulk-copy tile kernels for 16-byte elements, tiles of 5..6 ranks.
#define LT_ES 16
#define LT_NTR_LO 5
#define LT_NTR_HI 6
#define LT_FLAT_NAME launchFlat16C
#include "tile_flat.inc"
