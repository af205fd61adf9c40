// Flat and bulk-copy tile kernels for 4-byte elements, tiles of 3..4 ranks.
#define LT_ES 4
#define LT_NTR_LO 3
#define LT_NTR_HI 4
#define LT_FLAT_NAME launchFlat4B
#include "tile_flat.inc"
