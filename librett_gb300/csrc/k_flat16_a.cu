// Flat and bulk-copy tile kernels for 16-byte elements, tiles of 0..2 ranks (0: offset tables).
#define LT_ES 16
#define LT_NTR_LO 0
#define LT_NTR_HI 2
#define LT_FLAT_NAME launchFlat16A
#include "tile_flat.inc"
