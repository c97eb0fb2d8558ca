// The batched kernel with 16 x 64-cell tiles: half the rows per work item, so twice the items
// (finer load balance, smaller tissues fill more CTAs) at a larger halo share (24 u rows loaded
// per 16 computed instead of 40 per 32); one row of four cells per thread in pass 2.
#define FK_TILE_Y 16
#define FK_TILE_NS fk_rows16
#define FK_TILE_NS_VARIANT 1
#define FK_BATCH_LAUNCHER fk_batch_launch_rows16
#include "fk_batch_kernel.cuh"
