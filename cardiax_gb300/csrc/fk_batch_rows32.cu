// The batched kernel with 32 x 64-cell tiles (the default geometry of fk_step.cuh).
#define FK_BATCH_LAUNCHER fk_batch_launch_rows32
#include "fk_batch_kernel.cuh"
