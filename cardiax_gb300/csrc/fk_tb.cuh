// K2: temporally blocked Euler stepper (K steps per tile between one load and one store).
#pragma once
#include "fk_step.cuh"

namespace fk {

constexpr int kTbThreads = 512;  // one CTA per SM (the blocked tile fills shared memory)

// TMA descriptors of one blocked launch: the input planes u, v, w and D with the haloed box,
// and the output planes with the output-tile box.
struct TbMaps {
    CUtensorMap u, v, w, d, ov, ow, ou;
};

// Box (input, haloed) and output-tile sizes of the blocked kernel for depth 2, 4 or 8
// (zeros for other depths).
void tb_box(int depth, int *box_w, int *box_h, int *out_w, int *out_h);

// Steps t0 .. t0+depth-1 of the whole grid in one launch (depth 2, 4 or 8).
cudaError_t launch_tb(int depth, const TbMaps &maps, const StepArgs &a, int64_t t0,
                      cudaStream_t stream);

// ---- batched tissues, two steps per launch --------------------------------------------------
// Per tissue and ping-pong parity p: the blocked kernel's maps reading buffer p (0 = state,
// 1 = scratch) and writing buffer 1 - p.
struct BatchTbMaps {
    TbMaps maps[2];
};
constexpr int kBatchTbDepth = 2;    // steps per launch
constexpr int kBatchTbRows = 32;    // output tile: the batch's 32 x 64 work items
constexpr int kBatchTbCols = 64;
// Whether an H x W grid can be blocked (its last tile row and column hold more than one cell:
// the one-sided rows of a single-cell last row reach beyond the blocked halo).
inline bool tb_batchable(int64_t H, int64_t W) {
    return H % kBatchTbRows != 1 && W % kBatchTbCols != 1;
}
// Steps *t_dev + t_offset and the one after it of every tissue of a batch: CTA c (of `grid`,
// one per SM) takes items c, c + grid, ... of the 32 x 64 work list, reads buffer `parity` and
// writes the other one.
cudaError_t launch_batch_tb(const BatchTissue *tissues, const BatchTbMaps *maps,
                            const BatchItem *items, int n_items, const int *t_dev, int t_offset,
                            int parity, int *status, int grid, cudaStream_t stream);

}  // namespace fk
