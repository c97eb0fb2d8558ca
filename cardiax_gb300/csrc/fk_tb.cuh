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

}  // namespace fk
