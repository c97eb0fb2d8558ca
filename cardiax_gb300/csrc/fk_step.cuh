// Fused Fenton-Karma Euler step on one tissue: kernel declarations and shared tile geometry.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "fk_math.cuh"

// The tile geometry below is compile-time.  A translation unit that builds the batched kernel
// for another tile shape defines FK_TILE_Y / FK_TILE_X (and FK_CTAS_PER_SM) together with
// FK_TILE_NS, the namespace that the geometry-dependent code of this header and of fk_tile.cuh
// then lives in (the geometry-independent code of fk_math.cuh, fk_pack.cuh and fk_ptx.cuh stays
// in namespace fk), so that the variants do not collide.
#ifndef FK_TILE_NS
#define FK_TILE_NS fk
#endif
namespace FK_TILE_NS {
#ifdef FK_TILE_NS_VARIANT
using namespace fk;
#endif

// Tile geometry of the step kernel.  Persistent CTAs of NT threads (two per SM) walk over
// TY x TX tiles with a three-stage TMA ring for the haloed u and D tiles (the loads of tiles
// n+1 and n+2 are in flight while tile n is computed); v and w are read straight into
// registers at the start of each tile, and the new state goes out through TMA stores from
// dedicated output tiles.
//   pass 1: u_x on rows -2 .. TY+1 and u_y on columns -2 .. TX+1 go to shared memory;
//   pass 2: thread (tx, ty) owns columns 4tx .. 4tx+3 of rows RPT*ty .. RPT*ty+RPT-1.
#ifndef FK_TILE_X
#define FK_TILE_X 64
#endif
#ifndef FK_TILE_Y
#define FK_TILE_Y 32
#endif
#ifndef FK_THREADS
#define FK_THREADS 256
#endif
#ifndef FK_PASS1_UNROLL
#define FK_PASS1_UNROLL 1
#endif
constexpr int TX = FK_TILE_X;
constexpr int TY = FK_TILE_Y;
constexpr int NT = FK_THREADS;
#ifdef FK_CTAS_PER_SM
constexpr int CTAS_PER_SM = FK_CTAS_PER_SM;
#else
constexpr int CTAS_PER_SM = NT <= 256 ? 2 : 1;
#endif
constexpr int PASS1_UNROLL = FK_PASS1_UNROLL;
constexpr int NTX = TX / 4;          // float4 columns
constexpr int RPT = TY / (NT / NTX); // rows per thread in pass 2
constexpr int NSTAGE = 3;
constexpr int HALO_U = 4;  // u_xx composes two radius-2 derivatives
constexpr int HALO_D = 2;  // D_x is one radius-2 derivative
constexpr int SW = TX + 2 * HALO_U;   // row width of the u, D and u_y tiles (16-byte multiple)
constexpr int SU_H = TY + 2 * HALO_U;
constexpr int SD_H = TY + 2 * HALO_D;
constexpr int SUX_H = TY + 4;         // u_x rows -2 .. TY+1
constexpr int SMEM_U_BYTES = SW * SU_H * 4;
constexpr int SMEM_D_BYTES = SW * SD_H * 4;
constexpr int SMEM_STAGE_BYTES = SMEM_U_BYTES + SMEM_D_BYTES;
constexpr int SMEM_UX_BYTES = TX * SUX_H * 4;
constexpr int SMEM_UY_BYTES = SW * TY * 4;
constexpr int SMEM_PLANE_BYTES = TX * TY * 4;     // one dense output plane
constexpr int SMEM_ARGS_BYTES = 1024;  // staged StepArgs (static_assert in fk_step.cu)
constexpr int SMEM_STEP_BYTES = NSTAGE * SMEM_STAGE_BYTES + SMEM_UX_BYTES + SMEM_UY_BYTES +
                                3 * SMEM_PLANE_BYTES + 8 * NSTAGE + SMEM_ARGS_BYTES + 128;
// fk_step_kernel: no output tiles (the new state is stored from registers), u_x and u_y
// double-buffered
constexpr int SMEM_STEP_DIRECT_BYTES = NSTAGE * SMEM_STAGE_BYTES + 2 * (SMEM_UX_BYTES + SMEM_UY_BYTES) +
                                       8 * NSTAGE + SMEM_ARGS_BYTES + 128;
// Cells within this distance of an edge take the per-cell boundary path (one-sided stencils
// and edge padding reach 4 cells in).
constexpr int BAND = 4;

// Arguments of one step over one tissue.  Planes are H rows of `pitch` floats; the state is
// three planes (v, w, u) in the reference's State order.
struct StepArgs {
    const float *u, *v, *w, *D;
    float *uo, *vo, *wo;
    int H, W, pitch;
    float t, dt, rdx;
    int n_stim;
    Model m;
    Stim stim[kMaxStim];
    int *status;  // device error word: set on a barrier timeout
    // activation tracking (upstrokes of u through `act_threshold`); null when off
    int32_t *act_first, *act_last, *act_count;
    float act_threshold;
    // nonzero: the step's live data (the new state and D) fits in L2, so the step kernel marks
    // the input state's reads evict-first and D's evict-last (set by the host per device)
    int l2_hints;
    // Heun stages (cardiax/solve.py:73-85; fk_step_kernel only).  Stage 1 is the Euler step
    // x1 = x + dt d1 that also stores d1 = f(x, t) to `dso`; stage 2 reads x1 (the input state),
    // x0 = x and d1, and writes x0 + (d1 + f(x1, t)) h with h = dt / 2.  Three planes each.
    float *dso;
    const float *x0, *d1;
    float h;
};

enum : int { kStatusTimeout = 1 };

// TMA descriptors of one step: u (box SW x SU_H) of the input state, D (box SW x SD_H), and
// the three planes of the output state (box TX x TY, for the stores).
struct StepMaps {
    CUtensorMap u, d, ov, ow, ou;
};

// Launches one step (Euler update, or the derivative when `deriv`).  With a.act_last set, the
// Euler step also records activations: a cell whose u goes from below the threshold to at or
// above it during step t -> t+1 gets act_last = t+1, act_first = t+1 if it was -1, and
// act_count + 1.
cudaError_t launch_step(const StepMaps &maps, const StepArgs &a, bool deriv, cudaStream_t stream,
                        int heun = 0);
// Whether one step's live data on an H x pitch grid fits in L2 (sets StepArgs::l2_hints).
bool l2_fits_step(int64_t H, int64_t pitch);

// ---- batched tissues ------------------------------------------------------------------------
// Device-resident descriptors of one tissue in a batch: the step arguments and TMA maps for
// both ping-pong parities (parity p reads buffer p: 0 = state, 1 = scratch).
struct BatchTissue {
    StepArgs args[2];
};
struct BatchMaps {
    StepMaps maps[2];
};
// One unit of the work list: a TY x TX tile of one tissue.
struct BatchItem {
    int32_t tissue, i0, j0, pad;
};

constexpr int SMEM_BATCH_BYTES = SMEM_STEP_DIRECT_BYTES + SMEM_ARGS_BYTES;  // two argument slots

// One Euler step of every tissue: CTA c (of `grid`) processes items c, c + grid, ... when
// `interleave`, else items[ranges[c] .. ranges[c+1]); `packed` selects the packed arithmetic.
// The step index is *t_dev + t_offset (so that a captured graph can be replayed for successive
// steps).  n_items == 0 only configures the kernel (no launch).
cudaError_t launch_batch_step(const BatchTissue *tissues, const BatchMaps *maps,
                              const BatchItem *items, const int *ranges, int n_items,
                              int interleave, int packed, const int *t_dev, int t_offset,
                              int parity, bool act, int *status, int grid, cudaStream_t stream);
// The most CTAs a batched launch may use (the size of a plan's range table).
constexpr int kBatchMaxGrid = 4096;
// *p += v (advances the step counter of a captured graph).
cudaError_t launch_add_int(int *p, int v, cudaStream_t stream);
// Copies buffer 1 (scratch) of every tissue back to buffer 0 (state).
cudaError_t launch_batch_copyback(const BatchTissue *tissues, int n_tissues, cudaStream_t stream);

// ---- dataflow kernel: many steps of one tissue in one cooperative launch ----------------------
// Step k of the launch reads `src` (k = 0) or buffer (k-1)&1 and writes buffer k&1.  Tile T of
// step k starts once T and its eight neighbours have finished step k-1: each tile publishes the
// number of steps it has completed in flags[T] (flags[ntiles] is an abort word).
struct FlowMaps {
    CUtensorMap d;
    CUtensorMap uin[3];                  // u halo box of src, buffer 0, buffer 1
    CUtensorMap ov[2], ow[2], ou[2];     // store boxes of buffer 0, buffer 1
};
struct FlowArgs {
    StepArgs in[3];   // per input buffer (src, buffer 0, buffer 1): the planes read
    int64_t t0;       // step index of the launch's first step
    int nsteps;
    int *flags;       // ntiles + 1 zeroed words
};
constexpr int SMEM_FLOW_BYTES = SMEM_STEP_BYTES + 2 * SMEM_ARGS_BYTES;
// Number of int32 flag words the dataflow kernel needs for an H x W grid.
inline int64_t flow_flag_words(int64_t H, int64_t W) {
    return ((H + TY - 1) / TY) * ((W + TX - 1) / TX) + 1;
}
// Launches the dataflow kernel (cooperative: every CTA resident).  `act` selects activation
// tracking (FlowArgs::in[*].act_* set).
cudaError_t launch_flow(const FlowMaps &maps, const FlowArgs &a, bool act, cudaStream_t stream);

}  // namespace FK_TILE_NS
