// Strip kernel: the fused Fenton-Karma Euler step written around Blackwell's packed FP32
// instructions, for the single-tissue stepper.
//
// Geometry.  The grid is cut into strips of S_TX = 128 columns (one warp-row: 32 lanes x 4
// columns) and tiles of S_TY rows.  Persistent CTAs of S_WARPS warps walk the tiles; a TMA ring
// of S_NSTAGE stages brings each tile's u (rows -5 .. S_TY+3, columns -4 .. 131) and D (rows
// -3 .. S_TY+1) into shared memory.  Warp w owns rows S_RPW*w .. S_RPW*w + S_RPW-1 of the tile
// and walks them top to bottom with register windows of u_x and D (the x-direction stencils
// never touch shared memory twice for the same row), reads its row of u with three 16-byte
// loads for the y-direction stencils, and stores v, w, u with 16-byte global stores.  v and w
// are read straight into registers before the tile's TMA wait.
//
// Arithmetic: pairs of cells per instruction (fk_pack.cuh), bit-identical to fk_step_kernel.
// Edges: tiles within 4 cells of a grid edge replace the zero fill of their out-of-grid halo by
// the reference's edge padding in shared memory, and pick the one-sided stencil rows per row
// (uniform across a warp) and per column (in the lanes at an edge).
#pragma once
#include "fk_pack.cuh"
#include "fk_step.cuh"

namespace fk {

#ifndef FK_STRIP_RPW
#define FK_STRIP_RPW 4
#endif
#ifndef FK_STRIP_WARPS
#define FK_STRIP_WARPS 8
#endif
#ifndef FK_STRIP_STAGES
#define FK_STRIP_STAGES 2
#endif
constexpr int S_TX = 128;
constexpr int S_WARPS = FK_STRIP_WARPS;
constexpr int S_NT = 32 * S_WARPS;
constexpr int S_RPW = FK_STRIP_RPW;
constexpr int S_TY = S_WARPS * S_RPW;
constexpr int S_NSTAGE = FK_STRIP_STAGES;
constexpr int S_HC = 4;                      // halo columns on each side
constexpr int S_HU_TOP = 5, S_HU_BOT = 4;    // u rows above / below the tile
constexpr int S_HD_TOP = 3, S_HD_BOT = 2;    // D rows above / below the tile
constexpr int S_SW = S_TX + 2 * S_HC;        // 136 floats per shared row
constexpr int S_UH = S_TY + S_HU_TOP + S_HU_BOT;
constexpr int S_DH = S_TY + S_HD_TOP + S_HD_BOT;
constexpr int S_U_TX = S_SW * S_UH * 4;      // bytes a u box delivers
constexpr int S_D_TX = S_SW * S_DH * 4;
constexpr int S_U_BYTES = (S_U_TX + 127) / 128 * 128;
constexpr int S_D_BYTES = (S_D_TX + 127) / 128 * 128;
constexpr int S_STAGE_BYTES = S_U_BYTES + S_D_BYTES;
constexpr int S_SMEM_BYTES = S_NSTAGE * S_STAGE_BYTES + 8 * S_NSTAGE + 128;
constexpr int S_CTAS_PER_SM = (S_SMEM_BYTES + 1024) * 2 <= 227 * 1024 && S_NT <= 512 ? 2 : 1;

// TMA descriptors: the u plane of the input state (box S_SW x S_UH) and D (box S_SW x S_DH).
struct StripMaps {
    CUtensorMap u, d;
};

// The strip kernel handles every grid except one whose last strip is a single column
// (W = 1 mod 128): the one-sided stencil of that column reaches past the lanes of its warp.
inline bool strip_eligible(int64_t H, int64_t W) { return H >= 3 && W >= 3 && W % S_TX != 1; }

// One Euler step (not the derivative) from a.u/v/w to a.uo/vo/wo, with activation tracking when
// a.act_last is set.
cudaError_t launch_strip(const StripMaps &maps, const StepArgs &a, cudaStream_t stream);

}  // namespace fk
