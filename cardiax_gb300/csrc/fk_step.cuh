// Fused Fenton-Karma Euler step on one tissue: kernel declarations and shared tile geometry.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "fk_math.cuh"

namespace fk {

// Tile geometry of the single-step kernel: a CTA owns TY x TX cells; each thread owns a
// 4-column x MR-row micro-tile (float4 columns, MR rows streamed top to bottom).
constexpr int TX = 128;
constexpr int TY = 32;
constexpr int MR = 8;
constexpr int NTX = TX / 4;
constexpr int NTY = TY / MR;
constexpr int NT = NTX * NTY;
constexpr int HALO_U = 4;  // u_xx composes two radius-2 derivatives
constexpr int HALO_D = 2;  // D_x is one radius-2 derivative
constexpr int SU_W = TX + 2 * HALO_U;   // u box width (also used for D: 16-byte alignment)
constexpr int SU_H = TY + 2 * HALO_U;
constexpr int SD_H = TY + 2 * HALO_D;
constexpr int SMEM_U_BYTES = SU_W * SU_H * 4;
constexpr int SMEM_D_BYTES = SU_W * SD_H * 4;
constexpr int SMEM_STEP_BYTES = SMEM_U_BYTES + SMEM_D_BYTES + 16 + 128;  // + mbarrier + align
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
};

enum : int { kStatusTimeout = 1 };

// Launches one step (Euler update, or the derivative when `deriv`).
cudaError_t launch_step(const CUtensorMap &tm_u, const CUtensorMap &tm_d, const StepArgs &a,
                        bool deriv, cudaStream_t stream);

}  // namespace fk
