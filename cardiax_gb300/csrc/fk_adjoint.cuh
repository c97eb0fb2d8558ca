// Adjoint (reverse-mode) Euler step: declarations.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "fk_math.cuh"

namespace fk {

constexpr int kAdjParams = 13;       // differentiable parameters (cardiax/params.py fields 0..12)
constexpr int kAdjParamStride = 16;  // doubles per gradient slot
constexpr int ADJ_BAND = 6;          // cells this close to an edge use the explicit transposes

struct AdjointArgs {
    const float *u, *v, *w, *D;        // state x_t and diffusivity
    const float *lu, *lv, *lw;         // cotangent of x_{t+1}
    float *olu, *olv, *olw;            // cotangent of x_t (separate buffers)
    float *gD;                         // += dL/dD (null: not accumulated)
    double *gtheta;                    // += per-block partial dL/dtheta (null: not accumulated)
    int H, W, pitch;
    float t, dt, rdx;
    int n_stim;
    Model m;
    Stim stim[kMaxStim];
};

// Number of dL/dtheta slots (kAdjParamStride doubles each) written by launch_adjoint.
int64_t adjoint_slots(int H, int W);
cudaError_t launch_adjoint(const AdjointArgs &a, cudaStream_t stream);
// Reverse step k of a segment for n_exp experiments of the same H x W grid (device descriptors
// `exps`, see fk_adjoint_batch_kernel); parity selects the cotangent buffer read.
cudaError_t launch_adjoint_batch(const AdjointArgs *exps, int n_exp, int H, int W, int64_t k_stride,
                                 int k, int parity, float t, cudaStream_t stream);

}  // namespace fk
