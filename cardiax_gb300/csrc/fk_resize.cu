// Bilinear resize of state planes: cardiax/io.py:118-124 (imresize), used by the data-generation
// caller deepx/generate.py:187-199 on every checkpoint.
//
// The reference calls jax.image.resize(a, shape, "bilinear") (JAX is a dependency pinned through
// jaxlib 0.1.64 in install_jax.sh and not vendored).  Its published algorithm, restated here:
// each resized axis is resampled independently with the triangle kernel k(x) = max(0, 1 - |x|)
// at half-pixel centres: output index p samples input coordinate
//     s(p) = (p + 0.5) / scale - 0.5,   scale = out_size / in_size,
// with weights w_i = k(|s(p) - i| / ks), ks = max(1 / scale, 1) when antialiasing (the kernel
// is widened when downsampling) and 1 otherwise, normalised to sum 1 over i.  An axis whose size
// does not change is left alone (the weights are then the identity).
//
// One thread per output value; the weights are recomputed in the kernel (no scratch memory), in
// float32 as the reference's weight matrices are.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/cardiax_gb300.h"

namespace fk {

namespace {

struct Axis {
    float inv_scale, ks;
    int n_in;
    // input range and weight sum for output index p
    __device__ __forceinline__ float sample(int p) const {
        return ((float)p + 0.5f) * inv_scale - 0.5f;
    }
    __device__ __forceinline__ void range(float s, int &lo, int &hi) const {
        lo = max(0, (int)ceilf(s - ks));
        hi = min(n_in - 1, (int)floorf(s + ks));
    }
    __device__ __forceinline__ float weight(float s, int i) const {
        return fmaxf(0.0f, 1.0f - fabsf(s - (float)i) / ks);
    }
};

Axis make_axis(int64_t n_in, int64_t n_out, bool antialias) {
    const double scale = (double)n_out / (double)n_in;
    Axis a;
    a.inv_scale = (float)(1.0 / scale);
    a.ks = antialias ? std::fmax(a.inv_scale, 1.0f) : 1.0f;
    a.n_in = (int)n_in;
    return a;
}

__global__ void fk_resize_kernel(const float *__restrict__ in, int64_t in_pitch, int64_t in_plane,
                                 float *__restrict__ out, int64_t out_pitch, int64_t out_plane,
                                 int planes, int OH, int OW, Axis ay, Axis ax) {
    const int64_t n = (int64_t)planes * OH * OW;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(k % OW);
        const int p = (int)((k / OW) % OH);
        const int c = (int)(k / ((int64_t)OW * OH));
        const float sy = ay.sample(p), sx = ax.sample(q);
        int i0, i1, j0, j1;
        ay.range(sy, i0, i1);
        ax.range(sx, j0, j1);
        float wy_sum = 0.0f, wx_sum = 0.0f;
        for (int i = i0; i <= i1; ++i) wy_sum += ay.weight(sy, i);
        for (int j = j0; j <= j1; ++j) wx_sum += ax.weight(sx, j);
        const float *src = in + (int64_t)c * in_plane;
        float acc = 0.0f;
        if (wy_sum > 1000.0f * 1.1920929e-7f && wx_sum > 1000.0f * 1.1920929e-7f) {
            for (int i = i0; i <= i1; ++i) {
                const float wy = ay.weight(sy, i) / wy_sum;
                if (wy == 0.0f) continue;
                const float *row = src + (int64_t)i * in_pitch;
                float r = 0.0f;
                for (int j = j0; j <= j1; ++j) r = fmaf(ax.weight(sx, j) / wx_sum, __ldg(row + j), r);
                acc = fmaf(wy, r, acc);
            }
        }
        out[(int64_t)c * out_plane + (int64_t)p * out_pitch + q] = acc;
    }
}

}  // namespace

}  // namespace fk

extern "C" int fk_resize_bilinear(const float *in, int64_t planes, int64_t H, int64_t W,
                                  int64_t in_pitch, float *out, int64_t OH, int64_t OW,
                                  int64_t out_pitch, int antialias, void *stream) {
    if (!in || !out) return FK_ERR_NULL;
    if (planes < 1 || H < 1 || W < 1 || OH < 1 || OW < 1 || in_pitch < W || out_pitch < OW)
        return FK_ERR_SHAPE;
    if (planes * OH * OW > ((int64_t)1 << 40) || H > (1 << 30) || W > (1 << 30) ||
        OH > (1 << 30) || OW > (1 << 30))
        return FK_ERR_SHAPE;
    const fk::Axis ay = fk::make_axis(H, OH, antialias != 0);
    const fk::Axis ax = fk::make_axis(W, OW, antialias != 0);
    const int64_t n = planes * OH * OW;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    fk::fk_resize_kernel<<<(unsigned)(blocks < 65536 ? blocks : 65536), threads, 0,
                           (cudaStream_t)stream>>>(in, in_pitch, H * in_pitch, out, out_pitch,
                                                   OH * out_pitch, (int)planes, (int)OH, (int)OW,
                                                   ay, ax);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}
