// Rotated stimulus fields on the device: cardiax/stimulus.py:109-140 (triangular), which
// rotates a `linear` stripe with scipy.ndimage.rotate(field, angle, mode="nearest",
// prefilter=False, reshape=False).
//
// The restated algorithm (SciPy's published one, order-3 spline without prefilter): output
// (i, j) samples input coordinates (x, y) = R (i, j) + o about the array centre, with
// R = [[c, s], [-s, c]] (c, s the cosine and sine of the angle in degrees) and
// o = (n - 1)/2 - R (n - 1)/2; the value is sum_{a,b} B3(x - k_a) B3(y - l_b) f[k_a][l_b] over the
// 4 x 4 integer nodes around (x, y), B3 the cubic B-spline, f's indices clamped to the array
// (the "nearest" extension; without prefilter the samples are the spline coefficients).
// Coordinates and weights are computed in double, as SciPy does, and the result is rounded to
// float32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/cardiax_gb300.h"

namespace fk {

namespace {

__device__ __forceinline__ double bspline3(double t) {
    t = fabs(t);
    if (t < 1.0) return 2.0 / 3.0 - t * t + 0.5 * t * t * t;
    if (t < 2.0) {
        const double u = 2.0 - t;
        return u * u * u / 6.0;
    }
    return 0.0;
}

__global__ void fk_rotate_kernel(const float *__restrict__ in, int H, int W, int64_t pitch,
                                 float *__restrict__ out, int64_t out_pitch, double c, double s,
                                 double o0, double o1) {
    const int64_t n = (int64_t)H * W;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / W), j = (int)(k % W);
        const double x = c * i + s * j + o0;
        const double y = -s * i + c * j + o1;
        const int i0 = (int)floor(x) - 1, j0 = (int)floor(y) - 1;
        double acc = 0.0;
        for (int p = 0; p < 4; ++p) {
            const double wx = bspline3(x - (double)(i0 + p));
            const int ii = min(max(i0 + p, 0), H - 1);
            for (int q = 0; q < 4; ++q) {
                const int jj = min(max(j0 + q, 0), W - 1);
                acc += wx * bspline3(y - (double)(j0 + q)) * (double)__ldg(in + (int64_t)ii * pitch + jj);
            }
        }
        out[(int64_t)i * out_pitch + j] = (float)acc;
    }
}

// cos and sin of an angle in degrees, exact at multiples of 90
void cos_sin_deg(double deg, double *c, double *s) {
    double r = std::fmod(deg, 360.0);
    if (r < 0) r += 360.0;
    if (r == 0.0) { *c = 1; *s = 0; return; }
    if (r == 90.0) { *c = 0; *s = 1; return; }
    if (r == 180.0) { *c = -1; *s = 0; return; }
    if (r == 270.0) { *c = 0; *s = -1; return; }
    const double a = deg * (M_PI / 180.0);
    *c = std::cos(a);
    *s = std::sin(a);
}

}  // namespace

}  // namespace fk

extern "C" int fk_rotate_field(const float *in, int64_t H, int64_t W, int64_t pitch, float *out,
                               int64_t out_pitch, double angle_deg, void *stream) {
    if (!in || !out) return FK_ERR_NULL;
    if (H < 1 || W < 1 || pitch < W || out_pitch < W || H > (1 << 30) || W > (1 << 30))
        return FK_ERR_SHAPE;
    if (!std::isfinite(angle_deg)) return FK_ERR_ARGUMENT;
    if (in == out) return FK_ERR_ARGUMENT;
    double c, s;
    fk::cos_sin_deg(angle_deg, &c, &s);
    const double ch = (double)(H - 1) / 2.0, cw = (double)(W - 1) / 2.0;
    const double o0 = ch - (c * ch + s * cw), o1 = cw - (-s * ch + c * cw);
    const int64_t n = H * W;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    fk::fk_rotate_kernel<<<(unsigned)(blocks < 65536 ? blocks : 65536), threads, 0,
                           (cudaStream_t)stream>>>(in, (int)H, (int)W, pitch, out, out_pitch, c,
                                                   s, o0, o1);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}
