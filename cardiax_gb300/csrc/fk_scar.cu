// Scar maps for the diffusivity field: the field-sized steps of
// deepx/utils_scars.py:409-426 (random_diffusivity_scar).
//
// fk_scar_raster  -- the union of filled polygons (utils_scars.py:79-97 drawpolyintoemptycanvas
//                    through skimage.draw.polygon, summed and clipped at 1 in
//                    utils_scars.py:356-360).  Cell (r, c) is inside a polygon when the crossing
//                    test of W. R. Franklin's PNPOLY holds for the point (x = c, y = r): an odd
//                    number of edges (i, j = i - 1 cyclically) with
//                        (y_i <= y < y_j  or  y_j <= y < y_i)  and
//                        x < (x_j - x_i) * (y - y_i) / (y_j - y_i) + x_i,
//                    evaluated in IEEE double with every operation rounded separately (no fused
//                    multiply-add), so the mask is bit-identical to the host restatement.
//                    One block per row: the crossings of that row are computed once per edge into
//                    shared memory, then each column counts the crossings to its right.
// fk_conv2d_same  -- scipy.signal.convolve2d(a, k, "same") (what jax.scipy.signal.convolve2d
//                    restates; utils_scars.py:402-406): out[i][j] = sum_{a,b} k[a][b] *
//                    in[i + s - a][j + s - b], s = (K - 1) / 2, zero outside the plane,
//                    optionally stored as 1 - out (utils_scars.py:426).  A block computes a
//                    64 x 64 output tile: the kernel rows are taken 16 at a time, with the input
//                    rows they reach (79 rows of 64 + K + 4 columns) and those kernel rows
//                    (reversed, zero-padded to a multiple of 4) staged in shared memory; each
//                    thread accumulates a 4 x 4 block of outputs, reading per 4 kernel columns
//                    two 16-byte input words per row and one 16-byte weight word.  Kernels too
//                    wide for the staging (K > 512) take a plain per-output loop instead.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cardiax_gb300.h"

namespace fk {

namespace {

constexpr int RASTER_THREADS = 256;
constexpr int RASTER_MAX_EDGES = 4096;  // all polygons of one launch
constexpr int RASTER_MAX_POLYS = 16;

struct PolyOffsets {
    int v[RASTER_MAX_POLYS + 1];  // polygon p owns vertices [v[p], v[p + 1])
};

__global__ void __launch_bounds__(RASTER_THREADS)
    fk_scar_raster_kernel(const double *__restrict__ xs, const double *__restrict__ ys,
                          PolyOffsets offsets, int n_polys, int H, int W, float *out,
                          int64_t pitch, unsigned long long *count) {
    __shared__ double cross[RASTER_MAX_EDGES];
    __shared__ int n_cross[RASTER_MAX_POLYS];
    __shared__ int start[RASTER_MAX_POLYS + 1];
    __shared__ unsigned long long row_ones;
    const int r = blockIdx.x;
    const double y = (double)r;
    if (threadIdx.x <= n_polys) start[threadIdx.x] = offsets.v[threadIdx.x];
    if (threadIdx.x < n_polys) n_cross[threadIdx.x] = 0;
    if (threadIdx.x == 0) row_ones = 0ull;
    __syncthreads();
    const int n_edges = start[n_polys];
    for (int e = threadIdx.x; e < n_edges; e += blockDim.x) {
        int p = 0;
        while (e >= start[p + 1]) ++p;
        const int i = e, j = (e == start[p]) ? start[p + 1] - 1 : e - 1;
        const double yi = ys[i], yj = ys[j];
        if ((yi <= y && y < yj) || (yj <= y && y < yi)) {
            const double xi = xs[i], xj = xs[j];
            const double t = __ddiv_rn(__dmul_rn(__dsub_rn(xj, xi), __dsub_rn(y, yi)),
                                       __dsub_rn(yj, yi));
            const int slot = atomicAdd(&n_cross[p], 1);
            cross[start[p] + slot] = __dadd_rn(t, xi);
        }
    }
    __syncthreads();
    unsigned ones = 0;
    for (int c = threadIdx.x; c < W; c += blockDim.x) {
        const double x = (double)c;
        bool inside = false;
        for (int p = 0; p < n_polys && !inside; ++p) {
            bool odd = false;
            const double *cp = cross + start[p];
            for (int k = 0, n = n_cross[p]; k < n; ++k) odd ^= (x < cp[k]);
            inside = odd;
        }
        out[(int64_t)r * pitch + c] = inside ? 1.0f : 0.0f;
        ones += inside ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) ones += __shfl_xor_sync(0xffffffffu, ones, o);
    if ((threadIdx.x & 31) == 0 && ones) atomicAdd(&row_ones, (unsigned long long)ones);
    __syncthreads();
    if (threadIdx.x == 0 && row_ones) atomicAdd(count, row_ones);
}

constexpr int CONV_ROWS = 4;  // output rows per thread

__global__ void __launch_bounds__(256)
    fk_conv2d_same_kernel(const float *__restrict__ in, int H, int W, int64_t in_pitch,
                          const float *__restrict__ k, int K, float *__restrict__ out,
                          int64_t out_pitch, int one_minus) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * CONV_ROWS;
    if (j >= W || i0 >= H) return;
    const int s = (K - 1) / 2;
    float acc[CONV_ROWS] = {0.0f, 0.0f, 0.0f, 0.0f};
    // input rows y reach outputs i = y - s + a for kernel rows a in [0, K)
    const int y_lo = max(0, i0 + s - (K - 1)), y_hi = min(H - 1, i0 + CONV_ROWS - 1 + s);
    const int x_lo = max(0, j + s - (K - 1)), x_hi = min(W - 1, j + s);
    for (int y = y_lo; y <= y_hi; ++y) {
        const float *row = in + (int64_t)y * in_pitch;
        for (int x = x_lo; x <= x_hi; ++x) {
            const float v = __ldg(row + x);
            const int b = j + s - x;
#pragma unroll
            for (int q = 0; q < CONV_ROWS; ++q) {
                const int a = i0 + q + s - y;
                if (a >= 0 && a < K) acc[q] = fmaf(__ldg(k + a * K + b), v, acc[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < CONV_ROWS; ++q)
        if (i0 + q < H) out[(int64_t)(i0 + q) * out_pitch + j] = one_minus ? 1.0f - acc[q] : acc[q];
}

constexpr int CT = 64;   // output tile (rows and columns)
constexpr int CKA = 16;  // kernel rows per staged slab
constexpr int CONV_TILED_MAX_K = 512;  // staging within 227 KB of shared memory

__host__ __device__ constexpr int round4(int x) { return (x + 3) & ~3; }
// shared-memory words of the staged input slab row and of the whole staging
__host__ __device__ inline int conv_slab_width(int K) { return round4(CT + round4(K) + 4); }
inline size_t conv_smem_bytes(int K) {
    return sizeof(float) * ((size_t)(CT + CKA - 1) * conv_slab_width(K) + (size_t)CKA * round4(K));
}

__global__ void __launch_bounds__(256)
    fk_conv2d_tiled_kernel(const float *__restrict__ in, int H, int W, int64_t in_pitch,
                           const float *__restrict__ k, int K, float *__restrict__ out,
                           int64_t out_pitch, int one_minus) {
    extern __shared__ __align__(16) float conv_smem[];
    const int Kp = round4(K), SWc = conv_slab_width(K);
    float *slab = conv_smem;                         // (CT + CKA - 1) x SWc
    float *ks = conv_smem + (CT + CKA - 1) * SWc;    // CKA x Kp: ks[da][m] = k[a0 + da][K-1-m]
    const int s = (K - 1) / 2;
    const int r0 = blockIdx.y * CT, c0 = blockIdx.x * CT;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    // slab column cc holds input column x_lo + cc: output column c (tile-local) with kernel
    // column b = K-1-m reads input column c0 + c + s - b = x_lo + c + m
    const int x_lo = c0 + s - (K - 1);
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    for (int a0 = 0; a0 < K; a0 += CKA) {
        const int ka = min(CKA, K - a0);
        // slab row rr holds input row y_lo + rr: output row r (tile-local) with kernel row
        // a = a0 + da reads input row r0 + r + s - a = y_lo + r + (ka - 1 - da)
        const int y_lo = r0 + s - (a0 + ka - 1);
        const int nrows = CT + ka - 1;
        __syncthreads();  // the previous slab has been read
        for (int rr = threadIdx.x / 64; rr < nrows; rr += 4) {
            const int y = y_lo + rr;
            const bool row_in = y >= 0 && y < H;
            const float *src = in + (int64_t)(row_in ? y : 0) * in_pitch;
            for (int cc = threadIdx.x % 64; cc < SWc; cc += 64) {
                const int x = x_lo + cc;
                slab[rr * SWc + cc] = (row_in && x >= 0 && x < W) ? __ldg(src + x) : 0.0f;
            }
        }
        for (int q = threadIdx.x; q < ka * Kp; q += 256) {
            const int da = q / Kp, m = q % Kp;
            ks[q] = m < K ? __ldg(k + (int64_t)(a0 + da) * K + (K - 1 - m)) : 0.0f;
        }
        __syncthreads();
        for (int da = 0; da < ka; ++da) {
            const float *wrow = ks + da * Kp;
            const float *srow = slab + (4 * ty + (ka - 1 - da)) * SWc + 4 * tx;
            for (int m = 0; m < Kp; m += 4) {
                const float4 w4 = *reinterpret_cast<const float4 *>(wrow + m);
                const float w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float4 p = *reinterpret_cast<const float4 *>(srow + i * SWc + m);
                    const float4 q = *reinterpret_cast<const float4 *>(srow + i * SWc + m + 4);
                    const float v[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
#pragma unroll
                    for (int t = 0; t < 4; ++t)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(w[t], v[j + t], acc[i][j]);
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + 4 * ty + i;
        if (r >= H) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + 4 * tx + j;
            if (c < W) out[(int64_t)r * out_pitch + c] = one_minus ? 1.0f - acc[i][j] : acc[i][j];
        }
    }
}

}  // namespace

}  // namespace fk

extern "C" int fk_scar_raster(const double *xs, const double *ys, const int32_t *offsets,
                              int64_t n_polys, int64_t H, int64_t W, float *out, int64_t pitch,
                              unsigned long long *count, void *stream) {
    if (!out || !count || !offsets) return FK_ERR_NULL;
    if (n_polys < 0 || n_polys > fk::RASTER_MAX_POLYS || H < 1 || W < 1 || pitch < W ||
        H > (1 << 30) || W > (1 << 30))
        return FK_ERR_SHAPE;
    fk::PolyOffsets off{};
    if (offsets[0] != 0) return FK_ERR_ARGUMENT;
    for (int64_t p = 0; p <= n_polys; ++p) {
        off.v[p] = offsets[p];
        if (p && offsets[p] - offsets[p - 1] < 3) return FK_ERR_ARGUMENT;
    }
    if (offsets[n_polys] > fk::RASTER_MAX_EDGES) return FK_ERR_ARGUMENT;
    if (n_polys > 0 && (!xs || !ys)) return FK_ERR_NULL;
    fk::fk_scar_raster_kernel<<<(unsigned)H, fk::RASTER_THREADS, 0, (cudaStream_t)stream>>>(
        xs, ys, off, (int)n_polys, (int)H, (int)W, out, pitch, count);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

extern "C" int fk_conv2d_same(const float *in, int64_t H, int64_t W, int64_t in_pitch,
                              const float *kernel, int64_t K, float *out, int64_t out_pitch,
                              int one_minus, void *stream) {
    if (!in || !kernel || !out) return FK_ERR_NULL;
    if (H < 1 || W < 1 || K < 1 || K > 4096 || in_pitch < W || out_pitch < W ||
        H > (1 << 30) || W > (1 << 30))
        return FK_ERR_SHAPE;
    if (in == out) return FK_ERR_ARGUMENT;
    if (K <= fk::CONV_TILED_MAX_K) {
        const size_t smem = fk::conv_smem_bytes((int)K);
        if (cudaFuncSetAttribute(fk::fk_conv2d_tiled_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return FK_ERR_CUDA;
        const dim3 grid((unsigned)((W + fk::CT - 1) / fk::CT), (unsigned)((H + fk::CT - 1) / fk::CT));
        if (grid.y > 65535) return FK_ERR_SHAPE;
        fk::fk_conv2d_tiled_kernel<<<grid, 256, smem, (cudaStream_t)stream>>>(
            in, (int)H, (int)W, in_pitch, kernel, (int)K, out, out_pitch, one_minus);
        return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
    }
    const dim3 block(64, 4);
    const int64_t rows = (H + fk::CONV_ROWS - 1) / fk::CONV_ROWS;
    const dim3 grid((unsigned)((W + block.x - 1) / block.x), (unsigned)((rows + block.y - 1) / block.y));
    if (grid.y > 65535) return FK_ERR_SHAPE;
    fk::fk_conv2d_same_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(
        in, (int)H, (int)W, in_pitch, kernel, (int)K, out, out_pitch, one_minus);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}
