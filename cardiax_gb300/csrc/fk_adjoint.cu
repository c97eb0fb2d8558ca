// K3: reverse-mode (adjoint) Euler step of the Fenton-Karma stepper.
//
// Forward step (cardiax/solve.py:26-70), per cell:  v' = v + dt dv,  w' = w + dt dw,
// u' = u + dt (L(D) u + J), with J replaced by the stimulus value where one is active and
// L(D) u = D (A_x + A_y) u + (B_x D)(B_x u) + (B_y D)(B_y u).  Along one axis of length N,
// with E the edge pad (N+2 x N), G the derivative of cardiax/solve.py:225-254 on the padded
// line and C the crop:  B = C G E / dx,  A = C G G E / dx^2.
//
// Given the state x_t and the cotangent lam' of x_{t+1}, this computes the cotangent of x_t,
//   lam_v = lam'_v dv'/dv + lam'_u dt dJ/dv,   lam_w = lam'_w dw'/dw + lam'_u dt dJ/dw,
//   lam_u = lam'_u (1 + dt dJ/du) + L^T mu,     mu = dt lam'_u,
//   L^T mu = A_x^T (D mu) + A_y^T (D mu) + B_x^T ((B_x D) mu) + B_y^T ((B_y D) mu),
// and accumulates  dL/dD += mu (u_xx + u_yy) + B_x^T (mu u_x) + B_y^T (mu u_y)  per cell and
// dL/dtheta for the first 13 parameters (Cm fixed).  The Heaviside gates have zero derivative
// and a stimulated cell's J does not depend on the state or theta, exactly as jnp.where and
// jnp.greater_equal differentiate in the reference.
//
// Interior cells use G^T = -G on central rows (so A^T = A and B^T = -B); cells within
// ADJ_BAND of an edge use the explicit transposed rows, including the one-sided rows and the
// fold of the edge pad.
#include <cuda_runtime.h>

#include <cstdint>

#include "fk_adjoint.cuh"
#include "fk_math.cuh"

namespace fk {

namespace {

constexpr int AB = 16;  // block edge (AB x AB threads)

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// Coefficient of P[m] in row k of G on a padded line of length L (cardiax/solve.py:225-254).
__device__ __forceinline__ float gcoef(int k, int m, int L) {
    int o;
    if (k < 2) {  // head rows: P[k..k+3]
        o = m - k;
        switch (o) {
            case 0: return C_HEAD0;
            case 1: return C_THREE;
            case 2: return -C_3_2;
            case 3: return C_1_3;
            default: return 0.0f;
        }
    }
    if (k > L - 3) {  // tail rows: P[k-3..k]
        o = m - (k - 3);
        switch (o) {
            case 0: return C_TAIL0;
            case 1: return C_3_2;
            case 2: return -C_THREE;
            case 3: return C_TAIL3;
            default: return 0.0f;
        }
    }
    o = m - k;  // central rows: P[k-2], P[k-1], P[k+1], P[k+2]
    switch (o) {
        case -2: return C_1_12;
        case -1: return -C_2_3;
        case 1: return C_2_3;
        case 2: return -C_1_12;
        default: return 0.0f;
    }
}

// Accessor of a field along one line (a row or a column of the grid) at interior index r.
template <class F>
struct Line {
    F f;
    int N;
    // z = C^T a: padded index k -> a(k-1) for 1 <= k <= N, 0 at the pad
    __device__ __forceinline__ float z(int k) const { return (k >= 1 && k <= N) ? f(k - 1) : 0.0f; }
    // y1 = G^T z at padded index m
    __device__ float y1(int m) const {
        const int L = N + 2;
        float s = 0.0f;
        for (int k = max(0, m - 4); k <= min(L - 1, m + 4); ++k) {
            const float c = gcoef(k, m, L);
            if (c != 0.0f) s = fmaf(c, z(k), s);
        }
        return s;
    }
    // y2 = G^T y1 at padded index m
    __device__ float y2(int m) const {
        const int L = N + 2;
        float s = 0.0f;
        for (int k = max(0, m - 4); k <= min(L - 1, m + 4); ++k) {
            const float c = gcoef(k, m, L);
            if (c != 0.0f) s = fmaf(c, y1(k), s);
        }
        return s;
    }
    // (E^T y)[i]: the pad rows fold back onto the first and last cells
    __device__ float BT(int i) const {
        float s = y1(i + 1);
        if (i == 0) s += y1(0);
        if (i == N - 1) s += y1(N + 1);
        return s;
    }
    __device__ float AT(int i) const {
        float s = y2(i + 1);
        if (i == 0) s += y2(0);
        if (i == N - 1) s += y2(N + 1);
        return s;
    }
};

template <class F>
__device__ __forceinline__ Line<F> make_line(F f, int N) {
    return Line<F>{f, N};
}

// Forward first derivative (scaled by 1/dx later) at interior index i along a line accessed
// with clamped indices (the edge pad), as in the forward kernels' boundary path.
template <class F>
__device__ __forceinline__ float fwd_d1(F at, int i, int N) {
    // padded index i+1 of the derivative of the padded line
    const int x = i;
    if (x <= 0) return g_head(at(x), at(x + 1), at(x + 2), at(x + 3));
    if (x >= N - 1) return g_tail(at(x - 3), at(x - 2), at(x - 1), at(x));
    return g_central(at(x - 2), at(x - 1), at(x + 1), at(x + 2));
}
// u_x on the padded line at padded position x in [-1, N] (the first derivative that the
// second derivative is taken of).
template <class F>
__device__ __forceinline__ float fwd_ux_pad(F at, int x, int N) {
    if (x <= 0) return g_head(at(x), at(x + 1), at(x + 2), at(x + 3));
    if (x >= N - 1) return g_tail(at(x - 3), at(x - 2), at(x - 1), at(x));
    return g_central(at(x - 2), at(x - 1), at(x + 1), at(x + 2));
}
template <class F>
__device__ __forceinline__ float fwd_d2(F at, int i, int N, float rdx) {
    auto UX = [&](int x) { return fwd_ux_pad(at, x, N) * rdx; };
    float s;
    if (i == 0) s = g_head(UX(0), UX(1), UX(2), UX(3));
    else if (i == N - 1) s = g_tail(UX(N - 4), UX(N - 3), UX(N - 2), UX(N - 1));
    else s = g_central(UX(i - 2), UX(i - 1), UX(i + 1), UX(i + 2));
    return s * rdx;
}

__global__ void __launch_bounds__(AB *AB)
    fk_adjoint_kernel(const __grid_constant__ AdjointArgs a) {
    const int j = blockIdx.x * AB + threadIdx.x;
    const int i = blockIdx.y * AB + threadIdx.y;
    const int H = a.H, W = a.W, pitch = a.pitch;
    const bool in = i < H && j < W;
    const float dt = a.dt, rdx = a.rdx;
    const Model &m = a.m;

    float gth[kAdjParams];
#pragma unroll
    for (int k = 0; k < kAdjParams; ++k) gth[k] = 0.0f;

    if (in) {
        auto at = [&](const float *p, int r, int c) {
            return __ldg(p + (int64_t)clampi(r, 0, H - 1) * pitch + clampi(c, 0, W - 1));
        };
        const int64_t off = (int64_t)i * pitch + j;
        const float u = __ldg(a.u + off), v = __ldg(a.v + off), w = __ldg(a.w + off);
        const float lu = __ldg(a.lu + off), lv = __ldg(a.lv + off), lw = __ldg(a.lw + off);
        const float mu = dt * lu;

        // ---- pointwise part -------------------------------------------------------------
        bool stim = false;
        for (int s = 0; s < a.n_stim; ++s) {
            if (!stim_active(a.stim[s], a.t)) continue;
            const Stim &st = a.stim[s];
            const float fv = st.field ? __ldg(st.field + off)
                                      : ((i >= st.r0 && i < st.r1 && j >= st.c0 && j < st.c1)
                                             ? st.amplitude : 0.0f);
            if (fv != 0.0f) stim = true;
        }
        const bool p = u >= m.V_c, q = u >= m.V_v;
        const float S = one_plus_tanh(m.k * (u - m.V_csi));  // 1 + tanh
        const float sech2 = S * (2.0f - S);                  // 1 - tanh^2
        const float r_tvm = q ? m.r_tau_v2m : m.r_tau_v1m;
        const float dvdv = 1.0f + dt * (p ? -m.r_tau_vp : -r_tvm);
        const float dwdw = 1.0f + dt * (p ? -m.r_tau_wp : -m.r_tau_wm);
        float dJdu = 0.f, dJdv = 0.f, dJdw = 0.f;
        if (!stim) {
            const float dfi = p ? -v * (1.0f + m.V_c - 2.0f * u) * m.r_tau_d : 0.0f;
            const float dso = p ? 0.0f : m.r_tau_0;
            const float dsi = -w * m.k * sech2 * m.r_2tau_si;
            dJdu = -(dfi + dso + dsi) * m.r_Cm;
            dJdv = p ? (u - m.V_c) * (1.0f - u) * m.r_tau_d * m.r_Cm : 0.0f;
            dJdw = S * m.r_2tau_si * m.r_Cm;
        }
        float olv = lv * dvdv + mu * dJdv;
        float olw = lw * dwdw + mu * dJdw;
        float olu = lu * (1.0f + dt * dJdu);

        // ---- parameter gradients (cardiax/params.py fields 0..12) ------------------------
        const float pv = p ? 1.0f : 0.0f, qv = q ? 1.0f : 0.0f;
        gth[0] = lv * dt * pv * v * m.r_tau_vp * m.r_tau_vp;                           // tau_v_plus
        gth[1] = -lv * dt * (1.f - pv) * (1.f - v) * (1.f - qv) * m.r_tau_v1m * m.r_tau_v1m;
        gth[2] = -lv * dt * (1.f - pv) * (1.f - v) * qv * m.r_tau_v2m * m.r_tau_v2m;
        gth[3] = lw * dt * pv * w * m.r_tau_wp * m.r_tau_wp;                           // tau_w_plus
        gth[4] = -lw * dt * (1.f - pv) * (1.f - w) * m.r_tau_wm * m.r_tau_wm;           // tau_w_minus
        if (!stim) {
            gth[5] = mu * (-v * pv * (u - m.V_c) * (1.f - u) * m.r_tau_d * m.r_tau_d) * m.r_Cm;
            gth[6] = mu * (u * (1.f - pv) * m.r_tau_0 * m.r_tau_0) * m.r_Cm;            // tau_0
            gth[7] = mu * (pv * m.inv_tau_r * m.inv_tau_r) * m.r_Cm;                    // tau_r
            gth[8] = mu * (-w * S * 2.0f * m.r_2tau_si * m.r_2tau_si) * m.r_Cm;         // tau_si
            gth[9] = mu * (w * sech2 * (u - m.V_csi) * m.r_2tau_si) * m.r_Cm;           // k
            gth[10] = mu * (-w * m.k * sech2 * m.r_2tau_si) * m.r_Cm;                   // V_csi
            gth[11] = mu * (-v * pv * (1.f - u) * m.r_tau_d) * m.r_Cm;                  // V_c
        }
        // gth[12] (V_v) enters only through a Heaviside gate: zero

        // ---- diffusion transpose and dL/dD, axis by axis --------------------------------
        // Along an axis, a cell at least ADJ_BAND from both ends uses the interior form
        // (G^T = -G); otherwise the explicit transposed rows and the edge-pad fold.
        const float *D = a.D, *U = a.u, *LU = a.lu;
        auto Dat = [&](int r, int c) { return __ldg(D + (int64_t)r * pitch + c); };
        auto Uat = [&](int r, int c) { return __ldg(U + (int64_t)r * pitch + c); };
        auto Mat = [&](int r, int c) { return dt * __ldg(LU + (int64_t)r * pitch + c); };
        float ATx, BTx, uxx, gx, ATy, BTy, uyy, gy;
        if (i >= ADJ_BAND && i < H - ADJ_BAND) {
            auto Dx = [&](int r) {
                return g_central(Dat(r - 2, j), Dat(r - 1, j), Dat(r + 1, j), Dat(r + 2, j)) * rdx;
            };
            auto Ux = [&](int r) {
                return g_central(Uat(r - 2, j), Uat(r - 1, j), Uat(r + 1, j), Uat(r + 2, j)) * rdx;
            };
            auto Q1 = [&](int r) {  // G_x(D mu) at (r, j), scaled
                return g_central(Dat(r - 2, j) * Mat(r - 2, j), Dat(r - 1, j) * Mat(r - 1, j),
                                 Dat(r + 1, j) * Mat(r + 1, j), Dat(r + 2, j) * Mat(r + 2, j)) * rdx;
            };
            ATx = g_central(Q1(i - 2), Q1(i - 1), Q1(i + 1), Q1(i + 2)) * rdx;
            BTx = -g_central(Dx(i - 2) * Mat(i - 2, j), Dx(i - 1) * Mat(i - 1, j),
                             Dx(i + 1) * Mat(i + 1, j), Dx(i + 2) * Mat(i + 2, j)) * rdx;
            const float ux_m2 = Ux(i - 2), ux_m1 = Ux(i - 1), ux_p1 = Ux(i + 1), ux_p2 = Ux(i + 2);
            uxx = g_central(ux_m2, ux_m1, ux_p1, ux_p2) * rdx;
            gx = -g_central(Mat(i - 2, j) * ux_m2, Mat(i - 1, j) * ux_m1, Mat(i + 1, j) * ux_p1,
                            Mat(i + 2, j) * ux_p2) * rdx;
        } else {
            auto Dx_at = [&](int r) { return fwd_d1([&](int x) { return at(D, x, j); }, r, H) * rdx; };
            auto Ux_at = [&](int r) { return fwd_d1([&](int x) { return at(U, x, j); }, r, H) * rdx; };
            auto Mcol = [&](int r) { return dt * __ldg(LU + (int64_t)r * pitch + j); };
            const auto qx = make_line([&](int r) { return at(D, r, j) * Mcol(r); }, H);
            const auto bx = make_line([&](int r) { return Dx_at(r) * Mcol(r); }, H);
            const auto gxl = make_line([&](int r) { return Mcol(r) * Ux_at(r); }, H);
            ATx = qx.AT(i) * (rdx * rdx);
            BTx = bx.BT(i) * rdx;
            uxx = fwd_d2([&](int r) { return at(U, r, j); }, i, H, rdx);
            gx = gxl.BT(i) * rdx;
        }
        if (j >= ADJ_BAND && j < W - ADJ_BAND) {
            auto Dy = [&](int c) {
                return g_central(Dat(i, c - 2), Dat(i, c - 1), Dat(i, c + 1), Dat(i, c + 2)) * rdx;
            };
            auto Uy = [&](int c) {
                return g_central(Uat(i, c - 2), Uat(i, c - 1), Uat(i, c + 1), Uat(i, c + 2)) * rdx;
            };
            auto Q1 = [&](int c) {
                return g_central(Dat(i, c - 2) * Mat(i, c - 2), Dat(i, c - 1) * Mat(i, c - 1),
                                 Dat(i, c + 1) * Mat(i, c + 1), Dat(i, c + 2) * Mat(i, c + 2)) * rdx;
            };
            ATy = g_central(Q1(j - 2), Q1(j - 1), Q1(j + 1), Q1(j + 2)) * rdx;
            BTy = -g_central(Dy(j - 2) * Mat(i, j - 2), Dy(j - 1) * Mat(i, j - 1),
                             Dy(j + 1) * Mat(i, j + 1), Dy(j + 2) * Mat(i, j + 2)) * rdx;
            const float uy_m2 = Uy(j - 2), uy_m1 = Uy(j - 1), uy_p1 = Uy(j + 1), uy_p2 = Uy(j + 2);
            uyy = g_central(uy_m2, uy_m1, uy_p1, uy_p2) * rdx;
            gy = -g_central(Mat(i, j - 2) * uy_m2, Mat(i, j - 1) * uy_m1, Mat(i, j + 1) * uy_p1,
                            Mat(i, j + 2) * uy_p2) * rdx;
        } else {
            auto Dy_at = [&](int c) { return fwd_d1([&](int y) { return at(D, i, y); }, c, W) * rdx; };
            auto Uy_at = [&](int c) { return fwd_d1([&](int y) { return at(U, i, y); }, c, W) * rdx; };
            auto Mrow = [&](int c) { return dt * __ldg(LU + (int64_t)i * pitch + c); };
            const auto qy = make_line([&](int c) { return at(D, i, c) * Mrow(c); }, W);
            const auto by = make_line([&](int c) { return Dy_at(c) * Mrow(c); }, W);
            const auto gyl = make_line([&](int c) { return Mrow(c) * Uy_at(c); }, W);
            ATy = qy.AT(j) * (rdx * rdx);
            BTy = by.BT(j) * rdx;
            uyy = fwd_d2([&](int c) { return at(U, i, c); }, j, W, rdx);
            gy = gyl.BT(j) * rdx;
        }
        const float diff_u = (ATx + ATy) + (BTx + BTy);
        const float gD = mu * (uxx + uyy) + (gx + gy);
        olu += diff_u;
        a.olv[off] = olv;
        a.olw[off] = olw;
        a.olu[off] = olu;
        if (a.gD) a.gD[off] += gD;
    }

    // ---- deterministic block reduction of the parameter gradients into this block's slot ----
    if (a.gtheta) {
        __shared__ float red[kAdjParams][AB * AB / 32];
        const int tid = threadIdx.y * AB + threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
        for (int k = 0; k < kAdjParams; ++k) {
            float x = gth[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) red[k][warp] = x;
        }
        __syncthreads();
        if (tid < kAdjParams) {
            double s = 0.0;
            for (int w = 0; w < AB * AB / 32; ++w) s += (double)red[tid][w];
            a.gtheta[(int64_t)(blockIdx.y * gridDim.x + blockIdx.x) * kAdjParamStride + tid] += s;
        }
    }
}

}  // namespace

int64_t adjoint_slots(int H, int W) { return (int64_t)((W + AB - 1) / AB) * ((H + AB - 1) / AB); }

cudaError_t launch_adjoint(const AdjointArgs &a, cudaStream_t stream) {
    dim3 grid((a.W + AB - 1) / AB, (a.H + AB - 1) / AB), block(AB, AB);
    fk_adjoint_kernel<<<grid, block, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace fk
