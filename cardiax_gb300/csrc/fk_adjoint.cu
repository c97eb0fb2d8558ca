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

// Pointwise part of the adjoint of one cell: cotangents through the gates and currents, and the
// cell's contribution to dL/dtheta (added into gth).  Returns mu = dt lam'_u.
__device__ __forceinline__ float adjoint_pointwise(const AdjointArgs &a, int i, int j, int64_t off,
                                                  float &olv, float &olw, float &olu,
                                                  float *gth) {
    const Model &m = a.m;
    const float dt = a.dt;
    const float u = __ldg(a.u + off), v = __ldg(a.v + off), w = __ldg(a.w + off);
    const float lu = __ldg(a.lu + off), lv = __ldg(a.lv + off), lw = __ldg(a.lw + off);
    const float mu = dt * lu;
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
    olv = lv * dvdv + mu * dJdv;
    olw = lw * dwdw + mu * dJdw;
    olu = lu * (1.0f + dt * dJdu);

    // parameter gradients (cardiax/params.py fields 0..12)
    const float pv = p ? 1.0f : 0.0f, qv = q ? 1.0f : 0.0f;
    gth[0] += lv * dt * pv * v * m.r_tau_vp * m.r_tau_vp;                           // tau_v_plus
    gth[1] += -lv * dt * (1.f - pv) * (1.f - v) * (1.f - qv) * m.r_tau_v1m * m.r_tau_v1m;
    gth[2] += -lv * dt * (1.f - pv) * (1.f - v) * qv * m.r_tau_v2m * m.r_tau_v2m;
    gth[3] += lw * dt * pv * w * m.r_tau_wp * m.r_tau_wp;                           // tau_w_plus
    gth[4] += -lw * dt * (1.f - pv) * (1.f - w) * m.r_tau_wm * m.r_tau_wm;           // tau_w_minus
    if (!stim) {
        gth[5] += mu * (-v * pv * (u - m.V_c) * (1.f - u) * m.r_tau_d * m.r_tau_d) * m.r_Cm;
        gth[6] += mu * (u * (1.f - pv) * m.r_tau_0 * m.r_tau_0) * m.r_Cm;            // tau_0
        gth[7] += mu * (pv * m.inv_tau_r * m.inv_tau_r) * m.r_Cm;                    // tau_r
        gth[8] += mu * (-w * S * 2.0f * m.r_2tau_si * m.r_2tau_si) * m.r_Cm;         // tau_si
        gth[9] += mu * (w * sech2 * (u - m.V_csi) * m.r_2tau_si) * m.r_Cm;           // k
        gth[10] += mu * (-w * m.k * sech2 * m.r_2tau_si) * m.r_Cm;                   // V_csi
        gth[11] += mu * (-v * pv * (1.f - u) * m.r_tau_d) * m.r_Cm;                  // V_c
    }
    // gth[12] (V_v) enters only through a Heaviside gate: zero
    return mu;
}

// One axis of the diffusion transpose at a cell within ADJ_BAND of an edge along that axis:
// the explicit transposed rows (one-sided rows and the fold of the edge pad), reading global
// memory.  AXIS 0: along rows (x), 1: along columns (y).
struct AxisTerms {
    float AT, BT, d2, g;  // A^T(D mu), B^T((B D) mu), u_xx (or u_yy), B^T(mu u_x) (or y)
};
template <int AXIS>
__device__ AxisTerms axis_explicit(const AdjointArgs &a, int i, int j) {
    const int H = a.H, W = a.W, pitch = a.pitch;
    const float dt = a.dt, rdx = a.rdx;
    const float *D = a.D, *U = a.u, *LU = a.lu;
    auto at = [&](const float *p, int r, int c) {
        return __ldg(p + (int64_t)clampi(r, 0, H - 1) * pitch + clampi(c, 0, W - 1));
    };
    AxisTerms t;
    if (AXIS == 0) {
        auto Dx_at = [&](int r) { return fwd_d1([&](int x) { return at(D, x, j); }, r, H) * rdx; };
        auto Ux_at = [&](int r) { return fwd_d1([&](int x) { return at(U, x, j); }, r, H) * rdx; };
        auto Mcol = [&](int r) { return dt * __ldg(LU + (int64_t)r * pitch + j); };
        const auto qx = make_line([&](int r) { return at(D, r, j) * Mcol(r); }, H);
        const auto bx = make_line([&](int r) { return Dx_at(r) * Mcol(r); }, H);
        const auto gxl = make_line([&](int r) { return Mcol(r) * Ux_at(r); }, H);
        t.AT = qx.AT(i) * (rdx * rdx);
        t.BT = bx.BT(i) * rdx;
        t.d2 = fwd_d2([&](int r) { return at(U, r, j); }, i, H, rdx);
        t.g = gxl.BT(i) * rdx;
    } else {
        auto Dy_at = [&](int c) { return fwd_d1([&](int y) { return at(D, i, y); }, c, W) * rdx; };
        auto Uy_at = [&](int c) { return fwd_d1([&](int y) { return at(U, i, y); }, c, W) * rdx; };
        auto Mrow = [&](int c) { return dt * __ldg(LU + (int64_t)i * pitch + c); };
        const auto qy = make_line([&](int c) { return at(D, i, c) * Mrow(c); }, W);
        const auto by = make_line([&](int c) { return Dy_at(c) * Mrow(c); }, W);
        const auto gyl = make_line([&](int c) { return Mrow(c) * Uy_at(c); }, W);
        t.AT = qy.AT(j) * (rdx * rdx);
        t.BT = by.BT(j) * rdx;
        t.d2 = fwd_d2([&](int c) { return at(U, i, c); }, j, W, rdx);
        t.g = gyl.BT(j) * rdx;
    }
    return t;
}

// Corner blocks (cells 0..9 of a line) of the line operators B' = C G E and A' = C G G E
// (E the edge pad, G the padded-line derivative of cardiax/solve.py:225-254, C the crop), built
// in double at compile time on a line of 40 cells.  Both operators are banded (|r - i| <= 4),
// so the corner is the same for every line of at least 18 cells, and the far corner is the
// reflection: A'[N-1-r][N-1-i] = A'[r][i], B'[N-1-r][N-1-i] = -B'[r][i].
struct EdgeTables {
    float A[10][10], B[10][10];
};
constexpr double gd(int k, int m, int L) {  // G[k][m] on a padded line of length L
    if (k < 2) {
        const int o = m - k;
        return o == 0 ? -11.0 / 6.0 : o == 1 ? 3.0 : o == 2 ? -1.5 : o == 3 ? 1.0 / 3.0 : 0.0;
    }
    if (k > L - 3) {
        const int o = m - (k - 3);
        return o == 0 ? -1.0 / 3.0 : o == 1 ? 1.5 : o == 2 ? -3.0 : o == 3 ? 11.0 / 6.0 : 0.0;
    }
    const int o = m - k;
    return o == -2 ? 1.0 / 12.0 : o == -1 ? -2.0 / 3.0 : o == 1 ? 2.0 / 3.0 : o == 2 ? -1.0 / 12.0 : 0.0;
}
constexpr double ge(int m, int i, int N) {  // (G E)[m][i]
    const int L = N + 2;
    return gd(m, i + 1, L) + (i == 0 ? gd(m, 0, L) : 0.0) + (i == N - 1 ? gd(m, L - 1, L) : 0.0);
}
constexpr EdgeTables make_edge_tables() {
    constexpr int N = 40, L = N + 2;
    EdgeTables t{};
    for (int r = 0; r < 10; ++r)
        for (int i = 0; i < 10; ++i) {
            double a = 0.0;
            for (int m = 0; m < L; ++m) a += gd(r + 1, m, L) * ge(m, i, N);
            t.A[r][i] = (float)a;
            t.B[r][i] = (float)ge(r + 1, i, N);
        }
    return t;
}
constexpr EdgeTables kEdgeHost = make_edge_tables();
__constant__ EdgeTables kEdge = kEdgeHost;
constexpr int kEdgeMinLine = 20;  // shorter lines use the explicit rows of axis_explicit

// One axis of the diffusion transpose at a cell within ADJ_BAND of an end of its line, from
// the corner tables: 10 cells of the line nearest that end.
template <int AXIS>
__device__ AxisTerms axis_edge(const AdjointArgs &a, int i, int j) {
    const int N = AXIS == 0 ? a.H : a.W;
    const int pos = AXIS == 0 ? i : j;
    if (N < kEdgeMinLine) return axis_explicit<AXIS>(a, i, j);
    const int pitch = a.pitch;
    const float dt = a.dt, rdx = a.rdx;
    const bool near0 = pos < ADJ_BAND;
    const int pp = near0 ? pos : N - 1 - pos;  // distance from the near end
    auto at = [&](const float *f, int q) {
        q = clampi(q, 0, N - 1);
        return __ldg(f + (AXIS == 0 ? (int64_t)q * pitch + j : (int64_t)i * pitch + q));
    };
    float AT = 0.f, BT = 0.f, d2 = 0.f, g = 0.f;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const int q = near0 ? r : N - 1 - r;
        const float mu = dt * at(a.lu, q);
        const float dq = fwd_d1([&](int x) { return at(a.D, x); }, q, N) * rdx;
        const float uq = fwd_d1([&](int x) { return at(a.u, x); }, q, N) * rdx;
        AT = fmaf(kEdge.A[r][pp], at(a.D, q) * mu, AT);
        BT = fmaf(kEdge.B[r][pp], dq * mu, BT);
        d2 = fmaf(kEdge.A[pp][r], at(a.u, q), d2);
        g = fmaf(kEdge.B[r][pp], mu * uq, g);
    }
    const float sgn = near0 ? 1.0f : -1.0f;
    AxisTerms t;
    t.AT = AT * (rdx * rdx);
    t.BT = sgn * BT * rdx;
    t.d2 = d2 * (rdx * rdx);
    t.g = sgn * g * rdx;
    return t;
}

// axis_edge from a line's precomputed products (L[r] = (D mu, (B D) mu, u, mu u_x) at the r-th
// cell from the near end) and the corner tables in shared memory: the same fused multiply-adds
// in the same order, so the same bits.
__device__ __forceinline__ AxisTerms axis_edge_tab(const float4 *L, const float (*tA)[10],
                                                   const float (*tB)[10], int pp, bool near0,
                                                   float rdx) {
    float AT = 0.f, BT = 0.f, d2 = 0.f, g = 0.f;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const float4 l = L[r];
        AT = fmaf(tA[r][pp], l.x, AT);
        BT = fmaf(tB[r][pp], l.y, BT);
        d2 = fmaf(tA[pp][r], l.z, d2);
        g = fmaf(tB[r][pp], l.w, g);
    }
    const float sgn = near0 ? 1.0f : -1.0f;
    AxisTerms t;
    t.AT = AT * (rdx * rdx);
    t.BT = sgn * BT * rdx;
    t.d2 = d2 * (rdx * rdx);
    t.g = sgn * g * rdx;
    return t;
}

// Tile geometry: ATY x ATX cells per block, a 4-cell halo of u, D and mu in shared memory.
constexpr int ATX = 32, ATY = 16, AHALO = 4;
constexpr int ASW = ATX + 2 * AHALO, ASH = ATY + 2 * AHALO;
constexpr int ANT = 256;
constexpr int AXW = ATX;      // row width of the x-derivative planes (tile rows -2 .. ATY+1)
constexpr int AYW = ATX + 4;  // row width of the y-derivative planes (tile columns -2 .. ATX+1)

// Interior cells (at least ADJ_BAND from both ends of an axis) use G^T = -G on central rows:
// along x, A_x^T(D mu) = G G (D mu) / dx^2, B_x^T(D_x mu) = -G (D_x mu) / dx and
// B_x^T(mu u_x) = -G (mu u_x) / dx, from first derivatives staged in shared memory.
// Tile (bx, by) of the step described by `a` (a kernel parameter, or a block's shared copy);
// its dL/dtheta partial sums go to slot by * nbx + bx of a.gtheta.
__device__ __forceinline__ void adjoint_tile(const AdjointArgs &a, int bx, int by, int nbx) {
    // u, D, mu = dt lam'_u (16-byte aligned: filled with float4 stores when the halo is in-grid)
    __shared__ __align__(16) float su[ASH * ASW];
    __shared__ __align__(16) float sd[ASH * ASW];
    __shared__ __align__(16) float sm[ASH * ASW];
    __shared__ float sux[(ATY + 4) * AXW], sqx[(ATY + 4) * AXW], sbx[(ATY + 4) * AXW];
    __shared__ float suy[ATY * AYW], sqy[ATY * AYW], sby[ATY * AYW];
    __shared__ float red[kAdjParams][ANT / 32];
    // edge band: per line and end, the 10 products each band cell of that line needs (ex: the
    // x-direction lines of the tile's columns, ey: the y-direction lines of its rows), and the
    // corner tables (lanes of a column band index them with different pp)
    __shared__ float4 ex[2][ATX][10], ey[2][ATY][10];
    __shared__ float tA[10][10], tB[10][10];
    const int tid = threadIdx.x;
    const int H = a.H, W = a.W, pitch = a.pitch;
    const float dt = a.dt, rdx = a.rdx;
    const int i0 = by * ATY, j0 = bx * ATX;
    // which line ends have the cells their products read -- -1 .. 11 from the near end, the pad
    // cell included (a clamped copy in the halo) -- inside the shared halo (uniform per block)
    const bool tx0 = H >= kEdgeMinLine && i0 == 0;
    const bool tx1 = H >= kEdgeMinLine && i0 + ATY > H - ADJ_BAND && i0 <= H - 8 && i0 + ATY + 3 >= H;
    const bool ty0 = W >= kEdgeMinLine && j0 == 0;
    const bool ty1 = W >= kEdgeMinLine && j0 + ATX > W - ADJ_BAND && j0 <= W - 8 && j0 + ATX + 3 >= W;

    // u, D, mu with a 4-cell halo; out-of-grid positions hold clamped copies, read only by
    // cells that take the explicit path along that axis
    if (i0 >= AHALO && i0 + ATY + AHALO <= H && j0 >= AHALO && j0 + ATX + AHALO <= W) {
        // halo inside the grid: 16-byte loads (rows start at column j0 - 4, a multiple of 4)
        constexpr int SW4 = ASW / 4;
        for (int k = tid; k < ASH * SW4; k += ANT) {
            const int r = k / SW4, c4 = k % SW4;
            const int64_t g = (int64_t)(i0 - AHALO + r) * pitch + j0 - AHALO + 4 * c4;
            const float4 u4 = __ldg(reinterpret_cast<const float4 *>(a.u + g));
            const float4 d4 = __ldg(reinterpret_cast<const float4 *>(a.D + g));
            const float4 l4 = __ldg(reinterpret_cast<const float4 *>(a.lu + g));
            reinterpret_cast<float4 *>(su)[k] = u4;
            reinterpret_cast<float4 *>(sd)[k] = d4;
            reinterpret_cast<float4 *>(sm)[k] =
                make_float4(dt * l4.x, dt * l4.y, dt * l4.z, dt * l4.w);
        }
    } else {
        for (int k = tid; k < ASH * ASW; k += ANT) {
            const int r = k / ASW, c = k % ASW;
            const int64_t g = (int64_t)clampi(i0 - AHALO + r, 0, H - 1) * pitch +
                              clampi(j0 - AHALO + c, 0, W - 1);
            su[k] = __ldg(a.u + g);
            sd[k] = __ldg(a.D + g);
            sm[k] = dt * __ldg(a.lu + g);
        }
    }
    __syncthreads();
    // edge-band line products from the shared halo (edge tiles only)
    if (tx0 || tx1 || ty0 || ty1) {
        for (int k = tid; k < 200; k += ANT) {
            const int r = k / 10, c = k % 10;
            if (r < 10) tA[r][c] = kEdge.A[r][c];
            else tB[r - 10][c] = kEdge.B[r - 10][c];
        }
        const int nx = (tx0 + tx1) * ATX * 10, ny = (ty0 + ty1) * ATY * 10;
        for (int k = tid; k < nx + ny; k += ANT) {
            if (k < nx) {
                const int e = (!tx0 || k >= ATX * 10) ? 1 : 0;
                const int kk = k - (tx0 && e == 1 ? ATX * 10 : 0);
                const int c = kk / 10, r = kk % 10;
                const int q = e ? H - 1 - r : r;
                auto SR = [&](const float *f, int x) { return f[(x - i0 + AHALO) * ASW + c + AHALO]; };
                const float mu = SR(sm, q);
                const float dq = fwd_d1([&](int x) { return SR(sd, x); }, q, H) * rdx;
                const float uq = fwd_d1([&](int x) { return SR(su, x); }, q, H) * rdx;
                ex[e][c][r] = make_float4(SR(sd, q) * mu, dq * mu, SR(su, q), mu * uq);
            } else {
                const int k2 = k - nx;
                const int e = (!ty0 || k2 >= ATY * 10) ? 1 : 0;
                const int kk = k2 - (ty0 && e == 1 ? ATY * 10 : 0);
                const int rr = kk / 10, r = kk % 10;
                const int q = e ? W - 1 - r : r;
                auto SC = [&](const float *f, int y) { return f[(rr + AHALO) * ASW + y - j0 + AHALO]; };
                const float mu = SC(sm, q);
                const float dq = fwd_d1([&](int y) { return SC(sd, y); }, q, W) * rdx;
                const float uq = fwd_d1([&](int y) { return SC(su, y); }, q, W) * rdx;
                ey[e][rr][r] = make_float4(SC(sd, q) * mu, dq * mu, SC(su, q), mu * uq);
            }
        }
    }
    // x: u_x, G_x(D mu), D_x mu on tile rows -2 .. ATY+1
    for (int k = tid; k < (ATY + 4) * AXW; k += ANT) {
        const int r = k / AXW, c = k % AXW;
        const int b = (r - 2 + AHALO) * ASW + c + AHALO;
        auto U = [&](int d) { return su[b + d * ASW]; };
        auto Dd = [&](int d) { return sd[b + d * ASW]; };
        auto M = [&](int d) { return sm[b + d * ASW]; };
        sux[k] = g_central(U(-2), U(-1), U(1), U(2)) * rdx;
        sqx[k] = g_central(Dd(-2) * M(-2), Dd(-1) * M(-1), Dd(1) * M(1), Dd(2) * M(2)) * rdx;
        sbx[k] = (g_central(Dd(-2), Dd(-1), Dd(1), Dd(2)) * rdx) * M(0);
    }
    // y: the same on tile columns -2 .. ATX+1
    for (int k = tid; k < ATY * AYW; k += ANT) {
        const int r = k / AYW, c = k % AYW;
        const int b = (r + AHALO) * ASW + c - 2 + AHALO;
        auto U = [&](int d) { return su[b + d]; };
        auto Dd = [&](int d) { return sd[b + d]; };
        auto M = [&](int d) { return sm[b + d]; };
        suy[k] = g_central(U(-2), U(-1), U(1), U(2)) * rdx;
        sqy[k] = g_central(Dd(-2) * M(-2), Dd(-1) * M(-1), Dd(1) * M(1), Dd(2) * M(2)) * rdx;
        sby[k] = (g_central(Dd(-2), Dd(-1), Dd(1), Dd(2)) * rdx) * M(0);
    }
    __syncthreads();

    float gth[kAdjParams];
#pragma unroll
    for (int k = 0; k < kAdjParams; ++k) gth[k] = 0.0f;
    for (int k = tid; k < ATY * ATX; k += ANT) {
        const int r = k / ATX, c = k % ATX;
        const int i = i0 + r, j = j0 + c;
        if (i >= H || j >= W) continue;
        const int64_t off = (int64_t)i * pitch + j;
        float olv, olw, olu;
        const float mu = adjoint_pointwise(a, i, j, off, olv, olw, olu, gth);
        AxisTerms x, y;
        if (i >= ADJ_BAND && i < H - ADJ_BAND) {
            auto X = [&](const float *f, int d) { return f[(r + 2 + d) * AXW + c]; };
            auto M = [&](int d) { return sm[(r + AHALO + d) * ASW + c + AHALO]; };
            x.AT = g_central(X(sqx, -2), X(sqx, -1), X(sqx, 1), X(sqx, 2)) * rdx;
            x.BT = -g_central(X(sbx, -2), X(sbx, -1), X(sbx, 1), X(sbx, 2)) * rdx;
            x.d2 = g_central(X(sux, -2), X(sux, -1), X(sux, 1), X(sux, 2)) * rdx;
            x.g = -g_central(M(-2) * X(sux, -2), M(-1) * X(sux, -1), M(1) * X(sux, 1),
                             M(2) * X(sux, 2)) * rdx;
        } else {
            const bool near0 = i < ADJ_BAND;
            if (near0 ? tx0 : tx1)
                x = axis_edge_tab(ex[near0 ? 0 : 1][c], tA, tB, near0 ? i : H - 1 - i, near0, rdx);
            else
                x = axis_edge<0>(a, i, j);
        }
        if (j >= ADJ_BAND && j < W - ADJ_BAND) {
            auto Y = [&](const float *f, int d) { return f[r * AYW + c + 2 + d]; };
            auto M = [&](int d) { return sm[(r + AHALO) * ASW + c + AHALO + d]; };
            y.AT = g_central(Y(sqy, -2), Y(sqy, -1), Y(sqy, 1), Y(sqy, 2)) * rdx;
            y.BT = -g_central(Y(sby, -2), Y(sby, -1), Y(sby, 1), Y(sby, 2)) * rdx;
            y.d2 = g_central(Y(suy, -2), Y(suy, -1), Y(suy, 1), Y(suy, 2)) * rdx;
            y.g = -g_central(M(-2) * Y(suy, -2), M(-1) * Y(suy, -1), M(1) * Y(suy, 1),
                             M(2) * Y(suy, 2)) * rdx;
        } else {
            const bool near0 = j < ADJ_BAND;
            if (near0 ? ty0 : ty1)
                y = axis_edge_tab(ey[near0 ? 0 : 1][r], tA, tB, near0 ? j : W - 1 - j, near0, rdx);
            else
                y = axis_edge<1>(a, i, j);
        }
        const float diff_u = (x.AT + y.AT) + (x.BT + y.BT);
        const float gD = mu * (x.d2 + y.d2) + (x.g + y.g);
        a.olv[off] = olv;
        a.olw[off] = olw;
        a.olu[off] = olu + diff_u;
        if (a.gD) a.gD[off] += gD;
    }

    // ---- deterministic block reduction of the parameter gradients into this block's slot ----
    if (a.gtheta) {
        const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
        for (int k = 0; k < kAdjParams; ++k) {
            float x = gth[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) red[k][warp] = x;
        }
        __syncthreads();
        if (tid < kAdjParams) {
            double s = 0.0;
            for (int w = 0; w < ANT / 32; ++w) s += (double)red[tid][w];
            a.gtheta[(int64_t)(by * nbx + bx) * kAdjParamStride + tid] += s;
        }
    }
}

__global__ void __launch_bounds__(ANT, 4) fk_adjoint_kernel(const __grid_constant__ AdjointArgs a) {
    adjoint_tile(a, blockIdx.x, blockIdx.y, gridDim.x);
}

// One reverse step of many experiments (blockIdx.z): exps[e] describes step 0 of experiment e's
// segment with the cotangent ping-pong buffers (lu.. = buffer A, olu.. = buffer B); step k reads
// the state k * k_stride further on, and parity 1 swaps the two cotangent buffers.
__global__ void __launch_bounds__(ANT, 4) fk_adjoint_batch_kernel(const AdjointArgs *__restrict__ exps,
                                                               int64_t k_stride, int k, int parity,
                                                               float t) {
    __shared__ __align__(16) AdjointArgs sa;
    const uint32_t *src = reinterpret_cast<const uint32_t *>(exps + blockIdx.z);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&sa);
    for (int w = threadIdx.x; w < (int)(sizeof(AdjointArgs) / 4); w += ANT) dst[w] = __ldg(src + w);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int64_t o = (int64_t)k * k_stride;
        sa.u += o;
        sa.v += o;
        sa.w += o;
        sa.t = t;
        if (parity) {
            const float *lu = sa.lu, *lv = sa.lv, *lw = sa.lw;
            sa.lu = sa.olu;
            sa.lv = sa.olv;
            sa.lw = sa.olw;
            sa.olu = const_cast<float *>(lu);
            sa.olv = const_cast<float *>(lv);
            sa.olw = const_cast<float *>(lw);
        }
    }
    __syncthreads();
    adjoint_tile(sa, blockIdx.x, blockIdx.y, gridDim.x);
}

}  // namespace

int64_t adjoint_slots(int H, int W) {
    return (int64_t)((W + ATX - 1) / ATX) * ((H + ATY - 1) / ATY);
}

cudaError_t launch_adjoint(const AdjointArgs &a, cudaStream_t stream) {
    dim3 grid((a.W + ATX - 1) / ATX, (a.H + ATY - 1) / ATY);
    fk_adjoint_kernel<<<grid, ANT, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_batch(const AdjointArgs *exps, int n_exp, int H, int W, int64_t k_stride,
                                 int k, int parity, float t, cudaStream_t stream) {
    if (n_exp < 1) return cudaSuccess;
    dim3 grid((W + ATX - 1) / ATX, (H + ATY - 1) / ATY, n_exp);
    fk_adjoint_batch_kernel<<<grid, ANT, 0, stream>>>(exps, k_stride, k, parity, t);
    return cudaGetLastError();
}

}  // namespace fk
