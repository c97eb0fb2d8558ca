// K1: fused Fenton-Karma Euler step (reaction + gates + stimulus override + div(D grad u) +
// Euler update) over one tissue, one launch per time step.
//
// Replaces cardiax/solve.py:26-70 (step + step_euler, with gradient x6, stimulate and the edge
// pads fused).  Memory layout: SoA float32 planes, row pitch a multiple of 4 floats.
//
// Per CTA: one TMA transaction brings the u tile with a 4-cell halo and the D tile with a
// 2-row halo into shared memory (out-of-grid cells read as zero); v and w are read straight
// into registers with 16-byte loads.  Each thread streams 8 rows of 4 columns:
//   vertical derivatives   u_x, u_xx, D_x from register windows of shared-memory rows;
//   horizontal derivatives u_y, u_yy, D_y from three 16-byte shared-memory reads per row.
// Cells within 4 of an edge (one-sided stencils, edge padding) are recomputed by a per-cell
// path that reads global memory with clamped indices, exactly as the reference pads.
#include "fk_ptx.cuh"
#include "fk_step.cuh"

namespace fk {

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// ---- per-cell boundary path ---------------------------------------------------------------
// Reads the input planes with the reference's edge padding: index -1 maps to 0, N to N-1.
struct Clamped {
    const float *p;
    int H, W, pitch;
    __device__ __forceinline__ float at(int r, int c) const {
        return __ldg(p + (int64_t)clampi(r, 0, H - 1) * pitch + clampi(c, 0, W - 1));
    }
};

// d/dx of the padded u at padded row x in [-1, H] (cardiax/solve.py:225-254 along axis 0).
__device__ __forceinline__ float ux_at(const Clamped &u, int x, int c) {
    const int H = u.H;
    if (x <= 0) return g_head(u.at(x, c), u.at(x + 1, c), u.at(x + 2, c), u.at(x + 3, c));
    if (x >= H - 1) return g_tail(u.at(x - 3, c), u.at(x - 2, c), u.at(x - 1, c), u.at(x, c));
    return g_central(u.at(x - 2, c), u.at(x - 1, c), u.at(x + 1, c), u.at(x + 2, c));
}
__device__ __forceinline__ float uy_at(const Clamped &u, int r, int y) {
    const int W = u.W;
    if (y <= 0) return g_head(u.at(r, y), u.at(r, y + 1), u.at(r, y + 2), u.at(r, y + 3));
    if (y >= W - 1) return g_tail(u.at(r, y - 3), u.at(r, y - 2), u.at(r, y - 1), u.at(r, y));
    return g_central(u.at(r, y - 2), u.at(r, y - 1), u.at(r, y + 1), u.at(r, y + 2));
}

__device__ void boundary_cell(const StepArgs &a, unsigned active, bool deriv, int i, int j) {
    const Clamped U{a.u, a.H, a.W, a.pitch}, D{a.D, a.H, a.W, a.pitch};
    const int H = a.H, W = a.W;
    const float rdx = a.rdx;
    // first derivatives (scaled) at the padded positions the second derivative needs
    auto UX = [&](int x) { return ux_at(U, x, j) * rdx; };
    auto UY = [&](int y) { return uy_at(U, i, y) * rdx; };
    float uxx, uyy, dxD, dyD;
    if (i == 0) uxx = g_head(UX(0), UX(1), UX(2), UX(3));
    else if (i == H - 1) uxx = g_tail(UX(H - 4), UX(H - 3), UX(H - 2), UX(H - 1));
    else uxx = g_central(UX(i - 2), UX(i - 1), UX(i + 1), UX(i + 2));
    if (j == 0) uyy = g_head(UY(0), UY(1), UY(2), UY(3));
    else if (j == W - 1) uyy = g_tail(UY(W - 4), UY(W - 3), UY(W - 2), UY(W - 1));
    else uyy = g_central(UY(j - 2), UY(j - 1), UY(j + 1), UY(j + 2));
    uxx *= rdx;
    uyy *= rdx;
    if (i == 0) dxD = g_head(D.at(0, j), D.at(1, j), D.at(2, j), D.at(3, j));
    else if (i == H - 1) dxD = g_tail(D.at(i - 3, j), D.at(i - 2, j), D.at(i - 1, j), D.at(i, j));
    else dxD = g_central(D.at(i - 2, j), D.at(i - 1, j), D.at(i + 1, j), D.at(i + 2, j));
    if (j == 0) dyD = g_head(D.at(i, 0), D.at(i, 1), D.at(i, 2), D.at(i, 3));
    else if (j == W - 1) dyD = g_tail(D.at(i, j - 3), D.at(i, j - 2), D.at(i, j - 1), D.at(i, j));
    else dyD = g_central(D.at(i, j - 2), D.at(i, j - 1), D.at(i, j + 1), D.at(i, j + 2));
    dxD *= rdx;
    dyD *= rdx;
    const int64_t off = (int64_t)i * a.pitch + j;
    const float u = __ldg(a.u + off), v = __ldg(a.v + off), w = __ldg(a.w + off),
                d = __ldg(a.D + off);
    Reaction r = reaction(u, v, w, a.m);
    if (active) {
        float acc = 0.0f;
        for (int s = 0; s < a.n_stim; ++s) {
            if (!((active >> s) & 1u)) continue;
            const Stim &st = a.stim[s];
            float f = st.field ? __ldg(st.field + off)
                               : ((i >= st.r0 && i < st.r1 && j >= st.c0 && j < st.c1) ? st.amplitude : 0.0f);
            if (f != 0.0f) acc = f;
        }
        if (acc != 0.0f) r.j_ion = acc;
    }
    const float du = diffusion(d, dxD, dyD, UX(i), UY(j), uxx, uyy) + r.j_ion;
    if (deriv) {
        a.vo[off] = r.dv;
        a.wo[off] = r.dw;
        a.uo[off] = du;
    } else {
        a.vo[off] = fmaf(r.dv, a.dt, v);
        a.wo[off] = fmaf(r.dw, a.dt, w);
        a.uo[off] = fmaf(du, a.dt, u);
    }
}

// ---- the step kernel ----------------------------------------------------------------------
template <bool DERIV>
__global__ void __launch_bounds__(NT) fk_step_kernel(const __grid_constant__ CUtensorMap tm_u,
                                                     const __grid_constant__ CUtensorMap tm_d,
                                                     const __grid_constant__ StepArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *su = reinterpret_cast<float *>(smem);
    float *sd = reinterpret_cast<float *>(smem + SMEM_U_BYTES);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + SMEM_U_BYTES + SMEM_D_BYTES);

    const int tid = threadIdx.x;
    const int j0 = blockIdx.x * TX, i0 = blockIdx.y * TY;
    const int H = a.H, W = a.W, pitch = a.pitch;

    if (tid == 0) {
        prefetch_tensormap(&tm_u);
        prefetch_tensormap(&tm_d);
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, SMEM_U_BYTES + SMEM_D_BYTES);
        tma_load_2d(su, &tm_u, j0 - HALO_U, i0 - HALO_U, bar);
        tma_load_2d(sd, &tm_d, j0 - HALO_U, i0 - HALO_D, bar);
    }

    // stimulus protocol (uniform over the launch)
    unsigned active = 0;
    for (int s = 0; s < a.n_stim; ++s)
        if (stim_active(a.stim[s], a.t)) active |= 1u << s;

    const int tx = tid % NTX, ty = tid / NTX;
    const int j = j0 + 4 * tx;
    const int r0 = MR * ty;  // first row of this thread within the tile
    const bool interior = i0 >= BAND && i0 + TY <= H - BAND && j0 >= BAND && j0 + TX <= W - BAND;
    const bool col_in = j < W;

    if (!mbar_wait_bounded(bar, 0)) {
        if (tid == 0) atomicOr(a.status, kStatusTimeout);
        return;
    }

    const float rdx = a.rdx;
    const float *su_c = su + 4 * tx + HALO_U;  // this thread's first column, u tile
    const float *sd_c = sd + 4 * tx + HALO_U;  // this thread's first column, D tile
    auto LU = [&](int row) { return *reinterpret_cast<const float4 *>(su_c + row * SU_W); };
    auto LUo = [&](int row, int dcol) {
        return *reinterpret_cast<const float4 *>(su_c + row * SU_W + dcol);
    };
    auto LD = [&](int row) { return *reinterpret_cast<const float4 *>(sd_c + row * SU_W); };
    auto LDo = [&](int row, int dcol) {
        return *reinterpret_cast<const float4 *>(sd_c + row * SU_W + dcol);
    };

    // u rows of the vertical window, in u-tile rows (tile row + HALO_U)
    const int ub = r0 + HALO_U;
    float4 w0 = LU(ub - 4), w1 = LU(ub - 3), w2 = LU(ub - 2), w3 = LU(ub - 1), w4 = LU(ub);
    float4 x0 = mul4(g_central4(w0, w1, w3, w4), rdx);  // u_x at tile row r0-2
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = LU(ub + 1);
    float4 x1 = mul4(g_central4(w0, w1, w3, w4), rdx);  // r0-1
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = LU(ub + 2);
    float4 x2 = mul4(g_central4(w0, w1, w3, w4), rdx);  // r0
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = LU(ub + 3);
    float4 x3 = mul4(g_central4(w0, w1, w3, w4), rdx);  // r0+1
    // D rows of the vertical window, in D-tile rows (tile row + HALO_D)
    const int db = r0 + HALO_D;
    float4 d0 = LD(db - 2), d1 = LD(db - 1), d2 = LD(db), d3 = LD(db + 1), d4;

#pragma unroll
    for (int rr = 0; rr < MR; ++rr) {
        const int i = i0 + r0 + rr;
        const int64_t goff = (int64_t)i * pitch + j;
        float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f), wv4 = v4;
        if (i < H && col_in) {
            v4 = __ldg(reinterpret_cast<const float4 *>(a.v + goff));
            wv4 = __ldg(reinterpret_cast<const float4 *>(a.w + goff));
        }
        // vertical u: window now centred two rows below this cell
        w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = LU(ub + rr + 4);
        const float4 x4 = mul4(g_central4(w0, w1, w3, w4), rdx);  // u_x at r0+rr+2
        const float4 uxx = mul4(g_central4(x0, x1, x3, x4), rdx);
        const float4 uxc = x2;
        const float4 uc = w0;  // u at this cell row
        // horizontal u: columns j-4 .. j+7
        const float4 ul = LUo(ub + rr, -4), ur = LUo(ub + rr, 4);
        const float e[12] = {ul.x, ul.y, ul.z, ul.w, uc.x, uc.y, uc.z, uc.w,
                             ur.x, ur.y, ur.z, ur.w};
        float uy[8];  // u_y at columns j-2 .. j+5
#pragma unroll
        for (int m = 0; m < 8; ++m) uy[m] = g_central(e[m], e[m + 1], e[m + 3], e[m + 4]) * rdx;
        float uyy[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) uyy[m] = g_central(uy[m], uy[m + 1], uy[m + 3], uy[m + 4]) * rdx;
        // D and its derivatives
        d4 = LD(db + rr + 2);
        const float4 dxD = mul4(g_central4(d0, d1, d3, d4), rdx);
        const float4 dc = d2;
        const float4 dl = LDo(db + rr, -4), dr = LDo(db + rr, 4);
        const float f[12] = {dl.x, dl.y, dl.z, dl.w, dc.x, dc.y, dc.z, dc.w,
                             dr.x, dr.y, dr.z, dr.w};
        float dyD[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) dyD[m] = g_central(f[m + 2], f[m + 3], f[m + 5], f[m + 6]) * rdx;

        const float uu[4] = {uc.x, uc.y, uc.z, uc.w};
        const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
        const float ww[4] = {wv4.x, wv4.y, wv4.z, wv4.w};
        const float dd[4] = {dc.x, dc.y, dc.z, dc.w};
        const float dxv[4] = {dxD.x, dxD.y, dxD.z, dxD.w};
        const float uxv[4] = {uxc.x, uxc.y, uxc.z, uxc.w};
        const float uxxv[4] = {uxx.x, uxx.y, uxx.z, uxx.w};
        float ov[4], ow[4], ou[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            Reaction r = reaction(uu[m], vv[m], ww[m], a.m);
            if (active) {
                float acc = 0.0f;
                for (int s = 0; s < a.n_stim; ++s) {
                    if (!((active >> s) & 1u)) continue;
                    const Stim &st = a.stim[s];
                    const int jj = j + m;
                    float fv;
                    if (st.field) fv = (i < H && jj < W) ? __ldg(st.field + goff + m) : 0.0f;
                    else fv = (i >= st.r0 && i < st.r1 && jj >= st.c0 && jj < st.c1) ? st.amplitude : 0.0f;
                    if (fv != 0.0f) acc = fv;
                }
                if (acc != 0.0f) r.j_ion = acc;
            }
            const float du = diffusion(dd[m], dxv[m], dyD[m], uxv[m], uy[m + 2], uxxv[m], uyy[m]) + r.j_ion;
            if (DERIV) {
                ov[m] = r.dv;
                ow[m] = r.dw;
                ou[m] = du;
            } else {
                ov[m] = fmaf(r.dv, a.dt, vv[m]);
                ow[m] = fmaf(r.dw, a.dt, ww[m]);
                ou[m] = fmaf(du, a.dt, uu[m]);
            }
        }
        // store: whole float4 inside the band-free interior, else only the interior cells
        if (interior) {
            *reinterpret_cast<float4 *>(a.vo + goff) = make_float4(ov[0], ov[1], ov[2], ov[3]);
            *reinterpret_cast<float4 *>(a.wo + goff) = make_float4(ow[0], ow[1], ow[2], ow[3]);
            *reinterpret_cast<float4 *>(a.uo + goff) = make_float4(ou[0], ou[1], ou[2], ou[3]);
        } else if (i >= BAND && i < H - BAND) {
            const bool full = j >= BAND && j + 3 < W - BAND;
            if (full) {
                *reinterpret_cast<float4 *>(a.vo + goff) = make_float4(ov[0], ov[1], ov[2], ov[3]);
                *reinterpret_cast<float4 *>(a.wo + goff) = make_float4(ow[0], ow[1], ow[2], ow[3]);
                *reinterpret_cast<float4 *>(a.uo + goff) = make_float4(ou[0], ou[1], ou[2], ou[3]);
            } else {
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const int jj = j + m;
                    if (jj >= BAND && jj < W - BAND) {
                        a.vo[goff + m] = ov[m];
                        a.wo[goff + m] = ow[m];
                        a.uo[goff + m] = ou[m];
                    }
                }
            }
        }
        x0 = x1; x1 = x2; x2 = x3; x3 = x4;
        d0 = d1; d1 = d2; d2 = d3; d3 = d4;
    }

    if (!interior) {
        // cells of this tile within BAND of an edge
        const int ih = min(TY, H - i0), jw = min(TX, W - j0);
        for (int idx = tid; idx < ih * jw; idx += NT) {
            const int i = i0 + idx / jw, jj = j0 + idx % jw;
            if (i < BAND || i >= H - BAND || jj < BAND || jj >= W - BAND)
                boundary_cell(a, active, DERIV, i, jj);
        }
    }
}

cudaError_t launch_step(const CUtensorMap &tm_u, const CUtensorMap &tm_d, const StepArgs &a,
                        bool deriv, cudaStream_t stream) {
    dim3 grid((a.W + TX - 1) / TX, (a.H + TY - 1) / TY);
    if (deriv)
        fk_step_kernel<true><<<grid, NT, SMEM_STEP_BYTES, stream>>>(tm_u, tm_d, a);
    else
        fk_step_kernel<false><<<grid, NT, SMEM_STEP_BYTES, stream>>>(tm_u, tm_d, a);
    return cudaGetLastError();
}

}  // namespace fk
