// Tile-level device code shared by the step kernels (one launch per step, batched, dataflow):
// the per-cell boundary path, the two-pass tile computation, TMA issue/store helpers.
//
// Reference semantics: cardiax/solve.py:26-70 (step + step_euler, with gradient x6, stimulate
// and the edge pads fused).  Memory layout: SoA float32 planes, row pitch a multiple of 4
// floats.
//
// Per tile: one TMA transaction brings the u tile with a 4-cell halo and the D tile with a
// 2-row halo into shared memory (out-of-grid cells read as zero); v and w are read straight
// into registers with 16-byte loads.  Each thread streams RPT rows of 4 columns:
//   vertical derivatives   u_x, u_xx, D_x from register windows of shared-memory rows;
//   horizontal derivatives u_y, u_yy, D_y from three 16-byte shared-memory reads per row.
// Tiles that touch the grid edge clamp their halo to the reference's edge padding and pick
// the one-sided stencil rows; one-row or one-column sliver tiles recompute the cells within 4
// of an edge with a per-cell path that reads global memory with clamped indices.
//
// State planes are read with L2-coherent loads (ld.global.cg), never through the read-only
// path: in the dataflow kernel they are rewritten by other CTAs while the kernel runs.
//
// PK selects packed arithmetic (two cells per FP32 instruction, fk_pack.cuh) for every stencil
// whose formula is uniform across a thread's 4 columns, the reaction, the diffusion sum and the
// Euler update; it needs the launch's PackConsts.  Both modes produce the same bits.
#pragma once
#include "fk_pack.cuh"
#include "fk_ptx.cuh"
#include "fk_step.cuh"

namespace FK_TILE_NS {  // see fk_step.cuh

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// ---- per-cell boundary path ---------------------------------------------------------------
// Reads the input planes with the reference's edge padding: index -1 maps to 0, N to N-1.
struct Clamped {
    const float *p;
    int H, W, pitch;
    __device__ __forceinline__ float at(int r, int c) const {
        return __ldcg(p + (int64_t)clampi(r, 0, H - 1) * pitch + clampi(c, 0, W - 1));
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

// Activation bookkeeping for one cell (only touches memory on an upstroke).
__device__ __forceinline__ void record_activation(const StepArgs &a, float t, int64_t off,
                                                  float u_old, float u_new) {
    if (u_old < a.act_threshold && u_new >= a.act_threshold) {
        // through L2 (.cg): successive steps of a cell may run on different SMs
        const int32_t t1 = (int32_t)t + 1;
        __stcg(a.act_last + off, t1);
        if (__ldcg(a.act_first + off) < 0) __stcg(a.act_first + off, t1);
        __stcg(a.act_count + off, __ldcg(a.act_count + off) + 1);
    }
}

// Output tile in shared memory (dense TY x TX per plane) that the TMA stores write out; with
// null planes, cells go straight to the output state (a.vo, a.wo, a.uo) in global memory.
struct OutTile {
    float *v, *w, *u;
    int i0, j0;
};

template <bool ACT>
__device__ __noinline__ void boundary_cell(const StepArgs &a, float t, unsigned active, bool deriv,
                                           int i, int j, const OutTile &o, int heun = 0) {
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
    const float u = __ldcg(a.u + off), v = __ldcg(a.v + off), w = __ldcg(a.w + off),
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
    float ov, ow, ou;
    const int64_t plane = (int64_t)a.H * a.pitch;
    if (deriv) {
        ov = r.dv;
        ow = r.dw;
        ou = du;
    } else if (heun == 2) {  // x0 + (d1 + d2) h, d2 = this cell's derivative at x1
        ov = fmaf(__ldcg(a.d1 + off) + r.dv, a.h, __ldcg(a.x0 + off));
        ow = fmaf(__ldcg(a.d1 + plane + off) + r.dw, a.h, __ldcg(a.x0 + plane + off));
        ou = fmaf(__ldcg(a.d1 + 2 * plane + off) + du, a.h, __ldcg(a.x0 + 2 * plane + off));
    } else {
        ov = fmaf(r.dv, a.dt, v);
        ow = fmaf(r.dw, a.dt, w);
        ou = fmaf(du, a.dt, u);
        if (ACT) record_activation(a, t, off, u, ou);
        if (heun == 1) {
            __stcg(a.dso + off, r.dv);
            __stcg(a.dso + plane + off, r.dw);
            __stcg(a.dso + 2 * plane + off, du);
        }
    }
    if (o.v) {
        const int lo = (i - o.i0) * TX + (j - o.j0);
        o.v[lo] = ov;
        o.w[lo] = ow;
        o.u[lo] = ou;
    } else {
        __stcg(a.vo + off, ov);
        __stcg(a.wo + off, ow);
        __stcg(a.uo + off, ou);
    }
}

// Stimulus override for the 4 cells (i, j .. j+3) of one thread: later active stimuli win,
// a zero value leaves the ionic current (cardiax/solve.py:257-271).  Out of line: it runs only
// on the steps where some protocol is on.
static __device__ __noinline__ float4 apply_stimuli(const StepArgs &a, unsigned active, int i, int j,
                                                    int64_t goff, float4 jion4) {
    float j_ion[4] = {jion4.x, jion4.y, jion4.z, jion4.w};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int jj = j + m;
        if (i < 0 || i >= a.H || jj < 0 || jj >= a.W) continue;  // no stimulus outside the grid
        float acc = 0.0f;
        for (int s = 0; s < a.n_stim; ++s) {
            if (!((active >> s) & 1u)) continue;
            const Stim &st = a.stim[s];
            const float fv = st.field ? __ldg(st.field + goff + m)
                                      : ((i >= st.r0 && i < st.r1 && jj >= st.c0 && jj < st.c1)
                                             ? st.amplitude : 0.0f);
            if (fv != 0.0f) acc = fv;
        }
        if (acc != 0.0f) j_ion[m] = acc;
    }
    return make_float4(j_ion[0], j_ion[1], j_ion[2], j_ion[3]);
}

// Cells of tile (i0, j0) within BAND of an edge, enumerated compactly so that each thread
// takes ceil(count / NT) of them: a top strip, a bottom strip, and left/right strips between.
template <bool ACT>
__device__ __noinline__ void boundary_band(const StepArgs &a, float t, unsigned active, bool deriv,
                                           int i0, int j0, const OutTile &o, int heun = 0) {
    const int H = a.H, W = a.W;
    const int i1 = min(i0 + TY, H), j1 = min(j0 + TX, W);
    const int jw = j1 - j0;
    // interior rectangle of the tile (may be empty)
    const int ri0 = min(max(i0, BAND), i1), ri1 = max(min(i1, H - BAND), ri0);
    const int rj0 = min(max(j0, BAND), j1), rj1 = max(min(j1, W - BAND), rj0);
    const int n_top = (ri0 - i0) * jw, n_bot = (i1 - ri1) * jw;
    const int wl = rj0 - j0, wr = j1 - rj1, n_mid = (ri1 - ri0) * (wl + wr);
    const int total = n_top + n_bot + n_mid;
    for (int idx = threadIdx.x; idx < total; idx += NT) {
        int i, j;
        if (idx < n_top) {
            i = i0 + idx / jw;
            j = j0 + idx % jw;
        } else if (idx < n_top + n_bot) {
            const int k = idx - n_top;
            i = ri1 + k / jw;
            j = j0 + k % jw;
        } else {
            const int k = idx - n_top - n_bot;
            const int r = k / (wl + wr), c = k % (wl + wr);
            i = ri0 + r;
            j = c < wl ? j0 + c : rj1 + (c - wl);
        }
        boundary_cell<ACT>(a, t, active, deriv, i, j, o, heun);
    }
}

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }

// Shared-memory buffers of one pipeline stage (the haloed u and D tiles), and the tile's own
// v, w values (registers, loaded at the start of the tile) and output tiles.
struct Stage {
    float *u, *d;
};
struct TileIO {
    float4 v[RPT], w[RPT];   // input v, w of this thread's pass-2 cells
    float *ov, *ow, *ou;     // dense output tiles
};

__device__ __forceinline__ Stage stage_at(unsigned char *base, int s) {
    unsigned char *p = base + s * SMEM_STAGE_BYTES;
    Stage st;
    st.u = reinterpret_cast<float *>(p);
    st.d = reinterpret_cast<float *>(p + SMEM_U_BYTES);
    return st;
}

__device__ __forceinline__ void issue_tile(const CUtensorMap *u, const CUtensorMap *d,
                                           const Stage &st, uint64_t *bar, int i0, int j0) {
    mbar_arrive_expect_tx(bar, SMEM_STAGE_BYTES);
    tma_load_2d(st.u, u, j0 - HALO_U, i0 - HALO_U, bar);
    tma_load_2d(st.d, d, j0 - HALO_U, i0 - HALO_D, bar);
}
__device__ __forceinline__ void issue_tile(const StepMaps &tm, const Stage &st, uint64_t *bar,
                                           int i0, int j0) {
    issue_tile(&tm.u, &tm.d, st, bar, i0, j0);
}

// issue_tile with L2 policies: the input state's u (read for the last time: the next step
// overwrites this buffer) and D (re-read every step).
__device__ __forceinline__ void issue_tile_hinted(const StepMaps &tm, const Stage &st,
                                                  uint64_t *bar, int i0, int j0, uint64_t pol_u,
                                                  uint64_t pol_d) {
    mbar_arrive_expect_tx(bar, SMEM_STAGE_BYTES);
    tma_load_2d_hint(st.u, &tm.u, j0 - HALO_U, i0 - HALO_U, bar, pol_u);
    tma_load_2d_hint(st.d, &tm.d, j0 - HALO_U, i0 - HALO_D, bar, pol_d);
}

// A tile lying wholly inside the grid (its loads and stores need no bounds checks).
__device__ __forceinline__ bool tile_in_grid(int i0, int j0, int H, int W) {
    return i0 + TY <= H && j0 + TX <= W;
}

// This thread's v, w for pass 2 (16-byte loads, zero outside the grid), read with `load`.
template <class Load>
__device__ __forceinline__ void load_vw_with(const StepArgs &a, int i0, int j0, TileIO &io,
                                             Load load) {
    const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
    const int j = j0 + 4 * tx;
    if (tile_in_grid(i0, j0, a.H, a.W)) {
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int64_t off = (int64_t)(i0 + RPT * ty + k) * a.pitch + j;
            io.v[k] = load(a.v + off);
            io.w[k] = load(a.w + off);
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        const int i = i0 + RPT * ty + k;
        io.v[k] = io.w[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < a.H && j < a.W) {
            const int64_t off = (int64_t)i * a.pitch + j;
            io.v[k] = load(a.v + off);
            io.w[k] = load(a.w + off);
        }
    }
}

// load_vw with an L2 policy (the v, w read here are read for the last time).
__device__ __forceinline__ void load_vw_hinted(const StepArgs &a, int i0, int j0, TileIO &io,
                                               uint64_t pol) {
    load_vw_with(a, i0, j0, io, [pol](const float *p) { return ld_f4_hint(p, pol); });
}

__device__ __forceinline__ void load_vw(const StepArgs &a, int i0, int j0, TileIO &io) {
    load_vw_with(a, i0, j0, io,
                 [](const float *p) { return __ldcg(reinterpret_cast<const float4 *>(p)); });
}

// Edge tiles: replace the zero fill of the out-of-grid halo by the reference's edge padding
// (jnp.pad(..., "edge")): a cell at grid row x, column y outside the grid takes the value of
// (clamp(x, 0, H-1), clamp(y, 0, W-1)).  Only the 4 rows and columns beyond each edge are
// rewritten: the stencils of in-grid cells read at most 2 beyond (u_x, u_y and D at rows /
// columns -2 .. H+1 / W+1), and what is computed for out-of-grid cells is never stored.  Every
// source cell is inside the grid, hence never a target: one pass, no barrier inside.
// Buffer row b holds grid row i0 - halo_rows + b, buffer column c grid column j0 - HALO_U + c.
// Work: the band columns of the in-grid rows, one cell per item (4 or 8 items per row, only for
// the sides the tile touches), and the band rows as 16-byte groups (a group that straddles a
// column edge is copied cell by cell).
static __device__ __noinline__ void clamp_halo(float *buf, int rows, int halo_rows, int i0, int j0,
                                               int H, int W) {
    const int base_r = i0 - halo_rows, base_c = j0 - HALO_U;
    // band rows: grid rows -4 .. -1 and H .. H+3 inside the buffer; the in-grid rows between
    const int t_lo = max(0, -4 - base_r), t_hi = min(rows, -base_r);
    const int b_lo = max(0, H - base_r), b_hi = min(rows, H + 4 - base_r);
    const int nt = max(0, t_hi - t_lo), nb = max(0, b_hi - b_lo);
    const int g_lo = max(0, -base_r), g_hi = min(rows, H - base_r);
    // band columns inside the buffer: [lc0, lc1) left of the grid, [rc0, rc1) right of it
    const int lc0 = max(0, -4 - base_c), lc1 = max(0, min(SW, -base_c));
    const int rc0 = max(0, W - base_c), rc1 = min(SW, W + 4 - base_c);
    const int nl = max(0, lc1 - lc0), nr = max(0, rc1 - rc0);
    const int sh = (nl > 0 && nr > 0) ? 3 : 2;  // items per in-grid row: 8 (both sides) or 4
    const int n_cols = (nl + nr > 0) ? max(0, g_hi - g_lo) << sh : 0;
    constexpr int Q = SW / 4;  // 16-byte groups per buffer row
    const int n_rows = (nt + nb) * Q;
    for (int it = threadIdx.x; it < n_cols + n_rows; it += NT) {
        if (it < n_cols) {
            const int b = g_lo + (it >> sh), m = it & ((1 << sh) - 1);
            int c;
            if (sh == 3) c = m < 4 ? (m < nl ? lc0 + m : -1) : (m - 4 < nr ? rc0 + m - 4 : -1);
            else if (nl > 0) c = m < nl ? lc0 + m : -1;
            else c = m < nr ? rc0 + m : -1;
            if (c < 0) continue;
            buf[b * SW + c] = buf[b * SW + clampi(base_c + c, 0, W - 1) - base_c];
        } else {  // whole band rows, corners included
            const int k = it - n_cols, rr = k / Q, c = 4 * (k - rr * Q);
            const int b = rr < nt ? t_lo + rr : b_lo + (rr - nt);
            const float *src = buf + (clampi(base_r + b, 0, H - 1) - base_r) * SW;
            float *dst = buf + b * SW;
            if (base_c + c >= 0 && base_c + c + 3 <= W - 1) {
                st4(dst + c, ld4(src + c));
            } else {
#pragma unroll
                for (int m = 0; m < 4; ++m) dst[c + m] = src[clampi(base_c + c + m, 0, W - 1) - base_c];
            }
        }
    }
}

// One tile: pass 1 (first derivatives into shared memory), pass 2 (everything else).
// EDGE: the tile touches the grid edge (and is not a one-row or one-column sliver): the halo
// is clamped and every derivative picks the reference's row type, exactly as the padded
// arrays of cardiax/solve.py:29-32,49-54 do.
//
// DIRECT: pass 2 writes the new state straight to global memory with 16-byte stores
// instead of into output tiles for TMA stores.  The caller then needs no barrier after the tile:
// the one barrier between the passes also votes on `ok` (this thread's wait for the tile's TMA
// data; the tile is abandoned and false returned when any thread's wait failed) and is followed
// by `after_barrier` (every thread has finished the previous tile by then).  band_mask: store
// no cell within BAND of an edge (a sliver tile's band is recomputed per cell afterwards).
struct NoHook {
    __device__ void operator()() const {}
};
// The per-tissue pair constants of the packed path: 1/dx and dt, each held twice.  A one-tissue
// launch passes the fields of its PackConsts parameter (constant-bank operands after inlining);
// the batched kernel passes its current tissue's values in registers.
struct PairScale {
    float2 rdx, dt;
};
template <bool DERIV, bool ACT, bool EDGE, bool PK, bool DIRECT = false, int HEUN = 0, class P1,
          class P2 = NoHook>
__device__ __forceinline__ bool compute_tile(const StepArgs &a, const PackConsts *pk, PairScale ps,
                                             float t,
                                             const Stage &st, float *sux, float *suy,
                                             const TileIO &io, unsigned active, int i0, int j0,
                                             P1 &&after_pass1, bool ok = true,
                                             P2 &&after_barrier = P2{}, bool band_mask = false) {
    const int tid = threadIdx.x;
    const int H = a.H, W = a.W, pitch = a.pitch;
    const float rdx = a.rdx;
    float *su = st.u, *sd = st.d;

    if (EDGE) {
        clamp_halo(su, SU_H, HALO_U, i0, j0, H, W);
        clamp_halo(sd, SD_H, HALO_D, i0, j0, H, W);
        // the stage is refilled by TMA later: order these generic writes before that
        if (DIRECT) fence_async_smem();
        __syncthreads();
    }

    // ---- pass 1: u_x (tile rows -2 .. TY+1) and u_y (tile columns -2 .. TX+1) -------------
#pragma unroll PASS1_UNROLL
    for (int it = tid; it < SUX_H * NTX; it += NT) {
        const int r = it / NTX, q = it % NTX;
        const float *b = su + (r + 2) * SW + HALO_U + 4 * q;  // u row of ux row r
        if constexpr (PK) {
            const PackConsts &kc = *pk;
            Quad o;
            const int x = i0 - 2 + r;  // global row of this u_x row
            if (!EDGE || (x > 0 && x < H - 1))
                o = q_central(kc, ld_quad(b - 2 * SW), ld_quad(b - SW), ld_quad(b + SW),
                              ld_quad(b + 2 * SW));
            else if (x <= 0)
                o = q_head(kc, ld_quad(b), ld_quad(b + SW), ld_quad(b + 2 * SW), ld_quad(b + 3 * SW));
            else
                o = q_tail(kc, ld_quad(b - 3 * SW), ld_quad(b - 2 * SW), ld_quad(b - SW), ld_quad(b));
            o = q_scale(o, ps.rdx);
            st4(sux + r * TX + 4 * q, make_float4(o.lo.x, o.lo.y, o.hi.x, o.hi.y));
            continue;
        }
        float4 o;
        if (!EDGE) {
            o = g_central4(ld4(b - 2 * SW), ld4(b - SW), ld4(b + SW), ld4(b + 2 * SW));
        } else {
            const int x = i0 - 2 + r;  // global row of this u_x row
            if (x <= 0)
                o = [&] {
                    const float4 a0 = ld4(b), a1 = ld4(b + SW), a2 = ld4(b + 2 * SW), a3 = ld4(b + 3 * SW);
                    return make_float4(g_head(a0.x, a1.x, a2.x, a3.x), g_head(a0.y, a1.y, a2.y, a3.y),
                                       g_head(a0.z, a1.z, a2.z, a3.z), g_head(a0.w, a1.w, a2.w, a3.w));
                }();
            else if (x >= H - 1)
                o = [&] {
                    const float4 a0 = ld4(b - 3 * SW), a1 = ld4(b - 2 * SW), a2 = ld4(b - SW), a3 = ld4(b);
                    return make_float4(g_tail(a0.x, a1.x, a2.x, a3.x), g_tail(a0.y, a1.y, a2.y, a3.y),
                                       g_tail(a0.z, a1.z, a2.z, a3.z), g_tail(a0.w, a1.w, a2.w, a3.w));
                }();
            else
                o = g_central4(ld4(b - 2 * SW), ld4(b - SW), ld4(b + SW), ld4(b + 2 * SW));
        }
        st4(sux + r * TX + 4 * q, mul4(o, rdx));
    }
#pragma unroll PASS1_UNROLL
    for (int it = tid; it < TY * NTX; it += NT) {
        const int r = it / NTX, q = it % NTX;
        const float *b = su + (r + HALO_U) * SW + 4 * q;  // columns j0+4q-4 .. j0+4q+7
        const float4 x0 = ld4(b), x1 = ld4(b + 4), x2 = ld4(b + 8);
        const float e[12] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w,
                             x2.x, x2.y, x2.z, x2.w};
        // every quad takes the central rows; in an edge tile the elements at columns 0, W-1
        // and W are then recomputed with the one-sided rows (few threads, short)
        const int y0 = j0 + 4 * q;
        float o[4];
        if constexpr (PK) {
            const PackConsts &kc = *pk;  // u_y at columns c .. c+3 as the pairs (c, c+1), (c+2, c+3)
            const float2 lo = p_mul(pg_central_row(kc, e[2], e[3], e[4], e[5], e[6], e[7]), ps.rdx);
            const float2 hi = p_mul(pg_central_row(kc, e[4], e[5], e[6], e[7], e[8], e[9]), ps.rdx);
            o[0] = lo.x;
            o[1] = lo.y;
            o[2] = hi.x;
            o[3] = hi.y;
        } else {
#pragma unroll
            for (int m = 0; m < 4; ++m) o[m] = g_central(e[m + 2], e[m + 3], e[m + 5], e[m + 6]) * rdx;
        }
        // in an edge tile, few quads: column 0 (head row), columns W-1 and W (tail rows)
        if (EDGE && y0 == 0) o[0] = g_head(e[4], e[5], e[6], e[7]) * rdx;
        if (EDGE && y0 <= W && W - 1 <= y0 + 3) {
            if (y0 + 3 == W - 1) {  // the quad ends at column W-1 (W a multiple of 4)
                o[3] = g_tail(e[4], e[5], e[6], e[7]) * rdx;
            } else {
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (y0 + m == W - 1 || y0 + m == W)
                        o[m] = g_tail(e[m + 1], e[m + 2], e[m + 3], e[m + 4]) * rdx;
            }
        }
        st4(suy + r * SW + HALO_U + 4 * q, make_float4(o[0], o[1], o[2], o[3]));
    }
    if (tid >= NT - TY * 4) {  // the 2 + 2 halo columns of u_y (threads with one ux item less)
        const int h = tid - (NT - TY * 4);
        const int r = h / 4, k = h % 4;
        const int c = k < 2 ? 2 + k : TX + HALO_U + (k - 2);  // same column index in su and suy
        const float *row = su + (r + HALO_U) * SW;
        float o;
        if (!EDGE) {
            o = g_central(row[c - 2], row[c - 1], row[c + 1], row[c + 2]);
        } else {
            const int y = j0 - HALO_U + c;
            if (y <= 0) o = g_head(row[c], row[c + 1], row[c + 2], row[c + 3]);
            else if (y >= W - 1) o = g_tail(row[c - 3], row[c - 2], row[c - 1], row[c]);
            else o = g_central(row[c - 2], row[c - 1], row[c + 1], row[c + 2]);
        }
        suy[r * SW + c] = o * rdx;
    }
    after_pass1();  // every thread (the hook picks its warps): free the output tiles, start loads
    if constexpr (DIRECT) {
        if (__syncthreads_or(!ok)) return false;
        after_barrier();
    } else {
        __syncthreads();
    }

    // ---- pass 2: second derivatives, D terms, reaction, stimulus, Euler update --------------
    // whole: every cell of the tile is stored (an interior tile: inside the grid, no band)
    const bool whole = !EDGE && !band_mask;
    const int tx = tid % NTX, ty = tid / NTX;
    const int j = j0 + 4 * tx;
    // PK: the u_x and D rows RPT*ty-2 .. RPT*ty+RPT+1 of this thread's quad, read once for all
    // of its rows (entry q holds row RPT*ty - 2 + q)
    Quad uxr[PK ? RPT + 4 : 1], dxr[PK ? RPT + 4 : 1];
    if constexpr (PK) {
#pragma unroll
        for (int q = 0; q < RPT + 4; ++q) {
            uxr[q] = ld_quad(sux + (RPT * ty + q) * TX + 4 * tx);
            dxr[q] = ld_quad(sd + (RPT * ty + q) * SW + HALO_U + 4 * tx);
        }
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        const int r = RPT * ty + k;
        const int i = i0 + r;
        const int64_t goff = (int64_t)i * pitch + j;
        if constexpr (PK) {
            const PackConsts &kc = *pk;
            const float *db = sd + (r + HALO_D) * SW + HALO_U + 4 * tx;
            const int o = k + 2;  // window entry of row r
            const Quad uxc = uxr[o], dcq = dxr[o];
            Quad uxx, dxD;
            if (!EDGE || (i != 0 && i != H - 1)) {
                uxx = q_central(kc, uxr[o - 2], uxr[o - 1], uxr[o + 1], uxr[o + 2]);
                dxD = q_central(kc, dxr[o - 2], dxr[o - 1], dxr[o + 1], dxr[o + 2]);
            } else if (k == 0 && i == 0) {  // head rows on u_x rows 0..3 and D rows 0..3
                // row r+3 lies beyond the window when a thread owns one row (RPT == 1)
                const Quad ux3 = o + 3 < RPT + 4 ? uxr[o + 3 < RPT + 4 ? o + 3 : 0]
                                                 : ld_quad(sux + (r + 5) * TX + 4 * tx);
                const Quad d3 = o + 3 < RPT + 4 ? dxr[o + 3 < RPT + 4 ? o + 3 : 0]
                                                : ld_quad(sd + (r + 3 + HALO_D) * SW + HALO_U + 4 * tx);
                uxx = q_head(kc, uxr[o], uxr[o + 1], uxr[o + 2], ux3);
                dxD = q_head(kc, dxr[o], dxr[o + 1], dxr[o + 2], d3);
            } else {  // i == H-1: tail rows on rows H-4 .. H-1 (row r-3 read here when k == 0)
                const float *xb = sux + (r + 2) * TX + 4 * tx;
                const Quad ux3 = k >= 1 ? uxr[k >= 1 ? o - 3 : 0] : ld_quad(xb - 3 * TX);
                const Quad d3 = k >= 1 ? dxr[k >= 1 ? o - 3 : 0] : ld_quad(db - 3 * SW);
                uxx = q_tail(kc, ux3, uxr[o - 2], uxr[o - 1], uxc);
                dxD = q_tail(kc, d3, dxr[o - 2], dxr[o - 1], dcq);
            }
            uxx = q_scale(uxx, ps.rdx);
            dxD = q_scale(dxD, ps.rdx);
            const float *yb = suy + r * SW + 4 * tx;
            const float4 y0 = ld4(yb), y1 = ld4(yb + 4), y2 = ld4(yb + 8);
            const float4 dl = ld4(db - 4), dr = ld4(db + 4);
            const float4 uc = ld4(su + (r + HALO_U) * SW + HALO_U + 4 * tx);
            const float4 vc = io.v[k], wc = io.w[k];
            const float f[12] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w,
                                 y2.x, y2.y, y2.z, y2.w};  // u_y at columns j-4 .. j+7
            const float g[12] = {dl.x, dl.y, dl.z, dl.w, dcq.lo.x, dcq.lo.y, dcq.hi.x, dcq.hi.y,
                                 dr.x, dr.y, dr.z, dr.w};  // D at columns j-4 .. j+7
            float2 uyy_lo = p_mul(pg_central_row(kc, f[2], f[3], f[4], f[5], f[6], f[7]), ps.rdx);
            float2 uyy_hi = p_mul(pg_central_row(kc, f[4], f[5], f[6], f[7], f[8], f[9]), ps.rdx);
            float2 dyD_lo = p_mul(pg_central_row(kc, g[2], g[3], g[4], g[5], g[6], g[7]), ps.rdx);
            float2 dyD_hi = p_mul(pg_central_row(kc, g[4], g[5], g[6], g[7], g[8], g[9]), ps.rdx);
            if (EDGE && (j == 0 || (j <= W - 1 && W - 1 <= j + 3))) {
                // the one-sided rows at column 0 (head) and W-1 (tail), second derivative / D_y
                float uy4[4] = {uyy_lo.x, uyy_lo.y, uyy_hi.x, uyy_hi.y};
                float dy4[4] = {dyD_lo.x, dyD_lo.y, dyD_hi.x, dyD_hi.y};
                if (j == 0) {
                    uy4[0] = g_head(f[4], f[5], f[6], f[7]) * rdx;
                    dy4[0] = g_head(g[4], g[5], g[6], g[7]) * rdx;
                }
                if (j + 3 == W - 1) {  // the quad ends at column W-1 (W a multiple of 4)
                    uy4[3] = g_tail(f[4], f[5], f[6], f[7]) * rdx;
                    dy4[3] = g_tail(g[4], g[5], g[6], g[7]) * rdx;
                } else {
#pragma unroll
                    for (int m = 0; m < 3; ++m)
                        if (j + m == W - 1) {
                            uy4[m] = g_tail(f[m + 1], f[m + 2], f[m + 3], f[m + 4]) * rdx;
                            dy4[m] = g_tail(g[m + 1], g[m + 2], g[m + 3], g[m + 4]) * rdx;
                        }
                }
                uyy_lo = mk2(uy4[0], uy4[1]);
                uyy_hi = mk2(uy4[2], uy4[3]);
                dyD_lo = mk2(dy4[0], dy4[1]);
                dyD_hi = mk2(dy4[2], dy4[3]);
            }
            const float2 u_lo = mk2(uc.x, uc.y), u_hi = mk2(uc.z, uc.w);
            const float2 v_lo = mk2(vc.x, vc.y), v_hi = mk2(vc.z, vc.w);
            const float2 w_lo = mk2(wc.x, wc.y), w_hi = mk2(wc.z, wc.w);
            // the reaction per cell in scalar form (lane-wise the operations of p_reaction; at
            // 2048^2 the scalar form measured 2 % faster, register pairs cost moves here)
            const Reaction q0 = reaction(uc.x, vc.x, wc.x, a.m);
            const Reaction q1 = reaction(uc.y, vc.y, wc.y, a.m);
            const Reaction q2 = reaction(uc.z, vc.z, wc.z, a.m);
            const Reaction q3 = reaction(uc.w, vc.w, wc.w, a.m);
            PairReaction rl, rh;
            rl.dv = mk2(q0.dv, q1.dv);
            rl.dw = mk2(q0.dw, q1.dw);
            rl.j_ion = mk2(q0.j_ion, q1.j_ion);
            rh.dv = mk2(q2.dv, q3.dv);
            rh.dw = mk2(q2.dw, q3.dw);
            rh.j_ion = mk2(q2.j_ion, q3.j_ion);
            float2 j_lo = rl.j_ion, j_hi = rh.j_ion;
            if (active) {
                const float4 js = apply_stimuli(a, active, i, j, goff,
                                                make_float4(j_lo.x, j_lo.y, j_hi.x, j_hi.y));
                j_lo = mk2(js.x, js.y);
                j_hi = mk2(js.z, js.w);
            }
            // del u = D (u_xx + u_yy) + D_x u_x + D_y u_y, du = del u + J, with no packed
            // multiply feeding a packed add (fk_pack.cuh: contraction hazard)
            float2 du_lo = p_mul(dcq.lo, add_products(uxx.lo, uyy_lo));
            du_lo = p_fma(dxD.lo, uxc.lo, du_lo);
            du_lo = p_fma(dyD_lo, mk2(f[4], f[5]), du_lo);
            du_lo = p_add_product(kc, du_lo, j_lo);
            float2 du_hi = p_mul(dcq.hi, add_products(uxx.hi, uyy_hi));
            du_hi = p_fma(dxD.hi, uxc.hi, du_hi);
            du_hi = p_fma(dyD_hi, mk2(f[6], f[7]), du_hi);
            du_hi = p_add_product(kc, du_hi, j_hi);
            float2 nv_lo, nv_hi, nw_lo, nw_hi, nu_lo, nu_hi;
            if (DERIV) {
                nv_lo = rl.dv;
                nv_hi = rh.dv;
                nw_lo = rl.dw;
                nw_hi = rh.dw;
                nu_lo = du_lo;
                nu_hi = du_hi;
            } else if (HEUN == 2) {  // x0 + (d1 + d2) h; the input state is x1
                const int64_t pl = (int64_t)H * pitch;
                const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                float4 xv = z, xw = z, xu = z, dv1 = z, dw1 = z, du1 = z;
                if (whole || (i < H && j < W)) {
                    xv = __ldcg(reinterpret_cast<const float4 *>(a.x0 + goff));
                    xw = __ldcg(reinterpret_cast<const float4 *>(a.x0 + pl + goff));
                    xu = __ldcg(reinterpret_cast<const float4 *>(a.x0 + 2 * pl + goff));
                    dv1 = __ldcg(reinterpret_cast<const float4 *>(a.d1 + goff));
                    dw1 = __ldcg(reinterpret_cast<const float4 *>(a.d1 + pl + goff));
                    du1 = __ldcg(reinterpret_cast<const float4 *>(a.d1 + 2 * pl + goff));
                }
                const float2 hh = mk2(a.h, a.h);
                nv_lo = p_fma(p_add(mk2(dv1.x, dv1.y), rl.dv), hh, mk2(xv.x, xv.y));
                nv_hi = p_fma(p_add(mk2(dv1.z, dv1.w), rh.dv), hh, mk2(xv.z, xv.w));
                nw_lo = p_fma(p_add(mk2(dw1.x, dw1.y), rl.dw), hh, mk2(xw.x, xw.y));
                nw_hi = p_fma(p_add(mk2(dw1.z, dw1.w), rh.dw), hh, mk2(xw.z, xw.w));
                nu_lo = p_fma(p_add(mk2(du1.x, du1.y), du_lo), hh, mk2(xu.x, xu.y));
                nu_hi = p_fma(p_add(mk2(du1.z, du1.w), du_hi), hh, mk2(xu.z, xu.w));
            } else {
                nv_lo = p_fma(rl.dv, ps.dt, v_lo);
                nv_hi = p_fma(rh.dv, ps.dt, v_hi);
                nw_lo = p_fma(rl.dw, ps.dt, w_lo);
                nw_hi = p_fma(rh.dw, ps.dt, w_hi);
                nu_lo = p_fma(du_lo, ps.dt, u_lo);
                nu_hi = p_fma(du_hi, ps.dt, u_hi);
            }
            const float4 ov4 = make_float4(nv_lo.x, nv_lo.y, nv_hi.x, nv_hi.y);
            const float4 ow4 = make_float4(nw_lo.x, nw_lo.y, nw_hi.x, nw_hi.y);
            const float4 ou4 = make_float4(nu_lo.x, nu_lo.y, nu_hi.x, nu_hi.y);
            // a cell this tile stores: inside the grid, and outside the band when masked
            auto stored = [&](int jj) {
                return jj < W && !(band_mask && (i < BAND || i >= H - BAND || jj < BAND ||
                                                 jj >= W - BAND));
            };
            if constexpr (DIRECT) {
                if (whole || (i < H && j < W)) {
                    const int64_t pl = (int64_t)H * pitch;
                    // Heun stage 1 also stores d1 (the derivative at the input state)
                    const float4 d4v = make_float4(rl.dv.x, rl.dv.y, rh.dv.x, rh.dv.y);
                    const float4 d4w = make_float4(rl.dw.x, rl.dw.y, rh.dw.x, rh.dw.y);
                    const float4 d4u = make_float4(du_lo.x, du_lo.y, du_hi.x, du_hi.y);
                    if (whole || (!band_mask && j + 3 < W)) {
                        __stcg(reinterpret_cast<float4 *>(a.vo + goff), ov4);
                        __stcg(reinterpret_cast<float4 *>(a.wo + goff), ow4);
                        __stcg(reinterpret_cast<float4 *>(a.uo + goff), ou4);
                        if (HEUN == 1) {
                            __stcg(reinterpret_cast<float4 *>(a.dso + goff), d4v);
                            __stcg(reinterpret_cast<float4 *>(a.dso + pl + goff), d4w);
                            __stcg(reinterpret_cast<float4 *>(a.dso + 2 * pl + goff), d4u);
                        }
                    } else {
                        const float fv[4] = {ov4.x, ov4.y, ov4.z, ov4.w};
                        const float fw[4] = {ow4.x, ow4.y, ow4.z, ow4.w};
                        const float fu[4] = {ou4.x, ou4.y, ou4.z, ou4.w};
                        const float gv[4] = {d4v.x, d4v.y, d4v.z, d4v.w};
                        const float gw[4] = {d4w.x, d4w.y, d4w.z, d4w.w};
                        const float gu[4] = {d4u.x, d4u.y, d4u.z, d4u.w};
#pragma unroll
                        for (int m = 0; m < 4; ++m)
                            if (stored(j + m)) {
                                __stcg(a.vo + goff + m, fv[m]);
                                __stcg(a.wo + goff + m, fw[m]);
                                __stcg(a.uo + goff + m, fu[m]);
                                if (HEUN == 1) {
                                    __stcg(a.dso + goff + m, gv[m]);
                                    __stcg(a.dso + pl + goff + m, gw[m]);
                                    __stcg(a.dso + 2 * pl + goff + m, gu[m]);
                                }
                            }
                    }
                }
            } else {
                st4(io.ov + r * TX + 4 * tx, ov4);
                st4(io.ow + r * TX + 4 * tx, ow4);
                st4(io.ou + r * TX + 4 * tx, ou4);
            }
            if (ACT && !DERIV && i < H) {
                const float uo4[4] = {uc.x, uc.y, uc.z, uc.w};
                const float un4[4] = {ou4.x, ou4.y, ou4.z, ou4.w};
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (stored(j + m)) record_activation(a, t, goff + m, uo4[m], un4[m]);
            }
            continue;
        }
        const float *xb = sux + (r + 2) * TX + 4 * tx;
        const float4 uxc = ld4(xb);
        const float *db = sd + (r + HALO_D) * SW + HALO_U + 4 * tx;
        const float4 dc = ld4(db);
        float4 uxx, dxD;
        if (!EDGE || (i != 0 && i != H - 1)) {
            uxx = g_central4(ld4(xb - 2 * TX), ld4(xb - TX), ld4(xb + TX), ld4(xb + 2 * TX));
            dxD = g_central4(ld4(db - 2 * SW), ld4(db - SW), ld4(db + SW), ld4(db + 2 * SW));
        } else if (i == 0) {  // head rows on u_x rows 0..3 and D rows 0..3
            const float4 a0 = uxc, a1 = ld4(xb + TX), a2 = ld4(xb + 2 * TX), a3 = ld4(xb + 3 * TX);
            uxx = make_float4(g_head(a0.x, a1.x, a2.x, a3.x), g_head(a0.y, a1.y, a2.y, a3.y),
                              g_head(a0.z, a1.z, a2.z, a3.z), g_head(a0.w, a1.w, a2.w, a3.w));
            const float4 b0 = dc, b1 = ld4(db + SW), b2 = ld4(db + 2 * SW), b3 = ld4(db + 3 * SW);
            dxD = make_float4(g_head(b0.x, b1.x, b2.x, b3.x), g_head(b0.y, b1.y, b2.y, b3.y),
                              g_head(b0.z, b1.z, b2.z, b3.z), g_head(b0.w, b1.w, b2.w, b3.w));
        } else {  // i == H-1: tail rows on rows H-4 .. H-1
            const float4 a0 = ld4(xb - 3 * TX), a1 = ld4(xb - 2 * TX), a2 = ld4(xb - TX), a3 = uxc;
            uxx = make_float4(g_tail(a0.x, a1.x, a2.x, a3.x), g_tail(a0.y, a1.y, a2.y, a3.y),
                              g_tail(a0.z, a1.z, a2.z, a3.z), g_tail(a0.w, a1.w, a2.w, a3.w));
            const float4 b0 = ld4(db - 3 * SW), b1 = ld4(db - 2 * SW), b2 = ld4(db - SW), b3 = dc;
            dxD = make_float4(g_tail(b0.x, b1.x, b2.x, b3.x), g_tail(b0.y, b1.y, b2.y, b3.y),
                              g_tail(b0.z, b1.z, b2.z, b3.z), g_tail(b0.w, b1.w, b2.w, b3.w));
        }
        uxx = mul4(uxx, rdx);
        dxD = mul4(dxD, rdx);
        const float *yb = suy + r * SW + 4 * tx;
        const float4 y0 = ld4(yb), y1 = ld4(yb + 4), y2 = ld4(yb + 8);
        const float4 dl = ld4(db - 4), dr = ld4(db + 4);
        const float4 uc = ld4(su + (r + HALO_U) * SW + HALO_U + 4 * tx);
        const float4 vc = io.v[k], wc = io.w[k];

        const float f[12] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w,
                             y2.x, y2.y, y2.z, y2.w};
        const float g[12] = {dl.x, dl.y, dl.z, dl.w, dc.x, dc.y, dc.z, dc.w,
                             dr.x, dr.y, dr.z, dr.w};
        const float uu[4] = {uc.x, uc.y, uc.z, uc.w};
        const float vv[4] = {vc.x, vc.y, vc.z, vc.w};
        const float ww[4] = {wc.x, wc.y, wc.z, wc.w};
        const float dd[4] = {dc.x, dc.y, dc.z, dc.w};
        const float dxv[4] = {dxD.x, dxD.y, dxD.z, dxD.w};
        const float uxv[4] = {uxc.x, uxc.y, uxc.z, uxc.w};
        const float uxxv[4] = {uxx.x, uxx.y, uxx.z, uxx.w};
        float ov[4], ow[4], ou[4], jion[4], dv[4], dw[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const Reaction re = reaction(uu[m], vv[m], ww[m], a.m);
            jion[m] = re.j_ion;
            dv[m] = re.dv;
            dw[m] = re.dw;
        }
        if (active) {
            const float4 js = apply_stimuli(a, active, i, j, goff,
                                            make_float4(jion[0], jion[1], jion[2], jion[3]));
            jion[0] = js.x;
            jion[1] = js.y;
            jion[2] = js.z;
            jion[3] = js.w;
        }
        float uyy4[4], dyD4[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            uyy4[m] = g_central(f[m + 2], f[m + 3], f[m + 5], f[m + 6]);
            dyD4[m] = g_central(g[m + 2], g[m + 3], g[m + 5], g[m + 6]);
        }
        // in an edge tile, few quads: the one-sided rows at column 0 (head) and W-1 (tail)
        if (EDGE && j == 0) {
            uyy4[0] = g_head(f[4], f[5], f[6], f[7]);
            dyD4[0] = g_head(g[4], g[5], g[6], g[7]);
        }
        if (EDGE && j <= W - 1 && W - 1 <= j + 3) {
            if (j + 3 == W - 1) {  // the quad ends at column W-1 (W a multiple of 4)
                uyy4[3] = g_tail(f[4], f[5], f[6], f[7]);
                dyD4[3] = g_tail(g[4], g[5], g[6], g[7]);
            } else {
#pragma unroll
                for (int m = 0; m < 3; ++m)
                    if (j + m == W - 1) {
                        uyy4[m] = g_tail(f[m + 1], f[m + 2], f[m + 3], f[m + 4]);
                        dyD4[m] = g_tail(g[m + 1], g[m + 2], g[m + 3], g[m + 4]);
                    }
            }
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const float uyy = uyy4[m] * rdx;
            const float dyD = dyD4[m] * rdx;
            const float du = diffusion(dd[m], dxv[m], dyD, uxv[m], f[m + 4], uxxv[m], uyy) + jion[m];
            if (DERIV) {
                ov[m] = dv[m];
                ow[m] = dw[m];
                ou[m] = du;
            } else {
                ov[m] = fmaf(dv[m], a.dt, vv[m]);
                ow[m] = fmaf(dw[m], a.dt, ww[m]);
                ou[m] = fmaf(du, a.dt, uu[m]);
            }
        }
        auto stored = [&](int jj) {
            return jj < W && !(band_mask && (i < BAND || i >= H - BAND || jj < BAND ||
                                             jj >= W - BAND));
        };
        if constexpr (DIRECT) {
            if (whole || (i < H && j < W)) {
                if (whole || (!band_mask && j + 3 < W)) {
                    __stcg(reinterpret_cast<float4 *>(a.vo + goff), make_float4(ov[0], ov[1], ov[2], ov[3]));
                    __stcg(reinterpret_cast<float4 *>(a.wo + goff), make_float4(ow[0], ow[1], ow[2], ow[3]));
                    __stcg(reinterpret_cast<float4 *>(a.uo + goff), make_float4(ou[0], ou[1], ou[2], ou[3]));
                } else {
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        if (stored(j + m)) {
                            __stcg(a.vo + goff + m, ov[m]);
                            __stcg(a.wo + goff + m, ow[m]);
                            __stcg(a.uo + goff + m, ou[m]);
                        }
                }
            }
        } else {
            st4(io.ov + r * TX + 4 * tx, make_float4(ov[0], ov[1], ov[2], ov[3]));
            st4(io.ow + r * TX + 4 * tx, make_float4(ow[0], ow[1], ow[2], ow[3]));
            st4(io.ou + r * TX + 4 * tx, make_float4(ou[0], ou[1], ou[2], ou[3]));
        }
        if (ACT && !DERIV && i < H) {
#pragma unroll
            for (int m = 0; m < 4; ++m)
                if (stored(j + m)) record_activation(a, t, goff + m, uu[m], ou[m]);
        }
    }
    return true;
}

// A tile that needs the per-cell boundary path: the last row or column of tiles holds a
// single grid row or column (too few rows in the tile for the one-sided stencils).
__device__ __forceinline__ bool is_sliver(int i0, int j0, int H, int W) {
    return H - i0 < 2 || W - j0 < 2;
}

// A tile within BAND of a grid edge (a clamped edge tile, or a sliver).
__device__ __forceinline__ bool edge_tile(int i0, int j0, int H, int W) {
    return !(i0 >= BAND && i0 + TY <= H - BAND && j0 >= BAND && j0 + TX <= W - BAND);
}

// Interior tiles, clamped edge tiles, or slivers (interior passes + per-cell band).
// PK: packed arithmetic with the launch's constants *pk (null when !PK).
// DIRECT: see compute_tile; returns false when the tile was abandoned (a failed TMA wait).
// HEUN: 1 or 2 for the Heun stages (PK and DIRECT only).
template <bool DERIV, bool ACT, bool PK = false, bool DIRECT = false, int HEUN = 0, class P1,
          class P2 = NoHook>
__device__ __forceinline__ bool process_tile(const StepArgs &a, float t, const Stage &st,
                                             float *sux, float *suy, const TileIO &io,
                                             unsigned active, int i0, int j0, P1 &&after_pass1,
                                             const PackConsts *pk = nullptr,
                                             PairScale ps = PairScale{}, bool ok = true,
                                             P2 &&after_barrier = P2{}) {
    const int H = a.H, W = a.W;
    if (!edge_tile(i0, j0, H, W)) {
        return compute_tile<DERIV, ACT, false, PK, DIRECT, HEUN>(a, pk, ps, t, st, sux, suy, io, active,
                                                                 i0, j0, after_pass1, ok,
                                                                 after_barrier);
    } else if (!is_sliver(i0, j0, H, W)) {
        return compute_tile<DERIV, ACT, true, PK, DIRECT, HEUN>(a, pk, ps, t, st, sux, suy, io, active,
                                                                i0, j0, after_pass1, ok,
                                                                after_barrier);
    } else if (DIRECT) {
        // interior cells from the tile passes; the band cells per cell, straight to global memory
        if (!compute_tile<DERIV, ACT, false, PK, DIRECT, HEUN>(a, pk, ps, t, st, sux, suy, io, active,
                                                               i0, j0, after_pass1, ok,
                                                               after_barrier, true))
            return false;
        boundary_band<ACT && !DERIV>(a, t, active, DERIV, i0, j0,
                                     OutTile{nullptr, nullptr, nullptr, i0, j0}, HEUN);
        return true;
    } else {
        compute_tile<DERIV, false, false, PK>(a, pk, ps, t, st, sux, suy, io, active, i0, j0,
                                              after_pass1);
        __syncthreads();  // every cell of this tile is recomputed below where needed
        boundary_band<ACT && !DERIV>(a, t, active, DERIV, i0, j0,
                                     OutTile{io.ov, io.ow, io.ou, i0, j0});
        if (ACT && !DERIV) {  // interior cells of the sliver tile: record from the tile values
            const int tid = threadIdx.x;
            for (int idx = tid; idx < TY * TX; idx += NT) {
                const int i = i0 + idx / TX, j = j0 + idx % TX;
                if (i >= BAND && i < H - BAND && j >= BAND && j < W - BAND)
                    record_activation(a, t, (int64_t)i * a.pitch + j,
                                      st.u[(idx / TX + HALO_U) * SW + HALO_U + idx % TX],
                                      io.ou[idx]);
            }
        }
        return true;
    }
}

// Writes the output tiles with TMA stores (after all threads have written them).
__device__ __forceinline__ void store_tile(const CUtensorMap *ov, const CUtensorMap *ow,
                                           const CUtensorMap *ou, const TileIO &io, int i0,
                                           int j0, int issuer = 0) {
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == issuer) {
        tma_store_2d(ov, io.ov, j0, i0);
        tma_store_2d(ow, io.ow, j0, i0);
        tma_store_2d(ou, io.ou, j0, i0);
        bulk_commit();
    }
}
__device__ __forceinline__ void store_tile(const StepMaps &tm, const TileIO &io, int i0, int j0) {
    store_tile(&tm.ov, &tm.ow, &tm.ou, io, i0, j0);
}

// After an abandoned tile n (a TMA wait ran out): the loads still in flight are those of tiles
// n .. n+NSTAGE-2 that were issued -- issued(q) for tile n+q, i.e. first + q * stride < last --
// wait for each (bounded) so that no copy lands in shared memory after the CTA has exited.
// Thread 0 only; out of line, so that the abort path costs the step kernels no registers.
static __device__ __noinline__ void drain_stages(uint64_t *bar, int n, int first, int stride,
                                                 int last) {
    for (int q = 0; q < NSTAGE - 1; ++q)
        if (first + q * stride < last)
            mbar_wait_bounded(&bar[(n + q) % NSTAGE], ((n + q) / NSTAGE) & 1);
}

static_assert(sizeof(StepArgs) <= SMEM_ARGS_BYTES, "StepArgs does not fit its shared slot");

// Copies a StepArgs into shared memory (all threads; a barrier must follow).
__device__ __forceinline__ void stage_args(StepArgs *dst, const StepArgs *src) {
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(StepArgs) / 4); k += NT) d[k] = s[k];
}

}  // namespace FK_TILE_NS
