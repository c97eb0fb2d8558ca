// K2: temporally blocked Euler stepper -- K steps per tile between one load and one store.
//
// Replaces K consecutive step_euler calls of cardiax/solve.py:92-100 per launch.  A CTA loads
// its OY x OX output tile with a 4K-cell halo of u, v, w and D (plus 2 rows / 4 columns of
// margin so that every stencil read stays inside the buffer), then advances the region K times
// in shared memory: step s computes the region shrunk by 4(s+1) cells from the region shrunk by
// 4s (the u stencil reaches 4 cells: u_xx is the derivative of u_x), and the last step leaves
// exactly the output tile, which TMA stores write out.  v and w are updated in place (they are
// pointwise), u ping-pongs between two buffers.
//
// The per-cell arithmetic is the same code as the one-step kernel (fk_math.cuh, the same
// fused multiply-adds), so K blocked steps give the same bits as K single steps.  Tiles whose
// halo crosses the grid edge re-apply the reference's edge padding to u before every step
// (copies of row/column 0 and H-1/W-1 of the current state) and select the one-sided rows of
// cardiax/solve.py:225-254 per global row and column.  A grid whose last tile row or column is
// a single cell wide is not blocked (the one-sided rows there reach 5 cells inward, beyond the
// halo); the host runs it with the one-step kernel.
//
// Each blocked step recomputes the halo ring of the tile: the work per useful cell-update is
// sum_s |R_s| / (K |tile|), 1.2 for K = 2 on 32 x 64, 1.7 for K = 4, 8.9 for K = 8 on 16 x 16
// (the only K = 8 tile that fits in shared memory).
#include "fk_capi_internal.h"
#include "fk_tile.cuh"
#include "fk_tb.cuh"

namespace fk {

namespace {

template <int K, int OY, int OX>
struct TbGeom {
    static constexpr int RO = 2;                    // extra rows above / below the halo
    static constexpr int CO = 4;                    // extra columns left / right of the halo
    static constexpr int BY = OY + 8 * K + 2 * RO;  // buffer rows
    static constexpr int BX = OX + 8 * K + 2 * CO;  // buffer columns (multiple of 4)
    static constexpr int PLANE = BY * BX;           // floats per buffer
    // shared memory: u (2), v, w, D, u_x, u_y buffers; 3 dense output tiles
    static constexpr int BYTES = 7 * PLANE * 4 + 3 * OY * OX * 4;
    static constexpr int LOAD_BYTES = 4 * PLANE * 4;
    static_assert(BX % 4 == 0 && OX % 4 == 0, "float4 rows");
    static_assert(BX <= 256 && BY <= 256, "TMA box");
};

// Edge padding of the current state in a buffer whose element (0, 0) is global (gy0, gx0):
// rows -4..-1 take row 0, rows H..H+3 take row H-1, then the same for columns (corners get the
// corner cell).  Positions farther out are never read for in-grid cells.
template <int BY, int BX, int NTH>
__device__ __forceinline__ void tb_clamp(float *buf, int gy0, int gx0, int H, int W) {
    constexpr int BX4 = BX / 4;
    const int tid = threadIdx.x;
    for (int it = tid; it < 8 * BX4; it += NTH) {
        const int k = it / BX4, c4 = it % BX4;
        const int gr = k < 4 ? k - 4 : H + (k - 4);
        const int r = gr - gy0;
        const int src = (k < 4 ? 0 : H - 1) - gy0;
        if (r < 0 || r >= BY || src < 0 || src >= BY) continue;
        reinterpret_cast<float4 *>(buf + r * BX)[c4] = reinterpret_cast<const float4 *>(buf + src * BX)[c4];
    }
    __syncthreads();
    for (int it = tid; it < 8 * BY; it += NTH) {
        const int k = it & 7, r = it >> 3;
        const int gc = k < 4 ? k - 4 : W + (k - 4);
        const int c = gc - gx0;
        const int src = (k < 4 ? 0 : W - 1) - gx0;
        if (c < 0 || c >= BX || src < 0 || src >= BX) continue;
        buf[r * BX + c] = buf[r * BX + src];
    }
}

// One blocked step: from u_cur (and v, w, D) on region R_s to u_nxt, v, w on R_{s+1} (buffer
// rows [rr0, rr1), columns [cc0, cc1)), or into the dense output tiles when `last`.
template <int K, int OY, int OX, int NTH, bool EDGE>
__device__ __forceinline__ void tb_step(const StepArgs &a, float t, unsigned active, int s,
                                        bool last, const float *uc_buf, float *un_buf, float *vb,
                                        float *wb, const float *db, float *sux, float *suy,
                                        float *ov, float *ow, float *ou, int gy0, int gx0) {
    using G = TbGeom<K, OY, OX>;
    constexpr int BX = G::BX;
    const int tid = threadIdx.x;
    const int H = a.H, W = a.W;
    const float rdx = a.rdx;
    const int rr0 = G::RO + 4 * (s + 1), rr1 = G::BY - G::RO - 4 * (s + 1);
    const int cc0 = G::CO + 4 * (s + 1), cc1 = BX - G::CO - 4 * (s + 1);
    const int NR = rr1 - rr0, NC4 = (cc1 - cc0) / 4;

    // ---- pass 1: u_x on rows [rr0-4, rr1+4) x columns [cc0, cc1) -------------------------
    for (int it = tid; it < (NR + 8) * NC4; it += NTH) {
        const int r = rr0 - 4 + it / NC4, c = cc0 + 4 * (it % NC4);
        const float *b = uc_buf + r * BX + c;
        float4 o;
        const int x = gy0 + r;
        if (!EDGE || (x > 0 && x < H - 1)) {
            o = g_central4(ld4(b - 2 * BX), ld4(b - BX), ld4(b + BX), ld4(b + 2 * BX));
        } else if (x <= 0) {
            const float4 a0 = ld4(b), a1 = ld4(b + BX), a2 = ld4(b + 2 * BX), a3 = ld4(b + 3 * BX);
            o = make_float4(g_head(a0.x, a1.x, a2.x, a3.x), g_head(a0.y, a1.y, a2.y, a3.y),
                            g_head(a0.z, a1.z, a2.z, a3.z), g_head(a0.w, a1.w, a2.w, a3.w));
        } else {
            const float4 a0 = ld4(b - 3 * BX), a1 = ld4(b - 2 * BX), a2 = ld4(b - BX), a3 = ld4(b);
            o = make_float4(g_tail(a0.x, a1.x, a2.x, a3.x), g_tail(a0.y, a1.y, a2.y, a3.y),
                            g_tail(a0.z, a1.z, a2.z, a3.z), g_tail(a0.w, a1.w, a2.w, a3.w));
        }
        st4(sux + r * BX + c, mul4(o, rdx));
    }
    // ---- u_y on rows [rr0, rr1) x columns [cc0-4, cc1+4) ------------------------------------
    const int NY4 = NC4 + 2;
    for (int it = tid; it < NR * NY4; it += NTH) {
        const int r = rr0 + it / NY4, c = cc0 - 4 + 4 * (it % NY4);
        const float *b = uc_buf + r * BX + c;
        const float4 x0 = ld4(b - 4), x1 = ld4(b), x2 = ld4(b + 4);
        const float e[12] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w,
                             x2.x, x2.y, x2.z, x2.w};
        float o[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int y = gx0 + c + m;
            if (!EDGE || (y > 0 && y < W - 1)) o[m] = g_central(e[m + 2], e[m + 3], e[m + 5], e[m + 6]);
            else if (y <= 0) o[m] = g_head(e[m + 4], e[m + 5], e[m + 6], e[m + 7]);
            else o[m] = g_tail(e[m + 1], e[m + 2], e[m + 3], e[m + 4]);
        }
        st4(suy + r * BX + c, make_float4(o[0] * rdx, o[1] * rdx, o[2] * rdx, o[3] * rdx));
    }
    if (last && tid == 0) bulk_wait_read();  // the previous tile's stores have read the outputs
    __syncthreads();

    // ---- pass 2 on [rr0, rr1) x [cc0, cc1) ---------------------------------------------------
    for (int it = tid; it < NR * NC4; it += NTH) {
        const int r = rr0 + it / NC4, c = cc0 + 4 * (it % NC4);
        const int i = gy0 + r, j = gx0 + c;
        const float *xb = sux + r * BX + c;
        const float *dbp = db + r * BX + c;
        const float4 uxc = ld4(xb), dc = ld4(dbp);
        float4 uxx, dxD;
        if (!EDGE || (i != 0 && i != H - 1)) {
            uxx = g_central4(ld4(xb - 2 * BX), ld4(xb - BX), ld4(xb + BX), ld4(xb + 2 * BX));
            dxD = g_central4(ld4(dbp - 2 * BX), ld4(dbp - BX), ld4(dbp + BX), ld4(dbp + 2 * BX));
        } else if (i == 0) {
            const float4 a0 = uxc, a1 = ld4(xb + BX), a2 = ld4(xb + 2 * BX), a3 = ld4(xb + 3 * BX);
            uxx = make_float4(g_head(a0.x, a1.x, a2.x, a3.x), g_head(a0.y, a1.y, a2.y, a3.y),
                              g_head(a0.z, a1.z, a2.z, a3.z), g_head(a0.w, a1.w, a2.w, a3.w));
            const float4 b0 = dc, b1 = ld4(dbp + BX), b2 = ld4(dbp + 2 * BX), b3 = ld4(dbp + 3 * BX);
            dxD = make_float4(g_head(b0.x, b1.x, b2.x, b3.x), g_head(b0.y, b1.y, b2.y, b3.y),
                              g_head(b0.z, b1.z, b2.z, b3.z), g_head(b0.w, b1.w, b2.w, b3.w));
        } else {
            const float4 a0 = ld4(xb - 3 * BX), a1 = ld4(xb - 2 * BX), a2 = ld4(xb - BX), a3 = uxc;
            uxx = make_float4(g_tail(a0.x, a1.x, a2.x, a3.x), g_tail(a0.y, a1.y, a2.y, a3.y),
                              g_tail(a0.z, a1.z, a2.z, a3.z), g_tail(a0.w, a1.w, a2.w, a3.w));
            const float4 b0 = ld4(dbp - 3 * BX), b1 = ld4(dbp - 2 * BX), b2 = ld4(dbp - BX), b3 = dc;
            dxD = make_float4(g_tail(b0.x, b1.x, b2.x, b3.x), g_tail(b0.y, b1.y, b2.y, b3.y),
                              g_tail(b0.z, b1.z, b2.z, b3.z), g_tail(b0.w, b1.w, b2.w, b3.w));
        }
        uxx = mul4(uxx, rdx);
        dxD = mul4(dxD, rdx);
        const float *yb = suy + r * BX + c;
        const float4 y0 = ld4(yb - 4), y1 = ld4(yb), y2 = ld4(yb + 4);
        const float4 dl = ld4(dbp - 4), dr = ld4(dbp + 4);
        const float4 uc = ld4(uc_buf + r * BX + c);
        const float4 vc = ld4(vb + r * BX + c), wc = ld4(wb + r * BX + c);
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
        float ovv[4], oww[4], ouu[4], jion[4], dv[4], dw[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const Reaction re = reaction(uu[m], vv[m], ww[m], a.m);
            jion[m] = re.j_ion;
            dv[m] = re.dv;
            dw[m] = re.dw;
        }
        if (active) {
            const float4 js = apply_stimuli(a, active, i, j, (int64_t)i * a.pitch + j,
                                            make_float4(jion[0], jion[1], jion[2], jion[3]));
            jion[0] = js.x;
            jion[1] = js.y;
            jion[2] = js.z;
            jion[3] = js.w;
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            float uyy, dyD;
            const int y = j + m;
            if (!EDGE || (y != 0 && y != W - 1)) {
                uyy = g_central(f[m + 2], f[m + 3], f[m + 5], f[m + 6]);
                dyD = g_central(g[m + 2], g[m + 3], g[m + 5], g[m + 6]);
            } else if (y == 0) {
                uyy = g_head(f[m + 4], f[m + 5], f[m + 6], f[m + 7]);
                dyD = g_head(g[m + 4], g[m + 5], g[m + 6], g[m + 7]);
            } else {
                uyy = g_tail(f[m + 1], f[m + 2], f[m + 3], f[m + 4]);
                dyD = g_tail(g[m + 1], g[m + 2], g[m + 3], g[m + 4]);
            }
            uyy *= rdx;
            dyD *= rdx;
            const float du = diffusion(dd[m], dxv[m], dyD, uxv[m], f[m + 4], uxxv[m], uyy) + jion[m];
            ovv[m] = fmaf(dv[m], a.dt, vv[m]);
            oww[m] = fmaf(dw[m], a.dt, ww[m]);
            ouu[m] = fmaf(du, a.dt, uu[m]);
        }
        const float4 nv = make_float4(ovv[0], ovv[1], ovv[2], ovv[3]);
        const float4 nw = make_float4(oww[0], oww[1], oww[2], oww[3]);
        const float4 nu = make_float4(ouu[0], ouu[1], ouu[2], ouu[3]);
        if (last) {
            const int o = (r - rr0) * OX + (c - cc0);
            st4(ov + o, nv);
            st4(ow + o, nw);
            st4(ou + o, nu);
        } else {
            st4(vb + r * BX + c, nv);
            st4(wb + r * BX + c, nw);
            st4(un_buf + r * BX + c, nu);
        }
    }
    __syncthreads();
}

}  // namespace

template <int K, int OY, int OX, int NTH>
__global__ void __launch_bounds__(NTH, 1)
    fk_tb_kernel(const __grid_constant__ TbMaps tm, const __grid_constant__ StepArgs a0,
                 int64_t t0) {
    using G = TbGeom<K, OY, OX>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float *ua = reinterpret_cast<float *>(smem);
    float *vb = ua + G::PLANE, *wb = vb + G::PLANE, *db = wb + G::PLANE;
    float *ub = db + G::PLANE, *sux = ub + G::PLANE, *suy = sux + G::PLANE;
    float *ov = suy + G::PLANE, *ow = ov + OY * OX, *ou = ow + OY * OX;
    uint64_t *bar = reinterpret_cast<uint64_t *>(ou + OY * OX);
    StepArgs *sa = reinterpret_cast<StepArgs *>(bar + 2);

    const int tid = threadIdx.x;
    const int H = a0.H, W = a0.W;
    const int ntx = (W + OX - 1) / OX, nty = (H + OY - 1) / OY, ntiles = ntx * nty;
    for (int k = tid; k < (int)(sizeof(StepArgs) / 4); k += NTH)
        reinterpret_cast<uint32_t *>(sa)[k] = reinterpret_cast<const uint32_t *>(&a0)[k];
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        fence_barrier_init();
    }
    __syncthreads();
    grid_dependency_wait();  // the previous launch has written our input state
    grid_launch_dependents();
    const StepArgs &a = *sa;

    unsigned active_k[K];
#pragma unroll
    for (int s = 0; s < K; ++s) {
        active_k[s] = 0;
        for (int q = 0; q < a.n_stim; ++q)
            if (stim_active(a.stim[q], (float)(t0 + s))) active_k[s] |= 1u << q;
    }

    int n = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++n) {
        const int i0 = (tile / ntx) * OY, j0 = (tile % ntx) * OX;
        const int gy0 = i0 - 4 * K - G::RO, gx0 = j0 - 4 * K - G::CO;
        if (tid == 0) {
            mbar_arrive_expect_tx(&bar[0], G::LOAD_BYTES);
            tma_load_2d(ua, &tm.u, gx0, gy0, &bar[0]);
            tma_load_2d(vb, &tm.v, gx0, gy0, &bar[0]);
            tma_load_2d(wb, &tm.w, gx0, gy0, &bar[0]);
            tma_load_2d(db, &tm.d, gx0, gy0, &bar[0]);
        }
        const bool ok = mbar_wait_bounded(&bar[0], n & 1);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(a0.status, kStatusTimeout);
                bulk_wait_all();
            }
            return;
        }
        // interior: no stencil of the blocked region comes within 4 of an edge
        const bool edge = !(gy0 - 4 >= 0 && gy0 + G::BY + 4 <= H && gx0 - 4 >= 0 &&
                            gx0 + G::BX + 4 <= W);
        if (edge) {
            tb_clamp<G::BY, G::BX, NTH>(ua, gy0, gx0, H, W);
            tb_clamp<G::BY, G::BX, NTH>(db, gy0, gx0, H, W);
            __syncthreads();
        }
        float *cur = ua, *nxt = ub;
#pragma unroll 1
        for (int s = 0; s < K; ++s) {
            const bool last = s == K - 1;
            const float t = (float)(t0 + s);
            if (edge)
                tb_step<K, OY, OX, NTH, true>(a, t, active_k[s], s, last, cur, nxt, vb, wb, db, sux,
                                              suy, ov, ow, ou, gy0, gx0);
            else
                tb_step<K, OY, OX, NTH, false>(a, t, active_k[s], s, last, cur, nxt, vb, wb, db,
                                               sux, suy, ov, ow, ou, gy0, gx0);
            if (!last) {
                float *tmp = cur;
                cur = nxt;
                nxt = tmp;
                if (edge) {
                    tb_clamp<G::BY, G::BX, NTH>(cur, gy0, gx0, H, W);
                    __syncthreads();
                }
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tma_store_2d(&tm.ov, ov, j0, i0);
            tma_store_2d(&tm.ow, ow, j0, i0);
            tma_store_2d(&tm.ou, ou, j0, i0);
            bulk_commit();
        }
    }
    if (tid == 0) bulk_wait_all();
}

// Batched blocked stepping (depth K, OY x OX output tiles): the tile loop of fk_tb_kernel over
// the items of many tissues, each tissue's arguments staged into shared memory whenever the
// tissue changes (all threads have finished the previous item by then: every item ends with a
// CTA barrier), the TMA maps read from the device descriptors of the item's tissue.
template <int K, int OY, int OX, int NTH>
__global__ void __launch_bounds__(NTH, 1)
    fk_batch_tb_kernel(const BatchTissue *__restrict__ tissues,
                       const BatchTbMaps *__restrict__ maps, const BatchItem *__restrict__ items,
                       int n_items, const int *t_dev, int t_offset, int parity, int *status) {
    using G = TbGeom<K, OY, OX>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float *ua = reinterpret_cast<float *>(smem);
    float *vb = ua + G::PLANE, *wb = vb + G::PLANE, *db = wb + G::PLANE;
    float *ub = db + G::PLANE, *sux = ub + G::PLANE, *suy = sux + G::PLANE;
    float *ov = suy + G::PLANE, *ow = ov + OY * OX, *ou = ow + OY * OX;
    uint64_t *bar = reinterpret_cast<uint64_t *>(ou + OY * OX);
    StepArgs *sa = reinterpret_cast<StepArgs *>(bar + 2);

    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        fence_barrier_init();
    }
    __syncthreads();
    grid_dependency_wait();  // the previous launch (and the step counter) are complete
    grid_launch_dependents();
    const int64_t t0 = (int64_t)(*t_dev) + t_offset;
    int cur = -1;
    unsigned active_k[K];
#pragma unroll
    for (int s = 0; s < K; ++s) active_k[s] = 0;
    int n = 0;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x, ++n) {
        const BatchItem bi = items[it];
        if (bi.tissue != cur) {  // uniform
            stage_args(sa, &tissues[bi.tissue].args[parity]);
            __syncthreads();
            cur = bi.tissue;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                active_k[s] = 0;
                for (int q = 0; q < sa->n_stim; ++q)
                    if (stim_active(sa->stim[q], (float)(t0 + s))) active_k[s] |= 1u << q;
            }
        }
        const StepArgs &a = *sa;
        const TbMaps &tm = maps[bi.tissue].maps[parity];
        const int H = a.H, W = a.W, i0 = bi.i0, j0 = bi.j0;
        const int gy0 = i0 - 4 * K - G::RO, gx0 = j0 - 4 * K - G::CO;
        if (tid == 0) {
            mbar_arrive_expect_tx(&bar[0], G::LOAD_BYTES);
            tma_load_2d(ua, &tm.u, gx0, gy0, &bar[0]);
            tma_load_2d(vb, &tm.v, gx0, gy0, &bar[0]);
            tma_load_2d(wb, &tm.w, gx0, gy0, &bar[0]);
            tma_load_2d(db, &tm.d, gx0, gy0, &bar[0]);
        }
        const bool ok = mbar_wait_bounded(&bar[0], n & 1);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(status, kStatusTimeout);
                bulk_wait_all();
            }
            return;
        }
        const bool edge = !(gy0 - 4 >= 0 && gy0 + G::BY + 4 <= H && gx0 - 4 >= 0 &&
                            gx0 + G::BX + 4 <= W);
        if (edge) {
            tb_clamp<G::BY, G::BX, NTH>(ua, gy0, gx0, H, W);
            tb_clamp<G::BY, G::BX, NTH>(db, gy0, gx0, H, W);
            __syncthreads();
        }
        float *cu = ua, *nx = ub;
#pragma unroll 1
        for (int s = 0; s < K; ++s) {
            const bool last = s == K - 1;
            const float t = (float)(t0 + s);
            if (edge)
                tb_step<K, OY, OX, NTH, true>(a, t, active_k[s], s, last, cu, nx, vb, wb, db, sux,
                                              suy, ov, ow, ou, gy0, gx0);
            else
                tb_step<K, OY, OX, NTH, false>(a, t, active_k[s], s, last, cu, nx, vb, wb, db,
                                               sux, suy, ov, ow, ou, gy0, gx0);
            if (!last) {
                float *tmp = cu;
                cu = nx;
                nx = tmp;
                if (edge) {
                    tb_clamp<G::BY, G::BX, NTH>(cu, gy0, gx0, H, W);
                    __syncthreads();
                }
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tma_store_2d(&tm.ov, ov, j0, i0);
            tma_store_2d(&tm.ow, ow, j0, i0);
            tma_store_2d(&tm.ou, ou, j0, i0);
            bulk_commit();
        }
    }
    if (tid == 0) bulk_wait_all();
}

namespace {

template <int K, int OY, int OX>
cudaError_t launch_tb_k(const TbMaps &maps, const StepArgs &a, int64_t t0, cudaStream_t stream) {
    constexpr int NTH = kTbThreads;
    using G = TbGeom<K, OY, OX>;
    constexpr int SMEM = G::BYTES + 16 + SMEM_ARGS_BYTES + 128;
    static_assert(SMEM <= 227 * 1024, "blocked tile does not fit in shared memory");
    static thread_local uint64_t configured_ctx = 0;  // attributes belong to the context
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (context_changed(configured_ctx)) {
        if ((e = cudaFuncSetAttribute(fk_tb_kernel<K, OY, OX, NTH>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM)) !=
            cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
    }
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
    const int ntiles = ((a.H + OY - 1) / OY) * ((a.W + OX - 1) / OX);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ntiles < sms ? ntiles : sms);
    cfg.blockDim = dim3(NTH);
    cfg.dynamicSmemBytes = SMEM;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fk_tb_kernel<K, OY, OX, NTH>, maps, a, t0);
}

}  // namespace

void tb_box(int depth, int *box_w, int *box_h, int *out_w, int *out_h) {
    switch (depth) {
        case 2: *box_w = TbGeom<2, 32, 64>::BX; *box_h = TbGeom<2, 32, 64>::BY; *out_w = 64; *out_h = 32; break;
        case 4: *box_w = TbGeom<4, 32, 64>::BX; *box_h = TbGeom<4, 32, 64>::BY; *out_w = 64; *out_h = 32; break;
        case 8: *box_w = TbGeom<8, 16, 16>::BX; *box_h = TbGeom<8, 16, 16>::BY; *out_w = 16; *out_h = 16; break;
        default: *box_w = *box_h = *out_w = *out_h = 0;
    }
}

cudaError_t launch_batch_tb(const BatchTissue *tissues, const BatchTbMaps *maps,
                            const BatchItem *items, int n_items, const int *t_dev, int t_offset,
                            int parity, int *status, int grid, cudaStream_t stream) {
    constexpr int K = kBatchTbDepth, OY = kBatchTbRows, OX = kBatchTbCols, NTH = kTbThreads;
    using G = TbGeom<K, OY, OX>;
    constexpr int SMEM = G::BYTES + 16 + SMEM_ARGS_BYTES + 128;
    static_assert(SMEM <= 227 * 1024, "blocked tile does not fit in shared memory");
    static thread_local uint64_t configured_ctx = 0;  // attributes belong to the context
    if (context_changed(configured_ctx)) {
        cudaError_t e = cudaFuncSetAttribute(fk_batch_tb_kernel<K, OY, OX, NTH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
        if (e != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
    }
    if (grid < 1 || n_items < 1) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NTH);
    cfg.dynamicSmemBytes = SMEM;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fk_batch_tb_kernel<K, OY, OX, NTH>, tissues, maps, items,
                              n_items, t_dev, t_offset, parity, status);
}

cudaError_t launch_tb(int depth, const TbMaps &maps, const StepArgs &a, int64_t t0,
                      cudaStream_t stream) {
    switch (depth) {
        case 2: return launch_tb_k<2, 32, 64>(maps, a, t0, stream);
        case 4: return launch_tb_k<4, 32, 64>(maps, a, t0, stream);
        case 8: return launch_tb_k<8, 16, 16>(maps, a, t0, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fk
