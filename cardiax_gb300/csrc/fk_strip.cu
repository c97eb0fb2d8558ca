// K1 strip kernel: one fused Fenton-Karma Euler step per launch over one tissue, with the cell
// arithmetic on packed FP32 pairs (fk_pack.cuh).  Geometry and edge handling: fk_strip.cuh.
//
// Replaces cardiax/solve.py:26-70 (step + step_euler, with gradient x6, stimulate and the edge
// pads fused), like fk_step_kernel, and produces the same bits.
#include "fk_capi_internal.h"
#include "fk_strip.cuh"
#include "fk_tile.cuh"

namespace fk {

// Edge tiles: overwrite the zero-filled out-of-grid rows and columns of a shared buffer (grid rows
// i0-top .. i0-top+rows-1, columns c0-4 .. c0+131) with copies of the first/last grid row and
// column, as the reference's jnp.pad(..., "edge") does.  Rows first, then columns, so corners get
// the corner cell.  All threads; a barrier must follow before the buffer is read.
static __device__ __noinline__ void strip_clamp(float *buf, int rows, int top, int i0, int c0,
                                                int H, int W) {
    constexpr int SW4 = S_SW / 4;
    const int tid = threadIdx.x;
    const int src_top = top - i0;               // buffer row of grid row 0
    const int src_bot = H - 1 - i0 + top;       // buffer row of grid row H-1
    for (int it = tid; it < rows * SW4; it += S_NT) {
        const int b = it / SW4, c4 = it % SW4;
        const int x = i0 - top + b;             // grid row of buffer row b
        int src = -1;
        if (x < 0) src = src_top;
        else if (x >= H) src = src_bot;
        if (src >= 0)
            reinterpret_cast<float4 *>(buf + b * S_SW)[c4] =
                reinterpret_cast<const float4 *>(buf + src * S_SW)[c4];
    }
    __syncthreads();
    const int col0 = S_HC - c0;                 // buffer column of grid column 0
    const int colw = W - 1 - c0 + S_HC;         // buffer column of grid column W-1
    for (int it = tid; it < rows * S_SW; it += S_NT) {
        const int b = it / S_SW, j = it % S_SW;
        const int y = c0 - S_HC + j;            // grid column of buffer column j
        if (y < 0) buf[b * S_SW + j] = buf[b * S_SW + col0];
        else if (y >= W) buf[b * S_SW + j] = buf[b * S_SW + colw];
    }
}

// The S_RPW rows R .. R+S_RPW-1 of one warp (R < H).  ER: the tile is within 4 rows of the top or
// bottom edge; EC: within 4 columns of the left or right edge.
template <bool ACT, bool ER, bool EC>
__device__ __forceinline__ void strip_rows(const StepArgs &a, const PackConsts &k, float t,
                                           unsigned active, const float *su, const float *sd,
                                           int i0, int c0, int R, float4 vc, float4 wc) {
    const int lane = threadIdx.x & 31;
    const int H = a.H, W = a.W;
    const int64_t pitch = a.pitch;
    const int c = c0 + 4 * lane;                // first column of this lane's quad
    const float rdx = a.rdx;
    // shared row of grid row x, positioned at grid column c - 4 (this lane's left neighbour quad)
    const float *ub = su + (S_HU_TOP - i0) * S_SW + 4 * lane;
    const float *db = sd + (S_HD_TOP - i0) * S_SW + 4 * lane;
    auto U = [&](int x) { return ub + x * S_SW; };
    auto Dr = [&](int x) { return db + x * S_SW; };

    // u_x at row x for this lane's 4 columns (cardiax/solve.py:49 on the padded column)
    auto ux_at = [&](int x) -> Quad {
        Quad q;
        if (!ER || (x > 0 && x < H - 1))
            q = q_central(k, ld_quad(U(x - 2) + 4), ld_quad(U(x - 1) + 4), ld_quad(U(x + 1) + 4),
                          ld_quad(U(x + 2) + 4));
        else if (x <= 0)
            q = q_head(k, ld_quad(U(x) + 4), ld_quad(U(x + 1) + 4), ld_quad(U(x + 2) + 4),
                       ld_quad(U(x + 3) + 4));
        else
            q = q_tail(k, ld_quad(U(x - 3) + 4), ld_quad(U(x - 2) + 4), ld_quad(U(x - 1) + 4),
                       ld_quad(U(x) + 4));
        return q_scale(q, k.rdx);
    };

    // windows: entry j holds row R - WL + j (the rows a central second derivative needs; the
    // one-sided rows at r = 0 and r = H-1 reach one row further and fetch it themselves)
    constexpr int WL = 2;
    constexpr int NW = S_RPW + WL + 2;
    Quad uxw[NW], dwin[NW];
#pragma unroll
    for (int j = 0; j < WL + 2; ++j) {
        uxw[j] = ux_at(R - WL + j);
        dwin[j] = ld_quad(Dr(R - WL + j) + 4);
    }
    const int d_edge = W - 1 - c;               // position of the last grid column in the quad

#pragma unroll
    for (int kk = 0; kk < S_RPW; ++kk) {
        const int r = R + kk;
        if (r >= H) break;
        // v, w of the next row (this row's came with the previous iteration or the caller)
        float4 vn = make_float4(0.f, 0.f, 0.f, 0.f), wn = vn;
        if (kk + 1 < S_RPW && r + 1 < H && c < W) {
            const int64_t off = (int64_t)(r + 1) * pitch + c;
            vn = __ldcg(reinterpret_cast<const float4 *>(a.v + off));
            wn = __ldcg(reinterpret_cast<const float4 *>(a.w + off));
        }
        uxw[kk + WL + 2] = ux_at(r + 2);
        dwin[kk + WL + 2] = ld_quad(Dr(r + 2) + 4);
        const int o = kk + WL;                  // window entry of row r

        // ---- x-direction second derivatives: u_xx, D_x ----
        Quad uxx, dxD;
        if (ER && r == 0) {  // rows 0 .. 3
            uxx = q_head(k, uxw[o], uxw[o + 1], uxw[o + 2], ux_at(3));
            dxD = q_head(k, dwin[o], dwin[o + 1], dwin[o + 2], ld_quad(Dr(3) + 4));
        } else if (ER && r == H - 1) {  // rows H-4 .. H-1
            uxx = q_tail(k, ux_at(H - 4), uxw[o - 2], uxw[o - 1], uxw[o]);
            dxD = q_tail(k, ld_quad(Dr(H - 4) + 4), dwin[o - 2], dwin[o - 1], dwin[o]);
        } else {
            uxx = q_central(k, uxw[o - 2], uxw[o - 1], uxw[o + 1], uxw[o + 2]);
            dxD = q_central(k, dwin[o - 2], dwin[o - 1], dwin[o + 1], dwin[o + 2]);
        }
        uxx = q_scale(uxx, k.rdx);
        dxD = q_scale(dxD, k.rdx);

        // ---- y-direction: u_y at columns c-2 .. c+5, then u_yy and D_y at c .. c+3 ----
        const float *ur = U(r);
        const float4 q0 = ld4(ur), q1 = ld4(ur + 4), q2 = ld4(ur + 8);
        const float e[12] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                             q2.x, q2.y, q2.z, q2.w};  // u at columns c-4 .. c+7
        float s[8];                                     // u_y at columns c-2 .. c+5
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float2 v2 = p_mul(pg_central(k, mk2(e[2 * p], e[2 * p + 1]),
                                               mk2(e[2 * p + 1], e[2 * p + 2]),
                                               mk2(e[2 * p + 3], e[2 * p + 4]),
                                               mk2(e[2 * p + 4], e[2 * p + 5])),
                                    k.rdx);
            s[2 * p] = v2.x;
            s[2 * p + 1] = v2.y;
        }
        float s_m1 = 0.0f;  // u_y at column c-3 (the left neighbour lane's), for a tail at c
        if (EC) {
            if (c == 0) {  // columns -1 and 0 take the first-row formula
                s[1] = g_head(e[3], e[4], e[5], e[6]) * rdx;
                s[2] = g_head(e[4], e[5], e[6], e[7]) * rdx;
            }
            if (d_edge >= 0 && d_edge <= 5) {  // columns W-1 and W take the last-row formula
#pragma unroll
                for (int j = 1; j < 8; ++j)
                    if (j >= d_edge + 2) s[j] = g_tail(e[j - 1], e[j], e[j + 1], e[j + 2]) * rdx;
            }
            s_m1 = __shfl_up_sync(0xffffffffu, s[3], 1);
        }
        float2 uyy_lo = p_mul(pg_central(k, mk2(s[0], s[1]), mk2(s[1], s[2]), mk2(s[3], s[4]),
                                         mk2(s[4], s[5])), k.rdx);
        float2 uyy_hi = p_mul(pg_central(k, mk2(s[2], s[3]), mk2(s[3], s[4]), mk2(s[5], s[6]),
                                         mk2(s[6], s[7])), k.rdx);
        const float4 dl = ld4(Dr(r)), dr = ld4(Dr(r) + 8);
        const Quad dc = dwin[o];
        const float g[8] = {dl.z, dl.w, dc.lo.x, dc.lo.y, dc.hi.x, dc.hi.y, dr.x, dr.y};
        float2 dyD_lo = p_mul(pg_central(k, mk2(g[0], g[1]), mk2(g[1], g[2]), mk2(g[3], g[4]),
                                         mk2(g[4], g[5])), k.rdx);
        float2 dyD_hi = p_mul(pg_central(k, mk2(g[2], g[3]), mk2(g[3], g[4]), mk2(g[5], g[6]),
                                         mk2(g[6], g[7])), k.rdx);
        if (EC) {
            if (c == 0) {  // column 0: first-row formula
                uyy_lo.x = g_head(s[2], s[3], s[4], s[5]) * rdx;
                dyD_lo.x = g_head(g[2], g[3], g[4], g[5]) * rdx;
            }
            if (d_edge >= 0 && d_edge <= 3) {  // column W-1 = c + d_edge: last-row formula
                float uo[4] = {uyy_lo.x, uyy_lo.y, uyy_hi.x, uyy_hi.y};
                float dyo[4] = {dyD_lo.x, dyD_lo.y, dyD_hi.x, dyD_hi.y};
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (m == d_edge) {
                        uo[m] = g_tail(m == 0 ? s_m1 : s[m - 1], s[m], s[m + 1], s[m + 2]) * rdx;
                        dyo[m] = g_tail(m == 0 ? dl.y : g[m - 1], g[m], g[m + 1], g[m + 2]) * rdx;
                    }
                uyy_lo = mk2(uo[0], uo[1]);
                uyy_hi = mk2(uo[2], uo[3]);
                dyD_lo = mk2(dyo[0], dyo[1]);
                dyD_hi = mk2(dyo[2], dyo[3]);
            }
        }

        // ---- reaction, stimulus, diffusion, Euler update ----
        const float2 u_lo = mk2(q1.x, q1.y), u_hi = mk2(q1.z, q1.w);
        const float2 v_lo = mk2(vc.x, vc.y), v_hi = mk2(vc.z, vc.w);
        const float2 w_lo = mk2(wc.x, wc.y), w_hi = mk2(wc.z, wc.w);
        const PairReaction rl = p_reaction(k, a.m, u_lo, v_lo, w_lo);
        const PairReaction rh = p_reaction(k, a.m, u_hi, v_hi, w_hi);
        float2 j_lo = rl.j_ion, j_hi = rh.j_ion;
        const int64_t goff = (int64_t)r * pitch + c;
        if (active) {
            const float4 js = apply_stimuli(a, active, r, c, goff,
                                            make_float4(j_lo.x, j_lo.y, j_hi.x, j_hi.y));
            j_lo = mk2(js.x, js.y);
            j_hi = mk2(js.z, js.w);
        }
        // del u = D (u_xx + u_yy) + D_x u_x + D_y u_y  (cardiax/solve.py:55), du = del u + J
        const Quad ux = uxw[o];
        // (u_xx and u_yy are both products: scalar sum; j_ion is a product: fma(1, du, j))
        float2 du_lo = p_mul(dc.lo, add_products(uxx.lo, uyy_lo));
        du_lo = p_fma(dxD.lo, ux.lo, du_lo);
        du_lo = p_fma(dyD_lo, mk2(s[2], s[3]), du_lo);
        du_lo = p_add_product(k, du_lo, j_lo);
        float2 du_hi = p_mul(dc.hi, add_products(uxx.hi, uyy_hi));
        du_hi = p_fma(dxD.hi, ux.hi, du_hi);
        du_hi = p_fma(dyD_hi, mk2(s[4], s[5]), du_hi);
        du_hi = p_add_product(k, du_hi, j_hi);
        const float2 nv_lo = p_fma(rl.dv, k.dt, v_lo), nv_hi = p_fma(rh.dv, k.dt, v_hi);
        const float2 nw_lo = p_fma(rl.dw, k.dt, w_lo), nw_hi = p_fma(rh.dw, k.dt, w_hi);
        const float2 nu_lo = p_fma(du_lo, k.dt, u_lo), nu_hi = p_fma(du_hi, k.dt, u_hi);

        if (c < W) {
            const float4 ov = make_float4(nv_lo.x, nv_lo.y, nv_hi.x, nv_hi.y);
            const float4 ow = make_float4(nw_lo.x, nw_lo.y, nw_hi.x, nw_hi.y);
            const float4 ou = make_float4(nu_lo.x, nu_lo.y, nu_hi.x, nu_hi.y);
            if (c + 3 < W) {
                __stcg(reinterpret_cast<float4 *>(a.vo + goff), ov);
                __stcg(reinterpret_cast<float4 *>(a.wo + goff), ow);
                __stcg(reinterpret_cast<float4 *>(a.uo + goff), ou);
            } else {  // the quad that holds the last grid column
                const float fv[4] = {ov.x, ov.y, ov.z, ov.w}, fw[4] = {ow.x, ow.y, ow.z, ow.w},
                            fu[4] = {ou.x, ou.y, ou.z, ou.w};
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (c + m < W) {
                        __stcg(a.vo + goff + m, fv[m]);
                        __stcg(a.wo + goff + m, fw[m]);
                        __stcg(a.uo + goff + m, fu[m]);
                    }
            }
            if (ACT) {
                const float uo4[4] = {q1.x, q1.y, q1.z, q1.w};
                const float un4[4] = {ou.x, ou.y, ou.z, ou.w};
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (c + m < W) record_activation(a, t, goff + m, uo4[m], un4[m]);
            }
        }
        vc = vn;
        wc = wn;
    }
}

template <bool ACT>
__global__ void __launch_bounds__(S_NT, S_CTAS_PER_SM)
    fk_strip_kernel(const __grid_constant__ StripMaps tm, const __grid_constant__ StepArgs a,
                    const __grid_constant__ PackConsts k) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + S_NSTAGE * S_STAGE_BYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int H = a.H, W = a.W;
    const int nstrips = (W + S_TX - 1) / S_TX;
    const int ntiles = nstrips * ((H + S_TY - 1) / S_TY);
    if (tid == 0) {
        prefetch_tensormap(&tm.u);
        prefetch_tensormap(&tm.d);
        for (int s = 0; s < S_NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // the previous step (same stream) must have finished writing this step's input state
    grid_dependency_wait();
    grid_launch_dependents();

    auto stage_u = [&](int s) { return reinterpret_cast<float *>(smem + s * S_STAGE_BYTES); };
    auto stage_d = [&](int s) {
        return reinterpret_cast<float *>(smem + s * S_STAGE_BYTES + S_U_BYTES);
    };
    auto issue = [&](int tl, int s) {
        const int i0 = (tl / nstrips) * S_TY, c0 = (tl % nstrips) * S_TX;
        mbar_arrive_expect_tx(&bar[s], S_U_TX + S_D_TX);
        tma_load_2d(stage_u(s), &tm.u, c0 - S_HC, i0 - S_HU_TOP, &bar[s]);
        tma_load_2d(stage_d(s), &tm.d, c0 - S_HC, i0 - S_HD_TOP, &bar[s]);
    };
    int tile = blockIdx.x;
    if (tid == 0)
        for (int j = 0; j < S_NSTAGE - 1; ++j) {
            const int tl = tile + j * (int)gridDim.x;
            if (tl < ntiles) issue(tl, j);
        }
    unsigned active = 0;
    for (int s = 0; s < a.n_stim; ++s)
        if (stim_active(a.stim[s], a.t)) active |= 1u << s;

    for (int n = 0; tile < ntiles; ++n, tile += gridDim.x) {
        const int s = n % S_NSTAGE;
        const int i0 = (tile / nstrips) * S_TY, c0 = (tile % nstrips) * S_TX;
        const int R = i0 + warp * S_RPW;
        const int c = c0 + 4 * lane;
        float4 vq = make_float4(0.f, 0.f, 0.f, 0.f), wq = vq;  // v, w of row R
        if (R < H && c < W) {
            const int64_t off = (int64_t)R * a.pitch + c;
            vq = __ldcg(reinterpret_cast<const float4 *>(a.v + off));
            wq = __ldcg(reinterpret_cast<const float4 *>(a.w + off));
        }
        const bool ok = mbar_wait_bounded(&bar[s], (n / S_NSTAGE) & 1);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(a.status, kStatusTimeout);
                // tiles n .. n + S_NSTAGE - 2 may still be loading: wait (bounded) for them
                for (int q = 0; q < S_NSTAGE - 1; ++q)
                    if (tile + q * (int)gridDim.x < ntiles)
                        mbar_wait_bounded(&bar[(n + q) % S_NSTAGE], ((n + q) / S_NSTAGE) & 1);
            }
            return;
        }
        // every warp has finished tile n-1, whose stage now takes tile n + S_NSTAGE - 1
        const int ahead = tile + (S_NSTAGE - 1) * (int)gridDim.x;
        if (tid == 0 && ahead < ntiles) issue(ahead, (n + S_NSTAGE - 1) % S_NSTAGE);

        float *su = stage_u(s), *sd = stage_d(s);
        const bool er = i0 < BAND || i0 + S_TY > H - BAND;
        const bool ec = c0 < BAND || c0 + S_TX > W - BAND;
        if (er || ec) {
            strip_clamp(su, S_UH, S_HU_TOP, i0, c0, H, W);
            strip_clamp(sd, S_DH, S_HD_TOP, i0, c0, H, W);
            fence_async_smem();  // generic writes before the stage's next TMA load
            __syncthreads();
        }
        if (R < H) {
            if (!er && !ec)
                strip_rows<ACT, false, false>(a, k, a.t, active, su, sd, i0, c0, R, vq, wq);
            else if (!ec)
                strip_rows<ACT, true, false>(a, k, a.t, active, su, sd, i0, c0, R, vq, wq);
            else if (!er)
                strip_rows<ACT, false, true>(a, k, a.t, active, su, sd, i0, c0, R, vq, wq);
            else
                strip_rows<ACT, true, true>(a, k, a.t, active, su, sd, i0, c0, R, vq, wq);
        }
    }
    (void)lane;
}

cudaError_t launch_strip(const StripMaps &maps, const StepArgs &a, cudaStream_t stream) {
    static thread_local uint64_t configured_ctx = 0;  // attributes belong to the context
    static thread_local int n_sm = 0;
    if (context_changed(configured_ctx)) {
        cudaError_t e;
        int dev = -1;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_strip_kernel<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      S_SMEM_BYTES)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_strip_kernel<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      S_SMEM_BYTES)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
    }
    const int ntiles = (int)(((a.W + S_TX - 1) / S_TX) * ((a.H + S_TY - 1) / S_TY));
    const int cap = n_sm * S_CTAS_PER_SM;
    const PackConsts k = make_pack_consts(a.m, a.rdx, a.dt);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ntiles < cap ? ntiles : cap);
    cfg.blockDim = dim3(S_NT);
    cfg.dynamicSmemBytes = S_SMEM_BYTES;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (a.act_last) return cudaLaunchKernelEx(&cfg, fk_strip_kernel<true>, maps, a, k);
    return cudaLaunchKernelEx(&cfg, fk_strip_kernel<false>, maps, a, k);
}

}  // namespace fk
