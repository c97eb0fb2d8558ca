// K1: fused Fenton-Karma Euler step (reaction + gates + stimulus override + div(D grad u) +
// Euler update) over one tissue, one launch per time step; and the batched variant over the
// tiles of many tissues.  The tile computation itself lives in fk_tile.cuh.
//
// Replaces cardiax/solve.py:26-70 (step + step_euler, with gradient x6, stimulate and the edge
// pads fused).
#include "fk_capi_internal.h"
#include "fk_tile.cuh"

namespace fk {

// ---- tile order ------------------------------------------------------------------------------
// Edge tiles (those that take the clamped-halo path) cost more than interior tiles.  Handing
// them out first, one per CTA, keeps the persistent CTAs balanced; a plain row-major
// round-robin gives every 16th CTA an edge tile on every other turn.
struct TileOrder {
    int nc, r_lo, r_hi, c_lo, c_hi;  // interior tile rows [r_lo, r_hi], columns [c_lo, c_hi]
    int n_top, n_mid_row, n_mid, n_edge;
    __device__ TileOrder(int H, int W) {
        const int nr = (H + TY - 1) / TY;
        nc = (W + TX - 1) / TX;
        r_lo = (BAND + TY - 1) / TY;
        r_hi = (H - BAND) / TY - 1;
        c_lo = (BAND + TX - 1) / TX;
        c_hi = (W - BAND) / TX - 1;
        if (r_hi < r_lo || c_hi < c_lo) {  // no interior tile: plain row-major order
            r_lo = nr;
            r_hi = nr - 1;
            c_lo = 0;
            c_hi = nc - 1;
        }
        n_top = r_lo * nc;
        n_mid_row = c_lo + (nc - 1 - c_hi);
        n_mid = (r_hi - r_lo + 1) * n_mid_row;
        n_edge = nr * nc - (r_hi - r_lo + 1) * (c_hi - c_lo + 1);
    }
    // tile row and column of the k-th tile handed out
    __device__ void at(int k, int &tr, int &tc) const {
        if (k < n_edge) {
            if (k < n_top) {
                tr = k / nc;
                tc = k % nc;
            } else if (k < n_top + n_mid) {
                const int m = k - n_top;
                tr = r_lo + m / n_mid_row;
                const int q = m % n_mid_row;
                tc = q < c_lo ? q : c_hi + 1 + (q - c_lo);
            } else {
                const int m = k - n_top - n_mid;
                tr = r_hi + 1 + m / nc;
                tc = m % nc;
            }
        } else {
            const int m = k - n_edge, w = c_hi - c_lo + 1;
            tr = r_lo + m / w;
            tc = c_lo + m % w;
        }
    }
};

// ---- the step kernel: persistent CTAs over the tiles of one tissue ------------------------
template <bool DERIV, bool ACT, int HEUN>
__global__ void __launch_bounds__(NT, CTAS_PER_SM) fk_step_kernel(const __grid_constant__ StepMaps tm,
                                                        const __grid_constant__ StepArgs a,
                                                        const __grid_constant__ PackConsts k) {
    extern __shared__ unsigned char smem_raw[];
    // 128-byte aligned base, offset as a pointer so that the compiler keeps the shared-memory
    // state space (integer address arithmetic would turn every access into a generic one)
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    // u_x and u_y planes, double-buffered: pass 1 of tile n+1 may start while slower warps are
    // still in pass 2 of tile n (the new state goes straight to global memory, so the only CTA
    // barrier of an interior tile is the one between its passes)
    float *sux = reinterpret_cast<float *>(smem + NSTAGE * SMEM_STAGE_BYTES);  // [2][SUX_H][TX]
    float *suy = sux + 2 * TX * SUX_H;                                           // [2][TY][SW]
    TileIO io;
    io.ov = io.ow = io.ou = nullptr;
    uint64_t *bar = reinterpret_cast<uint64_t *>(suy + 2 * SW * TY);            // [NSTAGE]
    // the arguments are read in place (a __grid_constant__ parameter: constant-bank operands)

    const int tid = threadIdx.x;
    const int ntx = (a.W + TX - 1) / TX, nty = (a.H + TY - 1) / TY, ntiles = ntx * nty;
    if (tid == 0) {
        prefetch_tensormap(&tm.u);
        prefetch_tensormap(&tm.d);
        for (int q = 0; q < NSTAGE; ++q) mbar_init(&bar[q], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // the previous step's grid (same stream) must have finished writing our input state
    grid_dependency_wait();
    grid_launch_dependents();
    const TileOrder order(a.H, a.W);
    auto tile_at = [&](int tl) {  // (i0, j0) of the tl-th tile handed out
        int tr, tc;
        order.at(tl, tr, tc);
        return make_int2(tr * TY, tc * TX);
    };
    int tile = blockIdx.x;
    // L2 policies: the input state is read for the last time (the next step overwrites its
    // buffer), D is read again by every step.  Only worth it when the live data fits in L2.
    const bool hints = a.l2_hints != 0;
    const uint64_t pol_dead = l2_policy_evict_first(), pol_keep = l2_policy_evict_last();
    auto issue = [&](int tl, int s) {
        const int2 ij = tile_at(tl);
        if (hints)
            issue_tile_hinted(tm, stage_at(smem, s), &bar[s], ij.x, ij.y, pol_dead, pol_keep);
        else
            issue_tile(tm, stage_at(smem, s), &bar[s], ij.x, ij.y);
    };
    if (tid == 0)  // prologue: the first two tiles of this CTA
        for (int q = 0; q < NSTAGE - 1; ++q) {
            const int tl = tile + q * gridDim.x;
            if (tl < ntiles) issue(tl, q);
        }

    unsigned active = 0;
    for (int s = 0; s < a.n_stim; ++s)
        if (stim_active(a.stim[s], a.t)) active |= 1u << s;

    for (int n = 0; tile < ntiles; ++n, tile += gridDim.x) {
        const int s = n % NSTAGE;
        const int2 ij = tile_at(tile);
        const int i0 = ij.x, j0 = ij.y;
        if (hints)
            load_vw_hinted(a, i0, j0, io, pol_dead);
        else
            load_vw(a, i0, j0, io);
        const bool ok = mbar_wait_bounded(&bar[s], (n / NSTAGE) & 1);
        // after the barrier between this tile's passes every thread has finished tile n-1, so
        // its stage takes tile n+2
        const int ahead = tile + (NSTAGE - 1) * gridDim.x;
        auto refill = [&] {
            if (tid == 0 && ahead < ntiles) issue(ahead, (n + NSTAGE - 1) % NSTAGE);
        };
        float *ux_n = sux + (n & 1) * (TX * SUX_H), *uy_n = suy + (n & 1) * (SW * TY);
        if (!process_tile<DERIV, ACT, true, true, HEUN>(a, a.t, stage_at(smem, s), ux_n, uy_n,
                                                        io, active, i0, j0, NoHook{}, &k,
                                                        PairScale{k.rdx, k.dt}, ok, refill)) {
            if (tid == 0) {
                atomicOr(a.status, kStatusTimeout);
                drain_stages(bar, n, tile, (int)gridDim.x, ntiles);
            }
            return;
        }
    }
}

__global__ void add_int_kernel(int *p, int v) { *p += v; }

__global__ void batch_copyback_kernel(const BatchTissue *tissues) {
    const StepArgs &src = tissues[blockIdx.y].args[1];   // reads scratch ...
    const StepArgs &dst = tissues[blockIdx.y].args[0];   // ... into state
    const int64_t plane = (int64_t)src.H * src.pitch;
    const float *in[3] = {src.v, src.w, src.u};
    float *out[3] = {const_cast<float *>(dst.v), const_cast<float *>(dst.w),
                     const_cast<float *>(dst.u)};
    for (int p = 0; p < 3; ++p)
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < plane;
             k += (int64_t)gridDim.x * blockDim.x)
            out[p][k] = in[p][k];
}

cudaError_t launch_add_int(int *p, int v, cudaStream_t stream) {
    add_int_kernel<<<1, 1, 0, stream>>>(p, v);
    return cudaGetLastError();
}

cudaError_t launch_batch_copyback(const BatchTissue *tissues, int n_tissues, cudaStream_t stream) {
    if (n_tissues < 1) return cudaSuccess;
    batch_copyback_kernel<<<dim3(64, n_tissues), 256, 0, stream>>>(tissues);
    return cudaGetLastError();
}

template <bool DERIV, bool ACT, int HEUN = 0>
static cudaError_t set_smem_attr() {
    return cudaFuncSetAttribute(fk_step_kernel<DERIV, ACT, HEUN>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_STEP_DIRECT_BYTES);
}

// Whether the live data of a step on an H x pitch grid (the new state and D: 4 planes) fits in
// 3/4 of the current device's L2, so that L2 eviction hints pay off (looked up once per device).
bool l2_fits_step(int64_t H, int64_t pitch) {
    static thread_local int dev_cached = -1;
    static thread_local int64_t l2_bytes = 0;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (dev != dev_cached) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev) != cudaSuccess) v = 0;
        l2_bytes = v;
        dev_cached = dev;
    }
    return 4 * H * pitch * (int64_t)sizeof(float) * 4 <= 3 * l2_bytes;
}

cudaError_t launch_step(const StepMaps &maps, const StepArgs &a, bool deriv, cudaStream_t stream,
                        int heun) {
    // the attribute is per function and per context: set again whenever the context changes
    static thread_local uint64_t configured_ctx = 0;
    static thread_local int n_sm = 0;
    if (context_changed(configured_ctx)) {
        cudaError_t e;
        int dev = -1;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess || (e = set_smem_attr<true, false>()) != cudaSuccess ||
            (e = set_smem_attr<false, true>()) != cudaSuccess ||
            (e = set_smem_attr<false, false>()) != cudaSuccess ||
            (e = set_smem_attr<false, false, 1>()) != cudaSuccess ||
            (e = set_smem_attr<false, false, 2>()) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
    }
    const int ntiles = ((a.W + TX - 1) / TX) * ((a.H + TY - 1) / TY);
    const int grid = ntiles < n_sm * CTAS_PER_SM ? ntiles : n_sm * CTAS_PER_SM;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = SMEM_STEP_DIRECT_BYTES;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const PackConsts k = make_pack_consts(a.m, a.rdx, a.dt);
    if (deriv) return cudaLaunchKernelEx(&cfg, fk_step_kernel<true, false, 0>, maps, a, k);
    if (heun == 1) return cudaLaunchKernelEx(&cfg, fk_step_kernel<false, false, 1>, maps, a, k);
    if (heun == 2) return cudaLaunchKernelEx(&cfg, fk_step_kernel<false, false, 2>, maps, a, k);
    if (a.act_last) return cudaLaunchKernelEx(&cfg, fk_step_kernel<false, true, 0>, maps, a, k);
    return cudaLaunchKernelEx(&cfg, fk_step_kernel<false, false, 0>, maps, a, k);
}

}  // namespace fk
