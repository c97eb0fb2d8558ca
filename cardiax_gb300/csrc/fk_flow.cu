// K6: dataflow Euler kernel -- many steps of one tissue in one cooperative launch.
//
// Replaces the time loop of cardiax/solve.py:92-100 (_forward_euler: step_euler repeated) with
// one persistent launch.  There is no grid-wide barrier between steps: tile T of step k starts
// as soon as T and its eight neighbours have finished step k-1 (the stencil reaches 4 cells,
// less than a tile, so only the neighbours matter), so a step's tail overlaps the next step's
// head and the launch gap, prologue and pipeline drain of per-step launches disappear.
//
// Work split: the (step, tile) items are numbered i = k * ntiles + T and CTA c of G takes items
// c, c+G, c+2G, ... in order (every CTA gets the same number of tiles to within one over the
// launch); a CTA advances its (k, T) position incrementally, without divisions.
//
// Roles inside a CTA.  The last warp's lane 0 (the "store thread") issues the TMA stores of
// every item and, at the top of item x, waits for the stores of items <= x-2 (bulk wait_group 1,
// normally already done) and records that in shared memory.  Warp 0 then publishes those items
// (flags[T] = k+1) at its hook between the two passes, reads the flags of the next item to
// prefetch (relaxed loads made at the top of the item) and issues its TMA loads when its
// neighbourhood is ready; items of this CTA are judged from its own progress.  One
// fence.acq_rel.gpu in warp 0 per tile is both the release of the published flags and the
// acquire of the flags read; warp 0 has no bulk stores in flight, so the fence does not wait
// for them.  A prefetch that is not ready is retried at the next tile; an item whose loads were
// never issued publishes everything completed, waits for its flags (bounded), then loads.
//
// Hazards covered by the flags: step k of tile T reads buffer (k-1)&1 around T (its own cells
// and a 4-cell halo inside the neighbours), written by step k-1 of those tiles; it overwrites
// buffer k&1 over T, last read by step k-1 of T and of its neighbours.  Both are ordered by
// waiting for flags[T'] >= k over T and its neighbours.  Data written by another SM is only
// read through L2 (TMA loads, ld.global.cg).
//
// Every wait is bounded: a dependency not met within 1 s, or a TMA load not landed within 1 s,
// sets the abort word flags[ntiles] (which every waiting CTA polls) and the device status word;
// the CTA then waits (bounded) for its own loads in flight and its stores, and returns.  All CTAs
// are resident (cooperative launch), and an item only waits on items with smaller numbers, which
// every CTA processes in increasing order and publishes before it blocks, so no wait is
// circular.
#include "fk_capi_internal.h"
#include "fk_tile.cuh"

namespace fk {

namespace {

constexpr uint64_t kFlagWaitNs = 1000000000ull;   // one dependency wait
constexpr uint64_t kDrainWaitNs = 100000000ull;   // one in-flight load on the error path
constexpr int kStoreThread = NT - 32;             // lane 0 of the last warp

__device__ __forceinline__ void bulk_wait_all_but_one() {
    asm volatile("cp.async.bulk.wait_group 1;" ::: "memory");
}

// Position (step k, tile T) of an item; the next item of the CTA is G tiles further (G <= the
// tile count, so at most one wrap into the next step).
struct Pos {
    int k, T;
};
struct Plan {
    int ntx, nty, ntiles, G, c, r;  // r = ntiles mod G
    int64_t total;                  // items of this CTA
    __device__ __forceinline__ void next(Pos &p) const {
        p.T += G;
        if (p.T >= ntiles) {
            p.T -= ntiles;
            ++p.k;
        }
    }
    __device__ __forceinline__ Pos ahead(Pos p, int n) const {
        for (int i = 0; i < n; ++i) next(p);
        return p;
    }
};

// Dependency of the item at position p (local index x) on neighbour `lane` (0..8, row-major
// 3x3 around its tile).
struct Dep {
    int kind;         // 0: none, 1: an item of this CTA, 2: an item of another CTA
    int need;         // kind 2: flags[tile] must reach this
    int64_t own;      // kind 1: the local item that must have been published
    const int *flag;  // kind 2
};
__device__ __forceinline__ Dep dep_of(const Plan &P, const int *flags, Pos p, int64_t x,
                                      int lane) {
    Dep d{0, 0, 0, nullptr};
    if (p.k == 0 || lane >= 9) return d;
    const int ti = p.T / P.ntx + lane / 3 - 1, tj = p.T % P.ntx + lane % 3 - 1;
    if (ti < 0 || ti >= P.nty || tj < 0 || tj >= P.ntx) return d;
    const int tn = ti * P.ntx + tj;
    // global number of the dependency: i(p) - ntiles + (tn - T); it is this CTA's iff that
    // difference is a multiple of G, and then it lies (ntiles - dT) / G items back
    const int dT = tn - p.T;
    if ((dT - P.r) % P.G == 0) {
        d.kind = 1;
        d.own = x - (P.ntiles - dT) / P.G;
    } else {
        d.kind = 2;
        d.need = p.k;
        d.flag = flags + tn;
    }
    return d;
}

}  // namespace

template <bool ACT>
__global__ void __launch_bounds__(NT, CTAS_PER_SM)
    fk_flow_kernel(const __grid_constant__ FlowMaps fm, const __grid_constant__ FlowArgs fa) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float *sux = reinterpret_cast<float *>(smem + NSTAGE * SMEM_STAGE_BYTES);
    float *suy = sux + TX * SUX_H;
    TileIO io;
    io.ov = suy + SW * TY;
    io.ow = io.ov + TX * TY;
    io.ou = io.ow + TX * TY;
    uint64_t *bar = reinterpret_cast<uint64_t *>(io.ou + TX * TY);
    StepArgs *sa = reinterpret_cast<StepArgs *>(bar + NSTAGE);  // [3]: src, buffer 0, buffer 1
    __shared__ long long s_issued;  // local items whose loads have been issued (warp 0)
    __shared__ long long s_stored;  // local items whose stores have completed (store thread)

    const int tid = threadIdx.x, lane = tid & 31;
    const StepArgs &a0 = fa.in[0];
    Plan P;
    P.ntx = (a0.W + TX - 1) / TX;
    P.nty = (a0.H + TY - 1) / TY;
    P.ntiles = P.ntx * P.nty;
    P.G = gridDim.x;
    P.c = blockIdx.x;
    P.r = P.ntiles % P.G;
    const int64_t n_items = (int64_t)P.ntiles * fa.nsteps;
    P.total = (n_items - P.c + P.G - 1) / P.G;
    int *flags = fa.flags;
    int *abort_word = flags + P.ntiles;

    for (int k = 0; k < 3; ++k) stage_args(sa + k, &fa.in[k]);
    if (tid == 0) {
        prefetch_tensormap(&fm.d);
        for (int k = 0; k < NSTAGE; ++k) mbar_init(&bar[k], 1);
        fence_barrier_init();
        s_issued = 0;
        s_stored = 0;
    }
    __syncthreads();

    auto in_sel = [](int k) { return k == 0 ? 0 : 1 + ((k - 1) & 1); };
    auto issue = [&](Pos p, int stage) {  // lane 0 of warp 0
        fence_proxy_async_global();  // the flags read before are ordered before the TMA reads
        issue_tile(&fm.uin[in_sel(p.k)], &fm.d, stage_at(smem, stage), &bar[stage],
                   (p.T / P.ntx) * TY, (p.T % P.ntx) * TX);
    };
    // Warp 0: own items < published have their flags written; publish(n) writes the flags of
    // items published .. n-1 (their stores have completed; the caller has fenced).
    int64_t published = 0;
    Pos pub_pos{0, P.c};
    auto publish = [&](int64_t n) {
        for (; published < n; ++published) {
            if (lane == 0) st_relaxed_gpu(flags + pub_pos.T, pub_pos.k + 1);
            P.next(pub_pos);
        }
    };
    auto stores_completed = [&](int64_t upto) {  // store thread
        fence_proxy_async_global();
        s_stored = upto;
    };

    bool failed = false;
    int64_t x = 0;
    Pos cur{0, P.c};
    int stage = 0;
    uint32_t phase = 0;
    for (; x < P.total; ++x) {
        const int k = cur.k, T = cur.T;
        const int i0 = (T / P.ntx) * TY, j0 = (T % P.ntx) * TX;
        const StepArgs &a = sa[in_sel(k)];
        int64_t issued = *(volatile long long *)&s_issued;  // uniform: written before a barrier

        if (issued == x) {  // nothing prefetched: publish, wait for this item's inputs, load
            if (tid == kStoreThread) {
                bulk_wait_all();
                stores_completed(x);
            }
            __syncthreads();
            bool ok = true;
            if (tid < 32) {
                fence_acq_rel_gpu();
                publish(*(volatile long long *)&s_stored);
                const Dep d = dep_of(P, flags, cur, x, lane);
                if (d.kind == 2 && ld_relaxed_gpu(d.flag) < d.need) {
                    const uint64_t t_start = global_timer_ns();
                    while (ld_relaxed_gpu(d.flag) < d.need) {
                        if (ld_relaxed_gpu(abort_word) != 0 ||
                            global_timer_ns() - t_start > kFlagWaitNs) {
                            ok = false;
                            break;
                        }
                        __nanosleep(64);
                    }
                }
                ok = __all_sync(0xffffffffu, ok);
                if (ok) {
                    fence_acq_rel_gpu();
                    __syncwarp();
                    if (lane == 0) issue(cur, stage);
                }
            }
            // s_issued changes only after a barrier that every thread passes after reading it
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if (tid == 0) s_issued = x + 1;
            issued = x + 1;
        } else if (tid == kStoreThread && x >= 2) {
            bulk_wait_all_but_one();  // the stores of items <= x-2 have completed
            stores_completed(x - 1);
        }

        // warp 0: read the flags of the next item to prefetch (judged after pass 1)
        const int ahead = (int)(issued - x);  // 1 or 2
        const bool have_cand = issued < P.total && ahead < NSTAGE;
        Pos cpos{0, 0};
        Dep cd{0, 0, 0, nullptr};
        int cflag = 0;
        if (tid < 32 && have_cand) {
            cpos = P.ahead(cur, ahead);
            cd = dep_of(P, flags, cpos, issued, lane);
            if (cd.kind == 2) cflag = ld_relaxed_gpu(cd.flag);
        }

        load_vw(a, i0, j0, io);
        const bool landed = mbar_wait_bounded(&bar[stage], phase);
        if (__syncthreads_or(!landed)) {
            failed = true;
            break;
        }
        const float t = (float)(fa.t0 + k);
        unsigned active = 0;
        for (int s = 0; s < a.n_stim; ++s)
            if (stim_active(a.stim[s], t)) active |= 1u << s;

        auto after_pass1 = [&] {  // between the passes
            if (tid < 32) {
                const int64_t done = *(volatile long long *)&s_stored;
                const bool ready = have_cand &&
                                   (cd.kind == 0 || (cd.kind == 1 && cd.own < done) ||
                                    (cd.kind == 2 && cflag >= cd.need));
                const bool go = __all_sync(0xffffffffu, ready);
                if (go || published < done) {
                    fence_acq_rel_gpu();  // release for the flags below, acquire for cflag
                    publish(done);
                }
                if (go) {
                    __syncwarp();
                    if (lane == 0) {
                        int cs = stage + ahead;
                        if (cs >= NSTAGE) cs -= NSTAGE;
                        issue(cpos, cs);
                        s_issued = issued + 1;
                    }
                }
            }
            if (tid == kStoreThread) bulk_wait_read();  // the output tiles are free for pass 2
        };
        process_tile<false, ACT>(a, t, stage_at(smem, stage), sux, suy, io, active, i0, j0,
                                 after_pass1);
        const int o = k & 1;
        store_tile(&fm.ov[o], &fm.ow[o], &fm.ou[o], io, i0, j0, kStoreThread);
        P.next(cur);
        if (++stage == NSTAGE) {
            stage = 0;
            phase ^= 1u;
        }
    }

    if (!failed) {
        if (tid == kStoreThread) {
            bulk_wait_all();
            stores_completed(x);
        }
        __syncthreads();
        if (tid < 32) {
            fence_acq_rel_gpu();
            publish(x);
        }
        return;
    }
    // error path: stop the other CTAs, let this CTA's own transfers finish, return
    if (tid == 0) {
        st_relaxed_gpu(abort_word, 1);
        atomicOr(a0.status, kStatusTimeout);
        const int64_t issued = *(volatile long long *)&s_issued;
        int st = stage;
        uint32_t ph = phase;
        for (int64_t y = x; y < issued; ++y) {
            mbar_wait_bounded(&bar[st], ph, kDrainWaitNs);
            if (++st == NSTAGE) {
                st = 0;
                ph ^= 1u;
            }
        }
    }
    if (tid == kStoreThread) bulk_wait_all();
}

cudaError_t launch_flow(const FlowMaps &maps, const FlowArgs &a, bool act, cudaStream_t stream) {
    static thread_local uint64_t configured_ctx = 0;  // attributes belong to the context
    static thread_local int resident = 0;  // co-resident CTAs per device
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (context_changed(configured_ctx)) {
        resident = 0;
        if ((e = cudaFuncSetAttribute(fk_flow_kernel<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_FLOW_BYTES)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_flow_kernel<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_FLOW_BYTES)) != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
        int per_sm_t = 0, per_sm_f = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_t, fk_flow_kernel<true>, NT,
                                                               SMEM_FLOW_BYTES)) != cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_f, fk_flow_kernel<false>, NT,
                                                               SMEM_FLOW_BYTES)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
        resident = (per_sm_t < per_sm_f ? per_sm_t : per_sm_f) * sms;
    }
    if (resident < 1) return cudaErrorInvalidConfiguration;
    const int64_t ntiles = flow_flag_words(a.in[0].H, a.in[0].W) - 1;
    const int grid = (int)(ntiles < resident ? ntiles : resident);
    if (a.nsteps < 1) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = SMEM_FLOW_BYTES;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (act) return cudaLaunchKernelEx(&cfg, fk_flow_kernel<true>, maps, a);
    return cudaLaunchKernelEx(&cfg, fk_flow_kernel<false>, maps, a);
}

}  // namespace fk
