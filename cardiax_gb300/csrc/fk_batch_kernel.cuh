// K4: the batched kernel -- many tissues advanced by one persistent launch per Euler step --
// and its launcher, for the tile geometry of the including translation unit (fk_step.cuh:
// FK_TILE_Y / FK_TILE_X / FK_TILE_NS).  fk_batch_rows32.cu builds the default 32 x 64 tiles and
// fk_batch_rows16.cu 16 x 64 tiles; the batch plan picks one (fk_batch_set_tile_rows).
//
// Per tissue the arithmetic is that of fk_forward_euler (cardiax/solve.py:92-100), bit for bit.
#pragma once
#include "fk_capi_internal.h"
#include "fk_tile.cuh"

namespace FK_TILE_NS {

// ---- batched kernel: persistent CTAs over the tiles of many tissues ------------------------
// Work order (uniform flag `interleave`): CTA c takes items c, c + G, c + 2G, ... (G CTAs: every
// CTA sweeps the list at the same pace, so vertically neighbouring tiles of a tissue are loaded
// at about the same time and share their halo rows in L2), or the contiguous run
// items[ranges[c] .. ranges[c+1]) that the host balanced by cost (consecutive items of a CTA
// then mostly belong to one tissue).  A tissue's arguments are staged into shared memory, and
// its stimulus mask formed, whenever the tissue differs from the previous item's.
// PK: the packed arithmetic of the single-tissue kernel, with the launch-wide stencil
// coefficients of `kc` as constant-bank operands and the tissue's 1/dx and dt from its staged
// arguments; otherwise the scalar arithmetic.  Both give the same bits.
template <bool ACT, bool PK>
__global__ void __launch_bounds__(NT, CTAS_PER_SM)
    fk_batch_kernel(const BatchTissue *__restrict__ tissues, const BatchMaps *__restrict__ maps,
                    const BatchItem *__restrict__ items, const int *__restrict__ ranges,
                    int n_items, int interleave, const int *t_dev, int t_offset, int parity,
                    int *status, const __grid_constant__ PackConsts kc) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    // as fk_step_kernel: u_x / u_y double-buffered, new state stored from registers; two slots
    // for staged tissue arguments (a new tissue is staged while slower warps may still be in
    // pass 2 of the previous item)
    float *sux = reinterpret_cast<float *>(smem + NSTAGE * SMEM_STAGE_BYTES);  // [2][SUX_H][TX]
    float *suy = sux + 2 * TX * SUX_H;                                           // [2][TY][SW]
    TileIO io;
    io.ov = io.ow = io.ou = nullptr;
    uint64_t *bar = reinterpret_cast<uint64_t *>(suy + 2 * SW * TY);            // [NSTAGE]
    unsigned char *args = reinterpret_cast<unsigned char *>(bar + NSTAGE);       // [2] StepArgs

    const int tid = threadIdx.x;
    const int first = interleave ? (int)blockIdx.x : ranges[blockIdx.x];
    const int stop = interleave ? n_items : ranges[blockIdx.x + 1];
    const int stride = interleave ? (int)gridDim.x : 1;
    if (tid == 0) {
        for (int q = 0; q < NSTAGE; ++q) mbar_init(&bar[q], 1);
        fence_barrier_init();
    }
    __syncthreads();
    grid_dependency_wait();  // the previous step (and the step counter) are complete
    grid_launch_dependents();
    if (first >= stop) return;
    const float t = (float)(*t_dev + t_offset);
    auto issue = [&](int x, int st) {
        const BatchItem b = items[x];
        issue_tile(maps[b.tissue].maps[parity], stage_at(smem, st), &bar[st], b.i0, b.j0);
    };
    if (tid == 0)
        for (int q = 0; q < NSTAGE - 1; ++q)
            if (first + q * stride < stop) issue(first + q * stride, q);
    // A tissue's arguments are one 32-bit word per thread.  The next item's descriptor is loaded
    // at the start of an item and, when its tissue differs, that tissue's argument word right
    // after the item's pass barrier: both loads are in flight while the item computes, and a
    // tissue change costs a shared-memory store and a barrier.
    constexpr int AW = (int)(sizeof(StepArgs) / 4);
    static_assert(AW <= NT, "one argument word per thread");
    auto arg_word = [&](int tissue) -> uint32_t {
        return tid < AW
                   ? __ldg(reinterpret_cast<const uint32_t *>(&tissues[tissue].args[parity]) + tid)
                   : 0u;
    };
    BatchItem b = items[first];
    uint32_t pw = arg_word(b.tissue);
    int cur = -1, slot = 1;
    unsigned active = 0;
    for (int it = first, n = 0; it < stop; it += stride, ++n) {
        const int s = n % NSTAGE;
        const BatchItem nb = it + stride < stop ? items[it + stride] : b;
        if (b.tissue != cur) {  // uniform: every thread read the same item
            slot ^= 1;
            StepArgs *sa = reinterpret_cast<StepArgs *>(args + slot * SMEM_ARGS_BYTES);
            if (tid < AW) reinterpret_cast<uint32_t *>(sa)[tid] = pw;
            __syncthreads();
            cur = b.tissue;
            active = 0;
            for (int q = 0; q < sa->n_stim; ++q)
                if (stim_active(sa->stim[q], t)) active |= 1u << q;
        }
        const StepArgs &A = *reinterpret_cast<const StepArgs *>(args + slot * SMEM_ARGS_BYTES);
        load_vw(A, b.i0, b.j0, io);
        const bool ok = mbar_wait_bounded(&bar[s], (n / NSTAGE) & 1);
        const int ahead = it + (NSTAGE - 1) * stride;
        auto refill = [&] {  // after the pass barrier: item n-1 is done, its stage is free
            if (tid == 0 && ahead < stop) issue(ahead, (n + NSTAGE - 1) % NSTAGE);
            if (nb.tissue != b.tissue) pw = arg_word(nb.tissue);
        };
        float *ux_n = sux + (n & 1) * (TX * SUX_H), *uy_n = suy + (n & 1) * (SW * TY);
        PairScale ps;
        ps.rdx = make_float2(A.rdx, A.rdx);
        ps.dt = make_float2(A.dt, A.dt);
        if (!process_tile<false, ACT, PK, true>(A, t, stage_at(smem, s), ux_n, uy_n, io, active,
                                                b.i0, b.j0, NoHook{}, PK ? &kc : nullptr, ps, ok,
                                                refill)) {
            if (tid == 0) {
                atomicOr(status, kStatusTimeout);
                drain_stages(bar, n, it, stride, stop);
            }
            return;
        }
        b = nb;
    }
}

cudaError_t launch_batch_step(const BatchTissue *tissues, const BatchMaps *maps,
                              const BatchItem *items, const int *ranges, int n_items,
                              int interleave, int packed, const int *t_dev, int t_offset,
                              int parity, bool act, int *status, int grid, cudaStream_t stream) {
    // function attributes belong to the context: set again whenever it changes
    static thread_local uint64_t configured_ctx = 0;
    if (context_changed(configured_ctx)) {
        cudaError_t e;
        if ((e = cudaFuncSetAttribute(fk_batch_kernel<true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BATCH_BYTES)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_batch_kernel<false, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BATCH_BYTES)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_batch_kernel<true, false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BATCH_BYTES)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(fk_batch_kernel<false, false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BATCH_BYTES)) != cudaSuccess) {
            configured_ctx = 0;
            return e;
        }
    }
    if (grid < 1 || n_items < 1) return cudaSuccess;
    // launch-wide stencil coefficients (the per-tissue 1/dx, dt and model come from the
    // tissues' own arguments)
    static const PackConsts kc = make_pack_consts(Model{}, 1.0f, 1.0f);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = SMEM_BATCH_BYTES;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int il = interleave ? 1 : 0;
    if (act && packed)
        return cudaLaunchKernelEx(&cfg, fk_batch_kernel<true, true>, tissues, maps, items, ranges,
                                  n_items, il, t_dev, t_offset, parity, status, kc);
    if (act)
        return cudaLaunchKernelEx(&cfg, fk_batch_kernel<true, false>, tissues, maps, items, ranges,
                                  n_items, il, t_dev, t_offset, parity, status, kc);
    if (packed)
        return cudaLaunchKernelEx(&cfg, fk_batch_kernel<false, true>, tissues, maps, items, ranges,
                                  n_items, il, t_dev, t_offset, parity, status, kc);
    return cudaLaunchKernelEx(&cfg, fk_batch_kernel<false, false>, tissues, maps, items, ranges,
                              n_items, il, t_dev, t_offset, parity, status, kc);
}

}  // namespace FK_TILE_NS

// The launcher under a name of its own per tile geometry (FK_BATCH_LAUNCHER, set by the
// including translation unit), with the descriptor arrays passed untyped: the plan builds them
// once (their layout does not depend on the tile geometry) and calls the variant it chose.
cudaError_t FK_BATCH_LAUNCHER(const void *tissues, const void *maps, const void *items,
                              const int *ranges, int n_items, int interleave, int packed,
                              const int *t_dev, int t_offset, int parity, bool act, int *status,
                              int grid, cudaStream_t stream) {
    using namespace FK_TILE_NS;
    return launch_batch_step(static_cast<const BatchTissue *>(tissues),
                             static_cast<const BatchMaps *>(maps),
                             static_cast<const BatchItem *>(items), ranges, n_items, interleave,
                             packed, t_dev, t_offset, parity, act, status, grid, stream);
}
