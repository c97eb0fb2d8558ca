// C ABI of the batched path: many tissues advanced by one persistent kernel per step, with
// runs of steps captured into a CUDA graph.  No reference counterpart (the reference loops over
// tissues in Python, deepx/generate.py:135-210); per tissue the arithmetic is exactly that of
// fk_forward_euler (cardiax/solve.py:92-100), bit for bit.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/cardiax_gb300.h"
#include "fk_capi_internal.h"
#include "fk_step.cuh"

using namespace fk;

struct fk_batch {
    int n = 0, n_items = 0, grid = 0, device = -1;
    BatchMaps *d_maps = nullptr;
    BatchTissue *d_tissues = nullptr;
    BatchItem *d_items = nullptr;
    int *d_ranges = nullptr;  // kBatchMaxGrid + 1 item offsets: CTA c runs [r[c], r[c+1])
    int *d_t = nullptr;
    int *status = nullptr;
    bool act = false;
    // host staging (kept alive until destroy: the uploads are asynchronous)
    std::vector<BatchMaps> h_maps;
    std::vector<BatchTissue> h_tissues;
    std::vector<BatchItem> h_items;
    std::vector<int> h_ranges;
    std::vector<uint8_t> h_edge;  // per item: an edge tile
    // captured graph
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0, graph_grid = 0;
};

namespace {

constexpr size_t kAlign = 128;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

int64_t tiles_of(const fk_grid &g) { return ((g.H + TY - 1) / TY) * ((g.W + TX - 1) / TX); }

struct Layout {
    size_t maps, tissues, items, ranges, t, total;
};

Layout layout(int n, int64_t n_items) {
    Layout L;
    L.maps = 0;
    L.tissues = align_up(L.maps + sizeof(BatchMaps) * n);
    L.items = align_up(L.tissues + sizeof(BatchTissue) * n);
    L.ranges = align_up(L.items + sizeof(BatchItem) * n_items);
    L.t = align_up(L.ranges + sizeof(int) * (kBatchMaxGrid + 1));
    L.total = align_up(L.t + 16);
    return L;
}

// Relative cost of an edge tile (clamped halo, one-sided rows, bounds checks) against an
// interior one, for balancing the CTAs' runs of the work list.
constexpr double kEdgeCost = 1.1;

bool interior_tile(const fk_grid &g, int64_t i0, int64_t j0) {
    return i0 >= BAND && i0 + TY <= g.H - BAND && j0 >= BAND && j0 + TX <= g.W - BAND;
}

// Cuts the work list into `grid` contiguous runs of about equal cost: r[c] .. r[c+1] for CTA c.
void make_ranges(const std::vector<BatchItem> &items, const std::vector<uint8_t> &edge, int grid,
                 std::vector<int> &r) {
    const int n = (int)items.size();
    double total = 0.0;
    for (int k = 0; k < n; ++k) total += edge[k] ? kEdgeCost : 1.0;
    r.assign(grid + 1, n);
    r[0] = 0;
    double acc = 0.0;
    int c = 1;
    for (int k = 0; k < n && c < grid; ++k) {
        acc += edge[k] ? kEdgeCost : 1.0;
        while (c < grid && acc >= total * c / grid) r[c++] = k + 1;
    }
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

void release_graph(fk_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_steps = 0;
}

}  // namespace

extern "C" {

size_t fk_batch_workspace_bytes(const fk_tissue *tissues, int n) {
    if (!tissues || n <= 0) return 0;
    int64_t items = 0;
    for (int k = 0; k < n; ++k) items += tiles_of(tissues[k].g);
    return layout(n, items).total;
}

int fk_batch_create(const fk_tissue *tissues, int n, void *workspace, size_t bytes, void *stream,
                    fk_batch **out) {
    if (!tissues || !workspace || !out) return FK_ERR_NULL;
    if (n <= 0 || n > (1 << 20)) return FK_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(workspace) & (kAlign - 1)) != 0) return FK_ERR_ALIGN;
    int64_t n_items = 0;
    bool any_act = false, all_act = true;
    for (int k = 0; k < n; ++k) {
        const fk_tissue &t = tissues[k];
        int rc = check_grid(t.g);
        if (rc) return rc;
        if (!t.state || !t.scratch || !t.D) return FK_ERR_NULL;
        if (!aligned16(t.state) || !aligned16(t.scratch) || !aligned16(t.D)) return FK_ERR_ALIGN;
        if (!(t.dx > 0.0) || !std::isfinite(t.dx) || !std::isfinite(t.dt)) return FK_ERR_ARGUMENT;
        const bool a = t.act.last != nullptr;
        if (a && (!t.act.first || !t.act.count)) return FK_ERR_NULL;
        any_act |= a;
        all_act &= a;
        n_items += tiles_of(t.g);
    }
    if (any_act && !all_act) return FK_ERR_ARGUMENT;  // tracking is all or nothing per batch
    if (n_items > (int64_t(1) << 30)) return FK_ERR_SHAPE;
    const Layout L = layout(n, n_items);
    if (bytes < L.total) return FK_ERR_ARGUMENT;

    fk_batch *b = new (std::nothrow) fk_batch();
    if (!b) return FK_ERR_ARGUMENT;
    b->n = n;
    b->n_items = (int)n_items;
    b->act = any_act;
    b->status = status_ptr();
    if (!b->status || cudaGetDevice(&b->device) != cudaSuccess) {
        delete b;
        return FK_ERR_CUDA;
    }
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device);
    b->grid = n_sm > 0 ? n_sm * CTAS_PER_SM : 1;
    char *ws = static_cast<char *>(workspace);
    b->d_maps = reinterpret_cast<BatchMaps *>(ws + L.maps);
    b->d_tissues = reinterpret_cast<BatchTissue *>(ws + L.tissues);
    b->d_items = reinterpret_cast<BatchItem *>(ws + L.items);
    b->d_ranges = reinterpret_cast<int *>(ws + L.ranges);
    b->d_t = reinterpret_cast<int *>(ws + L.t);
    b->h_maps.resize(n);
    b->h_tissues.resize(n);
    b->h_items.reserve(n_items);

    // tiles of the larger tissues first: the persistent CTAs then finish together
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return tiles_of(tissues[x].g) > tiles_of(tissues[y].g);
    });
    for (int k = 0; k < n; ++k) {
        const fk_tissue &t = tissues[k];
        const int64_t plane = t.g.H * t.g.pitch;
        Stim st[kMaxStim];
        int rc = make_stims(t.stimuli, t.n_stimuli, t.g, st);
        if (!rc) rc = make_plane_map(&b->h_maps[k].maps[0].d, t.D, t.g.H, t.g.W, t.g.pitch, SW, SD_H);
        const Model m = make_model(t.params);
        for (int p = 0; p < 2 && !rc; ++p) {
            const float *in = p ? t.scratch : t.state;
            float *o = p ? t.state : t.scratch;
            StepMaps &sm = b->h_maps[k].maps[p];
            if (p) sm.d = b->h_maps[k].maps[0].d;
            if ((rc = make_plane_map(&sm.u, in + 2 * plane, t.g.H, t.g.W, t.g.pitch, SW, SU_H)) ||
                (rc = make_plane_map(&sm.ov, o, t.g.H, t.g.W, t.g.pitch, TX, TY)) ||
                (rc = make_plane_map(&sm.ow, o + plane, t.g.H, t.g.W, t.g.pitch, TX, TY)) ||
                (rc = make_plane_map(&sm.ou, o + 2 * plane, t.g.H, t.g.W, t.g.pitch, TX, TY)))
                break;
            StepArgs &a = b->h_tissues[k].args[p];
            std::memset(&a, 0, sizeof(a));
            a.v = in;
            a.w = in + plane;
            a.u = in + 2 * plane;
            a.D = t.D;
            a.vo = o;
            a.wo = o + plane;
            a.uo = o + 2 * plane;
            a.H = (int)t.g.H;
            a.W = (int)t.g.W;
            a.pitch = (int)t.g.pitch;
            a.dt = (float)t.dt;
            a.rdx = 1.0f / (float)t.dx;
            a.n_stim = t.n_stimuli;
            a.m = m;
            for (int s = 0; s < t.n_stimuli; ++s) a.stim[s] = st[s];
            a.status = b->status;
            if (any_act) {
                a.act_first = t.act.first;
                a.act_last = t.act.last;
                a.act_count = t.act.count;
                a.act_threshold = t.act.threshold;
            }
        }
        if (rc) {
            delete b;
            return rc;
        }
    }
    // work list: tissue by tissue (larger tissues first), each tissue's tiles row by row, so that
    // a CTA's contiguous run of items changes tissue rarely; the runs are balanced by cost
    for (int k : order) {
        const fk_grid &g = tissues[k].g;
        for (int64_t i0 = 0; i0 < g.H; i0 += TY)
            for (int64_t j0 = 0; j0 < g.W; j0 += TX) {
                b->h_items.push_back(BatchItem{k, (int32_t)i0, (int32_t)j0, 0});
                b->h_edge.push_back(interior_tile(g, i0, j0) ? 0 : 1);
            }
    }
    if (b->grid > kBatchMaxGrid) b->grid = kBatchMaxGrid;
    make_ranges(b->h_items, b->h_edge, b->grid, b->h_ranges);
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(b->d_maps, b->h_maps.data(), sizeof(BatchMaps) * n,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(BatchTissue) * n,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_items, b->h_items.data(), sizeof(BatchItem) * b->n_items,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_ranges, b->h_ranges.data(), sizeof(int) * b->h_ranges.size(),
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        delete b;
        return FK_ERR_CUDA;
    }
    *out = b;
    return FK_OK;
}

int fk_batch_set_grid(fk_batch *b, int ctas) {
    if (!b) return FK_ERR_NULL;
    if (ctas < 1 || ctas > kBatchMaxGrid) return FK_ERR_ARGUMENT;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return FK_ERR_CUDA;
    std::vector<int> r;
    make_ranges(b->h_items, b->h_edge, ctas, r);
    // ordered after the plan's earlier work on the legacy stream; the host copy stays alive
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(b->d_ranges, r.data(), sizeof(int) * r.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return FK_ERR_CUDA;
    b->h_ranges.swap(r);
    b->grid = ctas;
    release_graph(b);
    return FK_OK;
}

static int launch_steps(fk_batch *b, int count, cudaStream_t s) {
    for (int k = 0; k < count; ++k) {
        cudaError_t e = launch_batch_step(b->d_tissues, b->d_maps, b->d_items, b->d_ranges,
                                          b->n_items, b->d_t, k, k & 1, b->act, b->status,
                                          b->grid, s);
        if (e != cudaSuccess) return FK_ERR_CUDA;
    }
    return launch_add_int(b->d_t, count, s) == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

static int ensure_graph(fk_batch *b, int steps) {
    if (b->exec && b->graph_steps == steps && b->graph_grid == b->grid) return FK_OK;
    release_graph(b);
    if (!b->capture_stream &&
        cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
        return FK_ERR_CUDA;
    // first launch of each kernel outside capture (sets function attributes)
    if (cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return FK_ERR_CUDA;
    int rc = launch_steps(b, steps, b->capture_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : FK_ERR_CUDA;
    }
    if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return FK_ERR_CUDA;
    }
    b->graph = g;
    b->graph_steps = steps;
    b->graph_grid = b->grid;
    return FK_OK;
}

__global__ static void set_int_kernel(int *p, int v) { *p = v; }

int fk_batch_forward_euler(fk_batch *b, int64_t t0, int64_t t1, int graph_steps, void *stream) {
    if (!b) return FK_ERR_NULL;
    if (t1 < t0 || t1 > (int64_t(1) << 24) || t0 < -(int64_t(1) << 24) || graph_steps < 0)
        return FK_ERR_ARGUMENT;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return FK_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    int64_t n = t1 - t0;
    if (n == 0) return FK_OK;
    set_int_kernel<<<1, 1, 0, s>>>(b->d_t, (int)t0);
    if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
    // the smem attribute must be set outside any capture: one plain (empty-range) call does it
    int rc;
    if (graph_steps > 0) {
        const int G = (graph_steps + 1) / 2 * 2;
        if (n >= G) {
            if (!b->exec || b->graph_steps != G || b->graph_grid != b->grid) {
                if ((rc = launch_steps(b, 0, s))) return rc;  // configures the kernel
                if (launch_batch_step(b->d_tissues, b->d_maps, b->d_items, b->d_ranges, 0,
                                      b->d_t, 0, 0, b->act, b->status, b->grid, s) != cudaSuccess)
                    return FK_ERR_CUDA;
                if ((rc = ensure_graph(b, G))) return rc;
            }
            for (int64_t r = 0; r < n / G; ++r)
                if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return FK_ERR_CUDA;
            n %= G;
        }
    }
    if ((rc = launch_steps(b, (int)n, s))) return rc;
    if ((t1 - t0) & 1) {
        if (launch_batch_copyback(b->d_tissues, b->n, s) != cudaSuccess) return FK_ERR_CUDA;
    }
    return FK_OK;
}

// Copies the state held by buffer `parity` of every tissue (0: state, 1: scratch; three
// consecutive planes) to dst + e * exp_stride (tissue e, all on one grid of `ns` floats).
__global__ static void batch_state_out_kernel(const BatchTissue *tissues, int parity, float *dst,
                                              int64_t exp_stride, int64_t ns) {
    const float4 *src = reinterpret_cast<const float4 *>(tissues[blockIdx.y].args[parity].v);
    float4 *out = reinterpret_cast<float4 *>(dst + (int64_t)blockIdx.y * exp_stride);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ns / 4;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = __ldcg(src + k);
}

int fk_batch_recompute(fk_batch *b, int64_t s, int64_t n, float *bufs, int64_t exp_stride,
                       void *stream) {
    if (!b || !bufs) return FK_ERR_NULL;
    if (n < 1 || s < -(int64_t(1) << 24) || s + n > (int64_t(1) << 24)) return FK_ERR_ARGUMENT;
    if (b->act) return FK_ERR_ARGUMENT;  // recomputed steps must not record activations again
    const StepArgs &a0 = b->h_tissues[0].args[0];
    for (int e = 1; e < b->n; ++e) {
        const StepArgs &a = b->h_tissues[e].args[0];
        if (a.H != a0.H || a.W != a0.W || a.pitch != a0.pitch) return FK_ERR_SHAPE;
    }
    const int64_t ns = 3 * (int64_t)a0.H * a0.pitch;
    if (exp_stride < n * ns || (reinterpret_cast<uintptr_t>(bufs) & 15u) || (exp_stride & 3))
        return FK_ERR_ALIGN;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return FK_ERR_CUDA;
    cudaStream_t cs = (cudaStream_t)stream;
    set_int_kernel<<<1, 1, 0, cs>>>(b->d_t, (int)s);
    const dim3 cgrid(64, b->n);
    batch_state_out_kernel<<<cgrid, 256, 0, cs>>>(b->d_tissues, 0, bufs, exp_stride, ns);
    if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
    for (int64_t k = 1; k < n; ++k) {
        // step s+k-1 reads buffer (k-1)&1 and leaves x_{s+k} in buffer k&1
        if (launch_batch_step(b->d_tissues, b->d_maps, b->d_items, b->d_ranges, b->n_items,
                              b->d_t, (int)(k - 1), (int)((k - 1) & 1), false, b->status, b->grid,
                              cs) != cudaSuccess)
            return FK_ERR_CUDA;
        batch_state_out_kernel<<<cgrid, 256, 0, cs>>>(b->d_tissues, (int)(k & 1), bufs + k * ns,
                                                      exp_stride, ns);
        if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
    }
    return FK_OK;
}

int fk_batch_destroy(fk_batch *b) {
    if (!b) return FK_ERR_NULL;
    release_graph(b);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    delete b;
    return FK_OK;
}

}  // extern "C"
