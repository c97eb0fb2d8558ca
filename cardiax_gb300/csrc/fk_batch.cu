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
#include "fk_tb.cuh"

using namespace fk;

// The tile geometries the batched kernel is built for (fk_batch_rows32.cu, fk_batch_rows16.cu):
// rows x 64 columns, u loaded with a 4-cell halo (rows + 8 rows), D with a 2-row halo.
typedef cudaError_t (*BatchLaunchFn)(const void *, const void *, const void *, const int *, int,
                                     int, int, const int *, int, int, bool, int *, int,
                                     cudaStream_t);
cudaError_t fk_batch_launch_rows32(const void *, const void *, const void *, const int *, int, int,
                                   int, const int *, int, int, bool, int *, int, cudaStream_t);
cudaError_t fk_batch_launch_rows16(const void *, const void *, const void *, const int *, int, int,
                                   int, const int *, int, int, bool, int *, int, cudaStream_t);
namespace {
struct TileShape {
    int rows, cols, ctas_per_sm;
    BatchLaunchFn launch;
};
constexpr int kShapes = 2;
const TileShape kShape[kShapes] = {{32, 64, 2, fk_batch_launch_rows32},
                                   {16, 64, 2, fk_batch_launch_rows16}};
}  // namespace

struct fk_batch {
    int n = 0, grid = 0, device = -1;
    int shape = 0;  // index into kShape of the tile geometry in use
    // work order (0: contiguous runs; k = 1, 2, 4, 8: round-robin in chunks of k items) and
    // arithmetic of the batched kernel
    int interleave = 1, packed = 0;
    int depth = 1;                   // Euler steps per launch: 1, or 2 (blocked kernel)
    bool tb_ok = false;              // every tissue can be blocked (and no activation tracking)
    BatchTbMaps *d_tbmaps = nullptr;
    int grid_tb = 0;                 // CTAs of the blocked kernel (one per SM)
    std::vector<BatchTbMaps> h_tbmaps;
    BatchTissue *d_tissues = nullptr;
    int *d_t = nullptr;
    int *status = nullptr;
    bool act = false;
    // per tile geometry: TMA maps (box heights differ), the work list and the CTAs' runs of it
    struct PerShape {
        BatchMaps *d_maps = nullptr;
        BatchItem *d_items = nullptr;
        int *d_ranges = nullptr;  // kBatchMaxGrid + 1 item offsets: CTA c runs [r[c], r[c+1])
        int n_items = 0;
        std::vector<BatchMaps> h_maps;
        std::vector<BatchItem> h_items;
        std::vector<uint8_t> h_edge;  // per item: an edge tile
        std::vector<int> h_ranges;
    } sp[kShapes];
    // host staging (kept alive until destroy: the uploads are asynchronous)
    std::vector<BatchTissue> h_tissues;
    std::vector<int> order;        // tissues, larger first
    std::vector<fk_grid> grids;    // per tissue
    // captured graph
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0, graph_grid = 0, graph_shape = 0, graph_opts = 0, graph_depth = 1;
};

namespace {

constexpr size_t kAlign = 128;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

int64_t tiles_of(const fk_grid &g, int shape) {
    const TileShape &t = kShape[shape];
    return ((g.H + t.rows - 1) / t.rows) * ((g.W + t.cols - 1) / t.cols);
}

struct Layout {
    size_t maps[kShapes], tbmaps, tissues, items[kShapes], ranges[kShapes], t, total;
};

Layout layout(int n, const int64_t *n_items) {
    Layout L;
    size_t at = 0;
    for (int k = 0; k < kShapes; ++k) {
        L.maps[k] = at;
        at = align_up(at + sizeof(BatchMaps) * n);
    }
    L.tbmaps = at;
    at = align_up(at + sizeof(BatchTbMaps) * n);
    L.tissues = at;
    at = align_up(at + sizeof(BatchTissue) * n);
    for (int k = 0; k < kShapes; ++k) {
        L.items[k] = at;
        at = align_up(at + sizeof(BatchItem) * n_items[k]);
        L.ranges[k] = at;
        at = align_up(at + sizeof(int) * (kBatchMaxGrid + 1));
    }
    L.t = at;
    L.total = align_up(at + 16);
    return L;
}

// Relative cost of an edge tile (clamped halo, one-sided rows, bounds checks) against an
// interior one, for balancing the CTAs' runs of the work list.
constexpr double kEdgeCost = 1.1;

bool interior_tile(const fk_grid &g, int shape, int64_t i0, int64_t j0) {
    const TileShape &t = kShape[shape];
    return i0 >= BAND && i0 + t.rows <= g.H - BAND && j0 >= BAND && j0 + t.cols <= g.W - BAND;
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

// The work list of tile geometry `q` for the plan's work order, and the CTAs' runs of it.
// Interleaved order: every tissue's edge tiles (the costlier clamped-halo path) first, then the
// interior tiles, each group with the larger tissues first (CTAs take every G-th item).
// Contiguous runs: tissue by tissue (larger first), each tissue's tiles column by column, so
// that a CTA's run changes tissue rarely and its next item is usually the tile below the
// current one, whose top halo rows it has just loaded (they are still in L2).
// Round-robin in chunks of c: the kernel's CTA g of G takes items g, g + G, g + 2G, ...; the
// list is permuted so that those are c consecutive items of the natural order in turn
// (natural item x of chunk p = x / c goes to position (p / G) c G + (x % c) G + p % G), so a
// CTA steps through c neighbouring tiles, mostly of one tissue, before the next chunk.  A last
// partial block of chunks keeps the natural order.
void chunk_items(fk_batch::PerShape &P, int c, int G) {
    const int64_t n = (int64_t)P.h_items.size();
    if (c <= 1 || G < 1 || n == 0) return;
    const int64_t full = n / ((int64_t)c * G) * c * G;  // items in whole blocks
    std::vector<BatchItem> it(P.h_items);
    std::vector<uint8_t> ed(P.h_edge);
    for (int64_t x = 0; x < full; ++x) {
        const int64_t p = x / c, blk = p / G;
        const int64_t to = blk * c * G + (x % c) * G + p % G;
        P.h_items[to] = it[x];
        P.h_edge[to] = ed[x];
    }
}

void build_items(fk_batch *b, int q) {
    fk_batch::PerShape &P = b->sp[q];
    const TileShape &ts = kShape[q];
    P.h_items.clear();
    P.h_edge.clear();
    // want_edge: 1 edge only, 0 interior only, -1 both; by_column: column-major tile order
    auto add = [&](int k, int want_edge, bool by_column) {
        const fk_grid &g = b->grids[k];
        const int64_t nr = (g.H + ts.rows - 1) / ts.rows, nc = (g.W + ts.cols - 1) / ts.cols;
        for (int64_t a = 0; a < (by_column ? nc : nr); ++a)
            for (int64_t c = 0; c < (by_column ? nr : nc); ++c) {
                const int64_t i0 = (by_column ? c : a) * ts.rows, j0 = (by_column ? a : c) * ts.cols;
                const int edge = interior_tile(g, q, i0, j0) ? 0 : 1;
                if (want_edge >= 0 && edge != want_edge) continue;
                P.h_items.push_back(BatchItem{k, (int32_t)i0, (int32_t)j0, 0});
                P.h_edge.push_back((uint8_t)edge);
            }
    };
    if (b->interleave) {
        for (int k : b->order) add(k, 1, false);
        for (int k : b->order) add(k, 0, false);
        chunk_items(P, b->interleave, b->grid);
    } else {
        for (int k : b->order) add(k, -1, true);
    }
    make_ranges(P.h_items, P.h_edge, b->grid, P.h_ranges);
}

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
    int64_t items[kShapes] = {};
    for (int k = 0; k < n; ++k)
        for (int q = 0; q < kShapes; ++q) items[q] += tiles_of(tissues[k].g, q);
    return layout(n, items).total;
}

int fk_batch_create(const fk_tissue *tissues, int n, void *workspace, size_t bytes, void *stream,
                    fk_batch **out) {
    if (!tissues || !workspace || !out) return FK_ERR_NULL;
    if (n <= 0 || n > (1 << 20)) return FK_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(workspace) & (kAlign - 1)) != 0) return FK_ERR_ALIGN;
    int64_t n_items[kShapes] = {};
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
        for (int q = 0; q < kShapes; ++q) n_items[q] += tiles_of(t.g, q);
    }
    if (any_act && !all_act) return FK_ERR_ARGUMENT;  // tracking is all or nothing per batch
    for (int q = 0; q < kShapes; ++q)
        if (n_items[q] > (int64_t(1) << 30)) return FK_ERR_SHAPE;
    const Layout L = layout(n, n_items);
    if (bytes < L.total) return FK_ERR_ARGUMENT;

    fk_batch *b = new (std::nothrow) fk_batch();
    if (!b) return FK_ERR_ARGUMENT;
    b->n = n;
    b->act = any_act;
    b->status = status_ptr();
    if (!b->status || cudaGetDevice(&b->device) != cudaSuccess) {
        delete b;
        return FK_ERR_CUDA;
    }
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device);
    b->grid = n_sm > 0 ? n_sm * kShape[0].ctas_per_sm : 1;
    b->grid_tb = n_sm > 0 ? n_sm : 1;
    if (b->grid > kBatchMaxGrid) b->grid = kBatchMaxGrid;
    char *ws = static_cast<char *>(workspace);
    b->d_tissues = reinterpret_cast<BatchTissue *>(ws + L.tissues);
    b->d_tbmaps = reinterpret_cast<BatchTbMaps *>(ws + L.tbmaps);
    b->h_tbmaps.resize(n);
    b->tb_ok = !any_act;
    for (int k = 0; k < n; ++k) b->tb_ok &= tb_batchable(tissues[k].g.H, tissues[k].g.W);
    b->d_t = reinterpret_cast<int *>(ws + L.t);
    b->h_tissues.resize(n);
    for (int q = 0; q < kShapes; ++q) {
        fk_batch::PerShape &P = b->sp[q];
        P.d_maps = reinterpret_cast<BatchMaps *>(ws + L.maps[q]);
        P.d_items = reinterpret_cast<BatchItem *>(ws + L.items[q]);
        P.d_ranges = reinterpret_cast<int *>(ws + L.ranges[q]);
        P.n_items = (int)n_items[q];
        P.h_maps.resize(n);
    }

    // tiles of the larger tissues first: the persistent CTAs then finish together
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return tiles_of(tissues[x].g, 0) > tiles_of(tissues[y].g, 0);
    });
    for (int k = 0; k < n; ++k) {
        const fk_tissue &t = tissues[k];
        const int64_t plane = t.g.H * t.g.pitch;
        Stim st[kMaxStim];
        int rc = make_stims(t.stimuli, t.n_stimuli, t.g, st);
        const Model m = make_model(t.params);
        // TMA maps per geometry: u with a 4-cell halo, D with a 2-row halo (columns: 4 cells)
        for (int q = 0; q < kShapes && !rc; ++q) {
            const TileShape &ts = kShape[q];
            const int sw = ts.cols + 8, su_h = ts.rows + 8, sd_h = ts.rows + 4;
            BatchMaps &bm = b->sp[q].h_maps[k];
            if ((rc = make_plane_map(&bm.maps[0].d, t.D, t.g.H, t.g.W, t.g.pitch, sw, sd_h))) break;
            for (int p = 0; p < 2 && !rc; ++p) {
                const float *in = p ? t.scratch : t.state;
                float *o = p ? t.state : t.scratch;
                StepMaps &sm = bm.maps[p];
                if (p) sm.d = bm.maps[0].d;
                if ((rc = make_plane_map(&sm.u, in + 2 * plane, t.g.H, t.g.W, t.g.pitch, sw, su_h)) ||
                    (rc = make_plane_map(&sm.ov, o, t.g.H, t.g.W, t.g.pitch, ts.cols, ts.rows)) ||
                    (rc = make_plane_map(&sm.ow, o + plane, t.g.H, t.g.W, t.g.pitch, ts.cols,
                                         ts.rows)) ||
                    (rc = make_plane_map(&sm.ou, o + 2 * plane, t.g.H, t.g.W, t.g.pitch, ts.cols,
                                         ts.rows)))
                    break;
            }
        }
        // the blocked kernel's maps (haloed boxes of the loaded planes, output-tile boxes)
        if (!rc && b->tb_ok) {
            int bw = 0, bh = 0, ow = 0, oh = 0;
            tb_box(kBatchTbDepth, &bw, &bh, &ow, &oh);
            const fk_grid &g = t.g;
            for (int p = 0; p < 2 && !rc; ++p) {
                const float *in = p ? t.scratch : t.state;
                float *o = p ? t.state : t.scratch;
                TbMaps &tm = b->h_tbmaps[k].maps[p];
                if ((rc = make_plane_map(&tm.d, t.D, g.H, g.W, g.pitch, bw, bh)) ||
                    (rc = make_plane_map(&tm.v, in, g.H, g.W, g.pitch, bw, bh)) ||
                    (rc = make_plane_map(&tm.w, in + plane, g.H, g.W, g.pitch, bw, bh)) ||
                    (rc = make_plane_map(&tm.u, in + 2 * plane, g.H, g.W, g.pitch, bw, bh)) ||
                    (rc = make_plane_map(&tm.ov, o, g.H, g.W, g.pitch, ow, oh)) ||
                    (rc = make_plane_map(&tm.ow, o + plane, g.H, g.W, g.pitch, ow, oh)) ||
                    (rc = make_plane_map(&tm.ou, o + 2 * plane, g.H, g.W, g.pitch, ow, oh)))
                    break;
            }
        }
        for (int p = 0; p < 2 && !rc; ++p) {
            const float *in = p ? t.scratch : t.state;
            float *o = p ? t.state : t.scratch;
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
    b->order = order;
    b->grids.resize(n);
    for (int k = 0; k < n; ++k) b->grids[k] = tissues[k].g;
    for (int q = 0; q < kShapes; ++q) build_items(b, q);
    cudaStream_t s = (cudaStream_t)stream;
    bool ok = cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(BatchTissue) * n,
                              cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (ok && b->tb_ok)
        ok = cudaMemcpyAsync(b->d_tbmaps, b->h_tbmaps.data(), sizeof(BatchTbMaps) * n,
                             cudaMemcpyHostToDevice, s) == cudaSuccess;
    for (int q = 0; q < kShapes && ok; ++q) {
        const fk_batch::PerShape &P = b->sp[q];
        ok = cudaMemcpyAsync(P.d_maps, P.h_maps.data(), sizeof(BatchMaps) * n,
                             cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemcpyAsync(P.d_items, P.h_items.data(), sizeof(BatchItem) * P.n_items,
                             cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemcpyAsync(P.d_ranges, P.h_ranges.data(), sizeof(int) * P.h_ranges.size(),
                             cudaMemcpyHostToDevice, s) == cudaSuccess;
    }
    if (!ok || cudaStreamSynchronize(s) != cudaSuccess) {
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
    // ordered after the plan's earlier work; the host copies stay alive in the plan
    if (cudaDeviceSynchronize() != cudaSuccess) return FK_ERR_CUDA;
    b->grid = ctas;
    for (int q = 0; q < kShapes; ++q) {
        fk_batch::PerShape &P = b->sp[q];
        if (b->interleave > 1) {  // the chunk permutation depends on the CTA count
            build_items(b, q);
            if (cudaMemcpy(P.d_items, P.h_items.data(), sizeof(BatchItem) * P.n_items,
                           cudaMemcpyHostToDevice) != cudaSuccess)
                return FK_ERR_CUDA;
        }
        std::vector<int> r;
        make_ranges(P.h_items, P.h_edge, ctas, r);
        if (cudaMemcpy(P.d_ranges, r.data(), sizeof(int) * r.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return FK_ERR_CUDA;
        P.h_ranges.swap(r);
    }
    release_graph(b);
    return FK_OK;
}

int fk_batch_set_options(fk_batch *b, int interleave, int packed) {
    if (!b) return FK_ERR_NULL;
    if (interleave != 0 && interleave != 1 && interleave != 2 && interleave != 4 &&
        interleave != 8)
        return FK_ERR_ARGUMENT;
    const int il = interleave, pk = packed ? 1 : 0;
    if (il != b->interleave || pk != b->packed) release_graph(b);
    b->packed = pk;
    if (il == b->interleave) return FK_OK;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return FK_ERR_CUDA;
    b->interleave = il;
    // the work lists change order: rebuild and upload them after the plan's earlier work
    if (cudaDeviceSynchronize() != cudaSuccess) return FK_ERR_CUDA;
    for (int q = 0; q < kShapes; ++q) {
        build_items(b, q);
        const fk_batch::PerShape &P = b->sp[q];
        if (cudaMemcpy(P.d_items, P.h_items.data(), sizeof(BatchItem) * P.n_items,
                       cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(P.d_ranges, P.h_ranges.data(), sizeof(int) * P.h_ranges.size(),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return FK_ERR_CUDA;
    }
    return FK_OK;
}

int fk_batch_set_depth(fk_batch *b, int depth) {
    if (!b) return FK_ERR_NULL;
    if (depth != 1 && depth != kBatchTbDepth) return FK_ERR_ARGUMENT;
    if (depth != 1 && !b->tb_ok) return FK_ERR_ARGUMENT;
    if (depth != b->depth) release_graph(b);
    b->depth = depth;
    return FK_OK;
}

int fk_batch_set_tile_rows(fk_batch *b, int rows) {
    if (!b) return FK_ERR_NULL;
    for (int q = 0; q < kShapes; ++q)
        if (kShape[q].rows == rows) {
            if (b->shape != q) release_graph(b);
            b->shape = q;
            return FK_OK;
        }
    return FK_ERR_ARGUMENT;
}

static cudaError_t launch_one(const fk_batch *b, int n_items, int t_offset, int parity, bool act,
                              cudaStream_t s) {
    const fk_batch::PerShape &P = b->sp[b->shape];
    return kShape[b->shape].launch(b->d_tissues, P.d_maps, P.d_items, P.d_ranges, n_items,
                                   b->interleave, b->packed, b->d_t, t_offset, parity, act,
                                   b->status, b->grid, s);
}

// Buffer flips of `count` steps (each launch reads one buffer and writes the other): one per
// step at depth 1; at depth 2 one per pair of steps plus one for an odd last step.
static int64_t flips(const fk_batch *b, int64_t count) {
    return b->depth == 1 ? count : count / 2 + (count & 1);
}

static int launch_steps(fk_batch *b, int count, cudaStream_t s) {
    if (b->depth == 1) {
        const int n_items = b->sp[b->shape].n_items;
        for (int k = 0; k < count; ++k)
            if (launch_one(b, n_items, k, k & 1, b->act, s) != cudaSuccess) return FK_ERR_CUDA;
    } else {  // two steps per launch of the blocked kernel (32 x 64 work items), then the odd one
        const fk_batch::PerShape &P = b->sp[0];
        int k = 0, f = 0;
        for (; k + 2 <= count; k += 2, ++f)
            if (launch_batch_tb(b->d_tissues, b->d_tbmaps, P.d_items, P.n_items, b->d_t, k, f & 1,
                                b->status, b->grid_tb, s) != cudaSuccess)
                return FK_ERR_CUDA;
        if (k < count &&
            launch_one(b, b->sp[b->shape].n_items, k, f & 1, b->act, s) != cudaSuccess)
            return FK_ERR_CUDA;
    }
    return launch_add_int(b->d_t, count, s) == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

static int ensure_graph(fk_batch *b, int steps) {
    const int opts = b->interleave * 2 + b->packed;
    if (b->exec && b->graph_steps == steps && b->graph_grid == b->grid &&
        b->graph_shape == b->shape && b->graph_opts == opts && b->graph_depth == b->depth)
        return FK_OK;
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
    b->graph_shape = b->shape;
    b->graph_opts = opts;
    b->graph_depth = b->depth;
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
        // a replay must flip the buffers an even number of times: G steps, G even (depth 1) or
        // a multiple of 4 (depth 2: G / 2 launches)
        const int q = b->depth == 1 ? 2 : 4;
        const int G = (graph_steps + q - 1) / q * q;
        if (n >= G) {
            if (!b->exec || b->graph_steps != G || b->graph_grid != b->grid ||
                b->graph_shape != b->shape || b->graph_opts != b->interleave * 2 + b->packed ||
                b->graph_depth != b->depth) {
                if ((rc = launch_steps(b, 0, s))) return rc;
                if (launch_one(b, 0, 0, 0, b->act, s) != cudaSuccess)  // configures the kernel
                    return FK_ERR_CUDA;
                if (b->depth != 1 &&
                    launch_batch_tb(b->d_tissues, b->d_tbmaps, b->sp[0].d_items, 0, b->d_t, 0, 0,
                                    b->status, b->grid_tb, s) != cudaSuccess)
                    return FK_ERR_CUDA;
                if ((rc = ensure_graph(b, G))) return rc;
            }
            for (int64_t r = 0; r < n / G; ++r)
                if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return FK_ERR_CUDA;
            n %= G;
        }
    }
    if ((rc = launch_steps(b, (int)n, s))) return rc;
    if (flips(b, n) & 1) {  // the replayed graphs flipped an even number of times
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
        if (launch_one(b, b->sp[b->shape].n_items, (int)(k - 1), (int)((k - 1) & 1), false, cs) !=
            cudaSuccess)
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
