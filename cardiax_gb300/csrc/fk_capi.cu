// C ABI of the single-tissue stepper: argument checks, TMA descriptors, step loops.
//
// Entry points and the reference functions they replace:
//   fk_init           cardiax/solve.py:18-23   init
//   fk_step           cardiax/solve.py:26-65   step (time derivative)
//   fk_euler_step     cardiax/solve.py:68-70   step_euler
//   fk_forward_euler  cardiax/solve.py:92-100  _forward_euler
//   fk_forward_euler_tracked  the same, with activation-time maps (no reference counterpart)
//   fk_forward        cardiax/solve.py:168-222 forward (Euler integrator)
//   fk_heun_step      cardiax/solve.py:73-85   step_heun
//   fk_forward_heun   cardiax/solve.py:103-111 _forward_heun
//   fk_forward_euler_flow, fk_forward_flow   _forward_euler / forward through the dataflow
//                     kernel (one cooperative launch per call instead of one per step)
//   fk_forward_euler_tb   _forward_euler with `depth` steps per launch (temporal blocking)
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/cardiax_gb300.h"
#include "fk_capi_internal.h"
#include "fk_ptx.cuh"
#include "fk_adjoint.cuh"
#include "fk_step.cuh"
#include "fk_strip.cuh"
#include "fk_tb.cuh"

namespace fk {

// ---- device error word ---------------------------------------------------------------------
static __device__ int g_status_word;

static std::mutex g_mu;

// ---- current context ------------------------------------------------------------------------
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);
static PfnCtxGetCurrent g_ctx_get_current = nullptr;
static PfnCtxGetId g_ctx_get_id = nullptr;
static std::once_flag g_ctx_once;

uint64_t context_id() {
    std::call_once(g_ctx_once, [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) ==
                cudaSuccess && qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
                cudaSuccess && qb == cudaDriverEntryPointSuccess) {
            g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(a);
            g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(b);
        }
    });
    if (!g_ctx_get_current || !g_ctx_get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return (uint64_t)id;
}

bool context_changed(uint64_t &seen) {
    const uint64_t now = context_id();
    if (now != 0 && now == seen) return false;
    seen = now;
    return true;
}

// The device address of the error word in the current context (looked up again whenever the
// context changes: a cudaDeviceReset invalidates the previous address).
struct CtxAddr {
    uint64_t ctx;
    void *ptr;
};
static CtxAddr g_status_ptr[64];

int *status_ptr() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    CtxAddr &c = g_status_ptr[dev];
    const uint64_t ctx = context_id();
    if (!c.ptr || ctx == 0 || ctx != c.ctx) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_status_word) != cudaSuccess || !p) return nullptr;
        c.ptr = p;
        c.ctx = context_id();  // the lookup created the context if there was none
    }
    return static_cast<int *>(c.ptr);
}

// ---- TMA descriptors ---------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static bool encode_fn() {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_encode) return true;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return false;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return true;
}

int make_plane_map(CUtensorMap *map, const float *plane, int64_t H, int64_t W, int64_t pitch,
                   int box_w, int box_h) {
    if (!encode_fn()) return FK_ERR_TENSORMAP;
    cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
    cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(plane),
                          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FK_OK : FK_ERR_TENSORMAP;
}

// ---- argument preparation ----------------------------------------------------------------
static inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int check_grid(const fk_grid &g) {
    if (g.H < 3 || g.W < 3 || g.pitch < g.W) return FK_ERR_SHAPE;
    if (g.H > (1 << 24) || g.pitch > (1 << 24) || g.H * g.pitch > (int64_t(1) << 34))
        return FK_ERR_SHAPE;
    if (g.pitch % 4 != 0) return FK_ERR_ALIGN;
    return FK_OK;
}

Model make_model(const fk_params &p) {
    Model m{};
    m.V_c = p.V_c;
    m.V_v = p.V_v;
    m.V_csi = p.V_csi;
    m.k = p.k;
    m.r_tau_d = 1.0f / p.tau_d;
    m.r_tau_0 = 1.0f / p.tau_0;
    m.inv_tau_r = 1.0f / p.tau_r;
    m.r_2tau_si = 1.0f / (2.0f * p.tau_si);
    m.r_Cm = 1.0f / p.Cm;
    m.r_tau_v1m = 1.0f / p.tau_v1_minus;
    m.r_tau_v2m = 1.0f / p.tau_v2_minus;
    m.r_tau_vp = 1.0f / p.tau_v_plus;
    m.r_tau_wm = 1.0f / p.tau_w_minus;
    m.r_tau_wp = 1.0f / p.tau_w_plus;
    return m;
}

static_assert(kMaxStim == FK_MAX_ACTIVE_STIMULI, "kernel stimulus slots");

static int convert_stims(const fk_stimulus *s, int n, const fk_grid &g, Stim *out) {
    if (n > 0 && !s) return FK_ERR_NULL;
    for (int k = 0; k < n; ++k) {
        if (!std::isfinite(s[k].start) || !std::isfinite(s[k].duration) ||
            !std::isfinite(s[k].period) || s[k].period == 0.0)
            return FK_ERR_STIMULI;
        Stim &o = out[k];
        o.start = (float)s[k].start;
        o.duration = (float)s[k].duration;
        o.period = (float)s[k].period;
        o.amplitude = s[k].amplitude;
        o.field = s[k].field;
        o.field_plane = 0;
        if (s[k].field) {
            if (!aligned16(s[k].field)) return FK_ERR_ALIGN;
            o.r0 = o.r1 = o.c0 = o.c1 = 0;
        } else {
            o.r0 = s[k].r0 < 0 ? 0 : s[k].r0;
            o.r1 = s[k].r1 > g.H ? (int32_t)g.H : s[k].r1;
            o.c0 = s[k].c0 < 0 ? 0 : s[k].c0;
            o.c1 = s[k].c1 > g.W ? (int32_t)g.W : s[k].c1;
        }
    }
    return FK_OK;
}

int make_stims(const fk_stimulus *s, int n, const fk_grid &g, Stim *out) {
    if (n < 0 || n > kMaxStim) return FK_ERR_STIMULI;
    return convert_stims(s, n, g, out);
}

// The protocol test of the kernels (stim_active in fk_math.cuh), on the host: the same float32
// operations, so the host and the device agree on every step.
static bool stim_active_host(const Stim &s, float t) {
    if (!(t >= s.start)) return false;
    const float a = (s.start - t) + 1.0f;
    float m = std::fmod(a, s.period);
    if (m != 0.0f && ((s.period < 0.0f) != (m < 0.0f))) m += s.period;
    return m < s.duration;
}

int StimList::make(const fk_stimulus *s, int count, const fk_grid &g) {
    if (count < 0 || count > FK_MAX_STIMULI) return FK_ERR_STIMULI;
    n = count;
    return convert_stims(s, count, g, all);
}

int StimList::window(int64_t t0, int64_t t1, Stim *out, int *ns) const {
    int k = 0;
    for (int i = 0; i < n; ++i) {
        bool can = fixed();
        if (!can && t1 - t0 <= 64) {  // short windows: step by step
            for (int64_t t = t0; t < t1 && !can; ++t) can = stim_active_host(all[i], (float)t);
        } else if (!can) {  // long windows: any stimulus that has started by the last step
            can = (float)(t1 - 1) >= all[i].start;
        }
        if (!can) continue;
        if (k == kMaxStim) return FK_ERR_STIMULI;
        out[k++] = all[i];
    }
    *ns = k;
    return FK_OK;
}

// TMA descriptors of the state buffers seen by one call (the ping-pong buffers and checkpoint
// slots): u with its halo box, v and w with the plain tile box, and u with the tile box (for
// the stores of a step that writes this buffer).
struct MapCache {
    static constexpr int kSlots = 4;
    const float *ptr[kSlots] = {nullptr, nullptr, nullptr, nullptr};
    CUtensorMap u[kSlots], v[kSlots], w[kSlots], ut[kSlots], us[kSlots];
    int next = 0;
    const float *dptr = nullptr;  // D plane of `ds`
    CUtensorMap ds;               // D with the strip kernel's box
    // slot of `state`, building its maps if needed without evicting slot `keep`
    int lookup(const fk_grid &g, const float *state, int keep, int *slot) {
        for (int i = 0; i < kSlots; ++i)
            if (ptr[i] == state) {
                *slot = i;
                return FK_OK;
            }
        int k = next;
        if (k == keep) k = (k + 1) % kSlots;
        next = (k + 1) % kSlots;
        const int64_t plane = g.H * g.pitch;
        int rc;
        ptr[k] = nullptr;
        if ((rc = make_plane_map(&u[k], state + 2 * plane, g.H, g.W, g.pitch, SW, SU_H)) ||
            (rc = make_plane_map(&v[k], state, g.H, g.W, g.pitch, TX, TY)) ||
            (rc = make_plane_map(&w[k], state + plane, g.H, g.W, g.pitch, TX, TY)) ||
            (rc = make_plane_map(&ut[k], state + 2 * plane, g.H, g.W, g.pitch, TX, TY)) ||
            (rc = make_plane_map(&us[k], state + 2 * plane, g.H, g.W, g.pitch, S_SW, S_UH)))
            return rc;
        ptr[k] = state;
        *slot = k;
        return FK_OK;
    }
    // maps of a step reading `in` and writing `out`
    int get(const fk_grid &g, const float *in, const float *out, StepMaps &sm) {
        int ki, ko, rc;
        if ((rc = lookup(g, in, -1, &ki)) || (rc = lookup(g, out, ki, &ko))) return rc;
        sm.u = u[ki];
        sm.ov = v[ko];
        sm.ow = w[ko];
        sm.ou = ut[ko];
        return FK_OK;
    }
    // maps of a strip-kernel step reading `in` with diffusivity `D`
    int get_strip(const fk_grid &g, const float *in, const float *D, StripMaps &sm) {
        int ki, rc;
        if ((rc = lookup(g, in, -1, &ki))) return rc;
        if (dptr != D) {
            dptr = nullptr;
            if ((rc = make_plane_map(&ds, D, g.H, g.W, g.pitch, S_SW, S_DH))) return rc;
            dptr = D;
        }
        sm.u = us[ki];
        sm.d = ds;
        return FK_OK;
    }
};

// Which kernel takes an Euler step: 0 = the tiled kernel (fk_step_kernel, default), 1 = the
// strip kernel wherever it applies.  Set through fk_select_step_kernel.
static int g_step_kernel = 0;

// One step from `in` to `out` (Euler, or the derivative with `deriv`).
// heun: 0 = an Euler step (or the derivative); 1, 2 = the Heun stages (StepArgs: dso, x0, d1, h).
int step_once(const fk_grid &g, const float *in, float *out, const float *D, const Model &m,
              const Stim *st, int ns, int64_t t, float dt, float rdx, bool deriv,
              const CUtensorMap &tm_d, MapCache &maps, int *status, cudaStream_t stream,
              const fk_activation *act = nullptr, int heun = 0, float *dso = nullptr,
              const float *x0 = nullptr, const float *d1 = nullptr, float h = 0.0f) {
    const int64_t plane = g.H * g.pitch;
    StepMaps sm;
    int rc = maps.get(g, in, out, sm);
    if (rc) return rc;
    sm.d = tm_d;
    StepArgs a{};
    a.v = in;
    a.w = in + plane;
    a.u = in + 2 * plane;
    a.D = D;
    a.vo = out;
    a.wo = out + plane;
    a.uo = out + 2 * plane;
    a.H = (int)g.H;
    a.W = (int)g.W;
    a.pitch = (int)g.pitch;
    a.t = (float)t;
    a.dt = dt;
    a.rdx = rdx;
    a.n_stim = ns;
    a.m = m;
    for (int k = 0; k < ns; ++k) a.stim[k] = st[k];
    a.status = status;
    a.l2_hints = l2_fits_step(g.H, g.pitch) ? 1 : 0;
    if (act && !deriv) {
        a.act_first = act->first;
        a.act_last = act->last;
        a.act_count = act->count;
        a.act_threshold = act->threshold;
    }
    a.dso = dso;
    a.x0 = x0;
    a.d1 = d1;
    a.h = h;
    cudaError_t e;
    if (heun) {
        e = launch_step(sm, a, false, stream, heun);
    } else if (!deriv && g_step_kernel == 1 && strip_eligible(g.H, g.W)) {
        StripMaps xm;
        if ((rc = maps.get_strip(g, in, D, xm))) return rc;
        e = launch_strip(xm, a, stream);
    } else {
        e = launch_step(sm, a, deriv, stream);
    }
    return e == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

// ---- dataflow stepping ------------------------------------------------------------------------
static void fill_args(StepArgs &a, const fk_grid &g, const float *in, const float *D,
                      const Model &m, const Stim *st, int ns, float dt, float rdx, int *status,
                      const fk_activation *act) {
    const int64_t plane = g.H * g.pitch;
    a = StepArgs{};
    a.v = in;
    a.w = in + plane;
    a.u = in + 2 * plane;
    a.D = D;
    a.H = (int)g.H;
    a.W = (int)g.W;
    a.pitch = (int)g.pitch;
    a.dt = dt;
    a.rdx = rdx;
    a.n_stim = ns;
    a.m = m;
    for (int k = 0; k < ns; ++k) a.stim[k] = st[k];
    a.status = status;
    if (act) {
        a.act_first = act->first;
        a.act_last = act->last;
        a.act_count = act->count;
        a.act_threshold = act->threshold;
    }
}

// Steps t0 .. t0+n-1 from `src` so that the last one lands in `dst` (src == dst allowed);
// `scratch` is distinct from both.  Launches of at most 2^30 steps (the flags count steps in
// int32).
int flow_run(const fk_grid &g, const float *src, float *dst, float *scratch, const float *D,
             const CUtensorMap &tm_d, const Model &m, const Stim *st, int ns, int64_t t0,
             int64_t n, float dt, float rdx, const fk_activation *act, int32_t *flags,
             int *status, cudaStream_t stream) {
    const int64_t n_state = 3 * g.H * g.pitch;
    if (n == 0) {
        if (src != dst && cudaMemcpyAsync(dst, src, sizeof(float) * n_state,
                                          cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
            return FK_ERR_CUDA;
        return FK_OK;
    }
    const int64_t words = flow_flag_words(g.H, g.W);
    const int64_t cap = (int64_t)1 << 30;
    const float *cur = src;
    for (int64_t done = 0; done < n;) {
        const int64_t c = n - done < cap ? n - done : cap;  // cap is even
        // step k writes bufs[k & 1]; the last writes bufs[(c-1) & 1]
        float *bufs[2];
        bool copy_back = false;
        if (cur != dst) {
            bufs[(c - 1) & 1] = dst;
            bufs[c & 1] = scratch;
        } else {  // in place: step 0 must not write its own input
            bufs[0] = scratch;
            bufs[1] = dst;
            copy_back = (c & 1) != 0;
        }
        FlowMaps fm;
        fm.d = tm_d;
        FlowArgs fa;
        const float *ins[3] = {cur, bufs[0], bufs[1]};
        int rc;
        for (int k = 0; k < 3; ++k) {
            if ((rc = make_plane_map(&fm.uin[k], ins[k] + 2 * g.H * g.pitch, g.H, g.W, g.pitch,
                                     SW, SU_H)))
                return rc;
            fill_args(fa.in[k], g, ins[k], D, m, st, ns, dt, rdx, status, act);
        }
        for (int b = 0; b < 2; ++b) {
            const int64_t plane = g.H * g.pitch;
            if ((rc = make_plane_map(&fm.ov[b], bufs[b], g.H, g.W, g.pitch, TX, TY)) ||
                (rc = make_plane_map(&fm.ow[b], bufs[b] + plane, g.H, g.W, g.pitch, TX, TY)) ||
                (rc = make_plane_map(&fm.ou[b], bufs[b] + 2 * plane, g.H, g.W, g.pitch, TX, TY)))
                return rc;
        }
        fa.t0 = t0 + done;
        fa.nsteps = (int)c;
        fa.flags = flags;
        if (cudaMemsetAsync(flags, 0, sizeof(int32_t) * words, stream) != cudaSuccess)
            return FK_ERR_CUDA;
        if (launch_flow(fm, fa, act != nullptr, stream) != cudaSuccess) return FK_ERR_CUDA;
        if (copy_back && cudaMemcpyAsync(dst, scratch, sizeof(float) * n_state,
                                         cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
            return FK_ERR_CUDA;
        done += c;
        cur = dst;
    }
    return FK_OK;
}

__global__ void add_state_kernel(float *dst, const float *src, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] += src[i];
}

__global__ void fill_state_kernel(float *s, int64_t plane) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < 3 * plane; i += stride) s[i] = i < 2 * plane ? 1.0f : 0.0f;
}

}  // namespace fk

using namespace fk;

// ---- exported entry points ---------------------------------------------------------------
extern "C" {

const char *fk_status_string(int s) {
    switch (s) {
        case FK_OK: return "ok";
        case FK_ERR_NULL: return "null pointer";
        case FK_ERR_SHAPE: return "invalid grid shape (need H, W >= 3 and pitch >= W)";
        case FK_ERR_ALIGN: return "misaligned buffer (need pitch % 4 == 0 and 16-byte aligned pointers)";
        case FK_ERR_STIMULI: return "invalid stimuli (too many, or a non-finite or zero-period protocol)";
        case FK_ERR_ARGUMENT: return "invalid argument";
        case FK_ERR_CUDA: return "CUDA error";
        case FK_ERR_TENSORMAP: return "TMA descriptor encoding failed";
        case FK_ERR_DEVICE: return "device-side barrier timeout";
        case FK_ERR_CAPACITY:
            return "grid larger than the static scratch of fk_forward_euler_noalloc "
                   "(H * pitch must be <= FK_NOALLOC_MAX_CELLS = 512 * 512)";
        default: return "unknown status";
    }
}

int fk_select_step_kernel(int which) {
    if (which != 0 && which != 1) return FK_ERR_ARGUMENT;
    g_step_kernel = which;
    return FK_OK;
}

int fk_device_status(int reset, int *value) {
    int *p = status_ptr();
    if (!p || !value) return !value ? FK_ERR_NULL : FK_ERR_CUDA;
    if (cudaMemcpy(value, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return FK_ERR_CUDA;
    if (reset && cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return FK_ERR_CUDA;
    return FK_OK;
}

namespace fk {
namespace {
// One warp whose thread 0 waits on an mbarrier that nothing arrives on: the bounded wait of the
// step kernels runs out after `limit_ns` and the kernel reports it as they do.
__global__ void selftest_wait_kernel(uint64_t limit_ns, int *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_barrier_init();
    if (!mbar_wait_bounded(&bar, 0, limit_ns)) atomicOr(status, kStatusTimeout);
}
}  // namespace
}  // namespace fk

int fk_selftest_wait_timeout(int64_t limit_ns, void *stream) {
    if (limit_ns < 1000 || limit_ns > 2000000000ll) return FK_ERR_ARGUMENT;
    int *st = fk::status_ptr();
    if (!st) return FK_ERR_CUDA;
    fk::selftest_wait_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((uint64_t)limit_ns, st);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

int fk_init(fk_grid g, float *state, void *stream) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!state) return FK_ERR_NULL;
    fill_state_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(state, g.H * g.pitch);
    return cudaGetLastError() == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

static int common_checks(const fk_grid &g, const void *a, const void *b, const float *D,
                         const fk_params *p, double dx) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!a || !b || !D || !p) return FK_ERR_NULL;
    if (!aligned16(a) || !aligned16(b) || !aligned16(D)) return FK_ERR_ALIGN;
    if (!(dx > 0.0) || !std::isfinite(dx)) return FK_ERR_ARGUMENT;
    return FK_OK;
}

int fk_step(fk_grid g, const float *state, const float *D, const fk_params *p,
            const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dx, float *dstate,
            void *stream) {
    int rc = common_checks(g, state, dstate, D, p, dx);
    if (rc) return rc;
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t, t + 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    MapCache maps;
    return step_once(g, state, dstate, D, make_model(*p), st, ns, t, 0.0f,
                     1.0f / (float)dx, true, tm_d, maps, status, (cudaStream_t)stream);
}

int fk_euler_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                  const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                  float *state_out, void *stream) {
    int rc = common_checks(g, state, state_out, D, p, dx);
    if (rc) return rc;
    if (!std::isfinite(dt)) return FK_ERR_ARGUMENT;
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t, t + 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    MapCache maps;
    return step_once(g, state, state_out, D, make_model(*p), st, ns, t, (float)dt,
                     1.0f / (float)dx, false, tm_d, maps, status, (cudaStream_t)stream);
}

int fk_forward_euler_tracked(fk_grid g, float *state, float *scratch, const float *D,
                             const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
                             int64_t t0, int64_t t1, double dt, double dx,
                             const fk_activation *act, void *stream) {
    int rc = common_checks(g, state, scratch, D, p, dx);
    if (rc) return rc;
    if (t1 < t0 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    if (act) {
        if (!act->first || !act->last || !act->count) return FK_ERR_NULL;
        if (!std::isfinite(act->threshold)) return FK_ERR_ARGUMENT;
    }
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t0, t0 + 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const float rdx = 1.0f / (float)dx;
    cudaStream_t s = (cudaStream_t)stream;
    float *bufs[2] = {state, scratch};
    MapCache maps;
    for (int64_t t = t0; t < t1; ++t) {
        const int k = (int)((t - t0) & 1);
        if (!L.fixed() && (rc = L.window(t, t + 1, st, &ns))) return rc;
        rc = step_once(g, bufs[k], bufs[k ^ 1], D, m, st, ns, t, (float)dt, rdx, false,
                       tm_d, maps, status, s, act);
        if (rc) return rc;
    }
    if ((t1 - t0) & 1) {
        // odd number of steps: the result sits in scratch
        if (cudaMemcpyAsync(state, scratch, sizeof(float) * 3 * g.H * g.pitch,
                            cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return FK_ERR_CUDA;
    }
    return FK_OK;
}

int64_t fk_flow_flag_words(fk_grid g) {
    if (check_grid(g)) return -1;
    return flow_flag_words(g.H, g.W);
}

int fk_forward_euler_flow(fk_grid g, const float *src, float *dst, float *scratch,
                          const float *D, const fk_params *p, const fk_stimulus *stimuli,
                          int n_stimuli, int64_t t0, int64_t t1, double dt, double dx,
                          const fk_activation *act, int32_t *flags, int64_t n_flags,
                          void *stream) {
    int rc = common_checks(g, src, scratch, D, p, dx);
    if (rc) return rc;
    if (!dst || !flags) return FK_ERR_NULL;
    if (!aligned16(dst)) return FK_ERR_ALIGN;
    if (t1 < t0 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    if (scratch == src || scratch == dst) return FK_ERR_ARGUMENT;
    if (n_flags < flow_flag_words(g.H, g.W)) return FK_ERR_ARGUMENT;
    if (act) {
        if (!act->first || !act->last || !act->count) return FK_ERR_NULL;
        if (!std::isfinite(act->threshold)) return FK_ERR_ARGUMENT;
    }
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t0, t1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    return flow_run(g, src, dst, scratch, D, tm_d, make_model(*p), st, ns, t0, t1 - t0,
                    (float)dt, 1.0f / (float)dx, act, flags, status, (cudaStream_t)stream);
}

int fk_forward_flow(fk_grid g, const float *state0, float *scratch, const float *D,
                    const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
                    const int64_t *checkpoints, int n_checkpoints, double dt, double dx,
                    float *out, int32_t *flags, int64_t n_flags, void *stream) {
    int rc = common_checks(g, state0, scratch, D, p, dx);
    if (rc) return rc;
    if (!out || !checkpoints || !flags) return FK_ERR_NULL;
    if (!aligned16(out)) return FK_ERR_ALIGN;
    if (n_checkpoints < 1 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    if (n_flags < flow_flag_words(g.H, g.W)) return FK_ERR_ARGUMENT;
    for (int i = 0; i + 1 < n_checkpoints; ++i)
        if (checkpoints[i + 1] < checkpoints[i]) return FK_ERR_ARGUMENT;
    StimList L;
    if ((rc = L.make(stimuli, n_stimuli, g))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const int64_t n_state = 3 * g.H * g.pitch;
    const float *cur = state0;
    for (int i = 0; i + 1 < n_checkpoints; ++i) {
        float *dst = out + (int64_t)i * n_state;
        if (dst == scratch || cur == scratch) return FK_ERR_ARGUMENT;
        Stim st[kMaxStim];
        int ns = 0;
        if ((rc = L.window(checkpoints[i], checkpoints[i + 1], st, &ns))) return rc;
        if ((rc = flow_run(g, cur, dst, scratch, D, tm_d, m, st, ns, checkpoints[i],
                           checkpoints[i + 1] - checkpoints[i], (float)dt, 1.0f / (float)dx,
                           nullptr, flags, status, (cudaStream_t)stream)))
            return rc;
        cur = dst;
    }
    return FK_OK;
}

int fk_forward_euler_tb(fk_grid g, float *state, float *scratch, const float *D,
                        const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, int64_t t0,
                        int64_t t1, double dt, double dx, int depth, void *stream) {
    int rc = common_checks(g, state, scratch, D, p, dx);
    if (rc) return rc;
    if (t1 < t0 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    if (depth != 1 && depth != 2 && depth != 4 && depth != 8) return FK_ERR_ARGUMENT;
    int bw = 0, bh = 0, ow = 0, oh = 0;
    tb_box(depth, &bw, &bh, &ow, &oh);
    // one-cell last tile row/column: the one-sided rows reach beyond the blocked halo
    if (depth == 1 || g.H % oh == 1 || g.W % ow == 1)
        return fk_forward_euler(g, state, scratch, D, p, stimuli, n_stimuli, t0, t1, dt, dx,
                                stream);
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t0, t0 + 1, st, &ns))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const float rdx = 1.0f / (float)dx;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t plane = g.H * g.pitch;
    float *bufs[2] = {state, scratch};
    TbMaps tm[2];  // tm[k]: reads bufs[k], writes bufs[k^1]
    CUtensorMap dmap;
    if ((rc = make_plane_map(&dmap, D, g.H, g.W, g.pitch, bw, bh))) return rc;
    for (int k = 0; k < 2; ++k) {
        const float *in = bufs[k];
        float *out = bufs[k ^ 1];
        tm[k].d = dmap;
        if ((rc = make_plane_map(&tm[k].v, in, g.H, g.W, g.pitch, bw, bh)) ||
            (rc = make_plane_map(&tm[k].w, in + plane, g.H, g.W, g.pitch, bw, bh)) ||
            (rc = make_plane_map(&tm[k].u, in + 2 * plane, g.H, g.W, g.pitch, bw, bh)) ||
            (rc = make_plane_map(&tm[k].ov, out, g.H, g.W, g.pitch, ow, oh)) ||
            (rc = make_plane_map(&tm[k].ow, out + plane, g.H, g.W, g.pitch, ow, oh)) ||
            (rc = make_plane_map(&tm[k].ou, out + 2 * plane, g.H, g.W, g.pitch, ow, oh)))
            return rc;
    }
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    MapCache maps;
    int cur = 0;
    int64_t t = t0;
    for (; t + depth <= t1; t += depth) {
        StepArgs a;
        if (!L.fixed() && (rc = L.window(t, t + depth, st, &ns))) return rc;
        fill_args(a, g, bufs[cur], D, m, st, ns, (float)dt, rdx, status, nullptr);
        if (launch_tb(depth, tm[cur], a, t, s) != cudaSuccess) return FK_ERR_CUDA;
        cur ^= 1;
    }
    for (; t < t1; ++t) {  // the remainder, one step per launch
        if (!L.fixed() && (rc = L.window(t, t + 1, st, &ns))) return rc;
        if ((rc = step_once(g, bufs[cur], bufs[cur ^ 1], D, m, st, ns, t, (float)dt, rdx,
                            false, tm_d, maps, status, s)))
            return rc;
        cur ^= 1;
    }
    if (cur == 1 && cudaMemcpyAsync(state, scratch, sizeof(float) * 3 * plane,
                                    cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return FK_ERR_CUDA;
    return FK_OK;
}

int fk_forward_euler(fk_grid g, float *state, float *scratch, const float *D, const fk_params *p,
                     const fk_stimulus *stimuli, int n_stimuli, int64_t t0, int64_t t1,
                     double dt, double dx, void *stream) {
    return fk_forward_euler_tracked(g, state, scratch, D, p, stimuli, n_stimuli, t0, t1, dt, dx,
                                    nullptr, stream);
}

// One Heun step from `in` to `out` with work = [d1, x1, ...]: two launches of the step kernel.
// Stage 1 is the Euler step x1 = x + dt d1 that also stores d1 = f(x, t); stage 2 evaluates
// f(x1, t) and writes x + (d1 + f(x1, t)) dt/2 -- per cell the operations of the derivative,
// x1 = fmaf(d1, dt, x) and fmaf(d1 + d2, dt/2, x) of cardiax/solve.py:73-85.
static int heun_once(const fk_grid &g, const float *in, float *out, float *work, const float *D,
                     const Model &m, const Stim *st, int ns, int64_t t, float dt, float rdx,
                     const CUtensorMap &tm_d, MapCache &maps, int *status, cudaStream_t s) {
    const int64_t n = 3 * g.H * g.pitch;
    float *d1 = work, *x1 = work + n;
    int rc = step_once(g, in, x1, D, m, st, ns, t, dt, rdx, false, tm_d, maps, status, s, nullptr,
                       1, d1);
    if (rc) return rc;
    return step_once(g, x1, out, D, m, st, ns, t, dt, rdx, false, tm_d, maps, status, s, nullptr, 2,
                     nullptr, in, d1, dt * 0.5f);
}

int fk_heun_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                 const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                 float *state_out, float *work, void *stream) {
    int rc = common_checks(g, state, state_out, D, p, dx);
    if (rc) return rc;
    if (!work) return FK_ERR_NULL;
    if (!aligned16(work)) return FK_ERR_ALIGN;
    if (!std::isfinite(dt)) return FK_ERR_ARGUMENT;
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t, t + 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    MapCache maps;
    return heun_once(g, state, state_out, work, D, make_model(*p), st, ns, t, (float)dt,
                     1.0f / (float)dx, tm_d, maps, status, (cudaStream_t)stream);
}

int fk_forward_heun(fk_grid g, float *state, float *work, const float *D, const fk_params *p,
                    const fk_stimulus *stimuli, int n_stimuli, int64_t t0, int64_t t1, double dt,
                    double dx, void *stream) {
    int rc = common_checks(g, state, work, D, p, dx);
    if (rc) return rc;
    if (t1 < t0 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(t0, t0 + 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const float rdx = 1.0f / (float)dx;
    const int64_t n = 3 * g.H * g.pitch;
    cudaStream_t s = (cudaStream_t)stream;
    float *other = work + 3 * n;  // the 4th work buffer is the ping-pong state
    float *bufs[2] = {state, other};
    MapCache maps;
    for (int64_t t = t0; t < t1; ++t) {
        const int k = (int)((t - t0) & 1);
        if (!L.fixed() && (rc = L.window(t, t + 1, st, &ns))) return rc;
        if ((rc = heun_once(g, bufs[k], bufs[k ^ 1], work, D, m, st, ns, t, (float)dt, rdx,
                            tm_d, maps, status, s)))
            return rc;
    }
    if (((t1 - t0) & 1) &&
        cudaMemcpyAsync(state, other, sizeof(float) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return FK_ERR_CUDA;
    return FK_OK;
}

int fk_forward(fk_grid g, const float *state0, float *scratch, const float *D,
               const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
               const int64_t *checkpoints, int n_checkpoints, double dt, double dx, float *out,
               void *stream) {
    int rc = common_checks(g, state0, scratch, D, p, dx);
    if (rc) return rc;
    if (!out || !checkpoints) return FK_ERR_NULL;
    if (!aligned16(out)) return FK_ERR_ALIGN;
    if (n_checkpoints < 1 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    for (int i = 0; i + 1 < n_checkpoints; ++i)
        if (checkpoints[i + 1] < checkpoints[i]) return FK_ERR_ARGUMENT;
    StimList L;
    Stim st[kMaxStim];
    int ns = 0;
    if ((rc = L.make(stimuli, n_stimuli, g)) || (rc = L.window(0, 1, st, &ns))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const float rdx = 1.0f / (float)dx;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n_state = 3 * g.H * g.pitch;
    const float *cur = state0;
    MapCache maps;
    for (int i = 0; i + 1 < n_checkpoints; ++i) {
        float *dst = out + (int64_t)i * n_state;
        const int64_t a = checkpoints[i], b = checkpoints[i + 1], n = b - a;
        if (n == 0) {
            if (cudaMemcpyAsync(dst, cur, sizeof(float) * n_state, cudaMemcpyDeviceToDevice, s) !=
                cudaSuccess)
                return FK_ERR_CUDA;
        }
        // ping-pong so that the interval's last step lands in dst
        for (int64_t k = 0; k < n; ++k) {
            float *o = ((n - 1 - k) & 1) ? scratch : dst;
            if (!L.fixed() && (rc = L.window(a + k, a + k + 1, st, &ns))) return rc;
            rc = step_once(g, cur, o, D, m, st, ns, a + k, (float)dt, rdx, false, tm_d,
                           maps, status, s);
            if (rc) return rc;
            cur = o;
        }
        cur = dst;
    }
    return FK_OK;
}

int64_t fk_adjoint_slots(fk_grid g) {
    if (check_grid(g)) return 0;
    return adjoint_slots((int)g.H, (int)g.W);
}

int fk_adjoint_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                    const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                    const float *lam_next, float *lam, float *grad_D, double *grad_theta_slots,
                    void *stream) {
    int rc = common_checks(g, state, lam, D, p, dx);
    if (rc) return rc;
    if (!lam_next) return FK_ERR_NULL;
    if (!aligned16(lam_next) || (grad_D && !aligned16(grad_D))) return FK_ERR_ALIGN;
    if (!std::isfinite(dt)) return FK_ERR_ARGUMENT;
    AdjointArgs a{};
    if ((rc = make_stims(stimuli, n_stimuli, g, a.stim))) return rc;
    const int64_t plane = g.H * g.pitch;
    a.v = state;
    a.w = state + plane;
    a.u = state + 2 * plane;
    a.D = D;
    a.lv = lam_next;
    a.lw = lam_next + plane;
    a.lu = lam_next + 2 * plane;
    a.olv = lam;
    a.olw = lam + plane;
    a.olu = lam + 2 * plane;
    a.gD = grad_D;
    a.gtheta = grad_theta_slots;
    a.H = (int)g.H;
    a.W = (int)g.W;
    a.pitch = (int)g.pitch;
    a.t = (float)t;
    a.dt = (float)dt;
    a.rdx = 1.0f / (float)dx;
    a.n_stim = n_stimuli;
    a.m = make_model(*p);
    return launch_adjoint(a, (cudaStream_t)stream) == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

size_t fk_adjoint_batch_workspace_bytes(int n_exp) {
    if (n_exp <= 0) return 0;
    return ((size_t)n_exp * sizeof(AdjointArgs) + 255) / 256 * 256;
}

int fk_adjoint_batch_range(int n_exp, fk_grid g, const float *bufs, int64_t exp_stride, int64_t s,
                           int64_t n, const float *D, const fk_params *p,
                           const fk_stimulus *const *stimuli, const int *n_stimuli, double dt,
                           double dx, float *lam, float *lam_tmp, const int64_t *inj_steps,
                           const float *const *inj_grads, int n_inj, float *grad_D,
                           double *grad_theta_slots, void *workspace, size_t workspace_bytes,
                           void *stream) {
    int rc = common_checks(g, bufs, lam, D, p, dx);
    if (rc) return rc;
    if (!lam_tmp || !workspace || !stimuli || !n_stimuli ||
        (n_inj > 0 && (!inj_steps || !inj_grads)))
        return FK_ERR_NULL;
    if (n_exp < 1 || n_exp > 65535 || n < 1 || n_inj < 0 || !std::isfinite(dt))
        return FK_ERR_ARGUMENT;
    const int64_t plane = g.H * g.pitch, ns = 3 * plane;
    if (exp_stride < n * ns || (exp_stride & 3) || !aligned16(lam_tmp) || !aligned16(workspace) ||
        (grad_D && !aligned16(grad_D)))
        return FK_ERR_ALIGN;
    if (workspace_bytes < fk_adjoint_batch_workspace_bytes(n_exp)) return FK_ERR_ARGUMENT;
    const int64_t slots = adjoint_slots((int)g.H, (int)g.W);
    std::vector<AdjointArgs> h((size_t)n_exp);
    const Model m = make_model(*p);
    for (int e = 0; e < n_exp; ++e) {
        AdjointArgs &a = h[e];
        a = AdjointArgs{};
        if ((rc = make_stims(stimuli[e], n_stimuli[e], g, a.stim))) return rc;
        const float *x = bufs + e * exp_stride;
        float *la = lam + e * ns, *lb = lam_tmp + e * ns;
        a.v = x;
        a.w = x + plane;
        a.u = x + 2 * plane;
        a.D = D;
        a.lv = la;
        a.lw = la + plane;
        a.lu = la + 2 * plane;
        a.olv = lb;
        a.olw = lb + plane;
        a.olu = lb + 2 * plane;
        a.gD = grad_D ? grad_D + e * plane : nullptr;
        a.gtheta = grad_theta_slots ? grad_theta_slots + e * slots * kAdjParamStride : nullptr;
        a.H = (int)g.H;
        a.W = (int)g.W;
        a.pitch = (int)g.pitch;
        a.dt = (float)dt;
        a.rdx = 1.0f / (float)dx;
        a.n_stim = n_stimuli[e];
        a.m = m;
    }
    cudaStream_t cs = (cudaStream_t)stream;
    AdjointArgs *dexp = static_cast<AdjointArgs *>(workspace);
    if (cudaMemcpyAsync(dexp, h.data(), sizeof(AdjointArgs) * h.size(), cudaMemcpyHostToDevice,
                        cs) != cudaSuccess)
        return FK_ERR_CUDA;
    // reverse step r (k = n-1-r) reads buffer r&1 (0: lam, 1: lam_tmp) and writes the other
    for (int64_t k = n - 1, r = 0; k >= 0; --k, ++r) {
        if (launch_adjoint_batch(dexp, n_exp, (int)g.H, (int)g.W, ns, (int)k, (int)(r & 1),
                                 (float)(s + k), cs) != cudaSuccess)
            return FK_ERR_CUDA;
        float *cur = (r & 1) ? lam : lam_tmp;
        for (int j = 0; j < n_inj; ++j)
            if (inj_steps[j] == s + k) {
                add_state_kernel<<<1024, 256, 0, cs>>>(cur, inj_grads[j], n_exp * ns);
                if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
            }
    }
    if (((n - 1) & 1) == 0 &&  // the last step wrote lam_tmp
        cudaMemcpyAsync(lam, lam_tmp, sizeof(float) * n_exp * ns, cudaMemcpyDeviceToDevice, cs) !=
            cudaSuccess)
        return FK_ERR_CUDA;
    return FK_OK;
}

int fk_recompute(fk_grid g, const float *state, int64_t s, int64_t n, const float *D,
                 const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, double dt,
                 double dx, float *buf, void *stream) {
    int rc = common_checks(g, state, buf, D, p, dx);
    if (rc) return rc;
    if (n < 1 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    Stim st[kMaxStim];
    if ((rc = make_stims(stimuli, n_stimuli, g, st))) return rc;
    CUtensorMap tm_d;
    if ((rc = make_plane_map(&tm_d, D, g.H, g.W, g.pitch, SW, SD_H))) return rc;
    int *status = status_ptr();
    if (!status) return FK_ERR_CUDA;
    const Model m = make_model(*p);
    const float rdx = 1.0f / (float)dx;
    const int64_t ns = 3 * g.H * g.pitch;
    cudaStream_t cs = (cudaStream_t)stream;
    if (cudaMemcpyAsync(buf, state, sizeof(float) * ns, cudaMemcpyDeviceToDevice, cs) != cudaSuccess)
        return FK_ERR_CUDA;
    MapCache maps;
    for (int64_t k = 1; k < n; ++k) {
        rc = step_once(g, buf + (k - 1) * ns, buf + k * ns, D, m, st, n_stimuli, s + k - 1, (float)dt,
                       rdx, false, tm_d, maps, status, cs);
        if (rc) return rc;
    }
    return FK_OK;
}

int fk_adjoint_range(fk_grid g, const float *buf, int64_t s, int64_t n, const float *D,
                     const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, double dt,
                     double dx, float *lam, float *lam_tmp, const int64_t *inj_steps,
                     const float *const *inj_grads, int n_inj, float *grad_D,
                     double *grad_theta_slots, void *stream) {
    int rc = common_checks(g, buf, lam, D, p, dx);
    if (rc) return rc;
    if (!lam_tmp || (n_inj > 0 && (!inj_steps || !inj_grads))) return FK_ERR_NULL;
    if (n < 1 || n_inj < 0 || !std::isfinite(dt)) return FK_ERR_ARGUMENT;
    const int64_t ns = 3 * g.H * g.pitch;
    cudaStream_t cs = (cudaStream_t)stream;
    float *cur = lam, *other = lam_tmp;
    for (int64_t k = n - 1; k >= 0; --k) {
        rc = fk_adjoint_step(g, buf + k * ns, D, p, stimuli, n_stimuli, s + k, dt, dx, cur, other,
                             grad_D, grad_theta_slots, stream);
        if (rc) return rc;
        float *tmp = cur;
        cur = other;
        other = tmp;
        for (int j = 0; j < n_inj; ++j)
            if (inj_steps[j] == s + k) {
                add_state_kernel<<<1024, 256, 0, cs>>>(cur, inj_grads[j], ns);
                if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
            }
    }
    if (cur != lam &&
        cudaMemcpyAsync(lam, cur, sizeof(float) * ns, cudaMemcpyDeviceToDevice, cs) != cudaSuccess)
        return FK_ERR_CUDA;
    return FK_OK;
}

}  // extern "C"
