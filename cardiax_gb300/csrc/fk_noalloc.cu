// fk_forward_euler_noalloc: fk_forward_euler for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not available -- for example
// an XLA custom call (the reference is a JAX code base), which receives its operands and
// results from XLA's allocator and must not allocate inside the call, or a host runtime with a
// fixed, pre-reserved device memory budget.  Such a caller still owns the state and D buffers;
// only the ping-pong scratch state that fk_forward_euler otherwise takes as an argument comes
// from a file-scope device array of this library.
//
// Limits and sharing:
// * The array holds one state of at most FK_NOALLOC_MAX_CELLS cells (H * pitch <= 512 * 512,
//   3 MiB); larger grids are rejected with FK_ERR_CAPACITY.  Every GPU that loads the library
//   reserves these 3 MiB until the process exits.
// * All calls on a device share the one array.  Calls whose GPU work overlaps (different
//   streams, or different host threads without ordering) race on it; serialise them.
// * Nothing in it needs clearing between calls: every step writes every in-grid cell
//   (columns < W) of the scratch state before any step reads it.  The row padding (columns
//   W .. pitch-1) is never computed; so that a previous call's padding -- possibly another
//   caller's grid -- cannot reach this caller's state, the call first copies the state's own
//   padding columns into the array (a strided device-to-device copy on `stream`), and the
//   state's padding therefore comes out as it went in, whatever the step count.
// * The device address of the array is looked up (cudaGetSymbolAddress) on the first call on
//   each device, with that device current, and again whenever the device's CUDA context has
//   changed since (after a cudaDeviceReset the old address is dead).  Make the first call on a
//   device, and the first call after a context change, before any stream capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/cardiax_gb300.h"
#include "fk_capi_internal.h"

namespace {

constexpr int64_t kMaxCells = FK_NOALLOC_MAX_CELLS;

static __device__ __align__(256) float g_noalloc_scratch[3 * kMaxCells];

std::mutex g_mu;
struct Cached {
    uint64_t ctx;  // id of the context the address belongs to
    float *ptr;
};
Cached g_scratch[64] = {};

// Device address of the scratch array in the current context of the current device.
int scratch_for_current_device(float **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FK_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    Cached &c = g_scratch[dev];
    const uint64_t ctx = fk::context_id();
    if (!c.ptr || ctx == 0 || ctx != c.ctx) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FK_ERR_CUDA;
        c.ptr = static_cast<float *>(p);
        c.ctx = fk::context_id();  // the lookup created the context if there was none
    }
    *out = c.ptr;
    return FK_OK;
}

}  // namespace

extern "C" int fk_forward_euler_noalloc(fk_grid g, float *state, const float *D,
                                        const fk_params *p, const fk_stimulus *stimuli,
                                        int n_stimuli, int64_t t0, int64_t t1, double dt,
                                        double dx, void *stream) {
    int rc = fk::check_grid(g);
    if (rc) return rc;
    if (g.H * g.pitch > kMaxCells) return FK_ERR_CAPACITY;
    if (!state) return FK_ERR_NULL;
    float *scratch = nullptr;
    if ((rc = scratch_for_current_device(&scratch))) return rc;
    if (g.pitch > g.W && t1 > t0) {
        // the state's padding columns of all three planes (3H rows of pitch floats) go into the
        // array first, so that the final copy-back of an odd step count returns them unchanged
        const size_t row = (size_t)g.pitch * sizeof(float);
        if (cudaMemcpy2DAsync(scratch + g.W, row, state + g.W, row,
                              (size_t)(g.pitch - g.W) * sizeof(float), (size_t)(3 * g.H),
                              cudaMemcpyDeviceToDevice, (cudaStream_t)stream) != cudaSuccess)
            return FK_ERR_CUDA;
    }
    return fk_forward_euler(g, state, scratch, D, p, stimuli, n_stimuli, t0, t1, dt, dx, stream);
}
