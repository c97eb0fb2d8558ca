// Helpers shared by the C-ABI translation units (not part of the public ABI).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cardiax_gb300.h"
#include "fk_math.cuh"

namespace fk {

int *status_ptr();
// Unique id of the calling thread's current CUDA context (cuCtxGetId), 0 when there is none
// yet or the driver cannot tell.  Ids are never reused within a process, so a cache of
// per-context state (symbol addresses, function attributes) keyed on it is refreshed after a
// cudaDeviceReset or any other context teardown.
uint64_t context_id();
// True, and `seen` updated, when the current context differs from `seen` (or is unknown).
bool context_changed(uint64_t &seen);
int make_plane_map(CUtensorMap *map, const float *plane, int64_t H, int64_t W, int64_t pitch,
                   int box_w, int box_h);
int check_grid(const fk_grid &g);
Model make_model(const fk_params &p);
// Converts the n <= kMaxStim stimuli of a kernel that holds them all (batch, adjoint).
int make_stims(const fk_stimulus *s, int n, const fk_grid &g, Stim *out);

// The up to FK_MAX_STIMULI stimuli of one call, and the ones a launch needs: those that can be
// active at one of its steps, in list order (the later stimulus wins where two overlap, so the
// order is kept).  A list of at most kMaxStim passes whole.
struct StimList {
    Stim all[FK_MAX_STIMULI];
    int n = 0;
    int make(const fk_stimulus *s, int count, const fk_grid &g);
    // the stimuli that can be active at a step of [t0, t1) into out[kMaxStim]; FK_ERR_STIMULI
    // when more than kMaxStim can
    int window(int64_t t0, int64_t t1, Stim *out, int *ns) const;
    // whether every launch of a run can take the same stimuli (at most kMaxStim in the list)
    bool fixed() const { return n <= kMaxStim; }
};

}  // namespace fk
