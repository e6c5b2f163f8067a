// Per-config tallies: condition counts, fixed-point wavenumber sums and the
// 18 x 36 condition-1 exit histogram.  Integer atomics only, so totals do not
// depend on the order photons finish in.
#pragma once
#include "mcw_internal.cuh"

namespace mcw {

// (theta, phi) -> bin t * 36 + p, 5 deg zenith and 10 deg azimuth bins.
__device__ __forceinline__ int exit_bin(float theta, float phi) {
    int t = (int)(theta * (float)(36.0 / kPi));
    int p = (int)(phi * (float)(18.0 / kPi));
    t = min(max(t, 0), MCW_HIST_NTHETA - 1);
    p = min(max(p, 0), MCW_HIST_NPHI - 1);
    return t * MCW_HIST_NPHI + p;
}

__device__ __forceinline__ unsigned long long *u64p(uint64_t *p) {
    return reinterpret_cast<unsigned long long *>(p);
}

// Straight to global memory (replay kernel; tally flushes).
__device__ __forceinline__ void tally_global(mcw_tally *t, int cond, int n_scat,
                                             unsigned long long wvn_fx, float theta, float phi) {
    atomicAdd(u64p(&t->n_cond[cond]), 1ull);
    atomicAdd(u64p(&t->q_cond_fx[cond]), wvn_fx);
    atomicAdd(u64p(&t->n_events), (unsigned long long)n_scat);
    atomicMax(&t->max_n_scat, (uint32_t)n_scat);
    if (cond == 1) {
        int b = exit_bin(theta, phi);
        atomicAdd(u64p(&t->bin_wvn_fx[b]), wvn_fx);
        atomicAdd(&t->bin_count[b], 1u);
    }
}

// Histogram bins only (the scalar totals go through a WarpTally).
__device__ __forceinline__ void tally_bin(mcw_tally *t, unsigned long long wvn_fx, float theta, float phi) {
    int b = exit_bin(theta, phi);
    atomicAdd(u64p(&t->bin_wvn_fx[b]), wvn_fx);
    atomicAdd(&t->bin_count[b], 1u);
}

__device__ __forceinline__ void warp_tally_reset(WarpTally &w, int lane) {
    if (lane == 0) { w.cfg = -1; w.max_n_scat = 0; w.n_events = 0; }
    if (lane < 6) { w.n_cond[lane] = 0; w.q_cond_fx[lane] = 0; }
}

// Add the warp's running totals to the global tally of its config and clear
// them.  Warp-collective: every lane of the warp calls it.
__device__ __forceinline__ void warp_tally_flush(WarpTally &w, mcw_tally *tallies, int lane) {
    __syncwarp();
    const int c = w.cfg;
    if (c >= 0) {
        mcw_tally *t = tallies + c;
        if (lane >= 1 && lane < 6) {
            if (w.n_cond[lane]) atomicAdd(u64p(&t->n_cond[lane]), (unsigned long long)w.n_cond[lane]);
            if (w.q_cond_fx[lane]) atomicAdd(u64p(&t->q_cond_fx[lane]), w.q_cond_fx[lane]);
        }
        if (lane == 6 && w.n_events) atomicAdd(u64p(&t->n_events), w.n_events);
        if (lane == 7 && w.max_n_scat) atomicMax(&t->max_n_scat, w.max_n_scat);
    }
    __syncwarp();
    warp_tally_reset(w, lane);
    __syncwarp();
}

}  // namespace mcw
