// Internal device-side types of libmcwalk.
#pragma once
#include <cstdint>

#include "../../include/mcwalk.h"
#include "philox.cuh"

namespace mcw {

// Philox counter word 1 ("tag") separates the streams of one photon.
constexpr uint32_t kTagWalk = 0;    // replay: the walk's uniforms
constexpr uint32_t kTagWvl = 1;     // replay: wavelength Box-Muller
constexpr uint32_t kTagStep = 2;    // F32: per-step HG, azimuth, path, albedo draws
constexpr uint32_t kTagSpecies = 3; // F32: ice/impurity draw (only when imp_cnc > 0)
constexpr uint32_t kTagBirth = 5;   // F32: wavelength Box-Muller at photon birth
constexpr uint32_t kTagPolStep = 6;  // F32 polarised walk: a step's path, absorption, species, Lambertian words
constexpr uint32_t kTagPolRefl = 7;  // F32 polarised walk: a step's bottom reflectance draw
constexpr uint32_t kTagPolCand = 8;  // F32 polarised walk: rejection candidate j of a step (word y = 8 | j << 8)

// Device status bits.
constexpr uint32_t kStatusBudget = 1u;
constexpr uint32_t kStatusStream = 2u;

// Config flags.
constexpr uint32_t kFlagLamSurface = 1u;
constexpr uint32_t kFlagLamBottom = 2u;
constexpr uint32_t kFlagImpurity = 4u;  // imp_cnc > 0: the species draw matters
constexpr uint32_t kFlagNearest = 16u;  // ssp_nearest: nearest ice-table point, wavelength replaced
constexpr uint32_t kFlagPolarised = 32u;  // polarised walk (phase matrices, Stokes vector)

constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 6.283185307179586;  // 2*np.pi (monte_carlo3D.py:26)

// One SSP table as device pointers.
struct DevTable {
    const double *wvl, *ssa, *ext, *asm_;
    int32_t n;
    int32_t unit;        // MCW_WVL_METRES or MCW_WVL_MICRONS
};

// Per-config launch data computed on the host from mcw_config.
struct DevConfig {
    int64_t offset;       // record index of the config's first photon
    int64_t n_photon;
    uint64_t rng_base;    // stream id of photon 0: config << 40 | first_photon
    int32_t lut_off;      // first LUT entry of this config
    int32_t lut_n;        // LUT entries (wavelength grid points k_lo .. k_lo+lut_n-1)
    int32_t k_lo;         // lambda = k / 100 um for LUT entry 0
    uint32_t flags;
    int32_t ice_table;
    int32_t pad;
    // FP32 walk
    float wvl0_100;       // wvl0 * 100
    float sigma_100;      // sigma * 100, sigma = FWHM / 2.355
    float mux0, muz0;     // initial direction (sin theta0, 0, -cos theta0)
    float tau_tot, R;
    // FP64 replay walk
    double wvl0, scale, theta0, tau_tot_d, R_d, imp_cnc, rho_snw;
    double mux0_d, muz0_d;  // sin(theta0), -cos(theta0), evaluated on the host
    double ov_ssa_ice, ov_g, ov_ext_ice, ov_ssa_imp, ov_ext_imp;  // NaN = table
    double stokes0[4];    // polarised walk: incident Stokes vector
};

// Phase matrices of one ice table for the FP32 polarised walk (float copies).
struct DevPhase32 {
    const float *cos_asc[6];
    const float *p_asc[6];
    const float *a1, *a2, *b1, *b2;
    int32_t n_angle[6];
    int32_t n_rows;
    int32_t shared_grid;         // 1: the six elements share one cos grid (one search serves all)
    float cos_max, cos_min, cos_cutoff, pad2;
    // seeds of the search on the shared grid: seed[b] = first grid index with
    // cos >= the lower edge of bucket b, kPhaseBuckets buckets uniform on [cos_min, cos_max]
    const uint16_t *seed;
    float seed_lo, seed_scale;
};
constexpr int kPhaseBuckets = 2048;

// Phase matrices of one ice table on the device (mcw_phase_table, rows in the
// device table's order).
struct DevPhase {
    const double *cos_asc[6];
    const double *p_asc[6];
    const double *a1, *a2, *b1, *b2;
    int32_t n_angle[6];
    int32_t n_rows;
    int32_t pad;
    double cos_max, cos_min, cos_cutoff;
};

// Optics of one wavelength grid point, FP32 walk.  32 bytes + fixed-point wvn.
// Co-albedos (1 - ss_alb) are stored so small absorption keeps full precision.
struct LutEntry {
    float wvn;        // 1 / lambda [um^-1]
    float coalb_ice;  // 1 - ssa_ice
    float coalb_imp;  // 1 - ssa_imp
    float g;
    float inv_ext;    // 1 / (ext_cff_mss * rho_snw) [m]
    float p_imp;      // P_ext_imp
    float snow_depth; // [m]
    float pad;
    unsigned long long wvn_fx;  // wvn * 2^32, rounded
    unsigned long long pad2;    // the nearest ice-table row (the polarised walk's phase-matrix row)
};

// Per-warp running totals for the warp's current config (shared memory).
struct WarpTally {
    int32_t cfg;          // -1 = empty
    uint32_t max_n_scat;
    uint32_t n_cond[6];
    unsigned long long q_cond_fx[6];
    unsigned long long n_events;
};

struct WalkArgs {
    const DevConfig *cfgs;
    const int64_t *prefix;       // n_cfg + 1 global photon offsets
    // claim order: the walk hands out photons of config claim_cfg[k] for claim ids
    // claim_prefix[k] .. claim_prefix[k + 1] - 1 (null: configs in order, claim id =
    // record index)
    const int64_t *claim_prefix;
    const int32_t *claim_cfg;
    const LutEntry *lut;
    int32_t n_cfg;
    int32_t regen_chunk;
    int64_t total;               // photons over all configs
    unsigned long long *work;    // next unclaimed global photon id
    unsigned int *status;
    mcw_record32 *records;       // may be null
    mcw_tally *tallies;          // n_cfg device tallies
    unsigned long long budget_ns;
    PhiloxKeys keys;
    // drain handover: once the photon supply is exhausted, photons past drain_from
    // steps (in block mode) leave the walk for drain (kDrainSlot float4 each, at
    // most one per thread of the walk grid); the drain kernel after the walk walks
    // each with a whole thread block.  drain == null or drain_from == 0: no handover.
    float4 *drain;
    unsigned int *drain_count;   // slots written
    unsigned int *drain_next;    // the drain kernel's next slot
    int32_t drain_from;
    uint32_t drain_cap;          // slots in drain (grid * block)
    const DevPhase32 *phase;     // FP32 polarised walk: per ice table (records are mcw_record32p)
    int32_t deep;                // slabs optically deep (tau >= kDeepTau) for most of the scatter
                                 // events of the launch, no Lambertian surface and no isotropic
                                 // scattering: the kernel instance whose steps branch on the
                                 // (rare) bottom crossing and carry no surface or isotropic
                                 // alternatives; the records are the same either way
};

// Optical depth from which a slab counts as deep for WalkArgs::deep.
constexpr double kDeepTau = 32.0;

struct ReplayArgs {
    const DevConfig *cfgs;
    const int64_t *prefix;
    int32_t n_cfg;
    int32_t pol;                 // 1: the polarised walk, records mcw_record64p
    const DevPhase *phase;       // per ice table (pol)
    int64_t total;
    DevTable imp;
    const DevTable *ice;         // device array of ice tables
    unsigned int *status;
    void *records;               // mcw_record64, or mcw_record64p (pol)
    mcw_tally *tallies;
    unsigned long long budget_ns;
    uint64_t seed;
};

struct LutArgs {
    const DevConfig *cfgs;
    int32_t n_cfg;
    int32_t stage;               // stage table wavelengths in shared memory
    int32_t stage_doubles;       // largest ice table + impurity table length
    int32_t counters_words;      // 32-bit words of *counters to clear
    LutEntry *lut;
    DevTable imp;
    const DevTable *ice;
    mcw_tally *tallies;          // n_cfg tallies to clear, or null
    uint32_t *counters;          // work counter and status to clear, or null
    int32_t clear_only;          // 1: clear tallies and counters, leave the table as it is
};

// Why a config is invalid (nullptr when valid); n_ice = number of ice tables.
const char *config_problem(const mcw_config &c, int32_t n_ice);

// Kernel launchers (defined in the .cu files).
// recs: n records of `stride` bytes starting with an mcw_record64 (f64) or mcw_record32.
cudaError_t launch_post(const void *recs, bool f64, size_t stride, int64_t n, int n_cfg, int n_bins,
                        unsigned long long *bins_fx, unsigned int *bins_cnt, mcw_post_stats *stats, int sms,
                        cudaStream_t s);
cudaError_t launch_lut(const LutArgs &a, cudaStream_t s);
// Photons the walk hands over to its drain queue are packed as this many float4.
constexpr int kDrainSlot = 6;
// impurity: some config has imp_cnc > 0 (the kernel instance with the species draw).
// Launches the walk and, when a.drain_from > 0, the drain kernel after it
// (sm_count SMs; a.drain must then hold grid * block slots).
cudaError_t launch_walk_f32(const WalkArgs &a, bool impurity, int grid, int block, int sm_count, cudaStream_t s);
cudaError_t launch_walk_replay(const ReplayArgs &a, cudaStream_t s);
// The FP32 polarised walk (a.phase set, a.records holding mcw_record32p).
cudaError_t launch_walk_pol32(const WalkArgs &a, int sm_count, cudaStream_t s);
int walk_f32_max_blocks_per_sm(int block, int n_cfg, bool impurity);
// The walk and drain kernels (their one parameter is a WalkArgs).
bool walk_f32_is_kernel(const void *fn);
size_t walk_f32_smem_bytes(int block, int n_cfg);

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int kRngConfigShift = 40;  // stream id = config << 40 | photon index

// Config of a global photon id: largest c with prefix[c] <= gid.
__device__ __forceinline__ int find_config(const int64_t *prefix, int n_cfg, int64_t gid) {
    int lo = 0, hi = n_cfg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= gid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace mcw
