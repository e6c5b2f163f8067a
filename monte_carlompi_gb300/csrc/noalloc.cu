// mcw_walk_noalloc: the FP32 walk of one config for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not wanted,
// for example a plugin handed buffers by a host framework with its own memory
// pool, or a real-time loop that must not reach the allocator after start-up.
// Such a caller passes its own device buffers for the SSP tables, the records
// and the tally; everything else the walk needs (work counter, status word,
// per-config launch data, wavelength lookup table) lives in g_scratch below, a
// file-scope device array that every GPU loading this library holds until the
// process exits.  Nothing is allocated: no cudaMalloc, no cudaFree, no host
// heap.
//
// g_scratch is shared by every call on a device and keeps the last call's
// contents; each call clears what must start at zero.  Calls that overlap on
// the GPU (two streams, or two threads) race on it: serialise them.  The
// first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.  Later calls look the address up again unless
// their stream is capturing, so a device reset between calls is harmless.
//
// The caller's tables are checked on the device (ascending, distinct and
// finite wavelengths, finite values, ice extinction > 0) by the set-up kernel,
// and the call returns MCW_ERR_ARG before the lookup-table and walk kernels
// are launched when they fail.  The walk's time budget is the library's
// default, MCW_DEFAULT_BUDGET_S.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "mcw_internal.cuh"

namespace mcw {

namespace {

constexpr int kNoAllocLutMax = MCW_NOALLOC_MAX_LUT;  // wavelength grid points (include/mcwalk.h)
constexpr int kMaxDevices = 64;

struct NoAllocCounters {
    unsigned long long work;
    unsigned int status;
    unsigned int bad_table;
};

// Layout of the scratch array (offsets are multiples of 256 bytes).
struct __align__(256) NoAllocScratch {
    NoAllocCounters counters;
    alignas(256) DevConfig cfg;
    alignas(256) int64_t prefix[2];
    alignas(256) DevTable ice;
    alignas(256) mcw_tally tally;       // used when the caller passes no tally
    alignas(256) LutEntry lut[kNoAllocLutMax];
};

static __device__ __align__(256) unsigned char g_scratch[sizeof(NoAllocScratch)];

std::mutex g_mu;
NoAllocScratch *g_ptr[kMaxDevices] = {};

// One table column entry is usable: finite (and > 0 where positive is required).
__device__ __forceinline__ bool entry_ok(const double *col, int i, bool positive) {
    const double v = col[i];
    return isfinite(v) && (!positive || v > 0.0);
}

// Fill the scratch for this call from kernel parameters: zero the counters
// (and the caller's tally), store the config and table descriptors, and check
// the tables as mcw_set_tables checks host tables: finite values, strictly
// increasing wavelengths (the device lookups binary-search), and an ice
// extinction > 0 (its reciprocal sets the path length).
__global__ void noalloc_setup(NoAllocScratch *s, const DevConfig cfg, const DevTable ice, const DevTable imp,
                              mcw_tally *tally) {
    const int t = threadIdx.x;
    if (t == 0) {
        s->counters.work = 0;
        s->counters.status = 0;
        s->counters.bad_table = 0;
        s->cfg = cfg;
        s->prefix[0] = 0;
        s->prefix[1] = cfg.n_photon;
        s->ice = ice;
    }
    uint32_t *tw = reinterpret_cast<uint32_t *>(tally);
    for (int i = t; i < (int)(sizeof(mcw_tally) / 4); i += blockDim.x) tw[i] = 0u;
    __syncthreads();
    bool bad = false;
    for (int i = t; i < ice.n; i += blockDim.x) {
        bad |= !(entry_ok(ice.wvl, i, false) && entry_ok(ice.ssa, i, false) && entry_ok(ice.ext, i, true) &&
                 entry_ok(ice.asm_, i, false));
        if (i > 0) bad |= !(ice.wvl[i] > ice.wvl[i - 1]);
    }
    for (int i = t; i < imp.n; i += blockDim.x) {
        bad |= !(entry_ok(imp.wvl, i, false) && entry_ok(imp.ssa, i, false) && entry_ok(imp.ext, i, false));
        if (i > 0) bad |= !(imp.wvl[i] > imp.wvl[i - 1]);
    }
    if (bad) atomicOr(&s->counters.bad_table, 1u);
}

// Device address of g_scratch on the current device.  Resolved on every call
// whose stream is not capturing (cudaGetSymbolAddress allocates nothing), so a
// context torn down and recreated between calls gets the new address; a call
// made during capture uses the address of the last call outside it.
int scratch_for_device(int dev, cudaStream_t st, NoAllocScratch **out) {
    if (dev < 0 || dev >= kMaxDevices) return MCW_ERR_ARG;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const bool capturing = cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!capturing) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return MCW_ERR_CUDA;
        g_ptr[dev] = static_cast<NoAllocScratch *>(p);
    }
    if (!g_ptr[dev]) return MCW_ERR_STATE;   // first call on this device made during a capture
    *out = g_ptr[dev];
    return MCW_OK;
}

bool table_ok(const mcw_ssp_table *t, bool need_asm) {
    return t && t->n >= 2 && t->wvl && t->ss_alb && t->ext_cff_mss && (!need_asm || t->asm_prm) &&
           (t->wvl_unit == MCW_WVL_METRES || t->wvl_unit == MCW_WVL_MICRONS);
}

}  // namespace

}  // namespace mcw

using namespace mcw;

extern "C" int mcw_walk_noalloc(const mcw_config *cfg, const mcw_ssp_table *ice_dev, const mcw_ssp_table *imp_dev,
                                uint64_t seed, mcw_record32 *records_dev, mcw_tally *tally_dev, void *stream) {
    if (!cfg || !table_ok(ice_dev, true) || !table_ok(imp_dev, false)) return MCW_ERR_ARG;
    if (cfg->ice_table != 0 || cfg->polarised || config_problem(*cfg, 1)) return MCW_ERR_ARG;
    if (records_dev && ((uintptr_t)records_dev % 16) != 0) return MCW_ERR_ARG;
    if (tally_dev && ((uintptr_t)tally_dev % 8) != 0) return MCW_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // launch data of the config (same derivation as mcw_walk)
    const mcw_config &c = *cfg;
    const double sigma = c.half_width / 2.355;
    int64_t klo, khi;
    if (sigma > 0) {
        klo = (int64_t)std::floor((c.wvl0 - 6.5 * sigma) * 100.0) - 1;
        khi = (int64_t)std::ceil((c.wvl0 + 6.5 * sigma) * 100.0) + 1;
    } else {
        klo = khi = (int64_t)std::nearbyint(c.wvl0 * 100.0);
    }
    if (klo < 1) klo = 1;
    if (khi < klo) khi = klo;
    if (khi - klo + 1 > kNoAllocLutMax) return MCW_ERR_ARG;  // more grid points than the scratch holds
    DevConfig d;
    memset(&d, 0, sizeof(d));
    d.offset = 0;
    d.n_photon = c.n_photon;
    d.rng_base = (uint64_t)c.first_photon;  // config 0: stream id = first_photon + p
    d.lut_off = 0;
    d.lut_n = (int32_t)(khi - klo + 1);
    d.k_lo = (int32_t)klo;
    d.flags = (c.lambertian_surface ? kFlagLamSurface : 0u) | (c.lambertian_bottom ? kFlagLamBottom : 0u) |
              (c.imp_cnc > 0 ? kFlagImpurity : 0u) | (c.ssp_nearest ? kFlagNearest : 0u);
    d.ice_table = 0;
    const double theta0 = (kPi * c.theta0_deg) / 180.;
    d.wvl0_100 = (float)(c.wvl0 * 100.0);
    d.sigma_100 = (float)(sigma * 100.0);
    d.mux0 = (float)std::sin(theta0);
    d.muz0 = (float)(-std::cos(theta0));
    d.tau_tot = (float)c.tau_tot;
    d.R = (float)c.lambertian_reflectance;
    d.wvl0 = c.wvl0;
    d.scale = sigma;
    d.theta0 = theta0;
    d.mux0_d = std::sin(theta0);
    d.muz0_d = -std::cos(theta0);
    d.tau_tot_d = c.tau_tot;
    d.R_d = c.lambertian_reflectance;
    d.imp_cnc = c.imp_cnc;
    d.rho_snw = c.rho_snw;
    d.ov_ssa_ice = c.ssa_ice_override;
    d.ov_g = c.g_override;
    d.ov_ext_ice = c.ext_ice_override;
    d.ov_ssa_imp = c.ssa_imp_override;
    d.ov_ext_imp = c.ext_imp_override;
    DevTable ice{ice_dev->wvl, ice_dev->ss_alb, ice_dev->ext_cff_mss, ice_dev->asm_prm, ice_dev->n, ice_dev->wvl_unit};
    DevTable imp{imp_dev->wvl, imp_dev->ss_alb, imp_dev->ext_cff_mss, imp_dev->asm_prm, imp_dev->n, imp_dev->wvl_unit};

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCW_ERR_CUDA;
    NoAllocScratch *s = nullptr;
    int rc = scratch_for_device(dev, st, &s);
    if (rc) return rc;
    mcw_tally *tally = tally_dev ? tally_dev : &s->tally;

    noalloc_setup<<<1, 256, 0, st>>>(s, d, ice, imp, tally);
    if (cudaGetLastError() != cudaSuccess) return MCW_ERR_CUDA;
    // tables are checked before anything reads them
    unsigned int bad_table = 0;
    if (cudaMemcpyAsync(&bad_table, &s->counters.bad_table, sizeof(bad_table), cudaMemcpyDeviceToHost, st) !=
        cudaSuccess)
        return MCW_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCW_ERR_CUDA;
    if (bad_table) return MCW_ERR_ARG;
    LutArgs la;
    la.cfgs = &s->cfg;
    la.n_cfg = 1;
    la.stage = 0;
    la.stage_doubles = 0;
    la.counters_words = 0;
    la.lut = s->lut;
    la.imp = imp;
    la.ice = &s->ice;
    la.tallies = nullptr;   // cleared by noalloc_setup
    la.counters = nullptr;
    la.clear_only = 0;
    if (launch_lut(la, st) != cudaSuccess) return MCW_ERR_CUDA;
    if (c.n_photon > 0) {
        WalkArgs wa{};   // no drain handover: its queue would need an allocation
        wa.cfgs = &s->cfg;
        wa.prefix = s->prefix;
        wa.lut = s->lut;
        wa.n_cfg = 1;
        wa.regen_chunk = 8;
        wa.total = c.n_photon;
        wa.work = &s->counters.work;
        wa.status = &s->counters.status;
        wa.records = records_dev;
        wa.tallies = tally;
        wa.budget_ns = (unsigned long long)(MCW_DEFAULT_BUDGET_S * 1e9);
        wa.keys = philox_schedule(seed);
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MCW_ERR_CUDA;
        const bool impurity = c.imp_cnc > 0;
        int bps = walk_f32_max_blocks_per_sm(256, 1, impurity);
        if (bps < 1) bps = 1;
        int64_t grid = (int64_t)sms * bps;
        const int64_t needed = (c.n_photon + 255) / 256;
        if (grid > needed) grid = needed;
        if (launch_walk_f32(wa, impurity, (int)grid, 256, sms, st) != cudaSuccess) return MCW_ERR_CUDA;
    }
    NoAllocCounters h;
    if (cudaMemcpyAsync(&h, &s->counters, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MCW_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCW_ERR_CUDA;
    if (h.status & kStatusBudget) return MCW_ERR_BUDGET;
    return MCW_OK;
}
