// C ABI of libmcwalk: context, tables, walk dispatch, autotuner, CUDA graphs.
// Declarations and the reference interface each entry point replaces are in
// include/mcwalk.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "mcw_internal.cuh"

using namespace mcw;

static_assert(sizeof(mcw_config) == 176, "mcw_config layout");
static_assert(sizeof(mcw_record64p) == 80, "mcw_record64p layout");
static_assert(sizeof(mcw_record32p) == 48, "mcw_record32p layout");
static_assert(sizeof(mcw_record32) == 32, "mcw_record32 layout");
static_assert(sizeof(mcw_record64) == 56, "mcw_record64 layout");
static_assert(sizeof(mcw_stats) == 80, "mcw_stats layout");
static_assert(sizeof(mcw_tally) == 13 * 8 + 8 + 648 * 12, "mcw_tally layout");

namespace {

const char kVersion[] = "libmcwalk 0.1 (sm_103a)";

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Host-side plan of one walk: per-config launch data and the LUT layout.
struct Plan {
    std::vector<DevConfig> cfgs;
    std::vector<int64_t> prefix;
    // the order in which the FP32 walk hands out photons: configs whose walks are
    // expected to run longest first (claim_cfg[k] = config taken k-th, claim_prefix
    // its cumulative photon counts); records do not depend on it
    std::vector<int64_t> claim_prefix;
    std::vector<int32_t> claim_cfg;
    int64_t total = 0;
    int32_t lut_total = 0;
    bool impurity = false;  // some config has imp_cnc > 0
    // the deep-slab kernel instance (WalkArgs::deep): no config is a Lambertian surface
    // or scatters isotropically, and the configs with tau < kDeepTau hold at most a fifth
    // of the expected scatter events (records do not depend on it)
    bool deep = false;
};

struct Counters {
    unsigned long long work;
    unsigned int status;
    unsigned int drain_count;   // drain-queue slots written
    unsigned int drain_next;    // the drain kernel's next slot
    unsigned int pad[4];
};

}  // namespace

struct mcw_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs = nullptr, eve = nullptr;
    char err[512] = {0};
    // tables
    DevBuf tabdata, ice_tables;
    DevTable imp{};
    int32_t n_ice = 0;
    bool have_tables = false;
    std::vector<std::vector<int32_t>> ice_order;   // row permutation of each ice table (stored ascending)
    // host copy of the device tables (the claim order's estimate of walk lengths)
    std::vector<double> h_tab;
    std::vector<DevTable> h_ice;                   // offsets into h_tab (pointers unused)
    // per ice table: every asymmetry parameter is of one sign and at least 1e-3 away from
    // 0, so no photon scatters isotropically (the deep-slab instance's HG step)
    std::vector<char> h_ice_aniso;
    // phase matrices of the polarised walk, one per ice table (n_rows 0 = none)
    DevBuf phasedata, phase_tables, phasedata32, phase_tables32, phase_seeds;
    std::vector<int32_t> phase_rows;
    // workspace
    DevBuf cfgs, lut, tallies, counters, records, post, drain;
    HostBuf h_stage, h_tallies, h_counters;
    int32_t max_ice_n = 0;
    // the plan (configs + prefix bytes) whose lookup table ctx->lut holds, for
    // the tables of version tables_version; empty when none does
    std::vector<unsigned char> lut_plan;
    uint64_t tables_version = 0, lut_tables_version = 0;
    void *lut_cfgs_ptr = nullptr, *lut_ptr = nullptr;
    mcw_launch launch{256, 0, 8, 4096};
    double budget_s = MCW_DEFAULT_BUDGET_S;
};

struct mcw_graph {
    mcw_ctx *ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraphNode_t> walk_nodes;         // the walk and drain kernels (seeded per launch)
    std::vector<cudaKernelNodeParams> walk_params;
    WalkArgs args{};
    int32_t n_cfg = 0;
    int64_t total = 0;
    int grid = 0, block = 0;
    DevBuf cfgs, lut, tallies, counters, drain;
    HostBuf h_tallies, h_counters;
};

namespace {

int set_err(mcw_ctx *ctx, int code, const char *fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CUDA_TRY(ctx, call)                                                                      \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return set_err((ctx), _e == cudaErrorMemoryAllocation ? MCW_ERR_OOM : MCW_ERR_CUDA,  \
                           "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
    } while (0)

bool finite_pos(double x) { return std::isfinite(x) && x > 0; }

// Validate one config the way MonteCarlo.run's inputs must be for the HG
// sphere path.  Returns nullptr when valid.
const char *check_config(const mcw_config &c, int32_t n_ice) {
    if (c.n_photon < 0) return "n_photon < 0";
    if (c.first_photon < 0 || c.first_photon > (int64_t(1) << kRngConfigShift) - c.n_photon)
        return "first_photon + n_photon must lie in [0, 2^40]";
    if (!finite_pos(c.wvl0)) return "wvl0 must be finite and > 0";
    if (!std::isfinite(c.half_width) || c.half_width < 0) return "half_width must be finite and >= 0";
    if (!std::isfinite(c.theta0_deg) || c.theta0_deg < 0 || c.theta0_deg >= 90) return "theta0_deg must be in [0, 90)";
    if (!finite_pos(c.tau_tot)) return "tau_tot must be finite and > 0";
    if (!std::isfinite(c.imp_cnc) || c.imp_cnc < 0 || c.imp_cnc > 1) return "imp_cnc must be in [0, 1]";
    if (!finite_pos(c.rho_snw)) return "rho_snw must be finite and > 0";
    if (!std::isfinite(c.lambertian_reflectance) || c.lambertian_reflectance < 0 || c.lambertian_reflectance > 1)
        return "lambertian_reflectance must be in [0, 1]";
    if (c.ice_table < 0 || c.ice_table >= n_ice) return "ice_table out of range";
    if (c.ssp_nearest != 0 && c.ssp_nearest != 1) return "ssp_nearest must be 0 or 1";
    if (c.polarised != 0 && c.polarised != 1) return "polarised must be 0 or 1";
    if (c.polarised) {
        if (!c.ssp_nearest) return "the polarised walk needs ssp_nearest = 1 (aspherical tables)";
        for (int k = 0; k < 4; ++k)
            if (!std::isfinite(c.stokes0[k])) return "stokes0 must be finite";
        if (c.stokes0[0] == 0) return "stokes0[0] (I) must not be 0";
    }
    if (!std::isnan(c.ssa_ice_override) && !(c.ssa_ice_override >= 0 && c.ssa_ice_override <= 1)) return "ssa_ice_override must be in [0, 1]";
    if (!std::isnan(c.ssa_imp_override) && !(c.ssa_imp_override >= 0 && c.ssa_imp_override <= 1)) return "ssa_imp_override must be in [0, 1]";
    if (!std::isnan(c.g_override) && !(c.g_override > -1 && c.g_override < 1)) return "g_override must be in (-1, 1)";
    if (!std::isnan(c.ext_ice_override) && !finite_pos(c.ext_ice_override)) return "ext_ice_override must be > 0";
    if (!std::isnan(c.ext_imp_override) && !(std::isfinite(c.ext_imp_override) && c.ext_imp_override >= 0)) return "ext_imp_override must be >= 0";
    return nullptr;
}

constexpr int32_t kMaxLutPerConfig = 1 << 16;

// Linear interpolation of column col (1 ss_alb, 3 asm_prm) of ice table t at
// wavelength x [um], clamped to the table's ends (host copy; ordering only).
double host_column(const mcw_ctx *ctx, int32_t t, int col, double x_um) {
    const DevTable &d = ctx->h_ice[t];
    const double *base = ctx->h_tab.data() + (d.wvl - (const double *)ctx->tabdata.p);
    const double *w = base, *v = base + (size_t)col * d.n;
    const double x = d.unit == MCW_WVL_METRES ? x_um * 1e-6 : x_um;
    if (x <= w[0]) return v[0];
    if (x >= w[d.n - 1]) return v[d.n - 1];
    const int32_t hi = (int32_t)(std::upper_bound(w, w + d.n, x) - w);
    const double f = (x - w[hi - 1]) / (w[hi] - w[hi - 1]);
    return v[hi - 1] + f * (v[hi] - v[hi - 1]);
}

// Expected length (scatter events) of a config's longest walks, for the claim
// order: absorption ends a walk after about 1 / (1 - ssa) events (the smallest
// co-albedo within 2 sigma of the centre wavelength), a slab of optical depth tau
// after about tau^2 (1 - g) (diffusion across it).  Only the ranking matters.
double walk_length_estimate(const mcw_ctx *ctx, const mcw_config &c) {
    const double sigma = c.half_width / 2.355;
    double coalb = 1.0, g = 0.0;
    for (int k = -2; k <= 2; k += 2) {
        const double x = c.wvl0 + k * sigma;
        const double ssa = std::isnan(c.ssa_ice_override) ? host_column(ctx, c.ice_table, 1, x) : c.ssa_ice_override;
        coalb = std::min(coalb, 1.0 - ssa);
        if (k == 0) g = std::isnan(c.g_override) ? host_column(ctx, c.ice_table, 3, x) : c.g_override;
    }
    if (c.lambertian_surface) return 1.0 / std::max(1.0 - c.lambertian_reflectance, 1e-9);
    const double absorb = 1.0 / std::max(coalb, 1e-12);
    const double slab = c.tau_tot * c.tau_tot * std::max(1.0 - g, 1e-3) + c.tau_tot;
    return std::min(absorb, slab);
}

// Claim order of a plan: longest expected walks first (stable: ties keep the
// callers' order).
void make_claim_order(const mcw_ctx *ctx, const mcw_config *cfgs, Plan &plan) {
    const int32_t n = (int32_t)plan.cfgs.size();
    std::vector<double> key(n);
    for (int32_t i = 0; i < n; ++i) key[i] = (n > 1 && !ctx->h_ice.empty()) ? walk_length_estimate(ctx, cfgs[i]) : 0.0;
    plan.claim_cfg.resize(n);
    for (int32_t i = 0; i < n; ++i) plan.claim_cfg[i] = i;
    std::stable_sort(plan.claim_cfg.begin(), plan.claim_cfg.end(),
                     [&](int32_t a, int32_t b) { return key[a] > key[b]; });
    plan.claim_prefix.assign(n + 1, 0);
    for (int32_t k = 0; k < n; ++k) plan.claim_prefix[k + 1] = plan.claim_prefix[k] + plan.cfgs[plan.claim_cfg[k]].n_photon;
    // deep-slab instance: no config is a Lambertian surface, and the thin configs' share
    // of the expected events (photons x expected walk length) is small; one config: its
    // own depth
    // and no photon scatters isotropically (the asymmetry parameter of every config away
    // from 0: its override, or every value of its ice table)
    bool surface = false;
    for (int32_t i = 0; i < n; ++i) {
        surface = surface || cfgs[i].lambertian_surface;
        const double g = cfgs[i].g_override;
        const bool aniso = std::isnan(g) ? (cfgs[i].ice_table >= 0 && cfgs[i].ice_table < (int32_t)ctx->h_ice_aniso.size() &&
                                            ctx->h_ice_aniso[cfgs[i].ice_table])
                                         : std::fabs(g) > 1e-3;
        surface = surface || !aniso;
    }
    if (surface) {
        plan.deep = false;
    } else if (n == 1 || ctx->h_ice.empty()) {
        plan.deep = true;
        for (const DevConfig &c : plan.cfgs) plan.deep = plan.deep && c.tau_tot_d >= kDeepTau;
    } else {
        double thin = 0.0, all = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            const double w = (double)plan.cfgs[i].n_photon * key[i];
            all += w;
            if (!(plan.cfgs[i].tau_tot_d >= kDeepTau)) thin += w;
        }
        plan.deep = thin <= 0.2 * all;
    }
}

int make_plan(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, int32_t mode, Plan &plan) {
    if (!cfgs || n_cfg <= 0) return set_err(ctx, MCW_ERR_ARG, "need at least one config");
    if (n_cfg > (1 << 23)) return set_err(ctx, MCW_ERR_ARG, "at most 2^23 configs per call");
    const bool pol_mode = (mode == MCW_MODE_POL64 || mode == MCW_MODE_POL32);
    for (int32_t i = 0; i < n_cfg; ++i) {
        if (cfgs[i].polarised && !pol_mode)
            return set_err(ctx, MCW_ERR_ARG, "config %d: the polarised walk runs in MCW_MODE_POL32 or MCW_MODE_POL64", i);
        if (!cfgs[i].polarised && pol_mode)
            return set_err(ctx, MCW_ERR_ARG, "config %d: the polarised modes walk polarised configs only", i);
        if (cfgs[i].polarised && cfgs[i].ice_table >= 0 && cfgs[i].ice_table < ctx->n_ice &&
            ((int32_t)ctx->phase_rows.size() <= cfgs[i].ice_table || ctx->phase_rows[cfgs[i].ice_table] == 0))
            return set_err(ctx, MCW_ERR_STATE, "config %d: ice table %d has no phase matrices", i,
                           cfgs[i].ice_table);
    }
    plan.cfgs.resize(n_cfg);
    plan.prefix.resize(n_cfg + 1);
    int64_t off = 0;
    int32_t lut_off = 0;
    for (int32_t i = 0; i < n_cfg; ++i) {
        const mcw_config &c = cfgs[i];
        if (const char *why = check_config(c, ctx->n_ice)) return set_err(ctx, MCW_ERR_ARG, "config %d: %s", i, why);
        DevConfig d{};
        d.offset = off;
        d.n_photon = c.n_photon;
        d.rng_base = ((uint64_t)i << kRngConfigShift) | (uint64_t)c.first_photon;
        plan.prefix[i] = off;
        if (off > INT64_MAX - c.n_photon) return set_err(ctx, MCW_ERR_ARG, "total photon count overflows");
        off += c.n_photon;
        const double sigma = c.half_width / 2.355;
        // wavelength grid of the LUT: lambda = k / 100 um over wvl0 +- 6.5 sigma
        int64_t klo, khi;
        if (sigma > 0) {
            klo = (int64_t)std::floor((c.wvl0 - 6.5 * sigma) * 100.0) - 1;
            khi = (int64_t)std::ceil((c.wvl0 + 6.5 * sigma) * 100.0) + 1;
        } else {
            klo = khi = (int64_t)std::nearbyint(c.wvl0 * 100.0);
        }
        klo = std::max<int64_t>(klo, 1);
        khi = std::max<int64_t>(khi, klo);
        if (khi - klo + 1 > kMaxLutPerConfig) return set_err(ctx, MCW_ERR_ARG, "config %d: half_width too wide", i);
        d.k_lo = (int32_t)klo;
        d.lut_n = (int32_t)(khi - klo + 1);
        d.lut_off = lut_off;
        lut_off += d.lut_n;
        d.flags = (c.lambertian_surface ? kFlagLamSurface : 0u) | (c.lambertian_bottom ? kFlagLamBottom : 0u) |
                  (c.imp_cnc > 0 ? kFlagImpurity : 0u) | (c.ssp_nearest ? kFlagNearest : 0u) |
                  (c.polarised ? kFlagPolarised : 0u);
        for (int k = 0; k < 4; ++k) d.stokes0[k] = c.polarised ? c.stokes0[k] : (k == 0 ? 1.0 : 0.0);
        d.ice_table = c.ice_table;
        if (c.imp_cnc > 0) plan.impurity = true;
        const double theta0 = (kPi * c.theta0_deg) / 180.;  // monte_carlo3D.py:1508
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
        plan.cfgs[i] = d;
    }
    plan.prefix[n_cfg] = off;
    plan.total = off;
    plan.lut_total = lut_off;
    make_claim_order(ctx, cfgs, plan);
    return MCW_OK;
}

struct Shape {
    int grid, block, chunk, bps;
};

Shape pick_shape(const mcw_ctx *ctx, const mcw_launch &l, const Plan &plan) {
    const int64_t total = plan.total;
    Shape s;
    s.block = l.block_size;
    int occ = walk_f32_max_blocks_per_sm(s.block, (int)plan.cfgs.size(), plan.impurity);
    if (occ <= 0) occ = 1;
    s.bps = (l.blocks_per_sm > 0) ? std::min(l.blocks_per_sm, occ) : occ;
    s.chunk = l.regen_chunk;
    int64_t grid = (int64_t)ctx->sm_count * s.bps;
    const int64_t needed = (total + s.block - 1) / s.block;
    grid = std::max<int64_t>(1, std::min(grid, needed));
    s.grid = (int)grid;
    return s;
}

// Byte offset of the prefix array inside the plan buffer (after the configs).
size_t prefix_offset(size_t n_cfg) { return (n_cfg * sizeof(DevConfig) + 255) & ~size_t(255); }

// Upload a plan (configs then prefix, one copy) through a pinned staging buffer.
int upload_plan(mcw_ctx *ctx, const Plan &plan, DevBuf &cfgs, DevBuf &lut, DevBuf &tallies, DevBuf &counters,
                cudaStream_t st, cudaEvent_t start = nullptr, uint64_t *h2d = nullptr) {
    const size_t n_cfg = plan.cfgs.size();
    const size_t b_cfg = n_cfg * sizeof(DevConfig);
    const size_t off = prefix_offset(n_cfg);
    // configs | prefix (n + 1) | claim_prefix (n + 1) | claim_cfg (n)
    const size_t b_all = off + 2 * (n_cfg + 1) * sizeof(int64_t) + n_cfg * sizeof(int32_t);
    CUDA_TRY(ctx, cfgs.ensure(b_all));
    CUDA_TRY(ctx, lut.ensure(std::max<size_t>(1, plan.lut_total) * sizeof(LutEntry)));
    CUDA_TRY(ctx, tallies.ensure(n_cfg * sizeof(mcw_tally)));
    CUDA_TRY(ctx, counters.ensure(sizeof(Counters)));
    // the staging buffer must not be rewritten while a previous copy reads it
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    CUDA_TRY(ctx, ctx->h_stage.ensure(b_all));
    char *h = (char *)ctx->h_stage.p;
    memcpy(h, plan.cfgs.data(), b_cfg);
    memset(h + b_cfg, 0, off - b_cfg);
    memcpy(h + off, plan.prefix.data(), (n_cfg + 1) * sizeof(int64_t));
    memcpy(h + off + (n_cfg + 1) * sizeof(int64_t), plan.claim_prefix.data(), (n_cfg + 1) * sizeof(int64_t));
    memcpy(h + off + 2 * (n_cfg + 1) * sizeof(int64_t), plan.claim_cfg.data(), n_cfg * sizeof(int32_t));
    if (start) CUDA_TRY(ctx, cudaEventRecord(start, st));
    if (h2d) *h2d = b_all;
    CUDA_TRY(ctx, cudaMemcpyAsync(cfgs.p, h, b_all, cudaMemcpyHostToDevice, st));
    return MCW_OK;
}

// The plan's bytes as uploaded (configs, then prefix): equal bytes and equal
// tables give an equal lookup table.
std::vector<unsigned char> plan_bytes(const Plan &plan) {
    const size_t bc = plan.cfgs.size() * sizeof(DevConfig), bp = plan.prefix.size() * sizeof(int64_t);
    const size_t bk = plan.claim_cfg.size() * sizeof(int32_t);
    std::vector<unsigned char> v(bc + 2 * bp + bk);
    memcpy(v.data(), plan.cfgs.data(), bc);
    memcpy(v.data() + bc, plan.prefix.data(), bp);
    memcpy(v.data() + bc + bp, plan.claim_prefix.data(), bp);
    memcpy(v.data() + bc + 2 * bp, plan.claim_cfg.data(), bk);
    return v;
}

LutArgs lut_args(const mcw_ctx *ctx, const Plan &plan, DevBuf &cfgs, DevBuf &lut, DevBuf &tallies,
                 DevBuf &counters) {
    LutArgs la;
    la.clear_only = 0;
    la.cfgs = (const DevConfig *)cfgs.p;
    la.n_cfg = (int32_t)plan.cfgs.size();
    la.stage_doubles = ctx->max_ice_n + ctx->imp.n;
    la.stage = la.stage_doubles <= 12288 ? 1 : 0;  // up to 96 KB of shared memory
    la.counters_words = (int32_t)(sizeof(Counters) / 4);
    la.lut = (LutEntry *)lut.p;
    la.imp = ctx->imp;
    la.ice = (const DevTable *)ctx->ice_tables.p;
    la.tallies = (mcw_tally *)tallies.p;
    la.counters = (uint32_t *)counters.p;
    return la;
}

WalkArgs walk_args(const mcw_ctx *ctx, const Plan &plan, DevBuf &cfgs, DevBuf &lut, DevBuf &tallies,
                   DevBuf &counters, mcw_record32 *records, int chunk, uint64_t seed) {
    WalkArgs wa{};
    wa.cfgs = (const DevConfig *)cfgs.p;
    wa.prefix = (const int64_t *)((const char *)cfgs.p + prefix_offset(plan.cfgs.size()));
    wa.claim_prefix = wa.prefix + (plan.cfgs.size() + 1);
    wa.claim_cfg = (const int32_t *)(wa.claim_prefix + (plan.cfgs.size() + 1));
    wa.lut = (const LutEntry *)lut.p;
    wa.n_cfg = (int32_t)plan.cfgs.size();
    wa.regen_chunk = chunk;
    wa.total = plan.total;
    Counters *cn = (Counters *)counters.p;
    wa.work = &cn->work;
    wa.status = &cn->status;
    wa.records = records;
    wa.tallies = (mcw_tally *)tallies.p;
    wa.budget_ns = (unsigned long long)(ctx->budget_s * 1e9);
    wa.keys = philox_schedule(seed);
    wa.drain_count = &cn->drain_count;
    wa.drain_next = &cn->drain_next;
    wa.deep = plan.deep ? 1 : 0;
    return wa;
}

// Attach the drain queue (one slot per thread of the walk grid) when handover is on.
int attach_drain(mcw_ctx *ctx, WalkArgs &wa, DevBuf &drain, const Shape &shape) {
    wa.drain = nullptr;
    wa.drain_from = 0;
    if (ctx->launch.drain_from <= 0) return MCW_OK;
    CUDA_TRY(ctx, drain.ensure((size_t)shape.grid * shape.block * kDrainSlot * sizeof(float4)));
    wa.drain = (float4 *)drain.p;
    wa.drain_cap = (uint32_t)((size_t)shape.grid * shape.block);
    wa.drain_from = ctx->launch.drain_from;
    return MCW_OK;
}

}  // namespace

namespace mcw {
// Validation of one config, shared with entry points in other units.
const char *config_problem(const mcw_config &c, int32_t n_ice) { return check_config(c, n_ice); }
}  // namespace mcw

extern "C" {

int mcw_abi_version(void) { return MCW_ABI_VERSION; }
const char *mcw_version(void) { return kVersion; }

int mcw_create(int device, mcw_ctx **out) {
    if (!out) return MCW_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return MCW_ERR_CUDA;
    if (device < 0 || device >= n) return MCW_ERR_ARG;
    mcw_ctx *ctx = new (std::nothrow) mcw_ctx();
    if (!ctx) return MCW_ERR_OOM;
    ctx->device = device;
    int rc = MCW_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { rc = MCW_ERR_CUDA; break; }
        if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) { rc = MCW_ERR_CUDA; break; }
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = MCW_ERR_CUDA; break; }
        if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
            cudaEventCreate(&ctx->evs) != cudaSuccess || cudaEventCreate(&ctx->eve) != cudaSuccess) { rc = MCW_ERR_CUDA; break; }
        if (ctx->h_counters.ensure(sizeof(Counters)) != cudaSuccess) { rc = MCW_ERR_OOM; break; }
    } while (0);
    if (rc != MCW_OK) {
        mcw_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return MCW_OK;
}

int mcw_destroy(mcw_ctx *ctx) {
    if (!ctx) return MCW_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (DevBuf *b : {&ctx->tabdata, &ctx->ice_tables, &ctx->cfgs, &ctx->lut, &ctx->tallies, &ctx->counters,
                      &ctx->records, &ctx->post, &ctx->drain})
        b->release();
    ctx->h_stage.release();
    ctx->h_tallies.release();
    ctx->h_counters.release();
    for (cudaEvent_t e : {ctx->ev0, ctx->ev1, ctx->evs, ctx->eve})
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MCW_OK;
}

int mcw_last_error(const mcw_ctx *ctx, char *buf, size_t len) {
    if (!ctx || !buf || len == 0) return MCW_ERR_ARG;
    snprintf(buf, len, "%s", ctx->err);
    return MCW_OK;
}

int mcw_set_tables(mcw_ctx *ctx, const mcw_ssp_table *ice, int32_t n_ice, const mcw_ssp_table *imp) {
    if (!ctx) return MCW_ERR_ARG;
    if (!ice || n_ice <= 0 || !imp) return set_err(ctx, MCW_ERR_ARG, "need >= 1 ice table and an impurity table");
    auto check = [](const mcw_ssp_table &t, bool need_asm) -> const char * {
        if (t.n < 2) return "a table needs at least 2 wavelengths";
        if (t.wvl_unit != MCW_WVL_METRES && t.wvl_unit != MCW_WVL_MICRONS)
            return "wvl_unit must be MCW_WVL_METRES or MCW_WVL_MICRONS";
        if (!t.wvl || !t.ss_alb || !t.ext_cff_mss || (need_asm && !t.asm_prm)) return "missing table column";
        for (int32_t i = 0; i < t.n; ++i) {
            if (!std::isfinite(t.wvl[i]) || !std::isfinite(t.ss_alb[i]) || !std::isfinite(t.ext_cff_mss[i]))
                return "non-finite table value";
            if (need_asm && !std::isfinite(t.asm_prm[i])) return "non-finite table value";
            if (need_asm && !(t.ext_cff_mss[i] > 0)) return "ice extinction must be > 0";
        }
        return nullptr;
    };
    size_t total = 0;
    for (int32_t i = 0; i < n_ice; ++i) {
        if (const char *why = check(ice[i], true)) return set_err(ctx, MCW_ERR_ARG, "ice table %d: %s", i, why);
        total += 4 * (size_t)ice[i].n;
    }
    if (const char *why = check(*imp, false)) return set_err(ctx, MCW_ERR_ARG, "impurity table: %s", why);
    {
        std::vector<int32_t> tmp;
        auto distinct = [&](const mcw_ssp_table &t) {
            tmp.resize(t.n);
            for (int32_t i = 0; i < t.n; ++i) tmp[i] = i;
            std::stable_sort(tmp.begin(), tmp.end(), [&](int32_t a, int32_t b) { return t.wvl[a] < t.wvl[b]; });
            for (int32_t i = 1; i < t.n; ++i)
                if (!(t.wvl[tmp[i]] > t.wvl[tmp[i - 1]])) return false;
            return true;
        };
        for (int32_t i = 0; i < n_ice; ++i)
            if (!distinct(ice[i])) return set_err(ctx, MCW_ERR_ARG, "ice table %d: repeated wavelength", i);
        if (!distinct(*imp)) return set_err(ctx, MCW_ERR_ARG, "impurity table: repeated wavelength");
    }
    total += 4 * (size_t)imp->n;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // device lookups binary-search the wavelengths: store every table sorted
    // ascending and require distinct wavelengths
    auto order_of = [](const mcw_ssp_table &t, std::vector<int32_t> &ord) -> bool {
        ord.resize(t.n);
        for (int32_t i = 0; i < t.n; ++i) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return t.wvl[a] < t.wvl[b]; });
        for (int32_t i = 1; i < t.n; ++i)
            if (!(t.wvl[ord[i]] > t.wvl[ord[i - 1]])) return false;
        return true;
    };
    std::vector<double> host(total);
    std::vector<DevTable> tabs(n_ice);
    CUDA_TRY(ctx, ctx->tabdata.ensure(total * sizeof(double)));
    CUDA_TRY(ctx, ctx->ice_tables.ensure(n_ice * sizeof(DevTable)));
    const double *dbase = (const double *)ctx->tabdata.p;
    size_t o = 0;
    std::vector<int32_t> ord;
    auto put = [&](const mcw_ssp_table &t, DevTable &d) {
        const int32_t n = t.n;
        order_of(t, ord);
        for (int32_t i = 0; i < n; ++i) {
            host[o + i] = t.wvl[ord[i]];
            host[o + n + i] = t.ss_alb[ord[i]];
            host[o + 2 * n + i] = t.ext_cff_mss[ord[i]];
            host[o + 3 * n + i] = t.asm_prm ? t.asm_prm[ord[i]] : 0.0;
        }
        d.wvl = dbase + o;
        d.ssa = dbase + o + n;
        d.ext = dbase + o + 2 * n;
        d.asm_ = dbase + o + 3 * n;
        d.n = n;
        d.unit = t.wvl_unit;
        o += 4 * (size_t)n;
    };
    for (int32_t i = 0; i < n_ice; ++i) put(ice[i], tabs[i]);
    DevTable dimp{};
    put(*imp, dimp);
    CUDA_TRY(ctx, cudaMemcpy(ctx->tabdata.p, host.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(ctx->ice_tables.p, tabs.data(), n_ice * sizeof(DevTable), cudaMemcpyHostToDevice));
    ctx->h_tab = host;
    ctx->h_ice = tabs;
    ctx->h_ice_aniso.assign(n_ice, 0);
    for (int32_t i = 0; i < n_ice; ++i) {
        bool pos = true, neg = true;
        for (int32_t k = 0; k < ice[i].n; ++k) {
            pos = pos && ice[i].asm_prm[k] > 1e-3;
            neg = neg && ice[i].asm_prm[k] < -1e-3;
        }
        ctx->h_ice_aniso[i] = (pos || neg) ? 1 : 0;
    }
    ctx->imp = dimp;
    ctx->n_ice = n_ice;
    ctx->max_ice_n = 0;
    for (int32_t i = 0; i < n_ice; ++i) ctx->max_ice_n = std::max(ctx->max_ice_n, ice[i].n);
    ctx->ice_order.assign(n_ice, {});
    for (int32_t i = 0; i < n_ice; ++i) order_of(ice[i], ctx->ice_order[i]);
    ctx->phase_rows.assign(n_ice, 0);   // phase matrices belong to the previous tables
    ctx->have_tables = true;
    ctx->tables_version++;
    return MCW_OK;
}

int mcw_set_phase_matrices(mcw_ctx *ctx, const mcw_phase_table *tabs, int32_t n) {
    if (!ctx) return MCW_ERR_ARG;
    if (!ctx->have_tables) return set_err(ctx, MCW_ERR_STATE, "call mcw_set_tables first");
    if (!tabs || n != ctx->n_ice) return set_err(ctx, MCW_ERR_ARG, "need one phase table per ice table (%d)", ctx->n_ice);
    size_t total = 0;
    for (int32_t t = 0; t < n; ++t) {
        const mcw_phase_table &p = tabs[t];
        if (p.n_rows == 0) continue;
        if (p.n_rows != (int32_t)ctx->ice_order[t].size())
            return set_err(ctx, MCW_ERR_ARG, "phase table %d: n_rows must equal the ice table's rows", t);
        if (!p.a1 || !p.a2 || !p.b1 || !p.b2) return set_err(ctx, MCW_ERR_ARG, "phase table %d: missing maxima", t);
        if (!(p.cos_min <= p.cos_cutoff && p.cos_cutoff <= p.cos_max))
            return set_err(ctx, MCW_ERR_ARG, "phase table %d: cos_cutoff outside [cos_min, cos_max]", t);
        for (int e = 0; e < 6; ++e) {
            const int32_t m = p.n_angle[e];
            if (m < 2 || !p.cos_asc[e] || !p.p_asc[e]) return set_err(ctx, MCW_ERR_ARG, "phase table %d: element %d", t, e);
            for (int32_t j = 0; j < m; ++j) {
                if (!std::isfinite(p.cos_asc[e][j]) || (j > 0 && !(p.cos_asc[e][j] > p.cos_asc[e][j - 1])))
                    return set_err(ctx, MCW_ERR_ARG, "phase table %d: cos_asc[%d] must rise strictly", t, e);
            }
            if (p.cos_asc[e][0] > p.cos_min || p.cos_asc[e][m - 1] < p.cos_max)
                return set_err(ctx, MCW_ERR_ARG, "phase table %d: cos_asc[%d] must cover [cos_min, cos_max]", t, e);
            for (size_t k = 0; k < (size_t)p.n_rows * m; ++k) {
                const double v = p.p_asc[e][k];
                if (!std::isfinite(v) || (e == 0 && !(v > 0)))
                    return set_err(ctx, MCW_ERR_ARG, "phase table %d: element %d must be finite (P11 > 0)", t, e);
            }
            total += (size_t)m * (1 + p.n_rows);
        }
        total += 4 * (size_t)p.n_rows;
    }
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<double> host(std::max<size_t>(total, 1));
    std::vector<DevPhase> dev(n);
    CUDA_TRY(ctx, ctx->phasedata.ensure(host.size() * sizeof(double)));
    CUDA_TRY(ctx, ctx->phase_tables.ensure(n * sizeof(DevPhase)));
    const double *dbase = (const double *)ctx->phasedata.p;
    size_t o = 0;
    for (int32_t t = 0; t < n; ++t) {
        const mcw_phase_table &p = tabs[t];
        DevPhase d{};
        d.n_rows = p.n_rows;
        if (p.n_rows > 0) {
            // rows follow the device table, which mcw_set_tables stored in ascending wavelength
            const std::vector<int32_t> &ord = ctx->ice_order[t];
            for (int e = 0; e < 6; ++e) {
                const int32_t m = p.n_angle[e];
                d.n_angle[e] = m;
                memcpy(&host[o], p.cos_asc[e], m * sizeof(double));
                d.cos_asc[e] = dbase + o;
                o += m;
                for (int32_t r = 0; r < p.n_rows; ++r)
                    memcpy(&host[o + (size_t)r * m], p.p_asc[e] + (size_t)ord[r] * m, m * sizeof(double));
                d.p_asc[e] = dbase + o;
                o += (size_t)m * p.n_rows;
            }
            const double *src[4] = {p.a1, p.a2, p.b1, p.b2};
            const double **dst[4] = {&d.a1, &d.a2, &d.b1, &d.b2};
            for (int k = 0; k < 4; ++k) {
                for (int32_t r = 0; r < p.n_rows; ++r) host[o + r] = src[k][ord[r]];
                *dst[k] = dbase + o;
                o += p.n_rows;
            }
            d.cos_max = p.cos_max;
            d.cos_min = p.cos_min;
            d.cos_cutoff = p.cos_cutoff;
        }
        dev[t] = d;
    }
    CUDA_TRY(ctx, cudaMemcpy(ctx->phasedata.p, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(ctx->phase_tables.p, dev.data(), n * sizeof(DevPhase), cudaMemcpyHostToDevice));
    // float copies for the FP32 polarised walk, same layout
    std::vector<float> host32(host.begin(), host.end());
    std::vector<DevPhase32> dev32(n);
    CUDA_TRY(ctx, ctx->phasedata32.ensure(host32.size() * sizeof(float)));
    CUDA_TRY(ctx, ctx->phase_tables32.ensure(n * sizeof(DevPhase32)));
    const float *fbase = (const float *)ctx->phasedata32.p;
    auto f32 = [&](const double *p) { return p ? fbase + (p - dbase) : nullptr; };
    std::vector<uint16_t> seeds((size_t)n * kPhaseBuckets, 0);
    CUDA_TRY(ctx, ctx->phase_seeds.ensure(seeds.size() * sizeof(uint16_t)));
    for (int32_t t = 0; t < n; ++t) {
        const DevPhase &d = dev[t];
        DevPhase32 f{};
        for (int e = 0; e < 6; ++e) {
            f.cos_asc[e] = f32(d.cos_asc[e]);
            f.p_asc[e] = f32(d.p_asc[e]);
            f.n_angle[e] = d.n_angle[e];
        }
        f.a1 = f32(d.a1); f.a2 = f32(d.a2); f.b1 = f32(d.b1); f.b2 = f32(d.b2);
        f.n_rows = d.n_rows;
        f.shared_grid = 0;
        if (d.n_rows > 0) {
            const mcw_phase_table &p = tabs[t];
            bool same = true;
            for (int e = 1; e < 6 && same; ++e)
                same = p.n_angle[e] == p.n_angle[0] &&
                       memcmp(p.cos_asc[e], p.cos_asc[0], p.n_angle[0] * sizeof(double)) == 0;
            f.shared_grid = same ? 1 : 0;
            if (same && p.n_angle[0] <= 65535) {
                // bucket seeds on the float copy of the grid (what the kernel compares)
                const int32_t m = p.n_angle[0];
                const float lo = (float)p.cos_asc[0][0], hi = (float)p.cos_asc[0][m - 1];
                const float scale = (float)kPhaseBuckets / (hi - lo);
                uint16_t *sd = &seeds[(size_t)t * kPhaseBuckets];
                int32_t j = 0;
                for (int b = 0; b < kPhaseBuckets; ++b) {
                    const float edge = lo + (float)b / scale;
                    while (j < m && (float)p.cos_asc[0][j] < edge) ++j;
                    sd[b] = (uint16_t)j;
                }
                f.seed = (const uint16_t *)ctx->phase_seeds.p + (size_t)t * kPhaseBuckets;
                f.seed_lo = lo;
                f.seed_scale = scale;
            }
        }
        f.cos_max = (float)d.cos_max;
        f.cos_min = (float)d.cos_min;
        f.cos_cutoff = (float)d.cos_cutoff;
        dev32[t] = f;
    }
    CUDA_TRY(ctx, cudaMemcpy(ctx->phasedata32.p, host32.data(), host32.size() * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(ctx->phase_seeds.p, seeds.data(), seeds.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(ctx->phase_tables32.p, dev32.data(), n * sizeof(DevPhase32), cudaMemcpyHostToDevice));
    for (int32_t t = 0; t < n; ++t) ctx->phase_rows[t] = tabs[t].n_rows;
    return MCW_OK;
}

int mcw_set_launch(mcw_ctx *ctx, const mcw_launch *l) {
    if (!ctx || !l) return MCW_ERR_ARG;
    if (l->block_size < 32 || l->block_size > 256 || l->block_size % 32)
        return set_err(ctx, MCW_ERR_ARG, "block_size must be a multiple of 32 in [32, 256]");
    if (l->blocks_per_sm < 0 || l->blocks_per_sm > 64) return set_err(ctx, MCW_ERR_ARG, "blocks_per_sm must be in [0, 64]");
    if (l->regen_chunk < 1 || l->regen_chunk > 32) return set_err(ctx, MCW_ERR_ARG, "regen_chunk must be in [1, 32]");
    if (l->drain_from != 0 && (l->drain_from < 256 || l->drain_from > (1 << 30)))
        return set_err(ctx, MCW_ERR_ARG, "drain_from must be 0 (off) or in [256, 2^30]");
    ctx->launch = *l;
    return MCW_OK;
}

int mcw_get_launch(const mcw_ctx *ctx, mcw_launch *l) {
    if (!ctx || !l) return MCW_ERR_ARG;
    *l = ctx->launch;
    return MCW_OK;
}

int mcw_set_budget(mcw_ctx *ctx, double seconds) {
    if (!ctx) return MCW_ERR_ARG;
    if (!(seconds > 0) || !std::isfinite(seconds)) return set_err(ctx, MCW_ERR_ARG, "budget must be > 0 s");
    ctx->budget_s = seconds;
    return MCW_OK;
}

int mcw_walk(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, uint64_t seed, int32_t mode, void *records,
             int32_t records_where, mcw_tally *tallies, mcw_stats *stats) {
    if (!ctx) return MCW_ERR_ARG;
    const auto t_start = std::chrono::steady_clock::now();
    if (!ctx->have_tables) return set_err(ctx, MCW_ERR_STATE, "mcw_set_tables has not been called");
    if (mode != MCW_MODE_F32 && mode != MCW_MODE_REPLAY64 && mode != MCW_MODE_POL64 && mode != MCW_MODE_POL32)
        return set_err(ctx, MCW_ERR_ARG, "unknown mode %d", mode);
    if (records_where < MCW_RECORDS_NONE || records_where > MCW_RECORDS_DEVICE)
        return set_err(ctx, MCW_ERR_ARG, "unknown records_where %d", records_where);
    if (records_where != MCW_RECORDS_NONE && !records) return set_err(ctx, MCW_ERR_ARG, "records is NULL");
    if (records_where == MCW_RECORDS_DEVICE && ((uintptr_t)records % 16) != 0)
        return set_err(ctx, MCW_ERR_ARG, "device records must be 16-byte aligned");
    Plan plan;
    int rc = make_plan(ctx, cfgs, n_cfg, mode, plan);
    if (rc) return rc;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t rec_size = (mode == MCW_MODE_F32)     ? sizeof(mcw_record32)
                            : (mode == MCW_MODE_POL64) ? sizeof(mcw_record64p)
                            : (mode == MCW_MODE_POL32) ? sizeof(mcw_record32p)
                                                       : sizeof(mcw_record64);
    void *dev_records = nullptr;
    if (records_where == MCW_RECORDS_DEVICE) dev_records = records;
    bool direct = false;   // host records written by the kernels themselves
    if (records_where == MCW_RECORDS_HOST && plan.total > 0) {
        // pinned host memory the device can address (mcw_host_alloc, cudaHostAlloc,
        // cudaHostRegister): the walk writes the records straight into it over the
        // host link, so no copy follows the kernel.  Otherwise a device buffer and a copy.
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, records) == cudaSuccess && at.type == cudaMemoryTypeHost &&
            at.devicePointer && ((uintptr_t)at.devicePointer % 16) == 0) {
            dev_records = at.devicePointer;
            direct = true;
        } else {
            (void)cudaGetLastError();
            CUDA_TRY(ctx, ctx->records.ensure((size_t)plan.total * rec_size));
            dev_records = ctx->records.p;
        }
    }
    // the launch shape first (occupancy queries, allocations): once the copies and
    // kernels below are queued, nothing on the host stands between them
    Shape shape{0, 0, 0, 0};
    if (mode == MCW_MODE_F32) shape = pick_shape(ctx, ctx->launch, plan);
    uint64_t h2d = 0;
    // a call on the configs and tables of the previous F32 / POL32 call finds their
    // launch data and lookup table in place: no upload, and the lookup-table kernel
    // only clears the counters and tallies
    const bool lut_mode = (mode == MCW_MODE_F32 || mode == MCW_MODE_POL32);
    std::vector<unsigned char> pb;
    if (lut_mode) pb = plan_bytes(plan);
    const bool cached = lut_mode && !ctx->lut_plan.empty() && ctx->lut_tables_version == ctx->tables_version &&
                        ctx->lut_cfgs_ptr == ctx->cfgs.p && ctx->lut_ptr == ctx->lut.p && ctx->lut_plan == pb;
    if (cached) {
        CUDA_TRY(ctx, ctx->tallies.ensure((size_t)n_cfg * sizeof(mcw_tally)));
        CUDA_TRY(ctx, ctx->counters.ensure(sizeof(Counters)));
        CUDA_TRY(ctx, cudaEventRecord(ctx->evs, st));
    } else {
        ctx->lut_plan.clear();   // the upload below replaces the launch data
        rc = upload_plan(ctx, plan, ctx->cfgs, ctx->lut, ctx->tallies, ctx->counters, st, ctx->evs, &h2d);
        if (rc) return rc;
    }
    auto lut_launch = [&]() -> int {
        LutArgs la = lut_args(ctx, plan, ctx->cfgs, ctx->lut, ctx->tallies, ctx->counters);
        la.clear_only = cached ? 1 : 0;
        CUDA_TRY(ctx, launch_lut(la, st));
        if (!cached) {
            ctx->lut_plan = pb;
            ctx->lut_tables_version = ctx->tables_version;
            ctx->lut_cfgs_ptr = ctx->cfgs.p;
            ctx->lut_ptr = ctx->lut.p;
        }
        return MCW_OK;
    };
    if (mode == MCW_MODE_F32) {
        WalkArgs wa = walk_args(ctx, plan, ctx->cfgs, ctx->lut, ctx->tallies, ctx->counters,
                                (mcw_record32 *)dev_records, shape.chunk, seed);
        rc = attach_drain(ctx, wa, ctx->drain, shape);
        if (rc) return rc;
        // the lookup-table kernel also clears the counters and tallies
        if ((rc = lut_launch())) return rc;
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
        if (plan.total > 0)
            CUDA_TRY(ctx, launch_walk_f32(wa, plan.impurity, shape.grid, shape.block, ctx->sm_count, st));
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, st));
    } else if (mode == MCW_MODE_POL32) {
        // the lookup-table kernel also clears the counters and tallies
        if ((rc = lut_launch())) return rc;
        WalkArgs wa = walk_args(ctx, plan, ctx->cfgs, ctx->lut, ctx->tallies, ctx->counters,
                                (mcw_record32 *)dev_records, 1, seed);
        wa.phase = (const DevPhase32 *)ctx->phase_tables32.p;
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
        CUDA_TRY(ctx, launch_walk_pol32(wa, ctx->sm_count, st));
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, st));
        shape.block = 128;
    } else {
        CUDA_TRY(ctx, cudaMemsetAsync(ctx->tallies.p, 0, n_cfg * sizeof(mcw_tally), st));
        CUDA_TRY(ctx, cudaMemsetAsync(ctx->counters.p, 0, sizeof(Counters), st));
        ReplayArgs ra;
        ra.cfgs = (const DevConfig *)ctx->cfgs.p;
        ra.prefix = (const int64_t *)((const char *)ctx->cfgs.p + prefix_offset(plan.cfgs.size()));
        ra.n_cfg = n_cfg;
        ra.pol = (mode == MCW_MODE_POL64) ? 1 : 0;
        ra.phase = (const DevPhase *)ctx->phase_tables.p;
        ra.total = plan.total;
        ra.imp = ctx->imp;
        ra.ice = (const DevTable *)ctx->ice_tables.p;
        Counters *cn = (Counters *)ctx->counters.p;
        ra.status = &cn->status;
        ra.records = dev_records;
        ra.tallies = (mcw_tally *)ctx->tallies.p;
        ra.budget_ns = (unsigned long long)(ctx->budget_s * 1e9);
        ra.seed = seed;
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
        CUDA_TRY(ctx, launch_walk_replay(ra, st));
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, st));
        shape.block = 128;
        shape.grid = (int)((plan.total + 127) / 128);
    }
    if (records_where == MCW_RECORDS_HOST && plan.total > 0 && !direct)
        CUDA_TRY(ctx, cudaMemcpyAsync(records, dev_records, (size_t)plan.total * rec_size, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, ctx->h_tallies.ensure(n_cfg * sizeof(mcw_tally)));
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_tallies.p, ctx->tallies.p, n_cfg * sizeof(mcw_tally), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_counters.p, ctx->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, cudaEventRecord(ctx->eve, st));
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    const mcw_tally *ht = (const mcw_tally *)ctx->h_tallies.p;
    if (tallies) memcpy(tallies, ht, n_cfg * sizeof(mcw_tally));
    const Counters *hc = (const Counters *)ctx->h_counters.p;
    float ms = 0.f, dev_ms = 0.f;
    CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    CUDA_TRY(ctx, cudaEventElapsedTime(&dev_ms, ctx->evs, ctx->eve));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->kernel_ms = ms;
        stats->device_ms = dev_ms;
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = n_cfg * sizeof(mcw_tally) + sizeof(Counters) +
                           ((records_where == MCW_RECORDS_HOST) ? (uint64_t)plan.total * rec_size : 0);
        for (int32_t c = 0; c < n_cfg; ++c) {
            for (int k = 1; k < 6; ++k) stats->n_photon += ht[c].n_cond[k];
            stats->n_events += ht[c].n_events;
            stats->max_n_scat = std::max(stats->max_n_scat, ht[c].max_n_scat);
        }
        stats->status = hc->status;
        stats->block_size = shape.block;
        stats->blocks_per_sm = shape.bps;
        stats->regen_chunk = shape.chunk;
        stats->grid = shape.grid;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    if (hc->status & kStatusBudget)
        return set_err(ctx, MCW_ERR_BUDGET, "walk stopped by the %.3g s time budget; results are partial", ctx->budget_s);
    if (hc->status & kStatusStream)
        return set_err(ctx, MCW_ERR_STREAM, "a replay photon exhausted its 2^33-uniform stream");
    return MCW_OK;
}

int mcw_post(mcw_ctx *ctx, const void *records, int32_t records_where, int32_t mode, int64_t n, int32_t n_cfg,
             int32_t n_bins, uint64_t *bin_wvn_fx, uint32_t *bin_count, mcw_post_stats *stats) {
    if (!ctx) return MCW_ERR_ARG;
    if (mode != MCW_MODE_F32 && mode != MCW_MODE_REPLAY64 && mode != MCW_MODE_POL64 && mode != MCW_MODE_POL32)
        return set_err(ctx, MCW_ERR_ARG, "unknown mode %d", mode);
    if (records_where != MCW_RECORDS_HOST && records_where != MCW_RECORDS_DEVICE)
        return set_err(ctx, MCW_ERR_ARG, "records must be on the host or the device");
    if (n < 0 || (n > 0 && !records) || n_cfg <= 0 || n_bins < 0 || n_bins > (1 << 20) || !stats ||
        (n_bins > 0 && (!bin_wvn_fx || !bin_count)))
        return set_err(ctx, MCW_ERR_ARG, "invalid post-processing arguments");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t rec_size = (mode == MCW_MODE_F32)     ? sizeof(mcw_record32)
                            : (mode == MCW_MODE_POL32) ? sizeof(mcw_record32p)
                            : (mode == MCW_MODE_POL64) ? sizeof(mcw_record64p)
                                                       : sizeof(mcw_record64);
    const bool f64 = (mode == MCW_MODE_REPLAY64 || mode == MCW_MODE_POL64);
    const size_t b_bins = (size_t)n_cfg * n_bins * sizeof(unsigned long long);
    const size_t b_cnt = (size_t)n_cfg * n_bins * sizeof(unsigned int);
    const size_t b_cnt_pad = (b_cnt + 255) & ~size_t(255);
    const size_t b_stats = (size_t)n_cfg * sizeof(mcw_post_stats);
    CUDA_TRY(ctx, ctx->post.ensure(b_bins + b_cnt_pad + b_stats));
    char *dev = (char *)ctx->post.p;
    const void *drec = records;
    if (records_where == MCW_RECORDS_HOST && n > 0) {
        CUDA_TRY(ctx, ctx->records.ensure((size_t)n * rec_size));
        CUDA_TRY(ctx, cudaMemcpyAsync(ctx->records.p, records, (size_t)n * rec_size, cudaMemcpyHostToDevice, st));
        drec = ctx->records.p;
    }
    CUDA_TRY(ctx, cudaMemsetAsync(dev, 0, b_bins + b_cnt_pad + b_stats, st));
    CUDA_TRY(ctx, launch_post(drec, f64, rec_size, n, n_cfg, n_bins, (unsigned long long *)dev,
                              (unsigned int *)(dev + b_bins), (mcw_post_stats *)(dev + b_bins + b_cnt_pad),
                              ctx->sm_count, st));
    if (n_bins > 0) {
        CUDA_TRY(ctx, cudaMemcpyAsync(bin_wvn_fx, dev, b_bins, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(ctx, cudaMemcpyAsync(bin_count, dev + b_bins, b_cnt, cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(stats, dev + b_bins + b_cnt_pad, b_stats, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return MCW_OK;
}

int mcw_brf(const mcw_tally *t, int32_t n_cfg, double *brf, double *albedo) {
    if (!t || n_cfg <= 0) return MCW_ERR_ARG;
    double w[MCW_HIST_NTHETA], wsum = 0;
    for (int i = 0; i < MCW_HIST_NTHETA; ++i) {
        const double mid = (i + 0.5) * (kPi / 2) / MCW_HIST_NTHETA;
        w[i] = std::sin(mid) * std::cos(mid);
        wsum += w[i];
    }
    for (int32_t c = 0; c < n_cfg; ++c) {
        double q_down = 0;
        for (int k = 1; k < 6; ++k) q_down += (double)t[c].q_cond_fx[k];
        if (albedo) albedo[c] = q_down > 0 ? (double)t[c].q_cond_fx[1] / q_down : 0.0;
        if (brf) {
            for (int i = 0; i < MCW_HIST_NTHETA; ++i)
                for (int j = 0; j < MCW_HIST_NPHI; ++j) {
                    const int b = i * MCW_HIST_NPHI + j;
                    const double wt = w[i] / (MCW_HIST_NPHI * wsum);
                    brf[(size_t)c * MCW_HIST_BINS + b] = q_down > 0 ? (double)t[c].bin_wvn_fx[b] / (q_down * wt) : 0.0;
                }
        }
    }
    return MCW_OK;
}

int mcw_autotune(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, uint64_t seed, mcw_launch *best,
                 double *best_ms) {
    if (!ctx || !cfgs || n_cfg <= 0) return MCW_ERR_ARG;
    const mcw_launch saved = ctx->launch;
    bool imp_any = false;
    for (int32_t i = 0; i < n_cfg; ++i) imp_any = imp_any || cfgs[i].imp_cnc > 0;
    const int blocks[] = {128, 256};
    const int chunks[] = {1, 4, 8, 16, 32};
    mcw_launch win = saved;
    double win_ms = 1e300;
    for (int b : blocks) {
        const int occ = std::max(1, walk_f32_max_blocks_per_sm(b, n_cfg, imp_any));
        const int bps_opts[] = {occ, std::max(1, occ / 2)};
        for (int bi = 0; bi < 2; ++bi) {
            if (bi == 1 && bps_opts[1] == bps_opts[0]) continue;
            for (int ch : chunks) {
                mcw_launch l{b, bps_opts[bi], ch, saved.drain_from};
                ctx->launch = l;
                mcw_stats s;
                double t = 0;
                for (int rep = 0; rep < 2; ++rep) {
                    int rc = mcw_walk(ctx, cfgs, n_cfg, seed + rep, MCW_MODE_F32, nullptr, MCW_RECORDS_NONE, nullptr, &s);
                    if (rc) {
                        ctx->launch = saved;
                        return rc;
                    }
                    if (rep) t = s.kernel_ms;
                }
                if (t < win_ms) {
                    win_ms = t;
                    win = l;
                }
            }
        }
    }
    // then the drain handover for the winning shape
    const int32_t drains[] = {0, 512, 1024, 4096};
    const mcw_launch shape = win;
    for (int32_t d : drains) {
        if (d == shape.drain_from) continue;
        mcw_launch l = shape;
        l.drain_from = d;
        ctx->launch = l;
        mcw_stats s;
        double t = 0;
        for (int rep = 0; rep < 2; ++rep) {
            int rc = mcw_walk(ctx, cfgs, n_cfg, seed + rep, MCW_MODE_F32, nullptr, MCW_RECORDS_NONE, nullptr, &s);
            if (rc) {
                ctx->launch = saved;
                return rc;
            }
            if (rep) t = s.kernel_ms;
        }
        if (t < win_ms) {
            win_ms = t;
            win = l;
        }
    }
    ctx->launch = win;
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return MCW_OK;
}

int mcw_graph_create(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, mcw_record32 *device_records,
                     mcw_graph **out) {
    if (!ctx || !out) return MCW_ERR_ARG;
    *out = nullptr;
    if (!ctx->have_tables) return set_err(ctx, MCW_ERR_STATE, "mcw_set_tables has not been called");
    if (device_records && ((uintptr_t)device_records % 16) != 0)
        return set_err(ctx, MCW_ERR_ARG, "device records must be 16-byte aligned");
    Plan plan;
    int rc = make_plan(ctx, cfgs, n_cfg, MCW_MODE_F32, plan);
    if (rc) return rc;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mcw_graph *g = new (std::nothrow) mcw_graph();
    if (!g) return set_err(ctx, MCW_ERR_OOM, "out of host memory");
    g->ctx = ctx;
    g->n_cfg = n_cfg;
    g->total = plan.total;
    cudaStream_t st = ctx->stream;
    auto fail = [&](int code) {
        mcw_graph_destroy(g);
        return code;
    };
    rc = upload_plan(ctx, plan, g->cfgs, g->lut, g->tallies, g->counters, st);
    if (rc) return fail(rc);
    if (g->h_tallies.ensure(n_cfg * sizeof(mcw_tally)) != cudaSuccess || g->h_counters.ensure(sizeof(Counters)) != cudaSuccess)
        return fail(set_err(ctx, MCW_ERR_OOM, "pinned allocation failed"));
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(set_err(ctx, MCW_ERR_CUDA, "upload failed"));
    const Shape shape = pick_shape(ctx, ctx->launch, plan);
    g->grid = shape.grid;
    g->block = shape.block;
    g->args = walk_args(ctx, plan, g->cfgs, g->lut, g->tallies, g->counters, device_records, shape.chunk, 0);
    rc = attach_drain(ctx, g->args, g->drain, shape);
    if (rc) return fail(rc);
    const LutArgs la = lut_args(ctx, plan, g->cfgs, g->lut, g->tallies, g->counters);
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(set_err(ctx, MCW_ERR_CUDA, "stream capture failed to start"));
    cudaError_t e = launch_lut(la, st);  // clears counters and tallies too
    if (e == cudaSuccess && plan.total > 0)
        e = launch_walk_f32(g->args, plan.impurity, g->grid, g->block, ctx->sm_count, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->h_tallies.p, g->tallies.p, n_cfg * sizeof(mcw_tally), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->h_counters.p, g->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, st);
    cudaError_t e2 = cudaStreamEndCapture(st, &g->graph);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(set_err(ctx, MCW_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2)));
    // locate the walk kernel node so each launch can set its seed
    size_t n_nodes = 0;
    cudaGraphGetNodes(g->graph, nullptr, &n_nodes);
    std::vector<cudaGraphNode_t> nodes(n_nodes);
    cudaGraphGetNodes(g->graph, nodes.data(), &n_nodes);
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) != cudaSuccess || ty != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p;
        if (cudaGraphKernelNodeGetParams(nd, &p) != cudaSuccess) continue;
        if (walk_f32_is_kernel(p.func)) {
            g->walk_nodes.push_back(nd);
            g->walk_params.push_back(p);
        }
    }
    if (plan.total > 0 && g->walk_nodes.empty()) return fail(set_err(ctx, MCW_ERR_CUDA, "walk node not found in graph"));
    if (cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
        return fail(set_err(ctx, MCW_ERR_CUDA, "graph instantiation failed"));
    *out = g;
    return MCW_OK;
}

int mcw_graph_launch(mcw_graph *g, uint64_t seed, mcw_tally *tallies, mcw_stats *stats) {
    if (!g || !g->ctx) return MCW_ERR_ARG;
    mcw_ctx *ctx = g->ctx;
    const auto t_start = std::chrono::steady_clock::now();
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    g->args.keys = philox_schedule(seed);
    for (size_t i = 0; i < g->walk_nodes.size(); ++i) {
        void *kp[1] = {&g->args};
        cudaKernelNodeParams p = g->walk_params[i];
        p.kernelParams = kp;
        p.extra = nullptr;
        CUDA_TRY(ctx, cudaGraphExecKernelNodeSetParams(g->exec, g->walk_nodes[i], &p));
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
    CUDA_TRY(ctx, cudaGraphLaunch(g->exec, st));
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, st));
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    const mcw_tally *ht = (const mcw_tally *)g->h_tallies.p;
    if (tallies) memcpy(tallies, ht, g->n_cfg * sizeof(mcw_tally));
    const Counters *hc = (const Counters *)g->h_counters.p;
    if (stats) {
        float ms = 0.f;
        CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        memset(stats, 0, sizeof(*stats));
        stats->kernel_ms = ms;
        for (int32_t c = 0; c < g->n_cfg; ++c) {
            for (int k = 1; k < 6; ++k) stats->n_photon += ht[c].n_cond[k];
            stats->n_events += ht[c].n_events;
            stats->max_n_scat = std::max(stats->max_n_scat, ht[c].max_n_scat);
        }
        stats->status = hc->status;
        stats->block_size = g->block;
        stats->grid = g->grid;
        stats->regen_chunk = g->args.regen_chunk;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    if (hc->status & kStatusBudget)
        return set_err(ctx, MCW_ERR_BUDGET, "walk stopped by the %.3g s time budget; results are partial", ctx->budget_s);
    return MCW_OK;
}

int mcw_graph_destroy(mcw_graph *g) {
    if (!g) return MCW_OK;
    if (g->ctx) {
        cudaSetDevice(g->ctx->device);
        cudaStreamSynchronize(g->ctx->stream);
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    for (DevBuf *b : {&g->cfgs, &g->lut, &g->tallies, &g->counters, &g->drain}) b->release();
    g->h_tallies.release();
    g->h_counters.release();
    delete g;
    return MCW_OK;
}

int mcw_host_alloc(size_t bytes, void **out) {
    if (!out || bytes == 0) return MCW_ERR_ARG;
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? MCW_ERR_OOM : MCW_ERR_CUDA;
    return MCW_OK;
}

int mcw_host_free(void *p) {
    if (!p) return MCW_OK;
    return cudaFreeHost(p) == cudaSuccess ? MCW_OK : MCW_ERR_CUDA;
}

}  // extern "C"
