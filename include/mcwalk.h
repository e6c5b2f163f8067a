/*
 * mcwalk.h - C ABI of the GB300 photon random walk (libmcwalk.so).
 *
 * The library replaces the photon loop of monte_carloMPI's
 * MonteCarlo.run / MonteCarlo.monte_carlo3D (monte_carloMPI/monte_carlo3D.py)
 * and the MPI split/gather of monte_carloMPI/parallelize.py with CUDA
 * kernels on one GPU.  Every function returns an int status (MCW_OK or a
 * negative MCW_ERR_*); no exception, C++ type or torch type crosses this
 * boundary and every buffer is owned by the caller unless stated.  Calls on
 * one context are serialised on the context's CUDA stream and must not be
 * made concurrently from several threads.
 */
#ifndef MCWALK_H
#define MCWALK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCW_ABI_VERSION 3

/* status codes */
#define MCW_OK 0
#define MCW_ERR_ARG (-1)     /* invalid argument (reference: ValueError / bad kwargs) */
#define MCW_ERR_CUDA (-2)    /* a CUDA runtime call failed */
#define MCW_ERR_BUDGET (-3)  /* the kernel's time budget ran out; results are partial */
#define MCW_ERR_STREAM (-4)  /* a replay photon needed more than 2^33 uniforms */
#define MCW_ERR_OOM (-5)     /* device or pinned allocation failed */
#define MCW_ERR_STATE (-6)   /* call made in the wrong state (e.g. no SSP tables) */

/* walk modes */
#define MCW_MODE_F32 0       /* production: FP32 walk, Philox4x32-10 per (photon, step) */
#define MCW_MODE_REPLAY64 1  /* FP64 walk on the photon-indexed replay stream, reference order */
#define MCW_MODE_POL64 2     /* the polarised walk of aspherical grains (HG off): FP64, replay
                                stream, reference order; records mcw_record64p */
#define MCW_MODE_POL32 3     /* production polarised walk: FP32, a Philox4x32-10 stream per
                                photon; records mcw_record32p */

/* where mcw_walk writes per-photon records */
#define MCW_RECORDS_NONE 0
#define MCW_RECORDS_HOST 1   /* host pointer; pinned host memory (mcw_host_alloc, cudaHostAlloc,
                                cudaHostRegister) is written by the walk directly, other host
                                memory receives a device -> host copy after it */
#define MCW_RECORDS_DEVICE 2 /* device pointer owned by the caller */

/* exit-direction histogram: 18 zenith bins of 5 deg x 36 azimuth bins of 10 deg */
#define MCW_HIST_NTHETA 18
#define MCW_HIST_NPHI 36
#define MCW_HIST_BINS 648
/* wavenumber sums are fixed point: value = sum / 2^32 (exact, order-independent) */
#define MCW_WVN_FX_SCALE 4294967296.0

typedef struct mcw_ctx mcw_ctx;
typedef struct mcw_graph mcw_graph;

/* Units of mcw_ssp_table.wvl. */
#define MCW_WVL_METRES 0  /* the netCDF tables (monte_carlo3D.py:511-514, :666-671) */
#define MCW_WVL_MICRONS 1 /* the aspherical isca.dat rows (monte_carlo3D.py:215-236) */

/* One SSP table in the reference's netCDF layout (monte_carlo3D.py:511-514):
 * wvl (distinct; any order), ss_alb, ext_cff_mss [m^2/kg], asm_prm (NULL for
 * an impurity table).  Copied into device memory by mcw_set_tables. */
typedef struct {
    const double *wvl;
    const double *ss_alb;
    const double *ext_cff_mss;
    const double *asm_prm;
    int32_t n;
    int32_t wvl_unit;      /* MCW_WVL_METRES or MCW_WVL_MICRONS; wavelengths are compared
                              in this unit, as the reference compares them */
} mcw_ssp_table;

/* One run of MonteCarlo.run (monte_carlo3D.py:1492-1496) plus the model
 * kwargs it uses (:43-94).  Lengths in um, angles in degrees. */
typedef struct {
    int64_t n_photon;
    int64_t first_photon;          /* index of the first photon walked (shards of one run) */
    double wvl0;                   /* centre wavelength [um] */
    double half_width;             /* FWHM [um]; sigma = FWHM / 2.355 */
    double theta0_deg;             /* incident zenith angle */
    double tau_tot;                /* slab optical depth */
    double imp_cnc;                /* impurity mass fraction */
    double rho_snw;                /* snow density [kg/m^3] */
    double rho_ice;                /* ice density [kg/m^3] (bookkeeping) */
    double lambertian_reflectance; /* R of the Lambertian surface or bottom */
    int32_t lambertian_surface;
    int32_t lambertian_bottom;
    int32_t ice_table;             /* index into the ice tables of mcw_set_tables */
    int32_t ssp_nearest;           /* 0: the two nearest ice-table points, interpolated
                                      (spheres, monte_carlo3D.py:594-616); 1: the nearest
                                      point, and the photon's wavelength becomes that
                                      point's (HG-forced aspherical particles,
                                      :323-415, :1528-1545) */
    /* run(test=True) overrides (monte_carlo3D.py:1553-1573); NaN = use table */
    double ssa_ice_override;
    double g_override;
    double ext_ice_override;
    double ssa_imp_override;
    double ext_imp_override;
    /* 1: the polarised walk of aspherical grains (run(shape=...) with HG off): scattering
     * angles by rejection from the phase matrices of the ice table (mcw_set_phase_matrices)
     * and the photon's Stokes vector carried through every scattering (monte_carlo3D.py:
     * 905-1004, :1282-1342).  Needs ssp_nearest = 1 and MCW_MODE_POL64. */
    int32_t polarised;
    int32_t pad;
    double stokes0[4];             /* incident Stokes vector (I, Q, U, V), run(stokes_params=...) */
} mcw_config;

/* Per-photon answer of MCW_MODE_F32: the 7 CSV columns of
 * monte_carlo3D.py:1627-1636 plus the config index.  32 bytes. */
typedef struct {
    int32_t condition;  /* 1 top, 2 bottom diffuse, 3 bottom direct, 4 ice, 5 impurity */
    int32_t n_scat;
    float wvn;          /* 1 / lambda [um^-1] */
    float theta_n;
    float phi_n;        /* [0, 2 pi) */
    float path_length;  /* [m] */
    float snow_depth;   /* [m] */
    uint32_t config;
} mcw_record32;

/* Per-photon answer of MCW_MODE_REPLAY64.  flags bit 0: the reference's
 * quadrant test for phi_n fails (mux or muy exactly 0, monte_carlo3D.py:
 * 1472-1485); phi_n is NaN then. */
typedef struct {
    int32_t condition;
    int32_t n_scat;
    double wvn;
    double theta_n;
    double phi_n;
    double path_length;
    double snow_depth;
    uint32_t config;
    uint32_t flags;
} mcw_record64;

/* Per-photon answer of MCW_MODE_POL64: mcw_record64's fields and the final
 * Stokes vector's Q, U, V divided by I (the CSV's Q_n, U_n, V_n,
 * monte_carlo3D.py:1637-1646).  80 bytes. */
typedef struct {
    int32_t condition;
    int32_t n_scat;
    double wvn;
    double theta_n;
    double phi_n;
    double path_length;
    double snow_depth;
    uint32_t config;
    uint32_t flags;
    double stokes_q;
    double stokes_u;
    double stokes_v;
} mcw_record64p;

/* Per-photon answer of MCW_MODE_POL32: mcw_record32's fields and Q_n, U_n,
 * V_n.  48 bytes. */
typedef struct {
    int32_t condition;
    int32_t n_scat;
    float wvn;
    float theta_n;
    float phi_n;
    float path_length;
    float snow_depth;
    uint32_t config;
    float stokes_q;
    float stokes_u;
    float stokes_v;
    float pad;
} mcw_record32p;

/* Phase matrices of the polarised walk for one ice table (one row per table
 * row, in the order the table was given to mcw_set_tables), as
 * interpolate_phase_matrix (monte_carlo3D.py:819-883) prepares them: element e
 * (P11, P12, P22, P33, P43, P44) tabulated at cos_asc[e] (cos of the file's
 * scattering angles, strictly ascending, n_angle[e] points) with values
 * p_asc[e][row * n_angle[e] + j] (P12 ... P44 multiplied by P11; P11 > 0).
 * The rejection sampler's two areas meet at cos_cutoff in [cos_min, cos_max];
 * a1 / a2 hold each row's largest |P11| over the first (cos >= cos_cutoff) and
 * second area, b1 / b2 the same for |P12| (:929-947).  Host pointers, copied. */
typedef struct {
    int32_t n_rows;
    int32_t n_angle[6];
    int32_t pad;
    const double *cos_asc[6];
    const double *p_asc[6];
    const double *a1, *a2, *b1, *b2;
    double cos_max, cos_min, cos_cutoff;
} mcw_phase_table;

/* Per-config totals and the condition-1 exit histogram; the inputs of the
 * BRF and albedo of post_processing.py:73-81,125-128 and monte_carlo3D.py:
 * 1659-1671. */
typedef struct {
    uint64_t n_cond[6];          /* photons per end condition (index 0 unused) */
    uint64_t q_cond_fx[6];       /* sum of wvn per end condition, fixed point */
    uint64_t n_events;           /* sum of n_scat */
    uint32_t max_n_scat;
    uint32_t reserved;
    uint64_t bin_wvn_fx[MCW_HIST_BINS]; /* condition-1 wvn sum per (theta, phi) bin */
    uint32_t bin_count[MCW_HIST_BINS];  /* condition-1 photons per bin */
} mcw_tally;

typedef struct {
    double kernel_ms;      /* walk kernel, CUDA events on the context stream */
    double total_ms;       /* whole call, host wall clock */
    double device_ms;      /* first to last device operation of the call (CUDA events) */
    uint64_t h2d_bytes;    /* host -> device bytes copied by the call */
    uint64_t d2h_bytes;    /* device -> host bytes copied by the call */
    uint64_t n_photon;
    uint64_t n_events;
    uint32_t max_n_scat;
    uint32_t status;       /* device status bits (1 budget, 2 stream overrun) */
    int32_t block_size;
    int32_t blocks_per_sm;
    int32_t regen_chunk;
    int32_t grid;
} mcw_stats;

/* Launch shape of the FP32 walk (persistent grid). */
typedef struct {
    int32_t block_size;    /* threads per block, multiple of 32, 32..256 */
    int32_t blocks_per_sm; /* resident blocks per SM to launch (0 = occupancy maximum) */
    int32_t regen_chunk;   /* refill a warp once this many lanes are idle (1..32) */
    int32_t drain_from;    /* once every photon has started, a photon past this many steps
                              leaves the walk for a queue walked after it by a whole thread
                              block per photon (0 = never; else 256..2^30; default 4096).
                              Records do not depend on it. */
} mcw_launch;

/* Library identity.  No reference counterpart. */
int mcw_abi_version(void);
const char *mcw_version(void);

/* Context on one device: stream, workspace and tables.  Replaces the per-rank
 * MonteCarlo instance (monte_carlo3D.py:43-94) and parallelize.Parallel
 * (parallelize.py:6-12). */
int mcw_create(int device, mcw_ctx **out);
int mcw_destroy(mcw_ctx *ctx);

/* Last error message of the context (NUL-terminated, truncated to len). */
int mcw_last_error(const mcw_ctx *ctx, char *buf, size_t len);

/* Upload SSP tables: n_ice ice tables (one per grain size, ice_wrn_%04d.nc)
 * and one impurity table.  Replaces the netCDF reads of
 * get_optical_properties (monte_carlo3D.py:498-514) and get_impurity_optics
 * (:661-671); the per-photon interpolation (:594-658, :688-777) runs on the
 * device. */
int mcw_set_tables(mcw_ctx *ctx, const mcw_ssp_table *ice, int32_t n_ice,
                   const mcw_ssp_table *imp);

/* Attach phase matrices to the ice tables of the last mcw_set_tables: tabs[i]
 * belongs to ice table i (n = n_ice; n_rows 0 = none).  Replaces the P11.dat ...
 * P44.dat reads of get_aspherical_SSPs (monte_carlo3D.py:145-171, :267-475). */
int mcw_set_phase_matrices(mcw_ctx *ctx, const mcw_phase_table *tabs, int32_t n);

/* Launch shape and time budget of later walks.  The budget of a new context
 * (and of every mcw_walk_noalloc call) is MCW_DEFAULT_BUDGET_S: a walk still
 * running after it stops, and the call returns MCW_ERR_BUDGET. */
#define MCW_DEFAULT_BUDGET_S 300.0
int mcw_set_launch(mcw_ctx *ctx, const mcw_launch *launch);
int mcw_get_launch(const mcw_ctx *ctx, mcw_launch *launch);
int mcw_set_budget(mcw_ctx *ctx, double seconds);

/* Walk every photon of n_cfg configurations in one launch.  Replaces
 * MonteCarlo.run's photon loop and gather (monte_carlo3D.py:1515-1619,
 * parallelize.py:14-41) and monte_carlo3D (:1111-1490).  Photon p of config c
 * (p = 0 .. n_photon-1) is record sum(n_photon[:c]) + p; its random streams
 * are keyed by (seed, c << 40 | (first_photon + p)), so a run split into
 * shards by first_photon gives the same photons as the whole run.
 * records: mcw_record32 (F32), mcw_record64 (REPLAY64), mcw_record64p (POL64)
 * or mcw_record32p (POL32), or NULL with MCW_RECORDS_NONE.  Polarised configs
 * walk in MCW_MODE_POL32 or MCW_MODE_POL64 only, and those modes walk polarised
 * configs only.  tallies: n_cfg host structs or NULL.  stats: or NULL. */
int mcw_walk(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, uint64_t seed, int32_t mode,
             void *records, int32_t records_where, mcw_tally *tallies, mcw_stats *stats);

/* BRF and albedo of tallies: brf[c*648 + t*36 + p] = h / (Q_down * w_t) with
 * w_t = sin(theta_t) cos(theta_t) / (36 * sum_t sin cos) at bin midpoints,
 * and albedo[c] = Q_up / Q_down.  2-D form of post_processing.py:73-81;
 * albedo as monte_carlo3D.py:1659-1671.  Either output may be NULL. */
int mcw_brf(const mcw_tally *tallies, int32_t n_cfg, double *brf, double *albedo);

/* Time launch shapes on (a sample of) these configs and keep the fastest in
 * the context: block size, resident blocks and refill chunk first, then
 * drain_from (0, 512, 1024, 4096) for that shape.  No reference counterpart
 * (the reference has no tuning). */
int mcw_autotune(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg, uint64_t seed,
                 mcw_launch *best, double *best_ms);

/* Capture one F32 sweep (counter reset, SSP LUT, walk, tally copy-out) in a
 * CUDA graph and replay it with a new seed per launch.  device_records may be
 * NULL.  Replaces repeated MonteCarlo.run calls of the driver's sweeps
 * (monte_carlo3D-run.py:60-122). */
int mcw_graph_create(mcw_ctx *ctx, const mcw_config *cfgs, int32_t n_cfg,
                     mcw_record32 *device_records, mcw_graph **out);
int mcw_graph_launch(mcw_graph *g, uint64_t seed, mcw_tally *tallies, mcw_stats *stats);
int mcw_graph_destroy(mcw_graph *g);

/* Pinned host memory for records (fast device -> host copies). */
int mcw_host_alloc(size_t bytes, void **out);
int mcw_host_free(void *p);

/* Per-photon CSV in the reference's format (monte_carlo3D.py:1627-1636):
 * header line, then "%d %r %r %r %d %r %r" rows with Python's shortest
 * round-trip float repr.  mode selects mcw_record32 / mcw_record64, or
 * mcw_record32p / mcw_record64p with the polarised walk's header and three
 * more columns (Q_n, U_n, V_n, :1637-1646).
 * mcw_format_csv writes into buf (cap bytes; *used = bytes needed). */
int mcw_write_csv(const char *path, const void *records, int32_t mode, int64_t n,
                  int32_t n_threads);
int mcw_format_csv(const void *records, int32_t mode, int64_t n, int32_t header, char *buf,
                   size_t cap, size_t *used);

/* Per-config sums over records for the reference's post-processing. */
typedef struct {
    uint64_t q_cond_fx[6];     /* wvn sum per end condition, fixed point 2^-32 */
    uint64_t n_cond[6];        /* photons per end condition */
    uint64_t sum_n_scat;
    double sum_path_length;    /* [m] */
    double sum_wavelength;     /* sum of 1 / wvn [um] */
} mcw_post_stats;

/* Post-processing of records on the device (records: host or device pointer, see
 * records_where; mode selects mcw_record32 / mcw_record64 / mcw_record32p /
 * mcw_record64p, whose Stokes columns it does not read; photons are grouped by
 * their config field, which must be < n_cfg): the wvn-weighted condition-1 exit
 * zenith histogram with np.histogram's binning of [0, pi/2] into n_bins bins
 * (post_processing.py:73-77 brf, :132-134 polar BRFs), and per-config sums for
 * albedo, the albedo with transmitted photons, mean wavelength, mean n_scat and
 * mean path length (post_processing.py:250-312, :380-430; monte_carlo3D.py:
 * 1659-1671).  Outputs are host arrays: bin_wvn_fx and bin_count [n_cfg * n_bins]
 * (may be NULL when n_bins is 0), stats [n_cfg]. */
int mcw_post(mcw_ctx *ctx, const void *records, int32_t records_where, int32_t mode, int64_t n,
             int32_t n_cfg, int32_t n_bins, uint64_t *bin_wvn_fx, uint32_t *bin_count,
             mcw_post_stats *stats);

/* Largest wavelength lookup table mcw_walk_noalloc holds: grid points of
 * lambda = k / 100 um over wvl0 +- 6.5 sigma, so FWHM up to about 3.6 um. */
#define MCW_NOALLOC_MAX_LUT 2048

/* The F32 walk of one config for callers that cannot allocate device memory
 * (a plugin given buffers by a framework's own pool, a real-time loop that
 * must not reach the allocator).  No counterpart in the reference.  The caller
 * passes device buffers only: ice_dev / imp_dev hold DEVICE pointers to
 * ascending tables with distinct wavelengths (asm_prm may be NULL for the
 * impurity), records_dev (cfg->n_photon mcw_record32, 16-byte aligned) and
 * tally_dev may be NULL; stream is a cudaStream_t (NULL = default stream).
 * Allocates nothing: its scratch is a fixed device array of this library
 * (about 107 KB per GPU, held until the process exits) shared by all calls on
 * a device, so calls that overlap on the GPU race; the first call on a device
 * resolves the array's address and should come before any stream capture.
 * Sizes beyond MCW_NOALLOC_MAX_LUT return MCW_ERR_ARG; so do tables whose
 * wavelengths are not strictly ascending, whose values are not finite, or
 * whose ice extinction is not > 0 (checked on the device before the walk
 * starts).  The time budget is MCW_DEFAULT_BUDGET_S (MCW_ERR_BUDGET).
 * Same records and tally as mcw_walk with one config and this seed.
 * Synchronises the stream twice (after the table check and at the end). */
int mcw_walk_noalloc(const mcw_config *cfg, const mcw_ssp_table *ice_dev, const mcw_ssp_table *imp_dev,
                     uint64_t seed, mcw_record32 *records_dev, mcw_tally *tally_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MCWALK_H */
