/*
 * CPU restatement of the reference photon random walk, in plain C (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke check
 * and the CPU-baseline leg of bench.py load it (through ctypes) to check the
 * CUDA kernels and to time a CPU implementation of the same path.  Nothing in
 * the product links or calls it.
 *
 * Parity is pinned: the .npz fixtures under tests/golden hold per-photon answers of the
 * unmodified reference (monte_carloMPI/monte_carlo3D.py) run on the same
 * replay stream, and tests/test_oracle.py checks this file against them.
 *
 * Each function cites the reference lines it restates.  The arithmetic keeps
 * the reference's operation order; compile with -ffp-contract=off so no
 * multiply-add is fused.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>

#ifdef ORC_ULP_PERTURB
/* Test build only (liboracle_walk_ulp.so): log, sin and cos results moved by one
 * ulp up or down (or left alone), chosen by a hash of the argument.  It stands in
 * for a different libm (CUDA's on the GPU against glibc here), to measure how far
 * one-ulp differences carry through the walk. */
static double orc_ulp_(double r, double x)
{
    union { double d; uint64_t u; } a;
    a.d = x;
    const int k = (int)((a.u * 0x9E3779B97F4A7C15ull) >> 62);
    return k == 1 ? nextafter(r, INFINITY) : k == 2 ? nextafter(r, -INFINITY) : r;
}
static double orc_log_(double x) { return orc_ulp_(log(x), x); }
static double orc_sin_(double x) { return orc_ulp_(sin(x), x); }
static double orc_cos_(double x) { return orc_ulp_(cos(x), x); }
#define log(x) orc_log_(x)
#define sin(x) orc_sin_(x)
#define cos(x) orc_cos_(x)
#endif
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_TAG_WALK 0u
#define ORC_TAG_WVL 1u

static const double ORC_PI = 3.141592653589793;
static const double ORC_TWO_PI = 6.283185307179586; /* 2*np.pi, monte_carlo3D.py:26 */

/* ---------------------------------------------------------------- Philox */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform k of stream `tag` for `photon`: block k>>1, 64-bit word k&1,
 * ((word >> 12) + 0.5) * 2^-52 in [2^-53, 1 - 2^-53]. */
double orc_uniform(uint64_t seed, uint32_t tag, uint64_t photon, uint64_t k)
{
    uint32_t ctr[4] = {(uint32_t)(k >> 1), tag, (uint32_t)photon, (uint32_t)(photon >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    orc_philox4x32_10(ctr, key, x);
    int j = (int)(k & 1u);
    uint64_t w = ((uint64_t)x[2 * j + 1] << 32) | x[2 * j];
    return ((double)(w >> 12) + 0.5) * 0x1p-52;
}

/* Sequential reader over one photon's walk stream. */
typedef struct {
    uint64_t seed, photon, k;
    int have;             /* block index cached in x[] */
    uint64_t block;
    uint32_t x[4];
} orc_stream;

static double stream_next(orc_stream *s)
{
    uint64_t b = s->k >> 1;
    if (!s->have || b != s->block) {
        uint32_t ctr[4] = {(uint32_t)b, ORC_TAG_WALK, (uint32_t)s->photon, (uint32_t)(s->photon >> 32)};
        uint32_t key[2] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32)};
        orc_philox4x32_10(ctr, key, s->x);
        s->block = b;
        s->have = 1;
    }
    int j = (int)(s->k & 1u);
    uint64_t w = ((uint64_t)s->x[2 * j + 1] << 32) | s->x[2 * j];
    s->k++;
    return ((double)(w >> 12) + 0.5) * 0x1p-52;
}

/* ---------------------------------------------------------------- types */
typedef struct {
    const double *wvl;   /* metres (netCDF tables) or micrometres (aspherical isca.dat rows) */
    const double *ssa;
    const double *ext;
    const double *asm_;  /* may be NULL (impurity) */
    int32_t n;
    int32_t unit;        /* 0: wvl in metres, 1: in micrometres */
} orc_table;

typedef struct {
    int64_t n_photon;
    double wvl0, half_width, theta0_deg, tau_tot, imp_cnc, rho_snw, rho_ice;
    int32_t lam_surface, lam_bottom;
    double R;
    /* run(test=True) overrides (monte_carlo3D.py:1553-1573); NaN = from table */
    double ssa_ice_override, g_override, ext_ice_override, ssa_imp_override, ext_imp_override;
    /* 1: the HG-forced aspherical lookup (monte_carlo3D.py:323-334, :396-415,
     * :1528-1549): the nearest ice-table point, no interpolation, and the photon
     * takes that point's wavelength for the impurity lookup and wvn */
    int32_t nearest;
    int32_t pad;
    /* non-NULL: the polarised walk of aspherical grains (HG off), with these phase
     * matrices for the ice-table rows (requires nearest) */
    const struct orc_phase *phase;
} orc_config;

/* Phase matrices of the polarised walk for the rows of the ice table
 * (interpolate_phase_matrix, monte_carlo3D.py:819-883, and the envelope of the
 * rejection sampler, :866-883, :933-951).  Element e (P11, P12, P22, P33, P43,
 * P44) is tabulated at cos_asc[e] (cos of the file's angles, ascending) with
 * values p_asc[e][row * n_angle[e] + j] (P12 ... P44 multiplied by P11).  cos_max /
 * cos_min / cos_cutoff and the per-row maxima a1, a2 (|P11| over the two areas)
 * and b1, b2 (|P12|) are computed by the host exactly as :866-883, :933-951 do. */
typedef struct orc_phase {
    int32_t n_rows, pad;
    int32_t n_angle[6];
    const double *cos_asc[6];
    const double *p_asc[6];
    const double *a1, *a2, *b1, *b2;
    double cos_max, cos_min, cos_cutoff;
    double stokes0[4];
} orc_phase;

typedef struct {
    int32_t condition, n_scat;
    double wvn, theta_n, phi_n, path_length, snow_depth;
    int64_t n_draws;      /* uniforms consumed from the walk stream */
    int32_t phi_undefined;/* reference would raise: mux or muy exactly 0 (monte_carlo3D.py:1472-1485) */
    int32_t pad;
    double stokes[4];     /* final Stokes vector (polarised walk; the incident one otherwise) */
} orc_record;

/* ---------------------------------------------------------------- lookups */

/* Two nearest table points by |wvl - wvl_tab|, then scipy interp1d's linear
 * form between them; nearest value when wvl lies outside that pair
 * (interp1d raises ValueError).  monte_carlo3D.py:594-616 (ice) and :688-711
 * (impurity); scipy interp1d._call_linear for the formula. */
static void nearest_two(const orc_table *t, double wvl, int32_t *i0, int32_t *i1)
{
    int32_t a = -1, b = -1;
    double da = INFINITY, db = INFINITY;
    for (int32_t i = 0; i < t->n; ++i) {
        double d = fabs(wvl - t->wvl[i]);
        if (d < da) { b = a; db = da; a = i; da = d; }
        else if (d < db) { b = i; db = d; }
    }
    *i0 = a; *i1 = b;
}

static double interp_two(const orc_table *t, const double *y, int32_t i0, int32_t i1, double wvl)
{
    double x0 = t->wvl[i0], x1 = t->wvl[i1], y0 = y[i0], y1 = y[i1];
    double xl, xh, yl, yh;
    if (x0 < x1) { xl = x0; xh = x1; yl = y0; yh = y1; }
    else { xl = x1; xh = x0; yl = y1; yh = y0; }
    if (wvl < xl || wvl > xh) return y0;            /* ValueError -> nearest */
    return ((wvl - xl) / (xh - xl)) * yh + ((xh - wvl) / (xh - xl)) * yl;
}

/* Photon wavelength on the replay stream: monte_carlo3D.py:1516-1520.
 * scale = FWHM / 2.355; np.around(x, 2) == rint(x * 100) / 100. */
double orc_wavelength(uint64_t seed, uint64_t photon, double wvl0, double half_width)
{
    double scale = half_width / 2.355;
    double u0 = orc_uniform(seed, ORC_TAG_WVL, photon, 0);
    double u1 = orc_uniform(seed, ORC_TAG_WVL, photon, 1);
    double z = sqrt(-2.0 * log(u0)) * cos(ORC_TWO_PI * u1);
    double x = wvl0 + scale * z;
    return nearbyint(x * 100.0) / 100.0;
}

/* Per-photon optics: monte_carlo3D.py:1524-1612. */
typedef struct { double wvl, ssa_ice, ssa_imp, g, ext_cff_mss, P_ext_imp, snow_depth; int32_t row; } orc_optics;

/* A wavelength in um in a table's unit: the netCDF lookups compare wvl * 1e-6
 * with metres (monte_carlo3D.py:518, :673); the aspherical one compares um
 * with um (:323-334). */
static double in_unit(const orc_table *t, double wvl_um)
{
    return t->unit ? wvl_um : wvl_um * 1e-6;
}

static orc_optics photon_optics(const orc_config *c, const orc_table *ice, const orc_table *imp, double wvl_um)
{
    orc_optics o;
    double w = in_unit(ice, wvl_um);
    int32_t i0, i1;
    double ssa_ice, ext_ice, g;
    nearest_two(ice, w, &i0, &i1);
    o.row = i0;
    if (c->nearest) {
        /* argsort(|wvl - wvl_in|)[0]: ssa_in, Q_ext-derived ext_cff_mss and asm_in of that
         * row (:396-415); the photon's wavelength becomes wvl_in of that row (:399, :1536) */
        ssa_ice = ice->ssa[i0];
        ext_ice = ice->ext[i0];
        g = ice->asm_[i0];
        wvl_um = ice->unit ? ice->wvl[i0] : ice->wvl[i0] * 1e6;
    } else {
        ssa_ice = interp_two(ice, ice->ssa, i0, i1, w);
        ext_ice = interp_two(ice, ice->ext, i0, i1, w);
        g = interp_two(ice, ice->asm_, i0, i1, w);
    }
    w = in_unit(imp, wvl_um);
    nearest_two(imp, w, &i0, &i1);
    double ssa_imp = interp_two(imp, imp->ssa, i0, i1, w);
    double ext_imp = interp_two(imp, imp->ext, i0, i1, w);
    if (!isnan(c->ssa_ice_override)) ssa_ice = c->ssa_ice_override;
    if (!isnan(c->ext_ice_override)) ext_ice = c->ext_ice_override;
    if (!isnan(c->g_override)) g = c->g_override;
    if (!isnan(c->ssa_imp_override)) ssa_imp = c->ssa_imp_override;
    if (!isnan(c->ext_imp_override)) ext_imp = c->ext_imp_override;
    double cnc = c->imp_cnc;
    o.wvl = wvl_um;
    o.ssa_ice = ssa_ice;
    o.ssa_imp = ssa_imp;
    o.g = g;
    o.ext_cff_mss = ext_ice * (1 - cnc) + ext_imp * cnc;                       /* :1577 */
    o.P_ext_imp = (cnc * ext_imp) / (cnc * ext_imp + (1 - cnc) * ext_ice);     /* :1580-1581 */
    o.snow_depth = c->tau_tot / (o.ext_cff_mss * c->rho_snw);                  /* :1612 */
    return o;
}

/* scipy interp1d (linear) at x of a table with ascending x: searchsorted (left),
 * clipped to [1, n-1], then the two-term form of interp1d._call_linear. */
static double interp_n(const double *x, const double *y, int32_t n, double xn)
{
    int32_t lo = 0, hi = n;          /* first index with x[i] >= xn */
    while (lo < hi) {
        int32_t mid = (lo + hi) / 2;
        if (x[mid] < xn) lo = mid + 1; else hi = mid;
    }
    int32_t k = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
    double xl = x[k - 1], xh = x[k], yl = y[k - 1], yh = y[k];
    return ((xn - xl) / (xh - xl)) * yh + ((xh - xn) / (xh - xl)) * yl;
}

static double phase_el(const orc_phase *ph, int e, int32_t row, double ct)
{
    return interp_n(ph->cos_asc[e], ph->p_asc[e] + (size_t)row * ph->n_angle[e], ph->n_angle[e], ct);
}

/* rotate_stokes_vector, monte_carlo3D.py:1090-1109 */
static void rotate_stokes(double angle, const double in[4], double out[4])
{
    double d = 2 * angle;
    double cd = cos(d), sd = sin(d);
    out[0] = in[0];
    out[1] = in[1] * cd + in[2] * sd;
    out[2] = -in[1] * sd + in[2] * cd;
    out[3] = in[3];
}

/* Scattering cosine and azimuth of the polarised walk: the two-area rejection
 * sampler of populate_pdfs, monte_carlo3D.py:922-1004, for the photon's current
 * Stokes vector st. */
static void polarised_angles(const orc_phase *ph, int32_t row, const double st[4], orc_stream *s,
                             double *p_rand, double *phi_rand)
{
    double I = st[0], Q = st[1], U = st[2];
    double two_beta = (Q == 0) ? atan(U / 1e-15) : atan(U / Q);                /* :908-911 */
    double C = fabs(Q * cos(two_beta) + U * sin(two_beta));                     /* :935 */
    double max_val1 = fabs(I) * ph->a1[row] + ph->b1[row] * C;                  /* :931-937 */
    double max_val2 = fabs(I) * ph->a2[row] + ph->b2[row] * C;                  /* :940-947 */
    double area1 = (ph->cos_max - ph->cos_cutoff) * max_val1;                   /* :949-951 */
    double area2 = (ph->cos_cutoff - ph->cos_min) * max_val2;
    double percent_area1 = area1 / (area1 + area2);
    double area_rand = stream_next(s);                                          /* :953-957 */
    double cos_theta = stream_next(s);
    double two_phi = 2 * (stream_next(s) * ORC_TWO_PI);
    int area;
    if (area_rand < percent_area1) {                                            /* :963-973 */
        area = 1;
        cos_theta = cos_theta * (ph->cos_max - ph->cos_cutoff) + ph->cos_cutoff;
    } else {
        area = 2;
        cos_theta = -cos_theta * (ph->cos_cutoff - ph->cos_min) + ph->cos_cutoff;
    }
    double r3 = 1, pf = 0;                                                      /* :976-1001 */
    int64_t k = 0;
    while (r3 > pf) {
        if (k > 0) {
            area_rand = stream_next(s);
            if (area_rand < percent_area1) {
                area = 1;
                cos_theta = stream_next(s) * (ph->cos_max - ph->cos_cutoff) + ph->cos_cutoff;
            } else {
                area = 2;
                cos_theta = -stream_next(s) * (ph->cos_cutoff - ph->cos_min) + ph->cos_cutoff;
            }
            two_phi = stream_next(s) * (4 * ORC_PI);
        }
        r3 = 1.000001 * stream_next(s);
        if (area == 1) r3 = r3 * max_val1;
        else r3 = r3 * max_val2;
        double S11 = phase_el(ph, 0, row, cos_theta);
        double S12 = phase_el(ph, 1, row, cos_theta);
        pf = I * S11 + S12 * (Q * cos(two_phi) + U * sin(two_phi));
        k += 1;
    }
    *p_rand = cos_theta;
    *phi_rand = two_phi / 2.;
}

/* Henyey_Greenstein2, monte_carlo3D.py:790-800. */
static double hg2(double g, double r)
{
    if (g == 0) return 1 - 2 * r;
    double q = (1 - g * g) / (1 - g + 2 * g * r);
    return (1. / (2. * g)) * (1 + g * g - q * q);
}

/* ---------------------------------------------------------------- walk */

/* One photon: MonteCarlo.monte_carlo3D, monte_carlo3D.py:1111-1490 (HG
 * branch), with the draws of populate_pdfs (:905-1025) and initial_pdfs
 * (:1027-1044) taken from the replay stream. */
void orc_walk_photon(const orc_config *c, const orc_table *ice, const orc_table *imp,
                     uint64_t seed, uint64_t photon, orc_record *out)
{
    double wvl = orc_wavelength(seed, photon, c->wvl0, c->half_width);
    orc_optics o = photon_optics(c, ice, imp, wvl);
    double theta0 = (ORC_PI * c->theta0_deg) / 180.;                           /* :1508 */

    orc_stream s = {seed, photon, 0, 0, 0, {0, 0, 0, 0}};
    /* initial_pdfs: tau, ssa, ext (:1035-1038) */
    double tau_rand = -log(stream_next(&s));
    double ssa_rand = stream_next(&s);
    double ext_rand = stream_next(&s);
    double p_rand = 0, phi_rand = 0;
    const orc_phase *ph = c->phase;
    double st[4] = {1, 0, 0, 0};                                               /* :1132 */
    if (ph) { st[0] = ph->stokes0[0]; st[1] = ph->stokes0[1]; st[2] = ph->stokes0[2]; st[3] = ph->stokes0[3]; }

    double mux_0 = sin(theta0), muy_0 = 0, muz_0 = -cos(theta0);              /* :1121-1124 */
    double muz2_0 = muz_0 * muz_0;
    double mux_n = 0, muy_n = 0, muz_n = 0;
    double z_prev = 0, path_length = 0;
    double ext_cff = o.ext_cff_mss * c->rho_snw;                               /* :1355-1356 */
    int bottom_reflection = 0, condition = 0;
    int64_t i = 0, i_rand = 0;

    while (condition == 0) {                                                   /* :1212 */
        i += 1;
        i_rand += 1;
        if (i_rand > 1) {                                                      /* :1215-1224 */
            if (ph) {
                polarised_angles(ph, o.row, st, &s, &p_rand, &phi_rand);
            } else {
                p_rand = hg2(o.g, stream_next(&s));
                phi_rand = stream_next(&s) * ORC_TWO_PI;
            }
            tau_rand = -log(stream_next(&s));
            ssa_rand = stream_next(&s);
            ext_rand = stream_next(&s);
            i_rand = 1;
        }
        double dtau = tau_rand;                                                /* :1227 */
        if (c->lam_surface && i == 1) dtau = 0;
        double costheta, sintheta, cosphi = 0, sinphi = 0;
        if (i == 1) {                                                          /* :1232-1237 */
            costheta = 1; sintheta = 0;
        } else if (c->lam_surface || bottom_reflection) {                      /* :1238-1250 */
            mux_0 = 0.; muy_0 = 0.; muz_0 = 1.;
            for (;;) {
                double theta_rand = 0 + (ORC_PI / 2 - 0) * stream_next(&s);
                double r1 = stream_next(&s);
                if (r1 < 2 * sin(theta_rand) * cos(theta_rand)) {
                    costheta = cos(theta_rand);
                    sintheta = sqrt(1 - costheta * costheta);
                    break;
                }
            }
        } else {                                                               /* :1251-1253 */
            costheta = p_rand;
            sintheta = sqrt(1 - costheta * costheta);
        }
        if (i > 1) {                                                           /* :1255-1281 */
            cosphi = cos(phi_rand);
            sinphi = sin(phi_rand);
            if (muz_0 == 1) {
                mux_n = sintheta * cosphi;
                muy_n = sintheta * sinphi;
                muz_n = costheta;
            } else if (muz_0 == -1) {
                mux_n = sintheta * cosphi;
                muy_n = -sintheta * sinphi;
                muz_n = -costheta;
            } else {
                double sq = sqrt(1 - muz2_0);
                mux_n = (sintheta * (mux_0 * muz_0 * cosphi - muy_0 * sinphi)) / sq + mux_0 * costheta;
                muy_n = (sintheta * (muy_0 * muz_0 * cosphi + mux_0 * sinphi)) / sq + muy_0 * costheta;
                muz_n = -sq * sintheta * cosphi + muz_0 * costheta;
            }
            if (bottom_reflection) {                                           /* :1283-1285 */
                st[0] = 1; st[1] = 0; st[2] = 0; st[3] = 0;
                bottom_reflection = 0;
            } else if (ph) {                                                   /* :1287-1342 */
                double cos2theta = costheta * costheta;
                double phi_sca = acos(cosphi);
                double sp[4], sc[4], sm[4];
                rotate_stokes(phi_sca, st, sp);
                double P11 = phase_el(ph, 0, o.row, costheta), P12 = phase_el(ph, 1, o.row, costheta);
                double P22 = phase_el(ph, 2, o.row, costheta), P33 = phase_el(ph, 3, o.row, costheta);
                double P43 = phase_el(ph, 4, o.row, costheta), P44 = phase_el(ph, 5, o.row, costheta);
                sc[0] = sp[0] * P11 + sp[1] * P12;
                sc[1] = sp[0] * P12 + sp[1] * P22;
                sc[2] = sp[2] * P33 - sp[3] * P43;
                sc[3] = sp[2] * P43 + sp[3] * P44;
                double den = sqrt((1 - cos2theta) * (1 - muz_n * muz_n));
                double cos_i;
                if (den == 0) {
                    cos_i = 0;
                } else {
                    double num = muz_n * costheta - muz_0;
                    double sign = (phi_sca >= ORC_PI) ? 1 : -1;
                    cos_i = num / (sign * den);
                    if (cos_i < -1) cos_i = -1;
                    else if (cos_i > 1) cos_i = 1;
                }
                double i_2 = acos(cos_i);
                rotate_stokes(-i_2, sc, sm);
                double I_merd = sm[0];
                st[0] = sm[0] / I_merd; st[1] = sm[1] / I_merd;
                st[2] = sm[2] / I_merd; st[3] = sm[3] / I_merd;
            }
        } else {                                                               /* :1344-1347 */
            mux_n = mux_0; muy_n = muy_0; muz_n = muz_0;
        }
        double z_i = z_prev + dtau * muz_n;                                    /* :1352 */
        if (i > 1) {                                                           /* :1364-1369 */
            mux_0 = mux_n; muy_0 = muy_n; muz_0 = muz_n;
            muz2_0 = muz_0 * muz_0;
        }
        path_length += dtau / ext_cff;                                         /* :1372 */
        int ext_state;
        double ssa_event;
        if (ext_rand > o.P_ext_imp) { ext_state = 1; ssa_event = o.ssa_ice; }  /* :1375-1383 */
        else { ext_state = 2; ssa_event = o.ssa_imp; }
        if (c->lam_surface) ssa_event = c->R;                                  /* :1385-1387 */

        if (z_i > 0) {                                                         /* :1390-1397 */
            condition = 1;
            path_length += -((z_i * dtau) / ((z_i - z_prev) * ext_cff));
        } else if (z_i < -c->tau_tot) {                                        /* :1399-1459 */
            path_length += -(((z_i + c->tau_tot) * dtau) / ((z_i - z_prev) * ext_cff));
            double dtau_correction = -(((z_i + c->tau_tot) / (z_prev - z_i)) * dtau);
            z_i = z_i - (muz_n * dtau_correction);
            int direct = (i == 1);
            if (c->lam_bottom) {
                double reflectance_rand = stream_next(&s);
                if (reflectance_rand <= c->R) bottom_reflection = 1;
                else condition = direct ? 3 : 2;
            } else {
                condition = direct ? 3 : 2;
            }
        } else if (ssa_rand >= ssa_event) {                                    /* :1461-1466 */
            condition = (ext_state == 1) ? 4 : 5;
        }
        z_prev = z_i;
    }

    out->condition = condition;
    out->wvn = 1. / o.wvl;                                                     /* :1468 */
    out->theta_n = acos(muz_0);                                                /* :1469 */
    out->phi_undefined = 0;
    if (i == 1) out->phi_n = 0.;                                               /* :1472-1485 */
    else if (mux_0 > 0 && muy_0 > 0) out->phi_n = atan(muy_0 / mux_0);
    else if (mux_0 < 0 && muy_0 > 0) out->phi_n = atan(muy_0 / mux_0) + ORC_PI;
    else if (mux_0 < 0 && muy_0 < 0) out->phi_n = atan(muy_0 / mux_0) + ORC_PI;
    else if (mux_0 > 0 && muy_0 < 0) out->phi_n = atan(muy_0 / mux_0) + ORC_TWO_PI;
    else { out->phi_n = NAN; out->phi_undefined = 1; }
    out->n_scat = (int32_t)(i - 1);                                            /* :1487 */
    out->path_length = path_length;
    out->snow_depth = o.snow_depth;
    out->n_draws = (int64_t)s.k;
    out->pad = 0;
    out->stokes[0] = st[0]; out->stokes[1] = st[1]; out->stokes[2] = st[2]; out->stokes[3] = st[3];
}

/* Photons [p0, p1) of one run, in order (the loop of monte_carlo3D.py:1613-1616). */
void orc_walk_range(const orc_config *c, const orc_table *ice, const orc_table *imp,
                    uint64_t seed, int64_t p0, int64_t p1, orc_record *out)
{
    for (int64_t p = p0; p < p1; ++p) orc_walk_photon(c, ice, imp, seed, (uint64_t)p, out + (p - p0));
}

/* ---------------------------------------------------------------- threads */
typedef struct {
    const orc_config *c; const orc_table *ice, *imp; uint64_t seed;
    int64_t p0, p1; orc_record *out;
} orc_job;

static void *job_main(void *arg)
{
    orc_job *j = (orc_job *)arg;
    orc_walk_range(j->c, j->ice, j->imp, j->seed, j->p0, j->p1, j->out + j->p0);
    return NULL;
}

/* Photons [0, n) split across n_threads like np.array_split (parallelize.py:14-15):
 * the first n % n_threads shares get one extra photon.  Returns 0 on success. */
int orc_walk_threads(const orc_config *c, const orc_table *ice, const orc_table *imp,
                     uint64_t seed, int64_t n, int n_threads, orc_record *out)
{
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 1024) n_threads = 1024;
    pthread_t th[1024];
    orc_job jobs[1024];
    int64_t base = n / n_threads, extra = n % n_threads, p = 0;
    int started = 0, rc = 0;
    for (int t = 0; t < n_threads; ++t) {
        int64_t len = base + (t < extra ? 1 : 0);
        jobs[t] = (orc_job){c, ice, imp, seed, p, p + len, out};
        p += len;
        if (pthread_create(&th[t], NULL, job_main, &jobs[t]) != 0) { rc = -1; break; }
        started++;
    }
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    if (rc) return rc;
    return 0;
}
