// FP64 replay walk: one thread per photon, the reference's arithmetic order,
// uniforms from the photon-indexed Philox replay stream.  Compiled with
// --fmad=false so every product and sum is rounded on its own, as NumPy does.
//
// Restates MonteCarlo.monte_carlo3D (monte_carloMPI/monte_carlo3D.py:1111-1490,
// HG branch) with the draws of populate_pdfs (:905-1025) and initial_pdfs
// (:1027-1044), and the wavelength draw of MonteCarlo.run (:1515-1520).  The
// kernel instance kPol restates the polarised branch of aspherical grains: the
// rejection sampler of populate_pdfs (:922-1004) and the Stokes-vector update
// of monte_carlo3D (:1282-1342).
#include <cuda_runtime.h>

#include "mcw_internal.cuh"
#include "ssp_device.cuh"
#include "tally.cuh"

namespace mcw {

namespace {

// Sequential reader of one photon's replay stream: uniform k uses Philox
// block k >> 1 (counter (block, tag, photon lo, photon hi)), 64-bit word k & 1.
struct ReplayStream {
    uint64_t seed, photon, k;
    uint4 x;
    bool overrun;

    __device__ double next() {
        if ((k & 1) == 0) {
            uint64_t b = k >> 1;
            if (b > 0xffffffffull) overrun = true;
            x = philox10_seed(make_uint4((uint32_t)b, kTagWalk, (uint32_t)photon,
                                         (uint32_t)(photon >> 32)), seed);
        }
        uint64_t w = (k & 1) ? (((uint64_t)x.w << 32) | x.z) : (((uint64_t)x.y << 32) | x.x);
        ++k;
        return u01_f64(w);
    }
};

__device__ double replay_uniform(uint64_t seed, uint32_t tag, uint64_t photon, uint64_t k) {
    uint4 x = philox10_seed(make_uint4((uint32_t)(k >> 1), tag, (uint32_t)photon,
                                       (uint32_t)(photon >> 32)), seed);
    uint64_t w = (k & 1) ? (((uint64_t)x.w << 32) | x.z) : (((uint64_t)x.y << 32) | x.x);
    return u01_f64(w);
}

// Photon wavelength [um]: sigma = FWHM / 2.355, Box-Muller normal from the
// wavelength stream, np.around(x, 2) = rint(x * 100) / 100.
__device__ double replay_wavelength(const DevConfig &c, uint64_t seed, uint64_t gid) {
    double u0 = replay_uniform(seed, kTagWvl, gid, 0);
    double u1 = replay_uniform(seed, kTagWvl, gid, 1);
    double z = sqrt(-2.0 * log(u0)) * cos(kTwoPi * u1);
    double x = c.wvl0 + c.scale * z;
    return rint(x * 100.0) / 100.0;
}

// scipy interp1d (linear) on an ascending grid: searchsorted (left) clipped to
// [1, n-1], then the two-term form of interp1d._call_linear.
__device__ double interp_n(const double *x, const double *y, int n, double xn) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] < xn) lo = mid + 1; else hi = mid;
    }
    const int k = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
    const double xl = x[k - 1], xh = x[k], yl = y[k - 1], yh = y[k];
    return ((xn - xl) / (xh - xl)) * yh + ((xh - xn) / (xh - xl)) * yl;
}

__device__ __forceinline__ double phase_el(const DevPhase &ph, int e, int row, double ct) {
    return interp_n(ph.cos_asc[e], ph.p_asc[e] + (size_t)row * ph.n_angle[e], ph.n_angle[e], ct);
}

// rotate_stokes_vector (monte_carlo3D.py:1090-1109)
__device__ __forceinline__ void rotate_stokes(double angle, const double in[4], double out[4]) {
    const double d = 2 * angle;
    const double cd = cos(d), sd = sin(d);
    out[0] = in[0];
    out[1] = in[1] * cd + in[2] * sd;
    out[2] = -in[1] * sd + in[2] * cd;
    out[3] = in[3];
}

// Scattering cosine and azimuth of the polarised walk for the photon's Stokes
// vector st: the two-area rejection sampler of populate_pdfs (:905-1004).
// Returns false if the stream ran out or the time budget passed.
__device__ bool polarised_angles(const DevPhase &ph, int row, const double st[4], ReplayStream &s,
                                 double &p_rand, double &phi_rand, unsigned long long t0,
                                 unsigned long long budget_ns) {
    const double I = st[0], Q = st[1], U = st[2];
    const double two_beta = (Q == 0) ? atan(U / 1e-15) : atan(U / Q);          // :908-911
    const double C = fabs(Q * cos(two_beta) + U * sin(two_beta));               // :935
    const double max_val1 = fabs(I) * ph.a1[row] + ph.b1[row] * C;              // :931-937
    const double max_val2 = fabs(I) * ph.a2[row] + ph.b2[row] * C;              // :940-947
    const double area1 = (ph.cos_max - ph.cos_cutoff) * max_val1;               // :949-951
    const double area2 = (ph.cos_cutoff - ph.cos_min) * max_val2;
    const double percent_area1 = area1 / (area1 + area2);
    double area_rand = s.next();                                                // :953-957
    double cos_theta = s.next();
    double two_phi = 2 * (s.next() * kTwoPi);
    int area;
    if (area_rand < percent_area1) {                                            // :963-973
        area = 1;
        cos_theta = cos_theta * (ph.cos_max - ph.cos_cutoff) + ph.cos_cutoff;
    } else {
        area = 2;
        cos_theta = -cos_theta * (ph.cos_cutoff - ph.cos_min) + ph.cos_cutoff;
    }
    double r3 = 1, pf = 0;                                                      // :976-1001
    for (int64_t k = 0; r3 > pf; ++k) {
        if (k > 0) {
            area_rand = s.next();
            if (area_rand < percent_area1) {
                area = 1;
                cos_theta = s.next() * (ph.cos_max - ph.cos_cutoff) + ph.cos_cutoff;
            } else {
                area = 2;
                cos_theta = -s.next() * (ph.cos_cutoff - ph.cos_min) + ph.cos_cutoff;
            }
            two_phi = s.next() * (4 * kPi);
        }
        r3 = 1.000001 * s.next();
        if (area == 1) r3 = r3 * max_val1;
        else r3 = r3 * max_val2;
        const double S11 = phase_el(ph, 0, row, cos_theta);
        const double S12 = phase_el(ph, 1, row, cos_theta);
        pf = I * S11 + S12 * (Q * cos(two_phi) + U * sin(two_phi));
        if (s.overrun) return false;
        if ((k & 255) == 255 && global_ns() - t0 > budget_ns) return false;
    }
    p_rand = cos_theta;
    phi_rand = two_phi / 2.;
    return true;
}

// Henyey_Greenstein2 (monte_carlo3D.py:790-800).
__device__ __forceinline__ double hg2(double g, double r) {
    if (g == 0) return 1 - 2 * r;
    double q = (1 - g * g) / (1 - g + 2 * g * r);
    return (1. / (2. * g)) * (1 + g * g - q * q);
}

template <bool kPol>
__global__ void __launch_bounds__(128) walk_replay_kernel(const ReplayArgs a) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.total) return;
    const int ci = find_config(a.prefix, a.n_cfg, gid);
    const DevConfig c = a.cfgs[ci];

    const uint64_t rid = c.rng_base + (uint64_t)(gid - c.offset);  // stream id
    const double wvl = replay_wavelength(c, a.seed, rid);
    const Optics o = photon_optics(c, a.ice[c.ice_table], a.imp, wvl);
    const bool lam_surface = (c.flags & kFlagLamSurface) != 0;
    const bool lam_bottom = (c.flags & kFlagLamBottom) != 0;
    const double tau_tot = c.tau_tot_d, R = c.R_d;

    ReplayStream s{a.seed, rid, 0, make_uint4(0, 0, 0, 0), false};
    double tau_rand = -log(s.next());  // initial_pdfs, :1035-1038
    double ssa_rand = s.next();
    double ext_rand = s.next();
    double p_rand = 0, phi_rand = 0;
    double st[4] = {1, 0, 0, 0};                                      // :1132
    DevPhase ph{};
    if (kPol) {
        ph = a.phase[c.ice_table];
        for (int k = 0; k < 4; ++k) st[k] = c.stokes0[k];
    }

    double mux_0 = c.mux0_d, muy_0 = 0, muz_0 = c.muz0_d;             // :1121-1124
    double muz2_0 = muz_0 * muz_0;
    double mux_n = 0, muy_n = 0, muz_n = 0;
    double z_prev = 0, path_length = 0;
    const double ext_cff = o.ext_cff_mss * c.rho_snw;                 // :1355-1356
    bool bottom_reflection = false;
    int condition = 0;
    int64_t i = 0;
    const unsigned long long t0 = global_ns();

    while (condition == 0) {                                          // :1212
        i += 1;
        if (i > 1) {                                                  // :1215-1224
            if (kPol) {
                if (!polarised_angles(ph, o.row, st, s, p_rand, phi_rand, t0, a.budget_ns)) {
                    atomicOr(a.status, s.overrun ? kStatusStream : kStatusBudget);
                    break;
                }
            } else {
                p_rand = hg2(o.g, s.next());
                phi_rand = s.next() * kTwoPi;
            }
            tau_rand = -log(s.next());
            ssa_rand = s.next();
            ext_rand = s.next();
        }
        double dtau = tau_rand;                                       // :1227-1229
        if (lam_surface && i == 1) dtau = 0;
        double costheta, sintheta;
        if (i == 1) {                                                 // :1232-1237
            costheta = 1;
            sintheta = 0;
        } else if (lam_surface || bottom_reflection) {                // :1238-1250
            mux_0 = 0.;
            muy_0 = 0.;
            muz_0 = 1.;
            for (;;) {
                double theta_rand = 0 + (kPi / 2 - 0) * s.next();
                double r1 = s.next();
                if (r1 < 2 * sin(theta_rand) * cos(theta_rand)) {
                    costheta = cos(theta_rand);
                    sintheta = sqrt(1 - costheta * costheta);
                    break;
                }
                if (s.overrun) { costheta = 1; sintheta = 0; break; }
            }
        } else {                                                      // :1251-1253
            costheta = p_rand;
            sintheta = sqrt(1 - costheta * costheta);
        }
        if (i > 1) {                                                  // :1255-1281
            double cosphi = cos(phi_rand), sinphi = sin(phi_rand);
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
            if (bottom_reflection) {                                  // :1283-1285
                st[0] = 1; st[1] = 0; st[2] = 0; st[3] = 0;
                bottom_reflection = false;
            } else if (kPol) {                                        // :1287-1342
                const double cos2theta = costheta * costheta;
                const double phi_sca = acos(cosphi);
                double sp[4], sc[4], sm[4];
                rotate_stokes(phi_sca, st, sp);
                const double P11 = phase_el(ph, 0, o.row, costheta), P12 = phase_el(ph, 1, o.row, costheta);
                const double P22 = phase_el(ph, 2, o.row, costheta), P33 = phase_el(ph, 3, o.row, costheta);
                const double P43 = phase_el(ph, 4, o.row, costheta), P44 = phase_el(ph, 5, o.row, costheta);
                sc[0] = sp[0] * P11 + sp[1] * P12;
                sc[1] = sp[0] * P12 + sp[1] * P22;
                sc[2] = sp[2] * P33 - sp[3] * P43;
                sc[3] = sp[2] * P43 + sp[3] * P44;
                const double den = sqrt((1 - cos2theta) * (1 - muz_n * muz_n));
                double cos_i;
                if (den == 0) {
                    cos_i = 0;
                } else {
                    const double num = muz_n * costheta - muz_0;
                    const double sign = (phi_sca >= kPi) ? 1 : -1;
                    cos_i = num / (sign * den);
                    if (cos_i < -1) cos_i = -1;
                    else if (cos_i > 1) cos_i = 1;
                }
                rotate_stokes(-acos(cos_i), sc, sm);
                const double I_merd = sm[0];
                for (int k = 0; k < 4; ++k) st[k] = sm[k] / I_merd;
            }
        } else {                                                      // :1344-1347
            mux_n = mux_0;
            muy_n = muy_0;
            muz_n = muz_0;
        }
        double z_i = z_prev + dtau * muz_n;                           // :1352
        if (i > 1) {                                                  // :1364-1369
            mux_0 = mux_n;
            muy_0 = muy_n;
            muz_0 = muz_n;
            muz2_0 = muz_0 * muz_0;
        }
        path_length += dtau / ext_cff;                                // :1372
        bool ice = ext_rand > o.p_imp;                                // :1375-1383
        double ssa_event = ice ? o.ssa_ice : o.ssa_imp;
        if (lam_surface) ssa_event = R;                               // :1385-1387
        if (z_i > 0) {                                                // :1390-1397
            condition = 1;
            path_length += -((z_i * dtau) / ((z_i - z_prev) * ext_cff));
        } else if (z_i < -tau_tot) {                                  // :1399-1459
            path_length += -(((z_i + tau_tot) * dtau) / ((z_i - z_prev) * ext_cff));
            double dtau_correction = -(((z_i + tau_tot) / (z_prev - z_i)) * dtau);
            z_i = z_i - (muz_n * dtau_correction);
            const int leave = (i == 1) ? 3 : 2;
            if (lam_bottom) {
                if (s.next() <= R) bottom_reflection = true;
                else condition = leave;
            } else {
                condition = leave;
            }
        } else if (ssa_rand >= ssa_event) {                           // :1461-1466
            condition = ice ? 4 : 5;
        }
        z_prev = z_i;
        if (s.overrun) {
            atomicOr(a.status, kStatusStream);
            break;
        }
        if ((i & 1023) == 0 && global_ns() - t0 > a.budget_ns) {
            atomicOr(a.status, kStatusBudget);
            break;
        }
    }

    mcw_record64p r;
    r.condition = condition;
    r.n_scat = (int32_t)(i - 1);                                      // :1487
    r.wvn = 1. / o.wvl_um;                                            // :1468
    r.theta_n = acos(muz_0);                                          // :1469
    r.flags = 0;
    if (i == 1) r.phi_n = 0.;                                         // :1472-1485
    else if (mux_0 > 0 && muy_0 > 0) r.phi_n = atan(muy_0 / mux_0);
    else if (mux_0 < 0 && muy_0 > 0) r.phi_n = atan(muy_0 / mux_0) + kPi;
    else if (mux_0 < 0 && muy_0 < 0) r.phi_n = atan(muy_0 / mux_0) + kPi;
    else if (mux_0 > 0 && muy_0 < 0) r.phi_n = atan(muy_0 / mux_0) + kTwoPi;
    else { r.phi_n = __longlong_as_double(0x7ff8000000000000LL); r.flags = 1u; }
    r.path_length = path_length;
    r.snow_depth = o.snow_depth;
    r.config = (uint32_t)ci;
    r.stokes_q = st[1];
    r.stokes_u = st[2];
    r.stokes_v = st[3];
    if (a.records) {
        if (kPol) {
            static_cast<mcw_record64p *>(a.records)[gid] = r;
        } else {
            mcw_record64 &d = static_cast<mcw_record64 *>(a.records)[gid];
            d.condition = r.condition;
            d.n_scat = r.n_scat;
            d.wvn = r.wvn;
            d.theta_n = r.theta_n;
            d.phi_n = r.phi_n;
            d.path_length = r.path_length;
            d.snow_depth = r.snow_depth;
            d.config = r.config;
            d.flags = r.flags;
        }
    }

    if (a.tallies && condition > 0) {
        const unsigned long long wfx = (unsigned long long)llrint(r.wvn * 4294967296.0);
        float th = (float)r.theta_n, ph = (r.flags ? 0.f : (float)r.phi_n);
        tally_global(a.tallies + ci, condition, r.n_scat, wfx, th, ph);
    }
}

}  // namespace

cudaError_t launch_walk_replay(const ReplayArgs &a, cudaStream_t s) {
    if (a.total <= 0) return cudaSuccess;
    const int block = 128;
    const int64_t grid = (a.total + block - 1) / block;
    if (a.pol) walk_replay_kernel<true><<<(unsigned)grid, block, 0, s>>>(a);
    else walk_replay_kernel<false><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcw
