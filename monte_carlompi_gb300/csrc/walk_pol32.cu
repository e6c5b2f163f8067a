// Production FP32 polarised walk of aspherical grains: MonteCarlo.run(shape=...)
// with HG off (monte_carloMPI/monte_carlo3D.py:905-1004, :1111-1490, :1282-1342).
//
// Every step draws its scattering angles by rejection from the phase matrix of
// the photon's wavelength row, for the photon's current Stokes vector, and the
// Stokes vector is rotated into the scattering plane, scattered by the phase
// matrix and rotated back after every scattering.  The number of uniforms a
// step takes depends on the rejection loop, so each photon reads its own
// sequential stream: Philox4x32-10 blocks (block, kTagPol, stream id), four
// 32-bit words per block.  Results depend only on (seed, photon stream id).
//
// One thread walks one photon at a time, one scatter event per loop iteration;
// a thread whose photon ends claims the next from a global counter (warp-
// aggregated) in the same iteration, so the lanes of a warp stay together step
// by step instead of idling until the longest walk of the warp is done.
//
// Statistically equivalent restatements (identical distributions):
//  * the envelope factor |Q cos 2b + U sin 2b| with 2b = arctan(U / Q) (:908-935)
//    is sqrt(Q^2 + U^2), its closed form;
//  * cos / sin of the doubled angles of the two Stokes rotations (:1090-1109) come
//    from the cosines by the double-angle identities (phi_sca = arccos(cos phi) and
//    the meridian angle arccos(cos_i) lie in [0, pi], where the sines are >= 0);
//  * the rejection azimuth 2 phi = 4 pi u is taken as phi = 2 pi u with
//    cos 2 phi = 2 cos^2 phi - 1, sin 2 phi = 2 sin phi cos phi;
//  * the Lambertian direction (p(theta) ~ sin 2 theta, :1238-1250) by inversion
//    cos theta = sqrt(u) instead of rejection; absorption and species tests on
//    32-bit words (1 - u < 1 - ssa, u < P_imp);
//  * the pole case for |mu_z| > 0.99999 and renormalisation of the direction after
//    every rotation; phi_n = atan2 mapped to [0, 2 pi) (as the FP32 HG walk).
#include <cuda_runtime.h>

#include <algorithm>

#include "mcw_internal.cuh"
#include "tally.cuh"

namespace mcw {

namespace {

constexpr float kTwoPiF = 6.28318530717958648f;
constexpr float kPiF = 3.14159265358979324f;
constexpr float kTwo32Inv = 2.3283064365386963e-10f;  // 2^-32
constexpr int kPolBlock = 128;

// The photon's sequential uniforms: Philox4x32-10 (block, kTagPol, id lo, id hi).
struct PolStream {
    uint32_t lo, hi, block;
    int k;
    uint4 x;

    __device__ __forceinline__ uint32_t word(const PhiloxKeys &ks) {
        if (k == 4) {
            x = philox10(make_uint4(block++, kTagPol, lo, hi), ks);
            k = 0;
        }
        const uint32_t w = k == 0 ? x.x : (k == 1 ? x.y : (k == 2 ? x.z : x.w));
        ++k;
        return w;
    }
    // uniform in [2^-24, 1 - 2^-24]
    __device__ __forceinline__ float u(const PhiloxKeys &ks) { return u01_f32(word(ks)); }
};

// scipy interp1d (linear) on an ascending grid: the segment of the first grid
// point >= xn (clipped to [1, n - 1]), linear between its ends.
__device__ __forceinline__ float interp32(const float *x, const float *y, int n, float xn) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(x + mid) < xn) lo = mid + 1; else hi = mid;
    }
    const int k = min(max(lo, 1), n - 1);
    const float xl = __ldg(x + k - 1), xh = __ldg(x + k), yl = __ldg(y + k - 1), yh = __ldg(y + k);
    return fmaf(__fdividef(xn - xl, xh - xl), yh - yl, yl);
}

__device__ __forceinline__ float phase_el(const DevPhase32 &ph, int e, int row, float ct) {
    return interp32(ph.cos_asc[e], ph.p_asc[e] + (size_t)row * ph.n_angle[e], ph.n_angle[e], ct);
}

// cos / sin of an azimuth 2 pi u, u in (0, 1): sincos of the angle shifted into
// [-pi, pi) (where the fast intrinsic is accurate), negated back.
__device__ __forceinline__ void azimuth(float u, float &c, float &s) {
    float sn, cs;
    __sincosf(fmaf(kTwoPiF, u, -kPiF), &sn, &cs);
    c = -cs;
    s = -sn;
}

// One step's scattering cosine and azimuth: the two-area rejection sampler of
// populate_pdfs (monte_carlo3D.py:922-1004) for Stokes vector (I, Q, U).
// Returns false if the time budget ran out.
__device__ bool rejection_angles(const DevPhase32 &ph, int row, float I, float Q, float U, PolStream &s,
                                 const PhiloxKeys &ks, float &cos_theta, float &cphi, float &sphi,
                                 unsigned long long t0, unsigned long long budget_ns) {
    const float C = sqrtf(fmaf(Q, Q, U * U));
    const float max_val1 = fmaf(fabsf(I), __ldg(ph.a1 + row), __ldg(ph.b1 + row) * C);
    const float max_val2 = fmaf(fabsf(I), __ldg(ph.a2 + row), __ldg(ph.b2 + row) * C);
    const float w1 = ph.cos_max - ph.cos_cutoff, w2 = ph.cos_cutoff - ph.cos_min;
    const float area1 = w1 * max_val1, area2 = w2 * max_val2;
    const float percent_area1 = __fdividef(area1, area1 + area2);
    for (uint32_t k = 0;; ++k) {
        const bool one = s.u(ks) < percent_area1;
        const float uc = s.u(ks);
        azimuth(s.u(ks), cphi, sphi);
        cos_theta = one ? fmaf(uc, w1, ph.cos_cutoff) : fmaf(-uc, w2, ph.cos_cutoff);
        const float r3 = 1.000001f * s.u(ks) * (one ? max_val1 : max_val2);
        const float S11 = phase_el(ph, 0, row, cos_theta);
        const float S12 = phase_el(ph, 1, row, cos_theta);
        const float c2 = fmaf(2.f * cphi, cphi, -1.f), s2 = 2.f * sphi * cphi;
        const float pf = fmaf(I, S11, S12 * fmaf(Q, c2, U * s2));
        if (!(r3 > pf)) return true;
        if ((k & 255u) == 255u && global_ns() - t0 > budget_ns) return false;
    }
}

// Rotate a Stokes vector by an angle whose doubled cosine / sine are (cd, sd)
// (rotate_stokes_vector, monte_carlo3D.py:1090-1109).
__device__ __forceinline__ void rotate(float &Q, float &U, float cd, float sd) {
    const float q = fmaf(Q, cd, U * sd);
    const float u = fmaf(-Q, sd, U * cd);
    Q = q;
    U = u;
}

// A photon in flight (registers of its lane).
struct PolPhoton {
    int64_t gid;
    const DevPhase32 *ph;
    int32_t ci, row, i;
    bool lam_surface, lam_bottom, bref;
    float tau, R, inv_ext, p_imp, coalb_ice, coalb_imp, wvn, depth;
    unsigned long long wvn_fx;
    PolStream s;
    float dtau_next;
    uint32_t w_abs, w_ext;
    float mux, muy, muz, z, path, pathc;
    float I, Q, U, V;
};

// Birth of photon gid: wavelength (monte_carlo3D.py:1516-1520), optics row, the
// initial draws of initial_pdfs (:1035-1038) and the incident direction and Stokes
// vector (:1121-1132).
__device__ __forceinline__ void pol_birth(PolPhoton &P, const WalkArgs &a, int64_t gid) {
    const int ci = find_config(a.prefix, a.n_cfg, gid);
    const DevConfig &c = a.cfgs[ci];
    const uint64_t rid = c.rng_base + (uint64_t)(gid - c.offset);
    const uint32_t lo = (uint32_t)rid, hi = (uint32_t)(rid >> 32);
    const uint4 rb = philox10(make_uint4(0u, kTagBirth, lo, hi), a.keys);
    float sb, cb;
    __sincosf(kTwoPiF * (u01_f32(rb.y) - 0.5f), &sb, &cb);
    const float zb = sqrtf(-2.f * __logf(u01_f32(rb.x))) * cb;
    const int kw = __float2int_rn(fmaf(c.sigma_100, zb, c.wvl0_100));
    const LutEntry *e = a.lut + c.lut_off + min(max(kw - c.k_lo, 0), c.lut_n - 1);
    const float4 e0 = __ldg(reinterpret_cast<const float4 *>(e));       // wvn, coalb_ice, coalb_imp, g
    const float4 e1 = __ldg(reinterpret_cast<const float4 *>(e) + 1);   // inv_ext, p_imp, snow_depth, -
    P.gid = gid;
    P.ci = ci;
    P.ph = a.phase + c.ice_table;
    P.row = (int)__ldg(&e->pad2);
    P.i = 0;
    P.lam_surface = (c.flags & kFlagLamSurface) != 0;
    P.lam_bottom = (c.flags & kFlagLamBottom) != 0;
    P.bref = false;
    P.tau = c.tau_tot;
    P.R = c.R;
    P.inv_ext = e1.x;
    P.p_imp = e1.y;
    P.coalb_ice = P.lam_surface ? 1.f - P.R : e0.y;                     // :1385-1387
    P.coalb_imp = P.lam_surface ? 1.f - P.R : e0.z;
    P.wvn = e0.x;
    P.depth = e1.z;
    P.wvn_fx = __ldg(&e->wvn_fx);
    P.s = PolStream{lo, hi, 0u, 4, make_uint4(0, 0, 0, 0)};
    P.dtau_next = -__logf(P.s.u(a.keys));
    P.w_abs = P.s.word(a.keys);
    P.w_ext = P.s.word(a.keys);
    P.mux = c.mux0;
    P.muy = 0.f;
    P.muz = c.muz0;
    P.z = 0.f;
    P.path = 0.f;
    P.pathc = 0.f;
    P.I = (float)c.stokes0[0];
    P.Q = (float)c.stokes0[1];
    P.U = (float)c.stokes0[2];
    P.V = (float)c.stokes0[3];
}

// One scatter event of the photon (monte_carlo3D.py:1212-1466).  Returns the end
// condition (0: still walking), or -1 when the time budget ran out.
__device__ __forceinline__ int pol_step(PolPhoton &P, const WalkArgs &a, unsigned long long t0) {
    const DevPhase32 &ph = *P.ph;
    P.i += 1;
    float cphi = 0.f, sphi = 0.f, p_cos = 1.f;
    if (P.i > 1) {                                                        // :1215-1224
        if (!rejection_angles(ph, P.row, P.I, P.Q, P.U, P.s, a.keys, p_cos, cphi, sphi, t0, a.budget_ns))
            return -1;
        P.dtau_next = -__logf(P.s.u(a.keys));
        P.w_abs = P.s.word(a.keys);
        P.w_ext = P.s.word(a.keys);
    }
    const float dtau = (P.lam_surface && P.i == 1) ? 0.f : P.dtau_next;  // :1227-1229
    float nx = P.mux, ny = P.muy, nz = P.muz;
    if (P.i > 1) {
        // direction (:1238-1281): Lambertian about the vertical, or the rotation
        float m0x = P.mux, m0y = P.muy, m0z = P.muz, ct = p_cos;
        if (P.lam_surface || P.bref) {
            m0x = 0.f; m0y = 0.f; m0z = 1.f;
            ct = sqrtf(P.s.u(a.keys));
        }
        const float st = sqrtf(fmaxf(0.f, fmaf(-ct, ct, 1.f)));
        if (fabsf(m0z) > 0.99999f) {
            const float sg = copysignf(1.f, m0z);
            nx = st * cphi;
            ny = sg * st * sphi;
            nz = sg * ct;
        } else {
            const float s2 = fmaf(-m0z, m0z, 1.f);
            const float rs = rsqrtf(s2);
            const float tq = st * rs;
            nx = fmaf(tq, fmaf(m0x * m0z, cphi, -m0y * sphi), m0x * ct);
            ny = fmaf(tq, fmaf(m0y * m0z, cphi, m0x * sphi), m0y * ct);
            nz = fmaf(-s2 * rs * st, cphi, m0z * ct);
            const float inv = rsqrtf(fmaf(nx, nx, fmaf(ny, ny, nz * nz)));
            nx *= inv; ny *= inv; nz *= inv;
        }
        // Stokes vector (:1282-1342)
        if (P.bref) {
            P.I = 1.f; P.Q = 0.f; P.U = 0.f; P.V = 0.f;
            P.bref = false;
        } else {
            // into the scattering plane: phi_sca = arccos(cphi) in [0, pi]
            const float sps = sqrtf(fmaxf(0.f, fmaf(-cphi, cphi, 1.f)));
            float Q = P.Q, U = P.U;
            rotate(Q, U, fmaf(2.f * cphi, cphi, -1.f), 2.f * sps * cphi);
            const float P11 = phase_el(ph, 0, P.row, ct), P12 = phase_el(ph, 1, P.row, ct);
            const float P22 = phase_el(ph, 2, P.row, ct), P33 = phase_el(ph, 3, P.row, ct);
            const float P43 = phase_el(ph, 4, P.row, ct), P44 = phase_el(ph, 5, P.row, ct);
            const float Is = fmaf(P.I, P11, Q * P12), Qs = fmaf(P.I, P12, Q * P22);
            const float Us = fmaf(U, P33, -P.V * P43), Vs = fmaf(U, P43, P.V * P44);
            // back to the meridian plane of the new direction
            const float den = sqrtf(fmaf(-ct, ct, 1.f) * fmaf(-nz, nz, 1.f));
            float cos_i = 0.f;
            if (den != 0.f) {
                const float sign = (cphi == -1.f) ? 1.f : -1.f;   // phi_sca >= pi only at cos phi = -1
                cos_i = fminf(fmaxf(__fdividef(fmaf(nz, ct, -m0z), sign * den), -1.f), 1.f);
            }
            const float si = sqrtf(fmaxf(0.f, fmaf(-cos_i, cos_i, 1.f)));
            float Qm = Qs, Um = Us;
            rotate(Qm, Um, fmaf(2.f * cos_i, cos_i, -1.f), -2.f * si * cos_i);
            const float inv_i = 1.f / Is;
            P.I = 1.f;
            P.Q = Qm * inv_i;
            P.U = Um * inv_i;
            P.V = Vs * inv_i;
        }
    }
    // move, path, boundaries, absorption (:1349-1466)
    float zn = fmaf(dtau, nz, P.z);
    const float inc = dtau * P.inv_ext;
    {
        const float y = inc - P.pathc;
        const float tt = P.path + y;
        P.pathc = (tt - P.path) - y;
        P.path = tt;
    }
    P.mux = nx; P.muy = ny; P.muz = nz;
    const bool imp = (float)P.w_ext * kTwo32Inv < P.p_imp;
    const float coalb = imp ? P.coalb_imp : P.coalb_ice;
    int cond = 0;
    if (zn > 0.f) {
        cond = 1;
        P.path -= __fdividef(zn, zn - P.z) * inc;
    } else if (zn < -P.tau) {
        P.path -= __fdividef(zn + P.tau, zn - P.z) * inc;
        zn = -P.tau;
        if (P.lam_bottom && P.s.u(a.keys) <= P.R) P.bref = true;
        else cond = (P.i == 1) ? 3 : 2;
    } else if ((float)P.w_abs * kTwo32Inv < coalb) {
        cond = imp ? 5 : 4;
    }
    P.z = zn;
    return cond;
}

// Record and tallies of a photon that ended with condition cond.
__device__ __forceinline__ void pol_finish(const PolPhoton &P, const WalkArgs &a, int cond) {
    const float theta = acosf(fminf(fmaxf(P.muz, -1.f), 1.f));
    float phi = 0.f;
    if (P.i > 1) {
        phi = atan2f(P.muy, P.mux);
        if (phi < 0.f) phi += kTwoPiF;
        if (phi >= kTwoPiF) phi = 0.f;
    }
    if (a.records) {
        mcw_record32p r;
        r.condition = cond;
        r.n_scat = P.i - 1;
        r.wvn = P.wvn;
        r.theta_n = theta;
        r.phi_n = phi;
        r.path_length = P.path;
        r.snow_depth = P.depth;
        r.config = (uint32_t)P.ci;
        r.stokes_q = P.Q;
        r.stokes_u = P.U;
        r.stokes_v = P.V;
        r.pad = 0.f;
        reinterpret_cast<mcw_record32p *>(a.records)[P.gid] = r;
    }
    tally_global(a.tallies + P.ci, cond, P.i - 1, P.wvn_fx, theta, phi);
}

// One loop iteration is one scatter event of each lane's photon; a lane whose
// photon ends claims the next one in the same iteration, so the lanes of a warp
// stay together step by step instead of waiting for the warp's longest walk.
__global__ void __launch_bounds__(kPolBlock) walk_pol32_kernel(const WalkArgs a) {
    const unsigned long long t0 = global_ns();
    const int lane = threadIdx.x & 31;
    PolPhoton P;
    bool have = false;
    for (uint32_t it = 0;; ++it) {
        if (!have) {
            // claim the next photon; lanes that arrive together share one atomic
            const unsigned m = __activemask();
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.work, (unsigned long long)__popc(m));
            base = __shfl_sync(m, base, leader);
            const unsigned long long g = base + __popc(m & ((1u << lane) - 1u));
            if (g >= (unsigned long long)a.total) break;
            pol_birth(P, a, (int64_t)g);
            have = true;
        }
        const int cond = pol_step(P, a, t0);
        if (cond < 0) {
            atomicOr(a.status, kStatusBudget);
            break;
        }
        if (cond > 0) {
            pol_finish(P, a, cond);
            have = false;
        }
        if ((it & 1023u) == 1023u &&
            (global_ns() - t0 > a.budget_ns || (*(volatile unsigned int *)a.status & kStatusBudget))) {
            atomicOr(a.status, kStatusBudget);
            break;
        }
    }
}

}  // namespace

cudaError_t launch_walk_pol32(const WalkArgs &a, int sm_count, cudaStream_t s) {
    if (a.total <= 0) return cudaSuccess;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, walk_pol32_kernel, kPolBlock, 0);
    if (e != cudaSuccess) return e;
    const int64_t want = (a.total + kPolBlock - 1) / kPolBlock;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count * std::max(per_sm, 1), want));
    walk_pol32_kernel<<<grid, kPolBlock, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcw
