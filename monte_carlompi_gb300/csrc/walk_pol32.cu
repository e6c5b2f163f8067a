// Production FP32 polarised walk of aspherical grains: MonteCarlo.run(shape=...)
// with HG off (monte_carloMPI/monte_carlo3D.py:905-1004, :1111-1490, :1282-1342).
//
// Every step draws its scattering angles by rejection from the phase matrix of
// the photon's wavelength row, for the photon's current Stokes vector, and the
// Stokes vector is rotated into the scattering plane, scattered by the phase
// matrix and rotated back after every scattering.
//
// Random numbers are indexed, not sequential: step n of a photon takes one
// Philox4x32-10 block (n, kTagPolStep, stream id) for its optical path,
// absorption, species and Lambertian words, one (n, kTagPolRefl, id) for a
// bottom reflectance draw, and rejection candidate j one block
// (n, kTagPolCand | j << 8, id) for its area, cosine, azimuth and acceptance
// words; the accepted candidate is the lowest-indexed one that passes.  So any
// lane can test any photon's candidates, and results depend only on (seed,
// photon stream id).
//
// One thread walks one photon, one scatter event per loop iteration; a lane
// whose photon ends claims the next from a global counter in the same iteration
// (warp-aggregated), and lanes without a photon stay in the loop as helpers.
// The rejection runs as warp-wide rounds: the n photons still looking for an
// angle share the 32 lanes (lane l tests candidate jbase + l / n of photon
// l % n), so a step costs a few rounds instead of the slowest lane's candidate
// count, and the last walks of a launch get the whole warp.
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
constexpr uint32_t kMaxCandidates = 1u << 24;          // candidate index range of a step

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

// The segment interp32 would use: first grid point >= xn, clipped to [1, n - 1].
__device__ __forceinline__ int segment32(const float *x, int n, float xn) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(x + mid) < xn) lo = mid + 1; else hi = mid;
    }
    return min(max(lo, 1), n - 1);
}

// The same segment on the shared grid, the search seeded by its bucket: probe down
// while the point before is still >= xn, then up while the point is < xn.
__device__ __forceinline__ int segment_seeded(const DevPhase32 &ph, float xn) {
    const float *x = ph.cos_asc[0];
    const int n = ph.n_angle[0];
    if (!ph.seed) return segment32(x, n, xn);
    const int b = min(max(__float2int_rd((xn - ph.seed_lo) * ph.seed_scale), 0), kPhaseBuckets - 1);
    int k = __ldg(ph.seed + b);
    while (k > 0 && __ldg(x + k - 1) >= xn) --k;
    while (k < n && __ldg(x + k) < xn) ++k;
    return min(max(k, 1), n - 1);
}

// Element e at xn in segment k of the grid the elements share.
__device__ __forceinline__ float phase_at(const DevPhase32 &ph, int e, int row, int k, float xn) {
    const float *x = ph.cos_asc[0];
    const float *y = ph.p_asc[e] + (size_t)row * ph.n_angle[0];
    const float xl = __ldg(x + k - 1), xh = __ldg(x + k), yl = __ldg(y + k - 1), yh = __ldg(y + k);
    return fmaf(__fdividef(xn - xl, xh - xl), yh - yl, yl);
}

// cos / sin of an azimuth 2 pi u, u in (0, 1): sincos of the angle shifted into
// [-pi, pi) (where the fast intrinsic is accurate), negated back.
__device__ __forceinline__ void azimuth(float u, float &c, float &s) {
    float sn, cs;
    __sincosf(fmaf(kTwoPiF, u, -kPiF), &sn, &cs);
    c = -cs;
    s = -sn;
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
    uint32_t lo, hi;
    bool lam_surface, lam_bottom, bref;
    float tau, R, inv_ext, p_imp, coalb_ice, coalb_imp, wvn, depth;
    unsigned long long wvn_fx;
    uint4 sb;        // the current step's block (path, absorption, species, Lambertian)
    float mux, muy, muz, z, path, pathc;
    float I, Q, U, V;
};

__device__ __forceinline__ uint4 step_block(const PolPhoton &P, uint32_t n, uint32_t tag, const WalkArgs &a) {
    return philox10(make_uint4(n, tag, P.lo, P.hi), a.keys);
}

// Birth of photon gid: wavelength (monte_carlo3D.py:1516-1520), optics row, the
// incident direction and Stokes vector (:1121-1132) and step 1's draws
// (initial_pdfs, :1035-1038).
__device__ __forceinline__ void pol_birth(PolPhoton &P, const WalkArgs &a, int64_t gid) {
    const int ci = find_config(a.prefix, a.n_cfg, gid);
    const DevConfig &c = a.cfgs[ci];
    const uint64_t rid = c.rng_base + (uint64_t)(gid - c.offset);
    P.lo = (uint32_t)rid;
    P.hi = (uint32_t)(rid >> 32);
    const uint4 rb = philox10(make_uint4(0u, kTagBirth, P.lo, P.hi), a.keys);
    float sbn, cbn;
    __sincosf(kTwoPiF * (u01_f32(rb.y) - 0.5f), &sbn, &cbn);
    const float zb = sqrtf(-2.f * __logf(u01_f32(rb.x))) * cbn;
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

// The envelope of the rejection sampler for the photon's Stokes vector
// (populate_pdfs, monte_carlo3D.py:929-951).
struct Envelope {
    float max1, max2, pa1;
};

__device__ __forceinline__ Envelope envelope(const PolPhoton &P) {
    const DevPhase32 &ph = *P.ph;
    const float C = sqrtf(fmaf(P.Q, P.Q, P.U * P.U));
    Envelope v;
    v.max1 = fmaf(fabsf(P.I), __ldg(ph.a1 + P.row), __ldg(ph.b1 + P.row) * C);
    v.max2 = fmaf(fabsf(P.I), __ldg(ph.a2 + P.row), __ldg(ph.b2 + P.row) * C);
    const float area1 = (ph.cos_max - ph.cos_cutoff) * v.max1;
    const float area2 = (ph.cos_cutoff - ph.cos_min) * v.max2;
    v.pa1 = __fdividef(area1, area1 + area2);
    return v;
}

// Candidate j of step n (:953-1001): its cosine and azimuth, and whether it passes.
__device__ __forceinline__ bool candidate(const DevPhase32 &ph, int row, float I, float Q, float U,
                                          const Envelope &v, uint32_t n, uint32_t j, uint32_t lo, uint32_t hi,
                                          const PhiloxKeys &ks, float &cos_theta, float &cphi, float &sphi) {
    const uint4 r = philox10(make_uint4(n, kTagPolCand | (j << 8), lo, hi), ks);
    const bool one = u01_f32(r.x) < v.pa1;
    const float uc = u01_f32(r.y);
    azimuth(u01_f32(r.z), cphi, sphi);
    cos_theta = one ? fmaf(uc, ph.cos_max - ph.cos_cutoff, ph.cos_cutoff)
                    : fmaf(-uc, ph.cos_cutoff - ph.cos_min, ph.cos_cutoff);
    const float r3 = 1.000001f * u01_f32(r.w) * (one ? v.max1 : v.max2);
    float S11, S12;
    if (ph.shared_grid) {
        const int k = segment_seeded(ph, cos_theta);
        S11 = phase_at(ph, 0, row, k, cos_theta);
        S12 = phase_at(ph, 1, row, k, cos_theta);
    } else {
        S11 = phase_el(ph, 0, row, cos_theta);
        S12 = phase_el(ph, 1, row, cos_theta);
    }
    const float c2 = fmaf(2.f * cphi, cphi, -1.f), s2 = 2.f * sphi * cphi;
    const float pf = fmaf(I, S11, S12 * fmaf(Q, c2, U * s2));
    return !(r3 > pf);
}

// The rest of the step (monte_carlo3D.py:1227-1466) with its scattering angles.
// Returns the end condition (0: still walking).
__device__ __forceinline__ int pol_step_post(PolPhoton &P, const WalkArgs &a, float p_cos, float cphi, float sphi) {
    const DevPhase32 &ph = *P.ph;
    const float dtau = (P.lam_surface && P.i == 1) ? 0.f : -__logf(u01_f32(P.sb.x));   // :1227-1229
    float nx = P.mux, ny = P.muy, nz = P.muz;
    if (P.i > 1) {
        // direction (:1238-1281): Lambertian about the vertical, or the rotation
        float m0x = P.mux, m0y = P.muy, m0z = P.muz, ct = p_cos;
        if (P.lam_surface || P.bref) {
            m0x = 0.f; m0y = 0.f; m0z = 1.f;
            ct = sqrtf(u01_f32(P.sb.w));
        }
        const float st = sqrtf(fmaxf(0.f, fmaf(-ct, ct, 1.f)));
        // sqrt(mu_x^2 + mu_y^2) stands for sqrt(1 - mu_z^2) (equal for a unit
        // direction; the frame stays orthogonal next to the pole in FP32); the
        // pole formula when it is 0 (or below FLT_MIN, where the reciprocal square
        // root would not be finite), the reference's mu_z == +-1
        const float s2 = fmaf(m0x, m0x, m0y * m0y);
        if (!(s2 >= 1.17549435e-38f)) {
            const float sg = copysignf(1.f, m0z);
            nx = st * cphi;
            ny = sg * st * sphi;
            nz = sg * ct;
        } else {
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
            float Pe[6];
            if (ph.shared_grid) {
                const int k = segment_seeded(ph, ct);
#pragma unroll
                for (int e = 0; e < 6; ++e) Pe[e] = phase_at(ph, e, P.row, k, ct);
            } else {
#pragma unroll
                for (int e = 0; e < 6; ++e) Pe[e] = phase_el(ph, e, P.row, ct);
            }
            const float P11 = Pe[0], P12 = Pe[1], P22 = Pe[2], P33 = Pe[3], P43 = Pe[4], P44 = Pe[5];
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
    const bool imp = (float)P.sb.z * kTwo32Inv < P.p_imp;
    const float coalb = imp ? P.coalb_imp : P.coalb_ice;
    int cond = 0;
    if (zn > 0.f) {
        cond = 1;
        P.path -= __fdividef(zn, zn - P.z) * inc;
    } else if (zn < -P.tau) {
        P.path -= __fdividef(zn + P.tau, zn - P.z) * inc;
        zn = -P.tau;
        if (P.lam_bottom && u01_f32(step_block(P, (uint32_t)P.i, kTagPolRefl, a).x) <= P.R) P.bref = true;
        else cond = (P.i == 1) ? 3 : 2;
    } else if ((float)P.sb.y * kTwo32Inv < coalb) {
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

// Warp-synchronous: every lane of the warp stays in the loop until none has a
// photon left, so the rejection rounds and claims can use the whole warp.
__global__ void __launch_bounds__(kPolBlock) walk_pol32_kernel(const WalkArgs a) {
    const unsigned long long t0 = global_ns();
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    // lanes without a photon still source the round's shuffles (their values are
    // never selected), so the state starts defined
    PolPhoton P{};
    P.ph = a.phase;
    bool have = false, exhausted = false;
    for (uint32_t it = 0;; ++it) {
        // ---- claims: lanes without a photon take the next ones, one atomic per warp
        const unsigned need = __ballot_sync(0xffffffffu, !have && !exhausted);
        if (need) {
            unsigned long long base = 0;
            if (lane == __ffs(need) - 1) base = atomicAdd(a.work, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (!have && !exhausted) {
                const unsigned long long g = base + __popc(need & lt_mask);
                if (g < (unsigned long long)a.total) {
                    pol_birth(P, a, (int64_t)g);
                    have = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;

        // ---- this step's draws; scattering angles for steps after the first
        bool pending = false;
        Envelope env{0.f, 0.f, 0.f};
        uint32_t jbase = 0;
        float p_cos = 1.f, cphi = 0.f, sphi = 0.f;
        if (have) {
            P.i += 1;
            P.sb = step_block(P, (uint32_t)P.i, kTagPolStep, a);
            if (P.i > 1) {
                env = envelope(P);
                pending = true;
            }
        }
        // ---- rejection rounds (:953-1001): the n pending photons share the lanes;
        // lane l tests candidate jbase + l / n of the photon of rank l % n, and a
        // photon takes its lowest-indexed passing candidate
        unsigned pend = __ballot_sync(0xffffffffu, pending);
        for (uint32_t round = 0; pend; ++round) {
            const int np = __popc(pend);
            const int r = lane % np, q = lane / np;
            const int owner = __fns(pend, 0, r + 1);
            const int o_row = __shfl_sync(0xffffffffu, P.row, owner);
            const float o_I = __shfl_sync(0xffffffffu, P.I, owner);
            const float o_Q = __shfl_sync(0xffffffffu, P.Q, owner);
            const float o_U = __shfl_sync(0xffffffffu, P.U, owner);
            Envelope o_env;
            o_env.max1 = __shfl_sync(0xffffffffu, env.max1, owner);
            o_env.max2 = __shfl_sync(0xffffffffu, env.max2, owner);
            o_env.pa1 = __shfl_sync(0xffffffffu, env.pa1, owner);
            const uint32_t o_n = (uint32_t)__shfl_sync(0xffffffffu, P.i, owner);
            const uint32_t o_lo = __shfl_sync(0xffffffffu, P.lo, owner);
            const uint32_t o_hi = __shfl_sync(0xffffffffu, P.hi, owner);
            const uint32_t o_j = __shfl_sync(0xffffffffu, jbase, owner) + (uint32_t)q;
            const DevPhase32 *o_ph = reinterpret_cast<const DevPhase32 *>(
                __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(P.ph), owner));
            float c_cos, c_cphi, c_sphi;
            const bool pass = candidate(*o_ph, o_row, o_I, o_Q, o_U, o_env, o_n, o_j, o_lo, o_hi, a.keys,
                                        c_cos, c_cphi, c_sphi);
            const unsigned acc = __ballot_sync(0xffffffffu, pass);
            int src = lane;
            bool got = false;
            if (pending) {
                const int me = __popc(pend & lt_mask);
                unsigned group = 0;
                for (int l = me; l < 32; l += np) group |= 1u << l;
                const unsigned hit = acc & group;
                if (hit) {
                    src = __ffs(hit) - 1;
                    got = true;
                } else {
                    jbase += (uint32_t)__popc(group);
                }
            }
            const float w_cos = __shfl_sync(0xffffffffu, c_cos, src);
            const float w_cphi = __shfl_sync(0xffffffffu, c_cphi, src);
            const float w_sphi = __shfl_sync(0xffffffffu, c_sphi, src);
            if (got) {
                p_cos = w_cos;
                cphi = w_cphi;
                sphi = w_sphi;
                pending = false;
            } else if (pending && jbase >= kMaxCandidates) {
                atomicOr(a.status, kStatusStream);   // a candidate range no envelope should need
                pending = false;
            }
            pend = __ballot_sync(0xffffffffu, pending);
            if ((round & 255u) == 255u) {
                int over = 0;
                if (lane == 0) over = global_ns() - t0 > a.budget_ns;
                if (__shfl_sync(0xffffffffu, over, 0)) {
                    if (lane == 0) atomicOr(a.status, kStatusBudget);
                    return;
                }
            }
        }

        // ---- the rest of the step; finished photons leave their records
        if (have) {
            const int cond = pol_step_post(P, a, p_cos, cphi, sphi);
            if (cond > 0) {
                pol_finish(P, a, cond);
                have = false;
            }
        }
        if ((it & 1023u) == 1023u) {
            int stop = 0;
            if (lane == 0)
                stop = (global_ns() - t0 > a.budget_ns) || (*(volatile unsigned int *)a.status & kStatusBudget);
            if (__shfl_sync(0xffffffffu, stop, 0)) {
                if (lane == 0) atomicOr(a.status, kStatusBudget);
                return;
            }
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
