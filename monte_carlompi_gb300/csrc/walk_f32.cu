// Production FP32 photon walk: a persistent grid of warps, each lane walking
// one photon at a time.  Photon ids come from one global counter; a warp
// refills its idle lanes (photon regeneration) so lanes whose photons leave
// early keep working instead of idling until the warp's longest walk ends.
//
// Births and finishes are batched through per-warp shared-memory queues so
// their expensive parts run with all 32 lanes busy:
//  * births: when the warp's queue of ready photons runs short, every lane
//    starts one new photon (Philox + Box-Muller wavelength + SSP lookup) into
//    the queue; idle lanes then pop a ready photon (a few shared loads);
//  * finishes: a lane whose photon ends pushes its final state to the warp's
//    finish queue; once 32 are queued the warp computes theta_n / phi_n,
//    writes the 32 records and folds the tallies with warp reductions.
//
// The end of a launch: once the photon supply is exhausted, the warps empty
// out and the last, longest walks (a few hundred to ~1,500 events) would run
// with a few lanes of a warp each, bound by the latency of one photon's step
// chain.  A warp with at most kSparseWarp photons runs sparse rounds: its 32
// lanes compute the direction-independent part of the photons' next steps at
// once (Philox block, HG and Lambertian angles, azimuth, optical path; up to 32
// steps of a lone photon) and each photon's lane then runs only the chain that
// remains (rotation, move, boundaries).
//
// Photons past kBlockWalk steps walk in block passes of up to 512 steps, a warp
// per photon.  Optionally (WalkArgs::drain_from > 0), once the photon supply is
// exhausted, a photon past drain_from steps leaves the walk (its state packed
// into a device queue) and the drain kernel launched after the walk gives each
// such photon a whole thread block, a warp per 64 steps of every pass.  Nothing
// waits on anything: the queue is complete when the drain kernel starts.  The
// arithmetic of a step and of a pass is the same on every path, so records do
// not depend on where or how a photon ends its walk.
//
// Per step (monte_carloMPI/monte_carlo3D.py:1212-1466, HG branch) one
// Philox4x32-10 block keyed by (step, photon) supplies the four uniforms the
// step needs: HG cosine (:915), azimuth (:921), optical path (:1014) and the
// absorption draw (:1020).  The ice/impurity draw (:1023) and the bottom
// reflectance draw (:1422/:1453) take their own blocks only when the config
// needs them.  Results depend only on (seed, photon stream id): any launch
// shape, any number of GPUs or replicas gives the same records.
//
// Restatements whose distributions equal the reference's in exact arithmetic
// (the FP32 walk then differs from it by rounding and by the resolution of its
// draws: 2^-23 for the angle uniforms, 2^-32 for the path and absorption ones):
//  * the Lambertian direction (p(theta) ~ sin 2 theta, :1238-1250) is drawn by
//    inversion, cos theta = sqrt(u), instead of rejection;
//  * absorption tests 1 - u < 1 - ssa on a 32-bit uniform, so small
//    co-albedos (1e-6) are resolved; likewise the species test;
//  * the azimuth is uniform on (-pi, pi) instead of (0, 2 pi);
//  * the rotation (:1270-1281) takes sqrt(mu_x^2 + mu_y^2) where the reference
//    writes sqrt(1 - mu_z^2): equal for a unit direction, and with it the
//    rotation's frame stays orthogonal next to the pole, where 1 - mu_z^2 loses
//    its digits in FP32.  The pole branch (:1262-1269) is taken when that
//    horizontal part is exactly 0, the reference's mu_z == +-1;
//  * the direction is renormalised once per 4-step round (and at the end of
//    every block pass), which only removes rounding drift;
//  * past kBlockWalk steps the directions are composed in a moving frame
//    (block passes) instead of the z-referenced rotation formula (:1270-1281);
//  * phi_n = atan2(mu_y, mu_x) mapped to [0, 2 pi) (the quadrant arctan of
//    :1472-1485, defined on the axes too).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "mcw_internal.cuh"
#include "tally.cuh"

namespace mcw {

namespace {

constexpr float kTwoPiF = 6.28318530717958648f;
constexpr float kTwo32Inv = 2.3283064365386963e-10f;  // 2^-32
constexpr float kTwo33Inv = 1.16415321826934814e-10f; // 2^-33
constexpr uint32_t kFlagReflect = 8u;                  // bottom reflection pending
constexpr int kSmemCfgMax = 256;                       // configs staged in shared memory
constexpr int kFinishCap = 64;                         // finish queue entries per warp
#ifndef MCW_BLOCK_WALK
#define MCW_BLOCK_WALK 256
#endif
// steps after which a photon (not on a Lambertian surface) walks in block passes
// (block_pass); a multiple of 4, so every path reaches it at a round edge
constexpr int kBlockWalk = MCW_BLOCK_WALK;
#ifndef MCW_STEPS_PER_ROUND
#define MCW_STEPS_PER_ROUND 4
#endif
// scatter events per loop round: their Philox blocks are computed together so
// the ten dependent Philox rounds of one overlap those of the others
constexpr int kStepsPerRound = MCW_STEPS_PER_ROUND;
static_assert(kStepsPerRound >= 1 && kStepsPerRound <= 32 && (kStepsPerRound & (kStepsPerRound - 1)) == 0,
              "steps per round: a power of two");
constexpr int kLogStepsPerRound = __builtin_ctz(kStepsPerRound);
#ifndef MCW_SPARSE_WARP
#define MCW_SPARSE_WARP (32 / kStepsPerRound)
#endif
// a warp with at most this many active lanes runs sparse rounds; each lane
// precomputes one or two steps of them
constexpr int kSparseWarp = MCW_SPARSE_WARP;
constexpr int kSparseSlots = kSparseWarp * kStepsPerRound > 32 ? 64 : 32;
static_assert(kSparseWarp >= 1 && kSparseWarp * kStepsPerRound <= 64, "sparse rounds: at most 64 steps");

// Per-config values the FP32 walk reads at photon birth.
struct CfgF32 {
    int32_t lut_off, lut_n, k_lo;
    uint32_t flags;
    float wvl0_100, sigma_100, mux0, muz0;
    float tau_tot, R;
    uint64_t rng_base;
};

__device__ __forceinline__ CfgF32 make_cfg(const DevConfig &c) {
    CfgF32 f;
    f.lut_off = c.lut_off;
    f.lut_n = c.lut_n;
    f.k_lo = c.k_lo;
    f.flags = c.flags;
    f.wvl0_100 = c.wvl0_100;
    f.sigma_100 = c.sigma_100;
    f.mux0 = c.mux0;
    f.muz0 = c.muz0;
    f.tau_tot = c.tau_tot;
    f.R = c.R;
    f.rng_base = c.rng_base;
    return f;
}

// Live state of a walking photon (registers).
struct Photon {
    uint64_t rid;      // stream id: config << 40 | photon index
    int32_t cfg;       // -1: lane idle
    int32_t lut, i;
    uint32_t flags;
    float mux, muy, muz, z, path, pathc;
    float tau, R;
    float inv_ext, coalb_ice, coalb_imp, p_imp;
    float hg_a, hg_b, hg_c, hg_d, hg_e;  // 1+g^2, 1-g^2, 1-g, 2g, 1/(2g); hg_d == 0: isotropic
};

// A photon walks in block mode (block_pass) from kBlockWalk steps on, except on a
// Lambertian surface (whose directions do not follow from the previous one).
// kDeep: no config of the launch is a Lambertian surface (WalkArgs::deep).
template <bool kDeep>
__device__ __forceinline__ bool in_block_mode(const Photon &P) {
    return P.cfg >= 0 && P.i >= kBlockWalk && (kDeep || !(P.flags & kFlagLamSurface));
}

// A photon handed to the drain queue: kDrainSlot = 6 float4.
__device__ __forceinline__ void pack_photon(float4 *d, const Photon &P) {
    d[0] = make_float4(__uint_as_float((uint32_t)P.rid), __uint_as_float((uint32_t)(P.rid >> 32)),
                       __int_as_float(P.cfg), __int_as_float(P.lut));
    d[1] = make_float4(__int_as_float(P.i), __uint_as_float(P.flags), P.mux, P.muy);
    d[2] = make_float4(P.muz, P.z, P.path, P.pathc);
    d[3] = make_float4(P.tau, P.R, P.inv_ext, P.coalb_ice);
    d[4] = make_float4(P.coalb_imp, P.p_imp, P.hg_a, P.hg_b);
    d[5] = make_float4(P.hg_c, P.hg_d, P.hg_e, 0.f);
}

__device__ __forceinline__ void unpack_photon(Photon &P, const float4 *d) {
    const float4 a = d[0], b = d[1], c = d[2], e = d[3], f = d[4], g = d[5];
    P.rid = ((uint64_t)__float_as_uint(a.y) << 32) | __float_as_uint(a.x);
    P.cfg = __float_as_int(a.z);
    P.lut = __float_as_int(a.w);
    P.i = __float_as_int(b.x);
    P.flags = __float_as_uint(b.y);
    P.mux = b.z, P.muy = b.w;
    P.muz = c.x, P.z = c.y, P.path = c.z, P.pathc = c.w;
    P.tau = e.x, P.R = e.y, P.inv_ext = e.z, P.coalb_ice = e.w;
    P.coalb_imp = f.x, P.p_imp = f.y, P.hg_a = f.z, P.hg_b = f.w;
    P.hg_c = g.x, P.hg_d = g.y, P.hg_e = g.z;
}

// A born photon waiting in the queue: 20 words = 5 x float4.
struct __align__(16) BirthSlot {
    uint32_t rid_lo, rid_hi, cfg, lut;
    uint32_t flags;
    float mux, muz, tau;
    float R, inv_ext, coalb_ice, coalb_imp;
    float p_imp, hg_a, hg_b, hg_c;
    float hg_d, hg_e, pad0, pad1;
};

// A finished photon waiting for the batched epilogue: 12 words = 3 x float4.
struct __align__(16) FinishSlot {
    uint32_t rid_lo, rid_hi, cfg, lut;
    int32_t n_step, cond;
    float mux, muy;
    float muz, path, pad0, pad1;
};

struct WarpQueues {
    BirthSlot birth[32];
    FinishSlot fin[kFinishCap];
    uint4 rmeta[3 * kSparseWarp];             // sparse round: each photon's stream, step and constants
    float4 pbuf[2 * kSparseSlots];            // sparse round: StepPre of up to 64 steps
    WarpTally tally;
};

template <int N>
__device__ __forceinline__ void copy_f4(void *dst, const void *src) {
    float4 *d = reinterpret_cast<float4 *>(dst);
    const float4 *s = reinterpret_cast<const float4 *>(src);
#pragma unroll
    for (int q = 0; q < N; ++q) d[q] = s[q];
}

// Start photon p (index within its config) of config ci into a queue slot.
__device__ __forceinline__ void birth(BirthSlot &b, int64_t p, int ci, const CfgF32 &c, const WalkArgs &a) {
    const uint64_t rid = c.rng_base + (uint64_t)p;
    const uint4 r = philox10(make_uint4(0u, kTagBirth, (uint32_t)rid, (uint32_t)(rid >> 32)), a.keys);
    // Box-Muller normal for the wavelength (monte_carlo3D.py:1516-1520)
    const float u0 = u01_f32(r.x), u1 = u01_f32(r.y);
    float s, co;
    __sincosf(kTwoPiF * (u1 - 0.5f), &s, &co);
    const float zn = sqrtf(-2.f * __logf(u0)) * co;
    const int k = __float2int_rn(fmaf(c.sigma_100, zn, c.wvl0_100));
    const int idx = min(max(k - c.k_lo, 0), c.lut_n - 1);
    const int lut = c.lut_off + idx;
    const LutEntry *e = a.lut + lut;
    const float4 e0 = __ldg(reinterpret_cast<const float4 *>(e));      // wvn, coalb_ice, coalb_imp, g
    const float4 e1 = __ldg(reinterpret_cast<const float4 *>(e) + 1);  // inv_ext, p_imp, snow_depth, -
    const float g = e0.w;
    BirthSlot o;
    o.rid_lo = (uint32_t)rid;
    o.rid_hi = (uint32_t)(rid >> 32);
    o.cfg = (uint32_t)ci;
    o.lut = (uint32_t)lut;
    o.flags = c.flags;
    o.mux = c.mux0;
    o.muz = c.muz0;
    o.tau = c.tau_tot;
    o.R = c.R;
    o.inv_ext = e1.x;
    o.coalb_ice = e0.y;
    o.coalb_imp = e0.z;
    o.p_imp = e1.y;
    if (fabsf(g) > 1e-6f) {
        o.hg_a = 1.f + g * g;
        o.hg_b = 1.f - g * g;
        o.hg_c = 1.f - g;
        o.hg_d = 2.f * g;
        o.hg_e = 0.5f / g;
    } else {  // isotropic: keep the HG expression finite (t = 0); the step selects 1 - 2u
        o.hg_a = o.hg_b = o.hg_d = o.hg_e = 0.f;
        o.hg_c = 1.f;
    }
    o.pad0 = o.pad1 = 0.f;
    copy_f4<5>(&b, &o);
}

__device__ __forceinline__ void pop(Photon &P, const BirthSlot &b) {
    BirthSlot o;
    copy_f4<5>(&o, &b);
    P.rid = ((uint64_t)o.rid_hi << 32) | o.rid_lo;
    P.cfg = (int32_t)o.cfg;
    P.lut = (int32_t)o.lut;
    P.i = 0;
    P.flags = o.flags;
    P.mux = o.mux;
    P.muy = 0.f;
    P.muz = o.muz;
    P.z = 0.f;
    P.path = 0.f;
    P.pathc = 0.f;
    P.tau = o.tau;
    P.R = o.R;
    P.inv_ext = o.inv_ext;
    // on a Lambertian surface every step's absorption test uses 1 - R (:1455-1466)
    const bool lam_surface = (o.flags & kFlagLamSurface) != 0;
    P.coalb_ice = lam_surface ? 1.f - o.R : o.coalb_ice;
    P.coalb_imp = lam_surface ? 1.f - o.R : o.coalb_imp;
    P.p_imp = o.p_imp;
    P.hg_a = o.hg_a;
    P.hg_b = o.hg_b;
    P.hg_c = o.hg_c;
    P.hg_d = o.hg_d;
    P.hg_e = o.hg_e;
}

// The arithmetic shared by step() and step_post().  Every product and sum is
// rounded as written (explicit fmaf / __fmul_rn, no contraction left to the
// compiler), so the two paths give the same bits for the same draws.

// Independent pairs of operations go through the packed FP32 forms
// (__fadd2_rn, __fmul2_rn, __ffma2_rn): each lane of a pair is rounded as the
// scalar operation would be, in one issue slot instead of two.

// The step's four uniforms from its Philox block: (u1, u2) in [2^-24, 1 - 2^-24]
// from the top 23 bits (u01_f32), u3 = (z + 1/2) 2^-32 in (0, 1), u4 = w 2^-32.
__device__ __forceinline__ float4 step_uniforms(const uint4 r) {
    const float2 a = __fadd2_rn(make_float2(__uint_as_float(0x3F800000u | (r.x >> 9)),
                                            __uint_as_float(0x3F800000u | (r.y >> 9))),
                                make_float2(-0.99999994f, -0.99999994f));
    const float2 b = __ffma2_rn(make_float2((float)r.z, (float)r.w), make_float2(kTwo32Inv, kTwo32Inv),
                                make_float2(kTwo33Inv, 0.f));
    return make_float4(a.x, a.y, b.x, b.y);
}

// Henyey-Greenstein scattering cosine by inversion (monte_carlo3D.py:915), or
// 1 - 2u when isotropic (hg_d == 0).  kAniso: no photon of the launch is isotropic
// (WalkArgs::deep), the same value without the isotropic alternative.
template <bool kAniso = false>
__device__ __forceinline__ float hg_cos(const float u1, const float hg_a, const float hg_b, const float hg_c,
                                        const float hg_d, const float hg_e) {
    if (kAniso) {
        const float t = __fdividef(hg_b, fmaf(hg_d, u1, hg_c));
        return __fmul_rn(hg_e, fmaf(-t, t, hg_a));
    }
    const float2 d = __ffma2_rn(make_float2(hg_d, -2.f), make_float2(u1, u1), make_float2(hg_c, 1.f));
    const float t = __fdividef(hg_b, d.x);
    return (hg_d != 0.f) ? __fmul_rn(hg_e, fmaf(-t, t, hg_a)) : d.y;
}

__device__ __forceinline__ float sin_of(const float ct) { return sqrtf(fmaxf(0.f, fmaf(-ct, ct, 1.f))); }

// Squared horizontal part of a direction, mu_x^2 + mu_y^2 (= 1 - mu_z^2 for a
// unit direction).  0 exactly on the vertical: the pole case of the reference
// (mu_z == +-1, monte_carlo3D.py:1262-1269); the kernel flushes denormals, so a
// non-zero value is at least FLT_MIN and its reciprocal square root is finite.
__device__ __forceinline__ float horiz2(const float mx, const float my) { return fmaf(mx, mx, __fmul_rn(my, my)); }
constexpr float kFltMin = 1.17549435e-38f;

// General rotation of direction m by polar cosine/sine (ct, st) and azimuth
// (cp, sp) (monte_carlo3D.py:1270-1281), renormalised when `renorm`; s2 =
// horiz2(mx, my).  With s = sqrt(s2) taken from m's own horizontal part, the
// frame (m, (mx mz / s, my mz / s, -s), (-my / s, mx / s, 0)) is orthogonal and
// its second vector is as long as m, however close m is to the vertical.
__device__ __forceinline__ float3 rotate(const float mx, const float my, const float mz, const float s2in,
                                         const float ct, const float st, const float cp, const float sp,
                                         const bool renorm) {
    const float s2 = fmaxf(s2in, kFltMin);
    const float rs = rsqrtf(s2);
    const float tq = __fmul_rn(st, rs);
    // x and y as pairs: (mx mz cp - my sp, my mz cp + mx sp), then tq * that + (mx ct, my ct)
    const float2 m = make_float2(mx, my);
    const float2 mzp = __fmul2_rn(m, make_float2(mz, mz));
    const float2 spp = __fmul2_rn(make_float2(-my, mx), make_float2(sp, sp));
    const float2 in = __ffma2_rn(mzp, make_float2(cp, cp), spp);
    float2 gxy = __ffma2_rn(make_float2(tq, tq), in, __fmul2_rn(m, make_float2(ct, ct)));
    float gz = fmaf(-__fmul_rn(__fmul_rn(s2, rs), st), cp, __fmul_rn(mz, ct));
    if (renorm) {
        const float inv = rsqrtf(fmaf(gxy.x, gxy.x, fmaf(gxy.y, gxy.y, __fmul_rn(gz, gz))));
        gxy = __fmul2_rn(gxy, make_float2(inv, inv));
        gz = __fmul_rn(gz, inv);
    }
    return make_float3(gxy.x, gxy.y, gz);
}

// The pole case (monte_carlo3D.py:1262-1269): sg = sign of mu_z.
__device__ __forceinline__ float3 pole_dir(const float sg, const float ct, const float st, const float cp,
                                           const float sp) {
    return make_float3(__fmul_rn(st, cp), __fmul_rn(__fmul_rn(sg, st), sp), __fmul_rn(sg, ct));
}

// The end of a step's move (monte_carlo3D.py:1390-1466): the exit correction of the path
// at the top or bottom (:1390-1459), the clamp at the bottom and the reflectance draw of
// a Lambertian bottom (:1422, :1453; the step's absorption word, since a step that
// reaches the bottom is never tested for absorption), else the absorption test
// (:1461-1466).  Returns the end condition (0: walking on, or reflected).  kDeep: the
// bottom branch is rare in the warp and is a branch; otherwise every alternative is
// evaluated and selected.  Both give the same values.
template <bool kDeep>
__device__ __forceinline__ int boundary(Photon &P, float &zn, const float z0, const float inc, const float u4,
                                        const float coalb, const bool top, const bool bot, const bool first,
                                        const bool imp) {
    if (kDeep) {
        P.flags &= ~kFlagReflect;
        if (bot) {
            P.path = fmaf(-__fdividef(zn + P.tau, zn - z0), inc, P.path);
            zn = -P.tau;
            const bool refl = (P.flags & kFlagLamBottom) && u4 < P.R;
            if (refl) P.flags |= kFlagReflect;
            return refl ? 0 : (first ? 3 : 2);
        }
        if (top) P.path = fmaf(-__fdividef(zn, zn - z0), inc, P.path);
        return top ? 1 : ((u4 < coalb) ? (imp ? 5 : 4) : 0);
    }
    const float2 fd = __fadd2_rn(make_float2(zn, zn), make_float2(P.tau, -z0));
    const float frac = __fdividef(top ? zn : fd.x, fd.y);
    if (top || bot) P.path = fmaf(-frac, inc, P.path);
    zn = bot ? -P.tau : zn;
    const bool refl = bot && (P.flags & kFlagLamBottom) && u4 < P.R;
    P.flags = (P.flags & ~kFlagReflect) | (refl ? kFlagReflect : 0u);
    const bool absorb = u4 < coalb;
    return top ? 1 : (bot ? (refl ? 0 : (first ? 3 : 2)) : (absorb ? (imp ? 5 : 4) : 0));
}

// One scatter event (monte_carlo3D.py:1213-1466) with its step block r =
// Philox(step P.i + 1, photon) already computed.  Returns the end condition
// (0 = still walking).  The first step and the general rotation are evaluated
// together and selected; the Lambertian direction and the pole case are rare
// branches; top, bottom and absorption are selected (the deep instance branches
// on the rare bottom crossing, see boundary()).  The dense rounds of the other
// instances walk with it; the deep instance's dense rounds and every sparse round
// split it into step_pre / step_pre_dense and step_post, with the same values.
template <bool kImpurity, bool kDeep>
// may_first: this step can be a photon's first (photons start on a round edge, so only
// a round's step 0 can; a constant at every call, so the first-step selects of the
// other steps compile away).  kDeep: the slabs of the launch are optically deep, so a
// bottom crossing is rare in a warp and takes a branch (otherwise selects), and no config
// is a Lambertian surface.  The values are the same either way.
__device__ __forceinline__ int step(Photon &P, const WalkArgs &a, const uint4 r, const bool renorm,
                                    const bool may_first) {
    P.i += 1;
    const float4 uu = step_uniforms(r);
    const float u1 = uu.x, u2 = uu.y, u3 = uu.z;
    const bool first = may_first && (P.i == 1);
    const bool lam_surface = !kDeep && (P.flags & kFlagLamSurface) != 0;   // none in the deep instance
    const bool lamb = !first && (lam_surface || (P.flags & kFlagReflect));

    const float dtau = (first && lam_surface) ? 0.f : -__logf(u3);

    // scattering cosine: HG inversion (isotropic when hg_d == 0), or the
    // Lambertian cos = sqrt(u) after a bottom reflection
    float ct = hg_cos<kDeep>(u1, P.hg_a, P.hg_b, P.hg_c, P.hg_d, P.hg_e);
    if (lamb) ct = sqrtf(u1);                                   // rare: a branch, not a select
    const float st = sin_of(ct);
    float sp, cp;
    __sincosf(kTwoPiF * (u2 - 0.5f), &sp, &cp);

    const float s2 = horiz2(P.mux, P.muy);
    float3 g = rotate(P.mux, P.muy, P.muz, s2, ct, st, cp, sp, renorm);
    // the pole case (rare: a branch): the direction is exactly vertical, or it is drawn
    // about the vertical after a bottom reflection (the pole case of mu = (0, 0, 1))
    if (lamb || !(s2 > 0.f)) g = pole_dir(lamb ? 1.f : copysignf(1.f, P.muz), ct, st, cp, sp);
    const float nx = first ? P.mux : g.x;     // a first step is never after a reflection
    const float ny = first ? P.muy : g.y;
    const float nz = first ? P.muz : g.z;

    const float z0 = P.z;
    // zn = dtau nz + z0 and the path increment dtau / (ext rho) as one pair
    const float2 zi = __ffma2_rn(make_float2(dtau, dtau), make_float2(nz, P.inv_ext), make_float2(z0, 0.f));
    float zn = zi.x;
    // path length, compensated sum
    const float inc = zi.y;
    {
        const float y = inc - P.pathc;
        const float tt = P.path + y;
        P.pathc = (tt - P.path) - y;
        P.path = tt;
    }

    // ice or impurity (monte_carlo3D.py:1375-1383); the draw exists only when imp_cnc > 0
    bool imp = false;
    if (kImpurity && (P.flags & kFlagImpurity)) {
        const uint4 r2 = philox10(make_uint4((uint32_t)P.i, kTagSpecies, (uint32_t)P.rid,
                                             (uint32_t)(P.rid >> 32)), a.keys);
        imp = ((float)r2.x * kTwo32Inv) < P.p_imp;
    }
    const float coalb = imp ? P.coalb_imp : P.coalb_ice;       // 1 - R on a Lambertian surface

    const bool top = zn > 0.f;                                  // :1390-1397
    const bool bot = zn < -P.tau;                               // :1399-1459
    // r.w is the absorption draw; a step that reaches the bottom is never tested
    // for absorption (the reference's elif chain), so there it is the
    // Lambertian-bottom reflectance draw (:1422, :1453)
    const float u4 = uu.w;
    const int cond = boundary<kDeep>(P, zn, z0, inc, u4, coalb, top, bot, first, imp);
    P.mux = nx;
    P.muy = ny;
    P.muz = nz;
    P.z = zn;
    return cond;
}

// The same scatter event as step(), split for the sparse rounds: the part that
// does not depend on the photon's direction or position (everything drawn from the
// step's Philox block and the photon's phase-function constants), computed for up
// to 32 steps at once across the lanes of a warp, and the chain that does.  Every value is
// the same function of the same inputs as in step(): st is sqrt(1 - ct^2) of the
// selected cosine whichever way the selection is made.
struct StepPre {
    float ct_hg, st_hg;   // HG scattering cosine (monte_carlo3D.py:915), or 1 - 2u if isotropic
    float ct_l, st_l;     // Lambertian direction after a reflection, cos = sqrt(u)
    float sp, cp;         // azimuth (:921), uniform on (-pi, pi)
    float dtau;           // optical path -ln u (:1014)
    float u4;             // absorption draw (:1020), or the bottom reflectance draw
    __device__ __forceinline__ float2 lambertian() const { return make_float2(ct_l, st_l); }
};

// The same part for the dense rounds, the Lambertian cosine left to the rare
// reflected step (taken from u1 there: the same sqrt of the same uniform).
struct StepPreDense {
    float ct_hg, st_hg, sp, cp, dtau, u4, u1;
    __device__ __forceinline__ float2 lambertian() const {
        const float c = sqrtf(u1);
        return make_float2(c, sin_of(c));
    }
};

// hg = (hg_a, hg_b, hg_c, hg_d) and hg_e of the photon (Photon::hg_*).
template <bool kDeep>
__device__ __forceinline__ StepPre step_pre(const uint4 r, const float4 hg, const float hg_e) {
    StepPre o;
    const float4 uu = step_uniforms(r);
    const float u1 = uu.x, u2 = uu.y, u3 = uu.z;
    o.dtau = -__logf(u3);
    o.ct_hg = hg_cos<kDeep>(u1, hg.x, hg.y, hg.z, hg.w, hg_e);
    o.st_hg = sin_of(o.ct_hg);
    o.ct_l = sqrtf(u1);
    o.st_l = sin_of(o.ct_l);
    __sincosf(kTwoPiF * (u2 - 0.5f), &o.sp, &o.cp);
    o.u4 = uu.w;
    return o;
}

template <bool kDeep>
__device__ __forceinline__ StepPreDense step_pre_dense(const uint4 r, const Photon &P) {
    StepPreDense o;
    const float4 uu = step_uniforms(r);
    o.u1 = uu.x;
    o.dtau = -__logf(uu.z);
    o.ct_hg = hg_cos<kDeep>(uu.x, P.hg_a, P.hg_b, P.hg_c, P.hg_d, P.hg_e);
    o.st_hg = sin_of(o.ct_hg);
    __sincosf(kTwoPiF * (uu.y - 0.5f), &o.sp, &o.cp);
    o.u4 = uu.w;
    return o;
}

// Ice or impurity for step n (monte_carlo3D.py:1023, :1375-1383), as in step().
__device__ __forceinline__ bool impurity_draw(uint64_t rid, uint32_t n, float p_imp, const WalkArgs &a) {
    const uint4 r2 = philox10(make_uint4(n, kTagSpecies, (uint32_t)rid, (uint32_t)(rid >> 32)), a.keys);
    return ((float)r2.x * kTwo32Inv) < p_imp;
}

template <bool kDeep, class Pre>
__device__ __forceinline__ int step_post(Photon &P, const Pre &s, const bool imp, const bool renorm,
                                         const bool may_first) {
    P.i += 1;
    const bool first = may_first && (P.i == 1);
    const bool lam_surface = !kDeep && (P.flags & kFlagLamSurface) != 0;   // none in the deep instance
    const bool lamb = !first && (lam_surface || (P.flags & kFlagReflect));
    const float dtau = (first && lam_surface) ? 0.f : s.dtau;
    // The HG rotation of the current direction does not wait for `lamb` (which
    // depends on the previous step's bottom test): a Lambertian direction is the
    // pole case of mu = (0, 0, 1) and is selected afterwards, so only that select
    // sits on the chain between steps.  Same values as step().
    const float s2 = horiz2(P.mux, P.muy);
    float3 g = rotate(P.mux, P.muy, P.muz, s2, s.ct_hg, s.st_hg, s.cp, s.sp, renorm);
    // the first step, a reflected direction and the pole are rare: a branch
    if (first || lamb || !(s2 > 0.f)) {
        if (first) g = make_float3(P.mux, P.muy, P.muz);
        else if (lamb) {
            const float2 l = s.lambertian();
            g = pole_dir(1.f, l.x, l.y, s.cp, s.sp);
        }
        else g = pole_dir(copysignf(1.f, P.muz), s.ct_hg, s.st_hg, s.cp, s.sp);
    }
    const float nx = g.x, ny = g.y, nz = g.z;
    const float z0 = P.z;
    const float2 zi = __ffma2_rn(make_float2(dtau, dtau), make_float2(nz, P.inv_ext), make_float2(z0, 0.f));
    float zn = zi.x;
    const float inc = zi.y;
    {
        const float y = inc - P.pathc;
        const float tt = P.path + y;
        P.pathc = (tt - P.path) - y;
        P.path = tt;
    }
    const float coalb = imp ? P.coalb_imp : P.coalb_ice;       // 1 - R on a Lambertian surface
    const bool top = zn > 0.f;
    const bool bot = zn < -P.tau;
    const int cond = boundary<kDeep>(P, zn, z0, inc, s.u4, coalb, top, bot, first, imp);
    P.mux = nx;
    P.muy = ny;
    P.muz = nz;
    P.z = zn;
    return cond;
}

// One round of a sparse warp (at most kSparseWarp photons; the end of a launch,
// when the last and longest walks would otherwise advance one step per lane per
// round with most lanes idle).  The photons publish their stream, step and
// phase-function constants; entry t (lane t, and lane t - 32 for a second pass)
// is the direction-independent part of step k = t % S of photon t / S, where
// S = 32 / n_act rounded down to a power of two, at least kStepsPerRound; then
// each photon's lane runs the chain of its S steps (step_post), leaving at its end
// condition.  S is a multiple of kStepsPerRound and rounds start at a multiple of
// it, so renormalisation falls on the same steps as in the dense rounds and the
// records are bit-identical.
template <bool kImpurity, bool kDeep>
__device__ __forceinline__ int sparse_round(Photon &P, WarpQueues &q, const unsigned act, const int n_act,
                                            const int lane, const unsigned lt_mask, const WalkArgs &a) {
    // 1 <= n_act <= kSparseWarp; S = 2^ls
    const int ls = max(kLogStepsPerRound, 5 - (32 - __clz(n_act - 1)));
    const int S = 1 << ls;
    const bool me = (act >> lane) & 1u;
    const int rank = __popc(act & lt_mask);
    if (me) {
        q.rmeta[3 * rank] = make_uint4((uint32_t)P.rid, (uint32_t)(P.rid >> 32), (uint32_t)P.i, P.flags);
        q.rmeta[3 * rank + 1] = make_uint4(__float_as_uint(P.hg_a), __float_as_uint(P.hg_b),
                                           __float_as_uint(P.hg_c), __float_as_uint(P.hg_d));
        q.rmeta[3 * rank + 2] = make_uint4(__float_as_uint(P.hg_e), __float_as_uint(P.p_imp), 0u, 0u);
    }
    __syncwarp();
    uint64_t impm = 0;
#pragma unroll
    for (int pass = 0; pass < kSparseSlots / 32; ++pass) {
        if (pass > 0 && (n_act << ls) <= 32) break;            // warp-uniform
        const int e = lane + 32 * pass;
        const int j = e >> ls, k = e & (S - 1);
        bool imp_t = false;
        if (j < n_act) {
            const uint4 m0 = q.rmeta[3 * j], m1 = q.rmeta[3 * j + 1], m2 = q.rmeta[3 * j + 2];
            const uint32_t n = m0.z + 1u + (uint32_t)k;
            const uint4 r = philox10(make_uint4(n, kTagStep, m0.x, m0.y), a.keys);
            const StepPre t = step_pre<kDeep>(r, make_float4(__uint_as_float(m1.x), __uint_as_float(m1.y),
                                                      __uint_as_float(m1.z), __uint_as_float(m1.w)),
                                       __uint_as_float(m2.x));
            q.pbuf[2 * e] = make_float4(t.ct_hg, t.st_hg, t.ct_l, t.st_l);
            q.pbuf[2 * e + 1] = make_float4(t.sp, t.cp, t.dtau, t.u4);
            if (kImpurity && (m0.w & kFlagImpurity))
                imp_t = impurity_draw(((uint64_t)m0.y << 32) | m0.x, n, __uint_as_float(m2.y), a);
        }
        if (kImpurity) impm |= (uint64_t)__ballot_sync(0xffffffffu, imp_t) << (32 * pass);
    }
    __syncwarp();
    int cond = 0;
    if (me) {
        // groups of kStepsPerRound steps (renormalised on a group's last step, as in the
        // dense rounds)
        for (int k0 = 0; k0 < S; k0 += kStepsPerRound) {
            if (in_block_mode<kDeep>(P)) break;                 // block mode from kBlockWalk on
            const int t0 = (rank << ls) + k0;
            float4 xs[kStepsPerRound], ys[kStepsPerRound];
#pragma unroll
            for (int u = 0; u < kStepsPerRound; ++u) {
                xs[u] = q.pbuf[2 * (t0 + u)];
                ys[u] = q.pbuf[2 * (t0 + u) + 1];
            }
            // each photon's lane leaves at its end condition (at most kSparseWarp lanes walk
            // here, so the divergence costs little); the state is the one after that step,
            // as in the dense rounds
#pragma unroll
            for (int u = 0; u < kStepsPerRound; ++u) {
                StepPre st;
                st.ct_hg = xs[u].x, st.st_hg = xs[u].y, st.ct_l = xs[u].z, st.st_l = xs[u].w;
                st.sp = ys[u].x, st.cp = ys[u].y, st.dtau = ys[u].z, st.u4 = ys[u].w;
                // (a constant false in the instance without the species draw)
                const bool imp = kImpurity && ((impm >> (t0 + u)) & 1u);
                cond = step_post<kDeep>(P, st, imp, u == kStepsPerRound - 1, u == 0);
                if (cond != 0) break;
            }
            if (cond != 0) break;
        }
    }
    __syncwarp();
    return cond;
}

// ---- block mode: the walk beyond kBlockWalk steps (block_pass, cta_pass)
//
// Photons this long are deep in a weakly absorbing slab and still have hundreds
// to millions of steps to go; walked one step at a time they set the end of a
// launch.  A block pass advances one photon by up to kPassSteps = 512 steps from
// one frame O_0 (built from the direction by the branchless orthonormal basis of
// Duff et al. 2017; the lab frame after a bottom reflection).  The pass is cut
// into kPassChunks chunks of 32 lanes x kLaneSteps steps.  Lane l of chunk c draws
// its steps' angles, optical path and absorption words (the same Philox blocks,
// counter = step, as the step-by-step walk) and turns each step's rotation
// R = Rz(phi) Ry(theta) into a unit quaternion; the lane's product, an inclusive
// shuffle scan of Hamilton products across the chunk (rotations compose
// associatively) and the product W_c of the earlier chunks' totals give every
// step's composed rotation P_k = R_1 ... R_k, so step k's direction is
// O_0 P_k e_z.  Vertical positions and path lengths are scan sums the same way,
// and the first top/bottom crossing or absorption ends the pass there, as the
// step-by-step walk would.  The moving frame replaces the z-referenced rotation
// formula: with a uniform azimuth both give the same distribution of walks.
//
// The chunks' totals are combined in chunk order (W_{c+1} = W_c * T_c, sums
// likewise), so a warp that walks the chunks one after the other (block_pass,
// stopping at the first chunk with an event) and a thread block whose warps take
// one chunk each (cta_pass, in the drain kernel) do the same arithmetic: records
// do not depend on which walks a photon.  A photon enters block mode at exactly
// kBlockWalk steps on every path (the dense and sparse rounds stop there).

#ifndef MCW_BLOCK_LANE_STEPS
#define MCW_BLOCK_LANE_STEPS 2
#endif
constexpr int kLaneSteps = MCW_BLOCK_LANE_STEPS;          // steps per lane in a chunk
constexpr int kChunkSteps = 32 * kLaneSteps;              // steps per chunk (one warp)
#ifndef MCW_LONG_WALK
#define MCW_LONG_WALK 8192
#endif
// with MCW_LONG_LANE_STEPS=4, a pass that starts past kLongWalk steps uses chunks of 32
// lanes x 4 steps (1,024 steps per pass): fewer cycles per step for the longest walks,
// decided by the photon's own step count, so records do not depend on where it is
// walked.  Off by default: measured on one GB300, it made the 64-config sweep 3% faster
// (16% from 256 steps on) and the 1e6-photon launch 3% (8%) slower, its registers being
// live in the main loop
constexpr int kLongWalk = MCW_LONG_WALK;
#ifndef MCW_LONG_LANE_STEPS
#define MCW_LONG_LANE_STEPS 2
#endif
constexpr int kLongLaneSteps = MCW_LONG_LANE_STEPS;
constexpr int kPassChunks = 8;                            // chunks per block pass
constexpr int kPassSteps = kPassChunks * kChunkSteps;     // steps per block pass
constexpr int kCtaWalkThreads = 32 * kPassChunks;         // the drain kernel's block: a warp per chunk

// Hamilton product a b of quaternions stored as (.x, .y, .z, .w) = (w, x, y, z),
// every operation rounded as written (a pass must give the same bits in every
// kernel that walks it).
__device__ __forceinline__ float4 qmul(const float4 a, const float4 b) {
    return make_float4(
        fmaf(-a.y, b.y, fmaf(-a.z, b.z, fmaf(-a.w, b.w, __fmul_rn(a.x, b.x)))),   // w
        fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.z, b.w, -__fmul_rn(a.w, b.z)))),     // x
        fmaf(a.x, b.z, fmaf(-a.y, b.w, fmaf(a.z, b.x, __fmul_rn(a.w, b.y)))),     // y
        fmaf(a.x, b.w, fmaf(a.y, b.z, fmaf(-a.z, b.y, __fmul_rn(a.w, b.x)))));    // z
}

__device__ __forceinline__ float4 q_identity() { return make_float4(1.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ float4 shfl_q(const float4 q, int src) {
    return make_float4(__shfl_sync(0xffffffffu, q.x, src), __shfl_sync(0xffffffffu, q.y, src),
                       __shfl_sync(0xffffffffu, q.z, src), __shfl_sync(0xffffffffu, q.w, src));
}

// Inclusive scan of the lanes' quaternions, earlier lanes on the left.
__device__ __forceinline__ float4 warp_scan_q(float4 q, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        float4 l;
        l.x = __shfl_up_sync(0xffffffffu, q.x, off);
        l.y = __shfl_up_sync(0xffffffffu, q.y, off);
        l.z = __shfl_up_sync(0xffffffffu, q.z, off);
        l.w = __shfl_up_sync(0xffffffffu, q.w, off);
        if (lane >= off) q = qmul(l, q);
    }
    return q;
}

// Inclusive scan of two sums across the lanes.
__device__ __forceinline__ void warp_scan_2(float &x, float &y, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float xu = __shfl_up_sync(0xffffffffu, x, off);
        const float yu = __shfl_up_sync(0xffffffffu, y, off);
        if (lane >= off) { x = __fadd_rn(x, xu); y = __fadd_rn(y, yu); }
    }
}

// The frame O_0 = (e1, e2, d0) of a pass.
struct PassFrame {
    float e1x, e1y, e1z, e2x, e2y, e2z, d0x, d0y, d0z;
};

__device__ __forceinline__ PassFrame pass_frame(const Photon &Q, bool reflected) {
    PassFrame F{1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    if (!reflected) {
        const float inv = rsqrtf(fmaf(Q.mux, Q.mux, fmaf(Q.muy, Q.muy, __fmul_rn(Q.muz, Q.muz))));
        F.d0x = __fmul_rn(Q.mux, inv); F.d0y = __fmul_rn(Q.muy, inv); F.d0z = __fmul_rn(Q.muz, inv);
        const float sg = copysignf(1.f, F.d0z);
        const float aa = -1.f / __fadd_rn(sg, F.d0z);
        const float bb = __fmul_rn(__fmul_rn(F.d0x, F.d0y), aa);
        F.e1x = fmaf(__fmul_rn(sg, F.d0x), __fmul_rn(F.d0x, aa), 1.f);
        F.e1y = __fmul_rn(sg, bb);
        F.e1z = -__fmul_rn(sg, F.d0x);
        F.e2x = bb;
        F.e2y = fmaf(F.d0y, __fmul_rn(F.d0y, aa), sg);
        F.e2z = -F.d0y;
    }
    return F;
}

// One lane's steps of a chunk: their rotations (then their composed rotations),
// optical paths, and per step the absorption, reflectance and species bits.
template <int LS>
struct LaneSteps {
    float4 qs[LS];
    float dtau[LS];
    unsigned absm, reflm, impm;
};

// Draw steps s0 .. s0 + LS - 1 of photon Q; lamb: the first of them takes
// the Lambertian direction about the vertical (the first step after a bottom
// reflection, :1238-1250).
// kImp: the launch has impurity configs; kDeep: the deep-slab instance (no isotropic photon).
template <int LS, bool kImp, bool kDeep>
__device__ __forceinline__ void lane_draw(LaneSteps<LS> &L, const Photon &Q, uint32_t s0, bool lamb, const WalkArgs &a) {
    L.absm = L.reflm = L.impm = 0;
#pragma unroll
    for (int t = 0; t < LS; ++t) {
        const uint32_t n = s0 + (uint32_t)t;
        const uint4 r = philox10(make_uint4(n, kTagStep, (uint32_t)Q.rid, (uint32_t)(Q.rid >> 32)), a.keys);
        const float4 uu = step_uniforms(r);
        L.dtau[t] = -__logf(uu.z);                                      // :1014
        const bool imp = kImp && (Q.flags & kFlagImpurity) && impurity_draw(Q.rid, n, Q.p_imp, a);
        // absorption as 1 - u < 1 - ssa (:1461-1466); on a bottom crossing the same
        // word is the reflectance draw
        L.absm |= (uu.w < (imp ? Q.coalb_imp : Q.coalb_ice) ? 1u : 0u) << t;
        L.reflm |= (uu.w < Q.R ? 1u : 0u) << t;
        if (kImp) L.impm |= (imp ? 1u : 0u) << t;
        const float ct = (lamb && t == 0) ? sqrtf(uu.x) : hg_cos<kDeep>(uu.x, Q.hg_a, Q.hg_b, Q.hg_c, Q.hg_d, Q.hg_e);
        const float ch = sqrtf(fmaxf(0.f, __fmul_rn(0.5f, __fadd_rn(1.f, ct))));  // cos(theta / 2)
        const float sh = sqrtf(fmaxf(0.f, __fmul_rn(0.5f, __fsub_rn(1.f, ct))));  // sin(theta / 2)
        float sph, cph;                                                 // half the azimuth, uniform
        __sincosf(__fmul_rn(3.14159265358979324f, __fsub_rn(uu.y, 0.5f)), &sph, &cph);
        L.qs[t] = make_float4(__fmul_rn(cph, ch), -__fmul_rn(sph, sh), __fmul_rn(cph, sh), __fmul_rn(sph, ch));
    }
}

template <int LS>
__device__ __forceinline__ float4 lane_product(const LaneSteps<LS> &L) {
    float4 q = L.qs[0];
#pragma unroll
    for (int t = 1; t < LS; ++t) q = qmul(q, L.qs[t]);
    return q;
}

// x: the rotation up to the lane's first step; the lane's rotations become the
// composed rotations of its steps.
template <int LS>
__device__ __forceinline__ void lane_prefixes(LaneSteps<LS> &L, float4 x) {
#pragma unroll
    for (int t = 0; t < LS; ++t) {
        x = qmul(x, L.qs[t]);
        L.qs[t] = x;
    }
}

// The direction after a step of composed rotation p (O_0 p e_z).
__device__ __forceinline__ float3 pass_dir(const PassFrame &F, const float4 p) {
    const float c0 = __fmul_rn(2.f, fmaf(p.y, p.w, __fmul_rn(p.x, p.z)));
    const float c1 = __fmul_rn(2.f, fmaf(p.z, p.w, -__fmul_rn(p.x, p.y)));
    const float c2 = fmaf(-2.f, fmaf(p.y, p.y, __fmul_rn(p.z, p.z)), 1.f);
    return make_float3(fmaf(F.e1x, c0, fmaf(F.e2x, c1, __fmul_rn(F.d0x, c2))),
                       fmaf(F.e1y, c0, fmaf(F.e2y, c1, __fmul_rn(F.d0y, c2))),
                       fmaf(F.e1z, c0, fmaf(F.e2z, c1, __fmul_rn(F.d0z, c2))));
}

// Each step's vertical move, and the lane's sums of the moves and path increments.
template <int LS>
__device__ __forceinline__ void lane_moves(const LaneSteps<LS> &L, const PassFrame &F, float inv_ext,
                                           float (&dz)[LS], float &zs, float &ps) {
#pragma unroll
    for (int t = 0; t < LS; ++t) {
        const float4 p = L.qs[t];
        const float c0 = __fmul_rn(2.f, fmaf(p.y, p.w, __fmul_rn(p.x, p.z)));
        const float c1 = __fmul_rn(2.f, fmaf(p.z, p.w, -__fmul_rn(p.x, p.y)));
        const float c2 = fmaf(-2.f, fmaf(p.y, p.y, __fmul_rn(p.z, p.z)), 1.f);
        dz[t] = __fmul_rn(L.dtau[t], fmaf(F.e1z, c0, fmaf(F.e2z, c1, __fmul_rn(F.d0z, c2))));
        const float inc = __fmul_rn(L.dtau[t], inv_ext);
        zs = t == 0 ? dz[t] : __fadd_rn(zs, dz[t]);
        ps = t == 0 ? inc : __fadd_rn(ps, inc);
    }
}

// The lane's first event (a crossing, else absorption) or, without one, its last
// step: the step (ts), the event bits, z after and before the step, the path up to
// it.  zx, px: the moves and path before the lane's first step of the pass.
struct LaneEvent {
    int first, ts;        // first: the event step, LS if none
    unsigned what;        // 1 top, 2 bottom, 4 species impurity, 8 reflectance draw passed
    float zk, zp, pk;
};

template <int LS>
__device__ __forceinline__ LaneEvent lane_event(const LaneSteps<LS> &L, const float (&dz)[LS], const Photon &Q,
                                                float zx, float px) {
    LaneEvent E{LS, LS - 1, 0u, 0.f, 0.f, 0.f};
    float zl = 0.f, pl = 0.f;
#pragma unroll
    for (int t = 0; t < LS; ++t) {
        const float zp = t == 0 ? __fadd_rn(Q.z, zx) : __fadd_rn(Q.z, __fadd_rn(zx, zl));
        const float inc = __fmul_rn(L.dtau[t], Q.inv_ext);
        zl = t == 0 ? dz[t] : __fadd_rn(zl, dz[t]);
        pl = t == 0 ? inc : __fadd_rn(pl, inc);
        const float zk = __fadd_rn(Q.z, __fadd_rn(zx, zl));
        const bool top = zk > 0.f;
        const bool bot = zk < -Q.tau;
        const bool absb = !top && !bot && ((L.absm >> t) & 1u);
        const bool event = top || bot || absb;
        if (E.first == LS && (event || t == LS - 1)) {
            if (event) E.first = t;
            E.ts = t;
            E.what = (top ? 1u : 0u) | (bot ? 2u : 0u) | (((L.impm >> t) & 1u) << 2) | (((L.reflm >> t) & 1u) << 3);
            E.zk = zk;
            E.zp = zp;
            E.pk = __fadd_rn(px, pl);
        }
    }
    return E;
}

// The direction (x, y, z) and path increment (w) of the lane's step ts.
template <int LS>
__device__ __forceinline__ float4 lane_step_dir(const LaneSteps<LS> &L, const PassFrame &F, int ts, float inv_ext) {
    float4 p = L.qs[0];
    float dt = L.dtau[0];
#pragma unroll
    for (int t = 1; t < LS; ++t)
        if (t == ts) { p = L.qs[t]; dt = L.dtau[t]; }
    const float3 d = pass_dir(F, p);
    return make_float4(d.x, d.y, d.z, __fmul_rn(dt, inv_ext));
}

// The end of a pass: the photon advanced `adv` steps; dir: the direction and path
// increment of the last step, ze / zp: z after / before it, pe: the pass's path
// length, what: its event bits (ev: an event ended the pass).  Returns the end
// condition (0: still walking, or reflected at the bottom).
__device__ __forceinline__ int pass_end(Photon &Q, int adv, bool ev, const float4 dir, float ze, float zp, float pe,
                                        unsigned what) {
    Q.i += adv;
    {   // compensated path sum
        const float y = __fsub_rn(pe, Q.pathc);
        const float tt = __fadd_rn(Q.path, y);
        Q.pathc = __fsub_rn(__fsub_rn(tt, Q.path), y);
        Q.path = tt;
    }
    const float inv = rsqrtf(fmaf(dir.x, dir.x, fmaf(dir.y, dir.y, __fmul_rn(dir.z, dir.z))));
    Q.mux = __fmul_rn(dir.x, inv); Q.muy = __fmul_rn(dir.y, inv); Q.muz = __fmul_rn(dir.z, inv);
    Q.flags &= ~kFlagReflect;
    Q.z = ze;
    if (!ev) return 0;
    if (what & 1u) {                                                    // :1390-1397
        Q.path = fmaf(-__fdividef(ze, __fsub_rn(ze, zp)), dir.w, Q.path);
        return 1;
    }
    if (what & 2u) {                                                    // :1399-1459
        Q.path = fmaf(-__fdividef(__fadd_rn(ze, Q.tau), __fsub_rn(ze, zp)), dir.w, Q.path);
        Q.z = -Q.tau;
        if ((Q.flags & kFlagLamBottom) && (what & 8u)) {
            Q.flags |= kFlagReflect;
            return 0;
        }
        return 2;
    }
    return (what & 4u) ? 5 : 4;
}

// One block pass over photon Q, held alike by every lane of the warp, the chunks
// walked one after the other until the first with an event.  Q is updated alike
// on every lane; returns the end condition.  Warp-collective.
template <int LS, bool kImp, bool kDeep>
__device__ __forceinline__ int block_pass(Photon &Q, const WalkArgs &a, int lane) {
    const bool reflected = (Q.flags & kFlagReflect) != 0;
    const PassFrame F = pass_frame(Q, reflected);
    float4 W = q_identity();               // rotation of the earlier chunks
    float Wz = 0.f, Wp = 0.f;              // their vertical moves and path increments
    for (int c = 0;; ++c) {
        LaneSteps<LS> L;
        lane_draw<LS, kImp, kDeep>(L, Q, (uint32_t)Q.i + 1u + (uint32_t)((32 * LS) * c + LS * lane),
                  reflected && c == 0 && lane == 0, a);
        const float4 qi = warp_scan_q(lane_product<LS>(L), lane);
        float4 xl = shfl_q(qi, (lane + 31) & 31);
        if (lane == 0) xl = q_identity();
        lane_prefixes<LS>(L, qmul(W, xl));
        float dz[LS], zs, ps;
        lane_moves<LS>(L, F, Q.inv_ext, dz, zs, ps);
        warp_scan_2(zs, ps, lane);
        float zx = __shfl_up_sync(0xffffffffu, zs, 1), px = __shfl_up_sync(0xffffffffu, ps, 1);
        if (lane == 0) { zx = 0.f; px = 0.f; }
        const LaneEvent E = lane_event<LS>(L, dz, Q, __fadd_rn(Wz, zx), __fadd_rn(Wp, px));
        const unsigned ev = __ballot_sync(0xffffffffu, E.first < LS);
        if (ev || c == kPassChunks - 1) {
            const int e = ev ? __ffs(ev) - 1 : 31;
            const float4 d = lane_step_dir<LS>(L, F, E.ts, Q.inv_ext);
            const float4 dir = make_float4(__shfl_sync(0xffffffffu, d.x, e), __shfl_sync(0xffffffffu, d.y, e),
                                           __shfl_sync(0xffffffffu, d.z, e), __shfl_sync(0xffffffffu, d.w, e));
            const int ts = __shfl_sync(0xffffffffu, E.ts, e);
            const float ze = __shfl_sync(0xffffffffu, E.zk, e), zp = __shfl_sync(0xffffffffu, E.zp, e);
            const float pe = __shfl_sync(0xffffffffu, E.pk, e);
            const unsigned what = __shfl_sync(0xffffffffu, E.what, e);
            return pass_end(Q, (32 * LS) * c + LS * e + ts + 1, ev != 0, dir, ze, zp, pe, what);
        }
        W = qmul(W, shfl_q(qi, 31));
        Wz = __fadd_rn(Wz, __shfl_sync(0xffffffffu, zs, 31));
        Wp = __fadd_rn(Wp, __shfl_sync(0xffffffffu, ps, 31));
    }
}

// Shared memory of a block walking one photon in block passes (cta_pass).
struct CtaPassShared {
    float4 wq[kPassChunks];     // each chunk's rotation
    float2 wzp[kPassChunks];    // each chunk's vertical move and path length
    int wev[kPassChunks];       // each chunk's first lane with an event (32: none)
    float4 dir;                 // the last step's direction and path increment
    float4 zzp;                 // z after and before it, the pass's path length, event bits
    int adv, ev;
};

// One block pass over photon Q, held alike by every thread of a block of
// kCtaWalkThreads, warp w taking chunk w: the same arithmetic as block_pass.  Q is
// updated alike on every thread; returns the end condition.  Block-collective.
template <int LS, bool kImp, bool kDeep>
__device__ __forceinline__ int cta_pass(Photon &Q, const WalkArgs &a, CtaPassShared &S, int warp, int lane) {
    const bool reflected = (Q.flags & kFlagReflect) != 0;
    const PassFrame F = pass_frame(Q, reflected);
    LaneSteps<LS> L;
    lane_draw<LS, kImp, kDeep>(L, Q, (uint32_t)Q.i + 1u + (uint32_t)((32 * LS) * warp + LS * lane),
              reflected && warp == 0 && lane == 0, a);
    const float4 qi = warp_scan_q(lane_product<LS>(L), lane);
    if (lane == 31) S.wq[warp] = qi;
    __syncthreads();
    float4 W = q_identity();
    for (int c = 0; c < warp; ++c) W = qmul(W, S.wq[c]);
    float4 xl = shfl_q(qi, (lane + 31) & 31);
    if (lane == 0) xl = q_identity();
    lane_prefixes<LS>(L, qmul(W, xl));
    float dz[LS], zs, ps;
    lane_moves<LS>(L, F, Q.inv_ext, dz, zs, ps);
    warp_scan_2(zs, ps, lane);
    if (lane == 31) S.wzp[warp] = make_float2(zs, ps);
    __syncthreads();
    float Wz = 0.f, Wp = 0.f;
    for (int c = 0; c < warp; ++c) {
        const float2 t = S.wzp[c];
        Wz = __fadd_rn(Wz, t.x);
        Wp = __fadd_rn(Wp, t.y);
    }
    float zx = __shfl_up_sync(0xffffffffu, zs, 1), px = __shfl_up_sync(0xffffffffu, ps, 1);
    if (lane == 0) { zx = 0.f; px = 0.f; }
    const LaneEvent E = lane_event<LS>(L, dz, Q, __fadd_rn(Wz, zx), __fadd_rn(Wp, px));
    const unsigned ev = __ballot_sync(0xffffffffu, E.first < LS);
    if (lane == 0) S.wev[warp] = ev ? __ffs(ev) - 1 : 32;
    __syncthreads();
    int ec = kPassChunks - 1, el = 31;
    bool any = false;
    for (int c = kPassChunks - 1; c >= 0; --c) {
        const int l = S.wev[c];
        if (l < 32) { ec = c; el = l; any = true; }
    }
    if (warp == ec && lane == el) {
        S.dir = lane_step_dir<LS>(L, F, E.ts, Q.inv_ext);
        S.zzp = make_float4(E.zk, E.zp, E.pk, __uint_as_float(E.what));
        S.adv = (32 * LS) * ec + LS * el + E.ts + 1;
    }
    __syncthreads();
    const float4 zzp = S.zzp;
    return pass_end(Q, S.adv, any, S.dir, zzp.x, zzp.y, zzp.z, __float_as_uint(zzp.w));
}

__device__ __forceinline__ Photon shfl_photon(const Photon &P, int src) {
    Photon Q;
    Q.rid = __shfl_sync(0xffffffffu, P.rid, src);
    Q.cfg = __shfl_sync(0xffffffffu, P.cfg, src);
    Q.lut = __shfl_sync(0xffffffffu, P.lut, src);
    Q.i = __shfl_sync(0xffffffffu, P.i, src);
    Q.flags = __shfl_sync(0xffffffffu, P.flags, src);
    Q.mux = __shfl_sync(0xffffffffu, P.mux, src);
    Q.muy = __shfl_sync(0xffffffffu, P.muy, src);
    Q.muz = __shfl_sync(0xffffffffu, P.muz, src);
    Q.z = __shfl_sync(0xffffffffu, P.z, src);
    Q.path = __shfl_sync(0xffffffffu, P.path, src);
    Q.pathc = __shfl_sync(0xffffffffu, P.pathc, src);
    Q.tau = __shfl_sync(0xffffffffu, P.tau, src);
    Q.R = __shfl_sync(0xffffffffu, P.R, src);
    Q.inv_ext = __shfl_sync(0xffffffffu, P.inv_ext, src);
    Q.coalb_ice = __shfl_sync(0xffffffffu, P.coalb_ice, src);
    Q.coalb_imp = __shfl_sync(0xffffffffu, P.coalb_imp, src);
    Q.p_imp = __shfl_sync(0xffffffffu, P.p_imp, src);
    Q.hg_a = __shfl_sync(0xffffffffu, P.hg_a, src);
    Q.hg_b = __shfl_sync(0xffffffffu, P.hg_b, src);
    Q.hg_c = __shfl_sync(0xffffffffu, P.hg_c, src);
    Q.hg_d = __shfl_sync(0xffffffffu, P.hg_d, src);
    Q.hg_e = __shfl_sync(0xffffffffu, P.hg_e, src);
    return Q;
}


// Exact warp sum of 64-bit values below 2^47.
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    const unsigned lo = __reduce_add_sync(0xffffffffu, (unsigned)(v & 0xffffu));
    const unsigned mid = __reduce_add_sync(0xffffffffu, (unsigned)((v >> 16) & 0xffffffu));
    const unsigned hi = __reduce_add_sync(0xffffffffu, (unsigned)(v >> 40));
    return (unsigned long long)lo + ((unsigned long long)mid << 16) + ((unsigned long long)hi << 40);
}

// Epilogue of up to 32 finished photons (entries [base, base + n) of the
// finish queue): records, histogram bins and the warp's running totals.
// Warp-collective.
__device__ __noinline__ void finish_batch(const FinishSlot *fin, WarpTally &tally, int base, int n,
                                          const WalkArgs &a, const CfgF32 *scfg, const int64_t *prefix,
                                          bool staged, int lane) {
    const bool have = lane < n;
    int cfg = -1, cond = 0, nscat = 0;
    unsigned long long wfx = 0;
    if (have) {
        FinishSlot f;
        copy_f4<3>(&f, &fin[base + lane]);
        cfg = (int)f.cfg;
        cond = f.cond;
        nscat = f.n_step - 1;
        const LutEntry *e = a.lut + f.lut;
        const float wvn = __ldg(&e->wvn);
        const float depth = __ldg(&e->snow_depth);
        wfx = __ldg(&e->wvn_fx);
        const float theta = acosf(fminf(fmaxf(f.muz, -1.f), 1.f));
        float phi = 0.f;
        if (f.n_step > 1) {
            phi = atan2f(f.muy, f.mux);
            if (phi < 0.f) phi += kTwoPiF;
            if (phi >= kTwoPiF) phi = 0.f;
        }
        if (a.records) {
            const uint64_t rid = ((uint64_t)f.rid_hi << 32) | f.rid_lo;
            const uint64_t rbase = staged ? scfg[cfg].rng_base : a.cfgs[cfg].rng_base;
            const int64_t gid = prefix[cfg] + (int64_t)(rid - rbase);
            float4 *dst = reinterpret_cast<float4 *>(a.records + gid);
            dst[0] = make_float4(__int_as_float(cond), __int_as_float(nscat), wvn, theta);
            dst[1] = make_float4(phi, f.path, depth, __uint_as_float((uint32_t)cfg));
        }
        if (cond == 1) tally_bin(a.tallies + cfg, wfx, theta, phi);
    }
    // running totals per config (normally one config per batch)
    unsigned pending = __ballot_sync(0xffffffffu, have);
    while (pending) {
        const int c = __shfl_sync(0xffffffffu, cfg, __ffs(pending) - 1);
        const bool mine = have && cfg == c;
        pending &= ~__ballot_sync(0xffffffffu, mine);
        if (tally.cfg != c) {
            warp_tally_flush(tally, a.tallies, lane);
            if (lane == 0) tally.cfg = c;
            __syncwarp();
        }
        const unsigned ev = __reduce_add_sync(0xffffffffu, mine ? (unsigned)nscat : 0u);
        const unsigned mx = __reduce_max_sync(0xffffffffu, mine ? (unsigned)nscat : 0u);
        unsigned cnt[6];
        unsigned long long qs[6];
#pragma unroll
        for (int k = 1; k < 6; ++k) {
            const bool hit = mine && cond == k;
            cnt[k] = __popc(__ballot_sync(0xffffffffu, hit));
            qs[k] = cnt[k] ? warp_sum_u64(hit ? wfx : 0ull) : 0ull;
        }
        if (lane == 0) {
            tally.n_events += ev;
            tally.max_n_scat = max(tally.max_n_scat, mx);
#pragma unroll
            for (int k = 1; k < 6; ++k) {
                tally.n_cond[k] += cnt[k];
                tally.q_cond_fx[k] += qs[k];
            }
        }
        __syncwarp();
    }
}

// kDeep: the slabs of the launch are optically deep, none is a Lambertian surface and no
// photon scatters isotropically (WalkArgs::deep; see boundary()).
template <bool kImpurity, bool kDeep>
__global__ void __launch_bounds__(256, 2) walk_f32_kernel(const WalkArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    WarpQueues *queues = reinterpret_cast<WarpQueues *>(smem);
    const bool staged = a.n_cfg <= kSmemCfgMax;
    CfgF32 *scfg = reinterpret_cast<CfgF32 *>(smem + sizeof(WarpQueues) * nwarps);
    int64_t *sprefix = reinterpret_cast<int64_t *>(scfg + (staged ? a.n_cfg : 0));
    int64_t *sclaim = sprefix + (staged ? a.n_cfg : 0);
    int32_t *sclaim_cfg = reinterpret_cast<int32_t *>(sclaim + (staged ? a.n_cfg : 0));
    const bool ordered = a.claim_prefix != nullptr;
    if (staged) {
        for (int c = threadIdx.x; c < a.n_cfg; c += blockDim.x) {
            scfg[c] = make_cfg(a.cfgs[c]);
            sprefix[c] = a.prefix[c];
            sclaim[c] = ordered ? a.claim_prefix[c] : a.prefix[c];
            sclaim_cfg[c] = ordered ? a.claim_cfg[c] : c;
        }
    }
    const int64_t *prefix = staged ? sprefix : a.prefix;
    // photons are handed out in claim order (longest expected walks first)
    const int64_t *claim = staged ? sclaim : (ordered ? a.claim_prefix : a.prefix);
    const int32_t *claim_cfg = staged ? sclaim_cfg : a.claim_cfg;
    WarpQueues &q = queues[warp];
    warp_tally_reset(q.tally, lane);
    __syncthreads();

    Photon P;
    P.rid = 0;
    P.cfg = -1;
    P.lut = 0;
    P.i = 0;
    bool exhausted = false;
    int n_birth = 0, n_fin = 0;        // queue fill, warp-uniform (kept in registers)
    const unsigned long long t0 = global_ns();
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned idle = 0xffffffffu;       // lanes without a photon, warp-uniform

    for (uint32_t iter = 0;; ++iter) {
        // ---- regeneration: idle lanes pop ready photons; refill the queue in batches
        const int nidle = __popc(idle);
        if (nidle > 0 && (nidle >= a.regen_chunk || nidle == 32) && !(exhausted && n_birth == 0)) {
            int cnt = n_birth;
            if (cnt < nidle && !exhausted) {
                const int want = 32 - cnt;
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(a.work, (unsigned long long)want);
                base = __shfl_sync(0xffffffffu, base, 0);
                const int64_t left = a.total - (int64_t)base;
                const int valid = (int)max((int64_t)0, min((int64_t)want, left));
                if (left <= want) exhausted = true;
                if (lane < valid) {
                    const int64_t g = (int64_t)base + lane;
                    const int k = find_config(claim, a.n_cfg, g);
                    const int ci = claim_cfg ? claim_cfg[k] : k;
                    const CfgF32 c = staged ? scfg[ci] : make_cfg(a.cfgs[ci]);
                    birth(q.birth[cnt + lane], g - claim[k], ci, c, a);
                }
                cnt += valid;
                __syncwarp();
            }
            const int take = min(nidle, cnt);
            bool popped = false;
            if (idle & (1u << lane)) {
                const int r = __popc(idle & lt_mask);
                if (r < take) {
                    pop(P, q.birth[cnt - 1 - r]);
                    popped = true;
                }
            }
            idle &= ~__ballot_sync(0xffffffffu, popped);
            n_birth = cnt - take;
            __syncwarp();
        }
        if (idle == 0xffffffffu && exhausted && n_birth == 0) break;

        // ---- drain handover, once the supply is exhausted: photons past drain_from
        // steps go to the queue, walked after this kernel with a thread block each
        // (a lane hands over at most one photon: it takes none afterwards)
        if (a.drain_from > 0 && exhausted && n_birth == 0) {
            const bool leave = in_block_mode<kDeep>(P) && P.i >= a.drain_from;
            const unsigned lm = __ballot_sync(0xffffffffu, leave);
            if (lm) {
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(a.drain_count, (unsigned)__popc(lm));
                base = __shfl_sync(0xffffffffu, base, 0);
                const unsigned slot_i = base + __popc(lm & lt_mask);
                if (leave && slot_i < a.drain_cap) {
                    float4 *slot = a.drain + (size_t)slot_i * kDrainSlot;
                    float4 v[kDrainSlot];
                    pack_photon(v, P);
#pragma unroll
                    for (int k = 0; k < kDrainSlot; ++k) __stcg(&slot[k], v[k]);
                    P.cfg = -1;
                }
                idle |= __ballot_sync(0xffffffffu, leave && slot_i < a.drain_cap);
            }
            if (idle == 0xffffffffu) break;
        }

        // ---- kStepsPerRound scatter events per active lane of a well-filled warp;
        // their Philox blocks are independent of the walk, so they are computed
        // together first.  A sparse warp runs sparse_round instead.
        const unsigned bmask = __ballot_sync(0xffffffffu, in_block_mode<kDeep>(P));
        const unsigned act = ~idle & ~bmask;
        const bool me_active = (act >> lane) & 1u;
        const int n_act = __popc(act);
        int cond = 0;
        if (n_act <= kSparseWarp) {
            if (n_act > 0) cond = sparse_round<kImpurity, kDeep>(P, q, act, n_act, lane, lt_mask, a);
        } else if (me_active) {
            // the deep instance: the direction-independent part of the round's steps
            // first, then their chains (step_post, the same values as step(): the HG
            // cosine, azimuth and optical path of step k + 1 do not wait for the chain of
            // step k behind its rare branches); otherwise the Philox blocks first, then step()
            const uint32_t glo = (uint32_t)P.rid, ghi = (uint32_t)(P.rid >> 32);
            StepPreDense pre[kDeep ? kStepsPerRound : 1];
            bool impk[kDeep ? kStepsPerRound : 1];
            uint4 rb[kDeep ? 1 : kStepsPerRound];
#pragma unroll
            for (int k = 0; k < kStepsPerRound; ++k) {
                const uint32_t n = (uint32_t)P.i + 1u + k;
                if constexpr (kDeep) {
                    pre[k] = step_pre_dense<kDeep>(philox10(make_uint4(n, kTagStep, glo, ghi), a.keys), P);
                    impk[k] = kImpurity && (P.flags & kFlagImpurity) && impurity_draw(P.rid, n, P.p_imp, a);
                } else {
                    rb[k] = philox10(make_uint4(n, kTagStep, glo, ghi), a.keys);
                }
            }
#pragma unroll
            for (int k = 0; k < kStepsPerRound; ++k) {
                // a lane whose photon ended earlier in the round keeps its final state
                const bool alive = cond == 0;
                Photon Q = P;
                int c;
                if constexpr (kDeep)
                    c = step_post<kDeep>(Q, pre[k], impk[k], k == kStepsPerRound - 1, k == 0);
                else
                    c = step<kImpurity, kDeep>(Q, a, rb[k], k == kStepsPerRound - 1, k == 0);
                // a finished photon's record uses i, the direction and the path only;
                // its z, flags and path compensation are never read again
                P.i = alive ? Q.i : P.i;
                P.mux = alive ? Q.mux : P.mux;
                P.muy = alive ? Q.muy : P.muy;
                P.muz = alive ? Q.muz : P.muz;
                P.path = alive ? Q.path : P.path;
                P.flags = Q.flags;
                P.z = Q.z;
                P.pathc = Q.pathc;
                cond = alive ? c : cond;
            }
        }

        // ---- photons past kBlockWalk steps: one block pass (up to kPassSteps steps)
        // each, walked by the whole warp
        for (unsigned pend = bmask; pend; pend &= pend - 1) {
            const int src = __ffs(pend) - 1;
            Photon Q = shfl_photon(P, src);
            int c;
            if constexpr (kLongLaneSteps != kLaneSteps)
                c = Q.i >= kLongWalk ? block_pass<kLongLaneSteps, kImpurity, kDeep>(Q, a, lane)
                                     : block_pass<kLaneSteps, kImpurity, kDeep>(Q, a, lane);
            else
                c = block_pass<kLaneSteps, kImpurity, kDeep>(Q, a, lane);
            if (lane == src) {
                P.i = Q.i;
                P.flags = Q.flags;
                P.mux = Q.mux; P.muy = Q.muy; P.muz = Q.muz;
                P.z = Q.z;
                P.path = Q.path;
                P.pathc = Q.pathc;
                cond = c;
            }
        }

        // ---- finished photons go to the finish queue
        const unsigned fin_mask = __ballot_sync(0xffffffffu, cond != 0);
        if (fin_mask) {
            if (cond != 0) {
                FinishSlot f;
                f.rid_lo = (uint32_t)P.rid;
                f.rid_hi = (uint32_t)(P.rid >> 32);
                f.cfg = (uint32_t)P.cfg;
                f.lut = (uint32_t)P.lut;
                f.n_step = P.i;
                f.cond = cond;
                f.mux = P.mux;
                f.muy = P.muy;
                f.muz = P.muz;
                f.path = P.path;
                f.pad0 = f.pad1 = 0.f;
                copy_f4<3>(&q.fin[n_fin + __popc(fin_mask & lt_mask)], &f);
                P.cfg = -1;
            }
            idle |= fin_mask;
            __syncwarp();
            n_fin += __popc(fin_mask);
            if (n_fin >= 32) {
                finish_batch(q.fin, q.tally, n_fin - 32, 32, a, scfg, prefix, staged, lane);
                n_fin -= 32;
            }
        }

        // ---- time budget (watchdog; never a truncation in normal runs)
        if ((iter & 63u) == 63u) {
            int stop = 0;
            if (lane == 0) {
                const unsigned long long now = global_ns();
                if (now - t0 > a.budget_ns) {
                    atomicOr(a.status, kStatusBudget);
                    stop = 1;
                } else if (*(volatile unsigned int *)a.status & kStatusBudget) {
                    stop = 1;
                }
            }
            if (__shfl_sync(0xffffffffu, stop, 0)) break;
        }
    }
    __syncwarp();
    if (n_fin > 0) finish_batch(q.fin, q.tally, 0, n_fin, a, scfg, prefix, staged, lane);
    warp_tally_flush(q.tally, a.tallies, lane);
}

// Shared memory of a drain-kernel block.
struct DrainBlock {
    CtaPassShared pass;
    FinishSlot fin[32];
    WarpTally tally;
    unsigned job;
    int stop;
};

// After the walk: every photon handed over to the drain queue is walked to its end
// by a whole block (cta_pass), one photon after another; finished photons go
// through warp 0's finish queue.  The queue is complete when this kernel starts.
template <bool kImp, bool kDeep>
__global__ void __launch_bounds__(kCtaWalkThreads) drain_kernel(const WalkArgs a) {
    __shared__ DrainBlock S;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned cnt = min(*(volatile unsigned int *)a.drain_count, a.drain_cap);
    if (blockIdx.x >= cnt) return;          // blocks past the queue length would find no photon
    if (warp == 0) warp_tally_reset(S.tally, lane);
    const unsigned long long t0 = global_ns();
    int n_fin = 0;
    for (;;) {
        if (threadIdx.x == 0) S.job = atomicAdd(a.drain_next, 1u);
        __syncthreads();
        const unsigned j = S.job;
        if (j >= cnt) break;
        float4 v[kDrainSlot];
#pragma unroll
        for (int k = 0; k < kDrainSlot; ++k) v[k] = __ldcg(&a.drain[(size_t)j * kDrainSlot + k]);
        Photon P;
        unpack_photon(P, v);
        int cond = 0;
        bool over = false;
        for (uint32_t pass = 1; cond == 0; ++pass) {
            if constexpr (kLongLaneSteps != kLaneSteps)
                cond = P.i >= kLongWalk ? cta_pass<kLongLaneSteps, kImp, kDeep>(P, a, S.pass, warp, lane)
                                        : cta_pass<kLaneSteps, kImp, kDeep>(P, a, S.pass, warp, lane);
            else
                cond = cta_pass<kLaneSteps, kImp, kDeep>(P, a, S.pass, warp, lane);
            if ((pass & 63u) == 0u) {
                // time budget (watchdog; never a truncation in normal runs)
                if (threadIdx.x == 0)
                    S.stop = (global_ns() - t0 > a.budget_ns) || (*(volatile unsigned int *)a.status & kStatusBudget);
                __syncthreads();
                over = S.stop != 0;
                __syncthreads();
                if (over) break;
            }
        }
        if (over) {
            if (threadIdx.x == 0) atomicOr(a.status, kStatusBudget);
            break;
        }
        if (warp == 0) {
            if (lane == 0) {
                FinishSlot f;
                f.rid_lo = (uint32_t)P.rid;
                f.rid_hi = (uint32_t)(P.rid >> 32);
                f.cfg = (uint32_t)P.cfg;
                f.lut = (uint32_t)P.lut;
                f.n_step = P.i;
                f.cond = cond;
                f.mux = P.mux;
                f.muy = P.muy;
                f.muz = P.muz;
                f.path = P.path;
                f.pad0 = f.pad1 = 0.f;
                copy_f4<3>(&S.fin[n_fin], &f);
            }
            __syncwarp();
            if (++n_fin >= 32) {
                finish_batch(S.fin, S.tally, n_fin - 32, 32, a, nullptr, a.prefix, false, lane);
                n_fin -= 32;
            }
        }
    }
    if (warp == 0) {
        __syncwarp();
        if (n_fin > 0) finish_batch(S.fin, S.tally, 0, n_fin, a, nullptr, a.prefix, false, lane);
        warp_tally_flush(S.tally, a.tallies, lane);
    }
}

size_t smem_bytes(int block, int n_cfg) {
    const size_t cfg =
        n_cfg <= kSmemCfgMax ? (size_t)n_cfg * (sizeof(CfgF32) + 2 * sizeof(int64_t) + sizeof(int32_t)) : 0;
    return sizeof(WarpQueues) * (size_t)(block / 32) + cfg;
}

// The walk kernels may use up to 200 KB of dynamic shared memory; set once per device.
cudaError_t allow_smem() {
    static std::mutex m;
    static std::set<int> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(m);
    if (done.count(dev)) return cudaSuccess;
    for (const void *fn : {reinterpret_cast<const void *>(walk_f32_kernel<false, false>),
                           reinterpret_cast<const void *>(walk_f32_kernel<true, false>),
                           reinterpret_cast<const void *>(walk_f32_kernel<false, true>),
                           reinterpret_cast<const void *>(walk_f32_kernel<true, true>)}) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
    }
    done.insert(dev);
    return e;
}

}  // namespace

size_t walk_f32_smem_bytes(int block, int n_cfg) { return smem_bytes(block, n_cfg); }

// Resident blocks per SM of the walk kernel; the occupancy query is made once per
// device, block size, shared-memory size and kernel instance.
int walk_f32_max_blocks_per_sm(int block, int n_cfg, bool impurity) {
    if (allow_smem() != cudaSuccess) return 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    const size_t smem = smem_bytes(block, n_cfg);
    static std::mutex m;
    static std::map<std::tuple<int, int, size_t, bool>, int> cache;
    const auto key = std::make_tuple(dev, block, smem, impurity);
    {
        std::lock_guard<std::mutex> g(m);
        const auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    int n = 0;
    // the deep-slab instances have the same register count (checked with -Xptxas -v)
    const cudaError_t e = impurity
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_f32_kernel<true, false>, block, smem)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_f32_kernel<false, false>, block, smem);
    if (e != cudaSuccess) return 0;
    std::lock_guard<std::mutex> g(m);
    cache[key] = n;
    return n;
}

bool walk_f32_is_kernel(const void *fn) {
    return fn == reinterpret_cast<const void *>(walk_f32_kernel<false, false>) ||
           fn == reinterpret_cast<const void *>(walk_f32_kernel<true, false>) ||
           fn == reinterpret_cast<const void *>(walk_f32_kernel<false, true>) ||
           fn == reinterpret_cast<const void *>(walk_f32_kernel<true, true>) ||
           fn == reinterpret_cast<const void *>(drain_kernel<false, false>) ||
           fn == reinterpret_cast<const void *>(drain_kernel<true, false>) ||
           fn == reinterpret_cast<const void *>(drain_kernel<false, true>) ||
           fn == reinterpret_cast<const void *>(drain_kernel<true, true>);
}

cudaError_t launch_walk_f32(const WalkArgs &a, bool impurity, int grid, int block, int sm_count, cudaStream_t s) {
    cudaError_t e = allow_smem();
    if (e != cudaSuccess) return e;
    const size_t smem = smem_bytes(block, a.n_cfg);
    if (a.deep) {
        if (impurity) walk_f32_kernel<true, true><<<grid, block, smem, s>>>(a);
        else walk_f32_kernel<false, true><<<grid, block, smem, s>>>(a);
    } else {
        if (impurity) walk_f32_kernel<true, false><<<grid, block, smem, s>>>(a);
        else walk_f32_kernel<false, false><<<grid, block, smem, s>>>(a);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess || a.drain_from <= 0 || !a.drain) return e;
    // the drain kernel: as many blocks as fit at once, each taking the handed-over
    // photons one at a time
    static std::atomic<int> per_sm_cached{0};
    int per_sm = per_sm_cached.load();
    if (per_sm == 0) {
        // (the four instances hold the same block size and shared memory)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, drain_kernel<true, false>, kCtaWalkThreads, 0);
        if (e != cudaSuccess) return e;
        per_sm = std::max(1, per_sm);
        per_sm_cached.store(per_sm);
    }
    const int dgrid = std::max(1, sm_count) * per_sm;
    if (a.deep) {
        if (impurity) drain_kernel<true, true><<<dgrid, kCtaWalkThreads, 0, s>>>(a);
        else drain_kernel<false, true><<<dgrid, kCtaWalkThreads, 0, s>>>(a);
    } else {
        if (impurity) drain_kernel<true, false><<<dgrid, kCtaWalkThreads, 0, s>>>(a);
        else drain_kernel<false, false><<<dgrid, kCtaWalkThreads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace mcw
