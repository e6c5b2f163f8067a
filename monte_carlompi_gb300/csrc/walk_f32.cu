// Production FP32 photon walk: a persistent grid of warps, each lane walking
// one photon at a time.  Photon ids come from one global counter; a warp
// refills its idle lanes (photon regeneration) so lanes whose photons leave
// early keep working instead of idling until the warp's longest walk ends.
//
// Per step (monte_carloMPI/monte_carlo3D.py:1212-1466, HG branch) one
// Philox4x32-10 block keyed by (step, photon) supplies the four uniforms the
// step needs: HG cosine (:915), azimuth (:921), optical path (:1014) and the
// absorption draw (:1020).  The ice/impurity draw (:1023) and the bottom
// reflectance draw (:1422/:1453) take their own blocks only when the config
// needs them.  Results depend only on (seed, photon id): any launch shape,
// any number of GPUs or replicas gives the same records.
//
// Statistically equivalent restatements (identical distributions):
//  * the Lambertian direction (p(theta) ~ sin 2 theta, :1238-1250) is drawn by
//    inversion, cos theta = sqrt(u), instead of rejection;
//  * absorption tests 1 - u < 1 - ssa on a 32-bit uniform, so small
//    co-albedos (1e-6) are resolved; likewise the species test;
//  * the azimuth is uniform on (-pi, pi) instead of (0, 2 pi);
//  * the direction is renormalised after every rotation and the pole branch
//    (:1262-1269) is taken for |mu_z| > 0.99999 instead of |mu_z| == 1;
//  * phi_n = atan2(mu_y, mu_x) mapped to [0, 2 pi) (the quadrant arctan of
//    :1472-1485, defined on the axes too).
#include <cuda_runtime.h>

#include "mcw_internal.cuh"
#include "tally.cuh"

namespace mcw {

namespace {

constexpr float kTwoPiF = 6.28318530717958648f;
constexpr float kTwo32Inv = 2.3283064365386963e-10f;  // 2^-32
constexpr float kTwo33Inv = 1.16415321826934814e-10f; // 2^-33
constexpr uint32_t kFlagReflect = 8u;                  // bottom reflection pending
constexpr int kSmemCfgMax = 256;                       // configs staged in shared memory

// Per-config values the FP32 walk reads at photon birth (staged in shared memory).
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

// Start photon p (index within its config) of config ci.
__device__ __forceinline__ void birth(Photon &P, int64_t p, int ci, const CfgF32 &c,
                                      const WalkArgs &a) {
    const uint64_t rid = c.rng_base + (uint64_t)p;
    const uint4 r = philox10(make_uint4(0u, kTagBirth, (uint32_t)rid, (uint32_t)(rid >> 32)), a.keys);
    // Box-Muller normal for the wavelength (monte_carlo3D.py:1516-1520)
    const float u0 = u01_f32(r.x), u1 = u01_f32(r.y);
    float s, co;
    __sincosf(kTwoPiF * (u1 - 0.5f), &s, &co);
    const float zn = sqrtf(-2.f * __logf(u0)) * co;
    const int k = __float2int_rn(fmaf(c.sigma_100, zn, c.wvl0_100));
    const int idx = min(max(k - c.k_lo, 0), c.lut_n - 1);
    P.rid = rid;
    P.cfg = ci;
    P.lut = c.lut_off + idx;
    const LutEntry *e = a.lut + P.lut;
    const float4 e0 = __ldg(reinterpret_cast<const float4 *>(e));
    const float4 e1 = __ldg(reinterpret_cast<const float4 *>(e) + 1);
    // e0 = (wvn, coalb_ice, coalb_imp, g), e1 = (inv_ext, p_imp, snow_depth, -)
    P.coalb_ice = e0.y;
    P.coalb_imp = e0.z;
    const float g = e0.w;
    P.inv_ext = e1.x;
    P.p_imp = e1.y;
    if (fabsf(g) > 1e-6f) {
        P.hg_a = 1.f + g * g;
        P.hg_b = 1.f - g * g;
        P.hg_c = 1.f - g;
        P.hg_d = 2.f * g;
        P.hg_e = 1.f / (2.f * g);
    } else {
        P.hg_a = P.hg_b = P.hg_c = P.hg_e = 0.f;
        P.hg_d = 0.f;
    }
    P.flags = c.flags;
    P.tau = c.tau_tot;
    P.R = c.R;
    P.mux = c.mux0;
    P.muy = 0.f;
    P.muz = c.muz0;
    P.z = 0.f;
    P.path = 0.f;
    P.pathc = 0.f;
    P.i = 0;
}

// One scatter event (monte_carlo3D.py:1213-1466).  Returns the end condition
// (0 = still walking).
__device__ __forceinline__ int step(Photon &P, const WalkArgs &a) {
    P.i += 1;
    const uint32_t glo = (uint32_t)P.rid, ghi = (uint32_t)(P.rid >> 32);
    const uint4 r = philox10(make_uint4((uint32_t)P.i, kTagStep, glo, ghi), a.keys);
    const float u1 = u01_f32(r.x);
    const float u2 = u01_f32(r.y);
    const float u3 = fmaf((float)r.z, kTwo32Inv, kTwo33Inv);
    const bool first = (P.i == 1);
    const bool lam_surface = (P.flags & kFlagLamSurface) != 0;

    float dtau = -__logf(u3);
    if (first && lam_surface) dtau = 0.f;

    // scattering angle: HG inversion, or Lambertian after a bottom reflection
    const bool lamb = !first && (lam_surface || (P.flags & kFlagReflect));
    float ct;
    if (lamb) {
        ct = sqrtf(u1);
    } else if (P.hg_d != 0.f) {
        const float t = __fdividef(P.hg_b, fmaf(P.hg_d, u1, P.hg_c));
        ct = P.hg_e * (P.hg_a - t * t);
        ct = fminf(fmaxf(ct, -1.f), 1.f);
    } else {
        ct = 1.f - 2.f * u1;
    }
    const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
    float sp, cp;
    __sincosf(kTwoPiF * (u2 - 0.5f), &sp, &cp);

    float mx = P.mux, my = P.muy, mz = P.muz;
    if (lamb) { mx = 0.f; my = 0.f; mz = 1.f; }
    float nx, ny, nz;
    if (first) {
        nx = mx; ny = my; nz = mz;
    } else if (fabsf(mz) > 0.99999f) {
        const float sg = copysignf(1.f, mz);
        nx = st * cp;
        ny = sg * st * sp;
        nz = sg * ct;
    } else {
        const float s2 = 1.f - mz * mz;
        const float rs = rsqrtf(s2);
        const float tq = st * rs;
        nx = tq * (mx * mz * cp - my * sp) + mx * ct;
        ny = tq * (my * mz * cp + mx * sp) + my * ct;
        nz = -(s2 * rs) * st * cp + mz * ct;
        const float inv = rsqrtf(nx * nx + ny * ny + nz * nz);
        nx *= inv; ny *= inv; nz *= inv;
    }
    P.flags &= ~kFlagReflect;

    const float z0 = P.z;
    float zn = z0 + dtau * nz;
    // path length, compensated sum
    const float inc = dtau * P.inv_ext;
    {
        const float y = inc - P.pathc;
        const float t = P.path + y;
        P.pathc = (t - P.path) - y;
        P.path = t;
    }

    // ice or impurity (monte_carlo3D.py:1375-1383)
    bool imp = false;
    if (P.flags & kFlagImpurity) {
        const uint4 r2 = philox10(make_uint4((uint32_t)P.i, kTagSpecies, glo, ghi), a.keys);
        imp = ((float)r2.x * kTwo32Inv) < P.p_imp;
    }
    float coalb = imp ? P.coalb_imp : P.coalb_ice;
    if (lam_surface) coalb = 1.f - P.R;

    int cond = 0;
    if (zn > 0.f) {                                         // :1390-1397
        cond = 1;
        P.path -= (zn / (zn - z0)) * inc;
    } else if (zn < -P.tau) {                               // :1399-1459
        P.path -= ((zn + P.tau) / (zn - z0)) * inc;
        zn = -P.tau;
        bool leave = true;
        if (P.flags & kFlagLamBottom) {
            const uint4 r3 = philox10(make_uint4((uint32_t)P.i, kTagBottom, glo, ghi), a.keys);
            if ((float)r3.x * kTwo32Inv < P.R) {
                leave = false;
                P.flags |= kFlagReflect;
            }
        }
        if (leave) cond = first ? 3 : 2;
    } else if ((float)r.w * kTwo32Inv < coalb) {           // :1461-1466
        cond = imp ? 5 : 4;
    }
    P.mux = nx;
    P.muy = ny;
    P.muz = nz;
    P.z = zn;
    return cond;
}

__global__ void __launch_bounds__(256) walk_f32_kernel(const WalkArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    WarpTally *wtally = reinterpret_cast<WarpTally *>(smem);
    CfgF32 *scfg = reinterpret_cast<CfgF32 *>(smem + sizeof(WarpTally) * 32);
    int64_t *sprefix = reinterpret_cast<int64_t *>(smem + sizeof(WarpTally) * 32 + sizeof(CfgF32) * kSmemCfgMax);

    // stage configs in shared memory when they fit, else read them from global
    const bool staged = a.n_cfg <= kSmemCfgMax;
    if (staged) {
        for (int c = threadIdx.x; c < a.n_cfg; c += blockDim.x) {
            scfg[c] = make_cfg(a.cfgs[c]);
            sprefix[c] = a.prefix[c];
        }
    }
    const int64_t *prefix = staged ? sprefix : a.prefix;
    WarpTally &wt = wtally[warp];
    warp_tally_reset(wt, lane);
    __syncthreads();

    Photon P;
    P.rid = 0;
    P.cfg = -1;
    P.lut = 0;
    P.i = 0;
    bool exhausted = false;
    const unsigned long long t0 = global_ns();
    const unsigned lt_mask = (1u << lane) - 1u;

    for (uint32_t iter = 0;; ++iter) {
        // ---- regeneration: refill idle lanes from the global photon counter
        const unsigned idle = __ballot_sync(0xffffffffu, P.cfg < 0);
        const int nidle = __popc(idle);
        if (!exhausted && nidle > 0 && (nidle >= a.regen_chunk || nidle == 32)) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(a.work, (unsigned long long)nidle);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (unsigned long long)nidle >= (unsigned long long)a.total) exhausted = true;
            if (P.cfg < 0) {
                const int64_t g = (int64_t)base + __popc(idle & lt_mask);
                if (g < a.total) {
                    const int ci = find_config(prefix, a.n_cfg, g);
                    const CfgF32 c = staged ? scfg[ci] : make_cfg(a.cfgs[ci]);
                    birth(P, g - prefix[ci], ci, c, a);
                }
            }
        }
        const unsigned active = __ballot_sync(0xffffffffu, P.cfg >= 0);
        if (active == 0) break;  // nothing left: counter exhausted and all walks done

        // ---- one scatter event per active lane
        int cond = 0;
        if (P.cfg >= 0) cond = step(P, a);

        // ---- finished photons: record, tallies
        const unsigned fin_mask = __ballot_sync(0xffffffffu, cond != 0);
        if (fin_mask) {
            const bool fin = cond != 0;
            float wvn = 0.f, depth = 0.f, theta = 0.f, phi = 0.f;
            unsigned long long wfx = 0;
            const int nscat = P.i - 1;
            if (fin) {
                const LutEntry *e = a.lut + P.lut;
                wvn = __ldg(&e->wvn);
                depth = __ldg(&e->snow_depth);
                wfx = __ldg(&e->wvn_fx);
                theta = acosf(fminf(fmaxf(P.muz, -1.f), 1.f));
                if (P.i > 1) {
                    phi = atan2f(P.muy, P.mux);
                    if (phi < 0.f) phi += kTwoPiF;
                    if (phi >= kTwoPiF) phi = 0.f;
                }
                if (a.records) {
                    const uint64_t base_rid = staged ? scfg[P.cfg].rng_base : a.cfgs[P.cfg].rng_base;
                    const int64_t gid = prefix[P.cfg] + (int64_t)(P.rid - base_rid);
                    float4 *dst = reinterpret_cast<float4 *>(a.records + gid);
                    dst[0] = make_float4(__int_as_float(cond), __int_as_float(nscat), wvn, theta);
                    dst[1] = make_float4(phi, P.path, depth, __uint_as_float((uint32_t)P.cfg));
                }
                if (cond == 1) tally_bin(a.tallies + P.cfg, wfx, theta, phi);
            }
            // warp running totals (shared memory), flushed when the config changes
            const unsigned other = __ballot_sync(0xffffffffu, fin && P.cfg != wt.cfg);
            if (other) {
                unsigned pending = fin_mask;
                while (pending) {
                    const int leader = __ffs(pending) - 1;
                    const int c = __shfl_sync(0xffffffffu, P.cfg, leader);
                    const unsigned m = __ballot_sync(0xffffffffu, fin && P.cfg == c);
                    if (wt.cfg != c) {
                        warp_tally_flush(wt, a.tallies, lane);
                        if (lane == 0) wt.cfg = c;
                        __syncwarp();
                    }
                    if (m & (1u << lane)) {
                        atomicAdd(&wt.n_cond[cond], 1u);
                        atomicAdd(&wt.q_cond_fx[cond], wfx);
                        atomicAdd(&wt.n_events, (unsigned long long)nscat);
                        atomicMax(&wt.max_n_scat, (uint32_t)nscat);
                    }
                    __syncwarp();
                    pending &= ~m;
                }
            } else if (fin) {
                atomicAdd(&wt.n_cond[cond], 1u);
                atomicAdd(&wt.q_cond_fx[cond], wfx);
                atomicAdd(&wt.n_events, (unsigned long long)nscat);
                atomicMax(&wt.max_n_scat, (uint32_t)nscat);
            }
            if (fin) P.cfg = -1;
        }

        // ---- time budget (watchdog; never a truncation in normal runs)
        if ((iter & 255u) == 255u) {
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
    warp_tally_flush(wt, a.tallies, lane);
}

}  // namespace

size_t walk_f32_smem_bytes(int block) {
    (void)block;
    return sizeof(WarpTally) * 32 + sizeof(CfgF32) * kSmemCfgMax + sizeof(int64_t) * kSmemCfgMax;
}

int walk_f32_max_blocks_per_sm(int block) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, walk_f32_kernel, block,
                                                      walk_f32_smem_bytes(block)) != cudaSuccess)
        return 0;
    return n;
}

const void *walk_f32_kernel_fn() { return reinterpret_cast<const void *>(walk_f32_kernel); }

cudaError_t launch_walk_f32(const WalkArgs &a, int grid, int block, cudaStream_t s) {
    const size_t smem = walk_f32_smem_bytes(block);
    walk_f32_kernel<<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcw
