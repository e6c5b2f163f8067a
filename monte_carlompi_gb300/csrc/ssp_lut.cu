// Wavelength lookup table of the FP32 walk.
//
// Photon wavelengths are rounded to 0.01 um (np.around(..., 2),
// monte_carlo3D.py:1519-1520), so a config only ever sees the grid points
// lambda_k = k / 100 um within a few sigma of its centre.  One thread per grid
// point evaluates the per-photon optics of monte_carlo3D.py:1524-1612 (two
// nearest table points, scipy's linear form, nearest value outside them) in
// FP64 and stores what the walk reads at photon birth.  Compiled with
// --fmad=false, like the replay walk, so both see the same optics.
#include <cuda_runtime.h>

#include "mcw_internal.cuh"
#include "ssp_device.cuh"

namespace mcw {

namespace {

// One block per config: clears the call's counters and the config's tally
// (they must start at zero), stages the wavelength columns of its tables in
// shared memory when they fit, then fills the config's grid points (unless
// clear_only: a repeated call on the same configs and tables).
__global__ void lut_kernel(const LutArgs a) {
    extern __shared__ double s_wvl[];
    const int ci = blockIdx.x;
    const DevConfig c = a.cfgs[ci];
    if (a.tallies) {
        uint32_t *t = reinterpret_cast<uint32_t *>(a.tallies + ci);
        for (int i = threadIdx.x; i < (int)(sizeof(mcw_tally) / 4); i += blockDim.x) t[i] = 0u;
    }
    if (a.counters && ci == 0)
        for (int i = threadIdx.x; i < a.counters_words; i += blockDim.x) a.counters[i] = 0u;
    if (a.clear_only) return;   // the table of these configs is already in place
    DevTable ice = a.ice[c.ice_table];
    DevTable imp = a.imp;
    if (a.stage) {
        for (int i = threadIdx.x; i < ice.n; i += blockDim.x) s_wvl[i] = ice.wvl[i];
        for (int i = threadIdx.x; i < imp.n; i += blockDim.x) s_wvl[ice.n + i] = imp.wvl[i];
        __syncthreads();
        ice.wvl = s_wvl;
        imp.wvl = s_wvl + ice.n;
    }
    for (int j = threadIdx.x; j < c.lut_n; j += blockDim.x) {
        const int k = c.k_lo + j;
        const double wvl = (double)k / 100.0;
        const Optics o = photon_optics(c, ice, imp, wvl);
        const double wvn = 1.0 / o.wvl_um;
        LutEntry L;
        L.wvn = (float)wvn;
        L.coalb_ice = (float)(1.0 - o.ssa_ice);
        L.coalb_imp = (float)(1.0 - o.ssa_imp);
        L.g = (float)o.g;
        L.inv_ext = (float)(1.0 / (o.ext_cff_mss * c.rho_snw));
        L.p_imp = (float)o.p_imp;
        L.snow_depth = (float)o.snow_depth;
        L.pad = 0.f;
        L.wvn_fx = (unsigned long long)llrint(wvn * 4294967296.0);
        L.pad2 = (unsigned long long)o.row;   // the nearest ice-table row (polarised walk)
        a.lut[c.lut_off + j] = L;
    }
}

}  // namespace

cudaError_t launch_lut(const LutArgs &a, cudaStream_t s) {
    if (a.n_cfg <= 0) return cudaSuccess;
    const size_t smem = (a.stage && !a.clear_only) ? (size_t)a.stage_doubles * sizeof(double) : 0;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(lut_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    lut_kernel<<<a.n_cfg, 128, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcw
