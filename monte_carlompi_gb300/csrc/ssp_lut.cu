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

__global__ void lut_kernel(const LutArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.lut_total) return;
    const int ci = a.lut_cfg[e];
    const DevConfig c = a.cfgs[ci];
    const int k = c.k_lo + (e - c.lut_off);
    const double wvl = (double)k / 100.0;
    const Optics o = photon_optics(c, a.ice[c.ice_table], a.imp, wvl);
    const double wvn = 1.0 / wvl;
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
    L.pad2 = 0;
    a.lut[e] = L;
}

}  // namespace

cudaError_t launch_lut(const LutArgs &a, cudaStream_t s) {
    if (a.lut_total <= 0) return cudaSuccess;
    const int block = 128;
    lut_kernel<<<(a.lut_total + block - 1) / block, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcw
