// SSP lookup on the device, FP64, in the reference's operation order.
// Translation units that include this are compiled with --fmad=false so no
// multiply-add is contracted.
#pragma once
#include "mcw_internal.cuh"

namespace mcw {

// The two table points nearest to w (in the table's unit); ties keep the lower index.
// monte_carlo3D.py:594-597 (argsort of |wvl - wvl_in|, first two).  Tables are
// strictly increasing (mcw_set_tables sorts and checks them), so the two
// nearest points are among the two on either side of w: a binary search finds
// them, and scanning those four in index order picks the same pair a scan of
// the whole table would.
__device__ inline void ssp_nearest_two(const DevTable &t, double w, int &i0, int &i1) {
    int lo = 0, hi = t.n - 1;  // largest i with wvl[i] <= w, or -1
    int k = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (t.wvl[mid] <= w) { k = mid; lo = mid + 1; }
        else hi = mid - 1;
    }
    int a = -1, b = -1;
    double da = __longlong_as_double(0x7ff0000000000000LL), db = da;
    const int j0 = max(k - 1, 0), j1 = min(k + 2, t.n - 1);
    for (int i = j0; i <= j1; ++i) {
        double d = fabs(w - t.wvl[i]);
        if (d < da) { b = a; db = da; a = i; da = d; }
        else if (d < db) { b = i; db = d; }
    }
    i0 = a;
    i1 = b;
}

// scipy interp1d linear form between the two points; the nearest value when
// w lies outside them (interp1d raises ValueError, monte_carlo3D.py:612-616).
__device__ inline double ssp_interp_two(const DevTable &t, const double *y, int i0, int i1, double w) {
    double x0 = t.wvl[i0], x1 = t.wvl[i1], y0 = y[i0], y1 = y[i1];
    double xl, xh, yl, yh;
    if (x0 < x1) { xl = x0; xh = x1; yl = y0; yh = y1; }
    else { xl = x1; xh = x0; yl = y1; yh = y0; }
    if (w < xl || w > xh) return y0;
    return ((w - xl) / (xh - xl)) * yh + ((xh - w) / (xh - xl)) * yl;
}

struct Optics {
    int row;         // the nearest ice-table row
    double wvl_um;   // the photon's wavelength: its drawn one, or the nearest table point's (ssp_nearest)
    double ssa_ice, ssa_imp, g, ext_cff_mss, p_imp, snow_depth;
};

// A wavelength in um in the table's unit: wvl * 1e-6 for the netCDF tables
// (monte_carlo3D.py:518, :673), as is for the aspherical rows (:323-334).
__device__ inline double in_table_unit(const DevTable &t, double wvl_um) {
    return t.unit == MCW_WVL_MICRONS ? wvl_um : wvl_um * 1e-6;
}

// Per-photon optics at wavelength wvl_um: monte_carlo3D.py:1524-1612.  With
// ssp_nearest (HG-forced aspherical particles) the ice properties are those of
// the nearest table point and the photon carries that point's wavelength from
// then on: the impurity lookup and wvn use it (:323-334, :396-415, :1534-1549).
__device__ inline Optics photon_optics(const DevConfig &c, const DevTable &ice, const DevTable &imp,
                                       double wvl_um) {
    double w = in_table_unit(ice, wvl_um);
    int i0, i1;
    ssp_nearest_two(ice, w, i0, i1);
    const int i_row = i0;
    double ssa_ice, ext_ice, g;
    if (c.flags & kFlagNearest) {
        ssa_ice = ice.ssa[i0];
        ext_ice = ice.ext[i0];
        g = ice.asm_[i0];
        wvl_um = ice.unit == MCW_WVL_MICRONS ? ice.wvl[i0] : ice.wvl[i0] * 1e6;
    } else {
        ssa_ice = ssp_interp_two(ice, ice.ssa, i0, i1, w);
        ext_ice = ssp_interp_two(ice, ice.ext, i0, i1, w);
        g = ssp_interp_two(ice, ice.asm_, i0, i1, w);
    }
    w = in_table_unit(imp, wvl_um);
    ssp_nearest_two(imp, w, i0, i1);
    double ssa_imp = ssp_interp_two(imp, imp.ssa, i0, i1, w);
    double ext_imp = ssp_interp_two(imp, imp.ext, i0, i1, w);
    if (!isnan(c.ov_ssa_ice)) ssa_ice = c.ov_ssa_ice;
    if (!isnan(c.ov_ext_ice)) ext_ice = c.ov_ext_ice;
    if (!isnan(c.ov_g)) g = c.ov_g;
    if (!isnan(c.ov_ssa_imp)) ssa_imp = c.ov_ssa_imp;
    if (!isnan(c.ov_ext_imp)) ext_imp = c.ov_ext_imp;
    double cnc = c.imp_cnc;
    Optics o;
    o.row = i_row;
    o.wvl_um = wvl_um;
    o.ssa_ice = ssa_ice;
    o.ssa_imp = ssa_imp;
    o.g = g;
    o.ext_cff_mss = ext_ice * (1 - cnc) + ext_imp * cnc;
    o.p_imp = (cnc * ext_imp) / (cnc * ext_imp + (1 - cnc) * ext_ice);
    o.snow_depth = c.tau_tot_d / (o.ext_cff_mss * c.rho_snw);
    return o;
}

}  // namespace mcw
