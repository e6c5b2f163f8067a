"""Single-scattering-property (SSP) tables: synthetic formulas and netCDF I/O.

The reference reads ice SSPs from ``<optics_dir>/mie/snicar/ice_wrn_%04d.nc``
(monte_carlo3D.py:507-514) and impurity SSPs from ``<optics_dir>/mie/snicar/
<fi_imp>`` (monte_carlo3D.py:666-671).  Each file holds ``wvl`` in metres and
``ss_alb`` / ``ext_cff_mss`` (m^2/kg), plus ``asm_prm`` for ice.  The bundled
Bohren-and-Huffman tables are not part of the reference archive, so tables are
either read from such files when present or synthesised from the closed forms
below, on a 1 nm grid.

Synthetic ice spheres (r_eff in um, lambda in um, Q_ext = 2):

* ``ext_cff_mss = 3 Q_ext / (4 rho_ice r_eff[m])`` (independent of lambda);
* ``asm_prm = 0.89``;
* ``1 - ss_alb = 1e-4 * 100 ** ((lambda - 1.2) / 0.4) * (r_eff / 100)``, capped
  at 0.5 (the geometric-optics floor ss_alb >= 0.5) because the formula
  exceeds 1 for r_eff = 1500 um beyond 1.765 um.

Synthetic impurity (black carbon): ``ss_alb = 0.30``, ``ext_cff_mss = 12000``
m^2/kg, the hand-set 500 nm values of monte_carlo3D.py:1868-1894.
"""
import math
import os
from dataclasses import dataclass

import numpy as np

Q_EXT = 2.0
G_SYNTH = 0.89
CO_ALBEDO_CAP = 0.5
IMP_SSA = 0.30
IMP_EXT = 12000.0


@dataclass
class SSPTable:
    """One SSP table, as the reference's netCDF variables hold it."""
    wvl: np.ndarray          # metres, ascending
    ss_alb: np.ndarray
    ext_cff_mss: np.ndarray  # m^2/kg
    asm_prm: np.ndarray      # zeros for an impurity table

    def __post_init__(self):
        self.wvl = np.ascontiguousarray(self.wvl, dtype=np.float64)
        self.ss_alb = np.ascontiguousarray(self.ss_alb, dtype=np.float64)
        self.ext_cff_mss = np.ascontiguousarray(self.ext_cff_mss, dtype=np.float64)
        if self.asm_prm is None:
            self.asm_prm = np.zeros_like(self.wvl)
        self.asm_prm = np.ascontiguousarray(self.asm_prm, dtype=np.float64)
        n = self.wvl.size
        if n < 2:
            raise ValueError('an SSP table needs at least two wavelengths')
        for a in (self.ss_alb, self.ext_cff_mss, self.asm_prm):
            if a.size != n:
                raise ValueError('SSP table columns differ in length')


def ext_cff_mss_sphere(rds_um, rho_ice=917.0, q_ext=Q_EXT):
    """Mass extinction coefficient of ice spheres [m^2/kg]."""
    return 3.0 * q_ext / (4.0 * rho_ice * rds_um * 1e-6)


def co_albedo_synth(wvl_um, rds_um):
    """Synthetic 1 - ss_alb, capped at 0.5."""
    c = 1e-4 * 100.0 ** ((np.asarray(wvl_um, dtype=np.float64) - 1.2) / 0.4) * (rds_um / 100.0)
    return np.minimum(c, CO_ALBEDO_CAP)


def nm_grid(lo_nm, hi_nm):
    """Wavelengths in metres on a 1 nm grid from lo_nm to hi_nm inclusive."""
    return np.arange(int(lo_nm), int(hi_nm) + 1, dtype=np.float64) * 1e-9


def grid_for(wvl0, half_width, n_sigma=5.0):
    """1 nm grid [nm, nm] covering wvl0 +- n_sigma * sigma, sigma = FWHM / 2.355."""
    s = half_width / 2.355
    lo = int(math.floor((wvl0 - n_sigma * s) * 1000.0)) - 1
    hi = int(math.ceil((wvl0 + n_sigma * s) * 1000.0)) + 1
    return max(lo, 1), max(hi, max(lo, 1) + 1)


def synthetic_ice_table(rds_um, lo_nm, hi_nm, rho_ice=917.0):
    """Synthetic ice-sphere SSP table for effective radius ``rds_um``."""
    wvl = nm_grid(lo_nm, hi_nm)
    wvl_um = wvl * 1e6
    ssa = 1.0 - co_albedo_synth(wvl_um, rds_um)
    ext = np.full_like(wvl, ext_cff_mss_sphere(rds_um, rho_ice))
    asm = np.full_like(wvl, G_SYNTH)
    return SSPTable(wvl, ssa, ext, asm)


def synthetic_impurity_table(lo_nm, hi_nm):
    """Synthetic black-carbon SSP table."""
    wvl = nm_grid(lo_nm, hi_nm)
    return SSPTable(wvl, np.full_like(wvl, IMP_SSA), np.full_like(wvl, IMP_EXT),
                    np.zeros_like(wvl))


def ice_file_name(rds_snw):
    """File name the reference opens for grain size ``rds_snw`` (monte_carlo3D.py:508)."""
    return 'ice_wrn_%04d.nc' % rds_snw


def write_netcdf(path, table, with_asm=True):
    """Write ``table`` in the reference's netCDF layout (variables over dimension ``wvl``)."""
    from scipy.io import netcdf_file
    os.makedirs(os.path.dirname(path) or '.', exist_ok=True)
    f = netcdf_file(path, 'w')
    try:
        f.createDimension('wvl', table.wvl.size)
        names = [('wvl', table.wvl), ('ss_alb', table.ss_alb),
                 ('ext_cff_mss', table.ext_cff_mss)]
        if with_asm:
            names.append(('asm_prm', table.asm_prm))
        for name, data in names:
            v = f.createVariable(name, 'd', ('wvl',))
            v[:] = data
    finally:
        f.close()


def read_netcdf(path):
    """Read an SSP table written in the reference's layout.

    The reference indexes the variables directly (monte_carlo3D.py:511-514,
    668-671); values are widened to float64 here, which is exact for float32
    files.  Tables whose wavelengths are not ascending are sorted.
    """
    from scipy.io import netcdf_file
    f = netcdf_file(path, 'r', mmap=False)
    try:
        v = f.variables
        wvl = np.array(v['wvl'].data, dtype=np.float64)
        ssa = np.array(v['ss_alb'].data, dtype=np.float64)
        ext = np.array(v['ext_cff_mss'].data, dtype=np.float64)
        asm = np.array(v['asm_prm'].data, dtype=np.float64) if 'asm_prm' in v else None
    finally:
        f.close()
    order = np.argsort(wvl, kind='stable')
    if np.any(order != np.arange(wvl.size)):
        wvl, ssa, ext = wvl[order], ssa[order], ext[order]
        asm = asm[order] if asm is not None else None
    return SSPTable(wvl, ssa, ext, asm)


def load_tables(optics_dir, rds_snw, fi_imp):
    """Load (ice, impurity) tables from ``optics_dir`` like the reference does."""
    base = os.path.join(optics_dir, 'mie', 'snicar')
    ice = read_netcdf(os.path.join(base, ice_file_name(rds_snw)))
    imp = read_netcdf(os.path.join(base, fi_imp))
    return ice, imp
