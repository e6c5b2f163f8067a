"""ctypes front end of the C oracle (``oracle/walk_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'liboracle_walk.so')

RECORD_DTYPE = np.dtype([
    ('condition', np.int32), ('n_scat', np.int32), ('wvn', np.float64),
    ('theta_n', np.float64), ('phi_n', np.float64), ('path_length', np.float64),
    ('snow_depth', np.float64), ('n_draws', np.int64), ('phi_undefined', np.int32),
    ('pad', np.int32), ('stokes', np.float64, (4,))])


class Table(ctypes.Structure):
    _fields_ = [('wvl', ctypes.c_void_p), ('ssa', ctypes.c_void_p), ('ext', ctypes.c_void_p),
                ('asm_', ctypes.c_void_p), ('n', ctypes.c_int32), ('unit', ctypes.c_int32)]


class Config(ctypes.Structure):
    _fields_ = [('n_photon', ctypes.c_int64), ('wvl0', ctypes.c_double),
                ('half_width', ctypes.c_double), ('theta0_deg', ctypes.c_double),
                ('tau_tot', ctypes.c_double), ('imp_cnc', ctypes.c_double),
                ('rho_snw', ctypes.c_double), ('rho_ice', ctypes.c_double),
                ('lam_surface', ctypes.c_int32), ('lam_bottom', ctypes.c_int32),
                ('R', ctypes.c_double), ('ssa_ice_override', ctypes.c_double),
                ('g_override', ctypes.c_double), ('ext_ice_override', ctypes.c_double),
                ('ssa_imp_override', ctypes.c_double), ('ext_imp_override', ctypes.c_double),
                ('nearest', ctypes.c_int32), ('pad', ctypes.c_int32), ('phase', ctypes.c_void_p)]


class Phase(ctypes.Structure):
    _fields_ = [('n_rows', ctypes.c_int32), ('pad', ctypes.c_int32),
                ('n_angle', ctypes.c_int32 * 6), ('cos_asc', ctypes.c_void_p * 6),
                ('p_asc', ctypes.c_void_p * 6), ('a1', ctypes.c_void_p), ('a2', ctypes.c_void_p),
                ('b1', ctypes.c_void_p), ('b2', ctypes.c_void_p), ('cos_max', ctypes.c_double),
                ('cos_min', ctypes.c_double), ('cos_cutoff', ctypes.c_double),
                ('stokes0', ctypes.c_double * 4)]


def make_phase(pt, stokes0):
    """ctypes view of a monte_carlompi_gb300.ssp.PhaseTable (keeps its arrays alive)."""
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in pt.cos_asc + pt.p_asc]
    ext = [np.ascontiguousarray(a, dtype=np.float64) for a in (pt.a1, pt.a2, pt.b1, pt.b2)]
    ph = Phase()
    ph.n_rows = pt.p_asc[0].shape[0]
    for e in range(6):
        ph.n_angle[e] = keep[e].size
        ph.cos_asc[e] = keep[e].ctypes.data
        ph.p_asc[e] = keep[6 + e].ctypes.data
    ph.a1, ph.a2, ph.b1, ph.b2 = (a.ctypes.data for a in ext)
    ph.cos_max, ph.cos_min, ph.cos_cutoff = pt.cos_max, pt.cos_min, pt.cos_cutoff
    for k in range(4):
        ph.stokes0[k] = float(stokes0[k])
    ph._keep = keep + ext
    return ph


def build():
    """Compile the oracle (make, gcc) into oracle/_build."""
    subprocess.run(['make', '-s', '-C', HERE], check=True)


_lib = None


ULP_LIB_PATH = os.path.join(HERE, '_build', 'liboracle_walk_ulp.so')
_ulp_lib = None


def _bind(L):
    L.orc_uniform.restype = ctypes.c_double
    L.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64]
    L.orc_wavelength.restype = ctypes.c_double
    L.orc_wavelength.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
    L.orc_philox4x32_10.argtypes = [ctypes.c_void_p] * 3
    L.orc_walk_range.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Table),
                                 ctypes.POINTER(Table), ctypes.c_uint64, ctypes.c_int64,
                                 ctypes.c_int64, ctypes.c_void_p]
    L.orc_walk_threads.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Table),
                                   ctypes.POINTER(Table), ctypes.c_uint64, ctypes.c_int64,
                                   ctypes.c_int, ctypes.c_void_p]
    L.orc_walk_threads.restype = ctypes.c_int
    return L


def ulp_lib():
    """The oracle built with log, sin and cos moved by one ulp (a stand-in for a
    different libm, such as CUDA's on the GPU): tests measure how far one-ulp
    differences carry through the walk."""
    global _ulp_lib
    if _ulp_lib is None:
        if not os.path.exists(ULP_LIB_PATH):
            build()
        _ulp_lib = _bind(ctypes.CDLL(ULP_LIB_PATH))
    return _ulp_lib


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_uniform.restype = ctypes.c_double
        L.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_wavelength.restype = ctypes.c_double
        L.orc_wavelength.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
        L.orc_philox4x32_10.argtypes = [ctypes.c_void_p] * 3
        L.orc_walk_range.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Table),
                                     ctypes.POINTER(Table), ctypes.c_uint64, ctypes.c_int64,
                                     ctypes.c_int64, ctypes.c_void_p]
        L.orc_walk_threads.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Table),
                                       ctypes.POINTER(Table), ctypes.c_uint64, ctypes.c_int64,
                                       ctypes.c_int, ctypes.c_void_p]
        L.orc_walk_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


class _Tables:
    """Keeps the numpy arrays of two SSP tables alive while C reads them."""

    def __init__(self, ice, imp):
        self.arrays = []

        def mk(t):
            cols = [np.ascontiguousarray(t.wvl, dtype=np.float64),
                    np.ascontiguousarray(t.ss_alb, dtype=np.float64),
                    np.ascontiguousarray(t.ext_cff_mss, dtype=np.float64),
                    np.ascontiguousarray(t.asm_prm, dtype=np.float64)]
            self.arrays.extend(cols)
            return Table(cols[0].ctypes.data, cols[1].ctypes.data, cols[2].ctypes.data,
                         cols[3].ctypes.data, cols[0].size, int(getattr(t, 'wvl_unit', 0)))
        self.ice = mk(ice)
        self.imp = mk(imp)


def make_config(n_photon, wvl0, half_width, theta0_deg, tau_tot, imp_cnc=0.0, rho_snw=300.0,
                rho_ice=917.0, lam_surface=False, lam_bottom=True, R=1.0,
                ssa_ice_override=np.nan, g_override=np.nan, ext_ice_override=np.nan,
                ssa_imp_override=np.nan, ext_imp_override=np.nan, nearest=False, phase=None):
    """phase: a Phase (make_phase) for the polarised walk, or None."""
    c = Config(int(n_photon), wvl0, half_width, theta0_deg, tau_tot, imp_cnc, rho_snw, rho_ice,
               int(bool(lam_surface)), int(bool(lam_bottom)), R, ssa_ice_override,
               g_override, ext_ice_override, ssa_imp_override, ext_imp_override,
               int(bool(nearest)), 0, None if phase is None else ctypes.addressof(phase))
    c._phase = phase
    return c


def walk(cfg, ice, imp, seed, p0=0, p1=None, threads=1, ulp=False):
    """FP64 replay walk of photons [p0, p1) -> structured array (RECORD_DTYPE).
    ulp: walk with the one-ulp libm stand-in (ulp_lib) instead."""
    if p1 is None:
        p1 = cfg.n_photon
    L = ulp_lib() if ulp else lib()
    tabs = _Tables(ice, imp)
    out = np.zeros(p1 - p0, dtype=RECORD_DTYPE)
    if threads > 1 and p0 == 0:
        rc = L.orc_walk_threads(ctypes.byref(cfg), ctypes.byref(tabs.ice), ctypes.byref(tabs.imp),
                                    int(seed), int(p1), int(threads), out.ctypes.data)
        if rc:
            raise RuntimeError('oracle thread start failed')
    else:
        L.orc_walk_range(ctypes.byref(cfg), ctypes.byref(tabs.ice), ctypes.byref(tabs.imp),
                         int(seed), int(p0), int(p1), out.ctypes.data)
    return out


def config_from_golden(g):
    """Config of a golden fixture (tests/golden/*.npz)."""
    p = lambda k: g['param_' + k].item()  # noqa: E731
    return make_config(p('n_photon'), p('wvl0'), p('half_width'), p('theta0'), p('tau_tot'),
                       p('imp_cnc'), p('rho_snw'), p('rho_ice'), p('lam_surface'),
                       p('lam_bottom'), p('R'), ssa_ice_override=p('ssa_ice_override'),
                       g_override=p('g_override'),
                       nearest=bool(g['param_ssp_nearest'].item()) if 'param_ssp_nearest' in g else False,
                       phase=phase_from_golden(g))


def phase_from_golden(g):
    """The polarised walk's phase matrices of a golden fixture (None for the others)."""
    if 'param_polarised' not in g:
        return None
    from monte_carlompi_gb300 import ssp
    return make_phase(ssp_phase_from_golden(g), g['stokes0'])


def ssp_phase_from_golden(g):
    """PhaseTable of a golden fixture: its stored P rows (P12 ... P44 divided by P11)
    for the isca.dat rows of the selected size, in the SSP table's order."""
    from monte_carlompi_gb300 import ssp
    rows = g['isca_rows']
    re = 0.75 * rows[:, 2] / rows[:, 3]
    sel = np.where(re == re[np.argmin(np.abs(re - g['param_rds_selected'].item()))])[0]
    sel = sel[np.argsort(rows[sel, 0], kind='stable')]
    st = g['phase_stored']
    p11 = st[0][sel]
    els = [p11] + [e[sel] * p11 for e in st[1:]]
    theta = g['phase_theta']
    return ssp.phase_table([theta] * 6, els, rows[sel, 0], g['param_wvl0'].item())


def tables_from_golden(g):
    from monte_carlompi_gb300.ssp import SSPTable
    unit = int(g['ice_unit'].item()) if 'ice_unit' in g else 0
    ice = SSPTable(g['ice_wvl'], g['ice_ssa'], g['ice_ext'], g['ice_asm'], wvl_unit=unit)
    imp = SSPTable(g['imp_wvl'], g['imp_ssa'], g['imp_ext'], None)
    return ice, imp
