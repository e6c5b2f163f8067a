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


WVL_METRES = 0    # netCDF tables
WVL_MICRONS = 1   # aspherical isca.dat rows


@dataclass
class SSPTable:
    """One SSP table, as the reference's netCDF variables hold it."""
    wvl: np.ndarray          # metres (wvl_unit WVL_METRES) or um (WVL_MICRONS), ascending
    ss_alb: np.ndarray
    ext_cff_mss: np.ndarray  # m^2/kg
    asm_prm: np.ndarray      # zeros for an impurity table
    wvl_unit: int = WVL_METRES
    source_rows: object = None  # aspherical: the isca.dat row of each entry

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


# ---------------------------------------------------------------- aspherical particles
# The Yang et al. (2013) database the reference reads for non-spherical grains
# (get_aspherical_SSPs, monte_carlo3D.py:173-256): one text file per shape and
# roughness, <optics_dir>/ice_optics/<band>/<shape>/<roughness>/isca.dat.  The
# data are not part of the reference archive; the HG-forced path (run(shape=...)
# with HG=True) needs only isca.dat, so tests write synthetic ones.

SHAPE_DIRS = {  # monte_carlo3D.py:185-202
    'solid hexagonal column': 'solid_column',
    'hexagonal plate': 'plate',
    'hollow hexagonal column': 'hollow_column',
    'droxtal': 'droxtal',
    'hollow bullet rosette': 'hollow_bullet_rosette',
    'solid bullet rosette': 'solid_bullet_rosette',
    '8-element column aggregate': 'column_8elements',
    '5-element plate aggregate': 'plate_5elements',
    '10-element plate aggregate': 'plate_10elements',
}
ROUGHNESS_DIRS = {'smooth': 'Rough000', 'moderately rough': 'Rough003',  # :206-211
                  'severely rough': 'Rough050'}


def isca_path(optics_dir, shape, roughness, wvl0):
    """Path of the isca.dat the reference opens for this shape, roughness and
    centre wavelength (the 0.2-15.25 um or 16.4-99.0 um band, :180-183, :1528-1545)."""
    if shape not in SHAPE_DIRS:
        raise ValueError('unknown shape %r' % (shape,))
    if roughness not in ROUGHNESS_DIRS:
        raise ValueError('unknown roughness %r' % (roughness,))
    if 0.2 <= wvl0 <= 15.25:
        band = '0.2-15.25'
    elif 16.4 <= wvl0 <= 99.0:
        band = '16.4-99.0'
    else:
        raise ValueError('wvl0 = %r um lies in neither band of the aspherical database' % (wvl0,))
    return os.path.join(optics_dir, 'ice_optics', band, SHAPE_DIRS[shape], ROUGHNESS_DIRS[roughness],
                        'isca.dat')


def read_isca(path):
    """Columns of isca.dat as float64 (monte_carlo3D.py:220-245): wavelength [um],
    maximum dimension [um], particle volume [um^3], projected area G [um^2], Q_ext,
    single-scattering albedo, asymmetry factor.  Parsed field by field with float(),
    as the reference does."""
    rows = []
    with open(path) as f:
        for line in f:
            v = line.split()
            rows.append([float(v[k]) for k in range(7)])
    return np.array(rows, dtype=np.float64).reshape(-1, 7)


def aspherical_table(path, wvl0, rds_snw, rho_ice=917.0):
    """The HG-forced aspherical lookup table of get_aspherical_SSPs (monte_carlo3D.py:
    248-264, :396-415): the rows of the particle size whose effective radius
    RE = 3/4 V / G at wvl0 is nearest to rds_snw (wvl0 must be one of the file's
    wavelengths, as the reference requires), with ext_cff_mss = 1e6 G Q_ext /
    (rho_ice V) [m^2/kg], sorted by wavelength, in micrometres.  Walk it with
    WalkConfig(ssp_nearest=True).  Returns (table, RE)."""
    a = read_isca(path)
    wvl, vol, G, qext, ssa, asm = a[:, 0], a[:, 2], a[:, 3], a[:, 4], a[:, 5], a[:, 6]
    at0 = np.where(wvl == wvl0)[0]
    if at0.size == 0:
        raise ValueError('wvl0 = %r um is not a wavelength of %s' % (wvl0, path))
    re = (3. / 4.) * (vol / G)
    re_sel = re[at0][np.argsort(np.absolute(rds_snw - re[at0]))[0]]
    rows = np.where(re == re_sel)[0]
    ext = (1e6 * G[rows] * qext[rows]) / (rho_ice * vol[rows])
    order = np.argsort(wvl[rows], kind='stable')
    w = wvl[rows][order]
    if np.any(np.diff(w) <= 0):
        raise ValueError('%s: repeated wavelength for RE = %r um' % (path, re_sel))
    return (SSPTable(w, ssa[rows][order], ext[order], asm[rows][order], wvl_unit=WVL_MICRONS,
                     source_rows=rows[order]), float(re_sel))


def synthetic_isca_rows(wvls_um, re_um):
    """Synthetic isca.dat rows (for tests and fixtures): for every effective radius RE
    and wavelength, a particle with G = pi (1.25 RE)^2 and V = 4/3 RE G (so
    3/4 V / G = RE), Q_ext = 2 + 0.05 sin(lambda), the sphere co-albedo formula and
    g = 0.78 + 0.02 (lambda - 1)."""
    out = []
    for r in re_um:
        dmax = 2.5 * r
        G = math.pi * (1.25 * r) ** 2
        V = (4. / 3.) * r * G
        for w in wvls_um:
            q = 2.0 + 0.05 * math.sin(w)
            co = min(1e-4 * 100.0 ** ((w - 1.2) / 0.4) * (r / 100.0), CO_ALBEDO_CAP)
            out.append((w, dmax, V, G, q, 1.0 - co, 0.78 + 0.02 * (w - 1.0)))
    return out


def write_isca(path, rows):
    """Write isca.dat rows (wavelength printed with 4 decimals, the rest as repr)."""
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, 'w') as f:
        for r in rows:
            f.write('%.4f %r %r %r %r %r %r\n' % tuple(float(x) for x in r))


# Phase-matrix elements of the polarised walk (read_phase_matrix_elements,
# monte_carlo3D.py:145-171, :267-475): P11.dat, P12.dat, P22.dat, P33.dat,
# P43.dat, P44.dat beside isca.dat.  First line: the scattering angles [deg];
# then one line per isca.dat row with the element at those angles; P12 ... P44
# are stored divided by P11.
PHASE_ELEMENTS = ('P11', 'P12', 'P22', 'P33', 'P43', 'P44')


def read_phase_matrix(particle_dir, rows):
    """The six elements for isca.dat rows `rows` (indices into the file's rows, in
    the order given): returns (theta_deg[6][n_angle], P[6][len(rows)][n_angle]) with
    P12 ... P44 multiplied back by P11, as :418-475 do."""
    thetas, els = [], []
    for name in PHASE_ELEMENTS:
        with open(os.path.join(particle_dir, name + '.dat')) as f:
            head = f.readline().split()
            lines = f.readlines()
        thetas.append(np.array([float(t) for t in head], dtype=np.float64))
        els.append(np.array([[float(v) for v in lines[r].split()[:len(head)]] for r in rows],
                            dtype=np.float64).reshape(len(rows), len(head)))
    p11 = els[0]
    return thetas, [p11] + [e * p11 for e in els[1:]]


def synthetic_phase_rows(isca_rows, theta_deg):
    """Synthetic phase matrices for isca.dat rows (tests and fixtures): P11 a
    Henyey-Greenstein function with the row's asymmetry parameter; P12/P11 =
    -0.3 sin^2/(1 + cos^2); P22/P11 = 0.9 + 0.1 cos; P33/P11 = 0.8 cos + 0.1;
    P43/P11 = 0.05 sin (1 - cos); P44/P11 = 0.85 cos + 0.1.  Returns the six
    element arrays [n_rows][n_angle] as stored (P12 ... P44 divided by P11)."""
    th = np.deg2rad(np.asarray(theta_deg, dtype=np.float64))
    c, s = np.cos(th), np.sin(th)
    p11 = []
    for r in isca_rows:
        g = float(r[6])
        p11.append((1 - g * g) / (1 + g * g - 2 * g * c) ** 1.5)
    p11 = np.array(p11)
    n = p11.shape[0]
    ratios = [-0.3 * s * s / (1 + c * c), 0.9 + 0.1 * c, 0.8 * c + 0.1, 0.05 * s * (1 - c),
              0.85 * c + 0.1]
    return [p11] + [np.tile(q, (n, 1)) for q in ratios]


def write_phase_matrix(particle_dir, theta_deg, elements):
    """Write P11.dat ... P44.dat (element arrays as synthetic_phase_rows returns)."""
    os.makedirs(particle_dir, exist_ok=True)
    for name, e in zip(PHASE_ELEMENTS, elements):
        with open(os.path.join(particle_dir, name + '.dat'), 'w') as f:
            f.write(' '.join('%r' % float(t) for t in theta_deg) + '\n')
            for row in e:
                f.write(' '.join('%r' % float(v) for v in row) + '\n')


@dataclass
class PhaseTable:
    """Phase matrices of the polarised walk for the rows of an aspherical SSP table
    (same order), as interpolate_phase_matrix (monte_carlo3D.py:819-883) prepares
    them: element e (P11, P12, P22, P33, P43, P44) at cos_asc[e] = cos of the file's
    angles, ascending, with values p_asc[e][row, j] (P12 ... P44 multiplied by P11);
    the two areas of the rejection sampler split at cos_cutoff, and each row's
    maxima of |P11| (a1, a2) and |P12| (b1, b2) over them (:929-947)."""
    cos_asc: list
    p_asc: list
    cos_max: float
    cos_min: float
    cos_cutoff: float
    cutoff_idx: int
    a1: np.ndarray
    a2: np.ndarray
    b1: np.ndarray
    b2: np.ndarray


def phase_table(thetas_deg, elements, row_wvl_um, wvl0):
    """Build a PhaseTable from the six elements' angle grids [deg] and values
    [n_rows][n_angle] (P12 ... P44 already multiplied by P11; rows in the order of
    the SSP table whose wavelengths are row_wvl_um).  The area split comes from
    P11 at wvl0, with the reference's arithmetic (:850-883).  (The reference takes
    the last drawn wavelength instead when no photon drew wvl0, which a run of more
    than a handful of photons never meets.)"""
    cos_desc = [np.cos((np.asarray(t, dtype=np.float64) * np.pi) / 180.) for t in thetas_deg]
    rows0 = np.where(np.asarray(row_wvl_um) == wvl0)[0]
    if rows0.size == 0:
        raise ValueError('wvl0 = %r um is not a row of the table' % (wvl0,))
    P11 = elements[0][rows0[0]]
    c11 = cos_desc[0]
    cos_max, cos_min = c11[0], c11[-1]
    pct = []
    n = len(c11)
    for i, ct in enumerate(c11):
        if 0 < i < n - 1:
            m1 = P11[:i + 1].max()
            m2 = P11[i:].max()
            a1 = (cos_max - ct) * m1
            a2 = (ct - cos_min) * m2
            pct.append(a1 / (a1 + a2))
        else:
            pct.append(1e5)
    cut = int(np.argsort(np.absolute(0.5 - np.array(pct)))[0])
    p11, p12 = elements[0], elements[1]
    return PhaseTable(
        cos_asc=[np.ascontiguousarray(c[::-1]) for c in cos_desc],
        p_asc=[np.ascontiguousarray(np.asarray(e, dtype=np.float64)[:, ::-1]) for e in elements],
        cos_max=float(cos_max), cos_min=float(cos_min), cos_cutoff=float(c11[cut]), cutoff_idx=cut,
        a1=np.absolute(p11[:, :cut + 1]).max(axis=1), a2=np.absolute(p11[:, cut:]).max(axis=1),
        b1=np.absolute(p12[:, :cut + 1]).max(axis=1), b2=np.absolute(p12[:, cut:]).max(axis=1))


def aspherical_phase_table(isca_file, table, wvl0):
    """The PhaseTable of an aspherical SSP table made by aspherical_table from
    isca_file: P11.dat ... P44.dat of the same directory, rows of the selected size."""
    thetas, els = read_phase_matrix(os.path.dirname(isca_file), table.source_rows)
    return phase_table(thetas, els, table.wvl, wvl0)
