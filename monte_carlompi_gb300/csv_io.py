"""Per-photon CSV output in the reference's on-disk format.

Naming follows MonteCarlo.setup_output (monte_carlo3D.py:96-143):
``<output_dir>/sphere/<wvl0>_<half_width>_<rds_snw>_<n_photon>_<theta0deg>_HG.txt``
with ``_<i>`` appended until the name is free.  Rows are formatted by the
native writer (mcw_write_csv).  ``read_csv`` parses the files back
(post_processing.py:38 reads them whitespace-delimited).
"""
import ctypes
import os

import numpy as np

from . import _abi

HEADER = 'condition wvn[um^-1] theta_n phi_n n_scat path_length[m], snow_depth[m]\n'
COLUMNS = ['condition', 'wvn', 'theta_n', 'phi_n', 'n_scat', 'path_length', 'snow_depth']


def output_path(output_dir, wvl0, half_width, rds_snw, n_photon, theta0_deg, make_dirs=True,
                subdir=('sphere',), appendix='HG'):
    """Free output file name, as setup_output builds it (monte_carlo3D.py:96-143):
    under output_dir/sphere, or output_dir/<shape dir>/<roughness dir> for an
    aspherical run, with rds_snw the effective radius of the particles walked;
    appendix 'HG', or 'I%d%d%d%d' of the incident Stokes vector for the polarised
    walk (:125-130)."""
    save_dir = os.path.join(output_dir, *subdir)
    if make_dirs:
        os.makedirs(save_dir, exist_ok=True)
    stem = '%s_%s_%s_%s_%s_%s' % (wvl0, half_width, rds_snw, n_photon, theta0_deg, appendix)
    path = os.path.join(save_dir, stem + '.txt')
    i = 0
    while os.path.isfile(path):
        i += 1
        path = os.path.join(save_dir, '%s_%d.txt' % (stem, i))
    return path


def theta0_label(theta_0_deg):
    """theta0 as the reference prints it: degrees -> radians -> degrees (np.rad2deg)."""
    return np.rad2deg((np.pi * theta_0_deg) / 180.)


def _mode_of(records):
    if records.dtype == _abi.RECORD32:
        return _abi.MODE_F32
    if records.dtype == _abi.RECORD64:
        return _abi.MODE_REPLAY64
    if records.dtype == _abi.RECORD64P:
        return _abi.MODE_POL64
    if records.dtype == _abi.RECORD32P:
        return _abi.MODE_POL32
    raise TypeError('records must be RECORD32, RECORD64, RECORD32P or RECORD64P structured arrays')


def write_csv(path, records, n_threads=0):
    """Write records with the native formatter (header + one row per photon)."""
    rec = np.ascontiguousarray(records)
    rc = _abi.load().mcw_write_csv(os.fsencode(path), rec.ctypes.data, _mode_of(rec), rec.size,
                                   int(n_threads))
    _abi.check(rc, what='mcw_write_csv(%s) failed' % path)
    return path


def format_csv(records, header=True):
    """CSV text of records (native formatter), as bytes."""
    rec = np.ascontiguousarray(records)
    used = ctypes.c_size_t()
    L = _abi.load()
    _abi.check(L.mcw_format_csv(rec.ctypes.data, _mode_of(rec), rec.size, int(header), None, 0,
                                ctypes.byref(used)), what='mcw_format_csv size')
    buf = ctypes.create_string_buffer(used.value + 1)
    _abi.check(L.mcw_format_csv(rec.ctypes.data, _mode_of(rec), rec.size, int(header), buf,
                                used.value + 1, ctypes.byref(used)), what='mcw_format_csv')
    return buf.raw[:used.value]


def read_csv(path):
    """Parse a per-photon CSV into a dict of numpy columns."""
    with open(path) as f:
        head = f.readline()
        if head.split()[:2] != ['condition', 'wvn[um^-1]']:
            raise ValueError('%s: not a monte_carlo3D CSV' % path)
        ncol = 10 if head.rstrip('\n').endswith('V_n') else 7
        data = np.loadtxt(f, ndmin=2) if os.path.getsize(path) > len(head) else np.zeros((0, ncol))
    out = {name: data[:, i] for i, name in enumerate(COLUMNS)}
    if ncol == 10:   # the polarised walk's Q_n, U_n, V_n (monte_carlo3D.py:1637-1646)
        out['stokes_q'], out['stokes_u'], out['stokes_v'] = data[:, 7], data[:, 8], data[:, 9]
    out['condition'] = out['condition'].astype(np.int32)
    out['n_scat'] = out['n_scat'].astype(np.int64)
    return out
