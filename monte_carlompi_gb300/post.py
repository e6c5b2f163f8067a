"""BRF and albedo from per-photon records, on the device (mcw_post).

Restates the arithmetic of the reference's post_processing.py for records
already produced by the walk (no CSV round trip):

* ``calculate_bins`` - number of zenith bins of a photodiode of active area
  ``active_area`` [mm] in a dome of diameter ``d_dome`` [mm] (post_processing.py:
  435-444; defaults 1 mm and 175 mm give 137 bins);
* ``zenith_brf`` - Q_down = sum(wvn), the wvn-weighted histogram of theta_n over
  condition-1 photons on [0, pi/2] (np.histogram binning), bin midpoints, the
  sin * cos weights normalised to one and BRF = h / (Q_down * w)
  (post_processing.py:73-81); albedo = Q_up / Q_down (:125-128,
  monte_carlo3D.py:1659-1671); the albedo counting transmitted photons as not
  absorbed and the mean wavelength of spectral_albedo (:261-275); mean n_scat
  and mean path length (:418-430).
"""
import ctypes

import numpy as np

from . import _abi


def calculate_bins(active_area=1.0, d_dome=175.0):
    """int(pi * d_dome / (4 * active_area)) (post_processing.py:435-444)."""
    return int((np.pi * d_dome) / (4. * active_area))


def zenith_brf(walker, records, n_bins=None, n_cfg=None):
    """Per-config 1-D BRF and albedo statistics of a record array (RECORD32, RECORD64 or
    the polarised RECORD32P / RECORD64P, host numpy array) using the device kernel of
    ``walker``'s context."""
    rec = np.ascontiguousarray(records)
    modes = {_abi.RECORD32: _abi.MODE_F32, _abi.RECORD64: _abi.MODE_REPLAY64,
             _abi.RECORD32P: _abi.MODE_POL32, _abi.RECORD64P: _abi.MODE_POL64}
    if rec.dtype not in modes:
        raise TypeError('records must be RECORD32, RECORD64, RECORD32P or RECORD64P')
    mode = modes[rec.dtype]
    if n_bins is None:
        n_bins = calculate_bins()
    if n_cfg is None:
        n_cfg = int(rec['config'].max()) + 1 if rec.size else 1
    bins = np.zeros((n_cfg, n_bins), np.uint64)
    cnt = np.zeros((n_cfg, n_bins), np.uint32)
    stats = np.zeros(n_cfg, _abi.POST_STATS)
    rc = _abi.load().mcw_post(walker.handle, rec.ctypes.data, _abi.RECORDS_HOST, mode, rec.size, n_cfg,
                              n_bins, bins.ctypes.data, cnt.ctypes.data, stats.ctypes.data)
    _abi.check(rc, walker.handle)
    return summarize(bins, cnt, stats)


def summarize(bins_fx, counts, stats):
    n_bins = bins_fx.shape[1]
    edges = np.linspace(0., np.pi / 2, n_bins + 1)
    midpoints = (np.diff(edges) / 2.) + edges[:-1]
    w = np.sin(midpoints) * np.cos(midpoints) / np.sum(np.sin(midpoints) * np.cos(midpoints))
    q = stats['q_cond_fx'].astype(np.float64) / _abi.WVN_FX_SCALE
    n = stats['n_cond'].astype(np.float64)
    q_down = q[:, 1:].sum(1)
    h = bins_fx.astype(np.float64) / _abi.WVN_FX_SCALE
    with np.errstate(invalid='ignore', divide='ignore'):
        brf = h / (q_down[:, None] * w[None, :])
        total = n[:, 1:].sum(1)
        out = dict(midpoints=midpoints, theta_deg=np.rad2deg(midpoints), brf=brf, hist=h, counts=counts,
                   q_down=q_down, albedo=q[:, 1] / q_down,
                   albedo_non_absorbed=(q[:, 1] + q[:, 2] + q[:, 3]) / q_down,
                   mean_wavelength=stats['sum_wavelength'] / total,
                   mean_n_scat=stats['sum_n_scat'].astype(np.float64) / total,
                   mean_path_length=stats['sum_path_length'] / total, n_cond=n)
    return out
