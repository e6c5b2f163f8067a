"""Post-processing on the device against the reference's own numpy arithmetic
(post_processing.py:73-81 brf; np.histogram binning)."""
import dataclasses

import numpy as np
import pytest

from monte_carlompi_gb300 import _abi, post, ssp
from monte_carlompi_gb300.config import WalkConfig
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def reference_brf(wvn, theta, cond, n_bins):
    """post_processing.py:73-81, as the reference computes it."""
    q_down = wvn.sum()
    h = np.histogram(theta[cond == 1], bins=n_bins, range=(0., np.pi / 2), weights=wvn[cond == 1])
    counts = np.histogram(theta[cond == 1], bins=n_bins, range=(0., np.pi / 2))[0]
    midpoints = (np.diff(h[1]) / 2.) + h[1][:-1]
    w = np.sin(midpoints) * np.cos(midpoints) / np.sum(np.sin(midpoints) * np.cos(midpoints))
    return h[0] / (q_down * w), counts, wvn[cond == 1].sum() / q_down, midpoints


def _check(out, rec, n_bins, c=0):
    wvn = rec['wvn'].astype(np.float64)
    theta = rec['theta_n'].astype(np.float64)
    cond = rec['condition']
    brf, counts, albedo, mids = reference_brf(wvn, theta, cond, n_bins)
    assert np.array_equal(out['counts'][c], counts)
    assert np.allclose(out['brf'][c], brf, rtol=1e-9, atol=0)
    assert abs(out['albedo'][c] - albedo) < 1e-9 * albedo
    assert np.array_equal(out['midpoints'], mids)
    q = wvn.sum()
    assert abs(out['albedo_non_absorbed'][c] - wvn[np.isin(cond, (1, 2, 3))].sum() / q) < 1e-9
    assert abs(out['mean_wavelength'][c] - np.mean(1 / wvn)) < 1e-9
    assert abs(out['mean_n_scat'][c] - rec['n_scat'].mean()) < 1e-9
    assert abs(out['mean_path_length'][c] - rec['path_length'].astype(np.float64).mean()) < 1e-6 * abs(
        rec['path_length'].mean()) + 1e-12


@pytest.mark.parametrize('n_bins', [137, 90])
def test_golden_records_match_numpy(walker, n_bins):
    g = load_golden('cfg2')
    rec = np.zeros(g['condition'].size, _abi.RECORD64)
    for k in ('condition', 'n_scat', 'wvn', 'theta_n', 'phi_n', 'path_length', 'snow_depth'):
        rec[k] = g[k]
    out = post.zenith_brf(walker, rec, n_bins)
    _check(out, rec, n_bins)


def test_polarised_records_match_numpy(walker):
    """The polarised walks' records (their leading columns are the HG records') go
    through the same post-processing, FP64 and FP32."""
    from tests.helpers import golden_config, golden_phase, golden_tables
    g = load_golden('pol')
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    walker.set_phase_matrices([golden_phase(g)])
    for mode in ('pol64', 'pol32'):
        cfg = dataclasses.replace(golden_config(g), n_photon=20000)
        rec = walker.walk([cfg], 9, mode=mode).records
        out = post.zenith_brf(walker, rec, 137)
        _check(out, rec, 137)


def test_walk_records_match_numpy(walker):
    lo, hi = ssp.grid_for(1.55, 0.085)
    walker.set_tables([ssp.synthetic_ice_table(250.0, lo, hi)], ssp.synthetic_impurity_table(lo, hi))
    cfg = WalkConfig(n_photon=200000, wvl0=1.55, half_width=0.085, theta0_deg=60.0,
                     tau_tot=0.02 * ssp.ext_cff_mss_sphere(250.0) * 300.0, lambertian_reflectance=0.5)
    cfg2 = dataclasses.replace(cfg, theta0_deg=0.0, n_photon=50000)
    rec = walker.walk([cfg, cfg2], 3).records
    out = post.zenith_brf(walker, rec, 137)
    _check(out, rec[:200000], 137, c=0)
    _check(out, rec[200000:], 137, c=1)
    assert post.calculate_bins() == 137


def test_bin_edges_follow_numpy():
    """Values on and next to the bin edges land where np.histogram puts them."""
    import torch  # noqa: F401  (GPU context already up via the fixture in other tests)
    from monte_carlompi_gb300.walker import Walker
    n_bins = 90
    edges = np.linspace(0., np.pi / 2, n_bins + 1)
    theta = np.concatenate([edges, np.nextafter(edges, 0), np.nextafter(edges, 4)])
    theta = theta[(theta >= 0) & (theta <= np.pi / 2)]
    rec = np.zeros(theta.size, _abi.RECORD64)
    rec['condition'] = 1
    rec['wvn'] = 0.8
    rec['theta_n'] = theta
    with Walker(0) as w:
        out = post.zenith_brf(w, rec, n_bins)
    ref = np.histogram(theta, bins=n_bins, range=(0., np.pi / 2))[0]
    assert np.array_equal(out['counts'][0], ref)
