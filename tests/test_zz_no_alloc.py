"""mcw_walk_noalloc: the walk for callers that cannot allocate device memory.

Such callers (a plugin whose host framework owns all device memory, a loop that
must not touch the allocator once running) hand the library their own device
buffers; the entry point keeps its scratch in a fixed device array of the
library.  This test gives it device buffers made here, calls it twice in a row
through the C ABI, and checks each call against mcw_walk with the same config
and seed: the records and tallies must be identical, so the second call also
shows that the shared scratch is reset between calls.  It sits in its own file,
collected last, and passes alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_table(torch, t, keep):
    from monte_carlompi_gb300 import _abi
    cols = []
    for a in (t.wvl, t.ss_alb, t.ext_cff_mss, t.asm_prm):
        d = torch.from_numpy(np.ascontiguousarray(a, np.float64)).to('cuda')
        keep.append(d)
        cols.append(d.data_ptr())
    return _abi.SSPTableC(cols[0], cols[1], cols[2], cols[3], t.wvl.size, 0)


def test_noalloc_matches_walk_on_two_calls():
    torch = pytest.importorskip('torch')
    from monte_carlompi_gb300 import _abi, ssp
    from monte_carlompi_gb300.config import WalkConfig
    from monte_carlompi_gb300.walker import Walker

    lo, hi = ssp.grid_for(1.55, 0.085)
    ice = ssp.synthetic_ice_table(250.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.10 * ssp.ext_cff_mss_sphere(250.0) * 300.0
    cfg = WalkConfig(n_photon=200000, wvl0=1.55, half_width=0.085, theta0_deg=60.0, tau_tot=tau,
                     lambertian_reflectance=0.5)
    keep = []
    ice_c = _device_table(torch, ice, keep)
    imp_c = _device_table(torch, imp, keep)
    cfg_c = cfg.to_c()
    n = cfg.n_photon
    rec_dev = torch.zeros(n * _abi.RECORD32.itemsize, dtype=torch.uint8, device='cuda')
    tally_dev = torch.full((_abi.TALLY.itemsize,), 7, dtype=torch.uint8, device='cuda')
    lib = _abi.load()
    with Walker(0) as w:
        w.set_tables([ice], imp)
        for seed in (41, 42):
            ref = w.walk([cfg], seed, mode='f32', records='host')
            torch.cuda.synchronize()
            rc = lib.mcw_walk_noalloc(ctypes.byref(cfg_c), ctypes.byref(ice_c), ctypes.byref(imp_c),
                                      seed, rec_dev.data_ptr(), tally_dev.data_ptr(), None)
            assert rc == 0
            got = rec_dev.cpu().numpy().view(_abi.RECORD32)
            tally = tally_dev.cpu().numpy().view(_abi.TALLY)
            assert np.array_equal(got, ref.records)
            assert np.array_equal(tally, ref.tallies)
            assert int(tally[0]['n_cond'][1:].sum()) == n


def _grid_points(wvl0, half_width):
    """Wavelength grid points the entry point needs for a config: lambda = k / 100 um
    over wvl0 +- 6.5 sigma plus one point each side, k >= 1 (the host arithmetic of
    mcw_walk_noalloc)."""
    import math
    sigma = half_width / 2.355
    klo = max(1, math.floor((wvl0 - 6.5 * sigma) * 100.0) - 1)
    khi = max(klo, math.ceil((wvl0 + 6.5 * sigma) * 100.0) + 1)
    return khi - klo + 1


def _half_width_for(points, wvl0=20.0):
    """Smallest FWHM (bisected) whose grid has exactly `points` points."""
    lo, hi = 0.001, 20.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if _grid_points(wvl0, mid) >= points:
            hi = mid
        else:
            lo = mid
    assert _grid_points(wvl0, hi) == points
    return hi


def _small_tables(torch, keep):
    from monte_carlompi_gb300 import ssp
    lo, hi = ssp.grid_for(1.55, 0.085)
    ice = ssp.synthetic_ice_table(250.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    return ice, imp, _device_table(torch, ice, keep), _device_table(torch, imp, keep)


def test_noalloc_grid_limit_is_exact():
    """MCW_NOALLOC_MAX_LUT grid points fit; one more is refused before any kernel runs.
    Wavelengths far outside the tables take their nearest values, so the walk runs."""
    torch = pytest.importorskip('torch')
    from monte_carlompi_gb300 import _abi
    from monte_carlompi_gb300.config import WalkConfig
    keep = []
    _, _, ice_c, imp_c = _small_tables(torch, keep)
    lib = _abi.load()
    limit = _abi.NOALLOC_MAX_LUT
    for points, want in ((limit, 0), (limit + 1, -1)):
        cfg = WalkConfig(n_photon=64, wvl0=20.0, half_width=_half_width_for(points), tau_tot=10.0).to_c()
        rec = torch.zeros(64 * _abi.RECORD32.itemsize, dtype=torch.uint8, device='cuda')
        rc = lib.mcw_walk_noalloc(ctypes.byref(cfg), ctypes.byref(ice_c), ctypes.byref(imp_c),
                                  1, rec.data_ptr(), None, None)
        assert rc == want, (points, rc)
        if want == 0:
            got = rec.cpu().numpy().view(_abi.RECORD32)
            assert set(np.unique(got['condition'])) <= {1, 2, 3, 4}


@pytest.mark.parametrize('fault', ['descending', 'nan_ssa', 'zero_ext'])
def test_noalloc_rejects_bad_device_tables(fault):
    """Tables the device lookups cannot use (wavelengths out of order, a NaN, an ice
    extinction of 0) are found by the set-up kernel and refused with MCW_ERR_ARG before
    the lookup-table and walk kernels run; the next call with good tables walks."""
    torch = pytest.importorskip('torch')
    from monte_carlompi_gb300 import _abi, ssp
    from monte_carlompi_gb300.config import WalkConfig
    lo, hi = ssp.grid_for(1.55, 0.085)
    ice = ssp.synthetic_ice_table(250.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    bad = ssp.SSPTable(ice.wvl.copy(), ice.ss_alb.copy(), ice.ext_cff_mss.copy(), ice.asm_prm.copy())
    if fault == 'descending':
        bad.wvl[[3, 4]] = bad.wvl[[4, 3]]
    elif fault == 'nan_ssa':
        bad.ss_alb[7] = np.nan
    else:
        bad.ext_cff_mss[5] = 0.0
    keep = []
    bad_c = _device_table(torch, bad, keep)
    ice_c = _device_table(torch, ice, keep)
    imp_c = _device_table(torch, imp, keep)
    cfg = WalkConfig(n_photon=1000, wvl0=1.55, half_width=0.085, theta0_deg=60.0, tau_tot=20.0).to_c()
    rec = torch.zeros(1000 * _abi.RECORD32.itemsize, dtype=torch.uint8, device='cuda')
    lib = _abi.load()
    rc = lib.mcw_walk_noalloc(ctypes.byref(cfg), ctypes.byref(bad_c), ctypes.byref(imp_c),
                              1, rec.data_ptr(), None, None)
    assert rc == -1
    torch.cuda.synchronize()
    assert int(rec.count_nonzero()) == 0        # no record written: the walk never started
    rc = lib.mcw_walk_noalloc(ctypes.byref(cfg), ctypes.byref(ice_c), ctypes.byref(imp_c),
                              1, rec.data_ptr(), None, None)
    assert rc == 0
