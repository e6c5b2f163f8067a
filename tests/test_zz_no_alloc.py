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


def test_noalloc_rejects_oversized_grid():
    torch = pytest.importorskip('torch')
    from monte_carlompi_gb300 import _abi, ssp
    from monte_carlompi_gb300.config import WalkConfig
    lo, hi = ssp.grid_for(1.55, 0.085)
    keep = []
    ice_c = _device_table(torch, ssp.synthetic_ice_table(250.0, lo, hi), keep)
    imp_c = _device_table(torch, ssp.synthetic_impurity_table(lo, hi), keep)
    # FWHM 5 um spans about 2,760 grid points of 0.01 um, more than the scratch holds
    wide = WalkConfig(n_photon=10, wvl0=8.0, half_width=5.0, tau_tot=10.0).to_c()
    rc = _abi.load().mcw_walk_noalloc(ctypes.byref(wide), ctypes.byref(ice_c), ctypes.byref(imp_c),
                                      1, None, None, None)
    assert rc == -1
