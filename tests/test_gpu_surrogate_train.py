"""Surrogate end to end on the GPU: data from the walk, training on the tensor-core
kernels, what the network gains over plain Monte Carlo, and the Gauss-Newton inverse."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from monte_carlompi_gb300 import inverse, surrogate  # noqa: E402


@pytest.fixture(scope='module')
def trained(walker):
    ds = surrogate.make_dataset(walker, 1536, 50000, seed=101)
    hold = 96
    train = surrogate.Dataset(ds.x[hold:], ds.y[hold:], ds.raw[hold:], ds.brf[hold:], ds.albedo[hold:],
                              ds.photons)
    ens = surrogate.train(train, members=3, epochs=150, batch=256, lr=1e-3, seed=1)
    return ens, ds, hold


def test_network_beats_the_monte_carlo_it_learned_from(walker, trained):
    """Gain over the method without it: on held-out configs the network, trained on
    5e4-photon walks, is closer to a 2e6-photon walk than a 5e4-photon walk is, and it
    answers in microseconds instead of milliseconds."""
    ens, ds, hold = trained
    judge, _ = surrogate.mc_brf(walker, ds.raw[:hold], 2000000, seed=202)
    pred, _, _ = ens.predict(ds.raw[:hold])
    err_net = surrogate.rel_rms(pred, judge)
    err_mc = surrogate.rel_rms(ds.brf[:hold], judge)
    assert np.median(err_net) < 0.8 * np.median(err_mc), (np.median(err_net), np.median(err_mc))
    assert np.median(err_net) < 0.06
    assert surrogate.inference_rate(ens, batch=16384, reps=5) > 1e6


def test_jacobian_matches_finite_differences(trained):
    ens, ds, _ = trained
    known = ds.raw[:16, 1:]
    s = np.log(ds.raw[:16, 0])
    f, jac = inverse._brf_and_jacobian(ens, s, known)
    h = 1e-2
    fp, _, _ = ens.predict(np.column_stack([np.exp(s + h), known]))
    fm, _, _ = ens.predict(np.column_stack([np.exp(s - h), known]))
    fd = (fp - fm) / (2 * h)
    f0, _, _ = ens.predict(np.column_stack([np.exp(s), known]))
    assert np.max(np.abs(f - f0)) < 1e-3 * np.max(np.abs(f0))
    w = surrogate.bin_weights()
    rel = np.sqrt(((jac - fd) ** 2 * w).sum(1) / ((fd ** 2 * w).sum(1) + 1e-30))
    assert np.median(rel) < 0.05, np.median(rel)


def test_gauss_newton_recovers_r_eff_on_network_brfs(trained):
    ens, ds, _ = trained
    rng = np.random.default_rng(7)
    raw = surrogate.sample_inputs(64, 303)
    raw[:, 1] = rng.uniform(1.4, 1.8, 64)          # absorbing wavelengths: r_eff is well constrained
    obs, _, _ = ens.predict(raw)
    s, _, _ = inverse.surrogate_gn(ens, obs, raw[:, 1:])
    err = np.abs(np.exp(s) / raw[:, 0] - 1)
    assert np.median(err) < 0.01, np.median(err)
    assert np.all(np.isfinite(s)) and np.all(s >= math.log(50) - 1e-9)
