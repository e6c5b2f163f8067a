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


def test_jacobian_matches_cpu_autograd(trained):
    """d BRF / d log r_eff from the batched autograd pass through the kernels equals
    float64 CPU autograd of the same network (bf16 roundings included)."""
    from tests.helpers import reference_mlp
    ens, ds, _ = trained
    one = surrogate.Ensemble(ens.members[:1])
    m = ens.members[0]
    known = ds.raw[:8, 1:]
    s = np.log(ds.raw[:8, 0])
    f, jac = inverse._brf_and_jacobian(one, s, known)
    params = [p.detach().cpu().double() for p in m.params]
    y_mean, y_std = m.y_mean.cpu().double(), m.y_std.cpu().double()
    lo, hi = inverse.LOG_R

    def brf_of(sv):
        r = torch.exp(sv)
        x = torch.stack([2 * (torch.log(r) - lo) / (hi - lo) - 1,
                         *[torch.from_numpy(surrogate.encode(np.exp(s), known[:, 0], known[:, 1],
                                                             known[:, 2])[:, k]).double()
                           for k in (1, 2, 3)]], dim=1)
        y = reference_mlp(x, params) * y_std + y_mean
        alb = torch.exp(y[:, surrogate.N_BRF])
        return (torch.exp(y[:, :surrogate.N_BRF]) - surrogate.BRF_FLOOR) * alb[:, None]

    sv = torch.from_numpy(s).double().requires_grad_(True)
    ref_f = brf_of(sv)
    ref_j = torch.stack([torch.autograd.grad(ref_f[:, b].sum(), sv, retain_graph=True)[0]
                         for b in range(surrogate.N_BRF)], dim=1).numpy()
    w = surrogate.bin_weights()
    assert np.max(np.abs(f - ref_f.detach().numpy())) < 2e-2 * np.max(np.abs(f))
    rel = np.sqrt(((jac - ref_j) ** 2 * w).sum(1) / ((ref_j ** 2 * w).sum(1) + 1e-30))
    assert np.median(rel) < 0.03, np.median(rel)


def test_gauss_newton_recovers_r_eff_on_network_brfs(trained):
    ens, ds, _ = trained
    rng = np.random.default_rng(7)
    raw = surrogate.sample_inputs(64, 303)
    raw[:, 1] = rng.uniform(1.4, 1.8, 64)          # absorbing wavelengths: r_eff is well constrained
    obs, _, _ = ens.predict(raw)
    s, _, spread, spread_r = inverse.surrogate_gn(ens, obs, raw[:, 1:])
    err = np.abs(np.exp(s) / raw[:, 0] - 1)
    assert np.median(err) < 0.01, np.median(err)
    assert np.all(np.isfinite(s)) and np.all(s >= math.log(50) - 1e-9)
    assert np.all(np.isfinite(spread)) and np.all(np.isfinite(spread_r)) and np.all(spread_r >= 0)
