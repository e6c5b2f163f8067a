"""Host arithmetic of the grain-size retrieval (no GPU): the Gauss-Newton update and
the ensemble spread of the retrieved log r_eff."""
import numpy as np

from monte_carlompi_gb300 import inverse
from monte_carlompi_gb300 import surrogate as S


def test_logr_spread_recovers_member_offsets_of_a_linear_model():
    """Members whose BRFs are a linear model shifted in log r_eff by d_m: the spread of
    the linearised shifts is the standard deviation of the d_m about their mean."""
    rng = np.random.default_rng(3)
    n, bins = 7, S.N_BRF
    w = S.bin_weights()[None, :]
    jac = rng.uniform(0.05, 0.4, (n, bins)) * rng.choice([-1.0, 1.0], (n, 1))
    f0 = rng.uniform(0.2, 0.9, (n, bins))
    d = np.array([-0.03, 0.01, 0.0, 0.02, 0.05])[:, None] * np.linspace(0.5, 1.5, n)[None, :]
    members = f0[None] + d[:, :, None] * jac[None]
    got = inverse.logr_spread(members, jac, w)
    assert np.allclose(got, d.std(0), rtol=1e-12, atol=1e-15)
    # identical members: no spread
    assert np.all(inverse.logr_spread(np.repeat(f0[None], 5, 0), jac, w) == 0)


def test_logr_spread_grows_as_the_brf_loses_sensitivity():
    """The same BRF disagreement means a wider r_eff spread where the BRF depends weakly
    on r_eff (small Jacobian): the criterion flags weakly constrained retrievals."""
    rng = np.random.default_rng(5)
    bins = S.N_BRF
    w = S.bin_weights()[None, :]
    noise = rng.normal(0.0, 0.01, (5, 1, bins))
    base = np.full((1, bins), 0.5)
    strong = inverse.logr_spread(base[None] + noise, np.full((1, bins), 0.5), w)
    weak = inverse.logr_spread(base[None] + noise, np.full((1, bins), 0.05), w)
    assert np.isclose(weak[0], 10 * strong[0])


def test_gauss_newton_update_solves_a_linear_model_in_one_step():
    rng = np.random.default_rng(9)
    n, bins = 4, S.N_BRF
    w = S.bin_weights()[None, :]
    jac = rng.uniform(0.1, 0.3, (n, bins))
    s_true = np.log(np.array([80.0, 200.0, 450.0, 900.0]))
    s0 = s_true + np.array([0.2, -0.3, 0.1, -0.05])
    f0 = rng.uniform(0.2, 0.9, (n, bins))
    obs = f0 + jac * (s_true - s0)[:, None]
    s1 = inverse._gn_update(f0, jac, obs, s0, w, damping=0.0)
    assert np.allclose(s1, s_true, atol=1e-12)
