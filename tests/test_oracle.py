"""The oracle itself: Philox known answers and parity with the reference's golden runs."""
import numpy as np
import pytest

from oracle import oracle, philox
from tests.conftest import golden_names, load_golden
from tests.helpers import (ANGLE_ATOL, FULL_RUN_ANGLE_ATOL, FULL_RUN_ANGLE_FRAC, compare_replay,
                           golden_config, golden_tables)


@pytest.mark.parametrize('ctr,key,expect', philox.KAT_VECTORS)
def test_philox_known_answers(ctr, key, expect):
    got = philox.philox4x32_10(*ctr, *key)
    assert tuple(int(x) for x in got) == expect
    assert tuple(int(x) for x in oracle.philox(ctr, key)) == expect


def test_replay_uniforms_numpy_equals_c():
    seed = 0x1234_5678_9ABC_DEF0
    photons = np.array([0, 1, 7, 2 ** 32 + 5, 2 ** 40 - 1], dtype=np.uint64)
    for tag in (philox.TAG_WALK, philox.TAG_WVL):
        for k in range(7):
            a = philox.replay_uniform(seed, tag, photons, k)
            b = np.array([oracle.lib().orc_uniform(seed, tag, int(p), k) for p in photons])
            assert np.array_equal(a, b)


def test_replay_uniforms_open_interval_and_moments():
    u = philox.replay_uniform(99, philox.TAG_WALK, np.arange(200000, dtype=np.uint64) // 4,
                              np.arange(200000, dtype=np.uint64) % 4)
    assert u.min() > 0 and u.max() < 1
    assert abs(u.mean() - 0.5) < 4 * np.sqrt(1 / 12 / u.size)
    assert abs(np.median(-np.log(u)) - np.log(2)) < 0.01   # monte_carlo3D.py:1016-1017
    # the extreme words map inside (0, 1)
    assert ((0 >> 12) + 0.5) * 2.0 ** -52 > 0
    assert (((2 ** 64 - 1) >> 12) + 0.5) * 2.0 ** -52 < 1


def test_wavelength_matches_numpy_around():
    seed = 0x5EED0001
    n = 5000
    lam = philox.replay_wavelengths(seed, n, 1.3, 0.085)
    c = np.array([oracle.lib().orc_wavelength(seed, p, 1.3, 0.085) for p in range(n)])
    assert np.array_equal(lam, c)
    assert np.allclose(np.round(lam * 100), lam * 100)
    assert abs(lam.mean() - 1.3) < 0.005
    assert abs(lam.std() - 0.085 / 2.355) < 0.003


@pytest.mark.parametrize('name', golden_names())
def test_oracle_matches_reference_golden(name):
    g = load_golden(name)
    cfg = oracle.config_from_golden(g)
    ice, imp = oracle.tables_from_golden(g)
    first = int(g['param_first_photon']) if 'param_first_photon' in g else 0
    r = oracle.walk(cfg, ice, imp, int(g['param_seed']), p0=first, p1=first + cfg.n_photon,
                    threads=4)
    compare_replay(r, g)
    assert np.array_equal(r['n_draws'], g['n_draws'])


def test_goldens_cover_every_end_condition_and_branch():
    seen = set()
    lam = False
    for name in golden_names():
        g = load_golden(name)
        seen |= set(np.unique(g['condition']).tolist())
        lam |= bool(g['param_lam_surface'])
    assert seen == {1, 2, 3, 4, 5}
    assert lam


def test_oracle_known_answer_slab():
    """Wang et al. (1995) / van de Hulst slab: tau 2, ssa 0.9, g 0.75, no bottom
    reflection: albedo 0.09739, total transmittance 0.66096 (monte_carlo3D.py:1849-1866)."""
    g = load_golden('kat')
    cfg = oracle.config_from_golden(g)
    cfg.n_photon = 200000
    ice, imp = oracle.tables_from_golden(g)
    r = oracle.walk(cfg, ice, imp, 777, threads=8)
    n = cfg.n_photon
    c = r['condition']
    alb = r['wvn'][c == 1].sum() / r['wvn'].sum()
    t = np.mean((c == 2) | (c == 3))
    assert abs(alb - 0.09739) < 4 * np.sqrt(0.09739 * (1 - 0.09739) / n)
    assert abs(t - 0.66096) < 4 * np.sqrt(0.66096 * (1 - 0.66096) / n)
    assert abs(np.mean(c == 3) - np.exp(-2.0)) < 4 * np.sqrt(np.exp(-2) / n)


def test_oracle_threads_equal_serial():
    g = load_golden('thin')
    cfg = oracle.config_from_golden(g)
    ice, imp = oracle.tables_from_golden(g)
    a = oracle.walk(cfg, ice, imp, 5)
    b = oracle.walk(cfg, ice, imp, 5, threads=3)
    assert np.array_equal(a, b)


def test_planted_error_is_caught():
    """The parity check fails when the oracle's output is perturbed."""
    g = load_golden('cfg2')
    cfg = oracle.config_from_golden(g)
    ice, imp = oracle.tables_from_golden(g)
    r = oracle.walk(cfg, ice, imp, int(g['param_seed']))
    bad = r.copy()
    bad['path_length'][3] *= 1 + 1e-9
    with pytest.raises(AssertionError):
        compare_replay(bad, g)
    bad = r.copy()
    bad['n_scat'][5] += 1
    with pytest.raises(AssertionError):
        compare_replay(bad, g)


def test_oracle_polarised_stokes_matches_reference():
    """The polarised walk's final Stokes vectors (the CSV's Q_n, U_n, V_n) against the
    reference's own run on the same phase matrices."""
    g = load_golden('pol')
    cfg = oracle.config_from_golden(g)
    ice, imp = oracle.tables_from_golden(g)
    r = oracle.walk(cfg, ice, imp, int(g['param_seed']))
    assert np.array_equal(r['condition'], g['condition'])
    assert np.array_equal(r['n_draws'], g['n_draws'])
    err = np.abs(r['stokes'] - g['stokes']).max()
    assert err < 1e-10, err


def test_one_ulp_libm_difference_sets_the_full_run_tolerance():
    """Config 2's 1e6 photons walked by the oracle and by its one-ulp stand-in for
    another libm (log, sin, cos moved by one ulp, as CUDA's and glibc's may differ):
    conditions and n_scat stay bit-exact and the float fields within 1e-12, while a few
    directions that passed close to the vertical differ by more than 1e-12 (the
    reference's rotation divides by sqrt(1 - mu_z^2)).  The GPU full-run parity test
    holds the CUDA replay walk to the envelope measured here."""
    import dataclasses
    g = load_golden('cfg2_tail')
    ice, imp = golden_tables(g)
    cfg = dataclasses.replace(golden_config(g), first_photon=0, n_photon=1000000)
    c = oracle.make_config(cfg.n_photon, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot, R=0.5)
    seed = int(g['param_seed'])
    a = oracle.walk(c, ice, imp, seed, threads=8)
    b = oracle.walk(c, ice, imp, seed, threads=8, ulp=True)
    err = compare_replay(b, a, angle_atol=FULL_RUN_ANGLE_ATOL)
    assert err['path_length'] < 1e-12
    assert err['direction'] > ANGLE_ATOL                     # 1e-12 cannot hold at this N
    assert err['direction_frac_over'] <= FULL_RUN_ANGLE_FRAC, err
