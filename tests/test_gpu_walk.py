"""Parity of the CUDA walk with the oracle and the reference (GPU, through the C ABI).

* FP64 replay: per-photon condition and n_scat bit-exact, float fields within
  1e-12 relative, against the reference's golden runs and the C oracle.
* FP32 production walk: condition fractions within 4 sigma (two-sample
  binomial) and a two-sample chi-square of the 18 x 36 exit histogram
  (p > 1e-4) against the oracle at the same N.
"""
import dataclasses

import numpy as np
import pytest

from monte_carlompi_gb300 import _abi, replicas, ssp
from monte_carlompi_gb300.config import WalkConfig
from oracle import oracle
from tests.conftest import golden_names, load_golden
from tests.helpers import (FULL_RUN_ANGLE_ATOL, FULL_RUN_ANGLE_FRAC, chi2_two_sample, compare_replay,
                           condition_fractions_agree, exit_histogram, golden_config, golden_mode,
                           golden_phase, golden_tables)

pytestmark = pytest.mark.gpu


def cfg2_geometry(n, depth=0.10, rds=250.0):
    lo, hi = ssp.grid_for(1.55, 0.085)
    ice = ssp.synthetic_ice_table(rds, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = depth * ssp.ext_cff_mss_sphere(rds) * 300.0
    cfg = WalkConfig(n_photon=n, wvl0=1.55, half_width=0.085, theta0_deg=60.0, tau_tot=tau,
                     lambertian_reflectance=0.5)
    return cfg, ice, imp


def oracle_run(cfg, ice, imp, seed, threads=16):
    c = oracle.make_config(cfg.n_photon, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot,
                           cfg.imp_cnc, cfg.rho_snw, cfg.rho_ice, cfg.lambertian_surface,
                           cfg.lambertian_bottom, cfg.lambertian_reflectance,
                           ssa_ice_override=cfg.ssa_ice_override, g_override=cfg.g_override,
                           nearest=cfg.ssp_nearest)
    return oracle.walk(c, ice, imp, seed, p0=cfg.first_photon,
                       p1=cfg.first_photon + cfg.n_photon, threads=threads if cfg.first_photon == 0 else 1)


# ---------------------------------------------------------------- FP64 replay

@pytest.mark.parametrize('name', golden_names())
def test_replay_matches_reference(walker, name):
    g = load_golden(name)
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    if golden_phase(g) is not None:
        walker.set_phase_matrices([golden_phase(g)])
    res = walker.walk([golden_config(g)], int(g['param_seed']), mode=golden_mode(g))
    compare_replay(res.records, g)
    assert not np.any(res.records['flags'])
    if 'stokes' in g:   # the polarised walk's Q_n, U_n, V_n
        got = np.stack([res.records['stokes_q'], res.records['stokes_u'], res.records['stokes_v']], 1)
        err = np.abs(got - g['stokes'][:, 1:]).max()
        assert err < 1e-10, err


@pytest.mark.parametrize('n', [100000])
def test_pol32_statistics_match_oracle(walker, n):
    """FP32 polarised walk against the oracle's FP64 walk of the reference's algorithm
    at the same N: condition fractions (4 sigma), exit histogram (chi-square), mean
    n_scat and the mean final Stokes Q, U, V of the photons leaving the top (4 sigma)."""
    g = load_golden('pol')
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    walker.set_phase_matrices([golden_phase(g)])
    cfg = dataclasses.replace(golden_config(g), n_photon=n)
    rec = walker.walk([cfg], 31, mode='pol32').records
    from oracle import oracle as orc
    c = orc.make_config(n, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot, cfg.imp_cnc,
                        cfg.rho_snw, cfg.rho_ice, cfg.lambertian_surface, cfg.lambertian_bottom,
                        cfg.lambertian_reflectance, nearest=True, phase=orc.phase_from_golden(g))
    ref = orc.walk(c, ice, imp, 4321, threads=16)
    condition_fractions_agree(rec['condition'], ref['condition'])
    top_g, top_r = rec['condition'] == 1, ref['condition'] == 1
    x2, dof, p = chi2_two_sample(exit_histogram(rec['theta_n'][top_g], rec['phi_n'][top_g]),
                                 exit_histogram(ref['theta_n'][top_r], ref['phi_n'][top_r]))
    assert p > 1e-4, (x2, dof, p)
    for a, b in ((rec['n_scat'].astype(np.float64), ref['n_scat'].astype(np.float64)),
                 (rec['stokes_q'][top_g].astype(np.float64), ref['stokes'][top_r, 1]),
                 (rec['stokes_u'][top_g].astype(np.float64), ref['stokes'][top_r, 2]),
                 (rec['stokes_v'][top_g].astype(np.float64), ref['stokes'][top_r, 3])):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se + 1e-7, (a.mean(), b.mean(), se)
    # records depend only on (seed, photon): a second launch gives the same photons
    again = walker.walk([dataclasses.replace(cfg, n_photon=5000)], 31, mode='pol32').records
    assert np.array_equal(again, rec[:5000])


POL_VARIANTS = {
    # a Lambertian surface: the phase-matrix update at Lambertian angles (:1238-1342)
    'lamsurf': dict(lambertian_surface=True, lambertian_reflectance=0.7),
    # impurities: the species draw and condition 5
    'imp': dict(imp_cnc=2e-4),
    # no bottom reflection: conditions 2 and 3 from a thin slab
    'nobottom': dict(lambertian_bottom=False, tau_tot=3.0),
}


@pytest.mark.parametrize('variant', sorted(POL_VARIANTS))
def test_polarised_variants_match_oracle(walker, variant):
    """Branches of the polarised walk the golden run does not reach: the FP64 replay
    equals the oracle photon by photon (condition, n_scat bit-exact; Stokes within
    1e-10), and the FP32 walk agrees with the oracle statistically."""
    g = load_golden('pol')
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    walker.set_phase_matrices([golden_phase(g)])
    from oracle import oracle as orc
    cfg = dataclasses.replace(golden_config(g), n_photon=4000, **POL_VARIANTS[variant])
    c = orc.make_config(cfg.n_photon, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot,
                        cfg.imp_cnc, cfg.rho_snw, cfg.rho_ice, cfg.lambertian_surface,
                        cfg.lambertian_bottom, cfg.lambertian_reflectance, nearest=True,
                        phase=orc.phase_from_golden(g))
    ref = orc.walk(c, ice, imp, 77, threads=16)
    got = walker.walk([cfg], 77, mode='pol64').records
    compare_replay(got, ref)
    st = np.stack([got['stokes_q'], got['stokes_u'], got['stokes_v']], 1)
    assert np.abs(st - ref['stokes'][:, 1:]).max() < 1e-10
    big = dataclasses.replace(cfg, n_photon=100000)
    rec = walker.walk([big], 5, mode='pol32').records
    c.n_photon = big.n_photon
    ref = orc.walk(c, ice, imp, 55, threads=16)
    condition_fractions_agree(rec['condition'], ref['condition'])
    for a, b in ((rec['n_scat'].astype(np.float64), ref['n_scat'].astype(np.float64)),
                 (rec['stokes_q'].astype(np.float64), ref['stokes'][:, 1]),
                 (rec['stokes_u'].astype(np.float64), ref['stokes'][:, 2])):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se + 1e-7, (variant, a.mean(), b.mean(), se)
    if variant == 'imp':
        assert np.any(rec['condition'] == 5) and np.any(ref['condition'] == 5)
    if variant == 'nobottom':
        assert np.any(rec['condition'] == 2)


def test_polarised_walk_with_separate_element_grids(walker):
    """P33 tabulated on a grid of its own (every other angle): the walks look it up on
    that grid; FP64 replay equals the oracle photon by photon, FP32 agrees statistically."""
    from monte_carlompi_gb300 import ssp as S
    from oracle import oracle as orc
    g = load_golden('pol')
    ice, imp = golden_tables(g)
    pt = golden_phase(g)
    theta = g['phase_theta']
    keep = np.r_[np.arange(0, theta.size - 1, 2), theta.size - 1]      # keeps 0 and 180 deg
    rows = [e[:, ::-1] for e in pt.p_asc]                               # back to descending cos
    els = rows[:3] + [rows[3][:, keep]] + rows[4:]
    thetas = [theta] * 3 + [theta[keep]] + [theta] * 2
    pt2 = S.phase_table(thetas, els, ice.wvl, g['param_wvl0'].item())
    assert pt2.cos_asc[3].size == keep.size
    walker.set_tables([ice], imp)
    walker.set_phase_matrices([pt2])
    cfg = dataclasses.replace(golden_config(g), n_photon=3000)
    c = orc.make_config(cfg.n_photon, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot,
                        cfg.imp_cnc, cfg.rho_snw, cfg.rho_ice, cfg.lambertian_surface,
                        cfg.lambertian_bottom, cfg.lambertian_reflectance, nearest=True,
                        phase=orc.make_phase(pt2, g['stokes0']))
    ref = orc.walk(c, ice, imp, 8, threads=16)
    got = walker.walk([cfg], 8, mode='pol64').records
    compare_replay(got, ref)
    st = np.stack([got['stokes_q'], got['stokes_u'], got['stokes_v']], 1)
    assert np.abs(st - ref['stokes'][:, 1:]).max() < 1e-10
    big = dataclasses.replace(cfg, n_photon=100000)
    rec = walker.walk([big], 6, mode='pol32').records
    c.n_photon = big.n_photon
    ref = orc.walk(c, ice, imp, 66, threads=16)
    condition_fractions_agree(rec['condition'], ref['condition'])
    for a, b in ((rec['stokes_q'].astype(np.float64), ref['stokes'][:, 1]),
                 (rec['stokes_u'].astype(np.float64), ref['stokes'][:, 2])):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se + 1e-7


def test_polarised_walk_needs_its_mode_and_tables(walker):
    """Polarised configs walk in 'pol64' only, with phase matrices attached to their
    ice table; set_tables drops the matrices of the previous tables."""
    g = load_golden('pol')
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    cfg = golden_config(g)
    with pytest.raises(_abi.McwError):
        walker.walk([cfg], 1, mode='pol64')           # no phase matrices yet
    walker.set_phase_matrices([golden_phase(g)])
    with pytest.raises(_abi.McwError):
        walker.walk([cfg], 1, mode='replay64')
    with pytest.raises(_abi.McwError):
        walker.walk([cfg], 1, mode='f32')
    with pytest.raises(_abi.McwError):
        walker.walk([dataclasses.replace(cfg, polarised=False)], 1, mode='pol64')
    r = walker.walk([cfg], 1, mode='pol64')
    assert r.records.dtype == _abi.RECORD64P and r.records.size == cfg.n_photon
    walker.set_tables([ice], imp)
    with pytest.raises(_abi.McwError):
        walker.walk([cfg], 1, mode='pol64')


def test_replay_config2_full_run_matches_oracle_and_reference(walker):
    """Config 2 at its full size (monte_carlo3D.py:1212-1490 for 1,000,000 photons):
    every photon of the FP64 replay walk equals the oracle's (condition and n_scat
    bit-exact, float fields within 1e-12), and the last 1,000 photons equal the
    reference's own run of them (photons 999,000 .. 999,999 of the same stream)."""
    g = load_golden('cfg2_tail')
    ice, imp = golden_tables(g)
    cfg = dataclasses.replace(golden_config(g), first_photon=0, n_photon=1000000)
    walker.set_tables([ice], imp)
    res = walker.walk([cfg], int(g['param_seed']), mode='replay64')
    ref = oracle_run(cfg, ice, imp, int(g['param_seed']))
    err = compare_replay(res.records, ref, angle_atol=FULL_RUN_ANGLE_ATOL)
    assert err['path_length'] < 1e-12
    assert err['direction_frac_over'] <= FULL_RUN_ANGLE_FRAC, err
    compare_replay(res.records[999000:], g)
    # the FP64 walk reaches the bottom: the full run exercises conditions 1, 2 and 4
    assert set(np.unique(res.records['condition'])) >= {1, 4}


def test_replay_shard_equals_slice(walker):
    g = load_golden('thin')
    ice, imp = golden_tables(g)
    walker.set_tables([ice], imp)
    whole = walker.walk([golden_config(g)], 11, mode='replay64').records
    part = dataclasses.replace(golden_config(g), first_photon=500, n_photon=700)
    got = walker.walk([part], 11, mode='replay64').records
    compare_replay(got, whole[500:1200])


# ---------------------------------------------------------------- FP32 statistics

STAT_CASES = {
    # name: (config builder, N)
    'cfg2': (lambda: cfg2_geometry(0), 200000),
    'thin': (lambda: cfg2_geometry(0, depth=0.02, rds=1500.0), 200000),
    # normal incidence on the thin slab: every photon starts exactly on the vertical
    # (the pole branch) and near-vertical directions are common
    'thin0': (lambda: tuple([dataclasses.replace(cfg2_geometry(0, depth=0.02, rds=1500.0)[0], theta0_deg=0.0)])
              + cfg2_geometry(0, depth=0.02, rds=1500.0)[1:], 1000000),
}


def _golden_case(name, n):
    g = load_golden(name)
    ice, imp = golden_tables(g)
    return dataclasses.replace(golden_config(g), n_photon=n), ice, imp


@pytest.mark.parametrize('case,n', [('cfg2', 1000000), ('thin', 1000000), ('thin0', 1000000), ('kat', 200000),
                                    ('imp', 100000), ('lamsurf', 50000), ('edge', 50000),
                                    ('cfg1', 10000), ('cfg1', 40000), ('asph', 100000)])
def test_f32_statistics_match_oracle(walker, case, n):
    """The FP32 walk against the oracle's FP64 walk of the reference algorithm at the
    same N: config 2 and its thin-slab variant at the 1,000,000 photons the bench walks,
    config 1 at its 10,000 (and at 40,000 for more power)."""
    if case in STAT_CASES:
        cfg, ice, imp = STAT_CASES[case][0]()
        cfg = dataclasses.replace(cfg, n_photon=n)
    else:
        cfg, ice, imp = _golden_case(case, n)
    walker.set_tables([ice], imp)
    res = walker.walk([cfg], 1234, mode='f32')
    ref = oracle_run(cfg, ice, imp, 98765)
    rec = res.records
    condition_fractions_agree(rec['condition'], ref['condition'])
    top_g, top_r = rec['condition'] == 1, ref['condition'] == 1
    h_g = exit_histogram(rec['theta_n'][top_g], rec['phi_n'][top_g])
    h_r = exit_histogram(ref['theta_n'][top_r], ref['phi_n'][top_r])
    x2, dof, p = chi2_two_sample(h_g, h_r)
    assert p > 1e-4, (x2, dof, p)
    # mean scatter count and path length within 4 sigma (+ 1e-6 of the slab depth:
    # on a Lambertian surface the exact path is 0 and FP32 leaves rounding residue)
    depth = float(ref['snow_depth'].mean())
    for k in ('n_scat', 'path_length'):
        a = rec[k].astype(np.float64)
        b = ref[k].astype(np.float64)
        sd = np.sqrt(a.var() / a.size + b.var() / b.size)
        floor = 1e-6 * max(abs(b.mean()), depth if k == 'path_length' else 0.0)
        assert abs(a.mean() - b.mean()) <= 4 * sd + floor, (k, a.mean(), b.mean())


def test_f32_known_answer_slab(walker):
    cfg, ice, imp = _golden_case('kat', 1000000)
    walker.set_tables([ice], imp)
    res = walker.walk([cfg], 2024, mode='f32', records=None)
    t = res.tallies[0]
    n = int(t['n_cond'][1:].sum())
    assert n == 1000000
    albedo = res.albedo()[0]
    trans = (int(t['n_cond'][2]) + int(t['n_cond'][3])) / n
    assert abs(albedo - 0.09739) < 4 * np.sqrt(0.09739 * 0.90261 / n)
    assert abs(trans - 0.66096) < 4 * np.sqrt(0.66096 * 0.33904 / n)
    assert abs(int(t['n_cond'][3]) / n - np.exp(-2)) < 4 * np.sqrt(np.exp(-2) / n)


# ---------------------------------------------------------------- FP32 invariants

def test_f32_same_records_for_any_launch_shape(walker):
    """Records and tallies do not depend on the launch shape, nor on which photons end
    their walk in the drain queue (drain_from 0: none; 256: every photon in block mode
    once the supply is exhausted)."""
    cfg, ice, imp = cfg2_geometry(100000)
    walker.set_tables([ice], imp)
    saved = walker.get_launch()
    try:
        walker.set_launch(256, 0, 8, 512)
        a = walker.walk([cfg], 77, mode='f32')
        walker.set_launch(128, 2, 1, 0)
        b = walker.walk([cfg], 77, mode='f32')
        walker.set_launch(64, 1, 32, 256)
        c = walker.walk([cfg], 77, mode='f32')
    finally:
        walker.set_launch(**saved)
    assert np.array_equal(a.records, b.records) and np.array_equal(a.records, c.records)
    assert np.array_equal(a.tallies, b.tallies) and np.array_equal(a.tallies, c.tallies)


@pytest.mark.parametrize('case', ['cfg2', 'imp', 'lamsurf'])
def test_f32_records_independent_of_photon_count(walker, case):
    """Photon p's record depends only on (seed, config, p): a 300-photon launch, whose
    warps walk mostly with few active lanes (steps precomputed on the idle lanes), gives
    the first 300 records of a 100,000-photon launch (mostly full warps) bit for bit;
    with impurities (species draw) and a Lambertian surface too."""
    if case == 'cfg2':
        cfg, ice, imp = cfg2_geometry(100000)
    else:
        cfg, ice, imp = _golden_case(case, 100000)
    walker.set_tables([ice], imp)
    big = walker.walk([cfg], 91, mode='f32')
    small = walker.walk([dataclasses.replace(cfg, n_photon=300)], 91, mode='f32')
    assert np.array_equal(small.records, big.records[:300])


@pytest.mark.parametrize('n', [1, 2, 3, 5, 8, 12])
def test_f32_sparse_rounds_same_records(walker, n):
    """A launch of n photons walks them in sparse rounds (32 / n steps of each photon
    per round, drawn across the warp's lanes; n = 12 starts in full rounds): their
    records equal the first n of a 20,000-photon launch bit for bit, with impurities
    (the species draw) too."""
    for case in ('cfg2', 'imp'):
        if case == 'cfg2':
            cfg, ice, imp = cfg2_geometry(20000)
        else:
            cfg, ice, imp = _golden_case(case, 20000)
        walker.set_tables([ice], imp)
        big = walker.walk([cfg], 4242, mode='f32')
        small = walker.walk([dataclasses.replace(cfg, n_photon=n)], 4242, mode='f32')
        assert np.array_equal(small.records, big.records[:n]), case


def test_f32_long_walks_same_records_with_and_without_drain(walker):
    """Weakly absorbing, deep snow (lambda 1.0 um, r_eff 50 um, tau ~1000: walks of
    thousands of steps): the walks that leave for the drain queue, whose block passes a
    thread block computes a warp per chunk, end exactly as they would in the main loop,
    where one warp computes the chunks one after the other."""
    lo, hi = ssp.grid_for(1.0, 0.085)
    ice = ssp.synthetic_ice_table(50.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.1 * ssp.ext_cff_mss_sphere(50.0) * 300.0
    cfg = WalkConfig(n_photon=3000, wvl0=1.0, half_width=0.085, theta0_deg=30.0, tau_tot=tau,
                     lambertian_reflectance=0.5)
    walker.set_tables([ice], imp)
    saved = walker.get_launch()
    try:
        walker.set_launch(256, 0, 8, 0)
        a = walker.walk([cfg], 5, mode='f32')
        walker.set_launch(256, 0, 8, 256)
        b = walker.walk([cfg], 5, mode='f32')
        walker.set_launch(128, 1, 4, 2048)
        c = walker.walk([cfg], 5, mode='f32')
    finally:
        walker.set_launch(**saved)
    assert int(a.records['n_scat'].max()) > 4096
    assert np.array_equal(a.records, b.records) and np.array_equal(a.tallies, b.tallies)
    assert np.array_equal(a.records, c.records) and np.array_equal(a.tallies, c.tallies)


def test_f32_block_mode_statistics_match_oracle(walker):
    """Deep, weakly absorbing snow (lambda 1.0 um, r_eff 50 um, tau ~980): nearly every
    photon in four walks thousands of steps, all past the first 256 in warp-wide block passes.
    Condition fractions, exit histogram, mean n_scat and mean path length agree with
    the oracle's step-by-step FP64 walk of the reference algorithm."""
    lo, hi = ssp.grid_for(1.0, 0.085)
    ice = ssp.synthetic_ice_table(50.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.1 * ssp.ext_cff_mss_sphere(50.0) * 300.0
    cfg = WalkConfig(n_photon=20000, wvl0=1.0, half_width=0.085, theta0_deg=30.0, tau_tot=tau,
                     lambertian_reflectance=0.5)
    walker.set_tables([ice], imp)
    rec = walker.walk([cfg], 13, mode='f32').records
    ref = oracle_run(cfg, ice, imp, 31)
    assert np.mean(rec["n_scat"] > 256) > 0.2
    condition_fractions_agree(rec['condition'], ref['condition'])
    top_g, top_r = rec['condition'] == 1, ref['condition'] == 1
    x2, dof, p = chi2_two_sample(exit_histogram(rec['theta_n'][top_g], rec['phi_n'][top_g]),
                                 exit_histogram(ref['theta_n'][top_r], ref['phi_n'][top_r]))
    assert p > 1e-4, (x2, dof, p)
    for a, b in ((rec['n_scat'].astype(np.float64), ref['n_scat'].astype(np.float64)),
                 (rec['path_length'].astype(np.float64), ref['path_length'])):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se, (a.mean(), b.mean(), se)


def _very_long_walks(n):
    """Single-scattering albedo 0.9999 over tau 1e4 at normal incidence (r_eff 50 um,
    1.0 um): about 2% of the walks pass 8,192 steps (up to ~5e4), where block passes
    switch to chunks of 32 lanes x 4 steps."""
    lo, hi = ssp.grid_for(1.0, 0.085)
    ice = ssp.synthetic_ice_table(50.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    cfg = WalkConfig(n_photon=n, wvl0=1.0, half_width=0.085, theta0_deg=0.0, tau_tot=1e4,
                     lambertian_reflectance=0.5, ssa_ice_override=0.9999)
    return cfg, ice, imp


def test_f32_very_long_walks_same_records_with_and_without_drain(walker):
    """Walks past 8,192 steps take 4-step block passes in the warp and in the drain
    kernel alike: records and tallies do not depend on where a photon is walked."""
    cfg, ice, imp = _very_long_walks(20000)
    walker.set_tables([ice], imp)
    saved = walker.get_launch()
    try:
        walker.set_launch(256, 0, 8, 0)
        a = walker.walk([cfg], 21, mode='f32')
        walker.set_launch(256, 0, 8, 256)
        b = walker.walk([cfg], 21, mode='f32')
        walker.set_launch(128, 1, 4, 8192)
        c = walker.walk([cfg], 21, mode='f32')
    finally:
        walker.set_launch(**saved)
    assert int((a.records['n_scat'] > 8192).sum()) >= 100
    assert np.array_equal(a.records, b.records) and np.array_equal(a.tallies, b.tallies)
    assert np.array_equal(a.records, c.records) and np.array_equal(a.tallies, c.tallies)


def test_f32_very_long_walks_statistics_match_oracle(walker):
    """The same slab against the oracle's step-by-step FP64 walk of the reference
    algorithm: condition fractions, exit histogram, mean n_scat and path length, and the
    share of walks past 8,192 steps."""
    cfg, ice, imp = _very_long_walks(40000)
    walker.set_tables([ice], imp)
    rec = walker.walk([cfg], 17, mode='f32').records
    ref = oracle_run(cfg, ice, imp, 71)
    condition_fractions_agree(rec['condition'], ref['condition'])
    top_g, top_r = rec['condition'] == 1, ref['condition'] == 1
    x2, dof, p = chi2_two_sample(exit_histogram(rec['theta_n'][top_g], rec['phi_n'][top_g]),
                                 exit_histogram(ref['theta_n'][top_r], ref['phi_n'][top_r]))
    assert p > 1e-4, (x2, dof, p)
    for a, b in ((rec['n_scat'].astype(np.float64), ref['n_scat'].astype(np.float64)),
                 (rec['path_length'].astype(np.float64), ref['path_length'])):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se, (a.mean(), b.mean(), se)
    fa, fb = np.mean(rec['n_scat'] > 8192), np.mean(ref['n_scat'] > 8192)
    assert abs(fa - fb) < 4 * np.sqrt(fb * (1 - fb) * 2 / rec.size) + 1e-9, (fa, fb)


def test_records_into_pinned_host_memory(walker):
    """Pinned host buffers are written by the walk directly (no copy after the kernel);
    their records equal those copied into pageable memory, in both modes."""
    import ctypes
    cfg, ice, imp = cfg2_geometry(10000)
    walker.set_tables([ice], imp)
    lib = _abi.load()
    for mode, dtype in (('f32', _abi.RECORD32), ('replay64', _abi.RECORD64)):
        n = cfg.n_photon
        nbytes = n * dtype.itemsize
        ptr = ctypes.c_void_p()
        _abi.check(lib.mcw_host_alloc(nbytes, ctypes.byref(ptr)), what='host alloc')
        try:
            pinned = np.frombuffer((ctypes.c_char * nbytes).from_address(ptr.value), dtype=dtype, count=n)
            pinned[:] = np.zeros(1, dtype)
            a = walker.walk([cfg], 3, mode=mode, records='host', out=pinned)
            b = walker.walk([cfg], 3, mode=mode)
            assert np.array_equal(pinned, b.records)
            assert np.array_equal(a.tallies, b.tallies)
            assert a.stats['d2h_bytes'] == b.stats['d2h_bytes']
        finally:
            lib.mcw_host_free(ptr)


def test_pinned_host_records_with_drain_and_two_configs(walker):
    """Pinned host records of the FP32 walk, written by the kernels themselves, cover
    every photon: those finished by the drain kernel (weakly absorbing deep snow,
    handover from 256 steps), two configs in config order (20,003 photons), and a cfg2
    run of 100,000 photons; each against the same walk into pageable memory (records
    copied after the kernels), tallies and stats alike."""
    import ctypes
    lo, hi = ssp.grid_for(1.0, 0.085)
    ice = ssp.synthetic_ice_table(50.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.1 * ssp.ext_cff_mss_sphere(50.0) * 300.0
    weak = WalkConfig(n_photon=3000, wvl0=1.0, half_width=0.085, theta0_deg=30.0, tau_tot=tau,
                      lambertian_reflectance=0.5)
    thin = dataclasses.replace(weak, n_photon=17003, tau_tot=4.0, theta0_deg=60.0)
    c2, ice2, imp2 = cfg2_geometry(100000)
    lib = _abi.load()
    saved = walker.get_launch()
    try:
        for cfgs, tables, imp_t, launch in (([weak, thin], ice, imp, (256, 0, 8, 256)),
                                            ([c2], ice2, imp2, (256, 2, 1, 0))):
            walker.set_tables([tables], imp_t)
            walker.set_launch(*launch)
            n = sum(c.n_photon for c in cfgs)
            nbytes = n * _abi.RECORD32.itemsize
            ptr = ctypes.c_void_p()
            _abi.check(lib.mcw_host_alloc(nbytes, ctypes.byref(ptr)), what='host alloc')
            try:
                pinned = np.frombuffer((ctypes.c_char * nbytes).from_address(ptr.value),
                                       dtype=_abi.RECORD32, count=n)
                for seed in (5, 6):
                    pinned[:] = np.zeros(1, _abi.RECORD32)
                    a = walker.walk(cfgs, seed, mode='f32', records='host', out=pinned)
                    b = walker.walk(cfgs, seed, mode='f32')
                    assert np.array_equal(pinned, b.records)
                    assert np.array_equal(a.tallies, b.tallies)
                    assert a.stats['d2h_bytes'] == b.stats['d2h_bytes']
                if launch[3]:
                    assert int(b.records['n_scat'].max()) > 4096   # the drain kernel walked some
            finally:
                lib.mcw_host_free(ptr)
    finally:
        walker.set_launch(**saved)


def test_f32_tallies_agree_with_records(walker):
    cfg, ice, imp = cfg2_geometry(300000, depth=0.02, rds=1500.0)
    walker.set_tables([ice], imp)
    res = walker.walk([cfg], 5, mode='f32')
    rec, t = res.records, res.tallies[0]
    counts = np.bincount(rec['condition'], minlength=6)
    assert np.array_equal(counts[1:], t['n_cond'][1:].astype(np.int64))
    assert int(t['n_events']) == int(rec['n_scat'].astype(np.int64).sum())
    assert int(t['max_n_scat']) == int(rec['n_scat'].max())
    top = rec['condition'] == 1
    th = rec['theta_n'][top].astype(np.float32)
    ph = rec['phi_n'][top].astype(np.float32)
    tb = np.clip((th * np.float32(36.0 / np.pi)).astype(np.int64), 0, 17)
    pb = np.clip((ph * np.float32(18.0 / np.pi)).astype(np.int64), 0, 35)
    hist = np.bincount(tb * 36 + pb, minlength=648)
    assert np.array_equal(hist, t['bin_count'].astype(np.int64))
    q = t['q_cond_fx'].astype(np.float64) / _abi.WVN_FX_SCALE
    for k in range(1, 6):
        s = rec['wvn'][rec['condition'] == k].astype(np.float64).sum()
        assert abs(q[k] - s) <= 1e-6 * max(s, 1.0)
    assert np.all((rec['phi_n'] >= 0) & (rec['phi_n'] < 2 * np.pi))
    assert np.all(rec['theta_n'][top] <= np.pi / 2 + 1e-6)


def test_f32_shards_equal_whole_run(walker):
    cfg, ice, imp = cfg2_geometry(99999)
    walker.set_tables([ice], imp)
    whole = walker.walk([cfg], 31, mode='f32')
    world = 3
    parts, tallies = [], []
    for r in range(world):
        res = walker.walk(replicas.shard_configs([cfg], r, world), 31, mode='f32')
        parts.append(res.records)
        tallies.append(res.tallies)
    merged = replicas.merge_records(parts, [cfg], world)
    keep = [n for n in _abi.RECORD32.names if n != 'config']
    for k in keep:
        assert np.array_equal(merged[k], whole.records[k]), k
    m = replicas.merge_tallies(tallies)
    for k in ('n_cond', 'q_cond_fx', 'n_events', 'bin_count', 'bin_wvn_fx', 'max_n_scat'):
        assert np.array_equal(m[k], whole.tallies[k]), k


def test_batch_first_config_equals_single_run(walker):
    a, ice, imp = cfg2_geometry(50000)
    b = dataclasses.replace(a, theta0_deg=0.0, n_photon=30000)
    c = dataclasses.replace(a, wvl0=1.45, n_photon=0)
    d = dataclasses.replace(a, tau_tot=a.tau_tot / 5, n_photon=40000)
    walker.set_tables([ice], imp)
    batch = walker.walk([a, b, c, d], 9, mode='f32')
    alone = walker.walk([a], 9, mode='f32')
    assert np.array_equal(batch.records[:50000], alone.records)
    assert np.array_equal(batch.records['config'],
                          np.repeat(np.arange(4, dtype=np.uint32), [50000, 30000, 0, 40000]))
    assert int(batch.tallies[2]['n_cond'].sum()) == 0
    for i, cf in ((1, b), (3, d)):
        single = walker.walk([cf], 10 + i, mode='f32')
        lo = 50000 + (30000 if i == 3 else 0)
        condition_fractions_agree(batch.records['condition'][lo:lo + cf.n_photon],
                                  single.records['condition'])


@pytest.mark.parametrize('imp_cnc', [0.0, 2e-6])
@pytest.mark.parametrize('general', ['lambertian_surface', 'isotropic'])
def test_f32_records_independent_of_kernel_instance(walker, imp_cnc, general):
    """The deep-slab kernel instance (a branch on the bottom crossing, no surface or
    isotropic alternatives, dense rounds split into the direction-independent part of
    their steps and the chains) gives the same records and tallies as the general one.
    A deep slab walked alone takes the deep instance; the same slab next to a
    Lambertian-surface config, or next to an isotropically scattering one, takes the
    general instance.  Both species-draw variants (2e-6: ~8% of the photons end on an
    impurity and ~200 walk past the 256 steps of block mode; ~380 without impurities)."""
    a, ice, imp = cfg2_geometry(40000)
    a = dataclasses.replace(a, imp_cnc=imp_cnc)
    other = (dataclasses.replace(a, lambertian_surface=True, n_photon=2000) if general == 'lambertian_surface'
             else dataclasses.replace(a, g_override=0.0, n_photon=2000))
    walker.set_tables([ice], imp)
    alone = walker.walk([a], 17, mode='f32')
    mixed = walker.walk([a, other], 17, mode='f32')
    assert np.array_equal(mixed.records[:a.n_photon], alone.records)
    for k in ('n_cond', 'q_cond_fx', 'n_events', 'bin_count', 'bin_wvn_fx', 'max_n_scat'):
        assert np.array_equal(mixed.tallies[0][k], alone.tallies[0][k]), k
    assert (int(alone.tallies[0]['n_cond'][5]) > 0) == (imp_cnc > 0)
    assert int((alone.records['n_scat'] > 256).sum()) > 50


SWEEP_SAMPLE = [   # (r_eff um, lambda0 um, theta0 deg, depth m): configs of the 64-config sweep's grid
    (100.0, 1.30, 0.0, 0.10), (400.0, 1.60, 45.0, 0.02), (1500.0, 1.10, 60.0, 1.0),
    (50.0, 1.70, 30.0, 0.02), (200.0, 0.95, 0.0, 0.02), (800.0, 1.40, 60.0, 0.10)]


def test_sweep_configs_match_oracle_in_one_graph_launch(walker):
    """Six configs of the batched sweep (each its own grain-size table, wavelength, zenith
    and depth) walked together by one captured graph launch, each against the oracle at
    the same N: condition fractions within 4 sigma, the 648-bin exit histogram
    (two-sample chi-square, p > 1e-4) and mean n_scat within 4 sigma."""
    import torch
    n = 40000
    tables, cfgs = [], []
    for j, (r, wvl, th, depth) in enumerate(SWEEP_SAMPLE):
        tables.append(ssp.synthetic_ice_table(r, 600, 2100))
        cfgs.append(WalkConfig(n_photon=n, wvl0=wvl, half_width=0.085, theta0_deg=th,
                               tau_tot=depth * ssp.ext_cff_mss_sphere(r) * 300.0,
                               lambertian_reflectance=0.5, ice_table=j, rds_snw=r))
    imp = ssp.synthetic_impurity_table(600, 2100)
    walker.set_tables(tables, imp)
    buf = torch.zeros(n * len(cfgs) * _abi.RECORD32.itemsize, dtype=torch.uint8, device='cuda')
    g = walker.graph(cfgs, device_ptr=buf.data_ptr())
    try:
        g.launch(5)
        res = g.launch(6)
    finally:
        g.close()
    torch.cuda.synchronize()
    rec = buf.cpu().numpy().view(_abi.RECORD32)
    for j, cfg in enumerate(cfgs):
        got = rec[j * n:(j + 1) * n]
        assert np.all(got['config'] == j)
        assert int(res.tallies[j]['n_cond'][1:].sum()) == n
        ref = oracle_run(cfg, tables[j], imp, 600 + j)
        condition_fractions_agree(got['condition'], ref['condition'])
        top_g, top_r = got['condition'] == 1, ref['condition'] == 1
        x2, dof, p = chi2_two_sample(exit_histogram(got['theta_n'][top_g], got['phi_n'][top_g]),
                                     exit_histogram(ref['theta_n'][top_r], ref['phi_n'][top_r]))
        assert p > 1e-4, (j, x2, dof, p)
        a, b = got['n_scat'].astype(np.float64), ref['n_scat'].astype(np.float64)
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        assert abs(a.mean() - b.mean()) < 4 * se, (j, a.mean(), b.mean(), se)


def test_graph_replays_equal_walks(walker):
    cfg, ice, imp = cfg2_geometry(200000)
    cfgs = [cfg, dataclasses.replace(cfg, theta0_deg=30.0, n_photon=100000)]
    walker.set_tables([ice], imp)
    g = walker.graph(cfgs)
    try:
        for seed in (3, 4):
            gr = g.launch(seed)
            wr = walker.walk(cfgs, seed, mode='f32', records=None)
            assert np.array_equal(gr.tallies, wr.tallies)
    finally:
        g.close()


def test_device_records(walker):
    torch = pytest.importorskip('torch')
    cfg, ice, imp = cfg2_geometry(50000)
    walker.set_tables([ice], imp)
    host = walker.walk([cfg], 8, mode='f32').records
    buf = torch.empty(50000 * 32, dtype=torch.uint8, device='cuda')
    walker.walk([cfg], 8, mode='f32', records='device', device_ptr=buf.data_ptr())
    torch.cuda.synchronize()
    dev = buf.cpu().numpy().view(_abi.RECORD32)
    assert np.array_equal(dev, host)


def test_autotune_picks_a_valid_shape(walker):
    cfg, ice, imp = cfg2_geometry(50000)
    walker.set_tables([ice], imp)
    saved = walker.get_launch()
    try:
        best = walker.autotune([cfg])
        assert best['block_size'] in (128, 256) and 1 <= best['regen_chunk'] <= 32
        assert best['ms'] > 0
        assert walker.get_launch()['block_size'] == best['block_size']
    finally:
        walker.set_launch(**saved)


# ---------------------------------------------------------------- errors

def test_budget_stops_the_kernel_and_context_survives(walker):
    g = load_golden('cfg1')
    ice, imp = golden_tables(g)
    cfg = dataclasses.replace(golden_config(g), n_photon=200000)
    walker.set_tables([ice], imp)
    walker.set_budget(1e-4)
    try:
        with pytest.raises(_abi.BudgetExceeded):
            walker.walk([cfg], 1, mode='f32', records=None)
        with pytest.raises(_abi.BudgetExceeded):
            walker.walk([dataclasses.replace(cfg, n_photon=2000)], 1, mode='replay64', records=None)
    finally:
        walker.set_budget(_abi.DEFAULT_BUDGET_S)
    ok = walker.walk([dataclasses.replace(cfg, n_photon=1000)], 1, mode='f32')
    assert int(ok.tallies[0]['n_cond'][1:].sum()) == 1000


@pytest.mark.parametrize('launch', [(512, 0, 8, 0), (48, 0, 8, 0), (256, -1, 8, 0), (256, 0, 0, 0),
                                    (256, 0, 33, 0), (256, 0, 8, 100), (256, 0, 8, -1)])
def test_invalid_launch_shapes_are_refused(walker, launch):
    saved = walker.get_launch()
    with pytest.raises(_abi.McwError, match='MCW_ERR_ARG'):
        walker.set_launch(*launch)
    assert walker.get_launch() == saved


def test_budget_stops_the_drain_kernel_too(walker):
    """Deep, weakly absorbing snow with every photon past 256 steps handed to the drain
    kernel: a 0.1 ms budget stops the walk and the drain kernel (which checks it every 64
    block passes), the call raises, and the next walk is complete."""
    lo, hi = ssp.grid_for(1.0, 0.085)
    ice = ssp.synthetic_ice_table(50.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.1 * ssp.ext_cff_mss_sphere(50.0) * 300.0
    cfg = WalkConfig(n_photon=20000, wvl0=1.0, half_width=0.085, theta0_deg=30.0, tau_tot=tau,
                     lambertian_reflectance=0.5)
    walker.set_tables([ice], imp)
    saved = walker.get_launch()
    walker.set_launch(256, 0, 8, 256)
    walker.set_budget(1e-4)
    try:
        with pytest.raises(_abi.BudgetExceeded):
            walker.walk([cfg], 2, mode='f32', records=None)
    finally:
        walker.set_budget(_abi.DEFAULT_BUDGET_S)
    try:
        ok = walker.walk([dataclasses.replace(cfg, n_photon=2000)], 2, mode='f32')
    finally:
        walker.set_launch(**saved)
    assert int(ok.tallies[0]['n_cond'][1:].sum()) == 2000


@pytest.mark.parametrize('bad', [dict(n_photon=-1), dict(wvl0=0.0), dict(half_width=-0.1),
                                 dict(theta0_deg=90.0), dict(tau_tot=0.0), dict(imp_cnc=1.5),
                                 dict(lambertian_reflectance=1.5), dict(ice_table=3),
                                 dict(g_override=1.0), dict(first_photon=-2),
                                 dict(rho_snw=float('nan'))])
def test_invalid_config_rejected(walker, bad):
    cfg, ice, imp = cfg2_geometry(10)
    walker.set_tables([ice], imp)
    with pytest.raises(_abi.McwError) as e:
        walker.walk([dataclasses.replace(cfg, **bad)], 1)
    assert e.value.code == -1


def test_walk_without_tables_is_a_state_error():
    from monte_carlompi_gb300.walker import Walker
    with Walker(0) as w:
        cfg, _, _ = cfg2_geometry(10)
        with pytest.raises(_abi.McwError) as e:
            w.walk([cfg], 1)
        assert e.value.code == -6


def test_empty_run(walker):
    cfg, ice, imp = cfg2_geometry(0)
    walker.set_tables([ice], imp)
    res = walker.walk([cfg], 1)
    assert res.records.size == 0 and int(res.tallies[0]['n_cond'].sum()) == 0
