"""Comparison helpers shared by the parity tests."""
import numpy as np

from monte_carlompi_gb300 import ssp
from monte_carlompi_gb300.config import WalkConfig

FLOAT_RTOL = 1e-12   # FP64 replay: float fields, relative
ANGLE_ATOL = 1e-12   # FP64 replay: direction cosines rebuilt from theta_n / phi_n
# Runs of 1e6 photons: the reference's rotation divides by sqrt(1 - mu_z^2), so a
# one-ulp difference between two libms (CUDA's and glibc's sin, cos, log) grows by
# 1 / sin(theta) at directions near the vertical, and among ~4e7 rotations a few come
# close enough to carry it past 1e-12.  The oracle against its own one-ulp stand-in
# (oracle.walk(..., ulp=True)) measures 4.3e-12 at most on config 2's 1e6 photons, 6
# above 1e-12 (tests/test_oracle.py); the full runs are held to FULL_RUN_ANGLE_ATOL for
# every photon and to ANGLE_ATOL for all but FULL_RUN_ANGLE_FRAC of them.
FULL_RUN_ANGLE_ATOL = 1e-11
FULL_RUN_ANGLE_FRAC = 1e-4


def compare_replay(got, ref, skip_phi_undefined=True, angle_atol=ANGLE_ATOL):
    """Replay parity: condition and n_scat bit-exact; wvn, path_length and
    snow_depth within FLOAT_RTOL (path_length relative to max(|path|, depth));
    angles compared through the direction they
    encode (cos theta, sin theta cos phi, sin theta sin phi), because arccos
    and the quadrant arctan are ill-conditioned near the poles and axes, within
    angle_atol; err['direction_frac_over'] is the fraction of photons whose
    direction differs by more than ANGLE_ATOL.
    Returns a dict of maximum errors; raises AssertionError on failure."""
    assert np.array_equal(np.asarray(got['condition']), np.asarray(ref['condition']))
    assert np.array_equal(np.asarray(got['n_scat']), np.asarray(ref['n_scat']))
    err = {}
    depth = np.abs(np.asarray(ref['snow_depth'], np.float64))
    for k in ('wvn', 'path_length', 'snow_depth'):
        a = np.asarray(got[k], np.float64)
        b = np.asarray(ref[k], np.float64)
        # path_length: the exit correction cancels the last step, so a path that is
        # exactly 0 (Lambertian surface) carries rounding residue of the step length;
        # it is compared relative to max(|path|, slab depth)
        scale = np.maximum(np.abs(b), depth) if k == 'path_length' else np.abs(b)
        e = np.abs(a - b) / np.maximum(scale, 1e-300)
        err[k] = float(e.max()) if e.size else 0.0
        assert err[k] <= FLOAT_RTOL, (k, err[k])
    th_a, th_b = np.asarray(got['theta_n'], np.float64), np.asarray(ref['theta_n'], np.float64)
    ph_a, ph_b = np.asarray(got['phi_n'], np.float64), np.asarray(ref['phi_n'], np.float64)
    ok = np.isfinite(ph_a) & np.isfinite(ph_b)
    da = np.stack([np.cos(th_a), np.sin(th_a) * np.cos(ph_a), np.sin(th_a) * np.sin(ph_a)])
    db = np.stack([np.cos(th_b), np.sin(th_b) * np.cos(ph_b), np.sin(th_b) * np.sin(ph_b)])
    e = np.abs(da - db)[:, ok]
    err['direction'] = float(e.max()) if e.size else 0.0
    err['direction_frac_over'] = float(np.mean(e.max(0) > ANGLE_ATOL)) if e.size else 0.0
    assert err['direction'] <= angle_atol, err
    return err


def golden_config(g):
    p = lambda k: g['param_' + k].item()  # noqa: E731
    return WalkConfig(n_photon=int(p('n_photon')), wvl0=p('wvl0'), half_width=p('half_width'),
                      first_photon=int(p('first_photon')) if 'param_first_photon' in g else 0,
                      theta0_deg=p('theta0'), tau_tot=p('tau_tot'), imp_cnc=p('imp_cnc'),
                      rho_snw=p('rho_snw'), rho_ice=p('rho_ice'),
                      lambertian_reflectance=p('R'), lambertian_surface=bool(p('lam_surface')),
                      lambertian_bottom=bool(p('lam_bottom')),
                      ssa_ice_override=p('ssa_ice_override'), g_override=p('g_override'),
                      ssp_nearest=bool(p('ssp_nearest')) if 'param_ssp_nearest' in g else False,
                      polarised='param_polarised' in g,
                      stokes0=tuple(float(x) for x in g['stokes0']) if 'stokes0' in g else (1.0, 0.0, 0.0, 0.0))


def golden_phase(g):
    """Phase matrices of a polarised golden fixture (None for the others)."""
    if 'param_polarised' not in g:
        return None
    from oracle import oracle
    return oracle.ssp_phase_from_golden(g)


def golden_mode(g):
    return 'pol64' if 'param_polarised' in g else 'replay64'


def golden_tables(g):
    unit = int(g['ice_unit'].item()) if 'ice_unit' in g else ssp.WVL_METRES
    ice = ssp.SSPTable(g['ice_wvl'], g['ice_ssa'], g['ice_ext'], g['ice_asm'], wvl_unit=unit)
    imp = ssp.SSPTable(g['imp_wvl'], g['imp_ssa'], g['imp_ext'], None)
    return ice, imp


def condition_fractions_agree(c1, c2, n_sigma=4.0):
    """Two-sample binomial test of the fraction of each end condition."""
    n1, n2 = len(c1), len(c2)
    out = {}
    for k in range(1, 6):
        p1, p2 = np.mean(c1 == k), np.mean(c2 == k)
        p = (p1 * n1 + p2 * n2) / (n1 + n2)
        sd = np.sqrt(max(p * (1 - p), 1e-300) * (1.0 / n1 + 1.0 / n2))
        z = abs(p1 - p2) / sd if sd > 0 else 0.0
        out[k] = (p1, p2, z)
        assert z <= n_sigma, (k, p1, p2, z)
    return out


def exit_histogram(theta, phi, weights=None):
    """18 x 36 (theta, phi) histogram of condition-1 exits, 5 x 10 degree bins."""
    t = np.clip((np.asarray(theta, np.float64) * (36.0 / np.pi)).astype(np.int64), 0, 17)
    p = np.clip((np.asarray(phi, np.float64) * (18.0 / np.pi)).astype(np.int64), 0, 35)
    return np.bincount(t * 36 + p, weights=weights, minlength=648)


def chi2_two_sample(a, b):
    """Two-sample chi-square of two count histograms (equal totals not required).
    Returns (chi2, dof, p-value)."""
    from scipy.stats import chi2
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = (a + b) > 0
    a, b = a[m], b[m]
    ka, kb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    x2 = float(np.sum((ka * a - kb * b) ** 2 / (a + b)))
    dof = int(m.sum()) - 1
    return x2, dof, float(chi2.sf(x2, dof))


def reference_mlp(x, params):
    """float64 CPU copy of the surrogate network with the kernels' bf16 roundings of
    weights, input and activations (rounded in the forward pass, identity in the
    backward pass, as the kernels differentiate)."""
    import torch

    def st(v):
        return v + (v.to(torch.bfloat16).double() - v).detach()

    h = st(x)
    ws, bs = params[0::2], params[1::2]
    for layer in range(4):
        z = h @ st(ws[layer]).T + bs[layer]
        h = st(z * torch.sigmoid(z)) if layer < 3 else z
    return h
