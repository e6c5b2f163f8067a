"""Grain-size retrieval: batched Gauss-Newton on log r_eff through the BRF surrogate.

Given observed 648-bin BRFs with known wavelength, incident zenith and depth,
find r_eff.  Each iteration evaluates the ensemble and the Jacobian
d BRF / d log r_eff in forward mode through the surrogate's tensor-core kernels
(`surrogate.forward_tangent`: the input is one scalar, so one tangent pass replaces a
backward pass per output bin).  Retrievals whose ensemble spread at the solution
exceeds ``spread_tol`` fall back to plain Monte Carlo: the same Gauss-Newton
iteration with BRFs and central-difference Jacobians from the GPU walk.  The spread
is either that of the members' BRFs (criterion 'brf': weighted RMS of their standard
deviation over the weighted RMS BRF) or that of the retrieved quantity (criterion
'r_eff': each member's BRF, taken through the Gauss-Newton normal equation at the
solution, gives the log r_eff that member would move the answer to; their standard
deviation is the surrogate's own relative uncertainty in r_eff).  The reference has no inverse; this consumes the same BRF definition
(post_processing.py:73-81, 2-D form).
"""
import math
import time

import numpy as np

from . import surrogate as S

LOG_R = (math.log(S.R_RANGE[0]), math.log(S.R_RANGE[1]))


def noise_variance(f, photons, rel_noise=0.0, model_var=None):
    """Per-bin variance of a BRF about the model value f [n, 648]: the counting noise of
    a walk of `photons` photons (the bin holds photons * w_b * BRF_b of them, w_b its
    expected share, so Var BRF_b = BRF_b / (photons * w_b)), relative Gaussian noise
    rel_noise, and the model's own per-bin variance when given."""
    wt = S.bin_weights()[None, :]
    v = np.maximum(f, 1e-3) / (photons * wt) + (rel_noise * f) ** 2
    return v + model_var if model_var is not None else v


def _brf_and_jacobian(ens, s, known, chunk=65536, with_var=False):
    """Ensemble-mean BRF [n, 648] and d BRF / d log r [n, 648] at log r = s: one
    forward-mode pass per member through the tensor-core kernels (the tangent of the
    first input, d x0 / d log r = 2 / (log r_max - log r_min)), then the chain rule
    through the target standardisation, exp and the albedo factor.  with_var: also the
    variance of the members' BRFs per bin."""
    import torch
    n = s.shape[0]
    f_out = np.zeros((n, S.N_BRF))
    j_out = np.zeros((n, S.N_BRF))
    v_out = np.zeros((n, S.N_BRF))
    dxds = 2.0 / (LOG_R[1] - LOG_R[0])
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        x = torch.from_numpy(S.encode(np.exp(s[lo:hi]), known[lo:hi, 0], known[lo:hi, 1],
                                      known[lo:hi, 2])).cuda()
        xdot = torch.zeros_like(x)
        xdot[:, 0] = dxds
        x16, xdot16 = S._cast(torch, x), S._cast(torch, xdot)
        f_acc = torch.zeros((hi - lo, S.N_BRF), dtype=torch.float64, device='cuda')
        j_acc = torch.zeros_like(f_acc)
        f2_acc = torch.zeros_like(f_acc)
        for m in ens.members:
            y, ydot = S.forward_tangent(torch, x16, xdot16, m.w16, m.params[1::2])
            yp = y.double() * m.y_std + m.y_mean                  # log(BRF / albedo + floor), log(albedo)
            dp = ydot.double() * m.y_std
            alb = torch.exp(yp[:, S.N_BRF])
            shape = torch.exp(yp[:, :S.N_BRF])
            fm = (shape - S.BRF_FLOOR) * alb[:, None]
            f_acc += fm
            f2_acc += fm * fm
            j_acc += shape * dp[:, :S.N_BRF] * alb[:, None] + (shape - S.BRF_FLOOR) * (alb * dp[:, S.N_BRF])[:, None]
        k = len(ens.members)
        f_out[lo:hi] = (f_acc / k).cpu().numpy()
        j_out[lo:hi] = (j_acc / k).cpu().numpy()
        v_out[lo:hi] = torch.clamp(f2_acc / k - (f_acc / k) ** 2, min=0).cpu().numpy()
    return (f_out, j_out, v_out) if with_var else (f_out, j_out)


def _gn_update(f, jac, obs, s, w, damping=1e-3, max_step=0.7):
    r = f - obs
    jtr = (w * jac * r).sum(1)
    jtj = (w * jac * jac).sum(1)
    step = -jtr / (jtj * (1 + damping) + 1e-30)
    step = np.clip(step, -max_step, max_step)
    return np.clip(s + step, LOG_R[0], LOG_R[1])


def logr_spread(f_members, jac, w):
    """Standard deviation over the members of the log r_eff shift that takes the
    ensemble-mean BRF to each member's BRF, linearised at the solution:
    ds_m = sum_b w_b J_b (f_mb - mean_b) / sum_b w_b J_b^2.  f_members [M, n, bins],
    jac [n, bins] (d BRF / d log r), w [1, bins] or [bins]."""
    dev = f_members - f_members.mean(0, keepdims=True)
    ds = (w * jac * dev).sum(2) / np.maximum((w * jac * jac).sum(1), 1e-300)
    return ds.std(0)


def surrogate_gn(ens, obs, known, iters=6, obs_photons=None, obs_noise=0.0, with_noise=False):
    """Gauss-Newton on s = log r_eff through the surrogate; starts from the best of a
    16-point grid.  With obs_photons, every bin's residual is weighted by the inverse of
    its variance (noise_variance: the observation's counting noise for obs_photons
    photons and its relative noise obs_noise, plus the ensemble's variance in that bin);
    without, by the bin's photon share.  Returns (s, brf at s, BRF spread at s, log r_eff
    spread at s) and, with with_noise, the posterior width of s from the observation
    noise alone, 1 / sqrt(sum_b J_b^2 / var_b)."""
    n = obs.shape[0]
    share = S.bin_weights()[None, :]
    w0 = 1.0 / noise_variance(obs, obs_photons, obs_noise) if obs_photons else share
    grid = np.linspace(LOG_R[0], LOG_R[1], 16)
    best = np.full(n, np.inf)
    s = np.zeros(n)
    for g in grid:
        pred, _, _ = ens.predict(np.column_stack([np.full(n, math.exp(g)), known]))
        cost = (w0 * (pred - obs) ** 2).sum(1)
        better = cost < best
        best[better] = cost[better]
        s[better] = g
    for _ in range(iters):
        f, jac, var = _brf_and_jacobian(ens, s, known, with_var=True)
        w = 1.0 / noise_variance(f, obs_photons, obs_noise, var) if obs_photons else share
        s = _gn_update(f, jac, obs, s, w)
    pred, _, spread = ens.predict(np.column_stack([np.exp(s), known]))
    f, jac, var = _brf_and_jacobian(ens, s, known, with_var=True)
    members, _ = ens.predict_members(np.column_stack([np.exp(s), known]))
    w = 1.0 / noise_variance(f, obs_photons, obs_noise, var) if obs_photons else share
    spread_r = logr_spread(members, jac, w)
    if not with_noise:
        return s, pred, spread, spread_r
    wn = 1.0 / noise_variance(f, obs_photons, obs_noise) if obs_photons else share
    sigma = 1.0 / np.sqrt(np.maximum((wn * jac * jac).sum(1), 1e-300))
    return s, pred, spread, spread_r, sigma


def mc_gn(walker, obs, known, s0, n_photon=1000000, iters=3, h=0.05, seed=0x5EED0055, obs_photons=None,
          obs_noise=0.0):
    """Gauss-Newton on log r_eff with BRFs and central-difference Jacobians from the walk.
    With obs_photons the residuals are weighted by the inverse variance of the
    observation (noise_variance) plus the walk's own counting noise at n_photon."""
    share = S.bin_weights()[None, :]
    s = np.array(s0, dtype=np.float64)
    evals = 0
    for it in range(iters):
        rows = np.concatenate([np.column_stack([np.exp(s + d), known]) for d in (0.0, h, -h)])
        brf, _ = S.mc_brf(walker, rows, n_photon, seed + 1000 * it)
        evals += rows.shape[0]
        n = s.shape[0]
        f, fp, fm = brf[:n], brf[n:2 * n], brf[2 * n:]
        if obs_photons:
            w = 1.0 / (noise_variance(f, obs_photons, obs_noise) + noise_variance(f, n_photon))
        else:
            w = share
        s = _gn_update(f, (fp - fm) / (2 * h), obs, s, w)
    return s, evals


def mc_correct(ens, walker, obs, known, s0, iters=2, n_photon=1000000, seed=0x5EED0066, obs_photons=None,
               obs_noise=0.0):
    """Gauss-Newton on log r_eff whose residuals come from the walk and whose Jacobian
    comes from the surrogate: s <- s - sum w J (f_MC(s) - obs) / sum w J^2, J = d BRF /
    d log r of the ensemble at s.  One walk per retrieval and iteration (plain Monte
    Carlo Gauss-Newton needs three, for its central differences, and a grid search
    before); the answer converges to the Monte Carlo solution as fast as the network's
    Jacobian is close to the walk's (error times |1 - J_MC / J| per iteration), and the
    network's systematic BRF error drops out of the residual.  Returns (s, walks)."""
    share = S.bin_weights()[None, :]
    s = np.array(s0, dtype=np.float64)
    n = s.shape[0]
    evals = 0
    for it in range(iters):
        f, _ = S.mc_brf(walker, np.column_stack([np.exp(s), known]), n_photon, seed + 1000 * it)
        evals += n
        _, jac = _brf_and_jacobian(ens, s, known)
        if obs_photons:
            w = 1.0 / (noise_variance(f, obs_photons, obs_noise) + noise_variance(f, n_photon))
        else:
            w = share
        s = _gn_update(f, jac, obs, s, w)
    return s, evals


def mc_retrieve(walker, obs, known, grid=16, iters=4, n_photon=1000000, seed=0x5EED0077, obs_photons=None,
                obs_noise=0.0):
    """The same retrieval with plain Monte Carlo only: the 16-point log r_eff grid and the
    Gauss-Newton iterations evaluated by the walk, weighted as mc_gn.  Returns (s, BRF
    evaluations)."""
    n = obs.shape[0]
    w = 1.0 / noise_variance(obs, obs_photons, obs_noise) if obs_photons else S.bin_weights()[None, :]
    g = np.linspace(LOG_R[0], LOG_R[1], grid)
    rows = np.concatenate([np.column_stack([np.full(n, math.exp(v)), known]) for v in g])
    brf, _ = S.mc_brf(walker, rows, n_photon, seed)
    cost = np.stack([(w * (brf[k * n:(k + 1) * n] - obs) ** 2).sum(1) for k in range(grid)])
    s0 = g[np.argmin(cost, axis=0)]
    s, evals = mc_gn(walker, obs, known, s0, n_photon=n_photon, iters=iters, seed=seed + 1,
                     obs_photons=obs_photons, obs_noise=obs_noise)
    return s, evals + rows.shape[0]


def retrieve(ens, walker, obs, known, spread_tol=0.02, mc_photons=1000000, criterion='brf', obs_photons=None,
             obs_noise=0.0, kappa=1.0, fallback='gn', correct_iters=2):
    """Surrogate retrieval with Monte Carlo fallback.  Criterion 'brf': the ensemble
    spread of the BRF exceeds spread_tol; 'r_eff': the ensemble spread of the retrieved
    log r_eff exceeds spread_tol; 'posterior': the ensemble spread of log r_eff exceeds
    kappa times the posterior width the observation noise alone allows (the network's
    own uncertainty would dominate the error; needs obs_photons).  The fallback of a
    flagged retrieval: 'correct' (mc_correct: correct_iters walks at the surrogate's
    answer, the surrogate's Jacobian) or 'gn' (mc_gn: Monte Carlo Gauss-Newton with
    central differences).  With obs_photons the residuals of both paths are weighted by
    their inverse noise variance.  Returns dict of results and timings."""
    if criterion not in ('brf', 'r_eff', 'posterior'):
        raise ValueError("criterion must be 'brf', 'r_eff' or 'posterior'")
    if criterion == 'posterior' and not obs_photons:
        raise ValueError("the 'posterior' criterion needs obs_photons")
    if fallback not in ('gn', 'correct'):
        raise ValueError("fallback must be 'gn' or 'correct'")
    t0 = time.perf_counter()
    s, _, spread, spread_r, sigma = surrogate_gn(ens, obs, known, obs_photons=obs_photons, obs_noise=obs_noise,
                                                 with_noise=True)
    t_net = time.perf_counter() - t0
    if criterion == 'brf':
        flagged = spread > spread_tol
    elif criterion == 'r_eff':
        flagged = spread_r > spread_tol
    else:
        flagged = spread_r > kappa * sigma
    t0 = time.perf_counter()
    mc_evals = 0
    if np.any(flagged):
        if fallback == 'correct':
            s_mc, mc_evals = mc_correct(ens, walker, obs[flagged], known[flagged], s[flagged], iters=correct_iters,
                                        n_photon=mc_photons, obs_photons=obs_photons, obs_noise=obs_noise)
        else:
            s_mc, mc_evals = mc_gn(walker, obs[flagged], known[flagged], s[flagged], n_photon=mc_photons,
                                   obs_photons=obs_photons, obs_noise=obs_noise)
        s = s.copy()
        s[flagged] = s_mc
    t_mc = time.perf_counter() - t0
    return dict(r_eff=np.exp(s), flagged=flagged, spread=spread, spread_r_eff=spread_r, sigma_noise=sigma,
                seconds_net=t_net, seconds_mc=t_mc, mc_brf_evals=mc_evals, criterion=criterion, fallback=fallback)
