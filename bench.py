#!/usr/bin/env python
"""Throughput of the photon random walk on GB300 (one JSON line on rank 0).

Workload: 1,000,000 photons per GPU, r_eff 250 um, centre wavelength 1.55 um,
FWHM 0.085 um, incident zenith 60 deg, 0.10 m slab (tau 196.29), Lambertian
bottom R = 0.5, synthetic sphere SSPs, FP32 Philox walk, 18 x 36 exit
histogram, per-photon records.  One step = one walk of those photons
(mcw_walk: SSP lookup table, walk kernel, tallies).

* ``value``: photons/s with the SSP tables and config resident on the device
  and records written to device memory; per-step device time from CUDA
  events on the library's stream; L2 flushed (256 MB write) between steps.
* ``e2e``: the same walk through the public API with host buffers
  (Walker.walk -> mcw_walk, records copied into pinned host memory), host
  wall clock per call.
* ``roofline``: the walk kernel is bound by SM instruction issue (integer
  Philox rounds, FP32 rotation, SFU), not by HBM or tensor cores.
* ``cpu_baseline``: the C oracle (an FP64 port of the reference's walk) on all
  host cores, on a bounded sample of the same workload.

``--impl reference`` times the CPU implementation of the path (the oracle
port; the reference itself is Python and is not present on the GPU host) on
all host cores and prints the same line with ``"impl": "reference"``.
Multi-GPU (torchrun): replicas, each walking its own photon range (weak
scaling, no data-path collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'photons/s & scatter-events/s (1 GB300) vs plain; surrogate BRF/s at ≤2% err'
N_PER_GPU = 1000000
SEED = 0x5EED0002
# algorithmic thread-instructions per scatter event of the FP32 walk: Philox4x32-10
# (10 rounds x 2 wide multiplies + 2 three-input XORs = 40), four uniform
# conversions (8), HG inversion (6), sin/cos/sqrt of the angles (6), rotation and
# renormalisation (25), move, compensated path sum and boundary tests (15).
ALG_INST_PER_EVENT = 100
# algorithmic work per scatter event by pipe, as the survey of the reference's walk
# counts it (five uniforms = 1.25 Philox4x32-10 blocks of 10 rounds x (2 wide
# multiplies = 4 IMAD, 4 XOR/ADD, 2 key adds) = 125 integer ops; HG inversion,
# rotation, move, path and tests 30 FP32 ops; log, sin, cos and 2 square roots 5 SFU
# ops), and the per-SM rate of each pipe per clock (4 schedulers x 32 lanes for the
# integer and FP32 pipes, 16 for the SFU)
OPS_PER_EVENT = {'int': 125, 'fp32': 30, 'sfu': 5}
PIPE_LANES_PER_SM = {'int': 128, 'fp32': 128, 'sfu': 16}
RECORD_BYTES = 32


def workload(n=N_PER_GPU):
    from monte_carlompi_gb300 import ssp
    from monte_carlompi_gb300.config import WalkConfig
    lo, hi = ssp.grid_for(1.55, 0.085)
    ice = ssp.synthetic_ice_table(250.0, lo, hi)
    imp = ssp.synthetic_impurity_table(lo, hi)
    tau = 0.10 * ssp.ext_cff_mss_sphere(250.0) * 300.0
    cfg = WalkConfig(n_photon=n, wvl0=1.55, half_width=0.085, theta0_deg=60.0, tau_tot=tau,
                     lambertian_reflectance=0.5, rds_snw=250.0)
    return cfg, ice, imp


CONFIG_DESC = {'workload': 'photon walk, 1e6 photons/GPU: r_eff 250 um, lambda0 1.55 um, '
                           'FWHM 0.085 um, theta0 60 deg, depth 0.10 m (tau 196.29), '
                           'Lambertian bottom R 0.5, synthetic sphere SSPs, 18x36 BRF bins',
               'photons_per_gpu': N_PER_GPU, 'mode': 'FP32 Philox4x32-10',
               'l2': 'flushed between timed steps (256 MB write); records 32 MB/step'}


def dist_env():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_sample(n, threads, seed=SEED):
    """Time the C oracle (FP64 port) on n photons of the workload."""
    from oracle import oracle
    cfg, ice, imp = workload(n)
    c = oracle.make_config(n, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot, R=0.5)
    t0 = time.perf_counter()
    rec = oracle.walk(c, ice, imp, seed, threads=threads)
    dt = time.perf_counter() - t0
    return dt, int(rec['n_scat'].astype(np.int64).sum())


def cpu_baseline(target_s=8.0):
    from oracle import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    cores = cpu_cores()
    pilot_n = 20000
    dt, _ = oracle_sample(pilot_n, cores, seed=SEED + 1)
    n = int(min(N_PER_GPU, max(pilot_n, pilot_n * target_s / max(dt, 1e-3))))
    dt, ev = oracle_sample(n, cores)
    return {'value': n / dt, 'unit': 'photons/s', 'cores': cores, 'kind': 'port',
            'events_per_s': ev / dt,
            'sample': '%d of the 1e6 photons (FP64 C oracle, %d threads, %.2f s wall)' % (n, cores, dt)}


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(name)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), 'measured'
    return {'hbm_gbs': 6800.0, 'sm_max_mhz': 2070.0}, 'fallback'


def committed_traffic():
    """DRAM bytes per walk launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, 'profiles', 'walk_f32_traffic.json')
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get('dram_bytes_per_photon')
    return None


def sweep_workload():
    """Sweep workload: 64 configs from r_eff x lambda0 x theta0 x depth, photon counts
    log-uniform over 1e4-1e6, seeded (0x5EED0003)."""
    from monte_carlompi_gb300 import ssp
    from monte_carlompi_gb300.config import WalkConfig
    rng = np.random.default_rng(0x5EED0003)
    radii = [50.0, 100.0, 200.0, 400.0, 800.0, 1500.0]
    tables = [ssp.synthetic_ice_table(r, 600, 2100) for r in radii]
    imp = ssp.synthetic_impurity_table(600, 2100)
    cfgs = []
    for _ in range(64):
        ri = int(rng.integers(len(radii)))
        wvl0 = float(np.round(rng.uniform(0.9, 1.8), 3))
        theta0 = float(rng.choice([0.0, 30.0, 45.0, 60.0]))
        depth = float(rng.choice([0.02, 0.10, 1.0]))
        n = int(10 ** rng.uniform(4, 6))
        tau = depth * ssp.ext_cff_mss_sphere(radii[ri]) * 300.0
        cfgs.append(WalkConfig(n_photon=n, wvl0=wvl0, half_width=0.085, theta0_deg=theta0,
                               tau_tot=tau, lambertian_reflectance=0.5, ice_table=ri,
                               rds_snw=radii[ri]))
    return cfgs, tables, imp


def run_sweep(args, emit=True):
    """Batched sweep in one graph-captured launch vs one launch per config."""
    import torch
    from monte_carlompi_gb300.walker import Walker
    cfgs, tables, imp = sweep_workload()
    total = sum(c.n_photon for c in cfgs)
    w = Walker(0)
    w.set_tables(tables, imp)
    best = w.autotune(cfgs, seed=11)
    recs = torch.empty(total * RECORD_BYTES, dtype=torch.uint8, device='cuda')
    g = w.graph(cfgs, device_ptr=recs.data_ptr())
    for k in range(args.warmup):
        g.launch(SEED + k)
    t_batch, w_batch, events = [], [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        r = g.launch(SEED + 100 + k)          # returns after the sweep's tallies are on the host
        w_batch.append(1e3 * (time.perf_counter() - t0))
        t_batch.append(r.stats['kernel_ms'])
        events += r.stats['n_events']
    # per-config launches (same photons, same statistical error): device time of each
    # call summed, and the wall clock of the loop (a call returns after its tallies are on
    # the host, so the device waits for the next call between configs)
    for k in range(max(1, args.warmup // 2)):
        w.walk([cfgs[0]], SEED, mode='f32', records=None)
    t_plain, w_plain = [], []
    for k in range(args.steps):
        t = 0.0
        t0 = time.perf_counter()
        for c in cfgs:
            t += w.walk([c], SEED + 100 + k, mode='f32', records='device',
                        device_ptr=recs.data_ptr()).stats['device_ms']
        w_plain.append(1e3 * (time.perf_counter() - t0))
        t_plain.append(t)
    g.close()
    w.close()
    tb, tp = float(np.median(t_batch)), float(np.median(t_plain))
    wb, wp = float(np.median(w_batch)), float(np.median(w_plain))
    line = {'metric': METRIC, 'workload': 'sweep', 'value': total / (tb / 1e3), 'unit': 'photons/s',
            'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': tb,
            'higher_is_better': True, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': '64 configs: r_eff {50..1500} um x lambda0 U(0.9,1.8) um x '
                                   'theta0 {0,30,45,60} x depth {0.02,0.10,1.0} m, N log-U(1e4,1e6), '
                                   'seed 0x5EED0003', 'photons': total,
                       'launch': best},
            'scatter_events_per_s': events / args.steps / (tb / 1e3),
            'per_config_launches_ms': tp, 'batched_graph_ms': tb, 'speedup_vs_per_config': tp / tb,
            'wall_ms': {'per_config_loop': wp, 'batched_graph': wb, 'speedup': wp / wb,
                        'note': 'host wall clock of the 64 Walker.walk calls against one graph launch, '
                                'each returning with its tallies on the host'}}
    if emit:
        print(json.dumps(line))
    return line


def run_lone(args):
    """The latency of one photon's walk: single-photon launches of a nearly
    non-absorbing, semi-infinite slab (single-scattering albedo 0.99995, tau 1e7,
    normal incidence) over 30 seeds, the kernel time fitted against n_scat; walked in
    its warp (drain_from 0) and by a whole block in the drain kernel (drain_from 256).
    Records are the same either way.  The first drain-kernel launch of the run walks
    the longest of the 30 photons (the one to capture with ncu -k drain_kernel -c 1)."""
    import dataclasses
    import torch  # noqa: F401  (CUDA context set-up like the other workloads)
    from monte_carlompi_gb300.walker import Walker
    cfg, ice, imp = workload(1)
    lone = dataclasses.replace(cfg, ssa_ice_override=0.99995, tau_tot=1e7, theta0_deg=0.0)
    peaks, _ = measured_peaks()
    mhz = float(peaks.get('sm_max_mhz', 2070.0))
    w = Walker(0)
    w.set_tables([ice], imp)
    out, recs = {}, {}
    longest = SEED
    for drain in (0, 256):
        w.set_launch(128, 4, 1, drain)
        w.walk([lone], longest, records=None)
        xs, ys, rs = [], [], []
        for s in range(30):
            r = w.walk([lone], SEED + 100 + s)
            xs.append(int(r.records['n_scat'][0]))
            ys.append(r.stats['kernel_ms'])
            rs.append(r.records.tobytes())
        longest = SEED + 100 + int(np.argmax(xs))
        xs, ys = np.array(xs, dtype=np.float64), np.array(ys)
        slope = np.linalg.lstsq(np.vstack([xs, np.ones_like(xs)]).T, ys, rcond=None)[0][0]
        out[drain] = {'cycles_per_step': slope * 1e-3 * mhz * 1e6, 'max_n_scat': int(xs.max())}
        recs[drain] = rs
    w.close()
    print(json.dumps({'metric': 'cycles per scatter event of one photon walked alone', 'workload': 'lone',
                      'value': out[256]['cycles_per_step'], 'unit': 'SM cycles/step',
                      'higher_is_better': False, 'dtype': 'f32', 'data': 'synthetic',
                      'config': {'workload': '1 photon x 30 seeds: ssa 0.99995, tau 1e7, theta0 0, '
                                             'r_eff 250 um, 1.55 um', 'sm_mhz': mhz},
                      'in_warp': out[0], 'drain_block': out[256],
                      'same_records': recs[0] == recs[256]}))
    return 0


POL_WVLS = [round(1.0 + 0.025 * i, 4) for i in range(41)]              # um
POL_RE = [60.0, 120.0, 250.0]                                            # um
POL_THETA = [0.5 * k for k in range(20)] + [10.0 + 2.0 * k for k in range(86)]   # deg
POL_STOKES = (1.0, 0.3, 0.2, 0.1)


def pol_workload(n, tmp):
    """Polarised walk of hexagonal plates (r_eff nearest 100 um -> 120 um), lambda0 1.3 um,
    FWHM 0.085, theta0 30 deg, tau 20, Lambertian bottom R 0.5, incident Stokes
    (1, 0.3, 0.2, 0.1); synthetic isca.dat and P11 ... P44 (106 angles) written to tmp."""
    from monte_carlompi_gb300 import ssp
    from monte_carlompi_gb300.config import WalkConfig
    rows = ssp.synthetic_isca_rows(POL_WVLS, POL_RE)
    isca = ssp.isca_path(tmp, 'hexagonal plate', 'moderately rough', 1.3)
    ssp.write_isca(isca, rows)
    ssp.write_phase_matrix(os.path.dirname(isca), POL_THETA, ssp.synthetic_phase_rows(rows, POL_THETA))
    ice, _ = ssp.aspherical_table(isca, 1.3, 100.0)
    phase = ssp.aspherical_phase_table(isca, ice, 1.3)
    lo, hi = ssp.grid_for(1.3, 0.085)
    imp = ssp.synthetic_impurity_table(lo, hi)
    cfg = WalkConfig(n_photon=n, wvl0=1.3, half_width=0.085, theta0_deg=30.0, tau_tot=20.0,
                     lambertian_reflectance=0.5, ssp_nearest=True, polarised=True, stokes0=POL_STOKES)
    return cfg, ice, imp, phase


def run_pol(args):
    """The polarised walk of aspherical grains: the FP32 production kernel ('pol32',
    the line's value) and the FP64 replay kernel ('pol64'), against the C oracle of
    the same walk on the host cores."""
    import tempfile
    import torch  # noqa: F401  (CUDA context set-up like the other workloads)
    from monte_carlompi_gb300.walker import Walker
    n = 1000000
    with tempfile.TemporaryDirectory() as tmp:
        cfg, ice, imp, phase = pol_workload(n, tmp)
    w = Walker(0)
    w.set_tables([ice], imp)
    w.set_phase_matrices([phase])

    def timed(mode, steps, warmup):
        for k in range(warmup):
            w.walk([cfg], SEED + k, mode=mode, records=None)
        ms, ev = [], 0
        for k in range(steps):
            r = w.walk([cfg], SEED + 100 + k, mode=mode, records=None)
            ms.append(r.stats['kernel_ms'])
            ev += r.stats['n_events']
        return float(np.median(ms)), ev / steps
    t, events_per_step = timed('pol32', args.steps, args.warmup)
    t64, ev64 = timed('pol64', 2, 1)
    w.close()
    line = {'metric': 'photons/s (polarised aspherical walk)', 'workload': 'pol',
            'value': n / (t / 1e3), 'unit': 'photons/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t, 'higher_is_better': True, 'dtype': 'f32',
            'data': 'synthetic',
            'config': {'workload': '1e6 photons, hexagonal plates (RE 120 um), 1.3 um, FWHM 0.085, '
                                   '30 deg, tau 20, Lambertian bottom 0.5, Stokes (1, .3, .2, .1); '
                                   'synthetic isca.dat and P11..P44 (106 angles)',
                       'mode': 'MCW_MODE_POL32 (FP32, Philox4x32-10 blocks per step and per rejection candidate)'},
            'scatter_events_per_s': events_per_step / (t / 1e3),
            'pol64': {'value': n / (t64 / 1e3), 'unit': 'photons/s', 'ms_per_step': t64,
                      'scatter_events_per_s': ev64 / (t64 / 1e3),
                      'mode': 'MCW_MODE_POL64 (FP64, replay stream, reference order)'}}
    if not args.no_cpu_baseline:
        from oracle import oracle
        if not os.path.exists(oracle.LIB_PATH):
            oracle.build()
        cores = cpu_cores()
        ph = oracle.make_phase(phase, POL_STOKES)

        def sample(m, seed):
            c = oracle.make_config(m, cfg.wvl0, cfg.half_width, cfg.theta0_deg, cfg.tau_tot,
                                   R=0.5, nearest=True, phase=ph)
            t0 = time.perf_counter()
            rec = oracle.walk(c, ice, imp, seed, threads=cores)
            return time.perf_counter() - t0, int(rec['n_scat'].astype(np.int64).sum())
        dt, _ = sample(2000, SEED + 1)
        m = int(min(n, max(2000, 2000 * 8.0 / max(dt, 1e-3))))
        dt, ev = sample(m, SEED)
        line['cpu_baseline'] = {'value': m / dt, 'unit': 'photons/s', 'cores': cores, 'kind': 'port',
                                'events_per_s': ev / dt,
                                'sample': '%d photons of the workload (FP64 C oracle, %d threads, '
                                          '%.2f s wall)' % (m, cores, dt)}
    print(json.dumps(line))
    return 0


def run_surrogate(args, emit=True):
    """Surrogate workload: --surrogate-configs configs (4,096 by default, the surrogate-training workload) x 2e5 photons walked
    on the GPU, 5-member ensemble trained on the tensor-core kernels, 512 held-out configs
    judged by 1e6- and 1e7-photon Monte Carlo; BRF/s of the network against plain Monte
    Carlo; then the inverse workload."""
    import time as _t
    import torch
    from monte_carlompi_gb300 import surrogate as S
    from monte_carlompi_gb300.walker import Walker
    n_cfg, n_train_photons = args.surrogate_configs, 200000
    w = Walker(0)
    t0 = _t.perf_counter()
    ds = S.make_dataset(w, n_cfg, n_train_photons, seed=0x5EED0004)
    t_data = _t.perf_counter() - t0
    n_hold = min(512, n_cfg // 8)
    train_ds = S.Dataset(ds.x[n_hold:], ds.y[n_hold:], ds.raw[n_hold:], ds.brf[n_hold:],
                         ds.albedo[n_hold:], ds.photons)
    t0 = _t.perf_counter()
    ens = S.train(train_ds, members=5, epochs=args.surrogate_epochs, batch=256, lr=1e-3, seed=4)
    t_train = _t.perf_counter() - t0
    hold = ds.raw[:n_hold]
    t0 = _t.perf_counter()
    ref_brf, ref_alb = S.mc_brf(w, hold, 1000000, seed=0x5EED0044)
    t_ref = _t.perf_counter() - t0
    ref2_brf, _ = S.mc_brf(w, hold, 1000000, seed=0x5EED0045)
    ref7_brf, _ = S.mc_brf(w, hold, 10000000, seed=0x5EED0046)
    pred_brf, pred_alb, spread = ens.predict(hold)
    err = S.rel_rms(pred_brf, ref_brf)
    err7 = S.rel_rms(pred_brf, ref7_brf)
    floor = S.rel_rms(ref2_brf, ref_brf) / np.sqrt(2)
    # the network's own error against 1e6-photon Monte Carlo: that walk's noise (floor,
    # from two independent 1e6-photon walks) removed in quadrature, per config
    err_corr = np.sqrt(np.maximum(err ** 2 - floor ** 2, 0.0))
    err_small_mc = S.rel_rms(ds.brf[:n_hold], ref_brf)
    rate_net = S.inference_rate(ens)                  # every member (mean and spread)
    rate_one = S.inference_rate(ens, members=1)       # one member
    rate_mc = n_hold / t_ref
    inv = run_inverse(ens, w, args.inverse_configs) if args.inverse_configs > 0 else None
    line = {'metric': METRIC, 'workload': 'surrogate', 'value': rate_net, 'unit': 'BRF/s',
            'higher_is_better': True, 'dtype': 'bf16 (fp32 accumulate)', 'data': 'synthetic',
            'config': {'configs': n_cfg, 'held_out': n_hold, 'train_photons': n_train_photons,
                       'judge_photons': 1000000, 'members': 5, 'epochs': args.surrogate_epochs,
                       'batch': 256, 'net': '4-256-256-256-649 SiLU'},
            'brf_per_s_note': 'value: predictions of the whole ensemble (every member forwards the batch '
                              'of 65,536 on the fused kernel, L2 flushed before each timed repetition)',
            'brf_per_s_one_member': rate_one,
            'mc_brf_per_s': rate_mc, 'speedup_vs_mc': rate_net / rate_mc,
            'rms_rel_brf_err_vs_1e6_mc': {'median': float(np.median(err)), 'mean': float(np.mean(err)),
                                          'p90': float(np.percentile(err, 90))},
            'rms_rel_brf_err_vs_1e6_mc_noise_removed': {'median': float(np.median(err_corr)),
                                                        'mean': float(np.mean(err_corr)),
                                                        'p90': float(np.percentile(err_corr, 90))},
            'rms_rel_brf_err_vs_1e7_mc': {'median': float(np.median(err7)), 'mean': float(np.mean(err7)),
                                          'p90': float(np.percentile(err7, 90))},
            'mc_1e6_noise_floor': float(np.median(floor)),
            'mc_1e7_noise_floor_est': float(np.median(floor)) / np.sqrt(10),
            'mc_2e5_err_vs_1e6_mc': float(np.median(err_small_mc)),
            'albedo_abs_err_median': float(np.median(np.abs(pred_alb - ref_alb))),
            'ensemble_spread_median': float(np.median(spread)),
            'seconds': {'data': t_data, 'train': t_train, 'judge_mc': t_ref},
            'inverse': inv}
    if emit:
        print(json.dumps(line))
    w.close()
    return line


def run_mlp(args, emit=True):
    """Surrogate network inference on the fused tcgen05 kernel (mcw_mlp_forward): BRF/s,
    TFLOP/s of the four layers against the measured bf16 peak, and the output stream
    (f32 rows of 652) against the measured HBM copy bandwidth."""
    import torch
    from monte_carlompi_gb300 import surrogate as S
    batch = 65536
    net = S.SurrogateMLP(seed=0)
    x = torch.rand((batch, 4), device='cuda') * 2 - 1
    for _ in range(args.warmup):
        net.predict_std(x)
    # each timed forward after an L2 flush (the fp16 output, 86 MB, would otherwise stay in
    # the 126 MB L2 from one call to the next); the flush keeps the stream busy while the
    # forward is queued, so the events time the kernel, not the host
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device='cuda')
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0.record()
        net.predict_std(x)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    e0.record()
    for _ in range(args.steps):
        net.predict_std(x)
    e1.record()
    torch.cuda.synchronize()
    ms_b2b = e0.elapsed_time(e1) / args.steps
    # a 5-member ensemble on the same rows in one launch (mcw_mlp_forward_ensemble_f16),
    # the way the surrogate predicts with its spread
    ens = S.Ensemble([net] + [S.SurrogateMLP(seed=k) for k in range(1, 5)])
    for _ in range(args.warmup):
        ens.predict_std(x)
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0.record()
        ens.predict_std(x)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms_ens = float(np.median(times))
    flop = 2.0 * batch * sum(a * b for a, b in zip(S.DIMS[:-1], S.DIMS[1:]))
    out_bytes = batch * S.Y_PITCH_F16 * 2 + batch * 4 * 4
    peaks, src = measured_peaks()
    tflops = flop / (ms / 1e3) / 1e12
    gbs = out_bytes / (ms / 1e3) / 1e9
    peak = float(peaks.get('bf16_tflops') or 1900.0)
    hbm = float(peaks.get('hbm_gbs') or 6800.0)
    line = {'metric': METRIC, 'workload': 'mlp', 'value': batch / (ms / 1e3), 'unit': 'BRF/s',
                      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms, 'dtype': 'bf16',
                      'gpu_launches': args.steps,
                      'config': {'batch': batch, 'net': '4-256-256-256-649 SiLU',
                                 'kernels': 'one fused kernel: tcgen05.mma kind::f16 into tensor memory, '
                                            'cp.async.bulk weight ring, activations in shared memory, '
                                            'fp16 output',
                                 'l2': 'flushed (256 MB write) before every timed forward; median of the '
                                       'steps', 'ms_back_to_back': ms_b2b},
            'ensemble_5': {'ms': ms_ens, 'brf_per_s': batch / (ms_ens / 1e3),
                           'tflops': 5 * flop / (ms_ens / 1e3) / 1e12,
                           'frac': 5 * flop / (ms_ens / 1e3) / 1e12 / float(peaks.get('bf16_tflops') or 1900.0),
                           'what': 'five networks on the same 65,536 rows in one launch '
                                   '(mcw_mlp_forward_ensemble_f16), L2 flushed before each'},
                      'roofline': {'bound': 'tensor', 'achieved': tflops, 'peak': peak, 'unit': 'TFLOP/s',
                                   'frac': tflops / peak, 'peak_source': src,
                                   'hbm': {'achieved': gbs, 'peak': hbm, 'unit': 'GB/s', 'frac': gbs / hbm,
                                           'bytes': 'x in + y out (fp16, row pitch 656)'}}}
    if emit:
        print(json.dumps(line))
    return line


def run_train(args):
    """Surrogate training on the training engine: (a) one Adam step of a 5-member
    ensemble at batch 256 (the surrogate-training batch), all members at once from one
    captured CUDA graph, against the same step run member by member on the layer-wise
    kernels; (b) forward + backward of one network over 65,536 rows (split-K weight
    gradients) against the layer-wise autograd path.  FLOPs: 3 x 596,480 per row
    (forward, input and weight gradients)."""
    import torch
    from monte_carlompi_gb300 import surrogate as S
    peaks, src = measured_peaks()
    peak = float(peaks.get('bf16_tflops_sustained') or peaks.get('bf16_tflops') or 1700.0)
    flop_row = 3.0 * 2 * sum(a * b for a, b in zip(S.DIMS[:-1], S.DIMS[1:]))
    rng = np.random.default_rng(0x5EED0004)
    w = torch.from_numpy(S.output_weights()).cuda()
    big = 65536
    if args.train_part == 'big':
        # only the 65,536-row forward + backward (a short case for a profiler)
        xb = torch.from_numpy(rng.uniform(-1, 1, (big, 4)).astype(np.float32)).cuda()
        tb = torch.from_numpy(rng.standard_normal((big, 649)).astype(np.float32)).cuda()
        one = S.EnsembleTrainer([S.SurrogateMLP(seed=9)], big, xb, tb, w, use_graph=False)
        one.set_epoch([np.arange(big)], 1e-3)
        for _ in range(args.warmup + args.steps):
            one._launch(adam=False)
        torch.cuda.synchronize()
        print(json.dumps({'workload': 'train', 'part': 'big', 'rows': big, 'launch_sets': args.warmup + args.steps}))
        return 0
    n_rows, members, batch = 16384 - 512, 5, 256
    x = torch.from_numpy(rng.uniform(-1, 1, (n_rows, 4)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((n_rows, 649)).astype(np.float32)).cuda()
    nets = [S.SurrogateMLP(seed=k) for k in range(members)]
    tr = S.EnsembleTrainer(nets, batch, x, t, w, lr=1e-3)
    steps = min(max(args.steps, 10) * 10, n_rows // batch)
    tr.set_epoch([rng.permutation(n_rows) for _ in nets], 1e-3)
    for _ in range(args.warmup):
        tr.run_step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tr.set_epoch([rng.permutation(n_rows) for _ in nets], 1e-3)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        tr.run_step()
    e1.record()
    torch.cuda.synchronize()
    ms_grouped = e0.elapsed_time(e1) / steps
    # the same step member by member on the layer-wise kernels (host-launched)
    x16 = S._cast(torch, x)
    perm = torch.from_numpy(rng.permutation(n_rows)).cuda()
    for _ in range(args.warmup):
        for net in nets:
            net.train_step(x16[perm[:batch]].contiguous(), t[perm[:batch]].contiguous(), w)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 20
    for r in range(reps):
        idx = perm[r * batch:(r + 1) * batch]
        for net in nets:
            net.train_step(x16[idx].contiguous(), t[idx].contiguous(), w)
    torch.cuda.synchronize()
    ms_layer = (time.perf_counter() - t0) * 1e3 / reps
    # forward + backward of 65,536 rows, one network
    xb = torch.from_numpy(rng.uniform(-1, 1, (big, 4)).astype(np.float32)).cuda()
    tb = torch.from_numpy(rng.standard_normal((big, 649)).astype(np.float32)).cuda()
    one = S.EnsembleTrainer([S.SurrogateMLP(seed=9)], big, xb, tb, w, use_graph=False)
    one.set_epoch([np.arange(big)], 1e-3)
    for _ in range(args.warmup):
        one._launch(adam=False)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        one._launch(adam=False)
    e1.record()
    torch.cuda.synchronize()
    ms_big = e0.elapsed_time(e1) / args.steps
    # the same through the layer-wise autograd path
    params = [p.detach().clone().requires_grad_(True) for p in one.members[0].params]
    y = S.mlp_apply(xb, params)
    y.backward(torch.ones_like(y))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(2):
        y = S.mlp_apply(xb, params)
        y.backward(torch.ones_like(y))
    torch.cuda.synchronize()
    ms_big_layer = (time.perf_counter() - t0) * 1e3 / 2
    tflops = flop_row * big / (ms_big / 1e3) / 1e12
    line = {'metric': 'surrogate training: ensemble Adam step time', 'workload': 'train',
            'value': ms_grouped, 'unit': 'ms per 5-member step (batch 256)', 'higher_is_better': False,
            'steps': args.steps, 'warmup': args.warmup, 'dtype': 'bf16 (fp32 accumulate, fp32 Adam)',
            'data': 'synthetic',
            'config': {'net': '4-256-256-256-649 SiLU', 'members': members, 'batch': batch,
                       'engine': 'grouped tcgen05 GEMMs fed by TMA, one CUDA graph per step '
                                 '(16 launches for all members)'},
            'layerwise_ms_per_step': ms_layer, 'speedup_vs_layerwise': ms_layer / ms_grouped,
            'fwd_bwd_65536': {'ms': ms_big, 'layerwise_ms': ms_big_layer, 'speedup': ms_big_layer / ms_big,
                              'tflops': tflops, 'splits': one.splits},
            'roofline': {'bound': 'tensor', 'achieved': tflops, 'peak': peak, 'unit': 'TFLOP/s',
                         'frac': tflops / peak, 'peak_source': src + ' (bf16 sustained)',
                         'kernel': '65,536-row forward + backward'}}
    print(json.dumps(line))
    return 0


def run_inverse(ens, walker, n_obs):
    """Inverse configuration: observed BRFs from 1e6-photon MC at hidden r_eff
    (log-uniform 50-1500 um, known lambda, theta0, depth) plus 1% Gaussian noise; Gauss-Newton
    on log r_eff through the surrogate with MC fallback where the ensemble spread exceeds 2%,
    against the same retrieval (grid + Gauss-Newton) driven by plain MC on a subset."""
    import time as _t
    from monte_carlompi_gb300 import inverse as I
    from monte_carlompi_gb300 import surrogate as S
    raw = S.sample_inputs(n_obs, 0x5EED0005)
    t0 = _t.perf_counter()
    obs, _ = S.mc_brf(walker, raw, 1000000, seed=0x5EED0050)
    t_obs = _t.perf_counter() - t0
    obs = obs * (1 + 0.01 * np.random.default_rng(0x5EED0051).standard_normal(obs.shape))
    known = raw[:, 1:]
    noise = dict(obs_photons=1000000, obs_noise=0.01)
    # warm-up (untimed): the first float64 tensor operations of a fresh process take seconds
    # on this PyTorch build (their kernels are compiled for the GPU on first use)
    I.retrieve(ens, walker, obs[:32], known[:32], criterion='r_eff', fallback='correct', **noise)
    I.retrieve(ens, walker, obs[:32], known[:32], criterion='r_eff', fallback='gn', **noise)
    # residuals weighted by their inverse noise variance; where the ensemble spread of the
    # retrieved r_eff exceeds 2%, the answer is corrected by walks at it (the surrogate's
    # Jacobian, Monte Carlo residuals)
    res = I.retrieve(ens, walker, obs, known, criterion='r_eff', fallback='correct', **noise)
    err = np.abs(res['r_eff'] / raw[:, 0] - 1)
    # the same with Monte Carlo Gauss-Newton (central differences) as the fallback
    res_r = I.retrieve(ens, walker, obs, known, criterion='r_eff', fallback='gn', **noise)
    err_r = np.abs(res_r['r_eff'] / raw[:, 0] - 1)
    # the surrogate alone (no walk)
    s_net = I.surrogate_gn(ens, obs, known, **noise)[0]
    err_net = np.abs(np.exp(s_net) / raw[:, 0] - 1)
    # the same retrieval with plain Monte Carlo only, on a subset
    n_sub = min(64, n_obs)
    t0 = _t.perf_counter()
    s_mc, evals = I.mc_retrieve(walker, obs[:n_sub], known[:n_sub], **noise)
    t_mc = _t.perf_counter() - t0
    err_mc = np.abs(np.exp(s_mc) / raw[:n_sub, 0] - 1)
    t_sur = res['seconds_net'] + res['seconds_mc']
    net_evals = n_obs * (16 + 6 + 1)
    return {'observations': n_obs, 'obs_photons': 1000000, 'noise': 0.01,
            'weights': 'inverse noise variance per bin: counting noise of the 1e6-photon observation '
                       '+ 1% noise + ensemble variance',
            'flagged_for_mc': float(res['flagged'].mean()),
            'r_eff_rel_err': {'median': float(np.median(err)), 'p90': float(np.percentile(err, 90))},
            'r_eff_rel_err_unflagged_median':
                float(np.median(err[~res['flagged']])) if np.any(~res['flagged']) else None,
            'posterior_width_median': float(np.median(res['sigma_noise'])),
            'seconds': {'surrogate_gn': res['seconds_net'], 'mc_fallback': res['seconds_mc']},
            'seconds_per_retrieval': t_sur / n_obs,
            'brf_evals': {'surrogate': net_evals, 'mc_fallback': res['mc_brf_evals']},
            'mc_only': {'subset': n_sub, 'method': '16-point grid + 4 Gauss-Newton iterations, 1e6-photon '
                                                    'BRFs, central-difference Jacobians, same weights',
                        'r_eff_rel_err_median': float(np.median(err_mc)),
                        'r_eff_rel_err_p90': float(np.percentile(err_mc, 90)),
                        'surrogate_path_err_median_same_subset': float(np.median(err[:n_sub])),
                        'surrogate_path_err_p90_same_subset': float(np.percentile(err[:n_sub], 90)),
                        'seconds_per_retrieval': t_mc / n_sub, 'brf_evals': evals},
            'speedup_per_retrieval_vs_mc': (t_mc / n_sub) / (t_sur / n_obs),
            'seconds_obs_generation': t_obs,
            'criterion': 'ensemble spread of the retrieved r_eff > 2%; fallback: walks at the answer '
                         '(2 iterations, surrogate Jacobian)',
            'surrogate_only_r_eff_rel_err': {'median': float(np.median(err_net)),
                                             'p90': float(np.percentile(err_net, 90))},
            'r_eff_criterion': {
                'criterion': 'ensemble spread of the retrieved r_eff > 2%; fallback: Monte Carlo '
                             'Gauss-Newton (3 iterations, central differences)',
                'flagged_for_mc': float(res_r['flagged'].mean()),
                'r_eff_rel_err': {'median': float(np.median(err_r)), 'p90': float(np.percentile(err_r, 90))},
                'r_eff_rel_err_unflagged_median':
                    float(np.median(err_r[~res_r['flagged']])) if np.any(~res_r['flagged']) else None,
                'r_eff_rel_err_flagged_median':
                    float(np.median(err_r[res_r['flagged']])) if np.any(res_r['flagged']) else None,
                'seconds': {'surrogate_gn': res_r['seconds_net'], 'mc_fallback': res_r['seconds_mc']},
                'brf_evals_mc_fallback': res_r['mc_brf_evals'],
                'spread_r_eff_median': float(np.median(res_r['spread_r_eff']))}}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    cores = cpu_cores()
    from oracle import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    n = N_PER_GPU   # the whole workload each step (about 0.2-0.3 s on 16 cores)
    for k in range(args.warmup):
        oracle_sample(20000, cores, seed=SEED + 7 + k)
    times, events = [], 0
    for k in range(args.steps):
        dt, ev = oracle_sample(n, cores, seed=SEED + k)
        times.append(dt)
        events += ev
    tot = sum(times)
    value = n * args.steps / tot
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'photons/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * tot / args.steps, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': dict(CONFIG_DESC, photons_per_step=n,
                       mode='FP64 replay stream of the reference algorithm (C oracle on the host cores)'),
        'scatter_events_per_s': events / tot,
        'cpu_baseline': {'value': value, 'unit': 'photons/s', 'cores': cores, 'kind': 'port',
                         'sample': 'all %d photons of the workload each step (FP64 C oracle, '
                                   '%d threads, np.array_split shares as parallelize.py:14-15)' % (n, cores),
                         'python_reference': 'not run: the reference is a Python checkout without an '
                                             'installer and is absent on the GPU host'},
        'e2e': {'value': value, 'unit': 'photons/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    from monte_carlompi_gb300 import replicas
    from monte_carlompi_gb300.walker import Walker

    full, ice, imp = workload(N_PER_GPU * world)
    cfg = replicas.shard_configs([full], rank, world)[0]
    n = cfg.n_photon
    w = Walker(dev)
    w.set_tables([ice], imp)
    # launch shape: the library's autotuner, once, outside the timed region
    tuned = w.autotune([cfg], seed=11)
    tuned.pop('ms')
    w.set_launch(**tuned)
    kernels_per_walk = 3 if tuned['drain_from'] > 0 else 2   # lookup table, walk, drain
    dev_records = torch.empty(n * RECORD_BYTES, dtype=torch.uint8, device='cuda')
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device='cuda')

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step(seed):
        return w.walk([cfg], seed, mode='f32', records='device', device_ptr=dev_records.data_ptr())

    for k in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        step(SEED + 1000 + k)
    # host wall time of one walk (with its flush), to size the timed region
    t0 = time.perf_counter()
    for k in range(10):
        flush.zero_()
        torch.cuda.synchronize()
        step(SEED + 1100 + k)
    wall_per_walk = (time.perf_counter() - t0) / 10
    # inner repeats: each timed step walks the 1e6 photons `repeats` times (a new seed
    # and an L2 flush before each walk), so that the timed region lasts about 2 s and
    # the clock sampler sees it under load
    repeats = args.repeats or max(1, int(np.ceil(2.5 / max(1e-5, wall_per_walk * args.steps))))
    if world > 1:
        rt = torch.tensor([repeats], device='cuda')
        torch.distributed.all_reduce(rt, op=torch.distributed.ReduceOp.MAX)
        repeats = int(rt.item())
    clocks = Clocks(dev)
    clocks.start()
    barrier()
    dev_ms, kern_ms, events, launches = [], [], 0, 0
    for k in range(args.steps):
        for j in range(repeats):
            flush.zero_()
            torch.cuda.synchronize()
            r = step(SEED + k * repeats + j)
            dev_ms.append(r.stats['device_ms'])
            kern_ms.append(r.stats['kernel_ms'])
            events += r.stats['n_events']
            launches += kernels_per_walk
    barrier()
    clk = clocks.stop()
    t_dev = sum(dev_ms) / 1e3
    t_kern = sum(kern_ms) / 1e3

    # e2e: public API, host buffers (pinned), host wall clock per call
    from monte_carlompi_gb300 import _abi
    import ctypes
    host_ptr = ctypes.c_void_p()
    _abi.check(_abi.load().mcw_host_alloc(n * RECORD_BYTES, ctypes.byref(host_ptr)), what='host alloc')
    host_buf = (ctypes.c_char * (n * RECORD_BYTES)).from_address(host_ptr.value)
    host_rec = np.frombuffer(host_buf, dtype=_abi.RECORD32, count=n)
    for k in range(max(1, args.warmup)):
        w.walk([cfg], SEED + 2000 + k, mode='f32', records='host', out=host_rec)
    barrier()
    e2e_t, h2d, d2h = [], 0, 0
    e2e_dev, e2e_kern, e2e_lib = [], [], []
    e2e_calls = args.steps * min(repeats, 20)
    for k in range(e2e_calls):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = w.walk([cfg], SEED + 3000 + k, mode='f32', records='host', out=host_rec)
        e2e_t.append(time.perf_counter() - t0)
        h2d, d2h = r.stats['h2d_bytes'], r.stats['d2h_bytes']
        e2e_dev.append(r.stats['device_ms'])
        e2e_kern.append(r.stats['kernel_ms'])
        e2e_lib.append(r.stats['total_ms'])
    barrier()
    _abi.load().mcw_host_free(host_ptr)

    local_stats = np.array([t_dev, t_kern, sum(e2e_t), events], dtype=np.float64)
    if world > 1:
        t = torch.tensor(local_stats[:3], device='cuda')
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ev = torch.tensor([events], dtype=torch.float64, device='cuda')
        torch.distributed.all_reduce(ev)
        local_stats[:3] = t.cpu().numpy()
        local_stats[3] = float(ev.item())
    t_dev, t_kern, t_e2e, events_all = local_stats
    walks = args.steps * repeats
    photons_all = N_PER_GPU * world * walks
    value = photons_all / t_dev
    if rank == 0:
        peaks, src = measured_peaks()
        sm_max = float(peaks.get('sm_max_mhz') or 2070.0)
        ev_per_launch = events_all / walks / world
        kern_s = t_kern / walks
        ev_rate = ev_per_launch / kern_s
        pipes = {}
        for pipe, ops in OPS_PER_EVENT.items():
            pk = 152 * PIPE_LANES_PER_SM[pipe] * sm_max * 1e6 / 1e12
            pipes[pipe] = {'achieved': ev_rate * ops / 1e12, 'peak': pk, 'frac': ev_rate * ops / 1e12 / pk,
                           'ops_per_event': ops}
        limiting = max(pipes, key=lambda q: pipes[q]['frac'])
        achieved = pipes[limiting]['achieved']
        peak = pipes[limiting]['peak']
        issue_peak = 152 * 4 * 32 * sm_max * 1e6 / 1e12
        achieved_100 = ev_rate * ALG_INST_PER_EVENT / 1e12
        rec_gbs = (n * RECORD_BYTES) / kern_s / 1e9
        tb = committed_traffic()
        line = {
            'metric': METRIC, 'value': value, 'unit': 'photons/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * t_dev / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic',
            'config': dict(CONFIG_DESC, parallelism='replicas x%d' % world, launch=tuned,
                           walks_per_step=repeats,
                           step='%d walks of the 1e6 photons, each with its own seed and an L2 flush '
                                'before it' % repeats,
                           lookup_table='built by the first walk of a config and reused while the '
                                        'configs and SSP tables are unchanged (mcw_walk)'),
            'ms_per_walk': 1e3 * t_dev / walks,
            'scatter_events_per_s': events_all / t_dev,
            'kernel_ms_per_walk': 1e3 * kern_s,
            'clocks': clk,
            'gpu_launches': launches,
            'e2e': {'value': N_PER_GPU * world * e2e_calls / t_e2e, 'unit': 'photons/s',
                    'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h),
                    'calls': e2e_calls,
                    'ms_per_call': {'host_wall': 1e3 * t_e2e / e2e_calls,
                                    'library_call': float(np.median(e2e_lib)),
                                    'device': float(np.median(e2e_dev)),
                                    'kernel': float(np.median(e2e_kern))},
                    'path': 'Walker.walk -> mcw_walk, records written into pinned host memory, '
                            'tallies copied back; host wall clock per call'},
            'roofline': {
                'bound': 'issue (%s pipe)' % limiting, 'achieved': achieved, 'peak': peak, 'unit': 'Tops/s',
                'frac': achieved / peak,
                'traffic': (tb * n) if tb else None,
                'traffic_note': 'DRAM bytes inside one launch (ncu, profiles/walk_f32_traffic.json): tables '
                                'and launch data; the 32 MB of records (32 B per photon) stay in L2 during '
                                'the launch and are written back after it, so the write-back is not counted',
                'basis': 'max over pipes of events/s x algorithmic ops per event (int 125, fp32 30, sfu 5) '
                         'against the pipe rate (152 SMs x lanes per clock x %.0f MHz, sm_max_mhz, %s)' % (
                             sm_max, src),
                'pipes': pipes,
                'issue_100': {'achieved': achieved_100, 'peak': issue_peak, 'frac': achieved_100 / issue_peak,
                              'basis': '%d thread-instructions per scatter event against the issue rate '
                                       '(152 x 4 x 32 lanes x sm_max_mhz)' % ALG_INST_PER_EVENT},
                'hbm': {'achieved': rec_gbs, 'peak': peaks.get('hbm_gbs'), 'unit': 'GB/s',
                        'frac': rec_gbs / float(peaks.get('hbm_gbs') or 6800.0),
                        'bytes': 'records, 32 B/photon'},
            },
        }
        if not args.no_cpu_baseline:
            line['cpu_baseline'] = cpu_baseline()
        if world == 1 and not args.no_extras:
            line['extras'] = extras(args)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    w.close()
    return 0


def extras(args):
    """The other workloads, run after the walk's timed region and summarised in its line:
    the 64-config sweep, fused inference, and the surrogate (training, its error against
    Monte Carlo, inference rate, the inverse).  A workload that fails records its error."""
    out = {}

    def keep(d, keys):
        return {k: d[k] for k in keys if k in d}

    try:
        s = run_sweep(args, emit=False)
        out['sweep'] = keep(s, ['value', 'unit', 'batched_graph_ms', 'per_config_launches_ms',
                                'speedup_vs_per_config', 'wall_ms', 'scatter_events_per_s'])
        out['sweep']['config'] = s['config']['workload']
    except Exception as e:  # noqa: BLE001  (a failed extra must not lose the walk's line)
        out['sweep'] = {'error': repr(e)}
    try:
        m = run_mlp(args, emit=False)
        out['mlp'] = keep(m, ['value', 'unit', 'ms_per_step', 'ensemble_5'])
        out['mlp']['roofline'] = keep(m['roofline'], ['bound', 'achieved', 'peak', 'unit', 'frac'])
        out['mlp']['config'] = m['config']
    except Exception as e:  # noqa: BLE001
        out['mlp'] = {'error': repr(e)}
    try:
        g = run_surrogate(args, emit=False)
        out['surrogate'] = keep(g, ['value', 'unit', 'brf_per_s_one_member', 'mc_brf_per_s', 'speedup_vs_mc',
                                    'rms_rel_brf_err_vs_1e6_mc', 'rms_rel_brf_err_vs_1e6_mc_noise_removed',
                                    'rms_rel_brf_err_vs_1e7_mc', 'mc_1e6_noise_floor', 'seconds', 'config'])
        inv = g.get('inverse') or {}
        out['surrogate']['inverse'] = keep(inv, ['observations', 'r_eff_rel_err', 'flagged_for_mc',
                                                 'seconds_per_retrieval', 'speedup_per_retrieval_vs_mc',
                                                 'criterion'])
        if 'mc_only' in inv:
            out['surrogate']['inverse']['mc_only'] = keep(inv['mc_only'], [
                'subset', 'r_eff_rel_err_median', 'surrogate_path_err_median_same_subset',
                'seconds_per_retrieval'])
    except Exception as e:  # noqa: BLE001
        out['surrogate'] = {'error': repr(e)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--repeats', type=int, default=0,
                    help='walks per timed step (0: enough for about 2 s of timed work)')
    ap.add_argument('--workload', default='walk',
                    choices=['walk', 'sweep', 'surrogate', 'mlp', 'pol', 'lone', 'train'])
    ap.add_argument('--train-part', default='all', choices=['all', 'big'],
                    help="train workload: 'big' runs only the 65,536-row forward + backward")
    ap.add_argument('--surrogate-configs', type=int, default=4096)
    ap.add_argument('--surrogate-epochs', type=int, default=300)
    ap.add_argument('--inverse-configs', type=int, default=4096)
    ap.add_argument('--no-extras', action='store_true',
                    help='walk workload: skip the other workloads summarised under "extras"')
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)
    if args.workload == 'sweep':
        run_sweep(args)
        return 0
    if args.workload == 'surrogate':
        run_surrogate(args)
        return 0
    if args.workload == 'mlp':
        run_mlp(args)
        return 0
    if args.workload == 'pol':
        return run_pol(args)
    if args.workload == 'lone':
        return run_lone(args)
    if args.workload == 'train':
        return run_train(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
