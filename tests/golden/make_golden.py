#!/usr/bin/env python
"""Generate golden per-photon fixtures by running the UNMODIFIED reference.

Run where a checkout of the reference exists, naming it with ``--reference``
or the ``MC_REFERENCE`` environment variable::

    python tests/golden/make_golden.py --reference <checkout>            # all cases
    python tests/golden/make_golden.py --reference <checkout> kat cfg1   # selected cases

The reference (monte_carloMPI/monte_carlo3D.py) is imported as-is.  A small
harness supplies what it needs to run here:

* stub modules for matplotlib / mpl_toolkits (plots only) and mpi4py
  (a size-1 communicator: scatter returns the one partition, gather wraps the
  answer), because those packages are not installed;
* ``configparser.SafeConfigParser`` aliased to ``ConfigParser`` (removed in
  Python 3.12; monte_carlo3D.py:1781), a ``config.ini`` in the working
  directory (:1784) and a bare ``sys.argv`` for its argparse (:1841);
* synthetic SSP netCDF files in the reference's layout (:507-514, :666-671);
* ``np.set_printoptions(legacy='1.25')`` so its ``'%r'`` CSV rows print plain
  floats under NumPy 2 (:1627-1636);
* replay mode: ``np.random.rand / uniform / normal`` are replaced by the
  Philox replay stream of ``oracle/philox.py`` (photon-indexed, so the C
  oracle and the CUDA replay kernel can consume the same numbers).

Each case writes ``<case>.npz`` with the inputs, the SSP tables, and the
reference's per-photon answers (condition, wvn, theta_n, phi_n, n_scat,
path_length, snow_depth) plus the number of uniforms each photon consumed.
Cases marked ``csv`` also keep the reference's CSV output byte for byte.
"""
import configparser
import os
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import philox  # noqa: E402
from monte_carlompi_gb300 import ssp  # noqa: E402

REFERENCE = os.environ.get('MC_REFERENCE')   # checkout of the reference; or --reference

# name -> run parameters.  depth_m is converted to tau_tot with the synthetic
# extinction (tau = depth * ext_cff_mss * rho_snw); tau_tot given directly wins.
CASES = {
    # driver default geometry (monte_carlo3D-run.py:7-12,18-55) at theta0 = 0,
    # r_eff 100 um, 0.5 m deep; literal 1.20-1.40 um table
    'cfg1': dict(n_photon=1000, wvl0=1.3, half_width=0.085, rds=100.0, theta0=0.0,
                 depth_m=0.5, table_nm=(1200, 1400), lam_bottom=True, R=0.5,
                 seed=0x5EED0001, csv=True),
    # the same run at the driver's own size, 10,000 packets (monte_carlo3D-run.py:18);
    # its first 1,000 photons are cfg1's (the replay stream is photon-indexed)
    'cfg1_10k': dict(n_photon=10000, wvl0=1.3, half_width=0.085, rds=100.0, theta0=0.0,
                     depth_m=0.5, table_nm=(1200, 1400), lam_bottom=True, R=0.5,
                     seed=0x5EED0001, csv=False),
    # convergence-size geometry: r 250 um, 1.55 um, 60 deg, 0.10 m
    'cfg2': dict(n_photon=1000, wvl0=1.55, half_width=0.085, rds=250.0, theta0=60.0,
                 depth_m=0.10, lam_bottom=True, R=0.5, seed=0x5EED0002, csv=True),
    # the last 1,000 photons of the 1e6-photon convergence run (photons 999,000 ..
    # 999,999, the share np.array_split gives the last of 1,000 ranks,
    # parallelize.py:14-15): the replay stream far into a run
    'cfg2_tail': dict(n_photon=1000, first_photon=999000, wvl0=1.55, half_width=0.085,
                      rds=250.0, theta0=60.0, depth_m=0.10, lam_bottom=True, R=0.5,
                      seed=0x5EED0002, csv=False),
    # thin slab: exercises conditions 2 and 3 and the Lambertian bottom
    'thin': dict(n_photon=2000, wvl0=1.55, half_width=0.085, rds=1500.0, theta0=60.0,
                 depth_m=0.02, lam_bottom=True, R=0.5, seed=0x5EED0010, csv=False),
    # Wang et al. (1995) / van de Hulst known-answer slab, no bottom reflection
    'kat': dict(n_photon=4000, wvl0=0.5, half_width=0.085, rds=100.0, theta0=0.0,
                tau_tot=2.0, lam_bottom=False, R=1.0, test=dict(ssa_ice=0.9, g=0.75),
                table_nm=(300, 700), seed=0x5EED0011, csv=False),
    # Lambertian surface instead of snow
    'lamsurf': dict(n_photon=400, wvl0=1.3, half_width=0.085, rds=100.0, theta0=30.0,
                    depth_m=0.5, lam_surface=True, lam_bottom=True, R=0.7,
                    seed=0x5EED0012, csv=False),
    # impurity: condition 5
    'imp': dict(n_photon=600, wvl0=1.1, half_width=0.085, rds=250.0, theta0=30.0,
                depth_m=0.05, imp_cnc=2e-4, lam_bottom=True, R=0.3,
                seed=0x5EED0013, csv=False),
    # out-of-table wavelengths: 1.20-1.40 table, centre 1.39 um -> nearest-value fallback
    'edge': dict(n_photon=400, wvl0=1.39, half_width=0.085, rds=100.0, theta0=45.0,
                 depth_m=0.02, table_nm=(1200, 1400), lam_bottom=True, R=0.5,
                 seed=0x5EED0014, csv=False),
    # one photon: the scalar branch of the SSP lookup (monte_carlo3D.py:518-583)
    'single': dict(n_photon=1, wvl0=1.3, half_width=0.085, rds=100.0, theta0=15.0,
                   depth_m=0.5, lam_bottom=True, R=0.5, seed=0x5EED0015, csv=False),
    # HG-forced aspherical grains (run(shape=...), HG=True): a synthetic isca.dat with
    # three particle sizes on a 25 nm grid; nearest size and nearest wavelength, the
    # photon's wavelength replaced; an impurity table whose extinction varies with
    # wavelength, so the impurity lookup at the replaced wavelength shows in snow_depth
    'asph': dict(n_photon=600, wvl0=1.3, half_width=0.085, rds=100.0, theta0=30.0,
                 tau_tot=40.0, imp_cnc=1e-4, lam_bottom=True, R=0.5, seed=0x5EED0016,
                 shape='solid hexagonal column', roughness='smooth', csv=True),
    # polarised walk of aspherical grains (HG off): the same synthetic isca.dat plus
    # synthetic P11 ... P44 on a non-uniform angle grid; rejection-sampled scattering
    # angles and the Stokes vector of a partially polarised incident beam
    'pol': dict(n_photon=300, wvl0=1.3, half_width=0.085, rds=100.0, theta0=30.0,
                tau_tot=20.0, lam_bottom=True, R=0.5, seed=0x5EED0017,
                shape='hexagonal plate', roughness='moderately rough', hg=False,
                stokes=(1.0, 0.3, 0.2, 0.1), csv=True),
}

PHASE_THETA = [0.5 * k for k in range(20)] + [10.0 + 2.0 * k for k in range(86)]   # deg, 0 .. 180

ASPH_WVLS = [round(1.0 + 0.025 * i, 4) for i in range(41)]   # 1.0 .. 2.0 um
ASPH_RE = [60.0, 120.0, 250.0]


def _install_stubs():
    for name in ('matplotlib', 'matplotlib.pyplot', 'mpl_toolkits', 'mpl_toolkits.mplot3d'):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules['matplotlib'].pyplot = sys.modules['matplotlib.pyplot']
    sys.modules['mpl_toolkits.mplot3d'].Axes3D = object

    class _Comm:
        size = 1
        rank = 0

        def scatter(self, data, root=0):
            return data[0]

        def gather(self, data, root=0):
            return [data]

    mpi = types.ModuleType('mpi4py.MPI')
    mpi.COMM_WORLD = _Comm()
    pkg = types.ModuleType('mpi4py')
    pkg.MPI = mpi
    sys.modules['mpi4py'] = pkg
    sys.modules['mpi4py.MPI'] = mpi
    if not hasattr(configparser, 'SafeConfigParser'):
        configparser.SafeConfigParser = configparser.ConfigParser


class Replay:
    """Answers np.random calls from the photon-indexed Philox replay stream."""

    def __init__(self, seed, first_photon=0):
        self.seed = seed
        self.first = first_photon        # global index of the run's photon 0
        self.photon = None
        self.k = 0
        self.initial_calls = None
        self._cache = np.empty(0)
        self._cache_photon = None

    def _next(self, n):
        if self.initial_calls is not None:        # initial_pdfs: photon-major, 3 draws each
            out = []
            for _ in range(n):
                c = self.initial_calls
                self.initial_calls += 1
                out.append(float(philox.replay_uniform(self.seed, philox.TAG_WALK,
                                                       self.first + c // 3, c % 3)))
            return np.array(out)
        if self.photon is None:
            raise RuntimeError('uniform drawn outside a photon')
        if self._cache_photon != self.photon or self.k + n > self._cache.size:
            size = max(1024, 2 * (self.k + n))
            self._cache = philox.replay_uniform(self.seed, philox.TAG_WALK, self.photon,
                                                np.arange(size, dtype=np.uint64))
            self._cache_photon = self.photon
        out = self._cache[self.k:self.k + n].copy()
        self.k += n
        return out

    def rand(self, *shape):
        if not shape:
            return float(self._next(1)[0])
        return self._next(int(np.prod(shape))).reshape(shape)

    def uniform(self, low=0.0, high=1.0, size=None):
        if size is not None:
            raise NotImplementedError
        return low + (high - low) * float(self._next(1)[0])

    def normal(self, loc=0.0, scale=1.0, size=None):
        n = int(np.prod(size))
        z = philox.replay_normal(self.seed, np.arange(self.first, self.first + n, dtype=np.uint64))
        return (loc + scale * z).reshape(size)


def _config_ini(path):
    with open(path, 'w') as f:
        f.write('[model parameters]\ntau_tot=1000000.0\nimp_cnc=0e-9\nrho_snw = 300\n'
                'rho_ice = 917\n\n[plot options]\nflg_crt=1\nflg_3D=999\n\n[data]\n'
                'output_dir=monte_carlo_results\noptics_dir=inputdata\n'
                'fi_imp=mie_sot_ChC90_dns_1317.nc\n')


def run_case(name, spec, outdir):
    _install_stubs()
    sys.dont_write_bytecode = True
    if REFERENCE not in sys.path:
        sys.path.insert(0, REFERENCE)
    from monte_carloMPI import monte_carlo3D as ref

    rho_snw, rho_ice = 300.0, 917.0
    lo, hi = spec.get('table_nm') or ssp.grid_for(spec['wvl0'], spec['half_width'])
    ice = ssp.synthetic_ice_table(spec['rds'], lo, hi, rho_ice)
    imp = ssp.synthetic_impurity_table(lo, hi)
    shape = spec.get('shape', 'sphere')
    if shape != 'sphere':
        imp.ext_cff_mss = imp.ext_cff_mss * (1.0 + 2.0 * (imp.wvl * 1e6 - spec['wvl0']))
    if 'tau_tot' in spec:
        tau_tot = float(spec['tau_tot'])
    else:
        tau_tot = spec['depth_m'] * ssp.ext_cff_mss_sphere(spec['rds'], rho_ice) * rho_snw

    work = tempfile.mkdtemp(prefix='mcgold_')
    old_cwd, old_argv = os.getcwd(), sys.argv
    saved = (np.random.rand, np.random.uniform, np.random.normal)
    replay = Replay(spec['seed'], spec.get('first_photon', 0))
    answers, draws, stokes = [], [], []
    try:
        os.chdir(work)
        sys.argv = ['monte_carlo3D']
        _config_ini('config.ini')
        optics = os.path.join(work, 'optics')
        ssp.write_netcdf(os.path.join(optics, 'mie', 'snicar', ssp.ice_file_name(spec['rds'])), ice)
        ssp.write_netcdf(os.path.join(optics, 'mie', 'snicar', 'imp.nc'), imp, with_asm=False)
        isca_rows = None
        if shape != 'sphere':
            isca_rows = np.array(ssp.synthetic_isca_rows(ASPH_WVLS, ASPH_RE), dtype=np.float64)
            isca = ssp.isca_path(optics, shape, spec['roughness'], spec['wvl0'])
            ssp.write_isca(isca, isca_rows)
            if not spec.get('hg', True):
                ssp.write_phase_matrix(os.path.dirname(isca), PHASE_THETA,
                                       ssp.synthetic_phase_rows(isca_rows, PHASE_THETA))
            # what the library walks: this package's reader of the same file
            ice, re_sel = ssp.aspherical_table(isca, spec['wvl0'], spec['rds'], rho_ice)
            isca_rows = ssp.read_isca(isca)
        model = ref.MonteCarlo(tau_tot=tau_tot, imp_cnc=spec.get('imp_cnc', 0.0),
                               rho_snw=rho_snw, rho_ice=rho_ice,
                               output_dir=os.path.join(work, 'out'), optics_dir=optics,
                               fi_imp='imp.nc', HG=shape != 'sphere' and spec.get('hg', True))
        for k, v in spec.get('test', {}).items():
            setattr(model, k, v)

        orig_walk = ref.MonteCarlo.monte_carlo3D
        orig_init = ref.MonteCarlo.initial_pdfs

        def walk(self, wvl):
            replay.photon, replay.k = replay.first + self.photon, 3
            out = orig_walk(self, wvl)
            answers.append(out[:7])
            stokes.append([float(x) for x in np.asarray(out[7]).ravel()[:4]])
            draws.append(replay.k)
            replay.photon = None
            return out

        def init(self, wvls, RANDOM_NUMBERS=1):
            replay.initial_calls = 0
            try:
                return orig_init(self, wvls, RANDOM_NUMBERS)
            finally:
                replay.initial_calls = None

        ref.MonteCarlo.monte_carlo3D = walk
        ref.MonteCarlo.initial_pdfs = init
        np.random.rand, np.random.uniform, np.random.normal = replay.rand, replay.uniform, replay.normal
        np.set_printoptions(legacy='1.25')
        try:
            model.run(spec['n_photon'], spec['wvl0'], spec['half_width'], spec['rds'],
                      theta_0=spec['theta0'], test=bool(spec.get('test')),
                      shape=shape, roughness=spec.get('roughness', 'smooth'),
                      stokes_params=np.array(spec.get('stokes', (1, 0, 0, 0))),
                      Lambertian_surface=spec.get('lam_surface', False),
                      Lambertian_bottom=spec['lam_bottom'],
                      Lambertian_reflectance=spec['R'])
        finally:
            ref.MonteCarlo.monte_carlo3D = orig_walk
            ref.MonteCarlo.initial_pdfs = orig_init
            np.random.rand, np.random.uniform, np.random.normal = saved
            np.set_printoptions(legacy=False)
        out_dir = os.path.join(work, 'out', 'sphere')
        if shape != 'sphere':
            out_dir = os.path.join(work, 'out', ssp.SHAPE_DIRS[shape], ssp.ROUGHNESS_DIRS[spec['roughness']])
        outs = os.listdir(out_dir)
        assert len(outs) == 1, outs
        csv_name = outs[0]
        with open(os.path.join(out_dir, csv_name), 'rb') as f:
            csv_bytes = f.read()
    finally:
        os.chdir(old_cwd)
        sys.argv = old_argv
        shutil.rmtree(work, ignore_errors=True)

    a = np.array([[float(np.asarray(x).ravel()[0]) for x in row] for row in answers],
                 dtype=np.float64)
    rec = dict(
        condition=a[:, 0].astype(np.int32), wvn=a[:, 1], theta_n=a[:, 2], phi_n=a[:, 3],
        n_scat=a[:, 4].astype(np.int32), path_length=a[:, 5], snow_depth=a[:, 6],
        n_draws=np.array(draws, dtype=np.int64))
    params = dict(n_photon=spec['n_photon'], first_photon=spec.get('first_photon', 0), wvl0=spec['wvl0'], half_width=spec['half_width'],
                  rds=spec['rds'], theta0=spec['theta0'], tau_tot=tau_tot,
                  imp_cnc=spec.get('imp_cnc', 0.0), rho_snw=rho_snw, rho_ice=rho_ice,
                  lam_surface=int(spec.get('lam_surface', False)),
                  lam_bottom=int(spec['lam_bottom']), R=spec['R'], seed=spec['seed'],
                  ssa_ice_override=spec.get('test', {}).get('ssa_ice', np.nan),
                  g_override=spec.get('test', {}).get('g', np.nan))
    extra = {}
    if shape != 'sphere':
        params.update(ssp_nearest=1, rds_selected=re_sel)
        extra = dict(ice_unit=np.asarray(ice.wvl_unit), isca_rows=isca_rows,
                     shape=np.asarray(shape), roughness=np.asarray(spec['roughness']))
    if not spec.get('hg', True):
        params.update(polarised=1)
        extra.update(stokes0=np.array(spec['stokes'], dtype=np.float64),
                     stokes=np.array(stokes, dtype=np.float64),
                     phase_theta=np.array(PHASE_THETA, dtype=np.float64),
                     phase_stored=np.array(ssp.synthetic_phase_rows(isca_rows, PHASE_THETA)))
    np.savez_compressed(
        os.path.join(outdir, name + '.npz'),
        **rec, **{'param_' + k: np.asarray(v) for k, v in params.items()},
        ice_wvl=ice.wvl, ice_ssa=ice.ss_alb, ice_ext=ice.ext_cff_mss, ice_asm=ice.asm_prm,
        imp_wvl=imp.wvl, imp_ssa=imp.ss_alb, imp_ext=imp.ext_cff_mss,
        csv_name=np.asarray(csv_name), **extra)
    if spec.get('csv'):
        with open(os.path.join(outdir, name + '.csv'), 'wb') as f:
            f.write(csv_bytes)
    counts = np.bincount(rec['condition'], minlength=6)
    print('%-8s n=%d conditions=%s mean n_scat=%.1f max=%d file=%s' % (
        name, spec['n_photon'], counts[1:].tolist(), rec['n_scat'].mean(),
        rec['n_scat'].max(), csv_name))


def main(argv):
    global REFERENCE
    if argv[:1] == ['--reference']:
        REFERENCE, argv = argv[1], argv[2:]
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, 'monte_carloMPI')):
        sys.exit('name the reference checkout: --reference <dir> or MC_REFERENCE=<dir>')
    names = argv or list(CASES)
    for name in names:
        run_case(name, CASES[name], HERE)


if __name__ == '__main__':
    main(sys.argv[1:])
