"""Drop-in ``MonteCarlo`` with the reference's constructor and ``run`` signature.

Mirrors monte_carloMPI/monte_carlo3D.py's ``MonteCarlo`` for the
Henyey-Greenstein sphere path:

* ``MonteCarlo(**model_kwargs)`` reads ``config.ini`` from the working
  directory when present, then applies keyword overrides (monte_carlo3D.py:
  43-94).  Command-line arguments are not parsed (a library does not own
  ``sys.argv``).
* ``run(n_photon, wvl0, half_width, rds_snw, theta_0=0., ...)`` walks every
  photon on the GPU through libmcwalk, writes the per-photon CSV under
  ``output_dir/sphere/`` and prints its path, as :1492-1648 do.  It returns
  None like the reference; the records, tallies and stats stay on the
  instance (``records``, ``tallies``, ``stats``, ``output_file``).

Extra keyword arguments (not in the reference): ``device`` (CUDA device),
``seed`` (None draws one from os.urandom, like the reference's unseeded RNG),
``mode`` ('f32' production walk or 'replay64' FP64 replay), ``ssp``
('auto' reads the netCDF tables and falls back to the synthetic tables when
they are missing, 'file' requires them, 'synthetic' never reads them) and
``write_csv`` (False skips the file).

Non-spherical shapes run on the Henyey-Greenstein path when ``HG=True``
(get_aspherical_SSPs, monte_carlo3D.py:173-256, :313-415): the particle size
of ``<optics_dir>/ice_optics/<band>/<shape>/<roughness>/isca.dat`` whose
effective radius is nearest to ``rds_snw``, each photon's wavelength moved to the
nearest tabulated one, no interpolation; the CSV goes under
``output_dir/<shape>/<roughness>/`` named with that effective radius.

Non-spherical shapes without HG take the polarised walk (monte_carlo3D.py:
905-1004, :1282-1342): scattering angles by rejection from the phase matrices
P11.dat ... P44.dat beside isca.dat, the incident ``stokes_params`` carried
through every scattering, the CSV with Q_n, U_n, V_n and the name appendix
'I%d%d%d%d'; ``mode`` 'f32' walks it in FP32 ('pol32'), 'replay64' in FP64 on
the replay stream ('pol64').  (The Yang et al. 2013 files are not part of the
reference archive; any files in their layout work.)

Not available (raise): ``debug`` and ``phase_functions`` (matplotlib figures).
"""
import math
import os
import sys

import numpy as np

from . import csv_io, ssp
from .config import WalkConfig, read_model_args
from .walker import Walker


class MonteCarlo(object):
    def __init__(self, **model_kwargs):
        args = read_model_args('config.ini')
        extras = dict(device=0, seed=None, mode='f32', ssp='auto', write_csv=True)
        for k, v in model_kwargs.items():
            if k in extras:
                extras[k] = v
            else:
                args[k] = v
        for k, v in args.items():
            setattr(self, k, v)
        self.device = extras['device']
        self.seed = extras['seed']
        self.mode = extras['mode']
        self.ssp_source = extras['ssp']
        self.write_csv = extras['write_csv']
        if self.mode not in ('f32', 'replay64'):
            raise ValueError("mode must be 'f32' or 'replay64'")
        self._walker = None
        self.records = None
        self.tallies = None
        self.stats = None
        self.output_file = None

    # -- SSP tables (get_optical_properties :498-514, get_impurity_optics :661-671)
    def _imp_table(self, wvl0, half_width):
        imp_path = os.path.join(self.optics_dir, 'mie', 'snicar', self.fi_imp)
        if self.ssp_source == 'file' or (self.ssp_source == 'auto' and os.path.exists(imp_path)):
            return ssp.read_netcdf(imp_path)
        lo, hi = ssp.grid_for(wvl0, half_width)
        return ssp.synthetic_impurity_table(lo, hi)

    def _tables(self, wvl0, half_width, rds_snw):
        base = os.path.join(self.optics_dir, 'mie', 'snicar')
        ice_path = os.path.join(base, ssp.ice_file_name(rds_snw))
        imp_path = os.path.join(base, self.fi_imp)
        have = os.path.exists(ice_path) and os.path.exists(imp_path)
        if self.ssp_source == 'file' or (self.ssp_source == 'auto' and have):
            return ssp.read_netcdf(ice_path), ssp.read_netcdf(imp_path)
        if self.ssp_source == 'auto':
            sys.stderr.write('SSP tables not found under %s; using the synthetic sphere '
                             'tables\n' % base)
        lo, hi = ssp.grid_for(wvl0, half_width)
        return (ssp.synthetic_ice_table(rds_snw, lo, hi, self.rho_ice),
                ssp.synthetic_impurity_table(lo, hi))

    def _overrides(self, test):
        ov = {}
        if test:  # run(test=True) broadcasts attributes set on the instance (:1553-1573)
            for attr, key in (('ssa_ice', 'ssa_ice_override'), ('g', 'g_override'),
                              ('ext_cff_mss_ice', 'ext_ice_override'),
                              ('ssa_imp', 'ssa_imp_override'),
                              ('ext_cff_mss_imp', 'ext_imp_override')):
                v = getattr(self, attr, None)
                if v is not None and np.ndim(v) == 0:
                    ov[key] = float(v)
        return ov

    def walker(self):
        if self._walker is None:
            self._walker = Walker(self.device)
        return self._walker

    def run(self, n_photon, wvl0, half_width, rds_snw, theta_0=0.,
            stokes_params=np.array([1, 0, 0, 0]), shape='sphere', roughness='smooth', test=False,
            debug=False, Lambertian_surface=False, Lambertian_bottom=True,
            Lambertian_reflectance=1.):
        """Walk n_photon photons and write the per-photon CSV.  ALL VALUES IN MICRONS."""
        polarised = shape != 'sphere' and not self.HG
        stokes_params = np.asarray(stokes_params, dtype=np.float64)
        if stokes_params.shape != (4,):
            raise ValueError('stokes_params must hold I, Q, U, V')
        if debug:
            raise NotImplementedError('debug trajectories are matplotlib figures')
        if self.phase_functions:
            raise NotImplementedError('phase-function plots are matplotlib figures')
        self.Lambertian_surface = Lambertian_surface
        self.Lambertian_bottom = Lambertian_bottom
        self.R_Lambertian = Lambertian_reflectance
        self.theta_0 = (np.pi * theta_0) / 180.
        self.shape = shape
        self.roughness = roughness
        self.wvl0 = wvl0
        self.snow_effective_radius = rds_snw

        if shape == 'sphere':
            ice, imp = self._tables(wvl0, half_width, rds_snw)
            subdir = ('sphere',)
        else:
            path = ssp.isca_path(self.optics_dir, shape, roughness, wvl0)
            ice, self.snow_effective_radius = ssp.aspherical_table(path, wvl0, rds_snw, self.rho_ice)
            imp = self._imp_table(wvl0, half_width)
            self.shape_dir = ssp.SHAPE_DIRS[shape]
            self.roughness_dir = ssp.ROUGHNESS_DIRS[roughness]
            subdir = (self.shape_dir, self.roughness_dir)
        self.initial_stokes_params = stokes_params
        w = self.walker()
        w.set_tables([ice], imp)
        if polarised:
            w.set_phase_matrices([ssp.aspherical_phase_table(path, ice, wvl0)])
        cfg = WalkConfig(n_photon=int(n_photon), wvl0=float(wvl0), half_width=float(half_width),
                         theta0_deg=float(theta_0), tau_tot=float(self.tau_tot),
                         imp_cnc=float(self.imp_cnc), rho_snw=float(self.rho_snw),
                         rho_ice=float(self.rho_ice),
                         lambertian_reflectance=float(Lambertian_reflectance),
                         lambertian_surface=bool(Lambertian_surface),
                         lambertian_bottom=bool(Lambertian_bottom),
                         rds_snw=float(self.snow_effective_radius), ssp_nearest=shape != 'sphere',
                         polarised=polarised, stokes0=tuple(float(x) for x in stokes_params),
                         **self._overrides(test))
        seed = self.seed
        if seed is None:
            seed = int.from_bytes(os.urandom(8), 'little')
        self.last_seed = seed
        mode = self.mode
        if polarised:
            mode = 'pol32' if self.mode == 'f32' else 'pol64'
        res = w.walk([cfg], seed, mode=mode, records='host')
        self.records, self.tallies, self.stats = res.records, res.tallies, res.stats
        if self.write_csv:
            appendix = 'I%d%d%d%d' % tuple(stokes_params) if polarised else 'HG'   # :123-130
            path = csv_io.output_path(self.output_dir, wvl0, half_width, self.snow_effective_radius,
                                      n_photon, csv_io.theta0_label(theta_0), subdir=subdir,
                                      appendix=appendix)
            csv_io.write_csv(path, res.records)
            self.output_file = path
            print('%s' % path)
        return None

    def calculate_albedo(self, answers=None):
        """Black-sky albedo Q_up / Q_down (monte_carlo3D.py:1659-1671) of the last run
        (or of ``answers``, a record array)."""
        rec = self.records if answers is None else answers
        wvn = np.asarray(rec['wvn'], dtype=np.float64)
        up = wvn[np.asarray(rec['condition']) == 1].sum()
        down = wvn.sum()
        return up / down if down > 0 else math.nan

    @classmethod
    def flatten_list(klass, l):
        return [item for sublist in l for item in sublist]
