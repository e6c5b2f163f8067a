"""Run configuration: the driver's parameters as a dataclass, and config.ini.

``WalkConfig`` holds exactly what one ``MonteCarlo.run`` call of the reference
uses (monte_carlo3D.py:1492-1496 plus the model kwargs of :43-94) and maps
one-to-one onto the C struct ``mcw_config``.  ``read_model_args`` reads the
reference's ``config.ini`` keys (monte_carloMPI/config.ini; parsed at
monte_carlo3D.py:1778-1806).
"""
import configparser
import ctypes
import math
import os
from dataclasses import dataclass, field, asdict

from . import _abi

# defaults of monte_carloMPI/config.ini
MODEL_DEFAULTS = dict(tau_tot=1000000.0, imp_cnc=0e-9, rho_snw=300.0, rho_ice=917.0,
                      rsensor=None, hsensor=None, flg_crt=1, flg_3D=999,
                      output_dir='monte_carlo_results', optics_dir='inputdata',
                      fi_imp='mie_sot_ChC90_dns_1317.nc', HG=False, phase_functions=False)


def read_model_args(path='config.ini'):
    """Model kwargs from a config.ini (missing file or keys keep the defaults)."""
    args = dict(MODEL_DEFAULTS)
    if not os.path.exists(path):
        return args
    cp = configparser.ConfigParser()
    cp.read(path)
    get = {
        'tau_tot': ('model parameters', cp.getfloat), 'imp_cnc': ('model parameters', cp.getfloat),
        'rho_snw': ('model parameters', cp.getfloat), 'rho_ice': ('model parameters', cp.getfloat),
        'flg_crt': ('plot options', cp.getint), 'flg_3D': ('plot options', cp.getint),
        'output_dir': ('data', cp.get), 'optics_dir': ('data', cp.get), 'fi_imp': ('data', cp.get),
    }
    for key, (section, fn) in get.items():
        if cp.has_option(section, key):
            args[key] = fn(section, key)
    return args


@dataclass
class WalkConfig:
    """One MonteCarlo.run: photons, incident beam, slab and bottom boundary."""
    n_photon: int
    wvl0: float                      # centre wavelength [um]
    half_width: float                # FWHM [um]
    theta0_deg: float = 0.0
    tau_tot: float = 1000000.0
    imp_cnc: float = 0.0
    rho_snw: float = 300.0
    rho_ice: float = 917.0
    lambertian_reflectance: float = 1.0
    lambertian_surface: bool = False
    lambertian_bottom: bool = True
    ice_table: int = 0
    ssa_ice_override: float = math.nan
    g_override: float = math.nan
    ext_ice_override: float = math.nan
    ssa_imp_override: float = math.nan
    ext_imp_override: float = math.nan
    first_photon: int = 0            # first photon index (a shard of a larger run)
    ssp_nearest: bool = False        # HG-forced aspherical lookup: nearest table point, wavelength replaced
    polarised: bool = False          # polarised walk of aspherical grains (phase matrices, mode 'pol64')
    stokes0: tuple = (1.0, 0.0, 0.0, 0.0)  # incident Stokes vector of the polarised walk
    rds_snw: float = field(default=math.nan)  # grain size [um], bookkeeping (selects the table)

    def to_c(self):
        return _abi.ConfigC(int(self.n_photon), int(self.first_photon), float(self.wvl0), float(self.half_width),
                            float(self.theta0_deg), float(self.tau_tot), float(self.imp_cnc),
                            float(self.rho_snw), float(self.rho_ice),
                            float(self.lambertian_reflectance), int(bool(self.lambertian_surface)),
                            int(bool(self.lambertian_bottom)), int(self.ice_table),
                            int(bool(self.ssp_nearest)),
                            float(self.ssa_ice_override), float(self.g_override),
                            float(self.ext_ice_override), float(self.ssa_imp_override),
                            float(self.ext_imp_override), int(bool(self.polarised)), 0,
                            (ctypes.c_double * 4)(*[float(x) for x in self.stokes0]))

    def as_dict(self):
        return asdict(self)


def configs_to_c(configs):
    arr = (_abi.ConfigC * len(configs))()
    for i, c in enumerate(configs):
        arr[i] = c.to_c()
    return arr


def tau_from_depth(depth_m, ext_cff_mss, rho_snw):
    """Optical depth of a slab of depth ``depth_m`` (tau = depth * ext_cff_mss * rho_snw)."""
    return depth_m * ext_cff_mss * rho_snw
