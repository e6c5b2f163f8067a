"""SSP tables (synthetic and netCDF) and config.ini handling."""
import numpy as np

from monte_carlompi_gb300 import ssp
from monte_carlompi_gb300.config import read_model_args, WalkConfig

REFERENCE_CONFIG_INI = """; Set model kwargs here by editing the listed values below:

[model parameters]
; snow optical depth
tau_tot=1000000.0

; mass concentration of impurity [mIMP/(mIMP+mICE)]
imp_cnc=0e-9

; snow density (kg/m3, only needed if flg_crt=1)
rho_snw = 300

; ice density (kg/m3)
rho_ice = 917

[plot options]
flg_crt=1
flg_3D=999

[data]
output_dir=monte_carlo_results
optics_dir=inputdata
fi_imp=mie_sot_ChC90_dns_1317.nc
"""


def test_synthetic_formulas():
    t = ssp.synthetic_ice_table(100.0, 1200, 1400)
    assert t.wvl.size == 201
    assert np.isclose(t.ext_cff_mss[0], 16.357688113413303)
    assert np.allclose(1 - t.ss_alb[[0, 200]], [1e-4, 1e-4 * 100 ** 0.5])
    assert np.all(t.asm_prm == 0.89)
    big = ssp.synthetic_ice_table(1500.0, 1700, 1800)
    assert np.all(1 - big.ss_alb <= 0.5) and np.any(1 - big.ss_alb == 0.5)


def test_netcdf_round_trip(tmp_path):
    t = ssp.synthetic_ice_table(250.0, 1400, 1700)
    p = str(tmp_path / 'mie' / 'snicar' / ssp.ice_file_name(250.0))
    ssp.write_netcdf(p, t)
    r = ssp.read_netcdf(p)
    for k in ('wvl', 'ss_alb', 'ext_cff_mss', 'asm_prm'):
        assert np.array_equal(getattr(r, k), getattr(t, k))
    imp = ssp.synthetic_impurity_table(1400, 1700)
    ssp.write_netcdf(str(tmp_path / 'mie' / 'snicar' / 'imp.nc'), imp, with_asm=False)
    a, b = ssp.load_tables(str(tmp_path), 250.0, 'imp.nc')
    assert np.array_equal(b.ss_alb, imp.ss_alb) and np.all(b.asm_prm == 0)
    assert ssp.ice_file_name(100.0) == 'ice_wrn_0100.nc'


def test_config_ini(tmp_path):
    p = tmp_path / 'config.ini'
    p.write_text(REFERENCE_CONFIG_INI)
    a = read_model_args(str(p))
    assert a['tau_tot'] == 1e6 and a['imp_cnc'] == 0 and a['rho_snw'] == 300
    assert a['optics_dir'] == 'inputdata' and a['fi_imp'] == 'mie_sot_ChC90_dns_1317.nc'
    assert read_model_args(str(tmp_path / 'missing.ini'))['rho_ice'] == 917.0


def test_walk_config_c_layout():
    c = WalkConfig(n_photon=5, wvl0=1.3, half_width=0.085, first_photon=7).to_c()
    assert c.n_photon == 5 and c.first_photon == 7 and abs(c.wvl0 - 1.3) < 1e-15
    assert np.isnan(c.g_override)
