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


def test_aspherical_table_selects_like_the_reference():
    """get_aspherical_SSPs (HG-forced): the reference's own run on these isca.dat rows
    (tests/golden/asph.npz) selected RE = 120 um and gave each photon the nearest
    tabulated wavelength; the reader picks the same rows, k_ext = 1e6 G Q / (rho_ice V)."""
    from tests.conftest import load_golden
    g = load_golden('asph')
    rows = g['isca_rows']
    t = ssp.SSPTable(g['ice_wvl'], g['ice_ssa'], g['ice_ext'], g['ice_asm'], wvl_unit=ssp.WVL_MICRONS)
    assert g['param_rds_selected'].item() == 120.0
    assert '_120.0_' in str(g['csv_name'])
    # every photon's wavelength is a row of the selected size (wvn = 1 / that wavelength)
    assert np.all(np.isin(np.round(1.0 / g['wvn'], 12), np.round(t.wvl, 12)))
    sel = rows[np.isclose(0.75 * rows[:, 2] / rows[:, 3], 120.0)]
    assert np.array_equal(t.wvl, np.sort(sel[:, 0]))
    ext = (1e6 * sel[:, 3] * sel[:, 4]) / (917.0 * sel[:, 2])
    assert np.array_equal(t.ext_cff_mss, ext[np.argsort(sel[:, 0])])


def test_aspherical_reader_round_trip_and_errors(tmp_path):
    rows = ssp.synthetic_isca_rows([1.0, 1.05, 1.1, 1.3, 1.7], [50.0, 200.0])
    p = ssp.isca_path(str(tmp_path), 'droxtal', 'severely rough', 1.3)
    assert p.endswith('ice_optics/0.2-15.25/droxtal/Rough050/isca.dat')
    assert ssp.isca_path('o', 'hexagonal plate', 'smooth', 20.0).endswith(
        '16.4-99.0/plate/Rough000/isca.dat')
    ssp.write_isca(p, rows)
    assert np.array_equal(ssp.read_isca(p), np.array(rows))
    t, re = ssp.aspherical_table(p, 1.3, 150.0)
    assert abs(re - 200.0) < 1e-9 and t.wvl_unit == ssp.WVL_MICRONS and t.wvl.size == 5
    t, re = ssp.aspherical_table(p, 1.3, 110.0)   # nearer to 50 than to 200
    assert abs(re - 50.0) < 1e-9
    import pytest
    with pytest.raises(ValueError):
        ssp.aspherical_table(p, 1.31, 150.0)      # wvl0 must be a tabulated wavelength
    with pytest.raises(ValueError):
        ssp.isca_path('o', 'sphere', 'smooth', 1.3)
    with pytest.raises(ValueError):
        ssp.isca_path('o', 'droxtal', 'smooth', 15.8)


def test_walk_config_nearest_flag_in_c_layout():
    c = WalkConfig(n_photon=5, wvl0=1.3, half_width=0.085, ssp_nearest=True).to_c()
    assert c.ssp_nearest == 1 and c.ice_table == 0
