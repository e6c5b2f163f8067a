"""The reference-shaped API end to end on the GPU: MonteCarlo(...).run writes the
per-photon CSV the reference writes."""
import os

import numpy as np
import pytest

from monte_carlompi_gb300 import csv_io, ssp
from monte_carlompi_gb300.monte_carlo import MonteCarlo
from tests.conftest import GOLDEN, load_golden
from tests.helpers import compare_replay, golden_tables

pytestmark = pytest.mark.gpu


def _write_tables(optics, g, rds):
    from tests.helpers import golden_tables
    ice, imp = golden_tables(g)
    base = os.path.join(optics, 'mie', 'snicar')
    ssp.write_netcdf(os.path.join(base, ssp.ice_file_name(rds)), ice)
    ssp.write_netcdf(os.path.join(base, 'imp.nc'), imp, with_asm=False)


def test_run_aspherical_hg_reproduces_reference_csv(tmp_path, monkeypatch, capsys):
    """run(shape=..., HG=True) on the same isca.dat rows and impurity table: the file
    lands where the reference writes it (shape and roughness directories, named with
    the selected effective radius) and holds the reference's photons."""
    g = load_golden('asph')
    p = lambda k: g['param_' + k].item()  # noqa: E731
    monkeypatch.chdir(tmp_path)
    optics = str(tmp_path / 'optics')
    shape, rough = str(g['shape']), str(g['roughness'])
    ssp.write_isca(ssp.isca_path(optics, shape, rough, p('wvl0')), g['isca_rows'])
    _, imp = golden_tables(g)
    ssp.write_netcdf(os.path.join(optics, 'mie', 'snicar', 'imp.nc'), imp, with_asm=False)
    mc = MonteCarlo(tau_tot=p('tau_tot'), imp_cnc=p('imp_cnc'), rho_snw=p('rho_snw'),
                    rho_ice=p('rho_ice'), output_dir=str(tmp_path / 'out'), optics_dir=optics,
                    fi_imp='imp.nc', ssp='file', mode='replay64', seed=int(p('seed')), HG=True)
    mc.run(int(p('n_photon')), p('wvl0'), p('half_width'), p('rds'), theta_0=p('theta0'),
           shape=shape, roughness=rough, Lambertian_bottom=bool(p('lam_bottom')),
           Lambertian_reflectance=p('R'))
    printed = capsys.readouterr().out.strip()
    assert printed.endswith(os.path.join(ssp.SHAPE_DIRS[shape], ssp.ROUGHNESS_DIRS[rough],
                                         str(g['csv_name'])))
    assert mc.snow_effective_radius == p('rds_selected')
    got = csv_io.read_csv(printed)
    compare_replay(got, g)
    compare_replay(got, csv_io.read_csv(os.path.join(GOLDEN, 'asph.csv')))


def test_run_polarised_reproduces_reference_csv(tmp_path, monkeypatch, capsys):
    """run(shape=...) with HG off: the polarised walk on the same isca.dat and
    P11.dat ... P44.dat; the file (name appendix I%d%d%d%d, Q_n U_n V_n columns)
    holds the reference's photons and Stokes vectors."""
    g = load_golden('pol')
    p = lambda k: g['param_' + k].item()  # noqa: E731
    monkeypatch.chdir(tmp_path)
    optics = str(tmp_path / 'optics')
    shape, rough = str(g['shape']), str(g['roughness'])
    isca = ssp.isca_path(optics, shape, rough, p('wvl0'))
    ssp.write_isca(isca, g['isca_rows'])
    ssp.write_phase_matrix(os.path.dirname(isca), g['phase_theta'], list(g['phase_stored']))
    _, imp = golden_tables(g)
    ssp.write_netcdf(os.path.join(optics, 'mie', 'snicar', 'imp.nc'), imp, with_asm=False)
    mc = MonteCarlo(tau_tot=p('tau_tot'), imp_cnc=p('imp_cnc'), rho_snw=p('rho_snw'),
                    rho_ice=p('rho_ice'), output_dir=str(tmp_path / 'out'), optics_dir=optics,
                    fi_imp='imp.nc', ssp='file', mode='replay64', seed=int(p('seed')))
    mc.run(int(p('n_photon')), p('wvl0'), p('half_width'), p('rds'), theta_0=p('theta0'),
           stokes_params=g['stokes0'], shape=shape, roughness=rough,
           Lambertian_bottom=bool(p('lam_bottom')), Lambertian_reflectance=p('R'))
    printed = capsys.readouterr().out.strip()
    assert printed.endswith(os.path.join(ssp.SHAPE_DIRS[shape], ssp.ROUGHNESS_DIRS[rough],
                                         str(g['csv_name'])))
    got = csv_io.read_csv(printed)
    compare_replay(got, g)
    ref = csv_io.read_csv(os.path.join(GOLDEN, 'pol.csv'))
    for k in ('stokes_q', 'stokes_u', 'stokes_v'):
        assert np.abs(got[k] - ref[k]).max() < 1e-10


@pytest.mark.parametrize('name', ['cfg1', 'cfg2', 'cfg1_10k'])
def test_run_replay_reproduces_reference_csv(tmp_path, monkeypatch, capsys, name):
    """Same tables, same replay stream: the CSV holds the reference's photons.  cfg1_10k
    is config 1 at the driver's 10,000 packets (monte_carlo3D-run.py:18): all its rows
    match the reference's answers, and its first 1,000 rows match the reference's own
    CSV of cfg1."""
    g = load_golden(name)
    p = lambda k: g['param_' + k].item()  # noqa: E731
    monkeypatch.chdir(tmp_path)
    _write_tables(str(tmp_path / 'optics'), g, p('rds'))
    mc = MonteCarlo(tau_tot=p('tau_tot'), imp_cnc=p('imp_cnc'), rho_snw=p('rho_snw'),
                    rho_ice=p('rho_ice'), output_dir=str(tmp_path / 'out'),
                    optics_dir=str(tmp_path / 'optics'), fi_imp='imp.nc', ssp='file',
                    mode='replay64', seed=int(p('seed')))
    mc.run(int(p('n_photon')), p('wvl0'), p('half_width'), p('rds'), theta_0=p('theta0'),
           Lambertian_bottom=bool(p('lam_bottom')), Lambertian_reflectance=p('R'))
    printed = capsys.readouterr().out.strip()
    assert os.path.basename(printed) == str(g['csv_name'])
    got = csv_io.read_csv(printed)
    compare_replay(got, g)
    text = open(printed, 'rb').read()
    assert text.startswith(csv_io.HEADER.encode())
    assert text.count(b'\n') == int(p('n_photon')) + 1
    ref_csv = os.path.join(GOLDEN, name + '.csv')
    if os.path.exists(ref_csv):
        compare_replay(got, csv_io.read_csv(ref_csv))
    else:
        first = {k: v[:1000] for k, v in got.items()}
        compare_replay(first, csv_io.read_csv(os.path.join(GOLDEN, 'cfg1.csv')))


def test_run_f32_synthetic_and_albedo(tmp_path, monkeypatch, capsys):
    monkeypatch.chdir(tmp_path)
    mc = MonteCarlo(tau_tot=196.29, output_dir=str(tmp_path / 'out'), ssp='synthetic', seed=5)
    mc.run(20000, 1.55, 0.085, 250.0, theta_0=60.0, Lambertian_reflectance=0.5)
    path = capsys.readouterr().out.strip()
    d = csv_io.read_csv(path)
    assert d['condition'].size == 20000
    assert set(np.unique(d['condition'])) <= {1, 2, 3, 4}
    a = mc.calculate_albedo()
    t = mc.tallies[0]
    q = t['q_cond_fx'].astype(np.float64)
    assert abs(a - q[1] / q[1:].sum()) < 1e-5
    assert 0.2 < a < 0.9


def test_run_test_mode_overrides(tmp_path, monkeypatch):
    """run(test=True) uses ssa_ice / g set on the instance (the KAT set-up)."""
    monkeypatch.chdir(tmp_path)
    mc = MonteCarlo(tau_tot=2.0, imp_cnc=0, output_dir=str(tmp_path / 'o'), ssp='synthetic',
                    seed=3, write_csv=False)
    mc.ssa_ice = 0.9
    mc.g = 0.75
    mc.run(200000, 0.5, 0.085, 100, test=True, Lambertian_bottom=False)
    t = mc.tallies[0]
    n = int(t['n_cond'][1:].sum())
    assert abs(int(t['n_cond'][1]) / n - 0.09739) < 4 * np.sqrt(0.0974 * 0.9026 / n)


def test_missing_inputs_and_unsupported_paths_raise(tmp_path, monkeypatch):
    """Aspherical runs need the database files; debug trajectories (matplotlib) are not
    built; in HG mode the Stokes vector is carried but never changes, as in the
    reference (its CSV has no Stokes columns)."""
    monkeypatch.chdir(tmp_path)
    mc = MonteCarlo(output_dir=str(tmp_path), ssp='synthetic', write_csv=False,
                    optics_dir=str(tmp_path / 'none'))
    with pytest.raises(FileNotFoundError):
        mc.run(10, 1.3, 0.085, 100, shape='droxtal')            # polarised: isca.dat missing
    with pytest.raises(NotImplementedError):
        mc.run(10, 1.3, 0.085, 100, debug=True)
    with pytest.raises(ValueError):
        mc.run(10, 1.3, 0.085, 100, stokes_params=np.array([1, 0, 0]))
    mc.run(10, 1.3, 0.085, 100, stokes_params=np.array([1, 1, 0, 0]))
    assert mc.records.size == 10
    with pytest.raises(FileNotFoundError):
        MonteCarlo(output_dir=str(tmp_path), ssp='file', optics_dir=str(tmp_path / 'none'),
                   write_csv=False).run(10, 1.3, 0.085, 100)
