"""Native CSV writer: the reference's format byte for byte."""
import os

import numpy as np
import pytest

from monte_carlompi_gb300 import _abi, csv_io
from tests.conftest import GOLDEN, load_golden


def _records64(g):
    r = np.zeros(g['condition'].size, _abi.RECORD64P if 'stokes' in g else _abi.RECORD64)
    for k in ('condition', 'n_scat', 'wvn', 'theta_n', 'phi_n', 'path_length', 'snow_depth'):
        r[k] = g[k]
    if 'stokes' in g:
        r['stokes_q'], r['stokes_u'], r['stokes_v'] = g['stokes'][:, 1], g['stokes'][:, 2], g['stokes'][:, 3]
    return r


@pytest.mark.parametrize('name', ['cfg1', 'cfg2', 'asph', 'pol'])
def test_reference_csv_bytes(name, tmp_path):
    g = load_golden(name)
    ref = open(os.path.join(GOLDEN, name + '.csv'), 'rb').read()
    rec = _records64(g)
    assert csv_io.format_csv(rec) == ref
    p = tmp_path / 'x.txt'
    csv_io.write_csv(str(p), rec, n_threads=3)
    assert p.read_bytes() == ref


def test_python_repr_rules():
    rng = np.random.default_rng(3)
    vals = np.concatenate([
        rng.standard_normal(3000) * 10.0 ** rng.integers(-30, 30, 3000),
        [0.0, -0.0, 1e-4, 1e-5, 9.999999999999999e-05, 1e16, 9999999999999998.0, 1e15, 0.1,
         0.5, 1 / 3, 2.0, 123456789.0, 1e-300, 5e-324, 1.7976931348623157e308, 1e22, -1e-7]])
    rec = np.zeros(vals.size, _abi.RECORD64)
    rec['wvn'] = vals
    lines = csv_io.format_csv(rec, header=False).decode().splitlines()
    for v, line in zip(vals, lines):
        assert line.split()[1] == repr(float(v))


def test_float32_rows_round_trip_shortest():
    rng = np.random.default_rng(4)
    vals = (rng.standard_normal(2000) * 10.0 ** rng.integers(-8, 8, 2000)).astype(np.float32)
    rec = np.zeros(vals.size, _abi.RECORD32)
    rec['path_length'] = vals
    lines = csv_io.format_csv(rec, header=False).decode().splitlines()
    for v, line in zip(vals, lines):
        tok = line.split()[5]
        assert np.float32(float(tok)) == v
        # no shorter digit string reads back to the same float
        digits = len(np.format_float_scientific(v, unique=True).split('e')[0].replace('-', '').replace('.', ''))
        mant = tok.split('e')[0].replace('-', '').replace('.', '').lstrip('0').rstrip('0') or '0'
        assert len(mant) <= max(digits, 1)


def test_output_path_naming_and_dedup(tmp_path):
    th = csv_io.theta0_label(60.0)
    p1 = csv_io.output_path(str(tmp_path), 1.55, 0.085, 250.0, 1000, th)
    assert os.path.basename(p1) == '1.55_0.085_250.0_1000_59.99999999999999_HG.txt'
    open(p1, 'w').close()
    p2 = csv_io.output_path(str(tmp_path), 1.55, 0.085, 250.0, 1000, th)
    assert os.path.basename(p2) == '1.55_0.085_250.0_1000_59.99999999999999_HG_1.txt'
    g = load_golden('cfg1')
    assert os.path.basename(csv_io.output_path(str(tmp_path), 1.3, 0.085, 100.0, 1000,
                                               csv_io.theta0_label(0.0))) == str(g['csv_name'])


def test_read_back(tmp_path):
    g = load_golden('cfg2')
    p = tmp_path / 'r.txt'
    csv_io.write_csv(str(p), _records64(g))
    d = csv_io.read_csv(str(p))
    assert np.array_equal(d['condition'], g['condition'])
    assert np.array_equal(d['path_length'], g['path_length'])


def test_polarised_fp32_rows():
    """mcw_record32p: the polarised header and ten columns, each float the shortest
    repr that reads back to the FP32 value (like the FP32 HG records)."""
    rng = np.random.default_rng(7)
    rec = np.zeros(200, _abi.RECORD32P)
    rec['condition'] = rng.integers(1, 6, 200)
    rec['n_scat'] = rng.integers(0, 1000, 200)
    for k in ('wvn', 'theta_n', 'phi_n', 'path_length', 'snow_depth', 'stokes_q', 'stokes_u', 'stokes_v'):
        rec[k] = rng.standard_normal(200).astype(np.float32)
    text = csv_io.format_csv(rec).decode()
    lines = text.splitlines()
    assert lines[0] == ('condition wvn[um^-1] theta_n phi_n n_scat path_length[m], snow_depth[m], '
                        'Q_n, U_n, V_n')
    for r, line in zip(rec, lines[1:]):
        f = line.split()
        assert len(f) == 10 and int(f[0]) == r['condition'] and int(f[4]) == r['n_scat']
        for tok, k in zip(f[1:4] + f[5:], ('wvn', 'theta_n', 'phi_n', 'path_length', 'snow_depth',
                                           'stokes_q', 'stokes_u', 'stokes_v')):
            assert np.float32(float(tok)) == r[k]
            assert tok == repr(float(tok))
