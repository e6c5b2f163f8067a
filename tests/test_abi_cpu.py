"""The C ABI library without a GPU: it loads, exports exactly what include/mcwalk.h
declares, struct layouts agree, and the host-only entry points work."""
import ctypes
import os
import re

import numpy as np
import pytest

from monte_carlompi_gb300 import _abi, walker

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name='mcwalk.h'):
    text = open(os.path.join(ROOT, 'include', name)).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(mcw_[a-z_0-9]+)\s*\(', text)))


def test_library_exports_every_declared_symbol():
    declared = header_functions()
    assert sorted(_abi.EXPORTS) == declared
    assert sorted(_abi.MLP_EXPORTS) == header_functions('mcw_mlp.h')
    declared = declared + header_functions('mcw_mlp.h')
    lib = ctypes.CDLL(_abi.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


def test_version():
    L = _abi.load()
    assert L.mcw_abi_version() == 3
    assert b'sm_103a' in L.mcw_version()


def test_bindings_follow_the_header_abi_version():
    """The ctypes bindings state the header's MCW_ABI_VERSION, and loading refuses a
    library of another version (checked when the library is loaded)."""
    hdr = open(os.path.join(os.path.dirname(__file__), '..', 'include', 'mcwalk.h')).read()
    m = re.search(r'#define MCW_ABI_VERSION (\d+)', hdr)
    assert m and int(m.group(1)) == _abi.ABI_VERSION
    for name, value in (('MCW_NOALLOC_MAX_LUT', _abi.NOALLOC_MAX_LUT),
                        ('MCW_DEFAULT_BUDGET_S', _abi.DEFAULT_BUDGET_S),
                        ('MCW_HIST_BINS', _abi.HIST_BINS)):
        m = re.search(r'#define %s ([0-9.]+)' % name, hdr)
        assert m and float(m.group(1)) == value, name


def test_create_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip('a GPU is present')
    except ImportError:
        pass
    h = ctypes.c_void_p()
    rc = _abi.load().mcw_create(0, ctypes.byref(h))
    assert rc in (-1, -2) and not h.value


def test_null_arguments_are_rejected():
    L = _abi.load()
    assert L.mcw_create(0, None) == -1
    assert L.mcw_brf(None, 1, None, None) == -1
    assert L.mcw_destroy(None) == 0
    assert L.mcw_graph_destroy(None) == 0


def test_brf_of_a_lambertian_tally_is_flat():
    """BRF of an isotropic (Lambertian) reflector equals its albedo in every bin."""
    t = np.zeros(1, _abi.TALLY)
    fx = 2 ** 32
    n_down = 10 ** 6
    albedo = 0.4
    # cosine-weighted exits: bin weight ~ sin(theta) cos(theta) dtheta, split over phi
    mids = (np.arange(18) + 0.5) * (np.pi / 36)
    w = np.sin(mids) * np.cos(mids)
    w /= w.sum()
    per_bin = albedo * n_down * np.repeat(w / 36, 36)
    t['bin_wvn_fx'][0] = np.round(per_bin * fx).astype(np.uint64)
    t['q_cond_fx'][0, 1] = int(round(albedo * n_down)) * fx
    t['q_cond_fx'][0, 4] = int(round((1 - albedo) * n_down)) * fx
    brf, alb = walker.brf_from_tallies(t)
    assert abs(alb[0] - albedo) < 1e-12
    assert np.allclose(brf[0], albedo, rtol=1e-6)
