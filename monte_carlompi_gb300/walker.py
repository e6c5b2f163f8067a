"""Python handle on a libmcwalk context (one GPU).

``Walker`` replaces what ``parallelize.Parallel`` and the photon loop of
``MonteCarlo.run`` do in the reference (parallelize.py:6-41,
monte_carlo3D.py:1521-1619): one call walks every photon of one or many
configs on the device and returns per-photon records and per-config tallies.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi
from .config import configs_to_c


# walk modes: (ABI mode, record dtype)
MODES = {'f32': (_abi.MODE_F32, _abi.RECORD32),
         'replay64': (_abi.MODE_REPLAY64, _abi.RECORD64),
         'pol64': (_abi.MODE_POL64, _abi.RECORD64P),
         'pol32': (_abi.MODE_POL32, _abi.RECORD32P)}


def _phase_c(p, keep):
    """mcw_phase_table of a monte_carlompi_gb300.ssp.PhaseTable (None: an empty entry)."""
    c = _abi.PhaseTableC()
    if p is None:
        return c
    cols = [np.ascontiguousarray(a, np.float64) for a in list(p.cos_asc) + list(p.p_asc)]
    ext = [np.ascontiguousarray(a, np.float64) for a in (p.a1, p.a2, p.b1, p.b2)]
    keep.extend(cols + ext)
    c.n_rows = cols[6].shape[0]
    for e in range(6):
        c.n_angle[e] = cols[e].size
        c.cos_asc[e] = cols[e].ctypes.data
        c.p_asc[e] = cols[6 + e].ctypes.data
    c.a1, c.a2, c.b1, c.b2 = (a.ctypes.data for a in ext)
    c.cos_max, c.cos_min, c.cos_cutoff = float(p.cos_max), float(p.cos_min), float(p.cos_cutoff)
    return c


def _table_c(t, keep):
    cols = [np.ascontiguousarray(t.wvl, np.float64), np.ascontiguousarray(t.ss_alb, np.float64),
            np.ascontiguousarray(t.ext_cff_mss, np.float64), np.ascontiguousarray(t.asm_prm, np.float64)]
    keep.extend(cols)
    return _abi.SSPTableC(cols[0].ctypes.data, cols[1].ctypes.data, cols[2].ctypes.data,
                          cols[3].ctypes.data, cols[0].size, int(getattr(t, 'wvl_unit', 0)))


@dataclass
class WalkResult:
    records: object          # numpy structured array (host), device pointer owner, or None
    tallies: np.ndarray      # TALLY structured array, one per config
    stats: dict

    def albedo(self):
        """Q_up / Q_down per config (monte_carlo3D.py:1659-1671, post_processing.py:125-128)."""
        q = self.tallies['q_cond_fx'].astype(np.float64)
        return q[:, 1] / q[:, 1:].sum(axis=1)

    def brf(self):
        """648-bin BRF per config (mcw_brf)."""
        return brf_from_tallies(self.tallies)


def brf_from_tallies(tallies):
    t = np.ascontiguousarray(tallies)
    out = np.zeros((t.shape[0], _abi.HIST_BINS), np.float64)
    alb = np.zeros(t.shape[0], np.float64)
    _abi.check(_abi.load().mcw_brf(t.ctypes.data, t.shape[0], out.ctypes.data, alb.ctypes.data),
               what='mcw_brf')
    return out, alb


class Walker:
    """One context on one device: tables, launch shape, walks."""

    def __init__(self, device=0):
        self._lib = _abi.load()
        h = ctypes.c_void_p()
        rc = self._lib.mcw_create(int(device), ctypes.byref(h))
        _abi.check(rc, what='mcw_create(device=%d) failed: no usable CUDA device?' % device)
        self._ctx = h
        self.device = device
        self._tables_keep = []
        self._cfg_cache = (None, None)   # (field values of the last configs, their C array)

    def close(self):
        if getattr(self, '_ctx', None):
            self._lib.mcw_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._ctx

    def set_tables(self, ice_tables, imp_table):
        keep = []
        ice = (_abi.SSPTableC * len(ice_tables))(*[_table_c(t, keep) for t in ice_tables])
        imp = _table_c(imp_table, keep)
        rc = self._lib.mcw_set_tables(self._ctx, ice, len(ice_tables), ctypes.byref(imp))
        _abi.check(rc, self._ctx)
        self._tables_keep = keep

    def set_launch(self, block_size=256, blocks_per_sm=0, regen_chunk=8, drain_from=None):
        """Launch shape of the FP32 walk; drain_from: once every photon has started, a photon
        past this many steps leaves the walk for a queue walked after it by a whole thread
        block per photon (0 = never, else >= 256; None keeps the current value).  Records do
        not depend on the launch shape."""
        if drain_from is None:
            drain_from = self.get_launch()['drain_from']
        l = _abi.LaunchC(block_size, blocks_per_sm, regen_chunk, drain_from)
        _abi.check(self._lib.mcw_set_launch(self._ctx, ctypes.byref(l)), self._ctx)

    def get_launch(self):
        l = _abi.LaunchC()
        _abi.check(self._lib.mcw_get_launch(self._ctx, ctypes.byref(l)), self._ctx)
        return dict(block_size=l.block_size, blocks_per_sm=l.blocks_per_sm, regen_chunk=l.regen_chunk,
                    drain_from=l.drain_from)

    def set_budget(self, seconds):
        _abi.check(self._lib.mcw_set_budget(self._ctx, float(seconds)), self._ctx)

    def set_phase_matrices(self, tables):
        """Phase matrices of the polarised walk: one ssp.PhaseTable (or None) per ice
        table of the last set_tables, rows in that table's order."""
        keep = []
        arr = (_abi.PhaseTableC * len(tables))(*[_phase_c(t, keep) for t in tables])
        rc = self._lib.mcw_set_phase_matrices(self._ctx, arr, len(tables))
        _abi.check(rc, self._ctx)

    def walk(self, configs, seed, mode='f32', records='host', out=None, device_ptr=None):
        """Walk every photon of ``configs``.

        records: 'host' (returned as a numpy structured array, or written into
        ``out``), 'device' (written to ``device_ptr``, a 16-byte aligned device
        address the caller owns) or None.
        """
        if mode not in MODES:
            raise ValueError('mode must be one of %s' % ', '.join(sorted(MODES)))
        mode_c, dtype = MODES[mode]
        cfg = self._configs_c(configs)
        n = len(configs)
        total = int(sum(max(int(c.n_photon), 0) for c in configs))
        tallies = np.zeros(n, _abi.TALLY)
        stats = _abi.StatsC()
        rec = None
        if records == 'host':
            rec = out if out is not None else np.empty(total, dtype)
            if rec.dtype != dtype or rec.size < total or not rec.flags.c_contiguous:
                raise ValueError('out must be a contiguous %s array of >= %d records' % (dtype, total))
            ptr, where = rec.ctypes.data, _abi.RECORDS_HOST   # (__array_interface__ costs ~8 us here)
        elif records == 'device':
            if device_ptr is None:
                raise ValueError('records="device" needs device_ptr')
            ptr, where = int(device_ptr), _abi.RECORDS_DEVICE
        elif records is None:
            ptr, where = None, _abi.RECORDS_NONE
        else:
            raise ValueError('records must be "host", "device" or None')
        rc = self._lib.mcw_walk(self._ctx, cfg, n, int(seed) & (2 ** 64 - 1), mode_c, ptr, where,
                                tallies.ctypes.data, ctypes.byref(stats))
        _abi.check(rc, self._ctx)
        return WalkResult(rec, tallies, stats.as_dict())

    def _configs_c(self, configs):
        """The configs as a C array; a call on configs with the same field values as
        the previous call reuses its array (the library only reads it)."""
        key = tuple(tuple(vars(c).values()) for c in configs)
        if key != self._cfg_cache[0]:
            self._cfg_cache = (key, configs_to_c(configs))
        return self._cfg_cache[1]

    def autotune(self, configs, seed=1):
        cfg = configs_to_c(configs)
        best = _abi.LaunchC()
        ms = ctypes.c_double()
        rc = self._lib.mcw_autotune(self._ctx, cfg, len(configs), int(seed), ctypes.byref(best),
                                    ctypes.byref(ms))
        _abi.check(rc, self._ctx)
        return dict(block_size=best.block_size, blocks_per_sm=best.blocks_per_sm,
                    regen_chunk=best.regen_chunk, drain_from=best.drain_from, ms=ms.value)

    def graph(self, configs, device_ptr=None):
        return SweepGraph(self, configs, device_ptr)


class SweepGraph:
    """A captured F32 sweep (mcw_graph_*): replay with a new seed per launch."""

    def __init__(self, walker, configs, device_ptr=None):
        self._w = walker
        self._lib = walker._lib
        self.n_cfg = len(configs)
        cfg = configs_to_c(configs)
        h = ctypes.c_void_p()
        rc = self._lib.mcw_graph_create(walker.handle, cfg, self.n_cfg,
                                        None if device_ptr is None else int(device_ptr), ctypes.byref(h))
        _abi.check(rc, walker.handle)
        self._g = h

    def launch(self, seed):
        tallies = np.zeros(self.n_cfg, _abi.TALLY)
        stats = _abi.StatsC()
        rc = self._lib.mcw_graph_launch(self._g, int(seed) & (2 ** 64 - 1), tallies.ctypes.data,
                                        ctypes.byref(stats))
        _abi.check(rc, self._w.handle)
        return WalkResult(None, tallies, stats.as_dict())

    def close(self):
        if getattr(self, '_g', None):
            self._lib.mcw_graph_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
