"""Replica sharding across ranks (world size 2, gloo on CPU): the shards of a
run, walked independently and gathered, equal the whole run."""
import os
import sys

import numpy as np
import pytest

from monte_carlompi_gb300 import replicas
from tests.conftest import ROOT


def test_share_matches_array_split():
    for n in (0, 1, 7, 10, 1001):
        for world in (1, 2, 3, 8):
            parts = np.array_split(np.arange(n), world)
            for r in range(world):
                s, l = replicas.share(n, r, world)
                assert np.array_equal(np.arange(s, s + l), parts[r])


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from oracle import oracle
    from monte_carlompi_gb300.config import WalkConfig
    from tests.conftest import load_golden
    from tests.helpers import golden_tables
    dist.init_process_group('gloo', rank=rank, world_size=world)
    g = load_golden('thin')
    ice, imp = golden_tables(g)
    full = WalkConfig(n_photon=1001, wvl0=1.55, half_width=0.085, theta0_deg=60.0,
                      tau_tot=float(g['param_tau_tot']), lambertian_reflectance=0.5)
    mine = replicas.shard_configs([full], rank, world)[0]
    cfg = oracle.make_config(mine.n_photon, mine.wvl0, mine.half_width, mine.theta0_deg,
                             mine.tau_tot, R=mine.lambertian_reflectance)
    rec = oracle.walk(cfg, ice, imp, 42, p0=mine.first_photon,
                      p1=mine.first_photon + mine.n_photon)
    parts = [None] * world
    dist.all_gather_object(parts, rec)
    if rank == 0:
        merged = replicas.merge_records(parts, [full], world)
        np.save(os.path.join(out_dir, 'merged.npy'), merged)
    dist.destroy_process_group()


def test_two_rank_gather_equals_single_run(tmp_path):
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method='spawn')
    merged = np.load(tmp_path / 'merged.npy')
    from oracle import oracle
    from tests.conftest import load_golden
    from tests.helpers import golden_tables
    g = load_golden('thin')
    ice, imp = golden_tables(g)
    cfg = oracle.make_config(1001, 1.55, 0.085, 60.0, float(g['param_tau_tot']), R=0.5)
    whole = oracle.walk(cfg, ice, imp, 42)
    assert np.array_equal(merged, whole)


def test_merge_tallies_sums():
    from monte_carlompi_gb300 import _abi
    a = np.zeros(2, _abi.TALLY)
    b = np.zeros(2, _abi.TALLY)
    a['n_cond'][:, 1] = [3, 4]
    b['n_cond'][:, 1] = [5, 6]
    a['max_n_scat'] = [10, 2]
    b['max_n_scat'] = [7, 9]
    m = replicas.merge_tallies([a, b])
    assert list(m['n_cond'][:, 1]) == [8, 10] and list(m['max_n_scat']) == [10, 9]
