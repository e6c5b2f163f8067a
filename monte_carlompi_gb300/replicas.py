"""Photon-range sharding across independent replicas (one process per GPU).

The reference splits the photon wavelengths over MPI ranks with
``np.array_split`` (parallelize.py:14-15, :28-38) and gathers the per-photon
answers to rank 0 in rank order (parallelize.py:17-26, monte_carlo3D.py:
1845-1847).  Here each replica walks a contiguous photon range of every
config (``first_photon``/``n_photon``); because a photon's random streams are
keyed by its index, the concatenated shards equal the single-GPU run exactly.
The only exchange is the final gather: records concatenated per config in
rank order, tallies summed.
"""
import dataclasses

import numpy as np


def share(n, rank, world):
    """(start, length) of rank's share of n items, np.array_split order."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError('need 0 <= rank < world')
    base, extra = divmod(int(n), world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def shard_configs(configs, rank, world):
    """This rank's share of every config (first_photon / n_photon adjusted)."""
    out = []
    for c in configs:
        start, length = share(c.n_photon, rank, world)
        out.append(dataclasses.replace(c, first_photon=c.first_photon + start, n_photon=length))
    return out


def merge_records(parts, configs, world):
    """Rank-ordered record arrays (each config-major) -> records of the whole run."""
    chunks = []
    offsets = [np.cumsum([0] + [share(c.n_photon, r, world)[1] for c in configs]) for r in range(world)]
    for ci in range(len(configs)):
        for r in range(world):
            lo, hi = offsets[r][ci], offsets[r][ci + 1]
            chunks.append(parts[r][lo:hi])
    return np.concatenate(chunks) if chunks else parts[0][:0]


def merge_tallies(parts):
    """Sum per-config tallies of several replicas (max for max_n_scat)."""
    out = parts[0].copy()
    for p in parts[1:]:
        for name in out.dtype.names:
            if name == 'max_n_scat':
                out[name] = np.maximum(out[name], p[name])
            elif name != 'reserved':
                out[name] = out[name] + p[name]
    return out
