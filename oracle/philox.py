"""Philox4x32-10 and the replay uniform streams, in NumPy.

TEST INFRASTRUCTURE ONLY.  This module is part of the oracle: it is imported by
``tests/``, by the golden-fixture generator under ``tests/golden/`` and by the
CPU-baseline leg of ``bench.py``.  The product (``monte_carlompi_gb300``) never
imports it; the CUDA kernels carry their own Philox.

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11), with the round
multipliers 0xD2511F53 / 0xCD9E8D57 and the Weyl key increments
0x9E3779B9 / 0xBB67AE85 published there.  ``KAT_VECTORS`` holds the published
known-answer vectors of the Random123 distribution for this generator.

Replay stream (shared by the reference harness, the C oracle and the FP64 CUDA
replay kernel).  Key = (seed & 0xffffffff, seed >> 32).  Counter =
(block, tag, photon & 0xffffffff, photon >> 32).  One block yields two
uniforms: uniform ``k`` of a stream uses block ``k >> 1`` and the 64-bit word
``x[2j+1] << 32 | x[2j]`` with ``j = k & 1``.  The double is
``((word >> 12) + 0.5) * 2**-52``, which lies in [2**-53, 1 - 2**-53]: every
value is exact, so it can never round to 0 or 1.

* tag ``TAG_WALK`` (0): the walk's uniforms, in the order the reference draws
  them (monte_carlo3D.py:1035-1038 for k = 0..2, then :915, :921, :1014,
  :1020, :1023 per step, then the Lambertian pairs :1245-1246 and the bottom
  reflection draw :1422/:1453).
* tag ``TAG_WVL`` (1): photon wavelength.  Uniforms 0 and 1 of this stream
  feed one Box-Muller normal ``sqrt(-2 ln u0) * cos(2 pi u1)`` that stands in
  for ``np.random.normal`` at monte_carlo3D.py:1519.
"""
import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
TAG_WALK = 0
TAG_WVL = 1
TWO_PI = 2 * np.pi

# (counter, key, expected output) from the Random123 known-answer file for
# philox4x32 with 10 rounds.
KAT_VECTORS = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]

_MASK = np.uint64(0xFFFFFFFF)
_S32 = np.uint64(32)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10.  All arguments broadcast; returns 4 uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & _MASK for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint64) & _MASK
    k1 = np.asarray(k1, dtype=np.uint64) & _MASK
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & _MASK
            k1 = (k1 + np.uint64(W1)) & _MASK
        p0 = np.uint64(M0) * c0
        p1 = np.uint64(M1) * c2
        c0, c1, c2, c3 = ((p1 >> _S32) ^ c1 ^ k0, p1 & _MASK,
                          (p0 >> _S32) ^ c3 ^ k1, p0 & _MASK)
    return tuple(v.astype(np.uint32) for v in (c0, c1, c2, c3))


def replay_uniform(seed, tag, photon, k):
    """Uniform number ``k`` of stream ``tag`` for ``photon`` (vectorised over photon/k)."""
    seed = int(seed)
    photon = np.asarray(photon, dtype=np.uint64)
    k = np.asarray(k, dtype=np.uint64)
    block = k >> np.uint64(1)
    x0, x1, x2, x3 = philox4x32_10(block, tag, photon & _MASK, photon >> _S32,
                                   seed & 0xFFFFFFFF, seed >> 32)
    odd = (k & np.uint64(1)).astype(bool)
    lo = np.where(odd, x2, x0).astype(np.uint64)
    hi = np.where(odd, x3, x1).astype(np.uint64)
    word = (hi << _S32) | lo
    return ((word >> np.uint64(12)).astype(np.float64) + 0.5) * 2.0 ** -52


def replay_normal(seed, photon):
    """Standard normal of the wavelength stream for each photon (Box-Muller, cos branch)."""
    u0 = replay_uniform(seed, TAG_WVL, photon, 0)
    u1 = replay_uniform(seed, TAG_WVL, photon, 1)
    return np.sqrt(-2.0 * np.log(u0)) * np.cos(TWO_PI * u1)


def replay_wavelengths(seed, n_photon, wvl0, half_width):
    """Photon wavelengths [um] as monte_carlo3D.py:1515-1520 draws them, on the replay stream."""
    scale = half_width / 2.355
    z = replay_normal(seed, np.arange(n_photon, dtype=np.uint64))
    return np.around(wvl0 + scale * z, decimals=2)
