"""Seeded synthetic slice data, identical on the host (numpy) and the device.

Byte b of slice `s` for seed `seed` is byte (b % 8) (little-endian) of
splitmix64(seed*K1 + s*K2 + b//8), so any row can be regenerated
independently, and the CUDA generator (par2cuda_synth_fill) produces the
same bytes for the large benchmark workloads.
"""
from __future__ import annotations

import numpy as np

K1 = np.uint64(0xD1342543DE82EF95)
K2 = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z ^ (z >> np.uint64(30))
    z = z * M1
    z = z ^ (z >> np.uint64(27))
    z = z * M2
    return z ^ (z >> np.uint64(31))


def slice_bytes(seed: int, index: int, nbytes: int) -> np.ndarray:
    """uint8[nbytes] for slice `index`."""
    units = (nbytes + 7) // 8
    with np.errstate(over="ignore"):
        base = np.uint64(seed) * K1 + np.uint64(index) * K2
        z = _mix(base + np.arange(units, dtype=np.uint64))
    return z.view(np.uint8)[:nbytes].copy()


def slices(seed: int, first: int, count: int, nbytes: int) -> np.ndarray:
    """uint8[count, nbytes] for slices first..first+count-1."""
    units = (nbytes + 7) // 8
    with np.errstate(over="ignore"):
        base = (np.uint64(seed) * K1 + (np.uint64(first) + np.arange(count, dtype=np.uint64))[:, None] * K2)
        z = _mix(base + np.arange(units, dtype=np.uint64)[None, :])
    return np.ascontiguousarray(z.view(np.uint8)[:, :nbytes])
