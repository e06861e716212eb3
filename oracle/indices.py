"""Index conversion, restated in numpy (test infrastructure only).

Follows src/compression/indices.hpp:120-186 and src/parameters/parameters.cpp:143-180:
bounds/centering checks, sorted unique stick keys x*dimY+y (storage indices), value index
stick*dimZ+z, and the zero-zero stick position.
"""
from __future__ import annotations

import numpy as np

C2C, R2C = 0, 1


class IndexError_(ValueError):
    """Raised where the reference throws; ``code`` is the SpfftError value."""

    def __init__(self, code: int):
        super().__init__(f"SpfftError {code}")
        self.code = code


INVALID_PARAMETER = 5
INVALID_INDICES = 7


def storage(dim: int, idx: np.ndarray) -> np.ndarray:
    """to_storage_index (indices.hpp:49-55)."""
    return np.where(idx < 0, idx + dim, idx)


def convert(transform_type: int, dx: int, dy: int, dz: int, triplets) -> dict:
    t = np.asarray(triplets, dtype=np.int64).reshape(-1, 3)
    n = t.shape[0]
    if n > dx * dy * dz:
        raise IndexError_(INVALID_PARAMETER)
    herm = transform_type == R2C
    centered = bool(n and (t < 0).any())
    max_x = (dx // 2 + 1 if (herm or centered) else dx) - 1
    max_y = (dy // 2 + 1 if centered else dy) - 1
    max_z = (dz // 2 + 1 if centered else dz) - 1
    min_x = 0 if herm else max_x - dx + 1
    min_y = max_y - dy + 1
    min_z = max_z - dz + 1
    x, y, z = t[:, 0], t[:, 1], t[:, 2]
    if n and ((x < min_x).any() or (x > max_x).any() or (y < min_y).any() or (y > max_y).any()
              or (z < min_z).any() or (z > max_z).any()):
        raise IndexError_(INVALID_INDICES)
    xs, ys, zs = storage(dx, x), storage(dy, y), storage(dz, z)
    keys = xs * dy + ys
    sticks = np.unique(keys)
    stick_of = np.searchsorted(sticks, keys)
    value_idx = stick_of * dz + zs
    zz = int(np.searchsorted(sticks, 0)) if (sticks.size and sticks[0] == 0) else int(sticks.size)
    # parameters.cpp:173-179 counts keys until key == 0: sticks are sorted and non-negative, so
    # key 0 can only be first.
    return {
        "value_indices": value_idx.astype(np.int64),
        "stick_keys": sticks.astype(np.int64),
        "zero_zero_stick": zz,
        "x": xs, "y": ys, "z": zs,
        "centered": centered,
    }
