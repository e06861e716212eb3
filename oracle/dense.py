"""Dense 3D DFT oracle of the reference's tests (tests/test_util/test_transform.hpp:33-276):
scatter the sparse values into a full [x][y][z] grid and run an unnormalised 3D DFT.
Test infrastructure only."""
from __future__ import annotations

import numpy as np

from . import indices as _ix


def backward(transform_type: int, dx: int, dy: int, dz: int, triplets, values) -> np.ndarray:
    """Space domain [z][y][x] of the sparse values (complex for C2C, real for R2C).

    For R2C the values are completed by hermitian symmetry F(-k) = conj(F(k)) wherever -k was not
    given; this equals the reference's C2R result when the given values are consistent."""
    t = np.asarray(triplets, dtype=np.int64).reshape(-1, 3)
    x, y, z = _ix.storage(dx, t[:, 0]), _ix.storage(dy, t[:, 1]), _ix.storage(dz, t[:, 2])
    F = np.zeros((dx, dy, dz), dtype=np.complex128)
    if transform_type == _ix.R2C:
        F[(-x) % dx, (-y) % dy, (-z) % dz] = np.conj(values)
    F[x, y, z] = values
    f = np.fft.ifftn(F) * (dx * dy * dz)
    f = f.transpose(2, 1, 0)
    return np.ascontiguousarray(f.real if transform_type == _ix.R2C else f)


def forward(transform_type: int, dx: int, dy: int, dz: int, triplets, space) -> np.ndarray:
    """Unnormalised forward DFT of the space domain [z][y][x], gathered at the triplets."""
    t = np.asarray(triplets, dtype=np.int64).reshape(-1, 3)
    x, y, z = _ix.storage(dx, t[:, 0]), _ix.storage(dy, t[:, 1]), _ix.storage(dz, t[:, 2])
    f = np.asarray(space).reshape(dz, dy, dx).transpose(2, 1, 0)
    F = np.fft.fftn(f)
    return F[x, y, z]
