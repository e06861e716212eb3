"""Shared helpers of the test suite: index-set generators, golden fixture access, error norms."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)


def load_npz_group(name: str) -> dict:
    data = np.load(GOLDEN / name, allow_pickle=False)
    groups: dict = {}
    for k in data.files:
        if "/" not in k:
            continue
        g, field = k.split("/", 1)
        groups.setdefault(g, {})[field] = data[k]
    return groups


def sphere_indices(n: int, radius: float, r2c: bool = False) -> np.ndarray:
    """Centered (x, y, z) triplets with |k| <= radius on an n^3 grid, in z-stick order (x, y, z
    ascending). For R2C: x >= 0, and at x = 0 only y > 0 or (y = 0, z >= 0)."""
    lo, hi = n // 2 - n + 1, n // 2
    r = np.arange(lo, hi + 1)
    x, y, z = np.meshgrid(r, r, r, indexing="ij")
    m = x * x + y * y + z * z <= radius * radius
    if r2c:
        m &= (x > 0) | ((x == 0) & ((y > 0) | ((y == 0) & (z >= 0))))
    return np.stack([x[m], y[m], z[m]], axis=1).astype(np.int32)


def random_indices(rng, dx, dy, dz, r2c: bool, stick_frac: float = 0.7, fill_frac: float = 0.7,
                   centered: bool = False) -> np.ndarray:
    """Same construction as the reference's create_value_indices (generate_indices.hpp:38-85),
    drawn with numpy's generator: random sticks, random fill; R2C keeps x <= dx/2, y < dy/2+1 at
    x = 0 and half of the (0, 0) stick."""
    dxf = dx // 2 + 1 if r2c else dx
    dyf = dy // 2 + 1 if r2c else dy
    dzf = dz // 2 + 1 if r2c else dz
    out = []
    for x in range(dxf):
        for y in range(dy):
            if x == 0 and y >= dyf:
                continue
            if rng.uniform() < stick_frac:
                for z in range(dz):
                    if r2c and x == 0 and y == 0 and z >= dzf:
                        continue
                    if rng.uniform() < fill_frac:
                        out.append((x, y, z))
    idx = np.array(out, dtype=np.int32).reshape(-1, 3)
    if centered:
        for d, n in enumerate((dx, dy, dz)):
            col = idx[:, d]
            col[col >= n // 2 + 1] -= n
    return idx
