"""The reference's host transform pipeline, restated with numpy + scipy.fft (test infrastructure).

Stage order and data layouts follow src/execution/execution_host.cpp:
  backward_z  (:297-315)  decompress -> stick symmetry -> z transforms
  backward_xy (:324-352)  transpose unpack into [z][xFreq][y] -> plane symmetry ->
                          y transforms over the x columns that hold sticks only -> x C2C / C2R
  forward_xy / forward_z (:246-295) the mirror image, with compress (optionally scaled).
FFTW's unnormalised FFTW_BACKWARD / FFTW_FORWARD transforms become scipy.fft transforms with
norm="forward" (unscaled inverse) and norm="backward" (unscaled forward).
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft as sfft

from . import indices as _ix


def _workers(workers):
    return workers if workers is not None else (os.cpu_count() or 1)


def hermitian_line_fill(v: np.ndarray, axis: int = -1) -> None:
    """In-place conj fill along `axis`: for k in [1, n/2] then [n/2+1, n): v[n-k] = conj(v[k])
    where v[k] != 0 (symmetry_host.hpp:42-90)."""
    v = np.moveaxis(v, axis, -1)
    n = v.shape[-1]
    for lo, hi in ((1, n // 2 + 1), (n // 2 + 1, n)):
        if hi <= lo:
            continue
        k = np.arange(lo, hi)
        src = v[..., k].copy()
        mask = (src != 0)
        dst = v[..., n - k]
        v[..., n - k] = np.where(mask, np.conj(src), dst)


class HostPipeline:
    def __init__(self, transform_type: int, dx: int, dy: int, dz: int, triplets):
        self.type = transform_type
        self.dx, self.dy, self.dz = dx, dy, dz
        self.dxf = dx // 2 + 1 if transform_type == _ix.R2C else dx
        p = _ix.convert(transform_type, dx, dy, dz, triplets)
        self.value_indices = p["value_indices"]
        self.stick_keys = p["stick_keys"]
        self.zz = p["zero_zero_stick"]
        self.stick_x = self.stick_keys // dy
        self.stick_y = self.stick_keys - self.stick_x * dy
        # execution_host.cpp:61-64: the set of x indices that hold sticks
        self.unique_x = np.unique(self.stick_x)

    # ---- backward: frequency values -> space -------------------------------------------------
    def backward(self, values: np.ndarray, workers=None) -> np.ndarray:
        w = _workers(workers)
        ns, dz = self.stick_keys.size, self.dz
        sticks = np.zeros((ns, dz), dtype=np.complex128)
        sticks.reshape(-1)[self.value_indices] = values  # compression_host.hpp:76-92
        if self.type == _ix.R2C and self.zz < ns:
            hermitian_line_fill(sticks[self.zz])
        if ns:
            sticks = sfft.ifft(sticks, axis=1, norm="forward", workers=w)
        planes = np.zeros((dz, self.dxf, self.dy), dtype=np.complex128)  # [z][xFreq][y]
        planes[:, self.stick_x, self.stick_y] = sticks.T  # transpose_host.hpp:76-117
        if self.type == _ix.R2C:
            hermitian_line_fill(planes[:, 0, :], axis=-1)
        if self.unique_x.size:
            ux = self.unique_x
            planes[:, ux, :] = sfft.ifft(planes[:, ux, :], axis=2, norm="forward", workers=w)
        rows = np.ascontiguousarray(planes.transpose(0, 2, 1))  # [z][y][xFreq]
        if self.type == _ix.R2C:
            return sfft.irfft(rows, n=self.dx, axis=2, norm="forward", workers=w)
        return sfft.ifft(rows, axis=2, norm="forward", workers=w)

    # ---- forward: space -> frequency values ---------------------------------------------------
    def forward(self, space: np.ndarray, scaled: bool = False, workers=None,
                dtype=np.float64) -> np.ndarray:
        w = _workers(workers)
        space = np.asarray(space).reshape(self.dz, self.dy, self.dx)
        if self.type == _ix.R2C:
            rows = sfft.rfft(space, axis=2, workers=w)
        else:
            rows = sfft.fft(space, axis=2, workers=w)
        planes = rows.transpose(0, 2, 1)  # [z][xFreq][y]
        ux = self.unique_x
        ycols = sfft.fft(planes[:, ux, :], axis=2, workers=w) if ux.size else planes[:, ux, :]
        col_of_x = np.full(self.dxf, -1, dtype=np.int64)
        col_of_x[ux] = np.arange(ux.size)
        sticks = ycols[:, col_of_x[self.stick_x], self.stick_y].T  # [stick][z]
        if sticks.size:
            sticks = sfft.fft(sticks, axis=1, workers=w)
        out = sticks.reshape(-1)[self.value_indices]
        if scaled:
            # T(1 / (Nx Ny Nz)) computed in double, then applied in T (execution_host.cpp:57-58)
            s = dtype(1.0 / (float(self.dx) * self.dy * self.dz))
            out = out * float(s)
        return out
