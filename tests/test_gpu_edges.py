"""Edge cases of the transform path on the GPU, against the oracle: an empty index set, a single
value at k = 0, full grids (every frequency present), the largest size-specialised length, and
values in a shuffled user order. Both precisions."""
from __future__ import annotations

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

TOL = {"float64": 1e-12, "float32": 1e-5}
CT = {"float64": torch.complex128, "float32": torch.complex64}
RT = {"float64": torch.float64, "float32": torch.float32}


def _run(dtype, ttype, dims, idx, vals):
    """backward into a NaN-filled space buffer, then an unscaled forward; returns both."""
    n = idx.shape[0]
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, n, sp.SPFFT_INDEX_TRIPLETS, idx, dtype=dtype)
    v = torch.from_numpy(vals).to(CT[dtype]).cuda() if n else torch.zeros(1, dtype=CT[dtype], device="cuda")
    space = torch.full(dims[::-1], float("nan"), dtype=CT[dtype] if ttype == 0 else RT[dtype], device="cuda")
    tr.backward(v, space)
    out = torch.full((max(n, 1),), float("nan"), dtype=CT[dtype], device="cuda")
    tr.forward(space, out)
    torch.cuda.synchronize()
    return space.cpu().numpy(), out.cpu().numpy()[:n]


def _full_grid(dims, r2c):
    g = np.stack(np.meshgrid(*[np.arange(n) for n in dims], indexing="ij"), -1).reshape(-1, 3)
    if r2c:
        g = g[g[:, 0] <= dims[0] // 2]
    return np.ascontiguousarray(g.astype(np.int32))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("ttype", [0, 1])
def test_empty_index_set(lib, dtype, ttype):
    space, out = _run(dtype, ttype, (8, 8, 8), np.zeros((0, 3), dtype=np.int32), np.zeros(0))
    assert not np.isnan(space).any() and np.abs(space).max() == 0.0
    assert out.size == 0


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("ttype", [0, 1])
def test_single_value_at_k0(lib, dtype, ttype):
    dims = (12, 10, 8)
    idx = np.zeros((1, 3), dtype=np.int32)
    space, out = _run(dtype, ttype, dims, idx, np.array([2.5 + 0.0j]))
    np.testing.assert_allclose(space, np.full(dims[::-1], 2.5), rtol=TOL[dtype])
    np.testing.assert_allclose(out, [2.5 * np.prod(dims)], rtol=TOL[dtype])


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("ttype", [0, 1])
@pytest.mark.parametrize("dims", [(16, 12, 10), (64, 64, 64), (13, 7, 5)])
def test_full_grids(lib, dtype, ttype, dims):
    """Every frequency of the grid (the hermitian half for R2C): numValues at its maximum, every
    x column non-empty."""
    idx = _full_grid(dims, ttype == 1)
    rng = np.random.default_rng(11)
    vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
    oracle = pipeline.HostPipeline(ttype, *dims, idx)
    space, out = _run(dtype, ttype, dims, idx, vals)
    assert rel_l2(space, oracle.backward(vals)) <= TOL[dtype]
    want = oracle.forward(space.astype(np.complex128 if ttype == 0 else np.float64))
    assert rel_l2(out, want) <= TOL[dtype]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_largest_specialised_length(lib, dtype):
    """256^3 (the longest size-specialised length), R2C |k| <= 64 and C2C |k| <= 40, values in a
    shuffled user order, on the specialised kernels."""
    rng = np.random.default_rng(12)
    for ttype, radius in ((1, 64), (0, 40)):
        idx = sphere_indices(256, radius, r2c=(ttype == 1))
        idx = np.ascontiguousarray(idx[rng.permutation(len(idx))])
        vals = rng.uniform(-1, 1, len(idx)) + 1j * rng.uniform(-1, 1, len(idx))
        if ttype == 1:
            vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
        oracle = pipeline.HostPipeline(ttype, 256, 256, 256, idx)
        tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, 256, 256, 256, len(idx), sp.SPFFT_INDEX_TRIPLETS, idx,
                          dtype=dtype)
        info = tr.path_info()
        assert info["fast_z"] and (info["split_plane"] or info["fused_plane"]), info
        del tr
        space, out = _run(dtype, ttype, (256, 256, 256), idx, vals)
        assert rel_l2(space, oracle.backward(vals)) <= TOL[dtype], ttype
        want = oracle.forward(space.astype(np.complex128 if ttype == 0 else np.float64))
        assert rel_l2(out, want) <= TOL[dtype], ttype
