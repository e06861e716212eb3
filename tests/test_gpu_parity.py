"""GPU parity of the library against the oracle, through the C ABI.

Restates the reference's local transform suite (tests/local_tests/test_local_transform.cpp:95-111,
tests/test_util/test_transform.hpp:78-276): C2C backward (run twice, to prove the scratch is
re-zeroed), C2C forward, R2C forward then backward, over dims {1, 2, 11, 12, 13, 100}^3 plus the
centered variant over {1, 2, 11, 100}^3. Index sets with dims in {1, 2, 11, 12, 13} are the
reference generator's own (golden fixture); sets with a dim of 100 are drawn by the same rule with
numpy. The oracle is the restated host pipeline (oracle/pipeline.py).

Tolerances: FP64 relative L2 <= 1e-12 (and the reference's absolute 1e-6 on values of order one);
FP32 relative L2 <= 1e-5 against the FP64 oracle.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import load_npz_group, random_indices, rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU-only machines skip the whole module
    pytest.skip("no CUDA device", allow_module_level=True)

TOL = {"float64": 1e-12, "float32": 1e-5}
CT = {"float64": torch.complex128, "float32": torch.complex64}
RT = {"float64": torch.float64, "float32": torch.float32}


def _cases(kind: str):
    """(dims, indices) of the reference suite for `kind` in c2c / r2c, plain then centered."""
    gold = load_npz_group("ref_cases.npz")
    rng = np.random.default_rng(1234)
    out = []
    for centered, sizes in ((False, (1, 2, 11, 12, 13, 100)), (True, (1, 2, 11, 100))):
        for dims in itertools.product(sizes, sizes, sizes):
            key = f"{kind}_{'cen' if centered else 'pos'}_{dims[0]}_{dims[1]}_{dims[2]}"
            if key in gold:
                idx = gold[key]["indices"].astype(np.int32).reshape(-1, 3)
            else:
                frac = 1.0 if kind == "r2c" else 0.7
                idx = random_indices(rng, *dims, r2c=(kind == "r2c"), stick_frac=frac,
                                     fill_frac=frac, centered=centered)
            out.append((dims, idx))
    return out


def _values(rng, n):
    return rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)


def _transform(dtype, ttype, dims, idx):
    return sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, idx.shape[0], sp.SPFFT_INDEX_TRIPLETS,
                        idx, dtype=dtype)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_c2c_reference_matrix(lib, dtype):
    rng = np.random.default_rng(99)
    for dims, idx in _cases("c2c"):
        dx, dy, dz = dims
        oracle = pipeline.HostPipeline(0, dx, dy, dz, idx)
        vals = _values(rng, idx.shape[0])
        want = oracle.backward(vals)
        tr = _transform(dtype, sp.SPFFT_TRANS_C2C, dims, idx)
        v = torch.from_numpy(vals).to(CT[dtype]).cuda()
        out = torch.empty((dz, dy, dx), dtype=CT[dtype], device="cuda")
        tr.backward(v, out)
        tr.backward(v, out)  # twice: buffers must be re-zeroed
        got = out.cpu().numpy()
        assert rel_l2(got, want) <= TOL[dtype], (dims, rel_l2(got, want))
        if dtype == "float64":
            assert np.abs(got - want).max() <= 1e-6 * max(1.0, np.abs(want).max())
        # forward of a dense space field
        space = _values(rng, dx * dy * dz).reshape(dz, dy, dx)
        want_f = oracle.forward(space)
        s = torch.from_numpy(space).to(CT[dtype]).cuda()
        f = torch.empty(idx.shape[0], dtype=CT[dtype], device="cuda")
        tr.forward(s, f)
        assert rel_l2(f.cpu().numpy(), want_f) <= TOL[dtype], (dims, rel_l2(f.cpu().numpy(), want_f))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_r2c_reference_matrix(lib, dtype):
    rng = np.random.default_rng(77)
    for dims, idx in _cases("r2c"):
        dx, dy, dz = dims
        oracle = pipeline.HostPipeline(1, dx, dy, dz, idx)
        tr = _transform(dtype, sp.SPFFT_TRANS_R2C, dims, idx)
        field = rng.uniform(-1, 1, (dz, dy, dx))
        # forward of a real field, then backward of its frequency values (test_transform.hpp:221-276)
        want_f = oracle.forward(field)
        s = torch.from_numpy(field).to(RT[dtype]).cuda()
        f = torch.empty(idx.shape[0], dtype=CT[dtype], device="cuda")
        tr.forward(s, f)
        got_f = f.cpu().numpy()
        assert rel_l2(got_f, want_f) <= TOL[dtype], (dims, rel_l2(got_f, want_f))
        out = torch.empty((dz, dy, dx), dtype=RT[dtype], device="cuda")
        tr.backward(torch.from_numpy(want_f).to(CT[dtype]).cuda(), out)
        want_b = oracle.backward(want_f)
        got_b = out.cpu().numpy()
        assert rel_l2(got_b, want_b) <= TOL[dtype], (dims, rel_l2(got_b, want_b))
        # full half-space input reconstructs N * field
        if idx.shape[0] and dtype == "float64":
            assert rel_l2(got_b, field * dx * dy * dz) <= 1e-12


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_r2c_non_hermitian_input_semantics(lib, dtype):
    """Arbitrary (inconsistent) half-space values: the stick and plane symmetry fills and the C2R
    treatment of the x = 0 / Nyquist bins must match the reference pipeline element by element."""
    rng = np.random.default_rng(5)
    for dims in [(12, 11, 13), (11, 12, 12), (8, 8, 8), (2, 12, 11), (1, 12, 12), (12, 1, 12)]:
        idx = random_indices(rng, *dims, r2c=True, stick_frac=0.8, fill_frac=0.8, centered=True)
        vals = _values(rng, idx.shape[0])
        oracle = pipeline.HostPipeline(1, *dims, idx)
        tr = _transform(dtype, sp.SPFFT_TRANS_R2C, dims, idx)
        out = torch.empty(dims[::-1], dtype=RT[dtype], device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        assert rel_l2(out.cpu().numpy(), oracle.backward(vals)) <= TOL[dtype], dims


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_sphere_configs(lib, dtype):
    """The workloads the benchmark runs: 64^3 C2C |k|<=16 and 192^3 R2C half-space |k|<=48."""
    rng = np.random.default_rng(2024)
    for n, radius, ttype in [(64, 16, 0), (192, 48, 1)]:
        idx = sphere_indices(n, radius, r2c=(ttype == 1))
        vals = rng.uniform(-1, 1, idx.shape[0]) + 1j * rng.uniform(-1, 1, idx.shape[0])
        if ttype == 1:
            vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
        oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
        want = oracle.backward(vals)
        tr = _transform(dtype, ttype, (n, n, n), idx)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty((n, n, n), dtype=st, device="cuda")
        v = torch.from_numpy(vals).to(CT[dtype]).cuda()
        tr.backward(v, out)
        assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype]
        f = torch.empty_like(v)
        tr.forward(out, f, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(want, scaled=True)
        assert rel_l2(f.cpu().numpy(), want_f) <= TOL[dtype]
        # backward then scaled forward is the identity on the sparse values (details.rst:42-44)
        if ttype == 0:
            assert rel_l2(f.cpu().numpy(), vals) <= 10 * TOL[dtype]


def test_buffers_locations_inplace_and_modes(lib):
    """Internal space buffers on GPU and host, host pointers, in-place calls, scaling, clone,
    asynchronous mode, grids shared by transforms, and the multi-transform functions."""
    rng = np.random.default_rng(8)
    dims = (12, 13, 11)
    idx = random_indices(rng, *dims, r2c=False)
    n = idx.shape[0]
    vals = _values(rng, n)
    oracle = pipeline.HostPipeline(0, *dims, idx)
    want = oracle.backward(vals)
    tr = _transform("float64", 0, dims, idx)
    assert tr.dim_x() == 12 and tr.dim_y() == 13 and tr.dim_z() == 11
    assert tr.local_slice_size() == 12 * 13 * 11 and tr.num_local_elements() == n
    assert tr.global_size() == 12 * 13 * 11 and tr.local_z_offset() == 0 and tr.local_z_length() == 11

    # host input -> internal GPU buffer, read back through a forward from that buffer
    hv = np.ascontiguousarray(vals)
    tr.backward(hv, sp.SPFFT_PU_GPU)
    assert tr.space_domain_data(sp.SPFFT_PU_GPU) != 0
    buf = torch.empty((11, 13, 12), dtype=torch.complex128, device="cuda")
    f = np.zeros(n, dtype=np.complex128)
    tr.forward(sp.SPFFT_PU_GPU, f)
    assert rel_l2(f, oracle.forward(want)) <= 1e-12

    # host input -> internal host buffer
    import ctypes

    tr.backward(hv, sp.SPFFT_PU_HOST)
    hptr = tr.space_domain_data(sp.SPFFT_PU_HOST)
    host_view = np.ctypeslib.as_array((ctypes.c_double * (2 * 12 * 13 * 11)).from_address(hptr))
    got = host_view.view(np.complex128).reshape(11, 13, 12).copy()
    assert rel_l2(got, want) <= 1e-12
    f2 = np.zeros(n, dtype=np.complex128)
    tr.forward(sp.SPFFT_PU_HOST, f2, sp.SPFFT_FULL_SCALING)
    assert rel_l2(f2, oracle.forward(want, scaled=True)) <= 1e-12

    # host pointers both ways, in place (space buffer holds the values on input)
    space = np.zeros((11, 13, 12), dtype=np.complex128)
    space.reshape(-1)[:n] = vals
    tr.backward(space, space)
    assert rel_l2(space, want) <= 1e-12
    tr.forward(space, space)
    assert rel_l2(space.reshape(-1)[:n], oracle.forward(want)) <= 1e-12

    # device in place
    d = torch.zeros((11, 13, 12), dtype=torch.complex128, device="cuda")
    d.view(-1)[:n] = torch.from_numpy(vals).cuda()
    tr.backward(d, d)
    assert rel_l2(d.cpu().numpy(), want) <= 1e-12

    # clone: independent grid, same results
    tc = tr.clone()
    out = torch.empty_like(buf)
    tc.backward(torch.from_numpy(vals).cuda(), out)
    assert rel_l2(out.cpu().numpy(), want) <= 1e-12

    # asynchronous mode: ordered against the default stream
    tr.set_execution_mode(sp.SPFFT_EXEC_ASYNCHRONOUS)
    assert tr.execution_mode() == sp.SPFFT_EXEC_ASYNCHRONOUS
    out2 = torch.empty_like(buf)
    tr.backward(torch.from_numpy(vals).cuda(), out2)
    assert rel_l2(out2.cpu().numpy(), want) <= 1e-12  # .cpu() runs on the default stream
    tr.set_execution_mode(sp.SPFFT_EXEC_SYNCHRONOUS)

    # grid shared by two transforms of different size
    grid = sp.Grid(16, 16, 16, 16 * 16, sp.SPFFT_PU_GPU, 1)
    assert grid.max_dim_x() == 16 and grid.max_num_local_z_columns() == 256
    t1 = grid.create_transform(sp.SPFFT_PU_GPU, 0, *dims, dims[2], n, sp.SPFFT_INDEX_TRIPLETS, idx)
    idx2 = random_indices(rng, 16, 15, 14, r2c=True, stick_frac=0.5, fill_frac=0.5)
    t2 = grid.create_transform(sp.SPFFT_PU_GPU, 1, 16, 15, 14, 14, idx2.shape[0],
                               sp.SPFFT_INDEX_TRIPLETS, idx2)
    o1 = torch.empty_like(buf)
    t1.backward(torch.from_numpy(vals).cuda(), o1)
    assert rel_l2(o1.cpu().numpy(), want) <= 1e-12
    field = rng.uniform(-1, 1, (14, 15, 16))
    o2 = torch.empty(idx2.shape[0], dtype=torch.complex128, device="cuda")
    t2.forward(torch.from_numpy(field).cuda(), o2)
    assert rel_l2(o2.cpu().numpy(), pipeline.HostPipeline(1, 16, 15, 14, idx2).forward(field)) <= 1e-12
    # too large for the grid
    with pytest.raises(sp.SpfftError) as e:
        grid.create_transform(sp.SPFFT_PU_GPU, 0, 17, 4, 4, 4, 1, sp.SPFFT_INDEX_TRIPLETS,
                              np.array([0, 0, 0]))
    assert e.value.code == sp.ErrorCode.SPFFT_INVALID_PARAMETER_ERROR
    # host execution is not provided by this library
    with pytest.raises(sp.SpfftError):
        sp.Transform(1, sp.SPFFT_PU_HOST, 0, *dims, n, sp.SPFFT_INDEX_TRIPLETS, idx)

    # multi-transform: two independent transforms, rejected when they share a grid
    ta = _transform("float64", 0, dims, idx)
    tb = tr.clone()
    oa, ob = torch.empty_like(buf), torch.empty_like(buf)
    vin = torch.from_numpy(vals).cuda()
    sp.multi_transform_backward([ta, tb], [vin, vin], [oa, ob])
    assert rel_l2(oa.cpu().numpy(), want) <= 1e-12 and rel_l2(ob.cpu().numpy(), want) <= 1e-12
    fa = torch.empty(n, dtype=torch.complex128, device="cuda")
    fb = torch.empty(n, dtype=torch.complex128, device="cuda")
    sp.multi_transform_forward([ta, tb], [oa, ob], [fa, fb])
    assert rel_l2(fa.cpu().numpy(), oracle.forward(want)) <= 1e-12
    with pytest.raises(sp.SpfftError):
        sp.multi_transform_backward([t1, t2], [vin, vin], [oa, ob])


def test_kernel_paths_and_fallbacks(lib):
    """The size-specialised kernels serve the benchmark shapes; shapes they do not cover (odd or
    non-cubic sizes, planes too large for shared memory, an R2C space buffer aligned to 8 bytes
    only) fall back to the generic kernels with the same results."""
    rng = np.random.default_rng(31)
    # fast paths (both precisions: a kernel that cannot be prepared silently loses its fast path)
    for dtype in ("float64", "float32"):
        for dims, ttype in [((64, 64, 64), 0), ((192, 192, 192), 1), ((12, 12, 12), 1), ((100, 100, 13), 0)]:
            idx = sphere_indices(dims[0], dims[0] // 4, r2c=(ttype == 1)) if dims[2] == dims[0] else \
                random_indices(rng, *dims, r2c=(ttype == 1))
            tr = _transform(dtype, ttype, dims, idx)
            info = tr.path_info()
            # the fused plane pass is chosen where two blocks fit an SM and there is a plane per
            # SM (192^3 R2C in FP32); split y and x passes otherwise
            fused = dtype == "float32" and dims == (192, 192, 192)
            assert info["fused_plane"] == fused and info["split_plane"] != fused, (dtype, dims, info)
            assert info["fast_z"] == (dims[2] in (12, 64, 100, 192)), (dtype, dims, info)
    # 192^3 C2C |k| <= 48 FP64: 97 columns, a compact plane too large for a fused block -> split
    idx = sphere_indices(192, 48)
    tr = _transform("float64", 0, (192, 192, 192), idx)
    assert tr.path_info()["fast_z"] and tr.path_info()["split_plane"], tr.path_info()
    vals = _values(rng, len(idx))
    oracle = pipeline.HostPipeline(0, 192, 192, 192, idx)
    out = torch.empty((192, 192, 192), dtype=torch.complex128, device="cuda")
    tr.backward(torch.from_numpy(vals).cuda(), out)
    want = oracle.backward(vals)
    assert rel_l2(out.cpu().numpy(), want) <= 1e-12
    # R2C space buffer that is 8-byte but not 16-byte aligned: generic plane passes
    dims = (48, 48, 48)
    idx = sphere_indices(48, 12, r2c=True)
    tr = _transform("float64", 1, dims, idx)
    assert tr.path_info()["split_plane"]
    vals = _values(rng, len(idx))
    oracle = pipeline.HostPipeline(1, *dims, idx)
    big = torch.zeros(48 ** 3 + 1, dtype=torch.float64, device="cuda")
    shifted = big[1:]
    assert shifted.data_ptr() % 16 == 8
    tr.backward(torch.from_numpy(vals).cuda(), shifted)
    assert rel_l2(shifted.cpu().numpy().reshape(48, 48, 48), oracle.backward(vals)) <= 1e-12
    f = torch.empty(len(idx), dtype=torch.complex128, device="cuda")
    tr.forward(shifted, f)
    assert rel_l2(f.cpu().numpy(), oracle.forward(shifted.cpu().numpy().reshape(48, 48, 48))) <= 1e-12
    # misaligned complex data is rejected, not faulted
    vbig = torch.zeros(2 * len(idx) + 1, dtype=torch.float64, device="cuda")
    with pytest.raises(sp.SpfftError) as e:
        tr.backward(vbig[1:], torch.empty((48, 48, 48), dtype=torch.float64, device="cuda"))
    assert e.value.code == sp.ErrorCode.SPFFT_INVALID_PARAMETER_ERROR


@pytest.mark.parametrize("plane", ["generic", "fused", "split"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_plane_strategies_agree(lib, plane, dtype, monkeypatch):
    """Every plane strategy (generic kernels, one fused kernel per plane, split y / x kernels) gives
    the oracle's result, for C2C and R2C, backward and forward."""
    monkeypatch.setenv("SPFFT_GB300_PLANE", plane)
    rng = np.random.default_rng(17)
    for n, radius, ttype in [(64, 16, 0), (96, 24, 1), (48, 20, 1), (60, 13, 0)]:
        idx = sphere_indices(n, radius, r2c=(ttype == 1))
        tr = _transform(dtype, ttype, (n, n, n), idx)
        info = tr.path_info()
        assert info["fused_plane"] == (plane == "fused") and info["split_plane"] == (plane == "split"), info
        vals = _values(rng, len(idx))
        oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
        want = oracle.backward(vals)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty((n, n, n), dtype=st, device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype], (n, ttype, plane)
        f = torch.empty(len(idx), dtype=CT[dtype], device="cuda")
        tr.forward(out, f)
        assert rel_l2(f.cpu().numpy(), oracle.forward(out.cpu().numpy().astype(np.complex128 if ttype == 0 else np.float64))) <= TOL[dtype]


@pytest.mark.parametrize("rows", ["8", "12", "24"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_x_backward_rows_per_block(lib, rows, dtype, monkeypatch):
    """Split plane passes with the x backward kernel on its own row count (SPFFT_GB300_XB_ROWS, the
    autotuner's extra dimension): same results as the oracle, including a last block with fewer rows
    (96 rows over 24- and 12-row blocks, 100 over 8 / 12 / 24)."""
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    monkeypatch.setenv("SPFFT_GB300_XB_ROWS", rows)
    rng = np.random.default_rng(23)
    for n, radius, ttype in [(96, 24, 1), (100, 25, 0)]:
        idx = sphere_indices(n, radius, r2c=(ttype == 1))
        tr = _transform(dtype, ttype, (n, n, n), idx)
        assert tr.path_info()["split_plane"]
        assert tr.tuning()["rows_per_x_backward_block"] == int(rows), tr.tuning()
        vals = _values(rng, len(idx))
        want = pipeline.HostPipeline(ttype, n, n, n, idx).backward(vals)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty((n, n, n), dtype=st, device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype], (n, ttype, rows)


# Default two-pass split (A, B) of the z and split-y kernels per specialised length; the swapped
# split is (B, A) where B > 1 and A != B.
DEFAULT_SPLIT = {48: (8, 6), 60: (10, 6), 64: (8, 8), 72: (9, 8), 90: (10, 9), 96: (12, 8),
                 100: (10, 10), 108: (12, 9), 120: (12, 10), 128: (16, 8), 144: (12, 12),
                 150: (15, 10), 160: (16, 10), 180: (15, 12), 192: (12, 16), 240: (16, 15),
                 256: (16, 16)}


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("choice", ["1,1,1,1", "1,0,0,1", "0,1,1,0"])
def test_swapped_two_pass_splits(lib, dtype, choice, monkeypatch):
    """The z and split-y kernels in the swapped order of their two radices (SPFFT_GB300_SPLITS, the
    autotuner's split dimension), per pass, for every specialised length: same results as the
    oracle, and splits() / radix_plans() report the split each pass runs."""
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    monkeypatch.setenv("SPFFT_GB300_SPLITS", choice)
    want_swap = [c == "1" for c in choice.split(",")]
    rng = np.random.default_rng(29)
    lengths = sorted(DEFAULT_SPLIT) if choice == "1,1,1,1" else [96, 150, 192]
    for i, n in enumerate(lengths):
        ttype = i % 2
        dims = (48, n, n)  # x, y, z: y and z on the length under test
        idx = random_indices(rng, *dims, r2c=ttype == 1, stick_frac=0.3, fill_frac=0.5)
        tr = _transform(dtype, ttype, dims, idx)
        assert tr.path_info()["split_plane"]
        a, b = DEFAULT_SPLIT[n]
        swappable = b > 1 and a != b
        got = tr.splits()
        for name, sw in zip(["z_backward", "z_forward", "y_backward", "y_forward"], want_swap):
            assert got[name] == ((b, a) if sw and swappable else (a, b)), (n, name, got)
        plans = tr.radix_plans()
        assert plans[0] == list(got["z_backward"]) and plans[1] == list(got["y_backward"]), plans
        vals = _values(rng, len(idx))
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty(dims[::-1], dtype=st, device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        space = out.cpu().numpy()
        assert rel_l2(space, oracle.backward(vals)) <= TOL[dtype], (n, ttype, choice)
        f = torch.empty(len(idx), dtype=CT[dtype], device="cuda")
        tr.forward(out, f, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(space.astype(np.complex128 if ttype == 0 else np.float64), scaled=True)
        assert rel_l2(f.cpu().numpy(), want_f) <= TOL[dtype], (n, ttype, choice)


# Three-pass split (A, B1, B2) of the double-precision z and split-y kernels: the lengths whose
# second radix B is 12 or 16, with B = B1 * B2.
THREE_PASS = {144: (12, 4, 3), 180: (15, 4, 3), 192: (12, 4, 4), 256: (16, 4, 4)}


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("choice", ["2,2,2,2", "2,0,1,2", "0,2,2,1"])
def test_three_pass_splits(lib, dtype, choice, monkeypatch):
    """The z and split-y kernels with the three-pass split (SPFFT_GB300_SPLITS value 2), per pass,
    mixed with the default and swapped splits, for every length that has it: same results as the
    oracle, and splits() / radix_plans() report (A, B1, B2). Single precision has no three-pass
    kernels: a request for one keeps the default split."""
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    monkeypatch.setenv("SPFFT_GB300_SPLITS", choice)
    want = [int(c) for c in choice.split(",")]
    rng = np.random.default_rng(31)
    for i, n in enumerate(sorted(THREE_PASS)):
        ttype = i % 2
        dims = (48, n, n)
        idx = random_indices(rng, *dims, r2c=ttype == 1, stick_frac=0.3, fill_frac=0.5)
        tr = _transform(dtype, ttype, dims, idx)
        assert tr.path_info()["split_plane"]
        a, b = DEFAULT_SPLIT[n]
        got = tr.splits()
        for name, v in zip(["z_backward", "z_forward", "y_backward", "y_forward"], want):
            if v == 2 and dtype == "float64":
                expect = THREE_PASS[n]
            elif v == 1 and b > 1 and a != b:
                expect = (b, a)
            else:
                expect = (a, b)
            assert got[name] == expect, (n, name, got)
        plans = tr.radix_plans()
        assert plans[0] == list(got["z_backward"]) and plans[1] == list(got["y_backward"]), plans
        vals = _values(rng, len(idx))
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty(dims[::-1], dtype=st, device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        space = out.cpu().numpy()
        assert rel_l2(space, oracle.backward(vals)) <= TOL[dtype], (n, ttype, choice)
        f = torch.empty(len(idx), dtype=CT[dtype], device="cuda")
        tr.forward(out, f, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(space.astype(np.complex128 if ttype == 0 else np.float64), scaled=True)
        assert rel_l2(f.cpu().numpy(), want_f) <= TOL[dtype], (n, ttype, choice)


@pytest.mark.parametrize("access", ["direct", "copy"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_pinned_host_buffers(lib, access, dtype, monkeypatch):
    """Pinned host buffers: kernels read / write them directly over the host link (default) or
    through staged copies (SPFFT_GB300_HOST_ACCESS=copy); same results either way, including
    in-place calls."""
    monkeypatch.setenv("SPFFT_GB300_HOST_ACCESS", access)
    rng = np.random.default_rng(21)
    for n, radius, ttype in [(48, 12, 1), (64, 16, 0), (13, 4, 0)]:
        idx = sphere_indices(n, radius, r2c=(ttype == 1))
        tr = _transform(dtype, ttype, (n, n, n), idx)
        oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
        vals = _values(rng, len(idx))
        if ttype == 1:
            vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
        hv = torch.from_numpy(vals).to(CT[dtype]).pin_memory()
        st = CT[dtype] if ttype == 0 else RT[dtype]
        hs = torch.empty((n, n, n), dtype=st).pin_memory()
        tr.backward(hv, hs)
        want = oracle.backward(vals)
        assert rel_l2(hs.numpy(), want) <= TOL[dtype], (n, access)
        hf = torch.empty_like(hv)
        tr.forward(hs, hf, sp.SPFFT_FULL_SCALING)
        assert rel_l2(hf.numpy(), oracle.forward(hs.numpy().astype(np.float64 if ttype else np.complex128),
                                                   scaled=True)) <= TOL[dtype]
        if ttype == 0:  # in place through one pinned buffer
            buf = torch.zeros((n, n, n), dtype=st).pin_memory()
            buf.view(-1)[: len(idx)] = torch.from_numpy(vals).to(st)
            tr.backward(buf, buf)
            assert rel_l2(buf.numpy(), want) <= TOL[dtype]


@pytest.mark.parametrize("chunks", [None, "1", "7", "32"])
def test_pinned_host_buffers_chunk_schedules(lib, chunks, monkeypatch):
    """The staged host-buffer paths with the default plane chunks (doubling in size; 90 planes:
    4, 8, 16, 32, 30, taken in reverse by the forward) and with n equal chunks
    (SPFFT_GB300_STAGED_CHUNKS: 1, 7 of 13 planes and a last of 12, 30 of 3): same results."""
    if chunks is None:
        monkeypatch.delenv("SPFFT_GB300_STAGED_CHUNKS", raising=False)
    else:
        monkeypatch.setenv("SPFFT_GB300_STAGED_CHUNKS", chunks)
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    rng = np.random.default_rng(61)
    for dims, ttype in [((48, 60, 90), 1), ((60, 48, 90), 0)]:
        idx = random_indices(rng, *dims, r2c=ttype == 1, stick_frac=0.3, fill_frac=0.4)
        tr = _transform("float64", ttype, dims, idx)
        assert tr.path_info()["split_plane"]
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        vals = _values(rng, len(idx))
        hv = torch.from_numpy(vals).pin_memory()
        hs = torch.empty(dims[::-1], dtype=torch.complex128 if ttype == 0 else torch.float64).pin_memory()
        tr.backward(hv, hs)
        assert rel_l2(hs.numpy(), oracle.backward(vals)) <= TOL["float64"], (dims, chunks)
        hf = torch.empty_like(hv)
        tr.forward(hs, hf, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(hs.numpy().astype(np.complex128 if ttype == 0 else np.float64), scaled=True)
        assert rel_l2(hf.numpy(), want_f) <= TOL["float64"], (dims, chunks)


@pytest.mark.parametrize("access", ["direct", "copy"])
def test_pinned_host_buffers_three_pass(lib, access, monkeypatch):
    """Pinned host buffers on the split plane passes with the three-pass z and y splits: the
    staged paths run the y and x passes plane chunk by plane chunk (while the space domain crosses
    the host link), so the three-pass y kernels run on plane ranges; same results as the oracle."""
    monkeypatch.setenv("SPFFT_GB300_HOST_ACCESS", access)
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    monkeypatch.setenv("SPFFT_GB300_SPLITS", "2,2,2,2")
    rng = np.random.default_rng(53)
    for dims, ttype in [((48, 144, 144), 1), ((48, 192, 192), 0)]:
        idx = random_indices(rng, *dims, r2c=ttype == 1, stick_frac=0.2, fill_frac=0.4)
        tr = _transform("float64", ttype, dims, idx)
        assert tr.path_info()["split_plane"]
        assert len(tr.splits()["y_backward"]) == 3 and len(tr.splits()["z_forward"]) == 3, tr.splits()
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        vals = _values(rng, len(idx))
        hv = torch.from_numpy(vals).pin_memory()
        hs = torch.empty(dims[::-1], dtype=torch.complex128 if ttype == 0 else torch.float64).pin_memory()
        tr.backward(hv, hs)
        assert rel_l2(hs.numpy(), oracle.backward(vals)) <= TOL["float64"], (dims, access)
        hf = torch.empty_like(hv)
        tr.forward(hs, hf, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(hs.numpy().astype(np.complex128 if ttype == 0 else np.float64), scaled=True)
        assert rel_l2(hf.numpy(), want_f) <= TOL["float64"], (dims, access)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_every_specialised_length(lib, dtype):
    """Every length with size-specialised kernels, C2C and R2C, single transforms and one batch
    of them: shared-memory tables and buffers of each layout must be aligned for every length
    (the FP32 R2C twiddle tables of N = 90 and 150 end on an 8-byte boundary)."""
    rng = np.random.default_rng(41)
    items = []
    for n in (12, 48, 60, 64, 72, 90, 96, 100, 108, 120, 128, 144, 150, 160, 180, 192, 240, 256):
        for ttype in (0, 1):
            idx = sphere_indices(n, max(2, n // 6), r2c=(ttype == 1))
            vals = _values(rng, idx.shape[0])
            if ttype == 1:
                vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
            oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
            tr = _transform(dtype, ttype, (n, n, n), idx)
            assert tr.path_info()["fast_z"], (n, ttype)
            v = torch.from_numpy(vals).to(CT[dtype]).cuda()
            out = torch.empty((n, n, n), dtype=CT[dtype] if ttype == 0 else RT[dtype], device="cuda")
            tr.backward(v, out)
            want = oracle.backward(vals)
            assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype], (n, ttype)
            f = torch.empty_like(v)
            tr.forward(out, f)
            assert rel_l2(f.cpu().numpy(), oracle.forward(want)) <= TOL[dtype], (n, ttype)
            items.append((tr, v, torch.zeros_like(out), oracle, vals))
    batch = sp.Batch([it[0] for it in items])
    batch.bind([it[1] for it in items], [it[2] for it in items])
    stream = torch.cuda.Stream()
    batch.backward(stream)
    stream.synchronize()
    for tr, v, space, oracle, vals in items:
        assert rel_l2(space.cpu().numpy(), oracle.backward(vals)) <= TOL[dtype]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("xb_rows", ["32", "24"])
def test_x_chunk_layout_partial_row_groups(lib, dtype, xb_rows, monkeypatch):
    """The x-pass chunk layout of 12 x 8 rows (the x pass of 192 R2C and 96 C2C) takes pass-1 rows
    as 0, 2, 1, 3 within each complete group of four and in order in a last incomplete group: y
    lengths that leave chunks of 26, 22 and 18 rows on the split plane passes match the oracle."""
    monkeypatch.setenv("SPFFT_GB300_PLANE", "split")
    monkeypatch.setenv("SPFFT_GB300_XB_ROWS", xb_rows)
    rng = np.random.default_rng(47)
    for dims, ttype in [((192, 90, 48), 1), ((96, 150, 48), 0)]:
        idx = random_indices(rng, *dims, r2c=ttype == 1, stick_frac=0.4, fill_frac=0.5)
        tr = _transform(dtype, ttype, dims, idx)
        assert tr.path_info()["split_plane"], dims
        assert tr.tuning()["rows_per_x_backward_block"] == int(xb_rows)
        vals = _values(rng, len(idx))
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        st = CT[dtype] if ttype == 0 else RT[dtype]
        out = torch.empty(dims[::-1], dtype=st, device="cuda")
        tr.backward(torch.from_numpy(vals).to(CT[dtype]).cuda(), out)
        space = out.cpu().numpy()
        assert rel_l2(space, oracle.backward(vals)) <= TOL[dtype], (dims, xb_rows)
        f = torch.empty(len(idx), dtype=CT[dtype], device="cuda")
        tr.forward(out, f, sp.SPFFT_FULL_SCALING)
        want_f = oracle.forward(space.astype(np.complex128 if ttype == 0 else np.float64), scaled=True)
        assert rel_l2(f.cpu().numpy(), want_f) <= TOL[dtype], (dims, xb_rows)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_autotune_keeps_results(lib, dtype):
    """The autotuner picks one of the valid tile shapes and plane strategies; results after tuning
    still match the oracle."""
    rng = np.random.default_rng(43)
    for n, radius, ttype in [(64, 16, 0), (192, 48, 1)]:
        idx = sphere_indices(n, radius, r2c=(ttype == 1))
        tr = _transform(dtype, ttype, (n, n, n), idx)
        before = tr.tuning()
        ms = tr.autotune(2)
        after = tr.tuning()
        assert ms > 0 and after["plane"] in ("fused", "split"), (before, after)
        assert after["sticks_per_z_block"] in (6, 8, 12, 16, 24, 32)
        vals = _values(rng, idx.shape[0])
        if ttype == 1:
            vals[(idx == 0).all(axis=1)] = vals[(idx == 0).all(axis=1)].real
        oracle = pipeline.HostPipeline(ttype, n, n, n, idx)
        v = torch.from_numpy(vals).to(CT[dtype]).cuda()
        out = torch.empty((n, n, n), dtype=CT[dtype] if ttype == 0 else RT[dtype], device="cuda")
        tr.backward(v, out)
        want = oracle.backward(vals)
        assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype], (n, after)
        f = torch.empty_like(v)
        tr.forward(out, f)
        assert rel_l2(f.cpu().numpy(), oracle.forward(want)) <= TOL[dtype], (n, after)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_autotuned_radix_plans_on_generic_lengths(lib, dtype):
    """Lengths without specialised kernels run the runtime-radix kernels; the autotuner picks one
    of several radix plans per length (products equal the length) and the results stay those of
    the oracle, for every plan of every length forced through the plane strategy 'generic'."""
    rng = np.random.default_rng(47)
    for dims, ttype in [((40, 54, 45), 0), ((32, 36, 50), 1), ((11, 13, 7), 0)]:
        idx = random_indices(rng, *dims, r2c=(ttype == 1))
        tr = _transform(dtype, ttype, dims, idx)
        assert tr.tuning()["plane"] == "generic"
        ms = tr.autotune(2)
        plans = tr.radix_plans()
        assert ms > 0
        for d, n in zip((2, 1, 0), dims):  # plans are (z, y, x)
            assert int(np.prod(plans[d])) == n, (dims, plans)
        vals = _values(rng, idx.shape[0])
        oracle = pipeline.HostPipeline(ttype, *dims, idx)
        v = torch.from_numpy(vals).to(CT[dtype]).cuda()
        out = torch.empty(dims[::-1], dtype=CT[dtype] if ttype == 0 else RT[dtype], device="cuda")
        tr.backward(v, out)
        want = oracle.backward(vals)
        assert rel_l2(out.cpu().numpy(), want) <= TOL[dtype], (dims, plans)
        f = torch.empty_like(v)
        tr.forward(out, f)
        assert rel_l2(f.cpu().numpy(), oracle.forward(out.cpu().numpy().astype(
            np.complex128 if ttype == 0 else np.float64))) <= TOL[dtype], (dims, plans)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_reference_pipeline_golden(lib, dtype):
    """The library against golden vectors of the reference's OWN host transform path (run on the
    inputs of its local test suite, FP64; tests/golden/make_golden.py): C2C backward then forward,
    R2C forward then backward, the order of the reference's tests."""
    cases = load_npz_group("ref_pipeline.npz")
    assert len(cases) >= 28
    for name, c in cases.items():
        t, dx, dy, dz = map(int, c["args"])
        idx = np.ascontiguousarray(c["indices"].astype(np.int32).reshape(-1, 3))
        tr = _transform(dtype, t, (dx, dy, dz), idx)
        n = idx.shape[0]
        vals = torch.empty(n, dtype=CT[dtype], device="cuda")
        space = torch.empty((dz, dy, dx), dtype=CT[dtype] if t == 0 else RT[dtype], device="cuda")
        if t == 0:
            vals.copy_(torch.from_numpy(c["values_in"]).to(CT[dtype]))
            tr.backward(vals, space)
            torch.cuda.synchronize()
            assert rel_l2(space.cpu().numpy(), c["space_out"]) <= TOL[dtype], name
            tr.forward(space, vals)
            torch.cuda.synchronize()
            assert rel_l2(vals.cpu().numpy(), c["values_out"]) <= TOL[dtype], name
        else:
            space.copy_(torch.from_numpy(c["space_in"]).to(RT[dtype]))
            tr.forward(space, vals)
            torch.cuda.synchronize()
            assert rel_l2(vals.cpu().numpy(), c["values_out"]) <= TOL[dtype], name
            tr.backward(vals, space)
            torch.cuda.synchronize()
            assert rel_l2(space.cpu().numpy(), c["space_out"]) <= TOL[dtype], name
