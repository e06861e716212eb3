"""GPU parity of the FP64 transform on hard inputs, against the oracle, through the C ABI.

The FP64 kernels of the size-specialised and batched paths compute in double-float (pairs of FP32
values on the FP32 pipes) with one exact power-of-two scale per block of loaded data; the generic
kernels compute in native FP64. These tests check that the binary64 contract of the reference
(its FFTs run in binary64 end to end, src/fft/transform_1d_host.hpp, transform_real_2d_gpu.hpp)
holds on inputs where the FP32 exponent range of the double-float parts could matter:

* wide dynamic range: values spanning 1e-230 .. 1e+230 in one transform, stick (and space-plane)
  maxima that differ by far more than 2^126 and 2^300, values spanning 1e-30 .. 1e+30 inside one
  stick or row;
* magnitudes near the ends of the binary64 range (1e+300, 1e-300);
* subnormal inputs (all values below 2^-1022, and subnormals mixed with the smallest normals),
  whose results are mostly subnormal too;
* a single NaN or infinity, which must reach every output that it reaches in the oracle (NaN in,
  NaN out); afterwards the same transform must give correct results again.

Expected values come from oracle/pipeline.py (the restated host pipeline). For the subnormal and
tiny cases the oracle runs on the inputs times 2^600 and its result is scaled back by 2^-600 (both
exact), so the expectation is rounded once into the subnormal range instead of at every FFT stage.
Relative L2 errors are computed on max-normalised arrays, so that squares neither overflow nor
underflow. Tolerance: relative L2 <= 1e-12 (FP64), every output finite where the oracle's is.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import pipeline
from util import random_indices, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

TOL = 1e-12
UP = 600  # exact scale for the oracle on tiny inputs


def _workload(name):
    """(transform type, dims, triplets, creation environment): two on the size-specialised
    double-float kernels, one on them with the three-pass split of the z and y lengths (144 =
    12 x 4 x 3) on the split plane passes, one on the generic native-FP64 kernels."""
    if name == "c2c_64_sphere16":
        return sp.SPFFT_TRANS_C2C, (64, 64, 64), sphere_indices(64, 16), {}
    if name == "r2c_48_sphere12":
        return sp.SPFFT_TRANS_R2C, (48, 48, 48), sphere_indices(48, 12, r2c=True), {}
    if name == "r2c_48_144_144_three_pass":
        rng = np.random.default_rng(23)
        return (sp.SPFFT_TRANS_R2C, (48, 144, 144),
                random_indices(rng, 48, 144, 144, r2c=True, stick_frac=0.2, fill_frac=0.3),
                {"SPFFT_GB300_PLANE": "split", "SPFFT_GB300_SPLITS": "2,2,2,2"})
    if name == "c2c_22_26_34":
        rng = np.random.default_rng(17)
        return sp.SPFFT_TRANS_C2C, (22, 26, 34), random_indices(rng, 22, 26, 34, r2c=False,
                                                               stick_frac=0.5, fill_frac=0.6), {}
    raise KeyError(name)


WORKLOADS = ["c2c_64_sphere16", "r2c_48_sphere12", "r2c_48_144_144_three_pass", "c2c_22_26_34"]


class Case:
    def __init__(self, name, dtype="float64"):
        self.ttype, self.dims, self.idx, env = _workload(name)
        self.dtype = dtype
        self.oracle = pipeline.HostPipeline(self.ttype, *self.dims, self.idx)
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            self.tr = sp.Transform(1, sp.SPFFT_PU_GPU, self.ttype, *self.dims, len(self.idx),
                                   sp.SPFFT_INDEX_TRIPLETS, self.idx, dtype=dtype)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        if "SPFFT_GB300_SPLITS" in env and dtype == "float64":
            assert self.tr.splits()["z_backward"] == (12, 4, 3), self.tr.splits()
            assert self.tr.splits()["y_forward"] == (12, 4, 3), self.tr.splits()
        self.ct = torch.complex128 if dtype == "float64" else torch.complex64
        self.st = self.ct if self.ttype == sp.SPFFT_TRANS_C2C else (
            torch.float64 if dtype == "float64" else torch.float32)
        self.shape = self.dims[::-1]

    def backward(self, vals):
        v = torch.from_numpy(vals).to(self.ct).cuda()
        out = torch.full(self.shape, 7.0, dtype=self.st, device="cuda")
        self.tr.backward(v, out)
        return out.cpu().numpy()

    def forward(self, space, scaling=sp.SPFFT_NO_SCALING):
        s = torch.from_numpy(np.ascontiguousarray(space)).to(self.st).cuda()
        out = torch.full((len(self.idx),), 7.0, dtype=self.ct, device="cuda")
        self.tr.forward(s, out, scaling)
        return out.cpu().numpy()

    def random_space(self, rng):
        if self.ttype == sp.SPFFT_TRANS_C2C:
            return rng.uniform(-1, 1, self.shape) + 1j * rng.uniform(-1, 1, self.shape)
        return rng.uniform(-1, 1, self.shape)


def _values(rng, n):
    return rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)


def _scaled_rel_l2(got, want):
    """Relative L2 error after dividing both by max |want| (no overflow or underflow in the
    squares)."""
    s = np.abs(want).max()
    assert s > 0 and np.isfinite(s)
    g = np.asarray(got) / s
    w = np.asarray(want) / s
    return float(np.linalg.norm((g - w).ravel()) / np.linalg.norm(w.ravel()))


def _stick_of_value(case):
    """Stick number of every value (the oracle's storage index divided by dimZ)."""
    return case.oracle.value_indices // case.dims[2]


def _check(got, want):
    assert np.isfinite(want).all()
    assert np.isfinite(got).all(), "non-finite output for finite input"
    err = _scaled_rel_l2(got, want)
    assert err <= TOL, err
    return err


@pytest.mark.parametrize("name", WORKLOADS)
def test_wide_dynamic_range_backward(lib, name):
    c = Case(name)
    rng = np.random.default_rng(101)
    stick = _stick_of_value(c)
    nst = int(stick.max()) + 1
    stick_dec = rng.uniform(-200, 200, nst)
    dec = stick_dec[stick] + rng.uniform(-30, 30, len(c.idx))
    vals = _values(rng, len(c.idx)) * 10.0 ** dec
    maxima = np.array([np.abs(vals[stick == s]).max() for s in range(nst) if (stick == s).any()])
    assert np.log2(maxima.max() / maxima.min()) > 300  # stick maxima 2^300 apart and more
    want = c.oracle.backward(vals)
    _check(c.backward(vals), want)


@pytest.mark.parametrize("name", WORKLOADS)
def test_wide_dynamic_range_forward(lib, name):
    c = Case(name)
    rng = np.random.default_rng(102)
    dz, dy, _ = c.shape
    plane_dec = rng.uniform(-200, 200, (dz, 1, 1))
    row_dec = rng.uniform(-30, 30, (dz, dy, 1))
    space = c.random_space(rng) * 10.0 ** (plane_dec + row_dec)
    for scaling in (sp.SPFFT_NO_SCALING, sp.SPFFT_FULL_SCALING):
        want = c.oracle.forward(space, scaled=scaling == sp.SPFFT_FULL_SCALING)
        _check(c.forward(space, scaling), want)


@pytest.mark.parametrize("name", WORKLOADS)
@pytest.mark.parametrize("magnitude", [1e300, 1e-300])
def test_extreme_magnitudes(lib, name, magnitude):
    c = Case(name)
    rng = np.random.default_rng(103)
    vals = _values(rng, len(c.idx)) * magnitude
    up = 2.0 ** UP if magnitude < 1 else 1.0
    want_b = c.oracle.backward(vals * up) / up
    got_b = c.backward(vals)
    _check(got_b, want_b)
    space = c.random_space(rng) * magnitude
    want_f = c.oracle.forward(space * up) / up
    _check(c.forward(space), want_f)


@pytest.mark.parametrize("name", WORKLOADS)
@pytest.mark.parametrize("mix", ["subnormal", "subnormal_and_smallest_normal"])
def test_subnormal_inputs(lib, name, mix):
    c = Case(name)
    rng = np.random.default_rng(104)
    n = len(c.idx)
    vals = _values(rng, n) * 2.0 ** -1030
    if mix == "subnormal_and_smallest_normal":
        normal = rng.uniform(size=n) < 0.5
        vals[normal] *= 2.0 ** 12  # 2^-1018: normal
    sub = (vals.real != 0) & (np.abs(vals.real) < 2.0 ** -1022)
    assert sub.mean() > (0.9 if mix == "subnormal" else 0.4)
    up = 2.0 ** UP
    want_b = c.oracle.backward(vals * up) / up
    got_b = c.backward(vals)
    assert np.count_nonzero(got_b) > 0.9 * got_b.size
    _check(got_b, want_b)
    space = c.random_space(rng) * 2.0 ** -1030
    want_f = c.oracle.forward(space * up) / up
    got_f = c.forward(space)
    _check(got_f, want_f)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("name", WORKLOADS)
@pytest.mark.parametrize("bad", ["nan", "inf"])
def test_non_finite_propagates_then_clears(lib, name, bad, dtype):
    c = Case(name, dtype)
    rng = np.random.default_rng(105)
    b = complex(np.nan, np.nan) if bad == "nan" else complex(np.inf, -np.inf)
    vals = _values(rng, len(c.idx))
    vals[len(c.idx) // 3] = b
    want = c.oracle.backward(vals)
    got = c.backward(vals)
    assert (~np.isfinite(want)).any()
    missing = ~np.isfinite(want) & np.isfinite(got)
    assert not missing.any(), f"{int(missing.sum())} outputs finite where the oracle's are not"

    space = c.random_space(rng)
    dz, dy, dx = c.shape
    space[dz // 2, dy // 3, dx // 4] = np.nan if bad == "nan" else np.inf
    want_f = c.oracle.forward(space)
    got_f = c.forward(space)
    assert (~np.isfinite(want_f)).any()
    missing = ~np.isfinite(want_f) & np.isfinite(got_f)
    assert not missing.any(), f"{int(missing.sum())} values finite where the oracle's are not"

    # nothing of the non-finite call survives in the transform's scratch or exponent tables
    tol = TOL if dtype == "float64" else 1e-5
    vals = _values(rng, len(c.idx))
    assert _scaled_rel_l2(c.backward(vals), c.oracle.backward(vals)) <= tol
    space = c.random_space(rng)
    assert _scaled_rel_l2(c.forward(space), c.oracle.forward(space)) <= tol


def test_batch_hard_inputs_stay_per_transform(lib):
    """FP64 batched execution (one launch per pass over every transform of a shape group): a NaN
    in one transform, subnormals in another and a wide dynamic range in a third, each checked
    against the oracle; the NaN must not reach the other transforms of its launch."""
    specs = ["c2c_64_sphere16"] * 3 + ["r2c_48_sphere12"] * 3
    cases = [Case(n) for n in specs]
    vals_t = [torch.zeros(len(c.idx), dtype=torch.complex128, device="cuda") for c in cases]
    space_t = [torch.zeros(c.shape, dtype=c.st, device="cuda") for c in cases]
    batch = sp.Batch([c.tr for c in cases])
    batch.bind(vals_t, space_t)
    rng = np.random.default_rng(106)
    host = []
    for i, c in enumerate(cases):
        v = _values(rng, len(c.idx))
        kind = i % 3
        if kind == 0:
            v[5] = complex(np.nan, np.nan)
        elif kind == 1:
            v = v * 2.0 ** -1030
        else:
            stick = _stick_of_value(c)
            v = v * 10.0 ** rng.uniform(-200, 200, int(stick.max()) + 1)[stick]
        host.append(v)
        vals_t[i].copy_(torch.from_numpy(v))
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        batch.backward(stream)
    stream.synchronize()
    for i, (c, v) in enumerate(zip(cases, host)):
        got = space_t[i].cpu().numpy()
        if i % 3 == 0:
            assert not (np.isfinite(got) & ~np.isfinite(c.oracle.backward(v))).any()
            continue
        up = 2.0 ** UP if i % 3 == 1 else 1.0
        _check(got, c.oracle.backward(v * up) / up)
