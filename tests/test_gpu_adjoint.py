"""GPU tests of the differentiable transforms (spfft_gb300.autograd): adjointness (dot-product
test), central finite differences (h = 1e-6, 64 random coordinates) on the 96^3 C2C |k| <= 24
workload with loss L = sum V |psi|^2, and comparison with an FP64 numpy adjoint
(grad_c = 2 * gather(forward_DFT(V * psi))). R2C cases check the hermitian multiplicities."""
import numpy as np
import pytest

import spfft_gb300 as sp
from oracle import dense
from util import rel_l2, sphere_indices

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

from spfft_gb300 import autograd as sag  # noqa: E402


def _inner(a, b):
    """Real inner product Re <a, b> used by the adjoint convention."""
    return float(np.real(np.vdot(np.asarray(a).ravel(), np.asarray(b).ravel())))


@pytest.mark.parametrize("ttype,dims,radius", [(0, (24, 20, 18), 7), (1, (24, 20, 18), 7), (1, (16, 16, 16), 8),
                                               (1, (15, 13, 11), 5), (0, (12, 12, 12), 5)])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_dot_product_adjointness(lib, ttype, dims, radius, dtype):
    rng = np.random.default_rng(11)
    nx, ny, nz = dims
    idx = sphere_indices(max(dims), radius, r2c=(ttype == 1))
    idx = idx[(np.abs(idx[:, 0]) <= nx // 2) & (idx[:, 1] >= ny // 2 - ny + 1) & (idx[:, 1] <= ny // 2)
              & (idx[:, 2] >= nz // 2 - nz + 1) & (idx[:, 2] <= nz // 2)]
    if ttype == 0:
        idx = idx[idx[:, 0] >= nx // 2 - nx + 1]
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, ttype, *dims, len(idx), 0, idx, dtype=dtype)
    ct = torch.complex128 if dtype == "float64" else torch.complex64
    rt = torch.float64 if dtype == "float64" else torch.float32
    c = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    if ttype == 1:  # self-conjugate frequencies carry real values
        sc = np.all([(v == 0) | ((n % 2 == 0) & (np.abs(v) == n // 2)) for v, n in zip(idx.T, dims)], axis=0)
        c[sc] = c[sc].real
        g = rng.standard_normal(dims[::-1])
    else:
        g = rng.standard_normal(dims[::-1]) + 1j * rng.standard_normal(dims[::-1])
    psi = torch.empty(dims[::-1], dtype=ct if ttype == 0 else rt, device="cuda")
    tr.backward_device(torch.from_numpy(c).to(ct).cuda(), psi)
    adj = torch.empty(len(idx), dtype=ct, device="cuda")
    tr.adjoint_backward(torch.from_numpy(g).to(psi.dtype).cuda(), adj)
    torch.cuda.synchronize()
    lhs = _inner(g, psi.cpu().numpy())
    rhs = _inner(adj.cpu().numpy(), c)
    tol = 1e-11 if dtype == "float64" else 2e-5
    assert abs(lhs - rhs) <= tol * (abs(lhs) + abs(rhs)), (lhs, rhs)
    # adjoint of forward: <F s, w> = <s, F^H w>
    s = rng.standard_normal(dims[::-1]) if ttype == 1 else g
    w = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    fs = torch.empty(len(idx), dtype=ct, device="cuda")
    tr.forward_device(torch.from_numpy(s).to(psi.dtype).cuda(), fs, sp.SPFFT_FULL_SCALING)
    aw = torch.empty_like(psi)
    tr.adjoint_forward(torch.from_numpy(w).to(ct).cuda(), aw, sp.SPFFT_FULL_SCALING)
    torch.cuda.synchronize()
    lhs = _inner(w, fs.cpu().numpy())
    rhs = _inner(aw.cpu().numpy(), s)
    assert abs(lhs - rhs) <= tol * (abs(lhs) + abs(rhs)), (lhs, rhs)


def test_gradient_96_c2c_finite_differences_and_fp64_adjoint(lib):
    """L = sum V |psi|^2, psi = backward(c): autograd gradient vs central differences and vs the
    FP64 numpy adjoint 2 * gather(fftn(V psi))."""
    n, radius = 96, 24
    idx = sphere_indices(n, radius)
    rng = np.random.default_rng(2024)
    c0 = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    V = rng.uniform(0, 1, (n, n, n))
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, 0, n, n, n, len(idx), 0, idx)
    Vt = torch.from_numpy(V).cuda()

    def loss(c):
        psi = sag.backward(tr, c)
        return (Vt * psi.real ** 2 + Vt * psi.imag ** 2).sum()

    c = torch.from_numpy(c0).cuda().requires_grad_(True)
    L = loss(c)
    L.backward()
    grad = c.grad.cpu().numpy()

    # FP64 numpy adjoint
    psi = dense.backward(0, n, n, n, idx, c0)
    want = 2 * dense.forward(0, n, n, n, idx, V * psi)
    assert rel_l2(grad, want) <= 1e-12

    # central finite differences, h = 1e-6, on 64 random coordinates (real and imaginary parts)
    h = 1e-6
    pick = rng.choice(len(idx), 64, replace=False)
    with torch.no_grad():
        for j in pick:
            for part, unit in ((0, 1.0), (1, 1j)):
                cp = torch.from_numpy(c0).cuda()
                cm = cp.clone()
                cp[j] += h * unit
                cm[j] -= h * unit
                fd = (loss(cp).item() - loss(cm).item()) / (2 * h)
                an = grad[j].real if part == 0 else grad[j].imag
                assert abs(fd - an) <= 1e-5 * np.abs(grad).max(), (j, part, fd, an)


def test_gradient_r2c_and_forward_chain(lib):
    """R2C: a loss through backward then forward (scaled), gradients against finite differences."""
    n = 24
    idx = sphere_indices(n, 7, r2c=True)
    rng = np.random.default_rng(5)
    c0 = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    k0 = (idx == 0).all(axis=1)
    c0[k0] = c0[k0].real
    V = rng.uniform(0.5, 1.5, (n, n, n))
    W = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    tr = sp.Transform(1, sp.SPFFT_PU_GPU, 1, n, n, n, len(idx), 0, idx)
    Vt = torch.from_numpy(V).cuda()
    Wt = torch.from_numpy(W).cuda()

    def loss(c):
        psi = sag.backward(tr, c)
        back = sag.forward(tr, Vt * psi * psi, scaled=True)
        return (Wt.conj() * back).real.sum() + (psi ** 2).sum() * 1e-3

    c = torch.from_numpy(c0).cuda().requires_grad_(True)
    loss(c).backward()
    grad = c.grad.cpu().numpy()
    h = 1e-6
    with torch.no_grad():
        for j in rng.choice(len(idx), 24, replace=False):
            for part, unit in ((0, 1.0), (1, 1j)):
                if part == 1 and k0[j]:
                    continue  # the imaginary part of the k = 0 value does not enter the real field
                cp = torch.from_numpy(c0).cuda()
                cm = cp.clone()
                cp[j] += h * unit
                cm[j] -= h * unit
                fd = (loss(cp).item() - loss(cm).item()) / (2 * h)
                an = grad[j].real if part == 0 else grad[j].imag
                assert abs(fd - an) <= 1e-6 * max(1.0, np.abs(grad).max()), (j, part, fd, an)
