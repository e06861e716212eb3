"""Differentiable sparse transforms for PyTorch, bound over the C ABI.

``backward(transform, values)`` and ``forward(transform, space)`` run the library's GPU transforms
on the current CUDA stream and register the hand-written adjoints
(``spfft_gb300_transform_adjoint_backward`` / ``_adjoint_forward``) as their gradients:

* backward (values -> space) has the adjoint "unnormalised forward transform + gather" (the
  transpose of the backward's scatter), times each value's hermitian multiplicity for R2C;
* forward (space -> values) has the adjoint "backward transform of the value gradient", divided by
  those multiplicities for R2C, scaled like the forward.

Gradients use PyTorch's convention for complex tensors (dL/dRe + i dL/dIm).

Concurrency: every call (the transform and its adjoint alike) runs on the transform's one set of
intermediate buffers (its grid's stick and plane scratch). Calls that use the same transform must
therefore not overlap on the GPU: two autograd graphs that run one transform on different CUDA
streams at the same time race on that scratch and corrupt each other's results. Give each
concurrently used stream its own Transform (``Transform.clone()`` creates one with its own grid),
or order the streams.
"""
from __future__ import annotations

import torch

from . import SPFFT_FULL_SCALING, SPFFT_NO_SCALING, SPFFT_TRANS_R2C, Transform


def _complex_dtype(tr: Transform):
    return torch.complex128 if tr.dtype in ("float64", "double", "f64") else torch.complex64


def _real_dtype(tr: Transform):
    return torch.float64 if tr.dtype in ("float64", "double", "f64") else torch.float32


def _space_like(tr: Transform, device) -> torch.Tensor:
    shape = (tr.dim_z(), tr.dim_y(), tr.dim_x())
    dt = _real_dtype(tr) if tr.type() == SPFFT_TRANS_R2C else _complex_dtype(tr)
    return torch.empty(shape, dtype=dt, device=device)


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class _Backward(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values: torch.Tensor, tr: Transform):
        values = values.contiguous().to(_complex_dtype(tr))
        space = _space_like(tr, values.device)
        tr.backward_device(values, space, _stream())
        ctx.tr = tr
        return space

    @staticmethod
    def backward(ctx, grad_space: torch.Tensor):
        tr = ctx.tr
        g = grad_space.contiguous()
        grad_values = torch.empty(tr.num_local_elements(), dtype=_complex_dtype(tr), device=g.device)
        tr.adjoint_backward(g, grad_values, _stream())
        return grad_values, None


class _Forward(torch.autograd.Function):
    @staticmethod
    def forward(ctx, space: torch.Tensor, tr: Transform, scaling: int):
        dt = _real_dtype(tr) if tr.type() == SPFFT_TRANS_R2C else _complex_dtype(tr)
        space = space.contiguous().to(dt)
        values = torch.empty(tr.num_local_elements(), dtype=_complex_dtype(tr), device=space.device)
        tr.forward_device(space, values, scaling, _stream())
        ctx.tr, ctx.scaling = tr, scaling
        return values

    @staticmethod
    def backward(ctx, grad_values: torch.Tensor):
        tr = ctx.tr
        g = grad_values.contiguous().to(_complex_dtype(tr))
        grad_space = _space_like(tr, g.device)
        tr.adjoint_forward(g, grad_space, ctx.scaling, _stream())
        return grad_space, None, None


def backward(tr: Transform, values: torch.Tensor) -> torch.Tensor:
    """Differentiable frequency -> space transform of `values` (complex, on the GPU)."""
    return _Backward.apply(values, tr)


def forward(tr: Transform, space: torch.Tensor, scaled: bool = False) -> torch.Tensor:
    """Differentiable space -> frequency transform of `space` (on the GPU)."""
    return _Forward.apply(space, tr, SPFFT_FULL_SCALING if scaled else SPFFT_NO_SCALING)
