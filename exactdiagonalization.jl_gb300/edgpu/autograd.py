"""Differentiable H*x: a torch.autograd.Function over the library's forward product, adjoint product
and coupling gradient.

This is the PyTorch counterpart of a ChainRulesCore.rrule for mul!(y, represent(rhsr, H(J)), x) (the
reference has no derivative rule; the forward is abstract_operator_representation.jl:110-118 with the
reduced row iterator of reduced_operator_representation.jl:57-85).  With H(J) = sum_c J_c H_c and an
upstream gradient gy of y (PyTorch's convention for complex tensors: gy = dL/dRe(y) + i dL/dIm(y)):

    dL/dx   = H^dagger gy                        (edgpu_mul_adjoint_device: the adjoint of the mul!
                                                  matrix, orbit phases recomputed, not stored)
    dL/dJ_c = Re <gy | H_c x>                    (edgpu_coupling_grad_device)

Both are exact for the linear map x -> H(J) x, so torch.autograd.gradcheck holds in FP64.

    y = edgpu.apply_hamiltonian(opr, x, J)        # x: CUDA complex tensor, J: real tensor (or None)
    loss = (gy.conj() * y).real.sum(); loss.backward()

The operator's couplings are set to J at the forward call and again at the backward call when they
changed in between, so several forward passes with different J may be differentiated later.
"""
from __future__ import annotations

import numpy as np

from .representation import coupling_grad, mul_, mul_adjoint_

_PREC_OF = {"torch.complex128": "fp64", "torch.complex64": "mixed"}


def _precision_of(x):
    try:
        return _PREC_OF[str(x.dtype)]
    except KeyError:
        raise TypeError(f"x must be complex128 (fp64 product) or complex64 (mixed product), not {x.dtype}")


def _set(opr, J):
    """Give the operator the couplings J (a real tensor) unless it has them already."""
    if J is None:
        return
    import torch
    v = J.detach().to("cpu", dtype=torch.float64).numpy()
    if not np.array_equal(opr.couplings, v):
        opr.set_couplings(v)


def _function():
    import torch

    class HamiltonianApply(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, J, opr):
            prec = _precision_of(x)
            xc = x.contiguous()
            _set(opr, J)
            y = torch.empty_like(xc)
            mul_(y, opr, xc, precision=prec)
            ctx.opr = opr
            ctx.prec = prec
            ctx.save_for_backward(xc, J if J is not None else torch.empty(0))
            ctx.has_J = J is not None
            return y

        @staticmethod
        def backward(ctx, gy):
            xc, J = ctx.saved_tensors
            opr, prec = ctx.opr, ctx.prec
            if ctx.has_J:
                _set(opr, J)
            gy = gy.contiguous().to(xc.dtype)
            gx = gJ = None
            if ctx.needs_input_grad[0]:
                gx = torch.empty_like(gy)
                mul_adjoint_(gx, opr, gy, precision=prec)
            if ctx.has_J and ctx.needs_input_grad[1]:
                g = coupling_grad(opr, xc, gy, precision=prec)
                gJ = torch.from_numpy(g).to(device=J.device, dtype=J.dtype)
            return gx, gJ, None

    return HamiltonianApply


_FN = None


def apply_hamiltonian(opr, x, J=None):
    """y = H(J) x, differentiable in x (CUDA complex tensor) and in the couplings J (real tensor with
    one entry per coupling of an operator created with coupling ids; None keeps the operator's own)."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(x, J, opr)
