"""Basis contraction and small math helpers (dLux utils/math.py:137-196)."""

from __future__ import annotations

import math as _m

import torch

from .. import autograd

__all__ = ["factorial", "triangular_number", "eval_basis"]


def factorial(n):
    n = float(n)
    return 1.0 if n == 0 else _m.exp(_m.lgamma(n + 1.0))


def triangular_number(n):
    return n * (n + 1) / 2


def eval_basis(basis, coefficients, base=None):
    """tensordot of the basis with the coefficients over the leading dims (device kernel)."""
    coefficients = torch.as_tensor(coefficients, dtype=torch.float32, device=basis.device)
    if tuple(basis.shape[: coefficients.dim()]) != tuple(coefficients.shape):
        raise ValueError("The leading basis dimensions must match the coefficient shape, "
                         f"received {tuple(basis.shape)} and {tuple(coefficients.shape)}.")
    return autograd.eval_basis(basis.to(torch.float32), coefficients, base)
