"""NumPy emulator of the split-precision tensor-core MFT (TEST INFRASTRUCTURE ONLY).

Models what the tcgen05 kernel computes: each real operand x is stored as
hi = round(x) and lo = round(x - hi) in a 16-bit float format (bf16 or fp16,
round-to-nearest-even), each real product is hi*hi + hi*lo + lo*hi (the
lo*lo term is dropped), accumulation is in (at least) float32, and the
intermediate half-transformed field is rounded to float32 before it is split
again. Used to state the precision a form can reach before and beside the
GPU runs.
"""

from __future__ import annotations

import numpy as np


def round_bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def round_fp16(x):
    """Round float32 values to IEEE half (nearest even), returned as float32."""
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


def split(x, fmt="bf16", scale=1.0):
    """hi/lo split of a real float32 array in the given 16-bit format.

    ``scale`` (a power of two) is applied before the split and removed after,
    as the fp16 form does to keep values inside the half range.
    """
    rnd = round_bf16 if fmt == "bf16" else round_fp16
    xs = np.asarray(x, np.float32) * np.float32(scale)
    hi = rnd(xs)
    lo = rnd(xs - hi)
    return hi.astype(np.float64) / scale, lo.astype(np.float64) / scale


def split_matmul(a, b, fmt="bf16", scale_a=1.0, scale_b=1.0):
    """Emulated complex a @ b with 3-product split of every real product."""
    arh, arl = split(a.real, fmt, scale_a)
    aih, ail = split(a.imag, fmt, scale_a)
    brh, brl = split(b.real, fmt, scale_b)
    bih, bil = split(b.imag, fmt, scale_b)

    def prod(xh, xl, yh, yl):
        return xh @ yh + xh @ yl + xl @ yh

    re = prod(arh, arl, brh, brl) - prod(aih, ail, bih, bil)
    im = prod(arh, arl, bih, bil) + prod(aih, ail, brh, brl)
    return (re + 1j * im).astype(np.complex64)


def split_matmul_gauss(a, b, fmt="bf16"):
    """Emulated complex a @ b with Gauss's three real products instead of
    four: P1 = ar br, P2 = ai bi, P3 = (ar + ai)(br + bi), re = P1 - P2,
    im = P3 - P1 - P2. Each real product is the same 3-product split; the
    operand sums are formed in float32 and then split. 9 split products per
    complex multiply-add instead of 12."""
    ar, ai = np.asarray(a.real, np.float32), np.asarray(a.imag, np.float32)
    br, bi = np.asarray(b.real, np.float32), np.asarray(b.imag, np.float32)

    def prod(x, y):
        xh, xl = split(x, fmt)
        yh, yl = split(y, fmt)
        return xh @ yh + xh @ yl + xl @ yh

    p1 = prod(ar, br)
    p2 = prod(ai, bi)
    p3 = prod(ar + ai, br + bi)
    return ((p1 - p2) + 1j * (p3 - p1 - p2)).astype(np.complex64)


def pow2_scale(x, target=2.0 ** 14):
    """Power-of-two factor that brings max|x| near ``target``."""
    m = float(np.max(np.abs(x)))
    if m == 0.0:
        return 1.0
    return 2.0 ** np.floor(np.log2(target / m))


def split_mft(E, ay, ax, s, fmt="bf16", product="four"):
    """Emulated two-step split MFT: s * (ay^T @ E) @ ax with a float32 intermediate.
    ``product``: "four" real products per complex one (the kernel's form) or
    "gauss" (three, split_matmul_gauss)."""
    if product == "gauss":
        t1 = split_matmul_gauss(ay.T, E, fmt)
        out = split_matmul_gauss(t1, ax, fmt)
        return (out * np.float32(s)).astype(np.complex64)
    if fmt == "fp16":
        sa = pow2_scale(np.concatenate([ay.real.ravel(), ay.imag.ravel()]))
        se = pow2_scale(np.concatenate([E.real.ravel(), E.imag.ravel()]))
        t1 = split_matmul(ay.T, E, fmt, sa, se)
        st = pow2_scale(np.concatenate([t1.real.ravel(), t1.imag.ravel()]))
        out = split_matmul(t1, ax, fmt, st, sa)
    else:
        t1 = split_matmul(ay.T, E, fmt)
        out = split_matmul(t1, ax, fmt)
    return (out * np.float32(s)).astype(np.complex64)
