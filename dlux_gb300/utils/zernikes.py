"""Noll Zernike polynomials (dLux utils/zernikes.py:24-315), host-side setup.

The Noll index map and radial coefficients are exact integer/float64
arithmetic; the basis is evaluated once per configuration in float64 and
stored as float32 on the device.
"""

from __future__ import annotations

import math

import numpy as np

from .coordinates import to_device

__all__ = ["zernike_name", "noll_indices", "radial_orders_to_indices", "zernike_factors",
           "zernike", "zernike_fast", "zernike_basis"]

_NAMES = {
    1: "Piston", 2: "Tilt X", 3: "Tilt Y", 4: "Defocus", 5: "Astig X", 6: "Astig Y",
    7: "Coma X", 8: "Coma Y", 9: "Trefoil X", 10: "Trefoil Y", 11: "Spherical",
    12: "2nd Astig X", 13: "2nd Astig Y", 14: "Quadrafoil X", 15: "Quadrafoil Y",
    16: "2nd Coma X", 17: "2nd Coma Y", 18: "2nd Trefoil X", 19: "2nd Trefoil Y",
    20: "Pentafoil X", 21: "Pentafoil Y", 22: "2nd Spherical", 23: "3rd Coma X",
    24: "3rd Coma Y", 25: "3rd Astig X", 26: "3rd Astig Y", 27: "Hexafoil X",
    28: "Hexafoil Y", 29: "4th Coma X", 30: "4th Coma Y", 31: "4th Astig X",
    32: "4th Astig Y", 33: "3rd Trefoil X", 34: "3rd Trefoil Y", 35: "Heptafoil X",
    36: "Heptafoil Y",
}


def zernike_name(j: int) -> str:
    return _NAMES[int(j)] if 1 <= j <= 36 else f"Zernike {int(j)}"


def radial_orders_to_indices(radial_orders):
    out = []
    for order in radial_orders:
        order = int(order)
        if order < 0:
            raise ValueError("radial_orders must contain non-negative integers.")
        first = order * (order + 1) // 2 + 1
        out.extend(range(first, first + order + 1))
    return out


def noll_indices(j: int):
    """Noll index -> (n, m): the row n, then m alternating in sign with the parity of j."""
    j = int(j)
    if j < 1:
        raise ValueError("The Zernike index must be greater than 0.")
    n = int(math.ceil((-1 + math.sqrt(1 + 8 * j)) / 2) - 1)
    first = n * (n + 1) // 2 + 1
    k = j - first  # position in the row
    # |m| runs n%2, n%2, n%2+2, n%2+2, ... (m = 0 appears once for even n)
    if n % 2 == 0:
        mag = 2 * ((k + 1) // 2)
    else:
        mag = 2 * (k // 2) + 1
    sign = -1 if (j % 2 == 1) else 1
    m = sign * mag if mag != 0 else 0
    return n, m


def _fact(x):
    if x == 0:
        return 1.0
    if x < 0 and float(x).is_integer():
        return math.inf
    return math.exp(math.lgamma(x + 1.0))


def zernike_factors(j: int):
    """Radial coefficients c_k and exponents k (utils/zernikes.py:122-150)."""
    if j < 1:
        raise ValueError("The Zernike index must be greater than 0.")
    n, m = noll_indices(j)
    k = np.arange(((n - m) // 2) + 1, dtype=np.float64)
    c = np.array([(-1.0) ** kk * _fact(abs(n - kk)) / _fact(kk) / _fact((n + m) // 2 - kk)
                  / _fact((n - m) // 2 - kk) for kk in k])
    return c, k


def _radial(rho, n, c, k):
    # Only the non-zero coefficients contribute; dLux's JAX form also evaluates
    # the zero ones (which gives 0 * inf = nan at rho == 0 for odd grids).
    out = np.zeros_like(rho)
    for ck, kk in zip(c, k):
        if ck != 0.0:
            out = out + ck * rho ** (abs(n) - 2 * kk)
    return out


def zernike_fast(n, m, c, k, coordinates, diameter=2.0, as_numpy=False):
    coords = np.asarray(coordinates.cpu() if hasattr(coordinates, "cpu") else coordinates,
                        np.float64) / (diameter / 2)
    rho = np.hypot(coords[0], coords[1])
    theta = np.arctan2(coords[1], coords[0])
    norm = math.sqrt(n + 1) * (math.sqrt(2) if m != 0 else 1.0)
    az = norm * (np.cos(abs(m) * theta) if m >= 0 else np.sin(abs(m) * theta))
    out = (rho <= 1.0) * _radial(rho, n, c, k) * az
    return out if as_numpy else to_device(out)


def zernike(j, coordinates, diameter=2.0, as_numpy=False):
    n, m = noll_indices(j)
    c, k = zernike_factors(j)
    return zernike_fast(n, m, c, k, coordinates, diameter, as_numpy)


def zernike_basis(js, coordinates, diameter=2.0, as_numpy=False):
    out = np.array([zernike(j, coordinates, diameter, as_numpy=True) for j in js])
    return out if as_numpy else to_device(out)
