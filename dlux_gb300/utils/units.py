"""Angle-unit conversions (restating dLux utils/units.py:24-312 on the host)."""

from __future__ import annotations

import math

__all__ = [
    "unit_factor_to_rad", "convert", "rad2arcsec", "rad2deg", "rad2arcmin", "deg2rad",
    "deg2arcmin", "deg2arcsec", "arcmin2rad", "arcmin2deg", "arcmin2arcsec", "arcsec2rad",
    "arcsec2deg", "arcsec2arcmin",
]

_BASE_TO_RAD = {
    "rad": 1.0,
    "deg": math.pi / 180.0,
    "arcmin": math.pi / (180.0 * 60.0),
    "arcsec": math.pi / (180.0 * 3600.0),
}
_ALIASES = {
    "radian": "rad", "radians": "rad", "degree": "deg", "degrees": "deg", "am": "arcmin",
    "arcmins": "arcmin", "arcminute": "arcmin", "arcminutes": "arcmin", "as": "arcsec",
    "arcsecs": "arcsec", "arcsecond": "arcsec", "arcseconds": "arcsec",
}
_PREFIX = {"G": 1e9, "M": 1e6, "k": 1e3, "": 1.0, "m": 1e-3, "u": 1e-6, "n": 1e-9}
_SHORT = {"mas": ("m", "arcsec"), "uas": ("u", "arcsec"), "mrad": ("m", "rad"),
          "urad": ("u", "rad"), "nrad": ("n", "rad")}


def unit_factor_to_rad(unit: str) -> float:
    """Factor that converts a value in ``unit`` to radians."""
    u = str(unit)
    if u in _SHORT:
        p, base = _SHORT[u]
        return _PREFIX[p] * _BASE_TO_RAD[base]
    low = u.lower()
    if low in _BASE_TO_RAD:
        return _BASE_TO_RAD[low]
    if low in _ALIASES:
        return _BASE_TO_RAD[_ALIASES[low]]
    for p in ("G", "M", "k", "m", "u", "n"):
        if u.startswith(p):
            rest = u[len(p):].lower()
            rest = _ALIASES.get(rest, rest)
            if rest in _BASE_TO_RAD:
                return _PREFIX[p] * _BASE_TO_RAD[rest]
    raise ValueError(f"Unknown angular unit {unit!r}")


def convert(value, unit_in: str, unit_out: str, scale: float = 1.0):
    return value * (unit_factor_to_rad(unit_in) / (unit_factor_to_rad(unit_out) * scale))


def rad2arcsec(v): return convert(v, "rad", "arcsec")
def rad2deg(v): return convert(v, "rad", "deg")
def rad2arcmin(v): return convert(v, "rad", "arcmin")
def deg2rad(v): return convert(v, "deg", "rad")
def deg2arcmin(v): return convert(v, "deg", "arcmin")
def deg2arcsec(v): return convert(v, "deg", "arcsec")
def arcmin2rad(v): return convert(v, "arcmin", "rad")
def arcmin2deg(v): return convert(v, "arcmin", "deg")
def arcmin2arcsec(v): return convert(v, "arcmin", "arcsec")
def arcsec2rad(v): return convert(v, "arcsec", "rad")
def arcsec2deg(v): return convert(v, "arcsec", "deg")
def arcsec2arcmin(v): return convert(v, "arcsec", "arcmin")
