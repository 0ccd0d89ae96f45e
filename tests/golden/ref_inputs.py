"""Seeded inputs of the reference-made golden fixtures (tests/golden/ref_*.npz).

Shared by the generator (make_ref_golden.py, which runs dLux itself) and by the
tests that compare the oracle and the CUDA path with the fixtures. Every
random array comes from the PCG64 bit stream through ``Generator.random``
(raw 53-bit doubles) and the Box-Muller transform written out here, so the
inputs do not depend on NumPy's choice of normal or Dirichlet sampler.
"""

from __future__ import annotations

import numpy as np

ARCSEC = np.pi / 180.0 / 3600.0


def uniform(rng, shape=None):
    return rng.random(shape)


def normal(rng, shape=None):
    """Standard normal draws by Box-Muller from two uniform streams."""
    n = int(np.prod(shape)) if shape is not None else 1
    u1 = 1.0 - rng.random(n)  # (0, 1]
    u2 = rng.random(n)
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return z.reshape(shape) if shape is not None else float(z[0])


def dirichlet_ones(rng, n):
    """Dirichlet(1, ..., 1): normalised Exp(1) draws."""
    e = -np.log(1.0 - rng.random(n))
    return e / e.sum()


def field(seed, n):
    """A seeded complex field [n, n] for the transform fixtures."""
    rng = np.random.default_rng(seed)
    return (normal(rng, (n, n)) + 1j * normal(rng, (n, n))) / n


def case_field(name, n, salt=0):
    """The input field of the transform case called `name`."""
    return field(sum(map(ord, name)) + salt, n)


# Transform cases: (name, n_in, n_out, pixel_scale_in, pixel_scale_out, focal_length,
# shift, pixel, inverse, wavelength). Sizes cover the benchmark configurations'
# pupil -> focal transforms: 256 -> 128 (config 1), 512 -> 512 (config 2),
# 512 -> 256 (config 3), 1024 -> 128 (config 4).
MFT_CASES = [
    ("small_focal_shift", 32, 16, 0.1, 0.05, 2.0, (1.0, -2.0), True, False, 1.0),
    ("small_unit_shift_inverse", 32, 16, 0.1, 0.05, 2.0, (1.0, -2.0), False, True, 1.0),
    ("odd_inverse", 33, 17, 0.03, 1e-7, None, (-2.5, 0.5), True, True, 0.8e-6),
    ("cfg1", 256, 128, 1 / 256, 0.02 * ARCSEC, None, (0.0, 0.0), True, False, 1.0e-6),
    ("cfg1_shift", 256, 128, 1 / 256, 0.02 * ARCSEC, None, (3.5, -1.25), True, False, 1.0e-6),
    ("cfg2", 512, 512, 1 / 512, 0.005 * ARCSEC, None, (0.0, 0.0), True, False, 0.8e-6),
    ("cfg3", 512, 256, 1 / 512, 0.02 * ARCSEC, None, (0.0, 0.0), True, False, 1.1e-6),
    ("cfg4", 1024, 128, 1 / 1024, 0.02 * ARCSEC, None, (0.0, 0.0), True, False, 1.2e-6),
]

# FFT cases: (name, n, pixel_scale, wavelength, focal_length, pad, inverse).
FFT_CASES = [
    ("pad1", 64, 1 / 64, 1e-6, None, 1, False),
    ("pad2", 64, 1 / 64, 1e-6, None, 2, False),
    ("pad3", 64, 1 / 64, 1e-6, None, 3, False),
    ("pad2_focal", 64, 1 / 64, 0.9e-6, 5.0, 2, False),
    ("pad2_inverse", 64, 1 / 64, 1e-6, None, 2, True),
    ("odd_pad2", 33, 0.03, 1e-6, None, 2, False),
    ("n128_pad2", 128, 1 / 128, 1e-6, None, 2, False),
]


def cfg1():
    """Config 1: 256^2 pupil, Noll 4-13 ~ N(0, 50 nm), 1 um, 128^2 PSF at 0.02",
    loss sum(R * PSF)."""
    rng = np.random.default_rng(101)
    return {"coeffs": 50e-9 * normal(rng, 10), "R": normal(rng, (128, 128)),
            "wavelengths": np.array([1.0e-6]), "nolls": list(range(4, 14))}


def unaligned():
    """A system whose sides are not multiples of 8: 100^2 pupil (10% obscuration),
    Noll 4-9 ~ N(0, 50 nm), 4 wavelengths 0.9-1.1 um with Dirichlet(1) weights,
    67^2 PSF at 0.03", loss sum(R * PSF). (An odd pupil side is avoided: dLux's
    Zernike basis is NaN at the centre pixel of an odd grid.)"""
    rng = np.random.default_rng(107)
    return {"coeffs": 50e-9 * normal(rng, 6), "weights": dirichlet_ones(rng, 4),
            "R": normal(rng, (67, 67)), "wavelengths": np.linspace(0.9e-6, 1.1e-6, 4),
            "nolls": list(range(4, 10))}


def cfg2():
    """Config 2 (the benchmark): 512^2 pupil with spiders, Noll 4-24 ~ N(0, 30 nm),
    64 wavelengths 0.8-1.2 um with Dirichlet(1) weights, 512^2 focal at 4x
    oversampling, 4 x 4 sum downsample to 128^2, loss sum(R * image)."""
    rng = np.random.default_rng(102)
    return {"coeffs": 30e-9 * normal(rng, 21), "weights": dirichlet_ones(rng, 64),
            "R": normal(rng, (128, 128)), "wavelengths": np.linspace(0.8e-6, 1.2e-6, 64),
            "nolls": list(range(4, 25))}


def cfg3():
    """Config 3 (phase retrieval): 512^2 pupil, amplitude T (1 + N(0, 0.01)), Noll 4-39
    ~ N(0, 40 nm), 32 wavelengths 0.9-1.1 um equal weights, 256^2 detector at 0.02"
    with flat field 1 + N(0, 0.02); Poisson NLL of stored data. The directions of
    the amplitude and flat-field derivatives are seeded fields too."""
    rng = np.random.default_rng(103)
    return {"coeffs": 40e-9 * normal(rng, 36), "amp_pert": 0.01 * normal(rng, (512, 512)),
            "flat": 1.0 + 0.02 * normal(rng, (256, 256)),
            "wavelengths": np.linspace(0.9e-6, 1.1e-6, 32), "nolls": list(range(4, 40)),
            "dir_amp": normal(rng, (2, 512, 512)), "dir_flat": normal(rng, (2, 256, 256))}


def cfg4():
    """Config 4 at its pupil, focal and wavelength sizes with 4 of its sources:
    1024^2 pupil, Noll 4-24 ~ N(0, 30 nm), positions U(-2, 2)", fluxes 10^U(2, 6),
    16 wavelengths 0.8-1.2 um, 128^2 image at 0.02", loss sum(R * image)."""
    rng = np.random.default_rng(104)
    return {"coeffs": 30e-9 * normal(rng, 21),
            "positions": (4.0 * uniform(rng, (4, 2)) - 2.0) * ARCSEC,
            "fluxes": 10.0 ** (2.0 + 4.0 * uniform(rng, 4)), "R": normal(rng, (128, 128)),
            "wavelengths": np.linspace(0.8e-6, 1.2e-6, 16), "nolls": list(range(4, 25)),
            "dir_pos": normal(rng, (2, 4, 2)) * ARCSEC, "dir_flux": normal(rng, (1, 4))}


def layers():
    """Small systems for the layer-type fixtures: 64^2 pupil (1 m, 10% obscuration),
    Noll 4-11 basis, 2 wavelengths, 32^2 focal grid at 0.04"; loss sum(R * PSF).
    OPD, phase and transmission perturbations and the derivative directions are
    seeded fields."""
    rng = np.random.default_rng(105)
    return {"coeffs": 40e-9 * normal(rng, 8), "R": normal(rng, (32, 32)),
            "wavelengths": np.array([0.9e-6, 1.1e-6]), "weights": np.array([0.4, 0.6]),
            "nolls": list(range(4, 12)), "opd": 30e-9 * normal(rng, (64, 64)),
            "phase": 0.2 * normal(rng, (64, 64)), "amp_pert": 0.05 * normal(rng, (64, 64)),
            "tilt": np.array([0.03, -0.02]) * ARCSEC,
            "dir_opd": 1e-8 * normal(rng, (64, 64)), "dir_phase": normal(rng, (64, 64)),
            "dir_amp": normal(rng, (64, 64))}


# Dynamic aperture shapes: (name, class name, positional arguments) of dLux's
# layers/apertures.py, all under APERTURE_TRANSFORM, softening 1.5 pixels,
# aberrated by Noll 4-14 (APERTURE_NOLLS) on a 128^2 grid over 1 m.
APERTURE_SHAPES = [
    ("circle", "CircularAperture", (0.42,), ("circle", 0.42)),
    ("square", "SquareAperture", (0.6,), ("square", 0.6)),
    ("rectangle", "RectangularAperture", (0.5, 0.7), ("rectangle", 0.7, 0.5)),
    ("hexagon", "RegPolyAperture", (6, 0.45), ("polygon", 6, 0.45)),
    ("pentagon", "RegPolyAperture", (5, 0.44), ("polygon", 5, 0.44)),
]
APERTURE_TRANSFORM = dict(translation=(0.02, -0.015), rotation=0.3, compression=(1.05, 0.97),
                          shear=(0.03, -0.02))
APERTURE_NOLLS = list(range(4, 15))


def apertures():
    """Coefficients (N(0, 40 nm)), cotangent image and wavelengths of the aperture fixtures:
    the aberrated aperture alone on 128^2 pixels, and in a system to a 64^2 PSF at 0.03"."""
    rng = np.random.default_rng(106)
    return {"coeffs": 40e-9 * normal(rng, len(APERTURE_NOLLS)), "R": normal(rng, (64, 64)),
            "wavelengths": np.array([0.9e-6, 1.1e-6])}
