"""NumPy restatement of dLux's diffraction hot path (TEST INFRASTRUCTURE ONLY).

See ``oracle/__init__.py`` for the role of this module. Each function cites the
dLux v0.16.0 file:line it restates (paths relative to the dLux project root).
``precision="f64"`` computes in float64/complex128; ``precision="c64"`` mirrors
dLux's float32/complex64 arithmetic in the same operation order.
"""

from __future__ import annotations

import math

import numpy as np

__all__ = [
    "dtypes",
    "nd_coords_1d",
    "pixel_coords",
    "arcsec2rad",
    "transfer_matrix",
    "calc_nfringes",
    "mft",
    "fft_prop",
    "fft_spec",
    "fft_phase_ramp",
    "coord_xs",
    "propagate_fft",
    "pad_to",
    "crop_to",
    "resize",
    "downsample",
    "noll_indices",
    "zernike_factors",
    "zernike",
    "zernike_fast",
    "zernike_basis",
    "eval_basis",
    "circle",
    "spider",
    "combine",
    "circular_aperture",
    "poly_psf",
    "poly_psf_fields",
    "poly_psf_grad",
    "abcd_free_space",
    "abcd_lens",
    "abcd_mirror",
    "abcd_fraunhofer",
    "compose_abcd",
    "lct_direct",
    "asm_prop",
]


def dtypes(precision: str):
    """Real and complex dtypes for a precision tag ("f64" or "c64")."""
    if precision == "f64":
        return np.float64, np.complex128
    if precision == "c64":
        return np.float32, np.complex64
    raise ValueError(f"unknown precision {precision!r}")


# --------------------------------------------------------------------------
# Coordinates: utils/coordinates.py, coordinates.py, utils/units.py
# --------------------------------------------------------------------------
def nd_coords_1d(n: int, scale: float, offset: float = 0.0, precision="f64"):
    """1-D pixel-centre coordinates: linspace(-(n-1)/2*s - o, (n-1)/2*s - o, n).

    Follows utils/coordinates.py:325-341 (``pixel_fn`` inside ``nd_coords``).
    """
    rt, _ = dtypes(precision)
    start = -(n - 1) / 2 * scale - offset
    end = (n - 1) / 2 * scale - offset
    return np.linspace(rt(start), rt(end), n, dtype=rt)


def pixel_coords(npixels: int, diameter: float, precision="f64"):
    """(x, y) meshgrid of pixel centres, indexing "xy" (utils/coordinates.py:208-266)."""
    rt, _ = dtypes(precision)
    pixscale = diameter / npixels
    xs = nd_coords_1d(npixels, pixscale, 0.0, precision)
    return np.array(np.meshgrid(xs, xs, indexing="xy")).astype(rt)


def arcsec2rad(values):
    """arcsec -> radians (utils/units.py:263-277)."""
    return np.asarray(values, np.float64) * (np.pi / (180.0 * 3600.0))


def coord_xs(n: int, d: float, c: float = 0.0):
    """CoordSpec.xs = c + (arange(n) - (n-1)/2) * d (coordinates.py:117-129)."""
    return c + (np.arange(n) - (n - 1) / 2) * d


# --------------------------------------------------------------------------
# MFT: utils/propagation.py:67-256
# --------------------------------------------------------------------------
def transfer_matrix(
    wavelength,
    npixels_in,
    pixel_scale_in,
    npixels_out,
    pixel_scale_out,
    shift=0.0,
    focal_length=None,
    focal_shift=0.0,
    inverse=False,
    precision="f64",
):
    """1-D DFT matrix exp(-+2 pi i outer(in_vec, out_vec)), shape [N_in, N_out].

    Follows utils/propagation.py:67-127.
    """
    rt, ct = dtypes(precision)
    wavelength = rt(wavelength)
    fringe_size = wavelength / (rt(pixel_scale_in) * rt(npixels_in))
    scale_in = rt(1.0) / rt(npixels_in)
    in_vec = nd_coords_1d(npixels_in, scale_in, rt(shift) * scale_in, precision)
    scale_out = rt(pixel_scale_out) / fringe_size
    if focal_length is not None:
        scale_out = scale_out / (rt(focal_length) + rt(focal_shift))
    out_vec = nd_coords_1d(npixels_out, scale_out, rt(shift) * scale_out, precision)
    matrix = ct(-2j * np.pi) * np.outer(in_vec, out_vec).astype(ct)
    if inverse:
        matrix = -matrix
    return np.exp(matrix).astype(ct)


def calc_nfringes(
    wavelength,
    npixels_in,
    pixel_scale_in,
    npixels_out,
    pixel_scale_out,
    focal_length=None,
    focal_shift=0.0,
    precision="f64",
):
    """Number of fringes spanned by the output plane (utils/propagation.py:130-175)."""
    rt, _ = dtypes(precision)
    diameter = rt(npixels_in) * rt(pixel_scale_in)
    fringe_size = rt(wavelength) / diameter
    output_size = rt(npixels_out) * rt(pixel_scale_out)
    if focal_length is not None:
        output_size = output_size / (rt(focal_length) + rt(focal_shift))
    return output_size / fringe_size


def mft(
    phasor,
    wavelength,
    pixel_scale_in,
    npixels_out,
    pixel_scale_out,
    focal_length=None,
    shift=(0.0, 0.0),
    pixel=True,
    inverse=False,
    precision="f64",
):
    """Matrix Fourier transform (Ay^T @ E) @ Ax, normalised (utils/propagation.py:178-256)."""
    rt, ct = dtypes(precision)
    phasor = np.asarray(phasor).astype(ct)
    npixels_in = phasor.shape[-1]
    shift = np.asarray(shift, np.float64).astype(rt)
    if not pixel:
        shift = shift / rt(pixel_scale_out)
    mats = [
        transfer_matrix(
            wavelength,
            npixels_in,
            pixel_scale_in,
            npixels_out,
            pixel_scale_out,
            s,
            focal_length,
            0.0,
            inverse,
            precision,
        )
        for s in shift
    ]
    x_mat, y_mat = mats
    out = (y_mat.T @ phasor) @ x_mat
    nfringes = calc_nfringes(
        wavelength, npixels_in, pixel_scale_in, npixels_out, pixel_scale_out,
        focal_length, 0.0, precision,
    )
    scale = np.exp(np.log(nfringes) - (np.log(rt(npixels_in)) + np.log(rt(npixels_out))))
    return (out * ct(scale)).astype(ct)


# --------------------------------------------------------------------------
# FFT propagation: utils/propagation.py:8-64, utils/fourier.py:14-78,
# wavefronts.py:654-727
# --------------------------------------------------------------------------
def fft_prop(phasor, wavelength, pixel_scale, focal_length=None, pad=2,
             inverse=False, precision="f64"):
    """Padded, centred FFT (utils/propagation.py:8-64). Returns (phasor, pixel_scale)."""
    rt, ct = dtypes(precision)
    phasor = np.asarray(phasor).astype(ct)
    npixels = phasor.shape[-1]
    fringe_size = wavelength / (pixel_scale * npixels)
    new_pixel_scale = fringe_size / pad
    if focal_length is not None:
        new_pixel_scale *= focal_length
    npad = (npixels * (pad - 1)) // 2
    phasor = np.pad(phasor, npad)
    if inverse:
        out = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(phasor)))
        out = out * out.shape[-1]
    else:
        out = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(phasor)))
        out = out / out.shape[-1]
    return out.astype(ct), new_pixel_scale


def fft_spec(npixels_in, pixel_scale_in, wavelength, focal_length=None):
    """Native FFT output sampling and centre offset (utils/fourier.py:14-45)."""
    d_out = wavelength / (npixels_in * pixel_scale_in)
    if focal_length is not None:
        d_out = d_out * focal_length
    if npixels_in % 2 != 0:
        return d_out, 0.0
    return d_out, -0.5 * d_out


def fft_phase_ramp(xs, wavelength, shift, focal_length=None, inverse=False):
    """Separable 2-D phase ramp exp(+-2 pi i xs shift / alpha) (utils/fourier.py:48-78)."""
    sign = -1 if inverse else 1
    alpha = wavelength if focal_length is None else wavelength * focal_length
    ramp = np.exp(sign * 2j * np.pi * np.asarray(xs) * shift / alpha)
    return ramp[None, :] * ramp[:, None]


def propagate_fft(phasor, wavelength, pixel_scale, center=0.0, pad=2,
                  focal_length=None, spec_out_c=None, inverse=False):
    """Wavefront.propagate_FFT (wavefronts.py:654-727), FP64.

    ``spec_out_c`` None means no output spec (no ramps); a float means
    CoordSpec(c=spec_out_c). Returns (phasor, pixel_scale, center).
    """
    n_in = phasor.shape[-1]
    n_out = n_in * pad
    d_fft, c_fft = fft_spec(n_out, pixel_scale, wavelength, focal_length)
    if spec_out_c is not None:
        shift = c_fft - spec_out_c
        in_ramp = fft_phase_ramp(coord_xs(n_in, pixel_scale, center), wavelength,
                                 shift, focal_length, inverse)
        shift2 = fft_spec(n_out, d_fft, wavelength, focal_length)[1]
        out_ramp = fft_phase_ramp(coord_xs(n_out, d_fft, spec_out_c), wavelength,
                                  shift2, focal_length, inverse)
        c_out = spec_out_c
    else:
        in_ramp, out_ramp = 1.0, 1.0
        c_out = c_fft
    out, ps = fft_prop(np.asarray(phasor) * in_ramp, wavelength, pixel_scale,
                       focal_length, pad, inverse)
    return out * out_ramp, ps, c_out


# --------------------------------------------------------------------------
# Array ops: utils/array_ops.py:12-162
# --------------------------------------------------------------------------
def pad_to(array, npixels, fill=0.0):
    """Centre-preserving zero pad (utils/array_ops.py:12-48)."""
    n_in = array.shape[-1]
    if n_in % 2 != npixels % 2:
        raise ValueError("Center-preserving padding requires parity consistency")
    if npixels < n_in:
        raise ValueError("Cannot pad to smaller size")
    return np.pad(array, (npixels - n_in) // 2, constant_values=fill)


def crop_to(array, npixels):
    """Centre-preserving crop (utils/array_ops.py:51-90)."""
    n_in = array.shape[-1]
    if n_in % 2 != npixels % 2:
        raise ValueError("Center-preserving cropping requires parity consistency")
    if npixels > n_in:
        raise ValueError("Cannot crop to larger size")
    start, stop = (n_in - npixels) // 2, (n_in + npixels) // 2
    return array[start:stop, start:stop]


def resize(array, npixels, fill=0.0):
    """Pad or crop to npixels (utils/array_ops.py:93-121)."""
    n_in = array.shape[-1]
    if npixels == n_in:
        return array
    if npixels < n_in:
        return crop_to(array, npixels)
    return pad_to(array, npixels, fill)


def downsample(array, n, mean=True):
    """k x k block sum or mean (utils/array_ops.py:124-162)."""
    array = np.asarray(array)
    if array.shape[0] != array.shape[1]:
        raise ValueError(f"Input array has shape {array.shape}, which is not square")
    if array.shape[0] % n != 0:
        raise ValueError(f"Input array has {array.shape[0]} pixels, not divisible by {n}")
    method = np.mean if mean else np.sum
    size_in = array.shape[0]
    size_out = size_in // n
    array = method(array.reshape((size_in * size_out, n)), 1)
    array = array.reshape(size_in, size_out).T
    array = method(array.reshape((size_out * size_out, n)), 1)
    return array.reshape(size_out, size_out).T


# --------------------------------------------------------------------------
# Zernikes: utils/zernikes.py:99-315, utils/math.py:137-196
# --------------------------------------------------------------------------
def noll_indices(j: int):
    """Noll index j -> (n, m) (utils/zernikes.py:99-119), integer restatement."""
    n = int(math.ceil(-0.5 + math.sqrt(1 + 8 * j) / 2) - 1)
    smallest_j_in_row = n * (n + 1) / 2 + 1
    number_of_shifts = (j - smallest_j_in_row + ~(n & 1) + 2) // 2
    sign_of_shift = -(j & 1) + ~(j & 1) + 2
    base_case = n & 1
    m = int(sign_of_shift * (base_case + number_of_shifts * 2))
    return n, m


def _factorial(x: float) -> float:
    """exp(lgamma(x + 1)), 1 at 0 (utils/math.py:137-154).

    lgamma has poles at the non-positive integers, where JAX returns +inf; the
    factorial of a negative integer is therefore +inf and the matching radial
    coefficient in ``zernike_factors`` becomes exactly 0, as in dLux.
    """
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
    sign = (-1.0) ** k
    f1 = np.array([_factorial(abs(n - kk)) for kk in k])
    f2 = np.array([_factorial(kk) for kk in k])
    f3 = np.array([_factorial(((n + m) // 2) - kk) for kk in k])
    f4 = np.array([_factorial(((n - m) // 2) - kk) for kk in k])
    c = sign * f1 / f2 / f3 / f4
    return c, k


def _eval_radial(rho, n, c, k):
    """sum_k c_k rho^(n - 2k) (utils/zernikes.py:153-175)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        rads = rho[..., None] ** (abs(n) - 2 * k)
        return (c * rads).sum(axis=-1)


def _eval_azimuthal(theta, n, m):
    """sqrt(n+1) * (sqrt 2 if m != 0) * cos/sin(|m| theta) (utils/zernikes.py:178-204)."""
    norm = math.sqrt(n + 1)
    if m != 0:
        norm *= 1 + (math.sqrt(2) - 1)
    trig = np.cos if m >= 0 else np.sin
    return norm * trig(abs(m) * theta)


def zernike_fast(n, m, c, k, coordinates, diameter=2.0):
    """Zernike from precomputed factors (utils/zernikes.py:257-294)."""
    coords = np.asarray(coordinates, np.float64) / (diameter / 2)
    rho = np.hypot(coords[0], coords[1])
    theta = np.arctan2(coords[1], coords[0])
    aperture = rho <= 1.0
    return aperture * _eval_radial(rho, n, c, k) * _eval_azimuthal(theta, n, m)


def zernike(j, coordinates, diameter=2.0):
    """Noll Zernike j on the unit disk of the given diameter (utils/zernikes.py:227-254)."""
    n, m = noll_indices(j)
    c, k = zernike_factors(j)
    return zernike_fast(n, m, c, k, coordinates, diameter)


def zernike_basis(js, coordinates, diameter=2.0):
    """Stack of Zernikes (utils/zernikes.py:297-315)."""
    return np.array([zernike(j, coordinates, diameter) for j in js])


def eval_basis(basis, coefficients):
    """tensordot over the leading coefficient dims (utils/math.py:177-196)."""
    coefficients = np.asarray(coefficients)
    basis = np.asarray(basis)
    if basis.shape[: coefficients.ndim] != coefficients.shape:
        raise ValueError("The leading basis dimensions must match the coefficient shape")
    axes = tuple(range(coefficients.ndim))
    return np.tensordot(basis, coefficients, axes=(axes, axes))


# --------------------------------------------------------------------------
# Static masks: utils/geometry.py, utils/apertures.py:153-242
# --------------------------------------------------------------------------
def circle(coords, radius, invert=False):
    """Hard-edged disk (utils/geometry.py:95-116)."""
    dist = np.hypot(coords[0], coords[1]) - radius
    return (dist > 0).astype(float) if invert else (dist < 0).astype(float)


def _rotate_coords(coords, rotation):
    """utils/coordinates.py:77-96."""
    x, y = coords
    new_x = np.cos(-rotation) * x + np.sin(-rotation) * y
    new_y = -np.sin(-rotation) * x + np.cos(-rotation) * y
    return np.array([new_x, new_y])


def spider(coords, width, angles):
    """Spider vanes as the complement of the union of half-strips (utils/geometry.py:195-216)."""
    blocked = np.zeros(coords.shape[1:], bool)
    for angle in angles:
        c = _rotate_coords(coords, np.deg2rad(angle))
        dist = np.maximum(np.abs(c[0]) - width / 2, c[1])
        blocked |= dist < 0
    return (~blocked).astype(float)


def combine(arrays, oversample=1, use_sum=False):
    """Product (or sum) of layers then downsample-mean (utils/geometry.py:20-46)."""
    method = np.sum if use_sum else np.prod
    arr = method(np.array(arrays), 0)
    if oversample == 1:
        return arr
    return downsample(arr, oversample)


def coord_transform(coords, translation=None, rotation=None, compression=None, shear=None):
    """CoordTransform.__call__ (coordinates.py:305-314): translate, shear, compress, rotate.

    translate: coords - t (utils/coordinates.py:23-39); shear: coords + coords^T * s,
    the transposed planes of a square xy grid (utils/coordinates.py:61-78); compress:
    coords * c (:42-58); rotate clockwise (:81-101).
    """
    coords = np.asarray(coords, np.float64)
    if translation is not None:
        coords = coords - np.asarray(translation, np.float64)[:, None, None]
    if shear is not None:
        coords = coords + np.transpose(coords, (0, 2, 1)) * np.asarray(shear, np.float64)[:, None, None]
    if compression is not None:
        coords = coords * np.asarray(compression, np.float64)[:, None, None]
    if rotation is not None:
        coords = _rotate_coords(coords, float(rotation))
    return coords


def soften(distances, clip_dist, invert=False):
    """Clip to +-clip_dist, then rescale by the array's min/max (utils/geometry.py:49-91)."""
    d = np.asarray(distances, np.float64)
    if invert:
        d = -d
    d = np.clip(d, -clip_dist, clip_dist)
    if d.max() == d.min():
        return (d > 0).astype(np.float64)
    return (d - d.min()) / (d.max() - d.min())


def soft_circle(coords, radius, clip_dist=0.1, invert=False):
    """utils/geometry.py:229-255 with circ_distance :405-418."""
    return soften(-(np.hypot(coords[0], coords[1]) - radius), clip_dist, invert)


def aberrated_circular_aperture(npixels, diameter, radius, noll, coefficients,
                                transformation=None, softening=1.0, occulting=False):
    """AberratedAperture(CircularAperture(radius, ...), noll, coefficients) on a
    wavefront of ``npixels`` over ``diameter``: (transmission, opd).

    Transmission: CircularAperture.transmission (layers/apertures.py:302-306) with
    clip = pixel_scale * softening / 2. OPD: eval_basis of the dynamic Zernikes at the
    transformed coordinates divided by the extent (= radius)
    (layers/apertures.py:754-771; polynomials.py:20-51, nsides = 0).
    """
    coords = pixel_coords(npixels, diameter)
    pixel_scale = diameter / npixels
    t = transformation or {}
    c = coord_transform(coords, **t)
    trans = soft_circle(c, radius, pixel_scale * softening / 2, occulting)
    basis = np.array([zernike(j, c / radius, 2.0) for j in noll])
    opd = np.tensordot(basis, np.asarray(coefficients, np.float64), axes=(0, 0))
    return trans, opd, basis


def square_distance(coords, width):
    """utils/geometry.py:421-437."""
    return np.max(np.abs(coords), axis=0) - width / 2


def rectangle_distance(coords, width, height):
    """utils/geometry.py:440-460."""
    return np.maximum(np.abs(coords[0]) - width / 2, np.abs(coords[1]) - height / 2)


def reg_polygon_edges(n, radius):
    """Slope and a point of each edge of a regular polygon (utils/geometry.py:519-552):
    vertices at angles linspace(-pi, pi, n, endpoint=False); a vertical edge's slope is
    the fill value inf of utils/math.py nandiv."""
    ang = np.linspace(-np.pi, np.pi, n, endpoint=False)
    x, y = radius * np.cos(ang), radius * np.sin(ang)
    j = np.roll(np.arange(n), -1)
    dx, dy = x[j] - x, y[j] - y
    m = np.where(dx == 0, np.inf, dy / np.where(dx == 0, 1.0, dx))
    return m, np.stack([x, y], 1)


def line_distance(coords, m, xy):
    """Signed distance from an edge line (utils/geometry.py:486-516)."""
    x, y = coords
    if m == 0:
        sgn, dist = np.sign(xy[1]), xy[1] - y
    elif m == np.inf:
        sgn, dist = np.sign(xy[0]), xy[0] - x
    else:
        sgn = np.sign(xy[1] - m * xy[0])
        dist = (m * x - y + xy[1] - m * xy[0]) / np.sqrt(m ** 2 + 1)
    return -sgn * dist


def reg_polygon_distance(coords, nsides, radius):
    """utils/geometry.py:560-579: the largest edge distance."""
    m, xy = reg_polygon_edges(nsides, radius)
    return np.max([line_distance(coords, mi, p) for mi, p in zip(m, xy)], axis=0)


def polike(nsides, j, coordinates, diameter=2.0):
    """Zernike j stretched onto a regular nsides-gon (utils/zernikes.py:318-352):
    in the angular wedge of each edge, radii are scaled by r_alpha = cos(alpha) /
    cos(u_alpha) and the value by 1 / r_alpha."""
    if nsides < 3:
        raise ValueError(f"nsides must be >= 3, not {nsides}.")
    c = np.asarray(coordinates, np.float64) / (diameter / 2)
    theta = np.arctan2(c[1], c[0])
    alpha = np.pi / nsides
    phi = theta + alpha
    wedge = np.floor((phi + alpha) / (2.0 * alpha))
    u_alpha = phi - wedge * (2 * alpha)
    r_alpha = np.cos(alpha) / np.cos(u_alpha)
    return 1 / r_alpha * zernike(j, c / r_alpha, 2.0)


def aberrated_aperture(shape, npixels, diameter, noll, coefficients, transformation=None,
                       softening=1.0, occulting=False):
    """AberratedAperture over a dynamic aperture of any shape on a wavefront of
    ``npixels`` over ``diameter``: (transmission, opd, basis).

    ``shape`` is ("circle", radius), ("square", width), ("rectangle", width, height) or
    ("polygon", nsides, rmax) (layers/apertures.py:240-555). The transmission is the
    shape's soft mask with clip = pixel_scale * softening / 2 (utils/geometry.py:229-351);
    the OPD evaluates the dynamic Zernikes at the transformed coordinates divided by the
    aperture's extent -- radius, sqrt(2) width, hypot(h / 2, w / 2) or rmax -- as Zernikes
    (circle) or polygon-stretched Zernikes with the aperture's side count (4 for squares
    and rectangles) (layers/apertures.py:754-771, polynomials.py:20-51).
    """
    coords = pixel_coords(npixels, diameter)
    pixel_scale = diameter / npixels
    t = transformation or {}
    c = coord_transform(coords, **t)
    kind = shape[0]
    if kind == "circle":
        dist, extent, nsides = np.hypot(c[0], c[1]) - shape[1], shape[1], 0
    elif kind == "square":
        dist, extent, nsides = square_distance(c, shape[1]), np.sqrt(2) * shape[1], 4
    elif kind == "rectangle":
        dist = rectangle_distance(c, shape[1], shape[2])
        extent, nsides = np.hypot(shape[2] / 2.0, shape[1] / 2.0), 4
    elif kind == "polygon":
        dist, extent, nsides = reg_polygon_distance(c, shape[1], shape[2]), shape[2], shape[1]
    else:
        raise ValueError(f"unknown aperture shape {kind!r}")
    trans = soften(-dist, pixel_scale * softening / 2, occulting)
    cz = c / extent
    basis = np.array([zernike(j, cz, 2.0) if nsides == 0 else polike(nsides, j, cz, 2.0)
                      for j in noll])
    opd = np.tensordot(basis, np.asarray(coefficients, np.float64), axes=(0, 0))
    return trans, opd, basis


def convolve_same(array, kernel):
    """jax.scipy.signal.convolve(array, kernel, mode="same") (psfs.py:93-110; sources.py:516,
    :745): the full 2-d convolution, cropped at offset (K - 1) // 2 per axis."""
    a = np.asarray(array, np.float64)
    k = np.asarray(kernel, np.float64)
    H, W = a.shape
    K0, K1 = k.shape
    full = np.zeros((H + K0 - 1, W + K1 - 1))
    for i in range(K0):
        for j in range(K1):
            full[i:i + H, j:j + W] += k[i, j] * a
    s0, s1 = (K0 - 1) // 2, (K1 - 1) // 2
    return full[s0:s0 + H, s1:s1 + W]


def gaussian_kernel(std, npixels, extent=5.0):
    """Normalised separable normal pdf on linspace(-extent, extent, n) (utils/math.py:20-69)."""
    x = np.linspace(-extent, extent, npixels)
    g = np.exp(-0.5 * (x / std) ** 2) / (std * math.sqrt(2 * math.pi))
    k = g[None, :] * g[:, None]
    return k / k.sum()


def jitter_kernel(sigma, kernel_size=9, oversample=3):
    """ApplyJitter.kernel (layers/detector_layers.py:181-196): summed down by oversample."""
    return downsample(gaussian_kernel(sigma, kernel_size * oversample), oversample, mean=False)


def circular_aperture(npixels, diameter, oversample=5, secondary_diameter=None,
                      spider_width=None, spider_angles=None, zernike_nolls=None,
                      zernike_oversize=0.01):
    """Transmission (and masked Zernike basis) of a circular telescope.

    Follows utils/apertures.py:153-242 (array_diameter = diameter).
    """
    coords = pixel_coords(npixels * oversample, diameter)
    layers = [circle(coords, diameter / 2)]
    if secondary_diameter is not None and secondary_diameter > 0:
        layers.append(circle(coords, secondary_diameter / 2, invert=True))
    if spider_width is not None:
        layers.append(spider(coords, spider_width, spider_angles))
    transmission = combine(layers, oversample)
    if zernike_nolls is None:
        return transmission
    coords = pixel_coords(npixels, diameter)
    basis = zernike_basis(zernike_nolls, coords, diameter * (1.0 + zernike_oversize))
    support = downsample(layers[0], oversample) > 0
    return transmission, basis * support[None]


# --------------------------------------------------------------------------
# Polychromatic PSF through a layered system and its gradient.
# optical_systems.py:147-223 (lambda vmap, sqrt(w), sum |E|^2),
# optical_systems.py:363-425 (init + tilt + layer loop), :659-680 (to_focus),
# wavefronts.py:70-122 (1/N^2 init), :332-424 (add_phase/opd, tilt, normalise),
# layers/optical_layers.py:181-186, 304-327; layers/optics.py:77-175.
# --------------------------------------------------------------------------
def poly_psf_fields(amplitude, opd, wavelengths, weights, diameter,
                    psf_npixels_os, pixel_scale_out_rad, phase=None,
                    offset=(0.0, 0.0), normalise=True, precision="f64"):
    """Focal fields F_l (already multiplied by sqrt(w_l)) for a system

    [TransmissiveLayer(amplitude, normalise), BasisLayer/AberratedLayer(opd)]
    + AngularOpticalSystem.to_focus. Returns (F [L, M, M], E [L, N, N]).
    """
    rt, ct = dtypes(precision)
    amplitude = np.asarray(amplitude).astype(rt)
    opd = np.asarray(opd).astype(rt)
    n = amplitude.shape[-1]
    pixel_scale = rt(diameter) / rt(n)
    xs = coord_xs(n, float(pixel_scale)).astype(rt)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Fs, Es = [], []
    for wl, w in zip(np.asarray(wavelengths, np.float64), np.asarray(weights, np.float64)):
        wl_r = rt(wl)
        k = rt(2 * np.pi) / wl_r
        # Wavefront.__init__: amplitude 1/N^2, phase 0 (wavefronts.py:111-113)
        E = np.full((n, n), rt(1.0) / rt(n) ** 2, dtype=ct)
        # tilt (wavefronts.py:370-395) -> add_opd(theta_x X + theta_y Y)
        tilt_opd = rt(offset[0]) * X + rt(offset[1]) * Y
        E = E * np.exp(ct(1j) * (k * tilt_opd).astype(ct))
        # TransmissiveLayer: *= T, then normalise("power") (wavefronts.py:397-424)
        E = E * amplitude
        if normalise:
            E = E * np.sqrt(rt(1.0) / np.sum(np.abs(E) ** 2)).astype(rt)
        # BasisLayer (effect "opd"): add_opd -> exp(1j * k * opd)
        E = E * np.exp(ct(1j) * (k * opd).astype(ct))
        if phase is not None:
            E = E * np.exp(ct(1j) * np.asarray(phase).astype(ct))
        # vmap body multiplies by sqrt(weight) (optical_systems.py:213-215)
        E = E * rt(w) ** rt(0.5)
        F = mft(E, wl, pixel_scale, psf_npixels_os, pixel_scale_out_rad,
                precision=precision)
        Fs.append(F)
        Es.append(E)
    return np.array(Fs), np.array(Es)


def poly_psf(amplitude, opd, wavelengths, weights, diameter, psf_npixels_os,
             pixel_scale_out_rad, phase=None, offset=(0.0, 0.0), normalise=True,
             precision="f64"):
    """Sum over wavelengths of |F_l|^2 (optical_systems.py:222-223)."""
    F, _ = poly_psf_fields(amplitude, opd, wavelengths, weights, diameter,
                           psf_npixels_os, pixel_scale_out_rad, phase, offset,
                           normalise, precision)
    return (np.abs(F) ** 2).sum(0)


def poly_psf_grad(amplitude, opd, wavelengths, weights, diameter, psf_npixels_os,
                  pixel_scale_out_rad, g_psf, phase=None, offset=(0.0, 0.0), precision="f64"):
    """Analytic reverse-mode of poly_psf for a cotangent g_psf [M, M].

    Returns dict with g_opd (d/d opd, metres), g_phase (d/d phase), g_amp
    (d/d the post-normalisation amplitude) and g_w (d/d weight per
    wavelength), i.e. the adjoint JAX derives for the graph of
    optical_systems.py:211-223 with the amplitude normalisation held outside
    (the kernel computes gradients w.r.t. the effective amplitude; the
    normalisation chain is host logic). Checked against central finite
    differences of poly_psf in tests/test_oracle.py. ``precision="c64"`` runs
    the same reverse pass in float32/complex64 (the stand-in for dLux's CPU
    gradient).
    """
    rt, ct = dtypes(precision)
    amplitude = np.asarray(amplitude).astype(rt)
    opd = np.asarray(opd).astype(rt)
    n = amplitude.shape[-1]
    pixel_scale = diameter / n
    xs = coord_xs(n, pixel_scale).astype(rt)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    g_psf = np.asarray(g_psf).astype(rt)
    g_opd = np.zeros((n, n), rt)
    g_phase = np.zeros((n, n), rt)
    g_amp = np.zeros((n, n), rt)
    g_w = []
    ph0 = np.zeros((n, n), rt) if phase is None else np.asarray(phase).astype(rt)
    for wl, w in zip(np.asarray(wavelengths, np.float64), np.asarray(weights, np.float64)):
        k = rt(2 * np.pi / wl)
        u = np.exp(ct(1j) * (k * (opd + rt(offset[0]) * X + rt(offset[1]) * Y) + ph0)).astype(ct)
        E = (rt(np.sqrt(w)) * amplitude * u).astype(ct)
        ay = transfer_matrix(wl, n, pixel_scale, psf_npixels_os, pixel_scale_out_rad,
                             precision=precision)
        ax = ay
        nf = calc_nfringes(wl, n, pixel_scale, psf_npixels_os, pixel_scale_out_rad)
        s = rt(nf / (n * psf_npixels_os))
        F = s * (ay.T @ E @ ax)
        Fbar = rt(2.0) * g_psf * F
        Ebar = s * (ay.conj() @ Fbar @ ax.conj().T)
        inner = np.conj(E) * Ebar
        g_opd += k * inner.imag
        g_phase += inner.imag
        g_amp += (rt(np.sqrt(w)) * np.conj(u) * Ebar).real
        g_w.append(inner.real.sum() / (2.0 * w))
    return {"g_opd": g_opd, "g_phase": g_phase, "g_amp": g_amp, "g_w": np.array(g_w)}


# --------------------------------------------------------------------------
# ABCD propagators: layers/abcd_propagators.py:1-491. Their arithmetic is in
# the abcdLux package (pyproject.toml:21, "abcdLux>=0.0.2"; abcd.*, lct.lct_prop,
# lct.lct_prop_fft, asm.asm_prop), which is not vendored with the reference
# and has no pinned version, so these restate the published methods: ray-
# transfer matrices, Collins' diffraction integral (the linear canonical
# transform) and the angular-spectrum method. The reference's own tests
# (tests/layers/test_abcd_propagators.py) pin shapes and errors only: parity
# of values is unpinned.
# --------------------------------------------------------------------------
def abcd_free_space(distance):
    """Free space over `distance` (abcd_propagators.py:36-66 -> abcd.abcd_free_space)."""
    return np.array([[1.0, float(distance)], [0.0, 1.0]])


def abcd_lens(focal_length):
    """Thin lens (abcd_propagators.py:69-103 -> abcd.abcd_lens)."""
    return np.array([[1.0, 0.0], [-1.0 / float(focal_length), 1.0]])


def abcd_mirror(radius):
    """Curved mirror of radius R (abcd_propagators.py:106-136 -> abcd.abcd_mirror)."""
    return np.array([[1.0, 0.0], [-2.0 / float(radius), 1.0]])


def abcd_fraunhofer(focal_length):
    """Front-to-back focal-plane system (abcd_propagators.py:139-173 -> abcd.abcd_fraunhofer)."""
    f = float(focal_length)
    return np.array([[0.0, f], [-1.0 / f, 0.0]])


def compose_abcd(matrices):
    """Elements applied in order compose as M_n ... M_1 (abcd_propagators.py:236-245)."""
    out = np.eye(2)
    for m in matrices:
        out = np.asarray(m, np.float64) @ out
    return out


def _lct_matrix(xs_in, xs_out, wavelength, M):
    A, B, D = float(M[0, 0]), float(M[0, 1]), float(M[1, 1])
    lb = float(wavelength) * B
    dx = float(xs_in[1] - xs_in[0]) if len(xs_in) > 1 else 1.0
    x = np.asarray(xs_in, np.float64)[None, :]
    u = np.asarray(xs_out, np.float64)[:, None]
    phase = (A * x * x - 2.0 * x * u + D * u * u) / (2.0 * lb)  # cycles
    return np.exp(2j * np.pi * phase) * dx / np.sqrt(1j * lb)


def lct_direct(u, xs_in, xs_out, wavelength, M):
    """Collins integral of an ABCD system on explicit grids (MFTPropagator,
    abcd_propagators.py:248-300 -> lct.lct_prop), both axes:
    u_out(x', y') = (i lambda B)^-1 sum u(x, y) exp(i pi / (lambda B) *
    (A (x^2 + y^2) - 2 (x x' + y y') + D (x'^2 + y'^2))) dx dy, in FP64."""
    K = _lct_matrix(xs_in, xs_out, wavelength, M)
    return K @ np.asarray(u, np.complex128) @ K.T


def asm_prop(u, pixel_scale, wavelength, distance, n_pad):
    """Angular-spectrum propagation (ASMPropagator, abcd_propagators.py:380-459
    -> asm.asm_prop): centred zero padding to n_pad, centred FFT, transfer
    function exp(2 pi i z sqrt(1/lambda^2 - f^2)) with evanescent decay,
    inverse FFT; same pixel scale. FP64."""
    u = np.asarray(u, np.complex128)
    n = u.shape[-1]
    lo = (n_pad - n) // 2
    up = np.zeros((n_pad, n_pad), np.complex128)
    up[lo:lo + n, lo:lo + n] = u
    U = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(up)))
    f = (np.arange(n_pad) - n_pad // 2) / (n_pad * float(pixel_scale))
    s = float(wavelength) ** 2 * (f[None, :] ** 2 + f[:, None] ** 2)
    zl = float(distance) / float(wavelength)
    prop = s <= 1.0
    H = np.where(prop, np.exp(2j * np.pi * zl * np.sqrt(np.where(prop, 1.0 - s, 0.0))),
                 np.exp(-2.0 * np.pi * zl * np.sqrt(np.where(prop, 0.0, s - 1.0))))
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(U * H)))
