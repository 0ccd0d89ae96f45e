"""dLux-compatible utility namespace (``dlux_gb300.utils`` mirrors ``dLux.utils``)."""

from .units import *  # noqa: F401,F403
from .coordinates import nd_coords, pixel_coords, cart2polar, polar2cart  # noqa: F401
from .zernikes import (zernike_name, noll_indices, radial_orders_to_indices,  # noqa: F401
                       zernike_factors, zernike, zernike_fast, zernike_basis)
from .geometry import circle, spider, combine  # noqa: F401
from .apertures import circular_aperture  # noqa: F401
from .array_ops import pad_to, crop_to, resize, downsample  # noqa: F401
from .math import factorial, triangular_number, eval_basis  # noqa: F401
from .propagation import FFT, MFT, transfer_matrix, calc_nfringes  # noqa: F401
from .fourier import fft_spec, fft_phase_ramp  # noqa: F401
