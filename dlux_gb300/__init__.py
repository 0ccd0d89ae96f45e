"""dlux_gb300: GB300-native diffraction hot path with dLux's API.

Import as ``import dlux_gb300 as dl`` and ``import dlux_gb300.utils as dlu`` in
place of ``dLux`` / ``dLux.utils``. The compute path is the CUDA library
``libdluxgb.so`` (hand-written sm_103a kernels behind a C ABI); there is no
host fallback.
"""

from . import utils  # noqa: F401
from . import layers  # noqa: F401
from .base import Base  # noqa: F401
from .coordinates import CoordSpec, PadSpec  # noqa: F401
from .wavefronts import Wavefront  # noqa: F401
from .psfs import PSF  # noqa: F401
from .layers import (CoordTransform, CircularAperture, SquareAperture,  # noqa: F401
                     RectangularAperture, RegPolyAperture, AberratedAperture)
from .layers import (OpticalLayer, TransmissiveLayer, AberratedLayer, BasisLayer,  # noqa: F401
                     Tilt, Normalise, Optic, BasisOptic, MFT, FFT, DetectorLayer,
                     ApplyPixelResponse, Downsample, AddConstant, ApplySaturation,
                     ApplyJitter)
from .optical_systems import (OpticalSystem, LayeredOpticalSystem,  # noqa: F401
                              ParametricLayeredOpticalSystem, AngularOpticalSystem,
                              CartesianOpticalSystem)
from .spectra import Spectrum  # noqa: F401
from .sources import PointSource, PointSources, ResolvedSource, PointResolvedSource  # noqa: F401
from .detectors import LayeredDetector  # noqa: F401
from .instruments import Telescope  # noqa: F401
from .kernels import set_variant, get_variant, tensor_core_available  # noqa: F401

__version__ = "0.1.0"
