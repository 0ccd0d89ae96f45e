"""dLux-compatible layer namespace (``dlux_gb300.layers`` mirrors ``dLux.layers``)."""

from .optical_layers import (BaseLayer, OpticalLayer, TransmissiveLayer,  # noqa: F401
                             AberratedLayer, BasisLayer, Tilt, Normalise)
from .optics import Optic, BasisOptic  # noqa: F401
from .propagators import MFT, FFT  # noqa: F401
from .detector_layers import (DetectorLayer, ApplyPixelResponse, Downsample,  # noqa: F401
                              AddConstant, ApplySaturation, ApplyJitter)
from .apertures import (CoordTransform, CircularAperture, SquareAperture,  # noqa: F401
                        RectangularAperture, RegPolyAperture, AberratedAperture)
from . import abcd_propagators  # noqa: F401
from .abcd_propagators import (ABCDElement, ABCDFreeSpace, ABCDLens, ABCDMirror,  # noqa: F401
                               ABCDConjugatePlane, ABCDPropagator, MFTPropagator,
                               FFTPropagator, ASMPropagator)
