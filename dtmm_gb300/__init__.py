"""GB300-native engine for dtmm's field-transfer hot path (``transfer_field``).

``transfer_field`` keeps the reference's signature and data model
((field, wavelengths, pixelsize) field data, [(thickness, eps, angles)]
optical data) and runs the transfer as hand-written sm_103a CUDA kernels
behind a C ABI (``include/dtmm_gb300.h``).
"""
from .transfer import DTMM_NORM_FFT, DTMM_NORM_REF, set_precision, transfer_field  # noqa: F401
from .illumination import illumination_data  # noqa: F401
from . import samples  # noqa: F401

__version__ = "0.1.0"
__all__ = ["transfer_field", "illumination_data", "set_precision", "samples", "DTMM_NORM_FFT", "DTMM_NORM_REF"]
