"""ctypes binding of the C ABI in ``include/dtmm_gb300.h``.

The library is built in-tree (``dtmm_gb300/_lib/libdtmm_gb300.so``).  Loading
it never falls back to anything else: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

DTMM_OK = 0
DTMM_EINVAL = -1
DTMM_ENOSPACE = -2
DTMM_ECUDA = -3
DTMM_ENOTSUP = -4

PRECISION_MIXED = 0
PRECISION_DOUBLE = 1
DIFFRACTION_FULL = -1  # diffraction = inf

ABI_SYMBOLS = ("dtmm_abi_version", "dtmm_last_error", "dtmm_transfer_workspace_size", "dtmm_transfer",
               "dtmm_transfer_timed", "dtmm_transfer_noalloc", "dtmm_planewave_field", "dtmm_pom_field",
               "dtmm_field2specter", "dtmm_specter2color", "dtmm_pom_image", "dtmm_director2data",
               "dtmm_diffract_workspace_size", "dtmm_diffract", "dtmm_q2data", "dtmm_wave_field",
               "dtmm_field_diffraction_matrix", "dtmm_field_intensity", "dtmm_scale_fields",
               "dtmm_twisted_nematic_angles")
ABI_VERSION = 7
STATIC_SCRATCH_BYTES = 64 << 20


class TransferDesc(ctypes.Structure):
    _fields_ = [
        ("height", ctypes.c_int),
        ("width", ctypes.c_int),
        ("nlam", ctypes.c_int),
        ("npol", ctypes.c_int),
        ("nray", ctypes.c_int),
        ("method", ctypes.c_int),
        ("diffraction", ctypes.c_int),
        ("reflection", ctypes.c_int),
        ("npass", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("betamax", ctypes.c_double),
        ("nin", ctypes.c_double),
        ("nout", ctypes.c_double),
        ("smooth", ctypes.c_double),
        ("nlayers", ctypes.c_int),
        ("thickness", ctypes.POINTER(ctypes.c_double)),
        ("nstep", ctypes.POINTER(ctypes.c_int)),
        ("epsv", ctypes.c_void_p),
        ("eps_complex", ctypes.c_int),
        ("epsv_strides", ctypes.c_longlong * 3),
        ("epsa", ctypes.c_void_p),
        ("epsa_strides", ctypes.c_longlong * 3),
        ("ks", ctypes.POINTER(ctypes.c_double)),
        ("beta", ctypes.POINTER(ctypes.c_double)),
        ("phi", ctypes.POINTER(ctypes.c_double)),
        ("op_cache_bytes", ctypes.c_size_t),
        ("real_path", ctypes.c_int),
        ("row_group", ctypes.c_int),
        ("col_tile", ctypes.c_int),
        ("fft_schedule", ctypes.c_int),
        ("biaxial", ctypes.c_int),
        ("norm_total", ctypes.c_int),
        ("layer_block", ctypes.POINTER(ctypes.c_int)),
        ("norm_ref", ctypes.c_int),
        ("block_sym", ctypes.POINTER(ctypes.c_int)),
        ("block_eff", ctypes.POINTER(ctypes.c_double)),
    ]


class PomDesc(ctypes.Structure):
    _fields_ = [
        ("height", ctypes.c_int),
        ("width", ctypes.c_int),
        ("nlam", ctypes.c_int),
        ("nset", ctypes.c_int),
        ("npol", ctypes.c_int),
        ("jvec", ctypes.c_double * 4),
        ("pmat", ctypes.c_void_p),
        ("window", ctypes.c_void_p),
        ("precision", ctypes.c_int),
    ]


class TransferIO(ctypes.Structure):
    _fields_ = [
        ("field_in", ctypes.c_void_p),
        ("field_out", ctypes.c_void_p),
        ("out_given", ctypes.c_int),
        ("bulk", ctypes.c_void_p),
    ]


class KernelTimes(ctypes.Structure):
    _fields_ = [
        ("layer_row_ms", ctypes.c_double),
        ("layer_col_ms", ctypes.c_double),
        ("voxel_op_ms", ctypes.c_double),
        ("layer_row_launches", ctypes.c_int),
        ("layer_col_launches", ctypes.c_int),
        ("voxel_op_launches", ctypes.c_int),
        ("total_launches", ctypes.c_int),
    ]


class DtmmError(RuntimeError):
    """A failure reported by the GPU engine (negative status)."""

    def __init__(self, code, msg):
        super().__init__("dtmm_gb300 engine error %d: %s" % (code, msg))
        self.code = code


_LIB = None


def load(build_if_missing=True):
    """Load (building in-tree if needed) and return the ctypes library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.lib_path()
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise ImportError("dtmm_gb300 CUDA library not built: %s" % path)
    lib = ctypes.CDLL(path)
    lib.dtmm_abi_version.restype = ctypes.c_int
    lib.dtmm_abi_version.argtypes = []
    lib.dtmm_last_error.restype = ctypes.c_char_p
    lib.dtmm_last_error.argtypes = []
    lib.dtmm_transfer_workspace_size.restype = ctypes.c_size_t
    lib.dtmm_transfer_workspace_size.argtypes = [ctypes.POINTER(TransferDesc)]
    lib.dtmm_transfer.restype = ctypes.c_int
    lib.dtmm_transfer.argtypes = [ctypes.POINTER(TransferDesc), ctypes.POINTER(TransferIO), ctypes.c_void_p,
                                  ctypes.c_size_t, ctypes.c_void_p]
    lib.dtmm_transfer_timed.restype = ctypes.c_int
    lib.dtmm_transfer_timed.argtypes = [ctypes.POINTER(TransferDesc), ctypes.POINTER(TransferIO), ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(KernelTimes)]
    lib.dtmm_transfer_noalloc.restype = ctypes.c_int
    lib.dtmm_transfer_noalloc.argtypes = [ctypes.POINTER(TransferDesc), ctypes.POINTER(TransferIO), ctypes.c_void_p]
    lib.dtmm_planewave_field.restype = ctypes.c_int
    lib.dtmm_planewave_field.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_pom_field.restype = ctypes.c_int
    lib.dtmm_pom_field.argtypes = [ctypes.POINTER(PomDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_field2specter.restype = ctypes.c_int
    lib.dtmm_field2specter.argtypes = [ctypes.c_int] * 6 + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_specter2color.restype = ctypes.c_int
    lib.dtmm_specter2color.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p]
    lib.dtmm_pom_image.restype = ctypes.c_int
    lib.dtmm_pom_image.argtypes = [ctypes.POINTER(PomDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_director2data.restype = ctypes.c_int
    lib.dtmm_director2data.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_wave_field.restype = ctypes.c_int
    lib.dtmm_wave_field.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p,
                                                                              ctypes.c_void_p]
    lib.dtmm_field_diffraction_matrix.restype = ctypes.c_int
    lib.dtmm_field_diffraction_matrix.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] + [ctypes.c_double] * 3 + [
        ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_field_intensity.restype = ctypes.c_int
    lib.dtmm_field_intensity.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 3
    lib.dtmm_scale_fields.restype = ctypes.c_int
    lib.dtmm_scale_fields.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 5
    lib.dtmm_twisted_nematic_angles.restype = ctypes.c_int
    lib.dtmm_twisted_nematic_angles.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] + [
        ctypes.c_double] * 4 + [ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_q2data.restype = ctypes.c_int
    lib.dtmm_q2data.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_double] * 4 + [
        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dtmm_diffract_workspace_size.restype = ctypes.c_size_t
    lib.dtmm_diffract_workspace_size.argtypes = [ctypes.c_int] * 5
    lib.dtmm_diffract.restype = ctypes.c_int
    lib.dtmm_diffract.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_void_p]
    if lib.dtmm_abi_version() != ABI_VERSION:
        raise ImportError("dtmm_gb300 library ABI mismatch")
    _LIB = lib
    return lib


def last_error():
    return load().dtmm_last_error().decode()


def check(code):
    if code != DTMM_OK:
        msg = last_error()
        if code == DTMM_EINVAL:
            raise ValueError(msg)
        if code == DTMM_ENOTSUP:
            raise NotImplementedError(msg)
        raise DtmmError(code, msg)
