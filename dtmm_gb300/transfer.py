"""Drop-in ``transfer_field`` backed by the GB300 engine.

Same signature, defaults, option resolution, return values and in-place
behaviour as the reference's ``dtmm.transfer.transfer_field``
(dtmm/transfer.py:322-552).  Option resolution and the data model are Python;
the transfer itself is one call into the CUDA library
(``include/dtmm_gb300.h``).  Options outside the GPU path raise
``NotImplementedError`` -- there is no CPU fallback.

Extension: ``precision=`` selects the bulk arithmetic, "double" (complex128,
the reference's precision, the default) or "mixed" (complex64 bulk with the
FP64 eigen-solve and operator tables); ``set_precision`` changes the default.
"""
from __future__ import annotations

import ctypes
import warnings

import numpy as np

from . import _lib

# reference defaults (dtmm/dtmm.ini read by dtmm/conf.py:459-531)
BETAMAX = 0.8
SMOOTH = 0.1
N_COVER = 1.5
DTMM_NORM_FFT = 1 << 0
DTMM_NORM_REF = 1 << 1

_defaults = {
    "nin": N_COVER,
    "nout": N_COVER,
    # the ini file stores method = "2x2" and the reference reads the quotes
    # too (dtmm/conf.py:506): the default is the string '"2x2"', which selects
    # the 2x2 method and makes reflection resolve to 1
    "method": '"2x2"',
    "npass": 1,
    "diffraction": 1,
    "reflection": None,
    "eff_data": 0,
    "betamax": BETAMAX,
}
_precision = ["double"]


def set_precision(p):
    """Default bulk precision: "double" (complex128) or "mixed" (complex64 bulk, FP64 eigen-solve)."""
    if p not in ("double", "mixed"):
        raise ValueError("precision must be 'double' or 'mixed'")
    old = _precision[0]
    _precision[0] = p
    return old


def get_default_config_option(name, value=None):
    """(dtmm/conf.py:531)"""
    return _defaults[name] if value is None else value


def k0(wavelength, pixelsize=1.0):
    """2*pi/wavelength*pixelsize (dtmm/wave.py:280)."""
    return np.asarray(2 * np.pi / np.asarray(wavelength) * pixelsize, np.float64)


# ---------------------------------------------------------------------------
# optical data (dtmm/data.py:534-682, non-dispersive blocks)
# ---------------------------------------------------------------------------
def _validate_block(block, shape):
    thickness, material, angles = block
    if callable(material):
        # the reference's message for dispersive data outside split_wavelengths (dtmm/transfer.py:542-543)
        raise ValueError("You are using dispersive data, so you must use `split_wavelengths=True`")
    thickness = np.asarray(thickness, np.float64)
    material = np.asarray(material)
    material = material.astype(np.complex128 if np.iscomplexobj(material) else np.float64, copy=False)
    angles = np.asarray(angles, np.float64)
    if thickness.ndim == 0:
        thickness = thickness[None]
        material = material[None, ...]
        angles = angles[None, ...]
    elif thickness.ndim != 1:
        raise ValueError("Thickess dimension should be 1.")
    if material.ndim == 2:
        material = material[:, None, None, :]
    elif material.ndim == 3:
        material = material[:, None, :, :]
    elif material.ndim != 4:
        raise ValueError("Invalid material dimensions.")
    if angles.ndim == 2:
        angles = angles[:, None, None, :]
    elif angles.ndim == 3:
        angles = angles[:, None, :, :]
    n = len(thickness)
    target = (n,) + tuple(shape) + (3,)
    np.broadcast_shapes(material.shape, target)
    np.broadcast_shapes(angles.shape, target)
    return thickness, material, angles


def validate_optical_data(data, shape):
    if isinstance(data, list):
        return [_validate_block(b, shape) for b in data]
    warnings.warn("A single-block optical data must be a list of length 1. Converting optical data to list. "
                  "In the future, exception will be raised.", DeprecationWarning)
    return validate_optical_data([data], shape)


def is_optical_data_dispersive(optical_data):
    """True when a block's eps values are a callable of the wavelength (dtmm/data.py:1116-1122)."""
    blocks = optical_data if isinstance(optical_data, list) else [optical_data]
    return any(callable(b[1]) for b in blocks)


def evaluate_optical_data(optical_data, wavelength):
    """Blocks with callable (dispersive) eps values evaluated at one wavelength in
    nanometres (dtmm/data.py:684-693, as validate_optical_block does for
    split_wavelengths, dtmm/data.py:575-586); other blocks are returned as they are."""
    if not is_optical_data_dispersive(optical_data):
        return optical_data
    if np.ndim(wavelength) != 0:
        raise ValueError("dispersive optical data is evaluated at one wavelength per transfer; "
                         "use split_wavelengths=True")

    def ev(b):
        d, e, a = b
        return (d, e(wavelength) if callable(e) else e, a)

    if isinstance(optical_data, list):
        return [ev(b) for b in optical_data]
    return ev(optical_data)


def _compact(a, full_shape):
    """Device-upload form of a broadcastable (L,h,w,3) array: the distinct data
    plus element strides of the (layer, y, x) axes (0 on broadcast axes)."""
    a = np.asarray(a)
    b = np.broadcast_to(a, full_shape)
    idx = []
    for ax in range(3):
        idx.append(slice(None) if (b.strides[ax] != 0 and b.shape[ax] > 1) else slice(0, 1))
    if a.shape == tuple(full_shape) and all(i == slice(None) for i in idx):
        # nothing to compact: the caller's own (writeable) array, copied only if not contiguous
        base = np.ascontiguousarray(a)
    else:
        base = np.ascontiguousarray(b[tuple(idx)])
    strides = []
    step = 3
    for ax in (2, 1, 0):
        strides.append(step if base.shape[ax] > 1 else 0)
        step *= base.shape[ax]
    return base, tuple(reversed(strides))


# ---------------------------------------------------------------------------
# beam direction estimate for beta=None (dtmm/field.py:492, :866; window.py:33)
# ---------------------------------------------------------------------------
def _blackman(shape):
    ay, ax = (np.arange(-n / 2.0 + 0.5, n / 2.0 + 0.5) for n in shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    ny, nx = (n / 2 for n in shape)
    r = ((xx / nx) ** 2 + (yy / ny) ** 2) ** 0.5
    out = 0.42 + 0.5 * np.cos(np.pi * r) + 0.08 * np.cos(2 * np.pi * r)
    out[r >= 1.0] = 0.0
    return out


def _field2betaphi(field, ks, multiray):
    """Mean beta, phi of the input field; runs on the GPU with torch.fft on the
    already-uploaded field (input analysis before the transfer)."""
    import torch

    f = torch.fft.fft2(field * torch.as_tensor(_blackman(field.shape[-2:]), device=field.device, dtype=field.real.dtype))
    h, w = field.shape[-2:]
    fx = torch.as_tensor(np.fft.fftfreq(w), device=field.device, dtype=torch.float64)
    fy = torch.as_tensor(np.fft.fftfreq(h), device=field.device, dtype=torch.float64)
    l = (2 * np.pi / torch.as_tensor(np.asarray(ks, np.float64), device=field.device))[:, None, None]
    bx = l * fx[None, None, :]
    by = l * fy[None, :, None]
    s = (f.real.double() ** 2 + f.imag.double() ** 2)
    sx = (s * bx[:, None]).sum(dim=(-3, -2, -1))
    sy = (s * by[:, None]).sum(dim=(-3, -2, -1))
    ss = s.sum(dim=(-3, -2, -1))
    beta = (sx ** 2 + sy ** 2) ** 0.5 / ss
    phi = torch.atan2(sy, sx)
    beta = beta.cpu().numpy()
    phi = phi.cpu().numpy()
    if field.ndim > 4 and multiray:
        ax = tuple(range(1, field.ndim - 3))
        return beta.mean(axis=ax), phi.mean(axis=ax)
    return beta.mean(), phi.mean()


# ---------------------------------------------------------------------------
# the engine call
# ---------------------------------------------------------------------------
def _writeable(a):
    return a if a.flags.writeable else a.copy()


def split_blocks(optical_data):
    """One single-layer block per layer, each with its own effective medium
    (layered_data, dtmm/data.py:1516-1528), of validated blocks."""
    out = []
    for d, ev, ea in optical_data:
        for i in range(len(d)):
            out.append((d[i:i + 1], ev[i:i + 1] if ev.shape[0] > 1 else ev, ea[i:i + 1] if ea.shape[0] > 1 else ea))
    return out


_SYMMETRY = {"isotropic": 0, "uniaxial": 1, "biaxial": 2}


def _symmetry(arg):
    """Symmetry identifier -> 0 (isotropic), 1 (uniaxial) or 2 (biaxial; -1
    keeps the eigenvalues too), or a list of them (dtmm/data.py:1344-1362,
    :1276-1310)."""
    if isinstance(arg, str):
        if arg not in _SYMMETRY:
            raise ValueError("Invalid symmetry argument.")
        return _SYMMETRY[arg]
    if np.ndim(arg) == 0:
        if arg not in (0, 1, 2, -1):
            raise ValueError("Invalid symmetry argument.")
        return 2 if arg == -1 else int(arg)
    return [_symmetry(a) for a in arg]


def _is_effective_block(e):
    """An explicit effective block ``(thickness, epsv, epsa)`` rather than a
    symmetry (array): its eps values end in an axis of three (the reference
    first tries the argument as an optical block, dtmm/transfer.py:941-947)."""
    return (isinstance(e, tuple) and len(e) == 3 and not callable(e[1]) and np.ndim(e[1]) >= 1 and
            np.shape(e[1])[-1] == 3)


def effective_blocks(blocks, eff_data):
    """The blocks of validated optical data as the engine's blocks, with the
    effective medium of each one (dtmm/transfer.py:926-1005,
    dtmm/data.py:1364-1419): ``eff_data`` is one symmetry for every block or
    one entry per block -- a symmetry, a per-layer symmetry array (each layer
    averaged on its own, so that block becomes one block per layer), or an
    explicit effective block ``(thickness, epsv, epsa)`` homogeneous in each
    layer (one block per layer, its medium given).  Returns ``(blocks,
    block_sym, block_eff)``: ``block_sym`` per block 0 / 1 / 2 (isotropic /
    uniaxial / biaxial mean) or 3 (given), None when every block keeps its
    isotropic mean; ``block_eff`` the given media (rows of epsv re / im x 3,
    psi, theta, phi) or None."""
    nb = len(blocks)
    if isinstance(eff_data, (str, int, np.integer)):
        per = [eff_data] * nb
    else:
        per = list(eff_data)
        if len(per) != nb:
            raise ValueError("Number of elements in eff_data must match length of optical_data.")
    out, sym, given, split = [], [], [], False
    for (d, ev, ea), e in zip(blocks, per):
        if _is_effective_block(e):
            de, eve, eae = _validate_block(e, (1, 1))
            if len(de) != len(d) or not np.array_equal(de, d):
                # the effective layers' own thicknesses set the diffraction steps there
                raise NotImplementedError("effective blocks with layer thicknesses other than the optical "
                                          "block's are outside the GPU engine")
            eve = np.broadcast_to(eve, (len(d), 1, 1, 3))
            eae = np.broadcast_to(eae, (len(d), 1, 1, 3))
            split = True
            for i in range(len(d)):
                out.append((d[i:i + 1], ev[i:i + 1] if ev.shape[0] > 1 else ev, ea[i:i + 1] if ea.shape[0] > 1 else ea))
                sym.append(3)
                v = np.asarray(eve[i, 0, 0], np.complex128)
                given.append([v[0].real, v[0].imag, v[1].real, v[1].imag, v[2].real, v[2].imag,
                              *np.asarray(eae[i, 0, 0], np.float64)])
            continue
        s = _symmetry(e)
        if np.ndim(s) == 0:
            out.append((d, ev, ea))
            sym.append(s)
            given.append([0.0] * 9)
            continue
        if len(s) != len(d):
            raise ValueError("Shape of the symmetry argument is incompatible with block size.")
        split = True
        for i in range(len(d)):
            out.append((d[i:i + 1], ev[i:i + 1] if ev.shape[0] > 1 else ev, ea[i:i + 1] if ea.shape[0] > 1 else ea))
            sym.append(s[i])
            given.append([0.0] * 9)
    if not split and not any(sym):
        return blocks, None, None
    block_eff = np.ascontiguousarray(given, np.float64) if 3 in sym else None
    return out, sym, block_eff


def _aniso_blocks(block_sym, block_eff):
    """Some block's effective medium is uniaxial or biaxial (given media with
    three equal eigenvalues are isotropic)."""
    if block_sym is None:
        return False
    for b, s in enumerate(block_sym):
        if s in (1, 2):
            return True
        if s == 3:
            r = block_eff[b]
            if not (r[0] == r[2] == r[4] and r[1] == r[3] == r[5]):
                return True
    return False


def _joined(blocks, shape):
    """Validated blocks as one (thickness, epsv, epsa) of the whole stack: each
    block broadcast over the (y, x) axes along which any block varies, then
    concatenated along the layers; and the block of every layer."""
    var = [any(np.broadcast_shapes(b[k].shape, (1, 1, 1, 3))[ax] > 1 and np.asarray(b[k]).strides[ax] != 0
               for b in blocks for k in (1, 2)) for ax in (1, 2)]
    hv, wv = (shape[0] if var[0] else 1), (shape[1] if var[1] else 1)
    cplx = any(np.iscomplexobj(b[1]) for b in blocks)
    ev = np.concatenate([np.broadcast_to(np.asarray(b[1]), (len(b[0]), hv, wv, 3)) for b in blocks])
    ea = np.concatenate([np.broadcast_to(np.asarray(b[2]), (len(b[0]), hv, wv, 3)) for b in blocks])
    ev = ev.astype(np.complex128 if cplx else np.float64, copy=False)
    d = np.concatenate([np.asarray(b[0], np.float64) for b in blocks])
    lb = np.repeat(np.arange(len(blocks), dtype=np.int32), [len(b[0]) for b in blocks])
    return (d, ev, ea), lb


class _Material:
    """Optical data resident on the device (uploaded once per call, or kept by
    the caller): one block, or several joined along the layers with the block
    of every layer (each block keeps its own effective medium)."""

    def __init__(self, blocks, shape, device, block_sym=None, block_eff=None):
        import torch

        self.block_sym = None if block_sym is None else np.ascontiguousarray(block_sym, np.int32)
        self.block_eff = None if block_eff is None else np.ascontiguousarray(block_eff, np.float64)
        if isinstance(blocks, list) and len(blocks) > 1:
            block, self.layer_block = _joined(blocks, shape)
        else:
            block = blocks[0] if isinstance(blocks, list) else blocks
            self.layer_block = None
        d, epsv, epsa = block
        L = len(d)
        full = (L,) + tuple(shape) + (3,)
        ev, self.ev_strides = _compact(epsv, full)
        ea, self.ea_strides = _compact(epsa, full)
        self.eps_complex = bool(np.iscomplexobj(ev))
        # no host copies of arrays that already have the engine's dtype and layout
        # (read-only views of broadcast data are copied: torch wants writeable memory)
        ev = _writeable(np.ascontiguousarray(ev, np.complex128 if self.eps_complex else np.float64))
        flat = ev.reshape(-1, 3)
        # biaxial voxels take the general eigen-solve (complex FP64 path)
        self.biaxial = not bool(np.all(flat[:, 0] == flat[:, 1]))
        self.eps_min = float(np.min(ev)) if not self.eps_complex else None
        self.epsv = torch.from_numpy(ev).to(device)
        self.epsa = torch.from_numpy(_writeable(np.ascontiguousarray(ea, np.float64))).to(device)
        self.thickness = np.asarray(d, np.float64)
        self.nlayers = L


class DeviceMaterial:
    """Optical block already resident on the device.

    ``thickness`` is a host sequence of L layer thicknesses; ``epsv`` and
    ``epsa`` are device tensors (float64, or complex128 for absorbing
    ``epsv``) broadcastable to ``(L, H, W, 3)`` -- expanded axes cost no
    memory and reach the engine as zero strides.  Used by callers that keep
    director and eps state on the GPU between transfers.
    """

    def __init__(self, thickness, epsv, epsa, shape, eps_min=None, uniaxial=None):
        """``eps_min`` (smallest real eps) and ``uniaxial=True`` (no biaxial
        voxel) may be given by a caller that knows them, which skips the
        device reductions (and their host synchronisation) that would
        otherwise establish them."""
        import torch

        self.thickness = np.asarray(thickness, np.float64).reshape(-1)
        L = len(self.thickness)
        full = (L,) + tuple(shape) + (3,)
        ev = epsv.expand(full)
        ea = epsa.expand(full)
        if ev.dtype not in (torch.float64, torch.complex128) or ea.dtype != torch.float64:
            raise ValueError("epsv must be float64 or complex128 and epsa float64")
        if ev.stride(3) != 1 or ea.stride(3) != 1:
            raise ValueError("the last (component) axis of epsv and epsa must be contiguous")
        self.epsv, self.epsa = ev, ea
        self.layer_block = None
        self.ev_strides = tuple(int(x) for x in ev.stride()[:3])
        self.ea_strides = tuple(int(x) for x in ea.stride()[:3])
        self.eps_complex = bool(ev.is_complex())
        self.biaxial = False if uniaxial else not bool(torch.all(epsv[..., 0] == epsv[..., 1]))
        if self.eps_complex:
            self.eps_min = None
        else:
            self.eps_min = float(eps_min) if eps_min is not None else float(epsv.min())
        self.nlayers = L


class DevicePlan:
    """One resolved transfer bound to the device: descriptor, material and
    workspace, reusable for many input fields of the same shape.

    ``run(field_in, field_out)`` takes device tensors of shape
    ``(images..., 4, H, W)`` in the plan's complex dtype and enqueues the
    transfer on the current stream (nothing is copied to or from the host).
    """

    def __init__(self, field_shape, mat, ks, beta, phi, nray, npol, nlam, method, diffraction, reflection, npass,
                 nstep, betamax, nin, nout, smooth, precision, device, tuning=None, norm=DTMM_NORM_FFT,
                 block_sym=None):
        import torch

        self.lib = _lib.load()
        self.device = device
        self.precision = precision
        self.dtype = torch.complex128 if precision == "double" else torch.complex64
        self.field_shape = tuple(field_shape)
        self.mat = mat
        h, w = field_shape[-2:]
        L = mat.nlayers
        if mat.layer_block is not None and np.ndim(nstep) > 0:
            # the reference broadcasts nstep over each block's layers (dtmm/transfer.py:933)
            counts = np.bincount(mat.layer_block)
            nstep = np.concatenate([np.broadcast_to(np.asarray(nstep, np.int32), (c,)) for c in counts])
        self._keep = dict(
            thick=np.ascontiguousarray(mat.thickness, np.float64),
            nst=np.ascontiguousarray(np.broadcast_to(np.asarray(nstep, np.int32), (L,)), np.int32),
            ks=np.ascontiguousarray(ks, np.float64),
            beta=np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float64).reshape(-1), (nray,)), np.float64),
            phi=np.ascontiguousarray(np.broadcast_to(np.asarray(phi, np.float64).reshape(-1), (nray,)), np.float64),
        )
        k = self._keep
        d = _lib.TransferDesc()
        d.height, d.width = int(h), int(w)
        d.nlam, d.npol, d.nray = int(nlam), int(npol), int(nray)
        d.method = 4 if method == "4x4" else 2
        d.diffraction = _lib.DIFFRACTION_FULL if diffraction == np.inf else int(diffraction)
        d.reflection = int(reflection)
        d.npass = int(npass)
        d.precision = _lib.PRECISION_DOUBLE if precision == "double" else _lib.PRECISION_MIXED
        d.betamax, d.nin, d.nout, d.smooth = float(betamax), float(nin), float(nout), float(smooth)
        d.nlayers = L
        d.thickness = k["thick"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.nstep = k["nst"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        d.epsv = mat.epsv.data_ptr()
        d.eps_complex = int(mat.eps_complex)
        d.epsv_strides[:] = mat.ev_strides
        d.epsa = mat.epsa.data_ptr()
        d.epsa_strides[:] = mat.ea_strides
        d.ks = k["ks"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.beta = k["beta"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.phi = k["phi"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.op_cache_bytes = 0
        # real-arithmetic eigen-solve when every radicand is provably positive:
        # real uniaxial / isotropic eps with all eigenvalues above the largest
        # beam beta squared (biaxial voxels need the general complex solve)
        bmax = max(float(betamax), float(np.max(np.abs(k["beta"]))))
        d.real_path = int(mat.eps_min is not None and not mat.biaxial and mat.eps_min > bmax * bmax)
        d.biaxial = int(mat.biaxial)
        # norm = 0: the reference's "total" renormalisation between passes;
        # DTMM_NORM_FFT | DTMM_NORM_REF: the per-k one with a reference field
        d.norm_total = int(not (int(norm) & DTMM_NORM_FFT))
        d.norm_ref = int(bool(int(norm) & DTMM_NORM_REF))
        if mat.layer_block is not None:
            k["lb"] = np.ascontiguousarray(mat.layer_block, np.int32)
            d.layer_block = k["lb"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        if block_sym is None:
            block_sym = getattr(mat, "block_sym", None)
        if block_sym is not None:
            # the symmetry of every block's effective medium (0 isotropic, 1 uniaxial, 2 biaxial,
            # 3 given in block_eff)
            k["bs"] = np.ascontiguousarray(block_sym, np.int32)
            d.block_sym = k["bs"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        block_eff = getattr(mat, "block_eff", None)
        if block_eff is not None:
            k["be"] = np.ascontiguousarray(block_eff, np.float64)
            d.block_eff = k["be"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.desc = d
        self.set_tuning(**(tuning or {}))
        self.nbytes = int(self.lib.dtmm_transfer_workspace_size(ctypes.byref(d)))
        if self.nbytes == 0:
            msg = _lib.last_error()
            raise (NotImplementedError if ("supported" in msg or "factor" in msg or "above" in msg) else ValueError)(msg)
        self.workspace = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.updates = int(np.prod(field_shape[:-3])) * int(h) * int(w) * int(k["nst"].sum()) * int(npass)

    TUNABLES = ("fft_schedule", "row_group", "col_tile")

    def set_tuning(self, fft_schedule=0, row_group=0, col_tile=0):
        """Launch shapes and line-transform schedule (0 = the engine's own choice).

        ``row_group``/``col_tile`` change only how work is split into blocks
        (results are bit-identical); ``fft_schedule`` 1/2/3 selects the
        register two-step transform, radix-4-first or radix-8-first shared
        memory passes (results agree to rounding).
        """
        self.desc.fft_schedule = int(fft_schedule)
        self.desc.row_group = int(row_group)
        self.desc.col_tile = int(col_tile)

    @property
    def tuning(self):
        return {k: int(getattr(self.desc, k)) for k in self.TUNABLES}

    def capture(self, field_in, field_out, restore_from=None):
        """Capture one transfer of ``field_in`` -> ``field_out`` as a CUDA graph.

        With ``restore_from`` the graph first copies it into ``field_in`` (the
        engine rewrites its input when npass > 1), so every replay computes
        the same transfer.  Returns the graph; ``graph.replay()`` launches it
        on the current stream.  Replays are bit-identical to ``run``.
        """
        import torch

        st = torch.cuda.Stream(device=self.device)
        if restore_from is not None:
            field_in.copy_(restore_from)
        self.run(field_in, field_out)  # outside the capture: attributes and lazy loading
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st, capture_error_mode="relaxed"):
            if restore_from is not None:
                field_in.copy_(restore_from)
            self.run(field_in, field_out, stream=st.cuda_stream)
        torch.cuda.synchronize(self.device)
        return g

    def run(self, field_in, field_out, bulk=None, out_given=False, timed=False, stream=None):
        import torch

        io = _lib.TransferIO()
        io.field_in = field_in.data_ptr()
        io.field_out = field_out.data_ptr()
        io.out_given = int(out_given)
        io.bulk = bulk.data_ptr() if bulk is not None else None
        if stream is None:
            stream = torch.cuda.current_stream(self.device).cuda_stream
        args = (ctypes.byref(self.desc), ctypes.byref(io), ctypes.c_void_p(self.workspace.data_ptr()),
                ctypes.c_size_t(self.nbytes), ctypes.c_void_p(stream))
        if timed:
            t = _lib.KernelTimes()
            _lib.check(self.lib.dtmm_transfer_timed(*args, ctypes.byref(t)))
            return t
        _lib.check(self.lib.dtmm_transfer(*args))
        return None


def workspace_bytes(shape, nlayers, nlam, npol=2, nray=1, method="4x4", diffraction=1, npass=1, nstep=1,
                    precision="mixed"):
    """Device workspace of one transfer of these sizes (no allocation, no GPU needed)."""
    lib = _lib.load()
    d = _lib.TransferDesc()
    d.height, d.width = int(shape[0]), int(shape[1])
    d.nlam, d.npol, d.nray = int(nlam), int(npol), int(nray)
    d.method = 4 if method == "4x4" else 2
    full = diffraction == np.inf
    d.diffraction = _lib.DIFFRACTION_FULL if full else int(diffraction)
    d.npass = int(npass)
    if method == "4x4":
        d.reflection = 2 if not full and int(diffraction) == 0 else 1
    else:  # the 2x2 defaults of transfer_field
        d.reflection = 0 if npass == 1 else (2 if full or int(diffraction) > 1 else 1)
    d.precision = _lib.PRECISION_DOUBLE if precision == "double" else _lib.PRECISION_MIXED
    d.betamax, d.nin, d.nout, d.smooth = BETAMAX, N_COVER, N_COVER, SMOOTH
    th = np.ones(int(nlayers))
    ns = np.full(int(nlayers), int(nstep), np.int32)
    arr = np.zeros(max(int(nlam), int(nray)))
    d.nlayers = int(nlayers)
    d.thickness = th.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.nstep = ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.ks = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.beta = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.phi = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.epsv = d.epsa = 1  # sizes only: never dereferenced by the size query
    n = int(lib.dtmm_transfer_workspace_size(ctypes.byref(d)))
    if n == 0:
        raise ValueError(_lib.last_error())
    return n


def plan_transfer(field_shape, wavelengths, pixelsize, optical_data, beta=0.0, phi=0.0, nin=None, nout=None,
                  npass=None, nstep=1, diffraction=None, reflection=None, method=None, betamax=None, smooth=SMOOTH,
                  precision=None, device=None, tuning=None, norm=DTMM_NORM_FFT, eff_data=None):
    """Resolve options like transfer_field and bind a DevicePlan (explicit beta, phi).

    ``optical_data`` is the reference's list with one optical block, or a
    ``DeviceMaterial`` already on the device (one block: ``eff_data`` one
    symmetry).
    """
    torch = _require_cuda()
    nin = get_default_config_option("nin", nin)
    nout = get_default_config_option("nout", nout)
    method = get_default_config_option("method", method)
    npass = get_default_config_option("npass", npass)
    diffraction = get_default_config_option("diffraction", diffraction)
    reflection = get_default_config_option("reflection", reflection)
    betamax = get_default_config_option("betamax", betamax)
    eff_data = get_default_config_option("eff_data", eff_data)
    precision = _precision[0] if precision is None else precision
    if reflection is None:
        reflection = 0 if method == "2x2" else 1
        if method == "4x4" and diffraction == 0:
            reflection = 2
        if npass > 1:
            reflection = 1
            if diffraction > 1 and method == "2x2":
                reflection = 2
    _check_path(method, reflection, npass, diffraction, norm)
    shape = tuple(field_shape[-2:])
    dev = device or torch.device("cuda", torch.cuda.current_device())
    block_sym = None
    if isinstance(optical_data, DeviceMaterial):
        mat = optical_data
        if _is_effective_block(eff_data) or not isinstance(eff_data, (str, int, np.integer)):
            raise NotImplementedError("a DeviceMaterial takes one effective-medium symmetry")
        s = _symmetry(eff_data)
        if np.ndim(s) != 0:
            raise NotImplementedError("a DeviceMaterial takes one effective-medium symmetry")
        block_sym = [s] if s else None
    else:
        od, bs, be = effective_blocks(validate_optical_data(optical_data, shape), eff_data)
        mat = _Material(od, shape, dev, bs, be)
    beta = np.asarray(beta, np.float64)
    nray = 1 if beta.ndim == 0 else len(beta)
    nlam = field_shape[-4]
    npol = int(np.prod(field_shape[:-3])) // (nray * nlam)
    return DevicePlan(field_shape, mat, k0(wavelengths, pixelsize), beta, phi, nray, npol,
                      nlam, method, diffraction, reflection, npass, nstep, betamax, nin, nout, smooth, precision, dev,
                      tuning, norm, block_sym)


def _check_path(method, reflection, npass, diffraction, norm):
    if method == "4x4":
        if reflection not in (1, 2, 3, 4):
            raise ValueError("Invalid reflection. The 4x4 method is either reflection mode 1 or 2.")
    elif reflection not in (0, 1, 2):
        raise ValueError("Invalid reflection. The 2x2 method supports reflection mode 0,1 or 2.")
    if method != "4x4" and npass > 1 and reflection == 0:
        raise ValueError("Reflection mode `0` not compatible with npass > 1")
    # 4x4: reflection mode 2 or 4 without diffraction: the per-voxel transfer;
    # reflection modes 2-4 with diffraction: real-space half steps around the
    # corrected diffraction matrices; diffraction = inf: every eigenwave
    # exactly (any reflection mode).  2x2: reflection 0 / 1 in k-space (1 also
    # without diffraction), reflection 2 and no diffraction without
    # reflections in real space, diffraction = inf with reflection 0 or 2; any
    # npass
    local = method == "4x4" and reflection in (2, 4) and diffraction == 0
    full = diffraction == np.inf
    if full and method != "4x4" and reflection == 1:
        # the reference moves the field to k-space for reflection 1 and its modal
        # step transforms it once more (dtmm/transfer.py:1091-1098, :1172)
        raise NotImplementedError("2x2 with diffraction = inf is supported with reflection 0 or 2")
    if method == "4x4" and reflection == 3 and diffraction == 0:
        raise NotImplementedError("reflection mode 3 without diffraction (the reference has no such path)")
    if not (0 <= diffraction <= np.inf):
        raise ValueError("Invalid diffraction value")
    if diffraction == 0 and not local and method == "4x4":
        raise ValueError("Invalid diffraction value")
    if method != "4x4" and npass > 1 and reflection == 1 and diffraction == 0:
        # the reference's tracked reflection applies a diffraction matrix it does
        # not form without diffraction (dtmm/propagate_2x2.py:61) and fails
        raise NotImplementedError("2x2 reflection 1 without diffraction is not supported with npass > 1")
    if norm & DTMM_NORM_REF and method == "4x4" and npass > 1 and diffraction == np.inf:
        # the reference's reference field takes int(diffraction) windows (dtmm/propagate_2x2.py:330)
        raise NotImplementedError("norm with DTMM_NORM_REF is built for finite diffraction")
    if norm not in (0, DTMM_NORM_FFT, DTMM_NORM_REF, DTMM_NORM_FFT | DTMM_NORM_REF) and method == "4x4" and npass > 1:
        raise ValueError("norm must be a combination of DTMM_NORM_FFT and DTMM_NORM_REF")


def _require_cuda():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("dtmm_gb300.transfer_field needs a CUDA GPU (the engine has no CPU path)")
    return torch


def _beams(beta, phi, field_in):
    """beta, phi as float64 arrays and the number of rays: scalars, or one value
    per ray with the rays on the first field axis (dtmm/transfer.py:42-65)."""
    beta = np.asarray(beta, np.float64)
    phi = np.asarray(phi, np.float64)
    if beta.ndim != phi.ndim:
        raise ValueError("Beta nad phi should have same dimensions!")
    if beta.ndim == 1:
        if len(beta) != len(phi):
            raise ValueError("Beta nad phi should have same length!")
        nray = len(beta)
        if field_in.ndim < 5 or field_in.shape[0] != nray:
            if nray == 1:
                return beta[0], phi[0], 1
            raise ValueError("per-ray beta needs the rays on the first field axis")
        return beta, phi, nray
    if beta.ndim != 0:
        raise ValueError("Only length 1 or scalar values are supported for beta and phi")
    return beta, phi, 1


def _transfer_single(field_in, wavelengths, pixelsize, optical_data, beta, phi, nin, nout, npass, nstep,
                     diffraction, reflection, method, multiray, norm, betamax, smooth, ret_bulk, out, precision,
                     split_layers=False, eff_data=0):
    # every option and shape is checked on the host before the device is touched
    _check_path(method, reflection, npass, diffraction, norm)
    if smooth < 0:
        smooth = 0.0
    field_in = np.asarray(field_in)
    if field_in.ndim < 4:
        raise ValueError("Invald field dimensions")
    shape = field_in.shape[-2:]
    nlam = field_in.shape[-4]
    wavelengths = np.asarray(wavelengths)
    if wavelengths.ndim != 1 or len(wavelengths) != nlam:
        raise ValueError("Incompatible wavelengths shape.")
    od = validate_optical_data(optical_data, shape)
    if split_layers:
        od = split_blocks(od)
    od, block_sym, block_eff = effective_blocks(od, eff_data)
    aniso = _aniso_blocks(block_sym, block_eff)
    if aniso and method != "4x4" and reflection == 1 and diffraction != np.inf:
        # reflection 1: the interfaces between the effective media and their tracked reflections
        raise NotImplementedError("2x2 effective layers of uniaxial or biaxial symmetry are implemented with "
                                  "reflection 0 or 2, or with diffraction = inf")
    aniso = aniso and diffraction not in (0, np.inf)
    if ret_bulk and method == "4x4" and npass > 1 and (diffraction == 0 or diffraction == np.inf or
                                                        reflection in (2, 3, 4) or aniso):
        raise NotImplementedError("ret_bulk with npass > 1 is implemented for reflection mode 1 with diffraction >= 1")
    if ret_bulk and method != "4x4" and reflection in (0, 1) and diffraction > 1 and diffraction != np.inf:
        # the k-space sweep carries the sum of the windows, whose E -> H conversions differ
        raise NotImplementedError("2x2 ret_bulk in k-space (reflection 0 / 1) is implemented for diffraction <= 1")
    ks = k0(wavelengths, pixelsize)
    if (beta is None) != (phi is None):
        raise ValueError("Both beta and phi must be defined!")
    given = beta is not None
    if given:
        beta, phi, nray = _beams(beta, phi, field_in)
    torch = _require_cuda()
    cdt = torch.complex128 if precision == "double" else torch.complex64
    dev = torch.device("cuda", torch.cuda.current_device())
    field_dev = torch.from_numpy(np.ascontiguousarray(field_in, np.complex128)).to(dev)
    if not given:
        beta, phi = _field2betaphi(field_dev, ks, multiray)
        beta, phi, nray = _beams(beta, phi, field_in)
    nimg = int(np.prod(field_in.shape[:-3]))
    npol = nimg // (nray * nlam)
    mat = _Material(od, shape, dev, block_sym, block_eff)
    fdev = field_dev.to(cdt).contiguous()
    L = mat.nlayers
    bulk_dev = None
    if ret_bulk:
        bulk_dev = torch.zeros((L + 2,) + tuple(field_in.shape), dtype=cdt, device=dev)
        bulk_dev[0] = fdev
        fin_dev = bulk_dev[0]
        fout_dev = bulk_dev[-1]
        out_given = 0
        if out is not None and method == "4x4":  # 2x2 zeroes the caller's out (dtmm/transfer.py:1054)
            ob = np.asarray(out)
            bulk_dev[-1] = torch.from_numpy(np.ascontiguousarray(ob[-1], np.complex128)).to(dev).to(cdt)
            out_given = 1
    else:
        fin_dev = fdev
        if out is not None and method == "4x4":
            fout_dev = torch.from_numpy(np.ascontiguousarray(out, np.complex128)).to(dev).to(cdt).contiguous()
            out_given = 1
        else:
            fout_dev = torch.empty_like(fdev)
            out_given = 0
    plan = DevicePlan(field_in.shape, mat, ks, beta, phi, nray, npol, nlam, method, diffraction, reflection, npass,
                      nstep, betamax, nin, nout, smooth, precision, dev, norm=norm)
    plan.run(fin_dev, fout_dev, bulk=bulk_dev, out_given=out_given)
    if ret_bulk:
        res = _new_host(bulk_dev)
        if out is not None:
            out[...] = res
            res = out
        return res
    if out is not None:
        res = _to_host(fout_dev, out)
    else:
        res = _new_host(fout_dev)
    if npass > 1 and not ret_bulk:
        # the reference rewrites the caller's input with the reflected field
        # (with ret_bulk it rewrites the bulk's first slab instead)
        _to_host(fin_dev, field_in)
    return res


def _new_host(t):
    """A new complex128 numpy array holding device tensor ``t``: page-locked
    host memory from torch's caching host allocator, so the copy is one DMA
    (a pageable destination costs several times more) and freed results are
    reused by later calls."""
    import torch

    h = torch.empty(tuple(t.shape), dtype=torch.complex128, pin_memory=True)
    h.copy_(t.to(torch.complex128))
    return h.numpy()


def _to_host(t, dest):
    """Copy device field ``t`` into the complex128 numpy array ``dest``: straight
    into its memory when it is a writeable contiguous complex128 array (one
    device-to-host copy, a DMA when the array is pinned), else through a
    temporary."""
    import torch

    t = t.to(torch.complex128)
    if (isinstance(dest, np.ndarray) and dest.dtype == np.complex128 and dest.flags.c_contiguous
            and dest.flags.writeable and dest.shape == tuple(t.shape)):
        torch.from_numpy(dest).copy_(t)
    else:
        dest[...] = t.cpu().numpy()
    return dest


def transfer_field(field_data, optical_data, beta=None, phi=None, nin=None, nout=None, npass=None, nstep=1,
                   diffraction=None, reflection=None, method=None, multiray=False, norm=DTMM_NORM_FFT,
                   betamax=None, smooth=SMOOTH, split_rays=False, split_diffraction=False,
                   split_wavelengths=False, split_layers=False, eff_data=None, ret_bulk=False, out=None,
                   precision=None):
    """Transfer input field data through optical data (dtmm/transfer.py:322).

    Returns ``(field_out, wavelengths, pixelsize)``; with npass > 1 the input
    field array is overwritten with the reflected field, as in the reference.
    See the reference documentation for the meaning of every argument.
    ``split_diffraction`` only trades memory for time in the reference and
    has no effect here.
    """
    nin = get_default_config_option("nin", nin)
    nout = get_default_config_option("nout", nout)
    method = get_default_config_option("method", method)
    npass = get_default_config_option("npass", npass)
    eff_data = get_default_config_option("eff_data", eff_data)
    diffraction = get_default_config_option("diffraction", diffraction)
    reflection = get_default_config_option("reflection", reflection)
    betamax = get_default_config_option("betamax", betamax)
    precision = _precision[0] if precision is None else precision
    if precision not in ("double", "mixed"):
        raise ValueError("precision must be 'double' or 'mixed'")
    if method == "4x4" and npass > 1 and diffraction == False:  # noqa: E712 (reference semantics)
        warnings.warn("The 4x4 method with diffraction disabled is not yet supported for input fields with beta "
                      ">0. Use 2x2 method insted.")
    if npass == -1 or npass == np.inf:
        raise NotImplementedError("npass=-1 (exact modal transfer, dtmm/tmm3d.py) is outside the GPU engine")
    if reflection is None:
        reflection = 0 if method == "2x2" else 1
        if method == "4x4" and diffraction == 0:
            reflection = 2
        if npass > 1:
            reflection = 1
            if diffraction > 1 and method == "2x2":
                reflection = 2
    field_in, wavelengths, pixelsize = field_data
    if split_wavelengths and not isinstance(field_in, tuple) and not ret_bulk:
        # one transfer per wavelength, dispersive eps evaluated at it (dtmm/transfer.py:497-528);
        # a given out passes its wavelength slice on (4x4 keeps its reflected part), without
        # one every slice starts from zeros
        field_in = np.asarray(field_in)
        out_field = np.zeros_like(field_in, dtype=np.complex128) if out is None else out
        for i in range(len(wavelengths)):
            wl = np.asarray(wavelengths)[i]
            fi = field_in[..., i:i + 1, :, :, :]
            fcopy = np.array(fi)
            oi = None if out is None else out_field[..., i:i + 1, :, :, :]
            r = transfer_field((fcopy, np.asarray([wl]), pixelsize), evaluate_optical_data(optical_data, float(wl)),
                               beta, phi, nin, nout, npass, nstep, diffraction, reflection, method, multiray, norm,
                               betamax, smooth, split_rays, split_diffraction, False, split_layers, eff_data, False, oi,
                               precision)
            out_field[..., i, :, :, :] = r[0][..., 0, :, :, :]
            if npass > 1:
                field_in[..., i, :, :, :] = fcopy[..., 0, :, :, :]
        return out_field, wavelengths, pixelsize
    if isinstance(field_in, tuple):
        # one transfer per tuple entry (dtmm/transfer.py:510-528); a scalar wavelength
        # goes with a field that has no wavelength axis
        outs = []
        olist = out if out is not None else [None] * len(field_in)
        for f, wl, o in zip(field_in, wavelengths, olist):
            od = evaluate_optical_data(optical_data, wl)
            scalar = np.ndim(wl) == 0
            if scalar:
                f = np.asarray(f)[..., None, :, :, :]
                o = None if o is None else np.asarray(o)[..., None, :, :, :]
            r = transfer_field((f, [wl] if scalar else wl, pixelsize), od, beta, phi, nin, nout,
                               npass, nstep, diffraction, reflection, method, multiray, norm, betamax, smooth,
                               split_rays, split_diffraction, False, split_layers, eff_data, ret_bulk, o, precision)
            if scalar:
                r = (r[0][..., 0, :, :, :], wl, pixelsize)
            outs.append(r)
        return tuple(outs)
    if is_optical_data_dispersive(optical_data):
        raise ValueError("You are using dispersive data, so you must use `split_wavelengths=True`")
    if split_rays:
        # ray by ray into the caller's out (its ray i, or [:, i] of a bulk), as
        # dtmm/transfer.py:575-600; without out the result starts from zeros
        field_in = np.asarray(field_in)
        nrays = len(field_in)
        given = out is not None
        if given:
            res = out
        elif ret_bulk:
            blocks = optical_data if isinstance(optical_data, list) else [optical_data]
            res = np.zeros((len(np.atleast_1d(blocks[0][0])) + 2,) + field_in.shape, np.complex128)
        else:
            res = np.zeros_like(field_in, dtype=np.complex128)
        bl = [None] * nrays if beta is None else list(np.broadcast_to(beta, (nrays,)))
        pl = [None] * nrays if phi is None else list(np.broadcast_to(phi, (nrays,)))
        for i in range(nrays):
            fi = field_in[i]
            o = (res[:, i] if ret_bulk else res[i]) if given else None
            r = _transfer_single(fi, wavelengths, pixelsize, optical_data, bl[i], pl[i], nin, nout, npass, nstep,
                                 diffraction, reflection, method, False, norm, betamax, smooth, ret_bulk, o,
                                 precision, split_layers, eff_data)
            if not given:
                if ret_bulk:
                    res[:, i] = r
                else:
                    res[i] = r
        return res, wavelengths, pixelsize
    res = _transfer_single(field_in, wavelengths, pixelsize, optical_data, beta, phi, nin, nout, npass, nstep,
                           diffraction, reflection, method, multiray, norm, betamax, smooth, ret_bulk, out, precision,
                           split_layers, eff_data)
    return res, wavelengths, pixelsize


__all__ = ["transfer_field", "plan_transfer", "DevicePlan", "DeviceMaterial", "set_precision", "DTMM_NORM_FFT",
           "DTMM_NORM_REF", "evaluate_optical_data", "is_optical_data_dispersive"]
