"""POM image formation on transferred fields, on the GPU.

The consumer of ``transfer_field``'s output in dtmm's field viewer: the x / y
input polarisations are combined with the polarizer's jones vector, a window
and the analyzer (a 4x4 matrix in field space) are applied per pixel
(``calculate_pom_field``, dtmm/field_viewer.py:70-143), the normal Poynting
component gives a specter per pixel and wavelength (``field2specter``,
dtmm/field.py:784-847), and a colour matching function turns it into an
sRGB or gray image (``specter2color``, dtmm/color.py:52-224).  ``pom_image``
does the three steps in one pass per pixel.

Arrays may be numpy (copied to the device and back) or CUDA tensors (results
stay on the device).  A caller that enqueues the image behind other work on
the same stream passes ``pmat`` and ``cmf`` as device tensors: a host-to-device
copy from pageable memory would wait for that work.  The small jones / 4x4
matrices are built on the host (``jonesvec``, ``polarizer``,
``rotated_matrix``, ``ray_jonesmat4x4``).
Refocusing goes through a per-k diffraction matrix (``diffract``, the
library's ``dtmm_diffract``); k-space inputs are not on this path
(``NotImplementedError``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .illumination import _iso_fmat


# ---------------------------------------------------------------------------
# jones / 4x4 matrices (host, FP64)
# ---------------------------------------------------------------------------
def _rotation_matrix2(angle):
    angle = np.asarray(angle, np.float64)
    c, s = np.cos(angle), np.sin(angle)
    out = np.empty(c.shape + (2, 2), np.float64)
    out[..., 0, 0] = c
    out[..., 1, 1] = c
    out[..., 0, 1] = -s
    out[..., 1, 0] = s
    return out


def jonesvec(pol, phi=0.0):
    """Normalised jones vector, viewed in a frame rotated by ``phi`` (dtmm/jones.py:55)."""
    pol = np.asarray(pol, np.complex128)
    if pol.shape[-1] != 2:
        raise ValueError("Invalid input shape")
    norm = (pol[..., 0] * pol[..., 0].conj() + pol[..., 1] * pol[..., 1].conj()) ** 0.5
    pol = np.asarray(pol / norm[..., None], np.complex128)
    return np.einsum("...ij,...j->...i", _rotation_matrix2(-np.asarray(phi)), pol)


def polarizer(jones):
    """Jones polarizer matrix |j><j| (dtmm/jones.py:236)."""
    jones = np.asarray(jones)
    c, s = jones[..., 0], jones[..., 1]
    out = np.empty(jones.shape + (2,), np.complex128)
    out[..., 0, 0] = c * c.conj()
    out[..., 0, 1] = c * s.conj()
    out[..., 1, 0] = s * c.conj()
    out[..., 1, 1] = s * s.conj()
    return out


def rotated_matrix(jmat, phi):
    """Jones matrix viewed in a frame rotated by ``phi``: R^T jmat R (dtmm/jones.py:346)."""
    r = np.asarray(_rotation_matrix2(phi), np.complex128)
    return np.einsum("...ji,...jk,...kl->...il", r, np.asarray(jmat), r)


def ray_jonesmat4x4(jmat, beta=0.0, phi=0.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0)):
    """A 2x2 jones matrix as a 4x4 field-space matrix in the laboratory frame
    (dtmm/jones4.py:205): F . J4 . F^-1 with F the column-normalised field
    matrix of the medium at (beta, phi) and J4 = jmat on the forward and
    conj(jmat) on the backward modes.  Isotropic media only."""
    epsv = np.asarray(epsv, np.complex128)
    if not (epsv[..., 0] == epsv[..., 1]).all() or not (epsv[..., 1] == epsv[..., 2]).all():
        raise NotImplementedError("ray_jonesmat4x4: isotropic media only")
    f = _iso_fmat(beta, phi, epsv[..., 0])
    jm = rotated_matrix(jmat, phi)
    j4 = np.zeros(jm.shape[:-2] + (4, 4), np.complex128)
    j4[..., 0::2, 0::2] = jm
    j4[..., 1::2, 1::2] = np.conj(jm)
    return f @ j4 @ np.linalg.inv(f)


def field_diffraction_matrix(shape, ks, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0), mode="b",
                             betamax=0.8, device=None):
    """Per-k 4x4 propagation matrix F . diag(exp(i alpha ks d)) . F^-1 of a
    homogeneous isotropic medium over d pixels (dtmm/diffract.py:125), zero
    for beta >= betamax; mode "t" / "r" keeps the forward / backward modes
    only.  Shape (n_wavelengths, H, W, 4, 4), complex128: built on the host
    in FP64, or with ``device`` on the GPU by the library's
    ``dtmm_field_diffraction_matrix`` (a device tensor, nothing on the host
    grows with the grid)."""
    from .illumination import _fftfreq_grid

    epsv = np.asarray(epsv, np.complex128)
    if not (epsv[0] == epsv[1] == epsv[2]):
        raise NotImplementedError("field_diffraction_matrix: isotropic media only")
    ks = np.abs(np.asarray(ks, np.float64)).reshape(-1)
    if device is not None:
        torch = _torch()
        h, w = (int(x) for x in shape)
        out = torch.empty((len(ks), h, w, 4, 4), dtype=torch.complex128, device=device)
        m = {"b": 0, 0: 0, "t": 1, 1: 1, "r": -1, -1: -1}[mode]
        ksa = np.ascontiguousarray(ks)
        lib = _lib.load()
        _lib.check(lib.dtmm_field_diffraction_matrix(h, w, len(ks), ksa.ctypes.data_as(ctypes.c_void_p), float(d),
                                                     float(epsv[0].real), float(epsv[0].imag), m, float(betamax),
                                                     ctypes.c_void_p(out.data_ptr()), _stream(out.device)))
        return out
    beta, phi = _fftfreq_grid(shape, ks)
    eps = epsv[0]
    f = _iso_fmat(beta, phi, eps)
    a = np.sqrt(eps - beta ** 2 + 0j)
    alpha = np.stack([a, -a, a, -a], axis=-1)
    cut = beta >= betamax
    f[cut] = 0.0
    alpha[cut] = 0.0
    fi = np.zeros_like(f)
    ok = ~cut
    fi[ok] = np.linalg.inv(f[ok])
    ph = np.exp(1j * (ks * d)[:, None, None, None] * alpha)
    if mode in ("t", +1):
        ph[..., 1::2] = 0.0
    elif mode in ("r", -1):
        ph[..., ::2] = 0.0
    return (f * ph[..., None, :]) @ fi


# ---------------------------------------------------------------------------
# device plumbing
# ---------------------------------------------------------------------------
def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("dtmm_gb300.pom needs a CUDA GPU (there is no CPU path)")
    return torch


def _dev_field(field):
    torch = _torch()
    if isinstance(field, torch.Tensor):
        if not field.is_cuda:
            field = field.cuda()
        return field.contiguous(), False
    a = np.asarray(field)
    dtype = np.complex64 if a.dtype == np.complex64 else np.complex128
    return torch.from_numpy(np.ascontiguousarray(a, dtype)).cuda(), True


def _dev_real(x, device):
    torch = _torch()
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, np.float64)).to(device)


def _precision(t):
    torch = _torch()
    if t.dtype == torch.complex64:
        return _lib.PRECISION_MIXED
    if t.dtype == torch.complex128:
        return _lib.PRECISION_DOUBLE
    raise ValueError("fields must be complex64 or complex128")


def _stream(device):
    return ctypes.c_void_p(_torch().cuda.current_stream(device).cuda_stream)


def _desc(f, jvec, pmat, window):
    """Descriptor for a field tensor [..., (2,) lam, 4, H, W]; returns (desc, keep-alive list, leading shape)."""
    torch = _torch()
    h, w = f.shape[-2:]
    nlam = f.shape[-4]
    d = _lib.PomDesc()
    d.height, d.width, d.nlam = int(h), int(w), int(nlam)
    keep = []
    if jvec is not None:
        if f.ndim < 5 or f.shape[-5] != 2:
            raise ValueError("Invalid field shape.")
        lead = tuple(f.shape[:-5])
        d.npol = 2
        j = np.asarray(jvec, np.complex128).reshape(2)
        d.jvec[:] = (j[0].real, j[0].imag, j[1].real, j[1].imag)
    else:
        lead = tuple(f.shape[:-4])
        d.npol = 1
    d.nset = int(np.prod(lead)) if lead else 1
    if pmat is not None:
        if isinstance(pmat, torch.Tensor):  # already on the device: no upload behind queued work
            pt = pmat.to(device=f.device, dtype=torch.complex128).contiguous()
        else:
            pt = torch.from_numpy(np.ascontiguousarray(np.asarray(pmat, np.complex128))).to(f.device)
        if tuple(pt.shape) != (4, 4):
            raise NotImplementedError("one 4x4 analyzer matrix for every pixel and wavelength")
        keep.append(pt)
        d.pmat = pt.data_ptr()
    if window is not None:
        wt = _dev_real(window, f.device)
        if tuple(wt.shape) != (h, w):
            raise ValueError("window must have the grid's shape")
        keep.append(wt)
        d.window = wt.data_ptr()
    d.precision = _precision(f)
    return d, keep, lead


# ---------------------------------------------------------------------------
# the reference's functions
# ---------------------------------------------------------------------------
def _pom_field_dev(f, jvec, pmat, window):
    torch = _torch()
    d, keep, lead = _desc(f, jvec, pmat, window)
    res = torch.empty(lead + tuple(f.shape[-4:]), dtype=f.dtype, device=f.device)
    lib = _lib.load()
    _lib.check(lib.dtmm_pom_field(ctypes.byref(d), ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(res.data_ptr()),
                                  _stream(f.device)))
    res._dtmm_keep = keep
    return res


def _diffract_dev(f, dmat):
    torch = _torch()
    h, w = f.shape[-2:]
    nlam = f.shape[-4]
    nimg = int(np.prod(f.shape[:-3]))
    dm = dmat if isinstance(dmat, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(dmat, np.complex128))
    dm = dm.to(device=f.device, dtype=torch.complex128).contiguous()
    if tuple(dm.shape) != (nlam, h, w, 4, 4):
        raise ValueError("dmat must have shape (n_wavelengths, H, W, 4, 4)")
    prec = _precision(f)
    lib = _lib.load()
    nbytes = int(lib.dtmm_diffract_workspace_size(int(h), int(w), nimg, int(nlam), prec))
    if nbytes == 0:
        raise ValueError(_lib.last_error())
    ws = torch.empty(nbytes, dtype=torch.uint8, device=f.device)
    out = torch.empty_like(f)
    _lib.check(lib.dtmm_diffract(int(h), int(w), nimg, int(nlam), prec, ctypes.c_void_p(dm.data_ptr()),
                                 ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(nbytes), _stream(f.device)))
    out._dtmm_keep = (dm, ws)
    return out


def diffract(field, dmat, window=None, out=None):
    """fft2, per-k 4x4 matrix ``dmat`` (n_wavelengths, H, W, 4, 4), ifft2,
    optional real-space window (dtmm/diffract.py:254), on the GPU."""
    f, host = _dev_field(field)
    res = _diffract_dev(f, dmat)
    if window is not None:
        res = _pom_field_dev(res, None, None, window)
    if host:
        r = res.cpu().numpy().astype(np.complex128)
        if out is not None:
            out[...] = r
            return out
        return r
    return res


def calculate_pom_field(field, jvec=None, pmat=None, dmat=None, window=None, input_fft=False, output_fft=False,
                        out=None):
    """Polarizer, refocus, window and analyzer applied to a transferred field
    (dtmm/field_viewer.py:70, real-space path): field [..., (2,) lam, 4, H, W]
    -> [..., lam, 4, H, W]; ``dmat`` (n_wavelengths, H, W, 4, 4) refocuses
    through ``diffract``."""
    if input_fft or output_fft:
        raise NotImplementedError("k-space fields are outside the GPU POM path")
    f, host = _dev_field(field)
    if dmat is None:
        res = _pom_field_dev(f, jvec, pmat, window)
    else:
        g = _pom_field_dev(f, jvec, None, None) if jvec is not None else f
        res = _pom_field_dev(_diffract_dev(g, dmat), None, pmat, window)
    if host:
        r = res.cpu().numpy().astype(np.complex128)
        if out is not None:
            out[...] = r
            return out
        return r
    return res


def _specter(field, summed):
    torch = _torch()
    f, host = _dev_field(field)
    h, w = f.shape[-2:]
    nlam = f.shape[-4]
    if summed:
        if f.ndim < 5:
            raise ValueError("field2spectersum needs a leading axis to sum")
        outer, nsum = tuple(f.shape[:-5]), int(f.shape[-5])
    else:
        outer, nsum = tuple(f.shape[:-4]), 1
    nouter = int(np.prod(outer)) if outer else 1
    spec = torch.empty(outer + (h, w, nlam), dtype=torch.float64, device=f.device)
    lib = _lib.load()
    ff = f.reshape((nouter * nsum,) + tuple(f.shape[-4:]))
    sp = spec.reshape((nouter,) + (h, w, nlam))
    if summed:
        per = nsum * nlam * 4 * h * w * f.element_size()
        for o in range(nouter):
            _lib.check(lib.dtmm_field2specter(int(h), int(w), int(nlam), nsum, 1, _precision(f),
                                              ctypes.c_void_p(ff.data_ptr() + o * per),
                                              ctypes.c_void_p(sp[o].data_ptr()), _stream(f.device)))
    else:
        _lib.check(lib.dtmm_field2specter(int(h), int(w), int(nlam), nouter, 0, _precision(f),
                                          ctypes.c_void_p(ff.data_ptr()), ctypes.c_void_p(sp.data_ptr()),
                                          _stream(f.device)))
    return spec.cpu().numpy() if host else spec


def field2specter(field):
    """Normal Poynting component: [..., lam, 4, H, W] -> [..., H, W, lam] (dtmm/field.py:824)."""
    return _specter(field, False)


def field2spectersum(field):
    """field2specter summed over the axis before the wavelengths (dtmm/field.py:845)."""
    return _specter(field, True)


def _norm_args(norm):
    if norm is True:
        return 2, 0.0
    if norm is False or norm == 0:
        return 0, 0.0
    return 1, float(norm)


def _gamma_arg(gamma):
    if gamma is True:
        return -1.0
    if gamma is False:
        return 0.0
    g = float(gamma)
    if g <= 0:
        raise ValueError("gamma must be positive, True (sRGB) or False")
    return g


def specter2color(spec, cmf, norm=False, gamma=True, gray=False, out=None):
    """Specter [..., lam] -> RGB [..., 3] (dtmm/color.py:133): XYZ through ``cmf``
    [lam, 3], optional normalisation (a value, or True for the image maximum),
    sRGB (D65) or gray, then the sRGB curve (gamma True), a power curve
    (gamma float) or none (gamma False)."""
    torch = _torch()
    cmf = np.asarray(cmf, np.float64)
    if cmf.shape[-1] != 3:
        raise ValueError("Grayscale cmf! Cannot convert to color.")
    host = not isinstance(spec, torch.Tensor)
    s = spec if not host else torch.from_numpy(np.ascontiguousarray(spec, np.float64)).cuda()
    s = s.to(torch.float64).contiguous()
    nlam = s.shape[-1]
    if cmf.shape != (nlam, 3):
        raise ValueError("cmf must have one row per wavelength")
    c = torch.from_numpy(np.ascontiguousarray(cmf)).to(s.device)
    rgb = torch.empty(tuple(s.shape[:-1]) + (3,), dtype=torch.float64, device=s.device)
    mode, val = _norm_args(norm)
    npix = int(np.prod(s.shape[:-1])) if s.ndim > 1 else 1
    lib = _lib.load()
    _lib.check(lib.dtmm_specter2color(npix, int(nlam), ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                                      mode, val, _gamma_arg(gamma), int(bool(gray)),
                                      ctypes.c_void_p(rgb.data_ptr()), _stream(s.device)))
    if host:
        r = rgb.cpu().numpy()
        if out is not None:
            out[...] = r
            return out
        return r
    return rgb


def pom_image(field, cmf, jvec=None, pmat=None, window=None, norm=False, gamma=True, gray=False, stream=None):
    """The POM image of a transferred field in one pass: polarizer (``jvec``
    over the x / y axis), window, analyzer ``pmat``, Poynting summed over
    every leading set, XYZ, colour -> float32 [H, W, 3]."""
    torch = _torch()
    f, host = _dev_field(field)
    d, keep, lead = _desc(f, jvec, pmat, window)
    if isinstance(cmf, torch.Tensor):  # already on the device: no upload behind queued work
        c = cmf.to(device=f.device, dtype=torch.float64).contiguous()
    else:
        c = torch.from_numpy(np.ascontiguousarray(np.asarray(cmf, np.float64))).to(f.device)
    if tuple(c.shape) != (f.shape[-4], 3):
        raise ValueError("cmf must have one row per wavelength")
    rgb = torch.empty(tuple(f.shape[-2:]) + (3,), dtype=torch.float32, device=f.device)
    mode, val = _norm_args(norm)
    lib = _lib.load()
    st = ctypes.c_void_p(stream) if stream is not None else _stream(f.device)
    _lib.check(lib.dtmm_pom_image(ctypes.byref(d), ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                                  mode, val, _gamma_arg(gamma), int(bool(gray)), ctypes.c_void_p(rgb.data_ptr()),
                                  st))
    rgb._dtmm_keep = (keep, c)
    return rgb.cpu().numpy() if host else rgb


__all__ = ["jonesvec", "polarizer", "rotated_matrix", "ray_jonesmat4x4", "field_diffraction_matrix", "diffract",
           "calculate_pom_field", "field2specter", "field2spectersum", "specter2color", "pom_image"]
