"""Input field data: plane-wave illumination.

``illumination_data`` mirrors ``dtmm.field.illumination_data``
(dtmm/field.py:586-713): the eigenmode case (``window=None``), which is how
the reference builds the inputs of ``transfer_field``, and the windowed case
(finite beams: a plane wave times a real window, ``window.aperture`` /
``window.blackman``).  ``illumination_rays`` (dtmm/field.py:342-404) gives
the ray directions and weights of an illumination of numerical aperture NA.

The reference builds each plane wave on the full grid, replaces it by the
FFT-grid mode of largest power (``wave2eigenwave``, dtmm/wave.py:432), then
filters the field through the diffraction operator of the cover medium in
k-space (``diffracted_field``, dtmm/diffract.py:301) and rescales its total
intensity.  A field made of one FFT mode stays one mode under those steps, so
every image of the result is ``coef[c] * exp(2 pi i (my * y / H + mx * x / W))``:
``illumination_modes`` computes the per-image 4-vectors ``coef`` and the mode
indices (my, mx) with O(H + W) work per wave, and the grid is filled either on
the host (``illumination_data``) or on the device by the library's
``dtmm_planewave_field`` kernel (``illumination_device``).
"""
from __future__ import annotations

import numpy as np

N_COVER = 1.5
BETAMAX = 0.8


# ---------------------------------------------------------------------------
# ray sets of a finite numerical aperture
# ---------------------------------------------------------------------------
def illumination_aperture(diameter=5.0, smooth=0.1):
    """Field-aperture diaphragm of ``diameter`` pixels, annular for
    ``(inner, outer)``, with a raised-cosine edge (dtmm/field.py:356-369)."""
    from .window import aperture

    try:
        inner, outer = diameter
        inner, outer = int(round(inner)), int(round(outer))
        if inner >= outer:
            raise ValueError("Invalid dimater, rounded inner diameter should be lower that outer diameter.")
    except TypeError:
        inner, outer = 0, int(round(diameter))
    alpha = min(max(smooth, 0), 1)
    return aperture((outer, outer), (inner / outer, 1.0), alpha)


def aperture2rays(diaphragm, betastep=0.1, norm=True):
    """beta, phi, intensity of the rays through the open pixels of a
    diaphragm image; beta grows by ``betastep`` per pixel from the centre
    (dtmm/field.py:342-354)."""
    diaphragm = np.asarray(diaphragm)
    ay, ax = (np.arange(-n / 2.0 + 0.5, n / 2.0 + 0.5) for n in diaphragm.shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    phi = np.arctan2(yy, xx)
    beta = np.sqrt(xx ** 2 + yy ** 2) * betastep
    mask = diaphragm > 0.0
    intensity = diaphragm[mask]
    if norm:
        intensity = intensity / intensity.sum() * len(intensity)
    return (np.asarray(beta[mask], np.float64), np.asarray(phi[mask], np.float64),
            np.asarray(intensity, np.float64))


def illumination_rays(NA, diameter=5.0, smooth=0.1):
    """Ray directions (beta, phi) and intensities of an illumination of
    numerical aperture ``NA`` sampled by a diaphragm of ``diameter`` pixels,
    for ``illumination_data(beta=..., phi=..., intensity=...)``
    (dtmm/field.py:371-404)."""
    try:
        low, high = diameter
    except TypeError:
        low, high = 0, diameter
    betastep = 2.0 * NA / (high - 1)
    a = illumination_aperture((low, high), smooth)
    return aperture2rays(a, betastep=betastep, norm=True)


def _fftfreq_grid(shape, ks):
    ay, ax = (np.fft.fftfreq(n) for n in shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    k = np.abs(np.asarray(ks, np.float64))[..., None, None]
    return (2 * np.pi / k) * np.sqrt(xx ** 2 + yy ** 2), np.arctan2(yy, xx)


def _iso_fmat(beta, phi, eps):
    """Normalised isotropic field matrix, rotated by phi (dtmm/tmm.py:124, :372; normalize_f :701)."""
    beta = np.asarray(beta, np.float64)
    phi = np.asarray(phi, np.float64)
    shape = np.broadcast_shapes(beta.shape, phi.shape)
    beta = np.broadcast_to(beta, shape)
    phi = np.broadcast_to(phi, shape)
    a = np.sqrt(np.asarray(eps, np.complex128) - beta ** 2 + 0j)
    ok = a != 0
    gp = np.where(ok, eps / np.where(ok, a, 1.0), 0.0)
    F = np.zeros(shape + (4, 4), np.complex128)
    F[..., 0, 0] = 0.5
    F[..., 0, 1] = 0.5
    F[..., 1, 0] = 0.5 * gp
    F[..., 1, 1] = -0.5 * gp
    F[..., 2, 2] = 0.5
    F[..., 2, 3] = 0.5
    F[..., 3, 2] = -0.5 * a
    F[..., 3, 3] = 0.5 * a
    F[~ok] = 0.0
    c, s = np.cos(phi)[..., None], np.sin(phi)[..., None]
    R = F.copy()
    R[..., 0, :] = F[..., 0, :] * c - F[..., 2, :] * s
    R[..., 1, :] = F[..., 1, :] * c + F[..., 3, :] * s
    R[..., 2, :] = F[..., 0, :] * s + F[..., 2, :] * c
    R[..., 3, :] = -F[..., 1, :] * s + F[..., 3, :] * c
    # column normalisation to unit |Poynting| (normalize_f)
    p = np.abs((R[..., 0, :].real * R[..., 1, :].real + R[..., 0, :].imag * R[..., 1, :].imag)
               - (R[..., 2, :].real * R[..., 3, :].real + R[..., 2, :].imag * R[..., 3, :].imag)) ** 0.5
    scale = np.where(p == 0.0, 0.0, 1.0 / np.where(p == 0.0, 1.0, p))
    return R * scale[..., None, :]


def _inv4(m):
    out = np.zeros_like(m)
    flat = m.reshape(-1, 4, 4)
    o = out.reshape(-1, 4, 4)
    det = np.linalg.det(flat)
    good = det != 0
    o[good] = np.linalg.inv(flat[good])
    return out


def _intensity(field):
    f = field
    return (f[..., 0, :, :].real * f[..., 1, :, :].real + f[..., 0, :, :].imag * f[..., 1, :, :].imag) - (
        f[..., 2, :, :].real * f[..., 3, :, :].real + f[..., 2, :, :].imag * f[..., 3, :, :].imag)


def _peak_bins(k, n):
    """FFT bin of largest power of exp(i k a), a = -n//2+1 ... n//2 (one axis of wave2eigenwave)."""
    a = np.arange(-n // 2 + 1.0, n // 2 + 1.0)
    w = np.exp(1j * np.asarray(k, np.float64)[..., None] * a)
    return np.argmax(np.abs(np.fft.fft(w, axis=-1)) ** 2, axis=-1)


def _intensity_vec(c):
    return (c[..., 0].real * c[..., 1].real + c[..., 0].imag * c[..., 1].imag) - (
        c[..., 2].real * c[..., 3].real + c[..., 2].imag * c[..., 3].imag)


def _mode_vectors(beta, phi, n, jones, backdir, nlam):
    """4-vectors of the forward (or backward) eigenmode amplitude of each ray
    and input polarisation in a cover of index n: the jones vector rotated
    into the ray's plane of incidence, through the cover's field matrix
    (waves2field2 / field4, dtmm/field.py:566-582).  Shape
    ``([rays,] [2,] nlam, 4)``; the polarisation axis is present when
    ``jones is None``."""
    fm = _iso_fmat(beta, phi, n * n)  # (rays, 4, 4) or (4, 4)

    def one(pol):
        pol = np.asarray(pol, np.complex128)
        pol = pol / np.sqrt(pol[0] * np.conj(pol[0]) + pol[1] * np.conj(pol[1]))
        c, s = np.cos(-phi), np.sin(-phi)
        jv0 = c * pol[0] - s * pol[1]
        jv1 = s * pol[0] + c * pol[1]
        a = np.zeros(np.shape(jv0) + (4,), np.complex128)
        if backdir:
            a[..., 1] = jv0
            a[..., 3] = jv1
        else:
            a[..., 0] = jv0
            a[..., 2] = jv1
        v = np.einsum("...ij,...j->...i", fm, a)  # (rays, 4) or (4,)
        return np.broadcast_to(v[..., None, :], v.shape[:-1] + (nlam, 4))

    if jones is None:
        return np.stack([one((1, 0)), one((0, 1))], axis=-3)
    return np.array(one(jones))


_MODES_CACHE = {}
_MODES_CACHE_MAX = 512


def _key(x):
    a = np.asarray(x)
    return (a.dtype.str, a.shape, a.tobytes())


def illumination_modes(shape, wavelengths, pixelsize=1.0, beta=0.0, phi=0.0, intensity=1.0, n=None,
                       focus=0.0, backdir=False, jones=None, diffraction=True, betamax=BETAMAX):
    """Per-image 4-vectors and FFT modes of the plane-wave illumination
    (``_illumination_modes``), remembered for repeated arguments (a serving
    loop builds the same illumination for many requests); returns copies."""
    key = (tuple(int(v) for v in shape), _key(wavelengths), float(pixelsize), _key(beta), _key(phi), _key(intensity),
           None if n is None else float(n), float(focus), bool(backdir), None if jones is None else _key(jones),
           bool(diffraction), float(betamax))
    hit = _MODES_CACHE.get(key)
    if hit is None:
        hit = _illumination_modes(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, backdir, jones,
                                  diffraction, betamax)
        if len(_MODES_CACHE) >= _MODES_CACHE_MAX:
            _MODES_CACHE.pop(next(iter(_MODES_CACHE)))
        _MODES_CACHE[key] = hit
    return tuple(a.copy() for a in hit)


def _illumination_modes(shape, wavelengths, pixelsize=1.0, beta=0.0, phi=0.0, intensity=1.0, n=None,
                        focus=0.0, backdir=False, jones=None, diffraction=True, betamax=BETAMAX):
    """Per-image 4-vectors and FFT modes of the plane-wave illumination.

    Returns ``(coef, my, mx)``: ``coef`` complex128 of shape
    ``([nrays,] [2,] nwavelengths, 4)`` and integer mode indices ``my``,
    ``mx`` of shape ``([nrays,] [2,] nwavelengths)``, such that image ``i``
    of ``illumination_data(...)[0]`` is
    ``coef[i, c] * exp(2 pi i (my[i] * y / H + mx[i] * x / W))``.
    """
    n = N_COVER if n is None else n
    h, w = shape
    wavelengths = np.asarray(wavelengths)
    ks = 2 * np.pi / wavelengths * pixelsize
    if ks.ndim != 1:
        raise ValueError("Wavelengths should be 1D array")
    if jones is None:
        intensity = intensity / 2.0
    _beta = np.asarray(beta, np.float64)
    _phi = np.asarray(phi, np.float64)
    if _beta.ndim > 1 or _phi.ndim > 1 or _beta.ndim != _phi.ndim:
        raise NotImplementedError("illumination_modes: beta and phi must both be scalars or 1D ray arrays")
    multi = _beta.ndim == 1
    nrays = len(_beta) if multi else 1
    b = _beta[:, None] if multi else _beta
    p = _phi[:, None] if multi else _phi
    # mode indices per (ray, wavelength): the plane wave of wave.py:376 with
    # x along columns and y along rows, reduced to its strongest FFT bin
    kx = ks * b * np.cos(p)
    ky = ks * b * np.sin(p)
    mx = _peak_bins(kx, w)
    my = _peak_bins(ky, h)
    coef = _mode_vectors(_beta, _phi, n, jones, backdir, len(ks))
    myb = my[..., None, :] if jones is None else my
    mxb = mx[..., None, :] if jones is None else mx
    myb, mxb = np.broadcast_to(myb, coef.shape[:-1]), np.broadcast_to(mxb, coef.shape[:-1])
    inten = np.asarray(intensity, np.float64)
    if inten.ndim == 1 and multi:
        inten = inten.reshape((nrays,) + (1,) * (coef.ndim - 2))
    elif inten.ndim != 0:
        raise NotImplementedError("illumination_modes: intensity must be a scalar or one value per ray")
    norm = np.broadcast_to((inten / nrays) ** 0.5, coef.shape[:-1]).astype(np.float64)
    if diffraction:
        # diffracted_field with d = -focus (diffract.py:301, :125) at the mode's own k
        kabs = np.abs(ks)
        lam_axis = np.arange(len(ks))
        lam = np.broadcast_to(lam_axis, coef.shape[:-1])
        fx = np.fft.fftfreq(w)[mxb]
        fy = np.fft.fftfreq(h)[myb]
        beta_k = (2 * np.pi / kabs[lam]) * np.sqrt(fx ** 2 + fy ** 2)
        phi_k = np.arctan2(fy, fx)
        F = _iso_fmat(beta_k, phi_k, n * n)
        a = np.sqrt(n * n - beta_k ** 2 + 0j)
        alpha = np.stack([a, -a, a, -a], axis=-1)
        cut = beta_k >= betamax
        F[cut] = 0.0
        Fi = _inv4(F)
        alpha[cut] = 0.0
        ph = np.exp(1j * (ks[lam] * (-focus))[..., None] * alpha)
        if backdir:
            ph[..., ::2] = 0.0
        else:
            ph[..., 1::2] = 0.0
        D = np.matmul(F * ph[..., None, :], Fi)
        c2 = np.einsum("...ij,...j->...i", D, coef)
        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = (_intensity_vec(coef) / _intensity_vec(c2)) ** 0.5
        coef = c2
        norm = norm * ratio
    coef = coef * norm[..., None]
    return coef, np.ascontiguousarray(myb, np.int32), np.ascontiguousarray(mxb, np.int32)


def planewave_grid(shape, my, mx):
    """exp(2 pi i (my * y / H + mx * x / W)) on the (H, W) grid (exact phase reduction)."""
    h, w = shape
    y = np.arange(h)
    x = np.arange(w)
    my = np.asarray(my)[..., None, None]
    mx = np.asarray(mx)[..., None, None]
    num = ((my * y[:, None]) % h) * w + ((mx * x[None, :]) % w) * h
    return np.exp(2j * np.pi * (num / float(h * w)))


def illumination_data(shape, wavelengths, pixelsize=1.0, beta=0.0, phi=0.0, intensity=1.0, n=None,
                      focus=0.0, window=None, backdir=False, jones=None, diffraction=True,
                      eigenmodes=None, betamax=BETAMAX):
    """Forward (or backward) plane-wave illumination ``(field, wavelengths, pixelsize)``.

    Field shape: ``([nrays,] [2,] nwavelengths, 4, H, W)``; the polarisation
    axis is present when ``jones is None``.  Built on the host.  With a
    ``window`` the waves are plane waves times the window (not reduced to
    FFT eigenmodes), as in the reference; ``eigenmodes`` has no effect there
    either.
    """
    if window is not None:
        return _window_field(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, window, backdir, jones,
                             diffraction, betamax), np.asarray(wavelengths), pixelsize
    coef, my, mx = illumination_modes(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, backdir, jones,
                                      diffraction, betamax)
    field = coef[..., :, None, None] * planewave_grid(shape, my, mx)[..., None, :, :]
    return field, np.asarray(wavelengths), pixelsize


def _window_setup(shape, wavelengths, pixelsize, beta, phi, intensity, n, jones, backdir):
    """Shared by the host and device windowed paths: wavenumbers, the mode
    4-vectors ``coef`` ([rays,] [2,] nlam, 4), the per-image wave-vector
    components (kx, ky) and the per-image amplitude norm sqrt(I / nrays)."""
    n = N_COVER if n is None else n
    wavelengths = np.asarray(wavelengths)
    ks = 2 * np.pi / wavelengths * pixelsize
    if ks.ndim != 1:
        raise ValueError("Wavelengths should be 1D array")
    if jones is None:
        intensity = intensity / 2.0
    _beta = np.asarray(beta, np.float64)
    _phi = np.asarray(phi, np.float64)
    if _beta.ndim > 1 or _phi.ndim > 1 or _beta.ndim != _phi.ndim:
        raise NotImplementedError("illumination_data: beta and phi must both be scalars or 1D ray arrays")
    multi = _beta.ndim == 1
    nrays = len(_beta) if multi else 1
    coef = _mode_vectors(_beta, _phi, n, jones, backdir, len(ks))
    b = _beta[:, None] if multi else _beta
    p = _phi[:, None] if multi else _phi
    kx = ks * b * np.cos(p)  # (rays, nlam) or (nlam,): the plane wave of dtmm/wave.py:376
    ky = ks * b * np.sin(p)
    if jones is None:
        kx, ky = kx[..., None, :], ky[..., None, :]
    kx = np.ascontiguousarray(np.broadcast_to(kx, coef.shape[:-1]), np.float64)
    ky = np.ascontiguousarray(np.broadcast_to(ky, coef.shape[:-1]), np.float64)
    inten = np.asarray(intensity, np.float64)
    if inten.ndim == 1 and multi:
        inten = inten.reshape((nrays,) + (1,) * (coef.ndim - 2))
    elif inten.ndim != 0:
        raise NotImplementedError("illumination_data: intensity must be a scalar or one value per ray")
    norm = np.ascontiguousarray(np.broadcast_to((inten / nrays) ** 0.5, coef.shape[:-1]), np.float64)
    return n, ks, coef, kx, ky, norm


def _window_field(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, window, backdir, jones,
                  diffraction, betamax):
    """Windowed illumination on the host (dtmm/field.py:663-713): the mode
    vectors times the windowed plane waves, then the cover's diffraction over
    -focus and the rescale to the intensity before it."""
    from scipy import fft as sfft

    from .pom import field_diffraction_matrix

    n, ks, coef, kx, ky, norm = _window_setup(shape, wavelengths, pixelsize, beta, phi, intensity, n, jones, backdir)
    h, w = shape
    ay, ax = (np.arange(-l // 2 + 1.0, l // 2 + 1.0) for l in shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    wave = np.exp(1j * (kx[..., None, None] * xx + ky[..., None, None] * yy))
    wave = wave / wave[..., :1, :1]
    wave = wave * np.asarray(window, np.float64)
    field = coef[..., :, None, None] * wave[..., None, :, :]
    if diffraction:
        i1 = _intensity(field).sum((-2, -1))
        dmat = field_diffraction_matrix((h, w), ks, d=-focus, epsv=(n * n,) * 3, mode="r" if backdir else "t",
                                        betamax=betamax)
        f = sfft.fft2(field)
        f = np.einsum("...hwij,...jhw->...ihw", dmat, f)
        field = sfft.ifft2(f)
        i2 = _intensity(field).sum((-2, -1))
        norm = norm * (i1 / i2) ** 0.5
    return field * norm[..., None, None, None]


def _window_device(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, window, backdir, jones,
                   diffraction, betamax, precision, dev, out, stream):
    """Windowed illumination on the device: ``dtmm_wave_field`` (windowed
    plane waves), then ``dtmm_field_diffraction_matrix`` + ``dtmm_diffract``
    for the cover's diffraction over -focus, ``dtmm_field_intensity`` before
    and after it and ``dtmm_scale_fields`` for the rescale; nothing
    grid-sized is computed on the host."""
    import ctypes

    import torch

    from . import _lib

    n, ks, coef, kx, ky, norm = _window_setup(shape, wavelengths, pixelsize, beta, phi, intensity, n, jones, backdir)
    h, w = (int(x) for x in shape)
    nimg = int(np.prod(coef.shape[:-1]))
    nlam = len(ks)
    dtype = torch.complex128 if precision == "double" else torch.complex64
    prec = _lib.PRECISION_DOUBLE if precision == "double" else _lib.PRECISION_MIXED
    fshape = coef.shape[:-1] + (4, h, w)
    if out is not None and (tuple(out.shape) != fshape or out.dtype != dtype or not out.is_contiguous()):
        raise ValueError("out must be a contiguous %s tensor of shape %s" % (dtype, fshape))
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    st = ctypes.c_void_p(stream)
    up = lambda a: torch.from_numpy(np.array(a, order="C")).to(dev)  # noqa: E731
    c, tkx, tky, tnorm = up(coef.reshape(nimg, 4)), up(kx.reshape(nimg)), up(ky.reshape(nimg)), up(norm.reshape(nimg))
    if isinstance(window, torch.Tensor):
        win = window.to(device=dev, dtype=torch.float64).contiguous()
    else:
        win = up(np.asarray(window, np.float64))
    if tuple(win.shape) != (h, w):
        raise ValueError("window must have the grid's shape")
    lib = _lib.load()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(None)  # noqa: E731
    field = torch.empty(fshape, dtype=dtype, device=dev) if (out is None or diffraction) else out
    _lib.check(lib.dtmm_wave_field(h, w, nimg, ptr(c), ptr(tkx), ptr(tky), ptr(win), prec, ptr(field), st))
    keep = [c, tkx, tky, tnorm, win]
    if diffraction:
        i1 = torch.empty(nimg, dtype=torch.float64, device=dev)
        i2 = torch.empty(nimg, dtype=torch.float64, device=dev)
        _lib.check(lib.dtmm_field_intensity(h, w, nimg, prec, ptr(field), ptr(i1), st))
        dmat = torch.empty((nlam, h, w, 4, 4), dtype=torch.complex128, device=dev)
        ksa = np.ascontiguousarray(ks, np.float64)
        _lib.check(lib.dtmm_field_diffraction_matrix(h, w, nlam, ksa.ctypes.data_as(ctypes.c_void_p),
                                                     float(-focus), float(n * n), 0.0, -1 if backdir else 1,
                                                     float(betamax), ptr(dmat), st))
        nbytes = int(lib.dtmm_diffract_workspace_size(h, w, nimg, nlam, prec))
        if nbytes == 0:
            raise ValueError(_lib.last_error())
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        res = out if out is not None else torch.empty_like(field)
        _lib.check(lib.dtmm_diffract(h, w, nimg, nlam, prec, ptr(dmat), ptr(field), ptr(res), ptr(ws),
                                     ctypes.c_size_t(nbytes), st))
        _lib.check(lib.dtmm_field_intensity(h, w, nimg, prec, ptr(res), ptr(i2), st))
        _lib.check(lib.dtmm_scale_fields(h, w, nimg, prec, ptr(res), ptr(tnorm), ptr(i1), ptr(i2), st))
        keep += [i1, i2, dmat, ws, field]
        field = res
    else:
        _lib.check(lib.dtmm_scale_fields(h, w, nimg, prec, ptr(field), ptr(tnorm), None, None, st))
    field._dtmm_keep = keep  # inputs and scratch stay alive until the kernels have run
    return field


def illumination_device(shape, wavelengths, pixelsize=1.0, beta=0.0, phi=0.0, intensity=1.0, n=None,
                        focus=0.0, backdir=False, jones=None, diffraction=True, betamax=BETAMAX,
                        precision="double", device=None, out=None, stream=None, window=None):
    """``illumination_data`` with the grid filled on the device.

    Returns a device tensor of the field (complex128 for ``precision="double"``,
    complex64 for "mixed"), written by the ``dtmm_planewave_field`` kernel
    (or, with a ``window``, the windowed-wave, diffraction and rescale
    kernels); ``out`` may supply the destination tensor.
    """
    import ctypes

    import torch

    from . import _lib

    if window is not None:
        dev = device or torch.device("cuda", torch.cuda.current_device())
        return _window_device(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, window, backdir, jones,
                              diffraction, betamax, precision, dev, out, stream)
    coef, my, mx = illumination_modes(shape, wavelengths, pixelsize, beta, phi, intensity, n, focus, backdir, jones,
                                      diffraction, betamax)
    dev = device or torch.device("cuda", torch.cuda.current_device())
    dtype = torch.complex128 if precision == "double" else torch.complex64
    fshape = coef.shape[:-1] + (4,) + tuple(shape)
    if out is None:
        out = torch.empty(fshape, dtype=dtype, device=dev)
    elif tuple(out.shape) != fshape or out.dtype != dtype or not out.is_contiguous():
        raise ValueError("out must be a contiguous %s tensor of shape %s" % (dtype, fshape))
    nimg = int(np.prod(coef.shape[:-1]))
    c = torch.from_numpy(np.ascontiguousarray(coef.reshape(nimg, 4))).to(dev)
    iy = torch.from_numpy(my.reshape(nimg)).to(dev)
    ix = torch.from_numpy(mx.reshape(nimg)).to(dev)
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    lib = _lib.load()
    _lib.check(lib.dtmm_planewave_field(int(shape[0]), int(shape[1]), nimg, ctypes.c_void_p(c.data_ptr()),
                                        ctypes.c_void_p(iy.data_ptr()), ctypes.c_void_p(ix.data_ptr()),
                                        _lib.PRECISION_DOUBLE if precision == "double" else _lib.PRECISION_MIXED,
                                        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)))
    out._dtmm_keep = (c, iy, ix)  # the uploads stay alive until the kernel has read them
    return out
