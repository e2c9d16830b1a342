"""Input field data: plane-wave illumination (host-side, numpy).

``illumination_data`` mirrors ``dtmm.field.illumination_data``
(dtmm/field.py:586-713) for the eigenmode case (``window=None``), which is
how the reference builds the inputs of ``transfer_field``.  It prepares the
caller's input tuple ``(field, wavelengths, pixelsize)`` on the host before
any transfer starts; it is not part of the transfer path.
"""
from __future__ import annotations

import numpy as np

N_COVER = 1.5
BETAMAX = 0.8


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


def _nearest_eigenwave(waves):
    """Replace each 2D wave by the FFT-grid plane wave of largest power (dtmm/wave.py:432)."""
    shape = waves.shape
    flat = waves.reshape((-1,) + shape[-2:])
    out = np.empty(flat.shape, np.complex128)
    for i, w in enumerate(flat):
        s = np.abs(np.fft.fft2(w)) ** 2
        ii, jj = np.unravel_index(np.argmax(s), s.shape)
        f = np.zeros(s.shape, np.complex128)
        f[ii, jj] = s.sum() ** 0.5
        out[i] = np.fft.ifft2(f)
    return out.reshape(shape)


def illumination_data(shape, wavelengths, pixelsize=1.0, beta=0.0, phi=0.0, intensity=1.0, n=None,
                      focus=0.0, window=None, backdir=False, jones=None, diffraction=True,
                      eigenmodes=None, betamax=BETAMAX):
    """Forward (or backward) plane-wave illumination ``(field, wavelengths, pixelsize)``.

    Field shape: ``([nrays,] [2,] nwavelengths, 4, H, W)``; the polarisation
    axis is present when ``jones is None``.
    """
    if window is not None or eigenmodes is False:
        raise NotImplementedError("illumination_data: only window=None (eigenmode) input is supported")
    n = N_COVER if n is None else n
    wavelengths = np.asarray(wavelengths)
    ks = 2 * np.pi / wavelengths * pixelsize
    if ks.ndim != 1:
        raise ValueError("Wavelengths should be 1D array")
    if jones is None:
        intensity = intensity / 2.0
    mode = -1 if backdir else +1
    _beta = np.asarray(beta, np.float64)
    _phi = np.asarray(phi, np.float64)
    _int = np.asarray(intensity, np.float64)
    nrays = len(_beta) if _beta.ndim > 0 else 1
    b = _beta[:, None] if _beta.ndim == 1 else _beta
    p = _phi[:, None] if _phi.ndim == 1 else _phi
    # plane waves (dtmm/wave.py:376), normalised to the corner pixel
    k = ks[..., None, None]
    bb = np.asarray(b)[..., None, None]
    pp = np.asarray(p)[..., None, None]
    ay, ax = (np.arange(-l // 2 + 1.0, l // 2 + 1.0) for l in shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    waves = np.exp(1j * ((k * bb * np.cos(pp)) * xx + (k * bb * np.sin(pp)) * yy))
    waves = waves / waves[..., 0, 0][..., None, None]
    waves = _nearest_eigenwave(waves)
    b = _beta[:, None, None, None] if _beta.ndim == 1 else _beta[..., None, None]
    p = _phi[:, None, None, None] if _phi.ndim == 1 else _phi[..., None, None]
    intensity = _int[..., None, None, None, None]
    fmat = _iso_fmat(b, p, n * n)

    def one(pol):
        pol = np.asarray(pol, np.complex128)
        pol = pol / np.sqrt(pol[0] * np.conj(pol[0]) + pol[1] * np.conj(pol[1]))
        c, s = np.cos(-p), np.sin(-p)
        jv0 = c * pol[0] - s * pol[1]
        jv1 = s * pol[0] + c * pol[1]
        amp = np.broadcast_arrays(jv0, waves)
        a = np.zeros(np.broadcast_shapes(np.shape(jv0), waves.shape) + (4,), np.complex128)
        if mode == +1:
            a[..., 0] = jv0
            a[..., 2] = jv1
        else:
            a[..., 1] = jv0
            a[..., 3] = jv1
        a = a * amp[1][..., None]
        fv = np.einsum("...ij,...j->...i", fmat, a)
        return np.moveaxis(fv, -1, -3)

    if jones is None:
        f1, f2 = one((1, 0)), one((0, 1))
        sh = list(f1.shape)
        sh.insert(-4, 2)
        field = np.empty(sh, np.complex128)
        field[..., 0, :, :, :, :] = f1
        field[..., 1, :, :, :, :] = f2
    else:
        field = one(jones).copy()
    i1 = _intensity(field)
    norm = np.ones_like(i1)
    norm[:, ...] = (intensity / nrays) ** 0.5
    if diffraction:
        # diffracted_field with d = -focus, mode "t"/"r" (dtmm/diffract.py:301, :125)
        beta_k, phi_k = _fftfreq_grid(shape, ks)
        F = _iso_fmat(beta_k, phi_k, n * n)
        a = np.sqrt(n * n - beta_k ** 2 + 0j)
        alpha = np.stack([a, -a, a, -a], axis=-1)
        F[beta_k >= betamax] = 0.0
        Fi = _inv4(F)
        alpha[beta_k >= betamax] = 0.0
        ph = np.exp(1j * (ks * (-focus))[:, None, None, None] * alpha)
        if mode == +1:
            ph[..., 1::2] = 0.0
        else:
            ph[..., ::2] = 0.0
        D = np.matmul(F * ph[..., None, :], Fi)
        ff = np.fft.fft2(field)
        ff = np.einsum("...hwij,...jhw->...ihw", D, ff)
        field = np.fft.ifft2(ff)
        i2 = _intensity(field)
        ratio = (i1.sum((-2, -1)) / i2.sum((-2, -1))) ** 0.5
        norm = norm * ratio[..., None, None]
    field = field * norm[..., None, :, :]
    return field, wavelengths, pixelsize
