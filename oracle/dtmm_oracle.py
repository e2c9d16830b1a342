"""CPU restatement of dtmm's ``transfer_field`` hot path (numpy/scipy, complex128).

TEST INFRASTRUCTURE -- THIS IS THE ORACLE, NOT THE PRODUCT.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the checker / the timed CPU baseline.
The product (``dtmm_gb300``) never imports this module.

Parity pin: every function below restates the reference function cited in
its docstring (paths are relative to the reference project root).  The whole
restatement is pinned against outputs of the unmodified reference itself,
run in the build container under a pure-Python numba stand-in; those outputs
are committed as golden fixtures under ``tests/golden/`` together with the
script that produced them (``tests/golden/make_golden.py``), and
``tests/test_oracle_golden.py`` checks this module against them.  The
reference's own known-answer vectors for the k-grid maps
(``dtmm/test/test_wave.py``) and its dot-product property checks
(``dtmm/test/test_linalg.py``) are checked as well.

Scope (matches the product): ``method="4x4"`` with reflection mode 1 (the
k-space "effective" split-step operator) and ``method="2x2"`` with reflection
mode 0, diffraction >= 1 (diffraction > 1 = tent-window mode grouping),
npass >= 1 for 4x4 (norm "fft"), nstep >= 1, scalar or per-ray beta/phi or
beta/phi estimated from the field, real or complex eps, isotropic / uniaxial /
biaxial voxels, effective layers of isotropic, uniaxial or biaxial symmetry
(eff_data 0 / 1 / 2, per block or per layer) or given as optical blocks.
"""
from __future__ import annotations

import cmath
import math
import os
import warnings

import numpy as np
import scipy.fft as _sfft

FDTYPE = np.float64
CDTYPE = np.complex128

# defaults of the reference's shipped ini file (dtmm/dtmm.ini, dtmm/conf.py:459-522)
BETAMAX = 0.8
SMOOTH = 0.1
N_COVER = 1.5
DEFAULTS = {
    "nin": N_COVER,
    "nout": N_COVER,
    # the ini value is read with its quotes (dtmm/conf.py:506), so the
    # default never equals "4x4" and routes to the 2x2 method
    "method": '"2x2"',
    "npass": 1,
    "diffraction": 1,
    "reflection": None,
    "eff_data": 0,
    "betamax": BETAMAX,
}
DTMM_NORM_FFT = 1 << 0
DTMM_NORM_REF = 1 << 1

_WORKERS = int(os.environ.get("DTMM_ORACLE_THREADS", os.cpu_count() or 1))


def set_workers(n):
    """Number of threads used by the oracle's FFTs."""
    global _WORKERS
    _WORKERS = max(1, int(n))


def fft2(a):
    """Unnormalised 2D FFT over the last two axes (dtmm/fft.py:277, scipy backend :178-200)."""
    return _sfft.fft2(np.asarray(a, CDTYPE), workers=_WORKERS)


def ifft2(a):
    """1/N-normalised inverse 2D FFT over the last two axes (dtmm/fft.py:306)."""
    return _sfft.ifft2(np.asarray(a, CDTYPE), workers=_WORKERS)


# --------------------------------------------------------------------------
# k-space grids (dtmm/wave.py)
# --------------------------------------------------------------------------
def k0(wavelength, pixelsize=1.0):
    """Vacuum wavenumber in pixel units, 2*pi/lambda*pixelsize (dtmm/wave.py:280)."""
    return np.asarray(2 * np.pi / np.asarray(wavelength) * pixelsize, FDTYPE)


def betaphi(shape, k):
    """beta, phi of every FFT-grid eigenwave (dtmm/wave.py:54)."""
    k = np.abs(np.asarray(k, FDTYPE)[..., None, None])
    ay, ax = (np.asarray(np.fft.fftfreq(n), FDTYPE) for n in shape[-2:])
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    beta = (2 * np.pi / k) * np.sqrt(xx ** 2 + yy ** 2)
    phi = np.arctan2(yy, xx)
    return beta, phi


def betaxy(shape, k):
    """beta_x, beta_y of every FFT-grid eigenwave (dtmm/wave.py:84)."""
    k = np.asarray(k, FDTYPE)[..., None, None]
    ay, ax = (np.asarray(np.fft.fftfreq(n), FDTYPE) for n in shape[-2:])
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    scale = 2 * np.pi / k
    return scale * xx, scale * yy


# --------------------------------------------------------------------------
# small dense algebra on (..., n, n) stacks (dtmm/linalg.py)
# --------------------------------------------------------------------------
def inv(m):
    """Batched 2x2 / 4x4 complex inverse; an exactly singular matrix maps to 0.

    Restates ``inv`` (dtmm/linalg.py:521, ``_inv4x4`` :460, ``_inv2x2`` :428):
    adjugate over determinant, with ``det == 0`` giving an all-zero result.
    The 4x4 adjugate is formed from the 2x2 minors of the top and bottom row
    pairs (Laplace expansion by complementary minors).
    """
    m = np.asarray(m, CDTYPE)
    n = m.shape[-1]
    out = np.empty_like(m)
    if n == 2:
        a, b, c, d = m[..., 0, 0], m[..., 0, 1], m[..., 1, 0], m[..., 1, 1]
        det = a * d - b * c
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.where(det == 0, 0.0, 1.0 / np.where(det == 0, 1.0, det))
        out[..., 0, 0] = d * r
        out[..., 0, 1] = -b * r
        out[..., 1, 0] = -c * r
        out[..., 1, 1] = a * r
        return out
    if n != 4:
        raise ValueError("only 2x2 and 4x4 matrices are supported")
    a = [[m[..., i, j] for j in range(4)] for i in range(4)]
    s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1]
    s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2]
    s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3]
    s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2]
    s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3]
    s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3]
    c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3]
    c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3]
    c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2]
    c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3]
    c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2]
    c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1]
    det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(det == 0, 0.0, 1.0 / np.where(det == 0, 1.0, det))
    adj = [
        [a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3,
         -a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3,
         a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3,
         -a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3],
        [-a[1][0] * c5 + a[1][2] * c2 - a[1][3] * c1,
         a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1,
         -a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1,
         a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1],
        [a[1][0] * c4 - a[1][1] * c2 + a[1][3] * c0,
         -a[0][0] * c4 + a[0][1] * c2 - a[0][3] * c0,
         a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0,
         -a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0],
        [-a[1][0] * c3 + a[1][1] * c1 - a[1][2] * c0,
         a[0][0] * c3 - a[0][1] * c1 + a[0][2] * c0,
         -a[3][0] * s3 + a[3][1] * s1 - a[3][2] * s0,
         a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0],
    ]
    for i in range(4):
        for j in range(4):
            out[..., i, j] = adj[i][j] * r
    return out


def dotmm(a, b):
    """Batched matrix product (dtmm/linalg.py:1046)."""
    return np.matmul(np.asarray(a, CDTYPE), np.asarray(b, CDTYPE))


def dotmdm(a, d, b):
    """a . diag(d) . b per element (dtmm/linalg.py:1233)."""
    return np.matmul(np.asarray(a, CDTYPE) * np.asarray(d, CDTYPE)[..., None, :], np.asarray(b, CDTYPE))


def dotmf(a, f):
    """Per-pixel matrix times a (..., n, H, W) field (dtmm/linalg.py:979, ``_dotmf4``/``_dotmf2`` :833/:852)."""
    return np.einsum("...hwij,...jhw->...ihw", np.asarray(a, CDTYPE), np.asarray(f, CDTYPE), optimize=True)


def dotmdmf(a, d, b, f):
    """a . diag(d) . b . f per pixel (dtmm/linalg.py:1002, ``_dotmdmf4`` :905)."""
    return dotmf(dotmdm(a, d, b), f)


def dotmv(a, v):
    """Matrix times vector per element (dtmm/linalg.py:1219)."""
    return np.einsum("...ij,...j->...i", np.asarray(a, CDTYPE), np.asarray(v, CDTYPE))


# --------------------------------------------------------------------------
# rotations (dtmm/rotation.py)
# --------------------------------------------------------------------------
def rotation_vector2(angle):
    """(cos, sin) of an angle array (dtmm/rotation.py:36)."""
    angle = np.asarray(angle, FDTYPE)
    return np.stack([np.cos(angle), np.sin(angle)], axis=-1)


def _rotation_matrix_uniaxial(theta, phi):
    """R = R_phi . R_theta (dtmm/rotation.py:176)."""
    ct, st, cp, sp = np.cos(theta), np.sin(theta), np.cos(phi), np.sin(phi)
    R = np.zeros(np.shape(theta) + (3, 3), FDTYPE)
    R[..., 0, 0] = ct * cp
    R[..., 0, 1] = -sp
    R[..., 0, 2] = cp * st
    R[..., 1, 0] = ct * sp
    R[..., 1, 1] = cp
    R[..., 1, 2] = st * sp
    R[..., 2, 0] = -st
    R[..., 2, 2] = ct
    return R


def _rotation_matrix(psi, theta, phi):
    """Full Euler rotation R_phi . R_theta . R_psi (dtmm/rotation.py:125)."""
    cps, sps = np.cos(psi), np.sin(psi)
    ct, st = np.cos(theta), np.sin(theta)
    cp, sp = np.cos(phi), np.sin(phi)
    R = np.empty(np.shape(theta) + (3, 3), FDTYPE)
    R[..., 0, 0] = ct * (cp * cps) - sp * sps
    R[..., 0, 1] = -ct * (cp * sps) - sp * cps
    R[..., 0, 2] = cp * st
    R[..., 1, 0] = ct * (sp * cps) + cp * sps
    R[..., 1, 1] = cp * cps - ct * (sp * sps)
    R[..., 1, 2] = st * sp
    R[..., 2, 0] = -cps * st
    R[..., 2, 1] = st * sps
    R[..., 2, 2] = ct
    return R


def _rotate_diagonal_tensor(R, diag):
    """R . diag . R^T as 6 independent entries (dtmm/rotation.py:285)."""
    out = np.empty(R.shape[:-2] + (6,), CDTYPE)
    d0, d1, d2 = diag[..., 0], diag[..., 1], diag[..., 2]
    for i in range(3):
        out[..., i] = d0 * R[..., i, 0] ** 2 + d1 * R[..., i, 1] ** 2 + d2 * R[..., i, 2] ** 2
    for k, (i, j) in zip((3, 4, 5), ((0, 1), (0, 2), (1, 2))):
        out[..., k] = d0 * R[..., i, 0] * R[..., j, 0] + d1 * R[..., i, 1] * R[..., j, 1] + d2 * R[..., i, 2] * R[..., j, 2]
    return out


def _dotr2m(rv, F):
    """Rotate a field matrix about z by (cos, sin) = rv (dtmm/linalg.py:674)."""
    r0 = rv[..., 0][..., None]
    r1 = rv[..., 1][..., None]
    out = np.empty_like(F)
    out[..., 0, :] = F[..., 0, :] * r0 - F[..., 2, :] * r1
    out[..., 1, :] = F[..., 1, :] * r0 + F[..., 3, :] * r1
    out[..., 2, :] = F[..., 0, :] * r1 + F[..., 2, :] * r0
    out[..., 3, :] = -F[..., 1, :] * r1 + F[..., 3, :] * r0
    return out


# --------------------------------------------------------------------------
# Berreman eigen-solve (dtmm/tmm.py)
# --------------------------------------------------------------------------
def _alphaf_iso(beta, eps0):
    """Isotropic eigenvalues and field matrix, phi = 0 frame (dtmm/tmm.py:124)."""
    n = beta.shape[0]
    alpha = np.zeros((n, 4), CDTYPE)
    F = np.zeros((n, 4, 4), CDTYPE)
    aout = np.sqrt(eps0 - beta ** 2)
    ok = aout != 0
    with np.errstate(divide="ignore", invalid="ignore"):
        gp = np.where(ok, eps0 / np.where(ok, aout, 1.0), 0.0)
    gs = -aout
    alpha[:, 0] = aout
    alpha[:, 1] = -aout
    alpha[:, 2] = aout
    alpha[:, 3] = -aout
    F[:, 0, 0] = 0.5
    F[:, 0, 1] = 0.5
    F[:, 1, 0] = 0.5 * gp
    F[:, 1, 1] = -0.5 * gp
    F[:, 2, 2] = 0.5
    F[:, 2, 3] = 0.5
    F[:, 3, 2] = 0.5 * gs
    F[:, 3, 3] = -0.5 * gs
    alpha[~ok] = 0.0
    F[~ok] = 0.0
    return alpha, F


def _alphaf_uniaxial(beta, eps0, R):
    """Analytic uniaxial eigenvalues and column-normalised field matrix (dtmm/tmm.py:157)."""
    n = beta.shape[0]
    alpha = np.empty((n, 4), CDTYPE)
    F = np.empty((n, 4, 4), CDTYPE)
    ct = R[:, 2, 2]
    st = -R[:, 2, 0]
    st2 = st * st
    ct2 = ct * ct
    sf = -R[:, 0, 1]
    cf = R[:, 1, 1]
    eps11 = eps0[:, 0]
    delta = eps0[:, 2] - eps11
    z = beta == 0.0
    nz = ~z
    # beta == 0 branch
    evs = np.empty(n, CDTYPE)
    evpp = np.empty(n, CDTYPE)
    evpm = np.empty(n, CDTYPE)
    ev02 = np.empty(n, CDTYPE)
    if z.any():
        e11 = eps11[z]
        ev02[z] = e11
        evs[z] = np.sqrt(e11)
        u = e11 + delta[z] * ct2[z]
        w = e11 * (e11 + delta[z])
        sq = np.sqrt(u * w) / u
        evpp[z] = sq
        evpm[z] = -sq
    if nz.any():
        e11 = eps11[nz]
        b = beta[nz]
        e02 = e11 - b * b
        ev02[nz] = e02
        evs[nz] = np.sqrt(e02)
        u = e11 + delta[nz] * ct2[nz]
        gama = b * cf[nz]
        v = gama * delta[nz] * 2 * st[nz] * ct[nz]
        w = gama * gama * (delta[nz] * st2[nz]) - e11 * (e02 + delta[nz])
        sq = np.sqrt(v * v - 4 * u * w) / 2 / u
        v = v / 2 / u
        evpp[nz] = -v + sq
        evpm[nz] = -v - sq
    alpha[:, 0] = evpp
    alpha[:, 1] = evpm
    alpha[:, 2] = evs
    alpha[:, 3] = -evs
    if z.any():
        e11, s, c, es = eps11[z], sf[z], cf[z], evs[z]
        pp, pm = evpp[z], evpm[z]
        F[z, 0, 2] = -es * s
        F[z, 1, 2] = -e11 * s
        F[z, 2, 2] = es * c
        F[z, 3, 2] = -e11 * c
        F[z, 0, 3] = -es * s
        F[z, 1, 3] = e11 * s
        F[z, 2, 3] = es * c
        F[z, 3, 3] = e11 * c
        F[z, 0, 0] = c
        F[z, 1, 0] = pp * c
        F[z, 2, 0] = s
        F[z, 3, 0] = -pp * s
        F[z, 0, 1] = c
        F[z, 1, 1] = pm * c
        F[z, 2, 1] = s
        F[z, 3, 1] = -pm * s
    if nz.any():
        e11, es, e02 = eps11[nz], evs[nz], ev02[nz]
        pp, pm = evpp[nz], evpm[nz]
        sfst = R[nz, 1, 2]
        cfst = R[nz, 0, 2]
        ctbeta = ct[nz] * beta[nz]
        ctbetaeps11 = ctbeta / e11
        eps11sfst = e11 * sfst
        evssfst = es * sfst
        evscfst = es * cfst
        evsctbeta = es * ctbeta
        ev02cfst = e02 * cfst
        ev02cfsteps11 = ev02cfst / e11
        F[nz, 0, 2] = evssfst
        F[nz, 1, 2] = eps11sfst
        F[nz, 2, 2] = ctbeta - evscfst
        F[nz, 3, 2] = ev02cfst - evsctbeta
        F[nz, 0, 3] = -evssfst
        F[nz, 1, 3] = eps11sfst
        F[nz, 2, 3] = evscfst + ctbeta
        F[nz, 3, 3] = ev02cfst + evsctbeta
        F[nz, 0, 0] = pp * ctbetaeps11 - ev02cfsteps11
        F[nz, 1, 0] = ctbeta - pp * cfst
        F[nz, 2, 0] = -sfst
        F[nz, 3, 0] = pp * sfst
        F[nz, 0, 1] = -pm * ctbetaeps11 + ev02cfsteps11
        F[nz, 1, 1] = pm * cfst - ctbeta
        F[nz, 2, 1] = sfst
        F[nz, 3, 1] = -pm * sfst
    norm = np.sqrt((F.real ** 2 + F.imag ** 2).sum(axis=1))
    F = F / norm[:, None, :]
    return alpha, F


def _auxiliary_matrix(beta, eps):
    """Berreman auxiliary 4x4 matrix in the phi = 0 frame (dtmm/tmm.py:100)."""
    n = beta.shape[0]
    L = np.zeros((n, 4, 4), CDTYPE)
    eps2m = 1.0 / eps[:, 2]
    e4 = eps[:, 4] * eps2m
    e5 = eps[:, 5] * eps2m
    L[:, 0, 0] = -beta * e4
    L[:, 0, 1] = 1.0 - beta * beta * eps2m
    L[:, 0, 2] = -beta * e5
    L[:, 1, 0] = eps[:, 0] - eps[:, 4] * e4
    L[:, 1, 1] = L[:, 0, 0]
    L[:, 1, 2] = eps[:, 3] - eps[:, 5] * e4
    L[:, 2, 3] = -1.0
    L[:, 3, 0] = -L[:, 1, 2]
    L[:, 3, 1] = -L[:, 0, 2]
    L[:, 3, 2] = beta * beta + eps[:, 5] * e5 - eps[:, 1]
    return L


def _poynting_columns(F):
    """z-Poynting of every column of a field matrix (dtmm/tmm.py:293)."""
    return (F[:, 0, :].real * F[:, 1, :].real + F[:, 0, :].imag * F[:, 1, :].imag) - (
        F[:, 2, :].real * F[:, 3, :].real + F[:, 2, :].imag * F[:, 3, :].imag
    )


def _alphaf_biaxial(beta, phi, eps0, epsa):
    """General eigen-solve and Poynting sort (dtmm/tmm.py:395-401, ``_copy_sorted`` :300)."""
    R = _rotation_matrix(epsa[:, 0], epsa[:, 1], epsa[:, 2] - phi)
    eps = _rotate_diagonal_tensor(R, eps0)
    L = _auxiliary_matrix(beta, eps)
    a0, F0 = np.linalg.eig(L)
    n = beta.shape[0]
    alpha = np.empty((n, 4), CDTYPE)
    F = np.empty((n, 4, 4), CDTYPE)
    p = _poynting_columns(F0)
    for m in range(n):
        i, j, ok = 0, 1, True
        for k in range(4):
            if p[m, k] >= 0.0:
                if i >= 4:
                    ok = False
                if ok:
                    alpha[m, i] = a0[m, k]
                    F[m, :, i] = F0[m, :, k]
                i += 2
            else:
                if j >= 4:
                    ok = False
                if ok:
                    alpha[m, j] = a0[m, k]
                    F[m, :, j] = F0[m, :, k]
                j += 2
        if not ok:
            print("Could not sort eigenvectors! Proceed with caution!")
            alpha[m] = np.nan
            F[m] = 0.0
    return alpha, F


def alphaf(beta=None, phi=None, epsv=None, epsa=None):
    """Eigenvalues alpha (..., 4) and field matrix F (..., 4, 4).

    Restates ``alphaf`` (dtmm/tmm.py:435) -> ``_alphaf_vec`` (dtmm/tmm.py:372):
    the isotropic / uniaxial / biaxial branch is chosen per element by exact
    equality of the eps eigenvalues, the solution is found in the plane of
    incidence (phi = 0) and rotated back by phi.
    """
    beta = np.asarray(0.0 if beta is None else beta, FDTYPE)
    phi = np.asarray(0.0 if phi is None else phi, FDTYPE)
    epsv = np.asarray((1.0, 1.0, 1.0) if epsv is None else epsv, CDTYPE)
    epsa = np.asarray((0.0, 0.0, 0.0) if epsa is None else epsa, FDTYPE)
    shape = np.broadcast_shapes(beta.shape, phi.shape, epsv.shape[:-1], epsa.shape[:-1])
    b = np.broadcast_to(beta, shape).reshape(-1)
    p = np.broadcast_to(phi, shape).reshape(-1)
    ev = np.broadcast_to(epsv[..., :3], shape + (3,)).reshape(-1, 3)
    ea = np.broadcast_to(epsa[..., :3], shape + (3,)).reshape(-1, 3)
    n = b.shape[0]
    alpha = np.empty((n, 4), CDTYPE)
    F = np.empty((n, 4, 4), CDTYPE)
    iso = (ev[:, 0] == ev[:, 1]) & (ev[:, 1] == ev[:, 2])
    uni = (ev[:, 0] == ev[:, 1]) & ~iso
    bi = ~(ev[:, 0] == ev[:, 1])
    if iso.any():
        alpha[iso], F[iso] = _alphaf_iso(b[iso], ev[iso, 0])
    if uni.any():
        R = _rotation_matrix_uniaxial(ea[uni, 1], ea[uni, 2] - p[uni])
        alpha[uni], F[uni] = _alphaf_uniaxial(b[uni], ev[uni], R)
    if bi.any():
        alpha[bi], F[bi] = _alphaf_biaxial(b[bi], p[bi], ev[bi], ea[bi])
    F = _dotr2m(rotation_vector2(p), F)
    return alpha.reshape(shape + (4,)), F.reshape(shape + (4, 4))


def alphaffi(beta=None, phi=None, epsv=None, epsa=None):
    """alphaf plus the inverse field matrix (dtmm/tmm.py:466)."""
    a, f = alphaf(beta, phi, epsv, epsa)
    return a, f, inv(f)


def E_mat(fmat, mode=None):
    """E-field rows of the field matrix (dtmm/tmm.py:974).

    mode +1 / -1: the 2x2 block of forward / backward modes; mode None: the
    4x4 "Epn" matrix with the forward block at [::2, ::2] and the backward
    block at [1::2, 1::2].
    """
    fmat = np.asarray(fmat)
    if mode == +1:
        return fmat[..., ::2, ::2].copy()
    if mode == -1:
        return fmat[..., ::2, 1::2].copy()
    out = np.zeros_like(fmat)
    out[..., ::2, ::2] = fmat[..., ::2, ::2]
    out[..., 1::2, 1::2] = fmat[..., ::2, 1::2]
    return out


def E2H_mat(fmat, mode=+1):
    """H-from-E matrix B . A^-1 of one propagation direction (dtmm/tmm.py:1051)."""
    if mode == +1:
        A, B = fmat[..., ::2, ::2], fmat[..., 1::2, ::2]
    else:
        A, B = fmat[..., ::2, 1::2], fmat[..., 1::2, 1::2]
    return dotmm(B, inv(A))


def phasem(alpha, kd):
    """exp(i kd alpha) (dtmm/tmm.py:584-596)."""
    kd = np.asarray(kd, FDTYPE)[..., None]
    return np.exp(1j * kd * np.asarray(alpha, CDTYPE))


def phase_mat(alpha, kd, mode=None):
    """Phase diagonal, optionally of one direction only (dtmm/tmm.py:599)."""
    alpha = np.asarray(alpha)
    if mode == +1:
        return phasem(alpha[..., ::2], kd)
    if mode == -1:
        return phasem(alpha[..., 1::2], kd)
    return phasem(alpha, kd)


def alphaEEi(beta, phi, epsv, epsa, mode=+1):
    """2x2 E eigen-data of one direction and its inverse (dtmm/tmm.py:509-582)."""
    alpha, f = alphaf(beta, phi, epsv, epsa)
    e = E_mat(f, mode=mode)
    alpha = alpha[..., ::2] if mode == 1 else alpha[..., 1::2]
    return alpha, e, inv(e)


# --------------------------------------------------------------------------
# effective-medium diffraction matrices (dtmm/diffract.py, dtmm/matrix.py)
# --------------------------------------------------------------------------
def diffraction_alphaf(shape, ks, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0), betamax=BETAMAX):
    """Per-k eigen-data of a homogeneous layer; beta >= betamax zeroed (dtmm/diffract.py:22)."""
    ks = np.abs(np.asarray(ks))
    beta, phi = betaphi(shape, ks)
    alpha, f = alphaf(beta, phi, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE))
    mask = beta >= betamax
    f[mask] = 0.0
    alpha[mask] = 0.0
    return alpha, f


def diffraction_alphaffi(shape, ks, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0), betamax=BETAMAX):
    """diffraction_alphaf plus inverse (dtmm/diffract.py:47)."""
    ks = np.abs(np.asarray(ks))
    beta, phi = betaphi(shape, ks)
    alpha, f, fi = alphaffi(beta, phi, epsv, epsa)
    mask = beta >= betamax
    fi[mask] = 0.0
    f[mask] = 0.0
    alpha[mask] = 0.0
    return alpha, f, fi


def E_diffraction_alphaEEi(shape, ks, epsv=(1, 1, 1), epsa=(0.0, 0.0, 0.0), mode=+1, betamax=BETAMAX):
    """2x2 per-k E eigen-data; beta >= betamax zeroed (dtmm/diffract.py:79)."""
    ks = np.abs(np.asarray(ks))
    beta, phi = betaphi(shape, ks)
    alpha, j, ji = alphaEEi(beta, phi, epsv, epsa, mode=mode)
    mask = beta >= betamax
    ji[mask] = 0.0
    j[mask] = 0.0
    alpha[mask] = 0.0
    return alpha, j, ji


def phase_matrix(alpha, kd, mode=None):
    """Phase diagonal with optional direction mask (dtmm/diffract.py:113)."""
    kd = np.asarray(kd, FDTYPE)
    out = phase_mat(alpha, kd[..., None, None])
    if mode in ("t", +1):
        out[..., 1::2] = 0.0
    elif mode in ("r", -1):
        out[..., ::2] = 0.0
    return out


def tr_mat(fmatin, fmatout, fmatini=None, mode=+1):
    """2x2 interface transmission / reflection matrices (dtmm/tmm.py:925, ``Etri_mat`` :1025, ``S_mat`` :850)."""
    if fmatini is None:
        fmatini = inv(fmatin)
    er = E_mat(fmatin, mode=-mode)
    et = E_mat(fmatout, mode=mode)
    A = E_mat(fmatin, mode=mode)
    S = dotmm(fmatini, fmatout)
    if mode == +1:
        St, Sr = S[..., ::2, ::2], S[..., 1::2, 0::2]
    else:
        St, Sr = S[..., 1::2, 1::2], S[..., 0::2, 1::2]
    ei = dotmm(inv(St), inv(A))
    eri = dotmm(Sr, ei)
    return dotmm(et, ei), dotmm(er, eri)


def S_mat(fmatin, fmatout, fmatini=None, mode=+1):
    """Transmission / reflection blocks of F_in^-1 . F_out (dtmm/tmm.py:850-878)."""
    if fmatini is None:
        fmatini = inv(fmatin)
    S = dotmm(fmatini, fmatout)
    if mode == +1:
        return S[..., ::2, ::2], S[..., 1::2, 0::2]
    return S[..., 1::2, 1::2], S[..., 0::2, 1::2]


def Eti_mat(fmatin, fmatout, fmatini=None, mode=+1):
    """Inverse E matrix through an interface without reflections (dtmm/tmm.py:999-1022)."""
    Ai = inv(E_mat(fmatin, mode=mode))
    St, _ = S_mat(fmatin, fmatout, fmatini=fmatini, mode=mode)
    return dotmm(inv(St), Ai)


def projection_mat(fmat, fmati=None, mode=+1):
    """F . diag(forward or backward modes) . F^-1 (dtmm/tmm.py:742-768)."""
    if fmati is None:
        fmati = inv(fmat)
    diag = np.zeros(fmat.shape[:-1], fmat.dtype)
    if mode == 1:
        diag[..., 0::2] = 1.0
    else:
        diag[..., 1::2] = 1.0
    return dotmdm(fmat, diag, fmati)


def transmitted_field_direct(field, beta, phi, n=1.0):
    """The forward part of a field for one beam direction, in real space
    (dtmm/transfer.py:94-101)."""
    ev = refind2eps([n] * 3)
    ea = np.zeros_like(ev)
    alpha, fmat = alphaf(beta, phi, ev, ea)
    pmat = projection_mat(fmat)
    return np.moveaxis(dotmv(pmat, np.moveaxis(field, -3, -1)), -1, -3)


def E_tr_matrix(shape, ks, epsv_in=(1.0, 1.0, 1.0), epsa_in=(0.0, 0.0, 0.0), epsv_out=(1.0, 1.0, 1.0),
                epsa_out=(0.0, 0.0, 0.0), mode=+1, betamax=BETAMAX):
    """Per-k Fresnel t, r matrices between two homogeneous layers (dtmm/diffract.py:215)."""
    _, fin, fini = diffraction_alphaffi(shape, ks, epsv_in, epsa_in, betamax)
    _, fout, _ = diffraction_alphaffi(shape, ks, epsv_out, epsa_out, betamax)
    return tr_mat(fin, fout, fmatini=fini, mode=mode)


def E_diffraction_matrix(shape, ks, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1, betamax=BETAMAX):
    """2x2 E-basis diffraction over d (dtmm/diffract.py:173)."""
    ks = np.asarray(ks, FDTYPE)
    alpha, j, ji = E_diffraction_alphaEEi(shape, ks, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE), mode, betamax)
    return dotmdm(j, phase_matrix(alpha, ks * d), ji)


def projection_matrix(shape, ks, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1, betamax=BETAMAX):
    """Per-k projection onto forward (+1) or backward (-1) modes (dtmm/diffract.py:242)."""
    ks = np.asarray(ks, FDTYPE)
    alpha, f, fi = diffraction_alphaffi(shape, ks, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE), betamax)
    pmat = phase_matrix(alpha, np.zeros_like(ks), mode=mode)
    return dotmdm(f, pmat, fi)


def diffract(field, dmat):
    """fft2 -> per-k matrix -> ifft2 (dtmm/diffract.py:254)."""
    return ifft2(dotmf(dmat, fft2(field)))


def jones2H(jones, ks, n=1.0, betamax=BETAMAX, mode=+1):
    """H components of an E (Jones) field in the isotropic medium n, per k
    through the medium's E2H matrix, zero beyond betamax (dtmm/transfer.py:255-267)."""
    eps = refind2eps([n] * 3)
    _, f, _ = diffraction_alphaffi(jones.shape[-2:], ks, epsv=eps, epsa=np.zeros(3, FDTYPE), betamax=betamax)
    return diffract(jones, E2H_mat(f, mode=mode))


def E_correction_matrix(beta, phi, ks, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1):
    """Inverse phase of the beam's own 2x2 E mode over d (dtmm/matrix.py:32)."""
    alpha, j, ji = alphaEEi(beta, phi, epsv, epsa, mode=mode)
    return dotmdm(j, phase_matrix(alpha, -np.asarray(ks) * d), ji)


def first_E_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1, betamax=BETAMAX):
    """correction . diffraction, 2x2 (dtmm/matrix.py:54)."""
    dmat = E_diffraction_matrix(shape, ks, d, epsv, epsa, mode=mode, betamax=betamax)
    cmat = E_correction_matrix(beta, phi, ks, d, epsv, epsa, mode=mode)
    return dotmm(cmat, dmat)


def second_E_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1, betamax=BETAMAX):
    """diffraction . correction, 2x2 (dtmm/matrix.py:47)."""
    dmat = E_diffraction_matrix(shape, ks, d, epsv, epsa, mode=mode, betamax=betamax)
    cmat = E_correction_matrix(beta, phi, ks, d, epsv, epsa, mode=mode)
    return dotmm(dmat, cmat)


def corrected_E_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), mode=+1,
                                   betamax=BETAMAX):
    """C . D . C of one direction, 2x2, C over d / 2 (dtmm/matrix.py:38-43)."""
    dmat = E_diffraction_matrix(shape, ks, d, epsv, epsa, mode=mode, betamax=betamax)
    cmat = E_correction_matrix(beta, phi, ks, d / 2.0, epsv, epsa, mode=mode)
    return dotmm(cmat, dotmm(dmat, cmat))


def corrected_Epn_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), betamax=BETAMAX):
    """The forward and backward corrected E diffraction matrices (dtmm/matrix.py:61-68)."""
    ep = corrected_E_diffraction_matrix(shape, ks, beta, phi, d=d, epsv=epsv, epsa=epsa, mode=+1, betamax=betamax)
    en = corrected_E_diffraction_matrix(shape, ks, beta, phi, d=d, epsv=epsv, epsa=epsa, mode=-1, betamax=betamax)
    return ep, en


def first_Epn_diffraction_matrix(shape, ks, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), betamax=BETAMAX):
    """field -> Epn diffraction over d: E . P . F^-1 (dtmm/matrix.py:110)."""
    ks = np.asarray(ks, FDTYPE)
    alpha, f, fi = diffraction_alphaffi(shape, ks, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE), betamax)
    return dotmdm(E_mat(f), phase_mat(alpha, (ks * d)[..., None, None]), fi)


def second_Epn_diffraction_matrix(shape, ks, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), betamax=BETAMAX):
    """Epn -> field diffraction over d: F . P . E^-1 (dtmm/matrix.py:121)."""
    ks = np.asarray(ks, FDTYPE)
    alpha, f = diffraction_alphaf(shape, ks, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE), betamax)
    return dotmdm(f, phase_mat(alpha, (ks * d)[..., None, None]), inv(E_mat(f)))


def Epn_correction_matrix(beta, phi, ks, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0)):
    """Inverse phase of the beam's own Epn modes over d (dtmm/matrix.py:133)."""
    alpha, f = alphaf(beta, phi, epsv, epsa)
    pmat = phase_mat(alpha, (-np.asarray(ks) * d)[..., None, None])
    e = E_mat(f)
    return dotmdm(e, pmat, inv(e))


def first_corrected_Epn_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), betamax=BETAMAX):
    """(dtmm/matrix.py:142)"""
    return dotmm(Epn_correction_matrix(beta, phi, ks, d, epsv, epsa),
                 first_Epn_diffraction_matrix(shape, ks, d, epsv, epsa, betamax=betamax))


def second_corrected_Epn_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1, 1, 1), epsa=(0, 0, 0.0), betamax=BETAMAX):
    """(dtmm/matrix.py:160)"""
    return dotmm(second_Epn_diffraction_matrix(shape, ks, d, epsv, epsa, betamax=betamax),
                 Epn_correction_matrix(beta, phi, ks, d, epsv, epsa))


# --------------------------------------------------------------------------
# mode grouping windows (dtmm/mode.py)
# --------------------------------------------------------------------------
def _tent(db, typ):
    """One axis of a tent window, open-ended at the grid edges (dtmm/mode.py:18-40)."""
    c = 1.0 - np.abs(db)
    neg = c < 0.0
    c = np.where(neg, 0.0, c)
    if typ < 0:
        c = np.where(~neg & (db < 0), 1.0, c)
    elif typ > 0:
        c = np.where(~neg & (db > 0), 1.0, c)
    return c


def _nearest_offset(off, d):
    """Offset folded to the nearest multiple of d (dtmm/mode.py:54-70)."""
    a = np.mod(off, d)
    b = np.mod(off, -d)
    return np.where(np.abs(a) > np.abs(b), b, a)


def fft_windows(bx, by, n, betax_off=0.0, betay_off=0.0, betamax=BETAMAX):
    """n*n tent windows over (beta_x, beta_y) (dtmm/mode.py:52 with ``fft_window`` :11)."""
    d = 2 * betamax / (n - 1)
    xoff = _nearest_offset(np.asarray(betax_off, FDTYPE), d)
    yoff = _nearest_offset(np.asarray(betay_off, FDTYPE), d)
    ax = np.linspace(-betamax, betamax, n)
    step = ax[1] - ax[0]
    beta = (bx ** 2 + by ** 2) ** 0.5
    # a per-ray offset broadcasts as an extra loop dimension in front of the
    # grid's own loop dimensions, as in the reference's gufunc call
    xoff_b = xoff[..., None, None]
    yoff_b = yoff[..., None, None]
    out = []
    for i, cx0 in enumerate(ax):
        xt = -1 if i == 0 else (1 if i == n - 1 else 0)
        cx = _tent((bx - (cx0 + xoff_b)) / step, xt)
        for j, cy0 in enumerate(ax):
            yt = -1 if j == 0 else (1 if j == n - 1 else 0)
            cy = _tent((by - (cy0 + yoff_b)) / step, yt)
            coeff = np.where(beta >= betamax, 0.0, cx * cy)
            out.append(np.where(coeff > 0.0, coeff, 0.0))
    return np.asarray(out)


def fft_mask(shape, ks, n, betax_off=0.0, betay_off=0.0, betamax=BETAMAX):
    """Non-empty windows and their intensity-weighted mean beta, phi (dtmm/mode.py:104-139).

    The mean is taken over every axis of the grid, wavelengths included
    (``fft_betaxy_mean``, dtmm/mode.py:108).
    """
    bx, by = betaxy(shape[-2:], np.asarray(ks, FDTYPE)[..., None])
    w = fft_windows(bx, by, n, betax_off, betay_off, betamax)
    axis = tuple(range(-bx.ndim, 0))
    w2 = w ** 2
    norm = w2.sum(axis=axis)
    sx = (bx * w2).sum(axis=axis)
    sy = (by * w2).sum(axis=axis)
    mask = norm > 0
    mx = np.divide(sx, norm, where=mask, out=sx.copy())
    my = np.divide(sy, norm, where=mask, out=sy.copy())
    betas = (mx ** 2 + my ** 2) ** 0.5
    phis = np.arctan2(my, mx)
    nonzero = np.asarray([not np.all(x == 0.0) for x in w])
    return w[nonzero], (betas[nonzero], phis[nonzero])


# --------------------------------------------------------------------------
# field helpers (dtmm/field.py, dtmm/transfer.py, dtmm/denoise.py)
# --------------------------------------------------------------------------
def field2intensity(field):
    """z-Poynting per pixel of a (..., 4, H, W) field (dtmm/field.py:780)."""
    f = np.asarray(field)
    return (f[..., 0, :, :].real * f[..., 1, :, :].real + f[..., 0, :, :].imag * f[..., 1, :, :].imag) - (
        f[..., 2, :, :].real * f[..., 3, :, :].real + f[..., 2, :, :].imag * f[..., 3, :, :].imag
    )


def total_intensity(field):
    """Pixel sum of field2intensity (dtmm/transfer.py:200)."""
    i = field2intensity(field)
    return i.sum(axis=(-2, -1))


def normalize_field(field, intensity_in, intensity_out):
    """Scale each k so its intensity matches the reference, |ratio| clamped to 1 (dtmm/transfer.py:67)."""
    intensity_in = intensity_in.copy()
    intensity_out = intensity_out.copy()
    m = intensity_out == 0.0
    intensity_out[m] = 1.0
    intensity_in[m] = 0.0
    fact = (intensity_in / intensity_out)[..., None, :, :]
    fact = np.abs(np.clip(fact, -1, 1))
    return field * fact


def project_normalized_fft(field, dmat, ref=None):
    """Project in k-space and restore each mode's intensity (dtmm/transfer.py:78).
    With ``ref`` the intensities are the reference field's, and the field
    itself is not used: the reference's call passes out=field
    (dtmm/transfer.py:830), so fft2(ref) overwrites the field before the
    field's own transform, which then transforms fft2(ref) once more
    (dtmm/transfer.py:79-82); the projected field is fft2(fft2(ref))."""
    if ref is not None:
        fref = fft2(ref)
        i1 = field2intensity(fref)
        f1 = fft2(fref)
    else:
        f1 = fft2(field)
        i1 = field2intensity(f1)
    f2 = dotmf(dmat, f1)
    i2 = field2intensity(f2)
    return ifft2(normalize_field(f2, i1, i2))


def project_normalized_total(field, dmat):
    """Project in k-space and restore the total intensity of each image, |ratio|
    clamped to 1 (dtmm/transfer.py:123-155, norm "total", ref=None)."""
    i1 = total_intensity(field)
    out = ifft2(dotmf(dmat, fft2(field)))
    i2 = total_intensity(out)
    m = i2 == 0.0
    i2 = np.where(m, 1.0, i2)
    i1 = np.where(m, 0.0, i1)
    fact = np.abs(np.clip(i1 / i2, -1, 1))
    return out * fact[..., None, None, None]


def project_normalized_local(field, dmat, nout, ref=None):
    """Project in k-space, then per pixel split the field (or the reference
    field) by the polarizer of the projection's forward amplitudes at normal
    incidence in the output medium: the polarised part carries the
    projection's intensity restored to the polarised part's, the rest is
    added unchanged (dtmm/transfer.py:103-136; f_iso and fvec2avec
    dtmm/tmm.py:1074, :1851; jonesvec and polarizer dtmm/jones.py:55, :236;
    ray_jonesmat4x4 with jonesmat4x4 and as4x4 dtmm/jones4.py:205, :75,
    dtmm/jones.py:371, at beta = phi = 0)."""
    f = ifft2(dotmf(dmat, fft2(field)))
    epsv = np.asarray(refind2eps([nout] * 3), CDTYPE)
    _, fmat = alphaf(0.0, 0.0, epsv, np.zeros(3, FDTYPE))
    fn = normalize_f(fmat)
    fni = inv(fn)
    a = dotmv(fni, np.moveaxis(f, -3, -1))  # eigen-amplitudes per pixel
    jv = a[..., 0::2]
    norm = (jv[..., 0] * jv[..., 0].conj() + jv[..., 1] * jv[..., 1].conj()) ** 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        jv = jv / norm[..., None]
    jmat = np.empty(jv.shape + (2,), CDTYPE)
    c, sn = jv[..., 0], jv[..., 1]
    jmat[..., 0, 0] = c * c.conj()
    jmat[..., 0, 1] = c * sn.conj()
    jmat[..., 1, 0] = sn * c.conj()
    jmat[..., 1, 1] = sn * sn.conj()
    m4 = np.zeros(jmat.shape[:-2] + (4, 4), CDTYPE)
    m4[..., 0::2, 0::2] = jmat
    m4[..., 1::2, 1::2] = np.conj(jmat)
    pmat1 = dotmm(fn, dotmm(m4, fni))
    pmat2 = -pmat1
    for k in range(4):
        pmat2[..., k, k] += 1
    src = field if ref is None else ref
    i1 = field2intensity(dotmf(pmat1, src))
    rest = dotmf(pmat2, src)
    i2 = field2intensity(f)
    return normalize_field(f, i1, i2) + rest


def exp_notch_filter(x, x0, sigma):
    """Attenuation around beta = x0 (dtmm/denoise.py:21)."""
    return np.asarray((1 - np.exp(-np.abs(x - x0).clip(0, x0) / sigma)) / (1 - np.exp(-x0 / sigma)), FDTYPE)


def denoise_fftfield(ffield, ks, beta, smooth):
    """(dtmm/denoise.py:31)"""
    b, _ = betaphi(ffield.shape[-2:], ks)
    return ffield * exp_notch_filter(b, beta, smooth)[..., None, :, :]


def denoise_field(field, ks, beta, smooth):
    """(dtmm/denoise.py:24)"""
    return ifft2(denoise_fftfield(fft2(field), ks, beta, smooth))


def refind2eps(n):
    """n**2 (dtmm/data.py:1065)."""
    return np.asarray(n) ** 2


def transmitted_field(field, ks, n=1.0, betamax=BETAMAX):
    """Forward-propagating part of a field in medium n (dtmm/transfer.py:270)."""
    eps = refind2eps([n] * 3)
    pmat = projection_matrix(field.shape[-2:], ks, epsv=eps, epsa=(0.0, 0.0, 0.0), mode=+1, betamax=betamax)
    return diffract(field, pmat)


def reflected_field(field, ks, n=1.0, betamax=BETAMAX):
    """Backward-propagating part of a field in medium n (dtmm/transfer.py:295)."""
    eps = refind2eps([n] * 3)
    pmat = projection_matrix(field.shape[-2:], ks, epsv=eps, epsa=(0.0, 0.0, 0.0), mode=-1, betamax=betamax)
    return diffract(field, pmat)


def blackman(shape):
    """2D radial Blackman window (dtmm/window.py:33)."""
    ay, ax = (np.arange(-n / 2.0 + 0.5, n / 2.0 + 0.5) for n in shape)
    xx, yy = np.meshgrid(ax, ay, indexing="xy")
    ny, nx = (n / 2 for n in shape)
    r = ((xx / nx) ** 2 + (yy / ny) ** 2) ** 0.5
    out = 0.42 + 0.5 * np.cos(np.pi * r) + 0.08 * np.cos(2 * np.pi * r)
    out[r >= 1.0] = 0.0
    return out


def field2betaphi(field_in, ks, multiray=False):
    """Mean beta, phi of a field (dtmm/field.py:492, ``mean_betaphi`` :866, ``_fft_betaphi`` :846)."""
    f = fft2(field_in * blackman(field_in.shape[-2:]))
    bx, by = betaxy(field_in.shape[-2:], ks)
    s = f.real ** 2 + f.imag ** 2
    sx = (s * bx[..., None, :, :]).sum(axis=(-3, -2, -1))
    sy = (s * by[..., None, :, :]).sum(axis=(-3, -2, -1))
    ss = s.sum(axis=(-3, -2, -1))
    beta = (sx ** 2 + sy ** 2) ** 0.5 / ss
    phi = np.arctan2(sy, sx)
    if field_in.ndim > 4 and multiray:
        ax = tuple(range(1, field_in.ndim - 3))
        return beta.mean(axis=ax), phi.mean(axis=ax)
    return beta.mean(), phi.mean()


def _validate_betaphi(beta, phi, extendeddim=0):
    """Broadcastable beta, phi (dtmm/transfer.py:43)."""
    if beta is None or phi is None:
        raise ValueError("Both beta and phi must be defined!")
    beta = np.asarray(beta, FDTYPE)
    phi = np.asarray(phi, FDTYPE)
    if beta.ndim != phi.ndim:
        raise ValueError("Beta nad phi should have same dimensions!")
    if beta.ndim == 1:
        if len(beta) != len(phi):
            raise ValueError("Beta nad phi should have same length!")
        for _ in range(extendeddim):
            beta = beta[..., None]
            phi = phi[..., None]
    elif beta.ndim != 0:
        raise ValueError("Only length 1 or scalar values are supported for beta and phi")
    else:
        for _ in range(extendeddim + 1):
            beta = beta[..., None]
            phi = phi[..., None]
    return beta, phi


# --------------------------------------------------------------------------
# optical data and layer lists (dtmm/data.py, dtmm/transfer.py)
# --------------------------------------------------------------------------
def validate_optical_block(block, shape=None):
    """(thickness (L,), eps (L,h,w,3), angles (L,h,w,3)) (dtmm/data.py:534, non-dispersive)."""
    thickness, material, angles = block
    thickness = np.asarray(thickness, FDTYPE)
    material = np.asarray(material)
    material = np.asarray(material, CDTYPE if np.iscomplexobj(material) else FDTYPE)
    angles = np.asarray(angles, FDTYPE)
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
    n = len(thickness)
    target = (n, 1, 1, 3) if shape is None else (n,) + tuple(shape) + (3,)
    np.broadcast_shapes(material.shape, target)
    np.broadcast_shapes(angles.shape, target)
    return thickness, material, angles


def validate_optical_data(data, shape=None):
    """List of validated blocks (dtmm/data.py:645)."""
    if isinstance(data, list):
        if shape is None:
            raise ValueError("For heterogeneous data, you must provide the `shape` argument.")
        return [validate_optical_block(d, shape) for d in data]
    warnings.warn("A single-block optical data must be a list of length 1.", DeprecationWarning)
    return validate_optical_data([data], shape)


def _isotropic_mean(epsv):
    """Mean of (e0+e1+e2)/3 over every voxel (``effective_block`` symmetry 0, dtmm/data.py:1364-1392;
    ``_uniaxial_order`` order 0, dtmm/data.py:1217)."""
    m = (epsv[..., 0] + epsv[..., 1] + epsv[..., 2]) / 3.0
    return np.asarray(m.mean())


_SYMMETRY_NAMES = {"isotropic": 0, "uniaxial": 1, "biaxial": 2}


def _symmetry(arg):
    """Symmetry identifier -> 0 / 1 / 2, or an array of them (dtmm/data.py:1344-1362)."""
    if isinstance(arg, str):
        if arg not in _SYMMETRY_NAMES:
            raise ValueError("Invalid symmetry argument.")
        return _SYMMETRY_NAMES[arg]
    if np.ndim(arg) == 0:
        if arg not in (0, 1, 2, -1):
            raise ValueError("Invalid symmetry argument.")
        return int(arg)
    return np.asarray([_symmetry(a) for a in arg], int)


def _cross3(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _abs2(v):
    return sum(x.real ** 2 + x.imag ** 2 for x in v)


def _eigvec0(a, e):
    """Unit eigenvector of eigenvalue e: the largest pairwise cross product of
    the rows of A - e I (dtmm/linalg.py:50-93)."""
    r0 = [a[0][0] - e, a[0][1], a[0][2]]
    r1 = [a[0][1], a[1][1] - e, a[1][2]]
    r2 = [a[0][2], a[1][2], a[2][2] - e]
    x = [_cross3(r0, r1), _cross3(r0, r2), _cross3(r1, r2)]
    d = [_abs2(v) for v in x]
    imax, dmax = 0, d[0]
    if d[1] > dmax:
        imax, dmax = 1, d[1]
    if d[2] > dmax:
        imax = 2
    v = x[imax]
    inv = 1.0 / cmath.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [c * inv for c in v]


def _eigvec1(a, w, e):
    """Eigenvector of eigenvalue e in the orthogonal complement of w
    (dtmm/linalg.py:96-164)."""
    if abs(w[0]) > abs(w[1]):
        u = [-w[2], 0.0, w[0]]
    else:
        u = [0.0, w[2], -w[1]]
    sc = 1.0 / _abs2(u) ** 0.5
    u = [c * sc for c in u]
    v = _cross3(w, u)
    mul = lambda x: [a[i][0] * x[0] + a[i][1] * x[1] + a[i][2] * x[2] for i in range(3)]
    dot = lambda x, y: x[0] * y[0] + x[1] * y[1] + x[2] * y[2]
    au, av = mul(u), mul(v)
    m00, m01, m11 = dot(u, au) - e, dot(u, av), dot(v, av) - e
    a00, a01, a11 = abs(m00), abs(m01), abs(m11)
    out = list(u)
    if a00 >= a11:
        if max(a00, a01) > 0:
            if a00 >= a01:
                m01 /= m00
                m00 = 1 / (1 + m01 ** 2) ** 0.5
                m01 *= m00
            else:
                m00 /= m01
                m01 = 1 / (1 + m00 ** 2) ** 0.5
                m00 *= m01
            out = [m01 * u[i] - m00 * v[i] for i in range(3)]
    else:
        if max(a11, a01) > 0:
            if a11 >= a01:
                m01 /= m11
                m11 = 1 / (1 + m01 ** 2) ** 0.5
                m01 *= m11
            else:
                m11 /= m01
                m01 = 1 / (1 + m11 ** 2) ** 0.5
                m11 *= m01
            out = [m11 * u[i] - m01 * v[i] for i in range(3)]
    return out


def tensor_eig(eps6, is_real=True):
    """Eigenvalues and eigenvectors (columns) of one symmetric 3x3 tensor given
    as (00, 11, 22, 01, 02, 12), the third eigenvalue the most distinct
    (dtmm/linalg.py:225-318, :364-423): Eberly's non-iterative solver
    ("A Robust Eigensolver for 3x3 Symmetric Matrices", Geometric Tools) on
    the tensor scaled by its largest entry -- eigenvalues in increasing order
    from the trigonometric form (its argument clamped for a real tensor), the
    outer eigenvalue's eigenvector from the rows' cross products, the middle
    one in its orthogonal complement, the third their cross product; diagonal
    when the scaled off-diagonal sum of squares is at most 1e-12 -- then the
    cyclic permutation that moves the most distinct eigenvalue to the third
    place (``_sort_eigvec``, dtmm/linalg.py:166-218)."""
    t = [complex(x) for x in np.asarray(eps6, CDTYPE)]
    vec = [[1.0 + 0j, 0j, 0j], [0j, 1.0 + 0j, 0j], [0j, 0j, 1.0 + 0j]]  # rows
    scale = max(abs(x) for x in t)
    if scale == 0.0:
        eig = [0j, 0j, 0j]
    else:
        sm = 1.0 / scale
        a00, a11, a22, a01, a02, a12 = [x * sm for x in t]
        a = [[a00, a01, a02], [a01, a11, a12], [a02, a12, a22]]
        q = (a00 + a11 + a22) / 3
        b00, b11, b22 = a00 - q, a11 - q, a22 - q
        norm = a01 ** 2 + a02 ** 2 + a12 ** 2
        if abs(norm) > 1e-12:
            p = ((b00 ** 2 + b11 ** 2 + b22 ** 2 + 2 * norm) / 6) ** 0.5
            c00 = b11 * b22 - a12 * a12
            c01 = a01 * b22 - a12 * a02
            c02 = a01 * a12 - b11 * a02
            half_det = (b00 * c00 - a01 * c01 + a02 * c02) / (p * p * p * 2)
            if is_real:
                half_det = complex(min(max(half_det.real, -1.0), 1.0))
            phi = cmath.acos(half_det) / 3.0
            twothirdspi = 2.09439510239319549
            e0 = cmath.cos(phi + twothirdspi) * 2
            e2 = cmath.cos(phi) * 2
            e1 = -(e0 + e2)
            e0, e1, e2 = e0 * p + q, e1 * p + q, e2 * p + q
            if half_det.real >= 0:
                vec[2] = _eigvec0(a, e2)
                vec[1] = _eigvec1(a, vec[2], e1)
                vec[0] = _cross3(vec[1], vec[2])
            else:
                vec[0] = _eigvec0(a, e0)
                vec[1] = _eigvec1(a, vec[0], e1)
                vec[2] = _cross3(vec[0], vec[1])
            eig = [e0 * scale, e1 * scale, e2 * scale]
        else:
            eig = [a00 * scale, a11 * scale, a22 * scale]
    w = np.asarray(eig, CDTYPE)
    m2, m1, m0 = abs(w[1] - w[0]), abs(w[2] - w[0]), abs(w[2] - w[1])
    i, j, k = 0, 1, 2
    if m2 > m1 or m2 > m0:
        i, j, k = (1, 2, 0) if m1 > m0 else (2, 0, 1)
    idx = [i, j, k]
    v = np.asarray(vec, CDTYPE).T  # eigenvectors as columns
    return w[idx], v[:, idx]


def rotation_angles(R):
    """Euler angles (psi, theta, phi) of a rotation matrix (dtmm/rotation.py:154-171)."""
    theta = np.arccos(max(-1.0, min(1.0, R[2, 2])))
    if (R[1, 2] == 0.0 and R[0, 2] == 0.0) or theta == 0.0:
        return np.asarray([0.0, theta, np.arccos(max(-1.0, min(1.0, R[1, 1])))], FDTYPE)
    return np.asarray([np.arctan2(R[2, 1], -R[2, 0]), theta, np.arctan2(R[1, 2], R[0, 2])], FDTYPE)


def uniaxial_order(order, eig):
    """Uniaxial (1), isotropic (0) or unchanged (< 0) eigenvalues, [2] the
    extraordinary axis (dtmm/data.py:1215-1233, :1240-1274)."""
    e0, e1, e2 = eig
    if order < 0:
        return np.asarray([e0, e1, e2], CDTYPE)
    m = (e0 + e1 + e2) / 3.0
    delta = e2 - (e0 + e1) / 2.0
    if order == 0:
        return np.asarray([m, m, m], CDTYPE)
    a = m - order * delta / 3.0
    return np.asarray([a, a, m + 2.0 * order * delta / 3.0], CDTYPE)


def effective_block(block, symmetry):
    """Effective layers of an optical block (dtmm/data.py:1364-1419): isotropic
    (0) the mean of the voxels' isotropic eigenvalue; otherwise the mean of the
    lab-frame tensors (over every voxel, or per layer when ``symmetry`` is a
    per-layer array), its eigen-frame, and the eigenvalues made uniaxial (1) or
    kept (2, biaxial); each layer gets its block's medium.  Returns per-layer
    ``(epsv, epsa)`` arrays."""
    d, epsv, epsa = block
    n = len(d)
    sym = _symmetry(symmetry)
    if np.ndim(sym) == 0 and sym == 0:
        m = _isotropic_mean(epsv)
        ev = np.asarray([m, m, m])
        ev = ev.astype(CDTYPE if np.iscomplexobj(ev) else FDTYPE)
        return [ev] * n, [np.zeros(3, FDTYPE)] * n
    shape = np.broadcast_shapes(np.shape(epsv), np.shape(epsa))
    ev_b = np.broadcast_to(np.asarray(epsv), shape)
    ea_b = np.broadcast_to(np.asarray(epsa, FDTYPE), shape)
    R = _rotation_matrix(ea_b[..., 0], ea_b[..., 1], ea_b[..., 2])
    eps = _rotate_diagonal_tensor(R, ev_b.astype(CDTYPE))
    per_layer = np.ndim(sym) != 0
    if per_layer:
        if len(sym) != n:
            raise ValueError("Shape of the symmetry argument is incompatible with block size.")
        means = [eps[i].reshape(-1, 6).mean(axis=0) for i in range(n)]
        orders = list(sym)
    else:
        means = [eps.reshape(-1, 6).mean(axis=0)]
        orders = [sym]
    evs, eas = [], []
    for t, o in zip(means, orders):
        w, v = tensor_eig(t, is_real=not np.iscomplexobj(epsv))
        eas.append(rotation_angles(v.real))
        evs.append(uniaxial_order(-1 if o > 1 else o, w))
    if not per_layer:
        evs, eas = evs * n, eas * n
    return evs, eas


def _is_effective_block(e):
    """eff_data entry given as an optical block (its eps values end in an axis
    of three); the reference tries the entry as a block first
    (dtmm/transfer.py:941-947)."""
    return (isinstance(e, tuple) and len(e) == 3 and not callable(e[1]) and np.ndim(e[1]) >= 1 and
            np.shape(e[1])[-1] == 3)


def _layers_list(block, nin, nout, nstep, is_first, is_last, eff_data=0):
    """Layer and effective-layer lists with the input/output media (dtmm/transfer.py:926);
    the effective layers of a given effective block take its thicknesses and media."""
    d, epsv, epsa = block
    substeps = np.broadcast_to(np.asarray(nstep), (len(d),))
    layers = [(int(n), (t / n, ev, ea)) for n, t, ev, ea in zip(substeps, d, epsv, epsa)]
    eps_in = refind2eps([nin] * 3)
    eps_out = refind2eps([nout] * 3)
    zero = np.zeros(3, FDTYPE)
    if is_first:
        layers.insert(0, (1, (0.0, np.broadcast_to(eps_in, epsv[0].shape), np.broadcast_to(zero, epsa[0].shape))))
    if is_last:
        layers.append((1, (0.0, np.broadcast_to(eps_out, epsv[0].shape), np.broadcast_to(zero, epsa[0].shape))))
    if _is_effective_block(eff_data):
        d_eff, ev_e, ea_e = validate_optical_block(eff_data, shape=(1, 1))
        ea_e = np.asarray(ea_e, FDTYPE)
        if ea_e.ndim == 2:
            ea_e = ea_e[:, None, None, :]
        ev_e = np.broadcast_to(ev_e, (len(d_eff), 1, 1, 3))
        ea_e = np.broadcast_to(ea_e, (len(d_eff), 1, 1, 3))
        eff = [(int(n), (t / n, ev[0, 0], ea[0, 0])) for n, t, ev, ea in zip(substeps, d_eff, ev_e, ea_e)]
    else:
        ev_eff, ea_eff = effective_block(block, eff_data)
        eff = [(int(n), (t / n, ev, ea)) for n, t, ev, ea in zip(substeps, d, ev_eff, ea_eff)]
    if is_first:
        eff.insert(0, (1, (0.0, eps_in, zero)))
    if is_last:
        eff.append((1, (0.0, eps_out, zero)))
    return layers, eff


def _create_layers(optical_data, nin, nout, nstep, eff_data=0):
    """(dtmm/transfer.py:978): one symmetry for every block, or one per block."""
    layers, eff = [], []
    nb = len(optical_data)
    if isinstance(eff_data, (str, int, np.integer)):
        per_block = [eff_data] * nb
    else:
        if len(eff_data) != nb:
            raise ValueError("Number of elements in eff_data must match length of optical_data.")
        per_block = list(eff_data)
    for i, block in enumerate(optical_data):
        l, e = _layers_list(block, nin, nout, nstep, i == 0, i == nb - 1, per_block[i])
        layers += l
        eff += e
    return layers, eff


# --------------------------------------------------------------------------
# layer propagators (dtmm/propagate_4x4.py, dtmm/propagate_2x2.py)
# --------------------------------------------------------------------------
def _transfer_ray_4x4_1(field, ks, layer, dmat1, dmat2, beta, phi, nsteps):
    """dmat1 -> ifft2 -> E.P.E^-1 -> fft2 -> dmat2, nsteps times (dtmm/propagate_4x4.py:80)."""
    d, epsv, epsa = layer
    kd = ks * d
    alpha, f = alphaf(beta, phi, epsv, epsa)
    p = phasem(alpha, kd[..., None, None])
    e = E_mat(f)
    ei = inv(e)
    for _ in range(nsteps):
        field = dotmf(dmat1, field)
        field = ifft2(field)
        field = dotmdmf(e, p, ei, field)
        field = fft2(field)
        field = dotmf(dmat2, field)
    return field


def propagate_4x4_effective_1(field, ks, layer, eff_layer, beta, phi, nsteps, diffraction, betamax):
    """(dtmm/propagate_4x4.py:376)"""
    d_eff, epsv_eff, epsa_eff = eff_layer
    shape = field.shape[-2:]
    if diffraction == 1:
        dmat1 = first_corrected_Epn_diffraction_matrix(shape, ks, beta, phi, d_eff / 2, epsv_eff, epsa_eff, betamax)
        dmat2 = second_corrected_Epn_diffraction_matrix(shape, ks, beta, phi, d_eff / 2, epsv_eff, epsa_eff, betamax)
        return _transfer_ray_4x4_1(field, ks, layer, dmat1, dmat2, beta, phi, nsteps)
    if diffraction > 1:
        try:
            bshape = beta.shape
            b0, p0 = beta[..., 0], phi[..., 0]
        except IndexError:
            bshape = ()
            b0, p0 = beta, phi
        windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), b0 * np.cos(p0), b0 * np.sin(p0), betamax)
        n = len(windows)
        betas = betas.reshape((n,) + bshape)
        phis = phis.reshape((n,) + bshape)
        dm1 = first_corrected_Epn_diffraction_matrix(shape, ks, betas, phis, d_eff / 2, epsv_eff, epsa_eff, betamax)
        dm2 = second_corrected_Epn_diffraction_matrix(shape, ks, betas, phis, d_eff / 2, epsv_eff, epsa_eff, betamax)
        fout = np.zeros_like(field)
        for w, b, p, m1, m2 in zip(windows, betas, phis, dm1, dm2):
            fout = fout + _transfer_ray_4x4_1(field * w, ks, layer, m1, m2, b, p, nsteps)
        return fout
    raise ValueError("Invalid diffraction value")


def _transfer_ray_2x2_1(fft_field, ks, layer, dmat1, dmat2, beta, phi, nsteps, mode, bulk, tmat=None, rmat=None,
                        refl=None):
    """2x2 E-only split step (dtmm/propagate_2x2.py:19-87).  ``tmat`` is the
    interface transmission applied before the first step when reflections
    are on.  With tracked reflected waves (``refl``, npass > 1) the interface
    also stores ``rmat`` times the incoming field in ``refl`` and adds the
    wave stored there before; going backward (mode -1) the field past the
    interface is added to ``bulk`` (E and H parts).  Returns the field, and
    ``refl`` when it is tracked."""
    d, epsv, epsa = layer
    alpha, fmat = alphaf(beta, phi, epsv, epsa)
    if tmat is not None:
        if refl is not None:
            trans = refl.copy()
            refl[...] = dotmf(rmat, fft_field)
            fft_field = dotmf(tmat, fft_field) + trans
            if mode == -1 and bulk is not None:
                field = ifft2(fft_field)
                e2h = E2H_mat(fmat, mode=mode)
                bulk[..., ::2, :, :] += field
                bulk[..., 1::2, :, :] += dotmf(e2h, field)
        else:
            fft_field = dotmf(tmat, fft_field)
    e = E_mat(fmat, mode=mode)
    ei = inv(e)
    p = phase_mat(alpha, (ks * d)[..., None, None], mode=mode)
    for _ in range(nsteps):
        if dmat1 is not None:
            fft_field = dotmf(dmat1, fft_field)
        field = ifft2(fft_field)
        field = dotmdmf(e, p, ei, field)
        fft_field = fft2(field)
        if dmat2 is not None:
            fft_field = dotmf(dmat2, fft_field)
    if mode == +1 and bulk is not None:
        field = ifft2(fft_field)
        e2h = E2H_mat(fmat, mode=mode)
        bulk[..., 1::2, :, :] += dotmf(e2h, field)
        bulk[..., ::2, :, :] += field
    return fft_field


def _transfer_ray_2x2_2(field, ks, in_layer, out_layer, dmat, beta, phi, nsteps, mode, reflection, refl, bulk):
    """2x2 reflection mode 2 on the real-space E field (dtmm/propagate_2x2.py:91-190):
    per step E . P(d/2) . E^-1 halves around the corrected E matrix; at the
    first step the per-voxel interface from the input layer (transmission
    and reflection with tracked waves, or the inverse E matrix through the
    interface without them).  Returns the field and the reflected wave."""
    if in_layer is not None:
        _, epsv_in, epsa_in = in_layer
        _, fmat_in = alphaf(beta, phi, epsv_in, epsa_in)
    d, epsv, epsa = out_layer
    alpha, fmat = alphaf(beta, phi, epsv, epsa)
    e = E_mat(fmat, mode=mode)
    kd = ks * d / 2
    p = phase_mat(alpha, kd[..., None, None], mode=mode)
    ei0 = inv(e)
    ei = ei0
    for j in range(nsteps):
        if j == 0 and reflection != 0:
            if refl is not None:
                tmat, rmat = tr_mat(fmat_in, fmat, mode=mode)
                trans = refl.copy()
                refl[...] = field - dotmf(tmat, field)  # in place, as the reference's out= writes
                field = dotmf(tmat, field) + trans
                if mode == -1 and bulk is not None:
                    e2h = E2H_mat(fmat, mode=mode)
                    bulk[..., ::2, :, :] += field
                    bulk[..., 1::2, :, :] += dotmf(e2h, field)
                field = dotmf(ei, field)
                if d != 0.0:
                    field = dotmf(e * p[..., None, :], field)
                else:
                    field = dotmf(e, field)
                ei = ei0
            else:
                ei = Eti_mat(fmat_in, fmat, mode=mode)
                field = dotmdmf(e, p, ei, field)
                ei = ei0
        else:
            if d != 0.0:
                field = dotmdmf(e, p, ei, field)
        if dmat is not None:
            field = diffract(field, dmat)
        if d != 0.0:
            field = dotmdmf(e, p, ei, field)
    if mode == +1 and bulk is not None:
        e2h = E2H_mat(fmat, mode=mode)
        bulk[..., 1::2, :, :] += dotmf(e2h, field)
        bulk[..., ::2, :, :] += field
    return field, refl


def propagate_2x2_effective_2(field, ks, layer_in, layer_out, eff_in, eff_out, beta, phi, nsteps, diffraction,
                              reflection, betamax, mode, refl, bulk):
    """(dtmm/propagate_2x2.py:286-377, split_diffraction ignored): one corrected
    E matrix (diffraction 1), none (0), or n x n windows, each part (and its
    part of the tracked reflected wave) taken to real space and through mode 2."""
    shape = field.shape[-2:]
    d_eff, epsv_eff, epsa_eff = eff_out
    if diffraction <= 1:
        dmat = corrected_E_diffraction_matrix(shape, ks, beta, phi, d=d_eff, epsv=epsv_eff, epsa=epsa_eff, mode=mode,
                                              betamax=betamax) if diffraction else None
        return _transfer_ray_2x2_2(field, ks, layer_in, layer_out, dmat, beta, phi, nsteps, mode, reflection, refl,
                                   bulk)
    fout = 0.0
    ffield = fft2(field)
    if refl is not None:
        frefl = fft2(refl)
        new_refl = 0.0
    try:
        bshape = beta.shape
        beta = beta[..., 0]
        phi = phi[..., 0]
    except IndexError:
        bshape = ()
    windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), betax_off=beta * np.cos(phi),
                                      betay_off=beta * np.sin(phi), betamax=betamax)
    n = len(windows)
    betas = betas.reshape((n,) + bshape)
    phis = phis.reshape((n,) + bshape)
    dmats = corrected_E_diffraction_matrix(shape, ks, betas, phis, d=d_eff, epsv=epsv_eff, epsa=epsa_eff, mode=mode,
                                           betamax=betamax)
    for window, b, p, dmat in zip(windows, betas, phis, dmats):
        fpart = ifft2(ffield * window)
        rpart = None if refl is None else ifft2(frefl * window)
        out, r = _transfer_ray_2x2_2(fpart, ks, layer_in, layer_out, dmat, b, p, nsteps, mode, reflection, rpart,
                                     bulk)
        fout = fout + out
        if refl is not None and reflection != 0:
            new_refl = new_refl + r
    if refl is not None:
        refl[...] = new_refl
    return fout, refl


def propagate_2x2_effective_1(field, ks, layer_out, eff_in, eff_out, beta, phi, nsteps, diffraction, betamax, mode,
                              bulk, reflection=0, refl=None):
    """(dtmm/propagate_2x2.py:193-284, split_diffraction ignored).  ``refl``:
    the interface's tracked reflected wave (npass > 1), updated in place;
    with windows each window's part of it enters that window's transfer and
    the new reflections of the windows are summed."""
    d_out, epsv_out, epsa_out = eff_out
    shape = field.shape[-2:]
    tmat = rmat = None
    if reflection:
        tmat, rmat = E_tr_matrix(shape, ks, epsv_in=eff_in[1], epsa_in=eff_in[2], epsv_out=epsv_out,
                                 epsa_out=epsa_out, mode=mode, betamax=betamax)
    if diffraction <= 1:
        if diffraction == 1:
            dmat1 = first_E_diffraction_matrix(shape, ks, beta, phi, d_out / 2, epsv_out, epsa_out, mode, betamax)
            dmat2 = second_E_diffraction_matrix(shape, ks, beta, phi, d_out / 2, epsv_out, epsa_out, mode, betamax)
        else:
            dmat1 = dmat2 = None
        return _transfer_ray_2x2_1(field, ks, layer_out, dmat1, dmat2, beta, phi, nsteps, mode, bulk, tmat, rmat, refl)
    try:
        bshape = beta.shape
        b0, p0 = beta[..., 0], phi[..., 0]
    except IndexError:
        bshape = ()
        b0, p0 = beta, phi
    windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), b0 * np.cos(p0), b0 * np.sin(p0), betamax)
    n = len(windows)
    betas = betas.reshape((n,) + bshape)
    phis = phis.reshape((n,) + bshape)
    dm1 = first_E_diffraction_matrix(shape, ks, betas, phis, d_out / 2, epsv_out, epsa_out, mode, betamax)
    dm2 = second_E_diffraction_matrix(shape, ks, betas, phis, d_out / 2, epsv_out, epsa_out, mode, betamax)
    fout = np.zeros_like(field)
    new_refl = None if refl is None else np.zeros_like(refl)
    for w, b, p, m1, m2 in zip(windows, betas, phis, dm1, dm2):
        part = None if refl is None else refl * w
        fout = fout + _transfer_ray_2x2_1(field * w, ks, layer_out, m1, m2, b, p, nsteps, mode, bulk, tmat, rmat,
                                          part)
        if refl is not None and reflection != 0:
            new_refl = new_refl + part
    if refl is not None:
        refl[...] = new_refl
    return fout


# --------------------------------------------------------------------------
# drivers (dtmm/transfer.py)
# --------------------------------------------------------------------------
def _transfer_ray_4x4_2(field, ks, layer, beta, phi, nsteps, dmatpn=None):
    """Reflection mode 2 (dtmm/propagate_4x4.py:18-52): without diffraction
    matrices F . P . F^-1 per voxel over the layer, nsteps times; with them,
    per step E . P . F^-1 over half the layer (E the block E matrix of the
    forward and backward modes), the forward (0, 2) and backward (1, 3)
    components diffracted by their corrected E matrices, F . P . E^-1."""
    d, epsv, epsa = layer
    kd = ks * d if dmatpn is None else ks * d / 2
    alpha, f, fi = alphaffi(beta, phi, epsv, epsa)
    p = phasem(alpha, kd[..., None, None])
    if dmatpn is not None:
        dmatp, dmatn = dmatpn
        e = E_mat(f)
        ei = inv(e)
    for _ in range(nsteps):
        if dmatpn is None:
            field = dotmdmf(f, p, fi, field)
        else:
            field = dotmdmf(e, p, fi, field)
            field = np.array(field)
            field[..., 0::2, :, :] = diffract(field[..., 0::2, :, :], dmatp)
            field[..., 1::2, :, :] = diffract(field[..., 1::2, :, :], dmatn)
            field = dotmdmf(f, p, ei, field)
    return field


def propagate_4x4_effective_2(field, ks, layer, eff_layer, beta, phi, nsteps, diffraction, betamax):
    """Reflection mode 2 with diffraction (dtmm/propagate_4x4.py:156-230): one
    pair of corrected E matrices for diffraction 1; n x n mode windows
    otherwise, each part in real space through mode 2 with its window's
    beta, phi, summed."""
    d_eff, epsv_eff, epsa_eff = eff_layer
    shape = field.shape[-2:]
    if diffraction <= 1:
        dmatpn = None if diffraction == 0 else corrected_Epn_diffraction_matrix(
            shape, ks, beta, phi, d=d_eff, epsv=epsv_eff, epsa=epsa_eff, betamax=betamax)
        return _transfer_ray_4x4_2(field, ks, layer, beta, phi, nsteps, dmatpn)
    fout = np.zeros_like(field)
    field = fft2(field)
    try:
        broadcast_shape = beta.shape
        beta = beta[..., 0]
        phi = phi[..., 0]
    except IndexError:
        broadcast_shape = ()
    windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), betax_off=beta * np.cos(phi),
                                      betay_off=beta * np.sin(phi), betamax=betamax)
    n = len(windows)
    betas = betas.reshape((n,) + broadcast_shape)
    phis = phis.reshape((n,) + broadcast_shape)
    dmatps, dmatns = corrected_Epn_diffraction_matrix(shape, ks, betas, phis, d=d_eff, epsv=epsv_eff,
                                                      epsa=epsa_eff, betamax=betamax)
    for window, b, p, dmatp, dmatn in zip(windows, betas, phis, dmatps, dmatns):
        fpart = ifft2(field * window)
        fout = fout + _transfer_ray_4x4_2(fpart, ks, layer, b, p, nsteps, (dmatp, dmatn))
    return fout


def field_diffraction_matrix(shape, ks, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0), mode="b", betamax=BETAMAX):
    """Per-k F . P . F^-1 of a homogeneous layer, field basis (dtmm/diffract.py:125-136)."""
    ks = np.asarray(ks, FDTYPE)
    alpha, f, fi = diffraction_alphaffi(shape, ks, epsv=np.asarray(epsv, CDTYPE), epsa=np.asarray(epsa, FDTYPE),
                                        betamax=betamax)
    pmat = phase_matrix(alpha, ks * d, mode=mode)
    return dotmdm(f, pmat, fi)


def correction_matrix(beta, phi, ks, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0)):
    """F . P(-k d) . F^-1 of the beam's own mode (dtmm/matrix.py:17-22)."""
    alpha, f, fi = alphaffi(beta, phi, epsv, epsa)
    kd = -np.asarray(ks) * d
    pmat = phase_matrix(alpha, kd)
    return dotmdm(f, pmat, fi)


def corrected_field_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0),
                                       betamax=BETAMAX):
    """C . D . C with D the field diffraction matrix over d and C the
    correction over d / 2 (dtmm/matrix.py:86-93)."""
    dmat = field_diffraction_matrix(shape, ks, d, epsv, epsa, betamax=betamax)
    cmat = correction_matrix(beta, phi, ks, d / 2, epsv, epsa)
    dmat = dotmm(dmat, cmat)
    return dotmm(cmat, dmat)


def first_field_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0),
                                   betamax=BETAMAX):
    """D . C, both over d (dtmm/matrix.py:95-100)."""
    dmat = field_diffraction_matrix(shape, ks, d, epsv, epsa, betamax=betamax)
    cmat = correction_matrix(beta, phi, ks, d, epsv, epsa)
    return dotmm(dmat, cmat)


def second_field_diffraction_matrix(shape, ks, beta, phi, d=1.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0),
                                    betamax=BETAMAX):
    """C . D, both over d (dtmm/matrix.py:102-107)."""
    dmat = field_diffraction_matrix(shape, ks, d, epsv, epsa, betamax=betamax)
    cmat = correction_matrix(beta, phi, ks, d, epsv, epsa)
    return dotmm(cmat, dmat)


def _transfer_ray_4x4_3(field, ks, layer, dmat1, dmat2, beta, phi, nsteps):
    """Reflection mode 3 (dtmm/propagate_4x4.py:135-153): on the k-space
    field, per step dmat1, to real space, F . P . F^-1 over the layer, back,
    dmat2."""
    d, epsv, epsa = layer
    alpha, f, fi = alphaffi(beta, phi, epsv, epsa)
    p = phasem(alpha, (ks * d)[..., None, None])
    for _ in range(nsteps):
        field = dotmf(dmat1, field)
        field = ifft2(field)
        field = dotmdmf(f, p, fi, field)
        field = fft2(field)
        field = dotmf(dmat2, field)
    return field


def propagate_4x4_effective_3(field, ks, layer, eff_layer, beta, phi, nsteps, diffraction, betamax):
    """Reflection mode 3 with diffraction (dtmm/propagate_4x4.py:447-512):
    C . D and D . C over half the effective layer around the voxels, per mode
    window for diffraction > 1 (k-space field in and out)."""
    d_eff, epsv_eff, epsa_eff = eff_layer
    shape = field.shape[-2:]
    if diffraction == 1:
        dmat1 = second_field_diffraction_matrix(shape, ks, beta, phi, d_eff / 2, epsv_eff, epsa_eff, betamax=betamax)
        dmat2 = first_field_diffraction_matrix(shape, ks, beta, phi, d_eff / 2, epsv_eff, epsa_eff, betamax=betamax)
        return _transfer_ray_4x4_3(field, ks, layer, dmat1, dmat2, beta, phi, nsteps)
    if diffraction < 1:
        raise ValueError("Invalid diffraction value")
    fout = np.zeros_like(field)
    try:
        broadcast_shape = beta.shape
        beta = beta[..., 0]
        phi = phi[..., 0]
    except IndexError:
        broadcast_shape = ()
    windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), betax_off=beta * np.cos(phi),
                                      betay_off=beta * np.sin(phi), betamax=betamax)
    n = len(windows)
    betas = betas.reshape((n,) + broadcast_shape)
    phis = phis.reshape((n,) + broadcast_shape)
    dmats1 = second_field_diffraction_matrix(shape, ks, betas, phis, d_eff / 2, epsv_eff, epsa_eff, betamax=betamax)
    dmats2 = first_field_diffraction_matrix(shape, ks, betas, phis, d_eff / 2, epsv_eff, epsa_eff, betamax=betamax)
    for window, b, p, dmat1, dmat2 in zip(windows, betas, phis, dmats1, dmats2):
        fout = fout + _transfer_ray_4x4_3(field * window, ks, layer, dmat1, dmat2, b, p, nsteps)
    return fout


def _transfer_ray_4x4_4(field, ks, layer, beta, phi, nsteps, dmat):
    """Reflection mode 4 (dtmm/propagate_4x4.py:55-77): F . P . F^-1 over half
    the layer, the corrected field diffraction matrix, F . P . F^-1 again;
    without a matrix the whole layer at once."""
    d, epsv, epsa = layer
    kd = ks * d if dmat is None else ks * d / 2
    alpha, f, fi = alphaffi(beta, phi, epsv, epsa)
    p = phasem(alpha, kd[..., None, None])
    for _ in range(nsteps):
        field = dotmdmf(f, p, fi, field)
        if dmat is not None:
            field = diffract(field, dmat)
            field = dotmdmf(f, p, fi, field)
    return field


def propagate_4x4_effective_4(field, ks, layer, eff_layer, beta, phi, nsteps, diffraction, betamax):
    """Reflection mode 4 with diffraction (dtmm/propagate_4x4.py:233-287): one
    corrected matrix for diffraction 1; n x n mode windows otherwise, each
    part taken to real space and sent through mode 4 with its window's beta,
    phi (whose matrices are built with the default betamax, as there)."""
    d_eff, epsv_eff, epsa_eff = eff_layer
    shape = field.shape[-2:]
    if diffraction <= 1:
        dmat = None if diffraction == 0 else corrected_field_diffraction_matrix(
            shape, ks, beta, phi, d_eff, epsv_eff, epsa_eff, betamax=betamax)
        return _transfer_ray_4x4_4(field, ks, layer, beta, phi, nsteps, dmat)
    fout = np.zeros_like(field)
    field = fft2(field)
    try:
        broadcast_shape = beta.shape
        beta = beta[..., 0]
        phi = phi[..., 0]
    except IndexError:
        broadcast_shape = ()
    windows, (betas, phis) = fft_mask(field.shape, ks, int(diffraction), betax_off=beta * np.cos(phi),
                                      betay_off=beta * np.sin(phi), betamax=betamax)
    n = len(windows)
    betas = betas.reshape((n,) + broadcast_shape)
    phis = phis.reshape((n,) + broadcast_shape)
    dmats = corrected_field_diffraction_matrix(shape, ks, betas, phis, d_eff, epsv_eff, epsa_eff)
    for window, b, p, dmat in zip(windows, betas, phis, dmats):
        fpart = ifft2(field * window)
        fout = fout + _transfer_ray_4x4_4(fpart, ks, layer, b, p, nsteps, dmat)
    return fout


def propagate_4x4_full(field, ks, layer, nsteps, betamax):
    """diffraction = inf (dtmm/propagate_4x4.py:515-560): per wavelength the
    field's FFT amplitudes of every eigenwave with beta < betamax, taken in
    order of increasing beta, each as a plane wave through the voxels'
    F . P . F^-1 for that wave's (beta, phi), summed in real space.  The
    layer's thickness is already the sub-step d / nstep and is divided by
    nsteps again here, as the reference does."""
    shape = field.shape[-2:]
    d, epsv, epsa = layer
    kd = ks * d / nsteps
    out = np.empty_like(field)
    ii, jj = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    yy, xx = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    for _ in range(nsteps):
        for i in range(len(ks)):
            ffield = fft2(field[..., i, :, :, :])
            ofield = np.zeros_like(out[..., i, :, :, :])
            b, p = betaphi(shape, ks[i])
            mask = b < betamax
            amplitude = ffield[..., mask]
            order = sorted(zip(range(int(mask.sum())), b[mask], p[mask], ii[mask], jj[mask]), key=lambda e: e[1])
            for j, beta_, phi_, ie, je in order:
                alpha, f, fi = alphaffi(beta_, phi_, epsv, epsa)
                pm = phasem(alpha, kd[i])
                wave = np.exp(2j * np.pi * ((ie * yy % shape[0]) / shape[0] + (je * xx % shape[1]) / shape[1]))
                w = amplitude[..., j][..., None, None] * (wave / (shape[0] * shape[1]))
                ofield = ofield + dotmdmf(f, pm, fi, w)
            out[..., i, :, :, :] = ofield
        field = out.copy()
    return field


def Etri_mat(fmatin, fmatout, mode=+1):
    """Inverse E matrix through an interface with reflections and its reflected
    part (dtmm/tmm.py:1025-1048)."""
    A = E_mat(fmatin, mode=mode)
    St, Sr = S_mat(fmatin, fmatout, mode=mode)
    ei = dotmm(inv(St), inv(A))
    return ei, dotmm(Sr, ei)


def propagate_2x2_full(field, ks, layer, input_layer, nsteps, mode, reflection, betamax, refl, bulk):
    """2x2 with diffraction = inf (dtmm/propagate_2x2.py:379-464): per
    wavelength every in-band eigenwave of the E field (in order of increasing
    beta) through the voxels' E . P . E^-1 for its own (beta, phi); with
    reflections the first step passes the interface (Eti, or Etri with the
    tracked wave, whose reflected part is summed into refl); the summed waves
    (and their H parts) also added to bulk."""
    shape = field.shape[-2:]
    d, epsv, epsa = layer
    _, epsv_in, epsa_in = input_layer
    kd = ks * d / nsteps
    out = np.empty_like(field)
    ii, jj = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    yy, xx = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    npix = shape[0] * shape[1]
    for step in range(nsteps):
        for i in range(len(ks)):
            ffield = fft2(field[..., i, :, :, :])
            ofield = np.zeros_like(out[..., i, :, :, :])
            b, p = betaphi(shape, ks[i])
            mask = b < betamax
            amplitude = ffield[..., mask]
            if refl is not None:
                tampl = fft2(refl[..., i, :, :, :])[..., mask]
                orefl = refl[..., i, :, :, :]
                orefl[...] = 0.0
            order = sorted(zip(range(int(mask.sum())), b[mask], p[mask], ii[mask], jj[mask]), key=lambda e: e[1])
            for j, beta_, phi_, ie, je in order:
                alpha, fmat_out = alphaf(beta_, phi_, epsv, epsa)
                e = E_mat(fmat_out, mode=mode)
                ei0 = inv(e)
                pm = phase_mat(alpha, kd[i], mode=mode)
                wave = np.exp(2j * np.pi * ((ie * yy % shape[0]) / shape[0] + (je * xx % shape[1]) / shape[1])) / npix
                w = amplitude[..., j][..., None, None] * wave
                if step == 0 and reflection:
                    _, fmat_in = alphaf(beta_, phi_, epsv_in, epsa_in)
                    if refl is not None:
                        ei, eri = Etri_mat(fmat_in, fmat_out, mode=mode)
                        ein = E_mat(fmat_in, mode=-mode)
                        t = tampl[..., j][..., None, None] * wave
                        orefl += dotmf(ein, dotmf(eri, w))
                        w = dotmf(ei0, t) + dotmf(ei, w)
                    else:
                        w = dotmf(Eti_mat(fmat_in, fmat_out, mode=mode), w)
                    w = dotmf(e * pm[..., None, :], w)
                else:
                    w = dotmdmf(e, pm, ei0, w)
                ofield = ofield + w
                if bulk is not None:
                    obulk = bulk[..., i, :, :, :]
                    obulk[..., 1::2, :, :] += dotmf(E2H_mat(fmat_out, mode=mode), w)
                    obulk[..., ::2, :, :] += w
            out[..., i, :, :, :] = ofield
        field = out
    return out, refl


def transfer_4x4(field_data, optical_data, beta, phi, nin, nout, npass, nstep, diffraction,
                 reflection, multiray, norm, smooth, betamax, ret_bulk, out, eff_data=0):
    """4x4 pass x layer sweep (dtmm/transfer.py:618-884): reflection mode 1 in
    k-space, reflection mode 2 without diffraction (the per-voxel 4x4
    transfer) and diffraction = inf (every eigenwave exactly, any reflection
    mode) in real space."""
    if reflection not in (1, 2, 3, 4):
        raise ValueError("Invalid reflection. The 4x4 method is either reflection mode 1 or 2.")
    full = diffraction == np.inf
    if smooth < 0:
        smooth = 0.0
    if norm not in (0, DTMM_NORM_FFT, DTMM_NORM_REF, DTMM_NORM_FFT | DTMM_NORM_REF):
        raise ValueError("norm must be a combination of DTMM_NORM_FFT and DTMM_NORM_REF")
    # with DTMM_NORM_REF a 2x2 reference field goes through the forward passes
    # beside the transfer and sets the intensities of the normalisation
    # (dtmm/transfer.py:637-645, :710-713, :770-806, :824-834, :868-869)
    calc_reference = bool(norm & DTMM_NORM_REF)
    field_in, wavelengths, pixelsize = field_data
    shape = field_in.shape[-2:]
    layers, eff_layers = _create_layers(optical_data, nin, nout, nstep, eff_data)
    ks = k0(wavelengths, pixelsize)
    n = len(layers)
    if beta is None and phi is None:
        beta, phi = field2betaphi(field_in, ks, multiray)
    beta, phi = _validate_betaphi(beta, phi, extendeddim=field_in.ndim - 2)
    if out is None:
        if ret_bulk:
            bulk_out = np.zeros((n,) + field_in.shape, CDTYPE)
            bulk_out[0] = field_in
            field_in = bulk_out[0]
            field_out = bulk_out[-1]
        else:
            bulk_out = None
            field_out = np.zeros_like(field_in)
    else:
        if ret_bulk:
            bulk_out = out
            bulk_out[0] = field_in
            field_in = bulk_out[0]
            field_out = bulk_out[-1]
        else:
            bulk_out = None
            field_out = out
        field_out[...] = reflected_field(field_out, ks, n=nin, betamax=betamax)
    indices = list(range(1, n - 1))
    field0 = transmitted_field(field_in, ks, n=nin, betamax=betamax)
    field = field_in.copy()
    ref = field.copy() if calc_reference else None
    i0 = field2intensity(field0).sum(axis=(-2, -1))
    if not (0 <= diffraction <= np.inf):
        raise ValueError("Invalid diffraction value")
    work_in_fft = reflection not in (2, 4) and not full  # (dtmm/transfer.py:720-723)
    if work_in_fft:
        field = fft2(field)
    if npass > 1:
        pin_mat = projection_matrix(shape, ks, epsv=refind2eps([nin] * 3), mode=+1, betamax=betamax)
        pout_mat = projection_matrix(shape, ks, epsv=refind2eps([nout] * 3), mode=+1, betamax=betamax)
    for i in range(npass):
        direction = (-1) ** i
        for j in indices:
            nsub, (thickness, ev, ea) = layers[j]
            _, (de, ee, ae) = eff_layers[j]
            if calc_reference and i % 2 == 0:
                # the reference field's E part through the layer: 2x2 mode 2
                # without reflections (the input layer only matters with them)
                ref[..., ::2, :, :] = propagate_2x2_effective_2(
                    ref[..., ::2, :, :], ks, layers[j - 1][1], (thickness * direction, ev, ea), None,
                    (de * direction, ee, ae), beta, phi, nsub, diffraction, 0, betamax, direction, None, None)[0]
            if full:
                field = propagate_4x4_full(field, ks, (thickness * direction, ev, ea), nsub, betamax)
            elif reflection == 3:
                field = propagate_4x4_effective_3(field, ks, (thickness * direction, ev, ea),
                                                  (de * direction, ee, ae), beta, phi, nsub, diffraction, betamax)
            elif reflection == 4:
                field = propagate_4x4_effective_4(field, ks, (thickness * direction, ev, ea),
                                                  (de * direction, ee, ae), beta, phi, nsub, diffraction, betamax)
            elif reflection == 2:
                field = propagate_4x4_effective_2(field, ks, (thickness * direction, ev, ea),
                                                  (de * direction, ee, ae), beta, phi, nsub, diffraction, betamax)
            else:
                field = propagate_4x4_effective_1(field, ks, (thickness * direction, ev, ea),
                                                  (de * direction, ee, ae), beta, phi, nsub, diffraction, betamax)
            if bulk_out is not None:
                bulk_out[j] = field
        if ref is not None:
            ref[..., 1::2, :, :] = jones2H(ref[..., ::2, :, :], ks, n=nout, betamax=betamax)
        indices.reverse()
        if work_in_fft:
            field = ifft2(field)
        if npass > 1:
            if i % 2 == 0:
                if i == 0:
                    field = field - field_out
                if i != npass - 1:
                    sigma = smooth * (npass - i) / npass
                    if ref is not None:
                        ref = ref * (nin / nout) ** 0.5
                    if norm & DTMM_NORM_FFT:
                        field = project_normalized_fft(field, pout_mat, ref=ref)
                    elif calc_reference:
                        field = project_normalized_local(field, pout_mat, nout, ref=ref)
                    else:
                        field = project_normalized_total(field, pout_mat)
                    field = denoise_field(field, ks, nin, sigma)
                field_out[...] = field_out + field
                field = field_out.copy()
            else:
                field_in[...] = field
                if i != npass - 1:
                    sigma = smooth * (npass - i) / npass
                    ff = dotmf(pin_mat, fft2(field))
                    ff = denoise_fftfield(ff, ks, nin, sigma)
                    field = ifft2(ff)
                    i0f = total_intensity(field)
                    fact = (i0 / i0f)[..., None, None, None]
                    field = field * fact
                    field_out[...] = field_out * fact
                    field_in[...] = field_in * fact
                    field = field0 - field
                    field_in[...] = field_in + field
                    if calc_reference:
                        ref = field.copy()
            if work_in_fft:
                field = fft2(field)
        else:
            field_out[...] = field
    if ret_bulk:
        if work_in_fft:
            bulk_out[1:-1] = ifft2(bulk_out[1:-1])
        return bulk_out, wavelengths, pixelsize
    return field_out, wavelengths, pixelsize


def transfer_2x2(field_data, optical_data, beta, phi, nin, nout, npass, nstep, diffraction,
                 reflection, multiray, betamax, ret_bulk, out, eff_data=0):
    """2x2 interface sweep (dtmm/transfer.py:1009-1183): in k-space for
    reflection 0 / 1 with 0 < diffraction < inf and for reflection 1, in real
    space otherwise (reflection 2, or diffraction 0); npass passes alternating
    in direction, the reflected wave of every interface kept between passes
    (npass > 1); backward passes add the field leaving the stack into the
    input field."""
    if reflection not in (0, 1, 2):
        raise ValueError("Invalid reflection. The 2x2 method supports reflection mode 0,1 or 2.")
    if npass > 1 and reflection == 0:
        raise ValueError("Reflection mode `0` not compatible with npass > 1")
    field_in, wavelengths, pixelsize = field_data
    layers, eff_layers = _create_layers(optical_data, nin, nout, nstep, eff_data)
    ks = k0(wavelengths, pixelsize)
    n = len(layers) - 1
    if beta is None and phi is None:
        beta, phi = field2betaphi(field_in, ks, multiray)
    beta, phi = _validate_betaphi(beta, phi, extendeddim=field_in.ndim - 2)
    # with ret_bulk the input and output are the first and last slabs of the
    # bulk, every interface's output layer adds its field there
    # (dtmm/transfer.py:1039-1062, :1137-1146)
    bulk_out = None
    if out is None:
        if ret_bulk:
            bulk_out = np.zeros((n + 1,) + field_in.shape, field_in.dtype)
        else:
            field_out = np.zeros_like(field_in)
    else:
        out[...] = 0.0
        if ret_bulk:
            bulk_out = out
        else:
            field_out = out
    if bulk_out is not None:
        bulk_out[0] = field_in
        field_in = bulk_out[0]
        field_out = bulk_out[-1]
    if not (0 <= diffraction <= np.inf):
        raise ValueError("Invalid diffraction value")
    if diffraction == np.inf and reflection == 1:
        # the reference transforms the field to k-space for reflection 1 and its
        # modal step transforms it again (dtmm/transfer.py:1091-1098)
        raise NotImplementedError("oracle covers 2x2 diffraction = inf with reflection 0 or 2")
    if diffraction > 0:
        field0 = transmitted_field(field_in, ks, n=nin, betamax=betamax)
    else:
        field0 = transmitted_field_direct(field_in, beta, phi, n=nin)
    field = field0[..., ::2, :, :].copy()
    refl = None
    if npass > 1:
        field_in[...] = field0
        refl = np.zeros((n + 1,) + field.shape[:-3] + (2,) + field.shape[-2:], CDTYPE)
    work_in_fft = (reflection in (0, 1) and 0 < diffraction < np.inf) or reflection == 1
    if work_in_fft:
        field = fft2(field)
    indices = list(range(n))
    for i in range(npass):
        if i > 0:
            field = np.zeros_like(field)
        direction = (-1) ** i
        for j in indices:
            jin = j + (1 - direction) // 2
            jout = j + (1 + direction) // 2
            nsub, (thickness, ev, ea) = layers[jout]
            _, (di, ei_, ai) = eff_layers[jin]
            _, (de, ee, ae) = eff_layers[jout]
            if jout == 0:
                bulk = field_in
            elif jout == n:
                bulk = field_out
            else:
                bulk = None if bulk_out is None else bulk_out[jout]
            r = None if refl is None else refl[j]
            if diffraction == np.inf:
                _, (tin, evin, eain) = layers[jin]
                field, _ = propagate_2x2_full(field, ks, (thickness * direction, ev, ea), (tin, evin, eain), 1,
                                              direction, reflection, betamax, r, bulk)
            elif work_in_fft:
                field = propagate_2x2_effective_1(field, ks, (thickness * direction, ev, ea),
                                                  (di * direction, ei_, ai), (de * direction, ee, ae), beta, phi,
                                                  nsub, diffraction, betamax, direction, bulk, reflection, r)
            else:
                _, (tin, evin, eain) = layers[jin]
                field, _ = propagate_2x2_effective_2(field, ks, (tin, evin, eain), (thickness * direction, ev, ea),
                                                     (di * direction, ei_, ai), (de * direction, ee, ae), beta, phi,
                                                     nsub, diffraction, reflection, betamax, direction, r, bulk)
        indices.reverse()
    if bulk_out is not None:
        return bulk_out, wavelengths, pixelsize
    return field_out, wavelengths, pixelsize


def transfer_field(field_data, optical_data, beta=None, phi=None, nin=None, nout=None, npass=None, nstep=1,
                   diffraction=None, reflection=None, method=None, multiray=False, norm=DTMM_NORM_FFT,
                   betamax=None, smooth=SMOOTH, split_rays=False, split_diffraction=False,
                   split_wavelengths=False, split_layers=False, eff_data=None, ret_bulk=False, out=None):
    """Restates ``transfer_field`` (dtmm/transfer.py:322-552) for the covered options."""
    opt = lambda name, v: DEFAULTS[name] if v is None else v
    nin, nout = opt("nin", nin), opt("nout", nout)
    method, npass = opt("method", method), opt("npass", npass)
    eff_data = opt("eff_data", eff_data)
    diffraction, reflection = opt("diffraction", diffraction), opt("reflection", reflection)
    betamax = opt("betamax", betamax)
    if split_rays:
        raise NotImplementedError("oracle covers unsplit rays")
    if split_wavelengths and not isinstance(field_data[0], tuple) and not ret_bulk:
        # one transfer per wavelength with dispersive eps evaluated at it
        # (dtmm/transfer.py:497-528, dtmm/data.py:575-586); each slice is a view,
        # so the npass > 1 rewrite reaches the caller's field_in
        field_in, wavelengths, pixelsize = field_data
        out_field = np.empty_like(field_in) if out is None else out
        for i, w in enumerate(np.asarray(wavelengths)):
            od = [(d, e(w) if callable(e) else e, a) for d, e, a in optical_data]
            r = transfer_field((field_in[..., i:i + 1, :, :, :], np.asarray([w]), pixelsize), od, beta, phi, nin,
                               nout, npass, nstep, diffraction, reflection, method, multiray, norm, betamax, smooth,
                               False, split_diffraction, False, False, eff_data, False, None)
            out_field[..., i, :, :, :] = r[0][..., 0, :, :, :]
        return out_field, wavelengths, pixelsize
    if method == "4x4" and npass > 1 and diffraction == False:  # noqa: E712
        warnings.warn("The 4x4 method with diffraction disabled is not yet supported for input fields with beta >0.")
    if npass == -1 or npass == np.inf:
        raise NotImplementedError("oracle covers finite npass")
    if reflection is None:
        reflection = 0 if method == "2x2" else 1
        if method == "4x4" and diffraction == 0:
            reflection = 2
        if npass > 1:
            reflection = 1
            if diffraction > 1 and method == "2x2":
                reflection = 2
    field_in, wavelengths, pixelsize = field_data
    od = validate_optical_data(optical_data, shape=field_in.shape[-2:])
    if split_layers:
        # one block (and effective medium) per layer (dtmm/transfer.py:531-533, dtmm/data.py:1516-1528)
        od = [(d[i:i + 1], ev[i:i + 1] if ev.shape[0] > 1 else ev, ea[i:i + 1] if ea.shape[0] > 1 else ea)
              for d, ev, ea in od for i in range(len(d))]
    if method == "4x4":
        return transfer_4x4((field_in, wavelengths, pixelsize), od, beta, phi, nin, nout, npass, nstep,
                            diffraction, reflection, multiray, norm, smooth, betamax, ret_bulk, out, eff_data)
    return transfer_2x2((field_in, wavelengths, pixelsize), od, beta, phi, nin, nout, npass, nstep,
                        diffraction, reflection, multiray, betamax, ret_bulk, out, eff_data)


# ---------------------------------------------------------------------------
# POM image formation (the consumer of transfer_field's output)
# ---------------------------------------------------------------------------
def rotation_matrix2(angle):
    """2D rotation matrix [[c, -s], [s, c]] (dtmm/rotation.py:64-76)."""
    angle = np.asarray(angle, FDTYPE)
    c, s = np.cos(angle), np.sin(angle)
    out = np.empty(c.shape + (2, 2), FDTYPE)
    out[..., 0, 0] = c
    out[..., 1, 1] = c
    out[..., 0, 1] = -s
    out[..., 1, 0] = s
    return out


def jonesvec(pol, phi=0.0):
    """Normalised jones vector, viewed in a frame rotated by phi (dtmm/jones.py:55-102)."""
    pol = np.asarray(pol, CDTYPE)
    norm = (pol[..., 0] * pol[..., 0].conj() + pol[..., 1] * pol[..., 1].conj()) ** 0.5
    pol = np.asarray(pol / norm[..., None], CDTYPE)
    r = rotation_matrix2(-np.asarray(phi))
    return np.einsum("...ij,...j->...i", r, pol)


def polarizer(jones):
    """Jones polarizer matrix |j><j| (dtmm/jones.py:236-275)."""
    jones = np.asarray(jones)
    c, s = jones[..., 0], jones[..., 1]
    out = np.empty(jones.shape + (2,), CDTYPE)
    out[..., 0, 0] = c * c.conj()
    out[..., 0, 1] = c * s.conj()
    out[..., 1, 0] = s * c.conj()
    out[..., 1, 1] = s * s.conj()
    return out


def rotated_matrix(jmat, phi):
    """R^T . jmat . R with R = rotation_matrix2(phi) (dtmm/jones.py:346-369)."""
    r = np.asarray(rotation_matrix2(phi), CDTYPE)
    rT = np.swapaxes(r, -1, -2)
    return np.einsum("...ij,...jk,...kl->...il", rT, np.asarray(jmat), r)


def as4x4(jmat):
    """Jones 2x2 -> eigenfield 4x4: jmat on forward modes, conj(jmat) on backward (dtmm/jones.py:371-398)."""
    jmat = np.asarray(jmat)
    out = np.zeros(jmat.shape[:-2] + (4, 4), jmat.dtype)
    out[..., 0::2, 0::2] = jmat
    out[..., 1::2, 1::2] = np.conj(jmat)
    return out


def normalize_f(fmat):
    """Scale the columns of a field matrix to unit |Poynting| (dtmm/tmm.py:701-724)."""
    fmat = np.asarray(fmat, CDTYPE)
    p = np.abs((fmat[..., 0, :].real * fmat[..., 1, :].real + fmat[..., 0, :].imag * fmat[..., 1, :].imag)
               - (fmat[..., 2, :].real * fmat[..., 3, :].real + fmat[..., 2, :].imag * fmat[..., 3, :].imag)) ** 0.5
    n = np.where(p == 0.0, 0.0, 1.0 / np.where(p == 0.0, 1.0, p))
    return fmat * n[..., None, :]


def jonesmat4x4(jmat, fmat):
    """F . as4x4(jmat) . F^-1 with F column-normalised (dtmm/jones4.py:75-104)."""
    fmat = normalize_f(fmat)
    return dotmm(fmat, dotmm(as4x4(jmat), inv(fmat)))


def ray_jonesmat4x4(jmat, beta=0.0, phi=0.0, epsv=(1.0, 1.0, 1.0), epsa=(0.0, 0.0, 0.0)):
    """Jones matrix as a 4x4 field matrix in the laboratory frame (dtmm/jones4.py:205-240)."""
    alpha, f = alphaf(beta, phi, np.asarray(epsv, CDTYPE), np.asarray(epsa, FDTYPE))
    return jonesmat4x4(rotated_matrix(jmat, phi), f)


def calculate_pom_field(field, jvec=None, pmat=None, dmat=None, window=None):
    """Polarizer, refocus, analyzer on a transferred field, real-space path
    (dtmm/field_viewer.py:70-143 with input_fft = output_fft = False):
    combine the x / y input polarisations with the polarizer jones vector,
    diffract (dtmm/diffract.py:254-299: fft2, optional per-k matrix, ifft2,
    optional window), then apply the analyzer matrix per pixel."""
    field = np.asarray(field)
    if jvec is not None:
        if field.shape[-5] != 2:
            raise ValueError("Invalid field shape.")
        c, s = jvec
        field = field[..., 0, :, :, :, :] * c + field[..., 1, :, :, :, :] * s
    f = fft2(field)
    if dmat is not None:
        f = dotmf(dmat, f)
    out = ifft2(f)
    if window is not None:
        out = out * window
    if pmat is not None:
        # one matrix for every pixel: dotmf broadcasts it over the grid (broadcast_m, dtmm/linalg.py:967-991)
        out = np.einsum("...ij,...jhw->...ihw", np.asarray(pmat, CDTYPE), out)
    return out


def field2specter(field):
    """Normal Poynting component per pixel and wavelength: [..., λ, 4, H, W] ->
    [..., H, W, λ] (dtmm/field.py:784-808, :824-843)."""
    f = np.asarray(field)
    s = (f[..., 0, :, :].real * f[..., 1, :, :].real + f[..., 0, :, :].imag * f[..., 1, :, :].imag) - (
        f[..., 2, :, :].real * f[..., 3, :, :].real + f[..., 2, :, :].imag * f[..., 3, :, :].imag)
    return np.moveaxis(s, -3, -1)


def field2spectersum(field):
    """field2specter summed over the leading axis (dtmm/field.py:810-822, :845-847)."""
    return field2specter(field).sum(axis=-4)


XYZ2RGBD65 = np.array([[3.2404542, -1.5371385, -0.4985314],
                       [-0.9692660, 1.8760108, 0.0415560],
                       [0.0556434, -0.2040259, 1.0572252]])


def spec2xyz(spec, cmf):
    """sum_i cmf[i, j] spec[i] (dtmm/color.py:112-131)."""
    return np.einsum("...i,ij->...j", np.asarray(spec, FDTYPE), np.asarray(cmf, FDTYPE))


def xyz2srgb(xyz):
    """Linear sRGB (D65 white) from XYZ (dtmm/color.py:87-99)."""
    return np.einsum("kj,...j->...k", XYZ2RGBD65, xyz)


def xyz2gray(xyz):
    """(Y, Y, Y) (dtmm/color.py:101-110)."""
    y = xyz[..., 1]
    return np.stack([y, y, y], axis=-1)


def apply_srgb_gamma(v):
    """sRGB transfer curve with clipping to [0, 1] (dtmm/color.py:70-85)."""
    v = np.asarray(v, FDTYPE)
    lin = np.where(v < 0.0, 0.0, 12.92 * v)
    pw = np.where(v > 1.0, 1.0, (1 + 0.055) * np.maximum(v, 0.0) ** (1 / 2.4) - 0.055)
    return np.where(v < 0.0031308, lin, pw)


def apply_gamma(v, gamma):
    """Power-law transfer curve with clipping to [0, 1] (dtmm/color.py:52-68)."""
    v = np.asarray(v, FDTYPE)
    return np.where(v > 1.0, 1.0, np.where(v < 0, 0.0, np.maximum(v, 0.0) ** (1.0 / gamma)))


def specter2color(spec, cmf, norm=False, gamma=True, gray=False):
    """Specter -> XYZ -> (normalise) -> sRGB or gray -> transfer curve (dtmm/color.py:133-224)."""
    cmf = np.asarray(cmf)
    if cmf.shape[-1] != 3:
        raise ValueError("Grayscale cmf! Cannot convert to color.")
    out = spec2xyz(spec, cmf)
    if norm is True:
        out = out / out.max()
    elif norm != 0:
        out = out / norm
    out = xyz2gray(out) if gray else xyz2srgb(out)
    if gamma is True:
        out = apply_srgb_gamma(out)
    elif gamma is not False:
        out = apply_gamma(out, gamma)
    return out


# ---------------------------------------------------------------------------
# director -> optical data
# ---------------------------------------------------------------------------
def director2data(director, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0, thickness=None):
    """Optical block from a director field (dtmm/data.py:277-320): order
    parameter sqrt(|d|) (director2order, :963), uniaxial order of
    (no^2, no^2, ne^2) (_uniaxial_order, :1214), host eps outside the mask,
    angles (0, atan2(|d_xy|, d_z), atan2(d_y, d_x)) (director2angles, :975)."""
    d = np.asarray(director, FDTYPE)
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    order = np.sqrt(np.sqrt(x ** 2 + y ** 2 + z ** 2)) / scale_factor
    eo, ee = no ** 2, ne ** 2
    m = (eo + eo + ee) / 3.0
    delta = ee - (eo + eo) / 2.0
    e1 = np.where(order == 0.0, m, m - 1.0 / 3.0 * order * delta)
    e3 = np.where(order == 0.0, m, m + 2.0 / 3.0 * order * delta)
    epsv = np.stack([e1, e1, e3], axis=-1)
    if mask is not None:
        epsv[np.logical_not(mask), :] = nhost ** 2
    epsa = np.stack([np.zeros_like(x), np.arctan2(np.sqrt(x ** 2 + y ** 2), z), np.arctan2(y, x)], axis=-1)
    if thickness is None:
        thickness = np.ones((epsv.shape[0],))
    return thickness, epsv, epsa


# ---------------------------------------------------------------------------
# Q tensor -> optical data
# ---------------------------------------------------------------------------
def Q2eps(tensor, no=1.5, ne=1.6, scale_factor=1.0):
    """eps tensor (..., 6) from a Q tensor (..., 6): (ne^2 - no^2)/scale Q + mean eps on the diagonal
    (dtmm/data.py:432-487)."""
    q = np.asarray(tensor, FDTYPE)
    epsa = (ne ** 2 - no ** 2) / scale_factor
    epsm = (no ** 2 * 2 + ne ** 2) / 3.0
    out = np.empty_like(q)
    out[..., 0:3] = epsa * q[..., 0:3] + epsm
    out[..., 3:] = epsa * q[..., 3:]
    return out


def _cross3(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _sq3(v):
    # sum of squares in the order 0, 1, 2 (dtmm/linalg.py:14-20)
    out = 0.0
    for x in v:
        out = out + x * x
    return out


def _eigvec_first(a00, a11, a22, a01, a02, a12, ev):
    """Eigenvector of `ev`: the longest cross product of two rows of A - ev I, normalised
    (dtmm/linalg.py:44-89)."""
    r0 = [a00 - ev, a01, a02]
    r1 = [a01, a11 - ev, a12]
    r2 = [a02, a12, a22 - ev]
    c01, c12, c02 = _cross3(r0, r1), _cross3(r1, r2), _cross3(r0, r2)
    d0, d1, d2 = _sq3(c01), _sq3(c02), _sq3(c12)
    best, dmax = c01, d0
    if d1 > dmax:
        best, dmax = c02, d1
    if d2 > dmax:
        best = c12
    norm = 1.0 / (best[0] * best[0] + best[1] * best[1] + best[2] * best[2]) ** 0.5
    return [x * norm for x in best]


def _eigvec_second(a00, a11, a22, a01, a02, a12, w, ev):
    """Eigenvector of `ev` orthogonal to w: minimise in the plane orthogonal to w
    (dtmm/linalg.py:92-160)."""
    if abs(w[0]) > abs(w[1]):
        u = [-w[2], 0.0, w[0]]
    else:
        u = [0.0, w[2], -w[1]]
    scale = 1.0 / _sq3(u) ** 0.5
    u = [x * scale for x in u]
    v = _cross3(w, u)
    au = [a00 * u[0] + a01 * u[1] + a02 * u[2], a01 * u[0] + a11 * u[1] + a12 * u[2],
          a02 * u[0] + a12 * u[1] + a22 * u[2]]
    m00 = u[0] * au[0] + u[1] * au[1] + u[2] * au[2] - ev
    av = [a00 * v[0] + a01 * v[1] + a02 * v[2], a01 * v[0] + a11 * v[1] + a12 * v[2],
          a02 * v[0] + a12 * v[1] + a22 * v[2]]
    m01 = u[0] * av[0] + u[1] * av[1] + u[2] * av[2]
    m11 = v[0] * av[0] + v[1] * av[1] + v[2] * av[2] - ev
    if abs(m00) >= abs(m11):
        if max(abs(m00), abs(m01)) > 0:
            if abs(m00) >= abs(m01):
                m01 = m01 / m00
                m00 = 1.0 / (1.0 + m01 ** 2) ** 0.5
                m01 = m01 * m00
            else:
                m00 = m00 / m01
                m01 = 1.0 / (1.0 + m00 ** 2) ** 0.5
                m00 = m00 * m01
            return [m01 * u[i] - m00 * v[i] for i in range(3)]
        return u
    if max(abs(m11), abs(m01)) > 0:
        if abs(m11) >= abs(m01):
            m01 = m01 / m11
            m11 = 1.0 / (1.0 + m01 ** 2) ** 0.5
            m01 = m01 * m11
        else:
            m11 = m11 / m01
            m01 = 1.0 / (1.0 + m11 ** 2) ** 0.5
            m11 = m11 * m01
        return [m11 * u[i] - m01 * v[i] for i in range(3)]
    return u


def tensor_eig_1(t6):
    """Eigenvalues and eigenvectors (rows) of one real symmetric 3x3 tensor
    (t00, t11, t22, t01, t02, t12) by the non-iterative eigensolver of
    D. Eberly, "A Robust Eigensolver for 3x3 Symmetric Matrices" (Geometric
    Tools), as used by dtmm/linalg.py:225-300, then sorted so that the third
    eigenvalue is the most distinct, by a cyclic permutation (dtmm/linalg.py:171-218)."""
    t00, t11, t22, t01, t02, t12 = (float(x) for x in t6)
    scale = max(max(abs(t00), abs(t11)), max(abs(t22), abs(t01)), max(abs(t02), abs(t12)))
    vec = np.eye(3)
    if scale == 0.0:
        eig = np.zeros(3)
    else:
        s = 1.0 / scale
        a00, a11, a22, a01, a02, a12 = t00 * s, t11 * s, t22 * s, t01 * s, t02 * s, t12 * s
        q = (a00 + a11 + a22) / 3
        b00, b11, b22 = a00 - q, a11 - q, a22 - q
        norm = a01 ** 2 + a02 ** 2 + a12 ** 2
        if abs(norm) > 1e-12:
            p = ((b00 ** 2 + b11 ** 2 + b22 ** 2 + 2 * norm) / 6) ** 0.5
            c00 = b11 * b22 - a12 * a12
            c01 = a01 * b22 - a12 * a02
            c02 = a01 * a12 - b11 * a02
            half_det = (b00 * c00 - a01 * c01 + a02 * c02) / (p * p * p * 2)
            half_det = min(max(half_det, -1.0), 1.0)
            phi = math.acos(half_det) / 3.0
            e0 = math.cos(phi + 2.09439510239319549) * 2
            e2 = math.cos(phi) * 2
            e1 = -(e0 + e2)
            e0, e1, e2 = e0 * p + q, e1 * p + q, e2 * p + q
            if half_det >= 0:
                v2 = _eigvec_first(a00, a11, a22, a01, a02, a12, e2)
                v1 = _eigvec_second(a00, a11, a22, a01, a02, a12, v2, e1)
                v0 = _cross3(v1, v2)
            else:
                v0 = _eigvec_first(a00, a11, a22, a01, a02, a12, e0)
                v1 = _eigvec_second(a00, a11, a22, a01, a02, a12, v0, e1)
                v2 = _cross3(v0, v1)
            vec = np.array([v0, v1, v2])
            eig = np.array([e0 * scale, e1 * scale, e2 * scale])
        else:
            eig = np.array([a00 * scale, a11 * scale, a22 * scale])
    m2, m1, m0 = abs(eig[1] - eig[0]), abs(eig[2] - eig[0]), abs(eig[2] - eig[1])
    i, j, k = 0, 1, 2
    if m2 > m1 or m2 > m0:
        i, j, k = (1, 2, 0) if m1 > m0 else (2, 0, 1)
    return eig[[i, j, k]], vec[[i, j, k]]


def rotation_angles_1(R):
    """Euler angles (psi, theta, phi) of a rotation matrix (dtmm/rotation.py:154-174)."""
    r22 = max(-1.0, min(1.0, R[2, 2]))
    theta = np.arccos(r22)
    if (R[1, 2] == 0.0 and R[0, 2] == 0.0) or theta == 0.0:
        psi = 0.0
        phi = np.arccos(max(-1.0, min(1.0, R[1, 1])))
    else:
        phi = np.arctan2(R[1, 2], R[0, 2])
        psi = np.arctan2(R[2, 1], -R[2, 0])
    return np.array([psi, theta, phi])


def Q2data(tensor, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0, biaxial=False, thickness=None):
    """Optical block from a Q tensor field (..., 6) (dtmm/data.py:322-371): eps tensor (Q2eps),
    its sorted eigenvalues and the Euler angles of the eigenvector matrix (eps2epsva, :489),
    the uniaxial order 1 of the eigenvalues unless biaxial, host eps outside the mask."""
    eps = Q2eps(tensor, no, ne, scale_factor)
    flat = eps.reshape(-1, 6)
    epsv = np.empty((flat.shape[0], 3))
    epsa = np.empty((flat.shape[0], 3))
    for n, t in enumerate(flat):
        ev, vec = tensor_eig_1(t)
        epsv[n] = ev
        epsa[n] = rotation_angles_1(vec.T)  # eigenvectors in columns
    epsv = epsv.reshape(eps.shape[:-1] + (3,))
    epsa = epsa.reshape(eps.shape[:-1] + (3,))
    if not biaxial:
        m = (epsv[..., 0] + epsv[..., 1] + epsv[..., 2]) / 3.0
        delta = epsv[..., 2] - (epsv[..., 0] + epsv[..., 1]) / 2.0
        e1 = m - 1.0 / 3.0 * 1 * delta
        e3 = m + 2.0 / 3.0 * 1 * delta
        epsv = np.stack([e1, e1, e3], axis=-1)
    if mask is not None:
        epsv[np.logical_not(mask), :] = nhost ** 2
    if thickness is None:
        thickness = np.ones((epsv.shape[0],))
    return thickness, epsv, epsa
