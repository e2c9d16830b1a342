"""Seeded synthetic optical data for the benchmark and parity workloads.

The reference publishes no dataset for ``transfer_field``; its benchmarks are
described by director fields of stated shapes.  These generators produce them
deterministically from a seed (numpy ``Generator(PCG64)``), so the same
inputs can be rebuilt on any machine.

Smooth perturbation fields are sums of ``nmodes`` cosine Fourier modes with
integer wavevectors |kx|, |ky| <= kmax per 64 pixels (``round(k * N / 64)``
whole cycles across an N-pixel axis, so the field stays periodic), random
phases, and each mode's amplitude ``amplitude / nmodes`` -- the sum is bounded
by ``amplitude``.

Angles follow the reference's Euler convention (psi, theta, phi) with theta
measured from +z (dtmm/data.py:975-989): a director tilted by ``tilt`` out of
the xy plane has theta = pi/2 - tilt.
"""
from __future__ import annotations

import numpy as np


def _smooth_modes(shape, nmodes, kmax, seed):
    h, w = shape
    rng = np.random.Generator(np.random.PCG64(seed))
    modes = []
    for _ in range(nmodes):
        while True:
            kx, ky = rng.integers(-kmax, kmax + 1, size=2)
            if kx or ky:
                break
        cx = np.round(kx * max(w, 64) / 64.0)
        cy = np.round(ky * max(h, 64) / 64.0)
        ph = rng.uniform(0.0, 2 * np.pi)
        modes.append((float(cx), float(cy), float(ph)))
    return modes


def smooth_field(shape, nmodes=8, kmax=4, amplitude=0.2, seed=0):
    """(H, W) sum of ``nmodes`` random cosine modes, bounded by ``amplitude``."""
    h, w = shape
    y, x = np.meshgrid(np.arange(h, dtype=np.float64), np.arange(w, dtype=np.float64), indexing="ij")
    out = np.zeros((h, w), np.float64)
    for cx, cy, ph in _smooth_modes(shape, nmodes, kmax, seed):
        out += np.cos(2 * np.pi * (cx * x / w + cy * y / h) + ph)
    return out * (amplitude / nmodes)


def smooth_field_device(shape, nmodes=8, kmax=4, amplitude=0.2, seed=0, device=None):
    """``smooth_field`` evaluated on the device (same modes; cosines to FP64
    rounding), every mode in one batch of tensor operations."""
    import torch

    h, w = shape
    m = np.asarray(_smooth_modes(shape, nmodes, kmax, seed), np.float64)  # (nmodes, 3): cx, cy, phase
    # per-mode phase slopes along x and y and offsets, one small upload
    coef = torch.from_numpy(np.stack([2 * np.pi * m[:, 0] / w, 2 * np.pi * m[:, 1] / h, m[:, 2]], axis=1))
    coef = coef.to(device, non_blocking=False)
    y = torch.arange(h, dtype=torch.float64, device=device)[None, :, None]
    x = torch.arange(w, dtype=torch.float64, device=device)[None, None, :]
    arg = coef[:, 0, None, None] * x + coef[:, 1, None, None] * y + coef[:, 2, None, None]
    return torch.cos(arg).sum(0) * (amplitude / nmodes)


def twisted_nematic(shape, nlayers, no=1.5, ne=1.7, twist=np.pi / 2, tilt=0.3, amplitude=0.2,
                    nmodes=8, kmax=4, thickness=1.0, seed=0):
    """Twisted nematic slab with a smooth in-plane perturbation of azimuth and tilt.

    azimuth(z, y, x) = twist * z / nlayers + d_phi(y, x)
    tilt(y, x)       = tilt + d_tilt(y, x)
    Returns one optical block ``(d (L,), epsv (L,H,W,3), epsa (L,H,W,3))``;
    epsv is a read-only broadcast view of (no^2, no^2, ne^2).
    """
    h, w = shape
    dphi = smooth_field(shape, nmodes, kmax, amplitude, seed=seed)
    dtilt = smooth_field(shape, nmodes, kmax, amplitude, seed=seed + 7919)
    z = np.arange(nlayers, dtype=np.float64)
    epsa = np.empty((nlayers, h, w, 3), np.float64)
    epsa[..., 0] = 0.0
    epsa[..., 1] = (np.pi / 2 - (tilt + dtilt))[None]
    epsa[..., 2] = twist * z[:, None, None] / nlayers + dphi[None]
    epsv = np.broadcast_to(np.asarray((no * no, no * no, ne * ne), np.float64), (nlayers, h, w, 3))
    d = np.full((nlayers,), float(thickness))
    return d, epsv, epsa


def inplane_nematic(shape, nlayers, no=1.5, ne=1.6, amplitude=np.pi / 2, nmodes=16, kmax=4,
                    thickness=1.0, seed=0):
    """Random in-plane director (tilt 0) whose azimuth is a 16-mode smooth field.

    The azimuth field is 2D (shared by all layers) plus a linear twist of
    ``amplitude`` across the depth, so that layers differ.
    """
    h, w = shape
    az = smooth_field(shape, nmodes, kmax, amplitude, seed=seed)
    z = np.arange(nlayers, dtype=np.float64)
    epsa = np.empty((nlayers, h, w, 3), np.float64)
    epsa[..., 0] = 0.0
    epsa[..., 1] = np.pi / 2
    epsa[..., 2] = az[None] + amplitude * z[:, None, None] / nlayers
    epsv = np.broadcast_to(np.asarray((no * no, no * no, ne * ne), np.float64), (nlayers, h, w, 3))
    d = np.full((nlayers,), float(thickness))
    return d, epsv, epsa


def twisted_nematic_device(shape, nlayers, no=1.5, ne=1.7, twist=np.pi / 2, tilt=0.3, amplitude=0.2,
                           nmodes=8, kmax=4, thickness=1.0, seed=0, device=None, host_modes=True):
    """``twisted_nematic`` built on the device as a ``DeviceMaterial``.

    With ``host_modes`` the (H, W) perturbation fields come from the host
    (``smooth_field``) and the (L, H, W, 3) angle array is filled on the
    device with the same operation order as the host generator, so both give
    identical values.  Without it the perturbations are evaluated on the
    device too (``smooth_field_device``): no host work that grows with the
    grid, values equal to the host ones to FP64 rounding.
    """
    import torch

    from .transfer import DeviceMaterial

    dev = device or torch.device("cuda", torch.cuda.current_device())
    h, w = shape
    epsa = torch.empty((nlayers, h, w, 3), dtype=torch.float64, device=dev)
    if host_modes:
        dphi = torch.from_numpy(smooth_field(shape, nmodes, kmax, amplitude, seed=seed)).to(dev)
        dtilt = torch.from_numpy(smooth_field(shape, nmodes, kmax, amplitude, seed=seed + 7919)).to(dev)
        z = torch.arange(nlayers, dtype=torch.float64, device=dev)
        epsa[..., 0] = 0.0
        epsa[..., 1] = (np.pi / 2 - (dtilt + tilt))[None]
        epsa[..., 2] = (z * twist / nlayers)[:, None, None] + dphi[None]
    else:
        # one kernel, the modes passed by value (dtmm_twisted_nematic_angles)
        import ctypes

        from . import _lib

        rows = []
        for sd in (seed, seed + 7919):
            m = np.asarray(_smooth_modes(shape, nmodes, kmax, sd), np.float64)
            rows.append(np.stack([2 * np.pi * m[:, 0] / w, 2 * np.pi * m[:, 1] / h, m[:, 2]], axis=1))
        modes = np.ascontiguousarray(np.concatenate(rows))
        lib = _lib.load()
        _lib.check(lib.dtmm_twisted_nematic_angles(
            int(nlayers), int(h), int(w), modes.ctypes.data_as(ctypes.c_void_p), int(nmodes),
            float(amplitude / nmodes), float(amplitude / nmodes), float(twist), float(tilt),
            ctypes.c_void_p(epsa.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    epsv = torch.empty(3, dtype=torch.float64, device=dev)  # filled on the device: no blocking upload
    epsv[:2] = no * no
    epsv[2] = ne * ne
    return DeviceMaterial(np.full((nlayers,), float(thickness)), epsv, epsa, shape,
                          eps_min=min(no * no, ne * ne), uniaxial=True)


# ---------------------------------------------------------------------------
# batch / serving workloads: many heterogeneous 4x4 instances
# ---------------------------------------------------------------------------
def _is_7smooth(n):
    for q in (2, 3, 5, 7):
        while n % q == 0:
            n //= q
    return n == 1


# grid sides the engine's transforms factor (2, 3, 5, 7), multiples of 16
FFT_SIDES = tuple(n for n in range(64, 513, 16) if _is_7smooth(n))

# seven incidence rays: beta in {0, +-0.1, +-0.2} along phi = 0, and +-0.1
# along phi = 90 degrees; a negative beta is the ray (|beta|, phi + pi)
BATCH_RAYS = ((0.0, 0.0), (0.1, 0.0), (-0.1, 0.0), (0.2, 0.0), (-0.2, 0.0), (0.1, np.pi / 2), (-0.1, np.pi / 2))


def fft_side(x, sides=FFT_SIDES):
    """The supported side nearest to ``x`` on a log scale."""
    s = np.asarray(sides, np.float64)
    return int(s[np.argmin(np.abs(np.log(s) - np.log(float(x))))])


def ray_directions(rays=BATCH_RAYS):
    """(beta, phi) arrays with negative beta mapped to (|beta|, phi + pi)."""
    b = np.asarray([r[0] for r in rays], np.float64)
    p = np.asarray([r[1] for r in rays], np.float64)
    return np.abs(b), np.where(b < 0, p + np.pi, p)


def instance_specs(n, seed=0, sides=(64, 512), layers=(20, 120), nwavelengths=(1, 9), band=(400.0, 700.0),
                   rays=BATCH_RAYS, pixelsize=100.0):
    """Seeded specs of ``n`` heterogeneous 4x4 transfers.

    Grid side log-uniform in ``sides`` (rounded to ``FFT_SIDES``), layer count
    uniform in ``layers``, wavelength count uniform in ``nwavelengths`` spread
    evenly over ``band`` (its centre for one), the given rays (``None`` for a
    single normal-incidence ray), and the twisted-nematic director of
    ``twisted_nematic`` with a per-instance seed.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi = np.log(sides[0]), np.log(sides[1])
    out = []
    for i in range(n):
        side = fft_side(np.exp(rng.uniform(lo, hi)))
        nl = int(rng.integers(layers[0], layers[1] + 1))
        nw = int(rng.integers(nwavelengths[0], nwavelengths[1] + 1))
        wl = np.linspace(band[0], band[1], nw) if nw > 1 else np.asarray([0.5 * (band[0] + band[1])])
        if rays is None:
            beta, phi = 0.0, 0.0
        else:
            beta, phi = ray_directions(rays)
        out.append(dict(index=i, shape=(side, side), nlayers=nl, wavelengths=wl, pixelsize=float(pixelsize),
                        beta=beta, phi=phi, seed=int(seed) * 100003 + i))
    return out


def spec_updates(spec, npol=2):
    """voxel x wavelength updates of one spec (one pass, all fields)."""
    nray = 1 if np.ndim(spec["beta"]) == 0 else len(spec["beta"])
    h, w = spec["shape"]
    return h * w * spec["nlayers"] * len(spec["wavelengths"]) * nray * npol


# ---------------------------------------------------------------------------
# colour matching for synthetic POM images
# ---------------------------------------------------------------------------
def _lobe(x, mu, s1, s2):
    s = np.where(x < mu, s1, s2)
    return np.exp(-0.5 * ((x - mu) / s) ** 2)


def analytic_cmf(wavelengths):
    """CIE 1931 2-degree colour matching functions (x, y, z) at ``wavelengths``
    (nm) from the multi-lobe piecewise-Gaussian fit of Wyman, Sloan and
    Shirley, "Simple Analytic Approximations to the CIE XYZ Color Matching
    Functions", JCGT 2(2), 2013."""
    x = np.asarray(wavelengths, np.float64)
    xb = 1.056 * _lobe(x, 599.8, 37.9, 31.0) + 0.362 * _lobe(x, 442.0, 16.0, 26.7) - 0.065 * _lobe(x, 501.1, 20.4, 26.2)
    yb = 0.821 * _lobe(x, 568.8, 46.9, 40.5) + 0.286 * _lobe(x, 530.9, 16.3, 31.1)
    zb = 1.217 * _lobe(x, 437.0, 11.8, 36.0) + 0.681 * _lobe(x, 459.0, 26.0, 13.8)
    return np.stack([xb, yb, zb], axis=-1)


def transmission_cmf(wavelengths):
    """Transmission colour matching function [n, 3] for an equal-energy
    illuminant sampled at ``wavelengths``: ``analytic_cmf`` weighted by each
    sample's share of the band and scaled so that unit transmission gives
    Y = 1 (the role of dtmm.color.load_tcmf for synthetic images)."""
    wl = np.asarray(wavelengths, np.float64)
    if wl.size == 1:
        w = np.ones(1)
    else:
        edges = np.concatenate([[wl[0] - 0.5 * (wl[1] - wl[0])], 0.5 * (wl[1:] + wl[:-1]),
                                [wl[-1] + 0.5 * (wl[-1] - wl[-2])]])
        w = np.diff(edges)
    cmf = analytic_cmf(wl) * w[:, None]
    return cmf / cmf[:, 1].sum()
