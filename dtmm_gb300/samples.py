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


def smooth_field(shape, nmodes=8, kmax=4, amplitude=0.2, seed=0):
    """(H, W) sum of ``nmodes`` random cosine modes, bounded by ``amplitude``."""
    h, w = shape
    rng = np.random.Generator(np.random.PCG64(seed))
    y, x = np.meshgrid(np.arange(h, dtype=np.float64), np.arange(w, dtype=np.float64), indexing="ij")
    out = np.zeros((h, w), np.float64)
    for _ in range(nmodes):
        while True:
            kx, ky = rng.integers(-kmax, kmax + 1, size=2)
            if kx or ky:
                break
        cx = np.round(kx * max(w, 64) / 64.0)
        cy = np.round(ky * max(h, 64) / 64.0)
        ph = rng.uniform(0.0, 2 * np.pi)
        out += np.cos(2 * np.pi * (cx * x / w + cy * y / h) + ph)
    return out * (amplitude / nmodes)


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
