"""Real-space windows for input field shaping and POM images (host, FP64).

Mirrors dtmm.window (dtmm/window.py:17-153): circular / annular apertures with
a raised-cosine (Tukey) edge and the radial Blackman window, on the pixel
grid whose coordinates run from -n/2 + 1/2 to n/2 - 1/2 along each axis.
Windows are [H, W] float64 arrays; ``illumination_data(window=...)`` and
``pom.calculate_pom_field(window=...)`` take them.
"""
from __future__ import annotations

import numpy as np


def _centred_axes(shape):
    ay, ax = (np.arange(-n / 2.0 + 0.5, n / 2.0 + 0.5) for n in shape)
    return np.meshgrid(ax, ay, indexing="xy")


def _radius(shape, scale=1.0):
    """Radius normalised to the half extent of each axis times ``scale`` (dtmm/window.py:17-23)."""
    ny, nx = (n / 2 for n in shape)
    xx, yy = _centred_axes(shape)
    return ((xx / (nx * scale)) ** 2 + (yy / (ny * scale)) ** 2) ** 0.5


def tukey(r, alpha=0.1, rmax=1.0):
    """1 inside rmax - alpha rmax, a raised-cosine fall to 0 at rmax, 0 beyond (dtmm/window.py:139-151)."""
    r = np.asarray(r, np.float64)
    out = np.ones(r.shape, np.float64)
    alpha = alpha * rmax
    edge = r > rmax - alpha
    if alpha > 0.0:
        fall = 0.5 * (1 - np.cos(np.pi * (r - rmax) / alpha))
        out[edge] = fall[edge]
    out[r >= rmax] = 0.0
    return out


def aperture(shape, diameter=1.0, smooth=0.05):
    """Circular aperture of relative ``diameter`` (1: the full height / width),
    or annular for ``(inner, outer)``, with an edge of relative width
    ``smooth`` (dtmm/window.py:107-137)."""
    try:
        inner, outer = diameter
    except TypeError:
        inner, outer = 0, diameter
    a = tukey(_radius(shape, scale=outer), smooth)
    if inner == 0:
        return a
    return a * (1 - tukey(_radius(shape, scale=inner), smooth))


def blackman(shape):
    """Radial Blackman window 0.42 + 0.5 cos(pi r) + 0.08 cos(2 pi r), 0 for r >= 1 (dtmm/window.py:32-54)."""
    r = _radius(shape)
    out = 0.42 + 0.5 * np.cos(np.pi * r) + 0.08 * np.cos(2 * np.pi * r)
    out[r >= 1.0] = 0.0
    return out


def gaussian(shape, waist):
    """exp(-r^2) with r normalised by ``waist`` times the half extent (dtmm/window.py:56-74)."""
    return np.exp(-_radius(shape, waist) ** 2)


__all__ = ["aperture", "blackman", "gaussian", "tukey"]
