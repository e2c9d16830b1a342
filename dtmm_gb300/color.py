"""Colour-matching tables for POM images (host, FP64).

``load_tcmf`` mirrors dtmm.color.load_tcmf (dtmm/color.py:257-318): a CIE
XYZ colour-matching table and an illuminant spectrum become the transmission
colour-matching function ``[n_wavelengths, 3]`` that ``pom.pom_image`` and
``pom.specter2color`` take, normalised so that unit transmission maps to
Y = 1.  At other wavelengths than the table's the spectrum is treated as
piecewise linear and the table is integrated against a triangular kernel per
wavelength (``integrate_data``, dtmm/color.py:522-577), or interpolated for
single-wavelength spectra (``interpolate_data``, :487-519).

The tables are the reference's data files (text, first column the
wavelength: ``CIE1931XYZ.dat``, ``D65.dat`` ...): ``datapath`` names their
folder; by default the folder of an installed ``dtmm`` package is used.
Arrays may be passed instead of names.  These are arrays of a few hundred
numbers, built once per wavelength set; they stay on the host.
"""
from __future__ import annotations

import os
import warnings

import numpy as np

# sRGB primaries with the D65 white point and its inverse (dtmm/color.py:41-44)
XYZ2RGBD65 = np.array([[3.2404542, -1.5371385, -0.4985314],
                       [-0.9692660, 1.8760108, 0.0415560],
                       [0.0556434, -0.2040259, 1.0572252]])
RGB2XYZ = np.linalg.inv(XYZ2RGBD65)


def _datapath(datapath):
    if datapath is not None:
        return datapath
    import importlib.util

    spec = importlib.util.find_spec("dtmm")
    if spec is None or not spec.submodule_search_locations:
        raise FileNotFoundError("no colour tables: pass datapath= (the folder of dtmm's .dat tables) or arrays")
    return list(spec.submodule_search_locations)[0]


def _table(name, suffix, datapath):
    """A named table from the data folder, else ``name`` read as a file path."""
    if not isinstance(name, str):
        return np.asarray(name, np.float64)
    if os.path.isfile(name):
        return np.loadtxt(name)
    path = os.path.join(_datapath(datapath), name + suffix)
    if not os.path.isfile(path):
        raise FileNotFoundError("colour table %r not found" % name)
    return np.loadtxt(path)


def interpolate_data(x, x0, data):
    """Linear interpolation of 1D or [n, k] ``data`` at ``x``, zero outside
    ``x0`` (dtmm/color.py:487-519)."""
    data = np.asarray(data, np.float64)
    x0 = np.asarray(x0)
    x = np.asarray(x)
    if data.ndim not in (1, 2) or x0.ndim != 1 or x.ndim != 1:
        raise ValueError("Invalid dimensions of input data.")
    if data.ndim == 1:
        return np.interp(x, x0, data, left=0.0, right=0.0)
    out = np.zeros(x.shape + data.shape[1:], data.dtype)
    for i in range(data.shape[1]):
        out[..., i] = np.interp(x, x0, data[:, i], left=0.0, right=0.0)
    return out


def _kernel_side(x, i, dx0, ndim, right):
    """One side of the integration kernel of output point i: sample points
    from x[i] towards x[i + 1] (right) or x[i - 1] (left), at the table step
    dx0 or finer, and the triangle weights falling from x[i]
    (dtmm/color.py:579-609)."""
    lo, hi = (x[i], x[i + 1]) if right else (x[i - 1], x[i])
    span = (hi - lo) / dx0
    if span < 1:
        warnings.warn("The resolution of the integrand is too low.", stacklevel=3)
    n = int(span - 1) + 1
    step = span / n
    xs = np.linspace(lo, hi, n + 1) if right else np.linspace(hi, lo, n + 1)
    ys = np.linspace(1.0, 0.0, n + 1) * step
    return xs, (ys[:, None] if ndim == 2 else ys)


def integrate_data(x, x0, data):
    """Values at ``x`` of the table (x0, data) integrated against a triangular
    kernel reaching the neighbouring x on each side; the first and last x
    use one side only (dtmm/color.py:522-577).  x0 must be evenly spaced."""
    data = np.asarray(data)
    x0 = np.asarray(x0)
    xout = np.asarray(x)
    ndim = data.ndim
    if ndim not in (1, 2) or x0.ndim != 1 or xout.ndim != 1:
        raise ValueError("Invalid dimensions of input data.")
    dxs = x0[1:] - x0[:-1]
    dx0 = dxs[0]
    if not np.all(dxs == dx0):
        raise ValueError("x0 must have equal spacings")
    n = len(xout)
    out = np.zeros((n,) + data.shape[1:], data.dtype)
    for i in range(n):
        if i == 0:
            xs, ws = _kernel_side(xout, i, dx0, ndim, True)
            val = (interpolate_data(xs, x0, data) * ws).sum(0)
        elif i == n - 1:
            xs, ws = _kernel_side(xout, i, dx0, ndim, False)
            val = (interpolate_data(xs, x0, data) * ws).sum(0)
        else:
            xs, ws = _kernel_side(xout, i, dx0, ndim, True)
            t = interpolate_data(xs, x0, data) * ws
            t[0] = t[0] / 2  # the centre sample belongs to both sides
            val = t.sum(0)
            xs, ws = _kernel_side(xout, i, dx0, ndim, False)
            t = interpolate_data(xs, x0, data) * ws
            t[0] = t[0] / 2
            val = val + t.sum(0)
        out[i, ...] = val
    return out


def srf2cmf(srf):
    """XYZ colour matching from a spectral response (Y) of a gray camera (dtmm/color.py:203-224)."""
    srf = np.asarray(srf, np.float64)
    out = np.empty(srf.shape + (3,), srf.dtype)
    out[..., 0] = RGB2XYZ[0, 0] * srf + RGB2XYZ[0, 1] * srf + RGB2XYZ[0, 2] * srf
    out[..., 1] = srf
    out[..., 2] = RGB2XYZ[2, 0] * srf + RGB2XYZ[2, 1] * srf + RGB2XYZ[2, 2] * srf
    return out


def spec2xyz(spec, cmf):
    """sum_i cmf[i, j] spec[..., i] accumulated in wavelength order (dtmm/color.py:111-131)."""
    spec = np.asarray(spec, np.float64)
    cmf = np.asarray(cmf, np.float64)
    xyz = np.zeros(spec.shape[:-1] + (cmf.shape[1],))
    for i in range(cmf.shape[0]):
        xyz = xyz + cmf[i] * spec[..., i, None]
    return xyz


def normalize_specter(spec, cmf):
    """The spectrum scaled so that its Y is 1 (dtmm/color.py:226-255)."""
    cmf = np.asarray(cmf)
    if cmf.shape[-1] != 3:
        raise ValueError("Incompatible cmf shape")
    return np.asarray(spec, np.float64) / spec2xyz(spec, cmf)[..., 1]


def cmf2tcmf(cmf, spec, norm=True):
    """Transmission CMF: the (Y-normalised) illuminant times the CMF (dtmm/color.py:320-345)."""
    cmf = np.asarray(cmf, np.float64)
    spec = np.asarray(spec, np.float64)
    if norm == 1:  # True or 1 only, as the reference's `norm == True`: norm=2 leaves the spectrum as it is
        spec = normalize_specter(spec, cmf)
    return spec[:, None] * cmf


def load_specter(wavelengths=None, illuminant="D65", retx=False, datapath=None):
    """Illuminant spectrum from a table, interpolated at ``wavelengths`` (dtmm/color.py:347-405)."""
    data = _table(illuminant, ".dat", datapath)
    if data.ndim != 2 or data.shape[-1] != 2:
        raise ValueError("Not a valid illuminant data")
    if wavelengths is not None:
        spec = np.ascontiguousarray(interpolate_data(wavelengths, data[:, 0], data[:, 1:])[:, 0])
        x = wavelengths
    else:
        x = np.ascontiguousarray(data[:, 0])
        spec = np.ascontiguousarray(data[:, 1])
    return (x, spec) if retx else spec


def load_cmf(wavelengths=None, cmf="CIE1931", retx=False, single_wavelength=False, datapath=None):
    """XYZ colour matching at ``wavelengths`` from a table (dtmm/color.py:408-485)."""
    if isinstance(cmf, str) and cmf == "FLAT":
        if wavelengths is None:
            wavelengths = np.arange(380, 781, 5)
        data = np.zeros((len(wavelengths), 3))
        data[:, 1] = 100.0
        return (wavelengths, data) if retx else data
    if isinstance(cmf, str):
        table = _table(cmf, "XYZ.dat" if cmf.startswith("CIE") else "Y.dat", datapath)
    else:
        table = np.asarray(cmf, np.float64)
    if table.shape[-1] == 4:
        x, data = np.ascontiguousarray(table[:, 0]), np.ascontiguousarray(table[:, 1:])
    elif table.shape[-1] == 2:
        x, data = np.ascontiguousarray(table[:, 0]), np.ascontiguousarray(table[:, 1])
    else:
        raise ValueError("Not a valid cmf data!")
    if wavelengths is not None:
        wavelengths = np.asarray(wavelengths, np.float64)
        if wavelengths.ndim != 1:
            raise ValueError("Wavelengths has to be 1D array")
        if len(wavelengths) == 1:
            single_wavelength = True
        if single_wavelength:
            data = interpolate_data(wavelengths, x, data)
        else:
            data = integrate_data(wavelengths, x, data)
        x = wavelengths
    if data.ndim == 1:
        data = srf2cmf(data)
    return (x, data) if retx else data


def load_tcmf(wavelengths=None, illuminant="D65", cmf="CIE1931", norm=True, retx=False, single_wavelength=False,
              datapath=None):
    """Transmission colour-matching function ``[n, 3]`` (dtmm/color.py:257-318):
    unit transmission over the illuminant's band maps to Y = 1 (``norm``
    truthy); 0 keeps the illuminant's scale.  As in the reference, the
    second normalisation that ``norm=2`` asks for is a no-op (its
    ``cmf2tcmf`` call tests ``norm == True``), so 2 behaves as 1."""
    if wavelengths is not None and len(wavelengths) == 1:
        single_wavelength = True
    if single_wavelength:
        x, c = load_cmf(wavelengths, cmf=cmf, retx=True, single_wavelength=True, datapath=datapath)
        spec = load_specter(wavelengths=x, illuminant=illuminant, datapath=datapath)
        c = cmf2tcmf(c, spec, norm=bool(norm))
    else:
        x, c = load_cmf(cmf=cmf, retx=True, datapath=datapath)
        spec = load_specter(wavelengths=x, illuminant=illuminant, datapath=datapath)
        c = cmf2tcmf(c, spec, norm=bool(norm))
        if wavelengths is not None:
            c = integrate_data(wavelengths, x, c)
            x = wavelengths
            if norm == 2:
                c = cmf2tcmf(c, [1.0] * len(wavelengths), norm=norm)
    return (x, c) if retx else c


__all__ = ["load_tcmf", "load_cmf", "load_specter", "cmf2tcmf", "normalize_specter", "spec2xyz", "srf2cmf",
           "interpolate_data", "integrate_data"]
