"""Optical data from director fields, on the GPU.

``director2data`` mirrors dtmm.data.director2data (dtmm/data.py:277-320): a
director field [L, H, W, 3] (its length is the order parameter's square)
becomes the optical block ``(thickness, epsv, epsa)`` of eps eigenvalues and
Euler angles, computed per voxel by the library's ``dtmm_director2data``
kernel.  With a CUDA tensor the block stays on the device (``device_material``
wraps it for ``plan_transfer``); with a numpy array the result comes back as
numpy, as the reference returns it.

``Q2data`` mirrors dtmm.data.Q2data (dtmm/data.py:322-371): a Q-tensor field
[L, H, W, 6] (or [..., 3, 3]) becomes the same optical block through the
per-voxel eps tensor, its eigen-decomposition and the Euler angles of the
eigenvector frame (``dtmm_q2data``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class EpsilonDispersive:
    """Eps eigenvalues as a function of the wavelength, from per-voxel
    coefficients (the reference's dispersive materials, dtmm/data.py:1124-1204).

    ``values`` has a last axis of ``n`` coefficients after the three eigenvalue
    axes: ``(..., 3, n)`` (e.g. ``(L, 3, n)`` per layer or ``(L, H, W, 3, n)``
    per voxel); without values, ``shape`` and ``n`` give coefficients that
    evaluate to eps 1.  Calling the object with a wavelength in nanometres
    returns the eps values ``(..., 3)``; ``transfer_field`` evaluates it once
    per wavelength with ``split_wavelengths=True``, as the reference requires.
    """

    def __init__(self, values=None, shape=None, n=None):
        if values is None:
            if shape is None or n is None:
                raise ValueError("Coefficients were not set, so you need to provide n and shape parameters.")
            c = np.zeros(tuple(shape) + (3, int(n)), np.float64)
            c[..., 0] = 1.0
            self.coefficients = c
        else:
            c = np.asarray(values, np.float64)
            self.coefficients = np.broadcast_to(c, np.broadcast_shapes(c.shape, (3, c.shape[-1] if c.ndim else 1)))

    def __getitem__(self, index):
        return self.__class__(self.coefficients[index])


class EpsilonCauchy(EpsilonDispersive):
    """Cauchy dispersion: n = c0 + sum_i c_i / w^(2 i), eps = n^2, w in microns."""

    def __call__(self, wavelength):
        w = float(wavelength) / 1000.0
        c = self.coefficients
        n = np.array(c[..., 0])
        for i in range(1, c.shape[-1]):
            n = n + c[..., i] / w ** (2 * i)
        return n * n


class EpsilonSellmeier(EpsilonDispersive):
    """Sellmeier dispersion: eps = c0 + sum_i c_(2i+1) w^2 / (w^2 - c_(2i+2)), w in microns."""

    def __call__(self, wavelength):
        w = float(wavelength) / 1000.0
        c = self.coefficients
        eps = np.array(c[..., 0])
        for i in range((c.shape[-1] - 1) // 2):
            eps = eps + (c[..., 1 + 2 * i] * w ** 2) / (w ** 2 - c[..., 2 + 2 * i])
        return eps


def _run(director, mask, no, ne, nhost, scale_factor):
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("dtmm_gb300.data needs a CUDA GPU (there is no CPU path)")
    host = not isinstance(director, torch.Tensor)
    d = torch.from_numpy(np.ascontiguousarray(director)) if host else director
    if d.shape[-1] != 3:
        raise ValueError("director must have 3 components in its last axis")
    if d.dtype not in (torch.float32, torch.float64):
        d = d.to(torch.float64)
    d = d.cuda().contiguous()
    dev = d.device
    m = None
    if mask is not None:
        if nhost is None:
            raise ValueError("nhost must be given with a mask")
        mt = torch.from_numpy(np.ascontiguousarray(mask)) if not isinstance(mask, torch.Tensor) else mask
        m = mt.to(device=dev, dtype=torch.uint8).contiguous()
        if tuple(m.shape) != tuple(d.shape[:-1]):
            raise ValueError("mask must have the director's shape without its last axis")
    epsv = torch.empty(d.shape, dtype=torch.float64, device=dev)
    epsa = torch.empty(d.shape, dtype=torch.float64, device=dev)
    nvox = int(np.prod(d.shape[:-1]))
    lib = _lib.load()
    _lib.check(lib.dtmm_director2data(nvox, ctypes.c_void_p(d.data_ptr()), int(d.dtype == torch.float64),
                                      ctypes.c_void_p(m.data_ptr() if m is not None else None), float(no), float(ne),
                                      float(nhost if nhost is not None else 1.0), float(scale_factor),
                                      ctypes.c_void_p(epsv.data_ptr()), ctypes.c_void_p(epsa.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    return epsv, epsa, host, (m, d)


def director2data(director, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0, thickness=None):
    """Optical block ``(thickness, epsv, epsa)`` from a director field (dtmm/data.py:277)."""
    epsv, epsa, host, _ = _run(director, mask, no, ne, nhost, scale_factor)
    nl = epsv.shape[0]
    thickness = np.ones((nl,)) if thickness is None else np.asarray(thickness, np.float64)
    if host:
        return thickness, epsv.cpu().numpy(), epsa.cpu().numpy()
    return thickness, epsv, epsa


def director2angles(director):
    """Euler angles (0, theta, phi) of a director field [..., 3] (dtmm/data.py:975-990), from the
    same kernel as ``director2data``; numpy in, numpy out, device tensors stay on the device."""
    _, epsa, host, _ = _run(director, None, 1.5, 1.6, None, 1.0)
    return epsa.cpu().numpy() if host else epsa


_Q_ROWS = (0, 1, 2, 0, 0, 1)
_Q_COLS = (0, 1, 2, 1, 2, 2)


def _q_run(tensor, mask, no, ne, nhost, scale_factor, biaxial):
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("dtmm_gb300.data needs a CUDA GPU (there is no CPU path)")
    host = not isinstance(tensor, torch.Tensor)
    q = torch.from_numpy(np.ascontiguousarray(tensor)) if host else tensor
    if q.is_complex():
        raise ValueError("Q2data takes a real Q tensor")
    if q.shape[-1] != 6:
        if tuple(q.shape[-2:]) != (3, 3):
            raise ValueError("input tensor must be an array of shape (...,6) or (...,3,3)")
        q = q[..., list(_Q_ROWS), list(_Q_COLS)]
    q = q.to(dtype=torch.float64).cuda().contiguous()
    dev = q.device
    shape = tuple(q.shape[:-1])
    m = None
    if mask is not None:
        if nhost is None:
            raise ValueError("nhost must be given with a mask")
        mt = torch.from_numpy(np.ascontiguousarray(mask)) if not isinstance(mask, torch.Tensor) else mask
        m = mt.to(device=dev, dtype=torch.uint8).contiguous()
        if tuple(m.shape) != shape:
            raise ValueError("mask must have the tensor field's shape")
    epsv = torch.empty(shape + (3,), dtype=torch.float64, device=dev)
    epsa = torch.empty(shape + (3,), dtype=torch.float64, device=dev)
    lib = _lib.load()
    _lib.check(lib.dtmm_q2data(int(np.prod(shape)), ctypes.c_void_p(q.data_ptr()),
                               ctypes.c_void_p(m.data_ptr() if m is not None else None), float(no), float(ne),
                               float(nhost if nhost is not None else 1.0), float(scale_factor), int(bool(biaxial)),
                               ctypes.c_void_p(epsv.data_ptr()), ctypes.c_void_p(epsa.data_ptr()),
                               ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    return epsv, epsa, host, (m, q)


def Q2data(tensor, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0, biaxial=False, thickness=None):
    """Optical block ``(thickness, epsv, epsa)`` from a Q-tensor field (dtmm/data.py:322)."""
    epsv, epsa, host, _ = _q_run(tensor, mask, no, ne, nhost, scale_factor, biaxial)
    nl = epsv.shape[0]
    thickness = np.ones((nl,)) if thickness is None else np.asarray(thickness, np.float64)
    if host:
        return thickness, epsv.cpu().numpy(), epsa.cpu().numpy()
    return thickness, epsv, epsa


def device_material(director, shape=None, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0,
                    thickness=None):
    """``director2data`` kept on the device as a ``DeviceMaterial`` for ``plan_transfer``."""
    from .transfer import DeviceMaterial

    epsv, epsa, _, _ = _run(director, mask, no, ne, nhost, scale_factor)
    nl = epsv.shape[0]
    th = np.ones((nl,)) if thickness is None else np.asarray(thickness, np.float64)
    return DeviceMaterial(th, epsv, epsa, tuple(epsv.shape[1:3]) if shape is None else shape)


def q_material(tensor, shape=None, mask=None, no=1.5, ne=1.6, nhost=None, scale_factor=1.0, thickness=None,
               biaxial=False):
    """``Q2data`` kept on the device as a ``DeviceMaterial`` for ``plan_transfer``
    (``biaxial=True`` keeps the three eigenvalues; the transfer then takes the
    general eigen-solve)."""
    from .transfer import DeviceMaterial

    epsv, epsa, _, _ = _q_run(tensor, mask, no, ne, nhost, scale_factor, biaxial)
    nl = epsv.shape[0]
    th = np.ones((nl,)) if thickness is None else np.asarray(thickness, np.float64)
    return DeviceMaterial(th, epsv, epsa, tuple(epsv.shape[1:3]) if shape is None else shape,
                          uniaxial=not biaxial)


__all__ = ["director2data", "director2angles", "Q2data", "device_material", "q_material"]
