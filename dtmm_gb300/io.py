"""The reference's file formats for field data and optical stacks.

``.dtmf`` (dtmm/field.py:903-969): the magic ``b"dtmf"``, version byte 0, then
the field, wavelengths and pixel size as consecutive ``.npy`` records.
``.dtms`` (dtmm/data.py:1530-1632): the magic ``b"dtms"``, version byte 2, then
(thickness, eps values, eps angles) ``.npy`` records per block; version 1
files hold a single block whose angles may be missing.  Files written here are
byte-identical to the reference's for the same arrays, so either side reads
the other's files.  Dispersive (Cauchy / Sellmeier) eps records are outside the
transfer engine and are refused.

Device tensors are accepted and returned on request (``device=``), so a
serving loop can checkpoint request state to disk and restore it to the GPU.
"""
from __future__ import annotations

import numpy as np

FIELD_MAGIC = b"dtmf"
FIELD_VERSION = b"\x00"
STACK_MAGIC = b"dtms"
STACK_VERSION = b"\x02"
STACK_VERSION_1 = b"\x01"


def _host(a):
    try:
        import torch

        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


def _open(file, mode, ext):
    if isinstance(file, str):
        if "w" in mode and not file.endswith(ext):
            file = file + ext
        return open(file, mode), True
    return file, False


def save_field(file, field_data):
    """Write ``(field, wavelengths, pixelsize)`` in ``.dtmf`` format (dtmm/field.py:906)."""
    field, wavelengths, pixelsize = field_data
    field = _host(field)
    wavelengths = np.asarray(_host(wavelengths))
    if field.ndim < 4 or field.shape[-3] not in (2, 4):
        raise ValueError("Invald field dimensions")
    f, own = _open(file, "wb", ".dtmf")
    try:
        f.write(FIELD_MAGIC)
        f.write(FIELD_VERSION)
        np.save(f, field)
        np.save(f, wavelengths)
        np.save(f, pixelsize)
    finally:
        if own:
            f.close()


def load_field(file, device=None, dtype=None):
    """Read a ``.dtmf`` file (dtmm/field.py:941); with ``device`` the field is a tensor there."""
    f, own = _open(file, "rb", ".dtmf")
    try:
        magic = f.read(len(FIELD_MAGIC))
        if magic != FIELD_MAGIC:
            raise OSError("Failed to interpret file {}".format(file))
        if f.read(1) != FIELD_VERSION:
            raise OSError("This file was created with a more recent version of dtmm. Please upgrade your dtmm package!")
        field = np.load(f)
        wavelengths = np.load(f)
        pixelsize = float(np.load(f))
    finally:
        if own:
            f.close()
    if device is not None:
        import torch

        field = torch.from_numpy(field).to(device)
        if dtype is not None:
            field = field.to(dtype)
    return field, wavelengths, pixelsize


def save_stack(file, optical_data):
    """Write optical data (a list of blocks) in ``.dtms`` format, version 2 (dtmm/data.py:1539)."""
    blocks = optical_data if isinstance(optical_data, list) else [optical_data]
    f, own = _open(file, "wb", ".dtms")
    try:
        f.write(STACK_MAGIC)
        f.write(STACK_VERSION)
        for d, epsv, epsa in blocks:
            if callable(epsv):
                raise NotImplementedError("dispersive eps records are outside the transfer engine")
            np.save(f, np.asarray(_host(d)), allow_pickle=False)
            np.save(f, np.asarray(_host(epsv)), allow_pickle=True)
            np.save(f, np.asarray(_host(epsa)), allow_pickle=False)
    finally:
        if own:
            f.close()


def load_stack(file):
    """Read a ``.dtms`` file (dtmm/data.py:1580): a list of (thickness, epsv, epsa)
    blocks (version 2), or the single-block list [d, epsv, epsa] of version 1."""
    f, own = _open(file, "rb", ".dtms")
    try:
        magic = f.read(len(STACK_MAGIC))
        if magic != STACK_MAGIC:
            raise OSError("Failed to interpret file {}".format(file))
        version = f.read(1)
        if ord(version) > ord(STACK_VERSION):
            raise OSError("This file was created with a more recent version of dtmm. Please upgrade your dtmm package!")
        rest = f.read()
    finally:
        if own:
            f.close()
    import io as _io

    buf = _io.BytesIO(rest)

    def more():
        return buf.tell() < len(rest)

    if version == STACK_VERSION_1:
        d = np.load(buf)
        epsv = np.load(buf)
        epsa = np.load(buf) if more() else None
        return [d, epsv, epsa]
    out = []
    while more():
        d = np.load(buf)
        epsv = np.load(buf, allow_pickle=True)
        if epsv.dtype == object:
            raise NotImplementedError("dispersive eps records are outside the transfer engine")
        epsa = np.load(buf)
        out.append((d, epsv, epsa))
    return out


__all__ = ["save_field", "load_field", "save_stack", "load_stack"]
