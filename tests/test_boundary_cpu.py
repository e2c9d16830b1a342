"""The drop-in boundary's error behaviour, on the host: invalid options raise
the reference's ValueErrors (dtmm/transfer.py:42-65, :433-465, :536-543,
:627, :1020, :1083; dtmm/data.py:1344-1362, :1364-1419), option variants
the engine does not build raise NotImplementedError, and both happen before
the device is touched.  A valid call on a machine without a GPU raises: the
engine has no CPU path."""
import numpy as np
import pytest

import dtmm_gb300
from dtmm_gb300 import samples


def _field(nlam=1, shape=(8, 8), rays=0):
    f = np.zeros(((rays,) if rays else ()) + (nlam, 4) + shape, np.complex128)
    f[..., 0, :, :] = 1.0
    f[..., 1, :, :] = 1.5
    return f


def _call(field=None, wavelengths=(550.0,), optical=None, **kw):
    field = _field() if field is None else field
    optical = [samples.twisted_nematic(field.shape[-2:], 2, seed=3)] if optical is None else optical
    return dtmm_gb300.transfer_field((field, np.asarray(wavelengths), 100.0), optical, **kw)


@pytest.mark.parametrize("kw,match", [
    (dict(method="4x4", reflection=5), "Invalid reflection. The 4x4 method"),
    (dict(method="2x2", reflection=3), "Invalid reflection. The 2x2 method"),
    (dict(method="2x2", npass=2, reflection=0), "Reflection mode `0` not compatible with npass > 1"),
    (dict(method="4x4", diffraction=-1), "Invalid diffraction value"),
    (dict(method="4x4", beta=0.1), "Both beta and phi must be defined!"),
    (dict(method="4x4", beta=[0.1, 0.2], phi=0.0), "Beta nad phi should have same dimensions!"),
    (dict(method="4x4", beta=[0.1, 0.2], phi=[0.0]), "Beta nad phi should have same length!"),
    (dict(method="4x4", beta=[0.1, 0.2], phi=[0.0, 0.0]), "per-ray beta"),
    (dict(method="4x4", precision="half"), "precision"),
    (dict(method="4x4", npass=2, norm=4), "norm must be a combination"),
    (dict(method="4x4", eff_data="nematic"), "Invalid symmetry argument"),
    (dict(method="4x4", eff_data=[1, 2]), "Number of elements in eff_data"),
    (dict(method="4x4", eff_data=[[1, 0, 2]]), "incompatible with block size"),
])
def test_invalid_options_raise_value_error(kw, match):
    with pytest.raises(ValueError, match=match):
        _call(**kw)


def test_shape_errors():
    with pytest.raises(ValueError, match="Invald field dimensions"):
        _call(field=np.zeros((4, 8, 8), np.complex128), method="4x4")
    with pytest.raises(ValueError, match="Incompatible wavelengths shape"):
        _call(wavelengths=(500.0, 600.0), method="4x4")


def test_dispersive_data_needs_split_wavelengths():
    d, ev, ea = samples.twisted_nematic((8, 8), 2, seed=3)
    with pytest.raises(ValueError, match="split_wavelengths=True"):
        _call(optical=[(d, lambda w: ev, ea)], method="4x4")


@pytest.mark.parametrize("kw", [
    dict(method="4x4", npass=-1),
    dict(method="2x2", reflection=1, eff_data=1),
    dict(method="2x2", reflection=1, diffraction=np.inf),
    dict(method="4x4", reflection=3, diffraction=0),
    dict(method="4x4", reflection=2, npass=2, ret_bulk=True),
    dict(method="4x4", eff_data=[(2.0 * np.ones(2), np.full((2, 3), 2.4), np.zeros((2, 3)))]),
])
def test_unbuilt_variants_raise_not_implemented(kw):
    with pytest.raises(NotImplementedError):
        _call(**kw)


def test_valid_call_needs_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the call would run")
    with pytest.raises(RuntimeError, match="CUDA GPU"):
        _call(method="4x4", eff_data=1)
