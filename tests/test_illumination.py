"""Input field builder against the reference's own illumination_data.

``illumination_data`` (host) and ``illumination_modes`` restate
dtmm/field.py:586-713 as per-image 4-vectors times single FFT-grid modes.
The fixtures hold the reference's full-grid fields (``make_golden.py``):
the transfer cases' inputs and the extra illumination cases (seven rays of
the batch workload, focus, backward waves, cover index 1, large beta).
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from golden_cases import CASES, ILLUM_CASES  # noqa: E402

from dtmm_gb300.illumination import illumination_data, illumination_modes, planewave_grid  # noqa: E402

TOL = 1e-13


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", sorted(CASES))
def test_transfer_case_inputs(name):
    case = CASES[name]
    ref = np.load(os.path.join(HERE, "golden", name + ".npz"))["field_in"]
    f = illumination_data(case["shape"], case["wavelengths"], pixelsize=case["pixelsize"], **dict(case["illum"]))[0]
    assert f.shape == ref.shape
    assert rel(f, ref) < TOL


@pytest.mark.parametrize("name", sorted(ILLUM_CASES))
def test_illumination_cases(name):
    kw = dict(ILLUM_CASES[name])
    shape, wl, ps = kw.pop("shape"), kw.pop("wavelengths"), kw.pop("pixelsize")
    ref = np.load(os.path.join(HERE, "golden", "illum.npz"))[name]
    f = illumination_data(shape, wl, pixelsize=ps, **kw)[0]
    assert f.shape == ref.shape
    assert rel(f, ref) < TOL


def test_modes_describe_single_fft_bins():
    kw = dict(ILLUM_CASES["rays7"])
    shape, wl, ps = kw.pop("shape"), kw.pop("wavelengths"), kw.pop("pixelsize")
    coef, my, mx = illumination_modes(shape, wl, ps, **kw)
    assert coef.shape == my.shape + (4,) == mx.shape + (4,)
    f = coef[..., :, None, None] * planewave_grid(shape, my, mx)[..., None, :, :]
    spec = np.abs(np.fft.fft2(f)).reshape(f.shape[:-2] + (-1,))
    energy = (spec ** 2).sum(-1)
    peak = spec.max(-1) ** 2
    nz = energy > 0
    assert np.all(peak[nz] / energy[nz] > 1 - 1e-12)
    # the normal-incidence ray has mode (0, 0); the tilted ones do not
    assert np.all(my[0] == 0) and np.all(mx[0] == 0)
    assert np.any(mx[1] != 0)
