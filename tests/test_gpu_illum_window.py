"""Windowed illumination, its diffraction matrix and the plane-wave fill on
the GPU (``-m gpu``): ``illumination_device(window=...)`` against the
reference's fields (``tests/golden/illum_window.npz``) within 1e-10 relative
L2 in complex128 and 1e-5 with complex64 fields; the device
``field_diffraction_matrix`` against the host one within 1e-13 absolute."""
import os

import numpy as np
import pytest

from golden_cases import ILLUM_WINDOW_CASES

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(ILLUM_WINDOW_CASES))
def test_windowed_illumination_device(name, precision):
    import torch

    from dtmm_gb300.illumination import illumination_device
    from test_illumination_window import window_inputs

    z = np.load(os.path.join(HERE, "golden", "illum_window.npz"))
    shape, wl, ps, kw = window_inputs(name, z)
    got = illumination_device(shape, wl, ps, precision=precision, **kw)
    torch.cuda.synchronize()
    got = got.cpu().numpy().astype(np.complex128)
    want = z[name]
    assert got.shape == want.shape
    assert rel(got, want) < (1e-10 if precision == "double" else 1e-5)


@pytest.mark.parametrize("mode", ["b", "t", "r"])
def test_field_diffraction_matrix_device(mode):
    import torch

    from dtmm_gb300 import pom

    ks = 2 * np.pi / np.array([450.0, 560.0, 700.0]) * 90.0
    host = pom.field_diffraction_matrix((24, 30), ks, d=-3.5, epsv=(1.5 ** 2,) * 3, mode=mode, betamax=0.9)
    dev = pom.field_diffraction_matrix((24, 30), ks, d=-3.5, epsv=(1.5 ** 2,) * 3, mode=mode, betamax=0.9,
                                       device=torch.device("cuda"))
    torch.cuda.synchronize()
    assert np.abs(dev.cpu().numpy() - host).max() < 1e-13
