"""Windows, ray sets, windowed illumination and colour tables on the host,
against the reference's own outputs (``tests/golden/illum_window.npz``,
``tests/golden/tcmf.npz``, made by ``make_golden.py``):

* ``window.aperture`` / ``blackman`` / ``gaussian`` within 1e-15;
* ``illumination_rays`` (beta, phi, intensity) within 1e-15;
* ``illumination_data`` with a window (plane waves times the window, the
  cover's diffraction over -focus, the intensity rescale) within 1e-12
  relative L2;
* ``color.load_tcmf`` for every option within 1e-13 relative.
"""
import os

import numpy as np
import pytest

from golden_cases import ILLUM_WINDOW_CASES, RAYS_CASES, TCMF_CASES, TCMF_TABLES, WINDOW_CASES

HERE = os.path.dirname(os.path.abspath(__file__))


def _z(name):
    return np.load(os.path.join(HERE, "golden", name))


@pytest.mark.parametrize("name", sorted(WINDOW_CASES))
def test_windows(name):
    from dtmm_gb300 import window

    fn, args = WINDOW_CASES[name]
    want = _z("illum_window.npz")["window_" + name]
    got = getattr(window, fn)(*args)
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= 1e-15


@pytest.mark.parametrize("name", sorted(RAYS_CASES))
def test_illumination_rays(name):
    from dtmm_gb300.illumination import illumination_rays

    z = _z("illum_window.npz")
    b, p, i = illumination_rays(*RAYS_CASES[name])
    for got, key in ((b, "beta"), (p, "phi"), (i, "intensity")):
        want = z["rays_%s_%s" % (name, key)]
        assert got.shape == want.shape
        assert np.abs(got - want).max() <= 1e-15, key


def window_inputs(name, z):
    kw = dict(ILLUM_WINDOW_CASES[name])
    shape, wl, ps = kw.pop("shape"), kw.pop("wavelengths"), kw.pop("pixelsize")
    kw["window"] = z["window_" + kw.pop("window")]
    rays = kw.pop("rays", None)
    if rays is not None:
        kw["beta"], kw["phi"], kw["intensity"] = (z["rays_%s_%s" % (rays, k)] for k in ("beta", "phi", "intensity"))
    return shape, wl, ps, kw


@pytest.mark.parametrize("name", sorted(ILLUM_WINDOW_CASES))
def test_windowed_illumination_host(name):
    from dtmm_gb300 import illumination_data

    z = _z("illum_window.npz")
    shape, wl, ps, kw = window_inputs(name, z)
    got = illumination_data(shape, wl, pixelsize=ps, **kw)[0]
    want = z[name]
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


@pytest.mark.parametrize("name", sorted(TCMF_CASES))
def test_load_tcmf(name):
    from dtmm_gb300 import color

    z = _z("tcmf.npz")
    kw = dict(TCMF_CASES[name])
    cmf = kw.pop("cmf", "CIE1931")
    illuminant = kw.pop("illuminant", "D65")
    x, got = color.load_tcmf(retx=True, cmf=z["table_" + cmf], illuminant=z["table_" + illuminant], **kw)
    want = z[name]
    assert got.shape == want.shape
    assert np.allclose(np.asarray(x, float), z[name + "_x"], rtol=0, atol=0)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max(), name
    assert set(TCMF_TABLES) >= {cmf, illuminant}
