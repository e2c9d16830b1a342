"""POM image formation kernels against the reference's outputs (GPU).

Fixtures ``tests/golden/pom_*.npz`` hold the reference's POM field, specter
and colours for each case (one refocused through a diffraction matrix); the
fused image kernel has no refocus, so for that case it is checked against the
oracle's chain without refocus.
Tolerances: POM field 1e-12 relative (complex128) / 1e-6 (complex64);
specter 1e-13 relative; colours from a specter 1e-13 absolute; the fused
float32 image 2e-6 absolute (complex128 field) / 2e-5 (complex64).
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from golden_cases import POM_CASES, raised_cosine_window  # noqa: E402

COLOR_OPTS = [("rgb", {}), ("rgb_gray", dict(gray=True)), ("rgb_norm", dict(norm=True)),
              ("rgb_gamma", dict(norm=0.7, gamma=2.2)), ("rgb_linear", dict(norm=0.5, gamma=False))]


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _inputs(name):
    from dtmm_gb300 import pom

    case = POM_CASES[name]
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    jvec = pom.jonesvec(*case["jvec"]) if case["jvec"] is not None else None
    an = case["analyzer"]
    pmat = pom.ray_jonesmat4x4(pom.rotated_matrix(pom.polarizer(pom.jonesvec(an[0])), an[1]))
    win = raised_cosine_window(z["field_in"].shape[-2:]) if case.get("window") else None
    return case, z, jvec, pmat, win


def _expected_pom(case, z, jvec, pmat, win):
    """The reference's POM field, or the oracle's without refocus for the refocused case."""
    if "dmat" not in z.files:
        return z["pom"]
    import dtmm_oracle as O

    return O.calculate_pom_field(z["field_in"], jvec, pmat, None, win)


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(POM_CASES))
def test_pom_field(name, precision):
    """calculate_pom_field, with the refocus (diffraction matrix) where the case has one."""
    from dtmm_gb300 import pom

    case, z, jvec, pmat, win = _inputs(name)
    f = z["field_in"].astype(np.complex128 if precision == "double" else np.complex64)
    dmat = z["dmat"] if "dmat" in z.files else None
    got = pom.calculate_pom_field(f, jvec, pmat, dmat, window=win)
    assert rel(got, z["pom"]) < (1e-12 if precision == "double" else 1e-6)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_diffract_matches_oracle(precision):
    import dtmm_oracle as O
    from dtmm_gb300 import pom

    z = np.load(os.path.join(HERE, "golden", "pom_rotated.npz"))
    f = z["field_in"][0]  # x-polarised input: (lam, 4, H, W)
    want = O.diffract(f, z["dmat"])
    got = pom.diffract(f.astype(np.complex128 if precision == "double" else np.complex64), z["dmat"])
    assert rel(got, want) < (1e-12 if precision == "double" else 1e-6)


@pytest.mark.parametrize("name", sorted(POM_CASES))
def test_field2specter_and_colours(name):
    from dtmm_gb300 import pom

    case, z, _, _, _ = _inputs(name)
    spec = pom.field2spectersum(z["pom"]) if case.get("summed") else pom.field2specter(z["pom"])
    assert spec.shape == z["spec"].shape
    assert rel(spec, z["spec"]) < 1e-13
    for key, kw in COLOR_OPTS:
        got = pom.specter2color(z["spec"], z["cmf"], **kw)
        assert np.abs(got - z[key]).max() < 1e-13, key


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(POM_CASES))
def test_fused_pom_image(name, precision):
    import dtmm_oracle as O
    from dtmm_gb300 import pom

    case, z, jvec, pmat, win = _inputs(name)
    f = z["field_in"].astype(np.complex128 if precision == "double" else np.complex64)
    p = _expected_pom(case, z, jvec, pmat, win)
    spec = O.field2spectersum(p) if p.ndim == 5 else O.field2specter(p)
    if spec.ndim == 4:  # summed over the leading sets, as the image does
        spec = spec.sum(axis=0)
    tol = 2e-6 if precision == "double" else 2e-5
    for key, kw in COLOR_OPTS:
        want = O.specter2color(spec, z["cmf"], **kw)
        got = pom.pom_image(f, z["cmf"], jvec, pmat, window=win, **kw)
        assert got.shape == want.shape and got.dtype == np.float32
        assert np.abs(got - want).max() < tol, key
