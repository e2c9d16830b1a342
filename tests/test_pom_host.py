"""POM image formation: the oracle and the host-side matrices against the
reference's own outputs (``tests/golden/pom_*.npz`` from ``make_golden.py``:
``calculate_pom_field`` with polarizer, window, diffraction matrix and
analyzer, ``field2specter`` / ``field2spectersum``, ``specter2color`` with the
reference's ``load_tcmf`` and five option sets).  Tolerances: 1e-13 relative
for fields and specters, 1e-14 absolute for colours in [0, 1]."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import dtmm_oracle as O  # noqa: E402
from golden_cases import POM_CASES, raised_cosine_window  # noqa: E402

from dtmm_gb300 import pom  # noqa: E402

COLOR_OPTS = [("rgb", {}), ("rgb_gray", dict(gray=True)), ("rgb_norm", dict(norm=True)),
              ("rgb_gamma", dict(norm=0.7, gamma=2.2)), ("rgb_linear", dict(norm=0.5, gamma=False))]


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _case(name):
    return POM_CASES[name], np.load(os.path.join(HERE, "golden", name + ".npz"))


@pytest.mark.parametrize("name", sorted(POM_CASES))
def test_host_matrices_match_reference(name):
    case, z = _case(name)
    if case["jvec"] is not None:
        assert rel(pom.jonesvec(*case["jvec"]), z["jvec"]) < 1e-15
    an = case["analyzer"]
    pm = pom.ray_jonesmat4x4(pom.rotated_matrix(pom.polarizer(pom.jonesvec(an[0])), an[1]))
    assert np.abs(pm - z["pmat"]).max() < 1e-14


@pytest.mark.parametrize("name", sorted(POM_CASES))
def test_oracle_pom_pipeline_matches_reference(name):
    case, z = _case(name)
    f = z["field_in"]
    jvec = O.jonesvec(*case["jvec"]) if case["jvec"] is not None else None
    an = case["analyzer"]
    pmat = O.ray_jonesmat4x4(O.rotated_matrix(O.polarizer(O.jonesvec(an[0])), an[1]))
    win = raised_cosine_window(f.shape[-2:]) if case.get("window") else None
    dmat = z["dmat"] if "dmat" in z.files else None
    p = O.calculate_pom_field(f, jvec, pmat, dmat, win)
    assert rel(p, z["pom"]) < 1e-13
    spec = O.field2spectersum(p) if case.get("summed") else O.field2specter(p)
    assert rel(spec, z["spec"]) < 1e-13
    for key, kw in COLOR_OPTS:
        assert np.abs(O.specter2color(z["spec"], z["cmf"], **kw) - z[key]).max() < 1e-14, key


def test_field_diffraction_matrix_matches_reference():
    z = np.load(os.path.join(HERE, "golden", "pom_rotated.npz"))
    ks = 2 * np.pi / z["wavelengths"] * 50.0  # pixel size of the source case
    dm = pom.field_diffraction_matrix(z["field_in"].shape[-2:], ks, d=POM_CASES["pom_rotated"]["dmat_d"],
                                      epsv=(2.25, 2.25, 2.25))
    assert np.abs(dm - z["dmat"]).max() < 1e-14
