"""GPU engine vs the reference's own outputs (golden fixtures) and the oracle.

Tolerances (relative L2 of the output field):
  complex128 engine : 1e-10  (reference and engine are both complex128)
  mixed engine      : 1e-4   (complex64 bulk, FP64 eigen-solve)
"""
import numpy as np
import pytest

import dtmm_gb300
from golden_cases import CASES, build_optical_data

TOL = {"double": 1e-10, "mixed": 1e-4}

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_matches_reference(name, precision, golden):
    case = CASES[name]
    z = golden(name)
    field_in = z["field_in"].copy()
    out = dtmm_gb300.transfer_field((field_in, z["wavelengths"], float(z["pixelsize"])), build_optical_data(case),
                                    precision=precision, **case["transfer"])[0]
    assert out.shape == z["field_out"].shape
    err = rel_l2(out, z["field_out"])
    assert err < TOL[precision], err
    err_in = rel_l2(field_in, z["field_in_after"])
    assert err_in < TOL[precision], err_in
