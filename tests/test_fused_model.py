"""The restructured (fused) layer sweep the kernels implement equals the reference.

Checks the numpy model of tests/fused_model.py against the reference's
golden outputs; tolerance 1e-11 (both complex128).
"""
import numpy as np
import pytest

import fused_model as FM
from golden_cases import CASES, build_optical_data

FUSED_CASES = ["cfg0_4x4", "fourx4_d3_offaxis", "fourx4_mixed_voxels", "fourx4_absorbing"]


@pytest.mark.parametrize("name", FUSED_CASES)
def test_fused_formulation_matches_reference(name, golden):
    case = CASES[name]
    z = golden(name)
    tr = case["transfer"]
    out = FM.transfer_4x4_fused(z["field_in"], z["wavelengths"], float(z["pixelsize"]), build_optical_data(case)[0],
                                beta=tr.get("beta", 0.0), phi=tr.get("phi", 0.0), diffraction=tr.get("diffraction", 1))
    ref = z["field_out"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-11
