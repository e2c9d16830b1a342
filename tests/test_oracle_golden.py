"""The oracle (CPU restatement) against the reference's own outputs and known answers.

Fixtures under tests/golden/ were produced by running the unmodified reference
(tests/golden/make_golden.py).  Tolerances: the restatement is complex128 like
the reference, so whole transfers agree to rounding (rel. L2 <= 1e-11).
"""
import numpy as np
import pytest

import dtmm_oracle as O
from golden_cases import CASES, ORACLE_CASES, build_optical_data

GOLDEN_TOL = 1e-11


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("name", sorted(CASES) + sorted(ORACLE_CASES))
def test_oracle_matches_reference_transfer(name, golden):
    case = CASES[name] if name in CASES else ORACLE_CASES[name]
    z = golden(name)
    field_in = z["field_in"].copy()
    out = O.transfer_field((field_in, z["wavelengths"], float(z["pixelsize"])), build_optical_data(case),
                           **case["transfer"])[0]
    assert out.shape == z["field_out"].shape
    assert rel_l2(out, z["field_out"]) < GOLDEN_TOL
    # npass > 1 rewrites field_in in place with the reflected field
    assert rel_l2(field_in, z["field_in_after"]) < GOLDEN_TOL


def test_oracle_only_cases_are_separate_and_have_fixtures():
    """Cases pinned ahead of the engine stay out of the GPU parity set and each
    has its reference fixture."""
    import os

    from make_fullsize import FULL_CASES

    assert not set(ORACLE_CASES) & set(CASES)
    # the full-grid fixtures share the directory: no case may reuse their names
    assert not (set(CASES) | set(ORACLE_CASES)) & set(FULL_CASES)
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for name in list(CASES) + list(ORACLE_CASES):
        assert os.path.exists(os.path.join(here, name + ".npz")), name


def test_oracle_alphaf_biaxial_matches_reference(golden):
    """Biaxial voxels: the general eigen-solve and the Poynting sort give the
    reference's eigenvalues and field matrices (both call LAPACK; the rotated
    tensor is formed in a different operation order, which moves the
    eigenvectors of the closer eigenvalue pairs by up to a few 1e-13)."""
    z = golden("kat_alphaf_biaxial")
    alpha, f = O.alphaf(z["beta"], z["phi"], z["epsv"], z["epsa"])
    assert np.all(np.isfinite(z["alpha"]))
    assert np.abs(alpha - z["alpha"]).max() < 1e-13
    assert np.abs(f - z["f"]).max() < 1e-11
    assert np.abs(O.inv(f) - z["fi"]).max() < 1e-11


def test_oracle_wave_known_answers(golden):
    z = golden("kat_wave")
    shape = tuple(int(s) for s in z["shape"])
    beta, phi = O.betaphi(shape, z["ks"])
    bx, by = O.betaxy(shape, z["ks"])
    assert np.allclose(beta, z["beta"], rtol=1e-5, atol=1e-8)
    assert np.allclose(phi, z["phi"], rtol=1e-5, atol=1e-8)
    assert np.allclose(bx, z["betax"], rtol=1e-5, atol=1e-8)
    assert np.allclose(by, z["betay"], rtol=1e-5, atol=1e-8)


def test_oracle_alphaf_matches_reference(golden):
    z = golden("kat_alphaf")
    alpha, f = O.alphaf(z["beta"], z["phi"], z["epsv"], z["epsa"])
    assert np.abs(alpha - z["alpha"]).max() < 1e-13
    assert np.abs(f - z["f"]).max() < 1e-13
    assert np.abs(O.inv(f) - z["fi"]).max() < 1e-12


def test_oracle_dot_products_match_multi_dot():
    """Property checks of the reference's linalg tests (dtmm/test/test_linalg.py:28-66)."""
    rng = np.random.default_rng(0)
    f = rng.standard_normal((4, 15, 16)) + 0j
    a = rng.standard_normal((15, 16, 4, 4)) + 0j
    d = rng.standard_normal((15, 16, 4)) + 0j
    b = rng.standard_normal((15, 16, 4, 4)) + 0j
    out1 = O.dotmf(a, f)
    out2 = O.dotmdmf(a, np.exp(2.3j * d), b, f)
    for i in range(15):
        for j in range(16):
            assert np.allclose(out1[:, i, j], a[i, j] @ f[:, i, j])
            assert np.allclose(out2[:, i, j], np.linalg.multi_dot([a[i, j], np.diag(np.exp(2.3j * d[i, j])), b[i, j], f[:, i, j]]))


def test_oracle_inverse_singular_maps_to_zero():
    m = np.zeros((3, 4, 4), complex)
    m[1] = np.eye(4) * 2
    out = O.inv(m)
    assert np.all(out[0] == 0) and np.all(out[2] == 0)
    assert np.allclose(out[1], np.eye(4) / 2)


def test_oracle_alphaf_continuity_near_normal_incidence():
    """alphaf is continuous across the beta == 0 branch (dtmm/test/test_tmm.py:45-57)."""
    epsv = (2.25, 2.25, 2.89)
    epsa = (0.0, 0.4, 0.7)
    a0, f0 = O.alphaf(0.0, 0.3, epsv, epsa)
    a1, f1 = O.alphaf(1e-9, 0.3, epsv, epsa)
    assert np.allclose(a0, a1, atol=1e-7)
    assert np.allclose(np.abs(f0), np.abs(f1), atol=1e-7)
