"""director2data: the oracle against the reference's own output
(``tests/golden/director.npz``: seeded directors of lengths 0 to 1.3, default
parameters and a masked host region with a scale factor), within 1e-15."""
import os

import numpy as np

import dtmm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_director2data_matches_reference():
    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    th, ev, ea = O.director2data(z["director"])
    assert np.array_equal(th, z["thickness_default"])
    assert np.abs(ev - z["epsv_default"]).max() < 1e-15 * 4
    assert np.abs(ea - z["epsa_default"]).max() < 1e-15 * 4
    _, ev, ea = O.director2data(z["director"], mask=z["mask"], no=1.52, ne=1.71, nhost=1.4, scale_factor=0.8)
    assert np.abs(ev - z["epsv_masked"]).max() < 1e-15 * 4
    assert np.abs(ea - z["epsa_masked"]).max() < 1e-15 * 4


def _rebuild(epsv, epsa):
    """eps tensors [..., 3, 3] = R diag(epsv) R^T from eigenvalues and Euler angles."""
    R = O._rotation_matrix(epsa[..., 0], epsa[..., 1], epsa[..., 2])
    return np.einsum("...ij,...j,...kj->...ik", R, epsv, R)


def _full(eps6):
    rows, cols = (0, 1, 2, 0, 0, 1, 1, 2, 2), (0, 1, 2, 1, 2, 2, 0, 0, 1)
    out = np.empty(eps6.shape[:-1] + (3, 3))
    for k, (r, c) in enumerate(zip(rows, cols)):
        out[..., r, c] = eps6[..., (0, 1, 2, 3, 4, 5, 3, 4, 5)[k]]
    return out


def test_oracle_q2data_matches_reference():
    """Q2data: the oracle against the reference's output (``tests/golden/qtensor.npz``:
    layer 0 exactly uniaxial Q tensors of random directors and orders, three of
    them diagonal; layer 1 the same plus a biaxial perturbation), uniaxial,
    masked with other indices and scale factor, and biaxial; eigenvalues to
    4e-15, Euler angles to 1e-13."""
    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    cases = [("", {}), ("_masked", dict(mask=z["mask"], no=1.52, ne=1.71, nhost=1.4, scale_factor=0.9)),
             ("_biaxial", dict(biaxial=True))]
    for tag, kw in cases:
        th, ev, ea = O.Q2data(z["Q"], **kw)
        assert np.array_equal(th, np.ones(2))
        assert np.abs(ev - z["epsv" + tag]).max() < 4e-15, tag
        assert np.abs(ea - z["epsa" + tag]).max() < 1e-13, tag


def test_oracle_q2data_diagonalises_eps():
    """The biaxial eigenvalues and angles rebuild the eps tensor of Q2eps: to
    1e-12 where the eigenvalues are distinct, and to the eigenvalue split of
    rounding (1e-7) where two are equal."""
    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    _, ev, ea = O.Q2data(z["Q"], biaxial=True)
    eps = _full(O.Q2eps(z["Q"]))
    err = np.abs(_rebuild(ev, ea) - eps).max(axis=(-1, -2))
    assert err[1].max() < 1e-12
    assert err[0].max() < 1e-7
    # the eigenvalues are the spectrum of eps
    w = np.linalg.eigvalsh(eps)
    assert np.abs(np.sort(ev, axis=-1) - w).max() < 1e-7
