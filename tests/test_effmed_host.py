"""The engine's effective medium of uniaxial / biaxial symmetry, checked on
the host.

``effmed_host.cpp`` runs the library's ``dtmm_effmed.h`` (the eigen-frame of
a block's mean lab-frame tensor, its Euler angles and the uniaxial
eigenvalues) on mean tensors of seeded random voxels; the oracle's
``effective_block`` restatement, pinned on the reference's own effective
layers by the transfer fixtures, gives the expected media.  Both restate
the same eigensolver, so their eigenvalues and Euler angles agree (also where
the extraordinary axis lies exactly along z, whose angles keep only the
cosine of the in-plane rotation), and so do the tensors R(angles) diag(epsv)
R^T.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle.dtmm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _tensor(ev, angles):
    R = O._rotation_matrix(angles[0], angles[1], angles[2])
    return O._rotate_diagonal_tensor(R, np.asarray(ev, np.complex128))


def _cases():
    rng = np.random.Generator(np.random.PCG64(4321))
    out = []
    for i in range(40):
        n = 16
        no, ne = rng.uniform(1.4, 1.6), rng.uniform(1.6, 1.8)
        ev = np.tile([no * no, no * no, ne * ne], (n, 1))
        if i % 4 == 1:  # biaxial voxels
            ev[:, 1] += rng.uniform(0.05, 0.2)
        if i % 4 == 2:  # weakly absorbing, one eigen-frame for both parts
            ev = ev + 0.01j * ev
        ea = np.stack([rng.uniform(-np.pi, np.pi, n), rng.uniform(0.2, 1.4, n) if i % 5 else np.zeros(n),
                       rng.uniform(-np.pi, np.pi, n) * (0.3 if i % 3 else 1.0)], axis=-1)
        if i % 7 == 0:  # every voxel alike: an exactly diagonal tensor in its own frame
            ea[:] = 0.0
        block = (np.ones(1), ev[None, :, None, :], ea[None, :, None, :])
        for sym in (1, 2):
            out.append((block, sym))
    return out


def test_effective_medium_matches_oracle(tmp_path):
    gxx = shutil.which("g++") or shutil.which("c++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "effmed_host")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "dtmm_gb300", "csrc"), "-o", exe,
                        os.path.join(HERE, "effmed_host.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    cases = _cases()
    lines = []
    for (d, ev, ea), sym in cases:
        R = O._rotation_matrix(ea[..., 0], ea[..., 1], ea[..., 2])
        t = O._rotate_diagonal_tensor(R, ev).reshape(-1, 6).mean(axis=0)
        lines.append("%d %d " % (sym, int(not np.iscomplexobj(ev))) + " ".join("%.17g %.17g" % (c.real, c.imag) for c in t))
    res = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    got = np.array([[float(x) for x in l.split()] for l in res.stdout.splitlines()])
    assert got.shape == (len(cases), 10)
    for ((block, sym), g) in zip(cases, got):
        evs, eas = O.effective_block(block, sym)
        ev_o, ea_o = np.asarray(evs[0]), np.asarray(eas[0])
        ev_g = g[1:7:2] + 1j * g[2:7:2]
        assert g[0] == sym
        np.testing.assert_allclose(ev_g, ev_o, rtol=0, atol=1e-13)
        np.testing.assert_allclose(g[7:], ea_o, rtol=0, atol=1e-12)
        np.testing.assert_allclose(_tensor(ev_g, g[7:]), _tensor(ev_o, ea_o), rtol=0, atol=1e-13)
        if sym == 1:  # the optic axis: the angles' theta / phi up to the axis' sign
            a_g = np.array([np.sin(g[8]) * np.cos(g[9]), np.sin(g[8]) * np.sin(g[9]), np.cos(g[8])])
            a_o = np.array([np.sin(ea_o[1]) * np.cos(ea_o[2]), np.sin(ea_o[1]) * np.sin(ea_o[2]), np.cos(ea_o[1])])
            assert abs(abs(a_g @ a_o) - 1.0) < 1e-12


def test_oracle_tensor_eig_is_an_eigen_decomposition():
    """The oracle's restated eigensolver against numpy's on seeded symmetric
    tensors: the same eigenvalues, a right-handed orthonormal frame of
    eigenvectors, and the most distinct eigenvalue third."""
    rng = np.random.Generator(np.random.PCG64(99))
    for i in range(60):
        a = rng.normal(size=(3, 3))
        a = a + a.T + (4.0 if i % 2 else 0.0) * np.eye(3)
        t = np.array([a[0, 0], a[1, 1], a[2, 2], a[0, 1], a[0, 2], a[1, 2]])
        w, v = O.tensor_eig(t, is_real=True)
        w, v = np.asarray(w).real, np.asarray(v).real
        np.testing.assert_allclose(np.sort(w), np.linalg.eigvalsh(a), rtol=0, atol=1e-12 * np.abs(a).max())
        np.testing.assert_allclose(v.T @ v, np.eye(3), atol=1e-12)
        assert np.linalg.det(v) > 0
        np.testing.assert_allclose(a @ v, v * w[None, :], atol=1e-11 * np.abs(a).max())
        gaps = [abs(w[1] - w[0]), abs(w[2] - w[0]), abs(w[2] - w[1])]
        assert gaps[0] <= max(gaps[1], gaps[2]) + 1e-12  # the third is the most distinct
