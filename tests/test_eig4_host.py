"""The library's biaxial eigen-solve, compiled for the host and checked on the CPU.

``eig4_host.cu`` includes ``dtmm_gb300/csrc/dtmm_eig4.cuh`` (every function
there is __host__ __device__).  Checked here:

* the 4 x 4 complex eigen-decomposition against numpy on random, real,
  triangular, Hermitian, repeated-eigenvalue and zero matrices: eigenvalues
  to 1e-13 of the largest, residual |A V - V diag(lam)| to 1e-14;
* the biaxial field matrices against the reference's alphaf on its own
  random biaxial voxels (tests/golden/kat_alphaf_biaxial.npz): the forward
  (even) and backward (odd) eigenvalue sets, and the layer operator
  F diag(exp(i kd alpha)) F^-1, which does not depend on the order of the
  modes within a direction or on the scale of each eigenvector, to 1e-12.
"""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def eig4_exe(tmp_path_factory):
    from dtmm_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("eig4") / "eig4_host")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "dtmm_gb300", "csrc"), "-o", exe,
                        os.path.join(HERE, "eig4_host.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _run(exe, mode, records):
    data = np.concatenate([[len(records)], np.asarray(records, np.float64).reshape(-1)]).astype("<f8")
    out = subprocess.run([exe, str(mode)], input=data.tobytes(), capture_output=True, timeout=120)
    assert out.returncode == 0
    return np.frombuffer(out.stdout, "<f8").reshape(len(records), -1)


def _cplx(a):
    return a[..., 0::2] + 1j * a[..., 1::2]


def test_eig4_matches_numpy(eig4_exe):
    rng = np.random.default_rng(5)
    n = 600
    A = rng.normal(size=(n, 4, 4)) + 1j * rng.normal(size=(n, 4, 4))
    A[100:200] = A[100:200].real
    A[200:300] = np.triu(A[200:300])
    A[300:400] = A[300:400] + np.conj(np.swapaxes(A[300:400], 1, 2))
    q, _ = np.linalg.qr(rng.normal(size=(100, 4, 4)) + 1j * rng.normal(size=(100, 4, 4)))
    A[400:500] = q @ np.diag([1.0, 1.0, 2.0, 3.0]).astype(complex) @ np.conj(np.swapaxes(q, 1, 2))
    A[500:510] = 0.0
    o = _run(eig4_exe, 0, np.stack([A.real, A.imag], -1).reshape(n, -1))
    assert np.all(o[:, 0] == 1.0)
    lam = _cplx(o[:, 1:9])
    V = _cplx(o[:, 9:]).reshape(n, 4, 4)
    res = np.linalg.norm(A @ V - V * lam[:, None, :], axis=(1, 2))
    scale = np.linalg.norm(A, axis=(1, 2)) * np.linalg.norm(V, axis=(1, 2))
    assert np.all(res <= 1e-14 * np.maximum(scale, 1e-300))
    ref = np.linalg.eigvals(A)
    for i in range(n):
        rest = list(ref[i])
        for x in lam[i]:
            k = int(np.argmin([abs(x - y) for y in rest]))
            assert abs(x - rest.pop(k)) <= 1e-13 * max(1.0, np.abs(ref[i]).max())


def _operator(alpha, f, kd=1.7):
    return f @ (np.exp(1j * kd * alpha)[..., :, None] * np.linalg.inv(f))


def test_biaxial_fmat_matches_reference(eig4_exe, golden):
    z = golden("kat_alphaf_biaxial")
    ev = z["epsv"]
    rec = np.concatenate([z["beta"][:, None], z["phi"][:, None], np.stack([ev.real, ev.imag], -1).reshape(-1, 6),
                          z["epsa"]], axis=1)
    o = _run(eig4_exe, 1, rec)
    alpha = _cplx(o[:, :8])
    f = _cplx(o[:, 8:]).reshape(-1, 4, 4)
    ra, rf = z["alpha"], z["f"]
    for m in range(len(ra)):
        for par in (0, 1):  # forward (even) and backward (odd) modes as sets
            got = np.sort_complex(alpha[m, par::2])
            want = np.sort_complex(ra[m, par::2])
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    a, b = _operator(alpha, f), _operator(ra, rf)
    err = np.linalg.norm(a - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))
    assert err.max() < 1e-12
