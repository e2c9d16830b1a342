"""GPU transfers on the benchmark workloads' full grids against the oracle.

The precision workload (4x4, diffraction 3, npass 3, 256 x 256, 9 wavelengths,
x + y polarisation) and the 2x2 workload (diffraction 5, 1024 x 1024, 3
wavelengths, x + y) run on their full grids with fewer layers (4 and 2) and
are compared with the oracle's complex128 result of the same transfer
(``tests/golden/make_fullsize.py``): at 8192 seeded samples of the output, on
seeded complex projections of every (image, component) plane over the whole
grid, and on every plane's L2 norm; with npass > 1 also the rewritten input.
Tolerances (relative L2): complex128 1e-10, mixed 1e-4.
"""
import numpy as np
import pytest

from make_fullsize import FULL_CASES, build, projections

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-10, "mixed": 1e-4}


def _check(field, z, pre, tol):
    f = np.asarray(field)
    assert tuple(f.shape) == tuple(int(s) for s in z["shape"])
    vals = z[pre + "values"]
    err = np.linalg.norm(f.reshape(-1)[z[pre + "idx"]] - vals) / np.linalg.norm(vals)
    assert err < tol, ("samples", err)
    p = projections(f)
    err = np.linalg.norm(p - z[pre + "proj"]) / np.linalg.norm(z[pre + "proj"])
    assert err < tol, ("projections", err)
    norms = np.linalg.norm(f.reshape(-1, f.shape[-2] * f.shape[-1]), axis=1)
    err = np.abs(norms - z[pre + "norms"]).max() / z[pre + "norms"].max()
    assert err < tol, ("norms", err)


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(FULL_CASES))
def test_full_grid_matches_oracle(name, precision, golden):
    import dtmm_gb300

    case = FULL_CASES[name]
    z = golden(name)
    fd, od = build(case)
    fin = fd[0].copy()
    out = dtmm_gb300.transfer_field((fin, fd[1], fd[2]), od, precision=precision, **case["transfer"])[0]
    _check(out, z, "out_", TOL[precision])
    if "in_idx" in z:
        _check(fin, z, "in_", TOL[precision])
