"""Engine vs the oracle over grid shapes: power-of-two rows 64..1024 (the
register-transform row kernel), odd and mixed-radix 7-smooth sides (the generic
kernels), non-square grids.  Tolerances: 1e-10 (complex128), 1e-4 (mixed)."""
import numpy as np
import pytest

import dtmm_gb300
import dtmm_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-10, "mixed": 1e-4}

SHAPES = [
    ((32, 64), dict(method="4x4", diffraction=3, npass=2, beta=0.05, phi=0.3)),
    ((16, 128), dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
    ((8, 256), dict(method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0)),
    ((4, 512), dict(method="2x2", diffraction=3, reflection=0, beta=0.1, phi=0.2)),
    ((4, 1024), dict(method="2x2", diffraction=1, beta=0.0, phi=0.0)),
    ((4, 1024), dict(method="4x4", diffraction=1, beta=0.0, phi=0.0)),
    ((30, 42), dict(method="4x4", diffraction=3, npass=1, beta=0.0, phi=0.0)),
    ((27, 35), dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)),
    # tall grids: the register-transform column pass
    ((128, 16), dict(method="4x4", diffraction=3, npass=2, beta=0.0, phi=0.0)),
    ((256, 8), dict(method="4x4", diffraction=1, npass=1, beta=0.1, phi=0.5)),
    ((512, 6), dict(method="2x2", diffraction=3, reflection=0, beta=0.0, phi=0.0)),
    ((1024, 4), dict(method="4x4", diffraction=1, npass=3, beta=0.0, phi=0.0)),
    ((256, 256), dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
]


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("idx", range(len(SHAPES)))
def test_engine_matches_oracle_on_shape(idx, precision):
    shape, kw = SHAPES[idx]
    fd = dtmm_gb300.illumination_data(shape, [480.0, 620.0], pixelsize=60.0, beta=kw.get("beta", 0.0),
                                      phi=kw.get("phi", 0.0))
    od = [dtmm_gb300.samples.twisted_nematic(shape, 3, no=1.5, ne=1.65, amplitude=0.3, seed=idx)]
    f_ref = fd[0].copy()
    ref = O.transfer_field((f_ref, fd[1], fd[2]), od, **kw)[0]
    f_gpu = fd[0].copy()
    out = dtmm_gb300.transfer_field((f_gpu, fd[1], fd[2]), od, precision=precision, **kw)[0]
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < TOL[precision], err
    if kw.get("npass", 1) > 1:
        assert np.linalg.norm(f_gpu - f_ref) / np.linalg.norm(f_ref) < TOL[precision]
