"""Engine vs the oracle over grid shapes: sides with register transforms
(powers of two 64..1024 and 7-smooth multiples of 16 up to 480: the complex64
path), odd and other mixed-radix sides (the shared-memory kernels), sides with
prime factors 11..31, tiny sides, non-square grids.  Tolerances: 1e-10
(complex128), 1e-4 (mixed)."""
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
    # register transforms of 7-smooth sides (the complex64 path)
    ((80, 112), dict(method="4x4", diffraction=3, npass=2, beta=0.05, phi=0.3)),
    ((144, 96), dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
    ((160, 192), dict(method="2x2", diffraction=3, reflection=0, beta=0.0, phi=0.0)),
    ((240, 224), dict(method="4x4", diffraction=1, npass=1, beta=0.1, phi=0.5)),
    ((288, 336), dict(method="4x4", diffraction=3, npass=1, beta=0.0, phi=0.0)),
    ((384, 320), dict(method="2x2", diffraction=1, beta=0.0, phi=0.0)),
    ((400, 432), dict(method="4x4", diffraction=1, npass=3, beta=0.0, phi=0.0)),
    ((480, 448), dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
    # sides with prime factors from 11 to 31 (generic prime butterflies) and tiny sides
    ((22, 26), dict(method="4x4", diffraction=3, npass=2, beta=0.05, phi=0.3)),
    ((33, 17), dict(method="2x2", diffraction=3, reflection=0, beta=0.0, phi=0.0)),
    ((38, 46), dict(method="4x4", diffraction=1, npass=1, beta=0.1, phi=0.5)),
    ((29, 31), dict(method="4x4", diffraction=1, npass=3, beta=0.0, phi=0.0)),
    ((3, 4), dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
    ((2, 13), dict(method="2x2", diffraction=1, beta=0.0, phi=0.0)),
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



@pytest.mark.parametrize("shape", [(64, 1024), (1024, 64)])
def test_2x2_diffraction5_long_sides(shape):
    """The 2x2 diffraction-5 kernels on 1024-long rows / columns against the oracle."""
    import torch

    from dtmm_gb300.transfer import plan_transfer

    fd = dtmm_gb300.illumination_data(shape, [550.0], pixelsize=100.0)
    od = [dtmm_gb300.samples.inplane_nematic(shape, 2, no=1.5, ne=1.6, seed=4)]
    opts = dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)
    ref = O.transfer_field((fd[0].copy(), fd[1], fd[2]), od, **opts)[0]
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], od, precision="mixed", **opts)
    f = torch.from_numpy(fd[0]).cuda().to(plan.dtype)
    out = torch.empty_like(f)
    plan.run(f, out)
    torch.cuda.synchronize()
    got = out.to(torch.complex128).cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < TOL["mixed"]


def test_2x2_full_grid_properties():
    """The 1024x1024 2x2 diffraction-5 workload on its full grid (2 of its 100
    layers, one wavelength): linearity in the input field, and equivariance
    under a circular shift of material and field (the transfer is periodic),
    both exact up to rounding whatever the grid size."""
    import torch

    from dtmm_gb300.transfer import plan_transfer

    shape = (1024, 1024)
    fd = dtmm_gb300.illumination_data(shape, [550.0], pixelsize=100.0)
    d, epsv, epsa = dtmm_gb300.samples.inplane_nematic(shape, 2, no=1.5, ne=1.6, seed=4)
    opts = dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], [(d, epsv, epsa)], precision="mixed", **opts)
    f = torch.from_numpy(fd[0]).cuda().to(plan.dtype)
    # break the plane wave's translation symmetry so that the shift test means something
    yy = torch.arange(shape[0], device="cuda")[:, None]
    xx = torch.arange(shape[1], device="cuda")[None, :]
    f = (f * (1.0 + 0.3 * torch.cos(2 * np.pi * (3 * xx / shape[1] + 5 * yy / shape[0])))).contiguous()
    out = torch.empty_like(f)
    plan.run(f, out)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(torch.view_as_real(out)).all())
    # linearity: T(a f1 + b f2) = a T(f1) + b T(f2), f1/f2 the x/y-polarised inputs
    a, b = 0.6 - 0.3j, -0.2 + 0.9j
    mix = (a * f[0] + b * f[1])[None].contiguous()
    o1 = torch.empty_like(mix)
    plan1 = plan_transfer(mix.shape, fd[1], fd[2], [(d, epsv, epsa)], precision="mixed", **opts)
    plan1.run(mix, o1)
    torch.cuda.synchronize()
    lin = a * out[0] + b * out[1]
    assert float(torch.linalg.vector_norm(o1[0] - lin) / torch.linalg.vector_norm(lin)) < 1e-5
    # shift equivariance
    sy, sx = 37, 501
    es = np.roll(epsa, (sy, sx), axis=(1, 2))
    plan2 = plan_transfer(fd[0].shape, fd[1], fd[2], [(d, epsv, es)], precision="mixed", **opts)
    fs = torch.roll(f, (sy, sx), dims=(-2, -1)).contiguous()
    o2 = torch.empty_like(fs)
    plan2.run(fs, o2)
    torch.cuda.synchronize()
    want = torch.roll(out, (sy, sx), dims=(-2, -1))
    assert float(torch.linalg.vector_norm(o2 - want) / torch.linalg.vector_norm(want)) < 1e-5
