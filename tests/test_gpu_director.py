"""director2data and Q2data on the GPU against the reference's output
(director2data 4e-15 absolute; a float32 director against the oracle on the
same values, 4e-15; Q2data tolerances in its test), and transfers through the
device-resident materials built from them against the oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_director2data_matches_reference():
    from dtmm_gb300 import data

    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    th, ev, ea = data.director2data(z["director"])
    assert np.array_equal(th, z["thickness_default"])
    assert np.abs(ev - z["epsv_default"]).max() < 4e-15
    assert np.abs(ea - z["epsa_default"]).max() < 4e-15
    _, ev, ea = data.director2data(z["director"], mask=z["mask"], no=1.52, ne=1.71, nhost=1.4, scale_factor=0.8)
    assert np.abs(ev - z["epsv_masked"]).max() < 4e-15
    assert np.abs(ea - z["epsa_masked"]).max() < 4e-15


def test_director2angles_matches_reference():
    from dtmm_gb300 import data

    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    ea = data.director2angles(z["director"])
    assert np.abs(ea - z["epsa_default"]).max() < 4e-15


def test_float32_director():
    import dtmm_oracle as O
    from dtmm_gb300 import data

    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    d32 = z["director"].astype(np.float32)
    _, ev, ea = data.director2data(d32, mask=z["mask"], no=1.52, ne=1.71, nhost=1.4)
    _, rv, ra = O.director2data(d32.astype(np.float64), mask=z["mask"], no=1.52, ne=1.71, nhost=1.4)
    assert np.abs(ev - rv).max() < 4e-15 and np.abs(ea - ra).max() < 4e-15


def test_transfer_through_device_material():
    import torch

    import dtmm_oracle as O
    from dtmm_gb300 import data, illumination_data
    from dtmm_gb300.transfer import plan_transfer

    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    director = z["director"][:, :, :16]  # 12 x 16 grid, 3 layers
    director[..., 2] += 0.3  # no zero-length voxels: keep the stack uniaxial everywhere
    fd = illumination_data((12, 16), [500.0, 620.0], pixelsize=80.0)
    mat = data.device_material(torch.from_numpy(np.ascontiguousarray(director)).cuda(), no=1.5, ne=1.65)
    opts = dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], mat, precision="double", **opts)
    fin = torch.from_numpy(fd[0]).cuda()
    fout = torch.empty_like(fin)
    plan.run(fin, fout)
    torch.cuda.synchronize()
    od = [O.director2data(director, no=1.5, ne=1.65)]
    ref = O.transfer_field((fd[0].copy(), fd[1], fd[2]), od, **opts)[0]
    got = fout.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-10


def _wrap(d):
    return np.abs((d + np.pi) % (2 * np.pi) - np.pi)


def test_q2data_matches_reference():
    """Q2data on the GPU against the reference's output.  Eigenvalues to
    1e-12 (uniaxial and masked) and the polar angles theta, phi to 1e-10
    everywhere; psi to 1e-10 on layer 1, whose tensors are biaxial.  On
    layer 0 the tensors are exactly uniaxial: psi turns the frame about the
    optic axis and is fixed only by rounding, so there the test rebuilds eps
    from the eigenvalues and angles and compares with the reference's rebuild
    (1e-12).  Biaxial output: layer 1 to 1e-10; on layer 0 the two equal
    eigenvalues come out split by rounding (1e-8), so eigenvalues to 1e-7."""
    import test_director_host as H

    from dtmm_gb300 import data

    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    cases = [("", {}), ("_masked", dict(mask=z["mask"], no=1.52, ne=1.71, nhost=1.4, scale_factor=0.9)),
             ("_biaxial", dict(biaxial=True))]
    for tag, kw in cases:
        th, ev, ea = data.Q2data(z["Q"], **kw)
        rv, ra = z["epsv" + tag], z["epsa" + tag]
        assert np.array_equal(th, np.ones(2))
        d = _wrap(ea - ra)
        if tag == "_biaxial":
            assert np.abs(ev[1] - rv[1]).max() < 1e-10, tag
            assert np.abs(ev[0] - rv[0]).max() < 1e-7, tag
        else:
            assert np.abs(ev - rv).max() < 1e-12, tag
            assert np.abs(H._rebuild(ev, ea)[0] - H._rebuild(rv, ra)[0]).max() < 1e-12, tag
        assert d[..., 1:].max() < 1e-10, tag
        assert d[1, ..., 0].max() < 1e-10, tag


def test_q2data_matrix_input_and_device_tensors():
    """(..., 3, 3) input equals (..., 6) input bit for bit; a device tensor stays on the device."""
    import test_director_host as H
    import torch

    from dtmm_gb300 import data

    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    q6 = z["Q"]
    q33 = H._full(q6)
    a = data.Q2data(q6, biaxial=True)
    b = data.Q2data(q33, biaxial=True)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    c = data.Q2data(torch.from_numpy(q6).cuda())
    assert c[1].is_cuda and c[2].is_cuda
    d = data.Q2data(q6)
    assert np.array_equal(c[1].cpu().numpy(), d[1]) and np.array_equal(c[2].cpu().numpy(), d[2])


def test_transfer_through_q_material():
    """A transfer through the device material built by Q2data against the
    oracle on the oracle's own Q2data block (c128, 1e-10)."""
    import torch

    import dtmm_oracle as O
    from dtmm_gb300 import data, illumination_data
    from dtmm_gb300.transfer import plan_transfer

    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    q = np.ascontiguousarray(np.repeat(z["Q"], 2, axis=2)[:, :, :12])  # 2 layers, 6 x 12
    fd = illumination_data((6, 12), [510.0, 600.0], pixelsize=70.0)
    mat = data.q_material(torch.from_numpy(q).cuda(), no=1.5, ne=1.65)
    opts = dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], mat, precision="double", **opts)
    fin = torch.from_numpy(fd[0]).cuda()
    fout = torch.empty_like(fin)
    plan.run(fin, fout)
    torch.cuda.synchronize()
    od = [O.Q2data(q, no=1.5, ne=1.65)]
    ref = O.transfer_field((fd[0].copy(), fd[1], fd[2]), od, **opts)[0]
    got = fout.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-10


@pytest.mark.parametrize("diffraction", [0, 1])
def test_transfer_through_biaxial_q_material(diffraction):
    """Biaxial Q2data kept on the device, through the general eigen-solve of
    the transfer, against the oracle on the oracle's own biaxial block (c128,
    1e-10; layer 1 of the fixture holds biaxial tensors)."""
    import torch

    import dtmm_oracle as O
    from dtmm_gb300 import data, illumination_data
    from dtmm_gb300.transfer import plan_transfer

    z = np.load(os.path.join(HERE, "golden", "qtensor.npz"))
    q = np.ascontiguousarray(np.repeat(z["Q"], 2, axis=2)[:, :, :12])
    fd = illumination_data((6, 12), [510.0, 600.0], pixelsize=70.0, beta=0.1, phi=0.3)
    mat = data.q_material(torch.from_numpy(q).cuda(), no=1.5, ne=1.65, biaxial=True)
    assert mat.biaxial
    opts = dict(method="4x4", diffraction=diffraction, beta=0.1, phi=0.3)
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], mat, precision="double", **opts)
    fin = torch.from_numpy(fd[0]).cuda()
    fout = torch.empty_like(fin)
    plan.run(fin, fout)
    torch.cuda.synchronize()
    od = [O.Q2data(q, no=1.5, ne=1.65, biaxial=True)]
    ref = O.transfer_field((fd[0].copy(), fd[1], fd[2]), od, **opts)[0]
    got = fout.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-10
