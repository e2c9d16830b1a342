"""director2data on the GPU against the reference's output (4e-15 absolute;
a float32 director against the oracle on the same values, 4e-15), and a
transfer through the device-resident material built from it against the
oracle."""
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
