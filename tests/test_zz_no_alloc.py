"""The no-allocation entry point against the regular one, through the C ABI.

Some callers cannot allocate device memory when they call the engine: plugin
hosts that hand it only their own input and output buffers and keep every
other allocation to themselves, and latency-bound loops where a cudaMalloc
could synchronise or fail.  They call ``dtmm_transfer_noalloc``, whose
workspace is the library's static device scratch.  Here both entry points run
the same transfer (4x4, diffraction 3, npass 3, so the caller's input is
rewritten too) and the no-allocation one runs twice in a row; the outputs and
the rewritten inputs must match within the tolerances of the GPU parity tests
(rel. L2 1e-10 for complex128, 1e-4 for the mixed path).  A transfer too large
for the static scratch must be refused with a message naming both sizes.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-10, "mixed": 1e-4}


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_noalloc_matches_regular_entry_point(precision):
    import torch

    from dtmm_gb300 import _lib, illumination_data, samples
    from dtmm_gb300.transfer import plan_transfer

    shape = (24, 30)
    fd = illumination_data(shape, [450.0, 600.0], pixelsize=50.0)
    od = [samples.twisted_nematic(shape, 4, no=1.52, ne=1.71, amplitude=0.3, seed=1)]
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], od, method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0,
                         precision=precision)
    lib = _lib.load()
    dev = plan.device
    f0 = torch.from_numpy(fd[0]).to(dev).to(plan.dtype)
    stream = torch.cuda.current_stream(dev).cuda_stream

    fin = f0.clone()
    fout = torch.empty_like(f0)
    plan.run(fin, fout)  # regular entry point, caller-allocated workspace
    torch.cuda.synchronize()
    ref_out = fout.cpu().numpy()
    ref_in = fin.cpu().numpy()

    for _ in range(2):
        fin = f0.clone()
        fout = torch.full_like(f0, float("nan"))
        io = _lib.TransferIO()
        io.field_in = fin.data_ptr()
        io.field_out = fout.data_ptr()
        io.out_given = 0
        io.bulk = None
        rc = lib.dtmm_transfer_noalloc(ctypes.byref(plan.desc), ctypes.byref(io), ctypes.c_void_p(stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        out = fout.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert rel_l2(out, ref_out) < TOL[precision]
        assert rel_l2(fin.cpu().numpy(), ref_in) < TOL[precision]


def test_noalloc_rejects_oversized_transfer():
    from dtmm_gb300 import _lib

    lib = _lib.load()
    d = _lib.TransferDesc()
    d.height, d.width, d.nlam, d.npol, d.nray = 1024, 1024, 9, 2, 1
    d.method, d.diffraction, d.reflection, d.npass, d.precision = 4, 3, 1, 3, 0
    d.betamax, d.nin, d.nout, d.smooth = 0.8, 1.5, 1.5, 0.1
    th = np.ones(4)
    ns = np.ones(4, np.int32)
    arr = np.zeros(9)
    d.nlayers = 4
    d.thickness = th.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.nstep = ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.ks = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.beta = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.phi = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.epsv = 1
    d.epsa = 1
    io = _lib.TransferIO()
    io.field_in = 1
    io.field_out = 1
    rc = lib.dtmm_transfer_noalloc(ctypes.byref(d), ctypes.byref(io), None)
    assert rc == _lib.DTMM_ENOSPACE
    msg = _lib.last_error()
    assert "static scratch" in msg and str(_lib.STATIC_SCRATCH_BYTES) in msg
