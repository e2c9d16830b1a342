"""The no-allocation entry point against the regular one, through the C ABI.

Some callers cannot allocate device memory when they call the engine: plugin
hosts that hand it only their own input and output buffers and keep every
other allocation to themselves, and latency-bound loops where a cudaMalloc
could synchronise or fail.  They call ``dtmm_transfer_noalloc``, whose
workspace is the library's static device scratch.

Both entry points run the same kernels in the same order, so their results
must be bit-identical.  Checked here, in both precisions:
  * a 4x4 transfer (diffraction 3, npass 3, so the caller's input is rewritten
    too) through the no-allocation entry point, then a different transfer
    (2x2 on another grid) in the same scratch, then the first one again: all
    three equal the regular entry point's results bit for bit, so no call
    depends on what the previous one left in the scratch;
  * a second call on the same stream changes the device's free memory by
    nothing (the first call on a stream creates that stream's side stream);
  * an npass > 1 transfer whose every-layer operator cache would not fit the
    scratch runs with the two alternating operator buffers instead;
  * a transfer too large for the scratch is refused with both sizes named.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _io(lib_mod, fin, fout):
    io = lib_mod.TransferIO()
    io.field_in = fin.data_ptr()
    io.field_out = fout.data_ptr()
    io.out_given = 0
    io.bulk = None
    return io


def _regular(plan, f0):
    import torch

    fin = f0.clone()
    fout = torch.empty_like(f0)
    plan.run(fin, fout)
    torch.cuda.synchronize()
    return fin, fout


def _noalloc(lib, lib_mod, plan, f0, stream):
    import torch

    fin = f0.clone()
    fout = torch.full_like(f0, float("nan"))
    rc = lib.dtmm_transfer_noalloc(ctypes.byref(plan.desc), ctypes.byref(_io(lib_mod, fin, fout)),
                                   ctypes.c_void_p(stream))
    assert rc == 0, lib_mod.last_error()
    torch.cuda.synchronize()
    return fin, fout


def _plans(precision):
    import torch

    from dtmm_gb300 import illumination_data, samples
    from dtmm_gb300.transfer import plan_transfer

    out = []
    shape = (24, 30)
    fd = illumination_data(shape, [450.0, 600.0], pixelsize=50.0)
    od = [samples.twisted_nematic(shape, 4, no=1.52, ne=1.71, amplitude=0.3, seed=1)]
    p = plan_transfer(fd[0].shape, fd[1], fd[2], od, method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0,
                      precision=precision)
    out.append((p, torch.from_numpy(fd[0]).to(p.device).to(p.dtype)))
    shape = (20, 16)
    fd = illumination_data(shape, [520.0], pixelsize=100.0, beta=0.1, phi=0.3)
    od = [samples.twisted_nematic(shape, 3, seed=2)]
    p = plan_transfer(fd[0].shape, fd[1], fd[2], od, method="2x2", diffraction=1, beta=0.1, phi=0.3,
                      precision=precision)
    out.append((p, torch.from_numpy(fd[0]).to(p.device).to(p.dtype)))
    return out


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_noalloc_matches_regular_entry_point(precision):
    import torch

    from dtmm_gb300 import _lib

    lib = _lib.load()
    (pa, fa), (pb, fb) = _plans(precision)
    stream = torch.cuda.current_stream(pa.device).cuda_stream
    ra_in, ra_out = _regular(pa, fa)
    rb_in, rb_out = _regular(pb, fb)
    for plan, f0, r_in, r_out in ((pa, fa, ra_in, ra_out), (pb, fb, rb_in, rb_out), (pa, fa, ra_in, ra_out)):
        fin, fout = _noalloc(lib, _lib, plan, f0, stream)
        assert torch.all(torch.isfinite(torch.view_as_real(fout)))
        assert torch.equal(fout, r_out)
        assert torch.equal(fin, r_in)


def test_noalloc_allocates_nothing():
    import torch

    from dtmm_gb300 import _lib

    lib = _lib.load()
    (pa, fa), _ = _plans("mixed")
    stream = torch.cuda.Stream(device=pa.device)
    with torch.cuda.stream(stream):
        fin = fa.clone()
        fout = torch.empty_like(fa)
    torch.cuda.synchronize()
    io = _io(_lib, fin, fout)
    args = (ctypes.byref(pa.desc), ctypes.byref(io), ctypes.c_void_p(stream.cuda_stream))
    assert lib.dtmm_transfer_noalloc(*args) == 0, _lib.last_error()  # creates this stream's side stream
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(pa.device)
    for _ in range(2):
        assert lib.dtmm_transfer_noalloc(*args) == 0, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(pa.device)
    assert free1 == free0


def test_noalloc_uncached_operators():
    import torch

    from dtmm_gb300 import _lib, illumination_data, samples
    from dtmm_gb300.transfer import plan_transfer

    lib = _lib.load()
    shape = (64, 64)
    fd = illumination_data(shape, [550.0], pixelsize=50.0)
    od = [samples.twisted_nematic(shape, 60, no=1.52, ne=1.71, amplitude=0.3, seed=3)]
    plan = plan_transfer(fd[0].shape, fd[1], fd[2], od, method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0,
                         precision="mixed")
    # every layer's operators: 8 B x 9 windows x 14 records x 64^2 pixels x 60 layers, above the scratch
    assert 8 * 9 * 14 * 64 * 64 * 60 > _lib.STATIC_SCRATCH_BYTES
    f0 = torch.from_numpy(fd[0]).to(plan.device).to(plan.dtype)
    r_in, r_out = _regular(plan, f0)
    stream = torch.cuda.current_stream(plan.device).cuda_stream
    fin, fout = _noalloc(lib, _lib, plan, f0, stream)
    assert torch.equal(fout, r_out)
    assert torch.equal(fin, r_in)


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
