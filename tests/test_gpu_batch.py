"""Batched transfers, device-built inputs, autotuned launch shapes (GPU).

* ``illumination_device`` (the ``dtmm_planewave_field`` kernel) against the
  host ``illumination_data``, which the CPU tests pin to the reference:
  rel. L2 below 1e-13 in complex128 and 1e-6 in complex64.
* ``samples.twisted_nematic_device`` equals the host generator exactly.
* The radix-8 shared-memory schedule against the oracle (complex128, 1e-10).
* A ``TransferBatch`` captured as one CUDA graph and replayed twice gives
  bit-identical results to every plan run alone, and the first instance
  agrees with the oracle within the mixed-precision tolerance (1e-4).
* Autotuned plans: launch shapes (row group, column tile) leave results
  bit-identical; every line-transform schedule agrees with the oracle.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from golden_cases import ILLUM_CASES  # noqa: E402

TOL = {"double": 1e-10, "mixed": 1e-4}


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", sorted(ILLUM_CASES))
def test_planewave_device_matches_host(name, precision):
    import torch

    from dtmm_gb300.illumination import illumination_data, illumination_device

    kw = dict(ILLUM_CASES[name])
    shape, wl, ps = kw.pop("shape"), kw.pop("wavelengths"), kw.pop("pixelsize")
    host = illumination_data(shape, wl, pixelsize=ps, **kw)[0]
    dev = illumination_device(shape, wl, ps, precision=precision, **kw)
    torch.cuda.synchronize()
    got = dev.to(torch.complex128).cpu().numpy()
    assert got.shape == host.shape
    assert rel(got, host) < (1e-13 if precision == "double" else 1e-6)


def test_device_material_matches_host():
    import torch

    from dtmm_gb300 import samples

    d, epsv, epsa = samples.twisted_nematic((40, 48), 5, seed=17)
    mat = samples.twisted_nematic_device((40, 48), 5, seed=17)
    torch.cuda.synchronize()
    assert np.array_equal(mat.epsa.cpu().numpy(), epsa)
    assert np.array_equal(mat.epsv.cpu().numpy(), np.asarray(epsv))
    assert np.array_equal(mat.thickness, d)
    assert mat.ev_strides == (0, 0, 0)


def test_device_material_kernel_matches_host():
    """The one-kernel generator (modes by value, FP64 cosines on the device)
    equals the host generator to FP64 rounding (1e-13 absolute on angles)."""
    import torch

    from dtmm_gb300 import samples

    for shape, nl, seed in (((40, 48), 5, 17), ((64, 96), 3, 4), ((16, 16), 120, 9)):
        d, epsv, epsa = samples.twisted_nematic(shape, nl, seed=seed)
        mat = samples.twisted_nematic_device(shape, nl, seed=seed, host_modes=False)
        torch.cuda.synchronize()
        assert np.abs(mat.epsa.cpu().numpy() - epsa).max() < 1e-13
        assert np.array_equal(mat.epsv.cpu().numpy(), np.asarray(epsv))


@pytest.mark.parametrize("shape", [(48, 40), (64, 72), (96, 64)])
def test_radix8_schedule_matches_oracle(shape):
    import torch

    from dtmm_gb300 import illumination_data, samples
    from dtmm_gb300.transfer import plan_transfer
    import dtmm_oracle as oracle

    fd = illumination_data(shape, [480.0, 620.0], pixelsize=60.0, beta=0.1, phi=0.5)
    od = [samples.twisted_nematic(shape, 3, no=1.52, ne=1.71, amplitude=0.3, seed=3)]
    opts = dict(method="4x4", diffraction=3, npass=3, beta=0.1, phi=0.5)
    f_or = fd[0].copy()
    ref = oracle.transfer_field((f_or, fd[1], fd[2]), od, **opts)[0]
    for sched in (2, 3):
        plan = plan_transfer(fd[0].shape, fd[1], fd[2], od, precision="double", tuning=dict(fft_schedule=sched),
                             **opts)
        fin = torch.from_numpy(fd[0]).cuda()
        fout = torch.empty_like(fin)
        plan.run(fin, fout)
        torch.cuda.synchronize()
        assert rel(fout.cpu().numpy(), ref) < TOL["double"], sched
        assert rel(fin.cpu().numpy(), f_or) < TOL["double"], sched


def _small_specs():
    from dtmm_gb300 import samples

    return samples.instance_specs(4, seed=5, sides=(64, 96), layers=(3, 5), nwavelengths=(1, 3))


def test_batch_graph_replay_matches_single_runs():
    import torch

    from dtmm_gb300 import samples
    from dtmm_gb300.batch import TransferBatch, build_instance
    import dtmm_oracle as oracle

    specs = _small_specs()
    inst = [build_instance(s, precision="mixed") for s in specs]
    alone = []
    for plan, fin, fout in inst:
        plan.run(fin, fout)
        torch.cuda.synchronize()
        alone.append(fout.cpu().clone())
    batch = TransferBatch(nstreams=3)
    for plan, fin, fout in inst:
        fout.fill_(float("nan"))
        batch.add(plan, fin, fout)
    batch.capture()
    for _ in range(2):
        for _, _, fout in inst:
            fout.fill_(float("nan"))
        batch.replay()
        torch.cuda.synchronize()
        for (plan, fin, fout), a in zip(inst, alone):
            assert torch.equal(fout.cpu(), a)
    assert batch.updates == sum(p.updates for p, _, _ in inst)
    # first instance against the oracle (complex128 host inputs)
    from dtmm_gb300 import illumination_data

    s = specs[0]
    fd = illumination_data(s["shape"], s["wavelengths"], pixelsize=s["pixelsize"], beta=s["beta"], phi=s["phi"])
    od = [samples.twisted_nematic(s["shape"], s["nlayers"], seed=s["seed"])]
    ref = oracle.transfer_field(fd, od, method="4x4", diffraction=1, npass=1, beta=s["beta"], phi=s["phi"])[0]
    assert rel(alone[0].to(torch.complex128).numpy(), ref) < TOL["mixed"]


def test_batch_restores_inputs_for_npass_gt_1():
    import torch

    from dtmm_gb300.batch import TransferBatch, build_instance

    spec = _small_specs()[1]
    plan, fin, fout = build_instance(spec, precision="mixed", diffraction=3, npass=3)
    f0 = fin.clone()
    plan.run(fin, fout)
    torch.cuda.synchronize()
    want_out, want_in = fout.cpu().clone(), fin.cpu().clone()
    fin.copy_(f0)
    batch = TransferBatch(nstreams=2)
    batch.add(plan, fin, fout)
    batch.capture()
    for _ in range(2):
        batch.replay()
        torch.cuda.synchronize()
        assert torch.equal(fout.cpu(), want_out)
        assert torch.equal(fin.cpu(), want_in)


def test_tuner_keeps_results():
    import torch

    from dtmm_gb300 import samples
    from dtmm_gb300.batch import build_instance
    from dtmm_gb300.tune import Autotuner, schedules
    from dtmm_gb300 import illumination_data
    import dtmm_oracle as oracle

    spec = dict(_small_specs()[0])
    spec["shape"] = (64, 64)
    tuner = Autotuner(reps=1)
    plan, fin, fout = build_instance(spec, precision="mixed", tuner=tuner)
    assert tuner.lookup(plan) == plan.tuning
    fd = illumination_data(spec["shape"], spec["wavelengths"], pixelsize=spec["pixelsize"], beta=spec["beta"],
                           phi=spec["phi"])
    od = [samples.twisted_nematic(spec["shape"], spec["nlayers"], seed=spec["seed"])]
    ref = oracle.transfer_field(fd, od, method="4x4", diffraction=1, npass=1, beta=spec["beta"],
                                phi=spec["phi"])[0]
    for sched in schedules(plan):
        base = None
        for rg, ct in ((0, 0), (1, 1), (2, 4), (3, 8)):
            plan.set_tuning(fft_schedule=sched, row_group=rg, col_tile=ct)
            fout.fill_(float("nan"))
            plan.run(fin, fout)
            torch.cuda.synchronize()
            out = fout.cpu().clone()
            if base is None:
                base = out
                assert rel(out.to(torch.complex128).numpy(), ref) < TOL["mixed"], sched
            else:
                assert torch.equal(out, base), (sched, rg, ct)


def test_plan_capture_replays_match_eager_run():
    """One transfer (npass 3, so the input is restored inside the graph) as a
    CUDA graph: replays are bit-identical to the eager run."""
    import torch

    from dtmm_gb300.batch import build_instance

    spec = _small_specs()[2]
    plan, fin, fout = build_instance(spec, precision="mixed", diffraction=3, npass=3)
    f0 = fin.clone()
    plan.run(fin, fout)
    torch.cuda.synchronize()
    want_out, want_in = fout.clone(), fin.clone()
    g = plan.capture(fin, fout, restore_from=f0)
    for _ in range(2):
        fout.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(fout, want_out)
        assert torch.equal(fin, want_in)
