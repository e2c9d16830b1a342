"""Continuous-batching server (GPU).

Each request's result (transferred field and POM image) must be the same
whether it runs alone or among other
requests of different sizes that overlap it on the device (the server gives
every request its own stream and workspace, so the results are expected to
be bit-identical; the stated tolerance is the mixed-precision one, rel. L2
1e-4).  The mixed run must really overlap requests, admission must respect
the HBM budget, and one served result is checked against the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _specs(n=8, seed=11):
    from dtmm_gb300 import samples

    return samples.instance_specs(n, seed=seed, sides=(64, 160), layers=(3, 8), nwavelengths=(1, 4), rays=None)


def test_results_alone_equal_results_in_the_mix():
    import torch

    from dtmm_gb300.serve import Request, TransferServer

    specs = _specs()
    mixed = TransferServer(max_active=4, keep_results=True, hbm_budget=8e9)
    reqs = [Request(i, s, 0.0) for i, s in enumerate(specs)]
    st = mixed.serve(reqs)
    assert st["peak_active"] > 1
    assert all(r.finished is not None and r.latency >= 0 for r in reqs)
    for i, s in enumerate(specs):
        alone = TransferServer(max_active=1, keep_results=True)
        r = Request(0, s, 0.0)
        alone.serve([r])
        a = r.result.to(torch.complex128).numpy()
        b = reqs[i].result.to(torch.complex128).numpy()
        assert np.all(np.isfinite(a))
        assert rel(b, a) <= TOL
        assert torch.equal(r.result, reqs[i].result)
        # the request's POM image too
        assert r.image is not None and r.image.shape == tuple(s["shape"]) + (3,)
        assert torch.equal(r.image, reqs[i].image)


def test_budget_limits_admission():
    from dtmm_gb300.serve import Request, TransferServer

    specs = _specs(6, seed=12)
    srv = TransferServer(max_active=6, keep_results=False)
    big = max(srv.footprint(s) for s in specs)
    srv.hbm_budget = big * 1.01
    reqs = [Request(i, s, 0.0) for i, s in enumerate(specs)]
    st = srv.serve(reqs)
    assert st["peak_budget_bytes"] <= srv.hbm_budget
    assert all(r.finished is not None for r in reqs)
    # a request that can never fit is refused up front
    srv.hbm_budget = big * 0.5
    with pytest.raises(ValueError):
        srv.serve([Request(0, specs[int(np.argmax([srv.footprint(s) for s in specs]))], 0.0)])


def test_poisson_trace_and_statistics():
    from dtmm_gb300.serve import TransferServer, poisson_trace

    specs = _specs(20, seed=13)
    trace = poisson_trace(specs, rate=100.0, seed=1)
    assert trace[0].arrival == 0.0 and all(b.arrival >= a.arrival for a, b in zip(trace, trace[1:]))
    srv = TransferServer(max_active=4)
    st = srv.serve(trace)
    assert st["requests"] == 20
    assert st["latency_ms"]["p99"] >= st["latency_ms"]["p50"] > 0
    assert st["updates"] == sum(r.updates for r in trace)
    assert all(r.finished >= r.admitted >= r.arrival for r in trace)


def test_served_result_matches_oracle():
    import torch

    import dtmm_oracle as oracle
    from dtmm_gb300 import illumination_data, samples
    from dtmm_gb300.serve import Request, TransferServer

    s = _specs(1, seed=14)[0]
    srv = TransferServer(max_active=2, keep_results=True)
    r = Request(0, s, 0.0)
    srv.serve([r])
    fd = illumination_data(s["shape"], s["wavelengths"], pixelsize=s["pixelsize"])
    od = [samples.twisted_nematic(s["shape"], s["nlayers"], seed=s["seed"])]
    ref = oracle.transfer_field(fd, od, method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)[0]
    assert rel(r.result.to(torch.complex128).numpy(), ref) < TOL
