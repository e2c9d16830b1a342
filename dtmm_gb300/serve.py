"""Continuous-batching transfer server on one GPU.

Requests (seeded 4x4 ``transfer_field`` instances of any supported grid,
layer count and wavelength set) arrive over time.  A single host loop

* admits the oldest waiting request as soon as it has arrived, a stream slot
  is free and its device footprint (material, input and output fields,
  workspace: ``workspace_bytes``) fits in the HBM budget beside the requests
  already running;
* builds the request's state on the device, on the request's own stream:
  the director/angle field (``samples.twisted_nematic_device``), the input
  field (``illumination_device``) and the bound plan, whose launch shapes
  come from the autotuner's cache -- nothing that grows with the grid is
  computed on the host or copied from it;
* enqueues the transfer behind that on the same stream, then the request's
  POM image (x polarizer, crossed analyzer, ``pom.pom_image``), and records an
  event;
* retires finished requests (event query, no blocking), frees their memory
  and slot, and records each latency (finish - arrival).

Requests of different sizes therefore run concurrently on the device, and
new ones join while others are in flight.  Each request has its own
workspace and stream, so its result does not depend on what runs beside it.
"""
from __future__ import annotations

import collections
import time

import numpy as np

from .transfer import plan_transfer, workspace_bytes


class Request:
    __slots__ = ("rid", "spec", "arrival", "admitted", "finished", "footprint", "updates", "result", "image",
                 "_state")

    def __init__(self, rid, spec, arrival):
        self.rid = int(rid)
        self.spec = spec
        self.arrival = float(arrival)
        self.admitted = None
        self.finished = None
        self.footprint = 0
        self.updates = 0
        self.result = None
        self.image = None
        self._state = None

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def poisson_trace(specs, rate, seed=0):
    """Requests for ``specs`` with exponential inter-arrival times (mean 1/rate s)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.cumsum(rng.exponential(1.0 / float(rate), size=len(specs)))
    return [Request(i, s, t[i] - t[0]) for i, s in enumerate(specs)]


class TransferServer:
    """Admit, overlap and retire transfer requests under an HBM budget."""

    def __init__(self, precision="mixed", hbm_budget=150e9, max_active=16, tuner=None, device=None,
                 keep_results=False, npol=2, poll_s=2e-4, pom=True, **options):
        import torch

        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.precision = precision
        self.hbm_budget = float(hbm_budget)
        self.max_active = int(max_active)
        self.tuner = tuner
        self.keep_results = bool(keep_results)
        self.npol = int(npol)
        self.poll_s = float(poll_s)
        self.options = dict(method="4x4", diffraction=1, npass=1)
        self.options.update(options)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(self.max_active)]
        # POM image of every request: x polarizer on the x / y inputs, crossed
        # (y) analyzer, equal-energy transmission colour matching
        self.pom = bool(pom) and self.npol == 2
        if self.pom:
            from .pom import jonesvec, polarizer, ray_jonesmat4x4

            self.pom_jvec = jonesvec((1, 0))
            self.pom_pmat = torch.from_numpy(ray_jonesmat4x4(polarizer(jonesvec((0, 1))))).to(self.device)
        self._cmfs = {}
        self.stats = {}

    def _cmf(self, wavelengths):
        """Colour-matching table of a wavelength set on the device (uploaded once per set)."""
        import torch

        from . import samples

        key = np.asarray(wavelengths, np.float64).tobytes()
        t = self._cmfs.get(key)
        if t is None:
            t = torch.from_numpy(samples.transmission_cmf(wavelengths)).to(self.device)
            # later requests read it from other streams: let the copy land first
            # (the stream is idle apart from it when a request starts)
            torch.cuda.current_stream(self.device).synchronize()
            self._cmfs[key] = t
        return t

    # -- sizes -----------------------------------------------------------
    def footprint(self, spec):
        h, w = spec["shape"]
        nray = 1 if np.ndim(spec["beta"]) == 0 else len(spec["beta"])
        nlam = len(spec["wavelengths"])
        cbytes = 16 if self.precision == "double" else 8
        fields = 2 * nray * self.npol * nlam * 4 * h * w * cbytes
        material = spec["nlayers"] * h * w * 3 * 8
        ws = workspace_bytes(spec["shape"], spec["nlayers"], nlam, self.npol, nray, self.options["method"],
                             self.options["diffraction"], self.options["npass"], 1, self.precision)
        return fields + material + ws

    # -- one request -------------------------------------------------------
    def _start(self, req, slot):
        import torch

        from . import samples
        from .illumination import illumination_device

        s = self.streams[slot]
        spec = req.spec
        with torch.cuda.stream(s):
            # every upload happens here, while the slot's stream is idle: a
            # copy from pageable memory queued behind the transfer would hold
            # the host loop until the transfer finished
            cmf = self._cmf(spec["wavelengths"]) if self.pom else None
            mat = samples.twisted_nematic_device(spec["shape"], spec["nlayers"], seed=spec["seed"],
                                                 device=self.device, host_modes=False)
            jones = None if self.npol == 2 else (1, 0)
            fin = illumination_device(spec["shape"], spec["wavelengths"], spec["pixelsize"], beta=spec["beta"],
                                      phi=spec["phi"], jones=jones, precision=self.precision, device=self.device,
                                      stream=s.cuda_stream)
            plan = plan_transfer(tuple(fin.shape), spec["wavelengths"], spec["pixelsize"], mat, beta=spec["beta"],
                                 phi=spec["phi"], precision=self.precision, device=self.device, **self.options)
            if self.tuner is not None and self.tuner.lookup(plan) is not None:
                self.tuner.tune(plan)
            fout = torch.empty_like(fin)
            plan.run(fin, fout, stream=s.cuda_stream)
            image = None
            if self.pom:
                from .pom import pom_image

                image = pom_image(fout, cmf, self.pom_jvec, self.pom_pmat, stream=s.cuda_stream)
            done = torch.cuda.Event()
            done.record(s)
        req.updates = plan.updates
        req._state = (plan, mat, fin, fout, image, done, slot)

    def _finish(self, req):
        plan, mat, fin, fout, image, done, slot = req._state
        if self.keep_results:
            req.result = fout.cpu()
            req.image = image.cpu() if image is not None else None
        req._state = None
        return slot

    # -- the loop ----------------------------------------------------------
    def serve(self, requests):
        """Run a trace (requests sorted by arrival, seconds from start); return statistics."""
        import torch

        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            r.footprint = self.footprint(r.spec)
            if r.footprint > self.hbm_budget:
                raise ValueError("request %d needs %.1f GB, above the HBM budget" % (r.rid, r.footprint / 1e9))
        pending = collections.deque(reqs)
        active = []
        free = list(range(self.max_active))
        used = 0.0
        peak_used = 0.0
        peak_active = 0
        host_s = 0.0  # host time spent building and enqueueing requests
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while pending or active:
            now = time.perf_counter() - t0
            progressed = False
            still = []
            for r in active:
                if r._state[5].query():
                    r.finished = time.perf_counter() - t0
                    free.append(self._finish(r))
                    used -= r.footprint
                    progressed = True
                else:
                    still.append(r)
            active = still
            while (pending and pending[0].arrival <= now and free
                   and used + pending[0].footprint <= self.hbm_budget):
                r = pending.popleft()
                r.admitted = time.perf_counter() - t0
                self._start(r, free.pop())
                host_s += time.perf_counter() - t0 - r.admitted
                used += r.footprint
                active.append(r)
                progressed = True
            peak_used = max(peak_used, used)
            peak_active = max(peak_active, len(active))
            if not progressed:
                wait = self.poll_s
                if pending and not active:
                    wait = max(0.0, min(pending[0].arrival - now, 0.01))
                time.sleep(wait)
        torch.cuda.synchronize(self.device)
        wall = time.perf_counter() - t0
        lat = np.asarray([r.latency for r in reqs]) * 1e3
        ups = float(sum(r.updates for r in reqs))
        self.stats = dict(
            requests=len(reqs), wall_s=wall, updates=ups, updates_per_s=ups / wall,
            requests_per_s=len(reqs) / wall,
            latency_ms=dict(p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)),
                            mean=float(lat.mean()), max=float(lat.max())),
            queue_ms=dict(p50=float(np.percentile([(r.admitted - r.arrival) * 1e3 for r in reqs], 50)),
                          p99=float(np.percentile([(r.admitted - r.arrival) * 1e3 for r in reqs], 99))),
            peak_active=peak_active, peak_budget_bytes=peak_used, host_enqueue_s=host_s,
            arrival_span_s=float(reqs[-1].arrival - reqs[0].arrival) if reqs else 0.0,
        )
        return self.stats


def pretune(tuner, specs, precision="mixed", device=None, npol=2, **options):
    """Fill the tuner's cache for every distinct grid of ``specs`` (2-layer proxies)."""
    import torch

    from . import samples
    from .illumination import illumination_device

    seen = set()
    opts = dict(method="4x4", diffraction=1, npass=1)
    opts.update(options)
    for spec in specs:
        nray = 1 if np.ndim(spec["beta"]) == 0 else len(spec["beta"])
        key = (spec["shape"], nray)
        if key in seen:
            continue
        seen.add(key)
        sub = dict(spec, nlayers=2, wavelengths=np.linspace(400.0, 700.0, 9))
        mat = samples.twisted_nematic_device(sub["shape"], 2, seed=sub["seed"], device=device, host_modes=False)
        fin = illumination_device(sub["shape"], sub["wavelengths"], sub["pixelsize"], beta=sub["beta"],
                                  phi=sub["phi"], jones=None if npol == 2 else (1, 0), precision=precision,
                                  device=device)
        plan = plan_transfer(tuple(fin.shape), sub["wavelengths"], sub["pixelsize"], mat, beta=sub["beta"],
                             phi=sub["phi"], precision=precision, device=device, **opts)
        tuner.tune(plan)
        del plan, mat, fin
    torch.cuda.synchronize(device)
    return tuner


__all__ = ["TransferServer", "Request", "poisson_trace", "pretune"]
