"""Many independent transfers as one CUDA graph.

A ``TransferBatch`` holds bound ``DevicePlan`` objects (material, workspace
and fields resident on the device) and launches all of them as one graph: the
instances are spread over ``nstreams`` streams, longest first onto the least
loaded stream, so that small grids run beside large ones and the GPU stays
full, and the whole fork/join is captured once (``capture``) and replayed
with a single launch (``replay``).  Every instance keeps its own workspace,
so the instances share nothing and each result equals the one the plan gives
alone.

``build_instance`` binds one seeded workload spec (``samples.instance_specs``)
with its material and input field built on the device.
"""
from __future__ import annotations

import numpy as np

from .transfer import plan_transfer


class _Item:
    __slots__ = ("plan", "fin", "fout", "src", "cost", "stream", "tag")

    def __init__(self, plan, fin, fout, src, cost, tag):
        self.plan, self.fin, self.fout, self.src, self.cost, self.tag = plan, fin, fout, src, cost, tag
        self.stream = 0


class TransferBatch:
    """A set of device transfers launched together (eagerly or as one CUDA graph)."""

    def __init__(self, nstreams=2, device=None):
        import torch

        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.nstreams = int(nstreams)
        self.items = []
        self.graph = None
        self._streams = None

    def add(self, plan, field_in, field_out, tag=None, cost=None):
        """Add a bound plan with its device input and output fields.

        With npass > 1 the engine rewrites ``field_in``; the batch then keeps
        a pristine copy and restores it at the start of every launch, so
        repeated launches compute the same transfer.
        """
        if self.graph is not None:
            raise RuntimeError("batch already captured")
        src = field_in.clone() if plan.desc.npass > 1 else None
        self.items.append(_Item(plan, field_in, field_out, src, float(cost or plan.updates), tag))
        return len(self.items) - 1

    @property
    def updates(self):
        return sum(it.plan.updates for it in self.items)

    def _assign(self):
        import torch

        load = [0.0] * self.nstreams
        for it in sorted(self.items, key=lambda i: -i.cost):
            k = int(np.argmin(load))
            it.stream = k
            load[k] += it.cost
        if self._streams is None:
            self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.nstreams)]
        return load

    def _enqueue(self, origin):
        """Fork from ``origin``, run every item on its stream, join back into ``origin``."""
        import torch

        used = sorted({it.stream for it in self.items})
        for k in used:
            self._streams[k].wait_stream(origin)
        for it in sorted(self.items, key=lambda i: -i.cost):
            s = self._streams[it.stream]
            if it.src is not None:
                with torch.cuda.stream(s):
                    it.fin.copy_(it.src)
            it.plan.run(it.fin, it.fout, stream=s.cuda_stream)
        for k in used:
            origin.wait_stream(self._streams[k])

    def run_eager(self):
        """Launch every transfer now (no graph) on the batch's streams."""
        import torch

        self._assign()
        self._enqueue(torch.cuda.current_stream(self.device))

    def capture(self, warm=True):
        """Capture the whole batch into one CUDA graph.

        With ``warm`` one eager launch runs first, so that kernel attributes
        and lazy module loading happen outside the capture; pass False when
        every plan has already run once.
        """
        import torch

        self._assign()
        origin = torch.cuda.current_stream(self.device)
        if warm:
            self._enqueue(origin)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream(device=self.device)
        with torch.cuda.graph(g, stream=cs, capture_error_mode="relaxed"):
            self._enqueue(cs)
        torch.cuda.synchronize(self.device)
        self.graph = g
        return g

    def replay(self):
        """One launch of the captured graph on the current stream."""
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()


def build_instance(spec, precision="mixed", device=None, tuner=None, nstep=1, **options):
    """Bind one workload spec: device material, device input field, plan.

    ``options`` are transfer options (method, diffraction, npass, ...;
    default 4x4, diffraction 1, npass 1).  Returns ``(plan, field_in,
    field_out)``; with a ``tuner`` the plan carries its tuned launch shapes.
    """
    import torch

    from . import samples
    from .illumination import illumination_device
    from .tune import proxy_plan_device

    dev = device or torch.device("cuda", torch.cuda.current_device())
    opts = dict(method="4x4", diffraction=1, npass=1)
    opts.update(options)
    mat = samples.twisted_nematic_device(spec["shape"], spec["nlayers"], seed=spec["seed"], device=dev)
    fin = illumination_device(spec["shape"], spec["wavelengths"], spec["pixelsize"], beta=spec["beta"],
                              phi=spec["phi"], precision=precision, device=dev)
    plan = plan_transfer(tuple(fin.shape), spec["wavelengths"], spec["pixelsize"], mat, beta=spec["beta"],
                         phi=spec["phi"], nstep=nstep, precision=precision, device=dev, **opts)
    if tuner is not None:
        if tuner.lookup(plan) is None:
            tuner.tune(plan, proxy_plan_device(plan, mat, spec, precision, dev, nstep=nstep, **opts))
        else:
            tuner.tune(plan)
    fout = torch.empty_like(fin)
    return plan, fin, fout


__all__ = ["TransferBatch", "build_instance"]
