"""Autotuner for the engine's launch shapes and line-transform schedule.

The engine exposes three knobs per transfer (``DevicePlan.set_tuning``):

* ``fft_schedule`` -- how each row/column line is transformed: 1 = the
  two-step register transform (power-of-two sides 64..1024, complex64),
  2 = shared-memory mixed-radix passes with radix 4 first, 3 = the same with
  radix 8 first (fewer passes through shared memory for sides divisible by 8);
* ``row_group`` -- wavelengths per row block (lines resident per block);
* ``col_tile`` -- columns per column block.

``row_group`` and ``col_tile`` only change how the work is cut into blocks,
so results are bit-identical across them; the schedules agree to rounding.

``Autotuner.tune(plan)`` times candidates on a short proxy transfer with the
same grid and image axes (a few layers of the plan's own material) and keeps
the fastest, by coordinate descent: schedule first, then row group, then
column tile.  Results are cached per key (grid, method, precision, windows,
fields per wavelength) in memory and, optionally, in a JSON file.
"""
from __future__ import annotations

import json
import os

import numpy as np

# sides with a register line transform (the library's reg_lanes table); for
# sides that are not powers of two it covers real operator records only
SIDES_REG = (64, 80, 96, 112, 128, 144, 160, 192, 224, 240, 256, 288, 320, 336, 384, 400, 432, 448, 480, 512, 1024)


def tuning_key(plan):
    d = plan.desc
    return "%dx%d/m%d/%s/d%d/f%d" % (d.height, d.width, d.method, plan.precision,
                                     max(1, d.diffraction), d.npol * d.nray)


def schedules(plan):
    d = plan.desc
    out = []
    if plan.precision != "double" and (d.height in SIDES_REG or d.width in SIDES_REG):
        out.append(1)
    out.append(2)
    if d.height % 8 == 0 or d.width % 8 == 0:
        out.append(3)
    return out


class Autotuner:
    """Pick ``fft_schedule``, ``row_group`` and ``col_tile`` per transfer shape."""

    def __init__(self, path=None, reps=3, proxy_layers=2):
        self.path = path
        self.reps = int(reps)
        self.proxy_layers = int(proxy_layers)
        self.cache = {}
        self.timings = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.cache = {k: dict(v) for k, v in json.load(f).items()}

    def save(self):
        if self.path:
            tmp = self.path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(self.cache, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)

    def lookup(self, plan):
        return self.cache.get(tuning_key(plan))

    def _time(self, plan, fin, fout, cfg, stream):
        import torch

        plan.set_tuning(**cfg)
        with torch.cuda.stream(stream):
            plan.run(fin, fout, stream=stream.cuda_stream)  # warm-up (tables, attributes)
            best = float("inf")
            for _ in range(self.reps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                plan.run(fin, fout, stream=stream.cuda_stream)
                b.record(stream)
                b.synchronize()
                best = min(best, a.elapsed_time(b))
        return best

    def tune(self, plan, proxy=None):
        """Set the best known tuning on ``plan`` (timing ``proxy`` if not cached).

        ``proxy`` is a DevicePlan of the same grid and image axes, normally a
        few layers of the same material (``proxy_plan``); without one the
        plan itself is timed.  Returns the chosen tuning.
        """
        import torch

        key = tuning_key(plan)
        if key in self.cache:
            plan.set_tuning(**self.cache[key])
            return dict(self.cache[key])
        target = proxy if proxy is not None else plan
        d = target.desc
        shape = target.field_shape
        g = torch.Generator(device="cpu").manual_seed(1234)
        host = torch.randn(shape + (2,), generator=g, dtype=torch.float64)
        fin0 = torch.view_as_complex(host).to(target.device).to(target.dtype)
        fin = fin0.clone()
        fout = torch.empty_like(fin0)
        stream = torch.cuda.Stream(device=target.device)
        times = {}

        def measure(cfg):
            k = (cfg["fft_schedule"], cfg["row_group"], cfg["col_tile"])
            if k not in times:
                fin.copy_(fin0)
                times[k] = self._time(target, fin, fout, cfg, stream)
            return times[k]

        best = {"fft_schedule": 0, "row_group": 0, "col_tile": 0}
        cands = schedules(target)
        best["fft_schedule"] = min(cands, key=lambda s: measure(dict(best, fft_schedule=s)))
        groups = [0] + [gg for gg in (1, 2, 3, 4, 6, 8) if gg <= d.nlam]
        best["row_group"] = min(groups, key=lambda gg: measure(dict(best, row_group=gg)))
        tiles = [0, 1, 2, 4, 8] + ([16] if best["fft_schedule"] != 1 else [])
        best["col_tile"] = min(tiles, key=lambda t: measure(dict(best, col_tile=t)))
        torch.cuda.synchronize(target.device)
        self.cache[key] = dict(best)
        self.timings[key] = {"%d/%d/%d" % k: v for k, v in times.items()}
        plan.set_tuning(**best)
        if target is not plan:
            target.set_tuning(**best)
        return dict(best)


def proxy_plan(field_shape, wavelengths, pixelsize, optical_block, layers=2, **options):
    """A DevicePlan over the first ``layers`` layers of ``optical_block``."""
    from .transfer import plan_transfer

    d, epsv, epsa = optical_block
    n = min(int(layers), len(d))
    sub = (np.asarray(d)[:n], np.asarray(epsv)[:n] if np.ndim(epsv) >= 4 else epsv,
           np.asarray(epsa)[:n] if np.ndim(epsa) >= 4 else epsa)
    return plan_transfer(field_shape, wavelengths, pixelsize, [sub], **options)


def proxy_plan_device(plan, mat, spec, precision, device, layers=2, **options):
    """A DevicePlan over the first ``layers`` layers of a ``DeviceMaterial``."""
    from .transfer import DeviceMaterial, plan_transfer

    n = min(int(layers), mat.nlayers)
    sub = DeviceMaterial(mat.thickness[:n], mat.epsv[:n], mat.epsa[:n], spec["shape"])
    return plan_transfer(plan.field_shape, spec["wavelengths"], spec["pixelsize"], sub, beta=spec["beta"],
                         phi=spec["phi"], precision=precision, device=device, **options)


__all__ = ["Autotuner", "tuning_key", "proxy_plan", "proxy_plan_device", "schedules"]
