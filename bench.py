#!/usr/bin/env python3
"""Throughput of dtmm's transfer_field hot path on GB300.

Workload (the precision configuration of the reference's benchmark set):
4x4 method, npass = 3 (reflections), diffraction = 3 (9 mode windows),
256 x 256 grid, 60 layers of 1 pixel, 50 nm pixels, 9 wavelengths
380-780 nm, x and y polarisations at normal incidence, seeded twisted nematic
(no 1.52, ne 1.71, 8-mode perturbation of amplitude 0.3 rad), complex64 bulk
with the FP64 eigen-solve.  One step = one whole transfer_field of that
workload; the unit is voxel x wavelength updates (H*W*layers*lambdas*
polarisations*passes = 2.12e8 per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` times steps with inputs resident in HBM
(CUDA events, L2 flushed between steps); `e2e` times the drop-in call on
host numpy buffers (pinned), host<->device copies included.  The reference
arm (`--impl reference`) times the CPU restatement of the reference's
algorithm (numba is not installable here, so the reference's own numba path
cannot run) on the host cores over a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel·λ updates/s vs plain c128 GPU at ≤1e-4 err; served p50/p99 latency"
UNIT = "voxel·λ updates/s"
SHAPE = (256, 256)
NLAYERS = 60
WAVELENGTHS = np.linspace(380.0, 780.0, 9)
PIXELSIZE = 50.0
OPTS = dict(method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0)
# bytes that one voxel.lambda update must move at least: one read and one write of
# the 4-component complex64 field, plus the 48-byte material record amortised
# over the 9 wavelengths x 2 polarisations that share it
BYTES_PER_UPDATE = 2 * 4 * 8 + 48.0 / (len(WAVELENGTHS) * 2)
CONFIG = {
    "workload": "transfer_field 4x4 npass=3 diffraction=3, 256x256 grid, 60 layers, 9 wavelengths 380-780 nm, "
                "x+y polarisation, twisted nematic (no 1.52, ne 1.71, amp 0.3), complex64 bulk + FP64 eigen-solve",
    "grid": "256x256", "layers": 60, "wavelengths": 9, "polarisations": 2, "passes": 3, "windows": 9,
    "l2": "flushed between timed steps (256 MiB write)",
}


def inputs(nlayers=NLAYERS):
    from dtmm_gb300 import illumination_data, samples

    fd = illumination_data(SHAPE, WAVELENGTHS, pixelsize=PIXELSIZE)
    od = [samples.twisted_nematic(SHAPE, nlayers, no=1.52, ne=1.71, amplitude=0.3, seed=1)]
    return fd, od


def updates_of(field, nlayers, npass):
    return int(np.prod(field.shape[:-3])) * field.shape[-2] * field.shape[-1] * nlayers * npass


# ---------------------------------------------------------------------------
# CPU leg: the oracle (CPU restatement of the reference) on a bounded sample
# ---------------------------------------------------------------------------
def cpu_sample_rate():
    """updates/s of the CPU restatement on 1 layer x 1 pass of the same grid, wavelengths and polarisations."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import dtmm_oracle
    from dtmm_gb300 import illumination_data, samples

    cores = len(os.sched_getaffinity(0))
    dtmm_oracle.set_workers(cores)
    fd = illumination_data(SHAPE, WAVELENGTHS, pixelsize=PIXELSIZE)
    od = [samples.twisted_nematic(SHAPE, 1, no=1.52, ne=1.71, amplitude=0.3, seed=1)]
    kw = dict(OPTS)
    kw["npass"] = 1
    t0 = time.perf_counter()
    dtmm_oracle.transfer_field((fd[0].copy(), fd[1], fd[2]), od, **kw)
    dt = time.perf_counter() - t0
    upd = updates_of(fd[0], 1, 1)
    return upd / dt, cores, dt


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        busy = [v for v in sm if mx and v > 0.3 * max(mx)]
        return {"sm_mhz": float(np.median(busy or sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_summary():
    """The committed ncu summary of the dominant kernel ({} if absent)."""
    p = os.path.join(ROOT, "profiles", "layer_row_traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def ncu_traffic():
    """DRAM bytes per launch of the dominant kernel, from the committed ncu summary (None if absent)."""
    return ncu_summary().get("dram_bytes_per_launch_full")


# ---------------------------------------------------------------------------
def run_reference(args, rank):
    """Reference arm: every step is one bounded sample of the workload (1 of the
    60 layers, 1 of the 3 passes, the full grid, every wavelength and
    polarisation) through the CPU restatement on all host cores; value and
    ms_per_step are that sample's own, nothing is extrapolated."""
    if rank != 0:
        return
    times = []
    for i in range(args.warmup + args.steps):
        rate, cores, dt = cpu_sample_rate()
        if i >= args.warmup:
            times.append(dt)
    upd = SHAPE[0] * SHAPE[1] * len(WAVELENGTHS) * 2  # one layer, one pass
    ms = float(np.mean(times)) * 1e3
    value = upd / (ms / 1e3)
    sample = ("each step: 1 of 60 layers x 1 of 3 passes of the workload (full 256x256 grid, 9 wavelengths, "
              "2 polarisations) = %d updates" % upd)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "updates_per_step": upd, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic", "config": CONFIG,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference's algorithm (numpy/scipy, complex128, oracle/dtmm_oracle.py); the "
                "reference's numba path needs numba, which is not installed on this image",
    }))


# ---------------------------------------------------------------------------
# batching: 48 heterogeneous instances as one CUDA graph
# ---------------------------------------------------------------------------
def field_bytes_per_update(nlam, nfields, cbytes=8):
    return 2 * 4 * cbytes + 48.0 / (nlam * nfields)


def time_replays(fn, steps, dev):
    stream = torch_mod().cuda.current_stream(dev)
    times = []
    for _ in range(steps):
        e0 = torch_mod().cuda.Event(enable_timing=True)
        e1 = torch_mod().cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times


def torch_mod():
    import torch

    return torch


def run_batch(args, dev, ninst=48, seed=0):
    import torch

    from dtmm_gb300 import samples
    from dtmm_gb300.batch import TransferBatch, build_instance
    from dtmm_gb300.tune import Autotuner

    specs = samples.instance_specs(ninst, seed=seed)
    tuner = Autotuner()
    t0 = time.perf_counter()
    inst = [build_instance(s, precision="mixed", device=dev, tuner=tuner) for s in specs]
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    batch = TransferBatch(nstreams=args.streams, device=dev)
    for (plan, fin, fout), s in zip(inst, specs):
        batch.add(plan, fin, fout, tag=s["index"])
    # one eager pass, one instance at a time: the library's kernel launches
    # and device time per kernel family, grouped by grid side
    launches = 0
    by_side = {}
    for (plan, fin, fout), s in zip(inst, specs):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        kt = plan.run(fin, fout, timed=True)
        e1.record()
        e1.synchronize()
        launches += kt.total_launches
        b = by_side.setdefault(str(s["shape"][0]), {"instances": 0, "updates": 0, "ms": 0.0, "row_ms": 0.0,
                                                      "col_ms": 0.0, "op_ms": 0.0, "tuning": plan.tuning})
        b["instances"] += 1
        b["updates"] += plan.updates
        b["ms"] += e0.elapsed_time(e1)
        b["row_ms"] += kt.layer_row_ms
        b["col_ms"] += kt.layer_col_ms
        b["op_ms"] += kt.voxel_op_ms
    for b in by_side.values():
        b["updates_per_s_alone"] = b["updates"] / (b["ms"] / 1e3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.capture(warm=False)
    capture_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        batch.replay()
    torch.cuda.synchronize()
    with ClockSampler(dev.index or 0) as clk:
        times = time_replays(batch.replay, args.steps, dev)
    clocks = clk.summary()
    ms = float(np.mean(times))
    upd = batch.updates
    value = upd / (ms / 1e3)
    alg_bytes = sum(p.updates * field_bytes_per_update(len(s["wavelengths"]), 14) for (p, _, _), s in zip(inst, specs))
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    in_bytes = sum(fin.numel() * fin.element_size() for _, fin, _ in inst)
    # one graph launch vs the same plans launched one after another on one stream
    def serial():
        for plan, fin, fout in inst:
            plan.run(fin, fout)
    serial()
    torch.cuda.synchronize()
    serial_ms = float(np.mean(time_replays(serial, 1, dev)))
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic",
        "config": {"workload": "batch: %d seeded 4x4 transfer_field instances (diffraction 1, npass 1) as one CUDA "
                               "graph; grids log-uniform 64-512 rounded to 7-smooth multiples of 16, 20-120 "
                               "layers, 1-9 wavelengths in 400-700 nm, 7 rays (beta 0, +-0.1, +-0.2 at phi 0; "
                               "+-0.1 at phi 90 deg), x+y polarisation, twisted nematic (no 1.5, ne 1.7, amp 0.2), "
                               "complex64 bulk + FP64 eigen-solve, autotuned launch shapes" % ninst,
                   "instances": ninst, "streams": args.streams,
                   "l2": "inputs larger than L2 (%.1f GB of input fields)" % (in_bytes / 1e9)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "whole graph (algorithmic bytes / graph time)",
                     "peak_source": peak_kind},
        "gpu_launches": launches * args.steps, "clocks": clocks, "updates_per_step": upd,
        "graph": {"build_s": build_s, "capture_s": capture_s, "serial_one_stream_ms": serial_ms,
                  "graph_speedup_vs_serial": serial_ms / ms, "by_side": by_side},
    }
    # end to end: host inputs in pinned memory, copies in, one graph launch, copies out
    if not args.no_e2e:
        hin = [torch.empty(fin.shape, dtype=fin.dtype).pin_memory() for _, fin, _ in inst]
        hout = [torch.empty(fout.shape, dtype=fout.dtype).pin_memory() for _, _, fout in inst]
        for h, (_, fin, _) in zip(hin, inst):
            h.copy_(fin)
        def e2e_step():
            for h, (_, fin, _) in zip(hin, inst):
                fin.copy_(h, non_blocking=True)
            batch.replay()
            for h, (_, _, fout) in zip(hout, inst):
                h.copy_(fout, non_blocking=True)
        e2e_step()
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            e2e_step()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        e2e_s = float(np.median(ts))
        result["e2e"] = {"value": upd / e2e_s, "unit": UNIT, "h2d_bytes_per_step": in_bytes,
                         "d2h_bytes_per_step": in_bytes, "ms_per_step": e2e_s * 1e3}
    # complex128 comparison on a seeded subset (the full batch in complex128 takes minutes)
    if not args.no_c128:
        sub = specs[:args.c128_subset]
        res = {}
        outs = {}
        for prec in ("mixed", "double"):
            ii = [build_instance(s, precision=prec, device=dev) for s in sub]
            b = TransferBatch(nstreams=args.streams, device=dev)
            for plan, fin, fout in ii:
                b.add(plan, fin, fout)
            b.capture()
            b.replay()
            torch.cuda.synchronize()
            t = float(np.mean(time_replays(b.replay, 1, dev)))
            res[prec] = b.updates / (t / 1e3)
            outs[prec] = [fout.to(torch.complex128).cpu().numpy() for _, _, fout in ii]
            del ii, b
            torch.cuda.empty_cache()
        err = max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(outs["mixed"], outs["double"]))
        result["c128"] = {"subset": len(sub), "value": res["double"], "mixed_value": res["mixed"],
                          "mixed_speedup": res["mixed"] / res["double"], "mixed_rel_l2_vs_c128_max": err}
    return result


# ---------------------------------------------------------------------------
# 2x2 method, memory-bound sweep: 1024x1024, 100 layers, 3 wavelengths, 25 windows
# ---------------------------------------------------------------------------
def run_2x2(args, dev):
    import torch

    from dtmm_gb300 import samples
    from dtmm_gb300.illumination import illumination_device
    from dtmm_gb300.transfer import plan_transfer

    shape, nl = (1024, 1024), args.layers if args.layers != NLAYERS else 100
    wl = np.asarray([450.0, 550.0, 650.0])
    d, epsv, epsa = samples.inplane_nematic(shape, nl, no=1.5, ne=1.6, seed=4)
    opts = dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)
    fin = illumination_device(shape, wl, 100.0, precision="mixed", device=dev)
    plan = plan_transfer(tuple(fin.shape), wl, 100.0, [(d, epsv, epsa)], precision="mixed", device=dev, **opts)
    fout = torch.empty_like(fin)
    graph = plan.capture(fin, fout)  # npass 1: the input is not rewritten
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    times, kts = [], []
    stream = torch.cuda.current_stream(dev)
    with ClockSampler(dev.index or 0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            graph.replay()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    clocks = clk.summary()
    for _ in range(args.steps):  # per-kernel breakdown: eager runs with events
        flush.zero_()
        kts.append(plan.run(fin, fout, timed=True))
    ms = float(np.mean(times))
    upd = plan.updates
    nf = int(np.prod(fin.shape[:-3])) // len(wl)
    bpu = 2 * 2 * 8 + 48.0 / (len(wl) * nf)
    peak, peak_kind = measured_peaks()
    row_ms = sum(k.layer_row_ms for k in kts)
    row_n = sum(k.layer_row_launches for k in kts)
    per_launch = int(np.prod(fin.shape[:-3])) * shape[0] * shape[1]
    achieved_row = bpu * per_launch / (row_ms / row_n / 1e3) / 1e9
    return {
        "metric": METRIC, "value": upd / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": "transfer_field 2x2, diffraction 5 (25 windows), no reflection, 1024x1024 grid, "
                               "%d layers, 100 nm pixels, wavelengths 450/550/650 nm, x+y polarisation, in-plane "
                               "nematic (16-mode azimuth, ne 1.6, no 1.5), complex64 bulk + FP64 eigen-solve" % nl,
                   "l2": "flushed between timed steps (256 MiB write); fields (100 MB) are near L2 size"},
        "roofline": {"bound": "hbm", "achieved": achieved_row, "peak": peak, "unit": "GB/s",
                     "frac": achieved_row / peak, "traffic": None, "peak_source": peak_kind,
                     "kernel": "k_layer_row_reg (2x2, 1024-point rows, 25 windows)",
                     "bytes_per_update": bpu,
                     "step_achieved": bpu * upd / (ms / 1e3) / 1e9,
                     "device_ms_per_step": {"layer_row": row_ms / args.steps,
                                            "layer_col": sum(k.layer_col_ms for k in kts) / args.steps,
                                            "voxel_op": sum(k.voxel_op_ms for k in kts) / args.steps}},
        "gpu_launches": sum(k.total_launches for k in kts), "clocks": clocks, "updates_per_step": upd,
    }


# ---------------------------------------------------------------------------
# the plain method: 4x4, diffraction 1, npass 1, 64x64, 20 layers, 550 nm
# ---------------------------------------------------------------------------
def run_plain(args, dev):
    """The plain workload in complex128 (its stated precision) and mixed; one
    step = one transfer replayed from a CUDA graph, L2 flushed between steps.
    Launch-bound at this size (81,920 updates per step)."""
    import torch

    from dtmm_gb300 import illumination_data, samples
    from dtmm_gb300.transfer import plan_transfer

    shape, nl, wl = (64, 64), 20, [550.0]
    fd = illumination_data(shape, wl, pixelsize=100.0, jones=(1, 0))
    od = [samples.twisted_nematic(shape, nl, no=1.5, ne=1.7, amplitude=0.2, seed=0)]
    opts = dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    peak, peak_kind = measured_peaks()
    out = {"workload": "transfer_field 4x4, diffraction 1, npass 1, 64x64 grid, 20 layers, 100 nm pixels, 550 nm, "
                       "x polarisation, twisted nematic (no 1.5, ne 1.7, amp 0.2)"}
    for prec in ("double", "mixed"):
        plan = plan_transfer(fd[0].shape, fd[1], fd[2], od, precision=prec, device=dev, **opts)
        fin = torch.from_numpy(fd[0]).to(dev).to(plan.dtype).contiguous()
        fout = torch.empty_like(fin)
        graph = plan.capture(fin, fout)
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            graph.replay()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        kts = [plan.run(fin, fout, timed=True) for _ in range(2)]
        ms = float(np.mean(times))
        cb = 16 if prec == "double" else 8
        bpu = 2 * 4 * cb + 48.0
        row_ms = sum(k.layer_row_ms for k in kts) / sum(k.layer_row_launches for k in kts)
        per_launch = shape[0] * shape[1]
        achieved = bpu * per_launch / (row_ms / 1e3) / 1e9
        out["c128" if prec == "double" else "mixed"] = {
            "value": plan.updates / (ms / 1e3), "ms_per_step": ms,
            "roofline": {"bound": "hbm", "kernel": "row pass (%s)" % ("k_layer_row" if prec == "double"
                                                                      else "k_layer_row_reg"),
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "bytes_per_update": bpu, "peak_source": peak_kind},
            "gpu_launches_per_step": kts[-1].total_launches}
        del graph, plan, fin, fout
    out["unit"] = UNIT
    return out


# ---------------------------------------------------------------------------
# the rows either side of the transfer: POM image, refocus, director / Q-tensor
# -> optical data; each timed alone on inputs larger than L2
# ---------------------------------------------------------------------------
def run_rows(args, dev, cpu=True):
    import torch

    only = None if getattr(args, "rows", "all") == "all" else set(args.rows.split(","))

    from dtmm_gb300 import data, pom, samples

    O = None
    if cpu:  # the oracle, for the CPU baseline legs only
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import dtmm_oracle as O
    peak, peak_kind = measured_peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    def cpu_rate(fn, items):
        t0 = time.perf_counter()
        fn()
        return items / (time.perf_counter() - t0)

    def row(name, workload, items, unit, nbytes, ms, launches, cpu_value, cpu_sample, cores=1):
        gbs = nbytes / (ms / 1e3) / 1e9
        out = {"workload": workload, "value": items / (ms / 1e3), "unit": unit, "ms_per_call": ms,
               "gpu_launches_per_call": launches,
               "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                            "bytes_per_call": nbytes, "peak_source": peak_kind}}
        if cpu_value is not None:
            out["cpu_baseline"] = {"value": cpu_value, "unit": unit, "cores": cores, "kind": "port",
                                   "sample": cpu_sample}
        return name, out

    res = {}
    wl = WAVELENGTHS
    cmf_h = samples.transmission_cmf(wl)
    cmf = torch.from_numpy(cmf_h).to(dev)
    jvec = pom.jonesvec((1, 0))
    pmat_h = pom.ray_jonesmat4x4(pom.polarizer(pom.jonesvec((0, 1))))
    pmat = torch.from_numpy(pmat_h).to(dev)

    def pom_row():
        # POM image: x / y fields of 9 wavelengths on a 1024^2 grid -> sRGB
        H = W = 1024
        f = torch.randn((2, len(wl), 4, H, W), dtype=torch.complex64, device=dev, generator=gen)
        ms = timed(lambda: pom.pom_image(f, cmf, jvec, pmat, stream=stream.cuda_stream))
        nbytes = f.numel() * 8 + H * W * 3 * 4
        cv = None
        if cpu:
            fh = f[:, :, :, :512, :512].cpu().numpy().astype(np.complex128)
            cv = cpu_rate(lambda: O.specter2color(O.field2specter(O.calculate_pom_field(fh, jvec, pmat_h)), cmf_h),
                          512 * 512 * len(wl))
        res.update([row("pom_image", "POM image (x polarizer, crossed analyzer, sRGB) of x+y fields, 9 "
                                     "wavelengths, 1024x1024 grid, complex64", H * W * len(wl), "pixel·λ/s", nbytes,
                        ms, 1, cv, "same pipeline, 512x512 crop, oracle (numpy; FFTs on every core, the rest on one)",
                        os.cpu_count() or 1)])

    def diffract_row():
        # refocus: fft2, per-k 4x4 matrix, ifft2 of x+y fields, 9 wavelengths, 512^2
        H = W = 512
        f = torch.randn((2, len(wl), 4, H, W), dtype=torch.complex64, device=dev, generator=gen)
        ks = 2 * np.pi / wl * PIXELSIZE
        dm = pom.field_diffraction_matrix((H, W), ks, d=-20.0, epsv=(1.5 ** 2,) * 3, device=dev)
        ms = timed(lambda: pom.diffract(f, dm))
        nbytes = 2 * f.numel() * 8 + dm.numel() * 16
        cv = None
        if cpu:
            fh = f[:, :, :, :256, :256].cpu().numpy().astype(np.complex128)
            dmh = pom.field_diffraction_matrix((256, 256), ks, d=-20.0, epsv=(1.5 ** 2,) * 3)
            cv = cpu_rate(lambda: O.diffract(fh, dmh), 2 * 256 * 256 * len(wl))
        res.update([row("diffract", "refocus by -20 px in n=1.5 (fft2, per-k 4x4 matrix, ifft2) of x+y fields, "
                                    "9 wavelengths, 512x512 grid, complex64 fields, complex128 matrices",
                        2 * H * W * len(wl), "pixel·λ/s", nbytes, ms, 6, cv,
                        "same refocus, 256x256 grid, oracle (scipy fft on every core, matrices on one)",
                        os.cpu_count() or 1)])

    def director_row():
        # director -> optical data: 128 layers of 512^2
        L, H, W = 128, 512, 512
        d = torch.randn((L, H, W, 3), dtype=torch.float64, device=dev, generator=gen)
        ms = timed(lambda: data.director2data(d, no=1.52, ne=1.71))
        nvox = L * H * W
        cv = None
        if cpu:
            dh = d[:32, :256, :256].cpu().numpy()
            cv = cpu_rate(lambda: O.director2data(dh, no=1.52, ne=1.71), dh.size // 3)
        res.update([row("director2data", "director2data, 128x512x512 float64 directors", nvox, "voxel/s",
                        nvox * (24 + 48), ms, 1, cv, "32x256x256 directors, oracle (numpy)")])

    def q_row():
        # Q tensor -> optical data: 64 layers of 512^2, uniaxial Q of random directors and orders
        L, H, W = 64, 512, 512
        n = torch.randn((L, H, W, 3), dtype=torch.float64, device=dev, generator=gen)
        n = n / n.norm(dim=-1, keepdim=True)
        S = torch.rand((L, H, W), dtype=torch.float64, device=dev, generator=gen) * 0.7 + 0.2
        q = torch.stack([S * (n[..., 0] ** 2 - 1 / 3), S * (n[..., 1] ** 2 - 1 / 3), S * (n[..., 2] ** 2 - 1 / 3),
                         S * n[..., 0] * n[..., 1], S * n[..., 0] * n[..., 2], S * n[..., 1] * n[..., 2]], dim=-1)
        del n, S
        ms = timed(lambda: data.Q2data(q, no=1.52, ne=1.71))
        nvox = L * H * W
        cv = None
        if cpu:
            qh = q[:4, :64, :64].cpu().numpy()
            cv = cpu_rate(lambda: O.Q2data(qh, no=1.52, ne=1.71), qh.size // 6)
        name, r = row("q2data", "Q2data (uniaxial), 64x512x512 float64 Q tensors", nvox, "voxel/s",
                      nvox * (48 + 48), ms, 1, cv, "4x64x64 Q tensors, oracle (per-voxel Python, 1 core)")
        r["roofline"]["note"] = ("FP64-bound: one eigen-solve (acos, 2 cos, 3 sqrt, divides) and 2 atan2 + acos "
                                 "per voxel")
        res[name] = r

    for name, fn in (("pom_image", pom_row), ("diffract", diffract_row), ("director2data", director_row),
                     ("q2data", q_row)):
        if only is None or name in only:
            fn()
            torch.cuda.empty_cache()
    torch.cuda.synchronize(dev)
    return res


# ---------------------------------------------------------------------------
# serving: Poisson stream of requests, continuous batching under an HBM budget
# ---------------------------------------------------------------------------
def run_serve(args, dev):
    import torch

    from dtmm_gb300 import samples
    from dtmm_gb300.serve import TransferServer, poisson_trace, pretune
    from dtmm_gb300.tune import Autotuner

    specs = samples.instance_specs(args.requests, seed=1, rays=None)
    tuner = Autotuner()
    t0 = time.perf_counter()
    pretune(tuner, specs, device=dev)
    tune_s = time.perf_counter() - t0
    # warm-up: a few requests through the same server (allocator pools, lazy loading)
    srv = TransferServer(precision="mixed", hbm_budget=args.hbm_budget, max_active=args.slots, tuner=tuner,
                         device=dev)
    srv.serve(poisson_trace(specs[:min(16, len(specs))], args.rate, seed=2))
    torch.cuda.synchronize()
    trace = poisson_trace(specs, args.rate, seed=3)
    with ClockSampler(dev.index or 0) as clk:
        st = srv.serve(trace)
    clocks = clk.summary()
    offered = sum(samples.spec_updates(s) for s in specs) / max(st["arrival_span_s"], 1e-9)
    return {
        "metric": METRIC, "value": st["updates_per_s"], "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": st["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic",
        "config": {"workload": "serving: Poisson stream of %d POM simulation requests at %g req/s, each a 4x4 "
                               "transfer_field (diffraction 1, npass 1, normal incidence, x+y polarisation) and its "
                               "crossed-polarizer sRGB image, grids log-uniform 64-512, 20-120 layers, 1-9 "
                               "wavelengths, twisted nematic built on the device, complex64 bulk + FP64 eigen-solve; "
                               "continuous batching over %d stream slots, %g GB HBM admission budget"
                               % (args.requests, args.rate, args.slots, args.hbm_budget / 1e9),
                   "requests": args.requests, "rate": args.rate, "slots": args.slots,
                   "hbm_budget_bytes": args.hbm_budget},
        "latency_ms": st["latency_ms"], "queue_ms": st["queue_ms"], "requests_per_s": st["requests_per_s"],
        "offered_updates_per_s": offered, "peak_active": st["peak_active"],
        "peak_budget_bytes": st["peak_budget_bytes"], "host_enqueue_s": st["host_enqueue_s"], "pretune_s": tune_s,
        "clocks": clocks,
    }


def _g(d, *keys):
    for k in keys:
        if not isinstance(d, dict) or k not in d:
            return None
        d = d[k]
    return d


def _r(x, n=4):
    return None if x is None else float("%.*g" % (n, x))


def summary(res):
    """The line's key figures in a few hundred characters, printed last so that
    a reader of the line's tail sees them: the headline and its kernel, the
    complex128 comparison, the 2x2 and plain workloads, batch and serving."""
    s = {"precision_mixed": {"value": _r(res.get("value")), "ms": _r(res.get("ms_per_step")),
                             "row_frac": _r(_g(res, "roofline", "frac"), 3),
                             "e2e": _r(_g(res, "e2e", "value"))},
         "c128": {"value": _r(_g(res, "c128", "value")), "mixed_speedup": _r(_g(res, "c128", "mixed_speedup"), 3),
                  "mixed_rel_l2_vs_c128": _r(_g(res, "c128", "mixed_rel_l2_vs_c128"), 3)},
         "twox2": {"value": _r(_g(res, "twox2", "value")), "ms": _r(_g(res, "twox2", "ms_per_step")),
                   "row_gbs": _r(_g(res, "twox2", "roofline", "achieved")),
                   "row_frac": _r(_g(res, "twox2", "roofline", "frac"), 3),
                   "row_ms": _r(_g(res, "twox2", "roofline", "device_ms_per_step", "layer_row")),
                   "op_ms": _r(_g(res, "twox2", "roofline", "device_ms_per_step", "voxel_op"))},
         "plain": {"c128": _r(_g(res, "plain", "c128", "value")), "mixed": _r(_g(res, "plain", "mixed", "value")),
                   "c128_ms": _r(_g(res, "plain", "c128", "ms_per_step"))},
         "batch": {"value": _r(_g(res, "batch", "value")), "e2e": _r(_g(res, "batch", "e2e", "value")),
                   "launches": _g(res, "batch", "gpu_launches")},
         "serve": {"rps": _r(_g(res, "serve", "requests_per_s")), "p50_ms": _r(_g(res, "serve", "latency_ms", "p50")),
                   "p99_ms": _r(_g(res, "serve", "latency_ms", "p99"))},
         "cpu": _r(_g(res, "cpu_baseline", "value"))}
    return s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-c128", action="store_true", help="skip the complex128 comparison run")
    ap.add_argument("--layers", type=int, default=NLAYERS, help="layers (profiling runs use fewer; same kernels)")
    ap.add_argument("--npass", type=int, default=OPTS["npass"])
    ap.add_argument("--workload", default="precision", choices=["precision", "batch", "serve", "2x2", "rows"],
                    help="precision: 256x256 4x4 npass 3 (default); batch: 48 instances in one graph; "
                         "serve: Poisson request stream; 2x2: 1024x1024 2x2 diffraction 5; rows: POM image, "
                         "refocus, director2data and Q2data kernels")
    ap.add_argument("--streams", type=int, default=2, help="batch: streams in the graph")
    ap.add_argument("--c128-subset", type=int, default=8, help="batch: instances of the complex128 comparison")
    ap.add_argument("--requests", type=int, default=2000, help="serve: requests in the trace")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: mean arrival rate (req/s)")
    ap.add_argument("--slots", type=int, default=16, help="serve: concurrent request slots")
    ap.add_argument("--hbm-budget", type=float, default=150e9, help="serve: admission budget (bytes)")
    ap.add_argument("--no-batch", action="store_true", help="precision workload: skip the batch summary")
    ap.add_argument("--no-serve", action="store_true", help="precision workload: skip the serving summary")
    ap.add_argument("--rows", default="all",
                    help="rows workload: comma list of pom_image, diffract, director2data, q2data (default all)")
    ap.add_argument("--no-2x2", action="store_true", help="precision workload: skip the 2x2 workload summary")
    ap.add_argument("--no-plain", action="store_true", help="precision workload: skip the plain workload summary")
    ap.add_argument("--no-rows", action="store_true",
                    help="precision workload: skip the POM / refocus / director / Q-tensor kernel summary")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch

    import dtmm_gb300
    from dtmm_gb300.replicas import job_throughput, job_time_ms
    from dtmm_gb300.transfer import plan_transfer

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    dev = torch.device("cuda", local)
    if args.workload == "rows":
        rows = run_rows(args, dev, cpu=not args.no_cpu and rank == 0)
        if rank == 0:
            pi = rows["pom_image"] if "pom_image" in rows else next(iter(rows.values()))
            print(json.dumps({"metric": "POM image pixel·λ/s (with the refocus, director2data and Q2data rows)",
                              "value": pi["value"], "unit": pi["unit"], "n_gpus": 1, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": pi["ms_per_call"], "higher_is_better": True,
                              "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
                              "config": {"workload": pi["workload"], "l2": "flushed between timed calls"},
                              "roofline": pi["roofline"], "cpu_baseline": pi.get("cpu_baseline"),
                              "gpu_launches": args.steps, "rows": rows}))
        if dist is not None:
            dist.destroy_process_group()
        return
    if args.workload in ("batch", "serve", "2x2"):
        # independent replicas: every rank runs the whole workload on its own GPU
        res = {"batch": run_batch, "serve": run_serve, "2x2": run_2x2}[args.workload](args, dev)
        barrier()
        if dist is not None:
            ms_rank = res["ms_per_step"]
            res["ms_per_step"] = job_time_ms(ms_rank, dist, dev)
            # every rank ran the same workload: its units over the slowest rank's time
            res["value"] = job_throughput(res["value"] * ms_rank / 1e3, res["ms_per_step"], world)
            res["n_gpus"] = world
        if rank == 0:
            print(json.dumps(res))
        if dist is not None:
            dist.destroy_process_group()
        return
    fd, od = inputs(args.layers)
    OPTS["npass"] = args.npass
    if args.layers != NLAYERS or args.npass != 3:
        CONFIG["workload"] += " [reduced: %d layers, npass %d]" % (args.layers, args.npass)
        CONFIG["layers"] = args.layers
        CONFIG["passes"] = args.npass
    field_np = fd[0]
    plan = plan_transfer(field_np.shape, fd[1], fd[2], od, precision="mixed", device=dev, **OPTS)
    fin0 = torch.from_numpy(field_np).to(dev).to(plan.dtype).contiguous()
    fin = torch.empty_like(fin0)
    fout = torch.empty_like(fin0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    # one step = the input reset (the transfer rewrites its input, npass > 1)
    # and one transfer, captured once as a CUDA graph and replayed
    graph = plan.capture(fin, fout, restore_from=fin0)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream(dev)
    times = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            graph.replay()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    barrier()
    # per-kernel device time and launch count: the same steps run eagerly
    # with CUDA events around every row / column / operator launch
    ktimes, eager_ms = [], 0.0
    for _ in range(args.steps):
        flush.zero_()
        fin.copy_(fin0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ktimes.append(plan.run(fin, fout, timed=True))
        e1.record(stream)
        e1.synchronize()
        eager_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    clocks = clk.summary()
    total_ms = job_time_ms(float(sum(times)), dist, dev)
    upd = plan.updates
    value = job_throughput(upd * args.steps, total_ms, world)
    out_mixed = fout.to(torch.complex128).cpu().numpy()

    # dominant kernel: the fused row pass
    row_ms = sum(k.layer_row_ms for k in ktimes)
    row_n = sum(k.layer_row_launches for k in ktimes)
    col_ms = sum(k.layer_col_ms for k in ktimes)
    op_ms = sum(k.voxel_op_ms for k in ktimes)
    launches = sum(k.total_launches for k in ktimes)
    upd_per_row_launch = int(np.prod(field_np.shape[:-3])) * SHAPE[0] * SHAPE[1]
    row_avg_s = row_ms / row_n / 1e3
    achieved = BYTES_PER_UPDATE * upd_per_row_launch / row_avg_s / 1e9
    peak, peak_kind = measured_peaks()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(), "kernel": "k_layer_row_reg<float,4,real,16,16>", "peak_source": peak_kind,
                "kernel_share": row_ms / eager_ms,
                "issue_bound": {k: ncu_summary().get(k) for k in ("smsp_issue_active", "sm_pipe_fma_cycles_active",
                                                                   "sm_inst_executed_pipe_lsu", "note")},
                "device_ms_per_step": {"layer_row": row_ms / args.steps, "layer_col": col_ms / args.steps,
                                       "voxel_op": op_ms / args.steps}}

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic", "config": CONFIG, "roofline": roofline, "gpu_launches": launches,
        "clocks": clocks, "wall_s_timed_region": wall, "updates_per_step": upd,
        "step": "CUDA-graph replay of the input reset + one transfer (graph replays are bit-identical to eager runs)",
    }

    # complex128 drop-in on the same workload (the "plain c128 GPU" comparison)
    if not args.no_c128 and rank == 0:
        plan64 = plan_transfer(field_np.shape, fd[1], fd[2], od, precision="double", device=dev, **OPTS)
        f64 = torch.from_numpy(field_np).to(dev).contiguous()
        fi64 = torch.empty_like(f64)
        fo64 = torch.empty_like(f64)
        fi64.copy_(f64)
        plan64.run(fi64, fo64)
        torch.cuda.synchronize()
        fi64.copy_(f64)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        flush.zero_()
        e0.record()
        plan64.run(fi64, fo64)
        e1.record()
        e1.synchronize()
        c128_ms = e0.elapsed_time(e1)
        ref = fo64.cpu().numpy()
        result["c128"] = {"value": upd / (c128_ms / 1e3), "ms_per_step": c128_ms,
                          "mixed_speedup": (upd / (total_ms / args.steps / 1e3)) / (upd / (c128_ms / 1e3)),
                          "mixed_rel_l2_vs_c128": float(np.linalg.norm(out_mixed - ref) / np.linalg.norm(ref))}
        del plan64, f64, fi64, fo64

    # end to end through the drop-in call on host buffers: the field and the
    # director angles in page-locked host memory (the caller's buffers), both
    # copied to the device by every call
    if not args.no_e2e:
        pinned = torch.empty(field_np.shape, dtype=torch.complex128).pin_memory()
        pinned_np = pinned.numpy()
        od_pinned = []
        for d_, ev_, ea_ in od:
            ea_p = torch.empty(np.shape(ea_), dtype=torch.float64).pin_memory().numpy()
            ea_p[...] = ea_
            od_pinned.append((d_, ev_, ea_p))
        e2e = []
        for i in range(1 + args.steps):
            pinned_np[...] = field_np
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = dtmm_gb300.transfer_field((pinned_np, fd[1], fd[2]), od_pinned, precision="mixed", **OPTS)
            torch.cuda.synchronize()
            if i > 0:
                e2e.append(time.perf_counter() - t0)
        e2e_s = float(np.median(e2e))
        fbytes = field_np.size * 16
        mat_bytes = od[0][2].nbytes + 24 + od[0][0].nbytes
        result["e2e"] = {"value": upd / e2e_s, "unit": UNIT, "h2d_bytes_per_step": fbytes + mat_bytes,
                         "d2h_bytes_per_step": 2 * fbytes, "ms_per_step": e2e_s * 1e3}

    # the batching and serving configurations, summarised on the same line
    import copy

    if rank == 0 and not args.no_batch:
        a2 = copy.copy(args)
        a2.steps, a2.warmup, a2.c128_subset = 2, 1, 4
        try:
            b = run_batch(a2, dev)
            result["batch"] = {k: b[k] for k in ("value", "ms_per_step", "config", "roofline", "gpu_launches",
                                                  "clocks", "updates_per_step", "e2e", "c128") if k in b}
            result["batch"]["graph_speedup_vs_serial"] = b["graph"]["graph_speedup_vs_serial"]
        except Exception as e:  # reported, not fatal for the headline line
            result["batch"] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_serve:
        try:
            sv = run_serve(args, dev)
            result["serve"] = {k: sv[k] for k in ("value", "unit", "config", "latency_ms", "queue_ms",
                                                   "requests_per_s", "offered_updates_per_s", "peak_active",
                                                   "peak_budget_bytes", "host_enqueue_s", "ms_per_step", "clocks")
                               if k in sv}
        except Exception as e:
            result["serve"] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_rows:
        try:
            a2 = copy.copy(args)
            a2.steps, a2.warmup = 5, 3
            result["rows"] = run_rows(a2, dev, cpu=not args.no_cpu and world == 1)
        except Exception as e:
            result["rows"] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_2x2:
        try:
            a2 = copy.copy(args)
            a2.steps, a2.warmup, a2.layers = 5, 3, NLAYERS
            t2 = run_2x2(a2, dev)
            result["twox2"] = {k: t2[k] for k in ("value", "ms_per_step", "config", "roofline", "gpu_launches",
                                                   "clocks", "updates_per_step") if k in t2}
        except Exception as e:
            result["twox2"] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_plain:
        try:
            a2 = copy.copy(args)
            a2.steps, a2.warmup = 20, 5
            result["plain"] = run_plain(a2, dev)
        except Exception as e:
            result["plain"] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_cpu and world == 1:
        rate, cores, dt = cpu_sample_rate()
        result["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": "1 of 60 layers, 1 of 3 passes, full 256x256 grid, 9 wavelengths, "
                                            "2 polarisations (%.1f s of CPU work)" % dt}
    if rank == 0:
        result["summary"] = summary(result)
        print(json.dumps(result))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
