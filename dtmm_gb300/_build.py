"""In-tree build of the CUDA library (``dtmm_gb300/_lib/libdtmm_gb300.so``).

One translation unit, compiled for sm_103a with nvcc; no CMake, no torch
extension machinery.  The library exports the C ABI of
``include/dtmm_gb300.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libdtmm_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    cand = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), shutil.which("nvcc")]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu")]


def deps():
    return sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")] + [
        os.path.join(ROOT, "include", "dtmm_gb300.h")]


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def up_to_date():
    out = lib_path()
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps())


def build(force=False, verbose=False):
    """Compile the library if a source is newer than it; return its path."""
    out = lib_path()
    if not force and up_to_date():
        return out
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = out + ".tmp.%d" % os.getpid()
    cmd = [nvcc_path(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-I" + os.path.join(ROOT, "include"), "-o", tmp] + sources() + ["-lcudart"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    if verbose:
        print(r.stdout + r.stderr)
    os.replace(tmp, out)
    return out
