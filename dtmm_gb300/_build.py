"""In-tree build of the CUDA library (``dtmm_gb300/_lib/libdtmm_gb300.so``).

Every ``csrc/*.cu`` unit is compiled for sm_103a with nvcc in parallel (one
process per unit), then linked into one shared library; no CMake, no torch
extension machinery.  The library exports the C ABI of
``include/dtmm_gb300.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

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
    return sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "dtmm_gb300.h")]


# per-file options: the Q-tensor eigensolver rounds every sum and product
# separately, as the double arithmetic it restates does
FILE_FLAGS = {"dtmm_qdata.cu": ["-fmad=false"]}


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
    objdir = os.path.join(LIBDIR, "obj.%d" % os.getpid())
    os.makedirs(objdir, exist_ok=True)
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]
    if verbose:
        flags.insert(0, "-Xptxas=-v")
    srcs = sources()
    objs = [os.path.join(objdir, os.path.basename(f)[:-3] + ".o") for f in srcs]

    def compile_one(i):
        extra = FILE_FLAGS.get(os.path.basename(srcs[i]), [])
        return subprocess.run([nvcc_path()] + flags + extra + ["-c", srcs[i], "-o", objs[i]], capture_output=True,
                              text=True)

    jobs = max(1, min(len(srcs), os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(compile_one, range(len(srcs))))
    log = "".join(r.stdout + r.stderr for r in results)
    bad = [srcs[i] for i, r in enumerate(results) if r.returncode != 0]
    if bad:
        shutil.rmtree(objdir, ignore_errors=True)
        raise RuntimeError("nvcc failed on %s:\n%s" % (", ".join(os.path.basename(b) for b in bad), log))
    tmp = out + ".tmp.%d" % os.getpid()
    r = subprocess.run([nvcc_path(), ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"], capture_output=True,
                       text=True)
    shutil.rmtree(objdir, ignore_errors=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout + r.stderr)
    if verbose:
        print(log)
    os.replace(tmp, out)
    return out
