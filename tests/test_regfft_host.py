"""Register line transforms of the CUDA library, checked on the host.

``regfft_host.cu`` includes the library's ``dtmm_regfft.cuh`` (every
function there is __host__ __device__), runs the compile-time twiddles, the
in-register DFTs of 2..32 points and the two-step transform of every line
length that has one (lanes executed one after another, the lane barrier
between the steps) in complex128, and compares them with a direct DFT:
twiddles within 4e-16 of a long-double reference, transforms within 1e-13
relative L2.  Sparse-input DFTs (entries outside a band mask known to be
zero) and the band variants of the two-step inverse transform used by the
row pass are checked the same way.
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_register_transforms_on_host(tmp_path):
    from dtmm_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "regfft_host")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "dtmm_gb300", "csrc"), "-o", exe,
                        os.path.join(HERE, "regfft_host.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    lines = out.stdout.splitlines()
    assert lines[-1] == "OK"
    sizes = {int(l.split()[2]) for l in lines if l.startswith("max_err two_step_fwd")}
    assert {80, 96, 144, 240, 336, 480, 512, 1024} <= sizes
    band = {int(l.split()[2]) // 100 for l in lines if l.startswith("max_err band_line_inv")}
    assert {64, 256, 512, 1024} <= band
    assert any(l.startswith("max_err sparse_dft_fwd") for l in lines)
