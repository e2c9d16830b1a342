"""The library's FP64 -> FP32 conversion in integer arithmetic (used where
FP64 results are stored as FP32), checked on the host bit for bit against
the IEEE round-to-nearest-even conversion (``cvt_host.cu``): 18 million
random patterns, exact ties and their neighbours, range edges, zeros,
infinities and NaN."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_f32_rn_matches_ieee_conversion(tmp_path):
    from dtmm_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "cvt_host")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "dtmm_gb300", "csrc"), "-o", exe,
                        os.path.join(HERE, "cvt_host.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    assert out.stdout.splitlines()[-1] == "OK"
