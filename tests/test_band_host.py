"""Band variants of the register passes, checked on the host.

``band_host.cu`` includes the library's ``dtmm_regkern.cuh`` and enumerates,
for every side with a register transform and every band limit, the entries
each lane of the band variant chosen by ``row_band_pick`` loads: every entry
inside the band must be among them (the exactness condition of the variants;
the sparse transforms themselves are checked in ``test_regfft_host.py``).
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_band_variants_load_every_in_band_entry(tmp_path):
    from dtmm_gb300 import _build

    try:
        nvcc = _build.nvcc_path()
    except RuntimeError:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "band_host")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "dtmm_gb300", "csrc"), "-I",
                        os.path.join(ROOT, "include"), "-o", exe, os.path.join(HERE, "band_host.cu")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    lines = out.stdout.splitlines()
    assert lines[-1] == "OK"
    tested = {int(l.split()[1]): int(l.split()[2]) for l in lines if l.startswith("checked")}
    assert tested[256] > 0 and tested[1024] > 0
