"""Oracle fixtures on the benchmark workloads' full grids (fewer layers).

    python tests/golden/make_fullsize.py            # every case
    python tests/golden/make_fullsize.py prec_full  # one case

The oracle (``oracle/dtmm_oracle.py``, complex128, pinned against the
reference's own outputs by ``tests/test_oracle_golden.py``) transfers the
benchmark workloads on their full grids:

  prec_full   4x4, diffraction 3, npass 3, 256 x 256, 9 wavelengths 380-780 nm,
              x + y polarisation, 4 layers (the precision workload has 60)
  twox2_full  2x2, diffraction 5, no reflection, 1024 x 1024, wavelengths
              450 / 550 / 650 nm, x + y polarisation, 2 layers (of 100)

A whole output field is tens to hundreds of MB, so each fixture keeps what a
test needs to compare a full-grid GPU result with it:
  * the output (and, with npass > 1, the rewritten input) at 8192 seeded
    (image, component, y, x) positions;
  * ``NPROJ`` projections of every (image, component) plane on seeded complex
    Gaussian weight fields (sum over the grid of field * weight), which no
    local error escapes;
  * the L2 norm of every (image, component) plane.
The weights are regenerated from their seed by ``projections`` below, which
the GPU test imports.  Inputs are rebuilt from the case record (seeded
director, the product's host illumination restatement).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (HERE, ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

NSAMPLE = 8192
NPROJ = 4

FULL_CASES = {
    "prec_full": dict(shape=(256, 256), nlayers=4, wavelengths=list(np.linspace(380.0, 780.0, 9)), pixelsize=50.0,
                      material=dict(kind="twisted", no=1.52, ne=1.71, amplitude=0.3, seed=1),
                      transfer=dict(method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0)),
    "twox2_full": dict(shape=(1024, 1024), nlayers=2, wavelengths=[450.0, 550.0, 650.0], pixelsize=100.0,
                       material=dict(kind="inplane", no=1.5, ne=1.6, seed=4),
                       transfer=dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)),
}


def build(case):
    """(field_data, optical_data) of a full-size case (host numpy)."""
    from dtmm_gb300 import illumination_data, samples

    m = dict(case["material"])
    kind = m.pop("kind")
    gen = samples.twisted_nematic if kind == "twisted" else samples.inplane_nematic
    od = [gen(case["shape"], case["nlayers"], **m)]
    fd = illumination_data(case["shape"], case["wavelengths"], pixelsize=case["pixelsize"])
    return fd, od


def sample_index(shape, seed=11):
    """Seeded flat indices into a field of ``shape`` (images..., 4, H, W)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.sort(rng.choice(int(np.prod(shape)), size=min(NSAMPLE, int(np.prod(shape))), replace=False))


def projections(field, seed=12):
    """[NPROJ, planes] sums over the grid of every (image, component) plane times
    seeded complex Gaussian weight fields."""
    f = np.asarray(field)
    h, w = f.shape[-2:]
    planes = f.reshape(-1, h, w)
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((NPROJ, planes.shape[0]), np.complex128)
    for k in range(NPROJ):
        wt = rng.standard_normal((h, w)) + 1j * rng.standard_normal((h, w))
        out[k] = np.tensordot(planes, wt, axes=([1, 2], [0, 1]))
    return out


def summarize(field):
    f = np.asarray(field)
    idx = sample_index(f.shape)
    planes = f.reshape(-1, f.shape[-2] * f.shape[-1])
    return dict(idx=idx, values=f.reshape(-1)[idx], proj=projections(f), norms=np.linalg.norm(planes, axis=1))


def run(name):
    import dtmm_oracle as O

    case = FULL_CASES[name]
    O.set_workers(os.cpu_count() or 1)
    fd, od = build(case)
    fin = fd[0].copy()
    t0 = time.time()
    out = O.transfer_field((fin, fd[1], fd[2]), od, **case["transfer"])[0]
    dt = time.time() - t0
    rec = {"shape": np.asarray(out.shape)}
    for k, v in summarize(out).items():
        rec["out_" + k] = v
    if case["transfer"].get("npass", 1) > 1:
        for k, v in summarize(fin).items():
            rec["in_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print("%-12s %7.1fs  out %s" % (name, dt, out.shape))


if __name__ == "__main__":
    for n in sys.argv[1:] or list(FULL_CASES):
        run(n)
