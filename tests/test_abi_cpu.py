"""The C-ABI library builds, loads and validates descriptors without a GPU."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from dtmm_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    import re

    text = open(os.path.join(ROOT, "include", "dtmm_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(dtmm_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert set(declared) == set(_lib.ABI_SYMBOLS)
    out = subprocess.run(["nm", "-D", "--defined-only", _build.lib_path()], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for name in declared:
        assert name in exported, name
        assert getattr(lib, name) is not None


def test_abi_version(lib):
    assert lib.dtmm_abi_version() == _lib.ABI_VERSION == 7


def _desc(**kw):
    d = _lib.TransferDesc()
    d.height, d.width, d.nlam, d.npol, d.nray = 16, 16, 1, 1, 1
    d.method, d.diffraction, d.reflection, d.npass, d.precision = 4, 1, 1, 1, 0
    d.betamax, d.nin, d.nout, d.smooth = 0.8, 1.5, 1.5, 0.1
    th = np.ones(3)
    ns = np.ones(3, np.int32)
    arr = np.zeros(1)
    d._keep = (th, ns, arr)
    d.nlayers = 3
    d.thickness = th.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.nstep = ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    d.ks = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.beta = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.phi = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.epsv = 1
    d.epsa = 1
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_workspace_size_positive_for_valid_desc(lib):
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(_desc())) > 16 * 16 * 4 * 8


@pytest.mark.parametrize("field,value,needle", [
    ("method", 3, "method"),
    ("diffraction", 0, "diffraction"),
    ("reflection", 5, "reflection"),
    ("height", 37, "factor"),
    ("width", 2 * 41, "factor"),
    ("npass", 0, "npass"),
    ("fft_schedule", 4, "tuning"),
    ("diffraction", -2, "diffraction"),
    ("row_group", -1, "tuning"),
    ("col_tile", -2, "tuning"),
])
def test_invalid_descriptors_are_rejected(lib, field, value, needle):
    d = _desc(**{field: value})
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(d)) == 0
    assert needle in _lib.last_error()


def test_local_4x4_descriptor_rules(lib):
    """diffraction 0 is the per-voxel 4x4 transfer: reflection mode 2, npass 1 only."""
    ok = _desc(diffraction=0, reflection=2)
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(ok)) > 0
    for kw in (dict(diffraction=0, reflection=1), dict(diffraction=0, reflection=3)):
        assert lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(**kw))) == 0
    # npass > 1 adds the between-pass projection buffers
    two = _desc(diffraction=0, reflection=2, npass=2)
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(two)) > lib.dtmm_transfer_workspace_size(ctypes.byref(ok))


def test_full_diffraction_descriptor_rules(lib):
    """diffraction = inf (DTMM_DIFFRACTION_FULL): the 4x4 method with any
    reflection mode 1..4 and the 2x2 method with reflection 0 or 2, any npass;
    the workspace holds the mode tables."""
    for r in (1, 2, 3, 4):
        d = _desc(diffraction=_lib.DIFFRACTION_FULL, reflection=r)
        assert lib.dtmm_transfer_workspace_size(ctypes.byref(d)) > 2 * 16 * 16 * 16
    d = _desc(diffraction=_lib.DIFFRACTION_FULL, npass=3)
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(d)) > 0
    for kw in (dict(diffraction=_lib.DIFFRACTION_FULL, reflection=5),
               dict(diffraction=_lib.DIFFRACTION_FULL, method=2, reflection=1)):
        assert lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(**kw))) == 0
    # 2x2: the E field's mode amplitudes, and with npass > 1 every interface's reflected wave
    size2 = lambda **kw: lib.dtmm_transfer_workspace_size(ctypes.byref(
        _desc(method=2, diffraction=_lib.DIFFRACTION_FULL, **kw)))
    s0 = size2(reflection=0)
    assert s0 > 2 * 16 * 16 * 16 and size2(reflection=2) > 0
    assert size2(reflection=2, npass=3) - size2(reflection=2) >= 4 * 16 * 16 * 2 * 8
    assert size2(reflection=0, npass=2) == 0 and "npass" in _lib.last_error()
    assert size2(reflection=1) == 0 and "reflection 0 or 2" in _lib.last_error()
    # one DFT grid row per (image, E component)
    assert size2(reflection=0, npol=2, nlam=16384) == 0 and "32767" in _lib.last_error()


def test_reflection4_descriptor_rules(lib):
    """Reflection mode 4: without diffraction the per-voxel transfer, with
    diffraction the real-space half steps around the corrected field
    diffraction matrix (windows add one field of workspace)."""
    d0 = _desc(diffraction=0, reflection=4)
    d1 = _desc(diffraction=1, reflection=4)
    d3 = _desc(diffraction=3, reflection=4)
    s0, s1, s3 = (lib.dtmm_transfer_workspace_size(ctypes.byref(x)) for x in (d0, d1, d3))
    assert s0 > 0 and s1 > s0 and s3 > s1
    # per-ray window / beam tables: the table slots grow with the rays
    two_rays = _desc(diffraction=1, reflection=4, nray=2)
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(two_rays)) > s1
    # reflection modes 2 and 3 with diffraction take the same real-space path
    for r in (2, 3):
        assert lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(diffraction=1, reflection=r))) == s1


def test_2x2_descriptor_rules(lib):
    """2x2: reflection 0 / 1 in k-space (1 also without diffraction, npass 1),
    reflection 2 and diffraction 0 without reflections in real space; npass >
    1 keeps reflected waves (two outer ones in k-space, one per interface in
    real space); reflection 0 with npass > 1 is the reference's ValueError,
    reflection 1 without diffraction and npass > 1 fails in the reference
    itself and is refused; so is reflection 1 with diffraction = inf."""
    size = lambda **kw: lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(method=2, **kw)))
    k1 = size(reflection=1)
    assert k1 > 0 and size(reflection=0) > 0 and size(reflection=1, diffraction=0) > 0
    assert size(reflection=1, npass=3) > k1  # the two outer reflected waves and the exit state
    r2 = size(reflection=2)
    assert r2 > 0 and size(reflection=0, diffraction=0) > 0
    # every interface (3 layers -> 4) keeps its reflected wave
    assert size(reflection=2, npass=2) - r2 >= 4 * 16 * 16 * 2 * 8
    assert size(reflection=2, diffraction=3) > r2  # window parts
    assert size(reflection=0, npass=2) == 0 and "npass" in _lib.last_error()
    assert size(reflection=1, diffraction=0, npass=2) == 0 and "diffraction" in _lib.last_error()
    assert size(reflection=3) == 0 and "reflection" in _lib.last_error()
    assert size(reflection=1, diffraction=_lib.DIFFRACTION_FULL) == 0


def test_norm_ref_descriptor_rules(lib):
    """norm_ref (the reference's DTMM_NORM_REF, with DTMM_NORM_FFT or alone):
    4x4 with npass > 1 keeps the reference field, its E part and the 2x2
    window / H buffers, and with norm_total ("local") the output medium's
    field matrix and its inverse besides; it is refused with diffraction =
    inf (the reference takes int(diffraction) windows for the reference
    field) and has no effect with npass 1."""
    size = lambda **kw: lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(**kw)))
    a = size(npass=3)
    b = size(npass=3, norm_ref=1)
    assert b - a >= 2 * 16 * 16 * 4 * 8  # a field and two field halves at least
    assert size(npass=1, norm_ref=1) == size(npass=1)
    assert size(npass=3, norm_ref=1, diffraction=_lib.DIFFRACTION_FULL) == 0
    assert "norm_ref" in _lib.last_error()
    c = size(npass=3, norm_total=1)
    assert size(npass=3, norm_total=1, norm_ref=1) - c >= b - a + 2 * 16 * 16
    assert size(npass=3, norm_total=1, norm_ref=1, diffraction=_lib.DIFFRACTION_FULL) == 0


def test_norm_total_field(lib):
    """norm_total (the reference's norm = 0) needs no workspace of its own."""
    a = lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(npass=3)))
    b = lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(npass=3, norm_total=1)))
    assert a == b > 0


def test_transfer_rejects_small_workspace(lib):
    d = _desc()
    io = _lib.TransferIO()
    io.field_in = 1
    io.field_out = 1
    rc = lib.dtmm_transfer(ctypes.byref(d), ctypes.byref(io), ctypes.c_void_p(1), 16, None)
    assert rc == _lib.DTMM_ENOSPACE
    assert "workspace" in _lib.last_error()


def test_tuning_fields_do_not_change_the_workspace(lib):
    base = lib.dtmm_transfer_workspace_size(ctypes.byref(_desc()))
    for kw in ({"fft_schedule": 1}, {"fft_schedule": 3}, {"row_group": 4, "col_tile": 8}):
        assert lib.dtmm_transfer_workspace_size(ctypes.byref(_desc(**kw))) == base


@pytest.mark.parametrize("args,needle", [
    ((0, 16, 1, 1, 1, 1, 0, 1), "grid"),
    ((16, 16, 0, 1, 1, 1, 0, 1), "image count"),
    ((16, 16, 70000, 1, 1, 1, 0, 1), "image count"),
    ((16, 16, 2, 0, 1, 1, 0, 1), "null"),
    ((16, 16, 2, 1, 1, 1, 5, 1), "precision"),
])
def test_planewave_rejects_invalid_arguments(lib, args, needle):
    h, w, n, coef, my, mx, prec, field = args
    rc = lib.dtmm_planewave_field(h, w, n, ctypes.c_void_p(coef), ctypes.c_void_p(my), ctypes.c_void_p(mx), prec,
                                  ctypes.c_void_p(field), None)
    assert rc == _lib.DTMM_EINVAL
    assert needle in _lib.last_error()


def test_tuner_knows_the_register_transform_sides():
    """The autotuner's list of register-transform sides is the library's table."""
    import re

    from dtmm_gb300.tune import SIDES_REG

    text = open(os.path.join(ROOT, "dtmm_gb300", "csrc", "dtmm_regfft.cuh")).read()
    body = text[text.index("constexpr int reg_lanes(int n)"):]
    body = body[:body.index("default:")]
    sides = tuple(int(n) for n in re.findall(r"case (\d+):", body))
    assert sides == SIDES_REG
    macro = open(os.path.join(ROOT, "dtmm_gb300", "csrc", "dtmm_regkern.cuh")).read()
    listed = macro[macro.index("#define DTMM_REG_SIDES(X)"):]
    listed = listed[:listed.index("\n\n")]
    assert tuple(int(n) for n in re.findall(r"X\((\d+)\)", listed)) == SIDES_REG
    units = "".join(open(os.path.join(ROOT, "dtmm_gb300", "csrc", f)).read()
                    for f in sorted(os.listdir(os.path.join(ROOT, "dtmm_gb300", "csrc"))) if f.startswith("dtmm_reg_"))
    assert sorted(int(n) for n in re.findall(r"DTMM_REG_DEFINE\((\d+)\)", units)) == list(SIDES_REG)


def test_block_sym_descriptor_rules(lib):
    """block_sym (the symmetry of each block's effective medium): values 0-2;
    uniaxial / biaxial blocks take the 4x4 real-space chains (reflection 1
    included, with its per-ray 4x4 tables), norm_ref included; the 2x2
    method takes them on its real-space paths (reflection 0 and 2, no
    diffraction, diffraction = inf) and refuses reflection 1; they change nothing
    without diffraction or with diffraction = inf; all-isotropic block_sym is
    the default path."""
    size = lambda sym, **kw: lib.dtmm_transfer_workspace_size(ctypes.byref(_with_sym(_desc(**kw), sym)))
    assert size([0]) == size(None)
    a1 = size([1])
    assert a1 > 0 and size([2]) == a1
    assert size([1], nray=2) > a1  # per-ray tables of the windows' beams
    for bad in ([4], [-1], [3]):  # 3 without block_eff
        assert size(bad) == 0 and "block_sym" in _lib.last_error()
    # given media (block_sym 3): three equal eigenvalues keep the default path
    iso = np.array([2.4, 0.0, 2.4, 0.0, 2.4, 0.0, 0.0, 0.0, 0.0])
    uni = np.array([2.3, 0.0, 2.3, 0.0, 2.7, 0.0, 0.0, 0.5, 0.1])
    for rec, same in ((iso, True), (uni, False)):
        dd = _with_sym(_desc(), [3])
        dd._be = rec
        dd.block_eff = rec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s3 = lib.dtmm_transfer_workspace_size(ctypes.byref(dd))
        assert s3 > 0 and (s3 == size(None)) == same
    assert size([1], method=2, reflection=0) > 0  # the k-space step in real space
    assert size([1], method=2, reflection=1) == 0 and "reflection" in _lib.last_error()
    assert size([1], method=2, reflection=2) == size(None, method=2, reflection=2) > 0
    assert size([1], npass=3, norm_ref=1) > 0  # the real-space chains with the reference field
    assert size([1], diffraction=0, reflection=2) == size(None, diffraction=0, reflection=2)
    assert size([1], reflection=4) == size(None, reflection=4)
    # one entry per block of layer_block
    lb = np.array([0, 0, 1], np.int32)
    d = _with_sym(_desc(layer_block=lb.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), [0, 2])
    d._keep2 = lb
    assert lib.dtmm_transfer_workspace_size(ctypes.byref(d)) > 0


def _with_sym(d, sym):
    if sym is not None:
        bs = np.ascontiguousarray(sym, np.int32)
        d._bs = bs
        d.block_sym = bs.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    return d
