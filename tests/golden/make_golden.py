"""Generate the golden transfer_field fixtures from the unmodified reference.

Run where a reference checkout is present, naming it in DTMM_REFERENCE_ROOT:

    DTMM_REFERENCE_ROOT=/root/reference python tests/golden/make_golden.py            # all cases
    DTMM_REFERENCE_ROOT=/root/reference python tests/golden/make_golden.py cfg0_4x4   # one case

Each case builds its inputs with the reference's own ``illumination_data``
and the seeded director generators of ``dtmm_gb300.samples``, runs
``dtmm.transfer_field`` (complex128, numba replaced by a pure-Python stand-in,
see ``refload.py``) and stores ``field_in``, the returned field and, for
npass > 1, the reference's in-place update of ``field_in`` as
``tests/golden/<case>.npz``.  The optical data is not stored: the case
record (``CASES`` below) rebuilds it deterministically from its seed.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from golden_cases import (CASES, ORACLE_CASES, ILLUM_CASES, ILLUM_WINDOW_CASES, POM_CASES, RAYS_CASES, TCMF_CASES,  # noqa: E402
                          TCMF_TABLES, WINDOW_CASES, build_inputs, raised_cosine_window)


def reference_materials(optical_data, dtmm):
    """The reference's own dispersive eps classes in place of the product's
    (same coefficients), so that the fixture pins the reference's evaluation."""
    from dtmm_gb300 import data as gdata

    out = []
    for d, e, a in optical_data:
        if isinstance(e, gdata.EpsilonCauchy):
            e = dtmm.data.EpsilonCauchy(np.array(e.coefficients))
        elif isinstance(e, gdata.EpsilonSellmeier):
            e = dtmm.data.EpsilonSellmeier(np.array(e.coefficients))
        out.append((d, e, a))
    return out


def run_case(name, dtmm):
    case = CASES[name] if name in CASES else ORACLE_CASES[name]
    field_data, optical_data = build_inputs(case, dtmm.illumination_data)
    optical_data = reference_materials(optical_data, dtmm)
    field_in = field_data[0]
    saved_in = field_in.copy()
    kwargs = dict(case["transfer"])
    t0 = time.time()
    out = dtmm.transfer_field(field_data, optical_data, **kwargs)
    dt = time.time() - t0
    field_out = out[0]
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        field_in=saved_in,
        field_out=np.asarray(field_out),
        field_in_after=field_in,
        wavelengths=np.asarray(field_data[1]),
        pixelsize=np.asarray(field_data[2]),
    )
    print("%-22s %6.1fs  out %s" % (name, dt, np.asarray(field_out).shape))


def save_wave_kat(dtmm):
    """Known-answer k-grid maps held by the reference's own tests (dtmm/test/test_wave.py:21-69)."""
    import importlib

    tw = importlib.import_module("dtmm.test.test_wave")
    t = tw.TestWave("test_betaphi")
    t.setUp()
    np.savez_compressed(os.path.join(HERE, "kat_wave.npz"), shape=np.asarray(t.shape), ks=np.asarray(t.ks, float),
                        beta=t.beta, phi=t.phi, betax=t.betax, betay=t.betay)
    print("kat_wave               shape %s ks %s" % (t.shape, t.ks))


def save_alphaf_kat(dtmm):
    """Reference alphaf / inv / E_mat on random uniaxial and isotropic voxels, both beta branches."""
    rng = np.random.Generator(np.random.PCG64(1234))
    n = 64
    beta = rng.uniform(0.0, 0.8, n)
    beta[:8] = 0.0
    phi = rng.uniform(-np.pi, np.pi, n)
    no = rng.uniform(1.3, 1.7, n)
    ne = no + rng.uniform(-0.2, 0.3, n)
    ne[8:16] = no[8:16]
    epsv = np.stack([no ** 2, no ** 2, ne ** 2], axis=-1).astype(np.complex128)
    epsv[16:24] = epsv[16:24] + np.asarray([0.02j, 0.02j, 0.05j])
    epsa = np.stack([np.zeros(n), rng.uniform(0, np.pi, n), rng.uniform(-np.pi, np.pi, n)], axis=-1)
    alpha, f = dtmm.tmm.alphaf(beta, phi, epsv, epsa)
    fi = dtmm.linalg.inv(f)
    np.savez_compressed(os.path.join(HERE, "kat_alphaf.npz"), beta=beta, phi=phi, epsv=epsv, epsa=epsa,
                        alpha=alpha, f=f, fi=fi)
    print("kat_alphaf             %d voxels" % n)


def save_illum(dtmm):
    """Reference illumination_data fields for ILLUM_CASES, one array per case in illum.npz."""
    arrays = {}
    for name, case in ILLUM_CASES.items():
        kw = dict(case)
        shape = kw.pop("shape")
        wl = kw.pop("wavelengths")
        ps = kw.pop("pixelsize")
        arrays[name] = np.asarray(dtmm.illumination_data(shape, wl, pixelsize=ps, **kw)[0])
    np.savez_compressed(os.path.join(HERE, "illum.npz"), **arrays)
    print("illum                  %d cases" % len(arrays))


def save_pom(dtmm):
    """Reference POM pipeline on golden transferred fields, one pom_<case>.npz per POM_CASES entry:
    the jones vector, analyzer matrix, window, diffraction matrix and cmf it used, the POM
    field, the specter and RGB images for several specter2color options."""
    import importlib

    color, diffract, field, field_viewer, jones, jones4 = (
        importlib.import_module("dtmm." + m) for m in ("color", "diffract", "field", "field_viewer", "jones", "jones4"))

    for name, case in POM_CASES.items():
        src = np.load(os.path.join(HERE, case["source"] + ".npz"))
        f = np.array(src["field_out"])
        wl = np.asarray(src["wavelengths"], float)
        ps = float(src["pixelsize"])
        shape = f.shape[-2:]
        jvec = None if case["jvec"] is None else jones.jonesvec(case["jvec"][0], case["jvec"][1])
        an = case["analyzer"]
        jmat = jones.rotated_matrix(jones.polarizer(jones.jonesvec(an[0])), an[1])
        pmat = jones4.ray_jonesmat4x4(jmat)
        window = raised_cosine_window(shape) if case.get("window") else None
        dmat = None
        if case.get("dmat_d") is not None:
            ks = 2 * np.pi / wl * ps
            dmat = diffract.field_diffraction_matrix(shape, ks, d=case["dmat_d"], epsv=(2.25, 2.25, 2.25))
        # the reference writes its result into `out` (and returns it); without `out` it returns None
        out = np.empty_like(f[..., 0, :, :, :, :] if jvec is not None else f)
        pom = field_viewer.calculate_pom_field(f.copy(), jvec, pmat, dmat, window=window, out=out)
        spec = field.field2spectersum(pom) if case.get("summed") else field.field2specter(pom)
        cmf = color.load_tcmf(wl)
        arrays = dict(field_in=f, wavelengths=wl, jvec=np.zeros(2, complex) if jvec is None else np.asarray(jvec),
                      has_jvec=np.asarray(jvec is not None), pmat=np.asarray(pmat), pom=np.asarray(pom),
                      spec=np.asarray(spec), cmf=np.asarray(cmf),
                      rgb=color.specter2color(spec, cmf),
                      rgb_gray=color.specter2color(spec, cmf, gray=True),
                      rgb_norm=color.specter2color(spec, cmf, norm=True),
                      rgb_gamma=color.specter2color(spec, cmf, norm=0.7, gamma=2.2),
                      rgb_linear=color.specter2color(spec, cmf, norm=0.5, gamma=False))
        if window is not None:
            arrays["window"] = window
        if dmat is not None:
            arrays["dmat"] = np.asarray(dmat)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print("%-22s pom %s spec %s" % (name, np.asarray(pom).shape, np.asarray(spec).shape))


def save_director(dtmm):
    """Reference director2data on a seeded director field (lengths 0 to 1.3, a masked host region)."""
    rng = np.random.Generator(np.random.PCG64(77))
    director = rng.normal(size=(3, 12, 16, 3))
    director *= (rng.uniform(0.0, 1.3, size=(3, 12, 16)) / np.linalg.norm(director, axis=-1))[..., None]
    director[0, 0, :4] = 0.0
    zz, yy, xx = np.meshgrid(np.arange(3), np.arange(12), np.arange(16), indexing="ij")
    mask = (yy - 6) ** 2 + (xx - 8) ** 2 < 30
    a = dtmm.data.director2data(director)
    b = dtmm.data.director2data(director, mask=mask, no=1.52, ne=1.71, nhost=1.4, scale_factor=0.8)
    np.savez_compressed(os.path.join(HERE, "director.npz"), director=director, mask=mask,
                        epsv_default=a[1], epsa_default=a[2], thickness_default=a[0],
                        epsv_masked=b[1], epsa_masked=b[2])
    print("director               %s" % (director.shape,))


def save_files(dtmm):
    """Reference .dtmf / .dtms files of small seeded data (read back and rewritten by the IO tests)."""
    rng = np.random.Generator(np.random.PCG64(5))
    field = (rng.normal(size=(2, 3, 4, 6, 5)) + 1j * rng.normal(size=(2, 3, 4, 6, 5))).astype(np.complex128)
    dtmm.field.save_field(os.path.join(HERE, "io_field"), (field, np.asarray([450.0, 550.0, 650.0]), 80.0))
    d = np.asarray([1.0, 2.0, 0.5])
    epsv = np.broadcast_to(np.asarray([2.25, 2.25, 2.89]), (3, 6, 5, 3)).copy()
    epsa = rng.uniform(-1, 1, size=(3, 6, 5, 3))
    epsv2 = (np.full((2, 1, 1, 3), 2.1) + 0.01j).astype(np.complex128)
    epsa2 = np.zeros((2, 1, 1, 3))
    dtmm.data.save_stack(os.path.join(HERE, "io_stack"), [(d, epsv, epsa), (np.asarray([3.0, 1.0]), epsv2, epsa2)])
    print("io files               io_field.dtmf io_stack.dtms")


def save_qtensor(dtmm):
    """Reference Q2data on seeded Q tensors (uniaxial from random directors with random order,
    some exactly diagonal, plus small biaxial parts), uniaxial and biaxial variants."""
    rng = np.random.Generator(np.random.PCG64(91))
    shape = (2, 6, 7)
    n = rng.normal(size=shape + (3,))
    n /= np.linalg.norm(n, axis=-1)[..., None]
    S = rng.uniform(0.2, 0.9, size=shape)
    Q = np.empty(shape + (6,))
    Q[..., 0] = S * (n[..., 0] ** 2 - 1 / 3)
    Q[..., 1] = S * (n[..., 1] ** 2 - 1 / 3)
    Q[..., 2] = S * (n[..., 2] ** 2 - 1 / 3)
    Q[..., 3] = S * n[..., 0] * n[..., 1]
    Q[..., 4] = S * n[..., 0] * n[..., 2]
    Q[..., 5] = S * n[..., 1] * n[..., 2]
    Q[0, 0, :3, :3] = [[-0.2, -0.2, 0.4], [0.4, -0.2, -0.2], [-0.2, 0.4, -0.2]]  # diagonal tensors
    Q[0, 0, :3, 3:] = 0.0
    Q[1] += rng.normal(scale=0.02, size=Q[1].shape)
    mask = rng.uniform(size=shape) > 0.2
    a = dtmm.data.Q2data(Q)
    b = dtmm.data.Q2data(Q, mask=mask, no=1.52, ne=1.71, nhost=1.4, scale_factor=0.9)
    c = dtmm.data.Q2data(Q, biaxial=True)
    np.savez_compressed(os.path.join(HERE, "qtensor.npz"), Q=Q, mask=mask, epsv=a[1], epsa=a[2],
                        epsv_masked=b[1], epsa_masked=b[2], epsv_biaxial=c[1], epsa_biaxial=c[2])
    print("qtensor                %s" % (Q.shape,))


def save_illum_window(dtmm):
    """Reference windows, ray sets and windowed illumination_data fields (illum_window.npz)."""
    import importlib

    window = importlib.import_module("dtmm.window")
    field = importlib.import_module("dtmm.field")
    arrays = {}
    for name, (fn, args) in WINDOW_CASES.items():
        arrays["window_" + name] = np.asarray(getattr(window, fn)(*args))
    for name, (na, diameter, smooth) in RAYS_CASES.items():
        b, p, i = field.illumination_rays(na, diameter, smooth)
        arrays["rays_%s_beta" % name], arrays["rays_%s_phi" % name], arrays["rays_%s_intensity" % name] = b, p, i
    for name, case in ILLUM_WINDOW_CASES.items():
        kw = dict(case)
        shape, wl, ps = kw.pop("shape"), kw.pop("wavelengths"), kw.pop("pixelsize")
        kw["window"] = arrays["window_" + kw.pop("window")]
        rays = kw.pop("rays", None)
        if rays is not None:
            kw["beta"], kw["phi"], kw["intensity"] = (arrays["rays_%s_%s" % (rays, k)]
                                                      for k in ("beta", "phi", "intensity"))
        arrays[name] = np.asarray(dtmm.illumination_data(shape, wl, pixelsize=ps, **kw)[0])
    np.savez_compressed(os.path.join(HERE, "illum_window.npz"), **arrays)
    print("illum_window           %d arrays" % len(arrays))


def save_tcmf(dtmm):
    """Reference load_tcmf for TCMF_CASES, with the data tables it read (tcmf.npz)."""
    import importlib

    color = importlib.import_module("dtmm.color")
    arrays = {}
    for key, fname in TCMF_TABLES.items():
        arrays["table_" + key] = np.loadtxt(os.path.join(color.DATAPATH, fname))
    for name, kw in TCMF_CASES.items():
        x, c = color.load_tcmf(retx=True, **kw)
        arrays[name + "_x"], arrays[name] = np.asarray(x, float), np.asarray(c)
    np.savez_compressed(os.path.join(HERE, "tcmf.npz"), **arrays)
    print("tcmf                   %d cases" % len(TCMF_CASES))


def save_alphaf_biaxial_kat(dtmm):
    """Reference alphaf / inv on random biaxial voxels (general eigen-solve and
    Poynting sort), lossless and absorbing, both beta branches."""
    rng = np.random.Generator(np.random.PCG64(4321))
    n = 64
    beta = rng.uniform(0.0, 0.8, n)
    beta[:8] = 0.0
    phi = rng.uniform(-np.pi, np.pi, n)
    e0 = rng.uniform(1.9, 2.6, n)
    epsv = np.stack([e0, e0 + rng.uniform(0.05, 0.4, n), e0 + rng.uniform(0.5, 0.9, n)], axis=-1).astype(np.complex128)
    epsv[16:28] = epsv[16:28] + rng.uniform(0.0, 0.05, (12, 3)) * 1j
    epsa = np.stack([rng.uniform(-np.pi, np.pi, n), rng.uniform(0, np.pi, n), rng.uniform(-np.pi, np.pi, n)], axis=-1)
    alpha, f = dtmm.tmm.alphaf(beta, phi, epsv, epsa)
    fi = dtmm.linalg.inv(f)
    np.savez_compressed(os.path.join(HERE, "kat_alphaf_biaxial.npz"), beta=beta, phi=phi, epsv=epsv, epsa=epsa,
                        alpha=alpha, f=f, fi=fi)
    print("kat_alphaf_biaxial     %d voxels" % n)


def main(argv):
    import refload

    dtmm = refload.load_reference()
    names = argv[1:] or (["kat", "illum"] + list(CASES) + list(ORACLE_CASES) + ["pom", "director", "files", "qtensor", "illum_window",
                                                            "tcmf"])
    for name in names:
        if name == "kat":
            save_wave_kat(dtmm)
            save_alphaf_kat(dtmm)
            save_alphaf_biaxial_kat(dtmm)
        elif name == "illum":
            save_illum(dtmm)
        elif name == "pom":
            save_pom(dtmm)
        elif name == "director":
            save_director(dtmm)
        elif name == "files":
            save_files(dtmm)
        elif name == "qtensor":
            save_qtensor(dtmm)
        elif name == "illum_window":
            save_illum_window(dtmm)
        elif name == "tcmf":
            save_tcmf(dtmm)
        else:
            run_case(name, dtmm)


if __name__ == "__main__":
    main(sys.argv)
