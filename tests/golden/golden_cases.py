"""Case records of the golden transfer_field fixtures.

Each case fixes the grid, wavelengths, material generator and seed, the
illumination and the ``transfer_field`` keyword arguments.  ``build_inputs``
rebuilds ``(field_data, optical_data)`` for a case with a given
``illumination_data`` implementation (the reference's when generating the
fixtures, the product's or the fixture's stored field when testing).
"""
import numpy as np

from dtmm_gb300 import samples


def _twisted(shape, nlayers, seed, **kw):
    return samples.twisted_nematic(shape, nlayers, seed=seed, **kw)


def _absorbing(shape, nlayers, seed):
    d, _, epsa = samples.twisted_nematic(shape, nlayers, seed=seed, amplitude=0.3)
    epsv = np.broadcast_to(np.asarray((2.25 + 0.04j, 2.25 + 0.04j, 2.89 + 0.09j)), epsa.shape)
    return d, epsv, epsa


def _mixed_voxels(shape, nlayers, seed):
    """Isotropic and uniaxial voxels side by side, plus an isotropic layer."""
    d, epsv, epsa = samples.twisted_nematic(shape, nlayers, seed=seed, amplitude=0.3)
    epsv = np.array(epsv)
    rng = np.random.Generator(np.random.PCG64(seed + 3))
    kind = rng.integers(0, 3, size=epsv.shape[:-1])
    epsv[kind == 0] = (2.3, 2.3, 2.3)
    epsv[kind == 2] = (2.4, 2.4, 2.6)
    epsv[0] = (2.2, 2.2, 2.2)
    return d, epsv, epsa


def _biaxial(shape, nlayers, seed, absorbing=False):
    """Biaxial voxels (three distinct eigenvalues, a seeded psi per voxel) with
    uniaxial and isotropic voxels among them, on a twisted director."""
    d, _, epsa = samples.twisted_nematic(shape, nlayers, seed=seed, amplitude=0.3)
    epsa = np.array(epsa)
    rng = np.random.Generator(np.random.PCG64(seed + 5))
    epsa[..., 0] = rng.uniform(-np.pi, np.pi, size=epsa.shape[:-1])
    epsv = np.empty(epsa.shape, np.complex128 if absorbing else np.float64)
    epsv[...] = (2.25 + 0.03j, 2.42 + 0.01j, 2.89 + 0.05j) if absorbing else (2.25, 2.42, 2.89)
    kind = rng.integers(0, 5, size=epsv.shape[:-1])
    epsv[kind == 0] = (2.3, 2.3, 2.7)
    epsv[kind == 1] = (2.35, 2.35, 2.35)
    return d, epsv, epsa


def _cauchy(shape, nlayers, seed):
    """Dispersive twisted nematic: per-layer Cauchy coefficients (n = c0 + c1 / w^2,
    w in microns) of slightly different ordinary / extraordinary indices."""
    from dtmm_gb300.data import EpsilonCauchy

    d, _, epsa = samples.twisted_nematic(shape, nlayers, seed=seed, amplitude=0.3)
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    c = np.empty((nlayers, 3, 2))
    c[:, :2, 0] = 1.49 + rng.uniform(0.0, 0.01, (nlayers, 1))
    c[:, 2, 0] = 1.64 + rng.uniform(0.0, 0.01, nlayers)
    c[:, :2, 1] = 0.0045
    c[:, 2, 1] = 0.011
    return d, EpsilonCauchy(c), epsa


def _isotropic(shape, nlayers, seed, eps=2.1):
    """Homogeneous isotropic layers of eps (a glass or a cover block)."""
    d = np.ones(nlayers)
    epsv = np.tile(np.asarray((eps, eps, eps)), (nlayers, 1, 1, 1))
    return d, epsv, np.zeros((nlayers, 1, 1, 3))


MATERIALS = {
    "twisted": _twisted,
    "biaxial": _biaxial,
    "inplane": lambda shape, nlayers, seed, **kw: samples.inplane_nematic(shape, nlayers, seed=seed, **kw),
    "absorbing": _absorbing,
    "cauchy": _cauchy,
    "iso": _isotropic,
    "mixed": _mixed_voxels,
}

CASES = {
    # the plain workload at full size: 64x64, 20 layers, 550 nm, 100 nm pixels
    "cfg0_4x4": dict(shape=(64, 64), nlayers=20, wavelengths=[550.0], pixelsize=100.0,
                     material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.2)), seed=0,
                     illum=dict(jones=(1, 0)),
                     transfer=dict(method="4x4", diffraction=1, npass=1, beta=0.0, phi=0.0)),
    # the precision workload's options (4x4, diffraction 3, npass 3, both polarisations) on a small grid
    "cfg1_small": dict(shape=(24, 30), nlayers=4, wavelengths=[400.0, 600.0], pixelsize=50.0,
                       material=("twisted", dict(no=1.52, ne=1.71, amplitude=0.3)), seed=1,
                       illum=dict(),
                       transfer=dict(method="4x4", diffraction=3, npass=3, beta=0.0, phi=0.0)),
    # the 2x2 workload's options (2x2, diffraction 5, no reflection) on a small grid
    "cfg3_small": dict(shape=(30, 24), nlayers=4, wavelengths=[450.0, 550.0, 650.0], pixelsize=100.0,
                       material=("inplane", dict(no=1.5, ne=1.6)), seed=3,
                       illum=dict(),
                       transfer=dict(method="2x2", diffraction=5, reflection=0, beta=0.0, phi=0.0)),
    "twox2_d1_offaxis": dict(shape=(20, 28), nlayers=6, wavelengths=[500.0, 600.0], pixelsize=100.0,
                             material=("twisted", dict()), seed=4,
                             illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                             transfer=dict(method="2x2", diffraction=1, beta=0.1, phi=0.3)),
    "twox2_d3_offaxis": dict(shape=(20, 24), nlayers=3, wavelengths=[520.0], pixelsize=100.0,
                             material=("twisted", dict()), seed=5,
                             illum=dict(beta=0.2, phi=0.3),
                             transfer=dict(method="2x2", diffraction=3, beta=0.2, phi=0.3)),
    "fourx4_offaxis_npass2": dict(shape=(16, 20), nlayers=3, wavelengths=[500.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=6,
                                  illum=dict(beta=0.15, phi=0.7, jones=(1, 0.5j)),
                                  transfer=dict(method="4x4", diffraction=1, npass=2, beta=0.15, phi=0.7)),
    "fourx4_d3_offaxis": dict(shape=(18, 16), nlayers=3, wavelengths=[520.0, 640.0], pixelsize=80.0,
                              material=("twisted", dict()), seed=7,
                              illum=dict(beta=0.1, phi=0.4, jones=(0, 1)),
                              transfer=dict(method="4x4", diffraction=3, beta=0.1, phi=0.4)),
    "fourx4_multiray": dict(shape=(16, 16), nlayers=3, wavelengths=[520.0, 620.0], pixelsize=100.0,
                            material=("twisted", dict()), seed=8,
                            illum=dict(beta=[0.0, 0.1, 0.2], phi=[0.0, np.pi / 2, 0.0], jones=(1, 0)),
                            transfer=dict(method="4x4", diffraction=1, multiray=True,
                                          beta=[0.0, 0.1, 0.2], phi=[0.0, np.pi / 2, 0.0])),
    "fourx4_autobeta": dict(shape=(16, 18), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                            material=("twisted", dict()), seed=9,
                            illum=dict(beta=0.1, phi=0.2, jones=(1, 0)),
                            transfer=dict(method="4x4", diffraction=1)),
    "fourx4_absorbing": dict(shape=(16, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                             material=("absorbing", dict()), seed=11,
                             illum=dict(beta=0.05, jones=(1, 0)),
                             transfer=dict(method="4x4", diffraction=1, beta=0.05, phi=0.0)),
    "fourx4_mixed_voxels": dict(shape=(14, 16), nlayers=3, wavelengths=[600.0], pixelsize=100.0,
                                material=("mixed", dict()), seed=12,
                                illum=dict(beta=0.1, phi=1.0, jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, beta=0.1, phi=1.0)),
    "fourx4_nstep2": dict(shape=(16, 16), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                          material=("twisted", dict(thickness=2.0)), seed=13,
                          illum=dict(jones=(1, 0)),
                          transfer=dict(method="4x4", diffraction=1, nstep=2, beta=0.0, phi=0.0)),
    "fourx4_d3_nstep2": dict(shape=(16, 16), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                             material=("twisted", dict(thickness=2.0)), seed=14,
                             illum=dict(jones=(1, 0)),
                             transfer=dict(method="4x4", diffraction=3, nstep=2, beta=0.0, phi=0.0)),
    # dispersive eps (Cauchy coefficients per layer) evaluated per wavelength under
    # split_wavelengths; npass 1, because the reference's split path hands transfer_4x4
    # an uninitialised out array whose reflected part npass > 1 would keep
    "fourx4_cauchy_split": dict(shape=(16, 18), nlayers=3, wavelengths=[450.0, 550.0, 650.0], pixelsize=100.0,
                                material=("cauchy", dict()), seed=16,
                                illum=dict(jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, split_wavelengths=True,
                                              beta=0.0, phi=0.0)),
    "twox2_cauchy_split": dict(shape=(14, 16), nlayers=3, wavelengths=[480.0, 620.0], pixelsize=100.0,
                               material=("cauchy", dict()), seed=17,
                               illum=dict(beta=0.1, phi=0.5),
                               transfer=dict(method="2x2", diffraction=1, split_wavelengths=True,
                                             beta=0.1, phi=0.5)),
    # npass > 1 with norm = 0: the reference's "total" renormalisation of each image
    "fourx4_norm_total_npass3": dict(shape=(16, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                                     material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=18,
                                     illum=dict(beta=0.1, phi=0.6),
                                     transfer=dict(method="4x4", diffraction=1, npass=3, norm=0, beta=0.1,
                                                   phi=0.6)),
    # npass > 1 with norm = DTMM_NORM_FFT | DTMM_NORM_REF (3): a 2x2 reference field
    # through the forward passes sets the intensities of the per-mode normalisation
    "fourx4_norm_ref_npass2": dict(shape=(14, 12), nlayers=3, wavelengths=[520.0], pixelsize=100.0,
                                   material=("twisted", dict()), seed=69,
                                   illum=dict(beta=0.1, phi=0.4, jones=(1, 0)),
                                   transfer=dict(method="4x4", diffraction=1, npass=2, norm=3, beta=0.1, phi=0.4)),
    "fourx4_norm_ref_d3_npass3": dict(shape=(12, 12), nlayers=2, wavelengths=[480.0, 600.0], pixelsize=100.0,
                                      material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=70,
                                      illum=dict(),
                                      transfer=dict(method="4x4", diffraction=3, npass=3, norm=3, beta=0.0,
                                                    phi=0.0)),
    "fourx4_norm_ref_nstep2_npass4": dict(shape=(12, 14), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                          material=("twisted", dict(thickness=2.0)), seed=71,
                                          illum=dict(jones=(0, 1)),
                                          transfer=dict(method="4x4", diffraction=1, nstep=2, npass=4, norm=3,
                                                        beta=0.0, phi=0.0)),
    # npass > 1 with norm = DTMM_NORM_REF (2): the "local" per-pixel normalisation with the
    # reference field
    "fourx4_norm_local_npass2": dict(shape=(12, 14), nlayers=3, wavelengths=[540.0], pixelsize=100.0,
                                     material=("twisted", dict()), seed=72,
                                     illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                                     transfer=dict(method="4x4", diffraction=1, npass=2, norm=2, beta=0.1, phi=0.3)),
    "fourx4_norm_local_d3_npass3": dict(shape=(12, 12), nlayers=2, wavelengths=[470.0, 610.0], pixelsize=100.0,
                                        material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=73,
                                        illum=dict(),
                                        transfer=dict(method="4x4", diffraction=3, npass=3, norm=2, beta=0.0,
                                                      phi=0.0)),
    "fourx4_norm_total_d3_npass4": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                        material=("twisted", dict()), seed=19,
                                        illum=dict(jones=(1, 0)),
                                        transfer=dict(method="4x4", diffraction=3, npass=4, norm=0, beta=0.0,
                                                      phi=0.0)),
    # several optical blocks (each its own effective medium), and split_layers (one per layer)
    "fourx4_blocks": dict(shape=(14, 16), nlayers=5, wavelengths=[520.0, 640.0], pixelsize=100.0,
                          blocks=[("twisted", dict(no=1.5, ne=1.7), 2), ("iso", dict(eps=2.3), 1),
                                  ("twisted", dict(no=1.55, ne=1.65, amplitude=0.3), 2)], seed=20,
                          illum=dict(beta=0.1, phi=0.5, jones=(1, 0)),
                          transfer=dict(method="4x4", diffraction=1, beta=0.1, phi=0.5)),
    "fourx4_blocks_d3_npass2": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                    blocks=[("twisted", dict(), 2), ("iso", dict(eps=2.0), 1)], seed=21,
                                    illum=dict(jones=(1, 0)),
                                    transfer=dict(method="4x4", diffraction=3, npass=2, beta=0.0, phi=0.0)),
    # effective layers of uniaxial / biaxial symmetry (the mean lab-frame tensor of a
    # block, or of each layer), every 4x4 reflection mode with diffraction
    "fourx4_eff_uniaxial": dict(shape=(12, 14), nlayers=3, wavelengths=[540.0], pixelsize=100.0,
                                material=("twisted", dict()), seed=74,
                                illum=dict(beta=0.1, phi=0.4, jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, eff_data=1, beta=0.1, phi=0.4)),
    "fourx4_eff_biaxial_d3": dict(shape=(12, 12), nlayers=2, wavelengths=[480.0, 620.0], pixelsize=100.0,
                                  material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=75,
                                  illum=dict(),
                                  transfer=dict(method="4x4", diffraction=3, eff_data="biaxial", beta=0.0,
                                                phi=0.0)),
    "fourx4_eff_uniaxial_refl2": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                      material=("twisted", dict()), seed=76,
                                      illum=dict(beta=0.1, phi=0.2, jones=(0, 1)),
                                      transfer=dict(method="4x4", diffraction=1, reflection=2, eff_data="uniaxial",
                                                    beta=0.1, phi=0.2)),
    "fourx4_eff_biaxial_refl3_d3": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                        material=("twisted", dict(amplitude=0.3)), seed=77,
                                        illum=dict(jones=(1, 0)),
                                        transfer=dict(method="4x4", diffraction=3, reflection=3, eff_data=2,
                                                      beta=0.0, phi=0.0)),
    "fourx4_eff_uniaxial_refl4_nstep2": dict(shape=(12, 14), nlayers=2, wavelengths=[520.0], pixelsize=100.0,
                                             material=("twisted", dict(thickness=2.0)), seed=78,
                                             illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                                             transfer=dict(method="4x4", diffraction=1, reflection=4, nstep=2,
                                                           eff_data=1, beta=0.1, phi=0.3)),
    "fourx4_eff_blocks": dict(shape=(12, 12), nlayers=5, wavelengths=[520.0, 640.0], pixelsize=100.0,
                              blocks=[("twisted", dict(no=1.5, ne=1.7), 2), ("iso", dict(eps=2.3), 1),
                                      ("twisted", dict(no=1.55, ne=1.65, amplitude=0.3), 2)], seed=79,
                              illum=dict(beta=0.1, phi=0.5, jones=(1, 0)),
                              transfer=dict(method="4x4", diffraction=1, eff_data=[1, 0, "biaxial"], beta=0.1,
                                            phi=0.5)),
    "fourx4_eff_per_layer_d3": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                    material=("twisted", dict(amplitude=0.3)), seed=80,
                                    illum=dict(jones=(1, 0)),
                                    transfer=dict(method="4x4", diffraction=3, eff_data=[[1, 2, 0]], beta=0.0,
                                                  phi=0.0)),
    "fourx4_eff_uniaxial_npass2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                       material=("twisted", dict()), seed=81,
                                       illum=dict(jones=(1, 0)),
                                       transfer=dict(method="4x4", diffraction=1, npass=2, eff_data=1, beta=0.0,
                                                     phi=0.0)),
    # the reference field's 2x2 pass and the 2x2 method's real-space sweep around an
    # effective medium of uniaxial / biaxial symmetry
    "fourx4_eff_norm_ref_npass2": dict(shape=(12, 14), nlayers=3, wavelengths=[530.0], pixelsize=100.0,
                                       material=("twisted", dict()), seed=82,
                                       illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                                       transfer=dict(method="4x4", diffraction=1, npass=2, norm=3, eff_data=1,
                                                     beta=0.1, phi=0.3)),
    "fourx4_eff_norm_local_d3_npass3": dict(shape=(12, 12), nlayers=2, wavelengths=[560.0], pixelsize=100.0,
                                            material=("twisted", dict(amplitude=0.3)), seed=83,
                                            illum=dict(jones=(0, 1)),
                                            transfer=dict(method="4x4", diffraction=3, npass=3, norm=2,
                                                          eff_data="biaxial", beta=0.0, phi=0.0)),
    "twox2_eff_refl2_d3": dict(shape=(12, 12), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                               material=("twisted", dict()), seed=84,
                               illum=dict(beta=0.1, phi=0.2, jones=(1, 0)),
                               transfer=dict(method="2x2", diffraction=3, reflection=2, eff_data=1, beta=0.1,
                                             phi=0.2)),
    "twox2_eff_refl2_npass2": dict(shape=(14, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                   material=("twisted", dict(amplitude=0.3)), seed=85,
                                   illum=dict(jones=(1, 0)),
                                   transfer=dict(method="2x2", diffraction=1, reflection=2, npass=2,
                                                 eff_data="biaxial", beta=0.0, phi=0.0)),
    "twox2_eff_uniaxial_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[540.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=86,
                                  illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                                  transfer=dict(method="2x2", diffraction=1, eff_data=1, beta=0.1, phi=0.3)),
    "twox2_eff_biaxial_d3": dict(shape=(12, 12), nlayers=2, wavelengths=[480.0, 620.0], pixelsize=100.0,
                                 material=("twisted", dict(amplitude=0.3)), seed=87,
                                 illum=dict(),
                                 transfer=dict(method="2x2", diffraction=3, eff_data="biaxial", beta=0.0, phi=0.0)),
    "twox2_eff_blocks_nstep2": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                    blocks=[("twisted", dict(thickness=2.0), 2), ("iso", dict(eps=2.3), 1)],
                                    seed=88, illum=dict(jones=(1, 0)),
                                    transfer=dict(method="2x2", diffraction=1, nstep=2, eff_data=[1, 0], beta=0.0,
                                                  phi=0.0)),
    "twox2_eff_uniaxial_bulk": dict(shape=(12, 12), nlayers=2, wavelengths=[520.0], pixelsize=100.0,
                                    material=("twisted", dict()), seed=89,
                                    illum=dict(beta=0.1, phi=0.5, jones=(0, 1)),
                                    transfer=dict(method="2x2", diffraction=1, eff_data=1, ret_bulk=True, beta=0.1,
                                                  phi=0.5)),
    # effective layers given as optical blocks (one homogeneous medium per layer)
    "fourx4_eff_given": dict(shape=(12, 14), nlayers=3, wavelengths=[540.0], pixelsize=100.0,
                             material=("twisted", dict()), seed=90,
                             illum=dict(beta=0.1, phi=0.4, jones=(1, 0)),
                             transfer=dict(method="4x4", diffraction=1, beta=0.1, phi=0.4,
                                           eff_data=[(np.ones(3), np.array([[2.3, 2.3, 2.7], [2.28, 2.28, 2.75],
                                                                            [2.31, 2.35, 2.7]]),
                                                      np.array([[0.0, 0.9, 0.2], [0.0, 1.1, 0.7],
                                                                [0.3, 1.0, 1.2]]))])),
    "fourx4_eff_given_iso_d3_npass2": dict(shape=(12, 12), nlayers=2, wavelengths=[560.0], pixelsize=100.0,
                                           material=("twisted", dict(amplitude=0.3)), seed=91,
                                           illum=dict(jones=(0, 1)),
                                           transfer=dict(method="4x4", diffraction=3, npass=2, beta=0.0, phi=0.0,
                                                         eff_data=[(np.ones(2), np.array([[2.4, 2.4, 2.4],
                                                                                          [2.5, 2.5, 2.5]]),
                                                                    np.zeros((2, 3)))])),
    "twox2_eff_given_d3": dict(shape=(12, 12), nlayers=2, wavelengths=[500.0, 610.0], pixelsize=100.0,
                               material=("twisted", dict()), seed=92,
                               illum=dict(jones=(1, 0)),
                               transfer=dict(method="2x2", diffraction=3, beta=0.0, phi=0.0,
                                             eff_data=[(np.ones(2), np.array([[2.3, 2.3, 2.7], [2.3, 2.3, 2.7]]),
                                                        np.array([[0.0, 1.2, 0.4], [0.0, 1.2, 1.0]]))])),
    "fourx4_split_layers": dict(shape=(12, 14), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                material=("mixed", dict()), seed=22,
                                illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, split_layers=True, beta=0.1, phi=0.3)),
    "fourx4_blocks_refl4": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                blocks=[("twisted", dict(), 2), ("iso", dict(eps=2.2), 1)], seed=23,
                                illum=dict(beta=0.1, phi=0.2, jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, reflection=4, beta=0.1, phi=0.2)),
    "twox2_blocks": dict(shape=(14, 12), nlayers=3, wavelengths=[500.0, 600.0], pixelsize=100.0,
                         blocks=[("twisted", dict(), 2), ("iso", dict(eps=2.4), 1)], seed=24,
                         illum=dict(beta=0.1, phi=0.4, jones=(1, 0)),
                         transfer=dict(diffraction=1, beta=0.1, phi=0.4)),
    "twox2_blocks_refl2_npass2": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                      blocks=[("twisted", dict(no=1.45, ne=1.6), 1), ("twisted", dict(), 2)],
                                      seed=25,
                                      illum=dict(jones=(1, 0)),
                                      transfer=dict(method="2x2", diffraction=1, reflection=2, npass=2, beta=0.0,
                                                    phi=0.0)),
    "fourx4_bulk": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                        material=("twisted", dict()), seed=15,
                        illum=dict(jones=(1, 0)),
                        transfer=dict(method="4x4", diffraction=1, beta=0.0, phi=0.0, ret_bulk=True)),
    "default_method": dict(shape=(16, 16), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                           material=("twisted", dict()), seed=16,
                           illum=dict(jones=(1, 0)),
                           transfer=dict(beta=0.0, phi=0.0)),
    "fourx4_nin_nout": dict(shape=(16, 16), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                            material=("twisted", dict()), seed=17,
                            illum=dict(jones=(1, 0), n=1.0),
                            transfer=dict(method="4x4", diffraction=1, npass=3, nin=1.0, nout=1.33,
                                          betamax=0.9, beta=0.0, phi=0.0)),
    # 4x4 without diffraction (reflection resolves to 2): the per-voxel 4x4 transfer
    "nodiff_4x4": dict(shape=(16, 20), nlayers=5, wavelengths=[450.0, 600.0], pixelsize=100.0,
                       material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=18,
                       illum=dict(),
                       transfer=dict(method="4x4", diffraction=0, beta=0.0, phi=0.0)),
    "nodiff_4x4_offaxis_nstep2": dict(shape=(12, 14), nlayers=3, wavelengths=[520.0], pixelsize=100.0,
                                      material=("twisted", dict(thickness=2.0)), seed=19,
                                      illum=dict(beta=0.2, phi=0.7, jones=(1, 0.3j)),
                                      transfer=dict(method="4x4", diffraction=0, nstep=2, beta=0.2, phi=0.7)),
    "nodiff_4x4_mixed": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0, 650.0], pixelsize=100.0,
                                       material=("mixed", dict()), seed=20,
                                       illum=dict(beta=0.1, phi=1.2),
                                       transfer=dict(method="4x4", diffraction=0, beta=0.1, phi=1.2)),
    "nodiff_4x4_absorbing_bulk": dict(shape=(8, 10), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                      material=("absorbing", dict()), seed=21,
                                      illum=dict(jones=(1, 0)),
                                      transfer=dict(method="4x4", diffraction=0, beta=0.0, phi=0.0,
                                                    ret_bulk=True)),
    "nodiff_4x4_multiray": dict(shape=(12, 12), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                                material=("twisted", dict()), seed=22,
                                illum=dict(beta=[0.0, 0.1, 0.2], phi=[0.0, np.pi / 2, 0.0], jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=0, multiray=True,
                                              beta=[0.0, 0.1, 0.2], phi=[0.0, np.pi / 2, 0.0])),
    # biaxial voxels (the general eigen-solve and Poynting sort of dtmm/tmm.py:395-401)
    "fourx4_biaxial": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                           material=("biaxial", dict()), seed=23,
                           illum=dict(beta=0.1, phi=0.5, jones=(1, 0)),
                           transfer=dict(method="4x4", diffraction=1, beta=0.1, phi=0.5)),
    "fourx4_biaxial_d3_npass2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                     material=("biaxial", dict()), seed=24,
                                     illum=dict(),
                                     transfer=dict(method="4x4", diffraction=3, npass=2, beta=0.0, phi=0.0)),
    "fourx4_biaxial_absorbing": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                     material=("biaxial", dict(absorbing=True)), seed=25,
                                     illum=dict(beta=0.05, jones=(0, 1)),
                                     transfer=dict(method="4x4", diffraction=1, beta=0.05, phi=0.0)),
    "twox2_biaxial": dict(shape=(12, 16), nlayers=3, wavelengths=[550.0, 650.0], pixelsize=100.0,
                          material=("biaxial", dict()), seed=26,
                          illum=dict(beta=0.1, phi=1.1),
                          transfer=dict(method="2x2", diffraction=1, beta=0.1, phi=1.1)),
    # diffraction = inf: every eigenwave below betamax through the voxels exactly
    # (dtmm/propagate_4x4.py:515-560), in real space
    "full_4x4": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=150.0,
                     material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=28,
                     illum=dict(jones=(1, 0)),
                     transfer=dict(method="4x4", diffraction=np.inf, beta=0.0, phi=0.0)),
    "full_4x4_offaxis_nstep2_bulk": dict(shape=(10, 12), nlayers=2, wavelengths=[550.0], pixelsize=200.0,
                                         material=("twisted", dict(thickness=2.0)), seed=29,
                                         illum=dict(beta=0.1, phi=0.4),
                                         transfer=dict(method="4x4", diffraction=np.inf, nstep=2, beta=0.1,
                                                       phi=0.4, ret_bulk=True)),
    "full_4x4_biaxial_multiray": dict(shape=(10, 10), nlayers=2, wavelengths=[520.0, 600.0], pixelsize=150.0,
                                      material=("biaxial", dict()), seed=30,
                                      illum=dict(beta=[0.0, 0.15], phi=[0.0, 0.5], jones=(1, 0)),
                                      transfer=dict(method="4x4", diffraction=np.inf, multiray=True,
                                                    reflection=2, beta=[0.0, 0.15], phi=[0.0, 0.5])),
    # npass > 1 on the real-space paths (beta 0: the reference warns that the
    # 4x4 method without diffraction does not support npass > 1 off axis; with
    # npass > 1 reflection resolves to 1, so mode 2 is asked for explicitly)
    "nodiff_4x4_npass3": dict(shape=(12, 10), nlayers=3, wavelengths=[500.0, 650.0], pixelsize=100.0,
                              material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=31,
                              illum=dict(),
                              transfer=dict(method="4x4", diffraction=0, reflection=2, npass=3, beta=0.0, phi=0.0)),
    "full_4x4_npass2": dict(shape=(10, 12), nlayers=2, wavelengths=[550.0], pixelsize=150.0,
                            material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=32,
                            illum=dict(jones=(1, 0)),
                            transfer=dict(method="4x4", diffraction=np.inf, npass=2, beta=0.0, phi=0.0)),
    # reflection mode 4 (dtmm/propagate_4x4.py:55-77, :233-287): real space,
    # F P F^-1 half steps around the corrected field diffraction matrix
    "refl4_4x4_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                         material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=33,
                         illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                         transfer=dict(method="4x4", diffraction=1, reflection=4, beta=0.1, phi=0.3)),
    "refl4_4x4_d3_nstep2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(thickness=2.0)), seed=34,
                                illum=dict(),
                                transfer=dict(method="4x4", diffraction=3, reflection=4, nstep=2, beta=0.0,
                                              phi=0.0)),
    "refl4_4x4_d1_npass3": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=35,
                                illum=dict(jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, reflection=4, npass=3, beta=0.0,
                                              phi=0.0)),
    # reflection mode 2 with diffraction (dtmm/propagate_4x4.py:18-52, :156-230):
    # E P F^-1 and F P E^-1 half steps around the corrected E matrices of the
    # forward and backward modes
    "refl2_4x4_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                         material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=36,
                         illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                         transfer=dict(method="4x4", diffraction=1, reflection=2, beta=0.1, phi=0.3)),
    "refl2_4x4_d3_nstep2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(thickness=2.0)), seed=37,
                                illum=dict(),
                                transfer=dict(method="4x4", diffraction=3, reflection=2, nstep=2, beta=0.0,
                                              phi=0.0)),
    "refl2_4x4_d1_npass3": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=38,
                                illum=dict(jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, reflection=2, npass=3, beta=0.0,
                                              phi=0.0)),
    # reflection mode 3 (dtmm/propagate_4x4.py:135-153, :447-512): k-space,
    # C . D and D . C field diffraction matrices around F P F^-1
    "refl3_4x4_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                         material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=39,
                         illum=dict(beta=0.1, phi=0.3, jones=(1, 0)),
                         transfer=dict(method="4x4", diffraction=1, reflection=3, beta=0.1, phi=0.3)),
    "refl3_4x4_d3_nstep2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(thickness=2.0)), seed=40,
                                illum=dict(),
                                transfer=dict(method="4x4", diffraction=3, reflection=3, nstep=2, beta=0.0,
                                              phi=0.0)),
    "refl3_4x4_d1_npass3": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=41,
                                illum=dict(jones=(1, 0)),
                                transfer=dict(method="4x4", diffraction=1, reflection=3, npass=3, beta=0.0,
                                              phi=0.0)),
    # reflection modes 2-4 with diffraction and several rays (tables per ray)
    "refl4_4x4_d1_multiray": dict(shape=(10, 12), nlayers=2, wavelengths=[520.0, 600.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=42,
                                  illum=dict(beta=[0.0, 0.15], phi=[0.0, 0.5], jones=(1, 0)),
                                  transfer=dict(method="4x4", diffraction=1, reflection=4, multiray=True,
                                                beta=[0.0, 0.15], phi=[0.0, 0.5])),
    "refl2_4x4_d3_multiray": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=43,
                                  illum=dict(beta=[0.0, 0.1], phi=[0.0, 1.0], jones=(1, 0)),
                                  transfer=dict(method="4x4", diffraction=3, reflection=2, multiray=True,
                                                beta=[0.0, 0.1], phi=[0.0, 1.0])),
    "refl3_4x4_d1_multiray": dict(shape=(10, 10), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=44,
                                  illum=dict(beta=[0.05, 0.2], phi=[0.3, -0.4]),
                                  transfer=dict(method="4x4", diffraction=1, reflection=3, multiray=True,
                                                beta=[0.05, 0.2], phi=[0.3, -0.4])),
    "nodiff_4x4_biaxial": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                               material=("biaxial", dict()), seed=27,
                               illum=dict(beta=0.15, phi=0.4, jones=(1, 0)),
                               transfer=dict(method="4x4", diffraction=0, beta=0.15, phi=0.4)),

    # 2x2 in real space: no diffraction (reflection resolves to 0), and
    # reflection mode 2 with windows (dtmm/propagate_2x2.py:91-190, :286-377)
    "twox2_d0": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                     material=("twisted", dict()), seed=47,
                     illum=dict(beta=0.1, phi=0.3),
                     transfer=dict(method="2x2", diffraction=0, beta=0.1, phi=0.3)),
    "twox2_d3_refl2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                           material=("twisted", dict()), seed=48,
                           illum=dict(jones=(1, 0)),
                           transfer=dict(method="2x2", diffraction=3, reflection=2, beta=0.0, phi=0.0)),
    "twox2_npass2_d3": dict(shape=(10, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                            material=("twisted", dict()), seed=49,
                            illum=dict(jones=(1, 0)),
                            transfer=dict(method="2x2", diffraction=3, npass=2, beta=0.0, phi=0.0)),
    "twox2_npass3_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 600.0], pixelsize=100.0,
                            material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=45,
                            illum=dict(jones=(1, 0)),
                            transfer=dict(method="2x2", diffraction=1, npass=3, beta=0.0, phi=0.0)),
    "twox2_npass2_d3_offaxis": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                    material=("twisted", dict()), seed=46,
                                    illum=dict(beta=0.1, phi=0.4),
                                    transfer=dict(method="2x2", diffraction=3, reflection=1, npass=2, beta=0.1,
                                                  phi=0.4)),
    # more of the 2x2 option space: reflection 1 without diffraction (k-space, the
    # interfaces' betamax cut only; with npass > 1 the reference itself fails), reflection 2 without and with
    # diffraction matrices and tracked waves, several rays, sub-steps with windows,
    # biaxial voxels in real space
    "twox2_refl1_d0": dict(shape=(12, 16), nlayers=3, wavelengths=[500.0, 600.0], pixelsize=100.0,
                           material=("twisted", dict()), seed=50,
                           illum=dict(beta=0.1, phi=0.3),
                           transfer=dict(method="2x2", diffraction=0, reflection=1, beta=0.1, phi=0.3)),
    "twox2_refl2_d0_npass2": dict(shape=(12, 10), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                  material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=51,
                                  illum=dict(beta=0.15, phi=1.1),
                                  transfer=dict(method="2x2", diffraction=0, reflection=2, npass=2, beta=0.15,
                                                phi=1.1)),
    "twox2_refl2_d1": dict(shape=(14, 12), nlayers=3, wavelengths=[480.0, 640.0], pixelsize=100.0,
                           material=("twisted", dict()), seed=52,
                           illum=dict(beta=0.1, phi=0.2, jones=(1, 0)),
                           transfer=dict(method="2x2", diffraction=1, reflection=2, beta=0.1, phi=0.2)),
    "twox2_refl2_d1_npass3": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                  material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=53,
                                  illum=dict(jones=(1, 0)),
                                  transfer=dict(method="2x2", diffraction=1, reflection=2, npass=3, beta=0.0,
                                                phi=0.0)),
    "twox2_npass2_multiray": dict(shape=(16, 16), nlayers=2, wavelengths=[520.0, 620.0], pixelsize=100.0,
                                  material=("twisted", dict()), seed=54,
                                  illum=dict(beta=[0.0, 0.1], phi=[0.0, np.pi / 2], jones=(1, 0)),
                                  transfer=dict(method="2x2", diffraction=1, npass=2, multiray=True,
                                                beta=[0.0, 0.1], phi=[0.0, np.pi / 2])),
    "twox2_npass2_d3_nstep2": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                   material=("twisted", dict(thickness=2.0)), seed=55,
                                   illum=dict(jones=(1, 0)),
                                   transfer=dict(method="2x2", diffraction=3, reflection=1, npass=2, nstep=2,
                                                 beta=0.0, phi=0.0)),
    "twox2_refl2_d3_nstep2_npass2": dict(shape=(10, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                         material=("twisted", dict(thickness=2.0)), seed=56,
                                         illum=dict(jones=(1, 0)),
                                         transfer=dict(method="2x2", diffraction=3, npass=2, nstep=2, beta=0.0,
                                                       phi=0.0)),
    # ret_bulk: every layer's field (E and H) inside the stack
    "twox2_bulk_d1": dict(shape=(12, 14), nlayers=3, wavelengths=[500.0, 610.0], pixelsize=100.0,
                          material=("twisted", dict()), seed=58,
                          illum=dict(beta=0.1, phi=0.4),
                          transfer=dict(method="2x2", diffraction=1, beta=0.1, phi=0.4, ret_bulk=True)),
    "twox2_bulk_d1_npass2": dict(shape=(12, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                 material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=59,
                                 illum=dict(jones=(1, 0)),
                                 transfer=dict(method="2x2", diffraction=1, npass=2, beta=0.0, phi=0.0,
                                               ret_bulk=True)),
    "twox2_bulk_refl2_d3": dict(shape=(12, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                material=("twisted", dict()), seed=60,
                                illum=dict(jones=(1, 0)),
                                transfer=dict(method="2x2", diffraction=3, reflection=2, beta=0.0, phi=0.0,
                                              ret_bulk=True)),
    "twox2_bulk_refl2_d1_npass3": dict(shape=(10, 12), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                       material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=61,
                                       illum=dict(beta=0.1, phi=1.0, jones=(1, 0)),
                                       transfer=dict(method="2x2", diffraction=1, reflection=2, npass=3, beta=0.1,
                                                     phi=1.0, ret_bulk=True)),
    "twox2_bulk_d0": dict(shape=(10, 12), nlayers=3, wavelengths=[500.0, 620.0], pixelsize=100.0,
                          material=("twisted", dict()), seed=62,
                          illum=dict(beta=0.1, phi=0.3),
                          transfer=dict(method="2x2", diffraction=0, beta=0.1, phi=0.3, ret_bulk=True)),
    # 2x2 with diffraction = inf: every in-band eigenwave exactly, without and with
    # interfaces (reflection 2), tracked reflections (npass 2), ret_bulk, biaxial voxels
    "twox2_modal": dict(shape=(10, 12), nlayers=2, wavelengths=[500.0, 620.0], pixelsize=100.0,
                       material=("twisted", dict()), seed=63,
                       illum=dict(beta=0.1, phi=0.3),
                       transfer=dict(method="2x2", diffraction=np.inf, beta=0.1, phi=0.3)),
    "twox2_modal_refl2": dict(shape=(8, 10), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                             material=("twisted", dict(no=1.5, ne=1.7, amplitude=0.3)), seed=64,
                             illum=dict(jones=(1, 0)),
                             transfer=dict(method="2x2", diffraction=np.inf, reflection=2, beta=0.0, phi=0.0)),
    "twox2_modal_npass2_bulk": dict(shape=(8, 8), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                                   material=("twisted", dict()), seed=65,
                                   illum=dict(beta=0.1, phi=0.7, jones=(1, 0)),
                                   transfer=dict(method="2x2", diffraction=np.inf, npass=2, beta=0.1, phi=0.7,
                                                 ret_bulk=True)),
    "twox2_modal_biaxial": dict(shape=(8, 10), nlayers=2, wavelengths=[520.0], pixelsize=100.0,
                               material=("biaxial", dict()), seed=66,
                               illum=dict(jones=(1, 0)),
                               transfer=dict(method="2x2", diffraction=np.inf, reflection=2, beta=0.0, phi=0.0)),
    # the reference's modal 2x2 step advances one sub-step (d / nstep) per layer
    "twox2_modal_nstep2": dict(shape=(10, 8), nlayers=2, wavelengths=[480.0, 590.0], pixelsize=100.0,
                               material=("twisted", dict(amplitude=0.4)), seed=67,
                               illum=dict(beta=0.05, phi=1.1),
                               transfer=dict(method="2x2", diffraction=np.inf, nstep=2, beta=0.05, phi=1.1)),
    "twox2_modal_blocks_npass3": dict(shape=(8, 10), nlayers=3, wavelengths=[550.0], pixelsize=100.0,
                                      blocks=[("twisted", dict(no=1.45, ne=1.6), 1), ("twisted", dict(amplitude=0.5), 2)],
                                      seed=68,
                                      illum=dict(jones=(0, 1)),
                                      transfer=dict(method="2x2", diffraction=np.inf, npass=3, beta=0.0, phi=0.0)),
    "twox2_d0_biaxial": dict(shape=(10, 12), nlayers=2, wavelengths=[550.0], pixelsize=100.0,
                             material=("biaxial", dict()), seed=57,
                             illum=dict(beta=0.1, phi=0.5),
                             transfer=dict(method="2x2", diffraction=0, beta=0.1, phi=0.5)),
}


# every case with a reference fixture is also a GPU parity case
ORACLE_CASES = {}


def build_optical_data(case):
    """The case's optical data: one block, or with ``blocks`` = [(kind, kwargs,
    layers), ...] several blocks of their own materials and effective media."""
    if "blocks" in case:
        return [MATERIALS[k](case["shape"], nl, case["seed"] + i, **kw) for i, (k, kw, nl) in enumerate(case["blocks"])]
    kind, kw = case["material"]
    return [MATERIALS[kind](case["shape"], case["nlayers"], case["seed"], **kw)]


def build_inputs(case, illumination_data):
    illum = dict(case["illum"])
    field_data = illumination_data(case["shape"], case["wavelengths"], pixelsize=case["pixelsize"], **illum)
    return field_data, build_optical_data(case)


# illumination_data cases (dtmm/field.py:586): the batch workload's seven rays
# (negative beta as |beta| with phi + pi), a focus offset, backward waves and
# a cover index of 1
ILLUM_CASES = {
    "rays7": dict(shape=(64, 64), wavelengths=[400.0, 550.0, 700.0], pixelsize=100.0,
                  beta=[0.0, 0.1, 0.1, 0.2, 0.2, 0.1, 0.1],
                  phi=[0.0, 0.0, np.pi, 0.0, np.pi, np.pi / 2, 1.5 * np.pi]),
    "rays7_jones": dict(shape=(48, 40), wavelengths=[450.0, 600.0], pixelsize=100.0,
                        beta=[0.0, 0.1, 0.1, 0.2, 0.2, 0.1, 0.1],
                        phi=[0.0, 0.0, np.pi, 0.0, np.pi, np.pi / 2, 1.5 * np.pi], jones=(1, 1j)),
    "focus": dict(shape=(32, 36), wavelengths=[500.0, 650.0], pixelsize=80.0, beta=0.3, phi=0.4, focus=7.5),
    "backdir": dict(shape=(30, 24), wavelengths=[550.0], pixelsize=100.0, beta=0.15, phi=-0.8, backdir=True,
                    jones=(0, 1)),
    "cover1": dict(shape=(20, 20), wavelengths=[550.0, 600.0], pixelsize=120.0, beta=0.25, phi=2.0, n=1.0,
                   intensity=2.5),
    "big_beta": dict(shape=(16, 24), wavelengths=[500.0], pixelsize=100.0, beta=[0.5, 0.7], phi=[0.1, 3.0],
                     jones=(1, 0)),
}


# POM image formation cases on transferred fields of the cases above
# (dtmm/field_viewer.py:70 calculate_pom_field, dtmm/field.py field2specter,
# dtmm/color.py specter2color with the reference's own load_tcmf):
#   source   golden case whose field_out is the input
#   jvec     polarizer (jones vector, optional frame rotation) combining x / y inputs
#   analyzer analyzer jones vector and the rotation of its matrix
#   window   multiply by a separable raised-cosine window
#   dmat_d   refocus by d pixels in a cover of index 1.5 (field_diffraction_matrix)
#   summed   field2spectersum over the leading (ray) axis
POM_CASES = {
    "pom_crossed": dict(source="cfg1_small", jvec=((1, 0), 0.0), analyzer=((0, 1), 0.0)),
    "pom_rotated": dict(source="cfg1_small", jvec=((1, 0), np.pi / 8), analyzer=((1, 1), 0.3), window=True,
                        dmat_d=2.0),
    "pom_rays_summed": dict(source="fourx4_multiray", jvec=None, analyzer=((0, 1), 0.0), summed=True),
}


def raised_cosine_window(shape):
    """Separable window 0.5 - 0.5 cos(2 pi (i + 0.5) / n) on both axes."""
    wy, wx = (0.5 - 0.5 * np.cos(2 * np.pi * (np.arange(n) + 0.5) / n) for n in shape)
    return wy[:, None] * wx[None, :]


# illumination_rays (dtmm/field.py:371): (NA, diameter, smooth)
RAYS_CASES = {
    "na02_d5": (0.2, 5, 0.1),
    "na03_d7": (0.3, 7.4, 0.0),
    "na015_annulus": (0.15, (2, 6), 0.2),
    "na025_d9_soft": (0.25, 9, 0.5),
    "na01_d4_clip": (0.1, 4, 1.5),
}

# window functions (dtmm/window.py): name -> (function, args)
WINDOW_CASES = {
    "aperture_full": ("aperture", ((32, 40), 1.0, 0.05)),
    "aperture_small": ("aperture", ((24, 24), 0.6, 0.2)),
    "aperture_annulus": ("aperture", ((30, 26), (0.3, 0.9), 0.1)),
    "aperture_hard": ("aperture", ((17, 19), 0.8, 0.0)),
    "blackman": ("blackman", ((32, 40),)),
    "gaussian": ("gaussian", ((20, 28), 0.6)),
}

# windowed illumination_data (dtmm/field.py:586 with a window): the window is
# one of WINDOW_CASES (the reference's own array); rays may come from RAYS_CASES
ILLUM_WINDOW_CASES = {
    "win_blackman": dict(shape=(32, 40), wavelengths=[500.0, 600.0], pixelsize=100.0, beta=0.1, phi=0.3,
                         window="blackman"),
    "win_rays_focus": dict(shape=(24, 24), wavelengths=[550.0], pixelsize=80.0, rays="na015_annulus",
                           window="aperture_small", focus=3.0),
    "win_backdir_jones": dict(shape=(20, 28), wavelengths=[450.0, 650.0], pixelsize=100.0, beta=0.2, phi=-1.0,
                              jones=(1, 1j), backdir=True, window="gaussian", n=1.0),
    "win_no_diffraction": dict(shape=(30, 26), wavelengths=[600.0], pixelsize=90.0, beta=0.05, phi=2.0,
                               window="aperture_annulus", diffraction=False, intensity=3.0),
}

# load_tcmf (dtmm/color.py:257) options
TCMF_CASES = {
    "default": dict(),
    "nine": dict(wavelengths=list(np.linspace(380.0, 780.0, 9))),
    "single": dict(wavelengths=[550.0]),
    "seven_norm2": dict(wavelengths=list(np.linspace(400.0, 700.0, 7)), norm=2),
    "five_single_wavelength": dict(wavelengths=list(np.linspace(380.0, 780.0, 5)), single_wavelength=True),
    "eleven_norm0": dict(wavelengths=list(np.linspace(450.0, 650.0, 11)), norm=0),
    "illuminant_a": dict(wavelengths=list(np.linspace(380.0, 780.0, 9)), illuminant="A"),
    "cie1964": dict(wavelengths=list(np.linspace(400.0, 700.0, 13)), cmf="CIE1964"),
    "cmos": dict(wavelengths=list(np.linspace(400.0, 700.0, 9)), cmf="CMOS"),
}
TCMF_TABLES = {"CIE1931": "CIE1931XYZ.dat", "CIE1964": "CIE1964XYZ.dat", "CMOS": "CMOSY.dat", "D65": "D65.dat",
               "A": "A.dat"}
