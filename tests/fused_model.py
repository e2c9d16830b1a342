"""numpy model of the engine's fused layer sweep (test infrastructure).

Restates, in plain numpy, the restructured algorithm that the CUDA kernels
run, so that the restructuring itself can be checked against the oracle on
the CPU:

* consecutive half-step diffraction operators D1(j+1) . D2(j) merge into a
  diagonal (e+, e-) per k for an isotropic effective medium;
* the beam-phase correction C_w is a scalar per direction and folds into the
  per-voxel phases: C_w E P E^-1 C_w = E diag(exp(i k0 d (alpha_m -/+ a_w))) E^-1;
* the tent windows are separable, cx_i(beta_x) * cy_j(beta_y), and the
  forward FFT after the real-space step is shared by all windows.

Only the 4x4 / npass = 1 and 2x2 / reflection 0-1 / npass = 1 paths are
modelled (enough to pin the restructuring); tables come from the oracle.
"""
import numpy as np

import dtmm_oracle as O


def voxel_records(beta, phi, epsv, epsa, d, eps_eff):
    """E blocks (rows Ex, Ey; columns modes), 1/det and phase arguments per voxel."""
    beta = float(beta)
    phi = float(phi)
    alpha, F = O.alphaf(beta, phi, epsv, epsa)  # normalised columns; the model does not rely on scaling
    aw = np.sqrt(complex(eps_eff) - beta ** 2)
    Ef = np.stack([np.stack([F[..., 0, 0], F[..., 0, 2]], -1), np.stack([F[..., 2, 0], F[..., 2, 2]], -1)], -2)
    Eb = np.stack([np.stack([F[..., 0, 1], F[..., 0, 3]], -1), np.stack([F[..., 2, 1], F[..., 2, 3]], -1)], -2)
    phf = d * (alpha[..., [0, 2]] - aw)
    phb = d * (alpha[..., [1, 3]] + aw)
    return Ef, phf, Eb, phb


def apply_block(E, ph, k, h0, h1):
    Ei = np.linalg.inv(E)
    p = np.exp(1j * k[..., None] * ph)
    w0 = Ei[..., 0, 0] * h0 + Ei[..., 0, 1] * h1
    w1 = Ei[..., 1, 0] * h0 + Ei[..., 1, 1] * h1
    w0 = w0 * p[..., 0]
    w1 = w1 * p[..., 1]
    return E[..., 0, 0] * w0 + E[..., 0, 1] * w1, E[..., 1, 0] * w0 + E[..., 1, 1] * w1


def transfer_4x4_fused(field_in, wavelengths, pixelsize, block, beta=0.0, phi=0.0, diffraction=1, betamax=0.8,
                       nin=1.5, nout=1.5):
    d_arr, epsv, epsa = O.validate_optical_block(block, field_in.shape[-2:])
    ks = O.k0(wavelengths, pixelsize)
    H, W = field_in.shape[-2:]
    epsv_full = np.broadcast_to(epsv, (len(d_arr), H, W, 3))
    epsa_full = np.broadcast_to(epsa, (len(d_arr), H, W, 3))
    eps_eff = O._isotropic_mean(epsv_full)
    n = diffraction
    if n > 1:
        wins, (betas, phis) = O.fft_mask(field_in.shape, ks, n, beta * np.cos(phi), beta * np.sin(phi), betamax)
        # recover the full n x n grid and the separable factors
        bx, by = O.betaxy((H, W), ks)
        dwin = 2 * betamax / (n - 1)
        xoff = O._nearest_offset(np.asarray(beta * np.cos(phi)), dwin)
        yoff = O._nearest_offset(np.asarray(beta * np.sin(phi)), dwin)
        ax = np.linspace(-betamax, betamax, n)
        step = ax[1] - ax[0]
        cx = [O._tent((bx[:, 0, :] - (ax[i] + xoff)) / step, -1 if i == 0 else (1 if i == n - 1 else 0)) for i in range(n)]
        cy = [O._tent((by[:, :, 0] - (ax[j] + yoff)) / step, -1 if j == 0 else (1 if j == n - 1 else 0)) for j in range(n)]
        full_w = O.fft_windows(bx, by, n, beta * np.cos(phi), beta * np.sin(phi), betamax)
        nz = [not np.all(w == 0) for w in full_w]
        wl = []
        k = 0
        for i in range(n):
            for j in range(n):
                if nz[i * n + j]:
                    wl.append((i, j, betas[k], phis[k]))
                    k += 1
    else:
        wl = [(0, 0, beta, phi)]
        cx = [np.ones((len(ks), W))]
        cy = [np.ones((len(ks), H))]
    L = len(d_arr)
    kk = ks[:, None, None]
    S = O.fft2(field_in)
    T = O.dotmf(O.first_Epn_diffraction_matrix((H, W), ks, d_arr[0] / 2, [eps_eff] * 3, (0, 0, 0), betamax), S)
    for l in range(L):
        r = np.zeros_like(T)
        for (i, j, bw, pw) in wl:
            h = O.ifft2(T * cx[i][:, None, None, :] * cy[j][:, None, :, None])
            Ef, phf, Eb, phb = voxel_records(bw, pw, epsv_full[l], epsa_full[l], d_arr[l], eps_eff)
            o0, o2 = apply_block(Ef, phf, kk, h[..., 0, :, :], h[..., 2, :, :])
            o1, o3 = apply_block(Eb, phb, kk, h[..., 1, :, :], h[..., 3, :, :])
            r = r + np.stack([o0, o1, o2, o3], axis=-3)
        X = O.fft2(r)
        if l + 1 < L:
            beta_k, _ = O.betaphi((H, W), ks)
            a = np.sqrt(eps_eff - beta_k ** 2 + 0j)
            dsum = 0.5 * (d_arr[l] + d_arr[l + 1])
            ep = np.where(beta_k >= betamax, 0, np.exp(1j * kk * dsum * a))
            em = np.where(beta_k >= betamax, 0, np.exp(-1j * kk * dsum * a))
            T = np.stack([X[..., 0, :, :] * ep, X[..., 1, :, :] * em, X[..., 2, :, :] * ep, X[..., 3, :, :] * em], -3)
    S = O.dotmf(O.second_Epn_diffraction_matrix((H, W), ks, d_arr[-1] / 2, [eps_eff] * 3, (0, 0, 0), betamax), X)
    return O.ifft2(S)
