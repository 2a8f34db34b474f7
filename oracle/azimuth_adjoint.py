"""FP64 numpy restatement of the differentiable azimuth chain and its
adjoint.  TEST INFRASTRUCTURE ONLY: the reference gradient the CUDA adjoint
(s1g_azimuth_adjoint) is checked against; nothing here is shipped.

The reference has no gradients or autofocus; the chain is the range-Doppler
(stripmap) azimuth processing of one range-compressed burst X[a][r]:

  U[a][r] = X[a][r] exp(-i phi_a),  phi_a = sum_j theta_j x_a^(j+2),
            x_a = linspace(-1, 1, n_a)                  (phase-error multiply)
  V       = FFT_az(U)                                   (azimuth FFT, per range bin)
  f_k     = nu_k + f_c, nu_k the FFT bin frequency in [-prf/2, prf/2)
  D_k     = sqrt(1 - lambda^2 f_k^2 / (4 v^2))
  W[k]    = IFFT_r(FFT_r(V[k]) exp(i beta_k f_r)),  beta_k = 4 pi R_ref (1/D_k - 1) / c   (RCMC)
  Z[k][r] = W[k][r] exp(-i (4 pi / lambda) R_r (1 - D_k))  (azimuth matched filter, the
            constant per-range-bin phase 4 pi R_r / lambda of exp(i 4 pi R_r D_k / lambda) left out)
  Y       = IFFT_az(Z)                                  (1/n_a)
  L       = -sum p ln p,  p = |Y|^2 / sum |Y|^2          (image entropy)

Gradients dL/dtheta_j and dL/df_c by reverse mode (complex gradient
G = dL/dRe + i dL/dIm; a linear map's adjoint carries it back).
"""
from __future__ import annotations

import numpy as np

C = 299792458.0
CARRIER = 5.405000454334350e+09


def frequencies(n_a: int, prf: float, f_c: float) -> np.ndarray:
    k = np.arange(n_a)
    nu = np.where(k < (n_a + 1) // 2, k, k - n_a) * prf / n_a
    return nu + f_c


def range_freqs(n_r: int, fs: float) -> np.ndarray:
    f = np.arange(n_r)
    return np.where(f < (n_r + 1) // 2, f, f - n_r) * fs / n_r


def _geometry(n_a, prf, f_c, v, lam, r_ref):
    f = frequencies(n_a, prf, f_c)
    x = lam * lam * f * f / (4.0 * v * v)
    D = np.sqrt(1.0 - x)
    omd = x / (1.0 + D)                       # 1 - D without cancellation
    beta = 4.0 * np.pi * r_ref * (omd / D) / C
    return f, D, omd, beta


def forward(X, theta, f_c, prf, fs, v, slant):
    """Entropy of the focused image and the intermediates the adjoint needs."""
    n_a, n_r = X.shape
    lam = C / CARRIER
    xa = np.linspace(-1.0, 1.0, n_a)
    phi = sum(t * xa ** (j + 2) for j, t in enumerate(theta))
    U = X * np.exp(-1j * phi)[:, None]
    V = np.fft.fft(U, axis=0)
    f, D, omd, beta = _geometry(n_a, prf, f_c, v, lam, slant[n_r // 2])
    fr = range_freqs(n_r, fs)
    QM = np.fft.fft(V, axis=1) * np.exp(1j * beta[:, None] * fr[None, :])
    W = np.fft.ifft(QM, axis=1)
    Z = W * np.exp(-1j * (4.0 * np.pi / lam) * slant[None, :] * omd[:, None])
    Y = np.fft.ifft(Z, axis=0)
    I = np.abs(Y) ** 2
    S = I.sum()
    p = I / S
    with np.errstate(divide="ignore", invalid="ignore"):
        plogp = np.where(p > 0, p * np.log(p), 0.0)
    L = -plogp.sum()
    return L, dict(U=U, QM=QM, Z=Z, Y=Y, I=I, S=S, H=plogp.sum(), f=f, D=D, omd=omd, beta=beta, fr=fr, xa=xa,
                   lam=lam, slant=slant, v=v)


def gradient(X, theta, f_c, prf, fs, v, slant):
    """(L, dL/dtheta, dL/df_c)."""
    L, c = forward(X, theta, f_c, prf, fs, v, slant)
    n_a, n_r = X.shape
    I, S, H, Y = c["I"], c["S"], c["H"], c["Y"]
    with np.errstate(divide="ignore"):
        logI = np.where(I > 0, np.log(np.where(I > 0, I, 1.0)), 0.0)
    dEdI = -(logI - np.log(S) - H) / S
    GY = 2.0 * Y * np.where(I > 0, dEdI, 0.0)
    GZ = np.fft.fft(GY, axis=0) / n_a                     # adjoint of IFFT_az (1/n_a)
    lam, slant, D, f, fr, v = c["lam"], c["slant"], c["D"], c["f"], c["fr"], c["v"]
    Z = c["Z"]
    a_k = -(4.0 * np.pi / lam) * (np.imag(np.conj(GZ) * Z) * slant[None, :]).sum(axis=1)
    GW = GZ * np.exp(1j * (4.0 * np.pi / lam) * slant[None, :] * c["omd"][:, None])
    F = np.fft.fft(GW, axis=1)
    b_k = -(np.imag(np.conj(F) * c["QM"]) * fr[None, :]).sum(axis=1) / n_r
    M = np.exp(1j * c["beta"][:, None] * fr[None, :])
    GV = np.fft.ifft(np.conj(M) * F, axis=1)
    GU = np.fft.ifft(GV, axis=0) * n_a                   # adjoint of FFT_az (unnormalised)
    dphi = np.imag(np.conj(GU) * c["U"]).sum(axis=1)
    xa = c["xa"]
    g_theta = np.array([(dphi * xa ** (j + 2)).sum() for j in range(len(theta))])
    r_ref = slant[n_r // 2]
    dbeta_dD = -4.0 * np.pi * r_ref / (C * D * D)
    dD_df = -lam * lam * f / (4.0 * v * v * D)
    g_fc = float(((a_k + b_k * dbeta_dD) * dD_df).sum())
    return L, g_theta, g_fc
