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


# ---------------------------------------------------------------- TOPS chain
# The TOPS azimuth chain of one range-compressed IW burst up to the focused
# image before the time-domain unfolding (s1_decoder.cpp:511-682 without
# azimuth_time_ufr, which only regrids the focused burst):
#
#   U     = X exp(-i phi_a)                          phase-error polynomial
#   V     = azimuth_frequency_ufr(U)                 image_formation.cpp:125-219
#   Q     = FFT_r(V)
#   A1    = Q exp(i psi_src),  psi_src = -pi f_r^2 / K_src,
#           K_src = 2 v^2 f_c^3 D^2 / (c R F^2)      image_formation.cpp:422-455
#   B     = IFFT_r(A1) / sqrt((R_ref / R)^3)
#   Z     = B exp(i (psi_rcmc + psi_az)),
#           psi_rcmc = -4 pi f_r (R / D - R) / c, psi_az = 4 pi R D / lambda + 2 pi F tau
#                                                    image_formation.cpp:458-476, s1_decoder.cpp:643-676
#   Y     = IFFT_az(Z) / S,  L = image entropy of Y
#
# with F = f_a + f_dc(R) + delta: delta is the Doppler-centroid offset
# estimated together with the phase error.  f_r is linspace(-f_s/2, f_s/2)
# as the reference pairs it with the range spectrum.


def tops_setup(data: bytes, swath: str = "IW2", burst: int = 0):
    """X (range-compressed burst) and the fixed quantities of the TOPS chain,
    as the oracle's azimuth_compress forms them."""
    import math
    import s1_oracle as O
    d = O.S1Decoder(data)
    pk = d.echo[swath][burst]
    times, poss, vels = d.sv
    first = pk[0]
    X = O.range_compress(data, pk)
    n_a, n_r = X.shape
    slant = np.asarray(first.get_slant_ranges())
    v0 = vels[0]
    v_norm = math.sqrt(v0[0] ** 2 + v0[1] ** 2 + v0[2] ** 2)
    prf = 1 / (first.get_pri() * 1e-6)
    T = float(n_a) / prf
    bd = 675.0 if first.sh["swath_number"] == 11 else 600.0
    fs = first.get_range_sample_rate() * 1e6
    rate = O.doppler_centroid_rate(pk, v_norm)
    dc = O.doppler_centroid_from_sums(O.wrapped_sums(X, rate), first)
    nrep = abs(rate * T / prf)
    S = int(math.floor(nrep * n_a))
    time_delta = T / prf / (float(S) / float(n_a))
    t0 = first.get_time()
    veff = np.zeros((S, n_r))
    for i in range(S):
        p, v = O.interpolate_state(times, poss, vels, t0 + time_delta * i)
        veff[i] = O.effective_velocities(p, math.sqrt(v[0] ** 2 + v[1] ** 2 + v[2] ** 2), slant)
    return X, dict(rate=rate, T=T, prf=prf, bd=bd, dc=dc, S=S, az_freqs=O.linspace(-nrep * prf / 2, nrep * prf / 2, S),
                   veff=veff, slant=slant, fr=O.linspace(-fs / 2, fs / 2, n_r),
                   tc=np.asarray(first.get_timing_corrections()), ref=slant[n_r // 2])


def _tops_factors(g, delta):
    lam = C / CARRIER
    fa = g["az_freqs"][:, None] + g["dc"][None, :] + delta
    v2 = g["veff"] ** 2
    D = np.sqrt(1 - (lam * lam * fa * fa) / (4 * v2))
    dD = -(lam * lam * fa) / (4 * v2 * D)
    R = g["slant"][None, :]
    fr = g["fr"][None, :]
    K = np.pi * C * R / (2 * v2 * CARRIER ** 3)            # psi_src = -fr^2 K F^2 / D^2
    psi_src = -fr * fr * K * fa * fa / (D * D)
    dpsi_src = -fr * fr * K * (2 * fa / (D * D) - 2 * fa * fa * dD / D ** 3)
    psi_post = -4 * np.pi * fr * (R / D - R) / C + 4 * np.pi * R * D / lam + 2 * np.pi * fa * g["tc"][None, :]
    dpsi_post = 4 * np.pi * fr * R * dD / (C * D * D) + 4 * np.pi * R * dD / lam + 2 * np.pi * g["tc"][None, :]
    scale = 1.0 / np.sqrt((g["ref"] / g["slant"]) ** 3)
    return psi_src, dpsi_src, psi_post, dpsi_post, scale


def _ufr_parts(g, n_a):
    import math
    import s1_oracle as O
    nrep = abs(g["rate"] * g["T"] / g["prf"])
    S = g["S"]
    mid = S // 2
    start = int(mid - (math.floor(g["bd"]) / 2))
    end = int(mid + (math.floor(g["bd"]) / 2))
    f = O.linspace(-nrep * g["prf"] / 2, nrep * g["prf"] / 2, S)
    der = np.exp(1j * (-np.pi * (1 / g["rate"])) * f * f)
    offset = int(math.floor(nrep))
    tile_len = offset * n_a
    if math.floor(nrep) != nrep:
        tile_len += int(math.floor((nrep - math.floor(nrep)) * n_a))
    return start, end, der, min(tile_len, S)


def tops_forward(X, theta, delta, g):
    import s1_oracle as O
    n_a, n_r = X.shape
    S = g["S"]
    xa = np.linspace(-1.0, 1.0, n_a)
    phi = sum(t * xa ** (j + 2) for j, t in enumerate(theta))
    U = X * np.exp(-1j * phi)[:, None]
    V = O.azimuth_frequency_ufr(U, g["rate"], g["T"], g["prf"], g["bd"])
    psi_src, dpsi_src, psi_post, dpsi_post, scale = _tops_factors(g, delta)
    A1 = np.fft.fft(V, axis=1) * np.exp(1j * psi_src)
    B = np.fft.ifft(A1, axis=1) * n_r * scale[None, :]
    Z = B * np.exp(1j * psi_post)
    Y = np.fft.ifft(Z, axis=0)          # unnormalised IFFT x 1/S
    I = np.abs(Y) ** 2
    Ssum = I.sum()
    p = I / Ssum
    with np.errstate(divide="ignore", invalid="ignore"):
        plogp = np.where(p > 0, p * np.log(p), 0.0)
    return -plogp.sum(), dict(U=U, A1=A1, Z=Z, Y=Y, I=I, S=Ssum, H=plogp.sum(), xa=xa, psi_src=psi_src,
                              dpsi_src=dpsi_src, psi_post=psi_post, dpsi_post=dpsi_post, scale=scale)


def tops_gradient(X, theta, delta, g):
    """(L, dL/dtheta, dL/ddelta) of the TOPS chain by reverse mode."""
    L, c = tops_forward(X, theta, delta, g)
    n_a, n_r = X.shape
    S = g["S"]
    I, Ssum, H, Y = c["I"], c["S"], c["H"], c["Y"]
    with np.errstate(divide="ignore"):
        logI = np.where(I > 0, np.log(np.where(I > 0, I, 1.0)), 0.0)
    GY = 2.0 * Y * np.where(I > 0, -(logI - np.log(Ssum) - H) / Ssum, 0.0)
    GZ = np.fft.fft(GY, axis=0) / S                       # adjoint of IFFT_az / S
    g_delta = float(-(np.imag(np.conj(GZ) * c["Z"]) * c["dpsi_post"]).sum())
    GB = GZ * np.exp(-1j * c["psi_post"]) * c["scale"][None, :]
    GA1 = np.fft.fft(GB, axis=1)                          # adjoint of the unnormalised IFFT_r
    g_delta += float(-(np.imag(np.conj(GA1) * c["A1"]) * c["dpsi_src"]).sum())
    GV = np.fft.ifft(GA1 * np.exp(-1j * c["psi_src"]), axis=1) * n_r   # adjoint of FFT_r
    # adjoint of the frequency unfolding: re-ramp, (1/S) IFFT_S, band move,
    # FFT_S, deramp, tiling, fftshift, FFT_az -- each by its adjoint, reversed
    start, end, der, tile_len = _ufr_parts(g, n_a)
    bw = end - start
    Gz = GV * np.conj(1.0 / der)[:, None]                 # re-ramp = 1 / deramp (unit modulus)
    GZ2 = np.fft.fft(Gz, axis=0) / S
    GYs = np.zeros_like(GZ2)
    GYs[start:end] = GZ2[:bw]
    Gy = np.fft.ifft(GYs, axis=0) * S
    Gy = Gy * np.conj(der)[:, None]
    Gx = np.zeros((n_a, n_r), dtype=np.complex128)
    for s0 in range(0, tile_len, n_a):
        m = min(n_a, tile_len - s0)
        Gx[:m] += Gy[s0:s0 + m]
    Gx = np.roll(Gx, -(n_a // 2), axis=0)                 # adjoint of the fftshift (roll by n_a / 2)
    GU = np.fft.ifft(Gx, axis=0) * n_a                    # adjoint of the unnormalised FFT_az
    dphi = np.imag(np.conj(GU) * c["U"]).sum(axis=1)
    xa = c["xa"]
    g_theta = np.array([(dphi * xa ** (j + 2)).sum() for j in range(len(theta))])
    return L, g_theta, g_delta
