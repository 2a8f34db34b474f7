"""The time unfolding's band step as the fused kernel computes it
(csrc/s1g_fast.cu, k_tufr_fused), restated in FP64 numpy and checked against
the reference's direct form (image_formation.cpp:315-333: the length-TS DFT of
the deramped tiled line, the band [start, end) kept, inverse DFT, sampled at
integer positions):

  type 1  y[n] exp(-2 pi i n k_s / TS) gathered onto a grid of M >= 1.25 bw
          points at x_n = n M / TS with the exponential-of-semicircle kernel
          phi (width 13; every grid point takes the samples whose integer
          offset n M - l TS lies within the half-width), forward M-point FFT;
  band    bins p < bw - K0 or p >= M - K0 kept and divided by Phi(p / M)^2;
  type 2  inverse M-point FFT, then z[n] = exp(2 pi i k_s n / TS) / TS *
          sum_l G[l] phi(x_n - l).

Also checks the pass bounds the kernel uses: a pass of L grid points needs at
most (L - 1 + W) TS / M + 1 staged samples.
"""
import math

import numpy as np
import pytest

W = 13


def phi(t, beta):
    z = 2.0 * np.asarray(t, dtype=float) / W
    out = np.zeros_like(z)
    m = np.abs(z) < 1.0
    out[m] = np.exp(beta * (np.sqrt(1.0 - z[m] ** 2) - 1.0))
    return out


def phi_hat(xi, beta):
    x, w = np.polynomial.legendre.leggauss(128)
    t = 0.5 * W * x
    return 0.5 * W * np.sum(w * phi(t, beta) * np.cos(2.0 * np.pi * xi * t))


def window(l, TS, M):
    """First and last sample index within the kernel's half-width of grid point l."""
    lo = -((-(2 * l - W) * TS) // (2 * M))
    hi = ((2 * l + W) * TS) // (2 * M)
    return lo, hi


def direct(y, start, end):
    TS = y.size
    Z = np.fft.fft(y)
    Zb = np.zeros_like(Z)
    Zb[start:end] = Z[start:end]
    return np.fft.ifft(Zb)


def nufft_band(y, start, end, M, at):
    TS = y.size
    bw = end - start
    K0 = bw // 2
    ks = start + K0
    beta = 0.97 * math.pi * W * (1.0 - 1.0 / (2.0 * (M / bw)))
    n = np.arange(TS)
    yp = y * np.exp(-2j * np.pi * ((n * ks) % TS) / TS)
    G = np.zeros(M, complex)
    for l in range(M):
        lo, hi = window(l, TS, M)
        nn = np.arange(lo, hi + 1)
        G[l] = np.sum(phi((nn * M - l * TS) / TS, beta) * yp[nn % TS])
    F = np.fft.fft(G)
    band = np.zeros(M)
    for p in range(M):
        if p < bw - K0 or p >= M - K0:
            band[p] = 1.0 / phi_hat((p if p < bw - K0 else p - M) / M, beta) ** 2
    G2 = np.fft.ifft(F * band) * M          # unnormalised inverse
    out = []
    for q in at:
        x = q * M / TS
        l = np.arange(math.ceil(x - W / 2), math.floor(x + W / 2) + 1)
        v = np.sum(G2[l % M] * phi(x - l, beta))
        out.append(v * np.exp(2j * np.pi * ((q * ks) % TS) / TS) / TS)
    return np.array(out)


@pytest.mark.parametrize("T,S,bw,M", [(3, 500, 301, 384), (6, 331, 400, 512), (2, 777, 1100, 1400)])
def test_two_ended_nufft_matches_the_direct_band(T, S, bw, M):
    assert 4 * bw <= 5 * M
    rng = np.random.default_rng(T * 1000 + S)
    TS = T * S
    y = rng.standard_normal(TS) + 1j * rng.standard_normal(TS)
    mid = TS // 2
    start, end = mid - bw // 2, mid - bw // 2 + bw
    at = rng.integers(0, TS, 64)
    ref = direct(y, start, end)[at]
    got = nufft_band(y, start, end, M, at)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 1e-6, err


@pytest.mark.parametrize("T,S,M", [(6, 6908, 9216), (7, 7500, 10240), (2, 300, 640), (3, 200, 160)])
def test_pass_bounds(T, S, M):
    """Every pass's staged samples fit the chunk the kernel sizes them for,
    and every grid point's window lies inside its pass's samples."""
    TS = T * S
    cap = 7120
    lmax = ((cap - 2) * M) // TS - W + 1
    assert lmax >= 1
    Lc = (lmax // 1024) * 1024 if lmax >= 1024 else lmax
    for l0 in range(0, M, Lc):
        l1 = min(M, l0 + Lc)
        nA = window(l0, TS, M)[0]
        nB = window(l1 - 1, TS, M)[1]
        assert nB - nA + 1 <= cap
        assert -TS < nA and nB < 2 * TS
        for l in (l0, l1 - 1):
            lo, hi = window(l, TS, M)
            assert nA <= lo and hi <= nB
