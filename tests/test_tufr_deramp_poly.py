"""The deramp phase of the time unfolding as a per-knot-interval polynomial
(k_tufr_fused's deramp_poly / deramp_rot), restated in float64 and checked
against the direct expression of azimuth_time_ufr (image_formation.cpp:
305-313: -pi kt t^2 + 2 pi (kt + K_a) dct t with t = dct + az_time, which
equals -(tau + dct) [pi kt (tau - dct) + 2 pi f_dc]).

Over the samples n = n_a + d of one knot interval, pi kt and dct are linear in
d (K_a resampled linearly S -> T S) and so is az_time, so the argument is the
cubic H0 + G1 d + G2 d^2 + G3 d^3; the kernel keeps H0 and G1 (the slope
rewritten as dt (C0 + A0 P) + Dd (C0 - A0 P) + A0 Pd B0) and G2, and
evaluates the phase in 32-bit fixed-point turns with the band shift
n k_s / TS as a 64-bit fraction (floor(2^64 (k_s mod TS) / TS)).  Parameter
ranges are those of IW bursts (kt ~ -2e3..-6e3 Hz/s, |f_dc| <= 100 Hz,
focused time ~2.7 s, T S ~ 4e4)."""
import numpy as np

TWO32 = 2.0 ** 32


def _direct(p0, dpk, d0, ddc, al, tau, tpf):
    pkt = p0 + dpk * al
    dct = d0 + ddc * al
    return (tau + dct) * (pkt * (tau - dct) + tpf)


def _poly(p0, dpk, d0, ddc, al_a, tau_a, tpf, dt, g):
    P = p0 + dpk * al_a
    D = d0 + ddc * al_a
    Pd, Dd = dpk * g, ddc * g
    A0, B0 = tau_a + D, tau_a - D
    C0 = P * B0 + tpf
    H0 = A0 * C0
    Q = A0 * P
    G1 = dt * (C0 + Q) + Dd * (C0 - Q) + A0 * Pd * B0
    B1, A1 = dt - Dd, dt + Dd
    C1 = P * B1 + Pd * B0
    G2 = A0 * Pd * B1 + A1 * C1
    G3 = A1 * Pd * B1
    return H0, G1, G2, G3


def _frac_fx(x_turns):
    return np.uint32(np.int64(np.round((x_turns - np.round(x_turns)) * TWO32)) & 0xFFFFFFFF)


def test_interval_polynomial_matches_the_direct_phase():
    rng = np.random.default_rng(7)
    S, T = 6908, 6
    TS = T * S
    ft = 2.7
    dt = ft / (TS - 1)
    g = (S - 1) / (TS - 1)
    worst = 0.0
    worst_g3 = 0.0
    for _ in range(400):
        kt = rng.uniform(-6e3, -2e3)
        fdc = rng.uniform(-100.0, 100.0)
        ka = rng.uniform(-2.5e3, -1.5e3)
        p0 = np.pi * kt
        d0 = -fdc / ka
        # changes of pi kt and dct over one knot interval: 25x the largest on
        # an IW burst (K_a moves ~1.5e-4 relative over the aperture through
        # the F^2 term of the velocity factor, spread over S knots: <= 4e-8)
        dpk = np.pi * kt * rng.uniform(-1e-6, 1e-6)
        ddc = d0 * rng.uniform(-1e-6, 1e-6)
        tpf = 2 * np.pi * fdc
        iv = int(rng.integers(0, S - 1))
        na = -(-iv * (TS - 1) // (S - 1))                  # first sample of the interval
        al_a = (na * (S - 1) - iv * (TS - 1)) / (TS - 1)
        tau_a = -ft / 2 + na * dt
        H0, G1, G2, G3 = _poly(p0, dpk, d0, ddc, al_a, tau_a, tpf, dt, g)
        for d in range(8):
            ref = _direct(p0, dpk, d0, ddc, al_a + d * g, tau_a + d * dt, tpf)
            worst = max(worst, abs(H0 + G1 * d + G2 * d * d + G3 * d ** 3 - ref))
            worst_g3 = max(worst_g3, abs(G3) * d ** 3)
    # the cubic is exact up to float64 rounding of ~1e4 rad arguments; the
    # cubic term the kernel drops stays far below the FP32 sine/cosine error
    assert worst < 1e-9, worst
    assert worst_g3 < 1e-8, worst_g3


def test_fixed_point_turns_give_the_phase_mod_2pi():
    rng = np.random.default_rng(8)
    TS = 41448
    for _ in range(200):
        H0 = rng.uniform(-3e4, 3e4)
        G1 = rng.uniform(-4.0, 4.0)
        G2 = rng.uniform(-2e-4, 2e-4)
        ks = int(rng.integers(0, TS))
        na = int(rng.integers(0, TS - 8))
        base = np.uint32((-int(_frac_fx(H0 / (2 * np.pi)))) & 0xFFFFFFFF)
        slope = np.uint32((-int(_frac_fx(G1 / (2 * np.pi)))) & 0xFFFFFFFF)
        curv = -G2 * TWO32 / (2 * np.pi)
        hi, rem = divmod((ks % TS) << 32, TS)
        ks64 = (hi << 32) | ((rem << 32) // TS)
        for d in range(8):
            n = na + d
            pm = ((n * ks64) & 0xFFFFFFFFFFFFFFFF) >> 32
            ph = (int(base) + int(slope) * d + int(np.round(curv * d * d)) - pm) & 0xFFFFFFFF
            if ph >= 2 ** 31:
                ph -= 2 ** 32
            got = ph * 2 * np.pi / TWO32
            ref = -(H0 + G1 * d + G2 * d * d) - 2 * np.pi * ((n * ks) % TS) / TS
            err = (got - ref + np.pi) % (2 * np.pi) - np.pi
            # fixed-point resolution 2^-32 turn (1.5e-9 rad) per term
            assert abs(err) < 2e-8, (d, err)
