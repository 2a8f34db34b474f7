"""The differentiable azimuth chain (s1g_azimuth_adjoint): its hand-written
adjoint against central finite differences of the FP64 forward, against the
FP64 numpy restatement of the chain and its gradient
(oracle/azimuth_adjoint.py), FP32 against FP64, and the entropy-minimising
autofocus on a stripmap burst with a known azimuth phase error."""
import math

import numpy as np
import pytest

import azimuth_adjoint as AA
import s1_oracle as O
from conftest import golden_dat

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_path):
    return lib_path


def stripmap_scene(phase_error: bool) -> bytes:
    """1024 stripmap lines x 4096 samples (the 40 us chirp fits the range
    window), 4 point targets at 20 dB over clutter."""
    from sentinel1_decode_gb300 import synth
    spec = synth.StreamSpec([synth.BurstSpec(num_lines=1024, num_quads=2048, swath="S1", beam_start=512,
                                             beam_sweep=0, num_targets=4, snr_db=20.0, phase_error=phase_error)],
                            seed=31)
    return synth.generate(spec)


@pytest.fixture(scope="module")
def sm_phase_error():
    return stripmap_scene(True)


@pytest.fixture(scope="module")
def sm_clean():
    return stripmap_scene(False)


def chain_geometry(data: bytes, swath: str, burst: int):
    """prf, range sampling rate, effective velocity and slant ranges of a
    burst, from the oracle's packet and state-vector restatement."""
    pk = O.get_packets(data)
    bursts = O.get_packets_in_bursts(pk, swath)
    b = bursts[burst]
    p0 = b[0]
    prf = 1.0 / (p0.get_pri() * 1e-6)
    fs = p0.get_range_sample_rate() * 1e6
    n_a, n_r = len(b), 2 * p0.num_quads
    slant = np.asarray(p0.get_slant_ranges(n_r))
    t, pos, vel = O.state_vectors(pk)
    P, V = O.interpolate_state(t, pos, vel, p0.get_time() + 0.5 * n_a / prf)
    vn = float(np.linalg.norm(V))
    lat = P[2] / P[0]
    a, bb = 6378137.0, 6356752.3142
    re = math.sqrt(((a * a * math.cos(lat)) ** 2 + (bb * bb * math.sin(lat)) ** 2) /
                   ((a * math.cos(lat)) ** 2 + (bb * math.sin(lat)) ** 2))
    hh = float(np.linalg.norm(P))
    r_ref = slant[n_r // 2]
    beta = (re * re + hh * hh - r_ref * r_ref) / (2 * re * hh)
    v_eff = math.sqrt(vn * (re * vn * beta / hh))
    return prf, fs, v_eff, slant


def test_adjoint_matches_finite_differences(sm_phase_error):
    from sentinel1_decode_gb300 import S1Decoder
    d = S1Decoder(sm_phase_error, precision="fp64")
    theta = np.array([1.1, -0.6, 0.3])
    fc = 7.0
    L, g, gf = d.azimuth_adjoint("S1", 0, theta, fc)
    for j in range(theta.size):
        e = np.zeros_like(theta)
        e[j] = 1e-4
        fd = (d.azimuth_adjoint("S1", 0, theta + e, fc, grads=False)[0] -
              d.azimuth_adjoint("S1", 0, theta - e, fc, grads=False)[0]) / 2e-4
        assert abs(fd - g[j]) <= 1e-5 * max(abs(g[j]), 1e-3), (j, fd, g[j])
    fd = (d.azimuth_adjoint("S1", 0, theta, fc + 2e-3, grads=False)[0] -
          d.azimuth_adjoint("S1", 0, theta, fc - 2e-3, grads=False)[0]) / 4e-3
    assert abs(fd - gf) <= 1e-4 * max(abs(gf), 1e-6), (fd, gf)


@pytest.mark.parametrize("name,swath", [("sm_small", "S1"), ("iw_small", "IW2")])
def test_adjoint_matches_numpy_reference(name, swath):
    from sentinel1_decode_gb300 import S1Decoder
    data = golden_dat(name)
    d = S1Decoder(data, precision="fp64")
    X = d.get_range_compressed_burst(swath, 0)
    prf, fs, v_eff, slant = chain_geometry(data, swath, 0)
    theta = np.array([0.8, 0.25])
    fc = -12.5
    L0, g0, gf0 = AA.gradient(X, theta, fc, prf, fs, v_eff, slant)
    L, g, gf = d.azimuth_adjoint(swath, 0, theta, fc)
    assert abs(L - L0) <= 1e-12 * abs(L0), (L, L0)
    np.testing.assert_allclose(g, g0, rtol=1e-8, atol=1e-12 * np.abs(g0).max())
    assert abs(gf - gf0) <= 1e-8 * abs(gf0) + 1e-15, (gf, gf0)
    img = d.azimuth_focus(swath, 0, theta, fc, dtype=np.complex128)
    _, c = AA.forward(X, theta, fc, prf, fs, v_eff, slant)
    np.testing.assert_allclose(img, c["Y"], rtol=0, atol=1e-9 * np.abs(c["Y"]).max())


def test_adjoint_fp32_against_fp64(sm_phase_error):
    from sentinel1_decode_gb300 import S1Decoder
    theta = np.array([2.0, 1.0])
    L64, g64, f64 = S1Decoder(sm_phase_error, precision="fp64").azimuth_adjoint("S1", 0, theta, 3.0)
    L32, g32, f32 = S1Decoder(sm_phase_error, precision="fp32").azimuth_adjoint("S1", 0, theta, 3.0)
    print("fp32 vs fp64: loss %.3e, grad %.3e, centroid grad %.3e" % (
        abs(L32 - L64) / abs(L64), np.abs(g32 - g64).max() / np.abs(g64).max(), abs(f32 - f64) / abs(f64)))
    assert abs(L32 - L64) <= 1e-5 * abs(L64)
    assert np.abs(g32 - g64).max() <= 1e-3 * np.abs(g64).max()
    assert abs(f32 - f64) <= 1e-2 * abs(f64)


def test_autofocus_recovers_the_phase_error(sm_phase_error, sm_clean):
    """The scene carries exp(i (1.3 pi x^2 + 0.7 pi x^3)) over the burst's
    lines.  Autofocus from theta = 0 lowers the entropy of both scenes; the
    polynomial found for the scene with the error, minus the one found for
    the same scene without it (which absorbs the chain's own model mismatch),
    is the injected error."""
    import torch  # noqa: F401
    from sentinel1_decode_gb300 import S1Decoder
    from sentinel1_decode_gb300.autofocus import autofocus
    found = []
    for data in (sm_clean, sm_phase_error):
        d = S1Decoder(data, precision="fp32")
        r = autofocus(d, "S1", 0, terms=2, iterations=40)
        print("autofocus:", r)
        assert r["entropy_end"] < r["entropy_start"] - 0.1
        found.append(r["theta"])
    truth = np.array([1.3 * math.pi, 0.7 * math.pi])
    np.testing.assert_allclose(found[1] - found[0], truth, atol=0.05)
