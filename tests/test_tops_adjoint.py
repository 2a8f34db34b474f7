"""The differentiable TOPS azimuth chain (s1g_tops_adjoint / s1g_tops_focus):
its hand-written adjoint against central finite differences of the FP64
forward, against the FP64 numpy restatement of the chain and its gradient
(oracle/azimuth_adjoint.py tops_forward / tops_gradient, whose frequency
unfolding is the oracle's restatement of azimuth_frequency_ufr), FP32
against FP64, and the entropy autofocus over the phase-error polynomial and
the centroid offset on the autofocus scene (phase error
exp(i (1.3 pi x^2 + 0.7 pi x^3)) and a +30 Hz centroid offset).  The
reference has no gradients; there is no reference output to compare."""
import dataclasses
import math

import numpy as np
import pytest

import azimuth_adjoint as AA
from conftest import golden_dat

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_path):
    return lib_path


def test_tops_adjoint_matches_finite_differences():
    from sentinel1_decode_gb300 import S1Decoder
    d = S1Decoder(golden_dat("iw_small"), precision="fp64")
    theta = np.array([0.9, -0.4, 0.2])
    off = 3.0
    L, g, go = d.tops_adjoint("IW2", 0, theta, off)
    for j in range(theta.size):
        e = np.zeros_like(theta)
        e[j] = 1e-4
        fd = (d.tops_adjoint("IW2", 0, theta + e, off, grads=False)[0] -
              d.tops_adjoint("IW2", 0, theta - e, off, grads=False)[0]) / 2e-4
        assert abs(fd - g[j]) <= 1e-5 * max(abs(g[j]), 1e-4), (j, fd, g[j])
    # the loss curves fast along the centroid (a 1e-3 Hz step already leaves
    # a 3e-4 truncation error in the central difference): 1e-4 Hz steps
    fd = (d.tops_adjoint("IW2", 0, theta, off + 1e-4, grads=False)[0] -
          d.tops_adjoint("IW2", 0, theta, off - 1e-4, grads=False)[0]) / 2e-4
    assert abs(fd - go) <= 2e-4 * max(abs(go), 1e-7), (fd, go)


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd"])
def test_tops_adjoint_matches_numpy_reference(name):
    from sentinel1_decode_gb300 import S1Decoder
    data = golden_dat(name)
    swath = "IW2" if name == "iw_small" else "IW1"
    X, geo = AA.tops_setup(data, swath)
    theta = np.array([0.7, 0.3])
    off = -4.5
    L0, g0, go0 = AA.tops_gradient(X, theta, off, geo)
    d = S1Decoder(data, precision="fp64")
    L, g, go = d.tops_adjoint(swath, 0, theta, off)
    assert abs(L - L0) <= 1e-10 * abs(L0), (L, L0)
    np.testing.assert_allclose(g, g0, rtol=1e-6, atol=1e-9 * np.abs(g0).max())
    assert abs(go - go0) <= 1e-6 * abs(go0) + 1e-15, (go, go0)
    img = d.tops_focus(swath, 0, theta, off, dtype=np.complex128)
    _, c = AA.tops_forward(X, theta, off, geo)
    assert img.shape == c["Y"].shape
    # the azimuth filter's phase moves ~3 rad per Hz of centroid, so the two
    # centroid estimates' ~1e-5 Hz difference (FP64 sums in another order)
    # turns the image by ~3e-5 rad and moves magnitudes by ~2e-8 of the peak
    scale = np.abs(c["Y"]).max()
    np.testing.assert_allclose(np.abs(img), np.abs(c["Y"]), rtol=0, atol=1e-7 * scale)
    np.testing.assert_allclose(img, c["Y"], rtol=0, atol=1e-4 * scale)


def test_tops_adjoint_fp32_against_fp64():
    from sentinel1_decode_gb300 import S1Decoder
    data = golden_dat("iw_small")
    theta = np.array([2.0, 1.0])
    L64, g64, f64 = S1Decoder(data, precision="fp64").tops_adjoint("IW2", 0, theta, 5.0)
    L32, g32, f32 = S1Decoder(data, precision="fp32").tops_adjoint("IW2", 0, theta, 5.0)
    print("tops fp32 vs fp64: loss %.3e, grad %.3e, offset grad %.3e" % (
        abs(L32 - L64) / abs(L64), np.abs(g32 - g64).max() / np.abs(g64).max(), abs(f32 - f64) / abs(f64)))
    assert abs(L32 - L64) <= 1e-5 * abs(L64)
    assert np.abs(g32 - g64).max() <= 2e-3 * np.abs(g64).max()
    assert abs(f32 - f64) <= 2e-2 * abs(f64)


def test_tops_autofocus_on_the_autofocus_scene():
    """The autofocus scene at a quarter of its size (1100 lines x 3000
    samples), with and without the injected phase error.  Entropy gradient
    descent over the polynomial and the centroid offset (FP32 forward and
    adjoint) lowers the entropy, and the polynomial found with the error,
    minus the one found without it (the chain's own model mismatch), leaves
    less phase error at both aperture edges than no correction."""
    import torch  # noqa: F401
    from sentinel1_decode_gb300 import S1Decoder, synth
    from sentinel1_decode_gb300.autofocus import autofocus
    found = []
    for pe in (False, True):
        sp = synth.config_spec("c5", seed=0, scale=0.25)
        sp.bursts[0] = dataclasses.replace(sp.bursts[0], phase_error=pe)
        d = S1Decoder(synth.generate(sp), precision="fp32")
        r = autofocus(d, "IW2", 0, terms=2, fit_centroid=True, iterations=40, chain="tops")
        print("tops autofocus:", r)
        assert r["entropy_end"] < r["entropy_start"]
        found.append(r["theta"])
    truth = np.array([1.3 * math.pi, 0.7 * math.pi])
    est = found[1] - found[0]
    for x in (-1.0, 1.0):
        resid = abs((est[0] - truth[0]) * x * x + (est[1] - truth[1]) * x ** 3)
        print("aperture edge x=%+.0f: injected %.3f rad, residual %.3f rad" % (
            x, abs(truth[0] * x * x + truth[1] * x ** 3), resid))
        assert resid < abs(truth[0] * x * x + truth[1] * x ** 3)
