"""Parity at the benchmark workloads' full shapes, against the FP64 oracle run
in the test (oracle/s1_oracle.py, pinned to the reference's own output by
tests/test_oracle_pinned.py).

Workloads (sentinel1_decode_gb300.synth.config_spec):
  * stripmap swath 1024 lines x 2048 samples (range-Doppler azimuth chain);
  * IW burst 1500 x 12000;
  * the same IW burst with interference lines and the ECCM notch at
    detection 13000 / mitigation 100 (notch mask and SLC);
  * two IW bursts of uneven shape (1457 x 11838 and 1543 x 12406, range
    lengths that are not 7-smooth) through the graph-captured swath batch.

Tolerances: FP64 GPU products rel L2 <= 1e-9 (stripmap) / 1e-8 (TOPS, whose
chain resamples in azimuth); FP32 products <= 1e-4 against the FP64 oracle,
the bar of the FP32 mode; notch mask: every bin equal, except bins whose
gradient magnitude lies within 1e-9 (relative) of the mitigation threshold,
where FFTs of different rounding may decide either way.  Every product must
be finite everywhere (rel_l2 asserts it).
"""
import ctypes

import numpy as np
import pytest

import s1_oracle as O
from conftest import rel_l2
from sentinel1_decode_gb300 import (AZIMUTH_COMPRESSED, S1Decoder, batch_outputs, process_swath_batch,
                                    synth)

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
DET, MIT = 13000, 100


@pytest.fixture(scope="module", autouse=True)
def _built(lib_path):
    return lib_path


@pytest.fixture(scope="module")
def c2():
    data = synth.generate(synth.config_spec("c2", seed=5))
    ref = O.S1Decoder(data).get_azimuth_compressed_burst("IW2", 0)
    return data, ref


def test_c1_stripmap_swath_vs_oracle():
    data = synth.generate(synth.config_spec("c1", seed=4))
    ref = O.S1Decoder(data).get_azimuth_compressed_swath_sm("S1")
    assert ref.shape == (1024, 2048)
    for prec, tol in (("fp64", 1e-9), ("fp32", FP32_TOL), ("fp32_plain", FP32_TOL)):
        d = S1Decoder(data, precision=prec)
        out = d.get_azimuth_compressed_swath("S1")
        d.close()
        err = rel_l2(out, ref)
        print("C1 stripmap", prec, "rel L2 %.2e" % err)
        assert err < tol, (prec, err)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-8), ("fp32", FP32_TOL)])
def test_c2_burst_slc_vs_oracle(c2, prec, tol):
    data, ref = c2
    d = S1Decoder(data, precision=prec)
    out = d.get_azimuth_compressed_burst("IW2", 0)
    d.close()
    assert out.shape == ref.shape
    err = rel_l2(out, ref)
    print("C2 burst", prec, "rel L2 %.2e" % err)
    assert err < tol, (prec, err)


def test_eccm_mask_fixture_vs_oracle(golden):
    """The GPU notch mask of the ECCM fixture against the oracle's (whose
    notched lines equal the reference's eccm() output, test_oracle_pinned)."""
    from conftest import golden_dat
    data = golden_dat("iw_small_rfi")
    det, mit = golden["iw_small_rfi"]["eccm"]
    raw = O.S1Decoder(data).get_burst("IW2", 0).copy()
    mask, near = O.eccm(raw, det, mit, ties=1e-9)
    for prec in ("fp64", "fp32"):
        d = S1Decoder(data, precision=prec)
        d.apply_eccm(det, mit)
        got = d.get_eccm_mask("IW2", 0)
        d.close()
        assert got.shape == mask.shape
        assert mask.any()
        assert not ((got != mask) & ~near).any(), int(((got != mask) & ~near).sum())


def test_c4_eccm_mask_and_slc_vs_oracle():
    data = synth.generate(synth.config_spec("c4", seed=6))
    od = O.S1Decoder(data)
    raw = od.get_burst("IW2", 0).copy()
    flags = O.eccm_flags(raw, DET)
    mask, near = O.eccm(raw, DET, MIT, ties=1e-9)
    assert 0.1 < flags.mean() < 0.9 and mask.sum() > 1000
    od.apply_eccm(DET, MIT)
    ref = od.get_azimuth_compressed_burst("IW2", 0)
    d = S1Decoder(data, precision="fp32")
    d.apply_eccm(DET, MIT)
    got = d.get_eccm_mask("IW2", 0)
    assert got.shape == mask.shape == (1500, 187, 128)
    bad = (got != mask) & ~near
    print("C4 mask: %d bins zeroed on %d of %d lines, %d ties, %d other differences"
          % (mask.sum(), flags.sum(), flags.size, near.sum(), bad.sum()))
    assert not bad.any()
    slc = d.get_azimuth_compressed_burst("IW2", 0)
    d.close()
    err = rel_l2(slc, ref)
    print("C4 SLC fp32 rel L2 %.2e" % err)
    assert err < FP32_TOL, err


def _fetch(ptr, rows, cols, pitch, ty):
    assert ty == 0
    rt = None
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(n)
            break
        except OSError:
            continue
    assert rt is not None
    buf = np.empty((rows, pitch), np.complex64)
    assert rt.cudaMemcpy(buf.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(ptr), ctypes.c_size_t(buf.nbytes),
                         2) == 0
    return buf[:, :cols].copy()


def test_uneven_full_size_batch_vs_oracle():
    """Two IW bursts with the swath workload's uneven shapes (N_r 11838 and
    12406 are not 7-smooth) through s1g_process_swath_batch: the eager call,
    the graph capture and a graph replay equal the per-burst FP32 products
    bit for bit, and each burst is within the FP32 bar of the oracle."""
    spec = synth.StreamSpec([synth.BurstSpec(num_lines=1457, num_quads=5919, swath="IW2", num_targets=22,
                                             snr_db=15.0, gap_lines=250),
                             synth.BurstSpec(num_lines=1543, num_quads=6203, swath="IW2", num_targets=22,
                                             snr_db=15.0, gap_lines=251)], seed=8)
    data = synth.generate(spec, workers=2)
    d = S1Decoder(data, precision="fp32")
    assert d.num_bursts("IW2") == 2
    outs = []
    for call in range(3):
        process_swath_batch([d], "IW2", AZIMUTH_COMPRESSED)
        outs.append([_fetch(*o) for o in batch_outputs(d)])
    per_burst = [d.get_azimuth_compressed_burst("IW2", b, dtype=np.complex64) for b in range(2)]
    d.close()
    for k in range(2):
        np.testing.assert_array_equal(outs[1][k], outs[0][k])
        np.testing.assert_array_equal(outs[2][k], outs[0][k])
        np.testing.assert_array_equal(outs[0][k], per_burst[k])
    od = O.S1Decoder(data)
    for k in range(2):
        ref = od.get_azimuth_compressed_burst("IW2", k)
        assert outs[0][k].shape == ref.shape
        err = rel_l2(outs[0][k].astype(np.complex128), ref)
        print("batch burst", k, ref.shape, "rel L2 %.2e" % err)
        assert err < FP32_TOL, (k, err)
