"""The CPU oracle restatement against the reference's own compiled output.

The golden fixtures (tests/golden/, made by make_golden.py from the
reference sources built with oracle/Makefile) pin the oracle: FDBAQ decode
must be bit-exact (SHA-256 of the complex<double> samples), the FP64 products
must agree to rounding.  No GPU involved.
"""
import hashlib
import math

import numpy as np
import pytest

import s1_oracle as O
from conftest import golden_dat, golden_rows, rel_l2

FIXTURES = ["iw_small", "iw_small_rfi", "iw1_odd", "sm_small", "iw_two_bursts"]


@pytest.mark.parametrize("name", FIXTURES)
def test_packet_headers_and_bursts(golden, name):
    g = golden[name]
    d = O.S1Decoder(golden_dat(name))
    assert len(d.packets) == g["num_packets"]
    for key, pk in (("first_packet", d.packets[0]), ("last_packet", d.packets[-1])):
        ref = g[key]
        for field, _ in O.PRIMARY_HEADER + O.SECONDARY_HEADER:
            assert pk.ph.get(field, pk.sh.get(field)) == int(ref[field]), field
        assert pk.get_pri() == pytest.approx(float(ref["pri_us"]), rel=1e-15)
        assert pk.get_tx_ramp_rate() == pytest.approx(float(ref["txprr"]), rel=1e-15)
        assert pk.get_start_frequency() == pytest.approx(float(ref["txpsf"]), rel=1e-15)
        assert pk.get_time() == pytest.approx(float(ref["time"]), rel=1e-15)
        assert pk.get_replica_chirp_length() == int(ref["replica_len"])
    bursts = d.echo[g["swath"]]
    assert [[len(b), 2 * b[0].num_quads] for b in bursts] == g["bursts"]


@pytest.mark.parametrize("name", FIXTURES)
def test_state_vectors(golden, name):
    d = O.S1Decoder(golden_dat(name))
    t, p, v = d.sv
    ref = np.array(golden[name]["state_vectors"])
    assert len(t) == len(ref)
    np.testing.assert_array_equal(t, ref[:, 0])
    np.testing.assert_array_equal(p, ref[:, 1:4])
    np.testing.assert_array_equal(v, ref[:, 4:7])


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd", "sm_small"])
def test_decode_bit_exact(golden, name):
    d = O.S1Decoder(golden_dat(name))
    raw = d.get_burst(golden[name]["swath"], 0)
    ref = golden[name]["products"]["raw"]
    assert list(raw.shape) == ref["shape"]
    assert hashlib.sha256(np.ascontiguousarray(raw).tobytes()).hexdigest() == ref["sha256_cf64"]


@pytest.mark.parametrize("name,prod", [("iw_small", "range_compressed"), ("iw_small", "range_doppler"),
                                       ("iw1_odd", "range_compressed"), ("sm_small", "range_compressed"),
                                       ("sm_small", "range_doppler"), ("iw_small_rfi", "range_compressed")])
def test_range_products(golden, name, prod):
    g = golden[name]
    d = O.S1Decoder(golden_dat(name))
    if "eccm" in g:
        d.apply_eccm(*g["eccm"])
    out = d.get_range_compressed_burst(g["swath"], 0, prod == "range_doppler")
    assert list(out.shape) == g["products"][prod]["shape"]
    assert rel_l2(out[::g["stride"]], golden_rows(name)[prod]) < 1e-11


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd", "iw_small_rfi"])
def test_tops_azimuth(golden, name):
    g = golden[name]
    d = O.S1Decoder(golden_dat(name))
    if "eccm" in g:
        d.apply_eccm(*g["eccm"])
    pk = d.echo[g["swath"]][0]
    # the golden centroid was made from the burst without ECCM
    rc = O.range_compress(d.data, pk, False, None)
    t, p, v = d.sv
    rate = O.doppler_centroid_rate(pk, math.sqrt(sum(x * x for x in v[0])))
    assert rate == pytest.approx(g["doppler_rate"], rel=1e-15)
    dc = O.doppler_centroid_from_sums(O.wrapped_sums(rc, rate), pk[0])
    np.testing.assert_allclose(dc, g["doppler_centroid"], rtol=1e-9, atol=1e-9)
    out = d.get_azimuth_compressed_burst(g["swath"], 0)
    assert list(out.shape) == g["products"]["azimuth_compressed"]["shape"]
    assert rel_l2(out[::g["stride"]], golden_rows(name)["azimuth_compressed"]) < 1e-9


def test_stripmap_azimuth_swath(golden):
    g = golden["sm_small"]
    d = O.S1Decoder(golden_dat("sm_small"))
    out = d.get_azimuth_compressed_swath_sm("S1")
    assert list(out.shape) == g["products"]["azimuth_compressed_swath"]["shape"]
    assert rel_l2(out[::g["stride"]], golden_rows("sm_small")["azimuth_compressed_swath"]) < 1e-11


def test_two_burst_swath_range(golden):
    g = golden["iw_two_bursts"]
    d = O.S1Decoder(golden_dat("iw_two_bursts"))
    parts = [O.range_compress(d.data, pk) for pk in d.echo["IW3"]]
    out = np.concatenate(parts)
    assert list(out.shape) == g["products"]["range_compressed_swath"]["shape"]
    assert rel_l2(out[::g["stride"]], golden_rows("iw_two_bursts")["range_compressed_swath"]) < 1e-11


# ---- functions around the product path, against the reference's own output
# (tests/golden/extras.npz, made by make_extra_golden.py)

def test_eccm_notch_matches_reference(golden):
    """The oracle's ECCM notch of the decoded iw_small_rfi burst equals the
    reference's eccm() output (every 4th row stored) to rounding; the mask the
    oracle reports is the one that produced it."""
    from conftest import golden_extras
    ex = golden_extras()
    det, mit = golden["iw_small_rfi"]["eccm"]
    d = O.S1Decoder(golden_dat("iw_small_rfi"))
    raw = d.get_burst("IW2", 0).copy()
    flags = O.eccm_flags(raw, det)
    mask = O.eccm(raw, det, mit)
    step = int(ex["strides"][0])
    ref = ex["eccm_raw_iw_small_rfi"]
    assert ref.shape == raw[::step].shape
    assert flags.any() and not flags.all()
    assert mask[flags].any() and not mask[~flags].any()
    assert rel_l2(raw[::step], ref) < 1e-13
    # rows the detector passed over are the decoded rows, bit for bit
    orig = d.get_burst("IW2", 0)
    keep = ~flags[::step]
    np.testing.assert_array_equal(ref[keep], orig[::step][keep])


@pytest.mark.parametrize("level", ["raw", "azimuth_compressed"])
@pytest.mark.parametrize("mode", ["real", "imag", "mag", "norm", "norm_log"])
def test_scale_matches_reference(level, mode):
    from conftest import golden_extras
    ex = golden_extras()
    d = O.S1Decoder(golden_dat("iw_small"))
    x = d.get_burst("IW2", 0) if level == "raw" else d.get_azimuth_compressed_burst("IW2", 0)
    step = int(ex["strides"][1])
    got = O.scale(x, mode)[::step]
    ref = ex["scale_%s_%s" % (level, mode)]
    assert got.dtype == np.float32 and got.shape == ref.shape
    if level == "raw" and mode in ("real", "imag", "mag"):
        np.testing.assert_array_equal(got, ref)          # exact inputs, exact arithmetic
    else:
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 if mode == "norm_log" else 0)


@pytest.mark.parametrize("fft,stride", [(64, 32), (128, 48)])
def test_spectrogram_matches_reference(fft, stride):
    from conftest import golden_extras
    ex = golden_extras()
    raw = O.S1Decoder(golden_dat("iw_small")).get_burst("IW2", 0)
    for line in (0, 17, 399):
        ref = ex["spec_%d_%d_%d" % (fft, stride, line)]
        got = O.spectrogram(raw[line], fft, stride)
        assert got.shape == ref.shape
        assert rel_l2(got, ref) < 1e-14


@pytest.mark.parametrize("L", [4, 8])
def test_sinc_interpolate_matches_reference(L):
    from conftest import golden_extras
    ex = golden_extras()
    got = O.sinc_interpolate(ex["sinc_signal"], ex["sinc_t"], L)
    ref = ex["sinc_L%d" % L]
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14 * np.abs(ref).max())
