"""CUDA path (through the C ABI) against the oracle and the reference goldens.

Tolerances: FDBAQ decode bit-exact (FP64 output identical to the reference's
doubles; FP32 output identical to their float cast).  FP64 products to
rounding (rel L2 <= 1e-9 .. 1e-10).  FP32 products rel L2 <= 1e-4 against the
FP64 oracle, the bar of the FP32 mode.
"""
import hashlib

import numpy as np
import pytest

import s1_oracle as O
from conftest import golden_dat, golden_rows, rel_l2
from sentinel1_decode_gb300 import S1Decoder, S1GError, synth

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built(lib_path):
    return lib_path


def dec(name, prec):
    return S1Decoder(golden_dat(name), precision=prec)


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd", "sm_small"])
def test_decode_bit_exact(golden, name):
    g = golden[name]
    raw64 = dec(name, "fp64").get_burst(g["swath"], 0)
    assert list(raw64.shape) == g["products"]["raw"]["shape"]
    assert hashlib.sha256(raw64.tobytes()).hexdigest() == g["products"]["raw"]["sha256_cf64"]
    raw32 = dec(name, "fp32").get_burst(g["swath"], 0, dtype=np.complex64)
    np.testing.assert_array_equal(raw32, raw64.astype(np.complex64))


def test_packet_index_and_headers(golden):
    g = golden["iw_two_bursts"]
    d = dec("iw_two_bursts", "fp32")
    assert d.num_packets() == g["num_packets"]
    assert d.swath_counts() == {"IW3": g["num_packets"]}
    assert d.num_bursts("IW3") == len(g["bursts"])
    ref = g["last_packet"]
    for f in ("pri", "swst", "rank", "num_quadratures", "azimuth_beam_address", "pri_count", "sc_data_word"):
        assert d.packet_field(g["num_packets"] - 1, f) == int(ref[f])
    sv = d.get_state_vectors()
    np.testing.assert_array_equal(sv, np.array(g["state_vectors"]))


@pytest.mark.parametrize("name,prod", [("iw_small", "range_compressed"), ("iw_small", "range_doppler"),
                                       ("iw1_odd", "range_compressed"), ("sm_small", "range_doppler")])
@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32_plain"])
def test_range_products(golden, name, prod, prec):
    g = golden[name]
    out = dec(name, prec).get_range_compressed_burst(g["swath"], 0, prod == "range_doppler")
    assert list(out.shape) == g["products"][prod]["shape"]
    err = rel_l2(out[::g["stride"]], golden_rows(name)[prod])
    assert err < (1e-10 if prec == "fp64" else 1e-5), err


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd"])
def test_doppler_centroid(golden, name):
    g = golden[name]
    rate, dc = dec(name, "fp64").get_doppler(g["swath"], 0)
    assert rate == pytest.approx(g["doppler_rate"], rel=1e-14)
    np.testing.assert_allclose(dc, g["doppler_centroid"], rtol=1e-7, atol=1e-6)


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd", "iw_small_rfi"])
@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32_plain"])
def test_tops_azimuth_burst(golden, name, prec):
    g = golden[name]
    d = dec(name, prec)
    if "eccm" in g:
        d.apply_eccm(*g["eccm"])
    out = d.get_azimuth_compressed_burst(g["swath"], 0)
    assert list(out.shape) == g["products"]["azimuth_compressed"]["shape"]
    err = rel_l2(out[::g["stride"]], golden_rows(name)["azimuth_compressed"])
    assert err < (1e-8 if prec == "fp64" else FP32_TOL), err


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32_plain"])
def test_eccm_range_compressed(golden, prec):
    g = golden["iw_small_rfi"]
    d = dec("iw_small_rfi", prec)
    d.apply_eccm(*g["eccm"])
    out = d.get_range_compressed_burst("IW2", 0)
    err = rel_l2(out[::g["stride"]], golden_rows("iw_small_rfi")["range_compressed"])
    assert err < (1e-9 if prec == "fp64" else FP32_TOL), err


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32_plain"])
def test_stripmap_swath(golden, prec):
    g = golden["sm_small"]
    out = dec("sm_small", prec).get_azimuth_compressed_swath("S1")
    assert list(out.shape) == g["products"]["azimuth_compressed_swath"]["shape"]
    err = rel_l2(out[::g["stride"]], golden_rows("sm_small")["azimuth_compressed_swath"])
    assert err < (1e-10 if prec == "fp64" else FP32_TOL), err


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stripmap_azimuth_blocks(golden, prec):
    """A stripmap burst whose num_quadratures changes after 560 lines: two
    azimuth blocks (get_azimuth_blocks).  Raw rows keep their own widths
    (zero-filled on the right here); range / range-Doppler / azimuth
    products are formed per block, left-padded to the widest block, and the
    azimuth swath has 20 zero rows after every block."""
    g = golden["sm_blocks"]
    ref = golden_rows("sm_blocks")
    s = g["stride"]
    d = dec("sm_blocks", prec)
    if prec == "fp64":
        raw = d.get_swath("S1")
        assert list(raw.shape) == g["products"]["raw_swath"]["shape"]
        assert hashlib.sha256(raw.tobytes()).hexdigest() == g["products"]["raw_swath"]["sha256_cf64"]
        assert not raw[560:, 448:].any()
        np.testing.assert_array_equal(d.swath_row_widths("S1")[::s], ref["raw_swath_widths"])
    tol = 1e-9 if prec == "fp64" else FP32_TOL
    rc = d.get_range_compressed_swath("S1")
    assert list(rc.shape) == g["products"]["range_compressed_swath"]["shape"]
    assert rel_l2(rc[::s], ref["range_compressed_swath"]) < tol
    assert not rc[560:, :64].any() and rc[560:, 64:].any()
    rd = d.get_range_compressed_swath("S1", range_doppler=True)
    assert rel_l2(rd[::s], ref["range_doppler_swath"]) < tol
    az = d.get_azimuth_compressed_swath("S1")
    assert list(az.shape) == g["products"]["azimuth_compressed_swath"]["shape"] == [560 + 20 + 520 + 20, 512]
    err = rel_l2(az[::s], ref["azimuth_compressed_swath"])
    assert err < tol, err
    assert not az[560:580].any() and not az[1100:].any() and not az[580:1100, :64].any()


def test_two_burst_swaths(golden):
    g = golden["iw_two_bursts"]
    d = dec("iw_two_bursts", "fp64")
    raw = d.get_swath("IW3")
    assert list(raw.shape) == g["products"]["raw_swath"]["shape"]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == g["products"]["raw_swath"]["sha256_cf64"]
    rc = d.get_range_compressed_swath("IW3")
    assert rel_l2(rc[::g["stride"]], golden_rows("iw_two_bursts")["range_compressed_swath"]) < 1e-10


def test_ragged_iw_swath(golden):
    """IW bursts of different widths: the reference's swath rows keep their
    burst's width; here the buffer is as wide as the widest burst and the
    narrower rows are zero-filled on the right."""
    g = golden["iw_ragged"]
    ref = golden_rows("iw_ragged")
    d = dec("iw_ragged", "fp64")
    raw = d.get_swath("IW3")
    assert list(raw.shape) == g["products"]["raw_swath"]["shape"] == [2001, 208]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == g["products"]["raw_swath"]["sha256_cf64"]
    rc = d.get_range_compressed_swath("IW3")
    assert rel_l2(rc[::g["stride"]], ref["range_compressed_swath"]) < 1e-10
    assert not rc[:1000, 160:].any() and list(ref["range_compressed_swath_widths"][:2]) == [160, 160]
    from sentinel1_decode_gb300 import RANGE_COMPRESSED, RAW
    for level, key in ((RAW, "raw_swath_widths"), (RANGE_COMPRESSED, "range_compressed_swath_widths")):
        np.testing.assert_array_equal(d.swath_row_widths("IW3", level)[::g["stride"]], ref[key])
    rc32 = dec("iw_ragged", "fp32").get_range_compressed_swath("IW3")
    assert rel_l2(rc32[::g["stride"]], ref["range_compressed_swath"]) < FP32_TOL


def test_request_errors():
    d = dec("iw_small", "fp32")
    with pytest.raises(S1GError) as e:
        d.get_burst("IW3", 0)
    assert e.value.code == -2
    with pytest.raises(S1GError) as e:
        d.get_burst("IW2", 5)
    assert e.value.code == -3


def test_corrupt_brc_reports_status():
    data = bytearray(golden_dat("iw_small"))
    data[68] |= 0xE0        # first BRC of packet 0 -> 7
    raw, status = O.decode_packets(bytes(data), O.get_packets(bytes(data)))
    assert status[0] == 2 and not status[1:].any()     # oracle: "BRC value is invalid."
    d = S1Decoder(bytes(data), precision="fp64")
    with pytest.raises(S1GError) as e:
        d.get_burst("IW2", 0)
    assert e.value.code == -9


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("short", [200, 500])
def test_short_packet_reads_past_end(prec, short):
    """The last packet's declared length is cut by `short` bytes (the stream
    with it), so its codes run past its user data: the oracle reports
    read_n_bits' out_of_range for that packet alone, and the GPU walk (whose
    blocks near the end take the checked path) reports S1G_E_READ_PAST_END."""
    data = bytearray(golden_dat("iw_small"))
    h = O.get_packets(bytes(data))[-1].offset - 68
    pdl = ((data[h + 4] << 8) | data[h + 5]) - short
    data[h + 4], data[h + 5] = pdl >> 8, pdl & 0xFF
    cut = bytes(data[: h + pdl + 7])
    _, status = O.decode_packets(cut, O.get_packets(cut))
    assert status[-1] == 1 and not status[:-1].any()
    d = S1Decoder(cut, precision=prec)
    with pytest.raises(S1GError) as e:
        d.get_burst("IW2", 0)
    assert e.value.code == -8


def test_truncated_stream_matches_oracle():
    data = golden_dat("iw_small")
    cut = data[: len(data) - 400]           # last packet loses its tail
    pk = O.get_packets(cut)
    raw, status = O.decode_packets(cut, pk)
    d = S1Decoder(cut, precision="fp64")
    assert d.num_packets() == len(pk)
    if status.any():
        with pytest.raises(S1GError):
            d.get_burst("IW2", 0)
    else:
        np.testing.assert_array_equal(d.get_burst("IW2", 0), raw)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32_plain"])
def test_medium_burst_vs_oracle(prec):
    """A 600 x 3000 IW burst (S ~ 2760, N_a and S not 7-smooth) against the
    oracle run here."""
    spec = synth.StreamSpec([synth.BurstSpec(num_lines=601, num_quads=1500, swath="IW2", num_targets=10)], seed=21)
    data = synth.generate(spec)
    od = O.S1Decoder(data)
    ref = od.get_azimuth_compressed_burst("IW2", 0)
    out = S1Decoder(data, precision=prec).get_azimuth_compressed_burst("IW2", 0)
    assert out.shape == ref.shape
    err = rel_l2(out, ref)
    assert err < (1e-8 if prec == "fp64" else FP32_TOL), err


def test_full_size_fp32_vs_fp64():
    """C2-size burst (1500 x 12000): decode bit-exact against the oracle's C
    decoder, and the FP32 SLC within 1e-4 of the FP64 GPU SLC."""
    data = synth.generate(synth.config_spec("c2", seed=3))
    od = O.S1Decoder(data)
    raw_ref = od.get_burst("IW2", 0)
    d64 = S1Decoder(data, precision="fp64")
    np.testing.assert_array_equal(d64.get_burst("IW2", 0), raw_ref)
    slc64 = d64.get_azimuth_compressed_burst("IW2", 0)
    slc32 = S1Decoder(data, precision="fp32").get_azimuth_compressed_burst("IW2", 0)
    assert slc32.shape == slc64.shape == (1500, 12000)
    err = rel_l2(slc32, slc64)
    assert err < FP32_TOL, err


@pytest.fixture(scope="module")
def iw_burst_rfi():
    """A full-size IW burst (1500 lines x 12000 samples class) with
    interference lines: many spectral bins sit near the ECCM thresholds."""
    return synth.generate(synth.config_spec("c4", seed=0))


def test_eccm_fp32_takes_fp64_decisions(iw_burst_rfi):
    """The ECCM notch's line detection and bin mitigation are hard thresholds;
    FP32 rounding near them would flip decisions and move the product far
    beyond rounding.  The FP32 pipelines take the notch in FP64, so their
    range-compressed and azimuth-compressed bursts stay within the FP32
    tolerance of the FP64 pipeline's."""
    ref = S1Decoder(iw_burst_rfi, precision="fp64")
    ref.apply_eccm(13000, 100)
    rc64 = ref.get_range_compressed_burst("IW2", 0)
    az64 = ref.get_azimuth_compressed_burst("IW2", 0)
    for prec in ("fp32", "fp32_plain"):
        d = S1Decoder(iw_burst_rfi, precision=prec)
        d.apply_eccm(13000, 100)
        e_rc = rel_l2(d.get_range_compressed_burst("IW2", 0), rc64)
        e_az = rel_l2(d.get_azimuth_compressed_burst("IW2", 0), az64)
        print(prec, "ECCM range compressed %.2e azimuth compressed %.2e" % (e_rc, e_az))
        assert e_rc < 1e-5 and e_az < FP32_TOL, (prec, e_rc, e_az)


def test_eccm_fp32_detection_at_the_threshold(iw_burst_rfi):
    """The FP32 pipelines detect ECCM lines from an FP32 FFT and decide every
    line whose FP32 maximum lies within 1e-4 of the threshold from FP64 DFT
    bins.  The threshold is put on the integer nearest to the FP64 spectral
    maximum of an interference line whose maximum lies closest to an integer
    (a few 1e-4 away: below the FP32 FFT's error there), so that line's
    decision is the FP64 one only if the exact check ran; every range
    compressed line must then match the FP64 pipeline's to FP32 rounding."""
    raw = S1Decoder(iw_burst_rfi, precision="fp64").get_burst("IW2", 0)
    m = np.abs(np.fft.fft(raw, axis=1)).max(axis=1)
    order = np.argsort(np.abs(m - np.round(m)))
    line = None
    for i in order[:200]:
        if m[i] < 2000:
            continue
        mask = O.eccm(raw[i:i + 1].copy(), int(np.floor(m[i])), 100)
        if mask.any():
            line = int(i)
            break
    assert line is not None
    det = int(np.round(m[line]))
    print("line %d: FP64 maximum %.6f, threshold %d, %d lines within 1e-4 of it"
          % (line, m[line], det, int((np.abs(m - det) <= 1e-4 * det).sum())))
    ref = S1Decoder(iw_burst_rfi, precision="fp64")
    ref.apply_eccm(det, 100)
    rc64 = ref.get_range_compressed_burst("IW2", 0)
    off = S1Decoder(iw_burst_rfi, precision="fp64").get_range_compressed_burst("IW2", 0)
    notched = np.linalg.norm(rc64[line] - off[line]) > 1e-3 * np.linalg.norm(off[line])
    assert notched == (m[line] >= det)
    for prec in ("fp32", "fp32_plain"):
        d = S1Decoder(iw_burst_rfi, precision=prec)
        d.apply_eccm(det, 100)
        rc = d.get_range_compressed_burst("IW2", 0)
        assert rc.shape == rc64.shape and np.isfinite(rc).all()
        per_line = np.linalg.norm(rc - rc64, axis=1) / np.linalg.norm(rc64, axis=1)
        print(prec, "worst line rel L2 %.2e (line %d)" % (per_line.max(), int(per_line.argmax())))
        assert per_line.max() < 1e-4, (prec, int(per_line.argmax()), per_line.max())
