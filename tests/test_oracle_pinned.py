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
