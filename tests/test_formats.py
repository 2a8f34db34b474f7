"""The fixed-length data formats: bypass (A/B, baq_mode 0) and BAQ 3/4/5-bit
(C).  Golden streams baq_a, baq_b, baq_c3, baq_c4, baq_c5 were decoded by the
reference's own code; its A/B/C decoders read zero-filled container entries
instead of the decoded codes (see s1g_set_abc_decode), and the default mode
reproduces that output bit for bit.  The "fields" mode decodes each sample
from its own bits and is checked against the generator's reconstruction."""
import hashlib

import numpy as np
import pytest

import s1_oracle as O
from conftest import golden_dat, golden_rows, rel_l2

FIXED = ["baq_a", "baq_b", "baq_c3", "baq_c4", "baq_c5"]


def oracle_raw(name, fields=False):
    data = golden_dat(name)
    return np.array([O.decode_fixed_packet(data, p, fields) for p in O.get_packets(data)])


# ------------------------------------------------------------------ CPU
@pytest.mark.parametrize("name", FIXED)
def test_oracle_fixed_formats_pinned(golden, name):
    raw = oracle_raw(name)
    g = golden[name]["products"]["raw"]
    assert list(raw.shape) == g["shape"]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == g["sha256_cf64"]


@pytest.mark.parametrize("mode", [0, 3, 4, 5])
def test_oracle_fields_decode_inverts_the_generator(mode):
    from sentinel1_decode_gb300 import synth
    spec = synth.StreamSpec([synth.BurstSpec(num_lines=6, num_quads=333, swath="IW1", num_targets=1,
                                             baq_mode=mode)], seed=40 + mode, clutter_sigma=30.0)
    data, truth = synth.generate(spec, return_truth=True)
    pk = O.get_packets(data)
    for i, p in enumerate(pk):
        np.testing.assert_array_equal(O.decode_fixed_packet(data, p, fields=True), truth[0][i])


def test_reference_quirks_of_the_fixed_formats():
    """What the reference's containers do to the samples: A/B quads below 128
    are zero and quad q carries quad q - 128; C samples of a block are one
    value on both I and Q."""
    a = oracle_raw("baq_a")
    af = oracle_raw("baq_a", fields=True)
    assert not a[:, :256].any()
    np.testing.assert_array_equal(a[:, 256:], af[:, :a.shape[1] - 256])
    c = oracle_raw("baq_c4")
    assert np.array_equal(c.real, c.imag)
    for b0 in range(0, c.shape[1], 256):
        blk = c[:, b0:b0 + 256]
        assert (blk == blk[:, :1]).all()


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", FIXED)
def test_fixed_formats_bit_exact(golden, name, lib_path):
    from sentinel1_decode_gb300 import S1Decoder
    g = golden[name]
    raw64 = S1Decoder(golden_dat(name), precision="fp64").get_burst(g["swath"], 0)
    assert list(raw64.shape) == g["products"]["raw"]["shape"]
    assert hashlib.sha256(raw64.tobytes()).hexdigest() == g["products"]["raw"]["sha256_cf64"]
    raw32 = S1Decoder(golden_dat(name), precision="fp32").get_burst(g["swath"], 0, dtype=np.complex64)
    np.testing.assert_array_equal(raw32, raw64.astype(np.complex64))
    d = S1Decoder(golden_dat(name), precision="fp64")
    d.set_abc_decode("fields")
    np.testing.assert_array_equal(d.get_burst(g["swath"], 0), oracle_raw(name, fields=True))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["baq_a", "baq_c3"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_fixed_formats_range_compressed(golden, name, prec, lib_path):
    from sentinel1_decode_gb300 import S1Decoder
    g = golden[name]
    out = S1Decoder(golden_dat(name), precision=prec).get_range_compressed_burst(g["swath"], 0)
    err = rel_l2(out[::g["stride"]], golden_rows(name)["range_compressed"])
    assert err < (1e-9 if prec == "fp64" else 1e-4), err


@pytest.mark.gpu
def test_fixed_formats_in_the_batch_path(lib_path):
    """A swath batch over a bypass stream and a BAQ stream gives the
    per-burst products, in both decode modes."""
    from sentinel1_decode_gb300 import RANGE_COMPRESSED, S1Decoder, batch_outputs, process_swath_batch
    from test_batch import fetch
    decs = [S1Decoder(golden_dat(n), precision="fp32") for n in ("baq_a", "baq_c3")]
    for mode in ("reference", "fields"):
        for d in decs:
            d.set_abc_decode(mode)
        process_swath_batch(decs, "IW2", RANGE_COMPRESSED)
        outs = [fetch(*o) for o in batch_outputs(decs[0])]
        assert len(outs) == 2
        for d, o in zip(decs, outs):
            np.testing.assert_array_equal(o, d.get_range_compressed_burst("IW2", 0, dtype=np.complex64))


@pytest.mark.gpu
def test_invalid_baq_mode_and_short_packet(lib_path):
    from sentinel1_decode_gb300 import S1Decoder, S1GError
    data = bytearray(golden_dat("baq_c3"))
    data[37] = (data[37] & 0xE0) | 7          # packet 0: baq_mode 7 is not a format
    with pytest.raises(S1GError) as e:
        S1Decoder(bytes(data), precision="fp64").get_burst("IW2", 0)
    assert e.value.code == -13 and "BAQ Mode is invalid." in str(e.value)
    # a bypass packet whose length field leaves out its last bytes
    data = bytearray(golden_dat("baq_b"))
    pdl = (data[4] << 8) | data[5]
    data[4:6] = (pdl - 40).to_bytes(2, "big")
    data = bytes(data[:68 + pdl + 1 - 62 - 40]) + bytes(data[68 + pdl + 1 - 62:])
    p0 = O.get_packets(data)[0]
    with pytest.raises(IndexError):
        O.decode_fixed_packet(data, p0)        # the reference would throw too
    with pytest.raises(S1GError) as e:
        S1Decoder(data, precision="fp64").get_burst("IW2", 0)
    assert e.value.code == -8
