"""Level-0 ingestion and ancillary data: the index / annotation sidecars,
the state vectors with quaternions, angular rates and attitudes, the
s1_print-compatible s1g_print tool, and the memory-mapped file ingest.

The fixture aux_small (tests/golden/make_aux_golden.py) carries a varying
attitude in its sub-commutated words; aux_golden.json holds what the
reference's own code prints and computes for it (its s1_print binary and
STATE_VECTORS / index_decoder / annotation_decoder, compiled from its
sources).  CPU tests cover the oracle restatement and the host-only sidecar
readers; GPU tests cover everything that needs the GPU packet indexer and
decoder."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

AUX = os.path.join(GOLDEN, "aux_small.dat")
AUX_INDEX = os.path.join(GOLDEN, "aux_small-index.dat")
AUX_ANNOT = os.path.join(GOLDEN, "aux_small-annot.dat")
INDEX_KEYS = ["date_time", "time_delta", "data_size", "unit_offset", "byte_offset", "variable_flag", "spare_data"]
ANNOT_KEYS = ["days_ul", "milliseconds_ul", "microseconds_ul", "days_dl", "milliseconds_dl", "microseconds_dl",
              "packet_length", "num_transfer_frames", "error_flag", "bit_1_type", "bit_2_type", "bit_6_type",
              "spare_field"]


@pytest.fixture(scope="module")
def aux():
    with open(os.path.join(GOLDEN, "aux_golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def s1g_print(lib_path):
    from sentinel1_decode_gb300.build import PRINT_CLI
    assert os.path.exists(PRINT_CLI)
    return PRINT_CLI


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=600)


# ------------------------------------------------------------------ CPU
def test_oracle_state_vectors_with_attitude_pinned(aux):
    import s1_oracle
    with open(AUX, "rb") as f:
        sv = s1_oracle.state_vectors_full(s1_oracle.get_packets(f.read()))
    mine = np.concatenate([sv["times"][:, None], sv["positions"], sv["velocities"], sv["quaternions"],
                           sv["angular_rates"], sv["attitudes"]], axis=1)
    ref = np.array(aux["attitude"])
    assert mine.shape == ref.shape == (5, 17)
    np.testing.assert_array_equal(mine, ref)


def test_generator_attitude_survives_the_reference_parse(aux):
    """The attitude the generator wrote is what the reference recovers, up to
    the float32 words and the frame change of parse_quaternions: the
    quaternions are unit length and the angular rates are the written ones."""
    from sentinel1_decode_gb300 import synth
    ref = np.array(aux["attitude"])
    q = ref[:, 7:11]
    np.testing.assert_allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-6)
    for row, cyc in zip(ref, range(1, 6)):
        _, omega = synth.attitude_at(cyc)
        np.testing.assert_allclose(row[11:14], np.float32(omega), rtol=0, atol=0)


def test_sidecar_readers_match_reference(aux, lib_path):
    from sentinel1_decode_gb300 import annotation_times, read_annotation, read_index
    ix = read_index(AUX_INDEX, reference_tail=True)
    assert [[r[k] for k in INDEX_KEYS] for r in ix] == aux["sidecars"]["index"]
    an = read_annotation(AUX_ANNOT, reference_tail=True)
    assert [[r[k] for k in ANNOT_KEYS] for r in an] == aux["sidecars"]["annot"]
    t = annotation_times(AUX_ANNOT, reference_tail=True)
    np.testing.assert_array_equal(t, np.array(aux["sidecars"]["time"]))
    # without the reference's extra trailing record: exactly the file's records
    assert len(read_index(AUX_INDEX)) == os.path.getsize(AUX_INDEX) // 36 == len(ix) - 1
    assert len(read_annotation(AUX_ANNOT)) == aux["num_packets"] == len(an) - 1
    assert all(v == 0 for v in ix[-1].values()) and all(v == 0 for v in an[-1].values())


def _parse_index_bytes(rec: bytes) -> list:
    b = int.from_bytes(rec.ljust(36, b"\0"), "big")
    out, pos = [], 0
    for width in (64, 64, 32, 32, 64, 8, 24):
        out.append((b >> (288 - pos - width)) & ((1 << width) - 1))
        pos += width
    return out


def test_sidecar_partial_and_empty_files(tmp_path, lib_path):
    from sentinel1_decode_gb300 import read_annotation, read_index, S1GError
    raw = open(AUX_INDEX, "rb").read()
    p = tmp_path / "part-index.dat"
    p.write_bytes(raw[:36 * 2 + 11])
    full = read_index(str(p))
    assert len(full) == 2
    tail = read_index(str(p), reference_tail=True)
    assert len(tail) == 3
    # the partial record is parsed from its 11 bytes, zero-padded
    assert [tail[2][k] for k in INDEX_KEYS] == _parse_index_bytes(raw[72:83])
    e = tmp_path / "empty-annot.dat"
    e.write_bytes(b"")
    assert read_annotation(str(e)) == []
    assert len(read_annotation(str(e), reference_tail=True)) == 1
    with pytest.raises(S1GError):
        read_index(str(tmp_path / "missing.dat"))


def test_generated_sidecars_describe_the_stream():
    from sentinel1_decode_gb300 import synth
    data = open(AUX, "rb").read()
    offs = synth.packet_offsets(data)
    assert len(offs) == 400 and offs[0] == 0
    ix = open(AUX_INDEX, "rb").read()
    recs = [_parse_index_bytes(ix[i:i + 36]) for i in range(0, len(ix), 36)]
    units = [r[3] for r in recs] + [len(offs)]
    ends = offs[1:] + [len(data)]
    for r, nxt in zip(recs, units[1:]):
        assert r[4] == offs[r[3]] and r[2] == ends[nxt - 1] - offs[r[3]]


def test_s1g_print_host_commands_match_reference(aux, s1g_print):
    sp = aux["s1_print"]
    r = run(s1g_print, "index_records", AUX_INDEX)
    assert r.returncode == 0 and r.stdout == sp["index_records"]
    for key in [k for k in sp if k.startswith("annotation_record")]:
        r = run(s1g_print, "annotation_record", key.split()[1], AUX_ANNOT)
        assert r.returncode == 0 and r.stdout == sp[key], key


def test_s1g_print_arguments(s1g_print):
    r = run(s1g_print)
    assert r.returncode == 1 and r.stdout.startswith("Please enter a command:") and "state_vectors [path]" in r.stdout
    r = run(s1g_print, "frobnicate")
    assert r.returncode == 0 and r.stdout == "frobnicate is not a valid command.\n"
    r = run(s1g_print, "packet_info", "1")
    assert r.returncode == 1 and r.stdout == "packet_info is missing the following argument: path\n"
    r = run(s1g_print, "packet_info", "x", AUX)
    assert r.returncode == 1 and r.stdout == "x is not a valid packet_index\n"
    r = run(s1g_print, "state_vectors", "/nonexistent/file.dat")
    assert r.returncode == 1 and "or the file may not exist" in r.stdout
    r = run(s1g_print, "annotation_record", "100000", AUX_ANNOT)
    assert r.returncode == 134 and "Index is greater" in r.stderr
    r = run(s1g_print, "--help")
    assert r.returncode == 0 and "index_records [path]" in r.stdout


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_attitudes_match_reference(aux):
    from sentinel1_decode_gb300 import S1Decoder
    d = S1Decoder(AUX)
    ref = np.array(aux["attitude"])
    sv = d.get_state_vectors()
    np.testing.assert_array_equal(sv, ref[:, :7])
    a = d.get_attitudes()
    # host FP64 in the library (no contraction); 1e-14 covers libm ulps across hosts
    np.testing.assert_allclose(a["quaternions"], ref[:, 7:11], rtol=0, atol=1e-14)
    np.testing.assert_array_equal(a["angular_rates"], ref[:, 11:14])
    np.testing.assert_allclose(a["attitudes"], ref[:, 14:17], rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_s1g_print_gpu_commands_match_reference(aux, s1g_print):
    sp = aux["s1_print"]
    for key in [k for k in sp if k.startswith(("packet_info", "complex_samples"))]:
        cmd, idx = key.split()
        r = run(s1g_print, cmd, idx, AUX)
        assert r.returncode == 0, r.stderr
        assert r.stdout == sp[key], key
    r = run(s1g_print, "swath_names", AUX)
    assert r.returncode == 0 and sorted(r.stdout.splitlines()) == sorted(sp["swath_names"].splitlines())
    r = run(s1g_print, "state_vectors", AUX)
    assert r.returncode == 0
    mine, ref = r.stdout.splitlines(), sp["state_vectors"].splitlines()
    assert len(mine) == len(ref) and mine[:3] == ref[:3] and mine[-1] == ref[-1]
    for a, b in zip(mine[3:-1], ref[3:-1]):
        np.testing.assert_allclose([float(x) for x in a.split()], [float(x) for x in b.split()], rtol=0,
                                   atol=1.01e-4)
    r = run(s1g_print, "packet_info", "400", AUX)
    assert r.returncode == 134 and "Index is greater than the number of packets." in r.stderr


@pytest.mark.gpu
def test_packet_info_and_samples_api(aux):
    from sentinel1_decode_gb300 import S1Decoder
    d = S1Decoder(AUX)
    assert d.packet_info(64) == aux["s1_print"]["packet_info 64"]
    s = d.get_packet_samples(250)
    txt = aux["s1_print"]["complex_samples 250"].split()
    assert len(s) == len(txt) == 2 * d.packet_field(250, "num_quadratures")
    ref = np.array([complex(*map(float, t.strip("()").split(","))) for t in txt])
    np.testing.assert_allclose(s, ref, rtol=1e-5)   # the text has 6 significant digits
    np.testing.assert_array_equal(d.get_packet_samples(250, np.complex64), s.astype(np.complex64))


@pytest.mark.gpu
def test_sidecars_cross_check_gpu_indexer(aux, tmp_path):
    from sentinel1_decode_gb300 import S1Decoder, S1GError, synth
    d = S1Decoder(AUX)
    rep = d.check_sidecars(AUX_INDEX, AUX_ANNOT)
    assert rep["ok"] and rep["packets"] == 400 and rep["index_packets_covered"] == 400
    assert rep["index_records"] == os.path.getsize(AUX_INDEX) // 36 and rep["annotation_records"] == 400
    offs = synth.packet_offsets(open(AUX, "rb").read())
    assert [d.packet_offset(k) for k in range(400)] == offs
    # a wrong byte offset in index record 3
    ix = bytearray(open(AUX_INDEX, "rb").read())
    ix[3 * 36 + 31] ^= 0x10
    bad = tmp_path / "bad-index.dat"
    bad.write_bytes(bytes(ix))
    rep = d.check_sidecars(str(bad), None, raise_on_mismatch=False)
    assert not rep["ok"] and rep["index_mismatches"] == 1 and rep["index_first_mismatch"] == 3
    with pytest.raises(S1GError) as e:
        d.check_sidecars(str(bad), None)
    assert e.value.code == -17 and "record 3" in str(e.value)
    # a wrong packet length for packet 7, and a missing last record
    an = bytearray(open(AUX_ANNOT, "rb").read())
    an[7 * 26 + 17] ^= 0x01
    bad2 = tmp_path / "bad-annot.dat"
    bad2.write_bytes(bytes(an[:-26]))
    rep = d.check_sidecars(None, str(bad2), raise_on_mismatch=False)
    assert not rep["ok"] and rep["annotation_records"] == 399
    assert rep["annotation_mismatches"] == 1 and rep["annotation_first_mismatch"] == 7
    # every golden stream agrees with the sidecars generated for it
    for name in ("iw_small", "iw1_odd", "sm_small", "iw_two_bursts"):
        data = open(os.path.join(GOLDEN, name + ".dat"), "rb").read()
        ip, ap = tmp_path / (name + "-index.dat"), tmp_path / (name + "-annot.dat")
        ip.write_bytes(synth.index_sidecar(data, 32 * 1024))
        ap.write_bytes(synth.annotation_sidecar(data))
        rep = S1Decoder(os.path.join(GOLDEN, name + ".dat")).check_sidecars(str(ip), str(ap))
        assert rep["ok"] and rep["index_packets_covered"] == rep["packets"], name


@pytest.mark.gpu
def test_file_ingest_matches_buffer(tmp_path):
    from sentinel1_decode_gb300 import RAW, S1Decoder
    src = os.path.join(GOLDEN, "iw_small.dat")
    data = open(src, "rb").read()
    a = S1Decoder(src, precision="fp64")
    b = S1Decoder(data, precision="fp64")
    ms, n = a.ingest_stats()
    assert n == len(data) and ms > 0
    assert a.num_packets() == b.num_packets()
    np.testing.assert_array_equal(a.get_burst("IW2", 0), b.get_burst("IW2", 0))
    # a stream larger than one 32 MiB staging chunk: 100 copies of the
    # fixture back to back, every packet found at its place
    big = tmp_path / "big.dat"
    with open(big, "wb") as f:
        for _ in range(100):
            f.write(data)
    c = S1Decoder(str(big))
    ms, n = c.ingest_stats()
    assert n == 100 * len(data) and c.num_packets() == 100 * a.num_packets()
    assert c.packet_offset(c.num_packets() - 1) == 99 * len(data) + a.packet_offset(a.num_packets() - 1)
    empty = tmp_path / "empty.dat"
    empty.write_bytes(b"")
    assert S1Decoder(str(empty)).num_packets() == 0


@pytest.mark.gpu
def test_indexer_follows_the_sequential_chain_through_damage():
    """The GPU indexer reproduces the reference's sequential walk (next =
    cur + 7 + packet_data_length, packet.cpp:850-879) where speculative
    sync-marker anchors disagree with it: a damaged sync marker is walked
    over, and garbage bytes inserted between packets derail the chain the
    same way they derail the reference."""
    import s1_oracle as O
    from sentinel1_decode_gb300 import S1Decoder
    data = bytearray(open(AUX, "rb").read())
    offs = [p.offset - 68 for p in O.get_packets(bytes(data))]
    data[offs[5] + 12] ^= 0xFF                       # sync marker of packet 5
    damaged = bytes(data[:offs[200]]) + b"\x00\x17\x2a" + bytes(data[offs[200]:])
    for stream in (bytes(data), damaged):
        ref = [p.offset - 68 for p in O.get_packets(stream)]
        d = S1Decoder(stream)
        n = d.num_packets()
        got = [d.packet_offset(k) for k in range(n)]
        assert n == len(ref) and got == ref
