"""Batched swath processing (s1g_process_swath_batch): the eager call, the
CUDA-graph capture (second call) and graph replays (later calls) give the
same SLCs as the per-burst product calls, for two streams (VV/VH-like) with
uneven burst shapes."""
import ctypes

import numpy as np
import pytest

from sentinel1_decode_gb300 import (AZIMUTH_COMPRESSED, RANGE_COMPRESSED, S1Decoder, batch_outputs,
                                    process_swath_batch, synth)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def streams(lib_path):
    out = []
    for seed, pol in ((5, "VV"), (6, "VH")):
        spec = synth.StreamSpec([synth.BurstSpec(num_lines=1000 + 17 * seed, num_quads=96 + 8 * seed, swath="IW2",
                                                 num_targets=3),
                                 synth.BurstSpec(num_lines=1010, num_quads=104, swath="IW2", num_targets=3,
                                                 gap_lines=200)], seed=seed, polarisation=pol)
        out.append(synth.generate(spec))
    return out


def fetch(ptr, rows, cols, pitch, ty):
    assert ty == 0
    buf = np.empty((rows, pitch), np.complex64)
    rt = None
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(n)
            break
        except OSError:
            continue
    assert rt is not None
    assert rt.cudaMemcpy(buf.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(ptr),
                         ctypes.c_size_t(buf.nbytes), 2) == 0
    return buf[:, :cols].copy()


@pytest.mark.parametrize("level", [AZIMUTH_COMPRESSED, RANGE_COMPRESSED])
def test_batch_eager_graph_replay_match_per_burst(streams, level):
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    results = []
    for call in range(3):     # eager, capture + launch, replay
        n, ms = process_swath_batch(decs, "IW2", level)
        assert n == sum(d.get_burst("IW2", b).size for d in decs for b in range(d.num_bursts("IW2")))
        assert ms > 0
        results.append([fetch(*o) for o in batch_outputs(decs[0])])
    assert len(results[0]) == 4
    for k in range(4):
        np.testing.assert_array_equal(results[1][k], results[0][k])
        np.testing.assert_array_equal(results[2][k], results[0][k])
    ref = []
    for d in decs:
        for b in range(d.num_bursts("IW2")):
            if level == AZIMUTH_COMPRESSED:
                ref.append(d.get_azimuth_compressed_burst("IW2", b, dtype=np.complex64))
            else:
                ref.append(d.get_range_compressed_burst("IW2", b, dtype=np.complex64))
    for k in range(4):
        assert results[0][k].shape == ref[k].shape
        np.testing.assert_array_equal(results[0][k], ref[k])
    for d in decs:
        d.close()


def test_batch_graph_off_and_stage_timing(streams):
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    decs[0].set_batch_graph(False)
    process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    a = [fetch(*o) for o in batch_outputs(decs[0])]
    for d in decs:
        d.set_stage_timing(True)
    decs[0].set_batch_graph(True)
    process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)   # stage timing forces the eager path
    st = decs[0].stage_times()
    assert "time_unfold" in st and st["time_unfold"][0] > 0
    b = [fetch(*o) for o in batch_outputs(decs[0])]
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    for d in decs:
        d.close()


def test_reload_keeps_or_rebuilds_plans(streams):
    """s1g_reload_buffer: the same stream again keeps the plans and the
    captured graph (identical SLCs); another stream rebuilds them (SLCs of a
    fresh handle on that stream); a longer stream grows the buffers."""
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    for _ in range(2):   # eager, then capture
        process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    first = [fetch(*o) for o in batch_outputs(decs[0])]
    for d, s in zip(decs, streams):
        d.reload(s)
    process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)   # replay of the kept graph
    again = [fetch(*o) for o in batch_outputs(decs[0])]
    for x, y in zip(first, again):
        np.testing.assert_array_equal(x, y)
    # swap the two streams: plans rebuilt for the new layouts
    decs[0].reload(streams[1])
    decs[1].reload(streams[0])
    for _ in range(3):
        process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    swapped = [fetch(*o) for o in batch_outputs(decs[0])]
    np.testing.assert_array_equal(swapped[0], first[2])
    np.testing.assert_array_equal(swapped[2], first[0])
    # a longer stream (both bursts twice over) and back
    longer = streams[0] + streams[0]
    decs[0].reload(longer)
    assert decs[0].num_packets() == 2 * S1Decoder(streams[0]).num_packets()
    decs[0].reload(streams[0])
    ref = S1Decoder(streams[0], precision="fp32").get_azimuth_compressed_burst("IW2", 1, dtype=np.complex64)
    np.testing.assert_array_equal(decs[0].get_azimuth_compressed_burst("IW2", 1, dtype=np.complex64), ref)
    for d in decs:
        d.close()


def test_batch_host_outputs_overlapped_copies(streams):
    """s1g_batch_host_outputs: every burst lands in its page-locked host
    buffer, in the eager call, the capture and the graph replays."""
    from sentinel1_decode_gb300.decoder import batch_host_outputs
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    ref = [fetch(*o) for o in batch_outputs(decs[0])]
    rt = None
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(n)
            break
        except OSError:
            continue
    sizes = [r * pt * 8 for (_, r, c, pt, ty) in batch_outputs(decs[0])]
    base = ctypes.c_void_p()
    assert rt.cudaHostAlloc(ctypes.byref(base), ctypes.c_size_t(sum(sizes)), 0) == 0
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    batch_host_outputs(decs[0], [base.value + int(o) for o in offs])
    for call in range(3):
        ctypes.memset(base, 0, sum(sizes))
        process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
        for k, (_, r, c, pt, ty) in enumerate(batch_outputs(decs[0])):
            buf = (ctypes.c_char * sizes[k]).from_address(base.value + int(offs[k]))
            got = np.frombuffer(buf, np.complex64).reshape(r, pt)[:, :c]
            np.testing.assert_array_equal(got, ref[k])
    batch_host_outputs(decs[0], [])
    pageable = np.zeros(16)
    with pytest.raises(Exception):
        batch_host_outputs(decs[0], [pageable.ctypes.data])  # not page-locked
    rt.cudaFreeHost(base)
    for d in decs:
        d.close()


def test_per_burst_calls_share_one_swath_decode(streams):
    """Per-burst FP32 calls decode the whole swath once and serve every burst
    from it: results equal the FP64-checked per-burst decode, a burst with a
    damaged packet still reports its error while the other bursts work, and
    the in-place ECCM notch does not touch the cached rows."""
    from sentinel1_decode_gb300 import RAW, S1GError
    import s1_oracle as O
    data = streams[0]
    ref = S1Decoder(data, precision="fp64")
    d = S1Decoder(data, precision="fp32")
    for b in range(2):
        np.testing.assert_array_equal(d.get_burst("IW2", b, dtype=np.complex64),
                                      ref.get_burst("IW2", b).astype(np.complex64))
    # damage the first BRC of the first packet of burst 0
    bad = bytearray(data)
    p0 = O.get_packets(bytes(bad))[0]
    bad[p0.offset] |= 0xE0
    d2 = S1Decoder(bytes(bad), precision="fp32")
    np.testing.assert_array_equal(d2.get_burst("IW2", 1, dtype=np.complex64),
                                  ref.get_burst("IW2", 1).astype(np.complex64))
    with pytest.raises(S1GError) as e:
        d2.get_burst("IW2", 0)
    assert e.value.code == -9
    # ECCM on a cached burst, twice, then the raw rows again
    d.apply_eccm(13000, 100)
    a = d.get_range_compressed_burst("IW2", 1, dtype=np.complex64)
    b = d.get_range_compressed_burst("IW2", 1, dtype=np.complex64)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(d.get_burst("IW2", 1, dtype=np.complex64),
                                  ref.get_burst("IW2", 1).astype(np.complex64))


def test_batch_burst_selection_processes_only_the_share(streams):
    """s1g_set_batch_bursts (the multi-GPU share of one rank): the batch forms
    only the selected (stream, burst) units, each equal to its per-burst
    product, and the samples count only them; -1 restores every burst."""
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    decs[0].set_batch_bursts([1])
    decs[1].set_batch_bursts([])
    n, _ = process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    assert n == decs[0].get_burst("IW2", 1).size
    outs = [fetch(*o) for o in batch_outputs(decs[0])]
    assert len(outs) == 1
    np.testing.assert_array_equal(outs[0], decs[0].get_azimuth_compressed_burst("IW2", 1, dtype=np.complex64))
    for d in decs:
        d.set_batch_bursts(None)
    n, _ = process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
    assert len(batch_outputs(decs[0])) == 4
    for d in decs:
        d.close()


def test_stage_flops_counts_every_stage(streams):
    """s1g_burst_stage_flops: nominal FP32 work of each TOPS stage of a burst
    (the benchmark's compute roofline); the FFT-heavy stages dominate the
    pointwise ones and the time unfolding saw its device tile count."""
    d = S1Decoder(streams[0], precision="fp32")
    f = d.stage_flops("IW2", 0)
    for st in ("range_compress", "doppler", "freq_unfold", "row_pass", "azimuth_ifft", "time_unfold"):
        assert f[st] > 0, st
    assert f["tiles"] >= 1
    n_a, n_r = d.burst_shape("IW2", 0)
    assert f["range_compress"] >= 2 * 5 * n_a * (n_r + 1) * np.log2(n_r)
    d64 = S1Decoder(streams[0], precision="fp64")
    with pytest.raises(Exception):
        d64.stage_flops("IW2", 0)
    d.close()
    d64.close()


def test_batch_with_eccm_matches_per_burst(streams):
    """With the ECCM notch on, the batch reconstructs the FP64 samples the
    notch needs from its own decoded symbols instead of decoding the burst a
    second time; the SLCs equal the per-burst calls' (which decode again),
    bit for bit.  Detection 0 flags every line; mitigation 40 zeroes part of
    the bins (about half on these streams)."""
    decs = [S1Decoder(s, precision="fp32") for s in streams]
    for d in decs:
        d.apply_eccm(0, 40)
    for _ in range(2):      # eager, then graph capture
        process_swath_batch(decs, "IW2", AZIMUTH_COMPRESSED)
        got = [fetch(*o) for o in batch_outputs(decs[0])]
        ref = [d.get_azimuth_compressed_burst("IW2", b, dtype=np.complex64) for d in decs
               for b in range(d.num_bursts("IW2"))]
        assert len(got) == len(ref) == 4
        for g, r in zip(got, ref):
            np.testing.assert_array_equal(g, r)
    masks = decs[0].get_eccm_mask("IW2", 0)
    assert masks.any() and not masks.all()
    for d in decs:
        d.close()
