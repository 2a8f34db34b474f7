"""The allocation-free decode entry point (s1g_decode_fdbaq_noalloc), called
through the C ABI with caller-owned device buffers, must reproduce what the
regular entry point (s1g_burst_product, S1G_RAW, complex<float>) returns --
bit for bit, since FDBAQ decoding is exact -- on two calls in a row sharing
the library's fixed scratch array.  This file is collected last on purpose,
and also passes when run alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from conftest import golden_dat
from sentinel1_decode_gb300 import S1Decoder, load_library, synth

pytestmark = pytest.mark.gpu


def _cudart():
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(n)
        except OSError:
            pass
    raise RuntimeError("libcudart not found")


def _dev_alloc(rt, nbytes):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(nbytes)) == 0
    return p


def _h2d(rt, dst, arr):
    assert rt.cudaMemcpy(dst, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes), 1) == 0


def _d2h(rt, arr, src):
    assert rt.cudaMemcpy(arr.ctypes.data_as(ctypes.c_void_p), src, ctypes.c_size_t(arr.nbytes), 2) == 0


def _c2_stream():
    """An IW burst of the 1500 x 12000 workload: num_quads 6000 needs 24 KB
    of scratch per packet, so the 16 MiB array holds 696 packets and the
    1500 packets are decoded in three chunks."""
    return synth.generate(synth.config_spec("c2", seed=9))


@pytest.mark.parametrize("name,swath", [("iw_small", "IW2"), ("iw1_odd", "IW1"), ("c2", "IW2")])
def test_noalloc_decode_matches_regular_entry_point(lib_path, name, swath):
    data = _c2_stream() if name == "c2" else golden_dat(name)
    d = S1Decoder(data, precision="fp32")
    ref = d.get_burst(swath, 0, dtype=np.complex64)          # existing entry point
    npk, n_r = ref.shape
    offsets = np.array([d.packet_field(p, "offset") for p in range(npk)], dtype=np.int64)
    d.close()

    lib = load_library()
    rt = _cudart()
    stream_bytes = np.frombuffer(data, dtype=np.uint8).copy()
    d_stream = _dev_alloc(rt, stream_bytes.nbytes)
    d_off = _dev_alloc(rt, offsets.nbytes)
    d_out = _dev_alloc(rt, npk * n_r * 8)
    d_status = _dev_alloc(rt, npk * 4)
    try:
        _h2d(rt, d_stream, stream_bytes)
        _h2d(rt, d_off, offsets)
        for call in range(2):
            # leave garbage in the output so stale results cannot pass
            assert rt.cudaMemset(d_out, 0xA5 + call, ctypes.c_size_t(npk * n_r * 8)) == 0
            rc = lib.s1g_decode_fdbaq_noalloc(d_stream, stream_bytes.nbytes, d_off, npk, n_r // 2, d_out, n_r,
                                              d_status, None)
            assert rc == 0, rc
            assert rt.cudaDeviceSynchronize() == 0
            out = np.empty((npk, n_r), dtype=np.complex64)
            status = np.empty(npk, dtype=np.int32)
            _d2h(rt, out, d_out)
            _d2h(rt, status, d_status)
            assert not status.any()
            np.testing.assert_array_equal(out, ref)
    finally:
        for p in (d_stream, d_off, d_out, d_status):
            rt.cudaFree(p)


def test_noalloc_rejects_bad_sizes(lib_path):
    lib = load_library()
    # rejected on the host before anything is launched: num_quads wider than
    # the 16-bit num_quadratures field, zero quads, a row pitch too short
    dummy = ctypes.c_void_p(1)
    assert lib.s1g_decode_fdbaq_noalloc(dummy, 100, dummy, 1, 65536, dummy, 200_000, dummy, None) == -1
    assert lib.s1g_decode_fdbaq_noalloc(dummy, 100, dummy, 1, 5_000_000, dummy, 10_000_000, dummy, None) == -1
    assert lib.s1g_decode_fdbaq_noalloc(dummy, 100, dummy, 1, 0, dummy, 10, dummy, None) == -1
    assert lib.s1g_decode_fdbaq_noalloc(dummy, 100, dummy, 1, 512, dummy, 1000, dummy, None) == -1


def test_noalloc_offsets_outside_the_stream_give_status(lib_path):
    """Packet offsets come from the caller here; one whose 68-byte header
    would end past the stream (or that is negative) is reported as
    S1G_E_PACKET_LENGTH with a zero row, and the kernel reads nothing there;
    the other packets decode as usual."""
    data = golden_dat("iw_small")
    d = S1Decoder(data, precision="fp32")
    ref = d.get_burst("IW2", 0, dtype=np.complex64)
    npk, n_r = 6, ref.shape[1]
    offsets = np.array([d.packet_field(p, "offset") for p in range(npk)], dtype=np.int64)
    d.close()
    offsets[1] = len(data) - 10          # header would end past the stream
    offsets[3] = -68
    offsets[4] = len(data) + 4096
    lib = load_library()
    rt = _cudart()
    stream_bytes = np.frombuffer(data, dtype=np.uint8).copy()
    d_stream = _dev_alloc(rt, stream_bytes.nbytes)
    d_off = _dev_alloc(rt, offsets.nbytes)
    d_out = _dev_alloc(rt, npk * n_r * 8)
    d_status = _dev_alloc(rt, npk * 4)
    try:
        _h2d(rt, d_stream, stream_bytes)
        _h2d(rt, d_off, offsets)
        assert rt.cudaMemset(d_out, 0x5A, ctypes.c_size_t(npk * n_r * 8)) == 0
        assert lib.s1g_decode_fdbaq_noalloc(d_stream, stream_bytes.nbytes, d_off, npk, n_r // 2, d_out, n_r,
                                            d_status, None) == 0
        assert rt.cudaDeviceSynchronize() == 0
        out = np.empty((npk, n_r), dtype=np.complex64)
        status = np.empty(npk, dtype=np.int32)
        _d2h(rt, out, d_out)
        _d2h(rt, status, d_status)
    finally:
        for p in (d_stream, d_off, d_out, d_status):
            rt.cudaFree(p)
    bad = [1, 3, 4]
    good = [0, 2, 5]
    assert list(status[bad]) == [-7, -7, -7]
    assert not status[good].any()
    assert not out[bad].any()
    np.testing.assert_array_equal(out[good], ref[good])
