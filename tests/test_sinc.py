"""Hann-windowed sinc interpolation on the GPU (s1g_sinc_interpolate, the
warp-shuffle kernel) against the reference's own sinc_interpolate() output
(signal_processing.cpp:238-257, tests/golden/extras.npz) and the oracle, and
the sinc RCMC option of the TOPS row pass (S1G_RCMC_SINC) against the
oracle's restatement of it.

Tolerances: FP64 resampling 1e-13 of the line's peak (sin/cos of another
libm), FP32 2e-6; FP32 SLC with sinc RCMC rel L2 <= 1e-4 against the FP64
oracle, the bar of the FP32 mode."""
import ctypes

import numpy as np
import pytest

import s1_oracle as O
from conftest import golden_dat, golden_extras, golden_rows, rel_l2
from sentinel1_decode_gb300 import S1Decoder, S1GError, load_library

pytestmark = pytest.mark.gpu


def _cudart():
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(n)
        except OSError:
            pass
    raise RuntimeError("libcudart not found")


def gpu_sinc(x, t, L, dtype):
    """Lines x [rows, n] resampled at t ([m] shared or [rows, m]) through the
    C ABI, device buffers allocated here."""
    rt = _cudart()
    lib = load_library()
    x = np.ascontiguousarray(np.atleast_2d(x).astype(dtype))
    t = np.ascontiguousarray(np.asarray(t, dtype=np.float64))
    rows, n = x.shape
    m = t.shape[-1]
    t_pitch = m if t.ndim == 2 else 0
    out = np.empty((rows, m), dtype=dtype)
    ptrs = []
    try:
        for arr in (x, t, out):
            p = ctypes.c_void_p()
            assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(arr.nbytes, 16))) == 0
            ptrs.append(p)
        for p, arr in zip(ptrs[:2], (x, t)):
            assert rt.cudaMemcpy(p, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes), 1) == 0
        et = 0 if dtype == np.complex64 else 1
        rc = lib.s1g_sinc_interpolate(ptrs[0], rows, n, n, ptrs[1], m, t_pitch, L, ptrs[2], m, et, None)
        assert rc == 0, rc
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ptrs[2], ctypes.c_size_t(out.nbytes), 2) == 0
    finally:
        for p in ptrs:
            rt.cudaFree(p)
    return out


@pytest.mark.parametrize("L", [4, 8])
def test_sinc_interpolate_matches_reference(lib_path, L):
    ex = golden_extras()
    sig, t, ref = ex["sinc_signal"], ex["sinc_t"], ex["sinc_L%d" % L]
    scale = np.abs(ref).max()
    got64 = gpu_sinc(sig, t, L, np.complex128)[0]
    np.testing.assert_allclose(got64, ref, rtol=0, atol=1e-13 * scale)
    got32 = gpu_sinc(sig, t, L, np.complex64)[0]
    np.testing.assert_allclose(got32, ref, rtol=0, atol=2e-6 * scale)
    # the same positions in ascending order: windows of 64 samples per warp
    # (the warp-shuffle path) where the random positions used direct reads
    order = np.argsort(t)
    np.testing.assert_allclose(gpu_sinc(sig, t[order], L, np.complex128)[0], ref[order], rtol=0,
                               atol=1e-13 * scale)


def test_sinc_shift_rows_against_oracle(lib_path):
    """Many lines with their own smooth shifts (a range-migration pattern,
    up to +-5 samples): every warp takes the shuffle path."""
    rng = np.random.default_rng(5)
    rows, n = 37, 1500
    x = rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))
    j = np.arange(n, dtype=np.float64)
    t = j[None, :] + 5.0 * np.sin(np.linspace(0, 3, rows))[:, None] * (j[None, :] / n) + 0.37
    ref = np.stack([O.sinc_interpolate(x[r], t[r], 4) for r in range(rows)])
    np.testing.assert_allclose(gpu_sinc(x, t, 4, np.complex128), ref, rtol=0, atol=1e-12)
    assert rel_l2(gpu_sinc(x, t, 4, np.complex64).astype(np.complex128), ref) < 1e-6


@pytest.mark.parametrize("name", ["iw_small", "iw1_odd"])
def test_sinc_rcmc_slc_vs_oracle(lib_path, golden, name):
    g = golden[name]
    data = golden_dat(name)
    od = O.S1Decoder(data)
    od.set_rcmc("sinc", 4)
    ref = od.get_azimuth_compressed_burst(g["swath"], 0)
    d = S1Decoder(data, precision="fp32")
    d.set_rcmc("sinc", 4)
    out = d.get_azimuth_compressed_burst(g["swath"], 0)
    assert out.shape == ref.shape
    err = rel_l2(out, ref)
    print(name, "sinc RCMC fp32 rel L2 %.2e" % err)
    assert err < 1e-4, err
    # the default is the reference's phase RCMC
    d.set_rcmc("phase")
    base = d.get_azimuth_compressed_burst(g["swath"], 0)
    assert rel_l2(base[::g["stride"]], golden_rows(name)["azimuth_compressed"]) < 1e-4
    d64 = S1Decoder(data, precision="fp64")
    d64.set_rcmc("sinc", 4)
    with pytest.raises(S1GError) as e:
        d64.get_azimuth_compressed_burst(g["swath"], 0)
    assert e.value.code == -6
