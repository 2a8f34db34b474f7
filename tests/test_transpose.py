"""Corner turns on the GPU (s1g_transpose): the TMA-staged tile transpose
(complex<float> with an even row pitch) and the shared-memory tile transpose
(odd pitch, complex<double>) against numpy, bit for bit, on burst shapes and
on shapes with partial edge tiles; no bounded tile wait runs out."""
import ctypes

import numpy as np
import pytest

from sentinel1_decode_gb300 import load_library

pytestmark = pytest.mark.gpu


def _cudart():
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(n)
        except OSError:
            pass
    raise RuntimeError("libcudart not found")


def gpu_transpose(a, in_pitch, out_pitch):
    rt = _cudart()
    lib = load_library()
    rows, cols = a.shape
    src = np.zeros((rows, in_pitch), dtype=a.dtype)
    src[:, :cols] = a
    dst = np.full((cols, out_pitch), np.nan, dtype=a.dtype)
    pi, po = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(pi), ctypes.c_size_t(src.nbytes)) == 0
    assert rt.cudaMalloc(ctypes.byref(po), ctypes.c_size_t(dst.nbytes)) == 0
    try:
        assert rt.cudaMemcpy(pi, src.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(src.nbytes), 1) == 0
        assert rt.cudaMemcpy(po, dst.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(dst.nbytes), 1) == 0
        et = 0 if a.dtype == np.complex64 else 1
        assert lib.s1g_transpose(pi, rows, cols, in_pitch, po, out_pitch, et, None) == 0
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemcpy(dst.ctypes.data_as(ctypes.c_void_p), po, ctypes.c_size_t(dst.nbytes), 2) == 0
    finally:
        rt.cudaFree(pi)
        rt.cudaFree(po)
    flag = ctypes.c_int(-1)
    assert lib.s1g_take_device_timeout(ctypes.byref(flag)) == 0
    assert flag.value == 0
    return dst


@pytest.mark.parametrize("rows,cols,in_pitch,out_pitch,dtype", [
    (1500, 12000, 12000, 1500, np.complex64),      # range -> azimuth turn of a burst (TMA)
    (12406, 1542, 1542, 12406, np.complex64),      # the way back, uneven burst (TMA)
    (1457, 11838, 11838, 1457, np.complex64),
    (129, 17, 18, 131, np.complex64),              # partial tiles on both edges, padded pitches (TMA)
    (1, 5, 6, 1, np.complex64),
    (300, 101, 101, 300, np.complex64),            # odd pitch: shared-memory tile path
    (77, 130, 130, 77, np.complex128),             # complex<double>: shared-memory tile path
])
def test_transpose_bit_exact(lib_path, rows, cols, in_pitch, out_pitch, dtype):
    rng = np.random.default_rng(rows * 7 + cols)
    a = (rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols))).astype(dtype)
    out = gpu_transpose(a, in_pitch, out_pitch)
    np.testing.assert_array_equal(out[:, :rows], a.T)
    # columns beyond the matrix in the output pitch are left untouched
    if out_pitch > rows:
        assert np.isnan(out[:, rows:]).all()


def test_transpose_rejects_bad_arguments(lib_path):
    lib = load_library()
    p = ctypes.c_void_p(16)
    q = ctypes.c_void_p(32)
    assert lib.s1g_transpose(p, 4, 8, 7, q, 4, 0, None) == -1      # pitch shorter than a row
    assert lib.s1g_transpose(p, 4, 8, 8, p, 4, 0, None) == -1      # in place
    assert lib.s1g_transpose(p, 4, 8, 8, q, 4, 7, None) == -1      # element type
