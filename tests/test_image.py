"""Image output of the TIFF commands: the BigTIFF writer (CPU) and the GPU
scaling epilogue against the reference's scale() formulas
(signal_processing.cpp:366-400, 444-459, 1031-1071) applied to the FP64
product, plus the s1g_write TIFF commands end to end."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_dat

TYPES = {3: ("H", 2), 4: ("I", 4), 16: ("Q", 8)}


def read_bigtiff(path):
    """Minimal little-endian BigTIFF reader: (tags, float32 image as stored,
    top row first)."""
    b = open(path, "rb").read()
    assert b[:2] == b"II" and struct.unpack_from("<HHH", b, 2) == (43, 8, 0)
    off = struct.unpack_from("<Q", b, 8)[0]
    n = struct.unpack_from("<Q", b, off)[0]
    tags = {}
    for i in range(n):
        tag, typ, cnt = struct.unpack_from("<HHQ", b, off + 8 + 20 * i)
        fmt, size = TYPES[typ]
        vpos = off + 8 + 20 * i + 12
        if cnt * size > 8:
            vpos = struct.unpack_from("<Q", b, vpos)[0]
        vals = struct.unpack_from("<%d%s" % (cnt, fmt), b, vpos)
        tags[tag] = vals if cnt > 1 else vals[0]
    w, h = tags[256], tags[257]
    offs = tags[273] if isinstance(tags[273], tuple) else (tags[273],)
    cnts = tags[279] if isinstance(tags[279], tuple) else (tags[279],)
    data = b"".join(b[o:o + c] for o, c in zip(offs, cnts))
    img = np.frombuffer(data, dtype="<f4").reshape(h, w)
    return tags, img


def test_write_tiff_roundtrip_bottom_up(tmp_path, lib_path):
    from sentinel1_decode_gb300 import write_tiff
    for rows, cols in ((5, 7), (700, 3000), (1, 1)):
        img = np.random.default_rng(rows).standard_normal((rows, cols)).astype(np.float32)
        p = str(tmp_path / ("t%d.tif" % rows))
        write_tiff(p, img)
        tags, stored = read_bigtiff(p)
        assert tags[258] == 32 and tags[277] == 1 and tags[339] == 3 and tags[262] == 1 and tags[274] == 1
        # _write_tif writes data row rows-1 as image row 0
        np.testing.assert_array_equal(stored, img[::-1])


def ref_scale(x, mode):
    """scale() of the reference on a complex128 product, cast to float32."""
    a = np.abs(x)
    if mode == "real":
        return x.real.astype(np.float32)
    if mode == "imag":
        return x.imag.astype(np.float32)
    if mode == "mag":
        return (a ** 2).astype(np.float32)
    m = a.max()
    v = (a + 1e-12) / m
    return (20 * np.log10(v) if mode == "norm_log" else v).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["real", "imag", "mag", "norm", "norm_log"])
def test_gpu_scaling_matches_reference_formulas(mode):
    from sentinel1_decode_gb300 import AZIMUTH_COMPRESSED, RAW, S1Decoder
    d = S1Decoder(golden_dat("iw_small"), precision="fp64")
    for level, getter in ((RAW, lambda: d.get_burst("IW2", 0)),
                          (AZIMUTH_COMPRESSED, lambda: d.get_azimuth_compressed_burst("IW2", 0))):
        ref = ref_scale(getter(), mode)
        img = d.get_burst_image("IW2", 0, level, mode)
        assert img.shape == ref.shape
        if mode == "norm_log":
            np.testing.assert_allclose(img, ref, rtol=1e-6, atol=1e-4)
        else:
            np.testing.assert_allclose(img, ref, rtol=2e-6, atol=1e-30)


@pytest.mark.gpu
def test_cli_tiff_commands(lib_path, tmp_path, golden):
    from sentinel1_decode_gb300 import AZIMUTH_COMPRESSED, S1Decoder
    from sentinel1_decode_gb300.build import CLI
    src = os.path.join(GOLDEN, "iw_small.dat")
    out = str(tmp_path / "az.tif")
    r = subprocess.run([CLI, "azimuth_compressed_burst", "IW2", "0", src, out, "--norm_log", "--mag"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    _, stored = read_bigtiff(out)
    d = S1Decoder(golden_dat("iw_small"), precision="fp32")
    img = d.get_burst_image("IW2", 0, AZIMUTH_COMPRESSED, "norm_log")   # --norm_log outranks --mag
    np.testing.assert_array_equal(stored[::-1], img)
    out2 = str(tmp_path / "raw.tif")
    r = subprocess.run([CLI, "swath", "IW2", src, out2], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    _, raw = read_bigtiff(out2)
    np.testing.assert_array_equal(raw[::-1], d.get_swath("IW2", dtype=np.complex64).real)
    det, mit = golden["iw_small_rfi"]["eccm"]
    out3 = str(tmp_path / "eccm.tif")
    r = subprocess.run([CLI, "azimuth_compressed_burst_eccm", "IW2", "0", str(det), str(mit),
                        os.path.join(GOLDEN, "iw_small_rfi.dat"), out3, "--imag"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    _, e = read_bigtiff(out3)
    de = S1Decoder(golden_dat("iw_small_rfi"), precision="fp32")
    de.apply_eccm(det, mit)
    np.testing.assert_array_equal(e[::-1], de.get_azimuth_compressed_burst("IW2", 0, dtype=np.complex64).imag)


def ref_spectrogram(line, fft=64, stride=32):
    """spectrogram() of signal_processing.cpp:794-844 restated with numpy."""
    n = line.size
    nwin = int(np.floor((n / fft) * (fft / stride)))
    pi = 3.14159265358979
    hann = 0.5 * (1.0 - np.cos(2.0 * pi * np.arange(fft) / (fft - 1)))
    spec = np.zeros((nwin, fft), np.complex128)
    for i in range(nwin):
        s = i * stride
        e = s + fft
        if e > n:
            e = n - 1
        w = np.zeros(fft, np.complex128)
        w[:e - s] = line[s:e]
        spec[i] = np.fft.fft(w * hann)
    spec = np.roll(spec, fft // 2, axis=1)
    return spec.T


@pytest.mark.gpu
def test_spectrogram_matches_restatement(lib_path, tmp_path):
    from sentinel1_decode_gb300 import S1Decoder
    from sentinel1_decode_gb300.build import CLI
    d = S1Decoder(golden_dat("iw_small"), precision="fp32")
    raw = S1Decoder(golden_dat("iw_small"), precision="fp64").get_burst("IW2", 0)
    for line in (0, 17, raw.shape[0] - 1):
        sp = d.get_spectrogram("IW2", 0, line)
        ref = ref_spectrogram(raw[line])
        assert sp.shape == ref.shape
        np.testing.assert_allclose(sp, ref, rtol=1e-10, atol=1e-9 * np.abs(ref).max())
    img = d.get_spectrogram("IW2", 0, 17, scaling="norm_log")
    np.testing.assert_allclose(img, ref_scale(ref_spectrogram(raw[17]), "norm_log"), rtol=1e-6, atol=1e-4)
    out = str(tmp_path / "sp.tif")
    r = subprocess.run([CLI, "spectrogram", "IW2", "0", "17", os.path.join(GOLDEN, "iw_small.dat"), out, "--norm_log"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    _, stored = read_bigtiff(out)
    np.testing.assert_array_equal(stored[::-1], img)
