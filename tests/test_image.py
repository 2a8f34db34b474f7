"""Image output of the TIFF commands: the BigTIFF writer (CPU), the GPU
scaling epilogue and spectrogram against the reference's own scale() and
spectrogram() output (signal_processing.cpp:366-400, 444-459, 794-844,
1031-1071; tests/golden/extras.npz) and the oracle's restatement of them,
plus the s1g_write TIFF commands end to end."""
import os
import struct
import subprocess

import numpy as np
import pytest

import s1_oracle as O
from conftest import GOLDEN, golden_dat, golden_extras

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


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["real", "imag", "mag", "norm", "norm_log"])
def test_gpu_scaling_matches_reference(mode):
    """The GPU scaling epilogue against the reference's own scale() output
    (every 20th row, tests/golden/extras.npz) and against the oracle's
    scale() of the reference's product rows over the whole image."""
    from sentinel1_decode_gb300 import AZIMUTH_COMPRESSED, RAW, S1Decoder
    ex = golden_extras()
    step = int(ex["strides"][1])
    d = S1Decoder(golden_dat("iw_small"), precision="fp64")
    for level, name, getter in ((RAW, "raw", lambda: d.get_burst("IW2", 0)),
                                (AZIMUTH_COMPRESSED, "azimuth_compressed",
                                 lambda: d.get_azimuth_compressed_burst("IW2", 0))):
        img = d.get_burst_image("IW2", 0, level, mode)
        assert np.isfinite(img).all()
        ref = ex["scale_%s_%s" % (name, mode)]
        assert img[::step].shape == ref.shape
        full = O.scale(getter(), mode)
        assert img.shape == full.shape
        for r in (ref, full[::step]) if level == AZIMUTH_COMPRESSED else (ref,):
            if level == RAW and mode in ("real", "imag", "mag"):
                np.testing.assert_array_equal(img[::step], r)
            elif mode == "norm_log":
                np.testing.assert_allclose(img[::step], r, rtol=1e-6, atol=1e-4)
            else:
                np.testing.assert_allclose(img[::step], r, rtol=2e-6, atol=1e-30)
        if mode == "norm_log":
            np.testing.assert_allclose(img, full, rtol=1e-6, atol=1e-4)
        else:
            np.testing.assert_allclose(img, full, rtol=2e-6, atol=1e-30)


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


@pytest.mark.gpu
def test_spectrogram_matches_reference(lib_path, tmp_path):
    """The GPU spectrogram against the reference's spectrogram() output
    (tests/golden/extras.npz) for s1_write's fft 64 / stride 32 and for
    fft 128 / stride 48, and its scaled image against the oracle."""
    from sentinel1_decode_gb300 import S1Decoder
    from sentinel1_decode_gb300.build import CLI
    ex = golden_extras()
    d = S1Decoder(golden_dat("iw_small"), precision="fp32")
    for fft, stride in ((64, 32), (128, 48)):
        for line in (0, 17, 399):
            sp = d.get_spectrogram("IW2", 0, line, fft, stride)
            ref = ex["spec_%d_%d_%d" % (fft, stride, line)]
            assert sp.shape == ref.shape
            assert np.isfinite(sp).all()
            np.testing.assert_allclose(sp, ref, rtol=1e-10, atol=1e-9 * np.abs(ref).max())
    img = d.get_spectrogram("IW2", 0, 17, scaling="norm_log")
    np.testing.assert_allclose(img, O.scale(ex["spec_64_32_17"], "norm_log"), rtol=1e-6, atol=1e-4)
    out = str(tmp_path / "sp.tif")
    r = subprocess.run([CLI, "spectrogram", "IW2", "0", "17", os.path.join(GOLDEN, "iw_small.dat"), out, "--norm_log"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    _, stored = read_bigtiff(out)
    np.testing.assert_array_equal(stored[::-1], img)
