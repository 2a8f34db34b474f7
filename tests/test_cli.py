"""The s1_write-compatible CLI (s1g_write) and the S1_Decoder facade header.

CPU tests: the facade compiles as the reference's callers would include it,
and the CLI's argument handling and error paths (no GPU work).  GPU tests:
the cf32 files match the reference goldens the way save_*_as_cf32 writes
them (image_write_main.cpp:186-324): FP64 product cast to complex<float>.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_rows, rel_l2

INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def cli(lib_path):
    from sentinel1_decode_gb300.build import CLI
    assert os.path.exists(CLI)
    return CLI


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=600)


def test_facade_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "s1_decoder_gb300.hpp"\n'
        "int main(int argc, char** argv) {\n"
        "  if (argc < 2) return 0;\n"
        "  S1_Decoder s1(argv[1]);\n"
        "  s1.apply_eccm(13000, 100);\n"
        "  CF_VEC_2D a = s1.get_azimuth_compressed_burst(\"IW2\", 0);\n"
        "  CF_VEC_2D r = s1.get_range_compressed_swath(\"IW2\", true);\n"
        "  S1G_STATE_VECTORS sv = s1.get_state_vectors();\n"
        "  auto ix = index_decoder(\"x-index.dat\");\n"
        "  auto an = annotation_decoder(\"x-annot.dat\");\n"
        "  std::vector<double> t = annotation_time_decoder(\"x-annot.dat\");\n"
        "  s1g_sidecar_report rep = s1.check_sidecars(\"x-index.dat\", \"\");\n"
        "  return (int)(a.size() + r.size() + sv.times.size() + sv.attitudes.size() + ix.size() + an.size()\n"
        "               + t.size() + rep.packets) & 1;\n"
        "}\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", INCLUDE, str(src)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr


def test_cli_help_and_bad_command(cli):
    r = run(cli)
    assert r.returncode == 1 and "save_burst_as_cf32" in r.stdout
    r = run(cli, "nonsense")
    assert r.returncode == 0 and "is not a valid command" in r.stdout
    r = run(cli, "spectrogram", "IW2", "0", "x.dat", "y.tif")
    assert r.returncode == 1 and "expects" in r.stdout
    r = run(cli, "burst", "IW2", "0", "missing.dat", "y.tif")
    assert r.returncode != 0 and "Unable to open" in r.stderr
    r = run(cli, "burst", "IW2", "missing.dat", "y.tif")
    assert r.returncode == 1 and "expects" in r.stdout


def test_cli_missing_file_and_bad_level(cli, tmp_path):
    r = run(cli, "save_burst_as_cf32", "IW2", "0", "raw", str(tmp_path / "missing.dat"), str(tmp_path / "o.cf32"))
    assert r.returncode != 0 and "Unable to open" in r.stderr
    r = run(cli, "save_burst_as_cf32", "IW2", "0", "bogus", os.path.join(GOLDEN, "iw_small.dat"),
            str(tmp_path / "o.cf32"))
    assert r.returncode != 0 and "Invalid processing_level" in r.stderr


@pytest.mark.gpu
def test_cli_raw_burst_bit_exact(cli, golden, tmp_path):
    g = golden["iw_small"]
    out = tmp_path / "raw.cf32"
    r = run(cli, "save_burst_as_cf32", g["swath"], "0", "RAW", os.path.join(GOLDEN, "iw_small.dat"), str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    rows, cols = g["products"]["raw"]["shape"]
    assert "Num Rows: %d" % rows in r.stdout and "Num Cols: %d" % cols in r.stdout
    data = np.fromfile(out, dtype=np.complex64).reshape(rows, cols)
    from sentinel1_decode_gb300 import S1Decoder
    from conftest import golden_dat
    raw64 = S1Decoder(golden_dat("iw_small"), precision="fp64").get_burst(g["swath"], 0)
    assert hashlib.sha256(raw64.tobytes()).hexdigest() == g["products"]["raw"]["sha256_cf64"]
    np.testing.assert_array_equal(data, raw64.astype(np.complex64))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["--fp32", "--fp64"])
def test_cli_azimuth_burst(cli, golden, tmp_path, prec):
    g = golden["iw1_odd"]
    out = tmp_path / "slc.cf32"
    r = run(cli, "save_burst_as_cf32", g["swath"], "0", "azimuth_compressed", os.path.join(GOLDEN, "iw1_odd.dat"),
            str(out), prec)
    assert r.returncode == 0, r.stdout + r.stderr
    rows, cols = g["products"]["azimuth_compressed"]["shape"]
    data = np.fromfile(out, dtype=np.complex64).reshape(rows, cols)
    err = rel_l2(data[::g["stride"]], golden_rows("iw1_odd")["azimuth_compressed"])
    assert err < (1e-6 if prec == "--fp64" else 1e-4), err


@pytest.mark.gpu
def test_cli_swath_with_eccm(cli, golden, tmp_path):
    g = golden["iw_small_rfi"]
    out = tmp_path / "rc.cf32"
    det, mit = g["eccm"]
    r = run(cli, "save_swath_as_cf32", g["swath"], "range_compressed", os.path.join(GOLDEN, "iw_small_rfi.dat"),
            str(out), "--eccm", str(det), str(mit))
    assert r.returncode == 0, r.stdout + r.stderr
    rows, cols = g["products"]["range_compressed"]["shape"]
    data = np.fromfile(out, dtype=np.complex64).reshape(rows, cols)
    err = rel_l2(data[::g["stride"]], golden_rows("iw_small_rfi")["range_compressed"])
    assert err < 1e-4, err


@pytest.mark.gpu
def test_cli_ragged_swath_first_row_width(cli, golden, tmp_path):
    """save_swath_as_cf32 writes every row as wide as the first row
    (image_write_main.cpp:302-315): an IW swath whose second burst is wider
    is cut to the first burst's width."""
    g = golden["iw_ragged"]
    out = tmp_path / "raw.cf32"
    r = run(cli, "save_swath_as_cf32", "IW3", "raw", os.path.join(GOLDEN, "iw_ragged.dat"), str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Num Rows: 2001" in r.stdout and "Num Cols: 160" in r.stdout
    data = np.fromfile(out, dtype=np.complex64).reshape(2001, 160)
    ref = golden_rows("iw_ragged")["raw_swath"]
    np.testing.assert_array_equal(data[::g["stride"]], ref[:, :160].astype(np.complex64))


@pytest.mark.gpu
def test_cli_bad_swath_exits_like_reference(cli, tmp_path):
    r = run(cli, "save_burst_as_cf32", "IW3", "0", "raw", os.path.join(GOLDEN, "iw_small.dat"),
            str(tmp_path / "o.cf32"))
    assert r.returncode == 1
    assert "The requested swath, IW3, does not exist in the data." in r.stdout
    assert "IW2" in r.stdout
