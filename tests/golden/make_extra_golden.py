"""Regenerate tests/golden/extras.npz: reference outputs of the functions
around the product path that the product goldens do not cover.

Every array comes from the REFERENCE's own sources compiled here
(oracle/Makefile -> oracle/_ref/ref_driver, FFTW replaced by the project
shim), run single-threaded (norm_2d's maximum is an OpenMP loop without a
reduction, signal_processing.cpp:376-383, and races with more threads):

* eccm_raw_*      the decoded iw_small_rfi burst after eccm() (fft 128,
                  stride 64, thresholds of the fixture; signal_processing.cpp:
                  914-1004), every 4th row;
* scale_*         scale(CF_VEC_2D, mode) (signal_processing.cpp:1031-1071)
                  of iw_small's raw and azimuth-compressed bursts, every 20th
                  row;
* spec_*          spectrogram() (signal_processing.cpp:794-844) of decoded
                  iw_small lines, fft 64 / stride 32 as s1_write uses it,
                  and fft 128 / stride 48;
* sinc_*          sinc_interpolate() (signal_processing.cpp:238-257) of a
                  seeded random line at seeded fractional positions (inside,
                  at integers, and past both ends) for L = 4 and L = 8.

    python tests/golden/make_extra_golden.py [/path/to/reference]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import s1_oracle  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
ECCM_STRIDE = 4
SCALE_STRIDE = 20
SPEC_LINES = (0, 17, 399)
SINC_N = 300


def run(args):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([DRIVER] + [str(a) for a in args], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("ref_driver failed: %s\n%s" % (args, r.stderr[-2000:]))


def read_f32(path):
    with open(path, "rb") as f:
        assert f.read(4) == b"S1GF"
        rows, cols = np.frombuffer(f.read(16), dtype=np.int64)
        return np.frombuffer(f.read(), dtype=np.float32).reshape(int(rows), int(cols))


def sinc_positions(n, rng):
    inside = rng.uniform(0.0, n - 1.0, 400)
    ints = np.arange(0, n, 37, dtype=np.float64)
    edges = np.concatenate([rng.uniform(-6.0, 0.0, 20), rng.uniform(n - 1.0, n + 6.0, 20)])
    return np.concatenate([inside, ints, edges])


def main():
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "REF=" + REF, "-j8"],
                          stdout=subprocess.DEVNULL)
    tmp = tempfile.mkdtemp()
    out = {}
    dat = os.path.join(HERE, "iw_small_rfi.dat")
    b = os.path.join(tmp, "eccm.bin")
    run(["eccm_raw", dat, "IW2", 0, 13000, 100, b])
    out["eccm_raw_iw_small_rfi"] = np.array(s1_oracle.read_ref_dump(b))[::ECCM_STRIDE]
    dat = os.path.join(HERE, "iw_small.dat")
    for level in ("raw", "azimuth_compressed"):
        for mode in ("real", "imag", "mag", "norm", "norm_log"):
            f = os.path.join(tmp, "scale.bin")
            run(["scale", dat, "IW2", 0, level, mode, f])
            out["scale_%s_%s" % (level, mode)] = read_f32(f)[::SCALE_STRIDE].copy()
    for fft, stride in ((64, 32), (128, 48)):
        for line in SPEC_LINES:
            f = os.path.join(tmp, "spec.bin")
            run(["spectrogram", dat, "IW2", 0, line, fft, stride, f])
            out["spec_%d_%d_%d" % (fft, stride, line)] = np.array(s1_oracle.read_ref_dump(f))
    rng = np.random.default_rng(77)
    sig = rng.standard_normal(SINC_N) + 1j * rng.standard_normal(SINC_N)
    t = sinc_positions(SINC_N, rng)
    out["sinc_signal"] = sig
    out["sinc_t"] = t
    for L in (4, 8):
        f = os.path.join(tmp, "sinc_in.bin")
        with open(f, "wb") as fh:
            fh.write(np.int64(SINC_N).tobytes())
            fh.write(sig.astype(np.complex128).tobytes())
            fh.write(np.int64(t.size).tobytes())
            fh.write(t.astype(np.float64).tobytes())
        o = os.path.join(tmp, "sinc_out.bin")
        run(["sinc", f, L, o])
        out["sinc_L%d" % L] = s1_oracle.read_ref_dump(o)[0].copy()
    out["strides"] = np.array([ECCM_STRIDE, SCALE_STRIDE])
    np.savez_compressed(os.path.join(HERE, "extras.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
