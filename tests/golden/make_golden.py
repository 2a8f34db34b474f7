"""Regenerate the golden fixtures in this directory.

Inputs are small seeded synthetic Level-0 streams from
sentinel1_decode_gb300.synth; outputs come from the REFERENCE's own sources
compiled here (oracle/Makefile -> oracle/_ref/ref_driver, FFTW replaced by the
project shim).  Needs the reference tree, so it runs only in the build
container; the committed .dat / .npz / .json files are what the tests use.

    python tests/golden/make_golden.py [/path/to/reference] [fixture ...]

With fixture names, only those are regenerated and merged into golden.json.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from sentinel1_decode_gb300 import synth  # noqa: E402
import s1_oracle  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
ONLY = sys.argv[2:]
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name -> (stream spec, products to dump, row stride of the stored sample)
FIXTURES = {
    "iw_small": (synth.StreamSpec([synth.BurstSpec(num_lines=400, num_quads=512, swath="IW2", num_targets=6)], seed=11),
                 ["raw", "range_compressed", "range_doppler", "azimuth_compressed"], 20),
    "iw_small_rfi": (synth.StreamSpec([synth.BurstSpec(num_lines=400, num_quads=512, swath="IW2", num_targets=6,
                                                       rfi=True)], seed=12),
                     ["range_compressed", "azimuth_compressed"], 20),
    "iw1_odd": (synth.StreamSpec([synth.BurstSpec(num_lines=397, num_quads=449, swath="IW1", num_targets=4,
                                                  beam_sweep=700)], seed=13),
                ["raw", "range_compressed", "azimuth_compressed"], 20),
    "sm_small": (synth.StreamSpec([synth.BurstSpec(num_lines=1024, num_quads=256, swath="S1", beam_start=512,
                                                   beam_sweep=0, num_targets=5, snr_db=20.0)], seed=14),
                 ["raw", "range_compressed", "range_doppler", "azimuth_compressed_swath"], 32),
    "iw_two_bursts": (synth.StreamSpec([synth.BurstSpec(num_lines=1000, num_quads=96, swath="IW3", num_targets=2),
                                        synth.BurstSpec(num_lines=1003, num_quads=96, swath="IW3", num_targets=2)],
                                       seed=15),
                      ["raw_swath", "range_compressed_swath"], 50),
    # IW bursts of different widths: the swath rows are ragged
    "iw_ragged": (synth.StreamSpec([synth.BurstSpec(num_lines=1000, num_quads=80, swath="IW3", num_targets=2),
                                    synth.BurstSpec(num_lines=1001, num_quads=104, swath="IW3", num_targets=2)],
                                   seed=17),
                  ["raw_swath", "range_compressed_swath"], 50),
    # the fixed-length data formats: bypass A and B, BAQ 3/4/5-bit C
    "baq_a": (synth.StreamSpec([synth.BurstSpec(num_lines=200, num_quads=160, swath="IW2", num_targets=2,
                                                baq_mode=0)], seed=18),
              ["raw", "range_compressed"], 10),
    "baq_b": (synth.StreamSpec([synth.BurstSpec(num_lines=100, num_quads=144, swath="IW2", num_targets=2,
                                                baq_mode=0, test_mode=4)], seed=19),
              ["raw"], 10),
    "baq_c3": (synth.StreamSpec([synth.BurstSpec(num_lines=200, num_quads=300, swath="IW2", num_targets=2,
                                                 baq_mode=3)], seed=20),
               ["raw", "range_compressed"], 10),
    "baq_c4": (synth.StreamSpec([synth.BurstSpec(num_lines=100, num_quads=300, swath="IW2", num_targets=2,
                                                 baq_mode=4)], seed=21, clutter_sigma=40.0),
               ["raw"], 10),
    "baq_c5": (synth.StreamSpec([synth.BurstSpec(num_lines=100, num_quads=300, swath="IW2", num_targets=2,
                                                 baq_mode=5)], seed=22, clutter_sigma=90.0),
               ["raw"], 10),
    # stripmap with a num_quadratures change after 560 lines: two azimuth
    # blocks of different widths in one burst (get_azimuth_blocks)
    "sm_blocks": (synth.StreamSpec([synth.BurstSpec(num_lines=560, num_quads=256, swath="S1", beam_start=512,
                                                    beam_sweep=0, num_targets=4, snr_db=20.0),
                                    synth.BurstSpec(num_lines=520, num_quads=224, swath="S1", beam_start=512,
                                                    beam_sweep=0, num_targets=4, snr_db=20.0, gap_lines=0)],
                                   seed=16),
                  ["raw_swath", "range_compressed_swath", "range_doppler_swath", "azimuth_compressed_swath"], 27),
}
ECCM = {"iw_small_rfi": (13000, 100)}


def run(args):
    r = subprocess.run([DRIVER] + args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("ref_driver failed: %s\n%s" % (args, r.stderr[-2000:]))
    return r.stdout


def main():
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "REF=" + REF, "-j8"],
                          stdout=subprocess.DEVNULL)
    manifest = {}
    if ONLY:
        with open(os.path.join(HERE, "golden.json")) as f:
            manifest = json.load(f)
    tmp = tempfile.mkdtemp()
    for name, (spec, products, stride) in FIXTURES.items():
        if ONLY and name not in ONLY:
            continue
        data = synth.generate(spec)
        dat = os.path.join(HERE, name + ".dat")
        with open(dat, "wb") as f:
            f.write(data)
        swath = spec.bursts[0].swath
        entry = {"swath": swath, "stride": stride, "products": {}}
        store = {}
        for prod in products:
            is_swath = prod.endswith("_swath")
            level = prod[:-6] if is_swath else prod
            out = os.path.join(tmp, name + "_" + prod + ".bin")
            args = ["product", dat, swath, "-1" if is_swath else "0", level, out]
            if name in ECCM:
                args += [str(v) for v in ECCM[name]]
            run(args)
            rows = s1_oracle.read_ref_dump(out)
            widths = [len(r) for r in rows]
            if len(set(widths)) > 1:
                # ragged rows (swaths of different widths): stored
                # zero-filled on the right, with each row's length
                wide = max(widths)
                rows = [np.concatenate([r, np.zeros(wide - len(r), np.complex128)]) for r in rows]
                store[prod + "_widths"] = np.array(widths[::stride])
            arr = np.array(rows)
            entry["products"][prod] = {
                "shape": list(arr.shape),
                "sha256_cf64": hashlib.sha256(arr.astype(np.complex128).tobytes()).hexdigest(),
                "norm": float(np.linalg.norm(arr[np.isfinite(arr)])),
            }
            store[prod] = arr[::stride].astype(np.complex128)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **store)
        # header KATs and state vectors
        hdr = os.path.join(tmp, name + "_hdr.txt")
        run(["headers", dat, hdr])
        lines = open(hdr).read().splitlines()
        def kv(line):
            return dict(tok.split("=", 1) for tok in line.split())
        entry["first_packet"] = kv(lines[0])
        entry["last_packet"] = kv(lines[-1])
        entry["num_packets"] = len(lines)
        svp = os.path.join(tmp, name + "_sv.txt")
        run(["state_vectors", dat, svp])
        entry["state_vectors"] = [[float(x) for x in l.split()] for l in open(svp).read().splitlines()]
        entry["bursts"] = [[int(x) for x in l.split()] for l in run(["bursts", dat, swath]).splitlines()]
        if swath.startswith("IW") and "azimuth_compressed" in products:
            dop = os.path.join(tmp, name + "_dop.txt")
            run(["doppler", dat, swath, "0", dop])
            vals = open(dop).read().split()
            entry["doppler_rate"] = float(vals[1])
            entry["doppler_centroid"] = [float(x) for x in vals[2:]]
        if name in ECCM:
            entry["eccm"] = list(ECCM[name])
        manifest[name] = entry
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(ONLY) if ONLY else len(FIXTURES), "fixtures")


if __name__ == "__main__":
    main()
