"""Regenerate the ancillary fixtures: a small two-swath Level-0 stream with a
varying attitude in its sub-commutated words, its index and annotation
sidecars, and what the REFERENCE's own tools print for them.

Outputs (committed; the tests read only these):
  aux_small.dat, aux_small-index.dat, aux_small-annot.dat
  aux_golden.json:
    "attitude":  the reference's STATE_VECTORS of print_state_vectors
                 (print_main.cpp:17-23) at full precision, one row per
                 vector: time, position[3], velocity[3], quaternions[4],
                 angular_rates[3], attitudes[3]  (oracle/ref_driver attitude)
    "sidecars":  every field of every index / annotation record as the
                 reference decodes them (aux_decoding.cpp:61-145), including
                 the trailing record its read loop adds, and the annotation
                 times (aux_decoding.cpp:121-145)         (ref_driver sidecars)
    "s1_print":  stdout of the reference's s1_print binary (print_main.cpp)
                 for packet_info, complex_samples, swath_names,
                 index_records, annotation_record and state_vectors

Needs the reference tree (oracle/Makefile builds ref_driver and s1_print
from it), so it runs only in the build container.

    python tests/golden/make_aux_golden.py [/path/to/reference]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from sentinel1_decode_gb300 import synth  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
S1_PRINT = os.path.join(ROOT, "oracle", "_ref", "s1_print")

NAME = "aux_small"
# 2 x 200 packets, IW1 then IW2.  Each 64-packet sub-commutation cycle is
# stamped 0.5 s after the previous one: the reference's time-stamp parser
# keeps only the top and the ninth fine-time bits (state_vectors.cpp:5-16),
# so stamps closer than that would collapse into one vector.
SPEC = synth.StreamSpec([synth.BurstSpec(num_lines=200, num_quads=48, swath="IW1", num_targets=2),
                         synth.BurstSpec(num_lines=200, num_quads=40, swath="IW2", num_targets=2, gap_lines=5)],
                        seed=21, sv_cycle_step=0.5, attitude=True)
PACKET_INFO = [0, 1, 63, 64, 200, 399]
COMPLEX_SAMPLES = [0, 250]
ANNOTATION = [0, 1, 199, 399]
INDEX_BLOCK = 4096


def out(*args):
    r = subprocess.run(list(args), capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed:\n%s" % (args, r.stderr[-2000:]))
    return r.stdout


def main():
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "REF=" + REF, "-j8"],
                          stdout=subprocess.DEVNULL)
    data = synth.generate(SPEC)
    dat = os.path.join(HERE, NAME + ".dat")
    idx = os.path.join(HERE, NAME + "-index.dat")
    ann = os.path.join(HERE, NAME + "-annot.dat")
    with open(dat, "wb") as f:
        f.write(data)
    with open(idx, "wb") as f:
        f.write(synth.index_sidecar(data, INDEX_BLOCK))
    with open(ann, "wb") as f:
        f.write(synth.annotation_sidecar(data))
    tmp = tempfile.mkdtemp()
    g = {"num_packets": len(synth.packet_offsets(data)), "index_block_bytes": INDEX_BLOCK}
    p = os.path.join(tmp, "att.txt")
    out(DRIVER, "attitude", dat, p)
    g["attitude"] = [[float(x) for x in l.split()] for l in open(p).read().splitlines()]
    p = os.path.join(tmp, "side.txt")
    out(DRIVER, "sidecars", idx, ann, p)
    side = {"index": [], "annot": [], "time": []}
    for line in open(p).read().splitlines():
        k, *vals = line.split()
        side[k].append(float(vals[0]) if k == "time" else [int(v) for v in vals])
    g["sidecars"] = side
    sp = {}
    for i in PACKET_INFO:
        sp["packet_info %d" % i] = out(S1_PRINT, "packet_info", str(i), dat)
    for i in COMPLEX_SAMPLES:
        sp["complex_samples %d" % i] = out(S1_PRINT, "complex_samples", str(i), dat)
    sp["swath_names"] = out(S1_PRINT, "swath_names", dat)
    sp["index_records"] = out(S1_PRINT, "index_records", idx)
    for i in ANNOTATION:
        sp["annotation_record %d" % i] = out(S1_PRINT, "annotation_record", str(i), ann)
    sp["state_vectors"] = out(S1_PRINT, "state_vectors", dat)
    g["s1_print"] = sp
    with open(os.path.join(HERE, "aux_golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", NAME, len(g["attitude"]), "state vectors,", len(side["index"]), "index records")


if __name__ == "__main__":
    main()
