"""The FFT autotuner (s1g_tune.cu): it records radix orders and transform
lengths as the fused path first needs them, shares them through its file
with later processes (so a product computed in another process is bit for
bit the same), and can be switched off."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_dat

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, %r)
from sentinel1_decode_gb300 import S1Decoder
from sentinel1_decode_gb300.decoder import tuning_report
d = S1Decoder(%r, precision="fp32")
np.save(sys.argv[1], d.get_azimuth_compressed_burst("IW1", 0, dtype=np.complex64))
print(tuning_report())
"""


def run_child(tmp_path, env_extra, name):
    out = str(tmp_path / (name + ".npy"))
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT % (ROOT, os.path.join(GOLDEN, "iw1_odd.dat")), out],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out), r.stdout.strip()


def test_tuner_choices_shared_across_processes(tmp_path, lib_path):
    from sentinel1_decode_gb300 import S1Decoder
    from sentinel1_decode_gb300.decoder import tuning_report
    tune = str(tmp_path / "tune.txt")
    a, rep_a = run_child(tmp_path, {"S1G_FFT_TUNE_FILE": tune}, "a")
    assert rep_a.startswith("on") and " lengths " in rep_a and os.path.exists(tune)
    lines = open(tune).read().split("\n")
    assert any(l.startswith("R ") for l in lines) and any(l.startswith("L ") for l in lines)
    b, rep_b = run_child(tmp_path, {"S1G_FFT_TUNE_FILE": tune}, "b")
    np.testing.assert_array_equal(a, b)
    c, rep_c = run_child(tmp_path, {"S1G_AUTOTUNE": "0", "S1G_FFT_TUNE_FILE": tune + ".off"}, "c")
    assert rep_c.startswith("off") and not os.path.exists(tune + ".off")
    err = np.linalg.norm(c - a) / np.linalg.norm(a)
    assert err < 1e-5, err
    # this process: the tuner is on and has recorded what the path needed
    S1Decoder(golden_dat("iw_small"), precision="fp32").get_azimuth_compressed_burst("IW2", 0)
    assert tuning_report().startswith("on")
