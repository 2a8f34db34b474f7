"""Host-side helpers of bench.py (no GPU): the algorithmic-bytes formulas the
roofline is computed from, the per-unit figures read back from the committed
ncu summaries, the tuner-report summary and the point-target error metric."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_tops_algorithmic_bytes(bench):
    n_a, n_r, S, n_out, c_in = 1500, 12000, 6908, 1500, 15_000_000
    b = bench.algorithmic_bytes(n_a, n_r, S, n_out, c_in)
    assert b["total"] == c_in + 8 * n_r * (2 * n_a + 4 * S + n_out)
    assert b["time_unfold"] == 8 * n_r * (S + n_out)
    # per stage each pass reads and writes what it touches; the total is the
    # pipeline's minimum (intermediates written once, read once)
    stages = sum(v for k, v in b.items() if k != "total")
    assert stages == c_in + 8 * n_r * (5 * n_a + 6 * S + n_out)
    assert stages >= b["total"]


def test_stripmap_algorithmic_bytes(bench):
    b = bench.algorithmic_bytes_sm(1024, 2048, 1_000_000)
    assert b["total"] == 1_000_000 + 7 * 8 * 1024 * 2048
    stages = sum(v for k, v in b.items() if k != "total")
    assert stages == 1_000_000 + 9 * 8 * 1024 * 2048
    assert stages >= b["total"]


def test_profiled_values_come_from_the_committed_summary(bench):
    tpu = bench.profiled_value("k_tufr_fused", "traffic_per_unit")
    ipu = bench.profiled_value("k_tufr_fused", "warp_inst_per_unit")
    assert tpu is not None and ipu is not None
    # the summary states both figures as DRAM bytes / warp instructions over
    # range bins x unfolded samples of the C2 burst it was captured on
    lines = open(os.path.join(ROOT, "profiles", "k_tufr_fused_c2_burst.md")).read().splitlines()
    stated = {l.split(":")[0]: float(l.split(":")[1]) for l in lines if l.startswith(("traffic_per_unit:",
                                                                                      "warp_inst_per_unit:"))}
    assert stated == {"traffic_per_unit": tpu, "warp_inst_per_unit": ipu}
    assert 10.0 < tpu < 1000.0 and 10.0 < ipu < 1000.0
    assert bench.profiled_value("no_such_kernel") is None


def test_tuning_summary(bench):
    rep = "on radices 8192:16.16.16.2 9216:4.16.16.9 1024:16.16.4 lengths 8125>8192 7000>7056"
    s = bench.tuning_summary(rep)
    assert s == {"on": True, "radix_orders": 3, "orders_leading_16": 2, "lengths": 2, "lengths_padded_to_pow2": 1}
    assert bench.tuning_summary("off radices lengths")["on"] is False


def test_point_target_errors(bench):
    rng = np.random.default_rng(3)
    ref = (rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))) * 0.01
    for r, c in ((10, 10), (40, 50), (20, 45)):
        ref[r, c] = 100.0 * np.exp(0.3j)
    test = ref.copy()
    test[40, 50] *= 1.01 * np.exp(0.002j)
    e = bench.point_target_errors(ref, test, k=3)
    assert e["peaks"] == 3
    assert e["peak_phase_err_rad"] == pytest.approx(0.002, rel=1e-6)
    assert e["peak_mag_rel_err"] == pytest.approx(0.01, rel=1e-6)
    assert bench.rel_l2(test, ref) > 0
