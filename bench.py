#!/usr/bin/env python3
"""Benchmark: IW-swath Msamples/s on one GB300 (batched FP32 path).

Workload (default): the 9-burst dual-polarisation IW swath -- 9 bursts with
seeded uneven line counts (1450-1560) and range lengths (11800-12500 complex
samples), 200 point targets over clutter, VV and VH as two Level-0 streams,
all synthetic (seeded generator, no dataset).  A step processes every burst
of both streams from the device-resident raw byte streams (packet indexing
included) to device-resident SLC bursts.  One sample = one complex input echo
sample.  Inputs are far larger than L2 (~3 GB of intermediate data per burst),
so no explicit flush is needed.

Also reported: the same metric end to end through the C ABI with host
buffers (pinned host -> device copy of both streams, open, process, SLC
device -> host), the plain FP64 GPU path on one burst, the dominant stage's
HBM roofline, and the CPU oracle on a bounded sample of the workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "IW-swath Msamples/s on 1 GB300, batched FP32 vs plain FP64, at <=1e-4 rel L2"


def cudart():
    for n in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(n)
        except OSError:
            pass
    raise RuntimeError("libcudart not found")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        # the raw samples (S1G_CLOCKS_DIR, default the temporary directory); the
        # bench line carries their summary
        d = os.environ.get("S1G_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, "s1g_clocks_rank%d.csv" % device)
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        self.f = open(self.path, "w")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-i", str(device), "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
        self.f.close()
        if self.p and not any(len(l.split(",")) >= 9 for l in open(self.path)):
            # a timed region shorter than the 200 ms period: one sample at its end
            try:
                out = subprocess.run(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                      "-i", str(self.device)], capture_output=True, text=True, timeout=15).stdout
                with open(self.path, "a") as f:
                    f.write(out)
            except (OSError, subprocess.SubprocessError):
                pass
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def point_target_errors(ref: np.ndarray, test: np.ndarray, k: int = 20, win: int = 16):
    """Phase and relative magnitude errors of `test` at the k strongest,
    mutually separated peaks of |ref| (the point targets of the scene)."""
    mag = np.abs(ref)
    m = mag.copy()
    ph, mg = [], []
    for _ in range(k):
        i = int(np.argmax(m))
        r, c = divmod(i, m.shape[1])
        if m[r, c] <= 0:
            break
        ph.append(abs(float(np.angle(test[r, c] * np.conj(ref[r, c])))))
        mg.append(abs(float(abs(test[r, c]) / mag[r, c] - 1.0)))
        m[max(0, r - win):r + win + 1, max(0, c - win):c + win + 1] = 0
    return {"peaks": len(ph), "peak_phase_err_rad": max(ph) if ph else None,
            "peak_mag_rel_err": max(mg) if mg else None}


def tuning_summary(report: str) -> dict:
    """Counts of the FFT autotuner's choices (the full list is in its file)."""
    words = report.split()
    on = bool(words) and words[0] == "on"
    i_r = words.index("radices") if "radices" in words else len(words)
    i_l = words.index("lengths") if "lengths" in words else len(words)
    rad = words[i_r + 1:i_l]
    lens = words[i_l + 1:]
    default16 = sum(1 for w in rad if w.split(":")[1].startswith("16"))
    return {"on": on, "radix_orders": len(rad), "orders_leading_16": default16, "lengths": len(lens),
            "lengths_padded_to_pow2": sum(1 for w in lens if (int(w.split(">")[1]) & (int(w.split(">")[1]) - 1)) == 0)}


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_streams(workload: str, seed: int, workers: int):
    from sentinel1_decode_gb300 import synth
    if workload == "c3":
        specs = []
        for pol, s in (("VV", 0), ("VH", 1)):
            sp = synth.config_spec("c3", seed=seed)
            sp.seed = 1000 * seed + s
            sp.polarisation = pol
            specs.append(sp)
    elif workload in ("c1", "c2", "c4", "c5"):
        specs = [synth.config_spec(workload, seed=seed)]
    else:
        raise ValueError(workload)
    return [synth.generate(sp, workers=workers) for sp in specs]


def algorithmic_bytes(n_a: int, n_r: int, S: int, n_out: int, c_in: int) -> dict:
    """Minimum HBM bytes per burst and stage, FP32 complex (8 B):
    B = C_in + 8 N_r (2 N_a + 4 S + N_out) in total; the time unfolding alone
    reads the azimuth-IFFT output (S per range bin) and writes the SLC
    (N_out per range bin)."""
    b = 8 * n_r
    return {"batch_decode": c_in + b * n_a, "range_compress": 2 * b * n_a, "doppler": b * n_a,
            "freq_unfold": b * (n_a + S), "row_pass": 2 * b * S, "azimuth_ifft": 2 * b * S,
            "time_unfold": b * (S + n_out), "total": c_in + b * (2 * n_a + 4 * S + n_out)}


def burst_geometry(dec, swath: str, tops: bool = True, bursts=None):
    """(n_a, n_r, S, n_out) per burst (only those in `bursts` when given), from
    header fields (host-side); a stripmap burst is not unfolded
    (S = n_out = n_a)."""
    out = []
    for b in range(dec.num_bursts(swath)):
        if bursts is not None and b not in bursts:
            continue
        r, c = ctypes.c_int64(), ctypes.c_int64()
        dec._check(dec._lib.s1g_burst_shape(dec.handle, swath.encode(), b, 0, ctypes.byref(r), ctypes.byref(c)))
        if not tops:
            out.append((r.value, c.value, r.value, r.value))
            continue
        if r.value < 1000:
            continue
        S, n_out = dec.unfold_shape(swath, b)
        out.append((r.value, c.value, S, n_out))
    return out


def rank_bursts(units, world: int, rank: int, n_streams: int):
    """This rank's share of the (stream, burst, cost) units of one swath, as
    the burst indices of each stream: the longest-processing-time plan of
    shard.assign_units, which every rank computes alike without
    communicating."""
    from sentinel1_decode_gb300.shard import assign_units
    plan = assign_units([u[2] for u in units], world)
    out = [[] for _ in range(n_streams)]
    for i in plan[rank]:
        s, b, _ = units[i]
        out[s].append(b)
    return out


def reduce_rate(samples: float, seconds: float):
    """(samples of all ranks, slowest rank's seconds): the whole job's rate is
    their ratio.  Identity without torch.distributed."""
    from sentinel1_decode_gb300.shard import combine
    return combine(samples, seconds)


def fp32_peak_tflops(sms: int, sm_mhz: float) -> float:
    """Nominal FP32 peak: SMs x 128 FP32 lanes x 2 flops (FMA) x SM clock."""
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def algorithmic_bytes_sm(n_a: int, n_r: int, c_in: int) -> dict:
    """Stripmap (range-Doppler) chain, FP32 complex: B = C_in + 56 N_a N_r
    (decode + range compression write once, the azimuth FFT, row pass and
    azimuth IFFT passes each read and write the burst)."""
    b = 8 * n_r * n_a
    return {"batch_decode": c_in + b, "range_compress": 4 * b, "row_pass": 2 * b, "azimuth_ifft": 2 * b,
            "total": c_in + 7 * b}


def profiled_value(kernel: str, key: str = "traffic_per_unit"):
    """A per-unit figure (unit: range bin x unfolded sample) of `kernel` from
    the committed ncu summary (profiles/<kernel>_*.md, line '<key>: X'), or
    None: traffic_per_unit = DRAM bytes, warp_inst_per_unit = executed warp
    instructions."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if fn.startswith(kernel) and fn.endswith(".md"):
            for line in open(os.path.join(d, fn)):
                if line.startswith(key + ":"):
                    return float(line.split(":")[1])
    return None


def c5_autofocus(stream: bytes, device: int) -> dict:
    """Entropy autofocus of the autofocus scene (IW burst 1500 x 12000 with the
    phase error exp(i (1.3 pi x^2 + 0.7 pi x^3)) over its lines and a +30 Hz
    Doppler-centroid offset) through the TOPS chain's hand-written adjoint,
    FP32, L-BFGS over the polynomial (x^2, x^3) and the centroid offset.
    The same scene without the phase error gives the chain's own optimum (its
    model mismatch), which is subtracted; the same scene without the offset
    gives the centroid the estimator reports without it.  Reported: the
    recovered polynomial, its residual phase error at the aperture edges
    (x = -1, +1) against the injected one, and the recovered centroid offset
    (estimated centroid at mid-range plus the fitted offset, minus the
    no-offset scene's) against the injected +30 Hz."""
    import dataclasses
    from sentinel1_decode_gb300 import S1Decoder, synth
    from sentinel1_decode_gb300.autofocus import autofocus
    t0 = time.perf_counter()
    base = synth.config_spec("c5", seed=0)
    clean = synth.StreamSpec([dataclasses.replace(base.bursts[0], phase_error=False)], seed=0)
    no_off = synth.StreamSpec([dataclasses.replace(base.bursts[0], phase_error=False, dc_offset_hz=0.0)], seed=0)
    runs = {}
    for name, data in (("scene", stream), ("without_phase_error", synth.generate(clean)),
                       ("without_offset", synth.generate(no_off))):
        d = S1Decoder(data, device=device, precision="fp32")
        _, dc = d.get_doppler("IW2", 0)
        fit = name != "without_offset"
        r = autofocus(d, "IW2", 0, terms=2, fit_centroid=fit, iterations=40, chain="tops") if fit else \
            {"theta": np.zeros(2), "centroid": 0.0}
        r["centroid_mid_hz"] = float(dc[dc.size // 2]) + float(r["centroid"])
        runs[name] = r
        d.close()
    truth = np.array([1.3 * math.pi, 0.7 * math.pi])
    est = np.asarray(runs["scene"]["theta"]) - np.asarray(runs["without_phase_error"]["theta"])
    edge = {"x=-1": float((est[0] - truth[0]) - (est[1] - truth[1])),
            "x=+1": float((est[0] - truth[0]) + (est[1] - truth[1]))}
    off = runs["scene"]["centroid_mid_hz"] - runs["without_offset"]["centroid_mid_hz"]
    return {"chain": "tops (frequency unfolding, row pass, azimuth IFFT; hand-written adjoint, FP32)",
            "theta_found": [float(x) for x in runs["scene"]["theta"]],
            "theta_found_without_phase_error": [float(x) for x in runs["without_phase_error"]["theta"]],
            "theta_recovered": [float(x) for x in est], "theta_injected": [float(x) for x in truth],
            "residual_phase_error_rad": edge,
            "injected_phase_error_rad": {"x=-1": float(truth[0] - truth[1]), "x=+1": float(truth[0] + truth[1])},
            "entropy": [runs["scene"]["entropy_start"], runs["scene"]["entropy_end"]],
            "evaluations": runs["scene"]["evaluations"],
            "centroid_offset_recovered_hz": float(off), "centroid_offset_injected_hz": 30.0,
            "centroid_fit_hz": float(runs["scene"]["centroid"]), "seconds": time.perf_counter() - t0}


def cpu_baseline(threads: int):
    """The oracle (CPU restatement of the reference) on a bounded sample of the
    workload: one IW2 burst of 1000 lines x 2400 samples, decode -> SLC."""
    os.environ["S1G_ORACLE_THREADS"] = str(threads)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import s1_oracle as O
    from sentinel1_decode_gb300 import synth
    spec = synth.StreamSpec([synth.BurstSpec(num_lines=1000, num_quads=1200, swath="IW2", num_targets=10)], seed=7)
    data = synth.generate(spec)
    O.build_oracle()
    t = time.perf_counter()
    d = O.S1Decoder(data)
    out = d.get_azimuth_compressed_burst("IW2", 0)
    dt = time.perf_counter() - t
    samples = 1000 * 2400
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": "oracle decode->SLC of one IW2 burst 1000 lines x 2400 samples (%.1f s)" % dt,
            "seconds": dt, "shape": list(out.shape)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3", choices=["c3", "c1", "c2", "c4", "c5"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference's CPU path: its sources do not travel to the GPU host, so
        # the oracle restatement (numpy/scipy + C decoder) is timed on all cores
        steps = []
        cb = None
        for _ in range(args.warmup + args.steps):
            cb = cpu_baseline(threads)
            steps.append(cb["seconds"])
        timed = steps[args.warmup:]
        val = 2.4 / (sum(timed) / len(timed))
        line = {"metric": METRIC, "value": val, "unit": "Msamples/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * sum(timed) / len(timed), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "IW2 burst 1000 x 2400 (bounded sample of the 9-burst dual-pol swath)",
                           "parallelism": "cpu threads"},
                "impl": "reference",
                "cpu_baseline": {"value": val, "unit": "Msamples/s", "cores": threads, "kind": "port",
                                 "sample": cb["sample"]},
                "e2e": {"value": val, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    # data first (spawned generator processes, before CUDA is touched); with
    # N ranks every rank generates the same streams and processes its share
    # of their (stream, burst) units
    t_gen = time.perf_counter()
    streams = make_streams(args.workload, seed=0, workers=min(18, threads))
    t_gen = time.perf_counter() - t_gen

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from sentinel1_decode_gb300 import (AZIMUTH_COMPRESSED, S1Decoder, batch_outputs, build, launch_count,
                                        process_swath_batch)
    from sentinel1_decode_gb300.decoder import batch_host_outputs
    from sentinel1_decode_gb300.decoder import tuning_report
    build()
    rt = cudart()
    rt.cudaSetDevice(local)

    def sync_all():
        rt.cudaDeviceSynchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    swath = "S1" if args.workload == "c1" else "IW2"
    tops = swath != "S1"
    eccm = (13000, 100) if args.workload == "c4" else None

    def opened(s, precision="fp32"):
        d = S1Decoder(s, device=local, precision=precision)
        if eccm:
            d.apply_eccm(*eccm)
        return d

    decs = [opened(s) for s in streams]
    share = None          # per stream: the burst indices this rank processes
    if world > 1:
        from sentinel1_decode_gb300.shard import swath_units
        share = rank_bursts(swath_units(decs, swath), world, rank, len(decs))
        for d, bl in zip(decs, share):
            d.set_batch_bursts(bl)
    for _ in range(args.warmup):
        process_swath_batch(decs, swath, AZIMUTH_COMPRESSED)

    clocks = Clocks(local)
    sync_all()
    l0 = launch_count()
    dev_ms = 0.0
    samples = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        n, ms = process_swath_batch(decs, swath, AZIMUTH_COMPRESSED)
        samples += n
        dev_ms += ms
    sync_all()
    wall = time.perf_counter() - t0
    launches = launch_count() - l0
    # SLC outputs of one step of the whole workload (sizes the e2e host buffer)
    step_outs = batch_outputs(decs[0])
    clk = clocks.stop()
    samples_all, dev_ms_max = reduce_rate(float(samples), dev_ms)
    value = samples_all / (dev_ms_max / 1e3) / 1e6

    # stage breakdown: one untimed pass per stream alone, so that the event
    # times between stages are the stages' own (the timed step overlaps the
    # two polarisation streams)
    stages = {}
    for d in decs:
        d.set_stage_timing(True)
        process_swath_batch([d], swath, AZIMUTH_COMPRESSED)
        for k, (ms, cnt) in d.stage_times().items():
            stages[k] = stages.get(k, 0.0) + ms
        d.set_stage_timing(False)
    stages.pop("end", None)
    geo = []
    for k, d in enumerate(decs):
        geo.extend(burst_geometry(d, swath, tops, None if share is None else share[k]))
    nbursts = len(geo)
    c_in_total = sum(len(s) for s in streams)
    alg = {}
    for (n_a, n_r, S, n_out) in geo:
        per = algorithmic_bytes(n_a, n_r, S, n_out, c_in_total // nbursts) if tops else \
            algorithmic_bytes_sm(n_a, n_r, c_in_total // nbursts)
        for k, v in per.items():
            alg[k] = alg.get(k, 0) + v
    hbm, peak_kind = peaks()
    # dominant kernel: the time unfolding (k_tufr_fused, one launch per burst)
    # of the TOPS chain; for stripmap the slowest stage
    dom = "time_unfold" if tops else max((k for k in alg if k != "total"), key=lambda k: stages.get(k, 0.0))
    dom_kernel = {"time_unfold": "k_tufr_fused", "row_pass": "k_rowpass_fused", "azimuth_ifft": "k_czt_rows",
                  "range_compress": "k_rc_fused", "batch_decode": "k_decode_symbols"}[dom]
    dom_ms = stages.get(dom, 0.0) / nbursts
    achieved = (alg[dom] / nbursts) / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    tpu = profiled_value("k_tufr_fused") if tops else None
    traffic = tpu * sum(n_r * S for (_, n_r, S, _) in geo) / nbursts if tpu else None
    roofline = {"bound": "hbm", "kernel": dom_kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                "alg_bytes_per_launch": alg[dom] / nbursts, "launch_ms": dom_ms,
                "stage_ms_per_burst": {k: v / nbursts for k, v in sorted(stages.items())},
                "pipeline_alg_bytes_per_step": alg["total"],
                "pipeline_achieved_gbs": alg["total"] / (dev_ms / args.steps / 1e3) / 1e9,
                "note": ("instruction-issue and special-function bound: deramp staging (per-interval phase "
                         "polynomials), type-1 NUFFT gather (~58 samples per grid point, two range bins per "
                         "weight), forward and inverse ~9k grid FFT per range bin"
                         if tops else "shared-memory FFT bound (stripmap range-Doppler chain)")}

    # the compute roof: nominal FP32 flops of each stage (FFTs as 5 N log2 N,
    # chirp-z as its convolution FFTs plus pointwise products; the library's
    # s1g_burst_stage_flops) over the stage time, against SMs x 128 lanes x 2
    # x the SM clock sampled during the timed region
    if clk.get("sm_mhz") and geo:
        sms = ctypes.c_int()
        rt.cudaDeviceGetAttribute(ctypes.byref(sms), 16, local)
        peak_tf = fp32_peak_tflops(sms.value, clk["sm_mhz"])
        flops = {}
        for k, d in enumerate(decs):
            for b in range(d.num_bursts(swath)):
                if share is not None and b not in share[k]:
                    continue
                if tops and d.burst_shape(swath, b)[0] < 1000:
                    continue
                for st, v in d.stage_flops(swath, b).items():
                    if st != "tiles":
                        flops[st] = flops.get(st, 0.0) + v
        per_stage = {}
        for st, f in flops.items():
            ms = stages.get(st, 0.0)
            if ms > 0:
                tf = f / (ms / 1e3) / 1e12
                per_stage[st] = {"tflops": tf, "frac": tf / peak_tf, "gflop_per_burst": f / nbursts / 1e9}
        roofline["compute"] = {"unit": "TFLOP/s (FP32, nominal count)", "peak": peak_tf, "peak_kind":
                               "nominal: %d SMs x 128 lanes x 2 x %.0f MHz sampled" % (sms.value, clk["sm_mhz"]),
                               "kernel": dom_kernel, "frac": per_stage.get(dom, {}).get("frac"),
                               "stages": per_stage}

    # the roof this kernel meets: instruction issue (4 warp instructions per
    # SM per clock), at the SM clock sampled during the timed region
    ipu = profiled_value("k_tufr_fused", "warp_inst_per_unit") if tops else None
    if ipu and dom_ms > 0 and clk.get("sm_mhz"):
        sms = ctypes.c_int()
        rt.cudaDeviceGetAttribute(ctypes.byref(sms), 16, local)
        inst = ipu * sum(n_r * S for (_, n_r, S, _) in geo) / nbursts
        peak_issue = sms.value * 4 * clk["sm_mhz"] * 1e6
        roofline["issue"] = {"unit": "warp-inst/s", "inst_per_launch": inst, "achieved": inst / (dom_ms / 1e3),
                             "peak": peak_issue, "frac": inst / (dom_ms / 1e3) / peak_issue, "sms": sms.value}

    # plain FP64 GPU path on one burst of the workload
    fp64 = None
    if not args.no_fp64:
        d64 = opened(streams[0], "fp64")
        n_a, n_r = geo[0][0], geo[0][1]
        # a stripmap scene is focused by the swath product (the burst-level
        # azimuth product of the reference always runs the TOPS chain)
        az = (lambda d, **kw: d.get_azimuth_compressed_burst(swath, 0, **kw)) if tops else \
            (lambda d, **kw: d.get_azimuth_compressed_swath(swath, **kw))
        az(d64)
        az64 = az(d64)
        ms64 = d64.last_ms()
        fp64 = {"value": n_a * n_r / (ms64 / 1e3) / 1e6, "unit": "Msamples/s", "ms_per_burst": ms64,
                "burst": [n_a, n_r]}
        # accuracy of every product of the batched FP32 path on this burst,
        # against the FP64 path (the reference's arithmetic)
        d32 = opened(streams[0], "fp32")
        acc = {}
        for name, rd in (("range_compressed", False), ("range_doppler", True)):
            ref = d64.get_range_compressed_burst(swath, 0, range_doppler=rd)
            got = d32.get_range_compressed_burst(swath, 0, range_doppler=rd, dtype=np.complex64)
            acc[name] = {"rel_l2": rel_l2(got, ref)}
            if not rd:
                acc[name].update(point_target_errors(ref, got))
            del ref, got
        got = az(d32, dtype=np.complex64)
        acc["azimuth_compressed"] = {"rel_l2": rel_l2(got, az64), **point_target_errors(az64, got)}
        raw64 = d64.get_burst(swath, 0)
        acc["raw"] = {"bit_exact_f32": bool(np.array_equal(d32.get_burst(swath, 0, dtype=np.complex64),
                                                           raw64.astype(np.complex64)))}
        fp64["accuracy_fp32_vs_fp64"] = acc
        del az64, got, raw64
        d32.close()
        d64.close()

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        pinned = []
        for s in streams:
            p = ctypes.c_void_p()
            rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(len(s)), 0)
            ctypes.memmove(p, s, len(s))
            pinned.append((p, len(s)))
        out_bytes = sum(r * pt * (8 if t == 0 else 16) for (_, r, c, pt, t) in step_outs)
        host_out = ctypes.c_void_p()
        rt.cudaHostAlloc(ctypes.byref(host_out), ctypes.c_size_t(out_bytes), 0)
        e2e_t = 0.0
        e2e_samples = 0
        ds = None
        for it in range(args.warmup + args.steps):
            sync_all()
            t = time.perf_counter()
            # every step: the input byte streams from pinned host memory into
            # the handles (opened on the first step, reloaded after it: the
            # handles keep their plans when the packet layout is unchanged)
            if ds is None:
                ds = [S1Decoder.from_pointer(p.value, n, device=local, precision="fp32") for p, n in pinned]
                if eccm:
                    for d in ds:
                        d.apply_eccm(*eccm)
                if share is not None:
                    for d, bl in zip(ds, share):
                        d.set_batch_bursts(bl)
            else:
                for d, (p, n) in zip(ds, pinned):
                    d.reload_from_pointer(p.value, n)
            n, _ = process_swath_batch(ds, swath, AZIMUTH_COMPRESSED)
            if it == 0:
                # first step: read the SLCs back after the batch, then register
                # the same host slices so that later batches copy each burst
                # back as soon as it is formed (overlapping the other bursts)
                off = 0
                slices = []
                for (ptr, r, c, pt, ty) in batch_outputs(ds[0]):
                    nb = r * pt * (8 if ty == 0 else 16)
                    if off + nb > out_bytes:
                        raise RuntimeError("e2e: outputs exceed the host buffer")
                    rt.cudaMemcpy(ctypes.c_void_p(host_out.value + off), ctypes.c_void_p(ptr), ctypes.c_size_t(nb), 2)
                    slices.append(host_out.value + off)
                    off += nb
                batch_host_outputs(ds[0], slices)
            sync_all()
            if it >= args.warmup:
                e2e_t += time.perf_counter() - t
                e2e_samples += n
        for d in ds:
            d.close()
        e2e_all, e2e_tmax = reduce_rate(float(e2e_samples), e2e_t)
        e2e = {"value": e2e_all / e2e_tmax / 1e6, "unit": "Msamples/s",
               "h2d_bytes_per_step": sum(n for _, n in pinned), "d2h_bytes_per_step": out_bytes}

    # autofocus scene: entropy autofocus over the phase-error polynomial and
    # the centroid offset with the TOPS chain's hand-written adjoint (FP32)
    af = None
    if args.workload == "c5" and rank == 0:
        af = c5_autofocus(streams[0], local)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(threads)
        cpu.pop("seconds", None)
        cpu.pop("shape", None)

    if rank == 0:
        nb = nbursts
        line = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 phases and fits)",
                "data": "synthetic (seeded L0 generator)",
                "config": {"workload": "%s: %d %s bursts x %d pol, lines %d-%d, samples %d-%d%s" % (
                    args.workload, nb // max(len(streams), 1), swath, len(streams), min(g[0] for g in geo),
                    max(g[0] for g in geo), min(g[1] for g in geo), max(g[1] for g in geo),
                    ", ECCM %d/%d" % eccm if eccm else ""),
                    "samples_per_step": int(samples_all) // args.steps,
                    "parallelism": ("(stream, burst) units split over %d GPUs (LPT plan, no collective on the data "
                                    "path)" % world) if world > 1 else "1 GPU",
                    "l2": "inputs larger than L2 (no flush)"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk, "fp64_plain": fp64, "fft_tuning": tuning_summary(tuning_report()),
                "wall_s_timed": wall, "gen_s": t_gen}
        if af is not None:
            line["autofocus"] = af
        print(json.dumps(line), flush=True)
    for d in decs:
        d.close()


if __name__ == "__main__":
    main()
