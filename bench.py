#!/usr/bin/env python3
"""Benchmark: critical-curve points per second on one synthetic star field.

Workload (default): 2000 Salpeter stars (m in [0.08, 1.5] solar masses,
rescaled to mean 1), rectangular field, kappa_tot 0.45, kappa_star 0.35,
shear 0.35, theta_star 1, num_phi 2048 (the nearest value the reference
accepts for 2000: a multiple of 2 * num_branches), 32 branches -- 4056 roots,
8.44e6 critical-curve points per field.

A step is one full field solve: star generation, tree and FMM, the Aberth
solve at the branch centres, the phi continuation, the 1/mu residual and the
caustic map of every point, and the FP64 polish, all resident in HBM.
``value`` is points/s from the device-side span of each step (CUDA events in
the library, star generation -> polished caustics on the device); ``e2e`` is
the same metric through the public API with a host star array in and host
result arrays (roots, caustics, 1/mu errors) out, timed around the calls.  L2
is flushed (256 MiB write) before every timed step.

Beside the headline, the default run measures, each in full (nothing
extrapolated): the same field in plain FP64 and with the full-sum
continuation; the large field (20000 Kroupa stars, num_phi 10240, 128
branches) in mixed precision and in plain FP64; one pass over the 256-field
batch in both precisions; and the first 16 requests of the Poisson serving
stream, replayed at their arrival times once in each precision, with p50/p99
latencies.  ``--headline-only`` skips those records.

Multi-GPU: fields are independent, so N ranks run N replicas (seed + rank)
with no collective on the data path ("scaling": "weak"); value is all ranks'
points over the slowest rank's time.

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (the reference's own code cannot travel to this
machine).  A step is B complete branches of the field, one per host
thread (16 on a 16-core host) -- the Aberth solve at their centres and the
whole continuation of both sides, with the reference's sweep counts and
early return, the rows split over the threads; step k takes branches kB to
kB + B - 1 (mod num_branches).  ``value`` is the points of the timed steps
over their summed time: measured, not extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "single_field_n2000_salpeter_rect": dict(
        kappa_tot=0.45, kappa_star=0.35, shear=0.35, theta_star=1.0, mass_function="salpeter",
        m_lower=0.08, m_upper=1.5, m_solar=4.954984, rectangular=1, approx=1, num_stars=2000,
        num_phi=2048, num_branches=32, random_seed=1235),
    "small_field_n100_equal_disc": dict(
        kappa_tot=0.3, kappa_star=0.3, shear=0.1, theta_star=1.0, mass_function="equal", rectangular=0,
        approx=1, num_stars=100, num_phi=100, num_branches=1, random_seed=1234),
    "large_field_n20000_kroupa_rect": dict(
        kappa_tot=0.7, kappa_star=0.6, shear=0.2, theta_star=1.0, mass_function="kroupa", m_lower=0.08,
        m_upper=1.5, m_solar=1.0, rectangular=1, approx=1, num_stars=20000, num_phi=10240,
        num_branches=128, random_seed=1236),
}
DEFAULT = "single_field_n2000_salpeter_rect"
# workloads of many fields: a step is one pass over the whole set
MULTI_WORKLOADS = ("batch_256_fields_n50_1000_disc", "serving_poisson_salpeter_disc")


def _singular(kappa: float, shear: float) -> bool:
    """|1 - kappa| or |1 - kappa -/+ shear| near 0 blows up the field size."""
    return abs(1 - kappa) < 0.05 or abs(1 - kappa - shear) < 0.05 or abs(1 - kappa + shear) < 0.05


def batch_fields(count: int = 256) -> list[dict]:
    """256 independent disc fields of equal masses: N ~ U{50..1000}, kappa_star
    ~ U[0.05, 0.6], smooth fraction s ~ U[0, 0.3] (kappa_tot = kappa_star /
    (1 - s)), shear ~ U[0, 0.5], rejecting near-singular (kappa_tot, shear);
    num_phi 512 (the nearest value the reference accepts for 500: a multiple
    of 2 * num_branches), 8 branches, star seeds 10000 + i."""
    import numpy as np
    rng = np.random.default_rng(2024)
    out = []
    while len(out) < count:
        n = int(rng.integers(50, 1001))
        ks = float(rng.uniform(0.05, 0.6))
        s = float(rng.uniform(0.0, 0.3))
        g = float(rng.uniform(0.0, 0.5))
        k = ks / (1 - s)
        if _singular(k, g):
            continue
        out.append(dict(kappa_tot=k, kappa_star=ks, shear=g, theta_star=1.0, mass_function="equal", rectangular=0,
                        approx=1, num_stars=n, num_phi=512, num_branches=8, random_seed=10000 + len(out)))
    return out


def serving_requests(count: int) -> list[tuple[float, dict]]:
    """Poisson request stream (exponential inter-arrival times, mean 50 ms,
    seed 4242): N log-uniform in [100, 50000], kappa_star ~ U[0.1, 0.8]
    (kappa_tot = kappa_star), shear ~ U[0, 0.6] rejecting near-singular
    values, Salpeter masses on [0.08, 1.5] with mean 1, discs,
    num_branches in {8, 32, 128}, num_phi = 2 nb ceil(U[1000, 10000] / 2 nb),
    star seeds 20000 + i.  Returns (arrival time in s, parameters)."""
    import math
    import numpy as np
    rng = np.random.default_rng(4242)
    t = 0.0
    out = []
    while len(out) < count:
        ks = float(rng.uniform(0.1, 0.8))
        g = float(rng.uniform(0.0, 0.6))
        if _singular(ks, g):
            continue
        n = int(round(math.exp(rng.uniform(math.log(100), math.log(50000)))))
        nb = int(rng.choice([8, 32, 128]))
        nphi = 2 * nb * int(math.ceil(rng.uniform(1000, 10000) / (2 * nb)))
        t += float(rng.exponential(0.05))
        out.append((t, dict(kappa_tot=ks, kappa_star=ks, shear=g, theta_star=1.0, mass_function="salpeter",
                            m_lower=0.08, m_upper=1.5, m_solar=4.954984, rectangular=0, approx=1, num_stars=n,
                            num_phi=nphi, num_branches=nb, random_seed=20000 + len(out))))
    return out


def reduce_over_ranks(x: float, op: str, ws: int, device: str = "cuda") -> float:
    """Max or sum of a scalar over the ranks of the process group (the
    slowest replica's time, all replicas' points); the identity on one rank.
    The only collective of a multi-GPU run: replicas share no data."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return float(t.item())


def shard(items: list, rank: int, ws: int) -> list:
    """The independent units (fields, requests) rank takes: every ws-th one."""
    return items[rank::ws]


def replica_seed(seed: int, rank: int) -> int:
    """Star seed of rank's replica of the single-field workload."""
    return seed + rank


METRIC = "crit-curve pts/s mixed vs plain FP64 (err≤1e-9); fields/s, p50/p99 latency"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}




# DRAM bytes (read + write) of the continuation launch per continuation point,
# from the full-size one-pass capture summarised in
# profiles/track_kernel_n2000_salpeter_phi512.md: 35.5 + 172.2 MB for the
# 4056 * 2048 continuation points of the bench field's launch (the 40-byte
# outputs, part of which L2 still holds when the launch ends; leaf records
# and stars stay in L2).
CONT_DRAM_BYTES_PER_POINT = (35.51e6 + 172.24e6) / (4056 * 2048)
# FP64-pipe activity of the continuation kernel in the --set full capture of
# the same profile (sm__pipe_fp64_cycles_active over active cycles)
CONT_FP64_PIPE_ACTIVE = 0.251


def hbm_peak_gbs() -> float | None:
    """Measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except Exception:  # noqa: BLE001
        return None


def measure_peaks() -> dict:
    exe = os.path.join(ROOT, "ccf_gb300", "lib", "ccf_peaks")
    try:
        out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout.strip().splitlines()[-1]
        return json.loads(out)
    except Exception as e:  # noqa: BLE001
        return {"error": str(e)}


def unfolded_share(info: dict) -> float:
    """Share of the leaves whose expansion does not carry the smooth-mass
    series (the stand-in for the share of evaluations there)."""
    return 1.0 - info.get("leaves_folded", 0) / max(1, info["num_leaves"])


def algorithmic_flops_per_eval(info: dict, approx: int) -> float:
    """Algorithmic work of one evaluation of f and f' with the near-pole
    correction: 40 flops per near star (the two derivative sums, 20 each), 16
    per expansion order (two complex Horner passes) and 12 per Taylor term of
    the rectangular smooth-mass series (S = 12 (taylor_smooth - 1)), the
    series charged to the leaves that do not carry it folded into their
    expansion."""
    w = 40.0 * info["near_mean"] + 16.0 * info["expansion_order"]
    if info["rectangular"] and approx:
        w += 12.0 * (info["taylor_smooth"] - 1) * unfolded_share(info)
    return w


def continuation_algorithmic_flops(info: dict, approx: int) -> float:
    """Algorithmic work of the continuation: its evaluations (tracker steps
    and any full-sum updates) and 10 flops per reciprocal-sum term (complex
    difference 2, |d|^2 3, reciprocal 1, scale 2, accumulate 2)."""
    evals = info["root_updates"] - info["root_updates_init"]
    terms = info["sum_terms"] - info["sum_terms_init"]
    return 10.0 * terms + algorithmic_flops_per_eval(info, approx) * evals


def tracker_ops_per_eval(info: dict, approx: int) -> float:
    """FP32 operations one tracker evaluation executes (eval_track_df),
    counted from its double-float primitives: two_sum 6, fast_two_sum 3,
    df_add 20, df_mul 7, df_sumsq 19, df_dot2 19, df_rcp 13, a running-sum
    product (dfacc_fma) 12; a complex double-float Horner step (dfc_fma) 54.
    Per near star 174 (the difference, 1/d, 1/d^2, the m/d and m/d^2 sums in
    double-float, pole and m/d^3 in FP32); the alpha and d alpha/d zbar
    Horner passes over the local expansion; the FP32 f' pass; for the
    rectangular Taylor smooth mass the d alpha/d zbar and alpha series,
    charged to the unfolded share of the leaves; about 200 for the assembly
    of f, the step and the bookkeeping.  The ratio to
    algorithmic_flops_per_eval is the cost of the double-float emulation."""
    n = info["near_mean"]
    P = info["expansion_order"]
    per = 174.0 * n + 54.0 * (2 * P - 3) + 8.0 * max(P - 3, 0) + 200.0
    if info["rectangular"] and approx:
        ts = info["taylor_smooth"]
        m = (ts - 1) // 2
        per += (54.0 * (max(m - 1, 0) + ts + 1) + 8.0 * max(m - 1, 0) + 250.0) * unfolded_share(info)
    return per


def continuation_roofline(info: dict, approx: int, t_cont: float, peaks: dict, num_phi: int) -> dict:
    """Roofline of the dominant kernel (the continuation): algorithmic flops
    over its CUDA-event span, against the measured FP32 FMA peak (the
    double-float arithmetic runs on the FP32 pipe), with the FP64-pipe
    activity of its ncu capture beside it."""
    flops = continuation_algorithmic_flops(info, approx)
    achieved = flops / t_cont / 1e12 if t_cont > 0 else 0.0
    peak32, peak64 = peaks.get("fp32_tflops"), peaks.get("fp64_tflops")
    evals = info["root_updates"] - info["root_updates_init"]
    ops = tracker_ops_per_eval(info, approx)
    traffic = CONT_DRAM_BYTES_PER_POINT * info["num_roots"] * num_phi
    hbm_peak = hbm_peak_gbs()
    return {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
            "frac": (achieved / peak32) if peak32 else None, "traffic": traffic,
            "kernel": "track_kernel (phi continuation)",
            "work": "algorithmic: 40 n_near + 16 P + 12 (taylor_smooth - 1) x unfolded share per evaluation, "
                    "10 per reciprocal-sum term",
            "flops_per_evaluation": algorithmic_flops_per_eval(info, approx), "evaluations": evals,
            "frac_of_fp64_peak": (achieved / peak64) if peak64 else None,
            "executed_ops": {"fp32_ops_per_evaluation": ops, "tflops": evals * ops / t_cont / 1e12 if t_cont > 0 else 0,
                             "per_algorithmic_flop": ops / algorithmic_flops_per_eval(info, approx)},
            "fp64_pipe_active": CONT_FP64_PIPE_ACTIVE,
            "peak_source": "ccf_gb300/lib/ccf_peaks (FFMA and DFMA chains, measured on the box)",
            "traffic_source": "per-point DRAM bytes of the ncu capture in "
                              "profiles/track_kernel_n2000_salpeter_phi512.md, scaled by points",
            "hbm_gbs": traffic / t_cont / 1e9 if t_cont > 0 else None, "hbm_peak_gbs": hbm_peak,
            "hbm_frac": (traffic / t_cont / 1e9 / hbm_peak) if (t_cont > 0 and hbm_peak) else None}


def reference_branches_per_step(cfg: dict, threads: int) -> int:
    """Branches in one reference step: one per host thread (two rows each, one
    per side).  On the 16-core Grace host 16 branches of the 2000-star field
    run at the whole field's rate (4.6e5 points/s both); 8 branches lose 11 %
    to the rows' uneven costs."""
    return max(1, min(cfg["num_branches"], threads))


def cpu_reference_step(cfg: dict, threads: int, step: int, max_steps: int = 0) -> dict:
    """The reference algorithm (CPU restatement) on complete branches of the
    field -- step k takes branches [kB, kB + B) mod num_branches, B from
    reference_branches_per_step: the Aberth solve at their centres and the
    whole continuation of both sides, with the reference's 30/20 sweeps and
    early return, the rows split over the threads.  Time = the oracle's own
    timers over the library's span (stars, tree, initial solve,
    continuation, errors and caustics)."""
    from oracle import oracle as O
    nb = cfg["num_branches"]
    half = cfg["num_phi"] // (2 * nb)
    B = reference_branches_per_step(cfg, threads)
    first = (step * B) % nb
    r = O.run(num_threads=threads, max_branches=B, first_branch=first, branch_stride=1, max_steps=max_steps, **cfg)
    inf = r["info"]
    t = inf["t_stars"] + inf["t_tree"] + inf["t_init_roots"] + inf["t_ccs"] + inf["t_caustics"]
    steps = min(max_steps, half) if max_steps > 0 else half
    points = B * inf["num_roots"] * (2 * steps + 1)
    return {"value": points / t, "seconds": t, "points": points, "branches": [(first + i) % nb for i in range(B)]}


def _sync():
    import torch
    torch.cuda.synchronize()


def time_field(cfg: dict, precision: str, runs: int, warmup: int, local: int, flush=None, **extra) -> tuple:
    """(median device span in s, info of the last run) of `runs` solves of one
    field after `warmup` untimed ones, L2 flushed before each."""
    from ccf_gb300 import CCF
    c = CCF(**cfg)
    c.precision, c.device, c.write_mu_length_scales = precision, local, 0
    for k, v in extra.items():
        setattr(c, k, v)
    ts, info = [], None
    for i in range(warmup + runs):
        if flush is not None:
            flush.zero_()
        _sync()
        assert c.run(-1), c.last_error()
        if i >= warmup:
            info = c.info()
            ts.append(info["t_total"])
    return statistics.median(ts), info


def batch_handles(fields: list, precision: str, local: int) -> list:
    from ccf_gb300 import CCF
    cs = []
    for f in fields:
        c = CCF(**f)
        c.precision, c.device, c.write_mu_length_scales = precision, local, 0
        cs.append(c)
    return cs


def batch_pass(cs: list, barrier, results: bool = False, bufs=None) -> tuple:
    """One run_batch over every handle (wall time, device to device)."""
    from ccf_gb300 import run_batch
    barrier()
    t0 = time.perf_counter()
    assert run_batch(cs), cs[0].last_error()
    out = [c.results(stars=False, out=b) for c, b in zip(cs, bufs)] if results else None
    barrier()
    return time.perf_counter() - t0, out


def serving_stream(prec: str, requests: list, slots: int, budget: float, local: int) -> dict:
    """Replay (arrival time, parameters) requests through the request loop:
    submitted at their arrival times, each waited for and released in
    order; span from the first arrival to the last completion."""
    from ccf_gb300 import Server
    s = Server(slots=slots, hbm_budget=budget, device=local)
    ids = []
    t0 = time.perf_counter()

    def submitter():
        for t_arr, p in requests:
            dt = t0 + t_arr - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(s.submit(precision=prec, write_mu_length_scales=0, write_stars=0, **p))

    th = threading.Thread(target=submitter)
    th.start()
    infos, pts, failed, errs, unconv = [], 0, 0, [], 0
    k = 0
    while k < len(requests):
        if k >= len(ids):
            time.sleep(0.001)
            continue
        rid = ids[k]
        st = s.wait(rid)
        infos.append(s.info(rid))
        if st == 0:
            fi = s.field(rid).info()
            pts += fi["num_points"]
            errs.append(fi["max_error"])
            unconv += fi["unconverged"]
        else:
            failed += 1
        s.release(rid)
        k += 1
    th.join()
    stats = s.stats()
    s.close()
    span = max(i["t_end"] for i in infos) - min(i["t_submit"] for i in infos)
    lat = sorted(i["t_end"] - i["t_submit"] for i in infos)
    return {"points": pts, "span": span, "latency": lat, "stats": stats, "failed": failed,
            "max_error_1/mu": max(errs) if errs else None, "unconverged": unconv}


def serving_summary(r: dict, n: int) -> dict:
    import numpy as np
    return {"points_per_s": r["points"] / r["span"], "fields_per_s": n / r["span"], "span_s": r["span"],
            "latency_p50_s": float(np.percentile(r["latency"], 50)),
            "latency_p99_s": float(np.percentile(r["latency"], 99)), "failed": r["failed"],
            "max_error_1/mu": r["max_error_1/mu"], "unconverged": r["unconverged"]}


def large_field_record(local: int, flush) -> dict:
    """The 20000-star field in mixed precision and in plain FP64, both in full."""
    name = "large_field_n20000_kroupa_rect"
    cfg = WORKLOADS[name]
    tm, im = time_field(cfg, "mixed", 2, 1, local, flush)
    td, idd = time_field(cfg, "fp64", 1, 1, local, flush)
    pts = im["num_points"]
    return {"workload": name, "points": pts,
            "mixed": {"value": pts / tm, "ms": 1e3 * tm, "max_error_1/mu": im["max_error"],
                      "points_at_fp64_floor": im["points_at_fp64_floor"],
                      "points_above_target": im["points_above_target"], "unconverged": im["unconverged"],
                      "centres_solved": im["centres_solved"]},
            "fp64": {"value": pts / td, "ms": 1e3 * td, "max_error_1/mu": idd["max_error"],
                     "points_at_fp64_floor": idd["points_at_fp64_floor"],
                     "points_above_target": idd["points_above_target"], "unconverged": idd["unconverged"]},
            "mixed_over_fp64": td / tm, "unit": "points/s"}


def batch_record(local: int, barrier) -> dict:
    """One pass over the 256 batch fields per precision (mixed: median of 2)."""
    fields = batch_fields()
    out = {"workload": "batch_256_fields_n50_1000_disc", "fields": len(fields), "unit": "points/s"}
    for prec, runs in (("mixed", 2), ("fp64", 1)):
        cs = batch_handles(fields, prec, local)
        batch_pass(cs, barrier)
        t = statistics.median(batch_pass(cs, barrier)[0] for _ in range(runs))
        pts = float(sum(c.info()["num_points"] for c in cs))
        out[prec] = {"value": pts / t, "fields_per_s": len(fields) / t, "ms": 1e3 * t,
                     "max_error_1/mu": max(c.info()["max_error"] for c in cs),
                     "unconverged": int(sum(c.info()["unconverged"] for c in cs))}
        del cs
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def serving_record(n: int, slots: int, budget: float, local: int) -> dict:
    """The first n requests of the Poisson stream at their arrival times, once
    per precision on a fresh server."""
    reqs = serving_requests(n)
    warm = [(0.0, p) for _, p in serving_requests(n) if p["num_stars"] <= 1000][:2]
    out = {"workload": "serving_poisson_salpeter_disc", "requests": n, "slots": slots, "hbm_budget_bytes": budget}
    for prec in ("mixed", "fp64"):
        serving_stream(prec, warm, slots, budget, local)
        out[prec] = serving_summary(serving_stream(prec, reqs, slots, budget, local), n)
    out["mixed_over_fp64"] = out["mixed"]["points_per_s"] / out["fp64"]["points_per_s"]
    return out


def run_multi(args) -> None:
    """Workloads of many fields.  batch: one run_batch over 256 fields per
    step.  serving: a Poisson stream of requests through the request loop
    (ccf_server_*), timed from the first arrival to the last completion, with
    queue-inclusive latencies, in mixed precision and (same stream) plain
    FP64."""
    ws, rank, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def reduce(x: float, op: str) -> float:
        return reduce_over_ranks(x, op, ws)

    line = {"metric": METRIC, "unit": "points/s", "n_gpus": ws, "steps": args.steps, "warmup": max(3, args.warmup),
            "higher_is_better": True, "vs_baseline": None, "data": "synthetic (seeded star fields)",
            "dtype": "f32+df32+f64 (double-float f and caustics, FP32 f' and step, FP64 coordinates)"}
    with ClockSampler(local) as clocks:
        if args.workload == "batch_256_fields_n50_1000_disc":
            fields = batch_fields()
            mine = shard(fields, rank, ws)    # the fields are independent: split them between ranks
            cs = batch_handles(mine, "mixed", local)
            for _ in range(max(3, args.warmup)):
                batch_pass(cs, barrier)
            ts = [batch_pass(cs, barrier)[0] for _ in range(args.steps)]
            t = reduce(statistics.median(ts), "max")
            pts = reduce(float(sum(c.info()["num_points"] for c in cs)), "sum")
            # page-locked destinations for every field's results, allocated
            # once outside the timed pass (the copies themselves are timed)
            bufs = [c.result_buffers(pinned=True) for c in cs]
            te, outs = batch_pass(cs, barrier, results=True, bufs=bufs)
            te = reduce(te, "max")
            d2h = sum(o["ccs"].nbytes + o["caustics"].nbytes + o["errs"].nbytes for o in outs)
            fp = batch_handles(mine, "fp64", local)
            batch_pass(fp, barrier)
            t64 = reduce(batch_pass(fp, barrier)[0], "max")
            line.update({"value": pts / t, "ms_per_step": 1e3 * t, "scaling": "strong",
                         "fields_per_s": len(fields) / t,
                         "config": {"workload": args.workload, "fields": len(fields), "num_phi": 512,
                                    "num_branches": 8, "num_stars": "U{50..1000}", "mass_function": "equal",
                                    "geometry": "disc"},
                         "run": {"precision": "mixed", "l2": "inputs are 256 fields; no flush between passes",
                                 "parallelism": f"fields split over {ws} GPU(s)"},
                         "e2e": {"value": pts / te, "unit": "points/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": d2h},
                         "fp64_plain": {"value": pts / t64, "unit": "points/s", "ms_per_step": 1e3 * t64},
                         "gpu_launches": int(sum(c.info()["kernel_launches"] for c in cs)),
                         "detail": {"points": pts, "max_error_1/mu": max(c.info()["max_error"] for c in cs),
                                    "unconverged": int(sum(c.info()["unconverged"] for c in cs))}})
        else:
            reqs = shard(serving_requests(args.requests), rank, ws)
            warm = [(0.0, p) for _, p in reqs if p["num_stars"] <= 1000][:2]
            serving_stream("mixed", warm, args.slots, args.hbm_budget, local)
            r = serving_stream("mixed", reqs, args.slots, args.hbm_budget, local)
            span = reduce(r["span"], "max")
            pts = reduce(float(r["points"]), "sum")
            lat = r["latency"]
            # the same stream in plain FP64 (the first fp64_requests of it, at their arrival times)
            sub = reqs[:args.fp64_requests]
            r64 = rm = None
            if sub:
                serving_stream("fp64", warm, args.slots, args.hbm_budget, local)
                r64 = serving_summary(serving_stream("fp64", sub, args.slots, args.hbm_budget, local), len(sub))
                rm = serving_summary(serving_stream("mixed", sub, args.slots, args.hbm_budget, local), len(sub))
            line.update({"value": pts / span, "ms_per_step": 1e3 * span, "steps": 1, "scaling": "weak",
                         "fields_per_s": reduce(float(len(reqs)), "sum") / span,
                         "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                         "config": {"workload": args.workload, "requests": args.requests,
                                    "arrivals": "Poisson, mean 50 ms, seed 4242",
                                    "num_stars": "log-uniform [100, 50000]", "num_branches": "{8, 32, 128}",
                                    "num_phi": "2 nb ceil(U[1000, 10000] / 2 nb)", "mass_function": "salpeter",
                                    "geometry": "disc"},
                         "run": {"precision": "mixed", "slots": args.slots, "hbm_budget_bytes": args.hbm_budget,
                                 "l2": "inputs are whole fields; no flush",
                                 "parallelism": f"request streams split over {ws} GPU(s)"},
                         "e2e": {"value": pts / span, "unit": "points/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": 0},
                         "server": dict(r["stats"]),
                         "fp64_plain": {"requests": len(sub), "arrivals": "the stream's own arrival times",
                                        "fp64": r64, "mixed": rm,
                                        "mixed_over_fp64": rm["points_per_s"] / r64["points_per_s"]} if sub else None,
                         "gpu_launches": None,
                         "detail": {"points": pts, "failed": r["failed"], "max_error_1/mu": r["max_error_1/mu"],
                                    "unconverged": r["unconverged"]}})
    line["clocks"] = clocks.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference(args) -> None:
    """The reference algorithm on the host cores (see the module docstring):
    step k is branch k mod num_branches, complete."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfg = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    for k in range(args.warmup):
        cpu_reference_step(cfg, threads, k, max_steps=1)
    runs = [cpu_reference_step(cfg, threads, k) for k in range(args.steps)]
    t = sum(r["seconds"] for r in runs)
    pts = sum(r["points"] for r in runs)
    v = pts / t
    nb = cfg["num_branches"]
    B = reference_branches_per_step(cfg, threads)
    sample = (f"each step {B} complete branches of {nb} (step k: branches kB .. kB+B-1 mod {nb}): their centres' "
              f"Aberth solve and both sides' whole continuation, reference sweep counts and early return, the "
              f"rows split over {threads} host threads; value = the steps' points over their summed time")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded star field)",
        "config": {"workload": args.workload, **cfg},
        "run": {"precision": "fp64", "threads": threads},
        "cpu_baseline": {"value": v, "unit": "points/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "detail": {"points_per_step": pts / args.steps, "branches": [r["branches"] for r in runs]},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS) + list(MULTI_WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=1, help="plain-FP64 steps timed beside the main arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the large-field, batch and serving records of the default run")
    ap.add_argument("--requests", type=int, default=64, help="serving: requests in the stream")
    ap.add_argument("--serving-requests", type=int, default=16, help="default run: requests of the serving record")
    ap.add_argument("--slots", type=int, default=4, help="serving: requests running at once")
    ap.add_argument("--hbm-budget", type=float, default=60e9, help="serving: admission budget in bytes")
    ap.add_argument("--fp64-requests", type=int, default=16, help="serving: requests replayed in plain FP64")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload in MULTI_WORKLOADS:
        run_multi(args)
        return

    ws, rank, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from ccf_gb300 import CCF

    cfg = dict(WORKLOADS[args.workload])
    cfg["random_seed"] = replica_seed(cfg["random_seed"], rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def make(prec):
        c = CCF(**cfg)
        c.precision = prec
        c.device = local
        c.write_mu_length_scales = 0
        return c

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    c = make(args.precision)
    for _ in range(max(3, args.warmup)):
        flush.zero_()
        torch.cuda.synchronize()
        assert c.run(-1), c.last_error()
    infos = []
    barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            assert c.run(-1), c.last_error()
            infos.append(c.info())
        barrier()
    t_dev = reduce_over_ranks(sum(i["t_total"] for i in infos), "max", ws)
    info = infos[-1]
    points = info["num_points"]
    value = points * args.steps * ws / t_dev

    # end to end through the public API: host star array in, host roots,
    # caustics and 1/mu errors out
    res = c.results()
    stars_host = np.ascontiguousarray(res["stars"])
    corner = complex(info["corner_x1"], info["corner_x2"])
    e = make(args.precision)
    e.set_stars(stars_host, info["rectangular"], corner, info["theta_star"])
    assert e.run(-1), e.last_error()
    bufs = e.result_buffers(pinned=True)   # page-locked destinations, reused every step
    e.results(stars=False, out=bufs)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e.set_stars(stars_host, info["rectangular"], corner, info["theta_star"])
        assert e.run(-1), e.last_error()
        out = e.results(stars=False, out=bufs)
    barrier()
    t_e2e = time.perf_counter() - t0
    h2d = stars_host.nbytes
    d2h = out["ccs"].nbytes + out["caustics"].nbytes + out["errs"].nbytes
    del e, bufs, out, res

    peaks = measure_peaks()
    t_cont = statistics.median(i["t_ccs"] for i in infos)
    roofline = continuation_roofline(info, cfg.get("approx", 1), t_cont, peaks, cfg["num_phi"])
    roofline["kernel_share_of_step"] = t_cont / statistics.median(i["t_total"] for i in infos)

    fp64 = full_sum = None
    if args.precision == "mixed" and args.fp64_steps > 0:
        td, _ = time_field(cfg, "fp64", args.fp64_steps, 1, local, flush)
        fp64 = {"value": points / td, "unit": "points/s", "ms_per_step": 1e3 * td}
        if cfg["num_stars"] <= 5000:
            # the reference's continuation scheme (the full Aberth step for
            # every root of a row) on the same field and GPU, both precisions
            full_sum = {"unit": "points/s"}
            for prec in ("mixed", "fp64"):
                tf, _ = time_field(cfg, prec, args.fp64_steps, 1, local, flush, continuation="aberth")
                full_sum[prec] = points / tf
                full_sum[prec + "_ms_per_step"] = 1e3 * tf

    records = {}
    if rank == 0 and ws == 1 and args.workload == DEFAULT and not args.headline_only:
        del c
        records["large_field"] = large_field_record(local, flush)
        records["batch"] = batch_record(local, barrier)
        if args.serving_requests > 0:
            records["serving"] = serving_record(args.serving_requests, args.slots, args.hbm_budget, local)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cb = cpu_reference_step(cfg, threads, 0)
        cpu = {"value": cb["value"], "unit": "points/s", "cores": threads, "kind": "port",
               "sample": f"branches {cb['branches'][0]}..{cb['branches'][-1]} of the field, complete: their "
                         "centres' Aberth solve and both sides' whole continuation with the reference's sweep "
                         f"counts and early return, the rows split over {threads} host threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+df32+f64 (double-float f and caustics, FP32 f' and step, FP64 coordinates, FP64 polish)"
            if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded star field)",
            "config": {"workload": args.workload, **cfg},
            "run": {"precision": args.precision, "l2": "flushed before every timed step (256 MiB write)",
                    "parallelism": f"replicas x{ws}"},
            "e2e": {"value": points * args.steps * ws / t_e2e, "unit": "points/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roofline,
            "fp64_plain": fp64,
            "full_sum_continuation": full_sum,
            **records,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": int(info["kernel_launches"]) * args.steps,
            "detail": {"num_points": points, "num_roots": info["num_roots"], "tree_levels": info["tree_levels"],
                       "rerun_flags": info["rerun_flags"],
                       "expansion_order": info["expansion_order"], "max_error_1/mu": info["max_error"],
                       "unconverged": info["unconverged"], "sweeps_init": info["max_sweeps_init"],
                       "sweeps_step": info["max_sweeps_step"], "root_updates": info["root_updates"],
                       "sum_terms": info["sum_terms"], "rows_rerun": info["rows_rerun"],
                       "step_halvings": info["step_halvings"], "near_mean": info["near_mean"],
                       "num_leaves": info["num_leaves"], "leaves_folded": info["leaves_folded"],
                       "centres_solved": info["centres_solved"],
                       "t_stars": info["t_stars"], "t_tree": info["t_tree"],
                       "t_init_roots": info["t_init_roots"], "t_ccs": info["t_ccs"],
                       "t_polish": info["t_caustics"], "points_polished": info["points_polished"],
                       "points_above_target": info["points_above_target"],
                       "points_at_fp64_floor": info["points_at_fp64_floor"],
                       "max_error_unpolished": info["max_error_unpolished"],
                       "unconverged_unpolished": info["unconverged_unpolished"], "peaks": peaks},
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
