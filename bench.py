#!/usr/bin/env python3
"""Benchmark: critical-curve points per second on one synthetic star field.

Workload (default): 2000 Salpeter stars (m in [0.08, 1.5] solar masses,
rescaled to mean 1), rectangular field, kappa_tot 0.45, kappa_star 0.35,
shear 0.35, theta_star 1, num_phi 2048 (the nearest value the reference
accepts for 2000: a multiple of 2 * num_branches), 32 branches -- 4056 roots,
8.44e6 critical-curve points per field.

A step is one full field solve: star generation, tree and FMM, the Aberth
solve at every branch centre, the phi continuation, the 1/mu residual and
the caustic map of every point, all resident in HBM.  ``value`` is points/s
from the device-side span of each step (CUDA events in the library, star
generation -> caustics on the device); ``e2e`` is the same metric through the
public API with a host star array in and host result arrays (roots and
caustics) out, timed around the calls.  L2 is flushed (256 MiB write) before
every timed step.

Multi-GPU: fields are independent, so N ranks run N replicas (seed + rank)
with no collective on the data path ("scaling": "weak"); value is all ranks'
points over the slowest rank's time.

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (the reference's own code cannot travel to this
machine), on a bounded sample (the first branches for the first phi steps),
extrapolated to the full field from its initial-solve and per-step timers.
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
# from the ncu capture summarised in
# profiles/track_kernel_n2000_salpeter_phi512.md: 89.5 MB for the 4056 * 512
# continuation points of that launch (the 40-byte outputs and the column
# tables; leaf records and stars stay in L2).  It grows with the points written.
CONT_DRAM_BYTES_PER_POINT = 89.5e6 / (4056 * 512)


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


def tracker_flops_per_eval(info: dict, approx: int) -> float:
    """FP32 operations of one evaluation of the continuation tracker
    (eval_track_df), counted from its double-float primitives: two_sum 6,
    fast_two_sum 3, df_add 20, df_add_fast 11, df_mul 7, df_sqr 7, df_rcp 30;
    a complex double-float Horner step 81.  Per near star 234 (1/d, 1/d^2, the
    m/d and m/d^2 sums in double-float, pole and m/d^3 in FP32); the alpha and
    d alpha/d zbar Horner passes over the local expansion; the FP32 f' pass; for
    the rectangular Taylor smooth mass the d alpha/d zbar and alpha series;
    about 200 for the assembly of f, the step and the bookkeeping.  Leaves
    with the smooth-mass series folded into their expansion skip the series:
    it is charged to the unfolded share of the leaves (leaves_folded /
    num_leaves, the stand-in for the share of evaluations there)."""
    n = info["near_mean"]
    P = info["expansion_order"]
    per = 234.0 * n + 81.0 * (2 * P - 3) + 8.0 * max(P - 3, 0) + 200.0
    if info["rectangular"] and approx:
        ts = info["taylor_smooth"]
        m = (ts - 1) // 2
        unfolded = 1.0 - info.get("leaves_folded", 0) / max(1, info["num_leaves"])
        per += (81.0 * (max(m - 1, 0) + ts + 1) + 8.0 * max(m - 1, 0) + 250.0) * unfolded
    return per


def algorithmic_flops(info: dict, continuation_only: bool = True, n_near: int = 32) -> float:
    """FP work of the executed Aberth updates: 10 flops per reciprocal-sum
    term (complex difference 2, |d|^2 3, reciprocal 1, scale 2, accumulate 2)
    plus 40 per near star, 16 per expansion order and 12 per Taylor term of
    the smooth-mass series per update."""
    terms, updates = info["sum_terms"], info["root_updates"]
    if continuation_only:
        terms -= info["sum_terms_init"]
        updates -= info["root_updates_init"]
    extra = 40 * n_near + 16 * info["expansion_order"] + (12 * (info["taylor_smooth"] - 1) if info["rectangular"] else 0)
    return 10.0 * terms + float(extra) * updates


def cpu_reference(cfg: dict, threads: int, branches: int | None = None, steps: int = 2) -> dict:
    """Reference algorithm (CPU restatement) on a bounded sample, extrapolated."""
    from oracle import oracle as O
    nb = cfg["num_branches"]
    half = cfg["num_phi"] // (2 * nb)
    m = min(nb, branches or max(1, threads))
    st = min(steps, half)
    t0 = time.perf_counter()
    r = O.run(num_threads=threads, max_branches=m, max_steps=st, **cfg)
    wall = time.perf_counter() - t0
    inf = r["info"]
    t_full = inf["t_init_roots"] * (nb / m) + inf["t_ccs"] * (nb / m) * (half / st) + inf["t_caustics"] * (nb / m) * (half / st)
    points = inf["num_roots"] * (cfg["num_phi"] + nb)
    return {"value": points / t_full, "t_full_extrapolated": t_full, "sample_wall": wall,
            "sample": f"{m} of {nb} branches, {st} of {half} phi steps per side, fixed 30/20 sweeps; "
                      f"extrapolated linearly in branches and steps",
            "cores": threads}


def run_multi(args) -> None:
    """Workloads of many fields.  batch: one run_batch over 256 fields per
    step.  serving: a Poisson stream of requests through the request loop
    (ccf_server_*), timed from the first arrival to the last completion, with
    queue-inclusive latencies."""
    ws, rank, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from ccf_gb300 import CCF, Server, run_batch

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def reduce(x: float, op: str) -> float:
        return reduce_over_ranks(x, op, ws)

    MAX, SUM = "max", "sum"

    line = {"metric": METRIC, "unit": "points/s", "n_gpus": ws, "steps": args.steps, "warmup": max(3, args.warmup),
            "higher_is_better": True, "vs_baseline": None, "data": "synthetic (seeded star fields)",
            "dtype": "f32+df32+f64 (double-float f and caustics, FP32 f' and step, FP64 coordinates)"}
    with ClockSampler(local) as clocks:
        if args.workload == "batch_256_fields_n50_1000_disc":
            fields = batch_fields()
            mine = shard(fields, rank, ws)    # the fields are independent: split them between ranks

            def make(prec):
                cs = []
                for f in mine:
                    c = CCF(**f)
                    c.precision, c.device, c.write_mu_length_scales = prec, local, 0
                    cs.append(c)
                return cs

            def one_pass(cs, results=False, bufs=None):
                barrier()
                t0 = time.perf_counter()
                assert run_batch(cs), cs[0].last_error()
                out = [c.results(stars=False, out=b) for c, b in zip(cs, bufs)] if results else None
                barrier()
                return time.perf_counter() - t0, out

            cs = make("mixed")
            for _ in range(max(3, args.warmup)):
                one_pass(cs)
            ts = [one_pass(cs)[0] for _ in range(args.steps)]
            t = reduce(statistics.median(ts), MAX)
            pts = reduce(float(sum(c.info()["num_points"] for c in cs)), SUM)
            # page-locked destinations for every field's results, allocated
            # once outside the timed pass (the copies themselves are timed)
            bufs = [c.result_buffers(pinned=True) for c in cs]
            te, outs = one_pass(cs, results=True, bufs=bufs)
            te = reduce(te, MAX)
            d2h = sum(o["ccs"].nbytes + o["caustics"].nbytes + o["errs"].nbytes for o in outs)
            fp = make("fp64")
            one_pass(fp)
            t64 = reduce(one_pass(fp)[0], MAX)
            line.update({"value": pts / t, "ms_per_step": 1e3 * t, "scaling": "strong",
                         "fields_per_s": len(fields) / t,
                         "config": {"workload": args.workload, "fields": len(fields), "num_phi": 512,
                                    "num_branches": 8, "num_stars": "U{50..1000}", "mass_function": "equal",
                                    "geometry": "disc", "precision": "mixed",
                                    "l2": "inputs are 256 fields; no flush between passes",
                                    "parallelism": f"fields split over {ws} GPU(s)"},
                         "e2e": {"value": pts / te, "unit": "points/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": d2h},
                         "fp64_plain": {"value": pts / t64, "unit": "points/s", "ms_per_step": 1e3 * t64},
                         "gpu_launches": 2 + int(sum(c.info()["kernel_launches"] - 2 for c in cs)),
                         "detail": {"points": pts, "max_error_1/mu": max(c.info()["max_error"] for c in cs),
                                    "unconverged": int(sum(c.info()["unconverged"] for c in cs))}})
            if rank == 0 and ws == 1 and not args.no_cpu_baseline:
                threads = os.cpu_count() or 1
                tc, pc = 0.0, 0.0
                for f in fields[:16]:
                    cb = cpu_reference(f, threads, steps=2)
                    tc += cb["t_full_extrapolated"]
                    pc += cb["value"] * cb["t_full_extrapolated"]
                line["cpu_baseline"] = {"value": pc / tc, "unit": "points/s", "cores": threads, "kind": "port",
                                        "sample": "the first 16 of the 256 fields, each on all branches and 2 phi "
                                                  "steps per side, extrapolated in steps"}
        else:
            reqs = shard(serving_requests(args.requests), rank, ws)

            def stream(prec, requests):
                s = Server(slots=args.slots, hbm_budget=args.hbm_budget, device=local)
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
                infos, pts, failed = [], 0, 0
                k = 0
                while k < len(requests):
                    if k >= len(ids):
                        time.sleep(0.001)
                        continue
                    rid = ids[k]
                    st = s.wait(rid)
                    infos.append(s.info(rid))
                    if st == 0:
                        pts += s.field(rid).info()["num_points"]
                    else:
                        failed += 1
                    s.release(rid)
                    k += 1
                th.join()
                stats = s.stats()
                s.close()
                span = max(i["t_end"] for i in infos) - min(i["t_submit"] for i in infos)
                lat = sorted(i["t_end"] - i["t_submit"] for i in infos)
                return {"points": pts, "span": span, "latency": lat, "stats": stats, "failed": failed}

            stream("mixed", [(0.0, p) for _, p in serving_requests(4)])   # warm-up
            r = stream("mixed", reqs)
            span = reduce(r["span"], MAX)
            pts = reduce(float(r["points"]), SUM)
            lat = r["latency"]
            # the plain-FP64 comparison replays the first requests of at most
            # 5000 stars (a 50000-star field takes minutes in plain FP64), all
            # submitted at once in both precisions: a throughput comparison, not
            # bounded by the arrival times of the stream
            sub = [(0.0, q[1]) for q in reqs if q[1]["num_stars"] <= 5000][:args.fp64_requests]
            r64 = stream("fp64", sub) if sub else None
            rm = stream("mixed", sub) if sub else None
            line.update({"value": pts / span, "ms_per_step": 1e3 * span, "steps": 1, "scaling": "weak",
                         "fields_per_s": reduce(float(len(reqs)), SUM) / span,
                         "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                         "config": {"workload": args.workload, "requests": args.requests, "slots": args.slots,
                                    "hbm_budget_bytes": args.hbm_budget, "arrivals": "Poisson, mean 50 ms, seed 4242",
                                    "num_stars": "log-uniform [100, 50000]", "num_branches": "{8, 32, 128}",
                                    "num_phi": "2 nb ceil(U[1000, 10000] / 2 nb)", "mass_function": "salpeter",
                                    "geometry": "disc", "precision": "mixed", "l2": "inputs are whole fields; no flush",
                                    "parallelism": f"request streams split over {ws} GPU(s)"},
                         "e2e": {"value": pts / span, "unit": "points/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": 0},
                         "server": dict(r["stats"]),
                         "fp64_plain": {"requests": len(sub), "arrivals": "all at once",
                                        "value": r64["points"] / r64["span"],
                                        "mixed_same_requests": rm["points"] / rm["span"], "unit": "points/s",
                                        "ratio_mixed_over_fp64": (rm["points"] / rm["span"]) / (r64["points"] / r64["span"])}
                         if sub else None,
                         "gpu_launches": None,
                         "detail": {"points": pts, "failed": r["failed"]}})
    line["clocks"] = clocks.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfg = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference(cfg, threads, steps=1)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_reference(cfg, threads, steps=2))
    v = statistics.median([x["value"] for x in vals])
    points = vals[0]["value"] * vals[0]["t_full_extrapolated"]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * points / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded star field)",
        "config": {"workload": args.workload, **cfg},
        "cpu_baseline": {"value": v, "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    ap.add_argument("--requests", type=int, default=64, help="serving: requests in the stream")
    ap.add_argument("--slots", type=int, default=4, help="serving: requests running at once")
    ap.add_argument("--hbm-budget", type=float, default=60e9, help="serving: admission budget in bytes")
    ap.add_argument("--fp64-requests", type=int, default=6, help="serving: requests replayed in plain FP64")
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

    # end to end through the public API: host star array in, host roots and caustics out
    res = c.results()
    stars_host = np.ascontiguousarray(res["stars"])
    corner = complex(info["corner_x1"], info["corner_x2"])
    e = make(args.precision)
    e.set_stars(stars_host, info["rectangular"], corner, info["theta_star"])
    rows = info["num_roots"] * cfg["num_branches"]
    cols = cfg["num_phi"] // cfg["num_branches"] + 1
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

    # roofline of the dominant kernel: the continuation solver launch
    peaks = measure_peaks()
    t_cont = statistics.median(i["t_ccs"] for i in infos)
    cont_share = t_cont / statistics.median(i["t_total"] for i in infos)
    evals_cont = info["root_updates"] - info["root_updates_init"]
    flops = evals_cont * tracker_flops_per_eval(info, cfg.get("approx", 1))
    achieved = flops / t_cont / 1e12 if t_cont > 0 else 0.0
    peak32 = peaks.get("fp32_tflops")
    traffic = CONT_DRAM_BYTES_PER_POINT * info["num_roots"] * cfg["num_phi"]
    hbm_peak = hbm_peak_gbs()

    fp64 = None
    if args.precision == "mixed" and args.fp64_steps > 0 and cfg["num_stars"] > 5000:
        # a plain-FP64 run of a field this large takes minutes: time both
        # precisions on the same field with 2 phi steps per side and apply
        # their ratio to the full mixed run
        red = dict(cfg, num_phi=4 * cfg["num_branches"])
        tm, td = [], []
        for prec, acc in (("mixed", tm), ("fp64", td)):
            c2 = CCF(**red)
            c2.precision, c2.device, c2.write_mu_length_scales = prec, local, 0
            for _ in range(1 + args.fp64_steps):
                flush.zero_()
                torch.cuda.synchronize()
                assert c2.run(-1), c2.last_error()
                acc.append(c2.info()["t_total"])
        ratio = statistics.median(td[1:]) / statistics.median(tm[1:])
        fp64 = {"value": value / ratio, "unit": "points/s", "ms_per_step": 1e3 * t_dev / args.steps * ratio,
                "extrapolated": f"fp64/mixed time ratio {ratio:.2f} measured on the same field with num_phi "
                                f"{red['num_phi']} (2 phi steps per side), applied to the full mixed run"}
    elif args.precision == "mixed" and args.fp64_steps > 0:
        d = make("fp64")
        assert d.run(-1), d.last_error()
        tt = []
        for _ in range(args.fp64_steps):
            flush.zero_()
            torch.cuda.synchronize()
            assert d.run(-1), d.last_error()
            tt.append(d.info()["t_total"])
        fp64 = {"value": points / statistics.median(tt), "unit": "points/s",
                "ms_per_step": 1e3 * statistics.median(tt)}

    # the reference's continuation scheme (full Aberth step for every root of a
    # row) on the same field and GPU, both precisions, for fields small enough
    # to run it in seconds
    full_sum = None
    if args.precision == "mixed" and args.fp64_steps > 0 and cfg["num_stars"] <= 5000:
        full_sum = {"unit": "points/s"}
        for prec in ("mixed", "fp64"):
            g = make(prec)
            g.continuation = "aberth"
            assert g.run(-1), g.last_error()
            tt = []
            for _ in range(args.fp64_steps):
                flush.zero_()
                torch.cuda.synchronize()
                assert g.run(-1), g.last_error()
                tt.append(g.info()["t_total"])
            full_sum[prec] = points / statistics.median(tt)
            full_sum[prec + "_ms_per_step"] = 1e3 * statistics.median(tt)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        # large fields: the initial solve and 2 phi steps of 4 branches
        cb = cpu_reference(cfg, threads, branches=4 if cfg["num_stars"] > 5000 else None, steps=2)
        cpu = {"value": cb["value"], "unit": "points/s", "cores": threads, "kind": "port", "sample": cb["sample"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+df32+f64 (double-float f and caustics, FP32 f' and step, FP64 coordinates)" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded star field)",
            "config": {"workload": args.workload, **cfg, "precision": args.precision,
                       "l2": "flushed before every timed step (256 MiB write)", "parallelism": f"replicas x{ws}"},
            "e2e": {"value": points * args.steps * ws / t_e2e, "unit": "points/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                         "frac": (achieved / peak32) if peak32 else None, "traffic": traffic,
                         "kernel": "track_kernel (phi continuation)", "kernel_share_of_step": cont_share,
                         "flops_per_evaluation": tracker_flops_per_eval(info, cfg.get("approx", 1)),
                         "evaluations": evals_cont,
                         "peak_source": "ccf_gb300/lib/ccf_peaks (FFMA chains, measured)",
                         "fp64_peak_tflops": peaks.get("fp64_tflops"),
                         "traffic_source": "per-point DRAM bytes of the ncu capture in "
                                           "profiles/track_kernel_n2000_salpeter_phi512.md, scaled by points",
                         "hbm_gbs": traffic / t_cont / 1e9 if t_cont > 0 else None,
                         "hbm_peak_gbs": hbm_peak, "hbm_frac": (traffic / t_cont / 1e9 / hbm_peak)
                         if (t_cont > 0 and hbm_peak) else None},
            "fp64_plain": fp64,
            "full_sum_continuation": full_sum,
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
