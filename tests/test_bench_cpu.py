"""Host logic of bench.py on the CPU: the algorithmic work behind the
roofline and the executed FP32 operation count beside it, the seeded batch
and serving workloads, and the clock record."""
import math

import bench

HEADLINE_INFO = dict(near_mean=15.68, expansion_order=23, rectangular=1, taylor_smooth=57, num_leaves=1225)


def test_smooth_series_charged_to_unfolded_leaves_only():
    none = bench.tracker_ops_per_eval(dict(HEADLINE_INFO, leaves_folded=0), approx=1)
    some = bench.tracker_ops_per_eval(dict(HEADLINE_INFO, leaves_folded=1061), approx=1)
    every = bench.tracker_ops_per_eval(dict(HEADLINE_INFO, leaves_folded=1225), approx=1)
    # the base evaluation (near stars, two double-float Horner passes, f' pass, assembly)
    base = 174.0 * 15.68 + 54.0 * (2 * 23 - 3) + 8.0 * 20 + 200.0
    assert math.isclose(every, base)
    assert none > some > every
    # the series part scales with the unfolded share of the leaves
    assert math.isclose(some - every, (none - every) * (1225 - 1061) / 1225)


def test_no_series_without_the_rectangular_taylor_form():
    disc = bench.tracker_ops_per_eval(dict(HEADLINE_INFO, rectangular=0, leaves_folded=0), approx=1)
    exact = bench.tracker_ops_per_eval(dict(HEADLINE_INFO, leaves_folded=0), approx=0)
    assert math.isclose(disc, exact)
    assert disc < bench.tracker_ops_per_eval(dict(HEADLINE_INFO, leaves_folded=0), approx=1)


def test_algorithmic_work_of_the_headline_field():
    # 40 per near star, 16 per expansion order, 12 per Taylor term on the unfolded share
    info = dict(HEADLINE_INFO, leaves_folded=1061)
    w = bench.algorithmic_flops_per_eval(info, approx=1)
    assert math.isclose(w, 40 * 15.68 + 16 * 23 + 12 * 56 * (1225 - 1061) / 1225)
    # the continuation's work adds 10 per reciprocal-sum term outside the initial solve
    full = dict(info, root_updates=1000, root_updates_init=400, sum_terms=5000, sum_terms_init=2000)
    assert math.isclose(bench.continuation_algorithmic_flops(full, 1), 10 * 3000 + w * 600)
    # the double-float emulation executes several FP32 operations per algorithmic flop
    assert bench.tracker_ops_per_eval(info, 1) / w > 5


def test_batch_fields_are_seeded_and_valid():
    a, b = bench.batch_fields(), bench.batch_fields()
    assert a == b and len(a) == 256
    for i, f in enumerate(a):
        assert f["random_seed"] == 10000 + i
        assert 50 <= f["num_stars"] <= 1000
        assert f["num_phi"] % (2 * f["num_branches"]) == 0   # the reference's validity rule
        assert not bench._singular(f["kappa_tot"], f["shear"])


def test_serving_requests_are_a_seeded_poisson_stream():
    reqs = bench.serving_requests(64)
    assert reqs == bench.serving_requests(64)
    times = [t for t, _ in reqs]
    assert all(t1 > t0 for t0, t1 in zip(times, times[1:]))
    assert 0.5 < times[-1] / 64 / 0.05 < 2.0     # mean inter-arrival ~50 ms
    for _, p in reqs:
        assert 100 <= p["num_stars"] <= 50000
        assert p["num_branches"] in (8, 32, 128)
        assert p["num_phi"] % (2 * p["num_branches"]) == 0
        assert 1000 <= p["num_phi"] <= 10000 + 2 * p["num_branches"]
        assert not bench._singular(p["kappa_tot"], p["shear"])


def test_clock_summary_parses_samples_and_reasons():
    c = bench.ClockSampler(0)
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "garbage",
    ]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_max_mhz"] == 2070.0
    assert s["sm_mhz"] == (2070.0 + 1980.0) / 2
    assert s["reasons"] == ["sw_power_cap"]
    assert bench.ClockSampler(0).summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_continuation_roofline_record():
    """the bench's roofline record for the headline field's counts: the §8(d)
    algorithmic work over the continuation's span against the FP32 peak, the
    FP64 share beside it, the executed double-float operations per flop and
    the DRAM bytes scaled from the full-size capture"""
    info = dict(HEADLINE_INFO, leaves_folded=1061, num_roots=4056, root_updates=10206621, root_updates_init=641077,
                sum_terms=3095830675, sum_terms_init=3095830675)
    peaks = {"fp32_tflops": 78.477, "fp64_tflops": 1.2545}
    r = bench.continuation_roofline(info, 1, 0.00891, peaks, 2048)
    assert r["bound"] == "fp32" and r["unit"] == "TFLOP/s" and r["peak"] == 78.477
    evals = 10206621 - 641077
    flops = bench.algorithmic_flops_per_eval(info, 1) * evals
    assert math.isclose(r["achieved"], flops / 0.00891 / 1e12)
    assert math.isclose(r["frac"], r["achieved"] / 78.477)
    assert math.isclose(r["frac_of_fp64_peak"], r["achieved"] / 1.2545)
    assert 1.0 < r["achieved"] < 1.3
    assert 5.0 < r["executed_ops"]["per_algorithmic_flop"] < 6.0
    assert math.isclose(r["traffic"], bench.CONT_DRAM_BYTES_PER_POINT * 4056 * 2048)
