"""Parity at the benchmarked sizes: the CUDA path through the C ABI against
the oracle run on the same seeded fields, every column of the compared
branches matched as a set.

    single field  2000 Salpeter stars, rectangular, num_phi 2048, 32 branches:
                  every column of every branch (8.4e6 points)
    large field   20000 Kroupa stars, rectangular, num_phi 10240, 128
                  branches: two complete branches, both sides and all 40
                  steps of each -- branch 0 (a solved centre) and branch 8,
                  whose columns come from the tracked rows of two solved
                  centres (0 and 16, 16 branches apart)
    batch         8 of the 256 disc fields of the batch workload, run inside
                  the whole batch, every column

The oracle restates the reference's FP64 algorithm (include/ccf_functions.cuh,
include/ccf.cuh:979-1083) and is polished to convergence: every point takes
FP64 Newton steps on the oracle's own f until its step is below 1e-13
theta_star (the reference stops after fixed sweep counts, so its raw roots sit
up to ~1e-8 from the converged zeros).  The large field's oracle rows run in
the Jacobi order with the roots split over the host cores.  Bars:

    roots, caustics        <= 1e-9 theta_star, one-to-one per column
    1/mu error             <= 1e-9, or |f| at the point within four times
                           |f'| times half the FP64 spacing of the root (the
                           FP64 floor: no FP64 root does better), checked with
                           the library's own FP64 evaluation of f and f'
    unconverged points     none after the FP64 polish

The measured maxima are printed (run with -s to see them).
"""
import os

import numpy as np
import pytest

import bench
from ccf_gb300 import CCF, run_batch
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-9
THREADS = os.cpu_count() or 8
POLISH = dict(polish_tol=1e-13, polish_max_iters=20, polish_newton=1)


def gpu_run(cfg, precision="mixed"):
    c = CCF(**cfg)
    c.precision = precision
    c.write_mu_length_scales = 0
    assert c.run(-1), c.last_error()
    return c, c.results(stars=False)


def phases(cfg, rows, cols):
    nb = cfg["num_branches"]
    half = cfg["num_phi"] // (2 * nb)
    return np.pi / nb + (rows % nb) * 2 * np.pi / nb + (cols - half) * 2 * np.pi / cfg["num_phi"]


def check_errs(c, cfg, r):
    """every 1/mu error within 1e-9, or |f| at the FP64 floor of the root"""
    info = r["info"]
    assert info["unconverged"] == 0 and info["has_nan"] == 0
    assert info["points_above_target"] == 0
    errs = r["errs"]
    assert np.all(np.isfinite(errs)) and np.all(errs >= 0)
    rows, cols = np.nonzero(errs > TOL)
    if rows.size:
        z = r["ccs"][rows, cols]
        e = c.eval_points(z, phases(cfg, rows, cols))
        floor = 0.5 * np.hypot(np.spacing(np.abs(z.real)), np.spacing(np.abs(z.imag))) * np.abs(e["df"])
        assert np.all(np.abs(e["f"]) <= 4 * floor)
    return int(rows.size), float(errs.max())


def check_columns(name, a, b, wa, wb, theta):
    """a, b: (roots, cols) of one branch; wa, wb: their caustics"""
    m = O.match_sets(a, b, 1)
    assert m["non_finite"] == 0 and m["non_bijective_cols"] == 0, (name, m)
    assert m["max_dist"] <= TOL * theta, (name, m)
    idx, _ = O.match_index(a, b, 1)
    dw = float(np.max(np.abs(wa - O.take_matched(wb, idx))))
    assert dw <= TOL * theta, (name, dw)
    return m["max_dist"], dw


def test_single_field_every_column():
    cfg = bench.WORKLOADS["single_field_n2000_salpeter_rect"]
    c, r = gpu_run(cfg)
    ref = O.run(num_threads=THREADS, **POLISH, **cfg)
    theta = cfg["theta_star"]
    m = O.match_sets(r["ccs"], ref["ccs"], cfg["num_branches"])
    assert m["non_finite"] == 0 and m["non_bijective_cols"] == 0 and m["max_dist"] <= TOL * theta, m
    idx, _ = O.match_index(r["ccs"], ref["ccs"], cfg["num_branches"])
    dw = float(np.max(np.abs(r["caustics"] - O.take_matched(ref["caustics"], idx))))
    assert dw <= TOL * theta, dw
    n_hi, emax = check_errs(c, cfg, r)
    print(f"\nsingle field: {r['ccs'].size} points, max root displacement {m['max_dist']:.3e}, caustic {dw:.3e}, "
          f"max 1/mu {emax:.3e} ({n_hi} points above 1e-9, all at the FP64 floor)")


def test_single_field_precisions_agree():
    """mixed and plain FP64 on the 2000-star field: the same zero sets"""
    cfg = bench.WORKLOADS["single_field_n2000_salpeter_rect"]
    _, a = gpu_run(cfg, "mixed")
    _, b = gpu_run(cfg, "fp64")
    m = O.match_sets(a["ccs"], b["ccs"], cfg["num_branches"])
    assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-11, m
    print(f"\nmixed vs FP64, 2000 stars: max root displacement {m['max_dist']:.3e}")


def test_large_field_two_complete_branches():
    cfg = bench.WORKLOADS["large_field_n20000_kroupa_rect"]
    nb = cfg["num_branches"]
    c, r = gpu_run(cfg)
    assert r["info"]["centres_solved"] < nb   # the tracked rows span several branches
    branches = [0, 8]
    ref = O.run(num_threads=THREADS, max_branches=2, first_branch=0, branch_stride=8, jacobi=1, **POLISH, **cfg)
    out = []
    for b in branches:
        out.append(check_columns(f"branch {b}", r["ccs"][b::nb], ref["ccs"][b::nb], r["caustics"][b::nb],
                                 ref["caustics"][b::nb], cfg["theta_star"]))
    n_hi, emax = check_errs(c, cfg, r)
    print(f"\nlarge field, branches {branches}: max root displacement {max(o[0] for o in out):.3e}, "
          f"caustic {max(o[1] for o in out):.3e}; whole field: max 1/mu {emax:.3e} "
          f"({n_hi} points above 1e-9, all at the FP64 floor)")


def test_batch_fields_every_column():
    cfgs = bench.batch_fields()
    fields = []
    for cfg in cfgs:
        f = CCF(**cfg)
        f.write_mu_length_scales = 0
        fields.append(f)
    assert run_batch(fields, -1)
    worst = [0.0, 0.0, 0.0]
    for i in np.linspace(0, len(cfgs) - 1, 8).astype(int):
        cfg, c = cfgs[i], fields[i]
        r = c.results(stars=False)
        ref = O.run(num_threads=THREADS, **POLISH, **cfg)
        nb = cfg["num_branches"]
        for b in range(nb):
            d, dw = check_columns(f"field {i} branch {b}", r["ccs"][b::nb], ref["ccs"][b::nb], r["caustics"][b::nb],
                                  ref["caustics"][b::nb], cfg["theta_star"])
            worst[0] = max(worst[0], d)
            worst[1] = max(worst[1], dw)
        worst[2] = max(worst[2], check_errs(c, cfg, r)[1])
    print(f"\nbatch, 8 of 256 fields: max root displacement {worst[0]:.3e}, caustic {worst[1]:.3e}, "
          f"max 1/mu {worst[2]:.3e}")
