"""The solver and FMM settings beside the reference's parameters, and the
autotuner that picks them.

* expansion_order / leaf_max_stars: the far-field error of the built field
  (ccf_fmm_error: near sum and local expansion against the direct sum over
  every star, one point per leaf) stays within the reference's alpha_error =
  1e-7 theta_star at the orders the configurations name (20, 25) and at
  smaller leaves, with exact binomials (the reference's int32 table adds its
  own wrap-around error); the roots move by no more than that allows.
* init_cluster: the initial solve's CTAs per row change only the order of
  FP32 sums: the same zero sets.
* the autotuner returns valid settings, caches them per field shape, and a
  run with autotune set applies them.
* host_outputs: the same bits with the outputs in page-locked host memory.
"""
import os

import numpy as np
import pytest

import bench
from ccf_gb300 import CCF
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CFG1 = bench.WORKLOADS["single_field_n2000_salpeter_rect"]
ALPHA_ERROR = 1e-7   # theta_star = 1


def run(cfg, **kw):
    c = CCF(**cfg)
    c.write_mu_length_scales = 0
    for k, v in kw.items():
        setattr(c, k, v)
    assert c.run(-1), c.last_error()
    return c


@pytest.mark.parametrize("order", [20, 25])
def test_explicit_expansion_order_meets_alpha_error(order):
    c = run(CFG1, expansion_order=order, exact_binomials=1)
    info = c.info()
    assert info["expansion_order"] == order
    err = c.fmm_error()
    print(f"\norder {order}: far-field error {err:.3e}")
    assert err <= ALPHA_ERROR
    assert info["unconverged"] == 0 and info["points_above_target"] == 0


@pytest.mark.parametrize("leaf", [16, 24])
def test_smaller_leaves_meet_alpha_error(leaf):
    ref = run(CFG1, exact_binomials=1)
    c = run(CFG1, leaf_max_stars=leaf, exact_binomials=1)
    info = c.info()
    assert info["leaf_max_stars"] == leaf
    assert info["near_mean"] < ref.info()["near_mean"]
    assert info["tree_levels"] >= ref.info()["tree_levels"]
    err = c.fmm_error()
    print(f"\nleaf {leaf}: far-field error {err:.3e}, near stars {info['near_mean']:.2f}, levels {info['tree_levels']}")
    assert err <= ALPHA_ERROR
    # the roots move within what the far-field difference allows
    m = O.match_sets(c.results(stars=False)["ccs"], ref.results(stars=False)["ccs"], CFG1["num_branches"])
    assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-5, m


def test_default_fmm_error_is_the_references():
    """the reference's own order and wrapped binomial table: its far-field
    error, as the CPU known-answer test finds for the oracle (a few 1e-7)"""
    c = run(CFG1)
    err = c.fmm_error()
    print(f"\nreference order {c.info()['expansion_order']}, int32 binomials: far-field error {err:.3e}")
    assert err <= 1e-6


@pytest.mark.parametrize("cl", [2, 4, 16])
def test_initial_solve_cluster_sizes_give_the_same_zeros(cl):
    ref = run(CFG1)
    c = run(CFG1, init_cluster=cl)
    assert c.info()["init_cluster"] == cl
    m = O.match_sets(c.results(stars=False)["ccs"], ref.results(stars=False)["ccs"], CFG1["num_branches"])
    assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-11, m


def test_autotune_caches_and_applies(tmp_path, monkeypatch):
    cache = tmp_path / "autotune.txt"
    monkeypatch.setenv("CCF_GB300_AUTOTUNE_CACHE", str(cache))
    cfg = dict(CFG1, num_stars=600, num_phi=512, num_branches=16, random_seed=77)
    c = CCF(**cfg)
    c.write_mu_length_scales = 0
    tuned = c.tune(fmm=False)
    assert tuned["init_cluster"] in (0, 1, 2, 4, 8, 16)
    assert tuned["solved_centres"] == 0 or cfg["num_branches"] % tuned["solved_centres"] == 0
    assert tuned["leaf_max_stars"] == 0 and tuned["expansion_order"] == 0
    assert tuned["seconds"] > 0
    assert cache.exists() and "v1 " in cache.read_text()
    # a run with autotune set takes the cached settings of its shape
    d = CCF(**cfg)
    d.write_mu_length_scales = 0
    d.autotune = 1
    assert d.run(-1), d.last_error()
    info = d.info()
    if tuned["init_cluster"]:
        assert info["init_cluster"] == tuned["init_cluster"]
    if tuned["solved_centres"]:
        assert info["centres_solved"] == tuned["solved_centres"]
    # and its zeros are the default settings' zeros
    ref = run(cfg)
    m = O.match_sets(d.results(stars=False)["ccs"], ref.results(stars=False)["ccs"], cfg["num_branches"])
    assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-9, m


def test_host_outputs_are_the_same_bits_without_device_output_memory():
    """host_outputs: the kernels write the outputs into page-locked host
    memory mapped into the GPU; the results are bit for bit those of device
    outputs, the admission estimate drops by the outputs' bytes, and the
    library's output pointers read directly from the host."""
    import ctypes
    cfg = dict(CFG1, num_phi=512)
    a = run(cfg)
    b = run(cfg, host_outputs=1)
    ra, rb = a.results(stars=False), b.results(stars=False)
    for k in ("ccs", "caustics", "errs"):
        assert np.array_equal(ra[k], rb[k]), k
    assert b.estimate_device_bytes() < a.estimate_device_bytes()
    pts = ra["ccs"].size
    assert a.estimate_device_bytes() - b.estimate_device_bytes() == pts * 40
    # the output pointers of a host_outputs run address host memory
    ccs, caus, errs, mu = (ctypes.c_void_p() for _ in range(4))
    assert b._L.ccf_get_device_results(b._h, ctypes.byref(ccs), ctypes.byref(caus), ctypes.byref(errs),
                                       ctypes.byref(mu)) == 0
    host_errs = np.ctypeslib.as_array(ctypes.cast(errs.value, ctypes.POINTER(ctypes.c_double)), shape=(pts,))
    assert np.array_equal(host_errs.reshape(ra["errs"].shape), ra["errs"])


@pytest.mark.parametrize("continuation,centres", [("track", 4), ("aberth", 0)])
def test_streamed_outputs_are_the_same_bits(monkeypatch, continuation, centres):
    """host_outputs = 2: the continuation runs one group of solved centres at
    a time into two device chunk buffers that are copied to host memory while
    the next group computes.  With a small chunk target every centre is a
    group of its own; with 4 solved centres of 32 branches each group's
    window spans 9 branches, and the first one wraps around branch 0.  The
    results are bit for bit those of device outputs."""
    monkeypatch.setenv("CCF_GB300_CHUNK_BYTES", "1")
    cfg = dict(CFG1, num_stars=800, num_phi=512, random_seed=99)
    extra = dict(continuation=continuation, solved_centres=centres)
    a = run(cfg, **extra)
    b = run(cfg, host_outputs=2, **extra)
    ia, ib = a.info(), b.info()
    assert ib["centres_solved"] == ia["centres_solved"]
    assert ia["rows_rerun"] == 0 and ib["rows_rerun"] == 0
    ra, rb = a.results(stars=False), b.results(stars=False)
    for k in ("ccs", "caustics", "errs"):
        assert np.array_equal(ra[k], rb[k]), k
    assert ib["max_error"] == ia["max_error"] and ib["unconverged"] == ia["unconverged"]
