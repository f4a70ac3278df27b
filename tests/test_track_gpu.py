"""The two continuations on the GPU: per-root tracking (the default) and the
full Aberth step of the reference.

Both converge every root of a phi column to a zero of f to ~1e-13, so their
root sets agree per column well inside the 1e-9 theta_star tolerance.  A
tracked row that fails its column check is run again by the full-sum
continuation from the same branch-centre roots; with a cap of one
evaluation per phi step every tracked root is lost, every row is re-run,
and the results are the full-sum continuation's to the bit.
"""
import glob
import json
import os

import numpy as np
import pytest

from ccf_gb300 import CCF
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def run(cfg, continuation, **extra):
    c = CCF(**cfg)
    c.write_mu_length_scales = 0
    c.continuation = continuation
    for k, v in extra.items():
        setattr(c, k, v)
    assert c.run(-1), c.last_error()
    return c.results()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_tracking_finds_the_full_sum_zero_sets(path, precision):
    cfg = json.loads(str(np.load(path)["params"]))
    t = run(cfg, "track", precision=precision)
    a = run(cfg, "aberth", precision=precision)
    nb = cfg["num_branches"]
    assert t["info"]["unconverged"] == 0 and t["info"]["has_nan"] == 0
    if cfg.get("approx", 1) == 0:
        # exact smooth-mass forms: f jumps at the field edge, the zero set
        # reached there depends on the path (see test_gpu_parity); every
        # tracked root must still be a converged zero
        half = cfg["num_phi"] // (2 * nb)
        row, col = np.indices(t["ccs"].shape)
        phi = np.pi / nb + (row % nb) * 2 * np.pi / nb + (col - half) * 2 * np.pi / cfg["num_phi"]
        o = O.eval_field(t["ccs"].ravel(), phi.ravel(), **cfg)
        assert np.max(np.abs(o["f"])) < 1e-9
        return
    m = O.match_sets(t["ccs"], a["ccs"], nb)
    assert m["non_finite"] == 0 and m["non_bijective_cols"] == 0
    assert m["max_dist"] <= 1e-11 * cfg.get("theta_star", 1.0)
    mc = O.match_sets(t["caustics"], a["caustics"], nb)
    assert mc["max_dist"] <= 1e-10 * cfg.get("theta_star", 1.0)
    assert np.max(t["errs"]) <= 1e-9


def test_rows_that_fail_the_check_are_the_full_sum_rows():
    cfg = json.loads(str(np.load([p for p in GOLDEN if "exact" not in p][0])["params"]))
    t = run(cfg, "track", max_iters_step=1)
    a = run(cfg, "aberth", max_iters_step=1)
    assert t["info"]["rows_rerun"] == 2 * cfg["num_branches"]
    assert np.array_equal(t["ccs"], a["ccs"], equal_nan=True)
    assert np.array_equal(t["errs"], a["errs"], equal_nan=True)
    assert t["info"]["unconverged"] == a["info"]["unconverged"]


def test_tracked_field_is_checked_and_deterministic():
    cfg = dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, mass_function="salpeter", m_lower=0.08, m_upper=1.5,
               m_solar=4.954984, rectangular=1, approx=1, num_stars=500, num_phi=512, num_branches=8,
               random_seed=77)
    x = run(cfg, "track")
    y = run(cfg, "track")
    assert np.array_equal(x["ccs"], y["ccs"])
    info = x["info"]
    # almost every row passes the check; the others are full-sum rows
    assert info["rows_rerun"] <= 2 and info["unconverged"] == 0, (info["rows_rerun"], info["rerun_flags"])
    # per phi step the corrector needs a few evaluations per root
    R, nb, half = info["num_roots"], cfg["num_branches"], cfg["num_phi"] // (2 * cfg["num_branches"])
    cont = info["root_updates"] - info["root_updates_init"]
    assert 1.0 <= cont / (R * 2 * nb * half) < 4.0
    a = run(cfg, "aberth")
    m = O.match_sets(x["ccs"], a["ccs"], nb)
    assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-11


def test_results_into_pinned_buffers():
    from ccf_gb300 import pinned_empty
    cfg = json.loads(str(np.load(GOLDEN[0])["params"]))
    c = CCF(**cfg)
    c.write_mu_length_scales = 0
    assert c.run(-1), c.last_error()
    a = c.results(stars=False)
    bufs = c.result_buffers(pinned=True)
    b = c.results(stars=False, out=bufs)
    assert b["ccs"] is bufs["ccs"]
    for k in ("ccs", "caustics", "errs"):
        assert np.array_equal(a[k], b[k])
    with pytest.raises(ValueError):
        c.results(stars=False, out={"ccs": np.empty((3, 3), dtype=np.complex128)})
    p = pinned_empty((5, 7), np.complex128)
    assert p.shape == (5, 7) and p.dtype == np.complex128


@pytest.mark.parametrize("centres", [1, 2])
def test_rows_across_branches_from_few_solved_centres(centres):
    """Solving the initial roots at 1 or 2 of 4 branch centres and tracking the
    others gives the zero sets of the full-sum continuation at every column."""
    cfg = dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, mass_function="salpeter", m_lower=0.08, m_upper=1.5,
               m_solar=4.954984, rectangular=1, approx=1, num_stars=300, num_phi=128, num_branches=4,
               random_seed=91)
    t = run(cfg, "track", solved_centres=centres)
    a = run(cfg, "aberth")
    assert t["info"]["centres_solved"] == centres
    assert t["info"]["unconverged"] == 0
    m = O.match_sets(t["ccs"], a["ccs"], cfg["num_branches"])
    assert m["non_finite"] == 0 and m["non_bijective_cols"] == 0
    assert m["max_dist"] <= 1e-11
    mc = O.match_sets(t["caustics"], a["caustics"], cfg["num_branches"])
    assert mc["max_dist"] <= 1e-10
