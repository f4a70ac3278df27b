"""The batched setup (one CTA per field for stars, tree, FMM passes and leaf
records, a few launches for the whole batch) against the per-field setup of
the same fields run one by one: the same stars in the same tree order, the
same tree, expansion order and leaf records (the far-field error of each
field's FMM, a function of every expansion coefficient, is bit for bit the
same), and the same roots.  A field too large for the one-CTA build in the
batch takes the per-field path beside the others."""
import glob
import json
import os

import numpy as np
import pytest

from ccf_gb300 import CCF, run_batch
from oracle import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))

pytestmark = pytest.mark.gpu

SAME_INFO = ("num_stars", "num_roots", "tree_levels", "num_nodes", "num_leaves", "expansion_order", "near_mean",
             "leaves_folded", "kappa_star_actual", "mean_mass_actual", "corner_x1", "corner_x2", "leaf_max_stars")


def disc_field(n, seed):
    return dict(kappa_tot=0.4, kappa_star=0.35, shear=0.2, theta_star=1.0, mass_function="equal", rectangular=0, approx=1,
                num_stars=n, num_phi=64, num_branches=4, random_seed=seed)


def make(cfg, precision):
    c = CCF(**cfg)
    c.precision = precision
    c.write_mu_length_scales = 0
    return c


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_setup_is_the_per_field_setup(precision):
    cfgs = [json.loads(str(np.load(p)["params"])) for p in GOLDEN]
    cfgs += [disc_field(n, 500 + n) for n in (50, 333, 1000)]
    # one field beyond the one-CTA build's star bound runs the per-field path inside the batch
    cfgs.append(dict(disc_field(9000, 77), num_phi=16, num_branches=2))
    solo = []
    for cfg in cfgs:
        c = make(cfg, precision)
        assert c.run(-1), c.last_error()
        solo.append((c.info(), c.results(), c.fmm_error()))
    fields = [make(cfg, precision) for cfg in cfgs]
    assert run_batch(fields, -1), fields[0].last_error()
    for cfg, f, (si, sr, se) in zip(cfgs, fields, solo):
        bi, br = f.info(), f.results()
        for k in SAME_INFO:
            assert bi[k] == si[k], (cfg.get("num_stars"), k, bi[k], si[k])
        assert np.array_equal(br["stars"], sr["stars"]), cfg.get("num_stars")
        assert f.fmm_error() == se, cfg.get("num_stars")
        # the solver's launches split sweeps by the CTAs per row, which differ
        # between a batch and a solo run: FP32 summation order changes the last
        # bits of the roots, and in a large field can hand two roots each
        # other's zero (the columns are sets)
        nb = cfg["num_branches"]
        m = O.match_sets(br["ccs"], sr["ccs"], nb)
        assert m["non_bijective_cols"] == 0 and m["max_dist"] <= 1e-11, (cfg.get("num_stars"), m)
        mc = O.match_sets(br["caustics"], sr["caustics"], nb)
        assert mc["max_dist"] <= 1e-10, (cfg.get("num_stars"), mc)


def test_batched_setup_launches():
    """a batch of small fields: the setup's launches for the whole batch,
    counted with its first field"""
    fields = [make(disc_field(n, 900 + n), "mixed") for n in (60, 200, 450, 700, 950)]
    assert run_batch(fields, -1), fields[0].last_error()
    launches = [f.info()["kernel_launches"] for f in fields]
    solo = make(disc_field(450, 1350), "mixed")
    assert solo.run(-1), solo.last_error()
    # the solver's launches are shared by the batch too
    assert sum(launches) < solo.info()["kernel_launches"] + 10, launches


_CHILD = """
import json, sys
import numpy as np
from ccf_gb300 import CCF
out = {}
for k, cfg in enumerate(json.loads(sys.argv[1])):
    c = CCF(**cfg)
    c.write_mu_length_scales = 0
    assert c.run(-1), c.last_error()
    info = c.info()
    out[f"info{k}"] = np.array([info[n] for n in json.loads(sys.argv[3])], dtype=np.float64)
    out[f"stars{k}"] = c.results()["stars"]
    out[f"fmm{k}"] = np.array([c.fmm_error()])
np.savez(sys.argv[2], **out)
"""


def test_one_cta_tree_is_the_per_level_tree(tmp_path):
    """a field of up to 8192 stars builds its tree in one CTA; the per-level
    launches (kept for larger fields, and forced by CCF_GB300_TREE_LEVELS=1
    in a child process) give the same tree: stars in the same order, the same
    levels, nodes and leaves, and the same far-field error"""
    import subprocess
    import sys
    cfgs = [json.loads(str(np.load(GOLDEN[0])["params"])), disc_field(1000, 4242),
            dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, theta_star=1.0, mass_function="salpeter", m_lower=0.08,
                 m_upper=1.5, m_solar=4.954984, rectangular=1, approx=1, num_stars=2000, num_phi=64, num_branches=32,
                 random_seed=1235)]
    keys = list(SAME_INFO)
    env = dict(os.environ, CCF_GB300_TREE_LEVELS="1")
    out = tmp_path / "levels.npz"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _CHILD, json.dumps(cfgs), str(out), json.dumps(keys)], env=env, cwd=root,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lv = np.load(out)
    for k, cfg in enumerate(cfgs):
        c = make(cfg, "mixed")
        assert c.run(-1), c.last_error()
        info = c.info()
        assert np.array_equal(np.array([info[n] for n in keys], dtype=np.float64), lv[f"info{k}"]), cfg["num_stars"]
        assert np.array_equal(c.results()["stars"], lv[f"stars{k}"]), cfg["num_stars"]
        assert c.fmm_error() == lv[f"fmm{k}"][0], cfg["num_stars"]
