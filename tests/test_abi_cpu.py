"""CPU checks of the native library: it loads, exports every symbol that
include/*.h declares, fills the reference's defaults, and derives the
reference's parameters on the host.  No compute call needs a GPU here."""
import ctypes
import glob
import os
import re

import pytest

from ccf_gb300 import _lib
from ccf_gb300.ccf import CCF, derive_params
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        for m in re.finditer(r"^\s*(?:ccf_status|int|void|const char\*)\s+(ccf_\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.EXPORTED)
    assert L.ccf_abi_version() == 2


def test_default_params_are_the_reference_defaults():
    L = _lib.load()
    p = _lib.CcfParams()
    L.ccf_default_params(ctypes.byref(p))
    # include/ccf.cuh:42-62
    assert (p.kappa_tot, p.shear, p.kappa_star, p.theta_star) == (0.3, 0.3, 0.27, 1.0)
    assert p.mass_function == b"equal"
    assert (p.m_solar, p.m_lower, p.m_upper, p.safety_scale) == (1.0, 0.01, 50.0, 1.37)
    assert (p.rectangular, p.approx, p.num_stars, p.num_phi, p.num_branches, p.random_seed) == (0, 1, 137, 100, 1, 0)
    assert (p.write_stars, p.write_critical_curves, p.write_caustics, p.write_mu_length_scales) == (1, 1, 1, 0)
    assert p.outfile_prefix == b"./"
    c = CCF()
    assert c.kappa_star == 0.27 and c.mass_function_str == "equal" and c.num_stars == 137


CASES = [
    dict(kappa_tot=0.3, kappa_star=0.3, shear=0.1, mass_function="equal", rectangular=0, num_stars=100,
         num_phi=100, num_branches=1),
    dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, mass_function="salpeter", m_lower=0.08, m_upper=1.5,
         m_solar=4.954984, rectangular=1, approx=1, num_stars=2000, num_phi=2048, num_branches=32),
    dict(kappa_tot=0.7, kappa_star=0.6, shear=0.2, mass_function="kroupa", m_lower=0.08, m_upper=1.5, m_solar=1,
         rectangular=1, approx=1, num_stars=20000, num_phi=10240, num_branches=128),
    dict(kappa_tot=0.2, kappa_star=0.15, shear=0.5, mass_function="kroupa", m_lower=0.01, m_upper=50,
         rectangular=0, approx=0, num_stars=70, num_phi=24, num_branches=3, theta_star=1.7),
    dict(kappa_tot=0.5, kappa_star=0.4, shear=0.25, mass_function="uniform", m_lower=0.1, m_upper=2,
         rectangular=1, approx=0, num_stars=40, num_phi=16, num_branches=2),
    dict(kappa_tot=0.4, kappa_star=0.4, shear=0.3, mass_function="optical_depth", m_lower=0.3, m_upper=1.2,
         rectangular=0, num_stars=45, num_phi=16, num_branches=2, safety_scale=2.0),
]


@pytest.mark.parametrize("cfg", CASES)
def test_derived_params_match_oracle(cfg):
    a = derive_params(**cfg)
    b = O.derive(**cfg)
    assert a["rc"] == 0 and b["rc"] == 0
    assert a["num_roots"] == b["num_roots"]
    assert a["taylor_smooth"] == b["taylor_smooth"]
    assert a["corner_x1"] == pytest.approx(b["corner_re"], rel=1e-15)
    assert a["corner_x2"] == pytest.approx(b["corner_im"], rel=1e-15)
    assert a["mu_ave"] == pytest.approx(b["mu_ave"], rel=1e-15)
    for k in ("mean_mass", "mean_mass2", "mean_mass2_ln_mass", "m_lower", "m_upper"):
        assert a[k] == pytest.approx(b[k], rel=1e-12, abs=1e-300), k


@pytest.mark.parametrize("bad,msg", [
    (dict(num_phi=101), "num_phi must be an even integer"),
    (dict(num_phi=100, num_branches=3), "multiple of 2 * num_branches"),
    (dict(kappa_star=0.5, kappa_tot=0.3), "kappa_star must be <= kappa_tot"),
    (dict(mass_function="bogus"), "mass_function must be"),
    (dict(safety_scale=1.05), "safety_scale must be >= 1.1"),
    (dict(num_stars=0), "num_stars must be an integer > 0"),
    (dict(approx=2), "approx must be 1"),
    (dict(rectangular=3), "rectangular must be 1"),
    (dict(m_lower=2.0, m_upper=1.0), "m_upper must be >= m_lower"),
])
def test_invalid_inputs_are_rejected_with_the_reference_message(bad, msg):
    d = derive_params(**bad)
    assert d["rc"] == 1
    assert msg in d["error"]
    o = O.derive(**bad)
    assert o["rc"] != 0


def test_star_file_errors(tmp_path):
    p = tmp_path / "stars.bin"
    p.write_bytes(b"\x05\x00\x00\x00\x00\x00\x00\x00" + b"\x00" * 17)   # wrong size for 5 stars
    d = derive_params(starfile=str(p))
    assert d["rc"] == 5 and "validly formatted" in d["error"]
    q = tmp_path / "stars.dat"
    q.write_text("1 2 3\n")
    assert derive_params(starfile=str(q))["rc"] == 5


def test_txt_star_file_rectangle_vs_disc_rule(tmp_path):
    import numpy as np
    rng = np.random.default_rng(1)
    xy = rng.uniform(-5, 5, size=(400, 2))
    f = tmp_path / "rect.txt"
    f.write_text("\n".join(f"{x} {y} 1.0" for x, y in xy))
    d = derive_params(starfile=str(f))
    assert d["rc"] == 0 and d["rectangular"] == 1 and d["num_stars"] == 400
    r = np.sqrt(rng.uniform(0, 1, 400)) * 5
    a = rng.uniform(0, 2 * np.pi, 400)
    g = tmp_path / "disc.txt"
    g.write_text("\n".join(f"{x} {y} 1.0" for x, y in zip(r * np.cos(a), r * np.sin(a))))
    d = derive_params(starfile=str(g))
    assert d["rc"] == 0 and d["rectangular"] == 0


def test_run_without_a_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = CCF(num_stars=10, num_phi=4)
    assert not c.run(-1)
    assert c.last_status == 3 and "No CUDA capable devices" in c.last_error()


def test_continuation_parameter():
    """Default: per-root tracking; 1 selects the full Aberth continuation;
    anything else is refused on the host."""
    L = _lib.load()
    p = _lib.CcfParams()
    L.ccf_default_params(ctypes.byref(p))
    assert p.continuation == _lib.CONTINUATION_TRACK
    info = _lib.CcfInfo()
    msg = ctypes.create_string_buffer(512)
    for v, ok in ((0, True), (1, True), (2, False), (-1, False)):
        p.continuation = v
        rc = L.ccf_derive_params(ctypes.byref(p), ctypes.byref(info), msg, 512)
        assert (rc == 0) == ok, (v, msg.value)
        if not ok:
            assert b"continuation must be 0 (track) or 1 (aberth)" in msg.value
    assert derive_params(continuation="aberth")["rc"] == 0
    with pytest.raises(ValueError):
        derive_params(continuation="newton")
    # solved centres: 0 (automatic) or a divisor of num_branches
    assert derive_params(num_phi=64, num_branches=8, solved_centres=2)["rc"] == 0
    d = derive_params(num_phi=64, num_branches=8, solved_centres=3)
    assert d["rc"] != 0 and "solved_centres must be 0 or a divisor of num_branches" in d["error"]


def test_pinned_host_memory_needs_a_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("checks the path without a GPU")
    except ImportError:
        pass
    from ccf_gb300 import CCFError, pinned_empty
    with pytest.raises(CCFError):
        pinned_empty((4, 4))


@pytest.mark.parametrize("knob,good,bad,msg", [
    ("expansion_order", (0, 3, 20, 31), (1, 2, 32), "expansion_order must be 0"),
    ("leaf_max_stars", (0, 4, 16, 32), (1, 3, 33), "leaf_max_stars must be 0"),
    ("init_cluster", (0, 1, 2, 4, 8, 16), (3, 5, 32, -1), "init_cluster must be 0"),
    ("autotune", (0, 1, 2), (3, -1), "autotune must be 0, 1 or 2"),
])
def test_solver_and_fmm_settings_are_checked(knob, good, bad, msg):
    """Settings beside the reference's parameters: 0 keeps the reference's
    choice (its expansion-order formula, its 32-star leaves) or the
    library's; other values are range-checked on the host."""
    for v in good:
        assert derive_params(**{knob: v})["rc"] == 0, (knob, v)
    for v in bad:
        d = derive_params(**{knob: v})
        assert d["rc"] != 0 and msg in d["error"], (knob, v, d["error"])
