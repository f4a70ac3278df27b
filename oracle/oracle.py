"""CPU oracle bindings -- TEST INFRASTRUCTURE ONLY.

ctypes front end of ``oracle/ccf_oracle.cpp``, the FP64 CPU restatement of
the reference critical-curve / caustic algorithm (weisluke/ccf).  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module, and only as the checker; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libccf_oracle.so")
REF_HOST = os.path.join(HERE, "_ref", "ccf_ref_host")

MASS_FUNCTIONS = {"equal": 0, "uniform": 1, "salpeter": 2, "kroupa": 3, "optical_depth": 4}


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("kappa_tot", ctypes.c_double),
        ("shear", ctypes.c_double),
        ("kappa_star", ctypes.c_double),
        ("theta_star", ctypes.c_double),
        ("m_solar", ctypes.c_double),
        ("m_lower", ctypes.c_double),
        ("m_upper", ctypes.c_double),
        ("safety_scale", ctypes.c_double),
        ("mass_function", ctypes.c_int),
        ("rectangular", ctypes.c_int),
        ("approx", ctypes.c_int),
        ("num_stars", ctypes.c_int),
        ("num_phi", ctypes.c_int),
        ("num_branches", ctypes.c_int),
        ("random_seed", ctypes.c_int),
        ("write_mu_length_scales", ctypes.c_int),
        ("stars_in", ctypes.POINTER(ctypes.c_double)),
        ("stars_in_rectangular", ctypes.c_int),
        ("stars_in_corner_re", ctypes.c_double),
        ("stars_in_corner_im", ctypes.c_double),
        ("stars_in_theta", ctypes.c_double),
        ("num_threads", ctypes.c_int),
        ("init_iters", ctypes.c_int),
        ("step_iters", ctypes.c_int),
        ("early_out", ctypes.c_int),
        ("polish_tol", ctypes.c_double),
        ("polish_max_iters", ctypes.c_int),
        ("exact_binomials", ctypes.c_int),
        ("max_steps", ctypes.c_int),
        ("max_branches", ctypes.c_int),
        ("first_branch", ctypes.c_int),
        ("branch_stride", ctypes.c_int),
        ("polish_newton", ctypes.c_int),
        ("jacobi", ctypes.c_int),
        ("seed_curves", ctypes.c_int),
    ]


class OracleInfo(ctypes.Structure):
    _fields_ = [
        ("num_stars", ctypes.c_int),
        ("num_roots", ctypes.c_int),
        ("taylor_smooth", ctypes.c_int),
        ("tree_levels", ctypes.c_int),
        ("expansion_order", ctypes.c_int),
        ("num_nodes", ctypes.c_int),
        ("rectangular", ctypes.c_int),
        ("random_seed", ctypes.c_int),
        ("corner_re", ctypes.c_double),
        ("corner_im", ctypes.c_double),
        ("theta_star", ctypes.c_double),
        ("kappa_star", ctypes.c_double),
        ("mu_ave", ctypes.c_double),
        ("alpha_error", ctypes.c_double),
        ("root_half_length", ctypes.c_double),
        ("mean_mass", ctypes.c_double),
        ("mean_mass2", ctypes.c_double),
        ("mean_mass2_ln_mass", ctypes.c_double),
        ("kappa_star_actual", ctypes.c_double),
        ("m_lower_actual", ctypes.c_double),
        ("m_upper_actual", ctypes.c_double),
        ("mean_mass_actual", ctypes.c_double),
        ("mean_mass2_actual", ctypes.c_double),
        ("mean_mass2_ln_mass_actual", ctypes.c_double),
        ("m_lower", ctypes.c_double),
        ("m_upper", ctypes.c_double),
        ("max_error", ctypes.c_double),
        ("has_nan", ctypes.c_int),
        ("root_updates", ctypes.c_longlong),
        ("root_terms", ctypes.c_longlong),
        ("t_stars", ctypes.c_double),
        ("t_tree", ctypes.c_double),
        ("t_init_roots", ctypes.c_double),
        ("t_ccs", ctypes.c_double),
        ("t_caustics", ctypes.c_double),
        ("error", ctypes.c_char * 256),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.decode() if isinstance(v, bytes) else v
        return out


_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the oracle library with the committed Makefile (g++ only)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def build_reference() -> str | None:
    """Compile the reference's own code for the host, if its sources exist here."""
    # the reference checkout sits beside the repository unless CCF_REFERENCE_DIR says otherwise
    ref_dir = os.environ.get("CCF_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
    if not os.path.isdir(os.path.join(ref_dir, "include")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE_DIR={ref_dir}"], check=True)
    return REF_HOST


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P, I = ctypes.POINTER(OracleParams), ctypes.POINTER(OracleInfo)
            dp = ctypes.POINTER(ctypes.c_double)
            L.oracle_default_params.argtypes = [P]
            L.oracle_derive.argtypes = [P, I]
            L.oracle_run.argtypes = [P, I, dp, dp, dp, dp, dp]
            L.oracle_eval.argtypes = [P, I, ctypes.c_int, dp, dp, dp, dp, dp, dp]
            L.oracle_match_sets.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                                            ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
            _lib = L
        return _lib


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(stars=None, **kw) -> tuple[OracleParams, object]:
    """Build oracle parameters from reference-style field names.

    ``stars`` is an optional dict {"stars": (N,3) array, "rectangular",
    "corner": complex, "theta_star"} describing an exchanged star field.
    Returns the structure and the array that must stay alive with it."""
    p = OracleParams()
    lib().oracle_default_params(ctypes.byref(p))
    keep = None
    for k, v in kw.items():
        if k == "mass_function":
            v = MASS_FUNCTIONS.get(str(v).lower(), -1)
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    if stars is not None:
        arr = np.ascontiguousarray(stars["stars"], dtype=np.float64).reshape(-1, 3)
        keep = arr
        p.stars_in = _dp(arr)
        p.num_stars = arr.shape[0]
        p.stars_in_rectangular = int(stars["rectangular"])
        c = complex(stars["corner"])
        p.stars_in_corner_re = c.real
        p.stars_in_corner_im = c.imag
        p.stars_in_theta = float(stars["theta_star"])
    return p, keep


def derive(**kw) -> dict:
    p, keep = make_params(**kw)
    info = OracleInfo()
    rc = lib().oracle_derive(ctypes.byref(p), ctypes.byref(info))
    d = info.as_dict()
    d["rc"] = rc
    return d


def run(stars=None, want_mu=False, **kw) -> dict:
    """Full oracle pipeline; arrays come back in the reference's file layout."""
    p, keep = make_params(stars=stars, **kw)
    if want_mu:
        p.write_mu_length_scales = 1
    info = OracleInfo()
    d = derive(stars=stars, **kw)
    if d["rc"] != 0:
        raise ValueError(d["error"])
    n, R, nb, nphi = d["num_stars"], d["num_roots"], p.num_branches, p.num_phi
    rows, cols = R * nb, nphi // nb + 1
    stars_out = np.zeros((n, 3))
    ccs = np.zeros((rows, cols), dtype=np.complex128)
    caus = np.zeros((rows, cols), dtype=np.complex128)
    errs = np.zeros((rows, cols))
    mu = np.zeros((rows, cols)) if want_mu else None
    rc = lib().oracle_run(ctypes.byref(p), ctypes.byref(info), _dp(stars_out),
                          _dp(ccs.view(np.float64)), _dp(caus.view(np.float64)), _dp(errs), _dp(mu))
    if rc != 0:
        raise ValueError(info.error.decode())
    return {"info": info.as_dict(), "stars": stars_out, "ccs": ccs, "caustics": caus,
            "errs": errs, "mu_length_scales": mu}


def eval_field(z, phi=None, stars=None, **kw) -> dict:
    """alpha, f, df/dz and the lens map at points z, with the reference's tree/FMM."""
    p, keep = make_params(stars=stars, **kw)
    z = np.ascontiguousarray(z, dtype=np.complex128)
    phi = np.zeros(z.shape[0]) if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
    out = {k: np.zeros(z.shape[0], dtype=np.complex128) for k in ("alpha", "f", "df", "w")}
    info = OracleInfo()
    rc = lib().oracle_eval(ctypes.byref(p), ctypes.byref(info), z.shape[0], _dp(z.view(np.float64)), _dp(phi),
                           *(_dp(out[k].view(np.float64)) for k in ("alpha", "f", "df", "w")))
    if rc != 0:
        raise ValueError(info.error.decode())
    out["info"] = info.as_dict()
    return out


def match_sets(a, b, nb: int) -> dict:
    """Match root sets per (branch, phi) column by nearest neighbour."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    assert a.shape == b.shape
    rows, cols = a.shape
    md = ctypes.c_double()
    nbij = ctypes.c_longlong()
    nfin = ctypes.c_longlong()
    rc = lib().oracle_match_sets(rows, cols, nb, _dp(a.view(np.float64)), _dp(b.view(np.float64)),
                                 ctypes.byref(md), ctypes.byref(nbij), ctypes.byref(nfin))
    if rc != 0:
        raise ValueError("bad shapes")
    return {"max_dist": md.value, "non_bijective_cols": nbij.value, "non_finite": nfin.value}


def match_index(a, b, nb: int):
    """For every entry of a, the row of b holding its nearest root in the same
    (branch, phi) column, and that distance.  Use ``take_matched`` to bring any
    per-point array of b into a's order."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    rows, cols = a.shape
    idx = np.empty((rows, cols), dtype=np.int32)
    dist = np.empty((rows, cols))
    L = lib()
    L.oracle_match_index.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_double)]
    rc = L.oracle_match_index(rows, cols, nb, _dp(a.view(np.float64)), _dp(b.view(np.float64)),
                              idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(dist))
    if rc != 0:
        raise ValueError("bad shapes")
    return idx, dist


def take_matched(arr, idx):
    """arr (rows, cols) of b rearranged into a's order by match_index's idx."""
    cols = np.arange(arr.shape[1])[None, :]
    return arr[np.clip(idx, 0, None), cols]


# ---- readers for the reference's output layout (reference util.py:28-103) ----

def read_array(path, dtype=np.float64, is_complex=False):
    with open(path, "rb") as f:
        nrows, ncols = np.fromfile(f, dtype=np.int32, count=2)
        dat = np.fromfile(f, dtype=dtype)
    if is_complex:
        return dat.reshape(nrows, ncols, 2)[..., 0] + 1j * dat.reshape(nrows, ncols, 2)[..., 1]
    return dat.reshape(nrows, ncols)


def read_star_file(path, dtype=np.float64):
    with open(path, "rb") as f:
        nstars, rect = np.fromfile(f, dtype=np.int32, count=2)
        corner = np.fromfile(f, dtype=dtype, count=2)
        theta = np.fromfile(f, dtype=dtype, count=1)[0]
        stars = np.fromfile(f, dtype=dtype).reshape(nstars, 3)
    return {"stars": stars, "rectangular": int(rect), "corner": complex(corner[0], corner[1]),
            "theta_star": float(theta)}


def read_params(path) -> dict:
    out = {}
    with open(path) as f:
        for line in f:
            k, v = line.split()
            try:
                fv = float(v)
                out[k] = int(fv) if fv == int(fv) and "." not in v and "e" not in v else fv
            except ValueError:
                out[k] = v
    return out
