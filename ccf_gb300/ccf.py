"""Python mirror of the reference's operator API, the class CCF<T>
(include/ccf.cuh:34-1289): the same public fields with the same defaults,
``run(verbose) -> bool`` and ``save(verbose) -> bool``, backed by the C ABI
of include/ccf_gb300.h (no computation happens in Python).

Additions: ``precision`` ("mixed" or "fp64"), ``results()`` returning the
outputs as numpy arrays in the reference's file layout, ``info()`` with the
derived parameters and timings, ``set_stars()`` for an in-memory star field,
and ``run_batch()`` to solve many fields in shared persistent launches.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib

_FIELDS = {
    # name: (default, kind) -- include/ccf.cuh:42-62
    "kappa_tot": (0.3, float),
    "shear": (0.3, float),
    "kappa_star": (0.27, float),
    "theta_star": (1.0, float),
    "mass_function_str": ("equal", str),
    "m_solar": (1.0, float),
    "m_lower": (0.01, float),
    "m_upper": (50.0, float),
    "rectangular": (0, int),
    "approx": (1, int),
    "safety_scale": (1.37, float),
    "num_stars": (137, int),
    "starfile": ("", str),
    "num_phi": (100, int),
    "num_branches": (1, int),
    "random_seed": (0, int),
    "write_stars": (1, int),
    "write_critical_curves": (1, int),
    "write_caustics": (1, int),
    "write_mu_length_scales": (0, int),
    "outfile_prefix": ("./", str),
}


class CCFError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_lib.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class CCF:
    """Critical-curve and caustic finder for one star field."""

    def __init__(self, **kw):
        self._L = _lib.load()
        self._h = ctypes.c_void_p()
        rc = self._L.ccf_create(ctypes.byref(self._h))
        if rc != 0:
            raise CCFError(rc, "ccf_create failed")
        for k, (v, _) in _FIELDS.items():
            setattr(self, k, v)
        self.precision = "mixed"
        self.output_float = 0
        self.max_iters_init = 300
        self.max_iters_step = 60
        self.exact_binomials = 0
        self.device = 0
        self.continuation = "track"
        self.solved_centres = 0
        self.expansion_order = 0
        self.leaf_max_stars = 0
        self.init_cluster = 0
        self.autotune = 0
        self.host_outputs = 0
        self._stars_keep = None
        self.last_status = 0
        for k, v in kw.items():
            if k == "mass_function":
                k = "mass_function_str"
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)

    def __del__(self):
        try:
            if getattr(self, "_owned", True) and getattr(self, "_h", None) and self._h.value:
                self._L.ccf_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # ---- parameters ----
    def _params(self) -> _lib.CcfParams:
        p = _lib.CcfParams()
        self._L.ccf_default_params(ctypes.byref(p))
        for k, (_, kind) in _FIELDS.items():
            v = getattr(self, k)
            name = "mass_function" if k == "mass_function_str" else k
            if kind is str:
                setattr(p, name, str(v).encode())
            else:
                setattr(p, name, kind(v))
        prec = self.precision
        p.precision = _lib.PRECISION_MIXED if str(prec).lower() in ("mixed", "1") else _lib.PRECISION_FP64
        p.output_float = int(self.output_float)
        p.max_iters_init = int(self.max_iters_init)
        p.max_iters_step = int(self.max_iters_step)
        p.exact_binomials = int(self.exact_binomials)
        p.device = int(self.device)
        p.continuation = _continuation_code(self.continuation)
        p.solved_centres = int(self.solved_centres)
        p.expansion_order = int(self.expansion_order)
        p.leaf_max_stars = int(self.leaf_max_stars)
        p.init_cluster = int(self.init_cluster)
        p.autotune = int(self.autotune)
        p.host_outputs = int(self.host_outputs)
        return p

    def _push(self):
        p = self._params()
        rc = self._L.ccf_set_params(self._h, ctypes.byref(p))
        if rc != 0:
            raise CCFError(rc, self.last_error())

    def set_stars(self, stars, rectangular: int, corner: complex, theta_star: float = 1.0):
        """Use this star field ((N, 3) array of x1, x2, mass) instead of generating one."""
        if stars is None:
            self._L.ccf_set_stars(self._h, 0, None, 0, 0.0, 0.0, 1.0)
            self._stars_keep = None
            return
        a = np.ascontiguousarray(stars, dtype=np.float64).reshape(-1, 3)
        corner = complex(corner)
        rc = self._L.ccf_set_stars(self._h, a.shape[0], a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   int(rectangular), corner.real, corner.imag, float(theta_star))
        if rc != 0:
            raise CCFError(rc, self.last_error())
        self._stars_keep = a

    def last_error(self) -> str:
        return self._L.ccf_last_error(self._h).decode()

    def fmm_error(self) -> float:
        """Largest far-field error of the last run's field against the direct
        sum over every star, at one point per leaf (ccf_fmm_error)."""
        out = ctypes.c_double()
        rc = self._L.ccf_fmm_error(self._h, ctypes.byref(out))
        if rc != 0:
            raise CCFError(rc, self.last_error())
        return float(out.value)

    def tune(self, fmm: bool = False, verbose: int = 0) -> dict:
        """Run the autotuner (ccf_autotune) on this field and adopt the
        settings it finds; returns them with the tuned field's device time.
        The field must be run again for results."""
        self._push()
        best = _lib.CcfParams()
        secs = ctypes.c_double()
        rc = self._L.ccf_autotune(self._h, 1 if fmm else 0, int(verbose), ctypes.byref(best), ctypes.byref(secs))
        if rc != 0:
            raise CCFError(rc, self.last_error())
        out = {k: int(getattr(best, k)) for k in ("init_cluster", "solved_centres", "leaf_max_stars", "expansion_order")}
        for k, v in out.items():
            setattr(self, k, v)
        out["seconds"] = float(secs.value)
        return out

    def estimate_device_bytes(self) -> int:
        """Device memory a run with the current parameters holds (upper estimate)."""
        p = self._params()
        out = ctypes.c_ulonglong()
        rc = self._L.ccf_estimate_device_bytes(ctypes.byref(p), ctypes.byref(out))
        if rc != 0:
            raise CCFError(rc, "ccf_estimate_device_bytes failed")
        return int(out.value)

    # ---- the reference's API ----
    def run(self, verbose: int = 0) -> bool:
        """CCF<T>::run (include/ccf.cuh:1265-1280)."""
        self._push()
        self.last_status = self._L.ccf_run(self._h, int(verbose))
        if self.last_status == 0:
            self.random_seed = self.info()["random_seed"] or self.random_seed
        elif verbose >= 0:
            import sys
            sys.stderr.write(self.last_error() + "\n")
        return self.last_status == 0

    def save(self, verbose: int = 0) -> bool:
        """CCF<T>::save (include/ccf.cuh:1282-1287)."""
        self._push()
        self.last_status = self._L.ccf_save(self._h, int(verbose))
        if self.last_status != 0 and verbose >= 0:
            import sys
            sys.stderr.write(self.last_error() + "\n")
        return self.last_status == 0

    # ---- results ----
    def info(self) -> dict:
        i = _lib.CcfInfo()
        self._L.ccf_get_info(self._h, ctypes.byref(i))
        return i.as_dict()

    def results(self, stars: bool = True, out: dict | None = None) -> dict:
        """Outputs in the reference's file layout: rows = num_roots * num_branches,
        cols = num_phi / num_branches + 1, row = root * num_branches + branch.

        out: arrays to fill instead of new ones ("ccs", "caustics", "errs",
        "mu_length_scales", "stars"; C-contiguous, the shapes and dtypes of
        the returned arrays), e.g. from result_buffers(pinned=True), whose
        page-locked memory takes the device copies at full bandwidth."""
        inf = self.info()
        rows = inf["num_roots"] * self.num_branches
        cols = self.num_phi // self.num_branches + 1
        out = out or {}

        def buf(name, shape, dtype, want):
            if not want:
                return None
            a = out.get(name)
            if a is None:
                return np.empty(shape, dtype=dtype)
            if a.shape != shape or a.dtype != np.dtype(dtype) or not a.flags.c_contiguous:
                raise ValueError(f"out[{name!r}] must be a C-contiguous {np.dtype(dtype)} array of shape {shape}")
            return a

        ccs = buf("ccs", (rows, cols), np.complex128, True)
        errs = buf("errs", (rows, cols), np.float64, True)
        caus = buf("caustics", (rows, cols), np.complex128, self.write_caustics)
        mu = buf("mu_length_scales", (rows, cols), np.float64, self.write_mu_length_scales)
        st = buf("stars", (inf["num_stars"], 3), np.float64, stars)
        dp = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        rc = self._L.ccf_get_results(self._h, dp(ccs), dp(caus), dp(errs), dp(mu), dp(st))
        if rc != 0:
            raise CCFError(rc, self.last_error())
        return {"ccs": ccs, "caustics": caus, "errs": errs, "mu_length_scales": mu, "stars": st, "info": inf}


    def result_buffers(self, stars: bool = False, pinned: bool = True) -> dict:
        """Arrays for results(out=...) sized for the current parameters (after
        a run); page-locked when pinned."""
        inf = self.info()
        rows = inf["num_roots"] * self.num_branches
        cols = self.num_phi // self.num_branches + 1
        mk = pinned_empty if pinned else (lambda shape, dtype: np.empty(shape, dtype=dtype))
        out = {"ccs": mk((rows, cols), np.complex128), "errs": mk((rows, cols), np.float64)}
        if self.write_caustics:
            out["caustics"] = mk((rows, cols), np.complex128)
        if self.write_mu_length_scales:
            out["mu_length_scales"] = mk((rows, cols), np.float64)
        if stars:
            out["stars"] = mk((inf["num_stars"], 3), np.float64)
        return out

    def eval_points(self, z, phi) -> dict:
        """f, df/dz, lens map, 1/mu bound and length scale at points z (after run)."""
        z = np.ascontiguousarray(z, dtype=np.complex128).ravel()
        phi = np.ascontiguousarray(np.broadcast_to(phi, z.shape), dtype=np.float64)
        out = {"f": np.empty_like(z), "df": np.empty_like(z), "w": np.empty_like(z),
               "err": np.empty(z.shape), "mu_length": np.empty(z.shape)}
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        rc = self._L.ccf_eval_points(self._h, z.shape[0], dp(z.view(np.float64)), dp(phi), dp(out["f"].view(np.float64)),
                                     dp(out["df"].view(np.float64)), dp(out["w"].view(np.float64)), dp(out["err"]),
                                     dp(out["mu_length"]))
        if rc != 0:
            raise CCFError(rc, self.last_error())
        return out


def run_batch(fields: list[CCF], verbose: int = 0) -> bool:
    """Solve several fields in shared solver launches (one initial-solve and
    one continuation launch for the whole batch)."""
    if not fields:
        return True
    L = fields[0]._L
    for f in fields:
        f._push()
    arr = (ctypes.c_void_p * len(fields))(*[f._h.value for f in fields])
    rc = L.ccf_run_batch(arr, len(fields), int(verbose))
    for f in fields:
        f.last_status = rc
    return rc == 0


class BatchJob:
    """A batch of fields running on a host thread (ccf_batch_submit)."""

    def __init__(self, fields: list[CCF], verbose: int = 0):
        self._L = fields[0]._L
        self.fields = fields
        for f in fields:
            f._push()
        arr = (ctypes.c_void_p * len(fields))(*[f._h.value for f in fields])
        self._b = ctypes.c_void_p()
        rc = self._L.ccf_batch_submit(arr, len(fields), int(verbose), ctypes.byref(self._b))
        if rc != 0:
            raise CCFError(rc, "ccf_batch_submit failed")

    def done(self) -> bool:
        d = ctypes.c_int()
        self._L.ccf_batch_poll(self._b, ctypes.byref(d))
        return bool(d.value)

    def wait(self) -> bool:
        rc = self._L.ccf_batch_wait(self._b)
        for f in self.fields:
            f.last_status = rc
        return rc == 0

    def __del__(self):
        try:
            if self._b.value:
                self._L.ccf_batch_destroy(self._b)
                self._b = ctypes.c_void_p()
        except Exception:
            pass


def submit_batch(fields: list[CCF], verbose: int = 0) -> BatchJob:
    """run_batch without blocking: poll or wait on the returned job."""
    return BatchJob(fields, verbose)


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """An uninitialised array in page-locked host memory (ccf_host_alloc),
    freed when the array is collected."""
    L = _lib.load()
    shape = tuple(int(x) for x in np.atleast_1d(shape))
    dt = np.dtype(dtype)
    nbytes = max(1, int(np.prod(shape)) * dt.itemsize)
    p = ctypes.c_void_p()
    rc = L.ccf_host_alloc(nbytes, ctypes.byref(p))
    if rc != 0:
        raise CCFError(rc, "ccf_host_alloc failed")
    raw = (ctypes.c_char * nbytes).from_address(p.value)
    weakref.finalize(raw, L.ccf_host_free, p.value)
    a = np.frombuffer(raw, dtype=dt, count=int(np.prod(shape))).reshape(shape)
    return a


def _continuation_code(v) -> int:
    """'track' (per-root tracking, checked, with the full-sum re-run) or
    'aberth' (the full Aberth step of the reference for every root)."""
    k = str(v).lower()
    if k in ("track", "0"):
        return _lib.CONTINUATION_TRACK
    if k in ("aberth", "1"):
        return _lib.CONTINUATION_ABERTH
    raise ValueError(f"continuation must be 'track' or 'aberth', not {v!r}")


def _bare(**kw) -> CCF:
    """A CCF parameter holder without a native handle."""
    c = CCF.__new__(CCF)
    c._L = _lib.load()
    c._h = ctypes.c_void_p()
    c._owned = False
    for k, (v, _) in _FIELDS.items():
        setattr(c, k, v)
    c.precision, c.output_float, c.max_iters_init, c.max_iters_step, c.exact_binomials, c.device = \
        "mixed", 0, 300, 60, 0, 0
    c.continuation = "track"
    c.solved_centres = 0
    c.expansion_order = c.leaf_max_stars = c.init_cluster = c.autotune = c.host_outputs = 0
    c._stars_keep = None
    c.last_status = 0
    for k, v in kw.items():
        if k == "mass_function":
            k = "mass_function_str"
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


class Server:
    """Request loop over one GPU (ccf_server_*): requests are queued in arrival
    order and admitted while a slot is free and the device memory of the
    admitted requests stays within hbm_budget; each runs on its own stream, so
    concurrent requests overlap on the device.  Results stay on the device
    until release(id)."""

    def __init__(self, slots: int = 4, hbm_budget: float = 60e9, device: int = 0, verbose: int = 0):
        self._L = _lib.load()
        cfg = _lib.CcfServerConfig()
        cfg.device, cfg.slots, cfg.hbm_budget, cfg.verbose = int(device), int(slots), int(hbm_budget), int(verbose)
        self._s = ctypes.c_void_p()
        rc = self._L.ccf_server_create(ctypes.byref(cfg), ctypes.byref(self._s))
        if rc != 0:
            raise CCFError(rc, "ccf_server_create failed")
        self._kw = {}

    def submit(self, **kw) -> int:
        """Queue a field solve with CCF's parameters; returns its request id."""
        c = _bare(**kw)
        p = c._params()
        rid = ctypes.c_longlong()
        rc = self._L.ccf_server_submit(self._s, ctypes.byref(p), ctypes.byref(rid))
        if rc != 0:
            raise CCFError(rc, "ccf_server_submit failed")
        self._kw[rid.value] = dict(kw)
        return rid.value

    def wait(self, rid: int, timeout: float | None = None) -> int:
        """Status of the request once finished (CCF_ERR_TIMEOUT while running)."""
        return self._L.ccf_server_wait(self._s, rid, -1.0 if timeout is None else float(timeout))

    def info(self, rid: int) -> dict:
        i = _lib.CcfRequestInfo()
        rc = self._L.ccf_server_request_info(self._s, rid, ctypes.byref(i))
        if rc != 0:
            raise CCFError(rc, "unknown request")
        return i.as_dict()

    def field(self, rid: int) -> CCF:
        """The finished request as a CCF (results(), info(), save()); valid until release(rid)."""
        h = ctypes.c_void_p()
        rc = self._L.ccf_server_handle(self._s, rid, ctypes.byref(h))
        if rc != 0:
            raise CCFError(rc, "request has no field")
        c = _bare(**self._kw[rid])
        c._h = h
        return c

    def release(self, rid: int) -> None:
        rc = self._L.ccf_server_release(self._s, rid)
        if rc != 0:
            raise CCFError(rc, "ccf_server_release failed")
        self._kw.pop(rid, None)

    def stats(self) -> dict:
        st = _lib.CcfServerStats()
        self._L.ccf_server_get_stats(self._s, ctypes.byref(st))
        return st.as_dict()

    def close(self) -> None:
        if self._s.value:
            self._L.ccf_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def derive_params(**kw) -> dict:
    """Checks and derived parameters on the host (no GPU needed)."""
    c = _bare(**kw)
    p = c._params()
    info = _lib.CcfInfo()
    msg = ctypes.create_string_buffer(512)
    rc = c._L.ccf_derive_params(ctypes.byref(p), ctypes.byref(info), msg, 512)
    d = info.as_dict()
    d["rc"] = rc
    d["error"] = msg.value.decode()
    return d
