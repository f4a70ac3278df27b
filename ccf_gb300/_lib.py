"""ctypes binding of the C ABI in include/ccf_gb300.h.

The shared library is built in-tree (``ccf_gb300/lib/libccf_gb300.so``);
loading fails loudly when it is missing -- there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libccf_gb300.so")

CCF_OK = 0
STATUS_NAMES = {
    0: "CCF_OK", 1: "CCF_ERR_INVALID_ARGUMENT", 2: "CCF_ERR_CUDA", 3: "CCF_ERR_NO_DEVICE",
    4: "CCF_ERR_OUT_OF_MEMORY", 5: "CCF_ERR_IO", 6: "CCF_ERR_NOT_RUN", 7: "CCF_ERR_NUMERIC",
    8: "CCF_ERR_TIMEOUT", 9: "CCF_ERR_BUDGET",
}
STATUS_CODES = {name: code for code, name in STATUS_NAMES.items()}
PRECISION_FP64 = 0
PRECISION_MIXED = 1
CONTINUATION_TRACK = 0
CONTINUATION_ABERTH = 1


class CcfParams(ctypes.Structure):
    _fields_ = [
        ("kappa_tot", ctypes.c_double),
        ("shear", ctypes.c_double),
        ("kappa_star", ctypes.c_double),
        ("theta_star", ctypes.c_double),
        ("mass_function", ctypes.c_char * 32),
        ("m_solar", ctypes.c_double),
        ("m_lower", ctypes.c_double),
        ("m_upper", ctypes.c_double),
        ("rectangular", ctypes.c_int),
        ("approx", ctypes.c_int),
        ("safety_scale", ctypes.c_double),
        ("num_stars", ctypes.c_int),
        ("starfile", ctypes.c_char * 1024),
        ("num_phi", ctypes.c_int),
        ("num_branches", ctypes.c_int),
        ("random_seed", ctypes.c_int),
        ("write_stars", ctypes.c_int),
        ("write_critical_curves", ctypes.c_int),
        ("write_caustics", ctypes.c_int),
        ("write_mu_length_scales", ctypes.c_int),
        ("outfile_prefix", ctypes.c_char * 1024),
        ("precision", ctypes.c_int),
        ("output_float", ctypes.c_int),
        ("max_iters_init", ctypes.c_int),
        ("max_iters_step", ctypes.c_int),
        ("exact_binomials", ctypes.c_int),
        ("device", ctypes.c_int),
        ("continuation", ctypes.c_int),
        ("solved_centres", ctypes.c_int),
        ("expansion_order", ctypes.c_int),
        ("leaf_max_stars", ctypes.c_int),
        ("init_cluster", ctypes.c_int),
        ("autotune", ctypes.c_int),
        ("host_outputs", ctypes.c_int),
        ("reserved", ctypes.c_int * 1),
    ]


class CcfInfo(ctypes.Structure):
    _fields_ = [
        ("num_stars", ctypes.c_int),
        ("num_roots", ctypes.c_int),
        ("taylor_smooth", ctypes.c_int),
        ("tree_levels", ctypes.c_int),
        ("expansion_order", ctypes.c_int),
        ("num_nodes", ctypes.c_int),
        ("num_leaves", ctypes.c_int),
        ("rectangular", ctypes.c_int),
        ("random_seed", ctypes.c_int),
        ("has_nan", ctypes.c_int),
        ("kappa_star", ctypes.c_double),
        ("theta_star", ctypes.c_double),
        ("corner_x1", ctypes.c_double),
        ("corner_x2", ctypes.c_double),
        ("mu_ave", ctypes.c_double),
        ("alpha_error", ctypes.c_double),
        ("root_half_length", ctypes.c_double),
        ("mean_mass", ctypes.c_double),
        ("mean_mass2", ctypes.c_double),
        ("mean_mass2_ln_mass", ctypes.c_double),
        ("kappa_star_actual", ctypes.c_double),
        ("m_lower", ctypes.c_double),
        ("m_upper", ctypes.c_double),
        ("m_lower_actual", ctypes.c_double),
        ("m_upper_actual", ctypes.c_double),
        ("mean_mass_actual", ctypes.c_double),
        ("mean_mass2_actual", ctypes.c_double),
        ("mean_mass2_ln_mass_actual", ctypes.c_double),
        ("max_error", ctypes.c_double),
        ("num_points", ctypes.c_longlong),
        ("root_updates", ctypes.c_longlong),
        ("sum_terms", ctypes.c_longlong),
        ("unconverged", ctypes.c_longlong),
        ("max_sweeps_init", ctypes.c_int),
        ("max_sweeps_step", ctypes.c_int),
        ("t_stars", ctypes.c_double),
        ("t_tree", ctypes.c_double),
        ("t_init_roots", ctypes.c_double),
        ("t_ccs", ctypes.c_double),
        ("t_caustics", ctypes.c_double),
        ("t_total", ctypes.c_double),
        ("kernel_launches", ctypes.c_longlong),
        ("root_updates_init", ctypes.c_longlong),
        ("sum_terms_init", ctypes.c_longlong),
        ("rows_rerun", ctypes.c_longlong),
        ("step_halvings", ctypes.c_longlong),
        ("rerun_flags", ctypes.c_longlong),
        ("near_mean", ctypes.c_double),
        ("centres_solved", ctypes.c_int),
        ("rows_retracked", ctypes.c_int),
        ("leaves_folded", ctypes.c_int),
        ("max_error_unpolished", ctypes.c_double),
        ("unconverged_unpolished", ctypes.c_longlong),
        ("points_polished", ctypes.c_longlong),
        ("points_above_target", ctypes.c_longlong),
        ("init_cluster", ctypes.c_int),
        ("leaf_max_stars", ctypes.c_int),
        ("points_at_fp64_floor", ctypes.c_longlong),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


#: every symbol include/ccf_gb300.h declares
EXPORTED = [
    "ccf_abi_version", "ccf_default_params", "ccf_create", "ccf_destroy", "ccf_set_params", "ccf_get_params",
    "ccf_set_stars", "ccf_run", "ccf_save", "ccf_get_info", "ccf_get_results", "ccf_get_device_results",
    "ccf_last_error", "ccf_derive_params", "ccf_run_batch", "ccf_write_star_file", "ccf_eval_points",
    "ccf_continue_branch_noalloc", "ccf_estimate_device_bytes", "ccf_batch_submit", "ccf_batch_poll",
    "ccf_batch_wait", "ccf_batch_destroy", "ccf_server_create", "ccf_server_submit", "ccf_server_wait",
    "ccf_server_request_info", "ccf_server_handle", "ccf_server_release", "ccf_server_get_stats",
    "ccf_server_destroy", "ccf_host_alloc", "ccf_host_free", "ccf_fmm_error", "ccf_autotune",
]

REQUEST_QUEUED, REQUEST_RUNNING, REQUEST_DONE, REQUEST_FAILED, REQUEST_REJECTED = range(5)


class CcfServerConfig(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int),
        ("slots", ctypes.c_int),
        ("hbm_budget", ctypes.c_ulonglong),
        ("verbose", ctypes.c_int),
        ("reserved", ctypes.c_int * 7),
    ]


class CcfRequestInfo(ctypes.Structure):
    _fields_ = [
        ("state", ctypes.c_int),
        ("status", ctypes.c_int),
        ("deferred", ctypes.c_int),
        ("reserved0", ctypes.c_int),
        ("bytes", ctypes.c_ulonglong),
        ("t_submit", ctypes.c_double),
        ("t_start", ctypes.c_double),
        ("t_end", ctypes.c_double),
        ("reserved", ctypes.c_double * 4),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if not name.startswith("reserved")}


class CcfServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_longlong),
        ("admitted", ctypes.c_longlong),
        ("completed", ctypes.c_longlong),
        ("failed", ctypes.c_longlong),
        ("rejected", ctypes.c_longlong),
        ("deferred", ctypes.c_longlong),
        ("queued", ctypes.c_longlong),
        ("running", ctypes.c_longlong),
        ("bytes_in_use", ctypes.c_ulonglong),
        ("hbm_budget", ctypes.c_ulonglong),
        ("reserved", ctypes.c_double * 4),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load the native library (once).  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("CCF_GB300_LIB", LIB_PATH)
        if not os.path.exists(p):
            raise RuntimeError(f"native library {p} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(p)
        H = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        PP, PI = ctypes.POINTER(CcfParams), ctypes.POINTER(CcfInfo)
        L.ccf_abi_version.restype = ctypes.c_int
        L.ccf_default_params.argtypes = [PP]
        L.ccf_default_params.restype = None
        L.ccf_create.argtypes = [ctypes.POINTER(H)]
        L.ccf_destroy.argtypes = [H]
        L.ccf_destroy.restype = None
        L.ccf_set_params.argtypes = [H, PP]
        L.ccf_get_params.argtypes = [H, PP]
        L.ccf_set_stars.argtypes = [H, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ccf_run.argtypes = [H, ctypes.c_int]
        L.ccf_save.argtypes = [H, ctypes.c_int]
        L.ccf_get_info.argtypes = [H, PI]
        L.ccf_get_results.argtypes = [H, dp, dp, dp, dp, dp]
        L.ccf_get_device_results.argtypes = [H] + [ctypes.POINTER(ctypes.c_void_p)] * 4
        L.ccf_last_error.argtypes = [H]
        L.ccf_last_error.restype = ctypes.c_char_p
        L.ccf_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
        L.ccf_host_free.argtypes = [ctypes.c_void_p]
        L.ccf_derive_params.argtypes = [PP, PI, ctypes.c_char_p, ctypes.c_size_t]
        L.ccf_run_batch.argtypes = [ctypes.POINTER(H), ctypes.c_int, ctypes.c_int]
        L.ccf_write_star_file.argtypes = [H, ctypes.c_char_p]
        L.ccf_eval_points.argtypes = [H, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp]
        L.ccf_fmm_error.argtypes = [H, dp]
        L.ccf_autotune.argtypes = [H, ctypes.c_int, ctypes.c_int, PP, dp]
        vp = ctypes.c_void_p
        L.ccf_continue_branch_noalloc.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp]
        ull = ctypes.c_ulonglong
        L.ccf_estimate_device_bytes.argtypes = [PP, ctypes.POINTER(ull)]
        L.ccf_batch_submit.argtypes = [ctypes.POINTER(H), ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.ccf_batch_poll.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        L.ccf_batch_wait.argtypes = [vp]
        L.ccf_batch_destroy.argtypes = [vp]
        L.ccf_batch_destroy.restype = None
        L.ccf_server_create.argtypes = [ctypes.POINTER(CcfServerConfig), ctypes.POINTER(vp)]
        L.ccf_server_submit.argtypes = [vp, PP, ctypes.POINTER(ctypes.c_longlong)]
        L.ccf_server_wait.argtypes = [vp, ctypes.c_longlong, ctypes.c_double]
        L.ccf_server_request_info.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(CcfRequestInfo)]
        L.ccf_server_handle.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(H)]
        L.ccf_server_release.argtypes = [vp, ctypes.c_longlong]
        L.ccf_server_get_stats.argtypes = [vp, ctypes.POINTER(CcfServerStats)]
        L.ccf_server_destroy.argtypes = [vp]
        L.ccf_server_destroy.restype = None
        for name in EXPORTED:
            fn = getattr(L, name)
            if fn.restype is ctypes.c_int and name not in ("ccf_abi_version",):
                fn.restype = ctypes.c_int
        _lib = L
        return _lib
