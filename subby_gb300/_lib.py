"""ctypes binding of ``libsubby_gb300.so`` (the C ABI of include/subby_gb300.h).

There is no CPU fallback: if the library is missing or cannot be loaded,
every entry point raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as ct
import os
import threading

from . import _build

OK = 0
ERR_ARG, ERR_TREE, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT = -1, -2, -3, -4, -5, -6
DEVICE_PTRS, BT_FP32, BT_FP64, IRREV_EXACT = 1, 2, 4, 8
MASK_NONE, MASK_AUTO, MASK_GIVEN = 0, 1, 2
COUNTS_EIGEN, COUNTS_F81 = 0, 1

# Exported symbols, as declared in include/subby_gb300.h.
EXPORTS = (
    "subby_version", "subby_strerror", "subby_last_error", "subby_plan_create", "subby_plan_create_irrev", "subby_plan_create_rows",
    "subby_plan_destroy", "subby_plan_device_bytes", "subby_plan_trim", "subby_plan_branch_counts",
    "subby_plan_posteriors", "subby_plan_status", "subby_plan_set_root_prior", "subby_plan_run", "subby_plan_grad",
    "subby_loglike", "subby_counts", "subby_rootprob", "subby_last_launch_count",
    "subby_debug_set_kernel", "subby_debug_fail_waits", "subby_counts_noalloc", "subby_mixture_posterior",
    "subby_tokenize", "subby_gather_rows", "subby_server_create", "subby_server_submit", "subby_server_wait",
    "subby_server_release", "subby_server_set", "subby_server_clock", "subby_server_stats",
    "subby_server_destroy", "subby_debug_packed_queue_wait",
)
WANT_LOGLIKE, WANT_COUNTS, WANT_ROOTPROB = 1, 2, 4


class Job(ct.Structure):
    """struct subby_job of include/subby_gb300.h."""
    _fields_ = [("parent_index", ct.c_void_p), ("distances", ct.c_void_p), ("R", ct.c_int),
                ("eigenvalues", ct.c_void_p), ("eigenvectors", ct.c_void_p), ("pi", ct.c_void_p), ("A", ct.c_int),
                ("alignment", ct.c_void_p), ("pitch", ct.c_int64), ("row_map", ct.c_void_p), ("C", ct.c_int),
                ("want", ct.c_int), ("counts_kind", ct.c_int), ("mask_mode", ct.c_int), ("arrival", ct.c_double),
                ("tag", ct.c_int64)]


class JobResult(ct.Structure):
    """struct subby_job_result of include/subby_gb300.h."""
    _fields_ = [("tag", ct.c_int64), ("handle", ct.c_int64), ("status", ct.c_int),
                ("logLike", ct.c_void_p), ("counts", ct.c_void_p), ("rootProb", ct.c_void_p),
                ("t_arrival", ct.c_double), ("t_start", ct.c_double), ("t_finish", ct.c_double)]

_lock = threading.Lock()
_lib = None

_p = ct.c_void_p
_i32p = ct.POINTER(ct.c_int32)
_f64p = ct.POINTER(ct.c_double)


class SubbyError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = _lib
        name = lib.subby_strerror(code).decode() if lib else str(code)
        detail = lib.subby_last_error().decode() if lib else ""
        super().__init__(f"{where}: {name} ({code}){': ' + detail if detail else ''}")
        self.code = code


class TreeError(SubbyError, ValueError):
    pass


def _declare(lib):
    lib.subby_version.restype = ct.c_char_p
    lib.subby_strerror.restype = ct.c_char_p
    lib.subby_strerror.argtypes = [ct.c_int]
    lib.subby_last_error.restype = ct.c_char_p
    lib.subby_last_launch_count.restype = ct.c_int
    lib.subby_debug_set_kernel.restype = ct.c_int
    lib.subby_debug_set_kernel.argtypes = [ct.c_int]
    lib.subby_debug_fail_waits.restype = ct.c_int
    lib.subby_debug_fail_waits.argtypes = [ct.c_int]
    lib.subby_plan_create.restype = ct.c_int
    lib.subby_plan_create.argtypes = [_p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.POINTER(ct.c_void_p)]
    lib.subby_plan_create_rows.restype = ct.c_int
    lib.subby_plan_create_rows.argtypes = [_p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.POINTER(ct.c_void_p)]
    lib.subby_plan_create_irrev.restype = ct.c_int
    lib.subby_plan_create_irrev.argtypes = [_p, _p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.POINTER(ct.c_void_p)]
    lib.subby_plan_destroy.restype = ct.c_int
    lib.subby_plan_destroy.argtypes = [_p]
    lib.subby_plan_device_bytes.restype = ct.c_size_t
    lib.subby_plan_device_bytes.argtypes = [_p]
    lib.subby_plan_trim.restype = ct.c_int
    lib.subby_plan_trim.argtypes = [_p]
    lib.subby_plan_set_root_prior.restype = ct.c_int
    lib.subby_plan_set_root_prior.argtypes = [_p, _p]
    lib.subby_plan_status.restype = ct.c_int
    lib.subby_plan_status.argtypes = [_p]
    lib.subby_plan_branch_counts.restype = ct.c_int
    lib.subby_plan_branch_counts.argtypes = [_p, _p, ct.c_int, _p, ct.c_int, ct.c_int, _p, ct.c_int, _p]
    lib.subby_tokenize.restype = ct.c_int
    lib.subby_tokenize.argtypes = [_p, ct.c_int64, _p, _p, _p, _p]
    lib.subby_gather_rows.restype = ct.c_int
    lib.subby_server_create.restype = ct.c_int
    lib.subby_server_create.argtypes = [ct.c_int, ct.c_size_t, ct.c_size_t, ct.POINTER(ct.c_void_p)]
    lib.subby_server_submit.restype = ct.c_int
    lib.subby_server_submit.argtypes = [_p, ct.POINTER(Job)]
    lib.subby_server_wait.restype = ct.c_int
    lib.subby_server_wait.argtypes = [_p, ct.POINTER(JobResult), ct.c_int, ct.c_int, ct.POINTER(ct.c_int)]
    lib.subby_server_release.restype = ct.c_int
    lib.subby_server_release.argtypes = [_p, ct.c_int64]
    lib.subby_server_set.restype = ct.c_int
    lib.subby_server_set.argtypes = [_p, ct.c_char_p, ct.c_double]
    lib.subby_server_clock.restype = ct.c_double
    lib.subby_server_clock.argtypes = [_p]
    lib.subby_server_stats.restype = ct.c_int
    lib.subby_server_stats.argtypes = [_p, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int), ct.POINTER(ct.c_int),
                                       ct.POINTER(ct.c_int), ct.POINTER(ct.c_longlong), ct.POINTER(ct.c_longlong)]
    lib.subby_server_destroy.restype = ct.c_int
    lib.subby_server_destroy.argtypes = [_p]
    lib.subby_debug_packed_queue_wait.restype = ct.c_int
    lib.subby_debug_packed_queue_wait.argtypes = [ct.c_int, ct.c_int, ct.POINTER(ct.c_int)]
    lib.subby_gather_rows.argtypes = [_p, ct.c_int64, _p, ct.c_int, ct.c_int, _p, _p]
    lib.subby_mixture_posterior.restype = ct.c_int
    lib.subby_mixture_posterior.argtypes = [_p, _p, ct.c_int, ct.c_int, _p, ct.c_int, _p]
    lib.subby_plan_posteriors.restype = ct.c_int
    lib.subby_plan_posteriors.argtypes = [_p, _p, ct.c_int, ct.c_int, _p, _p, ct.c_int, _p]
    lib.subby_plan_run.restype = ct.c_int
    lib.subby_plan_run.argtypes = [_p, _p, ct.c_int, _p, _p, _p, ct.c_int, ct.c_int, _p, ct.c_int, _p]
    lib.subby_plan_grad.restype = ct.c_int
    lib.subby_plan_grad.argtypes = [_p, _p, ct.c_int, _p, _p, _p, _p, ct.c_int, _p]
    for name in ("subby_loglike", "subby_rootprob"):
        f = getattr(lib, name)
        f.restype = ct.c_int
        f.argtypes = [_p, _p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.c_int, _p, ct.c_int, _p]
    lib.subby_counts_noalloc.restype = ct.c_int
    lib.subby_counts_noalloc.argtypes = [_p, _p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.c_int,
                                         ct.c_int, _p, _p, _p, _p]
    lib.subby_counts.restype = ct.c_int
    lib.subby_counts.argtypes = [_p, _p, _p, _p, _p, _p, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                                 ct.c_int, _p, _p, ct.c_int, _p]
    return lib


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library; raise if impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not os.path.exists(path) or build_if_missing:
            try:
                path = _build.build()
            except Exception as e:  # noqa: BLE001
                if not os.path.exists(path):
                    raise RuntimeError(f"subby_gb300: CUDA library unavailable ({e})") from e
        try:
            _lib = _declare(ct.CDLL(path))
        except OSError as e:
            raise RuntimeError(f"subby_gb300: cannot load {path}: {e}") from e
        return _lib


def check(code: int, where: str):
    if code != OK:
        if code == ERR_TREE:
            raise TreeError(code, where)
        raise SubbyError(code, where)


def last_launch_count() -> int:
    return int(load().subby_last_launch_count())
