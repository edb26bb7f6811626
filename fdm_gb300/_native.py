"""ctypes binding of libfdmgpu.so (the C ABI of include/fdmgpu.h).

The library is the only compute path: if it is missing or fails to load,
importing anything that solves raises immediately.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_longlong, c_size_t, c_uint, c_ulonglong, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfdmgpu.so"

OK, EINVAL, ESIZE, ENOMEM, ECUDA, ETIMEOUT, ENOTSUP, EBUDGET, EBUSY = range(9)
F64, F32 = 0, 1
PLAIN, MIXED = 0, 1
RECT_TRIDIAG, RECT_FFT2 = 0, 1
MAX_N = 1023
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024

_STATUS_NAMES = {
    OK: "OK", EINVAL: "EINVAL", ESIZE: "ESIZE", ENOMEM: "ENOMEM", ECUDA: "ECUDA",
    ETIMEOUT: "ETIMEOUT", ENOTSUP: "ENOTSUP", EBUDGET: "EBUDGET", EBUSY: "EBUSY",
}


REQ_SOLVE, REQ_ADVANCE = 0, 1
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(5)


class ServerStats(ctypes.Structure):
    """fdmgpu_server_stats_t."""
    _fields_ = [(n, c_ulonglong) for n in ("submitted", "completed", "failed", "cancelled", "rejected")] + \
        [("queued", c_int), ("running", c_int), ("batches", c_ulonglong), ("batched_requests", c_ulonglong)] + \
        [(n, c_double) for n in ("used_bytes", "peak_bytes", "budget_bytes", "plan_bytes", "session_bytes",
                                 "p50_ms", "p99_ms", "p50_solve_ms", "p99_solve_ms", "p50_advance_ms",
                                 "p99_advance_ms", "mean_queue_ms")] + [("shed", c_ulonglong)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class FdmError(RuntimeError):
    """A non-zero status from libfdmgpu.  `status` is the code."""

    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (_STATUS_NAMES.get(status, status), message))
        self.status = status


# (name, restype, argtypes)
_SIGS = [
    ("fdmgpu_last_error", c_char_p, []),
    ("fdmgpu_version", c_int, []),
    ("fdmgpu_launch_count", c_ulonglong, []),
    ("fdmgpu_profile_enable", c_int, [c_int]),
    ("fdmgpu_profile_collect", c_int, [POINTER(c_int)]),
    ("fdmgpu_profile_entry", c_int, [c_int, c_char_p, c_int, POINTER(c_longlong), POINTER(c_double)]),
    ("fdmgpu_profile_reset", c_int, []),
    ("fdmgpu_lapl_cube_create", c_int,
     [POINTER(c_void_p), c_int, c_int] + [c_double] * 6 + [c_int] * 3),
    ("fdmgpu_lapl_cube_set_precision", c_int, [c_void_p, c_int, c_double, c_int]),
    ("fdmgpu_lapl_cube_solve", c_int, [c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_lapl_cube_solve_host_batch", c_int, [c_void_p, c_void_p, c_void_p, c_int]),
    ("fdmgpu_lapl_cube_solve_device", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("fdmgpu_lapl_cube_solve_mixed_noalloc", c_int,
     [c_double] * 6 + [c_int] * 3 + [c_double, c_void_p, c_void_p, c_int, c_void_p]),
    ("fdmgpu_lapl_cube_last_info", c_int, [c_void_p, POINTER(c_int), POINTER(c_double), c_int]),
    ("fdmgpu_lapl_cube_scratch_bytes", c_int, [c_void_p, POINTER(c_size_t)]),
    ("fdmgpu_lapl_cube_set_schedule", c_int, [c_void_p, c_int, c_int]),
    ("fdmgpu_lapl_cube_set_pipeline", c_int, [c_void_p, c_int]),
    ("fdmgpu_lapl_cube_set_refinement", c_int, [c_void_p, c_int]),
    ("fdmgpu_lapl_cube_tune", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, POINTER(c_double)]),
    ("fdmgpu_lapl_cube_get_schedule", c_int, [c_void_p, POINTER(c_int), POINTER(c_int), POINTER(c_int)]),
    ("fdmgpu_lapl_cube_pipeline_in_use", c_int, [c_void_p, POINTER(c_int)]),
    ("fdmgpu_lapl_cube_device_status", c_int, [c_void_p, POINTER(c_int)]),
    ("fdmgpu_lapl_cube_destroy", c_int, [c_void_p]),
    ("fdmgpu_batch_create", c_int,
     [POINTER(c_void_p), c_int, POINTER(c_int), POINTER(c_double), POINTER(c_double), c_int, c_double]),
    ("fdmgpu_batch_tune", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p)]),
    ("fdmgpu_batch_solve", c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p), c_void_p]),
    ("fdmgpu_batch_info", c_int, [c_void_p, POINTER(c_int), POINTER(c_int)]),
    ("fdmgpu_batch_schedule", c_int,
     [c_void_p, c_int, POINTER(c_int), POINTER(c_int), POINTER(c_int), POINTER(c_int), POINTER(c_int),
      POINTER(c_double)]),
    ("fdmgpu_batch_destroy", c_int, [c_void_p]),
    ("fdmgpu_lapl_cyl_create", c_int, [POINTER(c_void_p), c_int, c_int] + [c_double] * 5 + [c_int] * 3),
    ("fdmgpu_lapl_cyl_solve", c_int, [c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_lapl_cyl_solve_device", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("fdmgpu_lapl_cyl_destroy", c_int, [c_void_p]),
    ("fdmgpu_lapl_rect_create", c_int,
     [POINTER(c_void_p), c_int, c_int] + [c_double] * 4 + [c_int] * 2),
    ("fdmgpu_lapl_rect_solve", c_int, [c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_lapl_rect_solve_device", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("fdmgpu_lapl_rect_destroy", c_int, [c_void_p]),
    ("fdmgpu_sine_device", c_int, [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_check_bounded_wait", c_int, [c_uint]),
    ("fdmgpu_sine_tc_device", c_int, [c_int, c_int, c_int, c_longlong, c_double, c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_tridiag_device", c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_nscube_create", c_int,
     [POINTER(c_void_p), c_int, c_int, c_int] + [c_double] * 9),
    ("fdmgpu_nscube_step", c_int, [c_void_p, c_int]),
    ("fdmgpu_nscube_step_many", c_int, [c_void_p, c_void_p, c_int]),
    ("fdmgpu_nscube_set_exact", c_int, [c_void_p, c_int]),
    ("fdmgpu_nscube_set_stream", c_int, [c_void_p, c_void_p]),
    ("fdmgpu_nscube_field_info", c_int, [c_void_p, c_int, POINTER(c_size_t), POINTER(c_int)]),
    ("fdmgpu_nscube_get_field", c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    ("fdmgpu_nscube_set_field", c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    ("fdmgpu_nscube_field_device", c_int, [c_void_p, c_int, POINTER(c_void_p)]),
    ("fdmgpu_nscube_time_index", c_int, [c_void_p, POINTER(c_int)]),
    ("fdmgpu_nscube_vtk_out", c_int, [c_void_p, c_char_p]),
    ("fdmgpu_nscube_dtype", c_int, [c_void_p, POINTER(c_int)]),
    ("fdmgpu_nscube_destroy", c_int, [c_void_p]),
    ("fdmgpu_check_const_division", c_int, [c_longlong, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_check_dd_conversions", c_int, [c_longlong] + [c_void_p] * 10),
    ("fdmgpu_nscyl_create", c_int, [POINTER(c_void_p), c_int, c_int] + [c_double] * 7 + [c_int] * 3),
    ("fdmgpu_nscyl_step", c_int, [c_void_p, c_int]),
    ("fdmgpu_nscyl_field_info", c_int, [c_void_p, c_int, POINTER(c_size_t), POINTER(c_int)]),
    ("fdmgpu_nscyl_get_field", c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    ("fdmgpu_nscyl_time_index", c_int, [c_void_p, POINTER(c_int)]),
    ("fdmgpu_nscyl_set_field", c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    ("fdmgpu_nscyl_l_step", c_int, [c_void_p, c_int]),
    ("fdmgpu_nscyl_vrandom", c_int, [c_void_p]),
    ("fdmgpu_nscyl_destroy", c_int, [c_void_p]),
    ("fdmgpu_lapl_rect_create_flags", c_int, [POINTER(c_void_p), c_int, c_int, c_int] + [c_double] * 4
     + [c_int] * 2),
    ("fdmgpu_pfft3d_device", c_int, [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_int, c_void_p]),
    ("fdmgpu_pfft3d", c_int, [c_int, c_int, c_int, c_double, c_void_p, c_void_p]),
    ("fdmgpu_pfft_device", c_int, [c_int, c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]),
    ("fdmgpu_nbody_create", c_int, [POINTER(c_void_p), c_int] + [c_double] * 4 + [c_int] * 3 + [c_double] * 3
     + [c_int] * 3 + [c_double]),
    ("fdmgpu_nbody_info", c_int, [c_void_p, POINTER(c_int), POINTER(c_double), POINTER(c_double),
                                  POINTER(c_longlong)]),
    ("fdmgpu_nbody_set_bodies", c_int, [c_void_p] * 6),
    ("fdmgpu_nbody_get_bodies", c_int, [c_void_p] * 7),
    ("fdmgpu_nbody_step", c_int, [c_void_p, c_int]),
    ("fdmgpu_nbody_step_async", c_int, [c_void_p, c_int]),
    ("fdmgpu_nbody_sync", c_int, [c_void_p]),
    ("fdmgpu_nbody_calc_forces", c_int, [c_void_p]),
    ("fdmgpu_nbody_direct_forces", c_int, [c_void_p, c_void_p]),
    ("fdmgpu_nbody_get_field", c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    ("fdmgpu_nbody_destroy", c_int, [c_void_p]),
    ("fdmgpu_server_create", c_int, [POINTER(c_void_p), c_double, c_int, c_int]),
    ("fdmgpu_server_submit_solve", c_int,
     [c_void_p, POINTER(c_ulonglong), POINTER(c_int), POINTER(c_double), POINTER(c_double), c_double, c_void_p,
      c_void_p]),
    ("fdmgpu_server_session_create", c_int, [c_void_p, POINTER(c_int), c_int, c_int] + [c_double] * 9),
    ("fdmgpu_server_submit_advance", c_int, [c_void_p, POINTER(c_ulonglong), c_int, c_int]),
    ("fdmgpu_server_poll", c_int,
     [c_void_p, c_ulonglong, POINTER(c_int), POINTER(c_int), POINTER(c_double), POINTER(c_double), POINTER(c_int),
      POINTER(c_double)]),
    ("fdmgpu_server_wait", c_int,
     [c_void_p, c_ulonglong, c_double, POINTER(c_int), POINTER(c_int), POINTER(c_double), POINTER(c_double),
      POINTER(c_int), POINTER(c_double)]),
    ("fdmgpu_server_next_done", c_int,
     [c_void_p, c_double, POINTER(c_ulonglong), POINTER(c_int), POINTER(c_int), POINTER(c_double),
      POINTER(c_double), POINTER(c_int), POINTER(c_double)]),
    ("fdmgpu_server_cancel", c_int, [c_void_p, c_ulonglong]),
    ("fdmgpu_server_session_get_field", c_int,
     [c_void_p, c_int, c_int, c_void_p, c_size_t, POINTER(c_longlong), c_double]),
    ("fdmgpu_server_session_close", c_int, [c_void_p, c_int, c_double]),
    ("fdmgpu_server_stats", c_int, [c_void_p, c_void_p]),
    ("fdmgpu_server_stats_reset", c_int, [c_void_p]),
    ("fdmgpu_server_set_admission", c_int, [c_void_p, c_int, c_double]),
    ("fdmgpu_server_destroy", c_int, [c_void_p]),
]

EXPORTED = [s[0] for s in _SIGS]

_lib = None


def load(path: Path | str | None = None):
    """Loads libfdmgpu.so once and declares every entry point.  Raises
    OSError when the library is missing or lacks a symbol."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OSError("libfdmgpu.so not built at %s; run __graft_entry__.build()" % p)
    lib = ctypes.CDLL(str(p))
    for name, res, args in _SIGS:
        fn = getattr(lib, name)  # AttributeError -> missing export
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().fdmgpu_last_error()
        raise FdmError(status, msg.decode() if msg else "")


def launch_count() -> int:
    return int(load().fdmgpu_launch_count())


def profile_enable(on: bool = True) -> None:
    check(load().fdmgpu_profile_enable(1 if on else 0))


def profile_reset() -> None:
    check(load().fdmgpu_profile_reset())


def profile_collect() -> dict:
    """{kernel name: (launches, total ms)} of the launches timed so far."""
    lib = load()
    n = c_int()
    check(lib.fdmgpu_profile_collect(ctypes.byref(n)))
    out = {}
    for i in range(n.value):
        buf = ctypes.create_string_buffer(64)
        cnt = c_longlong()
        ms = c_double()
        check(lib.fdmgpu_profile_entry(i, buf, 64, ctypes.byref(cnt), ctypes.byref(ms)))
        out[buf.value.decode()] = (cnt.value, ms.value)
    return out
