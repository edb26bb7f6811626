"""Serving loop: Poisson solves and resident NSCube sessions behind one
scheduler (libfdmgpu.so, fdmgpu_server_*).

Requests are admitted first come first served while their device memory
fits under the budget, run concurrently on `lanes` CUDA streams, and
same-geometry solves that wait together share one launch (continuous
batching).  Solve buffers are page-locked host memory (numpy arrays are
registered by `pinned_empty`, or pinned CPU tensors).  The reference has no
serving layer: it solves one LaplCube (src/lapl_cube.h:58-102) or steps one
NSCube (src/ns_cube.cpp:27-62) on the caller's thread.
"""
from __future__ import annotations

import math
from ctypes import byref, c_double, c_int, c_longlong, c_ulonglong, c_void_p

import numpy as np

from . import _native as N

_FIELDS = {"u": 0, "v": 1, "w": 2, "p": 3, "x": 4, "F": 5, "G": 6, "H": 7, "RHS": 8}
STATE_NAMES = {N.REQ_QUEUED: "queued", N.REQ_RUNNING: "running", N.REQ_DONE: "done", N.REQ_FAILED: "failed",
               N.REQ_CANCELLED: "cancelled"}


def _ptr(a, count: int, writable: bool) -> int:
    if hasattr(a, "data_ptr"):
        if a.is_cuda or not a.is_contiguous() or a.numel() != count or a.element_size() != 8:
            raise N.FdmError(N.EINVAL, "expected a contiguous float64 CPU tensor of %d elements" % count)
        return a.data_ptr()
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous or a.size != count:
        raise N.FdmError(N.EINVAL, "expected a C-contiguous float64 array of %d elements" % count)
    if writable and not a.flags.writeable:
        raise N.FdmError(N.EINVAL, "output array is read-only")
    return a.ctypes.data


class Server:
    """A serving loop with a device-memory budget (bytes), `lanes`
    concurrent launches and up to `max_batch` solves per launch."""

    def __init__(self, budget_bytes: float = 150e9, lanes: int = 8, max_batch: int = 8):
        self._lib = N.load()
        h = c_void_p()
        N.check(self._lib.fdmgpu_server_create(byref(h), float(budget_bytes), int(lanes), int(max_batch)))
        self._h = h
        self._sessions = {}

    # ---- requests
    def submit_solve(self, ans, rhs, shape, spacings=None, lengths=None, tol: float = 1e-10) -> int:
        """Queues ans <- solution for rhs on the (nz, ny, nx) interior grid
        `shape` = (nx, ny, nz); spacings/lengths default to h = 1/(n+1),
        l = 1.  tol <= 0: plain FP64; otherwise mixed with refinement."""
        nx, ny, nz = (int(v) for v in shape)
        cnt = nx * ny * nz
        if spacings is None:
            spacings = (1.0 / (nx + 1), 1.0 / (ny + 1), 1.0 / (nz + 1))
        if lengths is None:
            lengths = (1.0, 1.0, 1.0)
        rid = c_ulonglong()
        N.check(self._lib.fdmgpu_server_submit_solve(
            self._h, byref(rid), (c_int * 3)(nx, ny, nz), (c_double * 3)(*map(float, spacings)),
            (c_double * 3)(*map(float, lengths)), float(tol), _ptr(rhs, cnt, False), _ptr(ans, cnt, True)))
        return rid.value

    def session_create(self, nx: int = 63, nz: int = 63, Re: float = 250.0, dt: float = 0.01, u0: float = 1.0,
                       box=(-math.pi, -math.pi, -math.pi, math.pi, math.pi, math.pi)) -> int:
        """A resident lid-driven cavity (fdm::NSCube, FP64) on the device."""
        sid = c_int()
        N.check(self._lib.fdmgpu_server_session_create(self._h, byref(sid), int(nx), int(nz), *map(float, box),
                                                       float(u0), float(Re), float(dt)))
        self._sessions[sid.value] = (int(nx), int(nz))
        return sid.value

    def submit_advance(self, session: int, steps: int) -> int:
        rid = c_ulonglong()
        N.check(self._lib.fdmgpu_server_submit_advance(self._h, byref(rid), int(session), int(steps)))
        return rid.value

    @staticmethod
    def _record(rid, state, status, lat, queue, batch, est):
        return {"id": rid, "state": STATE_NAMES[state.value], "status": status.value, "latency_ms": lat.value,
                "queue_ms": queue.value, "batch": batch.value, "err_est": est.value}

    def _out(self):
        return c_int(), c_int(), c_double(), c_double(), c_int(), c_double()

    def poll(self, rid: int) -> dict:
        """State of a request; a finished one is reported once.  err_est: a
        finished mixed solve's estimated relative error (0 for FP64, -1
        otherwise)."""
        st, status, lat, q, b, e = self._out()
        N.check(self._lib.fdmgpu_server_poll(self._h, int(rid), byref(st), byref(status), byref(lat), byref(q),
                                             byref(b), byref(e)))
        return self._record(rid, st, status, lat, q, b, e)

    def wait(self, rid: int, timeout_ms: float = 60000.0) -> dict:
        st, status, lat, q, b, e = self._out()
        N.check(self._lib.fdmgpu_server_wait(self._h, int(rid), float(timeout_ms), byref(st), byref(status),
                                             byref(lat), byref(q), byref(b), byref(e)))
        return self._record(rid, st, status, lat, q, b, e)

    def next_done(self, timeout_ms: float = 1000.0):
        """The next finished request, or None after timeout_ms."""
        rid = c_ulonglong()
        st, status, lat, q, b, e = self._out()
        rc = self._lib.fdmgpu_server_next_done(self._h, float(timeout_ms), byref(rid), byref(st), byref(status),
                                               byref(lat), byref(q), byref(b), byref(e))
        if rc == N.ETIMEOUT:
            return None
        N.check(rc)
        return self._record(rid.value, st, status, lat, q, b, e)

    def cancel(self, rid: int) -> None:
        N.check(self._lib.fdmgpu_server_cancel(self._h, int(rid)))

    # ---- sessions
    def session_field(self, session: int, name: str, timeout_ms: float = 60000.0):
        """(field storage as a flat array, steps advanced so far), read once
        the session's queued advances are done."""
        nx, nz = self._sessions[session]
        ny = nx
        ext = {"u": (nz + 2, ny + 2, nx + 3), "v": (nz + 2, ny + 3, nx + 2), "w": (nz + 3, ny + 2, nx + 2),
               "p": (nz + 2, ny + 2, nx + 2), "x": (nz, ny, nx)}[name]
        out = np.empty(ext)
        steps = c_longlong()
        N.check(self._lib.fdmgpu_server_session_get_field(self._h, int(session), _FIELDS[name], out.ctypes.data,
                                                          out.size, byref(steps), float(timeout_ms)))
        return out, steps.value

    def session_close(self, session: int, timeout_ms: float = 60000.0) -> None:
        N.check(self._lib.fdmgpu_server_session_close(self._h, int(session), float(timeout_ms)))
        self._sessions.pop(session, None)

    # ---- accounting
    def stats(self) -> dict:
        s = N.ServerStats()
        N.check(self._lib.fdmgpu_server_stats(self._h, byref(s)))
        return s.as_dict()

    def stats_reset(self) -> None:
        N.check(self._lib.fdmgpu_server_stats_reset(self._h))

    def set_admission(self, max_queued: int = 0, max_wait_ms: float = 0.0) -> None:
        """Load shedding: submits beyond max_queued queued requests raise
        FdmError(EBUSY); requests not started within max_wait_ms finish as
        failed with status EBUSY.  0 turns either limit off."""
        N.check(self._lib.fdmgpu_server_set_admission(self._h, int(max_queued), float(max_wait_ms)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
