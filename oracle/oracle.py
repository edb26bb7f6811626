"""Test infrastructure, not product code.

ctypes loaders for the two CPU checkers:
  * `port()`      -> oracle/liboracle.so, the C restatement (fdm_oracle.c),
                     built on every machine;
  * `reference()` -> oracle/_ref/libfdm_ref.so, the reference's own sources
                     compiled by oracle/Makefile, present only where the
                     reference tree was available at build time (None
                     otherwise).
Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
them, as checkers or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_long, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_dp = POINTER(c_double)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Port:
    """The C restatement (fdm_oracle.h)."""

    def __init__(self, path: Path = HERE / "liboracle.so"):
        L = ctypes.CDLL(str(path))
        L.orc_set_threads.argtypes = [c_int]
        L.orc_get_threads.restype = c_int
        L.orc_sfft.argtypes = [_dp, _dp, c_double, c_int]
        L.orc_sfft.restype = c_int
        L.orc_sft_naive.argtypes = [_dp, _dp, c_double, c_int]
        L.orc_lapl_cube_solve.argtypes = [c_int] * 3 + [c_double] * 6 + [_dp, _dp]
        L.orc_lapl_cube_solve.restype = c_int
        L.orc_lapl_rect_solve.argtypes = [c_int] * 2 + [c_double] * 4 + [_dp, _dp]
        L.orc_lapl_rect_solve.restype = c_int
        L.orc_lapl_rect_fft2_solve.argtypes = [c_int] * 2 + [c_double] * 4 + [_dp, _dp]
        L.orc_lapl_rect_fft2_solve.restype = c_int
        L.orc_cyclic_reduction.argtypes = [_dp, _dp, _dp, _dp, c_int, c_int, c_int]
        L.orc_thomas.argtypes = [_dp, _dp, _dp, _dp, c_int]
        L.orc_ns_create.restype = c_void_p
        L.orc_ns_create.argtypes = [c_int, c_int] + [c_double] * 9
        L.orc_ns_step.argtypes = [c_void_p, c_int]
        L.orc_ns_get.restype = c_long
        L.orc_ns_get.argtypes = [c_void_p, c_int, _dp]
        L.orc_ns_set.argtypes = [c_void_p, c_int, _dp]
        L.orc_ns_destroy.argtypes = [c_void_p]
        self.L = L

    def set_threads(self, n: int) -> None:
        self.L.orc_set_threads(int(n))

    def threads(self) -> int:
        return self.L.orc_get_threads()

    def sfft(self, s: np.ndarray, dx: float = 1.0) -> np.ndarray:
        N = s.size
        S = np.zeros(N)
        a = np.ascontiguousarray(s, np.float64).copy()
        if self.L.orc_sfft(_p(S), _p(a), float(dx), N):
            raise ValueError("N must be a power of two")
        return S

    def sft_naive(self, s: np.ndarray, dx: float = 1.0) -> np.ndarray:
        S = np.zeros(s.size)
        self.L.orc_sft_naive(_p(S), _p(np.ascontiguousarray(s, np.float64)), float(dx), s.size)
        return S

    def lapl_cube(self, rhs, dx, dy, dz, lx, ly, lz) -> np.ndarray:
        nz, ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        if self.L.orc_lapl_cube_solve(nx, ny, nz, dx, dy, dz, lx, ly, lz, _p(ans), _p(r)):
            raise ValueError("bad size")
        return ans

    def lapl_rect(self, rhs, dx, dy, lx, ly, fft2: bool = False) -> np.ndarray:
        ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        fn = self.L.orc_lapl_rect_fft2_solve if fft2 else self.L.orc_lapl_rect_solve
        if fn(nx, ny, dx, dy, lx, ly, _p(ans), _p(r)):
            raise ValueError("bad size")
        return ans

    def thomas(self, lower, diag, upper, b) -> np.ndarray:
        """lower[j] = A(j+1, j), upper[j] = A(j, j+1) (length n-1 used)."""
        l, d, u, x = (np.array(v, np.float64) for v in (lower, diag, upper, b))
        self.L.orc_thomas(_p(x), _p(l), _p(d), _p(u), x.size)
        return x

    def cyclic_reduction(self, d, e, f, b, general: bool) -> np.ndarray:
        d, e, f, x = (np.array(v, np.float64) for v in (d, e, f, b))
        n = x.size
        q = int(np.ceil(np.log2(n + 1)))
        self.L.orc_cyclic_reduction(_p(d), _p(e), _p(f), _p(x), q, n, 1 if general else 0)
        return x

    def nscube(self, nx, nz, Re, dt, u0=1.0, box=(-np.pi, -np.pi, -np.pi, np.pi, np.pi, np.pi)):
        return _NS(self.L, self.L.orc_ns_create(nx, nz, Re, dt, u0, *box), "orc")


class _NS:
    FIELDS = ("u", "v", "w", "p", "x", "F", "G", "H", "RHS")

    def __init__(self, L, h, kind):
        self.L, self.h, self.kind = L, h, kind
        if not h:
            raise ValueError("bad size")

    def _fn(self, what):
        return getattr(self.L, {"orc": "orc_ns_", "ref": "ref_nscube_", "reff": "ref_nscubef_"}[self.kind] + what)

    def step(self, k: int = 1) -> None:
        self._fn("step")(self.h, int(k))

    def get(self, name: str) -> np.ndarray:
        fid = self.FIELDS.index(name)
        getter = self._fn("get")
        n = getter(self.h, fid, None)
        out = np.zeros(n)
        getter(self.h, fid, _p(out))
        return out

    def close(self):
        if self.h:
            self._fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Reference:
    """The reference's own CPU code (oracle/_ref/libfdm_ref.so)."""

    def __init__(self, path: Path = HERE / "_ref" / "libfdm_ref.so"):
        L = ctypes.CDLL(str(path))
        L.ref_lapl_cube_solve_d.argtypes = [c_int] * 3 + [c_double] * 6 + [c_int, _dp, _dp, c_int]
        L.ref_lapl_rect_solve_d.argtypes = [c_int] * 2 + [c_double] * 4 + [c_int, _dp, _dp]
        L.ref_sfft_d.argtypes = [_dp, _dp, c_double, c_int]
        L.ref_cyclic_reduction_d.argtypes = [_dp, _dp, _dp, _dp, c_int, c_int, c_int]
        L.ref_thomas_d.argtypes = [_dp, _dp, _dp, _dp, c_int]
        L.ref_nscube_create.restype = c_void_p
        L.ref_nscube_create.argtypes = [c_int, c_int] + [c_double] * 9
        L.ref_nscube_step.argtypes = [c_void_p, c_int]
        L.ref_nscube_get.restype = c_long
        L.ref_nscube_get.argtypes = [c_void_p, c_int, _dp]
        L.ref_nscube_destroy.argtypes = [c_void_p]
        L.ref_nscubef_create.restype = c_void_p
        L.ref_nscubef_create.argtypes = [c_int, c_int] + [c_double] * 9
        L.ref_nscubef_step.argtypes = [c_void_p, c_int]
        L.ref_nscubef_get.restype = c_long
        L.ref_nscubef_get.argtypes = [c_void_p, c_int, _dp]
        L.ref_nscubef_destroy.argtypes = [c_void_p]
        self.L = L

    def sfft(self, s: np.ndarray, dx: float = 1.0) -> np.ndarray:
        S = np.zeros(s.size)
        a = np.array(s, np.float64)
        self.L.ref_sfft_d(_p(S), _p(a), float(dx), s.size)
        return S

    def lapl_cube(self, rhs, dx, dy, dz, lx, ly, lz, reps: int = 1) -> np.ndarray:
        nz, ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        self.L.ref_lapl_cube_solve_d(nx, ny, nz, dx, dy, dz, lx, ly, lz, 0, _p(ans), _p(r), int(reps))
        return ans

    def lapl_rect(self, rhs, dx, dy, lx, ly, fft2: bool = False) -> np.ndarray:
        ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        self.L.ref_lapl_rect_solve_d(nx, ny, dx, dy, lx, ly, 1 if fft2 else 0, _p(ans), _p(r))
        return ans

    def thomas(self, lower, diag, upper, b) -> np.ndarray:
        l, d, u, x = (np.array(v, np.float64) for v in (lower, diag, upper, b))
        self.L.ref_thomas_d(_p(x), _p(l), _p(d), _p(u), x.size)
        return x

    def cyclic_reduction(self, d, e, f, b, general: bool) -> np.ndarray:
        d, e, f, x = (np.array(v, np.float64) for v in (d, e, f, b))
        n = x.size
        q = int(np.ceil(np.log2(n + 1)))
        self.L.ref_cyclic_reduction_d(_p(d), _p(e), _p(f), _p(x), q, n, 1 if general else 0)
        return x

    def nscube(self, nx, nz, Re, dt, u0=1.0, box=(-np.pi, -np.pi, -np.pi, np.pi, np.pi, np.pi)):
        return _NS(self.L, self.L.ref_nscube_create(nx, nz, Re, dt, u0, *box), "ref")

    def nscube_float(self, nx, nz, Re, dt, u0=1.0, box=(-np.pi, -np.pi, -np.pi, np.pi, np.pi, np.pi)):
        """NSCube<float,false>; fields come back widened to float64."""
        return _NS(self.L, self.L.ref_nscubef_create(nx, nz, Re, dt, u0, *box), "reff")


_port = None
_ref = None


def vtk_text(u, v, w, nx, ny, nz, origin, spacing, time_index) -> str:
    """Restatement of velocity_plotter::vtk_out for a cube
    (src/velocity_plot.cpp:113-119, 200-217): header, then the cell-centred
    velocity 0.5(u[i][k][j]+u[i][k][j-1]), 0.5(v[i][k][j]+v[i][k-1][j]),
    0.5(w[i][k][j]+w[i-1][k][j]) of every interior cell, "%f %f %f", x
    fastest.  u, v, w are the NSCube field storages (flat or shaped) with
    the index ranges of src/ns_cube.h:64-66."""
    U = np.asarray(u, dtype=np.float64).reshape(nz + 2, ny + 2, nx + 3)   # z 0.., y 0.., x -1..
    V = np.asarray(v, dtype=np.float64).reshape(nz + 2, ny + 3, nx + 2)   # z 0.., y -1.., x 0..
    W = np.asarray(w, dtype=np.float64).reshape(nz + 3, ny + 2, nx + 2)   # z -1.., y 0.., x 0..
    out = ["# vtk DataFile Version 3.0", "step %d" % time_index, "ASCII", "DATASET STRUCTURED_POINTS",
           "DIMENSIONS %d %d %d" % (nx, ny, nz), "ASPECT_RATIO 1 1 1", "ORIGIN %f %f %f" % tuple(origin),
           "SPACING %f %f %f" % tuple(spacing), "POINT_DATA %d" % (nx * ny * nz), "VECTORS u double"]
    for i in range(1, nz + 1):
        for k in range(1, ny + 1):
            for j in range(1, nx + 1):
                out.append("%f %f %f" % (0.5 * (U[i, k, j + 1] + U[i, k, j]), 0.5 * (V[i, k + 1, j] + V[i, k, j]),
                                         0.5 * (W[i + 1, k, j] + W[i, k, j])))
    return "\n".join(out) + "\n"


def port() -> Port:
    global _port
    if _port is None:
        _port = Port()
    return _port


def reference():
    """The compiled reference, or None where it was not built."""
    global _ref
    if _ref is None:
        path = HERE / "_ref" / "libfdm_ref.so"
        if not path.exists():
            return None
        try:
            _ref = Reference(path)
        except OSError:
            return None
    return _ref
