"""Host-side mirror of the reference's fast Poisson solvers.

`LaplCube`, `LaplRect` and `LaplRectFFT2` keep the reference constructors and
`solve(ans, rhs)` (src/lapl_cube.h:58-102, src/lapl_rect.h:40-68, 89-105):
arrays hold the interior points, x fastest; `ans` is overwritten; `rhs` is
read only.  The work runs in libfdmgpu.so on the GPU; sizes the reference
rejects with verify() raise `FdmError` with status ESIZE here.

`solve_device` takes CUDA tensors (or raw device addresses) and batches
`nrhs` volumes stored back to back.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int, c_size_t, c_void_p

import numpy as np

from . import _native as N


def _dtype_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.float64:
        return N.F64
    if dt == np.float32:
        return N.F32
    raise N.FdmError(N.EINVAL, "dtype must be float64 or float32, got %s" % dt)


def _host_ptr(a: np.ndarray, dtype, count: int, writable: bool) -> int:
    if not isinstance(a, np.ndarray):
        raise N.FdmError(N.EINVAL, "expected a numpy array")
    if a.dtype != np.dtype(dtype) or not a.flags.c_contiguous or a.size != count:
        raise N.FdmError(N.EINVAL, "array must be C-contiguous %s with %d elements" % (np.dtype(dtype), count))
    if writable and not a.flags.writeable:
        raise N.FdmError(N.EINVAL, "output array is read-only")
    return a.ctypes.data


def _dev_ptr(t, elem_bytes: int, count: int) -> int:
    """Device address of a CUDA tensor (checked) or a raw integer address."""
    if isinstance(t, int):
        return t
    if not getattr(t, "is_cuda", False):
        raise N.FdmError(N.EINVAL, "expected a CUDA tensor")
    if not t.is_contiguous() or t.numel() < count or t.element_size() != elem_bytes:
        raise N.FdmError(N.EINVAL, "tensor must be contiguous with >= %d elements of %d bytes" % (count, elem_bytes))
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        try:
            import torch
            return torch.cuda.current_stream().cuda_stream or None
        except Exception:
            return None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


class LaplCube:
    """3-D Dirichlet Poisson solver, fdm::LaplCube<T,check,F> (src/lapl_cube.h:9-106).

    precision: "plain" (every stage in `dtype`) or "mixed" (float64 arrays;
    FP32 inner solves with refinement to `tol`).  adaptive: after the sweeps
    `tol` asks for, run further sweeps (up to max_sweeps) while a right-hand
    side's estimated remaining error exceeds `tol` (the solve then waits for
    the device).
    """

    def __init__(self, dx, dy, dz, lx, ly, lz, nx, ny, nz, dtype=np.float64, precision="plain",
                 tol=1e-10, max_sweeps=3, periodic=False, adaptive=False):
        self._lib = N.load()
        self.dtype = np.dtype(dtype)
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.dx, self.dy, self.dz = float(dx), float(dy), float(dz)
        self.lx, self.ly, self.lz = float(lx), float(ly), float(lz)
        self.count = self.nx * self.ny * self.nz
        h = c_void_p()
        flags = 7 if periodic else 0
        N.check(self._lib.fdmgpu_lapl_cube_create(byref(h), _dtype_code(dtype), flags, self.dx, self.dy, self.dz,
                                                  self.lx, self.ly, self.lz, self.nx, self.ny, self.nz))
        self._h = h
        self.precision = precision
        if precision not in ("plain", "mixed"):
            raise N.FdmError(N.EINVAL, "precision must be 'plain' or 'mixed'")
        N.check(self._lib.fdmgpu_lapl_cube_set_precision(self._h, N.MIXED if precision == "mixed" else N.PLAIN,
                                                         float(tol), int(max_sweeps)))
        if adaptive:
            N.check(self._lib.fdmgpu_lapl_cube_set_refinement(self._h, 1))

    def solve(self, ans: np.ndarray, rhs: np.ndarray) -> None:
        """ans <- solution for rhs (host arrays, synchronous)."""
        pa = _host_ptr(ans, self.dtype, self.count, True)
        pr = _host_ptr(np.ascontiguousarray(rhs), self.dtype, self.count, False)
        N.check(self._lib.fdmgpu_lapl_cube_solve(self._h, pa, pr))

    def solve_batch(self, ans, rhs, nrhs: int) -> None:
        """Host solve of nrhs volumes stored back to back (synchronous).
        ans / rhs: numpy arrays or CPU tensors (pinned memory is fastest)."""
        cnt = self.count * nrhs
        if hasattr(ans, "data_ptr"):
            if ans.is_cuda or rhs.is_cuda or ans.numel() != cnt or rhs.numel() != cnt:
                raise N.FdmError(N.EINVAL, "expected CPU tensors with %d elements" % cnt)
            pa, pr = ans.data_ptr(), rhs.data_ptr()
        else:
            pa = _host_ptr(ans, self.dtype, cnt, True)
            pr = _host_ptr(rhs, self.dtype, cnt, False)
        N.check(self._lib.fdmgpu_lapl_cube_solve_host_batch(self._h, pa, pr, int(nrhs)))

    def solve_device(self, ans, rhs, nrhs: int = 1, stream=None) -> None:
        """Device solve of nrhs volumes stored back to back (asynchronous)."""
        eb = self.dtype.itemsize
        N.check(self._lib.fdmgpu_lapl_cube_solve_device(self._h, _dev_ptr(ans, eb, self.count * nrhs),
                                                        _dev_ptr(rhs, eb, self.count * nrhs), int(nrhs),
                                                        _stream_ptr(stream)))

    def set_schedule(self, ztable: bool = True, dst_tc=False) -> None:
        """Mixed-form schedule: per-mode z factor table (default) or factors
        per solve; plain FP32 DST passes of 32/64/128-point axes on the
        tensor cores or as FFTs (default).  dst_tc: True for both axes, or a
        mask (1 = x, 2 = y)."""
        mask = 3 if dst_tc is True else int(dst_tc)
        N.check(self._lib.fdmgpu_lapl_cube_set_schedule(self._h, int(bool(ztable)), mask))

    def tune(self, ans, rhs, nrhs: int = 1, stream=None) -> float:
        """Times every mixed-form schedule (pipeline, z-solve variant,
        tensor-core axes) on these device arrays and keeps the fastest whose
        accuracy is assured; returns its time per call in ms."""
        eb = self.dtype.itemsize
        ms = c_double()
        N.check(self._lib.fdmgpu_lapl_cube_tune(self._h, _dev_ptr(ans, eb, self.count * nrhs),
                                                _dev_ptr(rhs, eb, self.count * nrhs), int(nrhs),
                                                _stream_ptr(stream), byref(ms)))
        return ms.value

    def schedule(self) -> dict:
        """The mixed form's schedule: pipeline asked for ('planes' or
        'five_pass'), table-driven z-solve, tensor-core axes (bit 0 x, 1 y)."""
        p, z, t = c_int(), c_int(), c_int()
        N.check(self._lib.fdmgpu_lapl_cube_get_schedule(self._h, byref(p), byref(z), byref(t)))
        return {"pipeline": "planes" if p.value == 1 else "five_pass", "ztable": bool(z.value), "dst_tc": t.value}

    def set_pipeline(self, planes: bool = True) -> None:
        """Mixed-form pass structure: the fused x-z plane pass between two
        DSTs along y (default, where the sizes allow it) or the five passes
        x, y, z, y, x."""
        N.check(self._lib.fdmgpu_lapl_cube_set_pipeline(self._h, 1 if planes else 0))

    def pipeline_in_use(self) -> str:
        """'planes' or 'five_pass': what a solve of this handle runs."""
        p = c_int()
        N.check(self._lib.fdmgpu_lapl_cube_pipeline_in_use(self._h, byref(p)))
        return "planes" if p.value == 1 else "five_pass"

    def device_failed(self) -> bool:
        """True if a tensor-core pass of this solver gave up waiting for its
        MMAs (synchronises the device)."""
        f = c_int()
        N.check(self._lib.fdmgpu_lapl_cube_device_status(self._h, byref(f)))
        return bool(f.value)

    def last_info(self, nrhs: int = 1):
        """(sweeps, [estimated relative error left per RHS]); -1 without a sweep."""
        s = c_int()
        est = (c_double * nrhs)()
        N.check(self._lib.fdmgpu_lapl_cube_last_info(self._h, byref(s), est, int(nrhs)))
        return s.value, list(est)

    def scratch_bytes(self) -> int:
        b = c_size_t()
        N.check(self._lib.fdmgpu_lapl_cube_scratch_bytes(self._h, byref(b)))
        return b.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_lapl_cube_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Many right-hand sides of uneven sizes solved by one graph launch.

    shapes: one (nx, ny, nz) per right-hand side; spacings / lengths: one
    (dx, dy, dz) / (lx, ly, lz) per right-hand side, or None for h = 1/(n+1),
    l = 1 on every axis.  Right-hand sides of equal geometry share a plan;
    each group's schedule is timed on the caller's data by `tune` and every
    `solve` after that replays one captured CUDA graph.  The reference solves
    these one LaplCube at a time (src/lapl_cube.h:58-102).
    """

    def __init__(self, shapes, spacings=None, lengths=None, precision="mixed", tol=1e-10):
        self._lib = N.load()
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        self.count = len(self.shapes)
        if spacings is None:
            spacings = [tuple(1.0 / (n + 1) for n in s) for s in self.shapes]
        if lengths is None:
            lengths = [(1.0, 1.0, 1.0)] * self.count
        if len(spacings) != self.count or len(lengths) != self.count:
            raise N.FdmError(N.EINVAL, "one spacing and one length triple per right-hand side")
        if precision not in ("plain", "mixed"):
            raise N.FdmError(N.EINVAL, "precision must be 'plain' or 'mixed'")
        n3 = (c_int * (3 * self.count))(*[v for s in self.shapes for v in s])
        h3 = (c_double * (3 * self.count))(*[float(v) for s in spacings for v in s])
        l3 = (c_double * (3 * self.count))(*[float(v) for s in lengths for v in s])
        h = c_void_p()
        N.check(self._lib.fdmgpu_batch_create(byref(h), self.count, n3, h3, l3,
                                              N.MIXED if precision == "mixed" else N.PLAIN, float(tol)))
        self._h = h

    def _ptrs(self, ans, rhs):
        if len(ans) != self.count or len(rhs) != self.count:
            raise N.FdmError(N.EINVAL, "expected %d volumes" % self.count)
        pa = (c_void_p * self.count)()
        pr = (c_void_p * self.count)()
        for i, (nx, ny, nz) in enumerate(self.shapes):
            pa[i] = _dev_ptr(ans[i], 8, nx * ny * nz)
            pr[i] = _dev_ptr(rhs[i], 8, nx * ny * nz)
        return pa, pr

    def tune(self, ans, rhs) -> None:
        """Times each group's schedules on these volumes (device FP64) and
        keeps the fastest; overwrites ans."""
        pa, pr = self._ptrs(ans, rhs)
        N.check(self._lib.fdmgpu_batch_tune(self._h, pa, pr))

    def solve(self, ans, rhs, stream=None) -> None:
        """ans[i] <- solution for rhs[i], all i (device FP64, asynchronous)."""
        pa, pr = self._ptrs(ans, rhs)
        N.check(self._lib.fdmgpu_batch_solve(self._h, pa, pr, _stream_ptr(stream)))

    def info(self):
        """(groups, kernel launches replayed per solve)."""
        g, l = c_int(), c_int()
        N.check(self._lib.fdmgpu_batch_info(self._h, byref(g), byref(l)))
        return g.value, l.value

    def schedule(self):
        """Per group: dict(shape, members, chunk, ztable, dst_tc, tuned_ms)."""
        out = []
        for k in range(self.info()[0]):
            n3 = (c_int * 3)()
            m, ch, zt, tc = c_int(), c_int(), c_int(), c_int()
            ms = c_double()
            N.check(self._lib.fdmgpu_batch_schedule(self._h, k, n3, byref(m), byref(ch), byref(zt), byref(tc),
                                                    byref(ms)))
            out.append(dict(shape=tuple(n3), members=m.value, chunk=ch.value, ztable=zt.value, dst_tc=tc.value,
                            tuned_ms=ms.value))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LaplCyl3FFT2:
    """Poisson in a cylindrical annulus, fdm::LaplCyl3FFT2<T,check,zflag>
    (src/lapl_cyl.h:178-262, src/lapl_cyl.cpp:10-166): arrays shaped
    (nphi, nz, nr), r fastest; phi periodic, z Dirichlet or periodic."""

    def __init__(self, dr, dz, r0, lr, lz, nr, nz, nphi, dtype=np.float64, periodic_z=False):
        self._lib = N.load()
        self.dtype = np.dtype(dtype)
        self.nr, self.nz, self.nphi = int(nr), int(nz), int(nphi)
        self.count = self.nr * self.nz * self.nphi
        h = c_void_p()
        N.check(self._lib.fdmgpu_lapl_cyl_create(byref(h), _dtype_code(dtype), int(bool(periodic_z)), float(dr),
                                                 float(dz), float(r0), float(lr), float(lz), self.nr, self.nz,
                                                 self.nphi))
        self._h = h

    def solve(self, ans: np.ndarray, rhs: np.ndarray) -> None:
        pa = _host_ptr(ans, self.dtype, self.count, True)
        pr = _host_ptr(np.ascontiguousarray(rhs), self.dtype, self.count, False)
        N.check(self._lib.fdmgpu_lapl_cyl_solve(self._h, pa, pr))

    def solve_device(self, ans, rhs, nrhs: int = 1, stream=None) -> None:
        eb = self.dtype.itemsize
        N.check(self._lib.fdmgpu_lapl_cyl_solve_device(self._h, _dev_ptr(ans, eb, self.count * nrhs),
                                                       _dev_ptr(rhs, eb, self.count * nrhs), int(nrhs),
                                                       _stream_ptr(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_lapl_cyl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LaplRect:
    """2-D Poisson solver, fdm::LaplRect<T,check,F>: DST (or, y periodic, the
    periodic transform) along y, tridiagonal solve along x per y-mode
    (src/lapl_rect.cpp:63-110).  periodic_y / periodic_x are the template's
    flags (F::head, F::tail::head); periodic=True sets both."""

    _method = N.RECT_TRIDIAG

    def __init__(self, dx, dy, lx, ly, nx, ny, dtype=np.float64, periodic=False, periodic_y=False,
                 periodic_x=False):
        if periodic:
            periodic_y = periodic_x = True
        flags = (2 if periodic_y else 0) | (1 if periodic_x else 0)
        self._lib = N.load()
        self.dtype = np.dtype(dtype)
        self.nx, self.ny = int(nx), int(ny)
        self.count = self.nx * self.ny
        h = c_void_p()
        N.check(self._lib.fdmgpu_lapl_rect_create_flags(byref(h), _dtype_code(dtype), self._method, flags, float(dx),
                                                        float(dy), float(lx), float(ly), self.nx, self.ny))
        self._h = h

    def solve(self, ans: np.ndarray, rhs: np.ndarray) -> None:
        pa = _host_ptr(ans, self.dtype, self.count, True)
        pr = _host_ptr(np.ascontiguousarray(rhs), self.dtype, self.count, False)
        N.check(self._lib.fdmgpu_lapl_rect_solve(self._h, pa, pr))

    def solve_device(self, ans, rhs, nrhs: int = 1, stream=None) -> None:
        eb = self.dtype.itemsize
        N.check(self._lib.fdmgpu_lapl_rect_solve_device(self._h, _dev_ptr(ans, eb, self.count * nrhs),
                                                        _dev_ptr(rhs, eb, self.count * nrhs), int(nrhs),
                                                        _stream_ptr(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_lapl_rect_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LaplRectFFT2(LaplRect):
    """2-D Poisson solver with transforms on both axes (DST, or the periodic
    transform on a periodic axis), fdm::LaplRectFFT2 (src/lapl_rect.cpp:113-207)."""

    _method = N.RECT_FFT2


def sine_transform_device(out, inp, N_points: int, nlines: int, scale: float = 1.0, dtype=np.float64,
                          stream=None) -> None:
    """DST-I of nlines contiguous lines of N-1 values on the device
    (FFT<T>::sFFT, src/fft.cpp:294-365, on entries 1..N-1)."""
    lib = N.load()
    eb = np.dtype(dtype).itemsize
    cnt = (N_points - 1) * nlines
    N.check(lib.fdmgpu_sine_device(_dtype_code(dtype), int(N_points), int(nlines), float(scale),
                                   _dev_ptr(out, eb, cnt), _dev_ptr(inp, eb, cnt), _stream_ptr(stream)))


def pfft_1_3d(S: np.ndarray, s: np.ndarray, dx: float) -> None:
    """FFT<T>::pFFT_1_3d (src/fft.cpp:254-292): the periodic forward transform
    of an N^3 host cube (N a power of two) along x, y, z, scale dx, into S."""
    _pfft3d_host(S, s, dx, 0)


def pfft_3d(S: np.ndarray, s: np.ndarray, dx: float) -> None:
    """FFT<T>::pFFT_3d (src/fft.cpp:214-251): the inverse layout, into S."""
    _pfft3d_host(S, s, dx, 1)


def _pfft3d_host(S, s, dx, inverse):
    lib = N.load()
    n = round(s.size ** (1.0 / 3.0))
    if n ** 3 != s.size or S.size != s.size or S.dtype != s.dtype:
        raise ValueError("pFFT_3d works on matching N^3 arrays")
    if not (s.flags.c_contiguous and S.flags.c_contiguous):
        raise ValueError("arrays must be C-contiguous")
    N.check(lib.fdmgpu_pfft3d(_dtype_code(s.dtype), int(n), int(inverse), float(dx), S.ctypes.data, s.ctypes.data))


def pfft_device(out, inp, N_points: int, nlines: int, dx: float = 1.0, inverse: bool = False, dtype=np.float64,
                stream=None) -> None:
    """FFT<T>::pFFT_1 (inverse False) / pFFT of nlines contiguous lines of
    N_points values on the device (src/fft.cpp:108-212)."""
    lib = N.load()
    eb = np.dtype(dtype).itemsize
    cnt = N_points * nlines
    N.check(lib.fdmgpu_pfft_device(_dtype_code(dtype), int(N_points), int(bool(inverse)), int(nlines), float(dx),
                                   _dev_ptr(out, eb, cnt), _dev_ptr(inp, eb, cnt), _stream_ptr(stream)))


def pfft3d_device(out, inp, n: int, dx: float, inverse: bool = False, count: int = 1, dtype=np.float64,
                  stream=None) -> None:
    """pFFT_1_3d / pFFT_3d of `count` device cubes of n^3 back to back,
    asynchronous on stream."""
    lib = N.load()
    eb = np.dtype(dtype).itemsize
    cnt = n * n * n * count
    N.check(lib.fdmgpu_pfft3d_device(_dtype_code(dtype), int(n), int(bool(inverse)), float(dx),
                                     _dev_ptr(out, eb, cnt), _dev_ptr(inp, eb, cnt), int(count), _stream_ptr(stream)))


def sine_transform_tc_device(out, inp, N_points: int, count: int, scale: float = 1.0, axis: int = 0, nx: int = 1,
                             stream=None) -> None:
    """FP32 DST-I on the tensor cores (N_points = 32, 64 or 128).  axis 0: `count`
    contiguous lines of N-1 values; axis 1: `count` planes of (N-1) x nx
    values transformed along their rows (stride nx).  Synchronous."""
    lib = N.load()
    cnt = (N_points - 1) * count * (nx if axis == 1 else 1)
    N.check(lib.fdmgpu_sine_tc_device(int(N_points), int(axis), int(nx), int(count), float(scale),
                                      _dev_ptr(out, 4, cnt), _dev_ptr(inp, 4, cnt), _stream_ptr(stream)))


def tridiag_device(lower, diag, upper, b, n: int, nsys: int, dtype=np.float64, stream=None) -> None:
    """Solves nsys tridiagonal systems in place in b (system-interleaved
    layout, element i of system s at [i*nsys + s])."""
    lib = N.load()
    eb = np.dtype(dtype).itemsize
    cnt = n * nsys
    N.check(lib.fdmgpu_tridiag_device(_dtype_code(dtype), int(n), int(nsys), _dev_ptr(lower, eb, cnt),
                                      _dev_ptr(diag, eb, cnt), _dev_ptr(upper, eb, cnt), _dev_ptr(b, eb, cnt),
                                      _stream_ptr(stream)))
