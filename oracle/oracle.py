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

    def lapl_rect_flags(self, rhs, dx, dy, lx, ly, fft2: bool, flags: int) -> np.ndarray:
        """LaplRect(FFT2)<double,false,F> with F periodic in y (flags 2) or in
        y and x (flags 3)."""
        ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        if self.L.ref_lapl_rect_flags_d(nx, ny, dx, dy, lx, ly, 1 if fft2 else 0, flags, _p(ans), _p(r)):
            raise ValueError("flags %d not instantiated" % flags)
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
    FIELDS = ("u", "v", "w", "p", "x", "F", "G", "H", "RHS", "u0", "v0", "w0")

    def __init__(self, L, h, kind):
        self.L, self.h, self.kind = L, h, kind
        if not h:
            raise ValueError("bad size")

    def _fn(self, what):
        return getattr(self.L, {"orc": "orc_ns_", "ref": "ref_nscube_", "reff": "ref_nscubef_",
                                "cyl": "ref_nscyl_"}[self.kind] + what)

    def step(self, k: int = 1) -> None:
        self._fn("step")(self.h, int(k))

    def get(self, name: str) -> np.ndarray:
        fid = self.FIELDS.index(name)
        getter = self._fn("get")
        n = getter(self.h, fid, None)
        out = np.zeros(n)
        getter(self.h, fid, _p(out))
        return out

    def l_step(self, k: int = 1) -> None:
        """NSCyl::L_step (cylindrical reference only)."""
        self._fn("l_step")(self.h, int(k))

    def set(self, name: str, values) -> None:
        """Overwrites a whole field, ghosts included (cylindrical reference only)."""
        a = np.ascontiguousarray(values, np.float64).ravel()
        assert a.size == self._fn("get")(self.h, self.FIELDS.index(name), None)
        self._fn("set")(self.h, self.FIELDS.index(name), _p(a))

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
        L.ref_pfft1_d.argtypes = [_dp, _dp, c_double, c_int]
        L.ref_pfft_d.argtypes = [_dp, _dp, c_double, c_int]
        L.ref_pfft3d_d.argtypes = [_dp, _dp, c_double, c_int, c_int]
        L.ref_lapl_rect_flags_d.argtypes = [c_int] * 2 + [c_double] * 4 + [c_int] * 2 + [_dp, _dp]
        L.ref_lapl_cube_periodic_d.argtypes = [c_int] * 3 + [c_double] * 6 + [_dp, _dp]
        L.ref_lapl_cyl_d.argtypes = [c_int] * 4 + [c_double] * 5 + [_dp, _dp]
        L.ref_nscyl_create.restype = c_void_p
        L.ref_nscyl_create.argtypes = [c_int] + [c_double] * 7 + [c_int] * 3
        L.ref_nscyl_step.argtypes = [c_void_p, c_int]
        L.ref_nscyl_get.restype = c_long
        L.ref_nscyl_get.argtypes = [c_void_p, c_int, _dp]
        L.ref_nscyl_destroy.argtypes = [c_void_p]
        L.ref_nscyl_create_v.restype = c_void_p
        L.ref_nscyl_create_v.argtypes = [c_int] + [c_double] * 7 + [c_int] * 4
        L.ref_nscyl_l_step.argtypes = [c_void_p, c_int]
        L.ref_nscyl_set.restype = c_long
        L.ref_nscyl_set.argtypes = [c_void_p, c_int, _dp]
        L.ref_nscubef_create.restype = c_void_p
        L.ref_nscubef_create.argtypes = [c_int, c_int] + [c_double] * 9
        L.ref_nscubef_step.argtypes = [c_void_p, c_int]
        L.ref_config_get.argtypes = [ctypes.c_char_p, c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.c_char_p,
                                     ctypes.c_char_p, c_int, ctypes.c_char_p, _dp, ctypes.POINTER(c_int),
                                     ctypes.c_char_p, c_int]
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

    def pfft1(self, s: np.ndarray, dx: float = 1.0) -> np.ndarray:
        """FFT<double>::pFFT_1: values -> coefficients (src/fft.cpp:108)."""
        S = np.zeros(s.size)
        a = np.array(s, np.float64)
        self.L.ref_pfft1_d(_p(S), _p(a), dx, s.size)
        return S

    def pfft(self, s: np.ndarray, dx: float = 1.0) -> np.ndarray:
        """FFT<double>::pFFT: coefficients -> values (src/fft.cpp:195)."""
        S = np.zeros(s.size)
        a = np.array(s, np.float64)
        self.L.ref_pfft_d(_p(S), _p(a), dx, s.size)
        return S

    def pfft3d(self, s: np.ndarray, dx: float, inverse: bool = False) -> np.ndarray:
        """FFT<double>::pFFT_1_3d (inverse False) / pFFT_3d of an N^3 cube."""
        a = np.ascontiguousarray(s, np.float64)
        S = np.zeros_like(a)
        self.L.ref_pfft3d_d(_p(S), _p(a), dx, a.shape[0], 1 if inverse else 0)
        return S

    def config_get(self, path, argv, section: str, key: str, default):
        """Config::open(path), rewrite(argv), get(section, key, default)
        (src/config.cpp:78-150, 255-297) with the default's type."""
        kind = 2 if isinstance(default, str) else 1 if isinstance(default, int) else 0
        av = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
        d = np.zeros(1)
        i = c_int(0)
        buf = ctypes.create_string_buffer(4096)
        self.L.ref_config_get(str(path).encode(), len(argv), av, section.encode(), key.encode(), kind,
                              (default if kind == 2 else repr(default)).encode(), _p(d), ctypes.byref(i), buf, 4096)
        return buf.value.decode() if kind == 2 else int(i.value) if kind == 1 else float(d[0])

    def lapl_cube_periodic(self, rhs, dx, dy, dz, lx, ly, lz) -> np.ndarray:
        nz, ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        self.L.ref_lapl_cube_periodic_d(nx, ny, nz, dx, dy, dz, lx, ly, lz, _p(ans), _p(r))
        return ans

    def lapl_cyl(self, rhs, dr, dz, r0, lr, lz, periodic_z: bool = False) -> np.ndarray:
        """LaplCyl3FFT2<double,false,zflag>::solve; rhs shaped (nphi, nz, nr)."""
        nphi, nz, nr = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        self.L.ref_lapl_cyl_d(1 if periodic_z else 0, nr, nz, nphi, dr, dz, r0, lr, lz, _p(ans), _p(r))
        return ans

    def lapl_rect_flags(self, rhs, dx, dy, lx, ly, fft2: bool, flags: int) -> np.ndarray:
        """LaplRect(FFT2)<double,false,F> with F periodic in y (flags 2) or in
        y and x (flags 3)."""
        ny, nx = rhs.shape
        r = np.ascontiguousarray(rhs, np.float64)
        ans = np.zeros_like(r)
        if self.L.ref_lapl_rect_flags_d(nx, ny, dx, dy, lx, ly, 1 if fft2 else 0, flags, _p(ans), _p(r)):
            raise ValueError("flags %d not instantiated" % flags)
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

    def nscyl(self, nr, nz, nphi, Re, dt, u0=1.0, R=np.pi, r0=np.pi / 2, h1=0.0, h2=10.0, periodic_z=False,
              vrandom=False):
        """NSCyl<double,false,zflag> (src/ns_cyl.h:18-134); vrandom sets
        ns:vrandom=1."""
        return _NS(self.L, self.L.ref_nscyl_create_v(1 if periodic_z else 0, R, r0, h1, h2, u0, Re, dt, nr, nz,
                                                     nphi, 1 if vrandom else 0), "cyl")

    def nscube_float(self, nx, nz, Re, dt, u0=1.0, box=(-np.pi, -np.pi, -np.pi, np.pi, np.pi, np.pi)):
        """NSCube<float,false>; fields come back widened to float64."""
        return _NS(self.L, self.L.ref_nscubef_create(nx, nz, Re, dt, u0, *box), "reff")


_port = None
_ref = None


def pfft1(f: np.ndarray, dx: float, axis: int = -1) -> np.ndarray:
    """Restatement of FFT<T>::pFFT_1 (src/fft.cpp:108-194) along `axis`:
    S[k] = dx sum_j f_j cos(2 pi jk/n) for k <= n/2 and S[n-k] =
    dx sum_j f_j sin(2 pi jk/n) for 0 < k < n/2 (the layout its recursion
    produces; checked against the compiled reference in tests)."""
    f = np.moveaxis(np.asarray(f, np.float64), axis, -1)
    n = f.shape[-1]
    F = np.fft.rfft(f, axis=-1) * dx
    S = np.empty_like(f)
    S[..., : n // 2 + 1] = F.real
    k = np.arange(1, n // 2)
    S[..., n - k] = -F.imag[..., k]
    return np.moveaxis(S, -1, axis)


def pfft(S: np.ndarray, dx: float, axis: int = -1) -> np.ndarray:
    """Restatement of FFT<T>::pFFT (src/fft.cpp:195-212), the inverse layout:
    f_j = dx (S_0/2 + sum_{0<k<n/2} (S_k cos + S_{n-k} sin)(2 pi jk/n)
    + S_{n/2}/2 cos(pi j))."""
    S = np.moveaxis(np.asarray(S, np.float64), axis, -1)
    n = S.shape[-1]
    H = np.zeros(S.shape[:-1] + (n // 2 + 1,), complex)
    H[..., 0] = S[..., 0]
    H[..., n // 2] = S[..., n // 2]
    k = np.arange(1, n // 2)
    H[..., k] = S[..., k] - 1j * S[..., n - k]
    f = np.fft.irfft(H, n=n, axis=-1) * (n * dx / 2)
    return np.moveaxis(f, -1, axis)


def pfft3d(s: np.ndarray, dx: float, inverse: bool = False) -> np.ndarray:
    """Restatement of FFT<T>::pFFT_1_3d / pFFT_3d (src/fft.cpp:214-292):
    the 1-D transform along the fastest axis (x), then y, then z of an N^3
    cube (z, y, x), scale dx on every pass."""
    f = pfft if inverse else pfft1
    a = f(np.asarray(s, np.float64), dx, axis=2)
    a = f(a, dx, axis=1)
    return f(a, dx, axis=0)


def lapl_cube_periodic(rhs, dx, dy, dz, lx, ly, lz) -> np.ndarray:
    """Restatement of LaplCube<double,check,periodic^3>::solve
    (src/lapl_cube.cpp:9-142; eigenvalues :145-172): pFFT_1 along z, y, x
    with scale h sqrt(2/l), divide by -(lz_i + ly_k + lx_j) with
    l_p = 4/h^2 sin^2(p pi/n) (lm_y shared with x / z when the point counts
    match), zero mode := 0, pFFT along x, y, z with scale sqrt(2/l).  The
    reference addresses its {1..n} tensors with periodic wrap from index 0,
    a cyclic shift that the shift-invariant solve undoes."""
    r = np.asarray(rhs, np.float64)
    nz, ny, nx = r.shape
    slx, sly, slz = np.sqrt(2 / lx), np.sqrt(2 / ly), np.sqrt(2 / lz)

    def lam(n, h):
        return 4.0 / (h * h) * np.sin(np.arange(n) * np.pi / n) ** 2
    ly_ = lam(ny, dy)
    lx_ = ly_ if nx == ny else lam(nx, dx)
    lz_ = ly_ if nz == ny else lam(nz, dz)
    a = pfft1(r, dz * slz, axis=0)
    a = pfft1(a, dy * sly, axis=1)
    a = pfft1(a, dx * slx, axis=2)
    k2 = lz_[:, None, None] + ly_[None, :, None] + lx_[None, None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        a = a / -k2
    a[0, 0, 0] = 0.0
    a = pfft(a, slx, axis=2)
    a = pfft(a, sly, axis=1)
    return pfft(a, slz, axis=0)


def dst1(x: np.ndarray, dx: float, axis: int = -1) -> np.ndarray:
    """FFT<T>::sFFT on the interior entries (src/fft.cpp:294-365): for n
    points along `axis`, N = n + 1, S_k = dx sum_{j=1}^{n} x_j sin(pi jk/N)."""
    x = np.moveaxis(np.asarray(x, np.float64), axis, -1)
    n = x.shape[-1]
    j = np.arange(1, n + 1)
    S = np.sin(np.pi * np.outer(j, j) / (n + 1))
    return np.moveaxis(x @ S * dx, -1, axis)


def lapl_rect_flags(rhs, dx, dy, lx, ly, fft2: bool, flags: int) -> np.ndarray:
    """Restatement of LaplRect / LaplRectFFT2 with periodic flags
    (src/lapl_rect.cpp:11-41, 63-207): flags 2 = y periodic (pFFT_1 / pFFT
    along y, lm_y = 4/dy^2 sin^2(k pi/ny)), 3 = y and x periodic (FFT2: pFFT
    along x too, lm_x = 4/dx^2 sin^2(j pi/nx), and the reference's
    double-period hack: the (0, 0) mode := 1).  LaplRect solves x as
    tridiagonal systems whatever the x flag.  rhs is (ny, nx)."""
    r = np.asarray(rhs, np.float64)
    ny, nx = r.shape
    sly, slx = np.sqrt(2.0 / ly), np.sqrt(2.0 / lx)
    lmy = 4.0 / (dy * dy) * np.sin(np.arange(ny) * np.pi / ny) ** 2
    a = pfft1(r, dy * sly, axis=0)
    px = bool(flags & 1) and fft2
    if not fft2:
        out = np.empty_like(a)
        for k in range(ny):
            A = (np.diag(np.full(nx, -2.0 / (dx * dx) - lmy[k])) + np.diag(np.full(nx - 1, 1.0 / (dx * dx)), 1)
                 + np.diag(np.full(nx - 1, 1.0 / (dx * dx)), -1))
            out[k] = np.linalg.solve(A, a[k])
        a = out
    elif px:
        lmx = 4.0 / (dx * dx) * np.sin(np.arange(nx) * np.pi / nx) ** 2
        b = pfft1(a, dx * slx, axis=1)
        with np.errstate(divide="ignore", invalid="ignore"):
            b = b / (-lmy[:, None] - lmx[None, :])
        b[0, 0] = 1.0
        a = pfft(b, slx, axis=1)
    else:
        lmx = 4.0 / (dx * dx) * np.sin(np.arange(1, nx + 1) * np.pi * 0.5 / (nx + 1)) ** 2
        b = dst1(a, dx * slx, axis=1)
        b = b / (-lmy[:, None] - lmx[None, :])
        a = dst1(b, slx, axis=1)
    return pfft(a, sly, axis=0)


def lapl_cyl(rhs, dr, dz, r0, lr, lz, periodic_z: bool = False) -> np.ndarray:
    """Restatement of LaplCyl3FFT2<double,check,zflag>::solve
    (src/lapl_cyl.cpp:10-128, init_solver :130-166) on arrays shaped
    (nphi, nz, nr), r fastest: pFFT_1 along phi (scale dphi/sqrt(pi)), sFFT
    (Dirichlet z) or pFFT_1 (periodic z) along z (scale dz sqrt(2/lz)), per
    (phi-mode i, z-mode k) the radial system D_j = -2/dr^2 - lm_phi_i/r^2 -
    lm_z_k, L_j = (r - dr/2)/(dr^2 r), U_j = (r + dr/2)/(dr^2 r),
    r = r0 + j dr, solved by elimination without row swaps (the matrices
    are diagonally dominant, so partial pivoting does not swap), then the
    inverse transforms (scales sqrt(2/lz), 1/sqrt(pi))."""
    f = np.asarray(rhs, np.float64)
    nphi, nz, nr = f.shape
    dphi = 2 * np.pi / nphi
    inv_sqrt_pi = 0.56418958354775629
    slz = np.sqrt(2.0 / lz)
    zpoints = nz if periodic_z else nz + 1
    lm_phi = 4.0 / dphi ** 2 * np.sin(np.arange(nphi) * dphi * 0.5) ** 2
    if periodic_z:
        lm_z = 4.0 / dz ** 2 * np.sin(np.arange(nz) * np.pi / zpoints) ** 2
    else:
        lm_z = 4.0 / dz ** 2 * np.sin(np.arange(1, nz + 1) * np.pi * 0.5 / zpoints) ** 2
    a = pfft1(f, dphi * inv_sqrt_pi, axis=0)
    a = pfft1(a, dz * slz, axis=1) if periodic_z else dst1(a, dz * slz, axis=1)
    r = r0 + np.arange(1, nr + 1) * dr
    lo = (r - 0.5 * dr) / (dr * dr) / r
    up = (r + 0.5 * dr) / (dr * dr) / r
    out = np.empty_like(a)
    for i in range(nphi):
        for k in range(nz):
            d = -2 / (dr * dr) - lm_phi[i] / r / r - lm_z[k]
            b = a[i, k].copy()
            dd = d.copy()
            for j in range(nr - 1):
                fact = lo[j + 1] / dd[j]
                dd[j + 1] -= fact * up[j]
                b[j + 1] -= fact * b[j]
            b[nr - 1] /= dd[nr - 1]
            for j in range(nr - 2, -1, -1):
                b[j] = (b[j] - up[j] * b[j + 1]) / dd[j]
            out[i, k] = b
    out = pfft(out, slz, axis=1) if periodic_z else dst1(out, slz, axis=1)
    return pfft(out, inv_sqrt_pi, axis=0)


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
