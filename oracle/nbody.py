"""Test infrastructure, not product code.

A numpy restatement of the reference's particle-mesh N-body driver,
NBody<T,check,CIC3<T>> of test/nbody.cpp, and a ctypes handle on the
reference's own class compiled into oracle/_ref/libfdm_ref.so
(oracle/ref_nbody.cpp).  Only the tests and bench.py's CPU-baseline leg use
them.

Arithmetic follows the reference's C++ types: T is float32 or float64, the
driver's own parameters (l, h, dt, G, the total mass) are double, so mixed
expressions are evaluated in double and rounded to T where the reference
stores them.  Two properties of the reference are reproduced as they are:

* distribute_masses (test/nbody.cpp:243-258) visits, for off = 0 and 1, the
  cells whose three indices are all congruent to off modulo 2: bodies in the
  other six parity classes deposit no mass;
* the periodic image offsets of the local particle-particle forces
  (test/nbody.cpp:353-376) tie off[0] (the x coordinate) to the y cell index
  k and off[1] (y) to the x cell index j, and the upper image (+l) is taken
  when a neighbour index reaches n, the mass grid's size, not npp.
"""
from __future__ import annotations

import ctypes
import math
from ctypes import c_double, c_int, c_void_p

import numpy as np

# ---- initial bodies (test/nbody.cpp:515-590) -------------------------------

_MINSTD_A = 16807
_MINSTD_M = 2147483647


def minstd_rand0(count: int, seed: int = 1) -> np.ndarray:
    """Outputs 1..count of the Park-Miller generator x <- 16807 x mod (2^31-1)
    (std::minstd_rand0, the default_random_engine of libstdc++)."""
    out = np.empty(count, np.int64)
    B = 4096
    pw = np.empty(B, np.int64)
    p = 1
    for j in range(B):
        p = p * _MINSTD_A % _MINSTD_M
        pw[j] = p
    s = seed
    for b in range(0, count, B):
        m = min(B, count - b)
        out[b : b + m] = s * pw[:m] % _MINSTD_M
        s = int(out[b + m - 1])
    return out


def uniform01(count: int, dtype) -> np.ndarray:
    """std::uniform_real_distribution<T>(0, 1) over minstd_rand0, i.e. the
    standard's generate_canonical<T, digits>: k = max(1, ceil(b / log2 R))
    draws, R = max - min + 1 = 2^31 - 2, S = sum_i (g_i - 1) R^i, u = S / R^k
    (k = 2 for double, 1 for float), evaluated in T."""
    T = np.dtype(dtype).type
    k = 2 if T == np.float64 else 1
    g = minstd_rand0(count * k).reshape(count, k) - 1
    R = T(2147483646.0)
    s = T(0)
    tmp = T(1)
    for i in range(k):
        s = s + g[:, i].astype(T) * tmp
        tmp = T(tmp * R)
    u = (s / tmp).astype(T)
    u[u >= 1] = np.nextafter(T(1), T(0))
    return u


# the fixed ten-body configuration of init_points' solar branch: name, x, y,
# vx, vy, mass (astronomical units, years / 2 pi, Earth masses)
SOLAR = (
    ("Sun", 0, 0, 0, 0, 333333),
    ("Mercury", 0, 0.39, 1.58, 0, 0.038),
    ("Venus", 0, 0.72, 1.17, 0, 0.82),
    ("Earth", 0, 1, 1, 0, 1),
    ("Moon", 0, 1.00256, 1.03, 0, 0.012),
    ("Mars", 0, 1.51, 0.8, 0, 0.1),
    ("Jupiter", 0, 5.2, 0.43, 0, 317),
    ("Saturn", 0, 9.3, 0.32, 0, 95),
    ("Uranus", 0, 19.3, 0.23, 0, 14.5),
    ("Neptune", 0, 30, 0.18, 0, 16.7),
)


def init_bodies(N: int, l: float, origin, vel: float, solar: bool, dtype):
    """NBody::init_points: returns x, v (N x 3), mass (N), G override (or
    None) and the total mass summed in index order in double."""
    T = np.dtype(dtype).type
    if solar:
        x = np.zeros((len(SOLAR), 3), T)
        v = np.zeros((len(SOLAR), 3), T)
        m = np.zeros(len(SOLAR), T)
        for i, (_, px, py, vx, vy, ms) in enumerate(SOLAR):
            x[i, 0], x[i, 1], v[i, 0], v[i, 1], m[i] = T(px), T(py), T(vx), T(vy), T(ms)
        total = 0.0
        for mi in m.astype(np.float64):  # mass += body.mass, in index order
            total += mi
        return x, v, m, 2.96e-6, total
    u = uniform01(4 * N, T).reshape(N, 4)
    org = np.asarray(origin, T)
    x = np.empty((N, 3), T)
    for i in range(3):
        x[:, i] = (l * u[:, i].astype(np.float64) + org[i].astype(np.float64)).astype(T)
    m = (0.2 + 1.5 * u[:, 3].astype(np.float64)).astype(T)
    # blas::dot(3, x, 1, x, 1) in T, left to right; std::sqrt in T
    d = (x[:, 0] * x[:, 0]).astype(T)
    d = (d + x[:, 1] * x[:, 1]).astype(T)
    d = (d + x[:, 2] * x[:, 2]).astype(T)
    R = np.sqrt(d).astype(np.float64)
    V = vel / np.sqrt(R)
    v = np.zeros((N, 3), T)
    v[:, 0] = (V * x[:, 1].astype(np.float64)).astype(T)
    v[:, 1] = (-V * x[:, 0].astype(np.float64)).astype(T)
    total = 0.0
    for mi in m.astype(np.float64):  # mass += body.mass, in index order
        total += mi
    return x, v, m, None, total


# ---- the step (test/nbody.cpp:134-143, 260-470) ----------------------------


class NBodyPort:
    """NBody<T,check,CIC3<T>> restated.  Bodies are arrays x, v, a, aprev, F
    (N x 3, T) and mass (N, T); the grids f, rhs, psi (n^3) and E (n^3 x 3)
    are stored z-slowest, x-fastest like the reference's tensors."""

    def __init__(self, x0, y0, z0, l, n, npp, N, dt, G, vel=4.0, sgn=-1, local=0, solar=0, crit=1.0,
                 dtype=np.float64, bodies=None):
        T = self.T = np.dtype(dtype).type
        self.origin = np.array([x0, y0, z0], T)
        self.l = float(l)
        self.n, self.npp = int(n), int(npp)
        self.h, self.hpp = self.l / n, self.l / npp
        self.dt, self.G, self.sgn, self.local = float(dt), float(G), int(sgn), int(local)
        self.rcrit = self.hpp * float(T(crit))
        if bodies is None:
            x, v, m, g, total = init_bodies(N, self.l, self.origin, vel, bool(solar), T)
            if g is not None:
                self.G = g
            self.set_bodies(x, v, m)
            # the solar branch of init_points fills no cell lists
            self.lists_empty = bool(solar)
        else:
            self.set_bodies(*bodies)

    def set_bodies(self, x, v, mass, a=None, aprev=None):
        T = self.T
        self.x = np.array(x, T).reshape(-1, 3)
        self.N = self.x.shape[0]
        self.v = np.array(v, T).reshape(-1, 3)
        self.mass = np.array(mass, T).reshape(-1)
        self.a = np.zeros((self.N, 3), T) if a is None else np.array(a, T).reshape(-1, 3)
        self.aprev = np.zeros((self.N, 3), T) if aprev is None else np.array(aprev, T).reshape(-1, 3)
        self.F = np.zeros((self.N, 3), T)
        # NBody's cell lists: filled by init_points / move, emptied at the end
        # of calc_a_pm
        self.lists_empty = False
        self.total_mass = 0.0
        for mi in self.mass.astype(np.float64):
            self.total_mass += mi

    # cell indices as NBody::move computes them: (x - origin) in T, / h in double
    def _cells(self, h):
        d = (self.x - self.origin).astype(self.T).astype(np.float64)
        return np.floor(d / h).astype(np.int64)  # columns j (x), k (y), i (z)

    def _cic(self):
        """CIC3<T>::distribute (src/interpolate.h:66-96) for every body: the
        corner (j0, k0, i0) and the weights M[i][k][j] (8, T)."""
        T = self.T
        hT = T(self.h)
        xx = (self.x - self.origin).astype(T)
        c0 = np.floor(xx / hT).astype(np.int64)
        r = ((xx - (c0.astype(T) * hT).astype(T)).astype(T) / hT).astype(T)
        wx = (T(1) - r[:, 0], r[:, 0])
        wy = (T(1) - r[:, 1], r[:, 1])
        wz = (T(1) - r[:, 2], r[:, 2])
        M = np.empty((8, self.N), T)
        for a in range(2):
            for b in range(2):
                for c in range(2):
                    M[4 * a + 2 * b + c] = ((wz[a] * wy[b]).astype(T) * wx[c]).astype(T)
        return c0, M

    def _corner_index(self, c0, a, b, c):
        n = self.n
        return ((c0[:, 2] + a) % n) * n * n + ((c0[:, 1] + b) % n) * n + (c0[:, 0] + c) % n

    def calc_a_pm(self):
        T, n = self.T, self.n
        l = self.l
        f = np.full(n ** 3, T(-self.total_mass / l / l / l), T)
        cells = self._cells(self.h)
        c0, M = self._cic()
        cells = cells % n  # the periodic cell tensor wraps an index of n to 0
        for off in range(0 if self.lists_empty else 2):  # only all-even / all-odd cells
            sel = np.all(cells % 2 == off, axis=1)
            idx = np.nonzero(sel)[0]  # ascending body index = cell-list order
            for a in range(2):
                for b in range(2):
                    for c in range(2):
                        w = (self.mass[idx] * M[4 * a + 2 * b + c, idx]).astype(T)
                        np.add.at(f, self._corner_index(c0[idx], a, b, c), w)
        self.f = f
        self.rhs = (4 * self.G * math.pi * f.astype(np.float64) / self.h / self.h / self.h).astype(T)
        from .oracle import lapl_cube_periodic

        h = self.h
        psi = lapl_cube_periodic(self.rhs.reshape(n, n, n).astype(np.float64), h, h, h, l, l, l)
        self.psi = psi.astype(T).reshape(-1)
        self.E = self._efield(self.psi.reshape(n, n, n)).reshape(-1, 3)
        self.F[:] = 0
        if self.local and not self.lists_empty:
            self._local_forces()
        self._accelerations(c0, M)
        self.lists_empty = True

    def _efield(self, psi):
        """E = -grad psi by Hockney's beta = 4/3 blend of 2nd and 4th order
        differences (test/nbody.cpp:327-342), periodic wrap."""
        T = self.T
        beta = T(4.0 / 3.0)
        h = self.h
        E = np.empty(psi.shape + (3,), T)
        for m, ax in ((0, 2), (1, 1), (2, 0)):
            d1 = (np.roll(psi, -1, ax) - np.roll(psi, 1, ax)).astype(T)
            d2 = (np.roll(psi, -2, ax) - np.roll(psi, 2, ax)).astype(T)
            t1 = ((-beta * d1).astype(T) / T(2)).astype(T).astype(np.float64) / h
            t2 = (((T(1) - beta) * d2).astype(T) / T(4)).astype(T).astype(np.float64) / h
            E[..., m] = (t1 - t2).astype(T)
        return E

    def _accelerations(self, c0, M):
        """calc_accelerations (test/nbody.cpp:431-470): a = F + sum E M."""
        T = self.T
        a = (T(0) + self.F).astype(T)
        E = self.E
        for ia in range(2):
            for ib in range(2):
                for ic in range(2):
                    e = self._corner_index(c0, ia, ib, ic)
                    w = M[4 * ia + 2 * ib + ic]
                    for m in range(3):
                        a[:, m] = (a[:, m] + (E[e, m] * w).astype(T)).astype(T)
        self.a = a

    def _local_forces(self):
        """The short-range particle-particle correction (test/nbody.cpp:
        353-376, apply_bi_bj :403-419), per body in the reference's order:
        the 27 neighbour cells of the pp grid (i0, k0, j0 = -1..1), each
        cell's bodies in index order."""
        T, npp, n, l = self.T, self.npp, self.n, self.l
        cells = self._cells(self.hpp) % npp  # list membership wraps like the periodic tensor
        key = cells[:, 2] * npp * npp + cells[:, 1] * npp + cells[:, 0]
        order = np.argsort(key, kind="stable")
        start = np.searchsorted(key[order], np.arange(npp ** 3 + 1))
        G, rc = self.G, self.rcrit
        x = self.x
        for bi in range(self.N):
            j, k, i = (int(cells[bi, 0]), int(cells[bi, 1]), int(cells[bi, 2]))
            F = [self.F[bi, 0], self.F[bi, 1], self.F[bi, 2]]
            for i0 in (-1, 0, 1):
                for k0 in (-1, 0, 1):
                    for j0 in (-1, 0, 1):
                        off = [T(0), T(0), T(0)]
                        if k + k0 < 0:
                            off[0] = T(-l)
                        if k + k0 >= n:
                            off[0] = T(l)
                        if j + j0 < 0:
                            off[1] = T(-l)
                        if j + j0 >= n:
                            off[1] = T(l)
                        if i + i0 < 0:
                            off[2] = T(-l)
                        if i + i0 >= n:
                            off[2] = T(l)
                        c = ((i + i0) % npp) * npp * npp + ((k + k0) % npp) * npp + (j + j0) % npp
                        for bj in order[start[c] : start[c + 1]]:
                            if bj == bi:
                                continue
                            d = [T(x[bi, m] - T(x[bj, m] + off[m])) for m in range(3)]
                            R = 0.0
                            for m in range(3):
                                R += float(d[m]) * float(d[m])
                            R = math.sqrt(R) + 0.001
                            if R < rc:
                                s = math.erfc(R / 2 / rc) + R / rc / math.sqrt(math.pi) * math.exp(-R * R / 4 / rc / rc)
                                mj = float(-self.mass[bj])
                                for m in range(3):
                                    F[m] = T(float(F[m]) + mj * G * float(d[m]) / R / R / R * s)
            self.F[bi] = F

    def move(self):
        """NBody::move (test/nbody.cpp:472-511): velocity Verlet with periodic
        wrap of the positions."""
        T, dt, l = self.T, self.dt, self.l
        x = self.x.astype(np.float64) + (dt * self.v.astype(np.float64) + 0.5 * dt * dt * self.aprev.astype(np.float64))
        x = x.astype(T)
        org = self.origin
        lo = x < org
        x[lo] = (x[lo].astype(np.float64) + l).astype(T)
        hi = x.astype(np.float64) >= org.astype(np.float64) + l
        hi = np.broadcast_to(hi, x.shape)
        x[hi] = (x[hi].astype(np.float64) - l).astype(T)
        self.x = x
        s = (self.a + self.aprev).astype(T)
        self.v = (self.v.astype(np.float64) + 0.5 * dt * s.astype(np.float64)).astype(T)
        self.aprev = self.a.copy()
        self.lists_empty = False

    def step(self, k: int = 1):
        for _ in range(k):
            self.calc_a_pm()
            self.move()

    def direct_forces(self, sgn: int | None = None, eps: float = 0.00001) -> np.ndarray:
        """calc_error's exact pairwise sum (test/nbody.cpp:145-170):
        F_i = sum_{j != i} sgn m_j G (x_i - x_j) / R^3, R = |x_i - x_j| + eps."""
        sgn = self.sgn if sgn is None else sgn
        x = self.x.astype(np.float64)
        m = self.mass.astype(np.float64)
        F = np.zeros((self.N, 3))
        for i in range(self.N):
            d = x[i] - x
            R = np.sqrt(np.sum(d * d, axis=1)) + eps
            w = sgn * m * self.G / R / R / R
            w[i] = 0.0
            F[i] = np.sum(w[:, None] * d, axis=0)
        return F


# ---- the reference's own class ---------------------------------------------


class RefNBody:
    """NBody<T,false,CIC3<T>> of test/nbody.cpp through oracle/ref_nbody.cpp."""

    def __init__(self, lib, x0, y0, z0, l, n, npp, N, dt, G, vel=4.0, sgn=-1, local=0, solar=0, crit=1.0,
                 dtype=np.float64):
        L = lib
        L.ref_nbody_create.restype = c_void_p
        L.ref_nbody_create.argtypes = [c_int] + [c_double] * 4 + [c_int] * 3 + [c_double] * 3 + [c_int] * 3 + [c_double]
        L.ref_nbody_destroy.argtypes = [c_void_p]
        L.ref_nbody_count.argtypes = [c_void_p]
        L.ref_nbody_count.restype = c_int
        L.ref_nbody_total_mass.argtypes = [c_void_p]
        L.ref_nbody_total_mass.restype = c_double
        L.ref_nbody_get_bodies.argtypes = [c_void_p] * 7
        L.ref_nbody_set_bodies.argtypes = [c_void_p] * 6
        L.ref_nbody_step.argtypes = [c_void_p, c_int]
        L.ref_nbody_get_fields.argtypes = [c_void_p] * 5
        self.L = L
        self.n = n
        self.h = L.ref_nbody_create(1 if np.dtype(dtype) == np.float32 else 0, x0, y0, z0, l, n, npp, N, dt, G, vel,
                                    sgn, local, solar, crit)
        self.N = L.ref_nbody_count(self.h)

    @staticmethod
    def _ptr(a):
        return None if a is None else a.ctypes.data

    def bodies(self):
        N = self.N
        x, v, a, ap, F = (np.zeros((N, 3)) for _ in range(5))
        m = np.zeros(N)
        self.L.ref_nbody_get_bodies(self.h, *(self._ptr(t) for t in (x, v, a, ap, m, F)))
        return dict(x=x, v=v, a=a, aprev=ap, mass=m, F=F)

    def set_bodies(self, x, v, mass, a=None, aprev=None):
        arrs = [None if t is None else np.ascontiguousarray(t, np.float64) for t in (x, v, a, aprev, mass)]
        self.L.ref_nbody_set_bodies(self.h, *(self._ptr(t) for t in arrs))

    @property
    def total_mass(self) -> float:
        return self.L.ref_nbody_total_mass(self.h)

    def step(self, k: int = 1):
        self.L.ref_nbody_step(self.h, k)

    def fields(self):
        n3 = self.n ** 3
        f, rhs, psi = np.zeros(n3), np.zeros(n3), np.zeros(n3)
        E = np.zeros((n3, 3))
        self.L.ref_nbody_get_fields(self.h, *(self._ptr(t) for t in (f, rhs, psi, E)))
        return dict(f=f, rhs=rhs, psi=psi, E=E)

    def close(self):
        if self.h:
            self.L.ref_nbody_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
