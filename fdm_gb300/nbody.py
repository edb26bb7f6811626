"""Host-side mirror of the reference's particle-mesh N-body driver,
NBody<T,check,CIC3<T>> (test/nbody.cpp:25-511).

The constructor takes the reference's arguments (x0, y0, z0, l, n, npp, N,
dt, G, vel, sgn, local, solar, crit) and draws the bodies as init_points does;
`from_config` reads them from the nbody section with the defaults of the
reference's calc() (test/nbody.cpp:593-611).  `step()` runs calc_a_pm + move
on the GPU; the bodies and grids stay on the device and are copied out on
request.  `calc_error()` is the reference's error mode: the PM accelerations
against the exact pairwise sum, relative per body.
"""
from __future__ import annotations

from ctypes import byref, c_double, c_int, c_longlong, c_void_p

import numpy as np

from . import _native as N
from .config import Config

FIELDS = {"f": 0, "rhs": 1, "psi": 2, "E": 3}


class NBody:
    def __init__(self, x0=-10.0, y0=-10.0, z0=-10.0, l=20.0, n=32, npp=64, N_bodies=100000, dt=0.001, G=1.0,
                 vel=4.0, sgn=-1, local=0, solar=0, crit=1.0, debug=0, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        self.n, self.npp = int(n), int(npp)
        self.origin = (x0, y0, z0)
        self.l, self.dt = float(l), float(dt)
        self.sgn, self.local, self.solar = int(sgn), int(local), int(solar)
        self._lib = N.load()
        h = c_void_p()
        N.check(self._lib.fdmgpu_nbody_create(
            byref(h), N.F64 if self.dtype == np.float64 else N.F32, float(x0), float(y0), float(z0), self.l,
            self.n, self.npp, int(N_bodies), self.dt, float(G), float(vel), self.sgn, self.local, self.solar,
            float(crit)))
        self._h = h

    @classmethod
    def from_config(cls, cfg: Config | None = None, **overrides) -> "NBody":
        cfg = cfg or Config()
        for k, v in overrides.items():
            cfg.set("nbody", k, v)
        g = lambda k, d: cfg.get("nbody", k, d)  # noqa: E731
        dtype = np.float32 if str(cfg.get("solver", "datatype", "double")) == "float" else np.float64
        return cls(g("x0", -10.0), g("y0", -10.0), g("z0", -10.0), g("l", 20.0), g("n", 32), g("npp", 64),
                   g("N", 100000), g("dt", 0.001), g("G", 1.0), g("vel", 4.0), g("sign", -1), g("local", 0),
                   g("solar", 0), g("rcrit", 1.0), g("debug", 0), dtype=dtype)

    # ---- state -------------------------------------------------------------
    def _info(self):
        nb, G, m, s = c_int(), c_double(), c_double(), c_longlong()
        N.check(self._lib.fdmgpu_nbody_info(self._h, byref(nb), byref(G), byref(m), byref(s)))
        return nb.value, G.value, m.value, s.value

    @property
    def N(self) -> int:
        return self._info()[0]

    @property
    def G(self) -> float:
        return self._info()[1]

    @property
    def mass(self) -> float:
        """Total mass, summed in body order as the reference does."""
        return self._info()[2]

    @property
    def steps(self) -> int:
        return self._info()[3]

    def bodies(self, fields=("x", "v", "a", "aprev", "mass", "F")) -> dict:
        """Host copies of the requested body arrays (x, v, a, aprev, F: N x 3;
        mass: N)."""
        n = self.N
        out = {k: np.empty((n,) if k == "mass" else (n, 3), self.dtype) for k in fields}
        N.check(self._lib.fdmgpu_nbody_get_bodies(self._h, *(out[k].ctypes.data if k in out else None for k in
                                                              ("x", "v", "a", "aprev", "mass", "F"))))
        return out

    def set_bodies(self, x, v, mass, a=None, aprev=None) -> None:
        n = self.N
        arr = lambda t, shape: None if t is None else np.ascontiguousarray(t, self.dtype).reshape(shape)  # noqa
        x3, v3, a3, p3 = (arr(t, (n, 3)) for t in (x, v, a, aprev))
        m = arr(mass, (n,))
        N.check(self._lib.fdmgpu_nbody_set_bodies(self._h, x3.ctypes.data, v3.ctypes.data,
                                                  None if a3 is None else a3.ctypes.data,
                                                  None if p3 is None else p3.ctypes.data, m.ctypes.data))

    def field(self, name: str) -> np.ndarray:
        """Grids of the last calc_a_pm: f, rhs, psi shaped (n, n, n) (z, y,
        x), E shaped (n, n, n, 3)."""
        n = self.n
        fid = FIELDS[name]
        out = np.empty((n, n, n, 3) if fid == 3 else (n, n, n), self.dtype)
        N.check(self._lib.fdmgpu_nbody_get_field(self._h, fid, out.ctypes.data, out.size))
        return out

    # ---- the driver ----------------------------------------------------------
    def step(self, k: int = 1) -> None:
        N.check(self._lib.fdmgpu_nbody_step(self._h, int(k)))

    def step_async(self, k: int = 1) -> None:
        N.check(self._lib.fdmgpu_nbody_step_async(self._h, int(k)))

    def sync(self) -> None:
        N.check(self._lib.fdmgpu_nbody_sync(self._h))

    def calc_a_pm(self) -> None:
        N.check(self._lib.fdmgpu_nbody_calc_forces(self._h))

    def direct_forces(self) -> np.ndarray:
        F = np.empty((self.N, 3), self.dtype)
        N.check(self._lib.fdmgpu_nbody_direct_forces(self._h, F.ctypes.data))
        return F

    def calc_error(self) -> np.ndarray:
        """calc_error (test/nbody.cpp:145-183): PM accelerations a against the
        exact sum F; returns |a - F| / |F| per body."""
        self.calc_a_pm()
        F = self.direct_forces().astype(np.float64)
        a = self.bodies()["a"].astype(np.float64)
        return np.sqrt(np.sum((a - F) ** 2, axis=1)) / np.sqrt(np.sum(F * F, axis=1))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_nbody_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
