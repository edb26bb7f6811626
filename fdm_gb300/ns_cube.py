"""Host-side mirror of fdm::NSCube<T,check> (src/ns_cube.h:14-92).

Constructed from a `Config` with the reference keys ns:{x1,y1,z1,x2,y2,z2,
u0,Re,dt,nx,nz} and defaults (src/ns_cube.h:46-78; ny is read from key "nx"
as in the reference).  `step()` advances one projection step on the GPU
(src/ns_cube.cpp:27-62); the state stays on the device.  The public tensors
u, v, w, p, x, F, G, H, RHS are returned as `Tensor3` copies in the reference
layout (inclusive index ranges, x fastest) with reference-style indexing
`t[i, k, j]` over those ranges.
"""
from __future__ import annotations

import math
from ctypes import byref, c_int, c_size_t, c_void_p

import numpy as np

from . import _native as N
from .config import Config

FIELDS = ("u", "v", "w", "p", "x", "F", "G", "H", "RHS")


class Tensor3:
    """A host copy of a reference tensor: `data` (z, y, x) plus the inclusive
    index ranges (z1, z2, y1, y2, x1, x2) of src/tensor.h:192-219."""

    def __init__(self, data: np.ndarray, ranges):
        self.data = data
        self.ranges = tuple(ranges)

    def __getitem__(self, idx):
        i, k, j = idx
        z1, _, y1, _, x1, _ = self.ranges
        return self.data[i - z1, k - y1, j - x1]

    def maxabs(self) -> float:
        return float(np.abs(self.data).max()) if self.data.size else 0.0


class NSCube:
    def __init__(self, cfg: Config | None = None, dtype=None, **overrides):
        cfg = cfg or Config()
        for k, v in overrides.items():
            cfg.set("ns", k, v)
        if dtype is None:
            # solver:datatype selects NSCube<float> or NSCube<double>, as the
            # reference's cavity driver does (test/test_ns_cube.cpp:89-97)
            dtype = np.float32 if str(cfg.get("solver", "datatype", "double")) == "float" else np.float64
        self.x1 = cfg.get("ns", "x1", -math.pi)
        self.y1 = cfg.get("ns", "y1", -math.pi)
        self.z1 = cfg.get("ns", "z1", -math.pi)
        self.x2 = cfg.get("ns", "x2", math.pi)
        self.y2 = cfg.get("ns", "y2", math.pi)
        self.z2 = cfg.get("ns", "z2", math.pi)
        self.U0 = cfg.get("ns", "u0", 1.0)
        self.Re = cfg.get("ns", "Re", 1.0)
        self.dt = cfg.get("ns", "dt", 0.001)
        self.nx = cfg.get("ns", "nx", 32)
        self.ny = cfg.get("ns", "nx", 32)
        self.nz = cfg.get("ns", "nz", 32)
        self.verbose = cfg.get("ns", "verbose", 0)
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.float64, np.float32):
            raise N.FdmError(N.ENOTSUP, "NSCube is implemented for float64 and float32")
        self._lib = N.load()
        h = c_void_p()
        code = N.F64 if self.dtype == np.float64 else N.F32
        N.check(self._lib.fdmgpu_nscube_create(byref(h), code, int(self.nx), int(self.nz), float(self.x1),
                                               float(self.y1), float(self.z1), float(self.x2), float(self.y2),
                                               float(self.z2), float(self.U0), float(self.Re), float(self.dt)))
        self._h = h
        self.dx = (self.x2 - self.x1) / self.nx
        self.dy = (self.y2 - self.y1) / self.ny
        self.dz = (self.z2 - self.z1) / self.nz

    def step(self, k: int = 1) -> None:
        N.check(self._lib.fdmgpu_nscube_step(self._h, int(k)))

    @staticmethod
    def step_many(cavities, steps) -> None:
        """steps[i] steps of each FP64 cavity, all of one geometry, as shared
        launches (fdmgpu_nscube_step_many); the fields are bit for bit those
        of stepping each cavity alone."""
        cav = list(cavities)
        ks = [int(k) for k in steps]
        if len(cav) != len(ks) or not cav:
            raise N.FdmError(N.EINVAL, "one step count per cavity")
        hs = (c_void_p * len(cav))(*[c._h for c in cav])
        arr = (c_int * len(ks))(*ks)
        N.check(cav[0]._lib.fdmgpu_nscube_step_many(hs, arr, len(cav)))

    def set_exact(self, exact: bool = True) -> None:
        """exact=True: quotients by the run constants correctly rounded, as
        the reference's divisions are; False (default): products with
        precomputed reciprocals (faster, last-bit differences)."""
        N.check(self._lib.fdmgpu_nscube_set_exact(self._h, 1 if exact else 0))

    @property
    def time_index(self) -> int:
        t = c_int()
        N.check(self._lib.fdmgpu_nscube_time_index(self._h, byref(t)))
        return t.value

    def field_info(self, name: str):
        fid = FIELDS.index(name)
        cnt = c_size_t()
        r = (c_int * 6)()
        N.check(self._lib.fdmgpu_nscube_field_info(self._h, fid, byref(cnt), r))
        return cnt.value, tuple(r)

    def get(self, name: str) -> Tensor3:
        fid = FIELDS.index(name)
        cnt, r = self.field_info(name)
        shape = (r[1] - r[0] + 1, r[3] - r[2] + 1, r[5] - r[4] + 1)
        out = np.empty(shape, self.dtype)
        N.check(self._lib.fdmgpu_nscube_get_field(self._h, fid, out.ctypes.data, cnt))
        return Tensor3(out, r)

    def set(self, name: str, data: np.ndarray) -> None:
        fid = FIELDS.index(name)
        cnt, _ = self.field_info(name)
        a = np.ascontiguousarray(data, self.dtype)
        if a.size != cnt:
            raise N.FdmError(N.EINVAL, "field %s has %d elements" % (name, cnt))
        N.check(self._lib.fdmgpu_nscube_set_field(self._h, fid, a.ctypes.data, cnt))

    def device_ptr(self, name: str) -> int:
        p = c_void_p()
        N.check(self._lib.fdmgpu_nscube_field_device(self._h, FIELDS.index(name), byref(p)))
        return p.value

    def __getattr__(self, name):
        if name in FIELDS:
            return self.get(name)
        raise AttributeError(name)

    def vtk_out(self, path: str) -> None:
        """ASCII VTK snapshot of the cell-centred velocity in the format of
        the reference's velocity_plotter::vtk_out (src/velocity_plot.cpp:113)."""
        N.check(self._lib.fdmgpu_nscube_vtk_out(self._h, str(path).encode()))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_nscube_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NSCyl:
    """Host-side mirror of fdm::NSCyl<T,check,zflag> (src/ns_cyl.h:18-134):
    flow between coaxial cylinders, inner one rotating with u0.  Config keys
    ns:{R, r, h1, h2, u0, Re, dt, nr, nz, nphi} with the reference defaults;
    periodic_z selects zflag = periodic.  Fields are (phi, z, r) with r
    fastest, returned as Tensor3 over their inclusive ranges."""

    FIELDS = FIELDS + ("u0", "v0", "w0")

    def __init__(self, cfg: Config | None = None, dtype=np.float64, periodic_z: bool = False, **overrides):
        cfg = cfg or Config()
        for k, v in overrides.items():
            cfg.set("ns", k, v)
        self.R = cfg.get("ns", "R", math.pi)
        self.r0 = cfg.get("ns", "r", math.pi / 2)
        self.h1 = cfg.get("ns", "h1", 0.0)
        self.h2 = cfg.get("ns", "h2", 10.0)
        self.U0 = cfg.get("ns", "u0", 1.0)
        self.Re = cfg.get("ns", "Re", 1.0)
        self.dt = cfg.get("ns", "dt", 0.001)
        self.nr = cfg.get("ns", "nr", 32)
        self.nz = cfg.get("ns", "nz", 31)
        self.nphi = cfg.get("ns", "nphi", 32)
        self.dtype = np.dtype(dtype)
        self._lib = N.load()
        h = c_void_p()
        N.check(self._lib.fdmgpu_nscyl_create(byref(h), N.F64 if self.dtype == np.float64 else N.F32,
                                              int(bool(periodic_z)), float(self.R), float(self.r0), float(self.h1),
                                              float(self.h2), float(self.U0), float(self.Re), float(self.dt),
                                              int(self.nr), int(self.nz), int(self.nphi)))
        self._h = h
        if int(cfg.get("ns", "vrandom", 0)) == 1:
            N.check(self._lib.fdmgpu_nscyl_vrandom(self._h))

    def step(self, k: int = 1) -> None:
        N.check(self._lib.fdmgpu_nscyl_step(self._h, int(k)))

    def L_step(self, k: int = 1) -> None:
        """NSCyl::L_step: the step linearised about u0, v0, w0."""
        N.check(self._lib.fdmgpu_nscyl_l_step(self._h, int(k)))

    def set(self, name: str, values) -> None:
        """Overwrites a whole field (ghosts included), e.g. the
        linearisation point w0 or a perturbation of u, v, w, p."""
        fid = self.FIELDS.index(name)
        cnt = c_size_t()
        N.check(self._lib.fdmgpu_nscyl_field_info(self._h, fid, byref(cnt), None))
        a = np.ascontiguousarray(values.data if isinstance(values, Tensor3) else values, self.dtype).ravel()
        if a.size != cnt.value:
            raise ValueError("%s has %d elements, got %d" % (name, cnt.value, a.size))
        N.check(self._lib.fdmgpu_nscyl_set_field(self._h, fid, a.ctypes.data, cnt.value))

    @property
    def time_index(self) -> int:
        t = c_int()
        N.check(self._lib.fdmgpu_nscyl_time_index(self._h, byref(t)))
        return t.value

    def get(self, name: str) -> Tensor3:
        fid = self.FIELDS.index(name)
        cnt = c_size_t()
        r = (c_int * 6)()
        N.check(self._lib.fdmgpu_nscyl_field_info(self._h, fid, byref(cnt), r))
        shape = (r[1] - r[0] + 1, r[3] - r[2] + 1, r[5] - r[4] + 1)
        out = np.empty(shape, self.dtype)
        N.check(self._lib.fdmgpu_nscyl_get_field(self._h, fid, out.ctypes.data, cnt.value))
        return Tensor3(out, tuple(r))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fdmgpu_nscyl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
