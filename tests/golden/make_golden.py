"""Generates the golden fixtures in tests/golden/ by running the reference's
own CPU code (oracle/_ref/libfdm_ref.so, built by `make -C oracle ref` from
the reference sources).  Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py

Inputs are seeded (numpy default_rng) or analytic; each fixture stores the
inputs it needs (or the seed plus checksums of the regenerated input) and the
reference outputs.  Small cases are stored in full; 31^3 cases as checksums
plus values at seeded sample positions.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from fdm_gb300 import workloads  # noqa: E402
from oracle.oracle import reference  # noqa: E402

OUT = Path(__file__).resolve().parent


def checksums(a: np.ndarray, nsamp: int = 256, seed: int = 1234):
    rng = np.random.default_rng(seed)
    flat = a.ravel()
    idx = rng.choice(flat.size, size=min(nsamp, flat.size), replace=False)
    return dict(sum=flat.sum(), l2=np.linalg.norm(flat), maxabs=np.abs(flat).max(), idx=idx, vals=flat[idx])


def ut_lapl_cube_rhs(n: int):
    """RHS and analytic answer of the reference's test_lapl_cube
    (ut/ut_lapl_cube.cpp:21-92): u = sin^2 x + cos^2 y + sin^2 z at cell
    centres of [0,1]^3, boundary values folded into the RHS."""
    x1 = y1 = z1 = 0.0
    x2 = y2 = z2 = 1.0
    dx = (x2 - x1) / n
    dy, dz = dx, dx

    def c(i, h, o):
        return o + h * i - h / 2

    def ans(i, k, j):
        return math.sin(c(j, dx, x1)) ** 2 + math.cos(c(k, dy, y1)) ** 2 + math.sin(c(i, dz, z1)) ** 2

    def rp(i, k, j):
        x, y, z = c(j, dx, x1), c(k, dy, y1), c(i, dz, z1)
        return (2 * math.sin(y) ** 2 - 2 * math.cos(y) ** 2 - 2 * math.sin(x) ** 2 + 2 * math.cos(x) ** 2
                - 2 * math.sin(z) ** 2 + 2 * math.cos(z) ** 2)

    rhs = np.zeros((n, n, n))
    exact = np.zeros((n, n, n))
    for i in range(1, n + 1):
        for k in range(1, n + 1):
            for j in range(1, n + 1):
                r = rp(i, k, j)
                if i <= 1: r -= ans(i - 1, k, j) / dz / dz
                if k <= 1: r -= ans(i, k - 1, j) / dy / dy
                if j <= 1: r -= ans(i, k, j - 1) / dx / dx
                if j >= n: r -= ans(i, k, j + 1) / dx / dx
                if k >= n: r -= ans(i, k + 1, j) / dy / dy
                if i >= n: r -= ans(i + 1, k, j) / dz / dz
                rhs[i - 1, k - 1, j - 1] = r
                exact[i - 1, k - 1, j - 1] = ans(i, k, j)
    args = (dx, dy, dz, x2 - x1 + dx, y2 - y1 + dy, z2 - z1 + dz)
    return rhs, exact, args


def f32_line(N: int, t: int) -> np.ndarray:
    """Line t of the FP32 round-trip inputs: N-1 values uniform in (-1, 1)."""
    return np.random.default_rng(1000 + t).uniform(-1, 1, N - 1).astype(np.float32)


def couette_w0(nr, nz, nphi, pz, R=math.pi, r0=math.pi / 2, U0=1.0, h1=0.0, h2=10.0):
    """The base flow test/test_ns_cyl_spectral.cpp:64-73 puts into w0:
    -U0 r0^2/(R^2-r0^2) + U0 r0^2 R^2/(R^2-r0^2)/r/r at r = r0 + dr j + dr/2,
    j = 0..nr, over w0's storage (phi, z0..znn, 0..nr+1); other entries 0."""
    dr = (R - r0) / nr
    zs = nz if pz else nz + 2
    w0 = np.zeros((nphi, zs, nr + 2))
    for j in range(nr + 1):
        r = r0 + dr * j + dr / 2
        w0[:, :nz, j] = (-U0 * r0 * r0 / (R * R - r0 * r0) + U0 * r0 * r0 * R * R / (R * R - r0 * r0) / r / r)
    return w0.ravel()


# tag, T, N, n, npp, local, solar (solar: the ten-body table, N ignored)
NBODY_CASES = (
    ("d", np.float64, 400, 16, 8, 0, 0),
    ("d_pp", np.float64, 400, 8, 8, 1, 0),
    ("f", np.float32, 400, 16, 8, 0, 0),
    ("f_pp", np.float32, 400, 8, 8, 1, 0),
    ("solar", np.float64, 0, 16, 8, 1, 1),
)


def _save(name: str, arrays: dict) -> None:
    """Writes tests/golden/<name>.npz unless the command line names other
    fixtures (`make_golden.py ns_cube` rewrites only ns_cube.npz)."""
    only = set(sys.argv[1:])
    if not only or name in only:
        np.savez_compressed(OUT / (name + ".npz"), **arrays)


def main():
    R = reference()
    if R is None:
        raise SystemExit("oracle/_ref/libfdm_ref.so missing: run `make -C oracle ref` first")

    # DST-I vectors (FFT<T>::sFFT)
    d = {}
    for N in (2, 8, 32, 256, 1024):
        s = np.random.default_rng(N).uniform(-1, 1, N)
        s[0] = 0.0
        d["s_%d" % N] = s
        d["S_%d" % N] = R.sfft(s, 1.0)
        d["Sh_%d" % N] = R.sfft(s, 0.5)
    # FP32 round trip S = sFFT(s, 1), s' = sFFT(S, 2/N) of the reference's
    # float instantiation, 64 lines uniform(-1,1) per N (ut/ut_fft.cpp:190-228
    # asserts 1e-5 at N=1024 for its one default-seeded line)
    import ctypes
    fp = ctypes.POINTER(ctypes.c_float)
    R.L.ref_sfft_f.argtypes = [fp, fp, ctypes.c_float, ctypes.c_int]

    def sfft32(v, dx):
        S = np.zeros(v.size, np.float32)
        a = v.astype(np.float32).copy()
        R.L.ref_sfft_f(S.ctypes.data_as(fp), a.ctypes.data_as(fp), dx, v.size)
        return S
    for N in (32, 256, 1024):
        worst = 0.0
        for t in range(64):
            v = np.zeros(N, np.float32)
            v[1:] = f32_line(N, t)
            v1 = sfft32(sfft32(v, 1.0), 2.0 / N)
            worst = max(worst, float(np.abs(v1[1:] - v[1:]).max()))
        d["f32_roundtrip_err_%d" % N] = np.array(worst)
    _save("dst", d)

    # LaplCube
    c = {}
    f, _ = workloads.manufactured(15, 15, 15, seed=3, kmax=4)
    a = workloads.solver_args(15, 15, 15)
    c["m15_rhs"] = f
    c["m15_ans"] = R.lapl_cube(f, *a[:6])
    rng = np.random.default_rng(11)
    rhs = rng.standard_normal((7, 15, 15))
    h = (0.1, 0.2, 0.3)
    args = (h[0], h[1], h[2], 16 * h[0], 16 * h[1], 8 * h[2])
    c["aniso_rhs"], c["aniso_args"] = rhs, np.array(args)
    c["aniso_ans"] = R.lapl_cube(rhs, *args)
    rhs = rng.standard_normal((15, 7, 31))
    args = (0.05, 0.3, 0.11, 32 * 0.05, 8 * 0.3, 16 * 0.11 * 1.5)  # lz not (nz+1)dz: scale convention
    c["lz_rhs"], c["lz_args"] = rhs, np.array(args)
    c["lz_ans"] = R.lapl_cube(rhs, *args)
    f, _ = workloads.manufactured(31, 31, 31, seed=0, kmax=12)
    a = workloads.solver_args(31, 31, 31)
    for k, v in checksums(f).items():
        c["c0_rhs_" + k] = v
    for k, v in checksums(R.lapl_cube(f, *a[:6])).items():
        c["c0_ans_" + k] = v
    rhs, exact, args = ut_lapl_cube_rhs(31)
    out = R.lapl_cube(rhs, *args)
    for k, v in checksums(out).items():
        c["ut31_ans_" + k] = v
    c["ut31_err"] = np.abs(out - exact).max() / np.abs(exact).max()
    _save("lapl_cube", c)

    # periodic LaplCube<double,false,periodic^3> and its transforms
    # (FFT<T>::pFFT_1 / pFFT); arrays of n_z*n_y*n_x as the periodic callers
    # pass them (ut/ut_lapl_cube.cpp:156-243)
    per = {}
    rng = np.random.default_rng(21)
    for N in (8, 64, 512):
        s = rng.uniform(-1, 1, N)
        per["pf_s_%d" % N] = s
        per["pf1_%d" % N] = R.pfft1(s, 0.7)
        per["pf_%d" % N] = R.pfft(s, 0.3)
    for name, shape, h in (("c16", (16, 16, 16), (0.3, 0.3, 0.3)), ("a8x16x32", (8, 16, 32), (0.1, 0.2, 0.3)),
                           ("b32x16x16", (32, 16, 16), (0.2, 0.1, 0.05))):
        nz, ny, nx = shape
        f = rng.standard_normal(shape)
        args = (h[0], h[1], h[2], nx * h[0], ny * h[1], nz * h[2])
        per["rhs_" + name] = f
        per["args_" + name] = np.array(args)
        per["ans_" + name] = R.lapl_cube_periodic(f, *args)
    # FFT<double>::pFFT_1_3d / pFFT_3d on the cube test/test_fft_3d_bench.cpp
    # fills (its formula, including the repeated j term)
    for N in (8, 32):
        i, j, k = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
        cube = (np.sin(2.0 * math.pi * i / N + 2.0 * math.pi * j / N + 2.0 * math.pi * j / N)
                + 0.5 * np.cos(4.0 * math.pi * i / N + 4.0 * math.pi * j / N + 4.0 * math.pi * k / N))
        per["fft3d_in_%d" % N] = cube
        per["fft3d_fwd_%d" % N] = R.pfft3d(cube, 1.0)
        per["fft3d_inv_%d" % N] = R.pfft3d(cube, 1.0, inverse=True)
    _save("lapl_cube_periodic", per)

    # LaplCyl3FFT2<double,false,zflag> (src/lapl_cyl.cpp:10-166): arrays
    # (nphi, nz, nr), r fastest
    cyl = {}
    rng = np.random.default_rng(33)
    for name, pz, shape, geo in (("d16x15x20", False, (16, 15, 20), (0.1, 0.2, 0.5)),
                                 ("p8x16x12", True, (8, 16, 12), (0.05, 0.3, 1.0)),
                                 ("d32x31x7", False, (32, 31, 7), (0.2, 0.1, 0.0))):
        nphi, nz, nr = shape
        dr, dz, r0 = geo
        args = (dr, dz, r0, (nr + 1) * dr, (nz if pz else nz + 1) * dz)
        f = rng.standard_normal(shape)
        cyl["rhs_" + name] = f
        cyl["args_" + name] = np.array(args)
        cyl["ans_" + name] = R.lapl_cyl(f, *args, periodic_z=pz)
    # NSCyl<double,false,zflag> (src/ns_cyl.cpp:22-485): Dirichlet z
    # (nr 16, nz 15, nphi 16) and periodic z (nr 16, nz 16, nphi 8), Re 100,
    # dt 0.01, the reference's default radii and heights; 20 steps
    for name, pz, (nr, nz, nphi) in (("d16x15x16", False, (16, 15, 16)), ("p16x16x8", True, (16, 16, 8))):
        m = R.nscyl(nr, nz, nphi, 100.0, 0.01, periodic_z=pz)
        m.step(20)
        for f in ("u", "v", "w", "p", "x"):
            cyl["ns_%s_s20_%s" % (name, f)] = m.get(f)
        m.close()
    # NSCyl::L_step (src/ns_cyl.cpp:65-77) as the spectral driver uses it
    # (test/test_ns_cyl_spectral.cpp:60-96): the Couette profile as w0 and the
    # wall speed set to 0.  Periodic z: the constructor's vrandom perturbation
    # of v (stored, to pin it).  Dirichlet z (where vrandom trips the
    # reference's own wall check, src/ns_cyl.cpp:160): a seeded perturbation
    # of u (r < R) and w.  The fields after 10 linearised steps.
    rng = np.random.default_rng(77)
    for name, pz, (nr, nz, nphi) in (("d16x15x16", False, (16, 15, 16)), ("p16x16x8", True, (16, 16, 8))):
        m = R.nscyl(nr, nz, nphi, 100.0, 0.01, u0=0.0, periodic_z=pz, vrandom=pz)
        if pz:
            cyl["lin_%s_v_init" % name] = m.get("v")
        else:
            u = m.get("u").reshape(nphi, nz + 2, nr + 3)  # z 0..nz+1, r -1..nr+1
            w = m.get("w").reshape(nphi, nz + 2, nr + 2)  # r 0..nr+1
            u[:, 1:nz + 1, 2:nr + 1] = 1e-3 * rng.standard_normal((nphi, nz, nr - 1))  # r 1..nr-1
            w[:, 1:nz + 1, 1:nr + 1] = 1e-3 * rng.standard_normal((nphi, nz, nr))
            cyl["lin_%s_u_init" % name] = u.ravel()
            cyl["lin_%s_w_init" % name] = w.ravel()
            m.set("u", u)
            m.set("w", w)
        w0 = couette_w0(nr, nz, nphi, pz)
        cyl["lin_%s_w0" % name] = w0
        m.set("w0", w0)
        m.l_step(10)
        for f in ("u", "v", "w", "p"):
            cyl["lin_%s_s10_%s" % (name, f)] = m.get(f)
        m.close()
    _save("lapl_cyl", cyl)

    # LaplRect / LaplRectFFT2
    r = {}
    rng = np.random.default_rng(5)
    for (nx, ny) in ((31, 31), (20, 63)):
        rhs = rng.standard_normal((ny, nx))
        dx, dy = 0.1, 0.07
        args = (dx, dy, (nx + 1) * dx, (ny + 1) * dy)
        r["rhs_%dx%d" % (nx, ny)] = rhs
        r["args_%dx%d" % (nx, ny)] = np.array(args)
        r["tri_%dx%d" % (nx, ny)] = R.lapl_rect(rhs, *args, fft2=False)
        if (nx + 1) & nx == 0:
            r["fft2_%dx%d" % (nx, ny)] = R.lapl_rect(rhs, *args, fft2=True)
    # periodic flags (src/lapl_rect.cpp:209-238): y periodic (2) for both
    # methods, y and x periodic (3) for LaplRectFFT2 (with the double-period
    # zero mode) and for LaplRect (whose x stays tridiagonal)
    for tag, fft2, flags, nx, ny in (("tri_py", False, 2, 20, 32), ("fft2_py", True, 2, 31, 64),
                                     ("fft2_pxy", True, 3, 32, 16), ("tri_pxy", False, 3, 15, 8)):
        px = fft2 and flags == 3
        rhs = rng.standard_normal((ny, nx))
        dx, dy = 0.09, 0.13
        args = (dx, dy, (nx if px else nx + 1) * dx, ny * dy)
        r["rhs_" + tag] = rhs
        r["args_" + tag] = np.array(args)
        r["ans_" + tag] = R.lapl_rect_flags(rhs, *args, fft2, flags)
    _save("lapl_rect", r)

    # tridiagonal: Thomas and cyclic reduction on U(-1,1) systems with a
    # dominant diagonal
    t = {}
    rng = np.random.default_rng(9)
    for n in (9, 31, 32, 63, 255):
        lo = rng.uniform(-1, 1, n)
        up = rng.uniform(-1, 1, n)
        dg = rng.uniform(-1, 1, n) + np.sign(rng.uniform(-1, 1, n)) * 3.0
        b = rng.uniform(-1, 1, n)
        lo[0] = 0.0
        up[-1] = 0.0
        t["lo_%d" % n], t["dg_%d" % n], t["up_%d" % n], t["b_%d" % n] = lo, dg, up, b
        # Thomas: lower[j] = A(j+1, j) = lo[j+1]
        t["thomas_%d" % n] = R.thomas(np.r_[lo[1:], 0.0], dg, up, b)
        t["crg_%d" % n] = R.cyclic_reduction(dg, lo, up, b, general=True)
        if (n + 1) & n == 0:
            t["cr_%d" % n] = R.cyclic_reduction(dg, lo, up, b, general=False)
    _save("tdiag", t)

    # NSCube lid-driven cavity, Re=250, dt=0.01, [-pi,pi]^3
    ns = {}
    m = R.nscube(15, 15, 250.0, 0.01)
    m.step(20)
    for name in ("u", "v", "w", "p"):
        ns["n15_s20_" + name] = m.get(name)
    m.step(80)
    for name in ("u", "v", "w", "p", "x"):
        for k, v in checksums(m.get(name)).items():
            ns["n15_s100_%s_%s" % (name, k)] = v
    m.close()
    m = R.nscube(31, 31, 250.0, 0.01)
    m.step(10)
    for name in ("u", "v", "w", "p"):
        for k, v in checksums(m.get(name)).items():
            ns["n31_s10_%s_%s" % (name, k)] = v
    m.close()
    # the 1000-step cavity's own size, 63^3 (64 intervals): the first 10 and
    # 50 steps, checksums plus values at seeded positions
    m = R.nscube(63, 63, 250.0, 0.01)
    for steps, done in ((10, 10), (40, 50)):
        m.step(steps)
        for name in ("u", "v", "w", "p", "x"):
            for k, v in checksums(m.get(name), nsamp=512).items():
                ns["n63_s%d_%s_%s" % (done, name, k)] = v
    m.close()
    # NSCube<float> (src/ns_cube.cpp:281-282), same cavity
    m = R.nscube_float(15, 15, 250.0, 0.01)
    m.step(20)
    for name in ("u", "v", "w", "p"):
        ns["f32_n15_s20_" + name] = m.get(name).astype(np.float32)
    m.step(80)
    for name in ("u", "v", "w", "p"):
        for k, v in checksums(m.get(name)).items():
            ns["f32_n15_s100_%s_%s" % (name, k)] = v
    m.close()
    _save("ns_cube", ns)

    # particle-mesh N-body driver, NBody<T,false,CIC3<T>> (test/nbody.cpp):
    # the constructor's bodies, then the state after 1 and 5 steps
    from oracle.nbody import RefNBody  # noqa: E402
    nb = {}
    for tag, T, N, n, npp, local, solar in NBODY_CASES:
        m = RefNBody(R.L, -10.0, -10.0, -10.0, 20.0, n, npp, N, 0.001, 1.0, 4.0, -1, local, solar, 1.0, dtype=T)
        b = m.bodies()
        for k in ("x", "v", "mass"):
            nb["%s_init_%s" % (tag, k)] = b[k].astype(T)
        nb[tag + "_total_mass"] = np.float64(m.total_mass)
        m.step(1)
        b, fl = m.bodies(), m.fields()
        for k in ("x", "v", "a", "F"):
            nb["%s_s1_%s" % (tag, k)] = b[k].astype(T)
        for k in ("f", "rhs", "psi", "E"):
            nb["%s_s1_%s" % (tag, k)] = fl[k].astype(T)
        m.step(4)
        b = m.bodies()
        for k in ("x", "v", "a", "aprev"):
            nb["%s_s5_%s" % (tag, k)] = b[k].astype(T)
        m.close()
    _save("nbody", nb)
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
