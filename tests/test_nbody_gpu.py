"""GPU parity of the particle-mesh N-body step (libfdmgpu.so, fdmgpu_nbody_*)
against the reference's own NBody (golden fixtures) and the restatement
(oracle/nbody.py)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD_PATH = Path(__file__).resolve().parent / "golden" / "nbody.npz"

CASES = (
    ("d", np.float64, 400, 16, 8, 0, 0),
    ("d_pp", np.float64, 400, 8, 8, 1, 0),
    ("f", np.float32, 400, 16, 8, 0, 0),
    ("f_pp", np.float32, 400, 8, 8, 1, 0),
    ("solar", np.float64, 0, 16, 8, 1, 1),
)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD_PATH)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make(case, **kw):
    from fdm_gb300 import NBody

    tag, T, N, n, npp, local, solar = case
    args = dict(x0=-10.0, y0=-10.0, z0=-10.0, l=20.0, n=n, npp=npp, N_bodies=N, dt=0.001, G=1.0, vel=4.0, sgn=-1,
                local=local, solar=solar, crit=1.0, dtype=T)
    args.update(kw)
    return NBody(**args)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_nbody_matches_reference(gold, case):
    tag, T, N, n, npp, local, solar = case
    nb = make(case)
    b = nb.bodies()
    # init_points: the same draws, bit for bit
    assert np.array_equal(b["x"], gold[tag + "_init_x"])
    assert np.array_equal(b["v"], gold[tag + "_init_v"])
    assert np.array_equal(b["mass"], gold[tag + "_init_mass"])
    assert nb.mass == float(gold[tag + "_total_mass"])
    nb.step(1)
    b = nb.bodies()
    # density and right-hand side gathered in the reference's order: exact
    assert np.array_equal(nb.field("f").ravel(), gold[tag + "_s1_f"])
    assert np.array_equal(nb.field("rhs").ravel(), gold[tag + "_s1_rhs"])
    # the periodic solve and everything after it: FFT round-off; the pair
    # forces use the device's erfc / exp
    tol = 1e-12 if T == np.float64 else 2e-6
    assert rel(nb.field("psi").ravel(), gold[tag + "_s1_psi"]) <= tol
    assert rel(nb.field("E").reshape(-1, 3), gold[tag + "_s1_E"]) <= tol
    assert rel(b["F"], gold[tag + "_s1_F"]) <= (1e-13 if T == np.float64 else 1e-6)
    assert rel(b["a"], gold[tag + "_s1_a"]) <= tol
    assert rel(b["x"], gold[tag + "_s1_x"]) <= (1e-15 if T == np.float64 else 1e-7)
    assert rel(b["v"], gold[tag + "_s1_v"]) <= tol
    nb.step(4)
    b = nb.bodies()
    assert nb.steps == 5
    xtol = 1e-12 if T == np.float64 else 1e-5
    assert np.abs(b["x"].astype(np.float64) - gold[tag + "_s5_x"]).max() <= xtol
    assert rel(b["a"], gold[tag + "_s5_a"]) <= (1e-11 if T == np.float64 else 1e-5)
    assert rel(b["aprev"], gold[tag + "_s5_aprev"]) <= (1e-11 if T == np.float64 else 1e-5)
    nb.close()


def test_nbody_full_size_density_and_forces():
    """N = 100000 bodies on the 32^3 mass grid (the driver's defaults): the
    density bit-exact and the accelerations to round-off against the
    restatement, on the same bodies."""
    from oracle.nbody import NBodyPort

    nb = make(("full", np.float64, 100000, 32, 64, 0, 0))
    b = nb.bodies()
    p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 32, 64, 100000, 0.001, 1.0, dtype=np.float64,
                  bodies=(b["x"], b["v"], b["mass"]))
    p.calc_a_pm()
    nb.step(1)
    assert np.array_equal(nb.field("f").ravel(), p.f)
    assert np.array_equal(nb.field("rhs").ravel(), p.rhs)
    assert rel(nb.bodies()["a"], p.a) <= 1e-12
    p.move()
    assert rel(nb.bodies()["x"], p.x) <= 1e-15
    nb.close()


def test_nbody_pair_forces_full_pp_grid():
    """local = 1 with an npp grid finer than n (the images at +l only when a
    neighbour index reaches n, as in the reference), against the restatement."""
    from oracle.nbody import NBodyPort

    case = ("pp", np.float64, 3000, 16, 32, 1, 0)
    nb = make(case)
    b = nb.bodies()
    p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 16, 32, 3000, 0.001, 1.0, local=1, dtype=np.float64,
                  bodies=(b["x"], b["v"], b["mass"]))
    nb.step(1)
    p.calc_a_pm()
    got = nb.bodies()
    assert np.count_nonzero(p.F) > 0
    assert rel(got["F"], p.F) <= 1e-13
    assert rel(got["a"], p.a) <= 1e-12
    nb.close()


def test_nbody_crowded_cell_uses_big_bins():
    """Hundreds of bodies in one cell take the warp rank sort; the density
    stays bit-exact (index order within the cell)."""
    from oracle.nbody import NBodyPort

    rng = np.random.default_rng(5)
    Nb = 700
    x = np.empty((Nb, 3))
    x[:500] = rng.uniform(0.1, 1.1, size=(500, 3))  # one cell of the 16^3 grid (h = 1.25)
    x[500:] = rng.uniform(-10, 10, size=(200, 3))
    perm = rng.permutation(Nb)
    x = x[perm]
    v = rng.normal(size=(Nb, 3))
    m = rng.uniform(0.2, 1.7, size=Nb)
    nb = make(("big", np.float64, Nb, 16, 8, 1, 0))
    nb.set_bodies(x, v, m)
    p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 16, 8, Nb, 0.001, 1.0, local=1, dtype=np.float64, bodies=(x, v, m))
    nb.step(1)
    p.calc_a_pm()
    assert np.array_equal(nb.field("f").ravel(), p.f)
    assert rel(nb.bodies()["F"], p.F) <= 1e-12
    assert rel(nb.bodies()["a"], p.a) <= 1e-12
    nb.close()


def test_nbody_calc_error_and_list_lifecycle():
    from oracle.nbody import NBodyPort

    nb = make(("err", np.float64, 2000, 32, 16, 0, 0))
    b = nb.bodies()
    p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 32, 16, 2000, 0.001, 1.0, dtype=np.float64,
                  bodies=(b["x"], b["v"], b["mass"]))
    err = nb.calc_error()
    assert err.shape == (2000,) and np.all(np.isfinite(err))
    # the pair sum against the restatement (pairwise numpy sums: round-off)
    assert rel(nb.direct_forces(), p.direct_forces()) <= 1e-12
    # calc_a_pm empties the cell lists: the next step deposits nothing
    nb.step(1)
    f = nb.field("f")
    assert np.all(f == f.ravel()[0])
    nb.close()


def test_nbody_errors():
    import ctypes

    from fdm_gb300 import FdmError
    from fdm_gb300 import _native as N

    with pytest.raises(FdmError) as e:
        make(("bad", np.float64, 10, 24, 8, 0, 0))  # n not a power of two
    assert e.value.status == N.ESIZE
    nb = make(("ok", np.float64, 10, 8, 8, 0, 0))
    buf = np.zeros(3)
    with pytest.raises(FdmError) as e:
        N.check(nb._lib.fdmgpu_nbody_get_field(nb._h, 0, buf.ctypes.data, ctypes.c_size_t(3)))
    assert e.value.status == N.EINVAL
    with pytest.raises(FdmError) as e:
        N.check(nb._lib.fdmgpu_nbody_get_field(nb._h, 7, buf.ctypes.data, ctypes.c_size_t(3)))
    assert e.value.status == N.EINVAL
    nb.close()


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_nbody_cic3_known_answers(T):
    """ut/ut_interpolate.cpp test_CIC3 (:67-114) through the device deposit:
    a body of mass 10 at (0.5, 0.5, 0.5) with h = 1 puts m/8 on each corner
    of cell 0; at (0.5, 0.6, 0.7) the eight shares sum to m."""
    nb = make(("cic", T, 1, 8, 8, 0, 0), x0=0.0, y0=0.0, z0=0.0, l=8.0)
    f0 = float(T(-10.0 / 8.0 / 8.0 / 8.0))
    for pos, exact in (((0.5, 0.5, 0.5), True), ((0.5, 0.6, 0.7), False)):
        nb.set_bodies(np.array([pos]), np.zeros((1, 3)), np.array([10.0]))
        nb.step(1)
        f = nb.field("f").astype(np.float64)
        corner = f[:2, :2, :2] - f0
        assert np.all(np.delete(f.ravel(), [i * 64 + k * 8 + j for i in (0, 1) for k in (0, 1) for j in (0, 1)])
                      == f0)
        if exact:
            assert np.all(np.abs(corner - 10.0 / 8.0) <= (1e-12 if T == np.float64 else 1e-5))
        assert abs(corner.sum() - 10.0) <= (1e-12 if T == np.float64 else 1e-5)
    nb.close()


def test_nbody_float_full_size_against_restatement():
    """NBody<float> at the driver's defaults (100000 bodies, 32^3): the
    density bit for bit and the accelerations to float round-off against the
    restatement in float."""
    from oracle.nbody import NBodyPort

    nb = make(("full32", np.float32, 100000, 32, 64, 0, 0))
    b = nb.bodies()
    p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 32, 64, 100000, 0.001, 1.0, dtype=np.float32,
                  bodies=(b["x"], b["v"], b["mass"]))
    p.calc_a_pm()
    nb.step(1)
    assert np.array_equal(nb.field("f").ravel(), p.f)
    assert np.array_equal(nb.field("rhs").ravel(), p.rhs)
    # the device solves the periodic problem in FP32 (as NBody<float> does),
    # the restatement in FP64: FP32 solve round-off, sharpened by the field's
    # differences
    assert rel(nb.bodies()["a"], p.a) <= 1e-5
    nb.close()
