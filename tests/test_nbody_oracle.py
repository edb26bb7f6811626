"""CPU checks of the N-body restatement (oracle/nbody.py) against the golden
fixtures made by the reference's own NBody class (tests/golden/nbody.npz,
tests/golden/make_golden.py).  No GPU."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle.nbody import NBodyPort, init_bodies, minstd_rand0, uniform01

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "nbody.npz")

# tag, T, N, n, npp, local, solar: the cases of make_golden.NBODY_CASES
CASES = (
    ("d", np.float64, 400, 16, 8, 0, 0),
    ("d_pp", np.float64, 400, 8, 8, 1, 0),
    ("f", np.float32, 400, 16, 8, 0, 0),
    ("f_pp", np.float32, 400, 8, 8, 1, 0),
    ("solar", np.float64, 0, 16, 8, 1, 1),
)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_minstd_known_answers():
    g = minstd_rand0(10000)
    assert list(g[:3]) == [16807, 282475249, 1622650073]
    # the C++ standard's check value for minstd_rand0: its 10000th output
    assert g[-1] == 1043618065
    u = uniform01(5, np.float64)
    assert np.all((u >= 0) & (u < 1))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_init_points_bit_exact(case):
    tag, T, N, n, npp, local, solar = case
    x, v, m, g, total = init_bodies(N, 20.0, np.array([-10.0] * 3, T), 4.0, bool(solar), T)
    assert np.array_equal(x, GOLD[tag + "_init_x"])
    assert np.array_equal(v, GOLD[tag + "_init_v"])
    assert np.array_equal(m, GOLD[tag + "_init_mass"])
    assert total == float(GOLD[tag + "_total_mass"])


def _port(case):
    tag, T, N, n, npp, local, solar = case
    return NBodyPort(-10.0, -10.0, -10.0, 20.0, n, npp, N, 0.001, 1.0, 4.0, -1, local, solar, 1.0, dtype=T)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_step_matches_reference(case):
    tag, T, N, n, npp, local, solar = case
    p = _port(case)
    p.step(1)
    # the density and right-hand side are gathered in the reference's order
    assert np.array_equal(p.f, GOLD[tag + "_s1_f"])
    assert np.array_equal(p.rhs, GOLD[tag + "_s1_rhs"])
    # pair forces in the reference's order and arithmetic
    assert np.array_equal(p.F, GOLD[tag + "_s1_F"])
    tol = 1e-13 if T == np.float64 else 2e-6  # the periodic solve: numpy FFT vs the reference's
    assert rel(p.psi, GOLD[tag + "_s1_psi"]) <= tol
    assert rel(p.E, GOLD[tag + "_s1_E"]) <= tol
    assert rel(p.a, GOLD[tag + "_s1_a"]) <= tol
    assert rel(p.x, GOLD[tag + "_s1_x"]) <= (1e-15 if T == np.float64 else 1e-7)
    assert rel(p.v, GOLD[tag + "_s1_v"]) <= tol
    p.step(4)
    assert np.abs(p.x.astype(np.float64) - GOLD[tag + "_s5_x"]).max() <= (1e-12 if T == np.float64 else 1e-5)
    assert rel(p.a, GOLD[tag + "_s5_a"]) <= (1e-12 if T == np.float64 else 1e-5)
    assert rel(p.aprev, GOLD[tag + "_s5_aprev"]) <= (1e-12 if T == np.float64 else 1e-5)


def test_parity_classes_and_list_lifecycle():
    """Only all-even / all-odd cells deposit; calc_a_pm without a move leaves
    the lists empty, so the next step deposits nothing."""
    p = _port(CASES[0])
    cells = np.floor((p.x - p.origin).astype(np.float64) / p.h).astype(int) % p.n
    visited = np.all(cells % 2 == cells[:, :1] % 2, axis=1)
    p.calc_a_pm()
    deposited = p.f.astype(np.float64).sum() - p.n ** 3 * float(np.float64(-p.total_mass / 20.0 ** 3))
    assert abs(deposited - float(p.mass[visited].astype(np.float64).sum())) <= 1e-9 * p.total_mass
    p.calc_a_pm()
    assert np.all(p.f == p.f[0])
    assert np.all(p.F == 0)


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_cic3_known_answers(T):
    """ut/ut_interpolate.cpp test_CIC3 (:67-114) on the restatement's CIC."""
    p = NBodyPort(0.0, 0.0, 0.0, 8.0, 8, 8, 1, 0.001, 1.0, dtype=T,
                  bodies=(np.array([[0.5, 0.5, 0.5]]), np.zeros((1, 3)), np.array([10.0])))
    c0, M = p._cic()
    assert list(c0[0]) == [0, 0, 0]
    assert np.all(np.abs(10.0 * M[:, 0].astype(np.float64) - 10.0 / 8.0) <= 1e-12)
    p.set_bodies(np.array([[0.5, 0.6, 0.7]]), np.zeros((1, 3)), np.array([10.0]))
    c0, M = p._cic()
    assert list(c0[0]) == [0, 0, 0]
    assert abs(float(np.sum(T(10.0) * M[:, 0])) - 10.0) <= (1e-12 if T == np.float64 else 1e-5)
