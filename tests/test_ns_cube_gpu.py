"""GPU parity of the NSCube projection step through the C ABI against the
reference's golden fields and the CPU oracle (the reference has no NSCube
unit test; its parity is pinned step by step here)."""
import math

import numpy as np
import pytest

from tests.helpers import rel_l2
from fdm_gb300 import Config, FdmError, NSCube

pytestmark = pytest.mark.gpu

# velocity/pressure relative L2 vs the reference after 1000 steps at 63^3
TOL_1000 = 1e-11


def make(n, Re=250.0, dt=0.01):
    c = Config()
    c.rewrite(["prog", "--ns:nx=%d" % n, "--ns:nz=%d" % n, "--ns:Re=%g" % Re, "--ns:dt=%g" % dt, "--ns:u0=1"])
    return NSCube(c)


def test_golden_15_cube(cuda, golden):
    g = golden("ns_cube")
    m = make(15)
    m.step(20)
    for name in ("u", "v", "w", "p"):
        ref = g["n15_s20_" + name]
        got = m.get(name).data.ravel()
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), name
    m.step(80)
    assert m.time_index == 100
    for name in ("u", "v", "w", "p", "x"):
        got = m.get(name).data.ravel()
        scale = max(1.0, float(g["n15_s100_%s_maxabs" % name]))
        assert np.abs(got[g["n15_s100_%s_idx" % name]] - g["n15_s100_%s_vals" % name]).max() <= 1e-11 * scale, name


def test_golden_31_cube(cuda, golden):
    g = golden("ns_cube")
    m = make(31)
    m.step(10)
    for name in ("u", "v", "w", "p"):
        got = m.get(name).data.ravel()
        scale = max(1.0, float(g["n31_s10_%s_maxabs" % name]))
        assert np.abs(got[g["n31_s10_%s_idx" % name]] - g["n31_s10_%s_vals" % name]).max() <= 1e-12 * scale, name


def test_all_fields_vs_oracle_31(cuda, port):
    m = make(31)
    o = port.nscube(31, 31, 250.0, 0.01)
    for _ in range(3):
        m.step(5)
        o.step(5)
        for name in ("u", "v", "w", "p", "x", "F", "G", "H", "RHS"):
            got = m.get(name).data.ravel()
            ref = o.get(name)
            assert np.abs(got - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max()), name


def test_config1_1000_steps_63(cuda, port):
    """Cavity at 63^3 (64 intervals), Re=250, dt=0.01, 1000 steps."""
    m = make(63)
    o = port.nscube(63, 63, 250.0, 0.01)
    m.step(1000)
    o.step(1000)
    for name in ("u", "v", "w", "p"):
        got = m.get(name).data.ravel()
        ref = o.get(name)
        assert rel_l2(got, ref) <= TOL_1000, name


def test_reference_field_layout(cuda):
    m = make(7)
    r = {k: m.field_info(k)[1] for k in ("u", "v", "w", "p", "x", "F", "G", "H", "RHS")}
    assert r["u"] == (0, 8, 0, 8, -1, 8)
    assert r["v"] == (0, 8, -1, 8, 0, 8)
    assert r["w"] == (-1, 8, 0, 8, 0, 8)
    assert r["p"] == (0, 8, 0, 8, 0, 8)
    assert r["x"] == r["RHS"] == (1, 7, 1, 7, 1, 7)
    assert r["F"] == (1, 7, 1, 7, 0, 7)
    assert r["G"] == (1, 7, 0, 7, 1, 7)
    assert r["H"] == (0, 7, 1, 7, 1, 7)
    m.step(1)
    u = m.u
    # lid ghost set at the start of step 1 from the zero state: 2*U0 - 0
    assert u[8, 3, 3] == 2.0


def test_bad_size(cuda):
    with pytest.raises(FdmError):
        make(64)


def test_constant_division_matches_ieee(cuda):
    """The stencils divide by run constants through a precomputed reciprocal
    and two remainder corrections; on dividends and divisors spread over the
    normal range (quotients normal too), zeros, the cavity's own constants
    and divisors with all-ones significands it equals IEEE a/b bit for bit."""
    import torch
    from fdm_gb300 import _native as N
    rng = np.random.default_rng(17)
    n = 1 << 22
    a = rng.uniform(1, 2, n) * np.exp2(rng.integers(-500, 500, n)) * rng.choice((-1, 1), n)
    b = rng.uniform(1, 2, n) * np.exp2(rng.integers(-500, 500, n)) * rng.choice((-1, 1), n)
    h = 2 * math.pi / 64
    consts = np.array([100.0, 250.0, 400.0, 0.01, h, h * h, 2 * math.pi / 32, (2 * math.pi / 32) ** 2,
                       np.nextafter(2.0, 0.0), np.nextafter(1.0, 0.0) * 2.0 ** 7, 3.0, 10.0])
    b[: 1 << 20] = np.resize(consts, 1 << 20) * rng.choice((-1, 1), 1 << 20)
    a[: 1 << 16] = rng.uniform(-1, 1, 1 << 16)
    a[1 << 16: (1 << 16) + 64] = 0.0
    a[(1 << 16) + 64: (1 << 16) + 128] = -0.0
    a[(1 << 17): (1 << 17) + 4096] = np.exp2(rng.integers(-60, 60, 4096))  # powers of two
    ta, tb = torch.tensor(a, device=cuda), torch.tensor(b, device=cuda)
    q1, q2 = torch.empty_like(ta), torch.empty_like(ta)
    N.check(N.load().fdmgpu_check_const_division(n, ta.data_ptr(), tb.data_ptr(), q1.data_ptr(), q2.data_ptr(),
                                                 None))
    torch.cuda.synchronize()
    x, y = q1.cpu().numpy(), q2.cpu().numpy()
    assert np.array_equal(x.view(np.int64), (a / b).view(np.int64))  # the device's IEEE division
    bad = np.flatnonzero(x.view(np.int64) != y.view(np.int64))
    assert bad.size == 0, (bad.size, a[bad[:4]], b[bad[:4]])
