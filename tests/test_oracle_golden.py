"""Pins the CPU oracle (oracle/fdm_oracle.c) to the reference's own outputs
stored in tests/golden (generated by tests/golden/make_golden.py from the
compiled reference), and ports the reference unit tests' assertions:
ut/ut_fft.cpp test_sin / test_sin_new, ut/ut_lapl_cube.cpp test_lapl_cube,
ut/ut_lapl_rect.cpp test_lapl_rect_fft1_fft2_cmp, ut/ut_tdiag.cpp."""
import math

import numpy as np
import pytest

from tests.helpers import rel_l2
from fdm_gb300 import workloads


@pytest.mark.parametrize("N", [2, 8, 32, 256, 1024])
def test_sfft_matches_reference(port, golden, N):
    g = golden("dst")
    s = g["s_%d" % N]
    assert np.abs(port.sfft(s, 1.0)[1:] - g["S_%d" % N][1:]).max() <= 1e-12 * max(1.0, np.abs(g["S_%d" % N]).max())
    assert np.abs(port.sfft(s, 0.5)[1:] - g["Sh_%d" % N][1:]).max() <= 1e-12 * max(1.0, np.abs(g["Sh_%d" % N]).max())


def test_sfft_roundtrip_and_naive(port):
    # ut/ut_fft.cpp:190-228: S = sFFT(s); s' = sFFT(S) * 2/N recovers s
    N = 1024
    s = np.random.default_rng(0).uniform(-1, 1, N)
    s[0] = 0
    S = port.sfft(s, 1.0)
    s1 = port.sfft(S, 2.0 / N)
    assert np.abs(s1[1:N - 1] - s[1:N - 1]).max() <= 1e-13
    S2 = port.sft_naive(S, 2.0 / N)
    assert np.abs(s1[1:N - 1] - S2[1:N - 1]).max() <= 1e-12


def test_sfft_rejects_non_power_of_two(port):
    with pytest.raises(ValueError):
        port.sfft(np.zeros(12))


def test_lapl_cube_matches_reference(port, golden):
    g = golden("lapl_cube")
    a = workloads.solver_args(15, 15, 15)
    assert rel_l2(port.lapl_cube(g["m15_rhs"], *a[:6]), g["m15_ans"]) <= 1e-14
    assert rel_l2(port.lapl_cube(g["aniso_rhs"], *g["aniso_args"]), g["aniso_ans"]) <= 1e-14
    assert rel_l2(port.lapl_cube(g["lz_rhs"], *g["lz_args"]), g["lz_ans"]) <= 1e-14


def test_lapl_cube_config0_checksums(port, golden):
    g = golden("lapl_cube")
    f, u = workloads.manufactured(31, 31, 31, seed=0, kmax=12)
    # the generator still produces the input the fixture was made from
    assert abs(f.sum() - g["c0_rhs_sum"]) <= 1e-9 * abs(g["c0_rhs_l2"])
    assert np.allclose(f.ravel()[g["c0_rhs_idx"]], g["c0_rhs_vals"], rtol=0, atol=1e-12 * g["c0_rhs_maxabs"])
    ans = port.lapl_cube(f, *workloads.solver_args(31, 31, 31)[:6])
    assert np.allclose(ans.ravel()[g["c0_ans_idx"]], g["c0_ans_vals"], rtol=0, atol=1e-13 * g["c0_ans_maxabs"])
    assert abs(np.linalg.norm(ans) - g["c0_ans_l2"]) <= 1e-13 * g["c0_ans_l2"]
    # manufactured solution recovered to round-off
    assert rel_l2(ans, u) <= 1e-13


def test_lapl_cube_reference_unit_case(port, golden):
    from tests.golden.make_golden import ut_lapl_cube_rhs
    g = golden("lapl_cube")
    rhs, exact, args = ut_lapl_cube_rhs(31)
    ans = port.lapl_cube(rhs, *args)
    err = np.abs(ans - exact).max() / np.abs(exact).max()
    assert err < 1e-4  # ut/ut_lapl_cube.cpp:124
    assert abs(err - g["ut31_err"]) <= 1e-12
    assert np.allclose(ans.ravel()[g["ut31_ans_idx"]], g["ut31_ans_vals"], rtol=0, atol=1e-13 * g["ut31_ans_maxabs"])


def test_lapl_rect_matches_reference(port, golden):
    g = golden("lapl_rect")
    for key in ("31x31", "20x63"):
        rhs, args = g["rhs_" + key], g["args_" + key]
        assert rel_l2(port.lapl_rect(rhs, *args), g["tri_" + key]) <= 1e-14
        if "fft2_" + key in g:
            assert rel_l2(port.lapl_rect(rhs, *args, fft2=True), g["fft2_" + key]) <= 1e-14


def _ut_lapl_rect_case(n=31):
    """ut/ut_lapl_rect.cpp:21-33, 48-88: u = sin^2 x + cos^2 y at the cell
    centres of [0,1]^2 (x = x1 + j dx - dx/2), f its Laplacian, the boundary
    values folded into the right-hand side; LaplRect(dx, dy, 1+dx, 1+dy, n, n)."""
    dx = dy = 1.0 / n
    k, j = np.meshgrid(np.arange(1, n + 1), np.arange(1, n + 1), indexing="ij")

    def ans(k, j):
        x, y = j * dx - dx / 2, k * dy - dy / 2
        return np.sin(x) ** 2 + np.cos(y) ** 2

    x, y = j * dx - dx / 2, k * dy - dy / 2
    rhs = 2 * np.sin(y) ** 2 - 2 * np.cos(y) ** 2 - 2 * np.sin(x) ** 2 + 2 * np.cos(x) ** 2
    rhs[0, :] -= ans(k[0, :] - 1, j[0, :]) / dy / dy
    rhs[:, 0] -= ans(k[:, 0], j[:, 0] - 1) / dx / dx
    rhs[:, -1] -= ans(k[:, -1], j[:, -1] + 1) / dx / dx
    rhs[-1, :] -= ans(k[-1, :] + 1, j[-1, :]) / dy / dy
    return rhs, ans(k, j), (dx, dy, 1.0 + dx, 1.0 + dy)


@pytest.mark.parametrize("fft2", [False, True])
def test_lapl_rect_reference_unit_case(port, fft2):
    """ut/ut_lapl_rect.cpp test_lapl_rect: relative max-norm error < 3e-3
    (:116) for the DST + tridiagonal and the all-DST formulations."""
    rhs, exact, args = _ut_lapl_rect_case(31)
    got = port.lapl_rect(rhs, *args, fft2=fft2)
    err = np.abs(got - exact).max() / np.abs(exact).max()
    assert err < 3e-3


def test_lapl_rect_two_formulations_agree(port):
    # ut/ut_lapl_rect.cpp:384-456 (511^2, |delta| <= 1e-15 absolute)
    n = 511
    rhs = np.random.default_rng(2).uniform(-1, 1, (n, n))
    h = 1.0 / (n + 1)
    a = port.lapl_rect(rhs, h, h, 1.0, 1.0)
    b = port.lapl_rect(rhs, h, h, 1.0, 1.0, fft2=True)
    assert np.abs(a - b).max() <= 1e-14 * max(1.0, np.abs(a).max())


@pytest.mark.parametrize("n", [9, 31, 32, 63, 255])
def test_tridiagonal_matches_reference(port, golden, n):
    g = golden("tdiag")
    lo, dg, up, b = g["lo_%d" % n], g["dg_%d" % n], g["up_%d" % n], g["b_%d" % n]
    th = port.thomas(np.r_[lo[1:], 0.0], dg, up, b)
    assert np.abs(th - g["thomas_%d" % n]).max() <= 1e-15 * 10
    crg = port.cyclic_reduction(dg, lo, up, b, general=True)
    assert np.abs(crg - g["crg_%d" % n]).max() <= 1e-15 * 10
    assert np.abs(crg - th).max() <= 1e-13  # ut/ut_tdiag.cpp: CR vs Thomas
    if "cr_%d" % n in g:
        cr = port.cyclic_reduction(dg, lo, up, b, general=False)
        assert np.abs(cr - g["cr_%d" % n]).max() <= 1e-15 * 10


def test_nscube_matches_reference(port, golden):
    g = golden("ns_cube")
    m = port.nscube(15, 15, 250.0, 0.01)
    m.step(20)
    for name in ("u", "v", "w", "p"):
        ref = g["n15_s20_" + name]
        assert np.abs(m.get(name) - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), name
    m.step(80)
    for name in ("u", "v", "w", "p", "x"):
        a = m.get(name)
        ref_vals = g["n15_s100_%s_vals" % name]
        scale = max(1.0, float(g["n15_s100_%s_maxabs" % name]))
        assert np.abs(a[g["n15_s100_%s_idx" % name]] - ref_vals).max() <= 1e-11 * scale, name
    m.close()


def _check_n63(get, g, done):
    for name in ("u", "v", "w", "p", "x"):
        a = get(name).ravel()
        pre = "n63_s%d_%s_" % (done, name)
        scale = max(1.0, float(g[pre + "maxabs"]))
        assert np.abs(a[g[pre + "idx"]] - g[pre + "vals"]).max() <= 1e-12 * scale, (done, name)
        assert abs(np.linalg.norm(a) - float(g[pre + "l2"])) <= 1e-12 * float(g[pre + "l2"]), (done, name)


def test_nscube_63_matches_reference(port, golden):
    """The 1000-step cavity's size (63^3): the restatement against the
    reference's fields after 10 and 50 steps (checksums and 512 sampled
    values per field)."""
    g = golden("ns_cube")
    m = port.nscube(63, 63, 250.0, 0.01)
    m.step(10)
    _check_n63(m.get, g, 10)
    m.step(40)
    _check_n63(m.get, g, 50)
    m.close()


def test_nscube_rejects_bad_size(port):
    with pytest.raises(ValueError):
        port.nscube(32, 32, 250.0, 0.01)


def test_periodic_transforms_match_reference(golden):
    """The restated pFFT_1 / pFFT layouts against the reference's own
    FFT<double> on the fixture vectors."""
    from oracle.oracle import pfft, pfft1
    g = golden("lapl_cube_periodic")
    for N in (8, 64, 512):
        s = g["pf_s_%d" % N]
        assert np.abs(pfft1(s, 0.7) - g["pf1_%d" % N]).max() <= 1e-13 * N
        assert np.abs(pfft(s, 0.3) - g["pf_%d" % N]).max() <= 1e-13 * N
        # round trip of the reference's convention: pFFT_1(pFFT(s, 1), 2/N) = s
        assert np.abs(pfft1(pfft(s, 1.0), 2.0 / N) - s).max() <= 1e-14 * N


def test_periodic_3d_transforms_match_reference(golden):
    """pFFT_1_3d / pFFT_3d restated (x, y, z passes of pFFT_1 / pFFT) against
    the reference's own FFT<double> on test_fft_3d_bench.cpp's cube."""
    from oracle.oracle import pfft3d
    g = golden("lapl_cube_periodic")
    for N in (8, 32):
        s = g["fft3d_in_%d" % N]
        for inv, key in ((False, "fft3d_fwd_%d"), (True, "fft3d_inv_%d")):
            ref = g[key % N]
            assert np.abs(pfft3d(s, 1.0, inverse=inv) - ref).max() <= 1e-13 * N * np.abs(ref).max()


def test_periodic_lapl_cube_reference_unit_case():
    """ut/ut_lapl_cube.cpp test_lapl_cube_periodic (:134-243): n = 32 on
    [0, 2 pi]^3, u = sin^3 x + cos^5 y - sin z and its Laplacian at the cell
    centres (x = j h - h/2), the answer's mean removed as the test does
    (dividing by nz*ny*nz), relative max-norm error < 1e-2."""
    from oracle.oracle import lapl_cube_periodic
    n = 32
    h = 2 * np.pi / n
    i, k, j = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    x, y, z = j * h - h / 2, k * h - h / 2, i * h - h / 2
    rhs = (1.0 / 16.0) * (-12.0 * np.sin(x) + 36.0 * np.sin(3 * x) - 10.0 * np.cos(y) - 45.0 * np.cos(3 * y)
                          - 25.0 * np.cos(5 * y) + 16.0 * np.sin(z))
    exact = np.sin(x) ** 3 + np.cos(y) ** 5 - np.sin(z)
    ans = lapl_cube_periodic(rhs, h, h, h, 2 * np.pi, 2 * np.pi, 2 * np.pi)
    ans = ans - ans.sum() / (n * n * n)
    err = np.abs(ans - exact).max() / np.abs(exact).max()
    assert err < 1e-2


def test_periodic_lapl_cube_matches_reference(golden):
    from oracle.oracle import lapl_cube_periodic
    g = golden("lapl_cube_periodic")
    for name in ("c16", "a8x16x32", "b32x16x16"):
        ans = lapl_cube_periodic(g["rhs_" + name], *g["args_" + name])
        ref = g["ans_" + name]
        assert np.linalg.norm(ans - ref) / np.linalg.norm(ref) <= 1e-14, name


def test_cylindrical_matches_reference(golden):
    """LaplCyl3FFT2 restated against the compiled reference (its LAPACK
    gttrf / gttrs mapped to elimination without row swaps)."""
    from oracle.oracle import lapl_cyl
    g = golden("lapl_cyl")
    for name, pz in (("d16x15x20", False), ("p8x16x12", True), ("d32x31x7", False)):
        ans = lapl_cyl(g["rhs_" + name], *g["args_" + name], periodic_z=pz)
        ref = g["ans_" + name]
        assert np.linalg.norm(ans - ref) / np.linalg.norm(ref) <= 1e-14, name


RECT_FLAG_CASES = (("tri_py", False, 2), ("fft2_py", True, 2), ("fft2_pxy", True, 3), ("tri_pxy", False, 3))


@pytest.mark.parametrize("tag,fft2,flags", RECT_FLAG_CASES)
def test_periodic_rect_matches_reference(golden, tag, fft2, flags):
    """LaplRect / LaplRectFFT2 with periodic flags restated against the
    reference's own instantiations."""
    from oracle.oracle import lapl_rect_flags
    g = golden("lapl_rect")
    ans = lapl_rect_flags(g["rhs_" + tag], *g["args_" + tag], fft2, flags)
    ref = g["ans_" + tag]
    assert np.linalg.norm(ans - ref) / np.linalg.norm(ref) <= 1e-13
