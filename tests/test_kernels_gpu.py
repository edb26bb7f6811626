"""GPU parity of the 1-D building blocks and LaplRect through the C ABI:
the DST-I line transform (FFT<T>::sFFT), the tridiagonal solver
(solve_tdiag_linear_my / cyclic_reduction) and LaplRect / LaplRectFFT2."""
import numpy as np
import pytest

from tests.helpers import rel_l2
from fdm_gb300 import LaplRect, LaplRectFFT2, sine_transform_device, tridiag_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [2, 4, 8, 32, 64, 128, 256, 512, 1024])
def test_sine_f64_vs_reference(cuda, golden, port, N):
    import torch
    g = golden("dst")
    rng = np.random.default_rng(N)
    lines = rng.uniform(-1, 1, (37, N - 1))
    if "s_%d" % N in g:
        lines[0] = g["s_%d" % N][1:]
    x = torch.from_numpy(lines).to(cuda)
    y = torch.empty_like(x)
    sine_transform_device(y, x, N, 37, 0.5)
    torch.cuda.synchronize()
    out = y.cpu().numpy()
    for i in range(37):
        s = np.r_[0.0, lines[i]]
        ref = port.sfft(s, 0.5)[1:]
        assert np.abs(out[i] - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    if "s_%d" % N in g:
        assert np.abs(out[0] - g["Sh_%d" % N][1:]).max() <= 1e-13 * max(1.0, np.abs(g["Sh_%d" % N]).max())


@pytest.mark.parametrize("N", [32, 256, 1024])
def test_sine_f32_roundtrip(cuda, golden, N):
    """FP32 round trip s' = DST(DST(s) * 1) * 2/N on 64 uniform(-1,1) lines.
    The bar is the reference's own float sFFT on the same lines (golden
    f32_roundtrip_err_N: 5.4e-6 at N=256, 1.9e-5 at N=1024): both compute the
    odd outputs as running sums, whose error grows like sqrt(N)."""
    import torch
    from tests.golden.make_golden import f32_line
    ref_err = float(golden("dst")["f32_roundtrip_err_%d" % N])
    x = torch.tensor(np.stack([f32_line(N, t) for t in range(64)]), device=cuda)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    sine_transform_device(y, x, N, 64, 1.0, dtype=np.float32)
    sine_transform_device(z, y, N, 64, 2.0 / N, dtype=np.float32)
    torch.cuda.synchronize()
    assert (z - x).abs().max().item() <= 3.0 * ref_err


@pytest.mark.parametrize("n", [9, 31, 32, 63, 255])
def test_tridiag_vs_reference(cuda, golden, n):
    import torch
    g = golden("tdiag")
    lo, dg, up, b = g["lo_%d" % n], g["dg_%d" % n], g["up_%d" % n], g["b_%d" % n]
    # two systems interleaved: the golden one and its negation
    L = torch.tensor(np.stack([lo, lo], 1).ravel(), device=cuda)
    D = torch.tensor(np.stack([dg, dg], 1).ravel(), device=cuda)
    U = torch.tensor(np.stack([up, up], 1).ravel(), device=cuda)
    B = torch.tensor(np.stack([b, -b], 1).ravel(), device=cuda)
    tridiag_device(L, D, U, B, n, 2)
    torch.cuda.synchronize()
    x = B.cpu().numpy().reshape(n, 2)
    assert np.abs(x[:, 0] - g["thomas_%d" % n]).max() <= 1e-13
    assert np.abs(x[:, 1] + g["crg_%d" % n]).max() <= 1e-13


def test_rect_vs_reference(cuda, golden):
    g = golden("lapl_rect")
    for key, (nx, ny) in (("31x31", (31, 31)), ("20x63", (20, 63))):
        rhs, args = g["rhs_" + key], tuple(g["args_" + key])
        r = LaplRect(*args, nx, ny)
        ans = np.zeros_like(rhs)
        r.solve(ans, rhs)
        assert rel_l2(ans, g["tri_" + key]) <= 1e-12
        if "fft2_" + key in g:
            r2 = LaplRectFFT2(*args, nx, ny)
            ans2 = np.zeros_like(rhs)
            r2.solve(ans2, rhs)
            assert rel_l2(ans2, g["fft2_" + key]) <= 1e-12


@pytest.mark.parametrize("tag,fft2,flags", [("tri_py", False, 2), ("fft2_py", True, 2), ("fft2_pxy", True, 3),
                                             ("tri_pxy", False, 3)])
def test_rect_periodic_flags_vs_reference(cuda, golden, tag, fft2, flags):
    """LaplRect / LaplRectFFT2 with the reference's periodic flags (y, or y
    and x; the doubly periodic FFT2 sets its zero mode to 1 as the reference
    does), FP64 and FP32, host and device entry points."""
    import torch
    g = golden("lapl_rect")
    rhs, args, ref = g["rhs_" + tag], tuple(g["args_" + tag]), g["ans_" + tag]
    ny, nx = rhs.shape
    cls = LaplRectFFT2 if fft2 else LaplRect
    kw = dict(periodic_y=True, periodic_x=flags == 3)
    r = cls(*args, nx, ny, **kw)
    ans = np.zeros_like(rhs)
    r.solve(ans, rhs)
    assert rel_l2(ans, ref) <= 1e-12
    r32 = cls(*args, nx, ny, dtype=np.float32, **kw)
    a32 = np.zeros(rhs.shape, np.float32)
    r32.solve(a32, rhs.astype(np.float32))
    assert rel_l2(a32.astype(np.float64), ref) <= 1e-5
    two = torch.tensor(np.stack([rhs, rhs]), device=cuda)
    out = torch.empty_like(two)
    r.solve_device(out, two, nrhs=2)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert np.array_equal(o[0], ans) and np.array_equal(o[1], ans)


def test_rect_flags_errors(cuda):
    from fdm_gb300 import FdmError
    from fdm_gb300 import _native as N
    with pytest.raises(FdmError) as e:
        LaplRectFFT2(0.1, 0.1, 1.0, 1.0, 16, 16, periodic_x=True)  # x alone: not instantiated
    assert e.value.status == N.ENOTSUP
    with pytest.raises(FdmError) as e:
        LaplRect(0.1, 0.1, 1.0, 1.0, 15, 24, periodic_y=True)  # periodic ny not a power of two
    assert e.value.status == N.ESIZE


def test_rect_formulations_agree_511(cuda):
    # ut/ut_lapl_rect.cpp:384-456
    n = 511
    rhs = np.random.default_rng(2).uniform(-1, 1, (n, n))
    h = 1.0 / (n + 1)
    a = np.zeros_like(rhs)
    b = np.zeros_like(rhs)
    LaplRect(h, h, 1.0, 1.0, n, n).solve(a, rhs)
    LaplRectFFT2(h, h, 1.0, 1.0, n, n).solve(b, rhs)
    assert np.abs(a - b).max() <= 1e-14 * max(1.0, np.abs(a).max())


def _dst_matrix(N):
    j = np.arange(1, N)
    return np.sin(np.pi * np.outer(j, j) / N)


@pytest.mark.parametrize("N", [32, 64, 128])
def test_sine_tc_lines_vs_fp64(cuda, N):
    """Tensor-core DST (split TF32, FP32 accumulation) of contiguous lines,
    including a ragged last tile, against the FP64 matrix product."""
    import torch
    from fdm_gb300 import sine_transform_tc_device
    rng = np.random.default_rng(N + 1)
    nl = 1000  # 7 full tiles of 128 lines and a ragged one
    x = rng.uniform(-1, 1, (nl, N - 1)).astype(np.float32)
    ref = 0.37 * x.astype(np.float64) @ _dst_matrix(N)
    tx = torch.tensor(x, device=cuda)
    ty = torch.full_like(tx, np.nan)
    sine_transform_tc_device(ty, tx, N, nl, 0.37)
    y = ty.cpu().numpy().astype(np.float64)
    assert np.isfinite(y).all()
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) <= 2e-6
    assert np.abs(y - ref).max() <= 5e-6 * np.abs(ref).max()
    # in place, as the solver uses it
    sine_transform_tc_device(tx, tx, N, nl, 0.37)
    assert torch.equal(tx, torch.tensor(y.astype(np.float32), device=cuda))


@pytest.mark.parametrize("N,nx", [(32, 37), (64, 63), (128, 129)])
def test_sine_tc_columns_vs_fp64(cuda, N, nx):
    """Along y: planes of (N-1) x nx, transformed along the stride-nx rows."""
    import torch
    from fdm_gb300 import sine_transform_tc_device
    rng = np.random.default_rng(N * nx)
    planes = 9
    x = rng.uniform(-1, 1, (planes, N - 1, nx)).astype(np.float32)
    ref = np.einsum("jk,pjx->pkx", _dst_matrix(N), x.astype(np.float64)) * 1.5
    tx = torch.tensor(x, device=cuda)
    ty = torch.empty_like(tx)
    sine_transform_tc_device(ty, tx, N, planes, 1.5, axis=1, nx=nx)
    y = ty.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) <= 2e-6


def test_cylindrical_vs_reference(cuda, golden):
    """LaplCyl3FFT2 (Dirichlet and periodic z) against the reference's
    outputs, FP64 and FP32; batched volumes equal single solves."""
    import torch
    from fdm_gb300 import LaplCyl3FFT2
    g = golden("lapl_cyl")
    for name, pz in (("d16x15x20", False), ("p8x16x12", True), ("d32x31x7", False)):
        rhs, ref = g["rhs_" + name], g["ans_" + name]
        nphi, nz, nr = rhs.shape
        lc = LaplCyl3FFT2(*g["args_" + name], nr, nz, nphi, periodic_z=pz)
        ans = np.zeros_like(rhs)
        lc.solve(ans, rhs)
        assert rel_l2(ans, ref) <= 1e-12, name
        l32 = LaplCyl3FFT2(*g["args_" + name], nr, nz, nphi, dtype=np.float32, periodic_z=pz)
        a32 = np.zeros(rhs.shape, np.float32)
        l32.solve(a32, rhs.astype(np.float32))
        assert rel_l2(a32.astype(np.float64), ref) <= 2e-5, name
        two = torch.tensor(np.stack([rhs, -rhs]), device=cuda)
        out = torch.empty_like(two)
        lc.solve_device(out, two, nrhs=2)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        assert np.array_equal(o[0], ans) and np.array_equal(o[1], -ans), name


def test_bounded_wait_gives_up_and_context_survives(cuda):
    """The tensor-core kernels wait for their MMAs with a bounded try_wait
    loop that records a failure instead of hanging.  Made to run out on an
    mbarrier that nothing arrives at, it reports ETIMEOUT, and the context
    keeps working afterwards."""
    import torch
    from fdm_gb300 import FdmError, sine_transform_tc_device
    from fdm_gb300 import _native as N
    lib = N.load()
    assert lib.fdmgpu_check_bounded_wait(1000) == N.ETIMEOUT
    assert b"gave up" in lib.fdmgpu_last_error()
    x = torch.ones((128, 31), dtype=torch.float32, device=cuda)
    y = torch.empty_like(x)
    sine_transform_tc_device(y, x, 32, 128, 1.0)  # the context is intact
    assert torch.isfinite(y).all()
    with pytest.raises(FdmError):
        N.check(lib.fdmgpu_check_bounded_wait(0))


@pytest.mark.parametrize("N", [8, 64, 512])
def test_pfft_lines_vs_reference(cuda, golden, N):
    """FFT<T>::pFFT_1 / pFFT of contiguous lines on the device against the
    reference's own outputs (lapl_cube_periodic.npz pf_* vectors)."""
    import torch
    from fdm_gb300 import pfft_device
    g = golden("lapl_cube_periodic")
    s = g["pf_s_%d" % N]
    x = torch.tensor(np.stack([s, 3 * s]), device=cuda)
    y = torch.empty_like(x)
    pfft_device(y, x, N, 2, dx=0.7)
    z = torch.empty_like(x)
    pfft_device(z, x, N, 2, dx=0.3, inverse=True)
    torch.cuda.synchronize()
    yy, zz = y.cpu().numpy(), z.cpu().numpy()
    assert np.abs(yy[0] - g["pf1_%d" % N]).max() <= 1e-13 * N
    assert np.abs(yy[1] - 3 * yy[0]).max() <= 1e-13 * N
    assert np.abs(zz[0] - g["pf_%d" % N]).max() <= 1e-13 * N


def _dd_inputs():
    """FP64 values over the whole exponent range (zero, subnormal doubles,
    float-subnormal results and their ties, the top float binade, overflow,
    inf, NaN) and float pairs (hi, lo) built from them."""
    rng = np.random.default_rng(11)
    sp = [0.0, 5e-324, 1e-310, 2.0 ** -150, 2.0 ** -149, 3 * 2.0 ** -150, 5 * 2.0 ** -151, 2.0 ** -126,
          np.nextafter(2.0 ** -126, 0), 2.0 ** -127, 2.0 ** -74, np.nextafter(2.0 ** -74, 0), 2.0 ** 127,
          np.nextafter(2.0 ** 127, 0), 2.0 ** 128, 2.0 ** 128 - 2.0 ** 103, 2.0 ** 128 - 2.0 ** 104,
          np.nextafter(2.0 ** 128 - 2.0 ** 103, 0), 2.0 ** 191, 1.7 * 2.0 ** 190, 1.7976931348623157e308,
          np.inf, np.nan, 1.0, 3e-40, 1e-45, 7e-46]
    e = np.repeat(np.arange(-1080, 1031), 12)
    m = 1.0 + rng.random(e.size)
    m[::12] = 1.0
    m[1::12] = 1.0 + 2.0 ** -24  # ties of the float rounding
    m[2::12] = 1.0 + 3 * 2.0 ** -25
    with np.errstate(over="ignore"):
        x = np.r_[sp, np.ldexp(m, e)]
    x = np.r_[x, -x]
    with np.errstate(over="ignore", invalid="ignore"):
        hi = x.astype(np.float32)
        lo = np.where(np.isfinite(hi), (x - hi.astype(np.float64)), 0.0).astype(np.float32)
    s = np.array([0.0, -0.0, 1e-45, -1e-45, 3e-40, -3e-40, 1.1754942e-38, 2.5e-38, -1e-37, np.inf, -np.inf, np.nan,
                  1.0], np.float32)
    hi = np.r_[hi, np.repeat(s, s.size)]
    lo = np.r_[lo, np.tile(s, s.size)]
    x = np.r_[x, np.ones(hi.size - x.size)]
    return x, hi, lo


def test_dd_conversions_match_hardware(cuda):
    """The mixed path's FP64 <-> float conversions use integer operations
    only; outside the normal float range (zero, subnormal results, the top
    binade, overflow, inf, NaN) they equal the hardware's conversions bit for
    bit, inside it they differ only at exact ties; split pairs hold x to
    2^-48 relative; the FP64 value of a float pair equals the hardware sum for
    zero, subnormal, inf and NaN parts and is within one FP64 ulp of it (half
    an ulp of the exact sum) for normalised pairs and for a normal lo beside a
    subnormal hi."""
    import torch
    from fdm_gb300 import _native as N
    x, hi, lo = _dd_inputs()
    n = x.size
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    tx, th, tl = t(x), t(hi), t(lo)
    f32, f32hw, sh, sl = (torch.empty(n, dtype=torch.float32, device=cuda) for _ in range(4))
    w, whw = (torch.empty(n, dtype=torch.float64, device=cuda) for _ in range(2))
    N.check(N.load().fdmgpu_check_dd_conversions(n, tx.data_ptr(), th.data_ptr(), tl.data_ptr(), f32.data_ptr(),
                                                 f32hw.data_ptr(), sh.data_ptr(), sl.data_ptr(), w.data_ptr(),
                                                 whw.data_ptr(), None))
    torch.cuda.synchronize()
    f32, f32hw, sh, sl, w, whw = (a.cpu().numpy() for a in (f32, f32hw, sh, sl, w, whw))

    def same(a, b):
        return (np.isnan(a) & np.isnan(b)) | (a.view(np.int64 if a.dtype == np.float64 else np.int32)
                                              == b.view(np.int64 if b.dtype == np.float64 else np.int32))

    ax = np.abs(x)
    edge = ~((ax >= 2.0 ** -126) & (ax < 2.0 ** 127))
    assert same(f32, f32hw)[edge].all()
    diff = ~same(f32, f32hw) & ~edge
    # inside the normal range only exact ties differ (rounded away from zero)
    assert np.array_equal(np.abs(f32[diff].astype(np.float64) - x[diff]), np.abs(f32hw[diff].astype(np.float64) - x[diff]))
    assert diff.sum() < 0.02 * n

    fin = np.isfinite(x) & (ax < 2.0 ** 191)
    tiny = fin & (ax < 2.0 ** -126)
    assert same(sh, f32hw)[tiny].all() and (sl[tiny] == 0).all()
    mid = fin & ~tiny & np.isfinite(sh)
    err = np.abs(x[mid] - (sh[mid].astype(np.float64) + sl[mid].astype(np.float64)))
    assert (err <= np.ldexp(ax[mid], -48) + 2.0 ** -149).all()
    big = ~np.isnan(x) & ~mid & ~tiny
    assert np.isinf(sh[big]).all() and same(sh, f32hw)[big].all()
    assert np.isnan(sh[np.isnan(x)]).all() and np.isnan(sl[np.isnan(x)]).all()

    eh = (hi.view(np.uint32) >> 23) & 0xFF
    el = (lo.view(np.uint32) >> 23) & 0xFF
    swapped = (eh == 0) & (el != 0) & (el != 255)  # hi zero or subnormal, lo normal: not a normalised pair
    pedge = ((eh == 0) | (eh == 255) | (el == 255)) & ~swapped
    assert same(w, whw)[pedge].all()
    ok = (~pedge & (np.abs(lo.astype(np.float64)) <= np.ldexp(np.abs(hi.astype(np.float64)), -24))) | swapped
    assert swapped.sum() >= 8
    ulp = np.abs(np.nextafter(whw[ok], np.inf) - whw[ok])
    assert (np.abs(w[ok] - whw[ok]) <= ulp).all()
