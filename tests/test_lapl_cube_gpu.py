"""GPU parity of the LaplCube path (plain and mixed precision) through the
C ABI of libfdmgpu.so, against the reference's golden outputs, the CPU oracle
and size-independent properties."""
import numpy as np
import pytest

from tests.helpers import lap7, rel_l2
from fdm_gb300 import FdmError, LaplCube, workloads

pytestmark = pytest.mark.gpu

# FP64 plain form vs the reference's CPU LaplCube::solve: relative L2 <= 1e-12
TOL_PLAIN = 1e-12
# mixed form with refinement vs the FP64 GPU form: relative L2 <= 1e-10
TOL_MIXED = 1e-10


def solve_host(args, rhs, **kw):
    lc = LaplCube(*args, **kw)
    ans = np.zeros_like(rhs)
    lc.solve(ans, rhs)
    return ans, lc


def test_golden_small_cases(cuda, golden):
    g = golden("lapl_cube")
    a = workloads.solver_args(15, 15, 15)
    ans, _ = solve_host(a, g["m15_rhs"])
    assert rel_l2(ans, g["m15_ans"]) <= TOL_PLAIN
    ans, _ = solve_host(tuple(g["aniso_args"]) + (15, 15, 7), g["aniso_rhs"])
    assert rel_l2(ans, g["aniso_ans"]) <= TOL_PLAIN
    ans, _ = solve_host(tuple(g["lz_args"]) + (31, 7, 15), g["lz_rhs"])
    assert rel_l2(ans, g["lz_ans"]) <= TOL_PLAIN


def test_config0_against_reference_checksums(cuda, golden):
    g = golden("lapl_cube")
    f, u = workloads.manufactured(31, 31, 31, seed=0, kmax=12)
    ans, _ = solve_host(workloads.solver_args(31, 31, 31), f)
    assert np.allclose(ans.ravel()[g["c0_ans_idx"]], g["c0_ans_vals"], rtol=0, atol=1e-12 * g["c0_ans_maxabs"])
    assert rel_l2(ans, u) <= 1e-13  # manufactured solution to round-off


def test_reference_unit_case(cuda, golden):
    from tests.golden.make_golden import ut_lapl_cube_rhs
    g = golden("lapl_cube")
    rhs, exact, args = ut_lapl_cube_rhs(31)
    ans, _ = solve_host(args + (31, 31, 31), rhs)
    err = np.abs(ans - exact).max() / np.abs(exact).max()
    assert err < 1e-4  # ut/ut_lapl_cube.cpp:124
    assert abs(err - g["ut31_err"]) <= 1e-10
    assert np.allclose(ans.ravel()[g["ut31_ans_idx"]], g["ut31_ans_vals"], rtol=0, atol=1e-12 * g["ut31_ans_maxabs"])


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 7, 1), (7, 15, 31), (63, 31, 15), (31, 127, 63), (63, 63, 63)])
def test_plain_f64_vs_oracle(cuda, port, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + ny * 3 + nz)
    rhs = rng.standard_normal((nz, ny, nx))
    h = (0.3, 0.11, 0.07)
    args = (h[0], h[1], h[2], (nx + 1) * h[0], (ny + 1) * h[1], (nz + 1) * h[2], nx, ny, nz)
    ans, _ = solve_host(args, rhs)
    ref = port.lapl_cube(rhs, *args[:6])
    assert rel_l2(ans, ref) <= TOL_PLAIN


def test_plain_f64_config2_size_vs_oracle(cuda, port):
    """The metric's own size, 255^3 interior, with its inputs (k in [1,60],
    N(0,1e-3) noise): the plain FP64 GPU solve against the oracle's
    LaplCube::solve, and the mixed form against both; without noise the
    manufactured u comes back to round-off (the discretisation error of
    these exact discrete modes is zero)."""
    n = 255
    args = workloads.solver_args(n, n, n)
    f, _ = workloads.manufactured(n, n, n, seed=0, kmax=60, noise=1e-3)
    ref = port.lapl_cube(f, *args[:6])
    ans, _ = solve_host(args, f)
    assert rel_l2(ans, ref) <= TOL_PLAIN
    mixed, m = solve_host(args, f, precision="mixed", tol=1e-10)
    assert m.last_info(1)[0] == 1
    assert rel_l2(mixed, ref) <= TOL_MIXED
    assert rel_l2(mixed, ans) <= TOL_MIXED
    f0, u0 = workloads.manufactured(n, n, n, seed=1, kmax=60)
    ans0, _ = solve_host(args, f0)
    assert rel_l2(ans0, u0) <= 1e-13
    assert rel_l2(ans0, port.lapl_cube(f0, *args[:6])) <= TOL_PLAIN


def test_plain_f32_vs_oracle(cuda, port):
    n = 31
    f, u = workloads.manufactured(n, n, n, seed=4, kmax=8)
    args = workloads.solver_args(n, n, n)
    lc = LaplCube(*args, dtype=np.float32)
    ans = np.zeros(f.shape, np.float32)
    lc.solve(ans, f.astype(np.float32))
    assert rel_l2(ans, port.lapl_cube(f, *args[:6])) <= 1e-5


@pytest.mark.parametrize("n", [127, 255])
def test_plain_large_residual_and_linearity(cuda, n):
    """Size-independent properties at full size: the 7-point residual of the
    answer and linearity in the right-hand side."""
    import torch
    f, u = workloads.manufactured_torch(n, n, n, seed=2, kmax=60 if n == 255 else 30, noise=1e-3)
    args = workloads.solver_args(n, n, n)
    lc = LaplCube(*args)
    ans = torch.empty_like(f)
    lc.solve_device(ans, f)
    f2 = torch.roll(f, 1, 0).contiguous()
    ans2 = torch.empty_like(f)
    lc.solve_device(ans2, f2)
    both = torch.empty_like(f)
    lc.solve_device(both, (2.0 * f - 3.0 * f2).contiguous())
    torch.cuda.synchronize()
    a, b, c = ans.cpu().numpy(), ans2.cpu().numpy(), both.cpu().numpy()
    h = args[0]
    fr = f.cpu().numpy()
    assert rel_l2(lap7(a, h, h, h), fr) <= 1e-12
    assert rel_l2(c, 2 * a - 3 * b) <= 1e-13


def test_batched_equals_single(cuda):
    import torch
    n = 63
    fs = [workloads.manufactured_torch(n, n, n, seed=s, kmax=16)[0] for s in range(3)]
    args = workloads.solver_args(n, n, n)
    lc = LaplCube(*args)
    batch = torch.stack(fs).contiguous()
    out = torch.empty_like(batch)
    lc.solve_device(out, batch, nrhs=3)
    for i, f in enumerate(fs):
        one = torch.empty_like(f)
        lc.solve_device(one, f)
        torch.cuda.synchronize()
        assert torch.equal(one, out[i])


@pytest.mark.parametrize("n,kmax", [(31, 8), (63, 16), (127, 32)])
def test_mixed_vs_plain(cuda, n, kmax):
    import torch
    f, u = workloads.manufactured_torch(n, n, n, seed=n, kmax=kmax, noise=1e-3)
    args = workloads.solver_args(n, n, n)
    plain = LaplCube(*args)
    mixed = LaplCube(*args, precision="mixed", tol=1e-10)
    a = torch.empty_like(f)
    b = torch.empty_like(f)
    plain.solve_device(a, f)
    mixed.solve_device(b, f)
    sweeps, est = mixed.last_info(1)
    err = (torch.linalg.norm(b - a) / torch.linalg.norm(a)).item()
    assert sweeps >= 1
    assert err <= TOL_MIXED
    assert 0 <= est[0] < 1e-4


def test_mixed_config2_full_size(cuda):
    """255^3, k in [1,60], N(0,1e-3) noise: two RHS batched."""
    import torch
    n = 255
    fs = [workloads.manufactured_torch(n, n, n, seed=s, kmax=60, noise=1e-3)[0] for s in (0, 1)]
    args = workloads.solver_args(n, n, n)
    batch = torch.stack(fs).contiguous()
    plain = LaplCube(*args)
    mixed = LaplCube(*args, precision="mixed", tol=1e-10)
    a = torch.empty_like(batch)
    b = torch.empty_like(batch)
    plain.solve_device(a, batch, nrhs=2)
    mixed.solve_device(b, batch, nrhs=2)
    torch.cuda.synchronize()
    for i in range(2):
        err = (torch.linalg.norm(b[i] - a[i]) / torch.linalg.norm(a[i])).item()
        assert err <= TOL_MIXED, (i, err)


def test_mixed_tolerance_levels(cuda):
    import torch
    n = 63
    f, _ = workloads.manufactured_torch(n, n, n, seed=9, kmax=16, noise=1e-3)
    args = workloads.solver_args(n, n, n)
    plain = LaplCube(*args)
    a = torch.empty_like(f)
    plain.solve_device(a, f)
    for tol, want_sweeps in ((1e-4, 0), (1e-6, 1), (1e-10, 1), (1e-13, 2)):
        m = LaplCube(*args, precision="mixed", tol=tol)
        b = torch.empty_like(f)
        m.solve_device(b, f)
        s, _ = m.last_info(1)
        assert s == want_sweeps
        err = (torch.linalg.norm(b - a) / torch.linalg.norm(a)).item()
        assert err <= max(tol, 1e-13), (tol, err)


@pytest.mark.parametrize("shape", [(63, 63, 63), (127, 127, 127), (255, 255, 255), (127, 63, 255), (255, 31, 127),
                                   (63, 127, 63), (255, 255, 31), (127, 15, 31)])
def test_mixed_plane_pipeline(cuda, shape):
    """The three-pass pipeline (DST-y, the fused x-z plane pass on clusters
    of 1 to 8 CTAs, inverse DST-y) against the FP64 form and the five-pass
    pipeline, for every refinement schedule (no sweep, one, two), two
    right-hand sides at once (white noise plus smooth modes)."""
    import torch
    nx, ny, nz = shape
    f = torch.stack([workloads.manufactured_torch(nx, ny, nz, seed=31 + s, kmax=min(shape) // 4 + 1,
                                                  noise=1e-3)[0] for s in (0, 1)]).contiguous()
    g = torch.Generator(device="cuda").manual_seed(5)
    f[1] += torch.randn(f[1].shape, dtype=torch.float64, device="cuda", generator=g)
    args = workloads.solver_args(nx, ny, nz)
    a = torch.empty_like(f)
    LaplCube(*args).solve_device(a, f, nrhs=2)
    for tol in (1e-4, 1e-10, 1e-13):
        planes = LaplCube(*args, precision="mixed", tol=tol)
        assert planes.pipeline_in_use() == "planes"
        five = LaplCube(*args, precision="mixed", tol=tol)
        five.set_pipeline(False)
        assert five.pipeline_in_use() == "five_pass"
        b = torch.empty_like(f)
        c = torch.empty_like(f)
        planes.solve_device(b, f, nrhs=2)
        five.solve_device(c, f, nrhs=2)
        torch.cuda.synchronize()
        for i in range(2):
            eb = (torch.linalg.norm(b[i] - a[i]) / torch.linalg.norm(a[i])).item()
            ec = (torch.linalg.norm(c[i] - a[i]) / torch.linalg.norm(a[i])).item()
            assert eb <= max(tol, 1e-12), (shape, tol, i, eb, ec)
            assert ec <= max(tol, 1e-12), (shape, tol, i, eb, ec)


def test_plane_pipeline_applicability(cuda):
    """Sizes the plane pass does not cover run the five-pass pipeline."""
    for shape in ((31, 31, 31), (63, 63, 31), (127, 127, 7), (255, 255, 511)):
        m = LaplCube(*workloads.solver_args(*shape), precision="mixed", tol=1e-10)
        assert m.pipeline_in_use() == "five_pass", shape
    m = LaplCube(*workloads.solver_args(127, 127, 127), precision="mixed", tol=1e-10)
    m.set_schedule(ztable=False)
    assert m.pipeline_in_use() == "five_pass"
    assert LaplCube(*workloads.solver_args(127, 127, 127)).pipeline_in_use() == "five_pass"  # plain FP64


def test_default_tensor_core_axes(cuda):
    """A mixed plan puts 32-point x axes on the tensor cores, and 32-point y
    axes where it runs the five passes; its answers stay within the mixed
    tolerance of the FP64 form, and set_schedule overrides the default."""
    import torch
    cases = {(31, 31, 31): 3, (31, 63, 63): 1, (63, 31, 63): 0, (63, 31, 31): 2, (127, 127, 127): 0,
             (63, 63, 63): 0}
    for shape, mask in cases.items():
        args = workloads.solver_args(*shape)
        m = LaplCube(*args, precision="mixed", tol=1e-10)
        assert m.schedule()["dst_tc"] == mask, shape
        f = workloads.manufactured_torch(*shape, seed=5, kmax=min(shape) // 4, noise=1e-3)[0]
        f = torch.stack([f, torch.flip(f, dims=[0])]).contiguous()
        a, u = torch.empty_like(f), torch.empty_like(f)
        m.solve_device(a, f, nrhs=2)
        LaplCube(*args).solve_device(u, f, nrhs=2)
        s, est = m.last_info(2)
        for i in range(2):
            err = (torch.linalg.norm(a[i] - u[i]) / torch.linalg.norm(u[i])).item()
            assert err <= TOL_MIXED and err <= est[i], (shape, i, err, est[i])
    assert LaplCube(*workloads.solver_args(31, 31, 31)).schedule()["dst_tc"] == 0  # plain FP64
    m = LaplCube(*workloads.solver_args(31, 31, 31), precision="mixed", tol=1e-10)
    m.set_schedule(ztable=True, dst_tc=0)
    assert m.schedule()["dst_tc"] == 0


@pytest.mark.parametrize("shape,nrhs,tol", [((31, 31, 31), 8, 1e-10), ((63, 31, 127), 2, 1e-10),
                                            ((63, 63, 63), 4, 1e-12), ((31, 63, 31), 4, 1e-4)])
def test_tune_keeps_an_accurate_schedule(cuda, shape, nrhs, tol):
    """tune() times the mixed schedules on the caller's data and keeps one
    whose answers meet the tolerance against the FP64 form."""
    import torch
    args = workloads.solver_args(*shape)
    f = torch.stack([workloads.manufactured_torch(*shape, seed=s, kmax=min(shape) // 4, noise=1e-3)[0]
                     for s in range(nrhs)]).contiguous()
    u, a = torch.empty_like(f), torch.empty_like(f)
    LaplCube(*args).solve_device(u, f, nrhs=nrhs)
    m = LaplCube(*args, precision="mixed", tol=tol)
    ms = m.tune(a, f, nrhs=nrhs)
    assert ms > 0.0
    sch = m.schedule()
    assert sch["dst_tc"] in (0, 1, 2, 3)
    a.fill_(float("nan"))
    m.solve_device(a, f, nrhs=nrhs)
    for i in range(nrhs):
        err = (torch.linalg.norm(a[i] - u[i]) / torch.linalg.norm(u[i])).item()
        assert err <= max(tol, 1e-12), (shape, sch, i, err)
    # a plain plan is left as it is
    p = LaplCube(*args)
    assert p.tune(a, f, nrhs=nrhs) == 0.0


def _white_or_smooth(shape, white, seed):
    import torch
    nx, ny, nz = shape
    if white:
        g = torch.Generator(device="cuda").manual_seed(seed)
        return torch.randn((nz, ny, nx), dtype=torch.float64, device="cuda", generator=g)
    return workloads.manufactured_torch(nx, ny, nz, seed=seed, kmax=min(shape) // 4, noise=1e-3)[0]


@pytest.mark.parametrize("shape,white", [((255, 255, 255), True), ((255, 255, 31), True), ((127, 63, 255), False),
                                         ((63, 31, 63), True), ((31, 31, 31), False), ((31, 31, 31), True),
                                         ((31, 255, 31), True), ((255, 31, 31), False), ((63, 31, 31), True)])
def test_error_estimate_bounds_error(cuda, shape, white):
    """last_info's per-RHS estimate of the remaining error is at least the
    error against the FP64 form, after one sweep and after two."""
    import torch
    f = _white_or_smooth(shape, white, 3)
    args = workloads.solver_args(*shape)
    u = torch.empty_like(f)
    LaplCube(*args).solve_device(u, f)
    for tol, sweeps in ((1e-10, 1), (1e-12, 2)):
        m = LaplCube(*args, precision="mixed", tol=tol)
        a = torch.empty_like(f)
        m.solve_device(a, f)
        s, est = m.last_info(1)
        err = (torch.linalg.norm(a - u) / torch.linalg.norm(u)).item()
        assert s == sweeps
        assert err <= est[0] <= 1e-8, (shape, tol, err, est)


def test_adaptive_refinement_adds_a_sweep(cuda):
    """A case the tolerance alone under-serves: 255 x 255 x 31 white noise at
    tol 2e-11 gets one sweep from the schedule and misses the tolerance
    (error ~5e-11); the closed loop sees the estimate above tol, runs a
    second sweep and meets it."""
    import torch
    shape, tol = (255, 255, 31), 2e-11
    f = _white_or_smooth(shape, True, 3)
    args = workloads.solver_args(*shape)
    u = torch.empty_like(f)
    LaplCube(*args).solve_device(u, f)
    fixed = LaplCube(*args, precision="mixed", tol=tol)
    a = torch.empty_like(f)
    fixed.solve_device(a, f)
    s, est = fixed.last_info(1)
    err = (torch.linalg.norm(a - u) / torch.linalg.norm(u)).item()
    assert s == 1 and est[0] > tol and err <= est[0]
    closed = LaplCube(*args, precision="mixed", tol=tol, adaptive=True)
    b = torch.empty_like(f)
    closed.solve_device(b, f)
    s2, est2 = closed.last_info(1)
    err2 = (torch.linalg.norm(b - u) / torch.linalg.norm(u)).item()
    assert s2 == 2
    assert err2 <= est2[0] <= tol, (err2, est2)
    # the host-array call runs the same loop
    h = np.zeros(f.shape)
    closed.solve(h, f.cpu().numpy())
    assert closed.last_info(1)[0] == 2
    assert rel_l2(h, u.cpu().numpy()) <= tol


@pytest.mark.parametrize("pinned", [True, False])
def test_host_batch_pipeline_equals_device(cuda, pinned):
    """The pipelined host-pointer batch (ring of 3 device slots) gives the
    same answers as device-pointer solves, for more volumes than slots."""
    import torch
    n = 63
    args = workloads.solver_args(n, n, n)
    fs = torch.stack([workloads.manufactured_torch(n, n, n, seed=s, kmax=16, noise=1e-3)[0] for s in range(5)])
    for prec in ("plain", "mixed"):
        lc = LaplCube(*args, precision=prec)
        dev_out = torch.empty_like(fs)
        for i in range(5):
            lc.solve_device(dev_out[i], fs[i].contiguous())
        hin = fs.cpu().pin_memory() if pinned else fs.cpu()
        hout = torch.empty_like(hin)
        if pinned:
            hout = hout.pin_memory()
        lc.solve_batch(hout, hin, 5)
        lc.solve_batch(hout, hin, 5)  # a second call reuses the ring
        torch.cuda.synchronize()
        assert torch.equal(hout, dev_out.cpu()), prec


def test_errors_like_reference(cuda):
    with pytest.raises(FdmError) as e:
        LaplCube(0.1, 0.1, 0.1, 3.3, 3.3, 3.3, 32, 31, 31)
    assert e.value.status == 2  # ESIZE: verify((1<<n) == N) in the reference
    with pytest.raises(FdmError):
        LaplCube(0.1, 0.1, 0.1, 3.2, 3.2, 3.2, 31, 31, 31, dtype=np.float32, precision="mixed")
    lc = LaplCube(*workloads.solver_args(7, 7, 7))
    with pytest.raises(FdmError):
        lc.solve(np.zeros(10), np.zeros(343))


@pytest.mark.parametrize("shape", [(31, 31, 31), (63, 63, 63), (31, 63, 127), (63, 127, 31), (127, 31, 63)])
def test_mixed_tensor_core_dst_vs_plain(cuda, shape):
    """The mixed form with its 32-/64-point DST passes on the tensor cores
    meets the same tolerance against the FP64 form, and the table / per-solve
    z variants agree with it."""
    import torch
    nx, ny, nz = shape
    f, _ = workloads.manufactured_torch(nx, ny, nz, seed=7, kmax=min(shape) // 4, noise=1e-3)
    args = workloads.solver_args(nx, ny, nz)
    plain = LaplCube(*args)
    a = torch.empty_like(f)
    plain.solve_device(a, f)
    for tol in (1e-10, 1e-8):
        m = LaplCube(*args, precision="mixed", tol=tol)
        m.set_schedule(ztable=True, dst_tc=True)
        b = torch.empty_like(f)
        m.solve_device(b, f)
        assert not m.device_failed()
        err = (torch.linalg.norm(b - a) / torch.linalg.norm(a)).item()
        assert err <= tol, (shape, tol, err)


def _periodic_manufactured(nx, ny, nz, h, seed):
    """u = sum of 6 exact discrete Fourier modes; f = periodic 7-point
    Laplacian of u.  The solve returns u minus its mean (zero here)."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    u = np.zeros((nz, ny, nx))
    for _ in range(6):
        kx, ky, kz = rng.integers(0, nx // 2), rng.integers(0, ny // 2), rng.integers(1, nz // 2)
        ph = rng.uniform(0, 2 * np.pi)
        u += rng.standard_normal() * np.cos(2 * np.pi * (kx * x / nx + ky * y / ny + kz * z / nz) + ph)

    def d2(a, ax, hh):
        return (np.roll(a, 1, ax) - 2 * a + np.roll(a, -1, ax)) / (hh * hh)
    f = d2(u, 2, h[0]) + d2(u, 1, h[1]) + d2(u, 0, h[2])
    return f, u


def test_periodic_vs_reference(cuda, golden):
    """All-periodic LaplCube (LaplCube<T,check,periodic^3>) against the
    reference's outputs, FP64 and FP32."""
    g = golden("lapl_cube_periodic")
    for name, (nz, ny, nx) in (("c16", (16, 16, 16)), ("a8x16x32", (8, 16, 32)), ("b32x16x16", (32, 16, 16))):
        args = tuple(g["args_" + name]) + (nx, ny, nz)
        rhs, ref = g["rhs_" + name], g["ans_" + name]
        lc = LaplCube(*args, periodic=True)
        ans = np.zeros_like(rhs)
        lc.solve(ans, rhs)
        assert rel_l2(ans, ref) <= 1e-12, name
        lc32 = LaplCube(*args, periodic=True, dtype=np.float32)
        a32 = np.zeros(rhs.shape, np.float32)
        lc32.solve(a32, rhs.astype(np.float32))
        assert rel_l2(a32.astype(np.float64), ref) <= 1e-5, name


@pytest.mark.parametrize("shape", [(64, 64, 64), (128, 32, 256), (512, 8, 16)])
def test_periodic_manufactured_and_batched(cuda, shape):
    """Exact discrete modes come back to round-off at larger sizes (x- and
    z-extents up to 512), and batched volumes equal single solves."""
    import torch
    nx, ny, nz = shape
    h = (2 * np.pi / nx, 0.7 * 2 * np.pi / ny, 1.3 * 2 * np.pi / nz)
    # distinct spacings only take effect when the point counts differ from ny
    args = (h[0], h[1], h[2], nx * h[0], ny * h[1], nz * h[2], nx, ny, nz)
    hx_eff = h[1] if nx == ny else h[0]
    hz_eff = h[1] if nz == ny else h[2]
    f, u = _periodic_manufactured(nx, ny, nz, (hx_eff, h[1], hz_eff), seed=nx + nz)
    lc = LaplCube(*args, periodic=True)
    tf = torch.tensor(np.stack([f, 2 * f]), device=cuda)
    out = torch.empty_like(tf)
    lc.solve_device(out, tf, nrhs=2)
    one = torch.empty_like(tf[0])
    lc.solve_device(one, tf[0].contiguous())
    torch.cuda.synchronize()
    a = out.cpu().numpy()
    assert rel_l2(a[0], u - u.mean()) <= 1e-12
    assert rel_l2(a[1], 2 * (u - u.mean())) <= 1e-12
    assert torch.equal(one, out[0])


def test_periodic_errors(cuda):
    with pytest.raises(FdmError) as e:
        LaplCube(0.1, 0.1, 0.1, 1.6, 1.6, 1.5, 16, 16, 15, periodic=True)
    assert e.value.status == 2
    with pytest.raises(FdmError) as e:
        LaplCube(0.1, 0.1, 0.1, 1.6, 1.6, 1.6, 16, 16, 16, periodic=True, precision="mixed")
    assert e.value.status == 6


def _lap7_torch(u, hx, hy, hz):
    """7-point Dirichlet Laplacian on the device (zero outside the box)."""
    import torch
    p = torch.nn.functional.pad(u, (1, 1, 1, 1, 1, 1))
    return ((p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2] - 2 * u) / hx ** 2
            + (p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1] - 2 * u) / hy ** 2
            + (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1] - 2 * u) / hz ** 2)


def test_maximum_size_1023_cubed(cuda):
    """The largest supported size, 1023^3 (8.6 GB per FP64 volume): the
    plain FP64 answer satisfies the 7-point equation to round-off and the
    mixed solve agrees with it at the requested tolerance (size-independent
    properties; the CPU oracle would take minutes here)."""
    import torch
    n = 1023
    f, _ = workloads.manufactured_torch(n, n, n, seed=9, kmax=100, noise=1e-3)
    args = workloads.solver_args(n, n, n)
    plain = LaplCube(*args)
    u = torch.empty_like(f)
    plain.solve_device(u, f)
    torch.cuda.synchronize()
    h = args[0]
    r = _lap7_torch(u, h, h, h)
    r -= f
    assert (torch.linalg.norm(r) / torch.linalg.norm(f)).item() <= 1e-12
    del r
    # beyond the mixed solve's conditioning limit: the mixed handle solves in
    # FP64 and says so
    mixed = LaplCube(*args, precision="mixed", tol=1e-10)
    um = torch.empty_like(f)
    mixed.solve_device(um, f)
    torch.cuda.synchronize()
    assert mixed.last_info(1)[0] == -1
    assert (torch.linalg.norm(um - u) / torch.linalg.norm(u)).item() <= 1e-10


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 3, 7), (3, 1, 1), (1023, 1, 3), (7, 1023, 1)])
def test_smallest_and_ragged_sizes_vs_oracle(cuda, port, shape):
    """Degenerate and ragged sizes (one interior point per axis, n = 1023 on
    one axis) against the oracle, plain FP64 and mixed.  The 1023-point axes
    are beyond the mixed solve's conditioning limit (FP32 inner solves stall
    near 1e-9 there), so the mixed handle solves them in FP64."""
    nz, ny, nx = shape
    rng = np.random.default_rng(sum(shape))
    f = rng.standard_normal(shape)
    args = workloads.solver_args(nx, ny, nz)
    ref = port.lapl_cube(f, *args[:6])
    ans = np.zeros_like(f)
    LaplCube(*args).solve(ans, f)
    # z is solved as tridiagonal systems where the reference transforms it: a
    # 1023-row z line (eigenvalue ratio ~4e5) carries round-off of a few 1e-12
    assert rel_l2(ans, ref) <= (5e-11 if nz == 1023 else 1e-12)
    ans2 = np.zeros_like(f)
    m = LaplCube(*args, precision="mixed", tol=1e-10)
    m.solve(ans2, f)
    assert rel_l2(ans2, ref) <= 1e-10
    assert m.last_info(1)[0] == (-1 if max(shape) == 1023 else 1)


def test_mixed_white_noise_at_the_conditioning_limit(cuda):
    """255^3 (kappa 2.7e4, just inside the limit) with white-noise data, the
    roughest right-hand side: one sweep still meets 1e-10."""
    import torch
    n = 255
    g = torch.Generator(device="cuda").manual_seed(11)
    f = torch.randn((n, n, n), dtype=torch.float64, device="cuda", generator=g)
    args = workloads.solver_args(n, n, n)
    u = torch.empty_like(f)
    LaplCube(*args).solve_device(u, f)
    m = LaplCube(*args, precision="mixed", tol=1e-10)
    um = torch.empty_like(f)
    m.solve_device(um, f)
    torch.cuda.synchronize()
    assert m.last_info(1)[0] == 1
    assert (torch.linalg.norm(um - u) / torch.linalg.norm(u)).item() <= 1e-10


@pytest.mark.parametrize("N", [8, 32])
def test_pfft3d_vs_reference(cuda, golden, N):
    """FFT<T>::pFFT_1_3d / pFFT_3d on the GPU against the reference's own
    answers (test_fft_3d_bench.cpp's cube), FP64 and FP32, host and device
    entry points; forward then inverse with scale 2/N returns the input."""
    import torch
    from fdm_gb300 import pfft3d_device, pfft_1_3d, pfft_3d
    g = golden("lapl_cube_periodic")
    s = np.ascontiguousarray(g["fft3d_in_%d" % N])
    for inv, key, fn in ((False, "fft3d_fwd_%d", pfft_1_3d), (True, "fft3d_inv_%d", pfft_3d)):
        ref = g[key % N]
        S = np.zeros_like(s)
        fn(S, s, 1.0)
        assert np.abs(S - ref).max() <= 1e-13 * N * np.abs(ref).max()
        S32 = np.zeros(s.shape, np.float32)
        fn(S32, s.astype(np.float32), 1.0)
        assert np.abs(S32.astype(np.float64) - ref).max() <= 2e-6 * N * np.abs(ref).max()
    # device entry point, two cubes back to back, and the round trip
    two = torch.tensor(np.stack([s, 2 * s]), device=cuda)
    fwd = torch.empty_like(two)
    pfft3d_device(fwd, two, N, 1.0, inverse=False, count=2)
    back = torch.empty_like(two)
    pfft3d_device(back, fwd, N, (2.0 / N), inverse=True, count=2)
    torch.cuda.synchronize()
    f = fwd.cpu().numpy()
    assert np.abs(f[0] - g["fft3d_fwd_%d" % N]).max() <= 1e-13 * N * np.abs(f[0]).max()
    assert np.abs(f[1] - 2 * f[0]).max() <= 1e-13 * np.abs(f[1]).max()
    assert np.abs(back.cpu().numpy() - np.stack([s, 2 * s])).max() <= 1e-12
