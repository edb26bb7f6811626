"""GPU test of fdmgpu_lapl_cube_solve_mixed_noalloc, the mixed-precision
solve for callers that must not allocate device memory while solving (their
device memory belongs to their own pool or another framework's allocator, or
they may not wait on an allocator after start-up).  It keeps its scratch in a
fixed array inside libfdmgpu.so instead of allocating.

Called through the C ABI; its result must match the existing mixed entry
point (fdmgpu_lapl_cube_solve_device on a FDMGPU_MIXED handle) within the
mixed-precision tolerance, on two calls in a row with different inputs (the
second call must not see the first call's leftovers).  This file is named to
be collected last."""
import pytest

from fdm_gb300 import _native as N
from fdm_gb300 import LaplCube, workloads

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-10  # relative L2, the tolerance of the mixed-precision tests


def _noalloc(lib, args, ans, rhs, nrhs, tol=1e-10, stream=None):
    dx, dy, dz, lx, ly, lz, nx, ny, nz = args
    return lib.fdmgpu_lapl_cube_solve_mixed_noalloc(dx, dy, dz, lx, ly, lz, nx, ny, nz, tol, ans.data_ptr(),
                                                    rhs.data_ptr(), nrhs, stream)


def _rel(a, b):
    import torch
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def test_noalloc_matches_mixed_entry_point_twice(cuda):
    import torch
    lib = N.load()
    nx, ny, nz = 63, 31, 63
    args = workloads.solver_args(nx, ny, nz)
    batch1 = torch.stack([workloads.manufactured_torch(nx, ny, nz, seed=s, kmax=(16, 8, 16), noise=1e-3)[0]
                          for s in (1, 2)]).contiguous()
    batch2 = torch.stack([workloads.manufactured_torch(nx, ny, nz, seed=s, kmax=(12, 6, 12), noise=1e-3)[0]
                          for s in (3, 4)]).contiguous()

    mixed = LaplCube(*args, precision="mixed", tol=1e-10)
    plain = LaplCube(*args)
    refs, exact = [], []
    for b in (batch1, batch2):
        r = torch.empty_like(b)
        mixed.solve_device(r, b, nrhs=2)
        p = torch.empty_like(b)
        plain.solve_device(p, b, nrhs=2)
        refs.append(r)
        exact.append(p)
    torch.cuda.synchronize()

    outs = []
    for b in (batch1, batch2):
        o = torch.full_like(b, float("nan"))
        assert _noalloc(lib, args, o, b, 2) == N.OK, lib.fdmgpu_last_error()
        outs.append(o)
    torch.cuda.synchronize()
    for o, r, p in zip(outs, refs, exact):
        for i in range(2):
            assert torch.isfinite(o[i]).all()
            assert _rel(o[i], r[i]) <= TOL_MIXED
            assert _rel(o[i], p[i]) <= TOL_MIXED


@pytest.mark.parametrize("tol", [1e-4, 1e-10, 1e-12])
def test_noalloc_tolerance_levels_match_handle(cuda, tol):
    """Every refinement schedule (no sweep for tol >= 1e-5, one down to
    1e-11, two below) against a mixed handle with the same tolerance and
    against the FP64 form, twice in a row (the second call starts from the
    first call's leftovers in the shared array)."""
    import torch
    lib = N.load()
    nx, ny, nz = 63, 31, 63
    args = workloads.solver_args(nx, ny, nz)
    mixed = LaplCube(*args, precision="mixed", tol=tol)
    plain = LaplCube(*args)
    for seed in (21, 22):
        f = torch.stack([workloads.manufactured_torch(nx, ny, nz, seed=seed + 10 * s, kmax=(16, 8, 16),
                                                      noise=1e-3)[0] for s in (0, 1)]).contiguous()
        r = torch.empty_like(f)
        mixed.solve_device(r, f, nrhs=2)
        p = torch.empty_like(f)
        plain.solve_device(p, f, nrhs=2)
        o = torch.full_like(f, float("nan"))
        assert _noalloc(lib, args, o, f, 2, tol=tol) == N.OK, lib.fdmgpu_last_error()
        torch.cuda.synchronize()
        for i in range(2):
            assert _rel(o[i], r[i]) <= tol
            assert _rel(o[i], p[i]) <= tol


def test_noalloc_anisotropic_grids(cuda, golden):
    """Anisotropic spacings, where FP32 factors computed per solve lose
    accuracy: the reference's own anisotropic case (golden fixture) and a
    63 x 31 x 63 grid with dz / dx = 10, against the reference's answer, the
    FP64 form and a mixed handle."""
    import torch
    lib = N.load()
    g = golden("lapl_cube")
    cases = [(tuple(g["aniso_args"]) + (15, 15, 7), torch.tensor(g["aniso_rhs"], device=cuda),
              torch.tensor(g["aniso_ans"], device=cuda))]
    nx, ny, nz = 63, 31, 63
    h = (0.05, 0.1, 0.5)
    a2 = (h[0], h[1], h[2], (nx + 1) * h[0], (ny + 1) * h[1], (nz + 1) * h[2], nx, ny, nz)
    gen = torch.Generator(device="cuda").manual_seed(77)
    f2 = torch.randn((nz, ny, nx), dtype=torch.float64, device=cuda, generator=gen)
    cases.append((a2, f2, None))
    for args, f, ref in cases:
        p = torch.empty_like(f)
        LaplCube(*args).solve_device(p, f)
        r = torch.empty_like(f)
        LaplCube(*args, precision="mixed", tol=1e-10).solve_device(r, f)
        for _ in range(2):
            o = torch.full_like(f, float("nan"))
            assert _noalloc(lib, args, o, f, 1) == N.OK, lib.fdmgpu_last_error()
            torch.cuda.synchronize()
            assert _rel(o, p) <= TOL_MIXED
            assert _rel(o, r) <= TOL_MIXED
            if ref is not None:
                assert _rel(o, ref) <= TOL_MIXED


def test_noalloc_allocates_nothing_and_rejects_oversize(cuda):
    import torch
    lib = N.load()
    n = 127
    args = workloads.solver_args(n, n, n)
    f = workloads.manufactured_torch(n, n, n, seed=5, kmax=32, noise=1e-3)[0].contiguous()
    out = torch.empty_like(f)
    assert _noalloc(lib, args, out, f, 1) == N.OK, lib.fdmgpu_last_error()  # first call: set-up on this device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    out2 = torch.empty_like(f)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert _noalloc(lib, args, out2, f, 1) == N.OK, lib.fdmgpu_last_error()
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    assert free2 == free1  # the call itself took no device memory
    assert free1 <= free0
    assert torch.equal(out, out2)
    plain = LaplCube(*args)
    p = torch.empty_like(f)
    plain.solve_device(p, f)
    torch.cuda.synchronize()
    assert _rel(out2, p) <= TOL_MIXED

    # 255^3 needs ~133 MB of scratch: refused with a clear status, nothing run
    n = 255
    big = workloads.solver_args(n, n, n)
    dummy = torch.empty(1, dtype=torch.float64, device=cuda)
    rc = _noalloc(lib, big, dummy, dummy, 1)
    assert rc == N.EBUDGET
    assert b"scratch" in lib.fdmgpu_last_error()
    # an axis of 1023 points is beyond the mixed solve's conditioning limit:
    # refused (the handle API solves it in FP64), nothing run
    ragged = workloads.solver_args(3, 1, 1023)
    rc = _noalloc(lib, ragged, dummy, dummy, 1)
    assert rc == N.ENOTSUP
    assert b"conditioning" in lib.fdmgpu_last_error()
