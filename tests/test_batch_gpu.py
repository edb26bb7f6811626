"""GPU parity of the batched uneven-size path (fdmgpu_batch_*): every
right-hand side of a mixed-size batch against its own single LaplCube solve,
results unchanged by the company a right-hand side keeps, and the schedule
tuner."""
import numpy as np
import pytest

from fdm_gb300 import BatchSolver, FdmError, LaplCube, workloads

pytestmark = pytest.mark.gpu


def _volumes(shapes, seed):
    import torch
    out = []
    for i, (nx, ny, nz) in enumerate(shapes):
        g = torch.Generator(device="cuda").manual_seed(seed * 1000 + i)
        out.append(torch.randn((nz, ny, nx), dtype=torch.float64, device="cuda", generator=g))
    return out


def _rel(a, b):
    import torch
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def _single_plain(shape, h, l, rhs):
    import torch
    nx, ny, nz = shape
    lc = LaplCube(h[0], h[1], h[2], l[0], l[1], l[2], nx, ny, nz)
    ans = torch.empty_like(rhs)
    lc.solve_device(ans, rhs)
    return ans


@pytest.mark.parametrize("tol", [1e-8, 1e-10])
def test_batch_uneven_vs_single_fp64(cuda, tol):
    """40 right-hand sides, each axis drawn from {31, 63, 127} (the uneven
    batch's own size set), mixed precision against the FP64 single solve."""
    import torch
    shapes = workloads.random_sizes(40, seed=3)
    hs = [tuple(1.0 / (n + 1) for n in s) for s in shapes]
    ls = [(1.0, 1.0, 1.0)] * len(shapes)
    rhs = _volumes(shapes, 1)
    ans = [torch.empty_like(r) for r in rhs]
    b = BatchSolver(shapes, hs, ls, precision="mixed", tol=tol)
    b.solve(ans, rhs)
    torch.cuda.synchronize()
    for i, s in enumerate(shapes):
        ref = _single_plain(s, hs[i], ls[i], rhs[i])
        assert _rel(ans[i], ref) <= tol, (i, s)


def test_batch_config3_inputs(cuda):
    """The uneven batch's own inputs (sizes per axis from {31, 63, 127},
    manufactured solutions with k in [1, (n+1)/4] per axis, tol 1e-8), 48 of
    them: every answer against its FP64 single solve and the manufactured u."""
    import torch
    shapes, rhs, exact = workloads.uneven_batch_torch(48, seed=2024)
    args = [workloads.solver_args(*s) for s in shapes]
    ans = [torch.empty_like(r) for r in rhs]
    b = BatchSolver(shapes, [a[0:3] for a in args], [a[3:6] for a in args], precision="mixed", tol=1e-8)
    b.tune(ans, rhs)
    b.solve(ans, rhs)
    torch.cuda.synchronize()
    for i, s in enumerate(shapes):
        ref = _single_plain(s, args[i][0:3], args[i][3:6], rhs[i])
        assert _rel(ans[i], ref) <= 1e-8, (i, s)
        assert _rel(ans[i], exact[i]) <= 1e-8, (i, s)
        assert _rel(ref, exact[i]) <= 1e-13, (i, s)


def test_batch_plain_equals_single(cuda):
    """Plain FP64 through pointer tables equals the contiguous FP64 solve."""
    import torch
    shapes = [(31, 15, 7), (63, 31, 31), (31, 15, 7), (15, 63, 127), (7, 7, 7)]
    hs = [(0.1, 0.07, 0.05)] * len(shapes)
    ls = [((s[0] + 1) * 0.1, (s[1] + 1) * 0.07, (s[2] + 1) * 0.05) for s in shapes]
    rhs = _volumes(shapes, 2)
    ans = [torch.empty_like(r) for r in rhs]
    b = BatchSolver(shapes, hs, ls, precision="plain")
    b.solve(ans, rhs)
    torch.cuda.synchronize()
    assert b.info()[0] == 4
    for i, s in enumerate(shapes):
        assert torch.equal(ans[i], _single_plain(s, hs[i], ls[i], rhs[i])), i


def test_batch_alone_equals_in_the_mix(cuda):
    """A right-hand side gets bit-identical answers alone and inside a
    batch of others with its schedule fixed (same group plan, same kernels)."""
    import torch
    shapes = workloads.random_sizes(24, seed=5) + [(63, 127, 31)]
    rhs = _volumes(shapes, 3)
    ans = [torch.empty_like(r) for r in rhs]
    BatchSolver(shapes, precision="mixed", tol=1e-10).solve(ans, rhs)
    alone = torch.empty_like(rhs[-1])
    BatchSolver([shapes[-1]], precision="mixed", tol=1e-10).solve([alone], [rhs[-1]])
    torch.cuda.synchronize()
    assert torch.equal(alone, ans[-1])


def test_batch_tune_then_replay_new_pointers(cuda):
    """tune picks a schedule per group; replays with other volumes give the
    answers of a fresh batch on those volumes within the tolerance, and
    the answers of the same volumes twice are identical."""
    import torch
    shapes = workloads.random_sizes(30, seed=7)
    r1, r2 = _volumes(shapes, 4), _volumes(shapes, 5)
    a1 = [torch.empty_like(r) for r in r1]
    a2 = [torch.empty_like(r) for r in r2]
    b = BatchSolver(shapes, precision="mixed", tol=1e-10)
    b.tune(a1, r1)
    sched = b.schedule()
    assert sum(g["members"] for g in sched) == 30
    assert all(g["tuned_ms"] > 0 and 1 <= g["chunk"] <= g["members"] for g in sched)
    b.solve(a1, r1)
    b.solve(a2, r2)
    torch.cuda.synchronize()
    first = [a.clone() for a in a2]
    b.solve(a2, r2)
    torch.cuda.synchronize()
    groups, launches = b.info()
    assert launches >= groups
    for i, s in enumerate(shapes):
        assert torch.equal(first[i], a2[i])
        h = tuple(1.0 / (n + 1) for n in s)
        assert _rel(a1[i], _single_plain(s, h, (1, 1, 1), r1[i])) <= 1e-10
        assert _rel(a2[i], _single_plain(s, h, (1, 1, 1), r2[i])) <= 1e-10


def test_batch_errors(cuda):
    import torch
    with pytest.raises(FdmError) as e:
        BatchSolver([(31, 31, 31), (32, 31, 31)])
    assert e.value.status == 2
    b = BatchSolver([(7, 7, 7)] * 2)
    x = torch.zeros(343, dtype=torch.float64, device="cuda")
    with pytest.raises(FdmError):
        b.solve([x], [x])
    with pytest.raises(FdmError):
        b.solve([x, torch.zeros(10, dtype=torch.float64, device="cuda")], [x, x])
