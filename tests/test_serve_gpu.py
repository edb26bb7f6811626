"""GPU tests of the serving loop (fdmgpu_server_*) through the C ABI: each
result is the same alone and in a mix of concurrent, batched requests;
per-request accuracy against the FP64 form; admission under a memory
budget; cancellation, timeouts and rejected buffers."""
import math

import numpy as np
import pytest

from fdm_gb300 import FdmError, LaplCube, NSCube, workloads
from fdm_gb300 import _native as N
from fdm_gb300.serve import Server

pytestmark = pytest.mark.gpu

SHAPES = [(31, 31, 31), (63, 31, 127), (31, 63, 63), (127, 127, 31), (63, 63, 63), (31, 31, 31), (63, 63, 63),
          (31, 31, 31)]
TOLS = [1e-6, 1e-10, 1e-10, 1e-6, 1e-10, 1e-10, 1e-6, 0.0]


def _pinned_rhs(shape, seed):
    import torch
    nx, ny, nz = shape
    g = torch.Generator().manual_seed(seed)
    return torch.randn((nz, ny, nx), dtype=torch.float64, generator=g).pin_memory()


def _pinned_like(t):
    import torch
    return torch.empty_like(t).pin_memory()


def _fp64(shape, rhs):
    """The plain FP64 LaplCube answer (h = 1/(n+1), l = 1)."""
    nx, ny, nz = shape
    lc = LaplCube(1 / (nx + 1), 1 / (ny + 1), 1 / (nz + 1), 1.0, 1.0, 1.0, nx, ny, nz)
    out = np.zeros(rhs.shape)
    lc.solve(out, rhs.numpy())
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_results_same_alone_and_in_the_mix(cuda):
    rhs = [_pinned_rhs(s, i) for i, s in enumerate(SHAPES)]
    # alone: one lane, one request per launch, each waited for in turn
    alone = []
    with Server(budget_bytes=8e9, lanes=1, max_batch=1) as srv:
        sid = srv.session_create(31, 31, Re=250.0, dt=0.01)
        for s, t, r in zip(SHAPES, TOLS, rhs):
            a = _pinned_like(r)
            rec = srv.wait(srv.submit_solve(a, r, s, tol=t))
            assert rec["state"] == "done" and rec["batch"] == 1
            alone.append(a)
        srv.wait(srv.submit_advance(sid, 12))
        u_alone, steps = srv.session_field(sid, "u")
        assert steps == 12
    # in the mix: eight lanes, batching on, two sessions advancing in
    # between, every request submitted before any finishes
    with Server(budget_bytes=8e9, lanes=8, max_batch=8) as srv:
        sids = [srv.session_create(31, 31, Re=250.0, dt=0.01), srv.session_create(31, 31, Re=100.0, dt=0.01)]
        mix = [_pinned_like(r) for r in rhs]
        ids = []
        for k, (s, t, r, a) in enumerate(zip(SHAPES, TOLS, rhs, mix)):
            ids.append(srv.submit_solve(a, r, s, tol=t))
            ids.append(srv.submit_advance(sids[k % 2], 3))
        done = 0
        while done < len(ids):
            rec = srv.next_done(10000.0)
            assert rec is not None and rec["state"] == "done", rec
            done += 1
        u_mix, steps = srv.session_field(sids[0], "u")
        assert steps == 12
        st = srv.stats()
        assert st["completed"] == len(ids) and st["failed"] == 0
    import torch
    for i in range(len(SHAPES)):
        assert torch.equal(alone[i], mix[i]), (i, SHAPES[i])
    assert np.array_equal(u_alone, u_mix)
    # and the session matches a standalone NSCube advanced as far
    ns = NSCube(nx=31, nz=31, Re=250.0, dt=0.01, u0=1.0, x1=-math.pi, y1=-math.pi, z1=-math.pi, x2=math.pi,
                y2=math.pi, z2=math.pi)
    ns.step(12)
    assert np.array_equal(ns.get("u").data.ravel(), u_mix.ravel())
    ns.close()


def test_advances_of_one_geometry_share_launches(cuda):
    """Waiting advances of sessions of one cavity geometry run as one launch
    per step over all of them; each session still matches a standalone
    NSCube advanced as far, whatever its Re and step count."""
    box = (-math.pi, -math.pi, -math.pi, math.pi, math.pi, math.pi)
    cases = [(250.0, 5), (100.0, 9), (400.0, 0), (250.0, 2)]
    with Server(budget_bytes=8e9, lanes=1, max_batch=8) as srv:
        sids = [srv.session_create(31, 31, Re=re, dt=0.01) for re, _ in cases]
        other = srv.session_create(15, 15)  # another geometry: launches of its own
        busy = srv.submit_advance(srv.session_create(63, 63), 200)  # holds the one lane
        ids = [srv.submit_advance(s, k) for s, (_, k) in zip(sids, cases)]
        alone = srv.submit_advance(other, 3)
        assert srv.wait(busy)["state"] == "done"
        recs = [srv.wait(i) for i in ids]
        assert all(r["state"] == "done" and r["batch"] == len(cases) for r in recs), recs
        rec = srv.wait(alone)
        assert rec["state"] == "done" and rec["batch"] == 1
        # steps of their own (the first captures the cavity's step), then
        # shared steps again, continue from the shared ones
        for s in sids:
            assert srv.wait(srv.submit_advance(s, 2))["batch"] == 1
        busy = srv.submit_advance(srv.session_create(63, 63), 200)
        more = [srv.submit_advance(s, 1) for s in sids]
        assert srv.wait(busy)["state"] == "done"
        assert all(srv.wait(i)["batch"] == len(cases) for i in more)
        fields = [srv.session_field(s, "u") for s in sids]
    for (re, k), (u, steps) in zip(cases, fields):
        assert steps == k + 3
        ns = NSCube(nx=31, nz=31, Re=re, dt=0.01, u0=1.0, x1=box[0], y1=box[1], z1=box[2], x2=box[3], y2=box[4],
                    z2=box[5])
        ns.step(k + 3)
        assert np.array_equal(ns.get("u").data.ravel(), u.ravel()), (re, k)
        ns.close()


def _wait_running(srv, rid):
    import time
    for _ in range(20000):
        if srv.poll(rid)["state"] == "running":
            return
        time.sleep(0.0005)
    raise AssertionError("request %d never started" % rid)


def test_load_shedding(cuda):
    """Requests that wait past the queue deadline finish as EBUSY without
    running; a full queue refuses submits with EBUSY; with the limits off
    everything runs again."""
    shape = (63, 63, 63)
    r = _pinned_rhs(shape, 3)
    outs = [_pinned_like(r) for _ in range(3)]
    with Server(budget_bytes=8e9, lanes=1, max_batch=1) as srv:
        sid = srv.session_create(63, 63)
        srv.wait(srv.submit_advance(sid, 2))
        srv.set_admission(max_queued=0, max_wait_ms=5.0)
        busy = srv.submit_advance(sid, 300)  # holds the one lane for ~40 ms
        late = [srv.submit_solve(a, r, shape, tol=1e-10) for a in outs]
        assert srv.wait(busy)["state"] == "done"
        for i in late:
            rec = srv.wait(i)
            assert rec["state"] == "failed" and rec["status"] == N.EBUSY, rec
            assert rec["latency_ms"] >= 5.0
        st = srv.stats()
        assert st["shed"] == 3 and st["failed"] == 0 and st["completed"] == 2
        # a full queue refuses at submit and queues nothing
        srv.set_admission(max_queued=2, max_wait_ms=0.0)
        busy = srv.submit_advance(sid, 300)
        _wait_running(srv, busy)
        queued = [srv.submit_solve(a, r, shape, tol=1e-10) for a in outs[:2]]
        with pytest.raises(FdmError) as e:
            srv.submit_solve(outs[2], r, shape, tol=1e-10)
        assert e.value.status == N.EBUSY
        for i in [busy] + queued:
            assert srv.wait(i)["state"] == "done"
        assert srv.stats()["shed"] == 4
        srv.set_admission(0, 0.0)
        ids = [srv.submit_solve(a, r, shape, tol=1e-10) for a in outs]
        assert all(srv.wait(i)["state"] == "done" for i in ids)
        _, steps = srv.session_field(sid, "u")
        assert steps == 602
    ref = _fp64(shape, r)
    assert _rel(outs[2].numpy(), ref) <= 1e-10


def test_submits_from_several_threads(cuda):
    """Four client threads submit solves and advances at once, with the
    queue deadline and a queue bound set high enough to shed nothing: every
    request completes and every answer is the same as alone."""
    import threading
    import torch
    shapes = [(31, 31, 31), (63, 31, 31), (31, 63, 63)]
    rhs = {s: _pinned_rhs(s, 70 + k) for k, s in enumerate(shapes)}
    alone = {}
    with Server(budget_bytes=8e9, lanes=1, max_batch=1) as srv:
        for s in shapes:
            a = _pinned_like(rhs[s])
            srv.wait(srv.submit_solve(a, rhs[s], s, tol=1e-10))
            alone[s] = a
    errors = []
    with Server(budget_bytes=8e9, lanes=8, max_batch=4) as srv:
        srv.set_admission(max_queued=10000, max_wait_ms=60000.0)
        sids = [srv.session_create(31, 31, Re=250.0, dt=0.01) for _ in range(4)]

        def client(k):
            try:
                mine = []
                for j in range(30):
                    s = shapes[(k + j) % len(shapes)]
                    a = _pinned_like(rhs[s])
                    mine.append((srv.submit_solve(a, rhs[s], s, tol=1e-10), s, a))
                    if j % 5 == 0:
                        mine.append((srv.submit_advance(sids[k], 2), None, None))
                for rid, s, a in mine:
                    rec = srv.wait(rid)
                    if rec["state"] != "done":
                        errors.append(rec)
                    elif s is not None and not torch.equal(a, alone[s]):
                        errors.append(("differs", s))
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append(repr(e))

        threads = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors[:3]
        st = srv.stats()
        assert st["completed"] == 4 * (30 + 6) and st["shed"] == 0 and st["failed"] == 0
        for sid in sids:
            assert srv.session_field(sid, "u")[1] == 12


def test_waiting_solves_share_a_launch(cuda):
    """Solves of one geometry that wait behind a busy lane go out as one
    launch; their answers equal the ones they get alone."""
    shape = (63, 63, 63)
    rhs = [_pinned_rhs(shape, 100 + i) for i in range(6)]
    outs = [_pinned_like(r) for r in rhs]
    with Server(budget_bytes=8e9, lanes=1, max_batch=8) as srv:
        sid = srv.session_create(63, 63)
        busy = srv.submit_advance(sid, 50)
        ids = [srv.submit_solve(a, r, shape, tol=1e-10) for a, r in zip(outs, rhs)]
        srv.wait(busy)
        recs = [srv.wait(i) for i in ids]
        assert max(r["batch"] for r in recs) >= 2
        st = srv.stats()
        assert st["batched_requests"] > st["batches"]
    with Server(budget_bytes=8e9, lanes=1, max_batch=1) as srv:
        for a, r in zip(outs, rhs):
            one = _pinned_like(r)
            srv.wait(srv.submit_solve(one, r, shape, tol=1e-10))
            import torch
            assert torch.equal(one, a)


def test_per_request_error_vs_fp64(cuda):
    with Server(budget_bytes=8e9, lanes=4, max_batch=4) as srv:
        cases = []
        for i, (s, t) in enumerate(zip(SHAPES, TOLS)):
            r = _pinned_rhs(s, 50 + i)
            a = _pinned_like(r)
            cases.append((s, t, r, a, srv.submit_solve(a, r, s, tol=t)))
        for s, t, r, a, rid in cases:
            rec = srv.wait(rid)
            assert rec["state"] == "done"
            err = _rel(a.numpy(), _fp64(s, r))
            assert err <= max(t, 1e-13), (s, t, err)
            # the server's per-request estimate bounds the error once a sweep ran
            if t < 1e-5:
                assert err <= rec["err_est"], (s, t, err, rec["err_est"])


def test_admission_under_budget(cuda):
    """A budget that holds a few 63^3 solves at a time: everything still
    completes and the accounted peak stays under the budget."""
    shape = (63, 63, 63)
    budget = 100e6
    rhs = [_pinned_rhs(shape, 200 + i) for i in range(12)]
    outs = [_pinned_like(r) for r in rhs]
    with Server(budget_bytes=budget, lanes=8, max_batch=8) as srv:
        ids = [srv.submit_solve(a, r, shape, tol=1e-10) for a, r in zip(outs, rhs)]
        for i in ids:
            assert srv.wait(i)["state"] == "done"
        st = srv.stats()
        assert 0 < st["peak_bytes"] <= budget
        assert st["plan_bytes"] > 0
    ref = _fp64(shape, rhs[0])
    assert _rel(outs[0].numpy(), ref) <= 1e-10


def test_rejections_cancel_and_timeout(cuda):
    import torch
    shape = (63, 63, 63)
    r = _pinned_rhs(shape, 1)
    a = _pinned_like(r)
    with Server(budget_bytes=10e6, lanes=1, max_batch=1) as srv:
        with pytest.raises(FdmError) as e:
            srv.submit_solve(a, r, shape)
        assert e.value.status == N.EBUDGET
    with Server(budget_bytes=8e9, lanes=1, max_batch=1) as srv:
        with pytest.raises(FdmError) as e:  # pageable buffers are refused
            srv.submit_solve(np.zeros(63 ** 3), r.numpy().ravel().copy(), shape)
        assert e.value.status == N.EINVAL
        odd = torch.zeros(64 * 63 * 63, dtype=torch.float64).pin_memory()
        with pytest.raises(FdmError) as e:  # n+1 = 65 is not a power of two
            srv.submit_solve(odd, odd, (64, 63, 63))
        assert e.value.status == N.ESIZE
        sid = srv.session_create(63, 63)
        busy = srv.submit_advance(sid, 50)
        queued = srv.submit_solve(a, r, shape)
        srv.cancel(queued)
        assert srv.poll(queued)["state"] == "cancelled"
        with pytest.raises(FdmError) as e:
            srv.wait(busy, timeout_ms=0.01)
        assert e.value.status == N.ETIMEOUT
        assert srv.wait(busy)["state"] == "done"
        with pytest.raises(FdmError):
            srv.submit_advance(sid + 5, 1)
        srv.session_close(sid)
        with pytest.raises(FdmError):
            srv.submit_advance(sid, 1)
        st = srv.stats()
        assert st["cancelled"] == 1 and st["completed"] == 1
