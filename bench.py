"""Benchmark of the GB300 Poisson hot path.

Workload (one "step"): 16 independent right-hand sides on a 256^3-interval
grid (255^3 interior unknowns, the reference LaplCube needs n+1 = 2^k), built
as manufactured solutions with k's in [1,60] plus N(0,1e-3) noise from the
seed, solved by the mixed-precision form (FP32 DST / tridiagonal inner
solves, FP64-accurate residual, iterative refinement to 1e-10 relative error
vs the FP64 GPU form).  Inputs (16 x 133 MB) are larger than L2, so no L2
flush is needed between steps.

value: solves/s with inputs resident in HBM (CUDA events around K steps on
the launching stream, barrier + synchronize both sides, max over ranks).
e2e:   solves/s through the host-pointer C-ABI batch entry point, with the
step's inputs copied from pinned host memory and the results copied back
inside the timed region.

--impl reference: the reference's CPU LaplCube::solve on the host cores (the
compiled reference where it was built on this machine, otherwise the C
restatement of it in oracle/), same metric, on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "256³ Poisson solves/s at ≤1e-10 rel err, mixed vs FP64 on 1 GB300; p50/p99 latency"
UNIT = "solves/s"
N_INT = 255
NRHS = 16
KMAX = 60
NOISE = 1e-3
TOL = 1e-10
# algorithmic bytes per interior point of one solve: read f, write u (FP64)
SOLVE_BYTES_PER_POINT = 16
# per-kernel algorithmic bytes per point: its input read + output write
KERNEL_BYTES = {
    "sine_x_round": 12, "sine_x_resid": 16, "sine_x_combine": 16, "sine_x_f32": 8, "sine_x_f32_out64": 12,
    "sine_y_f32": 8, "sine_x_f64": 16, "sine_y_f64": 16, "zsolve_f32": 8, "zsolve_f64": 16,
    "tridiag_f32": 8, "tridiag_f64": 16, "residual_ff": 16,
    "plane_xz_f32": 8, "sine_y_round": 12, "sine_y_combine": 16, "sine_y_f32_out64": 12,
}


def unixbench_score(samples):
    """The reference's own summary of repeated timings (src/unixbench_score.cpp:9-20):
    the geometric mean of the fastest two thirds of the samples."""
    data = sorted(samples)
    keep = (2 * len(data)) // 3
    if keep == 0:
        return None
    return math.exp(sum(math.log(d) for d in data[:keep]) / keep)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference_rate(sample_solves: int, n: int = N_INT, time_budget: float = 20.0):
    """Times the reference CPU solve (compiled reference if present, else the
    C restatement) on a bounded sample of the workload: up to
    `sample_solves` single-RHS 255^3 solves, stopping early once the budget
    is spent.  Returns (solves/s, kind, cores, sample text)."""
    from fdm_gb300 import workloads
    from oracle.oracle import port, reference
    import numpy as np
    ref = reference()
    kind = "reference" if ref is not None else "port"
    impl = ref if ref is not None else port()
    f, _ = workloads.manufactured(n, n, n, seed=0, kmax=KMAX, noise=NOISE)
    args = workloads.solver_args(n, n, n)[:6]
    impl.lapl_cube(f, *args)  # warm-up
    times = []
    t_start = time.perf_counter()
    for _ in range(sample_solves):
        t0 = time.perf_counter()
        impl.lapl_cube(f, *args)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > time_budget:
            break
    med = statistics.median(times)
    cores = port().threads()
    sample = "%d single-RHS %d^3 LaplCube<double> solves (median %.3f s each), OpenMP threads=%d" % (
        len(times), n, med, cores)
    cpu_reference_rate.last_times = times
    return 1.0 / med, kind, cores, sample


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    rate, kind, cores, sample = cpu_reference_rate(max(args.steps, 3), time_budget=60.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "poisson_dirichlet_255^3_x16rhs", "grid": [N_INT] * 3, "nrhs": NRHS,
                   "kmax": KMAX, "noise": NOISE, "tol": TOL},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                         "cpu_model": cpu_model(),
                         "unixbench_ms_per_solve": 1e3 * unixbench_score(cpu_reference_rate.last_times)},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure_uneven_batch(torch, fdm_gb300, workloads, stream, dev, count=512, tol=1e-8, reps=5):
    """Uneven batch: count right-hand sides, each axis drawn from {31, 63, 127},
    manufactured solutions with k along each axis uniform in [1, (n+1)/4]
    (seeded), mixed precision to tol, solved by one tuned graph launch per
    step; against the same right-hand sides solved one at a time by the FP64
    LaplCube form (one plan per size)."""
    with torch.cuda.stream(stream):
        shapes, rhs, exact = workloads.uneven_batch_torch(count, seed=2024, device=dev)
        ans = [torch.empty_like(r) for r in rhs]
        ref = [torch.empty_like(r) for r in rhs]
    stream.synchronize()
    points = sum(nx * ny * nz for nx, ny, nz in shapes)
    geo = [workloads.solver_args(*sh) for sh in shapes]
    b = fdm_gb300.BatchSolver(shapes, [g[0:3] for g in geo], [g[3:6] for g in geo], precision="mixed", tol=tol)
    t0 = time.perf_counter()
    b.tune(ans, rhs)
    tune_s = time.perf_counter() - t0
    for _ in range(2):
        b.solve(ans, rhs, stream=stream)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.solve(ans, rhs, stream=stream)
    e1.record(stream)
    stream.synchronize()
    batch_s = e0.elapsed_time(e1) * 1e-3 / reps
    # the per-size FP64 loop: one solve_device call per right-hand side
    plans = {}
    for nx, ny, nz in shapes:
        if (nx, ny, nz) not in plans:
            plans[(nx, ny, nz)] = fdm_gb300.LaplCube(*workloads.solver_args(nx, ny, nz))

    def loop():
        for i, s in enumerate(shapes):
            plans[s].solve_device(ref[i], rhs[i], stream=stream)
    loop()
    stream.synchronize()
    e0.record(stream)
    for _ in range(2):
        loop()
    e1.record(stream)
    stream.synchronize()
    loop_s = e0.elapsed_time(e1) * 1e-3 / 2
    errs = [(torch.linalg.norm(ans[i] - ref[i]) / torch.linalg.norm(ref[i])).item() for i in range(count)]
    errs_u = [(torch.linalg.norm(ans[i] - exact[i]) / torch.linalg.norm(exact[i])).item() for i in range(count)]
    groups, launches = b.info()
    sched = b.schedule()
    return {
        "workload": "%d RHS, each axis from {31,63,127}, tol %g" % (count, tol),
        "points": points, "groups": groups, "kernel_launches_per_graph": launches,
        "solves_per_s": count / batch_s, "ms_per_batch": batch_s * 1e3,
        "hbm_gbs_fp64_in_out": 16.0 * points / batch_s / 1e9,
        "fp64_per_size_loop": {"solves_per_s": count / loop_s, "ms_per_batch": loop_s * 1e3},
        "speedup_vs_fp64_loop": loop_s / batch_s,
        "rel_l2_vs_fp64_max": max(errs), "rel_l2_vs_manufactured_u_max": max(errs_u), "tune_s": tune_s,
        "chunks": sorted(set(g["chunk"] for g in sched)),
        "ztable_groups": sum(g["ztable"] for g in sched),
        "tensor_core_dst_groups": sum(1 for g in sched if g["dst_tc"]),
    }


# published Poisson-stage times of the reference's N-body driver, a periodic
# LaplCube<double> solve per step (test/nbody_result.org:9, 24, 39)
PERIODIC_PUBLISHED_MS = {32: {"ryzen_3700x_16t": 1.26, "apple_m1": 1.7},
                         64: {"ryzen_3700x_16t": 6.90, "apple_m1": 8.87},
                         128: {"ryzen_3700x_16t": 62.50, "apple_m1": 68.83}}


def measure_nbody(torch, fdm_gb300, steps=200):
    """The particle-mesh N-body driver at the reference's defaults
    (test/nbody.cpp:593-611: N 100000 bodies, 32^3 periodic mass grid, npp
    64, dt 0.001, G 1, FP64), without and with the pair forces (local 0 / 1).
    Bodies stay on the device; every step after the first is one CUDA graph
    launch.  e2e adds, per step, the copy of positions and velocities back to
    host arrays (what the reference's plot task takes)."""
    from fdm_gb300 import _native

    out = {"workload": "nbody_pm_100000_bodies_32^3", "N": 100000, "n": 32, "npp": 64, "dtype": "f64"}
    for local in (0, 1):
        nb = fdm_gb300.NBody(local=local)
        nb.step(3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nb.step_async(steps)
        nb.sync()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        e2e_steps = 20
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            nb.step(1)
            nb.bodies(("x", "v"))
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        # per-kernel device time of one eager calc_a_pm (the graph hides its
        # launches from the per-launch timers)
        _native.profile_reset()
        _native.profile_enable(True)
        l0 = _native.launch_count()
        nb.calc_a_pm()
        launches = _native.launch_count() - l0
        _native.profile_enable(False)
        prof = _native.profile_collect()
        out["local%d" % local] = {
            "ms_per_step": ms, "steps_per_s": 1e3 / ms, "e2e_ms_per_step": e2e_ms,
            "kernels_per_step": launches,
            "kernels_ms": {k: v[1] for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])},
        }
        nb.close()
    return out


# test/nbody_result.org: ms per step, 1000000 particles, per stage; the
# "Nvidia RTX 3060" column is the reference's Vulkan/GLSL port, the others
# its OpenMP CPU code
NBODY_PUBLISHED = {
    "n32_npp64_pp": {"apple_m1_cpu": 239.66, "apple_m1_gpu": 117.48, "ryzen_3700x_16t": 285.75, "rtx_3060": 31.49,
                     "stages_rtx_3060": {"density": 1.36, "poisson": 0.25, "field": 0.04, "local_forces": 28.84,
                                         "new_positions": 1.00}},
    "n64_npp64_pp": {"apple_m1_cpu": 420.98, "apple_m1_gpu": 128.78, "ryzen_3700x_16t": 440.89, "rtx_3060": 33.54,
                     "stages_rtx_3060": {"density": 2.26, "poisson": 0.86, "field": 0.14, "local_forces": 28.87,
                                         "new_positions": 1.41}},
    "n128_pm": {"apple_m1_cpu": 264.22, "apple_m1_gpu": 97.81, "ryzen_3700x_16t": 359.14, "rtx_3060": 17.57,
                "stages_rtx_3060": {"density": 6.58, "poisson": 5.50, "field": 3.71, "new_positions": 1.78}},
}
# the same file's PM totals on the Nvidia GPU (no local forces), ms per step
NBODY_PM_PUBLISHED = {(2, 32): 4.80, (2, 128): 19.33, (8, 32): 17.33, (8, 128): 43.00, (100, 32): 190.63,
                      (100, 128): 392.87}
NBODY_STAGES = {"density": ("nb_cic", "nb_scan_local", "nb_scan_partials", "nb_scan_add", "nb_fill",
                            "nb_sort_small", "nb_sort_big", "nb_deposit"),
                "poisson": ("pfft_forward", "pdivide", "pfft_inverse"), "field": ("nb_efield",),
                "local_forces": ("nb_pp",), "new_positions": ("nb_accel",)}


def measure_nbody_published(torch, fdm_gb300, steps=5):
    """The configurations of the reference's published N-body table
    (test/nbody_result.org): 10^6 particles on 32^3 and 64^3 mass grids with
    the 64^3 local-force grid, 128^3 without local forces; and PM-only totals
    for 2, 8 and 100 million particles on 32^3 and 128^3 grids.  FP64, the
    driver's other defaults (l 20, dt 0.001, G 1).  Totals are graph-launched
    steps timed with a host clock around a synchronised run; per-stage times
    come from CUDA events of one eager calc_a_pm (the stage grouping of the
    published table)."""
    from fdm_gb300 import _native

    def run(N, n, npp, local, stages):
        nb = fdm_gb300.NBody(n=n, npp=npp, N_bodies=N, local=local)
        nb.step(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nb.step_async(steps)
        nb.sync()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        out = {"ms_per_step": ms}
        if stages:
            _native.profile_reset()
            _native.profile_enable(True)
            nb.calc_a_pm()
            _native.profile_enable(False)
            prof = _native.profile_collect()
            out["stages_ms"] = {st: sum(prof.get(k, (0, 0.0))[1] for k in ks) for st, ks in NBODY_STAGES.items()
                                if local or st != "local_forces"}
        nb.close()
        return out

    res = {"N": 1000000, "dtype": "f64", "published_ms": NBODY_PUBLISHED}
    res["n32_npp64_pp"] = run(1000000, 32, 64, 1, True)
    res["n64_npp64_pp"] = run(1000000, 64, 64, 1, True)
    res["n128_pm"] = run(1000000, 128, 64, 0, True)
    pm = {}
    for (mil, n), pub in NBODY_PM_PUBLISHED.items():
        r = run(mil * 1000000, n, 64, 0, False)
        pm["%dM_n%d" % (mil, n)] = {"ms_per_step": r["ms_per_step"], "published_rtx_3060_ms": pub}
    res["pm_large"] = pm
    return res


def measure_fft3d(torch, fdm_gb300, stream, reps=20):
    """The reference's own 3-D transform benchmark (test/test_fft_3d_bench.cpp:
    FFT<T>::pFFT_1_3d and pFFT_3d of an N^3 cube, N = 32 .. 256, double and
    float) on device-resident cubes: ms per transform, CUDA events over
    `reps` calls."""
    import numpy as np
    out = {"workload": "pFFT_1_3d / pFFT_3d of an N^3 cube (test_fft_3d_bench.cpp)", "reps": reps}
    for dt, tdt in (("double", torch.float64), ("float", torch.float32)):
        for N in (32, 64, 128, 256):
            g = torch.Generator(device="cuda").manual_seed(N)
            s = torch.randn((N, N, N), dtype=tdt, device="cuda", generator=g)
            S = torch.empty_like(s)
            npdt = np.float64 if tdt == torch.float64 else np.float32
            res = {}
            for name, inv in (("pFFT_1_3d", False), ("pFFT_3d", True)):
                fdm_gb300.pfft3d_device(S, s, N, 1.0, inverse=inv, dtype=npdt, stream=stream)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    fdm_gb300.pfft3d_device(S, s, N, 1.0, inverse=inv, dtype=npdt, stream=stream)
                e1.record(stream)
                stream.synchronize()
                res[name + "_ms"] = e0.elapsed_time(e1) / reps
            out["%s_%d" % (dt, N)] = res
    return out


def measure_periodic(torch, fdm_gb300, stream, reps=50):
    """Periodic LaplCube<double> solve (FP64) at 32^3, 64^3, 128^3: device
    time per solve (CUDA events, median of reps) and the host-array call the
    reference's N-body driver makes (copies in and out included)."""
    import numpy as np
    out = {}
    for n in (32, 64, 128):
        h = 1.0 / n
        lc = fdm_gb300.LaplCube(h, h, h, 1.0, 1.0, 1.0, n, n, n, periodic=True)
        rng = np.random.default_rng(n)
        f = rng.standard_normal((n, n, n))
        f -= f.mean()
        df = torch.tensor(f, device="cuda")
        du = torch.empty_like(df)
        for _ in range(3):
            lc.solve_device(du, df, stream=stream)
        stream.synchronize()
        times = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lc.solve_device(du, df, stream=stream)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ans = np.zeros_like(f)
        lc.solve(ans, f)
        t0 = time.perf_counter()
        for _ in range(10):
            lc.solve(ans, f)
        host_ms = (time.perf_counter() - t0) * 100.0
        dev_ms = statistics.median(times)
        pub = PERIODIC_PUBLISHED_MS[n]
        out["%d^3" % n] = {"device_ms": dev_ms, "host_call_ms": host_ms, "published_cpu_ms": pub,
                           "speedup_vs_published_m1_host_call": pub["apple_m1"] / host_ms}
        lc.close()
    return out


SERVE_RATES = (100, 300, 1000, 1500, 3000, 5000)


def measure_serving(torch, fdm_gb300, workloads, dev, rates=SERVE_RATES, seconds=4.0, max_requests=20000,
                    max_outstanding=1024, lanes=48, max_batch=8, max_wait_ms=0.0):
    """Serving loop under Poisson arrivals at each rate: 70% single solves
    (each axis from {31,63,127}, 5% at 255^3, tol 1e-6 or 1e-10 half and
    half), 30% advances of k ~ U{1..50} steps on 64 resident 63^3 cavity
    sessions (Re in {100,250,400}, dt 0.01), 150 GB budget.  Each rate runs
    min(20000, rate x seconds) requests; at most max_outstanding are held by
    the client, later arrivals wait and that wait counts in their latency.
    Every solve's answer is checked against the FP64 form.  max_wait_ms > 0:
    the server sheds requests not started within that time of submission
    (status EBUSY); they count as shed, not in the latencies."""
    import concurrent.futures as cf
    from fdm_gb300 import _native as N
    import numpy as np
    from fdm_gb300.serve import Server
    rng = np.random.default_rng(4242)
    small = [(a, b, c) for a in (31, 63, 127) for b in (31, 63, 127) for c in (31, 63, 127)]
    big = (255, 255, 255)
    geo = {}
    rhs = {}
    ref = {}
    for k, sh in enumerate(small + [big]):
        nx, ny, nz = sh
        args = workloads.solver_args(nx, ny, nz)
        geo[sh] = (args[0:3], args[3:6])
        f = workloads.manufactured_torch(nx, ny, nz, seed=500 + k, kmax=(min(sh) + 1) // 4, device=dev)[0]
        u = torch.empty_like(f)
        fdm_gb300.LaplCube(*args).solve_device(u, f)
        torch.cuda.synchronize()
        rhs[sh] = f.cpu().pin_memory()
        ref[sh] = u.cpu().numpy()
    free = {sh: [] for sh in rhs}

    def out_buf(sh):
        return free[sh].pop() if free[sh] else torch.empty_like(rhs[sh]).pin_memory()

    ref_sq = {sh: float(np.sum(np.square(r))) for sh, r in ref.items()}

    def check(sh, buf, est):
        # relative L2 error of one answer against the FP64 form, beside the
        # server's own estimate of it
        d = buf.numpy() - ref[sh]
        return sh, buf, math.sqrt(float(np.sum(d * d)) / ref_sq[sh]), est

    srv = Server(150e9, lanes=lanes, max_batch=max_batch)
    sess = [srv.session_create(63, 63, Re=(100.0, 250.0, 400.0)[i % 3], dt=0.01) for i in range(64)]
    # warm-up: every plan and every session graph exists before timing
    ids = []
    for sh in rhs:
        for tol in (1e-6, 1e-10):
            b = out_buf(sh)
            ids.append((srv.submit_solve(b, rhs[sh], sh, *geo[sh], tol=tol), sh, b))
    for sid in sess:
        ids.append((srv.submit_advance(sid, 2), None, None))
    for rid, sh, b in ids:
        srv.wait(rid)
        if sh:
            free[sh].append(b)
    if max_wait_ms > 0:
        srv.set_admission(0, max_wait_ms)
    pool = cf.ThreadPoolExecutor(8)
    out = []
    for lam in rates:
        n = int(min(max_requests, max(200, lam * seconds)))
        arrive = np.cumsum(rng.exponential(1.0 / lam, n))
        is_solve = rng.random(n) < 0.7
        is_big = rng.random(n) < 0.05
        axes = rng.choice((31, 63, 127), size=(n, 3))
        tols = np.where(rng.random(n) < 0.5, 1e-6, 1e-10)
        sids = rng.integers(0, 64, n)
        ks = rng.integers(1, 51, n)
        srv.stats_reset()
        live = {}
        lat, lat_solve, lat_adv, errs, ests, futs = [], [], [], [], [], []
        shed = 0
        i = 0
        t0 = time.perf_counter()
        t_last = t0
        while i < n or live:
            now = time.perf_counter() - t0
            while i < n and arrive[i] <= now and len(live) < max_outstanding:
                ts = time.perf_counter() - t0
                if is_solve[i]:
                    sh = big if is_big[i] else tuple(int(v) for v in axes[i])
                    b = out_buf(sh)
                    rid = srv.submit_solve(b, rhs[sh], sh, *geo[sh], tol=float(tols[i]))
                    live[rid] = (arrive[i], ts, sh, b)
                else:
                    rid = srv.submit_advance(sess[sids[i]], int(ks[i]))
                    live[rid] = (arrive[i], ts, None, None)
                i += 1
            wait_ms = 2.0 if i >= n else max(0.0, min(2.0, (arrive[i] - (time.perf_counter() - t0)) * 1e3))
            rec = srv.next_done(wait_ms) if live else None
            while rec is not None:
                a_t, s_t, sh, b = live.pop(rec["id"])
                if rec["state"] == "failed" and rec["status"] == N.EBUSY and max_wait_ms > 0:
                    shed += 1
                    if sh:
                        free[sh].append(b)
                    t_last = time.perf_counter()
                    rec = srv.next_done(0.0) if live else None
                    continue
                if rec["state"] != "done":
                    raise RuntimeError("request failed: %s" % rec)
                l_ms = rec["latency_ms"] + (s_t - a_t) * 1e3
                lat.append(l_ms)
                t_last = time.perf_counter()
                if sh:
                    lat_solve.append(l_ms)
                    futs.append(pool.submit(check, sh, b, rec["err_est"]))
                else:
                    lat_adv.append(l_ms)
                rec = srv.next_done(0.0) if live else None
            keep = []
            for fu in futs:
                if fu.done():
                    sh, b, e, es = fu.result()
                    errs.append(e)
                    ests.append(es)
                    free[sh].append(b)
                else:
                    keep.append(fu)
            futs = keep
        for fu in futs:
            sh, b, e, es = fu.result()
            errs.append(e)
            ests.append(es)
            free[sh].append(b)
        wall = t_last - t0
        st = srv.stats()

        def pct(v, q):
            return float(np.percentile(v, q)) if v else None
        out.append({
            "offered_req_per_s": lam, "requests": n, "achieved_req_per_s": (n - shed) / wall,
            "shed": shed, "shed_fraction": shed / n,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "p50_solve_ms": pct(lat_solve, 50), "p99_solve_ms": pct(lat_solve, 99),
            "p50_advance_ms": pct(lat_adv, 50), "p99_advance_ms": pct(lat_adv, 99),
            "solve_err_vs_fp64_max": max(errs) if errs else None,
            "solve_err_vs_fp64_median": pct(errs, 50), "solves_checked": len(errs),
            "solve_err_est_max": max(ests) if ests else None,
            "solve_err_est_bounds_fraction": (sum(1 for e, es in zip(errs, ests) if es >= e) / len(errs))
            if errs else None,
            "solve_launches": st["batches"], "solves_batched": st["batched_requests"],
            "peak_device_gb": st["peak_bytes"] / 1e9, "mean_queue_ms": st["mean_queue_ms"],
            # the server's own clock, submit to completion (no client-side wait)
            "server_p50_ms": st["p50_ms"], "server_p99_ms": st["p99_ms"], "server_shed": st["shed"],
        })
    pool.shutdown()
    srv.close()
    return {"workload": "70% solves {31,63,127}^3 + 5% 255^3, tol 1e-6/1e-10; 30% advance k~U[1,50] on 64 "
                        "resident 63^3 sessions; Poisson arrivals; 150 GB budget",
            "lanes": lanes, "max_batch": max_batch, "max_outstanding": max_outstanding,
            "queue_deadline_ms": max_wait_ms if max_wait_ms > 0 else None,
            "latency": "arrival to answer in pinned host memory (server clock from submit, plus client wait)",
            "advance_error": "sessions are the plain FP64 NSCube (bit-identical to a lone NSCube)",
            "rates": out}


def run_ncu_case(which: str = "solve"):
    """solve: two mixed solves of 2 RHS at 255^3 (266 MB of FP64 input,
    larger than L2) with nothing else on the GPU.  nscube: a 63^3 cavity,
    Re 250, dt 0.01, stepped 4 times (the first eager, then one captured
    graph replayed).  tc: two mixed solves of 16 RHS at 63^3 (2 MB of FP64
    input per RHS, 32 MB in all) with the tensor-core DST passes.  nbody /
    nbody_pp: four N-body steps, 100000 bodies on the 32^3 mass grid.  The
    cases the committed ncu summaries capture."""
    import torch
    import fdm_gb300
    from fdm_gb300 import workloads
    if which == "tc":
        n = 63
        f = torch.stack([workloads.manufactured_torch(n, n, n, seed=s, kmax=16, noise=NOISE)[0] for s in range(16)])
        out = torch.empty_like(f)
        m = fdm_gb300.LaplCube(*workloads.solver_args(n, n, n), precision="mixed", tol=TOL)
        m.set_schedule(ztable=True, dst_tc=True)
        for _ in range(2):
            m.solve_device(out, f, nrhs=16)
        torch.cuda.synchronize()
        print("ncu case done")
        return
    if which in ("nbody", "nbody_pp"):
        nb = fdm_gb300.NBody(local=1 if which == "nbody_pp" else 0)
        nb.step(4)
        nb.close()
        print("ncu case done")
        return
    if which == "nscube":
        ns = fdm_gb300.NSCube(nx=63, nz=63, Re=250.0, dt=0.01, u0=1.0)
        ns.step(4)
        torch.cuda.synchronize()
        ns.close()
        print("ncu case done")
        return
    n = N_INT
    f = torch.stack([workloads.manufactured_torch(n, n, n, seed=s, kmax=KMAX, noise=NOISE)[0] for s in (0, 1)])
    out = torch.empty_like(f)
    m = fdm_gb300.LaplCube(*workloads.solver_args(n, n, n), precision="mixed", tol=TOL)
    for _ in range(2):
        m.solve_device(out, f.contiguous(), nrhs=2)
    torch.cuda.synchronize()
    print("ncu case done")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop sweep")
    ap.add_argument("--serve-rates", default=None,
                    help="comma-separated arrival rates (req/s) of the serving sweep (default 100,300,1000,1500,3000,5000)")
    ap.add_argument("--ncu-case", nargs="?", const="solve", default=None,
                    choices=["solve", "nscube", "tc", "nbody", "nbody_pp"],
                    help="run only a small case for profiler captures: 'solve' (two mixed solves of 2 RHS at "
                         "255^3), 'nscube' (four 63^3 cavity steps), 'tc' (two mixed solves of 16 RHS at 63^3 "
                         "with the tensor-core DST passes), 'nbody' / 'nbody_pp' (four N-body steps at the "
                         "driver's defaults, without / with the pair forces)")
    ap.add_argument("--chunk", type=int, default=NRHS,
                    help="right-hand sides per solve call within a step (divides 16)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world, rank, local = dist_setup()
    if args.ncu_case:
        run_ncu_case(args.ncu_case)
        return
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import numpy as np
    import torch
    import fdm_gb300
    from fdm_gb300 import _native, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    n = N_INT
    vol = n ** 3
    sargs = workloads.solver_args(n, n, n)

    # inputs: each rank gets its own seeds (replicas, no collective)
    with torch.cuda.stream(stream):
        f = torch.empty((NRHS, n, n, n), dtype=torch.float64, device=dev)
        for i in range(NRHS):
            f[i] = workloads.manufactured_torch(n, n, n, seed=1000 * rank + i, kmax=KMAX, noise=NOISE,
                                                device=dev)[0]
        out = torch.empty_like(f)
        ref64 = torch.empty_like(f)
    stream.synchronize()

    mixed = fdm_gb300.LaplCube(*sargs, precision="mixed", tol=TOL)
    plain = fdm_gb300.LaplCube(*sargs)

    # accuracy of the measured form vs the FP64 GPU form, per RHS
    plain.solve_device(ref64, f, nrhs=NRHS, stream=stream)
    mixed.solve_device(out, f, nrhs=NRHS, stream=stream)
    stream.synchronize()
    errs = [(torch.linalg.norm(out[i] - ref64[i]) / torch.linalg.norm(ref64[i])).item() for i in range(NRHS)]
    sweeps, est = mixed.last_info(NRHS)
    # the closed loop: a handle that checks every right-hand side's estimate
    # and sweeps again while one exceeds tol (the estimates bound the errors)
    adaptive = fdm_gb300.LaplCube(*sargs, precision="mixed", tol=TOL, adaptive=True)
    out2 = torch.empty_like(out)
    adaptive.solve_device(out2, f, nrhs=NRHS, stream=stream)
    a_sweeps, a_est = adaptive.last_info(NRHS)
    del out2, adaptive
    del ref64
    torch.cuda.empty_cache()

    chunk = max(1, min(NRHS, args.chunk))

    def step():
        for i in range(0, NRHS, chunk):
            mixed.solve_device(out[i:i + chunk], f[i:i + chunk], nrhs=chunk, stream=stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()

    sampler = ClockSampler(local)
    with sampler:
        # ---- value: device-resident inputs
        barrier(world)
        torch.cuda.synchronize()
        l0 = _native.launch_count()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        ev[0].record(stream)
        for k in range(args.steps):
            step()
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
        barrier(world)
        launches = _native.launch_count() - l0
        ms = ev[0].elapsed_time(ev[-1])
        step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ms = allreduce_max(world, ms)

        # ---- e2e: host-pointer batch entry point, pinned host buffers
        hf = torch.empty((NRHS, n, n, n), dtype=torch.float64, pin_memory=True)
        hout = torch.empty_like(hf, pin_memory=True)
        hf.copy_(f)
        mixed.solve_batch(hout, hf, NRHS)  # warm-up of the staging buffers
        e2e_steps = max(2, min(args.steps, 5))
        barrier(world)
        torch.cuda.synchronize()
        e2e_step_s = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            mixed.solve_batch(hout, hf, NRHS)  # synchronous: returns with the answers in hout
            e2e_step_s.append(time.perf_counter() - t0)
        torch.cuda.synchronize()
        e2e_s = sum(e2e_step_s)
        barrier(world)
        e2e_s = allreduce_max(world, e2e_s)
    clocks = sampler.summary()

    # ---- per-kernel CUDA-event timing of the same step (after the timed
    # region, so the events do not perturb it)
    _native.profile_reset()
    _native.profile_enable(True)
    for _ in range(2):
        step()
    stream.synchronize()
    _native.profile_enable(False)
    prof = _native.profile_collect()
    dominant = max(prof.items(), key=lambda kv: kv[1][1])
    dname, (dcount, dms) = dominant
    per_launch_ms = dms / dcount
    bpp = KERNEL_BYTES.get(dname)
    hbm, peak_kind = peaks()
    achieved = (bpp * vol * NRHS / (per_launch_ms * 1e-3) / 1e9) if bpp else None
    traffic = None
    tfile = ROOT / "profiles" / "ncu_traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get(dname)
    # what bounds the dominant kernel when it is not HBM (ncu, committed)
    limiter = None
    lfile = ROOT / "profiles" / "ncu_limiters.json"
    if lfile.exists():
        limiter = json.loads(lfile.read_text()).get(dname)

    # ---- context numbers (untimed for the headline): the plain FP64 GPU form
    # on the same inputs, and the NSCube cavity step at 63^3
    e0.record(stream)
    for _ in range(2):
        plain.solve_device(out, f, nrhs=NRHS, stream=stream)
    e1.record(stream)
    stream.synchronize()
    plain_rate = 2 * NRHS / (e0.elapsed_time(e1) * 1e-3)
    # the 1000-step cavity (63^3, Re 250, dt 0.01) from the zero state, as
    # the CPU baseline runs it
    def cavity_ms(exact):
        ns = fdm_gb300.NSCube(nx=63, nz=63, Re=250.0, dt=0.01, u0=1.0)
        ns.set_exact(exact)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ns.step(1000)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / 1000
        ns.close()
        return ms
    ns_ms = cavity_ms(False)
    ns_exact_ms = cavity_ms(True)
    # the cylindrical step at the reference's defaults (nr 32, nz 31, nphi 32)
    cyl = fdm_gb300.NSCyl(Re=100.0, dt=0.001)
    cyl.step(5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cyl.step(200)
    torch.cuda.synchronize()
    cyl_ms = (time.perf_counter() - t0) * 1e3 / 200
    cyl.close()

    del out, f
    torch.cuda.empty_cache()
    uneven = measure_uneven_batch(torch, fdm_gb300, workloads, stream, dev)
    periodic = measure_periodic(torch, fdm_gb300, stream)
    periodic["fft3d"] = measure_fft3d(torch, fdm_gb300, stream)
    nbody = measure_nbody(torch, fdm_gb300)
    nbody["published_configs"] = measure_nbody_published(torch, fdm_gb300)
    rates = tuple(int(x) for x in args.serve_rates.split(",")) if args.serve_rates else SERVE_RATES
    serving = measure_serving(torch, fdm_gb300, workloads, dev, rates=rates) if not args.no_serving else None
    # the same load past saturation with a 100 ms queue deadline: what is
    # not started in time is shed (EBUSY) and the served requests keep
    # bounded latency
    serving_shed = (measure_serving(torch, fdm_gb300, workloads, dev, rates=(1500, 3000, 5000), max_wait_ms=100.0)
                    if not args.no_serving else None)

    solves = args.steps * NRHS * world
    value = solves / (ms * 1e-3)
    e2e_value = e2e_steps * NRHS * world / e2e_s
    step_ms_samples = step_ms
    step_ms = ms / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 in/out; f32 inner solves", "data": "synthetic",
        "config": {"workload": "poisson_dirichlet_255^3_x16rhs", "grid": [n, n, n], "nrhs_per_step": NRHS,
                   "kmax": KMAX, "noise": NOISE, "tol": TOL, "precision": "mixed",
                   "l2_flush": "inputs 2.1 GB per step > 135 MB L2", "parallelism": "replicas%d" % world,
                   "rhs_per_call": chunk},
        "accuracy": {"rel_l2_vs_fp64_gpu_max": max(errs), "rel_l2_vs_fp64_gpu_median": statistics.median(errs),
                     "sweeps": sweeps, "error_estimate_max": max(est),
                     "error_estimate_per_rhs": est, "error_per_rhs": errs,
                     "estimate_bounds_error": all(e >= x for e, x in zip(est, errs)),
                     "adaptive": {"sweeps": a_sweeps, "error_estimate_max": max(a_est)}},
        "latency_ms_per_solve": step_ms / NRHS,
        "unixbench_ms_per_step": unixbench_score(step_ms_samples),
        "pipeline": mixed.pipeline_in_use(),
        "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": [round(1e3 * t, 2) for t in e2e_step_s],
                "h2d_bytes_per_step": NRHS * vol * 8,
                "d2h_bytes_per_step": NRHS * vol * 8},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "peak_source": peak_kind, "algorithmic_bytes_per_point": bpp,
                     "launch_ms": per_launch_ms, "limiter": limiter},
        "solve_roofline": {"achieved_gbs": value / world * SOLVE_BYTES_PER_POINT * vol / 1e9, "peak": hbm,
                           "frac": value / world * SOLVE_BYTES_PER_POINT * vol / 1e9 / hbm,
                           "bytes_per_point": SOLVE_BYTES_PER_POINT},
        "kernels_ms_per_step": {k: v[1] / 2 for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])},
        "plain_fp64_gpu": {"value": plain_rate, "unit": UNIT},
        "nscube_63cubed": {"ms_per_step": ns_ms, "steps_timed": 1000, "Re": 250.0, "dt": 0.01,
                           "clock": "host clock around 1000 graph-launched steps from the zero state",
                           "exact_quotients_ms_per_step": ns_exact_ms},
        "nscyl_32x31x32": {"ms_per_step": cyl_ms, "steps_timed": 200, "Re": 100.0, "dt": 0.001},
        "uneven_batch": uneven,
        "periodic_poisson": periodic,
        "nbody": nbody,
        "serving": serving,
        "serving_with_queue_deadline": serving_shed,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        rate, kind, cores, sample = cpu_reference_rate(5)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                                "cpu_model": cpu_model(),
                                "unixbench_ms_per_solve": 1e3 * unixbench_score(cpu_reference_rate.last_times)}
        # the cavity of the 1000-step case (63^3, Re 250, dt 0.01), every
        # step timed: mean and the reference's unixbench summary
        from oracle.oracle import port
        o = port().nscube(63, 63, 250.0, 0.01)
        nst = []
        for _ in range(1000):
            t0 = time.perf_counter()
            o.step(1)
            nst.append((time.perf_counter() - t0) * 1e3)
        o.close()
        line["cpu_baseline"]["nscube_63cubed_1000_steps"] = {
            "ms_per_step": statistics.fmean(nst), "unixbench_ms_per_step": unixbench_score(nst),
            "total_s": sum(nst) / 1e3, "kind": "port", "threads": cores}
        line["cpu_baseline"]["nscube_63cubed_ms_per_step"] = statistics.fmean(nst)
        # the same solve on one host thread (one 255^3 solve)
        pt = port()
        threads = pt.threads()
        pt.set_threads(1)
        f1, _ = workloads.manufactured(N_INT, N_INT, N_INT, seed=0, kmax=KMAX, noise=NOISE)
        t0 = time.perf_counter()
        pt.lapl_cube(f1, *workloads.solver_args(N_INT, N_INT, N_INT)[:6])
        line["cpu_baseline"]["one_thread_solves_per_s"] = 1.0 / (time.perf_counter() - t0)
        pt.set_threads(threads)
        from oracle.nbody import NBodyPort
        p = NBodyPort(-10.0, -10.0, -10.0, 20.0, 32, 64, 100000, 0.001, 1.0)
        p.step(1)
        t0 = time.perf_counter()
        p.step(3)
        line["cpu_baseline"]["nbody_100000_ms_per_step"] = (time.perf_counter() - t0) * 1e3 / 3
        line["cpu_baseline"]["nbody_kind"] = "port (numpy, 1 thread)"
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
