"""The multi-GPU path of bench.py is replicas only (independent right-hand
sides per rank, no collective on the data path): two gloo ranks on the CPU
check its rendezvous, barrier and max-over-ranks timing reduction, and that
only rank 0 runs the reference arm."""
import io
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    # CPU ranks only (gloo), whatever machine runs the test: no GPU is
    # shared between ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank's step time differs; every rank sees the slowest one
    mx = bench.allreduce_max(w, 10.0 + rank)
    # ranks other than 0 leave the reference arm without work or output
    out = io.StringIO()
    if rank != 0:
        with redirect_stdout(out):
            bench.run_reference_arm(None, w, r)
    q.put((rank, mx, out.getvalue()))
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    assert all(mx == 11.0 for _, mx, _ in res)
    assert res[1][2] == ""
