"""CPU, world size 2 over gloo (127.0.0.1): the replica path of bench.py — the
max-over-ranks time and summed work of allreduce_max_sum, and the reference
arm under torchrun, where rank 0 alone prints one JSON line and every rank
exits 0."""

import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench

    w, r, _, pg = bench.dist_setup()
    mx, sm = bench.allreduce_max_sum(pg, [float(r + 1), 10.0 * r], [float(r + 1)])
    out.put((r, w, mx, sm))
    pg.barrier()
    pg.destroy_process_group()


def test_allreduce_max_sum_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r, w, mx, sm in res:
        assert w == 2
        assert mx == [2.0, 10.0]  # max over ranks
        assert sm == [3.0]        # work summed over ranks


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--steps", "2",
           "--warmup", "3"]  # (torchrun's parser would take "--n" for its own options)
    p = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
