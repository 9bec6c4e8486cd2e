"""The multi-rank path of bench.py on the CPU (gloo, world size 2): the barrier and the
max / sum reductions the timing uses, the disjoint per-rank trajectory ids of the
replica batches, and the reference arm launched under torchrun (rank 0 prints the one
JSON line, rank 1 exits without work)."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    out.put((rank, d.max(rank + 1.5), d.sum(rank + 1.0), d.world, bench.replica_trajs(list(range(8)), rank)))
    d.barrier()
    d.close()


def test_gloo_reductions_and_replica_ids():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, world, ids in res:
        assert world == 2 and mx == 2.5 and sm == 3.0
    ids0, ids1 = res[0][4], res[1][4]
    assert ids0 == list(range(8)) and ids1 == list(range(8, 16))
    assert not set(ids0) & set(ids1)


def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-steps", "3000"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
