"""The multi-process path of the benchmark without a GPU: the solver path does not shard
(independent virtual sources run as replicas), so N > 1 means N independent replicas joined
only by a barrier and a max-reduction of the timed region, over gloo.  World size 2 on
127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    worst = d.max(local_ms)
    value = bench.replica_value(world, 1_000_000, 32, worst)
    d.barrier()
    d.close()
    out.put((rank, worst, value))


def test_barrier_and_max_over_two_gloo_ranks():
    torch_mp = pytest.importorskip("torch.multiprocessing")
    ctx = torch_mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    # both ranks see the slowest replica's time; the value counts both replicas' points
    assert [g[1] for g in got] == [15.0, 15.0]
    assert got[0][2] == got[1][2] == pytest.approx(2 * 1_000_000 * 32 / 15.0e-3 / 1e9)


def test_reference_arm_prints_one_line_under_torchrun():
    """--impl reference under a 2-process launch: rank 0 times the restatement and prints the
    line, rank 1 exits 0 without work"""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--config", "media", "--grid", "24x20x12", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
