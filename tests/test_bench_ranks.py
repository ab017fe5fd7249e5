"""Host side of bench.py's multi-GPU contract, on CPU: replicas only, one
process per GPU, the timed region's time maximised over ranks with gloo, and
the reference arm printed by rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, seconds, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(dist, seconds[rank])
    out.put((rank, t, bench.replica_rate(world, 10, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_timed_region_is_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    seconds = [0.70, 0.75]
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == max(seconds)
        assert abs(v - 2 * 10 / max(seconds)) < 1e-12


def test_replica_rate_without_process_group():
    import bench

    assert bench.max_over_ranks(None, 1.5) == 1.5
    assert bench.replica_rate(1, 10, 2.0) == 5.0


def test_reference_arm_prints_on_rank_zero_only(oracle_lib):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--grid", "32", "--steps", "1", "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_increment_bytes_follow_the_launch_mix():
    """The dominant kernel's algorithmic bytes per cell: each pseudo-iteration
    is one exact anchor or one incremental update (56 B) plus stages 1 (24 B),
    2 and 3 (32 B each); the figure is weighted by the profiled launches."""
    import bench

    # 69 iterations with 3 exact anchors: 66 updates and 207 stage launches
    assert abs(bench.increment_bytes_per_cell({"anchor": (3, 1.0), "increment": (273, 1.0)})
               - (88 * 69 + 56 * 66) / 273) < 1e-12
    # every iteration with an exact anchor: stages only, 88 / 3 B
    assert abs(bench.increment_bytes_per_cell({"anchor": (5, 1.0), "increment": (15, 1.0)}) - 88 / 3) < 1e-12
    # no profile: the fixed figure
    assert bench.increment_bytes_per_cell({}) == bench.ALGO_BYTES_PER_CELL["increment"]
