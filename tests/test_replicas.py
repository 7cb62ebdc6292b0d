"""Replicas on several ranks (CPU, gloo): the bench's barrier and max-over-ranks timing,
and the reference arm under torchrun, where rank 0 alone runs and prints one JSON line.
The path has no data exchange between ranks (q-vectors are independent), so these are the
only multi-rank pieces."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(1.5 + rank)
    d.barrier()
    d.close()
    with open(os.path.join(out, "r%d" % rank), "w") as f:
        f.write(repr(m))


def test_dist_barrier_and_max_two_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert [float(open(tmp_path / ("r%d" % r)).read()) for r in range(2)] == [2.5, 2.5]


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.5", "--workload", "incoherent_fqt"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
