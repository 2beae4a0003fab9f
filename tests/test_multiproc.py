"""The N > 1 harness of bench.py on the CPU: two gloo ranks (replicas only).

The sweep has no data-path exchange on one GPU per process, so bench.py runs N
independent replicas; what needs testing is the harness: rendezvous on
127.0.0.1, barrier, max over ranks, and rank 0 alone printing the line.
"""

import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist("reference")  # gloo
    m = d.max(float(10 * (rank + 1)))
    d.barrier()
    q.put((rank, m, d.backend))
    d.close()


def test_dist_max_over_ranks_gloo():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in out) == [0, 1]
    assert all(m == 20.0 and b == "gloo" for _, m, b in out)


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--nnz", "40000",
           "--cpu-sample", "4000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_no_product_library():
    """The reference arm times the oracle port on a numpy-drawn sample: neither the
    package nor its shared library may be loaded in that process."""
    code = (
        "import sys, json, bench\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--cpu-sample', '3000']\n"
        "bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libgputucker_gb300' not in maps, 'product library mapped'\n"
        "assert 'gputucker_gb300' not in sys.modules, 'product package imported'\n"
        "assert 'libgtk_oracle' in maps\n"
    )
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["impl"] == "reference" and d["config"]["workload"] == "zipf4d_100M_rank10_P4"
