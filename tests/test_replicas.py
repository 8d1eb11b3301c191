"""The multi-process path of bench.py on CPU: two gloo ranks, 127.0.0.1.

The single-domain step does not shard (replicas only): under torchrun every
rank integrates its own domain with no data-path collective, and the only
collectives are the barriers around the timed region and the max over ranks
of its time.  These tests run that host logic without a GPU.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["REPO_ROOT"])
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank, world = dist.get_rank(), dist.get_world_size()
bench.barrier(dist)
ms, value = bench.replica_result(dist, 10.0 + 5.0 * rank, world, 1000, 4, "cpu")
bench.barrier(dist)
print(json.dumps({"rank": rank, "ms": ms, "value": value}), flush=True)
dist.destroy_process_group()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code, world, extra_args=()):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r), LOCAL_RANK=str(r),
                   WORLD_SIZE=str(world), REPO_ROOT=ROOT)
        cmd = [sys.executable, "-c", code] if code else [sys.executable, os.path.join(ROOT, "bench.py"), *extra_args]
        procs.append(subprocess.Popen(cmd, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=180)
            assert p.returncode == 0, err[-2000:]
            outs.append(out)
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    return outs


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    outs = _launch(WORKER, 2)
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in res) == [0, 1]
    for r in res:
        assert r["ms"] == 15.0  # the slower rank's timed region
        assert abs(r["value"] - 2 * 1000 * 4 / 15e-3) < 1e-6 * r["value"]


def test_reference_arm_prints_on_rank_zero_only():
    """--impl reference under torchrun: ranks other than 0 exit 0 without work
    or output (rank 0 alone times the CPU step)"""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_reference_arm_aggregates_replicas_on_host_cores():
    """the reference arm's all-core timing: spawned replicas of the serial
    step (here 2 on a small thunderstorm), each warmed up and stepping behind
    one barrier; the value is replicas x points x steps over the slowest"""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench  # spawned workers import it by name
    out = bench.cpu_all_cores(2, ncores=2, nx=20, ny=18, nz=12)
    assert out["cores"] == 2 and out["kind"] == "port"
    slow = out["slowest_replica_s"]
    assert slow > 0
    assert abs(out["value"] - 2 * 20 * 18 * 12 * 2 / slow) <= 1e-6 * out["value"]
