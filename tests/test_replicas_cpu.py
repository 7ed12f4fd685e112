"""Several GPUs run independent replicas: only timing scalars cross ranks.
These run as world_size-2 gloo process groups on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, size, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(size),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    from fvm2d_gb300 import replicas
    assert replicas.init("gloo")
    assert replicas.world() == (rank, rank, size)
    replicas.barrier()
    mx = replicas.max_over_ranks(10.0 + rank)
    sm = replicas.sum_over_ranks(100 * (rank + 1))
    mine = replicas.shard(list(range(7)), rank, size)
    seeds = [replicas.seed_for(rank, k) for k in range(3)]
    replicas.finish()
    out.put((rank, mx, sm, mine, seeds))


def test_timing_reductions_and_sharding_over_two_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, mx0, sm0, sh0, sd0), (r1, mx1, sm1, sh1, sd1) = res
    assert mx0 == mx1 == 11.0                    # max of elapsed times
    assert sm0 == sm1 == 300.0                   # total work of the job
    assert sorted(sh0 + sh1) == list(range(7)) and not set(sh0) & set(sh1)
    assert not set(sd0) & set(sd1)               # distinct meshes per replica


def test_reference_arm_prints_once_under_torchrun():
    """bench.py --impl reference on two ranks: rank 0 times the CPU
    reference and prints one line; the other rank exits without work."""
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
