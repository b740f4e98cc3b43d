"""The multi-GPU path of the benchmark: replicas only (the pressure solve does
not shard).  With world size 2 on the gloo backend (CPU), each rank's timed
seconds reduce to the job's maximum, the whole-job throughput counts every
rank's solves, and the reference arm's non-zero ranks exit without work."""
import json
import os
import socket
import subprocess
import sys
import textwrap
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

CHILD = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="env://")
    rank, world, _ = bench.dist_env()
    local = [0.75, 1.25][rank]
    job = bench.job_seconds(local, world, device="cpu")
    thr = bench.replica_throughput(world, 5, job)
    print(json.dumps({{"rank": rank, "job": job, "throughput": thr}}), flush=True)
    dist.barrier()
    dist.destroy_process_group()
""")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_to_the_job_time():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=str(ROOT))], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["job"] == 1.25
        assert abs(o["throughput"] - 2 * 5 / 1.25) < 1e-12


def test_reference_arm_other_ranks_exit_without_work(capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    ns = type("A", (), dict(n=128, seed=3, tol=1e-8, steps=1, warmup=0, gpus=2))()
    bench.run_reference(ns, rank=1, world=2)
    err = capsys.readouterr().err
    assert json.loads(err.strip())["skipped"] is True
