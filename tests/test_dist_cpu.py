"""Multi-GPU host logic on CPU: two gloo ranks (no GPU).

bench.py runs one replica per GPU: images are independent, so the only
cross-rank steps are the timing barrier and the max-over-ranks of the timed
region; under the reference arm only rank 0 works and prints.  These run
here as two processes on 127.0.0.1.
"""
import json
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import json, os, sys, time
    sys.path.insert(0, %r)
    import bench
    rank, world, local, dist = bench.dist_setup()
    assert (rank, world) == (int(os.environ["RANK"]), 2)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.5 + rank)          # rank 1 is the slow one
    bench.barrier(dist)
    print(json.dumps({"rank": rank, "max": t}), flush=True)
    dist.destroy_process_group()
""") % ROOT


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_barrier_and_max_over_ranks():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=240) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    got = sorted(json.loads(o.strip().splitlines()[-1])["max"] for o, _ in outs)
    assert got == [2.5, 2.5], "every rank sees the slowest rank's time"


def test_reference_arm_only_rank0_works():
    """A non-zero rank of `bench.py --impl reference` exits 0 without output."""
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="1", CUDA_VISIBLE_DEVICES="")
    code = textwrap.dedent("""
        import sys; sys.path.insert(0, %r)
        import bench
        bench.dist_setup = lambda: (1, 2, 1, None)     # rank 1 of 2, no group needed for this path
        class A: steps = 1; warmup = 0; gpus = 2; workload = "c1"
        bench.run_reference(A())
    """) % ROOT
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
