"""Multi-rank bench plumbing on CPU: two gloo ranks over 127.0.0.1 (replicas
only -- the DIC path has no data-path collective; the bench's only exchange is
the max of the per-rank timed region, and the aggregate throughput counts the
POIs of every rank)."""
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    import bench
    world, rank, local = bench.dist_setup(2)
    assert world == 2 and rank == int(os.environ["RANK"])
    bench.dist_barrier(world)
    ms = [100.0, 250.0][rank]  # per-rank timed region
    total = bench.max_over_ranks(ms, world)
    pois, steps = 1000, 5
    value = pois * steps * world / (total / 1000.0)
    print(json.dumps({{"rank": rank, "max_ms": total, "value": value}}))
    import torch.distributed as dist
    dist.destroy_process_group()
""")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_take_the_max_and_aggregate():
    import json
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), TWDIC_BENCH_BACKEND="gloo", CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["max_ms"] == 250.0
        assert abs(o["value"] - 1000 * 5 * 2 / 0.25) < 1e-6
