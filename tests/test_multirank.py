"""bench.py's multi-rank plumbing on CPU: two processes over the gloo backend
(one process per GPU is the contract on a GPU machine; the path shards by
replicas, so the only cross-rank steps are the barriers around the timed
region and the max over ranks of the elapsed time)."""
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = textwrap.dedent("""
    import os, sys, time, json
    sys.path.insert(0, {root!r})
    import bench
    world, rank, local = bench.dist_setup()
    # a slower rank: the barrier holds the other, and the max over ranks is its time
    t0 = time.perf_counter()
    if rank == 1:
        time.sleep(0.3)
    bench.barrier(world)
    waited = time.perf_counter() - t0
    mine = 1.0 + rank
    slowest = bench.allreduce_max(world, mine)
    # the reference arm: ranks other than 0 leave without work
    r = bench.run_reference(None, world, rank) if rank != 0 else None
    print(json.dumps({{"world": world, "rank": rank, "waited": waited, "max": slowest, "ref": r}}))
    import torch.distributed as dist
    dist.destroy_process_group()
""")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_ranks_barrier_and_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    import json
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                   LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    by_rank = {o["rank"]: o for o in outs}
    assert by_rank[0]["world"] == 2 and by_rank[1]["world"] == 2
    assert by_rank[0]["waited"] >= 0.25  # rank 0 waited for rank 1 at the barrier
    assert by_rank[0]["max"] == by_rank[1]["max"] == 2.0
    assert by_rank[1]["ref"] is None
