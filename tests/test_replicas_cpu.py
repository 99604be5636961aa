"""Replicas on CPU: bench.py's multi-rank plumbing with two gloo ranks.

The smoothing path has no exchange step, so N GPUs run N independent
replicas: each rank takes a round-robin share of the independent units
(meshes of the batched workload, jobs of the served stream), and the only
collectives are the timing barrier, the max of the step times and the sum of
the units processed.  These tests run that plumbing as two processes over
gloo on 127.0.0.1, with no GPU.
"""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "GM_DIST_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import json

    import torch.distributed as dist

    import bench
    from gpumesh_gb300 import meshgen, serve

    r, w, local = bench.dist_init(1)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(w)
    res = {
        "max": bench.max_over_ranks(1.5 + rank, w),
        "sum": bench.sum_over_ranks(10 * (rank + 1), w),
        # C4: this rank's meshes of a 2 x 64 mesh stream
        "meshes": bench.shard(range(64 * w), r, w),
        "sizes": [int(s) for s in meshgen.batch_sizes(64 * w, 4, 24, 3)],
        # C5: this rank's jobs of a stream at world x the rate
        "jobs": [j.job_id for j in bench.shard(serve.poisson_stream(200.0 * w, 0.5, 4), r, w)],
    }
    bench.barrier(w)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    import json

    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    # timing: the max over ranks; units: the sum
    assert all(x["max"] == 2.5 for x in res)
    assert all(x["sum"] == 30 for x in res)
    # every mesh and every job is served by exactly one rank, and each rank
    # gets the same share (weak scaling)
    meshes = res[0]["meshes"] + res[1]["meshes"]
    assert sorted(meshes) == list(range(128)) and len(res[0]["meshes"]) == 64
    assert res[0]["sizes"] == res[1]["sizes"]
    jobs = res[0]["jobs"] + res[1]["jobs"]
    assert sorted(jobs) == list(range(len(jobs)))
    assert abs(len(res[0]["jobs"]) - len(res[1]["jobs"])) <= 1


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.sum_over_ranks(7, 1) == 7
    assert bench.shard(range(5), 0, 1) == [0, 1, 2, 3, 4]
