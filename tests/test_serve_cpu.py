"""Served workload host logic (no GPU): the Poisson stream, and the
template/job equivalence that lets a job reuse a resident topology."""

import math

import numpy as np

from gpumesh_gb300 import mesh as M
from gpumesh_gb300 import meshgen, serve


def test_stream_is_deterministic_and_poisson():
    a = serve.poisson_stream(200.0, 5.0, 4)
    b = serve.poisson_stream(200.0, 5.0, 4)
    assert [(j.arrival, j.n, j.kind, j.smoother) for j in a] == [(j.arrival, j.n, j.kind, j.smoother) for j in b]
    assert 850 < len(a) < 1150  # ~ rate * seconds
    gaps = np.diff([0.0] + [j.arrival for j in a])
    assert abs(gaps.mean() - 1 / 200.0) < 0.2 / 200.0
    assert {j.smoother for j in a} == set(serve.SMOOTHERS)
    assert {j.kind for j in a} == {"cube", "sphere"}


def test_sizes_cover_the_range():
    jobs = serve.poisson_stream(200.0, 20.0, 4)
    tets = [6 * j.n ** 3 if j.kind == "cube" else math.pi * j.n ** 3 for j in jobs]
    assert min(tets) < 3e3 and max(tets) > 1e6


def test_job_positions_from_template_equal_the_generator():
    for kind, n, seed in (("cube", 5, 17), ("sphere", 9, 23)):
        if kind == "cube":
            base = meshgen.box_mesh(n, "tet", 0.0, 0)
            job = meshgen.box_mesh(n, "tet", 0.3, seed)
            pos = meshgen.box_positions(n, 0.3, seed)
        else:
            base = meshgen.sphere_mesh(n, 0.0, 0)
            job = meshgen.sphere_mesh(n, 0.25, seed)
            pos = meshgen.sphere_positions(n, 0.25, seed)
        assert np.array_equal(pos, job.pos)
        assert np.array_equal(base.tets, job.tets) and np.array_equal(base.cid, job.cid)
        p0, g0 = M.node_groups_build(base)
        p1, g1 = M.node_groups_build(job)
        # the colouring depends on the topology only, so jobs share it
        assert np.array_equal(p0, p1) and np.array_equal(g0.members, g1.members)
