"""The device order mode of the NodeGroups build (gm_node_groups_build_device):
GPU Jones-Plassmann colours instead of the reference's greedy breadth-first
ones.  The groups must be independent sets (no two vertices of one colour
share an element), deterministic, about as few as the reference's, and a
relocation pass in this order must match the FP64 oracle run in the same
order."""

import numpy as np
import pytest

from gpumesh_gb300 import meshgen, workloads
from gpumesh_gb300 import mesh as M

from helpers import device_for, edge_lengths, oracle_for

pytestmark = pytest.mark.gpu

MR = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")


def colour_of(groups, nv):
    c = np.full(nv, -1, np.int64)
    gb = groups.group_base
    for g in range(groups.count()):
        c[groups.members[gb[g]:gb[g + 1]]] = g
    return c


@pytest.mark.parametrize("kind", ["tet", "hex", "mixed"])
def test_device_groups_are_independent_and_deterministic(kind):
    raw = meshgen.box_mesh(9, kind, 0.2, 1)
    perm, groups = M.node_groups_build(raw, order="device")
    perm2, groups2 = M.node_groups_build(raw, order="device")
    assert np.array_equal(perm, perm2) and np.array_equal(groups.members, groups2.members)
    pr = M.permute_mesh(raw, perm)
    c = colour_of(groups, pr.nv)
    movable = pr.cid >= 0
    assert np.all(c[movable] >= 0) and np.all(c[~movable] < 0)
    for conn in (pr.tets, pr.pris, pr.hexs):
        for e in conn:
            cs = [c[v] for v in e if c[v] >= 0]
            assert len(cs) == len(set(cs)), e
    _, ref_groups = M.node_groups_build(raw)
    assert groups.count() <= 2 * ref_groups.count()


def test_device_order_pass_matches_oracle_in_the_same_order():
    raw0 = meshgen.box_mesh(10, "tet", 0.3, 0)
    perm, groups = M.node_groups_build(raw0, order="device")
    raw = M.permute_mesh(raw0, perm)
    dev = device_for(raw, groups, MR)
    orc = oracle_for(raw, MR)
    orc.pos = raw.pos.astype(np.float32).astype(np.float64)
    b, e = int(groups.group_base[0]), int(groups.group_base[1])
    dev.smooth_group("nelder_mead", b, e - b, workloads.NM_PARAMS)
    orc.smooth_pass("nelder_mead", np.array([0, e - b], np.int64), groups.members[b:e], params=workloads.NM_PARAMS)
    err = (np.linalg.norm(dev.fetch_positions() - orc.pos, axis=1) / edge_lengths(raw))[groups.members[b:e]]
    assert np.mean(err < 1e-4) >= 0.97 and np.median(err) < 1e-5
    # a whole spring-Laplace pass in this order (no decisions): every vertex
    dev = device_for(raw, groups, MR)
    orc = oracle_for(raw, MR)
    orc.pos = raw.pos.astype(np.float32).astype(np.float64)
    dev.smooth_pass("spring_laplace", None)
    orc.smooth_pass("spring_laplace", groups.group_base, groups.members)
    err = np.linalg.norm(dev.fetch_positions() - orc.pos, axis=1) / edge_lengths(raw)
    assert err.max() < 1e-5
