"""Host topology: independent groups (no two vertices of one colour share an
element), the colour-major member order, and the vertex classes of
NodeGroups::determineTypes (DataStructures/NodeGroups.cpp:124-241)."""

import numpy as np
import pytest

from gpumesh_gb300 import meshgen
from gpumesh_gb300 import mesh as M


def elements(raw):
    return [raw.tets, raw.pris, raw.hexs]


@pytest.mark.parametrize("kind", ["tet", "hex", "mixed"])
def test_groups_are_independent(kind):
    raw = meshgen.box_mesh(5, kind, 0.2, 1)
    perm, groups = M.node_groups_build(raw)
    pr = M.permute_mesh(raw, perm)
    colour = -np.ones(raw.nv, np.int64)
    for g in range(groups.count()):
        colour[groups.members[groups.group_base[g]:groups.group_base[g + 1]]] = g
    for E in elements(pr):
        if E.size == 0:
            continue
        c = colour[E]
        for i in range(E.shape[1]):
            for j in range(i + 1, E.shape[1]):
                clash = (c[:, i] == c[:, j]) & (c[:, i] >= 0)
                assert not clash.any()


def test_permutation_and_classes():
    raw = meshgen.box_mesh(6, "tet", 0.3, 0)
    perm, groups = M.node_groups_build(raw)
    assert sorted(perm.tolist()) == list(range(raw.nv))
    pr = M.permute_mesh(raw, perm)
    # fixed vertices first, then boundary / subsurface / interior ranges per colour
    nfixed = int(np.count_nonzero(raw.cid < 0))
    assert (pr.cid[:nfixed] < 0).all() and (pr.cid[nfixed:] >= 0).all()
    assert groups.members.size == raw.nv - nfixed
    for g, pg in enumerate(groups.parallelGroups()):
        b0, b1 = pg.boundaryRange
        assert (pr.cid[b0:b1] > 0).all()
        s0, s1 = pg.subsurfaceRange
        i0, i1 = pg.interiorRange
        assert (pr.cid[s0:s1] == 0).all() and (pr.cid[i0:i1] == 0).all()
        n = (b1 - b0) + (s1 - s0) + (i1 - i0)
        assert n == pg.undispatchedNodes.size
    # permutation keeps the geometry
    assert np.allclose(pr.pos, raw.pos[perm])


def test_build_is_deterministic():
    raw = meshgen.sphere_mesh(12, 0.25, 1)
    a = M.node_groups_build(raw)
    b = M.node_groups_build(raw)
    assert (a[0] == b[0]).all() and (a[1].members == b[1].members).all()
