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


# Mesh::compileNeighborhoods / Mesh::addEdge (DataStructures/Mesh.cpp:365-460)
# restated with numpy: every element's edges in element order (tets, prisms,
# hexes) and edge-table order; a vertex's neighbours in the order their edge
# is first met; its elements in element order.
_EDGES = {4: ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)),
          6: ((0, 1), (0, 2), (1, 2), (0, 3), (1, 4), (2, 5), (3, 4), (3, 5), (4, 5)),
          8: ((0, 1), (0, 3), (1, 2), (2, 3), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (4, 7), (5, 6), (6, 7))}


def _reference_neighbourhoods(raw):
    nv = raw.nv
    a, b, refs_v, refs = [], [], [], []
    for type_code, conn in ((0, raw.tets), (2, raw.pris), (3, raw.hexs)):
        k = conn.shape[1]
        if not conn.shape[0]:
            continue
        ids = np.arange(conn.shape[0], dtype=np.uint64)
        for local in range(k):
            refs_v.append(conn[:, local].astype(np.int64))
            refs.append((np.uint64(type_code) << np.uint64(30)) | (np.uint64(local) << np.uint64(27)) | ids)
        # element-major edge events
        ea = np.stack([conn[:, e0] for e0, _ in _EDGES[k]], axis=1).reshape(-1)
        eb = np.stack([conn[:, e1] for _, e1 in _EDGES[k]], axis=1).reshape(-1)
        a.append(ea.astype(np.int64))
        b.append(eb.astype(np.int64))
    # element refs: by vertex, then element order (tets < prisms < hexes, then id)
    rv = np.concatenate(refs_v)
    rr = np.concatenate(refs).astype(np.uint64)
    tcode = rr >> np.uint64(30)
    eid = rr & np.uint64((1 << 27) - 1)
    order = np.lexsort((eid, tcode, rv))
    ve_off = np.concatenate([[0], np.cumsum(np.bincount(rv, minlength=nv))]).astype(np.uint32)
    ve = rr[order].astype(np.uint32)
    # edge neighbours: both directions, first occurrence of each pair, by vertex then first occurrence
    a, b = np.concatenate(a), np.concatenate(b)
    seq = np.arange(a.shape[0], dtype=np.int64)
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    sq = np.concatenate([seq, seq])
    key = src * nv + dst
    o = np.lexsort((sq, key))
    key, sq, src, dst = key[o], sq[o], src[o], dst[o]
    first = np.ones(key.shape[0], bool)
    first[1:] = key[1:] != key[:-1]
    src, dst, sq = src[first], dst[first], sq[first]
    o = np.lexsort((sq, src))
    vv_off = np.concatenate([[0], np.cumsum(np.bincount(src, minlength=nv))]).astype(np.uint32)
    return ve_off, ve, vv_off, dst[o].astype(np.uint32)


@pytest.mark.parametrize("build", [lambda: meshgen.box_mesh(5, "mixed", 0.2, 1),      # sequential path
                                   lambda: meshgen.box_mesh(44, "tet", 0.2, 1),       # threaded path (91k vertices)
                                   lambda: meshgen.box_mesh(42, "mixed", 0.2, 1)])
def test_neighbourhoods_follow_the_reference_order(build):
    raw = build()
    got = M.neighbourhoods(raw)
    want = _reference_neighbourhoods(raw)
    for g, w, name in zip(got, want, ("ve_off", "ve", "vv_off", "vv")):
        assert np.array_equal(g, w), name
