"""The reference-layout uploads of the drop-in (the calls the shim's
updateCudaVerts / updateCudaTets / Pris / Hexs / updateCudaTopo /
updateCudaGroupMembers make, resources/cuda/Mesh.cu:74-259) against the
native upload of the same mesh.

The buffers are laid out as DataStructures/GpuMesh.h:11-141 defines them:
GpuVert {vec3 p; uint c} (16 bytes), GpuTet {uint v[4]; uint c[1]} (5
words), GpuPri {uint v[6]; uint c[6]} (12), GpuHex {uint v[8]; uint c[8]}
(16), GpuTopo {int type; uint neigVertBase, neigVertCount, neigElemBase,
neigElemCount} with type -1 for fixed vertices and the constraint id
otherwise (GpuMesh::buildGpuTopoBuffers, GpuMesh.cpp:380-414), GpuNeigVert
{uint v}, GpuNeigElem {uint id; int type; int vId}, in the order
Mesh::compileNeighborhoods builds the neighbourhoods.  The cache words hold
arbitrary values, which the library ignores.  Evaluation and every smoother
must then give the native upload's results bit for bit.
"""

import ctypes

import numpy as np
import pytest

from gpumesh_gb300 import _native as N
from gpumesh_gb300 import meshgen, workloads
from gpumesh_gb300 import mesh as M

pytestmark = pytest.mark.gpu

MR = ("uniform", "metric_free", "mean_ratio", 1.0, 1.0)


def legacy_buffers(raw, seed=7):
    rng = np.random.default_rng(seed)
    nv = raw.nv
    verts = np.zeros((nv, 4), np.float32)
    verts[:, :3] = raw.pos
    verts = verts.view(np.uint32)
    verts[:, 3] = rng.integers(0, 2 ** 32, nv, dtype=np.uint64).astype(np.uint32)  # the cache word c

    def records(conn, words):
        rec = rng.integers(0, 2 ** 32, (conn.shape[0], words), dtype=np.uint64).astype(np.uint32)
        rec[:, :conn.shape[1]] = conn
        return np.ascontiguousarray(rec)

    tets, pris, hexs = records(raw.tets, 5), records(raw.pris, 12), records(raw.hexs, 16)
    ve_off, ve, vv_off, vv = M.neighbourhoods(raw)
    topo = np.zeros((nv, 5), np.int32)
    topo[:, 0] = np.where(raw.cid < 0, -1, raw.cid)
    topo[:, 1] = vv_off[:-1]
    topo[:, 2] = np.diff(vv_off)
    topo[:, 3] = ve_off[:-1]
    topo[:, 4] = np.diff(ve_off)
    neig_elem = np.zeros((ve.size, 3), np.int32)
    neig_elem[:, 0] = ve & ((1 << 27) - 1)   # element id
    neig_elem[:, 1] = ve >> 30               # MeshTet / MeshPri / MeshHex::ELEMENT_TYPE
    neig_elem[:, 2] = (ve >> 27) & 7         # the vertex's index in the element
    return verts, tets, pris, hexs, topo, np.ascontiguousarray(vv, np.uint32), neig_elem


class LegacyMesh(M.DeviceMesh):
    """A gm_mesh uploaded only through the reference-layout calls."""

    def __init__(self, raw, groups):
        L = N.lib()
        h = ctypes.c_void_p()
        N.check(L.gm_mesh_create(ctypes.byref(h)))
        self.h, self.nv = h, raw.nv
        verts, tets, pris, hexs, topo, neig_verts, neig_elems = legacy_buffers(raw)
        self._keep = (verts, tets, pris, hexs, topo, neig_verts, neig_elems)
        N.check(L.gm_mesh_upload_gpu_verts(h, raw.nv, N.ptr(verts)))
        N.check(L.gm_mesh_upload_tets(h, tets.shape[0], N.ptr(tets), 5))
        N.check(L.gm_mesh_upload_pris(h, pris.shape[0], N.ptr(pris), 12))
        N.check(L.gm_mesh_upload_hexs(h, hexs.shape[0], N.ptr(hexs), 16))
        N.check(L.gm_mesh_upload_topo(h, raw.nv, N.ptr(topo), neig_verts.size, N.ptr(neig_verts),
                                      neig_elems.shape[0], N.ptr(neig_elems)))
        ck = np.ascontiguousarray(raw.con_kind, np.int32)
        cp = np.ascontiguousarray(raw.con_param, np.float64)
        N.check(L.gm_mesh_set_constraints(h, ck.size, N.ptr(ck), N.ptr(cp)))
        if groups is not None:
            self.set_groups(groups)


def both(raw, groups, crew=MR):
    native, legacy = M.DeviceMesh(raw, groups), LegacyMesh(raw, groups)
    for d in (native, legacy):
        d.set_crew(*crew)
    return native, legacy


def same_quality(a, b):
    qa, qb = a.evaluate().as_dict(), b.evaluate().as_dict()
    assert qa["min"] == qb["min"] and qa["count"] == qb["count"]
    assert qa["inv_sum"] == qb["inv_sum"] or (np.isinf(qa["inv_sum"]) and np.isinf(qb["inv_sum"]))
    assert list(qa["buckets"]) == list(qb["buckets"])


@pytest.mark.parametrize("kind", ["tet", "mixed", "hex"])
def test_reference_layout_uploads_match_native(kind):
    raw = meshgen.box_mesh(7, kind, 0.25, 11, gaussian=(kind != "tet"))
    perm, groups = M.node_groups_build(raw)
    raw = M.permute_mesh(raw, perm)
    native, legacy = both(raw, groups)
    same_quality(native, legacy)
    smoothers = [("nelder_mead", workloads.NM_PARAMS), ("gradient_descent", None), ("spawn_search", None),
                 ("spring_laplace", None), ("getme", workloads.GETME_PARAMS)]
    for smoother, params in smoothers:
        native.smooth_pass(smoother, params)
        legacy.smooth_pass(smoother, params)
        a, b = native.fetch_positions(), legacy.fetch_positions()
        assert np.array_equal(a, b), smoother
        same_quality(native, legacy)


def test_reference_split_by_colour_with_range_transfers():
    """The reference's legacy loop (AbstractVertexWiseSmoother::smoothMeshCuda,
    Smoothers/VertexWise/AbstractVertexWiseSmoother.cpp:419-499): per colour
    the GPU relocates the non-boundary members (NodeGroups::gpuGroupsBuffer,
    one dispatch per colour), the host reads the colour's subsurface range
    back (fetchCudaSubsurfaceVertices) and sends its boundary range
    (sendCudaBoundaryVertices).  Here the boundary vertices are held fixed on
    both sides; the range reads equal the full read."""
    raw = meshgen.box_mesh(8, "tet", 0.3, 4)
    perm, groups = M.node_groups_build(raw)
    raw = M.permute_mesh(raw, perm)
    native, legacy = both(raw, groups)
    gpu_buf = groups.gpuGroupsBuffer()
    legacy_groups = M.NodeGroups(np.array([0, gpu_buf.size], np.uint32), gpu_buf, groups.ranges)
    legacy.set_groups(legacy_groups)
    L = N.lib()
    base = 0
    for g, pg in enumerate(groups.parallelGroups()):
        members = groups.members[groups.group_base[g]:groups.group_base[g + 1]]
        nb = pg.boundaryRange[1] - pg.boundaryRange[0]
        count = members.size - nb
        legacy.smooth_group("nelder_mead", base, count, workloads.NM_PARAMS)
        native.smooth_group("nelder_mead", int(groups.group_base[g]) + nb, count, workloads.NM_PARAMS)
        base += count
        s0, s1 = pg.subsurfaceRange
        sub = np.zeros((max(1, s1 - s0), 4), np.float32)
        N.check(L.gm_mesh_fetch_gpu_verts_range(legacy.h, int(s0), int(s1 - s0), N.ptr(sub)))
        full = legacy.fetch_positions()
        assert np.array_equal(sub[: s1 - s0, :3].astype(np.float64), full[s0:s1])
        b0, b1 = pg.boundaryRange
        if b1 > b0:
            rec = np.zeros((b1 - b0, 4), np.float32)
            rec[:, :3] = full[b0:b1]
            N.check(L.gm_mesh_upload_gpu_verts_range(legacy.h, int(b0), int(b1 - b0), N.ptr(rec)))
    assert base == gpu_buf.size
    assert np.array_equal(native.fetch_positions(), legacy.fetch_positions())
    same_quality(native, legacy)
