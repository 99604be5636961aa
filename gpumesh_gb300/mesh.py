"""Host-side mirror of GpuMesh's plugin interfaces over the native C ABI.

The class and method names follow the reference (DataStructures/Mesh.h,
MeshCrew.h, NodeGroups.h, QualityHistogram.h, Schedule.h;
Evaluators/AbstractEvaluator.h; Smoothers/AbstractSmoother.h; Samplers/;
Measurers/) so that driver code reads like the reference's own callers
(GpuMeshCharacter::smoothMesh / evaluateMesh).  The only implementation is
"CUDA": every evaluation and relocation runs in libgpumesh_gb300.so on the
current CUDA device, with the mesh kept resident between calls.
"""

from __future__ import annotations

import ctypes
import dataclasses
import math
import time
import warnings

import numpy as np

from . import _native as N
from .meshgen import RawMesh

CUDA_IMPL_NAME = "CUDA"


# ---------------------------------------------------------------------------
# QualityHistogram / Schedule / OptimizationPass
# ---------------------------------------------------------------------------
class QualityHistogram:
    """DataStructures/QualityHistogram.h: min, harmonic mean, 20 buckets."""

    def __init__(self, bucket_count: int = 20):
        self._buckets = np.zeros(bucket_count, np.int64)
        self.clear()

    def clear(self):
        self._sample_count = 0
        self._minimum = 1.0
        self._inv_sum = 0.0
        self._buckets[:] = 0

    def bucketCount(self) -> int:
        return int(self._buckets.size)

    def buckets(self) -> np.ndarray:
        return self._buckets

    def sampleCount(self) -> int:
        return self._sample_count

    def setSampleCount(self, n: int):
        self._sample_count = int(n)

    def minimumQuality(self) -> float:
        return self._minimum

    def setMinimumQuality(self, v: float):
        self._minimum = float(v)

    def harmonicMean(self) -> float:
        # QualityHistogram.h:72-75
        with np.errstate(divide="ignore", invalid="ignore"):
            return float(np.float64(self._sample_count) / np.float64(self._inv_sum))

    def invQualitySum(self) -> float:
        return self._inv_sum

    def setInvQualitySum(self, v: float):
        self._inv_sum = float(v)

    def nonPositiveCount(self) -> int:
        return getattr(self, "_nbad", 0)

    @classmethod
    def from_native(cls, q: N.Quality) -> "QualityHistogram":
        h = cls(20)
        h._minimum = q.min
        h._inv_sum = q.inv_sum
        h._sample_count = int(q.count)
        h._nbad = int(q.nbad)
        h._buckets[:] = np.frombuffer(bytes(q.buckets), dtype=np.uint64).astype(np.int64)
        return h

    def as_dict(self) -> dict:
        return {"min": self._minimum, "mean": self.harmonicMean(), "inv_sum": self._inv_sum,
                "count": self._sample_count, "buckets": self._buckets.tolist()}


@dataclasses.dataclass
class Schedule:
    """DataStructures/Schedule.cpp:4-12 defaults, topology operations off."""

    autoPilotEnabled: bool = False
    minQualThreshold: float = 0.001
    qualMeanThreshold: float = 0.0
    topoOperationEnabled: bool = False
    topoOperationPassCount: int = 5
    globalPassCount: int = 5
    relocationPassCount: int = 10


@dataclasses.dataclass
class OptimizationPass:
    timeStamp: float
    histogram: QualityHistogram


# ---------------------------------------------------------------------------
# samplers / measurers
# ---------------------------------------------------------------------------
class AbstractSampler:
    kind = "uniform"
    metric_wise = False

    def __init__(self):
        self._scaling = 1.0
        self._aspect = 1.0
        self._depth = -1

    def isMetricWise(self) -> bool:
        return self.metric_wise

    def discretizationDepth(self) -> int:
        return self._depth

    def setDiscretizationDepth(self, depth: int):
        """AbstractSampler::setDiscretizationDepth: the kd-tree height /
        texture resolution of the sampled samplers; -1 picks it from the
        vertex count."""
        self._depth = int(depth)

    def scaling(self) -> float:
        return self._scaling

    def setScaling(self, s: float):
        self._scaling = float(s)

    def aspectRatio(self) -> float:
        return self._aspect

    def setAspectRatio(self, r: float):
        self._aspect = float(r)


class UniformSampler(AbstractSampler):
    """Samplers/UniformSampler.cpp: M = scaling^2 I."""
    kind = "uniform"
    metric_wise = False


class AnalyticSampler(AbstractSampler):
    """Samplers/AnalyticSampler.cpp + AbstractSampler::vertMetric (AbstractSampler.cpp:190-208)."""
    kind = "analytic"
    metric_wise = True


class LocalSampler(AbstractSampler):
    """Samplers/LocalSampler.cpp: the analytic metric stored at the vertices
    of a background tet mesh (the mesh when the sampling was last updated,
    split into tets) and interpolated barycentrically in the tet holding the
    point.  updateAnalyticalMetric (:193-203) rebuilds the background from
    the mesh's current positions."""
    kind = "local"
    metric_wise = True

    def updateAnalyticalMetric(self, mesh):
        dev = mesh.device()
        dev.set_discretization_depth(self.discretizationDepth())
        dev.set_crew(self.kind, "metric_wise", "mean_ratio", self.scaling(), self.aspectRatio())
        dev.build_local_background()


class KdTreeSampler(LocalSampler):
    """Samplers/KdTreeSampler.cpp: the local metric sampled once per leaf of
    a kd-tree over the vertices (median splits on the widest extent),
    constant inside a leaf."""
    kind = "kdtree"


class TextureSampler(LocalSampler):
    """Samplers/TextureSampler.cpp: the local metric sampled at the cell
    centres of a grid of about one cell per vertex, trilinear in between."""
    kind = "texture"


class SineSampler(AbstractSampler):
    """Sine-graded anisotropic metric scaling^2 * diag(1 + 9 sin^2(4 pi x), 1, 1)."""
    kind = "sine"
    metric_wise = True


class MetricFreeMeasurer:
    kind = "metric_free"


class MetricWiseMeasurer:
    kind = "metric_wise"


# ---------------------------------------------------------------------------
# NodeGroups / Mesh
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class ParallelGroup:
    boundaryRange: tuple
    subsurfaceRange: tuple
    interiorRange: tuple
    undispatchedNodes: np.ndarray


class NodeGroups:
    """DataStructures/NodeGroups.h: colour-major independent vertex groups."""

    def __init__(self, group_base: np.ndarray, members: np.ndarray, ranges: np.ndarray):
        self.group_base = group_base.astype(np.int64)
        self.members = members.astype(np.uint32)
        self.ranges = ranges.reshape(-1, 6).astype(np.int64)

    def count(self) -> int:
        return int(self.group_base.size - 1)

    def parallelGroups(self):
        out = []
        for g in range(self.count()):
            r = self.ranges[g]
            out.append(ParallelGroup((int(r[0]), int(r[1])), (int(r[2]), int(r[3])), (int(r[4]), int(r[5])),
                                     self.members[self.group_base[g]:self.group_base[g + 1]]))
        return out

    def serialGroup(self) -> np.ndarray:
        return np.sort(self.members)

    def gpuGroupsBuffer(self) -> np.ndarray:
        """Non-boundary members of each colour (NodeGroups.cpp:589-618)."""
        parts = []
        for g in range(self.count()):
            r = self.ranges[g]
            m = self.members[self.group_base[g]:self.group_base[g + 1]]
            parts.append(m[(r[1] - r[0]):])
        return np.concatenate(parts) if parts else np.zeros(0, np.uint32)


def node_groups_build(raw: RawMesh, permute: bool = True, order: str = "reference"):
    """NodeGroups::build on the host (native): returns (perm, NodeGroups).
    order "reference": the reference's greedy breadth-first colouring (the
    same groups as the reference); "device": colours from Jones-Plassmann
    rounds on the GPU (a different relocation order)."""
    nv = raw.nv
    perm = np.zeros(nv, np.uint32)
    gb = np.zeros(nv + 1, np.uint32)
    members = np.zeros(nv, np.uint32)
    ranges = np.zeros(6 * nv, np.uint32)
    ng = ctypes.c_uint32(0)
    L = N.lib()
    fn = {"reference": L.gm_node_groups_build, "device": L.gm_node_groups_build_device}[order]
    N.check(fn(nv, N.ptr(raw.cid), raw.tets.shape[0], N.ptr(raw.tets), raw.pris.shape[0], N.ptr(raw.pris),
               raw.hexs.shape[0], N.ptr(raw.hexs), int(permute), N.ptr(perm), N.ptr(gb), N.ptr(members),
               N.ptr(ranges), ctypes.byref(ng)))
    g = ng.value
    return perm, NodeGroups(gb[:g + 1].copy(), members[:gb[g]].copy(), ranges[:6 * g].copy())


def launch_count() -> int:
    """Kernel launches this library has made in this process (gm_launch_count)."""
    c = ctypes.c_uint64(0)
    N.check(N.lib().gm_launch_count(ctypes.byref(c)))
    return int(c.value)


def neighbourhoods(raw: RawMesh):
    """(ve_off, ve, vv_off, vv): the vertex neighbourhoods the library builds
    for an upload (Mesh::compileNeighborhoods order, input indices)."""
    L = N.lib()
    t, r, h = (np.ascontiguousarray(a, np.uint32) for a in (raw.tets, raw.pris, raw.hexs))
    el, vl = ctypes.c_uint64(0), ctypes.c_uint64(0)
    args = (raw.nv, t.shape[0], N.ptr(t), r.shape[0], N.ptr(r), h.shape[0], N.ptr(h))
    N.check(L.gm_mesh_neighbourhoods(*args, None, None, ctypes.byref(el), None, None, ctypes.byref(vl)))
    eo, vo = np.zeros(raw.nv + 1, np.uint32), np.zeros(raw.nv + 1, np.uint32)
    e, v = np.zeros(el.value, np.uint32), np.zeros(vl.value, np.uint32)
    N.check(L.gm_mesh_neighbourhoods(*args, N.ptr(eo), N.ptr(e), ctypes.byref(el), N.ptr(vo), N.ptr(v),
                                     ctypes.byref(vl)))
    return eo, e, vo, v


def permute_mesh(raw: RawMesh, perm: np.ndarray) -> RawMesh:
    """Apply a vertex permutation (new index -> old index) like NodeGroups::clusterNodes."""
    new_of_old = np.empty_like(perm)
    new_of_old[perm] = np.arange(perm.size, dtype=perm.dtype)
    return RawMesh(pos=np.ascontiguousarray(raw.pos[perm]), tets=new_of_old[raw.tets].astype(np.uint32),
                   pris=new_of_old[raw.pris].astype(np.uint32), hexs=new_of_old[raw.hexs].astype(np.uint32),
                   cid=np.ascontiguousarray(raw.cid[perm]), con_kind=raw.con_kind, con_param=raw.con_param,
                   name=raw.name, h=raw.h)


class DeviceMesh:
    """A gm_mesh handle: the mesh resident in HBM."""

    def __init__(self, raw: RawMesh | None, groups: NodeGroups | None = None, stream: int | None = None,
                 clone_of: "DeviceMesh | None" = None):
        L = N.lib()
        h = ctypes.c_void_p()
        N.check(L.gm_mesh_create(ctypes.byref(h)))
        self.h = h
        if clone_of is not None:
            if stream is not None:
                N.check(L.gm_mesh_set_stream(self.h, ctypes.c_void_p(stream)))
            N.check(L.gm_mesh_clone(self.h, clone_of.h))
            self.nv = clone_of.nv
            return
        self.nv = raw.nv
        if stream is not None:
            N.check(L.gm_mesh_set_stream(self.h, ctypes.c_void_p(stream)))
        N.check(L.gm_mesh_upload(self.h, raw.nv, N.ptr(raw.pos), N.ptr(raw.cid), raw.tets.shape[0], N.ptr(raw.tets),
                                 raw.pris.shape[0], N.ptr(raw.pris), raw.hexs.shape[0], N.ptr(raw.hexs)))
        ck = np.ascontiguousarray(raw.con_kind, np.int32)
        cp = np.ascontiguousarray(raw.con_param, np.float64)
        N.check(L.gm_mesh_set_constraints(self.h, ck.size, N.ptr(ck), N.ptr(cp)))
        if groups is not None:
            self.set_groups(groups)

    def set_groups(self, groups: NodeGroups):
        gb = np.ascontiguousarray(groups.group_base, np.uint32)
        mb = np.ascontiguousarray(groups.members, np.uint32)
        N.check(N.lib().gm_mesh_upload_groups(self.h, mb.size, N.ptr(mb), gb.size - 1, N.ptr(gb)))

    def set_crew(self, sampler: str, measurer: str, evaluator: str, scaling=1.0, aspect_ratio=1.0):
        N.check(N.lib().gm_mesh_set_crew(self.h, N.SAMPLERS[sampler], N.MEASURERS[measurer],
                                         N.EVALUATORS[evaluator], float(scaling), float(aspect_ratio)))

    def build_local_background(self):
        """The local sampler's background from the resident mesh (the crew's
        scaling and aspect ratio)."""
        N.check(N.lib().gm_mesh_build_local_background(self.h))

    def set_discretization_depth(self, depth: int):
        N.check(N.lib().gm_mesh_set_discretization_depth(self.h, int(depth)))

    def set_kd_nodes(self, children2: np.ndarray, separators4: np.ndarray, metrics6: np.ndarray):
        """kd-tree nodes in pre-order: children (-1: none), separator plane
        (normal, offset), metric (xx yy zz xy xz yz)."""
        c = np.ascontiguousarray(children2, np.int32).reshape(-1, 2)
        sp = np.ascontiguousarray(separators4, np.float64).reshape(-1, 4)
        m = np.ascontiguousarray(metrics6, np.float64).reshape(-1, 6)
        if not (c.shape[0] == sp.shape[0] == m.shape[0]):
            raise ValueError("one separator and one metric per node")
        N.check(N.lib().gm_mesh_set_kd_nodes(self.h, c.shape[0], N.ptr(c), N.ptr(sp), N.ptr(m)))

    def set_texture(self, dims, lo, extents, metrics6: np.ndarray):
        """Metric samples at the cell centres of a dims grid over
        [lo, lo + extents], x fastest."""
        d = np.ascontiguousarray(dims, np.int32).reshape(3)
        a = np.ascontiguousarray(lo, np.float64).reshape(3)
        e = np.ascontiguousarray(extents, np.float64).reshape(3)
        m = np.ascontiguousarray(metrics6, np.float64).reshape(-1, 6)
        if m.shape[0] != int(np.prod(d)):
            raise ValueError("one metric per texture cell")
        N.check(N.lib().gm_mesh_set_texture(self.h, N.ptr(d), N.ptr(a), N.ptr(e), N.ptr(m)))

    def set_local_background(self, tets8: np.ndarray, verts: np.ndarray, metrics6: np.ndarray):
        """A background given as the reference's GpuLocalTet records (4
        vertices, 4 face neighbours), vertex positions and symmetric vertex
        metrics (xx yy zz xy xz yz)."""
        t = np.ascontiguousarray(tets8, np.uint32).reshape(-1, 8)
        p = np.ascontiguousarray(verts, np.float64).reshape(-1, 3)
        m = np.ascontiguousarray(metrics6, np.float64).reshape(-1, 6)
        if m.shape[0] != p.shape[0]:
            raise ValueError("one metric per background vertex")
        N.check(N.lib().gm_mesh_set_local_background(self.h, t.shape[0], N.ptr(t), p.shape[0], N.ptr(p), N.ptr(m)))

    def set_stream(self, stream: int):
        N.check(N.lib().gm_mesh_set_stream(self.h, ctypes.c_void_p(stream)))

    def upload_positions(self, pos: np.ndarray):
        p = np.ascontiguousarray(pos, np.float64)
        N.check(N.lib().gm_mesh_upload_verts(self.h, self.nv, N.ptr(p)))

    def fetch_positions(self) -> np.ndarray:
        out = np.empty((self.nv, 3), np.float64)
        N.check(N.lib().gm_mesh_fetch_verts(self.h, self.nv, N.ptr(out)))
        return out

    def evaluate(self) -> QualityHistogram:
        q = N.Quality()
        N.check(N.lib().gm_evaluate(self.h, ctypes.byref(q)))
        return QualityHistogram.from_native(q)

    def evaluate_async(self, slot: int):
        N.check(N.lib().gm_evaluate_async(self.h, slot))

    def read_quality(self, slot: int) -> QualityHistogram:
        q = N.Quality()
        N.check(N.lib().gm_quality_read(self.h, slot, ctypes.byref(q)))
        return QualityHistogram.from_native(q)

    def smooth_pass(self, smoother: str, params=None):
        p = N.params_array(params)
        N.check(N.lib().gm_smooth_pass(self.h, N.SMOOTHERS[smoother], N.ptr(p)))

    def smooth_group(self, smoother: str, base: int, count: int, params=None):
        p = N.params_array(params)
        N.check(N.lib().gm_smooth_group(self.h, N.SMOOTHERS[smoother], N.ptr(p), base, count))

    def sync(self):
        N.check(N.lib().gm_mesh_sync(self.h))

    def device_bytes(self) -> int:
        b = ctypes.c_uint64()
        N.check(N.lib().gm_mesh_device_bytes(self.h, ctypes.byref(b)))
        return int(b.value)

    # device-resident job: the whole stop-rule schedule as one graph launch
    def job_prepare(self, smoother: str, params=None, max_passes: int = 20, min_gain: float = 1e-3):
        p = N.params_array(params)
        N.check(N.lib().gm_job_prepare(self.h, N.SMOOTHERS[smoother], N.ptr(p), int(max_passes), float(min_gain)))

    def job_launch(self):
        N.check(N.lib().gm_job_launch(self.h))

    def job_done(self) -> bool:
        d = ctypes.c_int32()
        N.check(N.lib().gm_job_query(self.h, ctypes.byref(d)))
        return bool(d.value)

    def job_result(self):
        """(passes run, quality before the first pass, quality after the last)"""
        n = ctypes.c_uint32()
        first, last = N.Quality(), N.Quality()
        N.check(N.lib().gm_job_result(self.h, ctypes.byref(n), ctypes.byref(first), ctypes.byref(last)))
        return int(n.value), QualityHistogram.from_native(first), QualityHistogram.from_native(last)

    def save_positions(self):
        N.check(N.lib().gm_mesh_save_positions(self.h))

    def restore_positions(self):
        N.check(N.lib().gm_mesh_restore_positions(self.h))

    def upload_gpu_verts(self, buf: np.ndarray):
        """positions in the reference's GpuVert layout (float x, y, z, uint c)"""
        N.check(N.lib().gm_mesh_upload_gpu_verts(self.h, self.nv, N.ptr(buf)))

    def upload_gpu_verts_async(self, buf: np.ndarray):
        """GpuVert positions from pinned host memory, asynchronous on the mesh's
        stream: keep `buf` unchanged until the stream has passed the copy"""
        N.check(N.lib().gm_mesh_upload_gpu_verts_async(self.h, self.nv, N.ptr(buf)))

    def fetch_gpu_verts(self, buf: np.ndarray):
        N.check(N.lib().gm_mesh_fetch_gpu_verts(self.h, self.nv, N.ptr(buf)))

    def counters(self, reset: bool = False) -> dict:
        out = np.zeros(5, np.uint64)
        N.check(N.lib().gm_mesh_counters(self.h, N.ptr(out), int(reset)))
        return {"patch_evals": int(out[0]), "elem_evals": int(out[1] + out[2] + out[3]),
                "fp64_vertices": int(out[4])}

    def close(self):
        if getattr(self, "h", None):
            N.lib().gm_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """DataStructures/Mesh.h: vertices, elements and their constraints.

    compileTopology() builds the neighbourhoods and the NodeGroups and
    permutes the vertices exactly as Mesh::compileTopology does; after it the
    mesh can be uploaded with updateCudaTopology()/updateCudaVertices()."""

    def __init__(self, raw: RawMesh):
        self.raw = raw
        self.modelName = raw.name
        self._groups: NodeGroups | None = None
        self._device: DeviceMesh | None = None
        self.perm = np.arange(raw.nv, dtype=np.uint32)

    @property
    def verts(self) -> np.ndarray:
        return self.raw.pos

    @verts.setter
    def verts(self, value):
        self.raw.pos = np.ascontiguousarray(value, np.float64)

    @classmethod
    def fromJson(cls, path: str) -> "Mesh":
        """A mesh file in the reference tool's JSON layout (JsonDeserializer)."""
        from .meshio import read_json

        return cls(read_json(path))

    def toJson(self, path: str, precision: str = "exact"):
        """Write the mesh in the reference tool's JSON layout (JsonSerializer)."""
        from .meshio import write_json

        write_json(path, self.raw, model=self.modelName, precision=precision)

    def compileTopology(self):
        perm, groups = node_groups_build(self.raw, permute=True)
        self.raw = permute_mesh(self.raw, perm)
        self.perm = self.perm[perm]
        # the group lists refer to the new order already
        self._groups = groups
        self._device = None

    def nodeGroups(self) -> NodeGroups:
        if self._groups is None:
            raise RuntimeError("compileTopology() first")
        return self._groups

    def device(self) -> DeviceMesh:
        if self._device is None:
            self._device = DeviceMesh(self.raw, self._groups)
        return self._device

    def updateCudaTopology(self):
        self._device = DeviceMesh(self.raw, self._groups)

    def updateCudaVertices(self):
        self.device().upload_positions(self.raw.pos)

    def fetchCudaVertices(self):
        self.raw.pos = self.device().fetch_positions()

    def clearCudaMemory(self):
        if self._device is not None:
            self._device.close()
            self._device = None


class MeshCrew:
    """DataStructures/MeshCrew.cpp: the sampler picks the measurer (:93-103)."""

    def __init__(self):
        self._sampler = UniformSampler()
        self._measurer = MetricFreeMeasurer()
        self._evaluator = None

    def sampler(self):
        return self._sampler

    def measurer(self):
        return self._measurer

    def evaluator(self):
        return self._evaluator

    def setSampler(self, mesh, sampler: AbstractSampler):
        self._sampler = sampler
        self._measurer = MetricWiseMeasurer() if sampler.isMetricWise() else MetricFreeMeasurer()

    def setEvaluator(self, mesh, evaluator):
        self._evaluator = evaluator

    def install(self, dev: DeviceMesh):
        dev.set_discretization_depth(self._sampler.discretizationDepth())
        dev.set_crew(self._sampler.kind, self._measurer.kind, self._evaluator.kind,
                     self._sampler.scaling(), self._sampler.aspectRatio())


# ---------------------------------------------------------------------------
# evaluators
# ---------------------------------------------------------------------------
class AbstractEvaluator:
    kind = "mean_ratio"

    def evaluateMesh(self, mesh: Mesh, sampler, measurer, histogram: QualityHistogram,
                     implementationName: str = CUDA_IMPL_NAME):
        """AbstractEvaluator::evaluateMesh (Evaluators/AbstractEvaluator.cpp:340-382):
        an unknown implementation name leaves a NaN histogram."""
        histogram.clear()
        if implementationName != CUDA_IMPL_NAME:
            histogram.setMinimumQuality(float("nan"))
            histogram.setInvQualitySum(float("nan"))
            return
        self.evaluateMeshQualityCuda(mesh, sampler, measurer, histogram)

    def evaluateMeshQualityCuda(self, mesh: Mesh, sampler, measurer, histogram: QualityHistogram):
        dev = mesh.device()
        dev.set_discretization_depth(sampler.discretizationDepth())
        dev.set_crew(sampler.kind, measurer.kind, self.kind, sampler.scaling(), sampler.aspectRatio())
        h = dev.evaluate()
        histogram.__dict__.update(h.__dict__)


class MeanRatioEvaluator(AbstractEvaluator):
    kind = "mean_ratio"


class MetricConformityEvaluator(AbstractEvaluator):
    kind = "metric_conformity"


# ---------------------------------------------------------------------------
# smoothers
# ---------------------------------------------------------------------------
class AbstractSmoother:
    """Smoothers/AbstractSmoother.cpp: pass control with an evaluation before
    and after every pass (evaluateMeshQuality, :103-211)."""

    kind = "nelder_mead"
    element_wise = False

    def __init__(self, params=None):
        self.params = params
        self.passes: list[OptimizationPass] = []

    def smoothMesh(self, mesh: Mesh, crew: MeshCrew, implementationName: str = CUDA_IMPL_NAME,
                   schedule: Schedule | None = None):
        if implementationName != CUDA_IMPL_NAME:
            warnings.warn(f"'{implementationName}' is not a valid option for 'Smoothing Implementations'")
            return
        schedule = schedule or Schedule()
        if schedule.topoOperationEnabled:
            raise NotImplementedError("topology operations are not part of this library")
        dev = mesh.device()
        crew.install(dev)
        self.passes = []
        t0 = time.perf_counter()
        last = dev.evaluate()
        self.passes.append(OptimizationPass(0.0, last))
        # vertex-wise: INITIAL evaluation then relocationPassCount passes;
        # element-wise starts its pass counter at 0 (AbstractElementWiseSmoother.cpp:53-83)
        reloc = 0
        while True:
            if schedule.autoPilotEnabled and reloc > 0:
                prev = self.passes[-2].histogram
                cur = self.passes[-1].histogram
                go = (cur.harmonicMean() - prev.harmonicMean() > schedule.minQualThreshold) or \
                     (cur.minimumQuality() - prev.minimumQuality() > schedule.qualMeanThreshold)
            else:
                go = reloc < schedule.relocationPassCount
            if not go:
                break
            dev.smooth_pass(self.kind, self.params)
            h = dev.evaluate()
            self.passes.append(OptimizationPass(time.perf_counter() - t0, h))
            reloc += 1
        mesh.fetchCudaVertices()


class NelderMeadSmoother(AbstractSmoother):
    kind = "nelder_mead"


class GradientDescentSmoother(AbstractSmoother):
    kind = "gradient_descent"


class SpawnSearchSmoother(AbstractSmoother):
    kind = "spawn_search"


class GetmeSmoother(AbstractSmoother):
    kind = "getme"
    element_wise = True


class SpringLaplaceSmoother(AbstractSmoother):
    kind = "spring_laplace"


class QualityLaplaceSmoother(AbstractSmoother):
    kind = "quality_laplace"


# The reference's multi-thread-per-vertex smoothers run Nelder-Mead and
# gradient descent with the parameters their CUDA drivers install; their
# kernels spread one patch's elements (or sample positions) over several
# threads, a decomposition the warp-per-vertex kernels here already make.
class MultiElemNMSmoother(NelderMeadSmoother):
    """Smoothers/VertexWise/MultiElemNMSmoother.cpp: Nelder-Mead with the
    constants of :7-13, those of NelderMeadSmoother."""


class MultiElemGradDsntSmoother(GradientDescentSmoother):
    """Smoothers/VertexWise/MultiElemGradDsntSmoother.cpp: gradient descent
    with the constants its CUDA driver installs (:7-8): 5 cycles, node shift
    local size / 25."""

    def __init__(self, params=None):
        super().__init__(params if params is not None else [1.0 / 25.0, 5])


class MultiPosGradDsntSmoother(MultiElemGradDsntSmoother):
    """Smoothers/VertexWise/MultiPosGradDsntSmoother.cpp (:7-8, the same
    constants)."""


class PatchGradDsntSmoother(MultiElemGradDsntSmoother):
    """Smoothers/VertexWise/PatchGradDsntSmoother.cpp (:7-8, the same
    constants)."""


SMOOTHER_CLASSES = {"nelder_mead": NelderMeadSmoother, "gradient_descent": GradientDescentSmoother,
                    "spawn_search": SpawnSearchSmoother, "getme": GetmeSmoother,
                    "spring_laplace": SpringLaplaceSmoother, "quality_laplace": QualityLaplaceSmoother}


class Batch:
    """gm_batch: many resident meshes relocated by one persistent launch per pass."""

    def __init__(self, devices: list):
        self.devices = list(devices)  # keeps the meshes alive
        arr = (ctypes.c_void_p * len(self.devices))(*[d.h.value if hasattr(d.h, "value") else d.h
                                                      for d in self.devices])
        h = ctypes.c_void_p()
        N.check(N.lib().gm_batch_create(ctypes.byref(h), ctypes.cast(arr, ctypes.c_void_p), len(self.devices)))
        self.h = h
        s = ctypes.c_void_p()
        N.check(N.lib().gm_batch_stream(self.h, ctypes.byref(s)))
        self.stream = s.value or 0

    def info(self) -> dict:
        out = np.zeros(4, np.uint32)
        N.check(N.lib().gm_batch_info(self.h, N.ptr(out)))
        return {"meshes": int(out[0]), "vertices": int(out[1]), "segments": int(out[2]), "eval_blocks": int(out[3])}

    def latencies_ms(self) -> np.ndarray:
        out = np.zeros(len(self.devices), np.float64)
        N.check(N.lib().gm_batch_latencies(self.h, N.ptr(out)))
        return out

    def set_config(self, warps_per_block: int, ctas_per_sm: int = 0):
        N.check(N.lib().gm_batch_set_config(self.h, warps_per_block, ctas_per_sm))

    def tune(self, smoother: str, params=None):
        w, c, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        p = N.params_array(params)
        N.check(N.lib().gm_batch_tune(self.h, N.SMOOTHERS[smoother], N.ptr(p), ctypes.byref(w), ctypes.byref(c),
                                      ctypes.byref(ms)))
        return w.value, c.value, ms.value

    def smooth_pass(self, smoother: str, params=None):
        p = N.params_array(params)
        N.check(N.lib().gm_batch_smooth_pass(self.h, N.SMOOTHERS[smoother], N.ptr(p)))

    def evaluate(self, slot: int = 0):
        N.check(N.lib().gm_batch_evaluate(self.h, slot))

    def read_quality(self, slot: int = 0):
        n = len(self.devices)
        arr = (N.Quality * n)()
        N.check(N.lib().gm_batch_read_quality(self.h, slot, ctypes.cast(arr, ctypes.c_void_p)))
        return [QualityHistogram.from_native(q) for q in arr]

    def capture(self, smoother: str, params=None, eval_slot: int = -1):
        p = N.params_array(params)
        N.check(N.lib().gm_batch_capture_pass(self.h, N.SMOOTHERS[smoother], N.ptr(p), eval_slot))

    def replay(self):
        N.check(N.lib().gm_batch_replay(self.h))

    def sync(self):
        N.check(N.lib().gm_batch_sync(self.h))

    def status(self) -> int:
        return N.lib().gm_batch_status(self.h)

    def set_spin_limit(self, polls: int):
        N.check(N.lib().gm_batch_set_spin_limit(self.h, polls))

    def inject_stall(self, mesh: int):
        N.check(N.lib().gm_batch_inject_stall(self.h, mesh))

    def counters(self, reset=False) -> dict:
        out = np.zeros(5, np.uint64)
        N.check(N.lib().gm_batch_counters(self.h, N.ptr(out), int(reset)))
        return {"patch_evals": int(out[0]), "elem_evals": int(out[1] + out[2] + out[3]), "fp64_vertices": int(out[4])}

    def close(self):
        if getattr(self, "h", None):
            N.lib().gm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
