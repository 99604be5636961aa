"""gm_evaluate_noalloc: quality evaluation for callers that cannot allocate
device memory (a framework that owns every device buffer, a fully committed
memory budget, a loop that must not allocate).  The test allocates the
mesh's device buffers itself, as such a caller's framework would, calls the
entry point twice in a row through the C ABI, and compares each result with
gm_evaluate on the same mesh.  Collected last on purpose."""

import ctypes

import numpy as np
import pytest

from gpumesh_gb300 import _native as N
from gpumesh_gb300 import mesh as M
from gpumesh_gb300 import meshgen

pytestmark = pytest.mark.gpu


def device_inputs(torch, raw):
    pos = np.zeros((raw.nv, 4), np.float32)
    pos[:, :3] = raw.pos
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()
    return (t(pos, np.float32), t(raw.tets.view(np.int32), np.int32), t(raw.pris.view(np.int32), np.int32),
            t(raw.hexs.view(np.int32), np.int32))


def noalloc(torch, raw, crew, out):
    pos, tets, pris, hexs = device_inputs(torch, raw)
    st = N.lib().gm_evaluate_noalloc(raw.nv, pos.data_ptr(), raw.tets.shape[0], tets.data_ptr() or None,
                                     raw.pris.shape[0], pris.data_ptr() or None, raw.hexs.shape[0],
                                     hexs.data_ptr() or None, N.SAMPLERS[crew["sampler"]],
                                     N.MEASURERS[crew["measurer"]], N.EVALUATORS[crew["evaluator"]],
                                     float(crew.get("scaling", 1.0)), float(crew.get("aspect_ratio", 1.0)),
                                     out.data_ptr(), None)
    N.check(st)
    torch.cuda.synchronize()
    q = N.Quality.from_buffer_copy(out.cpu().numpy().tobytes())
    return M.QualityHistogram.from_native(q)


# every kernel variant the entry point selects: the tet and hex-only
# mean-ratio streams, mixed meshes under the diagonal (sine) and the general
# (analytic) metric, the metric-wise mean ratio, and a mesh of more than
# 1024 x 256 elements, whose grid is the one-wave cap rather than one block
# per 256 elements
CASES = {
    "tet": (lambda: meshgen.box_mesh(12, "tet", 0.3, 0),
            dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")),
    "hex": (lambda: meshgen.box_mesh(10, "hex", 0.15, 2, gaussian=True),
            dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")),
    "mixed_mc": (lambda: meshgen.box_mesh(7, "mixed", 0.15, 2, gaussian=True),
                 dict(sampler="sine", measurer="metric_wise", evaluator="metric_conformity", scaling=3.0)),
    "mixed_mc_analytic": (lambda: meshgen.box_mesh(6, "mixed", 0.1, 5),
                          dict(sampler="analytic", measurer="metric_wise", evaluator="metric_conformity",
                               scaling=2.0, aspect_ratio=3.0)),
    "mixed_mr_wise": (lambda: meshgen.box_mesh(6, "mixed", 0.1, 5),
                      dict(sampler="analytic", measurer="metric_wise", evaluator="mean_ratio", scaling=2.0,
                           aspect_ratio=3.0)),
    "tet_large": (lambda: meshgen.box_mesh(40, "tet", 0.3, 1),
                  dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")),
}


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_gm_evaluate_twice(case):
    torch = pytest.importorskip("torch")
    build, crew = CASES[case]
    raw = build()
    dev = M.DeviceMesh(raw, None)
    dev.set_crew(crew["sampler"], crew["measurer"], crew["evaluator"], crew.get("scaling", 1.0),
                 crew.get("aspect_ratio", 1.0))
    ref = dev.evaluate()
    out = torch.zeros(ctypes.sizeof(N.Quality), dtype=torch.uint8, device="cuda")
    for _ in range(2):
        h = noalloc(torch, raw, crew, out)
        assert h.sampleCount() == ref.sampleCount()
        assert h.minimumQuality() == ref.minimumQuality()
        assert (h.buckets() == ref.buckets()).all()
        if np.isfinite(ref.invQualitySum()):
            assert abs(h.invQualitySum() - ref.invQualitySum()) <= 1e-6 * ref.invQualitySum()
        else:
            assert not np.isfinite(h.invQualitySum())


def test_noalloc_rejects_meshes_above_its_limit():
    torch = pytest.importorskip("torch")
    raw = meshgen.box_mesh(2, "tet", 0.0, 0)
    pos, tets, pris, hexs = device_inputs(torch, raw)
    out = torch.zeros(ctypes.sizeof(N.Quality), dtype=torch.uint8, device="cuda")
    st = N.lib().gm_evaluate_noalloc(raw.nv, pos.data_ptr(), 1 << 24, tets.data_ptr(), 1, tets.data_ptr(), 0, None,
                                     0, 0, 0, 1.0, 1.0, out.data_ptr(), None)
    assert st == 4
    assert b"at most 16777216 elements" in N.lib().gm_last_error()


def test_noalloc_rejects_the_background_samplers():
    # a background mesh, kd-tree or texture lives with a resident mesh
    torch = pytest.importorskip("torch")
    raw = meshgen.box_mesh(2, "tet", 0.0, 0)
    pos, tets, pris, hexs = device_inputs(torch, raw)
    out = torch.zeros(ctypes.sizeof(N.Quality), dtype=torch.uint8, device="cuda")
    for name in ("local", "kdtree", "texture"):
        st = N.lib().gm_evaluate_noalloc(raw.nv, pos.data_ptr(), raw.tets.shape[0], tets.data_ptr(), 0, None, 0,
                                         None, N.SAMPLERS[name], 1, 1, 1.0, 1.0, out.data_ptr(), None)
        assert st == 4
        assert b"need a resident mesh" in N.lib().gm_last_error()
