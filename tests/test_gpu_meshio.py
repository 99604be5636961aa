"""A mesh read from a JSON file written by the reference's own serializer
goes through the GPU path: evaluation and a relocation pass against the FP64
oracle on the same input."""

import os

import numpy as np
import pytest

from gpumesh_gb300 import meshio, workloads
from gpumesh_gb300 import mesh as M

from helpers import coloured, device_for, oracle_for

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MR = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")


def test_reference_json_mesh_on_the_gpu():
    raw, groups = coloured(meshio.read_json(os.path.join(HERE, "golden", "tet_box_2_ref.json")))
    dev = device_for(raw, groups, MR)
    orc = oracle_for(raw, MR)
    g, o = dev.evaluate(), orc.evaluate()
    assert abs(g.minimumQuality() - o["min"]) <= 1e-6
    dev.smooth_pass("nelder_mead", workloads.NM_PARAMS)
    orc.smooth_pass("nelder_mead", groups.group_base, groups.members, params=workloads.NM_PARAMS)
    check = oracle_for(raw, MR)
    check.pos = dev.fetch_positions()
    assert abs(check.evaluate()["min"] - orc.evaluate()["min"]) <= 1e-4


def test_json_round_trip_through_the_host_mirror(tmp_path):
    from gpumesh_gb300 import meshgen

    m = M.Mesh(meshgen.box_mesh(4, "hex", 0.15, 2, gaussian=True))
    path = str(tmp_path / "hex.json")
    m.toJson(path)
    back = M.Mesh.fromJson(path)
    assert np.array_equal(back.raw.pos, m.raw.pos)
    back.compileTopology()
    dev = back.device()
    q = dev.evaluate()
    assert q.minimumQuality() <= 1.0
