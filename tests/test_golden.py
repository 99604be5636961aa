"""The FP64 oracle against golden vectors produced by the reference's own
CPU code (tests/golden/make_golden.py): evaluation and one pass of each
smoother on small seeded meshes, and both the oracle's and the product's
NodeGroups against the reference's permutation and colour groups.  Runs
without the reference tree."""

import glob
import os

import numpy as np
import pytest

import pyoracle
from gpumesh_gb300 import mesh as M
from gpumesh_gb300 import meshgen

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load(path):
    d = dict(np.load(path, allow_pickle=False))
    raw = meshgen.RawMesh(pos=d["pos"], tets=d["tets"], pris=d["pris"], hexs=d["hexs"], cid=d["cid"],
                          con_kind=d["con_kind"], con_param=d["con_param"])
    return d, raw


def oracle(d, raw):
    perm = d["perm"]
    pr = M.permute_mesh(raw, perm)
    sampler = str(d["sampler"])
    measurer = "metric_free" if sampler == "uniform" else "metric_wise"
    return pr, pyoracle.OracleMesh.from_raw(pr, sampler=sampler, measurer=measurer, evaluator=str(d["evaluator"]),
                                            scaling=float(d["scaling"]),
                                            aspect_ratio=float(d.get("aspect_ratio", 1.0)),
                                            depth=int(d.get("depth", -1)))


def test_fixtures_exist():
    assert len(FIXTURES) >= 3


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_node_groups_match_golden(path):
    d, raw = load(path)
    perm, groups = M.node_groups_build(raw)
    assert np.array_equal(perm, d["perm"])
    assert np.array_equal(groups.group_base, d["group_base"])
    assert np.array_equal(groups.members, d["members"])


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_node_groups_match_golden(path):
    d, raw = load(path)
    perm, base, members, ranges = pyoracle.node_groups_build(raw)
    assert np.array_equal(perm, d["perm"])
    assert np.array_equal(base, d["group_base"])
    assert np.array_equal(members, d["members"])


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_evaluation_matches_golden(path):
    d, raw = load(path)
    pr, orc = oracle(d, raw)
    e = orc.evaluate()
    assert e["count"] == int(d["eval_count"])
    assert abs(e["min"] - float(d["eval_min"])) <= 1e-12
    if np.isfinite(float(d["eval_inv_sum"])):
        assert abs(e["inv_sum"] - float(d["eval_inv_sum"])) <= 1e-12 * float(d["eval_inv_sum"])
        assert np.array_equal(e["buckets"], d["eval_buckets"])


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
@pytest.mark.parametrize("smoother", ["nelder_mead", "gradient_descent", "spawn_search", "getme", "spring_laplace",
                                      "quality_laplace"])
def test_smoothers_match_golden(path, smoother):
    d, raw = load(path)
    pr, orc = oracle(d, raw)
    orc.smooth_pass(smoother, d["group_base"], d["members"])
    assert np.allclose(orc.pos, d["after_" + smoother], rtol=0, atol=1e-12)
