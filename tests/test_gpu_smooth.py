"""GPU relocation against the FP64 oracle on the same coloured mesh, in the
same colour-major order.  Both final meshes are re-evaluated by the FP64
oracle evaluator; the gate is |delta min|, |delta harmonic mean| <= 1e-4.
Per-vertex position differences are reported relative to the local mean edge
length: FP32 rounding can flip a comparison inside a vertex's search, so a
few vertices may end at a different (equally good) position."""

import numpy as np
import pytest

from gpumesh_gb300 import meshgen, workloads

from helpers import coloured, device_for, edge_lengths, oracle_for

pytestmark = pytest.mark.gpu

TOL = 1e-4


def run_both(raw, groups, crew, schedule):
    dev = device_for(raw, groups, crew)
    orc = oracle_for(raw, crew)
    for smoother, passes, params in schedule:
        for _ in range(passes):
            dev.smooth_pass(smoother, params)
            orc.smooth_pass(smoother, groups.group_base, groups.members, params=params, nthreads=4)
    gpos = dev.fetch_positions()
    check = oracle_for(raw, crew)
    check.pos = gpos
    return gpos, orc.pos, check.evaluate(), orc.evaluate(), dev


def assert_parity(raw, gq, oq, gpos, opos, tol=TOL):
    assert abs(gq["min"] - oq["min"]) <= tol, (gq["min"], oq["min"])
    if np.isfinite(oq["inv_sum"]) and np.isfinite(gq["inv_sum"]):
        assert abs(gq["mean"] - oq["mean"]) <= tol, (gq["mean"], oq["mean"])
    err = np.linalg.norm(gpos - opos, axis=1) / edge_lengths(raw)
    return err


def test_c1_nelder_mead_baseline_params():
    w = workloads.WORKLOADS["C1"]
    raw, groups = coloured(w.mesh())
    gpos, opos, gq, oq, dev = run_both(raw, groups, w.crew(raw), w.schedule)
    err = assert_parity(raw, gq, oq, gpos, opos)
    assert np.median(err) < 1e-3


def test_c1_nelder_mead_reference_params():
    raw, groups = coloured(meshgen.box_mesh(10, "tet", 0.3, 0))
    crew = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")
    gpos, opos, gq, oq, dev = run_both(raw, groups, crew, [("nelder_mead", 1, None)])
    assert_parity(raw, gq, oq, gpos, opos)


def test_gradient_descent_and_spawn_on_sphere_metric_conformity():
    raw, groups = coloured(meshgen.sphere_mesh(16, 0.25, 1))
    crew = dict(sampler="sine", measurer="metric_wise", evaluator="metric_conformity", scaling=1.0 / raw.h)
    sched = [("gradient_descent", 2, workloads.GD_PARAMS), ("spawn_search", 2, workloads.SPAWN_PARAMS)]
    gpos, opos, gq, oq, dev = run_both(raw, groups, crew, sched)
    # all sphere boundary vertices stay on the sphere
    b = raw.cid == 1
    assert np.abs(np.linalg.norm(gpos[b], axis=1) - 1.0).max() < 1e-5
    assert_parity(raw, gq, oq, gpos, opos, tol=1e-3)


def test_getme_hex():
    raw, groups = coloured(meshgen.box_mesh(12, "hex", 0.15, 2, gaussian=True))
    crew = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")
    gpos, opos, gq, oq, dev = run_both(raw, groups, crew, [("getme", 3, workloads.GETME_PARAMS)])
    err = assert_parity(raw, gq, oq, gpos, opos)
    assert err.max() < 1e-3


def test_getme_mixed():
    raw, groups = coloured(meshgen.box_mesh(9, "mixed", 0.15, 2, gaussian=True))
    crew = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")
    gpos, opos, gq, oq, dev = run_both(raw, groups, crew, [("getme", 2, [0.78])])
    assert_parity(raw, gq, oq, gpos, opos)


def test_box_constraints_hold():
    raw, groups = coloured(meshgen.box_mesh(8, "tet", 0.3, 4))
    crew = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")
    dev = device_for(raw, groups, crew)
    dev.smooth_pass("spawn_search", None)
    p = dev.fetch_positions()
    fixed = raw.cid < 0
    assert np.array_equal(p[fixed], raw.pos[fixed].astype(np.float32).astype(np.float64))
    for cid, axis, val in ((1, 0, -1), (2, 0, 1), (3, 1, -1), (4, 1, 1), (5, 2, -1), (6, 2, 1)):
        sel = raw.cid == cid
        assert np.abs(p[sel, axis] - val).max() < 1e-6


def test_quality_never_drops_per_pass():
    raw, groups = coloured(meshgen.box_mesh(10, "tet", 0.3, 0))
    crew = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")
    dev = device_for(raw, groups, crew)
    prev = dev.evaluate()
    for smoother in ("nelder_mead", "gradient_descent", "spawn_search"):
        dev.smooth_pass(smoother, None)
        cur = dev.evaluate()
        assert cur.harmonicMean() >= prev.harmonicMean() - 1e-6
        prev = cur
