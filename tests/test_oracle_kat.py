"""The oracle against the reference's only golden values: the regular-element
known-answer test of AbstractEvaluator::assessMeasureValidy
(Evaluators/AbstractEvaluator.cpp:281-338, VALIDITY_EPSILON = 1e-6)."""

import numpy as np
import pytest

import pyoracle

S3 = np.sqrt(3.0)
KAT_POS = np.array([[0, 0, 0], [1, 0, 0], [0.5, S3 / 2, 0], [0.5, S3 / 6, np.sqrt(2 / 3)],
                    [0, 0, 0], [0, 1, 0], [0, 0.5, S3 / 2], [1, 0, 0], [1, 1, 0], [1, 0.5, S3 / 2],
                    [0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                   dtype=np.float64)
KAT_TET = np.array([[0, 1, 2, 3]], np.uint32)
KAT_PRI = np.array([[4, 5, 6, 7, 8, 9]], np.uint32)
KAT_HEX = np.array([[10, 11, 12, 13, 14, 15, 16, 17]], np.uint32)


def kat_mesh(**crew):
    return pyoracle.OracleMesh(KAT_POS, KAT_TET, KAT_PRI, KAT_HEX, np.zeros(18, np.int32), [0],
                               np.zeros((1, 6)), **crew)


@pytest.mark.parametrize("evaluator", ["mean_ratio", "metric_conformity"])
@pytest.mark.parametrize("measurer", ["metric_free", "metric_wise"])
def test_regular_elements_have_quality_one(evaluator, measurer):
    # the reference runs this check with a UniformSampler + MetricWiseMeasurer
    # (GpuMeshCharacter.cpp:243-253); every crew must pass it
    m = kat_mesh(sampler="uniform", measurer=measurer, evaluator=evaluator)
    for etype in (0, 2, 3):
        assert abs(m.element_quality(etype, 0) - 1.0) < 1e-6


def test_mean_ratio_is_scale_invariant():
    for s in (0.1, 3.0):
        m = kat_mesh(sampler="uniform", measurer="metric_free", evaluator="mean_ratio", scaling=s)
        assert abs(m.element_quality(3, 0) - 1.0) < 1e-12


def test_inverted_tet_is_negative_and_histogram_rules():
    pos = KAT_POS[:4].copy()
    pos[3, 2] = -pos[3, 2]  # mirror the apex: inverted tet
    m = pyoracle.OracleMesh(pos, KAT_TET, np.zeros((0, 6)), np.zeros((0, 8)), np.zeros(4, np.int32), [0],
                            np.zeros((1, 6)))
    q = m.element_quality(0, 0)
    assert q < 0
    h = m.evaluate()
    # QualityHistogram::add: an element with q <= 0 makes the harmonic mean 0
    assert h["inv_sum"] == float("inf") and h["mean"] == 0.0
    assert h["min"] == q and h["buckets"][0] == 1


def test_uniform_metric_and_distances():
    m = kat_mesh(sampler="uniform", measurer="metric_wise", evaluator="mean_ratio", scaling=2.0)
    M = m.metric_at([0.3, 0.2, 0.1])
    assert np.allclose(M, 4.0 * np.eye(3))
    d = m.riemannian_distance if hasattr(m, "riemannian_distance") else None
    a, b = np.array([0.0, 0, 0]), np.array([1.0, 2, 2])
    import ctypes
    lib = pyoracle.lib()
    dist = lib.om_riemannian_distance(m.h, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p))
    assert abs(dist - 6.0) < 1e-12
