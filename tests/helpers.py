"""Shared helpers for the parity tests: build a workload mesh, colour it,
run the GPU path through the C ABI and the FP64 oracle on identical input."""

from __future__ import annotations

import numpy as np

from gpumesh_gb300 import mesh as M
from gpumesh_gb300 import meshgen

import pyoracle


def coloured(raw):
    perm, groups = M.node_groups_build(raw)
    return M.permute_mesh(raw, perm), groups


def oracle_for(raw, crew):
    return pyoracle.OracleMesh.from_raw(raw, **crew)


def device_for(raw, groups, crew):
    dev = M.DeviceMesh(raw, groups)
    dev.set_crew(crew["sampler"], crew["measurer"], crew["evaluator"], crew.get("scaling", 1.0),
                 crew.get("aspect_ratio", 1.0))
    return dev


TET_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))
PRI_EDGES = ((0, 1), (0, 2), (1, 2), (0, 3), (1, 4), (2, 5), (3, 4), (3, 5), (4, 5))
HEX_EDGES = ((0, 1), (0, 3), (1, 2), (2, 3), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (4, 7), (5, 6), (6, 7))


def edge_lengths(raw):
    """Mean edge length around each vertex (the local element size)."""
    pairs = []
    for E, edges in ((raw.tets, TET_EDGES), (raw.pris, PRI_EDGES), (raw.hexs, HEX_EDGES)):
        if E.shape[0]:
            for a, b in edges:
                pairs.append(np.stack([E[:, a], E[:, b]], axis=1))
    e = np.unique(np.sort(np.concatenate(pairs).astype(np.int64), axis=1), axis=0)
    L = np.linalg.norm(raw.pos[e[:, 0]] - raw.pos[e[:, 1]], axis=1)
    s = np.zeros(raw.nv)
    c = np.zeros(raw.nv)
    np.add.at(s, e[:, 0], L)
    np.add.at(s, e[:, 1], L)
    np.add.at(c, e[:, 0], 1)
    np.add.at(c, e[:, 1], 1)
    return s / np.maximum(c, 1)


def fp32_outcomes(raw, groups, crew, schedule, draws=4):
    """The FP64 oracle's final evaluation from the GPU's input, then its runs
    at FP32 resolution: patch qualities rounded to FP32, and `draws` seeded
    (1 + u 2^-23) draws (the q32 measurement build)."""
    out = []
    for variant, seed in [("", 0)] + [("q32", s) for s in range(draws + 1)]:
        if variant:
            pyoracle.set_fp32_resolution_seed(seed)
        orc = pyoracle.OracleMesh.from_raw(raw, **crew, variant=variant)
        orc.pos = raw.pos.astype(np.float32).astype(np.float64)
        for smoother, passes, params in schedule:
            for _ in range(passes):
                orc.smooth_pass(smoother, groups.group_base, groups.members, params=params, nthreads=4)
        chk = oracle_for(raw, crew)
        chk.pos = orc.pos
        out.append(chk.evaluate())
    return out


def within_fp32_resolution(gpu, fp64, draws):
    """Within 1e-4 of the FP64 result, of one of its FP32-resolution
    outcomes, or within twice the outcomes' spread around the FP64 result."""
    draws = np.asarray(draws, np.float64)
    if abs(gpu - fp64) <= 1e-4 or np.min(np.abs(draws - gpu)) <= 1e-4:
        return True
    return abs(gpu - fp64) <= 2 * float(np.max(np.abs(draws - fp64)))
