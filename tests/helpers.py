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
