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


def edge_lengths(raw):
    """Mean edge length around each vertex (the local element size)."""
    edges = set()
    for t in raw.tets:
        for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)):
            edges.add((min(t[a], t[b]), max(t[a], t[b])))
    e = np.array(sorted(edges), dtype=np.int64)
    L = np.linalg.norm(raw.pos[e[:, 0]] - raw.pos[e[:, 1]], axis=1)
    s = np.zeros(raw.nv)
    c = np.zeros(raw.nv)
    np.add.at(s, e[:, 0], L)
    np.add.at(s, e[:, 1], L)
    np.add.at(c, e[:, 0], 1)
    np.add.at(c, e[:, 1], 1)
    return s / np.maximum(c, 1)
