"""Seeded synthetic meshes for the smoothing and evaluation workloads.

All randomness comes from a counter-based generator (splitmix64 finaliser of
seed, stream and index, 53-bit uniforms), so the same seed gives the same mesh
on any machine and in any process.  Box meshes live on [-1, 1]^3 with the
vertex classification of the reference's debug hex grid
(Meshers/DebugMesher.cpp:167-300) and the constraint ids of BoxBoundary
(Boundaries/BoxBoundary.cpp:4-38); the sphere mesh uses SphereBoundary's single
face constraint (Boundaries/SphereBoundary.cpp:37-45).

A mesh is returned as a :class:`RawMesh`: float64 positions, uint32
connectivity per element type, and one int32 constraint id per vertex
(< 0 fixed, 0 free, > 0 boundary constraint), plus the constraint table.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

# constraint kinds (shared with the C ABI)
CON_VOLUME = 0
CON_PLANE = 1
CON_SEGMENT = 2
CON_SPHERE = 3
CON_POINT = 4
CON_SHELL_INNER = 5   # ShellBoundary::InFace (radius 0.5 sphere)
CON_PIPE_CYLINDER = 6  # PipeBoundary::CylinderFace
CON_PIPE_CIRCLE = 7    # PipeBoundary::YNeg/YPosCircleEdge (params: circle centre)

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z ^= z >> np.uint64(30)
        z *= np.uint64(0xBF58476D1CE4E5B9)
        z ^= z >> np.uint64(27)
        z *= np.uint64(0x94D049BB133111EB)
        z ^= z >> np.uint64(31)
    return z


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1) for (seed, stream); element i depends only on i."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([seed], dtype=np.uint64) + _GOLDEN * np.uint64(stream + 1))[0]
        idx = np.arange(1, n + 1, dtype=np.uint64)
        x = _mix(key + _GOLDEN * idx)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Box-Muller normals from two uniform streams (stream, stream + 1)."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 1, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


@dataclasses.dataclass
class RawMesh:
    pos: np.ndarray  # (V, 3) float64
    tets: np.ndarray  # (T, 4) uint32
    pris: np.ndarray  # (P, 6) uint32
    hexs: np.ndarray  # (H, 8) uint32
    cid: np.ndarray  # (V,) int32
    con_kind: np.ndarray  # (C,) int32, indexed by constraint id >= 0
    con_param: np.ndarray  # (C, 6) float64
    name: str = ""
    h: float = 0.0

    @property
    def nv(self) -> int:
        return int(self.pos.shape[0])

    @property
    def nelem(self) -> int:
        return int(self.tets.shape[0] + self.pris.shape[0] + self.hexs.shape[0])

    def movable(self) -> int:
        return int(np.count_nonzero(self.cid >= 0))


def box_constraints():
    """BoxBoundary's constraint table, ids 0..18 (Boundaries/BoxBoundary.cpp:4-38)."""
    kind = np.zeros(19, dtype=np.int32)
    par = np.zeros((19, 6), dtype=np.float64)
    faces = {1: ((-1, 0, 0), (-1, 0, 0)), 2: ((1, 0, 0), (1, 0, 0)),
             3: ((0, -1, 0), (0, -1, 0)), 4: ((0, 1, 0), (0, 1, 0)),
             5: ((0, 0, -1), (0, 0, -1)), 6: ((0, 0, 1), (0, 0, 1))}
    for i, (p, n) in faces.items():
        kind[i] = CON_PLANE
        par[i] = p + n
    edges = {7: ((-1, -1, -1), (1, -1, -1)), 8: ((-1, 1, -1), (1, 1, -1)),
             9: ((-1, -1, 1), (1, -1, 1)), 10: ((-1, 1, 1), (1, 1, 1)),
             11: ((-1, -1, -1), (-1, 1, -1)), 12: ((1, -1, -1), (1, 1, -1)),
             13: ((-1, -1, 1), (-1, 1, 1)), 14: ((1, -1, 1), (1, 1, 1)),
             15: ((-1, -1, -1), (-1, -1, 1)), 16: ((1, -1, -1), (1, -1, 1)),
             17: ((-1, 1, -1), (-1, 1, 1)), 18: ((1, 1, -1), (1, 1, 1))}
    for i, (a, b) in edges.items():
        kind[i] = CON_SEGMENT
        par[i] = a + b
    return kind, par


def sphere_constraints():
    kind = np.array([CON_VOLUME, CON_SPHERE], dtype=np.int32)
    par = np.zeros((2, 6), dtype=np.float64)
    return kind, par


def _box_ids(n: int) -> np.ndarray:
    """Constraint id of every grid vertex (x fastest), as genHexGrid assigns them."""
    r = np.arange(n + 1)
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    bx = np.where(x == 0, 0, np.where(x == n, 1, 2))
    by = np.where(y == 0, 0, np.where(y == n, 1, 2))
    bz = np.where(z == 0, 0, np.where(z == n, 1, 2))
    # table[bz][by][bx] following DebugMesher.cpp:177-261
    table = np.zeros((3, 3, 3), dtype=np.int32)
    table[0] = [[-1, -2, 7], [-4, -3, 8], [11, 12, 5]]
    table[1] = [[-5, -6, 9], [-8, -7, 10], [13, 14, 6]]
    table[2] = [[15, 16, 3], [17, 18, 4], [1, 2, 0]]
    return table[bz, by, bx].astype(np.int32)


def _grid_positions(n: int) -> np.ndarray:
    r = np.arange(n + 1, dtype=np.float64) / n
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    a = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    return -1.0 + a * 2.0


def _cell_corners(n: int, cells: np.ndarray | None = None) -> np.ndarray:
    """Hex vertex ids (MeshHex order) of every cell, x fastest."""
    r = np.arange(n)
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    if cells is not None:
        x, y, z = x[cells], y[cells], z[cells]
    W = n + 1

    def vid(dx, dy, dz):
        return (x + dx) + (y + dy) * W + (z + dz) * W * W

    return np.stack([vid(0, 0, 0), vid(1, 0, 0), vid(1, 1, 0), vid(0, 1, 0),
                     vid(0, 0, 1), vid(1, 0, 1), vid(1, 1, 1), vid(0, 1, 1)], axis=1)


# Kuhn (Freudenthal) split of a cube into 6 tets around the v0-v6 diagonal,
# each listed with positive orientation for the mean-ratio convention
# (det[v3-v0, v3-v1, v3-v2] > 0).
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6],
                  [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]], dtype=np.int64)


def _orient_kuhn():
    cube = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.float64)
    out = []
    for t in _KUHN:
        p = cube[t]
        d = np.linalg.det(np.stack([p[3] - p[0], p[3] - p[1], p[3] - p[2]], axis=1))
        out.append(t if d > 0 else t[[1, 0, 2, 3]])
    return np.array(out, dtype=np.int64)


KUHN = _orient_kuhn()
# two prisms per cell, extruded along +z (bottom triangle normal points up)
PRISM_SPLIT = np.array([[0, 1, 2, 4, 5, 6], [0, 2, 3, 4, 6, 7]], dtype=np.int64)


def _mk(pos, tets, pris, hexs, cid, kind, par, name, h):
    e = np.zeros((0, 4), np.uint32)
    return RawMesh(pos=np.ascontiguousarray(pos, dtype=np.float64),
                   tets=np.ascontiguousarray(tets if tets is not None else e, dtype=np.uint32).reshape(-1, 4),
                   pris=np.ascontiguousarray(pris if pris is not None else np.zeros((0, 6)), dtype=np.uint32).reshape(-1, 6),
                   hexs=np.ascontiguousarray(hexs if hexs is not None else np.zeros((0, 8)), dtype=np.uint32).reshape(-1, 8),
                   cid=np.ascontiguousarray(cid, dtype=np.int32), con_kind=kind, con_param=par,
                   name=name, h=h)


def box_positions(n: int, jitter: float = 0.3, seed: int = 0, gaussian: bool = False) -> np.ndarray:
    """Vertex positions of box_mesh(n, ..., jitter, seed, gaussian) (input order)."""
    h = 2.0 / n
    pos = _grid_positions(n)
    cid = _box_ids(n)
    interior = np.nonzero(cid == 0)[0]
    nv = pos.shape[0]
    if jitter > 0:
        if gaussian:
            d = np.stack([normal(seed, 2 * a, nv) for a in range(3)], axis=1) * (jitter * h)
        else:
            d = (np.stack([uniform(seed, a, nv) for a in range(3)], axis=1) * 2.0 - 1.0) * (jitter * h)
        pos[interior] += d[interior]
    return pos


def box_mesh(n: int, kind: str = "tet", jitter: float = 0.3, seed: int = 0,
             gaussian: bool = False) -> RawMesh:
    """Structured n^3-cell mesh of [-1,1]^3 under BoxBoundary.

    kind: "tet" (6 Kuhn tets per cell), "hex", "pri" (2 prisms per cell) or
    "mixed" (z-slabs: first third tets, second third prisms, rest hexes).
    Interior vertices move by U(+-jitter*h) per axis, or by N(0, jitter*h)
    when gaussian is true; boundary vertices stay on the box.
    """
    h = 2.0 / n
    pos = box_positions(n, jitter, seed, gaussian)
    cid = _box_ids(n)
    cells = _cell_corners(n)
    tets = pris = hexs = None
    if kind == "tet":
        tets = cells[:, KUHN].reshape(-1, 4)
    elif kind == "hex":
        hexs = cells
    elif kind == "pri":
        pris = cells[:, PRISM_SPLIT].reshape(-1, 6)
    elif kind == "mixed":
        cz = np.repeat(np.arange(n), n * n)
        a, b = (n + 2) // 3, (2 * n + 2) // 3
        tets = cells[cz < a][:, KUHN].reshape(-1, 4)
        pris = cells[(cz >= a) & (cz < b)][:, PRISM_SPLIT].reshape(-1, 6)
        hexs = cells[cz >= b]
    else:
        raise ValueError(f"unknown element kind {kind!r}")
    ck, cp = box_constraints()
    return _mk(pos, tets, pris, hexs, cid, ck, cp, f"box-{kind}-{n}", h)


def _sphere_layout(n: int):
    """Kept cells, kept vertex ids (grid numbering) and boundary mask of the
    n^3 grid clipped to the unit ball."""
    h = 2.0 / n
    r = np.arange(n)
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    cent = -1.0 + (np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1) + 0.5) * h
    keep = np.einsum("ij,ij->i", cent, cent) < 1.0
    kept = np.zeros((n + 2, n + 2, n + 2), dtype=bool)
    kept[1:-1, 1:-1, 1:-1] = keep.reshape(n, n, n)
    cells = _cell_corners(n, np.nonzero(keep)[0])
    W = n + 1
    # a vertex is on the boundary when any of its 8 surrounding cells is not kept
    vz, vy, vx = np.meshgrid(np.arange(W), np.arange(W), np.arange(W), indexing="ij")
    allk = np.ones((W, W, W), dtype=bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                allk &= kept[vz + dz, vy + dy, vx + dx]
    used = np.zeros(W ** 3, dtype=bool)
    used[cells.ravel()] = True
    ids = np.nonzero(used)[0]
    boundary = ~allk.ravel()[ids]
    return cells, ids, boundary


def sphere_positions(n: int, jitter: float = 0.25, seed: int = 1, layout=None) -> np.ndarray:
    """Vertex positions of sphere_mesh(n, jitter, seed) (input order)."""
    h = 2.0 / n
    cells, ids, boundary = layout if layout is not None else _sphere_layout(n)
    pos = _grid_positions(n)[ids]
    nv = ids.size
    d = (np.stack([uniform(seed, a, nv) for a in range(3)], axis=1) * 2.0 - 1.0) * (jitter * h)
    pos[~boundary] += d[~boundary]
    b = pos[boundary]
    pos[boundary] = b * (1.0 / np.sqrt(np.einsum("ij,ij->i", b, b)))[:, None]
    return pos


def sphere_mesh(n: int = 80, jitter: float = 0.25, seed: int = 1) -> RawMesh:
    """The n^3-cell grid of [-1,1]^3 clipped to the unit ball (cells whose
    centroid lies inside), split into Kuhn tets.  Vertices on the boundary of
    the kept cell set carry the sphere face constraint and are projected onto
    the sphere; interior vertices move by U(+-jitter*h) per axis."""
    h = 2.0 / n
    layout = _sphere_layout(n)
    cells, ids, boundary = layout
    W = n + 1
    remap = -np.ones(W ** 3, dtype=np.int64)
    remap[ids] = np.arange(ids.size)
    pos = sphere_positions(n, jitter, seed, layout)
    cid = np.where(boundary, 1, 0).astype(np.int32)
    tets = remap[cells][:, KUHN].reshape(-1, 4)
    ck, cp = sphere_constraints()
    return _mk(pos, tets, None, None, cid, ck, cp, f"sphere-{n}", h)


def batch_sizes(count: int = 4096, lo: int = 4, hi: int = 24, seed: int = 3) -> np.ndarray:
    """Cells per axis of each mesh of the batched workload, log-uniform in [lo, hi]."""
    u = uniform(seed, 1000, count)
    return np.clip(np.rint(np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))), lo, hi).astype(np.int64)


def batch_meshes(count: int = 4096, lo: int = 4, hi: int = 24, jitter: float = 0.3, seed: int = 3):
    """The batched workload: `count` jittered tet cubes of uneven size."""
    sizes = batch_sizes(count, lo, hi, seed)
    return [box_mesh(int(n), "tet", jitter, seed * 1000003 + i) for i, n in enumerate(sizes)]
