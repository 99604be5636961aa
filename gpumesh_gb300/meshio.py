"""JSON mesh files in the reference tool's layout.

The reference writes a mesh as one JSON object (Serialization/
JsonSerializer.cpp:25-120, tags in JsonMeshTags.cpp:4-12):

    {
        "Model": "<model name>",
        "Boundary": "<boundary name>",
        "verts": [ [x, y, z], ... ],
        "topos": [ <constraint id of each vertex>, ... ],
        "tets": [ [4 ids], ... ], "pris": [ [6 ids], ... ], "hexs": [ [8 ids], ... ]
    }

and reads it back tag by tag (JsonDeserializer.cpp:23-131): a missing
"topos" leaves every vertex free, an unknown tag is an error, and the
boundary name selects one of the reference's boundaries (AbstractDeserializer
.cpp:10-29; an unknown name selects "Free").  `read_json` returns a RawMesh
whose constraint table is that boundary's (Free, Box, Sphere, Tet, Shell and
Pipe: the planes, segments, spheres and pipe surfaces the relocation kernels
project onto);
`write_json` writes the same layout, with the reference's 6 significant
digits (`ostream <<` defaults) or with every double written exactly.
"""

from __future__ import annotations

import json
import math
import os

import numpy as np

from .meshgen import (CON_PIPE_CIRCLE, CON_PIPE_CYLINDER, CON_PLANE, CON_SEGMENT, CON_SHELL_INNER, CON_SPHERE,
                      CON_VOLUME, RawMesh, box_constraints, sphere_constraints)

TAGS = ("Model", "Boundary", "verts", "topos", "tets", "pris", "hexs")


def _normalize(v):
    # glm::normalize: v * (1 / sqrt(v . v))
    s = 1.0 / math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return (v[0] * s, v[1] * s, v[2] * s)


def _cross(x, y):
    return (x[1] * y[2] - y[1] * x[2], x[2] * y[0] - y[2] * x[0], x[0] * y[1] - y[0] * x[1])


def tet_constraints():
    """TetBoundary's constraint table (Boundaries/TetBoundary.cpp:1-25): a
    regular tetrahedron with unit edges, centred on its first moment and
    scaled by 2; faces 1-4 (planes through the face centroid), edges 7-12
    (segments), corners -1..-4 (fixed)."""
    m = (0.5, 0.288675, 0.204124)
    corners = [(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.5, math.sqrt(3.0) / 2, 0.0),
               (0.5, math.sqrt(3.0) / 6, math.sqrt(2.0 / 3))]
    v = [tuple(2.0 * (c[k] - m[k]) for k in range(3)) for c in corners]
    edges = {7: (0, 1), 8: (0, 2), 9: (0, 3), 10: (1, 2), 11: (2, 3), 12: (3, 1)}
    u = {i: _normalize(tuple(v[b][k] - v[a][k] for k in range(3))) for i, (a, b) in edges.items()}

    def centroid(a, b, c):
        return tuple((v[a][k] + v[b][k] + v[c][k]) / 3.0 for k in range(3))

    def neg(x):
        return (-x[0], -x[1], -x[2])

    faces = {1: (centroid(0, 2, 1), _cross(u[8], neg(u[10]))),
             2: (centroid(0, 1, 3), _cross(u[7], neg(u[12]))),
             3: (centroid(0, 3, 2), _cross(u[9], neg(u[11]))),
             4: (centroid(1, 2, 3), _cross(u[10], u[11]))}
    kind = np.zeros(13, np.int32)
    par = np.zeros((13, 6), np.float64)
    for i, (p, n) in faces.items():
        kind[i] = CON_PLANE
        par[i] = p + n
    for i, (a, b) in edges.items():
        kind[i] = CON_SEGMENT
        par[i] = v[a] + v[b]
    return kind, par


def free_constraints():
    return np.array([CON_VOLUME], np.int32), np.zeros((1, 6), np.float64)


def shell_constraints():
    """ShellBoundary (Boundaries/ShellBoundary.cpp:3-56): outer face 1 the
    unit sphere, inner face 2 the radius-0.5 sphere."""
    kind = np.array([CON_VOLUME, CON_SPHERE, CON_SHELL_INNER], np.int32)
    return kind, np.zeros((3, 6), np.float64)


def pipe_constraints():
    """PipeBoundary (Boundaries/PipeBoundary.cpp:3-116): the U-bend wall 1,
    the two end disks 2 and 3 (planes through (-1, -+0.5, 0) with normal
    (-1, 0, 0)), their rim circles 4 and 5."""
    kind = np.array([CON_VOLUME, CON_PIPE_CYLINDER, CON_PLANE, CON_PLANE, CON_PIPE_CIRCLE, CON_PIPE_CIRCLE],
                    np.int32)
    par = np.zeros((6, 6), np.float64)
    par[2] = (-1.0, -0.5, 0.0, -1.0, 0.0, 0.0)
    par[3] = (-1.0, 0.5, 0.0, -1.0, 0.0, 0.0)
    par[4, :3] = (-1.0, -0.5, 0.0)
    par[5, :3] = (-1.0, 0.5, 0.0)
    return kind, par


BOUNDARIES = {"Free": free_constraints, "Box": box_constraints, "Sphere": sphere_constraints,
              "Tet": tet_constraints, "Shell": shell_constraints, "Pipe": pipe_constraints}


def boundary_table(name: str):
    """(kind, params) of a reference boundary by name ("Free" for an unknown name)."""
    return BOUNDARIES.get(name, free_constraints)()


def boundary_name(raw: RawMesh) -> str:
    """The reference boundary whose table the mesh carries."""
    for name, make in BOUNDARIES.items():
        kind, par = make()
        if (raw.con_kind.shape == kind.shape and np.array_equal(raw.con_kind, kind)
                and np.array_equal(raw.con_param, par)):
            return name
    if np.any(raw.con_kind == CON_SPHERE):
        return "Sphere"
    return "Free"


def _mean_edge(pos, tets, pris, hexs):
    d = []
    for e, pairs in ((tets, ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))),
                     (pris, ((0, 1), (1, 2), (2, 0), (0, 3), (1, 4), (2, 5))),
                     (hexs, ((0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 5), (2, 6), (3, 7)))):
        for a, b in pairs:
            if e.shape[0]:
                d.append(np.linalg.norm(pos[e[:, a]] - pos[e[:, b]], axis=1))
    return float(np.mean(np.concatenate(d))) if d else 0.0


def read_json(path: str) -> RawMesh:
    """A mesh file written by the reference tool (or write_json)."""
    with open(path) as f:
        doc = json.load(f)
    if not isinstance(doc, dict):
        raise ValueError(f"{path}: not a JSON mesh object")
    unknown = [k for k in doc if k not in TAGS]
    if unknown:
        raise ValueError(f"{path}: unknown tag {unknown[0]!r} in a JSON mesh")
    pos = np.asarray(doc.get("verts", []), np.float64).reshape(-1, 3)
    nv = pos.shape[0]

    def conn(tag, k):
        a = np.asarray(doc.get(tag, []), np.int64).reshape(-1, k)
        if a.size and (a.min() < 0 or a.max() >= nv):
            raise ValueError(f"{path}: {tag} reference a vertex outside 0..{nv - 1}")
        return a.astype(np.uint32)

    tets, pris, hexs = conn("tets", 4), conn("pris", 6), conn("hexs", 8)
    bname = doc.get("Boundary", "Free")
    kind, par = boundary_table(bname)
    if "topos" in doc:
        cid = np.asarray(doc["topos"], np.int64).reshape(-1)
        if cid.shape[0] != nv:
            raise ValueError(f"{path}: {cid.shape[0]} topos for {nv} vertices")
        if cid.size and cid.max() >= kind.shape[0]:
            raise ValueError(f"{path}: constraint id {int(cid.max())} is not a {bname} constraint")
        cid = cid.astype(np.int32)
    else:
        cid = np.zeros(nv, np.int32)
    name = doc.get("Model", os.path.splitext(os.path.basename(path))[0])
    return RawMesh(pos=pos, tets=tets, pris=pris, hexs=hexs, cid=cid, con_kind=kind, con_param=par, name=name,
                   h=_mean_edge(pos, tets, pris, hexs))


def _fmt_reference(x: float) -> str:
    # std::ostream << double with the default precision (6, %g style)
    return "%g" % x


def _fmt_exact(x: float) -> str:
    return repr(float(x))


def write_json(path: str, raw: RawMesh, boundary: str | None = None, model: str | None = None,
               precision: str = "exact") -> None:
    """Write the mesh in the reference's layout.  precision "reference"
    writes positions as the reference does (6 significant digits);
    "exact" writes every double so that read_json gives it back bit for bit."""
    fmt = {"reference": _fmt_reference, "exact": _fmt_exact}[precision]
    boundary = boundary or boundary_name(raw)
    model = raw.name if model is None else model
    ind = "    "
    out = ["{\n", f'{ind}"Model": "{model}",\n', f'{ind}"Boundary": "{boundary}",\n']

    def block(tag, rows, last=False):
        out.append(f'{ind}"{tag}": [\n')
        n = len(rows)
        for i, r in enumerate(rows):
            out.append(ind + ind + r + ("," if i != n - 1 else "") + "\n")
        out.append(ind + ("]\n" if last else "],\n"))

    block("verts", ["[" + ", ".join(fmt(c) for c in p) + "]" for p in raw.pos.tolist()])
    block("topos", [str(int(c)) for c in raw.cid.tolist()])
    block("tets", ["[" + ", ".join(str(i) for i in e) + "]" for e in raw.tets.tolist()])
    block("pris", ["[" + ", ".join(str(i) for i in e) + "]" for e in raw.pris.tolist()])
    block("hexs", ["[" + ", ".join(str(i) for i in e) + "]" for e in raw.hexs.tolist()], last=True)
    out.append("}\n")
    with open(path, "w") as f:
        f.write("".join(out))
