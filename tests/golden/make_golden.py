"""Generate tests/golden/*.npz from the reference's own CPU code.

Each fixture holds a small seeded mesh (inputs), the reference's NodeGroups
permutation and colour groups, its mesh evaluation, and the vertex positions
after one pass of each smoother (reference constants), all produced by the
reference compiled from its sources (oracle/refbuild.py).  Run from the repo
root where the reference tree exists:

    python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyref  # noqa: E402
from gpumesh_gb300 import meshgen  # noqa: E402

CASES = {
    "tet_box_6": (lambda: meshgen.box_mesh(6, "tet", 0.3, 0), "box", dict(sampler="uniform", evaluator="mean_ratio")),
    "mixed_box_5": (lambda: meshgen.box_mesh(5, "mixed", 0.15, 2, gaussian=True), "box",
                    dict(sampler="uniform", evaluator="mean_ratio")),
    "sphere_mc_8": (lambda: meshgen.sphere_mesh(8, 0.25, 1), "sphere",
                    dict(sampler="sine", evaluator="metric_conformity", scaling=4.0)),
    # the background-mesh samplers: local (walk + barycentric), kd-tree
    # (leaf samples), texture (grid samples, trilinear)
    "mixed_local_4": (lambda: meshgen.box_mesh(4, "mixed", 0.15, 21, gaussian=True), "box",
                      dict(sampler="local", evaluator="metric_conformity", scaling=2.0, aspect_ratio=3.0)),
    "mixed_kdtree_4": (lambda: meshgen.box_mesh(4, "mixed", 0.15, 22, gaussian=True), "box",
                       dict(sampler="kdtree", evaluator="metric_conformity", scaling=2.0, aspect_ratio=3.0)),
    "mixed_texture_4": (lambda: meshgen.box_mesh(4, "mixed", 0.15, 23, gaussian=True), "box",
                        dict(sampler="texture", evaluator="metric_conformity", scaling=2.0, aspect_ratio=3.0)),
}
SMOOTHERS = ["nelder_mead", "gradient_descent", "spawn_search", "getme", "spring_laplace", "quality_laplace"]


def make(name):
    build, boundary, crew = CASES[name]
    raw = build()
    out = dict(pos=raw.pos, tets=raw.tets, pris=raw.pris, hexs=raw.hexs, cid=raw.cid, con_kind=raw.con_kind,
               con_param=raw.con_param, boundary=boundary, sampler=crew["sampler"], evaluator=crew["evaluator"],
               scaling=crew.get("scaling", 1.0), aspect_ratio=crew.get("aspect_ratio", 1.0),
               depth=crew.get("depth", -1))
    ref = pyref.RefMesh(raw, boundary)
    # the harness reads the permutation from the vertex cache words, which
    # the background-mesh samplers overwrite with their walk caches
    out["perm"] = ref.perm()
    ref.set_crew(**crew)
    base, members, ranges = ref.groups()
    out.update(group_base=base, members=members, ranges=ranges)
    e = ref.evaluate()
    out.update(eval_min=e["min"], eval_inv_sum=e["inv_sum"], eval_count=e["count"], eval_buckets=e["buckets"])
    start = ref.pos
    for s in SMOOTHERS:
        ref.pos = start
        ref.smooth(s, 1)
        out["after_" + s] = ref.pos
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


# a small mesh file written by the reference's own JsonSerializer
JSON_CASE = ("tet_box_2_ref.json", lambda: meshgen.box_mesh(2, "tet", 0.3, 0), "box", "box-tet-2")


def make_json():
    fname, build, boundary, model = JSON_CASE
    pyref.json_write(os.path.join(HERE, fname), build(), boundary, model)


if __name__ == "__main__":
    for n in (sys.argv[1:] or CASES):
        make(n)
        print("wrote", n)
    make_json()
    print("wrote", JSON_CASE[0])
