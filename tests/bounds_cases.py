"""Small in-range cases through every kernel family (evaluation of tet /
mixed / hex meshes, Nelder-Mead, gradient descent, spawn search, the Laplace
smoothers, GETMe, metric conformity under the sine metric, the batched
pass), shared by tests/test_gpu_bounds_checked.py: run once with the
ordinary library and once, in a child process, with the bounds-checked one
(GPUMESH_GB300_LIB=checked).  Writes every result and the meshes' bounds
status words to an .npz given on the command line."""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gpumesh_gb300 import meshgen, workloads  # noqa: E402
from gpumesh_gb300 import mesh as M  # noqa: E402
from gpumesh_gb300 import _native as N  # noqa: E402

MR = ("uniform", "metric_free", "mean_ratio", 1.0, 1.0)


def coloured(raw):
    perm, groups = M.node_groups_build(raw)
    return M.permute_mesh(raw, perm), groups


def status(dev):
    import ctypes

    what, index = ctypes.c_uint32(), ctypes.c_uint32()
    N.check(N.lib().gm_mesh_bounds_status(dev.h, ctypes.byref(what), ctypes.byref(index)))
    return int(what.value)


def run_cases() -> dict:
    import ctypes

    out = {}
    on = ctypes.c_int32()
    N.check(N.lib().gm_bounds_checked(ctypes.byref(on)))
    out["checked"] = np.int32(on.value)
    cases = {
        "tet": (meshgen.box_mesh(6, "tet", 0.3, 0), MR,
                [("nelder_mead", workloads.NM_PARAMS), ("gradient_descent", None), ("spawn_search", None),
                 ("spring_laplace", None), ("quality_laplace", None)]),
        "mixed": (meshgen.box_mesh(5, "mixed", 0.15, 2, gaussian=True), MR,
                  [("nelder_mead", None), ("getme", workloads.GETME_PARAMS)]),
        "hex": (meshgen.box_mesh(6, "hex", 0.15, 2, gaussian=True), MR, [("getme", workloads.GETME_PARAMS),
                                                                          ("gradient_descent", None)]),
    }
    sphere = meshgen.sphere_mesh(8, 0.25, 1)
    cases["sphere_mc"] = (sphere, ("sine", "metric_wise", "metric_conformity", 1.0 / sphere.h, 1.0),
                          [("gradient_descent", workloads.GD_PARAMS), ("spawn_search", workloads.SPAWN_PARAMS)])
    words = []
    for name, (raw, crew, steps) in cases.items():
        raw, groups = coloured(raw)
        dev = M.DeviceMesh(raw, groups)
        dev.set_crew(*crew)
        out[f"{name}_q0"] = np.array(list(dev.evaluate().as_dict().values())[:4], dtype=object).astype(float)
        for k, (smoother, params) in enumerate(steps):
            dev.smooth_pass(smoother, params)
            out[f"{name}_pos{k}"] = dev.fetch_positions()
        q = dev.evaluate().as_dict()
        out[f"{name}_q1"] = np.array([q["min"], q["inv_sum"], q["count"]], float)
        out[f"{name}_buckets"] = np.array(q["buckets"], np.int64)
        words.append(status(dev))
        dev.close()
    devs = []
    for i, n in enumerate((4, 6, 5)):
        raw, groups = coloured(meshgen.box_mesh(n, "tet", 0.3, 40 + i))
        d = M.DeviceMesh(raw, groups)
        d.set_crew(*MR)
        devs.append(d)
    batch = M.Batch(devs)
    batch.smooth_pass("nelder_mead", workloads.NM_PARAMS)
    batch.evaluate(0)
    batch.sync()
    out["batch_status"] = np.int32(batch.status())
    out["batch_q"] = np.array([[q.minimumQuality(), q.invQualitySum()] for q in batch.read_quality(0)])
    for i, d in enumerate(devs):
        out[f"batch_pos{i}"] = d.fetch_positions()
        words.append(status(d))
    batch.close()
    out["bounds_words"] = np.array(words, np.int64)
    return out


if __name__ == "__main__":
    np.savez(sys.argv[1], **run_cases())
