"""Profiling drivers: a few launches of one kernel family on a fixed
workload, small enough for an ncu capture, with no timing of their own.

    python -m gpumesh_gb300.profiling eval         evaluation, 128^3 hex mesh, 4 launches
    python -m gpumesh_gb300.profiling eval_tet     evaluation, 128^3 x 6 tet cube, 4 launches
    python -m gpumesh_gb300.profiling eval_local   metric-conformity evaluation of the C2 sphere
                                                   under the local sampler, 4 launches
    python -m gpumesh_gb300.profiling relocate [W] one pass of each smoother of workload W's
                                                   schedule (default C2)
    python -m gpumesh_gb300.profiling batch [N]    two batched Nelder-Mead passes over the
                                                   first N meshes of the C4 stream (default 256)
    python -m gpumesh_gb300.profiling eval_roofline  the two evaluation roofline objects, as JSON
"""

from __future__ import annotations

import json
import os
import sys

from . import meshgen, workloads
from . import mesh as M
from . import measure

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def coloured(raw):
    perm, groups = M.node_groups_build(raw)
    return M.permute_mesh(raw, perm), groups


def main(argv):
    import torch

    what = argv[0] if argv else "eval"
    if what == "eval_roofline":
        stream = torch.cuda.Stream()
        peak = measure.hbm_peak_gbs(ROOT)
        print(json.dumps({"roofline_eval": measure.eval_roofline(torch, stream, peak, "hex"),
                          "roofline_eval_tet": measure.eval_roofline(torch, stream, peak, "tet")}), flush=True)
    elif what in ("eval", "eval_tet"):
        raw, _ = measure.eval_mesh("hex" if what == "eval" else "tet")
        dev = M.DeviceMesh(raw, None)
        dev.set_crew("uniform", "metric_free", "mean_ratio")
        for _ in range(4):
            h = dev.evaluate()
        print(what, h.minimumQuality(), h.harmonicMean())
    elif what == "eval_local":
        w = workloads.WORKLOADS["C2"]
        raw, groups = coloured(w.mesh())
        dev = M.DeviceMesh(raw, None)
        dev.set_crew("local", "metric_wise", "metric_conformity", w.crew(raw)["scaling"], 3.0)
        for _ in range(4):
            h = dev.evaluate()
        print("eval_local", h.minimumQuality(), h.sampleCount())
    elif what == "batch":
        count = int(argv[1]) if len(argv) > 1 else 256
        sizes = meshgen.batch_sizes(count, 4, 24, 3)
        devs = []
        for i, n in enumerate(sizes):
            raw, groups = coloured(meshgen.box_mesh(int(n), "tet", 0.3, 3 * 1000003 + i))
            d = M.DeviceMesh(raw, groups)
            d.set_crew("uniform", "metric_free", "mean_ratio")
            devs.append(d)
        batch = M.Batch(devs)
        batch.set_config(8, 0)
        for _ in range(2):
            batch.smooth_pass("nelder_mead", workloads.NM_PARAMS)
            batch.sync()
        print("batch", batch.status(), batch.counters())
    elif what == "relocate":
        w = workloads.WORKLOADS[argv[1] if len(argv) > 1 else "C2"]
        raw, groups = coloured(w.mesh())
        dev = M.DeviceMesh(raw, groups)
        dev.set_crew(**w.crew(raw))
        for smoother, passes, params in w.schedule:
            dev.smooth_pass(smoother, params)
        print("relocate", dev.evaluate().as_dict()["mean"])
    else:
        raise SystemExit(f"unknown driver {what!r}; see the module docstring")
    torch.cuda.synchronize()


if __name__ == "__main__":
    main(sys.argv[1:])
