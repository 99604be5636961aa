"""Benchmark: vertex relocations/s of the GB300 smoothing path.

Headline workload: the sphere mesh -- 80^3 grid clipped to the unit ball,
~1.6M Kuhn tets, 283k vertices -- under SphereBoundary with the metric-wise
measurer, the sine-graded metric s^2 diag(1 + 9 sin^2(4 pi x), 1, 1) (s = 1/h)
and metric-conformity quality: five gradient-descent passes then five
spawn-search passes, with a full quality evaluation after every pass, as
AbstractSmoother's pass loop does.  One step = that whole schedule from the
same input mesh.

  value   relocations/s with the mesh resident in HBM (CUDA events)
  e2e     the same through the C ABI with host buffers: pinned-host upload of
          the positions, the schedule, and the read-back of positions and the
          per-pass quality histograms, all inside the timed region
  quality_vs_oracle  the final mesh re-evaluated by the FP64 oracle and
          compared with the oracle's own run of the schedule at full size
  c4      the batched configuration (4,096 tet cubes, one Nelder-Mead pass in
          one CUDA graph) against the plain path, with per-mesh latency
  c5      the served configuration (Poisson job stream, 60 s) against the
          plain path, p50 / p99 latency in real time and saturated
  --impl reference  the reference's CPU algorithm (the FP64 oracle port, with
          the oracle's own NodeGroups colouring), all host threads, on a
          bounded strided sample of the same workload

Run under torchrun with N > 1: every rank runs an independent replica (the
path has no exchange step); value is the sum over ranks.  The c4 / c5
objects are measured at N = 1 only.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from gpumesh_gb300 import workloads  # noqa: E402

METRIC = "vertex relocations/s"
UNIT = "relocations/s"
L2_NOTE = "GPU arm: L2 flushed (256 MiB write) before every step"

# FP32 operations per element-quality evaluation as the relocation kernels
# execute it (an add, multiply, reciprocal, square root or exp2/log2 counts
# 1, an FMA counts 2), counted by hand from gm_kernels.cuh / gm_device.cuh:
#   mean ratio, canonical tet (canonical_quality): 9 column subtractions,
#     det 14, |F|^2 17, power 3, 1/q 2, accumulate 1                     = 46
#   metric conformity, canonical tet, sine-graded metric (the paired
#     evaluation, canonical_mc_pair): 9 columns, 5 Keast sines by angle
#     addition 15, 5 metric values with the quadrature weight folded in 15,
#     quadrature sum 4, cofactors + det + F F^T + cofactor products 92,
#     weights 5, tNc 27 (tNc_yz = tNc_zy), |tNc|^2 16, two square roots +
#     add 3, accumulate 1                                                  = 187
#   the same under the uniform metric (no quadrature work)                 = 153
#   mean ratio, hex (mr_hex): 12 edges 36, 8 corners x 36, combination 9  = 333
# Per-candidate work (the frame columns, 3 sincospi) is shared by all the
# elements of a patch and not counted.
FLOPS_PER_ELEM_EVAL = {
    ("mean_ratio", "tet"): 46,
    ("mean_ratio", "hex"): 333,
    ("metric_conformity", "tet", "sine"): 187,
    ("metric_conformity", "tet", "uniform"): 153,
}

# DRAM traffic of the first spawn-search colour of the C2 sphere (61,699
# vertices) from an ncu capture, scaled to a pass by vertices
SPAWN_C2_TRAFFIC_PER_VERTEX = (39_982_848 + 16_128) / 61_699

FINALS = os.path.join(ROOT, "tests", "golden", "finals")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="C2", help="C1 | C2 | C3 | C3m (headline form), C4, C5, rows")
    ap.add_argument("--headline-only", action="store_true", help="skip the c4 / c5 objects of the default run")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-eval-roofline", action="store_true")
    ap.add_argument("--batch-meshes", type=int, default=4096, help="C4: number of meshes")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="C5: arrival window")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="C5: mean arrivals per second")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0, help="C5: HBM admission budget")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# Replicas: the path has no exchange step, so N GPUs run N independent
# replicas.  The only collectives are the timing barrier and the reductions
# of the step time (max) and of the units processed (sum).
def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = os.environ.get("GM_DIST_BACKEND") or ("nccl" if torch.cuda.is_available() else "gloo")
        dist.init_process_group(backend)
    return rank, world, local


def shard(items, rank, world):
    """Round-robin share of independent units (meshes, jobs) for one rank."""
    return list(items)[rank::world]


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _reduce(x, world, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world):
    import torch.distributed as dist

    return _reduce(x, world, dist.ReduceOp.MAX if world > 1 else None)


def sum_over_ranks(x, world):
    import torch.distributed as dist

    return _reduce(x, world, dist.ReduceOp.SUM if world > 1 else None)


# ---------------------------------------------------------------------------
def workload_config(w, raw, ncolours, world):
    """The `config` object of both arms' lines for a headline-form workload."""
    return {"workload": w.name, "vertices": int(raw.nv), "tets": int(raw.tets.shape[0]),
            "prisms": int(raw.pris.shape[0]), "hexes": int(raw.hexs.shape[0]), "colours": int(ncolours),
            "passes": w.passes(), "relocations_per_step": relocations_per_step(raw, w),
            "parallelism": f"replicas x{world}", "l2": L2_NOTE}


def relocations_per_step(raw, w):
    return int(np.count_nonzero(raw.cid >= 0)) * w.passes()


class CpuSample:
    """The reference's CPU algorithm -- the FP64 oracle port, bit-exact to the
    reference's own smoothers on every pinned case -- timed on a bounded
    sample of a workload: every `stride`-th member of every colour (starting
    at stride // 2), the whole schedule, colour-major with a barrier per
    colour on all the given threads.  NodeGroups orders each colour's members
    boundary, then subsurface, then interior vertices, so a strided sample
    keeps the three classes in their proportions in every colour."""

    def __init__(self, w, raw, group_base, members, ranges, threads):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        self.w, self.raw, self.threads = w, raw, threads
        self.gb = np.asarray(group_base, np.int64)
        self.members = np.asarray(members, np.uint32)
        self.ranges = np.asarray(ranges, np.int64).reshape(-1, 6)
        self.orc = pyoracle.OracleMesh.from_raw(raw, **w.crew(raw))

    def sample(self, stride):
        base, mem = [0], []
        for g in range(self.gb.size - 1):
            m = self.members[self.gb[g]:self.gb[g + 1]]
            s = m[min(stride // 2, max(0, m.size - 1))::stride]
            mem.append(s)
            base.append(base[-1] + s.size)
        return np.array(base, np.int64), np.concatenate(mem).astype(np.uint32)

    def classes(self, members, base):
        """(boundary, subsurface, interior) counts of a member list."""
        out = np.zeros(3, np.int64)
        for g in range(base.size - 1):
            m = members[base[g]:base[g + 1]].astype(np.int64)
            r = self.ranges[g]
            for c in range(3):
                out[c] += int(np.count_nonzero((m >= r[2 * c]) & (m < r[2 * c + 1])))
        return out

    def timed(self, stride):
        b, m = self.sample(stride)
        self.orc.pos = self.raw.pos
        t0 = time.perf_counter()
        for smoother, passes, params in self.w.schedule:
            for _ in range(passes):
                self.orc.smooth_pass(smoother, b, m, params=params, nthreads=self.threads)
        return time.perf_counter() - t0, int(m.size) * self.w.passes()

    def calibrate(self, seconds):
        """The stride whose sample takes about `seconds`."""
        stride = max(1, self.members.size // 1500)
        t, n = self.timed(stride)
        for _ in range(2):  # per-pass barriers make the time sublinear in the sample: refine twice
            stride = int(min(self.members.size, max(1, round(stride * t / seconds))))
            t, n = self.timed(stride)
            if 0.6 * seconds < t < 1.6 * seconds:
                break
        return stride

    def describe(self, stride, n, t):
        b, m = self.sample(stride)
        mix = self.classes(m, b)
        full = self.classes(self.members, self.gb)
        pct = lambda c: [round(100.0 * float(x) / max(1, int(c.sum())), 1) for x in c]  # noqa: E731
        return (f"every {stride}th member of every colour ({m.size} of {self.members.size} movable vertices), "
                f"the full schedule: {n} relocations in {t:.2f} s on {self.threads} threads; class mix "
                f"boundary/subsurface/interior % {pct(mix)} (whole mesh {pct(full)})")

    def close(self):
        self.orc.close()


# ---------------------------------------------------------------------------
def bench_reference(args, rank, world):
    """The reference arm: the reference's CPU algorithm (the oracle port) on
    this workload, on the host cores, loading no library of the product: the
    mesh comes from the seeded generator, its colouring and vertex order from
    the oracle's restatement of NodeGroups::build."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    w = workloads.WORKLOADS[args.workload]
    raw = w.mesh()
    perm, base, members, ranges = pyoracle.node_groups_build(raw)
    raw = pyoracle.permute(raw, perm)
    threads = os.cpu_count() or 1
    cs = CpuSample(w, raw, base, members, ranges, threads)
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    stride = cs.calibrate(per_step)
    vals, last = [], None
    for i in range(args.warmup + args.steps):
        t, n = cs.timed(stride)
        if i >= args.warmup:
            vals.append(n / t)
            last = (n, t)
    cs_desc = cs.describe(stride, *last)
    cs.close()
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": last[1] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(w, raw, base.size - 1, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": cs_desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def prepare(workload_name):
    from gpumesh_gb300 import mesh as M

    w = workloads.WORKLOADS[workload_name]
    raw = w.mesh()
    perm, groups = M.node_groups_build(raw)
    raw = M.permute_mesh(raw, perm)
    return w, raw, groups


def run_schedule(dev, w, torch, stream, ev_pass=None):
    """The whole schedule with an evaluation after every pass (slot k)."""
    slot = 0
    dev.evaluate_async(slot)
    slot += 1
    for smoother, passes, params in w.schedule:
        for _ in range(passes):
            if ev_pass is not None:
                ev_pass.append((smoother, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)))
                ev_pass[-1][1].record(stream)
            dev.smooth_pass(smoother, params)
            if ev_pass is not None:
                ev_pass[-1][2].record(stream)
            dev.evaluate_async(slot)
            slot += 1
    return slot


def flops_per_elem(w, raw):
    etype = "tet" if raw.tets.shape[0] else "hex"
    if w.evaluator == "metric_conformity":
        return FLOPS_PER_ELEM_EVAL.get((w.evaluator, etype, w.sampler))
    return FLOPS_PER_ELEM_EVAL.get((w.evaluator, etype))


def quality_vs_oracle(name, raw, crew, gpu_pos):
    """The GPU's final mesh against the FP64 oracle's run of the same
    schedule from the same FP32 input (tests/golden/finals, made by
    tests/golden/make_oracle_finals.py): both final meshes evaluated by the
    oracle's evaluator; per-vertex position error over the local mean edge
    length at the fixture's sampled vertices; the oracle's own spread under
    one-rounding input perturbations at the same size."""
    path = os.path.join(FINALS, name + ".npz")
    if not os.path.exists(path):
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    d = np.load(path)
    if int(d["nv"]) != raw.nv:
        return None
    chk = pyoracle.OracleMesh.from_raw(raw, **crew)
    chk.pos = np.asarray(gpu_pos, np.float64)
    e = chk.evaluate(nthreads=os.cpu_count() or 1)
    chk.close()
    idx = d["sample_idx"]
    err = np.linalg.norm(np.asarray(gpu_pos, np.float64)[idx] - d["sample_pos"], axis=1) / d["sample_edge"]
    dmin, dmean = abs(e["min"] - float(d["final_min"])), abs(e["mean"] - float(d["final_mean"]))
    ok_min, how_min = verdict(e["min"], float(d["final_min"]), d["fp32_min"], float(d["spread_min"]))
    ok_mean, how_mean = verdict(e["mean"], float(d["final_mean"]), d["fp32_mean"], float(d["spread_mean"]))
    return {"gpu_min": e["min"], "gpu_mean": e["mean"], "oracle_min": float(d["final_min"]),
            "oracle_mean": float(d["final_mean"]), "abs_dmin": dmin, "abs_dmean": dmean,
            "oracle_fp32_resolution_outcomes_min": [float(x) for x in d["fp32_min"]],
            "oracle_fp32_resolution_outcomes_mean": [float(x) for x in d["fp32_mean"]],
            "oracle_spread_min": float(d["spread_min"]), "oracle_spread_mean": float(d["spread_mean"]),
            "min_within": how_min if ok_min else None, "mean_within": how_mean if ok_mean else None,
            "pos_err_over_edge": {"max": float(err.max()), "p99": float(np.percentile(err, 99)),
                                  "mean": float(err.mean()), "samples": int(idx.size)},
            "oracle_spread_pos_max": float(d["spread_pos"]),
            "note": "GPU final mesh evaluated by the FP64 oracle; the oracle ran the same schedule from the same "
                    "FP32-rounded input.  Passing = within 1e-4 of the FP64 result ('fp64'), or of one of the "
                    "oracle's outcomes with its patch qualities at FP32 resolution (rounded, or seeded "
                    "(1 + u 2^-23) draws: 'fp32-resolution outcome'), or within 2 x the oracle's own spread: the "
                    "larger of its change under one-rounding-step input perturbations and of the FP32-resolution "
                    "draws' distance from the FP64 result ('2x oracle spread')"}


def verdict(gpu, fp64, draws, spread):
    """(passes, how) for one value: within 1e-4 of the FP64 oracle ("fp64"),
    or of one of its FP32-resolution outcomes ("fp32-resolution outcome"),
    or within twice the oracle's own spread -- the larger of its change
    under one-rounding-step input perturbations and of its FP32-resolution
    draws' distance from the FP64 result ("2x oracle spread")."""
    draws = np.asarray(draws, np.float64)
    if abs(gpu - fp64) <= 1e-4:
        return True, "fp64"
    if np.min(np.abs(draws - gpu)) <= 1e-4:
        return True, "fp32-resolution outcome"
    own = max(float(spread), float(np.max(np.abs(draws - fp64))))
    return bool(abs(gpu - fp64) <= 2 * own), "2x oracle spread"


def bench_gpu(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    from gpumesh_gb300 import _native as N
    from gpumesh_gb300 import measure
    from gpumesh_gb300 import mesh as M

    hbm_peak = measure.hbm_peak_gbs(ROOT)

    w, raw, groups = prepare(args.workload)
    crew = w.crew(raw)
    stream = torch.cuda.Stream()
    dev = M.DeviceMesh(raw, groups, stream=stream.cuda_stream)
    dev.set_crew(**crew)
    dev.save_positions()
    dev.sync()
    reloc = relocations_per_step(raw, w)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_step(record=None):
        dev.restore_positions()
        return run_schedule(dev, w, torch, stream, record)

    for _ in range(args.warmup):
        one_step()
    dev.sync()
    dev.counters(reset=True)

    pass_events = []
    step_times = []
    barrier(world)
    torch.cuda.synchronize()
    launches0 = M.launch_count()
    with measure.ClockSampler(local) as clocks:
        for _ in range(args.steps):
            measure.l2_flush(torch, flush, stream)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            nslots = one_step(pass_events)
            b.record(stream)
            b.synchronize()
            step_times.append(a.elapsed_time(b) * 1e-3)
        torch.cuda.synchronize()
    launches = M.launch_count() - launches0
    barrier(world)
    total = max_over_ranks(sum(step_times), world)
    value = reloc * args.steps * world / total
    ctr = dev.counters(reset=True)
    final = dev.read_quality(nslots - 1)
    first = dev.read_quality(0)
    final_pos = dev.fetch_positions()

    # dominant relocation kernel family: the smoother with the most pass time
    per = {}
    for sm, e0, e1 in pass_events:
        per.setdefault(sm, []).append(e0.elapsed_time(e1) * 1e-3)
    dom = max(per, key=lambda k: sum(per[k]))
    fpe = flops_per_elem(w, raw)
    fp32 = ctypes.c_double(0)
    N.check(N.lib().gm_probe_fp32_tflops(ctypes.byref(fp32)))
    # element evaluations of the dominant smoother's passes: measured by a
    # dedicated counted pass of that smoother from the same input
    dev.restore_positions()
    dc = {"elem_evals": 0}
    for smoother, passes, params in w.schedule:
        if smoother == dom:
            dev.counters(reset=True)
            dev.smooth_pass(smoother, params)
            dc = dev.counters(reset=True)
            break
        for _ in range(passes):
            dev.smooth_pass(smoother, params)
    dom_pass_s = statistics.median(per[dom])
    achieved = dc["elem_evals"] * fpe / dom_pass_s / 1e12 if fpe else None
    traffic = None
    if args.workload == "C2" and dom == "spawn_search":
        traffic = int(SPAWN_C2_TRAFFIC_PER_VERTEX * reloc / w.passes())
    roofline = {"bound": "fp32", "kernel": f"relocate_kernel ({dom}, {w.evaluator})",
                "achieved": round(achieved, 3) if achieved else None, "peak": round(fp32.value, 2),
                "unit": "TFLOP/s", "frac": round(achieved / fp32.value, 4) if achieved else None, "traffic": traffic,
                "traffic_note": "DRAM bytes per pass (8 launches), ncu capture of one colour scaled by vertices",
                "flops_per_element_eval": fpe, "element_evals_per_pass": dc["elem_evals"],
                "ms_per_pass": round(dom_pass_s * 1e3, 3),
                "note": "peak = FFMA probe measured in this run (no FP32 entry in MEASURED_PEAKS.json)"}

    # ---- e2e through the C ABI with host buffers ----
    host = torch.empty((raw.nv, 4), dtype=torch.float32, pin_memory=True)
    hv = host.numpy()
    hv[:, :3] = raw.pos
    hv[:, 3] = 0
    out = torch.empty((raw.nv, 4), dtype=torch.float32, pin_memory=True).numpy()
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.upload_gpu_verts(hv)
        n = run_schedule(dev, w, torch, stream)
        dev.fetch_gpu_verts(out)
        [dev.read_quality(s) for s in range(n)]
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_total = max_over_ranks(sum(e2e_times), world)
    e2e = {"value": reloc * args.steps * world / e2e_total, "unit": UNIT, "h2d_bytes_per_step": raw.nv * 16,
           "d2h_bytes_per_step": raw.nv * 16 + n * ctypes.sizeof(N.Quality)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(w, raw, groups.count(), world),
            "quality": {"initial_min": first.minimumQuality(), "initial_mean": first.harmonicMean(),
                        "final_min": final.minimumQuality(), "final_mean": final.harmonicMean()},
            "gpu_launches": launches, "roofline": roofline, "e2e": e2e, "clocks": clocks.summary(),
            "counters": ctr}
    if rank == 0:
        q = quality_vs_oracle(args.workload, raw, crew, final_pos)
        if q is not None:
            line["quality_vs_oracle"] = q
    if not args.no_eval_roofline and rank == 0:
        line["roofline_eval"] = measure.eval_roofline(torch, stream, hbm_peak, "hex")
        line["roofline_eval_tet"] = measure.eval_roofline(torch, stream, hbm_peak, "tet")
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cs = CpuSample(w, raw, groups.group_base, groups.members, groups.ranges, os.cpu_count() or 1)
        stride = cs.calibrate(args.cpu_seconds)
        t, n = cs.timed(stride)
        line["cpu_baseline"] = {"value": n / t, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": cs.describe(stride, n, t)}
        cs.close()
    dev.close()
    return line


# ---------------------------------------------------------------------------
def c4_quality_sample(qual):
    """The batched pass's per-mesh quality (the GPU evaluation) on the meshes
    the C4 oracle fixture samples, against the oracle's FP64 run from the
    same FP32 input."""
    path = os.path.join(FINALS, "C4.npz")
    if not os.path.exists(path):
        return None
    fx = np.load(path)
    rows, fmin, fmean = fx["rows"], fx["fp32_min"], fx["fp32_mean"]
    dmin, dmean, how = [], [], {}
    ok = True
    for k, r in enumerate(rows):
        i = int(r[0])
        if i >= len(qual):
            continue
        gmin, gmean = qual[i].minimumQuality(), qual[i].harmonicMean()
        dmin.append(abs(gmin - r[2]))
        dmean.append(abs(gmean - r[3]))
        a, ha = verdict(gmin, r[2], fmin[k], r[4])
        b, hb = verdict(gmean, r[3], fmean[k], r[5])
        ok = ok and a and b
        how[ha] = how.get(ha, 0) + 1
        how[hb] = how.get(hb, 0) + 1
    if not dmin:
        return None
    return {"meshes": len(dmin), "max_abs_dmin": float(max(dmin)), "max_abs_dmean": float(max(dmean)),
            "all_within": bool(ok), "values_within_by": how,
            "note": "GPU per-mesh evaluation of the batched pass vs the FP64 oracle's pass on the same mesh from "
                    "the same FP32 input; within = 1e-4 of the FP64 result, of an FP32-resolution outcome of the "
                    "oracle, or 2 x the oracle's own spread (input perturbations, FP32-resolution draws)"}


def bench_batched(args, rank, world, local):
    """C4: 4,096 jittered tet cubes (cells per axis log-uniform in [4, 24],
    jitter U(+-0.3h), seed 3), one Nelder-Mead pass (workloads.NM_PARAMS) plus
    a per-mesh evaluation, as ONE captured CUDA graph (one persistent
    relocation launch, one evaluation launch) with an autotuned launch shape;
    against the plain path, one mesh per launch sequence."""
    import torch

    torch.cuda.set_device(local)
    from gpumesh_gb300 import _native as N
    from gpumesh_gb300 import measure, meshgen
    from gpumesh_gb300 import mesh as M

    count = args.batch_meshes
    # weak scaling: `count` meshes per rank, dealt round-robin from one
    # stream of count * world meshes (N = 1 is the 4096-mesh workload itself)
    sizes = meshgen.batch_sizes(count * world, 4, 24, 3)
    mine = shard(range(count * world), rank, world)
    t0 = time.perf_counter()
    devs, movable, tets = [], 0, 0
    for i in mine:
        raw = meshgen.box_mesh(int(sizes[i]), "tet", 0.3, 3 * 1000003 + i)
        perm, groups = M.node_groups_build(raw)
        raw = M.permute_mesh(raw, perm)
        d = M.DeviceMesh(raw, groups)
        d.set_crew("uniform", "metric_free", "mean_ratio")
        d.save_positions()
        devs.append(d)
        movable += int(np.count_nonzero(raw.cid >= 0))
        tets += int(raw.tets.shape[0])
    setup_s = time.perf_counter() - t0
    params = workloads.NM_PARAMS
    batch = M.Batch(devs)
    wpb, cps, tune_ms = batch.tune("nelder_mead", params)
    batch.capture("nelder_mead", params, eval_slot=0)
    stream = torch.cuda.ExternalStream(batch.stream)

    def restore():
        for d in devs:
            d.restore_positions()
        torch.cuda.synchronize()

    # ---- batched ----
    for _ in range(args.warmup):
        restore()
        batch.replay()
        batch.sync()
    times, lat = [], []
    barrier(world)
    torch.cuda.synchronize()
    launches0 = M.launch_count()
    with measure.ClockSampler(local) as clocks:
        for _ in range(args.steps):
            restore()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            batch.replay()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b) * 1e-3)
            lat.append(batch.latencies_ms())
    torch.cuda.synchronize()
    launches = M.launch_count() - launches0
    barrier(world)
    assert batch.status() == 0
    qual = batch.read_quality(0)
    t_batched = max_over_ranks(statistics.median(times), world)
    units = sum_over_ranks(movable, world)
    lat = np.concatenate(lat)
    # ---- e2e through the public API: every mesh's positions uploaded from
    # pinned host memory, the captured pass, per-mesh histograms and
    # positions read back ----
    host_in = [torch.empty((d.nv, 4), dtype=torch.float32, pin_memory=True).numpy() for d in devs]
    host_out = [torch.empty((d.nv, 4), dtype=torch.float32, pin_memory=True).numpy() for d in devs]
    restore()
    for d, h in zip(devs, host_in):
        d.fetch_gpu_verts(h)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for d, h in zip(devs, host_in):
            d.upload_gpu_verts(h)
        torch.cuda.synchronize()
        batch.replay()
        e2e_qual = batch.read_quality(0)
        for d, h in zip(devs, host_out):
            d.fetch_gpu_verts(h)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_t = max_over_ranks(statistics.median(e2e_times), world)
    nv_total = sum(d.nv for d in devs)
    e2e = {"value": units / e2e_t, "unit": UNIT, "h2d_bytes_per_step": nv_total * 16,
           "d2h_bytes_per_step": nv_total * 16 + len(devs) * ctypes.sizeof(N.Quality)}
    assert len(e2e_qual) == len(devs)
    # ---- plain: one mesh per launch sequence (every colour of that mesh,
    # then its evaluation); per-mesh latency from a synchronised run ----
    plain_times, plain_lat = [], []
    for step in range(max(2, min(args.steps, 3))):
        restore()
        t1 = time.perf_counter()
        for d in devs:
            ta = time.perf_counter()
            d.smooth_pass("nelder_mead", params)
            d.evaluate_async(0)
            if step == 0:
                d.sync()
                plain_lat.append((time.perf_counter() - ta) * 1e3)
        torch.cuda.synchronize()
        plain_times.append(time.perf_counter() - t1)
    t_plain = max_over_ranks(statistics.median(plain_times[1:]), world)
    value = units / t_batched
    plain_value = units / t_plain
    ok = lat[lat >= 0]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_batched * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"C4 batched: {count} tet cubes, cells/axis log-uniform [4, 24], NM 1 pass + "
                                   "per-mesh evaluation, one CUDA graph", "meshes": count, "tets": tets,
                       "relocations_per_step": movable, "launch_shape": {"warps_per_block": wpb, "ctas_per_sm": cps},
                       "setup_s": round(setup_s, 1), "parallelism": f"replicas x{world}",
                       "l2": "not flushed: the 4,096 meshes' buffers (positions restored before every step) "
                             "exceed the L2"},
            "plain": {"value": plain_value, "unit": UNIT, "s_per_step": t_plain,
                      "p50_mesh_ms": float(np.percentile(plain_lat, 50)),
                      "p99_mesh_ms": float(np.percentile(plain_lat, 99)),
                      "note": "one launch sequence per mesh (its colours, then its evaluation), host-driven"},
            "batched_vs_plain": value / plain_value, "target_batched_vs_plain": 20.0,
            "latency_ms": {"p50": float(np.percentile(ok, 50)), "p99": float(np.percentile(ok, 99)),
                           "note": "per mesh: persistent-kernel start to the mesh's last relocated vertex"},
            "quality": {"min_of_mins": min(q.minimumQuality() for q in qual),
                        "mean_of_means": float(np.mean([q.harmonicMean() for q in qual]))},
            "e2e": e2e, "gpu_launches": launches, "clocks": clocks.summary()}
    qs = c4_quality_sample(qual) if world == 1 else None
    if qs is not None:
        line["quality_vs_oracle"] = qs
    batch.close()
    for d in devs:
        d.close()
    return line


def bench_served(args, rank, world, local):
    """C5: Poisson stream (mean 200 jobs/s, seed 4) of jittered cube / sphere
    tet meshes, 1k-2M tets log-uniform, smoother uniform in {NM, GD, GETMe},
    until the min-quality gain < 1e-3 or 20 passes, under an HBM budget.
    The served loop (one device-resident job graph per job, jobs overlapping
    on their own streams) and the plain path (one job at a time, passes
    launched and checked from the host) each run the stream twice: in real
    time, for p50/p99 latency from arrival to completion, and saturated (every
    job queued at the start), for the relocations/s each sustains.  value =
    the served loop's saturated relocations/s."""
    import torch

    torch.cuda.set_device(local)
    from gpumesh_gb300 import measure, serve
    from gpumesh_gb300 import mesh as M

    # weak scaling: one stream at world x the rate, jobs dealt round-robin,
    # so every rank serves ~serve_rate jobs/s
    stream = shard(serve.poisson_stream(args.serve_rate * world, args.serve_seconds, 4), rank, world)
    server = serve.Server(hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)))
    t0 = time.perf_counter()
    server.prepare(stream)
    setup_s = time.perf_counter() - t0
    warm = server.run(stream[: min(len(stream), 64)], realtime=False)  # slot creation for early jobs
    barrier(world)
    torch.cuda.synchronize()
    launches0 = M.launch_count()
    with measure.ClockSampler(local) as clocks_sat:
        sat = server.run(stream, realtime=False)
        torch.cuda.synchronize()
    launches = M.launch_count() - launches0
    with measure.ClockSampler(local) as clocks_rt:
        rt = server.run(stream, realtime=True)
        torch.cuda.synchronize()
    barrier(world)
    with measure.ClockSampler(local) as clocks_plain:
        plain_sat = serve.run_plain(server, stream, realtime=False)
    plain_rt = serve.run_plain(server, stream, realtime=True)
    wall = max_over_ranks(sat.wall_s, world)
    units = sum_over_ranks(sat.relocations, world)
    plain_wall = max_over_ranks(plain_sat.wall_s, world)
    line = {"metric": METRIC, "value": units / wall, "unit": UNIT, "n_gpus": world,
            "steps": 1, "warmup": 1, "ms_per_step": wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"C5 served: Poisson {args.serve_rate:g} jobs/s for {args.serve_seconds:g} s, "
                                   "1k-2M tets, NM/GD/GETMe, stop at min gain < 1e-3 or 20 passes",
                       "jobs": len(stream), "hbm_budget_gb": args.serve_budget_gb,
                       "setup_s": round(setup_s, 1), "warm_jobs": warm.jobs, "parallelism": f"replicas x{world}"},
            "served_saturated": sat.summary(),
            "served_realtime": rt.summary(),
            "plain_saturated": {"relocations_per_s": sum_over_ranks(plain_sat.relocations, world) / plain_wall,
                                "wall_s": round(plain_sat.wall_s, 3)},
            "plain_realtime": plain_rt.summary(),
            "served_vs_plain": (units / wall) / (sum_over_ranks(plain_sat.relocations, world) / plain_wall),
            "gpu_launches": launches,
            "clocks": clocks_sat.summary(), "clocks_realtime": clocks_rt.summary(),
            "clocks_plain_saturated": clocks_plain.summary()}
    server.close()
    return line


def c4_object(line):
    keep = ("value", "unit", "ms_per_step", "config", "plain", "batched_vs_plain", "target_batched_vs_plain",
            "latency_ms", "quality", "quality_vs_oracle", "e2e", "gpu_launches", "clocks")
    return {k: line[k] for k in keep if k in line}


def c5_object(line):
    keep = ("value", "unit", "config", "served_saturated", "served_realtime", "plain_saturated", "plain_realtime",
            "served_vs_plain", "gpu_launches", "clocks", "clocks_realtime", "clocks_plain_saturated")
    return {k: line[k] for k in keep if k in line}


# ---------------------------------------------------------------------------
def rows_measurement():
    """The rows widened beyond the headline path, on the C2 sphere (283,409
    vertices, 1,608,576 tets): per sampler the time to build its sampling
    (background mesh, kd-tree, texture) and one metric-conformity evaluation
    (5 metric samples per tet), beside the FP64 oracle's evaluation on all
    host cores; one pass of each Laplace smoother beside the oracle on a
    strided sample of every colour; one JSON write and read of the mesh."""
    import tempfile

    import torch

    from gpumesh_gb300 import measure, meshio
    from gpumesh_gb300 import mesh as M

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    w, raw, groups = prepare("C2")
    crew = w.crew(raw)
    stream = torch.cuda.Stream()
    threads = os.cpu_count() or 1
    out = {"mesh": "C2 sphere 80^3 clipped tets", "vertices": int(raw.nv), "tets": int(raw.tets.shape[0]),
           "cpu_threads": threads, "samplers": {}, "laplace": {}, "json": {}}

    def timed(fn, reps):
        # queued behind a sleep kernel, so no launch waits for Python; the
        # median of 3 rounds
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()
        torch.cuda.synchronize()
        rounds = []
        for _ in range(3):
            measure.gpu_ahead(torch, stream, 5.0)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            rounds.append(a.elapsed_time(b) / reps)
        return statistics.median(rounds)

    dev = M.DeviceMesh(raw, groups, stream=stream.cuda_stream)
    for sampler in ("uniform", "analytic", "local", "kdtree", "texture"):
        t0 = time.perf_counter()
        dev.set_crew(sampler, "metric_wise", "metric_conformity", crew["scaling"], 3.0)
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        ms = timed(lambda: dev.evaluate_async(0), 10)
        q = dev.evaluate().as_dict()
        t0 = time.perf_counter()
        orc = pyoracle.OracleMesh.from_raw(raw, sampler=sampler, measurer="metric_wise",
                                           evaluator="metric_conformity", scaling=crew["scaling"], aspect_ratio=3.0)
        cpu_build_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        o = orc.evaluate(nthreads=threads)
        cpu_s = time.perf_counter() - t0
        orc.close()
        out["samplers"][sampler] = {
            "build_s": round(build_s, 4), "eval_ms": round(ms, 4),
            "metric_samples_per_s": 5 * raw.tets.shape[0] / (ms * 1e-3),
            "cpu_build_s": round(cpu_build_s, 3), "cpu_eval_s": round(cpu_s, 3),
            "speedup_eval": round(cpu_s / (ms * 1e-3), 1),
            # the C2 start has inverted tets (harmonic mean 0): compare the
            # minimum
            "min": q["min"], "oracle_min": o["min"], "abs_diff_min": abs(q["min"] - o["min"]),
            "count": q["count"], "oracle_count": o["count"]}
    dev.set_crew(**crew)
    for smoother in ("spring_laplace", "quality_laplace"):
        saved = dev.fetch_positions()
        ms = timed(lambda: dev.smooth_pass(smoother, None), 3)
        dev.upload_positions(saved)
        movable = int(np.count_nonzero(raw.cid >= 0))
        lw = workloads.Workload("C2 " + smoother, None, w.sampler, w.measurer, w.evaluator, w.scaling,
                                [(smoother, 1, None)])
        cs = CpuSample(lw, raw, groups.group_base, groups.members, groups.ranges, threads)
        stride = 8
        t, n = cs.timed(stride)
        cs.close()
        out["laplace"][smoother] = {"pass_ms": round(ms, 4), "relocations_per_s": movable / (ms * 1e-3),
                                    "cpu_relocations_per_s": n / t, "cpu_sample_vertices": n}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "c2.json")
        t0 = time.perf_counter()
        meshio.write_json(path, raw, precision="exact")
        wr = time.perf_counter() - t0
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        back = meshio.read_json(path)
        rd = time.perf_counter() - t0
        out["json"] = {"bytes": size, "write_s": round(wr, 3), "read_s": round(rd, 3),
                       "exact_round_trip": bool(np.array_equal(back.pos, raw.pos))}
    return out


def main():
    args = parse()
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        bench_reference(args, rank, world)
    elif args.workload == "rows":
        if rank == 0:
            print(json.dumps(rows_measurement()), flush=True)
    elif args.workload == "C4":
        line = bench_batched(args, rank, world, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
    elif args.workload == "C5":
        line = bench_served(args, rank, world, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
    else:
        line = bench_gpu(args, rank, world, local)
        if args.workload == "C2" and world == 1 and not args.headline_only:
            line["c4"] = c4_object(bench_batched(args, rank, world, local))
            line["c5"] = c5_object(bench_served(args, rank, world, local))
        if rank == 0:
            print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
