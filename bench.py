"""Benchmark: vertex relocations/s of the GB300 smoothing path.

Workload (default): the sphere mesh -- 80^3 grid clipped to the unit ball,
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
  --impl reference  the reference's CPU algorithm (the FP64 oracle port),
          all host threads, on a bounded sample of the same workload

Run under torchrun with N > 1: every rank runs an independent replica (the
path has no exchange step); value is the sum over ranks.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertex relocations/s"
UNIT = "relocations/s"

# FP32 operations per element-quality evaluation as the relocation kernels
# execute it (an add, multiply, reciprocal, square root or exp2/log2 counts
# 1, an FMA counts 2), counted by hand from gm_kernels.cuh / gm_device.cuh:
#   mean ratio, canonical tet (canonical_quality): 9 column subtractions,
#     det 14, |F|^2 17, power 3, 1/q 2, accumulate 1                     = 46
#   metric conformity, canonical tet, sine-graded metric: 9 columns, 5
#     Keast sines by angle addition 15, 5 metric values 20, quadrature 6,
#     cofactors + det + F F^T + cofactor products 92, weights 6, tNc 30,
#     |tNc|^2 17, two square roots + add 3, accumulate 1                    = 199
#   the same under the uniform metric (no quadrature work)                 = 158
#   mean ratio, hex (mr_hex): 12 edges 36, 8 corners x 36, combination 9  = 333
# Per-candidate work (the frame columns, 3 sincospi) is shared by all the
# elements of a patch and not counted.
FLOPS_PER_ELEM_EVAL = {
    ("mean_ratio", "tet"): 46,
    ("mean_ratio", "hex"): 333,
    ("metric_conformity", "tet", "sine"): 199,
    ("metric_conformity", "tet", "uniform"): 158,
}

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of the same kernels on the same workloads: one evaluation of the
# 128^3 hex mesh and of the 128^3 x 6 tet cube, and the first spawn-search
# colour of the C2 sphere (61,699 vertices), scaled to a pass by vertices.
EVAL_HEX128_TRAFFIC_BYTES = 101_477_376 + 3_631_872
EVAL_TET128_TRAFFIC_BYTES = 235_710_976 + 4_071_168
SPAWN_C2_TRAFFIC_PER_VERTEX = (39_982_848 + 16_128) / 61_699


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="C2")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-eval-roofline", action="store_true")
    ap.add_argument("--batch-meshes", type=int, default=4096, help="C4: number of meshes")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="C5: arrival window")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="C5: mean arrivals per second")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0, help="C5: HBM admission budget")
    ap.add_argument("--only", choices=["eval", "eval_tet", "eval_local", "relocate", "batch", "eval_roofline", "rows"],
                    default=None,
                    help="profiling driver: a few launches of one kernel family, no JSON line "
                         "(eval_roofline: the two evaluation roofline objects, as JSON; rows: the "
                         "samplers, Laplace smoothers and JSON mesh files on the C2 mesh, as JSON)")
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


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = [r.split(", ") for r in self.out.strip().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def prepare(workload_name):
    from gpumesh_gb300 import mesh as M
    from gpumesh_gb300 import workloads

    w = workloads.WORKLOADS[workload_name]
    raw = w.mesh()
    perm, groups = M.node_groups_build(raw)
    raw = M.permute_mesh(raw, perm)
    return w, raw, groups


def relocations_per_step(raw, w):
    return int(np.count_nonzero(raw.cid >= 0)) * w.passes()


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


def l2_flush(torch, buf, stream):
    with torch.cuda.stream(stream):
        buf.zero_()


def flops_per_elem(w, raw):
    etype = "tet" if raw.tets.shape[0] else "hex"
    if w.evaluator == "metric_conformity":
        return FLOPS_PER_ELEM_EVAL.get((w.evaluator, etype, w.sampler))
    return FLOPS_PER_ELEM_EVAL.get((w.evaluator, etype))


def hbm_peak_gbs():
    """The measured copy bandwidth of MEASURED_PEAKS.json, else the 6.8 TB/s
    fallback of an earlier GB300 measurement."""
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        with open(pp) as f:
            return json.load(f).get("hbm_gbs", 6800.0)
    return 6800.0


def gpu_ahead(torch, stream, ms=20.0):
    """Queue a sleep kernel of about `ms` on the stream, so that the launches
    queued after it by Python are all on the device before it ends: no timed
    launch then waits for the host."""
    with torch.cuda.stream(stream):
        torch.cuda._sleep(int(ms * 2.0e6))  # cycles at ~2 GHz


def eval_roofline(torch, stream, hbm_peak, kind="hex", launches=24, singles=10):
    """HBM roofline of the evaluation kernel: kind "hex" = the 128^3 hex mesh
    (C3: Gaussian jitter 0.15 h, seed 2), algorithmic bytes = 32 B/hex
    connectivity + 16 B/vertex; kind "tet" = the 128^3-cell tet cube (6 Kuhn
    tets per cell, jitter U(+-0.3 h), seed 0), 16 B/tet + 16 B/vertex.
    Metric-free mean ratio.

    Reported (`achieved`): R device copies of the mesh, together more than
    twice the L2, evaluated round robin back to back, so that every launch
    reads a mesh the other R-1 have pushed out of L2; the average launch
    duration is the timed region over the launches.  Also reported
    (`single_*`): one launch at a time after a 256 MiB L2 flush, which adds
    the launch and DRAM ramp latency of an isolated launch.  Both are queued
    behind a sleep kernel, so no launch waits for Python."""
    from gpumesh_gb300 import mesh as M
    from gpumesh_gb300 import meshgen

    if kind == "hex":
        raw = meshgen.box_mesh(128, "hex", 0.15, 2, gaussian=True)
        algo = raw.hexs.shape[0] * 32 + raw.nv * 16
    else:
        raw = meshgen.box_mesh(128, "tet", 0.3, 0)
        algo = raw.tets.shape[0] * 16 + raw.nv * 16
    dev = M.DeviceMesh(raw, None)
    dev.set_stream(stream.cuda_stream)
    dev.set_crew("uniform", "metric_free", "mean_ratio")
    l2 = getattr(torch.cuda.get_device_properties(0), "L2_cache_size", 0) or 132 * 1024 * 1024
    R = max(2, -(-2 * l2 // algo) + 1)
    copies = [dev] + [M.DeviceMesh(None, clone_of=dev, stream=stream.cuda_stream) for _ in range(R - 1)]
    for c in copies:
        for _ in range(2):
            c.evaluate_async(0)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    # back to back over the copies
    stream.synchronize()
    gpu_ahead(torch, stream)
    a, b = ev(), ev()
    a.record(stream)
    for k in range(launches):
        copies[k % R].evaluate_async(0)
    b.record(stream)
    b.synchronize()
    t = a.elapsed_time(b) * 1e-3 / launches
    # isolated launches after an L2 flush
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    gpu_ahead(torch, stream)
    pairs = []
    for _ in range(singles):
        l2_flush(torch, flush, stream)
        a, b = ev(), ev()
        a.record(stream)
        dev.evaluate_async(0)
        b.record(stream)
        pairs.append((a, b))
    stream.synchronize()
    t1 = statistics.median(a.elapsed_time(b) * 1e-3 for a, b in pairs)
    achieved = algo / t / 1e9
    h = dev.read_quality(0)
    for c in copies:
        c.close()
    mesh = "128^3 hexes" if kind == "hex" else "128^3 x 6 tets"
    return {"bound": "hbm", "kernel": f"evaluate_kernel (mean ratio, {mesh})", "achieved": round(achieved, 1),
            "peak": hbm_peak, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
            "traffic": EVAL_HEX128_TRAFFIC_BYTES if kind == "hex" else EVAL_TET128_TRAFFIC_BYTES,
            "algorithmic_bytes": algo, "us_per_launch": round(t * 1e6, 2),
            "timing": f"{launches} launches back to back over {R} device copies ({R * algo / 1e6:.0f} MB, "
                      f"> 2x the {l2 / 1e6:.0f} MB L2)",
            "single_us_per_launch": round(t1 * 1e6, 2), "single_frac": round(algo / t1 / 1e9 / hbm_peak, 4),
            "single_timing": "one launch after a 256 MiB L2 flush (write)",
            "min": h.minimumQuality(), "mean": h.harmonicMean(), "note": "of measured"}


def cpu_sample_run(w, raw, groups, seconds, threads):
    """Time the FP64 oracle (the reference's algorithm) on a bounded sample:
    the first fraction f of every colour, the whole schedule, all threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    crew = w.crew(raw)
    orc = pyoracle.OracleMesh.from_raw(raw, **crew)
    gb = groups.group_base

    def sample(frac):
        base, mem = [0], []
        for g in range(groups.count()):
            m = groups.members[gb[g]:gb[g + 1]]
            k = max(1, int(round(frac * m.size))) if m.size else 0
            mem.append(m[:k])
            base.append(base[-1] + k)
        return np.array(base, np.int64), np.concatenate(mem).astype(np.uint32)

    def timed(frac):
        b, m = sample(frac)
        orc.pos = raw.pos
        t0 = time.perf_counter()
        for smoother, passes, params in w.schedule:
            for _ in range(passes):
                orc.smooth_pass(smoother, b, m, params=params, nthreads=threads)
        return time.perf_counter() - t0, int(m.size) * w.passes()

    frac = 0.002
    t, n = timed(frac)
    for _ in range(2):  # per-pass overheads make the time sublinear in the sample: refine twice
        frac = min(1.0, frac * (0.5 * seconds) / max(t, 1e-3))
        t, n = timed(frac)
        if t > 0.3 * seconds:
            break
    return n / t, frac, n, t


# ---------------------------------------------------------------------------
def bench_reference(args, rank, world):
    if rank != 0:
        return
    w, raw, groups = prepare(args.workload)
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    vals = []
    for i in range(args.warmup + args.steps):
        rate, frac, n, t = cpu_sample_run(w, raw, groups, per_step if i >= args.warmup else 1.0, threads)
        if i >= args.warmup:
            vals.append(rate)
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "vertices": raw.nv, "tets": int(raw.tets.shape[0]),
                       "parallelism": "cpu threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"first {frac:.4f} of every colour, full schedule ({n} relocations per step)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_gpu(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    from gpumesh_gb300 import _native as N
    from gpumesh_gb300 import mesh as M

    hbm_peak = hbm_peak_gbs()

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
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            l2_flush(torch, flush, stream)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            nslots = one_step(pass_events)
            b.record(stream)
            b.synchronize()
            step_times.append(a.elapsed_time(b) * 1e-3)
        torch.cuda.synchronize()
    barrier(world)
    total = max_over_ranks(sum(step_times), world)
    value = reloc * args.steps * world / total
    ctr = dev.counters(reset=True)
    final = dev.read_quality(nslots - 1)
    first = dev.read_quality(0)

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
        hist = [dev.read_quality(s) for s in range(n)]
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_total = max_over_ranks(sum(e2e_times), world)
    e2e = {"value": reloc * args.steps * world / e2e_total, "unit": UNIT, "h2d_bytes_per_step": raw.nv * 16,
           "d2h_bytes_per_step": raw.nv * 16 + n * ctypes.sizeof(N.Quality)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "vertices": raw.nv, "tets": int(raw.tets.shape[0]),
                       "colours": groups.count(), "passes": w.passes(), "relocations_per_step": reloc,
                       "parallelism": f"replicas x{world}", "l2": "flushed (256 MiB write) before every step"},
            "quality": {"initial_min": first.minimumQuality(), "initial_mean": first.harmonicMean(),
                        "final_min": final.minimumQuality(), "final_mean": final.harmonicMean()},
            "gpu_launches": None, "roofline": roofline, "e2e": e2e, "clocks": clocks.summary(),
            "counters": ctr}
    # launches in the timed region: per pass, relocation + FP64 acceptance per colour,
    # one counter reset, evaluation (2) after every pass, plus the initial evaluation and restore
    ng = groups.count()
    launches_per_step = 2 + w.passes() * (2 * ng + 2)
    if any(s == "getme" for s, _, _ in w.schedule):
        launches_per_step += sum(p for s, p, _ in w.schedule if s == "getme")
    line["gpu_launches"] = launches_per_step * args.steps
    if not args.no_eval_roofline and rank == 0:
        line["roofline_eval"] = eval_roofline(torch, stream, hbm_peak, "hex")
        line["roofline_eval_tet"] = eval_roofline(torch, stream, hbm_peak, "tet")
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, frac, n, t = cpu_sample_run(w, raw, groups, args.cpu_seconds, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"first {frac:.4f} of every colour, full schedule, {n} relocations "
                                          f"in {t:.1f} s"}
    dev.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def profile_driver(args):
    """A few launches of one kernel family, for ncu: `eval` = the evaluation
    kernel on the 128^3 hex mesh (4 launches), `eval_tet` = the same on the
    128^3 x 6 tet cube; `relocate` = one pass of each
    smoother of the workload's schedule; `batch` = two batched Nelder-Mead
    passes over the first --batch-meshes meshes of C4."""
    import torch

    from gpumesh_gb300 import mesh as M
    from gpumesh_gb300 import meshgen, workloads

    if args.only == "rows":
        print(json.dumps(rows_measurement(torch)), flush=True)
    elif args.only == "eval_roofline":
        stream = torch.cuda.Stream()
        peak = hbm_peak_gbs()
        print(json.dumps({"roofline_eval": eval_roofline(torch, stream, peak, "hex"),
                          "roofline_eval_tet": eval_roofline(torch, stream, peak, "tet")}), flush=True)
    elif args.only == "eval_local":
        # metric-conformity evaluation of the C2 mesh under the local sampler
        # (a background walk per Keast point), 4 launches
        w, raw, groups = prepare("C2")
        dev = M.DeviceMesh(raw, None)
        dev.set_crew("local", "metric_wise", "metric_conformity", w.crew(raw)["scaling"], 3.0)
        for _ in range(4):
            h = dev.evaluate()
        print("eval_local", h.minimumQuality(), h.sampleCount())
    elif args.only in ("eval", "eval_tet"):
        if args.only == "eval":
            raw = meshgen.box_mesh(128, "hex", 0.15, 2, gaussian=True)
        else:
            raw = meshgen.box_mesh(128, "tet", 0.3, 0)
        dev = M.DeviceMesh(raw, None)
        dev.set_crew("uniform", "metric_free", "mean_ratio")
        for _ in range(4):
            h = dev.evaluate()
        print("eval", h.minimumQuality(), h.harmonicMean())
    elif args.only == "batch":
        # the first --batch-meshes meshes of the C4 stream, 8 warps per block,
        # two Nelder-Mead passes of the persistent kernel
        sizes = meshgen.batch_sizes(args.batch_meshes, 4, 24, 3)
        devs = []
        for i, n in enumerate(sizes):
            raw = meshgen.box_mesh(int(n), "tet", 0.3, 3 * 1000003 + i)
            perm, groups = M.node_groups_build(raw)
            d = M.DeviceMesh(M.permute_mesh(raw, perm), groups)
            d.set_crew("uniform", "metric_free", "mean_ratio")
            devs.append(d)
        batch = M.Batch(devs)
        batch.set_config(8, 0)
        for _ in range(2):
            batch.smooth_pass("nelder_mead", workloads.NM_PARAMS)
            batch.sync()
        print("batch", batch.status(), batch.counters())
    else:
        w, raw, groups = prepare(args.workload)
        dev = M.DeviceMesh(raw, groups)
        dev.set_crew(**w.crew(raw))
        for smoother, passes, params in w.schedule:
            dev.smooth_pass(smoother, params)
        print("relocate", dev.evaluate().as_dict()["mean"])
    torch.cuda.synchronize()


def rows_measurement(torch):
    """The rows widened beyond the headline path, on the C2 sphere (283,409
    vertices, 1,608,576 tets): per sampler the time to build its sampling
    (background mesh, kd-tree, texture) and one metric-conformity evaluation
    (5 metric samples per tet), beside the FP64 oracle's evaluation on all
    host cores; one pass of each Laplace smoother beside the oracle on a
    sample of its first colour; one JSON write and read of the mesh."""
    import os
    import tempfile

    from gpumesh_gb300 import mesh as M
    from gpumesh_gb300 import meshio

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
            gpu_ahead(torch, stream, 5.0)
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
        # the oracle on the first eighth of every colour, scaled
        base = groups.group_base
        sample_base, sample_members = [0], []
        for g in range(len(base) - 1):
            m = groups.members[base[g]:base[g + 1]]
            sample_members.append(m[: max(1, m.size // 8)])
            sample_base.append(sample_base[-1] + sample_members[-1].size)
        orc = pyoracle.OracleMesh.from_raw(raw, **crew)
        t0 = time.perf_counter()
        orc.smooth_pass(smoother, np.array(sample_base, np.int64), np.concatenate(sample_members), nthreads=threads)
        cpu_s = time.perf_counter() - t0
        orc.close()
        out["laplace"][smoother] = {"pass_ms": round(ms, 4), "relocations_per_s": movable / (ms * 1e-3),
                                    "cpu_relocations_per_s": sample_base[-1] / cpu_s,
                                    "cpu_sample_vertices": int(sample_base[-1])}
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


def bench_batched(args, rank, world, local):
    """C4: 4,096 jittered tet cubes (cells per axis log-uniform in [4, 24],
    jitter U(+-0.3h), seed 3), one Nelder-Mead pass (workloads.NM_PARAMS) plus
    a per-mesh evaluation, as ONE captured CUDA graph (one persistent
    relocation launch, one evaluation launch) with an autotuned launch shape;
    against the plain path, one mesh per launch sequence."""
    import torch

    torch.cuda.set_device(local)
    from gpumesh_gb300 import mesh as M
    from gpumesh_gb300 import meshgen, workloads

    count = args.batch_meshes
    # weak scaling: `count` meshes per rank, dealt round-robin from one
    # stream of count * world meshes (N = 1 is the 4096-mesh workload itself)
    sizes = meshgen.batch_sizes(count * world, 4, 24, 3)
    mine = shard(range(count * world), rank, world)
    t0 = time.perf_counter()
    devs, movable, tets = [], 0, 0
    for i in mine:
        n = sizes[i]
        raw = meshgen.box_mesh(int(n), "tet", 0.3, 3 * 1000003 + i)
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
    with ClockSampler(local) as clocks:
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
    import ctypes

    from gpumesh_gb300 import _native as N

    e2e = {"value": units / e2e_t, "unit": UNIT, "h2d_bytes_per_step": nv_total * 16,
           "d2h_bytes_per_step": nv_total * 16 + len(devs) * ctypes.sizeof(N.Quality)}
    assert len(e2e_qual) == len(devs)
    # ---- plain: one mesh per launch sequence (every colour of that mesh, then its evaluation) ----
    restore()
    plain_times, plain_lat = [], []
    for step in range(max(1, args.steps)):
        restore()
        torch.cuda.synchronize()
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
    t_plain = max_over_ranks(statistics.median(plain_times[1:] if len(plain_times) > 1 else plain_times), world)
    value = units / t_batched
    plain_value = units / t_plain
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_batched * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"C4 batched: {count} tet cubes, cells/axis log-uniform [4, 24], NM 1 pass + "
                                   "per-mesh evaluation, one CUDA graph", "meshes": count, "tets": tets,
                       "relocations_per_step": movable, "launch_shape": {"warps_per_block": wpb, "ctas_per_sm": cps},
                       "setup_s": round(setup_s, 1), "parallelism": f"replicas x{world}"},
            "plain": {"value": plain_value, "unit": UNIT, "s_per_step": t_plain,
                      "p50_mesh_ms": float(np.percentile(plain_lat, 50)), "p99_mesh_ms": float(np.percentile(plain_lat, 99))},
            "batched_vs_plain": value / plain_value,
            "latency_ms": {"p50": float(np.percentile(lat[lat >= 0], 50)), "p99": float(np.percentile(lat[lat >= 0], 99)),
                           "note": "per mesh: persistent-kernel start to the mesh's last relocated vertex"},
            "quality": {"min_of_mins": min(q.minimumQuality() for q in qual),
                        "mean_of_means": float(np.mean([q.harmonicMean() for q in qual]))},
            "e2e": e2e, "gpu_launches": 2 * args.steps + 1 * args.steps, "clocks": clocks.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


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
    from gpumesh_gb300 import serve

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
    with ClockSampler(local) as clocks:
        sat = server.run(stream, realtime=False)
        torch.cuda.synchronize()
        rt = server.run(stream, realtime=True)
        torch.cuda.synchronize()
    barrier(world)
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
            "gpu_launches": None, "clocks": clocks.summary()}
    server.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.only:
        profile_driver(args)
        return
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        bench_reference(args, rank, world)
    elif args.workload == "C4":
        bench_batched(args, rank, world, local)
    elif args.workload == "C5":
        bench_served(args, rank, world, local)
    else:
        bench_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
