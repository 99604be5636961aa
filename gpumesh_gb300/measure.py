"""Timing helpers shared by the benchmark and the profiling drivers: clock
sampling during a timed region, an L2 flush, a sleep kernel that keeps the
device ahead of the host, and the HBM roofline of the evaluation kernel.
"""

from __future__ import annotations

import json
import os
import statistics
import subprocess

from . import meshgen
from . import mesh as M


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons, utilisation) taken
    every 200 ms while the context is open."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = [r.split(", ") for r in self.out.strip().splitlines() if r.strip()]
        sm, util, mx, reasons = [], [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
                util.append(float(r[9]))
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}
        if util:
            out["gpu_util_pct_mean"] = round(statistics.fmean(util), 1)
        return out


def hbm_peak_gbs(root: str) -> float:
    """The measured copy bandwidth of MEASURED_PEAKS.json under `root`, else
    the 6.8 TB/s fallback of an earlier GB300 measurement."""
    pp = os.path.join(root, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        with open(pp) as f:
            return json.load(f).get("hbm_gbs", 6800.0)
    return 6800.0


def l2_flush(torch, buf, stream):
    with torch.cuda.stream(stream):
        buf.zero_()


def gpu_ahead(torch, stream, ms=20.0):
    """Queue a sleep kernel of about `ms` on the stream, so that the launches
    queued after it by Python are all on the device before it ends: no timed
    launch then waits for the host."""
    with torch.cuda.stream(stream):
        torch.cuda._sleep(int(ms * 2.0e6))  # cycles at ~2 GHz


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of one evaluation of the 128^3 hex mesh and of the 128^3 x 6 tet
# cube (profiles/evaluate_kernel_*).
EVAL_TRAFFIC_BYTES = {"hex": 101_477_376 + 3_631_872, "tet": 235_710_976 + 4_071_168}


def eval_mesh(kind: str):
    """The evaluation roofline meshes: kind "hex" = the 128^3 hex mesh (C3:
    Gaussian jitter 0.15 h, seed 2), algorithmic bytes = 32 B/hex
    connectivity + 16 B/vertex; kind "tet" = the 128^3-cell tet cube (6 Kuhn
    tets per cell, jitter U(+-0.3 h), seed 0), 16 B/tet + 16 B/vertex."""
    if kind == "hex":
        raw = meshgen.box_mesh(128, "hex", 0.15, 2, gaussian=True)
        return raw, raw.hexs.shape[0] * 32 + raw.nv * 16
    raw = meshgen.box_mesh(128, "tet", 0.3, 0)
    return raw, raw.tets.shape[0] * 16 + raw.nv * 16


def eval_roofline(torch, stream, hbm_peak, kind="hex", launches=24, singles=10):
    """HBM roofline of the evaluation kernel (metric-free mean ratio) on the
    mesh of eval_mesh(kind).

    Reported (`achieved`): R device copies of the mesh, together more than
    twice the L2, evaluated round robin back to back, so that every launch
    reads a mesh the other R-1 have pushed out of L2; the average launch
    duration is the timed region over the launches.  Also reported
    (`single_*`): one launch at a time after a 256 MiB L2 flush, which adds
    the launch and DRAM ramp latency of an isolated launch.  Both are queued
    behind a sleep kernel, so no launch waits for Python."""
    raw, algo = eval_mesh(kind)
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
    stream.synchronize()
    gpu_ahead(torch, stream)
    a, b = ev(), ev()
    a.record(stream)
    for k in range(launches):
        copies[k % R].evaluate_async(0)
    b.record(stream)
    b.synchronize()
    t = a.elapsed_time(b) * 1e-3 / launches
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
            "traffic": EVAL_TRAFFIC_BYTES[kind], "algorithmic_bytes": algo, "us_per_launch": round(t * 1e6, 2),
            "timing": f"{launches} launches back to back over {R} device copies ({R * algo / 1e6:.0f} MB, "
                      f"> 2x the {l2 / 1e6:.0f} MB L2)",
            "single_us_per_launch": round(t1 * 1e6, 2), "single_frac": round(algo / t1 / 1e9 / hbm_peak, 4),
            "single_timing": "one launch after a 256 MiB L2 flush (write)",
            "min": h.minimumQuality(), "mean": h.harmonicMean(), "note": "of measured"}
