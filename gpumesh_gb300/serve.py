"""Served smoothing: a continuous-batching request loop.

Jobs arrive over time (a Poisson stream).  Each job is a jittered cube or
sphere tet mesh with its own seed and a smoother (Nelder-Mead, gradient
descent or GETMe); it runs relocation passes until its min-quality gain
drops below a threshold or a pass cap is reached (the stop rule of the
served workload; the reference's autopilot compares mean and min gains,
Smoothers/AbstractSmoother.cpp:182-193).

The loop works in ticks.  At each tick it admits arrived jobs while their
device footprint fits the HBM budget, then runs ONE pass for every active
job: the active jobs of each smoother form a gm_batch relocated by one
persistent launch and evaluated per mesh by one launch.  Jobs join and
leave between ticks, so requests that arrive while others are on the GPU
share the next launches with them, and every job's mesh stays resident on
the device from admission to completion.

Job meshes reuse resident topology templates: all jobs of one (kind, cells
per axis) share the connectivity, constraints and colouring, which are
built once; a job is a device-to-device clone of its template plus its own
positions, identical to what meshgen.box_mesh / sphere_mesh produce for the
job's seed.
"""

from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import meshgen
from . import mesh as M

SMOOTHERS = ("nelder_mead", "gradient_descent", "getme")
DEFAULT_PARAMS = {"nelder_mead": [0.1, 32, 1e-4, 1.0, 0.5, 2.0], "gradient_descent": [0.01, 5],
                  "getme": [0.5], "spawn_search": [1.0 / 20.0, 2]}
MR = dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio")


@dataclasses.dataclass
class JobSpec:
    job_id: int
    arrival: float  # seconds after the start of the stream
    kind: str       # "cube" or "sphere"
    n: int          # cells per axis
    seed: int
    smoother: str

    def raw(self) -> meshgen.RawMesh:
        """The job's mesh from the standalone generator (input order)."""
        if self.kind == "cube":
            return meshgen.box_mesh(self.n, "tet", 0.3, self.seed)
        return meshgen.sphere_mesh(self.n, 0.25, self.seed)


def cells_for(kind: str, tets: float) -> int:
    """Cells per axis for a target tet count (cube: 6 n^3; ball: ~pi n^3)."""
    if kind == "cube":
        return max(2, int(round((tets / 6.0) ** (1.0 / 3.0))))
    return max(4, int(round((tets / math.pi) ** (1.0 / 3.0))))


def poisson_stream(rate: float = 200.0, seconds: float = 60.0, seed: int = 4, lo: float = 1e3, hi: float = 2e6,
                   smoothers=SMOOTHERS) -> list[JobSpec]:
    """The served workload: Poisson arrivals (mean `rate` jobs/s for
    `seconds`), sizes log-uniform in [lo, hi] tets, kind and smoother drawn
    uniformly."""
    cap = int(rate * seconds * 2 + 64)
    gaps = -np.log1p(-meshgen.uniform(seed, 10, cap)) / rate
    t = np.cumsum(gaps)
    n_jobs = int(np.searchsorted(t, seconds))
    u_size = meshgen.uniform(seed, 11, n_jobs)
    u_kind = meshgen.uniform(seed, 12, n_jobs)
    u_sm = meshgen.uniform(seed, 13, n_jobs)
    jobs = []
    for k in range(n_jobs):
        tets = math.exp(math.log(lo) + u_size[k] * (math.log(hi) - math.log(lo)))
        kind = "cube" if u_kind[k] < 0.5 else "sphere"
        jobs.append(JobSpec(k, float(t[k]), kind, cells_for(kind, tets), seed * 1000003 + k,
                            smoothers[min(len(smoothers) - 1, int(u_sm[k] * len(smoothers)))]))
    return jobs


class Template:
    """Resident topology of one (kind, n): permuted connectivity, colouring,
    constraints; job positions are generated per seed in the same order."""

    def __init__(self, kind: str, n: int):
        self.kind, self.n = kind, n
        if kind == "cube":
            raw = meshgen.box_mesh(n, "tet", 0.0, 0)
            self.layout = None
        else:
            self.layout = meshgen._sphere_layout(n)
            raw = meshgen.sphere_mesh(n, 0.0, 0)
        perm, groups = M.node_groups_build(raw)
        self.perm = perm
        self.raw = M.permute_mesh(raw, perm)
        self.groups = groups
        self.movable = int(np.count_nonzero(self.raw.cid >= 0))
        self.tets = int(self.raw.tets.shape[0])
        self.device = M.DeviceMesh(self.raw, groups)
        self.device.set_crew(**MR)
        self.bytes = self.device.device_bytes()

    def positions(self, seed: int) -> np.ndarray:
        if self.kind == "cube":
            p = meshgen.box_positions(self.n, 0.3, seed)
        else:
            p = meshgen.sphere_positions(self.n, 0.25, seed, self.layout)
        return np.ascontiguousarray(p[self.perm])


@dataclasses.dataclass
class Job:
    spec: JobSpec
    template: Template
    device: M.DeviceMesh
    admitted: float
    passes: int = 0
    last_min: float = 0.0
    first_min: float = 0.0
    done_at: float | None = None
    final_min: float = 0.0
    final_mean: float = 0.0
    relocations: int = 0
    charged: int = 0  # bytes counted against the budget while the job is active


@dataclasses.dataclass
class ServeStats:
    jobs: int
    relocations: int
    wall_s: float
    busy_s: float
    ticks: int
    latencies_s: list
    peak_active: int
    peak_bytes: int
    results: dict
    phase_s: dict = dataclasses.field(default_factory=dict)  # host time by loop phase

    def summary(self) -> dict:
        lat = np.array(self.latencies_s) if self.latencies_s else np.zeros(1)
        return {"jobs": self.jobs, "relocations": self.relocations, "wall_s": round(self.wall_s, 3),
                "relocations_per_s": self.relocations / max(self.wall_s, 1e-9),
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "ticks": self.ticks, "peak_active_jobs": self.peak_active, "peak_device_bytes": self.peak_bytes,
                "phase_s": {k: round(v, 4) for k, v in self.phase_s.items()}}


class Server:
    def __init__(self, hbm_budget_bytes: int = 64 << 30, max_passes: int = 20, min_gain: float = 1e-3,
                 params: dict | None = None, keep_results: bool = False):
        self.budget = int(hbm_budget_bytes)
        self.max_passes = max_passes
        self.min_gain = min_gain
        self.params = dict(DEFAULT_PARAMS, **(params or {}))
        self.keep_results = keep_results
        self.templates: dict = {}

    def template(self, spec: JobSpec) -> Template:
        key = (spec.kind, spec.n)
        if key not in self.templates:
            self.templates[key] = Template(spec.kind, spec.n)
        return self.templates[key]

    def prepare(self, stream):
        """Build every template the stream needs (topology set-up, not timed)."""
        for s in stream:
            self.template(s)

    def _admit(self, spec: JobSpec, now: float) -> Job:
        t = self.template(spec)
        d = M.DeviceMesh(None, clone_of=t.device)
        d.upload_positions(t.positions(spec.seed))
        q = d.evaluate()
        return Job(spec, t, d, now, last_min=q.minimumQuality(), first_min=q.minimumQuality())

    def run(self, stream: list[JobSpec], realtime: bool = True) -> ServeStats:
        """Serve the stream.  realtime=False admits each job as soon as the
        loop reaches it (arrival times only order the jobs)."""
        pending = collections.deque()
        active: list[Job] = []
        lat, results = [], {}
        relocations, ticks, peak_active, peak_bytes, used = 0, 0, 0, 0, 0
        phase = {"admit_s": 0.0, "batch_setup_s": 0.0, "pass_s": 0.0, "batch_close_s": 0.0, "retire_s": 0.0}
        i = 0
        t0 = time.perf_counter()
        busy = 0.0
        while i < len(stream) or pending or active:
            now = time.perf_counter() - t0
            while i < len(stream) and (not realtime or stream[i].arrival <= now):
                pending.append(stream[i])
                i += 1
            if not active and not pending:
                if realtime and i < len(stream):
                    time.sleep(max(0.0, min(0.01, stream[i].arrival - now)))
                continue
            # admission against the HBM budget
            # (a job is charged its template's footprint on admission and the
            # same amount is released when it retires, so the books balance
            # even though its per-pass buffers grow once it runs)
            ta = time.perf_counter()
            while pending:
                need = self.template(pending[0]).bytes
                if active and used + need > self.budget:
                    break
                job = self._admit(pending.popleft(), time.perf_counter() - t0)
                job.charged = max(need, job.device.device_bytes())
                used += job.charged
                active.append(job)
            phase["admit_s"] += time.perf_counter() - ta
            peak_active = max(peak_active, len(active))
            peak_bytes = max(peak_bytes, used)
            # one pass of every active job: one batch per smoother
            tb = time.perf_counter()
            for sm in SMOOTHERS + ("spawn_search",):
                jobs = [j for j in active if j.spec.smoother == sm]
                if not jobs:
                    continue
                t1 = time.perf_counter()
                b = M.Batch([j.device for j in jobs])
                t2 = time.perf_counter()
                b.smooth_pass(sm, self.params[sm])
                b.evaluate(0)
                qs = b.read_quality(0)
                if b.status() != 0:
                    raise RuntimeError("batched pass reported a dependency timeout")
                t3 = time.perf_counter()
                b.close()
                t4 = time.perf_counter()
                phase["batch_setup_s"] += t2 - t1
                phase["pass_s"] += t3 - t2
                phase["batch_close_s"] += t4 - t3
                for j, q in zip(jobs, qs):
                    j.passes += 1
                    j.relocations += j.template.movable
                    gain = q.minimumQuality() - j.last_min
                    j.last_min = q.minimumQuality()
                    if j.passes >= self.max_passes or gain < self.min_gain:
                        j.done_at = time.perf_counter() - t0
                        j.final_min, j.final_mean = q.minimumQuality(), q.harmonicMean()
            busy += time.perf_counter() - tb
            ticks += 1
            still = []
            tr = time.perf_counter()
            for j in active:
                if j.done_at is None:
                    still.append(j)
                    continue
                relocations += j.relocations
                lat.append(j.done_at - j.spec.arrival if realtime else j.done_at - j.admitted)
                if self.keep_results:
                    results[j.spec.job_id] = {"pos": j.device.fetch_positions(), "passes": j.passes,
                                              "min": j.final_min, "mean": j.final_mean}
                used -= j.charged
                j.device.close()
            phase["retire_s"] += time.perf_counter() - tr
            active = still
        wall = time.perf_counter() - t0
        return ServeStats(len(stream), relocations, wall, busy, ticks, lat, peak_active, peak_bytes, results, phase)
