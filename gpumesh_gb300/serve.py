"""Served smoothing: a continuous request loop over device-resident jobs.

Jobs arrive over time (a Poisson stream).  Each job is a jittered cube or
sphere tet mesh with its own seed and a smoother (Nelder-Mead, gradient
descent or GETMe); it runs relocation passes until its min-quality gain
drops below a threshold or a pass cap is reached (the stop rule of the
served workload; the reference's autopilot compares mean and min gains,
Smoothers/AbstractSmoother.cpp:182-193).

Each job runs as ONE launch of a CUDA graph (gm_job_*): the evaluation,
then a conditional loop of (relocation pass, evaluation, stop test) that the
device drives, on the job's own stream.  Jobs that arrive while others are
on the GPU are admitted as soon as a slot (a stream) and HBM budget are
free, and their kernels overlap with the running jobs' on the device, so a
small job finishes in its own service time instead of waiting for the
passes of larger ones.  The host only admits, launches and polls.

Job meshes come from resident slots: a slot is a device mesh of one
(kind, cells per axis) with its prepared job graph for one smoother, cloned
once from a topology template (connectivity, constraints, colouring built
once per (kind, n)); a job uploads only its own positions into a free slot
of its key.  Finished jobs return their slot to the pool; idle slots are
freed when the HBM budget needs room.
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
        """The job's positions as float32 GpuVert records (x, y, z, 0)."""
        if self.kind == "cube":
            p = meshgen.box_positions(self.n, 0.3, seed)
        else:
            p = meshgen.sphere_positions(self.n, 0.25, seed, self.layout)
        out = np.zeros((p.shape[0], 4), np.float32)
        out[:, :3] = p[self.perm]
        return out


class Slot:
    """A device mesh of one template on its own stream, with the job graph
    of one smoother prepared."""

    def __init__(self, template: Template, smoother: str, params, max_passes: int, min_gain: float):
        import torch

        self.template = template
        self.stream = torch.cuda.Stream()
        self.device = M.DeviceMesh(None, stream=self.stream.cuda_stream, clone_of=template.device)
        self.device.job_prepare(smoother, params, max_passes, min_gain)
        self.bytes = self.device.device_bytes()
        # pinned staging of the job's positions: the upload is asynchronous,
        # and the slot's next job reuses the buffer only after this one ends
        self._pinned = torch.empty((template.raw.nv, 4), dtype=torch.float32, pin_memory=True)
        self.pinned = self._pinned.numpy()

    def launch(self, payload: np.ndarray):
        np.copyto(self.pinned, payload)
        self.device.upload_gpu_verts_async(self.pinned)
        self.device.job_launch()

    def close(self):
        self.device.close()


@dataclasses.dataclass
class Job:
    spec: JobSpec
    slot: Slot
    admitted: float
    done_at: float | None = None


@dataclasses.dataclass
class ServeStats:
    jobs: int
    relocations: int
    wall_s: float
    latencies_s: list
    peak_active: int
    peak_bytes: int
    results: dict
    phase_s: dict = dataclasses.field(default_factory=dict)  # host time by loop phase
    slots_created: int = 0

    def summary(self) -> dict:
        lat = np.array(self.latencies_s) if self.latencies_s else np.zeros(1)
        return {"jobs": self.jobs, "relocations": self.relocations, "wall_s": round(self.wall_s, 3),
                "relocations_per_s": self.relocations / max(self.wall_s, 1e-9),
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "peak_active_jobs": self.peak_active, "peak_device_bytes": self.peak_bytes,
                "slots_created": self.slots_created, "phase_s": {k: round(v, 4) for k, v in self.phase_s.items()}}


class Server:
    def __init__(self, hbm_budget_bytes: int = 64 << 30, max_passes: int = 20, min_gain: float = 1e-3,
                 params: dict | None = None, keep_results: bool = False, max_concurrent: int = 64):
        self.budget = int(hbm_budget_bytes)
        self.max_passes = max_passes
        self.min_gain = min_gain
        self.params = dict(DEFAULT_PARAMS, **(params or {}))
        self.keep_results = keep_results
        self.max_concurrent = max_concurrent
        self.templates: dict = {}
        self.payloads: dict = {}
        self.idle: dict = collections.defaultdict(list)  # (kind, n, smoother) -> [Slot]
        self.idle_order: collections.OrderedDict = collections.OrderedDict()  # Slot -> key, least recent first
        self.used = 0  # device bytes of every slot, busy or idle
        self.slots_created = 0

    def template(self, spec: JobSpec) -> Template:
        key = (spec.kind, spec.n)
        if key not in self.templates:
            self.templates[key] = Template(spec.kind, spec.n)
        return self.templates[key]

    def prepare(self, stream):
        """Build every template and the jobs' input positions (what a client
        would send); not part of serving."""
        for s in stream:
            t = self.template(s)
            self.payloads[s.job_id] = t.positions(s.seed)

    def _take_slot(self, spec: JobSpec, busy: int):
        """A free slot for the job, or None when the budget has no room."""
        key = (spec.kind, spec.n, spec.smoother)
        if self.idle[key]:
            slot = self.idle[key].pop()
            self.idle_order.pop(slot, None)
            return slot
        t = self.template(spec)
        need = t.bytes
        while self.used + need > self.budget and self.idle_order:
            old, okey = self.idle_order.popitem(last=False)  # evict the least recently used idle slot
            self.idle[okey].remove(old)
            self.used -= old.bytes
            old.close()
        if busy and self.used + need > self.budget:
            return None  # wait for running jobs to free memory (an empty GPU always admits)
        slot = Slot(t, spec.smoother, self.params[spec.smoother], self.max_passes, self.min_gain)
        self.used += slot.bytes
        self.slots_created += 1
        return slot

    def _release(self, spec: JobSpec, slot: Slot):
        key = (spec.kind, spec.n, spec.smoother)
        self.idle[key].append(slot)
        self.idle_order[slot] = key

    def run(self, stream: list[JobSpec], realtime: bool = True) -> ServeStats:
        """Serve the stream.  realtime=False admits each job as soon as the
        loop reaches it (arrival times only order the jobs)."""
        pending = collections.deque()
        running: list[Job] = []
        lat, results = [], {}
        relocations, peak_active, peak_bytes = 0, 0, 0
        phase = {"admit_s": 0.0, "poll_s": 0.0, "retire_s": 0.0}
        i = 0
        t0 = time.perf_counter()
        while i < len(stream) or pending or running:
            now = time.perf_counter() - t0
            while i < len(stream) and (not realtime or stream[i].arrival <= now):
                pending.append(stream[i])
                i += 1
            # admission: a free stream slot and room in the HBM budget
            ta = time.perf_counter()
            while pending and len(running) < self.max_concurrent:
                spec = pending[0]
                slot = self._take_slot(spec, len(running))
                if slot is None:
                    break
                pending.popleft()
                payload = self.payloads.get(spec.job_id)
                if payload is None:
                    payload = slot.template.positions(spec.seed)
                slot.launch(payload)
                running.append(Job(spec, slot, time.perf_counter() - t0))
            phase["admit_s"] += time.perf_counter() - ta
            peak_active = max(peak_active, len(running))
            peak_bytes = max(peak_bytes, self.used)
            # completions
            tp = time.perf_counter()
            still = []
            finished = []
            for j in running:
                if j.slot.device.job_done():
                    j.done_at = time.perf_counter() - t0
                    finished.append(j)
                else:
                    still.append(j)
            phase["poll_s"] += time.perf_counter() - tp
            tr = time.perf_counter()
            for j in finished:
                passes, first, last = j.slot.device.job_result()
                relocations += passes * j.slot.template.movable
                lat.append(j.done_at - j.spec.arrival if realtime else j.done_at - j.admitted)
                if self.keep_results:
                    results[j.spec.job_id] = {"pos": j.slot.device.fetch_positions(), "passes": passes,
                                              "min": last.minimumQuality(), "mean": last.harmonicMean()}
                self._release(j.spec, j.slot)
            phase["retire_s"] += time.perf_counter() - tr
            running = still
            if not finished and (not pending or len(running) >= self.max_concurrent):
                time.sleep(50e-6)
        wall = time.perf_counter() - t0
        return ServeStats(len(stream), relocations, wall, lat, peak_active, peak_bytes, results, phase,
                          self.slots_created)

    def close(self):
        for slots in self.idle.values():
            for s in slots:
                s.close()
        self.idle.clear()
        self.idle_order.clear()
        self.used = 0


def run_plain(server: Server, stream: list[JobSpec], realtime: bool = True) -> ServeStats:
    """The plain path under the same stream: one job at a time in arrival
    order, each pass launched from the host (one launch per colour), the
    evaluation read back after every pass for the stop rule.  A device mesh
    per (kind, n) is kept across jobs, so only positions are uploaded."""
    meshes: dict = {}
    lat, relocations, results = [], 0, {}
    t0 = time.perf_counter()
    for spec in stream:
        if realtime:
            wait = spec.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        start = time.perf_counter() - t0
        t = server.template(spec)
        d = meshes.get((spec.kind, spec.n))
        if d is None:
            d = meshes[(spec.kind, spec.n)] = M.DeviceMesh(None, clone_of=t.device)
        payload = server.payloads.get(spec.job_id)
        d.upload_gpu_verts(payload if payload is not None else t.positions(spec.seed))
        last = d.evaluate().minimumQuality()
        passes = 0
        q = None
        for _ in range(server.max_passes):
            d.smooth_pass(spec.smoother, server.params[spec.smoother])
            q = d.evaluate()
            passes += 1
            gain = q.minimumQuality() - last
            last = q.minimumQuality()
            if gain < server.min_gain:
                break
        relocations += passes * t.movable
        done = time.perf_counter() - t0
        lat.append(done - spec.arrival if realtime else done - start)
        if server.keep_results:
            results[spec.job_id] = {"pos": d.fetch_positions(), "passes": passes, "min": q.minimumQuality(),
                                    "mean": q.harmonicMean()}
    wall = time.perf_counter() - t0
    for d in meshes.values():
        d.close()
    return ServeStats(len(stream), relocations, wall, lat, 1, 0, results)
