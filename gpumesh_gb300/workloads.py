"""The five benchmark workloads as concrete seeded meshes, crews and schedules.

  C1  10^3-cell cube, 6 Kuhn tets per cell (6,000 tets, 1,331 vertices), interior
      jitter U(+-0.3h), seed 0; BoxBoundary; metric-free mean ratio; one
      Nelder-Mead pass (initial simplex 0.1 x local edge length, at most 64
      iterations per vertex: 32 cycles, then 32 more after the restart).
  C2  80^3-cell grid clipped to the unit ball (~1.6M tets), interior jitter
      U(+-0.25h), seed 1; SphereBoundary; metric-wise measurer with the metric
      s^2 diag(1 + 9 sin^2(4 pi x), 1, 1), s = 1/h, and metric conformity;
      five gradient-descent passes (step 0.01 x local edge length), then five
      spawn-search passes (64 candidates).
  C3  128^3 hexes (2,097,152 hexes, 2,146,689 vertices), interior Gaussian
      noise sigma = 0.15h, seed 2; BoxBoundary; metric-free mean ratio; ten
      GETMe passes with lambda = 0.5.  C3m: the same grid as tet / prism /
      hex z-slabs.
  C4  4,096 jittered tet cubes, cells per axis log-uniform in [4, 24], jitter
      U(+-0.3h), seed 3; one Nelder-Mead pass each.
"""

from __future__ import annotations

import dataclasses

from . import meshgen

NM_PARAMS = [0.1, 32, 1e-4, 1.0, 0.5, 2.0]
GD_PARAMS = [0.01, 5]
SPAWN_PARAMS = [1.0 / 20.0, 2]
GETME_PARAMS = [0.5]


@dataclasses.dataclass
class Workload:
    name: str
    build: object          # () -> RawMesh
    sampler: str
    measurer: str
    evaluator: str
    scaling: object        # float or (RawMesh) -> float
    schedule: list         # [(smoother, passes, params)]

    def mesh(self):
        return self.build()

    def crew(self, raw):
        s = self.scaling(raw) if callable(self.scaling) else self.scaling
        return dict(sampler=self.sampler, measurer=self.measurer, evaluator=self.evaluator, scaling=s)

    def passes(self) -> int:
        return sum(p for _, p, _ in self.schedule)


WORKLOADS = {
    "C1": Workload("C1 tet cube 10^3 x6, NM 1 pass", lambda: meshgen.box_mesh(10, "tet", 0.3, 0),
                   "uniform", "metric_free", "mean_ratio", 1.0, [("nelder_mead", 1, NM_PARAMS)]),
    "C2": Workload("C2 sphere 80^3 clipped tets, MC sine metric, GD x5 + spawn x5",
                   lambda: meshgen.sphere_mesh(80, 0.25, 1), "sine", "metric_wise", "metric_conformity",
                   lambda raw: 1.0 / raw.h, [("gradient_descent", 5, GD_PARAMS), ("spawn_search", 5, SPAWN_PARAMS)]),
    "C3": Workload("C3 hex cube 128^3, GETMe x10", lambda: meshgen.box_mesh(128, "hex", 0.15, 2, gaussian=True),
                   "uniform", "metric_free", "mean_ratio", 1.0, [("getme", 10, GETME_PARAMS)]),
    "C3m": Workload("C3m mixed tet/prism/hex 128^3, GETMe x10",
                    lambda: meshgen.box_mesh(128, "mixed", 0.15, 2, gaussian=True),
                    "uniform", "metric_free", "mean_ratio", 1.0, [("getme", 10, GETME_PARAMS)]),
}


def small(name: str, n: int):
    """A reduced copy of a workload on an n^3 grid (for parity tests)."""
    w = WORKLOADS[name]
    if name == "C2":
        b = lambda: meshgen.sphere_mesh(n, 0.25, 1)
    elif name == "C1":
        b = lambda: meshgen.box_mesh(n, "tet", 0.3, 0)
    elif name == "C3":
        b = lambda: meshgen.box_mesh(n, "hex", 0.15, 2, gaussian=True)
    else:
        b = lambda: meshgen.box_mesh(n, "mixed", 0.15, 2, gaussian=True)
    return dataclasses.replace(w, name=f"{w.name} (n={n})", build=b)
