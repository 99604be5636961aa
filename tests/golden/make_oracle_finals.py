"""Generate tests/golden/finals/*.npz: the FP64 oracle's result of every
benchmark configuration at its full size, the reference point of the GPU
path's error statement.

For each configuration the oracle colours and orders the seeded mesh with
its restatement of NodeGroups::build, then runs the configuration's whole
schedule in colour-major order from the input the GPU path receives (the
positions rounded to FP32), evaluating after every pass.  Stored:

  * the per-pass minimum and harmonic mean;
  * a strided sample of the final vertex positions (about 2048 movable
    vertices) with the mean length of the edges around each, so that a GPU
    run can state its per-vertex position error as a fraction of the local
    mean edge length;
  * the oracle's own spread: the same schedule from that input with every
    free vertex moved by one FP32 rounding step (nextafter, direction drawn
    per coordinate from a seeded stream; three draws), giving how far the
    FP64 algorithm itself moves the final minimum, mean and positions when
    only the input's last bit changes;
  * the FP32-resolution runs: the same schedule by the oracle's measurement
    build (libgm_oracle_q32.so) whose patch qualities are brought to FP32
    resolution -- rounded to FP32 once, then multiplied by seeded draws of
    (1 + u 2^-23), |u| <= 1 -- so that every comparison the smoothers make
    (candidate against candidate, a quality gain against a stop threshold)
    sees differences below FP32 resolution resolved one way or the other.
    Where a decision rests on such a difference the runs part ways and
    later colours carry the difference on: the set of their results is the
    set of outcomes the reference algorithm has at FP32 resolution.

C4 is sampled: every 256th of its 4,096 meshes (16 meshes), one Nelder-Mead
pass each.  Eight FP32-resolution draws per configuration (three for C2,
whose runs take minutes each).

Run from the repo root (CPU only; C2 takes a few minutes per run):

    python tests/golden/make_oracle_finals.py [C1 C2 C3 C3m C4]
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "finals")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
from gpumesh_gb300 import meshgen, workloads  # noqa: E402

THREADS = os.cpu_count() or 1
SAMPLES = 2048
PERTURB_SEEDS = (101, 102, 103)
FP32_DRAWS = {"C2": 3}
DEFAULT_FP32_DRAWS = 8

TET_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))
PRI_EDGES = ((0, 1), (0, 2), (1, 2), (0, 3), (1, 4), (2, 5), (3, 4), (3, 5), (4, 5))
HEX_EDGES = ((0, 1), (0, 3), (1, 2), (2, 3), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (4, 7), (5, 6), (6, 7))


def mean_edge_length(raw, pos):
    """Mean length of the edges around each vertex."""
    pairs = []
    for E, edges in ((raw.tets, TET_EDGES), (raw.pris, PRI_EDGES), (raw.hexs, HEX_EDGES)):
        if E.shape[0]:
            for a, b in edges:
                pairs.append(np.stack([E[:, a], E[:, b]], axis=1))
    e = np.unique(np.sort(np.concatenate(pairs).astype(np.int64), axis=1), axis=0)
    L = np.linalg.norm(pos[e[:, 0]] - pos[e[:, 1]], axis=1)
    s = np.bincount(e[:, 0], L, raw.nv) + np.bincount(e[:, 1], L, raw.nv)
    c = np.bincount(e[:, 0], None, raw.nv) + np.bincount(e[:, 1], None, raw.nv)
    return s / np.maximum(c, 1)


def fp32_input(pos):
    return pos.astype(np.float32).astype(np.float64)


def perturbed(raw, pos32, seed):
    """Every free vertex's FP32 coordinates moved by one rounding step."""
    p = pos32.astype(np.float32)
    free = raw.cid == 0
    u = meshgen.uniform(seed, 0, p.size).reshape(p.shape)
    up = np.nextafter(p, np.float32(np.inf))
    down = np.nextafter(p, np.float32(-np.inf))
    q = np.where(u < 0.5, down, up)
    p[free] = q[free]
    return p.astype(np.float64)


def run(raw, crew, schedule, pos, variant="", seed=0):
    """The schedule from `pos`, evaluating before and after every pass (with
    the FP64 oracle's evaluator whatever the variant; `seed` selects the
    FP32-resolution draw of the q32 build)."""
    if variant == "q32":
        pyoracle.set_fp32_resolution_seed(seed)
    m = pyoracle.OracleMesh.from_raw(raw, **crew, variant=variant)
    m.pos = pos
    perm_base, members = raw._groups
    hist = []
    e = m.evaluate(nthreads=THREADS)
    hist.append((e["min"], e["mean"]))
    for smoother, passes, params in schedule:
        for _ in range(passes):
            m.smooth_pass(smoother, perm_base, members, params=params, nthreads=THREADS)
            e = m.evaluate(nthreads=THREADS)
            hist.append((e["min"], e["mean"]))
    out = m.pos
    m.close()
    if variant:
        hist = []
        chk = pyoracle.OracleMesh.from_raw(raw, **crew)
        chk.pos = out
        e = chk.evaluate(nthreads=THREADS)
        chk.close()
        return np.array([(e["min"], e["mean"])]), out
    return np.array(hist), out


def coloured(raw):
    perm, base, members, ranges = pyoracle.node_groups_build(raw)
    pr = pyoracle.permute(raw, perm)
    pr._groups = (base, members)
    return pr


def make_one(raw, crew, schedule, draws=DEFAULT_FP32_DRAWS):
    pos32 = fp32_input(raw.pos)
    hist, final = run(raw, crew, schedule, pos32)
    movable = np.flatnonzero(raw.cid >= 0)
    idx = movable[:: max(1, movable.size // SAMPLES)]
    out = dict(hist=hist, final_min=hist[-1, 0], final_mean=hist[-1, 1], sample_idx=idx.astype(np.int64),
               sample_pos=final[idx], sample_edge=mean_edge_length(raw, final)[idx], nv=raw.nv)
    spreads = []
    for s in PERTURB_SEEDS:
        h2, f2 = run(raw, crew, schedule, perturbed(raw, pos32, s))
        spreads.append((abs(h2[-1, 0] - hist[-1, 0]), abs(h2[-1, 1] - hist[-1, 1]),
                        float(np.max(np.linalg.norm(f2[idx] - final[idx], axis=1) / out["sample_edge"]))))
    sp = np.array(spreads)
    out.update(spread_min=sp[:, 0].max(), spread_mean=sp[:, 1].max(), spread_pos=sp[:, 2].max(), spreads=sp)
    fmin, fmean, fpos = [], [], []
    for seed in range(draws + 1):
        hq, fq = run(raw, crew, schedule, pos32, variant="q32", seed=seed)
        fmin.append(hq[-1, 0])
        fmean.append(hq[-1, 1])
        fpos.append(float(np.max(np.linalg.norm(fq[idx] - final[idx], axis=1) / out["sample_edge"])))
    fmin, fmean = np.array(fmin), np.array(fmean)
    out.update(fp32_min=fmin, fp32_mean=fmean, q32_min=fmin[0], q32_mean=fmean[0],
               q32_dmin=float(np.abs(fmin - hist[-1, 0]).max()), q32_dmean=float(np.abs(fmean - hist[-1, 1]).max()),
               q32_dpos=float(max(fpos)))
    return out


def make_config(name):
    t0 = time.time()
    os.makedirs(OUT, exist_ok=True)
    if name == "C4":
        sizes = meshgen.batch_sizes(4096, 4, 24, 3)
        picks = list(range(0, 4096, 256))
        rows, fmins, fmeans = [], [], []
        for i in picks:
            raw = coloured(meshgen.box_mesh(int(sizes[i]), "tet", 0.3, 3 * 1000003 + i))
            o = make_one(raw, dict(sampler="uniform", measurer="metric_free", evaluator="mean_ratio"),
                         [("nelder_mead", 1, workloads.NM_PARAMS)])
            rows.append((i, int(sizes[i]), o["final_min"], o["final_mean"], o["spread_min"], o["spread_mean"],
                         o["spread_pos"], o["q32_min"], o["q32_mean"]))
            fmins.append(o["fp32_min"])
            fmeans.append(o["fp32_mean"])
        np.savez_compressed(os.path.join(OUT, "C4.npz"), rows=np.array(rows, np.float64),
                            fp32_min=np.array(fmins), fp32_mean=np.array(fmeans),
                            columns=np.array(["mesh", "cells", "final_min", "final_mean", "spread_min",
                                              "spread_mean", "spread_pos", "q32_min", "q32_mean"]))
    else:
        w = workloads.WORKLOADS[name]
        raw = coloured(w.mesh())
        o = make_one(raw, w.crew(raw), w.schedule, FP32_DRAWS.get(name, DEFAULT_FP32_DRAWS))
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **o)
        print(name, "final", o["final_min"], o["final_mean"], "spread", o["spread_min"], o["spread_mean"],
              o["spread_pos"], "fp32 draws min", np.round(o["fp32_min"], 7), "mean", np.round(o["fp32_mean"], 7),
              flush=True)
    print(f"wrote {name} in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    for n in (sys.argv[1:] or ["C1", "C4", "C3", "C3m", "C2"]):
        make_config(n)
