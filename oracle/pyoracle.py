"""ctypes binding of the FP64 CPU oracle (oracle/gm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py as the checker.  The product package never imports it.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgm_oracle.so")

SAMPLER = {"uniform": 0, "analytic": 1, "sine": 2, "local": 3, "kdtree": 4, "texture": 5}
MEASURER = {"metric_free": 0, "metric_wise": 1}
EVALUATOR = {"mean_ratio": 0, "metric_conformity": 1}
SMOOTHER = {"nelder_mead": 0, "gradient_descent": 1, "spawn_search": 2, "getme": 3, "spring_laplace": 4,
            "quality_laplace": 5}

# Reference constants (Smoothers/VertexWise/NelderMeadSmoother.cpp:17-23,
# GradientDescentSmoother.cpp:14-15, SpawnSearchSmoother.cpp:14 and :181,
# GetmeSmoother.cpp:22, SpringLaplaceSmoother.cpp:10, QualityLaplaceSmoother.cpp:12)
REFERENCE_PARAMS = {
    "nelder_mead": [1.0 / 24.0, 12, 1e-4, 1.0, 0.5, 2.0],
    "gradient_descent": [1.0 / 75.0, 5],
    "spawn_search": [1.0 / 20.0, 2],
    "getme": [0.78],
    "spring_laplace": [0.35],
    "quality_laplace": [0.35],
}


def lib_path(variant: str = "") -> str:
    """The oracle library; variant "q32" is the measurement build whose patch
    qualities are rounded to FP32 (OM_PATCH_QUALITY_FP32 in gm_oracle.c)."""
    return LIB_PATH if not variant else os.path.join(BUILD_DIR, f"libgm_oracle_{variant}.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gm_oracle.c")
    sort_src = os.path.join(HERE, "om_sort.cpp")
    newest = max(os.path.getmtime(src), os.path.getmtime(sort_src), os.path.getmtime(os.path.join(HERE, "gm_oracle.h")))
    flags = ["-O2", "-ffp-contract=off", "-fPIC"]
    for variant, defs in (("", []), ("q32", ["-DOM_PATCH_QUALITY_FP32"])):
        path = lib_path(variant)
        if force or not os.path.exists(path) or os.path.getmtime(path) < newest:
            os.makedirs(BUILD_DIR, exist_ok=True)
            tag = variant or "fp64"
            obj_c = os.path.join(BUILD_DIR, f"gm_oracle_{tag}.o")
            obj_s = os.path.join(BUILD_DIR, "om_sort.o")
            subprocess.check_call(["gcc", *flags, *defs, "-c", src, "-o", obj_c])
            subprocess.check_call(["g++", *flags, "-std=c++17", "-c", sort_src, "-o", obj_s])
            subprocess.check_call(["g++", "-shared", "-o", path, obj_c, obj_s, "-lm", "-lpthread"])
    return LIB_PATH


_libs: dict = {}


def lib(variant: str = ""):
    if variant not in _libs:
        build()
        L = ctypes.CDLL(lib_path(variant))
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.om_create.restype = vp
        L.om_create.argtypes = [i64, vp, i64, vp, i64, vp, i64, vp, vp]
        L.om_destroy.argtypes = [vp]
        L.om_set_constraints.argtypes = [vp, i32, vp, vp]
        L.om_set_crew.argtypes = [vp, i32, i32, i32, dbl, dbl]
        L.om_set_discretization_depth.argtypes = [vp, i32]
        L.om_get_pos.argtypes = [vp, vp]
        L.om_set_pos.argtypes = [vp, vp]
        L.om_element_quality.restype = dbl
        L.om_element_quality.argtypes = [vp, i32, i64]
        L.om_patch_quality.restype = dbl
        L.om_patch_quality.argtypes = [vp, i64]
        L.om_local_size.restype = dbl
        L.om_local_size.argtypes = [vp, i64]
        L.om_project.argtypes = [vp, i64, vp, vp]
        L.om_metric_at.argtypes = [vp, vp, vp]
        L.om_riemannian_distance.restype = dbl
        L.om_riemannian_distance.argtypes = [vp, vp, vp]
        L.om_evaluate.argtypes = [vp, vp, i32]
        L.om_smooth_pass.argtypes = [vp, i32, vp, i64, vp, vp, i32]
        L.om_patch_eval_count.restype = i64
        L.om_patch_eval_count.argtypes = [vp]
        L.om_reset_patch_eval_count.argtypes = [vp]
        L.om_node_groups_build.restype = i64
        L.om_node_groups_build.argtypes = [vp, vp, vp, vp, vp]
        if variant == "q32":
            L.om_set_fp32_resolution_seed.argtypes = [ctypes.c_uint64]
        _libs[variant] = L
    return _libs[variant]


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_fp32_resolution_seed(seed: int):
    """The measurement build's mode (libgm_oracle_q32.so): 0 = patch
    qualities rounded to FP32, s > 0 = multiplied by a seeded draw of
    (1 + u 2^-23), |u| <= 1."""
    lib("q32").om_set_fp32_resolution_seed(int(seed))


def permute(raw, perm: np.ndarray):
    """The mesh with its vertices in NodeGroups' order (perm[new] = old), as
    NodeGroups::clusterNodes renumbers it (DataStructures/NodeGroups.cpp:452-514)."""
    import dataclasses

    new_of_old = np.empty_like(perm)
    new_of_old[perm] = np.arange(perm.size, dtype=perm.dtype)
    return dataclasses.replace(raw, pos=np.ascontiguousarray(raw.pos[perm]),
                               tets=new_of_old[raw.tets].astype(np.uint32),
                               pris=new_of_old[raw.pris].astype(np.uint32),
                               hexs=new_of_old[raw.hexs].astype(np.uint32),
                               cid=np.ascontiguousarray(raw.cid[perm]))


def node_groups_build(raw):
    """NodeGroups::build by the oracle: (perm, group_base, members, ranges)."""
    m = OracleMesh.from_raw(raw)
    try:
        return m.node_groups()
    finally:
        m.close()


class OracleMesh:
    """FP64 CPU mesh: arrays in, smoothing / evaluation by the oracle."""

    def __init__(self, pos, tets, pris, hexs, cid, con_kind, con_param,
                 sampler="uniform", measurer="metric_free", evaluator="mean_ratio",
                 scaling=1.0, aspect_ratio=1.0, depth=-1, variant: str = ""):
        self._L = L = lib(variant)
        self._keep = [np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(tets, np.uint32),
                      np.ascontiguousarray(pris, np.uint32), np.ascontiguousarray(hexs, np.uint32),
                      np.ascontiguousarray(cid, np.int32)]
        p, t, r, h, c = self._keep
        self.nv = p.shape[0]
        self.h = L.om_create(self.nv, _p(p), t.shape[0], _p(t), r.shape[0], _p(r), h.shape[0], _p(h), _p(c))
        ck = np.ascontiguousarray(con_kind, np.int32)
        cp = np.ascontiguousarray(con_param, np.float64).reshape(-1, 6)
        L.om_set_constraints(self.h, ck.shape[0], _p(ck), _p(cp))
        L.om_set_discretization_depth(self.h, int(depth))
        L.om_set_crew(self.h, SAMPLER[sampler], MEASURER[measurer], EVALUATOR[evaluator],
                      float(scaling), float(aspect_ratio))

    @classmethod
    def from_raw(cls, raw, **crew):
        return cls(raw.pos, raw.tets, raw.pris, raw.hexs, raw.cid, raw.con_kind, raw.con_param, **crew)

    def close(self):
        if self.h:
            self._L.om_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def pos(self) -> np.ndarray:
        out = np.empty((self.nv, 3), np.float64)
        self._L.om_get_pos(self.h, _p(out))
        return out

    @pos.setter
    def pos(self, value):
        v = np.ascontiguousarray(value, np.float64)
        self._L.om_set_pos(self.h, _p(v))

    def element_quality(self, etype: int, idx: int) -> float:
        return self._L.om_element_quality(self.h, etype, idx)

    def patch_quality(self, v: int) -> float:
        return self._L.om_patch_quality(self.h, v)

    def local_size(self, v: int) -> float:
        return self._L.om_local_size(self.h, v)

    def project(self, v: int, p) -> np.ndarray:
        a = np.ascontiguousarray(p, np.float64)
        out = np.empty(3, np.float64)
        self._L.om_project(self.h, v, _p(a), _p(out))
        return out

    def metric_at(self, p) -> np.ndarray:
        a = np.ascontiguousarray(p, np.float64)
        out = np.empty(9, np.float64)
        self._L.om_metric_at(self.h, _p(a), _p(out))
        return out.reshape(3, 3)  # row c = column c of the GLM matrix

    def evaluate(self, nthreads: int = 1) -> dict:
        out = np.zeros(23, np.float64)
        self._L.om_evaluate(self.h, _p(out), nthreads)
        count = out[2]
        return {"min": out[0], "inv_sum": out[1], "count": int(count),
                "mean": (count / out[1]) if out[1] != 0 else float("nan"),
                "buckets": out[3:].astype(np.int64)}

    def smooth_pass(self, smoother: str, group_base, members, params=None, nthreads: int = 1):
        prm = np.zeros(8, np.float64)
        src = REFERENCE_PARAMS[smoother] if params is None else params
        prm[:len(src)] = src
        gb = np.ascontiguousarray(group_base, np.int64)
        mb = np.ascontiguousarray(members, np.uint32)
        self._L.om_smooth_pass(self.h, SMOOTHER[smoother], _p(prm), gb.shape[0] - 1, _p(gb), _p(mb), nthreads)

    def node_groups(self):
        """NodeGroups::build on this mesh: (perm, group_base, members, ranges)
        with perm[new] = input vertex, the colour-major groups of the
        permuted mesh and their boundary / subsurface / interior ranges."""
        perm = np.zeros(self.nv, np.uint32)
        base = np.zeros(self.nv + 1, np.int64)
        members = np.zeros(self.nv, np.uint32)
        ranges = np.zeros(6 * self.nv, np.int64)
        n = self._L.om_node_groups_build(self.h, _p(perm), _p(base), _p(members), _p(ranges))
        return perm, base[:n + 1].copy(), members[:base[n]].copy(), ranges[:6 * n].reshape(-1, 6).copy()

    @property
    def patch_evals(self) -> int:
        return self._L.om_patch_eval_count(self.h)

    def reset_patch_evals(self):
        self._L.om_reset_patch_eval_count(self.h)
