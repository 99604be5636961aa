"""ctypes binding of oracle/_ref/libgmref.so: the reference's own CPU code.

TEST INFRASTRUCTURE ONLY (the checker of the checker): built from the
reference tree by oracle/refbuild.py where that tree exists.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

import refbuild

BOUNDARY = {"free": 0, "box": 1, "sphere": 2, "tet": 3, "pipe": 4, "shell": 5}
SMOOTHER = {"nelder_mead": 0, "gradient_descent": 1, "spawn_search": 2, "getme": 3, "spring_laplace": 4,
            "quality_laplace": 5}
SAMPLER = {"uniform": 0, "analytic": 1, "sine": 2, "local": 3, "kdtree": 4, "texture": 5}
EVALUATOR = {"mean_ratio": 0, "metric_conformity": 1}

_lib = None


def available() -> bool:
    return os.path.exists(refbuild.LIB) or refbuild.available()


def lib():
    global _lib
    if _lib is None:
        path = refbuild.build()
        L = ctypes.CDLL(path)
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.ref_create.restype = vp
        cp = ctypes.c_char_p
        L.ref_json_write.restype = i32
        L.ref_json_write.argtypes = [cp, cp, i32, i64, vp, vp, i64, vp, i64, vp, i64, vp]
        L.ref_json_read.restype = vp
        L.ref_json_read.argtypes = [cp]
        L.ref_json_counts.argtypes = [vp, vp]
        L.ref_json_get.argtypes = [vp, vp, vp, vp, vp, vp, vp, i64, vp, i64]
        L.ref_json_destroy.argtypes = [vp]
        L.ref_boundary_project.argtypes = [i32, i32, i64, vp, vp]
        L.ref_create.argtypes = [i32, i64, vp, vp, i64, vp, i64, vp, i64, vp]
        L.ref_destroy.argtypes = [vp]
        L.ref_get_perm.argtypes = [vp, vp]
        L.ref_ngroups.restype = i64
        L.ref_ngroups.argtypes = [vp]
        L.ref_get_groups.argtypes = [vp, vp, vp, vp]
        L.ref_get_tets.argtypes = [vp, vp]
        L.ref_set_crew.argtypes = [vp, i32, i32, dbl, dbl, i32]
        L.ref_evaluate.argtypes = [vp, i32, vp]
        L.ref_element_quality.restype = dbl
        L.ref_element_quality.argtypes = [vp, i32, i64]
        L.ref_patch_quality.restype = dbl
        L.ref_patch_quality.argtypes = [vp, i64]
        L.ref_local_size.restype = dbl
        L.ref_local_size.argtypes = [vp, i64]
        L.ref_smooth.argtypes = [vp, i32, i32]
        L.ref_get_pos.argtypes = [vp, vp]
        L.ref_set_pos.argtypes = [vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefMesh:
    """The reference's Mesh after compileTopology (vertices permuted by NodeGroups)."""

    def __init__(self, raw, boundary: str):
        L = lib()
        self._keep = [np.ascontiguousarray(raw.pos, np.float64), np.ascontiguousarray(raw.cid, np.int32),
                      np.ascontiguousarray(raw.tets, np.uint32), np.ascontiguousarray(raw.pris, np.uint32),
                      np.ascontiguousarray(raw.hexs, np.uint32)]
        p, c, t, r, h = self._keep
        self.nv = p.shape[0]
        self.h = L.ref_create(BOUNDARY[boundary], self.nv, _p(p), _p(c), t.shape[0], _p(t), r.shape[0], _p(r),
                              h.shape[0], _p(h))

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def perm(self) -> np.ndarray:
        out = np.zeros(self.nv, np.uint32)
        lib().ref_get_perm(self.h, _p(out))
        return out

    def groups(self):
        n = lib().ref_ngroups(self.h)
        base = np.zeros(n + 1, np.int64)
        members = np.zeros(self.nv, np.uint32)
        ranges = np.zeros(6 * n, np.int64)
        lib().ref_get_groups(self.h, _p(base), _p(members), _p(ranges))
        return base, members[:base[-1]].copy(), ranges.reshape(-1, 6)

    def set_crew(self, sampler="uniform", evaluator="mean_ratio", scaling=1.0, aspect_ratio=1.0, depth=-1):
        lib().ref_set_crew(self.h, SAMPLER[sampler], EVALUATOR[evaluator], float(scaling), float(aspect_ratio),
                           int(depth))

    def evaluate(self, thread: bool = False) -> dict:
        out = np.zeros(23, np.float64)
        lib().ref_evaluate(self.h, int(thread), _p(out))
        return {"min": out[0], "inv_sum": out[1], "count": int(out[2]), "buckets": out[3:].astype(np.int64)}

    def element_quality(self, etype: int, idx: int) -> float:
        return lib().ref_element_quality(self.h, etype, idx)

    def patch_quality(self, v: int) -> float:
        return lib().ref_patch_quality(self.h, v)

    def local_size(self, v: int) -> float:
        return lib().ref_local_size(self.h, v)

    def smooth(self, smoother: str, passes: int = 1):
        lib().ref_smooth(self.h, SMOOTHER[smoother], passes)

    @property
    def pos(self) -> np.ndarray:
        out = np.zeros((self.nv, 3), np.float64)
        lib().ref_get_pos(self.h, _p(out))
        return out

    @pos.setter
    def pos(self, v):
        a = np.ascontiguousarray(v, np.float64)
        lib().ref_set_pos(self.h, _p(a))


def json_write(path: str, raw, boundary: str, model: str = "") -> None:
    """The reference's JsonSerializer on the mesh as given (no permutation)."""
    p = np.ascontiguousarray(raw.pos, np.float64)
    c = np.ascontiguousarray(raw.cid, np.int32)
    t, r, h = (np.ascontiguousarray(a, np.uint32) for a in (raw.tets, raw.pris, raw.hexs))
    ok = lib().ref_json_write(path.encode(), model.encode(), BOUNDARY[boundary], p.shape[0], _p(p), _p(c),
                              t.shape[0], _p(t), r.shape[0], _p(r), h.shape[0], _p(h))
    if not ok:
        raise OSError(f"reference JsonSerializer could not write {path}")


def json_read(path: str) -> dict:
    """The reference's JsonDeserializer: positions, constraint ids,
    connectivity, model and boundary names."""
    L = lib()
    h = L.ref_json_read(path.encode())
    if not h:
        raise OSError(f"reference JsonDeserializer could not read {path}")
    try:
        n = np.zeros(5, np.int64)
        L.ref_json_counts(h, _p(n))
        pos = np.zeros((n[0], 3), np.float64)
        cid = np.zeros(n[1], np.int32)
        tets = np.zeros((n[2], 4), np.uint32)
        pris = np.zeros((n[3], 6), np.uint32)
        hexs = np.zeros((n[4], 8), np.uint32)
        model = ctypes.create_string_buffer(4096)
        bound = ctypes.create_string_buffer(256)
        L.ref_json_get(h, _p(pos), _p(cid), _p(tets), _p(pris), _p(hexs), model, 4096, bound, 256)
        return dict(pos=pos, cid=cid, tets=tets, pris=pris, hexs=hexs, model=model.value.decode(),
                    boundary=bound.value.decode())
    finally:
        L.ref_json_destroy(h)


def boundary_project(boundary: str, cid: int, pts: np.ndarray) -> np.ndarray:
    """The reference boundary's constraint `cid` applied to each point."""
    p = np.ascontiguousarray(pts, np.float64)
    out = np.zeros_like(p)
    lib().ref_boundary_project(BOUNDARY[boundary], int(cid), p.shape[0], _p(p), _p(out))
    return out
