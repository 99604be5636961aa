"""ctypes binding of libgpumesh_gb300.so (include/gpumesh_gb300.h).

The library is built in-tree by gpumesh_gb300.build; importing this module
without it raises, so nothing silently falls back to a CPU path.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

GM_OK = 0
STATUS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "unsupported",
          5: "timeout", 6: "invalid state"}

SAMPLERS = {"uniform": 0, "analytic": 1, "sine": 2, "local": 3, "kdtree": 4, "texture": 5}
MEASURERS = {"metric_free": 0, "metric_wise": 1}
EVALUATORS = {"mean_ratio": 0, "metric_conformity": 1}
SMOOTHERS = {"nelder_mead": 0, "gradient_descent": 1, "spawn_search": 2, "getme": 3, "spring_laplace": 4,
             "quality_laplace": 5}


class GpuMeshError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Quality(ctypes.Structure):
    _fields_ = [("min", ctypes.c_double), ("inv_sum", ctypes.c_double), ("count", ctypes.c_uint64),
                ("nbad", ctypes.c_uint64), ("buckets", ctypes.c_uint64 * 20)]


_lib = None


def library_path() -> str:
    """The library this process loads: the bounds-checked build when the
    environment sets GPUMESH_GB300_LIB=checked, else the ordinary one."""
    return _build.LIB_CHECKED if os.environ.get("GPUMESH_GB300_LIB") == "checked" else _build.LIB


def lib():
    """Load the native library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m gpumesh_gb300.build` "
                          "(or __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp, u32, i32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64
    L.gm_last_error.restype = ctypes.c_char_p
    L.gm_version.restype = ctypes.c_char_p
    sigs = {
        "gm_node_groups_build": [u32, vp, u32, vp, u32, vp, u32, vp, i32, vp, vp, vp, vp, vp],
        "gm_node_groups_build_device": [u32, vp, u32, vp, u32, vp, u32, vp, i32, vp, vp, vp, vp, vp],
        "gm_mesh_neighbourhoods": [u32, u32, vp, u32, vp, u32, vp, vp, vp, vp, vp, vp, vp],
        "gm_mesh_create": [ctypes.POINTER(vp)],
        "gm_mesh_destroy": [vp],
        "gm_mesh_set_stream": [vp, vp],
        "gm_mesh_sync": [vp],
        "gm_mesh_upload": [vp, u32, vp, vp, u32, vp, u32, vp, u32, vp],
        "gm_mesh_upload_verts": [vp, u32, vp],
        "gm_mesh_upload_gpu_verts": [vp, u32, vp],
        "gm_mesh_upload_tets": [vp, u32, vp, u32],
        "gm_mesh_upload_pris": [vp, u32, vp, u32],
        "gm_mesh_upload_hexs": [vp, u32, vp, u32],
        "gm_mesh_upload_topo": [vp, u32, vp, u32, vp, u32, vp],
        "gm_mesh_upload_groups": [vp, u32, vp, u32, vp],
        "gm_mesh_set_constraints": [vp, u32, vp, vp],
        "gm_mesh_set_crew": [vp, i32, i32, i32, ctypes.c_double, ctypes.c_double],
        "gm_mesh_fetch_verts": [vp, u32, vp],
        "gm_mesh_fetch_gpu_verts": [vp, u32, vp],
        "gm_evaluate": [vp, ctypes.POINTER(Quality)],
        "gm_evaluate_async": [vp, u32],
        "gm_quality_read": [vp, u32, ctypes.POINTER(Quality)],
        "gm_smooth_group": [vp, i32, vp, u32, u32],
        "gm_smooth_pass": [vp, i32, vp],
        "gm_getme_elements": [vp, vp],
        "gm_getme_update_group": [vp, vp, u32, u32],
        "gm_mesh_counters": [vp, vp, i32],
        "gm_mesh_save_positions": [vp],
        "gm_mesh_clone": [vp, vp],
        "gm_mesh_build_local_background": [vp],
        "gm_mesh_set_local_background": [vp, u32, vp, u32, vp, vp],
        "gm_mesh_set_discretization_depth": [vp, i32],
        "gm_mesh_set_kd_nodes": [vp, u32, vp, vp, vp],
        "gm_mesh_set_texture": [vp, vp, vp, vp, vp],
        "gm_mesh_device_bytes": [vp, ctypes.POINTER(u64)],
        "gm_mesh_restore_positions": [vp],
        "gm_probe_fp32_tflops": [ctypes.POINTER(ctypes.c_double)],
        "gm_launch_count": [ctypes.POINTER(ctypes.c_uint64)],
        "gm_mesh_fetch_gpu_verts_range": [vp, u32, u32, vp],
        "gm_bounds_checked": [ctypes.POINTER(ctypes.c_int32)],
        "gm_mesh_bounds_status": [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)],
        "gm_mesh_upload_gpu_verts_range": [vp, u32, u32, vp],
        "gm_batch_create": [ctypes.POINTER(vp), vp, u32],
        "gm_batch_destroy": [vp],
        "gm_batch_stream": [vp, ctypes.POINTER(vp)],
        "gm_batch_sync": [vp],
        "gm_batch_set_config": [vp, i32, i32],
        "gm_batch_tune": [vp, i32, vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_double)],
        "gm_batch_smooth_pass": [vp, i32, vp],
        "gm_batch_evaluate": [vp, u32],
        "gm_batch_read_quality": [vp, u32, vp],
        "gm_batch_capture_pass": [vp, i32, vp, i32],
        "gm_batch_replay": [vp],
        "gm_batch_status": [vp],
        "gm_batch_set_spin_limit": [vp, u64],
        "gm_batch_inject_stall": [vp, u32],
        "gm_batch_counters": [vp, vp, i32],
        "gm_batch_info": [vp, vp],
        "gm_mesh_upload_gpu_verts_async": [vp, u32, vp],
        "gm_job_prepare": [vp, i32, vp, u32, ctypes.c_double],
        "gm_job_launch": [vp],
        "gm_job_query": [vp, vp],
        "gm_job_result": [vp, vp, vp, vp],
        "gm_batch_latencies": [vp, vp],
        "gm_evaluate_noalloc": [u32, vp, u32, vp, u32, vp, u32, vp, i32, i32, i32, ctypes.c_double,
                                ctypes.c_double, vp, vp],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    _lib = L
    return L


def check(status: int):
    if status != GM_OK:
        msg = lib().gm_last_error().decode(errors="replace")
        raise GpuMeshError(status, msg)


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def params_array(values) -> np.ndarray | None:
    if values is None:
        return None
    p = np.zeros(8, np.float64)
    p[:len(values)] = values
    return p
