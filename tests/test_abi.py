"""The C ABI library loads and exports every function include/*.h declares
(no compute calls: this runs without a GPU)."""

import ctypes
import glob
import os
import re

import pytest

from gpumesh_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"^\s*(?:gm_status|const char\*)\s+(gm_\w+)\s*\(", text, re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(B.LIB):
        B.build()
    return ctypes.CDLL(B.LIB)


def test_header_declares_entry_points():
    names = declared()
    assert "gm_evaluate" in names and "gm_smooth_pass" in names and len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_strings(lib):
    lib.gm_version.restype = ctypes.c_char_p
    lib.gm_status_string.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.gm_version()
    assert lib.gm_status_string(1) == b"invalid argument"


def test_host_validation_rejects_bad_input_without_gpu(lib):
    # gm_node_groups_build is host-only: an out-of-range vertex index is an error
    import numpy as np
    lib.gm_last_error.restype = ctypes.c_char_p
    cid = np.zeros(4, np.int32)
    tets = np.array([[0, 1, 2, 9]], np.uint32)
    out = [np.zeros(8, np.uint32) for _ in range(4)]
    ng = ctypes.c_uint32()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    st = lib.gm_node_groups_build(4, p(cid), 1, p(tets), 0, None, 0, None, 1, p(out[0]), p(out[1]), p(out[2]),
                                  p(out[3]), ctypes.byref(ng))
    assert st == 1 and b"vertex" in lib.gm_last_error()
