"""The drop-in shim (gpumesh_gb300/shim/GpuMeshGb300Shim.cpp) against the
reference's own host code, on the CPU.

The shim is compiled against the reference's headers where they lie (with
the compile stand-ins of oracle/ref_shim for GLM, Qt and the GL loader) and
linked, with --no-undefined, against the reference's host objects that call
CUDA drivers (AbstractVertexWiseSmoother, AbstractEvaluator, the samplers,
the GETMe smoother, ... as oracle/refbuild.py compiles them, without the
abort-if-called driver stubs the checker build uses) and libgpumesh_gb300.so.
The link succeeding shows that every driver those classes call resolves to
the shim; the drivers that GpuMesh.cpp declares (its upload / fetch calls,
DataStructures/GpuMesh.cpp:14-26; that file needs the OpenGL loader and is
not compiled here) are checked by name among the shim's definitions.

Link-only: the reference sources do not travel to GPU machines, so the
linked library is not run there; the GPU test of the same uploads through
the C ABI is tests/test_gpu_dropin.py.
"""

import os
import re
import subprocess

import pytest

import pyref
import refbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "gpumesh_gb300", "shim", "GpuMeshGb300Shim.cpp")
LIBDIR = os.path.join(ROOT, "gpumesh_gb300", "_lib")
OUT = os.path.join(refbuild.OUT, "dropin")

pytestmark = pytest.mark.skipif(not pyref.available(), reason="reference tree not available")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, f"{' '.join(cmd)}\n{r.stderr[-4000:]}"
    return r.stdout


@pytest.fixture(scope="module")
def shim_object():
    refbuild.build()
    os.makedirs(OUT, exist_ok=True)
    obj = os.path.join(OUT, "GpuMeshGb300Shim.o")
    _run(["g++", "-std=c++14", "-fPIC", "-w", "-DNDEBUG", "-I" + os.path.join(ROOT, "oracle", "ref_shim"),
          "-I" + refbuild.REF, "-I" + os.path.join(ROOT, "include"), "-c", SHIM, "-o", obj])
    return obj


def test_shim_links_the_reference_host_code(shim_object):
    from gpumesh_gb300 import build

    lib = build.build()
    objs = sorted(os.path.join(refbuild.OUT, "obj", f) for f in os.listdir(os.path.join(refbuild.OUT, "obj"))
                  if f.endswith(".o") and f not in ("ref_stubs.cpp.o", "ref_harness.cpp.o"))
    assert any("AbstractVertexWiseSmoother" in o for o in objs)
    out = os.path.join(OUT, "libgpumesh_reference_dropin.so")
    _run(["g++", "-shared", "-o", out] + objs + [shim_object, "-L" + LIBDIR, "-lgpumesh_gb300", "-lpthread",
                                                  "-Wl,--no-undefined", "-Wl,-rpath," + os.path.dirname(lib)])
    # the reference's driver calls resolve to the shim, not to stubs
    undefined = _run(["nm", "-C", "--undefined-only", out])
    assert "smoothCudaVertices" not in undefined and "evaluateCudaMeshQuality" not in undefined
    defined = _run(["nm", "-C", "--defined-only", out])
    for name in ("smoothCudaVertices(NodeGroups::GpuDispatch const&)", "fetchCudaSubsurfaceVertices",
                 "sendCudaBoundaryVertices", "evaluateCudaMeshQuality", "installCudaNelderMeadSmoother"):
        assert name in defined, name
    # ... and the shim reaches the library's C ABI
    assert "gm_smooth_group" in undefined or "gm_smooth_group" in _run(["nm", "-D", out])


def test_shim_defines_the_gpumesh_upload_drivers(shim_object):
    """GpuMesh::updateCudaTopology / updateCudaVertices / fetchCudaVertices /
    clearCudaMemory call the drivers declared at the top of GpuMesh.cpp."""
    with open(os.path.join(refbuild.REF, "DataStructures", "GpuMesh.cpp")) as f:
        head = f.read().split("GpuMesh::GpuMesh", 1)[0]
    names = set(re.findall(r"^\s*void\s+(\w+)\s*\(", head, flags=re.M))
    assert {"updateCudaVerts", "fetchCudaVerts", "updateCudaTets", "updateCudaTopo"} <= names
    defined = _run(["nm", "-C", "--defined-only", shim_object])
    for name in sorted(names):
        assert re.search(r"\b" + name + r"\(", defined), name
