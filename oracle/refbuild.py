"""Compile the reference's own CPU smoothers and evaluators into the checker
library oracle/_ref/libgmref.so.

TEST INFRASTRUCTURE ONLY.  The sources are compiled in place from the
reference tree (never copied) against the project-written stand-ins in
oracle/ref_shim/ for its external dependencies (GLM, the CellarWorkbench log
and GLSL wrapper, the GL loader), plus oracle/ref_stubs.cpp (the CUDA driver
entry points, which abort if called) and the harness oracle/ref_harness.cpp.
Nothing is built when the reference tree is absent.  The tree is
GM_REFERENCE_TREE, else a directory named `reference` beside the
repository.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libgmref.so")



def _reference_tree() -> str:
    """The GpuMesh source tree: GM_REFERENCE_TREE, else a directory named
    `reference` beside this repository's root."""
    if os.environ.get("GM_REFERENCE_TREE"):
        return os.environ["GM_REFERENCE_TREE"]
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


REF = _reference_tree()

SOURCES = [
    "DataStructures/Mesh.cpp", "DataStructures/NodeGroups.cpp", "DataStructures/MeshCrew.cpp",
    "DataStructures/QualityHistogram.cpp", "DataStructures/Schedule.cpp", "DataStructures/OptimizationPlot.cpp",
    "Evaluators/AbstractEvaluator.cpp", "Evaluators/MeanRatioEvaluator.cpp", "Evaluators/MetricConformityEvaluator.cpp",
    "Measurers/AbstractMeasurer.cpp", "Measurers/MetricFreeMeasurer.cpp", "Measurers/MetricWiseMeasurer.cpp",
    "Samplers/AbstractSampler.cpp", "Samplers/AnalyticSampler.cpp", "Samplers/UniformSampler.cpp",
    "Samplers/LocalSampler.cpp", "DataStructures/TriSet.cpp", "Samplers/KdTreeSampler.cpp",
    "Samplers/TextureSampler.cpp",
    "Boundaries/AbstractBoundary.cpp", "Boundaries/BoxBoundary.cpp", "Boundaries/SphereBoundary.cpp",
    "Boundaries/TetBoundary.cpp", "Boundaries/PipeBoundary.cpp", "Boundaries/ShellBoundary.cpp",
    "Boundaries/BoundaryFree.cpp", "Boundaries/Constraints/AbstractConstraint.cpp",
    "Boundaries/Constraints/VertexConstraint.cpp", "Boundaries/Constraints/EdgeConstraint.cpp",
    "Boundaries/Constraints/FaceConstraint.cpp", "Boundaries/Constraints/VolumeConstraint.cpp",
    "Smoothers/AbstractSmoother.cpp", "Smoothers/VertexWise/AbstractVertexWiseSmoother.cpp",
    "Smoothers/VertexWise/NelderMeadSmoother.cpp", "Smoothers/VertexWise/GradientDescentSmoother.cpp",
    "Smoothers/VertexWise/SpawnSearchSmoother.cpp", "Smoothers/VertexWise/SpringLaplaceSmoother.cpp",
    "Smoothers/VertexWise/QualityLaplaceSmoother.cpp", "Smoothers/ElementWise/AbstractElementWiseSmoother.cpp",
    "Smoothers/ElementWise/GetmeSmoother.cpp", "Smoothers/ElementWise/VertexAccum.cpp",
    "Topologists/AbstractTopologist.cpp", "Topologists/BatrTopologist.cpp",
    "Serialization/AbstractSerializer.cpp", "Serialization/AbstractDeserializer.cpp",
    "Serialization/JsonSerializer.cpp", "Serialization/JsonDeserializer.cpp", "Serialization/JsonMeshTags.cpp",
]
LOCAL = ["ref_harness.cpp", "ref_stubs.cpp"]
FLAGS = ["-O2", "-std=c++14", "-fPIC", "-ffp-contract=off", "-w", "-DNDEBUG",
         "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF]


def available() -> bool:
    return os.path.isdir(os.path.join(REF, "DataStructures"))


def _obj(src: str) -> str:
    return os.path.join(OUT, "obj", src.replace("/", "_") + ".o")


def _compile(src: str, path: str) -> str:
    obj = _obj(src)
    deps = [path] + [os.path.join(HERE, "ref_shim", d) for d in ()]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in deps):
        return obj
    r = subprocess.run(["g++"] + FLAGS + ["-c", path, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed on {src}:\n{r.stderr[-4000:]}")
    return obj


def build(force: bool = False) -> str:
    if not available():
        raise FileNotFoundError(f"reference tree not found at {REF}")
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    jobs = [(s, os.path.join(REF, s)) for s in SOURCES] + [(s, os.path.join(HERE, s)) for s in LOCAL]
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        r = subprocess.run(["g++", "-shared", "-o", LIB] + objs + ["-lpthread", "-Wl,--no-undefined"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference link failed:\n{r.stderr[-6000:]}")
    return LIB


def build_if_available():
    if available():
        return build()
    return None


if __name__ == "__main__":
    print(build("--force" in sys.argv))
