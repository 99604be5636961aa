"""GB300-native node-relocation smoothing and element-quality evaluation.

A from-scratch sm_103a implementation of the hot path of the GpuMesh mesh
optimiser: vertex-wise Nelder-Mead, gradient-descent and spawn-search
relocation and GETMe element-wise smoothing over graph-coloured independent
vertex groups, and mean-ratio / metric-conformity quality evaluation, behind a
C ABI (include/gpumesh_gb300.h) and a host mirror of the reference's plugin
interfaces (gpumesh_gb300.mesh).
"""

from .meshgen import RawMesh, box_mesh, sphere_mesh, batch_meshes  # noqa: F401

__all__ = ["RawMesh", "box_mesh", "sphere_mesh", "batch_meshes"]
