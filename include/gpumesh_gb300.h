/*
 * gpumesh_gb300.h -- C ABI of libgpumesh_gb300.so, the GB300 (sm_103a)
 * implementation of GpuMesh's vertex-wise relocation smoothing and
 * element-quality evaluation.
 *
 * The reference host code (GpuMesh's C++ Mesh / MeshCrew / NodeGroups and
 * its AbstractSmoother / AbstractEvaluator plugins) calls CUDA through
 * C++-linkage "driver" functions defined under resources/cuda/.  Every entry
 * point below names the driver it replaces (file:line in the GpuMesh tree);
 * a thin C++ shim with the legacy signatures forwards to these calls.
 *
 * Conventions
 *  - Every function returns a gm_status; GM_OK is 0.  gm_last_error()
 *    returns a message for the last failure on the calling thread.
 *  - Arrays are plain host pointers with explicit counts.  Nothing here
 *    takes ownership of caller memory.
 *  - A gm_mesh owns its device buffers.  Work is issued on the mesh's
 *    stream (gm_mesh_set_stream, default: the legacy default stream);
 *    functions that return host results synchronise that stream.
 *  - One process may hold any number of meshes (the reference keeps one
 *    mesh in file-scope device globals, resources/cuda/Mesh.cu:9-31).
 */
#ifndef GPUMESH_GB300_H
#define GPUMESH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gm_status;
#define GM_OK 0
#define GM_ERR_INVALID_ARG 1
#define GM_ERR_CUDA 2
#define GM_ERR_OUT_OF_MEMORY 3
#define GM_ERR_UNSUPPORTED 4
#define GM_ERR_TIMEOUT 5
#define GM_ERR_STATE 6

/* element type codes = MeshTet/MeshPri/MeshHex::ELEMENT_TYPE (DataStructures/Mesh.h:89,171,213) */
#define GM_TET 0
#define GM_PRI 2
#define GM_HEX 3

/* samplers: UniformSampler (Samplers/UniformSampler.cpp:45), AnalyticSampler
 * (Samplers/AbstractSampler.cpp:190-208), the sine-graded anisotropic
 * metric s^2 diag(1 + 9 sin^2(4 pi x), 1, 1) and LocalSampler
 * (Samplers/LocalSampler.cpp:212-311: the metric interpolated in a
 * background tet mesh) */
#define GM_SAMPLER_UNIFORM 0
#define GM_SAMPLER_ANALYTIC 1
#define GM_SAMPLER_SINE 2
#define GM_SAMPLER_LOCAL 3
/* KdTreeSampler (Samplers/KdTreeSampler.cpp:218-247: the local metric
 * sampled once per kd-tree leaf) and TextureSampler (TextureSampler.cpp:
 * 450-488: the local metric sampled at grid cell centres, trilinear) */
#define GM_SAMPLER_KDTREE 4
#define GM_SAMPLER_TEXTURE 5
/* measurers: MetricFreeMeasurer, MetricWiseMeasurer (Measurers/) */
#define GM_MEASURER_METRIC_FREE 0
#define GM_MEASURER_METRIC_WISE 1
/* evaluators: MeanRatioEvaluator, MetricConformityEvaluator (Evaluators/) */
#define GM_EVALUATOR_MEAN_RATIO 0
#define GM_EVALUATOR_METRIC_CONFORMITY 1
/* constraint kinds (Boundaries/Constraints/, Boundaries/SphereBoundary.cpp) */
#define GM_CON_VOLUME 0
#define GM_CON_PLANE 1
#define GM_CON_SEGMENT 2
#define GM_CON_SPHERE 3
#define GM_CON_POINT 4
#define GM_CON_SHELL_INNER 5   /* ShellBoundary::InFace (radius 0.5 sphere) */
#define GM_CON_PIPE_CYLINDER 6 /* PipeBoundary::CylinderFace */
#define GM_CON_PIPE_CIRCLE 7   /* PipeBoundary::YNeg/YPosCircleEdge; params: circle centre */
/* smoothers */
#define GM_SMOOTH_NELDER_MEAD 0
#define GM_SMOOTH_GRADIENT_DESCENT 1
#define GM_SMOOTH_SPAWN_SEARCH 2
#define GM_SMOOTH_GETME 3
#define GM_SMOOTH_SPRING_LAPLACE 4  /* SpringLaplaceSmoother: params[0] = move coefficient (0.35) */
#define GM_SMOOTH_QUALITY_LAPLACE 5 /* QualityLaplaceSmoother: params[0] = move coefficient (0.35) */

#define GM_HIST_BUCKETS 20

/* QualityHistogram (DataStructures/QualityHistogram.h): minimum, sum of
 * 1/q (+inf once any q <= 0, so the harmonic mean count/inv_sum is 0),
 * element count, elements with q <= 0, and 20 clamped buckets. */
typedef struct gm_quality
{
    double min;
    double inv_sum;
    uint64_t count;
    uint64_t nbad;
    uint64_t buckets[GM_HIST_BUCKETS];
} gm_quality;

/* Smoother parameters.  params[] layout per smoother (defaults are the
 * reference's file-scope constants):
 *   NM    [local size -> node shift (1/24), security cycles (12),
 *          value convergence (1e-4), alpha (1), beta (0.5), gamma (2)]
 *          Smoothers/VertexWise/NelderMeadSmoother.cpp:17-23
 *   GD    [local size -> node shift (1/75), security cycles (5)]
 *          Smoothers/VertexWise/GradientDescentSmoother.cpp:14-15
 *   spawn [move coefficient (1/20), iterations (2)]
 *          Smoothers/VertexWise/SpawnSearchSmoother.cpp:14,181
 *   GETMe [lambda (0.78)]  Smoothers/ElementWise/GetmeSmoother.cpp:22
 *   spring Laplace  [move coefficient (0.35)]
 *          Smoothers/VertexWise/SpringLaplaceSmoother.cpp:10
 *   quality Laplace [move coefficient (0.35)]
 *          Smoothers/VertexWise/QualityLaplaceSmoother.cpp:12
 * A NULL params pointer selects the defaults. */
#define GM_PARAMS 8

typedef struct gm_mesh gm_mesh;

const char* gm_last_error(void);
const char* gm_status_string(gm_status s);
/* library build identification: "sm_103a <date>" */
const char* gm_version(void);

/* ---- host topology -------------------------------------------------------
 * Replaces Mesh::compileTopology's neighbourhood pass and NodeGroups::build
 * (DataStructures/Mesh.cpp:213-285, DataStructures/NodeGroups.cpp:104-122)
 * for callers that do not run the reference host code.  Outputs are caller
 * allocated:
 *   perm[nv]          new vertex index -> input vertex index
 *   group_base[nv+1]  colour g owns members[group_base[g] .. group_base[g+1])
 *   members[nv]       colour-major relocation order (new indices)
 *   ranges[6*nv]      per colour: boundary, subsurface, interior [begin,end)
 *   *ngroups          number of colours
 * Connectivity passed in uses input indices. */
gm_status gm_node_groups_build(uint32_t nv, const int32_t* cid, uint32_t nt, const uint32_t* tets,
                               uint32_t np, const uint32_t* pris, uint32_t nh, const uint32_t* hexs,
                               int32_t permute, uint32_t* perm, uint32_t* group_base, uint32_t* members,
                               uint32_t* ranges, uint32_t* ngroups);
/* The same outputs in the device order mode: the colours come from
 * Jones-Plassmann rounds on the GPU (two vertices conflict when they share
 * an element; each round colours the uncoloured vertices whose hashed index
 * beats every uncoloured conflicting vertex, with the lowest colour their
 * coloured neighbours leave free; deterministic), not from the reference's
 * greedy breadth-first colouring, so the relocation order differs from the
 * reference's.  Classes, sort and groups as gm_node_groups_build.  Fixed
 * vertices take colour 0 and are in no group. */
gm_status gm_node_groups_build_device(uint32_t nv, const int32_t* cid, uint32_t nt, const uint32_t* tets, uint32_t np,
                                      const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t permute,
                                      uint32_t* perm, uint32_t* group_base, uint32_t* members, uint32_t* ranges,
                                      uint32_t* ngroups);
/* The vertex neighbourhoods Mesh::compileNeighborhoods builds
 * (DataStructures/Mesh.cpp:365-460), as the library builds them for an
 * upload, in input indices:
 *   ve_off[nv+1], ve[]  incident elements, packed (type << 30 | local << 27
 *                       | id), tets then prisms then hexes, each by id
 *   vv_off[nv+1], vv[]  edge neighbours in Mesh::addEdge order
 * Call with ve == vv == NULL to get *ve_len and *vv_len, then with arrays of
 * those lengths. */
gm_status gm_mesh_neighbourhoods(uint32_t nv, uint32_t nt, const uint32_t* tets, uint32_t np, const uint32_t* pris,
                                 uint32_t nh, const uint32_t* hexs, uint32_t* ve_off, uint32_t* ve, uint64_t* ve_len,
                                 uint32_t* vv_off, uint32_t* vv, uint64_t* vv_len);

/* ---- device mesh ---------------------------------------------------------- */
gm_status gm_mesh_create(gm_mesh** out);
gm_status gm_mesh_destroy(gm_mesh* mesh);
/* stream: a cudaStream_t; 0 is the legacy default stream */
gm_status gm_mesh_set_stream(gm_mesh* mesh, void* stream);
gm_status gm_mesh_sync(gm_mesh* mesh);

/* Upload a whole mesh in the order given (no permutation): positions (FP64,
 * 3 per vertex), constraint id per vertex (<0 fixed, 0 free, >0 constraint),
 * connectivity.  Builds the vertex->element and vertex->vertex CSR on the
 * host.  Replaces GpuMesh::updateCudaTopology + updateCudaVertices
 * (DataStructures/GpuMesh.cpp:227-276). */
gm_status gm_mesh_upload(gm_mesh* mesh, uint32_t nv, const double* xyz, const int32_t* cid, uint32_t nt,
                         const uint32_t* tets, uint32_t np, const uint32_t* pris, uint32_t nh,
                         const uint32_t* hexs);

/* Replaces updateCudaVerts (resources/cuda/Mesh.cu:74).  xyz: FP64 x,y,z. */
gm_status gm_mesh_upload_verts(gm_mesh* mesh, uint32_t nv, const double* xyz);
/* Replaces updateCudaVerts with the reference's GpuVert layout
 * {vec3 p; uint c} (16 bytes per vertex, DataStructures/GpuMesh.h:11-19). */
gm_status gm_mesh_upload_gpu_verts(gm_mesh* mesh, uint32_t nv, const void* gpu_verts);
/* The same, asynchronous on the mesh's stream, for a mesh whose vertices
 * are already uploaded (nv must match): `gpu_verts` should be pinned host
 * memory and must stay unchanged until the stream has passed the copy. */
gm_status gm_mesh_upload_gpu_verts_async(gm_mesh* mesh, uint32_t nv, const void* gpu_verts);
/* Replace the copies of fetchCudaSubsurfaceVertices and
 * sendCudaBoundaryVertices (resources/cuda/Smoothing/Utils.cu:85,117): the
 * GpuVert records of vertices [first, first + count), device to host and
 * host to device.  Synchronous on the mesh's stream. */
gm_status gm_mesh_fetch_gpu_verts_range(gm_mesh* mesh, uint32_t first, uint32_t count, void* gpu_verts);
gm_status gm_mesh_upload_gpu_verts_range(gm_mesh* mesh, uint32_t first, uint32_t count, const void* gpu_verts);
/* Replace updateCudaTets / updateCudaPris / updateCudaHexs
 * (resources/cuda/Mesh.cu:100,126,152).  stride_words = 32-bit words per
 * element record: 4/6/8 for bare connectivity, 5/12/16 for GpuTet, GpuPri,
 * GpuHex (DataStructures/GpuMesh.h:41-85), whose cache words are ignored. */
gm_status gm_mesh_upload_tets(gm_mesh* mesh, uint32_t n, const uint32_t* words, uint32_t stride_words);
gm_status gm_mesh_upload_pris(gm_mesh* mesh, uint32_t n, const uint32_t* words, uint32_t stride_words);
gm_status gm_mesh_upload_hexs(gm_mesh* mesh, uint32_t n, const uint32_t* words, uint32_t stride_words);
/* Replaces updateCudaTopo (resources/cuda/Mesh.cu:185): GpuTopo records
 * {int type; uint neigVertBase, neigVertCount, neigElemBase, neigElemCount}
 * (type: -1 fixed, 0 free, >0 constraint id), GpuNeigVert {uint v},
 * GpuNeigElem {uint id; int type; int vId} (DataStructures/GpuMesh.h:87-141). */
gm_status gm_mesh_upload_topo(gm_mesh* mesh, uint32_t nv, const int32_t* topo5, uint32_t n_neig_verts,
                              const uint32_t* neig_verts, uint32_t n_neig_elems, const int32_t* neig_elems3);
/* Replaces updateCudaGroupMembers (resources/cuda/Mesh.cu:259): the
 * concatenated relocation order; group_base gives each colour's slice. */
gm_status gm_mesh_upload_groups(gm_mesh* mesh, uint32_t n_members, const uint32_t* members, uint32_t ngroups,
                                const uint32_t* group_base);
/* Constraint table indexed by constraint id (id 0 = volume).  params: 6
 * doubles per id -- plane: point, normal; segment: a, b; point: position.
 * The reference's constraint objects (Boundaries/Constraints/) carry these
 * as private members; the drop-in shim recovers them from the boundary's
 * geometry (box faces / edges / corners, unit sphere). */
gm_status gm_mesh_set_constraints(gm_mesh* mesh, uint32_t n, const int32_t* kind, const double* params);
/* Sampler / measurer / evaluator plugins and their uniforms.  Replaces the
 * install* drivers (Evaluating/MeanRatio.cu:156, MetricConformity.cu:196,
 * Measuring/MetricFree.cu:124, MetricWise.cu:168, Sampling/Analytic.cu:15,
 * Uniform.cu:13) and setCudaMetricScaling/ScalingSqr/ScalingCube/AspectRatio,
 * setCudaRotMat (Sampling/Base.cu:110-153); the rotation is the reference
 * sampler's fixed one and is rebuilt here. */
gm_status gm_mesh_set_crew(gm_mesh* mesh, int32_t sampler, int32_t measurer, int32_t evaluator, double scaling,
                           double aspect_ratio);
/* GM_SAMPLER_LOCAL samples a background tet mesh kept with the mesh.
 * gm_mesh_build_local_background builds it from the resident mesh as
 * LocalSampler::updateAnalyticalMetric does (Samplers/LocalSampler.cpp:
 * 193-203, 352-429): prisms and hexes split into tets as Tetrahedralizer.h
 * splits them, face neighbours, the analytic metric (the crew's scaling and
 * aspect ratio) at every vertex.  gm_mesh_set_crew with GM_SAMPLER_LOCAL
 * builds it when the mesh has none, or has one built with another scaling or
 * aspect ratio; a topology upload rebuilds it while the local sampler is
 * installed.  Vertex moves leave it as it is, as in the reference. */
gm_status gm_mesh_build_local_background(gm_mesh* mesh);
/* Replaces updateCudaLocalTets / updateCudaRefVerts / updateCudaRefMetrics
 * (resources/cuda/Sampling/Local.cu:143-230; LocalSampler::updateCudaData,
 * Samplers/LocalSampler.cpp:126-158): a background given by the caller.
 * tets8: per tet its 4 vertices, then the neighbour across the face opposite
 * each vertex (0xffffffff: none), as GpuLocalTet (DataStructures/GpuMesh.h:
 * 166-180); xyz: 3 doubles per vertex; metrics6: xx yy zz xy xz yz per
 * vertex (GpuMetric is a mat4; the shim passes its symmetric 3x3 part).
 * The per-vertex walk caches (updateCudaLocalCache) are not needed: walks
 * start from a uniform grid over the background. */
gm_status gm_mesh_set_local_background(gm_mesh* mesh, uint32_t ntets, const uint32_t* tets8, uint32_t nverts,
                                       const double* xyz, const double* metrics6);
/* GM_SAMPLER_KDTREE / GM_SAMPLER_TEXTURE sample a local-sampler background
 * built from the resident mesh, as KdTreeSampler / TextureSampler::
 * updateAnalyticalMetric do (KdTreeSampler.cpp:116-180, 268-372;
 * TextureSampler.cpp:257-448), when installed; rebuilt on a scaling, aspect
 * ratio or depth change and by gm_mesh_build_local_background.
 * AbstractSampler::setDiscretizationDepth (AbstractSampler.cpp:61-64): the
 * kd-tree height / texture resolution, -1 (default) from the vertex count. */
gm_status gm_mesh_set_discretization_depth(gm_mesh* mesh, int32_t depth);
/* Replaces updateCudaKdNodes (resources/cuda/Sampling/KdTree.cu:58-87;
 * KdTreeSampler::updateCudaData, KdTreeSampler.cpp:94-103): n nodes in
 * pre-order (children after their parent), per node its left and right child
 * (-1: none), its separator plane (normal xyz, offset w: a point p goes left
 * when dot(p, n) - w < 0) and its metric (xx yy zz xy xz yz). */
gm_status gm_mesh_set_kd_nodes(gm_mesh* mesh, uint32_t n, const int32_t* children2, const double* separators4,
                               const double* metrics6);
/* Replaces updateCudaSamplerTextures (resources/cuda/Sampling/Texture.cu:
 * 66-147): metric samples at the cell centres of a dims3 grid over
 * [min3, min3 + extents3], x fastest (6 doubles per cell), read as
 * TextureSampler::metricAt reads its grid. */
gm_status gm_mesh_set_texture(gm_mesh* mesh, const int32_t* dims3, const double* min3, const double* extents3,
                              const double* metrics6);

/* Copy a resident mesh (topology, groups, constraints, crew, positions)
 * device to device into `dst`: a new job on an existing topology needs only
 * its own positions uploaded afterwards.  Synchronous. */
gm_status gm_mesh_clone(gm_mesh* dst, const gm_mesh* src);
/* device bytes currently held by the mesh (for admission budgets) */
gm_status gm_mesh_device_bytes(const gm_mesh* mesh, uint64_t* bytes);

/* Keep a device copy of the current positions / restore it (no host
 * traffic); used to replay a smoothing schedule from the same input. */
gm_status gm_mesh_save_positions(gm_mesh* mesh);
gm_status gm_mesh_restore_positions(gm_mesh* mesh);

/* Replaces fetchCudaVerts (resources/cuda/Mesh.cu:56): FP64 x,y,z. */
gm_status gm_mesh_fetch_verts(gm_mesh* mesh, uint32_t nv, double* xyz);
gm_status gm_mesh_fetch_gpu_verts(gm_mesh* mesh, uint32_t nv, void* gpu_verts);

/* ---- evaluation ----------------------------------------------------------
 * Replaces evaluateCudaMeshQuality (resources/cuda/Evaluating/Evaluate.cu:55)
 * and AbstractEvaluator::evaluateMeshQualityCuda
 * (Evaluators/AbstractEvaluator.cpp:574-610).  Synchronous: fills *out. */
gm_status gm_evaluate(gm_mesh* mesh, gm_quality* out);
/* Asynchronous: leaves the result in device result slot `slot` (slots are
 * allocated on demand, so a whole smoothing schedule can record one result
 * per pass without a host round trip); gm_quality_read copies a slot back
 * and synchronises the mesh's stream. */
gm_status gm_evaluate_async(gm_mesh* mesh, uint32_t slot);
gm_status gm_quality_read(gm_mesh* mesh, uint32_t slot, gm_quality* out);

/* ---- relocation ----------------------------------------------------------
 * One colour: replaces smoothCudaVertices (Smoothing/VertexWise/
 * SmoothVertices.cu:28) and smoothCudaSpawnVertices (SpawnSearch.cu:220),
 * i.e. one NodeGroups::GpuDispatch {gpuBufferBase, gpuBufferSize} slice of
 * the uploaded members.  Relocates constrained (boundary) vertices too, with
 * in-kernel projection.  Asynchronous. */
gm_status gm_smooth_group(gm_mesh* mesh, int32_t smoother, const double* params, uint32_t member_base,
                          uint32_t member_count);
/* A whole relocation pass: every colour in order, one launch per colour, no
 * host round trip.  For GETMe: the element pass then one vertex-update launch
 * per colour.  Asynchronous. */
gm_status gm_smooth_pass(gm_mesh* mesh, int32_t smoother, const double* params);
/* GETMe halves for the drop-in: smoothCudaElements (Smoothing/ElementWise/
 * SmoothElements.cu:41) and updateCudaSmoothedElementsVertices
 * (UpdateVertices.cu:47). */
gm_status gm_getme_elements(gm_mesh* mesh, const double* params);
gm_status gm_getme_update_group(gm_mesh* mesh, const double* params, uint32_t member_base, uint32_t member_count);

/* Work counters since the last reset: [patch evaluations, tet, prism, hex
 * element evaluations, vertices relocated in FP64].  Synchronous. */
gm_status gm_mesh_counters(gm_mesh* mesh, uint64_t* out5, int32_t reset);

/* ---- batched path ----------------------------------------------------------
 * No single counterpart in the reference (one mesh per process, one launch
 * and one host synchronisation per colour: SmoothVertices.cu:28-47).  A
 * batch relocates the independent groups of many device-resident meshes in
 * ONE persistent kernel launch per pass: vertices are taken from a device
 * work queue ordered by (colour, mesh), and a mesh's colour g starts as soon
 * as that mesh's colours < g are done (device counters, bounded waits).
 * Meshes keep their own buffers; upload them, their groups, constraints and
 * crew before creating the batch, and do not re-upload them while it lives.
 * All meshes of a batch share the evaluator / measurer pair (mean ratio with
 * the metric-free measurer, or metric conformity with a diagonal metric). */
typedef struct gm_batch gm_batch;
gm_status gm_batch_create(gm_batch** out, gm_mesh* const* meshes, uint32_t n);
gm_status gm_batch_destroy(gm_batch* batch);
/* the batch's own (non-blocking) stream, as a cudaStream_t */
gm_status gm_batch_stream(gm_batch* batch, void** stream);
gm_status gm_batch_sync(gm_batch* batch);
/* launch shape of the persistent kernel: warps per block (1, 2, 4, 8) and
 * CTAs per SM (0: as many as fit; never more than fit, since every CTA of
 * the persistent grid must be resident) */
gm_status gm_batch_set_config(gm_batch* batch, int32_t warps_per_block, int32_t ctas_per_sm);
/* autotuner: times one pass per candidate shape from the same positions
 * (kept in each mesh's save slot), restores them, keeps the fastest */
gm_status gm_batch_tune(gm_batch* batch, int32_t smoother, const double* params, int32_t* best_warps_per_block,
                        int32_t* best_ctas_per_sm, double* best_ms);
/* one relocation pass of every mesh (GETMe: per-mesh element passes, then
 * the batched vertex update); asynchronous on the batch stream */
gm_status gm_batch_smooth_pass(gm_batch* batch, int32_t smoother, const double* params);
/* per-mesh quality (one gm_quality per mesh) into device slot `slot` */
gm_status gm_batch_evaluate(gm_batch* batch, uint32_t slot);
gm_status gm_batch_read_quality(gm_batch* batch, uint32_t slot, gm_quality* out_per_mesh);
/* capture one pass (and, if eval_slot >= 0, its evaluation) as a CUDA graph;
 * gm_batch_replay launches it */
gm_status gm_batch_capture_pass(gm_batch* batch, int32_t smoother, const double* params, int32_t eval_slot);
gm_status gm_batch_replay(gm_batch* batch);
/* GM_ERR_TIMEOUT if a dependency wait of the last pass gave up; synchronous */
gm_status gm_batch_status(gm_batch* batch);
/* bound of the dependency waits, in polls of ~100 ns (default 2e7) */
gm_status gm_batch_set_spin_limit(gm_batch* batch, uint64_t polls);
/* fault injection for tests: colours > 0 of `mesh` wait for a count that
 * never arrives, so the pass must end with GM_ERR_TIMEOUT */
gm_status gm_batch_inject_stall(gm_batch* batch, uint32_t mesh);
gm_status gm_batch_counters(gm_batch* batch, uint64_t* out5, int32_t reset);
/* per mesh: milliseconds from the start of the last pass's persistent
 * kernel to that mesh's last relocated vertex (-1: no vertex moved) */
gm_status gm_batch_latencies(gm_batch* batch, double* out_ms_per_mesh);
/* [meshes, queued vertices, segments, evaluation blocks] */
gm_status gm_batch_info(gm_batch* batch, uint32_t* out4);

/* ---- device-resident jobs --------------------------------------------------
 * No single counterpart in the reference, whose pass loop runs on the host
 * (AbstractSmoother::smoothMesh, Smoothers/AbstractSmoother.cpp:103-211).
 * A job is a whole smoothing schedule under a stop rule: an evaluation, then
 * relocation passes, each followed by an evaluation, until the minimum
 * quality rises by less than min_gain or max_passes passes are done.
 * gm_job_prepare captures it as one CUDA graph whose loop is a conditional
 * node that the device drives, so a job costs one launch and no host round
 * trip per pass.  Re-uploading the mesh's topology, groups, constraints or
 * crew drops the prepared job; new positions of the same size do not.  The
 * quality after pass p is in result slot p (gm_quality_read). */
gm_status gm_job_prepare(gm_mesh* mesh, int32_t smoother, const double* params, uint32_t max_passes,
                         double min_gain);
/* asynchronous, on the mesh's stream */
gm_status gm_job_launch(gm_mesh* mesh);
/* *done = 1 once the mesh's stream has no work left */
gm_status gm_job_query(gm_mesh* mesh, int32_t* done);
/* passes run, quality before the first pass and after the last; synchronous */
gm_status gm_job_result(gm_mesh* mesh, uint32_t* passes, gm_quality* first, gm_quality* last);

/* No counterpart in the reference.  Quality evaluation that allocates
 * nothing, for callers that cannot call cudaMalloc (a host framework that
 * owns every device allocation, a fully committed memory budget, a loop
 * that must not allocate once running).  Every pointer is a device pointer:
 * pos = nv float4 (x, y, z, unused; 16-byte aligned), tets / hexs = 4 / 8
 * uint32 per element (16-byte aligned), pris = 6 uint32 per element (8-byte
 * aligned); *out receives the gm_quality on the device, asynchronously on
 * `stream`.  The only scratch is a 104 KiB array inside this library that
 * every GPU which loads the library holds until exit; meshes above
 * 16,777,216 elements are rejected with GM_ERR_UNSUPPORTED.  The first call
 * on a device looks up that array's device address, so make it before any
 * stream capture; the address is kept until exit, so calls after a reset of
 * that device (cudaDeviceReset) are not supported.  All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Precondition, not checked: every tet, prism and hex index is
 * below nv (the kernel gathers positions by these indices, and an index out
 * of range reads outside the position buffer). */
gm_status gm_evaluate_noalloc(uint32_t nv, const void* pos, uint32_t nt, const uint32_t* tets, uint32_t np,
                              const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t sampler,
                              int32_t measurer, int32_t evaluator, double scaling, double aspect_ratio,
                              gm_quality* out, void* stream);

/* Device bounds checks.  The library built with GM_BOUNDS_CHECK
 * (libgpumesh_gb300_checked.so) compares every connectivity and
 * neighbourhood index its evaluation, relocation, GETMe and batched kernels
 * read through with the length of the array it indexes; the first index out
 * of range is recorded in the mesh's status word and read as 0, so the
 * access stays inside the array.  Its synchronising calls (gm_mesh_sync,
 * gm_quality_read / gm_evaluate, gm_mesh_fetch_gpu_verts) then fail with
 * GM_ERR_STATE and a gm_last_error() message naming the array and the index.
 * The reference's counterpart is cudaCheckErrors (resources/cuda/Mesh.cuh:
 * 169-183), which reports only CUDA's own errors.
 *   gm_bounds_checked: *on = 1 in the checked build, 0 otherwise.
 *   gm_mesh_bounds_status: *what = 0 when clean, else the array (1 vertex,
 *   2 vertex->element CSR, 3 vertex->vertex CSR, 4 tet, 5 prism, 6 hex,
 *   7 GETMe corner) and *index the index read; clears the word.  In the
 *   ordinary build the word stays 0.  Synchronous.  A batch's kernels
 *   record into each member mesh's word. */
gm_status gm_bounds_checked(int32_t* on);
gm_status gm_mesh_bounds_status(gm_mesh* mesh, uint32_t* what, uint32_t* index);

/* No counterpart in the reference (its drivers launch on the legacy default
 * stream and keep no count).  *count receives the number of kernel launches
 * this library has made in this process: every direct launch counts one,
 * and a captured graph (gm_batch_replay, a job of gm_job_launch) counts the
 * kernels it runs, a job's loop body once per pass it ran (added when
 * gm_job_result reads the pass count).  Kernels of other libraries are not
 * counted.  Thread-safe. */
gm_status gm_launch_count(uint64_t* count);

/* Device peak probe: a dependent-FFMA loop over every SM; *tflops receives
 * the achieved FP32 rate (2 flops per FFMA).  The roofline denominator of
 * the relocation kernels. */
gm_status gm_probe_fp32_tflops(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* GPUMESH_GB300_H */
