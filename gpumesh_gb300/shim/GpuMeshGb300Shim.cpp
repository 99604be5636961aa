// The legacy CUDA drivers of GpuMesh implemented over libgpumesh_gb300.so.
//
// A maintainer drops the reference's resources/cuda/*.cu translation units
// from its build, adds this file, and links libgpumesh_gb300.so: the
// reference's host classes (GpuMesh::updateCuda*, AbstractVertexWiseSmoother::
// smoothMeshCuda, AbstractEvaluator::evaluateMeshQualityCuda, the samplers'
// updateCudaData, the plugins' installPlugin) then run on the GB300 kernels
// unchanged.  Each function defines the driver of the same signature that
// the reference declares extern in its host .cpp files; the comment names
// the driver it replaces (file:line under resources/cuda/).
//
// The drivers act on one "current mesh" (the reference keeps one mesh in
// file-scope device globals, Mesh.cu:9-31).  Errors follow the reference's
// cudaCheckErrors (Mesh.cuh:169-183): a build without NDEBUG prints the
// failure and exits; an NDEBUG build carries on, and the message stays
// readable through gm_last_error().
//
// Legacy mode, as the reference runs: the host relocates boundary vertices
// and sends the GPU the non-boundary members of each colour
// (NodeGroups::gpuGroupsBuffer); no constraint table is uploaded.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "DataStructures/GpuMesh.h"
#include "DataStructures/NodeGroups.h"
#include "DataStructures/QualityHistogram.h"
#include "gpumesh_gb300.h"

bool verboseCuda = true;  // Mesh.cu:49

namespace {

gm_mesh* g_mesh = nullptr;
int g_sampler = GM_SAMPLER_UNIFORM, g_measurer = GM_MEASURER_METRIC_FREE, g_evaluator = GM_EVALUATOR_MEAN_RATIO;
double g_scaling = 1.0, g_aspect = 1.0;
int g_smoother = GM_SMOOTH_NELDER_MEAD;
double g_params[GM_PARAMS] = {};

void check(gm_status s, const char* what)
{
    if (s == GM_OK) return;
#ifndef NDEBUG
    std::fprintf(stderr, "Fatal error: %s (%s)\n", what, gm_last_error());
    std::fprintf(stderr, "*** FAILED - ABORTING\n");
    std::exit(1);
#else
    (void)what;
#endif
}

gm_mesh* mesh()
{
    if (!g_mesh) check(gm_mesh_create(&g_mesh), "gm_mesh_create");
    return g_mesh;
}

void apply_crew()
{
    check(gm_mesh_set_crew(mesh(), g_sampler, g_measurer, g_evaluator, g_scaling, g_aspect), "set_crew");
}

template <class E>
const uint32_t* words(const std::vector<E>& v)
{
    static const uint32_t none = 0;
    return v.empty() ? &none : &v.data()->v[0];
}

}  // namespace

// ---- Mesh.cu ----------------------------------------------------------------

// updateCudaVerts (Mesh.cu:74); an empty vector (GpuMesh::clearCudaMemory)
// releases the mesh
void updateCudaVerts(const std::vector<GpuVert>& v)
{
    if (v.empty())
    {
        if (g_mesh) gm_mesh_destroy(g_mesh);
        g_mesh = nullptr;
        return;
    }
    check(gm_mesh_upload_gpu_verts(mesh(), (uint32_t)v.size(), v.data()), "updateCudaVerts");
}

// fetchCudaVerts (Mesh.cu:56)
void fetchCudaVerts(std::vector<GpuVert>& v)
{
    check(gm_mesh_fetch_gpu_verts(mesh(), (uint32_t)v.size(), v.data()), "fetchCudaVerts");
}

// updateCudaTets / Pris / Hexs (Mesh.cu:100,126,152): GpuTet / GpuPri / GpuHex
// records of 5 / 12 / 16 words, whose cache words the library ignores
void updateCudaTets(const std::vector<GpuTet>& t)
{
    static_assert(sizeof(GpuTet) == 5 * sizeof(uint32_t), "GpuTet layout");
    check(gm_mesh_upload_tets(mesh(), (uint32_t)t.size(), words(t), 5), "updateCudaTets");
}
void updateCudaPris(const std::vector<GpuPri>& p)
{
    static_assert(sizeof(GpuPri) == 12 * sizeof(uint32_t), "GpuPri layout");
    check(gm_mesh_upload_pris(mesh(), (uint32_t)p.size(), words(p), 12), "updateCudaPris");
}
void updateCudaHexs(const std::vector<GpuHex>& h)
{
    static_assert(sizeof(GpuHex) == 16 * sizeof(uint32_t), "GpuHex layout");
    check(gm_mesh_upload_hexs(mesh(), (uint32_t)h.size(), words(h), 16), "updateCudaHexs");
}

// updateCudaTopo (Mesh.cu:185)
void updateCudaTopo(const std::vector<GpuTopo>& topos, const std::vector<GpuNeigVert>& nv,
                    const std::vector<GpuNeigElem>& ne)
{
    static_assert(sizeof(GpuTopo) == 5 * sizeof(int32_t) && sizeof(GpuNeigVert) == sizeof(uint32_t) &&
                      sizeof(GpuNeigElem) == 3 * sizeof(int32_t),
                  "GpuTopo / GpuNeigVert / GpuNeigElem layout");
    if (topos.empty()) return;  // GpuMesh::clearCudaMemory
    check(gm_mesh_upload_topo(mesh(), (uint32_t)topos.size(), &topos.data()->type, (uint32_t)nv.size(),
                              nv.empty() ? nullptr : &nv.data()->v, (uint32_t)ne.size(),
                              ne.empty() ? nullptr : reinterpret_cast<const int32_t*>(ne.data())),
          "updateCudaTopo");
}

// updateCudaGroupMembers (Mesh.cu:259): one slice; every GpuDispatch
// addresses its part by gpuBufferBase / gpuBufferSize
void updateCudaGroupMembers(const std::vector<GLuint>& members)
{
    if (members.empty() && !g_mesh) return;  // GpuMesh::clearCudaMemory
    const uint32_t base[2] = {0, (uint32_t)members.size()};
    static const uint32_t none = 0;
    check(gm_mesh_upload_groups(mesh(), (uint32_t)members.size(), members.empty() ? &none : members.data(), 1, base),
          "updateCudaGroupMembers");
}

// cppCudaCheckErrors (Mesh.cu:339)
void cppCudaCheckErrors(const char* msg)
{
#ifndef NDEBUG
    if (gm_last_error()[0])
    {
        std::fprintf(stderr, "Fatal error: %s (%s)\n", msg, gm_last_error());
        std::fprintf(stderr, "*** FAILED - ABORTING\n");
        std::exit(1);
    }
#else
    (void)msg;
#endif
}

// ---- Smoothing/Utils.cu ------------------------------------------------------

// fetchCudaSubsurfaceVertices (Smoothing/Utils.cu:85): the colour's
// subsurface vertices, relocated on the GPU, back into the host mesh
void fetchCudaSubsurfaceVertices(std::vector<MeshVert>& meshVerts, const NodeGroups::ParallelGroup& group)
{
    const size_t n = group.subsurfaceRange.end - group.subsurfaceRange.begin;
    if (!n) return;
    std::vector<GpuVert> buf(n);
    check(gm_mesh_fetch_gpu_verts_range(mesh(), (uint32_t)group.subsurfaceRange.begin, (uint32_t)n, buf.data()),
          "fetchCudaSubsurfaceVertices");
    for (size_t i = 0; i < n; ++i) meshVerts[group.subsurfaceRange.begin + i] = MeshVert(buf[i]);
}

// sendCudaBoundaryVertices (Smoothing/Utils.cu:117): the colour's boundary
// vertices, relocated by the host workers, to the GPU
void sendCudaBoundaryVertices(const std::vector<MeshVert>& meshVerts, const NodeGroups::ParallelGroup& group)
{
    const size_t n = group.boundaryRange.end - group.boundaryRange.begin;
    if (!n) return;
    std::vector<GpuVert> buf(n);
    for (size_t i = 0; i < n; ++i) buf[i] = GpuVert(meshVerts[group.boundaryRange.begin + i]);
    check(gm_mesh_upload_gpu_verts_range(mesh(), (uint32_t)group.boundaryRange.begin, (uint32_t)n, buf.data()),
          "sendCudaBoundaryVertices");
}

// ---- plugins and uniforms ----------------------------------------------------

void installCudaMeanRatioEvaluator() { g_evaluator = GM_EVALUATOR_MEAN_RATIO; apply_crew(); }  // MeanRatio.cu:156
void installCudaMetricConformityEvaluator()  // MetricConformity.cu:196
{
    g_evaluator = GM_EVALUATOR_METRIC_CONFORMITY;
    apply_crew();
}
void installCudaMetricFreeMeasurer() { g_measurer = GM_MEASURER_METRIC_FREE; apply_crew(); }  // MetricFree.cu:124
void installCudaMetricWiseMeasurer() { g_measurer = GM_MEASURER_METRIC_WISE; apply_crew(); }  // MetricWise.cu:168
void installCudaUniformSampler() { g_sampler = GM_SAMPLER_UNIFORM; apply_crew(); }            // Uniform.cu:13
void installCudaAnalyticSampler() { g_sampler = GM_SAMPLER_ANALYTIC; apply_crew(); }          // Analytic.cu:15
void installCudaLocalSampler() { g_sampler = GM_SAMPLER_LOCAL; apply_crew(); }                // Local.cu:127

// Sampling/Base.cu:110-153: the scaling and aspect ratio; the square, the
// cube and the rotation are derived inside (the rotation is the sampler's
// fixed one)
void setCudaMetricScaling(double s) { g_scaling = s; apply_crew(); }
void setCudaMetricScalingSqr(double) {}
void setCudaMetricScalingCube(double) {}
void setCudaMetricAspectRatio(double a) { g_aspect = a; apply_crew(); }
void setCudaRotMat(const glm::dmat3&, const glm::dmat3&) {}

// ---- the local sampler's background mesh (LocalSampler::updateCudaData) -------

namespace {
std::vector<uint32_t> g_local_tets;  // GpuLocalTet: v[4], then n[4]
std::vector<double> g_ref_xyz, g_ref_metrics;
}  // namespace

// updateCudaLocalTets (Sampling/Local.cu:143)
void updateCudaLocalTets(const std::vector<GpuLocalTet>& tets)
{
    g_local_tets.clear();
    for (const GpuLocalTet& t : tets)
        g_local_tets.insert(g_local_tets.end(), {t.v[0], t.v[1], t.v[2], t.v[3], t.n[0], t.n[1], t.n[2], t.n[3]});
}
// updateCudaLocalCache: walks start at the element's first background tet or
// at a start grid, so the vertex cache is not needed
void updateCudaLocalCache(const std::vector<GLuint>&) {}
// updateCudaRefVerts
void updateCudaRefVerts(const std::vector<GpuVert>& verts)
{
    g_ref_xyz.clear();
    for (const GpuVert& v : verts) g_ref_xyz.insert(g_ref_xyz.end(), {v.p.x, v.p.y, v.p.z});
}
// updateCudaRefMetrics: the last of the three; hands the background over
void updateCudaRefMetrics(const std::vector<GpuMetric>& metrics)
{
    g_ref_metrics.clear();
    for (const GpuMetric& m : metrics)  // glm::mat4, column-major; the symmetric 3x3 part
        g_ref_metrics.insert(g_ref_metrics.end(), {m[0][0], m[1][1], m[2][2], m[0][1], m[0][2], m[1][2]});
    if (!g_local_tets.empty() && !metrics.empty() && g_ref_xyz.size() == 3 * metrics.size())
        check(gm_mesh_set_local_background(mesh(), (uint32_t)(g_local_tets.size() / 8), g_local_tets.data(),
                                           (uint32_t)metrics.size(), g_ref_xyz.data(), g_ref_metrics.data()),
              "updateCudaRefMetrics");
}

// ---- the kd-tree and texture samplers ------------------------------------------

void installCudaKdTreeSampler() { g_sampler = GM_SAMPLER_KDTREE; apply_crew(); }  // KdTree.cu:50

// updateCudaKdNodes (KdTree.cu:58)
void updateCudaKdNodes(const std::vector<GpuKdNode>& nodes)
{
    if (nodes.empty()) return;  // clearCudaMemory
    std::vector<int32_t> children;
    std::vector<double> sep, metrics;
    for (const GpuKdNode& n : nodes)
    {
        children.insert(children.end(), {n.left, n.right});
        sep.insert(sep.end(), {n.separator.x, n.separator.y, n.separator.z, n.separator.w});
        const GpuMetric& m = n.metric;
        metrics.insert(metrics.end(), {m[0][0], m[1][1], m[2][2], m[0][1], m[0][2], m[1][2]});
    }
    check(gm_mesh_set_kd_nodes(mesh(), (uint32_t)nodes.size(), children.data(), sep.data(), metrics.data()),
          "updateCudaKdNodes");
}

void installCudaTextureSampler() { g_sampler = GM_SAMPLER_TEXTURE; apply_crew(); }  // Texture.cu:33

// updateCudaSamplerTextures (Texture.cu:66)
void updateCudaSamplerTextures(const std::vector<glm::vec4>& topLine, const std::vector<glm::vec4>& sideTri,
                               const glm::mat4& texTransform, const glm::ivec3 texDims)
{
    if (texDims.x == 0 || texDims.y == 0 || texDims.z == 0) return;  // clearCudaMemory
    // texTransform = scale(1 / extents) * translate(-minBounds) (TextureSampler.cpp:306-309)
    const int32_t dims[3] = {texDims.x, texDims.y, texDims.z};
    double lo[3], ext[3];
    for (int k = 0; k < 3; ++k)
    {
        ext[k] = 1.0 / texTransform[k][k];
        lo[k] = -texTransform[3][k] * ext[k];
    }
    // topLine = the metric's first column (xx, xy, xz), sideTri = (yy, yz, zz)
    std::vector<double> metrics;
    for (size_t c = 0; c < topLine.size(); ++c)
        metrics.insert(metrics.end(),
                       {topLine[c].x, sideTri[c].x, sideTri[c].z, topLine[c].y, topLine[c].z, sideTri[c].y});
    check(gm_mesh_set_texture(mesh(), dims, lo, ext, metrics.data()), "updateCudaSamplerTextures");
}

// ---- evaluation ---------------------------------------------------------------

// evaluateCudaMeshQuality (Evaluating/Evaluate.cu:55): the launch shape
// arguments are the reference's; the library sizes its own grid
void evaluateCudaMeshQuality(size_t, size_t, QualityHistogram& histogram)
{
    gm_quality q;
    check(gm_evaluate(mesh(), &q), "evaluateCudaMeshQuality");
    for (size_t b = 0; b < histogram.bucketCount() && b < GM_HIST_BUCKETS; ++b)
        histogram.setBucket(b, (int)q.buckets[b]);
    histogram.setSampleCount(q.count);
    histogram.setMinimumQuality(q.min);
    histogram.setInvQualitySum(q.inv_sum);
}

// ---- vertex-wise smoothers ------------------------------------------------------

// installCudaNelderMeadSmoother (Smoothing/VertexWise/NelderMead.cu:157)
void installCudaNelderMeadSmoother(float conv, int cycles, float shift, float a, float b, float g, float)
{
    g_smoother = GM_SMOOTH_NELDER_MEAD;
    const double p[6] = {shift, (double)cycles, conv, a, b, g};
    std::copy(p, p + 6, g_params);
}
// installCudaGradientDescentSmoother (GradientDescent.cu:115)
void installCudaGradientDescentSmoother(int cycles, float shift)
{
    g_smoother = GM_SMOOTH_GRADIENT_DESCENT;
    g_params[0] = shift;
    g_params[1] = cycles;
}
// the multi-thread-per-vertex drivers (MultiElemNM.cu:294, MultiElemGradDsnt.cu:270,
// MultiPosGradDsnt.cu, PatchGradDsnt.cu): the warp-per-vertex kernels already
// spread a patch over 32 lanes, so they bind to the same smoothers
void installCudaMultiElemNMSmoother(float conv, int cycles, float shift, float a, float b, float g, float d)
{
    installCudaNelderMeadSmoother(conv, cycles, shift, a, b, g, d);
}
void installCudaMultiElemGradDsntSmoother(int cycles, float shift) { installCudaGradientDescentSmoother(cycles, shift); }
void installCudaMultiPosGradDsntSmoother(int cycles, float shift) { installCudaGradientDescentSmoother(cycles, shift); }
void installCudaPatchGradDsntSmoother(int cycles, float shift) { installCudaGradientDescentSmoother(cycles, shift); }
// installCudaSpawnSearchSmoother (SpawnSearch.cu:192): the offsets are the
// fixed 4x4x4 lattice, built inside
void installCudaSpawnSearchSmoother(float moveCoeff, const std::vector<glm::vec4>)
{
    g_smoother = GM_SMOOTH_SPAWN_SEARCH;
    g_params[0] = moveCoeff;
    g_params[1] = 2;
}
// installCudaSpringLaplaceSmoother (SpringLaplace.cu:18), installCudaQualityLaplaceSmoother (QualityLaplace.cu:65)
void installCudaSpringLaplaceSmoother(float moveCoeff)
{
    g_smoother = GM_SMOOTH_SPRING_LAPLACE;
    g_params[0] = moveCoeff;
}
void installCudaQualityLaplaceSmoother(float moveCoeff)
{
    g_smoother = GM_SMOOTH_QUALITY_LAPLACE;
    g_params[0] = moveCoeff;
}

// smoothCudaVertices (SmoothVertices.cu:28), smoothCudaSpawnVertices (SpawnSearch.cu:220)
// and the multi-thread drivers' launchers: one colour's GPU dispatch
void smoothCudaVertices(const NodeGroups::GpuDispatch& d)
{
    check(gm_smooth_group(mesh(), g_smoother, g_params, (uint32_t)d.gpuBufferBase, (uint32_t)d.gpuBufferSize),
          "smoothCudaVertices");
    check(gm_mesh_sync(mesh()), "smoothCudaVertices");
}
void smoothCudaSpawnVertices(const NodeGroups::GpuDispatch& d) { smoothCudaVertices(d); }
void smoothCudaMultiElemNMVertices(const NodeGroups::GpuDispatch& d) { smoothCudaVertices(d); }
void smoothCudaMultiElemGradDsntVertices(const NodeGroups::GpuDispatch& d) { smoothCudaVertices(d); }
void smoothCudaMultiPosGradDsntVertices(const NodeGroups::GpuDispatch& d) { smoothCudaVertices(d); }
void smoothCudaPatchGradDsntVertices(const NodeGroups::GpuDispatch& d) { smoothCudaVertices(d); }

// ---- GETMe -------------------------------------------------------------------------

// installCudaGetmeSmoother (Smoothing/ElementWise/GETMe.cu:268): lambda 0.78
void installCudaGetmeSmoother() { g_params[0] = 0.78; }
// vertexAccumCudaInstall / Deinstall (VertexAccum.cu:46,70): the corner
// buffer is the mesh's own
void vertexAccumCudaInstall(size_t) {}
void vertexAccumCudaDeinstall() {}
// smoothCudaElements (SmoothElements.cu:41)
void smoothCudaElements(size_t, size_t) { check(gm_getme_elements(mesh(), g_params), "smoothCudaElements"); }
// updateCudaSmoothedElementsVertices (UpdateVertices.cu:47)
void updateCudaSmoothedElementsVertices(const NodeGroups::GpuDispatch& d, size_t)
{
    check(gm_getme_update_group(mesh(), g_params, (uint32_t)d.gpuBufferBase, (uint32_t)d.gpuBufferSize),
          "updateCudaSmoothedElementsVertices");
    check(gm_mesh_sync(mesh()), "updateCudaSmoothedElementsVertices");
}
