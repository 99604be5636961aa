// Checker harness around the reference's own CPU code (compiled from the
// reference's sources by oracle/refbuild.py into oracle/_ref/libgmref.so).
//
// TEST INFRASTRUCTURE ONLY: the tests load this library to pin the FP64 port
// (oracle/gm_oracle.c) and the product's topology against the reference
// itself.  It drives the reference's public classes: Mesh::compileTopology
// (with NodeGroups::build), MeshCrew, the evaluators' Serial / Thread mesh
// evaluation, and AbstractSmoother::smoothMesh with the "Thread"
// implementation for the vertex-wise smoothers (colour-major, one barrier per
// colour).  GETMe has only a Serial driver in the reference; a subclass
// replays it colour-major through the protected smoothTets / smoothPris /
// smoothHexs / updateVertexPositions.  The sine-graded metric is added as a
// sampler plugin through AbstractSampler's interface.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "Boundaries/BoundaryFree.h"
#include "Boundaries/BoxBoundary.h"
#include "Boundaries/PipeBoundary.h"
#include "Boundaries/ShellBoundary.h"
#include "Boundaries/SphereBoundary.h"
#include "Boundaries/TetBoundary.h"
#include "DataStructures/Mesh.h"
#include "DataStructures/MeshCrew.h"
#include "DataStructures/NodeGroups.h"
#include "DataStructures/OptimizationPlot.h"
#include "DataStructures/QualityHistogram.h"
#include "DataStructures/Schedule.h"
#include "Evaluators/MeanRatioEvaluator.h"
#include "Evaluators/MetricConformityEvaluator.h"
#include "Measurers/AbstractMeasurer.h"
#include "Samplers/AnalyticSampler.h"
#include "Samplers/KdTreeSampler.h"
#include "Samplers/LocalSampler.h"
#include "Samplers/TextureSampler.h"
#include "Samplers/UniformSampler.h"
#include "Smoothers/ElementWise/GetmeSmoother.h"
#include "Smoothers/ElementWise/VertexAccum.h"
#include "Smoothers/VertexWise/GradientDescentSmoother.h"
#include "Smoothers/VertexWise/NelderMeadSmoother.h"
#include "Smoothers/VertexWise/QualityLaplaceSmoother.h"
#include "Smoothers/VertexWise/SpawnSearchSmoother.h"
#include "Smoothers/VertexWise/SpringLaplaceSmoother.h"
#include "Serialization/JsonDeserializer.h"
#include "Serialization/JsonSerializer.h"

namespace {

void no_cuda_install() {}

// s^2 diag(1 + 9 sin^2(4 pi x), 1, 1): a sampler plugin with UniformSampler's shape
class SineSampler : public AbstractSampler
{
public:
    SineSampler() : AbstractSampler("Sine", "", no_cuda_install) {}
    bool isMetricWise() const override { return true; }
    bool useComputedMetric() const override { return false; }
    void updateAnalyticalMetric(const Mesh&) override {}
    void updateComputedMetric(const Mesh&, const std::shared_ptr<LocalSampler>&) override {}
    MeshMetric metricAt(const glm::dvec3& p, uint&) const override
    {
        double sx = std::sin(4.0 * 3.14159265358979323846 * p.x);
        double s2 = scalingSqr();
        return MeshMetric(glm::dvec3(s2 * (1.0 + 9.0 * sx * sx), 0, 0), glm::dvec3(0, s2, 0), glm::dvec3(0, 0, s2));
    }
    void releaseDebugMesh() override {}
    const Mesh& debugMesh() override { return _mesh; }

private:
    Mesh _mesh;
};

// GETMe in colour-major order: element pass, then the vertex update group by group
class ColourMajorGetme : public GetmeSmoother
{
public:
    void pass(Mesh& mesh, const MeshCrew& crew)
    {
        size_t nv = mesh.verts.size();
        _vertexAccums = new IVertexAccum*[nv];
        for (size_t i = 0; i < nv; ++i) _vertexAccums[i] = new NotThreadSafeVertexAccum();
        smoothTets(mesh, crew, 0, mesh.tets.size());
        smoothPris(mesh, crew, 0, mesh.pris.size());
        smoothHexs(mesh, crew, 0, mesh.hexs.size());
        for (const NodeGroups::ParallelGroup& g : mesh.nodeGroups().parallelGroups())
            updateVertexPositions(mesh, crew, g.undispatchedNodes);
        for (size_t i = 0; i < nv; ++i) delete _vertexAccums[i];
        delete[] _vertexAccums;
        _vertexAccums = nullptr;
    }
};

// 0 free, 1 box, 2 sphere, 3 tet, 4 pipe, 5 shell
std::shared_ptr<AbstractBoundary> make_boundary(int b)
{
    switch (b)
    {
    case 1: return std::shared_ptr<AbstractBoundary>(new BoxBoundary());
    case 2: return std::shared_ptr<AbstractBoundary>(new SphereBoundary());
    case 3: return std::shared_ptr<AbstractBoundary>(new TetBoundary());
    case 4: return std::shared_ptr<AbstractBoundary>(new PipeBoundary());
    case 5: return std::shared_ptr<AbstractBoundary>(new ShellBoundary());
    default: return std::shared_ptr<AbstractBoundary>(new BoundaryFree());
    }
}

void fill_mesh(Mesh& mesh, const std::shared_ptr<AbstractBoundary>& b, int64_t nv, const double* pos,
               const int32_t* cid, int64_t nt, const uint32_t* tets, int64_t np, const uint32_t* pris, int64_t nh,
               const uint32_t* hexs)
{
    mesh.setBoundary(b);
    for (int64_t v = 0; v < nv; ++v)
    {
        mesh.verts.push_back(MeshVert(glm::dvec3(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]), (uint)v));
        mesh.topos.push_back(MeshTopo(b->constraint(cid[v])));
    }
    for (int64_t i = 0; i < nt; ++i)
        mesh.tets.push_back(MeshTet(tets[4 * i], tets[4 * i + 1], tets[4 * i + 2], tets[4 * i + 3]));
    for (int64_t i = 0; i < np; ++i)
    {
        const uint32_t* e = pris + 6 * i;
        mesh.pris.push_back(MeshPri(e[0], e[1], e[2], e[3], e[4], e[5]));
    }
    for (int64_t i = 0; i < nh; ++i)
    {
        const uint32_t* e = hexs + 8 * i;
        mesh.hexs.push_back(MeshHex(e[0], e[1], e[2], e[3], e[4], e[5], e[6], e[7]));
    }
}

struct RefJson
{
    Mesh mesh;
};

struct Ref
{
    Mesh mesh;
    std::shared_ptr<AbstractBoundary> boundary;
    MeshCrew crew;
    std::shared_ptr<AbstractSampler> sampler;
    std::shared_ptr<AbstractEvaluator> evaluator;
};

}  // namespace

extern "C" {

// boundary: 0 free, 1 box, 2 sphere, 3 tet; cid: constraint id per vertex
void* ref_create(int boundary, int64_t nv, const double* pos, const int32_t* cid, int64_t nt, const uint32_t* tets,
                 int64_t np, const uint32_t* pris, int64_t nh, const uint32_t* hexs)
{
    Ref* r = new Ref();
    r->boundary = make_boundary(boundary);
    fill_mesh(r->mesh, r->boundary, nv, pos, cid, nt, tets, np, pris, nh, hexs);
    r->mesh.compileTopology(false);
    return r;
}

void ref_destroy(void* h) { delete static_cast<Ref*>(h); }

// new vertex index -> input index (the vertex cache word carries it through NodeGroups' permutation)
void ref_get_perm(void* h, uint32_t* perm)
{
    Ref* r = static_cast<Ref*>(h);
    for (size_t i = 0; i < r->mesh.verts.size(); ++i) perm[i] = r->mesh.verts[i].c;
}

int64_t ref_ngroups(void* h) { return (int64_t) static_cast<Ref*>(h)->mesh.nodeGroups().count(); }

void ref_get_groups(void* h, int64_t* base, uint32_t* members, int64_t* ranges)
{
    Ref* r = static_cast<Ref*>(h);
    const auto& groups = r->mesh.nodeGroups().parallelGroups();
    base[0] = 0;
    for (size_t g = 0; g < groups.size(); ++g)
    {
        const auto& G = groups[g];
        std::memcpy(members + base[g], G.undispatchedNodes.data(), sizeof(uint32_t) * G.undispatchedNodes.size());
        base[g + 1] = base[g] + (int64_t)G.undispatchedNodes.size();
        int64_t* rr = ranges + 6 * g;
        rr[0] = G.boundaryRange.begin;
        rr[1] = G.boundaryRange.end;
        rr[2] = G.subsurfaceRange.begin;
        rr[3] = G.subsurfaceRange.end;
        rr[4] = G.interiorRange.begin;
        rr[5] = G.interiorRange.end;
    }
}

void ref_get_tets(void* h, uint32_t* out)
{
    Ref* r = static_cast<Ref*>(h);
    for (size_t i = 0; i < r->mesh.tets.size(); ++i)
        for (int k = 0; k < 4; ++k) out[4 * i + k] = r->mesh.tets[i].v[k];
}

// sampler: 0 uniform, 1 analytic, 2 sine, 3 local, 4 kd-tree, 5 texture;
// evaluator: 0 mean ratio, 1 metric conformity; depth: the discretization
// depth of the kd-tree and texture samplers (-1: from the vertex count)
void ref_set_crew(void* h, int sampler, int evaluator, double scaling, double aspect, int depth)
{
    Ref* r = static_cast<Ref*>(h);
    if (sampler == 1) r->sampler.reset(new AnalyticSampler());
    else if (sampler == 2) r->sampler.reset(new SineSampler());
    else if (sampler == 3) r->sampler.reset(new LocalSampler());
    else if (sampler == 4) r->sampler.reset(new KdTreeSampler());
    else if (sampler == 5) r->sampler.reset(new TextureSampler());
    else r->sampler.reset(new UniformSampler());
    r->sampler->setScaling(scaling);
    r->sampler->setAspectRatio(aspect);
    r->sampler->setDiscretizationDepth(depth);
    // GpuMeshCharacter::updateSampling: the background mesh (and the kd-tree
    // or texture sampled from it) from the mesh as it is now
    if (sampler >= 3) r->sampler->updateAnalyticalMetric(r->mesh);
    if (evaluator == 1) r->evaluator.reset(new MetricConformityEvaluator());
    else r->evaluator.reset(new MeanRatioEvaluator());
    r->crew.setSampler(r->mesh, r->sampler);
    r->crew.setEvaluator(r->mesh, r->evaluator);
}

int ref_measurer_is_metric_wise(void* h)
{
    Ref* r = static_cast<Ref*>(h);
    return r->crew.sampler().isMetricWise() ? 1 : 0;
}

// out: min, inv_sum (from count / harmonic mean), count, 20 buckets
void ref_evaluate(void* h, int thread, double* out)
{
    Ref* r = static_cast<Ref*>(h);
    QualityHistogram hist;
    if (thread) r->crew.evaluator().evaluateMeshQualityThread(r->mesh, r->crew.sampler(), r->crew.measurer(), hist);
    else r->crew.evaluator().evaluateMeshQualitySerial(r->mesh, r->crew.sampler(), r->crew.measurer(), hist);
    out[0] = hist.minimumQuality();
    out[1] = hist.sampleCount() / hist.harmonicMean();
    out[2] = (double)hist.sampleCount();
    for (int b = 0; b < 20; ++b) out[3 + b] = hist.buckets()[b];
}

double ref_element_quality(void* h, int type, int64_t idx)
{
    Ref* r = static_cast<Ref*>(h);
    const AbstractEvaluator& e = r->crew.evaluator();
    if (type == 0) return e.tetQuality(r->mesh, r->crew.sampler(), r->crew.measurer(), r->mesh.tets[idx]);
    if (type == 2) return e.priQuality(r->mesh, r->crew.sampler(), r->crew.measurer(), r->mesh.pris[idx]);
    return e.hexQuality(r->mesh, r->crew.sampler(), r->crew.measurer(), r->mesh.hexs[idx]);
}

double ref_patch_quality(void* h, int64_t v)
{
    Ref* r = static_cast<Ref*>(h);
    return r->crew.evaluator().patchQuality(r->mesh, r->crew.sampler(), r->crew.measurer(), (size_t)v);
}

double ref_local_size(void* h, int64_t v)
{
    Ref* r = static_cast<Ref*>(h);
    return r->crew.measurer().computeLocalElementSize(r->mesh, (uint)v);
}

// smoother: 0 NM, 1 GD, 2 spawn, 4 spring Laplace, 5 quality Laplace
// (reference "Thread" driver, colour-major), 3 GETMe (colour-major replay of
// the Serial driver)
void ref_smooth(void* h, int smoother, int passes)
{
    Ref* r = static_cast<Ref*>(h);
    if (smoother == 3)
    {
        ColourMajorGetme g;
        for (int p = 0; p < passes; ++p) g.pass(r->mesh, r->crew);
        return;
    }
    std::unique_ptr<AbstractSmoother> s;
    if (smoother == 0) s.reset(new NelderMeadSmoother());
    else if (smoother == 1) s.reset(new GradientDescentSmoother());
    else if (smoother == 4) s.reset(new SpringLaplaceSmoother());
    else if (smoother == 5) s.reset(new QualityLaplaceSmoother());
    else s.reset(new SpawnSearchSmoother());
    Schedule schedule;
    schedule.topoOperationEnabled = false;
    schedule.autoPilotEnabled = false;
    schedule.relocationPassCount = passes;
    OptimizationImpl impl;
    s->smoothMesh(r->mesh, r->crew, "Thread", schedule, impl);
}

void ref_get_pos(void* h, double* out)
{
    Ref* r = static_cast<Ref*>(h);
    for (size_t i = 0; i < r->mesh.verts.size(); ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + k] = r->mesh.verts[i].p[k];
}

void ref_set_pos(void* h, const double* in)
{
    Ref* r = static_cast<Ref*>(h);
    for (size_t i = 0; i < r->mesh.verts.size(); ++i)
        r->mesh.verts[i].p = glm::dvec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
}

// ---- JSON mesh files (Serialization/JsonSerializer.cpp, JsonDeserializer.cpp) ----

// JsonSerializer::serialize of a mesh given in arrays (before any topology
// compilation); returns 1 on success
int ref_json_write(const char* path, const char* model, int boundary, int64_t nv, const double* pos, const int32_t* cid,
                   int64_t nt, const uint32_t* tets, int64_t np, const uint32_t* pris, int64_t nh, const uint32_t* hexs)
{
    Mesh mesh;
    fill_mesh(mesh, make_boundary(boundary), nv, pos, cid, nt, tets, np, pris, nh, hexs);
    mesh.modelName = model;
    MeshCrew crew;
    return JsonSerializer().serialize(path, crew, mesh) ? 1 : 0;
}

// JsonDeserializer::deserialize; null when it fails
void* ref_json_read(const char* path)
{
    RefJson* r = new RefJson();
    std::vector<MeshMetric> metrics;
    if (!JsonDeserializer().deserialize(path, r->mesh, metrics))
    {
        delete r;
        return nullptr;
    }
    return r;
}

// out: vertices, topos, tets, prisms, hexes
void ref_json_counts(void* h, int64_t* out)
{
    const Mesh& m = static_cast<RefJson*>(h)->mesh;
    out[0] = (int64_t)m.verts.size();
    out[1] = (int64_t)m.topos.size();
    out[2] = (int64_t)m.tets.size();
    out[3] = (int64_t)m.pris.size();
    out[4] = (int64_t)m.hexs.size();
}

void ref_json_get(void* h, double* pos, int32_t* cid, uint32_t* tets, uint32_t* pris, uint32_t* hexs, char* model,
                  int64_t model_cap, char* bound, int64_t bound_cap)
{
    const Mesh& m = static_cast<RefJson*>(h)->mesh;
    for (size_t i = 0; i < m.verts.size(); ++i)
        for (int k = 0; k < 3; ++k) pos[3 * i + k] = m.verts[i].p[k];
    for (size_t i = 0; i < m.topos.size(); ++i) cid[i] = m.topos[i].snapToBoundary->id();
    for (size_t i = 0; i < m.tets.size(); ++i)
        for (int k = 0; k < 4; ++k) tets[4 * i + k] = m.tets[i].v[k];
    for (size_t i = 0; i < m.pris.size(); ++i)
        for (int k = 0; k < 6; ++k) pris[6 * i + k] = m.pris[i].v[k];
    for (size_t i = 0; i < m.hexs.size(); ++i)
        for (int k = 0; k < 8; ++k) hexs[8 * i + k] = m.hexs[i].v[k];
    std::snprintf(model, (size_t)model_cap, "%s", m.modelName.c_str());
    std::snprintf(bound, (size_t)bound_cap, "%s", m.boundary().name().c_str());
}

void ref_json_destroy(void* h) { delete static_cast<RefJson*>(h); }

// the boundary's constraint `id` applied to n points
void ref_boundary_project(int boundary, int id, int64_t n, const double* in, double* out)
{
    std::shared_ptr<AbstractBoundary> b = make_boundary(boundary);
    const AbstractConstraint* c = b->constraint(id);
    for (int64_t i = 0; i < n; ++i)
    {
        const glm::dvec3 p = (*c)(glm::dvec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        for (int k = 0; k < 3; ++k) out[3 * i + k] = p[k];
    }
}

}  // extern "C"
