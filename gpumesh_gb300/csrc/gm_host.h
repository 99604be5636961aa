// Host-side declarations shared by the C ABI translation units: error
// handling, device buffers and the gm_mesh object.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gpumesh_gb300.h"
#include "gm_internal.h"
#include "gm_launch.h"

namespace gm {

// An NVTX range for the lifetime of the object (per pass, per colour, per
// evaluation, per batch or job launch), for a profiler's timeline; without
// an attached tool a range costs one branch.
struct NvtxRange
{
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace gm

namespace gm {


struct ApiError : std::runtime_error
{
    gm_status status;
    ApiError(gm_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define GM_CUDA(call)                                                                                      \
    do                                                                                                     \
    {                                                                                                      \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            throw ApiError(e_ == cudaErrorMemoryAllocation ? GM_ERR_OUT_OF_MEMORY : GM_ERR_CUDA,           \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                            \
    } while (0)

inline void require(bool ok, const std::string& msg)
{
    if (!ok) throw ApiError(GM_ERR_INVALID_ARG, msg);
}

template <class F>
gm_status guarded(F&& f)
{
    try
    {
        f();
        return GM_OK;
    }
    catch (const ApiError& e)
    {
        set_error(e.what());
        return e.status;
    }
    catch (const std::bad_alloc&)
    {
        set_error("host allocation failed");
        return GM_ERR_OUT_OF_MEMORY;
    }
    catch (const std::exception& e)
    {
        set_error(e.what());
        return GM_ERR_STATE;
    }
}

// growable device buffer, owning its allocation (freed on destruction;
// moved, never copied)
template <class T>
struct DBuf
{
    T* p = nullptr;
    size_t cap = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), cap(o.cap)
    {
        o.p = nullptr;
        o.cap = 0;
    }
    DBuf& operator=(DBuf&& o) noexcept
    {
        if (this != &o)
        {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    // true when the buffer was (re)allocated
    bool reserve(size_t n)
    {
        if (n <= cap && p) return false;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        GM_CUDA(cudaMalloc(&p, bytes));
        cap = std::max<size_t>(n, 1);
        return true;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

template <class T>
void upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s)
{
    b.reserve(n);
    if (n) GM_CUDA(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
}

// the smoother parameter block of the C ABI (GM_PARAMS doubles), with defaults
SmoothParams parse_smooth_params(int smoother, const double* params);

// LocalSampler's background mesh in device memory.  `part` holds the local
// members of a LocalField pointing into the buffers, `field` a device copy of
// it alone (the walks of the kd-tree and texture builds); host copies of the
// positions and tets serve those builds.  Shared by a mesh and its clones.
struct LocalBackground
{
    DBuf<uint4> tv, tn;
    DBuf<float4> pf;
    DBuf<double> pd, md;
    DBuf<float4> mf;  // 2 per vertex
    DBuf<uint32_t> cell, ecache;
    DBuf<LocalField> field;
    LocalField part{};
    std::vector<double> pd_h;
    std::vector<uint4> tv_h;
    uint32_t nbg = 0, nref = 0;
    bool from_mesh = false;  // built from the mesh (analytic vertex metrics) rather than given
    double scaling = 0.0, aspect = 0.0;
    size_t bytes() const
    {
        return (tv.cap + tn.cap) * 16 + pf.cap * 16 + pd.cap * 8 + md.cap * 8 + mf.cap * 16 +
               (cell.cap + ecache.cap) * 4 + sizeof(LocalField);
    }
};

// KdTreeSampler's nodes (pre-order) and TextureSampler's grid in device
// memory; `given` when handed over by the caller rather than built from the
// mesh (then kept across scaling changes and topology uploads)
struct KdTreeData
{
    DBuf<int2> child;
    DBuf<float4> sepf;
    DBuf<Plane4d> sepd;
    DBuf<float4> mf;  // 2 per node
    DBuf<double> md;
    uint32_t n = 0;
    bool given = false;
    int depth = -1;
    double scaling = 0.0, aspect = 0.0;
    size_t bytes() const { return child.cap * 8 + sepf.cap * 16 + sepd.cap * 32 + mf.cap * 16 + md.cap * 8; }
};

struct TextureData
{
    DBuf<float4> mf;  // 2 per cell
    DBuf<double> md;
    int g[3] = {0, 0, 0};
    double lo[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
    bool given = false;
    int depth = -1;
    double scaling = 0.0, aspect = 0.0;
    size_t bytes() const { return mf.cap * 16 + md.cap * 8; }
};

}  // namespace gm

using namespace gm;

struct gm_mesh
{
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = 0;
    uint32_t nv = 0, nt = 0, np = 0, nh = 0;
    DBuf<float4> pos;
    DBuf<uint4> tets;
    DBuf<uint32_t> pris;
    DBuf<uint4> hexs;
    DBuf<uint32_t> ve_off, ve, vv_off, vv;
    uint32_t n_ve = 0, n_vv = 0;  // entries of ve / vv
    DBuf<unsigned int> bounds;    // bounds status {what, index} (checked builds report it)
    DBuf<int32_t> cid;
    DBuf<Constraint> con;
    int ncon = 0;
    DBuf<uint32_t> members;
    uint32_t n_members = 0;
    std::vector<uint32_t> group_base;
    DBuf<Quality> quality;
    uint32_t n_quality_slots = 0;
    DBuf<EvalPartial> parts;
    DBuf<float4> corners;
    DBuf<float4> saved;
    DBuf<Counters> ctr;
    // FP64 acceptance hand-over: per-member slots and one counter per group
    DBuf<uint32_t> def_v;
    DBuf<float4> def_old, def_new;
    DBuf<uint32_t> def_count;
    Crew crew{};
    int ks = 4;
    int maxe = 32;
    int max_incident = 0;  // the largest number of elements around a vertex (maxe is it padded to 32)
    int warps_per_block = 4;
    std::vector<float4> staging;  // host conversion buffer
    // device-resident job (gm_job_*): a CUDA graph running a whole stop-rule
    // schedule; it captures the buffers and crew above, so anything that
    // changes them drops it
    cudaGraph_t job_graph = nullptr;
    cudaGraphExec_t job_exec = nullptr;
    DBuf<int> job_counter;    // passes done
    DBuf<Quality> job_fresh;  // evaluation of the pass just run
    uint32_t job_max_passes = 0;
    unsigned long long job_body_kernels = 0;  // kernels of one pass of the job loop
    // background-mesh samplers: the parts, and the LocalField assembled from
    // them that crew.local points to
    std::shared_ptr<LocalBackground> local;
    std::shared_ptr<KdTreeData> kd;
    std::shared_ptr<TextureData> tex;
    DBuf<LocalField> field;
    int depth = -1;  // AbstractSampler::discretizationDepth

    MeshView view() const
    {
        MeshView v;
        v.nv = nv;
        v.nt = nt;
        v.np = np;
        v.nh = nh;
        v.pos = pos.p;
        v.tets = tets.p;
        v.pris = pris.p;
        v.hexs = hexs.p;
        v.ve_off = ve_off.p;
        v.ve = ve.p;
        v.vv_off = vv_off.p;
        v.vv = vv.p;
        v.cid = cid.p;
        v.con = con.p;
        v.ncon = ncon;
        v.ve_len = n_ve;
        v.vv_len = n_vv;
        v.bounds = bounds.p;
        return v;
    }

    // evaluator x measurer variant of the vertex kernels
    int variant() const
    {
        if (crew.evaluator == GM_EVALUATOR_METRIC_CONFORMITY)  // general metric, or a diagonal one
            return (crew.sampler == GM_SAMPLER_UNIFORM || crew.sampler == GM_SAMPLER_SINE) ? kVarMCDiag : kVarMC;
        return crew.measurer == GM_MEASURER_METRIC_WISE ? kVarMRWise : kVarMRFree;
    }
    // variant of the GETMe element pass, whose volumes also follow the measurer
    int element_variant() const
    {
        if (crew.evaluator == GM_EVALUATOR_METRIC_CONFORMITY)
            return crew.measurer == GM_MEASURER_METRIC_WISE ? kVarMCWise : kVarMC;
        return crew.measurer == GM_MEASURER_METRIC_WISE ? kVarMRWise : kVarMRFree;
    }
    int maxk() const { return (np || nh) ? 8 : 4; }
    // element set of the evaluation kernel: 4 tets only, 8 mixed, 9 hexes only
    int elem_set() const { return (nt == 0 && np == 0 && nh) ? 9 : maxk(); }
};

namespace gm {
// Background-mesh samplers (gm_local.cu).  LocalSampler backgrounds: from
// the resident mesh with the analytic metric of `crew` at its vertices, or
// given by the caller; kd-trees and textures: sampled from a background built
// from the mesh, or given.
std::shared_ptr<LocalBackground> local_background_from_mesh(gm_mesh* m, const Crew& crew);
std::shared_ptr<LocalBackground> local_background_given(gm_mesh* m, uint32_t ntets, const uint32_t* tets8,
                                                        uint32_t nverts, const double* xyz, const double* metrics6);
std::shared_ptr<KdTreeData> kdtree_from_mesh(gm_mesh* m, const LocalBackground& bg, const Crew& crew, int depth);
std::shared_ptr<KdTreeData> kdtree_given(gm_mesh* m, uint32_t n, const int32_t* children2, const double* sep4,
                                         const double* metrics6);
std::shared_ptr<TextureData> texture_from_mesh(gm_mesh* m, const LocalBackground& bg, const Crew& crew, int depth);
std::shared_ptr<TextureData> texture_given(gm_mesh* m, const int32_t* dims3, const double* lo3, const double* ext3,
                                           const double* metrics6);
// builds what crew c's sampler needs (keeping what is still valid), commits
// the parts to the mesh and points c.local at the assembled field
void prepare_sampler(gm_mesh* m, Crew& c);
// uploads the LocalField assembled from the mesh's parts; its device address
const LocalField* assemble_field(gm_mesh* m);
// a new topology: parts built from the old mesh are dropped, and rebuilt
// while a background-mesh sampler is installed
void sampler_topology_changed(gm_mesh* m);
size_t sampler_bytes(const gm_mesh* m);
}  // namespace gm

