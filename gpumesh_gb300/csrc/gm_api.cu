// C ABI of libgpumesh_gb300.so (include/gpumesh_gb300.h): device-resident
// meshes, uploads in the reference's buffer layouts, evaluation and
// relocation launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

#include "gm_host.h"

namespace gm {

static std::atomic<unsigned long long> g_launches{0};
static thread_local CaptureTally* tl_tally = nullptr;

void note_launch()
{
    if (tl_tally) ++tl_tally->kernels;
    else g_launches.fetch_add(1, std::memory_order_relaxed);
}

void add_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

CaptureTally::CaptureTally() : prev(tl_tally) { tl_tally = this; }
CaptureTally::~CaptureTally() { tl_tally = prev; }

}  // namespace gm

namespace gm {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace gm

using namespace gm;

namespace {

#ifdef GM_BOUNDS_CHECK
constexpr bool kBoundsChecked = true;
#else
constexpr bool kBoundsChecked = false;
#endif

// In a bounds-checked build, the synchronising calls read the mesh's bounds
// status and turn a recorded failure into an error (and clear it).
void report_bounds(gm_mesh* m)
{
    if (!kBoundsChecked || !m->bounds.p) return;
    unsigned int w[2] = {0, 0};
    GM_CUDA(cudaMemcpyAsync(w, m->bounds.p, sizeof(w), cudaMemcpyDeviceToHost, m->stream));
    GM_CUDA(cudaStreamSynchronize(m->stream));
    if (!w[0]) return;
    GM_CUDA(cudaMemsetAsync(m->bounds.p, 0, sizeof(w), m->stream));
    static const char* names[] = {"", "vertex", "vertex->element CSR", "vertex->vertex CSR", "tet", "prism", "hex",
                                  "GETMe corner"};
    throw ApiError(GM_ERR_STATE, std::string("device bounds check: ") + (w[0] < 8 ? names[w[0]] : "?") +
                                     " index " + std::to_string(w[1]) + " out of range (read as 0)");
}

void set_crew(gm_mesh* m, int sampler, int measurer, int evaluator, double scaling, double aspect)
{
    require(sampler >= 0 && sampler <= GM_SAMPLER_TEXTURE, "unknown sampler");
    require(measurer >= 0 && measurer <= 1, "unknown measurer");
    require(evaluator >= 0 && evaluator <= 1, "unknown evaluator");
    Crew c = m->crew;
    c.sampler = sampler;
    c.measurer = measurer;
    c.evaluator = evaluator;
    c.scaling = scaling;
    c.scaling2 = c.scaling * scaling;
    c.scaling3 = c.scaling2 * scaling;
    c.aspect = aspect;
    // AbstractSampler's fixed rotation (Samplers/AbstractSampler.cpp:30-40):
    // pi/4 about +z, then pi/4 about -y, composed on the right
    auto rot = [](const double* m3, double ang, double ax, double ay, double az, double* out) {
        double c_ = std::cos(ang), s_ = std::sin(ang);
        double n = 1.0 / std::sqrt(ax * ax + ay * ay + az * az);
        double a[3] = {ax * n, ay * n, az * n};
        double t[3] = {(1 - c_) * a[0], (1 - c_) * a[1], (1 - c_) * a[2]};
        double R[9];  // column-major
        R[0] = c_ + t[0] * a[0];
        R[1] = t[0] * a[1] + s_ * a[2];
        R[2] = t[0] * a[2] - s_ * a[1];
        R[3] = t[1] * a[0] - s_ * a[2];
        R[4] = c_ + t[1] * a[1];
        R[5] = t[1] * a[2] + s_ * a[0];
        R[6] = t[2] * a[0] + s_ * a[1];
        R[7] = t[2] * a[1] - s_ * a[0];
        R[8] = c_ + t[2] * a[2];
        for (int j = 0; j < 3; ++j)
            for (int r = 0; r < 3; ++r)
                out[j * 3 + r] = m3[0 * 3 + r] * R[j * 3 + 0] + m3[1 * 3 + r] * R[j * 3 + 1] + m3[2 * 3 + r] * R[j * 3 + 2];
    };
    double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, A[9];
    const double pi = 3.14159265358979323846;
    rot(I, pi / 4.0, 0, 0, 1, A);
    rot(A, pi / 4.0, 0, -1, 0, c.rot);
    for (int j = 0; j < 3; ++j)
        for (int r = 0; r < 3; ++r) c.rotinv[j * 3 + r] = c.rot[r * 3 + j];
    // the background mesh, kd-tree or texture the sampler samples
    prepare_sampler(m, c);
    m->crew = c;  // only once everything above succeeded
}

void update_patch_shape(gm_mesh* m, const uint32_t* ve_off_host)
{
    uint32_t mx = 0;
    for (uint32_t v = 0; v < m->nv; ++v) mx = std::max(mx, ve_off_host[v + 1] - ve_off_host[v]);
    m->maxe = std::max<int>(32, (int)((mx + 31) / 32 * 32));
    m->max_incident = (int)mx;
    m->ks = (m->nh || m->np) ? 8 : 4;
    size_t per = patch_smem_per_warp(m->ks, m->maxe);
    int wpb = 4;
    while (wpb > 1 && per * wpb > 96 * 1024) wpb >>= 1;
    if (per * wpb > 200 * 1024)
        throw ApiError(GM_ERR_UNSUPPORTED, "a vertex has " + std::to_string(mx) +
                                               " incident elements, more than the relocation kernels stage");
    m->warps_per_block = wpb;
}

void upload_csr(gm_mesh* m, const std::vector<uint32_t>& ve_off, const std::vector<uint32_t>& ve,
                const std::vector<uint32_t>& vv_off, const std::vector<uint32_t>& vv)
{
    upload(m->ve_off, ve_off.data(), ve_off.size(), m->stream);
    upload(m->ve, ve.data(), ve.size(), m->stream);
    upload(m->vv_off, vv_off.data(), vv_off.size(), m->stream);
    upload(m->vv, vv.data(), vv.size(), m->stream);
    m->n_ve = (uint32_t)ve.size();
    m->n_vv = (uint32_t)vv.size();
    update_patch_shape(m, ve_off.data());
}

void check_conn(const uint32_t* c, size_t n, uint32_t nv, const char* what)
{
    for (size_t i = 0; i < n; ++i)
        if (c[i] >= nv) throw ApiError(GM_ERR_INVALID_ARG, std::string(what) + " references vertex " +
                                                                std::to_string(c[i]) + " >= vertex count");
}

void upload_positions(gm_mesh* m, uint32_t nv, const double* xyz)
{
    m->staging.resize(nv);
    for (uint32_t v = 0; v < nv; ++v)
    {
        double x = xyz[3 * (size_t)v], y = xyz[3 * (size_t)v + 1], z = xyz[3 * (size_t)v + 2];
        if (!(std::isfinite(x) && std::isfinite(y) && std::isfinite(z)))
            throw ApiError(GM_ERR_INVALID_ARG, "vertex " + std::to_string(v) + " has a non-finite position");
        m->staging[v] = make_float4((float)x, (float)y, (float)z, 0.f);
    }
    upload(m->pos, m->staging.data(), nv, m->stream);
    m->nv = nv;
}

template <int K>
void upload_conn(gm_mesh* m, uint32_t n, const uint32_t* words, uint32_t stride, std::vector<uint32_t>& packed)
{
    require(stride >= (uint32_t)K, "element stride shorter than the element");
    packed.resize((size_t)n * K);
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < K; ++k) packed[(size_t)i * K + k] = words[(size_t)i * stride + k];
}

SmoothParams parse_params(int smoother, const double* p)
{
    SmoothParams sp{};
    sp.alpha = 1.f;
    sp.beta = 0.5f;
    sp.gamma = 2.f;
    sp.convergence = 1e-4f;
    sp.accept_q = 1e-3f;
    switch (smoother)
    {
    case GM_SMOOTH_NELDER_MEAD:
        sp.shift = (float)(p ? p[0] : 1.0 / 24.0);
        sp.cycles = p ? (int)p[1] : 12;
        sp.convergence = (float)(p ? p[2] : 1e-4);
        sp.alpha = (float)(p ? p[3] : 1.0);
        sp.beta = (float)(p ? p[4] : 0.5);
        sp.gamma = (float)(p ? p[5] : 2.0);
        break;
    case GM_SMOOTH_GRADIENT_DESCENT:
        sp.shift = (float)(p ? p[0] : 1.0 / 75.0);
        sp.cycles = p ? (int)p[1] : 5;
        break;
    case GM_SMOOTH_SPAWN_SEARCH:
        sp.shift = (float)(p ? p[0] : 1.0 / 20.0);
        sp.cycles = p ? (int)p[1] : 2;
        break;
    case GM_SMOOTH_GETME:
        sp.lambda = (float)(p ? p[0] : 0.78);
        break;
    case GM_SMOOTH_SPRING_LAPLACE:
    case GM_SMOOTH_QUALITY_LAPLACE:
        sp.shift = (float)(p ? p[0] : 0.35);  // SLMoveCoeff / QLMoveCoeff
        break;
    default:
        throw ApiError(GM_ERR_INVALID_ARG, "unknown smoother " + std::to_string(smoother));
    }
    if (p && p[7] > 0) sp.accept_q = (float)p[7];
    require(sp.cycles >= 0 && sp.cycles <= 4096, "cycle count out of range");
    return sp;
}

void require_mesh(const gm_mesh* m)
{
    require(m != nullptr, "null mesh");
    require(m->nv > 0 && m->pos.p, "mesh has no vertices");
    require(m->cid.p != nullptr, "mesh has no topology");
}

void require_groups(const gm_mesh* m) { require(!m->group_base.empty(), "mesh has no independent groups"); }

void ensure_deferred(gm_mesh* m)
{
    require(m->n_members > 0 || !m->group_base.empty(), "mesh has no independent groups");
    m->def_v.reserve(m->n_members);
    m->def_old.reserve(m->n_members);
    m->def_new.reserve(m->n_members);
    m->def_count.reserve(m->group_base.size() + 2);
}

// one group: the FP32 relocation (or GETMe update) launch, then the FP64
// acceptance launch for the vertices it handed over
void relocate_group(gm_mesh* m, int smoother, const SmoothParams& sp, uint32_t base, uint32_t count, uint32_t slot)
{
    NvtxRange range("gm colour");
    if (count == 0) return;
    RelocLaunch L;
    L.variant = m->variant();
    L.maxk = m->maxk();
    L.m = m->view();
    L.crew = m->crew;
    L.sp = sp;
    L.members = m->members.p + base;
    L.count = count;
    L.maxe = m->maxe;
    L.max_incident = m->max_incident;
    L.warps_per_block = m->warps_per_block;
    L.sm_count = m->sm_count;
    L.ctr = m->ctr.p;
    L.def = Deferred{m->def_v.p, m->def_old.p, m->def_new.p, m->def_count.p + slot};
    L.slot_base = base;
    L.stream = m->stream;
    switch (smoother)
    {
    case GM_SMOOTH_NELDER_MEAD: GM_CUDA(launch_relocate_nm(L)); break;
    case GM_SMOOTH_GRADIENT_DESCENT: GM_CUDA(launch_relocate_gd(L)); break;
    case GM_SMOOTH_SPAWN_SEARCH: GM_CUDA(launch_relocate_spawn(L)); break;
    case GM_SMOOTH_SPRING_LAPLACE: GM_CUDA(launch_relocate_spring(L)); break;
    case GM_SMOOTH_QUALITY_LAPLACE: GM_CUDA(launch_relocate_qlaplace(L)); break;
    default: GM_CUDA(launch_getme_update(L, m->corners.p)); break;
    }
    GM_CUDA(launch_accept(L));
}

// one relocation pass: every colour in order (GETMe: the element pass first)
void enqueue_pass(gm_mesh* m, int smoother, const SmoothParams& sp)
{
    NvtxRange range("gm pass");
    ensure_deferred(m);
    size_t ng = m->group_base.size() - 1;
    GM_CUDA(cudaMemsetAsync(m->def_count.p, 0, (ng + 2) * sizeof(uint32_t), m->stream));
    if (smoother == GM_SMOOTH_GETME)
    {
        m->corners.reserve(4 * (size_t)m->nt + 6 * (size_t)m->np + 8 * (size_t)m->nh);
        GM_CUDA(launch_getme_elements(m->element_variant(), m->view(), m->crew, sp.lambda, m->corners.p, m->sm_count,
                                      m->stream));
    }
    for (size_t g = 0; g < ng; ++g)
        relocate_group(m, smoother, sp, m->group_base[g], m->group_base[g + 1] - m->group_base[g], (uint32_t)g);
}

// at least n quality slots, keeping the recorded ones (synchronises on growth)
void ensure_quality_slots(gm_mesh* m, uint32_t n)
{
    if (n <= m->n_quality_slots) return;
    n = std::max<uint32_t>(n, 2 * m->n_quality_slots);
    Quality* fresh = nullptr;
    GM_CUDA(cudaMalloc(&fresh, n * sizeof(Quality)));
    if (m->quality.p && m->n_quality_slots)
        GM_CUDA(cudaMemcpyAsync(fresh, m->quality.p, m->n_quality_slots * sizeof(Quality), cudaMemcpyDeviceToDevice,
                                m->stream));
    GM_CUDA(cudaStreamSynchronize(m->stream));
    m->quality.release();
    m->quality.p = fresh;
    m->quality.cap = n;
    m->n_quality_slots = n;
}

// one evaluation into `out` (device)
void enqueue_evaluate(gm_mesh* m, Quality* out)
{
    NvtxRange range("gm evaluate");
    uint32_t total = m->nt + m->np + m->nh;
    int nb = evaluate_blocks(total, m->sm_count);
    if (m->parts.reserve(eval_scratch_slots(nb)))  // a fresh scratch starts with its ticket and bucket totals at 0
        GM_CUDA(cudaMemsetAsync(m->parts.p, 0, kEvalScratchHead, m->stream));
    // the launch uses at most nb blocks, whose scratch the reservation holds
    GM_CUDA(launch_evaluate(m->variant(), m->elem_set(), m->view(), m->crew, m->parts.p, nb, out, m->stream));
}

void drop_job(gm_mesh* m)
{
    if (m->job_exec) cudaGraphExecDestroy(m->job_exec);
    if (m->job_graph) cudaGraphDestroy(m->job_graph);
    m->job_exec = nullptr;
    m->job_graph = nullptr;
    m->job_max_passes = 0;
}

// The stop test of a device-resident job, one warp: store the evaluation of
// the pass just run in the next slot, count the pass, and continue while
// fewer than max_passes passes are done and the minimum quality rose by at
// least min_gain (the served workload's stop rule).
__global__ void job_rule_kernel(Quality* slots, const Quality* fresh, int* counter, double min_gain, int max_passes,
                                cudaGraphConditionalHandle loop)
{
    const int lane = threadIdx.x;
    const int c = __shfl_sync(0xffffffffu, lane == 0 ? *counter + 1 : 0, 0);
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(fresh);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(slots + c);
    if (lane < (int)(sizeof(Quality) / 8)) dst[lane] = src[lane];
    if (lane == 0)
    {
        *counter = c;
        const double gain = fresh->min - slots[c - 1].min;
        cudaGraphSetConditional(loop, (c < max_passes && gain >= min_gain) ? 1u : 0u);
    }
}

}  // namespace

namespace gm {
SmoothParams parse_smooth_params(int smoother, const double* p) { return parse_params(smoother, p); }
}  // namespace gm

extern "C" {

const char* gm_last_error(void) { return g_last_error.c_str(); }

const char* gm_status_string(gm_status s)
{
    switch (s)
    {
    case GM_OK: return "ok";
    case GM_ERR_INVALID_ARG: return "invalid argument";
    case GM_ERR_CUDA: return "CUDA error";
    case GM_ERR_OUT_OF_MEMORY: return "out of memory";
    case GM_ERR_UNSUPPORTED: return "unsupported";
    case GM_ERR_TIMEOUT: return "timeout";
    case GM_ERR_STATE: return "invalid state";
    default: return "unknown status";
    }
}

const char* gm_version(void) { return "gpumesh_gb300 sm_103a " __DATE__; }

namespace {

gm_status node_groups(uint32_t nv, const int32_t* cid, uint32_t nt, const uint32_t* tets, uint32_t np,
                      const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t permute, uint32_t* perm,
                      uint32_t* group_base, uint32_t* members, uint32_t* ranges, uint32_t* ngroups, bool device)
{
    return guarded([&] {
        require(nv > 0 && cid && perm && group_base && members && ngroups, "null argument");
        require((nt == 0 || tets) && (np == 0 || pris) && (nh == 0 || hexs), "null connectivity");
        check_conn(tets, (size_t)nt * 4, nv, "tet");
        check_conn(pris, (size_t)np * 6, nv, "prism");
        check_conn(hexs, (size_t)nh * 8, nv, "hex");
        HostMeshView in;
        in.nv = nv;
        in.nt = nt;
        in.np = np;
        in.nh = nh;
        in.cid = cid;
        in.tets = tets;
        in.pris = pris;
        in.hexs = hexs;
        ColourSource source;
        if (device)
            source = [&](const std::vector<uint32_t>& e_off, const std::vector<uint32_t>& e, std::vector<int>& c) {
                device_colours(in, e_off, e, c);
            };
        Topology t = build_topology(in, permute != 0, source);
        std::copy(t.perm.begin(), t.perm.end(), perm);
        std::copy(t.group_base.begin(), t.group_base.end(), group_base);
        std::copy(t.members.begin(), t.members.end(), members);
        if (ranges) std::copy(t.ranges.begin(), t.ranges.end(), ranges);
        *ngroups = (uint32_t)(t.group_base.size() - 1);
    });
}

}  // namespace

gm_status gm_node_groups_build(uint32_t nv, const int32_t* cid, uint32_t nt, const uint32_t* tets, uint32_t np,
                               const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t permute, uint32_t* perm,
                               uint32_t* group_base, uint32_t* members, uint32_t* ranges, uint32_t* ngroups)
{
    return node_groups(nv, cid, nt, tets, np, pris, nh, hexs, permute, perm, group_base, members, ranges, ngroups,
                       false);
}

gm_status gm_node_groups_build_device(uint32_t nv, const int32_t* cid, uint32_t nt, const uint32_t* tets, uint32_t np,
                                      const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t permute,
                                      uint32_t* perm, uint32_t* group_base, uint32_t* members, uint32_t* ranges,
                                      uint32_t* ngroups)
{
    return node_groups(nv, cid, nt, tets, np, pris, nh, hexs, permute, perm, group_base, members, ranges, ngroups,
                       true);
}

gm_status gm_mesh_neighbourhoods(uint32_t nv, uint32_t nt, const uint32_t* tets, uint32_t np, const uint32_t* pris,
                                 uint32_t nh, const uint32_t* hexs, uint32_t* ve_off, uint32_t* ve, uint64_t* ve_len,
                                 uint32_t* vv_off, uint32_t* vv, uint64_t* vv_len)
{
    return guarded([&] {
        require(nv > 0 && ve_len && vv_len, "null argument");
        require((nt == 0 || tets) && (np == 0 || pris) && (nh == 0 || hexs), "null connectivity");
        check_conn(tets, (size_t)nt * 4, nv, "tet");
        check_conn(pris, (size_t)np * 6, nv, "prism");
        check_conn(hexs, (size_t)nh * 8, nv, "hex");
        HostMeshView in;
        in.nv = nv;
        in.nt = nt;
        in.np = np;
        in.nh = nh;
        in.tets = tets;
        in.pris = pris;
        in.hexs = hexs;
        std::vector<uint32_t> eo, e, vo, v;
        build_csr(in, eo, e, vo, v);
        const bool fill = ve || vv;
        if (fill)
        {
            require(ve && vv && ve_off && vv_off, "null output array");
            require(*ve_len >= e.size() && *vv_len >= v.size(), "output arrays shorter than the neighbourhoods");
            std::copy(eo.begin(), eo.end(), ve_off);
            std::copy(e.begin(), e.end(), ve);
            std::copy(vo.begin(), vo.end(), vv_off);
            std::copy(v.begin(), v.end(), vv);
        }
        *ve_len = e.size();
        *vv_len = v.size();
    });
}

gm_status gm_mesh_create(gm_mesh** out)
{
    return guarded([&] {
        require(out != nullptr, "null output");
        gm_mesh* m = new gm_mesh();
        try
        {
            GM_CUDA(cudaGetDevice(&m->device));
            GM_CUDA(cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device));
            m->ctr.reserve(1);
            GM_CUDA(cudaMemset(m->ctr.p, 0, sizeof(Counters)));
            m->bounds.reserve(2);
            GM_CUDA(cudaMemset(m->bounds.p, 0, 2 * sizeof(unsigned int)));
            set_crew(m, GM_SAMPLER_UNIFORM, GM_MEASURER_METRIC_FREE, GM_EVALUATOR_MEAN_RATIO, 1.0, 1.0);
        }
        catch (...)
        {
            delete m;
            throw;
        }
        *out = m;
    });
}

gm_status gm_mesh_destroy(gm_mesh* m)
{
    return guarded([&] {
        if (!m) return;
        cudaStreamSynchronize(m->stream);
        drop_job(m);
        m->job_counter.release();
        m->job_fresh.release();
        m->pos.release();
        m->tets.release();
        m->pris.release();
        m->hexs.release();
        m->ve_off.release();
        m->ve.release();
        m->vv_off.release();
        m->vv.release();
        m->cid.release();
        m->con.release();
        m->members.release();
        m->quality.release();
        m->parts.release();
        m->corners.release();
        m->saved.release();
        m->ctr.release();
        m->def_v.release();
        m->def_old.release();
        m->def_new.release();
        m->def_count.release();
        delete m;
    });
}

gm_status gm_mesh_set_stream(gm_mesh* m, void* stream)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        m->stream = (cudaStream_t)stream;
    });
}

gm_status gm_mesh_sync(gm_mesh* m)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        GM_CUDA(cudaStreamSynchronize(m->stream));
        report_bounds(m);
    });
}

gm_status gm_bounds_checked(int32_t* on)
{
    return guarded([&] {
        require(on != nullptr, "null output");
        *on = kBoundsChecked ? 1 : 0;
    });
}

gm_status gm_mesh_bounds_status(gm_mesh* m, uint32_t* what, uint32_t* index)
{
    return guarded([&] {
        require(m && what && index, "null argument");
        unsigned int w[2] = {0, 0};
        if (m->bounds.p)
        {
            GM_CUDA(cudaMemcpyAsync(w, m->bounds.p, sizeof(w), cudaMemcpyDeviceToHost, m->stream));
            GM_CUDA(cudaStreamSynchronize(m->stream));
            if (w[0]) GM_CUDA(cudaMemsetAsync(m->bounds.p, 0, sizeof(w), m->stream));
        }
        *what = w[0];
        *index = w[1];
    });
}

gm_status gm_mesh_upload(gm_mesh* m, uint32_t nv, const double* xyz, const int32_t* cid, uint32_t nt,
                         const uint32_t* tets, uint32_t np, const uint32_t* pris, uint32_t nh, const uint32_t* hexs)
{
    return guarded([&] {
        require(m && xyz && cid && nv > 0, "null argument");
        drop_job(m);
        require((nt == 0 || tets) && (np == 0 || pris) && (nh == 0 || hexs), "null connectivity");
        require((uint64_t)nt + np + nh <= kMaxElemId, "too many elements");
        check_conn(tets, (size_t)nt * 4, nv, "tet");
        check_conn(pris, (size_t)np * 6, nv, "prism");
        check_conn(hexs, (size_t)nh * 8, nv, "hex");
        HostMeshView in;
        in.nv = nv;
        in.nt = nt;
        in.np = np;
        in.nh = nh;
        in.cid = cid;
        in.tets = tets;
        in.pris = pris;
        in.hexs = hexs;
        std::vector<uint32_t> ve_off, ve, vv_off, vv;
        build_csr(in, ve_off, ve, vv_off, vv);
        upload_positions(m, nv, xyz);
        upload(m->cid, cid, nv, m->stream);
        m->nt = nt;
        m->np = np;
        m->nh = nh;
        upload(m->tets, reinterpret_cast<const uint4*>(tets), nt, m->stream);
        upload(m->pris, pris, (size_t)np * 6, m->stream);
        upload(m->hexs, reinterpret_cast<const uint4*>(hexs), (size_t)nh * 2, m->stream);
        upload_csr(m, ve_off, ve, vv_off, vv);
        GM_CUDA(cudaStreamSynchronize(m->stream));
        sampler_topology_changed(m);
    });
}

gm_status gm_mesh_upload_verts(gm_mesh* m, uint32_t nv, const double* xyz)
{
    return guarded([&] {
        require(m && xyz, "null argument");
        require(m->nv == 0 || m->nv == nv, "vertex count differs from the uploaded topology");
        upload_positions(m, nv, xyz);
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_upload_gpu_verts(gm_mesh* m, uint32_t nv, const void* gpu_verts)
{
    return guarded([&] {
        require(m && gpu_verts, "null argument");
        require(m->nv == 0 || m->nv == nv, "vertex count differs from the uploaded topology");
        upload(m->pos, reinterpret_cast<const float4*>(gpu_verts), nv, m->stream);
        m->nv = nv;
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_upload_gpu_verts_async(gm_mesh* m, uint32_t nv, const void* gpu_verts)
{
    return guarded([&] {
        require(m && gpu_verts, "null argument");
        require(m->nv == nv && m->pos.p && m->pos.cap >= nv, "vertex count differs from the uploaded vertices");
        GM_CUDA(cudaMemcpyAsync(m->pos.p, gpu_verts, (size_t)nv * sizeof(float4), cudaMemcpyHostToDevice, m->stream));
    });
}

#define GM_UPLOAD_ELEMS(NAME, K, FIELD, COUNT, VEC)                                                       \
    gm_status NAME(gm_mesh* m, uint32_t n, const uint32_t* words, uint32_t stride)                       \
    {                                                                                                    \
        return guarded([&] {                                                                             \
            require(m && (n == 0 || words), "null argument");                                            \
            drop_job(m);                                                                                 \
            std::vector<uint32_t> packed;                                                                \
            upload_conn<K>(m, n, words, stride, packed);                                                 \
            if (m->nv) check_conn(packed.data(), packed.size(), m->nv, #FIELD);                          \
            upload(m->FIELD, reinterpret_cast<const VEC*>(packed.data()), packed.size() * 4 / (sizeof(VEC)), \
                   m->stream);                                                                           \
            m->COUNT = n;                                                                                \
            GM_CUDA(cudaStreamSynchronize(m->stream));                                                   \
        });                                                                                              \
    }
GM_UPLOAD_ELEMS(gm_mesh_upload_tets, 4, tets, nt, uint4)
GM_UPLOAD_ELEMS(gm_mesh_upload_pris, 6, pris, np, uint32_t)
GM_UPLOAD_ELEMS(gm_mesh_upload_hexs, 8, hexs, nh, uint4)
#undef GM_UPLOAD_ELEMS

gm_status gm_mesh_upload_topo(gm_mesh* m, uint32_t nv, const int32_t* topo5, uint32_t n_nv, const uint32_t* neig_verts,
                              uint32_t n_ne, const int32_t* neig_elems3)
{
    return guarded([&] {
        require(m && topo5 && (n_nv == 0 || neig_verts) && (n_ne == 0 || neig_elems3), "null argument");
        drop_job(m);
        require(m->nv == 0 || m->nv == nv, "vertex count differs from the uploaded vertices");
        std::vector<int32_t> cid(nv);
        std::vector<uint32_t> ve_off((size_t)nv + 1, 0), vv_off((size_t)nv + 1, 0), ve, vv;
        ve.reserve(n_ne);
        vv.reserve(n_nv);
        for (uint32_t v = 0; v < nv; ++v)
        {
            const int32_t* t = topo5 + 5 * (size_t)v;
            cid[v] = t[0];
            uint32_t vb = (uint32_t)t[1], vc = (uint32_t)t[2], eb = (uint32_t)t[3], ec = (uint32_t)t[4];
            require((uint64_t)vb + vc <= n_nv && (uint64_t)eb + ec <= n_ne, "topology range out of bounds");
            for (uint32_t i = 0; i < vc; ++i)
            {
                require(neig_verts[vb + i] < nv, "neighbour vertex out of range");
                vv.push_back(neig_verts[vb + i]);
            }
            for (uint32_t i = 0; i < ec; ++i)
            {
                const int32_t* ne = neig_elems3 + 3 * (size_t)(eb + i);
                require(ne[1] == GM_TET || ne[1] == GM_PRI || ne[1] == GM_HEX, "unsupported neighbour element type");
                require(ne[2] >= 0 && ne[2] < 8 && (uint32_t)ne[0] <= kMaxElemId, "neighbour element out of range");
                ve.push_back(pack_elem_ref(ne[1], ne[2], (uint32_t)ne[0]));
            }
            vv_off[v + 1] = (uint32_t)vv.size();
            ve_off[v + 1] = (uint32_t)ve.size();
        }
        upload(m->cid, cid.data(), nv, m->stream);
        m->nv = nv;
        upload_csr(m, ve_off, ve, vv_off, vv);
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_upload_groups(gm_mesh* m, uint32_t n_members, const uint32_t* members, uint32_t ngroups,
                                const uint32_t* group_base)
{
    return guarded([&] {
        require(m && (n_members == 0 || members) && group_base, "null argument");
        drop_job(m);
        require(group_base[0] == 0 && group_base[ngroups] == n_members, "group bases must span the members");
        for (uint32_t g = 0; g < ngroups; ++g) require(group_base[g] <= group_base[g + 1], "group bases must ascend");
        for (uint32_t i = 0; i < n_members; ++i) require(members[i] < m->nv, "group member out of range");
        upload(m->members, members, n_members, m->stream);
        m->n_members = n_members;
        m->group_base.assign(group_base, group_base + ngroups + 1);
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_set_constraints(gm_mesh* m, uint32_t n, const int32_t* kind, const double* params)
{
    return guarded([&] {
        require(m && kind && params && n > 0, "null argument");
        drop_job(m);
        std::vector<Constraint> table(n);
        for (uint32_t i = 0; i < n; ++i)
        {
            Constraint& c = table[i];
            std::memset(&c, 0, sizeof(c));
            c.kind = kind[i];
            require(c.kind >= GM_CON_VOLUME && c.kind <= GM_CON_PIPE_CIRCLE, "unknown constraint kind");
            const double* p = params + 6 * (size_t)i;
            double a[3] = {p[0], p[1], p[2]}, b[3] = {p[3], p[4], p[5]}, u[3] = {0, 0, 0}, len = 0;
            if (c.kind == GM_CON_PLANE)
            {
                // PlaneConstraint normalizes its normal (FaceConstraint.cpp:172-176)
                double s = 1.0 / std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
                for (int k = 0; k < 3; ++k) b[k] *= s;
            }
            else if (c.kind == GM_CON_SEGMENT)
            {
                // SegmentConstraint keeps the unit direction and length (EdgeConstraint.cpp:176-181)
                double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                double l2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                double s = 1.0 / std::sqrt(l2);
                for (int k = 0; k < 3; ++k) u[k] = d[k] * s;
                len = std::sqrt(l2);
            }
            for (int k = 0; k < 3; ++k)
            {
                c.a[k] = (float)a[k];
                c.b[k] = (float)b[k];
                c.u[k] = (float)u[k];
                c.ad[k] = a[k];
                c.bd[k] = b[k];
                c.ud[k] = u[k];
            }
            c.len = (float)len;
            c.lend = len;
        }
        upload(m->con, table.data(), n, m->stream);
        m->ncon = (int)n;
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_set_crew(gm_mesh* m, int32_t sampler, int32_t measurer, int32_t evaluator, double scaling,
                           double aspect_ratio)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        drop_job(m);
        set_crew(m, sampler, measurer, evaluator, scaling, aspect_ratio);
    });
}

gm_status gm_mesh_build_local_background(gm_mesh* m)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        drop_job(m);
        // LocalSampler / KdTreeSampler / TextureSampler::updateAnalyticalMetric:
        // everything sampled again from the mesh as it is now
        auto bg = local_background_from_mesh(m, m->crew);
        m->local = bg;
        if (m->kd && !m->kd->given) m->kd.reset();
        if (m->tex && !m->tex->given) m->tex.reset();
        Crew c = m->crew;
        prepare_sampler(m, c);
        m->crew = c;
    });
}

namespace {
// a part handed over by the caller: installed, and the field re-assembled
// while a background-mesh sampler is installed
void refresh_crew(gm_mesh* m)
{
    if (m->crew.sampler >= GM_SAMPLER_LOCAL) m->crew.local = assemble_field(m);
}
}  // namespace

gm_status gm_mesh_set_local_background(gm_mesh* m, uint32_t ntets, const uint32_t* tets8, uint32_t nverts,
                                       const double* xyz, const double* metrics6)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        drop_job(m);
        m->local = local_background_given(m, ntets, tets8, nverts, xyz, metrics6);
        refresh_crew(m);
    });
}

gm_status gm_mesh_set_kd_nodes(gm_mesh* m, uint32_t n, const int32_t* children2, const double* separators4,
                               const double* metrics6)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        drop_job(m);
        m->kd = kdtree_given(m, n, children2, separators4, metrics6);
        refresh_crew(m);
    });
}

gm_status gm_mesh_set_texture(gm_mesh* m, const int32_t* dims3, const double* min3, const double* extents3,
                              const double* metrics6)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        drop_job(m);
        m->tex = texture_given(m, dims3, min3, extents3, metrics6);
        refresh_crew(m);
    });
}

gm_status gm_mesh_set_discretization_depth(gm_mesh* m, int32_t depth)
{
    return guarded([&] {
        require(m != nullptr, "null mesh");
        require(depth < 4096, "discretization depth out of range");
        const int old = m->depth;
        if ((depth < 0 ? -1 : depth) == old) return;
        drop_job(m);
        m->depth = depth < 0 ? -1 : depth;
        if (m->crew.sampler == GM_SAMPLER_KDTREE || m->crew.sampler == GM_SAMPLER_TEXTURE)
        {
            Crew c = m->crew;
            try
            {
                prepare_sampler(m, c);
            }
            catch (...)
            {
                m->depth = old;
                throw;
            }
            m->crew = c;
        }
    });
}

gm_status gm_mesh_clone(gm_mesh* dst, const gm_mesh* src)
{
    return guarded([&] {
        require(dst && src && dst != src, "invalid argument");
        require(src->nv > 0 && src->cid.p, "source mesh has no topology");
        drop_job(dst);
        cudaStream_t s = dst->stream;
        GM_CUDA(cudaStreamSynchronize(src->stream));
        auto copy = [&](auto& d, const auto& from, size_t n) {
            d.reserve(n);
            if (n) GM_CUDA(cudaMemcpyAsync(d.p, from.p, n * sizeof(*from.p), cudaMemcpyDeviceToDevice, s));
        };
        copy(dst->pos, src->pos, src->nv);
        copy(dst->tets, src->tets, src->nt);
        copy(dst->pris, src->pris, (size_t)src->np * 6);
        copy(dst->hexs, src->hexs, (size_t)src->nh * 2);
        copy(dst->ve_off, src->ve_off, (size_t)src->nv + 1);
        copy(dst->vv_off, src->vv_off, (size_t)src->nv + 1);
        std::vector<uint32_t> last(2);
        GM_CUDA(cudaMemcpy(&last[0], src->ve_off.p + src->nv, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        GM_CUDA(cudaMemcpy(&last[1], src->vv_off.p + src->nv, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        copy(dst->ve, src->ve, last[0]);
        copy(dst->vv, src->vv, last[1]);
        copy(dst->cid, src->cid, src->nv);
        copy(dst->con, src->con, (size_t)src->ncon);
        copy(dst->members, src->members, src->n_members);
        dst->nv = src->nv;
        dst->nt = src->nt;
        dst->np = src->np;
        dst->nh = src->nh;
        dst->ncon = src->ncon;
        dst->n_ve = last[0];
        dst->n_vv = last[1];
        dst->n_members = src->n_members;
        dst->group_base = src->group_base;
        dst->crew = src->crew;
        dst->local = src->local;  // shared parts; dst assembles its own field
        dst->kd = src->kd;
        dst->tex = src->tex;
        dst->depth = src->depth;
        if (dst->crew.sampler >= GM_SAMPLER_LOCAL) dst->crew.local = assemble_field(dst);
        dst->ks = src->ks;
        dst->maxe = src->maxe;
        dst->max_incident = src->max_incident;
        dst->warps_per_block = src->warps_per_block;
        GM_CUDA(cudaStreamSynchronize(s));
    });
}

gm_status gm_mesh_device_bytes(const gm_mesh* m, uint64_t* bytes)
{
    return guarded([&] {
        require(m && bytes, "null argument");
        uint64_t b = 0;
        b += m->pos.cap * sizeof(float4) + m->tets.cap * sizeof(uint4) + m->pris.cap * 4 + m->hexs.cap * sizeof(uint4);
        b += (m->ve_off.cap + m->ve.cap + m->vv_off.cap + m->vv.cap + m->members.cap) * 4 + m->cid.cap * 4;
        b += m->con.cap * sizeof(Constraint) + m->parts.cap * sizeof(EvalPartial) + m->corners.cap * sizeof(float4);
        b += m->saved.cap * sizeof(float4) + m->def_v.cap * 4 + (m->def_old.cap + m->def_new.cap) * sizeof(float4);
        b += m->quality.cap * sizeof(Quality);
        b += sampler_bytes(m);
        *bytes = b;
    });
}

gm_status gm_mesh_save_positions(gm_mesh* m)
{
    return guarded([&] {
        require_mesh(m);
        m->saved.reserve(m->nv);
        GM_CUDA(cudaMemcpyAsync(m->saved.p, m->pos.p, m->nv * sizeof(float4), cudaMemcpyDeviceToDevice, m->stream));
    });
}

gm_status gm_mesh_restore_positions(gm_mesh* m)
{
    return guarded([&] {
        require_mesh(m);
        require(m->saved.p != nullptr && m->saved.cap >= m->nv, "no saved positions");
        GM_CUDA(cudaMemcpyAsync(m->pos.p, m->saved.p, m->nv * sizeof(float4), cudaMemcpyDeviceToDevice, m->stream));
    });
}

gm_status gm_mesh_fetch_verts(gm_mesh* m, uint32_t nv, double* xyz)
{
    return guarded([&] {
        require(m && xyz, "null argument");
        require(nv == m->nv, "vertex count mismatch");
        m->staging.resize(nv);
        GM_CUDA(cudaMemcpyAsync(m->staging.data(), m->pos.p, nv * sizeof(float4), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
        for (uint32_t v = 0; v < nv; ++v)
        {
            xyz[3 * (size_t)v] = m->staging[v].x;
            xyz[3 * (size_t)v + 1] = m->staging[v].y;
            xyz[3 * (size_t)v + 2] = m->staging[v].z;
        }
    });
}

gm_status gm_mesh_fetch_gpu_verts(gm_mesh* m, uint32_t nv, void* gpu_verts)
{
    return guarded([&] {
        require(m && gpu_verts, "null argument");
        require(nv == m->nv, "vertex count mismatch");
        GM_CUDA(cudaMemcpyAsync(gpu_verts, m->pos.p, nv * sizeof(float4), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
        report_bounds(m);
    });
}

gm_status gm_mesh_fetch_gpu_verts_range(gm_mesh* m, uint32_t first, uint32_t count, void* gpu_verts)
{
    return guarded([&] {
        require(m && (count == 0 || gpu_verts), "null argument");
        require((uint64_t)first + count <= m->nv, "vertex range out of bounds");
        if (!count) return;
        GM_CUDA(cudaMemcpyAsync(gpu_verts, m->pos.p + first, (size_t)count * sizeof(float4), cudaMemcpyDeviceToHost,
                                m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_mesh_upload_gpu_verts_range(gm_mesh* m, uint32_t first, uint32_t count, const void* gpu_verts)
{
    return guarded([&] {
        require(m && (count == 0 || gpu_verts), "null argument");
        require((uint64_t)first + count <= m->nv, "vertex range out of bounds");
        if (!count) return;
        GM_CUDA(cudaMemcpyAsync(m->pos.p + first, gpu_verts, (size_t)count * sizeof(float4), cudaMemcpyHostToDevice,
                                m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_evaluate_async(gm_mesh* m, uint32_t slot)
{
    return guarded([&] {
        require_mesh(m);
        require(slot < 65536, "quality slot out of range");
        if (slot >= m->n_quality_slots)
        {
            if (m->job_exec) drop_job(m);  // the job graph captured the old slots
            ensure_quality_slots(m, slot + 1);
        }
        enqueue_evaluate(m, m->quality.p + slot);
    });
}

gm_status gm_quality_read(gm_mesh* m, uint32_t slot, gm_quality* out)
{
    return guarded([&] {
        require(m && out, "null argument");
        require(slot < m->n_quality_slots, "quality slot never evaluated");
        static_assert(sizeof(Quality) == sizeof(gm_quality), "quality layout");
        GM_CUDA(cudaMemcpyAsync(out, m->quality.p + slot, sizeof(Quality), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
        report_bounds(m);
    });
}

gm_status gm_evaluate(gm_mesh* m, gm_quality* out)
{
    gm_status s = gm_evaluate_async(m, 0);
    if (s != GM_OK) return s;
    return gm_quality_read(m, 0, out);
}

gm_status gm_smooth_group(gm_mesh* m, int32_t smoother, const double* params, uint32_t base, uint32_t count)
{
    return guarded([&] {
        require_mesh(m);
        require((uint64_t)base + count <= m->n_members, "group slice outside the uploaded members");
        require(smoother != GM_SMOOTH_GETME, "GETMe relocates through gm_getme_elements / gm_getme_update_group");
        SmoothParams sp = parse_params(smoother, params);
        ensure_deferred(m);
        uint32_t slot = (uint32_t)m->group_base.size();
        GM_CUDA(cudaMemsetAsync(m->def_count.p + slot, 0, sizeof(uint32_t), m->stream));
        relocate_group(m, smoother, sp, base, count, slot);
    });
}

gm_status gm_getme_elements(gm_mesh* m, const double* params)
{
    return guarded([&] {
        require_mesh(m);
        SmoothParams sp = parse_params(GM_SMOOTH_GETME, params);
        m->corners.reserve(4 * (size_t)m->nt + 6 * (size_t)m->np + 8 * (size_t)m->nh);
        GM_CUDA(launch_getme_elements(m->element_variant(), m->view(), m->crew, sp.lambda, m->corners.p, m->sm_count,
                                      m->stream));
    });
}

gm_status gm_getme_update_group(gm_mesh* m, const double* params, uint32_t base, uint32_t count)
{
    return guarded([&] {
        require_mesh(m);
        require(m->corners.p != nullptr, "gm_getme_elements must run before the vertex update");
        require((uint64_t)base + count <= m->n_members, "group slice outside the uploaded members");
        SmoothParams sp = parse_params(GM_SMOOTH_GETME, params);
        ensure_deferred(m);
        uint32_t slot = (uint32_t)m->group_base.size();
        GM_CUDA(cudaMemsetAsync(m->def_count.p + slot, 0, sizeof(uint32_t), m->stream));
        relocate_group(m, GM_SMOOTH_GETME, sp, base, count, slot);
    });
}

gm_status gm_smooth_pass(gm_mesh* m, int32_t smoother, const double* params)
{
    return guarded([&] {
        require_mesh(m);
        require_groups(m);
        SmoothParams sp = parse_params(smoother, params);
        if (smoother == GM_SMOOTH_GETME && m->job_exec &&
            m->corners.cap < 4 * (size_t)m->nt + 6 * (size_t)m->np + 8 * (size_t)m->nh)
            drop_job(m);  // the corner buffer is about to be allocated
        enqueue_pass(m, smoother, sp);
    });
}

gm_status gm_mesh_counters(gm_mesh* m, uint64_t* out5, int32_t reset)
{
    return guarded([&] {
        require(m && out5, "null argument");
        Counters c;
        GM_CUDA(cudaMemcpyAsync(&c, m->ctr.p, sizeof(c), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
        out5[0] = c.patch_evals;
        out5[1] = c.elem_evals[0];
        out5[2] = c.elem_evals[2];
        out5[3] = c.elem_evals[3];
        out5[4] = c.fp64_vertices;
        if (reset) GM_CUDA(cudaMemsetAsync(m->ctr.p, 0, sizeof(Counters), m->stream));
    });
}

// ---- device-resident jobs ----
// The graph: a conditional WHILE node whose body is one relocation pass, one
// evaluation into job_fresh, and job_rule_kernel, which files the evaluation
// in the next quality slot and sets the loop condition.  gm_job_launch puts
// the counter reset and the first evaluation (slot 0) in front of it.
gm_status gm_job_prepare(gm_mesh* m, int32_t smoother, const double* params, uint32_t max_passes, double min_gain)
{
    return guarded([&] {
        require_mesh(m);
        require_groups(m);
        require(max_passes >= 1 && max_passes < 65535, "max_passes out of range");
        drop_job(m);
        const SmoothParams sp = parse_params(smoother, params);
        // allocate everything the graph refers to before capturing it, and run
        // one evaluation so that the launch configuration is cached
        ensure_deferred(m);
        if (smoother == GM_SMOOTH_GETME)
            m->corners.reserve(4 * (size_t)m->nt + 6 * (size_t)m->np + 8 * (size_t)m->nh);
        ensure_quality_slots(m, max_passes + 1);
        m->job_counter.reserve(1);
        m->job_fresh.reserve(1);
        enqueue_evaluate(m, m->job_fresh.p);
        GM_CUDA(cudaStreamSynchronize(m->stream));

        cudaGraph_t g = nullptr;
        GM_CUDA(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle loop;
        cudaError_t e = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = loop;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(m->stream, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
        {
            cudaGraphDestroy(g);
            throw ApiError(GM_ERR_CUDA, std::string("job graph: ") + cudaGetErrorString(e));
        }
        CaptureTally body_kernels;
        try
        {
            enqueue_pass(m, smoother, sp);
            enqueue_evaluate(m, m->job_fresh.p);
            job_rule_kernel<<<1, 32, 0, m->stream>>>(m->quality.p, m->job_fresh.p, m->job_counter.p, min_gain,
                                                     (int)max_passes, loop);
            note_launch();
            GM_CUDA(cudaGetLastError());
        }
        catch (...)
        {
            cudaGraph_t body = nullptr;
            cudaStreamEndCapture(m->stream, &body);
            cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(m->stream, &body);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&m->job_exec, g, 0);
        if (e != cudaSuccess)
        {
            cudaGraphDestroy(g);
            m->job_exec = nullptr;
            throw ApiError(GM_ERR_CUDA, std::string("job graph: ") + cudaGetErrorString(e));
        }
        m->job_graph = g;
        m->job_max_passes = max_passes;
        m->job_body_kernels = body_kernels.kernels;
    });
}

gm_status gm_job_launch(gm_mesh* m)
{
    NvtxRange range("gm job launch");
    return guarded([&] {
        require(m && m->job_exec, "no job prepared on this mesh");
        GM_CUDA(cudaMemsetAsync(m->job_counter.p, 0, sizeof(int), m->stream));
        enqueue_evaluate(m, m->quality.p);
        GM_CUDA(cudaGraphLaunch(m->job_exec, m->stream));
    });
}

gm_status gm_job_query(gm_mesh* m, int32_t* done)
{
    return guarded([&] {
        require(m && done, "null argument");
        cudaError_t e = cudaStreamQuery(m->stream);
        if (e == cudaErrorNotReady)
        {
            *done = 0;
            return;
        }
        GM_CUDA(e);
        *done = 1;
    });
}

gm_status gm_job_result(gm_mesh* m, uint32_t* passes, gm_quality* first, gm_quality* last)
{
    return guarded([&] {
        require(m && m->job_exec && passes, "no job prepared on this mesh");
        int c = 0;
        GM_CUDA(cudaMemcpyAsync(&c, m->job_counter.p, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
        require(c >= 0 && (uint32_t)c <= m->job_max_passes, "job counter out of range");
        *passes = (uint32_t)c;
        add_launches((unsigned long long)c * m->job_body_kernels);  // the loop body ran c times
        if (first)
            GM_CUDA(cudaMemcpyAsync(first, m->quality.p, sizeof(Quality), cudaMemcpyDeviceToHost, m->stream));
        if (last)
            GM_CUDA(cudaMemcpyAsync(last, m->quality.p + c, sizeof(Quality), cudaMemcpyDeviceToHost, m->stream));
        GM_CUDA(cudaStreamSynchronize(m->stream));
    });
}

gm_status gm_launch_count(uint64_t* count)
{
    return guarded([&] {
        require(count != nullptr, "null output");
        *count = g_launches.load(std::memory_order_relaxed);
    });
}

gm_status gm_probe_fp32_tflops(double* tflops)
{
    return guarded([&] {
        require(tflops != nullptr, "null output");
        int dev = 0, sms = 0;
        GM_CUDA(cudaGetDevice(&dev));
        GM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        float* sink = nullptr;
        GM_CUDA(cudaMalloc(&sink, sizeof(float) * 1024));
        cudaEvent_t a, b;
        GM_CUDA(cudaEventCreate(&a));
        GM_CUDA(cudaEventCreate(&b));
        const int iters = 1 << 14, blocks = sms * 8, threads = 256;
        GM_CUDA(launch_ffma_probe(blocks, threads, iters, sink, 0));  // warm-up
        GM_CUDA(cudaEventRecord(a, 0));
        GM_CUDA(launch_ffma_probe(blocks, threads, iters, sink, 0));
        GM_CUDA(cudaEventRecord(b, 0));
        GM_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        GM_CUDA(cudaEventElapsedTime(&ms, a, b));
        // 8 independent FFMA chains per thread, 2 flops each
        double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
        *tflops = flops / (ms * 1e-3) / 1e12;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaFree(sink);
    });
}

}  // extern "C"
