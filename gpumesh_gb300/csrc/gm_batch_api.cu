// C ABI of the batched path: gm_batch over many gm_mesh objects, one
// persistent relocation launch per pass, per-mesh evaluation in one launch,
// CUDA-graph capture of a pass, and the launch-shape autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "gm_batch.h"
#include "gm_host.h"

struct gm_batch
{
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<gm_mesh*> meshes;
    int variant = 0, maxk = 4, maxe = 32;
    uint32_t nseg = 0, total = 0;
    DBuf<BatchMesh> table;
    DBuf<Segment> segs;
    DBuf<uint32_t> seg_start;
    DBuf<unsigned int> done;
    DBuf<BatchCtl> ctl;
    DBuf<Counters> ctr;
    DBuf<unsigned long long> finish;
    // evaluation
    DBuf<EvalBlock> eval_blocks;
    DBuf<uint32_t> mesh_block;
    DBuf<EvalPartial> eval_parts;
    uint32_t n_eval_blocks = 0;
    DBuf<Quality> quality;
    uint32_t n_slots = 0;
    // launch shape (0: as many CTAs per SM as fit)
    int wpb = 4, cps = 0;
    unsigned long long spin_limit = 20000000ull;
    std::vector<Segment> host_segs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    unsigned long long graph_kernels = 0;  // kernels of one replay of the captured pass

    BatchArgs args() const
    {
        BatchArgs a;
        a.meshes = table.p;
        a.segs = segs.p;
        a.seg_start = seg_start.p;
        a.nseg = nseg;
        a.total = total;
        a.done = done.p;
        a.ctl = ctl.p;
        a.ctr = ctr.p;
        a.finish = finish.p;
        a.maxe = maxe;
        a.spin_limit = spin_limit;
        return a;
    }
};

namespace {

void build_tables(gm_batch* b, bool with_corners)
{
    const uint32_t n = (uint32_t)b->meshes.size();
    std::vector<BatchMesh> table(n);
    uint32_t ngmax = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        gm_mesh* m = b->meshes[i];
        if (with_corners) m->corners.reserve(4 * (size_t)m->nt + 6 * (size_t)m->np + 8 * (size_t)m->nh);
        table[i].view = m->view();
        table[i].crew = m->crew;
        table[i].members = m->members.p;
        table[i].corners = m->corners.p;
        table[i].nmembers = m->n_members;
        ngmax = std::max<uint32_t>(ngmax, (uint32_t)m->group_base.size() - 1);
    }
    upload(b->table, table.data(), n, b->stream);
    // segments ordered by colour, then mesh
    b->host_segs.clear();
    std::vector<uint32_t> start(1, 0);
    for (uint32_t g = 0; g < ngmax; ++g)
        for (uint32_t i = 0; i < n; ++i)
        {
            const std::vector<uint32_t>& gb = b->meshes[i]->group_base;
            if (g + 1 >= gb.size()) continue;
            uint32_t cnt = gb[g + 1] - gb[g];
            if (!cnt) continue;
            b->host_segs.push_back(Segment{i, gb[g], cnt, gb[g]});
            start.push_back(start.back() + cnt);
        }
    b->nseg = (uint32_t)b->host_segs.size();
    b->total = start.back();
    upload(b->segs, b->host_segs.data(), b->host_segs.size(), b->stream);
    upload(b->seg_start, start.data(), start.size(), b->stream);
    b->done.reserve(n);
    b->finish.reserve(n);
    b->ctl.reserve(1);
    // evaluation blocks: ~2048 elements per block
    std::vector<EvalBlock> blocks;
    std::vector<uint32_t> mb(1, 0);
    for (uint32_t i = 0; i < n; ++i)
    {
        gm_mesh* m = b->meshes[i];
        uint32_t E = m->nt + m->np + m->nh;
        for (uint32_t s = 0; s < E; s += 2048) blocks.push_back(EvalBlock{i, s, std::min(E, s + 2048), 0});
        mb.push_back((uint32_t)blocks.size());
    }
    b->n_eval_blocks = (uint32_t)blocks.size();
    upload(b->eval_blocks, blocks.data(), blocks.size(), b->stream);
    upload(b->mesh_block, mb.data(), mb.size(), b->stream);
    b->eval_parts.reserve(std::max<size_t>(1, blocks.size()));
    GM_CUDA(cudaStreamSynchronize(b->stream));
}

void drop_graph(gm_batch* b)
{
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph_exec = nullptr;
    b->graph = nullptr;
}

// the batched kernels relocate with the four smoothers of the reference's
// CUDA path; the Laplace smoothers run on the plain path only
void require_batch_smoother(int smoother)
{
    if (smoother == GM_SMOOTH_SPRING_LAPLACE || smoother == GM_SMOOTH_QUALITY_LAPLACE)
        throw ApiError(GM_ERR_UNSUPPORTED, "the batched path relocates with Nelder-Mead, gradient descent, spawn "
                                           "search or GETMe; use gm_smooth_pass for the Laplace smoothers");
}

void enqueue_pass(gm_batch* b, int smoother, const SmoothParams& sp)
{
    NvtxRange range("gm batch pass");
    if (smoother == GM_SMOOTH_GETME)
        for (gm_mesh* m : b->meshes)
            GM_CUDA(launch_getme_elements(m->element_variant(), m->view(), m->crew, sp.lambda, m->corners.p,
                                          b->sm_count, b->stream));
    GM_CUDA(cudaMemsetAsync(b->done.p, 0, b->meshes.size() * sizeof(unsigned int), b->stream));
    GM_CUDA(cudaMemsetAsync(b->ctl.p, 0, sizeof(BatchCtl), b->stream));
    GM_CUDA(cudaMemsetAsync(b->finish.p, 0, b->meshes.size() * sizeof(unsigned long long), b->stream));
    GM_CUDA(launch_batch_relocate(smoother, b->args(), sp, b->variant, b->maxk, b->wpb, b->cps, b->sm_count,
                                  b->stream));
}

void ensure_slots(gm_batch* b, uint32_t slot)
{
    if (slot < b->n_slots) return;
    uint32_t n = std::max<uint32_t>(slot + 1, 2 * b->n_slots);
    size_t per = b->meshes.size();
    Quality* fresh = nullptr;
    GM_CUDA(cudaMalloc(&fresh, (size_t)n * per * sizeof(Quality)));
    if (b->quality.p && b->n_slots)
        GM_CUDA(cudaMemcpyAsync(fresh, b->quality.p, (size_t)b->n_slots * per * sizeof(Quality),
                                cudaMemcpyDeviceToDevice, b->stream));
    GM_CUDA(cudaStreamSynchronize(b->stream));
    b->quality.release();
    b->quality.p = fresh;
    b->quality.cap = (size_t)n * per;
    b->n_slots = n;
}

void enqueue_evaluate(gm_batch* b, uint32_t slot)
{
    NvtxRange range("gm batch evaluate");
    GM_CUDA(launch_batch_evaluate(b->table.p, (uint32_t)b->meshes.size(), b->eval_blocks.p, b->n_eval_blocks,
                                  b->mesh_block.p, b->eval_parts.p, b->quality.p + (size_t)slot * b->meshes.size(),
                                  b->variant, b->maxk, b->stream));
}

}  // namespace

extern "C" {

gm_status gm_batch_create(gm_batch** out, gm_mesh* const* meshes, uint32_t n)
{
    return guarded([&] {
        require(out && meshes && n > 0, "null argument");
        gm_batch* b = new gm_batch();
        try
        {
            GM_CUDA(cudaGetDevice(&b->device));
            GM_CUDA(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device));
            GM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
            b->own_stream = true;
            b->meshes.assign(meshes, meshes + n);
            for (uint32_t i = 0; i < n; ++i)
            {
                gm_mesh* m = meshes[i];
                require(m && m->nv && !m->group_base.empty(), "mesh " + std::to_string(i) + " has no groups");
                require(m->device == b->device, "all meshes of a batch must live on the current device");
                int v = m->variant();
                require(v == kVarMRFree || v == kVarMCDiag || v == kVarMC || v == kVarMRWise, "unknown kernel variant");
                if (i == 0) b->variant = v;
                require(v == b->variant, "all meshes of a batch must use the same evaluator and measurer");
                b->maxk = std::max(b->maxk, m->maxk());
                b->maxe = std::max(b->maxe, m->maxe);
                GM_CUDA(cudaStreamSynchronize(m->stream));
            }
            b->ctr.reserve(1);
            GM_CUDA(cudaMemset(b->ctr.p, 0, sizeof(Counters)));
            build_tables(b, false);
        }
        catch (...)
        {
            if (b->stream) cudaStreamDestroy(b->stream);
            delete b;
            throw;
        }
        *out = b;
    });
}

gm_status gm_batch_destroy(gm_batch* b)
{
    return guarded([&] {
        if (!b) return;
        cudaStreamSynchronize(b->stream);
        drop_graph(b);
        b->table.release();
        b->segs.release();
        b->seg_start.release();
        b->done.release();
        b->ctl.release();
        b->ctr.release();
        b->finish.release();
        b->eval_blocks.release();
        b->mesh_block.release();
        b->eval_parts.release();
        b->quality.release();
        if (b->own_stream) cudaStreamDestroy(b->stream);
        delete b;
    });
}

gm_status gm_batch_stream(gm_batch* b, void** stream)
{
    return guarded([&] {
        require(b && stream, "null argument");
        *stream = (void*)b->stream;
    });
}

gm_status gm_batch_set_config(gm_batch* b, int32_t warps_per_block, int32_t ctas_per_sm)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        require(warps_per_block == 1 || warps_per_block == 2 || warps_per_block == 4 || warps_per_block == 8,
                "warps per block must be 1, 2, 4 or 8");
        require(ctas_per_sm >= 0 && ctas_per_sm <= 64, "CTAs per SM out of range");
        b->wpb = warps_per_block;
        b->cps = ctas_per_sm;
        drop_graph(b);
    });
}

gm_status gm_batch_set_spin_limit(gm_batch* b, uint64_t polls)
{
    return guarded([&] {
        require(b && polls > 0, "invalid argument");
        b->spin_limit = polls;
        drop_graph(b);
    });
}

gm_status gm_batch_inject_stall(gm_batch* b, uint32_t mesh)
{
    return guarded([&] {
        require(b && mesh < b->meshes.size(), "invalid argument");
        bool any = false;
        for (Segment& s : b->host_segs)
            if (s.mesh == mesh && s.need > 0)
            {
                s.need += 1u << 30;  // a count its mesh never reaches
                any = true;
            }
        require(any, "mesh has a single colour: nothing waits");
        upload(b->segs, b->host_segs.data(), b->host_segs.size(), b->stream);
        GM_CUDA(cudaStreamSynchronize(b->stream));
        drop_graph(b);
    });
}

gm_status gm_batch_smooth_pass(gm_batch* b, int32_t smoother, const double* params)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        SmoothParams sp = parse_smooth_params(smoother, params);
        require_batch_smoother(smoother);
        if (smoother == GM_SMOOTH_GETME) build_tables(b, true);
        enqueue_pass(b, smoother, sp);
    });
}

gm_status gm_batch_evaluate(gm_batch* b, uint32_t slot)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        require(slot < 65536, "slot out of range");
        ensure_slots(b, slot);
        enqueue_evaluate(b, slot);
    });
}

gm_status gm_batch_read_quality(gm_batch* b, uint32_t slot, gm_quality* out)
{
    return guarded([&] {
        require(b && out, "null argument");
        require(slot < b->n_slots, "slot never evaluated");
        GM_CUDA(cudaMemcpyAsync(out, b->quality.p + (size_t)slot * b->meshes.size(),
                                b->meshes.size() * sizeof(Quality), cudaMemcpyDeviceToHost, b->stream));
        GM_CUDA(cudaStreamSynchronize(b->stream));
    });
}

gm_status gm_batch_sync(gm_batch* b)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        GM_CUDA(cudaStreamSynchronize(b->stream));
    });
}

gm_status gm_batch_status(gm_batch* b)
{
    gm_status st = guarded([&] { require(b != nullptr, "null batch"); });
    if (st != GM_OK) return st;
    BatchCtl c{};
    st = guarded([&] {
        GM_CUDA(cudaMemcpyAsync(&c, b->ctl.p, sizeof(c), cudaMemcpyDeviceToHost, b->stream));
        GM_CUDA(cudaStreamSynchronize(b->stream));
    });
    if (st != GM_OK) return st;
    if (c.error)
    {
        set_error("a batched pass gave up waiting for a mesh's earlier colours (dependency wait limit reached)");
        return GM_ERR_TIMEOUT;
    }
    return GM_OK;
}

gm_status gm_batch_capture_pass(gm_batch* b, int32_t smoother, const double* params, int32_t eval_slot)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        SmoothParams sp = parse_smooth_params(smoother, params);
        require_batch_smoother(smoother);
        if (smoother == GM_SMOOTH_GETME) build_tables(b, true);
        if (eval_slot >= 0) ensure_slots(b, (uint32_t)eval_slot);
        drop_graph(b);
        GM_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        CaptureTally graph_kernels;
        try
        {
            enqueue_pass(b, smoother, sp);
            if (eval_slot >= 0) enqueue_evaluate(b, (uint32_t)eval_slot);
        }
        catch (...)
        {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(b->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        GM_CUDA(cudaStreamEndCapture(b->stream, &b->graph));
        GM_CUDA(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
        b->graph_kernels = graph_kernels.kernels;
    });
}

gm_status gm_batch_replay(gm_batch* b)
{
    NvtxRange range("gm batch replay");
    return guarded([&] {
        require(b && b->graph_exec, "no captured pass");
        GM_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
        add_launches(b->graph_kernels);
    });
}

gm_status gm_batch_counters(gm_batch* b, uint64_t* out5, int32_t reset)
{
    return guarded([&] {
        require(b && out5, "null argument");
        Counters c;
        GM_CUDA(cudaMemcpyAsync(&c, b->ctr.p, sizeof(c), cudaMemcpyDeviceToHost, b->stream));
        GM_CUDA(cudaStreamSynchronize(b->stream));
        out5[0] = c.patch_evals;
        out5[1] = c.elem_evals[0];
        out5[2] = c.elem_evals[2];
        out5[3] = c.elem_evals[3];
        out5[4] = c.fp64_vertices;
        if (reset) GM_CUDA(cudaMemsetAsync(b->ctr.p, 0, sizeof(Counters), b->stream));
    });
}

gm_status gm_batch_latencies(gm_batch* b, double* out_ms)
{
    return guarded([&] {
        require(b && out_ms, "null argument");
        size_t n = b->meshes.size();
        std::vector<unsigned long long> fin(n);
        BatchCtl c{};
        GM_CUDA(cudaMemcpyAsync(fin.data(), b->finish.p, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                b->stream));
        GM_CUDA(cudaMemcpyAsync(&c, b->ctl.p, sizeof(c), cudaMemcpyDeviceToHost, b->stream));
        GM_CUDA(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < n; ++i) out_ms[i] = fin[i] ? (double)(fin[i] - c.t0) * 1e-6 : -1.0;
    });
}

gm_status gm_batch_info(gm_batch* b, uint32_t* out4)
{
    return guarded([&] {
        require(b && out4, "null argument");
        out4[0] = (uint32_t)b->meshes.size();
        out4[1] = b->total;
        out4[2] = b->nseg;
        out4[3] = b->n_eval_blocks;
    });
}

// Autotuner: time one pass for every launch shape (warps per block x CTAs per
// SM) from the same saved positions and keep the fastest.
gm_status gm_batch_tune(gm_batch* b, int32_t smoother, const double* params, int32_t* best_wpb, int32_t* best_cps,
                        double* best_ms)
{
    return guarded([&] {
        require(b != nullptr, "null batch");
        SmoothParams sp = parse_smooth_params(smoother, params);
        require_batch_smoother(smoother);
        if (smoother == GM_SMOOTH_GETME) build_tables(b, true);
        for (gm_mesh* m : b->meshes)
        {
            m->saved.reserve(m->nv);
            GM_CUDA(cudaMemcpyAsync(m->saved.p, m->pos.p, m->nv * sizeof(float4), cudaMemcpyDeviceToDevice, b->stream));
        }
        cudaEvent_t e0, e1;
        GM_CUDA(cudaEventCreate(&e0));
        GM_CUDA(cudaEventCreate(&e1));
        const int shapes[][2] = {{2, 0}, {4, 0}, {8, 0}, {4, 2}, {8, 1}, {2, 4}, {1, 0}};
        float best = 1e30f;
        int bw = b->wpb, bc = b->cps;
        for (const auto& sh : shapes)
        {
            b->wpb = sh[0];
            b->cps = sh[1];
            for (gm_mesh* m : b->meshes)
                GM_CUDA(cudaMemcpyAsync(m->pos.p, m->saved.p, m->nv * sizeof(float4), cudaMemcpyDeviceToDevice,
                                        b->stream));
            GM_CUDA(cudaEventRecord(e0, b->stream));
            enqueue_pass(b, smoother, sp);
            GM_CUDA(cudaEventRecord(e1, b->stream));
            GM_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            GM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best)
            {
                best = ms;
                bw = sh[0];
                bc = sh[1];
            }
        }
        for (gm_mesh* m : b->meshes)
            GM_CUDA(cudaMemcpyAsync(m->pos.p, m->saved.p, m->nv * sizeof(float4), cudaMemcpyDeviceToDevice, b->stream));
        GM_CUDA(cudaStreamSynchronize(b->stream));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->wpb = bw;
        b->cps = bc;
        drop_graph(b);
        if (best_wpb) *best_wpb = bw;
        if (best_cps) *best_cps = bc;
        if (best_ms) *best_ms = best;
    });
}

}  // extern "C"
