// Batched smoothing kernels (included by gm_batch.cu, which instantiates
// the metric-free mean-ratio and diagonal-metric variants, and by
// gm_batch_general_mc.cu and gm_batch_general_mrwise.cu, the general-metric
// ones): many meshes of uneven size relocated by one persistent
// kernel launch, and evaluated per mesh by one launch.
//
// Work queue.  The vertices to relocate are enumerated as segments
// (colour g, mesh m) ordered by colour first, then mesh; a segment of colour
// g of mesh m may start once every vertex of mesh m in colours < g is done.
// Warps claim small chunks of consecutive items with one atomic and process
// them in order.  Everything a claimed item waits for sits earlier in the
// queue and was therefore already claimed by a running warp, so the oldest
// unfinished item can always proceed: with every warp of the grid resident
// (the grid is sized to the occupancy), the queue cannot deadlock.  Waits
// are still bounded: after `spin_limit` polls a warp sets the batch error
// word, gives up its item and every other waiter gives up as soon as it sees
// the error, so a broken dependency ends the launch with an error instead of
// a hang.
//
// Memory ordering: the finishing warp stores the vertex, issues a device
// fence and increments the mesh's done counter; the waiting warp polls the
// counter with a volatile load and fences before reading positions, which
// the relocation code loads with __ldcg (L2, coherent across SMs).
#pragma once

#include <cuda_runtime.h>

#include "gm_batch.h"
#include "gm_relocate.cuh"

namespace gm {

constexpr uint32_t kClaimChunk = 8;

__device__ __forceinline__ uint32_t find_segment(const uint32_t* seg_start, uint32_t nseg, uint32_t i)
{
    uint32_t lo = 0, hi = nseg;  // seg_start has nseg + 1 entries
    while (hi - lo > 1)
    {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&seg_start[mid]) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int SMOOTHER, int VAR, int MAXK>
__device__ __forceinline__ void batch_one(const BatchMesh& bm, const SmoothParams& sp, WarpPatch& P, uint32_t v,
                                          int lane, Counters* ctr)
{
    const MeshView& m = bm.view;
    const Crew& crew = bm.crew;
    const int cid = m.cid[v];
    const float4 old = __ldcg(&m.pos[v]);
    V3<float> out;
    float q0, q1;
    int evals = 0;
    if (SMOOTHER == kSmoothGetme)
    {
        // GETMe vertex update: weighted average of the element corners
        const size_t base[4] = {0, 0, 4 * (size_t)m.nt, 4 * (size_t)m.nt + 6 * (size_t)m.np};
        uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
        float sx = 0, sy = 0, sz = 0, sw = 0;
        for (uint32_t i = b + lane; i < e; i += kWarp)
        {
            uint32_t r = m.ve[GM_IX(m, i, m.ve_len, kBoundsNeighbourElem)];
            int type = ref_type(r);
            const size_t ci = base[type] + (size_t)ref_id(r) * type_size(type) + ref_local(r);
            float4 c = bm.corners[GM_IX(m, ci, 4 * m.nt + 6 * m.np + 8 * m.nh, kBoundsCorner)];
            sx += c.x * c.w;
            sy += c.y * c.w;
            sz += c.z * c.w;
            sw += c.w;
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
            sz += __shfl_xor_sync(0xffffffffu, sz, o);
            sw += __shfl_xor_sync(0xffffffffu, sw, o);
        }
        if (sw == 0.f) return;
        out = mk(sx / sw, sy / sw, sz / sw);
        if (cid != 0) out = snap(m, cid, out);
        stage_patch_fp32<VAR, MAXK>(m, crew, v, to<float>(old), P, lane);
        if (lane == 0)
        {
            P.cand[0] = old;
            P.cand[1] = make_float4(out.x, out.y, out.z, 0.f);
        }
        __syncwarp();
        patch_multi<VAR, MAXK, float>(crew, P, 2, lane);
        q0 = P.res[0];
        q1 = P.res[1];
        evals = 2;
        __syncwarp();
    }
    else
    {
        const V3<float> pos = to<float>(old);
        stage_patch_fp32<VAR, MAXK>(m, crew, v, pos, P, lane);
        evals = 2;
        q0 = patch_uniform<VAR, MAXK, float>(crew, P, pos, lane);
        if (SMOOTHER == kSmoothNM) out = nelder_mead<VAR, MAXK>(m, crew, sp, P, v, cid, pos, q0, lane, evals);
        else if (SMOOTHER == kSmoothGD) out = gradient_descent<VAR, MAXK>(m, crew, sp, P, v, cid, pos, lane, evals);
        else out = spawn_search<VAR, MAXK>(m, crew, sp, P, v, cid, pos, lane, evals);
        q1 = patch_uniform<VAR, MAXK, float>(crew, P, out, lane);
    }
    bool accept;
    const bool fp64 = !(q0 >= sp.accept_q && q1 >= sp.accept_q);
    if (fp64)
    {
        // near-degenerate patch: the acceptance test in FP64, on the corner
        // positions (the FP32 search may have staged the canonical form)
        if constexpr (TetCanon<VAR, MAXK>::on)
        {
            __syncwarp();
            stage_patch(m, v, P, lane);
        }
        const double d0 = patch_uniform<VAR, MAXK, double>(crew, P, to<double>(old), lane);
        const double d1 = patch_uniform<VAR, MAXK, double>(crew, P, mk<double>(out.x, out.y, out.z), lane);
        accept = !(d1 < d0);
    }
    else
        accept = SMOOTHER == kSmoothGetme ? !(q1 < q0) : true;
    if (lane == 0 && accept) m.pos[v] = make_float4(out.x, out.y, out.z, old.w);
    count_work(ctr, evals, P.E, MAXK == 4 ? kTet : kHex, fp64, lane);
}

// Nelder-Mead on canonical tet patches in lockstep (gm_nm_lockstep.cuh):
// the warp claims chunks of the queue and hands items to its idle groups in
// queue order; a group whose mesh has not finished the item's earlier
// colours waits without holding up the other groups (one poll per step,
// bounded by spin_limit).  The FP64 acceptance test of a near-degenerate
// patch runs warp-wide, one group at a time, with the positions read from
// the mesh (patch_quality_global: the arithmetic of the acceptance kernel of
// the plain path).  Deadlock freedom is the queue's: an item waits only
// for items earlier in the queue, which were handed out before it.
template <int VAR>
__device__ void nm_lockstep_batch(const BatchArgs& a, const SmoothParams& sp, char* wsm, int lane)
{
    const int gi = lane / kNMGroup, sub = lane & (kNMGroup - 1), leader = gi * kNMGroup;
    WarpPatch P = nm_group_patch<VAR>(wsm, gi, a.maxe);
    float* con = nm_group_con<VAR>(wsm, gi, a.maxe);
    float4* st = nm_group_state<VAR>(wsm, gi, a.maxe);
    const unsigned gmask = 0xffu << leader;
    NMGroup g;
    g.phase = kNMIdle;
    g.E = 0;
    g.cid = 0;
    const BatchMesh* bm = a.meshes;  // the group's mesh (any valid entry while idle)
    uint32_t mesh = 0, need = 0;
    unsigned int seen = 0;  // the mesh's done count, polled one step ahead of its use
    unsigned int spins = 0;
    const unsigned int spin_limit = a.spin_limit < 0xffffffffull ? (unsigned int)a.spin_limit : 0xffffffffu;
    TetConst kc = tet_const<VAR>(bm->crew);
    bool sine = false;
    uint32_t cur = 0, last = 0, seg = 0;  // the warp's chunk [cur, last) and the segment of cur
    bool exhausted = false;
    unsigned int n_evals = 0, n_elems = 0, n_fp64 = 0;
    while (true)
    {
        // (1) idle groups take the next items, in group order (skipped while
        // no group is idle, the common case)
        const unsigned ball = __ballot_sync(kFullMask, g.phase == kNMIdle && sub == 0);
        if (ball)
        {
            const bool idle = g.phase == kNMIdle;
            if (cur >= last && !exhausted)
            {
                uint32_t first = 0;
                if (lane == 0) first = atomicAdd(&a.ctl->next, kClaimChunk);
                first = __shfl_sync(kFullMask, first, 0);
                if (first >= a.total) exhausted = true;
                else
                {
                    cur = first;
                    last = min(first + kClaimChunk, a.total);
                    seg = find_segment(a.seg_start, a.nseg, first);
                }
            }
            const uint32_t rank = __popc(ball & ((1u << leader) - 1u));
            const uint32_t avail = cur < last ? last - cur : 0u;
            if (idle && rank < avail)
            {
                const uint32_t item = cur + rank;
                uint32_t s = seg;
                while (item >= __ldg(&a.seg_start[s + 1])) ++s;
                const Segment sg = a.segs[s];
                bm = &a.meshes[sg.mesh];
                mesh = sg.mesh;
                need = sg.need;
                spins = 0;
                seen = 0;
                g.v = GM_IX(bm->view, bm->members[sg.member_begin + (item - __ldg(&a.seg_start[s]))], bm->view.nv,
                            kBoundsPosition);
                g.phase = kNMWait;
            }
            cur += min((uint32_t)__popc(ball), avail);
            while (cur < last && cur >= __ldg(&a.seg_start[seg + 1])) ++seg;
            if (!__any_sync(kFullMask, g.phase != kNMIdle))
            {
                if (exhausted) break;
                continue;
            }
        }
        // (2) a waiting group starts once its mesh's earlier colours are done
        // (the done count was loaded at the end of the previous step); skipped
        // while no group waits
        int give_up = 0;
        if (__ballot_sync(kFullMask, g.phase == kNMWait))
        {
            int ok = 0;
            if (g.phase == kNMWait && sub == 0)
            {
                if (need == 0 || seen >= need) ok = 1;
                else if (++spins > spin_limit || __ldcv(&a.ctl->error))
                {
                    atomicOr(&a.ctl->error, 1u);
                    give_up = 1;
                }
            }
            ok = __shfl_sync(kFullMask, ok, leader);
            give_up = __shfl_sync(kFullMask, give_up, leader);
            if (__any_sync(kFullMask, ok))
            {
                float ls = 0.f;
                uint32_t nvv = 1;
                if (ok)
                {
                    __threadfence();
                    sine = VAR == kVarMCDiag && sine_metric(bm->crew);
                    kc = tet_const<VAR>(bm->crew);
                    ls = nm_begin<VAR>(g, bm->view, sine, P, con, g.v, sub, nvv);
                }
                __syncwarp();
                nm_finish_begin(g, sp, ok, ls, nvv);
            }
        }
        // (3) one evaluation per busy group
        const bool busy = g.phase >= kNMQ0;
        if (!__any_sync(kFullMask, busy)) __nanosleep(100);
        // poll for the still-waiting groups; the value is used at the next
        // step, so the load's latency overlaps this step's evaluation
        if (g.phase == kNMWait && sub == 0 && !give_up && need) seen = __ldcv(&a.done[mesh]);
        const float f = nm_group_quality<VAR>(P, busy ? g.E : 0, g.vo.p, g.cand, kc, sine, sub);
        bool finishing = false, need64 = false, accept = true;
        if (busy)
        {
            ++g.evals;
            if (g.phase != kNMFinal) nm_step(g, f, sp, con, st, gmask, sub);
            else
            {
                finishing = true;
                need64 = !(g.q0 >= sp.accept_q && f >= sp.accept_q);
            }
        }
        // (4) near-degenerate patches: the acceptance test in FP64, warp-wide
        unsigned m64;
        while ((m64 = __ballot_sync(kFullMask, need64 && sub == 0)) != 0u)
        {
            const int src = __ffs(m64) - 1;
            const BatchMesh* bx =
                reinterpret_cast<const BatchMesh*>(__shfl_sync(kFullMask, reinterpret_cast<unsigned long long>(bm), src));
            const uint32_t vx = __shfl_sync(kFullMask, g.v, src);
            const double ox = __shfl_sync(kFullMask, g.vo.p.x, src), oy = __shfl_sync(kFullMask, g.vo.p.y, src);
            const double oz = __shfl_sync(kFullMask, g.vo.p.z, src);
            const double nx = __shfl_sync(kFullMask, g.cand.x, src), ny = __shfl_sync(kFullMask, g.cand.y, src);
            const double nz = __shfl_sync(kFullMask, g.cand.z, src);
            const double d0 = patch_quality_global<VAR, 4>(bx->view, bx->crew, vx, mk(ox, oy, oz), lane);
            const double d1 = patch_quality_global<VAR, 4>(bx->view, bx->crew, vx, mk(nx, ny, nz), lane);
            if (gi == src / kNMGroup)
            {
                accept = !(d1 < d0);
                need64 = false;
            }
            __syncwarp();
        }
        // (5) finished vertices: commit, count the vertex done for its mesh
        if (finishing || give_up)
        {
            if (sub == 0)
            {
                if (finishing)
                {
                    if (accept) bm->view.pos[g.v] = make_float4(g.cand.x, g.cand.y, g.cand.z, g.ow);
                    n_evals += (unsigned int)g.evals;
                    n_elems += (unsigned int)(g.evals * g.E);
                    n_fp64 += (g.q0 >= sp.accept_q && f >= sp.accept_q) ? 0u : 1u;
                }
                __threadfence();
                const unsigned int d = atomicAdd(&a.done[mesh], 1u) + 1u;
                if (d == bm->nmembers)
                {
                    unsigned long long now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    a.finish[mesh] = now;
                }
            }
            g.phase = kNMIdle;
        }
    }
    nm_flush_counters(a.ctr, n_evals, n_elems, n_fp64, lane);
}

template <int SMOOTHER, int VAR, int MAXK>
struct BatchLockstep
{
    static constexpr bool on = SMOOTHER == kSmoothNM && TetCanon<VAR, MAXK>::on;
};

template <int SMOOTHER, int VAR, int MAXK>
__device__ __forceinline__ void batch_queue_loop(const BatchArgs& a, const SmoothParams& sp, char* smem);

template <int SMOOTHER, int VAR, int MAXK>
__global__ void __launch_bounds__(256, BatchLockstep<SMOOTHER, VAR, MAXK>::on ? (VAR == kVarMRFree ? 3 : 2)
                                      : (VAR == kVarMC || VAR == kVarMRWise) ? 1
                                      : (VAR == kVarMCDiag && MAXK == 4 && SMOOTHER != kSmoothGetme) ? 2
                                      : (MAXK == 4 ? 3 : 1))
    batch_relocate_kernel(BatchArgs a, SmoothParams sp)
{
    extern __shared__ __align__(16) char smem[];
    if constexpr (BatchLockstep<SMOOTHER, VAR, MAXK>::on)
    {
        const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
        if (threadIdx.x == 0)
        {
            unsigned long long now;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            atomicCAS(&a.ctl->t0, 0ull, now);
        }
        nm_lockstep_batch<VAR>(a, sp, smem + wib * nm_warp_bytes<VAR>(a.maxe), lane);
    }
    else
        batch_queue_loop<SMOOTHER, VAR, MAXK>(a, sp, smem);
}

// one warp per vertex: claim chunks of the queue, wait for each item's
// dependencies, relocate it
template <int SMOOTHER, int VAR, int MAXK>
__device__ __forceinline__ void batch_queue_loop(const BatchArgs& a, const SmoothParams& sp, char* smem)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpPatch P = carve_patch(smem + wib * warp_patch_bytes(MAXK, a.maxe), MAXK, a.maxe);
    if (threadIdx.x == 0)
    {
        unsigned long long now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        atomicCAS(&a.ctl->t0, 0ull, now);
    }
    while (true)
    {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(&a.ctl->next, kClaimChunk);
        first = __shfl_sync(0xffffffffu, first, 0);
        if (first >= a.total) break;
        const uint32_t last = min(first + kClaimChunk, a.total);
        // one search per chunk; later items of the chunk walk forward
        uint32_t s = find_segment(a.seg_start, a.nseg, first);
        uint32_t s_end = __ldg(&a.seg_start[s + 1]);
        for (uint32_t i = first; i < last; ++i)
        {
            while (i >= s_end)
            {
                ++s;
                s_end = __ldg(&a.seg_start[s + 1]);
            }
            const Segment sg = a.segs[s];
            int ok = 1;
            if (sg.need)
            {
                if (lane == 0)
                {
                    unsigned long long spins = 0;
                    while (__ldcv(&a.done[sg.mesh]) < sg.need)
                    {
                        if (++spins > a.spin_limit || __ldcv(&a.ctl->error))
                        {
                            atomicOr(&a.ctl->error, 1u);
                            ok = 0;
                            break;
                        }
                        __nanosleep(100);
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                __threadfence();
            }
            if (ok)
            {
                const BatchMesh& bm = a.meshes[sg.mesh];
                const uint32_t v =
                    GM_IX(bm.view, bm.members[sg.member_begin + (i - __ldg(&a.seg_start[s]))], bm.view.nv, kBoundsPosition);
                batch_one<SMOOTHER, VAR, MAXK>(bm, sp, P, v, lane, a.ctr);
            }
            __syncwarp();
            if (lane == 0)
            {
                __threadfence();
                const unsigned int d = atomicAdd(&a.done[sg.mesh], 1u) + 1u;
                if (d == a.meshes[sg.mesh].nmembers)
                {
                    unsigned long long now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    a.finish[sg.mesh] = now;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// batched evaluation: a block table covering every mesh's elements, then one
// warp per mesh sums its blocks in order (deterministic)
// ---------------------------------------------------------------------------
template <int VAR, int MAXK>
__global__ void __launch_bounds__(256) batch_eval_kernel(const BatchMesh* meshes, const EvalBlock* blocks,
                                                          EvalPartial* parts)
{
    __shared__ int hist[20];
    __shared__ float wmin[8];
    __shared__ double wsum[8];
    __shared__ int wbad[8];
    if (threadIdx.x < 20) hist[threadIdx.x] = 0;
    __syncthreads();
    const EvalBlock eb = blocks[blockIdx.x];
    const MeshView& m = meshes[eb.mesh].view;
    const Crew& crew = meshes[eb.mesh].crew;
    EvalAcc acc;
    for (uint32_t base = eb.begin; base < eb.end; base += blockDim.x)  // block-uniform trip count
    {
        const uint32_t i = base + threadIdx.x;
        int b = -1;
        if (i < eb.end)
        {
            int type;
            uint32_t id;
            if (MAXK == 4 || i < m.nt) { type = kTet; id = i; }
            else if (i < m.nt + m.np) { type = kPri; id = i - m.nt; }
            else { type = kHex; id = i - m.nt - m.np; }
            uint32_t vid[8];
            elem_vertices(m, type, id, vid);
            V3<float> p[MAXK];
            const int n = MAXK == 4 ? 4 : type_size(type);
#pragma unroll
            for (int k = 0; k < MAXK; ++k) p[k] = to<float>(__ldg(&m.pos[vid[k < n ? k : 0]]));
            // the element hint as gm_evaluate gives it: the background-mesh
            // samplers start their walk at the element's first background tet
            b = acc.add(elem_quality<VAR, MAXK, float>(crew, type, p, elem_hint(type, id)));
        }
        hist_add_warp(hist, b);
    }
    double ds = acc.rs;
    float mn = acc.min_quality();
    int nbad = acc.nbad;
    for (int o = 16; o > 0; o >>= 1)
    {
        ds += __shfl_xor_sync(0xffffffffu, ds, o);
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
    {
        wmin[w] = mn;
        wsum[w] = ds;
        wbad[w] = nbad;
    }
    __syncthreads();
    if (threadIdx.x < 20) parts[blockIdx.x].hist[threadIdx.x] = hist[threadIdx.x];
    if (threadIdx.x == 0)
    {
        EvalPartial& p = parts[blockIdx.x];
        float bmin = wmin[0];
        double bsum = wsum[0];
        int bbad = wbad[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
        {
            bmin = fminf(bmin, wmin[k]);
            bsum += wsum[k];
            bbad += wbad[k];
        }
        p.min = bmin;
        p.rsum = bsum;
        p.nbad = bbad;
        p.pad = 0;
    }
}


// one persistent launch of the relocation kernel, sized to full residency
template <int SMOOTHER, int VAR, int MAXK>
inline cudaError_t launch_batch_t(const BatchArgs& a, const SmoothParams& sp, int wpb, int ctas_per_sm, int sm_count,
                                  cudaStream_t s)
{
    auto kern = batch_relocate_kernel<SMOOTHER, VAR, MAXK>;
    size_t smem =
        (BatchLockstep<SMOOTHER, VAR, MAXK>::on ? nm_warp_bytes<VAR>(a.maxe) : patch_smem_per_warp(MAXK, a.maxe)) * wpb;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    // every CTA must be resident: never more than the occupancy allows
    int cps = (ctas_per_sm <= 0 || ctas_per_sm > occ) ? occ : ctas_per_sm;
    kern<<<sm_count * cps, 32 * wpb, smem, s>>>(a, sp);
    note_launch();
    return cudaGetLastError();
}

// one launch of the per-mesh evaluation blocks
template <int VAR, int MAXK>
inline void launch_batch_eval_t(const BatchMesh* meshes, const EvalBlock* blocks, uint32_t nblocks, EvalPartial* parts,
                                cudaStream_t s)
{
    batch_eval_kernel<VAR, MAXK><<<nblocks, 256, 0, s>>>(meshes, blocks, parts);
}

}  // namespace gm
