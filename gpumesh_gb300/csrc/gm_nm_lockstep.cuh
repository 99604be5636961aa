// Nelder-Mead in lockstep: several vertices per warp.
//
// Nelder-Mead evaluates one candidate position at a time.  A warp that
// relocates one vertex spreads each patch evaluation over its lanes (one
// element per lane) and runs the simplex logic and a 5-step reduction on all
// 32 lanes; with canonical tet patches, where an element costs a few fused
// operations, that overhead dominates.  Here a warp holds kNMGroups vertices,
// each on a group of kNMGroup lanes with its own staged patch, and the
// search is a state machine that needs exactly one patch evaluation per
// step: every step evaluates the current candidate of every group at once
// (elements over the group's lanes, 3-step reduction), then advances each
// group's state.  A group whose vertex is done takes the warp's next vertex
// at the next step, so the groups stay busy until the warp's work runs out.
//
// Each vertex follows nelder_mead() (NelderMeadSmoother.cpp:100-260)
// decision for decision: initial simplex, sort, reflection / expansion /
// contraction, insertion, convergence test, one reset with the mirrored
// simplex, final projection.
#pragma once

#include "gm_kernels.cuh"

namespace gm {

constexpr int kNMGroup = 8;                   // lanes per vertex
constexpr int kNMGroups = kWarp / kNMGroup;   // vertices per warp
constexpr unsigned kFullMask = 0xffffffffu;

enum : int { kNMIdle = 0, kNMWait, kNMQ0, kNMInit, kNMReflect, kNMProbe, kNMFinal };

// one group's search; every lane of the group holds the same copy
struct NMGroup
{
    int phase;
    int cid;
    int E;
    int k;      // initial simplex vertex being evaluated
    int cycle;
    int evals;
    bool reset;
    uint32_t v;
    float ns;   // node shift
    float q0;
    float fr;   // reflection value of the current cycle
    float4 old;
    S4 s0, s1, s2, s3, vo;
    V3<float> c, xr, cand;
};

// shared memory of one warp: the groups' canonical patches, then a
// corner-position patch for the FP64 acceptance test of the batched path
__host__ __device__ constexpr size_t nm_warp_bytes(int maxe)
{
    return ((size_t)kNMGroups * patch_slots(4) * maxe + 4 * (size_t)maxe) * 16 + (size_t)maxe * 4;
}

__device__ __forceinline__ WarpPatch nm_group_patch(char* wsm, int gi, int maxe)
{
    WarpPatch P;
    P.sp = reinterpret_cast<float4*>(wsm) + (size_t)gi * patch_slots(4) * maxe;
    P.meta = nullptr;
    P.cand = nullptr;
    P.res = nullptr;
    P.maxe = maxe;
    P.E = 0;
    P.o = V3<float>{0.f, 0.f, 0.f};
    return P;
}

__device__ __forceinline__ WarpPatch nm_fp64_patch(char* wsm, int maxe)
{
    WarpPatch P = nm_group_patch(wsm, kNMGroups, maxe);
    P.meta = reinterpret_cast<int*>(P.sp + 4 * (size_t)maxe);
    return P;
}

__device__ __forceinline__ V3<float> nm_snap(const MeshView& m, int cid, V3<float> x)
{
    return cid != 0 ? snap(m, cid, x) : x;
}

// patch quality of the group's candidate (E = 0: an idle group, result unused)
template <int VAR>
__device__ __forceinline__ float nm_group_quality(const Crew& crew, const WarpPatch& P, int E, V3<float> c,
                                                  const TetConst& kc, bool sine, int sub)
{
    const TetCand t = tet_cand<VAR>(crew, P.o, c);
    PatchAcc<float> a{0.f, 3.0e38f, 0};
    for (int e = sub; e < E; e += kNMGroup) acc_add(a, canonical_quality<VAR>(P, e, t, kc, sine));
    acc_reduce(a, kNMGroup);
    return acc_final(a, E);
}

// the next cycle: reflection, or the final point, or the reset simplex
__device__ __forceinline__ void nm_next_cycle(NMGroup& g, const SmoothParams& sp, const MeshView& m)
{
    if (g.cycle < sp.cycles)
    {
        g.c = (g.s1.p + g.s2.p + g.s3.p) * (1.f / 3.f);
        g.cand = nm_snap(m, g.cid, g.c + (g.c - g.s0.p) * sp.alpha);
        g.phase = kNMReflect;
    }
    else if (g.reset)
    {
        g.cand = nm_snap(m, g.cid, g.s3.p);
        g.phase = kNMFinal;
    }
    else
    {
        g.s0 = S4{g.vo.p - mk(g.ns, 0.f, 0.f), g.vo.w};
        g.s1 = S4{g.vo.p - mk(0.f, g.ns, 0.f), g.vo.w};
        g.s2 = S4{g.vo.p - mk(0.f, 0.f, g.ns), g.vo.w};
        g.s3 = g.vo;
        g.reset = true;
        g.cycle = 0;
        g.k = 0;
        g.cand = nm_snap(m, g.cid, g.s0.p);
        g.phase = kNMInit;
    }
}

__device__ __forceinline__ void nm_insert(NMGroup& g, S4 vx, const SmoothParams& sp, const MeshView& m)
{
    if (vx.w > g.s3.w) swp(g.s3, vx);
    if (vx.w > g.s2.w) swp(g.s2, vx);
    if (vx.w > g.s1.w) swp(g.s1, vx);
    if (vx.w > g.s0.w) swp(g.s0, vx);
    if ((g.s3.w - g.s1.w) < sp.convergence)
    {
        g.cand = nm_snap(m, g.cid, g.s3.p);
        g.phase = kNMFinal;
        return;
    }
    ++g.cycle;
    nm_next_cycle(g, sp, m);
}

// advance the group with the quality f of its candidate
__device__ __forceinline__ void nm_step(NMGroup& g, float f, const SmoothParams& sp, const MeshView& m)
{
    switch (g.phase)
    {
    case kNMQ0:
    {
        const V3<float> pos = to<float>(g.old);
        g.q0 = f;
        g.vo = S4{pos, f};
        g.s0 = S4{pos + mk(g.ns, 0.f, 0.f), 0.f};
        g.s1 = S4{pos + mk(0.f, g.ns, 0.f), 0.f};
        g.s2 = S4{pos + mk(0.f, 0.f, g.ns), 0.f};
        g.s3 = g.vo;
        g.cycle = 0;
        g.reset = false;
        g.k = 0;
        g.cand = nm_snap(m, g.cid, g.s0.p);
        g.phase = kNMInit;
        break;
    }
    case kNMInit:
    {
        const S4 nv{g.cand, f};
        if (g.k == 0) g.s0 = nv;
        else if (g.k == 1) g.s1 = nv;
        else g.s2 = nv;
        ++g.k;
        if (g.k < 3)
        {
            g.cand = nm_snap(m, g.cid, g.k == 1 ? g.s1.p : g.s2.p);
            break;
        }
        if (g.s0.w > g.s1.w) swp(g.s0, g.s1);
        if (g.s1.w > g.s2.w) swp(g.s1, g.s2);
        if (g.s2.w > g.s3.w) swp(g.s2, g.s3);
        if (g.s0.w > g.s1.w) swp(g.s0, g.s1);
        if (g.s1.w > g.s2.w) swp(g.s1, g.s2);
        if (g.s0.w > g.s1.w) swp(g.s0, g.s1);
        nm_next_cycle(g, sp, m);
        break;
    }
    case kNMReflect:
    {
        g.fr = f;
        g.xr = g.cand;
        V3<float> x = g.xr;
        bool probe = true;
        if (g.s3.w < f) x = g.c + (g.xr - g.c) * sp.gamma;                                 // expand
        else if (g.s1.w >= f) x = g.c + ((f > g.s0.w ? g.xr : g.s0.p) - g.c) * sp.beta;  // contract
        else probe = false;                                                               // accept
        if (probe)
        {
            g.cand = nm_snap(m, g.cid, x);
            g.phase = kNMProbe;
        }
        else
            nm_insert(g, S4{g.xr, f}, sp, m);
        break;
    }
    case kNMProbe:
    {
        S4 vx{g.cand, f};
        if (g.s3.w < g.fr && f <= g.fr) vx = S4{g.xr, g.fr};
        nm_insert(g, vx, sp, m);
        break;
    }
    default: break;
    }
}

// a group takes vertex v: canonical patch over its lanes, start position
template <int VAR>
__device__ __forceinline__ void nm_begin(NMGroup& g, const MeshView& m, const Crew& crew, WarpPatch& P, uint32_t v,
                                         int sub)
{
    g.v = v;
    g.cid = m.cid[v];
    g.old = __ldcg(&m.pos[v]);
    stage_canonical_range<VAR>(m, crew, v, to<float>(g.old), P, sub, kNMGroup);
    g.E = P.E;
    g.evals = 0;
    g.cand = to<float>(g.old);
    g.phase = kNMQ0;
}

// local element size of the starting groups' vertices (all lanes take part)
__device__ __forceinline__ void nm_local_size(NMGroup& g, const MeshView& m, const SmoothParams& sp, bool start,
                                              int sub)
{
    float s = 0.f;
    uint32_t b = 0, e = 0;
    if (start)
    {
        b = m.vv_off[g.v];
        e = m.vv_off[g.v + 1];
        const V3<float> pos = to<float>(g.old);
        for (uint32_t i = b + sub; i < e; i += kNMGroup) s += length(to<float>(__ldcg(&m.pos[m.vv[i]])) - pos);
    }
    for (int o = kNMGroup / 2; o > 0; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
    if (start) g.ns = s / (float)(e - b) * sp.shift;
}

__device__ __forceinline__ void nm_flush_counters(Counters* ctr, unsigned long long evals,
                                                  unsigned long long elems, unsigned long long fp64, int lane)
{
    if (!ctr) return;
    for (int o = 16; o > 0; o >>= 1)
    {
        evals += __shfl_xor_sync(kFullMask, evals, o);
        elems += __shfl_xor_sync(kFullMask, elems, o);
        fp64 += __shfl_xor_sync(kFullMask, fp64, o);
    }
    if (lane == 0)
    {
        atomicAdd(&ctr->patch_evals, evals);
        atomicAdd(&ctr->elem_evals[kTet], elems);
        if (fp64) atomicAdd(&ctr->fp64_vertices, fp64);
    }
}

// Plain path: the warp relocates members[begin, end) of one colour; a vertex
// whose old or new patch quality is below the acceptance threshold is
// deferred to the FP64 acceptance kernel.
template <int VAR>
__device__ void nm_lockstep_plain(const MeshView& m, const Crew& crew, const SmoothParams& sp,
                                  const uint32_t* members, uint32_t begin, uint32_t end, char* wsm, int maxe,
                                  Counters* ctr, const Deferred& def, uint32_t slot_base, int lane)
{
    const int gi = lane / kNMGroup, sub = lane & (kNMGroup - 1);
    WarpPatch P = nm_group_patch(wsm, gi, maxe);
    const TetConst kc = tet_const<VAR>(crew);
    const bool sine = VAR == kVarMCDiag && sine_metric(crew);
    NMGroup g;
    g.phase = kNMIdle;
    g.E = 0;
    uint32_t next = begin;
    unsigned long long n_evals = 0, n_elems = 0, n_fp64 = 0;
    while (true)
    {
        // idle groups take the next vertices, in group order
        const bool idle = g.phase == kNMIdle;
        const unsigned ball = __ballot_sync(kFullMask, idle && sub == 0);
        const uint32_t rank = __popc(ball & ((1u << (gi * kNMGroup)) - 1u));
        const uint32_t base = next;
        const bool start = idle && base + rank < end;
        next += __popc(ball);
        if (!__any_sync(kFullMask, start || !idle)) break;
        if (start) nm_begin<VAR>(g, m, crew, P, members[base + rank], sub);
        __syncwarp();
        if (__any_sync(kFullMask, start)) nm_local_size(g, m, sp, start, sub);
        // one evaluation per busy group
        const bool busy = g.phase != kNMIdle;
        const float f = nm_group_quality<VAR>(crew, P, busy ? g.E : 0, g.cand, kc, sine, sub);
        if (!busy) continue;
        ++g.evals;
        if (g.phase != kNMFinal)
        {
            nm_step(g, f, sp, m);
            continue;
        }
        // done: commit, or defer to the FP64 acceptance kernel
        const bool defer = !(g.q0 >= sp.accept_q && f >= sp.accept_q);
        if (sub == 0)
        {
            const float4 nw = make_float4(g.cand.x, g.cand.y, g.cand.z, g.old.w);
            if (defer)
            {
                const uint32_t k = atomicAdd(def.count, 1u);
                def.v[slot_base + k] = g.v;
                def.oldp[slot_base + k] = g.old;
                def.newp[slot_base + k] = nw;
            }
            else
                m.pos[g.v] = nw;
            n_evals += (unsigned long long)g.evals;
            n_elems += (unsigned long long)g.evals * (unsigned long long)g.E;
            n_fp64 += defer ? 1ull : 0ull;
        }
        g.phase = kNMIdle;
    }
    nm_flush_counters(ctr, n_evals, n_elems, n_fp64, lane);
}

}  // namespace gm
