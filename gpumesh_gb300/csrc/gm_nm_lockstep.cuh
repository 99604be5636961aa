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
// Everything a step needs is in registers or shared memory: the patch, and
// the vertex's boundary constraint copied next to it when the vertex starts.
// The simplex, centroid, reflection and cycle counters are read only by the
// step's state update, so they live in a per-group shared record between
// steps instead of holding registers through the patch evaluation.
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
constexpr int kNMConWords = 16;               // constraint record per group
constexpr int kNMStateVecs = 7;               // search record per group, float4s
constexpr unsigned kFullMask = 0xffffffffu;

enum : int { kNMIdle = 0, kNMWait, kNMQ0, kNMInit, kNMReflect, kNMProbe, kNMFinal };

// one group's search; every lane of the group holds the same copy
struct NMGroup
{
    int phase;
    int cid;
    int E;
    int evals;
    uint32_t v;
    float ns;   // node shift
    float q0;
    float ow;   // the w word of the vertex's position record, kept on commit
    S4 vo;      // vo.p: the position at the start (the patch origin)
    V3<float> cand;
};

// the rest of the search, in the group's shared record between steps
struct NMState
{
    S4 s0, s1, s2, s3;
    V3<float> c, xr;
    float fr;    // reflection value of the current cycle
    int k;       // initial simplex vertex being evaluated
    int cycle;
    bool reset;
};

__device__ __forceinline__ NMState nm_load(const float4* st)
{
    const float4 a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], h = st[6];
    NMState S;
    S.s0 = S4{mk(a.x, a.y, a.z), a.w};
    S.s1 = S4{mk(b.x, b.y, b.z), b.w};
    S.s2 = S4{mk(c.x, c.y, c.z), c.w};
    S.s3 = S4{mk(d.x, d.y, d.z), d.w};
    S.c = mk(e.x, e.y, e.z);
    S.fr = e.w;
    S.xr = mk(f.x, f.y, f.z);
    S.k = __float_as_int(f.w);
    S.cycle = __float_as_int(h.x);
    S.reset = __float_as_int(h.y) != 0;
    return S;
}

__device__ __forceinline__ void nm_store(float4* st, const NMState& S)
{
    st[0] = make_float4(S.s0.p.x, S.s0.p.y, S.s0.p.z, S.s0.w);
    st[1] = make_float4(S.s1.p.x, S.s1.p.y, S.s1.p.z, S.s1.w);
    st[2] = make_float4(S.s2.p.x, S.s2.p.y, S.s2.p.z, S.s2.w);
    st[3] = make_float4(S.s3.p.x, S.s3.p.y, S.s3.p.z, S.s3.w);
    st[4] = make_float4(S.c.x, S.c.y, S.c.z, S.fr);
    st[5] = make_float4(S.xr.x, S.xr.y, S.xr.z, __int_as_float(S.k));
    st[6] = make_float4(__int_as_float(S.cycle), __int_as_float(S.reset ? 1 : 0), 0.f, 0.f);
}

// canonical slots per element: mean ratio reads the three frame columns,
// metric conformity also the staged sines and cosines
template <int VAR>
__host__ __device__ constexpr int nm_slots()
{
    return VAR == kVarMRFree ? 3 : patch_slots(4);
}

// shared memory of one warp: the groups' canonical patches, then one
// constraint record per group, then one search record per group
template <int VAR>
__host__ __device__ constexpr size_t nm_warp_bytes(int maxe)
{
    return (size_t)kNMGroups * nm_slots<VAR>() * maxe * 16 + (size_t)kNMGroups * kNMConWords * 4 +
           (size_t)kNMGroups * kNMStateVecs * 16;
}

template <int VAR>
__device__ __forceinline__ WarpPatch nm_group_patch(char* wsm, int gi, int maxe)
{
    WarpPatch P;
    P.sp = reinterpret_cast<float4*>(wsm) + (size_t)gi * nm_slots<VAR>() * maxe;
    P.pp = nullptr;  // one candidate at a time: no paired evaluation
    P.meta = nullptr;
    P.cand = nullptr;
    P.res = nullptr;
    P.maxe = maxe;
    P.E = 0;
    P.o = V3<float>{0.f, 0.f, 0.f};
    return P;
}

template <int VAR>
__device__ __forceinline__ float* nm_group_con(char* wsm, int gi, int maxe)
{
    return reinterpret_cast<float*>(wsm + (size_t)kNMGroups * nm_slots<VAR>() * maxe * 16) + gi * kNMConWords;
}

template <int VAR>
__device__ __forceinline__ float4* nm_group_state(char* wsm, int gi, int maxe)
{
    return reinterpret_cast<float4*>(wsm + (size_t)kNMGroups * nm_slots<VAR>() * maxe * 16 +
                                     (size_t)kNMGroups * kNMConWords * 4) +
           gi * kNMStateVecs;
}

// project() on a constraint record copied from a Constraint's FP32 head
// (kind, a, b, u, len), the same formulas
__device__ __forceinline__ V3<float> project_rec(const float* r, V3<float> p)
{
    const V3<float> a = mk(r[1], r[2], r[3]);
    switch (__float_as_int(r[0]))
    {
    case kConPlane:
    {
        const V3<float> n = mk(r[4], r[5], r[6]);
        const float l = dot(p - a, n);
        return p - n * l;
    }
    case kConSegment:
    {
        const V3<float> u = mk(r[7], r[8], r[9]);
        const V3<float> dist = p - a;
        const float l = dot(dist, u);
        if (l < 0.f) return a;
        if (l > r[10]) return mk(r[4], r[5], r[6]);
        return p - (dist - u * l);
    }
    case kConSphere: return normalize(p);
    case kConPoint: return a;
    case kConShellInner: return normalize(p) * 0.5f;
    case kConPipeCylinder: return pipe_cylinder(p);
    case kConPipeCircle: return pipe_circle(a, p);
    default: return p;
    }
}

__device__ __forceinline__ V3<float> nm_snap(const NMGroup& g, const float* con, V3<float> x)
{
    return g.cid != 0 ? project_rec(con, x) : x;
}

// patch quality of the group's candidate (E = 0: an idle group, result unused)
template <int VAR>
__device__ __forceinline__ float nm_group_quality(const WarpPatch& P, int E, V3<float> origin, V3<float> c,
                                                  const TetConst& kc, bool sine, int sub)
{
    const TetCand t = tet_cand<VAR>(sine, origin, c);
    PatchAcc<float> a{0.f, 3.0e38f, 0};
    for (int e = sub; e < E; e += kNMGroup) acc_add(a, canonical_quality<VAR>(P, e, t, kc, sine));
    acc_reduce(a, kNMGroup);
    return acc_final(a, E);
}

// Advance the group with the quality f of its candidate.  The groups of a
// warp are usually in different phases, and SIMT runs each distinct path
// once for the groups on it, so the phase-specific parts are short and the
// common tail (insertion, convergence test, next cycle, projection of the
// next candidate) is one block shared by every group that reaches it.  The
// group's lanes read its shared record, update their copies alike, and lane
// 0 writes it back once all of them have read it (gmask: the group's lanes).
__device__ __forceinline__ void nm_step(NMGroup& g, float f, const SmoothParams& sp, const float* con, float4* st,
                                        unsigned gmask, int sub)
{
    NMState S = nm_load(st);
    bool insert = false, next = false, snap_next = true;
    S4 vx{g.cand, f};
    V3<float> x = g.cand;  // the next candidate before projection
    const int phase = g.phase;
    if (phase == kNMReflect)
    {
        S.fr = f;
        S.xr = g.cand;
        if (S.s3.w < f)  // expand
        {
            x = S.c + (S.xr - S.c) * sp.gamma;
            g.phase = kNMProbe;
        }
        else if (S.s1.w >= f)  // contract
        {
            x = S.c + ((f > S.s0.w ? S.xr : S.s0.p) - S.c) * sp.beta;
            g.phase = kNMProbe;
        }
        else  // accept the reflection
        {
            insert = true;
            snap_next = false;
        }
    }
    else if (phase == kNMProbe)
    {
        if (S.s3.w < S.fr && f <= S.fr) vx = S4{S.xr, S.fr};
        insert = true;
        snap_next = false;
    }
    else if (phase == kNMInit)
    {
        if (S.k == 0) S.s0 = vx;
        else if (S.k == 1) S.s1 = vx;
        else S.s2 = vx;
        ++S.k;
        if (S.k < 3) x = S.k == 1 ? S.s1.p : S.s2.p;
        else
        {
            if (S.s0.w > S.s1.w) swp(S.s0, S.s1);
            if (S.s1.w > S.s2.w) swp(S.s1, S.s2);
            if (S.s2.w > S.s3.w) swp(S.s2, S.s3);
            if (S.s0.w > S.s1.w) swp(S.s0, S.s1);
            if (S.s1.w > S.s2.w) swp(S.s1, S.s2);
            if (S.s0.w > S.s1.w) swp(S.s0, S.s1);
            next = true;
            snap_next = false;
        }
    }
    else  // kNMQ0
    {
        const V3<float> pos = g.vo.p;
        g.q0 = f;
        g.vo = S4{pos, f};
        S.s0 = S4{pos + mk(g.ns, 0.f, 0.f), 0.f};
        S.s1 = S4{pos + mk(0.f, g.ns, 0.f), 0.f};
        S.s2 = S4{pos + mk(0.f, 0.f, g.ns), 0.f};
        S.s3 = g.vo;
        S.cycle = 0;
        S.reset = false;
        S.k = 0;
        x = S.s0.p;
        g.phase = kNMInit;
    }
    if (insert)
    {
        if (vx.w > S.s3.w) swp(S.s3, vx);
        if (vx.w > S.s2.w) swp(S.s2, vx);
        if (vx.w > S.s1.w) swp(S.s1, vx);
        if (vx.w > S.s0.w) swp(S.s0, vx);
        if ((S.s3.w - S.s1.w) < sp.convergence)
        {
            x = S.s3.p;
            g.phase = kNMFinal;
            snap_next = true;
        }
        else
        {
            ++S.cycle;
            next = true;
        }
    }
    if (next)
    {
        snap_next = true;
        if (S.cycle < sp.cycles)
        {
            S.c = (S.s1.p + S.s2.p + S.s3.p) * (1.f / 3.f);
            x = S.c + (S.c - S.s0.p) * sp.alpha;
            g.phase = kNMReflect;
        }
        else if (S.reset)
        {
            x = S.s3.p;
            g.phase = kNMFinal;
        }
        else
        {
            S.s0 = S4{g.vo.p - mk(g.ns, 0.f, 0.f), g.vo.w};
            S.s1 = S4{g.vo.p - mk(0.f, g.ns, 0.f), g.vo.w};
            S.s2 = S4{g.vo.p - mk(0.f, 0.f, g.ns), g.vo.w};
            S.s3 = g.vo;
            S.reset = true;
            S.cycle = 0;
            S.k = 0;
            x = S.s0.p;
            g.phase = kNMInit;
        }
    }
    if (snap_next) g.cand = nm_snap(g, con, x);
    __syncwarp(gmask);
    if (sub == 0) nm_store(st, S);
    __syncwarp(gmask);
}

// A group takes vertex v: canonical patch and constraint record over its
// lanes, start position; returns this lane's part of the local element size
// sum (AbstractMeasurer::computeLocalElementSize), reduced by nm_finish_begin.
// The element and neighbour loads go out in the same loop so that their
// latencies overlap.
template <int VAR>
__device__ __forceinline__ float nm_begin(NMGroup& g, const MeshView& m, bool sine, WarpPatch& P, float* con,
                                          uint32_t v, int sub, uint32_t& nvv)
{
    g.v = v;
    g.cid = m.cid[v];
    const float4 old = __ldcg(&m.pos[v]);
    g.ow = old.w;
    const uint32_t eb = m.ve_off[v], ee = m.ve_off[v + 1];
    const uint32_t vb = m.vv_off[v], ve = m.vv_off[v + 1];
    const V3<float> o = to<float>(old);
    g.vo.p = o;
    P.E = (int)(ee - eb);
    nvv = ve - vb;
    float ls = 0.f;
    const uint32_t n = max(ee - eb, ve - vb);
    for (uint32_t i = sub; i < n; i += kNMGroup)
    {
        if (i < ve - vb)
        {
            const uint32_t w = m.vv[GM_IX(m, vb + i, m.vv_len, kBoundsNeighbourVert)];
            ls += length(to<float>(__ldcg(&m.pos[GM_IX(m, w, m.nv, kBoundsPosition)])) - o);
        }
        if (i < ee - eb)
        {
            const uint32_t r = m.ve[GM_IX(m, eb + i, m.ve_len, kBoundsNeighbourElem)];
            const int x = 3 ^ ref_local(r);
            const uint4 t = m.tets[GM_IX(m, ref_id(r), m.nt, kBoundsTet)];
            const float4 a0 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, x), m.nv, kBoundsPosition)]);
            const float4 a1 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, 1 ^ x), m.nv, kBoundsPosition)]);
            const float4 a2 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, 2 ^ x), m.nv, kBoundsPosition)]);
            stage_canonical_element<VAR>(P, (int)i, a0, a1, a2, o, sine);
        }
    }
    // the FP32 head of the vertex's Constraint (identity for a free vertex or
    // an id outside the table, as project() treats them)
    const bool has = g.cid > 0 && g.cid < m.ncon;
    for (int w = sub; w < 11; w += kNMGroup)
        con[w] = has ? reinterpret_cast<const float*>(&m.con[g.cid])[w] : __int_as_float(kConVolume);
    g.E = P.E;
    g.evals = 0;
    g.cand = o;
    g.phase = kNMQ0;
    return ls;
}

// reduce the local size sums of starting groups (all lanes take part)
__device__ __forceinline__ void nm_finish_begin(NMGroup& g, const SmoothParams& sp, bool start, float ls,
                                                uint32_t nvv)
{
    for (int o = kNMGroup / 2; o > 0; o >>= 1) ls += __shfl_xor_sync(kFullMask, ls, o);
    if (start) g.ns = ls / (float)nvv * sp.shift;
}

__device__ __forceinline__ void nm_flush_counters(Counters* ctr, unsigned int evals, unsigned int elems,
                                                  unsigned int fp64, int lane)
{
    if (!ctr) return;
    unsigned long long e = evals, el = elems, f = fp64;
    for (int o = 16; o > 0; o >>= 1)
    {
        e += __shfl_xor_sync(kFullMask, e, o);
        el += __shfl_xor_sync(kFullMask, el, o);
        f += __shfl_xor_sync(kFullMask, f, o);
    }
    if (lane == 0)
    {
        atomicAdd(&ctr->patch_evals, e);
        atomicAdd(&ctr->elem_evals[kTet], el);
        if (f) atomicAdd(&ctr->fp64_vertices, f);
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
    WarpPatch P = nm_group_patch<VAR>(wsm, gi, maxe);
    float* con = nm_group_con<VAR>(wsm, gi, maxe);
    float4* st = nm_group_state<VAR>(wsm, gi, maxe);
    const unsigned gmask = 0xffu << (gi * kNMGroup);
    const TetConst kc = tet_const<VAR>(crew);
    const bool sine = VAR == kVarMCDiag && sine_metric(crew);
    NMGroup g;
    g.phase = kNMIdle;
    g.E = 0;
    g.cid = 0;
    uint32_t next = begin;
    unsigned int n_evals = 0, n_elems = 0, n_fp64 = 0;  // per warp: well within 32 bits
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
        if (__any_sync(kFullMask, start))
        {
            float ls = 0.f;
            uint32_t nvv = 1;
            if (start)
                ls = nm_begin<VAR>(g, m, sine, P, con, GM_IX(m, members[base + rank], m.nv, kBoundsPosition), sub, nvv);
            __syncwarp();
            nm_finish_begin(g, sp, start, ls, nvv);
        }
        // one evaluation per busy group
        const bool busy = g.phase != kNMIdle;
        const float f = nm_group_quality<VAR>(P, busy ? g.E : 0, g.vo.p, g.cand, kc, sine, sub);
        if (!busy) continue;
        ++g.evals;
        if (g.phase != kNMFinal)
        {
            nm_step(g, f, sp, con, st, gmask, sub);
            continue;
        }
        // done: commit, or defer to the FP64 acceptance kernel
        const bool defer = !(g.q0 >= sp.accept_q && f >= sp.accept_q);
        if (sub == 0)
        {
            const float4 nw = make_float4(g.cand.x, g.cand.y, g.cand.z, g.ow);
            if (defer)
            {
                const uint32_t k = atomicAdd(def.count, 1u);
                def.v[slot_base + k] = g.v;
                def.oldp[slot_base + k] = make_float4(g.vo.p.x, g.vo.p.y, g.vo.p.z, g.ow);
                def.newp[slot_base + k] = nw;
            }
            else
                m.pos[g.v] = nw;
            n_evals += (unsigned int)g.evals;
            n_elems += (unsigned int)(g.evals * g.E);
            n_fp64 += defer ? 1u : 0u;
        }
        g.phase = kNMIdle;
    }
    nm_flush_counters(ctr, n_evals, n_elems, n_fp64, lane);
}

}  // namespace gm
