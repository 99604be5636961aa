// Kernel bodies shared by the plain (one launch per colour) and batched
// (persistent, work-queue) paths.
#pragma once

#include "gm_device.cuh"

namespace gm {

constexpr int kWarp = 32;
enum : int { kSmoothNM = 0, kSmoothGD = 1, kSmoothSpawn = 2, kSmoothGetme = 3, kSmoothSpring = 4, kSmoothQLaplace = 5 };
constexpr int kMaxCand = 64;  // spawn search evaluates 64 candidates at once

// evaluation output (QualityHistogram, DataStructures/QualityHistogram.h:72-75)
struct Quality
{
    double min;
    double inv_sum;  // +inf once any element has q <= 0
    unsigned long long count;
    unsigned long long nbad;
    unsigned long long buckets[20];
};

struct EvalPartial
{
    float min;
    int nbad;
    double rsum;
    int hist[20];
    int pad;
};

// Scratch of one evaluation launch of nb blocks, carved from EvalPartial
// slots: a ticket word (8 bytes), the 20 bucket totals every block adds to
// (80 bytes, padded to 88), then one 16-byte record per block (its Σ1/q as
// a double; its minimum's bits and its inverted count packed in the second
// word), which the last block reads with one 16-byte load per block --
// 96 + 16 nb bytes, which eval_scratch_slots(nb) slots hold (two for a
// single block).  The ticket and the totals are zero between launches: a
// fresh scratch is cleared once, and the last block of every launch resets
// them.
struct EvalScratch
{
    unsigned int* ticket;
    unsigned int* hist;  // hist[b], summed over the blocks
    double2* rec;        // rec[block] = (Σ1/q, min | nbad << 32)
};
constexpr size_t kEvalScratchHead = 96;  // ticket + bucket totals, cleared together
static_assert(sizeof(EvalPartial) >= kEvalScratchHead, "evaluation scratch layout");

// EvalPartial slots that hold the scratch of an evaluation launch of nb blocks
__host__ __device__ constexpr size_t eval_scratch_slots(size_t nb)
{
    return (kEvalScratchHead + 16 * nb + sizeof(EvalPartial) - 1) / sizeof(EvalPartial);
}

__host__ __device__ inline EvalScratch eval_scratch(EvalPartial* base, int)
{
    char* p = reinterpret_cast<char*>(base);
    EvalScratch s;
    s.ticket = reinterpret_cast<unsigned int*>(p);
    s.hist = reinterpret_cast<unsigned int*>(p + 8);
    s.rec = reinterpret_cast<double2*>(p + kEvalScratchHead);
    return s;
}

// First statement of every kernel that launch_pdl (gm_launch.h) launches:
// wait for the stream's previous kernel to complete and its memory to be
// visible before any global access, then let the stream's next kernel be
// scheduled as this one's blocks retire.  Launched without the programmatic
// attribute (inside a capture, or by another launcher) both return at once.
#define GM_PDL_ENTRY()                                                      \
    do                                                                      \
    {                                                                       \
        asm volatile("griddepcontrol.wait;" ::: "memory");                  \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");     \
    } while (0)

// Per-thread accumulation of evaluated elements (QualityHistogram::add,
// DataStructures/QualityHistogram.cpp:63-76).  The minimum over valid
// elements is the reciprocal of the maximum 1/q (a correctly rounded
// reciprocal is monotonic, so this equals the minimum of the elements'
// rounded qualities) and costs one division per thread, not per element;
// the bucket of a valid element uses a one-instruction reciprocal.  The
// minimum starts at 1, as the reference histogram's does; a non-positive
// quality goes to bucket 0.
struct EvalAcc
{
    float rs = 0.f;
    float rmax = 0.f;
    float bmin = 1.0f;
    int nbad = 0;
    // returns the element's bucket
    __device__ __forceinline__ int add(const EQ<float>& q)
    {
        float qv;
        if (q.pos)
        {
            rs += q.v;
            rmax = fmaxf(rmax, q.v);
            qv = rcp_fast(q.v);
        }
        else
        {
            ++nbad;
            bmin = fminf(bmin, q.v);
            qv = 0.f;
        }
        // floor(20 q) without a float-to-int conversion (a quarter-rate
        // instruction): 2^23 added with rounding toward zero leaves the
        // integer part of x < 2^23 in the low mantissa bits; x >= 2^23 and
        // infinity give more than 19, NaN gives bucket 0
        const float x = fmaxf(qv * 20.f, 0.f);
        return min(__float_as_int(__fadd_rz(x, 8388608.f)) - 0x4B000000, 19);
    }
    __device__ __forceinline__ float min_quality() const { return nbad ? bmin : fminf(1.0f, __frcp_rn(rmax)); }
};

// Add each lane's bucket b (-1: no element) to a shared histogram; lanes
// with the same bucket are counted by one atomic.  Every lane of the warp
// must call it.
__device__ __forceinline__ void hist_add_warp(int* hist, int b)
{
    const unsigned same = __match_any_sync(0xffffffffu, b);
    if (b >= 0 && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&hist[b], __popc(same));
}

// relocation parameters (the reference's file-scope constants, now runtime)
struct SmoothParams
{
    float shift;        // NM / GD: local size -> node shift; spawn: move coefficient
    int cycles;         // NM / GD security cycle count; spawn iterations
    float convergence;  // NM value convergence
    float alpha, beta, gamma;
    float lambda;       // GETMe
    float accept_q;     // patches below this quality are relocated / accepted in FP64
};

// vertices whose old or new patch quality is below the acceptance threshold,
// handed from the FP32 relocation kernel to the FP64 acceptance kernel
struct Deferred
{
    uint32_t* v;
    float4* oldp;
    float4* newp;
    uint32_t* count;
};

// per-launch counters for FLOP accounting
struct Counters
{
    unsigned long long patch_evals;
    unsigned long long elem_evals[4];  // by element type
    unsigned long long fp64_vertices;
};

// Position loads in the relocation kernels bypass L1 (__ldcg): inside the
// persistent batched kernel other SMs move vertices while this SM reads
// them, and L1 is not coherent across SMs.

// ---------------------------------------------------------------------------
// warp-level patch: the incident elements of one vertex staged in shared
// memory as [slot][element] float4 (conflict-free: lane e reads element e).
// Mixed patches stage the corner positions (8 slots); tet patches stage
// either the 4 corner positions or the 5-slot canonical form below.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int patch_slots(int maxk) { return maxk == 4 ? 5 : maxk; }
// canonical tet patches also keep the 5 slots with the elements of each pair
// (2j, 2j + 1) interleaved, for the paired FP32 evaluation (canonical_mc_pair)
__host__ __device__ constexpr int patch_pair_slots(int maxk) { return maxk == 4 ? 5 : 0; }
// element stride of the interleaved slots: maxe rounded up to a pair
__host__ __device__ constexpr int pair_stride(int maxe) { return (maxe + 1) & ~1; }
struct WarpPatch
{
    float4* sp;    // patch_slots(maxk) * maxe
    // patch_pair_slots(maxk) * pair_stride(maxe), or null: slot k of element
    // pair j is pp[k * pair_stride + 2j] = (x0, x1, y0, y1) and
    // pp[k * pair_stride + 2j + 1] = (z0, z1, w0, w1), elements 2j and 2j + 1
    // side by side, so one 16-byte load yields two ready operand pairs
    float4* pp;
    int* meta;     // maxe: type | local << 2
    float4* cand;  // kMaxCand candidate positions
    float* res;    // kMaxCand patch qualities
    int maxe;
    int E;
    V3<float> o;   // canonical tet staging: the origin (the vertex at staging)
};

// maxk: corners of the largest element type (4 tets only, 8 otherwise)
__device__ __forceinline__ size_t warp_patch_bytes(int maxk, int maxe)
{
    return (size_t)patch_slots(maxk) * maxe * sizeof(float4) +
           (size_t)patch_pair_slots(maxk) * pair_stride(maxe) * sizeof(float4) + (size_t)maxe * sizeof(int) +
           kMaxCand * sizeof(float4) + kMaxCand * sizeof(float);
}

__device__ __forceinline__ WarpPatch carve_patch(char* base, int maxk, int maxe)
{
    WarpPatch p;
    p.sp = reinterpret_cast<float4*>(base);
    base += (size_t)patch_slots(maxk) * maxe * sizeof(float4);
    p.pp = patch_pair_slots(maxk) ? reinterpret_cast<float4*>(base) : nullptr;
    base += (size_t)patch_pair_slots(maxk) * pair_stride(maxe) * sizeof(float4);
    p.cand = reinterpret_cast<float4*>(base);
    base += kMaxCand * sizeof(float4);
    p.res = reinterpret_cast<float*>(base);
    base += kMaxCand * sizeof(float);
    p.meta = reinterpret_cast<int*>(base);
    p.maxe = maxe;
    p.E = 0;
    p.o = V3<float>{0.f, 0.f, 0.f};
    return p;
}

__device__ __forceinline__ void stage_patch(const MeshView& m, uint32_t v, WarpPatch& P, int lane)
{
    uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
    P.E = (int)(e - b);
    for (int i = lane; i < P.E; i += kWarp)
    {
        uint32_t r = m.ve[GM_IX(m, b + i, m.ve_len, kBoundsNeighbourElem)];
        int type = ref_type(r), loc = ref_local(r);
        uint32_t vid[8];
        elem_vertices(m, type, ref_id(r), vid);
        int n = type_size(type);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < n) P.sp[k * P.maxe + i] = __ldcg(&m.pos[vid[k]]);
        P.meta[i] = (int)((uint32_t)type | ((uint32_t)loc << 2) | (ref_id(r) << 5));
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Canonical tet patches.  With the metric-free mean ratio, or metric
// conformity under a diagonal metric, on tets only, the FP32 searches stage
// each patch in a form where one more candidate position costs a few fused
// operations per element:
//  * each tet's corners are reordered by the even permutation
//    new j = old (j xor (3 xor local)), which puts the moving vertex last;
//    both measures are invariant under it (the regular-tet frame Fr_TET_INV
//    is symmetric under the rotations of the element, and an even
//    permutation keeps the orientation, i.e. the sign of det);
//  * positions are relative to the moving vertex's position at staging, o,
//    so the staged numbers are edge-sized;
//  * the frame is applied to the fixed corners once: for a candidate with
//    d = c - o, the corner-matrix columns [e03 e13 e23] Fr_TET_INV are
//    kj d - Qj with k = (1, 1/sqrt 3, 1/sqrt 6) and Qj staged per element
//    (slots 0-2, xyz);
//  * under the sine-graded metric s^2 diag(1 + 9 sin^2(4 pi x), 1, 1) the
//    Keast point k has x_k = X_k + w_k c.x with X_k fixed and w_k = 1/4
//    (centroid), 1/6 (points weighting a fixed corner) or 1/2 (the point
//    weighting the moving corner).  sin and cos of 4 pi X_k are staged
//    (slots 0-2 w, 3, 4), so sin(4 pi x_k) follows by angle addition from the
//    three per-candidate values sincospi(4 w c.x).
// ---------------------------------------------------------------------------
template <int VAR, int MAXK>
struct TetCanon
{
    static constexpr bool on = MAXK == 4 && (VAR == kVarMRFree || VAR == kVarMCDiag);
};

// Fr_TET_INV (AbstractEvaluator.cpp:28-31) and the column sums k1, k2
constexpr float kFrA = -0.5773502691896257645091f, kFrB = 1.154700538379251529018f;
constexpr float kFrD = -0.4082482904638630163662f, kFrG = 1.224744871391589049099f;
constexpr float kK1 = 0.5773502691896257645091f;  // kFrA + kFrB
constexpr float kK2 = 0.4082482904638630163662f;  // 2 kFrD + kFrG
// Keast 5-point rule (MetricConformityEvaluator.cpp:38-44)
constexpr float kKeastH = 0.5f, kKeastQ = (1.0f - 0.5f) / 3.0f;

__device__ __forceinline__ uint32_t tet_corner(uint4 t, int k)
{
    return k == 0 ? t.x : k == 1 ? t.y : k == 2 ? t.z : t.w;
}

__device__ __forceinline__ bool sine_metric(const Crew& c) { return c.sampler == kSamplerSine; }

// element i of a canonical patch from its fixed corners a0, a1, a2 (in
// canonical order) and the origin o
template <int VAR>
__device__ __forceinline__ void stage_canonical_element(WarpPatch& P, int i, float4 a0, float4 a1, float4 a2,
                                                        V3<float> o, bool sine)
{
    const V3<float> r0 = to<float>(a0) - o, r1 = to<float>(a1) - o, r2 = to<float>(a2) - o;
    const V3<float> q1 = r0 * kFrA + r1 * kFrB, q2 = (r0 + r1) * kFrD + r2 * kFrG;
    float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, c[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (VAR == kVarMCDiag && sine)
    {
        const float sum = a0.x + a1.x + a2.x;
        const float X[5] = {sum * 0.25f, a0.x * kKeastH + (a1.x + a2.x) * kKeastQ,
                            a1.x * kKeastH + (a0.x + a2.x) * kKeastQ, a2.x * kKeastH + (a0.x + a1.x) * kKeastQ,
                            sum * kKeastQ};
#pragma unroll
        for (int k = 0; k < 5; ++k) sincospif(4.f * X[k], &s[k], &c[k]);
    }
    const float4 v[5] = {make_float4(r0.x, r0.y, r0.z, s[0]), make_float4(q1.x, q1.y, q1.z, c[0]),
                         make_float4(q2.x, q2.y, q2.z, s[1]), make_float4(c[1], s[2], c[2], s[3]),
                         make_float4(c[3], s[4], c[4], 0.f)};
    constexpr int nslot = VAR == kVarMCDiag ? 5 : 3;
#pragma unroll
    for (int k = 0; k < nslot; ++k) P.sp[k * P.maxe + i] = v[k];
    if (VAR == kVarMCDiag && P.pp)
    {
        // the interleaved copy: this element's half of its pair's two float4
        const int h = i & 1, ps = pair_stride(P.maxe);
#pragma unroll
        for (int k = 0; k < 5; ++k)
        {
            float* f = reinterpret_cast<float*>(P.pp + k * ps + (i & ~1));
            f[h] = v[k].x;
            f[2 + h] = v[k].y;
            f[4 + h] = v[k].z;
            f[6 + h] = v[k].w;
        }
    }
}

// stage elements first, first + stride, ... of v's patch in canonical form
template <int VAR>
__device__ __forceinline__ void stage_canonical_range(const MeshView& m, const Crew& crew, uint32_t v, V3<float> o,
                                                      WarpPatch& P, int first, int stride)
{
    const uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
    P.E = (int)(e - b);
    P.o = o;
    const bool sine = VAR == kVarMCDiag && sine_metric(crew);
    for (int i = first; i < P.E; i += stride)
    {
        const uint32_t r = m.ve[GM_IX(m, b + i, m.ve_len, kBoundsNeighbourElem)];
        const int x = 3 ^ ref_local(r);
        const uint4 t = m.tets[GM_IX(m, ref_id(r), m.nt, kBoundsTet)];
        const float4 a0 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, x), m.nv, kBoundsPosition)]);
        const float4 a1 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, 1 ^ x), m.nv, kBoundsPosition)]);
        const float4 a2 = __ldcg(&m.pos[GM_IX(m, tet_corner(t, 2 ^ x), m.nv, kBoundsPosition)]);
        stage_canonical_element<VAR>(P, i, a0, a1, a2, o, sine);
    }
}

template <int VAR>
__device__ __forceinline__ void stage_patch_canonical(const MeshView& m, const Crew& crew, uint32_t v, V3<float> o,
                                                      WarpPatch& P, int lane)
{
    stage_canonical_range<VAR>(m, crew, v, o, P, lane, kWarp);
    __syncwarp();
}

// per-candidate part of a canonical element evaluation
struct TetCand
{
    V3<float> k0, k1, k2;
    float sa, ca, sq, cq, sh, ch;  // sincospi(4 w c.x) for w = 1/4, 1/6, 1/2
};

// per-crew constants of the diagonal metric: the y and z entries of the
// specified metric (constant for both diagonal samplers) and their inverses
struct TetConst
{
    float s2, my, mz, iy, iz;
    // the sine metric's x entry at a Keast point is s2 (1 + 9 s^2); the
    // paired evaluation folds the quadrature weight into it: w s2 and 9 w s2
    // for w = 0.45 (points 1-4) and w = -0.8 (the centroid)
    float q1, q9, c1, c9;
};

template <int VAR>
__device__ __forceinline__ TetConst tet_const(const Crew& crew)
{
    TetConst k{};
    if (VAR == kVarMCDiag)
    {
        // specified_metric_diag with metric_diag_at = {., s2, s2}, same operation order
        const float s2 = (float)crew.scaling2;
        k.s2 = s2;
        k.my = s2 * -0.8f + (s2 + s2 + s2 + s2) * 0.45f;
        k.mz = k.my;
        k.iy = rcp_fast(k.my);
        k.iz = k.iy;
        k.q1 = 0.45f * s2;
        k.q9 = 9.f * k.q1;
        k.c1 = -0.8f * s2;
        k.c9 = 9.f * k.c1;
    }
    return k;
}

// sine: the crew's sampler is the sine-graded one (metric conformity only)
template <int VAR>
__device__ __forceinline__ TetCand tet_cand(bool sine, V3<float> o, V3<float> c)
{
    TetCand t;
    const V3<float> d = c - o;
    t.k0 = d;
    t.k1 = d * kK1;
    t.k2 = d * kK2;
    t.sa = t.ca = t.sq = t.cq = t.sh = t.ch = 0.f;
    if (VAR == kVarMCDiag && sine)
    {
        sincospif(c.x, &t.sa, &t.ca);                  // 4 * (1/4) * c.x
        sincospif(c.x * (2.0f / 3.0f), &t.sq, &t.cq);  // 4 * (1/6) * c.x
        sincospif(c.x * 2.0f, &t.sh, &t.ch);           // 4 * (1/2) * c.x
    }
    return t;
}

// MetricConformityEvaluator::metricConformity with Ms = diag(m), from the
// rows R_i of the corner matrix F: the cofactor rows C_i (C0 = R1 x R2, ...)
// give det F = R0 . C0 and Mk = F^-T F^-1 = (C_i . C_j) / det^2, and
// F F^T = (R_i . R_j); tNc_ij = (F F^T)_ij m_j + Mk_ij / m_i - 2 delta_ij.
__device__ __forceinline__ void mc_corner_diag_fast(V3<float> c0, V3<float> c1, V3<float> c2, V3<float> m,
                                                    const TetConst& k, float& rq, float& q, bool& pos)
{
    const V3<float> R0 = mk(c0.x, c1.x, c2.x), R1 = mk(c0.y, c1.y, c2.y), R2 = mk(c0.z, c1.z, c2.z);
    const V3<float> C0 = cross(R1, R2), C1 = cross(R2, R0), C2 = cross(R0, R1);
    const float det = dot(R0, C0);
    const float Axx = dot(R0, R0), Ayy = dot(R1, R1), Azz = dot(R2, R2);
    const float Axy = dot(R0, R1), Axz = dot(R0, R2), Ayz = dot(R1, R2);
    const float Nxx = dot(C0, C0), Nyy = dot(C1, C1), Nzz = dot(C2, C2);
    const float Nxy = dot(C0, C1), Nxz = dot(C0, C2), Nyz = dot(C1, C2);
    const float id2 = rcp_fast(det * det);
    const float wx = id2 * rcp_fast(m.x), wy = id2 * k.iy, wz = id2 * k.iz;
    const float txx = Axx * m.x + Nxx * wx - 2.f, tyy = Ayy * m.y + Nyy * wy - 2.f, tzz = Azz * m.z + Nzz * wz - 2.f;
    const float txy = Axy * m.y + Nxy * wx, tyx = Axy * m.x + Nxy * wy;
    const float txz = Axz * m.z + Nxz * wx, tzx = Axz * m.x + Nxz * wz;
    const float tyz = Ayz * m.z + Nyz * wy, tzy = Ayz * m.y + Nyz * wz;
    const float f2 = txx * txx + tyy * tyy + tzz * tzz + txy * txy + tyx * tyx + txz * txz + tzx * tzx +
                     tyz * tyz + tzy * tzy;
    if (isnan(f2))
    {
        pos = false;
        q = 0.f;
        return;
    }
    const float sg = sgn(det);
    pos = sg > 0.f;
    const float r = sqrt_fast(1.f + sqrt_fast(f2));
    if (pos) rq = r;
    else q = sg * rcp_fast(r);
}

// quality of canonical element e for candidate t
template <int VAR>
__device__ __forceinline__ EQ<float> canonical_quality(const WarpPatch& P, int e, const TetCand& t, const TetConst& k,
                                                       bool sine)
{
    const float4 A = P.sp[e], B = P.sp[P.maxe + e], C = P.sp[2 * P.maxe + e];
    const V3<float> c0 = t.k0 - mk(A.x, A.y, A.z), c1 = t.k1 - mk(B.x, B.y, B.z), c2 = t.k2 - mk(C.x, C.y, C.z);
    float rq = 0.f, q = 0.f;
    bool pos;
    if (VAR == kVarMRFree)
        mr_corner(c0, c1, c2, rq, q, pos);
    else
    {
        V3<float> m = mk(k.my, k.my, k.mz);
        if (sine)
        {
            const float4 D = P.sp[3 * P.maxe + e], F = P.sp[4 * P.maxe + e];
            // sin(4 pi x_k) at the 5 Keast points; staged S0 C0 S1 C1 S2 C2 S3 C3 S4 C4
            const float s0 = A.w * t.ca + B.w * t.sa;
            const float s1 = C.w * t.cq + D.x * t.sq;
            const float s2 = D.y * t.cq + D.z * t.sq;
            const float s3 = D.w * t.cq + F.x * t.sq;
            const float s4 = F.y * t.ch + F.z * t.sh;
            const float m0 = k.s2 * (1.f + 9.f * s0 * s0), m1 = k.s2 * (1.f + 9.f * s1 * s1);
            const float m2 = k.s2 * (1.f + 9.f * s2 * s2), m3 = k.s2 * (1.f + 9.f * s3 * s3);
            const float m4 = k.s2 * (1.f + 9.f * s4 * s4);
            m.x = m0 * -0.8f + (m1 + m2 + m3 + m4) * 0.45f;
        }
        else
            m.x = k.my;  // uniform: every entry is s2 (-0.8 + 4 * 0.45)
        mc_corner_diag_fast(c0, c1, c2, m, k, rq, q, pos);
    }
    return EQ<float>{pos ? rq : q, pos};
}

// ---------------------------------------------------------------------------
// Two canonical elements of one candidate at once, in Blackwell's paired FP32
// operations (add / mul / fma .f32x2: one instruction, two lanes of IEEE
// arithmetic).  The scalar evaluation above is issue bound with its FMA pipe
// partly idle, so evaluating elements e0 and e1 of a patch in the two halves
// of every operation halves the instructions of the element algebra; the
// per-element transcendentals (reciprocals, square roots) stay scalar.  Each
// half computes the quantities of mc_corner_diag_fast in a fixed contraction
// (explicit fma), with the quadrature weights folded into the metric
// constants and the equal y / z metric entries used (tNc_yz = tNc_zy), so its
// result is an FP32 evaluation of the same formula.
// ---------------------------------------------------------------------------
struct Pair3
{
    float2 x, y, z;
};
__device__ __forceinline__ float2 pdup(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pneg(float2 a) { return make_float2(-a.x, -a.y); }
// a - b, exact (the product b * -1 is exact)
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, pdup(-1.f), a); }
__device__ __forceinline__ float2 pdot(const Pair3& a, const Pair3& b)
{
    return pfma(a.z, b.z, pfma(a.y, b.y, pmul(a.x, b.x)));
}
__device__ __forceinline__ Pair3 pcross(const Pair3& a, const Pair3& b)
{
    return {pfma(a.y, b.z, pneg(pmul(b.y, a.z))), pfma(a.z, b.x, pneg(pmul(b.z, a.x))),
            pfma(a.x, b.y, pneg(pmul(b.x, a.y)))};
}

// one half's element result from its determinant and |tNc|^2
__device__ __forceinline__ EQ<float> pair_corner_result(float det, float f2)
{
    if (isnan(f2)) return EQ<float>{0.f, false};
    const float r = sqrt_fast(1.f + sqrt_fast(f2));
    if (det > 0.f) return EQ<float>{r, true};
    return EQ<float>{det < 0.f ? -rcp_fast(r) : 0.f, false};
}

// metric conformity under a diagonal metric, canonical elements 2j and 2j + 1
// from the interleaved slots (element 2j + 1 may be a padding slot whose
// result the caller drops)
__device__ __forceinline__ void canonical_mc_pair(const WarpPatch& P, int j, const TetCand& t, const TetConst& k,
                                                  bool sine, EQ<float>& q0, EQ<float>& q1)
{
    const int ps = pair_stride(P.maxe);
    const float4* pp = P.pp + 2 * j;
    // slot s: lo = (x0, x1, y0, y1), hi = (z0, z1, w0, w1)
    const float4 Alo = pp[0], Ahi = pp[1], Blo = pp[ps], Bhi = pp[ps + 1], Clo = pp[2 * ps], Chi = pp[2 * ps + 1];
    // corner-matrix columns c_j = k_j (c - o) - Q_j, as rows R_i = (c0_i, c1_i, c2_i)
    const Pair3 R0 = {psub(pdup(t.k0.x), make_float2(Alo.x, Alo.y)), psub(pdup(t.k1.x), make_float2(Blo.x, Blo.y)),
                      psub(pdup(t.k2.x), make_float2(Clo.x, Clo.y))};
    const Pair3 R1 = {psub(pdup(t.k0.y), make_float2(Alo.z, Alo.w)), psub(pdup(t.k1.y), make_float2(Blo.z, Blo.w)),
                      psub(pdup(t.k2.y), make_float2(Clo.z, Clo.w))};
    const Pair3 R2 = {psub(pdup(t.k0.z), make_float2(Ahi.x, Ahi.y)), psub(pdup(t.k1.z), make_float2(Bhi.x, Bhi.y)),
                      psub(pdup(t.k2.z), make_float2(Chi.x, Chi.y))};
    float2 mxx = pdup(k.my);
    if (sine)
    {
        const float4 Dlo = pp[3 * ps], Dhi = pp[3 * ps + 1], Flo = pp[4 * ps], Fhi = pp[4 * ps + 1];
        // sin(4 pi x) at the 5 Keast points by angle addition
        const float2 s0 = pfma(make_float2(Ahi.z, Ahi.w), pdup(t.ca), pmul(make_float2(Bhi.z, Bhi.w), pdup(t.sa)));
        const float2 s1 = pfma(make_float2(Chi.z, Chi.w), pdup(t.cq), pmul(make_float2(Dlo.x, Dlo.y), pdup(t.sq)));
        const float2 s2 = pfma(make_float2(Dlo.z, Dlo.w), pdup(t.cq), pmul(make_float2(Dhi.x, Dhi.y), pdup(t.sq)));
        const float2 s3 = pfma(make_float2(Dhi.z, Dhi.w), pdup(t.cq), pmul(make_float2(Flo.x, Flo.y), pdup(t.sq)));
        const float2 s4 = pfma(make_float2(Flo.z, Flo.w), pdup(t.ch), pmul(make_float2(Fhi.x, Fhi.y), pdup(t.sh)));
        // the quadrature sum -0.8 m0 + 0.45 (m1 + m2 + m3 + m4), each weighted
        // metric value one multiply and one fused multiply-add
        const float2 q1 = pdup(k.q1), q9 = pdup(k.q9);
        const float2 m0 = pfma(s0, pmul(s0, pdup(k.c9)), pdup(k.c1));
        const float2 m1 = pfma(s1, pmul(s1, q9), q1), m2 = pfma(s2, pmul(s2, q9), q1);
        const float2 m3 = pfma(s3, pmul(s3, q9), q1), m4 = pfma(s4, pmul(s4, q9), q1);
        mxx = padd(padd(padd(padd(m0, m1), m2), m3), m4);
    }
    // cofactor rows, det, F F^T and the cofactor products (mc_corner_diag_fast)
    const Pair3 N0 = pcross(R1, R2), N1 = pcross(R2, R0), N2 = pcross(R0, R1);
    const float2 det = pdot(R0, N0);
    const float2 Axx = pdot(R0, R0), Ayy = pdot(R1, R1), Azz = pdot(R2, R2);
    const float2 Axy = pdot(R0, R1), Axz = pdot(R0, R2), Ayz = pdot(R1, R2);
    const float2 Nxx = pdot(N0, N0), Nyy = pdot(N1, N1), Nzz = pdot(N2, N2);
    const float2 Nxy = pdot(N0, N1), Nxz = pdot(N0, N2), Nyz = pdot(N1, N2);
    const float2 d2 = pmul(det, det);
    const float2 id2 = make_float2(rcp_fast(d2.x), rcp_fast(d2.y));
    const float2 wx = pmul(id2, make_float2(rcp_fast(mxx.x), rcp_fast(mxx.y)));
    // the diagonal metrics here have equal y and z entries (my = mz, so
    // wy = wz), which makes tNc_yz = tNc_zy
    const float2 wy = pmul(id2, pdup(k.iy));
    const float2 my = pdup(k.my), two = pdup(-2.f);
    const float2 txx = pfma(Nxx, wx, pfma(Axx, mxx, two));
    const float2 tyy = pfma(Nyy, wy, pfma(Ayy, my, two));
    const float2 tzz = pfma(Nzz, wy, pfma(Azz, my, two));
    const float2 txy = pfma(Nxy, wx, pmul(Axy, my)), tyx = pfma(Nxy, wy, pmul(Axy, mxx));
    const float2 txz = pfma(Nxz, wx, pmul(Axz, my)), tzx = pfma(Nxz, wy, pmul(Axz, mxx));
    const float2 tyz = pfma(Nyz, wy, pmul(Ayz, my));
    float2 f2 = pmul(txx, txx);
    f2 = pfma(tyy, tyy, f2);
    f2 = pfma(tzz, tzz, f2);
    f2 = pfma(txy, txy, f2);
    f2 = pfma(tyx, tyx, f2);
    f2 = pfma(txz, txz, f2);
    f2 = pfma(tzx, tzx, f2);
    f2 = pfma(padd(tyz, tyz), tyz, f2);
    q0 = pair_corner_result(det.x, f2.x);
    q1 = pair_corner_result(det.y, f2.y);
}

// the staging the FP32 patch functions of this variant expect; o is the
// moving vertex's current position
template <int VAR, int MAXK>
__device__ __forceinline__ void stage_patch_fp32(const MeshView& m, const Crew& crew, uint32_t v, V3<float> o,
                                                 WarpPatch& P, int lane)
{
    if constexpr (TetCanon<VAR, MAXK>::on) stage_patch_canonical<VAR>(m, crew, v, o, P, lane);
    else stage_patch(m, v, P, lane);
}

// quality of staged element e with its moving vertex at c
template <int VAR, int MAXK, class R>
__device__ __forceinline__ EQ<R> staged_quality(const Crew& crew, const WarpPatch& P, int e, V3<R> c)
{
    const uint32_t meta = (uint32_t)P.meta[e];
    int type = MAXK == 4 ? kTet : (int)(meta & 3u);
    int loc = (int)((meta >> 2) & 7u);
    V3<R> p[MAXK];
    int n = MAXK == 4 ? 4 : type_size(type);
#pragma unroll
    for (int k = 0; k < MAXK; ++k)
    {
        if (k < n) p[k] = (k == loc) ? c : to<R>(P.sp[k * P.maxe + e]);
        else p[k] = c;
    }
    return elem_quality<VAR, MAXK, R>(crew, type, p, elem_hint(type, meta >> 5));
}

// patch quality semantics of AbstractEvaluator::accumulatePatchQuality /
// finalizePatchQuality (Evaluators/AbstractEvaluator.cpp:778-803): harmonic
// mean when every element is valid, else the minimum element quality
template <class R>
struct PatchAcc
{
    R rsum;
    R minq;
    int nbad;
};

template <class R>
__device__ __forceinline__ void acc_add(PatchAcc<R>& a, EQ<R> q)
{
    if (q.pos) a.rsum += q.v;
    else
    {
        a.nbad += 1;
        a.minq = q.v < a.minq ? q.v : a.minq;
    }
}

template <class R>
__device__ __forceinline__ R shfl_xor(R v, int o)
{
    return __shfl_xor_sync(0xffffffffu, v, o);
}

// reduce within aligned segments of S lanes (S a power of two); when no
// lane saw a non-positive element (the common case) only the 1/q sums move
template <class R>
__device__ __forceinline__ void acc_reduce(PatchAcc<R>& a, int S)
{
    if (!__any_sync(0xffffffffu, a.nbad))
    {
        for (int o = S >> 1; o > 0; o >>= 1) a.rsum += shfl_xor(a.rsum, o);
        return;
    }
    for (int o = S >> 1; o > 0; o >>= 1)
    {
        a.rsum += shfl_xor(a.rsum, o);
        R mq = shfl_xor(a.minq, o);
        a.minq = mq < a.minq ? mq : a.minq;
        a.nbad += __shfl_xor_sync(0xffffffffu, a.nbad, o);
    }
}

template <class R>
__device__ __forceinline__ R acc_final(const PatchAcc<R>& a, int E)
{
    if (a.nbad > 0) return a.minq;
    if (E == 0) return R(0);
    return R(E) / a.rsum;
}

// patch quality with the vertex at c (same c on every lane), whole warp
// (FP32 with a canonical variant: the patch must be staged canonically;
// FP64 and every other variant: the corner positions)
template <int VAR, int MAXK, class R>
__device__ __forceinline__ R patch_uniform(const Crew& crew, const WarpPatch& P, V3<R> c, int lane)
{
    PatchAcc<R> a{R(0), R(3.0e38), 0};
    if constexpr (TetCanon<VAR, MAXK>::on && sizeof(R) == sizeof(float))
    {
        const TetConst k = tet_const<VAR>(crew);
        const bool sine = VAR == kVarMCDiag && sine_metric(crew);
        const TetCand t = tet_cand<VAR>(sine, P.o, c);
        for (int e = lane; e < P.E; e += kWarp) acc_add(a, canonical_quality<VAR>(P, e, t, k, sine));
    }
    else
    {
        for (int e = lane; e < P.E; e += kWarp) acc_add(a, staged_quality<VAR, MAXK, R>(crew, P, e, c));
    }
    acc_reduce(a, kWarp);
    return acc_final(a, P.E);
}

// patch quality of K candidates held in P.cand; results land in P.res
template <int VAR, int MAXK, class R>
__device__ __forceinline__ void patch_multi(const Crew& crew, WarpPatch& P, int K, int lane)
{
    int S = 32;
    while (S > 1 && K * S > 32) S >>= 1;
    int G = 32 / S;
    int slot = lane / S, sub = lane & (S - 1);
    const TetConst k = tet_const<VAR>(crew);
    const bool sine = VAR == kVarMCDiag && sine_metric(crew);
    for (int r = 0; r < K; r += G)
    {
        int c = r + slot;
        PatchAcc<R> a{R(0), R(3.0e38), 0};
        if (c < K)
        {
            float4 cf = P.cand[c];
            V3<R> cp = to<R>(cf);
            if constexpr (VAR == kVarMCDiag && TetCanon<VAR, MAXK>::on && sizeof(R) == sizeof(float))
            {
                // element pairs (2j, 2j + 1) in paired FP32 operations
                const TetCand t = tet_cand<VAR>(sine, P.o, cp);
                for (int j = sub; 2 * j < P.E; j += S)
                {
                    EQ<float> q0, q1;
                    canonical_mc_pair(P, j, t, k, sine, q0, q1);
                    acc_add(a, q0);
                    if (2 * j + 1 < P.E) acc_add(a, q1);
                }
            }
            else if constexpr (TetCanon<VAR, MAXK>::on && sizeof(R) == sizeof(float))
            {
                const TetCand t = tet_cand<VAR>(sine, P.o, cp);
                for (int e = sub; e < P.E; e += S) acc_add(a, canonical_quality<VAR>(P, e, t, k, sine));
            }
            else
            {
                for (int e = sub; e < P.E; e += S) acc_add(a, staged_quality<VAR, MAXK, R>(crew, P, e, cp));
            }
        }
        acc_reduce(a, S);
        if (c < K && sub == 0) P.res[c] = (float)acc_final(a, P.E);
    }
    __syncwarp();
}

// Patch quality in FP64 straight from the mesh, without staging: lanes over
// the incident elements and the per-element arithmetic of patch_uniform, so
// it equals patch_uniform<VAR, MAXK, double> on a patch staged from the same
// positions.  For the rare FP64 acceptance test of a vertex whose patch is
// staged in a form the FP64 measures do not read.
template <int VAR, int MAXK>
__device__ double patch_quality_global(const MeshView& m, const Crew& crew, uint32_t v, V3<double> c, int lane)
{
    const uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
    const int E = (int)(e - b);
    PatchAcc<double> a{0.0, 3.0e38, 0};
    for (int i = lane; i < E; i += kWarp)
    {
        const uint32_t r = m.ve[GM_IX(m, b + i, m.ve_len, kBoundsNeighbourElem)];
        const int type = MAXK == 4 ? kTet : ref_type(r), loc = ref_local(r);
        uint32_t vid[8];
        elem_vertices(m, type, ref_id(r), vid);
        const int n = MAXK == 4 ? 4 : type_size(type);
        V3<double> p[MAXK];
#pragma unroll
        for (int k = 0; k < MAXK; ++k)
        {
            if (k < n) p[k] = (k == loc) ? c : to<double>(__ldcg(&m.pos[vid[k]]));
            else p[k] = c;
        }
        acc_add(a, elem_quality<VAR, MAXK, double>(crew, type, p, elem_hint(type, ref_id(r))));
    }
    acc_reduce(a, kWarp);
    return acc_final(a, E);
}

template <class R>
__device__ __forceinline__ V3<R> snap(const MeshView& m, int cid, V3<R> p)
{
    return project<R>(m.con, m.ncon, cid, p);
}

// AbstractMeasurer::computeLocalElementSize (Measurers/AbstractMeasurer.cpp:137-155)
template <class R>
__device__ __forceinline__ R local_size(const MeshView& m, uint32_t v, V3<R> pos, int lane)
{
    uint32_t b = m.vv_off[v], e = m.vv_off[v + 1];
    R s = 0;
    for (uint32_t i = b + lane; i < e; i += kWarp)
    {
        const uint32_t w = m.vv[GM_IX(m, i, m.vv_len, kBoundsNeighbourVert)];
        s += length(to<R>(__ldcg(&m.pos[GM_IX(m, w, m.nv, kBoundsPosition)])) - pos);
    }
    for (int o = 16; o > 0; o >>= 1) s += shfl_xor(s, o);
    return s / R(e - b);
}

// ---------------------------------------------------------------------------
// Nelder-Mead (Smoothers/VertexWise/NelderMeadSmoother.cpp:100-260), one warp
// ---------------------------------------------------------------------------
struct S4
{
    V3<float> p;
    float w;
};
__device__ __forceinline__ void swp(S4& a, S4& b)
{
    S4 t = a;
    a = b;
    b = t;
}

template <int VAR, int MAXK>
__device__ V3<float> nelder_mead(const MeshView& m, const Crew& crew, const SmoothParams& sp, WarpPatch& P,
                                 uint32_t v, int cid, V3<float> pos, float q0, int lane, int& evals)
{
    const bool constrained = cid != 0;
    const float nodeShift = local_size<float>(m, v, pos, lane) * sp.shift;
    const S4 vo{pos, q0};
    S4 s[4] = {{pos + mk(nodeShift, 0.f, 0.f), 0.f}, {pos + mk(0.f, nodeShift, 0.f), 0.f},
               {pos + mk(0.f, 0.f, nodeShift), 0.f}, vo};
    int cycle = 0;
    bool reset = false, terminated = false;
    while (!terminated)
    {
        for (int p = 0; p < 3; ++p)
        {
            V3<float> x = s[p].p;
            if (constrained) x = snap(m, cid, x);
            ++evals;
            s[p] = S4{x, patch_uniform<VAR, MAXK, float>(crew, P, x, lane)};
        }
        if (s[0].w > s[1].w) swp(s[0], s[1]);
        if (s[1].w > s[2].w) swp(s[1], s[2]);
        if (s[2].w > s[3].w) swp(s[2], s[3]);
        if (s[0].w > s[1].w) swp(s[0], s[1]);
        if (s[1].w > s[2].w) swp(s[1], s[2]);
        if (s[0].w > s[1].w) swp(s[0], s[1]);

        for (; cycle < sp.cycles; ++cycle)
        {
            V3<float> c = (s[1].p + s[2].p + s[3].p) * (1.f / 3.f);
            V3<float> x = c + (c - s[0].p) * sp.alpha;
            if (constrained) x = snap(m, cid, x);
            ++evals;
            const float fr = patch_uniform<VAR, MAXK, float>(crew, P, x, lane);
            float f = fr;
            const V3<float> xr = x;
            bool probe = true;
            if (s[3].w < fr) x = c + (x - c) * sp.gamma;                      // expand
            else if (s[1].w >= fr) x = c + ((fr > s[0].w ? xr : s[0].p) - c) * sp.beta;  // contract
            else probe = false;                                                // accept reflection
            if (probe)
            {
                if (constrained) x = snap(m, cid, x);
                ++evals;
                f = patch_uniform<VAR, MAXK, float>(crew, P, x, lane);
                if (s[3].w < fr && f <= fr)
                {
                    x = xr;
                    f = fr;
                }
            }
            S4 vx{x, f};
            if (vx.w > s[3].w) swp(s[3], vx);
            if (vx.w > s[2].w) swp(s[2], vx);
            if (vx.w > s[1].w) swp(s[1], vx);
            if (vx.w > s[0].w) swp(s[0], vx);
            if ((s[3].w - s[1].w) < sp.convergence)
            {
                terminated = true;
                break;
            }
        }
        if (terminated || (cycle >= sp.cycles && reset)) break;
        s[0] = S4{vo.p - mk(nodeShift, 0.f, 0.f), vo.w};
        s[1] = S4{vo.p - mk(0.f, nodeShift, 0.f), vo.w};
        s[2] = S4{vo.p - mk(0.f, 0.f, nodeShift), vo.w};
        s[3] = vo;
        reset = true;
        cycle = 0;
    }
    V3<float> out = s[3].p;
    if (constrained) out = snap(m, cid, out);
    return out;
}

// ---------------------------------------------------------------------------
// Gradient descent (Smoothers/VertexWise/GradientDescentSmoother.cpp:73-202)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gd_offset(int i)
{
    // -0.25, 0, 0.1, 0.2, 0.4, 0.8, 1.2, 1.6
    return i == 0 ? -0.25f : i == 1 ? 0.f : i == 2 ? 0.1f : i == 3 ? 0.2f : i == 4 ? 0.4f : i == 5 ? 0.8f
           : i == 6 ? 1.2f : 1.6f;
}

template <int VAR, int MAXK>
__device__ V3<float> gradient_descent(const MeshView& m, const Crew& crew, const SmoothParams& sp, WarpPatch& P,
                                      uint32_t v, int cid, V3<float> pos, int lane, int& evals)
{
    const bool constrained = cid != 0;
    float nodeShift = local_size<float>(m, v, pos, lane) * sp.shift;
    const float original = nodeShift;
    for (int c = 0; c < sp.cycles; ++c)
    {
        if (lane < 6)
        {
            int axis = lane >> 1;
            float d = (lane & 1) ? nodeShift : -nodeShift;
            V3<float> g = pos + mk(axis == 0 ? d : 0.f, axis == 1 ? d : 0.f, axis == 2 ? d : 0.f);
            if (constrained) g = snap(m, cid, g);
            P.cand[lane] = make_float4(g.x, g.y, g.z, 0.f);
        }
        __syncwarp();
        patch_multi<VAR, MAXK, float>(crew, P, 6, lane);
        evals += 6;
        V3<float> gradQ = mk(P.res[1] - P.res[0], P.res[3] - P.res[2], P.res[5] - P.res[4]);
        float gn = length(gradQ);
        __syncwarp();
        if (gn == 0.f) break;
        V3<float> shift = gradQ * (nodeShift / gn);
        V3<float> mine = pos;
        if (lane < 8)
        {
            V3<float> x = pos + shift * gd_offset(lane);
            if (constrained) x = snap(m, cid, x);
            P.cand[lane] = make_float4(x.x, x.y, x.z, 0.f);
            mine = x;
        }
        __syncwarp();
        patch_multi<VAR, MAXK, float>(crew, P, 8, lane);
        evals += 8;
        int best = 0;
        float bestQ = -3.0e38f;
        for (int p = 0; p < 8; ++p)
        {
            float q = P.res[p];
            if (q > bestQ)
            {
                bestQ = q;
                best = p;
            }
        }
        pos.x = __shfl_sync(0xffffffffu, mine.x, best);
        pos.y = __shfl_sync(0xffffffffu, mine.y, best);
        pos.z = __shfl_sync(0xffffffffu, mine.z, best);
        nodeShift *= fabsf(gd_offset(best));
        __syncwarp();
        if (nodeShift < original / 10.f) break;
    }
    return pos;
}

// ---------------------------------------------------------------------------
// Spawn search (Smoothers/VertexWise/SpawnSearchSmoother.cpp:161-226)
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3<float> spawn_offset(int p)
{
    // 4x4x4 lattice minus 1.5, offset 0 replaced by the origin
    if (p == 0) return mk(0.f, 0.f, 0.f);
    return mk((float)(p & 3) - 1.5f, (float)((p >> 2) & 3) - 1.5f, (float)(p >> 4) - 1.5f);
}

template <int VAR, int MAXK>
__device__ V3<float> spawn_search(const MeshView& m, const Crew& crew, const SmoothParams& sp, WarpPatch& P,
                                  uint32_t v, int cid, V3<float> pos, int lane, int& evals)
{
    const bool constrained = cid != 0;
    float scale = local_size<float>(m, v, pos, lane) * sp.shift;
    for (int it = 0; it < sp.cycles; ++it)
    {
        V3<float> mine[2];
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            int p = lane + 32 * h;
            V3<float> x = pos + spawn_offset(p) * scale;
            if (constrained) x = snap(m, cid, x);
            mine[h] = x;
            P.cand[p] = make_float4(x.x, x.y, x.z, 0.f);
        }
        __syncwarp();
        patch_multi<VAR, MAXK, float>(crew, P, 64, lane);
        evals += 64;
        // argmax; the first maximum wins, as in the reference's strict '>' scan
        float bestQ = P.res[lane];
        int best = lane;
        float q1 = P.res[lane + 32];
        if (q1 > bestQ)
        {
            bestQ = q1;
            best = lane + 32;
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            float oq = __shfl_xor_sync(0xffffffffu, bestQ, o);
            int ob = __shfl_xor_sync(0xffffffffu, best, o);
            if (oq > bestQ || (oq == bestQ && ob < best))
            {
                bestQ = oq;
                best = ob;
            }
        }
        V3<float> sel = (best >> 5) ? mine[1] : mine[0];
        int src = best & 31;
        pos.x = __shfl_sync(0xffffffffu, sel.x, src);
        pos.y = __shfl_sync(0xffffffffu, sel.y, src);
        pos.z = __shfl_sync(0xffffffffu, sel.z, src);
        scale /= 3.f;
        __syncwarp();
    }
    return pos;
}

// ---------------------------------------------------------------------------
// Laplace smoothers toward AbstractMeasurer::computeVertexEquilibrium
// ---------------------------------------------------------------------------
// Metric-free (Measurers/MetricFreeMeasurer.cpp:107-152): pos + the sum over
// the incident elements of (p_i - pos) for every element vertex, over the sum
// of (vertex count - 1).  Metric-wise (MetricWiseMeasurer.cpp:190-255): every
// element vertex with d = p_i - pos != 0 adds w = sqrt(n . M(p_i) n),
// n = d / |d|, to the weight and w d to the displacement.  Elements over the
// lanes, then a warp reduction.
template <int MAXK>
__device__ V3<float> vertex_equilibrium(const MeshView& m, const Crew& crew, uint32_t v, V3<float> pos, int lane)
{
    const bool wise = crew.measurer == kMeasurerMetricWise;
    const uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
    V3<float> disp = mk(0.f, 0.f, 0.f);
    float weight = 0.f;
    for (uint32_t i = b + lane; i < e; i += kWarp)
    {
        const uint32_t r = m.ve[GM_IX(m, i, m.ve_len, kBoundsNeighbourElem)];
        const int type = MAXK == 4 ? kTet : ref_type(r);
        uint32_t vid[8];
        elem_vertices(m, type, ref_id(r), vid);
        const int n = MAXK == 4 ? 4 : type_size(type);
        if (!wise) weight += (float)(n - 1);
#pragma unroll
        for (int k = 0; k < MAXK; ++k)
        {
            if (k >= n) break;
            const V3<float> p = to<float>(__ldcg(&m.pos[vid[k]]));
            const V3<float> d = p - pos;
            if (!wise) disp = disp + d;
            else if (d.x != 0.f || d.y != 0.f || d.z != 0.f)
            {
                const float w = sqrtf(quad_form(metric_at(crew, p), normalize(d)));
                weight += w;
                disp = disp + d * w;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        disp.x += __shfl_xor_sync(0xffffffffu, disp.x, o);
        disp.y += __shfl_xor_sync(0xffffffffu, disp.y, o);
        disp.z += __shfl_xor_sync(0xffffffffu, disp.z, o);
        weight += __shfl_xor_sync(0xffffffffu, weight, o);
    }
    return pos + disp * (1.f / weight);
}

// SpringLaplaceSmoother::smoothVertices (Smoothers/VertexWise/SpringLaplaceSmoother.cpp:51-78):
// mix(pos, equilibrium, moveCoeff) = pos + moveCoeff (equilibrium - pos), projected
template <int MAXK>
__device__ V3<float> spring_laplace(const MeshView& m, const Crew& crew, const SmoothParams& sp, uint32_t v, int cid,
                                    V3<float> pos, int lane)
{
    const V3<float> c = vertex_equilibrium<MAXK>(m, crew, v, pos, lane);
    const V3<float> out = pos + (c - pos) * sp.shift;
    return cid != 0 ? snap(m, cid, out) : out;
}

// QualityLaplaceSmoother::smoothVertices (Smoothers/VertexWise/QualityLaplaceSmoother.cpp:55-129):
// 8 propositions pos + shift * {-0.25, 0, 0.1, 0.2, 0.4, 0.8, 1.2, 1.6} along
// shift = moveCoeff (equilibrium - pos), projected, evaluated at once; the
// first best patch quality wins
template <int VAR, int MAXK>
__device__ V3<float> quality_laplace(const MeshView& m, const Crew& crew, const SmoothParams& sp, WarpPatch& P,
                                     uint32_t v, int cid, V3<float> pos, int lane, int& evals)
{
    const V3<float> c = vertex_equilibrium<MAXK>(m, crew, v, pos, lane);
    const V3<float> shift = (c - pos) * sp.shift;
    V3<float> mine = pos;
    if (lane < 8)
    {
        V3<float> x = pos + shift * gd_offset(lane);
        if (cid != 0) x = snap(m, cid, x);
        P.cand[lane] = make_float4(x.x, x.y, x.z, 0.f);
        mine = x;
    }
    __syncwarp();
    patch_multi<VAR, MAXK, float>(crew, P, 8, lane);
    evals += 8;
    int best = 0;
    float bestQ = -3.0e38f;
    for (int p = 0; p < 8; ++p)
    {
        const float q = P.res[p];
        if (q > bestQ)
        {
            bestQ = q;
            best = p;
        }
    }
    V3<float> out;
    out.x = __shfl_sync(0xffffffffu, mine.x, best);
    out.y = __shfl_sync(0xffffffffu, mine.y, best);
    out.z = __shfl_sync(0xffffffffu, mine.z, best);
    __syncwarp();
    return out;
}

// ---------------------------------------------------------------------------
// GETMe element transform (Smoothers/ElementWise/GetmeSmoother.cpp:55-374)
// ---------------------------------------------------------------------------
template <int VAR, class R>
__device__ __forceinline__ R tet_volume(const Crew& c, const V3<R>* vp)
{
    if (VarTraits<VAR>::metric_wise)
        return det3(segment<VAR, R>(c, vp[0], vp[3]), segment<VAR, R>(c, vp[1], vp[3]), segment<VAR, R>(c, vp[2], vp[3])) / R(6);
    return (R)c.scaling3 * det3(vp[3] - vp[0], vp[3] - vp[1], vp[3] - vp[2]) / R(6);
}

template <int VAR, class R>
__device__ __forceinline__ R pri_volume(const Crew& c, const V3<R>* vp)
{
    V3<R> e02, e12, e32, e42, e52;
    constexpr bool mw = VarTraits<VAR>::metric_wise;
    if (mw)
    {
        e02 = segment<VAR, R>(c, vp[0], vp[2]); e12 = segment<VAR, R>(c, vp[1], vp[2]); e32 = segment<VAR, R>(c, vp[3], vp[2]);
        e42 = segment<VAR, R>(c, vp[4], vp[2]); e52 = segment<VAR, R>(c, vp[5], vp[2]);
    }
    else
    {
        e02 = vp[2] - vp[0]; e12 = vp[2] - vp[1]; e32 = vp[2] - vp[3]; e42 = vp[2] - vp[4]; e52 = vp[2] - vp[5];
    }
    R d = det3(e32, e52, e42) + det3(e02, e32, e42) + det3(e12, e02, e42);
    return mw ? d / R(6) : (R)c.scaling3 * d / R(6);
}

template <int VAR, class R>
__device__ __forceinline__ R hex_volume(const Crew& c, const V3<R>* vp)
{
    if (VarTraits<VAR>::metric_wise)
    {
        R d = det3(segment<VAR, R>(c, vp[1], vp[0]), segment<VAR, R>(c, vp[4], vp[0]), segment<VAR, R>(c, vp[3], vp[0]));
        d += det3(segment<VAR, R>(c, vp[1], vp[2]), segment<VAR, R>(c, vp[3], vp[2]), segment<VAR, R>(c, vp[6], vp[2]));
        d += det3(segment<VAR, R>(c, vp[4], vp[5]), segment<VAR, R>(c, vp[1], vp[5]), segment<VAR, R>(c, vp[6], vp[5]));
        d += det3(segment<VAR, R>(c, vp[4], vp[7]), segment<VAR, R>(c, vp[6], vp[7]), segment<VAR, R>(c, vp[3], vp[7]));
        d += det3(segment<VAR, R>(c, vp[1], vp[4]), segment<VAR, R>(c, vp[6], vp[4]), segment<VAR, R>(c, vp[3], vp[4]));
        return d / R(6);
    }
    R d = det3(vp[0] - vp[1], vp[0] - vp[4], vp[0] - vp[3]);
    d += det3(vp[2] - vp[1], vp[2] - vp[3], vp[2] - vp[6]);
    d += det3(vp[5] - vp[4], vp[5] - vp[1], vp[5] - vp[6]);
    d += det3(vp[7] - vp[4], vp[7] - vp[6], vp[7] - vp[3]);
    d += det3(vp[4] - vp[1], vp[4] - vp[6], vp[4] - vp[3]);
    return (R)c.scaling3 * d / R(6);
}

template <int VAR, class R>
__device__ __forceinline__ R quality_value(const Crew& c, int type, const V3<R>* p, uint32_t hint)
{
    EQ<R> q = elem_quality<VAR, 8, R>(c, type, p, hint);
    return q.pos ? R(1) / q.v : q.v;
}

// transformed corners and weight of one element; fixed corners keep their
// position (their VertexConstraint), constrained corners are projected
template <int VAR, class R, int N>
__device__ __forceinline__ R getme_transform(const MeshView& m, const Crew& c, R lambda, int type, const uint32_t* vi,
                                             const V3<R>* vp, V3<R>* vpp, uint32_t hint)
{
    V3<R> nrm[N];
    if (N == 4)
    {
        nrm[0] = cross(vp[3] - vp[1], vp[2] - vp[1]);
        nrm[1] = cross(vp[3] - vp[2], vp[0] - vp[2]);
        nrm[2] = cross(vp[1] - vp[3], vp[0] - vp[3]);
        nrm[3] = cross(vp[1] - vp[0], vp[2] - vp[0]);
        for (int k = 0; k < N; ++k) vpp[k] = vp[k] + nrm[k] * (lambda * rsqrt_<R>(length(nrm[k])));
    }
    else if (N == 6)
    {
        V3<R> aux[5] = {(vp[0] + vp[1] + vp[2]) * R(1.0 / 3.0), (vp[0] + vp[1] + vp[4] + vp[3]) * R(0.25),
                        (vp[1] + vp[2] + vp[5] + vp[4]) * R(0.25), (vp[2] + vp[0] + vp[3] + vp[5]) * R(0.25),
                        (vp[3] + vp[4] + vp[5]) * R(1.0 / 3.0)};
        nrm[0] = cross(aux[1] - aux[0], aux[3] - aux[0]);
        nrm[1] = cross(aux[2] - aux[0], aux[1] - aux[0]);
        nrm[2] = cross(aux[3] - aux[0], aux[2] - aux[0]);
        nrm[3] = cross(aux[3] - aux[4], aux[1] - aux[4]);
        nrm[4] = cross(aux[1] - aux[4], aux[2] - aux[4]);
        nrm[5] = cross(aux[2] - aux[4], aux[3] - aux[4]);
        R t = R(4.0 / 5.0) * (R(1) - pow(R(4.0 / 39.0), R(0.25)) * lambda);
        R it = R(1) - t;
        V3<R> bases[6] = {aux[0] * it + (aux[3] + aux[1]) * (t * R(0.5)), aux[0] * it + (aux[1] + aux[2]) * (t * R(0.5)),
                          aux[0] * it + (aux[2] + aux[3]) * (t * R(0.5)), aux[4] * it + (aux[3] + aux[1]) * (t * R(0.5)),
                          aux[4] * it + (aux[1] + aux[2]) * (t * R(0.5)), aux[4] * it + (aux[2] + aux[3]) * (t * R(0.5))};
        for (int k = 0; k < N; ++k) vpp[k] = bases[k] + nrm[k] * (lambda * rsqrt_<R>(length(nrm[k])));
    }
    else
    {
        V3<R> aux[6] = {(vp[0] + vp[1] + vp[2] + vp[3]) * R(0.25), (vp[0] + vp[4] + vp[5] + vp[1]) * R(0.25),
                        (vp[1] + vp[5] + vp[6] + vp[2]) * R(0.25), (vp[2] + vp[6] + vp[7] + vp[3]) * R(0.25),
                        (vp[0] + vp[3] + vp[7] + vp[4]) * R(0.25), (vp[4] + vp[7] + vp[6] + vp[5]) * R(0.25)};
        nrm[0] = cross(aux[1] - aux[0], aux[4] - aux[0]);
        nrm[1] = cross(aux[2] - aux[0], aux[1] - aux[0]);
        nrm[2] = cross(aux[3] - aux[0], aux[2] - aux[0]);
        nrm[3] = cross(aux[4] - aux[0], aux[3] - aux[0]);
        nrm[4] = cross(aux[4] - aux[5], aux[1] - aux[5]);
        nrm[5] = cross(aux[1] - aux[5], aux[2] - aux[5]);
        nrm[6] = cross(aux[2] - aux[5], aux[3] - aux[5]);
        nrm[7] = cross(aux[3] - aux[5], aux[4] - aux[5]);
        const int B[8][3] = {{0, 1, 4}, {0, 2, 1}, {0, 3, 2}, {0, 4, 3}, {5, 4, 1}, {5, 1, 2}, {5, 2, 3}, {5, 3, 4}};
        for (int k = 0; k < N; ++k)
        {
            V3<R> base = (aux[B[k][0]] + aux[B[k][1]] + aux[B[k][2]]) * R(1.0 / 3.0);
            vpp[k] = base + nrm[k] * (lambda * rsqrt_<R>(length(nrm[k])));
        }
    }
    R vol, volp;
    if (N == 4) { vol = tet_volume<VAR, R>(c, vp); volp = tet_volume<VAR, R>(c, vpp); }
    else if (N == 6) { vol = pri_volume<VAR, R>(c, vp); volp = pri_volume<VAR, R>(c, vpp); }
    else { vol = hex_volume<VAR, R>(c, vp); volp = hex_volume<VAR, R>(c, vpp); }
    R var = cbrt_(fabs(vol / volp));
    V3<R> center = vp[0];
    for (int k = 1; k < N; ++k) center = center + vp[k];
    center = center * (R(1) / R(N));
    for (int k = 0; k < N; ++k)
    {
        vpp[k] = center + (vpp[k] - center) * var;
        int id = m.cid[vi[k]];
        if (id < 0) vpp[k] = vp[k];
        else if (id > 0) vpp[k] = snap(m, id, vpp[k]);
    }
    R q = quality_value<VAR, R>(c, type, vp, hint);
    R qp = quality_value<VAR, R>(c, type, vpp, hint);
    return qp / (R(1) + q);
}

}  // namespace gm
