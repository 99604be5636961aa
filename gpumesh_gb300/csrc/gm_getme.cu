// GETMe element-wise smoothing: the element transform pass and the
// per-group vertex update with the patch-quality acceptance test
// (Smoothers/ElementWise/GetmeSmoother.cpp:55-374,
//  Smoothers/ElementWise/AbstractElementWiseSmoother.cpp:406-444).
//
// The element pass writes each element's transformed corners and weight to
// a per-(element, corner) buffer instead of accumulating them with atomics;
// the update pass gathers a vertex's corners through its vertex->element
// list, so the sums are deterministic.
#include <cuda_runtime.h>

#include "gm_relocate.cuh"

namespace gm {

template <int VAR, int N>
__device__ __forceinline__ void getme_one(const MeshView& m, const Crew& crew, float lambda, int type, uint32_t id,
                                          float4* out)
{
    uint32_t vi[8];
    elem_vertices(m, type, id, vi);
    V3<float> vp[N], vpp[N];
#pragma unroll
    for (int k = 0; k < N; ++k) vp[k] = to<float>(m.pos[vi[k]]);  // vi checked by elem_vertices
    float w = getme_transform<VAR, float, N>(m, crew, lambda, type, vi, vp, vpp, elem_hint(type, id));
#pragma unroll
    // streaming stores: each corner is read once, by its vertex's update, and
    // the corner buffer (16 B per element corner) is larger than the L2, so it
    // should not push out the positions and connectivity the updates stage
    for (int k = 0; k < N; ++k) __stcs(&out[(size_t)id * N + k], make_float4(vpp[k].x, vpp[k].y, vpp[k].z, w));
}

template <int VAR>
__global__ void __launch_bounds__(256) getme_elements_kernel(MeshView m, Crew crew, float lambda, float4* corners)
{
    GM_PDL_ENTRY();
    const uint32_t total = m.nt + m.np + m.nh;
    float4* ctet = corners;
    float4* cpri = corners + 4 * (size_t)m.nt;
    float4* chex = cpri + 6 * (size_t)m.np;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
    {
        if (i < m.nt) getme_one<VAR, 4>(m, crew, lambda, kTet, i, ctet);
        else if (i < m.nt + m.np) getme_one<VAR, 6>(m, crew, lambda, kPri, i - m.nt, cpri);
        else getme_one<VAR, 8>(m, crew, lambda, kHex, i - m.nt - m.np, chex);
    }
}

cudaError_t launch_getme_elements(int variant, const MeshView& m, const Crew& crew, float lambda, float4* corners,
                                  int sm_count, cudaStream_t s)
{
    uint32_t total = m.nt + m.np + m.nh;
    if (total == 0) return cudaSuccess;
    long need = ((long)total + 255) / 256;
    long cap = (long)sm_count * 8;
    int blocks = (int)(need < cap ? need : cap);
    void (*k)(MeshView, Crew, float, float4*);
    switch (variant)
    {
    case kVarMRFree: k = getme_elements_kernel<kVarMRFree>; break;
    case kVarMRWise: k = getme_elements_kernel<kVarMRWise>; break;
    case kVarMC: k = getme_elements_kernel<kVarMC>; break;
    default: k = getme_elements_kernel<kVarMCWise>; break;
    }
    const cudaError_t e = launch_pdl(k, dim3(blocks), dim3(256), 0, s, m, crew, lambda, corners);
    note_launch();
    return e;
}

// weighted average of the vertex's transformed corners
__device__ __forceinline__ bool getme_average(const MeshView& m, const float4* corners, uint32_t v, int lane,
                                              V3<float>& out)
{
    const size_t base[4] = {0, 0, 4 * (size_t)m.nt, 4 * (size_t)m.nt + 6 * (size_t)m.np};
    uint32_t b = m.ve_off[v], e = m.ve_off[v + 1];
    float sx = 0, sy = 0, sz = 0, sw = 0;
    for (uint32_t i = b + lane; i < e; i += kWarp)
    {
        uint32_t r = m.ve[GM_IX(m, i, m.ve_len, kBoundsNeighbourElem)];
        int type = ref_type(r);
        const size_t ci = base[type] + (size_t)ref_id(r) * type_size(type) + ref_local(r);
        float4 c = __ldcs(&corners[GM_IX(m, ci, 4 * m.nt + 6 * m.np + 8 * m.nh, kBoundsCorner)]);  // read once
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
    if (sw == 0.f) return false;
    out = mk(sx / sw, sy / sw, sz / sw);
    return true;
}

template <int VAR, int MAXK>
__global__ void __launch_bounds__(128) getme_update_kernel(MeshView m, Crew crew, SmoothParams sp,
                                                           const float4* corners, const uint32_t* members,
                                                           uint32_t count, int maxe, Counters* ctr, Deferred def,
                                                           uint32_t slot_base)
{
    GM_PDL_ENTRY();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= count) return;
    WarpPatch P = carve_patch(smem + wib * warp_patch_bytes(MAXK, maxe), MAXK, maxe);
    const uint32_t v = GM_IX(m, members[w], m.nv, kBoundsPosition);
    V3<float> prim;
    if (!getme_average(m, corners, v, lane, prim)) return;
    const int cid = m.cid[v];
    if (cid != 0) prim = snap(m, cid, prim);
    const float4 old = m.pos[v];
    stage_patch_fp32<VAR, MAXK>(m, crew, v, to<float>(old), P, lane);
    if (lane == 0)
    {
        P.cand[0] = old;
        P.cand[1] = make_float4(prim.x, prim.y, prim.z, 0.f);
    }
    __syncwarp();
    patch_multi<VAR, MAXK, float>(crew, P, 2, lane);
    const float q = P.res[0], qp = P.res[1];
    const bool defer = !(q >= sp.accept_q && qp >= sp.accept_q);
    if (lane == 0)
    {
        float4 nw = make_float4(prim.x, prim.y, prim.z, old.w);
        if (defer)
        {
            uint32_t k = atomicAdd(def.count, 1u);
            def.v[slot_base + k] = v;
            def.oldp[slot_base + k] = old;
            def.newp[slot_base + k] = nw;
        }
        else if (!(qp < q))
            m.pos[v] = nw;
    }
    count_work(ctr, 2, P.E, MAXK == 4 ? kTet : kHex, defer, lane);
}

// ---------------------------------------------------------------------------
// Hex and mixed meshes: four vertices per warp, one per group of 8 lanes.
// With a hex patch of 8 elements, one vertex per warp leaves three quarters
// of the lanes idle in the weighted average and half of them in the two patch
// evaluations, and the kernel is bound by the latency of its gathers; four
// vertices per warp keep four times as many patches in flight.  Every sum is
// taken in the order of the one-vertex-per-warp form (getme_average's 32-lane
// butterfly, patch_multi's 16 lanes per candidate): each lane keeps the
// partial sums of the virtual lanes it stands for and folds them as that
// butterfly does, so positions and decisions equal the warp-per-vertex form
// and the batched path bit for bit.
constexpr int kGetmeGroup = 8;
constexpr int kGetmeGroups = kWarp / kGetmeGroup;
constexpr int kGetmeGroupWarps = 4;  // warps per block

// shared memory of one group: the patch's corner slots (8 x maxe float4),
// then the element meta words (maxe ints, padded to 16 bytes)
__host__ __device__ constexpr size_t getme_group_bytes(int maxe)
{
    return (size_t)8 * maxe * sizeof(float4) + (((size_t)maxe * sizeof(int) + 15) & ~(size_t)15);
}

template <int VAR>
__global__ void __launch_bounds__(kGetmeGroupWarps * 32) getme_update_groups_kernel(
    MeshView m, Crew crew, SmoothParams sp, const float4* corners, const uint32_t* members, uint32_t count, int maxe,
    Counters* ctr, Deferred def, uint32_t slot_base)
{
    GM_PDL_ENTRY();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gi = lane / kGetmeGroup, sub = lane % kGetmeGroup;
    const uint32_t w = (blockIdx.x * kGetmeGroupWarps + wib) * kGetmeGroups + gi;
    const bool active = w < count;
    if (!__any_sync(0xffffffffu, active)) return;  // warp-uniform
    char* gsm = smem + (size_t)(wib * kGetmeGroups + gi) * getme_group_bytes(maxe);
    WarpPatch P;
    P.sp = reinterpret_cast<float4*>(gsm);
    P.pp = nullptr;
    P.meta = reinterpret_cast<int*>(gsm + (size_t)8 * maxe * sizeof(float4));
    P.cand = nullptr;
    P.res = nullptr;
    P.maxe = maxe;
    P.o = V3<float>{0.f, 0.f, 0.f};
    const uint32_t v = active ? GM_IX(m, members[w], m.nv, kBoundsPosition) : 0u;
    const uint32_t b = active ? m.ve_off[v] : 0u, e = active ? m.ve_off[v + 1] : 0u;

    // weighted average of the transformed corners: virtual lanes sub + 8k
    // (k = 0..3) of a 32-lane pass over the incident elements
    const size_t base[4] = {0, 0, 4 * (size_t)m.nt, 4 * (size_t)m.nt + 6 * (size_t)m.np};
    float4 acc[4] = {};
#pragma unroll
    for (int k = 0; k < 4; ++k)
        for (uint32_t i = b + sub + kGetmeGroup * k; i < e; i += kWarp)
        {
            const uint32_t r = m.ve[GM_IX(m, i, m.ve_len, kBoundsNeighbourElem)];
            const int type = ref_type(r);
            const size_t ci = base[type] + (size_t)ref_id(r) * type_size(type) + ref_local(r);
            const float4 c = __ldcs(&corners[GM_IX(m, ci, 4 * m.nt + 6 * m.np + 8 * m.nh, kBoundsCorner)]);  // read once
            acc[k].x += c.x * c.w;
            acc[k].y += c.y * c.w;
            acc[k].z += c.z * c.w;
            acc[k].w += c.w;
        }
    // the butterfly's steps 16 and 8 inside the lane, then 4, 2, 1 across the group
    float sx = (acc[0].x + acc[2].x) + (acc[1].x + acc[3].x), sy = (acc[0].y + acc[2].y) + (acc[1].y + acc[3].y);
    float sz = (acc[0].z + acc[2].z) + (acc[1].z + acc[3].z), sw = (acc[0].w + acc[2].w) + (acc[1].w + acc[3].w);
    for (int o = kGetmeGroup / 2; o > 0; o >>= 1)
    {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
    }
    const bool ok = active && sw != 0.f;
    V3<float> prim = mk(0.f, 0.f, 0.f);
    float4 old = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ok)
    {
        prim = mk(sx / sw, sy / sw, sz / sw);
        const int cid = m.cid[v];
        if (cid != 0) prim = snap(m, cid, prim);
        old = m.pos[v];
    }

    // the patch, staged by the group (stage_patch's layout)
    P.E = ok ? (int)(e - b) : 0;
    for (int i = sub; i < P.E; i += kGetmeGroup)
    {
        const uint32_t r = m.ve[GM_IX(m, b + i, m.ve_len, kBoundsNeighbourElem)];
        const int type = ref_type(r), loc = ref_local(r);
        uint32_t vid[8];
        elem_vertices(m, type, ref_id(r), vid);
        const int n = type_size(type);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < n) P.sp[k * P.maxe + i] = __ldcg(&m.pos[vid[k]]);
        P.meta[i] = (int)((uint32_t)type | ((uint32_t)loc << 2) | (ref_id(r) << 5));
    }
    __syncwarp();

    // the two candidates (old position, average): virtual lanes sub and
    // sub + 8 of the 16 lanes patch_multi gives each candidate
    PatchAcc<float> a[2][2] = {{{0.f, 3.0e38f, 0}, {0.f, 3.0e38f, 0}}, {{0.f, 3.0e38f, 0}, {0.f, 3.0e38f, 0}}};
    const V3<float> cpos[2] = {to<float>(old), prim};
#pragma unroll
    for (int h = 0; h < 2; ++h)
        for (int i = sub + kGetmeGroup * h; i < P.E; i += 2 * kGetmeGroup)
        {
            acc_add(a[0][h], staged_quality<VAR, 8, float>(crew, P, i, cpos[0]));
            acc_add(a[1][h], staged_quality<VAR, 8, float>(crew, P, i, cpos[1]));
        }
    float q[2];
#pragma unroll
    for (int c = 0; c < 2; ++c)
    {
        // acc_reduce's steps: 8 inside the lane, then 4, 2, 1 across the group
        PatchAcc<float> t{a[c][0].rsum + a[c][1].rsum,
                          a[c][1].minq < a[c][0].minq ? a[c][1].minq : a[c][0].minq, a[c][0].nbad + a[c][1].nbad};
        for (int o = kGetmeGroup / 2; o > 0; o >>= 1)
        {
            t.rsum += __shfl_xor_sync(0xffffffffu, t.rsum, o);
            const float mq = __shfl_xor_sync(0xffffffffu, t.minq, o);
            t.minq = mq < t.minq ? mq : t.minq;
            t.nbad += __shfl_xor_sync(0xffffffffu, t.nbad, o);
        }
        q[c] = acc_final(t, P.E);
    }
    if (!ok) return;
    const bool defer = !(q[0] >= sp.accept_q && q[1] >= sp.accept_q);
    if (sub == 0)
    {
        const float4 nw = make_float4(prim.x, prim.y, prim.z, old.w);
        if (defer)
        {
            const uint32_t k = atomicAdd(def.count, 1u);
            def.v[slot_base + k] = v;
            def.oldp[slot_base + k] = old;
            def.newp[slot_base + k] = nw;
        }
        else if (!(q[1] < q[0]))
            m.pos[v] = nw;
    }
    count_work(ctr, 2, P.E, kHex, defer, sub);
}

template <int VAR>
static cudaError_t launch_update_groups_t(const RelocLaunch& L, const float4* corners)
{
    // a group's patch is sized by the mesh's largest vertex valence (8 on a
    // hex mesh), not by the 32-padded maxe of the warp-per-vertex kernels:
    // the shared memory then allows the 5 resident blocks per SM the
    // registers do, instead of 3
    const int maxe = L.max_incident > 0 ? L.max_incident : L.maxe;
    const size_t smem = getme_group_bytes(maxe) * kGetmeGroups * kGetmeGroupWarps;
    if (smem > 48 * 1024)
    {
        cudaError_t e = cudaFuncSetAttribute(getme_update_groups_kernel<VAR>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const uint32_t per_block = kGetmeGroups * kGetmeGroupWarps;
    const unsigned blocks = (L.count + per_block - 1) / per_block;
    const cudaError_t e = launch_pdl(getme_update_groups_kernel<VAR>, dim3(blocks), dim3(32 * kGetmeGroupWarps), smem,
                                     L.stream, L.m, L.crew, L.sp, corners, L.members, L.count, maxe, L.ctr, L.def,
                                     L.slot_base);
    note_launch();
    return e;
}

template <int VAR, int MAXK>
static cudaError_t launch_update_t(const RelocLaunch& L, const float4* corners)
{
    if constexpr (MAXK == 8)
        return launch_update_groups_t<VAR>(L, corners);
    else
    {
        size_t smem = patch_smem_per_warp(MAXK, L.maxe) * L.warps_per_block;
        if (smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(getme_update_kernel<VAR, MAXK>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        unsigned blocks = (L.count + L.warps_per_block - 1) / L.warps_per_block;
        const cudaError_t e = launch_pdl(getme_update_kernel<VAR, MAXK>, dim3(blocks), dim3(32 * L.warps_per_block),
                                         smem, L.stream, L.m, L.crew, L.sp, corners, L.members, L.count, L.maxe,
                                         L.ctr, L.def, L.slot_base);
        note_launch();
        return e;
    }
}

cudaError_t launch_getme_update(const RelocLaunch& L, const float4* corners)
{
    if (L.count == 0) return cudaSuccess;
    switch (L.variant)
    {
    case kVarMRFree: return L.maxk == 4 ? launch_update_t<kVarMRFree, 4>(L, corners)
                                        : launch_update_t<kVarMRFree, 8>(L, corners);
    case kVarMRWise: return launch_update_t<kVarMRWise, 8>(L, corners);
    case kVarMCDiag: return L.maxk == 4 ? launch_update_t<kVarMCDiag, 4>(L, corners)
                                        : launch_update_t<kVarMCDiag, 8>(L, corners);
    default: return L.maxk == 4 ? launch_update_t<kVarMC, 4>(L, corners) : launch_update_t<kVarMC, 8>(L, corners);
    }
}

}  // namespace gm
