// Vertex-relocation kernels: one warp per vertex of one independent group.
// Included by one translation unit per smoother so that each kernel family
// compiles in parallel.
#pragma once

#include <cuda_runtime.h>

#include "gm_kernels.cuh"
#include "gm_launch.h"
#include "gm_nm_lockstep.cuh"

namespace gm {

__device__ __forceinline__ void count_work(Counters* ctr, int evals, int E, int type, bool fp64, int lane)
{
    if (!ctr || lane != 0) return;
    atomicAdd(&ctr->patch_evals, (unsigned long long)evals);
    atomicAdd(&ctr->elem_evals[type & 3], (unsigned long long)evals * (unsigned long long)E);
    if (fp64) atomicAdd(&ctr->fp64_vertices, 1ull);
}

// Move v to `out` unless either its old or new patch quality is below the
// acceptance threshold; those vertices are handed to the FP64 acceptance
// kernel, which keeps the move only if FP64 agrees it does not lower the
// patch quality.
__device__ __forceinline__ bool commit_or_defer(const MeshView& m, const SmoothParams& sp, const Deferred& def,
                                                uint32_t slot_base, uint32_t v, float4 old, V3<float> out, float q0,
                                                float q1, int lane)
{
    bool defer = !(q0 >= sp.accept_q && q1 >= sp.accept_q);
    if (lane == 0)
    {
        float4 nw = make_float4(out.x, out.y, out.z, old.w);
        if (defer)
        {
            uint32_t k = atomicAdd(def.count, 1u);
            def.v[slot_base + k] = v;
            def.oldp[slot_base + k] = old;
            def.newp[slot_base + k] = nw;
        }
        else
            m.pos[v] = nw;
    }
    return defer;
}

// resident blocks per SM the register allocation aims for: the paired FP32
// metric-conformity evaluation on tets (gradient descent, spawn search)
// fits in 95 registers without spilling at 5 blocks of 4 warps; the other
// variants take what they need
template <int SMOOTHER, int VAR, int MAXK>
constexpr int kRelocMinBlocks = (VAR == kVarMCDiag && MAXK == 4 && (SMOOTHER == kSmoothGD || SMOOTHER == kSmoothSpawn))
                                    ? 5 : 1;

template <int SMOOTHER, int VAR, int MAXK>
__global__ void __launch_bounds__(128, kRelocMinBlocks<SMOOTHER, VAR, MAXK>) relocate_kernel(MeshView m, Crew crew, SmoothParams sp,
                                                       const uint32_t* members, uint32_t count, int maxe,
                                                       Counters* ctr, Deferred def, uint32_t slot_base)
{
    GM_PDL_ENTRY();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t w = blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= count) return;
    WarpPatch P = carve_patch(smem + wib * warp_patch_bytes(MAXK, maxe), MAXK, maxe);
    const uint32_t v = GM_IX(m, members[w], m.nv, kBoundsPosition);
    const int cid = m.cid[v];
    const float4 old = m.pos[v];
    const V3<float> pos = to<float>(old);
    if constexpr (SMOOTHER == kSmoothSpring)
    {
        // no quality test: the reference moves the vertex unconditionally
        const V3<float> out = spring_laplace<MAXK>(m, crew, sp, v, cid, pos, lane);
        if (lane == 0) m.pos[v] = make_float4(out.x, out.y, out.z, old.w);
        return;
    }
    stage_patch_fp32<VAR, MAXK>(m, crew, v, pos, P, lane);
    int evals = 1;
    const float q0 = patch_uniform<VAR, MAXK, float>(crew, P, pos, lane);
    V3<float> out;
    if (SMOOTHER == kSmoothNM) out = nelder_mead<VAR, MAXK>(m, crew, sp, P, v, cid, pos, q0, lane, evals);
    else if (SMOOTHER == kSmoothGD)
        out = gradient_descent<VAR, MAXK>(m, crew, sp, P, v, cid, pos, lane, evals);
    else if (SMOOTHER == kSmoothQLaplace)
        out = quality_laplace<VAR, MAXK>(m, crew, sp, P, v, cid, pos, lane, evals);
    else out = spawn_search<VAR, MAXK>(m, crew, sp, P, v, cid, pos, lane, evals);
    ++evals;
    const float q1 = patch_uniform<VAR, MAXK, float>(crew, P, out, lane);
    bool deferred = commit_or_defer(m, sp, def, slot_base, v, old, out, q0, q1, lane);
    count_work(ctr, evals, P.E, MAXK == 4 ? kTet : kHex, deferred, lane);
}

// Nelder-Mead on canonical tet patches: kNMGroups vertices per warp in
// lockstep (gm_nm_lockstep.cuh); each warp owns `per_warp` consecutive
// members of the colour.  A colour too small to give every SM 16 warps gets
// one vertex per warp (the launch is latency bound: every vertex starts at
// once and no group waits for another's search); a large one up to four per
// group, so the groups of a warp refill and the tail where some groups idle
// is short against the warp's work.
constexpr int kNMWarpsPerBlock = 4;

template <int VAR>
__global__ void __launch_bounds__(kNMWarpsPerBlock * 32, 4)
    relocate_nm_lockstep_kernel(MeshView m, Crew crew, SmoothParams sp, const uint32_t* members, uint32_t count,
                                uint32_t per_warp, int maxe, Counters* ctr, Deferred def, uint32_t slot_base)
{
    GM_PDL_ENTRY();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t begin = (blockIdx.x * (blockDim.x >> 5) + wib) * per_warp;
    if (begin >= count) return;
    const uint32_t end = min(begin + per_warp, count);
    nm_lockstep_plain<VAR>(m, crew, sp, members, begin, end, smem + wib * nm_warp_bytes<VAR>(maxe), maxe, ctr, def,
                           slot_base, lane);
}

template <int VAR>
static cudaError_t launch_nm_lockstep(const RelocLaunch& L)
{
    const size_t smem = nm_warp_bytes<VAR>(L.maxe) * kNMWarpsPerBlock;
    if (smem > 48 * 1024)
    {
        cudaError_t e = cudaFuncSetAttribute(relocate_nm_lockstep_kernel<VAR>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // enough warps for every SM to hold 16, then more vertices per warp
    const uint64_t target_warps = (uint64_t)(L.sm_count > 0 ? L.sm_count : 152) * 16;
    uint32_t per_warp = (uint32_t)((L.count + target_warps - 1) / target_warps);
    per_warp = per_warp > 4u * kNMGroups ? 4u * kNMGroups : per_warp;
    const uint64_t per_block = (uint64_t)per_warp * kNMWarpsPerBlock;
    const unsigned blocks = (unsigned)((L.count + per_block - 1) / per_block);
    const cudaError_t e = launch_pdl(relocate_nm_lockstep_kernel<VAR>, dim3(blocks), dim3(32 * kNMWarpsPerBlock), smem,
                                     L.stream, L.m, L.crew, L.sp, L.members, L.count, per_warp, L.maxe, L.ctr, L.def,
                                     L.slot_base);
    note_launch();
    return e;
}

template <int SMOOTHER, int VAR, int MAXK>
static cudaError_t launch_relocate_t(const RelocLaunch& L)
{
    if constexpr (SMOOTHER == kSmoothNM && TetCanon<VAR, MAXK>::on)
        return launch_nm_lockstep<VAR>(L);
    else
    {
        size_t smem = patch_smem_per_warp(MAXK, L.maxe) * L.warps_per_block;
        if (smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(relocate_kernel<SMOOTHER, VAR, MAXK>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        unsigned blocks = (L.count + L.warps_per_block - 1) / L.warps_per_block;
        const cudaError_t e =
            launch_pdl(relocate_kernel<SMOOTHER, VAR, MAXK>, dim3(blocks), dim3(32 * L.warps_per_block), smem, L.stream,
                       L.m, L.crew, L.sp, L.members, L.count, L.maxe, L.ctr, L.def, L.slot_base);
        note_launch();
        return e;
    }
}

template <int SMOOTHER>
static cudaError_t launch_relocate_smoother(const RelocLaunch& L)
{
    if (L.count == 0) return cudaSuccess;
    switch (L.variant)
    {
    case kVarMRFree: return L.maxk == 4 ? launch_relocate_t<SMOOTHER, kVarMRFree, 4>(L)
                                        : launch_relocate_t<SMOOTHER, kVarMRFree, 8>(L);
    case kVarMRWise: return launch_relocate_t<SMOOTHER, kVarMRWise, 8>(L);
    case kVarMCDiag: return L.maxk == 4 ? launch_relocate_t<SMOOTHER, kVarMCDiag, 4>(L)
                                        : launch_relocate_t<SMOOTHER, kVarMCDiag, 8>(L);
    default: return L.maxk == 4 ? launch_relocate_t<SMOOTHER, kVarMC, 4>(L) : launch_relocate_t<SMOOTHER, kVarMC, 8>(L);
    }
}

}  // namespace gm
