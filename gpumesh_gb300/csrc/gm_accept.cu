// FP64 acceptance test for near-degenerate patches.
//
// The FP32 relocation kernels hand over every vertex whose old or new patch
// quality is below the acceptance threshold (1e-3 by default).  Here a warp
// per such vertex (a grid-stride loop over them) evaluates both patch
// qualities in FP64 and keeps the move only if the new quality is not lower
// -- the rule of
// AbstractElementWiseSmoother::updateVertexPositions
// (Smoothers/ElementWise/AbstractElementWiseSmoother.cpp:433-441).  The
// vertex-wise smoothers always include the old position among their
// candidates, so in exact arithmetic the rule never rejects their moves; in
// FP32 on an almost flat patch it can, and FP64 decides.
#include <cuda_runtime.h>

#include "gm_relocate.cuh"

namespace gm {

template <int VAR, int MAXK>
__global__ void __launch_bounds__(128) accept_kernel(MeshView m, Crew crew, Deferred def, uint32_t slot_base,
                                                     uint32_t cap, int maxe)
{
    GM_PDL_ENTRY();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t n = min(*def.count, cap);
    const uint32_t stride = gridDim.x * (blockDim.x >> 5);
    WarpPatch P = carve_patch(smem + wib * warp_patch_bytes(MAXK, maxe), MAXK, maxe);
    // the deferred vertices of one colour: an independent set, so the order
    // in which the warps take them does not matter
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + wib; w < n; w += stride)
    {
        const uint32_t v = GM_IX(m, def.v[slot_base + w], m.nv, kBoundsPosition);
        stage_patch(m, v, P, lane);
        const float4 oldp = def.oldp[slot_base + w], newp = def.newp[slot_base + w];
        const double q0 = patch_uniform<VAR, MAXK, double>(crew, P, to<double>(oldp), lane);
        const double q1 = patch_uniform<VAR, MAXK, double>(crew, P, to<double>(newp), lane);
        if (lane == 0 && !(q1 < q0)) m.pos[v] = newp;
        __syncwarp();  // the patch is staged again for the next vertex
    }
}

template <int VAR, int MAXK>
static cudaError_t launch_accept_t(const RelocLaunch& L)
{
    size_t smem = patch_smem_per_warp(MAXK, L.maxe) * L.warps_per_block;
    if (smem > 48 * 1024)
    {
        cudaError_t e = cudaFuncSetAttribute(accept_kernel<VAR, MAXK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    // the deferred count is on the device: a grid of a few blocks per SM loops
    // over however many there are (usually a few dozen of a colour's
    // thousands of vertices, so a grid sized to the colour was mostly warps
    // that read the count and left)
    unsigned blocks = (L.count + L.warps_per_block - 1) / L.warps_per_block;
    const unsigned cap_blocks = (unsigned)(L.sm_count > 0 ? L.sm_count : 152) * 4u;
    blocks = blocks < cap_blocks ? blocks : cap_blocks;
    const cudaError_t e = launch_pdl(accept_kernel<VAR, MAXK>, dim3(blocks), dim3(32 * L.warps_per_block), smem,
                                     L.stream, L.m, L.crew, L.def, L.slot_base, L.count, L.maxe);
    note_launch();
    return e;
}

cudaError_t launch_accept(const RelocLaunch& L)
{
    if (L.count == 0) return cudaSuccess;
    switch (L.variant)
    {
    case kVarMRFree: return L.maxk == 4 ? launch_accept_t<kVarMRFree, 4>(L) : launch_accept_t<kVarMRFree, 8>(L);
    case kVarMRWise: return launch_accept_t<kVarMRWise, 8>(L);
    case kVarMCDiag: return L.maxk == 4 ? launch_accept_t<kVarMCDiag, 4>(L) : launch_accept_t<kVarMCDiag, 8>(L);
    default: return L.maxk == 4 ? launch_accept_t<kVarMC, 4>(L) : launch_accept_t<kVarMC, 8>(L);
    }
}

}  // namespace gm
