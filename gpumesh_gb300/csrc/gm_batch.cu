// Launches of the batched kernels (gm_batch_kernels.cuh) for the metric-free
// mean ratio and metric conformity under a diagonal metric; the
// general-metric variants are compiled in gm_batch_general_mc.cu and
// gm_batch_general_mrwise.cu.
#include <cuda_runtime.h>

#include "gm_batch_kernels.cuh"

namespace gm {

template <int SMOOTHER>
static cudaError_t launch_batch_smoother(const BatchArgs& a, const SmoothParams& sp, int variant, int maxk, int wpb,
                                         int cps, int sm_count, cudaStream_t s)
{
    switch (variant)
    {
    case kVarMRFree:
        return maxk == 4 ? launch_batch_t<SMOOTHER, kVarMRFree, 4>(a, sp, wpb, cps, sm_count, s)
                         : launch_batch_t<SMOOTHER, kVarMRFree, 8>(a, sp, wpb, cps, sm_count, s);
    case kVarMCDiag:
        return maxk == 4 ? launch_batch_t<SMOOTHER, kVarMCDiag, 4>(a, sp, wpb, cps, sm_count, s)
                         : launch_batch_t<SMOOTHER, kVarMCDiag, 8>(a, sp, wpb, cps, sm_count, s);
    case kVarMC: return launch_batch_relocate_mc(SMOOTHER, a, sp, maxk, wpb, cps, sm_count, s);
    case kVarMRWise: return launch_batch_relocate_mrwise(SMOOTHER, a, sp, maxk, wpb, cps, sm_count, s);
    default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_batch_relocate(int smoother, const BatchArgs& a, const SmoothParams& sp, int variant, int maxk,
                                  int wpb, int cps, int sm_count, cudaStream_t s)
{
    if (a.total == 0) return cudaSuccess;
    switch (smoother)
    {
    case kSmoothNM: return launch_batch_smoother<kSmoothNM>(a, sp, variant, maxk, wpb, cps, sm_count, s);
    case kSmoothGD: return launch_batch_smoother<kSmoothGD>(a, sp, variant, maxk, wpb, cps, sm_count, s);
    case kSmoothSpawn: return launch_batch_smoother<kSmoothSpawn>(a, sp, variant, maxk, wpb, cps, sm_count, s);
    default: return launch_batch_smoother<kSmoothGetme>(a, sp, variant, maxk, wpb, cps, sm_count, s);
    }
}

__global__ void __launch_bounds__(256) batch_eval_finalize_kernel(const BatchMesh* meshes, const uint32_t* mesh_block,
                                                                   uint32_t nmesh, const EvalPartial* parts,
                                                                   Quality* out)
{
    const uint32_t m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= nmesh) return;
    const uint32_t b = mesh_block[m], e = mesh_block[m + 1];
    double sum = 0;
    float mn = 1.0f;
    unsigned long long bad = 0, h = 0;
    for (uint32_t i = b; i < e; ++i)
    {
        const EvalPartial& p = parts[i];
        sum += p.rsum;
        mn = fminf(mn, p.min);
        bad += (unsigned long long)p.nbad;
        if (lane < 20) h += (unsigned long long)p.hist[lane];
    }
    Quality& q = out[m];
    if (lane < 20) q.buckets[lane] = h;
    if (lane == 0)
    {
        const MeshView& v = meshes[m].view;
        q.min = (double)mn;
        q.nbad = bad;
        q.inv_sum = bad ? (double)INFINITY : sum;
        q.count = v.nt + v.np + v.nh;
    }
}

cudaError_t launch_batch_evaluate(const BatchMesh* meshes, uint32_t nmesh, const EvalBlock* blocks, uint32_t nblocks,
                                  const uint32_t* mesh_block, EvalPartial* parts, Quality* out, int variant, int maxk,
                                  cudaStream_t s)
{
    if (nblocks == 0) return cudaSuccess;
    switch (variant)
    {
    case kVarMRFree:
        if (maxk == 4) batch_eval_kernel<kVarMRFree, 4><<<nblocks, 256, 0, s>>>(meshes, blocks, parts);
        else batch_eval_kernel<kVarMRFree, 8><<<nblocks, 256, 0, s>>>(meshes, blocks, parts);
        break;
    case kVarMCDiag:
        if (maxk == 4) batch_eval_kernel<kVarMCDiag, 4><<<nblocks, 256, 0, s>>>(meshes, blocks, parts);
        else batch_eval_kernel<kVarMCDiag, 8><<<nblocks, 256, 0, s>>>(meshes, blocks, parts);
        break;
    case kVarMC:
    case kVarMRWise:
    {
        const cudaError_t e = variant == kVarMC ? launch_batch_eval_mc(meshes, blocks, nblocks, parts, maxk, s)
                                                : launch_batch_eval_mrwise(meshes, blocks, nblocks, parts, maxk, s);
        if (e != cudaSuccess) return e;
        break;
    }
    default: return cudaErrorNotSupported;
    }
    batch_eval_finalize_kernel<<<(nmesh + 7) / 8, 256, 0, s>>>(meshes, mesh_block, nmesh, parts, out);
    note_launch();
    note_launch();
    return cudaGetLastError();
}

}  // namespace gm
