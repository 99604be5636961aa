// Launches of the batched kernels (gm_batch_kernels.cuh) for one of the
// general-metric variants: the metric-wise mean ratio (kVarMRWise).  The general-metric evaluation needs
// more registers than the metric-free and diagonal-metric variants, so these
// kernels are compiled in units of their own (one per variant, built in
// parallel), with launch bounds of one 256-thread block per SM, instead of
// inflating the other variants' build.
#include <cuda_runtime.h>

#include "gm_batch_kernels.cuh"

namespace gm {

template <int SMOOTHER>
static cudaError_t launch_one(const BatchArgs& a, const SmoothParams& sp, int maxk, int wpb, int cps, int sm_count,
                              cudaStream_t s)
{
    return maxk == 4 ? launch_batch_t<SMOOTHER, kVarMRWise, 4>(a, sp, wpb, cps, sm_count, s)
                     : launch_batch_t<SMOOTHER, kVarMRWise, 8>(a, sp, wpb, cps, sm_count, s);
}

cudaError_t launch_batch_relocate_mrwise(int smoother, const BatchArgs& a, const SmoothParams& sp, int maxk, int wpb, int cps,
                          int sm_count, cudaStream_t s)
{
    switch (smoother)
    {
    case kSmoothNM: return launch_one<kSmoothNM>(a, sp, maxk, wpb, cps, sm_count, s);
    case kSmoothGD: return launch_one<kSmoothGD>(a, sp, maxk, wpb, cps, sm_count, s);
    case kSmoothSpawn: return launch_one<kSmoothSpawn>(a, sp, maxk, wpb, cps, sm_count, s);
    default: return launch_one<kSmoothGetme>(a, sp, maxk, wpb, cps, sm_count, s);
    }
}

cudaError_t launch_batch_eval_mrwise(const BatchMesh* meshes, const EvalBlock* blocks, uint32_t nblocks, EvalPartial* parts, int maxk,
                      cudaStream_t s)
{
    if (maxk == 4) launch_batch_eval_t<kVarMRWise, 4>(meshes, blocks, nblocks, parts, s);
    else launch_batch_eval_t<kVarMRWise, 8>(meshes, blocks, nblocks, parts, s);
    return cudaGetLastError();
}

}  // namespace gm
