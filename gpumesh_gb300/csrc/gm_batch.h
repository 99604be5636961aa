// Device tables of the batched path (gm_batch.cu) and their launchers.
#pragma once

#include <cuda_runtime.h>

#include "gm_kernels.cuh"

namespace gm {

// one mesh of a batch: views of its own device buffers
struct BatchMesh
{
    MeshView view;
    Crew crew;
    const uint32_t* members;  // colour-major relocation order
    const float4* corners;    // GETMe element corners (update pass)
    uint32_t nmembers;        // vertices relocated per pass
    uint32_t pad;
};

// the vertices of colour g of one mesh: members[member_begin, +count); they
// may start once `need` vertices of that mesh (its colours < g) are done
struct Segment
{
    uint32_t mesh, member_begin, count, need;
};

struct BatchCtl
{
    unsigned int next;   // work-queue head
    unsigned int error;  // non-zero: a dependency wait gave up
    unsigned long long t0;  // %globaltimer when the first warp started
};

struct BatchArgs
{
    const BatchMesh* meshes;
    const Segment* segs;
    const uint32_t* seg_start;  // nseg + 1 prefix sums of segment counts
    uint32_t nseg, total;
    unsigned int* done;  // per mesh: vertices finished this pass
    BatchCtl* ctl;
    Counters* ctr;
    unsigned long long* finish;  // per mesh: %globaltimer when its last vertex finished
    int maxe;
    unsigned long long spin_limit;
};

// a contiguous element range of one mesh evaluated by one block
struct EvalBlock
{
    uint32_t mesh, begin, end, pad;
};

cudaError_t launch_batch_relocate(int smoother, const BatchArgs& a, const SmoothParams& sp, int variant, int maxk,
                                  int wpb, int cps, int sm_count, cudaStream_t s);
cudaError_t launch_batch_evaluate(const BatchMesh* meshes, uint32_t nmesh, const EvalBlock* blocks, uint32_t nblocks,
                                  const uint32_t* mesh_block, EvalPartial* parts, Quality* out, int variant, int maxk,
                                  cudaStream_t s);
// the general-metric variants, compiled apart (gm_batch_general_mc.cu:
// metric conformity under the analytic and background-mesh samplers;
// gm_batch_general_mrwise.cu: the metric-wise mean ratio) with one
// 256-thread block per SM, the register budget of their metric evaluation
cudaError_t launch_batch_relocate_mc(int smoother, const BatchArgs& a, const SmoothParams& sp, int maxk, int wpb,
                                     int cps, int sm_count, cudaStream_t s);
cudaError_t launch_batch_relocate_mrwise(int smoother, const BatchArgs& a, const SmoothParams& sp, int maxk, int wpb,
                                         int cps, int sm_count, cudaStream_t s);
cudaError_t launch_batch_eval_mc(const BatchMesh* meshes, const EvalBlock* blocks, uint32_t nblocks,
                                 EvalPartial* parts, int maxk, cudaStream_t s);
cudaError_t launch_batch_eval_mrwise(const BatchMesh* meshes, const EvalBlock* blocks, uint32_t nblocks,
                                     EvalPartial* parts, int maxk, cudaStream_t s);

}  // namespace gm
