// Launchers of the device kernels (defined in the .cu files).
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "gm_kernels.cuh"

namespace gm {

// Launch a kernel that begins with GM_PDL_ENTRY with programmatic stream
// serialisation (programmatic dependent launch) unless the stream is being
// captured: its launch and block scheduling overlap the previous kernel's
// last blocks, and its first instruction waits for that kernel's completion
// and memory, so nothing is read early.  A captured launch keeps plain graph
// edges.  Returns the launch's status and clears it from the last error.
template <class... P, class... A>
inline cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t qe = cudaStreamIsCapturing(s, &cap);
    if (qe == cudaSuccess && cap == cudaStreamCaptureStatusNone)
    {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    else if (qe != cudaSuccess)
        cudaGetLastError();  // the query's own error (a capture elsewhere): plain edges
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
    const cudaError_t last = cudaGetLastError();
    return e != cudaSuccess ? e : last;
}

// Kernel launches made by this library, reported by gm_launch_count.  Every
// launch site calls note_launch() after its launch.  Outside stream capture
// that adds one to the process-wide count; while a CaptureTally is open on
// the calling thread (a capture begun by this library) it adds to the
// tally, and the graph's owner adds the tally each time the graph runs.
void note_launch();
void add_launches(unsigned long long n);
struct CaptureTally
{
    unsigned long long kernels = 0;
    CaptureTally* prev;
    CaptureTally();
    ~CaptureTally();
};

// shared memory of one warp's patch; maxk: 4 = tets only, 8 = any element type
size_t patch_smem_per_warp(int maxk, int maxe);

int evaluate_blocks(uint32_t total, int sm_count);
// maxk: 4 = tets only, 8 = any element types, 9 = hexes only
cudaError_t launch_evaluate(int variant, int maxk, const MeshView& m, const Crew& crew, EvalPartial* parts,
                            int nblocks, Quality* out, cudaStream_t s);

// one relocation launch over one independent group
struct RelocLaunch
{
    int variant;  // kVarMRFree / kVarMRWise / kVarMC
    int maxk;     // 4: tets only, 8: any element type
    MeshView m;
    Crew crew;
    SmoothParams sp;
    const uint32_t* members;
    uint32_t count;
    int maxe;
    int max_incident;  // the largest number of elements around a vertex (maxe is it padded)
    int warps_per_block;
    int sm_count;
    Counters* ctr;
    Deferred def;
    uint32_t slot_base;  // this group's region of the deferred arrays
    cudaStream_t stream;
};

cudaError_t launch_relocate_nm(const RelocLaunch& L);
cudaError_t launch_relocate_gd(const RelocLaunch& L);
cudaError_t launch_relocate_spawn(const RelocLaunch& L);
cudaError_t launch_relocate_spring(const RelocLaunch& L);
cudaError_t launch_relocate_qlaplace(const RelocLaunch& L);
cudaError_t launch_getme_update(const RelocLaunch& L, const float4* corners);
// FP64 acceptance of the vertices the preceding launch deferred
cudaError_t launch_accept(const RelocLaunch& L);

cudaError_t launch_getme_elements(int variant, const MeshView& m, const Crew& crew, float lambda, float4* corners,
                                  int sm_count, cudaStream_t s);

// FP32 peak probe: 8 independent FFMA chains per thread
cudaError_t launch_ffma_probe(int blocks, int threads, int iters, float* sink, cudaStream_t s);

}  // namespace gm
