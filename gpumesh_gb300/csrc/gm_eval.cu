// Quality evaluation: a coalesced stream over the element arrays, vertex
// positions gathered through L2, and a fused min / harmonic-sum / 20-bucket
// histogram reduction (AbstractEvaluator::evaluateMeshQualityThread,
// Evaluators/AbstractEvaluator.cpp:404-453; QualityHistogram::add/merge,
// DataStructures/QualityHistogram.cpp:63-92).
//
// Each thread accumulates 1/q of its elements in FP32; warps, blocks and the
// final reduction sum in FP64 in a fixed order, so the result does not depend
// on scheduling.  The bucket of a non-positive quality is 0.
#include <cuda_runtime.h>

#include "gm_launch.h"

namespace gm {

constexpr int kEvalThreads = 256;

// SET: 4 = tets only, 8 = any element types, 9 = hexes only
template <int VAR, int SET>
__device__ __forceinline__ void eval_element(const MeshView& m, const Crew& crew, uint32_t i, EvalAcc& acc, int* hist)
{
    constexpr int MAXK = SET == 4 ? 4 : 8;
    int type;
    uint32_t id;
    if (SET == 9) { type = kHex; id = i; }
    else if (SET == 4 || i < m.nt) { type = kTet; id = i; }
    else if (i < m.nt + m.np) { type = kPri; id = i - m.nt; }
    else { type = kHex; id = i - m.nt - m.np; }
    V3<float> p[MAXK];
    if (SET == 9)
    {
        const uint4 a = __ldg(&m.hexs[2 * (size_t)id]), b = __ldg(&m.hexs[2 * (size_t)id + 1]);
        p[0] = to<float>(__ldg(&m.pos[a.x]));
        p[1] = to<float>(__ldg(&m.pos[a.y]));
        p[2] = to<float>(__ldg(&m.pos[a.z]));
        p[3] = to<float>(__ldg(&m.pos[a.w]));
        p[4] = to<float>(__ldg(&m.pos[b.x]));
        p[5] = to<float>(__ldg(&m.pos[b.y]));
        p[6] = to<float>(__ldg(&m.pos[b.z]));
        p[7] = to<float>(__ldg(&m.pos[b.w]));
    }
    else if (MAXK == 4)
    {
        uint4 t = __ldg(&m.tets[id]);
        p[0] = to<float>(__ldg(&m.pos[t.x]));
        p[1] = to<float>(__ldg(&m.pos[t.y]));
        p[2] = to<float>(__ldg(&m.pos[t.z]));
        p[3] = to<float>(__ldg(&m.pos[t.w]));
    }
    else
    {
        uint32_t vid[8];
        elem_vertices(m, type, id, vid);
        int n = type_size(type);
#pragma unroll
        for (int k = 0; k < MAXK; ++k) p[k] = to<float>(__ldg(&m.pos[vid[k < n ? k : 0]]));
    }
    EQ<float> q = SET == 9 ? (VarTraits<VAR>::mean_ratio ? mr_hex<VAR, float>(crew, p)
                                                          : elem_quality<VAR, MAXK, float>(crew, kHex, p))
                           : elem_quality<VAR, MAXK, float>(crew, type, p);
    acc.add(q, hist);
}

constexpr int kEvalWarps = kEvalThreads / 32;

// Block-wide sum / min / sum over kEvalThreads threads in a fixed order;
// thread 0 gets the results.
__device__ __forceinline__ void block_reduce(double& sum, float& mn, int& bad, double* wsum, float* wmin, int* wbad)
{
    for (int o = 16; o > 0; o >>= 1)
    {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
    {
        wsum[w] = sum;
        wmin[w] = mn;
        wbad[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 1; k < kEvalWarps; ++k)
        {
            sum += wsum[k];
            mn = fminf(mn, wmin[k]);
            bad += wbad[k];
        }
}

// One launch per evaluation: every block reduces its elements to a partial;
// the last block to finish (a ticket taken after a release fence) reduces
// all partials in a fixed order and writes the Quality, so the result does
// not depend on which block finishes last.  atomicInc wraps the ticket back
// to 0, so the scratch is ready for the next launch.
template <int VAR, int SET>
__global__ void __launch_bounds__(kEvalThreads) evaluate_kernel(MeshView m, Crew crew, EvalPartial* parts,
                                                                Quality* out)
{
    __shared__ int hist[20];
    __shared__ float wmin[kEvalWarps];
    __shared__ double wsum[kEvalWarps];
    __shared__ int wbad[kEvalWarps];
    __shared__ unsigned int whist[kEvalWarps][20];
    __shared__ bool last;
    if (threadIdx.x < 20) hist[threadIdx.x] = 0;
    __syncthreads();
    EvalAcc acc;
    const uint32_t total = m.nt + m.np + m.nh;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        eval_element<VAR, SET>(m, crew, i, acc, hist);
    double sum = acc.rs;
    float mn = acc.min_quality();
    int bad = acc.nbad;
    block_reduce(sum, mn, bad, wsum, wmin, wbad);
    const int nb = gridDim.x;
    const EvalScratch S = eval_scratch(parts, nb);
    if (threadIdx.x < 20) S.hist[threadIdx.x * nb + blockIdx.x] = hist[threadIdx.x];
    if (threadIdx.x == 0)
    {
        S.rsum[blockIdx.x] = sum;
        S.min[blockIdx.x] = mn;
        S.nbad[blockIdx.x] = bad;
    }
    __threadfence();  // every writer publishes its part of the partial
    __syncthreads();
    if (threadIdx.x == 0) last = atomicInc(S.ticket, (unsigned int)nb - 1u) == (unsigned int)nb - 1u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: every partial, coalesced, in a fixed order
    double tsum = 0;
    float tmin = 1.0f;
    int tbad = 0;
    unsigned int h[20];
#pragma unroll
    for (int b = 0; b < 20; ++b) h[b] = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
    {
        tsum += __ldcg(&S.rsum[i]);
        tmin = fminf(tmin, __ldcg(&S.min[i]));
        tbad += __ldcg(&S.nbad[i]);
#pragma unroll
        for (int b = 0; b < 20; ++b) h[b] += (unsigned int)__ldcg(&S.hist[b * nb + i]);
    }
    __syncthreads();  // the shared reduction arrays are reused
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int b = 0; b < 20; ++b)
    {
        unsigned int x = h[b];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) whist[w][b] = x;
    }
    block_reduce(tsum, tmin, tbad, wsum, wmin, wbad);
    if (threadIdx.x < 20)
    {
        unsigned long long hb = 0;
        for (int k = 0; k < kEvalWarps; ++k) hb += whist[k][threadIdx.x];
        out->buckets[threadIdx.x] = hb;
    }
    if (threadIdx.x == 0)
    {
        out->min = (double)tmin;
        out->nbad = (unsigned long long)tbad;
        out->inv_sum = tbad ? (double)INFINITY : tsum;
        out->count = total;
    }
}

int evaluate_blocks(uint32_t total, int sm_count)
{
    long need = ((long)total + kEvalThreads - 1) / kEvalThreads;
    long cap = (long)sm_count * 8;
    long n = need < cap ? need : cap;
    return n < 1 ? 1 : (int)n;
}

template <int VAR, int SET>
static void launch_eval_t(const MeshView& m, const Crew& crew, EvalPartial* parts, int nblocks, Quality* out,
                          cudaStream_t s)
{
    evaluate_kernel<VAR, SET><<<nblocks, kEvalThreads, 0, s>>>(m, crew, parts, out);
}

cudaError_t launch_evaluate(int variant, int maxk, const MeshView& m, const Crew& crew, EvalPartial* parts,
                            int nblocks, Quality* out, cudaStream_t s)
{
    switch (variant)
    {
    case kVarMRFree:
        if (maxk == 4) launch_eval_t<kVarMRFree, 4>(m, crew, parts, nblocks, out, s);
        else if (maxk == 9) launch_eval_t<kVarMRFree, 9>(m, crew, parts, nblocks, out, s);
        else launch_eval_t<kVarMRFree, 8>(m, crew, parts, nblocks, out, s);
        break;
    case kVarMCDiag:
        if (maxk == 4) launch_eval_t<kVarMCDiag, 4>(m, crew, parts, nblocks, out, s);
        else launch_eval_t<kVarMCDiag, 8>(m, crew, parts, nblocks, out, s);
        break;
    case kVarMRWise: launch_eval_t<kVarMRWise, 8>(m, crew, parts, nblocks, out, s); break;
    default:
        if (maxk == 4) launch_eval_t<kVarMC, 4>(m, crew, parts, nblocks, out, s);
        else launch_eval_t<kVarMC, 8>(m, crew, parts, nblocks, out, s);
        break;
    }
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) ffma_probe_kernel(int iters, float* sink)
{
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i)
    {
        a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
        a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
    float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678f) sink[threadIdx.x & 1023] = r;
}

cudaError_t launch_ffma_probe(int blocks, int threads, int iters, float* sink, cudaStream_t s)
{
    ffma_probe_kernel<<<blocks, threads, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

size_t patch_smem_per_warp(int maxk, int maxe)
{
    return (size_t)patch_slots(maxk) * maxe * sizeof(float4) + (size_t)maxe * sizeof(int) +
           kMaxCand * sizeof(float4) + kMaxCand * sizeof(float);
}

}  // namespace gm
