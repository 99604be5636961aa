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
__device__ __forceinline__ void eval_element(const MeshView& m, const Crew& crew, uint32_t i, float& mn, float& rs,
                                             int& nbad, int* hist)
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
    float qv;
    if (q.pos)
    {
        rs += q.v;
        qv = __frcp_rn(q.v);
    }
    else
    {
        ++nbad;
        qv = q.v;
    }
    mn = fminf(mn, qv);
    int b = qv > 0.f ? min((int)(qv * 20.f), 19) : 0;
    atomicAdd(&hist[b], 1);
}

template <int VAR, int SET>
__global__ void __launch_bounds__(kEvalThreads) evaluate_kernel(MeshView m, Crew crew, EvalPartial* parts)
{
    __shared__ int hist[20];
    __shared__ float wmin[kEvalThreads / 32];
    __shared__ double wsum[kEvalThreads / 32];
    __shared__ int wbad[kEvalThreads / 32];
    if (threadIdx.x < 20) hist[threadIdx.x] = 0;
    __syncthreads();
    float mn = 1.0f, rs = 0.f;
    int nbad = 0;
    const uint32_t total = m.nt + m.np + m.nh;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        eval_element<VAR, SET>(m, crew, i, mn, rs, nbad, hist);
    double ds = rs;
    for (int o = 16; o > 0; o >>= 1)
    {
        ds += __shfl_xor_sync(0xffffffffu, ds, o);
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
    {
        wmin[w] = mn;
        wsum[w] = ds;
        wbad[w] = nbad;
    }
    __syncthreads();
    if (threadIdx.x < 32)
    {
        EvalPartial* p = &parts[blockIdx.x];
        if (threadIdx.x < 20) p->hist[threadIdx.x] = hist[threadIdx.x];
        if (threadIdx.x == 0)
        {
            float bmin = wmin[0];
            double bsum = wsum[0];
            int bbad = wbad[0];
            for (int k = 1; k < kEvalThreads / 32; ++k)
            {
                bmin = fminf(bmin, wmin[k]);
                bsum += wsum[k];
                bbad += wbad[k];
            }
            p->min = bmin;
            p->rsum = bsum;
            p->nbad = bbad;
            p->pad = 0;
        }
    }
}

__global__ void __launch_bounds__(256) evaluate_finalize_kernel(const EvalPartial* parts, int nparts, uint32_t count,
                                                                 Quality* out)
{
    __shared__ double s_sum[256];
    __shared__ float s_min[256];
    __shared__ unsigned long long s_bad[256];
    __shared__ unsigned long long s_hist[8][20];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double sum = 0;
    float mn = 1.0f;
    unsigned long long bad = 0;
    for (int i = t; i < nparts; i += 256)
    {
        sum += parts[i].rsum;
        mn = fminf(mn, parts[i].min);
        bad += (unsigned long long)parts[i].nbad;
    }
    s_sum[t] = sum;
    s_min[t] = mn;
    s_bad[t] = bad;
    // histogram: warp w sums partials w, w + 8, ...; lane b < 20 owns bucket b
    unsigned long long h = 0;
    if (lane < 20)
        for (int i = w; i < nparts; i += 8) h += (unsigned long long)parts[i].hist[lane];
    if (lane < 20) s_hist[w][lane] = h;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1)
    {
        if (t < s)
        {
            s_sum[t] += s_sum[t + s];
            s_min[t] = fminf(s_min[t], s_min[t + s]);
            s_bad[t] += s_bad[t + s];
        }
        __syncthreads();
    }
    if (t < 20)
    {
        unsigned long long hb = 0;
        for (int k = 0; k < 8; ++k) hb += s_hist[k][t];
        out->buckets[t] = hb;
    }
    if (t == 0)
    {
        out->min = (double)s_min[0];
        out->nbad = s_bad[0];
        out->inv_sum = s_bad[0] ? (double)INFINITY : s_sum[0];
        out->count = count;
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
static void launch_eval_t(const MeshView& m, const Crew& crew, EvalPartial* parts, int nblocks, cudaStream_t s)
{
    evaluate_kernel<VAR, SET><<<nblocks, kEvalThreads, 0, s>>>(m, crew, parts);
}

cudaError_t launch_evaluate(int variant, int maxk, const MeshView& m, const Crew& crew, EvalPartial* parts,
                            int nblocks, Quality* out, cudaStream_t s)
{
    switch (variant)
    {
    case kVarMRFree:
        if (maxk == 4) launch_eval_t<kVarMRFree, 4>(m, crew, parts, nblocks, s);
        else if (maxk == 9) launch_eval_t<kVarMRFree, 9>(m, crew, parts, nblocks, s);
        else launch_eval_t<kVarMRFree, 8>(m, crew, parts, nblocks, s);
        break;
    case kVarMCDiag:
        if (maxk == 4) launch_eval_t<kVarMCDiag, 4>(m, crew, parts, nblocks, s);
        else launch_eval_t<kVarMCDiag, 8>(m, crew, parts, nblocks, s);
        break;
    case kVarMRWise: launch_eval_t<kVarMRWise, 8>(m, crew, parts, nblocks, s); break;
    default:
        if (maxk == 4) launch_eval_t<kVarMC, 4>(m, crew, parts, nblocks, s);
        else launch_eval_t<kVarMC, 8>(m, crew, parts, nblocks, s);
        break;
    }
    evaluate_finalize_kernel<<<1, 256, 0, s>>>(parts, nblocks, m.nt + m.np + m.nh, out);
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

size_t patch_smem_per_warp(int ks, int maxe)
{
    return (size_t)ks * maxe * sizeof(float4) + (size_t)maxe * sizeof(int) + kMaxCand * sizeof(float4) +
           kMaxCand * sizeof(float);
}

}  // namespace gm
