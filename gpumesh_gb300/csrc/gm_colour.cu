// Independent vertex groups coloured on the GPU: the device order mode of
// the NodeGroups build.
//
// NodeGroups::determineGroups (DataStructures/NodeGroups.cpp:243-363) colours
// the vertices greedily in breadth-first order, one vertex at a time.  Here
// the same conflict relation (two vertices conflict when they share an
// element) is coloured by rounds of Jones-Plassmann: in each round every
// uncoloured movable vertex whose priority (a bijective hash of its index)
// beats every uncoloured conflicting vertex takes the lowest colour none of
// its coloured neighbours has.  Two vertices coloured in one round never
// conflict, and every round reads the colours of the previous round only
// (double buffer), so the result does not depend on thread scheduling.  The
// colours differ from the reference's greedy ones, so this is a separate
// relocation order; the classes, the (class, colour, valence) sort and the
// colour-major groups are then built on the host as for the reference order.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "gm_host.h"
#include "gm_internal.h"

namespace gm {

namespace {

__device__ __forceinline__ uint32_t colour_priority(uint32_t v)
{
    // a bijection of 32-bit integers (no two vertices tie)
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    v ^= v >> 16;
    return v;
}

struct ColourMesh
{
    uint32_t nv;
    const uint32_t* ve_off;
    const uint32_t* ve;
    const uint32_t* tets;
    const uint32_t* pris;
    const uint32_t* hexs;
    const int32_t* cid;
};

// one round: cin holds -1 for uncoloured movable vertices, a colour >= 0
// otherwise (fixed vertices -2, ignored); cout gets cin plus this round's
// colours.  done counts the vertices coloured; overflow flags a vertex whose
// neighbours use all 128 colours.
__global__ void __launch_bounds__(256) colour_round_kernel(ColourMesh m, const int* __restrict__ cin,
                                                           int* __restrict__ cout, unsigned int* done,
                                                           unsigned int* overflow)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nv) return;
    const int cv = cin[v];
    if (cv != -1)
    {
        cout[v] = cv;
        return;
    }
    const uint32_t pv = colour_priority(v);
    unsigned long long used[2] = {0ull, 0ull};
    bool is_max = true;
    for (uint32_t j = m.ve_off[v]; j < m.ve_off[v + 1] && is_max; ++j)
    {
        const uint32_t r = m.ve[j];
        const int type = (int)(r >> 30);
        const uint32_t id = r & kMaxElemId;
        const uint32_t* el;
        int k;
        if (type == kTypeTet) { el = m.tets + 4 * (size_t)id; k = 4; }
        else if (type == kTypePri) { el = m.pris + 6 * (size_t)id; k = 6; }
        else { el = m.hexs + 8 * (size_t)id; k = 8; }
        for (int q = 0; q < k; ++q)
        {
            const uint32_t w = el[q];
            if (w == v) continue;
            const int cw = cin[w];
            if (cw == -1)
            {
                if (colour_priority(w) > pv)
                {
                    is_max = false;
                    break;
                }
            }
            else if (cw >= 0)
                used[cw >> 6] |= 1ull << (cw & 63);
        }
    }
    if (!is_max)
    {
        cout[v] = -1;
        return;
    }
    int c;
    if (~used[0]) c = __ffsll(~used[0]) - 1;
    else if (~used[1]) c = 64 + __ffsll(~used[1]) - 1;
    else
    {
        atomicExch(overflow, 1u);
        c = 0;
    }
    cout[v] = c;
    atomicAdd(done, 1u);
}

}  // namespace

// Colours of every movable vertex (fixed vertices 0) by device
// Jones-Plassmann rounds.
void device_colours(const HostMeshView& in, const std::vector<uint32_t>& e_off, const std::vector<uint32_t>& e,
                    std::vector<int>& colour)
{
    const uint32_t nv = in.nv;
    DBuf<uint32_t> d_off, d_e, d_tets, d_pris, d_hexs;
    DBuf<int32_t> d_cid;
    DBuf<int> a, b;
    DBuf<unsigned int> ctr;
    cudaStream_t s = nullptr;
    upload(d_off, e_off.data(), e_off.size(), s);
    upload(d_e, e.data(), e.size(), s);
    upload(d_tets, in.tets, (size_t)in.nt * 4, s);
    upload(d_pris, in.pris, (size_t)in.np * 6, s);
    upload(d_hexs, in.hexs, (size_t)in.nh * 8, s);
    upload(d_cid, in.cid, nv, s);
    std::vector<int> init(nv);
    uint32_t movable = 0;
    for (uint32_t v = 0; v < nv; ++v)
    {
        init[v] = in.cid[v] < 0 ? -2 : -1;
        movable += in.cid[v] < 0 ? 0u : 1u;
    }
    upload(a, init.data(), nv, s);
    b.reserve(nv);
    ctr.reserve(2);
    GM_CUDA(cudaMemset(ctr.p, 0, 2 * sizeof(unsigned int)));
    ColourMesh cm{nv, d_off.p, d_e.p, d_tets.p, d_pris.p, d_hexs.p, d_cid.p};
    const unsigned blocks = (nv + 255) / 256;
    unsigned int h[2] = {0, 0};
    // each round colours at least the uncoloured vertex of highest priority,
    // so at most `movable` rounds; in practice O(log n)
    for (uint32_t round = 0; h[0] < movable; ++round)
    {
        if (round > movable) throw std::runtime_error("device colouring did not converge");
        colour_round_kernel<<<blocks, 256, 0, s>>>(cm, a.p, b.p, ctr.p, ctr.p + 1);
        note_launch();
        GM_CUDA(cudaGetLastError());
        GM_CUDA(cudaMemcpy(h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost));
        if (h[1]) throw ApiError(GM_ERR_UNSUPPORTED, "device colouring needs more than 128 colours");
        std::swap(a, b);
    }
    colour.resize(nv);
    GM_CUDA(cudaMemcpy(colour.data(), a.p, nv * sizeof(int), cudaMemcpyDeviceToHost));
    for (uint32_t v = 0; v < nv; ++v)
        if (colour[v] < 0) colour[v] = 0;  // fixed vertices
}

}  // namespace gm
