// LocalSampler's background mesh on the device.
//
// The reference's LocalSampler (Samplers/LocalSampler.cpp) samples the metric
// by walking a background tet mesh -- the mesh as it was when the sampling was
// last updated, split into tets -- and interpolating the metric stored at its
// vertices.  Its CUDA driver receives that mesh from the host
// (updateCudaLocalTets / updateCudaRefVerts / updateCudaRefMetrics,
// resources/cuda/Sampling/Local.cu:143-230) and starts each walk at a cached
// tet carried by the vertex being measured.
//
// Here the background is either given in that form (gm_mesh_set_local_background)
// or built from the device mesh as LocalSampler::updateAnalyticalMetric does
// (:193-203, the analytic metric at every vertex; buildBackgroundMesh
// :352-429, the split into tets and the face neighbours).  Instead of the
// per-vertex cache, a uniform grid over the background's bounding box names,
// for every cell, a tet near it, so that a walk starts a step or two from its
// goal whatever the vertex did since the background was built.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "gm_host.h"

namespace gm {

namespace {

constexpr uint32_t kNoTet = 0xffffffffu;

// MeshTet::tris (DataStructures/Mesh.cpp:30-35): the face opposite each vertex
constexpr int kFace[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};

// Prism and hex vertex rotations that bring the smallest vertex id first, and
// the hex cases by diagonal pattern (Tetrahedralizer.h:9-34).  The split of
// a face follows its smallest vertex id, so neighbouring elements split their
// shared faces alike and the background is conforming.
constexpr uint8_t kPriRot[6][6] = {{0, 1, 2, 3, 4, 5}, {1, 2, 0, 4, 5, 3}, {2, 0, 1, 5, 3, 4},
                                   {3, 5, 4, 0, 2, 1}, {4, 3, 5, 1, 0, 2}, {5, 4, 3, 2, 1, 0}};
constexpr uint8_t kHexRot[8][8] = {{0, 1, 2, 3, 4, 5, 6, 7}, {1, 0, 4, 5, 2, 3, 7, 6}, {2, 1, 5, 6, 3, 0, 4, 7},
                                   {3, 0, 1, 2, 7, 4, 5, 6}, {4, 0, 3, 7, 5, 1, 2, 6}, {5, 1, 0, 4, 6, 2, 3, 7},
                                   {6, 2, 1, 5, 7, 3, 0, 4}, {7, 3, 2, 6, 4, 0, 1, 5}};
// rotation of the hex about its 0-6 diagonal that brings the diagonal
// pattern to a canonical one: 0, 120 or 240 degrees
constexpr uint16_t kHexTurn[8] = {0, 120, 240, 0, 0, 240, 120, 0};

// Tetrahedralizer.h:37-200: tets as they are, a prism into 3 tets, a hex into
// 5 or 6 by the diagonals its faces take.  first[e]: element e's first tet
// (tets, then prisms, then hexes), the cache its measures start walks from.
void split_elements(const std::vector<uint4>& tets, const std::vector<uint32_t>& pris, const std::vector<uint4>& hexs,
                    std::vector<uint4>& out, std::vector<uint32_t>& first)
{
    const size_t nt = tets.size(), np = pris.size() / 6, nh = hexs.size() / 2;
    out.clear();
    out.reserve(nt + 3 * np + 6 * nh);
    first.resize(nt + np + nh);
    out.insert(out.end(), tets.begin(), tets.end());
    for (size_t i = 0; i < nt; ++i) first[i] = (uint32_t)i;
    auto push = [&](uint32_t a, uint32_t b, uint32_t c, uint32_t d) { out.push_back(make_uint4(a, b, c, d)); };
    for (size_t i = 0; i < np; ++i)
    {
        first[nt + i] = (uint32_t)out.size();
        const uint32_t* e = &pris[6 * i];
        int s = 0;
        for (int k = 1; k < 6; ++k)
            if (e[k] < e[s]) s = k;
        uint32_t v[6];
        for (int k = 0; k < 6; ++k) v[k] = e[kPriRot[s][k]];
        if (std::min(v[1], v[5]) < std::min(v[2], v[4]))
        {
            push(v[0], v[1], v[2], v[5]);
            push(v[0], v[1], v[5], v[4]);
            push(v[0], v[4], v[5], v[3]);
        }
        else
        {
            push(v[0], v[1], v[2], v[4]);
            push(v[0], v[4], v[2], v[5]);
            push(v[0], v[4], v[5], v[3]);
        }
    }
    for (size_t i = 0; i < nh; ++i)
    {
        first[nt + np + i] = (uint32_t)out.size();
        const uint4 lo = hexs[2 * i], hi = hexs[2 * i + 1];
        const uint32_t e[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        int s = 0;
        for (int k = 1; k < 8; ++k)
            if (e[k] < e[s]) s = k;
        uint32_t v[8];
        for (int k = 0; k < 8; ++k) v[k] = e[kHexRot[s][k]];
        unsigned diag = 0;
        if (std::min(v[1], v[6]) < std::min(v[2], v[5])) diag |= 4u;
        if (std::min(v[3], v[6]) < std::min(v[2], v[7])) diag |= 2u;
        if (std::min(v[4], v[6]) < std::min(v[5], v[7])) diag |= 1u;
        if (kHexTurn[diag] == 120)
        {
            const uint32_t a = v[1], b = v[5];
            v[1] = v[4], v[4] = v[3], v[3] = a;
            v[5] = v[7], v[7] = v[2], v[2] = b;
        }
        else if (kHexTurn[diag] == 240)
        {
            const uint32_t a = v[1], b = v[5];
            v[1] = v[3], v[3] = v[4], v[4] = a;
            v[5] = v[2], v[2] = v[7], v[7] = b;
        }
        switch (__builtin_popcount(diag))
        {
        case 0:
            push(v[0], v[1], v[2], v[5]);
            push(v[0], v[2], v[7], v[5]);
            push(v[0], v[2], v[3], v[7]);
            push(v[0], v[5], v[7], v[4]);
            push(v[2], v[7], v[5], v[6]);
            break;
        case 1:
            push(v[0], v[5], v[7], v[4]);
            push(v[0], v[1], v[7], v[5]);
            push(v[1], v[6], v[7], v[5]);
            push(v[0], v[7], v[2], v[3]);
            push(v[0], v[7], v[1], v[2]);
            push(v[1], v[7], v[6], v[2]);
            break;
        case 2:
            push(v[0], v[4], v[5], v[6]);
            push(v[0], v[3], v[7], v[6]);
            push(v[0], v[7], v[4], v[6]);
            push(v[0], v[1], v[2], v[5]);
            push(v[0], v[3], v[6], v[2]);
            push(v[0], v[6], v[5], v[2]);
            break;
        default:
            push(v[0], v[2], v[3], v[6]);
            push(v[0], v[3], v[7], v[6]);
            push(v[0], v[7], v[4], v[6]);
            push(v[0], v[5], v[6], v[4]);
            push(v[1], v[5], v[6], v[0]);
            push(v[1], v[6], v[2], v[0]);
            break;
        }
    }
}

// The two tets of every shared face as neighbours across it
// (buildBackgroundMesh pairs a face's first and second owner): faces bucketed
// by their smallest vertex, sorted within the bucket by the other two and by
// (tet, side), and equal consecutive faces paired.
void face_neighbours(const std::vector<uint4>& tv, uint32_t nref, std::vector<uint4>& tn)
{
    const size_t n = tv.size();
    tn.assign(n, make_uint4(kNoTet, kNoTet, kNoTet, kNoTet));
    struct Rec
    {
        uint32_t b, c, ts;
    };
    std::vector<uint32_t> off((size_t)nref + 1, 0);
    auto key = [&](size_t t, int s, uint32_t& a, uint32_t& b, uint32_t& c) {
        const uint32_t v[4] = {tv[t].x, tv[t].y, tv[t].z, tv[t].w};
        uint32_t x = v[kFace[s][0]], y = v[kFace[s][1]], z = v[kFace[s][2]];
        if (x > y) std::swap(x, y);
        if (y > z) std::swap(y, z);
        if (x > y) std::swap(x, y);
        a = x, b = y, c = z;
    };
    for (size_t t = 0; t < n; ++t)
        for (int s = 0; s < 4; ++s)
        {
            uint32_t a, b, c;
            key(t, s, a, b, c);
            ++off[a + 1];
        }
    for (size_t i = 0; i < nref; ++i) off[i + 1] += off[i];
    std::vector<Rec> rec(4 * n);
    std::vector<uint32_t> fill(off.begin(), off.end() - 1);
    for (size_t t = 0; t < n; ++t)
        for (int s = 0; s < 4; ++s)
        {
            uint32_t a, b, c;
            key(t, s, a, b, c);
            rec[fill[a]++] = Rec{b, c, (uint32_t)(4 * t + s)};
        }
    auto set = [&](uint32_t ts, uint32_t other) {
        uint4& q = tn[ts >> 2];
        switch (ts & 3u)
        {
        case 0: q.x = other; break;
        case 1: q.y = other; break;
        case 2: q.z = other; break;
        default: q.w = other; break;
        }
    };
    for (size_t a = 0; a < nref; ++a)
    {
        Rec* lo = rec.data() + off[a];
        Rec* hi = rec.data() + off[a + 1];
        std::sort(lo, hi, [](const Rec& x, const Rec& y) {
            if (x.b != y.b) return x.b < y.b;
            if (x.c != y.c) return x.c < y.c;
            return x.ts < y.ts;
        });
        for (Rec* r = lo; r + 1 < hi;)
        {
            if (r[0].b == r[1].b && r[0].c == r[1].c)
            {
                set(r[0].ts, r[1].ts >> 2);
                set(r[1].ts, r[0].ts >> 2);
                r += 2;
            }
            else
                ++r;
        }
    }
}

// start grid: about one background tet per cell; each cell holds the first tet
// whose centroid falls in it, empty cells the tet of the nearest filled cell
// (breadth-first over face-adjacent cells)
void start_grid(const std::vector<uint4>& tv, const std::vector<double>& pd, LocalField& f,
                std::vector<uint32_t>& cell)
{
    const size_t nref = pd.size() / 3;
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    for (size_t v = 0; v < nref; ++v)
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], pd[3 * v + k]);
            hi[k] = std::max(hi[k], pd[3 * v + k]);
        }
    double ext[3], emax = 0.0;
    for (int k = 0; k < 3; ++k)
    {
        ext[k] = hi[k] - lo[k];
        emax = std::max(emax, ext[k]);
    }
    if (!(emax > 0.0)) emax = 1.0;
    for (int k = 0; k < 3; ++k) ext[k] = std::max(ext[k], 1e-6 * emax);
    const double target = (double)std::max<size_t>(tv.size(), 1);
    double h = std::cbrt(ext[0] * ext[1] * ext[2] / target);
    for (;;)
    {
        size_t cells = 1;
        for (int k = 0; k < 3; ++k)
        {
            f.g[k] = (int)std::min(1024.0, std::max(1.0, std::ceil(ext[k] / h)));
            cells *= (size_t)f.g[k];
        }
        if (cells <= 2 * (size_t)target + 64) break;
        h *= 1.25;
    }
    for (int k = 0; k < 3; ++k)
    {
        f.lo[k] = lo[k];
        f.inv_h[k] = f.g[k] / ext[k];
    }
    const size_t gx = f.g[0], gy = f.g[1], gz = f.g[2];
    cell.assign(gx * gy * gz, kNoTet);
    auto index = [&](double x, int k) {
        const double q = (x - f.lo[k]) * f.inv_h[k];
        return q >= f.g[k] ? f.g[k] - 1 : (q > 0.0 ? (int)q : 0);
    };
    std::deque<size_t> queue;
    for (size_t t = 0; t < tv.size(); ++t)
    {
        const uint32_t v[4] = {tv[t].x, tv[t].y, tv[t].z, tv[t].w};
        int ci[3];
        for (int k = 0; k < 3; ++k)
            ci[k] = index(0.25 * (pd[3 * v[0] + k] + pd[3 * v[1] + k] + pd[3 * v[2] + k] + pd[3 * v[3] + k]), k);
        const size_t c = ((size_t)ci[2] * gy + ci[1]) * gx + ci[0];
        if (cell[c] == kNoTet)
        {
            cell[c] = (uint32_t)t;
            queue.push_back(c);
        }
    }
    while (!queue.empty())
    {
        const size_t c = queue.front();
        queue.pop_front();
        const size_t x = c % gx, y = (c / gx) % gy, z = c / (gx * gy);
        const size_t nb[6][3] = {{x - 1, y, z}, {x + 1, y, z}, {x, y - 1, z}, {x, y + 1, z}, {x, y, z - 1}, {x, y, z + 1}};
        for (const auto& q : nb)
        {
            if (q[0] >= gx || q[1] >= gy || q[2] >= gz) continue;  // also catches the wrapped -1
            const size_t d = (q[2] * gy + q[1]) * gx + q[0];
            if (cell[d] == kNoTet)
            {
                cell[d] = cell[c];
                queue.push_back(d);
            }
        }
    }
}

__global__ void __launch_bounds__(256) vertex_metrics_kernel(Crew c, const double* __restrict__ pd, uint32_t n,
                                                             double* __restrict__ md, float* __restrict__ mf)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const Sym3<double> M = analytic_metric<double>(c, V3<double>{pd[3 * (size_t)v], pd[3 * (size_t)v + 1],
                                                                  pd[3 * (size_t)v + 2]});
    const double m[6] = {M.xx, M.yy, M.zz, M.xy, M.xz, M.yz};
    for (int j = 0; j < 6; ++j)
    {
        md[6 * (size_t)v + j] = m[j];
        mf[6 * (size_t)v + j] = (float)m[j];
    }
}

// uploads the background; the vertex metrics are the given ones, or the
// analytic metric computed on the device when metrics_host is null; first:
// the element caches (empty: none), for nt tets and np prisms
std::shared_ptr<LocalBackground> finish(const std::vector<uint4>& tv, const std::vector<uint4>& tn,
                                        const std::vector<double>& pd, const double* metrics_host, const Crew& crew,
                                        const std::vector<uint32_t>& first, uint32_t nt, uint32_t np, cudaStream_t s)
{
    auto bg = std::make_shared<LocalBackground>();
    const uint32_t nref = (uint32_t)(pd.size() / 3);
    bg->nbg = (uint32_t)tv.size();
    bg->nref = nref;
    LocalField f{};
    std::vector<uint32_t> cell;
    start_grid(tv, pd, f, cell);
    std::vector<float4> pf(nref);
    for (uint32_t v = 0; v < nref; ++v)
        pf[v] = make_float4((float)pd[3 * v], (float)pd[3 * v + 1], (float)pd[3 * v + 2], 0.f);
    upload(bg->tv, tv.data(), tv.size(), s);
    upload(bg->tn, tn.data(), tn.size(), s);
    upload(bg->pf, pf.data(), pf.size(), s);
    upload(bg->pd, pd.data(), pd.size(), s);
    upload(bg->cell, cell.data(), cell.size(), s);
    if (!first.empty()) upload(bg->ecache, first.data(), first.size(), s);
    bg->md.reserve((size_t)6 * nref);
    bg->mf.reserve((size_t)6 * nref);
    if (metrics_host)
    {
        std::vector<float> m32((size_t)6 * nref);
        for (size_t i = 0; i < m32.size(); ++i) m32[i] = (float)metrics_host[i];
        upload(bg->md, metrics_host, (size_t)6 * nref, s);
        upload(bg->mf, m32.data(), m32.size(), s);
    }
    else
    {
        vertex_metrics_kernel<<<(nref + 255) / 256, 256, 0, s>>>(crew, bg->pd.p, nref, bg->md.p, bg->mf.p);
        GM_CUDA(cudaGetLastError());
    }
    f.nbg = bg->nbg;
    f.tv = bg->tv.p;
    f.tn = bg->tn.p;
    f.pf = bg->pf.p;
    f.pd = bg->pd.p;
    f.mf = bg->mf.p;
    f.md = bg->md.p;
    f.cell = bg->cell.p;
    f.ecache = first.empty() ? nullptr : bg->ecache.p;
    f.nt = nt;
    f.np = np;
    f.ne = (uint32_t)first.size();
    upload(bg->field, &f, 1, s);
    GM_CUDA(cudaStreamSynchronize(s));
    return bg;
}

template <class T>
std::vector<T> fetch(const DBuf<T>& b, size_t n, cudaStream_t s)
{
    std::vector<T> h(n);
    if (n) GM_CUDA(cudaMemcpyAsync(h.data(), b.p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    return h;
}

}  // namespace

std::shared_ptr<LocalBackground> local_background_from_mesh(gm_mesh* m, const Crew& crew)
{
    if (m->nv == 0 || (m->nt + m->np + m->nh) == 0 || !m->tets.p)
        throw ApiError(GM_ERR_STATE, "the local sampler needs an uploaded mesh to build its background from");
    require((uint64_t)m->nt + 3ull * m->np + 6ull * m->nh < (1ull << 30), "background mesh too large");
    cudaStream_t s = m->stream;
    std::vector<float4> pos = fetch(m->pos, m->nv, s);
    std::vector<uint4> tets = fetch(m->tets, m->nt, s);
    std::vector<uint32_t> pris = fetch(m->pris, (size_t)m->np * 6, s);
    std::vector<uint4> hexs = fetch(m->hexs, (size_t)m->nh * 2, s);
    GM_CUDA(cudaStreamSynchronize(s));
    std::vector<double> pd((size_t)3 * m->nv);
    for (uint32_t v = 0; v < m->nv; ++v)
    {
        pd[3 * (size_t)v] = pos[v].x;
        pd[3 * (size_t)v + 1] = pos[v].y;
        pd[3 * (size_t)v + 2] = pos[v].z;
    }
    std::vector<uint4> tv, tn;
    std::vector<uint32_t> first;
    split_elements(tets, pris, hexs, tv, first);
    face_neighbours(tv, m->nv, tn);
    auto bg = finish(tv, tn, pd, nullptr, crew, first, m->nt, m->np, s);
    bg->from_mesh = true;
    bg->scaling = crew.scaling;
    bg->aspect = crew.aspect;
    return bg;
}

std::shared_ptr<LocalBackground> local_background_given(gm_mesh* m, uint32_t ntets, const uint32_t* tets8,
                                                        uint32_t nverts, const double* xyz, const double* metrics6)
{
    require(tets8 && xyz && metrics6, "null argument");
    require(ntets > 0 && nverts > 0 && ntets < (1u << 30), "empty or too large background mesh");
    std::vector<uint4> tv(ntets), tn(ntets);
    for (uint32_t t = 0; t < ntets; ++t)
    {
        const uint32_t* r = tets8 + 8 * (size_t)t;
        for (int k = 0; k < 4; ++k)
            if (r[k] >= nverts)
                throw ApiError(GM_ERR_INVALID_ARG, "background tet " + std::to_string(t) + " names vertex " +
                                                       std::to_string(r[k]) + " of " + std::to_string(nverts));
        for (int k = 4; k < 8; ++k)
            if (r[k] != kNoTet && r[k] >= ntets)
                throw ApiError(GM_ERR_INVALID_ARG, "background tet " + std::to_string(t) + " names neighbour " +
                                                       std::to_string(r[k]) + " of " + std::to_string(ntets));
        tv[t] = make_uint4(r[0], r[1], r[2], r[3]);
        tn[t] = make_uint4(r[4], r[5], r[6], r[7]);
    }
    std::vector<double> pd(xyz, xyz + 3 * (size_t)nverts);
    for (size_t i = 0; i < pd.size(); ++i)
        require(std::isfinite(pd[i]), "non-finite background vertex position");
    for (size_t i = 0; i < 6 * (size_t)nverts; ++i)
        require(std::isfinite(metrics6[i]), "non-finite background vertex metric");
    // neighbours are range-checked only: the walk is bounded, so neighbours
    // that disagree with the tets give a clamped metric, never a stray access
    auto bg = finish(tv, tn, pd, metrics6, m->crew, {}, 0, 0, m->stream);
    bg->from_mesh = false;
    return bg;
}

}  // namespace gm
