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
#include <numeric>
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
                                                             double* __restrict__ md, float4* __restrict__ mf)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const Sym3<double> M = analytic_metric<double>(c, V3<double>{pd[3 * (size_t)v], pd[3 * (size_t)v + 1],
                                                                  pd[3 * (size_t)v + 2]});
    const double m[6] = {M.xx, M.yy, M.zz, M.xy, M.xz, M.yz};
    for (int j = 0; j < 6; ++j) md[6 * (size_t)v + j] = m[j];
    mf[2 * (size_t)v] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)m[3]);
    mf[2 * (size_t)v + 1] = make_float4((float)m[4], (float)m[5], 0.f, 0.f);
}

// FP32 copies of 6-entry metrics as float4 pairs (xx yy zz xy), (xz yz 0 0)
std::vector<float4> metric_pairs(const double* md, size_t n)
{
    std::vector<float4> mf(2 * n);
    for (size_t i = 0; i < n; ++i)
    {
        const double* m = md + 6 * i;
        mf[2 * i] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)m[3]);
        mf[2 * i + 1] = make_float4((float)m[4], (float)m[5], 0.f, 0.f);
    }
    return mf;
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
    bg->mf.reserve((size_t)2 * nref);
    if (metrics_host)
    {
        const std::vector<float4> m32 = metric_pairs(metrics_host, nref);
        upload(bg->md, metrics_host, (size_t)6 * nref, s);
        upload(bg->mf, m32.data(), m32.size(), s);
    }
    else
    {
        vertex_metrics_kernel<<<(nref + 255) / 256, 256, 0, s>>>(crew, bg->pd.p, nref, bg->md.p, bg->mf.p);
        note_launch();
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
    bg->part = f;
    bg->pd_h = pd;
    bg->tv_h = tv;
    upload(bg->field, &f, 1, s);
    GM_CUDA(cudaStreamSynchronize(s));
    return bg;
}

// the local metric at points, each walk from its own start tet (FP64)
__global__ void __launch_bounds__(128) local_query_kernel(const LocalField* __restrict__ L, const double* __restrict__ pts,
                                                          const uint32_t* __restrict__ start, uint32_t n,
                                                          double* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3<double> p{pts[3 * (size_t)i], pts[3 * (size_t)i + 1], pts[3 * (size_t)i + 2]};
    const Sym3<double> M = local_walk<double>(*L, p, start[i]);
    const double m[6] = {M.xx, M.yy, M.zz, M.xy, M.xz, M.yz};
    for (int j = 0; j < 6; ++j) out[6 * (size_t)i + j] = m[j];
}

// LocalSampler::metricAt on the device for a batch of points
std::vector<double> local_queries(const LocalBackground& bg, const std::vector<double>& pts,
                                  const std::vector<uint32_t>& start, cudaStream_t s)
{
    const uint32_t n = (uint32_t)start.size();
    std::vector<double> out((size_t)6 * n);
    if (!n) return out;
    DBuf<double> d_pts, d_out;
    DBuf<uint32_t> d_start;
    upload(d_pts, pts.data(), pts.size(), s);
    upload(d_start, start.data(), start.size(), s);
    d_out.reserve((size_t)6 * n);
    local_query_kernel<<<(n + 127) / 128, 128, 0, s>>>(bg.field.p, d_pts.p, d_start.p, n, d_out.p);
    note_launch();
    GM_CUDA(cudaGetLastError());
    GM_CUDA(cudaMemcpyAsync(out.data(), d_out.p, out.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    GM_CUDA(cudaStreamSynchronize(s));
    return out;
}

// per vertex the last background tet holding it (the walk cache the
// reference's background build leaves on each vertex)
std::vector<uint32_t> vertex_caches(const LocalBackground& bg)
{
    std::vector<uint32_t> vc(bg.nref, 0);
    for (size_t t = 0; t < bg.tv_h.size(); ++t)
    {
        const uint4 q = bg.tv_h[t];
        vc[q.x] = vc[q.y] = vc[q.z] = vc[q.w] = (uint32_t)t;
    }
    return vc;
}

template <class D>
void upload_metrics(D& data, const std::vector<double>& md, cudaStream_t s)
{
    const std::vector<float4> mf = metric_pairs(md.data(), md.size() / 6);
    upload(data.md, md.data(), md.size(), s);
    upload(data.mf, mf.data(), mf.size(), s);
}

void upload_kd(KdTreeData& kd, const std::vector<int2>& child, const std::vector<Plane4d>& sep,
               const std::vector<double>& md, cudaStream_t s)
{
    std::vector<float4> sf(sep.size());
    for (size_t i = 0; i < sep.size(); ++i)
        sf[i] = make_float4((float)sep[i].x, (float)sep[i].y, (float)sep[i].z, (float)sep[i].w);
    kd.n = (uint32_t)child.size();
    upload(kd.child, child.data(), child.size(), s);
    upload(kd.sepd, sep.data(), sep.size(), s);
    upload(kd.sepf, sf.data(), sf.size(), s);
    upload_metrics(kd, md, s);
    GM_CUDA(cudaStreamSynchronize(s));
}

// KdTreeSampler::build (Samplers/KdTreeSampler.cpp:268-372), nodes numbered
// in the pre-order of buildGpuBuffers (:374-397)
struct KdBuilder
{
    const std::vector<double>& pd;
    const std::vector<uint32_t>& vcache;
    std::vector<int2> child;
    std::vector<Plane4d> sep;
    std::vector<double> qpts;
    std::vector<uint32_t> qstart, qnode;
    // vertices on a separator go to both sides, so coincident coordinates can
    // make the lists grow with the height: the build stops at a budget
    size_t entries = 0, budget = 0;

    double at(uint32_t v, int a) const { return pd[3 * (size_t)v + a]; }

    int build(int height, std::vector<uint32_t>& xs, std::vector<uint32_t>& ys, std::vector<uint32_t>& zs)
    {
        entries += xs.size();
        if (entries > budget)
            throw ApiError(GM_ERR_UNSUPPORTED, "kd-tree build: too many vertices on separators for this depth");
        const int id = (int)child.size();
        child.push_back(make_int2(-1, -1));
        sep.push_back(Plane4d{0, 0, 0, 0});
        const size_t n = xs.size();
        if (height > 0 && n > 3)
        {
            const double ex = at(xs.back(), 0) - at(xs.front(), 0);
            const double ey = at(ys.back(), 1) - at(ys.front(), 1);
            const double ez = at(zs.back(), 2) - at(zs.front(), 2);
            int axis = 0;
            const std::vector<uint32_t>* list = &xs;
            if (ey >= ex && ey >= ez) axis = 1, list = &ys;
            else if (ez >= ex && ez >= ey) axis = 2, list = &zs;
            const size_t r = n / 2, l = r - 1;
            const uint32_t sl = (*list)[l], sr = (*list)[r];
            // dot(axis, separator position) of a unit axis is that coordinate
            const double sv = n % 2 == 0 ? (at(sl, axis) + at(sr, axis)) / 2.0 : at(sr, axis);
            sep[id] = Plane4d{axis == 0 ? 1.0 : 0.0, axis == 1 ? 1.0 : 0.0, axis == 2 ? 1.0 : 0.0, sv};
            std::vector<uint32_t> L[3], R[3];
            std::vector<uint32_t>* src[3] = {&xs, &ys, &zs};
            for (int q = 0; q < 3; ++q)
            {
                for (uint32_t v : *src[q])
                {
                    const double d = at(v, axis) - sv;
                    if (d <= 0.0) L[q].push_back(v);
                    if (d >= 0.0) R[q].push_back(v);
                }
                std::vector<uint32_t>().swap(*src[q]);
            }
            const int left = build(height - 1, L[0], L[1], L[2]);
            child[id].x = left;
            const int right = build(height - 1, R[0], R[1], R[2]);
            child[id].y = right;
        }
        else
        {
            double mean[3] = {0, 0, 0};
            for (uint32_t v : xs)
                for (int a = 0; a < 3; ++a) mean[a] += at(v, a);
            for (int a = 0; a < 3; ++a) qpts.push_back(mean[a] / (double)n);
            qstart.push_back(vcache[xs.front()]);
            qnode.push_back((uint32_t)id);
        }
        return id;
    }
};

}  // namespace

std::shared_ptr<KdTreeData> kdtree_from_mesh(gm_mesh* m, const LocalBackground& bg, const Crew& crew, int depth)
{
    const uint32_t nv = bg.nref;
    require(nv > 0, "the kd-tree sampler needs an uploaded mesh");
    int height = depth;
    if (height < 0) height = (int)std::log2(std::ceil(nv / 3.0));
    require(height < kKdMaxDepth, "kd-tree depth above " + std::to_string(kKdMaxDepth - 1));
    const std::vector<uint32_t> vc = vertex_caches(bg);
    std::vector<uint32_t> sorted[3];
    for (int a = 0; a < 3; ++a)
    {
        sorted[a].resize(nv);
        std::iota(sorted[a].begin(), sorted[a].end(), 0u);
        const double* pd = bg.pd_h.data();
        std::sort(sorted[a].begin(), sorted[a].end(),
                  [pd, a](uint32_t x, uint32_t y) { return pd[3 * (size_t)x + a] < pd[3 * (size_t)y + a]; });
    }
    KdBuilder b{bg.pd_h, vc, {}, {}, {}, {}, {}, 0, (size_t)64 * nv + 4096};
    b.build(height, sorted[0], sorted[1], sorted[2]);
    const std::vector<double> leaf = local_queries(bg, b.qpts, b.qstart, m->stream);
    // inner nodes keep the identity (MeshMetric's default), never returned
    std::vector<double> md((size_t)6 * b.child.size(), 0.0);
    for (size_t i = 0; i < b.child.size(); ++i) md[6 * i] = md[6 * i + 1] = md[6 * i + 2] = 1.0;
    for (size_t q = 0; q < b.qnode.size(); ++q)
        for (int j = 0; j < 6; ++j) md[6 * (size_t)b.qnode[q] + j] = leaf[6 * q + j];
    auto kd = std::make_shared<KdTreeData>();
    upload_kd(*kd, b.child, b.sep, md, m->stream);
    kd->given = false;
    kd->depth = depth;
    kd->scaling = crew.scaling;
    kd->aspect = crew.aspect;
    return kd;
}

std::shared_ptr<KdTreeData> kdtree_given(gm_mesh* m, uint32_t n, const int32_t* children2, const double* sep4,
                                         const double* metrics6)
{
    require(children2 && sep4 && metrics6, "null argument");
    require(n > 0 && n < (1u << 30), "empty or too large kd-tree");
    std::vector<int2> child(n);
    std::vector<Plane4d> sep(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        const int32_t l = children2[2 * (size_t)i], r = children2[2 * (size_t)i + 1];
        // pre-order: children come after their parent, so every descent ends
        require((l == -1 || ((uint32_t)l > i && (uint32_t)l < n)) && (r == -1 || ((uint32_t)r > i && (uint32_t)r < n)),
                "kd-tree node " + std::to_string(i) + " names a child out of pre-order");
        child[i] = make_int2(l, r);
        sep[i] = Plane4d{sep4[4 * (size_t)i], sep4[4 * (size_t)i + 1], sep4[4 * (size_t)i + 2],
                         sep4[4 * (size_t)i + 3]};
    }
    std::vector<double> md(metrics6, metrics6 + 6 * (size_t)n);
    for (double x : md) require(std::isfinite(x), "non-finite kd-tree metric");
    auto kd = std::make_shared<KdTreeData>();
    upload_kd(*kd, child, sep, md, m->stream);
    kd->given = true;
    return kd;
}

namespace {

// TextureSampler::cellId (TextureSampler.cpp:513-524)
void tex_cell_host(const TextureData& t, const double* pos, int* id)
{
    for (int k = 0; k < 3; ++k)
    {
        const int c = (int)((pos[k] - t.lo[k]) / t.ext[k] * (double)t.g[k]);
        id[k] = std::min(std::max(c, 0), t.g[k] - 1);
    }
}

}  // namespace

// TextureSampler::buildGrid (TextureSampler.cpp:275-448)
std::shared_ptr<TextureData> texture_from_mesh(gm_mesh* m, const LocalBackground& bg, const Crew& crew, int depth)
{
    require(bg.nref > 0, "the texture sampler needs an uploaded mesh");
    auto t = std::make_shared<TextureData>();
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    for (uint32_t v = 0; v < bg.nref; ++v)
        for (int k = 0; k < 3; ++k)
        {
            const double x = bg.pd_h[3 * (size_t)v + k];
            lo[k] = x < lo[k] ? x : lo[k];
            hi[k] = hi[k] < x ? x : hi[k];
        }
    for (int k = 0; k < 3; ++k)
    {
        t->lo[k] = lo[k];
        t->ext[k] = hi[k] - lo[k];
    }
    double cells = (double)bg.nref;
    if (depth > 0) cells = (double)((size_t)depth * depth * depth);
    const double alpha = std::pow(cells / (t->ext[0] * t->ext[1] * t->ext[2]), 1 / 3.0);
    size_t total = 1;
    for (int k = 0; k < 3; ++k)
    {
        const double e = alpha * t->ext[k];
        const double g = std::round(e > 1.0 ? e : 1.0);
        require(g < 4096.0, "texture grid too large (a flat mesh?)");
        t->g[k] = (int)g;
        total *= (size_t)t->g[k];
    }
    require(total <= (size_t)1 << 28, "texture grid too large");
    // the first tet (in order) whose cell box, grown by one, holds a cell
    // samples it, its walk starting there; cells no box reaches keep the
    // identity
    std::vector<uint32_t> owner(total, kNoTet);
    std::vector<double> qpts;
    std::vector<uint32_t> qstart, qcell;
    double cs[3];
    for (int k = 0; k < 3; ++k) cs[k] = t->ext[k] / (double)t->g[k];
    for (size_t e = 0; e < bg.tv_h.size(); ++e)
    {
        const uint4 q = bg.tv_h[e];
        const uint32_t vv[4] = {q.x, q.y, q.z, q.w};
        double bmin[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, bmax[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        for (uint32_t v : vv)
            for (int k = 0; k < 3; ++k)
            {
                const double x = bg.pd_h[3 * (size_t)v + k];
                bmin[k] = x < bmin[k] ? x : bmin[k];
                bmax[k] = bmax[k] < x ? x : bmax[k];
            }
        int a[3], b[3];
        tex_cell_host(*t, bmin, a);
        tex_cell_host(*t, bmax, b);
        for (int k = 0; k < 3; ++k)
        {
            a[k] = std::max(a[k] - 1, 0);
            b[k] = std::min(b[k] + 1, t->g[k] - 1);
        }
        for (int z = a[2]; z <= b[2]; ++z)
            for (int y = a[1]; y <= b[1]; ++y)
                for (int x = a[0]; x <= b[0]; ++x)
                {
                    const size_t c = ((size_t)z * t->g[1] + y) * t->g[0] + x;
                    if (owner[c] != kNoTet) continue;
                    owner[c] = (uint32_t)e;
                    qpts.push_back(t->lo[0] + cs[0] * ((double)x + 0.5));
                    qpts.push_back(t->lo[1] + cs[1] * ((double)y + 0.5));
                    qpts.push_back(t->lo[2] + cs[2] * ((double)z + 0.5));
                    qstart.push_back((uint32_t)e);
                    qcell.push_back((uint32_t)c);
                }
    }
    const std::vector<double> res = local_queries(bg, qpts, qstart, m->stream);
    std::vector<double> md(6 * total, 0.0);
    for (size_t c = 0; c < total; ++c) md[6 * c] = md[6 * c + 1] = md[6 * c + 2] = 1.0;
    for (size_t q = 0; q < qcell.size(); ++q)
        for (int j = 0; j < 6; ++j) md[6 * (size_t)qcell[q] + j] = res[6 * q + j];
    upload_metrics(*t, md, m->stream);
    GM_CUDA(cudaStreamSynchronize(m->stream));
    t->given = false;
    t->depth = depth;
    t->scaling = crew.scaling;
    t->aspect = crew.aspect;
    return t;
}

std::shared_ptr<TextureData> texture_given(gm_mesh* m, const int32_t* dims3, const double* lo3, const double* ext3,
                                           const double* metrics6)
{
    require(dims3 && lo3 && ext3 && metrics6, "null argument");
    auto t = std::make_shared<TextureData>();
    size_t total = 1;
    for (int k = 0; k < 3; ++k)
    {
        require(dims3[k] > 0 && dims3[k] < 4096, "texture dimensions out of range");
        require(std::isfinite(lo3[k]) && std::isfinite(ext3[k]) && ext3[k] > 0.0, "texture bounds must be finite");
        t->g[k] = dims3[k];
        t->lo[k] = lo3[k];
        t->ext[k] = ext3[k];
        total *= (size_t)dims3[k];
    }
    require(total <= (size_t)1 << 28, "texture grid too large");
    std::vector<double> md(metrics6, metrics6 + 6 * total);
    for (double x : md) require(std::isfinite(x), "non-finite texture metric");
    upload_metrics(*t, md, m->stream);
    GM_CUDA(cudaStreamSynchronize(m->stream));
    t->given = true;
    return t;
}

const LocalField* assemble_field(gm_mesh* m)
{
    LocalField f{};
    if (m->local) f = m->local->part;
    if (m->kd)
    {
        f.kd_child = m->kd->child.p;
        f.kd_sepf = m->kd->sepf.p;
        f.kd_sepd = m->kd->sepd.p;
        f.kd_mf = m->kd->mf.p;
        f.kd_md = m->kd->md.p;
    }
    if (m->tex)
    {
        for (int k = 0; k < 3; ++k)
        {
            f.tg[k] = m->tex->g[k];
            f.tmin[k] = m->tex->lo[k];
            f.text[k] = m->tex->ext[k];
        }
        f.tex_mf = m->tex->mf.p;
        f.tex_md = m->tex->md.p;
    }
    upload(m->field, &f, 1, m->stream);
    GM_CUDA(cudaStreamSynchronize(m->stream));
    return m->field.p;
}

void prepare_sampler(gm_mesh* m, Crew& c)
{
    c.local = nullptr;
    if (c.sampler < GM_SAMPLER_LOCAL) return;
    auto built_here = [&](const std::shared_ptr<LocalBackground>& b) {
        return b && b->from_mesh && b->scaling == c.scaling && b->aspect == c.aspect;
    };
    std::shared_ptr<LocalBackground> bg = m->local;
    std::shared_ptr<KdTreeData> kd = m->kd;
    std::shared_ptr<TextureData> tex = m->tex;
    // GpuMeshCharacter::updateSampling rebuilds the sampling when the scaling
    // or the aspect ratio changes (GpuMeshCharacter.cpp:1115-1129); a given
    // background, kd-tree or texture is the caller's and stays
    if (c.sampler == GM_SAMPLER_LOCAL && (!bg || (bg->from_mesh && !built_here(bg))))
        bg = local_background_from_mesh(m, c);
    auto source = [&]() {
        if (!built_here(bg)) bg = local_background_from_mesh(m, c);
        return bg;
    };
    if (c.sampler == GM_SAMPLER_KDTREE &&
        !(kd && (kd->given || (kd->depth == m->depth && kd->scaling == c.scaling && kd->aspect == c.aspect))))
    {
        std::shared_ptr<LocalBackground> keep = bg;
        kd = kdtree_from_mesh(m, *source(), c, m->depth);
        if (keep && !keep->from_mesh) bg = keep;  // a given background stays the local sampler's
    }
    if (c.sampler == GM_SAMPLER_TEXTURE &&
        !(tex && (tex->given || (tex->depth == m->depth && tex->scaling == c.scaling && tex->aspect == c.aspect))))
    {
        std::shared_ptr<LocalBackground> keep = bg;
        tex = texture_from_mesh(m, *source(), c, m->depth);
        if (keep && !keep->from_mesh) bg = keep;
    }
    m->local = bg;
    m->kd = kd;
    m->tex = tex;
    c.local = assemble_field(m);
}

void sampler_topology_changed(gm_mesh* m)
{
    if (m->local && m->local->from_mesh) m->local.reset();
    if (m->kd && !m->kd->given) m->kd.reset();
    if (m->tex && !m->tex->given) m->tex.reset();
    if (m->crew.sampler >= GM_SAMPLER_LOCAL) prepare_sampler(m, m->crew);
}

size_t sampler_bytes(const gm_mesh* m)
{
    size_t b = m->field.cap * sizeof(LocalField);
    if (m->local) b += m->local->bytes();
    if (m->kd) b += m->kd->bytes();
    if (m->tex) b += m->tex->bytes();
    return b;
}

namespace {

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
