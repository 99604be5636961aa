// Host-side mesh topology: vertex neighbourhoods and independent vertex
// groups, built the way the reference builds them so that the device path
// consumes the same permuted mesh and the same colour-major group order.
//
//   neighbourhoods  : Mesh::compileNeighborhoods / Mesh::addEdge
//                     (DataStructures/Mesh.cpp:365-460)
//   vertex classes  : NodeGroups::determineTypes (DataStructures/NodeGroups.cpp:124-241)
//   colouring       : NodeGroups::determineGroups (NodeGroups.cpp:243-363), a
//                     breadth-first greedy first-fit colouring in which two
//                     vertices conflict when they share an element
//   vertex order    : NodeGroups::determinePositions / clusterNodes
//                     (NodeGroups.cpp:365-619): sort by (class, colour,
//                     element valence) with std::sort, then permute
//
// The sort key and the use of std::sort are kept identical to the reference
// on purpose: ties inside one (class, colour, valence) bucket are broken by
// libstdc++'s introsort, and reproducing the reference's vertex numbering
// requires the same algorithm on the same input.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <vector>

#include "gm_internal.h"

namespace gm {

namespace {

const int kTetEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kPriEdges[9][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {3, 5}, {4, 5}};
const int kHexEdges[12][2] = {{0, 1}, {0, 3}, {1, 2}, {2, 3}, {0, 4}, {1, 5},
                              {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};

// Per-vertex neighbourhoods as flat CSR arrays (Mesh::compileNeighborhoods
// keeps a std::vector per vertex; the lists here hold the same entries in
// the same order):
//   elems: packed (type, local, id) refs, in element order -- tets, then
//          prisms, then hexes, each by id
//   verts: edge neighbours in the order the edges are first met, element by
//          element and edge by edge (Mesh::addEdge: a neighbour is appended
//          to both ends when the first end's list does not hold it yet)
struct Neighbourhoods
{
    std::vector<uint32_t> e_off, e;
    std::vector<uint32_t> v_off, v;
    uint32_t elem_count(uint32_t x) const { return e_off[x + 1] - e_off[x]; }
};

template <int K>
void count_refs(const uint32_t* conn, uint32_t count, std::vector<uint32_t>& deg)
{
    for (size_t i = 0; i < (size_t)count * K; ++i) ++deg[conn[i] + 1];
}

template <int K>
void fill_refs(const uint32_t* conn, uint32_t count, int type, std::vector<uint32_t>& cur, std::vector<uint32_t>& e)
{
    for (uint32_t i = 0; i < count; ++i)
        for (int k = 0; k < K; ++k)
        {
            const uint32_t x = conn[(size_t)K * i + k];
            e[cur[x]++] = pack_elem_ref(type, k, i);
        }
}

// f(range, begin, end) over [0, n) in contiguous ranges, one per host thread
// (a single range when n is small); returns the number of ranges
template <class F>
unsigned parallel_ranges(uint32_t n, F f)
{
    unsigned t = std::thread::hardware_concurrency();
    t = std::min<unsigned>(t == 0 ? 1 : t, 16);
    if (n < 65536 || t == 1)
    {
        f(0u, 0u, n);
        return 1;
    }
    std::vector<std::thread> pool;
    const uint32_t chunk = (n + t - 1) / t;
    for (unsigned i = 0; i < t; ++i)
    {
        const uint32_t b = std::min<uint32_t>(n, i * chunk), e = std::min<uint32_t>(n, b + chunk);
        pool.emplace_back(f, i, b, e);
    }
    for (std::thread& th : pool) th.join();
    return t;
}

// Mesh::addEdge over every element's edges in element order, appending to
// bounded per-vertex lists (the sequential form, for small meshes)
template <int K, int NE>
void add_edges(const uint32_t* conn, uint32_t count, const int (*edges)[2], const std::vector<uint32_t>& base,
               std::vector<uint32_t>& n, std::vector<uint32_t>& slot)
{
    for (uint32_t i = 0; i < count; ++i)
    {
        const uint32_t* el = conn + (size_t)K * i;
        for (int k = 0; k < NE; ++k)
        {
            const uint32_t a = el[edges[k][0]], b = el[edges[k][1]];
            const uint32_t* la = slot.data() + base[a];
            bool seen = false;
            for (uint32_t j = 0; j < n[a] && !seen; ++j) seen = la[j] == b;
            if (seen) continue;
            slot[base[a] + n[a]++] = b;
            slot[base[b] + n[b]++] = a;
        }
    }
}

// The edge neighbours of vertex x.  Mesh::addEdge appends b to a's list and a
// to b's when a's list does not hold b; the lists stay symmetric, so x's
// list is the other ends of the edges at x in the order they are met:
// x's elements in element order (its element refs), each element's edges in
// edge-table order.  That makes every vertex independent of the others.
uint32_t vertex_neighbours(const HostMeshView& in, const Neighbourhoods& nb, uint32_t x, uint32_t* out)
{
    uint32_t cnt = 0;
    for (uint32_t j = nb.e_off[x]; j < nb.e_off[x + 1]; ++j)
    {
        const uint32_t r = nb.e[j];
        const int type = (int)(r >> 30), local = (int)((r >> 27) & 7u);
        const uint32_t id = r & kMaxElemId;
        const uint32_t* el;
        const int(*edges)[2];
        int ne;
        if (type == kTypeTet) { el = in.tets + 4 * (size_t)id; edges = kTetEdges; ne = 6; }
        else if (type == kTypePri) { el = in.pris + 6 * (size_t)id; edges = kPriEdges; ne = 9; }
        else { el = in.hexs + 8 * (size_t)id; edges = kHexEdges; ne = 12; }
        for (int k = 0; k < ne; ++k)
        {
            uint32_t w;
            if (edges[k][0] == local) w = el[edges[k][1]];
            else if (edges[k][1] == local) w = el[edges[k][0]];
            else continue;
            bool seen = false;
            for (uint32_t q = 0; q < cnt && !seen; ++q) seen = out[q] == w;
            if (!seen) out[cnt++] = w;
        }
    }
    return cnt;
}

Neighbourhoods build_neighbourhoods(const HostMeshView& in)
{
    const uint32_t nv = in.nv;
    Neighbourhoods nb;
    nb.e_off.assign((size_t)nv + 1, 0);
    count_refs<4>(in.tets, in.nt, nb.e_off);
    count_refs<6>(in.pris, in.np, nb.e_off);
    count_refs<8>(in.hexs, in.nh, nb.e_off);
    for (uint32_t x = 0; x < nv; ++x) nb.e_off[x + 1] += nb.e_off[x];
    nb.e.resize(nb.e_off[nv]);
    std::vector<uint32_t> cur(nb.e_off.begin(), nb.e_off.end() - 1);
    fill_refs<4>(in.tets, in.nt, kTypeTet, cur, nb.e);
    fill_refs<6>(in.pris, in.np, kTypePri, cur, nb.e);
    fill_refs<8>(in.hexs, in.nh, kTypeHex, cur, nb.e);

    // every corner of a tet, prism or hex has three edges, so a vertex has at
    // most 3 x (its element count) distinct neighbours
    if (nv < 65536)
    {
        std::vector<uint32_t> base((size_t)nv + 1, 0), n(nv, 0);
        for (uint32_t x = 0; x < nv; ++x) base[x + 1] = base[x] + 3 * nb.elem_count(x);
        std::vector<uint32_t> slot(base[nv]);
        add_edges<4, 6>(in.tets, in.nt, kTetEdges, base, n, slot);
        add_edges<6, 9>(in.pris, in.np, kPriEdges, base, n, slot);
        add_edges<8, 12>(in.hexs, in.nh, kHexEdges, base, n, slot);
        nb.v_off.assign((size_t)nv + 1, 0);
        for (uint32_t x = 0; x < nv; ++x) nb.v_off[x + 1] = nb.v_off[x] + n[x];
        nb.v.resize(nb.v_off[nv]);
        for (uint32_t x = 0; x < nv; ++x) std::copy_n(slot.begin() + base[x], n[x], nb.v.begin() + nb.v_off[x]);
        return nb;
    }
    // large meshes: vertex by vertex on the host's threads, each range of
    // vertices filling its own list, concatenated in order
    uint32_t most = 0;
    for (uint32_t x = 0; x < nv; ++x) most = std::max(most, nb.elem_count(x));
    std::vector<uint32_t> n(nv, 0);
    std::vector<std::vector<uint32_t>> lists(16);
    std::vector<uint32_t> first(17, 0);
    const unsigned ranges = parallel_ranges(nv, [&](unsigned r, uint32_t b, uint32_t e) {
        std::vector<uint32_t>& out = lists[r];
        std::vector<uint32_t> tmp(3 * (size_t)most + 1);
        out.reserve((size_t)(e - b) * 16);
        first[r] = b;
        for (uint32_t x = b; x < e; ++x)
        {
            n[x] = vertex_neighbours(in, nb, x, tmp.data());
            out.insert(out.end(), tmp.begin(), tmp.begin() + n[x]);
        }
    });
    nb.v_off.assign((size_t)nv + 1, 0);
    for (uint32_t x = 0; x < nv; ++x) nb.v_off[x + 1] = nb.v_off[x] + n[x];
    nb.v.resize(nb.v_off[nv]);
    for (unsigned r = 0; r < ranges; ++r)
        std::copy(lists[r].begin(), lists[r].end(), nb.v.begin() + nb.v_off[first[r]]);
    return nb;
}

}  // namespace

void build_csr(const HostMeshView& in, std::vector<uint32_t>& ve_off, std::vector<uint32_t>& ve,
               std::vector<uint32_t>& vv_off, std::vector<uint32_t>& vv)
{
    Neighbourhoods nb = build_neighbourhoods(in);
    ve_off = std::move(nb.e_off);
    ve = std::move(nb.e);
    vv_off = std::move(nb.v_off);
    vv = std::move(nb.v);
}

Topology build_topology(const HostMeshView& in, bool permute, ColourSource colour_source)
{
    const uint32_t nv = in.nv;
    Neighbourhoods nb = build_neighbourhoods(in);

    // ---- vertex classes ----
    enum { FIXED = 0, BOUND = 1, SUBSU = 2, INTER = 3 };
    auto movable_bound = [&](uint32_t v) { return in.cid[v] > 0; };
    std::vector<char> bounding_tet(in.nt), bounding_pri(in.np), bounding_hex(in.nh);
    for (uint32_t i = 0; i < in.nt; ++i)
        for (int k = 0; k < 4 && !bounding_tet[i]; ++k) bounding_tet[i] = movable_bound(in.tets[4 * (size_t)i + k]);
    for (uint32_t i = 0; i < in.np; ++i)
        for (int k = 0; k < 6 && !bounding_pri[i]; ++k) bounding_pri[i] = movable_bound(in.pris[6 * (size_t)i + k]);
    for (uint32_t i = 0; i < in.nh; ++i)
        for (int k = 0; k < 8 && !bounding_hex[i]; ++k) bounding_hex[i] = movable_bound(in.hexs[8 * (size_t)i + k]);
    std::vector<int> types(nv);
    for (uint32_t v = 0; v < nv; ++v)
    {
        if (in.cid[v] < 0) types[v] = FIXED;
        else if (in.cid[v] != 0) types[v] = BOUND;
        else
        {
            bool sub = false;
            for (uint32_t j = nb.e_off[v]; j < nb.e_off[v + 1] && !sub; ++j)
            {
                const uint32_t r = nb.e[j];
                const int type = (int)(r >> 30);
                const uint32_t id = r & kMaxElemId;
                sub = (type == kTypeTet && bounding_tet[id]) || (type == kTypePri && bounding_pri[id]) ||
                      (type == kTypeHex && bounding_hex[id]);
            }
            types[v] = sub ? SUBSU : INTER;
        }
    }

    // ---- colours: the reference's greedy breadth-first colouring, or one
    //      given by the caller (the device colouring order mode) ----
    const int NO_GROUP = -2, UNSET = -1;
    std::vector<int> groups(nv, NO_GROUP);
    if (colour_source)
    {
        colour_source(nb.e_off, nb.e, groups);
        for (uint32_t v = 0; v < nv; ++v)
            if (types[v] != FIXED && groups[v] < 0) throw std::runtime_error("a movable vertex has no colour");
    }
    else
    {
        // The reference copies the set of existing colours for every vertex
        // and erases its neighbours' colours; the first remaining colour (or
        // a new one) is taken.  A bitmask of the neighbours' colours gives
        // the same first-fit choice without the set copies.
        size_t seek = 0;
        uint32_t ncolours = 0;
        std::vector<uint64_t> used;  // colours taken by the current vertex's neighbours
        std::vector<uint32_t> queue;
        queue.reserve(nv);
        auto visit = [&](uint32_t w) {
            int& g = groups[w];
            if (g == NO_GROUP)
            {
                g = UNSET;
                queue.push_back(w);
            }
            else if (g != UNSET)
                used[(uint32_t)g >> 6] |= 1ull << ((uint32_t)g & 63);
        };
        while (queue.size() < nv)
        {
            size_t first = queue.size();
            for (size_t v = seek; v < nv; ++v)
            {
                ++seek;
                if (groups[v] == NO_GROUP)
                {
                    groups[v] = UNSET;
                    queue.push_back((uint32_t)v);
                    break;
                }
            }
            for (size_t qi = first; qi < queue.size(); ++qi)
            {
                uint32_t v = queue[qi];
                std::fill(used.begin(), used.end(), 0ull);
                for (uint32_t j = nb.e_off[v]; j < nb.e_off[v + 1]; ++j)
                {
                    const uint32_t r = nb.e[j];
                    const int type = (int)(r >> 30);
                    const uint32_t id = r & kMaxElemId;
                    const uint32_t* e;
                    int k;
                    if (type == kTypeTet) { e = in.tets + 4 * (size_t)id; k = 4; }
                    else if (type == kTypePri) { e = in.pris + 6 * (size_t)id; k = 6; }
                    else { e = in.hexs + 8 * (size_t)id; k = 8; }
                    for (int q = 0; q < k; ++q) visit(e[q]);
                }
                // lowest existing colour no neighbour has, else a new one
                uint32_t g = ncolours;
                for (uint32_t wi = 0; wi < used.size(); ++wi)
                {
                    const uint64_t freebits = ~used[wi];
                    if (freebits)
                    {
                        const uint32_t c = wi * 64 + (uint32_t)__builtin_ctzll(freebits);
                        if (c < ncolours) g = c;
                        break;
                    }
                }
                if (g == ncolours)
                {
                    ++ncolours;
                    if (((ncolours + 63) >> 6) > used.size()) used.push_back(0ull);
                }
                groups[v] = (int)g;
            }
        }
    }

    // ---- vertex order ----
    std::vector<int> order(nv);
    std::iota(order.begin(), order.end(), 0);
    if (permute)
    {
        std::sort(order.begin(), order.end(), [&](int a, int b) {
            if (types[a] == types[b])
            {
                if (types[a] == FIXED) return false;
                if (groups[a] == groups[b]) return nb.elem_count(a) < nb.elem_count(b);
                return groups[a] < groups[b];
            }
            return types[a] < types[b];
        });
    }
    std::vector<uint32_t> new_of_old(nv);
    for (uint32_t p = 0; p < nv; ++p) new_of_old[order[p]] = p;

    Topology t;
    t.nv = nv;
    t.perm.assign(order.begin(), order.end());
    t.vtype.resize(nv);
    t.colour.resize(nv);
    for (uint32_t p = 0; p < nv; ++p)
    {
        t.vtype[p] = types[order[p]];
        t.colour[p] = groups[order[p]];
    }

    // ---- colour-major groups: boundary, then subsurface, then interior
    //      members of each colour, in the new order (clusterNodes) ----
    int ngroups = 0;
    for (uint32_t p = 0; p < nv; ++p)
        if (t.vtype[p] != FIXED) ngroups = std::max(ngroups, t.colour[p] + 1);
    std::vector<std::vector<uint32_t>> members(ngroups);
    t.ranges.assign((size_t)ngroups * 6, 0);
    for (uint32_t p = 0; p < nv; ++p)
    {
        int ty = t.vtype[p];
        if (ty == FIXED) continue;
        int g = t.colour[p];
        uint32_t* r = &t.ranges[(size_t)g * 6 + (size_t)(ty - 1) * 2];
        if (r[0] == r[1]) r[0] = r[1] = p;
        r[1] = p + 1;
        members[g].push_back(p);
    }
    t.group_base.assign((size_t)ngroups + 1, 0);
    for (int g = 0; g < ngroups; ++g)
    {
        t.group_base[g + 1] = t.group_base[g] + (uint32_t)members[g].size();
        t.members.insert(t.members.end(), members[g].begin(), members[g].end());
    }

    // ---- permuted neighbourhood CSR ----
    t.ve_off.assign((size_t)nv + 1, 0);
    t.vv_off.assign((size_t)nv + 1, 0);
    for (uint32_t p = 0; p < nv; ++p)
    {
        const uint32_t x = (uint32_t)order[p];
        t.ve_off[p + 1] = t.ve_off[p] + nb.elem_count(x);
        t.vv_off[p + 1] = t.vv_off[p] + (nb.v_off[x + 1] - nb.v_off[x]);
    }
    t.ve.resize(t.ve_off[nv]);
    t.vv.resize(t.vv_off[nv]);
    parallel_ranges(nv, [&](unsigned, uint32_t b, uint32_t e) {
        for (uint32_t p = b; p < e; ++p)
        {
            const uint32_t x = (uint32_t)order[p];
            std::copy(nb.e.begin() + nb.e_off[x], nb.e.begin() + nb.e_off[x + 1], t.ve.begin() + t.ve_off[p]);
            uint32_t o = t.vv_off[p];
            for (uint32_t j = nb.v_off[x]; j < nb.v_off[x + 1]; ++j) t.vv[o++] = new_of_old[nb.v[j]];
        }
    });
    t.new_of_old = std::move(new_of_old);
    return t;
}

}  // namespace gm
