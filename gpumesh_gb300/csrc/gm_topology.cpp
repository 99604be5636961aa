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
#include <vector>

#include "gm_internal.h"

namespace gm {

namespace {

const int kTetEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kPriEdges[9][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {3, 5}, {4, 5}};
const int kHexEdges[12][2] = {{0, 1}, {0, 3}, {1, 2}, {2, 3}, {0, 4}, {1, 5},
                              {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};

struct ElemRef
{
    uint32_t id;
    int8_t type;
    int8_t local;
};

struct Neighbourhoods
{
    std::vector<std::vector<ElemRef>> elems;
    std::vector<std::vector<uint32_t>> verts;
};

void add_edge(Neighbourhoods& nb, uint32_t a, uint32_t b)
{
    std::vector<uint32_t>& list = nb.verts[a];
    for (uint32_t x : list)
        if (x == b) return;
    nb.verts[a].push_back(b);
    nb.verts[b].push_back(a);
}

template <int K, int NE>
void add_elements(Neighbourhoods& nb, const uint32_t* conn, uint32_t count, int type, const int (*edges)[2])
{
    for (uint32_t i = 0; i < count; ++i)
    {
        const uint32_t* e = conn + (size_t)K * i;
        for (int k = 0; k < K; ++k) nb.elems[e[k]].push_back(ElemRef{i, (int8_t)type, (int8_t)k});
        for (int k = 0; k < NE; ++k) add_edge(nb, e[edges[k][0]], e[edges[k][1]]);
    }
}

Neighbourhoods build_neighbourhoods(const HostMeshView& in)
{
    Neighbourhoods nb;
    nb.elems.resize(in.nv);
    nb.verts.resize(in.nv);
    add_elements<4, 6>(nb, in.tets, in.nt, kTypeTet, kTetEdges);
    add_elements<6, 9>(nb, in.pris, in.np, kTypePri, kPriEdges);
    add_elements<8, 12>(nb, in.hexs, in.nh, kTypeHex, kHexEdges);
    return nb;
}

}  // namespace

void build_csr(const HostMeshView& in, std::vector<uint32_t>& ve_off, std::vector<uint32_t>& ve,
               std::vector<uint32_t>& vv_off, std::vector<uint32_t>& vv)
{
    Neighbourhoods nb = build_neighbourhoods(in);
    const uint32_t nv = in.nv;
    ve_off.assign((size_t)nv + 1, 0);
    vv_off.assign((size_t)nv + 1, 0);
    for (uint32_t v = 0; v < nv; ++v)
    {
        ve_off[v + 1] = ve_off[v] + (uint32_t)nb.elems[v].size();
        vv_off[v + 1] = vv_off[v] + (uint32_t)nb.verts[v].size();
    }
    ve.resize(ve_off[nv]);
    vv.resize(vv_off[nv]);
    for (uint32_t v = 0; v < nv; ++v)
    {
        uint32_t o = ve_off[v];
        for (const ElemRef& r : nb.elems[v]) ve[o++] = pack_elem_ref(r.type, r.local, r.id);
        std::copy(nb.verts[v].begin(), nb.verts[v].end(), vv.begin() + vv_off[v]);
    }
}

Topology build_topology(const HostMeshView& in, bool permute)
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
            for (const ElemRef& r : nb.elems[v])
            {
                if ((r.type == kTypeTet && bounding_tet[r.id]) || (r.type == kTypePri && bounding_pri[r.id]) ||
                    (r.type == kTypeHex && bounding_hex[r.id]))
                {
                    sub = true;
                    break;
                }
            }
            types[v] = sub ? SUBSU : INTER;
        }
    }

    // ---- greedy breadth-first colouring ----
    // The reference copies the set of existing colours for every vertex and
    // erases its neighbours' colours; the first remaining colour (or a new
    // one) is taken.  A bitmask of the neighbours' colours gives the same
    // first-fit choice without the set copies.
    const int NO_GROUP = -2, UNSET = -1;
    std::vector<int> groups(nv, NO_GROUP);
    {
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
                for (const ElemRef& r : nb.elems[v])
                {
                    const uint32_t* e;
                    int k;
                    if (r.type == kTypeTet) { e = in.tets + 4 * (size_t)r.id; k = 4; }
                    else if (r.type == kTypePri) { e = in.pris + 6 * (size_t)r.id; k = 6; }
                    else { e = in.hexs + 8 * (size_t)r.id; k = 8; }
                    for (int j = 0; j < k; ++j) visit(e[j]);
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
                if (groups[a] == groups[b]) return nb.elems[a].size() < nb.elems[b].size();
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
        t.ve_off[p + 1] = t.ve_off[p] + (uint32_t)nb.elems[order[p]].size();
        t.vv_off[p + 1] = t.vv_off[p] + (uint32_t)nb.verts[order[p]].size();
    }
    t.ve.resize(t.ve_off[nv]);
    t.vv.resize(t.vv_off[nv]);
    for (uint32_t p = 0; p < nv; ++p)
    {
        uint32_t o = t.ve_off[p];
        for (const ElemRef& r : nb.elems[order[p]]) t.ve[o++] = pack_elem_ref(r.type, r.local, r.id);
        o = t.vv_off[p];
        for (uint32_t w : nb.verts[order[p]]) t.vv[o++] = new_of_old[w];
    }
    t.new_of_old = std::move(new_of_old);
    return t;
}

}  // namespace gm
