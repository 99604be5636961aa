// Internal declarations shared by the host translation units of
// libgpumesh_gb300.so.  Nothing here is part of the C ABI.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace gm {

// element type codes, equal to MeshTet/MeshPri/MeshHex::ELEMENT_TYPE
// (DataStructures/Mesh.h:89,171,213)
constexpr int kTypeTet = 0;
constexpr int kTypePyr = 1;
constexpr int kTypePri = 2;
constexpr int kTypeHex = 3;

// one vertex->element reference: type (2 bits) | local vertex index (3 bits)
// | element id (27 bits), the packed form of MeshNeigElem{id, type, vId}
constexpr uint32_t kMaxElemId = (1u << 27) - 1;
inline uint32_t pack_elem_ref(int type, int local, uint32_t id)
{
    return ((uint32_t)type << 30) | ((uint32_t)local << 27) | id;
}

struct HostMeshView
{
    uint32_t nv = 0, nt = 0, np = 0, nh = 0;
    const int32_t* cid = nullptr;
    const uint32_t* tets = nullptr;
    const uint32_t* pris = nullptr;
    const uint32_t* hexs = nullptr;
};

struct Topology
{
    uint32_t nv = 0;
    std::vector<uint32_t> perm;        // new index -> old index
    std::vector<uint32_t> new_of_old;  // old index -> new index
    std::vector<int> vtype;            // per new vertex: 0 fixed, 1 boundary, 2 subsurface, 3 interior
    std::vector<int> colour;           // per new vertex
    std::vector<uint32_t> group_base;  // ngroups + 1
    std::vector<uint32_t> members;     // colour-major, new indices
    std::vector<uint32_t> ranges;      // 6 per group: boundary, subsurface, interior [begin, end)
    std::vector<uint32_t> ve_off, ve;  // vertex -> packed element refs (new vertex ids)
    std::vector<uint32_t> vv_off, vv;  // vertex -> neighbour vertices (new ids)
};

// Fills colour[v] (>= 0) for every vertex that is not fixed, from the
// vertex -> element refs of the mesh (e_off, e: the neighbourhood CSR).
using ColourSource = std::function<void(const std::vector<uint32_t>& e_off, const std::vector<uint32_t>& e,
                                        std::vector<int>& colour)>;

// the device order mode's colours (gm_colour.cu)
void device_colours(const HostMeshView& in, const std::vector<uint32_t>& e_off, const std::vector<uint32_t>& e,
                    std::vector<int>& colour);

// colour_source empty: NodeGroups::determineGroups' greedy colouring
Topology build_topology(const HostMeshView& in, bool permute, ColourSource colour_source = nullptr);
void build_csr(const HostMeshView& in, std::vector<uint32_t>& ve_off, std::vector<uint32_t>& ve,
               std::vector<uint32_t>& vv_off, std::vector<uint32_t>& vv);

// thread-local last-error message for gm_last_error()
void set_error(const std::string& msg);

}  // namespace gm
