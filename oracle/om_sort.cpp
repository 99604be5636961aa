// TEST INFRASTRUCTURE: part of the oracle (oracle/gm_oracle.c).
//
// KdTreeSampler::updateAnalyticalMetric (Samplers/KdTreeSampler.cpp:144-153)
// orders the vertex ids by each coordinate with std::sort, whose order among
// equal coordinates is the library's own; the kd-tree's leaves average their
// vertices in that order.  The oracle makes the same call so that its sums
// see the same order.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

extern "C" void om_argsort_axis(const double* pos, int64_t n, int axis, uint32_t* out)
{
    std::iota(out, out + n, 0u);
    std::sort(out, out + n, [pos, axis](uint32_t a, uint32_t b) { return pos[3 * (size_t)a + axis] < pos[3 * (size_t)b + axis]; });
}

// NodeGroups::determinePositions (DataStructures/NodeGroups.cpp:413-443)
// sorts the vertex ids with std::sort by (class, colour, number of neighbour
// elements), every fixed vertex comparing equal to every other; the order
// among equal keys is the library's own, so the oracle makes the same call.
extern "C" void om_sort_node_order(int64_t n, const int* types, const int* groups, const int64_t* valence, int* out)
{
    std::vector<int> indices(n);
    std::iota(indices.begin(), indices.end(), 0);
    std::sort(indices.begin(), indices.end(), [&](int a, int b) {
        if (types[a] == types[b])
        {
            if (types[a] == 0) return false;
            if (groups[a] == groups[b]) return valence[a] < valence[b];
            return groups[a] < groups[b];
        }
        return types[a] < types[b];
    });
    std::copy(indices.begin(), indices.end(), out);
}
