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

extern "C" void om_argsort_axis(const double* pos, int64_t n, int axis, uint32_t* out)
{
    std::iota(out, out + n, 0u);
    std::sort(out, out + n, [pos, axis](uint32_t a, uint32_t b) { return pos[3 * (size_t)a + axis] < pos[3 * (size_t)b + axis]; });
}
