// Quality evaluation for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs inside
// a host framework which owns every device allocation (and hands out only
// views of buffers it manages), code that runs under a memory budget that is
// already fully committed, or code that must not allocate once a real-time
// loop has started.  They can still evaluate a mesh they hold in device
// memory through gm_evaluate_noalloc, which allocates nothing: its only
// scratch, the evaluation kernel's per-block partial results, lives in the
// file-scope device array below.
//
// That array is part of this library's image, so every GPU that loads the
// library holds it (kNoAllocMaxPartials * sizeof(EvalPartial) = 104 KiB)
// until the process exits.  All calls on one device share it and it keeps
// the last call's contents; each call overwrites every partial it reads, and
// the evaluation kernel returns the array's ticket word and bucket totals
// (zero when the library is loaded) to zero at the end of every launch, so
// no clearing is needed, but two calls that overlap on the GPU (for instance
// on two streams) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/gpumesh_gb300.h"
#include "gm_internal.h"
#include "gm_launch.h"

namespace gm {

// 1024 block partials: a grid of at most 1024 blocks of 256 threads (the
// evaluation launch also caps the grid at one wave, its resident blocks per
// SM times the SMs, which is below 1024 on a 152-SM GB300 for every kernel
// variant).  The element limit, 2^24, bounds each thread's FP32 partial sum
// of 1/q: the smallest one-wave grid of the variants (2 resident blocks per
// SM for the general-metric kernels, 304 blocks on 152 SMs) gives a thread
// at most 216 elements before the FP64 block reduction; the tet and hex
// mean-ratio kernels (4-6 blocks per SM) give at most 108.
constexpr int kNoAllocMaxPartials = 1024;
constexpr uint64_t kNoAllocMaxElements = (uint64_t)1 << 24;
static_assert(eval_scratch_slots(kNoAllocMaxPartials) <= kNoAllocMaxPartials, "scratch of a 1024-block grid");

static __device__ __align__(256) EvalPartial g_noalloc_partials[kNoAllocMaxPartials];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
EvalPartial* g_partials_addr[kMaxDevices] = {};

// The device address of g_noalloc_partials on the current device.  In host
// code the array's name is only a host-side stand-in, so the address is
// looked up once per device (with that device current, on the first call)
// and cached until the process exits.  A device reset (cudaDeviceReset, or
// the primary context torn down and created again) reloads the library's
// module, possibly at another address, so this entry point does not support
// calls after a reset of a device it has already been called on.
cudaError_t partials_address(int device, EvalPartial** out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[device])
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_partials_addr[device] = static_cast<EvalPartial*>(p);
    }
    *out = g_partials_addr[device];
    return cudaSuccess;
}

// The sampler uniforms, as AbstractSampler sets them (scaling, its square
// and cube, the aspect ratio, and its fixed rotation: pi/4 about +z then
// pi/4 about -y, Samplers/AbstractSampler.cpp:30-51).
Crew make_crew(int sampler, int measurer, int evaluator, double scaling, double aspect)
{
    Crew c{};
    c.sampler = sampler;
    c.measurer = measurer;
    c.evaluator = evaluator;
    c.scaling = scaling;
    c.scaling2 = scaling * scaling;
    c.scaling3 = c.scaling2 * scaling;
    c.aspect = aspect;
    auto rotate = [](const double* m, double angle, const double* axis_in, double* out) {
        double n = 1.0 / std::sqrt(axis_in[0] * axis_in[0] + axis_in[1] * axis_in[1] + axis_in[2] * axis_in[2]);
        double a[3] = {axis_in[0] * n, axis_in[1] * n, axis_in[2] * n};
        double co = std::cos(angle), si = std::sin(angle);
        double R[9];  // column-major rotation about a
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i)
            {
                double v = (1.0 - co) * a[j] * a[i];
                if (i == j) v += co;
                else
                {
                    int k = 3 - i - j;
                    double sgn = ((j + 1) % 3 == i) ? 1.0 : -1.0;
                    v += sgn * si * a[k];
                }
                R[j * 3 + i] = v;
            }
        for (int j = 0; j < 3; ++j)
            for (int r = 0; r < 3; ++r)
                out[j * 3 + r] = m[r] * R[j * 3] + m[3 + r] * R[j * 3 + 1] + m[6 + r] * R[j * 3 + 2];
    };
    const double pi = 3.14159265358979323846;
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, z[3] = {0, 0, 1}, my[3] = {0, -1, 0};
    double A[9];
    rotate(I, pi / 4.0, z, A);
    rotate(A, pi / 4.0, my, c.rot);
    for (int j = 0; j < 3; ++j)
        for (int r = 0; r < 3; ++r) c.rotinv[j * 3 + r] = c.rot[r * 3 + j];
    return c;
}

gm_status fail(gm_status s, const std::string& msg)
{
    set_error(msg);
    return s;
}

}  // namespace
}  // namespace gm

using namespace gm;

extern "C" gm_status gm_evaluate_noalloc(uint32_t nv, const void* pos, uint32_t nt, const uint32_t* tets, uint32_t np,
                                         const uint32_t* pris, uint32_t nh, const uint32_t* hexs, int32_t sampler,
                                         int32_t measurer, int32_t evaluator, double scaling, double aspect_ratio,
                                         gm_quality* out, void* stream)
{
    const uint64_t total = (uint64_t)nt + np + nh;
    if (total > kNoAllocMaxElements)
        return fail(GM_ERR_UNSUPPORTED, "gm_evaluate_noalloc evaluates at most " +
                                            std::to_string(kNoAllocMaxElements) + " elements; this mesh has " +
                                            std::to_string(total));
    if (!pos || !out || nv == 0) return fail(GM_ERR_INVALID_ARG, "gm_evaluate_noalloc: null positions or output");
    if ((nt && !tets) || (np && !pris) || (nh && !hexs))
        return fail(GM_ERR_INVALID_ARG, "gm_evaluate_noalloc: null connectivity");
    if (sampler >= GM_SAMPLER_LOCAL && sampler <= GM_SAMPLER_TEXTURE)
        return fail(GM_ERR_UNSUPPORTED, "gm_evaluate_noalloc: the background-mesh samplers need a resident mesh "
                                        "(gm_mesh_set_crew, gm_evaluate)");
    if (sampler < 0 || sampler > 2 || measurer < 0 || measurer > 1 || evaluator < 0 || evaluator > 1)
        return fail(GM_ERR_INVALID_ARG, "gm_evaluate_noalloc: unknown sampler, measurer or evaluator");
    if (total == 0) return fail(GM_ERR_INVALID_ARG, "gm_evaluate_noalloc: mesh has no elements");
    if (((uintptr_t)pos & 15) || ((uintptr_t)tets & 15) || ((uintptr_t)hexs & 15) || ((uintptr_t)pris & 7))
        return fail(GM_ERR_INVALID_ARG, "gm_evaluate_noalloc: positions, tets and hexs must be 16-byte aligned, "
                                        "prisms 8-byte aligned");

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return fail(GM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (device < 0 || device >= kMaxDevices) return fail(GM_ERR_UNSUPPORTED, "device index out of range");
    EvalPartial* partials = nullptr;
    e = partials_address(device, &partials);
    if (e != cudaSuccess) return fail(GM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

    MeshView m{};
    m.nv = nv;
    m.nt = nt;
    m.np = np;
    m.nh = nh;
    m.pos = const_cast<float4*>(static_cast<const float4*>(pos));
    m.tets = reinterpret_cast<const uint4*>(tets);
    m.pris = pris;
    m.hexs = reinterpret_cast<const uint4*>(hexs);
    const Crew crew = make_crew(sampler, measurer, evaluator, scaling, aspect_ratio);
    // the same kernel variant gm_evaluate selects, so both give the same per-element qualities
    int variant = evaluator == GM_EVALUATOR_METRIC_CONFORMITY
                      ? (sampler == GM_SAMPLER_ANALYTIC ? kVarMC : kVarMCDiag)
                      : (measurer == GM_MEASURER_METRIC_WISE ? kVarMRWise : kVarMRFree);
    int maxk = (nt == 0 && np == 0 && nh) ? 9 : ((np || nh) ? 8 : 4);
    uint64_t need = (total + 255) / 256;
    int blocks = (int)(need < (uint64_t)kNoAllocMaxPartials ? need : (uint64_t)kNoAllocMaxPartials);
    static_assert(sizeof(Quality) == sizeof(gm_quality), "quality layout");
    e = launch_evaluate(variant, maxk, m, crew, partials, blocks, reinterpret_cast<Quality*>(out),
                        static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(GM_ERR_CUDA, std::string("evaluation launch: ") + cudaGetErrorString(e));
    return GM_OK;
}
