// Device-side data views, geometry and quality measures for sm_103a.
//
// Every measure is a template on the arithmetic type: the relocation and
// evaluation kernels run them in FP32, and the acceptance test on
// near-degenerate patches re-runs them in FP64.  The formulas restate the
// reference's CPU measures:
//   mean ratio       Evaluators/MeanRatioEvaluator.cpp:22-167
//   metric conform.  Evaluators/MetricConformityEvaluator.cpp:25-224
//   measurers        Measurers/MetricFreeMeasurer.cpp:27-105,
//                    Measurers/MetricWiseMeasurer.cpp:64-188
//   samplers         Samplers/UniformSampler.cpp:45, AbstractSampler.cpp:190-208
//   projections      Boundaries/Constraints/{Face,Edge,Vertex,Volume}Constraint.cpp,
//                    Boundaries/SphereBoundary.cpp:42-45, ShellBoundary.cpp:41-49,
//                    PipeBoundary.cpp:42-116
// Positive element qualities are carried as reciprocals (1/q), which is all
// a harmonic mean needs, so the common path has no division.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gm {

constexpr int kTet = 0;
constexpr int kPri = 2;
constexpr int kHex = 3;

enum : int { kSamplerUniform = 0, kSamplerAnalytic = 1, kSamplerSine = 2, kSamplerLocal = 3, kSamplerKdTree = 4,
              kSamplerTexture = 5 };
// bound of a kd-tree descent (trees are built at most this deep)
constexpr int kKdMaxDepth = 64;
enum : int { kMeasurerMetricFree = 0, kMeasurerMetricWise = 1 };
enum : int { kEvalMeanRatio = 0, kEvalMetricConformity = 1 };
enum : int
{
    kConVolume = 0,
    kConPlane = 1,
    kConSegment = 2,
    kConSphere = 3,
    kConPoint = 4,
    kConShellInner = 5,   // ShellBoundary::InFace: the radius-0.5 sphere
    kConPipeCylinder = 6, // PipeBoundary::CylinderFace: the U-bend pipe wall
    kConPipeCircle = 7    // PipeBoundary::Y*CircleEdge: a pipe-end circle, centre in a
};

// a kd-tree separator plane in FP64: normal xyz, offset w
struct alignas(32) Plane4d
{
    double x, y, z, w;
};

// LocalSampler's background mesh in device memory (Samplers/LocalSampler.cpp:
// 352-429): the mesh as it was when the crew was set, split into tets, their
// face neighbours, the analytic metric at its vertices, and a uniform grid
// whose every cell names a tet near it, where a walk starts.
struct LocalField
{
    uint32_t nbg;
    const uint4* tv;      // background tet vertices
    const uint4* tn;      // neighbour across the face opposite vertex k (0xffffffff: none)
    const float4* pf;     // background vertex positions
    const double* pd;     // the same in FP64, 3 per vertex
    const float4* mf;     // vertex metrics, 2 per vertex: (xx yy zz xy), (xz yz 0 0)
    const double* md;
    const uint32_t* cell;    // grid cell -> start tet
    const uint32_t* ecache;  // element (tets, prisms, hexes) -> its first background tet; null: none
    uint32_t nt, np, ne;     // tets, prisms and elements the caches were built for
    int g[3];
    double lo[3], inv_h[3];
    // KdTreeSampler: nodes in pre-order; children (-1: none), separator plane
    // (normal xyz, offset w), per node the leaf metric xx yy zz xy xz yz
    const int2* kd_child;
    const float4* kd_sepf;
    const Plane4d* kd_sepd;
    const float4* kd_mf;  // 2 per node, as mf
    const double* kd_md;
    // TextureSampler: metric samples at the cell centres of a tg[0] x tg[1] x
    // tg[2] grid over [tmin, tmin + text], x fastest
    int tg[3];
    double tmin[3], text[3];
    const float4* tex_mf;  // 2 per cell, as mf
    const double* tex_md;
};

// the element a metric is sampled for, as a walk start hint:
// type << 27 | element id (kNoHint: none)
constexpr uint32_t kNoHint = 0xffffffffu;
__device__ __forceinline__ uint32_t elem_hint(int type, uint32_t id) { return ((uint32_t)type << 27) | id; }

// smoothing-wide parameters, passed by value to every kernel
struct Crew
{
    int sampler, measurer, evaluator, pad;
    double scaling, scaling2, scaling3, aspect;
    double rot[9], rotinv[9];  // column-major, AbstractSampler::_rotMat / _rotInv
    const LocalField* local;   // kSamplerLocal, kSamplerKdTree, kSamplerTexture
};

// one boundary constraint (index = constraint id)
struct Constraint
{
    int kind;
    float a[3];  // plane point / segment start / point
    float b[3];  // plane normal (normalized) / segment end
    float u[3];  // segment direction (normalized)
    float len;   // segment length
    double ad[3], bd[3], ud[3];
    double lend;
};

// read-only device view of one mesh
struct MeshView
{
    uint32_t nv, nt, np, nh;
    float4* pos;
    const uint4* tets;
    const uint32_t* pris;  // 6 per prism
    const uint4* hexs;     // 2 per hex
    const uint32_t* ve_off;
    const uint32_t* ve;    // packed (type, local, id)
    const uint32_t* vv_off;
    const uint32_t* vv;
    const int32_t* cid;
    const Constraint* con;
    int ncon;
    uint32_t ve_len, vv_len;  // entries of ve / vv (bounds-checked builds)
    unsigned int* bounds;     // the mesh's bounds status: {what, index}, 0 = clean
};

// Bounds-checked indices.  In a library built with GM_BOUNDS_CHECK, every
// connectivity and CSR index the kernels read through is compared with the
// length of the array it indexes; the first index found out of range is
// recorded in the mesh's status word (which array, then the index) and
// replaced by 0, so that the read stays inside the array.  The host reads
// the word back (gm_mesh_bounds_status, and every synchronising call of that
// build) and reports it through gm_last_error.  In the ordinary build the
// macro is the bare index.
enum BoundsWhat : unsigned int
{
    kBoundsPosition = 1,   // a vertex index (connectivity, neighbour, member) >= nv
    kBoundsNeighbourElem,  // a vertex->element CSR index >= its length
    kBoundsNeighbourVert,  // a vertex->vertex CSR index >= its length
    kBoundsTet,            // a tet id >= nt
    kBoundsPrism,          // a prism id >= np
    kBoundsHex,            // a hex id >= nh
    kBoundsCorner,         // a GETMe corner index >= 4 nt + 6 np + 8 nh
};
#ifdef GM_BOUNDS_CHECK
static __device__ __noinline__ uint32_t bounds_fail(unsigned int* status, unsigned int what, uint32_t index)
{
    if (status && atomicCAS(status, 0u, what) == 0u) atomicExch(status + 1, index);
    return 0u;
}
#define GM_IX(m, index, len, what)                                                                      \
    ((uint32_t)(index) < (uint32_t)(len) ? (uint32_t)(index)                                           \
                                         : ::gm::bounds_fail((m).bounds, (what), (uint32_t)(index)))
#else
#define GM_IX(m, index, len, what) (index)
#endif

__device__ __forceinline__ int ref_type(uint32_t r) { return (int)(r >> 30); }
__device__ __forceinline__ int ref_local(uint32_t r) { return (int)((r >> 27) & 7u); }
__device__ __forceinline__ uint32_t ref_id(uint32_t r) { return r & ((1u << 27) - 1); }

// ---------------------------------------------------------------------------
// small vector algebra
// ---------------------------------------------------------------------------
template <class R>
struct V3
{
    R x, y, z;
};
template <class R> __device__ __forceinline__ V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> __device__ __forceinline__ V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> __device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> __device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b)
{
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class R> __device__ __forceinline__ R det3(V3<R> c0, V3<R> c1, V3<R> c2)
{
    // determinant of the matrix with columns c0, c1, c2
    return c0.x * (c1.y * c2.z - c2.y * c1.z) - c1.x * (c0.y * c2.z - c2.y * c0.z) + c2.x * (c0.y * c1.z - c1.y * c0.z);
}
template <class R> __device__ __forceinline__ R rsqrt_(R x);
template <> __device__ __forceinline__ float rsqrt_<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_<double>(double x) { return rsqrt(x); }
template <class R> __device__ __forceinline__ R sqrt_(R x);
template <> __device__ __forceinline__ float sqrt_<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <class R> __device__ __forceinline__ V3<R> normalize(V3<R> a) { return a * rsqrt_<R>(dot(a, a)); }
template <class R> __device__ __forceinline__ R length(V3<R> a) { return sqrt_<R>(dot(a, a)); }

// the U-bend pipe (Boundaries/PipeBoundary.cpp:3-6, 42-56, 95-116): radius 0.3,
// end faces normal to -x
template <class R>
__device__ __forceinline__ V3<R> pipe_cylinder(V3<R> p)
{
    V3<R> center;
    if (p.x < R(0.5)) center = V3<R>{p.x, p.y < R(0) ? R(-0.5) : R(0.5), R(0)};  // straights
    else  // arc
    {
        center = p - V3<R>{R(0.5), R(0), p.z};
        center = normalize(center) * R(0.5);
        center = V3<R>{R(0.5), R(0), R(0)} + center;
    }
    const V3<R> dist = p - center;
    return center + normalize(dist) * R(0.3);
}

template <class R>
__device__ __forceinline__ V3<R> pipe_circle(V3<R> c, V3<R> p)
{
    const V3<R> n{R(-1), R(0), R(0)};
    const V3<R> dist = p - c;
    const R offset = dot(dist, n);
    const V3<R> ext = dist - n * offset;
    return c + normalize(ext) * R(0.3);
}

// Single-instruction FP32 approximations (PTX ISA: ex2 / lg2 / rcp / sqrt
// .approx.ftz.f32, relative error of order 2^-22).  Subnormal inputs flush
// to zero; no quantity of the quality measures is subnormal for meshes whose
// edges are above 1e-12.
__device__ __forceinline__ float ex2_fast(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_fast(float x)
{
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_fast(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_fast(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// |x|^(-2/3) for x != 0, and |x|^(2/3): 2^(-+2/3 log2|x|)
__device__ __forceinline__ float pow_m23(float x) { return ex2_fast(-0.666666666666666667f * lg2_fast(fabsf(x))); }
__device__ __forceinline__ double pow_m23(double x) { return pow(fabs(x), -2.0 / 3.0); }
__device__ __forceinline__ float pow_23(float x) { return ex2_fast(0.666666666666666667f * lg2_fast(fabsf(x))); }
__device__ __forceinline__ double pow_23(double x) { return pow(fabs(x), 2.0 / 3.0); }
__device__ __forceinline__ float cbrt_(float x) { return cbrtf(x); }
__device__ __forceinline__ double cbrt_(double x) { return cbrt(x); }

template <class R> __device__ __forceinline__ R sgn(R x) { return (R)((R(0) < x) - (x < R(0))); }

// symmetric 3x3 metric
template <class R>
struct Sym3
{
    R xx, yy, zz, xy, xz, yz;
};

template <class R> __device__ __forceinline__ V3<R> to(float4 p) { return {(R)p.x, (R)p.y, (R)p.z}; }

// ---------------------------------------------------------------------------
// samplers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sinpi_(float x) { return sinpif(x); }
__device__ __forceinline__ double sinpi_(double x) { return sinpi(x); }

// AbstractSampler::vertMetric (Samplers/AbstractSampler.cpp:190-208):
// R^T diag(sx^2, s^2, s^2) R with sx = s * a^(((1 - cos(2.5 pi (Rp).x))/2)^a)
template <class R>
__device__ __noinline__ Sym3<R> analytic_metric(const Crew& c, V3<R> p)
{
    const double* m = c.rot;
    R rx = (R)m[0] * p.x + (R)m[3] * p.y + (R)m[6] * p.z;
    R x = rx * R(2.5 * 3.14159265358979323846);
    R a = (R)c.aspect;
    R cc = (R(1) - cos(x)) / R(2);
    R sizeX = (R)c.scaling * pow(a, pow(cc, a));
    R Mx = sizeX * sizeX, My = (R)c.scaling2;
    // rows of R are (m[0],m[3],m[6]), (m[1],m[4],m[7]), (m[2],m[5],m[8]); M = sum_i d_i r_i r_i^T
    R r0[3] = {(R)m[0], (R)m[3], (R)m[6]};
    R r1[3] = {(R)m[1], (R)m[4], (R)m[7]};
    R r2[3] = {(R)m[2], (R)m[5], (R)m[8]};
    Sym3<R> M;
    M.xx = Mx * r0[0] * r0[0] + My * (r1[0] * r1[0] + r2[0] * r2[0]);
    M.yy = Mx * r0[1] * r0[1] + My * (r1[1] * r1[1] + r2[1] * r2[1]);
    M.zz = Mx * r0[2] * r0[2] + My * (r1[2] * r1[2] + r2[2] * r2[2]);
    M.xy = Mx * r0[0] * r0[1] + My * (r1[0] * r1[1] + r2[0] * r2[1]);
    M.xz = Mx * r0[0] * r0[2] + My * (r1[0] * r1[2] + r2[0] * r2[2]);
    M.yz = Mx * r0[1] * r0[2] + My * (r1[1] * r1[2] + r2[1] * r2[2]);
    return M;
}

// LocalSampler::metricAt (Samplers/LocalSampler.cpp:212-311) on the device:
// the walk starts at the grid cell's tet instead of a per-element cache (the
// reference starts at the element's first background tet); each step leaves
// the current tet through the face that a ray from its centroid (or from one
// of four weighted interior points) crosses, at most kLocalWalk steps; then
// the vertex metrics are interpolated barycentrically, with the coordinates
// clamped when the point lies outside the background mesh.  A point within
// the reference's -1e-4 tolerance of a face may settle in either tet, so the
// metric agrees with the CPU walk's to that tolerance, not bit for bit.
constexpr int kLocalWalk = 512;
// MeshTet::tris (DataStructures/Mesh.cpp:30-35): the face opposite vertex f,
// three 2-bit vertex indices
__device__ __forceinline__ int tet_face(int f) { return f == 0 ? 0x39 : f == 1 ? 0x2c : f == 2 ? 0x34 : 0x18; }

template <class R>
__device__ __forceinline__ V3<R> local_pos(const LocalField& L, uint32_t v)
{
    if constexpr (sizeof(R) == 8)
        return V3<R>{(R)L.pd[3 * (size_t)v], (R)L.pd[3 * (size_t)v + 1], (R)L.pd[3 * (size_t)v + 2]};
    else
    {
        const float4 q = __ldg(&L.pf[v]);
        return V3<R>{(R)q.x, (R)q.y, (R)q.z};
    }
}

// a metric stored as two float4 (xx yy zz xy), (xz yz 0 0): two vector loads
template <class R>
__device__ __forceinline__ void metric_pair(const float4* base, size_t i, R* m)
{
    const float4 a = __ldg(&base[2 * i]), b = __ldg(&base[2 * i + 1]);
    m[0] = (R)a.x;
    m[1] = (R)a.y;
    m[2] = (R)a.z;
    m[3] = (R)a.w;
    m[4] = (R)b.x;
    m[5] = (R)b.y;
}

template <class R>
__device__ __forceinline__ bool local_params(const V3<R>* vp, V3<R> p, R coor[4])
{
    // y = T^-1 (p - v3), T = [v0 - v3, v1 - v3, v2 - v3]
    const V3<R> c0 = vp[0] - vp[3], c1 = vp[1] - vp[3], c2 = vp[2] - vp[3], d = p - vp[3];
    const R det = det3(c0, c1, c2);
    const R id = R(1) / det;
    coor[0] = det3(d, c1, c2) * id;
    coor[1] = det3(c0, d, c2) * id;
    coor[2] = det3(c0, c1, d) * id;
    coor[3] = R(1) - (coor[0] + coor[1] + coor[2]);
    const R eps = R(-1e-4);
    return coor[0] >= eps && coor[1] >= eps && coor[2] >= eps && coor[3] >= eps;
}

template <class R>
__device__ __forceinline__ bool local_tri_intersect(V3<R> v1, V3<R> v2, V3<R> v3, V3<R> orig, V3<R> dir)
{
    const V3<R> e1 = v2 - v1, e2 = v3 - v1;
    const V3<R> pvec = cross(dir, e2);
    const R det = dot(pvec, e1);
    if (det < R(1e-12)) return false;
    const V3<R> tvec = orig - v1;
    const R u = dot(tvec, pvec);
    if (u < R(0) || u > det) return false;
    const V3<R> qvec = cross(tvec, e1);
    const R v = dot(dir, qvec);
    return !(v < R(0) || v + u > det);
}

// start of the walk: the element's first background tet, as the reference's
// measures set the sampler cache per element (so that a point outside the
// background clamps in the same tet), else the grid cell's tet
__device__ __forceinline__ uint32_t local_start_elem(const LocalField& L, uint32_t hint)
{
    if (hint == kNoHint || !L.ecache) return kNoHint;
    const uint32_t type = hint >> 27, id = hint & ((1u << 27) - 1);
    const uint32_t e = id + (type == (uint32_t)kTet ? 0u : type == (uint32_t)kPri ? L.nt : L.nt + L.np);
    return e < L.ne ? __ldg(&L.ecache[e]) : kNoHint;  // a mesh since re-uploaded: no cache
}

// the walk from background tet t to the tet holding p, then the interpolation
template <class R>
__device__ __forceinline__ Sym3<R> local_walk(const LocalField& L, V3<R> p, uint32_t t)
{
    uint4 tv = __ldg(&L.tv[t]);
    V3<R> vp[4] = {local_pos<R>(L, tv.x), local_pos<R>(L, tv.y), local_pos<R>(L, tv.z), local_pos<R>(L, tv.w)};
    R coor[4];
    bool unreachable = false;
    int steps = 0;
    while (!local_params(vp, p, coor))
    {
        if (++steps > kLocalWalk)
        {
            unreachable = true;
            break;
        }
        V3<R> orig = (vp[0] + vp[1] + vp[2] + vp[3]) * R(0.25);
        V3<R> dir = normalize(orig - p);
        int exit_face = -1;
        for (int trial = -1; trial < 4 && exit_face < 0; ++trial)
        {
            if (trial >= 0)
            {
                const R w[4] = {R(1), R(2), R(3), R(4)};
                orig = (vp[0] * w[(trial + 0) % 4] + vp[1] * w[(trial + 1) % 4] + vp[2] * w[(trial + 2) % 4] +
                        vp[3] * w[(trial + 3) % 4]) * R(0.1);
                dir = normalize(orig - p);
            }
#pragma unroll
            for (int f = 0; f < 4; ++f)
            {
                const int q = tet_face(f);
                if (local_tri_intersect(vp[q & 3], vp[(q >> 2) & 3], vp[q >> 4], orig, dir))
                {
                    exit_face = f;
                    break;
                }
            }
        }
        if (exit_face < 0)
        {
            unreachable = true;
            break;
        }
        const uint4 tn = __ldg(&L.tn[t]);
        const uint32_t nb = exit_face == 0 ? tn.x : exit_face == 1 ? tn.y : exit_face == 2 ? tn.z : tn.w;
        if (nb == 0xffffffffu)
        {
            unreachable = true;
            break;
        }
        t = nb;
        tv = __ldg(&L.tv[t]);
        vp[0] = local_pos<R>(L, tv.x);
        vp[1] = local_pos<R>(L, tv.y);
        vp[2] = local_pos<R>(L, tv.z);
        vp[3] = local_pos<R>(L, tv.w);
    }
    if (unreachable)
    {
        R sum = R(0);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            if (coor[k] < R(0)) coor[k] = R(0);
            else sum += coor[k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) coor[k] /= sum;
    }
    const uint32_t vv[4] = {tv.x, tv.y, tv.z, tv.w};
    Sym3<R> M{R(0), R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        R m6[6];
        if constexpr (sizeof(R) == 8)
            for (int j = 0; j < 6; ++j) m6[j] = (R)L.md[6 * (size_t)vv[k] + j];
        else
            metric_pair(L.mf, vv[k], m6);
        M.xx += coor[k] * m6[0];
        M.yy += coor[k] * m6[1];
        M.zz += coor[k] * m6[2];
        M.xy += coor[k] * m6[3];
        M.xz += coor[k] * m6[4];
        M.yz += coor[k] * m6[5];
    }
    return M;
}

template <class R>
__device__ __noinline__ Sym3<R> local_metric(const LocalField& L, V3<R> p, uint32_t hint)
{
    uint32_t t = local_start_elem(L, hint);
    if (t == kNoHint)
    {
        int ci[3];
        const R pc[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            const R f = (pc[k] - (R)L.lo[k]) * (R)L.inv_h[k];
            int i = f > R(0) ? (int)f : 0;
            ci[k] = i < L.g[k] ? i : L.g[k] - 1;
        }
        t = L.cell[((size_t)ci[2] * L.g[1] + ci[1]) * L.g[0] + ci[0]];
    }
    return local_walk(L, p, t);
}

// KdTreeSampler::metricAt (Samplers/KdTreeSampler.cpp:218-247; the CUDA
// driver resources/cuda/Sampling/KdTree.cu:24-45): descend to the leaf on the
// side of each node's separator plane, return the leaf's metric
template <class R>
__device__ __noinline__ Sym3<R> kd_metric(const LocalField& L, V3<R> p)
{
    int node = 0;
    for (int depth = 0; depth < kKdMaxDepth; ++depth)
    {
        const int2 ch = __ldg(&L.kd_child[node]);
        if (ch.x < 0 && ch.y < 0) break;
        R d;
        if constexpr (sizeof(R) == 8)
        {
            const Plane4d s = L.kd_sepd[node];
            d = p.x * s.x + p.y * s.y + p.z * s.z - s.w;
        }
        else
        {
            const float4 s = __ldg(&L.kd_sepf[node]);
            d = p.x * s.x + p.y * s.y + p.z * s.z - s.w;
        }
        const int next = d < R(0) ? ch.x : ch.y;
        if (next < 0) break;
        node = next;
    }
    R m[6];
    if constexpr (sizeof(R) == 8)
    {
#pragma unroll
        for (int j = 0; j < 6; ++j) m[j] = (R)L.kd_md[6 * (size_t)node + j];
    }
    else
        metric_pair(L.kd_mf, (size_t)node, m);
    return Sym3<R>{m[0], m[1], m[2], m[3], m[4], m[5]};
}

// TextureSampler::metricAt (Samplers/TextureSampler.cpp:450-488): trilinear
// interpolation between the eight cell centres around p, clamped at the
// grid's border; glm::mix(a, b, t) = a + (b - a) t per entry
template <class R>
__device__ __forceinline__ void tex_cell_metric(const LocalField& L, int i, int j, int k, R* m)
{
    const size_t c = ((size_t)k * L.tg[1] + j) * L.tg[0] + i;
    if constexpr (sizeof(R) == 8)
    {
#pragma unroll
        for (int q = 0; q < 6; ++q) m[q] = (R)L.tex_md[6 * c + q];
    }
    else
        metric_pair(L.tex_mf, c, m);
}

template <class R>
__device__ __noinline__ Sym3<R> tex_metric(const LocalField& L, V3<R> p)
{
    const R pc[3] = {p.x, p.y, p.z};
    int i0[3], i1[3];
    R a[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        const R ext = (R)L.text[k], mn = (R)L.tmin[k];
        const int n = L.tg[k];
        const R cs = ext / (R)n;
        const R minb = mn, maxb = mn + ext - cs * R(1.5);
        const R q = pc[k] + (-cs) / R(2);
        const R t1 = q < minb ? minb : q;     // glm::max(q, minb)
        const R cp0 = maxb < t1 ? maxb : t1;  // glm::min(., maxb)
        // cellId: truncation, then clamped to the grid; cp0 is clamped above,
        // so |r| <= n + 1 (a NaN converts to 0)
        const R r = (cp0 - mn) / ext * (R)n;
        int c = (int)r;
        c = c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
        i0[k] = c;
        i1[k] = c + 1 < n - 1 ? c + 1 : n - 1;
        const R c0 = cs * ((R)c + R(0.5));
        const R f = (pc[k] - (mn + c0)) / cs;
        a[k] = f < R(0) ? R(0) : (f > R(1) ? R(1) : f);
    }
    R m000[6], m100[6], m010[6], m110[6], m001[6], m101[6], m011[6], m111[6];
    tex_cell_metric(L, i0[0], i0[1], i0[2], m000);
    tex_cell_metric(L, i1[0], i0[1], i0[2], m100);
    tex_cell_metric(L, i0[0], i1[1], i0[2], m010);
    tex_cell_metric(L, i1[0], i1[1], i0[2], m110);
    tex_cell_metric(L, i0[0], i0[1], i1[2], m001);
    tex_cell_metric(L, i1[0], i0[1], i1[2], m101);
    tex_cell_metric(L, i0[0], i1[1], i1[2], m011);
    tex_cell_metric(L, i1[0], i1[1], i1[2], m111);
    R r[6];
#pragma unroll
    for (int q = 0; q < 6; ++q)
    {
        const R x00 = m000[q] + (m100[q] - m000[q]) * a[0], x10 = m010[q] + (m110[q] - m010[q]) * a[0];
        const R x01 = m001[q] + (m101[q] - m001[q]) * a[0], x11 = m011[q] + (m111[q] - m011[q]) * a[0];
        const R y0 = x00 + (x10 - x00) * a[1], y1 = x01 + (x11 - x01) * a[1];
        r[q] = y0 + (y1 - y0) * a[2];
    }
    return Sym3<R>{r[0], r[1], r[2], r[3], r[4], r[5]};
}

template <class R>
__device__ __forceinline__ Sym3<R> metric_at(const Crew& c, V3<R> p, uint32_t hint = kNoHint)
{
    if (c.sampler == kSamplerSine)
    {
        // s^2 * diag(1 + 9 sin^2(4 pi x), 1, 1)
        R s = sinpi_(R(4) * p.x);
        R s2 = (R)c.scaling2;
        return {s2 * (R(1) + R(9) * s * s), s2, s2, R(0), R(0), R(0)};
    }
    if (c.sampler == kSamplerAnalytic) return analytic_metric(c, p);
    if (c.sampler == kSamplerLocal) return local_metric(*c.local, p, hint);
    if (c.sampler == kSamplerKdTree) return kd_metric(*c.local, p);
    if (c.sampler == kSamplerTexture) return tex_metric(*c.local, p);
    R s2 = (R)c.scaling2;
    return {s2, s2, s2, R(0), R(0), R(0)};
}

template <class R> __device__ __forceinline__ R quad_form(const Sym3<R>& M, V3<R> v)
{
    return v.x * (M.xx * v.x + M.xy * v.y + M.xz * v.z) + v.y * (M.xy * v.x + M.yy * v.y + M.yz * v.z) +
           v.z * (M.xz * v.x + M.yz * v.y + M.zz * v.z);
}

// ---------------------------------------------------------------------------
// measurers
// ---------------------------------------------------------------------------

// MetricWiseMeasurer::riemannianDistance, localized segment division
// (Measurers/MetricWiseMeasurer.cpp:64-116), with the subdivision depth
// bounded at 2^16 segments so that a pathological metric cannot loop forever.
template <class R>
__device__ __noinline__ R metric_wise_distance(const Crew& c, V3<R> a, V3<R> b)
{
    int curr = 0, base = 2;
    R len = 0;
    V3<R> d = b - a;
    V3<R> bv = d * (R(1) / (R)base);
    for (int guard = 0; curr < base && guard < 4096; ++guard)
    {
        R p0 = (R(curr) + R(0.5)) / (R)base;
        R p1 = (R(curr) + R(1.5)) / (R)base;
        R l0 = sqrt_<R>(quad_form(metric_at(c, a + d * p0), bv));
        R l1 = sqrt_<R>(quad_form(metric_at(c, a + d * p1), bv));
        R sum = l0 + l1;
        R diff = fabs(l0 - l1) / (sum / R(2));
        if (diff < R(0.01) || base >= (1 << 16))
        {
            len += sum;
            curr += 2;
            if ((curr & 2) == 0)
            {
                base >>= 1;
                curr >>= 1;
            }
            bv = d * (R(1) / (R)base);
        }
        else
        {
            base <<= 1;
            curr <<= 1;
            bv = bv * R(0.5);
        }
    }
    return len;
}

// crew variants the kernels are specialised on: evaluator x measurer
// kVarMCDiag: metric conformity with a diagonal metric (the uniform and the
// sine-graded samplers), whose 3x3 products reduce to their diagonals
enum : int { kVarMRFree = 0, kVarMRWise = 1, kVarMC = 2, kVarMCWise = 3, kVarMCDiag = 4 };
template <int VAR> struct VarTraits
{
    static constexpr bool mean_ratio = VAR == kVarMRFree || VAR == kVarMRWise;
    static constexpr bool metric_wise = VAR == kVarMRWise || VAR == kVarMCWise;
    static constexpr bool diag_metric = VAR == kVarMCDiag;
};

// MetricFreeMeasurer::riemannianSegment = (b - a) * scaling.  The FP32 path
// leaves the scaling out: every quantity built from metric-free segments
// (mean ratio, volume ratios) is invariant to a common scale, so only the
// FP64 path, which restates the reference operation for operation, applies it.
template <int VAR, class R>
__device__ __forceinline__ V3<R> segment(const Crew& c, V3<R> a, V3<R> b)
{
    if (VarTraits<VAR>::metric_wise) return normalize(b - a) * metric_wise_distance(c, a, b);
    if (sizeof(R) == sizeof(float)) return b - a;
    return (b - a) * (R)c.scaling;
}

// ---------------------------------------------------------------------------
// element quality.  EQ carries 1/q when the element is valid (q > 0) and q
// itself otherwise.
// ---------------------------------------------------------------------------
template <class R>
struct EQ
{
    R v;       // 1/q if pos, else q
    bool pos;  // q > 0
};

// mean-ratio corner: q = sign(det) 3 |det|^(2/3) / |F|^2
template <class R>
__device__ __forceinline__ void mr_corner(V3<R> c0, V3<R> c1, V3<R> c2, R& rq, R& q, bool& pos)
{
    R det = det3(c0, c1, c2);
    R f2 = dot(c0, c0) + dot(c1, c1) + dot(c2, c2);
    pos = det > R(0);
    if (pos)
        rq = f2 * pow_m23(det) * R(1.0 / 3.0);
    else
        q = sgn(det) * R(3) * pow_23(det) / f2;
}

// Fr_TET_INV applied on the right of [e03 e13 e23] (AbstractEvaluator.cpp:28-31)
template <class R>
__device__ __forceinline__ void tet_frame(V3<R> e03, V3<R> e13, V3<R> e23, V3<R>& c0, V3<R>& c1, V3<R>& c2)
{
    c0 = e03;
    c1 = e03 * R(-0.5773502691896257645091) + e13 * R(1.154700538379251529018);
    c2 = e03 * R(-0.4082482904638630163662) + e13 * R(-0.4082482904638630163662) + e23 * R(1.224744871391589049099);
}
// Fr_PRI_INV (AbstractEvaluator.cpp:32-35)
template <class R>
__device__ __forceinline__ void pri_frame(V3<R> a, V3<R> b, V3<R> e, V3<R>& c0, V3<R>& c1, V3<R>& c2)
{
    c0 = a;
    c1 = a * R(-0.5773502691896257645091) + b * R(1.154700538379251529018);
    c2 = e;
}

// Running combination of corner qualities (MeanRatioEvaluator.cpp:91-110,
// 140-166): the harmonic mean when every corner is valid, else the minimum
// corner quality -- which is then the minimum over the non-positive corners,
// so the valid corners never need their q, only their 1/q.
template <class R>
struct CornerAcc
{
    R rsum = R(0);
    R minbad = R(3.0e38);
    bool all = true;
    __device__ __forceinline__ void add(R rq, R q, bool pos)
    {
        if (pos) rsum += rq;
        else
        {
            all = false;
            minbad = q < minbad ? q : minbad;
        }
    }
    __device__ __forceinline__ EQ<R> result(int n) const
    {
        if (all) return EQ<R>{rsum / R(n), true};
        return EQ<R>{minbad, false};
    }
};

template <int VAR, class R>
__device__ __forceinline__ EQ<R> mr_tet(const Crew& c, const V3<R>* p)
{
    V3<R> c0, c1, c2;
    tet_frame(segment<VAR, R>(c, p[0], p[3]), segment<VAR, R>(c, p[1], p[3]), segment<VAR, R>(c, p[2], p[3]), c0, c1, c2);
    R rq = 0, q = 0;
    bool pos;
    mr_corner(c0, c1, c2, rq, q, pos);
    return EQ<R>{pos ? rq : q, pos};
}

template <int VAR, class R>
__device__ __forceinline__ EQ<R> mr_pri(const Crew& c, const V3<R>* p)
{
    V3<R> e03 = segment<VAR, R>(c, p[0], p[3]), e14 = segment<VAR, R>(c, p[1], p[4]), e25 = segment<VAR, R>(c, p[2], p[5]);
    V3<R> e01 = segment<VAR, R>(c, p[0], p[1]), e12 = segment<VAR, R>(c, p[1], p[2]), e20 = segment<VAR, R>(c, p[2], p[0]);
    V3<R> e34 = segment<VAR, R>(c, p[3], p[4]), e45 = segment<VAR, R>(c, p[4], p[5]), e53 = segment<VAR, R>(c, p[5], p[3]);
    CornerAcc<R> acc;
    V3<R> a, b, d;
    R rq = 0, q = 0;
    bool pos;
    pri_frame(-e01, e20, e03, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e12, e01, e14, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e20, e12, e25, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e34, e53, e03, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e45, e34, e14, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e53, e45, e25, a, b, d); mr_corner(a, b, d, rq, q, pos); acc.add(rq, q, pos);
    return acc.result(6);
}

template <int VAR, class R>
__device__ __forceinline__ EQ<R> mr_hex(const Crew& c, const V3<R>* p)
{
    V3<R> e01 = segment<VAR, R>(c, p[0], p[1]), e03 = segment<VAR, R>(c, p[0], p[3]), e04 = segment<VAR, R>(c, p[0], p[4]);
    V3<R> e12 = segment<VAR, R>(c, p[1], p[2]), e15 = segment<VAR, R>(c, p[1], p[5]), e23 = segment<VAR, R>(c, p[2], p[3]);
    V3<R> e26 = segment<VAR, R>(c, p[2], p[6]), e37 = segment<VAR, R>(c, p[3], p[7]), e45 = segment<VAR, R>(c, p[4], p[5]);
    V3<R> e47 = segment<VAR, R>(c, p[4], p[7]), e56 = segment<VAR, R>(c, p[5], p[6]), e67 = segment<VAR, R>(c, p[6], p[7]);
    CornerAcc<R> acc;
    R rq = 0, q = 0;
    bool pos;
    mr_corner(e01, e04, -e03, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e01, e12, e15, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e12, e26, -e23, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e03, e23, e37, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e04, e45, e47, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e15, -e56, e45, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e26, e56, e67, rq, q, pos); acc.add(rq, q, pos);
    mr_corner(e37, e67, -e47, rq, q, pos); acc.add(rq, q, pos);
    return acc.result(8);
}

// mr_hex for the FP32 metric-free evaluation stream: the same 8 corners,
// with each of the 12 edges' squared length computed once (a corner's
// |F|^2 is the sum of its three edges'), and the factors 1/3 of the corner
// measure and 1/8 of the harmonic combination applied once to the sum.
// Branch-free: every corner yields r = |F|^2 |det|^(-2/3) (3 / q for a
// valid corner); an inverted corner's quality is q = -3 / r, so the
// element's minimum over its inverted corners is -3 / (their smallest r),
// and a flat corner (det = 0, r = inf) gives q = -0.
__device__ __forceinline__ void mr_hex_corner_fast(V3<float> a, V3<float> b, V3<float> c, float f2, float sign,
                                                   float& rsum, float& minr, bool& bad)
{
    const float det = sign * det3(a, b, c);
    const float r = f2 * pow_m23(det);
    rsum += r;
    const bool inverted = !(det > 0.f);
    bad |= inverted;
    minr = inverted ? fminf(minr, r) : minr;
}

__device__ __forceinline__ EQ<float> mr_hex_fast(const V3<float>* p)
{
    const V3<float> e01 = p[1] - p[0], e03 = p[3] - p[0], e04 = p[4] - p[0], e12 = p[2] - p[1];
    const V3<float> e15 = p[5] - p[1], e23 = p[3] - p[2], e26 = p[6] - p[2], e37 = p[7] - p[3];
    const V3<float> e45 = p[5] - p[4], e47 = p[7] - p[4], e56 = p[6] - p[5], e67 = p[7] - p[6];
    const float l01 = dot(e01, e01), l03 = dot(e03, e03), l04 = dot(e04, e04), l12 = dot(e12, e12);
    const float l15 = dot(e15, e15), l23 = dot(e23, e23), l26 = dot(e26, e26), l37 = dot(e37, e37);
    const float l45 = dot(e45, e45), l47 = dot(e47, e47), l56 = dot(e56, e56), l67 = dot(e67, e67);
    float rsum = 0.f, minr = INFINITY;
    bool bad = false;
    mr_hex_corner_fast(e01, e04, e03, l01 + l04 + l03, -1.f, rsum, minr, bad);
    mr_hex_corner_fast(e01, e12, e15, l01 + l12 + l15, 1.f, rsum, minr, bad);
    mr_hex_corner_fast(e12, e26, e23, l12 + l26 + l23, -1.f, rsum, minr, bad);
    mr_hex_corner_fast(e03, e23, e37, l03 + l23 + l37, 1.f, rsum, minr, bad);
    mr_hex_corner_fast(e04, e45, e47, l04 + l45 + l47, 1.f, rsum, minr, bad);
    mr_hex_corner_fast(e15, e56, e45, l15 + l56 + l45, -1.f, rsum, minr, bad);
    mr_hex_corner_fast(e26, e56, e67, l26 + l56 + l67, 1.f, rsum, minr, bad);
    mr_hex_corner_fast(e37, e67, e47, l37 + l67 + l47, -1.f, rsum, minr, bad);
    if (!bad) return EQ<float>{rsum * (1.f / 24.f), true};
    return EQ<float>{-3.f * rcp_fast(minr), false};
}

// MetricConformityEvaluator::specifiedMetric: 5-point Keast rule
template <class R>
__device__ __forceinline__ Sym3<R> specified_metric(const Crew& c, V3<R> v0, V3<R> v1, V3<R> v2, V3<R> v3,
                                                    uint32_t hint)
{
    const R H = R(0.5), Q = R((1.0 - 0.5) / 3.0);
    Sym3<R> m0 = metric_at(c, (v0 + v1 + v2 + v3) * R(0.25), hint);
    Sym3<R> m1 = metric_at(c, v0 * H + v1 * Q + v2 * Q + v3 * Q, hint);
    Sym3<R> m2 = metric_at(c, v0 * Q + v1 * H + v2 * Q + v3 * Q, hint);
    Sym3<R> m3 = metric_at(c, v0 * Q + v1 * Q + v2 * H + v3 * Q, hint);
    Sym3<R> m4 = metric_at(c, v0 * Q + v1 * Q + v2 * Q + v3 * H, hint);
    const R a = R(-0.8), b = R(0.45);
    Sym3<R> r;
    r.xx = m0.xx * a + (m1.xx + m2.xx + m3.xx + m4.xx) * b;
    r.yy = m0.yy * a + (m1.yy + m2.yy + m3.yy + m4.yy) * b;
    r.zz = m0.zz * a + (m1.zz + m2.zz + m3.zz + m4.zz) * b;
    r.xy = m0.xy * a + (m1.xy + m2.xy + m3.xy + m4.xy) * b;
    r.xz = m0.xz * a + (m1.xz + m2.xz + m3.xz + m4.xz) * b;
    r.yz = m0.yz * a + (m1.yz + m2.yz + m3.yz + m4.yz) * b;
    return r;
}

template <class R>
__device__ __forceinline__ Sym3<R> sym_inverse(const Sym3<R>& m)
{
    R c00 = m.yy * m.zz - m.yz * m.yz;
    R c01 = m.xz * m.yz - m.xy * m.zz;
    R c02 = m.xy * m.yz - m.xz * m.yy;
    R det = m.xx * c00 + m.xy * c01 + m.xz * c02;
    R id = R(1) / det;
    Sym3<R> r;
    r.xx = c00 * id;
    r.xy = c01 * id;
    r.xz = c02 * id;
    r.yy = (m.xx * m.zz - m.xz * m.xz) * id;
    r.yz = (m.xy * m.xz - m.xx * m.yz) * id;
    r.zz = (m.xx * m.yy - m.xy * m.xy) * id;
    return r;
}

// MetricConformityEvaluator::metricConformity: with F the corner matrix,
// Mk^-1 = F F^T (no inversion) and Mk = F^-T F^-1 = G^T G with G = F^-1, so
// only F (not F F^T, whose condition number is squared) is inverted;
// tNc = Mk^-1 Ms + Ms^-1 Mk - 2I and q = sign(det F) / sqrt(1 + |tNc|_F).
// Returns 1/q for valid corners.
template <class R>
__device__ __forceinline__ void mc_corner(V3<R> c0, V3<R> c1, V3<R> c2, const Sym3<R>& Ms, R& rq, R& q, bool& pos)
{
    // F has columns c0, c1, c2: F[r][c] = c_c.r
    const R F[3][3] = {{c0.x, c1.x, c2.x}, {c0.y, c1.y, c2.y}, {c0.z, c1.z, c2.z}};
    const R det = det3(c0, c1, c2);
    // G = F^-1 = adj(F) / det
    const R id = R(1) / det;
    R G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
            const int r0 = (j + 1) % 3, r1 = (j + 2) % 3, k0 = (i + 1) % 3, k1 = (i + 2) % 3;
            G[i][j] = (F[r0][k0] * F[r1][k1] - F[r0][k1] * F[r1][k0]) * id;
        }
    // A = F F^T (= Mk^-1), Mk = G^T G
    Sym3<R> A, Mk;
    A.xx = c0.x * c0.x + c1.x * c1.x + c2.x * c2.x;
    A.yy = c0.y * c0.y + c1.y * c1.y + c2.y * c2.y;
    A.zz = c0.z * c0.z + c1.z * c1.z + c2.z * c2.z;
    A.xy = c0.x * c0.y + c1.x * c1.y + c2.x * c2.y;
    A.xz = c0.x * c0.z + c1.x * c1.z + c2.x * c2.z;
    A.yz = c0.y * c0.z + c1.y * c1.z + c2.y * c2.z;
    Mk.xx = G[0][0] * G[0][0] + G[1][0] * G[1][0] + G[2][0] * G[2][0];
    Mk.yy = G[0][1] * G[0][1] + G[1][1] * G[1][1] + G[2][1] * G[2][1];
    Mk.zz = G[0][2] * G[0][2] + G[1][2] * G[1][2] + G[2][2] * G[2][2];
    Mk.xy = G[0][0] * G[0][1] + G[1][0] * G[1][1] + G[2][0] * G[2][1];
    Mk.xz = G[0][0] * G[0][2] + G[1][0] * G[1][2] + G[2][0] * G[2][2];
    Mk.yz = G[0][1] * G[0][2] + G[1][1] * G[1][2] + G[2][1] * G[2][2];
    Sym3<R> Msi = sym_inverse(Ms);
    R t[9];
#define GM_SYM(m, i, j) ((i) == (j) ? ((i) == 0 ? m.xx : (i) == 1 ? m.yy : m.zz) \
    : (((i) + (j)) == 1 ? m.xy : ((i) + (j)) == 2 ? m.xz : m.yz))
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
            R pij = GM_SYM(A, i, 0) * GM_SYM(Ms, 0, j) + GM_SYM(A, i, 1) * GM_SYM(Ms, 1, j) + GM_SYM(A, i, 2) * GM_SYM(Ms, 2, j);
            R qij = GM_SYM(Msi, i, 0) * GM_SYM(Mk, 0, j) + GM_SYM(Msi, i, 1) * GM_SYM(Mk, 1, j) + GM_SYM(Msi, i, 2) * GM_SYM(Mk, 2, j);
            t[i * 3 + j] = pij + qij - (i == j ? R(2) : R(0));
        }
#undef GM_SYM
    R f2 = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) f2 += t[i] * t[i];
    if (isnan(f2))
    {
        pos = false;
        q = R(0);
        return;
    }
    R s = sgn(det);
    pos = s > R(0);
    R r = sqrt_<R>(R(1) + sqrt_<R>(f2));
    if (pos) rq = r;
    else q = s / r;
}

// ---- diagonal metrics (uniform, sine-graded): M = diag(d.x, d.y, d.z) ----
template <class R>
__device__ __forceinline__ V3<R> metric_diag_at(const Crew& c, V3<R> p)
{
    R s2 = (R)c.scaling2;
    if (c.sampler == kSamplerSine)
    {
        R s = sinpi_(R(4) * p.x);
        return {s2 * (R(1) + R(9) * s * s), s2, s2};
    }
    return {s2, s2, s2};
}

template <class R>
__device__ __forceinline__ V3<R> specified_metric_diag(const Crew& c, V3<R> v0, V3<R> v1, V3<R> v2, V3<R> v3)
{
    const R H = R(0.5), Q = R((1.0 - 0.5) / 3.0);
    V3<R> m0 = metric_diag_at(c, (v0 + v1 + v2 + v3) * R(0.25));
    V3<R> m1 = metric_diag_at(c, v0 * H + v1 * Q + v2 * Q + v3 * Q);
    V3<R> m2 = metric_diag_at(c, v0 * Q + v1 * H + v2 * Q + v3 * Q);
    V3<R> m3 = metric_diag_at(c, v0 * Q + v1 * Q + v2 * H + v3 * Q);
    V3<R> m4 = metric_diag_at(c, v0 * Q + v1 * Q + v2 * Q + v3 * H);
    return m0 * R(-0.8) + (m1 + m2 + m3 + m4) * R(0.45);
}

// mc_corner with Ms = diag(m): tNc_ij = A_ij m_j + Mk_ij / m_i - 2 delta_ij
template <class R>
__device__ __forceinline__ void mc_corner_diag(V3<R> c0, V3<R> c1, V3<R> c2, V3<R> m, R& rq, R& q, bool& pos)
{
    const R F[3][3] = {{c0.x, c1.x, c2.x}, {c0.y, c1.y, c2.y}, {c0.z, c1.z, c2.z}};
    const R det = det3(c0, c1, c2);
    const R id = R(1) / det;
    R G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
            const int r0 = (j + 1) % 3, r1 = (j + 2) % 3, k0 = (i + 1) % 3, k1 = (i + 2) % 3;
            G[i][j] = (F[r0][k0] * F[r1][k1] - F[r0][k1] * F[r1][k0]) * id;
        }
    const R Axx = c0.x * c0.x + c1.x * c1.x + c2.x * c2.x, Ayy = c0.y * c0.y + c1.y * c1.y + c2.y * c2.y;
    const R Azz = c0.z * c0.z + c1.z * c1.z + c2.z * c2.z, Axy = c0.x * c0.y + c1.x * c1.y + c2.x * c2.y;
    const R Axz = c0.x * c0.z + c1.x * c1.z + c2.x * c2.z, Ayz = c0.y * c0.z + c1.y * c1.z + c2.y * c2.z;
    const R Kxx = G[0][0] * G[0][0] + G[1][0] * G[1][0] + G[2][0] * G[2][0];
    const R Kyy = G[0][1] * G[0][1] + G[1][1] * G[1][1] + G[2][1] * G[2][1];
    const R Kzz = G[0][2] * G[0][2] + G[1][2] * G[1][2] + G[2][2] * G[2][2];
    const R Kxy = G[0][0] * G[0][1] + G[1][0] * G[1][1] + G[2][0] * G[2][1];
    const R Kxz = G[0][0] * G[0][2] + G[1][0] * G[1][2] + G[2][0] * G[2][2];
    const R Kyz = G[0][1] * G[0][2] + G[1][1] * G[1][2] + G[2][1] * G[2][2];
    const R ix = R(1) / m.x, iy = R(1) / m.y, iz = R(1) / m.z;
    const R txx = Axx * m.x + Kxx * ix - R(2), tyy = Ayy * m.y + Kyy * iy - R(2), tzz = Azz * m.z + Kzz * iz - R(2);
    const R txy = Axy * m.y + Kxy * ix, tyx = Axy * m.x + Kxy * iy;
    const R txz = Axz * m.z + Kxz * ix, tzx = Axz * m.x + Kxz * iz;
    const R tyz = Ayz * m.z + Kyz * iy, tzy = Ayz * m.y + Kyz * iz;
    const R f2 = txx * txx + tyy * tyy + tzz * tzz + txy * txy + tyx * tyx + txz * txz + tzx * tzx + tyz * tyz +
                 tzy * tzy;
    if (isnan(f2))
    {
        pos = false;
        q = R(0);
        return;
    }
    R sg = sgn(det);
    pos = sg > R(0);
    R r = sqrt_<R>(R(1) + sqrt_<R>(f2));
    if (pos) rq = r;
    else q = sg / r;
}

template <class R>
__device__ __forceinline__ EQ<R> mc_tet_diag(const Crew& c, const V3<R>* p)
{
    V3<R> c0, c1, c2;
    tet_frame(p[3] - p[0], p[3] - p[1], p[3] - p[2], c0, c1, c2);
    R rq = 0, q = 0;
    bool pos;
    mc_corner_diag(c0, c1, c2, specified_metric_diag(c, p[0], p[1], p[2], p[3]), rq, q, pos);
    return EQ<R>{pos ? rq : q, pos};
}

template <class R>
__device__ __noinline__ EQ<R> mc_pri_diag(const Crew& c, const V3<R>* p)
{
    V3<R> e03 = p[3] - p[0], e14 = p[4] - p[1], e25 = p[5] - p[2];
    V3<R> e01 = p[1] - p[0], e12 = p[2] - p[1], e20 = p[0] - p[2];
    V3<R> e34 = p[4] - p[3], e45 = p[5] - p[4], e53 = p[3] - p[5];
    CornerAcc<R> acc;
    V3<R> a, b, d;
    R rq = 0, q = 0;
    bool pos;
    pri_frame(-e01, e20, e03, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[0], p[1], p[2], p[3]), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e12, e01, e14, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[0], p[1], p[2], p[4]), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e20, e12, e25, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[0], p[1], p[2], p[5]), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e34, e53, e03, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[0], p[3], p[4], p[5]), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e45, e34, e14, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[1], p[3], p[4], p[5]), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e53, e45, e25, a, b, d); mc_corner_diag(a, b, d, specified_metric_diag(c, p[2], p[3], p[4], p[5]), rq, q, pos); acc.add(rq, q, pos);
    return acc.result(6);
}

template <class R>
__device__ __noinline__ EQ<R> mc_hex_diag(const Crew& c, const V3<R>* p)
{
    V3<R> e01 = p[1] - p[0], e03 = p[3] - p[0], e04 = p[4] - p[0], e12 = p[2] - p[1];
    V3<R> e15 = p[5] - p[1], e23 = p[3] - p[2], e26 = p[6] - p[2], e37 = p[7] - p[3];
    V3<R> e45 = p[5] - p[4], e47 = p[7] - p[4], e56 = p[6] - p[5], e67 = p[7] - p[6];
    CornerAcc<R> acc;
    R rq = 0, q = 0;
    bool pos;
    mc_corner_diag(e01, e04, -e03, specified_metric_diag(c, p[0], p[1], p[3], p[4]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e01, e12, e15, specified_metric_diag(c, p[0], p[1], p[2], p[5]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e12, e26, -e23, specified_metric_diag(c, p[1], p[2], p[3], p[6]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e03, e23, e37, specified_metric_diag(c, p[0], p[2], p[3], p[7]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e04, e45, e47, specified_metric_diag(c, p[0], p[4], p[5], p[7]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e15, -e56, e45, specified_metric_diag(c, p[1], p[4], p[5], p[6]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e26, e56, e67, specified_metric_diag(c, p[2], p[5], p[6], p[7]), rq, q, pos); acc.add(rq, q, pos);
    mc_corner_diag(e37, e67, -e47, specified_metric_diag(c, p[3], p[4], p[6], p[7]), rq, q, pos); acc.add(rq, q, pos);
    return acc.result(8);
}

template <class R>
__device__ __forceinline__ EQ<R> mc_tet(const Crew& c, const V3<R>* p, uint32_t hint)
{
    V3<R> c0, c1, c2;
    tet_frame(p[3] - p[0], p[3] - p[1], p[3] - p[2], c0, c1, c2);
    Sym3<R> Ms = specified_metric(c, p[0], p[1], p[2], p[3], hint);
    R rq = 0, q = 0;
    bool pos;
    mc_corner(c0, c1, c2, Ms, rq, q, pos);
    return EQ<R>{pos ? rq : q, pos};
}

template <class R>
__device__ __noinline__ EQ<R> mc_pri(const Crew& c, const V3<R>* p, uint32_t hint)
{
    V3<R> e03 = p[3] - p[0], e14 = p[4] - p[1], e25 = p[5] - p[2];
    V3<R> e01 = p[1] - p[0], e12 = p[2] - p[1], e20 = p[0] - p[2];
    V3<R> e34 = p[4] - p[3], e45 = p[5] - p[4], e53 = p[3] - p[5];
    CornerAcc<R> acc;
    V3<R> a, b, d;
    R rq = 0, q = 0;
    bool pos;
    pri_frame(-e01, e20, e03, a, b, d); mc_corner(a, b, d, specified_metric(c, p[0], p[1], p[2], p[3], hint), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e12, e01, e14, a, b, d); mc_corner(a, b, d, specified_metric(c, p[0], p[1], p[2], p[4], hint), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e20, e12, e25, a, b, d); mc_corner(a, b, d, specified_metric(c, p[0], p[1], p[2], p[5], hint), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e34, e53, e03, a, b, d); mc_corner(a, b, d, specified_metric(c, p[0], p[3], p[4], p[5], hint), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e45, e34, e14, a, b, d); mc_corner(a, b, d, specified_metric(c, p[1], p[3], p[4], p[5], hint), rq, q, pos); acc.add(rq, q, pos);
    pri_frame(-e53, e45, e25, a, b, d); mc_corner(a, b, d, specified_metric(c, p[2], p[3], p[4], p[5], hint), rq, q, pos); acc.add(rq, q, pos);
    return acc.result(6);
}

template <class R>
__device__ __noinline__ EQ<R> mc_hex(const Crew& c, const V3<R>* p, uint32_t hint)
{
    V3<R> e01 = p[1] - p[0], e03 = p[3] - p[0], e04 = p[4] - p[0], e12 = p[2] - p[1];
    V3<R> e15 = p[5] - p[1], e23 = p[3] - p[2], e26 = p[6] - p[2], e37 = p[7] - p[3];
    V3<R> e45 = p[5] - p[4], e47 = p[7] - p[4], e56 = p[6] - p[5], e67 = p[7] - p[6];
    CornerAcc<R> acc;
    R rq = 0, q = 0;
    bool pos;
    mc_corner(e01, e04, -e03, specified_metric(c, p[0], p[1], p[3], p[4], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e01, e12, e15, specified_metric(c, p[0], p[1], p[2], p[5], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e12, e26, -e23, specified_metric(c, p[1], p[2], p[3], p[6], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e03, e23, e37, specified_metric(c, p[0], p[2], p[3], p[7], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e04, e45, e47, specified_metric(c, p[0], p[4], p[5], p[7], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e15, -e56, e45, specified_metric(c, p[1], p[4], p[5], p[6], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e26, e56, e67, specified_metric(c, p[2], p[5], p[6], p[7], hint), rq, q, pos); acc.add(rq, q, pos);
    mc_corner(e37, e67, -e47, specified_metric(c, p[3], p[4], p[6], p[7], hint), rq, q, pos); acc.add(rq, q, pos);
    return acc.result(8);
}

// quality of an element of the given type; MAXK = 4 means tets only
// hint: the element (elem_hint) when known, for the local sampler's walk
template <int VAR, int MAXK, class R>
__device__ __forceinline__ EQ<R> elem_quality(const Crew& c, int type, const V3<R>* p, uint32_t hint = kNoHint)
{
    if (VarTraits<VAR>::diag_metric)
    {
        if (MAXK == 4 || type == kTet) return mc_tet_diag(c, p);
        if (type == kPri) return mc_pri_diag(c, p);
        return mc_hex_diag(c, p);
    }
    if (!VarTraits<VAR>::mean_ratio)
    {
        if (MAXK == 4 || type == kTet) return mc_tet(c, p, hint);
        if (type == kPri) return mc_pri(c, p, hint);
        return mc_hex(c, p, hint);
    }
    if (MAXK == 4 || type == kTet) return mr_tet<VAR, R>(c, p);
    if (type == kPri) return mr_pri<VAR, R>(c, p);
    return mr_hex<VAR, R>(c, p);
}

__device__ __forceinline__ int type_size(int type) { return type == kTet ? 4 : type == kPri ? 6 : 8; }

// vertex ids of element (type, id)
__device__ __forceinline__ void elem_vertices(const MeshView& m, int type, uint32_t id, uint32_t* v)
{
    if (type == kTet)
    {
        uint4 t = m.tets[GM_IX(m, id, m.nt, kBoundsTet)];
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    else if (type == kPri)
    {
        const uint2* p = reinterpret_cast<const uint2*>(m.pris + 6 * (size_t)GM_IX(m, id, m.np, kBoundsPrism));
        uint2 a = p[0], b = p[1], c = p[2];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
    }
    else
    {
        const size_t h = 2 * (size_t)GM_IX(m, id, m.nh, kBoundsHex);
        uint4 a = m.hexs[h], b = m.hexs[h + 1];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
#ifdef GM_BOUNDS_CHECK
    const int n = type == kTet ? 4 : type == kPri ? 6 : 8;
    for (int k = 0; k < n; ++k) v[k] = GM_IX(m, v[k], m.nv, kBoundsPosition);
#endif
}

// ---------------------------------------------------------------------------
// boundary projection by constraint id (-1 fixed: never moved; 0 free)
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ V3<R> project(const Constraint* con, int ncon, int id, V3<R> p)
{
    if (id <= 0 || id >= ncon) return p;
    const Constraint& k = con[id];
    const bool dbl = sizeof(R) == 8;
    switch (k.kind)
    {
    case kConPlane:
    {
        V3<R> a = dbl ? mk<R>((R)k.ad[0], (R)k.ad[1], (R)k.ad[2]) : mk<R>((R)k.a[0], (R)k.a[1], (R)k.a[2]);
        V3<R> n = dbl ? mk<R>((R)k.bd[0], (R)k.bd[1], (R)k.bd[2]) : mk<R>((R)k.b[0], (R)k.b[1], (R)k.b[2]);
        R l = dot(p - a, n);
        return p - n * l;
    }
    case kConSegment:
    {
        V3<R> a = dbl ? mk<R>((R)k.ad[0], (R)k.ad[1], (R)k.ad[2]) : mk<R>((R)k.a[0], (R)k.a[1], (R)k.a[2]);
        V3<R> u = dbl ? mk<R>((R)k.ud[0], (R)k.ud[1], (R)k.ud[2]) : mk<R>((R)k.u[0], (R)k.u[1], (R)k.u[2]);
        R len = dbl ? (R)k.lend : (R)k.len;
        V3<R> dist = p - a;
        R l = dot(dist, u);
        if (l < R(0)) return a;
        if (l > len) return dbl ? mk<R>((R)k.bd[0], (R)k.bd[1], (R)k.bd[2]) : mk<R>((R)k.b[0], (R)k.b[1], (R)k.b[2]);
        return p - (dist - u * l);
    }
    case kConSphere:
        return normalize(p);
    case kConPoint:
        return dbl ? mk<R>((R)k.ad[0], (R)k.ad[1], (R)k.ad[2]) : mk<R>((R)k.a[0], (R)k.a[1], (R)k.a[2]);
    case kConShellInner:
        return normalize(p) * R(0.5);
    case kConPipeCylinder:
        return pipe_cylinder(p);
    case kConPipeCircle:
        return pipe_circle(dbl ? mk<R>((R)k.ad[0], (R)k.ad[1], (R)k.ad[2]) : mk<R>((R)k.a[0], (R)k.a[1], (R)k.a[2]), p);
    default:
        return p;
    }
}

}  // namespace gm
