/*
 * gm_oracle.c -- FP64 CPU restatement of GpuMesh's node-relocation smoothers
 * and element-quality evaluators.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load
 * it.  The product never calls it.
 *
 * Parity is pinned two ways: against the reference's regular-element
 * known-answer test (Evaluators/AbstractEvaluator.cpp:281-338), and against
 * the reference's own C++ compiled from its sources by oracle/Makefile into
 * oracle/_ref (tests/test_oracle_vs_reference.py, tests/golden/).
 *
 * Conventions follow GLM as used by the reference: dmat3 is column-major,
 * mat*vec / mat*mat sum columns left to right, normalize(v) = v*(1/sqrt(v.v)),
 * sign() returns -1/0/+1.  Build with -ffp-contract=off.
 */
#include "gm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* small GLM-like vector / matrix algebra                                    */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z; } v3;
typedef struct { v3 c[3]; } m3; /* column-major, like glm::dmat3 */

static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 neg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 mul(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 dvs(v3 a, double s) { return V(a.x / s, a.y / s, a.z / s); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double length(v3 a) { return sqrt(dot(a, a)); }
static inline v3 normalize(v3 a) { return mul(a, 1.0 / sqrt(dot(a, a))); }
static inline v3 cross(v3 a, v3 b)
{
    return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline double gsign(double x) { return (double)((0.0 < x) - (x < 0.0)); }
static inline double gmin(double a, double b) { return (b < a) ? b : a; }

static inline m3 M(v3 c0, v3 c1, v3 c2) { m3 r; r.c[0] = c0; r.c[1] = c1; r.c[2] = c2; return r; }
static inline m3 mdiag(double a, double b, double c)
{
    return M(V(a, 0, 0), V(0, b, 0), V(0, 0, c));
}
static inline double el(const m3* m, int c, int r)
{
    const double* p = &m->c[c].x;
    return p[r];
}
static inline v3 mmulv(m3 m, v3 v)
{
    return V(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z,
             m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
             m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
static inline m3 mmul(m3 a, m3 b)
{
    return M(mmulv(a, b.c[0]), mmulv(a, b.c[1]), mmulv(a, b.c[2]));
}
static inline m3 madd(m3 a, m3 b) { return M(add(a.c[0], b.c[0]), add(a.c[1], b.c[1]), add(a.c[2], b.c[2])); }
static inline m3 msub(m3 a, m3 b) { return M(sub(a.c[0], b.c[0]), sub(a.c[1], b.c[1]), sub(a.c[2], b.c[2])); }
static inline m3 mscale(m3 a, double s) { return M(mul(a.c[0], s), mul(a.c[1], s), mul(a.c[2], s)); }
static inline m3 mtranspose(m3 m)
{
    return M(V(m.c[0].x, m.c[1].x, m.c[2].x), V(m.c[0].y, m.c[1].y, m.c[2].y),
             V(m.c[0].z, m.c[1].z, m.c[2].z));
}
static inline double mdet(m3 m)
{
#define E(c, r) el(&m, c, r)
    return +E(0, 0) * (E(1, 1) * E(2, 2) - E(2, 1) * E(1, 2))
           - E(1, 0) * (E(0, 1) * E(2, 2) - E(2, 1) * E(0, 2))
           + E(2, 0) * (E(0, 1) * E(1, 2) - E(1, 1) * E(0, 2));
}
static inline m3 minverse(m3 m)
{
    double ood = 1.0 / (+E(0, 0) * (E(1, 1) * E(2, 2) - E(2, 1) * E(1, 2))
                        - E(1, 0) * (E(0, 1) * E(2, 2) - E(2, 1) * E(0, 2))
                        + E(2, 0) * (E(0, 1) * E(1, 2) - E(1, 1) * E(0, 2)));
    m3 r;
    r.c[0].x = +(E(1, 1) * E(2, 2) - E(2, 1) * E(1, 2)) * ood;
    r.c[1].x = -(E(1, 0) * E(2, 2) - E(2, 0) * E(1, 2)) * ood;
    r.c[2].x = +(E(1, 0) * E(2, 1) - E(2, 0) * E(1, 1)) * ood;
    r.c[0].y = -(E(0, 1) * E(2, 2) - E(2, 1) * E(0, 2)) * ood;
    r.c[1].y = +(E(0, 0) * E(2, 2) - E(2, 0) * E(0, 2)) * ood;
    r.c[2].y = -(E(0, 0) * E(2, 1) - E(2, 0) * E(0, 1)) * ood;
    r.c[0].z = +(E(0, 1) * E(1, 2) - E(1, 1) * E(0, 2)) * ood;
    r.c[1].z = -(E(0, 0) * E(1, 2) - E(1, 0) * E(0, 2)) * ood;
    r.c[2].z = +(E(0, 0) * E(1, 1) - E(1, 0) * E(0, 1)) * ood;
#undef E
    return r;
}

/* Rodrigues rotation applied on the right of m, the algebra of
 * glm::rotate(dmat4, angle, axis) restricted to the 3x3 block. */
static m3 mrotate(m3 m, double angle, v3 axis_in)
{
    double c = cos(angle), s = sin(angle);
    v3 axis = normalize(axis_in);
    v3 temp = mul(axis, 1.0 - c);
    m3 R;
    R.c[0].x = c + temp.x * axis.x;
    R.c[0].y = temp.x * axis.y + s * axis.z;
    R.c[0].z = temp.x * axis.z - s * axis.y;
    R.c[1].x = temp.y * axis.x - s * axis.z;
    R.c[1].y = c + temp.y * axis.y;
    R.c[1].z = temp.y * axis.z + s * axis.x;
    R.c[2].x = temp.z * axis.x + s * axis.y;
    R.c[2].y = temp.z * axis.y - s * axis.x;
    R.c[2].z = c + temp.z * axis.z;
    m3 out;
    for (int j = 0; j < 3; ++j)
    {
        const double* rj = &R.c[j].x;
        out.c[j] = add(add(mul(m.c[0], rj[0]), mul(m.c[1], rj[1])), mul(m.c[2], rj[2]));
    }
    return out;
}

/* ------------------------------------------------------------------------ */
/* mesh                                                                      */
/* ------------------------------------------------------------------------ */

typedef struct
{
    uint32_t id;
    int32_t type;
    int32_t vid;
} neig_elem;

struct om_mesh
{
    int64_t nv, nt, np, nh;
    double* pos; /* nv*3 */
    uint32_t* tets;
    uint32_t* pris;
    uint32_t* hexs;
    int32_t* cid;

    /* vertex -> element, in the order Mesh::compileNeighborhoods builds
     * topos[v].neighborElems (DataStructures/Mesh.cpp:365-445) */
    int64_t* ne_base;
    neig_elem* ne;
    /* vertex -> vertex, in MeshTopo::neighborVerts order (Mesh::addEdge,
     * DataStructures/Mesh.cpp:447-460) */
    int64_t* nvx_base;
    uint32_t* nvx;

    int32_t ncon;
    int32_t* con_kind;
    double* con_param; /* 6 per id */
    /* derived segment data: u, length (EdgeConstraint.cpp:176-181) */
    double* con_derived; /* 4 per id */

    int32_t sampler, measurer, evaluator;
    double scaling, scaling2, scaling3, aspect_ratio;
    m3 rot, rotinv;

    /* LocalSampler's background mesh (Samplers/LocalSampler.cpp:352-429):
     * the mesh at crew set-up split into tets, their face neighbours, the
     * analytic metric at every vertex, and the sampler caches -- per vertex
     * the last background tet holding it, per element its first background
     * tet (Tetrahedralizer.h:39-200) */
    int64_t nbg;
    uint32_t* bg; /* 8 per background tet: v[4], n[4] (0xffffffff: no neighbour) */
    double* bg_pos;
    m3* bg_metric;
    uint32_t* vcache;
    uint32_t* ecache; /* tets, then prisms, then hexes */

    /* KdTreeSampler (Samplers/KdTreeSampler.cpp): nodes in the pre-order of
     * buildGpuBuffers (:374-397); TextureSampler (TextureSampler.cpp): the
     * metric grid of buildGrid (:275-448) */
    int32_t depth;
    int64_t nkd, kd_cap;
    struct om_kd* kd;
    int tex_size[3];
    double tex_min[3], tex_ext[3];
    m3* tex;

    int64_t patch_evals;
};

static const m3* fr_tet_inv(void)
{
    /* AbstractEvaluator.cpp:28-31 */
    static m3 m;
    static int init = 0;
    if (!init)
    {
        m = M(V(1, 0, 0), V(-0.5773502691896257645091, 1.154700538379251529018, 0),
              V(-0.4082482904638630163662, -0.4082482904638630163662, 1.224744871391589049099));
        init = 1;
    }
    return &m;
}
static const m3* fr_pri_inv(void)
{
    /* AbstractEvaluator.cpp:32-35 */
    static m3 m;
    static int init = 0;
    if (!init)
    {
        m = M(V(1.0, 0.0, 0.0), V(-0.5773502691896257645091, 1.154700538379251529018, 0.0),
              V(0.0, 0.0, 1.0));
        init = 1;
    }
    return &m;
}

static inline v3 P(const om_mesh* m, uint32_t v)
{
    const double* p = m->pos + 3 * (int64_t)v;
    return V(p[0], p[1], p[2]);
}
static inline void setP(om_mesh* m, uint32_t v, v3 p)
{
    double* q = m->pos + 3 * (int64_t)v;
    q[0] = p.x;
    q[1] = p.y;
    q[2] = p.z;
}

/* Mesh::addEdge (Mesh.cpp:447-460): linear scan of the first vertex's list */
typedef struct
{
    uint32_t* items;
    int32_t n, cap;
} ulist;
static void ulist_push(ulist* l, uint32_t v)
{
    if (l->n == l->cap)
    {
        l->cap = l->cap ? l->cap * 2 : 16;
        l->items = (uint32_t*)realloc(l->items, sizeof(uint32_t) * l->cap);
    }
    l->items[l->n++] = v;
}
static void add_edge(ulist* lists, uint32_t a, uint32_t b)
{
    ulist* l = &lists[a];
    for (int32_t i = 0; i < l->n; ++i)
        if (l->items[i] == b)
            return;
    ulist_push(&lists[a], b);
    ulist_push(&lists[b], a);
}

static const int TET_EDGES[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
static const int PRI_EDGES[9][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 4},
                                    {2, 5}, {3, 4}, {3, 5}, {4, 5}};
static const int HEX_EDGES[12][2] = {{0, 1}, {0, 3}, {1, 2}, {2, 3}, {0, 4}, {1, 5},
                                     {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};

static void build_topology(om_mesh* m)
{
    int64_t nv = m->nv;
    /* neighbour elements: counts then fill, tets -> pris -> hexs */
    m->ne_base = (int64_t*)calloc((size_t)nv + 1, sizeof(int64_t));
    for (int64_t i = 0; i < m->nt * 4; ++i) m->ne_base[m->tets[i] + 1]++;
    for (int64_t i = 0; i < m->np * 6; ++i) m->ne_base[m->pris[i] + 1]++;
    for (int64_t i = 0; i < m->nh * 8; ++i) m->ne_base[m->hexs[i] + 1]++;
    for (int64_t v = 0; v < nv; ++v) m->ne_base[v + 1] += m->ne_base[v];
    m->ne = (neig_elem*)malloc(sizeof(neig_elem) * (size_t)(m->ne_base[nv] + 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1));
    memcpy(fill, m->ne_base, sizeof(int64_t) * (size_t)nv);

    ulist* lists = (ulist*)calloc((size_t)nv, sizeof(ulist));
    for (int64_t i = 0; i < m->nt; ++i)
    {
        const uint32_t* e = m->tets + 4 * i;
        for (int k = 0; k < 4; ++k)
        {
            neig_elem n = {(uint32_t)i, OM_TET, k};
            m->ne[fill[e[k]]++] = n;
        }
        for (int k = 0; k < 6; ++k) add_edge(lists, e[TET_EDGES[k][0]], e[TET_EDGES[k][1]]);
    }
    for (int64_t i = 0; i < m->np; ++i)
    {
        const uint32_t* e = m->pris + 6 * i;
        for (int k = 0; k < 6; ++k)
        {
            neig_elem n = {(uint32_t)i, OM_PRI, k};
            m->ne[fill[e[k]]++] = n;
        }
        for (int k = 0; k < 9; ++k) add_edge(lists, e[PRI_EDGES[k][0]], e[PRI_EDGES[k][1]]);
    }
    for (int64_t i = 0; i < m->nh; ++i)
    {
        const uint32_t* e = m->hexs + 8 * i;
        for (int k = 0; k < 8; ++k)
        {
            neig_elem n = {(uint32_t)i, OM_HEX, k};
            m->ne[fill[e[k]]++] = n;
        }
        for (int k = 0; k < 12; ++k) add_edge(lists, e[HEX_EDGES[k][0]], e[HEX_EDGES[k][1]]);
    }
    free(fill);

    m->nvx_base = (int64_t*)calloc((size_t)nv + 1, sizeof(int64_t));
    for (int64_t v = 0; v < nv; ++v) m->nvx_base[v + 1] = m->nvx_base[v] + lists[v].n;
    m->nvx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(m->nvx_base[nv] + 1));
    for (int64_t v = 0; v < nv; ++v)
    {
        if (lists[v].n)
            memcpy(m->nvx + m->nvx_base[v], lists[v].items, sizeof(uint32_t) * lists[v].n);
        free(lists[v].items);
    }
    free(lists);
}

om_mesh* om_create(int64_t nv, const double* pos, int64_t nt, const uint32_t* tets,
                   int64_t np, const uint32_t* pris, int64_t nh, const uint32_t* hexs,
                   const int32_t* cid)
{
    om_mesh* m = (om_mesh*)calloc(1, sizeof(om_mesh));
    m->nv = nv;
    m->nt = nt;
    m->np = np;
    m->nh = nh;
    m->pos = (double*)malloc(sizeof(double) * (size_t)(3 * nv + 1));
    memcpy(m->pos, pos, sizeof(double) * (size_t)(3 * nv));
    m->tets = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(4 * nt + 1));
    if (nt) memcpy(m->tets, tets, sizeof(uint32_t) * (size_t)(4 * nt));
    m->pris = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(6 * np + 1));
    if (np) memcpy(m->pris, pris, sizeof(uint32_t) * (size_t)(6 * np));
    m->hexs = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(8 * nh + 1));
    if (nh) memcpy(m->hexs, hexs, sizeof(uint32_t) * (size_t)(8 * nh));
    m->cid = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nv + 1));
    memcpy(m->cid, cid, sizeof(int32_t) * (size_t)nv);
    build_topology(m);
    m->depth = -1;
    om_set_crew(m, OM_SAMPLER_UNIFORM, OM_MEASURER_METRIC_FREE, OM_EVALUATOR_MEAN_RATIO, 1.0, 1.0);
    return m;
}

void om_destroy(om_mesh* m)
{
    if (!m) return;
    free(m->bg);
    free(m->bg_pos);
    free(m->bg_metric);
    free(m->vcache);
    free(m->ecache);
    free(m->kd);
    free(m->tex);
    free(m->pos);
    free(m->tets);
    free(m->pris);
    free(m->hexs);
    free(m->cid);
    free(m->ne_base);
    free(m->ne);
    free(m->nvx_base);
    free(m->nvx);
    free(m->con_kind);
    free(m->con_param);
    free(m->con_derived);
    free(m);
}

void om_set_constraints(om_mesh* m, int32_t n, const int32_t* kind, const double* params)
{
    free(m->con_kind);
    free(m->con_param);
    free(m->con_derived);
    m->ncon = n;
    m->con_kind = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    m->con_param = (double*)malloc(sizeof(double) * 6 * (size_t)(n + 1));
    m->con_derived = (double*)calloc(4 * (size_t)(n + 1), sizeof(double));
    memcpy(m->con_kind, kind, sizeof(int32_t) * (size_t)n);
    memcpy(m->con_param, params, sizeof(double) * 6 * (size_t)n);
    for (int32_t i = 0; i < n; ++i)
    {
        double* pp = m->con_param + 6 * i;
        double* d = m->con_derived + 4 * i;
        if (kind[i] == OM_CON_PLANE)
        {
            /* PlaneConstraint ctor normalizes n (FaceConstraint.cpp:172-176) */
            v3 nn = normalize(V(pp[3], pp[4], pp[5]));
            d[0] = nn.x;
            d[1] = nn.y;
            d[2] = nn.z;
        }
        else if (kind[i] == OM_CON_SEGMENT)
        {
            /* SegmentConstraint ctor (EdgeConstraint.cpp:176-181) */
            v3 a = V(pp[0], pp[1], pp[2]), b = V(pp[3], pp[4], pp[5]);
            v3 u = normalize(sub(b, a));
            d[0] = u.x;
            d[1] = u.y;
            d[2] = u.z;
            d[3] = length(sub(b, a));
        }
    }
}

/* ---- LocalSampler background mesh ---- */

#define BG_NONE 0xffffffffu

/* MeshTet::tris (DataStructures/Mesh.cpp:30-35): the face opposite each vertex */
static const int TET_TRIS[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};

static m3 analytic_metric(const om_mesh* m, v3 p);

/* the vertex rotations of tetrahedrize (DataStructures/Tetrahedralizer.h:9-34):
 * each prism / hex is turned so that its smallest vertex id comes first */
static const unsigned PRI_ROT[6][6] = {{0, 1, 2, 3, 4, 5}, {1, 2, 0, 4, 5, 3}, {2, 0, 1, 5, 3, 4},
                                       {3, 5, 4, 0, 2, 1}, {4, 3, 5, 1, 0, 2}, {5, 4, 3, 2, 1, 0}};
static const unsigned HEX_ROT[8][8] = {{0, 1, 2, 3, 4, 5, 6, 7}, {1, 0, 4, 5, 2, 3, 7, 6}, {2, 1, 5, 6, 3, 0, 4, 7},
                                       {3, 0, 1, 2, 7, 4, 5, 6}, {4, 0, 3, 7, 5, 1, 2, 6}, {5, 1, 0, 4, 6, 2, 3, 7},
                                       {6, 2, 1, 5, 7, 3, 0, 4}, {7, 3, 2, 6, 4, 0, 1, 5}};
static const unsigned HEX_LOOP[8] = {0, 120, 240, 0, 0, 240, 120, 0};

static inline unsigned umin(unsigned a, unsigned b) { return b < a ? b : a; }

static void bg_push(om_mesh* m, unsigned a, unsigned b, unsigned c, unsigned d)
{
    uint32_t* t = m->bg + 8 * (size_t)m->nbg++;
    t[0] = a;
    t[1] = b;
    t[2] = c;
    t[3] = d;
    t[4] = t[5] = t[6] = t[7] = BG_NONE;
}

/* tetrahedrize (Tetrahedralizer.h:37-200): tets as they are; a prism into 3
 * tets and a hex into 5 or 6, the diagonals chosen from the vertex ids so that
 * neighbouring elements split their shared faces alike; every element's cache
 * is its first background tet */
static void tetrahedrize(om_mesh* m)
{
    m->nbg = 0;
    for (int64_t i = 0; i < m->nt; ++i)
    {
        const uint32_t* e = m->tets + 4 * i;
        m->ecache[i] = (uint32_t)m->nbg;
        bg_push(m, e[0], e[1], e[2], e[3]);
    }
    for (int64_t i = 0; i < m->np; ++i)
    {
        const uint32_t* pv = m->pris + 6 * i;
        m->ecache[m->nt + i] = (uint32_t)m->nbg;
        unsigned s = 0;
        for (unsigned k = 1; k < 6; ++k)
            if (pv[k] < pv[s]) s = k;
        unsigned v[6];
        for (int k = 0; k < 6; ++k) v[k] = pv[PRI_ROT[s][k]];
        if (umin(v[1], v[5]) < umin(v[2], v[4]))
        {
            bg_push(m, v[0], v[1], v[2], v[5]);
            bg_push(m, v[0], v[1], v[5], v[4]);
            bg_push(m, v[0], v[4], v[5], v[3]);
        }
        else
        {
            bg_push(m, v[0], v[1], v[2], v[4]);
            bg_push(m, v[0], v[4], v[2], v[5]);
            bg_push(m, v[0], v[4], v[5], v[3]);
        }
    }
    for (int64_t i = 0; i < m->nh; ++i)
    {
        const uint32_t* hv = m->hexs + 8 * i;
        m->ecache[m->nt + m->np + i] = (uint32_t)m->nbg;
        unsigned s = 0;
        for (unsigned k = 1; k < 8; ++k)
            if (hv[k] < hv[s]) s = k;
        unsigned v[8];
        for (int k = 0; k < 8; ++k) v[k] = hv[HEX_ROT[s][k]];
        unsigned diag = 0;
        if (umin(v[1], v[6]) < umin(v[2], v[5])) diag |= 4u;
        if (umin(v[3], v[6]) < umin(v[2], v[7])) diag |= 2u;
        if (umin(v[4], v[6]) < umin(v[5], v[7])) diag |= 1u;
        unsigned tmp;
        if (HEX_LOOP[diag] == 120)
        {
            tmp = v[1]; v[1] = v[4]; v[4] = v[3]; v[3] = tmp;
            tmp = v[5]; v[5] = v[7]; v[7] = v[2]; v[2] = tmp;
        }
        else if (HEX_LOOP[diag] == 240)
        {
            tmp = v[1]; v[1] = v[3]; v[3] = v[4]; v[4] = tmp;
            tmp = v[5]; v[5] = v[2]; v[2] = v[7]; v[7] = tmp;
        }
        switch ((diag & 1u) + ((diag & 2u) >> 1) + ((diag & 4u) >> 2))
        {
        case 0:
            bg_push(m, v[0], v[1], v[2], v[5]);
            bg_push(m, v[0], v[2], v[7], v[5]);
            bg_push(m, v[0], v[2], v[3], v[7]);
            bg_push(m, v[0], v[5], v[7], v[4]);
            bg_push(m, v[2], v[7], v[5], v[6]);
            break;
        case 1:
            bg_push(m, v[0], v[5], v[7], v[4]);
            bg_push(m, v[0], v[1], v[7], v[5]);
            bg_push(m, v[1], v[6], v[7], v[5]);
            bg_push(m, v[0], v[7], v[2], v[3]);
            bg_push(m, v[0], v[7], v[1], v[2]);
            bg_push(m, v[1], v[7], v[6], v[2]);
            break;
        case 2:
            bg_push(m, v[0], v[4], v[5], v[6]);
            bg_push(m, v[0], v[3], v[7], v[6]);
            bg_push(m, v[0], v[7], v[4], v[6]);
            bg_push(m, v[0], v[1], v[2], v[5]);
            bg_push(m, v[0], v[3], v[6], v[2]);
            bg_push(m, v[0], v[6], v[5], v[2]);
            break;
        default:
            bg_push(m, v[0], v[2], v[3], v[6]);
            bg_push(m, v[0], v[3], v[7], v[6]);
            bg_push(m, v[0], v[7], v[4], v[6]);
            bg_push(m, v[0], v[5], v[6], v[4]);
            bg_push(m, v[1], v[5], v[6], v[0]);
            bg_push(m, v[1], v[6], v[2], v[0]);
            break;
        }
    }
}

typedef struct
{
    uint32_t key[3];
    uint32_t tet, side;
} face_rec;

static int face_cmp(const void* pa, const void* pb)
{
    const face_rec* a = (const face_rec*)pa;
    const face_rec* b = (const face_rec*)pb;
    for (int k = 0; k < 3; ++k)
        if (a->key[k] != b->key[k]) return a->key[k] < b->key[k] ? -1 : 1;
    if (a->tet != b->tet) return a->tet < b->tet ? -1 : 1;
    return a->side < b->side ? -1 : (a->side > b->side);
}

/* LocalSampler::buildBackgroundMesh (Samplers/LocalSampler.cpp:352-429) at
 * the current positions: the background tets, the analytic metric at every
 * vertex (LocalSampler::updateAnalyticalMetric, :186-203), the two tets of
 * every shared face linked as neighbours (the XOR set of TriSet pairs a face's
 * first and second owner; sorting the faces pairs them alike), and every
 * vertex's cache the last tet holding it */
static void build_background(om_mesh* m)
{
    free(m->bg);
    free(m->bg_pos);
    free(m->bg_metric);
    free(m->vcache);
    free(m->ecache);
    const int64_t maxbg = m->nt + 3 * m->np + 6 * m->nh;
    m->bg = (uint32_t*)malloc(sizeof(uint32_t) * 8 * (size_t)(maxbg + 1));
    m->ecache = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(m->nt + m->np + m->nh + 1));
    m->vcache = (uint32_t*)calloc((size_t)m->nv + 1, sizeof(uint32_t));
    m->bg_pos = (double*)malloc(sizeof(double) * 3 * (size_t)(m->nv + 1));
    m->bg_metric = (m3*)malloc(sizeof(m3) * (size_t)(m->nv + 1));
    memcpy(m->bg_pos, m->pos, sizeof(double) * 3 * (size_t)m->nv);
    for (int64_t v = 0; v < m->nv; ++v) m->bg_metric[v] = analytic_metric(m, P(m, (uint32_t)v));
    tetrahedrize(m);
    face_rec* f = (face_rec*)malloc(sizeof(face_rec) * 4 * (size_t)(m->nbg + 1));
    for (int64_t t = 0; t < m->nbg; ++t)
        for (int s = 0; s < 4; ++s)
        {
            face_rec* r = f + 4 * t + s;
            uint32_t a = m->bg[8 * t + TET_TRIS[s][0]], b = m->bg[8 * t + TET_TRIS[s][1]], c = m->bg[8 * t + TET_TRIS[s][2]];
            uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            if (c < lo) { r->key[0] = c; r->key[1] = lo; r->key[2] = hi; }
            else if (c < hi) { r->key[0] = lo; r->key[1] = c; r->key[2] = hi; }
            else { r->key[0] = lo; r->key[1] = hi; r->key[2] = c; }
            r->tet = (uint32_t)t;
            r->side = (uint32_t)s;
        }
    qsort(f, (size_t)(4 * m->nbg), sizeof(face_rec), face_cmp);
    for (int64_t i = 0; i + 1 < 4 * m->nbg;)
    {
        if (memcmp(f[i].key, f[i + 1].key, sizeof(f[i].key)) == 0)
        {
            m->bg[8 * (size_t)f[i].tet + 4 + f[i].side] = f[i + 1].tet;
            m->bg[8 * (size_t)f[i + 1].tet + 4 + f[i + 1].side] = f[i].tet;
            i += 2;
        }
        else
            ++i;
    }
    free(f);
    for (int64_t t = 0; t < m->nbg; ++t)
        for (int k = 0; k < 4; ++k) m->vcache[m->bg[8 * t + k]] = (uint32_t)t;
}

/* ------------------------------------------------------------------------ */
/* kd-tree and texture samplers                                              */
/* ------------------------------------------------------------------------ */

static m3 local_metric(const om_mesh* m, v3 position, uint32_t cache);

/* the reference sorts vertex ids by one coordinate with std::sort; the same
 * call (same comparisons, same order among equal coordinates) is made from
 * the C++ helper oracle/om_sort.cpp */
void om_argsort_axis(const double* pos, int64_t n, int axis, uint32_t* out);

struct om_kd
{
    int64_t left, right;
    double sep[4]; /* axis, then the separator value; a leaf keeps zeros */
    m3 metric;
};

static int64_t kd_push(om_mesh* m)
{
    if (m->nkd == m->kd_cap)
    {
        m->kd_cap = m->kd_cap ? 2 * m->kd_cap : 64;
        m->kd = (struct om_kd*)realloc(m->kd, sizeof(struct om_kd) * (size_t)m->kd_cap);
    }
    struct om_kd* k = m->kd + m->nkd;
    memset(k, 0, sizeof(*k));
    k->left = k->right = -1;
    return m->nkd++;
}

static double coord(const om_mesh* m, uint32_t v, int axis) { return m->pos[3 * (size_t)v + axis]; }

/* KdTreeSampler::build (KdTreeSampler.cpp:268-372): split at the median of
 * the widest extent (x, then y, then z on ties), vertices on the separator
 * going to both sides; a leaf (height 0 or at most 3 vertices) holds the
 * local metric at its vertices' mean, its walk started at the first vertex's
 * cache */
static int64_t kd_build(om_mesh* m, int height, uint32_t* xs, uint32_t* ys, uint32_t* zs, int64_t n)
{
    const int64_t id = kd_push(m);
    if (height > 0 && n > 3)
    {
        const double ex = coord(m, xs[n - 1], 0) - coord(m, xs[0], 0);
        const double ey = coord(m, ys[n - 1], 1) - coord(m, ys[0], 1);
        const double ez = coord(m, zs[n - 1], 2) - coord(m, zs[0], 2);
        v3 axis = V(1, 0, 0);
        const int64_t r = n / 2, l = r - 1;
        uint32_t sl = xs[l], sr = xs[r];
        if (ey >= ex && ey >= ez)
        {
            axis = V(0, 1, 0);
            sl = ys[l];
            sr = ys[r];
        }
        else if (ez >= ex && ez >= ey)
        {
            axis = V(0, 0, 1);
            sl = zs[l];
            sr = zs[r];
        }
        v3 sp;
        if (n % 2 == 0)
        {
            v3 a = P(m, sl), b = P(m, sr);
            sp = V((a.x + b.x) / 2.0, (a.y + b.y) / 2.0, (a.z + b.z) / 2.0);
        }
        else
            sp = P(m, sr);
        const double sv = dot(axis, sp);
        m->kd[id].sep[0] = axis.x;
        m->kd[id].sep[1] = axis.y;
        m->kd[id].sep[2] = axis.z;
        m->kd[id].sep[3] = sv;
        uint32_t* lists[6];
        int64_t cnt[6] = {0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 6; ++q) lists[q] = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n + 1));
        uint32_t* src[3] = {xs, ys, zs};
        for (int64_t v = 0; v < n; ++v)
            for (int q = 0; q < 3; ++q)
            {
                const double d = dot(P(m, src[q][v]), axis) - sv;
                if (d <= 0.0) lists[2 * q][cnt[2 * q]++] = src[q][v];
                if (d >= 0.0) lists[2 * q + 1][cnt[2 * q + 1]++] = src[q][v];
            }
        const int64_t left = kd_build(m, height - 1, lists[0], lists[2], lists[4], cnt[0]);
        m->kd[id].left = left;
        const int64_t right = kd_build(m, height - 1, lists[1], lists[3], lists[5], cnt[1]);
        m->kd[id].right = right;
        for (int q = 0; q < 6; ++q) free(lists[q]);
    }
    else
    {
        v3 mean = V(0, 0, 0);
        for (int64_t v = 0; v < n; ++v) mean = add(mean, P(m, xs[v]));
        const double dn = (double)n;
        mean = V(mean.x / dn, mean.y / dn, mean.z / dn);
        m->kd[id].metric = local_metric(m, mean, m->vcache[xs[0]]);
    }
    return id;
}

/* KdTreeSampler::updateAnalyticalMetric (KdTreeSampler.cpp:116-180) */
static void build_kdtree(om_mesh* m)
{
    m->nkd = 0;
    int height = m->depth;
    if (height < 0) height = (int)log2(ceil((double)m->nv / 3.0));
    uint32_t* s[3];
    for (int a = 0; a < 3; ++a)
    {
        s[a] = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(m->nv + 1));
        om_argsort_axis(m->pos, m->nv, a, s[a]);
    }
    kd_build(m, height, s[0], s[1], s[2], m->nv);
    for (int a = 0; a < 3; ++a) free(s[a]);
}

/* KdTreeSampler::metricAt (KdTreeSampler.cpp:218-247) */
static m3 kd_metric(const om_mesh* m, v3 p)
{
    int64_t node = -1, child = 0;
    while (child != -1)
    {
        node = child;
        const struct om_kd* k = m->kd + node;
        child = dot(p, V(k->sep[0], k->sep[1], k->sep[2])) - k->sep[3] < 0.0 ? k->left : k->right;
    }
    return m->kd[node].metric;
}

/* TextureSampler::cellId (TextureSampler.cpp:513-524) */
static void tex_cell(const om_mesh* m, const double* pos, int* id)
{
    for (int k = 0; k < 3; ++k)
    {
        const double r = (pos[k] - m->tex_min[k]) / m->tex_ext[k];
        int c = (int)(r * (double)m->tex_size[k]);
        id[k] = c < 0 ? 0 : c > m->tex_size[k] - 1 ? m->tex_size[k] - 1 : c;
    }
}

static size_t tex_index(const om_mesh* m, int i, int j, int k)
{
    return ((size_t)k * m->tex_size[1] + j) * m->tex_size[0] + i;
}

/* TextureSampler::buildGrid (TextureSampler.cpp:275-448): a grid of about
 * one cell per vertex over the bounding box; each background tet, in order,
 * fills the unset cells of its cell box grown by one with the local metric
 * at the cell centres, its walk started at that tet.  Cells no tet box
 * reaches keep the default metric (identity). */
static void build_texture(om_mesh* m)
{
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t v = 0; v < m->nv; ++v)
        for (int k = 0; k < 3; ++k)
        {
            const double x = m->pos[3 * v + k];
            lo[k] = x < lo[k] ? x : lo[k];
            hi[k] = x > hi[k] ? x : hi[k];
        }
    for (int k = 0; k < 3; ++k)
    {
        m->tex_min[k] = lo[k];
        m->tex_ext[k] = hi[k] - lo[k];
    }
    double cells = (double)m->nv;
    if (m->depth > 0) cells = (double)((size_t)m->depth * m->depth * m->depth);
    const double alpha = pow(cells / (m->tex_ext[0] * m->tex_ext[1] * m->tex_ext[2]), 1 / 3.0);
    for (int k = 0; k < 3; ++k)
    {
        const double e = alpha * m->tex_ext[k];
        m->tex_size[k] = (int)round(e > 1.0 ? e : 1.0);
    }
    const size_t n = (size_t)m->tex_size[0] * m->tex_size[1] * m->tex_size[2];
    free(m->tex);
    m->tex = (m3*)malloc(sizeof(m3) * n);
    unsigned char* set = (unsigned char*)calloc(n, 1);
    for (size_t c = 0; c < n; ++c) m->tex[c] = mdiag(1, 1, 1);
    double cs[3];
    for (int k = 0; k < 3; ++k) cs[k] = m->tex_ext[k] / (double)m->tex_size[k];
    for (int64_t e = 0; e < m->nbg; ++e)
    {
        double bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int v = 0; v < 4; ++v)
            for (int k = 0; k < 3; ++k)
            {
                const double x = m->pos[3 * (size_t)m->bg[8 * e + v] + k];
                bmin[k] = x < bmin[k] ? x : bmin[k];
                bmax[k] = x > bmax[k] ? x : bmax[k];
            }
        int a[3], b[3];
        tex_cell(m, bmin, a);
        tex_cell(m, bmax, b);
        for (int k = 0; k < 3; ++k)
        {
            a[k] = a[k] - 1 < 0 ? 0 : a[k] - 1;
            b[k] = b[k] + 1 > m->tex_size[k] - 1 ? m->tex_size[k] - 1 : b[k] + 1;
        }
        for (int z = a[2]; z <= b[2]; ++z)
            for (int y = a[1]; y <= b[1]; ++y)
                for (int x = a[0]; x <= b[0]; ++x)
                {
                    const size_t c = tex_index(m, x, y, z);
                    if (set[c]) continue;
                    const v3 p = V(m->tex_min[0] + cs[0] * ((double)x + 0.5), m->tex_min[1] + cs[1] * ((double)y + 0.5),
                                   m->tex_min[2] + cs[2] * ((double)z + 0.5));
                    m->tex[c] = local_metric(m, p, (uint32_t)e);
                    set[c] = 1;
                }
    }
    free(set);
}

/* glm::mix of two metrics: a + (b - a) t, per entry */
static m3 mmix(m3 a, m3 b, double t) { return madd(a, mscale(msub(b, a), t)); }

/* TextureSampler::metricAt (TextureSampler.cpp:450-488): trilinear between
 * the eight cell centres around the point, clamped at the grid's border */
static m3 tex_metric(const om_mesh* m, v3 p)
{
    const double pc[3] = {p.x, p.y, p.z};
    double cs[3], cp0[3], a[3];
    int i0[3], i1[3];
    for (int k = 0; k < 3; ++k)
    {
        cs[k] = m->tex_ext[k] / (double)m->tex_size[k];
        const double minb = m->tex_min[k], maxb = m->tex_min[k] + m->tex_ext[k] - cs[k] * 1.5;
        const double q = pc[k] + (-cs[k]) / 2.0;
        cp0[k] = q < minb ? minb : q > maxb ? maxb : q;
    }
    tex_cell(m, cp0, i0);
    for (int k = 0; k < 3; ++k)
    {
        i1[k] = i0[k] + 1 < m->tex_size[k] - 1 ? i0[k] + 1 : m->tex_size[k] - 1;
        const double c0 = cs[k] * ((double)i0[k] + 0.5);
        const double t = (pc[k] - (m->tex_min[k] + c0)) / cs[k];
        a[k] = t < 0.0 ? 0.0 : t > 1.0 ? 1.0 : t;
    }
    const m3 m000 = m->tex[tex_index(m, i0[0], i0[1], i0[2])], m100 = m->tex[tex_index(m, i1[0], i0[1], i0[2])];
    const m3 m010 = m->tex[tex_index(m, i0[0], i1[1], i0[2])], m110 = m->tex[tex_index(m, i1[0], i1[1], i0[2])];
    const m3 m001 = m->tex[tex_index(m, i0[0], i0[1], i1[2])], m101 = m->tex[tex_index(m, i1[0], i0[1], i1[2])];
    const m3 m011 = m->tex[tex_index(m, i0[0], i1[1], i1[2])], m111 = m->tex[tex_index(m, i1[0], i1[1], i1[2])];
    const m3 mx00 = mmix(m000, m100, a[0]), mx10 = mmix(m010, m110, a[0]);
    const m3 mx01 = mmix(m001, m101, a[0]), mx11 = mmix(m011, m111, a[0]);
    const m3 mxy0 = mmix(mx00, mx10, a[1]), mxy1 = mmix(mx01, mx11, a[1]);
    return mmix(mxy0, mxy1, a[2]);
}

void om_set_discretization_depth(om_mesh* m, int32_t depth) { m->depth = depth; }

void om_set_crew(om_mesh* m, int32_t sampler, int32_t measurer, int32_t evaluator,
                 double scaling, double aspect_ratio)
{
    m->sampler = sampler;
    m->measurer = measurer;
    m->evaluator = evaluator;
    /* AbstractSampler::setScaling (Samplers/AbstractSampler.cpp:46-51) */
    m->scaling = scaling;
    m->scaling2 = m->scaling * scaling;
    m->scaling3 = m->scaling2 * scaling;
    m->aspect_ratio = aspect_ratio;
    /* AbstractSampler ctor rotation (Samplers/AbstractSampler.cpp:30-40) */
    m3 id = mdiag(1, 1, 1);
    m->rot = mrotate(id, 3.14159265358979323846 / 4.0, V(0, 0, 1));
    m->rot = mrotate(m->rot, 3.14159265358979323846 / 4.0, V(0, -1, 0));
    m->rotinv = mtranspose(m->rot);
    /* GpuMeshCharacter::updateSampling: updateAnalyticalMetric at crew set-up;
     * the kd-tree and texture samplers sample a local sampler built the same
     * way (KdTreeSampler.cpp:157-161, TextureSampler.cpp:257-267) */
    if (sampler >= OM_SAMPLER_LOCAL) build_background(m);
    if (sampler == OM_SAMPLER_KDTREE) build_kdtree(m);
    if (sampler == OM_SAMPLER_TEXTURE) build_texture(m);
}

void om_get_pos(const om_mesh* m, double* out) { memcpy(out, m->pos, sizeof(double) * 3 * (size_t)m->nv); }
void om_set_pos(om_mesh* m, const double* in) { memcpy(m->pos, in, sizeof(double) * 3 * (size_t)m->nv); }
int64_t om_patch_eval_count(const om_mesh* m) { return m->patch_evals; }
void om_reset_patch_eval_count(om_mesh* m) { m->patch_evals = 0; }

/* ------------------------------------------------------------------------ */
/* boundary projection                                                       */
/* ------------------------------------------------------------------------ */

static inline int is_constrained(const om_mesh* m, uint32_t v) { return m->cid[v] != 0; }

static v3 project_id(const om_mesh* m, int32_t id, v3 pos)
{
    if (id <= 0 || id >= m->ncon) return pos; /* VolumeConstraint: identity */
    const double* pp = m->con_param + 6 * id;
    const double* d = m->con_derived + 4 * id;
    switch (m->con_kind[id])
    {
    case OM_CON_PLANE:
    {
        /* PlaneConstraint::operator() (FaceConstraint.cpp:180-185) */
        v3 n = V(d[0], d[1], d[2]);
        v3 dist = sub(pos, V(pp[0], pp[1], pp[2]));
        double l = dot(dist, n);
        return sub(pos, mul(n, l));
    }
    case OM_CON_SEGMENT:
    {
        /* SegmentConstraint::operator() (EdgeConstraint.cpp:185-199) */
        v3 a = V(pp[0], pp[1], pp[2]);
        v3 u = V(d[0], d[1], d[2]);
        v3 dist = sub(pos, a);
        double l = dot(dist, u);
        if (l < 0) return a;
        else if (l > d[3]) return V(pp[3], pp[4], pp[5]);
        else
        {
            v3 t = sub(dist, mul(u, l));
            return sub(pos, t);
        }
    }
    case OM_CON_SPHERE:
        /* SphereBoundary::Face::operator() (SphereBoundary.cpp:42-45) */
        return normalize(pos);
    case OM_CON_POINT:
        return V(pp[0], pp[1], pp[2]);
    case OM_CON_SHELL_INNER:
        /* ShellBoundary::InFace::operator() (ShellBoundary.cpp:41-44) */
        return mul(normalize(pos), 0.5);
    case OM_CON_PIPE_CYLINDER:
    {
        /* PipeBoundary::CylinderFace::operator() (PipeBoundary.cpp:43-56),
         * PIPE_RADIUS 0.3 (:3) */
        v3 center;
        if (pos.x < 0.5)
            center = V(pos.x, (pos.y < 0.0 ? -0.5 : 0.5), 0.0);
        else
        {
            center = sub(pos, V(0.5, 0.0, pos.z));
            center = mul(normalize(center), 0.5);
            center = add(V(0.5, 0, 0), center);
        }
        v3 dist = sub(pos, center);
        v3 extProj = mul(normalize(dist), 0.3);
        return add(center, extProj);
    }
    case OM_CON_PIPE_CIRCLE:
    {
        /* PipeBoundary::YNeg/YPosCircleEdge::operator() (PipeBoundary.cpp:
         * 100-105, 111-116): the circle of radius 0.3 about the end-face
         * centre, in the face of normal EXT_FACE_NORMAL = (-1, 0, 0) */
        v3 c = V(pp[0], pp[1], pp[2]);
        v3 n = V(-1, 0, 0);
        v3 dist = sub(pos, c);
        double offset = dot(dist, n);
        v3 extProj = sub(dist, mul(n, offset));
        return add(c, mul(normalize(extProj), 0.3));
    }
    default:
        return pos;
    }
}

/* (*topo.snapToBoundary)(pos).  A fixed vertex (id < 0) carries a
 * VertexConstraint built from its own position (MeshTopo(fixedPosition),
 * DataStructures/Mesh.cpp:149-152; VertexConstraint.cpp:60-63), and fixed
 * vertices never move, so its projection is its current position. */
static inline v3 snap(const om_mesh* m, uint32_t v, v3 pos)
{
    if (m->cid[v] < 0) return P(m, v);
    return project_id(m, m->cid[v], pos);
}

void om_project(const om_mesh* m, int64_t v, const double* in, double* out)
{
    v3 r = snap(m, (uint32_t)v, V(in[0], in[1], in[2]));
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

/* ------------------------------------------------------------------------ */
/* samplers                                                                  */
/* ------------------------------------------------------------------------ */

/* AbstractSampler::vertMetric(position) (AbstractSampler.cpp:190-208) */
static m3 analytic_metric(const om_mesh* m, v3 p)
{
    double x = mmulv(m->rot, p).x * (2.5 * 3.14159265358979323846);
    double a = m->aspect_ratio;
    double c = (1.0 - cos(x)) / 2.0;
    double sizeX = m->scaling * pow(a, pow(c, a));
    double Mx = sizeX * sizeX;
    double My = m->scaling2;
    double Mz = My;
    m3 Mm = mdiag(Mx, My, Mz);
    return mmul(mmul(m->rotinv, Mm), m->rot);
}

/* The sampler cache of the element or vertex being measured: LocalSampler::
 * metricAt starts its walk at the background tet it names.  The measures set
 * it per element (its first background tet) and per sampled vertex (the
 * vertex's cache); thread-local, since passes run on several threads. */
static __thread uint32_t tl_cache;

/* tetParams (DataStructures/Tetrahedralizer.h:211-234): barycentric
 * coordinates of p in background tet t; inside within -1e-4 */
static int bg_params(const om_mesh* m, const uint32_t* t, v3 p, double coor[4])
{
    v3 vp0 = V(m->bg_pos[3 * t[0]], m->bg_pos[3 * t[0] + 1], m->bg_pos[3 * t[0] + 2]);
    v3 vp1 = V(m->bg_pos[3 * t[1]], m->bg_pos[3 * t[1] + 1], m->bg_pos[3 * t[1] + 2]);
    v3 vp2 = V(m->bg_pos[3 * t[2]], m->bg_pos[3 * t[2] + 1], m->bg_pos[3 * t[2] + 2]);
    v3 vp3 = V(m->bg_pos[3 * t[3]], m->bg_pos[3 * t[3] + 1], m->bg_pos[3 * t[3] + 2]);
    m3 T = M(sub(vp0, vp3), sub(vp1, vp3), sub(vp2, vp3));
    v3 y = mmulv(minverse(T), sub(p, vp3));
    coor[0] = y.x;
    coor[1] = y.y;
    coor[2] = y.z;
    coor[3] = 1.0 - (y.x + y.y + y.z);
    const double EPSILON_IN = -1e-4;
    return coor[0] >= EPSILON_IN && coor[1] >= EPSILON_IN && coor[2] >= EPSILON_IN && coor[3] >= EPSILON_IN;
}

/* triIntersect (Tetrahedralizer.h:236-271): the ray orig + s dir crosses the
 * triangle (v1, v2, v3) from its front */
static int tri_intersect(v3 v1, v3 v2, v3 v3_, v3 orig, v3 dir)
{
    const double EPSILON = 1e-12;
    v3 e1 = sub(v2, v1);
    v3 e2 = sub(v3_, v1);
    v3 pvec = cross(dir, e2);
    double det = dot(pvec, e1);
    if (det < EPSILON) return 0;
    v3 tvec = sub(orig, v1);
    double u = dot(tvec, pvec);
    if (u < 0.0 || u > det) return 0;
    v3 qvec = cross(tvec, e1);
    double v = dot(dir, qvec);
    if (v < 0.0 || v + u > det) return 0;
    return 1;
}

/* LocalSampler::metricAt (Samplers/LocalSampler.cpp:212-311): walk the
 * background mesh from tet `cache` (through the face a ray from the current
 * tet's centroid, or from one of four weighted interior points, leaves), then
 * interpolate the vertex metrics barycentrically; a point outside the mesh
 * takes the clamped coordinates of the last tet.
 *
 * One addition: the reference's walk has no step limit, and on some inputs
 * its rays cycle through a ring of tets and it never returns (a mixed box
 * mesh jittered by 0.3 of a cell after one gradient-descent pass is one).
 * Here, as on the GPU, a walk that has moved OM_LOCAL_WALK times without
 * reaching the tet holding the point stops and takes the current tet's
 * clamped coordinates, as an unreachable point does.  Walks that end within
 * the limit are the reference's step for step. */
#define OM_LOCAL_WALK 512
static m3 local_metric(const om_mesh* m, v3 position, uint32_t cache)
{
    const uint32_t* tet = m->bg + 8 * (size_t)cache;
    double coor[4];
    int isUnreachable = 0;
    int steps = 0;
    while (!isUnreachable && !bg_params(m, tet, position, coor))
    {
        if (++steps > OM_LOCAL_WALK)
        {
            isUnreachable = 1;
            break;
        }
        v3 vp[4];
        for (int k = 0; k < 4; ++k)
            vp[k] = V(m->bg_pos[3 * tet[k]], m->bg_pos[3 * tet[k] + 1], m->bg_pos[3 * tet[k] + 2]);
        v3 orig = mul(add(add(add(vp[0], vp[1]), vp[2]), vp[3]), 0.25);
        v3 dir = normalize(sub(orig, position));
        int t = 4;
        int trialCount = -1;
        while (t == 4 && !isUnreachable)
        {
            for (t = 0; t < 4; ++t)
            {
                if (tri_intersect(vp[TET_TRIS[t][0]], vp[TET_TRIS[t][1]], vp[TET_TRIS[t][2]], orig, dir))
                {
                    if (tet[4 + t] != BG_NONE) tet = m->bg + 8 * (size_t)tet[4 + t];
                    else isUnreachable = 1;
                    break;
                }
            }
            if (t == 4)
            {
                ++trialCount;
                if (trialCount < 4)
                {
                    const double INV_MASS = 1.0 / 10.0;
                    const double WEIGHTS[] = {1.0, 2.0, 3.0, 4.0};
                    v3 s = add(add(add(mul(vp[0], WEIGHTS[(trialCount + 0) % 4]), mul(vp[1], WEIGHTS[(trialCount + 1) % 4])),
                                   mul(vp[2], WEIGHTS[(trialCount + 2) % 4])),
                               mul(vp[3], WEIGHTS[(trialCount + 3) % 4]));
                    orig = mul(s, INV_MASS);
                    dir = normalize(sub(orig, position));
                }
                else
                {
                    isUnreachable = 1;
                    break;
                }
            }
        }
    }
    if (isUnreachable)
    {
        double sum = 0.0;
        for (int k = 0; k < 4; ++k)
        {
            if (coor[k] < 0.0) coor[k] = 0.0;
            else sum += coor[k];
        }
        for (int k = 0; k < 4; ++k) coor[k] /= sum;
    }
    m3 r = mscale(m->bg_metric[tet[0]], coor[0]);
    r = madd(r, mscale(m->bg_metric[tet[1]], coor[1]));
    r = madd(r, mscale(m->bg_metric[tet[2]], coor[2]));
    r = madd(r, mscale(m->bg_metric[tet[3]], coor[3]));
    return r;
}

static m3 metric_at(const om_mesh* m, v3 p)
{
    switch (m->sampler)
    {
    case OM_SAMPLER_ANALYTIC:
        /* AnalyticSampler::metricAt (AnalyticSampler.cpp:45-49) */
        return analytic_metric(m, p);
    case OM_SAMPLER_LOCAL:
        return local_metric(m, p, tl_cache);
    case OM_SAMPLER_KDTREE:
        return kd_metric(m, p);
    case OM_SAMPLER_TEXTURE:
        return tex_metric(m, p);
    case OM_SAMPLER_SINE:
    {
        /* sine-graded anisotropic metric s^2 * diag(1 + 9 sin^2(4 pi x), 1, 1):
         * a new sampler plugin with the shape of UniformSampler::metricAt */
        double sx = sin(4.0 * 3.14159265358979323846 * p.x);
        double s2 = m->scaling2;
        return mdiag(s2 * (1.0 + 9.0 * sx * sx), s2, s2);
    }
    default:
        /* UniformSampler::metricAt (UniformSampler.cpp:45-51) */
        return mdiag(m->scaling * m->scaling, m->scaling * m->scaling, m->scaling * m->scaling);
    }
}

void om_metric_at(const om_mesh* m, const double* p, double* out9)
{
    m3 r = metric_at(m, V(p[0], p[1], p[2]));
    memcpy(out9, &r, sizeof(double) * 9);
}

/* ------------------------------------------------------------------------ */
/* measurers                                                                 */
/* ------------------------------------------------------------------------ */

/* MetricWiseMeasurer::riemannianDistance, localized segment division
 * (Measurers/MetricWiseMeasurer.cpp:9,64-116) */
static double metric_wise_distance(const om_mesh* m, v3 a, v3 b)
{
    const double DIFF_THRESHOLD = 0.01;
    int curr = 0;
    int base = 2;
    double len = 0.0;
    v3 d = sub(b, a);
    v3 bv = dvs(d, (double)base);
    while (curr < base)
    {
        double p0 = (curr + 0.5) / base;
        double p1 = (curr + 1.5) / base;
        m3 M0 = metric_at(m, add(a, mul(d, p0)));
        m3 M1 = metric_at(m, add(a, mul(d, p1)));
        double l0 = sqrt(dot(bv, mmulv(M0, bv)));
        double l1 = sqrt(dot(bv, mmulv(M1, bv)));
        double sum = (l0 + l1);
        double diff = fabs(l0 - l1) / (sum / 2.0);
        if (diff < DIFF_THRESHOLD)
        {
            len += sum;
            curr += 2;
            if ((curr & 2) == 0)
            {
                base >>= 1;
                curr >>= 1;
            }
            bv = dvs(d, (double)base);
        }
        else
        {
            base <<= 1;
            curr <<= 1;
            bv = dvs(bv, 2.0);
        }
    }
    return len;
}

double om_riemannian_distance(const om_mesh* m, const double* a, const double* b)
{
    v3 A = V(a[0], a[1], a[2]), B = V(b[0], b[1], b[2]);
    if (m->measurer == OM_MEASURER_METRIC_WISE) return metric_wise_distance(m, A, B);
    return length(sub(B, A)) * m->scaling;
}

/* riemannianSegment: MetricFreeMeasurer.cpp:36-43 / MetricWiseMeasurer.cpp:119-126 */
static inline v3 segment(const om_mesh* m, v3 a, v3 b)
{
    if (m->measurer == OM_MEASURER_METRIC_WISE)
        return mul(normalize(sub(b, a)), metric_wise_distance(m, a, b));
    return mul(sub(b, a), m->scaling);
}

/* tet/pri/hex volumes: MetricFreeMeasurer.cpp:45-105, MetricWiseMeasurer.cpp:128-188 */
static double tet_volume(const om_mesh* m, const v3* vp)
{
    if (m->measurer == OM_MEASURER_METRIC_WISE)
    {
        double detSum = mdet(M(segment(m, vp[0], vp[3]), segment(m, vp[1], vp[3]),
                               segment(m, vp[2], vp[3])));
        return detSum / 6.0;
    }
    double detSum = mdet(M(sub(vp[3], vp[0]), sub(vp[3], vp[1]), sub(vp[3], vp[2])));
    return m->scaling3 * detSum / 6.0;
}

static double pri_volume(const om_mesh* m, const v3* vp)
{
    v3 e02, e12, e32, e42, e52;
    if (m->measurer == OM_MEASURER_METRIC_WISE)
    {
        e02 = segment(m, vp[0], vp[2]);
        e12 = segment(m, vp[1], vp[2]);
        e32 = segment(m, vp[3], vp[2]);
        e42 = segment(m, vp[4], vp[2]);
        e52 = segment(m, vp[5], vp[2]);
    }
    else
    {
        e02 = sub(vp[2], vp[0]);
        e12 = sub(vp[2], vp[1]);
        e32 = sub(vp[2], vp[3]);
        e42 = sub(vp[2], vp[4]);
        e52 = sub(vp[2], vp[5]);
    }
    double detSum = 0.0;
    detSum += mdet(M(e32, e52, e42));
    detSum += mdet(M(e02, e32, e42));
    detSum += mdet(M(e12, e02, e42));
    if (m->measurer == OM_MEASURER_METRIC_WISE) return detSum / 6.0;
    return m->scaling3 * detSum / 6.0;
}

static double hex_volume(const om_mesh* m, const v3* vp)
{
    double detSum = 0.0;
    if (m->measurer == OM_MEASURER_METRIC_WISE)
    {
        detSum += mdet(M(segment(m, vp[1], vp[0]), segment(m, vp[4], vp[0]), segment(m, vp[3], vp[0])));
        detSum += mdet(M(segment(m, vp[1], vp[2]), segment(m, vp[3], vp[2]), segment(m, vp[6], vp[2])));
        detSum += mdet(M(segment(m, vp[4], vp[5]), segment(m, vp[1], vp[5]), segment(m, vp[6], vp[5])));
        detSum += mdet(M(segment(m, vp[4], vp[7]), segment(m, vp[6], vp[7]), segment(m, vp[3], vp[7])));
        detSum += mdet(M(segment(m, vp[1], vp[4]), segment(m, vp[6], vp[4]), segment(m, vp[3], vp[4])));
        return detSum / 6.0;
    }
    detSum += mdet(M(sub(vp[0], vp[1]), sub(vp[0], vp[4]), sub(vp[0], vp[3])));
    detSum += mdet(M(sub(vp[2], vp[1]), sub(vp[2], vp[3]), sub(vp[2], vp[6])));
    detSum += mdet(M(sub(vp[5], vp[4]), sub(vp[5], vp[1]), sub(vp[5], vp[6])));
    detSum += mdet(M(sub(vp[7], vp[4]), sub(vp[7], vp[6]), sub(vp[7], vp[3])));
    detSum += mdet(M(sub(vp[4], vp[1]), sub(vp[4], vp[6]), sub(vp[4], vp[3])));
    return m->scaling3 * detSum / 6.0;
}

/* AbstractMeasurer::computeLocalElementSize (Measurers/AbstractMeasurer.cpp:137-155) */
static double local_size(const om_mesh* m, uint32_t v)
{
    v3 pos = P(m, v);
    double total = 0.0;
    int64_t b = m->nvx_base[v], e = m->nvx_base[v + 1];
    for (int64_t n = b; n < e; ++n) total += length(sub(pos, P(m, m->nvx[n])));
    return total / (double)(e - b);
}

double om_local_size(const om_mesh* m, int64_t v) { return local_size(m, (uint32_t)v); }

/* ------------------------------------------------------------------------ */
/* evaluators                                                                */
/* ------------------------------------------------------------------------ */

/* MeanRatioEvaluator::cornerQuality (Evaluators/MeanRatioEvaluator.cpp:22-32) */
static inline double corner_quality(m3 Fk)
{
    double det = mdet(Fk);
    double frob2 = dot(Fk.c[0], Fk.c[0]) + dot(Fk.c[1], Fk.c[1]) + dot(Fk.c[2], Fk.c[2]);
    return gsign(det) * 3.0 * pow(fabs(det), 2.0 / 3.0) / frob2;
}

/* combine corner qualities: min if any <= 0, else harmonic mean
 * (MeanRatioEvaluator.cpp:91-110, 140-166) */
static inline double combine_corners(const double* q, int n)
{
    int bad = 0;
    for (int i = 0; i < n; ++i)
        if (q[i] <= 0.0) bad = 1;
    if (bad)
    {
        double mn = q[0];
        for (int i = 1; i < n; ++i)
            if (q[i] < mn) mn = q[i];
        return mn;
    }
    double s = 1 / q[0];
    for (int i = 1; i < n; ++i) s = s + 1 / q[i];
    return (double)n / s;
}

/* MeanRatioEvaluator::tetQuality (MeanRatioEvaluator.cpp:34-50) */
static double mr_tet(const om_mesh* m, const v3* vp)
{
    v3 e03 = segment(m, vp[0], vp[3]);
    v3 e13 = segment(m, vp[1], vp[3]);
    v3 e23 = segment(m, vp[2], vp[3]);
    m3 Fk0 = mmul(M(e03, e13, e23), *fr_tet_inv());
    return corner_quality(Fk0);
}

/* MeanRatioEvaluator::priQuality (MeanRatioEvaluator.cpp:52-111) */
static double mr_pri(const om_mesh* m, const v3* vp)
{
    v3 e03 = segment(m, vp[0], vp[3]);
    v3 e14 = segment(m, vp[1], vp[4]);
    v3 e25 = segment(m, vp[2], vp[5]);
    v3 e01 = segment(m, vp[0], vp[1]);
    v3 e12 = segment(m, vp[1], vp[2]);
    v3 e20 = segment(m, vp[2], vp[0]);
    v3 e34 = segment(m, vp[3], vp[4]);
    v3 e45 = segment(m, vp[4], vp[5]);
    v3 e53 = segment(m, vp[5], vp[3]);
    const m3* F = fr_pri_inv();
    double q[6];
    q[0] = corner_quality(mmul(M(neg(e01), e20, e03), *F));
    q[1] = corner_quality(mmul(M(neg(e12), e01, e14), *F));
    q[2] = corner_quality(mmul(M(neg(e20), e12, e25), *F));
    q[3] = corner_quality(mmul(M(neg(e34), e53, e03), *F));
    q[4] = corner_quality(mmul(M(neg(e45), e34, e14), *F));
    q[5] = corner_quality(mmul(M(neg(e53), e45, e25), *F));
    return combine_corners(q, 6);
}

/* MeanRatioEvaluator::hexQuality (MeanRatioEvaluator.cpp:113-167); note the
 * reference passes hex.c[3] for e23, which only matters for local samplers */
static double mr_hex(const om_mesh* m, const v3* vp)
{
    v3 e01 = segment(m, vp[0], vp[1]);
    v3 e03 = segment(m, vp[0], vp[3]);
    v3 e04 = segment(m, vp[0], vp[4]);
    v3 e12 = segment(m, vp[1], vp[2]);
    v3 e15 = segment(m, vp[1], vp[5]);
    v3 e23 = segment(m, vp[2], vp[3]);
    v3 e26 = segment(m, vp[2], vp[6]);
    v3 e37 = segment(m, vp[3], vp[7]);
    v3 e45 = segment(m, vp[4], vp[5]);
    v3 e47 = segment(m, vp[4], vp[7]);
    v3 e56 = segment(m, vp[5], vp[6]);
    v3 e67 = segment(m, vp[6], vp[7]);
    double q[8];
    q[0] = corner_quality(M(e01, e04, neg(e03)));
    q[1] = corner_quality(M(e01, e12, e15));
    q[2] = corner_quality(M(e12, e26, neg(e23)));
    q[3] = corner_quality(M(e03, e23, e37));
    q[4] = corner_quality(M(e04, e45, e47));
    q[5] = corner_quality(M(e15, neg(e56), e45));
    q[6] = corner_quality(M(e26, e56, e67));
    q[7] = corner_quality(M(e37, e67, neg(e47)));
    return combine_corners(q, 8);
}

/* MetricConformityEvaluator::specifiedMetric (MetricConformityEvaluator.cpp:25-44) */
static m3 specified_metric(const om_mesh* m, v3 v0, v3 v1, v3 v2, v3 v3_)
{
    const double H = 0.5;
    const double Q = (1.0 - H) / 3.0;
    m3 r = mscale(metric_at(m, dvs(add(add(add(v0, v1), v2), v3_), 4.0)), -0.8);
    r = madd(r, mscale(metric_at(m, add(add(add(mul(v0, H), mul(v1, Q)), mul(v2, Q)), mul(v3_, Q))), 0.45));
    r = madd(r, mscale(metric_at(m, add(add(add(mul(v0, Q), mul(v1, H)), mul(v2, Q)), mul(v3_, Q))), 0.45));
    r = madd(r, mscale(metric_at(m, add(add(add(mul(v0, Q), mul(v1, Q)), mul(v2, H)), mul(v3_, Q))), 0.45));
    r = madd(r, mscale(metric_at(m, add(add(add(mul(v0, Q), mul(v1, Q)), mul(v2, Q)), mul(v3_, H))), 0.45));
    return r;
}

/* MetricConformityEvaluator::metricConformity (MetricConformityEvaluator.cpp:46-71) */
static double metric_conformity(m3 Fk, m3 Ms)
{
    m3 Fk_inv = minverse(mtranspose(Fk));
    m3 Mk = mmul(Fk_inv, mtranspose(Fk_inv));
    m3 Mk_inv = minverse(Mk);
    m3 Ms_inv = minverse(Ms);
    m3 tNc = msub(madd(mmul(Mk_inv, Ms), mmul(Ms_inv, Mk)), mdiag(2.0, 2.0, 2.0));
    double frob2 = dot(tNc.c[0], tNc.c[0]) + dot(tNc.c[1], tNc.c[1]) + dot(tNc.c[2], tNc.c[2]);
    if (!isnan(frob2))
    {
        double Fk_sign = gsign(mdet(Fk));
        return Fk_sign / sqrt(1.0 + sqrt(frob2));
    }
    return 0.0;
}

/* MetricConformityEvaluator::tetQuality (MetricConformityEvaluator.cpp:73-89) */
static double mc_tet(const om_mesh* m, const v3* vp)
{
    v3 e03 = sub(vp[3], vp[0]);
    v3 e13 = sub(vp[3], vp[1]);
    v3 e23 = sub(vp[3], vp[2]);
    m3 Fk = mmul(M(e03, e13, e23), *fr_tet_inv());
    m3 Ms0 = specified_metric(m, vp[0], vp[1], vp[2], vp[3]);
    return metric_conformity(Fk, Ms0);
}

/* MetricConformityEvaluator::priQuality (MetricConformityEvaluator.cpp:91-148) */
static double mc_pri(const om_mesh* m, const v3* vp)
{
    v3 e03 = sub(vp[3], vp[0]);
    v3 e14 = sub(vp[4], vp[1]);
    v3 e25 = sub(vp[5], vp[2]);
    v3 e01 = sub(vp[1], vp[0]);
    v3 e12 = sub(vp[2], vp[1]);
    v3 e20 = sub(vp[0], vp[2]);
    v3 e34 = sub(vp[4], vp[3]);
    v3 e45 = sub(vp[5], vp[4]);
    v3 e53 = sub(vp[3], vp[5]);
    const m3* F = fr_pri_inv();
    double q[6];
    q[0] = metric_conformity(mmul(M(neg(e01), e20, e03), *F), specified_metric(m, vp[0], vp[1], vp[2], vp[3]));
    q[1] = metric_conformity(mmul(M(neg(e12), e01, e14), *F), specified_metric(m, vp[0], vp[1], vp[2], vp[4]));
    q[2] = metric_conformity(mmul(M(neg(e20), e12, e25), *F), specified_metric(m, vp[0], vp[1], vp[2], vp[5]));
    q[3] = metric_conformity(mmul(M(neg(e34), e53, e03), *F), specified_metric(m, vp[0], vp[3], vp[4], vp[5]));
    q[4] = metric_conformity(mmul(M(neg(e45), e34, e14), *F), specified_metric(m, vp[1], vp[3], vp[4], vp[5]));
    q[5] = metric_conformity(mmul(M(neg(e53), e45, e25), *F), specified_metric(m, vp[2], vp[3], vp[4], vp[5]));
    return combine_corners(q, 6);
}

/* MetricConformityEvaluator::hexQuality (MetricConformityEvaluator.cpp:150-224) */
static double mc_hex(const om_mesh* m, const v3* vp)
{
    v3 e01 = sub(vp[1], vp[0]);
    v3 e03 = sub(vp[3], vp[0]);
    v3 e04 = sub(vp[4], vp[0]);
    v3 e12 = sub(vp[2], vp[1]);
    v3 e15 = sub(vp[5], vp[1]);
    v3 e23 = sub(vp[3], vp[2]);
    v3 e26 = sub(vp[6], vp[2]);
    v3 e37 = sub(vp[7], vp[3]);
    v3 e45 = sub(vp[5], vp[4]);
    v3 e47 = sub(vp[7], vp[4]);
    v3 e56 = sub(vp[6], vp[5]);
    v3 e67 = sub(vp[7], vp[6]);
    double q[8];
    q[0] = metric_conformity(M(e01, e04, neg(e03)), specified_metric(m, vp[0], vp[1], vp[3], vp[4]));
    q[1] = metric_conformity(M(e01, e12, e15), specified_metric(m, vp[0], vp[1], vp[2], vp[5]));
    q[2] = metric_conformity(M(e12, e26, neg(e23)), specified_metric(m, vp[1], vp[2], vp[3], vp[6]));
    q[3] = metric_conformity(M(e03, e23, e37), specified_metric(m, vp[0], vp[2], vp[3], vp[7]));
    q[4] = metric_conformity(M(e04, e45, e47), specified_metric(m, vp[0], vp[4], vp[5], vp[7]));
    q[5] = metric_conformity(M(e15, neg(e56), e45), specified_metric(m, vp[1], vp[4], vp[5], vp[6]));
    q[6] = metric_conformity(M(e26, e56, e67), specified_metric(m, vp[2], vp[5], vp[6], vp[7]));
    q[7] = metric_conformity(M(e37, e67, neg(e47)), specified_metric(m, vp[3], vp[4], vp[6], vp[7]));
    return combine_corners(q, 8);
}

static double quality_vp(const om_mesh* m, int type, const v3* vp)
{
    if (m->evaluator == OM_EVALUATOR_METRIC_CONFORMITY)
    {
        if (type == OM_TET) return mc_tet(m, vp);
        if (type == OM_PRI) return mc_pri(m, vp);
        if (type == OM_HEX) return mc_hex(m, vp);
    }
    else
    {
        if (type == OM_TET) return mr_tet(m, vp);
        if (type == OM_PRI) return mr_pri(m, vp);
        if (type == OM_HEX) return mr_hex(m, vp);
    }
    return 0.0;
}

static inline const uint32_t* elem_verts(const om_mesh* m, int type, int64_t idx, int* n)
{
    if (type == OM_TET) { *n = 4; return m->tets + 4 * idx; }
    if (type == OM_PRI) { *n = 6; return m->pris + 6 * idx; }
    *n = 8;
    return m->hexs + 8 * idx;
}

/* the element's sampler cache (its first background tet) for the measures
 * that follow; only the local sampler reads it */
static inline void use_elem_cache(const om_mesh* m, int type, int64_t idx)
{
    if (!m->ecache) return;
    int64_t off = type == OM_TET ? 0 : type == OM_PRI ? m->nt : m->nt + m->np;
    tl_cache = m->ecache[off + idx];
}

static double element_quality(const om_mesh* m, int type, int64_t idx)
{
    use_elem_cache(m, type, idx);
    int n;
    const uint32_t* e = elem_verts(m, type, idx, &n);
    v3 vp[8];
    for (int k = 0; k < n; ++k) vp[k] = P(m, e[k]);
    return quality_vp(m, type, vp);
}

double om_element_quality(const om_mesh* m, int32_t type, int64_t idx) { return element_quality(m, type, idx); }

#ifdef OM_PATCH_QUALITY_FP32
/* Measurement variant (libgm_oracle_q32.so), not the reference.  Every patch
 * quality the smoothers compare is brought to the resolution an FP32
 * implementation has, to measure how far the reference algorithm's result
 * depends on quality differences below that resolution:
 *   seed 0: the quality rounded to FP32;
 *   seed s > 0: the quality times (1 + u 2^-23), u uniform in [-1, 1] drawn
 *     from a counter hash of (s, vertex, the vertex's evaluation count in
 *     this relocation), so a draw does not depend on the thread count. */
static uint64_t fp32_noise_seed = 0;
static __thread uint32_t fp32_noise_vertex = 0xffffffffu;
static __thread uint64_t fp32_noise_count = 0;

void om_set_fp32_resolution_seed(uint64_t seed) { fp32_noise_seed = seed; }

static double fp32_resolution(double q, uint32_t v)
{
    if (!fp32_noise_seed) return (double)(float)q;
    if (v != fp32_noise_vertex)
    {
        fp32_noise_vertex = v;
        fp32_noise_count = 0;
    }
    uint64_t z = fp32_noise_seed * 0x9E3779B97F4A7C15ull ^ ((uint64_t)v << 20) ^ ++fp32_noise_count;
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    return q * (1.0 + u * (1.0 / 8388608.0));
}
#endif

/* AbstractEvaluator::patchQuality + accumulatePatchQuality +
 * finalizePatchQuality (Evaluators/AbstractEvaluator.cpp:236-279, 778-803) */
static double patch_quality(const om_mesh* m, uint32_t v)
{
    double weight = 0.0, quality = 0.0;
    for (int64_t n = m->ne_base[v]; n < m->ne_base[v + 1]; ++n)
    {
        const neig_elem* ne = &m->ne[n];
        double q = element_quality(m, ne->type, ne->id);
        if (weight != -1.0 && q > 0.0)
        {
            weight += 1.0;
            quality += 1 / q;
        }
        else
        {
            weight = -1.0;
            quality = gmin(quality, q);
        }
    }
    if (weight > 0.0) quality = weight / quality;
#ifdef OM_PATCH_QUALITY_FP32
    quality = fp32_resolution(quality, v);
#endif
    return quality;
}

double om_patch_quality(const om_mesh* m, int64_t v) { return patch_quality(m, (uint32_t)v); }

/* QualityHistogram::add (DataStructures/QualityHistogram.cpp:63-76).  The
 * reference's size_t(value*20) is undefined for negative values; it is
 * read here as bucket 0. */
typedef struct
{
    double mn, inv_sum, count;
    double buckets[OM_HIST_BUCKETS];
} hist;

static inline void hist_add(hist* h, double value)
{
    h->count += 1;
    h->mn = gmin(h->mn, value);
    if (value > 0.0) h->inv_sum += 1.0 / value;
    else h->inv_sum = INFINITY;
    double b = value * OM_HIST_BUCKETS;
    int64_t bi = (b > 0.0) ? (int64_t)b : 0;
    if (bi > OM_HIST_BUCKETS - 1) bi = OM_HIST_BUCKETS - 1;
    h->buckets[bi] += 1;
}

typedef struct
{
    const om_mesh* m;
    int t, nthreads;
    hist h;
} eval_job;

static void* eval_worker(void* arg)
{
    /* AbstractEvaluator::evaluateMeshQualityThread (AbstractEvaluator.cpp:404-453):
     * contiguous element ranges per worker, per-worker histograms merged in
     * worker order */
    eval_job* j = (eval_job*)arg;
    const om_mesh* m = j->m;
    int64_t T = j->nthreads, t = j->t;
    int64_t tb = (m->nt * t) / T, te = (m->nt * (t + 1)) / T;
    int64_t pb = (m->np * t) / T, pe = (m->np * (t + 1)) / T;
    int64_t hb = (m->nh * t) / T, he = (m->nh * (t + 1)) / T;
    for (int64_t i = tb; i < te; ++i) hist_add(&j->h, element_quality(m, OM_TET, i));
    for (int64_t i = pb; i < pe; ++i) hist_add(&j->h, element_quality(m, OM_PRI, i));
    for (int64_t i = hb; i < he; ++i) hist_add(&j->h, element_quality(m, OM_HEX, i));
    return NULL;
}

void om_evaluate(const om_mesh* m, double* out, int32_t nthreads)
{
    if (nthreads < 1) nthreads = 1;
    hist total;
    memset(&total, 0, sizeof(total));
    total.mn = 1.0;
    eval_job* jobs = (eval_job*)calloc((size_t)nthreads, sizeof(eval_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t)
    {
        jobs[t].m = m;
        jobs[t].t = t;
        jobs[t].nthreads = nthreads;
        jobs[t].h.mn = 1.0;
        if (nthreads == 1) eval_worker(&jobs[t]);
        else pthread_create(&th[t], NULL, eval_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t)
    {
        if (nthreads > 1) pthread_join(th[t], NULL);
        /* QualityHistogram::merge (QualityHistogram.cpp:78-92) */
        if (jobs[t].h.count == 0) continue;
        total.count += jobs[t].h.count;
        total.mn = gmin(total.mn, jobs[t].h.mn);
        total.inv_sum += jobs[t].h.inv_sum;
        for (int b = 0; b < OM_HIST_BUCKETS; ++b) total.buckets[b] += jobs[t].h.buckets[b];
    }
    out[0] = total.mn;
    out[1] = total.inv_sum;
    out[2] = total.count;
    for (int b = 0; b < OM_HIST_BUCKETS; ++b) out[3 + b] = total.buckets[b];
    free(jobs);
    free(th);
}

/* ------------------------------------------------------------------------ */
/* vertex-wise smoothers                                                     */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z, w; } v4;
static inline v4 V4(v3 p, double w) { v4 r = {p.x, p.y, p.z, w}; return r; }
static inline v3 xyz(v4 a) { return V(a.x, a.y, a.z); }
static inline void swap4(v4* a, v4* b) { v4 t = *a; *a = *b; *b = t; }

typedef struct
{
    double p[8];
} smooth_params;

/* evaluate the patch of v with the vertex at `at` (the reference writes the
 * trial position into verts[vId] and calls patchQuality) */
static inline double eval_at(om_mesh* m, uint32_t v, v3 at, int64_t* evals)
{
    setP(m, v, at);
    ++*evals;
    return patch_quality(m, v);
}

/* NelderMeadSmoother::smoothVertices (Smoothers/VertexWise/NelderMeadSmoother.cpp:100-260) */
static void nm_vertex(om_mesh* m, uint32_t vId, const smooth_params* sp, int64_t* evals)
{
    const double shiftFactor = sp->p[0];
    const int securityCycles = (int)sp->p[1];
    const double valueConvergence = sp->p[2];
    const double alpha = sp->p[3], beta = sp->p[4], gamma = sp->p[5];
    const int constrained = is_constrained(m, vId);

    double localSize = local_size(m, vId);
    double nodeShift = localSize * shiftFactor;

    v3 pos = P(m, vId);
    ++*evals;
    v4 vo = V4(pos, patch_quality(m, vId));
    v4 simplex[4] = {V4(add(pos, V(nodeShift, 0, 0)), 0), V4(add(pos, V(0, nodeShift, 0)), 0),
                     V4(add(pos, V(0, 0, nodeShift)), 0), vo};

    int cycle = 0;
    int reset = 0;
    int terminated = 0;
    while (!terminated)
    {
        for (int p = 0; p < 3; ++p)
        {
            pos = xyz(simplex[p]);
            if (constrained) pos = snap(m, vId, pos);
            simplex[p] = V4(pos, eval_at(m, vId, pos, evals));
        }

        if (simplex[0].w > simplex[1].w) swap4(&simplex[0], &simplex[1]);
        if (simplex[1].w > simplex[2].w) swap4(&simplex[1], &simplex[2]);
        if (simplex[2].w > simplex[3].w) swap4(&simplex[2], &simplex[3]);
        if (simplex[0].w > simplex[1].w) swap4(&simplex[0], &simplex[1]);
        if (simplex[1].w > simplex[2].w) swap4(&simplex[1], &simplex[2]);
        if (simplex[0].w > simplex[1].w) swap4(&simplex[0], &simplex[1]);

        for (; cycle < securityCycles; ++cycle)
        {
            v3 c = mul(add(add(xyz(simplex[1]), xyz(simplex[2])), xyz(simplex[3])), 1 / 3.0);
            double f = 0.0;

            pos = add(c, mul(sub(c, xyz(simplex[0])), alpha));
            if (constrained) pos = snap(m, vId, pos);
            double fr = f = eval_at(m, vId, pos, evals);
            v3 xr = pos;

            if (simplex[3].w < fr)
            {
                pos = add(c, mul(sub(pos, c), gamma));
                if (constrained) pos = snap(m, vId, pos);
                double fe = f = eval_at(m, vId, pos, evals);
                if (fe <= fr)
                {
                    pos = xr;
                    f = fr;
                }
            }
            else if (simplex[1].w >= fr)
            {
                if (fr > simplex[0].w)
                {
                    pos = add(c, mul(sub(xr, c), beta));
                    if (constrained) pos = snap(m, vId, pos);
                    f = eval_at(m, vId, pos, evals);
                }
                else
                {
                    pos = add(c, mul(sub(xyz(simplex[0]), c), beta));
                    if (constrained) pos = snap(m, vId, pos);
                    f = eval_at(m, vId, pos, evals);
                }
            }

            v4 vertex = V4(pos, f);
            if (vertex.w > simplex[3].w) swap4(&simplex[3], &vertex);
            if (vertex.w > simplex[2].w) swap4(&simplex[2], &vertex);
            if (vertex.w > simplex[1].w) swap4(&simplex[1], &vertex);
            if (vertex.w > simplex[0].w) swap4(&simplex[0], &vertex);

            if ((simplex[3].w - simplex[1].w) < valueConvergence)
            {
                terminated = 1;
                break;
            }
        }

        if (terminated || (cycle >= securityCycles && reset)) break;
        simplex[0] = V4(sub(xyz(vo), V(nodeShift, 0, 0)), vo.w);
        simplex[1] = V4(sub(xyz(vo), V(0, nodeShift, 0)), vo.w);
        simplex[2] = V4(sub(xyz(vo), V(0, 0, nodeShift)), vo.w);
        simplex[3] = vo;
        reset = 1;
        cycle = 0;
    }

    pos = xyz(simplex[3]);
    if (constrained) pos = snap(m, vId, pos);
    setP(m, vId, pos);
}

/* GradientDescentSmoother::smoothVertices (Smoothers/VertexWise/GradientDescentSmoother.cpp:73-202) */
static void gd_vertex(om_mesh* m, uint32_t vId, const smooth_params* sp, int64_t* evals)
{
    const double shiftFactor = sp->p[0];
    const int securityCycles = (int)sp->p[1];
    const int constrained = is_constrained(m, vId);
    static const double OFFSETS[8] = {-0.25, 0.00, 0.10, 0.20, 0.40, 0.80, 1.20, 1.60};

    double localSize = local_size(m, vId);
    double nodeShift = localSize * shiftFactor;
    double originalNodeShift = nodeShift;

    for (int c = 0; c < securityCycles; ++c)
    {
        v3 pos = P(m, vId);
        double q[6];
        v3 g[6] = {add(pos, V(-nodeShift, 0.0, 0.0)), add(pos, V(nodeShift, 0.0, 0.0)),
                   add(pos, V(0.0, -nodeShift, 0.0)), add(pos, V(0.0, nodeShift, 0.0)),
                   add(pos, V(0.0, 0.0, -nodeShift)), add(pos, V(0.0, 0.0, nodeShift))};
        if (constrained)
            for (int p = 0; p < 6; ++p) g[p] = snap(m, vId, g[p]);
        v3 originalPos = pos;
        for (int p = 0; p < 6; ++p) q[p] = eval_at(m, vId, g[p], evals);
        pos = originalPos;
        setP(m, vId, pos);

        v3 gradQ = V(q[1] - q[0], q[3] - q[2], q[5] - q[4]);
        double gradQNorm = length(gradQ);
        if (gradQNorm == 0) break;

        v3 shift = mul(gradQ, nodeShift / gradQNorm);
        v3 props[8];
        for (int p = 0; p < 8; ++p) props[p] = add(pos, mul(shift, OFFSETS[p]));
        if (constrained)
            for (int p = 0; p < 8; ++p) props[p] = snap(m, vId, props[p]);

        int best = 0;
        double bestQ = -INFINITY;
        for (int p = 0; p < 8; ++p)
        {
            double pq = eval_at(m, vId, props[p], evals);
            if (pq > bestQ)
            {
                bestQ = pq;
                best = p;
            }
        }
        setP(m, vId, props[best]);

        nodeShift *= fabs(OFFSETS[best]);
        if (nodeShift < originalNodeShift / 10.0) break;
    }
}

/* AbstractMeasurer::computeVertexEquilibrium.  Metric-free
 * (Measurers/MetricFreeMeasurer.cpp:107-152): pos plus the sum over the
 * incident elements of (p_i - pos) for every element vertex, over the sum of
 * (vertex count - 1).  Metric-wise (Measurers/MetricWiseMeasurer.cpp:190-255,
 * sumNode): every element vertex with d = p_i - pos != 0 adds weight
 * w = sqrt(n . M(p_i) n), n = d / |d|, and w d. */
static v3 vertex_equilibrium(const om_mesh* m, uint32_t v)
{
    const v3 pos = P(m, v);
    double totalWeight = 0.0;
    v3 displacement = V(0.0, 0.0, 0.0);
    for (int64_t i = m->ne_base[v]; i < m->ne_base[v + 1]; ++i)
    {
        int n;
        const uint32_t* ev = elem_verts(m, m->ne[i].type, m->ne[i].id, &n);
        if (m->measurer == OM_MEASURER_METRIC_WISE)
        {
            for (int k = 0; k < n; ++k)
            {
                const v3 p = P(m, ev[k]);
                const v3 d = sub(p, pos);
                if (d.x != 0.0 || d.y != 0.0 || d.z != 0.0)
                {
                    const v3 nn = normalize(d);
                    if (m->vcache) tl_cache = m->vcache[ev[k]]; /* sampler.metricAt(v.p, v.c) */
                    const m3 Mm = metric_at(m, p);
                    const double weight = sqrt(dot(nn, mmulv(Mm, nn)));
                    totalWeight += weight;
                    displacement = add(displacement, mul(d, weight));
                }
            }
        }
        else
        {
            totalWeight += n - 1;
            for (int k = 0; k < n; ++k) displacement = add(displacement, sub(P(m, ev[k]), pos));
        }
    }
    return add(pos, dvs(displacement, totalWeight));
}

/* SpringLaplaceSmoother::smoothVertices (Smoothers/VertexWise/
 * SpringLaplaceSmoother.cpp:51-78): pos = mix(pos, equilibrium, moveCoeff),
 * mix(x, y, a) = x + a (y - x), then the boundary projection */
static void spring_vertex(om_mesh* m, uint32_t vId, const smooth_params* sp)
{
    const double moveCoeff = sp->p[0];
    const v3 pos = P(m, vId);
    const v3 center = vertex_equilibrium(m, vId);
    v3 out = add(pos, mul(sub(center, pos), moveCoeff));
    if (is_constrained(m, vId)) out = snap(m, vId, out);
    setP(m, vId, out);
}

/* QualityLaplaceSmoother::smoothVertices (Smoothers/VertexWise/
 * QualityLaplaceSmoother.cpp:55-129): 8 propositions pos + shift * OFFSETS[p]
 * along shift = (equilibrium - pos) * moveCoeff, projected, the first best
 * patch quality kept */
static void qlaplace_vertex(om_mesh* m, uint32_t vId, const smooth_params* sp, int64_t* evals)
{
    static const double OFFSETS[8] = {-0.25, 0.00, 0.10, 0.20, 0.40, 0.80, 1.20, 1.60};
    const double moveCoeff = sp->p[0];
    const v3 pos = P(m, vId);
    const v3 center = vertex_equilibrium(m, vId);
    const v3 shift = mul(sub(center, pos), moveCoeff);
    v3 props[8];
    for (int p = 0; p < 8; ++p) props[p] = add(pos, mul(shift, OFFSETS[p]));
    if (is_constrained(m, vId))
        for (int p = 0; p < 8; ++p) props[p] = snap(m, vId, props[p]);
    int best = 0;
    double bestQ = -INFINITY;
    for (int p = 0; p < 8; ++p)
    {
        const double q = eval_at(m, vId, props[p], evals);
        if (q > bestQ)
        {
            bestQ = q;
            best = p;
        }
    }
    setP(m, vId, props[best]);
}

/* SpawnSearchSmoother offsets (SpawnSearchSmoother.cpp:33-55) and
 * smoothVertices (SpawnSearchSmoother.cpp:161-226) */
static v3 SPAWN_OFFSETS[64];
static pthread_once_t spawn_once = PTHREAD_ONCE_INIT;
static void spawn_init(void)
{
    int n = 0;
    for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 4; ++i) SPAWN_OFFSETS[n++] = sub(V(i, j, k), V(1.5, 1.5, 1.5));
    SPAWN_OFFSETS[0] = V(0, 0, 0);
}

static void spawn_vertex(om_mesh* m, uint32_t vId, const smooth_params* sp, int64_t* evals)
{
    pthread_once(&spawn_once, spawn_init);
    const double moveCoeff = sp->p[0];
    const int iterations = (int)sp->p[1];
    const int constrained = is_constrained(m, vId);
    double localSize = local_size(m, vId);
    double scale = moveCoeff * localSize;
    for (int iter = 0; iter < iterations; ++iter)
    {
        v3 pos = P(m, vId);
        v3 props[64];
        for (int p = 0; p < 64; ++p) props[p] = add(pos, mul(SPAWN_OFFSETS[p], scale));
        if (constrained)
            for (int p = 0; p < 64; ++p) props[p] = snap(m, vId, props[p]);
        int best = 0;
        double bestQ = -INFINITY;
        for (int p = 0; p < 64; ++p)
        {
            double pq = eval_at(m, vId, props[p], evals);
            if (pq > bestQ)
            {
                bestQ = pq;
                best = p;
            }
        }
        setP(m, vId, props[best]);
        scale /= 3.0;
    }
}

/* ------------------------------------------------------------------------ */
/* GETMe (element-wise)                                                      */
/* ------------------------------------------------------------------------ */

/* per (element, corner) transformed position and the element's weight */
typedef struct
{
    v3 p;
    double w;
} corner_out;

/* GetmeSmoother::smoothTets (Smoothers/ElementWise/GetmeSmoother.cpp:55-125) */
static void getme_tet(const om_mesh* m, int64_t eId, double lambda, corner_out* out)
{
    use_elem_cache(m, OM_TET, eId);
    const uint32_t* vi = m->tets + 4 * eId;
    v3 vp[4], vpp[4];
    for (int k = 0; k < 4; ++k) vp[k] = P(m, vi[k]);
    v3 n[4] = {cross(sub(vp[3], vp[1]), sub(vp[2], vp[1])), cross(sub(vp[3], vp[2]), sub(vp[0], vp[2])),
               cross(sub(vp[1], vp[3]), sub(vp[0], vp[3])), cross(sub(vp[1], vp[0]), sub(vp[2], vp[0]))};
    for (int k = 0; k < 4; ++k) vpp[k] = add(vp[k], mul(n[k], lambda / sqrt(length(n[k]))));
    double volume = tet_volume(m, vp);
    double volumePrime = tet_volume(m, vpp);
    double absVolumeRation = fabs(volume / volumePrime);
    double volumeVar = pow(absVolumeRation, 1.0 / 3.0);
    v3 center = mul(add(add(add(vp[0], vp[1]), vp[2]), vp[3]), 1.0 / 4.0);
    for (int k = 0; k < 4; ++k) vpp[k] = add(center, mul(sub(vpp[k], center), volumeVar));
    for (int k = 0; k < 4; ++k)
        if (is_constrained(m, vi[k])) vpp[k] = snap(m, vi[k], vpp[k]);
    double quality = quality_vp(m, OM_TET, vp);
    double qualityPrime = quality_vp(m, OM_TET, vpp);
    double weight = qualityPrime / (1.0 + quality);
    for (int k = 0; k < 4; ++k)
    {
        out[k].p = vpp[k];
        out[k].w = weight;
    }
}

/* GetmeSmoother::smoothPris (GetmeSmoother.cpp:127-233) */
static void getme_pri(const om_mesh* m, int64_t eId, double lambda, corner_out* out)
{
    use_elem_cache(m, OM_PRI, eId);
    const uint32_t* vi = m->pris + 6 * eId;
    v3 vp[6], vpp[6];
    for (int k = 0; k < 6; ++k) vp[k] = P(m, vi[k]);
    v3 aux[5] = {dvs(add(add(vp[0], vp[1]), vp[2]), 3.0),
                 dvs(add(add(add(vp[0], vp[1]), vp[4]), vp[3]), 4.0),
                 dvs(add(add(add(vp[1], vp[2]), vp[5]), vp[4]), 4.0),
                 dvs(add(add(add(vp[2], vp[0]), vp[3]), vp[5]), 4.0),
                 dvs(add(add(vp[3], vp[4]), vp[5]), 3.0)};
    v3 n[6] = {cross(sub(aux[1], aux[0]), sub(aux[3], aux[0])), cross(sub(aux[2], aux[0]), sub(aux[1], aux[0])),
               cross(sub(aux[3], aux[0]), sub(aux[2], aux[0])), cross(sub(aux[3], aux[4]), sub(aux[1], aux[4])),
               cross(sub(aux[1], aux[4]), sub(aux[2], aux[4])), cross(sub(aux[2], aux[4]), sub(aux[3], aux[4]))};
    double t = (4.0 / 5.0) * (1.0 - pow(4.0 / 39.0, 0.25) * lambda);
    double it = 1.0 - t;
    v3 bases[6] = {add(mul(aux[0], it), dvs(mul(add(aux[3], aux[1]), t), 2.0)),
                   add(mul(aux[0], it), dvs(mul(add(aux[1], aux[2]), t), 2.0)),
                   add(mul(aux[0], it), dvs(mul(add(aux[2], aux[3]), t), 2.0)),
                   add(mul(aux[4], it), dvs(mul(add(aux[3], aux[1]), t), 2.0)),
                   add(mul(aux[4], it), dvs(mul(add(aux[1], aux[2]), t), 2.0)),
                   add(mul(aux[4], it), dvs(mul(add(aux[2], aux[3]), t), 2.0))};
    for (int k = 0; k < 6; ++k) vpp[k] = add(bases[k], mul(n[k], lambda / sqrt(length(n[k]))));
    double volume = pri_volume(m, vp);
    double volumePrime = pri_volume(m, vpp);
    double volumeVar = pow(fabs(volume / volumePrime), 1.0 / 3.0);
    v3 center = mul(add(add(add(add(add(vp[0], vp[1]), vp[2]), vp[3]), vp[4]), vp[5]), 1.0 / 6.0);
    for (int k = 0; k < 6; ++k) vpp[k] = add(center, mul(sub(vpp[k], center), volumeVar));
    for (int k = 0; k < 6; ++k)
        if (is_constrained(m, vi[k])) vpp[k] = snap(m, vi[k], vpp[k]);
    double quality = quality_vp(m, OM_PRI, vp);
    double qualityPrime = quality_vp(m, OM_PRI, vpp);
    double weight = qualityPrime / (1.0 + quality);
    for (int k = 0; k < 6; ++k)
    {
        out[k].p = vpp[k];
        out[k].w = weight;
    }
}

/* GetmeSmoother::smoothHexs (GetmeSmoother.cpp:235-374) */
static void getme_hex(const om_mesh* m, int64_t eId, double lambda, corner_out* out)
{
    use_elem_cache(m, OM_HEX, eId);
    const uint32_t* vi = m->hexs + 8 * eId;
    v3 vp[8], vpp[8];
    for (int k = 0; k < 8; ++k) vp[k] = P(m, vi[k]);
    v3 aux[6] = {dvs(add(add(add(vp[0], vp[1]), vp[2]), vp[3]), 4.0),
                 dvs(add(add(add(vp[0], vp[4]), vp[5]), vp[1]), 4.0),
                 dvs(add(add(add(vp[1], vp[5]), vp[6]), vp[2]), 4.0),
                 dvs(add(add(add(vp[2], vp[6]), vp[7]), vp[3]), 4.0),
                 dvs(add(add(add(vp[0], vp[3]), vp[7]), vp[4]), 4.0),
                 dvs(add(add(add(vp[4], vp[7]), vp[6]), vp[5]), 4.0)};
    v3 n[8] = {cross(sub(aux[1], aux[0]), sub(aux[4], aux[0])), cross(sub(aux[2], aux[0]), sub(aux[1], aux[0])),
               cross(sub(aux[3], aux[0]), sub(aux[2], aux[0])), cross(sub(aux[4], aux[0]), sub(aux[3], aux[0])),
               cross(sub(aux[4], aux[5]), sub(aux[1], aux[5])), cross(sub(aux[1], aux[5]), sub(aux[2], aux[5])),
               cross(sub(aux[2], aux[5]), sub(aux[3], aux[5])), cross(sub(aux[3], aux[5]), sub(aux[4], aux[5]))};
    v3 bases[8] = {dvs(add(add(aux[0], aux[1]), aux[4]), 3.0), dvs(add(add(aux[0], aux[2]), aux[1]), 3.0),
                   dvs(add(add(aux[0], aux[3]), aux[2]), 3.0), dvs(add(add(aux[0], aux[4]), aux[3]), 3.0),
                   dvs(add(add(aux[5], aux[4]), aux[1]), 3.0), dvs(add(add(aux[5], aux[1]), aux[2]), 3.0),
                   dvs(add(add(aux[5], aux[2]), aux[3]), 3.0), dvs(add(add(aux[5], aux[3]), aux[4]), 3.0)};
    for (int k = 0; k < 8; ++k) vpp[k] = add(bases[k], mul(n[k], lambda / sqrt(length(n[k]))));
    double volume = hex_volume(m, vp);
    double volumePrime = hex_volume(m, vpp);
    double volumeVar = pow(fabs(volume / volumePrime), 1.0 / 3.0);
    v3 center = mul(add(add(add(add(add(add(add(vp[0], vp[1]), vp[2]), vp[3]), vp[4]), vp[5]), vp[6]), vp[7]),
                    1.0 / 8.0);
    for (int k = 0; k < 8; ++k) vpp[k] = add(center, mul(sub(vpp[k], center), volumeVar));
    for (int k = 0; k < 8; ++k)
        if (is_constrained(m, vi[k])) vpp[k] = snap(m, vi[k], vpp[k]);
    double quality = quality_vp(m, OM_HEX, vp);
    double qualityPrime = quality_vp(m, OM_HEX, vpp);
    double weight = qualityPrime / (1.0 + quality);
    for (int k = 0; k < 8; ++k)
    {
        out[k].p = vpp[k];
        out[k].w = weight;
    }
}

/* AbstractElementWiseSmoother::updateVertexPositions
 * (Smoothers/ElementWise/AbstractElementWiseSmoother.cpp:406-444), with the
 * vertex accumulator (VertexAccum.cpp: NotThreadSafeVertexAccum) summed in
 * element order, which is the vertex's neighbour-element order */
static void getme_update_vertex(om_mesh* m, uint32_t vId, const int64_t* corner_base,
                                const corner_out* corners, int64_t* evals)
{
    v3 posAccum = V(0, 0, 0);
    double weightAccum = 0.0;
    for (int64_t n = m->ne_base[vId]; n < m->ne_base[vId + 1]; ++n)
    {
        const neig_elem* ne = &m->ne[n];
        const corner_out* c = &corners[corner_base[ne->type] + (int64_t)ne->id *
                                       (ne->type == OM_TET ? 4 : ne->type == OM_PRI ? 6 : 8) + ne->vid];
        posAccum = add(posAccum, mul(c->p, c->w));
        weightAccum += c->w;
    }
    v3 pos = P(m, vId);
    if (weightAccum != 0.0)
    {
        v3 posPrim = dvs(posAccum, weightAccum);
        if (is_constrained(m, vId)) posPrim = snap(m, vId, posPrim);
        ++*evals;
        double patchQuality = patch_quality(m, vId);
        setP(m, vId, posPrim);
        ++*evals;
        double patchQualityPrime = patch_quality(m, vId);
        if (patchQualityPrime < patchQuality) setP(m, vId, pos);
    }
}

/* ------------------------------------------------------------------------ */
/* pass driver: colour-major groups, strided worker slices and a barrier per */
/* colour, as AbstractVertexWiseSmoother::smoothMeshThread                    */
/* (Smoothers/VertexWise/AbstractVertexWiseSmoother.cpp:84-152) and          */
/* NodeGroups::dispatchCpuWorkgroups (DataStructures/NodeGroups.cpp:621-659)  */
/* ------------------------------------------------------------------------ */

typedef struct
{
    om_mesh* m;
    int32_t smoother;
    smooth_params sp;
    int64_t ngroups;
    const int64_t* group_base;
    const uint32_t* members;
    int nthreads;
    pthread_barrier_t* barrier;
    /* GETMe */
    const int64_t* corner_base;
    corner_out* corners;
    int64_t evals[64];
} pass_ctx;

typedef struct
{
    pass_ctx* ctx;
    int t;
} pass_arg;

static void* pass_worker(void* arg)
{
    pass_arg* a = (pass_arg*)arg;
    pass_ctx* c = a->ctx;
    int t = a->t, T = c->nthreads;
    int64_t evals = 0;

    if (c->smoother == OM_SMOOTH_GETME)
    {
        /* element pass: every element reads the positions at pass start
         * (GetmeSmoother::smoothTets/Pris/Hexs run before any update) */
        om_mesh* m = c->m;
        double lambda = c->sp.p[0];
        for (int64_t i = t; i < m->nt; i += T) getme_tet(m, i, lambda, c->corners + c->corner_base[OM_TET] + 4 * i);
        for (int64_t i = t; i < m->np; i += T) getme_pri(m, i, lambda, c->corners + c->corner_base[OM_PRI] + 6 * i);
        for (int64_t i = t; i < m->nh; i += T) getme_hex(m, i, lambda, c->corners + c->corner_base[OM_HEX] + 8 * i);
        if (T > 1) pthread_barrier_wait(c->barrier);
    }

    for (int64_t g = 0; g < c->ngroups; ++g)
    {
        int64_t b = c->group_base[g], e = c->group_base[g + 1];
        for (int64_t i = b + t; i < e; i += T)
        {
            uint32_t v = c->members[i];
            switch (c->smoother)
            {
            case OM_SMOOTH_NELDER_MEAD: nm_vertex(c->m, v, &c->sp, &evals); break;
            case OM_SMOOTH_GRADIENT_DESCENT: gd_vertex(c->m, v, &c->sp, &evals); break;
            case OM_SMOOTH_SPAWN_SEARCH: spawn_vertex(c->m, v, &c->sp, &evals); break;
            case OM_SMOOTH_GETME: getme_update_vertex(c->m, v, c->corner_base, c->corners, &evals); break;
            case OM_SMOOTH_SPRING_LAPLACE: spring_vertex(c->m, v, &c->sp); break;
            case OM_SMOOTH_QUALITY_LAPLACE: qlaplace_vertex(c->m, v, &c->sp, &evals); break;
            default: break;
            }
        }
        if (T > 1) pthread_barrier_wait(c->barrier);
    }
    c->evals[t] = evals;
    return NULL;
}

void om_smooth_pass(om_mesh* m, int32_t smoother, const double* params, int64_t ngroups,
                    const int64_t* group_base, const uint32_t* members, int32_t nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    pass_ctx c;
    memset(&c, 0, sizeof(c));
    c.m = m;
    c.smoother = smoother;
    memcpy(c.sp.p, params, sizeof(c.sp.p));
    c.ngroups = ngroups;
    c.group_base = group_base;
    c.members = members;
    c.nthreads = nthreads;
    int64_t corner_base[4] = {0, 0, 4 * m->nt, 4 * m->nt + 6 * m->np};
    if (smoother == OM_SMOOTH_GETME)
    {
        c.corner_base = corner_base;
        c.corners = (corner_out*)malloc(sizeof(corner_out) * (size_t)(4 * m->nt + 6 * m->np + 8 * m->nh + 1));
    }
    pthread_barrier_t barrier;
    if (nthreads > 1) pthread_barrier_init(&barrier, NULL, (unsigned)nthreads);
    c.barrier = &barrier;
    pass_arg args[64];
    pthread_t th[64];
    for (int t = 0; t < nthreads; ++t)
    {
        args[t].ctx = &c;
        args[t].t = t;
        if (nthreads == 1) pass_worker(&args[t]);
        else pthread_create(&th[t], NULL, pass_worker, &args[t]);
    }
    if (nthreads > 1)
    {
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
        pthread_barrier_destroy(&barrier);
    }
    for (int t = 0; t < nthreads; ++t) m->patch_evals += c.evals[t];
    free(c.corners);
}

/* ------------------------------------------------------------------------ */
/* NodeGroups::build (DataStructures/NodeGroups.cpp:104-122): vertex classes,  */
/* the breadth-first greedy colouring, the (class, colour, valence) order and  */
/* the colour-major groups of the permuted mesh                               */
/* ------------------------------------------------------------------------ */

/* the std::sort call of NodeGroups::determinePositions (om_sort.cpp) */
void om_sort_node_order(int64_t n, const int* types, const int* groups, const int64_t* valence, int* out);

#define OM_FIXED_TYPE 0
#define OM_BOUND_TYPE 1
#define OM_SUBSU_TYPE 2
#define OM_INTER_TYPE 3
#define OM_NO_GROUP (-2)
#define OM_UNSET_GROUP (-1)

/* NodeGroups::isMovableBound (NodeGroups.cpp:695-704): constrained, not fixed */
static inline int movable_bound(const om_mesh* m, uint32_t v) { return m->cid[v] != 0 && !(m->cid[v] < 0); }

/* NodeGroups::determineTypes (NodeGroups.cpp:124-241) */
static void ng_types(const om_mesh* m, int* types)
{
    char* btet = (char*)calloc((size_t)m->nt + 1, 1);
    char* bpri = (char*)calloc((size_t)m->np + 1, 1);
    char* bhex = (char*)calloc((size_t)m->nh + 1, 1);
    for (int64_t e = 0; e < m->nt; ++e)
        for (int k = 0; k < 4; ++k)
            if (movable_bound(m, m->tets[4 * e + k])) btet[e] = 1;
    for (int64_t e = 0; e < m->np; ++e)
        for (int k = 0; k < 6; ++k)
            if (movable_bound(m, m->pris[6 * e + k])) bpri[e] = 1;
    for (int64_t e = 0; e < m->nh; ++e)
        for (int k = 0; k < 8; ++k)
            if (movable_bound(m, m->hexs[8 * e + k])) bhex[e] = 1;
    for (int64_t v = 0; v < m->nv; ++v)
    {
        if (m->cid[v] < 0) types[v] = OM_FIXED_TYPE;           /* isFixed */
        else if (m->cid[v] != 0) types[v] = OM_BOUND_TYPE;     /* isConstrained */
        else
        {
            int sub = 0;
            for (int64_t j = m->ne_base[v]; j < m->ne_base[v + 1] && !sub; ++j)
            {
                const neig_elem* ne = &m->ne[j];
                sub = (ne->type == OM_TET && btet[ne->id]) || (ne->type == OM_PRI && bpri[ne->id]) ||
                      (ne->type == OM_HEX && bhex[ne->id]);
            }
            types[v] = sub ? OM_SUBSU_TYPE : OM_INTER_TYPE;
        }
    }
    free(btet);
    free(bpri);
    free(bhex);
}

/* NodeGroups::determineGroups (NodeGroups.cpp:243-363).  The reference takes
 * the first element of a copy of the existing colours {0 .. G-1} from which
 * the already coloured neighbours' colours are erased (or a new colour G when
 * none is left); here the neighbours' colours are stamped in `seen` and the
 * lowest unstamped colour below G is taken, which is the same choice. */
static void ng_groups(const om_mesh* m, int* groups)
{
    const int64_t nv = m->nv;
    for (int64_t v = 0; v < nv; ++v) groups[v] = OM_NO_GROUP;
    int64_t* next = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1));
    int64_t* seen = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1)); /* colour -> last stamp */
    int64_t nnext = 0, seek = 0, existing = 0;
    while (nnext < nv)
    {
        int64_t first = nnext;
        for (int64_t v = seek; v < nv; ++v)
        {
            ++seek;
            if (groups[v] == OM_NO_GROUP)
            {
                groups[v] = OM_UNSET_GROUP;
                next[nnext++] = v;
                break;
            }
        }
        for (int64_t q = first; q < nnext; ++q)
        {
            const int64_t vId = next[q];
            for (int64_t j = m->ne_base[vId]; j < m->ne_base[vId + 1]; ++j)
            {
                int n;
                const uint32_t* el = elem_verts(m, m->ne[j].type, m->ne[j].id, &n);
                for (int k = 0; k < n; ++k)
                {
                    int* g = &groups[el[k]];
                    if (*g == OM_NO_GROUP)
                    {
                        *g = OM_UNSET_GROUP;
                        next[nnext++] = el[k];
                    }
                    else if (*g != OM_UNSET_GROUP)
                        seen[*g] = vId;
                }
            }
            int group = (int)existing;
            for (int64_t c = 0; c < existing; ++c)
                if (seen[c] != vId)
                {
                    group = (int)c;
                    break;
                }
            if (group == existing)
            {
                seen[existing] = -1;
                ++existing;
            }
            groups[vId] = group;
        }
    }
    free(next);
    free(seen);
}

int64_t om_node_groups_build(const om_mesh* m, uint32_t* perm, int64_t* group_base, uint32_t* members,
                             int64_t* ranges)
{
    const int64_t nv = m->nv;
    int* types = (int*)malloc(sizeof(int) * (size_t)(nv + 1));
    int* groups = (int*)malloc(sizeof(int) * (size_t)(nv + 1));
    int64_t* valence = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1));
    int* indices = (int*)malloc(sizeof(int) * (size_t)(nv + 1));
    ng_types(m, types);
    ng_groups(m, groups);
    /* NodeGroups::determinePositions (NodeGroups.cpp:365-450): sort by class,
     * then colour, then the number of neighbour elements */
    for (int64_t v = 0; v < nv; ++v) valence[v] = m->ne_base[v + 1] - m->ne_base[v];
    om_sort_node_order(nv, types, groups, valence, indices);

    /* NodeGroups::clusterNodes (NodeGroups.cpp:452-619): vertex vId of the
     * permuted mesh is input vertex indices[vId]; every movable vertex joins
     * its colour's undispatched list, and the first vertex of a (class,
     * colour) run opens that class's range of the colour */
    int64_t ngroups = 0;
    for (int64_t v = 0; v < nv; ++v)
        if (types[v] != OM_FIXED_TYPE && groups[v] + 1 > ngroups) ngroups = groups[v] + 1;
    int64_t* count = (int64_t*)calloc((size_t)ngroups + 1, sizeof(int64_t));
    memset(ranges, 0, sizeof(int64_t) * 6 * (size_t)ngroups);
    int last_type = -1, last_group = -1;
    for (int64_t vId = 0; vId < nv; ++vId)
    {
        const int old = indices[vId];
        perm[vId] = (uint32_t)old;
        const int type = types[old];
        if (type != last_type)
        {
            last_type = type;
            last_group = -1;
        }
        if (type == OM_FIXED_TYPE) continue;
        const int g = groups[old];
        int64_t* r = ranges + 6 * (int64_t)g + 2 * (type - 1);
        if (g != last_group)
        {
            last_group = g;
            r[0] = r[1] = vId;
        }
        ++r[1];
        ++count[g];
    }
    group_base[0] = 0;
    for (int64_t g = 0; g < ngroups; ++g) group_base[g + 1] = group_base[g] + count[g];
    memset(count, 0, sizeof(int64_t) * (size_t)(ngroups + 1));
    for (int64_t vId = 0; vId < nv; ++vId)
    {
        const int old = indices[vId];
        if (types[old] == OM_FIXED_TYPE) continue;
        const int g = groups[old];
        members[group_base[g] + count[g]++] = (uint32_t)vId;
    }
    free(count);
    free(types);
    free(groups);
    free(valence);
    free(indices);
    return ngroups;
}
