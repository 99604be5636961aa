/*
 * gm_oracle.h -- FP64 CPU restatement of GpuMesh's relocation smoothers and
 * quality evaluators.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm may load it.  Nothing in the product package calls it.
 *
 * Every function restates the reference C++ (cited file:line, paths relative
 * to the GpuMesh project root) in plain C, FP64, in the same expression
 * order as the GLM calls it replaces, compiled with -ffp-contract=off so that
 * x86 and aarch64 builds round identically.
 */
#ifndef GM_ORACLE_H
#define GM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element type codes: MeshTet/MeshPyr/MeshPri/MeshHex::ELEMENT_TYPE
 * (DataStructures/Mesh.h:89,130,171,213) */
#define OM_TET 0
#define OM_PYR 1
#define OM_PRI 2
#define OM_HEX 3

/* samplers (Samplers/UniformSampler.cpp:45, Samplers/AbstractSampler.cpp:190,
 * and the sine-graded anisotropic metric added as a new sampler plugin) */
#define OM_SAMPLER_UNIFORM 0
#define OM_SAMPLER_ANALYTIC 1
#define OM_SAMPLER_SINE 2
#define OM_SAMPLER_LOCAL 3 /* LocalSampler: the analytic metric on a background copy of the mesh */
#define OM_SAMPLER_KDTREE 4 /* KdTreeSampler: the local metric sampled once per kd-tree leaf */
#define OM_SAMPLER_TEXTURE 5 /* TextureSampler: the local metric sampled on a grid, trilinear */

#define OM_MEASURER_METRIC_FREE 0
#define OM_MEASURER_METRIC_WISE 1

#define OM_EVALUATOR_MEAN_RATIO 0
#define OM_EVALUATOR_METRIC_CONFORMITY 1

/* constraint kinds (Boundaries/Constraints) */
#define OM_CON_VOLUME 0  /* identity, VolumeConstraint.cpp:47 */
#define OM_CON_PLANE 1   /* PlaneConstraint, FaceConstraint.cpp:180 */
#define OM_CON_SEGMENT 2 /* SegmentConstraint, EdgeConstraint.cpp:185 */
#define OM_CON_SPHERE 3  /* SphereBoundary::Face, SphereBoundary.cpp:42 */
#define OM_CON_POINT 4   /* VertexConstraint, VertexConstraint.cpp:60 */
#define OM_CON_SHELL_INNER 5   /* ShellBoundary::InFace, ShellBoundary.cpp:41-44 */
#define OM_CON_PIPE_CYLINDER 6 /* PipeBoundary::CylinderFace, PipeBoundary.cpp:42-56 */
#define OM_CON_PIPE_CIRCLE 7   /* PipeBoundary::Y*CircleEdge, PipeBoundary.cpp:95-116 */

/* smoothers */
#define OM_SMOOTH_NELDER_MEAD 0
#define OM_SMOOTH_GRADIENT_DESCENT 1
#define OM_SMOOTH_SPAWN_SEARCH 2
#define OM_SMOOTH_GETME 3
#define OM_SMOOTH_SPRING_LAPLACE 4
#define OM_SMOOTH_QUALITY_LAPLACE 5

#define OM_HIST_BUCKETS 20

typedef struct om_mesh om_mesh;

om_mesh* om_create(int64_t nv, const double* pos, int64_t nt,
                   const uint32_t* tets, int64_t np, const uint32_t* pris,
                   int64_t nh, const uint32_t* hexs, const int32_t* cid);
void om_destroy(om_mesh* m);

/* constraint table indexed by constraint id (id 0 = volume). params: 6 per
 * id (plane: point, normal; segment: a, b; point: position). */
void om_set_constraints(om_mesh* m, int32_t n, const int32_t* kind,
                        const double* params);
/* AbstractSampler::setDiscretizationDepth (Samplers/AbstractSampler.cpp:61-64):
 * the kd-tree height / texture resolution; -1 (the default) picks it from the
 * vertex count.  Takes effect at the next om_set_crew. */
void om_set_discretization_depth(om_mesh* m, int32_t depth);
void om_set_crew(om_mesh* m, int32_t sampler, int32_t measurer,
                 int32_t evaluator, double scaling, double aspect_ratio);

void om_get_pos(const om_mesh* m, double* out);
void om_set_pos(om_mesh* m, const double* in);

double om_element_quality(const om_mesh* m, int32_t type, int64_t idx);
double om_patch_quality(const om_mesh* m, int64_t v);
double om_local_size(const om_mesh* m, int64_t v);
void om_project(const om_mesh* m, int64_t v, const double* in, double* out);
void om_metric_at(const om_mesh* m, const double* p, double* out9);
double om_riemannian_distance(const om_mesh* m, const double* a,
                              const double* b);

/* out: [min, inv_sum, count, bucket0..bucket19] */
void om_evaluate(const om_mesh* m, double* out, int32_t nthreads);

/* One relocation pass in colour-major order over the given independent
 * groups: group g is members[group_base[g] .. group_base[g+1]).
 * params (8 doubles) depend on the smoother:
 *   NM:    [node_shift_factor, security_cycles, value_convergence, alpha,
 *           beta, gamma]
 *   GD:    [node_shift_factor, security_cycles]
 *   spawn: [move_coeff, iterations]
 *   GETMe: [lambda]
 *   spring / quality Laplace: [move_coeff]
 */
void om_smooth_pass(om_mesh* m, int32_t smoother, const double* params,
                    int64_t ngroups, const int64_t* group_base,
                    const uint32_t* members, int32_t nthreads);

/* NodeGroups::build (DataStructures/NodeGroups.cpp:104-122) on the mesh as
 * given: perm[new] = input vertex (nv), the colour-major groups of the
 * permuted mesh -- group g is members[group_base[g] .. group_base[g+1]) --
 * and per group the boundary / subsurface / interior ranges (6 per group).
 * Capacities: group_base nv + 1, members nv, ranges 6 nv.  Returns the
 * number of groups. */
int64_t om_node_groups_build(const om_mesh* m, uint32_t* perm, int64_t* group_base, uint32_t* members,
                             int64_t* ranges);

/* Only in the measurement build libgm_oracle_q32.so (OM_PATCH_QUALITY_FP32):
 * 0 rounds every patch quality to FP32, s > 0 multiplies it by a seeded
 * draw of (1 + u 2^-23), |u| <= 1 (gm_oracle.c, fp32_resolution). */
void om_set_fp32_resolution_seed(uint64_t seed);

/* patch-evaluation counter (number of patchQuality calls since the last
 * reset), used for the FLOP accounting of the relocation roofline */
int64_t om_patch_eval_count(const om_mesh* m);
void om_reset_patch_eval_count(om_mesh* m);

#ifdef __cplusplus
}
#endif

#endif
