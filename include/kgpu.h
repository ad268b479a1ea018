/*
 * kgpu.h — C ABI of the GB300 configuration-validity and proximity engine.
 *
 * This is the drop-in boundary for Klamp't's hot path: forward kinematics of
 * a robot at configurations q, robot-vs-environment and robot self-collision
 * over triangle-mesh BVHs, planner edge checks, and signed distance with its
 * gradient.  Every entry point is `extern "C"`, takes plain pointers and
 * sizes, returns a status code and never lets a C++ exception cross.  Query
 * entry points take caller-owned DEVICE buffers and a CUDA stream and are
 * asynchronous on that stream; the `_host` variants take host buffers and
 * return when the results are in them.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the Klamp't source tree).  The reference reaches these through
 * KrisLibrary (UpdateFrames / AnyCollisionQuery / EpsilonEdgeChecker), which
 * is not part of the Klamp't tree; the call sites cited below are where
 * Klamp't binds them.
 *
 * Conventions
 *   - Rigid transforms are 12 doubles (or floats): rotation row-major R[3*r+c]
 *     then translation t.  (Klamp't's Python so3/se3 lists are column-major;
 *     the Python layer converts.)
 *   - A robot has one DOF per link, as a Klamp't RobotModel does: q has
 *     num_links entries.
 *   - Environment objects carry a group id.  Group 0 holds rigid objects and
 *     group 1 terrains; others are free for the caller.  Each link has a
 *     32-bit mask of the groups it is checked against.
 */
#ifndef KGPU_H
#define KGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (Python/klampt/src/robotsim.i:41-53 maps the reference's
 *      PyException to RuntimeError; these codes are what the Python layer
 *      maps the same way) ---------------------------------------------------- */
typedef int32_t kgpu_status;
#define KGPU_OK 0
#define KGPU_ERR_INVALID 1     /* bad argument: null handle, size, index        */
#define KGPU_ERR_CUDA 2        /* a CUDA runtime call failed                     */
#define KGPU_ERR_OOM 3         /* device or pinned allocation failed             */
#define KGPU_ERR_OVERFLOW 4    /* traversal stack spill area exhausted           */
#define KGPU_ERR_TIMEOUT 5     /* a bounded device-side wait ran out             */
#define KGPU_ERR_NOT_FINITE 6  /* NaN/Inf (or |q| >= 1e6) in a configuration     */
#define KGPU_ERR_EMPTY 7       /* query on empty geometry (robotsim.cpp:1786-1787) */
#define KGPU_ERR_UNSUPPORTED 8 /* feature not available for this input           */

#define KGPU_GROUP_RIGID_OBJECT 0
#define KGPU_GROUP_TERRAIN 1

#define KGPU_JOINT_REVOLUTE 0
#define KGPU_JOINT_PRISMATIC 1
#define KGPU_JOINT_WELD 2

#define KGPU_MAX_LINKS 32

typedef struct kgpu_robot_s* kgpu_robot;
typedef struct kgpu_env_s* kgpu_env;
typedef struct kgpu_world_s* kgpu_world;
typedef struct kgpu_edge_plan_s* kgpu_edge_plan;
typedef struct kgpu_config_plan_s* kgpu_config_plan;
typedef void* kgpu_stream; /* cudaStream_t; NULL selects the legacy default stream */

/* Robot model: links in topological order (parent index < link index, -1 =
 * attached to the world), Cpp/docs/Manual-Modeling.md:59,107.  Replaces the
 * model that Klampt::RobotModel::LoadRob builds (Cpp/Modeling/Robot.cpp:216,
 * T0_Parent/axes/types at :961-973, geommargin :1048-1051, self-collision
 * pairs :1275-1380). */
typedef struct {
  int32_t num_links;          /* 1..KGPU_MAX_LINKS                              */
  const int32_t* parents;     /* [num_links]                                    */
  const int32_t* joint_types; /* [num_links] KGPU_JOINT_*                       */
  const double* T0_parent;    /* [num_links*12] link frame in parent frame      */
  const double* axes;         /* [num_links*3] unit joint axis (link frame)     */
  const double* qmin;         /* [num_links]                                    */
  const double* qmax;         /* [num_links]                                    */
  const int32_t* vert_offset; /* [num_links+1] into verts (vertex units)        */
  const double* verts;        /* link-local vertex coordinates, 3 per vertex    */
  const int32_t* tri_offset;  /* [num_links+1] into tris (triangle units)       */
  const int32_t* tris;        /* 3 vertex indices per triangle, local to link   */
  const double* margins;     /* [num_links] collision margin, or NULL (= 0)     */
  const uint8_t* self_mask;  /* [num_links*num_links], entry [i*n+j] (i<j) != 0
                                enables pair (i,j); NULL = every pair except
                                link-parent (Cpp/docs/Manual-FileTypes.md:212) */
} kgpu_robot_desc;

/* Static environment: rigid objects and terrains, vertices in world frame.
 * Replaces the geometry that WorldModel::InitCollisions hands to the
 * collision queries (Cpp/Modeling/World.cpp:266-274). */
typedef struct {
  int32_t num_objects;
  const int32_t* vert_offset; /* [num_objects+1] */
  const double* verts;        /* world-frame coordinates */
  const int32_t* tri_offset;  /* [num_objects+1] */
  const int32_t* tris;        /* per-object vertex indices */
  const int32_t* groups;      /* [num_objects] in 0..31, or NULL (= 0) */
  const uint8_t* convex;      /* [num_objects] 1 = closed convex mesh (enables
                                 signed distance), or NULL (= none) */
  const double* margins;      /* [num_objects] or NULL (= 0) */
} kgpu_env_desc;

typedef struct {
  uint64_t items;          /* configurations (or edge steps) examined          */
  uint64_t node_pairs;     /* BVH node pairs tested in FP32                     */
  uint64_t tri_pairs;      /* triangle pairs tested in FP32                     */
  uint64_t band_pairs;     /* triangle pairs re-tested in FP64                  */
  uint64_t spills;         /* traversal stack spills to global memory           */
  uint64_t certified;      /* contacts certified in FP32 (no FP64 needed)       */
  uint64_t fp64_hits;      /* contacts confirmed by the FP64 re-test            */
  uint64_t dist_pairs;     /* (link, object) pairs evaluated by distance queries */
  uint64_t dist_node_pairs;/* BVH node pairs tested by distance queries          */
  uint64_t dist_tri_pairs; /* triangle pairs evaluated in FP32 by distance queries */
  uint64_t dist_fp64;      /* triangle pairs finalised in FP64                     */
} kgpu_stats;

/* ---- model construction --------------------------------------------------- */

/* Builds link BVHs on the host and uploads them.  Replaces RobotModel
 * construction + InitCollisions for the robot's links
 * (Python/klampt/src/robotsim.cpp:4118-4165). */
kgpu_status kgpu_robot_create(const kgpu_robot_desc* desc, kgpu_robot* out);
kgpu_status kgpu_robot_destroy(kgpu_robot robot);

/* Builds the environment BVHs (one per object group, plus per-object trees
 * for distance queries) and uploads them.  Replaces WorldModel geometry
 * initialisation (Cpp/Modeling/World.cpp:266-284). */
kgpu_status kgpu_env_create(const kgpu_env_desc* desc, kgpu_env* out);

/* kgpu_env_create with build flags.  KGPU_ENV_BUILD_GPU builds the
 * environment trees on the current GPU (linear BVH: Morton-code radix sort
 * and radix tree, boxes bottom up) instead of the host surface-area builder;
 * the layout, the results of every query and the FP32 conservativeness are
 * the same, the tree shape (and so the traversal cost) differs.  The host
 * builder stands in for the PQP precompute InitCollisions runs
 * (Cpp/Modeling/World.cpp:266-274); the GPU build is for scenes whose
 * precompute dominates. */
#define KGPU_ENV_BUILD_GPU 1
kgpu_status kgpu_env_create_ex(const kgpu_env_desc* desc, int32_t flags, kgpu_env* out);
kgpu_status kgpu_env_destroy(kgpu_env env);

/* Joins an environment and robots.  Collision masks start at Klamp't's
 * defaults: WorldPlannerSettings::InitializeDefault
 * (Cpp/Planning/PlannerSettings.cpp:16-42) — every link against every rigid
 * object, links whose parent is -1 not against terrains, self pairs as in the
 * robot description.  The world keeps references; destroy it before its
 * robots and environment. */
kgpu_status kgpu_world_create(kgpu_env env, const kgpu_robot* robots, int32_t num_robots,
                              kgpu_world* out);
kgpu_status kgpu_world_destroy(kgpu_world world);

/* Per-link group mask, the analogue of WorldPlannerSettings::collisionEnabled
 * rows (PlannerSettings.cpp:16-42) and WorldCollider.ignoreCollision
 * (Python/klampt/model/collide.py:314-362). */
kgpu_status kgpu_world_set_link_env_mask(kgpu_world world, int32_t robot, int32_t link,
                                         uint32_t group_mask);
/* Enables or disables self-collision testing of link pair (i,j), as
 * RobotModel::enableSelfCollision (robotsim.cpp:5513-5527). */
kgpu_status kgpu_world_enable_self_pair(kgpu_world world, int32_t robot, int32_t i, int32_t j,
                                        int32_t enabled);

/* Named options: "eps_extra" (m, additional inflation of every FP32 test on
 * top of the computed error bounds, default 0), "blocks_per_sm" (2, 3 or 4
 * resident engine blocks per SM), "grab" (work items per queue atomic, 1..16),
 * "job_flush" (triangle-pair jobs batched before testing, 8..64),
 * "edge_chunk" (consecutive steps of an edge per work item, 1..64, default
 * 16; the item checks them in groups of 32 / L steps, L the robot's link
 * count rounded up to 8, 16 or 32, earliest step first), "fp64_inline" (1: triangle pairs the FP32 tests
 * leave undecided get the FP64 test inside the traversal kernel; 0: they are
 * listed and decided by a second kernel, keeping FP64 code out of the
 * traversal kernel and letting configurations of one robot be checked in
 * groups; -1, the default: 0), "stage_nodes" (0..1024, default 0: at 2
 * blocks per SM with the FP64 test deferred, each engine block copies this
 * many top nodes of the breadth-first environment node array into shared
 * memory and reads them there; results do not change), read-only
 * "eps_env", "warps_per_block", "num_sms".  Test options that shrink a
 * bound until it is reached: "pend_cap" (undecided-pair list records),
 * "spill_cap" (spill entries per warp), "share_wait_polls" and
 * "share_no_release" (the work-sharing wait).  The autotuner
 * (klampt_gb300/autotune.py) sets blocks_per_sm, grab, job_flush and
 * edge_chunk or fp64_inline.
 * Unknown names are KGPU_ERR_INVALID. */
kgpu_status kgpu_world_set_option(kgpu_world world, const char* name, double value);
kgpu_status kgpu_world_get_option(kgpu_world world, const char* name, double* value);

/* Waits for the stream, then returns (and clears) the status word that the
 * world's kernels set on the device (overflow, non-finite input, timeout). */
kgpu_status kgpu_world_sync(kgpu_world world, kgpu_stream stream);
kgpu_status kgpu_world_get_stats(kgpu_world world, kgpu_stats* out);
kgpu_status kgpu_world_reset_stats(kgpu_world world);

/* ---- queries (device buffers, asynchronous on `stream`) ------------------- */

/* Forward kinematics.  Replaces RobotModel::setConfig -> UpdateFrames
 * (Python/klampt/src/robotsim.cpp:5311-5321).  q: [B*num_links] float,
 * T_out: [B*num_links*12] float world transforms, err_out: [B*num_links]
 * (may be NULL) a rigorous bound, per link, on the distance between any
 * vertex of the link placed with T_out and the same vertex placed with the
 * exact (FP64) transform. */
kgpu_status kgpu_fk(kgpu_world world, int32_t robot, const float* q, int32_t B, float* T_out,
                    float* err_out, kgpu_stream stream);

/* Forward kinematics in the canonical FP64 arithmetic (include/kgpu_exact.h):
 * the link transforms every FP64 decision of the engine and the oracle uses,
 * bit for bit (RobotModel::setConfig -> UpdateFrames in double precision,
 * robotsim.cpp:5311-5321).  q: [B*num_links] float (widened exactly),
 * T_out: [B*num_links*12] double. */
kgpu_status kgpu_fk64(kgpu_world world, int32_t robot, const float* q, int32_t B, double* T_out,
                      kgpu_stream stream);

/* Batched inverse kinematics: B problems, each moving point plocal[b] (link
 * frame) of link links[b] (or `link` when links is NULL) to ptarget[b] and,
 * when Rtarget is not NULL, the link's rotation to Rtarget[b] (row-major).
 * q [B * num_links]: initial guesses in, results out (clamped to the joint
 * limits).  ok[b] = 1 when max |residual| <= tol within max_iters
 * iterations, residual[b] = that maximum, iters[b] (may be NULL) the
 * iterations used.  Replaces IKSolver.solve over IKObjective point and
 * transform constraints (Python/klampt/src/robotik.cpp:556-689), one call for
 * B problems; the iteration is damped least squares (Levenberg-Marquardt) on
 * the link's ancestor DOFs, the reference's KrisLibrary solver being absent. */
kgpu_status kgpu_ik_solve(kgpu_world world, int32_t robot, int32_t B, float* q, const int32_t* links, int32_t link,
                          const float* plocal, const float* ptarget, const float* Rtarget, int32_t max_iters,
                          float tol, uint8_t* ok, float* residual, int32_t* iters, kgpu_stream stream);

/* Self-collision pairs that occur in a batch of B configurations: for every
 * enabled link pair (i < j) found colliding in some configuration, bit j of
 * pair_mask[i] is set (pair_mask: num_links words, OR-accumulated, so calls
 * can continue a sampling run).  Replaces the sampling loop of
 * RandomizedSelfCollisionPairs (Cpp/Modeling/RandomizedSelfCollisions.cpp:
 * 19-38): the caller supplies the configurations (uniform samples within the
 * joint limits there). */
kgpu_status kgpu_self_collision_pairs(kgpu_world world, int32_t robot, const float* q, int32_t B,
                                      uint32_t* pair_mask, kgpu_stream stream);

/* Independent self-collision pairs (RandomizedIndependentSelfCollisionPairs'
 * second pass, TestIndependentCollisions,
 * Cpp/Modeling/RandomizedSelfCollisions.cpp:42-66): for each of B
 * configurations the enabled pairs set in candidates (num_links words, as
 * kgpu_self_collision_pairs fills them) are tested; when exactly one of them
 * collides, its bit is set in pair_mask (OR-accumulated). */
kgpu_status kgpu_independent_self_collision_pairs(kgpu_world world, int32_t robot, const float* q, int32_t B,
                                                  const uint32_t* candidates, uint32_t* pair_mask,
                                                  kgpu_stream stream);

/* Full Jacobians of points on links at B configurations: J[b] is 6 x
 * num_links (row-major), rows 0-2 the angular part, rows 3-5 the linear
 * part of the world velocity of the point plocal[b] (link frame) on link
 * links[b] (or `link` for every configuration when links is NULL).
 * Replaces RobotModelLink::getJacobian / getPositionJacobian
 * (Python/klampt/src/robotsim.cpp:4817-4845; KrisLibrary GetFullJacobian),
 * one call for B configurations.  FP32, from the error-bounded FK. */
kgpu_status kgpu_jacobian(kgpu_world world, int32_t robot, const float* q, int32_t B, const int32_t* links,
                          int32_t link, const float* plocal, float* J, kgpu_stream stream);

/* Environment and self collision verdicts of B configurations, FP32 BVH
 * traversal with the FP64 band re-test.  Replaces, per configuration,
 * WorldPlannerSettings::CheckCollision(world, {robot}, others)
 * (PlannerSettings.cpp:269-331) and RobotModel::selfCollides
 * (robotsim.cpp:5529-5539).  env_hit/self_hit: [B] bytes (0/1); either may be
 * NULL to skip that test. */
kgpu_status kgpu_check_configs(kgpu_world world, int32_t robot, const float* q, int32_t B,
                               uint8_t* env_hit, uint8_t* self_hit, kgpu_stream stream);

/* Heterogeneous batch: configuration b belongs to robot robot_ids[b] and its
 * joint values start at q + b*q_stride.  One launch for all robots. */
kgpu_status kgpu_check_configs_multi(kgpu_world world, const int32_t* robot_ids, const float* q,
                                     int32_t q_stride, int32_t B, uint8_t* env_hit,
                                     uint8_t* self_hit, kgpu_stream stream);

/* Feasibility: joint limits, then environment, then self collision, as
 * SingleRobotCSpace::IsFeasible (Cpp/Planning/RobotCSpace.cpp:786-823).
 * feasible: [B] bytes. */
kgpu_status kgpu_is_feasible(kgpu_world world, int32_t robot, const float* q, int32_t B,
                             uint8_t* feasible, kgpu_stream stream);

/* Straight-line edge checks: edge e is discretised into configurations
 * q_k = qa + (k/n)(qb-qa), k = 0..n (n = nsteps[e] >= 1), and first_hit[e] is
 * the smallest k whose configuration is infeasible (-1 when all are
 * feasible).  Replaces EpsilonEdgeChecker / BisectionEpsilonEdgePlanner
 * visibility tests (Cpp/Planning/RobotCSpace.cpp:835-840,
 * Python/klampt/src/motionplanning.cpp:383-400) with interpolation as
 * Cpp/Modeling/Interpolate.cpp:10-14.  One persistent launch over all steps
 * of all edges. */
kgpu_status kgpu_check_edges(kgpu_world world, int32_t robot, const float* qa, const float* qb,
                             const int32_t* nsteps, int32_t E, int32_t* first_hit,
                             kgpu_stream stream);

/* The same outputs computed by the plain FP64 method: one thread per
 * configuration, FP64 forward kinematics, FP64 traversal and triangle tests,
 * no batching machinery.  The comparison baseline for the engine. */
kgpu_status kgpu_check_configs_plain64(kgpu_world world, int32_t robot, const float* q, int32_t B,
                                       uint8_t* env_hit, uint8_t* self_hit, kgpu_stream stream);
kgpu_status kgpu_check_edges_plain64(kgpu_world world, int32_t robot, const float* qa,
                                     const float* qb, const int32_t* nsteps, int32_t E,
                                     int32_t* first_hit, kgpu_stream stream);
/* The plain FP64 method with one thread per (edge, step): every
 * configuration of every edge checked on its own (no in-order early exit),
 * the smallest infeasible step kept; same outputs as kgpu_check_edges. */
kgpu_status kgpu_check_edges_plain64_steps(kgpu_world world, int32_t robot, const float* qa,
                                           const float* qb, const int32_t* nsteps, int32_t E,
                                           int32_t* first_hit, kgpu_stream stream);
/* The plain FP64 method with one thread per (edge, step, query): each
 * thread forms its step's FP64 transforms and checks one link-group or
 * link-link pair (the per-pair loop of PlannerSettings.cpp:269-331 split
 * across threads); same outputs as kgpu_check_edges. */
kgpu_status kgpu_check_edges_plain64_pairs(kgpu_world world, int32_t robot, const float* qa,
                                           const float* qb, const int32_t* nsteps, int32_t E,
                                           int32_t* first_hit, kgpu_stream stream);

/* Minimum signed link-obstacle distance per configuration, clamped at
 * `cutoff`, with its gradient d/dq.  Replaces the per-pair
 * Geometry3D::distance_ext loop (robotsim.cpp:1782-1819, settings
 * upperBound = cutoff) and WorldPlannerSettings::DistanceLowerBound
 * (PlannerSettings.cpp:372-483).  d: [B] (cutoff when nothing is closer),
 * pair: [B*2] (link, object) or (-1,-1), cp: [B*6] closest points in world
 * frame (link side, object side), grad: [B*num_links] (may be NULL). */
kgpu_status kgpu_distance(kgpu_world world, int32_t robot, const float* q, int32_t B,
                          double cutoff, double* d, int32_t* pair, double* cp, float* grad,
                          kgpu_stream stream);

/* Minimum distance between the robot's own links over its enabled self pairs,
 * clamped at `cutoff`, with its gradient d/dq: the link-link part of
 * WorldPlannerSettings::DistanceLowerBound when a robot is checked against
 * itself (Cpp/Planning/PlannerSettings.cpp:385-395) and of geometry_ad.MinDistance over
 * link geometries.  d(i, j) = exact minimum triangle distance (0 when the
 * surfaces meet); d: [B] = min over enabled pairs i < j, equal distances to the
 * smallest (i, j) (cutoff when nothing is closer); pair: [B*2] (i, j) or (-1,-1); cp:
 * [B*6] closest points in world frame (link i side, link j side; 0 when
 * d = 0); grad: [B*num_links] (may be NULL; 0 when d = 0). */
kgpu_status kgpu_self_distance(kgpu_world world, int32_t robot, const float* q, int32_t B, double cutoff,
                               double* d, int32_t* pair, double* cp, float* grad, kgpu_stream stream);

/* Each self pair's own minimum distance, for the per-pair minima and maxima
 * over sampled configurations of RandomizedSelfCollisionDistances
 * (Cpp/Modeling/RandomizedSelfCollisions.cpp:142-180, which keeps, for each
 * pair i < j whose links both have geometry, the smallest and largest
 * distance seen over numSamples samples).  all_pairs != 0 queries every such
 * pair, as that function does, whatever the self-collision mask says;
 * all_pairs == 0 only the enabled self pairs.
 * dpair: [B * L(L-1)/2], entry i*L - i(i+1)/2 + (j-i-1) for the pair i < j:
 * the pair's exact minimum triangle distance (0 when the surfaces meet),
 * clamped at `cutoff`; -1 for pairs that are not queried or lack geometry. */
kgpu_status kgpu_self_pair_distances(kgpu_world world, int32_t robot, const float* q, int32_t B, double cutoff,
                                     int32_t all_pairs, double* dpair, kgpu_stream stream);

/* Soft-min over all (waypoint, link, object) pairs of a trajectory of the
 * signed distance, L = -tau * log sum exp(-d/tau), and dL/dq by the adjoint
 * kernel.  Replaces geometry_ad.MinDistance + pytorch.ADModule backward
 * (Python/klampt/math/autodiff/geometry_ad.py:613-814,
 * Python/klampt/math/autodiff/pytorch.py:72-115).  q: [T*W*num_links],
 * L: [T], dLdq: [T*W*num_links] (may be NULL). */
kgpu_status kgpu_softmin_grad(kgpu_world world, int32_t robot, const float* q, int32_t T,
                              int32_t W, double tau, double* L, float* dLdq, kgpu_stream stream);

/* Batched ray casting against every object of the world's environment: ray
 * i is s[3i..3i+2] + t d[3i..3i+2], t >= 0.  Per ray: obj = index of the
 * object hit first (-1: none), tri = the hit triangle's index in that
 * object's mesh, t = the ray parameter (FP64, +inf on a miss), point = the
 * hit point s + t d (FP64).  Nearest hit, ties to the smaller object, then
 * triangle; a ray in a triangle's plane does not hit it.  Replaces
 * Geometry3D::rayCast / rayCast_ext (Python/klampt/src/robotsim.cpp:
 * 1821-1852), the environment part of WorldModel::RayCast
 * (Cpp/Modeling/World.cpp:465-515) and collide.ray_cast
 * (Python/klampt/model/collide.py:219-243), one call for R rays. */
kgpu_status kgpu_raycast(kgpu_world world, const float* s, const float* d, int32_t R, int32_t* obj,
                         int32_t* tri, double* t, double* point, kgpu_stream stream);

/* ---- free geometries: Geometry3D pair queries -------------------------------- */
/* A triangle mesh with its own BVH, placed by a caller-supplied transform per
 * query: the analogue of a TriangleMesh Geometry3D (Python/klampt/src/
 * geometry.h:810) with its collision margin (setCollisionMargin,
 * geometry.h:930).  Vertices are in the geometry's own frame. */
typedef struct kgpu_geom_s* kgpu_geom;
typedef struct {
  int32_t num_verts;
  const double* verts;  /* [num_verts*3] */
  int32_t num_tris;
  const int32_t* tris;  /* [num_tris*3] vertex indices */
  double margin;        /* collision margin (>= 0) */
} kgpu_geom_desc;
kgpu_status kgpu_geom_create(const kgpu_geom_desc* desc, kgpu_geom* out);
kgpu_status kgpu_geom_destroy(kgpu_geom geom);
/* Geometry3D::setCollisionMargin / getCollisionMargin (robotsim.cpp). */
kgpu_status kgpu_geom_set_margin(kgpu_geom geom, double margin);
kgpu_status kgpu_geom_get_margin(kgpu_geom geom, double* margin);

/* Batched pair queries between geometry a at transform Ta[b] and geometry
 * b at transform Tb[b] (device buffers of B*12 doubles, R row-major then t;
 * with KGPU_GEOM_FIXED_A / _B in flags, Ta / Tb is one transform used for
 * every query).  Results are those of the canonical FP64 arithmetic on the
 * world-placed triangles (include/kgpu_exact.h). */
#define KGPU_GEOM_FIXED_A 1
#define KGPU_GEOM_FIXED_B 2
/* hit[b] = 1 when the geometries are within (m_a + tol) + m_b of each other
 * (tol = 0: Geometry3D::collides, robotsim.cpp:1656-1662, touching counts;
 * tol > 0: Geometry3D::withinDistance, robotsim.cpp:1685-1690 and
 * ::CheckCollision(m1, m2, tol), Cpp/Planning/PlannerSettings.cpp:96-107). */
kgpu_status kgpu_geom_collide(kgpu_geom a, kgpu_geom b, const double* Ta, const double* Tb, int32_t B, int32_t flags,
                              double tol, uint8_t* hit, kgpu_stream stream);
/* Geometry3D::distance_ext (robotsim.cpp:1782-1819) with
 * DistanceQuerySettings.upperBound = upper_bound (+inf for none; relErr and
 * absErr are met with 0): d[b] = mesh distance - (m_a + m_b) (triangle
 * meshes give unsigned mesh distances, 0 when they meet), or upper_bound
 * when nothing is closer; cp[b*6] the closest points (on a, then on b, world
 * frame; on contact both are a vertex of a's touching triangle); elem[b*2]
 * the closest triangle pair (mesh order; ties to the smallest, (-1,-1) when
 * nothing is closer); dir[b*3] (may be NULL) grad1 = (cp_a - cp_b)/|cp_a -
 * cp_b| (grad2 = -grad1, geometry.h:660-662), 0 on contact.  An empty
 * geometry is KGPU_ERR_EMPTY (robotsim.cpp:1786-1787). */
kgpu_status kgpu_geom_distance(kgpu_geom a, kgpu_geom b, const double* Ta, const double* Tb, int32_t B, int32_t flags,
                               double upper_bound, double* d, double* cp, int32_t* elem, double* dir,
                               kgpu_stream stream);
/* Waits for the stream, then returns (and clears) geometry a's device status
 * word set by the pair queries it was the first geometry of (non-finite or
 * |entry| >= 1e6 transforms: KGPU_ERR_NOT_FINITE). */
kgpu_status kgpu_geom_sync(kgpu_geom a, kgpu_stream stream);

/* ---- host-buffer variants (pinned staging inside; synchronous) ------------ */
kgpu_status kgpu_check_configs_host(kgpu_world world, int32_t robot, const float* q, int32_t B,
                                    uint8_t* env_hit, uint8_t* self_hit);
kgpu_status kgpu_check_edges_host(kgpu_world world, int32_t robot, const float* qa,
                                  const float* qb, const int32_t* nsteps, int32_t E,
                                  int32_t* first_hit);

/* ---- edge checks without allocation --------------------------------------- */
/* No counterpart in the reference (Klamp't's checkers run on the host).  For
 * callers that may not allocate device memory while they run — a real-time
 * planning or control loop that cannot afford cudaMalloc's device-wide
 * synchronisation, or a host application that hands all device memory to its
 * own pool — this variant of kgpu_check_edges gives the same results but
 * works only inside one fixed 32 MiB file-scope device array, which every
 * GPU that loads the library keeps until the process exits.  At most
 * KGPU_NOALLOC_MAX_EDGES edges per call (larger E: KGPU_ERR_INVALID).
 * kgpu_world_create looks the array up (and so loads it) on the world's
 * device, so no call allocates; each call clears the parts that must start
 * at zero, and calls that overlap on the GPU race on the shared array, so
 * serialise them.  It uses the world's launch options, with blocks_per_sm
 * capped at what the array's per-warp regions serve (2560 warps).  The
 * world's collision masks must not have changed since its last regular
 * query (re-uploading them would allocate). */
#define KGPU_NOALLOC_MAX_EDGES 65536
kgpu_status kgpu_check_edges_noalloc(kgpu_world world, int32_t robot, const float* qa,
                                     const float* qb, const int32_t* nsteps, int32_t E,
                                     int32_t* first_hit, kgpu_stream stream);

/* ---- captured edge-check plans (CUDA-graph replay) ------------------------ */
/* Records the whole edge-check pipeline for fixed device buffers into a CUDA
 * graph; each launch replays it on `stream`.  The plan keeps using the
 * world's scratch buffers it was recorded with (buffers that later calls
 * grow are kept until the world is destroyed); destroy plans before their
 * world. */
kgpu_status kgpu_edge_plan_create(kgpu_world world, int32_t robot, const float* qa,
                                  const float* qb, const int32_t* nsteps, int32_t E,
                                  int32_t* first_hit, kgpu_edge_plan* out);
kgpu_status kgpu_edge_plan_launch(kgpu_edge_plan plan, kgpu_stream stream);
/* Device time (ms) of the main traversal pass of the plan's last launch,
 * between two events the graph records around it; call after that launch
 * has completed (the next launch records them again).  No reference
 * counterpart: it exposes the timing the bench's roofline uses. */
kgpu_status kgpu_edge_plan_main_pass_ms(kgpu_edge_plan plan, float* ms);
kgpu_status kgpu_edge_plan_destroy(kgpu_edge_plan plan);

/* ---- captured configuration-batch plans (CUDA-graph replay) -------------- */
/* The configuration-batch check of kgpu_check_configs (robot >= 0) or, with
 * robot = -1, of kgpu_check_configs_multi (robot_ids, q_stride) recorded for
 * fixed device buffers into a CUDA graph with the world's current launch
 * options; each launch replays it on `stream`.  Replaces, per batch, the
 * WorldPlannerSettings::CheckCollision / RobotModel::selfCollides loop
 * (Cpp/Planning/PlannerSettings.cpp:269-331, robotsim.cpp:5529-5539).  As
 * for edge plans: destroy plans before their world. */
kgpu_status kgpu_config_plan_create(kgpu_world world, int32_t robot, const int32_t* robot_ids, const float* q,
                                    int32_t q_stride, int32_t B, uint8_t* env_hit, uint8_t* self_hit,
                                    kgpu_config_plan* out);
kgpu_status kgpu_config_plan_launch(kgpu_config_plan plan, kgpu_stream stream);
kgpu_status kgpu_config_plan_destroy(kgpu_config_plan plan);

/* ---- diagnostics ------------------------------------------------------------ */
/* Last error message of the calling thread ("" when none). */
const char* kgpu_last_error(void);
/* Library version string. */
const char* kgpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KGPU_H */
