// kgpu_internal.h — device data layouts and host-side objects of the engine.
//
// HBM layout (all arrays are device-resident for the life of the handles):
//   link BVH nodes    KNode[] for every link of every robot, concatenated;
//                     child/leaf indices are global into the same array
//   link triangles    float4[3] per triangle (FP32, link frame) in BVH leaf
//                     order, plus double[9] per triangle (FP64 copy for the
//                     band re-test)
//   env BVH nodes     KNode[] for every object group; each group tree is
//                     object-aware: its top levels split objects, and every
//                     object owns a subtree (its root is obj_root[o])
//   env triangles     float4[3] + double[9] per triangle (world frame), and
//                     the owning object of each triangle
// A node is 32 bytes (two float4): (center.xyz, index) and (half.xyz, count);
// count == 0 marks an internal node whose children are index and index+1, a
// leaf holds triangles [index, index+count).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/kgpu.h"

namespace kgpu {

constexpr int kMaxLinks = KGPU_MAX_LINKS;
constexpr int kMaxGroups = 32;
constexpr int kLeafSize = 4;
constexpr int kMaxSteps = 65535;

struct KNode {
  float4 a;  // center.xyz, index (int bits)
  float4 b;  // half.xyz, count (int bits)
};

// Host-side BVH result in the device layout.
struct HostBvh {
  std::vector<KNode> nodes;          // local indices (root = 0)
  std::vector<double> node_c64;      // 3 per node, FP64 center
  std::vector<double> node_h64;      // 3 per node, FP64 half extent
  std::vector<double> node_r;        // per node: radius of the sphere about the box
                                     // centre that holds the node's vertices
  std::vector<int> order;            // triangle ids in leaf order
  std::vector<int> node_obj;         // object owning each node (-1 above objects)
};

// Builds a BVH over triangles `ids` (tri: 9 doubles per triangle id).  When
// tri_obj is given, the top levels split whole objects so that every object
// owns one subtree.  Binned surface-area splits of the triangles, leaves of
// at most kLeafSize triangles, children adjacent.
void build_bvh(const std::vector<double>& tri, const std::vector<int>& ids,
               const std::vector<int>* tri_obj, HostBvh& out);

// The same object-aware layout built on the current GPU (linear BVH over
// Morton codes; kgpu_lbvh.cu).  tri_obj maps every triangle id to its object.
cudaError_t lbvh_build(const std::vector<double>& tri, const std::vector<int>& ids, const std::vector<int>& tri_obj,
                       HostBvh& out);

// Device tables of one robot (read through the read-only cache).
struct KRobotDev {
  int nlinks;
  int nqueries_env;   // (link, group) queries
  int nqueries_self;  // (link, link) queries
  int query_off;      // into KWorldDev::queries (env queries first)
  int parents[kMaxLinks];
  int jtype[kMaxLinks];
  int link_root[kMaxLinks];  // global node index or -1
  int link_depth[kMaxLinks];
  int link_vert_first[kMaxLinks], link_vert_count[kMaxLinks];  // unique vertices (global)
  uint32_t env_mask[kMaxLinks];
  float link_margin[kMaxLinks];
  float link_r[kMaxLinks];   // largest vertex norm of the link mesh in its frame (rounded up)
  float qmin[kMaxLinks], qmax[kMaxLinks];
  float T0P[kMaxLinks][12];
  float axis[kMaxLinks][3];
  double T0P64[kMaxLinks][12];
  double axis64[kMaxLinks][3];
  double qmin64[kMaxLinks], qmax64[kMaxLinks];
  double link_margin64[kMaxLinks];
};

struct KWorldDev {
  // robots
  const KRobotDev* robots;
  const uint32_t* queries;   // a | tgt << 8 ; tgt < 32: link, tgt >= 32: env group tgt-32
  const KNode* lnodes;
  const float4* ltri32;      // 3 per tri
  const double* ltri64;      // 9 per tri
  const double* lnode64;     // 6 per node (c, h) FP64 (plain kernel)
  const float* lnode_r;      // per link node: radius about its FP32 centre holding its vertices
  const int* ltri_orig;      // per link triangle: index in its link's mesh order
  const float4* lvert32;     // unique link vertices (link frame), mesh order
  const double* lvert64;     // 3 per unique link vertex
  // environment
  const KNode* enodes;
  const float4* etri32;
  const double* etri64;
  const double* enode64;     // 6 per node
  const int* etri_obj;
  const float* obj_margin;
  const double* obj_margin64;
  const int* obj_root;       // per object: node index of its subtree root
  const int* obj_group;
  const uint8_t* obj_convex;
  const int* node_obj;       // per env node
  const int* etri_orig;      // per env triangle (leaf order): global input index
  const float4* eface32;     // per env triangle: unit outward normal, n . a  (FP32)
  const double* eface64;     // 4 per env triangle: the same in canonical FP64
  const int* obj_leaf_first; // per object: its triangles' leaf-order range
  const int* obj_leaf_count;
  const int* obj_tri_first;  // per object: its first triangle in the input order
  int group_root[kMaxGroups];
  float group_margin[kMaxGroups];
  int num_objects;
  int env_nodes;             // nodes in enodes (laid out breadth first from the group roots)
  // tolerances (m): the per-link FP32 error bounds come from warp_fk32; the
  // environment's FP32 coordinates are off by at most eps_env; eps_extra is
  // an optional additional inflation (world option, default 0)
  float eps_env;
  float eps_extra;
  // work sharing of the edge engine: polls a warp waits for a claimed
  // hand-over before it reports KGPU_ERR_TIMEOUT (0: the default bound), and
  // a failure-path test switch under which a donor claims a waiting warp but
  // never hands work over (it keeps its entries, so no work is lost)
  int share_wait;
  int share_no_release;
  // diagnostics
  int* status;               // device status word
  unsigned long long* stats; // kgpu_stats counters
};

// scratch owned by the world (allocated at creation, grown on demand)
struct Scratch {
  uint2* spill = nullptr;          // per-warp spill stacks
  size_t spill_per_warp = 0;
  int max_warps = 0;
  unsigned int* counters = nullptr;  // work-queue heads and the re-test list count
  uint4* pend = nullptr;             // triangle pairs left to the FP64 re-test
  int pend_cap = 0;
  int* edge_hist = nullptr;          // kMaxSteps+2
  int* edge_round_off = nullptr;     // kMaxSteps+2
  int* edge_perm = nullptr;
  int* edge_meta = nullptr;          // 4 meta words, fill counters, count_ge (2 x (kMaxSteps+2))
  size_t edge_cap = 0;
  double* dist_work = nullptr;       // soft-min per-waypoint minima, sums, trajectory minima
  size_t dist_work_cap = 0;
  // launch setting carried with the scratch: environment nodes a staged
  // engine block copies to shared memory (0: the unstaged kernels)
  int stage_nodes = 0;
  // edge plans: events recorded (as graph nodes) around the main pass, so
  // that its own device time can be read after a launch
  cudaEvent_t main_pass_ev[2] = {nullptr, nullptr};
};

}  // namespace kgpu

// ---- host objects -----------------------------------------------------------
struct kgpu_robot_s {
  int nlinks = 0;
  std::vector<int> parents, jtypes;
  std::vector<double> T0P, axes, qmin, qmax, margins;
  std::vector<uint8_t> self_mask;   // [L*L] upper triangle
  std::vector<int> link_tri_count;
  std::vector<double> link_r;              // largest vertex norm per link (link frame)
  // device arrays of this robot's links (local indices per link)
  std::vector<kgpu::HostBvh> bvh;
  std::vector<std::vector<double>> tri64;  // per link, leaf order, 9 per tri
  std::vector<std::vector<double>> vert64; // per link, unique vertices in mesh order
  double reach = 0.0;                      // bound on |world coordinate| of any link point
};

struct kgpu_env_s {
  int nobj = 0;
  std::vector<int> groups;
  std::vector<uint8_t> convex;
  std::vector<double> margins;
  std::vector<int> tri_off;
  // per group BVH (object-aware) over global triangle ids
  kgpu::HostBvh gbvh[kgpu::kMaxGroups];
  std::vector<double> tri64;   // global, original order, 9 per tri
  std::vector<int> tri_obj;
  double extent = 0.0;
  // device
  kgpu::KNode* d_nodes = nullptr;
  float4* d_tri32 = nullptr;
  double* d_tri64 = nullptr;
  double* d_node64 = nullptr;
  int* d_tri_obj = nullptr;
  float* d_obj_margin = nullptr;
  double* d_obj_margin64 = nullptr;
  int* d_obj_root = nullptr;
  int* d_obj_group = nullptr;
  uint8_t* d_obj_convex = nullptr;
  int* d_node_obj = nullptr;
  int* d_tri_orig = nullptr;
  float4* d_face32 = nullptr;
  double* d_face64 = nullptr;
  int* d_obj_leaf_first = nullptr;
  int* d_obj_leaf_count = nullptr;
  int* d_obj_tri_first = nullptr;
  int group_root[kgpu::kMaxGroups];
  float group_margin[kgpu::kMaxGroups];
  size_t n_nodes = 0, n_tris = 0;
};

struct kgpu_world_s {
  kgpu_env env = nullptr;
  std::vector<kgpu_robot> robots;
  std::vector<std::vector<uint32_t>> env_mask;     // per robot per link
  std::vector<std::vector<uint8_t>> self_enabled;  // per robot [L*L]
  // device copies
  kgpu::KRobotDev* d_robots = nullptr;
  uint32_t* d_queries = nullptr;
  kgpu::KNode* d_lnodes = nullptr;
  float4* d_ltri32 = nullptr;
  double* d_ltri64 = nullptr;
  double* d_lnode64 = nullptr;
  float* d_lnode_r = nullptr;
  int* d_ltri_orig = nullptr;
  float4* d_lvert32 = nullptr;
  double* d_lvert64 = nullptr;
  std::vector<int> robot_vert_base;
  int* d_status = nullptr;
  unsigned long long* d_stats = nullptr;
  std::vector<int> robot_node_base, robot_tri_base;
  kgpu::KWorldDev dev;                // host copy of the descriptor
  kgpu::KWorldDev* d_dev = nullptr;   // device copy read by the engine kernels
  kgpu::Scratch scratch;
  // tolerances
  double eps_env = 0.0;
  double eps_extra = 0.0;
  int blocks_per_sm = 3;   // resident 8-warp engine blocks per SM (2, 3 or 4)
  int grab = 2;            // work items per queue atomic (1..16)
  int job_flush = 64;      // triangle-pair jobs collected before testing them (8..64)
  int edge_chunk = 16;     // consecutive steps of an edge per work item (1..64)
  int fp64_inline = -1;    // FP64 triangle tests inline (1) or deferred to k_band (0); -1: deferred
  // caps below the allocated scratch (0 = none): the undecided-pair list and
  // the traversal spill stack per warp; they exist to drive the list-overflow
  // fallback pass and spill exhaustion in tests
  int pend_cap_opt = 0;
  int spill_cap_opt = 0;
  int stage_nodes = 0;     // world option: environment nodes staged per engine block (0..1024; 2 blocks per SM)
  int num_sms = 0;
  bool tables_dirty = true;
  // pinned staging for the host-buffer entry points
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  void* dstage = nullptr;
  size_t dstage_bytes = 0;
  cudaStream_t host_stream = nullptr;
  // edge plans record scratch pointers: while any is alive, buffers that
  // grow are kept (freed with the world) instead of freed
  int live_plans = 0;
  std::vector<void*> retired;
};

struct kgpu_edge_plan_s {
  kgpu_world world = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};  // around the main pass
};

struct kgpu_config_plan_s {
  kgpu_world world = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace kgpu {
// launchers implemented in the .cu files (return a CUDA error code).  The
// engine kernels read the world descriptor from device memory (Wd); the
// plain and distance kernels take it by value (W).
cudaError_t launch_fk(const KWorldDev* Wd, int robot, const float* q, int B, float* T, float* err,
                      cudaStream_t s);
// per_sm selects the register budget of the engine instantiation; grab = items
// per work-queue atomic, job_flush = triangle-pair job batch size (0 = default)
cudaError_t launch_check_configs(const KWorldDev* Wd, const Scratch& S, int robot,
                                 const int* robot_ids, const float* q, int q_stride, int B,
                                 uint8_t* env_hit, uint8_t* self_hit, uint8_t* feasible,
                                 int blocks, int per_sm, cudaStream_t s, int grab = 0,
                                 int job_flush = 0, int fp64_inline = -1,
                                 int nrobots = 0, int* status = nullptr);
cudaError_t launch_check_edges(const KWorldDev* Wd, int* status, const Scratch& S, int robot,
                               const float* qa, const float* qb, const int* nsteps, int E,
                               int* first_hit, int blocks, int per_sm, cudaStream_t s,
                               int grab = 0, int job_flush = 0, int chunk = 0, int fp64_inline = -1);
cudaError_t launch_fk64(const KWorldDev* Wd, int robot, const float* q, int B, double* T, cudaStream_t s);
cudaError_t launch_plain64_configs(const KWorldDev& W, int robot, const float* q, int B,
                                   uint8_t* env_hit, uint8_t* self_hit, cudaStream_t s);
cudaError_t launch_plain64_edges(const KWorldDev& W, int robot, const float* qa,
                                 const float* qb, const int* nsteps, int E, int* first_hit,
                                 cudaStream_t s);
// one thread per (edge, step); off: E + 1 ints of scratch
cudaError_t launch_plain64_edge_pairs(const KWorldDev& W, int robot, const float* qa, const float* qb,
                                      const int* nsteps, int E, int* first_hit, int* off, int num_sms,
                                      cudaStream_t s);
cudaError_t launch_plain64_edge_steps(const KWorldDev& W, int robot, const float* qa, const float* qb,
                                      const int* nsteps, int E, int* first_hit, int* off, int num_sms,
                                      cudaStream_t s);
cudaError_t launch_ik(const KWorldDev* W, int robot, int B, float* q, const int* links, int link_all,
                      const float* plocal, const float* ptarget, const float* Rtarget, int max_iters, float tol,
                      uint8_t* ok, float* residual, int* iters, cudaStream_t s);
cudaError_t launch_self_pairs(const KWorldDev* W, const Scratch& S, int robot, const float* q, int B,
                              const unsigned int* cand, unsigned int* pair_mask, int num_sms, cudaStream_t s);
cudaError_t launch_jacobian(const KWorldDev* W, int robot, const float* q, const int* links, int link_all,
                            const float* plocal, int B, float* J, cudaStream_t s);
cudaError_t launch_raycast(const KWorldDev* Wd, const float* s, const float* d, int R, int* obj, int* tri,
                           double* t, double* point, cudaStream_t st);
cudaError_t dist_init();
// loads kgpu_check_edges_noalloc's static array on the current device and
// caches its address (kgpu_noalloc.cu)
cudaError_t noalloc_prepare();
// the world's scratch with its optional test caps applied (kgpu_api.cu)
Scratch engine_scratch(kgpu_world w, Scratch S);
cudaError_t launch_distance(const KWorldDev* Wd, const Scratch& S, int robot, const float* q, int B,
                            double cutoff, double* d, int* pair, double* cp, float* grad, int num_sms,
                            cudaStream_t s);
// dpair != null: per-pair mode; all_pairs: every pair whose links have
// geometry instead of the enabled self pairs
cudaError_t launch_self_distance(const KWorldDev* Wd, int robot, const float* q, int B, double cutoff, double* d,
                                 int* pair, double* cp, float* grad, double* dpair, int all_pairs, int num_sms,
                                 cudaStream_t s);
// work: 2*T*Wn + T doubles of device scratch
cudaError_t launch_softmin(const KWorldDev* Wd, const Scratch& S, int robot, const float* q, int T,
                           int Wn, double tau, double* L, float* dLdq, int nl, double* work,
                           int num_sms, cudaStream_t s);
}  // namespace kgpu
