// kgpu_api.cu — the C ABI of include/kgpu.h: handle construction (host BVH
// build + upload), argument validation, launches, device status words,
// host-buffer variants and CUDA-graph edge plans.
//
// Error behaviour mirrors the reference's binding layer: where Klamp't throws
// PyException (mapped to RuntimeError by Python/klampt/src/robotsim.i:41-53),
// e.g. a configuration of the wrong size (robotsim.cpp:5314-5316), these
// functions return a status code and record a message for kgpu_last_error().
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/kgpu_exact.h"
#include "kgpu_internal.h"

using namespace kgpu;

namespace {
thread_local std::string g_err;
}

namespace kgpu {
// lets other translation units of the library set kgpu_last_error()
kgpu_status record_error(kgpu_status code, const char* msg)
{
  g_err = msg;
  return code;
}
cudaError_t engine_init();
size_t engine_smem_per_warp();
int engine_warps_per_block();
int engine_scratch_doubles();
}

namespace {

kgpu_status fail(kgpu_status code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
kgpu_status fail(kgpu_status code, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

kgpu_status cuda_fail(cudaError_t e, const char* what)
{
  return fail(e == cudaErrorMemoryAllocation ? KGPU_ERR_OOM : KGPU_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

template <class T>
cudaError_t upload(T** dst, const T* src, size_t n)
{
  *dst = nullptr;
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

template <class T>
void dfree(T*& p)
{
  if (p) cudaFree((void*)p);
  p = nullptr;
}

inline float round_up_f(double x)
{
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, 1e30f);
  return f;
}

inline float as_float(int i)
{
  float f;
  memcpy(&f, &i, 4);
  return f;
}
inline int as_int(float f)
{
  int i;
  memcpy(&i, &f, 4);
  return i;
}

// appends `b` to the concatenated arrays with node/triangle index shifts
void append_bvh(const HostBvh& b, int node_base, int tri_base, std::vector<KNode>& nodes,
                std::vector<double>& node64, std::vector<float>* node_r = nullptr)
{
  for (size_t k = 0; k < b.nodes.size(); ++k) {
    KNode n = b.nodes[k];
    int cnt = as_int(n.b.w), idx = as_int(n.a.w);
    n.a.w = as_float(cnt > 0 ? idx + tri_base : idx + node_base);
    nodes.push_back(n);
    for (int i = 0; i < 3; ++i) node64.push_back(b.node_c64[3 * k + i]);
    for (int i = 0; i < 3; ++i) node64.push_back(b.node_h64[3 * k + i]);
    if (node_r) {
      // sphere about the FP32 centre: the FP64 radius plus the centre's rounding
      const double cf[3] = {b.nodes[k].a.x, b.nodes[k].a.y, b.nodes[k].a.z};
      double off2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double d = b.node_c64[3 * k + i] - cf[i];
        off2 += d * d;
      }
      double r = b.node_r[k] + std::sqrt(off2);
      float f = (float)r;
      if ((double)f < r) f = std::nextafter(f, 3.0e38f);
      node_r->push_back(f);
    }
  }
}

void free_world_device(kgpu_world w)
{
  for (void* p : w->retired) cudaFree(p);
  w->retired.clear();
  dfree(w->d_robots);
  dfree(w->d_queries);
  dfree(w->d_dev);
  dfree(w->d_lnodes);
  dfree(w->d_ltri32);
  dfree(w->d_ltri64);
  dfree(w->d_lnode64);
  dfree(w->d_lnode_r);
  dfree(w->d_ltri_orig);
  dfree(w->d_lvert32);
  dfree(w->d_lvert64);
  dfree(w->d_status);
  dfree(w->d_stats);
  dfree(w->scratch.spill);
  dfree(w->scratch.counters);
  dfree(w->scratch.pend);
  dfree(w->scratch.edge_hist);
  dfree(w->scratch.edge_round_off);
  dfree(w->scratch.edge_perm);
  dfree(w->scratch.edge_meta);
  dfree(w->scratch.dist_work);
  if (w->pinned) cudaFreeHost(w->pinned);
  w->pinned = nullptr;
  dfree(w->dstage);
  if (w->host_stream) cudaStreamDestroy(w->host_stream);
  w->host_stream = nullptr;
}

// (re)builds the per-robot device tables and query lists
kgpu_status refresh_tables(kgpu_world w)
{
  if (!w->tables_dirty) return KGPU_OK;
  std::vector<KRobotDev> rd(w->robots.size());
  std::vector<uint32_t> queries;
  kgpu_env env = w->env;
  for (size_t r = 0; r < w->robots.size(); ++r) {
    kgpu_robot R = w->robots[r];
    KRobotDev& d = rd[r];
    memset(&d, 0, sizeof d);
    d.nlinks = R->nlinks;
    int node_base = w->robot_node_base[r];
    int vert_base = w->robot_vert_base[r];
    int depth_max = 0;
    for (int i = 0; i < R->nlinks; ++i) {
      d.link_vert_first[i] = vert_base;
      d.link_vert_count[i] = (int)(R->vert64[i].size() / 3);
      vert_base += d.link_vert_count[i];
      d.parents[i] = R->parents[i];
      d.jtype[i] = R->jtypes[i];
      d.link_root[i] = R->bvh[i].nodes.empty() ? -1 : node_base;
      node_base += (int)R->bvh[i].nodes.size();
      int dep = 0;
      for (int j = i; j >= 0; j = R->parents[j]) ++dep;
      d.link_depth[i] = dep;
      depth_max = dep > depth_max ? dep : depth_max;
      d.env_mask[i] = w->env_mask[r][i];
      d.link_margin[i] = round_up_f(R->margins[i]);
      d.link_r[i] = round_up_f(R->link_r[i] * (1.0 + 1e-6));
      d.link_margin64[i] = R->margins[i];
      d.qmin[i] = (float)R->qmin[i];
      d.qmax[i] = (float)R->qmax[i];
      d.qmin64[i] = R->qmin[i];
      d.qmax64[i] = R->qmax[i];
      for (int k = 0; k < 12; ++k) {
        d.T0P[i][k] = (float)R->T0P[12 * i + k];
        d.T0P64[i][k] = R->T0P[12 * i + k];
      }
      for (int k = 0; k < 3; ++k) {
        d.axis[i][k] = (float)R->axes[3 * i + k];
        d.axis64[i][k] = R->axes[3 * i + k];
      }
    }
    d.query_off = (int)queries.size();
    for (int i = 0; i < R->nlinks; ++i) {
      if (d.link_root[i] < 0) continue;
      for (int g = 0; g < kMaxGroups; ++g)
        if (((d.env_mask[i] >> g) & 1u) && env && env->group_root[g] >= 0) {
          queries.push_back((uint32_t)i | ((uint32_t)(32 + g) << 8));
          d.nqueries_env++;
        }
    }
    for (int i = 0; i < R->nlinks; ++i)
      for (int j = i + 1; j < R->nlinks; ++j)
        if (w->self_enabled[r][i * R->nlinks + j] && d.link_root[i] >= 0 && d.link_root[j] >= 0) {
          queries.push_back((uint32_t)i | ((uint32_t)j << 8));
          d.nqueries_self++;
        }
  }
  dfree(w->d_robots);
  dfree(w->d_queries);
  CK(upload(&w->d_robots, rd.data(), rd.size()));
  if (queries.empty()) queries.push_back(0);
  CK(upload(&w->d_queries, queries.data(), queries.size()));
  w->dev.robots = w->d_robots;
  w->dev.queries = w->d_queries;
  if (!w->d_dev) CK(cudaMalloc((void**)&w->d_dev, sizeof(KWorldDev)));
  CK(cudaMemcpy(w->d_dev, &w->dev, sizeof(KWorldDev), cudaMemcpyHostToDevice));
  w->tables_dirty = false;
  return KGPU_OK;
}

int grid_blocks(kgpu_world w) { return w->num_sms * w->blocks_per_sm; }

}  // namespace

namespace kgpu {
// The world's engine scratch with the optional caps applied (a copy: the
// allocation is unchanged).
Scratch engine_scratch(kgpu_world w, Scratch S)
{
  if (w->pend_cap_opt > 0 && w->pend_cap_opt < S.pend_cap) S.pend_cap = w->pend_cap_opt;
  const size_t spill = (size_t)w->spill_cap_opt + (size_t)engine_scratch_doubles();
  if (w->spill_cap_opt > 0 && spill < S.spill_per_warp) S.spill_per_warp = spill;
  S.stage_nodes = w->stage_nodes;
  return S;
}
}  // namespace kgpu

namespace {

kgpu_status ensure_edge_scratch(kgpu_world w, int E)
{
  if ((size_t)E <= w->scratch.edge_cap) return KGPU_OK;
  if (w->live_plans > 0) {
    w->retired.push_back(w->scratch.edge_perm);  // a captured plan still uses it
    w->scratch.edge_perm = nullptr;
  } else {
    dfree(w->scratch.edge_perm);
  }
  size_t cap = (size_t)E < 1024 ? 1024 : (size_t)E;
  CK(cudaMalloc((void**)&w->scratch.edge_perm, cap * sizeof(int)));
  w->scratch.edge_cap = cap;
  return KGPU_OK;
}

kgpu_status check_world(kgpu_world w, int robot)
{
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  if (robot < 0 || robot >= (int)w->robots.size())
    return fail(KGPU_ERR_INVALID, "robot index %d out of range [0,%d)", robot, (int)w->robots.size());
  return refresh_tables(w);
}

kgpu_status launch_status(cudaError_t e, const char* what)
{
  if (e != cudaSuccess) return cuda_fail(e, what);
  return KGPU_OK;
}

}  // namespace

extern "C" {

const char* kgpu_last_error(void) { return g_err.c_str(); }
const char* kgpu_version(void) { return "kgpu 0.1 (sm_103a)"; }

kgpu_status kgpu_robot_create(const kgpu_robot_desc* d, kgpu_robot* out)
{
  if (!d || !out) return fail(KGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  int L = d->num_links;
  if (L < 1 || L > KGPU_MAX_LINKS)
    return fail(KGPU_ERR_INVALID, "num_links %d outside [1,%d]", L, KGPU_MAX_LINKS);
  if (!d->parents || !d->joint_types || !d->T0_parent || !d->axes || !d->qmin || !d->qmax ||
      !d->vert_offset || !d->tri_offset)
    return fail(KGPU_ERR_INVALID, "robot description has a null array");
  kgpu_robot R = new (std::nothrow) kgpu_robot_s();
  if (!R) return fail(KGPU_ERR_OOM, "host allocation");
  R->nlinks = L;
  R->parents.assign(d->parents, d->parents + L);
  R->jtypes.assign(d->joint_types, d->joint_types + L);
  R->T0P.assign(d->T0_parent, d->T0_parent + 12 * L);
  R->axes.assign(d->axes, d->axes + 3 * L);
  R->qmin.assign(d->qmin, d->qmin + L);
  R->qmax.assign(d->qmax, d->qmax + L);
  R->margins.assign(L, 0.0);
  if (d->margins) R->margins.assign(d->margins, d->margins + L);
  for (int i = 0; i < L; ++i) {
    const int par = R->parents[i], jt = R->jtypes[i];
    if (par >= i || par < -1) {
      delete R;
      return fail(KGPU_ERR_INVALID, "link %d: parent %d must be -1 or a smaller index", i, par);
    }
    if (jt < 0 || jt > 2) {
      delete R;
      return fail(KGPU_ERR_INVALID, "link %d: joint type %d unknown", i, jt);
    }
    double n2 = R->axes[3 * i] * R->axes[3 * i] + R->axes[3 * i + 1] * R->axes[3 * i + 1] +
                R->axes[3 * i + 2] * R->axes[3 * i + 2];
    if (R->jtypes[i] != KGPU_JOINT_WELD && std::fabs(n2 - 1.0) > 1e-9) {
      delete R;
      return fail(KGPU_ERR_INVALID, "link %d: joint axis is not a unit vector", i);
    }
    if (!(R->qmin[i] <= R->qmax[i]) || R->margins[i] < 0) {
      delete R;
      return fail(KGPU_ERR_INVALID, "link %d: bad joint limits or negative margin", i);
    }
  }
  R->self_mask.assign(L * L, 0);
  for (int i = 0; i < L; ++i)
    for (int j = i + 1; j < L; ++j) {
      if (d->self_mask) R->self_mask[i * L + j] = d->self_mask[i * L + j] ? 1 : 0;
      else R->self_mask[i * L + j] = (R->parents[j] != i && R->parents[i] != j) ? 1 : 0;
    }
  R->bvh.resize(L);
  R->tri64.resize(L);
  R->vert64.resize(L);
  R->link_tri_count.assign(L, 0);
  R->link_r.assign(L, 0.0);
  double reach_link = 0.0;
  for (int l = 0; l < L; ++l) {
    int v0 = d->vert_offset[l], v1 = d->vert_offset[l + 1];
    int t0 = d->tri_offset[l], t1 = d->tri_offset[l + 1];
    if (v1 < v0 || t1 < t0 || (t1 > t0 && (!d->verts || !d->tris))) {
      delete R;
      return fail(KGPU_ERR_INVALID, "link %d: bad mesh offsets", l);
    }
    int nt = t1 - t0, nv = v1 - v0;
    std::vector<double> tri(9 * (size_t)nt);
    for (int t = 0; t < nt; ++t)
      for (int v = 0; v < 3; ++v) {
        int vi = d->tris[3 * (size_t)(t0 + t) + v];
        if (vi < 0 || vi >= nv) {
          delete R;
          return fail(KGPU_ERR_INVALID, "link %d triangle %d: vertex index %d out of range", l, t, vi);
        }
        for (int i = 0; i < 3; ++i) {
          double x = d->verts[3 * (size_t)(v0 + vi) + i];
          if (!std::isfinite(x)) {
            delete R;
            return fail(KGPU_ERR_NOT_FINITE, "link %d: non-finite vertex", l);
          }
          tri[9 * (size_t)t + 3 * v + i] = x;
        }
      }
    double rl = 0.0;
    for (size_t k = 0; k < tri.size(); k += 3) {
      double r = std::sqrt(tri[k] * tri[k] + tri[k + 1] * tri[k + 1] + tri[k + 2] * tri[k + 2]);
      rl = std::max(rl, r);
    }
    reach_link = std::max(reach_link, rl);
    R->link_r[l] = rl;
    std::vector<int> ids(nt);
    for (int t = 0; t < nt; ++t) ids[t] = t;
    build_bvh(tri, ids, nullptr, R->bvh[l]);
    R->tri64[l].resize(9 * (size_t)nt);
    for (int k = 0; k < nt; ++k)
      for (int i = 0; i < 9; ++i) R->tri64[l][9 * (size_t)k + i] = tri[9 * (size_t)R->bvh[l].order[k] + i];
    R->link_tri_count[l] = nt;
    R->vert64[l].assign(d->verts + 3 * (size_t)v0, d->verts + 3 * (size_t)v1);
  }
  double chain = 0.0;
  for (int i = 0; i < L; ++i)
    chain += std::sqrt(R->T0P[12 * i + 9] * R->T0P[12 * i + 9] + R->T0P[12 * i + 10] * R->T0P[12 * i + 10] +
                       R->T0P[12 * i + 11] * R->T0P[12 * i + 11]);
  R->reach = chain + reach_link;
  *out = R;
  return KGPU_OK;
}

kgpu_status kgpu_robot_destroy(kgpu_robot r)
{
  delete r;
  return KGPU_OK;
}

kgpu_status kgpu_env_create(const kgpu_env_desc* d, kgpu_env* out) { return kgpu_env_create_ex(d, 0, out); }

kgpu_status kgpu_env_create_ex(const kgpu_env_desc* d, int32_t flags, kgpu_env* out)
{
  if (!d || !out) return fail(KGPU_ERR_INVALID, "null argument");
  if (flags & ~KGPU_ENV_BUILD_GPU) return fail(KGPU_ERR_INVALID, "unknown environment build flag");
  *out = nullptr;
  int N = d->num_objects;
  if (N < 0 || (N > 0 && (!d->vert_offset || !d->tri_offset)))
    return fail(KGPU_ERR_INVALID, "bad environment description");
  kgpu_env E = new (std::nothrow) kgpu_env_s();
  if (!E) return fail(KGPU_ERR_OOM, "host allocation");
  E->nobj = N;
  E->groups.assign(N, 0);
  if (d->groups) E->groups.assign(d->groups, d->groups + N);
  E->convex.assign(N, 0);
  if (d->convex) E->convex.assign(d->convex, d->convex + N);
  E->margins.assign(N, 0.0);
  if (d->margins) E->margins.assign(d->margins, d->margins + N);
  size_t ntot = N > 0 ? (size_t)d->tri_offset[N] : 0;
  E->tri64.resize(9 * ntot);
  E->tri_obj.resize(ntot);
  for (int o = 0; o < N; ++o) {
    if (E->groups[o] < 0 || E->groups[o] >= kMaxGroups || E->margins[o] < 0) {
      delete E;
      return fail(KGPU_ERR_INVALID, "object %d: bad group or margin", o);
    }
    int v0 = d->vert_offset[o], v1 = d->vert_offset[o + 1];
    int nv = v1 - v0;
    for (int t = d->tri_offset[o]; t < d->tri_offset[o + 1]; ++t) {
      E->tri_obj[t] = o;
      for (int v = 0; v < 3; ++v) {
        int vi = d->tris[3 * (size_t)t + v];
        if (vi < 0 || vi >= nv) {
          delete E;
          return fail(KGPU_ERR_INVALID, "object %d: vertex index out of range", o);
        }
        for (int i = 0; i < 3; ++i) {
          double x = d->verts[3 * ((size_t)v0 + vi) + i];
          if (!std::isfinite(x)) {
            delete E;
            return fail(KGPU_ERR_NOT_FINITE, "object %d: non-finite vertex", o);
          }
          E->tri64[9 * (size_t)t + 3 * v + i] = x;
          E->extent = std::max(E->extent, std::fabs(x));
        }
      }
    }
  }
  // per-group object-aware trees, concatenated
  std::vector<KNode> nodes;
  std::vector<double> node64;
  std::vector<int> node_obj, leaf_tris;
  std::vector<int> obj_root(N, -1);
  for (int g = 0; g < kMaxGroups; ++g) {
    E->group_root[g] = -1;
    E->group_margin[g] = 0.f;
    std::vector<int> ids;
    double gm = 0.0;
    for (int o = 0; o < N; ++o)
      if (E->groups[o] == g) {
        gm = std::max(gm, E->margins[o]);
        for (int t = d->tri_offset[o]; t < d->tri_offset[o + 1]; ++t) ids.push_back(t);
      }
    if (ids.empty()) continue;
    HostBvh& b = E->gbvh[g];
    if (flags & KGPU_ENV_BUILD_GPU) {
      cudaError_t be = lbvh_build(E->tri64, ids, E->tri_obj, b);
      if (be != cudaSuccess) {
        delete E;
        return cuda_fail(be, "environment tree build on the GPU");
      }
    } else {
      build_bvh(E->tri64, ids, &E->tri_obj, b);
    }
    int node_base = (int)nodes.size(), tri_base = (int)leaf_tris.size();
    append_bvh(b, node_base, tri_base, nodes, node64);
    for (size_t k = 0; k < b.nodes.size(); ++k) {
      int o = b.node_obj[k];
      node_obj.push_back(o);
      // the first (shallowest) node owned by an object is its root: nodes are
      // appended parent-before-child, so the first occurrence wins
      if (o >= 0 && obj_root[o] < 0) obj_root[o] = node_base + (int)k;
    }
    for (int t : b.order) leaf_tris.push_back(t);
    E->group_root[g] = node_base;
    E->group_margin[g] = round_up_f(gm);
  }
  // breadth-first order from the group roots: the top levels of every group
  // tree, which every traversal visits, share the first cache lines of the
  // array; siblings stay adjacent
  {
    const size_t nn = nodes.size();
    std::vector<int> order, perm(nn, -1);
    order.reserve(nn);
    for (int g = 0; g < kMaxGroups; ++g)
      if (E->group_root[g] >= 0) order.push_back(E->group_root[g]);
    for (size_t h = 0; h < order.size(); ++h) {
      const KNode& n = nodes[order[h]];
      if (as_int(n.b.w) == 0) {  // internal: children c, c + 1
        order.push_back(as_int(n.a.w));
        order.push_back(as_int(n.a.w) + 1);
      }
    }
    if (order.size() != nn) {
      delete E;
      return fail(KGPU_ERR_INVALID, "environment tree layout: %zu of %zu nodes reachable", order.size(), nn);
    }
    for (size_t k = 0; k < nn; ++k) perm[order[k]] = (int)k;
    std::vector<KNode> n2(nn);
    std::vector<double> n64(6 * nn);
    std::vector<int> nobj(nn);
    for (size_t k = 0; k < nn; ++k) {
      KNode n = nodes[order[k]];
      if (as_int(n.b.w) == 0) n.a.w = as_float(perm[as_int(n.a.w)]);
      n2[k] = n;
      for (int i = 0; i < 6; ++i) n64[6 * k + i] = node64[6 * (size_t)order[k] + i];
      nobj[k] = node_obj[order[k]];
    }
    nodes.swap(n2);
    node64.swap(n64);
    node_obj.swap(nobj);
    for (int g = 0; g < kMaxGroups; ++g)
      if (E->group_root[g] >= 0) E->group_root[g] = perm[E->group_root[g]];
    for (int o = 0; o < N; ++o)
      if (obj_root[o] >= 0) obj_root[o] = perm[obj_root[o]];
  }
  E->n_nodes = nodes.size();
  E->n_tris = leaf_tris.size();
  std::vector<float4> tri32(3 * leaf_tris.size());
  std::vector<double> tri64l(9 * leaf_tris.size());
  std::vector<int> tobj(leaf_tris.size());
  // canonical FP64 face planes (unit outward normal n = e0 x e1 / |.|, and
  // n . a with a the first vertex), as the oracle computes them, in leaf order
  std::vector<double> face64(4 * leaf_tris.size());
  std::vector<float4> face32(leaf_tris.size());
  std::vector<int> obj_leaf_first(N, -1), obj_leaf_count(N, 0);
  for (size_t k = 0; k < leaf_tris.size(); ++k) {
    const double* F = &E->tri64[9 * (size_t)leaf_tris[k]];
    double e0[3], e1[3], c[3], n[3];
    kx_sub3(F + 3, F, e0);
    kx_sub3(F + 6, F, e1);
    kx_cross3(e0, e1, c);
    double len = kx_sqrt(kx_dot3(c, c));
    for (int i = 0; i < 3; ++i) n[i] = kx_div(c[i], len);
    double top = kx_dot3(n, F);
    for (int i = 0; i < 3; ++i) face64[4 * k + i] = n[i];
    face64[4 * k + 3] = top;
    face32[k] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)top);
    int o = E->tri_obj[leaf_tris[k]];
    if (obj_leaf_first[o] < 0) obj_leaf_first[o] = (int)k;
    obj_leaf_count[o]++;
  }
  for (size_t k = 0; k < leaf_tris.size(); ++k) {
    int t = leaf_tris[k];
    for (int v = 0; v < 3; ++v)
      tri32[3 * k + v] = make_float4((float)E->tri64[9 * (size_t)t + 3 * v], (float)E->tri64[9 * (size_t)t + 3 * v + 1],
                                     (float)E->tri64[9 * (size_t)t + 3 * v + 2], 0.f);
    for (int i = 0; i < 9; ++i) tri64l[9 * k + i] = E->tri64[9 * (size_t)t + i];
    tobj[k] = E->tri_obj[t];
  }
  std::vector<float> om(N);
  std::vector<double> om64(N);
  for (int o = 0; o < N; ++o) {
    om[o] = round_up_f(E->margins[o]);
    om64[o] = E->margins[o];
  }
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = upload(&E->d_nodes, nodes.data(), nodes.size());
  if (e == cudaSuccess) e = upload(&E->d_node64, node64.data(), node64.size());
  if (e == cudaSuccess) e = upload(&E->d_tri32, tri32.data(), tri32.size());
  if (e == cudaSuccess) e = upload(&E->d_tri64, tri64l.data(), tri64l.size());
  if (e == cudaSuccess) e = upload(&E->d_tri_obj, tobj.data(), tobj.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_margin, om.data(), om.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_margin64, om64.data(), om64.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_root, obj_root.data(), obj_root.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_group, E->groups.data(), E->groups.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_convex, E->convex.data(), E->convex.size());
  if (e == cudaSuccess) e = upload(&E->d_node_obj, node_obj.data(), node_obj.size());
  if (e == cudaSuccess) e = upload(&E->d_tri_orig, leaf_tris.data(), leaf_tris.size());
  if (e == cudaSuccess) e = upload(&E->d_face64, face64.data(), face64.size());
  if (e == cudaSuccess) e = upload(&E->d_face32, face32.data(), face32.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_leaf_first, obj_leaf_first.data(), obj_leaf_first.size());
  if (e == cudaSuccess) e = upload(&E->d_obj_leaf_count, obj_leaf_count.data(), obj_leaf_count.size());
  if (e == cudaSuccess && N > 0) e = upload(&E->d_obj_tri_first, d->tri_offset, (size_t)N);
  if (e != cudaSuccess) {
    kgpu_env_destroy(E);
    return cuda_fail(e, "environment upload");
  }
  *out = E;
  return KGPU_OK;
}

kgpu_status kgpu_env_destroy(kgpu_env E)
{
  if (!E) return KGPU_OK;
  dfree(E->d_nodes);
  dfree(E->d_node64);
  dfree(E->d_tri32);
  dfree(E->d_tri64);
  dfree(E->d_tri_obj);
  dfree(E->d_obj_margin);
  dfree(E->d_obj_margin64);
  dfree(E->d_obj_root);
  dfree(E->d_obj_group);
  dfree(E->d_obj_convex);
  dfree(E->d_node_obj);
  dfree(E->d_tri_orig);
  dfree(E->d_face64);
  dfree(E->d_face32);
  dfree(E->d_obj_leaf_first);
  dfree(E->d_obj_tri_first);
  dfree(E->d_obj_leaf_count);
  delete E;
  return KGPU_OK;
}

kgpu_status kgpu_world_create(kgpu_env env, const kgpu_robot* robots, int32_t n, kgpu_world* out)
{
  if (!out || n < 0 || (n > 0 && !robots)) return fail(KGPU_ERR_INVALID, "bad arguments");
  *out = nullptr;
  for (int r = 0; r < n; ++r)
    if (!robots[r]) return fail(KGPU_ERR_INVALID, "null robot %d", r);
  kgpu_world w = new (std::nothrow) kgpu_world_s();
  if (!w) return fail(KGPU_ERR_OOM, "host allocation");
  w->env = env;
  w->robots.assign(robots, robots + n);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&w->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = engine_init();
  if (e == cudaSuccess) e = dist_init();
  if (e == cudaSuccess) e = noalloc_prepare();  // kgpu_check_edges_noalloc's array, loaded now
  if (e != cudaSuccess) {
    delete w;
    return cuda_fail(e, "device query");
  }
  // link BVHs of every robot, concatenated
  std::vector<KNode> nodes;
  std::vector<double> node64, tri64, lvert64;
  std::vector<float4> tri32, lvert32;
  std::vector<int> ltri_orig;
  std::vector<float> lnode_r;
  double reach = 0.0;
  for (int r = 0; r < n; ++r) {
    kgpu_robot R = robots[r];
    w->robot_node_base.push_back((int)nodes.size());
    w->robot_tri_base.push_back((int)(tri32.size() / 3));
    w->robot_vert_base.push_back((int)lvert32.size());
    for (int l = 0; l < R->nlinks; ++l) {
      append_bvh(R->bvh[l], (int)nodes.size(), (int)(tri32.size() / 3), nodes, node64, &lnode_r);
      for (size_t k = 0; k < R->tri64[l].size(); k += 3)
        tri32.push_back(make_float4((float)R->tri64[l][k], (float)R->tri64[l][k + 1], (float)R->tri64[l][k + 2], 0.f));
      tri64.insert(tri64.end(), R->tri64[l].begin(), R->tri64[l].end());
      for (int t : R->bvh[l].order) ltri_orig.push_back(t);
      for (size_t k = 0; k < R->vert64[l].size(); k += 3) {
        lvert32.push_back(make_float4((float)R->vert64[l][k], (float)R->vert64[l][k + 1],
                                      (float)R->vert64[l][k + 2], 0.f));
        lvert64.insert(lvert64.end(), R->vert64[l].begin() + k, R->vert64[l].begin() + k + 3);
      }
    }
    reach = std::max(reach, R->reach);
    std::vector<uint32_t> mask(R->nlinks, 0xffffffffu);
    for (int l = 0; l < R->nlinks; ++l)
      if (R->parents[l] < 0) mask[l] &= ~(1u << KGPU_GROUP_TERRAIN);
    w->env_mask.push_back(mask);
    w->self_enabled.push_back(R->self_mask);
  }
  if (nodes.size() >= (1u << 20) || tri32.size() / 3 >= (1u << 28)) {
    delete w;
    return fail(KGPU_ERR_UNSUPPORTED, "link BVHs exceed 2^20 nodes");
  }
  if (nodes.empty()) nodes.push_back(KNode());
  if (tri32.empty()) tri32.resize(3);
  if (tri64.empty()) tri64.resize(9);
  if (node64.empty()) node64.resize(6);
  if (lnode_r.empty()) lnode_r.resize(1);
  if (ltri_orig.empty()) ltri_orig.resize(1);
  if (lvert32.empty()) lvert32.resize(1);
  if (lvert64.empty()) lvert64.resize(3);
  e = cudaSuccess;
  if (e == cudaSuccess) e = upload(&w->d_lnodes, nodes.data(), nodes.size());
  if (e == cudaSuccess) e = upload(&w->d_lnode64, node64.data(), node64.size());
  if (e == cudaSuccess) e = upload(&w->d_lnode_r, lnode_r.data(), lnode_r.size());
  if (e == cudaSuccess) e = upload(&w->d_ltri32, tri32.data(), tri32.size());
  if (e == cudaSuccess) e = upload(&w->d_ltri64, tri64.data(), tri64.size());
  if (e == cudaSuccess) e = upload(&w->d_ltri_orig, ltri_orig.data(), ltri_orig.size());
  if (e == cudaSuccess) e = upload(&w->d_lvert32, lvert32.data(), lvert32.size());
  if (e == cudaSuccess) e = upload(&w->d_lvert64, lvert64.data(), lvert64.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(w->d_status, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->d_stats, 16 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(w->d_stats, 0, 16 * sizeof(unsigned long long));
  // scratch: per-warp spill stacks, queue heads, edge ordering tables
  Scratch& S = w->scratch;
  S.max_warps = w->num_sms * 4 * engine_warps_per_block();  // up to 4 blocks per SM
  S.spill_per_warp = 8192;
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.spill, (size_t)S.max_warps * S.spill_per_warp * sizeof(uint2));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.counters, 64 * sizeof(unsigned int));
  S.pend_cap = 1 << 18;
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.pend, (size_t)S.pend_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.edge_hist, (kMaxSteps + 2) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.edge_round_off, (kMaxSteps + 2) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&S.edge_meta, (4 + 2 * (kMaxSteps + 2)) * sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w->host_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    free_world_device(w);
    delete w;
    return cuda_fail(e, "world allocation");
  }
  // environment coordinates are FP64 rounded to FP32 once: a vertex moves by
  // at most u/2 * |x|_2 <= u * extent (the per-link bounds come from the
  // kernels' running error analysis)
  w->eps_env = env ? 5.9604644775390625e-08 * 2.0 * (env->extent + 1e-3) : 0.0;
  w->eps_extra = 0.0;
  KWorldDev& D = w->dev;
  memset(&D, 0, sizeof D);
  D.lnodes = w->d_lnodes;
  D.ltri32 = w->d_ltri32;
  D.ltri64 = w->d_ltri64;
  D.ltri_orig = w->d_ltri_orig;
  D.lvert32 = w->d_lvert32;
  D.lvert64 = w->d_lvert64;
  D.lnode64 = w->d_lnode64;
  D.lnode_r = w->d_lnode_r;
  if (env) {
    D.enodes = env->d_nodes;
    D.etri32 = env->d_tri32;
    D.etri64 = env->d_tri64;
    D.enode64 = env->d_node64;
    D.etri_obj = env->d_tri_obj;
    D.obj_margin = env->d_obj_margin;
    D.obj_margin64 = env->d_obj_margin64;
    D.obj_root = env->d_obj_root;
    D.obj_group = env->d_obj_group;
    D.obj_convex = env->d_obj_convex;
    D.node_obj = env->d_node_obj;
    D.etri_orig = env->d_tri_orig;
    D.eface32 = env->d_face32;
    D.eface64 = env->d_face64;
    D.obj_leaf_first = env->d_obj_leaf_first;
    D.obj_leaf_count = env->d_obj_leaf_count;
    D.obj_tri_first = env->d_obj_tri_first;
    D.num_objects = env->nobj;
    D.env_nodes = (int)env->n_nodes;
    for (int g = 0; g < kMaxGroups; ++g) {
      D.group_root[g] = env->group_root[g];
      D.group_margin[g] = env->group_margin[g];
    }
  } else {
    for (int g = 0; g < kMaxGroups; ++g) D.group_root[g] = -1;
  }
  D.eps_env = round_up_f(w->eps_env);
  D.eps_extra = 0.f;
  D.status = w->d_status;
  D.stats = w->d_stats;
  w->tables_dirty = true;
  kgpu_status st = refresh_tables(w);
  if (st != KGPU_OK) {
    free_world_device(w);
    delete w;
    return st;
  }
  *out = w;
  return KGPU_OK;
}

kgpu_status kgpu_world_destroy(kgpu_world w)
{
  if (!w) return KGPU_OK;
  free_world_device(w);
  delete w;
  return KGPU_OK;
}

kgpu_status kgpu_world_set_link_env_mask(kgpu_world w, int32_t robot, int32_t link, uint32_t mask)
{
  if (!w || robot < 0 || robot >= (int)w->robots.size()) return fail(KGPU_ERR_INVALID, "bad robot");
  if (link < 0 || link >= w->robots[robot]->nlinks) return fail(KGPU_ERR_INVALID, "bad link %d", link);
  w->env_mask[robot][link] = mask;
  w->tables_dirty = true;
  return KGPU_OK;
}

kgpu_status kgpu_world_enable_self_pair(kgpu_world w, int32_t robot, int32_t i, int32_t j,
                                        int32_t enabled)
{
  if (!w || robot < 0 || robot >= (int)w->robots.size()) return fail(KGPU_ERR_INVALID, "bad robot");
  int L = w->robots[robot]->nlinks;
  if (i < 0 || j < 0 || i >= L || j >= L || i == j) return fail(KGPU_ERR_INVALID, "bad link pair");
  if (i > j) std::swap(i, j);
  w->self_enabled[robot][i * L + j] = enabled ? 1 : 0;
  w->tables_dirty = true;
  return KGPU_OK;
}

kgpu_status kgpu_world_set_option(kgpu_world w, const char* name, double v)
{
  if (!w || !name) return fail(KGPU_ERR_INVALID, "null argument");
  if (!strcmp(name, "eps_extra")) {
    if (!(v >= 0 && v < 1)) return fail(KGPU_ERR_INVALID, "eps_extra must be in [0,1)");
    w->eps_extra = v;
    w->dev.eps_extra = round_up_f(v);
    w->tables_dirty = true;
  } else if (!strcmp(name, "blocks_per_sm")) {
    int k = (int)v;
    if (k < 2 || k > 4) return fail(KGPU_ERR_INVALID, "blocks_per_sm must be 2, 3 or 4");
    w->blocks_per_sm = k;
  } else if (!strcmp(name, "grab")) {
    int k = (int)v;
    if (k < 1 || k > 16) return fail(KGPU_ERR_INVALID, "grab must be in [1,16]");
    w->grab = k;
  } else if (!strcmp(name, "job_flush")) {
    int k = (int)v;
    if (k < 8 || k > 64) return fail(KGPU_ERR_INVALID, "job_flush must be in [8,64]");
    w->job_flush = k;
  } else if (!strcmp(name, "fp64_inline")) {
    int k = (int)v;
    if (k < -1 || k > 1) return fail(KGPU_ERR_INVALID, "fp64_inline must be -1, 0 or 1");
    w->fp64_inline = k;
  } else if (!strcmp(name, "edge_chunk")) {
    int k = (int)v;
    if (k < 1 || k > 64) return fail(KGPU_ERR_INVALID, "edge_chunk must be in [1,64]");
    w->edge_chunk = k;
  } else if (!strcmp(name, "pend_cap")) {
    if (!(v >= 0 && v <= 1e9)) return fail(KGPU_ERR_INVALID, "pend_cap must be in [0, 1e9] (0: no cap)");
    w->pend_cap_opt = (int)v;
  } else if (!strcmp(name, "spill_cap")) {
    if (!(v >= 0 && v <= 1e9)) return fail(KGPU_ERR_INVALID, "spill_cap must be in [0, 1e9] (0: no cap)");
    w->spill_cap_opt = (int)v;
  } else if (!strcmp(name, "stage_nodes")) {
    if (!(v >= 0 && v <= 1024)) return fail(KGPU_ERR_INVALID, "stage_nodes must be in [0, 1024]");
    w->stage_nodes = (int)v;
  } else if (!strcmp(name, "share_wait_polls")) {
    if (!(v >= 0 && v <= (double)(1 << 20))) return fail(KGPU_ERR_INVALID, "share_wait_polls must be in [0, 2^20]");
    w->dev.share_wait = (int)v;
    w->tables_dirty = true;
  } else if (!strcmp(name, "share_no_release")) {
    if (v != 0 && v != 1) return fail(KGPU_ERR_INVALID, "share_no_release must be 0 or 1");
    w->dev.share_no_release = (int)v;
    w->tables_dirty = true;
  } else {
    return fail(KGPU_ERR_INVALID, "unknown option '%s'", name);
  }
  if (w->num_sms * w->blocks_per_sm * engine_warps_per_block() > w->scratch.max_warps)
    return fail(KGPU_ERR_INVALID, "launch shape exceeds the scratch sized at creation");
  return KGPU_OK;
}

kgpu_status kgpu_world_get_option(kgpu_world w, const char* name, double* v)
{
  if (!w || !name || !v) return fail(KGPU_ERR_INVALID, "null argument");
  if (!strcmp(name, "eps_extra")) *v = w->eps_extra;
  else if (!strcmp(name, "eps_env")) *v = w->eps_env;
  else if (!strcmp(name, "warps_per_block")) *v = engine_warps_per_block();
  else if (!strcmp(name, "blocks_per_sm")) *v = w->blocks_per_sm;
  else if (!strcmp(name, "grab")) *v = w->grab;
  else if (!strcmp(name, "job_flush")) *v = w->job_flush;
  else if (!strcmp(name, "edge_chunk")) *v = w->edge_chunk;
  else if (!strcmp(name, "fp64_inline")) *v = w->fp64_inline;
  else if (!strcmp(name, "num_sms")) *v = w->num_sms;
  else if (!strcmp(name, "pend_cap")) *v = w->pend_cap_opt;
  else if (!strcmp(name, "spill_cap")) *v = w->spill_cap_opt;
  else if (!strcmp(name, "stage_nodes")) *v = w->stage_nodes;
  else if (!strcmp(name, "share_wait_polls")) *v = w->dev.share_wait;
  else if (!strcmp(name, "share_no_release")) *v = w->dev.share_no_release;
  else return fail(KGPU_ERR_INVALID, "unknown option '%s'", name);
  return KGPU_OK;
}

// The status word a sync read: 0, or the code the kernels set (then cleared
// on the device and reported with its message).
static kgpu_status status_result(kgpu_world w, int st)
{
  if (st != 0) {
    CK(cudaMemset(w->d_status, 0, sizeof(int)));
    const char* what = st == KGPU_ERR_NOT_FINITE ? "non-finite or out-of-range configuration value"
                       : st == KGPU_ERR_OVERFLOW ? "traversal stack spill area exhausted"
                       : st == KGPU_ERR_INVALID  ? "invalid step count (must be 1..65535)"
                       : st == KGPU_ERR_TIMEOUT  ? "bounded device wait ran out"
                                                 : "device error";
    return fail(st, "device status: %s", what);
  }
  return KGPU_OK;
}

kgpu_status kgpu_world_sync(kgpu_world w, kgpu_stream stream)
{
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  int st = 0;
  CK(cudaMemcpy(&st, w->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  return status_result(w, st);
}

// kgpu_world_sync for the host-buffer calls: the status word is copied into
// pinned memory on the call's stream behind its results, so that one wait
// returns both
static kgpu_status sync_status_pinned(kgpu_world w, cudaStream_t s, int* pinned_status)
{
  CK(cudaMemcpyAsync(pinned_status, w->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return status_result(w, *pinned_status);
}

kgpu_status kgpu_world_get_stats(kgpu_world w, kgpu_stats* out)
{
  if (!w || !out) return fail(KGPU_ERR_INVALID, "null argument");
  unsigned long long s[16];
  CK(cudaMemcpy(s, w->d_stats, sizeof s, cudaMemcpyDeviceToHost));
  out->items = s[0];
  out->node_pairs = s[1];
  out->tri_pairs = s[2];
  out->band_pairs = s[3];
  out->spills = s[4];
  out->certified = s[5];
  out->fp64_hits = s[6];
  out->dist_pairs = s[8];
  out->dist_node_pairs = s[9];
  out->dist_tri_pairs = s[10];
  out->dist_fp64 = s[11];
  return KGPU_OK;
}

kgpu_status kgpu_world_reset_stats(kgpu_world w)
{
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  CK(cudaMemset(w->d_stats, 0, 16 * sizeof(unsigned long long)));
  return KGPU_OK;
}

kgpu_status kgpu_fk(kgpu_world w, int32_t robot, const float* q, int32_t B, float* T, float* err,
                    kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !T))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_fk(w->d_dev, robot, q, B, T, err, (cudaStream_t)s), "kgpu_fk");
}

kgpu_status kgpu_fk64(kgpu_world w, int32_t robot, const float* q, int32_t B, double* T, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !T))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_fk64(w->d_dev, robot, q, B, T, (cudaStream_t)s), "kgpu_fk64");
}

kgpu_status kgpu_check_configs(kgpu_world w, int32_t robot, const float* q, int32_t B,
                               uint8_t* env_hit, uint8_t* self_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && !q)) return fail(KGPU_ERR_INVALID, "bad buffers");
  if (!env_hit && !self_hit) return KGPU_OK;
  return launch_status(launch_check_configs(w->d_dev, engine_scratch(w, w->scratch), robot, nullptr, q, w->robots[robot]->nlinks, B,
                                            env_hit, self_hit, nullptr, grid_blocks(w), w->blocks_per_sm,
                                            (cudaStream_t)s, w->grab, w->job_flush, w->fp64_inline),
                       "kgpu_check_configs");
}

kgpu_status kgpu_check_configs_multi(kgpu_world w, const int32_t* robot_ids, const float* q,
                                     int32_t q_stride, int32_t B, uint8_t* env_hit, uint8_t* self_hit,
                                     kgpu_stream s)
{
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  kgpu_status st = refresh_tables(w);
  if (st) return st;
  int maxl = 0;
  for (auto R : w->robots) maxl = std::max(maxl, R->nlinks);
  if (B < 0 || (B > 0 && (!q || !robot_ids)) || q_stride < maxl)
    return fail(KGPU_ERR_INVALID, "bad buffers or q_stride %d < max links %d", q_stride, maxl);
  if (!env_hit && !self_hit) return KGPU_OK;
  // the edge permutation buffer holds the robot-sorted order (grown on demand)
  st = ensure_edge_scratch(w, B);
  if (st) return st;
  return launch_status(launch_check_configs(w->d_dev, engine_scratch(w, w->scratch), -1, robot_ids, q, q_stride, B, env_hit, self_hit,
                                            nullptr, grid_blocks(w), w->blocks_per_sm, (cudaStream_t)s, w->grab,
                                            w->job_flush, w->fp64_inline, (int)w->robots.size(), w->d_status),
                       "kgpu_check_configs_multi");
}

kgpu_status kgpu_is_feasible(kgpu_world w, int32_t robot, const float* q, int32_t B, uint8_t* feasible,
                             kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !feasible))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_check_configs(w->d_dev, engine_scratch(w, w->scratch), robot, nullptr, q, w->robots[robot]->nlinks, B,
                                            nullptr, nullptr, feasible, grid_blocks(w), w->blocks_per_sm,
                                            (cudaStream_t)s, w->grab, w->job_flush, w->fp64_inline),
                       "kgpu_is_feasible");
}

kgpu_status kgpu_check_edges(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                             const int32_t* nsteps, int32_t E, int32_t* first_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E < 0 || (E > 0 && (!qa || !qb || !nsteps || !first_hit))) return fail(KGPU_ERR_INVALID, "bad buffers");
  if ((st = ensure_edge_scratch(w, E))) return st;
  return launch_status(launch_check_edges(w->d_dev, w->d_status, engine_scratch(w, w->scratch), robot, qa, qb, nsteps, E, first_hit, grid_blocks(w),
                                          w->blocks_per_sm, (cudaStream_t)s, w->grab, w->job_flush, w->edge_chunk,
                                          w->fp64_inline),
                       "kgpu_check_edges");
}

kgpu_status kgpu_check_configs_plain64(kgpu_world w, int32_t robot, const float* q, int32_t B,
                                       uint8_t* env_hit, uint8_t* self_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && !q)) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_plain64_configs(w->dev, robot, q, B, env_hit, self_hit, (cudaStream_t)s),
                       "kgpu_check_configs_plain64");
}

kgpu_status kgpu_check_edges_plain64(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                     const int32_t* nsteps, int32_t E, int32_t* first_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E < 0 || (E > 0 && (!qa || !qb || !nsteps || !first_hit))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_plain64_edges(w->dev, robot, qa, qb, nsteps, E, first_hit, (cudaStream_t)s),
                       "kgpu_check_edges_plain64");
}

kgpu_status kgpu_check_edges_plain64_steps(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                           const int32_t* nsteps, int32_t E, int32_t* first_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E < 0 || E == INT32_MAX || (E > 0 && (!qa || !qb || !nsteps || !first_hit)))
    return fail(KGPU_ERR_INVALID, "bad buffers");
  if ((st = ensure_edge_scratch(w, E + 1))) return st;  // the step offsets
  return launch_status(launch_plain64_edge_steps(w->dev, robot, qa, qb, nsteps, E, first_hit, w->scratch.edge_perm,
                                                 w->num_sms, (cudaStream_t)s),
                       "kgpu_check_edges_plain64_steps");
}

kgpu_status kgpu_check_edges_plain64_pairs(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                           const int32_t* nsteps, int32_t E, int32_t* first_hit, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E < 0 || E == INT32_MAX || (E > 0 && (!qa || !qb || !nsteps || !first_hit)))
    return fail(KGPU_ERR_INVALID, "bad buffers");
  if ((st = ensure_edge_scratch(w, E + 1))) return st;  // the step offsets
  return launch_status(launch_plain64_edge_pairs(w->dev, robot, qa, qb, nsteps, E, first_hit, w->scratch.edge_perm,
                                                 w->num_sms, (cudaStream_t)s),
                       "kgpu_check_edges_plain64_pairs");
}

kgpu_status kgpu_distance(kgpu_world w, int32_t robot, const float* q, int32_t B, double cutoff, double* d,
                          int32_t* pair, double* cp, float* grad, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !d || !pair || !cp))) return fail(KGPU_ERR_INVALID, "bad buffers");
  if (!(cutoff > 0) || !(cutoff < 1e30)) return fail(KGPU_ERR_INVALID, "cutoff must be positive and finite");
  if (!w->env) return fail(KGPU_ERR_EMPTY, "distance query without an environment (robotsim.cpp:1786-1787)");
  return launch_status(launch_distance(w->d_dev, w->scratch, robot, q, B, cutoff, d, pair, cp, grad, w->num_sms,
                                       (cudaStream_t)s),
                       "kgpu_distance");
}

kgpu_status kgpu_self_distance(kgpu_world w, int32_t robot, const float* q, int32_t B, double cutoff, double* d,
                               int32_t* pair, double* cp, float* grad, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !d || !pair || !cp))) return fail(KGPU_ERR_INVALID, "bad buffers");
  if (!(cutoff > 0) || !(cutoff < 1e30)) return fail(KGPU_ERR_INVALID, "cutoff must be positive and finite");
  return launch_status(launch_self_distance(w->d_dev, robot, q, B, cutoff, d, pair, cp, grad, nullptr, 0, w->num_sms,
                                            (cudaStream_t)s),
                       "kgpu_self_distance");
}

kgpu_status kgpu_self_pair_distances(kgpu_world w, int32_t robot, const float* q, int32_t B, double cutoff,
                                     int32_t all_pairs, double* dpair, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (!(cutoff > 0) || !(cutoff < 1e30)) return fail(KGPU_ERR_INVALID, "cutoff must be positive and finite");
  if (w->robots[robot]->nlinks < 2) return B < 0 ? fail(KGPU_ERR_INVALID, "bad buffers") : KGPU_OK;  // no pairs
  if (B < 0 || (B > 0 && (!q || !dpair))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(launch_self_distance(w->d_dev, robot, q, B, cutoff, nullptr, nullptr, nullptr, nullptr, dpair,
                                            all_pairs, w->num_sms, (cudaStream_t)s),
                       "kgpu_self_pair_distances");
}

kgpu_status kgpu_softmin_grad(kgpu_world w, int32_t robot, const float* q, int32_t T, int32_t Wn, double tau,
                              double* L, float* dLdq, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (T < 0 || Wn < 1 || (T > 0 && (!q || !L))) return fail(KGPU_ERR_INVALID, "bad buffers");
  if (!(tau > 0)) return fail(KGPU_ERR_INVALID, "tau must be positive");
  if (!w->env) return fail(KGPU_ERR_EMPTY, "distance query without an environment (robotsim.cpp:1786-1787)");
  size_t need = 2 * (size_t)T * Wn + T;
  if (need > w->scratch.dist_work_cap) {
    dfree(w->scratch.dist_work);
    w->scratch.dist_work_cap = 0;
    CK(cudaMalloc((void**)&w->scratch.dist_work, need * sizeof(double)));
    w->scratch.dist_work_cap = need;
  }
  return launch_status(launch_softmin(w->d_dev, w->scratch, robot, q, T, Wn, tau, L, dLdq, w->robots[robot]->nlinks,
                                      w->scratch.dist_work, w->num_sms, (cudaStream_t)s),
                       "kgpu_softmin_grad");
}

kgpu_status kgpu_ik_solve(kgpu_world w, int32_t robot, int32_t B, float* q, const int32_t* links, int32_t link,
                          const float* plocal, const float* ptarget, const float* Rtarget, int32_t max_iters,
                          float tol, uint8_t* ok, float* residual, int32_t* iters, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !plocal || !ptarget || !ok || !residual)))
    return fail(KGPU_ERR_INVALID, "bad buffers");
  const int nl = w->robots[robot]->nlinks;
  if (!links && (link < 0 || link >= nl)) return fail(KGPU_ERR_INVALID, "link %d out of range [0,%d)", link, nl);
  if (max_iters < 0 || !(tol > 0)) return fail(KGPU_ERR_INVALID, "max_iters must be >= 0 and tol > 0");
  return launch_status(launch_ik(w->d_dev, robot, B, q, links, link, plocal, ptarget, Rtarget, max_iters, tol, ok,
                                 residual, iters, (cudaStream_t)s),
                       "kgpu_ik_solve");
}

kgpu_status kgpu_self_collision_pairs(kgpu_world w, int32_t robot, const float* q, int32_t B, uint32_t* pair_mask,
                                      kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !pair_mask))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(
      launch_self_pairs(w->d_dev, w->scratch, robot, q, B, nullptr, pair_mask, w->num_sms, (cudaStream_t)s),
      "kgpu_self_collision_pairs");
}

kgpu_status kgpu_independent_self_collision_pairs(kgpu_world w, int32_t robot, const float* q, int32_t B,
                                                  const uint32_t* candidates, uint32_t* pair_mask, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !candidates || !pair_mask))) return fail(KGPU_ERR_INVALID, "bad buffers");
  return launch_status(
      launch_self_pairs(w->d_dev, w->scratch, robot, q, B, candidates, pair_mask, w->num_sms, (cudaStream_t)s),
      "kgpu_independent_self_collision_pairs");
}

kgpu_status kgpu_jacobian(kgpu_world w, int32_t robot, const float* q, int32_t B, const int32_t* links,
                          int32_t link, const float* plocal, float* J, kgpu_stream s)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && (!q || !plocal || !J))) return fail(KGPU_ERR_INVALID, "bad buffers");
  const int nl = w->robots[robot]->nlinks;
  if (!links && (link < 0 || link >= nl)) return fail(KGPU_ERR_INVALID, "link %d out of range [0,%d)", link, nl);
  return launch_status(launch_jacobian(w->d_dev, robot, q, links, link, plocal, B, J, (cudaStream_t)s),
                       "kgpu_jacobian");
}

kgpu_status kgpu_raycast(kgpu_world w, const float* s, const float* d, int32_t R, int32_t* obj, int32_t* tri,
                         double* t, double* point, kgpu_stream st)
{
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  if (R < 0 || (R > 0 && (!s || !d || !obj || !tri || !t || !point))) return fail(KGPU_ERR_INVALID, "bad buffers");
  kgpu_status e = refresh_tables(w);
  if (e) return e;
  return launch_status(launch_raycast(w->d_dev, s, d, R, obj, tri, t, point, (cudaStream_t)st), "kgpu_raycast");
}

// ---- host-buffer variants ----------------------------------------------------
static kgpu_status ensure_stage(kgpu_world w, size_t bytes)
{
  if (bytes <= w->pinned_bytes && bytes <= w->dstage_bytes) return KGPU_OK;
  size_t cap = bytes < ((size_t)1 << 20) ? ((size_t)1 << 20) : bytes;
  if (w->pinned) cudaFreeHost(w->pinned);
  w->pinned = nullptr;
  w->pinned_bytes = 0;
  dfree(w->dstage);
  w->dstage_bytes = 0;
  CK(cudaMallocHost(&w->pinned, cap));
  w->pinned_bytes = cap;
  CK(cudaMalloc(&w->dstage, cap));
  w->dstage_bytes = cap;
  return KGPU_OK;
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

kgpu_status kgpu_check_configs_host(kgpu_world w, int32_t robot, const float* q, int32_t B, uint8_t* env_hit,
                                    uint8_t* self_hit)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (B < 0 || (B > 0 && !q)) return fail(KGPU_ERR_INVALID, "bad buffers");
  int L = w->robots[robot]->nlinks;
  size_t qb = al((size_t)B * L * sizeof(float)), ob = al((size_t)B);
  if ((st = ensure_stage(w, qb + 2 * ob + al(sizeof(int))))) return st;
  char* hp = (char*)w->pinned;
  char* dp = (char*)w->dstage;
  cudaStream_t s = w->host_stream;
  memcpy(hp, q, (size_t)B * L * sizeof(float));
  CK(cudaMemcpyAsync(dp, hp, (size_t)B * L * sizeof(float), cudaMemcpyHostToDevice, s));
  st = kgpu_check_configs(w, robot, (const float*)dp, B, env_hit ? (uint8_t*)(dp + qb) : nullptr,
                          self_hit ? (uint8_t*)(dp + qb + ob) : nullptr, s);
  if (st) return st;
  if (env_hit) CK(cudaMemcpyAsync(hp + qb, dp + qb, B, cudaMemcpyDeviceToHost, s));
  if (self_hit) CK(cudaMemcpyAsync(hp + qb + ob, dp + qb + ob, B, cudaMemcpyDeviceToHost, s));
  if ((st = sync_status_pinned(w, s, (int*)(hp + qb + 2 * ob)))) return st;
  if (env_hit) memcpy(env_hit, hp + qb, B);
  if (self_hit) memcpy(self_hit, hp + qb + ob, B);
  return KGPU_OK;
}

kgpu_status kgpu_check_edges_host(kgpu_world w, int32_t robot, const float* qa, const float* qbuf,
                                  const int32_t* nsteps, int32_t E, int32_t* first_hit)
{
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E < 0 || (E > 0 && (!qa || !qbuf || !nsteps || !first_hit))) return fail(KGPU_ERR_INVALID, "bad buffers");
  int L = w->robots[robot]->nlinks;
  size_t qbytes = (size_t)E * L * sizeof(float);
  size_t o1 = al(qbytes), o2 = o1 + al(qbytes), o3 = o2 + al((size_t)E * 4);
  size_t o4 = o3 + al((size_t)E * 4), total = o4 + al(sizeof(int));
  if ((st = ensure_stage(w, total))) return st;
  char* hp = (char*)w->pinned;
  char* dp = (char*)w->dstage;
  cudaStream_t s = w->host_stream;
  memcpy(hp, qa, qbytes);
  memcpy(hp + o1, qbuf, qbytes);
  memcpy(hp + o2, nsteps, (size_t)E * 4);
  CK(cudaMemcpyAsync(dp, hp, o3, cudaMemcpyHostToDevice, s));
  st = kgpu_check_edges(w, robot, (const float*)dp, (const float*)(dp + o1), (const int32_t*)(dp + o2), E,
                        (int32_t*)(dp + o3), s);
  if (st) return st;
  CK(cudaMemcpyAsync(hp + o3, dp + o3, (size_t)E * 4, cudaMemcpyDeviceToHost, s));
  if ((st = sync_status_pinned(w, s, (int*)(hp + o4)))) return st;
  memcpy(first_hit, hp + o3, (size_t)E * 4);
  return KGPU_OK;
}

// ---- CUDA-graph edge plans ----------------------------------------------------
kgpu_status kgpu_edge_plan_create(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                  const int32_t* nsteps, int32_t E, int32_t* first_hit, kgpu_edge_plan* out)
{
  if (!out) return fail(KGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  kgpu_status st = check_world(w, robot);
  if (st) return st;
  if (E <= 0 || !qa || !qb || !nsteps || !first_hit) return fail(KGPU_ERR_INVALID, "bad buffers");
  if ((st = ensure_edge_scratch(w, E))) return st;
  cudaStream_t cs;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  kgpu_edge_plan p = new kgpu_edge_plan_s();
  p->world = w;
  cudaError_t e = cudaEventCreate(&p->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&p->ev[1]);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    Scratch S = engine_scratch(w, w->scratch);
    S.main_pass_ev[0] = p->ev[0];
    S.main_pass_ev[1] = p->ev[1];
    cudaError_t le = launch_check_edges(w->d_dev, w->d_status, S, robot, qa, qb, nsteps, E, first_hit, grid_blocks(w),
                                        w->blocks_per_sm, cs, w->grab, w->job_flush, w->edge_chunk, w->fp64_inline);
    e = cudaStreamEndCapture(cs, &p->graph);
    if (e == cudaSuccess && le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    kgpu_edge_plan_destroy(p);
    return cuda_fail(e, "edge plan capture");
  }
  w->live_plans++;
  *out = p;
  return KGPU_OK;
}

kgpu_status kgpu_edge_plan_launch(kgpu_edge_plan p, kgpu_stream s)
{
  if (!p || !p->exec) return fail(KGPU_ERR_INVALID, "null plan");
  CK(cudaGraphLaunch(p->exec, (cudaStream_t)s));
  return KGPU_OK;
}

kgpu_status kgpu_edge_plan_main_pass_ms(kgpu_edge_plan p, float* ms)
{
  if (!p || !p->exec || !ms) return fail(KGPU_ERR_INVALID, "null argument");
  CK(cudaEventElapsedTime(ms, p->ev[0], p->ev[1]));
  return KGPU_OK;
}

kgpu_status kgpu_edge_plan_destroy(kgpu_edge_plan p)
{
  if (!p) return KGPU_OK;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->world->live_plans--;
  }
  if (p->graph) cudaGraphDestroy(p->graph);
  for (cudaEvent_t ev : p->ev)
    if (ev) cudaEventDestroy(ev);
  delete p;
  return KGPU_OK;
}

kgpu_status kgpu_config_plan_create(kgpu_world w, int32_t robot, const int32_t* robot_ids, const float* q,
                                    int32_t q_stride, int32_t B, uint8_t* env_hit, uint8_t* self_hit,
                                    kgpu_config_plan* out)
{
  if (!out) return fail(KGPU_ERR_INVALID, "null argument");
  *out = nullptr;
  if (!w) return fail(KGPU_ERR_INVALID, "null world");
  kgpu_status st = robot >= 0 ? check_world(w, robot) : refresh_tables(w);
  if (st) return st;
  if (B <= 0 || !q || (!env_hit && !self_hit) || (robot < 0 && !robot_ids))
    return fail(KGPU_ERR_INVALID, "bad buffers");
  int maxl = 0;
  for (auto R : w->robots) maxl = std::max(maxl, R->nlinks);
  if (robot >= 0) q_stride = w->robots[robot]->nlinks;
  else if (q_stride < maxl) return fail(KGPU_ERR_INVALID, "q_stride %d < max links %d", q_stride, maxl);
  if (robot < 0 && (st = ensure_edge_scratch(w, B))) return st;  // the robot-sorted order
  cudaStream_t cs;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  kgpu_config_plan p = new kgpu_config_plan_s();
  p->world = w;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t le = launch_check_configs(w->d_dev, engine_scratch(w, w->scratch), robot, robot < 0 ? robot_ids : nullptr,
                                          q, q_stride, B, env_hit, self_hit, nullptr, grid_blocks(w), w->blocks_per_sm,
                                          cs, w->grab, w->job_flush, w->fp64_inline,
                                          robot < 0 ? (int)w->robots.size() : 0, robot < 0 ? w->d_status : nullptr);
    e = cudaStreamEndCapture(cs, &p->graph);
    if (e == cudaSuccess && le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    kgpu_config_plan_destroy(p);
    return cuda_fail(e, "configuration plan capture");
  }
  w->live_plans++;
  *out = p;
  return KGPU_OK;
}

kgpu_status kgpu_config_plan_launch(kgpu_config_plan p, kgpu_stream s)
{
  if (!p || !p->exec) return fail(KGPU_ERR_INVALID, "null plan");
  CK(cudaGraphLaunch(p->exec, (cudaStream_t)s));
  return KGPU_OK;
}

kgpu_status kgpu_config_plan_destroy(kgpu_config_plan p)
{
  if (!p) return KGPU_OK;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->world->live_plans--;
  }
  if (p->graph) cudaGraphDestroy(p->graph);
  delete p;
  return KGPU_OK;
}

}  // extern "C"
