/*
 * oracle.cpp — FP64 CPU oracle for the configuration-validity and proximity
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of bench.py load it as the checker.  The product never
 * links, loads or calls it.
 *
 * The reference's arithmetic for this path lives in KrisLibrary (forward
 * kinematics, PQP collision/distance, epsilon edge checkers), which Klamp't
 * clones at build time without pinning a version (Cpp/Dependencies/
 * Makefile:17-18, CMakeModules/KlamptDependencies.cmake:20-21) and which is
 * absent here, so this file restates the semantics from Klamp't's own call
 * sites and documentation:
 *
 *   forward kinematics   T_W[i] = T_W[parent(i)] * T0_Parent[i] * J(q_i)
 *                        Cpp/docs/Manual-Modeling.md:94,115;
 *                        Cpp/Modeling/Robot.cpp:961-981
 *   joint limits         Cpp/Planning/RobotCSpace.cpp:610-630
 *   feasibility order    limits, environment, self:
 *                        Cpp/Planning/RobotCSpace.cpp:786-823
 *   environment test     every enabled (link, object) pair, mesh-mesh
 *                        collide (within-distance when margins are set):
 *                        Cpp/Planning/PlannerSettings.cpp:96-107,269-331
 *   collision masks      Cpp/Planning/PlannerSettings.cpp:16-42,
 *                        Python/klampt/model/collide.py:314-362
 *   self collision       enabled link pairs, robotsim.cpp:5529-5539,
 *                        Cpp/Modeling/Robot.cpp:1275-1380
 *   margin               Cpp/docs/Manual-Geometry.md:17 (collide iff the
 *                        distance is <= the summed margins)
 *   edge checks          configurations a + (k/n)(b-a), k = 0..n,
 *                        Cpp/Modeling/Interpolate.cpp:10-14,
 *                        Cpp/Planning/RobotCSpace.cpp:835-840
 *   distance             mesh-mesh minimum triangle distance with closest
 *                        points (PQP semantics; robotsim.cpp:1782-1819,
 *                        Python/klampt/src/geometry.h:641-673), negative
 *                        penetration for convex obstacles (see below)
 *   soft-min, gradient   Python/klampt/math/autodiff/geometry_ad.py:613-814
 *                        (MinDistance), here as a log-sum-exp soft-min
 *   ray casting          first hit of s + t d (t >= 0) over the environment's
 *                        objects: Geometry3D::rayCast_ext (robotsim.cpp:
 *                        1821-1852), WorldModel::RayCast (Cpp/Modeling/
 *                        World.cpp:465-515), collide.ray_cast (Python/klampt/
 *                        model/collide.py:219-243); nearest hit, ties to the
 *                        smaller object, then triangle
 *
 * The FP64 values that decide verdicts and distances come from the canonical
 * arithmetic in include/kgpu_exact.h; everything else here (BVH build,
 * traversal, masks, edge semantics, penetration, soft-min, gradients) is this
 * file's own.  Compile with -ffp-contract=off.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/kgpu_exact.h"

#define ORC_MAXL 32

namespace {

struct Node {
  double c[3], h[3];
  int left;   // -1 for a leaf; children are left and left+1
  int first;  // leaf: first index into order[]
  int count;  // leaf: number of triangles
};

struct Bvh {
  std::vector<Node> nodes;
  std::vector<int> order;  // triangle ids in leaf order
  bool empty() const { return nodes.empty(); }
};

// median split on the widest centroid axis, leaves of <= 4 triangles,
// children stored adjacently, ties on the split key broken by triangle id.
// tri: 9 doubles per triangle (indexed by the ids given).
void build_bvh(const std::vector<double>& tri, const std::vector<int>& ids, Bvh& out)
{
  out.nodes.clear();
  out.order = ids;
  if (ids.empty()) return;
  auto cen = [&](int t, int i) {
    return (tri[9 * (size_t)t + i] + tri[9 * (size_t)t + 3 + i] + tri[9 * (size_t)t + 6 + i]) / 3.0;
  };
  struct Job { int node, b, e; };
  out.nodes.push_back(Node());
  std::vector<Job> st{{0, 0, (int)ids.size()}};
  while (!st.empty()) {
    Job j = st.back();
    st.pop_back();
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int k = j.b; k < j.e; ++k) {
      int t = out.order[k];
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < 3; ++i) {
          double x = tri[9 * (size_t)t + 3 * v + i];
          lo[i] = std::min(lo[i], x);
          hi[i] = std::max(hi[i], x);
        }
      for (int i = 0; i < 3; ++i) {
        clo[i] = std::min(clo[i], cen(t, i));
        chi[i] = std::max(chi[i], cen(t, i));
      }
    }
    Node& n = out.nodes[j.node];
    for (int i = 0; i < 3; ++i) {
      n.c[i] = 0.5 * (lo[i] + hi[i]);
      n.h[i] = 0.5 * (hi[i] - lo[i]);
    }
    if (j.e - j.b <= 4) {
      n.left = -1;
      n.first = j.b;
      n.count = j.e - j.b;
      continue;
    }
    int ax = 0;
    for (int i = 1; i < 3; ++i)
      if (chi[i] - clo[i] > chi[ax] - clo[ax]) ax = i;
    int mid = (j.b + j.e) / 2;
    std::nth_element(out.order.begin() + j.b, out.order.begin() + mid, out.order.begin() + j.e,
                     [&](int a, int b) {
                       double ka = cen(a, ax), kb = cen(b, ax);
                       return ka < kb || (ka == kb && a < b);
                     });
    int l = (int)out.nodes.size();
    n.left = l;
    n.first = 0;
    n.count = 0;
    out.nodes.push_back(Node());
    out.nodes.push_back(Node());
    st.push_back({l + 1, mid, j.e});
    st.push_back({l, j.b, mid});
  }
}

struct Robot {
  int L = 0;
  std::vector<int> parents, jtypes;
  std::vector<double> T0P, axes, qmin, qmax, margins;
  std::vector<uint8_t> self_mask;             // [L*L], upper triangle used
  std::vector<std::vector<double>> vloc;      // per link: local vertices
  std::vector<std::vector<int>> tidx;         // per link: vertex indices
  std::vector<std::vector<double>> tloc;      // per link: 9 doubles per tri
  std::vector<Bvh> bvh;
};

struct Env {
  int N = 0;
  std::vector<int> groups;
  std::vector<uint8_t> convex;
  std::vector<double> margins;
  std::vector<double> tri;      // all triangles, world frame, 9 per tri
  std::vector<int> tri_obj;     // object of each triangle
  std::vector<int> obj_first, obj_count;
  Bvh group_bvh[32];
  double group_margin[32];
  std::vector<Bvh> obj_bvh;     // ids are global triangle ids
  std::vector<double> obj_c, obj_h;
  std::vector<double> face_n, face_top;  // unit outward normal and n . a per triangle
};

inline void xform_box(const double* T, const Node& n, double* c, double* h)
{
  kx_xform_point(T, n.c, c);
  for (int r = 0; r < 3; ++r)
    h[r] = fabs(T[3 * r]) * n.h[0] + fabs(T[3 * r + 1]) * n.h[1] + fabs(T[3 * r + 2]) * n.h[2];
}

inline double node_size(const Node& n) { return n.h[0] + n.h[1] + n.h[2]; }

struct Counters {
  long long node_pairs = 0, tri_pairs = 0, items = 0;
};

struct Ctx {
  const Robot* R = nullptr;
  const Env* E = nullptr;
  const uint32_t* masks = nullptr;
  double T[ORC_MAXL][12];
  std::vector<std::vector<double>> wtri;   // per link world triangles
  std::vector<std::vector<double>> wvert;  // per link world vertices
  std::vector<char> tri_ready, vert_ready;
  Counters cnt;

  void init(const Robot* r, const Env* e, const uint32_t* m)
  {
    R = r; E = e; masks = m;
    wtri.assign(r->L, {});
    wvert.assign(r->L, {});
    tri_ready.assign(r->L, 0);
    vert_ready.assign(r->L, 0);
  }
  void set_config(const double* q)
  {
    for (int i = 0; i < R->L; ++i) {
      double Lc[12];
      kx_joint_local(&R->T0P[12 * i], &R->axes[3 * i], R->jtypes[i], q[i], Lc);
      int p = R->parents[i];
      if (p < 0) std::memcpy(T[i], Lc, sizeof(Lc));
      else kx_compose(T[p], Lc, T[i]);
    }
    std::fill(tri_ready.begin(), tri_ready.end(), 0);
    std::fill(vert_ready.begin(), vert_ready.end(), 0);
  }
  // world transforms given directly (free geometries: one per link)
  void set_transforms(const double* const* Ts)
  {
    for (int i = 0; i < R->L; ++i) std::memcpy(T[i], Ts[i], sizeof(T[i]));
    std::fill(tri_ready.begin(), tri_ready.end(), 0);
    std::fill(vert_ready.begin(), vert_ready.end(), 0);
  }
  const double* link_tri(int l, int t)
  {
    if (!tri_ready[l]) {
      const std::vector<double>& src = R->tloc[l];
      std::vector<double>& dst = wtri[l];
      dst.resize(src.size());
      for (size_t k = 0; k < src.size(); k += 3) kx_xform_point(T[l], &src[k], &dst[k]);
      tri_ready[l] = 1;
    }
    return &wtri[l][9 * (size_t)t];
  }
  const std::vector<double>& link_verts(int l)
  {
    if (!vert_ready[l]) {
      const std::vector<double>& src = R->vloc[l];
      std::vector<double>& dst = wvert[l];
      dst.resize(src.size());
      for (size_t k = 0; k < src.size(); k += 3) kx_xform_point(T[l], &src[k], &dst[k]);
      vert_ready[l] = 1;
    }
    return wvert[l];
  }
};

// ---------------------------------------------------------------------------
// collision: BVH-vs-BVH traversal (descend the larger node), boxes inflated by
// 1e-9 m + margins so that culling never removes a pair the FP64 predicate
// would accept.  lb < 0: environment group `grp`; else link lb.
// ---------------------------------------------------------------------------
bool bvtt_collide(Ctx& c, int la, int lb, int grp, double tol_extra = 0.0)
{
  const Robot& R = *c.R;
  const Bvh& A = R.bvh[la];
  const int g = grp < 0 ? 0 : grp;  // a group only when lb < 0
  const Bvh& B = lb >= 0 ? R.bvh[lb] : c.E->group_bvh[g];
  if (A.empty() || B.empty()) return false;
  // (a link-link query may add a distance tolerance to the first margin)
  double mA = tol_extra != 0.0 ? R.margins[la] + tol_extra : R.margins[la];
  double mB = lb >= 0 ? R.margins[lb] : c.E->group_margin[g];
  double tol = 1e-9 + mA + mB;
  std::vector<std::pair<int, int>> st;
  st.reserve(256);
  st.push_back({0, 0});
  while (!st.empty()) {
    auto pr = st.back();
    st.pop_back();
    const Node& na = A.nodes[pr.first];
    const Node& nb = B.nodes[pr.second];
    double ca[3], ha[3], cb[3], hb[3];
    xform_box(c.T[la], na, ca, ha);
    if (lb >= 0) xform_box(c.T[lb], nb, cb, hb);
    else { std::memcpy(cb, nb.c, sizeof cb); std::memcpy(hb, nb.h, sizeof hb); }
    c.cnt.node_pairs++;
    bool sep = false;
    for (int i = 0; i < 3; ++i)
      if (fabs(ca[i] - cb[i]) > ha[i] + hb[i] + tol) sep = true;
    if (sep) continue;
    bool la_leaf = na.left < 0, lb_leaf = nb.left < 0;
    if (la_leaf && lb_leaf) {
      for (int i = 0; i < na.count; ++i) {
        int ta = A.order[na.first + i];
        const double* P = c.link_tri(la, ta);
        for (int j = 0; j < nb.count; ++j) {
          int tb = B.order[nb.first + j];
          const double* Q = lb >= 0 ? c.link_tri(lb, tb) : &c.E->tri[9 * (size_t)tb];
          double m = mA + (lb >= 0 ? mB : c.E->margins[c.E->tri_obj[tb]]);
          c.cnt.tri_pairs++;
          bool hit;
          if (m == 0.0) hit = kx_tri_tri_overlap(P, Q) != 0;
          else {
            double cp[3], cq[3];
            hit = kx_tri_tri_dist2(P, Q, cp, cq) <= m * m;
          }
          if (hit) return true;
        }
      }
    } else if (la_leaf || (!lb_leaf && node_size(nb) > node_size(na))) {
      st.push_back({pr.first, nb.left + 1});
      st.push_back({pr.first, nb.left});
    } else {
      st.push_back({na.left + 1, pr.second});
      st.push_back({na.left, pr.second});
    }
  }
  return false;
}

bool env_collides(Ctx& c)
{
  const Robot& R = *c.R;
  for (int l = 0; l < R.L; ++l) {
    if (R.tloc[l].empty()) continue;
    for (int g = 0; g < 32; ++g)
      if (((c.masks[l] >> g) & 1u) && !c.E->group_bvh[g].empty())
        if (bvtt_collide(c, l, -1, g)) return true;
  }
  return false;
}

bool self_collides(Ctx& c)
{
  const Robot& R = *c.R;
  for (int i = 0; i < R.L; ++i)
    for (int j = i + 1; j < R.L; ++j)
      if (R.self_mask[i * R.L + j] && !R.tloc[i].empty() && !R.tloc[j].empty())
        if (bvtt_collide(c, i, j, -1)) return true;
  return false;
}

bool in_limits(const Robot& R, const double* q)
{
  for (int i = 0; i < R.L; ++i)
    if (q[i] < R.qmin[i] || q[i] > R.qmax[i]) return false;
  return true;
}

// ---------------------------------------------------------------------------
// distance between link l and object o (world frame).
//   Unsigned part: min over triangle pairs of kx_tri_tri_dist2 (PQP
//   semantics), ties resolved to the lexicographically smallest
//   (link triangle, object triangle) pair; search bounded by ub2.
//   Signed part (convex obstacles only): if the surfaces meet (distance 0),
//   d = -depth, depth = the largest depth of a link vertex inside the
//   obstacle, depth(v) = min over obstacle faces f of (n_f . a_f - n_f . v)
//   (n_f the unit outward face normal, a_f the face's first vertex; for a
//   convex obstacle this is v's distance to the boundary when v is inside),
//   0 when no vertex is strictly inside.  d is continuous at the onset of
//   contact.  Feature pair (v*, f*), d/dv* = n_f*; ties resolve to the first
//   vertex, then the first face, in mesh order.
// ---------------------------------------------------------------------------
struct PairResult {
  double d;          // signed distance (or the bound when nothing is closer)
  double cp[3], cq[3];
  double dir[3];     // d(d)/d(cp): unit vector
  int found;         // 1 if d < bound
  int ta, tb;        // feature ids: triangles (unsigned) or vertex/face (signed)
  int signed_pen;    // 1 if the penetration branch produced d
};

void face_normal(const double* F, double* n)
{
  double e0[3], e1[3], c[3];
  kx_sub3(F + 3, F, e0);
  kx_sub3(F + 6, F, e1);
  kx_cross3(e0, e1, c);
  double len = kx_sqrt(kx_dot3(c, c));
  for (int i = 0; i < 3; ++i) n[i] = kx_div(c[i], len);
}

// deepest link vertex inside convex object o; returns the depth (0 if no
// vertex is strictly inside), its vertex and face.  Vertices outside the
// object's bounding box cannot be inside and are skipped.
double penetration(Ctx& c, int l, int o, int* fbest, int* vbest, double* nbest)
{
  const Env& E = *c.E;
  const std::vector<double>& V = c.link_verts(l);
  int nv = (int)(V.size() / 3);
  double best = 0.0;
  *fbest = -1;
  *vbest = -1;
  const double* oc = &E.obj_c[3 * o];
  const double* oh = &E.obj_h[3 * o];
  for (int v = 0; v < nv; ++v) {
    const double* x = &V[3 * (size_t)v];
    if (fabs(x[0] - oc[0]) > oh[0] * (1 + 1e-12) + 1e-12 || fabs(x[1] - oc[1]) > oh[1] * (1 + 1e-12) + 1e-12 ||
        fabs(x[2] - oc[2]) > oh[2] * (1 + 1e-12) + 1e-12)
      continue;
    double dmin = 1e300;
    int fmin = -1;
    for (int f = E.obj_first[o]; f < E.obj_first[o] + E.obj_count[o]; ++f) {
      double dep = kx_sub(E.face_top[f], kx_dot3(&E.face_n[3 * (size_t)f], x));
      if (dep < dmin) { dmin = dep; fmin = f; }
    }
    if (dmin > best) {
      best = dmin;
      *vbest = v;
      *fbest = fmin;
    }
  }
  if (*fbest >= 0)
    for (int i = 0; i < 3; ++i) nbest[i] = E.face_n[3 * (size_t)*fbest + i];
  return best;
}

PairResult pair_distance(Ctx& c, int l, int o, double bound)
{
  const Robot& R = *c.R;
  const Env& E = *c.E;
  PairResult res;
  res.found = 0;
  res.d = bound;
  res.signed_pen = 0;
  res.ta = res.tb = -1;
  const Bvh& A = R.bvh[l];
  const Bvh& B = E.obj_bvh[o];
  if (A.empty() || B.empty()) return res;
  // unsigned search bounded by max(bound, 0); with a non-positive bound only
  // contact (squared distance exactly 0) matters
  double ub = bound > 0 ? bound : 0.0;
  double best2 = ub * ub > 1e-300 ? ub * ub : 1e-300;  // (a tiny bound must not underflow to 0)
  int bta = -1, btb = -1;
  double bcp[3] = {0, 0, 0}, bcq[3] = {0, 0, 0};
  bool have = false;
  std::vector<std::pair<int, int>> st;
  st.push_back({0, 0});
  while (!st.empty()) {
    auto pr = st.back();
    st.pop_back();
    const Node& na = A.nodes[pr.first];
    const Node& nb = B.nodes[pr.second];
    double ca[3], ha[3];
    xform_box(c.T[l], na, ca, ha);
    double lb2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      double g = fabs(ca[i] - nb.c[i]) - ha[i] - nb.h[i];
      if (g > 0) lb2 += g * g;
    }
    c.cnt.node_pairs++;
    // keep ties (slack) so that the tie-break sees every equal pair
    if (have ? lb2 > best2 * (1 + 1e-9) + 1e-24 : lb2 >= best2 * (1 + 1e-9) + 1e-24) continue;
    bool la_leaf = na.left < 0, lb_leaf = nb.left < 0;
    if (la_leaf && lb_leaf) {
      for (int i = 0; i < na.count; ++i) {
        int ta = A.order[na.first + i];
        const double* P = c.link_tri(l, ta);
        for (int j = 0; j < nb.count; ++j) {
          int tb = B.order[nb.first + j];
          c.cnt.tri_pairs++;
          double cp[3], cq[3];
          double d2 = kx_tri_tri_dist2(P, &E.tri[9 * (size_t)tb], cp, cq);
          bool better = have ? (d2 < best2 || (d2 == best2 && (ta < bta || (ta == bta && tb < btb))))
                             : (d2 < best2);
          if (better) {
            have = true;
            best2 = d2;
            bta = ta; btb = tb;
            std::memcpy(bcp, cp, sizeof bcp);
            std::memcpy(bcq, cq, sizeof bcq);
          }
        }
      }
    } else if (la_leaf || (!lb_leaf && node_size(nb) > node_size(na))) {
      st.push_back({pr.first, nb.left + 1});
      st.push_back({pr.first, nb.left});
    } else {
      st.push_back({na.left + 1, pr.second});
      st.push_back({na.left, pr.second});
    }
  }
  if (!have) return res;
  if (best2 == 0.0 && E.convex[o]) {
    int f, v;
    double n[3];
    double pen = penetration(c, l, o, &f, &v, n);
    if (v < 0) {  // surfaces meet, no vertex inside: d = 0 with no direction
      if (0.0 < bound) {
        res.found = 1;
        res.d = 0.0;
        std::memcpy(res.cp, bcp, sizeof bcp);
        std::memcpy(res.cq, bcq, sizeof bcq);
        res.dir[0] = res.dir[1] = res.dir[2] = 0.0;
        res.ta = bta;
        res.tb = btb;
      }
      return res;
    }
    double d = -pen;
    if (d < bound) {
      const std::vector<double>& V = c.link_verts(l);
      res.found = 1;
      res.signed_pen = 1;
      res.d = d;
      res.ta = v;
      res.tb = f;
      for (int i = 0; i < 3; ++i) {
        res.cp[i] = V[3 * (size_t)v + i];
        res.cq[i] = kx_add(V[3 * (size_t)v + i], kx_mul(pen, n[i]));
        res.dir[i] = n[i];
      }
    }
    return res;
  }
  double d = kx_sqrt(best2);
  if (!(d < bound)) return res;
  res.found = 1;
  res.d = d;
  res.ta = bta;
  res.tb = btb;
  std::memcpy(res.cp, bcp, sizeof bcp);
  std::memcpy(res.cq, bcq, sizeof bcq);
  if (d > 0) {
    for (int i = 0; i < 3; ++i) res.dir[i] = (bcp[i] - bcq[i]) / d;
  } else {
    res.dir[0] = res.dir[1] = res.dir[2] = 0.0;
  }
  return res;
}

// d(d)/dq for a feature point p (world) on link l moving with the link, with
// d(d)/dp = u.  Revolute joint j on the chain: u . (w_j x (p - o_j)), w_j the
// world joint axis, o_j the origin of link j's frame; prismatic: u . w_j.
void feature_gradient(const Ctx& c, int l, const double* p, const double* u, double scale,
                      double* g)
{
  const Robot& R = *c.R;
  for (int j = l; j >= 0; j = R.parents[j]) {
    if (R.jtypes[j] == KX_JOINT_WELD) continue;
    const double* T = c.T[j];
    const double* wl = &R.axes[3 * j];
    double w[3];
    for (int r = 0; r < 3; ++r) w[r] = T[3 * r] * wl[0] + T[3 * r + 1] * wl[1] + T[3 * r + 2] * wl[2];
    double v;
    if (R.jtypes[j] == KX_JOINT_REVOLUTE) {
      double rr[3] = {p[0] - T[9], p[1] - T[10], p[2] - T[11]};
      double x[3] = {w[1] * rr[2] - w[2] * rr[1], w[2] * rr[0] - w[0] * rr[2], w[0] * rr[1] - w[1] * rr[0]};
      v = u[0] * x[0] + u[1] * x[1] + u[2] * x[2];
    } else {
      v = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
    }
    g[j] += scale * v;
  }
}

// distance between links i and j of the robot (both in the world frame):
// min over triangle pairs of kx_tri_tri_dist2, ties to the smallest
// (triangle of i, triangle of j) in mesh order; only distances strictly
// below `bound` are found.  No signed part: 0 when the surfaces meet.
PairResult self_pair_distance(Ctx& c, int i, int j, double bound, bool bound_check = true)
{
  const Robot& R = *c.R;
  PairResult res;
  res.found = 0;
  res.d = bound;
  res.signed_pen = 0;
  res.ta = res.tb = -1;
  const Bvh& A = R.bvh[i];
  const Bvh& B = R.bvh[j];
  if (A.empty() || B.empty()) return res;
  double ub = bound > 0 ? bound : 0.0;
  double best2 = ub * ub > 1e-300 ? ub * ub : 1e-300;
  int bta = -1, btb = -1;
  double bcp[3] = {0, 0, 0}, bcq[3] = {0, 0, 0};
  bool have = false;
  std::vector<std::pair<int, int>> st;
  st.push_back({0, 0});
  while (!st.empty()) {
    auto pr = st.back();
    st.pop_back();
    const Node& na = A.nodes[pr.first];
    const Node& nb = B.nodes[pr.second];
    double ca[3], ha[3], cb[3], hb[3];
    xform_box(c.T[i], na, ca, ha);
    xform_box(c.T[j], nb, cb, hb);
    double lb2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      double g = fabs(ca[k] - cb[k]) - ha[k] - hb[k];
      if (g > 0) lb2 += g * g;
    }
    c.cnt.node_pairs++;
    if (have ? lb2 > best2 * (1 + 1e-9) + 1e-24 : lb2 >= best2 * (1 + 1e-9) + 1e-24) continue;
    bool la_leaf = na.left < 0, lb_leaf = nb.left < 0;
    if (la_leaf && lb_leaf) {
      for (int x = 0; x < na.count; ++x) {
        int ta = A.order[na.first + x];
        const double* P = c.link_tri(i, ta);
        for (int y = 0; y < nb.count; ++y) {
          int tb = B.order[nb.first + y];
          c.cnt.tri_pairs++;
          double cp[3], cq[3];
          double d2 = kx_tri_tri_dist2(P, c.link_tri(j, tb), cp, cq);
          bool better = have ? (d2 < best2 || (d2 == best2 && (ta < bta || (ta == bta && tb < btb))))
                             : (d2 < best2);
          if (better) {
            have = true;
            best2 = d2;
            bta = ta; btb = tb;
            std::memcpy(bcp, cp, sizeof bcp);
            std::memcpy(bcq, cq, sizeof bcq);
          }
        }
      }
    } else if (la_leaf || (!lb_leaf && node_size(nb) > node_size(na))) {
      st.push_back({pr.first, nb.left + 1});
      st.push_back({pr.first, nb.left});
    } else {
      st.push_back({na.left + 1, pr.second});
      st.push_back({na.left, pr.second});
    }
  }
  if (!have) return res;
  double d = kx_sqrt(best2);
  if (bound_check && !(d < bound)) return res;
  res.found = 1;
  res.d = d;
  res.ta = bta;
  res.tb = btb;
  std::memcpy(res.cp, bcp, sizeof bcp);
  std::memcpy(res.cq, bcq, sizeof bcq);
  return res;
}

bool pair_enabled(const Ctx& c, int l, int o)
{
  return ((c.masks[l] >> c.E->groups[o]) & 1u) && !c.R->tloc[l].empty();
}

// lower bound on the distance between link l (world box of its BVH root)
// and object o's box
double link_obj_lb(const Ctx& c, int l, int o)
{
  const Node& na = c.R->bvh[l].nodes[0];
  double ca[3], ha[3];
  xform_box(c.T[l], na, ca, ha);
  double lb2 = 0;
  for (int i = 0; i < 3; ++i) {
    double g = fabs(ca[i] - c.E->obj_c[3 * o + i]) - ha[i] - c.E->obj_h[3 * o + i];
    if (g > 0) lb2 += g * g;
  }
  return sqrt(lb2);
}

// minimum signed distance over enabled (link, object) pairs, below `bound`;
// ties resolved to the smallest (link, object).
struct MinResult {
  double d;
  int link, obj;
  PairResult pr;
};

// Pairs are visited nearest first by their box lower bound, as
// DistanceLowerBound sorts its pairs (Cpp/Planning/PlannerSettings.cpp:
// 543-567), so the running minimum prunes the rest early; the result is the
// minimum with ties to the smallest (link, object), whatever the order.
MinResult min_distance(Ctx& c, double bound)
{
  MinResult m;
  m.d = bound;
  m.link = m.obj = -1;
  std::vector<std::pair<double, int>> cand;  // (lower bound, l * N + o)
  for (int l = 0; l < c.R->L; ++l) {
    if (c.R->bvh[l].empty()) continue;
    for (int o = 0; o < c.E->N; ++o) {
      if (!pair_enabled(c, l, o)) continue;
      const double lb = link_obj_lb(c, l, o);
      if (lb > std::max(bound, 0.0) + 1e-9) continue;
      cand.push_back({lb, l * c.E->N + o});
    }
  }
  std::sort(cand.begin(), cand.end());
  for (const auto& x : cand) {
    // the box bound limits the unsigned distance; a pair can be negative
    // only when its boxes meet (bound 0)
    if (x.first > std::max(m.d, 0.0) + 1e-9) break;
    const int l = x.second / c.E->N, o = x.second % c.E->N;
    // a pair's distance is at least 0 unless its object is convex, and then
    // at least minus the smallest half-extent of the object's box; a pair
    // that cannot go below the best, and could at most tie without winning
    // the tie, cannot change the result
    if (m.link >= 0) {
      const double* h = &c.E->obj_h[3 * (size_t)o];
      const double dlow = c.E->convex[o] ? -std::min(h[0], std::min(h[1], h[2])) : 0.0;
      if (dlow > m.d || (dlow == m.d && !(l < m.link || (l == m.link && o < m.obj)))) continue;
    }
    // ties must reach the comparison: search with a bound slightly above m.d
    PairResult pr = pair_distance(c, l, o, std::nextafter(m.d, 1e300));
    if (pr.found && (pr.d < m.d || (pr.d == m.d && m.link >= 0 && (l < m.link || (l == m.link && o < m.obj))))) {
      m.d = pr.d; m.link = l; m.obj = o; m.pr = pr;
    }
  }
  return m;
}

// per-thread counters summed into counters[3] = {node pairs, triangle pairs,
// items} (when given)
void sum_counters(const std::vector<Counters>& cs, long long* counters)
{
  if (!counters) return;
  counters[0] = counters[1] = counters[2] = 0;
  for (const auto& x : cs) {
    counters[0] += x.node_pairs;
    counters[1] += x.tri_pairs;
    counters[2] += x.items;
  }
}

template <class F>
void parallel_for(int n, int nthreads, F&& fn)
{
  if (nthreads <= 1 || n <= 1) {
    fn(0, 0, n);
    return;
  }
  nthreads = std::min(nthreads, n);
  std::atomic<int> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&, t]() {
      for (;;) {
        int i = next.fetch_add(16);
        if (i >= n) break;
        fn(t, i, std::min(n, i + 16));
      }
    });
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void* orc_robot_create(int L, const int* parents, const int* jtypes, const double* T0P,
                       const double* axes, const double* qmin, const double* qmax,
                       const int* vert_off, const double* verts, const int* tri_off,
                       const int* tris, const double* margins, const unsigned char* self_mask)
{
  if (L <= 0 || L > ORC_MAXL) return nullptr;
  Robot* R = new Robot();
  R->L = L;
  R->parents.assign(parents, parents + L);
  R->jtypes.assign(jtypes, jtypes + L);
  R->T0P.assign(T0P, T0P + 12 * L);
  R->axes.assign(axes, axes + 3 * L);
  R->qmin.assign(qmin, qmin + L);
  R->qmax.assign(qmax, qmax + L);
  R->margins.assign(L, 0.0);
  if (margins) R->margins.assign(margins, margins + L);
  R->self_mask.assign(L * L, 0);
  for (int i = 0; i < L; ++i)
    for (int j = i + 1; j < L; ++j) {
      if (self_mask) R->self_mask[i * L + j] = self_mask[i * L + j] ? 1 : 0;
      else R->self_mask[i * L + j] = (parents[j] != i && parents[i] != j) ? 1 : 0;
    }
  R->vloc.resize(L);
  R->tidx.resize(L);
  R->tloc.resize(L);
  R->bvh.resize(L);
  for (int l = 0; l < L; ++l) {
    R->vloc[l].assign(verts + 3 * (size_t)vert_off[l], verts + 3 * (size_t)vert_off[l + 1]);
    int nt = tri_off[l + 1] - tri_off[l];
    R->tidx[l].assign(tris + 3 * (size_t)tri_off[l], tris + 3 * (size_t)tri_off[l + 1]);
    R->tloc[l].resize(9 * (size_t)nt);
    for (int t = 0; t < nt; ++t)
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < 3; ++i)
          R->tloc[l][9 * t + 3 * v + i] = R->vloc[l][3 * R->tidx[l][3 * t + v] + i];
    std::vector<int> ids(nt);
    for (int t = 0; t < nt; ++t) ids[t] = t;
    build_bvh(R->tloc[l], ids, R->bvh[l]);
  }
  return R;
}

void orc_robot_destroy(void* r) { delete (Robot*)r; }

void* orc_env_create(int N, const int* vert_off, const double* verts, const int* tri_off,
                     const int* tris, const int* groups, const unsigned char* convex,
                     const double* margins)
{
  Env* E = new Env();
  E->N = N;
  E->groups.assign(N, 0);
  if (groups) E->groups.assign(groups, groups + N);
  E->convex.assign(N, 0);
  if (convex) E->convex.assign(convex, convex + N);
  E->margins.assign(N, 0.0);
  if (margins) E->margins.assign(margins, margins + N);
  size_t ntot = (size_t)tri_off[N];
  E->tri.resize(9 * ntot);
  E->tri_obj.resize(ntot);
  E->obj_first.resize(N);
  E->obj_count.resize(N);
  for (int o = 0; o < N; ++o) {
    E->obj_first[o] = tri_off[o];
    E->obj_count[o] = tri_off[o + 1] - tri_off[o];
    for (int t = tri_off[o]; t < tri_off[o + 1]; ++t) {
      E->tri_obj[t] = o;
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < 3; ++i)
          E->tri[9 * (size_t)t + 3 * v + i] = verts[3 * ((size_t)vert_off[o] + tris[3 * (size_t)t + v]) + i];
    }
  }
  E->face_n.resize(3 * ntot);
  E->face_top.resize(ntot);
  for (size_t t = 0; t < ntot; ++t) {
    face_normal(&E->tri[9 * t], &E->face_n[3 * t]);
    E->face_top[t] = kx_dot3(&E->face_n[3 * t], &E->tri[9 * t]);
  }
  for (int g = 0; g < 32; ++g) {
    std::vector<int> ids;
    double gm = 0;
    for (int o = 0; o < N; ++o)
      if (E->groups[o] == g) {
        gm = std::max(gm, E->margins[o]);
        for (int t = tri_off[o]; t < tri_off[o + 1]; ++t) ids.push_back(t);
      }
    E->group_margin[g] = gm;
    build_bvh(E->tri, ids, E->group_bvh[g]);
  }
  E->obj_bvh.resize(N);
  E->obj_c.resize(3 * N);
  E->obj_h.resize(3 * N);
  for (int o = 0; o < N; ++o) {
    std::vector<int> ids;
    for (int t = tri_off[o]; t < tri_off[o + 1]; ++t) ids.push_back(t);
    build_bvh(E->tri, ids, E->obj_bvh[o]);
    if (!E->obj_bvh[o].empty())
      for (int i = 0; i < 3; ++i) {
        E->obj_c[3 * o + i] = E->obj_bvh[o].nodes[0].c[i];
        E->obj_h[3 * o + i] = E->obj_bvh[o].nodes[0].h[i];
      }
  }
  return E;
}

void orc_env_destroy(void* e) { delete (Env*)e; }

/* forward kinematics of one configuration: T [L*12] */
void orc_fk(void* robot, const double* q, double* T)
{
  Robot* R = (Robot*)robot;
  Ctx c;
  c.init(R, nullptr, nullptr);
  c.set_config(q);
  for (int i = 0; i < R->L; ++i) std::memcpy(T + 12 * i, c.T[i], 12 * sizeof(double));
}

void orc_sincos(const double* x, int n, double* s, double* c)
{
  for (int i = 0; i < n; ++i) kx_sincos(x[i], &s[i], &c[i]);
}

int orc_tri_tri(const double* P, const double* Q, double* d2, double* cp, double* cq)
{
  *d2 = kx_tri_tri_dist2(P, Q, cp, cq);
  return kx_tri_tri_overlap(P, Q);
}

/* the canonical FP64 predicate over n pairs: out[i] = kx_tri_tri_overlap */
int orc_tri_tri_batch(const double* P, const double* Q, int n, unsigned char* out)
{
  for (int i = 0; i < n; ++i) out[i] = (unsigned char)kx_tri_tri_overlap(P + 9 * (size_t)i, Q + 9 * (size_t)i);
  return 0;
}

/* environment / self verdicts of B configurations; counters[3] =
 * {node pairs, triangle pairs, configurations} */
int orc_check_configs(void* robot, void* env, const unsigned* masks, const float* q, int B,
                      unsigned char* env_hit, unsigned char* self_hit, int nthreads,
                      long long* counters)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  std::vector<Counters> cs(std::max(1, nthreads));
  parallel_for(B, nthreads, [&](int t, int b0, int b1) {
    Ctx c;
    c.init(R, E, masks);
    double qd[ORC_MAXL];
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < R->L; ++i) qd[i] = (double)q[(size_t)b * R->L + i];
      c.set_config(qd);
      if (env_hit) env_hit[b] = env_collides(c) ? 1 : 0;
      if (self_hit) self_hit[b] = self_collides(c) ? 1 : 0;
      c.cnt.items++;
    }
    cs[t].node_pairs += c.cnt.node_pairs;
    cs[t].tri_pairs += c.cnt.tri_pairs;
    cs[t].items += c.cnt.items;
  });
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (auto& x : cs) {
      counters[0] += x.node_pairs;
      counters[1] += x.tri_pairs;
      counters[2] += x.items;
    }
  }
  return 0;
}

/* the same verdicts by testing every triangle pair (no BVH): validates the
 * oracle's own culling on small meshes */
int orc_check_configs_brute(void* robot, void* env, const unsigned* masks, const float* q, int B,
                            unsigned char* env_hit, unsigned char* self_hit)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  Ctx c;
  c.init(R, E, masks);
  double qd[ORC_MAXL];
  for (int b = 0; b < B; ++b) {
    for (int i = 0; i < R->L; ++i) qd[i] = (double)q[(size_t)b * R->L + i];
    c.set_config(qd);
    bool eh = false, sh = false;
    for (int l = 0; l < R->L && !eh; ++l) {
      int nt = (int)(R->tloc[l].size() / 9);
      for (int o = 0; o < E->N && !eh; ++o) {
        if (!((masks[l] >> E->groups[o]) & 1u)) continue;
        double m = R->margins[l] + E->margins[o];
        for (int ta = 0; ta < nt && !eh; ++ta)
          for (int tb = E->obj_first[o]; tb < E->obj_first[o] + E->obj_count[o] && !eh; ++tb) {
            const double* P = c.link_tri(l, ta);
            const double* Q = &E->tri[9 * (size_t)tb];
            double cp[3], cq[3];
            eh = m == 0.0 ? kx_tri_tri_overlap(P, Q) != 0 : kx_tri_tri_dist2(P, Q, cp, cq) <= m * m;
          }
      }
    }
    for (int i = 0; i < R->L && !sh; ++i)
      for (int j = i + 1; j < R->L && !sh; ++j) {
        if (!R->self_mask[i * R->L + j]) continue;
        int na = (int)(R->tloc[i].size() / 9), nb = (int)(R->tloc[j].size() / 9);
        double m = R->margins[i] + R->margins[j];
        for (int ta = 0; ta < na && !sh; ++ta)
          for (int tb = 0; tb < nb && !sh; ++tb) {
            const double* P = c.link_tri(i, ta);
            const double* Q = c.link_tri(j, tb);
            double cp[3], cq[3];
            sh = m == 0.0 ? kx_tri_tri_overlap(P, Q) != 0 : kx_tri_tri_dist2(P, Q, cp, cq) <= m * m;
          }
      }
    if (env_hit) env_hit[b] = eh;
    if (self_hit) self_hit[b] = sh;
  }
  return 0;
}

/* feasibility (limits, environment, self) of B configurations */
int orc_is_feasible(void* robot, void* env, const unsigned* masks, const float* q, int B,
                    unsigned char* feasible, int nthreads)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  parallel_for(B, nthreads, [&](int, int b0, int b1) {
    Ctx c;
    c.init(R, E, masks);
    double qd[ORC_MAXL];
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < R->L; ++i) qd[i] = (double)q[(size_t)b * R->L + i];
      bool ok = in_limits(*R, qd);
      if (ok) {
        c.set_config(qd);
        ok = !env_collides(c) && !self_collides(c);
      }
      feasible[b] = ok ? 1 : 0;
    }
  });
  return 0;
}

/* first infeasible step index of each edge (-1 if none); counters[3] as above
 * with configurations = steps examined */
int orc_check_edges(void* robot, void* env, const unsigned* masks, const float* qa,
                    const float* qb, const int* nsteps, int E_, int* first_hit, int nthreads,
                    long long* counters)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  std::vector<Counters> cs(std::max(1, nthreads));
  parallel_for(E_, nthreads, [&](int t, int e0, int e1) {
    Ctx c;
    c.init(R, E, masks);
    double qd[ORC_MAXL];
    for (int e = e0; e < e1; ++e) {
      int n = nsteps[e];
      int hit = -1;
      for (int k = 0; k <= n && hit < 0; ++k) {
        for (int i = 0; i < R->L; ++i)
          qd[i] = kx_interp((double)qa[(size_t)e * R->L + i], (double)qb[(size_t)e * R->L + i], k, n);
        c.cnt.items++;
        if (!in_limits(*R, qd)) { hit = k; break; }
        c.set_config(qd);
        if (env_collides(c) || self_collides(c)) hit = k;
      }
      first_hit[e] = hit;
    }
    cs[t].node_pairs += c.cnt.node_pairs;
    cs[t].tri_pairs += c.cnt.tri_pairs;
    cs[t].items += c.cnt.items;
  });
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (auto& x : cs) {
      counters[0] += x.node_pairs;
      counters[1] += x.tri_pairs;
      counters[2] += x.items;
    }
  }
  return 0;
}

/* signed distance between link `link` and object `obj` at configuration q:
 * out[0] = d, out[1..3] = cp, out[4..6] = cq, out[7..9] = dir; feat[0..2] =
 * (feature a, feature b, signed-branch flag).  Returns 1 if d < bound. */
int orc_pair_distance(void* robot, void* env, const float* q, int link, int obj, double bound,
                      double* out, int* feat)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  unsigned masks[ORC_MAXL];
  for (int i = 0; i < ORC_MAXL; ++i) masks[i] = 0xffffffffu;
  Ctx c;
  c.init(R, E, masks);
  double qd[ORC_MAXL];
  for (int i = 0; i < R->L; ++i) qd[i] = (double)q[i];
  c.set_config(qd);
  PairResult pr = pair_distance(c, link, obj, bound);
  out[0] = pr.d;
  for (int i = 0; i < 3; ++i) {
    out[1 + i] = pr.found ? pr.cp[i] : 0;
    out[4 + i] = pr.found ? pr.cq[i] : 0;
    out[7 + i] = pr.found ? pr.dir[i] : 0;
  }
  feat[0] = pr.ta;
  feat[1] = pr.tb;
  feat[2] = pr.signed_pen;
  return pr.found;
}

/* The enabled (link, object) pairs of one configuration whose signed
 * distance lies below `bound`, each with its deciding feature pair: out[5k..]
 * = (link, object, feature a, feature b, signed-branch flag), in (link,
 * object) order; dist[k] the pair's distance.  Returns the number of pairs
 * (at most max_out are written).  Lets a test tell where a closest feature
 * switches between nearby configurations (a kink of the distance). */
int orc_pair_features(void* robot, void* env, const unsigned* masks, const float* q, double bound, int* out,
                      double* dist, int max_out)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  Ctx c;
  c.init(R, E, masks);
  double qd[ORC_MAXL];
  for (int i = 0; i < R->L; ++i) qd[i] = (double)q[i];
  c.set_config(qd);
  int n = 0;
  for (int l = 0; l < R->L; ++l) {
    if (R->bvh[l].empty()) continue;
    for (int o = 0; o < E->N; ++o) {
      if (!pair_enabled(c, l, o)) continue;
      if (link_obj_lb(c, l, o) > std::max(bound, 0.0) + 1e-9) continue;
      PairResult pr = pair_distance(c, l, o, bound);
      if (!pr.found) continue;
      if (n < max_out) {
        int* r = out + 5 * (size_t)n;
        r[0] = l; r[1] = o; r[2] = pr.ta; r[3] = pr.tb; r[4] = pr.signed_pen;
        dist[n] = pr.d;
      }
      ++n;
    }
  }
  return n;
}

/* Free-geometry pair queries (the engine's kgpu_geom_collide /
 * kgpu_geom_distance; Geometry3D::collides / withinDistance / distance_ext,
 * Python/klampt/src/robotsim.cpp:1656-1690, 1782-1819).  `robot` is an oracle
 * robot of two links: link 0 holds geometry a's mesh and margin, link 1
 * geometry b's; their world transforms are Ta[b], Tb[b] (stride 0 under the
 * fixed flags 1 / 2).  collide: the pair is within (m_a + tol) + m_b
 * (tol = 0 and no margins: the triangles meet).  distance: d_mesh searched
 * below max(upper + (m_a + m_b), 0) (accepting d^2 below the square of that
 * bound, or 1e-300), reported as d_mesh - (m_a + m_b), else `upper`. */
int orc_geom_collide(void* robot, const double* Ta, const double* Tb, int B, int flags, double tol, uint8_t* hit,
                     int nthreads)
{
  Robot* R = (Robot*)robot;
  if (R->L != 2) return -1;
  parallel_for(B, nthreads, [&](int, int b0, int b1) {
    Ctx c;
    c.init(R, nullptr, nullptr);
    for (int b = b0; b < b1; ++b) {
      const double* Ts[2] = {Ta + ((flags & 1) ? 0 : 12 * (size_t)b), Tb + ((flags & 2) ? 0 : 12 * (size_t)b)};
      c.set_transforms(Ts);
      hit[b] = bvtt_collide(c, 0, 1, -1, tol) ? 1 : 0;
    }
  });
  return 0;
}

int orc_geom_distance(void* robot, const double* Ta, const double* Tb, int B, int flags, double upper, double* d,
                      double* cp, int* elem, double* dir, int nthreads)
{
  Robot* R = (Robot*)robot;
  if (R->L != 2) return -1;
  const double msum = R->margins[0] + R->margins[1];
  const double bound = upper < 1e30 ? std::max(0.0, upper + msum) : HUGE_VAL;
  parallel_for(B, nthreads, [&](int, int b0, int b1) {
    Ctx c;
    c.init(R, nullptr, nullptr);
    for (int b = b0; b < b1; ++b) {
      const double* Ts[2] = {Ta + ((flags & 1) ? 0 : 12 * (size_t)b), Tb + ((flags & 2) ? 0 : 12 * (size_t)b)};
      c.set_transforms(Ts);
      PairResult pr = self_pair_distance(c, 0, 1, bound, false);
      d[b] = pr.found ? pr.d - msum : upper;
      elem[2 * b] = pr.found ? pr.ta : -1;
      elem[2 * b + 1] = pr.found ? pr.tb : -1;
      for (int i = 0; i < 3; ++i) {
        cp[6 * b + i] = pr.found ? pr.cp[i] : 0.0;
        cp[6 * b + 3 + i] = pr.found ? pr.cq[i] : 0.0;
        if (dir) dir[3 * b + i] = pr.found && pr.d > 0.0 ? (pr.cp[i] - pr.cq[i]) / pr.d : 0.0;
      }
    }
  });
  return 0;
}

/* minimum signed link-object distance of B configurations, clamped at
 * `cutoff`: d[B], pair[2B] (link, object or -1), cp[6B], grad[B*L] */
int orc_min_distance(void* robot, void* env, const unsigned* masks, const float* q, int B,
                     double cutoff, double* d, int* pair, double* cp, double* grad, int nthreads,
                     long long* counters)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  std::vector<Counters> cs(std::max(1, nthreads));
  parallel_for(B, nthreads, [&](int t, int b0, int b1) {
    Ctx c;
    c.init(R, E, masks);
    c.cnt.items += b1 - b0;
    double qd[ORC_MAXL];
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < R->L; ++i) qd[i] = (double)q[(size_t)b * R->L + i];
      c.set_config(qd);
      MinResult m = min_distance(c, cutoff);
      d[b] = m.d;
      pair[2 * b] = m.link;
      pair[2 * b + 1] = m.obj;
      double* g = grad ? grad + (size_t)b * R->L : nullptr;
      if (g) for (int i = 0; i < R->L; ++i) g[i] = 0;
      for (int i = 0; i < 6; ++i) cp[6 * b + i] = 0;
      if (m.link >= 0) {
        for (int i = 0; i < 3; ++i) {
          cp[6 * b + i] = m.pr.cp[i];
          cp[6 * b + 3 + i] = m.pr.cq[i];
        }
        if (g) feature_gradient(c, m.link, m.pr.cp, m.pr.dir, 1.0, g);
      }
    }
    cs[t].node_pairs += c.cnt.node_pairs;
    cs[t].tri_pairs += c.cnt.tri_pairs;
    cs[t].items += c.cnt.items;
  });
  sum_counters(cs, counters);
  return 0;
}

/* soft-min of the signed distance over all (waypoint, link, object) pairs of
 * each trajectory: L = m - tau*log(sum exp(-(d-m)/tau)), m the trajectory's
 * minimum, summing pairs with d < m + 30 tau (a pair beyond contributes less
 * than e^-30 of the leading term and is left out by definition); dL/dq by the
 * chain rule through each pair's feature point.  q [T*W*L]; Lout [T]; grad
 * [T*W*L] or NULL. */
int orc_softmin(void* robot, void* env, const unsigned* masks, const float* q, int T, int W,
                double tau, double* Lout, double* grad, int nthreads, long long* counters)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  const double K = 30.0;
  std::vector<Counters> cs(std::max(1, nthreads));
  parallel_for(T, nthreads, [&](int th, int t0, int t1) {
    Ctx c;
    c.init(R, E, masks);
    c.cnt.items += (long long)(t1 - t0) * W;
    double qd[ORC_MAXL];
    for (int t = t0; t < t1; ++t) {
      // pass 1: the trajectory minimum (distances searched up to 1000 m)
      double m = 1e300;
      for (int w = 0; w < W; ++w) {
        const float* qw = q + ((size_t)t * W + w) * R->L;
        for (int i = 0; i < R->L; ++i) qd[i] = (double)qw[i];
        c.set_config(qd);
        MinResult r = min_distance(c, 1e3);
        m = std::min(m, r.d);
      }
      double bound = m + K * tau;
      double sum = 0.0;
      std::vector<double> g(W * R->L, 0.0);
      for (int w = 0; w < W; ++w) {
        const float* qw = q + ((size_t)t * W + w) * R->L;
        for (int i = 0; i < R->L; ++i) qd[i] = (double)qw[i];
        c.set_config(qd);
        for (int l = 0; l < R->L; ++l) {
          if (R->bvh[l].empty()) continue;
          for (int o = 0; o < E->N; ++o) {
            if (!pair_enabled(c, l, o)) continue;
            if (link_obj_lb(c, l, o) > std::max(bound, 0.0) + 1e-9) continue;
            PairResult pr = pair_distance(c, l, o, bound);
            if (!pr.found) continue;
            double e = exp(-(pr.d - m) / tau);
            sum += e;
            if (grad) feature_gradient(c, l, pr.cp, pr.dir, e, &g[(size_t)w * R->L]);
          }
        }
      }
      Lout[t] = m - tau * log(sum);
      if (grad) {
        for (size_t k = 0; k < g.size(); ++k) grad[(size_t)t * W * R->L + k] = g[k] / sum;
      }
    }
    cs[th].node_pairs += c.cnt.node_pairs;
    cs[th].tri_pairs += c.cnt.tri_pairs;
    cs[th].items += c.cnt.items;
  });
  sum_counters(cs, counters);
  return 0;
}

/* Batched inverse kinematics, the same Levenberg-Marquardt iteration as the
   engine's (klampt_gb300/csrc/kgpu_ik.cu) in FP64: residual e = [p(q) - p*]
   or [p(q) - p*; 1/2 sum_k R*_k x R_k], steps -J^T (J J^T + mu I)^-1 e on the
   link's ancestor DOFs, clamped to the limits, mu / 4 on an accepted step,
   mu * 8 on a rejected one, converged at max |e_i| <= tol.  q: [B, L] in/out. */
int orc_ik(void* robot, int B, double* q, const int* links, const double* plocal, const double* ptarget,
           const double* Rtarget, int max_iters, double tol, unsigned char* ok, double* residual, int* iters)
{
  Robot* R = (Robot*)robot;
  const int L = R->L;
  const int m = Rtarget ? 6 : 3;
  std::vector<double> T((size_t)L * 12), Tn((size_t)L * 12);
  auto resid = [&](const std::vector<double>& TT, int b, int li, double* e) {
    double p[3];
    kx_xform_point(&TT[12 * (size_t)li], plocal + 3 * (size_t)b, p);
    for (int k = 0; k < 3; ++k) e[k] = p[k] - ptarget[3 * (size_t)b + k];
    if (m == 6) {
      const double* Rt = Rtarget + 9 * (size_t)b;
      const double* Rq = &TT[12 * (size_t)li];
      double ex = 0, ey = 0, ez = 0;
      for (int k = 0; k < 3; ++k) {
        const double ax = Rt[k], ay = Rt[3 + k], az = Rt[6 + k], bx = Rq[k], by = Rq[3 + k], bz = Rq[6 + k];
        ex += ay * bz - az * by;
        ey += az * bx - ax * bz;
        ez += ax * by - ay * bx;
      }
      e[3] = 0.5 * ex;
      e[4] = 0.5 * ey;
      e[5] = 0.5 * ez;
    }
  };
  for (int b = 0; b < B; ++b) {
    double* qb = q + (size_t)b * L;
    const int li = links[b];
    std::vector<char> active(L, 0);
    for (int j = li; j >= 0; j = R->parents[j]) active[j] = R->jtypes[j] != KX_JOINT_WELD;
    for (int i = 0; i < L; ++i) qb[i] = std::min(std::max(qb[i], R->qmin[i]), R->qmax[i]);
    orc_fk(R, qb, T.data());
    double e[6], en[6];
    resid(T, b, li, e);
    double E = 0, emax = 0;
    for (int a = 0; a < m; ++a) { E += e[a] * e[a]; emax = std::max(emax, fabs(e[a])); }
    double mu = 1e-4;
    int it = 0;
    std::vector<double> J((size_t)6 * L), qn(L);
    for (; it < max_iters && emax > tol; ++it) {
      double p[3];
      kx_xform_point(&T[12 * (size_t)li], plocal + 3 * (size_t)b, p);
      std::fill(J.begin(), J.end(), 0.0);
      for (int j = 0; j < L; ++j) {
        if (!active[j]) continue;
        const double* Tj = &T[12 * (size_t)j];
        const double* ax = &R->axes[3 * (size_t)j];
        double w[3];
        for (int r = 0; r < 3; ++r) w[r] = Tj[3 * r] * ax[0] + Tj[3 * r + 1] * ax[1] + Tj[3 * r + 2] * ax[2];
        if (R->jtypes[j] == KX_JOINT_REVOLUTE) {
          const double rx = p[0] - Tj[9], ry = p[1] - Tj[10], rz = p[2] - Tj[11];
          J[0 * L + j] = w[1] * rz - w[2] * ry;
          J[1 * L + j] = w[2] * rx - w[0] * rz;
          J[2 * L + j] = w[0] * ry - w[1] * rx;
          J[3 * L + j] = w[0];
          J[4 * L + j] = w[1];
          J[5 * L + j] = w[2];
        } else {
          J[0 * L + j] = w[0];
          J[1 * L + j] = w[1];
          J[2 * L + j] = w[2];
        }
      }
      double A[6][6], Lc[6][6], y[6], z[6];
      bool spd = true;
      for (int r = 0; r < m; ++r)
        for (int s = 0; s <= r; ++s) {
          double v = 0;
          for (int j = 0; j < L; ++j) v += J[r * L + j] * J[s * L + j];
          A[r][s] = v + (r == s ? mu : 0.0);
        }
      for (int r = 0; r < m; ++r)
        for (int s = 0; s <= r; ++s) {
          double v = A[r][s];
          for (int t = 0; t < s; ++t) v -= Lc[r][t] * Lc[s][t];
          if (s == r) {
            spd = spd && v > 0;
            Lc[r][r] = sqrt(std::max(v, 1e-300));
          } else {
            Lc[r][s] = v / Lc[s][s];
          }
        }
      if (!spd) {
        mu *= 8;
        if (mu > 1e6) break;
        continue;
      }
      for (int r = 0; r < m; ++r) {
        double v = e[r];
        for (int t = 0; t < r; ++t) v -= Lc[r][t] * z[t];
        z[r] = v / Lc[r][r];
      }
      for (int r = m - 1; r >= 0; --r) {
        double v = z[r];
        for (int t = r + 1; t < m; ++t) v -= Lc[t][r] * y[t];
        y[r] = v / Lc[r][r];
      }
      for (int j = 0; j < L; ++j) {
        double dq = 0;
        for (int r = 0; r < m; ++r) dq -= J[r * L + j] * y[r];
        qn[j] = std::min(std::max(qb[j] + dq, R->qmin[j]), R->qmax[j]);
      }
      orc_fk(R, qn.data(), Tn.data());
      resid(Tn, b, li, en);
      double En = 0, enmax = 0;
      for (int a = 0; a < m; ++a) { En += en[a] * en[a]; enmax = std::max(enmax, fabs(en[a])); }
      if (En < E) {
        for (int j = 0; j < L; ++j) qb[j] = qn[j];
        T.swap(Tn);
        for (int a = 0; a < m; ++a) e[a] = en[a];
        E = En;
        emax = enmax;
        mu = std::max(mu * 0.25, 1e-10);
      } else {
        mu *= 8;
        if (mu > 1e6) break;
      }
    }
    ok[b] = emax <= tol;
    residual[b] = emax;
    if (iters) iters[b] = it;
  }
  return 0;
}

/* Self-collision pairs occurring over B configurations (the sampling loop of
   RandomizedSelfCollisionPairs, Cpp/Modeling/RandomizedSelfCollisions.cpp:
   19-38): bit j of mask[i] (i < j) is set when enabled pair (i, j) collides
   in some configuration.  mask is OR-accumulated. */
int orc_self_pairs(void* robot, void* env, const float* q, int B, unsigned* mask, int nthreads)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  const int L = R->L;
  std::vector<std::vector<unsigned>> part((size_t)std::max(1, nthreads), std::vector<unsigned>(L, 0u));
  parallel_for(B, nthreads, [&](int t, int b0, int b1) {
    Ctx c;
    std::vector<uint32_t> masks(L, 0u);
    c.init(R, E, masks.data());
    std::vector<double> qd(L);
    std::vector<unsigned>& m = part[t];
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < L; ++i) qd[i] = (double)q[(size_t)b * L + i];
      c.set_config(qd.data());
      for (int i = 0; i < L; ++i)
        for (int j = i + 1; j < L; ++j)
          if (R->self_mask[i * L + j] && !((m[i] >> j) & 1u) && !R->tloc[i].empty() && !R->tloc[j].empty() &&
              bvtt_collide(c, i, j, -1))
            m[i] |= 1u << j;
    }
  });
  for (auto& m : part)
    for (int i = 0; i < L; ++i) mask[i] |= m[i];
  return 0;
}

/* Independent self-collision pairs: the second pass of
   RandomizedIndependentSelfCollisionPairs (TestIndependentCollisions,
   Cpp/Modeling/RandomizedSelfCollisions.cpp:42-66).  Per configuration the
   enabled candidate pairs (bit j of cand[i]) are tested; when exactly one
   collides, its bit is set in mask.  The reference stops counting at the
   second collision; the result is the same. */
int orc_indep_pairs(void* robot, void* env, const float* q, int B, const unsigned* cand, unsigned* mask,
                    int nthreads)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  const int L = R->L;
  std::vector<std::vector<unsigned>> part((size_t)std::max(1, nthreads), std::vector<unsigned>(L, 0u));
  parallel_for(B, nthreads, [&](int t, int b0, int b1) {
    Ctx c;
    std::vector<uint32_t> masks(L, 0u);
    c.init(R, E, masks.data());
    std::vector<double> qd(L);
    std::vector<unsigned>& m = part[t];
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < L; ++i) qd[i] = (double)q[(size_t)b * L + i];
      c.set_config(qd.data());
      int found = 0, fi = 0, fj = 0;
      for (int i = 0; i < L && found < 2; ++i)
        for (int j = i + 1; j < L && found < 2; ++j)
          if (R->self_mask[i * L + j] && ((cand[i] >> j) & 1u) && !R->tloc[i].empty() && !R->tloc[j].empty() &&
              bvtt_collide(c, i, j, -1)) {
            ++found;
            fi = i;
            fj = j;
          }
      if (found == 1) m[fi] |= 1u << fj;
    }
  });
  for (auto& m : part)
    for (int i = 0; i < L; ++i) mask[i] |= m[i];
  return 0;
}

/* Minimum distance between the robot's own links over its enabled self
   pairs: the link-link part of WorldPlannerSettings::DistanceLowerBound when
   a robot is checked against itself (Cpp/Planning/PlannerSettings.cpp:
   385-395).  d = min over enabled pairs i < j of self_pair_distance, pairs
   below `cutoff` only, ties to the smallest (i, j); none: d = cutoff, pair
   (-1, -1).  cp = (point on i, point on j), 0 when none or d = 0; grad[L]
   (may be null) = u . (dcp/dq - dcq/dq), u = (cp - cq) / d, 0 when d = 0. */
int orc_self_distance(void* robot, void* env, const float* q, int B, double cutoff, double* d, int* pair,
                      double* cp, double* grad, int nthreads)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  const int L = R->L;
  parallel_for(B, nthreads, [&](int, int b0, int b1) {
    Ctx c;
    std::vector<uint32_t> masks(L, 0u);
    c.init(R, E, masks.data());
    std::vector<double> qd(L);
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < L; ++i) qd[i] = (double)q[(size_t)b * L + i];
      c.set_config(qd.data());
      double best = cutoff;
      int bi = -1, bj = -1;
      double bcp[3] = {0, 0, 0}, bcq[3] = {0, 0, 0};
      for (int i = 0; i < L && best > 0.0; ++i)
        for (int j = i + 1; j < L && best > 0.0; ++j) {
          if (!R->self_mask[i * L + j] || R->tloc[i].empty() || R->tloc[j].empty()) continue;
          PairResult pr = self_pair_distance(c, i, j, best);
          if (!pr.found) continue;
          best = pr.d;
          bi = i;
          bj = j;
          std::memcpy(bcp, pr.cp, sizeof bcp);
          std::memcpy(bcq, pr.cq, sizeof bcq);
        }
      d[b] = best;
      pair[2 * (size_t)b] = bi;
      pair[2 * (size_t)b + 1] = bj;
      const bool pos = bi >= 0 && best > 0.0;
      for (int k = 0; k < 3; ++k) {
        cp[6 * (size_t)b + k] = pos ? bcp[k] : 0.0;
        cp[6 * (size_t)b + 3 + k] = pos ? bcq[k] : 0.0;
      }
      if (grad) {
        double* g = grad + (size_t)b * L;
        for (int k = 0; k < L; ++k) g[k] = 0.0;
        if (pos) {
          double u[3];
          for (int k = 0; k < 3; ++k) u[k] = (bcp[k] - bcq[k]) / best;
          feature_gradient(c, bi, bcp, u, 1.0, g);
          feature_gradient(c, bj, bcq, u, -1.0, g);
        }
      }
    }
  });
  return 0;
}

/* Each self pair's own minimum distance, clamped at the cutoff (the
   per-sample distances RandomizedSelfCollisionDistances reduces to per-pair
   minima and maxima, Cpp/Modeling/RandomizedSelfCollisions.cpp:142-180):
   dpair[b * P + i*L - i(i+1)/2 + (j-i-1)], P = L(L-1)/2; -1 for pairs not
   queried.  all_pairs: every pair whose links have geometry (that function's
   pair set, :145-151); otherwise the enabled self pairs. */
int orc_self_pair_distances(void* robot, void* env, const float* q, int B, double cutoff, double* dpair,
                            int all_pairs, int nthreads)
{
  Robot* R = (Robot*)robot;
  Env* E = (Env*)env;
  const int L = R->L, P = L * (L - 1) / 2;
  parallel_for(B, nthreads, [&](int, int b0, int b1) {
    Ctx c;
    std::vector<uint32_t> masks(L, 0u);
    c.init(R, E, masks.data());
    std::vector<double> qd(L);
    for (int b = b0; b < b1; ++b) {
      for (int i = 0; i < L; ++i) qd[i] = (double)q[(size_t)b * L + i];
      c.set_config(qd.data());
      double* out = dpair + (size_t)b * P;
      for (int k = 0; k < P; ++k) out[k] = -1.0;
      for (int i = 0; i < L; ++i)
        for (int j = i + 1; j < L; ++j) {
          if ((!all_pairs && !R->self_mask[i * L + j]) || R->tloc[i].empty() || R->tloc[j].empty()) continue;
          PairResult pr = self_pair_distance(c, i, j, cutoff);
          out[i * L - i * (i + 1) / 2 + (j - i - 1)] = pr.found ? pr.d : cutoff;
        }
    }
  });
  return 0;
}

/* Full Jacobians (KrisLibrary GetFullJacobian as called by
   RobotModelLink::getJacobian, Python/klampt/src/robotsim.cpp:4817-4825):
   J[b] = 6 x L row-major, rows 0-2 angular (world axis of each revolute
   ancestor joint), rows 3-5 linear (w x (p - o) revolute, w prismatic) for
   the point plocal[b] on link links[b]. */
int orc_jacobian(void* robot, const float* q, int B, const int* links, const float* plocal, double* J)
{
  Robot* R = (Robot*)robot;
  const int L = R->L;
  std::vector<double> T((size_t)L * 12), qd(L);
  for (int b = 0; b < B; ++b) {
    for (int i = 0; i < L; ++i) qd[i] = (double)q[(size_t)b * L + i];
    orc_fk(R, qd.data(), T.data());
    const int li = links[b];
    double pl[3] = {plocal[3 * (size_t)b], plocal[3 * (size_t)b + 1], plocal[3 * (size_t)b + 2]}, p[3];
    kx_xform_point(&T[12 * (size_t)li], pl, p);
    double* Jb = J + (size_t)b * 6 * L;
    for (int k = 0; k < 6 * L; ++k) Jb[k] = 0.0;
    for (int j = li; j >= 0; j = R->parents[j]) {
      if (R->jtypes[j] == KX_JOINT_WELD) continue;
      const double* Tj = &T[12 * (size_t)j];
      const double* a = &R->axes[3 * (size_t)j];
      double w[3];
      for (int r = 0; r < 3; ++r) w[r] = Tj[3 * r] * a[0] + Tj[3 * r + 1] * a[1] + Tj[3 * r + 2] * a[2];
      if (R->jtypes[j] == KX_JOINT_REVOLUTE) {
        const double rx = p[0] - Tj[9], ry = p[1] - Tj[10], rz = p[2] - Tj[11];
        Jb[0 * L + j] = w[0];
        Jb[1 * L + j] = w[1];
        Jb[2 * L + j] = w[2];
        Jb[3 * L + j] = w[1] * rz - w[2] * ry;
        Jb[4 * L + j] = w[2] * rx - w[0] * rz;
        Jb[5 * L + j] = w[0] * ry - w[1] * rx;
      } else {
        Jb[3 * L + j] = w[0];
        Jb[4 * L + j] = w[1];
        Jb[5 * L + j] = w[2];
      }
    }
  }
  return 0;
}

/* Ray casting against every object of the environment.  s, d: R rays (FP32,
   widened exactly); per ray obj (-1: no hit), tri (triangle index within the
   object's mesh), t (FP64) and the hit point s + t d.  Nearest t, ties to the
   smaller global triangle index (= smaller object, then triangle). */
int orc_raycast(void* env, const float* s, const float* d, int R, int* obj, int* tri, double* tout,
                double* point, int nthreads)
{
  Env* E = (Env*)env;
  parallel_for(R, nthreads, [&](int, int r0, int r1) {
    std::vector<int> st;
    for (int r = r0; r < r1; ++r) {
      double S[3], D[3];
      for (int i = 0; i < 3; ++i) {
        S[i] = (double)s[3 * (size_t)r + i];
        D[i] = (double)d[3 * (size_t)r + i];
      }
      double best = INFINITY;
      int bt = -1;
      for (int g = 0; g < 32; ++g) {
        const Bvh& B = E->group_bvh[g];
        if (B.empty()) continue;
        st.assign(1, 0);
        while (!st.empty()) {
          const Node& n = B.nodes[st.back()];
          st.pop_back();
          // slab test, widened by a relative 1e-9 so that rounding never
          // drops a box the ray touches
          double tn = 0.0, tf = best;
          bool miss = false;
          for (int i = 0; i < 3 && !miss; ++i) {
            const double pad = 1e-9 * (fabs(n.c[i]) + n.h[i] + 1.0);
            const double lo = n.c[i] - n.h[i] - pad, hi = n.c[i] + n.h[i] + pad;
            if (D[i] == 0.0) {
              if (S[i] < lo || S[i] > hi) miss = true;
              continue;
            }
            double a = (lo - S[i]) / D[i], b = (hi - S[i]) / D[i];
            if (a > b) std::swap(a, b);
            a -= 1e-9 * (fabs(a) + 1e-9);
            b += 1e-9 * (fabs(b) + 1e-9);
            tn = std::max(tn, a);
            tf = std::min(tf, b);
            if (tn > tf) miss = true;
          }
          if (miss) continue;
          if (n.left < 0) {
            for (int k = n.first; k < n.first + n.count; ++k) {
              const int t = B.order[k];
              double tt;
              if (kx_ray_tri(S, D, &E->tri[9 * (size_t)t], &tt) && (tt < best || (tt == best && t < bt))) {
                best = tt;
                bt = t;
              }
            }
          } else {
            st.push_back(n.left + 1);
            st.push_back(n.left);
          }
        }
      }
      if (bt < 0) {
        obj[r] = -1;
        tri[r] = -1;
        tout[r] = INFINITY;
        for (int i = 0; i < 3; ++i) point[3 * (size_t)r + i] = 0.0;
      } else {
        obj[r] = E->tri_obj[bt];
        tri[r] = bt - E->obj_first[obj[r]];
        tout[r] = best;
        for (int i = 0; i < 3; ++i) point[3 * (size_t)r + i] = kx_add(S[i], kx_mul(best, D[i]));
      }
    }
  });
  return 0;
}

}  // extern "C"
