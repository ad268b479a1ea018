// kgpu_dist.cu — signed link-obstacle distance, its minimum per configuration,
// the soft-min over a trajectory, and the adjoint (gradient) kernels.
//
// Replaces the per-pair Geometry3D::distance_ext loop
// (Python/klampt/src/robotsim.cpp:1782-1819; DistanceQueryResult conventions
// Python/klampt/src/geometry.h:641-673), WorldPlannerSettings::
// DistanceLowerBound (Cpp/Planning/PlannerSettings.cpp:372-483) and the
// autodiff MinDistance / ADModule path (Python/klampt/math/autodiff/
// geometry_ad.py:613-814, pytorch.py:72-115).
//
// Definition (the FP64 oracle's, bit for bit on the value):
//   d(l, o) = min over triangle pairs of the canonical triangle distance
//             (kx_tri_tri_dist2), ties to the smallest (link triangle, object
//             triangle) index;  if that is 0 (surfaces meet) and o is convex,
//             d = -(largest depth of a link vertex inside o), depth(v) =
//             min over o's faces of (n_f . a_f - n_f . v), 0 if no vertex is
//             strictly inside.
//   min distance  = min over enabled (link, object) pairs, ties to the
//                   smallest (link, object);
//   soft-min      = m - tau log sum exp(-(d - m)/tau) over the trajectory's
//                   pairs with d < m + K tau (K = 30), m the trajectory minimum.
//
// GPU method, one warp per configuration (waypoint):
//   * FP32 FK with per-link error bounds (warp_fk32);
//   * candidate (link, object) pairs from the object-aware environment tree by
//     box lower bounds, evaluated nearest first; for the minimum, the bound
//     starts at 5 cm and grows x4 until a pair is found below it;
//   * per pair a warp-cooperative BVH-vs-BVH distance traversal in FP32 with
//     conservative pruning; triangle pairs whose FP32 distance lies within the
//     error band of the running minimum become candidates and are finalised
//     in canonical FP64 (one pair per lane, lexicographic warp reduction);
//     a pair certified intersecting in FP32 ends the search (distance 0);
//   * depth: link vertices inside the object's box, FP32 min over faces,
//     FP64 for those within the band of the deepest;
//   * gradient: dd/dq_j = u . (w_j x (p - o_j)) (revolute), u . w_j
//     (prismatic), with u = dd/dp at the link feature point p, accumulated as
//     per-link force/moment sums and pulled back through the chain once per
//     configuration (the adjoint of FK), on FP32 transforms.
#include <cfloat>
#include <climits>

#include "kgpu_device.cuh"
#include "kgpu_dist32.cuh"

namespace kgpu {

namespace {

constexpr int kDW = 8;         // warps per block
constexpr int kDStack = 512;   // node-pair stack entries per warp
constexpr int kDGStack = 512;  // environment-tree stack for gathering objects
constexpr int kDJobs = 64;     // leaf-pair jobs
constexpr int kDCand = 64;     // FP64 triangle-pair candidates
constexpr int kDPairs = 128;   // gathered (link, object) candidates
constexpr double kSoftK = 30.0;  // pairs beyond m + 30 tau weigh < e^-30 of the leading term

struct __align__(16) DistSmem {
  uint2 stack[kDStack];
  uint32_t gstack[kDGStack];
  uint32_t jobA[kDJobs], jobB[kDJobs], jobOff[kDJobs + 1];
  uint32_t candA[kDCand], candB[kDCand];
  float candD[kDCand];
  int pobj[kDPairs];
  int plink[kDPairs];
  float plb[kDPairs];
  float T[kMaxLinks][12];
  float delta[kMaxLinks];
  float F[kMaxLinks][3], M[kMaxLinks][3];
  double q64[kMaxLinks];
  const float* item_qa;
  const float* item_qb;
  int item_k, item_n;
  // running exact best of the current pair (FP64 finalisation)
  double b2;
  int bA, bB;
  double bcp[3], bcq[3];
};

struct DistArgs {
  int mode;            // 0 min distance, 1 soft-min pass 1 (minimum), 2 soft-min pass 2
  int robot;
  const float* q;      // [B, L]
  int B;
  double cutoff;
  double* d;           // [B]
  int* pair;           // [B*2]
  double* cp;          // [B*6]
  float* grad;         // [B*L] (mode 0: dd/dq, mode 2: unnormalised soft-min gradient)
  const double* m_traj;  // mode 2: [T] trajectory minima
  double* wsum;        // mode 2: [B] per-waypoint sums
  int W;               // waypoints per trajectory
  double tau;
  unsigned int* head;
  uint2* scratch;
  int scratch_per_warp;
};

struct DCnt {
  unsigned long long pairs = 0, tri = 0, band = 0, nodes = 0;
};

__device__ __forceinline__ double item_q64(const DistSmem& S, int lane)
{
  if (S.item_qb == nullptr) return (double)S.item_qa[lane];
  return kx_interp((double)S.item_qa[lane], (double)S.item_qb[lane], S.item_k, S.item_n);
}

__device__ __noinline__ void dist_fk64(DistSmem& S, const KRobotDev& R, double (*T64)[12], int lane, int& fk64)
{
  if (fk64) return;
  if (lane < R.nlinks) S.q64[lane] = item_q64(S, lane);
  __syncwarp();
  warp_fk64(R, S.q64, T64, lane);
  fk64 = 1;
}

// FP64 finalisation of the pending candidates of pair (l, o): exact squared
// distances, merged into the running lexicographic best (S.b2, S.bA, S.bB).
__device__ __noinline__ void flush_cands(DistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                         double (*T64)[12], int& fk64, int lane, int l, int ncand, DCnt& cnt)
{
  dist_fk64(S, R, T64, lane, fk64);
  for (int base = 0; base < ncand; base += 32) {
    const int k = base + lane;
    double d2 = DBL_MAX;
    int oa = INT_MAX, ob = INT_MAX;
    double cp[3] = {0, 0, 0}, cq[3] = {0, 0, 0};
    if (k < ncand) {
      const int tA = (int)S.candA[k], tB = (int)S.candB[k];
      double P[9], Q[9];
      const double* pa = W->ltri64 + 9 * (size_t)tA;
      for (int v = 0; v < 3; ++v) kx_xform_point(T64[l], pa + 3 * v, P + 3 * v);
      const double* pb = W->etri64 + 9 * (size_t)tB;
      for (int i = 0; i < 9; ++i) Q[i] = pb[i];
      d2 = kx_tri_tri_dist2(P, Q, cp, cq);
      oa = W->ltri_orig[tA];
      ob = W->etri_orig[tB];
      cnt.band++;
    }
    int src;
    double m2 = d2;
    int ma = oa, mb = ob;
    warp_lexmin(m2, ma, mb, src, lane);
    const bool better = m2 < S.b2 || (m2 == S.b2 && (ma < S.bA || (ma == S.bA && mb < S.bB)));
    __syncwarp();
    if (better && lane == src) {
      S.b2 = d2;
      S.bA = oa;
      S.bB = ob;
      for (int i = 0; i < 3; ++i) { S.bcp[i] = cp[i]; S.bcq[i] = cq[i]; }
    }
    __syncwarp();
  }
}

// An upper bound on the distance between the surfaces of link l and object
// o: the link vertex nearest the centre of o's box and the vertex of o (the
// first vertex of each of its triangles) nearest that link vertex are both
// surface points; widened by the FP32 placement bounds and rounding.  Seeds
// a pair's running minimum, so that its traversal prunes from the start.
constexpr int kSeedMaxTris = 4096;  // objects up to this size are scanned for a seed

__device__ __noinline__ float pair_seed(DistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R, int lane,
                                        int l, int o)
{
  const int ff = W->obj_leaf_first[o], fc = W->obj_leaf_count[o];
  if (fc > kSeedMaxTris) return FLT_MAX;  // large objects (terrains): no seed
  const KNode ob = W->enodes[W->obj_root[o]];
  const float* TA = S.T[l];
  const int vf = R.link_vert_first[l], vc = R.link_vert_count[l];
  float bd = FLT_MAX;
  float3 bv = make_float3(ob.a.x, ob.a.y, ob.a.z);
  for (int v = lane; v < vc; v += 32) {
    const float4 x = __ldg(W->lvert32 + vf + v);
    const float3 w = xform32(TA, make_float3(x.x, x.y, x.z));
    const float dx = w.x - ob.a.x, dy = w.y - ob.a.y, dz = w.z - ob.a.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < bd) { bd = d2; bv = w; }
  }
  const float m = warp_min(bd);
  if (!(m < FLT_MAX)) return FLT_MAX;  // no vertex: no surface point, no seed
  const unsigned mm = __ballot_sync(0xffffffffu, bd == m);
  const int src = __ffs(mm) - 1;
  bv = make_float3(__shfl_sync(0xffffffffu, bv.x, src), __shfl_sync(0xffffffffu, bv.y, src),
                   __shfl_sync(0xffffffffu, bv.z, src));
  float bo = FLT_MAX;
  for (int t = lane; t < fc; t += 32) {
    const float4 y = __ldg(W->etri32 + 3 * (size_t)(ff + t));
    const float dx = y.x - bv.x, dy = y.y - bv.y, dz = y.z - bv.z;
    bo = fminf(bo, dx * dx + dy * dy + dz * dz);
  }
  bo = warp_min(bo);
  if (!(bo < FLT_MAX)) return FLT_MAX;
  return sqrtf(bo) * (1.f + 1e-5f) + 2.f * (S.delta[l] + W->eps_env + 2.f * W->eps_extra) + 1e-6f;
}

struct PairOut {
  int found;
  double d;
  double cp[3], cq[3];
  float dir[3];
};

// Signed distance of (link l, object o) below `bound` (found = d < bound).
__device__ __noinline__ void eval_pair(DistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                       double (*T64)[12], int& fk64, int lane, int l, int o, double bound,
                                       PairOut& out, DCnt& cnt, float seed = FLT_MAX)
{
  cnt.pairs++;
  const unsigned lt = lanemask_lt();
  const float dl = S.delta[l] + W->eps_extra;
  const float de = W->eps_env + W->eps_extra;
  const float fb = bound > 0.0 ? (bound < 1e30 ? (float)bound * 1.000001f + 1e-7f : FLT_MAX) : 0.f;
  float m32 = seed;  // running FP32 minimum (warp-uniform); seed: an upper bound known in advance
  bool overlap = false;
  int top = 0, njobs = 0, ncand = 0;
  int certA = -1;  // link triangle of the certified contact
  if (lane == 0) {
    S.b2 = DBL_MAX;
    S.bA = INT_MAX;
    S.bB = INT_MAX;
    S.stack[0] = make_uint2((uint32_t)W->obj_root[o], (uint32_t)R.link_root[l]);
  }
  __syncwarp();
  top = 1;
  const float* TA = S.T[l];
#pragma unroll 1
  while (top > 0 || njobs > 0) {
    // triangle jobs are tested early (16 at a time): the running minimum they
    // produce is what prunes the rest of the traversal
    if (njobs >= 16 || (top == 0 && njobs > 0)) {
      // ---- triangle pairs, one per lane
      uint32_t carry = 0;
      for (int b = 0; b < njobs; b += 32) {
        const int j = b + lane;
        uint32_t c = 0;
        if (j < njobs) c = ((S.jobA[j] >> 28) + 1) * ((S.jobB[j] >> 28) + 1);
        uint32_t incl = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
          if (lane >= off) incl += v;
        }
        if (j < njobs) S.jobOff[j] = carry + incl - c;
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
      __syncwarp();
      const uint32_t total = carry;
#pragma unroll 1
      for (uint32_t base = 0; base < total && !overlap; base += 32) {
        const uint32_t p = base + lane;
        float d32 = FLT_MAX, e = 0.f;
        bool certain = false;
        int tA = 0, tB = 0;
        if (p < total) {
          int lo = 0, hi = njobs - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.jobOff[mid] <= p) lo = mid; else hi = mid - 1;
          }
          const uint32_t r = p - S.jobOff[lo];
          const uint32_t cb = (S.jobB[lo] >> 28) + 1;
          tA = (int)(S.jobA[lo] & 0x0fffffffu) + (int)(r / cb);
          tB = (int)(S.jobB[lo] & 0x0fffffffu) + (int)(r % cb);
          float3 P[3], Q[3];
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const float4 x = __ldg(W->ltri32 + 3 * (size_t)tA + v);
            P[v] = xform32(TA, make_float3(x.x, x.y, x.z));
            const float4 y = __ldg(W->etri32 + 3 * (size_t)tB + v);
            Q[v] = make_float3(y.x, y.y, y.z);
          }
          float3 lo3 = P[0], hi3 = P[0];
#pragma unroll
          for (int k = 1; k < 6; ++k) {
            const float3 v = k < 3 ? P[k] : Q[k - 3];
            lo3 = make_float3(fminf(lo3.x, v.x), fminf(lo3.y, v.y), fminf(lo3.z, v.z));
            hi3 = make_float3(fmaxf(hi3.x, v.x), fmaxf(hi3.y, v.y), fmaxf(hi3.z, v.z));
          }
          const float span = fmaxf(fmaxf(hi3.x - lo3.x, hi3.y - lo3.y), hi3.z - lo3.z);
          e = dl + de + 128.f * kU * span + 1e-8f;
          // triangle-box lower bound: skip the full distance when it cannot
          // be a candidate
          float3 pl = P[0], ph = P[0], ql = Q[0], qh = Q[0];
#pragma unroll
          for (int k = 1; k < 3; ++k) {
            pl = make_float3(fminf(pl.x, P[k].x), fminf(pl.y, P[k].y), fminf(pl.z, P[k].z));
            ph = make_float3(fmaxf(ph.x, P[k].x), fmaxf(ph.y, P[k].y), fmaxf(ph.z, P[k].z));
            ql = make_float3(fminf(ql.x, Q[k].x), fminf(ql.y, Q[k].y), fminf(ql.z, Q[k].z));
            qh = make_float3(fmaxf(qh.x, Q[k].x), fmaxf(qh.y, Q[k].y), fmaxf(qh.z, Q[k].z));
          }
          const float gx = fmaxf(0.f, fmaxf(ql.x - ph.x, pl.x - qh.x));
          const float gy = fmaxf(0.f, fmaxf(ql.y - ph.y, pl.y - qh.y));
          const float gz = fmaxf(0.f, fmaxf(ql.z - ph.z, pl.z - qh.z));
          const float blb = sqrtf(gx * gx + gy * gy + gz * gz) * (1.f - 4.f * kU);
          const float skip = fminf(m32 * (1.f + 2e-5f) + 2.f * e, fb + e);
          if (blb - e > skip || tri_axis_lb32(P, Q, span) - e > skip) {
            d32 = FLT_MAX;  // not a candidate (and no better than the running minimum)
          } else if (!tri_separated32(P, Q, dl + de, 0.f)) {
            d32 = 0.f;
            certain = tri_certain_hit32(P[0], P[1], P[2], Q[0], Q[1], Q[2], fmaxf(dl, de));
          } else {
            d32 = sqrtf(tri_dist2_32(P, Q));
          }
          cnt.tri++;
        }
        const unsigned mc = __ballot_sync(0xffffffffu, certain);
        if (mc) {
          overlap = true;
          const int src = __ffs(mc) - 1;
          certA = __shfl_sync(0xffffffffu, tA, src);
          break;
        }
        m32 = fminf(m32, warp_min(d32));
        const float emax = warp_min(-e) * -1.f;  // largest band in this batch
        const float lim = fminf(m32 * (1.f + 2e-5f) + 2.f * emax, fb + emax);
        const bool cand = p < total && d32 - e <= lim;
        const unsigned mcand = __ballot_sync(0xffffffffu, cand);
        if (ncand + __popc(mcand) > kDCand) {
          flush_cands(S, W, R, T64, fk64, lane, l, ncand, cnt);
          ncand = 0;
          if (S.b2 < DBL_MAX) m32 = fminf(m32, (float)sqrt(S.b2) * (1.f + 1e-6f));
        }
        if (cand) {
          const int r = ncand + __popc(mcand & lt);
          S.candA[r] = (uint32_t)tA;
          S.candB[r] = (uint32_t)tB;
          S.candD[r] = d32 - e;
        }
        ncand += __popc(mcand);
        __syncwarp();
      }
      njobs = 0;
      if (overlap) break;
      continue;
    }
    // ---- node pairs.  A batch of n pops grows the stack by at most n; near
    // the capacity the batch narrows down to plain depth-first order (one
    // pair), whose growth is bounded by the depth of the two trees, so a
    // wide front (a link deep inside an obstacle, where no box is pruned)
    // does not overflow the stack
    const int n = min(min(top, 32), max(1, kDStack - 64 - top));
    const bool have = lane < n;
    uint2 en = make_uint2(0, 0);
    if (have) en = S.stack[top - 1 - lane];
    __syncwarp();
    top -= n;
    int outcome = 0;
    uint2 c0 = make_uint2(0, 0), c1 = make_uint2(0, 0);
    uint32_t jA = 0, jB = 0;
    cnt.nodes += have ? 1 : 0;
    if (have) {
      const int nodeB = (int)en.x, nodeA = (int)en.y;
      const KNode na = W->lnodes[nodeA];
      const KNode nb = W->enodes[nodeB];
      const Box32 A = xform_box(TA, na.a, na.b);
      const float slack = 4.f * kU * (fabsf(A.c.x) + fabsf(A.c.y) + fabsf(A.c.z) + 1.f);
      const float lb_box = box_dist32(A, make_float3(nb.a.x, nb.a.y, nb.a.z), make_float3(nb.b.x, nb.b.y, nb.b.z)) -
                           (dl + de) * 1.7321f - slack;
      // the rotation-invariant sphere about the node centre is tighter than the
      // world box of a rotated node in most directions
      const float gx = fmaxf(0.f, fabsf(A.c.x - nb.a.x) - nb.b.x);
      const float gy = fmaxf(0.f, fabsf(A.c.y - nb.a.y) - nb.b.y);
      const float gz = fmaxf(0.f, fabsf(A.c.z - nb.a.z) - nb.b.z);
      const float lb_sph = sqrtf(gx * gx + gy * gy + gz * gz) * (1.f - 4.f * kU) - __ldg(W->lnode_r + nodeA) -
                           (dl + de) * 1.7321f - slack;
      const float lb = fmaxf(lb_box, lb_sph);
      const float lim = fminf(m32 * (1.f + 2e-5f) + 3.f * (dl + de) + 1e-5f, fb + 2.f * (dl + de) + 1e-5f);
      if (lb <= lim) {
        const int cntA = f2i(na.b.w), cntB = f2i(nb.b.w);
        const int ia = f2i(na.a.w), ib = f2i(nb.a.w);
        if (cntA > 0 && cntB > 0) {
          outcome = 2;
          jA = (uint32_t)ia | ((uint32_t)(cntA - 1) << 28);
          jB = (uint32_t)ib | ((uint32_t)(cntB - 1) << 28);
        } else {
          outcome = 1;
          const bool splitB = cntA > 0 || (cntB == 0 && (nb.b.x + nb.b.y + nb.b.z) > (na.b.x + na.b.y + na.b.z));
          if (splitB) { c0 = make_uint2((uint32_t)ib, (uint32_t)nodeA); c1 = make_uint2((uint32_t)ib + 1, (uint32_t)nodeA); }
          else { c0 = make_uint2((uint32_t)nodeB, (uint32_t)ia); c1 = make_uint2((uint32_t)nodeB, (uint32_t)ia + 1); }
        }
      }
    }
    const unsigned m1 = __ballot_sync(0xffffffffu, outcome == 1);
    const unsigned m2 = __ballot_sync(0xffffffffu, outcome == 2);
    if (top + 2 * __popc(m1) > kDStack) {
      // stack would overflow: the pair is evaluated conservatively by giving up
      // pruning precision is not an option, so flag and stop
      if (lane == 0) set_status(W->status, KGPU_ERR_OVERFLOW);
      out.found = 0;
      return;
    }
    if (outcome == 1) {
      const int r = top + 2 * __popc(m1 & lt);
      S.stack[r] = c1;
      S.stack[r + 1] = c0;
    } else if (outcome == 2) {
      const int r = njobs + __popc(m2 & lt);
      S.jobA[r] = jA;
      S.jobB[r] = jB;
    }
    top += 2 * __popc(m1);
    njobs += __popc(m2);
    __syncwarp();
  }

  // ---- unsigned distance: exact zero (certified contact) or FP64 finalisation
  bool zero = overlap;
  if (!overlap) {
    // drop stale candidates, then finalise
    const float lim = fminf(m32 * (1.f + 2e-5f), fb);
    int keep = 0;
    for (int base = 0; base < ncand; base += 32) {
      const int k = base + lane;
      bool ok = false;
      uint32_t a = 0, b = 0;
      float dd = 0.f;
      if (k < ncand) {
        a = S.candA[k]; b = S.candB[k]; dd = S.candD[k];
        ok = dd <= lim + 1e-6f;
      }
      __syncwarp();
      const unsigned mk = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        const int r = keep + __popc(mk & lt);
        S.candA[r] = a; S.candB[r] = b; S.candD[r] = dd;
      }
      keep += __popc(mk);
      __syncwarp();
    }
    if (keep > 0) flush_cands(S, W, R, T64, fk64, lane, l, keep, cnt);
    if (S.b2 == DBL_MAX) { out.found = 0; return; }
    zero = S.b2 == 0.0;
  }
  if (!zero) {
    const double d = kx_sqrt(S.b2);
    out.found = d < bound;
    out.d = d;
    for (int i = 0; i < 3; ++i) {
      out.cp[i] = S.bcp[i];
      out.cq[i] = S.bcq[i];
      out.dir[i] = (float)((S.bcp[i] - S.bcq[i]) / d);
    }
    return;
  }
  // ---- surfaces meet
  int vbest = -1, fbest = -1;
  double depth = 0.0;
  if (W->obj_convex[o]) {
    // deepest link vertex inside the convex object
    const int vf = R.link_vert_first[l], vc = R.link_vert_count[l];
    const KNode ob = W->enodes[W->obj_root[o]];
    const float tolb = dl + de + 8.f * kU * (fabsf(ob.a.x) + fabsf(ob.a.y) + fabsf(ob.a.z) + 1.f);
    const int ff = W->obj_leaf_first[o], fc = W->obj_leaf_count[o];
    const float ed = dl + de + 32.f * kU * (fabsf(ob.a.x) + fabsf(ob.a.y) + fabsf(ob.a.z) + fabsf(ob.b.x) +
                                           fabsf(ob.b.y) + fabsf(ob.b.z) + 1.f);
    float lmax = -FLT_MAX;
    // pass 1: FP32 depths, lane-local maximum.  Each lane also keeps the (at
    // most two) vertices whose pass-1 value lies within 2 ed of its running
    // maximum: pass 1's value bounds a vertex's full FP32 minimum from
    // above, and the global maximum is at least the lane's, so every vertex
    // that pass 2 can accept is among them, unless more than two qualified
    // (then the lane rescans all of its vertices)
    int cv0 = 0, cv1 = 0, nc = 0;
    float cd0 = 0.f, cd1 = 0.f;
    bool rescan = false;
    for (int v = lane; v < vc; v += 32) {
      const float4 x = __ldg(W->lvert32 + vf + v);
      const float3 w = xform32(TA, make_float3(x.x, x.y, x.z));
      if (fabsf(w.x - ob.a.x) > ob.b.x + tolb || fabsf(w.y - ob.a.y) > ob.b.y + tolb ||
          fabsf(w.z - ob.a.z) > ob.b.z + tolb)
        continue;
      // a vertex stops counting once it is no deeper than the deepest so far
      // (or outside the band): its final minimum can only be lower
      const float stop = fmaxf(lmax, -ed);
      float dmin = FLT_MAX;
      for (int f = ff; f < ff + fc && dmin > stop; ++f) {
        const float4 pl = __ldg(W->eface32 + f);
        dmin = fminf(dmin, pl.w - (pl.x * w.x + pl.y * w.y + pl.z * w.z));
      }
      lmax = fmaxf(lmax, dmin);
      const float thr = lmax - 2.f * ed;
      if (dmin > -ed && dmin >= thr) {
        if (nc == 2 && cd1 < thr) nc = 1;
        if (nc >= 1 && cd0 < thr) {
          if (nc == 2) { cv0 = cv1; cd0 = cd1; }
          --nc;
        }
        if (nc == 0) { cv0 = v; cd0 = dmin; nc = 1; }
        else if (nc == 1) { cv1 = v; cd1 = dmin; nc = 2; }
        else rescan = true;
      }
    }
    const float gmax = -warp_min(-lmax);
    if (gmax > -ed) {
      dist_fk64(S, R, T64, lane, fk64);
      // pass 2: FP64 depth of every vertex within the band of the deepest
      double bd = 0.0;
      int bv = INT_MAX, bf = -1;
      auto depth64 = [&](int v) {
        const float4 x = __ldg(W->lvert32 + vf + v);
        const float3 w = xform32(TA, make_float3(x.x, x.y, x.z));
        if (fabsf(w.x - ob.a.x) > ob.b.x + tolb || fabsf(w.y - ob.a.y) > ob.b.y + tolb ||
            fabsf(w.z - ob.a.z) > ob.b.z + tolb)
          return;
        const float stop = fmaxf(gmax - 2.f * ed, -ed);
        float dmin = FLT_MAX;
        for (int f = ff; f < ff + fc && dmin >= stop; ++f) {
          const float4 pl = __ldg(W->eface32 + f);
          dmin = fminf(dmin, pl.w - (pl.x * w.x + pl.y * w.y + pl.z * w.z));
        }
        if (dmin < gmax - 2.f * ed || dmin <= -ed) return;
        double w64[3];
        kx_xform_point(T64[l], W->lvert64 + 3 * (size_t)(vf + v), w64);
        double dm = DBL_MAX;
        int fm = -1, fo = INT_MAX;
        for (int f = ff; f < ff + fc; ++f) {
          const double* pl = W->eface64 + 4 * (size_t)f;
          const double dep = kx_sub(pl[3], kx_dot3(pl, w64));
          const int orig = W->etri_orig[f];
          if (dep < dm || (dep == dm && orig < fo)) { dm = dep; fm = f; fo = orig; }
        }
        if (dm > bd || (dm == bd && dm > 0.0 && v < bv)) { bd = dm; bv = v; bf = fm; }
      };
      if (rescan) {
        for (int v = lane; v < vc; v += 32) depth64(v);
      } else {
        if (nc >= 1 && cd0 >= gmax - 2.f * ed) depth64(cv0);
        if (nc >= 2 && cd1 >= gmax - 2.f * ed) depth64(cv1);
      }
      // warp maximum of (depth, -vertex)
      double wd = bd;
      int wv = bd > 0.0 ? bv : INT_MAX, wf = bf, src = lane;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, wd, off);
        const int ov = __shfl_xor_sync(0xffffffffu, wv, off);
        const int ofc = __shfl_xor_sync(0xffffffffu, wf, off);
        const int os = __shfl_xor_sync(0xffffffffu, src, off);
        if (od > wd || (od == wd && (ov < wv || (ov == wv && os < src)))) { wd = od; wv = ov; wf = ofc; src = os; }
      }
      if (wd > 0.0) {
        depth = wd;
        vbest = wv;
        fbest = wf;
      }
    }
  }
  if (vbest >= 0) {
    double w64[3];
    kx_xform_point(T64[l], W->lvert64 + 3 * (size_t)(R.link_vert_first[l] + vbest), w64);
    const double* pl = W->eface64 + 4 * (size_t)fbest;
    out.d = -depth;
    out.found = -depth < bound;
    for (int i = 0; i < 3; ++i) {
      out.cp[i] = w64[i];
      out.cq[i] = kx_add(w64[i], kx_mul(depth, pl[i]));
      out.dir[i] = (float)pl[i];
    }
    return;
  }
  // contact without a vertex inside (or a non-convex object): d = 0, no direction
  out.d = 0.0;
  out.found = 0.0 < bound;
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
  if (certA >= 0) x = __ldg(W->ltri32 + 3 * (size_t)certA);
  const float3 w = xform32(TA, make_float3(x.x, x.y, x.z));
  out.cp[0] = out.cq[0] = w.x;
  out.cp[1] = out.cq[1] = w.y;
  out.cp[2] = out.cq[2] = w.z;
  out.dir[0] = out.dir[1] = out.dir[2] = 0.f;
}

// Gathers objects of group g whose root box is within `bound` of link l's
// world box (lower bound lb in plb) and lb > lower (already handled), into
// S.pobj/plb starting at `count`; stops early when the list is full (the
// caller then evaluates and calls again with `resume` state in the stack).
// Returns the new count; `top` carries the traversal stack between calls.
__device__ int gather_objects(DistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R, int lane, int l,
                              float bound, float lower, int count, int& top)
{
  const unsigned lt = lanemask_lt();
  const KNode la = W->lnodes[R.link_root[l]];
  const Box32 A = xform_box(S.T[l], la.a, la.b);
  const float slack = (S.delta[l] + W->eps_env + 2.f * W->eps_extra) * 1.7321f +
                      4.f * kU * (fabsf(A.c.x) + fabsf(A.c.y) + fabsf(A.c.z) + 1.f) + 1e-7f;
  const float rad = __ldg(W->lnode_r + R.link_root[l]);
  while (top > 0 && count <= kDPairs - 32) {
    if (top > kDGStack - 64) {
      if (lane == 0) set_status(W->status, KGPU_ERR_OVERFLOW);
      top = 0;
      break;
    }
    const int n = min(top, 32);
    const bool have = lane < n;
    int node = 0;
    if (have) node = (int)S.gstack[top - 1 - lane];
    __syncwarp();
    top -= n;
    int outcome = 0;
    float lbv = 0.f;
    int child = 0;
    if (have) {
      const KNode nb = W->enodes[node];
      const float gx = fmaxf(0.f, fabsf(A.c.x - nb.a.x) - nb.b.x);
      const float gy = fmaxf(0.f, fabsf(A.c.y - nb.a.y) - nb.b.y);
      const float gz = fmaxf(0.f, fabsf(A.c.z - nb.a.z) - nb.b.z);
      lbv = fmaxf(box_dist32(A, make_float3(nb.a.x, nb.a.y, nb.a.z), make_float3(nb.b.x, nb.b.y, nb.b.z)),
                  sqrtf(gx * gx + gy * gy + gz * gz) * (1.f - 4.f * kU) - rad) -
            slack;
      if (lbv <= bound) {
        const int o = W->node_obj[node];
        if (o >= 0) {
          outcome = lbv > lower ? 2 : 0;
          child = o;
        } else {
          outcome = 1;
          child = f2i(nb.a.w);
        }
      }
    }
    const unsigned m1 = __ballot_sync(0xffffffffu, outcome == 1);
    const unsigned m2 = __ballot_sync(0xffffffffu, outcome == 2);
    if (outcome == 1) {
      const int r = top + 2 * __popc(m1 & lt);
      S.gstack[r] = (uint32_t)child + 1;
      S.gstack[r + 1] = (uint32_t)child;
    } else if (outcome == 2) {
      const int r = count + __popc(m2 & lt);
      S.pobj[r] = child;
      S.plink[r] = l;
      S.plb[r] = lbv;
    }
    top += 2 * __popc(m1);
    count += __popc(m2);
    __syncwarp();
  }
  return count;
}

// Adds a pair's contribution (weight wgt, feature point p, direction u) to
// the per-link force / moment accumulators.
__device__ __forceinline__ void add_wrench(DistSmem& S, int lane, int l, float wgt, const PairOut& po)
{
  if (lane == 0) {
    const float ux = wgt * po.dir[0], uy = wgt * po.dir[1], uz = wgt * po.dir[2];
    const float px = (float)po.cp[0], py = (float)po.cp[1], pz = (float)po.cp[2];
    S.F[l][0] += ux; S.F[l][1] += uy; S.F[l][2] += uz;
    S.M[l][0] += py * uz - pz * uy;
    S.M[l][1] += pz * ux - px * uz;
    S.M[l][2] += px * uy - py * ux;
  }
  __syncwarp();
}

// Adjoint of FK: gradient g_j = w_j . (M_sub(j) - o_j x F_sub(j)) for a
// revolute joint, w_j . F_sub(j) for a prismatic one, with F_sub/M_sub the
// sums over link j's subtree (children have larger indices than parents).
__device__ void pullback(DistSmem& S, const KRobotDev& R, int lane, float* g_out)
{
  const int nl = R.nlinks;
  if (lane == 0) {
    for (int i = nl - 1; i > 0; --i) {
      const int p = R.parents[i];
      if (p < 0) continue;
      for (int k = 0; k < 3; ++k) {
        S.F[p][k] += S.F[i][k];
        S.M[p][k] += S.M[i][k];
      }
    }
  }
  __syncwarp();
  if (lane < nl && g_out) {
    const float* T = S.T[lane];
    const float wx = T[0] * R.axis[lane][0] + T[1] * R.axis[lane][1] + T[2] * R.axis[lane][2];
    const float wy = T[3] * R.axis[lane][0] + T[4] * R.axis[lane][1] + T[5] * R.axis[lane][2];
    const float wz = T[6] * R.axis[lane][0] + T[7] * R.axis[lane][1] + T[8] * R.axis[lane][2];
    float g = 0.f;
    if (R.jtype[lane] == KX_JOINT_REVOLUTE) {
      const float ox = T[9], oy = T[10], oz = T[11];
      const float* F = S.F[lane];
      const float* M = S.M[lane];
      const float tx = M[0] - (oy * F[2] - oz * F[1]);
      const float ty = M[1] - (oz * F[0] - ox * F[2]);
      const float tz = M[2] - (ox * F[1] - oy * F[0]);
      g = wx * tx + wy * ty + wz * tz;
    } else if (R.jtype[lane] == KX_JOINT_PRISMATIC) {
      g = wx * S.F[lane][0] + wy * S.F[lane][1] + wz * S.F[lane][2];
    }
    g_out[lane] = g;
  }
  __syncwarp();
}

// MODE (A.mode): 0 minimum distance with closest points and gradient, 1
// soft-min pass 1 (waypoint minima), 2 soft-min pass 2 (every pair below
// m + K tau); one instantiation each, so that a launch carries only its
// mode's code
template <int MODE>
__global__ void __launch_bounds__(kDW * 32, 2) k_dist(const KWorldDev* __restrict__ W, const DistArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DistSmem* all = reinterpret_cast<DistSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  DistSmem& S = all[warp];
  const int gwarp = blockIdx.x * kDW + warp;
  double(*T64)[12] = reinterpret_cast<double(*)[12]>(A.scratch + (size_t)gwarp * A.scratch_per_warp);
  const KRobotDev& R = W->robots[A.robot];
  const int nl = R.nlinks;
  DCnt cnt;

  for (;;) {
    unsigned int it = 0;
    if (lane == 0) it = atomicAdd(A.head, 1u);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= (unsigned)A.B) break;
    const int b = (int)it;
    if (lane == 0) {
      S.item_qa = A.q + (size_t)b * nl;
      S.item_qb = nullptr;
      S.item_k = 0;
      S.item_n = 0;
    }
    float q = lane < nl ? __ldg(A.q + (size_t)b * nl + lane) : 0.f;
    __syncwarp();
    if (__any_sync(0xffffffffu, lane < nl && !(fabsf(q) < 1.0e6f))) {
      if (lane == 0) set_status(W->status, KGPU_ERR_NOT_FINITE);
      continue;
    }
    float P[12], delta;
    warp_fk32(R, lane, q, 0.f, P, &delta);
    if (lane < nl) {
      for (int i = 0; i < 12; ++i) S.T[lane][i] = P[i];
      S.delta[lane] = delta;
      S.F[lane][0] = S.F[lane][1] = S.F[lane][2] = 0.f;
      S.M[lane][0] = S.M[lane][1] = S.M[lane][2] = 0.f;
    }
    __syncwarp();
    int fk64 = 0;

    if (MODE == 0 || MODE == 1) {
      // ---- minimum over pairs, iterative deepening of the search bound
      double best = A.cutoff;
      int bl = -1, bo = -1;
      PairOut bp;
      bp.found = 0;
      // rounds: objects whose box lower bound lies in (lower, bound]; done
      // once the best distance is <= bound (every unvisited object is
      // farther) or the bound reached the cutoff
      float lower = -1.f;
      double round_bound = fmin(A.cutoff, 0.05);
      // evaluates the gathered (link, object) pairs nearest first, over all
      // links at once, so that the closest pair of any link sets the bound
      // that prunes the rest
      auto eval_list = [&](int np) {
        for (int done = 0; done < np; ++done) {
          float v = FLT_MAX;
          int idx = -1;
          for (int k = lane; k < np; k += 32)
            if (S.plb[k] < v) { v = S.plb[k]; idx = k; }
          const float vm = warp_min(v);
          const unsigned mm = __ballot_sync(0xffffffffu, v == vm && idx >= 0);
          if (mm == 0u) break;
          const int owner = __ffs(mm) - 1;
          const int k = __shfl_sync(0xffffffffu, idx, owner);
          if (lane == 0) S.plb[k] = FLT_MAX;
          __syncwarp();
          if (vm > (float)fmax(best, 0.0) * 1.00001f + 1e-6f) break;
          const int o = S.pobj[k], l = S.plink[k];
          // a pair cannot go below 0 unless its object is convex, and then
          // not below minus the smallest half-extent of the object's box
          // (no point lies deeper inside a convex body that fits in the
          // box): once the best is at or under that, the pair can at most
          // tie, which only a smaller (link, object) would win
          const double dlow = W->obj_convex[o] ? -(double)fminf(fminf(W->enodes[W->obj_root[o]].b.x,
                                                                       W->enodes[W->obj_root[o]].b.y),
                                                                 W->enodes[W->obj_root[o]].b.z)
                                               : 0.0;
          if (bl >= 0 && (dlow > best || (dlow == best && !(l < bl || (l == bl && o < bo))))) continue;
          PairOut po;
          // the first pair has no running bound to prune with yet: seed it
          eval_pair(S, W, R, T64, fk64, lane, l, o, nextafter(best, 1e300), po, cnt,
                    bl < 0 ? pair_seed(S, W, R, lane, l, o) : FLT_MAX);
          if (po.found && (po.d < best || (po.d == best && (l < bl || (l == bl && o < bo))))) {
            best = po.d;
            bl = l;
            bo = o;
            bp = po;
          }
        }
      };
      for (;;) {
        const float bound = round_bound >= A.cutoff ? FLT_MAX : (float)round_bound * 1.000001f;
        int np = 0;
        for (int l = 0; l < nl; ++l) {
          if (R.link_root[l] < 0) continue;
          for (int g = 0; g < kMaxGroups; ++g) {
            if (!((R.env_mask[l] >> g) & 1u) || W->group_root[g] < 0) continue;
            int top = 1;
            if (lane == 0) S.gstack[0] = (uint32_t)W->group_root[g];
            __syncwarp();
            while (top > 0) {
              // box bounds limit the unsigned distance: a pair can be
              // negative only when its boxes meet, hence max(best, 0)
              const float reach = (float)fmax(best, 0.0) * 1.00001f + 1e-6f;
              np = gather_objects(S, W, R, lane, l, fminf(bound, reach), lower, np, top);
              if (top > 0) {
                // list full: evaluate what it holds, then keep gathering
                eval_list(np);
                np = 0;
              }
            }
          }
        }
        eval_list(np);
        if (best <= round_bound || round_bound >= A.cutoff) break;
        lower = bound;
        round_bound = fmin(A.cutoff, round_bound * 4.0);
      }
      if (lane == 0) {
        A.d[b] = bl >= 0 ? best : A.cutoff;
        if (MODE == 0) {
          A.pair[2 * b] = bl;
          A.pair[2 * b + 1] = bo;
          for (int i = 0; i < 3; ++i) {
            A.cp[6 * b + i] = bl >= 0 ? bp.cp[i] : 0.0;
            A.cp[6 * b + 3 + i] = bl >= 0 ? bp.cq[i] : 0.0;
          }
        }
      }
      if (MODE == 0 && A.grad) {
        if (bl >= 0) add_wrench(S, lane, bl, 1.f, bp);
        pullback(S, R, lane, A.grad + (size_t)b * nl);
      }
    } else {
      // ---- soft-min pass 2: every pair below m + K tau
      const int t = b / A.W;
      const double m = A.m_traj[t];
      const double bnd = m + kSoftK * A.tau;
      double sum = 0.0;
      const float fbnd = (float)fmax(bnd, 0.0) * 1.000001f + 1e-6f;
      for (int l = 0; l < nl; ++l) {
        if (R.link_root[l] < 0) continue;
        for (int g = 0; g < kMaxGroups; ++g) {
          if (!((R.env_mask[l] >> g) & 1u) || W->group_root[g] < 0) continue;
          int top = 1;
          if (lane == 0) S.gstack[0] = (uint32_t)W->group_root[g];
          __syncwarp();
          while (top > 0) {
            const int np = gather_objects(S, W, R, lane, l, fbnd, -1.f, 0, top);
            for (int k = 0; k < np; ++k) {
              PairOut po;
              const int o = S.pobj[k];
              eval_pair(S, W, R, T64, fk64, lane, l, o, bnd, po, cnt, pair_seed(S, W, R, lane, l, o));
              if (!po.found) continue;
              const double e = exp(-(po.d - m) / A.tau);
              sum += e;
              add_wrench(S, lane, l, (float)e, po);
            }
          }
        }
      }
      if (lane == 0) A.wsum[b] = sum;
      pullback(S, R, lane, A.grad ? A.grad + (size_t)b * nl : nullptr);
    }
  }
  // counters: pairs are counted once per warp (lane 0), the rest per lane
  unsigned long long nd = cnt.nodes, tp = cnt.tri, bd = cnt.band;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nd += __shfl_down_sync(0xffffffffu, nd, o);
    tp += __shfl_down_sync(0xffffffffu, tp, o);
    bd += __shfl_down_sync(0xffffffffu, bd, o);
  }
  if (lane == 0 && W->stats) {
    atomicAdd(W->stats + 8, cnt.pairs);
    atomicAdd(W->stats + 9, nd);
    atomicAdd(W->stats + 10, tp);
    atomicAdd(W->stats + 11, bd);
  }
}

// per-trajectory minimum of the waypoint minima
__global__ void k_traj_min(const double* dwp, int T, int Wn, double* m)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double v = dwp[(size_t)t * Wn];
  for (int w = 1; w < Wn; ++w) v = fmin(v, dwp[(size_t)t * Wn + w]);
  m[t] = v;
}

// L = m - tau log(sum), gradient normalised by the sum (waypoints in order)
__global__ void k_softmin_final(const double* wsum, const double* m, int T, int Wn, int L, double tau,
                                double* out, float* grad)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double s = 0.0;
  for (int w = 0; w < Wn; ++w) s += wsum[(size_t)t * Wn + w];
  out[t] = m[t] - tau * log(s);
  if (grad) {
    const float inv = (float)(1.0 / s);
    for (int k = 0; k < Wn * L; ++k) grad[(size_t)t * Wn * L + k] *= inv;
  }
}

// ---- self distance ----------------------------------------------------------
// Minimum distance between the robot's own links over its enabled self pairs
// (the link-link part of WorldPlannerSettings::DistanceLowerBound when a
// robot is checked against itself, Cpp/Planning/PlannerSettings.cpp:385-395,
// and of geometry_ad.MinDistance over link geometries).  Definition (the FP64
// oracle's, bit for bit on the value and the closest points):
//   d(i, j) = sqrt of the minimum canonical triangle distance (kx_tri_tri_dist2)
//             over the pair's triangles, ties to the smallest (triangle of i,
//             triangle of j) in mesh order; 0 when the surfaces meet;
//   d      = min over enabled pairs i < j with d(i, j) < cutoff; pairs are
//            visited in (i, j) order and a pair replaces the best so far
//            only if its squared minimum is below the square of the best
//            distance and its distance is strictly smaller (equal distances
//            keep the earlier pair, even when the squares differ in the last
//            bit); none: d = cutoff and pair (-1, -1).
// Gradient: dd/dq_k = u . (dcp/dq_k - dcq/dq_k), u = (cp - cq) / d at the
// closest points cp on link i and cq on link j (0 when d = 0), from FP64
// transforms.  One warp per configuration: FP32 traversal of each pair with
// conservative pruning against the running upper bound of the minimum,
// triangle pairs within the error band finalised in canonical FP64.
constexpr int kSDStack = 512;
constexpr int kSDJobs = 64;
constexpr int kSDCand = 128;

struct __align__(16) SelfDistSmem;
__device__ __noinline__ float link_pair_seed(SelfDistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                             int lane, int i, int j);

struct __align__(16) SelfDistSmem {
  float T[kMaxLinks][12];
  float delta[kMaxLinks];
  double T64[kMaxLinks][12];
  double q64[kMaxLinks];
  uint2 stack[kSDStack];
  uint32_t jobA[kSDJobs], jobB[kSDJobs], jobOff[kSDJobs + 1];
  uint32_t candA[kSDCand], candB[kSDCand];
  float candD[kSDCand];
  double b2, bcp[3], bcq[3];  // best over the pairs so far: squared distance, closest points
  double bd;                   // its distance (the cutoff before any pair is found)
  int bi, bj;
  double pb2, pcp[3], pcq[3];  // best of the current pair (pb2 starts at the acceptance bound)
  int pA, pB, phave;
};

struct SelfDistArgs {
  int robot;
  const float* q;
  int B;
  double cutoff;
  double* d;       // [B]
  int* pair;       // [B, 2]
  double* cp;      // [B, 6] (point on link i, point on link j)
  float* grad;     // [B, L] or null
  double* dpair;   // per-pair mode: [B, L (L - 1) / 2], each pair's own minimum
  int all_pairs;   // per-pair mode: every pair i < j whose links have geometry, enabled or not
};

// An upper bound on the distance between the surfaces of links i and j:
// the vertex of i nearest the centre of j's root box and the vertex of j
// nearest that vertex (both surface points), widened by the links' FP32
// placement bounds and rounding.
__device__ __noinline__ float link_pair_seed(SelfDistSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                             int lane, int i, int j)
{
  const KNode nj = W->lnodes[R.link_root[j]];
  const float3 cj = xform32(S.T[j], make_float3(nj.a.x, nj.a.y, nj.a.z));
  float bd = FLT_MAX;
  float3 bv = cj;
  {
    const int vf = R.link_vert_first[i], vc = R.link_vert_count[i];
    for (int v = lane; v < vc; v += 32) {
      const float4 x = __ldg(W->lvert32 + vf + v);
      const float3 w = xform32(S.T[i], make_float3(x.x, x.y, x.z));
      const float dx = w.x - cj.x, dy = w.y - cj.y, dz = w.z - cj.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < bd) { bd = d2; bv = w; }
    }
  }
  const float m = warp_min(bd);
  if (!(m < FLT_MAX)) return FLT_MAX;  // no vertex: no surface point, no seed
  const unsigned mm = __ballot_sync(0xffffffffu, bd == m);
  const int src = __ffs(mm) - 1;
  bv = make_float3(__shfl_sync(0xffffffffu, bv.x, src), __shfl_sync(0xffffffffu, bv.y, src),
                   __shfl_sync(0xffffffffu, bv.z, src));
  float bo = FLT_MAX;
  {
    const int vf = R.link_vert_first[j], vc = R.link_vert_count[j];
    for (int v = lane; v < vc; v += 32) {
      const float4 x = __ldg(W->lvert32 + vf + v);
      const float3 w = xform32(S.T[j], make_float3(x.x, x.y, x.z));
      const float dx = w.x - bv.x, dy = w.y - bv.y, dz = w.z - bv.z;
      bo = fminf(bo, dx * dx + dy * dy + dz * dz);
    }
  }
  bo = warp_min(bo);
  if (!(bo < FLT_MAX)) return FLT_MAX;
  return sqrtf(bo) * (1.f + 1e-5f) + 2.f * (S.delta[i] + S.delta[j]) + 1e-6f;
}

// FP64 finalisation of candidates of pair (i, j), merged into the pair's
// best: the lexicographic minimum (squared distance, triangle of i, triangle
// of j) over the triangle pairs whose squared distance is below the pair's
// acceptance bound (the square of the best distance of the earlier pairs)
__device__ __noinline__ void sd_flush(SelfDistSmem& S, const KWorldDev* __restrict__ W, int lane, int i, int j,
                                      int ncand, float lim)
{
  for (int base = 0; base < ncand; base += 32) {
    const int k = base + lane;
    double d2 = DBL_MAX;
    int oa = INT_MAX, ob = INT_MAX;
    double cp[3] = {0, 0, 0}, cq[3] = {0, 0, 0};
    if (k < ncand && S.candD[k] <= lim) {
      const int tA = (int)S.candA[k], tB = (int)S.candB[k];
      double P[9], Q[9];
      const double* pa = W->ltri64 + 9 * (size_t)tA;
      const double* pb = W->ltri64 + 9 * (size_t)tB;
      for (int v = 0; v < 3; ++v) {
        kx_xform_point(S.T64[i], pa + 3 * v, P + 3 * v);
        kx_xform_point(S.T64[j], pb + 3 * v, Q + 3 * v);
      }
      d2 = kx_tri_tri_dist2(P, Q, cp, cq);
      oa = W->ltri_orig[tA];
      ob = W->ltri_orig[tB];
    }
    int src;
    double m2 = d2;
    int ma = oa, mb = ob;
    warp_lexmin(m2, ma, mb, src, lane);
    // below the acceptance bound, or equal to the pair's best with smaller
    // triangles
    const bool better = S.phave ? (m2 < S.pb2 || (m2 == S.pb2 && (ma < S.pA || (ma == S.pA && mb < S.pB))))
                                : m2 < S.pb2;
    __syncwarp();
    if (m2 < DBL_MAX && better && lane == src) {
      S.pb2 = d2;
      S.pA = oa;
      S.pB = ob;
      S.phave = 1;
      for (int c = 0; c < 3; ++c) { S.pcp[c] = cp[c]; S.pcq[c] = cq[c]; }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kDW * 32, 2) k_self_dist(const KWorldDev* __restrict__ W, const SelfDistArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  SelfDistSmem& S = reinterpret_cast<SelfDistSmem*>(smem_raw)[warp];
  const unsigned lt = lanemask_lt();
  const KRobotDev& R = W->robots[A.robot];
  const int nl = R.nlinks;
  const float fcut = A.cutoff < 1e30 ? (float)A.cutoff * 1.000001f + 1e-7f : FLT_MAX;
  const int nwarps = gridDim.x * kDW;
#pragma unroll 1
  for (int b = blockIdx.x * kDW + warp; b < A.B; b += nwarps) {
    const float qv = lane < nl ? __ldg(A.q + (size_t)b * nl + lane) : 0.f;
    if (__any_sync(0xffffffffu, lane < nl && !(fabsf(qv) < 1.0e6f))) {
      if (lane == 0) set_status(W->status, KGPU_ERR_NOT_FINITE);
      continue;
    }
    float P32[12], delta;
    warp_fk32(R, lane, qv, 0.f, P32, &delta);
    if (lane < nl) {
#pragma unroll
      for (int k = 0; k < 12; ++k) S.T[lane][k] = P32[k];
      S.delta[lane] = delta + W->eps_extra;
      S.q64[lane] = (double)qv;
    }
    if (lane == 0) {
      S.b2 = DBL_MAX;
      S.bd = A.cutoff;
      S.bi = S.bj = -1;
    }
    __syncwarp();
    warp_fk64(R, S.q64, S.T64, lane);
    const bool per_pair = A.dpair != nullptr;
    const int npair = nl * (nl - 1) / 2;
    if (per_pair) {
      for (int k = lane; k < npair; k += 32) A.dpair[(size_t)b * npair + k] = -1.0;  // pairs not queried
      __syncwarp();
    }
    float m32 = fcut;  // upper bound on the minimum so far (warp-uniform)
    bool contact = false;
    const int nq = A.all_pairs ? npair : R.nqueries_self;
#pragma unroll 1
    for (int qi = 0; qi < nq && !contact; ++qi) {
      int i, j;
      if (A.all_pairs) {  // qi in upper-triangle order (0,1), (0,2), ..., (L-2, L-1)
        i = 0;
        int r = qi;
        while (r >= nl - 1 - i) { r -= nl - 1 - i; ++i; }
        j = i + 1 + r;
      } else {
        const uint32_t qw = __ldg(W->queries + R.query_off + R.nqueries_env + qi);
        i = qw & 0xff;
        j = (qw >> 8) & 0xff;
      }
      if (R.link_root[i] < 0 || R.link_root[j] < 0) continue;
      const float* TA = S.T[i];
      const float* TB = S.T[j];
      const float dd = S.delta[i] + S.delta[j];
      int top = 1, njobs = 0, ncand = 0;
      bool pc = false;  // certified contact of this pair
      if (per_pair) m32 = fcut;  // every pair on its own
      // a pair without a running bound to prune with (the first, or every
      // pair in per-pair mode) starts from a vertex-pair upper bound of its
      // own distance (>= the running minimum including it, so the bound
      // stays valid for the later pairs)
      if (m32 >= fcut) m32 = fminf(m32, link_pair_seed(S, W, R, lane, i, j));
      if (lane == 0) {
        if (per_pair) S.bd = A.cutoff;
        S.stack[0] = make_uint2((uint32_t)R.link_root[i], (uint32_t)R.link_root[j]);
        const double bb = kx_mul(S.bd, S.bd);
        S.pb2 = bb > 1e-300 ? bb : 1e-300;
        S.pA = S.pB = INT_MAX;
        S.phave = 0;
      }
      __syncwarp();
#pragma unroll 1
      while ((top > 0 || njobs > 0) && !pc) {
        if (njobs >= 16 || (top == 0 && njobs > 0)) {
          // ---- triangle pairs, one per lane
          uint32_t carry = 0;
          for (int bb = 0; bb < njobs; bb += 32) {
            const int jj = bb + lane;
            uint32_t c = 0;
            if (jj < njobs) c = ((S.jobA[jj] >> 28) + 1) * ((S.jobB[jj] >> 28) + 1);
            uint32_t incl = c;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
              const uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
              if (lane >= off) incl += v;
            }
            if (jj < njobs) S.jobOff[jj] = carry + incl - c;
            carry += __shfl_sync(0xffffffffu, incl, 31);
          }
          __syncwarp();
          const uint32_t total = carry;
#pragma unroll 1
          for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t p = base + lane;
            float d32 = FLT_MAX, e = 0.f;
            int tA = 0, tB = 0;
            bool certain = false;
            if (p < total) {
              int lo = 0, hi = njobs - 1;
              while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (S.jobOff[mid] <= p) lo = mid; else hi = mid - 1;
              }
              const uint32_t r = p - S.jobOff[lo];
              const uint32_t cb = (S.jobB[lo] >> 28) + 1;
              tA = (int)(S.jobA[lo] & 0x0fffffffu) + (int)(r / cb);
              tB = (int)(S.jobB[lo] & 0x0fffffffu) + (int)(r % cb);
              float3 P[3], Q[3];
#pragma unroll
              for (int v = 0; v < 3; ++v) {
                const float4 x = __ldg(W->ltri32 + 3 * (size_t)tA + v);
                P[v] = xform32(TA, make_float3(x.x, x.y, x.z));
                const float4 y = __ldg(W->ltri32 + 3 * (size_t)tB + v);
                Q[v] = xform32(TB, make_float3(y.x, y.y, y.z));
              }
              float3 lo3 = P[0], hi3 = P[0];
#pragma unroll
              for (int k = 1; k < 6; ++k) {
                const float3 v = k < 3 ? P[k] : Q[k - 3];
                lo3 = make_float3(fminf(lo3.x, v.x), fminf(lo3.y, v.y), fminf(lo3.z, v.z));
                hi3 = make_float3(fmaxf(hi3.x, v.x), fmaxf(hi3.y, v.y), fmaxf(hi3.z, v.z));
              }
              const float span = fmaxf(fmaxf(hi3.x - lo3.x, hi3.y - lo3.y), hi3.z - lo3.z);
              e = dd + 128.f * kU * span + 1e-8f;
              if (tri_axis_lb32(P, Q, span) - e > m32 * (1.f + 2e-5f) + 2.f * e) {
                d32 = FLT_MAX;  // cannot be a candidate
              } else if (!tri_separated32(P, Q, dd, 0.f)) {
                d32 = 0.f;
                certain = tri_certain_hit32(P[0], P[1], P[2], Q[0], Q[1], Q[2], dd);
              } else {
                d32 = sqrtf(tri_dist2_32(P, Q));
              }
            }
            if (__any_sync(0xffffffffu, certain)) {
              pc = true;  // distance 0: no later pair can be smaller
              if (lane == 0 && !per_pair) {
                S.b2 = 0.0;
                S.bd = 0.0;
                S.bi = i;
                S.bj = j;
              }
              __syncwarp();
              break;
            }
            m32 = fminf(m32, warp_min(d32 < FLT_MAX ? d32 + e : FLT_MAX));
            const bool cand = d32 < FLT_MAX && d32 - e <= m32 * (1.f + 2e-5f);
            const unsigned mc = __ballot_sync(0xffffffffu, cand);
            if (ncand + __popc(mc) > kSDCand) {
              sd_flush(S, W, lane, i, j, ncand, m32 * (1.f + 2e-5f) + 1e-6f);
              ncand = 0;
              if (S.phave) m32 = fminf(m32, (float)sqrt(S.pb2) * (1.f + 1e-6f));
            }
            if (cand) {
              const int rr = ncand + __popc(mc & lt);
              S.candA[rr] = (uint32_t)tA;
              S.candB[rr] = (uint32_t)tB;
              S.candD[rr] = d32 - e;
            }
            ncand += __popc(mc);
            __syncwarp();
          }
          njobs = 0;
          continue;
        }
        // ---- node pairs; near the stack capacity the batch narrows to
        // depth-first order, whose growth is bounded by the trees' depth
        const int n = min(min(top, 32), max(1, kSDStack - 64 - top));
        const bool have = lane < n;
        uint2 en = make_uint2(0, 0);
        if (have) en = S.stack[top - 1 - lane];
        __syncwarp();
        top -= n;
        int outcome = 0;
        uint2 c0 = make_uint2(0, 0), c1 = make_uint2(0, 0);
        uint32_t jA = 0, jB = 0;
        if (have) {
          const int nodeA = (int)en.x, nodeB = (int)en.y;
          const KNode na = W->lnodes[nodeA];
          const KNode nb = W->lnodes[nodeB];
          const Box32 BA = xform_box(TA, na.a, na.b);
          const Box32 BB = xform_box(TB, nb.a, nb.b);
          const float slack = 4.f * kU * (fabsf(BA.c.x) + fabsf(BA.c.y) + fabsf(BA.c.z) + fabsf(BB.c.x) +
                                          fabsf(BB.c.y) + fabsf(BB.c.z) + 1.f);
          const float lb_box = box_dist32(BA, BB.c, BB.h) - dd * 1.7321f - slack;
          const float cx = BA.c.x - BB.c.x, cy = BA.c.y - BB.c.y, cz = BA.c.z - BB.c.z;
          const float lb_sph = sqrtf(cx * cx + cy * cy + cz * cz) * (1.f - 4.f * kU) - __ldg(W->lnode_r + nodeA) -
                               __ldg(W->lnode_r + nodeB) - dd * 1.7321f - slack;
          const float lb = fmaxf(lb_box, lb_sph);
          if (lb <= m32 * (1.f + 2e-5f) + 3.f * dd + 1e-5f) {
            const int cntA = f2i(na.b.w), cntB = f2i(nb.b.w);
            const int ia = f2i(na.a.w), ib = f2i(nb.a.w);
            if (cntA > 0 && cntB > 0) {
              outcome = 2;
              jA = (uint32_t)ia | ((uint32_t)(cntA - 1) << 28);
              jB = (uint32_t)ib | ((uint32_t)(cntB - 1) << 28);
            } else {
              outcome = 1;
              const bool splitB = cntA > 0 || (cntB == 0 && (nb.b.x + nb.b.y + nb.b.z) > (na.b.x + na.b.y + na.b.z));
              if (splitB) { c0 = make_uint2((uint32_t)nodeA, (uint32_t)ib); c1 = make_uint2((uint32_t)nodeA, (uint32_t)ib + 1); }
              else { c0 = make_uint2((uint32_t)ia, (uint32_t)nodeB); c1 = make_uint2((uint32_t)ia + 1, (uint32_t)nodeB); }
            }
          }
        }
        const unsigned m1 = __ballot_sync(0xffffffffu, outcome == 1);
        const unsigned m2 = __ballot_sync(0xffffffffu, outcome == 2);
        if (top + 2 * __popc(m1) > kSDStack) {
          // cannot happen with the narrowing above (growth bounded by the
          // trees' depth); checked so that an error is reported, not hidden
          if (lane == 0) set_status(W->status, KGPU_ERR_OVERFLOW);
          top = 0;
          njobs = 0;
          ncand = 0;
          break;
        }
        if (outcome == 1) {
          const int rr = top + 2 * __popc(m1 & lt);
          S.stack[rr] = c1;
          S.stack[rr + 1] = c0;
        } else if (outcome == 2) {
          const int rr = njobs + __popc(m2 & lt);
          S.jobA[rr] = jA;
          S.jobB[rr] = jB;
        }
        top += 2 * __popc(m1);
        njobs += __popc(m2);
        __syncwarp();
      }
      if (!pc && ncand > 0) {
        sd_flush(S, W, lane, i, j, ncand, m32 * (1.f + 2e-5f) + 1e-6f);
        if (S.phave) m32 = fminf(m32, (float)sqrt(S.pb2) * (1.f + 1e-6f));
      }
      if (per_pair) {
        if (lane == 0)
          A.dpair[(size_t)b * npair + i * nl - i * (i + 1) / 2 + (j - i - 1)] =
              pc ? 0.0 : (S.phave ? kx_sqrt(S.pb2) : A.cutoff);
        __syncwarp();
        continue;
      }
      // the pair replaces the best only with a strictly smaller distance
      if (!pc && S.phave) {
        const double dp = kx_sqrt(S.pb2);
        if (dp < S.bd) {
          __syncwarp();
          if (lane == 0) {
            S.b2 = S.pb2;
            S.bd = dp;
            S.bi = i;
            S.bj = j;
            for (int c = 0; c < 3; ++c) { S.bcp[c] = S.pcp[c]; S.bcq[c] = S.pcq[c]; }
          }
        }
      }
      __syncwarp();
      if (S.b2 == 0.0) contact = true;
    }
    if (per_pair) continue;
    // ---- outputs and the gradient (FP64 transforms)
    const bool found = S.b2 < DBL_MAX;
    const double d = found ? kx_sqrt(S.b2) : A.cutoff;
    if (lane == 0) {
      A.d[b] = d;
      A.pair[2 * (size_t)b] = found ? S.bi : -1;
      A.pair[2 * (size_t)b + 1] = found ? S.bj : -1;
    }
    if (lane < 6) A.cp[6 * (size_t)b + lane] = found && d > 0.0 ? (lane < 3 ? S.bcp[lane] : S.bcq[lane - 3]) : 0.0;
    if (A.grad && lane < nl) {
      double g = 0.0;
      if (found && d > 0.0 && R.jtype[lane] != KX_JOINT_WELD) {
        double u[3];
        for (int c = 0; c < 3; ++c) u[c] = (S.bcp[c] - S.bcq[c]) / d;
        const double* Tk = S.T64[lane];
        double w[3];
        for (int r = 0; r < 3; ++r) w[r] = Tk[3 * r] * R.axis64[lane][0] + Tk[3 * r + 1] * R.axis64[lane][1] +
                                          Tk[3 * r + 2] * R.axis64[lane][2];
        for (int side = 0; side < 2; ++side) {
          const int link = side == 0 ? S.bi : S.bj;
          bool anc = false;
          for (int a = link; a >= 0; a = R.parents[a])
            if (a == lane) { anc = true; break; }
          if (!anc) continue;
          const double* x = side == 0 ? S.bcp : S.bcq;
          double v[3];
          if (R.jtype[lane] == KX_JOINT_REVOLUTE) {
            const double rx = x[0] - Tk[9], ry = x[1] - Tk[10], rz = x[2] - Tk[11];
            v[0] = w[1] * rz - w[2] * ry;
            v[1] = w[2] * rx - w[0] * rz;
            v[2] = w[0] * ry - w[1] * rx;
          } else {
            v[0] = w[0]; v[1] = w[1]; v[2] = w[2];
          }
          const double t = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
          g += side == 0 ? t : -t;
        }
      }
      A.grad[(size_t)b * nl + lane] = (float)g;
    }
    __syncwarp();
  }
}

}  // namespace

cudaError_t dist_init()
{
  cudaError_t e =
      cudaFuncSetAttribute(k_dist<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(DistSmem) * kDW));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_dist<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(DistSmem) * kDW));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_dist<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(DistSmem) * kDW));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_self_dist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(SelfDistSmem) * kDW));
}

cudaError_t launch_distance(const KWorldDev* Wd, const Scratch& S, int robot, const float* q, int B, double cutoff,
                            double* d, int* pair, double* cp, float* grad, int num_sms, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(S.counters + 8, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  DistArgs A = {};
  A.mode = 0;
  A.robot = robot;
  A.q = q;
  A.B = B;
  A.cutoff = cutoff;
  A.d = d;
  A.pair = pair;
  A.cp = cp;
  A.grad = grad;
  A.head = S.counters + 8;
  A.scratch = S.spill;
  A.scratch_per_warp = (int)S.spill_per_warp;
  k_dist<0><<<num_sms * 2, kDW * 32, sizeof(DistSmem) * kDW, s>>>(Wd, A);
  return cudaGetLastError();
}

cudaError_t launch_softmin(const KWorldDev* Wd, const Scratch& S, int robot, const float* q, int T, int Wn,
                           double tau, double* L, float* dLdq, int nl, double* work, int num_sms, cudaStream_t s)
{
  if (T <= 0) return cudaSuccess;
  const int B = T * Wn;
  double* dwp = work;            // [B]
  double* mt = work + B;         // [T]
  double* wsum = work + B + T;   // [B]
  cudaError_t e = cudaMemsetAsync(S.counters + 8, 0, 2 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  DistArgs A = {};
  A.robot = robot;
  A.q = q;
  A.B = B;
  A.scratch = S.spill;
  A.scratch_per_warp = (int)S.spill_per_warp;
  // pass 1: waypoint minima (no cutoff)
  A.mode = 1;
  A.cutoff = 1e3;
  A.d = dwp;
  A.head = S.counters + 8;
  k_dist<1><<<num_sms * 2, kDW * 32, sizeof(DistSmem) * kDW, s>>>(Wd, A);
  k_traj_min<<<(T + 127) / 128, 128, 0, s>>>(dwp, T, Wn, mt);
  // pass 2: every pair below m + K tau, unnormalised gradients
  A.mode = 2;
  A.m_traj = mt;
  A.wsum = wsum;
  A.W = Wn;
  A.tau = tau;
  A.grad = dLdq;
  A.head = S.counters + 9;
  k_dist<2><<<num_sms * 2, kDW * 32, sizeof(DistSmem) * kDW, s>>>(Wd, A);
  k_softmin_final<<<(T + 127) / 128, 128, 0, s>>>(wsum, mt, T, Wn, nl, tau, L, dLdq);
  return cudaGetLastError();
}

}  // namespace kgpu

namespace kgpu {

cudaError_t launch_self_distance(const KWorldDev* Wd, int robot, const float* q, int B, double cutoff, double* d,
                                 int* pair, double* cp, float* grad, double* dpair, int all_pairs, int num_sms,
                                 cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  const size_t smem = sizeof(SelfDistSmem) * kDW;  // attribute set by dist_init()
  SelfDistArgs A;
  A.robot = robot;
  A.q = q;
  A.B = B;
  A.cutoff = cutoff;
  A.d = d;
  A.pair = pair;
  A.cp = cp;
  A.grad = grad;
  A.dpair = dpair;
  A.all_pairs = dpair != nullptr && all_pairs != 0;
  const int blocks = min((B + kDW - 1) / kDW, 4 * num_sms);
  k_self_dist<<<blocks, kDW * 32, smem, s>>>(Wd, A);
  return cudaGetLastError();
}

}  // namespace kgpu
