// kgpu_collide.cu — batched collision engine: configuration checks, feasibility
// and planner edge checks in one persistent launch.
//
// Replaces, per configuration, the reference's serial chain
//   SingleRobotCSpace::IsFeasible -> CheckJointLimits -> UpdateConfig (FK)
//   -> WorldPlannerSettings::CheckCollision(robot, others) (env)
//   -> WorldPlannerSettings::CheckCollision(robot) (self)
// (Cpp/Planning/RobotCSpace.cpp:610-630,786-823,
//  Cpp/Planning/PlannerSettings.cpp:241-331) and, per edge, the epsilon edge
// checker loop over interpolated configurations
// (Cpp/Planning/RobotCSpace.cpp:835-840, Cpp/Modeling/Interpolate.cpp:10-14).
//
// Execution model
//   * One warp processes one work item (a configuration or an edge step) at
//     a time and pulls items from a device work queue (persistent grid sized
//     to the SM count).  An edge item is a chunk of consecutive steps
//     (`chunk`, default 4) checked in order; chunks are ordered round-major
//     across edges, so every edge's early steps run first and a step beyond
//     an edge's first collision is skipped.
//   * FK: lane i owns link i (warp_fk32); transforms go to shared memory.
//   * All queries of the item — (link, env group) and (link, link) pairs —
//     share one warp stack of BVH node pairs tagged with their query, so the
//     32 lanes stay busy across queries.  Lanes pop 32 pairs, test them, and
//     push children with ballot/popc compaction; leaf/leaf pairs become
//     triangle-pair jobs that are expanded one triangle pair per lane.
//   * A triangle pair the FP32 filter cannot separate is either certified
//     as a contact in FP32 (tri_certain_hit32) or listed for the FP64 test
//     (band_retest on FP64 transforms), run by k_band after the main pass or
//     inline in the single-pass variant.
//   * After the queue drains, idle warps of a block take over halves of their
//     siblings' deep traversal stacks (edge batches).
//   * The shared-memory stack spills its lower half to a per-warp region of
//     global scratch when full; exhausting that region sets
//     KGPU_ERR_OVERFLOW instead of dropping work.
//   * Code size matters more than inlining here: the traversal and the
//     triangle jobs are out-of-line functions with rolled loops, so the hot
//     loop stays resident in the instruction cache.
#include <climits>

#include "kgpu_device.cuh"

namespace kgpu {

namespace {

constexpr int kStackCap = 384;
constexpr int kJobCap = 96;
constexpr int kGrab = 2;  // items taken from the queue per atomic
constexpr int kWarps = 8; // warps per block
constexpr int kMaxChunk = 64;  // most consecutive edge steps per work item
constexpr int kDefaultChunk = 16;
constexpr int kTailItemsPerWarp = 2;  // single-step rounds once fewer items than this per warp remain

enum Mode { MODE_CONFIGS = 0, MODE_FEASIBLE = 1, MODE_EDGES = 2 };

// per-warp shared memory (~6.4 KB, so that up to 32 warps fit on an SM)
struct __align__(16) WarpSmem {
  float T[kMaxLinks][12];     // first: every row starts on a 16-byte boundary
  uint2 stack[kStackCap];
  uint32_t jobA[kJobCap];
  uint32_t jobB[kJobCap];
  uint32_t jobM[kJobCap];
  uint32_t jobOff[kJobCap + 1];
  float delta[kMaxLinks];     // per-link bound on |FP32 - exact| world coordinates
  float gerr[kMaxLinks];      // per-link max |R^T R - I| of the FP32 rotation (+ rounding)
  float tol64[64];            // box-test tolerance parts: rows 0-31 per link row, 32-63 per group
  double q64[kMaxLinks];      // canonical FP64 joint values (filled with T64)
  const float* item_qa;       // the item's joint values: configuration, or edge
  const float* item_qb;       //   endpoints qa/qb (item_qb null for configurations)
  int item_k, item_n;         // edge step k of n
  int item_id;                // configuration index b, or edge index e
  int item_cfg[4];            // configuration index of each step of a configuration group
  int item_rid;               // robot of the item
  int don_top;                // stack entries handed over by a sibling warp
  unsigned don_live;          // steps of the handed-over group still to decide
};
static_assert(sizeof(float) * 12 % 16 == 0, "link rows of WarpSmem::T stay 16-byte aligned");

// Work sharing inside a block once the queue is drained (edge batches, whose
// long items would otherwise end the launch on one warp; a contact found by
// any part settles the step through first_hit): a warp with nothing
// left sets flag 0 (waiting) and counts itself in `idle`; a sibling whose
// traversal stack is deep claims it (flag 0 -> 3), copies the item context and
// the bottom half of its stack into the waiting warp's shared memory and
// releases it (flag 1).  A waiting warp leaves (flag 0 -> 4, so it can no
// longer be claimed) once every warp of the block waits.  Flag 2: busy.
struct BlockShare {
  int idle;
  int flag[kWarps];
  int no_release;  // failure-path test switch (KWorldDev::share_no_release)
};
constexpr size_t kBlockSmem = sizeof(WarpSmem) * kWarps + sizeof(BlockShare);
// Optional (world option stage_nodes, 2 blocks per SM): the first nodes of
// the environment node array, which is laid out breadth first from the group
// roots, are the top levels every traversal starts with; a staged block
// copies up to kStageNodes of them into shared memory and reads them there.
constexpr int kStageNodes = 1024;
constexpr size_t kStageOffset = (kBlockSmem + 15) / 16 * 16;
// MINB blocks (plus the 1 KB the hardware reserves per block) fit in the
// 228 KB of shared memory of an SM
static_assert(4 * (kBlockSmem + 1024) <= 228 * 1024, "4 blocks per SM");
static_assert(2 * (kStageOffset + 32 * kStageNodes + 1024) <= 228 * 1024, "2 staged blocks per SM");
constexpr int kDonateMin = 32;     // stack entries a warp needs before it shares
constexpr int kShareSpins = 1 << 20;  // bound on a waiting warp's polls (~0.3 s)

// canonical FP64 joint values of the current item (lane < nl), as the oracle
// forms them: float input widened, or the FP64 edge interpolation
__device__ __forceinline__ double item_q64(const WarpSmem& S, int lane)
{
  if (S.item_qb == nullptr) return (double)S.item_qa[lane];
  return kx_interp((double)S.item_qa[lane], (double)S.item_qb[lane], S.item_k, S.item_n);
}

__device__ __noinline__ void ensure_fk64(WarpSmem& S, const KRobotDev& R, double (*T64)[12], int lane, int& fk64)
{
  if (fk64) return;
  if (lane < R.nlinks) S.q64[lane] = item_q64(S, lane);
  __syncwarp();
  warp_fk64(R, S.q64, T64, lane);
  fk64 = 1;
}

// per-warp global scratch: FP64 link transforms (filled on the first band
// pair of a configuration) followed by the stack spill area
constexpr int kT64Doubles = kMaxLinks * 12;

struct EngineArgs {
  int mode;
  int robot;             // fixed robot, or -1 with robot_ids
  const int* robot_ids;
  const float* q;
  int q_stride;
  int B;
  uint8_t* env_hit;
  uint8_t* self_hit;
  uint8_t* feasible;
  // edges
  const float* qa;
  const float* qb;
  const int* nsteps;
  int E;
  int* first_hit;
  const int* round_off;
  const int* perm;
  const int* meta;       // [0] max n, [1] total items
  // queue / scratch
  unsigned int* head;
  uint2* spill;
  int spill_per_warp;
  // work split (autotuned): items per queue grab, triangle-job flush size,
  // consecutive edge steps per work item
  int grab;
  int job_flush;
  int chunk;
  // deferred FP64 re-tests: triangle pairs the FP32 tests left undecided,
  // {item (b or e), k | la << 16 | tgt << 21, tA, tB}
  uint4* pend;
  unsigned int* pend_count;
  int pend_cap;
  int inline64;          // 1: one pass with the FP64 test inline (no list)
  int stage_nodes;       // environment nodes a staged block copies to shared memory
};

struct Cnt {
  unsigned long long node_pairs = 0, tri_pairs = 0, band = 0, spills = 0, cert = 0, hit64 = 0;
};

// a link row of S.T (16-byte aligned) into registers with three 16-byte loads
__device__ __forceinline__ void load_row(const float* T, float* o)
{
  const float4* p = reinterpret_cast<const float4*>(T);
  const float4 a = p[0], b = p[1], c = p[2];
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
  o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  o[8] = c.x; o[9] = c.y; o[10] = c.z; o[11] = c.w;
}

// traversal result flag: the spill area ran out (step bits are 0..3)
constexpr unsigned kTrOverflow = 1u << 31;

__device__ __forceinline__ uint2 make_entry(int nodeA, int la, int tgt, int nodeB)
{
  return make_uint2((uint32_t)nodeB, (uint32_t)nodeA | ((uint32_t)la << 20) | ((uint32_t)tgt << 25));
}

// Tests the triangle-pair jobs of the warp, one triangle pair per lane.
// Triangle-pair jobs of a step group: bit g of `live` marks step (or
// configuration) g still undecided; a job's step is its link row >> lgL.
// Per pair: FP32 separating-axis filter (separated beyond the band: done),
// FP32 intersection certificate (crossing beyond the band: contact),
// otherwise the pair is undecided in FP32.  The main pass (FP64 = false)
// appends such a pair to A.pend and goes on (k_band decides it afterwards);
// the fallback pass (FP64 = true, groups of one) decides it here with the
// FP64 test on transforms computed once per configuration (fk64 tracks
// whether T64 is valid).  Keeping the FP64 code out of the main pass's
// kernel keeps that kernel's hot loop in the instruction cache.  A contact
// at step g clears bit g of `live` (edge steps: bits g and above, later
// steps need no decision).  Returns the steps found in contact.
template <bool FP64, bool EDGES>
__device__ __noinline__ unsigned run_jobs(WarpSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                          int njobs, int lane, double (*T64)[12], int& fk64, const EngineArgs& A,
                                          Cnt& cnt, unsigned live, int lgL)
{
  const int lmask = (1 << lgL) - 1;
  constexpr bool seq = EDGES;
  unsigned hits = 0;
  // exclusive prefix over job sizes
  uint32_t carry = 0;
#pragma unroll 1
  for (int b = 0; b < njobs; b += 32) {
    int j = b + lane;
    uint32_t c = 0;
    if (j < njobs) {
      uint32_t ca = (S.jobA[j] >> 28) + 1;
      uint32_t cb = ((S.jobM[j] >> 16) & 3u) + 1;
      c = ca * cb;
    }
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (j < njobs) S.jobOff[j] = carry + incl - c;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) S.jobOff[njobs] = carry;
  __syncwarp();
  const uint32_t total = carry;
  const float4* __restrict__ ltri = W->ltri32;
  const float4* __restrict__ etri = W->etri32;
#pragma unroll 1
  for (uint32_t base = 0; base < total; base += 32) {
    uint32_t p = base + lane;
    bool band = false, certain = false, mine = false;
    int la = 0, tgt = 0, tA = 0, tB = 0, step = 0;
    if (p < total) {
      // job holding p: largest j with jobOff[j] <= p
      int lo = 0, hi = njobs - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (S.jobOff[mid] <= p) lo = mid; else hi = mid - 1;
      }
      const int j = lo;
      const uint32_t jm = S.jobM[j];
      la = jm & 0xff;
      tgt = (jm >> 8) & 0xff;
      step = la >> lgL;
      mine = (live >> step) & 1u;
      if (mine) {
        const uint32_t r = p - S.jobOff[j];
        const uint32_t cb = ((jm >> 16) & 3u) + 1;
        tA = (int)(S.jobA[j] & 0x0fffffffu) + (int)(r / cb);
        tB = (int)S.jobB[j] + (int)(r % cb);
        float3 P[3], Q[3];
        const bool self = tgt < 32;
        float TA[12], TB[12];
        load_row(S.T[la], TA);
        load_row(S.T[self ? tgt : la], TB);
        const float4* qsrc = self ? ltri : etri;
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          float4 x = __ldg(ltri + 3 * (size_t)tA + v);
          P[v] = xform32(TA, make_float3(x.x, x.y, x.z));
          float4 y = __ldg(qsrc + 3 * (size_t)tB + v);
          Q[v] = self ? xform32(TB, make_float3(y.x, y.y, y.z)) : make_float3(y.x, y.y, y.z);
        }
        const float margin =
            R.link_margin[la & lmask] + (self ? R.link_margin[tgt & lmask] : W->group_margin[tgt - 32]);
        const float dA = S.delta[la] + W->eps_extra;
        const float dB = (self ? S.delta[tgt] : W->eps_env) + W->eps_extra;
        band = !tri_separated32(P, Q, dA + dB, margin);
        if (band && margin == 0.f) certain = tri_certain_hit32(P[0], P[1], P[2], Q[0], Q[1], Q[2], fmaxf(dA, dB));
        cnt.tri_pairs++;
      }
    }
    if (__any_sync(0xffffffffu, certain)) {
      cnt.cert++;
      const unsigned hm = __reduce_or_sync(0xffffffffu, certain ? 1u << step : 0u);
      hits |= hm;
      live &= seq ? (1u << (__ffs(hm) - 1)) - 1u : ~hm;
      if (live == 0) return hits | (live << 16);
    }
    const bool need64 = band && !certain && ((live >> step) & 1u);
    if (__any_sync(0xffffffffu, need64)) {
      if (!FP64) {
        const unsigned m = __ballot_sync(0xffffffffu, need64);
        unsigned at = 0;
        if (lane == 0) at = atomicAdd(A.pend_count, (unsigned)__popc(m));
        at = __shfl_sync(0xffffffffu, at, 0) + __popc(m & lanemask_lt());
        if (need64 && at < (unsigned)A.pend_cap) {
          // the record names the edge step (or the configuration) and link
          // indices, not link rows
          const unsigned tl = tgt < 32 ? (unsigned)(tgt & lmask) : (unsigned)tgt;
          const unsigned item = seq ? (unsigned)S.item_id : (unsigned)S.item_cfg[step];
          const unsigned k = seq ? (unsigned)(S.item_k + step) : 0u;
          A.pend[at] = make_uint4(item, k | ((unsigned)(la & lmask) << 16) | (tl << 21), (unsigned)tA, (unsigned)tB);
        }
      } else {
        ensure_fk64(S, R, T64, lane, fk64);
        int hit = 0;
        if (need64) {
          cnt.band++;
          hit = band_retest(W, R, T64, la, tA, tgt, tB);
        }
        if (__any_sync(0xffffffffu, hit)) {
          cnt.hit64++;
          const unsigned hm = __reduce_or_sync(0xffffffffu, hit ? 1u << step : 0u);
          hits |= hm;
          live &= seq ? (1u << (__ffs(hm) - 1)) - 1u : ~hm;
          if (live == 0) return hits | (live << 16);
        }
      }
    }
  }
  return hits | (live << 16);
}

// Separation of two link boxes along their six face axes (the columns of the
// two FP32 rotations), for self pairs: the world boxes of two rotated link
// nodes are loose, and nearly parallel links would otherwise be traversed
// down to most of their leaves.  Both boxes are the exact images of their
// local boxes under the FP32 transforms; a column a has |a| <= 1 + g and
// |a_i . a_k| <= g (i != k), so a box's projection onto its own axis i is at
// most h_i + g (hx + hy + hz) and a gap along a overstates the Euclidean one
// by at most the factor 1 + g.  16 u covers the rounding of the centres,
// the products and the sums.  Out of line: only link-link pairs take it, and
// inlined it lengthens the hot loop of every pair.
__device__ __noinline__ bool obb_separated(const float* TA, const float* TB, float4 hA, float4 hB, float3 cA,
                                              float3 cB, float tol, float g)
{
  const float dx = cB.x - cA.x, dy = cB.y - cA.y, dz = cB.z - cA.z;
  const float sa = hA.x + hA.y + hA.z, sb = hB.x + hB.y + hB.z;
  const float slack = tol * (1.f + g) + 2.f * g * (sa + sb) +
                      16.f * kU * (fabsf(cA.x) + fabsf(cA.y) + fabsf(cA.z) + fabsf(cB.x) + fabsf(cB.y) + fabsf(cB.z) +
                                   sa + sb + 1e-3f);
  float C[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = fabsf(TA[i] * TB[j] + TA[3 + i] * TB[3 + j] + TA[6 + i] * TB[6 + j]);
  const float ha[3] = {hA.x, hA.y, hA.z}, hb[3] = {hB.x, hB.y, hB.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float pa = fabsf(TA[i] * dx + TA[3 + i] * dy + TA[6 + i] * dz);
    if (pa > ha[i] + hb[0] * C[i][0] + hb[1] * C[i][1] + hb[2] * C[i][2] + slack) return true;
    const float pb = fabsf(TB[i] * dx + TB[3 + i] * dy + TB[6 + i] * dz);
    if (pb > hb[i] + ha[0] * C[0][i] + ha[1] * C[1][i] + ha[2] * C[2][i] + slack) return true;
  }
  return false;
}

// Node-pair test for one stack entry; returns 0 (culled), 1 (children in c0,
// c1) or 2 (leaf job in jA, jB, jM).
// box-test tolerance of a (link row la, target tgt) pair: error bounds of
// both sides, the optional extra inflation and the summed margins, from the
// per-row and per-group parts in S.tol64; the factor covers the rounding of
// the sums (all terms are non-negative)
__device__ __forceinline__ float pair_tol(const WarpSmem& S, int la, int tgt)
{
  return (S.tol64[la] + S.tol64[tgt]) * (1.f + 16.f * kU);
}

template <bool STAGE>
__device__ __forceinline__ int test_entry(const WarpSmem& S, const KWorldDev* __restrict__ W,
                                          const KRobotDev& R, uint2 e, uint2& c0, uint2& c1,
                                          uint32_t& jA, uint32_t& jB, uint32_t& jM, const KNode* stage,
                                          int nstage)
{
  const int nodeA = e.y & 0xfffff;
  const int la = (e.y >> 20) & 31;
  const int tgt = (e.y >> 25) & 63;
  const int nodeB = (int)e.x;
  const bool self = tgt < 32;
  const KNode na = W->lnodes[nodeA];
  const KNode nb = self ? W->lnodes[nodeB] : (STAGE && nodeB < nstage ? stage[nodeB] : W->enodes[nodeB]);
  float TA[12];
  load_row(S.T[la], TA);
  const Box32 A = xform_box(TA, na.a, na.b);
  Box32 Bx;
  if (self) {
    float TB[12];
    load_row(S.T[tgt], TB);
    Bx = xform_box(TB, nb.a, nb.b);
  } else {
    Bx.c = make_float3(nb.a.x, nb.a.y, nb.a.z);
    Bx.h = make_float3(nb.b.x, nb.b.y, nb.b.z);
  }
  const float tol = pair_tol(S, la, tgt);
  if (!boxes_overlap(A, Bx, tol)) return 0;
  if (self && obb_separated(S.T[la], S.T[tgt], na.b, nb.b, A.c, Bx.c, tol, fmaxf(S.gerr[la], S.gerr[tgt])))
    return 0;
  const int cntA = f2i(na.b.w), cntB = f2i(nb.b.w);
  const int ia = f2i(na.a.w), ib = f2i(nb.a.w);
  if (cntA > 0 && cntB > 0) {
    jA = (uint32_t)ia | ((uint32_t)(cntA - 1) << 28);
    jB = (uint32_t)ib;
    jM = (uint32_t)la | ((uint32_t)tgt << 8) | ((uint32_t)(cntB - 1) << 16);
    return 2;
  }
  const bool splitB = cntA > 0 || (cntB == 0 && (nb.b.x + nb.b.y + nb.b.z) > (na.b.x + na.b.y + na.b.z));
  if (splitB) {
    c0 = make_entry(nodeA, la, tgt, ib);
    c1 = make_entry(nodeA, la, tgt, ib + 1);
  } else {
    c0 = make_entry(ia, la, tgt, nodeB);
    c1 = make_entry(ia + 1, la, tgt, nodeB);
  }
  return 1;
}

// Gives the bottom half of this warp's stack (and the item context) to a
// waiting sibling, if one can be claimed; returns the entries given.
__device__ __noinline__ int share_stack(WarpSmem* all, int me, BlockShare& B, int lane, int top, unsigned live)
{
  int t = -1;
  if (lane == 0) {
    for (int w = 0; w < kWarps && t < 0; ++w)
      if (w != me && *((volatile int*)&B.flag[w]) == 0 && atomicCAS(&B.flag[w], 0, 3) == 0) t = w;
  }
  t = __shfl_sync(0xffffffffu, t, 0);
  if (t < 0 || B.no_release) return 0;  // (test switch: claimed, never handed over, entries kept)
  WarpSmem& S = all[me];
  WarpSmem& D = all[t];
  const int h = top / 2;
  for (int k = lane; k < h; k += 32) D.stack[k] = S.stack[k];
  for (int i = lane; i < kMaxLinks * 12; i += 32) D.T[i / 12][i % 12] = S.T[i / 12][i % 12];
  D.delta[lane] = S.delta[lane];
  D.gerr[lane] = S.gerr[lane];
  if (lane == 0) {
    D.item_qa = S.item_qa;
    D.item_qb = S.item_qb;
    D.item_k = S.item_k;
    D.item_n = S.item_n;
    D.item_id = S.item_id;
    D.item_rid = S.item_rid;
    D.don_top = h;
    D.don_live = live;
  }
  __syncwarp();
  {
    // the kept entries move down in two phases (all loads, then all stores):
    // the ranges overlap, and lanes of a warp are not guaranteed to run the
    // iterations of an in-place copy in lockstep
    uint2 keep[kStackCap / 64 + 1];
#pragma unroll
    for (int i = 0; i < kStackCap / 64 + 1; ++i) {
      const int k = lane + 32 * i;
      if (k < top - h) keep[i] = S.stack[h + k];
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < kStackCap / 64 + 1; ++i) {
      const int k = lane + 32 * i;
      if (k < top - h) S.stack[k] = keep[i];
    }
  }
  __syncwarp();
  if (lane == 0) {
    __threadfence_block();
    atomicExch(&B.flag[t], 1);
  }
  return h;
}

// Moves the lower half of a full stack to the spill area (false: the area
// is exhausted), and back (restore_half); out of line, so that the
// traversal loop stays small: 5% faster edge plans than inline.
__device__ __noinline__ bool spill_half(WarpSmem& S, uint2* spill, int spill_cap, int spill_top, int top, int lane)
{
  const int H = kStackCap / 2;
  if (spill_top + H > spill_cap) return false;
  for (int k = lane; k < H; k += 32) spill[spill_top + k] = S.stack[k];
  __syncwarp();
  for (int k = lane; k < top - H; k += 32) S.stack[k] = S.stack[H + k];  // disjoint: top <= 2 H
  __syncwarp();
  return true;
}

__device__ __noinline__ void restore_half(WarpSmem& S, const uint2* spill, int spill_top, int n, int lane)
{
  for (int k = lane; k < n; k += 32) S.stack[k] = spill[spill_top - n + k];
  __syncwarp();
}

// Traverses queries [qbase, qbase+qcount) of robot R for the steps (or
// configurations) g of a group whose bit is set in `live` (link row
// g * 2^lgL + link of S.T holds link `link` at step g), or (preset > 0) the
// preset entries S.stack[0, preset) handed over by a sibling.  All steps
// share one stack; an entry's step is its link row >> lgL, and the entries
// of a step found in contact are dropped (of an edge step: also those of the
// later steps).  Returns the steps found in contact (bits 0..3: a group has
// at most 32 / 8 steps), plus kTrOverflow when the spill area ran out.
// Warp-uniform control flow.
template <bool FP64, bool EDGES, bool STAGE = false>
__device__ __noinline__ unsigned traverse(WarpSmem& S, const KWorldDev* __restrict__ W, const KRobotDev& R,
                                          int qbase, int qcount, int lane, uint2* spill, int spill_cap,
                                          double (*T64)[12], int& fk64, const EngineArgs& A, int job_flush,
                                          Cnt& cnt, WarpSmem* all, int me, BlockShare& B, int preset, unsigned live,
                                          int lgL, int nstage = 0)
{
  const unsigned lt = lanemask_lt();
  const int lmask = (1 << lgL) - 1;
  const KNode* stage =
      STAGE ? reinterpret_cast<const KNode*>(reinterpret_cast<const unsigned char*>(all) + kStageOffset) : nullptr;
  int top = preset, njobs = 0, spill_top = 0;
  unsigned hits = 0, np = 0;  // np: node pairs tested (added to cnt on return)
  S.tol64[lane] = S.delta[lane] + W->eps_extra + R.link_margin[lane & lmask];
  S.tol64[32 + lane] = W->eps_env + W->eps_extra + W->group_margin[lane];
  __syncwarp();
  const int nroot = preset > 0 || live == 0 ? 0 : qcount * (32 - __clz(live));

  // root pairs of every query and step, tested in parallel; pushed so that
  // step 0 ends on top (batches from the last, lane 0 highest), and children
  // below keep that order: the earliest steps are traversed first, later
  // steps fill the lanes they leave idle, and a contact at step g drops the
  // work of the steps after it
#pragma unroll 1
  for (int qb = (nroot - 1) & ~31; qb >= 0; qb -= 32) {
    if (top > kStackCap - 32) {
      if (!spill_half(S, spill, spill_cap, spill_top, top, lane)) {
        cnt.node_pairs += np;
        return hits | kTrOverflow;
      }
      spill_top += kStackCap / 2;
      top -= kStackCap / 2;
      cnt.spills++;
    }
    const int qi = qb + lane;
    bool push = false;
    uint2 ent = make_uint2(0, 0);
    if (qi < nroot) {
      const int g = qi / qcount;
      if ((live >> g) & 1u) {
        const uint32_t qw = __ldg(W->queries + qbase + (qi - g * qcount));
        const int a = qw & 0xff, tgt = (qw >> 8) & 0xff;
        const int ra = R.link_root[a];
        const int rb = tgt < 32 ? R.link_root[tgt] : W->group_root[tgt - 32];
        if (ra >= 0 && rb >= 0) {
          const int row = (g << lgL) | a;
          const int trow = tgt < 32 ? ((g << lgL) | tgt) : tgt;
          ent = make_entry(ra, row, trow, rb);
          // box cull of the root pair; survivors are pushed and expanded below
          const KNode na = W->lnodes[ra];
          const KNode nb = (tgt < 32 ? W->lnodes : W->enodes)[rb];
          const Box32 A = xform_box(S.T[row], na.a, na.b);
          Box32 Bx;
          if (tgt < 32) Bx = xform_box(S.T[trow], nb.a, nb.b);
          else { Bx.c = make_float3(nb.a.x, nb.a.y, nb.a.z); Bx.h = make_float3(nb.b.x, nb.b.y, nb.b.z); }
          push = boxes_overlap(A, Bx, pair_tol(S, row, trow));
          np++;
        }
      }
    }
    const unsigned mp = __ballot_sync(0xffffffffu, push);
    if (push) S.stack[top + __popc(mp) - 1 - __popc(mp & lt)] = ent;
    top += __popc(mp);
    __syncwarp();
  }

#pragma unroll 1
  for (;;) {
    if (top == 0) {
      if (spill_top > 0) {
        const int n = min(kStackCap / 2, spill_top);
        restore_half(S, spill, spill_top, n, lane);
        spill_top -= n;
        top = n;
      } else if (njobs == 0) {
        cnt.node_pairs += np;
        return hits;
      }
    }
    if (njobs >= job_flush || (top == 0 && njobs > 0)) {
      const unsigned r = run_jobs<FP64, EDGES>(S, W, R, njobs, lane, T64, fk64, A, cnt, live, lgL);
      hits |= r & 0xffffu;
      live = r >> 16;
      __syncwarp();
      njobs = 0;
      if (live == 0) {
        cnt.node_pairs += np;
        return hits;
      }
      continue;
    }
    if (top > kStackCap - 32) {
      if (!spill_half(S, spill, spill_cap, spill_top, top, lane)) {
        cnt.node_pairs += np;
        return hits | kTrOverflow;
      }
      spill_top += kStackCap / 2;
      top -= kStackCap / 2;
      cnt.spills++;
    }
    if (EDGES && top >= kDonateMin) {
      int idle = 0;
      if (lane == 0) idle = *((volatile int*)&B.idle);
      if (__shfl_sync(0xffffffffu, idle, 0) > 0) top -= share_stack(all, me, B, lane, top, live);
    }
    const int n = min(top, 32);
    bool have = lane < n;
    uint2 e = make_uint2(0, 0);
    if (have) {
      e = S.stack[top - 1 - lane];
      have = (live >> (((e.y >> 20) & 31u) >> lgL)) & 1u;  // entries of decided steps are dropped
    }
    __syncwarp();
    top -= n;
    int outcome = 0;  // 1: two children, 2: leaf job
    uint2 c0 = make_uint2(0, 0), c1 = make_uint2(0, 0);
    uint32_t jA = 0, jB = 0, jM = 0;
    if (have) outcome = test_entry<STAGE>(S, W, R, e, c0, c1, jA, jB, jM, stage, nstage);
    np += have ? 1u : 0u;
    const unsigned m1 = __ballot_sync(0xffffffffu, outcome == 1);
    const unsigned m2 = __ballot_sync(0xffffffffu, outcome == 2);
    if (outcome == 1) {
      const int r = top + 2 * (__popc(m1) - 1 - __popc(m1 & lt));
      S.stack[r] = c1;
      S.stack[r + 1] = c0;
    } else if (outcome == 2) {
      const int r = njobs + __popc(m2 & lt);
      S.jobA[r] = jA;
      S.jobB[r] = jB;
      S.jobM[r] = jM;
    }
    top += 2 * __popc(m1);
    njobs += __popc(m2);
    __syncwarp();
  }
}

// MINB: resident blocks of kWarps warps per SM the register allocation is
// sized for (2 -> 128 registers/thread, 3 -> 80, 4 -> 64).
// FP64 = false: the main pass over all items; undecided triangle pairs go to
// A.pend for k_band.  FP64 = true: every item with the FP64 triangle test
// inline, either as the only pass (A.inline64, for batches where undecided
// pairs are common and an inline FP64 contact ends an item early) or as the
// fallback after a main pass whose list overflowed (otherwise it returns at
// once); its verdicts overwrite the main pass's.
template <int MINB, bool FP64, bool EDGES, bool STAGE = false>
__global__ void __launch_bounds__(kWarps * 32, MINB)
    k_engine(const KWorldDev* __restrict__ W, const EngineArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem* all = reinterpret_cast<WarpSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem& S = all[warp];
  const int gwarp = blockIdx.x * kWarps + warp;
  uint2* wscratch = A.spill + (size_t)gwarp * A.spill_per_warp;
  double(*T64)[12] = reinterpret_cast<double(*)[12]>(wscratch);
  uint2* spill = wscratch + kT64Doubles;
  const int spill_cap = A.spill_per_warp - kT64Doubles;
  Cnt cnt;
  unsigned long long items = 0;
  if (FP64 && !A.inline64 && *((volatile unsigned int*)A.pend_count) <= (unsigned)A.pend_cap)
    return;  // k_band decided the list
  BlockShare& B = *reinterpret_cast<BlockShare*>(smem_raw + sizeof(WarpSmem) * kWarps);
  if (threadIdx.x == 0) {
    B.idle = 0;
    for (int w = 0; w < kWarps; ++w) B.flag[w] = 2;
    B.no_release = W->share_no_release;
  }
  int nstage = 0;
  if (STAGE) {
    // the environment tree's top levels into shared memory (coalesced
    // 16-byte loads, 2 per node)
    nstage = min(min(A.stage_nodes, kStageNodes), W->env_nodes);
    const float4* __restrict__ src = reinterpret_cast<const float4*>(W->enodes);
    float4* dst = reinterpret_cast<float4*>(smem_raw + kStageOffset);
    for (int i = threadIdx.x; i < 2 * nstage; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  // configurations of one robot go in groups of G = 32 / L (L = its link
  // count rounded up to 8, 16 or 32) per work item in the main pass; mixed
  // robots sorted by robot (A.perm set) in groups of their robot's G, mixed
  // robots otherwise and the FP64 pass one configuration per item
  const int lgC = EDGES || FP64 || A.robot < 0
                      ? 5
                      : (W->robots[A.robot].nlinks <= 8 ? 3 : (W->robots[A.robot].nlinks <= 16 ? 4 : 5));
  const int Gcfg = 32 >> lgC;
  // (k_cfg_offsets counts the items of the sorted order)
  const int total = EDGES ? A.meta[1] : (A.perm ? A.meta[0] : (A.B + Gcfg - 1) / Gcfg);
  const int maxn = EDGES ? A.meta[0] : 0;  // last round index
  const int grab = A.grab >= 1 && A.grab <= 16 ? A.grab : kGrab;
  const int job_flush = A.job_flush >= 8 && A.job_flush <= kJobCap - 32 ? A.job_flush : kJobCap - 32;
  const int chunk = A.chunk >= 1 && A.chunk <= kMaxChunk ? A.chunk : 1;
  const int nchunked = EDGES ? A.meta[2] : 0;
  const int split = EDGES ? A.meta[3] : 0;

#pragma unroll 1
  for (;;) {
    unsigned int base = 0;
    if (lane == 0) base = atomicAdd(A.head, (unsigned)grab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned)total) break;
#pragma unroll 1
    for (unsigned it = base; it < base + grab && it < (unsigned)total; ++it) {
      // ---- decode the item
      int rid = A.robot;
      int b = 0, e = 0, k0 = 0, k1 = 0, n = 0;
      if (EDGES) {
        // rounds r < J: steps [r*chunk, r*chunk + chunk) of every edge that
        // reaches r*chunk, checked in order; rounds r >= J: the single step
        // split + (r - J)
        int lo = 0, hi = maxn;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (__ldg(A.round_off + mid) <= (int)it) lo = mid; else hi = mid - 1;
        }
        e = __ldg(A.perm + ((int)it - __ldg(A.round_off + lo)));
        n = __ldg(A.nsteps + e);
        if (n < 1 || n > kMaxSteps) n = 0;
        if (lo < nchunked) {
          k0 = lo * chunk;
          k1 = min(k0 + chunk - 1, n);
        } else {
          k0 = k1 = split + (lo - nchunked);
        }
      } else if (!A.perm) {
        // configurations b .. b + k1 of the item
        b = (int)it * Gcfg;
        k1 = min(Gcfg, A.B - b) - 1;
        if (rid < 0) rid = __ldg(A.robot_ids + b);
      } else {
        // slot sl's configurations perm[cfg_off[sl], cfg_off[sl + 1]) in
        // groups of G: item it is group it - item_off[sl]; b is a position in perm
        const int nrob = A.meta[1];
        int sl = 0;
        while (sl + 1 < nrob && __ldg(A.meta + 3 + sl) <= (int)it) ++sl;
        rid = __ldg(A.meta + 4 + 3 * nrob + sl);
        const int Gr = __ldg(A.meta + 4 + 2 * nrob + sl);
        b = __ldg(A.meta + 3 + nrob + sl) + ((int)it - __ldg(A.meta + 2 + sl)) * Gr;
        k1 = min(Gr, __ldg(A.meta + 4 + nrob + sl) - b) - 1;
      }
      // Steps (configurations) in groups of up to G = 32 / L: lanes g L +
      // link compute FK of link `link` at step g of the group, link row
      // g L + link of S.T holds it, and one traversal per query set decides
      // the group's steps together.  The FP64 pass uses groups of one.
      const KRobotDev& R = W->robots[rid];
      const int nl = R.nlinks;
      const int lgL = nl <= 8 ? 3 : (nl <= 16 ? 4 : 5);
      const int L = 1 << lgL;
      const int Gmax = FP64 ? 1 : 32 / L;
#pragma unroll 1
      for (int kb = k0; kb <= k1; kb += Gmax) {
        const int gn = min(Gmax, k1 - kb + 1);
        unsigned live = gn >= 32 ? 0xffffffffu : (1u << gn) - 1u;
        if (EDGES) {
          int fh = 0;
          if (lane == 0) fh = *((volatile int*)(A.first_hit + e));
          fh = __shfl_sync(0xffffffffu, fh, 0);
          if (fh <= kb) break;  // this or an earlier step of the edge already hit
          if (fh - kb < 32) live &= (1u << (fh - kb)) - 1u;
        }
        // configuration groups: position cb + i holds configuration
        // perm[cb + i] (mixed robots) or cb + i
        const int cb = EDGES ? 0 : b + kb;
        const int lane_cfg = EDGES || lane >= gn ? 0 : (A.perm ? __ldg(A.perm + cb + lane) : cb + lane);
        const int cfg0 = __shfl_sync(0xffffffffu, lane_cfg, 0);
        if (!EDGES && lane < gn) S.item_cfg[lane] = lane_cfg;
        if (lane == 0) {
          if (EDGES) {
            S.item_qa = A.qa + (size_t)e * nl;
            S.item_qb = A.qb + (size_t)e * nl;
          } else {
            S.item_qa = A.q + (size_t)cfg0 * A.q_stride;
            S.item_qb = nullptr;
          }
          S.item_k = EDGES ? kb : 0;
          S.item_n = n;
          S.item_id = EDGES ? e : cfg0;
          S.item_rid = rid;
        }
        // joint values in FP32 with an error bound e_q against the canonical
        // FP64 values (exact for configurations; FMA interpolation for edges)
        const int g = lane >> lgL, link = lane & (L - 1);
        const bool valid = ((live >> g) & 1u) && link < nl;
        const int my_cfg = __shfl_sync(0xffffffffu, lane_cfg, g < 32 ? g : 0);  // configuration of step g
        float q = 0.f, e_q = 0.f;
        if (valid) {
          if (EDGES) {
            const float a = __ldg(A.qa + (size_t)e * nl + link), bq = __ldg(A.qb + (size_t)e * nl + link);
            const float d = bq - a;
            q = fmaf((float)(kb + g) / (float)n, d, a);
            e_q = kU * (fabsf(d) + fabsf(q) + fabsf(a)) * 1.01f + 1e-30f;
          } else {
            q = __ldg(A.q + (size_t)my_cfg * A.q_stride + link);
          }
        }
        __syncwarp();
        if (!FP64) items += (unsigned long long)__popc(live);
        if (__any_sync(0xffffffffu, valid && !(fabsf(q) < 1.0e6f))) {
          if (lane == 0) set_status(W->status, KGPU_ERR_NOT_FINITE);
          continue;
        }
        if (A.mode != MODE_CONFIGS) {
          // joint limits: certain in FP32 away from the bounds, canonical FP64
          // comparison (RobotCSpace.cpp:610-630) within rounding of them
          bool unsure = false;
          if (valid) {
            const float lo = R.qmin[link], hi = R.qmax[link];
            const float tolq = e_q + 4.f * kU * (fabsf(q) + fmaxf(fabsf(lo), fabsf(hi))) + 1e-30f;
            unsure = !((q - lo) > tolq && (hi - q) > tolq);
          }
          bool viol = false;
          if (unsure) {
            const double q64 = EDGES ? kx_interp((double)S.item_qa[link], (double)S.item_qb[link], kb + g, n)
                                     : (double)q;  // configurations are exact in FP32
            viol = q64 < R.qmin64[link] || q64 > R.qmax64[link];
          }
          const unsigned vm = __reduce_or_sync(0xffffffffu, viol ? 1u << g : 0u);
          if (vm) {
            if (EDGES) {
              // the first violating step ends the edge there
              const int gv = __ffs(vm) - 1;
              if (lane == 0) atomicMin(A.first_hit + e, kb + gv);
              live &= (1u << gv) - 1u;
            } else {
              if ((vm >> lane) & 1u) A.feasible[lane_cfg] = 0;
              live &= ~vm;
            }
          }
          if (live == 0) {
            if (EDGES) break;
            continue;
          }
        }
        float P[12], delta;
        warp_fk32_group(R, lane, L, valid, q, e_q, P, &delta);
        if (valid) {
#pragma unroll
          for (int i = 0; i < 12; ++i) S.T[lane][i] = P[i];
          S.delta[lane] = delta;
          S.gerr[lane] = rot_gram_err32(P);
        }
        __syncwarp();
        unsigned env_hits = 0, self_hits = 0;
        int fk64 = 0;
        if (A.mode != MODE_CONFIGS) {
          // edges and feasibility: any contact decides a step, so the
          // environment and self queries share one traversal (one stack
          // drain per group instead of two)
          const int nq = R.nqueries_env + R.nqueries_self;
          if (nq > 0)
            env_hits = traverse<FP64, EDGES, STAGE>(S, W, R, R.query_off, nq, lane, spill, spill_cap, T64, fk64,
                                                    A, job_flush, cnt, all, warp, B, 0, live, lgL, nstage);
        } else {
          // configurations report the environment and self verdicts apart
          if (A.env_hit != nullptr && R.nqueries_env > 0)
            env_hits = traverse<FP64, EDGES, STAGE>(S, W, R, R.query_off, R.nqueries_env, lane, spill, spill_cap,
                                                    T64, fk64, A, job_flush, cnt, all, warp, B, 0, live, lgL, nstage);
          if (A.self_hit != nullptr && R.nqueries_self > 0)
            self_hits = traverse<FP64, EDGES, STAGE>(S, W, R, R.query_off + R.nqueries_env, R.nqueries_self, lane,
                                                     spill, spill_cap, T64, fk64, A, job_flush, cnt, all, warp, B, 0,
                                                     live, lgL, nstage);
        }
        if ((env_hits | self_hits) & kTrOverflow) {
          if (lane == 0) set_status(W->status, KGPU_ERR_OVERFLOW);
          continue;
        }
        // verdicts only ever turn into contacts (the outputs start as
        // "free"), so shared traversals and the FP64 pass can add theirs in
        // any order
        const unsigned any_hits = env_hits | self_hits;
        if (EDGES) {
          if (any_hits) {
            if (lane == 0) atomicMin(A.first_hit + e, kb + __ffs(any_hits) - 1);
            __syncwarp();
            break;
          }
        } else if (lane < 32) {
          if (A.mode == MODE_CONFIGS) {
            if ((env_hits >> lane) & 1u) A.env_hit[lane_cfg] = 1;
            if ((self_hits >> lane) & 1u) A.self_hit[lane_cfg] = 1;
          } else if ((any_hits >> lane) & 1u) {
            A.feasible[lane_cfg] = 0;
          }
        }
        __syncwarp();
      }  // step groups of the item
    }
  }

  // ---- queue drained: take over halves of the block's deep traversals
  // (edge batches; configuration items are short and their warps just end)
  if (EDGES) {
    if (lane == 0) {
      atomicExch(&B.flag[warp], 0);
      atomicAdd(&B.idle, 1);
    }
    __syncwarp();
#pragma unroll 1
    for (int spins = 0, waits = 0;;) {
      int f = 0;
      if (lane == 0) f = *((volatile int*)&B.flag[warp]);
      f = __shfl_sync(0xffffffffu, f, 0);
      if (f == 1) {
        __threadfence_block();
        if (lane == 0) atomicSub(&B.idle, 1);
        __syncwarp();
        const KRobotDev& R = W->robots[S.item_rid];
        const int nl = R.nlinks;
        const int lgL = nl <= 8 ? 3 : (nl <= 16 ? 4 : 5);
        unsigned live = S.don_live;
        if (EDGES) {
          int fh = 0;
          if (lane == 0) fh = *((volatile int*)(A.first_hit + S.item_id));
          fh = __shfl_sync(0xffffffffu, fh, 0);
          // steps not decided yet
          if (fh <= S.item_k) live = 0;
          else if (fh - S.item_k < 32) live &= (1u << (fh - S.item_k)) - 1u;
        }
        if (live != 0) {
          int fk64 = 0;
          const bool self = ((S.stack[0].y >> 25) & 63u) < 32u;
          const unsigned hits = traverse<FP64, EDGES, STAGE>(S, W, R, 0, 0, lane, spill, spill_cap, T64, fk64, A,
                                                             job_flush, cnt, all, warp, B, S.don_top, live, lgL,
                                                             nstage);
          if (lane == 0) {
            if (hits & kTrOverflow) {
              set_status(W->status, KGPU_ERR_OVERFLOW);
            } else if (hits) {
              const int g = __ffs(hits) - 1;
              if (EDGES) atomicMin(A.first_hit + S.item_id, S.item_k + g);
              else if (A.mode == MODE_FEASIBLE) A.feasible[S.item_id + g] = 0;
              else if (self && A.self_hit) A.self_hit[S.item_id + g] = 1;
              else if (!self && A.env_hit) A.env_hit[S.item_id + g] = 1;
            }
          }
        }
        if (lane == 0) {
          atomicExch(&B.flag[warp], 0);
          atomicAdd(&B.idle, 1);
        }
        __syncwarp();
        spins = 0;
        waits = 0;
        continue;
      }
      if (f == 0) {
        int idle = 0;
        if (lane == 0) idle = *((volatile int*)&B.idle);
        idle = __shfl_sync(0xffffffffu, idle, 0);
        if (idle >= kWarps || spins >= kShareSpins) {
          int old = 0;
          if (lane == 0) old = atomicCAS(&B.flag[warp], 0, 4);
          if (__shfl_sync(0xffffffffu, old, 0) == 0) break;  // left: no longer claimable
          continue;  // claimed meanwhile: the hand-over is in progress
        }
      } else if (++waits > (W->share_wait > 0 ? W->share_wait : kShareSpins)) {
        // a hand-over that does not complete: report it and stop
        if (lane == 0) set_status(W->status, KGPU_ERR_TIMEOUT);
        break;
      }
      ++spins;
      __nanosleep(256);
    }
  }
  unsigned long long np = cnt.node_pairs, tp = cnt.tri_pairs, bd = cnt.band;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    np += __shfl_down_sync(0xffffffffu, np, o);
    tp += __shfl_down_sync(0xffffffffu, tp, o);
    bd += __shfl_down_sync(0xffffffffu, bd, o);
  }
  if (lane == 0 && W->stats) {
    atomicAdd(W->stats + 0, items);
    atomicAdd(W->stats + 1, np);
    atomicAdd(W->stats + 2, tp);
    atomicAdd(W->stats + 3, bd);
    atomicAdd(W->stats + 4, cnt.spills);
    atomicAdd(W->stats + 5, cnt.cert);
    atomicAdd(W->stats + 6, cnt.hit64);
  }
}

// Which self-collision pairs occur over a batch of configurations
// (RandomizedSelfCollisionPairs, Cpp/Modeling/RandomizedSelfCollisions.cpp:
// 19-38, batched): per configuration, FK then every enabled link pair on its
// own, FP64 decisions inline; a pair found colliding sets bit tgt of
// pair_mask[a] (OR-accumulated across calls), and pairs already set are not
// tested again.  With `cand` (TestIndependentCollisions,
// RandomizedSelfCollisions.cpp:42-66): only the candidate pairs are tested,
// and a configuration in which exactly one of them collides sets that pair.
__global__ void __launch_bounds__(kWarps * 32, 2) k_self_pairs(const KWorldDev* __restrict__ W, const EngineArgs A,
                                                                 const unsigned int* __restrict__ cand,
                                                                 unsigned int* pair_mask)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem* all = reinterpret_cast<WarpSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem& S = all[warp];
  BlockShare& B = *reinterpret_cast<BlockShare*>(smem_raw + sizeof(WarpSmem) * kWarps);
  const int gwarp = blockIdx.x * kWarps + warp;
  uint2* wscratch = A.spill + (size_t)gwarp * A.spill_per_warp;
  double(*T64)[12] = reinterpret_cast<double(*)[12]>(wscratch);
  uint2* spill = wscratch + kT64Doubles;
  const int spill_cap = A.spill_per_warp - kT64Doubles;
  const int job_flush = kJobCap - 32;
  Cnt cnt;
  const KRobotDev& R = W->robots[A.robot];
  const int nl = R.nlinks;
#pragma unroll 1
  for (;;) {
    unsigned int b = 0;
    if (lane == 0) b = atomicAdd(A.head, 1u);
    b = __shfl_sync(0xffffffffu, b, 0);
    if (b >= (unsigned)A.B) break;
    const float q = lane < nl ? __ldg(A.q + (size_t)b * nl + lane) : 0.f;
    if (__any_sync(0xffffffffu, lane < nl && !(fabsf(q) < 1.0e6f))) {
      if (lane == 0) set_status(W->status, KGPU_ERR_NOT_FINITE);
      continue;
    }
    if (lane == 0) {
      S.item_qa = A.q + (size_t)b * nl;
      S.item_qb = nullptr;
      S.item_k = 0;
      S.item_n = 0;
      S.item_id = (int)b;
      S.item_rid = A.robot;
    }
    float P[12], delta;
    warp_fk32(R, lane, q, 0.f, P, &delta);
    if (lane < nl) {
#pragma unroll
      for (int i = 0; i < 12; ++i) S.T[lane][i] = P[i];
      S.delta[lane] = delta;
      S.gerr[lane] = rot_gram_err32(P);
    }
    __syncwarp();
    int fk64 = 0;
    int found = 0, fa = 0, ft = 0;
#pragma unroll 1
    for (int qi = 0; qi < R.nqueries_self; ++qi) {
      const int qidx = R.query_off + R.nqueries_env + qi;
      const uint32_t qw = __ldg(W->queries + qidx);
      const int a = qw & 0xff, tgt = (qw >> 8) & 0xff;
      if (cand) {
        if (!((__ldg(cand + a) >> tgt) & 1u)) continue;  // not a candidate pair
      } else {
        unsigned int known = 0;
        if (lane == 0) known = *((volatile unsigned int*)(pair_mask + a));
        if ((__shfl_sync(0xffffffffu, known, 0) >> tgt) & 1u) continue;
      }
      const unsigned hits = traverse<true, false>(S, W, R, qidx, 1, lane, spill, spill_cap, T64, fk64, A, job_flush,
                                                  cnt, all, warp, B, 0, 1u, 5);
      if (hits & kTrOverflow) {
        if (lane == 0) set_status(W->status, KGPU_ERR_OVERFLOW);
        found = 2;  // no verdict for this configuration
        break;
      }
      if (hits) {
        if (!cand) {
          if (lane == 0) atomicOr(pair_mask + a, 1u << tgt);
        } else if (++found > 1) {
          break;  // more than one candidate pair collides
        } else {
          fa = a;
          ft = tgt;
        }
      }
      __syncwarp();
    }
    // independent pairs: the configuration's only colliding candidate pair
    if (cand && found == 1 && lane == 0) atomicOr(pair_mask + fa, 1u << ft);
    __syncwarp();
  }
}

// FP64 decision of the triangle pairs the main pass left undecided.  A warp
// takes `per` consecutive records (one per lane; per = the list length over
// the warps, 1..32, so a short list is spread over all warps and its latency
// is one record's); records of the same item are contiguous (a warp appends
// its batch with one atomic), so for each item in its records the warp
// computes the FP64 transforms once (canonical joint
// values: the float input widened, or the FP64 edge interpolation) and the
// item's lanes run the FP64 triangle test (band_retest) in parallel.  A
// contact sets the item's verdict: first_hit = min(first_hit, k) for an edge
// step, env_hit / self_hit = 1 or feasible = 0 for a configuration (the main
// pass wrote the verdict from the decided pairs; these writes only turn it
// into a contact).  Does nothing when the list overflowed (the fallback pass
// re-checks every item then).
__global__ void __launch_bounds__(kWarps * 32) k_band(const KWorldDev* __restrict__ W, const EngineArgs A)
{
  __shared__ double q64s[kWarps][kMaxLinks];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gwarp = blockIdx.x * kWarps + warp;
  const unsigned npend = *((volatile unsigned int*)A.pend_count);
  if (npend > (unsigned)A.pend_cap) return;
  double(*T64)[12] = reinterpret_cast<double(*)[12]>(A.spill + (size_t)gwarp * A.spill_per_warp);
  unsigned long long band = 0, hits = 0;
  const unsigned nwarps = gridDim.x * kWarps;
  const unsigned per = min(32u, max(1u, (npend + nwarps - 1) / nwarps));
#pragma unroll 1
  for (unsigned base = (unsigned)gwarp * per; base < npend; base += nwarps * per) {
    const bool have = (unsigned)lane < per && base + lane < npend;
    const uint4 r = have ? A.pend[base + lane] : make_uint4(0u, 0u, 0u, 0u);
    const int item = (int)r.x, k = (int)(r.y & 0xffffu);
    unsigned todo = __ballot_sync(0xffffffffu, have);
#pragma unroll 1
    while (todo) {
      const int src = __ffs(todo) - 1;
      const int gi = __shfl_sync(0xffffffffu, item, src), gk = __shfl_sync(0xffffffffu, k, src);
      const bool mine = have && item == gi && k == gk;
      todo &= ~__ballot_sync(0xffffffffu, mine);
      if (A.mode == MODE_EDGES) {
        // one read, broadcast: lanes reading separately could see another
        // warp's update at different times and split the warp
        int fh = 0;
        if (lane == 0) fh = *((volatile int*)(A.first_hit + gi));
        if (__shfl_sync(0xffffffffu, fh, 0) <= gk) continue;  // decided already
      }
      int rid = A.robot;
      if (A.mode != MODE_EDGES && rid < 0) rid = __ldg(A.robot_ids + gi);
      const KRobotDev& R = W->robots[rid];
      const int nl = R.nlinks;
      if (lane < nl) {
        double q;
        if (A.mode == MODE_EDGES) {
          int n = __ldg(A.nsteps + gi);
          if (n < 1 || n > kMaxSteps) n = 0;
          q = kx_interp((double)__ldg(A.qa + (size_t)gi * nl + lane), (double)__ldg(A.qb + (size_t)gi * nl + lane),
                        gk, n);
        } else {
          q = (double)__ldg(A.q + (size_t)gi * A.q_stride + lane);
        }
        q64s[warp][lane] = q;
      }
      __syncwarp();
      warp_fk64(R, q64s[warp], T64, lane);
      __syncwarp();
      int hit = 0, tgt = 0;
      if (mine) {
        band++;
        tgt = (int)((r.y >> 21) & 63u);
        hit = band_retest(W, R, T64, (int)((r.y >> 16) & 31u), (int)r.z, tgt, (int)r.w);
        hits += hit ? 1 : 0;
      }
      const bool env_hit = __any_sync(0xffffffffu, hit && tgt >= 32);
      const bool self_hit = __any_sync(0xffffffffu, hit && tgt < 32);
      if (lane == 0 && (env_hit || self_hit)) {
        if (A.mode == MODE_EDGES) atomicMin(A.first_hit + gi, gk);
        else if (A.mode == MODE_FEASIBLE) A.feasible[gi] = 0;
        else {
          if (env_hit) A.env_hit[gi] = 1;
          if (self_hit) A.self_hit[gi] = 1;
        }
      }
      __syncwarp();
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    band += __shfl_down_sync(0xffffffffu, band, o);
    hits += __shfl_down_sync(0xffffffffu, hits, o);
  }
  if (lane == 0 && W->stats && band) {
    atomicAdd(W->stats + 3, band);
    atomicAdd(W->stats + 6, hits);
  }
}

// ---- mixed-robot configuration batches ------------------------------------
// Configurations are counted and scattered by robot so that one robot's
// configurations form groups of G_r = 32 / L_r (1 with the FP64 test
// inline).  Robots with more links (costlier items) come first, so that the
// queue ends on cheap items.  meta, per slot s (s = 0..nrob; robot of slot s
// = rob[s]): [0] work items, [1] robots, [2 + s] first item of slot s,
// [3 + nrob + s] first position of slot s in perm, [4 + 2 nrob + s] its G,
// [4 + 3 nrob + s] rob[s], [4 + 4 nrob + r] slot of robot r.  The order
// inside a robot's range depends on atomics; verdicts do not.
__global__ void k_cfg_count(const int* robot_ids, int B, int nrob, int* counts, int* status)
{
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int r = robot_ids[b];
  if (r < 0 || r >= nrob) atomicCAS(status, 0, KGPU_ERR_INVALID);
  else atomicAdd(counts + r, 1);
}

__global__ void k_cfg_offsets(const KWorldDev* __restrict__ W, const int* counts, int nrob, int single, int* fill,
                              int* meta)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int io = 0, co = 0;
  unsigned placed = 0;
  for (int sl = 0; sl < nrob; ++sl) {
    int r = -1;  // the unplaced robot with the most links (lowest index on ties)
    for (int c = 0; c < nrob; ++c)
      if (!((placed >> c) & 1u) && (r < 0 || W->robots[c].nlinks > W->robots[r].nlinks)) r = c;
    placed |= 1u << r;
    const int nl = W->robots[r].nlinks;
    const int G = single ? 1 : (nl <= 8 ? 4 : (nl <= 16 ? 2 : 1));
    meta[2 + sl] = io;
    meta[3 + nrob + sl] = co;
    meta[4 + 2 * nrob + sl] = G;
    meta[4 + 3 * nrob + sl] = r;
    meta[4 + 4 * nrob + r] = sl;
    io += (counts[r] + G - 1) / G;
    co += counts[r];
    fill[r] = 0;
  }
  meta[2 + nrob] = io;
  meta[3 + 2 * nrob] = co;
  meta[0] = io;
  meta[1] = nrob;
}

__global__ void k_cfg_scatter(const int* robot_ids, int B, int nrob, const int* meta, int* fill, int* perm)
{
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int r = robot_ids[b];
  if (r < 0 || r >= nrob) return;
  perm[meta[3 + nrob + meta[4 + 4 * nrob + r]] + atomicAdd(fill + r, 1)] = b;
}

// ---- edge preparation ------------------------------------------------------
// Work items of an edge batch.  Edges are sorted by descending step count n
// (perm), so the edges with n >= s are exactly perm[0, count_ge[s]).  The
// steps are grouped in rounds: while much work remains, a round is a chunk of
// `chunk` consecutive steps [r*chunk, r*chunk + chunk) of every edge that
// reaches it (one work item per edge, its steps checked in order); from step
// S_split on, a round is one step, so that the last items in the queue are
// short and the launch does not end on one warp's long chunk.  S_split is
// the first multiple of `chunk` from which fewer than `tail_items` items
// remain.  meta: [0] last round index, [1] total items, [2] number of chunked
// rounds J, [3] S_split (= J * chunk).
__global__ void k_edges_prep1(const int* nsteps, int E, int* hist, int* meta, int* first_hit,
                              int* status)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  int n = nsteps[e];
  first_hit[e] = INT_MAX;
  if (n < 1 || n > kMaxSteps) {
    atomicCAS(status, 0, KGPU_ERR_INVALID);
    n = 0;  // treated as a single configuration
  }
  atomicAdd(hist + n, 1);
  atomicMax(meta + 0, n);
}

// inclusive scan of one value per thread over a 1024-thread block
__device__ __forceinline__ long long block_scan_incl(long long v, long long* sh)
{
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long x = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += x;
    __syncthreads();
  }
  long long r = sh[t];
  __syncthreads();
  return r;
}

// One block of 1024 threads.  hist[v] (edges with n == v) becomes the base
// position of those edges in perm (= count_ge[v+1]); cge[v] = count_ge[v];
// round_off[r] = items in rounds < r.
__global__ void __launch_bounds__(1024) k_edges_prep2(int* hist, int* cge, int* round_off, int* meta, int* status,
                                                      int chunk, long long tail_items)
{
  __shared__ long long sh[1024];
  __shared__ int s_star;
  const int t = threadIdx.x;
  const int maxn = meta[0];
  const int len = maxn + 1;
  const int per = (len + 1023) / 1024;
  // suffix sums of the histogram: thread t owns steps [maxn - (t+1)*per, maxn - t*per)
  long long local = 0;
  for (int i = 0; i < per; ++i) {
    const int v = maxn - (t * per + i);
    if (v >= 0) local += hist[v];
  }
  long long run = block_scan_incl(local, sh) - local;  // edges with larger n
  for (int i = 0; i < per; ++i) {
    const int v = maxn - (t * per + i);
    if (v >= 0) {
      const int h = hist[v];
      hist[v] = (int)run;  // base = count_ge[v+1]
      run += h;
      cge[v] = (int)run;   // count_ge[v]
    }
  }
  if (t == 0) s_star = len;
  __syncthreads();
  // items remaining from step v on: rem(v) = sum of count_ge over [v, maxn];
  // S* = the first v with rem(v) < tail_items (rem is non-increasing)
  local = 0;
  for (int i = 0; i < per; ++i) {
    const int v = maxn - (t * per + i);
    if (v >= 0) local += cge[v];
  }
  long long rem = block_scan_incl(local, sh) - local;
  for (int i = 0; i < per; ++i) {
    const int v = maxn - (t * per + i);
    if (v >= 0) {
      rem += cge[v];
      if (rem < tail_items) atomicMin(&s_star, v);
    }
  }
  __syncthreads();
  const int J = s_star / chunk;            // chunked rounds cover steps [0, J*chunk)
  const int split = J * chunk;
  const int rounds = J + (len - split);    // then one round per step up to maxn
  const int rper = (rounds + 1023) / 1024;
  // prefix sums of the round sizes; thread t owns rounds [t*rper, (t+1)*rper)
  local = 0;
  for (int i = 0; i < rper; ++i) {
    const int r = t * rper + i;
    if (r < rounds) local += cge[r < J ? r * chunk : split + (r - J)];
  }
  long long acc = block_scan_incl(local, sh) - local;
  for (int i = 0; i < rper; ++i) {
    const int r = t * rper + i;
    if (r < rounds) {
      round_off[r] = acc > INT_MAX ? INT_MAX : (int)acc;
      acc += cge[r < J ? r * chunk : split + (r - J)];
    }
  }
  if (t == 1023) {
    if (acc > INT_MAX) atomicCAS(status, 0, KGPU_ERR_INVALID);
    round_off[rounds] = acc > INT_MAX ? INT_MAX : (int)acc;
    meta[0] = rounds - 1;
    meta[1] = acc > INT_MAX ? INT_MAX : (int)acc;
    meta[2] = J;
    meta[3] = split;
  }
}

__global__ void k_edges_prep3(const int* nsteps, int E, const int* base, int* fill, int* perm)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  int n = nsteps[e];
  if (n < 1 || n > kMaxSteps) n = 0;
  perm[base[n] + atomicAdd(fill + n, 1)] = e;
}

__global__ void k_edges_finalize(int* first_hit, int E)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < E && first_hit[e] == INT_MAX) first_hit[e] = -1;
}

__global__ void k_fk(const KWorldDev* __restrict__ W, int robot, const float* q, int B, float* T, float* err)
{
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= B) return;
  const KRobotDev& R = W->robots[robot];
  int nl = R.nlinks;
  float qv = lane < nl ? q[(size_t)warp * nl + lane] : 0.f;
  float P[12], delta;
  warp_fk32(R, lane, qv, 0.f, P, &delta);
  if (lane < nl) {
    for (int i = 0; i < 12; ++i) T[((size_t)warp * nl + lane) * 12 + i] = P[i];
    if (err) err[(size_t)warp * nl + lane] = delta;
  }
}

// Canonical FP64 forward kinematics (the transforms every FP64 decision of
// the engine uses), one warp per configuration, lane i link i by the
// sequential chain root -> i (bit-identical to the composition in link
// order).
__global__ void k_fk64(const KWorldDev* __restrict__ W, int robot, const float* q, int B, double* T)
{
  __shared__ double qs[8][kMaxLinks];
  const int lane = threadIdx.x & 31, wib = (threadIdx.x >> 5) & 7;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= B) return;
  const KRobotDev& R = W->robots[robot];
  const int nl = R.nlinks;
  const float qv = lane < nl ? q[(size_t)warp * nl + lane] : 0.f;
  if (__any_sync(0xffffffffu, lane < nl && !(fabsf(qv) < 1.0e6f))) {
    if (lane == 0) set_status(W->status, KGPU_ERR_NOT_FINITE);
    return;
  }
  if (lane < nl) qs[wib][lane] = (double)qv;
  __syncwarp();
  if (lane < nl) {
    double Tl[12];
    chain64(R, qs[wib], lane, Tl);
    for (int i = 0; i < 12; ++i) T[((size_t)warp * nl + lane) * 12 + i] = Tl[i];
  }
}

// Full Jacobian of a point on a link, one warp per configuration: rows 0-2
// the angular part (column j = world axis of joint j for a revolute ancestor,
// 0 otherwise), rows 3-5 the linear part (w_j x (p - o_j) revolute, w_j
// prismatic), p = T_link * plocal, o_j the origin of link j's frame; columns
// of links that are not the link or its ancestors are 0
// (RobotModelLink::getJacobian, Python/klampt/src/robotsim.cpp:4817-4825).
__global__ void k_jacobian(const KWorldDev* __restrict__ W, int robot, const float* q, const int* links,
                           int link_all, const float* plocal, int B, float* J)
{
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= B) return;
  const KRobotDev& R = W->robots[robot];
  const int nl = R.nlinks;
  const int li = links ? __ldg(links + warp) : link_all;
  float* Jb = J + (size_t)warp * 6 * nl;
  if (li < 0 || li >= nl) {
    if (lane == 0) set_status(W->status, KGPU_ERR_INVALID);
    return;
  }
  const float qv = lane < nl ? __ldg(q + (size_t)warp * nl + lane) : 0.f;
  float P[12], delta;
  warp_fk32(R, lane, qv, 0.f, P, &delta);
  // the point in world coordinates, from link li's transform
  float Ti[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) Ti[k] = __shfl_sync(0xffffffffu, P[k], li);
  const float px = plocal[3 * (size_t)warp], py = plocal[3 * (size_t)warp + 1], pz = plocal[3 * (size_t)warp + 2];
  const float3 p = xform32(Ti, make_float3(px, py, pz));
  if (lane < nl) {
    bool anc = false;
    for (int j = li; j >= 0; j = R.parents[j])
      if (j == lane) { anc = true; break; }
    float c[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (anc && R.jtype[lane] != KX_JOINT_WELD) {
      const float ax = R.axis[lane][0], ay = R.axis[lane][1], az = R.axis[lane][2];
      const float wx = P[0] * ax + P[1] * ay + P[2] * az;
      const float wy = P[3] * ax + P[4] * ay + P[5] * az;
      const float wz = P[6] * ax + P[7] * ay + P[8] * az;
      if (R.jtype[lane] == KX_JOINT_REVOLUTE) {
        const float rx = p.x - P[9], ry = p.y - P[10], rz = p.z - P[11];
        c[0] = wx; c[1] = wy; c[2] = wz;
        c[3] = wy * rz - wz * ry;
        c[4] = wz * rx - wx * rz;
        c[5] = wx * ry - wy * rx;
      } else {
        c[3] = wx; c[4] = wy; c[5] = wz;
      }
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) Jb[(size_t)r * nl + lane] = c[r];
  }
}

template <bool STAGE>
constexpr size_t engine_smem() { return STAGE ? kStageOffset + sizeof(KNode) * kStageNodes : kBlockSmem; }

template <int MINB, bool FP64, bool EDGES, bool STAGE = false>
cudaError_t init_engine()
{
  return cudaFuncSetAttribute(k_engine<MINB, FP64, EDGES, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)engine_smem<STAGE>());
}

// the shared-memory attribute is set once per process by engine_init(), so
// that launches can be captured into CUDA graphs
template <int MINB, bool FP64, bool STAGE = false>
cudaError_t launch_engine(const KWorldDev* W, const EngineArgs& A, int blocks, cudaStream_t s)
{
  const size_t smem = engine_smem<STAGE>();
  if (A.mode == MODE_EDGES)
    k_engine<MINB, FP64, true, STAGE><<<blocks, kWarps * 32, smem, s>>>(W, A);
  else
    k_engine<MINB, FP64, false, STAGE><<<blocks, kWarps * 32, smem, s>>>(W, A);
  return cudaGetLastError();
}

// Main pass, FP64 decision of its undecided pairs (k_band), and the fallback
// pass (which returns at once unless the pair list overflowed).  `blocks` =
// SMs x blocks per SM; the blocks-per-SM value selects the register budget
// of the main pass's instantiation.  Queue heads and the list count live in
// S.counters ([0] main head, [1] pair count, [2] fallback head), cleared
// here.
cudaError_t dispatch_engine(const KWorldDev* W, EngineArgs A, const Scratch& S, int blocks, int per_sm,
                            cudaStream_t s)
{
  cudaError_t err = cudaMemsetAsync(S.counters, 0, 3 * sizeof(unsigned int), s);
  if (err != cudaSuccess) return err;
  A.head = S.counters;
  A.pend_count = S.counters + 1;
  A.pend = S.pend;
  A.pend_cap = S.pend_cap;
  A.stage_nodes = S.stage_nodes;
  if (S.main_pass_ev[0] != nullptr &&
      (err = cudaEventRecordWithFlags(S.main_pass_ev[0], s, cudaEventRecordExternal)) != cudaSuccess)
    return err;
  if (A.inline64) return per_sm == 3 ? launch_engine<3, true>(W, A, blocks, s) : launch_engine<2, true>(W, A, blocks, s);
  switch (per_sm) {
    case 3: err = launch_engine<3, false>(W, A, blocks, s); break;
    case 4: err = launch_engine<4, false>(W, A, blocks, s); break;
    default:
      err = A.stage_nodes > 0 ? launch_engine<2, false, true>(W, A, blocks, s) : launch_engine<2, false>(W, A, blocks, s);
      break;
  }
  if (err != cudaSuccess) return err;
  if (S.main_pass_ev[1] != nullptr &&
      (err = cudaEventRecordWithFlags(S.main_pass_ev[1], s, cudaEventRecordExternal)) != cudaSuccess)
    return err;
  const int sms = per_sm > 0 && blocks / per_sm > 0 ? blocks / per_sm : 1;
  k_band<<<2 * sms, kWarps * 32, 0, s>>>(W, A);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  A.head = S.counters + 2;
  return launch_engine<2, true>(W, A, 2 * sms, s);
}

}  // namespace

size_t engine_smem_per_warp() { return sizeof(WarpSmem); }
int engine_warps_per_block() { return kWarps; }
int engine_scratch_doubles() { return kT64Doubles; }

cudaError_t engine_init()
{
  cudaError_t e = init_engine<2, false, true>();
  if (e == cudaSuccess) e = init_engine<3, false, true>();
  if (e == cudaSuccess) e = init_engine<4, false, true>();
  if (e == cudaSuccess) e = init_engine<2, true, true>();
  if (e == cudaSuccess) e = init_engine<3, true, true>();
  if (e == cudaSuccess) e = init_engine<2, false, false>();
  if (e == cudaSuccess) e = init_engine<3, false, false>();
  if (e == cudaSuccess) e = init_engine<4, false, false>();
  if (e == cudaSuccess) e = init_engine<2, true, false>();
  if (e == cudaSuccess) e = init_engine<3, true, false>();
  if (e == cudaSuccess) e = init_engine<2, false, true, true>();
  if (e == cudaSuccess) e = init_engine<2, false, false, true>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_self_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(WarpSmem) * kWarps + sizeof(BlockShare)));
  return e;
}

cudaError_t launch_fk(const KWorldDev* W, int robot, const float* q, int B, float* T, float* err,
                      cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  int threads = 256;
  long long warps = B;
  int blocks = (int)((warps * 32 + threads - 1) / threads);
  k_fk<<<blocks, threads, 0, s>>>(W, robot, q, B, T, err);
  return cudaGetLastError();
}

cudaError_t launch_fk64(const KWorldDev* W, int robot, const float* q, int B, double* T, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  const int threads = 256;
  const int blocks = (int)(((long long)B * 32 + threads - 1) / threads);
  k_fk64<<<blocks, threads, 0, s>>>(W, robot, q, B, T);
  return cudaGetLastError();
}

cudaError_t launch_self_pairs(const KWorldDev* W, const Scratch& S, int robot, const float* q, int B,
                              const unsigned int* cand, unsigned int* pair_mask, int num_sms, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  cudaError_t err = cudaMemsetAsync(S.counters, 0, sizeof(unsigned int), s);
  if (err != cudaSuccess) return err;
  EngineArgs A = {};
  A.mode = MODE_CONFIGS;
  A.robot = robot;
  A.q = q;
  A.q_stride = 0;
  A.B = B;
  A.head = S.counters;
  A.spill = S.spill;
  A.spill_per_warp = (int)S.spill_per_warp;
  A.inline64 = 1;
  const size_t smem = sizeof(WarpSmem) * kWarps + sizeof(BlockShare);
  k_self_pairs<<<2 * num_sms, kWarps * 32, smem, s>>>(W, A, cand, pair_mask);
  return cudaGetLastError();
}

cudaError_t launch_jacobian(const KWorldDev* W, int robot, const float* q, const int* links, int link_all,
                            const float* plocal, int B, float* J, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  const int threads = 256;
  const int blocks = (int)(((long long)B * 32 + threads - 1) / threads);
  k_jacobian<<<blocks, threads, 0, s>>>(W, robot, q, links, link_all, plocal, B, J);
  return cudaGetLastError();
}

cudaError_t launch_check_configs(const KWorldDev* W, const Scratch& S, int robot, const int* robot_ids,
                                 const float* q, int q_stride, int B, uint8_t* env_hit, uint8_t* self_hit,
                                 uint8_t* feasible, int blocks, int per_sm, cudaStream_t s, int grab,
                                 int job_flush, int fp64_inline, int nrobots, int* status)
{
  if (B <= 0) return cudaSuccess;
  // the kernels only ever record contacts: start from "free"
  cudaError_t err = cudaSuccess;
  if (env_hit) err = cudaMemsetAsync(env_hit, 0, (size_t)B, s);
  if (err == cudaSuccess && self_hit) err = cudaMemsetAsync(self_hit, 0, (size_t)B, s);
  if (err == cudaSuccess && feasible) err = cudaMemsetAsync(feasible, 1, (size_t)B, s);
  if (err != cudaSuccess) return err;
  EngineArgs A = {};
  A.grab = grab;
  A.job_flush = job_flush;
  A.mode = feasible ? MODE_FEASIBLE : MODE_CONFIGS;
  A.robot = robot;
  A.robot_ids = robot_ids;
  A.q = q;
  A.q_stride = q_stride;
  A.B = B;
  A.env_hit = env_hit;
  A.self_hit = self_hit;
  A.feasible = feasible;
  A.inline64 = fp64_inline == 1;  // default (-1): deferred, as for edge batches
  A.spill = S.spill;
  A.spill_per_warp = (int)S.spill_per_warp;
  if (robot < 0 && nrobots > 0 && nrobots <= 32 && status && S.edge_perm && (size_t)B <= S.edge_cap) {
    // mixed robots: sort by robot so that each robot's configurations go in groups
    int* counts = S.edge_hist;
    int* fill = S.edge_hist + 32;
    if ((err = cudaMemsetAsync(counts, 0, 32 * sizeof(int), s)) != cudaSuccess) return err;
    const int tb = 256, gb = (B + tb - 1) / tb;
    k_cfg_count<<<gb, tb, 0, s>>>(robot_ids, B, nrobots, counts, status);
    k_cfg_offsets<<<1, 32, 0, s>>>(W, counts, nrobots, A.inline64, fill, S.edge_meta);
    k_cfg_scatter<<<gb, tb, 0, s>>>(robot_ids, B, nrobots, S.edge_meta, fill, S.edge_perm);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    A.perm = S.edge_perm;
    A.meta = S.edge_meta;
  }
  return dispatch_engine(W, A, S, blocks, per_sm, s);
}

cudaError_t launch_check_edges(const KWorldDev* W, int* status, const Scratch& S, int robot, const float* qa,
                               const float* qb, const int* nsteps, int E, int* first_hit, int blocks,
                               int per_sm, cudaStream_t s, int grab, int job_flush, int chunk, int fp64_inline)
{
  if (E <= 0) return cudaSuccess;
  cudaError_t err;
  if ((err = cudaMemsetAsync(S.edge_hist, 0, sizeof(int) * (kMaxSteps + 2), s)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(S.edge_meta, 0, sizeof(int) * 4, s)) != cudaSuccess) return err;
  int* fill = S.edge_meta + 4;  // kMaxSteps+2 ints after the meta words
  if ((err = cudaMemsetAsync(fill, 0, sizeof(int) * (kMaxSteps + 2), s)) != cudaSuccess) return err;
  int tb = 256, gb = (E + tb - 1) / tb;
  chunk = chunk >= 1 && chunk <= kMaxChunk ? chunk : kDefaultChunk;
  int* cge = fill + kMaxSteps + 2;  // count_ge table after the fill counters
  const long long tail_items = (long long)kTailItemsPerWarp * blocks * kWarps;
  k_edges_prep1<<<gb, tb, 0, s>>>(nsteps, E, S.edge_hist, S.edge_meta, first_hit, status);
  k_edges_prep2<<<1, 1024, 0, s>>>(S.edge_hist, cge, S.edge_round_off, S.edge_meta, status, chunk, tail_items);
  k_edges_prep3<<<gb, tb, 0, s>>>(nsteps, E, S.edge_hist, fill, S.edge_perm);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  EngineArgs A = {};
  A.grab = grab;
  A.job_flush = job_flush;
  A.chunk = chunk;
  A.inline64 = fp64_inline == 1;  // default (-1): deferred for edge batches
  A.mode = MODE_EDGES;
  A.robot = robot;
  A.qa = qa;
  A.qb = qb;
  A.nsteps = nsteps;
  A.E = E;
  A.first_hit = first_hit;
  A.round_off = S.edge_round_off;
  A.perm = S.edge_perm;
  A.meta = S.edge_meta;
  A.spill = S.spill;
  A.spill_per_warp = (int)S.spill_per_warp;
  if ((err = dispatch_engine(W, A, S, blocks, per_sm, s)) != cudaSuccess) return err;
  k_edges_finalize<<<gb, tb, 0, s>>>(first_hit, E);
  return cudaGetLastError();
}

}  // namespace kgpu
