// kgpu_geom.cu — proximity queries between two free triangle-mesh
// geometries under caller-supplied transforms, batched over transforms:
// Geometry3D::collides / withinDistance / distance_ext
// (Python/klampt/src/robotsim.cpp:1656-1662, 1685-1690, 1782-1819;
// declarations Python/klampt/src/geometry.h:1020, 1031, 1103-1108).
//
// Definitions (the FP64 oracle's, oracle/oracle.cpp orc_geom_*):
//   world triangles  kx_xform_point(T, v) of the mesh's FP64 vertices;
//   collide(tol)     threshold m = (m_a + tol) + m_b (collision margins of
//                    the two geometries); m = 0: some triangle pair
//                    intersects (kx_tri_tri_overlap, touching counts);
//                    m > 0: some triangle pair has kx_tri_tri_dist2 <= m^2;
//   distance         the mesh distance d_mesh = min over triangle pairs of
//                    the canonical triangle distance (0 when they meet), its
//                    pair the lexicographically smallest (triangle of a,
//                    triangle of b) among the minimisers; searched below
//                    the bound upper + (m_a + m_b); reported as
//                    d = d_mesh - (m_a + m_b) (the margins fatten both
//                    geometries), or d = upper with elements (-1, -1) when
//                    nothing is closer.  Triangle meshes give unsigned mesh
//                    distances (geometry.h:1077-1092: TriangleMesh pairs are
//                    not among the signed combinations).
//
// GPU method, one warp per query: FP32 transforms with a rigorous bound on
// |FP32 - FP64| world placement of every vertex, FP32 BVH-vs-BVH traversal
// with inflated boxes and triangle tests; for collisions, triangle pairs the
// FP32 separating-axis test cannot separate are certified in FP32 or decided
// by the canonical FP64 test inline; for distances, the pairs within the
// error band of the running FP32 minimum are finalised in FP64 with a
// lexicographic warp reduction.
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "kgpu_dist32.cuh"

namespace kgpu {
kgpu_status record_error(kgpu_status code, const char* msg);
}  // namespace kgpu

struct kgpu_geom_s {
  int ntri = 0;
  double margin = 0.0;
  float r32 = 0.f;  // largest vertex norm (geometry frame), rounded up
  kgpu::KNode* d_nodes = nullptr;
  float* d_node_r = nullptr;
  float4* d_tri32 = nullptr;
  double* d_tri64 = nullptr;
  int* d_tri_orig = nullptr;
  int* d_status = nullptr;
};

namespace kgpu {
namespace {

constexpr int kGW = 4;        // warps per block
constexpr int kGStack = 512;  // node-pair stack entries per warp
constexpr int kGJobs = 64;    // leaf-pair jobs
constexpr int kGCand = 128;   // FP64 candidates (distance)

struct GeomDev {
  const KNode* nodes;
  const float* node_r;
  const float4* tri32;  // 3 per triangle, leaf order, geometry frame
  const double* tri64;  // 9 per triangle, leaf order
  const int* tri_orig;  // leaf order -> mesh order
  float r;
  int ntri;
};

struct GeomArgs {
  const double* Ta;
  const double* Tb;
  int sa, sb;      // transform strides in doubles: 12, or 0 for one transform for every query
  int B;
  double m;        // collide: threshold
  double bound;    // distance: bound on the mesh distance (+inf: none)
  double msum;     // distance: m_a + m_b
  double upper;    // distance: value reported when nothing is closer
  uint8_t* hit;
  double* d;
  double* cp;
  int* elem;
  double* dir;
  int* status;
};

struct __align__(16) GeomSmem {
  double T64[2][12];
  float T[2][12];
  float delta[2];
  uint2 stack[kGStack];
  uint32_t jobA[kGJobs], jobB[kGJobs], jobOff[kGJobs + 1];
  uint32_t candA[kGCand], candB[kGCand];
  float candD[kGCand];
  double pb2, pcp[3], pcq[3];
  int pA, pB, phave;
};

// world placement of geometry triangle t (leaf order) in FP64
__device__ __forceinline__ void tri_world64(const GeomDev& G, const double* T, int t, double* o)
{
  const double* p = G.tri64 + 9 * (size_t)t;
  for (int v = 0; v < 3; ++v) kx_xform_point(T, p + 3 * v, o + 3 * v);
}

__device__ __forceinline__ void tri_world32(const GeomDev& G, const float* T, int t, float3* o)
{
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const float4 x = __ldg(G.tri32 + 3 * (size_t)t + v);
    o[v] = xform32(T, make_float3(x.x, x.y, x.z));
  }
}

// Bound on |FP32 placement - FP64 placement| of any vertex of a geometry of
// vertex norm <= r under T: entry rounding of R, t and the vertex (2u |R||v|
// + u |t| per coordinate) plus the three FMA roundings (3u (|R||v| + |t|)),
// in 2-norm <= 5u ||R||_F r + 4u |t|, taken with headroom.
__device__ __forceinline__ float placement_err32(const float* T, float r)
{
  float nR = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) nR = fmaf(T[k], T[k], nR);
  nR = sqrtf(nR);
  const float nt = sqrtf(T[9] * T[9] + T[10] * T[10] + T[11] * T[11]);
  return kU * (6.f * nR * r + 5.f * nt) * 1.01f + 1e-30f;
}

// FP64 finalisation of distance candidates into the running lexicographic
// best (pb2, pA, pB): pairs whose squared distance is below the bound, or
// equal to the best with smaller (triangle of a, triangle of b)
constexpr int kSeedMaxTris = 4096;  // geometries up to this size are scanned for a seed

// An upper bound on the distance between the two placed surfaces: A's
// vertex nearest the centre of B's root box, then B's vertex nearest that
// vertex (the first vertex of each triangle), widened by the placement
// bounds and rounding.  Seeds the running minimum, so that the traversal
// prunes from the start.
__device__ __noinline__ float geom_seed(const GeomDev& GA, const GeomDev& GB, const float* TA, const float* TB,
                                        int lane, float dd)
{
  if (GA.ntri > kSeedMaxTris || GB.ntri > kSeedMaxTris) return FLT_MAX;
  const float3 cb = xform32(TB, make_float3(GB.nodes[0].a.x, GB.nodes[0].a.y, GB.nodes[0].a.z));
  float bd = FLT_MAX;
  float3 bv = cb;
  for (int t = lane; t < GA.ntri; t += 32) {
    const float4 x = __ldg(GA.tri32 + 3 * (size_t)t);
    const float3 w = xform32(TA, make_float3(x.x, x.y, x.z));
    const float dx = w.x - cb.x, dy = w.y - cb.y, dz = w.z - cb.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < bd) { bd = d2; bv = w; }
  }
  const float m = warp_min(bd);
  const unsigned mm = __ballot_sync(0xffffffffu, bd == m);
  const int src = mm ? __ffs(mm) - 1 : 0;
  bv = make_float3(__shfl_sync(0xffffffffu, bv.x, src), __shfl_sync(0xffffffffu, bv.y, src),
                   __shfl_sync(0xffffffffu, bv.z, src));
  float bo = FLT_MAX;
  for (int t = lane; t < GB.ntri; t += 32) {
    const float4 y = __ldg(GB.tri32 + 3 * (size_t)t);
    const float3 w = xform32(TB, make_float3(y.x, y.y, y.z));
    const float dx = w.x - bv.x, dy = w.y - bv.y, dz = w.z - bv.z;
    bo = fminf(bo, dx * dx + dy * dy + dz * dz);
  }
  bo = warp_min(bo);
  if (!(bo < FLT_MAX)) return FLT_MAX;
  return sqrtf(bo) * (1.f + 1e-5f) + 2.f * dd + 1e-6f;
}

__device__ __noinline__ void geom_flush(GeomSmem& S, const GeomDev& GA, const GeomDev& GB, int lane, int ncand,
                                        float lim)
{
  for (int base = 0; base < ncand; base += 32) {
    const int k = base + lane;
    double d2 = DBL_MAX;
    int oa = INT_MAX, ob = INT_MAX;
    double cp[3] = {0, 0, 0}, cq[3] = {0, 0, 0};
    if (k < ncand && S.candD[k] <= lim) {
      const int tA = (int)S.candA[k], tB = (int)S.candB[k];
      double P[9], Q[9];
      tri_world64(GA, S.T64[0], tA, P);
      tri_world64(GB, S.T64[1], tB, Q);
      d2 = kx_tri_tri_dist2(P, Q, cp, cq);
      oa = GA.tri_orig[tA];
      ob = GB.tri_orig[tB];
    }
    int src;
    double m2 = d2;
    int ma = oa, mb = ob;
    warp_lexmin(m2, ma, mb, src, lane);
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

template <bool DIST>
__global__ void __launch_bounds__(kGW * 32) k_geom(const GeomDev GA, const GeomDev GB, const GeomArgs A)
{
  __shared__ GeomSmem smem[kGW];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  GeomSmem& S = smem[warp];
  const unsigned lt = lanemask_lt();
  const int nwarps = gridDim.x * kGW;
  // collide: the FP32 threshold rounded up; distance: the FP32 search bound
  const float m32 = A.m > 0.0 ? (float)A.m * 1.000001f + 1e-12f : 0.f;
  const float fcut = A.bound < 1e30 ? (float)A.bound * 1.000001f + 1e-7f : FLT_MAX;
#pragma unroll 1
  for (int b = blockIdx.x * kGW + warp; b < A.B; b += nwarps) {
    // ---- transforms
    double tv = 0.0;
    if (lane < 12) tv = A.Ta[(size_t)b * A.sa + lane];
    else if (lane < 24) tv = A.Tb[(size_t)b * A.sb + lane - 12];
    if (__any_sync(0xffffffffu, lane < 24 && !(fabs(tv) < 1e6))) {
      if (lane == 0) set_status(A.status, KGPU_ERR_NOT_FINITE);
      continue;
    }
    if (lane < 12) { S.T64[0][lane] = tv; S.T[0][lane] = (float)tv; }
    else if (lane < 24) { S.T64[1][lane - 12] = tv; S.T[1][lane - 12] = (float)tv; }
    __syncwarp();
    if (lane < 2) S.delta[lane] = placement_err32(S.T[lane], lane == 0 ? GA.r : GB.r);
    if (lane == 0) {
      S.stack[0] = make_uint2(0u, 0u);
      const double bb = kx_mul(A.bound, A.bound);
      S.pb2 = bb > 1e-300 ? bb : 1e-300;
      S.pA = S.pB = INT_MAX;
      S.phave = 0;
    }
    __syncwarp();
    const float* TA = S.T[0];
    const float* TB = S.T[1];
    const float dd = S.delta[0] + S.delta[1];
    int top = (GA.ntri > 0 && GB.ntri > 0) ? 1 : 0, njobs = 0, ncand = 0;
    bool hit = false;
    float run = fcut;  // distance: FP32 upper bound on the minimum (warp-uniform)
    if (DIST && top > 0) run = fminf(run, geom_seed(GA, GB, TA, TB, lane, dd));
#pragma unroll 1
    while ((top > 0 || njobs > 0) && !hit) {
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
        for (uint32_t base = 0; base < total && !hit; base += 32) {
          const uint32_t p = base + lane;
          int tA = 0, tB = 0;
          float3 P[3], Q[3];
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
            tri_world32(GA, TA, tA, P);
            tri_world32(GB, TB, tB, Q);
          }
          if (!DIST) {
            bool h = false;
            if (p < total && !tri_separated32(P, Q, dd, m32)) {
              if (A.m == 0.0 && tri_certain_hit32(P[0], P[1], P[2], Q[0], Q[1], Q[2], dd)) {
                h = true;
              } else {
                // the band: the canonical FP64 decision
                double P64[9], Q64[9];
                tri_world64(GA, S.T64[0], tA, P64);
                tri_world64(GB, S.T64[1], tB, Q64);
                if (A.m == 0.0) {
                  h = kx_tri_tri_overlap(P64, Q64) != 0;
                } else {
                  double c1[3], c2[3];
                  h = kx_tri_tri_dist2(P64, Q64, c1, c2) <= kx_mul(A.m, A.m);
                }
              }
            }
            hit = __any_sync(0xffffffffu, h);
          } else {
            float d32 = FLT_MAX, e = 0.f;
            if (p < total) {
              float3 lo3 = P[0], hi3 = P[0];
#pragma unroll
              for (int k = 1; k < 6; ++k) {
                const float3 v = k < 3 ? P[k] : Q[k - 3];
                lo3 = make_float3(fminf(lo3.x, v.x), fminf(lo3.y, v.y), fminf(lo3.z, v.z));
                hi3 = make_float3(fmaxf(hi3.x, v.x), fmaxf(hi3.y, v.y), fmaxf(hi3.z, v.z));
              }
              const float span = fmaxf(fmaxf(hi3.x - lo3.x, hi3.y - lo3.y), hi3.z - lo3.z);
              e = dd + 128.f * kU * span + 1e-8f;
              if (tri_axis_lb32(P, Q, span) - e > run * (1.f + 2e-5f) + 2.f * e) d32 = FLT_MAX;
              else if (!tri_separated32(P, Q, dd, 0.f)) d32 = 0.f;
              else d32 = sqrtf(tri_dist2_32(P, Q));
            }
            run = fminf(run, warp_min(d32 < FLT_MAX ? d32 + e : FLT_MAX));
            const bool cand = d32 < FLT_MAX && d32 - e <= run * (1.f + 2e-5f);
            const unsigned mc = __ballot_sync(0xffffffffu, cand);
            if (ncand + __popc(mc) > kGCand) {
              geom_flush(S, GA, GB, lane, ncand, run * (1.f + 2e-5f) + 1e-6f);
              ncand = 0;
              if (S.phave) run = fminf(run, (float)sqrt(S.pb2) * (1.f + 1e-6f));
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
        }
        njobs = 0;
        continue;
      }
      // ---- node pairs; near the stack capacity the batch narrows to
      // depth-first order, whose growth is bounded by the trees' depth
      const int n = min(min(top, 32), max(1, kGStack - 64 - top));
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
        const KNode na = GA.nodes[nodeA];
        const KNode nb = GB.nodes[nodeB];
        const Box32 BA = xform_box(TA, na.a, na.b);
        const Box32 BB = xform_box(TB, nb.a, nb.b);
        const float slack = 4.f * kU * (fabsf(BA.c.x) + fabsf(BA.c.y) + fabsf(BA.c.z) + fabsf(BB.c.x) +
                                        fabsf(BB.c.y) + fabsf(BB.c.z) + 1.f);
        bool keep;
        if (!DIST) {
          keep = boxes_overlap(BA, BB, dd + m32 + slack);
        } else {
          const float lb_box = box_dist32(BA, BB.c, BB.h) - dd * 1.7321f - slack;
          const float cx = BA.c.x - BB.c.x, cy = BA.c.y - BB.c.y, cz = BA.c.z - BB.c.z;
          const float lb_sph = sqrtf(cx * cx + cy * cy + cz * cz) * (1.f - 4.f * kU) -
                               __ldg(GA.node_r + nodeA) - __ldg(GB.node_r + nodeB) - dd * 1.7321f - slack;
          keep = fmaxf(lb_box, lb_sph) <= run * (1.f + 2e-5f) + 3.f * dd + 1e-5f;
        }
        if (keep) {
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
      if (top + 2 * __popc(m1) > kGStack || njobs + __popc(m2) > kGJobs) {
        // cannot happen: the batch narrowing bounds the stack, and jobs are
        // processed once 16 are pending (at most 16 + 32 < kGJobs); checked
        // so that an error is reported, not hidden
        if (lane == 0) set_status(A.status, KGPU_ERR_OVERFLOW);
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
    if (!DIST) {
      if (lane == 0) A.hit[b] = hit ? 1 : 0;
      continue;
    }
    if (ncand > 0) geom_flush(S, GA, GB, lane, ncand, run * (1.f + 2e-5f) + 1e-6f);
    // ---- outputs
    const bool found = S.phave != 0;
    const double dm = found ? kx_sqrt(S.pb2) : 0.0;
    if (lane == 0) {
      A.d[b] = found ? kx_sub(dm, A.msum) : A.upper;
      A.elem[2 * (size_t)b] = found ? S.pA : -1;
      A.elem[2 * (size_t)b + 1] = found ? S.pB : -1;
    }
    if (lane < 6) A.cp[6 * (size_t)b + lane] = found ? (lane < 3 ? S.pcp[lane] : S.pcq[lane - 3]) : 0.0;
    if (A.dir && lane < 3)
      A.dir[3 * (size_t)b + lane] = found && dm > 0.0 ? kx_div(kx_sub(S.pcp[lane], S.pcq[lane]), dm) : 0.0;
    __syncwarp();
  }
}

GeomDev dev_view(const kgpu_geom_s* g)
{
  GeomDev d;
  d.nodes = g->d_nodes;
  d.node_r = g->d_node_r;
  d.tri32 = g->d_tri32;
  d.tri64 = g->d_tri64;
  d.tri_orig = g->d_tri_orig;
  d.r = g->r32;
  d.ntri = g->ntri;
  return d;
}

template <class T>
cudaError_t upload_vec(T** dst, const std::vector<T>& v)
{
  *dst = nullptr;
  if (v.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)dst, v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void free_geom(kgpu_geom_s* g)
{
  cudaFree(g->d_nodes);
  cudaFree(g->d_node_r);
  cudaFree(g->d_tri32);
  cudaFree(g->d_tri64);
  cudaFree(g->d_tri_orig);
  cudaFree(g->d_status);
  delete g;
}

int blocks_for(int B)
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int want = (B + kGW - 1) / kGW;
  return std::max(1, std::min(want, 8 * std::max(1, sms)));
}

kgpu_status check_pair(kgpu_geom a, kgpu_geom b, const double* Ta, const double* Tb, int32_t B, int32_t flags)
{
  if (!a || !b) return record_error(KGPU_ERR_INVALID, "kgpu_geom: null geometry");
  if (B < 0 || (B > 0 && (!Ta || !Tb))) return record_error(KGPU_ERR_INVALID, "kgpu_geom: bad transform buffers");
  if (flags & ~(KGPU_GEOM_FIXED_A | KGPU_GEOM_FIXED_B)) return record_error(KGPU_ERR_INVALID, "kgpu_geom: unknown flag");
  return KGPU_OK;
}

}  // namespace
}  // namespace kgpu

using namespace kgpu;

extern "C" kgpu_status kgpu_geom_create(const kgpu_geom_desc* d, kgpu_geom* out)
{
  if (!d || !out) return record_error(KGPU_ERR_INVALID, "kgpu_geom_create: null argument");
  *out = nullptr;
  if (d->num_verts < 0 || d->num_tris < 0 || (d->num_tris > 0 && (!d->verts || !d->tris)))
    return record_error(KGPU_ERR_INVALID, "kgpu_geom_create: bad mesh sizes or buffers");
  if (!(d->margin >= 0.0) || !(d->margin < 1e30))
    return record_error(KGPU_ERR_INVALID, "kgpu_geom_create: margin must be finite and non-negative");
  if (d->num_tris >= (1 << 28)) return record_error(KGPU_ERR_UNSUPPORTED, "kgpu_geom_create: too many triangles");
  const int nt = d->num_tris, nv = d->num_verts;
  std::vector<double> tri(9 * (size_t)nt);
  double rmax = 0.0;
  for (int t = 0; t < nt; ++t)
    for (int v = 0; v < 3; ++v) {
      const int vi = d->tris[3 * (size_t)t + v];
      if (vi < 0 || vi >= nv) return record_error(KGPU_ERR_INVALID, "kgpu_geom_create: vertex index out of range");
      double n2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double x = d->verts[3 * (size_t)vi + i];
        if (!std::isfinite(x) || !(std::fabs(x) < 1e6))
          return record_error(KGPU_ERR_NOT_FINITE, "kgpu_geom_create: non-finite or huge vertex coordinate");
        tri[9 * (size_t)t + 3 * v + i] = x;
        n2 += x * x;
      }
      rmax = std::max(rmax, std::sqrt(n2));
    }
  kgpu_geom_s* g = new (std::nothrow) kgpu_geom_s();
  if (!g) return record_error(KGPU_ERR_OOM, "kgpu_geom_create: host allocation");
  g->ntri = nt;
  g->margin = d->margin;
  float r = (float)(rmax * (1.0 + 1e-6));
  if ((double)r < rmax) r = std::nextafter(r, 3.0e38f);
  g->r32 = r;
  std::vector<KNode> nodes;
  std::vector<float> node_r;
  std::vector<float4> t32;
  std::vector<double> t64;
  std::vector<int> orig;
  if (nt > 0) {
    HostBvh hb;
    std::vector<int> ids(nt);
    for (int t = 0; t < nt; ++t) ids[t] = t;
    build_bvh(tri, ids, nullptr, hb);
    nodes = hb.nodes;  // local indices: children / first triangle in leaf order
    for (size_t k = 0; k < hb.nodes.size(); ++k) {
      // sphere about the FP32 centre holding the node's vertices
      double off2 = 0.0;
      const double cf[3] = {hb.nodes[k].a.x, hb.nodes[k].a.y, hb.nodes[k].a.z};
      for (int i = 0; i < 3; ++i) {
        const double dc = hb.node_c64[3 * k + i] - cf[i];
        off2 += dc * dc;
      }
      const double rr = hb.node_r[k] + std::sqrt(off2);
      float f = (float)rr;
      if ((double)f < rr) f = std::nextafter(f, 3.0e38f);
      node_r.push_back(f);
    }
    for (int k = 0; k < nt; ++k) {
      const int t = hb.order[k];
      orig.push_back(t);
      for (int v = 0; v < 3; ++v)
        t32.push_back(make_float4((float)tri[9 * (size_t)t + 3 * v], (float)tri[9 * (size_t)t + 3 * v + 1],
                                  (float)tri[9 * (size_t)t + 3 * v + 2], 0.f));
      for (int i = 0; i < 9; ++i) t64.push_back(tri[9 * (size_t)t + i]);
    }
  }
  cudaError_t e = upload_vec(&g->d_nodes, nodes);
  if (e == cudaSuccess) e = upload_vec(&g->d_node_r, node_r);
  if (e == cudaSuccess) e = upload_vec(&g->d_tri32, t32);
  if (e == cudaSuccess) e = upload_vec(&g->d_tri64, t64);
  if (e == cudaSuccess) e = upload_vec(&g->d_tri_orig, orig);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(g->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    free_geom(g);
    return record_error(e == cudaErrorMemoryAllocation ? KGPU_ERR_OOM : KGPU_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = g;
  return KGPU_OK;
}

extern "C" kgpu_status kgpu_geom_destroy(kgpu_geom g)
{
  if (g) free_geom(g);
  return KGPU_OK;
}

extern "C" kgpu_status kgpu_geom_set_margin(kgpu_geom g, double margin)
{
  if (!g) return record_error(KGPU_ERR_INVALID, "kgpu_geom_set_margin: null geometry");
  if (!(margin >= 0.0) || !(margin < 1e30))
    return record_error(KGPU_ERR_INVALID, "kgpu_geom_set_margin: margin must be finite and non-negative");
  g->margin = margin;
  return KGPU_OK;
}

extern "C" kgpu_status kgpu_geom_get_margin(kgpu_geom g, double* margin)
{
  if (!g || !margin) return record_error(KGPU_ERR_INVALID, "kgpu_geom_get_margin: null argument");
  *margin = g->margin;
  return KGPU_OK;
}

extern "C" kgpu_status kgpu_geom_collide(kgpu_geom a, kgpu_geom b, const double* Ta, const double* Tb, int32_t B,
                                         int32_t flags, double tol, uint8_t* hit, kgpu_stream stream)
{
  kgpu_status st = check_pair(a, b, Ta, Tb, B, flags);
  if (st) return st;
  if (!(tol >= 0.0) || !(tol < 1e30)) return record_error(KGPU_ERR_INVALID, "kgpu_geom_collide: bad tolerance");
  if (B > 0 && !hit) return record_error(KGPU_ERR_INVALID, "kgpu_geom_collide: null output");
  if (B == 0) return KGPU_OK;
  GeomArgs A = {};
  A.Ta = Ta;
  A.Tb = Tb;
  A.sa = (flags & KGPU_GEOM_FIXED_A) ? 0 : 12;
  A.sb = (flags & KGPU_GEOM_FIXED_B) ? 0 : 12;
  A.B = B;
  A.m = kx_add(kx_add(a->margin, tol), b->margin);
  A.bound = 0.0;
  A.hit = hit;
  A.status = a->d_status;
  k_geom<false><<<blocks_for(B), kGW * 32, 0, (cudaStream_t)stream>>>(dev_view(a), dev_view(b), A);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? KGPU_OK : record_error(KGPU_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" kgpu_status kgpu_geom_distance(kgpu_geom a, kgpu_geom b, const double* Ta, const double* Tb, int32_t B,
                                          int32_t flags, double upper_bound, double* d, double* cp, int32_t* elem,
                                          double* dir, kgpu_stream stream)
{
  kgpu_status st = check_pair(a, b, Ta, Tb, B, flags);
  if (st) return st;
  if (std::isnan(upper_bound)) return record_error(KGPU_ERR_INVALID, "kgpu_geom_distance: upper bound is NaN");
  if (a->ntri == 0 || b->ntri == 0)
    return record_error(KGPU_ERR_EMPTY, "kgpu_geom_distance: geometry is empty (robotsim.cpp:1786-1787)");
  if (B > 0 && (!d || !cp || !elem)) return record_error(KGPU_ERR_INVALID, "kgpu_geom_distance: null output");
  if (B == 0) return KGPU_OK;
  GeomArgs A = {};
  A.Ta = Ta;
  A.Tb = Tb;
  A.sa = (flags & KGPU_GEOM_FIXED_A) ? 0 : 12;
  A.sb = (flags & KGPU_GEOM_FIXED_B) ? 0 : 12;
  A.B = B;
  A.msum = kx_add(a->margin, b->margin);
  A.upper = upper_bound;
  // mesh distances are searched below upper + (m_a + m_b); a bound at or
  // below zero finds contacts only when it is exactly 0 after the margins
  A.bound = upper_bound < 1e30 ? std::max(0.0, kx_add(upper_bound, A.msum)) : HUGE_VAL;
  A.d = d;
  A.cp = cp;
  A.elem = elem;
  A.dir = dir;
  A.status = a->d_status;
  k_geom<true><<<blocks_for(B), kGW * 32, 0, (cudaStream_t)stream>>>(dev_view(a), dev_view(b), A);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? KGPU_OK : record_error(KGPU_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" kgpu_status kgpu_geom_sync(kgpu_geom g, kgpu_stream stream)
{
  if (!g) return record_error(KGPU_ERR_INVALID, "kgpu_geom_sync: null geometry");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  int s = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&s, g->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return record_error(KGPU_ERR_CUDA, cudaGetErrorString(e));
  if (s != 0) {
    cudaMemset(g->d_status, 0, sizeof(int));
    return record_error(s, s == KGPU_ERR_NOT_FINITE ? "device status: non-finite or huge (>= 1e6) transform entry"
                                                    : "device status: traversal stack overflow");
  }
  return KGPU_OK;
}
