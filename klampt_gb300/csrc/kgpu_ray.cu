// kgpu_ray.cu — batched ray casting against the environment.
//
// Replaces, per ray, Geometry3D::rayCast / rayCast_ext
// (Python/klampt/src/robotsim.cpp:1821-1852), the environment part of
// WorldModel::RayCast (Cpp/Modeling/World.cpp:465-515) and
// collide.ray_cast (Python/klampt/model/collide.py:219-243): the first
// triangle hit by s + t d, t >= 0, over every object of every group.
//
// Definition (the FP64 oracle's, bit for bit): t = the smallest parameter at
// which the canonical FP64 ray/triangle test (kx_ray_tri) reports a hit, ties
// to the smaller object, then triangle; the hit point is s + t d in canonical
// FP64.
//
// GPU method, one thread per ray: the environment tree is traversed in FP32
// with conservative slab tests (boxes widened by the environment's FP32
// error bound and the tests' rounding), nearer child first; every triangle of
// a reached leaf goes through an FP32 filter whose four triple products
// (det, and the barycentric and distance numerators) carry rigorous error
// bounds, so it rejects only triangles the FP64 test cannot accept or whose
// hit lies beyond the best one found; the rest are decided in FP64.
#include <math_constants.h>

#include <cfloat>
#include <climits>

#include "kgpu_device.cuh"

namespace kgpu {

namespace {

constexpr int kRayStack = 64;

// Error bound of the FP32 triple product x . (y x z) computed from
// approximations of x, y, z off by at most ex, ey, ez (Euclidean) with norms
// at most nx, ny, nz: perturbation (all cross terms) plus the rounding of the
// cross and dot products (<= 8u of the product of the norms; 10u here also
// covers the FP64 side's own rounding).
__device__ __forceinline__ float tp_err(float nx, float ny, float nz, float ex, float ey, float ez)
{
  const float X = nx + ex, Y = ny + ey, Z = nz + ez;
  return (X * Y * Z - nx * ny * nz + 10.f * kU * X * Y * Z) * 1.0001f + 1e-30f;
}

__device__ __forceinline__ float norm3(float3 a) { return sqrtf(dot3(a, a)) * 1.0001f; }

// Conservative slab test: can the ray meet the box (centre c, half h, widened
// by pad) at some t in [0, tmax]?
__device__ __forceinline__ bool ray_box(const float3 S, const float3 inv, const float3 D, float4 c, float4 h,
                                        float pad, float tmax, float* tnear)
{
  float tn = 0.f, tf = tmax;
  const float sv[3] = {S.x, S.y, S.z}, iv[3] = {inv.x, inv.y, inv.z}, dv[3] = {D.x, D.y, D.z};
  const float cv[3] = {c.x, c.y, c.z}, hv[3] = {h.x, h.y, h.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float p = pad + 2.f * kU * (fabsf(cv[i]) + hv[i]);
    const float lo = cv[i] - hv[i] - p, hi = cv[i] + hv[i] + p;
    if (fabsf(dv[i]) < 1e-30f) {
      // (nearly) parallel to the slab: outside it, the ray reaches it only
      // at an enormous t — no constraint is taken from this axis then
      continue;
    }
    float a = (lo - sv[i]) * iv[i], b = (hi - sv[i]) * iv[i];
    if (a > b) { const float x = a; a = b; b = x; }
    // (lo - s) and 1/d each round once, the product once: <= 3u relative
    a -= 4.f * kU * fabsf(a) + 1e-30f;
    b += 4.f * kU * fabsf(b) + 1e-30f;
    tn = fmaxf(tn, a);
    tf = fminf(tf, b);
  }
  *tnear = tn;
  return tn <= tf;
}

__global__ void __launch_bounds__(256) k_ray(const KWorldDev* __restrict__ W, const float* __restrict__ s,
                                             const float* __restrict__ d, int R, int* obj, int* tri,
                                             double* tout, double* point)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const float3 S = make_float3(s[3 * (size_t)r], s[3 * (size_t)r + 1], s[3 * (size_t)r + 2]);
  const float3 D = make_float3(d[3 * (size_t)r], d[3 * (size_t)r + 1], d[3 * (size_t)r + 2]);
  obj[r] = -1;
  tri[r] = -1;
  tout[r] = CUDART_INF;
  point[3 * (size_t)r] = point[3 * (size_t)r + 1] = point[3 * (size_t)r + 2] = 0.0;
  if (!(fabsf(S.x) < 1e18f && fabsf(S.y) < 1e18f && fabsf(S.z) < 1e18f && fabsf(D.x) < 1e18f &&
        fabsf(D.y) < 1e18f && fabsf(D.z) < 1e18f)) {
    set_status(W->status, KGPU_ERR_NOT_FINITE);
    return;
  }
  if (D.x == 0.f && D.y == 0.f && D.z == 0.f) return;  // no direction: meets nothing (det = 0)
  const double S64[3] = {S.x, S.y, S.z}, D64[3] = {D.x, D.y, D.z};
  const float3 inv = make_float3(1.f / D.x, 1.f / D.y, 1.f / D.z);
  const float nD = norm3(D);
  const float de = W->eps_env + W->eps_extra;  // bound on |FP32 vertex - FP64 vertex|
  double best = CUDART_INF;
  float bestf = FLT_MAX;  // >= best
  int bleaf = -1, borig = INT_MAX;

  uint32_t stack[kRayStack];
  int top = 0;
#pragma unroll 1
  for (int g = 0; g < kMaxGroups; ++g)
    if (W->group_root[g] >= 0 && top < kRayStack) stack[top++] = (uint32_t)W->group_root[g];

#pragma unroll 1
  while (top > 0) {
    const int node = (int)stack[--top];
    const float4 na = __ldg(&W->enodes[node].a), nb = __ldg(&W->enodes[node].b);
    float tn;
    if (!ray_box(S, inv, D, na, nb, de, bestf, &tn)) continue;
    const int cnt = f2i(nb.w), idx = f2i(na.w);
    if (cnt == 0) {
      if (top + 2 > kRayStack) {
        set_status(W->status, KGPU_ERR_OVERFLOW);
        return;
      }
      // nearer child on top
      const float4 la = __ldg(&W->enodes[idx].a), lb = __ldg(&W->enodes[idx].b);
      const float4 ra = __ldg(&W->enodes[idx + 1].a), rb = __ldg(&W->enodes[idx + 1].b);
      float tl, tr;
      const bool hl = ray_box(S, inv, D, la, lb, de, bestf, &tl);
      const bool hr = ray_box(S, inv, D, ra, rb, de, bestf, &tr);
      if (hl && hr) {
        const bool lfirst = tl <= tr;
        stack[top++] = (uint32_t)(lfirst ? idx + 1 : idx);
        stack[top++] = (uint32_t)(lfirst ? idx : idx + 1);
      } else if (hl) {
        stack[top++] = (uint32_t)idx;
      } else if (hr) {
        stack[top++] = (uint32_t)(idx + 1);
      }
      continue;
    }
    // leaf: FP32 filter, FP64 decision
#pragma unroll 1
    for (int k = idx; k < idx + cnt; ++k) {
      const float4 p0 = __ldg(W->etri32 + 3 * (size_t)k), p1 = __ldg(W->etri32 + 3 * (size_t)k + 1),
                   p2 = __ldg(W->etri32 + 3 * (size_t)k + 2);
      const float3 P0 = make_float3(p0.x, p0.y, p0.z);
      const float3 e1 = sub3(make_float3(p1.x, p1.y, p1.z), P0), e2 = sub3(make_float3(p2.x, p2.y, p2.z), P0);
      const float3 w = sub3(S, P0);
      const float3 p = cross3(D, e2), q = cross3(w, e1);
      const float det = dot3(e1, p), U = dot3(w, p), V = dot3(D, q), Tn = dot3(e2, q);
      const float n1 = norm3(e1), n2 = norm3(e2), nw = norm3(w);
      const float x1 = 2.f * de + 2.f * kU * n1, x2 = 2.f * de + 2.f * kU * n2, xw = de + 2.f * kU * nw;
      const float eDet = tp_err(n1, nD, n2, x1, 0.f, x2);
      bool cand = true;
      if (fabsf(det) > eDet) {
        const float sg = det > 0.f ? 1.f : -1.f;
        const float eU = tp_err(nw, nD, n2, xw, 0.f, x2), eV = tp_err(nD, nw, n1, 0.f, xw, x1),
                    eT = tp_err(n2, nw, n1, x2, xw, x1);
        const float Us = sg * U, Vs = sg * V, Ts = sg * Tn, ad = fabsf(det);
        if (Us < -eU || Vs < -eV || Ts < -eT ||
            (Us + Vs) - ad > eU + eV + eDet + 2.f * kU * (fabsf(U) + fabsf(V) + ad))
          cand = false;
        else if (Ts - eT > 0.f && (Ts - eT) / (ad + eDet) * (1.f - 4.f * kU) > bestf)
          cand = false;  // certainly beyond the best hit
      }
      if (!cand) continue;
      double t;
      if (kx_ray_tri(S64, D64, W->etri64 + 9 * (size_t)k, &t)) {
        const int orig = __ldg(W->etri_orig + k);
        if (t < best || (t == best && orig < borig)) {
          best = t;
          borig = orig;
          bleaf = k;
          const float bf = (float)t;
          bestf = (double)bf < t ? nextafterf(bf, FLT_MAX) : bf;
        }
      }
    }
  }
  if (bleaf >= 0) {
    const int o = __ldg(W->etri_obj + bleaf);
    obj[r] = o;
    tri[r] = borig - __ldg(W->obj_tri_first + o);
    tout[r] = best;
    for (int i = 0; i < 3; ++i) point[3 * (size_t)r + i] = kx_add(S64[i], kx_mul(best, D64[i]));
  }
}

}  // namespace

cudaError_t launch_raycast(const KWorldDev* Wd, const float* s, const float* d, int R, int* obj, int* tri,
                           double* t, double* point, cudaStream_t st)
{
  if (R <= 0) return cudaSuccess;
  const int threads = 256;
  k_ray<<<(R + threads - 1) / threads, threads, 0, st>>>(Wd, s, d, R, obj, tri, t, point);
  return cudaGetLastError();
}

}  // namespace kgpu
