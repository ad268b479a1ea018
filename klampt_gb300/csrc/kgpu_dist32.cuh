// kgpu_dist32.cuh — FP32 distance helpers shared by the distance kernels
// (kgpu_dist.cu: link-obstacle and link-link distances; kgpu_geom.cu:
// distances between two free geometries).  Values only: the closest
// features and the reported distances always come from the canonical FP64
// arithmetic of include/kgpu_exact.h; these FP32 values prune and select
// candidates, with the error bands their callers add.
#pragma once

#include <cfloat>
#include <climits>

#include "kgpu_device.cuh"

namespace kgpu {

__device__ __forceinline__ float box_dist32(const Box32& A, float3 c, float3 h)
{
  float gx = fmaxf(0.f, fabsf(A.c.x - c.x) - A.h.x - h.x);
  float gy = fmaxf(0.f, fabsf(A.c.y - c.y) - A.h.y - h.y);
  float gz = fmaxf(0.f, fabsf(A.c.z - c.z) - A.h.z - h.z);
  return sqrtf(gx * gx + gy * gy + gz * gz);
}

__device__ __forceinline__ float warp_min(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---- FP32 triangle distance (value only; features come from FP64) --------
// The parameters use the fast reciprocal divide (__fdividef): a parameter off
// by a few ulp moves the evaluated points along their segments by a few ulp of
// the edge length, well inside the 128 u x span band the callers allow for the
// FP32 value (at an interior optimum the error is even second order).
__device__ __forceinline__ float clamp01f(float x) { return fminf(1.f, fmaxf(0.f, x)); }

static __device__ float seg_seg2_32(float3 p1, float3 d1, float3 p2, float3 d2)
{
  const float3 r = sub3(p1, p2);
  const float a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
  float s, t;
  if (a <= 1e-30f && e <= 1e-30f) {
    s = 0.f; t = 0.f;
  } else if (a <= 1e-30f) {
    s = 0.f; t = clamp01f(__fdividef(f, e));
  } else {
    const float c = dot3(d1, r);
    if (e <= 1e-30f) {
      t = 0.f; s = clamp01f(__fdividef(-c, a));
    } else {
      const float b = dot3(d1, d2);
      const float den = a * e - b * b;
      s = den > 0.f ? clamp01f(__fdividef(b * f - c * e, den)) : 0.f;
      t = __fdividef(b * s + f, e);
      if (t < 0.f) { t = 0.f; s = clamp01f(__fdividef(-c, a)); }
      else if (t > 1.f) { t = 1.f; s = clamp01f(__fdividef(b - c, a)); }
    }
  }
  const float3 w = make_float3(r.x + d1.x * s - d2.x * t, r.y + d1.y * s - d2.y * t, r.z + d1.z * s - d2.z * t);
  return dot3(w, w);
}

static __device__ float pt_tri2_32(float3 p, float3 a, float3 b, float3 c)
{
  const float3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
  const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  float3 q;
  if (d1 <= 0.f && d2 <= 0.f) { q = a; goto done; }
  {
    const float3 bp = sub3(p, b);
    const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.f && d4 <= d3) { q = b; goto done; }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
      const float v = __fdividef(d1, d1 - d3);
      q = make_float3(a.x + ab.x * v, a.y + ab.y * v, a.z + ab.z * v);
      goto done;
    }
    const float3 cp = sub3(p, c);
    const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.f && d5 <= d6) { q = c; goto done; }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
      const float w = __fdividef(d2, d2 - d6);
      q = make_float3(a.x + ac.x * w, a.y + ac.y * w, a.z + ac.z * w);
      goto done;
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
      const float w = __fdividef(d4 - d3, (d4 - d3) + (d5 - d6));
      q = make_float3(b.x + (c.x - b.x) * w, b.y + (c.y - b.y) * w, b.z + (c.z - b.z) * w);
      goto done;
    }
    const float den = __fdividef(1.f, va + vb + vc);
    const float v = vb * den, w = vc * den;
    q = make_float3(a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w, a.z + ab.z * v + ac.z * w);
  }
done:
  const float3 dd = sub3(p, q);
  return dot3(dd, dd);
}

// squared distance of two separated triangles: 9 edge-edge + 6 vertex-face
static __device__ float tri_dist2_32(const float3* P, const float3* Q)
{
  float best = FLT_MAX;
#pragma unroll 1
  for (int k = 0; k < 9; ++k) {
    const int i = k / 3, j = k % 3;
    const float3 pa = sel3(i, P[0], P[1], P[2]), pb = sel3(i == 2 ? 0 : i + 1, P[0], P[1], P[2]);
    const float3 qa = sel3(j, Q[0], Q[1], Q[2]), qb = sel3(j == 2 ? 0 : j + 1, Q[0], Q[1], Q[2]);
    best = fminf(best, seg_seg2_32(pa, sub3(pb, pa), qa, sub3(qb, qa)));
  }
#pragma unroll 1
  for (int k = 0; k < 3; ++k) {
    best = fminf(best, pt_tri2_32(sel3(k, P[0], P[1], P[2]), Q[0], Q[1], Q[2]));
    best = fminf(best, pt_tri2_32(sel3(k, Q[0], Q[1], Q[2]), P[0], P[1], P[2]));
  }
  return best;
}

// lexicographic (d2, a, b) minimum across the warp; result in every lane
__device__ __forceinline__ void warp_lexmin(double& d2, int& a, int& b, int& src, int lane)
{
  src = lane;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double od = __shfl_xor_sync(0xffffffffu, d2, o);
    const int oa = __shfl_xor_sync(0xffffffffu, a, o);
    const int ob = __shfl_xor_sync(0xffffffffu, b, o);
    const int os = __shfl_xor_sync(0xffffffffu, src, o);
    const bool take = od < d2 || (od == d2 && (oa < a || (oa == a && (ob < b || (ob == b && os < src)))));
    if (take) { d2 = od; a = oa; b = ob; src = os; }
  }
}

// Lower bound on the distance of two triangles from the separating direction
// through their centroids (projections onto a unit vector are 1-Lipschitz);
// nearly tight for facing triangles, which the box bound is not.  The FP32
// rounding of the centroids, the normalisation and the projections is
// covered by the (1 - 8u) factor and the 16 u span term.
__device__ __forceinline__ float tri_axis_lb32(const float3* P, const float3* Q, float span)
{
  const float k3 = 1.f / 3.f;
  const float3 cP = make_float3((P[0].x + P[1].x + P[2].x) * k3, (P[0].y + P[1].y + P[2].y) * k3,
                                (P[0].z + P[1].z + P[2].z) * k3);
  const float3 cQ = make_float3((Q[0].x + Q[1].x + Q[2].x) * k3, (Q[0].y + Q[1].y + Q[2].y) * k3,
                                (Q[0].z + Q[1].z + Q[2].z) * k3);
  float3 u = sub3(cQ, cP);
  const float nn = sqrtf(dot3(u, u));
  if (!(nn > 1e-20f)) return 0.f;
  const float inv = 1.f / nn;
  u = make_float3(u.x * inv, u.y * inv, u.z * inv);
  float pm = -FLT_MAX, qm = FLT_MAX;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pm = fmaxf(pm, dot3(sub3(P[k], cP), u));
    qm = fminf(qm, dot3(sub3(Q[k], cP), u));
  }
  return (qm - pm) * (1.f - 8.f * kU) - 16.f * kU * span;
}

}  // namespace kgpu
