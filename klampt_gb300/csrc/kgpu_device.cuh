// kgpu_device.cuh — device helpers shared by the engine kernels.
//
// FP32 side: forward kinematics, link-node boxes in world frame, and a
// conservative triangle/triangle separating-axis filter.  "Conservative"
// means: when the filter reports separation, the canonical FP64 triangles
// (include/kgpu_exact.h, evaluated on the FP64 forward kinematics) are
// separated too.  Every FP32 comparison therefore carries an inflation that
// bounds the difference between FP32 and FP64 world coordinates — computed
// per configuration and per link by a running error analysis of the FP32
// forward kinematics (warp_fk32) — plus the FP32 rounding of the test
// itself.  Pairs the filter cannot separate form the "band": an FP32
// intersection certificate or the FP64 re-test decides them, so verdicts
// equal the FP64 ones bit for bit.
#pragma once

#include "../../include/kgpu_exact.h"
#include "kgpu_internal.h"

namespace kgpu {

__device__ __forceinline__ int f2i(float f) { return __float_as_int(f); }

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---- FP32 rigid transforms (R row-major, then t) -------------------------
__device__ __forceinline__ void compose32(const float* A, const float* B, float* o)
{
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      o[3 * r + c] = fmaf(A[3 * r + 0], B[c], fmaf(A[3 * r + 1], B[3 + c], A[3 * r + 2] * B[6 + c]));
    o[9 + r] = fmaf(A[3 * r + 0], B[9], fmaf(A[3 * r + 1], B[10], fmaf(A[3 * r + 2], B[11], A[9 + r])));
  }
}

__device__ __forceinline__ float3 xform32(const float* T, float3 v)
{
  return make_float3(fmaf(T[0], v.x, fmaf(T[1], v.y, fmaf(T[2], v.z, T[9]))),
                     fmaf(T[3], v.x, fmaf(T[4], v.y, fmaf(T[5], v.z, T[10]))),
                     fmaf(T[6], v.x, fmaf(T[7], v.y, fmaf(T[8], v.z, T[11]))));
}

constexpr float kU = 5.9604645e-08f;  // unit roundoff of FP32, 2^-24

// sin and cos in FP32 with a known error bound: Cody–Waite reduction modulo
// pi/2 with a three-part split (pi/2 = C1 + C2 + C3, C1 and C2 of 12
// significant bits, so k*C1 and k*C2 are exact for |x| < 4096; larger
// arguments reduce in FP64), then the Taylor series of sin to r^9 and cos to
// r^10 on |r| <= pi/4 (truncation < 2e-9).  |error| <= kSinCosErr.
constexpr float kSinCosErr = 4.0f * kU;
// argument reduction for |x| >= 4096 in FP64 (out of line: never on the hot
// path, and its code would otherwise sit inside every caller's loop)
static __device__ __noinline__ float2 sincos32_reduce_big(float x)
{
  const double kd = rint((double)x * 0.6366197723675814);
  const float r = (float)(((double)x - kd * 1.5707963267948966) - kd * 6.123233995736766e-17);
  return make_float2(r, (float)fmod(kd, 4.0));
}

__device__ __forceinline__ void sincos32(float x, float* s, float* c)
{
  float k, r;
  if (fabsf(x) < 4096.f) {
    k = rintf(x * 0.63661975f);
    r = fmaf(-k, -8.705516e-10f, fmaf(-k, -4.4535846e-06f, fmaf(-k, 1.57080078125f, x)));
  } else {
    const float2 rk = sincos32_reduce_big(x);
    r = rk.x;
    k = rk.y;
  }
  float r2 = r * r;
  float ps = fmaf(fmaf(fmaf(fmaf(2.7557319e-06f, r2, -1.98412698e-04f), r2, 8.33333333e-03f), r2,
                       -1.66666667e-01f), r2 * r, r);
  float pc = fmaf(fmaf(fmaf(fmaf(fmaf(-2.75573192e-07f, r2, 2.48015873e-05f), r2, -1.38888889e-03f), r2,
                            4.16666667e-02f), r2, -0.5f), r2, 1.0f);
  int q = ((int)k) & 3;
  float sn = (q & 1) ? pc : ps, cs = (q & 1) ? ps : pc;
  *s = (q & 2) ? -sn : sn;
  *c = ((q + 1) & 2) ? -cs : cs;
}

__device__ __forceinline__ float tnorm(const float* T)
{
  return sqrtf(T[9] * T[9] + T[10] * T[10] + T[11] * T[11]) * 1.0001f;
}

// Running error bound of an FP32 rigid transform T~ against the exact
// transform T of the same configuration computed in FP64:
//   rho >= ||R~ - R||_2   and   tau >= |t~ - t|_2.
// Composition C = A * B (FP32 with FMA) propagates as
//   rho_C = rho_A (1 + rho_B) + rho_B + 6u (1 + rho_A)(1 + rho_B)
//   tau_C = rho_A |t_B| + tau_B + tau_A + 3u (sqrt3 (1 + rho_A)|t_B| + |t_A|)
// (first-order terms from the operands, the second from FMA rounding of the
// 3-term dot products, bounded with Cauchy-Schwarz on rows of norm <= 1+rho).
__device__ __forceinline__ void compose_err(float rA, float tA, float nA, float rB, float tB, float nB,
                                            float* r, float* t)
{
  *r = (rA * (1.f + rB) + rB + 6.f * kU * (1.f + rA) * (1.f + rB)) * 1.0001f;
  *t = (rA * nB + tB + tA + 3.f * kU * (1.7320509f * (1.f + rA) * nB + nA)) * 1.0001f;
}

// local transform T0_Parent * J(q) of link i in FP32 and its error bound.
// e_q bounds |q_fp32 - q_exact|.  For a revolute joint
//   ||R_J(q~) - R_J(q)|| <= |dq| ;  sin/cos errors: <= 2 kSinCosErr
//   (R = cI + s[w]x + (1-c)ww^T);  entry rounding and axis rounding <= 12u.
// T0_Parent rounded to FP32: rho <= u, tau <= u/2 |t0|.
__device__ __forceinline__ void joint_local32(const KRobotDev& R, int i, float q, float e_q, float* L,
                                              float* rho, float* tau)
{
  const float* T0 = R.T0P[i];
  int jt = R.jtype[i];
  const float r0 = kU, t0 = 0.5f * kU * tnorm(T0);
  if (jt == KX_JOINT_REVOLUTE) {
    float s, c;
    sincos32(q, &s, &c);
    float wx = R.axis[i][0], wy = R.axis[i][1], wz = R.axis[i][2];
    float v = 1.f - c;
    float J[12];
    J[0] = c + wx * wx * v;  J[1] = wx * wy * v - wz * s; J[2] = wx * wz * v + wy * s;
    J[3] = wy * wx * v + wz * s; J[4] = c + wy * wy * v;  J[5] = wy * wz * v - wx * s;
    J[6] = wz * wx * v - wy * s; J[7] = wz * wy * v + wx * s; J[8] = c + wz * wz * v;
    J[9] = 0.f; J[10] = 0.f; J[11] = 0.f;
    compose32(T0, J, L);
    const float rJ = e_q + 2.f * kSinCosErr + 12.f * kU;
    compose_err(r0, t0, tnorm(T0), rJ, 0.f, 0.f, rho, tau);
  } else if (jt == KX_JOINT_PRISMATIC) {
    float J[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    J[9] = R.axis[i][0] * q; J[10] = R.axis[i][1] * q; J[11] = R.axis[i][2] * q;
    compose32(T0, J, L);
    const float tJ = (e_q + 2.f * kU * fabsf(q)) * 1.0001f;
    compose_err(r0, t0, tnorm(T0), 0.f, tJ, tnorm(J), rho, tau);
  } else {
#pragma unroll
    for (int k = 0; k < 12; ++k) L[k] = T0[k];
    *rho = r0;
    *tau = t0;
  }
}

// Warp-cooperative forward kinematics: lane i < nlinks owns link i.  Local
// transforms are formed in parallel and chained to the root by pointer
// jumping (ceil(log2(depth)) rounds of shuffles), which handles serial
// chains and trees alike.  Result: world transform of link `lane` in P and
// delta, a bound on |v_world_fp32 - v_world_exact| for every vertex of the
// link and for every point of its FP32 node boxes:
//   delta = rho r + tau + u (12 r + 6 |t|),
// r the largest vertex norm of the link in its own frame (the u-term covers
// the FP32 rounding of the vertex and box transforms).
//
// warp_fk32_group runs G = 32 / L independent configurations at once: lanes
// [g L, g L + L) hold configuration g, lane g L + i link i (active when
// `valid`); warp_fk32 is the single-configuration case (L = 32).
__device__ __forceinline__ void warp_fk32_group(const KRobotDev& R, int lane, int L, bool valid, float q,
                                                float e_q, float* P, float* delta)
{
  const int link = lane & (L - 1), gbase = lane & ~(L - 1);
  int anc = -1;
  float rho = 0.f, tau = 0.f;
  if (valid) {
    joint_local32(R, link, q, e_q, P, &rho, &tau);
    anc = R.parents[link] >= 0 ? gbase + R.parents[link] : -1;
  } else {
#pragma unroll
    for (int k = 0; k < 12; ++k) P[k] = 0.f;
  }
  while (__any_sync(0xffffffffu, anc >= 0)) {
    int src = anc >= 0 ? anc : lane;
    float Pa[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) Pa[k] = __shfl_sync(0xffffffffu, P[k], src);
    const int anc2 = __shfl_sync(0xffffffffu, anc, src);
    const float ra = __shfl_sync(0xffffffffu, rho, src);
    const float ta = __shfl_sync(0xffffffffu, tau, src);
    if (anc >= 0) {
      float o[12];
      compose32(Pa, P, o);
      float r2, t2;
      compose_err(ra, ta, tnorm(Pa), rho, tau, tnorm(P), &r2, &t2);
      rho = r2;
      tau = t2;
#pragma unroll
      for (int k = 0; k < 12; ++k) P[k] = o[k];
      anc = anc2;
    }
  }
  const float rl = valid ? R.link_r[link] : 0.f;
  *delta = (rho * rl + tau + kU * (12.f * rl + 6.f * tnorm(P))) * 1.001f + 1e-9f;
}

__device__ __forceinline__ void warp_fk32(const KRobotDev& R, int lane, float q, float e_q, float* P,
                                          float* delta)
{
  warp_fk32_group(R, lane, 32, lane < R.nlinks, q, e_q, P, delta);
}

// ---- boxes -------------------------------------------------------------
// max |R^T R - I| over the entries for the rotation rows P[0..8] of an FP32
// transform, plus 8 u for the rounding of the Gram products
__device__ __forceinline__ float rot_gram_err32(const float* P)
{
  float g = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      const float v = P[i] * P[j] + P[3 + i] * P[3 + j] + P[6 + i] * P[6 + j];
      g = fmaxf(g, fabsf(i == j ? v - 1.f : v));
    }
  return g + 8.f * kU;
}

struct Box32 {
  float3 c, h;
};

__device__ __forceinline__ Box32 xform_box(const float* T, float4 a, float4 b)
{
  Box32 o;
  o.c = xform32(T, make_float3(a.x, a.y, a.z));
  o.h = make_float3(fabsf(T[0]) * b.x + fabsf(T[1]) * b.y + fabsf(T[2]) * b.z,
                    fabsf(T[3]) * b.x + fabsf(T[4]) * b.y + fabsf(T[5]) * b.z,
                    fabsf(T[6]) * b.x + fabsf(T[7]) * b.y + fabsf(T[8]) * b.z);
  return o;
}

__device__ __forceinline__ bool boxes_overlap(const Box32& A, const Box32& B, float eps)
{
  return fabsf(A.c.x - B.c.x) <= A.h.x + B.h.x + eps &&
         fabsf(A.c.y - B.c.y) <= A.h.y + B.h.y + eps &&
         fabsf(A.c.z - B.c.z) <= A.h.z + B.h.z + eps;
}

// ---- FP32 triangle filter ------------------------------------------------
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float l1(float3 a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }

// true if axis a separates p and q by more than the tolerance
__device__ __forceinline__ bool sep_axis32(float3 a, const float3* p, const float3* q, float eps,
                                           float margin)
{
  float p0 = dot3(a, p[0]), p1 = dot3(a, p[1]), p2 = dot3(a, p[2]);
  float q0 = dot3(a, q[0]), q1 = dot3(a, q[1]), q2 = dot3(a, q[2]);
  float pmin = fminf(p0, fminf(p1, p2)), pmax = fmaxf(p0, fmaxf(p1, p2));
  float qmin = fminf(q0, fminf(q1, q2)), qmax = fmaxf(q0, fmaxf(q1, q2));
  float gap = fmaxf(qmin - pmax, pmin - qmax);
  float tol = l1(a) * eps;
  if (margin > 0.f) tol += margin * sqrtf(dot3(a, a));
  return gap > tol;
}

__device__ __forceinline__ float3 sel3(int i, float3 a, float3 b, float3 c)
{
  return i == 0 ? a : (i == 1 ? b : c);
}

// Conservative separation of world-frame triangles P and Q (FP32): box
// pre-test, the two face normals, then the 9 edge-edge and 6 in-plane axes in
// a rolled loop (small code keeps the hot loop in the instruction cache).
// eps = delta_P + delta_Q (vertex error bounds of the two triangles); the
// FP32 rounding of the projections adds 8u x span (span bounds every
// coordinate relative to P's first vertex).
__device__ __forceinline__ bool tri_separated32(const float3* P, const float3* Q, float eps,
                                                float margin)
{
  const float3 pmn = make_float3(fminf(P[0].x, fminf(P[1].x, P[2].x)), fminf(P[0].y, fminf(P[1].y, P[2].y)),
                                 fminf(P[0].z, fminf(P[1].z, P[2].z)));
  const float3 pmx = make_float3(fmaxf(P[0].x, fmaxf(P[1].x, P[2].x)), fmaxf(P[0].y, fmaxf(P[1].y, P[2].y)),
                                 fmaxf(P[0].z, fmaxf(P[1].z, P[2].z)));
  const float3 qmn = make_float3(fminf(Q[0].x, fminf(Q[1].x, Q[2].x)), fminf(Q[0].y, fminf(Q[1].y, Q[2].y)),
                                 fminf(Q[0].z, fminf(Q[1].z, Q[2].z)));
  const float3 qmx = make_float3(fmaxf(Q[0].x, fmaxf(Q[1].x, Q[2].x)), fmaxf(Q[0].y, fmaxf(Q[1].y, Q[2].y)),
                                 fmaxf(Q[0].z, fmaxf(Q[1].z, Q[2].z)));
  const float bt = eps + margin;
  if (qmn.x - pmx.x > bt || pmn.x - qmx.x > bt || qmn.y - pmx.y > bt || pmn.y - qmx.y > bt ||
      qmn.z - pmx.z > bt || pmn.z - qmx.z > bt)
    return true;
  const float span = fmaxf(fmaxf(fmaxf(pmx.x, qmx.x) - fminf(pmn.x, qmn.x), fmaxf(pmx.y, qmx.y) - fminf(pmn.y, qmn.y)),
                           fmaxf(pmx.z, qmx.z) - fminf(pmn.z, qmn.z));
  eps += 8.f * kU * span;
  float3 p[3], q[3];
  p[0] = make_float3(0.f, 0.f, 0.f);
  p[1] = sub3(P[1], P[0]);
  p[2] = sub3(P[2], P[0]);
  q[0] = sub3(Q[0], P[0]);
  q[1] = sub3(Q[1], P[0]);
  q[2] = sub3(Q[2], P[0]);
  const float3 ep0 = p[1], ep1 = sub3(p[2], p[1]), ep2 = make_float3(-p[2].x, -p[2].y, -p[2].z);
  const float3 eq0 = sub3(q[1], q[0]), eq1 = sub3(q[2], q[1]), eq2 = sub3(q[0], q[2]);
  const float3 np = cross3(ep0, ep1);
  const float3 nq = cross3(eq0, eq1);
  // one rolled loop over the 17 axes: the two face normals first (the most
  // frequent separators), then edge x edge, then the in-plane axes
#pragma unroll 1
  for (int k = 0; k < 17; ++k) {
    float3 a;
    if (k < 2) a = k == 0 ? np : nq;
    else if (k < 11) a = cross3(sel3((k - 2) / 3, ep0, ep1, ep2), sel3((k - 2) % 3, eq0, eq1, eq2));
    else if (k < 14) a = cross3(np, sel3(k - 11, ep0, ep1, ep2));
    else a = cross3(nq, sel3(k - 14, eq0, eq1, eq2));
    if (sep_axis32(a, p, q, eps, margin)) return true;
  }
  return false;
}

// Sign of orient3d(a,b,c,d) = det[a-d, b-d, c-d] that holds for every
// placement of the four points within `delta` (Euclidean) of the given ones,
// or 0 when the sign is not certain.  With columns u, v, w each moved by at
// most 2 delta:  |det change| <= 2d(|v||w| + |u||w| + |u||v|)
// + 4d^2(|u|+|v|+|w|) + 8d^3, plus FP32 rounding <= 12 u |u||v||w|.
__device__ __forceinline__ int orient_sign32(float3 a, float3 b, float3 c, float3 d, float delta)
{
  float3 u = sub3(a, d), v = sub3(b, d), w = sub3(c, d);
  float det = dot3(u, cross3(v, w));
  float nu = sqrtf(dot3(u, u)), nv = sqrtf(dot3(v, v)), nw = sqrtf(dot3(w, w));
  float B = 2.f * delta * (nv * nw + nu * nw + nu * nv) + 4.f * delta * delta * (nu + nv + nw) +
            8.f * delta * delta * delta + 12.f * 5.9604645e-08f * nu * nv * nw;
  B *= 1.01f;
  return det > B ? 1 : (det < -B ? -1 : 0);
}

// Certain intersection of world-frame triangles P and Q despite vertex
// errors of up to `delta` per vertex: an edge of one triangle crosses the
// other's interior — its endpoints lie on opposite sides of the other
// triangle's plane and the three edge-edge orientations agree in sign — with
// every sign certain (orient_sign32).  A "true" therefore holds for the exact
// FP64 triangles too, and the canonical FP64 test reports the same contact.
// Pairs it cannot certify go to the FP64 re-test.  Called for band pairs
// only, so it is kept out of line.
static __device__ __noinline__ bool tri_certain_hit32(float3 P0, float3 P1, float3 P2, float3 Q0, float3 Q1,
                                                      float3 Q2, float delta)
{
  int sq = 0, sp = 0;  // 2 bits per vertex: 1 = +, 2 = -, 0 = unsure
#pragma unroll 1
  for (int k = 0; k < 3; ++k) {
    int a = orient_sign32(Q0, Q1, Q2, sel3(k, P0, P1, P2), delta);
    int b = orient_sign32(P0, P1, P2, sel3(k, Q0, Q1, Q2), delta);
    sq |= (a > 0 ? 1 : (a < 0 ? 2 : 0)) << (2 * k);
    sp |= (b > 0 ? 1 : (b < 0 ? 2 : 0)) << (2 * k);
  }
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    int i1 = i == 2 ? 0 : i + 1;
    int a0 = (sq >> (2 * i)) & 3, a1 = (sq >> (2 * i1)) & 3;
    int b0 = (sp >> (2 * i)) & 3, b1 = (sp >> (2 * i1)) & 3;
    // edge i of P through the interior of Q
    if (a0 && a1 && a0 != a1) {
      float3 pa = sel3(i, P0, P1, P2), pb = sel3(i1, P0, P1, P2);
      int e0 = orient_sign32(pa, pb, Q0, Q1, delta);
      if (e0 != 0 && orient_sign32(pa, pb, Q1, Q2, delta) == e0 && orient_sign32(pa, pb, Q2, Q0, delta) == e0)
        return true;
    }
    // edge i of Q through the interior of P
    if (b0 && b1 && b0 != b1) {
      float3 qa = sel3(i, Q0, Q1, Q2), qb = sel3(i1, Q0, Q1, Q2);
      int e0 = orient_sign32(P0, P1, qa, qb, delta);
      if (e0 != 0 && orient_sign32(P1, P2, qa, qb, delta) == e0 && orient_sign32(P2, P0, qa, qb, delta) == e0)
        return true;
    }
  }
  return false;
}

// ---- FP64 side (canonical arithmetic) ------------------------------------
// World transform of link l at q64 by the sequential chain root -> l, the
// same operation sequence as the oracle's forward kinematics.
__device__ __forceinline__ void chain64(const KRobotDev& R, const double* q64, int l, double* T)
{
  int path[kMaxLinks];
  int n = 0;
  for (int j = l; j >= 0; j = R.parents[j]) path[n++] = j;
  double A[12], Lc[12];
  int j = path[n - 1];
  kx_joint_local(R.T0P64[j], R.axis64[j], R.jtype[j], q64[j], A);
  for (int k = n - 2; k >= 0; --k) {
    j = path[k];
    kx_joint_local(R.T0P64[j], R.axis64[j], R.jtype[j], q64[j], Lc);
    kx_compose(A, Lc, T);
#pragma unroll
    for (int i = 0; i < 12; ++i) A[i] = T[i];
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) T[i] = A[i];
}

// Warp-cooperative FP64 forward kinematics into T64[link][12]: the local
// transforms are formed in parallel (lane i, link i), then composed by lane 0
// in link order exactly as the oracle does (T[i] = T[parent] * L_i), so the
// result is bit-identical to the sequential chain.
static __device__ __noinline__ void warp_fk64(const KRobotDev& R, const double* q64, double (*T64)[12],
                                              int lane)
{
  int nl = R.nlinks;
  if (lane < nl) kx_joint_local(R.T0P64[lane], R.axis64[lane], R.jtype[lane], q64[lane], T64[lane]);
  __syncwarp();
  if (lane == 0) {
    for (int i = 0; i < nl; ++i) {
      int p = R.parents[i];
      if (p < 0) continue;
      double o[12];
      kx_compose(T64[p], T64[i], o);
      for (int k = 0; k < 12; ++k) T64[i][k] = o[k];
    }
  }
  __syncwarp();
}

// FP64 re-test of one band pair: link triangle tA of link la against link
// triangle tB of link tgt (tgt < 32) or environment triangle tB, with the
// link transforms T64 of the configuration.  Returns 1 if the canonical
// predicate reports collision.
static __device__ __noinline__ int band_retest(const KWorldDev* __restrict__ W, const KRobotDev& R,
                                               const double (*T64)[12], int la, int tA, int tgt, int tB)
{
  double P[9], Q[9];
  const double* pa = W->ltri64 + 9 * (size_t)tA;
  for (int v = 0; v < 3; ++v) kx_xform_point(T64[la], pa + 3 * v, P + 3 * v);
  double m = R.link_margin64[la];
  if (tgt < 32) {
    const double* pb = W->ltri64 + 9 * (size_t)tB;
    for (int v = 0; v < 3; ++v) kx_xform_point(T64[tgt], pb + 3 * v, Q + 3 * v);
    m = kx_add(m, R.link_margin64[tgt]);
  } else {
    const double* pb = W->etri64 + 9 * (size_t)tB;
    for (int i = 0; i < 9; ++i) Q[i] = pb[i];
    m = kx_add(m, W->obj_margin64[W->etri_obj[tB]]);
  }
  if (m == 0.0) return kx_tri_tri_overlap(P, Q);
  double cp[3], cq[3];
  return kx_tri_tri_dist2(P, Q, cp, cq) <= kx_mul(m, m);
}

__device__ __forceinline__ void set_status(int* status, int code) { atomicCAS(status, 0, code); }

}  // namespace kgpu
