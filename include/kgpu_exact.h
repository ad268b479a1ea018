/*
 * kgpu_exact.h — the canonical FP64 arithmetic of the configuration-validity
 * and proximity path.
 *
 * Collision verdicts must be identical between the GPU engine and the FP64
 * CPU oracle, bit for bit.  Klamp't computes them in double precision
 * (KrisLibrary `Real` = double) through RobotKinematics3D::UpdateFrames
 * (called from Cpp/Modeling/Robot.cpp:981 and Python/klampt/src/robotsim.cpp:5318)
 * and PQP's triangle tests.  To make "identical" checkable, every FP64 value
 * that decides a verdict or a reported distance is defined here ONCE, as a
 * fixed sequence of IEEE-754 round-to-nearest operations with no fused
 * multiply-add:
 *   - on the device, each operation is an explicit __dadd_rn/__dmul_rn/...
 *     intrinsic (never contracted into an FMA by nvcc);
 *   - on the host, translation units that include this header are compiled
 *     with -ffp-contract=off (and never with -ffast-math).
 * Division and square root are IEEE correctly rounded on both sides, so the
 * same inputs give the same bits on an x86 host, an Arm host and sm_103a.
 *
 * Contents
 *   kx_sincos          sin/cos by Cody–Waite reduction modulo pi/2 (three-part
 *                      split of pi/2, derived at 300-bit precision) followed by
 *                      the Taylor series of sin and cos on |r| <= pi/4
 *                      (truncation error < 1e-19).  Library sin/cos are not
 *                      used because glibc and CUDA round differently.
 *   kx_joint_local     T0_Parent * J(q): revolute = rotation about axis w by q
 *                      (Rodrigues), prismatic = translation by w*q, weld = I
 *                      (Cpp/docs/Manual-Modeling.md:94,115; Robot.cpp:961-965).
 *   kx_compose         rigid-transform product.
 *   kx_xform_point     R*v + t.
 *   kx_tri_tri_overlap closed-triangle intersection by the separating-axis
 *                      theorem on 17 candidate axes (2 normals, 9 edge-edge
 *                      crosses, 6 in-plane edge normals); touching counts as
 *                      intersecting.
 *   kx_tri_tri_dist2   squared distance between two triangles with the
 *                      closest points (9 segment-segment + 6 point-triangle
 *                      candidates; 0 when they intersect).
 *   kx_ray_tri         ray s + t d (t >= 0) against a closed triangle by the
 *                      triple-product form of Moller-Trumbore (divisions
 *                      deferred to the one for t); a ray in the triangle's
 *                      plane (determinant exactly 0) does not hit.
 *
 * Rigid transforms are 12 doubles: R row-major (R[3*r+c]) followed by t.
 */
#ifndef KGPU_EXACT_H
#define KGPU_EXACT_H

#include <math.h>

#if defined(__CUDACC__)
#define KX_HD __host__ __device__ __forceinline__
#else
#define KX_HD static inline
#endif

/* ---- unfused IEEE operations ------------------------------------------ */
#if defined(__CUDA_ARCH__)
KX_HD double kx_add(double a, double b) { return __dadd_rn(a, b); }
KX_HD double kx_sub(double a, double b) { return __dsub_rn(a, b); }
KX_HD double kx_mul(double a, double b) { return __dmul_rn(a, b); }
KX_HD double kx_div(double a, double b) { return __ddiv_rn(a, b); }
KX_HD double kx_sqrt(double a) { return __dsqrt_rn(a); }
#else
KX_HD double kx_add(double a, double b) { return a + b; }
KX_HD double kx_sub(double a, double b) { return a - b; }
KX_HD double kx_mul(double a, double b) { return a * b; }
KX_HD double kx_div(double a, double b) { return a / b; }
KX_HD double kx_sqrt(double a) { return sqrt(a); }
#endif
KX_HD double kx_rint(double a) { return rint(a); }
KX_HD double kx_abs(double a) { return fabs(a); }

/* ---- sin / cos ---------------------------------------------------------- */
/* pi/2 = KX_PIO2_1 + KX_PIO2_2 + KX_PIO2_3; the first two have 33 significant
 * bits so k*KX_PIO2_1 and k*KX_PIO2_2 are exact for |k| < 2^20. */
#define KX_PIO2_1 1.5707963267341256
#define KX_PIO2_2 6.077100506303966e-11
#define KX_PIO2_3 2.0222662487959506e-21
#define KX_TWO_OVER_PI 0.6366197723675814

/* valid for |x| < 1.6e6 (|k| < 2^20); larger arguments are rejected by the
 * callers (joint values are validated against that bound on the host). */
KX_HD void kx_sincos(double x, double* s, double* c)
{
  double k = kx_rint(kx_mul(x, KX_TWO_OVER_PI));
  double r = kx_sub(kx_sub(kx_sub(x, kx_mul(k, KX_PIO2_1)), kx_mul(k, KX_PIO2_2)),
                    kx_mul(k, KX_PIO2_3));
  double r2 = kx_mul(r, r);
  /* sin r = r - r^3 * ps,  ps = 1/3! - r^2/5! + r^4/7! - ... - r^14/17!
   * (Horner in r^2, highest power first) */
  double ps = -2.8114572543455206e-15;                  /* -1/17! */
  ps = kx_add(kx_mul(ps, r2), 7.647163731819816e-13);   /* +1/15! */
  ps = kx_add(kx_mul(ps, r2), -1.6059043836821613e-10); /* -1/13! */
  ps = kx_add(kx_mul(ps, r2), 2.505210838544172e-08);   /* +1/11! */
  ps = kx_add(kx_mul(ps, r2), -2.7557319223985893e-06); /* -1/9!  */
  ps = kx_add(kx_mul(ps, r2), 0.0001984126984126984);   /* +1/7!  */
  ps = kx_add(kx_mul(ps, r2), -0.008333333333333333);   /* -1/5!  */
  ps = kx_add(kx_mul(ps, r2), 0.16666666666666666);     /* +1/3!  */
  double sn = kx_sub(r, kx_mul(kx_mul(r, r2), ps));
  /* cos r = 1 - r^2 * pc,  pc = 1/2! - r^2/4! + ... + r^16/18! */
  double pc = 1.5619206968586225e-16;                   /* +1/18! */
  pc = kx_add(kx_mul(pc, r2), -4.779477332387385e-14);  /* -1/16! */
  pc = kx_add(kx_mul(pc, r2), 1.1470745597729725e-11);  /* 1/14! */
  pc = kx_add(kx_mul(pc, r2), -2.08767569878681e-09);   /* -1/12! */
  pc = kx_add(kx_mul(pc, r2), 2.755731922398589e-07);   /* 1/10! */
  pc = kx_add(kx_mul(pc, r2), -2.48015873015873e-05);   /* -1/8! */
  pc = kx_add(kx_mul(pc, r2), 0.001388888888888889);    /* 1/6! */
  pc = kx_add(kx_mul(pc, r2), -0.041666666666666664);   /* -1/4! */
  pc = kx_add(kx_mul(pc, r2), 0.5);                     /* 1/2! */
  double cs = kx_sub(1.0, kx_mul(r2, pc));
  int q = ((int)k) & 3;
  if (q == 0) { *s = sn; *c = cs; }
  else if (q == 1) { *s = cs; *c = -sn; }
  else if (q == 2) { *s = -sn; *c = -cs; }
  else { *s = -cs; *c = sn; }
}

/* ---- rigid transforms --------------------------------------------------- */
KX_HD double kx_dot3(const double* a, const double* b)
{
  return kx_add(kx_add(kx_mul(a[0], b[0]), kx_mul(a[1], b[1])), kx_mul(a[2], b[2]));
}

KX_HD void kx_cross3(const double* a, const double* b, double* o)
{
  o[0] = kx_sub(kx_mul(a[1], b[2]), kx_mul(a[2], b[1]));
  o[1] = kx_sub(kx_mul(a[2], b[0]), kx_mul(a[0], b[2]));
  o[2] = kx_sub(kx_mul(a[0], b[1]), kx_mul(a[1], b[0]));
}

KX_HD void kx_sub3(const double* a, const double* b, double* o)
{
  o[0] = kx_sub(a[0], b[0]);
  o[1] = kx_sub(a[1], b[1]);
  o[2] = kx_sub(a[2], b[2]);
}

/* o = A*B  (o may not alias A or B) */
KX_HD void kx_compose(const double* A, const double* B, double* o)
{
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c)
      o[3 * r + c] = kx_add(kx_add(kx_mul(A[3 * r + 0], B[c]), kx_mul(A[3 * r + 1], B[3 + c])),
                            kx_mul(A[3 * r + 2], B[6 + c]));
    o[9 + r] = kx_add(kx_add(kx_add(kx_mul(A[3 * r + 0], B[9]), kx_mul(A[3 * r + 1], B[10])),
                             kx_mul(A[3 * r + 2], B[11])),
                      A[9 + r]);
  }
}

KX_HD void kx_xform_point(const double* T, const double* v, double* o)
{
  for (int r = 0; r < 3; ++r)
    o[r] = kx_add(kx_add(kx_add(kx_mul(T[3 * r + 0], v[0]), kx_mul(T[3 * r + 1], v[1])),
                         kx_mul(T[3 * r + 2], v[2])),
                  T[9 + r]);
}

/* Rotation about unit axis w by angle q:  R = c I + s [w]x + (1-c) w w^T */
KX_HD void kx_axis_rotation(const double* w, double q, double* R)
{
  double s, c;
  kx_sincos(q, &s, &c);
  double v = kx_sub(1.0, c);
  double wx = w[0], wy = w[1], wz = w[2];
  R[0] = kx_add(c, kx_mul(kx_mul(wx, wx), v));
  R[1] = kx_sub(kx_mul(kx_mul(wx, wy), v), kx_mul(wz, s));
  R[2] = kx_add(kx_mul(kx_mul(wx, wz), v), kx_mul(wy, s));
  R[3] = kx_add(kx_mul(kx_mul(wy, wx), v), kx_mul(wz, s));
  R[4] = kx_add(c, kx_mul(kx_mul(wy, wy), v));
  R[5] = kx_sub(kx_mul(kx_mul(wy, wz), v), kx_mul(wx, s));
  R[6] = kx_sub(kx_mul(kx_mul(wz, wx), v), kx_mul(wy, s));
  R[7] = kx_add(kx_mul(kx_mul(wz, wy), v), kx_mul(wx, s));
  R[8] = kx_add(c, kx_mul(kx_mul(wz, wz), v));
}

#define KX_JOINT_REVOLUTE 0
#define KX_JOINT_PRISMATIC 1
#define KX_JOINT_WELD 2

/* Local transform of a link relative to its parent: T0_Parent * J(q). */
KX_HD void kx_joint_local(const double* T0P, const double* w, int type, double q, double* L)
{
  if (type == KX_JOINT_REVOLUTE) {
    double J[12];
    kx_axis_rotation(w, q, J);
    J[9] = 0.0; J[10] = 0.0; J[11] = 0.0;
    kx_compose(T0P, J, L);
  } else if (type == KX_JOINT_PRISMATIC) {
    double J[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    J[9] = kx_mul(w[0], q); J[10] = kx_mul(w[1], q); J[11] = kx_mul(w[2], q);
    kx_compose(T0P, J, L);
  } else {
    for (int i = 0; i < 12; ++i) L[i] = T0P[i];
  }
}

/* Edge interpolation, Cpp/Modeling/Interpolate.cpp:10-14 for Normal joints
 * (out = x*(1-u) + y*u there; here the algebraically equal a + u*(b-a), which
 * is exact at both ends).  u = k / n. */
KX_HD double kx_interp(double a, double b, int k, int n)
{
  double u = kx_div((double)k, (double)n);
  return kx_add(a, kx_mul(u, kx_sub(b, a)));
}

/* ---- triangle / triangle ------------------------------------------------ */
/* projection interval test along axis a; returns 1 if a separates p and q */
KX_HD int kx_sep_axis(const double* a, const double p[3][3], const double q[3][3])
{
  double p0 = kx_dot3(a, p[0]), p1 = kx_dot3(a, p[1]), p2 = kx_dot3(a, p[2]);
  double q0 = kx_dot3(a, q[0]), q1 = kx_dot3(a, q[1]), q2 = kx_dot3(a, q[2]);
  double pmin = fmin(p0, fmin(p1, p2)), pmax = fmax(p0, fmax(p1, p2));
  double qmin = fmin(q0, fmin(q1, q2)), qmax = fmax(q0, fmax(q1, q2));
  return (pmax < qmin) || (qmax < pmin);
}

/* P, Q: 9 doubles each (three vertices).  Returns 1 if the closed triangles
 * intersect (touching included).  Coordinates are taken relative to P's
 * first vertex before any product. */
KX_HD int kx_tri_tri_overlap(const double* P, const double* Q)
{
  double p[3][3], q[3][3];
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i) {
      p[k][i] = kx_sub(P[3 * k + i], P[i]);
      q[k][i] = kx_sub(Q[3 * k + i], P[i]);
    }
  double ep[3][3], eq[3][3];
  for (int k = 0; k < 3; ++k) {
    kx_sub3(p[(k + 1) % 3], p[k], ep[k]);
    kx_sub3(q[(k + 1) % 3], q[k], eq[k]);
  }
  double np[3], nq[3], a[3];
  kx_cross3(ep[0], ep[1], np);
  kx_cross3(eq[0], eq[1], nq);
  if (kx_sep_axis(np, p, q)) return 0;
  if (kx_sep_axis(nq, p, q)) return 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      kx_cross3(ep[i], eq[j], a);
      if (kx_sep_axis(a, p, q)) return 0;
    }
  for (int i = 0; i < 3; ++i) {
    kx_cross3(np, ep[i], a);
    if (kx_sep_axis(a, p, q)) return 0;
    kx_cross3(nq, eq[i], a);
    if (kx_sep_axis(a, p, q)) return 0;
  }
  return 1;
}

KX_HD double kx_clamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

/* Closest points between segments p1+s*d1 and p2+t*d2, s,t in [0,1]
 * (minimiser of a convex quadratic on the unit square: interior stationary
 * point, then clamping of each parameter in turn).  Returns the squared
 * distance. */
KX_HD double kx_seg_seg(const double* p1, const double* d1, const double* p2, const double* d2,
                        double* c1, double* c2)
{
  double r[3];
  kx_sub3(p1, p2, r);
  double a = kx_dot3(d1, d1), e = kx_dot3(d2, d2), f = kx_dot3(d2, r);
  double s, t;
  if (a <= 1e-300 && e <= 1e-300) {
    s = 0.0; t = 0.0;
  } else if (a <= 1e-300) {
    s = 0.0; t = kx_clamp01(kx_div(f, e));
  } else {
    double c = kx_dot3(d1, r);
    if (e <= 1e-300) {
      t = 0.0; s = kx_clamp01(kx_div(-c, a));
    } else {
      double b = kx_dot3(d1, d2);
      double den = kx_sub(kx_mul(a, e), kx_mul(b, b));
      s = den > 0.0 ? kx_clamp01(kx_div(kx_sub(kx_mul(b, f), kx_mul(c, e)), den)) : 0.0;
      t = kx_div(kx_add(kx_mul(b, s), f), e);
      if (t < 0.0) {
        t = 0.0; s = kx_clamp01(kx_div(-c, a));
      } else if (t > 1.0) {
        t = 1.0; s = kx_clamp01(kx_div(kx_sub(b, c), a));
      }
    }
  }
  for (int i = 0; i < 3; ++i) {
    c1[i] = kx_add(p1[i], kx_mul(d1[i], s));
    c2[i] = kx_add(p2[i], kx_mul(d2[i], t));
  }
  double dd[3];
  kx_sub3(c1, c2, dd);
  return kx_dot3(dd, dd);
}

/* Closest point on triangle (a,b,c) to point p, by Voronoi-region
 * classification with barycentric coordinates.  Returns squared distance. */
KX_HD double kx_pt_tri(const double* p, const double* a, const double* b, const double* c,
                       double* cp)
{
  double ab[3], ac[3], ap[3];
  kx_sub3(b, a, ab); kx_sub3(c, a, ac); kx_sub3(p, a, ap);
  double d1 = kx_dot3(ab, ap), d2 = kx_dot3(ac, ap);
  int done = 0;
  if (d1 <= 0.0 && d2 <= 0.0) {
    cp[0] = a[0]; cp[1] = a[1]; cp[2] = a[2]; done = 1;
  }
  double bp[3];
  kx_sub3(p, b, bp);
  double d3 = kx_dot3(ab, bp), d4 = kx_dot3(ac, bp);
  if (!done && d3 >= 0.0 && d4 <= d3) {
    cp[0] = b[0]; cp[1] = b[1]; cp[2] = b[2]; done = 1;
  }
  double vc = kx_sub(kx_mul(d1, d4), kx_mul(d3, d2));
  if (!done && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    double v = kx_div(d1, kx_sub(d1, d3));
    for (int i = 0; i < 3; ++i) cp[i] = kx_add(a[i], kx_mul(ab[i], v));
    done = 1;
  }
  double cpv[3];
  kx_sub3(p, c, cpv);
  double d5 = kx_dot3(ab, cpv), d6 = kx_dot3(ac, cpv);
  if (!done && d6 >= 0.0 && d5 <= d6) {
    cp[0] = c[0]; cp[1] = c[1]; cp[2] = c[2]; done = 1;
  }
  double vb = kx_sub(kx_mul(d5, d2), kx_mul(d1, d6));
  if (!done && vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    double w = kx_div(d2, kx_sub(d2, d6));
    for (int i = 0; i < 3; ++i) cp[i] = kx_add(a[i], kx_mul(ac[i], w));
    done = 1;
  }
  double va = kx_sub(kx_mul(d3, d6), kx_mul(d5, d4));
  if (!done && va <= 0.0 && kx_sub(d4, d3) >= 0.0 && kx_sub(d5, d6) >= 0.0) {
    double w = kx_div(kx_sub(d4, d3), kx_add(kx_sub(d4, d3), kx_sub(d5, d6)));
    for (int i = 0; i < 3; ++i) cp[i] = kx_add(b[i], kx_mul(kx_sub(c[i], b[i]), w));
    done = 1;
  }
  if (!done) {
    double den = kx_add(kx_add(va, vb), vc);
    double v = kx_div(vb, den), w = kx_div(vc, den);
    for (int i = 0; i < 3; ++i)
      cp[i] = kx_add(kx_add(a[i], kx_mul(ab[i], v)), kx_mul(ac[i], w));
  }
  double dd[3];
  kx_sub3(p, cp, dd);
  return kx_dot3(dd, dd);
}

/* Squared distance between closed triangles P and Q (9 doubles each) and a
 * pair of closest points (cp on P, cq on Q).  Zero when they intersect, in
 * which case cp = cq = P's first vertex (the pair is then not meaningful).
 * Candidates are scanned in a fixed order and replaced only on a strictly
 * smaller value, so ties resolve identically on every platform. */
KX_HD double kx_tri_tri_dist2(const double* P, const double* Q, double* cp, double* cq)
{
  if (kx_tri_tri_overlap(P, Q)) {
    for (int i = 0; i < 3; ++i) { cp[i] = P[i]; cq[i] = P[i]; }
    return 0.0;
  }
  double o[3] = {P[0], P[1], P[2]};
  double p[3][3], q[3][3];
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i) {
      p[k][i] = kx_sub(P[3 * k + i], o[i]);
      q[k][i] = kx_sub(Q[3 * k + i], o[i]);
    }
  double best = 1e300, bp[3] = {0, 0, 0}, bq[3] = {0, 0, 0};
  double c1[3], c2[3], d1[3], d2[3];
  for (int i = 0; i < 3; ++i) {
    kx_sub3(p[(i + 1) % 3], p[i], d1);
    for (int j = 0; j < 3; ++j) {
      kx_sub3(q[(j + 1) % 3], q[j], d2);
      double d = kx_seg_seg(p[i], d1, q[j], d2, c1, c2);
      if (d < best) {
        best = d;
        for (int t = 0; t < 3; ++t) { bp[t] = c1[t]; bq[t] = c2[t]; }
      }
    }
  }
  for (int k = 0; k < 3; ++k) {
    double d = kx_pt_tri(p[k], q[0], q[1], q[2], c2);
    if (d < best) {
      best = d;
      for (int t = 0; t < 3; ++t) { bp[t] = p[k][t]; bq[t] = c2[t]; }
    }
  }
  for (int k = 0; k < 3; ++k) {
    double d = kx_pt_tri(q[k], p[0], p[1], p[2], c1);
    if (d < best) {
      best = d;
      for (int t = 0; t < 3; ++t) { bp[t] = c1[t]; bq[t] = q[k][t]; }
    }
  }
  for (int t = 0; t < 3; ++t) {
    cp[t] = kx_add(bp[t], o[t]);
    cq[t] = kx_add(bq[t], o[t]);
  }
  return best;
}

/* ---- ray / triangle ----------------------------------------------------- */
/* With e1 = b - a, e2 = c - a, w = s - a, p = d x e2, q = w x e1:
   det = e1 . p, U = w . p, V = d . q, Tn = e2 . q; the ray meets the closed
   triangle at t = Tn / det iff U, V, det - (U + V) and Tn all have the sign
   of det (zero allowed).  T: 9 doubles (a, b, c).  Returns 1 and *t on a hit. */
KX_HD int kx_ray_tri(const double* s, const double* d, const double* T, double* t)
{
  double e1[3], e2[3], w[3], p[3], q[3];
  kx_sub3(T + 3, T, e1);
  kx_sub3(T + 6, T, e2);
  kx_sub3(s, T, w);
  kx_cross3(d, e2, p);
  const double det = kx_dot3(e1, p);
  if (det == 0.0) return 0;
  const double U = kx_dot3(w, p);
  kx_cross3(w, e1, q);
  const double V = kx_dot3(d, q);
  const double Tn = kx_dot3(e2, q);
  const double UV = kx_add(U, V);
  if (det > 0.0) {
    if (U < 0.0 || V < 0.0 || UV > det || Tn < 0.0) return 0;
  } else {
    if (U > 0.0 || V > 0.0 || UV < det || Tn > 0.0) return 0;
  }
  *t = kx_div(Tn, det);
  return 1;
}

#endif /* KGPU_EXACT_H */
