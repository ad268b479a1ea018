// kgpu_ik.cu — batched inverse kinematics, one warp per problem.
//
// Replaces IKSolver.solve over IKObjective point / transform constraints
// (Python/klampt/src/robotik.cpp:556-689; KrisLibrary RobotIKSolver, absent
// here) for B independent problems in one launch.  The method is this
// project's own (the reference's solver internals are not available):
// Levenberg-Marquardt on the residual
//   e = [p(q) - p*]                                   (position only), or
//   e = [p(q) - p*; 1/2 sum_k R*_k x R_k(q)]           (position + rotation;
//        the second block is sin(theta) u for R = Rot(u, theta) R*),
// with the full Jacobian's rows as derivative (angular rows for the rotation
// block), steps dq = -J^T (J J^T + mu I)^-1 e on the link's ancestor DOFs,
// q clamped to the joint limits after every step, mu / 4 on an accepted step
// (residual norm decreased), mu * 8 on a rejected one.  Converged when
// max |e_i| <= tol.  The FP64 oracle runs the same iteration.
#include <cfloat>

#include "kgpu_device.cuh"

namespace kgpu {

namespace {

struct IkArgs {
  int robot;
  int B;
  float* q;              // [B, L] in: initial guesses, out: results
  const int* links;      // [B] or null (link_all)
  int link_all;
  const float* plocal;   // [B, 3]
  const float* ptarget;  // [B, 3]
  const float* Rtarget;  // [B, 9] row-major or null (position only)
  int max_iters;
  float tol;
  uint8_t* ok;           // [B]
  float* residual;       // [B] max |e_i| at the result
  int* iters;            // [B] iterations used (may be null)
};

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// residual of link li at the FP32 transforms held in lanes (P of lane li)
__device__ __forceinline__ void ik_residual(const float* P, int li, float3 pl, const float* pt, const float* Rt,
                                            int m, float* e)
{
  float T[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) T[k] = __shfl_sync(0xffffffffu, P[k], li);
  const float3 p = xform32(T, pl);
  e[0] = p.x - pt[0];
  e[1] = p.y - pt[1];
  e[2] = p.z - pt[2];
  if (m == 6) {
    // 1/2 sum over columns k of R*_k x R_k
    float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float ax = Rt[k], ay = Rt[3 + k], az = Rt[6 + k];
      const float bx = T[k], by = T[3 + k], bz = T[6 + k];
      ex += ay * bz - az * by;
      ey += az * bx - ax * bz;
      ez += ax * by - ay * bx;
    }
    e[3] = 0.5f * ex;
    e[4] = 0.5f * ey;
    e[5] = 0.5f * ez;
  }
}

__global__ void __launch_bounds__(256) k_ik(const KWorldDev* __restrict__ W, const IkArgs A)
{
  const int lane = threadIdx.x & 31;
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= A.B) return;
  const KRobotDev& R = W->robots[A.robot];
  const int nl = R.nlinks;
  const int li = A.links ? __ldg(A.links + b) : A.link_all;
  if (li < 0 || li >= nl) {
    if (lane == 0) set_status(W->status, KGPU_ERR_INVALID);
    return;
  }
  const int m = A.Rtarget ? 6 : 3;
  const float3 pl = make_float3(A.plocal[3 * (size_t)b], A.plocal[3 * (size_t)b + 1], A.plocal[3 * (size_t)b + 2]);
  float pt[3], Rt[9];
  for (int k = 0; k < 3; ++k) pt[k] = A.ptarget[3 * (size_t)b + k];
  for (int k = 0; k < 9; ++k) Rt[k] = A.Rtarget ? A.Rtarget[9 * (size_t)b + k] : 0.f;
  // active DOFs: the link and its ancestors (other columns of J are 0)
  bool active = false;
  if (lane < nl)
    for (int j = li; j >= 0; j = R.parents[j])
      if (j == lane) { active = true; break; }
  active = active && R.jtype[lane < nl ? lane : 0] != KX_JOINT_WELD;
  const float lo = lane < nl ? R.qmin[lane] : 0.f, hi = lane < nl ? R.qmax[lane] : 0.f;
  float q = lane < nl ? A.q[(size_t)b * nl + lane] : 0.f;
  q = fminf(fmaxf(q, lo), hi);

  float P[12], delta, e[6];
  warp_fk32(R, lane, q, 0.f, P, &delta);
  ik_residual(P, li, pl, pt, Rt, m, e);
  float E = 0.f, emax = 0.f;
  for (int a = 0; a < m; ++a) {
    E += e[a] * e[a];
    emax = fmaxf(emax, fabsf(e[a]));
  }
  float mu = 1e-4f;
  int it = 0;
#pragma unroll 1
  for (; it < A.max_iters && emax > A.tol; ++it) {
    // column `lane` of J at q (angular rows 0-2, linear rows 3-5 as in
    // k_jacobian); the residual orders position first, so row a of the
    // system is linear row a (a < 3) and angular row a - 3 (a >= 3)
    float c[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    {
      float Ti[12];
#pragma unroll
      for (int k = 0; k < 12; ++k) Ti[k] = __shfl_sync(0xffffffffu, P[k], li);
      const float3 p = xform32(Ti, pl);
      if (active) {
        const float ax = R.axis[lane][0], ay = R.axis[lane][1], az = R.axis[lane][2];
        const float wx = P[0] * ax + P[1] * ay + P[2] * az;
        const float wy = P[3] * ax + P[4] * ay + P[5] * az;
        const float wz = P[6] * ax + P[7] * ay + P[8] * az;
        if (R.jtype[lane] == KX_JOINT_REVOLUTE) {
          const float rx = p.x - P[9], ry = p.y - P[10], rz = p.z - P[11];
          c[0] = wy * rz - wz * ry;
          c[1] = wz * rx - wx * rz;
          c[2] = wx * ry - wy * rx;
          c[3] = wx; c[4] = wy; c[5] = wz;
        } else {
          c[0] = wx; c[1] = wy; c[2] = wz;
        }
      }
    }
    // A = J J^T + mu I (symmetric, lower triangle), y = A^-1 e by Cholesky,
    // every lane the same values
    float Am[21];
    int k = 0;
    for (int r = 0; r < m; ++r)
      for (int s = 0; s <= r; ++s)  // lane 0's sum for all: the lanes' orders differ
        Am[k++] = __shfl_sync(0xffffffffu, warp_sum(c[r] * c[s]), 0) + (r == s ? mu : 0.f);
    float y[6];
    bool spd = true;
    {
      float Lc[21];
      k = 0;
      for (int r = 0; r < m; ++r) {
        for (int s = 0; s <= r; ++s, ++k) {
          float v = Am[k];
          for (int t = 0; t < s; ++t) v -= Lc[r * (r + 1) / 2 + t] * Lc[s * (s + 1) / 2 + t];
          if (s == r) {
            spd = spd && v > 0.f;
            Lc[k] = sqrtf(fmaxf(v, 1e-30f));
          } else {
            Lc[k] = v / Lc[s * (s + 1) / 2 + s];
          }
        }
      }
      float z[6];
      for (int r = 0; r < m; ++r) {
        float v = e[r];
        for (int t = 0; t < r; ++t) v -= Lc[r * (r + 1) / 2 + t] * z[t];
        z[r] = v / Lc[r * (r + 1) / 2 + r];
      }
      for (int r = m - 1; r >= 0; --r) {
        float v = z[r];
        for (int t = r + 1; t < m; ++t) v -= Lc[t * (t + 1) / 2 + r] * y[t];
        y[r] = v / Lc[r * (r + 1) / 2 + r];
      }
    }
    if (!spd) {
      mu *= 8.f;
      if (mu > 1e6f) break;
      continue;
    }
    float dq = 0.f;
    for (int r = 0; r < m; ++r) dq -= c[r] * y[r];
    const float qn = lane < nl ? fminf(fmaxf(q + dq, lo), hi) : 0.f;
    float Pn[12], dn, en[6];
    warp_fk32(R, lane, qn, 0.f, Pn, &dn);
    ik_residual(Pn, li, pl, pt, Rt, m, en);
    float En = 0.f, enmax = 0.f;
    for (int a = 0; a < m; ++a) {
      En += en[a] * en[a];
      enmax = fmaxf(enmax, fabsf(en[a]));
    }
    if (En < E) {
      q = qn;
#pragma unroll
      for (int t = 0; t < 12; ++t) P[t] = Pn[t];
      for (int a = 0; a < m; ++a) e[a] = en[a];
      E = En;
      emax = enmax;
      mu = fmaxf(mu * 0.25f, 1e-10f);
    } else {
      mu *= 8.f;
      if (mu > 1e6f) break;
    }
  }
  if (lane < nl) A.q[(size_t)b * nl + lane] = q;
  if (lane == 0) {
    A.ok[b] = emax <= A.tol ? 1 : 0;
    A.residual[b] = emax;
    if (A.iters) A.iters[b] = it;
  }
}

}  // namespace

cudaError_t launch_ik(const KWorldDev* W, int robot, int B, float* q, const int* links, int link_all,
                      const float* plocal, const float* ptarget, const float* Rtarget, int max_iters, float tol,
                      uint8_t* ok, float* residual, int* iters, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  IkArgs A;
  A.robot = robot;
  A.B = B;
  A.q = q;
  A.links = links;
  A.link_all = link_all;
  A.plocal = plocal;
  A.ptarget = ptarget;
  A.Rtarget = Rtarget;
  A.max_iters = max_iters;
  A.tol = tol;
  A.ok = ok;
  A.residual = residual;
  A.iters = iters;
  const int threads = 256;
  k_ik<<<(int)(((long long)B * 32 + threads - 1) / threads), threads, 0, s>>>(W, A);
  return cudaGetLastError();
}

}  // namespace kgpu
