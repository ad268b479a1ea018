// kgpu_plain.cu — the plain FP64 GPU method, kept as the comparison baseline
// for the batched engine.
//
// One thread per configuration (or per edge, stepping through its
// configurations in order, or per (edge, step)), FP64 forward kinematics, FP64 BVH-vs-BVH
// traversal with a per-thread stack, and the canonical FP64 triangle test on
// every candidate pair.  No warp cooperation, no FP32 filter, no work queue:
// this is the straightforward port of the reference's serial loops
// (Cpp/Planning/RobotCSpace.cpp:786-823, PlannerSettings.cpp:241-331) to one
// thread each.  Its verdicts equal the oracle's by construction.
#include <climits>

#include "kgpu_device.cuh"

namespace kgpu {

namespace {

constexpr int kPlainStack = 128;

__device__ __forceinline__ void box64_world(const double* T, const double* n, double* c, double* h)
{
  for (int r = 0; r < 3; ++r) {
    c[r] = T[3 * r] * n[0] + T[3 * r + 1] * n[1] + T[3 * r + 2] * n[2] + T[9 + r];
    h[r] = fabs(T[3 * r]) * n[3] + fabs(T[3 * r + 1]) * n[4] + fabs(T[3 * r + 2]) * n[5];
  }
}

// 0 free, 1 hit, 2 stack overflow
__device__ int plain_query(const KWorldDev& W, const KRobotDev& R, const double (*T)[12], int la,
                           int tgt)
{
  int ra = R.link_root[la];
  int rb = tgt < 32 ? R.link_root[tgt] : W.group_root[tgt - 32];
  if (ra < 0 || rb < 0) return 0;
  double mA = R.link_margin64[la];
  double mB = tgt < 32 ? R.link_margin64[tgt] : (double)W.group_margin[tgt - 32];
  double tol = 1e-9 + mA + mB;
  int2 st[kPlainStack];
  int top = 0;
  st[top++] = make_int2(ra, rb);
  while (top > 0) {
    int2 pr = st[--top];
    const double* na = W.lnode64 + 6 * (size_t)pr.x;
    const double* nb = tgt < 32 ? W.lnode64 + 6 * (size_t)pr.y : W.enode64 + 6 * (size_t)pr.y;
    double ca[3], ha[3], cb[3], hb[3];
    box64_world(T[la], na, ca, ha);
    if (tgt < 32) box64_world(T[tgt], nb, cb, hb);
    else for (int i = 0; i < 3; ++i) { cb[i] = nb[i]; hb[i] = nb[3 + i]; }
    bool sep = false;
    for (int i = 0; i < 3; ++i)
      if (fabs(ca[i] - cb[i]) > ha[i] + hb[i] + tol) sep = true;
    if (sep) continue;
    KNode ka = W.lnodes[pr.x];
    KNode kb = tgt < 32 ? W.lnodes[pr.y] : W.enodes[pr.y];
    int cntA = f2i(ka.b.w), cntB = f2i(kb.b.w);
    int ia = f2i(ka.a.w), ib = f2i(kb.a.w);
    if (cntA > 0 && cntB > 0) {
      for (int i = 0; i < cntA; ++i) {
        double P[9];
        const double* pa = W.ltri64 + 9 * (size_t)(ia + i);
        for (int v = 0; v < 3; ++v) kx_xform_point(T[la], pa + 3 * v, P + 3 * v);
        for (int j = 0; j < cntB; ++j) {
          double Q[9];
          double m;
          if (tgt < 32) {
            const double* pb = W.ltri64 + 9 * (size_t)(ib + j);
            for (int v = 0; v < 3; ++v) kx_xform_point(T[tgt], pb + 3 * v, Q + 3 * v);
            m = kx_add(mA, mB);
          } else {
            const double* pb = W.etri64 + 9 * (size_t)(ib + j);
            for (int k = 0; k < 9; ++k) Q[k] = pb[k];
            m = kx_add(mA, W.obj_margin64[W.etri_obj[ib + j]]);
          }
          int hit;
          if (m == 0.0) hit = kx_tri_tri_overlap(P, Q);
          else {
            double cp[3], cq[3];
            hit = kx_tri_tri_dist2(P, Q, cp, cq) <= kx_mul(m, m);
          }
          if (hit) return 1;
        }
      }
    } else {
      if (top + 2 > kPlainStack) return 2;
      bool splitB = cntA > 0 || (cntB == 0 && (kb.b.x + kb.b.y + kb.b.z) > (ka.b.x + ka.b.y + ka.b.z));
      if (splitB) {
        st[top++] = make_int2(pr.x, ib + 1);
        st[top++] = make_int2(pr.x, ib);
      } else {
        st[top++] = make_int2(ia + 1, pr.y);
        st[top++] = make_int2(ia, pr.y);
      }
    }
  }
  return 0;
}

__device__ void fk64_all(const KRobotDev& R, const double* q, double (*T)[12])
{
  for (int i = 0; i < R.nlinks; ++i) {
    double Lc[12];
    kx_joint_local(R.T0P64[i], R.axis64[i], R.jtype[i], q[i], Lc);
    int p = R.parents[i];
    if (p < 0) for (int k = 0; k < 12; ++k) T[i][k] = Lc[k];
    else kx_compose(T[p], Lc, T[i]);
  }
}

// returns bit 0 env hit, bit 1 self hit, bit 2 overflow
__device__ int plain_config(const KWorldDev& W, const KRobotDev& R, const double (*T)[12],
                            bool do_env, bool do_self, bool stop_any)
{
  int res = 0;
  if (do_env) {
    for (int k = 0; k < R.nqueries_env; ++k) {
      uint32_t qw = W.queries[R.query_off + k];
      int r = plain_query(W, R, T, qw & 0xff, (qw >> 8) & 0xff);
      if (r == 2) return 4;
      if (r == 1) { res |= 1; break; }
    }
  }
  if (stop_any && res) return res;
  if (do_self) {
    for (int k = 0; k < R.nqueries_self; ++k) {
      uint32_t qw = W.queries[R.query_off + R.nqueries_env + k];
      int r = plain_query(W, R, T, qw & 0xff, (qw >> 8) & 0xff);
      if (r == 2) return 4;
      if (r == 1) { res |= 2; break; }
    }
  }
  return res;
}

__global__ void k_plain_configs(KWorldDev W, int robot, const float* q, int B, uint8_t* env_hit,
                                uint8_t* self_hit)
{
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const KRobotDev& R = W.robots[robot];
  double qd[kMaxLinks];
  for (int i = 0; i < R.nlinks; ++i) {
    qd[i] = (double)q[(size_t)b * R.nlinks + i];
    if (!(fabs(qd[i]) < 1.0e6)) { set_status(W.status, KGPU_ERR_NOT_FINITE); return; }
  }
  double T[kMaxLinks][12];
  fk64_all(R, qd, T);
  int r = plain_config(W, R, T, env_hit != nullptr, self_hit != nullptr, false);
  if (r & 4) { set_status(W.status, KGPU_ERR_OVERFLOW); return; }
  if (env_hit) env_hit[b] = (r & 1) ? 1 : 0;
  if (self_hit) self_hit[b] = (r & 2) ? 1 : 0;
}

__global__ void k_plain_edges(KWorldDev W, int robot, const float* qa, const float* qb,
                              const int* nsteps, int E, int* first_hit)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const KRobotDev& R = W.robots[robot];
  int nl = R.nlinks;
  int n = nsteps[e];
  if (n < 1 || n > kMaxSteps) { set_status(W.status, KGPU_ERR_INVALID); first_hit[e] = -1; return; }
  int hit = -1;
  double qd[kMaxLinks];
  double T[kMaxLinks][12];
  for (int k = 0; k <= n && hit < 0; ++k) {
    bool ok = true;
    for (int i = 0; i < nl; ++i) {
      qd[i] = kx_interp((double)qa[(size_t)e * nl + i], (double)qb[(size_t)e * nl + i], k, n);
      if (!(fabs(qd[i]) < 1.0e6)) { set_status(W.status, KGPU_ERR_NOT_FINITE); first_hit[e] = -1; return; }
      if (qd[i] < R.qmin64[i] || qd[i] > R.qmax64[i]) ok = false;
    }
    if (!ok) { hit = k; break; }
    fk64_all(R, qd, T);
    int r = plain_config(W, R, T, true, true, true);
    if (r & 4) { set_status(W.status, KGPU_ERR_OVERFLOW); first_hit[e] = -1; return; }
    if (r) hit = k;
  }
  first_hit[e] = hit;
}

// The plain method with one thread per (edge, step): every configuration
// of every edge is checked independently (no in-order early exit), the
// smallest infeasible step of each edge kept by atomicMin.  off[e] = number
// of steps of the edges before e (one block, a chunked scan).
__global__ void k_plain_step_offsets(const int* nsteps, int E, int* off, int* status)
{
  __shared__ int carry;
  __shared__ int part[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < E; base += 1024) {
    const int e = base + threadIdx.x;
    const int n = e < E ? nsteps[e] : 0;
    int own = e < E ? n + 1 : 0;
    if (e < E && (n < 1 || n > kMaxSteps)) {
      set_status(status, KGPU_ERR_INVALID);
      own = 0;  // an invalid edge has no steps (its result stays -1)
    }
    part[threadIdx.x] = own;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive scan (Hillis-Steele)
      const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += v;
      __syncthreads();
    }
    if (e < E) off[e] = carry + part[threadIdx.x] - own;
    __syncthreads();
    if (threadIdx.x == 0) carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) off[E] = carry;
}

__global__ void k_plain_edge_steps(KWorldDev W, int robot, const float* qa, const float* qb, const int* nsteps,
                                   int E, const int* off, int* first_hit)
{
  const KRobotDev& R = W.robots[robot];
  const int nl = R.nlinks;
  const int total = off[E];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < total; s += gridDim.x * blockDim.x) {
    int lo = 0, hi = E - 1;  // the edge e with off[e] <= s < off[e + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= s) lo = mid; else hi = mid - 1;
    }
    const int e = lo, k = s - off[e], n = nsteps[e];
    double qd[kMaxLinks];
    bool ok = true, finite = true;
    for (int i = 0; i < nl; ++i) {
      qd[i] = kx_interp((double)qa[(size_t)e * nl + i], (double)qb[(size_t)e * nl + i], k, n);
      if (!(fabs(qd[i]) < 1.0e6)) finite = false;
      if (qd[i] < R.qmin64[i] || qd[i] > R.qmax64[i]) ok = false;
    }
    if (!finite) { set_status(W.status, KGPU_ERR_NOT_FINITE); continue; }
    if (!ok) { atomicMin(first_hit + e, k); continue; }
    double T[kMaxLinks][12];
    fk64_all(R, qd, T);
    const int r = plain_config(W, R, T, true, true, true);
    if (r & 4) { set_status(W.status, KGPU_ERR_OVERFLOW); continue; }
    if (r) atomicMin(first_hit + e, k);
  }
}

// The plain method with one thread per (edge, step, query): each thread
// forms its step's FP64 transforms itself and traverses one (link, group)
// or (link, link) query; a contact or a joint-limit violation records the
// step by atomicMin.  The finest grain the plain method has (a configuration
// check split into its pair checks).
__global__ void k_plain_edge_pairs(KWorldDev W, int robot, const float* qa, const float* qb, const int* nsteps,
                                   int E, const int* off, int* first_hit)
{
  const KRobotDev& R = W.robots[robot];
  const int nl = R.nlinks;
  const int nq = R.nqueries_env + R.nqueries_self;
  if (nq <= 0) return;
  const long long total = (long long)off[E] * nq;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(t / nq), qi = (int)(t - (long long)s * nq);
    int lo = 0, hi = E - 1;  // the edge e with off[e] <= s < off[e + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= s) lo = mid; else hi = mid - 1;
    }
    const int e = lo, k = s - off[e], n = nsteps[e];
    double qd[kMaxLinks];
    bool ok = true, finite = true;
    for (int i = 0; i < nl; ++i) {
      qd[i] = kx_interp((double)qa[(size_t)e * nl + i], (double)qb[(size_t)e * nl + i], k, n);
      if (!(fabs(qd[i]) < 1.0e6)) finite = false;
      if (qd[i] < R.qmin64[i] || qd[i] > R.qmax64[i]) ok = false;
    }
    if (!finite) { set_status(W.status, KGPU_ERR_NOT_FINITE); continue; }
    if (!ok) { atomicMin(first_hit + e, k); continue; }
    double T[kMaxLinks][12];
    fk64_all(R, qd, T);
    const uint32_t qw = W.queries[R.query_off + qi];
    const int r = plain_query(W, R, T, qw & 0xff, (qw >> 8) & 0xff);
    if (r == 2) { set_status(W.status, KGPU_ERR_OVERFLOW); continue; }
    if (r == 1) atomicMin(first_hit + e, k);
  }
}

__global__ void k_plain_fill(int* a, int n, int v)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

__global__ void k_plain_unset(int* a, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && a[i] == INT_MAX) a[i] = -1;
}

}  // namespace

cudaError_t launch_plain64_edge_steps(const KWorldDev& W, int robot, const float* qa, const float* qb,
                                      const int* nsteps, int E, int* first_hit, int* off, int num_sms,
                                      cudaStream_t s)
{
  if (E <= 0) return cudaSuccess;
  const int tb = 256, gb = (E + tb - 1) / tb;
  k_plain_fill<<<gb, tb, 0, s>>>(first_hit, E, INT_MAX);
  k_plain_step_offsets<<<1, 1024, 0, s>>>(nsteps, E, off, W.status);
  k_plain_edge_steps<<<num_sms * 16, 64, 0, s>>>(W, robot, qa, qb, nsteps, E, off, first_hit);
  k_plain_unset<<<gb, tb, 0, s>>>(first_hit, E);
  return cudaGetLastError();
}

cudaError_t launch_plain64_edge_pairs(const KWorldDev& W, int robot, const float* qa, const float* qb,
                                      const int* nsteps, int E, int* first_hit, int* off, int num_sms,
                                      cudaStream_t s)
{
  if (E <= 0) return cudaSuccess;
  const int tb = 256, gb = (E + tb - 1) / tb;
  k_plain_fill<<<gb, tb, 0, s>>>(first_hit, E, INT_MAX);
  k_plain_step_offsets<<<1, 1024, 0, s>>>(nsteps, E, off, W.status);
  k_plain_edge_pairs<<<num_sms * 16, 64, 0, s>>>(W, robot, qa, qb, nsteps, E, off, first_hit);
  k_plain_unset<<<gb, tb, 0, s>>>(first_hit, E);
  return cudaGetLastError();
}

cudaError_t launch_plain64_configs(const KWorldDev& W, int robot, const float* q, int B,
                                   uint8_t* env_hit, uint8_t* self_hit, cudaStream_t s)
{
  if (B <= 0) return cudaSuccess;
  int tb = 64;
  k_plain_configs<<<(B + tb - 1) / tb, tb, 0, s>>>(W, robot, q, B, env_hit, self_hit);
  return cudaGetLastError();
}

cudaError_t launch_plain64_edges(const KWorldDev& W, int robot, const float* qa, const float* qb,
                                 const int* nsteps, int E, int* first_hit, cudaStream_t s)
{
  if (E <= 0) return cudaSuccess;
  int tb = 64;
  k_plain_edges<<<(E + tb - 1) / tb, tb, 0, s>>>(W, robot, qa, qb, nsteps, E, first_hit);
  return cudaGetLastError();
}

}  // namespace kgpu
