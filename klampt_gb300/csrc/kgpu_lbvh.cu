// kgpu_lbvh.cu — environment BVH built on the GPU (linear BVH), the
// alternative to the host surface-area builder (bvh.cpp) for large scenes.
//
// Replaces the PQP hierarchy precompute Klamp't runs in InitCollisions
// (Cpp/Modeling/World.cpp:266-274, Python/klampt/src/robotsim.cpp:
// 4118-4165) and produces the same layout as bvh.cpp: object-aware (every
// object owns one subtree, its triangles one contiguous run of the leaf
// order), children in adjacent slots, at most kLeafSize triangles per leaf,
// FP64 boxes plus FP32 boxes rounded outward.  Verdicts and distances do not
// depend on the tree's shape, only the traversal cost does.
//
// Method (Karras, "Maximizing parallelism in the construction of BVHs,
// octrees and k-d trees", HPG 2012):
//   1. keys: each object gets a rank (objects sorted by the Morton code of
//      their centroid box centre, host, one entry per object); each triangle
//      the 30-bit Morton code of its centroid within its object's centroid
//      box; key = rank << 32 | code, so an object's triangles sort into one
//      run and the radix tree has one node whose range is exactly that run;
//   2. one radix sort of (key, triangle) pairs (CUB);
//   3. the binary radix tree, one thread per internal node, ties between
//      equal keys broken by position;
//   4. boxes bottom up, one thread per leaf climbing to the root; the second
//      child to arrive at a node (atomic counter) forms the union.  Min and
//      max are exact, so the FP64 boxes equal those of the triangle sets;
//   5. host relayout, breadth first: a node whose range holds at most
//      kLeafSize triangles of one object becomes a leaf, the others get two
//      adjacent child slots.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "kgpu_internal.h"

namespace kgpu {

namespace {

__host__ __device__ __forceinline__ uint32_t expand_bits10(uint32_t v)
{
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__host__ __device__ __forceinline__ uint32_t quant10(double u)
{
  u = u < 0.0 ? 0.0 : (u > 1.0 ? 1.0 : u);
  const double s = u * 1024.0;
  return s >= 1023.0 ? 1023u : (uint32_t)s;
}

__host__ __device__ __forceinline__ uint32_t morton30(double x, double y, double z)
{
  return (expand_bits10(quant10(x)) << 2) | (expand_bits10(quant10(y)) << 1) | expand_bits10(quant10(z));
}

// keys: tri9 = 9 doubles per triangle (group order), obj = its object
// (group-local index), olo/oinv = per object the centroid box's low corner
// and 1/extent per axis (0 for a flat axis), rank = per object rank
__global__ void k_lbvh_keys(const double* __restrict__ tri9, const int* __restrict__ obj,
                            const double* __restrict__ olo, const double* __restrict__ oinv,
                            const uint32_t* __restrict__ rank, int n, unsigned long long* __restrict__ keys,
                            int* __restrict__ vals)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* T = tri9 + 9 * (size_t)i;
  const int o = obj[i];
  double u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double c = (T[a] + T[3 + a] + T[6 + a]) / 3.0;
    u[a] = (c - olo[3 * (size_t)o + a]) * oinv[3 * (size_t)o + a];
  }
  keys[i] = ((unsigned long long)rank[o] << 32) | morton30(u[0], u[1], u[2]);
  vals[i] = i;
}

// common-prefix length of sorted keys i and j (-1 outside [0, n)); equal
// keys continue with the prefix of their positions
__device__ __forceinline__ int lbvh_delta(const unsigned long long* __restrict__ k, int n, int i, int j)
{
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = k[i], b = k[j];
  if (a != b) return __clzll((long long)(a ^ b));
  return 64 + __clz(i ^ j);
}

// internal node i of the radix tree over n sorted keys: children (>= 0
// internal node, < 0 leaf -1-position), covered range [lo, hi], parents
__global__ void k_lbvh_tree(const unsigned long long* __restrict__ k, int n, int* __restrict__ left,
                            int* __restrict__ right, int* __restrict__ lo, int* __restrict__ hi,
                            int* __restrict__ pint, int* __restrict__ pleaf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = lbvh_delta(k, n, i, i + 1) - lbvh_delta(k, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = lbvh_delta(k, n, i, i - d);
  int lmax = 2;
  while (lbvh_delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (lbvh_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = lbvh_delta(k, n, i, j);
  int s = 0;
  for (int div = 2;; div <<= 1) {
    const int t = (l + div - 1) / div;
    if (lbvh_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int g = i + s * d + min(d, 0);
  const int a = min(i, j), b = max(i, j);
  if (a == g) {
    left[i] = -1 - g;
    pleaf[g] = i;
  } else {
    left[i] = g;
    pint[g] = i;
  }
  if (b == g + 1) {
    right[i] = -1 - (g + 1);
    pleaf[g + 1] = i;
  } else {
    right[i] = g + 1;
    pint[g + 1] = i;
  }
  lo[i] = a;
  hi[i] = b;
  if (i == 0) pint[0] = -1;
}

__device__ __forceinline__ void load_box(const double* ibox, const double* lbox, int c, double* b)
{
  const double* src = c >= 0 ? ibox + 6 * (size_t)c : lbox + 6 * (size_t)(-1 - c);
#pragma unroll
  for (int a = 0; a < 6; ++a) b[a] = __ldcg(src + a);
}

// boxes (lo.xyz, hi.xyz) of every leaf and internal node; flags zeroed
__global__ void k_lbvh_boxes(const double* __restrict__ tri9, const int* __restrict__ vals, int n,
                             const int* __restrict__ left, const int* __restrict__ right,
                             const int* __restrict__ pint, const int* __restrict__ pleaf, int* flags, double* lbox,
                             double* ibox)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* T = tri9 + 9 * (size_t)vals[k];
  double b[6];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b[a] = fmin(fmin(T[a], T[3 + a]), T[6 + a]);
    b[3 + a] = fmax(fmax(T[a], T[3 + a]), T[6 + a]);
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) __stcg(lbox + 6 * (size_t)k + a, b[a]);
  int p = n > 1 ? pleaf[k] : -1;
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(flags + p, 1) == 0) return;  // the sibling's thread finishes this node
    __threadfence();
    double x[6], y[6];
    load_box(ibox, lbox, left[p], x);
    load_box(ibox, lbox, right[p], y);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      b[a] = fmin(x[a], y[a]);
      b[3 + a] = fmax(x[3 + a], y[3 + a]);
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) __stcg(ibox + 6 * (size_t)p + a, b[a]);
    p = pint[p];
  }
}

inline float round_up_f32(double x)
{
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
  return f;
}

inline float as_float_bits(int i)
{
  float f;
  memcpy(&f, &i, 4);
  return f;
}

// device buffers freed together; the first failure is kept
struct DevBufs {
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  template <class T>
  T* alloc(size_t n)
  {
    void* p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (p) ptrs.push_back(p);
    return (T*)p;
  }
  ~DevBufs()
  {
    for (void* p : ptrs) cudaFree(p);
  }
};

}  // namespace

cudaError_t lbvh_build(const std::vector<double>& tri, const std::vector<int>& ids, const std::vector<int>& tri_obj,
                       HostBvh& out)
{
  out.nodes.clear();
  out.node_c64.clear();
  out.node_h64.clear();
  out.node_r.clear();
  out.node_obj.clear();
  out.order.clear();
  const int n = (int)ids.size();
  if (n == 0) return cudaSuccess;
  if (ids.size() >= (size_t)1 << 30) return cudaErrorInvalidValue;
  // objects of this group: dense local indices, centroid boxes, ranks
  std::vector<int> objs(n), local_obj(n);
  for (int k = 0; k < n; ++k) objs[k] = tri_obj[ids[k]];
  std::sort(objs.begin(), objs.end());
  objs.erase(std::unique(objs.begin(), objs.end()), objs.end());
  const int no = (int)objs.size();
  for (int k = 0; k < n; ++k)
    local_obj[k] = (int)(std::lower_bound(objs.begin(), objs.end(), tri_obj[ids[k]]) - objs.begin());
  std::vector<double> tri_g(9 * (size_t)n), clo(3 * (size_t)no, 1e300), chi(3 * (size_t)no, -1e300);
  for (int k = 0; k < n; ++k) {
    const double* T = &tri[9 * (size_t)ids[k]];
    memcpy(&tri_g[9 * (size_t)k], T, 9 * sizeof(double));
    const int o = local_obj[k];
    for (int a = 0; a < 3; ++a) {
      const double c = (T[a] + T[3 + a] + T[6 + a]) / 3.0;
      clo[3 * (size_t)o + a] = std::min(clo[3 * (size_t)o + a], c);
      chi[3 * (size_t)o + a] = std::max(chi[3 * (size_t)o + a], c);
    }
  }
  std::vector<double> ocen(3 * (size_t)no), oinv(3 * (size_t)no);
  double glo[3] = {1e300, 1e300, 1e300}, ghi[3] = {-1e300, -1e300, -1e300};
  for (int o = 0; o < no; ++o)
    for (int a = 0; a < 3; ++a) {
      const double lo = clo[3 * (size_t)o + a], hi = chi[3 * (size_t)o + a];
      ocen[3 * (size_t)o + a] = 0.5 * (lo + hi);
      oinv[3 * (size_t)o + a] = hi > lo ? 1.0 / (hi - lo) : 0.0;
      glo[a] = std::min(glo[a], ocen[3 * (size_t)o + a]);
      ghi[a] = std::max(ghi[a], ocen[3 * (size_t)o + a]);
    }
  std::vector<std::pair<uint64_t, int>> okey(no);
  for (int o = 0; o < no; ++o) {
    double u[3];
    for (int a = 0; a < 3; ++a)
      u[a] = ghi[a] > glo[a] ? (ocen[3 * (size_t)o + a] - glo[a]) / (ghi[a] - glo[a]) : 0.0;
    okey[o] = {((uint64_t)morton30(u[0], u[1], u[2]) << 32) | (uint32_t)o, o};
  }
  std::sort(okey.begin(), okey.end());
  std::vector<uint32_t> rank(no);
  for (int r = 0; r < no; ++r) rank[okey[r].second] = (uint32_t)r;

  // device: keys, sort, radix tree, boxes
  const int ni = std::max(n - 1, 1);
  std::vector<unsigned long long> keys(n);
  std::vector<int> vals(n), L(ni), Rr(ni), LO(ni), HI(ni);
  std::vector<double> lbox(6 * (size_t)n), ibox(6 * (size_t)ni);
  {
    DevBufs D;
    double* d_tri = D.alloc<double>(tri_g.size());
    double* d_olo = D.alloc<double>(clo.size());
    double* d_oinv = D.alloc<double>(oinv.size());
    int* d_obj = D.alloc<int>(n);
    uint32_t* d_rank = D.alloc<uint32_t>(no);
    unsigned long long* d_keys = D.alloc<unsigned long long>(n);
    unsigned long long* d_keys2 = D.alloc<unsigned long long>(n);
    int* d_vals = D.alloc<int>(n);
    int* d_vals2 = D.alloc<int>(n);
    int* d_l = D.alloc<int>(ni);
    int* d_r = D.alloc<int>(ni);
    int* d_lo = D.alloc<int>(ni);
    int* d_hi = D.alloc<int>(ni);
    int* d_pint = D.alloc<int>(ni);
    int* d_pleaf = D.alloc<int>(n);
    int* d_flags = D.alloc<int>(ni);
    double* d_lbox = D.alloc<double>(6 * (size_t)n);
    double* d_ibox = D.alloc<double>(6 * (size_t)ni);
    size_t tmp_bytes = 0;
    cudaError_t& e = D.err;
    auto chk = [&](cudaError_t x) {
      if (e == cudaSuccess) e = x;
    };
    chk(cudaMemcpy(d_tri, tri_g.data(), tri_g.size() * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(d_olo, clo.data(), clo.size() * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(d_oinv, oinv.data(), oinv.size() * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(d_obj, local_obj.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(d_rank, rank.data(), no * sizeof(uint32_t), cudaMemcpyHostToDevice));
    chk(cudaMemset(d_flags, 0, ni * sizeof(int)));
    if (e != cudaSuccess) return e;
    k_lbvh_keys<<<(n + 255) / 256, 256>>>(d_tri, d_obj, d_olo, d_oinv, d_rank, n, d_keys, d_vals);
    chk(cudaGetLastError());
    chk(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_keys, d_keys2, d_vals, d_vals2, n));
    void* d_tmp = D.alloc<char>(tmp_bytes);
    chk(cub::DeviceRadixSort::SortPairs(d_tmp, tmp_bytes, d_keys, d_keys2, d_vals, d_vals2, n));
    if (e != cudaSuccess) return e;
    if (n > 1) {
      k_lbvh_tree<<<(n - 1 + 255) / 256, 256>>>(d_keys2, n, d_l, d_r, d_lo, d_hi, d_pint, d_pleaf);
      chk(cudaGetLastError());
    }
    k_lbvh_boxes<<<(n + 255) / 256, 256>>>(d_tri, d_vals2, n, d_l, d_r, d_pint, d_pleaf, d_flags, d_lbox, d_ibox);
    chk(cudaGetLastError());
    chk(cudaMemcpy(keys.data(), d_keys2, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(vals.data(), d_vals2, n * sizeof(int), cudaMemcpyDeviceToHost));
    chk(cudaMemcpy(lbox.data(), d_lbox, lbox.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (n > 1) {
      chk(cudaMemcpy(L.data(), d_l, (n - 1) * sizeof(int), cudaMemcpyDeviceToHost));
      chk(cudaMemcpy(Rr.data(), d_r, (n - 1) * sizeof(int), cudaMemcpyDeviceToHost));
      chk(cudaMemcpy(LO.data(), d_lo, (n - 1) * sizeof(int), cudaMemcpyDeviceToHost));
      chk(cudaMemcpy(HI.data(), d_hi, (n - 1) * sizeof(int), cudaMemcpyDeviceToHost));
      chk(cudaMemcpy(ibox.data(), d_ibox, ibox.size() * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (e != cudaSuccess) return e;
  }

  // host relayout: breadth first, children in adjacent slots
  out.order.resize(n);
  for (int k = 0; k < n; ++k) out.order[k] = ids[vals[k]];
  struct Item { int code, slot; };  // code >= 0 internal node, < 0 leaf -1-position
  std::vector<Item> queue;
  queue.reserve(n);
  queue.push_back({n > 1 ? 0 : -1, 0});
  out.nodes.resize(1);
  out.node_c64.resize(3);
  out.node_h64.resize(3);
  out.node_r.resize(1);
  out.node_obj.resize(1);
  for (size_t qi = 0; qi < queue.size(); ++qi) {
    const Item it = queue[qi];
    const int lo = it.code < 0 ? -1 - it.code : LO[it.code];
    const int hi = it.code < 0 ? -1 - it.code : HI[it.code];
    const bool one_obj = (keys[lo] >> 32) == (keys[hi] >> 32);
    const double* bx = it.code < 0 ? &lbox[6 * (size_t)(-1 - it.code)] : &ibox[6 * (size_t)it.code];
    double c[3], h[3];
    float cf[3], hf[3];
    for (int a = 0; a < 3; ++a) {
      c[a] = 0.5 * (bx[a] + bx[3 + a]);
      h[a] = 0.5 * (bx[3 + a] - bx[a]);
      out.node_c64[3 * (size_t)it.slot + a] = c[a];
      out.node_h64[3 * (size_t)it.slot + a] = h[a];
      cf[a] = (float)c[a];
      // conservative FP32 half extent: covers the rounding of the centre
      hf[a] = round_up_f32(h[a] + std::fabs(c[a] - (double)cf[a]));
    }
    // the sphere about the box centre through its corners holds every vertex
    out.node_r[it.slot] = std::sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) * (1.0 + 1e-9) + 1e-12;
    out.node_obj[it.slot] = one_obj ? tri_obj[out.order[lo]] : -1;
    int index, count;
    if (it.code < 0 || (one_obj && hi - lo + 1 <= kLeafSize)) {
      index = lo;
      count = hi - lo + 1;
    } else {
      const int l = (int)out.nodes.size();
      out.nodes.resize(l + 2);
      out.node_c64.resize(3 * (size_t)(l + 2));
      out.node_h64.resize(3 * (size_t)(l + 2));
      out.node_r.resize(l + 2);
      out.node_obj.resize(l + 2);
      queue.push_back({L[it.code], l});
      queue.push_back({Rr[it.code], l + 1});
      index = l;
      count = 0;
    }
    out.nodes[it.slot].a = make_float4(cf[0], cf[1], cf[2], as_float_bits(index));
    out.nodes[it.slot].b = make_float4(hf[0], hf[1], hf[2], as_float_bits(count));
  }
  return cudaSuccess;
}

}  // namespace kgpu
