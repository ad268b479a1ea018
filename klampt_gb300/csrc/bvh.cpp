// bvh.cpp — host BVH builder for link meshes and the environment.
//
// Replaces the PQP hierarchy that KrisLibrary builds when Klamp't calls
// InitCollisions (Cpp/Modeling/World.cpp:266-274,
// Python/klampt/src/robotsim.cpp:4118-4165).  Axis-aligned boxes, binary,
// binned surface-area split of the triangles (median split on the widest
// centroid axis where the bins cannot separate them), at most kLeafSize
// triangles per leaf, the two children of a node stored next to each other.
// Against the median split the surface-area trees halve the triangle pairs
// the edge checks test and cut the node pairs by 12%.  For the
// environment the top levels split whole objects first, so that every object
// owns one subtree: one tree then serves the collision traversal (which
// ignores object boundaries) and the per-object distance queries (which start
// at the object's subtree root).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "kgpu_internal.h"

namespace kgpu {

namespace {

inline float as_float(int i)
{
  float f;
  memcpy(&f, &i, 4);
  return f;
}

inline float round_up(double x)
{
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
  return f;
}

struct Builder {
  const std::vector<double>& tri;
  HostBvh& out;
  std::vector<double> cen;  // centroid per triangle id (3 doubles)

  Builder(const std::vector<double>& t, HostBvh& o) : tri(t), out(o) {}

  double centroid(int t, int i) const { return cen[3 * (size_t)t + i]; }

  void make_box(int node, const int* ids, int n)
  {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < n; ++k) {
      const double* T = &tri[9 * (size_t)ids[k]];
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < 3; ++i) {
          lo[i] = std::min(lo[i], T[3 * v + i]);
          hi[i] = std::max(hi[i], T[3 * v + i]);
        }
    }
    KNode& nd = out.nodes[node];
    double c[3], h[3];
    for (int i = 0; i < 3; ++i) {
      c[i] = 0.5 * (lo[i] + hi[i]);
      h[i] = 0.5 * (hi[i] - lo[i]);
      out.node_c64[3 * (size_t)node + i] = c[i];
      out.node_h64[3 * (size_t)node + i] = h[i];
    }
    double r2 = 0.0;
    for (int k = 0; k < n; ++k) {
      const double* T = &tri[9 * (size_t)ids[k]];
      for (int v = 0; v < 3; ++v) {
        double dx = T[3 * v] - c[0], dy = T[3 * v + 1] - c[1], dz = T[3 * v + 2] - c[2];
        r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
      }
    }
    out.node_r[node] = std::sqrt(r2) * (1.0 + 1e-9) + 1e-12;
    float cf[3], hf[3];
    for (int i = 0; i < 3; ++i) {
      cf[i] = (float)c[i];
      // conservative FP32 half extent: covers the rounding of the center
      hf[i] = round_up(h[i] + std::fabs(c[i] - (double)cf[i]));
    }
    nd.a = make_float4(cf[0], cf[1], cf[2], nd.a.w);
    nd.b = make_float4(hf[0], hf[1], hf[2], nd.b.w);
  }

  int alloc_pair()
  {
    int l = (int)out.nodes.size();
    out.nodes.resize(l + 2);
    out.node_c64.resize(3 * (size_t)(l + 2));
    out.node_h64.resize(3 * (size_t)(l + 2));
    out.node_r.resize(l + 2, 0.0);
    out.node_obj.resize(l + 2, -1);
    return l;
  }

  // Binned surface-area split of order[b, e): 16 bins per axis over the
  // centroid box, cost = area(left) * n(left) + area(right) * n(right) (the
  // expected number of node tests a box query makes below the node).
  // Returns the split position, or -1 when no split separates the bins.
  int sah_split(int b, int e, const double* clo, const double* chi)
  {
    constexpr int NB = 16;
    struct Bin { double lo[3], hi[3]; int n; };
    auto empty = [](Bin& x) {
      for (int i = 0; i < 3; ++i) { x.lo[i] = 1e300; x.hi[i] = -1e300; }
      x.n = 0;
    };
    auto area = [](const double* lo, const double* hi) {
      const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
      return dx * dy + dy * dz + dz * dx;
    };
    double best = 1e300;
    int best_ax = -1, best_bin = -1;
    for (int ax = 0; ax < 3; ++ax) {
      const double ext = chi[ax] - clo[ax];
      if (!(ext > 0)) continue;
      Bin bins[NB];
      for (int i = 0; i < NB; ++i) empty(bins[i]);
      for (int k = b; k < e; ++k) {
        const int t = out.order[k];
        int bi = (int)((centroid(t, ax) - clo[ax]) / ext * NB);
        bi = bi < 0 ? 0 : (bi >= NB ? NB - 1 : bi);
        Bin& x = bins[bi];
        const double* T = &tri[9 * (size_t)t];
        for (int v = 0; v < 3; ++v)
          for (int i = 0; i < 3; ++i) {
            x.lo[i] = std::min(x.lo[i], T[3 * v + i]);
            x.hi[i] = std::max(x.hi[i], T[3 * v + i]);
          }
        x.n++;
      }
      double rA[NB];
      int rN[NB];
      Bin acc;
      empty(acc);
      for (int i = NB - 1; i >= 0; --i) {
        for (int d = 0; d < 3; ++d) {
          acc.lo[d] = std::min(acc.lo[d], bins[i].lo[d]);
          acc.hi[d] = std::max(acc.hi[d], bins[i].hi[d]);
        }
        acc.n += bins[i].n;
        rA[i] = acc.n ? area(acc.lo, acc.hi) : 0.0;
        rN[i] = acc.n;
      }
      empty(acc);
      for (int i = 1; i < NB; ++i) {
        for (int d = 0; d < 3; ++d) {
          acc.lo[d] = std::min(acc.lo[d], bins[i - 1].lo[d]);
          acc.hi[d] = std::max(acc.hi[d], bins[i - 1].hi[d]);
        }
        acc.n += bins[i - 1].n;
        if (acc.n == 0 || rN[i] == 0) continue;
        const double cost = area(acc.lo, acc.hi) * acc.n + rA[i] * rN[i];
        if (cost < best) { best = cost; best_ax = ax; best_bin = i; }
      }
    }
    if (best_ax < 0) return -1;
    const double ext = chi[best_ax] - clo[best_ax];
    auto it = std::partition(out.order.begin() + b, out.order.begin() + e, [&](int t) {
      int bi = (int)((centroid(t, best_ax) - clo[best_ax]) / ext * NB);
      bi = bi < 0 ? 0 : (bi >= NB ? NB - 1 : bi);
      return bi < best_bin;
    });
    const int mid = (int)(it - out.order.begin());
    return (mid > b && mid < e) ? mid : -1;
  }

  // triangle-level subtree over order[b, e)
  void build_tris(int root, int b, int e, int obj)
  {
    struct Job { int node, b, e; };
    std::vector<Job> st{{root, b, e}};
    while (!st.empty()) {
      Job j = st.back();
      st.pop_back();
      out.node_obj[j.node] = obj;
      make_box(j.node, &out.order[j.b], j.e - j.b);
      KNode& nd = out.nodes[j.node];
      if (j.e - j.b <= kLeafSize) {
        nd.a.w = as_float(j.b);
        nd.b.w = as_float(j.e - j.b);
        continue;
      }
      double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
      for (int k = j.b; k < j.e; ++k)
        for (int i = 0; i < 3; ++i) {
          clo[i] = std::min(clo[i], centroid(out.order[k], i));
          chi[i] = std::max(chi[i], centroid(out.order[k], i));
        }
      int mid = sah_split(j.b, j.e, clo, chi);
      if (mid < 0) {
        int ax = 0;
        for (int i = 1; i < 3; ++i)
          if (chi[i] - clo[i] > chi[ax] - clo[ax]) ax = i;
        mid = (j.b + j.e) / 2;
        std::nth_element(out.order.begin() + j.b, out.order.begin() + mid, out.order.begin() + j.e,
                         [&](int x, int y) {
                           double kx = centroid(x, ax), ky = centroid(y, ax);
                           return kx < ky || (kx == ky && x < y);
                         });
      }
      int l = alloc_pair();
      KNode& nd2 = out.nodes[j.node];  // re-fetch after resize
      nd2.a.w = as_float(l);
      nd2.b.w = as_float(0);
      st.push_back({l + 1, mid, j.e});
      st.push_back({l, j.b, mid});
    }
  }
};

}  // namespace

void build_bvh(const std::vector<double>& tri, const std::vector<int>& ids,
               const std::vector<int>* tri_obj, HostBvh& out)
{
  out.nodes.clear();
  out.node_c64.clear();
  out.node_h64.clear();
  out.node_r.clear();
  out.node_obj.clear();
  out.order.clear();
  if (ids.empty()) return;
  Builder B(tri, out);
  int maxid = *std::max_element(ids.begin(), ids.end());
  B.cen.assign(3 * (size_t)(maxid + 1), 0.0);
  for (int t : ids)
    for (int i = 0; i < 3; ++i)
      B.cen[3 * (size_t)t + i] =
          (tri[9 * (size_t)t + i] + tri[9 * (size_t)t + 3 + i] + tri[9 * (size_t)t + 6 + i]) / 3.0;
  out.nodes.resize(1);
  out.node_c64.resize(3);
  out.node_h64.resize(3);
  out.node_r.assign(1, 0.0);
  out.node_obj.assign(1, -1);
  if (!tri_obj) {
    out.order = ids;
    B.build_tris(0, 0, (int)ids.size(), -1);
    return;
  }
  // group triangle ids by object (stable), then split objects at the top
  std::vector<int> sorted = ids;
  std::stable_sort(sorted.begin(), sorted.end(),
                   [&](int a, int b) { return (*tri_obj)[a] < (*tri_obj)[b]; });
  struct Obj { int id, b, e; double c[3]; };
  std::vector<Obj> objs;
  for (size_t k = 0; k < sorted.size();) {
    size_t m = k;
    int o = (*tri_obj)[sorted[k]];
    while (m < sorted.size() && (*tri_obj)[sorted[m]] == o) ++m;
    Obj ob;
    ob.id = o;
    ob.b = (int)k;
    ob.e = (int)m;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t t = k; t < m; ++t)
      for (int i = 0; i < 3; ++i) {
        lo[i] = std::min(lo[i], B.centroid(sorted[t], i));
        hi[i] = std::max(hi[i], B.centroid(sorted[t], i));
      }
    for (int i = 0; i < 3; ++i) ob.c[i] = 0.5 * (lo[i] + hi[i]);
    objs.push_back(ob);
    k = m;
  }
  // object-level recursion; the leaf order concatenates objects in the order
  // the recursion reaches them
  out.order.clear();
  out.order.reserve(sorted.size());
  struct Job { int node, b, e; };
  std::vector<Job> st{{0, 0, (int)objs.size()}};
  std::vector<int> tmp;
  while (!st.empty()) {
    Job j = st.back();
    st.pop_back();
    if (j.e - j.b == 1) {
      const Obj& ob = objs[j.b];
      int b = (int)out.order.size();
      for (int t = ob.b; t < ob.e; ++t) out.order.push_back(sorted[t]);
      B.build_tris(j.node, b, (int)out.order.size(), ob.id);
      continue;
    }
    // box over every triangle of the objects in range
    tmp.clear();
    for (int k = j.b; k < j.e; ++k)
      for (int t = objs[k].b; t < objs[k].e; ++t) tmp.push_back(sorted[t]);
    B.make_box(j.node, tmp.data(), (int)tmp.size());
    out.node_obj[j.node] = -1;
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int k = j.b; k < j.e; ++k)
      for (int i = 0; i < 3; ++i) {
        clo[i] = std::min(clo[i], objs[k].c[i]);
        chi[i] = std::max(chi[i], objs[k].c[i]);
      }
    int ax = 0;
    for (int i = 1; i < 3; ++i)
      if (chi[i] - clo[i] > chi[ax] - clo[ax]) ax = i;
    int mid = (j.b + j.e) / 2;
    std::nth_element(objs.begin() + j.b, objs.begin() + mid, objs.begin() + j.e,
                     [&](const Obj& x, const Obj& y) {
                       return x.c[ax] < y.c[ax] || (x.c[ax] == y.c[ax] && x.id < y.id);
                     });
    int l = B.alloc_pair();
    out.nodes[j.node].a.w = as_float(l);
    out.nodes[j.node].b.w = as_float(0);
    st.push_back({l + 1, mid, j.e});
    st.push_back({l, j.b, mid});
  }
}

}  // namespace kgpu
