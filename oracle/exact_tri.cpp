// exact_tri.cpp — an independent, exact closed-triangle intersection test.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle library): it cross-checks the
// canonical FP64 separating-axis predicate (kx_tri_tri_overlap in
// include/kgpu_exact.h, the restatement of PQP's TriContact that decides
// every collision verdict of the engine and of the oracle) with a different
// method and exact arithmetic, so that a wrong axis or tie rule in the
// shared predicate cannot hide behind "GPU equals oracle".  This file does
// not include kgpu_exact.h.
//
// Method: two closed triangles P, Q intersect iff the linear system
//   a1 P1 + a2 P2 + a3 P3 - b1 Q1 - b2 Q2 - b3 Q3 = 0,
//   a1 + a2 + a3 = 1,   b1 + b2 + b3 = 1,   a, b >= 0
// (a common point in barycentric coordinates of both) is feasible.  A
// feasible system A x = c, x >= 0 has a basic feasible solution: one whose
// support S indexes linearly independent columns of A (the fundamental
// theorem of linear programming).  So the test enumerates the 62 nonempty
// column subsets S of size <= 5 (rank A <= 5), keeps those whose columns
// are independent and whose system A_S x_S = c is consistent, and accepts
// when the unique solution is non-negative.  All arithmetic is on integers
// (__int128): coordinates must be integers of magnitude <= 1024, so that
// every minor (at most 56 * 2048^5 after translating P1 to the origin) and
// every fraction-free elimination product fits in 127 bits.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

typedef __int128 i128;

// Determinant of the n x n integer matrix m (row-major, stride 6) by
// fraction-free (Bareiss) elimination with row pivoting; m is overwritten.
i128 det_bareiss(i128 m[5][6], int n)
{
  i128 prev = 1;
  int sign = 1;
  for (int k = 0; k < n; ++k) {
    int p = k;
    while (p < n && m[p][k] == 0) ++p;
    if (p == n) return 0;
    if (p != k) {
      for (int c = 0; c < n; ++c) std::swap(m[p][c], m[k][c]);
      sign = -sign;
    }
    for (int i = k + 1; i < n; ++i) {
      for (int j = k + 1; j < n; ++j) m[i][j] = (m[i][j] * m[k][k] - m[i][k] * m[k][j]) / prev;
      m[i][k] = 0;
    }
    prev = m[k][k];
  }
  return sign > 0 ? m[n - 1][n - 1] : -m[n - 1][n - 1];
}

int sgn(i128 v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

// Rank of the 5 x k matrix M (columns) and of [M | c]; picks k independent
// rows when rank M = k.
int rank_rows(const i128 M[5][5], int k, const i128 c[5], int rows[5], bool* consistent)
{
  // fraction-free elimination on a copy of [M | c], remembering the pivot rows
  i128 a[5][6];
  int id[5];
  for (int r = 0; r < 5; ++r) {
    for (int j = 0; j < k; ++j) a[r][j] = M[r][j];
    a[r][k] = c[r];
    id[r] = r;
  }
  i128 prev = 1;
  int rank = 0;
  for (int col = 0; col < k && rank < 5; ++col) {
    int p = rank;
    while (p < 5 && a[p][col] == 0) ++p;
    if (p == 5) return -1;  // column dependent on the previous ones
    if (p != rank) {
      for (int j = 0; j <= k; ++j) std::swap(a[p][j], a[rank][j]);
      std::swap(id[p], id[rank]);
    }
    for (int i = rank + 1; i < 5; ++i) {
      for (int j = col + 1; j <= k; ++j) a[i][j] = (a[i][j] * a[rank][col] - a[i][col] * a[rank][j]) / prev;
      a[i][col] = 0;
    }
    prev = a[rank][col];
    ++rank;
  }
  *consistent = true;
  for (int r = rank; r < 5; ++r)
    if (a[r][k] != 0) *consistent = false;
  for (int r = 0; r < rank; ++r) rows[r] = id[r];
  return rank;
}

bool intersect_exact(const int32_t* P, const int32_t* Q)
{
  // columns: P_i - P_1 (translated: the system is translation invariant) with
  // a 1 in row 3; -(Q_j - P_1) with a 1 in row 4
  i128 A[5][6];
  for (int i = 0; i < 3; ++i) {
    for (int r = 0; r < 3; ++r) {
      A[r][i] = (i128)P[3 * i + r] - P[r];
      A[r][3 + i] = -((i128)Q[3 * i + r] - P[r]);
    }
    A[3][i] = 1; A[4][i] = 0;
    A[3][3 + i] = 0; A[4][3 + i] = 1;
  }
  const i128 c[5] = {0, 0, 0, 1, 1};
  for (int S = 1; S < 64; ++S) {
    const int k = __builtin_popcount(S);
    if (k > 5) continue;
    // a point of both triangles needs some a > 0 and some b > 0
    if (!(S & 7) || !(S & 56)) continue;
    int cols[5], n = 0;
    for (int j = 0; j < 6; ++j)
      if (S >> j & 1) cols[n++] = j;
    i128 M[5][5];
    for (int r = 0; r < 5; ++r)
      for (int j = 0; j < k; ++j) M[r][j] = A[r][cols[j]];
    int rows[5];
    bool consistent = false;
    if (rank_rows(M, k, c, rows, &consistent) != k || !consistent) continue;
    // Cramer on the k independent rows: x_j = det(M_j) / det(M)
    i128 m[5][6];
    for (int r = 0; r < k; ++r)
      for (int j = 0; j < k; ++j) m[r][j] = M[rows[r]][j];
    const int sd = sgn(det_bareiss(m, k));
    if (sd == 0) continue;
    bool ok = true;
    for (int t = 0; t < k && ok; ++t) {
      for (int r = 0; r < k; ++r)
        for (int j = 0; j < k; ++j) m[r][j] = j == t ? c[rows[r]] : M[rows[r]][j];
      if (sgn(det_bareiss(m, k)) * sd < 0) ok = false;
    }
    if (ok) return true;
  }
  return false;
}

}  // namespace

extern "C" {

/* Exact intersection of n closed triangle pairs with integer coordinates of
 * magnitude <= 1024: P, Q [n * 9]; out[n] = 1 (intersect, touching
 * included) or 0.  Returns -1 if a coordinate is out of range. */
int orc_tri_tri_exact(const int32_t* P, const int32_t* Q, int n, uint8_t* out, int nthreads)
{
  for (long long i = 0; i < 9LL * n; ++i)
    if (P[i] < -1024 || P[i] > 1024 || Q[i] < -1024 || Q[i] > 1024) return -1;
  nthreads = std::max(1, std::min(nthreads, 64));
  std::atomic<int> next(0);
  auto work = [&]() {
    for (;;) {
      const int i0 = next.fetch_add(256);
      if (i0 >= n) break;
      for (int i = i0; i < std::min(n, i0 + 256); ++i)
        out[i] = intersect_exact(P + 9 * (size_t)i, Q + 9 * (size_t)i) ? 1 : 0;
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(work);
  work();
  for (auto& x : th) x.join();
  return 0;
}

}  // extern "C"
