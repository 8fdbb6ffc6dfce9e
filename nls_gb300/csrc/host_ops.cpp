// host_ops.cpp -- operator construction on the host (no GPU needed).
//
// The band matrices are those of the reference's make_laplacian / make_laplacian_2d
// (nls/nls.f90:132-403) and must come out identical, entry for entry, in the same precision.
// They are produced here from one rule instead of the reference's sequence of band edits:
//   * the Toeplitz taps of D2 (second derivative) and D1 (first derivative) are laid onto each
//     row p; a tap that lands on a node q < 0 is folded onto its mirror image -q (u(-r) = u(r)
//     at the axis) and a tap beyond node n-1 is dropped (zero Dirichlet by truncation);
//   * row 0 (r = 0) keeps only the folded D2, doubled (the axial limit of u'' + u'/r is 2 u'');
//   * rows p >= 1 are D2 + D1 / (p h).
// Folding reproduces every near-axis edit of make_laplacian_o3/o5/o7 (nls/nls.f90:154-155,
// 185-189, 219-253) with identical rounding, because the folded additions are exact doublings or
// the same single addition the reference performs.
#include <cmath>
#include <cstring>
#include <vector>

#include "nls_types.h"

namespace nlsg {

// Integer taps of the central stencils (numerators), their denominators, in units of h and h^2.
static bool radial_taps(int order, int* K, const int** d1, const int** d2, int* den1, int* den2) {
  static const int o3_1[3] = {-1, 0, 1}, o3_2[3] = {1, -2, 1};
  static const int o5_1[5] = {1, -8, 0, 8, -1}, o5_2[5] = {-1, 16, -30, 16, -1};
  static const int o7_1[7] = {-1, 9, -45, 0, 45, -9, 1}, o7_2[7] = {2, -27, 270, -490, 270, -27, 2};
  // index d + K is the weight of u_{p+d}
  switch (order) {
    case 3: *K = 1; *d1 = o3_1; *d2 = o3_2; *den1 = 2; *den2 = 1; return true;
    case 5: *K = 2; *d1 = o5_1; *d2 = o5_2; *den1 = 12; *den2 = 12; return true;
    case 7: *K = 3; *d1 = o7_1; *d2 = o7_2; *den1 = 60; *den2 = 180; return true;
  }
  return false;
}

// Dense-row form: A(p, q) for |q - p| <= K; returns 0 or a status.
static int radial_rows(int n, int order, double h, std::vector<double>& rows /* n x (2K+1) */,
                       double* w1_out, double* w2_out) {
  int K, den1, den2;
  const int *t1, *t2;
  if (!radial_taps(order, &K, &t1, &t2, &den1, &den2)) return 2;
  if (n < 2 * K + 1) return 1;
  const double dx1 = (double)den1 * h, dx2 = (double)den2 * (h * h);
  double w1[7], w2[7];
  for (int i = 0; i < 2 * K + 1; ++i) { w1[i] = (double)t1[i] / dx1; w2[i] = (double)t2[i] / dx2; }
  if (w1_out) std::memcpy(w1_out, w1, sizeof(double) * (2 * K + 1));
  if (w2_out) std::memcpy(w2_out, w2, sizeof(double) * (2 * K + 1));
  const int W = 2 * K + 1;
  rows.assign((size_t)n * W, 0.0);
  std::vector<double> a1(W), a2(W);
  for (int p = 0; p < n; ++p) {
    std::fill(a1.begin(), a1.end(), 0.0);
    std::fill(a2.begin(), a2.end(), 0.0);
    for (int d = -K; d <= K; ++d) {
      int q = p + d;
      if (q < 0) q = -q;
      if (q >= n) continue;
      a2[q - p + K] += w2[d + K];
      a1[q - p + K] += w1[d + K];
    }
    for (int i = 0; i < W; ++i) {
      double v;
      if (p == 0) v = 2.0 * a2[i];
      else v = a1[i] / ((double)p * h) + a2[i];
      rows[(size_t)p * W + i] = v;
    }
  }
  return 0;
}

int host_make_laplacian(int n, int order, double h, double* op) {
  std::vector<double> rows;
  int st = radial_rows(n, order, h, rows, nullptr, nullptr);
  if (st) return st;
  const int K = (order - 1) / 2, W = 2 * K + 1;
  // band storage: op(K + p - q, q) = A(p, q), column-major (order, n)
  for (size_t i = 0; i < (size_t)order * n; ++i) op[i] = 0.0;
  for (int p = 0; p < n; ++p)
    for (int d = -K; d <= K; ++d) {
      int q = p + d;
      if (q < 0 || q >= n) continue;
      op[(size_t)(K - d) + (size_t)q * order] = rows[(size_t)p * W + d + K];
    }
  return 0;
}

int host_stencil_1d(int n, int order, double h, Stencil1D* s) {
  std::vector<double> rows;
  std::memset(s, 0, sizeof(*s));
  int st = radial_rows(n, order, h, rows, s->w1, s->w2);
  if (st) return st;
  s->order = order;
  s->K = (order - 1) / 2;
  s->h = h;
  const int W = 2 * s->K + 1;
  for (int p = 0; p < s->K; ++p)
    for (int i = 0; i < W; ++i) {
      const int q = p + i - s->K;
      s->near[p][i] = (q >= 0 && q < n) ? rows[(size_t)p * W + i] : 0.0;
    }
  for (int i = 0; i < 7; ++i) {
    s->w2f[i] = (float)s->w2[i];
    s->w1f[i] = (float)s->w1[i];
    for (int p = 0; p < 3; ++p) s->nearf[p][i] = (float)s->near[p][i];
  }
  return 0;
}

// 2-D cross stencil: the contiguous axis carries the full central stencil with both axes'
// centre terms (middle block); the other axis contributes scalar multiples of the identity at
// distances 1..K (left/right blocks).
int host_stencil_2d(int order, double h, Stencil2D* s) {
  std::memset(s, 0, sizeof(*s));
  if (order == 3) {
    const double dx2 = 1.0 * (h * h);
    s->order = 3; s->K = 1;
    s->center = -4.0 / dx2;
    s->w[0] = 1.0 / dx2;
    s->w[1] = 0.0;
    return 0;
  }
  if (order == 5) {
    const double dx2 = 12.0 * (h * h);
    s->order = 5; s->K = 2;
    s->center = -60.0 / dx2;
    s->w[0] = 16.0 / dx2;
    s->w[1] = -1.0 / dx2;
    return 0;
  }
  return 2;
}

// blocks (n, 2m-1) column-major: the reference's block pieces, each a band matrix of a constant
// row sequence-associated into consecutive columns (nls/nls.f90:316-318, 344-348).
int host_make_laplacian_2d(int n, int order, double h, double* blocks, int* orders) {
  Stencil2D s;
  int st = host_stencil_2d(order, h, &s);
  if (st) return st;
  if (n < order) return 1;
  const int m = order, K = s.K;
  for (size_t i = 0; i < (size_t)n * (2 * m - 1); ++i) blocks[i] = 0.0;
  // side blocks: one value per node
  auto fill_diag = [&](int first_col, double v) {
    for (int i = 0; i < n; ++i) blocks[(size_t)(first_col - 1) * n + i] = v;
  };
  // middle block: band matrix (m, n) of the row (w_K..w_1, center, w_1..w_K) at blocks(:, K+1..)
  double row[5];
  if (K == 1) { row[0] = s.w[0]; row[1] = s.center; row[2] = s.w[0]; }
  else { row[0] = s.w[1]; row[1] = s.w[0]; row[2] = s.center; row[3] = s.w[0]; row[4] = s.w[1]; }
  double* mid = blocks + (size_t)K * n;  // starts at column K+1 for o3 (col 2) / col 3 for o5
  for (int q = 0; q < n; ++q)
    for (int b = 0; b < m; ++b) {
      const int p = q + b - (m - 1) / 2;    // matrix row of band row b in column q
      mid[(size_t)q * m + b] = (p >= 0 && p < n) ? row[b] : 0.0;
    }
  if (K == 1) {
    fill_diag(1, s.w[0]);
    fill_diag(5, s.w[0]);
    orders[0] = 0; orders[1] = 1; orders[2] = 0;
  } else {
    fill_diag(1, s.w[1]);
    fill_diag(2, s.w[0]);
    fill_diag(8, s.w[0]);
    fill_diag(9, s.w[1]);
    orders[0] = 0; orders[1] = 0; orders[2] = 2; orders[3] = 0; orders[4] = 0;
  }
  return 0;
}

}  // namespace nlsg
