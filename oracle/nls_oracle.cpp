// nls_oracle.cpp -- CPU restatement of the nls time-stepping path (TEST INFRASTRUCTURE).
//
// This file is the parity oracle.  It is test infrastructure only: the test suite, the smoke check
// and the CPU-baseline leg of the benchmark load it as a checker or as the timed CPU reference.
// The shipped solver (nls_gb300/) never links, loads or calls it.
//
// It restates, in C++ templated on the floating-point type, the algorithm of the reference module
// `nls` in nls/nls.f90 (daskol/nls 0.2.0):
//   make_banded_matrix               nls/nls.f90:61-91
//   clear_first_row_of_derivative    nls/nls.f90:93-107
//   divide_derivative_on_radius      nls/nls.f90:109-130
//   make_laplacian_o3/o5/o7          nls/nls.f90:132-259, dispatcher :278-295
//   make_laplacian_2d_o3/o5          nls/nls.f90:297-351, dispatcher :388-403
//   rgbmv -> BLAS ?gbmv('N')         nls/nls.f90:530-541 (reference-BLAS column loop)
//   rbbmv_o3/o5                      nls/nls.f90:408-466
//   revervoir[_2d]                   nls/nls.f90:570-581, 829-839
//   hamiltonian[_2d]                 nls/nls.f90:621-650, 841-870
//   runge_kutta[_2d]                 nls/nls.f90:705-734, 873-901
//   solve_nls / solve_nls_2d         nls/nls.f90:797-813, 903-919
//   chemical_potential_1d/2d         nls/nls.f90:921-971
//
// Parity pins: the band-storage and banded-matvec known answers of test/test_nls.f95:36-76 and
// :151-202, and a second restatement that calls scipy's ?gbmv (the BLAS routine the reference
// links) for small sizes.  No end-to-end golden output of the Fortran exists, and no Fortran
// compiler is available to produce one, so end-to-end parity is pinned by these restatements.
//
// Layouts follow the Fortran module exactly: band matrices are column-major (m, n); 2-D fields
// are column-major (n, n) with the first index contiguous; complex values are interleaved
// (re, im) pairs as in complex(kind=4/8).  The 2-D order-7 operator is not restated: the
// reference declares its block array with the wrong leading dimension (nls/nls.f90:360) and
// writes out of bounds for n > 7, so it has no defined result.
//
// Evaluation order follows the Fortran source statement by statement.  OpenMP (when compiled
// with -fopenmp and threads > 1) splits loops over independent rows/columns only, which keeps
// every element's sequence of floating-point operations identical to the single-thread order.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- operator construction

// Band storage of the Toeplitz matrix A(i, i+d) = row(k+1-d), truncated at the edges;
// mat(k+1+i-j, j) = A(i, j) in 1-based Fortran indices (nls/nls.f90:61-91).
template <typename T>
void make_banded_matrix(int n, int m, const T* row, T* mat) {
  const int k = (m - 1) / 2;
  auto M = [&](int i, int j) -> T& { return mat[(i - 1) + (size_t)(j - 1) * m]; };
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= m; ++i) M(i, j) = T(0);
  for (int j = 1; j <= k && j <= n; ++j) {          // left triangle
    for (int i = k + 2 - j; i <= m; ++i) M(i, j) = row[i - 1];
  }
  for (int j = k + 1; j <= n - k; ++j) {            // body
    for (int i = 1; i <= m; ++i) M(i, j) = row[i - 1];
  }
  for (int j = 1; j <= k; ++j) {                    // right triangle
    int col = n - k + j;
    if (col < 1) continue;
    for (int i = 1; i <= m - j; ++i) M(i, col) = row[i - 1];
    for (int i = m - j + 1; i <= m; ++i) M(i, col) = T(0);
  }
}

// nls/nls.f90:93-107: zero the band entries of matrix row 1 (node 0) of the first derivative.
template <typename T>
void clear_first_row_of_derivative(int n, int m, T* L1) {
  for (int i = 1; i <= (m + 1) / 2; ++i) {
    int j = (m + 1) / 2 - i + 1;
    if (j <= n) L1[(i - 1) + (size_t)(j - 1) * m] = T(0);
  }
}

// nls/nls.f90:109-130: divide matrix row p (0-based node index p = i + j - (m+3)/2) by p*h.
template <typename T>
void divide_derivative_on_radius(int n, int m, T h, T* L1) {
  for (int i = 1; i <= m; ++i)
    for (int j = 1; j <= n; ++j) {
      int row = i + j - (m + 3) / 2;
      if (row > 0) {
        T& v = L1[(i - 1) + (size_t)(j - 1) * m];
        v = v / (T(row) * h);
      }
    }
}

template <typename T>
void finish_radial(int n, int m, T h, std::vector<T>& L1, const std::vector<T>& L2, T* op) {
  clear_first_row_of_derivative<T>(n, m, L1.data());
  divide_derivative_on_radius<T>(n, m, h, L1.data());
  for (size_t q = 0; q < (size_t)m * n; ++q) op[q] = L1[q] + L2[q];
}

// nls/nls.f90:132-161
template <typename T>
void make_laplacian_o3(int n, T h, T* op) {
  const int m = 3;
  T dx1 = T(2) * h, dx2 = T(1) * (h * h);
  T row1d[3] = {T(1) / dx1, T(0) / dx1, T(-1) / dx1};
  T row2d[3] = {T(1) / dx2, T(-2) / dx2, T(1) / dx2};
  std::vector<T> L1((size_t)m * n), L2((size_t)m * n);
  make_banded_matrix<T>(n, m, row1d, L1.data());
  make_banded_matrix<T>(n, m, row2d, L2.data());
  auto A = [&](std::vector<T>& L, int i, int j) -> T& { return L[(i - 1) + (size_t)(j - 1) * m]; };
  A(L2, 2, 1) = T(2) * A(L2, 2, 1);
  if (n >= 2) A(L2, 1, 2) = T(4) * A(L2, 1, 2);
  finish_radial<T>(n, m, h, L1, L2, op);
}

// nls/nls.f90:163-195
template <typename T>
void make_laplacian_o5(int n, T h, T* op) {
  const int m = 5;
  T dx1 = T(12) * h, dx2 = T(12) * (h * h);
  const int r1[5] = {-1, 8, 0, -8, 1}, r2[5] = {-1, 16, -30, 16, -1};
  T row1d[5], row2d[5];
  for (int i = 0; i < 5; ++i) { row1d[i] = T(r1[i]) / dx1; row2d[i] = T(r2[i]) / dx2; }
  std::vector<T> L1((size_t)m * n), L2((size_t)m * n);
  make_banded_matrix<T>(n, m, row1d, L1.data());
  make_banded_matrix<T>(n, m, row2d, L2.data());
  auto A = [&](std::vector<T>& L, int i, int j) -> T& { return L[(i - 1) + (size_t)(j - 1) * m]; };
  if (n >= 2) {
    A(L1, 3, 2) = A(L1, 3, 2) + T(1) / dx1;
    A(L2, 3, 2) = A(L2, 3, 2) - T(1) / dx2;
    A(L2, 2, 2) = T(4) * A(L2, 2, 2);
  }
  A(L2, 3, 1) = T(2) * A(L2, 3, 1);
  if (n >= 3) A(L2, 1, 3) = T(4) * A(L2, 1, 3);
  finish_radial<T>(n, m, h, L1, L2, op);
}

// nls/nls.f90:197-259 (statements that only copy an entry onto itself are omitted)
template <typename T>
void make_laplacian_o7(int n, T h, T* op) {
  const int m = 7;
  T dx1 = T(60) * h, dx2 = T(180) * (h * h);
  const int r1[7] = {1, -9, 45, 0, -45, 9, -1}, r2[7] = {2, -27, 270, -490, 270, -27, 2};
  T row1d[7], row2d[7];
  for (int i = 0; i < 7; ++i) { row1d[i] = T(r1[i]) / dx1; row2d[i] = T(r2[i]) / dx2; }
  std::vector<T> L1((size_t)m * n), L2((size_t)m * n);
  make_banded_matrix<T>(n, m, row1d, L1.data());
  make_banded_matrix<T>(n, m, row2d, L2.data());
  auto A = [&](std::vector<T>& L, int i, int j) -> T& { return L[(i - 1) + (size_t)(j - 1) * m]; };
  // Reference requires n >= 7 for these band positions to be inside the matrix.
  A(L1, 4, 2) = A(L1, 4, 2) + T(9) / dx1;
  A(L1, 3, 3) = A(L1, 3, 3) - T(1) / dx1;
  A(L1, 5, 2) = A(L1, 5, 2) - T(1) / dx1;
  A(L2, 4, 1) = T(2) * A(L2, 4, 1);
  A(L2, 3, 2) = T(4) * A(L2, 3, 2);
  A(L2, 2, 3) = T(4) * A(L2, 2, 3);
  A(L2, 1, 4) = T(4) * A(L2, 1, 4);
  A(L2, 4, 2) = A(L2, 4, 2) - T(27) / dx2;
  A(L2, 3, 3) = A(L2, 3, 3) + T(2) / dx2;
  A(L2, 5, 2) = A(L2, 5, 2) + T(2) / dx2;
  finish_radial<T>(n, m, h, L1, L2, op);
}

template <typename T>
int make_laplacian(int n, int order, T h, T* op) {
  if (n < 1) return 1;
  if (order == 3) { make_laplacian_o3<T>(n, h, op); return 0; }
  if (order == 5) { if (n < 3) return 1; make_laplacian_o5<T>(n, h, op); return 0; }
  if (order == 7) { if (n < 7) return 1; make_laplacian_o7<T>(n, h, op); return 0; }
  return 2;
}

// nls/nls.f90:297-351.  blocks is (n, 2m-1) column-major; each band piece is the sub-array
// blocks(:, a:b) sequence-associated as a (b-a+1, n) band matrix.
template <typename T>
int make_laplacian_2d(int n, int order, T h, T* blocks, int* orders) {
  if (n < 1) return 1;
  if (order == 3) {
    T dx2 = T(1) * (h * h);
    T left[1] = {T(1) / dx2}, right[1] = {T(1) / dx2};
    T middle[3] = {T(1) / dx2, T(-4) / dx2, T(1) / dx2};
    make_banded_matrix<T>(n, 1, left, blocks + 0 * (size_t)n);
    make_banded_matrix<T>(n, 3, middle, blocks + 1 * (size_t)n);
    make_banded_matrix<T>(n, 1, right, blocks + 4 * (size_t)n);
    orders[0] = 0; orders[1] = 1; orders[2] = 0;
    return 0;
  }
  if (order == 5) {
    if (n < 3) return 1;
    T dx2 = T(12) * (h * h);
    T left2[1] = {T(-1) / dx2}, left1[1] = {T(16) / dx2};
    T right1[1] = {T(16) / dx2}, right2[1] = {T(-1) / dx2};
    const int mid[5] = {-1, 16, -60, 16, -1};
    T middle[5];
    for (int i = 0; i < 5; ++i) middle[i] = T(mid[i]) / dx2;
    make_banded_matrix<T>(n, 1, left2, blocks + 0 * (size_t)n);
    make_banded_matrix<T>(n, 1, left1, blocks + 1 * (size_t)n);
    make_banded_matrix<T>(n, 5, middle, blocks + 2 * (size_t)n);
    make_banded_matrix<T>(n, 1, right1, blocks + 7 * (size_t)n);
    make_banded_matrix<T>(n, 1, right2, blocks + 8 * (size_t)n);
    orders[0] = 0; orders[1] = 0; orders[2] = 2; orders[3] = 0; orders[4] = 0;
    return 0;
  }
  return 2;
}

// ---------------------------------------------------------------- banded matvec

// y := y + alpha*A*x for a square band matrix with kl = ku = klu in BLAS band storage
// (nls/nls.f90:530-541 -> ?gbmv('N', n, n, klu, klu, alpha, a, 2klu+1, x, 1, 1.0, y, 1)).
// The reference-BLAS loop visits columns j in increasing order and adds temp*a into y(i); for
// any fixed i that is the same sequence of operations as the row loop below, which is what lets
// rows be split across threads without changing a single rounding.
template <typename T>
void gbmv_rows(int n, int klu, T alpha, const T* a, const T* x, T* y, int i_begin, int i_end) {
  const int lda = 2 * klu + 1;
  for (int i = i_begin; i < i_end; ++i) {                 // 0-based row
    int jlo = i - klu < 0 ? 0 : i - klu;
    int jhi = i + klu > n - 1 ? n - 1 : i + klu;
    T acc = y[i];
    for (int j = jlo; j <= jhi; ++j) {
      T temp = alpha * x[j];
      acc = acc + temp * a[(klu + i - j) + (size_t)j * lda];
    }
    y[i] = acc;
  }
}

template <typename T>
void gbmv(int n, int klu, T alpha, const T* a, const T* x, T* y) {
  gbmv_rows<T>(n, klu, alpha, a, x, y, 0, n);
}

// nls/nls.f90:408-466, one output column at a time (x_c, y_c are column c of the n x n field).
// The contributions for a column arrive in exactly the order the reference's loops produce.
template <typename T>
void rbbmv_column(int n, int order, const T* blocks, T sign, const T* x, T* y, int c) {
  const T* xc = x + (size_t)c * n;
  T* yc = y + (size_t)c * n;
  auto blk = [&](int first_col) { return blocks + (size_t)(first_col - 1) * n; };
  if (order == 3) {
    if (c >= 1) gbmv<T>(n, 0, sign, blk(1), xc - n, yc);          // do i = 2, n
    gbmv<T>(n, 1, sign, blk(2), xc, yc);                         // do i = 1, n
    if (c <= n - 2) gbmv<T>(n, 0, sign, blk(5), xc + n, yc);     // do i = 1, n - 1
  } else {  // order 5
    if (c <= n - 3) gbmv<T>(n, 0, sign, blk(9), xc + 2 * (size_t)n, yc);
    if (c <= n - 2) gbmv<T>(n, 0, sign, blk(8), xc + n, yc);
    gbmv<T>(n, 2, sign, blk(3), xc, yc);
    if (c >= 1) gbmv<T>(n, 0, sign, blk(2), xc - n, yc);
    if (c >= 2) gbmv<T>(n, 0, sign, blk(1), xc - 2 * (size_t)n, yc);
  }
}

// ---------------------------------------------------------------- right-hand side

// Pointwise part of hamiltonian (nls/nls.f90:637-644 with revervoir :580).
// c is the 23-vector with 0-based index = Fortran index - 1.
template <typename T>
inline void pointwise(const T* c, T p, T ur, T ui, T& vr, T& vi) {
  T s = ur * ur + ui * ui;
  T r = c[11] * p / (c[12] + c[13] * s);
  T a = c[2] * r - c[3];
  T b = c[4] * s + c[5] * r;
  vr = a * ur + b * ui;
  vi = a * ui - b * ur;
}

template <typename T>
struct Work {
  std::vector<T> ur, ui, vr, vi;
  explicit Work(size_t N) : ur(N), ui(N), vr(N), vi(N) {}
};

// nls/nls.f90:621-650; u, v interleaved complex of length n.
template <typename T>
void hamiltonian_1d(int n, int order, const T* op, const T* P, const T* c, const T* u, T* v,
                    Work<T>& w, int threads) {
  const int klu = (order - 1) / 2;
  (void)threads;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
  for (int i = 0; i < n; ++i) {
    w.ur[i] = u[2 * i];
    w.ui[i] = u[2 * i + 1];
    pointwise<T>(c, P[i], w.ur[i], w.ui[i], w.vr[i], w.vi[i]);
  }
  const int chunk = 1024;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
  for (int b = 0; b < (n + chunk - 1) / chunk; ++b) {
    int lo = b * chunk, hi = lo + chunk < n ? lo + chunk : n;
    gbmv_rows<T>(n, klu, T(-1), op, w.ui.data(), w.vr.data(), lo, hi);
    gbmv_rows<T>(n, klu, T(+1), op, w.ur.data(), w.vi.data(), lo, hi);
  }
  for (int i = 0; i < n; ++i) { v[2 * i] = w.vr[i]; v[2 * i + 1] = w.vi[i]; }
}

// nls/nls.f90:841-870; fields column-major (n, n).
template <typename T>
void hamiltonian_2d(int n, int order, const T* blocks, const T* P, const T* c, const T* u, T* v,
                    Work<T>& w, int threads) {
  const size_t N = (size_t)n * n;
  (void)threads;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
  for (long q = 0; q < (long)N; ++q) {
    w.ur[q] = u[2 * q];
    w.ui[q] = u[2 * q + 1];
    pointwise<T>(c, P[q], w.ur[q], w.ui[q], w.vr[q], w.vi[q]);
  }
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
  for (int col = 0; col < n; ++col) {
    rbbmv_column<T>(n, order, blocks, T(-1), w.ui.data(), w.vr.data(), col);
    rbbmv_column<T>(n, order, blocks, T(+1), w.ur.data(), w.vi.data(), col);
  }
  for (size_t q = 0; q < N; ++q) { v[2 * q] = w.vr[q]; v[2 * q + 1] = w.vi[q]; }
}

// Classical RK4 of nls/nls.f90:705-734 / :873-901, including the operation order of
// `u + k*dt/2` and `u + (k1 + 2*k2 + 2*k3 + k4)*dt/6`.
template <typename T, typename H>
void runge_kutta(size_t N, T dt, int iters, const T* u0, T* u, H&& ham) {
  std::vector<T> k1(2 * N), k2(2 * N), k3(2 * N), k4(2 * N), tmp(2 * N);
  std::memcpy(u, u0, sizeof(T) * 2 * N);
  for (int it = 0; it < iters; ++it) {
    for (size_t q = 0; q < 2 * N; ++q) tmp[q] = u[q] + T(0) * dt / T(2);
    ham(tmp.data(), k1.data());
    for (size_t q = 0; q < 2 * N; ++q) tmp[q] = u[q] + k1[q] * dt / T(2);
    ham(tmp.data(), k2.data());
    for (size_t q = 0; q < 2 * N; ++q) tmp[q] = u[q] + k2[q] * dt / T(2);
    ham(tmp.data(), k3.data());
    for (size_t q = 0; q < 2 * N; ++q) tmp[q] = u[q] + k3[q] * dt / T(1);
    ham(tmp.data(), k4.data());
    for (size_t q = 0; q < 2 * N; ++q)
      u[q] = u[q] + (k1[q] + T(2) * k2[q] + T(2) * k3[q] + k4[q]) * dt / T(6);
  }
}

template <typename T>
int solve_1d(T dt, T dx, int n, int order, int iters, const T* P, const T* c, const T* u0, T* u,
             int threads) {
  std::vector<T> op((size_t)order * n);
  int st = make_laplacian<T>(n, order, dx, op.data());
  if (st) return st;
  Work<T> w(n);
  runge_kutta<T>((size_t)n, dt, iters, u0, u, [&](const T* x, T* y) {
    hamiltonian_1d<T>(n, order, op.data(), P, c, x, y, w, threads);
  });
  return 0;
}

template <typename T>
int solve_2d(T dt, T dx, int n, int order, int iters, const T* P, const T* c, const T* u0, T* u,
             int threads) {
  if (order != 3 && order != 5) return 2;
  std::vector<T> blocks((size_t)n * (2 * order - 1));
  std::vector<int> orders(order);
  int st = make_laplacian_2d<T>(n, order, dx, blocks.data(), orders.data());
  if (st) return st;
  Work<T> w((size_t)n * n);
  runge_kutta<T>((size_t)n * n, dt, iters, u0, u, [&](const T* x, T* y) {
    hamiltonian_2d<T>(n, order, blocks.data(), P, c, x, y, w, threads);
  });
  return 0;
}

// nls/nls.f90:921-948: mu = i <u0, H u0 * r> / <u0, u0 * r>, r_i = (i-1) dx, order 5.
template <typename T>
int chemical_potential_1d(T dx, int n, const T* P, const T* c, const T* u0, T* mu) {
  std::vector<T> op((size_t)5 * n), v(2 * (size_t)n);
  int st = make_laplacian<T>(n, 5, dx, op.data());
  if (st) return st;
  Work<T> w(n);
  hamiltonian_1d<T>(n, 5, op.data(), P, c, u0, v.data(), w, 1);
  T Mr = 0, Mi = 0, Er = 0, Ei = 0;
  for (int i = 0; i < n; ++i) {
    T r = (T(i + 1) - T(1)) * dx;
    T ar = u0[2 * i], ai = -u0[2 * i + 1];                 // conjg(u0)
    T br = u0[2 * i] * r, bi = u0[2 * i + 1] * r;          // u0 * r
    Mr += ar * br - ai * bi; Mi += ar * bi + ai * br;
    T cr = v[2 * i] * r, ci = v[2 * i + 1] * r;            // u * r
    Er += ar * cr - ai * ci; Ei += ar * ci + ai * cr;
  }
  T Er2 = -Ei, Ei2 = Er;                                    // (0, 1) * E
  T den = Mr * Mr + Mi * Mi;
  mu[0] = (Er2 * Mr + Ei2 * Mi) / den;
  mu[1] = (Ei2 * Mr - Er2 * Mi) / den;
  return 0;
}

// nls/nls.f90:950-971: mu = real(i <u0, H u0> / <u0, u0>), order 5.
template <typename T>
int chemical_potential_2d(T dx, int n, const T* P, const T* c, const T* u0, T* mu) {
  const size_t N = (size_t)n * n;
  std::vector<T> blocks((size_t)n * 9), v(2 * N);
  int orders[5];
  int st = make_laplacian_2d<T>(n, 5, dx, blocks.data(), orders);
  if (st) return st;
  Work<T> w(N);
  hamiltonian_2d<T>(n, 5, blocks.data(), P, c, u0, v.data(), w, 1);
  T Mr = 0, Mi = 0, Er = 0, Ei = 0;
  for (size_t q = 0; q < N; ++q) {
    T ar = u0[2 * q], ai = -u0[2 * q + 1];
    Mr += ar * u0[2 * q] - ai * u0[2 * q + 1];
    Mi += ar * u0[2 * q + 1] + ai * u0[2 * q];
    Er += ar * v[2 * q] - ai * v[2 * q + 1];
    Ei += ar * v[2 * q + 1] + ai * v[2 * q];
  }
  T Er2 = -Ei, Ei2 = Er;
  T den = Mr * Mr + Mi * Mi;
  *mu = (Er2 * Mr + Ei2 * Mi) / den;
  return 0;
}

}  // namespace

// ---------------------------------------------------------------- C entry points (ctypes)

#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

#define ORC_DEFINE(SFX, T)                                                                        \
  ORC_EXPORT void orc_make_banded_matrix_##SFX(int n, int m, const T* row, T* mat) {              \
    make_banded_matrix<T>(n, m, row, mat);                                                        \
  }                                                                                               \
  ORC_EXPORT int orc_make_laplacian_##SFX(int n, int order, T h, T* op) {                         \
    return make_laplacian<T>(n, order, h, op);                                                    \
  }                                                                                               \
  ORC_EXPORT int orc_make_laplacian_2d_##SFX(int n, int order, T h, T* blocks, int* orders) {     \
    return make_laplacian_2d<T>(n, order, h, blocks, orders);                                     \
  }                                                                                               \
  ORC_EXPORT void orc_gbmv_##SFX(int n, int klu, T alpha, const T* a, const T* x, T* y) {         \
    gbmv<T>(n, klu, alpha, a, x, y);                                                              \
  }                                                                                               \
  ORC_EXPORT int orc_hamiltonian_1d_##SFX(int n, int order, T dx, const T* P, const T* c,         \
                                          const T* u, T* v) {                                     \
    std::vector<T> op((size_t)order * n);                                                         \
    int st = make_laplacian<T>(n, order, dx, op.data());                                          \
    if (st) return st;                                                                            \
    Work<T> w(n);                                                                                 \
    hamiltonian_1d<T>(n, order, op.data(), P, c, u, v, w, 1);                                     \
    return 0;                                                                                     \
  }                                                                                               \
  ORC_EXPORT int orc_hamiltonian_2d_##SFX(int n, int order, T dx, const T* P, const T* c,         \
                                          const T* u, T* v) {                                     \
    if (order != 3 && order != 5) return 2;                                                       \
    std::vector<T> blocks((size_t)n * (2 * order - 1));                                           \
    std::vector<int> orders(order);                                                               \
    int st = make_laplacian_2d<T>(n, order, dx, blocks.data(), orders.data());                    \
    if (st) return st;                                                                            \
    Work<T> w((size_t)n * n);                                                                     \
    hamiltonian_2d<T>(n, order, blocks.data(), P, c, u, v, w, 1);                                 \
    return 0;                                                                                     \
  }                                                                                               \
  ORC_EXPORT int orc_solve_1d_##SFX(T dt, T dx, int n, int order, int iters, const T* P,          \
                                    const T* c, const T* u0, T* u, int threads) {                 \
    return solve_1d<T>(dt, dx, n, order, iters, P, c, u0, u, threads);                            \
  }                                                                                               \
  ORC_EXPORT int orc_solve_2d_##SFX(T dt, T dx, int n, int order, int iters, const T* P,          \
                                    const T* c, const T* u0, T* u, int threads) {                 \
    return solve_2d<T>(dt, dx, n, order, iters, P, c, u0, u, threads);                            \
  }                                                                                               \
  ORC_EXPORT int orc_chemical_potential_1d_##SFX(T dx, int n, const T* P, const T* c,             \
                                                 const T* u0, T* mu) {                            \
    return chemical_potential_1d<T>(dx, n, P, c, u0, mu);                                         \
  }                                                                                               \
  ORC_EXPORT int orc_chemical_potential_2d_##SFX(T dx, int n, const T* P, const T* c,             \
                                                 const T* u0, T* mu) {                            \
    return chemical_potential_2d<T>(dx, n, P, c, u0, mu);                                         \
  }

ORC_DEFINE(f32, float)
ORC_DEFINE(f64, double)

ORC_EXPORT int orc_openmp_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
