// kdiag.cu -- FP64 diagnostics on the device: norms, chemical potential sums, error vs a
// double-precision reference.  Two-pass reductions with a fixed block count and a fixed order,
// so a result never depends on what else runs on the GPU.
#include "kernels.h"
#include "nls_common.cuh"

namespace nlsg {

static constexpr int kDiagBlocks = 304;  // 2 x 152 SMs
static constexpr int kDiagThreads = 256;
static constexpr int kDiagMaxNV = 4;

size_t diag_partials_bytes(long long) { return (size_t)kDiagBlocks * kDiagMaxNV * sizeof(double); }

__device__ __forceinline__ double weight(int mode, long long i, double dx) {
  return mode == 1 ? (double)i * dx : 1.0;
}

template <typename T>
__global__ void __launch_bounds__(kDiagThreads) k_norm(long long n, const void* __restrict__ u_, int mode,
                                                       double dx, double* __restrict__ part) {
  typedef typename C2<T>::type C;
  __shared__ double sm[32 * 2];
  const C* u = reinterpret_cast<const C*>(u_);
  double v[2] = {0.0, 0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C a = u[i];
    const double x = (double)a.x, y = (double)a.y;
    v[0] += weight(mode, i, dx) * (x * x + y * y);
    v[1] += (isfinite(x) && isfinite(y)) ? 0.0 : 1.0;
  }
  block_sum<2>(v, sm);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 2 + 0] = v[0];
    part[blockIdx.x * 2 + 1] = v[1];
  }
}

template <typename T>
__global__ void __launch_bounds__(kDiagThreads) k_mu(long long n, const void* __restrict__ u_,
                                                     const void* __restrict__ h_, int mode, double dx,
                                                     double* __restrict__ part) {
  typedef typename C2<T>::type C;
  __shared__ double sm[32 * 3];
  const C* u = reinterpret_cast<const C*>(u_);
  const C* hv = reinterpret_cast<const C*>(h_);
  double v[3] = {0.0, 0.0, 0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C a = u[i], b = hv[i];
    const double w = weight(mode, i, dx);
    const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
    // conj(a) * b
    v[0] += w * (ax * bx + ay * by);
    v[1] += w * (ax * by - ay * bx);
    v[2] += w * (ax * ax + ay * ay);
  }
  block_sum<3>(v, sm);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 3 + 0] = v[0];
    part[blockIdx.x * 3 + 1] = v[1];
    part[blockIdx.x * 3 + 2] = v[2];
  }
}

template <typename T>
__global__ void __launch_bounds__(kDiagThreads) k_relerr(long long n, const void* __restrict__ a_,
                                                         const double2* __restrict__ b,
                                                         const double* __restrict__ P, double c12,
                                                         double c13, double c14,
                                                         double* __restrict__ part) {
  typedef typename C2<T>::type C;
  __shared__ double sm[32 * 4];
  const C* a = reinterpret_cast<const C*>(a_);
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C x = a[i];
    const double2 y = b[i];
    const double da = (double)x.x * (double)x.x + (double)x.y * (double)x.y;
    const double db = y.x * y.x + y.y * y.y;
    const double na = c12 * P[i] / (c13 + c14 * da);
    const double nb = c12 * P[i] / (c13 + c14 * db);
    v[0] += (da - db) * (da - db);
    v[1] += db * db;
    v[2] += (na - nb) * (na - nb);
    v[3] += nb * nb;
  }
  block_sum<4>(v, sm);
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; ++k) part[blockIdx.x * 4 + k] = v[k];
}

// Damping integral of Solution.getDampingIntegral (nls/model.py:350-365): the rectangle rule of
// (n_res - 1) |u|^2 with n_res = c12 P / (c13 + c14 |u|^2), weighted by w_i = 2 pi r_i dx on the
// radial grid r_i = i * r_step (r_step = n dx / (n - 1), the spacing of linspace(0, n dx, n)) when
// radial, else by dx^2.
template <typename T>
__global__ void __launch_bounds__(kDiagThreads) k_damping(long long n, const void* __restrict__ u_,
                                                          const void* __restrict__ P_, int radial,
                                                          double r_step, double dx, double c12, double c13,
                                                          double c14, double* __restrict__ part) {
  typedef typename C2<T>::type C;
  __shared__ double sm[32 * 1];
  const C* u = reinterpret_cast<const C*>(u_);
  const T* P = reinterpret_cast<const T*>(P_);
  const double two_pi = 6.283185307179586476925286766559;
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C a = u[i];
    const double d = (double)a.x * (double)a.x + (double)a.y * (double)a.y;
    const double res = c12 * (double)P[i] / (c13 + c14 * d);
    const double w = radial ? two_pi * ((double)i * r_step) * dx : dx * dx;
    v[0] += (res - 1.0) * d * w;
  }
  block_sum<1>(v, sm);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// Sum the per-block partials in a fixed order (one warp per value).
__global__ void k_final(const double* __restrict__ part, int nblocks, int nv, double* __restrict__ out) {
  const int k = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= nv) return;
  double s = 0.0;
  for (int b = lane; b < nblocks; b += 32) s += part[b * nv + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[k] = s;
}

static int blocks_for(long long n) {
  long long b = (n + kDiagThreads - 1) / kDiagThreads;
  return (int)(b < kDiagBlocks ? (b < 1 ? 1 : b) : kDiagBlocks);
}

cudaError_t diag_norm(int dtype, long long n, const void* u, int mode, double dx, double* part,
                      double* out, cudaStream_t st) {
  const int nb = blocks_for(n);
  if (dtype == NLS_C128) k_norm<double><<<nb, kDiagThreads, 0, st>>>(n, u, mode, dx, part);
  else k_norm<float><<<nb, kDiagThreads, 0, st>>>(n, u, mode, dx, part);
  k_final<<<1, 32 * 2, 0, st>>>(part, nb, 2, out);
  return cudaGetLastError();
}

cudaError_t diag_mu(int dtype, long long n, const void* u, const void* v, int mode, double dx,
                    double* part, double* out, cudaStream_t st) {
  const int nb = blocks_for(n);
  if (dtype == NLS_C128) k_mu<double><<<nb, kDiagThreads, 0, st>>>(n, u, v, mode, dx, part);
  else k_mu<float><<<nb, kDiagThreads, 0, st>>>(n, u, v, mode, dx, part);
  k_final<<<1, 32 * 3, 0, st>>>(part, nb, 3, out);
  return cudaGetLastError();
}

cudaError_t diag_damping(int dtype, long long n, const void* u, const void* P, int radial, double r_step,
                         double dx, double c12, double c13, double c14, double* part, double* out,
                         cudaStream_t st) {
  const int nb = blocks_for(n);
  if (dtype == NLS_C128) k_damping<double><<<nb, kDiagThreads, 0, st>>>(n, u, P, radial, r_step, dx, c12, c13, c14, part);
  else k_damping<float><<<nb, kDiagThreads, 0, st>>>(n, u, P, radial, r_step, dx, c12, c13, c14, part);
  k_final<<<1, 32, 0, st>>>(part, nb, 1, out);
  return cudaGetLastError();
}

cudaError_t diag_relerr(int dtype_a, long long n, const void* a, const void* b, const double* P,
                        double c12, double c13, double c14, double* part, double* out,
                        cudaStream_t st) {
  const int nb = blocks_for(n);
  const double2* bb = reinterpret_cast<const double2*>(b);
  if (dtype_a == NLS_C128) k_relerr<double><<<nb, kDiagThreads, 0, st>>>(n, a, bb, P, c12, c13, c14, part);
  else k_relerr<float><<<nb, kDiagThreads, 0, st>>>(n, a, bb, P, c12, c13, c14, part);
  k_final<<<1, 32 * 4, 0, st>>>(part, nb, 4, out);
  return cudaGetLastError();
}

}  // namespace nlsg
