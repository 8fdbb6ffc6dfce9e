// k2d.cu -- 2-D (Cartesian cross stencil) RK4 kernels for sm_103a.
//
// rk4_2d_fused: one launch applies one complete RK4 step (the four `hamiltonian_2d` calls and the
// update of `runge_kutta_2d`, nls/nls.f90:892-900) to a list of tiles.  A CTA stages its tile plus
// a halo of 4K nodes (K = 1 for order 3, 2 for order 5) in shared memory, evaluates stage s on the
// region shrunk by s*K, keeps u, the pump and the RK4 accumulator of its nodes in registers, and
// writes only the new state: per node-step HBM sees one read of u and P and one write of u.  The
// tile list may span many independent solves (batched and served forms), each with its own size,
// coefficients and ping-pong buffers; the persistent grid strides over the list.
//
// rk4_2d_stage: one RK4 stage from global memory (no halo recomputation), used where tiles would
// be too small to amortise their halo (double precision on modest grids) and as the general path.
#include "kernels.h"
#include "nls_common.cuh"

namespace nlsg {

template <typename T>
__device__ __forceinline__ typename C2<T>::type cadd4(typename C2<T>::type a, typename C2<T>::type b,
                                                      typename C2<T>::type c, typename C2<T>::type d) {
  return mk<T>((a.x + b.x) + (c.x + d.x), (a.y + b.y) + (c.y + d.y));
}

template <typename T, int K, int RX, int RY, int NT>
__global__ void __launch_bounds__(NT, 2)
rk4_2d_fused(const Inst2D* __restrict__ insts, const TileItem* __restrict__ items, int n_items,
             int j_step) {
  typedef typename C2<T>::type C;
  constexpr int H = 4 * K;
  constexpr int TX = RX - 2 * H;
  constexpr int TY = RY - 2 * H;
  constexpr int G = NT / RX;
  constexpr int NJ = RY / G;
  static_assert(NT % RX == 0 && RY % G == 0, "thread layout");
  static_assert(TX > 0 && TY > 0, "tile too small for halo");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* bufA = reinterpret_cast<C*>(smem_raw);
  C* bufB = bufA + RX * RY;
  const int x = threadIdx.x % RX;
  const int g = threadIdx.x / RX;

  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const TileItem ti = items[it];
    const Inst2D& I = insts[ti.inst];
    if ((int64_t)j_step >= I.steps) continue;
    const int n = I.n;
    const int par = (I.parity + j_step) & 1;
    const C* __restrict__ src = reinterpret_cast<const C*>(I.u[par]);
    C* __restrict__ dst = reinterpret_cast<C*>(I.u[par ^ 1]);
    const T* __restrict__ Pg = reinterpret_cast<const T*>(I.P);
    const int tyi = ti.tile / I.tiles_x;
    const int txi = ti.tile - tyi * I.tiles_x;
    const int gx = txi * TX - H + x;
    const int gy0 = tyi * TY - H;
    const bool xin = gx >= 0 && gx < n;
    const Phys<T> ph = phys_from<T>(I.ph);
    const RK<T> rk = rk_from<T>(I.dt);
    const T wc = (T)I.op.center, w1 = (T)I.op.w[0], w2 = (T)I.op.w[1];

    C u[NJ], acc[NJ];
    T P[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int y = g + G * j;
      const int gy = gy0 + y;
      const bool inb = xin && gy >= 0 && gy < n;
      const size_t q = (size_t)gy * n + gx;
      u[j] = inb ? src[q] : mk<T>(0, 0);
      P[j] = inb ? Pg[q] : (T)0;
      acc[j] = mk<T>(0, 0);
      bufA[y * RX + x] = u[j];
    }
    __syncthreads();

#pragma unroll 1
    for (int s = 1; s <= 4; ++s) {
      const C* in = (s & 1) ? bufA : bufB;
      C* out = (s & 1) ? bufB : bufA;
      const int lo = s * K;
      const bool xact = x >= lo && x < RX - lo;
      const T coef = s == 3 ? rk.dt : rk.half_dt;
      const T wk = (s == 1 || s == 4) ? (T)1 : (T)2;
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int y = g + G * j;
        if (xact && y >= lo && y < RY - lo) {
          const int c = y * RX + x;
          const C v = in[c];
          const C s1 = cadd4<T>(in[c - 1], in[c + 1], in[c - RX], in[c + RX]);
          C lu = mk<T>(wc * v.x + w1 * s1.x, wc * v.y + w1 * s1.y);
          if (K == 2) {
            const C s2 = cadd4<T>(in[c - 2], in[c + 2], in[c - 2 * RX], in[c + 2 * RX]);
            lu.x += w2 * s2.x;
            lu.y += w2 * s2.y;
          }
          const C k = rhs<T>(v, P[j], lu, ph);
          if (s == 1) {
            acc[j] = k;
          } else {
            acc[j].x += wk * k.x;
            acc[j].y += wk * k.y;
          }
          const int gy = gy0 + y;
          const bool inb = xin && gy >= 0 && gy < n;
          if (s < 4) {
            C t = mk<T>(u[j].x + coef * k.x, u[j].y + coef * k.y);
            if (!inb) t = mk<T>(0, 0);
            out[c] = t;
          } else if (inb) {
            dst[(size_t)gy * n + gx] = mk<T>(u[j].x + rk.dt6 * acc[j].x, u[j].y + rk.dt6 * acc[j].y);
          }
        }
      }
      if (s < 4) __syncthreads();
    }
  }
}

// One RK4 stage of an n x n grid in global memory; thread block 32 x 8 nodes.
template <typename T, int K>
__global__ void __launch_bounds__(256) rk4_2d_stage(int n, int s, const void* __restrict__ src_,
                                                    void* __restrict__ u_, const void* __restrict__ P_,
                                                    void* __restrict__ acc_, void* __restrict__ dst_,
                                                    double dt, PhysD phd, Stencil2D op) {
  typedef typename C2<T>::type C;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= n || y >= n) return;
  const C* __restrict__ src = reinterpret_cast<const C*>(src_);
  C* __restrict__ U = reinterpret_cast<C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  C* __restrict__ acc = reinterpret_cast<C*>(acc_);
  C* __restrict__ dst = reinterpret_cast<C*>(dst_);
  const Phys<T> ph = phys_from<T>(phd);
  const RK<T> rk = rk_from<T>(dt);
  const size_t q = (size_t)y * n + x;
  auto at = [&](int xx, int yy) -> C {
    return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? src[(size_t)yy * n + xx] : mk<T>(0, 0);
  };
  const C v = src[q];
  const C s1 = cadd4<T>(at(x - 1, y), at(x + 1, y), at(x, y - 1), at(x, y + 1));
  const T wc = (T)op.center, w1 = (T)op.w[0], w2 = (T)op.w[1];
  C lu = mk<T>(wc * v.x + w1 * s1.x, wc * v.y + w1 * s1.y);
  if (K == 2) {
    const C s2 = cadd4<T>(at(x - 2, y), at(x + 2, y), at(x, y - 2), at(x, y + 2));
    lu.x += w2 * s2.x;
    lu.y += w2 * s2.y;
  }
  const C k = rhs<T>(v, P[q], lu, ph);
  const C u = U[q];
  if (s == 1) {
    acc[q] = k;
    dst[q] = mk<T>(u.x + rk.half_dt * k.x, u.y + rk.half_dt * k.y);
  } else if (s == 2 || s == 3) {
    C a = acc[q];
    a.x += (T)2 * k.x;
    a.y += (T)2 * k.y;
    acc[q] = a;
    const T c = s == 2 ? rk.half_dt : rk.dt;
    dst[q] = mk<T>(u.x + c * k.x, u.y + c * k.y);
  } else {
    C a = acc[q];
    a.x += k.x;
    a.y += k.y;
    U[q] = mk<T>(u.x + rk.dt6 * a.x, u.y + rk.dt6 * a.y);
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(256) rhs_2d(int n, const void* __restrict__ u_, const void* __restrict__ P_,
                                              void* __restrict__ v_, PhysD phd, Stencil2D op) {
  typedef typename C2<T>::type C;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= n || y >= n) return;
  const C* __restrict__ src = reinterpret_cast<const C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  const Phys<T> ph = phys_from<T>(phd);
  auto at = [&](int xx, int yy) -> C {
    return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? src[(size_t)yy * n + xx] : mk<T>(0, 0);
  };
  const size_t q = (size_t)y * n + x;
  const C v = src[q];
  const C s1 = cadd4<T>(at(x - 1, y), at(x + 1, y), at(x, y - 1), at(x, y + 1));
  const T wc = (T)op.center, w1 = (T)op.w[0], w2 = (T)op.w[1];
  C lu = mk<T>(wc * v.x + w1 * s1.x, wc * v.y + w1 * s1.y);
  if (K == 2) {
    const C s2 = cadd4<T>(at(x - 2, y), at(x + 2, y), at(x, y - 2), at(x, y + 2));
    lu.x += w2 * s2.x;
    lu.y += w2 * s2.y;
  }
  reinterpret_cast<C*>(v_)[q] = rhs<T>(v, P[q], lu, ph);
}

// ------------------------------------------------------------------ launchers

int tile_region_x(int shape) {
  switch (shape) { case TILE_64x64: return 64; case TILE_128x32: return 128; case TILE_32x32: return 32; }
  return 0;
}
int tile_region_y(int shape) {
  switch (shape) { case TILE_64x64: return 64; case TILE_128x32: return 32; case TILE_32x32: return 32; }
  return 0;
}
int tile_out_x(int shape, int K) { return tile_region_x(shape) - 8 * K; }
int tile_out_y(int shape, int K) { return tile_region_y(shape) - 8 * K; }
bool tile_supported(int shape, int dtype) {
  if (shape == TILE_32x32) return true;
  if (shape == TILE_64x64 || shape == TILE_128x32) return dtype == NLS_C64;
  return false;
}

template <typename T, int K, int RX, int RY>
static cudaError_t launch_f(const Inst2D* d_insts, const TileItem* d_items, int n_items, int j_step,
                            int grid, cudaStream_t s) {
  auto kern = rk4_2d_fused<T, K, RX, RY, 256>;
  const size_t smem = (size_t)2 * RX * RY * sizeof(typename C2<T>::type);
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  kern<<<grid, 256, smem, s>>>(d_insts, d_items, n_items, j_step);
  return cudaGetLastError();
}

template <typename T, int K, int RX, int RY>
static int occ_f() {
  auto kern = rk4_2d_fused<T, K, RX, RY, 256>;
  const size_t smem = (size_t)2 * RX * RY * sizeof(typename C2<T>::type);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 256, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

#define NLSG_SHAPE_DISPATCH(T, K, shape, CALL)                 \
  switch (shape) {                                            \
    case TILE_64x64: return CALL<T, K, 64, 64>();             \
    case TILE_128x32: return CALL<T, K, 128, 32>();           \
    case TILE_32x32: return CALL<T, K, 32, 32>();             \
  }

int fused_2d_blocks_per_sm(int dtype, int K, int shape) {
  if (!tile_supported(shape, dtype)) return 0;
  if (dtype == NLS_C128) {
    if (K == 1) { if (shape == TILE_32x32) return occ_f<double, 1, 32, 32>(); }
    if (K == 2) { if (shape == TILE_32x32) return occ_f<double, 2, 32, 32>(); }
    return 0;
  }
  if (K == 1) { NLSG_SHAPE_DISPATCH(float, 1, shape, occ_f) }
  if (K == 2) { NLSG_SHAPE_DISPATCH(float, 2, shape, occ_f) }
  return 0;
}

cudaError_t launch_2d_fused(int dtype, int K, int shape, const Inst2D* d_insts,
                            const TileItem* d_items, int n_items, int j_step, int grid,
                            cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  if (!tile_supported(shape, dtype)) return cudaErrorInvalidValue;
  if (dtype == NLS_C128) {
    if (shape != TILE_32x32) return cudaErrorInvalidValue;
    if (K == 1) return launch_f<double, 1, 32, 32>(d_insts, d_items, n_items, j_step, grid, s);
    if (K == 2) return launch_f<double, 2, 32, 32>(d_insts, d_items, n_items, j_step, grid, s);
    return cudaErrorInvalidValue;
  }
  if (K == 1) {
    switch (shape) {
      case TILE_64x64: return launch_f<float, 1, 64, 64>(d_insts, d_items, n_items, j_step, grid, s);
      case TILE_128x32: return launch_f<float, 1, 128, 32>(d_insts, d_items, n_items, j_step, grid, s);
      case TILE_32x32: return launch_f<float, 1, 32, 32>(d_insts, d_items, n_items, j_step, grid, s);
    }
  } else if (K == 2) {
    switch (shape) {
      case TILE_64x64: return launch_f<float, 2, 64, 64>(d_insts, d_items, n_items, j_step, grid, s);
      case TILE_128x32: return launch_f<float, 2, 128, 32>(d_insts, d_items, n_items, j_step, grid, s);
      case TILE_32x32: return launch_f<float, 2, 32, 32>(d_insts, d_items, n_items, j_step, grid, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_2d_stage(int dtype, int n, int s, const void* src, void* u, const void* P,
                            void* acc, void* dst, double dt, const PhysD& ph, const Stencil2D& op,
                            cudaStream_t st) {
  dim3 grid((n + 31) / 32, (n + 7) / 8);
  if (dtype == NLS_C128) {
    if (op.K == 1) rk4_2d_stage<double, 1><<<grid, 256, 0, st>>>(n, s, src, u, P, acc, dst, dt, ph, op);
    else if (op.K == 2) rk4_2d_stage<double, 2><<<grid, 256, 0, st>>>(n, s, src, u, P, acc, dst, dt, ph, op);
    else return cudaErrorInvalidValue;
  } else {
    if (op.K == 1) rk4_2d_stage<float, 1><<<grid, 256, 0, st>>>(n, s, src, u, P, acc, dst, dt, ph, op);
    else if (op.K == 2) rk4_2d_stage<float, 2><<<grid, 256, 0, st>>>(n, s, src, u, P, acc, dst, dt, ph, op);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_rhs_2d(int dtype, int n, const void* u, const void* P, void* v, const PhysD& ph,
                          const Stencil2D& op, cudaStream_t st) {
  dim3 grid((n + 31) / 32, (n + 7) / 8);
  if (dtype == NLS_C128) {
    if (op.K == 1) rhs_2d<double, 1><<<grid, 256, 0, st>>>(n, u, P, v, ph, op);
    else if (op.K == 2) rhs_2d<double, 2><<<grid, 256, 0, st>>>(n, u, P, v, ph, op);
    else return cudaErrorInvalidValue;
  } else {
    if (op.K == 1) rhs_2d<float, 1><<<grid, 256, 0, st>>>(n, u, P, v, ph, op);
    else if (op.K == 2) rhs_2d<float, 2><<<grid, 256, 0, st>>>(n, u, P, v, ph, op);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace nlsg
