// k2d.cu -- 2-D (Cartesian cross stencil) RK4 kernels for sm_103a.
//
// rk4_2d_fused: one launch applies one complete RK4 step (the four `hamiltonian_2d` calls and the
// update of `runge_kutta_2d`, nls/nls.f90:892-900) to a list of tiles.  A CTA stages its tile plus
// a halo of 4K nodes (K = 1 for order 3, 2 for order 5) in shared memory, evaluates the four stages
// back to back (stage s is valid on the region shrunk by s*K), keeps u, the pump and the RK4
// accumulator of its nodes in registers, and writes only the new state: per node-step HBM sees
// one read of u and P and one write of u.  The
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

// Complex pair arithmetic: Blackwell's packed FP32x2 pipe (FADD2/FMUL2/FFMA2) for complex64,
// plain FP64 for complex128.
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float s, float2 b, float2 c) { return __ffma2_rn(make_float2(s, s), b, c); }
__device__ __forceinline__ float2 pmul(float s, float2 b) { return __fmul2_rn(make_float2(s, s), b); }
__device__ __forceinline__ double2 padd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 pfma(double s, double2 b, double2 c) {
  return make_double2(fma(s, b.x, c.x), fma(s, b.y, c.y));
}
__device__ __forceinline__ double2 pmul(double s, double2 b) { return make_double2(s * b.x, s * b.y); }

// Right-hand side with the pump already multiplied by c12 (the reference evaluates
// coeffs(12) * pumping first, nls/nls.f90:580, so folding it changes no rounding).
template <typename T>
__device__ __forceinline__ typename C2<T>::type rhs_pc(typename C2<T>::type u, T pc,
                                                       typename C2<T>::type lu, const Phys<T>& ph) {
  const T s = fma(u.x, u.x, u.y * u.y);
  const T r = rdiv(pc, fma(ph.c14, s, ph.c13));
  const T a = fma(ph.c3, r, -ph.c4);
  const T b = fma(ph.c5, s, ph.c6 * r);
  typename C2<T>::type v;
  v.x = fma(a, u.x, fma(b, u.y, -lu.y));
  v.y = fma(a, u.y, fma(-b, u.x, lu.x));
  return v;
}

// Tile geometry: a region of RX x RY nodes (the output tile plus a halo of H = 4K on every
// side) computed by (RX/32) x NS warps; warp (xw, strip) owns columns xw*32 .. xw*32+31 of rows
// strip*NJ .. strip*NJ+NJ-1, so every branch below is warp-uniform.
template <typename T, int K, int RX, int RY, int NS>
struct TileCfg {
  static constexpr int WX = RX / 32;
  static constexpr int NT = WX * NS * 32;
  static constexpr int NJ = RY / NS;
  static constexpr int H = 4 * K;
  static constexpr int TX = RX - 2 * H;
  static constexpr int TY = RY - 2 * H;
  static constexpr int ROWS = RY + 2 * K;     // K guard rows above and below each buffer
  static constexpr size_t SMEM = (size_t)2 * ROWS * RX * sizeof(typename C2<T>::type);
  // CTAs per SM the register budget is sized for: 2 x 256 threads, else one CTA
  static constexpr int MINB = NT <= 256 ? 2 : 1;
  static_assert(RX % 32 == 0 && RY % NS == 0 && NJ <= 32, "tile layout");
  static_assert(TX > 0 && TY > 0, "tile too small for its halo");
};

// One RK4 stage S over the thread's column strip.  Every node of the region is evaluated (the
// stage's valid region shrinks by K per stage; values computed outside it are never read again),
// and only in-domain nodes are stored, so out-of-domain halo stays exactly zero.
template <typename T, int K, int RX, int NJ, int S>
__device__ __forceinline__ void tile_stage(const typename C2<T>::type* __restrict__ in,
                                           typename C2<T>::type* __restrict__ out, int x, int y0,
                                           typename C2<T>::type (&u)[NJ], typename C2<T>::type (&acc)[NJ],
                                           const T (&pc)[NJ], unsigned dom, const Phys<T>& ph,
                                           const RK<T>& rk, T wc, T w1, T w2) {
  typedef typename C2<T>::type C;
  C w[2 * K + 1];
#pragma unroll
  for (int d = 0; d <= 2 * K; ++d) w[d] = in[(y0 - K + d) * RX + x];
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int c = (y0 + j) * RX + x;
    const C v = w[K];
    C s1 = padd(padd(in[c - 1], in[c + 1]), padd(w[K - 1], w[K + 1]));
    C lu = pfma(w1, s1, pmul(wc, v));
    if (K == 2) {
      C s2 = padd(padd(in[c - 2], in[c + 2]), padd(w[0], w[2 * K]));
      lu = pfma(w2, s2, lu);
    }
    const C k = rhs_pc<T>(v, pc[j], lu, ph);
    if (S == 1) acc[j] = k;
    else acc[j] = pfma(S == 4 ? (T)1 : (T)2, k, acc[j]);
    if (S < 4) {
      const C t = pfma(S == 3 ? rk.dt : rk.half_dt, k, u[j]);
      if (dom & (1u << j)) out[c] = t;
    } else {
      u[j] = pfma(rk.dt6, acc[j], u[j]);
    }
#pragma unroll
    for (int d = 0; d < 2 * K; ++d) w[d] = w[d + 1];
    if (j + 1 < NJ) w[2 * K] = in[(y0 + j + 1 + K) * RX + x];
  }
}

template <typename T, int K, int RX, int RY, int NS>
__global__ void __launch_bounds__(TileCfg<T, K, RX, RY, NS>::NT, TileCfg<T, K, RX, RY, NS>::MINB)
rk4_2d_fused(const Inst2D* __restrict__ insts, const TileItem* __restrict__ items, int n_items,
             int j_step) {
  typedef typename C2<T>::type C;
  typedef TileCfg<T, K, RX, RY, NS> G;
  constexpr int NJ = G::NJ, H = G::H;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* base = reinterpret_cast<C*>(smem_raw);
  C* buf0 = base + K * RX;                   // row 0 of buffer 0 (rows -K .. RY+K-1 exist)
  C* buf1 = base + G::ROWS * RX + K * RX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x = (warp % G::WX) * 32 + lane;
  const int y0 = (warp / G::WX) * NJ;
  // guard rows are read by the edge rows' stencils and never written: zero them once
  for (int i = threadIdx.x; i < K * RX; i += G::NT) {
    buf0[-K * RX + i] = mk<T>(0, 0);
    buf0[RY * RX + i] = mk<T>(0, 0);
    buf1[-K * RX + i] = mk<T>(0, 0);
    buf1[RY * RX + i] = mk<T>(0, 0);
  }
  const bool x_interior = x >= H && x < RX - H;

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
    const int gx = txi * G::TX - H + x;
    const int gy0 = tyi * G::TY - H + y0;
    const bool xin = gx >= 0 && gx < n;
    const Phys<T> ph = phys_from<T>(I.ph);
    const RK<T> rk = rk_from<T>(I.dt);
    const T wc = (T)I.op.center, w1 = (T)I.op.w[0], w2 = (T)I.op.w[1];
    const T c12 = (T)I.ph.c12;

    C u[NJ], acc[NJ];
    T pc[NJ];
    unsigned dom = 0, store = 0;
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int gy = gy0 + j;
      const bool inb = xin && gy >= 0 && gy < n;
      const size_t q = (size_t)gy * n + gx;
      u[j] = inb ? src[q] : mk<T>(0, 0);
      pc[j] = inb ? c12 * Pg[q] : (T)0;
      acc[j] = mk<T>(0, 0);
      dom |= (unsigned)inb << j;
      const int y = y0 + j;
      store |= (unsigned)(inb && x_interior && y >= H && y < RY - H) << j;
    }
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      buf0[(y0 + j) * RX + x] = u[j];
      if (!(dom & (1u << j))) buf1[(y0 + j) * RX + x] = mk<T>(0, 0);
    }
    __syncthreads();
    tile_stage<T, K, RX, NJ, 1>(buf0, buf1, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 2>(buf1, buf0, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 3>(buf0, buf1, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 4>(buf1, nullptr, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (store & (1u << j)) dst[(size_t)(gy0 + j) * n + gx] = u[j];
    __syncthreads();  // the next tile's load rewrites both buffers
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

// Shape table: region RX x RY computed by (RX/32) x NS warps.
//   TILE_64x64   : 64 x 64,  8 strips of 8 rows  (512 threads)
//   TILE_128x32  : 128 x 32, 4 strips of 8 rows  (512 threads)
//   TILE_32x32   : 32 x 32,  8 strips of 4 rows  (256 threads)
//   TILE_64x64W  : 64 x 64,  16 strips of 4 rows (1024 threads)
//   TILE_128x32W : 128 x 32, 8 strips of 4 rows  (1024 threads)
int tile_region_x(int shape) {
  switch (shape) {
    case TILE_64x64: return 64; case TILE_128x32: return 128; case TILE_32x32: return 32;
    case TILE_64x64W: return 64; case TILE_128x32W: return 128;
  }
  return 0;
}
int tile_region_y(int shape) {
  switch (shape) {
    case TILE_64x64: return 64; case TILE_128x32: return 32; case TILE_32x32: return 32;
    case TILE_64x64W: return 64; case TILE_128x32W: return 32;
  }
  return 0;
}
int tile_out_x(int shape, int K) { return tile_region_x(shape) - 8 * K; }
int tile_out_y(int shape, int K) { return tile_region_y(shape) - 8 * K; }
bool tile_supported(int shape, int dtype) {
  if (shape == TILE_32x32) return true;
  if (shape == TILE_64x64 || shape == TILE_128x32 || shape == TILE_64x64W || shape == TILE_128x32W)
    return dtype == NLS_C64;
  return false;
}

template <typename T, int K, int RX, int RY, int NS>
static cudaError_t launch_f(const Inst2D* d_insts, const TileItem* d_items, int n_items, int j_step,
                            int grid, cudaStream_t s) {
  typedef TileCfg<T, K, RX, RY, NS> G;
  auto kern = rk4_2d_fused<T, K, RX, RY, NS>;
  kern<<<grid, G::NT, G::SMEM, s>>>(d_insts, d_items, n_items, j_step);
  return cudaGetLastError();
}

// Sets the shared-memory attribute (outside any capture) and returns CTAs per SM.
template <typename T, int K, int RX, int RY, int NS>
static int occ_f() {
  typedef TileCfg<T, K, RX, RY, NS> G;
  auto kern = rk4_2d_fused<T, K, RX, RY, NS>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, G::NT, G::SMEM) != cudaSuccess) return 0;
  return nb;
}

#define NLSG_SHAPES(T, K, CALL, ...)                                        \
  switch (shape) {                                                         \
    case TILE_64x64: return CALL<T, K, 64, 64, 8>(__VA_ARGS__);            \
    case TILE_128x32: return CALL<T, K, 128, 32, 4>(__VA_ARGS__);          \
    case TILE_32x32: return CALL<T, K, 32, 32, 8>(__VA_ARGS__);            \
    case TILE_64x64W: return CALL<T, K, 64, 64, 16>(__VA_ARGS__);          \
    case TILE_128x32W: return CALL<T, K, 128, 32, 8>(__VA_ARGS__);         \
  }

int fused_2d_blocks_per_sm(int dtype, int K, int shape) {
  if (!tile_supported(shape, dtype)) return 0;
  if (dtype == NLS_C128) {
    if (shape != TILE_32x32) return 0;
    if (K == 1) return occ_f<double, 1, 32, 32, 8>();
    if (K == 2) return occ_f<double, 2, 32, 32, 8>();
    return 0;
  }
  if (K == 1) { NLSG_SHAPES(float, 1, occ_f) }
  if (K == 2) { NLSG_SHAPES(float, 2, occ_f) }
  return 0;
}

cudaError_t launch_2d_fused(int dtype, int K, int shape, const Inst2D* d_insts,
                            const TileItem* d_items, int n_items, int j_step, int grid,
                            cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  if (!tile_supported(shape, dtype)) return cudaErrorInvalidValue;
  if (dtype == NLS_C128) {
    if (shape != TILE_32x32) return cudaErrorInvalidValue;
    if (K == 1) return launch_f<double, 1, 32, 32, 8>(d_insts, d_items, n_items, j_step, grid, s);
    if (K == 2) return launch_f<double, 2, 32, 32, 8>(d_insts, d_items, n_items, j_step, grid, s);
    return cudaErrorInvalidValue;
  }
  if (K == 1) { NLSG_SHAPES(float, 1, launch_f, d_insts, d_items, n_items, j_step, grid, s) }
  if (K == 2) { NLSG_SHAPES(float, 2, launch_f, d_insts, d_items, n_items, j_step, grid, s) }
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
