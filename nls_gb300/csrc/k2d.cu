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
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <functional>
#include <queue>
#include <utility>
#include <vector>

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
  return make_double2(__fma_rn(s, b.x, c.x), __fma_rn(s, b.y, c.y));
}
__device__ __forceinline__ double2 pmul(double s, double2 b) { return make_double2(s * b.x, s * b.y); }

// Fused multiply-add in the working precision (single-precision arguments must not be promoted
// to the FP64 pipe, which runs at a small fraction of the FP32 rate on GB300).
__device__ __forceinline__ float mad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mad(double a, double b, double c) { return __fma_rn(a, b, c); }

// Right-hand side with the pump already multiplied by c12 (the reference evaluates
// coeffs(12) * pumping first, nls/nls.f90:580, so folding it changes no rounding).
template <typename T>
__device__ __forceinline__ typename C2<T>::type rhs_pc(typename C2<T>::type u, T pc,
                                                       typename C2<T>::type lu, const Phys<T>& ph) {
  const T s = mad(u.x, u.x, u.y * u.y);
  const T r = rdiv(pc, mad(ph.c14, s, ph.c13));
  const T a = mad(ph.c3, r, -ph.c4);
  const T b = mad(ph.c5, s, ph.c6 * r);
  typename C2<T>::type v;
  v.x = mad(a, u.x, mad(b, u.y, -lu.y));
  v.y = mad(a, u.y, mad(-b, u.x, lu.x));
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
  // rows per shared-memory load batch in a stage, sized to the register budget
  static constexpr int CJMAX = (NT >= 1024 || sizeof(T) == 8) ? 2 : 4;
  static constexpr int CJ = (CJMAX >= 4 && NJ % 4 == 0) ? 4 : (CJMAX >= 3 && NJ % 3 == 0) ? 3 : (NJ % 2 == 0 ? 2 : 1);
  static_assert(RX % 32 == 0 && RY % NS == 0 && NJ <= 32, "tile layout");
  static_assert(TX > 0 && TY > 0, "tile too small for its halo");
};

// One RK4 stage S over the thread's column strip.  Every node of the region is evaluated (the
// stage's valid region shrinks by K per stage; values computed outside it are never read again),
// and only in-domain nodes are stored, so out-of-domain halo stays exactly zero.  Rows are taken
// in batches of CJ: all shared-memory loads of a batch are issued before any of its stores, so
// the independent rows overlap their load and arithmetic latencies.
template <typename T, int K, int RX, int NJ, int S, int CJ>
__device__ __forceinline__ void tile_stage(const typename C2<T>::type* __restrict__ in,
                                           typename C2<T>::type* __restrict__ out, int x, int y0,
                                           typename C2<T>::type (&u)[NJ], typename C2<T>::type (&acc)[NJ],
                                           const T (&pc)[NJ], unsigned dom, const Phys<T>& ph,
                                           const RK<T>& rk, T wc, T w1, T w2) {
  typedef typename C2<T>::type C;
  static_assert(NJ % CJ == 0, "row batches");
#pragma unroll
  for (int j0 = 0; j0 < NJ; j0 += CJ) {
    C cv[CJ + 2 * K];
    C hl[K][CJ], hr[K][CJ];
#pragma unroll
    for (int i = 0; i < CJ + 2 * K; ++i) cv[i] = in[(y0 + j0 - K + i) * RX + x];
#pragma unroll
    for (int d = 1; d <= K; ++d)
#pragma unroll
      for (int i = 0; i < CJ; ++i) {
        hl[d - 1][i] = in[(y0 + j0 + i) * RX + x - d];
        hr[d - 1][i] = in[(y0 + j0 + i) * RX + x + d];
      }
    // The arithmetic below is written phase by phase across the CJ rows of the batch, so the
    // rows' independent dependency chains are interleaved in the instruction stream.
    C lu[CJ];
#pragma unroll
    for (int i = 0; i < CJ; ++i) {
      const C s1 = padd(padd(hl[0][i], hr[0][i]), padd(cv[i + K - 1], cv[i + K + 1]));
      lu[i] = pfma(w1, s1, pmul(wc, cv[i + K]));
      if (K == 2) {
        const C s2 = padd(padd(hl[K - 1][i], hr[K - 1][i]), padd(cv[i], cv[i + 2 * K]));
        lu[i] = pfma(w2, s2, lu[i]);
      }
    }
    T sq[CJ], r[CJ];
#pragma unroll
    for (int i = 0; i < CJ; ++i) sq[i] = mad(cv[i + K].x, cv[i + K].x, cv[i + K].y * cv[i + K].y);
#pragma unroll
    for (int i = 0; i < CJ; ++i) r[i] = rdiv(pc[j0 + i], mad(ph.c14, sq[i], ph.c13));
    C k[CJ];
#pragma unroll
    for (int i = 0; i < CJ; ++i) {
      const T a = mad(ph.c3, r[i], -ph.c4);
      const T b = mad(ph.c5, sq[i], ph.c6 * r[i]);
      const C v = cv[i + K];
      k[i].x = mad(a, v.x, mad(b, v.y, -lu[i].y));
      k[i].y = mad(a, v.y, mad(-b, v.x, lu[i].x));
    }
#pragma unroll
    for (int i = 0; i < CJ; ++i) {
      const int j = j0 + i;
      if (S == 1) acc[j] = k[i];
      else acc[j] = pfma(S == 4 ? (T)1 : (T)2, k[i], acc[j]);
      if (S < 4) {
        const C t = pfma(S == 3 ? rk.dt : rk.half_dt, k[i], u[j]);
        if (dom & (1u << j)) out[(y0 + j) * RX + x] = t;
      } else {
        u[j] = pfma(rk.dt6, acc[j], u[j]);
      }
    }
  }
}

// ---- TMA / mbarrier helpers (inline PTX, sm_90+ forms valid on sm_103a)

// Extra bytes the register-tile kernel arms its tile barrier for (0 in normal operation): a test
// control that makes the bounded wait expire without any fault.
__device__ unsigned g_tile_tx_extra = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 2-D tiled TMA load of the box at (x, y) (x = innermost coordinate) into shared memory.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait for phase `parity` of the barrier: at most kWaitIters polls with a 1 us suspend
// hint each (about a second); returns false if the phase never completed.
constexpr int kWaitIters = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (int i = 0; i < kWaitIters; ++i) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
        : "=r"(done) : "r"(a), "r"(parity), "r"(1000) : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace nlsg

#include "k2d_reg.cuh"
#include "k2d_stream.cuh"

namespace nlsg {

template <typename T, int K, int RX, int RY, int NS, bool TMA>
__global__ void __launch_bounds__(TileCfg<T, K, RX, RY, NS>::NT, TileCfg<T, K, RX, RY, NS>::MINB)
rk4_2d_fused(const Inst2D* __restrict__ insts, const TileItem* __restrict__ items, int n_items,
             int j_step, int* __restrict__ wait_flag) {
  typedef typename C2<T>::type C;
  typedef TileCfg<T, K, RX, RY, NS> G;
  constexpr int NJ = G::NJ, H = G::H;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  C* base = reinterpret_cast<C*>(smem_raw);
  C* buf0 = base + K * RX;                   // row 0 of buffer 0 (rows -K .. RY+K-1 exist)
  C* buf1 = base + G::ROWS * RX + K * RX;
  // TMA path only: staging for the next tile's state and pump boxes, and their barrier
  C* stage_u = reinterpret_cast<C*>(smem_raw + G::SMEM);
  T* stage_p = reinterpret_cast<T*>(smem_raw + G::SMEM + (size_t)RX * RY * sizeof(C));
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + G::SMEM + (size_t)RX * RY * (sizeof(C) + sizeof(T)));
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
  pdl_wait();      // the previous launch's states (programmatic launch)
  pdl_trigger();

  auto active = [&](int idx) -> bool {
    return idx < n_items && (int64_t)j_step < insts[items[idx].inst].steps;
  };
  // thread 0 arms the barrier and issues the state and pump boxes of tile idx
  auto issue = [&](int idx) {
    const TileItem ti = items[idx];
    const Inst2D& I = insts[ti.inst];
    const int tyi = ti.tile / I.tiles_x;
    const int txi = ti.tile - tyi * I.tiles_x;
    const int par = (I.parity + j_step) & 1;
    const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(I.tmap);
    fence_proxy_async_smem();
    mbar_expect_tx(bar, (uint32_t)((size_t)RX * RY * (sizeof(C) + sizeof(T))));
    tma_load_2d(stage_u, maps + par, txi * G::TX - H, tyi * G::TY - H, bar);
    tma_load_2d(stage_p, maps + 2, txi * G::TX - H, tyi * G::TY - H, bar);
  };
  uint32_t phase = 0;
  int it = blockIdx.x;
  if (TMA) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    while (it < n_items && !active(it)) it += gridDim.x;
    if (threadIdx.x == 0 && it < n_items) issue(it);
  }

  while (it < n_items) {
    const TileItem ti = items[it];
    const Inst2D& I = insts[ti.inst];
    int nxt = it + gridDim.x;
    if (TMA) {
      while (nxt < n_items && !active(nxt)) nxt += gridDim.x;
    } else if ((int64_t)j_step >= I.steps) {
      it = nxt;
      continue;
    }
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
    const Params<T>& prm = ParamsOf<T>::get(I);
    const Phys<T> ph = phys_of<T>(prm);
    const RK<T> rk = rk_of<T>(prm);
    const T wc = prm.wc, w1 = prm.w1, w2 = prm.w2;
    const T c12 = prm.c12;

    C u[NJ], acc[NJ];
    T pc[NJ];
    unsigned dom = 0, store = 0;
    if (TMA) {
      // one bounded wait per tile; a timeout ends every thread of the CTA together
      bool ok = true;
      if (threadIdx.x == 0) ok = mbar_wait(bar, phase);
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
          atomicExch(wait_flag, 1);  // the launching context's own status word
          mbar_wait(bar, phase);   // let the copy in flight land before the CTA leaves
        }
        return;
      }
      phase ^= 1u;
    }
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int gy = gy0 + j;
      const bool inb = xin && gy >= 0 && gy < n;
      if (TMA) {
        // out-of-range parts of the box arrive zero-filled
        u[j] = stage_u[(y0 + j) * RX + x];
        pc[j] = c12 * stage_p[(y0 + j) * RX + x];
      } else {
        const size_t q = (size_t)gy * n + gx;
        u[j] = inb ? src[q] : mk<T>(0, 0);
        pc[j] = inb ? c12 * Pg[q] : (T)0;
      }
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
    // the staging buffer is free again: fetch the next tile while this one is computed
    if (TMA && threadIdx.x == 0 && nxt < n_items) issue(nxt);
    tile_stage<T, K, RX, NJ, 1, G::CJ>(buf0, buf1, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 2, G::CJ>(buf1, buf0, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 3, G::CJ>(buf0, buf1, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
    __syncthreads();
    tile_stage<T, K, RX, NJ, 4, G::CJ>(buf1, nullptr, x, y0, u, acc, pc, dom, ph, rk, wc, w1, w2);
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (store & (1u << j)) dst[(size_t)(gy0 + j) * n + gx] = u[j];
    __syncthreads();  // the next tile's load rewrites both buffers
    it = nxt;
  }
}

// One RK4 stage of an n x n grid in global memory; thread block 32 x 8 nodes.
template <typename T, int K>
__global__ void __launch_bounds__(256) rk4_2d_stage(int n, int s, const void* __restrict__ src_,
                                                    void* __restrict__ u_, const void* __restrict__ P_,
                                                    void* __restrict__ acc_, void* __restrict__ dst_,
                                                    Params<T> prm) {
  typedef typename C2<T>::type C;
  pdl_wait();
  pdl_trigger();
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (x >= n || y >= n) return;
  const C* __restrict__ src = reinterpret_cast<const C*>(src_);
  C* __restrict__ U = reinterpret_cast<C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  C* __restrict__ acc = reinterpret_cast<C*>(acc_);
  C* __restrict__ dst = reinterpret_cast<C*>(dst_);
  const Phys<T> ph = phys_of<T>(prm);
  const RK<T> rk = rk_of<T>(prm);
  const size_t q = (size_t)y * n + x;
  auto at = [&](int xx, int yy) -> C {
    return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? src[(size_t)yy * n + xx] : mk<T>(0, 0);
  };
  const C v = src[q];
  const C s1 = cadd4<T>(at(x - 1, y), at(x + 1, y), at(x, y - 1), at(x, y + 1));
  const T wc = prm.wc, w1 = prm.w1, w2 = prm.w2;
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
                                              void* __restrict__ v_, Params<T> prm) {
  typedef typename C2<T>::type C;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= n || y >= n) return;
  const C* __restrict__ src = reinterpret_cast<const C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  const Phys<T> ph = phys_of<T>(prm);
  auto at = [&](int xx, int yy) -> C {
    return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? src[(size_t)yy * n + xx] : mk<T>(0, 0);
  };
  const size_t q = (size_t)y * n + x;
  const C v = src[q];
  const C s1 = cadd4<T>(at(x - 1, y), at(x + 1, y), at(x, y - 1), at(x, y + 1));
  const T wc = prm.wc, w1 = prm.w1, w2 = prm.w2;
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
//   TILE_64xO64  : 64 x (64 + 8K), 8 strips (512 threads): output tiles exactly 64 rows high
//   TILE_64xO64M : the same region with 12 (K = 1) or 10 (K = 2) strips (768 / 640 threads)
//   TILE_R64x*   : rk4_2d_reg, region 64 x (warps x rows per warp), see k2d_reg.cuh; 72 and 80
//                  rows give output tiles exactly 64 rows high at order 3 and 5
int tile_region_x(int shape) {
  switch (shape) {
    case TILE_64x64: return 64; case TILE_128x32: return 128; case TILE_32x32: return 32;
    case TILE_64x64W: return 64; case TILE_128x32W: return 128;
    case TILE_64xO64: return 64; case TILE_64xO64M: return 64;
    case TILE_R64x80: case TILE_R64x96: case TILE_R64x96S: case TILE_R64x64: case TILE_R64x72:
    case TILE_R64x72W: case TILE_R64x80S: case TILE_STREAM: return 64;
  }
  return 0;
}
int tile_region_y(int shape, int K) {
  switch (shape) {
    case TILE_64x64: return 64; case TILE_128x32: return 32; case TILE_32x32: return 32;
    case TILE_64x64W: return 64; case TILE_128x32W: return 32;
    case TILE_64xO64: return 64 + 8 * K; case TILE_64xO64M: return 64 + 8 * K;
    case TILE_R64x80: return 80; case TILE_R64x96: return 96; case TILE_R64x96S: return 96;
    case TILE_R64x64: return 64;
    case TILE_R64x72: case TILE_R64x72W: return 72; case TILE_R64x80S: return 80;
  }
  return 0;
}
static bool reg_shape(int shape) {
  return shape >= TILE_R64x80 && shape <= TILE_R64x80S;
}
int tile_out_x(int shape, int K) { return tile_region_x(shape) - 8 * K; }
int tile_out_y(int shape, int K) { return tile_region_y(shape, K) - 8 * K; }
bool tile_supported(int shape, int dtype) {
  if (shape == TILE_32x32) return true;
  if (shape == TILE_STREAM) return dtype == NLS_C64;
  if (shape == TILE_64x64 || shape == TILE_128x32 || shape == TILE_64x64W || shape == TILE_128x32W ||
      shape == TILE_64xO64 || shape == TILE_64xO64M || reg_shape(shape))
    return dtype == NLS_C64;
  return false;
}

template <typename T, int K, int RX, int RY, int NS, bool TMA>
static size_t smem_f() {
  typedef TileCfg<T, K, RX, RY, NS> G;
  return TMA ? G::SMEM + (size_t)RX * RY * (sizeof(typename C2<T>::type) + sizeof(T)) + 128 : G::SMEM;
}

template <typename T, int K, int RX, int RY, int NS, bool TMA = false>
static cudaError_t launch_f(const Inst2D* d_insts, const TileItem* d_items, int n_items, int j_step,
                            int grid, cudaStream_t s, int* wait_flag = nullptr) {
  typedef TileCfg<T, K, RX, RY, NS> G;
  return launch_pdl(rk4_2d_fused<T, K, RX, RY, NS, TMA>, dim3(grid), dim3(G::NT), smem_f<T, K, RX, RY, NS, TMA>(), s,
                    d_insts, d_items, n_items, j_step, wait_flag);
}

// Sets the shared-memory attribute (outside any capture) and returns CTAs per SM.
template <typename T, int K, int RX, int RY, int NS, bool TMA = false>
static int occ_f() {
  typedef TileCfg<T, K, RX, RY, NS> G;
  auto kern = rk4_2d_fused<T, K, RX, RY, NS, TMA>;
  const size_t smem = smem_f<T, K, RX, RY, NS, TMA>();
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, G::NT, smem) != cudaSuccess) return 0;
  return nb;
}

template <typename T, int K, int RX, int RY, int NS>
static cudaError_t launch_ft(const Inst2D* d_insts, const TileItem* d_items, int n_items, int j_step,
                             int grid, cudaStream_t s, int* wait_flag) {
  return launch_f<T, K, RX, RY, NS, true>(d_insts, d_items, n_items, j_step, grid, s, wait_flag);
}
template <typename T, int K, int RX, int RY, int NS>
static int occ_ft() {
  return occ_f<T, K, RX, RY, NS, true>();
}

template <int K, int NW, int NJ, bool TMA>
static cudaError_t launch_r(const Inst2D* d_insts, const TileItem* d_items, int n_items, int j_step,
                            int grid, cudaStream_t s, int* wait_flag = nullptr) {
  typedef RegCfg<K, NW, NJ> G;
  return launch_pdl(rk4_2d_reg<K, NW, NJ, TMA>, dim3(grid), dim3(G::NT), G::SMEM, s, d_insts, d_items, n_items, j_step,
                    wait_flag);
}
// Sets the shared-memory attribute (outside any capture) and returns CTAs per SM.
template <int K, int NW, int NJ, bool TMA>
static int occ_r() {
  typedef RegCfg<K, NW, NJ> G;
  auto kern = rk4_2d_reg<K, NW, NJ, TMA>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, G::NT, G::SMEM) != cudaSuccess) return 0;
  return nb;
}

#define NLSG_REG_SHAPES(K, TMA, CALL, ...)                                 \
  switch (shape) {                                                         \
    case TILE_R64x80: return CALL<K, 16, 5, TMA>(__VA_ARGS__);             \
    case TILE_R64x96: return CALL<K, 12, 8, TMA>(__VA_ARGS__);             \
    case TILE_R64x96S: return CALL<K, 8, 12, TMA>(__VA_ARGS__);            \
    case TILE_R64x64: return CALL<K, 16, 4, TMA>(__VA_ARGS__);             \
    case TILE_R64x72: return CALL<K, 8, 9, TMA>(__VA_ARGS__);              \
    case TILE_R64x72W: return CALL<K, 12, 6, TMA>(__VA_ARGS__);            \
    case TILE_R64x80S: return CALL<K, 8, 10, TMA>(__VA_ARGS__);            \
  }

#define NLSG_SHAPES(T, K, CALL, ...)                                        \
  switch (shape) {                                                         \
    case TILE_64x64: return CALL<T, K, 64, 64, 8>(__VA_ARGS__);            \
    case TILE_128x32: return CALL<T, K, 128, 32, 4>(__VA_ARGS__);          \
    case TILE_32x32: return CALL<T, K, 32, 32, 8>(__VA_ARGS__);            \
    case TILE_64x64W: return CALL<T, K, 64, 64, 16>(__VA_ARGS__);          \
    case TILE_128x32W: return CALL<T, K, 128, 32, 8>(__VA_ARGS__);         \
    case TILE_64xO64: return CALL<T, K, 64, 64 + 8 * K, 8>(__VA_ARGS__);   \
    case TILE_64xO64M: return CALL<T, K, 64, 64 + 8 * K, (K == 1 ? 12 : 10)>(__VA_ARGS__); \
  }

int fused_2d_blocks_per_sm(int dtype, int K, int shape) {
  if (!tile_supported(shape, dtype)) return 0;
  if (dtype == NLS_C128) {
    if (shape != TILE_32x32) return 0;
    if (K == 1) return occ_f<double, 1, 32, 32, 8>();
    if (K == 2) return occ_f<double, 2, 32, 32, 8>();
    return 0;
  }
  if (reg_shape(shape)) {
    if (K == 1) { NLSG_REG_SHAPES(1, false, occ_r) }
    if (K == 2) { NLSG_REG_SHAPES(2, false, occ_r) }
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
  if (reg_shape(shape)) {
    if (K == 1) { NLSG_REG_SHAPES(1, false, launch_r, d_insts, d_items, n_items, j_step, grid, s) }
    if (K == 2) { NLSG_REG_SHAPES(2, false, launch_r, d_insts, d_items, n_items, j_step, grid, s) }
    return cudaErrorInvalidValue;
  }
  if (K == 1) { NLSG_SHAPES(float, 1, launch_f, d_insts, d_items, n_items, j_step, grid, s) }
  if (K == 2) { NLSG_SHAPES(float, 2, launch_f, d_insts, d_items, n_items, j_step, grid, s) }
  return cudaErrorInvalidValue;
}

// ---- TMA path (complex64): tensor maps, launch, occupancy, wait-timeout flag

int fused_2d_tma_blocks_per_sm(int K, int shape) {
  if (!tile_supported(shape, NLS_C64)) return 0;
  if (reg_shape(shape)) {
    if (K == 1) { NLSG_REG_SHAPES(1, true, occ_r) }
    if (K == 2) { NLSG_REG_SHAPES(2, true, occ_r) }
    return 0;
  }
  if (K == 1) { NLSG_SHAPES(float, 1, occ_ft) }
  if (K == 2) { NLSG_SHAPES(float, 2, occ_ft) }
  return 0;
}

cudaError_t launch_2d_fused_tma(int K, int shape, const Inst2D* d_insts, const TileItem* d_items,
                                int n_items, int j_step, int grid, cudaStream_t s, int* wait_flag) {
  if (n_items <= 0) return cudaSuccess;
  if (!tile_supported(shape, NLS_C64) || !wait_flag) return cudaErrorInvalidValue;
  if (reg_shape(shape)) {
    if (K == 1) { NLSG_REG_SHAPES(1, true, launch_r, d_insts, d_items, n_items, j_step, grid, s, wait_flag) }
    if (K == 2) { NLSG_REG_SHAPES(2, true, launch_r, d_insts, d_items, n_items, j_step, grid, s, wait_flag) }
    return cudaErrorInvalidValue;
  }
  if (K == 1) { NLSG_SHAPES(float, 1, launch_ft, d_insts, d_items, n_items, j_step, grid, s, wait_flag) }
  if (K == 2) { NLSG_SHAPES(float, 2, launch_ft, d_insts, d_items, n_items, j_step, grid, s, wait_flag) }
  return cudaErrorInvalidValue;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool tma_eligible(int dtype, int n, const void* u0, const void* u1, const void* P) {
  if (dtype != NLS_C64 || n % 4 != 0) return false;     // row pitch of the pump: multiple of 16 B
  auto al = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  return al(u0) && al(u1) && al(P) && encode_fn() != nullptr;
}

int tma_encode_2d(int shape, int K, int n, const void* u0, const void* u1, const void* P, void* out_maps) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return 1;
  CUtensorMap* m = reinterpret_cast<CUtensorMap*>(out_maps);
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint32_t box[2] = {(cuuint32_t)tile_region_x(shape), (cuuint32_t)tile_region_y(shape, K)};
  const cuuint32_t estr[2] = {1, 1};
  const cuuint64_t su[1] = {(cuuint64_t)n * 8};
  const cuuint64_t sp[1] = {(cuuint64_t)n * 4};
  const void* srcs[2] = {u0, u1};
  for (int b = 0; b < 2; ++b)
    if (enc(&m[b], CU_TENSOR_MAP_DATA_TYPE_INT64, 2, const_cast<void*>(srcs[b]), dims, su, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 2;
  if (enc(&m[2], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(P), dims, sp, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 3;
  return 0;
}

size_t tma_map_bytes() { return 3 * sizeof(CUtensorMap); }

cudaError_t tile_tx_extra_set(unsigned bytes) {
  return cudaMemcpyToSymbol(g_tile_tx_extra, &bytes, sizeof(bytes));
}

// ---- streaming step (complex64): occupancy, launch, work items

template <int K, bool EVEN>
static int occ_s() {
  typedef StreamCfg<K> G;
  auto kern = rk4_2d_stream<K, EVEN>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, G::NT, G::SMEM) != cudaSuccess) return 0;
  return nb;
}

int stream_2d_blocks_per_sm(int K) {
  if (K == 1) return std::min(occ_s<1, true>(), occ_s<1, false>());
  if (K == 2) return std::min(occ_s<2, true>(), occ_s<2, false>());
  return 0;
}
int stream_2d_warps_per_block() { return StreamCfg<1>::WARPS; }

int stream_kind(int n, const void* u0, const void* u1, const void* P) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(u0) | reinterpret_cast<uintptr_t>(u1) | reinterpret_cast<uintptr_t>(P);
  return (n % 2 == 0 && (a & 15) == 0) ? STREAM_EVEN : STREAM_ODD;
}

template <int K>
static cudaError_t launch_s(int kinds, const StreamLaunch& L, int j0, int nsteps, int grid, cudaStream_t s) {
  typedef StreamCfg<K> G;
  if (K != 1) {
    if (kinds & STREAM_EVEN)
      rk4_2d_stream<K, true><<<grid, G::NT, G::SMEM, s>>>(L.insts, L.items, L.n_items, j0, nsteps, L.counter,
                                                          L.dep_range, L.deps, L.flags, L.wait_flag);
    if (kinds & STREAM_ODD)
      rk4_2d_stream<K, false><<<grid, G::NT, G::SMEM, s>>>(L.insts, L.items, L.n_items, j0, nsteps, L.counter,
                                                           L.dep_range, L.deps, L.flags, L.wait_flag);
    return cudaGetLastError();
  }
  cudaError_t e = cudaSuccess;
  if (kinds & STREAM_EVEN)
    e = launch_pdl(rk4_2d_stream<K, true>, dim3(grid), dim3(G::NT), G::SMEM, s, L.insts, L.items, L.n_items, j0,
                   nsteps, L.counter, L.dep_range, L.deps, L.flags, L.wait_flag);
  if (!e && (kinds & STREAM_ODD))
    e = launch_pdl(rk4_2d_stream<K, false>, dim3(grid), dim3(G::NT), G::SMEM, s, L.insts, L.items, L.n_items, j0,
                   nsteps, L.counter, L.dep_range, L.deps, L.flags, L.wait_flag);
  return e;
}

cudaError_t launch_2d_stream(int K, int kinds, const StreamLaunch& L, int j0, int nsteps, int grid, cudaStream_t s) {
  if (L.n_items <= 0 || nsteps <= 0 || !(kinds & (STREAM_EVEN | STREAM_ODD))) return cudaSuccess;
  if (!L.counter || grid <= 0) return cudaErrorInvalidValue;
  // several steps per launch: one kind only (the 16-byte paired copies bypass L1), a dependency
  // list, flags, a status word, and a work index that fits an int
  if (nsteps > 1 && (kinds != STREAM_EVEN || !L.dep_range || !L.deps || !L.flags || !L.wait_flag ||
                     (int64_t)L.n_items * nsteps > INT32_MAX))
    return cudaErrorInvalidValue;
  if (K == 1) return launch_s<1>(kinds, L, j0, nsteps, grid, s);
  if (K == 2) return launch_s<2>(kinds, L, j0, nsteps, grid, s);
  return cudaErrorInvalidValue;
}

cudaError_t stream_dep_extra_set(unsigned extra) {
  return cudaMemcpyToSymbol(g_stream_dep_extra, &extra, sizeof(extra));
}

void stream_strips(int n, int K, std::vector<StripGeom>& out) {
  const int H = 4 * K;
  out.clear();
  if (n <= 64) {
    out.push_back(StripGeom{0, 0, n});
    return;
  }
  // first strip against the left grid edge (no left halo), interior strips with a halo of H on
  // both sides, last strip against the right grid edge
  out.push_back(StripGeom{0, 0, 64 - H});
  int ox = 64 - H;
  while (ox + 64 - H < n) {
    out.push_back(StripGeom{ox - H, ox, ox + 64 - 2 * H});
    ox += 64 - 2 * H;
  }
  out.push_back(StripGeom{n - 64, ox, n});
}

// Row segments of one strip: nseg = ceil(n / ly) pieces of near-equal height.
static void segments(int n, int ly, std::vector<std::pair<int, int>>& out) {
  out.clear();
  const int nseg = std::max(1, (n + ly - 1) / std::max(1, ly));
  for (int k = 0; k < nseg; ++k) {
    const int a = (int)((int64_t)k * n / nseg), b = (int)((int64_t)(k + 1) * n / nseg);
    if (b > a) out.emplace_back(a, b);
  }
}

int stream_choose_ly_search(const std::vector<int>& ns, int K, int64_t slots);

// Makespan (in row iterations) of the items that segment height ly gives, taken longest first by
// `slots` warps that each take the next item when done (the kernel's dynamic schedule).  An item
// costs its rows, the 4K rows of drain past its end and, below the grid's first row, 4K rows of
// warm-up, plus a start-up of kStartup row iterations (taking the item, reading the instance,
// waiting for the first prefetched row).
static double stream_makespan(const std::vector<int>& ns, const std::vector<int>& nstrips, int K, int ly,
                              int64_t slots, double bound) {
  constexpr double kStartup = 8.0;
  std::vector<std::pair<int, int>> sg;
  std::vector<double> cost;
  double total = 0.0, longest = 0.0;
  for (size_t k = 0; k < ns.size(); ++k) {
    segments(ns[k], ly, sg);
    for (auto& g : sg) {
      const double it = (double)(g.second - g.first) + 4 * K + (g.first > 0 ? 4 * K : 0) + kStartup;
      for (int q = 0; q < nstrips[k]; ++q) cost.push_back(it);
      total += it * nstrips[k];
      longest = std::max(longest, it);
    }
  }
  slots = std::max<int64_t>(1, slots);
  if ((int64_t)cost.size() <= slots) return longest;
  const double lower = std::max(longest, total / (double)slots);
  if (lower >= bound) return lower;          // cannot beat the best so far
  std::sort(cost.begin(), cost.end(), std::greater<double>());
  std::priority_queue<double, std::vector<double>, std::greater<double>> warps;
  for (int64_t w = 0; w < slots; ++w) warps.push(0.0);
  for (double c : cost) {
    const double t = warps.top();
    warps.pop();
    warps.push(t + c);
  }
  double end = 0.0;
  while (!warps.empty()) {
    end = std::max(end, warps.top());
    warps.pop();
  }
  return end;
}

int stream_choose_ly(const std::vector<int>& ns, int K, int64_t slots) {
  // a single grid's choice depends only on (n, K, slots): remember it
  static std::mutex mu;
  static std::map<std::tuple<int, int, int64_t>, int> single;
  if (ns.size() == 1) {
    std::lock_guard<std::mutex> lk(mu);
    auto it = single.find(std::make_tuple(ns[0], K, slots));
    if (it != single.end()) return it->second;
  }
  const int ly = stream_choose_ly_search(ns, K, slots);
  if (ns.size() == 1) {
    std::lock_guard<std::mutex> lk(mu);
    single[std::make_tuple(ns[0], K, slots)] = ly;
  }
  return ly;
}

int stream_choose_ly_search(const std::vector<int>& ns, int K, int64_t slots) {
  int nmax = 1;
  for (int n : ns) nmax = std::max(nmax, n);
  std::vector<int> nstrips(ns.size());
  std::vector<StripGeom> st;
  for (size_t k = 0; k < ns.size(); ++k) {
    stream_strips(ns[k], K, st);
    nstrips[k] = (int)st.size();
  }
  // candidate heights: the largest grid split into 1..64 segments, and a coarse ladder below
  std::vector<int> cand;
  for (int seg = 1; seg <= 64; ++seg) cand.push_back(std::max(16, (nmax + seg - 1) / seg));
  for (int ly = 16; ly < nmax; ly += (ly < 128 ? 8 : (ly < 512 ? 32 : 128))) cand.push_back(ly);
  std::sort(cand.begin(), cand.end());
  cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  int best = nmax;
  double best_c = stream_makespan(ns, nstrips, K, nmax, slots, 1e300);
  for (int ly : cand) {
    const double c = stream_makespan(ns, nstrips, K, ly, slots, best_c);
    if (c < best_c * 0.999) {
      best_c = c;
      best = ly;
    }
  }
  return best;
}

int stream_choose_ly_multi(const std::vector<int>& ns, int K, int64_t slots, double items_per_slot, int min_ly) {
  // the tallest segment (least warm-up and drain) whose items still number items_per_slot per
  // resident warp; -1 when that needs segments below min_ly rows
  int nmax = 1;
  std::vector<int> nstrips(ns.size());
  std::vector<StripGeom> st;
  for (size_t k = 0; k < ns.size(); ++k) {
    nmax = std::max(nmax, ns[k]);
    stream_strips(ns[k], K, st);
    nstrips[k] = (int)st.size();
  }
  std::vector<std::pair<int, int>> sg;
  for (int seg = 1;; ++seg) {
    const int ly = (nmax + seg - 1) / seg;
    if (ly < min_ly) return -1;
    int64_t items = 0;
    for (size_t k = 0; k < ns.size(); ++k) {
      segments(ns[k], ly, sg);
      items += (int64_t)sg.size() * nstrips[k];
    }
    if ((double)items >= items_per_slot * (double)slots) return ly;
  }
}

void stream_items(int inst, int n, int K, int ly, std::vector<StripItem>& out, int extra_strips) {
  std::vector<StripGeom> st;
  std::vector<std::pair<int, int>> sg, sg1;
  stream_strips(n, K, st);
  segments(n, ly, sg);
  // the first extra_strips strips are cut into one segment more
  const int nseg = (int)sg.size();
  for (int k = 0; k < nseg + 1; ++k) {
    const int a = (int)((int64_t)k * n / (nseg + 1)), b = (int)((int64_t)(k + 1) * n / (nseg + 1));
    if (b > a) sg1.emplace_back(a, b);
  }
  for (size_t q = 0; q < st.size(); ++q)
    for (auto& y : ((int)q < extra_strips && nseg < n ? sg1 : sg))
      out.push_back(StripItem{inst, (uint16_t)st[q].x0, (uint16_t)st[q].ox0, (uint16_t)st[q].ox1, (uint16_t)y.first,
                              (uint16_t)y.second, 0});
}

void stream_list_items(const std::vector<int>& ns, int K, int ly, int64_t slots, std::vector<StripItem>& out) {
  // A list of fewer items than resident warps, short of them by no more than its strip count,
  // takes exactly one item per warp: strips of the largest grids get one segment more.  Every SM
  // then holds as many items as warps (an SM holding one item fewer than the others would finish
  // its share early and idle while the rest finish theirs).
  std::vector<StripGeom> st;
  std::vector<std::pair<int, int>> sg;
  std::vector<int> nstrips(ns.size()), extra(ns.size(), 0);
  int64_t items = 0, strips = 0;
  for (size_t k = 0; k < ns.size(); ++k) {
    stream_strips(ns[k], K, st);
    segments(ns[k], ly, sg);
    nstrips[k] = (int)st.size();
    items += (int64_t)st.size() * sg.size();
    strips += (int64_t)st.size();
  }
  int64_t deficit = slots - items;
  // order 3 only: at order 5 the extra segments' 16 rows of warm-up and drain each cost more than
  // the balance gains (4096^2: 1.24e11 -> 1.20e11 node-steps/s; order 3: 2.17e11 -> 2.22e11)
  if (K == 1 && deficit > 0 && deficit <= strips) {
    std::vector<int> order(ns.size());
    for (size_t k = 0; k < ns.size(); ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ns[a] > ns[b]; });
    for (int k : order) {
      const int take = (int)std::min<int64_t>(deficit, nstrips[k]);
      extra[k] = take;
      deficit -= take;
      if (!deficit) break;
    }
  }
  for (size_t k = 0; k < ns.size(); ++k) stream_items((int)k, ns[k], K, ly, out, extra[k]);
}

void stream_deps(const std::vector<StripItem>& items, const std::vector<int>& ns, int K, std::vector<int2>& range,
                 std::vector<int>& deps) {
  const int H = 4 * K;
  range.assign(items.size(), int2{0, 0});
  deps.clear();
  // per instance and strip (by x0): its items; a strip's read and write columns only meet those of
  // the strips within two of it, and segments may differ from strip to strip
  std::map<int, std::map<int, std::vector<int>>> by;
  for (size_t k = 0; k < items.size(); ++k) by[items[k].inst][items[k].x0].push_back((int)k);
  std::vector<std::vector<int>> lists(items.size());
  auto meets = [](int a0, int a1, int b0, int b1) { return a0 < b1 && b0 < a1; };
  for (auto& inst : by) {
    const int n = ns[inst.first];
    std::vector<const std::vector<int>*> strips;
    for (auto& kv : inst.second) strips.push_back(&kv.second);
    for (size_t s = 0; s < strips.size(); ++s)
      for (int k : *strips[s]) {
        const StripItem& a = items[k];
        // read region: the strip's columns and the segment's rows widened by the 4K-row warm-up
        // and drain; written region: the output columns and the segment's rows
        const int ar0 = std::max(0, (int)a.y0 - H), ar1 = std::min(n, (int)a.y1 + H);
        const int ac1 = std::min(n, (int)a.x0 + 64);
        for (size_t s2 = s >= 2 ? s - 2 : 0; s2 < std::min(strips.size(), s + 3); ++s2)
          for (int d : *strips[s2]) {
            const StripItem& b = items[d];
            const int br0 = std::max(0, (int)b.y0 - H), br1 = std::min(n, (int)b.y1 + H);
            const int bc1 = std::min(n, (int)b.x0 + 64);
            const bool raw = meets(ar0, ar1, b.y0, std::min(n, (int)b.y1)) && meets(a.x0, ac1, b.ox0, b.ox1);
            const bool war = meets(br0, br1, a.y0, std::min(n, (int)a.y1)) && meets(b.x0, bc1, a.ox0, a.ox1);
            if (raw || war) lists[k].push_back(d);
          }
      }
  }
  for (size_t k = 0; k < items.size(); ++k) {
    std::sort(lists[k].begin(), lists[k].end());
    range[k] = int2{(int)deps.size(), (int)lists[k].size()};
    deps.insert(deps.end(), lists[k].begin(), lists[k].end());
  }
}

void stream_sort_items(std::vector<StripItem>& items) {
  std::stable_sort(items.begin(), items.end(), [](const StripItem& a, const StripItem& b) {
    return (a.y1 - a.y0) > (b.y1 - b.y0);
  });
}

// Rows of 32 nodes per CTA of the stage kernels.  Two (64-thread CTAs) spread a small grid evenly
// over the SMs: 256^2 is 1024 CTAs (6-7 per SM) instead of 256 of 8 rows, where 104 SMs ran two
// and 48 one, idle for half the kernel (config 1: 23.2 -> 21.5 us per step; 1024^2 unchanged).
#ifndef NLSG_STAGE2D_ROWS
#define NLSG_STAGE2D_ROWS 2
#endif
cudaError_t launch_2d_stage(int dtype, int n, int s, const void* src, void* u, const void* P,
                            void* acc, void* dst, double dt, const PhysD& ph, const Stencil2D& op,
                            cudaStream_t st) {
  constexpr int RY = NLSG_STAGE2D_ROWS;
  const dim3 grid((n + 31) / 32, (n + RY - 1) / RY);
  if (dtype == NLS_C128) {
    const Params<double> p = make_params<double>(ph, dt, op.center, op.w[0], op.w[1]);
    if (op.K == 1) return launch_pdl(rk4_2d_stage<double, 1>, grid, dim3(32 * RY), 0, st, n, s, src, u, P, acc, dst, p);
    if (op.K == 2) return launch_pdl(rk4_2d_stage<double, 2>, grid, dim3(32 * RY), 0, st, n, s, src, u, P, acc, dst, p);
    return cudaErrorInvalidValue;
  }
  const Params<float> p = make_params<float>(ph, dt, op.center, op.w[0], op.w[1]);
  if (op.K == 1) return launch_pdl(rk4_2d_stage<float, 1>, grid, dim3(32 * RY), 0, st, n, s, src, u, P, acc, dst, p);
  if (op.K == 2) return launch_pdl(rk4_2d_stage<float, 2>, grid, dim3(32 * RY), 0, st, n, s, src, u, P, acc, dst, p);
  return cudaErrorInvalidValue;
}

cudaError_t launch_rhs_2d(int dtype, int n, const void* u, const void* P, void* v, const PhysD& ph,
                          const Stencil2D& op, cudaStream_t st) {
  dim3 grid((n + 31) / 32, (n + 7) / 8);
  if (dtype == NLS_C128) {
    const Params<double> p = make_params<double>(ph, 0.0, op.center, op.w[0], op.w[1]);
    if (op.K == 1) rhs_2d<double, 1><<<grid, 256, 0, st>>>(n, u, P, v, p);
    else if (op.K == 2) rhs_2d<double, 2><<<grid, 256, 0, st>>>(n, u, P, v, p);
    else return cudaErrorInvalidValue;
  } else {
    const Params<float> p = make_params<float>(ph, 0.0, op.center, op.w[0], op.w[1]);
    if (op.K == 1) rhs_2d<float, 1><<<grid, 256, 0, st>>>(n, u, P, v, p);
    else if (op.K == 2) rhs_2d<float, 2><<<grid, 256, 0, st>>>(n, u, P, v, p);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace nlsg
