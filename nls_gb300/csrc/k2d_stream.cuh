// k2d_stream.cuh -- streaming (wavefront) fused RK4 step over 2-D strips (complex64, sm_103a).
//
// Same contract as the tile kernels (one launch = one complete RK4 step of every listed piece of
// every listed instance, nls/nls.f90:892-900, one HBM pass per step), organised for a warp that
// never waits for another warp:
//   * a work item is a vertical strip of 64 columns and a segment of rows [y0, y1) of one
//     instance; lane l holds the node pair (x0 + 2l, x0 + 2l + 1), planar (X = real parts of both
//     nodes, Y = imaginary parts) so the right-hand side runs on the packed FP32x2 pipe;
//   * the warp walks down the rows.  At row i it loads row i (state and pump) and evaluates the
//     four RK4 stages as a wavefront: stage 1 at row i-K, stage 2 at row i-2K, stage 3 at row i-3K
//     and stage 4 (the update) at row i-4K, each from the window of its input rows held in
//     registers (window of W = 4K+1 rows, indexed by row modulo W; the loop is unrolled by W so
//     every index is a compile-time constant).  Rows are read and written exactly once per step;
//     the only recomputation is the 4K columns of horizontal halo at strip edges inside the grid
//     and the 4K rows of warm-up and drain at segment ends inside the grid;
//   * horizontal neighbours come from the adjacent lanes by warp shuffle; at a strip edge that is
//     the grid edge the missing neighbours are masked to zero (the reference's truncated
//     operator), and columns beyond the grid hold zero state with a zero stencil weight, so their
//     stage values stay exactly zero;
//   * rows are prefetched D rows ahead with cp.async into a per-warp shared-memory ring (each lane
//     copies and later reads only its own bytes, so no warp synchronisation is involved; rows
//     outside the grid arrive zero-filled through the copy's source size);
//   * warps take items from a launch-wide atomic counter (items are listed longest first), so
//     uneven items balance across the GPU; the last warp of the launch resets the counter for the
//     next launch.  No thread ever waits on another thread.
#pragma once

#include <type_traits>

namespace nlsg {

// Calls f(std::integral_constant<int, P>) for P = B .. E-1 (compile-time unrolling).
template <int B, int E>
struct StaticFor {
  template <typename F>
  __device__ __forceinline__ static void run(F&& f) {
    f(std::integral_constant<int, B>{});
    StaticFor<B + 1, E>::run(f);
  }
};
template <int E>
struct StaticFor<E, E> {
  template <typename F>
  __device__ __forceinline__ static void run(F&&) {}
};

// Unroll period (= window length = ring depth) at order 3, and warps per CTA (the warps of a CTA
// share nothing, so this only sets the granularity of occupancy).
#ifndef NLSG_STREAM_W_K1
#define NLSG_STREAM_W_K1 5
#endif
#ifndef NLSG_STREAM_WARPS
#define NLSG_STREAM_WARPS 1
#endif

// Ring depth in blocks of W rows per order (the prefetch distance grows with it; registers do
// not).  Order 3: two blocks (8 rows ahead; one block, 3 rows ahead, left the warps waiting for
// their rows: 2.04e11 against 2.17e11 node-steps/s on a 4096^2 grid); order 5: one block (16 rows
// ahead with two blocks was 6 % slower).
#ifndef NLSG_STREAM_RING_K1
#define NLSG_STREAM_RING_K1 2
#endif
#ifndef NLSG_STREAM_RING_K2
#define NLSG_STREAM_RING_K2 1
#endif

template <int K>
struct StreamCfg {
  static constexpr int H = 4 * K;          // horizontal halo of a strip edge inside the grid
  // W is the number of rows each register window holds (at least 4K + 1) and the unroll period,
  // so the window slot of row i is the unroll phase (i - first row) mod W, a compile-time
  // constant.  The shared-memory row ring holds M blocks of W rows: row i sits in block
  // ((i - first row) / W) mod M at the same phase, so a ring address is a block base (one
  // register, advanced once per W rows) plus a compile-time offset.
  static constexpr int W = K == 1 ? NLSG_STREAM_W_K1 : 9;
  static constexpr int M = K == 1 ? NLSG_STREAM_RING_K1 : NLSG_STREAM_RING_K2;
  static constexpr int R = W * M;          // ring slots per warp
  static constexpr int D = R - 2;          // rows prefetched ahead of the one being consumed
  static constexpr int ROWB = 64 * 8 + 64 * 4;   // one row of a strip: 64 complex64 + 64 float32
  static constexpr int WARPS = NLSG_STREAM_WARPS;   // independent warps per CTA
  static constexpr int NT = 32 * WARPS;
  // per warp: its row ring, then (after all rings) 16 bytes for the item being worked on
  static constexpr size_t SMEM = (size_t)WARPS * R * ROWB + (size_t)WARPS * 16;
  static_assert(W >= 4 * K + 1 && R % W == 0 && R >= D + 2, "window and ring");
};

// Per-warp constants of an item: broadcast pairs of the step coefficients (pre-multiplied by
// dt/2 like the register tile's, see RegConst) and per-lane stencil weights and edge masks.
struct StreamConst {
  float2 w1, nw1, w2, nw2;     // +-dt/2 w_d, zero for columns outside the grid
  float2 nwc, c3, nc4, c5, c6, c13, c14, c12, two, third;
  float mL, mR;                // 0 where the left / right neighbour lies beyond the grid edge
  float2 mL2, mR2;
};

template <int BYTES>
__device__ __forceinline__ void cp_async_sz(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "n"(BYTES), "r"(src_bytes) : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// 16-byte copy that bypasses L1 (state rows written by other SMs earlier in the same launch must
// not be served from a stale L1 line).
__device__ __forceinline__ void cp_async_cg16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Predicated global stores of a node pair and of one node (no branch around them).
__device__ __forceinline__ void st_pair_if(bool p, float2* dst, float a, float b, float c, float d) {
  asm volatile("{ .reg .pred q; setp.ne.b32 q, %0, 0; @q st.global.v4.f32 [%1], {%2, %3, %4, %5}; }"
               ::"r"((int)p), "l"(dst), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}
__device__ __forceinline__ void st_node_if(bool p, float2* dst, float a, float b) {
  asm volatile("{ .reg .pred q; setp.ne.b32 q, %0, 0; @q st.global.v2.f32 [%1], {%2, %3}; }"
               ::"r"((int)p), "l"(dst), "f"(a), "f"(b) : "memory");
}

// |u|^2 on the packed pipe (order 3, measured 2 % faster) or in scalar FMAs (order 5, where the
// packed square costs more register moves than it saves).
#ifndef NLSG_STREAM_PACKED_SQ
#define NLSG_STREAM_PACKED_SQ (K == 1)
#endif
// RK4 accumulation and stage-input updates in scalar FMAs (the packed FP32x2 operations all issue
// to one FMA pipe, scalar ones can use the other).  Measured 0.3 % slower on a 4096^2 grid; so are
// |u|^2 in scalar FMAs at order 3 (0.9 %) and the new state in four scalar FMAs (0.8 %).
#ifndef NLSG_STREAM_SCALAR_UPDATE
#define NLSG_STREAM_SCALAR_UPDATE 0
#endif


// c = m * a + b per component with a scalar multiplier (scalar FMAs)
__device__ __forceinline__ float2 sfma(float m, float2 a, float2 b) {
  return f2(__fmaf_rn(m, a.x, b.x), __fmaf_rn(m, a.y, b.y));
}
__device__ __forceinline__ float2 sadd(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }

// Slope of one stage at the centre row of the window (slot C), pre-multiplied by dt/2:
//   q = a u - i (b - wc) u + i L'u,  L'u = w1 s1 + w2 s2,  a = c3 r - c4,  b = c5 |u|^2 + c6 r,
//   r = c12 P / (c13 + c14 |u|^2)                                     (nls/nls.f90:570-650)
template <int K, int W, int C>
__device__ __forceinline__ void stream_slope(const float2 (&inX)[W], const float2 (&inY)[W], float2 pcv,
                                             const StreamConst& c, float2& qX, float2& qY) {
  constexpr int U1 = (C - 1 + W) % W, D1 = (C + 1) % W;
  const float2 X = inX[C], Y = inY[C];
  float2 mX, nmY;
  if (K == 1) {
    const float lx = __shfl_up_sync(0xffffffffu, X.y, 1), ly = __shfl_up_sync(0xffffffffu, Y.y, 1);
    const float rx = __shfl_down_sync(0xffffffffu, X.x, 1), ry = __shfl_down_sync(0xffffffffu, Y.x, 1);
    const float2 sX = add2(add2(f2(__fmaf_rn(c.mL, lx, X.y), __fmaf_rn(c.mR, rx, X.x)), inX[U1]), inX[D1]);
    const float2 sY = add2(add2(f2(__fmaf_rn(c.mL, ly, Y.y), __fmaf_rn(c.mR, ry, Y.x)), inY[U1]), inY[D1]);
    mX = mul2(c.w1, sX);
    nmY = mul2(c.nw1, sY);
  } else {
    constexpr int U2 = (C - 2 + 2 * W) % W, D2 = (C + 2) % W;
    const float2 LX = f2(__shfl_up_sync(0xffffffffu, X.x, 1), __shfl_up_sync(0xffffffffu, X.y, 1));
    const float2 LY = f2(__shfl_up_sync(0xffffffffu, Y.x, 1), __shfl_up_sync(0xffffffffu, Y.y, 1));
    const float2 RX = f2(__shfl_down_sync(0xffffffffu, X.x, 1), __shfl_down_sync(0xffffffffu, X.y, 1));
    const float2 RY = f2(__shfl_down_sync(0xffffffffu, Y.x, 1), __shfl_down_sync(0xffffffffu, Y.y, 1));
    const float2 s1X = add2(add2(f2(__fmaf_rn(c.mL, LX.y, X.y), __fmaf_rn(c.mR, RX.x, X.x)), inX[U1]), inX[D1]);
    const float2 s1Y = add2(add2(f2(__fmaf_rn(c.mL, LY.y, Y.y), __fmaf_rn(c.mR, RY.x, Y.x)), inY[U1]), inY[D1]);
    const float2 s2X = add2(add2(fma2(c.mL2, LX, mul2(c.mR2, RX)), inX[U2]), inX[D2]);
    const float2 s2Y = add2(add2(fma2(c.mL2, LY, mul2(c.mR2, RY)), inY[U2]), inY[D2]);
    mX = fma2(c.w2, s2X, mul2(c.w1, s1X));
    nmY = fma2(c.nw2, s2Y, mul2(c.nw1, s1Y));
  }
  const float2 sq = NLSG_STREAM_PACKED_SQ ? fma2(X, X, mul2(Y, Y))
                                         : f2(__fmaf_rn(X.x, X.x, Y.x * Y.x), __fmaf_rn(X.y, X.y, Y.y * Y.y));
  const float2 den = fma2(c.c14, sq, c.c13);
  const float2 r = mul2(pcv, f2(rcp_approx(den.x), rcp_approx(den.y)));
  const float2 a = fma2(c.c3, r, c.nc4);
  const float2 bw = fma2(c.c5, sq, fma2(c.c6, r, c.nwc));
  qX = fma2(a, X, fma2(bw, Y, nmY));
  qY = fma2(a, Y, fma2(neg2(bw), X, mX));
}

// The rolling windows of one warp (registers): state, c12 * pump, RK4 accumulator and the inputs
// of stages 2, 3 and 4, each by row modulo W.
template <int W>
struct StreamWin {
  float2 uX[W], uY[W], pc[W], aX[W], aY[W];
  float2 t2X[W], t2Y[W], t3X[W], t3Y[W], t4X[W], t4Y[W];
};

// EVEN: the instance's side is even and its buffers are 16-byte aligned, so a lane's node pair
// moves as one 16-byte copy (state) and one 8-byte copy (pump) and is stored as one 16-byte store;
// otherwise every node moves on its own.  Items of the other kind are skipped (the runtime
// launches both instantiations over the same item list when a group mixes them).
// Register cap a thread.  Order 3: 152 (the 5-row window fits without spilling; registers are
// allocated per SM sub-partition, so caps from 129 to 168 all give 3 warps per scheduler, 12 one-
// warp CTAs per SM, and 128, for 16, spills); order 5: 255 (8 one-warp CTAs per SM).
#ifndef NLSG_STREAM_MAXNREG_K1
#define NLSG_STREAM_MAXNREG_K1 152
#endif
#define NLSG_STREAM_BOUNDS(K) __maxnreg__(K == 1 ? NLSG_STREAM_MAXNREG_K1 : 255)

// Bound of a dependency wait: polls with a back-off of up to 1 us, about one second in all.
#ifndef NLSG_STREAM_WAIT_POLLS
#define NLSG_STREAM_WAIT_POLLS (1u << 20)
#endif

// Added to every dependency a warp waits for (a test control: a large value makes every wait
// expire, to exercise the timeout path).
__device__ unsigned g_stream_dep_extra = 0;

// One launch runs nsteps RK4 steps (j0 .. j0 + nsteps - 1) of every listed item.  Global work
// index g = t * n_items + k is step t of item k; warps take g from counter[0] in order.  With
// nsteps > 1, step t of item k first waits until every item in its dependency list (the items of
// the same instance whose writes it reads, or whose reads it overwrites, in the ping-pong buffers)
// has published step t - 1: flags[d] >= epoch + t, where epoch = counter[2] at launch (the number
// of steps published before it; the last warp advances it by nsteps).  A warp only ever waits on
// smaller indices, all taken by running warps, so the waits always end; each is also bounded
// (about a second), after which the warp sets the context's status word and goes on (the state is
// then wrong and the host reports the timeout), and warps that see the status word set stop
// waiting.
template <int K, bool EVEN>
__global__ void NLSG_STREAM_BOUNDS(K)
rk4_2d_stream(const Inst2D* __restrict__ insts, const StripItem* __restrict__ items, int n_items, int j0,
              int nsteps, unsigned* __restrict__ counter, const int2* __restrict__ dep_range,
              const int* __restrict__ deps, unsigned* __restrict__ flags, int* __restrict__ wait_flag) {
  typedef StreamCfg<K> G;
  constexpr int W = G::W, D = G::D;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // this lane's bytes of ring slot 0 (state pair, pump pair); slot s is ROWB * s further
  unsigned char* const ring_u = smem_raw + (size_t)warp * G::R * G::ROWB + lane * 16;
  unsigned char* const ring_p = smem_raw + (size_t)warp * G::R * G::ROWB + 512 + lane * 8;
  const uint32_t ring_u32 = smem_u32(ring_u), ring_p32 = smem_u32(ring_p);

  auto fetch = [&]() -> int {
    unsigned v = 0;
    if (lane == 0) v = atomicAdd(&counter[0], 1u);
    return (int)__shfl_sync(0xffffffffu, v, 0);
  };
  // the previous launch's states and its reset of the counter first (programmatic launch; order 3
  // only, where launches are short enough for it to matter: at order 5 the two instructions push
  // the 255-register loop into spilling)
  if (K == 1) {
    pdl_wait();
    pdl_trigger();
  }

  const bool multi = nsteps > 1;
  // the flag index and value this warp publishes when its item is done (kept in shared memory,
  // out of the registers of the row loop)
  volatile unsigned* const pub = reinterpret_cast<volatile unsigned*>(smem_raw + (size_t)G::WARPS * G::R * G::ROWB) +
                                 4 * warp;
  const int total = n_items * nsteps;
  for (int g = fetch(); g < total; g = fetch()) {
    const int t = multi ? g / n_items : 0;
    const int idx = g - t * n_items;
    const int j_step = j0 + t;
    const unsigned epoch = multi ? *reinterpret_cast<volatile unsigned*>(&counter[2]) : 0u;
    if (multi && lane == 0) {
      pub[0] = (unsigned)idx;
      pub[1] = epoch + (unsigned)t + 1u;
    }
    if (multi && t > 0) {
      // wait for the dependencies' step t - 1 (32 flags per poll, one per lane)
      const int2 dr = dep_range[idx];
      const unsigned need = epoch + (unsigned)t + g_stream_dep_extra;
      for (int base = 0; base < dr.y; base += 32) {
        const int d = base + lane < dr.y ? deps[dr.x + base + lane] : -1;
        unsigned ns = 32, polls = 0;
        while (true) {
          const bool ok = d < 0 || (int)(ld_acquire_gpu(&flags[d]) - need) >= 0;
          if (__all_sync(0xffffffffu, ok)) break;
          // another warp timed out (decided for the whole warp: lanes may read the word at
          // different moments)
          if (__any_sync(0xffffffffu, *reinterpret_cast<volatile int*>(wait_flag) != 0)) break;
          if (++polls >= NLSG_STREAM_WAIT_POLLS) {
            if (lane == 0) atomicExch(wait_flag, 1);
            break;
          }
          __nanosleep(ns);
          ns = ns < 1024 ? 2 * ns : 1024;
        }
      }
      __syncwarp();
    }
    {
    const StripItem it = items[idx];
    const Inst2D& I = insts[it.inst];
    if ((int64_t)j_step >= I.steps) goto published;
    const int n = I.n;
    const int par = (I.parity + j_step) & 1;
    const float2* __restrict__ src = reinterpret_cast<const float2*>(I.u[par]);
    float2* __restrict__ dst = reinterpret_cast<float2*>(I.u[par ^ 1]);
    const float* __restrict__ Pg = reinterpret_cast<const float*>(I.P);
    const bool even = !(n & 1) &&
                      ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) |
                        reinterpret_cast<uintptr_t>(Pg)) & 15) == 0;
    if (even != EVEN) goto published;
    const int x = (int)it.x0 + 2 * lane;
    const bool in0 = x < n, in1 = x + 1 < n;
    const bool out0 = in0 && x >= (int)it.ox0 && x < (int)it.ox1;
    const bool out1 = in1 && x + 1 >= (int)it.ox0 && x + 1 < (int)it.ox1;
    const int y0 = it.y0, y1 = it.y1;
    // per-lane column offsets clamped into the grid (a lane beyond it copies zero bytes from
    // column 0) and the byte counts of its copies
    const float2* __restrict__ src0 = src + (in0 ? x : 0);
    const float2* __restrict__ src1 = src + (in1 ? x + 1 : 0);
    const float* __restrict__ P0 = Pg + (in0 ? x : 0);
    const float* __restrict__ P1 = Pg + (in1 ? x + 1 : 0);
    const uint32_t szu0 = EVEN ? (in0 ? 16u : 0u) : (in0 ? 8u : 0u), szu1 = in1 ? 8u : 0u;
    const uint32_t szp0 = EVEN ? (in0 ? 8u : 0u) : (in0 ? 4u : 0u), szp1 = in1 ? 4u : 0u;

    StreamConst c;
    {
      const Params<float>& p = I.pf;
      const float h = p.half_dt;
      const float w1 = h * p.w1, w2 = h * p.w2;
      c.w1 = f2(in0 ? w1 : 0.f, in1 ? w1 : 0.f);
      c.nw1 = f2(in0 ? -w1 : 0.f, in1 ? -w1 : 0.f);
      c.w2 = f2(in0 ? w2 : 0.f, in1 ? w2 : 0.f);
      c.nw2 = f2(in0 ? -w2 : 0.f, in1 ? -w2 : 0.f);
      c.nwc = f2(-(h * p.wc), -(h * p.wc));
      c.c3 = f2(h * p.c3, h * p.c3);
      c.nc4 = f2(-(h * p.c4), -(h * p.c4));
      c.c5 = f2(h * p.c5, h * p.c5);
      c.c6 = f2(h * p.c6, h * p.c6);
      c.c13 = f2(p.c13, p.c13);
      c.c14 = f2(p.c14, p.c14);
      c.c12 = f2(p.c12, p.c12);
      c.two = f2(2.f, 2.f);
      c.third = f2(1.f / 3.f, 1.f / 3.f);
      c.mL = (lane == 0 && it.x0 == 0) ? 0.f : 1.f;
      c.mR = (lane == 31 && (int)it.x0 + 64 == n) ? 0.f : 1.f;
      c.mL2 = f2(c.mL, c.mL);
      c.mR2 = f2(c.mR, c.mR);
    }

    const int ib = y0 - 4 * K > 0 ? y0 - 4 * K : 0;   // first row loaded
    const int ie = y1 + 4 * K;                        // one past the last iteration
    // iterations whose load row and four stage rows all lie inside the grid and inside the rows
    // this segment needs, and whose prefetch row lies inside the grid and the segment: no checks
    const int clean_lo = y0 + 4 * K, clean_hi = (n < ie ? n : ie) - D;

    // cp.async of one row into the ring slot at byte offset base + SLOT * ROWB, the row at element
    // offset roff (row * n) from the lane's columns; every lane copies its own node pair.  FULL:
    // the row lies inside the grid; otherwise rows beyond it arrive zero-filled.
    auto issue_row = [&](uint32_t base, auto SLOTc, auto FULLc, int row, uint32_t roff) {
      constexpr int SLOT = decltype(SLOTc)::value;
      constexpr bool FULL = decltype(FULLc)::value;
      const bool rin = FULL || row < n;
      const uint32_t o = rin ? roff : 0u;
      const uint32_t du = ring_u32 + base + SLOT * G::ROWB, dp = ring_p32 + base + SLOT * G::ROWB;
      if (EVEN) {
        cp_async_cg16(du, src0 + o, rin ? szu0 : 0u);
        cp_async_sz<8>(dp, P0 + o, rin ? szp0 : 0u);
      } else {
        cp_async_sz<8>(du, src0 + o, rin ? szu0 : 0u);
        cp_async_sz<8>(du + 8, src1 + o, rin ? szu1 : 0u);
        cp_async_sz<4>(dp, P0 + o, rin ? szp0 : 0u);
        cp_async_sz<4>(dp + 4, P1 + o, rin ? szp1 : 0u);
      }
    };

    StreamWin<W> w;
#pragma unroll
    for (int s = 0; s < W; ++s) {
      w.uX[s] = w.uY[s] = w.pc[s] = w.aX[s] = w.aY[s] = f2(0.f, 0.f);
      w.t2X[s] = w.t2Y[s] = w.t3X[s] = w.t3Y[s] = w.t4X[s] = w.t4Y[s] = f2(0.f, 0.f);
    }

    // element offsets (row * n) of the next row to prefetch (row ib first) and of the row stage 4
    // writes (negative only in iterations that write nothing)
    uint32_t roff = (uint32_t)ib * (uint32_t)n;
    int soff = (ib - 4 * K) * n;
    float2* const dst0 = dst + x;
    StaticFor<0, D>::run([&](auto Dc) {
      constexpr int d = decltype(Dc)::value;
      if (ib + d < ie) issue_row(0u, std::integral_constant<int, d>{}, std::false_type{}, ib + d, roff);
      async_commit();
      roff += (uint32_t)n;
    });
    // byte offsets of the ring block holding the current W rows and of the block before it
    constexpr uint32_t BLK = (uint32_t)(W * G::ROWB), RING = (uint32_t)(G::R * G::ROWB);
    uint32_t rb = 0, rbp = RING - BLK;

    // One iteration of the wavefront at row i, unroll phase P = (i - ib) mod W (row i's window
    // slot and its slot within the current ring block).  CHECK: decide per stage whether its row
    // is needed by this segment (skip it otherwise) and zero stage values of rows beyond the grid
    // (rows before the grid keep the zeros the windows start with).
    auto iter = [&](int i, auto Pc, auto CHECKc) {
      constexpr int P = decltype(Pc)::value;
      constexpr bool CHECK = decltype(CHECKc)::value;
      // row i: wait for its copy, move it into the window, prefetch row i + D (= i - 2 modulo the
      // ring: phase P - 2 of this block, or of the previous block for P < 2)
      cp_async_wait_group<D - 1>();
      {
        const float4 v = *reinterpret_cast<const float4*>(ring_u + rb + P * G::ROWB);
        const float2 p = *reinterpret_cast<const float2*>(ring_p + rb + P * G::ROWB);
        w.uX[P] = f2(v.x, v.z);
        w.uY[P] = f2(v.y, v.w);
        w.pc[P] = mul2(c.c12, p);
      }
      constexpr int SN = (P + W - 2) % W;
      const uint32_t nb = P >= 2 ? rb : rbp;
      if (!CHECK) issue_row(nb, std::integral_constant<int, SN>{}, std::true_type{}, i + D, roff);
      else if (i + D < ie) issue_row(nb, std::integral_constant<int, SN>{}, std::false_type{}, i + D, roff);
      async_commit();
      roff += (uint32_t)n;

      // stage 1 at row i - K: input u, output t2 = u + q1, a = q1
      {
        constexpr int C = ((P - K) % W + W) % W;
        const int r = i - K;
        const bool run = !CHECK || (r < n && r >= 0 && r >= y0 - 3 * K && r < y1 + 3 * K);
        if (!run) {
          // a stage that is not run still writes its slots (zero: the value rows outside the
          // grid must hold, and never read by the rows this segment needs), so every slot is
          // written once per window cycle on every path and dead until then
          w.t2X[C] = w.t2Y[C] = w.aX[C] = w.aY[C] = f2(0.f, 0.f);
        } else {
          float2 qX, qY;
          stream_slope<K, W, C>(w.uX, w.uY, w.pc[C], c, qX, qY);
          w.aX[C] = qX;
          w.aY[C] = qY;
          w.t2X[C] = NLSG_STREAM_SCALAR_UPDATE ? sadd(w.uX[C], qX) : add2(w.uX[C], qX);
          w.t2Y[C] = NLSG_STREAM_SCALAR_UPDATE ? sadd(w.uY[C], qY) : add2(w.uY[C], qY);
        }
      }
      // stage 2 at row i - 2K: input t2, output t3 = u + q2, a += 2 q2
      {
        constexpr int C = ((P - 2 * K) % W + W) % W;
        const int r = i - 2 * K;
        const bool run = !CHECK || (r < n && r >= 0 && r >= y0 - 2 * K && r < y1 + 2 * K);
        if (!run) {
          w.t3X[C] = w.t3Y[C] = f2(0.f, 0.f);
        } else {
          float2 qX, qY;
          stream_slope<K, W, C>(w.t2X, w.t2Y, w.pc[C], c, qX, qY);
          if (NLSG_STREAM_SCALAR_UPDATE) {
            w.aX[C] = sfma(2.f, qX, w.aX[C]);
            w.aY[C] = sfma(2.f, qY, w.aY[C]);
            w.t3X[C] = sadd(w.uX[C], qX);
            w.t3Y[C] = sadd(w.uY[C], qY);
          } else {
            w.aX[C] = fma2(c.two, qX, w.aX[C]);
            w.aY[C] = fma2(c.two, qY, w.aY[C]);
            w.t3X[C] = add2(w.uX[C], qX);
            w.t3Y[C] = add2(w.uY[C], qY);
          }
        }
      }
      // stage 3 at row i - 3K: input t3, output t4 = u + 2 q3, a += 2 q3
      {
        constexpr int C = ((P - 3 * K) % W + W) % W;
        const int r = i - 3 * K;
        const bool run = !CHECK || (r < n && r >= 0 && r >= y0 - K && r < y1 + K);
        if (!run) {
          w.t4X[C] = w.t4Y[C] = f2(0.f, 0.f);
        } else {
          float2 qX, qY;
          stream_slope<K, W, C>(w.t3X, w.t3Y, w.pc[C], c, qX, qY);
          if (NLSG_STREAM_SCALAR_UPDATE) {
            w.aX[C] = sfma(2.f, qX, w.aX[C]);
            w.aY[C] = sfma(2.f, qY, w.aY[C]);
            w.t4X[C] = sfma(2.f, qX, w.uX[C]);
            w.t4Y[C] = sfma(2.f, qY, w.uY[C]);
          } else {
            w.aX[C] = fma2(c.two, qX, w.aX[C]);
            w.aY[C] = fma2(c.two, qY, w.aY[C]);
            w.t4X[C] = fma2(c.two, qX, w.uX[C]);
            w.t4Y[C] = fma2(c.two, qY, w.uY[C]);
          }
        }
      }
      // stage 4 at row i - 4K: input t4; u' = u + (q1 + 2 q2 + 2 q3 + q4) / 3, stored at the row
      // offset soff (row i - 4K)
      {
        constexpr int C = ((P - 4 * K) % W + W) % W;
        const int r = i - 4 * K;
        bool run = true;
        if (CHECK) run = r >= y0 && r < y1 && r < n;
        if (run) {
          float2 qX, qY;
          stream_slope<K, W, C>(w.t4X, w.t4Y, w.pc[C], c, qX, qY);
          float2* const gst = dst0 + soff;
          const float2 nX = fma2(c.third, add2(w.aX[C], qX), w.uX[C]);
          const float2 nY = fma2(c.third, add2(w.aY[C], qY), w.uY[C]);
          if (EVEN) {
            st_pair_if(out0, gst, nX.x, nY.x, nX.y, nY.y);
          } else {
            st_node_if(out0, gst, nX.x, nY.x);
            st_node_if(out1, gst + 1, nX.y, nY.y);
          }
        }
      }
      soff += n;
    };

    for (int b = ib; b < ie; b += W) {
      if (b >= clean_lo && b + W <= clean_hi) {
        StaticFor<0, W>::run([&](auto Pc) { iter(b + decltype(Pc)::value, Pc, std::false_type{}); });
      } else {
        StaticFor<0, W>::run([&](auto Pc) {
          if (b + decltype(Pc)::value < ie) iter(b + decltype(Pc)::value, Pc, std::true_type{});
        });
      }
      rbp = rb;
      rb = rb + BLK == RING ? 0u : rb + BLK;
    }
    cp_async_wait_group<0>();
    }
  published:
    if (multi) {
      // this item's stores, then its flag (release: a warp that sees the flag sees the stores)
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release_gpu(&flags[pub[0]], pub[1]);
    }
  }

  // every warp of the launch is done taking items: the last one resets the counter (and advances
  // the epoch past the steps this launch published)
  if (lane == 0) {
    __threadfence();
    const unsigned done = atomicAdd(&counter[1], 1u);
    if (done == gridDim.x * G::WARPS - 1) {
      counter[0] = 0u;
      counter[1] = 0u;
      if (multi) counter[2] = counter[2] + (unsigned)nsteps;
      __threadfence();
    }
  }
}

}  // namespace nlsg
