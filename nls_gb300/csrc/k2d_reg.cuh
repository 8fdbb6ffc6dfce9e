// k2d_reg.cuh -- register-resident fused RK4 step over 2-D tiles (complex64, sm_103a).
//
// Same contract as rk4_2d_fused (one launch = one complete RK4 step of every listed tile, a halo
// of H = 4K nodes recomputed so the four stages need no HBM round trip), with a different
// placement of the tile on the SM:
//   * the region is 64 nodes wide and NW*NJ rows high; warp w owns rows w*NJ .. w*NJ+NJ-1 across
//     the full width, lane l the two adjacent columns 2l and 2l+1;
//   * every node's state, RK4 accumulator, pump and current stage value stay in registers for the
//     whole step, held planar per node pair (X = real parts of both nodes, Y = imaginary parts) so
//     the right-hand side runs on the packed FP32x2 pipe (FADD2/FMUL2/FFMA2);
//   * horizontal neighbours come from the adjacent lanes by warp shuffle (a warp spans the whole
//     region width, so no other warp is involved), vertical neighbours from the thread's own
//     registers; only the K rows at either end of a strip pass through shared memory, once per
//     stage, for the strips above and below.
// Shared memory then carries a few bytes per node-stage instead of every stencil operand, which
// was the limiter of the column-strip layout.  With TMA (grids whose rows are 16-byte multiples),
// one elected thread fetches the next tile's state and pump boxes (cp.async.bulk.tensor) and its
// instance descriptor (cp.async.bulk) on one mbarrier while the current tile is computed, and
// looks up the work item after that with cp.async, so no thread waits on global memory at a tile
// boundary; otherwise every thread loads its own node pairs from global memory.
#pragma once

namespace nlsg {

template <int K, int NW, int NJ>
struct RegCfg {
  static constexpr int RX = 64;
  static constexpr int RY = NW * NJ;
  static constexpr int NT = NW * 32;
  static constexpr int H = 4 * K;
  static constexpr int TX = RX - 2 * H;
  static constexpr int TY = RY - 2 * H;
  static constexpr size_t STAGE_U = (size_t)RX * RY * 8;            // complex64 state box
  static constexpr size_t STAGE_P = (size_t)RX * RY * 4;            // pump box
  static constexpr size_t EXCH = (size_t)2 * NW * 2 * K * RX * 8;   // strip-end rows, 2 parities
  static constexpr size_t DESC = sizeof(Inst2D);                   // descriptor copy (TMA path)
  static constexpr size_t OFF_DESC = STAGE_U + STAGE_P + EXCH;      // two descriptor slots
  static constexpr size_t OFF_CTRL = OFF_DESC + 2 * DESC;
  static constexpr size_t SMEM = OFF_CTRL + 128;                    // + control block
  static_assert(NJ >= K && NJ <= 32 && TY > 0, "tile layout");
  static_assert(DESC % 16 == 0, "a descriptor bulk copy moves a multiple of 16 bytes");
};

// Control block of the TMA path in shared memory.  Slot b (b = tile count & 1) names the work
// item whose boxes and descriptor the current or the next copy brings; the cand* fields are
// filled by the elected thread's asynchronous lookups of the item after that.
struct RegCtrl {
  uint64_t bar;               // transaction barrier of the boxes and the descriptor
  int item[2];                // work-list index of slot b (>= n_items: none)
  TileItem ti[2];
  int nx_idx;                 // next item to issue (elected thread)
  TileItem nx_ti;
  int nx_tiles_x, nx_parity;
  const void* nx_tmap;
  int cand_idx, slot;         // candidate after the next item; slot of the current tile
  TileItem cand_ti;           // asynchronous lookups (cp.async) of the candidate after that
  long long cand_steps;
  int cand_tiles_x, cand_parity;
  const void* cand_tmap;
};
static_assert(sizeof(RegCtrl) <= 128, "control block");


// Untiled bulk copy global -> shared, completing on the transaction barrier.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Small asynchronous global -> shared copies (cp.async), so a lookup's latency is not waited on
// until its result is needed.
template <int BYTES>
__device__ __forceinline__ void async_copy(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)),
               "l"(reinterpret_cast<uint64_t>(src)), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void async_commit_wait() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_all;" ::: "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Per-tile constants as broadcast pairs (both halves equal) for the packed pipe.  The stage
// slopes are carried pre-multiplied by dt/2 (q = dt/2 * k), so the weights and coefficients of
// the linear terms hold that factor and RK4 reads
//   t2 = u + q1, t3 = u + q2, t4 = u + 2 q3, u' = u + (q1 + 2 q2 + 2 q3 + q4) / 3.
// With L u = wc u + w1 s1 + w2 s2 (s_d: sum of the four neighbours at distance d),
//   q = a u - i (b - wc) u + i (w1 s1 + w2 s2),   a = c3 r - c4,  b = c5 |u|^2 + c6 r.
struct RegConst {
  float2 nwc, w1, w2, c3, nc4, c5, c6, c13, c14, two, third;
};

__device__ __forceinline__ RegConst reg_const(const Params<float>& p) {
  RegConst c;
  const float h = p.half_dt;
  c.nwc = f2(-(h * p.wc), -(h * p.wc)); c.w1 = f2(h * p.w1, h * p.w1); c.w2 = f2(h * p.w2, h * p.w2);
  c.c3 = f2(h * p.c3, h * p.c3); c.nc4 = f2(-(h * p.c4), -(h * p.c4));
  c.c5 = f2(h * p.c5, h * p.c5); c.c6 = f2(h * p.c6, h * p.c6);
  c.c13 = f2(p.c13, p.c13); c.c14 = f2(p.c14, p.c14);
  c.two = f2(2.f, 2.f);
  c.third = f2(1.f / 3.f, 1.f / 3.f);
  return c;
}

// One RK4 stage S over the warp's strip.  tX/tY hold the stage input of the NJ rows (planar node
// pairs); on return they hold the next stage's input (S < 4), or u holds the new state (S = 4).
// Every node of the region is evaluated; values near the region edge are wrong (their stencils
// reach outside the region) but the valid part shrinks by K per stage and the output tile is what
// remains after four.  EDGE: the region reaches outside the grid, whose nodes must read as zero
// (the reference's truncated operator), so stage outputs there are reset to zero.
template <int K, int NW, int NJ, int S, bool EDGE>
__device__ __forceinline__ void reg_stage(float2 (&tX)[NJ], float2 (&tY)[NJ], float2 (&aX)[NJ],
                                          float2 (&aY)[NJ], float2 (&uX)[NJ], float2 (&uY)[NJ],
                                          const float2 (&pc)[NJ], unsigned dom0, unsigned dom1,
                                          float4* __restrict__ exch, int warp, int lane,
                                          const RegConst& c) {
  float4* ex = exch + (S & 1) * (NW * 2 * K * 32);
  // publish the strip's first and last K rows of the stage input, then read the neighbours'
#pragma unroll
  for (int k = 0; k < K; ++k) {
    ex[((warp * 2 + 0) * K + k) * 32 + lane] = make_float4(tX[k].x, tX[k].y, tY[k].x, tY[k].y);
    ex[((warp * 2 + 1) * K + k) * 32 + lane] =
        make_float4(tX[NJ - K + k].x, tX[NJ - K + k].y, tY[NJ - K + k].x, tY[NJ - K + k].y);
  }
  __syncthreads();
  float2 upX[K], upY[K], dnX[K], dnY[K];  // rows y0 - K + k and y0 + NJ + k
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (warp > 0) a = ex[(((warp - 1) * 2 + 1) * K + k) * 32 + lane];
    if (warp < NW - 1) b = ex[(((warp + 1) * 2 + 0) * K + k) * 32 + lane];
    upX[k] = f2(a.x, a.y); upY[k] = f2(a.z, a.w);
    dnX[k] = f2(b.x, b.y); dnY[k] = f2(b.z, b.w);
  }
  auto rowX = [&](int r) -> float2 { return r < 0 ? upX[K + r] : (r >= NJ ? dnX[r - NJ] : tX[r]); };
  auto rowY = [&](int r) -> float2 { return r < 0 ? upY[K + r] : (r >= NJ ? dnY[r - NJ] : tY[r]); };

  float2 nX[NJ], nY[NJ];
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float2 X = tX[j], Y = tY[j];
    float2 mX, mY;  // w1 s1 + w2 s2 per plane
    if (K == 1) {
      // left neighbour of the pair's first node, right neighbour of its second
      const float lx = __shfl_up_sync(0xffffffffu, X.y, 1), ly = __shfl_up_sync(0xffffffffu, Y.y, 1);
      const float rx = __shfl_down_sync(0xffffffffu, X.x, 1), ry = __shfl_down_sync(0xffffffffu, Y.x, 1);
      const float2 sX = add2(add2(f2(lx + X.y, X.x + rx), rowX(j - 1)), rowX(j + 1));
      const float2 sY = add2(add2(f2(ly + Y.y, Y.x + ry), rowY(j - 1)), rowY(j + 1));
      mX = mul2(c.w1, sX);
      mY = mul2(c.w1, sY);
    } else {
      // both nodes of the pairs to the left (L) and right (R)
      const float2 LX = f2(__shfl_up_sync(0xffffffffu, X.x, 1), __shfl_up_sync(0xffffffffu, X.y, 1));
      const float2 LY = f2(__shfl_up_sync(0xffffffffu, Y.x, 1), __shfl_up_sync(0xffffffffu, Y.y, 1));
      const float2 RX = f2(__shfl_down_sync(0xffffffffu, X.x, 1), __shfl_down_sync(0xffffffffu, X.y, 1));
      const float2 RY = f2(__shfl_down_sync(0xffffffffu, Y.x, 1), __shfl_down_sync(0xffffffffu, Y.y, 1));
      const float2 s1X = add2(add2(f2(LX.y + X.y, X.x + RX.x), rowX(j - 1)), rowX(j + 1));
      const float2 s1Y = add2(add2(f2(LY.y + Y.y, Y.x + RY.x), rowY(j - 1)), rowY(j + 1));
      const float2 s2X = add2(add2(add2(LX, RX), rowX(j - 2)), rowX(j + 2));
      const float2 s2Y = add2(add2(add2(LY, RY), rowY(j - 2)), rowY(j + 2));
      mX = fma2(c.w2, s2X, mul2(c.w1, s1X));
      mY = fma2(c.w2, s2Y, mul2(c.w1, s1Y));
    }
    // r = c12 P / (c13 + c14 |u|^2), |u|^2 per node in scalar arithmetic (a packed square of a
    // register pair with itself costs extra register moves)
    const float2 sq = f2(__fmaf_rn(X.x, X.x, Y.x * Y.x), __fmaf_rn(X.y, X.y, Y.y * Y.y));
    const float2 den = fma2(c.c14, sq, c.c13);
    const float2 r = mul2(pc[j], f2(rcp_approx(den.x), rcp_approx(den.y)));
    const float2 a = fma2(c.c3, r, c.nc4);
    const float2 bw = fma2(c.c5, sq, fma2(c.c6, r, c.nwc));
    const float2 kX = fma2(a, X, fma2(bw, Y, neg2(mY)));
    const float2 kY = fma2(a, Y, fma2(neg2(bw), X, mX));
    if (S == 1) {
      aX[j] = kX;
      aY[j] = kY;
    } else if (S == 4) {
      aX[j] = add2(aX[j], kX);
      aY[j] = add2(aY[j], kY);
    } else {
      aX[j] = fma2(c.two, kX, aX[j]);
      aY[j] = fma2(c.two, kY, aY[j]);
    }
    if (S < 4) {
      float2 vX, vY;
      // Next stage input u + q (u + 2 q before stage 4).  Packed or scalar by tile shape, as
      // measured on the GB300: scalar is faster for strips of up to 10 rows and at order 5,
      // packed for 12-row strips at order 3 (the register allocation differs, not the work).
      constexpr bool kScalarUpdate = NJ <= 10 || K == 2;
      if (kScalarUpdate) {
        const float m = S == 3 ? 2.f : 1.f;
        vX = f2(__fmaf_rn(m, kX.x, uX[j].x), __fmaf_rn(m, kX.y, uX[j].y));
        vY = f2(__fmaf_rn(m, kY.x, uY[j].x), __fmaf_rn(m, kY.y, uY[j].y));
      } else if (S == 3) {
        vX = fma2(c.two, kX, uX[j]);
        vY = fma2(c.two, kY, uY[j]);
      } else {
        vX = add2(uX[j], kX);
        vY = add2(uY[j], kY);
      }
      if (EDGE) {
        const bool i0 = (dom0 >> j) & 1u, i1 = (dom1 >> j) & 1u;
        vX = f2(i0 ? vX.x : 0.f, i1 ? vX.y : 0.f);
        vY = f2(i0 ? vY.x : 0.f, i1 ? vY.y : 0.f);
      }
      nX[j] = vX;
      nY[j] = vY;
    } else {
      if (NJ <= 10 || K == 2) {  // scalar for the same shapes as the stage-input update
        const float th = 1.f / 3.f;
        uX[j] = f2(__fmaf_rn(th, aX[j].x, uX[j].x), __fmaf_rn(th, aX[j].y, uX[j].y));
        uY[j] = f2(__fmaf_rn(th, aY[j].x, uY[j].x), __fmaf_rn(th, aY[j].y, uY[j].y));
      } else {
        uX[j] = fma2(c.third, aX[j], uX[j]);
        uY[j] = fma2(c.third, aY[j], uY[j]);
      }
    }
  }
  if (S < 4) {
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      tX[j] = nX[j];
      tY[j] = nY[j];
    }
  }
}

// The four stages of a step; mid() runs between the second and the third.
template <int K, int NW, int NJ, bool EDGE, typename Mid>
__device__ __forceinline__ void reg_step(float2 (&uX)[NJ], float2 (&uY)[NJ], const float2 (&pc)[NJ],
                                         unsigned dom0, unsigned dom1, float4* __restrict__ exch,
                                         int warp, int lane, const RegConst& c, Mid&& mid) {
  float2 tX[NJ], tY[NJ], aX[NJ], aY[NJ];
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    tX[j] = uX[j];
    tY[j] = uY[j];
  }
  reg_stage<K, NW, NJ, 1, EDGE>(tX, tY, aX, aY, uX, uY, pc, dom0, dom1, exch, warp, lane, c);
  reg_stage<K, NW, NJ, 2, EDGE>(tX, tY, aX, aY, uX, uY, pc, dom0, dom1, exch, warp, lane, c);
  mid();
  reg_stage<K, NW, NJ, 3, EDGE>(tX, tY, aX, aY, uX, uY, pc, dom0, dom1, exch, warp, lane, c);
  reg_stage<K, NW, NJ, 4, EDGE>(tX, tY, aX, aY, uX, uY, pc, dom0, dom1, exch, warp, lane, c);
}

template <int K, int NW, int NJ, bool TMA>
__global__ void __launch_bounds__(NW * 32, 1)
rk4_2d_reg(const Inst2D* __restrict__ insts, const TileItem* __restrict__ items, int n_items, int j_step,
           int* __restrict__ wait_flag) {
  typedef RegCfg<K, NW, NJ> G;
  constexpr int H = G::H;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float4* stage_u = reinterpret_cast<float4*>(smem_raw);                   // [RY][32] node pairs
  float2* stage_p = reinterpret_cast<float2*>(smem_raw + G::STAGE_U);      // [RY][32]
  float4* exch = reinterpret_cast<float4*>(smem_raw + G::STAGE_U + G::STAGE_P);
  Inst2D* desc = reinterpret_cast<Inst2D*>(smem_raw + G::OFF_DESC);       // [2]
  RegCtrl* ctrl = reinterpret_cast<RegCtrl*>(smem_raw + G::OFF_CTRL);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x0 = 2 * lane;  // region column of the pair's first node
  const int y0 = warp * NJ;
  pdl_wait();      // the previous launch's states (programmatic launch)
  pdl_trigger();

  // One tile: load this thread's rows (from the staging boxes or from global memory), run the
  // step, store the output rows.
  auto run_tile = [&](const Inst2D& I, TileItem ti, auto&& boxes_read, auto&& mid) {
    const int n = I.n;
    const int par = (I.parity + j_step) & 1;
    const float2* __restrict__ src = reinterpret_cast<const float2*>(I.u[par]);
    float2* __restrict__ dst = reinterpret_cast<float2*>(I.u[par ^ 1]);
    const float* __restrict__ Pg = reinterpret_cast<const float*>(I.P);
    const int tyi = ti.tile / I.tiles_x;
    const int txi = ti.tile - tyi * I.tiles_x;
    const int rx0 = txi * G::TX - H, ry0 = tyi * G::TY - H;  // grid position of region node (0, 0)
    const int gx = rx0 + x0;
    const int gy0 = ry0 + y0;
    const bool edge = rx0 < 0 || ry0 < 0 || rx0 + G::RX > n || ry0 + G::RY > n;
    const Params<float>& prm = I.pf;
    const RegConst c = reg_const(prm);
    const float2 c12 = f2(prm.c12, prm.c12);
    float2 uX[NJ], uY[NJ], pc[NJ];
    unsigned dom0 = 0, dom1 = 0;
    const bool xin0 = gx >= 0 && gx < n, xin1 = gx + 1 >= 0 && gx + 1 < n;
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int gy = gy0 + j;
      const bool yin = gy >= 0 && gy < n;
      const bool i0 = yin && xin0, i1 = yin && xin1;
      float4 v;
      float2 p;
      if (TMA) {
        // out-of-range parts of the boxes arrive zero-filled
        v = stage_u[(y0 + j) * 32 + lane];
        p = stage_p[(y0 + j) * 32 + lane];
      } else {
        const size_t q = (size_t)gy * n + gx;
        const float2 a = i0 ? src[q] : f2(0.f, 0.f), b = i1 ? src[q + 1] : f2(0.f, 0.f);
        v = make_float4(a.x, a.y, b.x, b.y);
        p = f2(i0 ? Pg[q] : 0.f, i1 ? Pg[q + 1] : 0.f);
      }
      uX[j] = f2(v.x, v.z);
      uY[j] = f2(v.y, v.w);
      pc[j] = mul2(c12, p);
      dom0 |= (unsigned)i0 << j;
      dom1 |= (unsigned)i1 << j;
    }
    boxes_read();
    if (edge) reg_step<K, NW, NJ, true>(uX, uY, pc, dom0, dom1, exch, warp, lane, c, mid);
    else reg_step<K, NW, NJ, false>(uX, uY, pc, dom0, dom1, exch, warp, lane, c, mid);
    // output tile: region rows and columns [H, R - H) inside the grid
    const bool xout = x0 >= H && x0 < G::RX - H;
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int y = y0 + j;
      if (xout && y >= H && y < G::RY - H) {
        const size_t q = (size_t)(gy0 + j) * n + gx;
        const bool i0 = (dom0 >> j) & 1u, i1 = (dom1 >> j) & 1u;
        if (TMA) {
          // n is a multiple of 4 and gx even: the pair is wholly inside or outside, 16-byte aligned
          if (i0) *reinterpret_cast<float4*>(dst + q) = make_float4(uX[j].x, uY[j].x, uX[j].y, uY[j].y);
        } else {
          if (i0) dst[q] = f2(uX[j].x, uY[j].x);
          if (i1) dst[q + 1] = f2(uX[j].y, uY[j].y);
        }
      }
    }
  };

  if (!TMA) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
      const TileItem ti = items[it];
      const Inst2D& I = insts[ti.inst];
      if ((int64_t)j_step >= I.steps) continue;
      run_tile(I, ti, [] {}, [] {});
    }
    return;
  }

  // ---- TMA path: the elected thread (thread 0) keeps one tile in flight and looks up the one
  // after it while the current tile is computed.
  uint64_t* bar = &ctrl->bar;
  const uint32_t tx_extra = threadIdx.x == 0 ? g_tile_tx_extra : 0u;  // test control, normally 0
  // synchronous scan for the first active item at idx, idx + grid, ...; result in ctrl->nx_*
  auto scan = [&](int idx) {
    TileItem ti = {0, 0};
    for (; idx < n_items; idx += gridDim.x) {
      ti = items[idx];
      if ((int64_t)j_step < insts[ti.inst].steps) break;
    }
    ctrl->nx_idx = idx;
    if (idx < n_items) {
      const Inst2D& I = insts[ti.inst];
      ctrl->nx_ti = ti;
      ctrl->nx_tiles_x = I.tiles_x;
      ctrl->nx_parity = I.parity;
      ctrl->nx_tmap = I.tmap;
    }
  };
  // copy the boxes and the descriptor of item ctrl->nx_* into slot b
  auto issue = [&](int b) {
    const TileItem ti = ctrl->nx_ti;
    const int tyi = ti.tile / ctrl->nx_tiles_x;
    const int txi = ti.tile - tyi * ctrl->nx_tiles_x;
    const int par = (ctrl->nx_parity + j_step) & 1;
    const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(ctrl->nx_tmap);
    ctrl->item[b] = ctrl->nx_idx;
    ctrl->ti[b] = ti;
    fence_proxy_async_smem();
    mbar_expect_tx(bar, (uint32_t)(G::STAGE_U + G::STAGE_P + G::DESC) + tx_extra);
    tma_load_2d(stage_u, maps + par, txi * G::TX - H, tyi * G::TY - H, bar);
    tma_load_2d(stage_p, maps + 2, txi * G::TX - H, tyi * G::TY - H, bar);
    bulk_load(desc + b, insts + ti.inst, (uint32_t)G::DESC, bar);
  };
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    scan(blockIdx.x);
    if (ctrl->nx_idx < n_items) {
      issue(0);
      scan(ctrl->nx_idx + gridDim.x);
    } else {
      ctrl->item[0] = n_items;
    }
  }
  __syncthreads();
  uint32_t phase = 0;
  for (int b = 0;; b ^= 1) {
    if (ctrl->item[b] >= n_items) break;
    bool ok = true;
    if (threadIdx.x == 0) ok = mbar_wait(bar, phase);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(wait_flag, 1);  // the launching context's own status word
        mbar_wait(bar, phase);  // let the copies in flight land before the CTA leaves
      }
      return;
    }
    phase ^= 1u;
    // Hooks of the elected thread: once every thread holds its rows, fetch the next tile into
    // the staging boxes and start the lookup of the candidate after it (work-list entry now,
    // its descriptor fields after two stages, the decision after the step), all by cp.async so
    // that no load is waited on while it is in flight.  Its state lives in the control block.
    if (threadIdx.x == 0) {
      ctrl->slot = b;
      ctrl->cand_idx = ctrl->nx_idx < n_items ? ctrl->nx_idx + gridDim.x : n_items;
    }
    auto boxes_read = [&] {
      __syncthreads();  // the staging boxes are free again
      if (threadIdx.x != 0) return;
      if (ctrl->nx_idx < n_items) {
        issue(ctrl->slot ^ 1);
        if (ctrl->cand_idx < n_items) {
          async_copy<8>(&ctrl->cand_ti, items + ctrl->cand_idx);
          async_commit();
        }
      } else {
        ctrl->item[ctrl->slot ^ 1] = n_items;
      }
    };
    auto mid = [&] {
      if (threadIdx.x != 0 || ctrl->cand_idx >= n_items) return;
      async_commit_wait();
      const Inst2D* J = insts + ctrl->cand_ti.inst;
      async_copy<8>(&ctrl->cand_steps, &J->steps);
      async_copy<4>(&ctrl->cand_tiles_x, &J->tiles_x);
      async_copy<4>(&ctrl->cand_parity, &J->parity);
      async_copy<8>(&ctrl->cand_tmap, &J->tmap);
      async_commit();
    };
    run_tile(desc[b], ctrl->ti[b], boxes_read, mid);
    if (threadIdx.x == 0 && ctrl->nx_idx < n_items) {
      const int cand = ctrl->cand_idx;
      if (cand < n_items) {
        async_commit_wait();
        if ((int64_t)j_step < ctrl->cand_steps) {
          ctrl->nx_idx = cand;
          ctrl->nx_ti = ctrl->cand_ti;
          ctrl->nx_tiles_x = ctrl->cand_tiles_x;
          ctrl->nx_parity = ctrl->cand_parity;
          ctrl->nx_tmap = ctrl->cand_tmap;
        } else {
          scan(cand + gridDim.x);
        }
      } else {
        ctrl->nx_idx = n_items;
      }
    }
  }
}

}  // namespace nlsg
