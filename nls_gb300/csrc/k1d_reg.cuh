// k1d_reg.cuh -- register-resident single-CTA RK4 kernel for complex64 radial grids (sm_103a).
//
// Same contract as rk4_1d_resident on one CTA (all steps of one grid per launch, the state read
// and written once), with the grid held in registers instead of shared memory: thread t owns the
// NPT consecutive nodes t*NPT .. t*NPT+NPT-1, so a node's stencil neighbours are the thread's own
// registers except the K nodes beyond either end, which come from the adjacent lanes by warp
// shuffle and, at a warp boundary, from the adjacent warp through a few bytes of shared memory.
// Every node's state, RK4 accumulator, stage value, pump and 1/r stay in registers for the whole
// launch; the radial operator (D2 + D1 / r, make_laplacian, nls/nls.f90:132-295) and the stage
// updates run on the packed FP32x2 pipe over (re, im) pairs.  As in the 2-D register tile, the
// stage slopes are carried pre-multiplied by dt/2 (q = dt/2 k, constants scaled on the fly).
#pragma once

namespace nlsg {

// Weights of one launch in the working form: scaled by dt/2, as broadcast (w, w) pairs.
template <int K>
struct Reg1DConst {
  float2 w2[2 * K + 1], w1[2 * K + 1];  // D2 and D1 taps (index d + K weights u_{p+d})
  float2 near[K][2 * K + 1];            // the full near-axis rows p < K
  float c3, nc4, c5, c6, c13, c14;      // c3, c4, c5, c6 scaled by dt/2
};

template <int K>
__device__ __forceinline__ Reg1DConst<K> reg1d_const(const Inst1D& I) {
  Reg1DConst<K> c;
  const Params<float>& p = I.pf;
  const float h = p.half_dt;
#pragma unroll
  for (int i = 0; i < 2 * K + 1; ++i) {
    c.w2[i] = f2(h * I.op.w2f[i], h * I.op.w2f[i]);
    c.w1[i] = f2(h * I.op.w1f[i], h * I.op.w1f[i]);
#pragma unroll
    for (int r = 0; r < K; ++r) c.near[r][i] = f2(h * I.op.nearf[r][i], h * I.op.nearf[r][i]);
  }
  c.c3 = h * p.c3; c.nc4 = -(h * p.c4); c.c5 = h * p.c5; c.c6 = h * p.c6;
  c.c13 = p.c13; c.c14 = p.c14;
  return c;
}

// One RK4 stage S over the thread's NPT nodes.  t holds the stage input (re, im per node); on
// return it holds the next stage's input (S < 4), or u the new state (S = 4).  L / R: the K nodes
// before the thread's first and after its last node.  Nodes at or beyond n stay zero.
template <int K, int NPT, int S>
__device__ __forceinline__ void reg1d_stage(float2 (&t)[NPT], float2 (&acc)[NPT], float2 (&u)[NPT],
                                            const float (&pc)[NPT], const float (&ir)[NPT],
                                            const float2 (&L)[K], const float2 (&R)[K], int p0, int n,
                                            const Reg1DConst<K>& c) {
  auto at = [&](int idx) -> float2 { return idx < 0 ? L[K + idx] : (idx >= NPT ? R[idx - NPT] : t[idx]); };
  float2 nt[NPT];
#pragma unroll
  for (int i = 0; i < NPT; ++i) {
    const int p = p0 + i;
    float2 lu;
    if (i < K && p0 == 0) {
      // near-axis rows (only thread 0 holds nodes p = i < K, as NPT >= K) carry the mirror folds
      // at r = 0; the weights of nodes before 0 are zero
      lu = mul2(c.near[i < K ? i : 0][0], at(i - K));
#pragma unroll
      for (int d = 1; d <= 2 * K; ++d) lu = fma2(c.near[i < K ? i : 0][d], at(i - K + d), lu);
    } else {
      // D2 u + (1/r) D1 u, the centre tap of D1 being zero
      float2 d2 = mul2(c.w2[K], at(i));
      float2 d1 = mul2(c.w1[0], at(i - K));
#pragma unroll
      for (int d = 1; d <= K; ++d) {
        d2 = fma2(c.w2[K - d], at(i - d), d2);
        d2 = fma2(c.w2[K + d], at(i + d), d2);
        if (d < K) d1 = fma2(c.w1[K - d], at(i - d), d1);
        d1 = fma2(c.w1[K + d], at(i + d), d1);
      }
      lu = fma2(f2(ir[i], ir[i]), d1, d2);
    }
    // q = (a - i b) u + i L u, r = c12 P / (c13 + c14 |u|^2), a = c3 r - c4, b = c5 |u|^2 + c6 r
    const float2 v = t[i];
    const float sq = __fmaf_rn(v.x, v.x, v.y * v.y);
    const float r = pc[i] * rcp_approx(__fmaf_rn(c.c14, sq, c.c13));
    const float a = __fmaf_rn(c.c3, r, c.nc4);
    const float b = __fmaf_rn(c.c5, sq, c.c6 * r);
    const float2 q = f2(__fmaf_rn(a, v.x, __fmaf_rn(b, v.y, -lu.y)), __fmaf_rn(a, v.y, __fmaf_rn(-b, v.x, lu.x)));
    if (S == 1) acc[i] = q;
    else if (S == 4) acc[i] = add2(acc[i], q);
    else acc[i] = fma2(f2(2.f, 2.f), q, acc[i]);
    if (S < 4) {
      const float2 w = S == 3 ? fma2(f2(2.f, 2.f), q, u[i]) : add2(u[i], q);
      nt[i] = p < n ? w : f2(0.f, 0.f);
    } else {
      // the state stays in registers across steps: nodes beyond the grid must stay zero
      const float2 w = fma2(f2(1.f / 3.f, 1.f / 3.f), acc[i], u[i]);
      u[i] = p < n ? w : f2(0.f, 0.f);
    }
  }
  if (S < 4) {
#pragma unroll
    for (int i = 0; i < NPT; ++i) t[i] = nt[i];
  }
}

// The K nodes before the thread's first node (L) and after its last (R): from the adjacent lanes
// by shuffle, across a warp boundary from the neighbouring warp's published end nodes (stage
// parity double-buffers them, so one CTA barrier per stage suffices), zero beyond the grid.
template <int K, int NPT, int S>
__device__ __forceinline__ void reg1d_halo(const float2 (&t)[NPT], float2 (&L)[K], float2 (&R)[K],
                                           float2* __restrict__ ex, int warp, int lane, int nw) {
  float2* e = ex + (S & 1) * (nw * 2 * K);
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (lane == 0) e[(warp * 2 + 0) * K + k] = t[k];
    if (lane == 31) e[(warp * 2 + 1) * K + k] = t[NPT - K + k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    L[k] = f2(__shfl_up_sync(0xffffffffu, t[NPT - K + k].x, 1), __shfl_up_sync(0xffffffffu, t[NPT - K + k].y, 1));
    R[k] = f2(__shfl_down_sync(0xffffffffu, t[k].x, 1), __shfl_down_sync(0xffffffffu, t[k].y, 1));
    if (lane == 0) L[k] = warp > 0 ? e[((warp - 1) * 2 + 1) * K + k] : f2(0.f, 0.f);
    if (lane == 31) R[k] = warp < nw - 1 ? e[((warp + 1) * 2 + 0) * K + k] : f2(0.f, 0.f);
  }
}

template <int K, int NPT>
__global__ void __launch_bounds__(512) rk4_1d_reg(const Inst1D* __restrict__ insts) {
  static_assert(NPT >= K, "a thread's neighbours must lie within the adjacent lanes");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* ex = reinterpret_cast<float2*>(smem_raw);  // [2 parities][warps][2 ends][K]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const Inst1D& I = insts[blockIdx.x];
  const int n = I.n;
  const int p0 = tid * NPT;
  const Reg1DConst<K> c = reg1d_const<K>(I);
  const float h = (float)I.op.h;
  const float c12 = I.pf.c12;
  const float2* __restrict__ Ug = reinterpret_cast<const float2*>(I.u);
  const float* __restrict__ Pg = reinterpret_cast<const float*>(I.P);
  float2 u[NPT], t[NPT], acc[NPT];
  float pc[NPT], ir[NPT];
#pragma unroll
  for (int i = 0; i < NPT; ++i) {
    const int p = p0 + i;
    const bool in = p < n;
    u[i] = in ? Ug[p] : f2(0.f, 0.f);
    pc[i] = in ? c12 * Pg[p] : 0.f;
    ir[i] = p >= K ? 1.f / ((float)p * h) : 0.f;
    acc[i] = f2(0.f, 0.f);
  }
  float2 L[K], R[K];
  const int64_t steps = I.steps;
  for (int64_t step = 0; step < steps; ++step) {
#pragma unroll
    for (int i = 0; i < NPT; ++i) t[i] = u[i];
    reg1d_halo<K, NPT, 1>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 1>(t, acc, u, pc, ir, L, R, p0, n, c);
    reg1d_halo<K, NPT, 2>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 2>(t, acc, u, pc, ir, L, R, p0, n, c);
    reg1d_halo<K, NPT, 3>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 3>(t, acc, u, pc, ir, L, R, p0, n, c);
    reg1d_halo<K, NPT, 4>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 4>(t, acc, u, pc, ir, L, R, p0, n, c);
  }
  float2* __restrict__ Uo = reinterpret_cast<float2*>(I.u);
#pragma unroll
  for (int i = 0; i < NPT; ++i)
    if (p0 + i < n) Uo[p0 + i] = u[i];
}

// Cluster form (grids too long for one CTA): the grid is cut into cl segments [q0, q1), one per
// CTA of a thread-block cluster.  Each CTA holds its segment and up to H = 4K halo nodes on either
// side, [lo, hi), in registers with the single-CTA layout above, and runs the four stages over all
// of them with CTA-local barriers only; a node within K of [lo, hi)'s ends reads zeros past them,
// so after stage s the values within sK of those ends are wrong, and after the four stages exactly
// the segment itself is exact.  At the end of each step every CTA pushes the H new values at
// either end of its segment into its neighbours' halo buffers (distributed shared memory, double
// buffered by step parity: a buffer written at step s is read at the start of step s + 1 and
// written again only after the cluster's next meeting) and the cluster meets once; the next step
// starts by taking its halo nodes from those buffers.  Every CTA runs the same loop with no early
// exit, so the cluster's barriers always match.
template <int K, int NPT>
__global__ void __launch_bounds__(512) rk4_1d_reg_cl(const Inst1D* __restrict__ insts, int cl) {
  static_assert(NPT >= K, "a thread's neighbours must lie within the adjacent lanes");
  constexpr int H = 4 * K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  float2* ex = reinterpret_cast<float2*>(smem_raw);   // [2 parities][warps][2 ends][K]
  float2* halo = ex + 2 * nw * 2 * K;                 // [2 parities][2 sides: left, right][H]
  cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
  const int inst = blockIdx.x / cl, rank = blockIdx.x % cl;
  const Inst1D& I = insts[inst];
  const int n = I.n;
  const int seg = (n + cl - 1) / cl;
  const int q0 = min(n, rank * seg), q1 = min(n, q0 + seg);
  const int lo = max(0, q0 - H), hi = min(n, q1 + H);
  const int p0 = lo + tid * NPT;
  const Reg1DConst<K> c = reg1d_const<K>(I);
  const float h = (float)I.op.h;
  const float c12 = I.pf.c12;
  const float2* __restrict__ Ug = reinterpret_cast<const float2*>(I.u);
  const float* __restrict__ Pg = reinterpret_cast<const float*>(I.P);
  float2 u[NPT], t[NPT], acc[NPT];
  float pc[NPT], ir[NPT];
#pragma unroll
  for (int i = 0; i < NPT; ++i) {
    const int p = p0 + i;
    const bool in = p < hi;
    u[i] = in ? Ug[p] : f2(0.f, 0.f);
    pc[i] = in ? c12 * Pg[p] : 0.f;
    ir[i] = p >= K ? 1.f / ((float)p * h) : 0.f;
    acc[i] = f2(0.f, 0.f);
  }
  // the neighbours' halo buffers (their right side takes this segment's first H nodes, their
  // left side its last H)
  float2* const lnb = rank > 0 ? cluster.map_shared_rank(halo, rank - 1) : nullptr;
  float2* const rnb = rank < cl - 1 ? cluster.map_shared_rank(halo, rank + 1) : nullptr;
  cluster.sync();   // every CTA of the cluster is running before the first push
  float2 L[K], R[K];
  const int64_t steps = I.steps;
  for (int64_t step = 0; step < steps; ++step) {
    const int par = (int)(step & 1);
    if (step > 0) {
      const float2* hb = halo + (par ^ 1) * 2 * H;
#pragma unroll
      for (int i = 0; i < NPT; ++i) {
        const int p = p0 + i;
        if (p >= lo && p < q0) u[i] = hb[p - (q0 - H)];
        if (p >= q1 && p < hi) u[i] = hb[H + (p - q1)];
      }
    }
#pragma unroll
    for (int i = 0; i < NPT; ++i) t[i] = u[i];
    reg1d_halo<K, NPT, 1>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 1>(t, acc, u, pc, ir, L, R, p0, hi, c);
    reg1d_halo<K, NPT, 2>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 2>(t, acc, u, pc, ir, L, R, p0, hi, c);
    reg1d_halo<K, NPT, 3>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 3>(t, acc, u, pc, ir, L, R, p0, hi, c);
    reg1d_halo<K, NPT, 4>(t, L, R, ex, warp, lane, nw);
    reg1d_stage<K, NPT, 4>(t, acc, u, pc, ir, L, R, p0, hi, c);
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      const int p = p0 + i;
      if (lnb && p >= q0 && p < q0 + H) lnb[(par * 2 + 1) * H + (p - q0)] = u[i];
      if (rnb && p >= q1 - H && p < q1) rnb[(par * 2 + 0) * H + (p - (q1 - H))] = u[i];
    }
    cluster.sync();
  }
  float2* __restrict__ Uo = reinterpret_cast<float2*>(I.u);
#pragma unroll
  for (int i = 0; i < NPT; ++i) {
    const int p = p0 + i;
    if (p >= q0 && p < q1) Uo[p] = u[i];
  }
}

}  // namespace nlsg
