// k1d.cu -- 1-D (axially symmetric, radial) RK4 kernels for sm_103a.
//
// rk4_1d_resident: the whole grid of one solve lives in shared memory of one CTA or of a thread
// block cluster (distributed shared memory) for every step of the launch.  Each RK4 stage
// (nls/nls.f90:726-729) reads the previous stage's values from shared memory, evaluates the
// radial Laplacian (make_laplacian, nls/nls.f90:132-295) and the pointwise terms of
// `hamiltonian` (nls/nls.f90:621-650), and writes the next stage input; CTAs of a cluster push
// their K edge values into their neighbours' halo slots and meet at one cluster barrier per
// stage.  HBM is touched once per launch (load and store of the state).
//
// rk4_1d_stage: one RK4 stage over an arbitrary-size grid from global memory, the general path
// for grids too large to stay resident.
#include <cooperative_groups.h>

#include "kernels.h"
#include "nls_common.cuh"
#include "k1d_reg.cuh"

namespace cg = cooperative_groups;

namespace nlsg {

template <typename T, int K>
struct Weights1D {
  T w2[2 * K + 1];
  T w1[2 * K + 1];
};

template <typename T, int K>
__device__ __forceinline__ Weights1D<T, K> load_w(const Stencil1D& s) {
  Weights1D<T, K> w;
#pragma unroll
  for (int i = 0; i < 2 * K + 1; ++i) {
    w.w2[i] = ParamsOf<T>::w2(s, i);
    w.w1[i] = ParamsOf<T>::w1(s, i);
  }
  return w;
}

// (L u)_p from a buffer whose element c holds u_p (and c +- d hold u_{p +- d}).
template <typename T, int K>
__device__ __forceinline__ typename C2<T>::type lap1d(const typename C2<T>::type* in, int c, int p,
                                                      T inv_r, const Weights1D<T, K>& w,
                                                      const Stencil1D& s) {
  typedef typename C2<T>::type C;
  C lu;
  if (p >= K) {
    T d2x = 0, d2y = 0, d1x = 0, d1y = 0;
#pragma unroll
    for (int d = -K; d <= K; ++d) {
      C v = in[c + d];
      d2x += w.w2[d + K] * v.x;
      d2y += w.w2[d + K] * v.y;
      if (d != 0) {
        d1x += w.w1[d + K] * v.x;
        d1y += w.w1[d + K] * v.y;
      }
    }
    lu.x = d2x + inv_r * d1x;
    lu.y = d2y + inv_r * d1y;
  } else {
    T lx = 0, ly = 0;
#pragma unroll
    for (int d = -K; d <= K; ++d) {
      T a = ParamsOf<T>::near(s, p, d + K);
      C v = in[c + d];
      lx += a * v.x;
      ly += a * v.y;
    }
    lu.x = lx;
    lu.y = ly;
  }
  return lu;
}

template <typename T, int K, int NPT>
__global__ void __launch_bounds__(512) rk4_1d_resident(const Inst1D* __restrict__ insts, int cl,
                                                       int seg_cap) {
  typedef typename C2<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int inst = blockIdx.x / cl;
  const int rank = blockIdx.x % cl;
  const Inst1D& I = insts[inst];
  const int n = I.n;
  const int seg = (n + cl - 1) / cl;
  const int p0 = rank * seg;
  const int len = max(0, min(seg, n - p0));
  const int NT = blockDim.x;
  const int tid = threadIdx.x;
  const int L = seg_cap + 2 * K;
  C* buf[2] = {reinterpret_cast<C*>(smem_raw), reinterpret_cast<C*>(smem_raw) + L};

  cg::cluster_group cluster = cg::this_cluster();
  C* left_buf[2] = {nullptr, nullptr};
  C* right_buf[2] = {nullptr, nullptr};
  if (cl > 1) {
    if (rank > 0) {
      left_buf[0] = cluster.map_shared_rank(buf[0], rank - 1);
      left_buf[1] = cluster.map_shared_rank(buf[1], rank - 1);
    }
    if (rank < cl - 1) {
      right_buf[0] = cluster.map_shared_rank(buf[0], rank + 1);
      right_buf[1] = cluster.map_shared_rank(buf[1], rank + 1);
    }
  }

  for (int i = tid; i < 2 * L; i += NT) buf[0][i] = mk<T>(0, 0);
  if (cl > 1) cluster.sync(); else __syncthreads();

  const Params<T>& prm = ParamsOf<T>::get(I);
  const Phys<T> ph = phys_of<T>(prm);
  const RK<T> rk = rk_of<T>(prm);
  const Weights1D<T, K> w = load_w<T, K>(I.op);
  const T h = (T)I.op.h;
  const C* __restrict__ Ug = reinterpret_cast<const C*>(I.u);
  const T* __restrict__ Pg = reinterpret_cast<const T*>(I.P);

  C u[NPT], acc[NPT];
  T P[NPT], ir[NPT];
  // Double precision: each node's full operator row (w2 + w1 / (p h), as in the band matrix, or
  // the near-axis row), built once per launch, so a stage evaluates one (2K+1)-term dot product
  // per node instead of separate D2 and D1 sums (FP64 runs at a small fraction of FP32 on GB300).
  constexpr bool ROWS = sizeof(T) == 8;
  T wrow[ROWS ? NPT : 1][2 * K + 1];
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int li = tid + j * NT;
    u[j] = mk<T>(0, 0);
    acc[j] = mk<T>(0, 0);
    P[j] = 0;
    ir[j] = 0;
    if (ROWS) {
#pragma unroll
      for (int i = 0; i < 2 * K + 1; ++i) wrow[ROWS ? j : 0][i] = 0;
    }
    if (li < len) {
      const int p = p0 + li;
      u[j] = Ug[p];
      P[j] = Pg[p];
      ir[j] = p >= K ? (T)1 / ((T)p * h) : (T)0;
      if (ROWS) {
#pragma unroll
        for (int i = 0; i < 2 * K + 1; ++i)
          wrow[ROWS ? j : 0][i] = p >= K ? w.w1[i] / ((T)p * h) + w.w2[i] : ParamsOf<T>::near(I.op, p, i);
      }
      buf[0][K + li] = u[j];
      if (left_buf[0] && li < K) left_buf[0][seg + K + li] = u[j];
      if (right_buf[0] && li >= seg - K) right_buf[0][li - (seg - K)] = u[j];
    }
  }
  if (cl > 1) cluster.sync(); else __syncthreads();

  // the pump enters as c12 * P (the reference evaluates coeffs(12) * pumping first)
#pragma unroll
  for (int j = 0; j < NPT; ++j) P[j] = ph.c12 * P[j];
  // Nodes are processed in batches of CB: a batch's shared-memory loads are all issued before any
  // of its stores and its arithmetic is written phase by phase across the batch, so the nodes'
  // independent dependency chains overlap.
  constexpr int CB0 = (sizeof(T) == 8 || K == 3) ? 2 : 4;
  constexpr int CB = NPT < CB0 ? NPT : CB0;
  const int64_t steps = I.steps;
  for (int64_t step = 0; step < steps; ++step) {
#pragma unroll 1
    for (int s = 1; s <= 4; ++s) {
      const C* in = buf[(s & 1) ? 0 : 1];
      const int ob = (s & 1) ? 1 : 0;
      C* out = buf[ob];
      const T coef = s == 3 ? rk.dt : rk.half_dt;
      const T wk = (s == 2 || s == 3) ? (T)2 : (T)1;
#pragma unroll
      for (int j0 = 0; j0 < NPT; j0 += CB) {
        C v[CB][2 * K + 1];
#pragma unroll
        for (int i = 0; i < CB; ++i) {
          const int li = tid + (j0 + i) * NT;
          const int c = K + (li < len ? li : 0);
#pragma unroll
          for (int d = -K; d <= K; ++d) v[i][d + K] = in[c + d];
        }
        C lu[CB];
#pragma unroll
        for (int i = 0; i < CB; ++i) {
          const int p = p0 + tid + (j0 + i) * NT;
          if (ROWS) {
            T lx = 0, ly = 0;
#pragma unroll
            for (int d = 0; d < 2 * K + 1; ++d) {
              lx += wrow[ROWS ? j0 + i : 0][d] * v[i][d].x;
              ly += wrow[ROWS ? j0 + i : 0][d] * v[i][d].y;
            }
            lu[i].x = lx;
            lu[i].y = ly;
          } else if (p >= K) {
            T d2x = 0, d2y = 0, d1x = 0, d1y = 0;
#pragma unroll
            for (int d = -K; d <= K; ++d) {
              d2x += w.w2[d + K] * v[i][d + K].x;
              d2y += w.w2[d + K] * v[i][d + K].y;
              if (d != 0) {
                d1x += w.w1[d + K] * v[i][d + K].x;
                d1y += w.w1[d + K] * v[i][d + K].y;
              }
            }
            lu[i].x = d2x + ir[j0 + i] * d1x;
            lu[i].y = d2y + ir[j0 + i] * d1y;
          } else {
            T lx = 0, ly = 0;
#pragma unroll
            for (int d = -K; d <= K; ++d) {
              const T a = ParamsOf<T>::near(I.op, p, d + K);
              lx += a * v[i][d + K].x;
              ly += a * v[i][d + K].y;
            }
            lu[i].x = lx;
            lu[i].y = ly;
          }
        }
        T sq[CB], r[CB];
#pragma unroll
        for (int i = 0; i < CB; ++i) sq[i] = v[i][K].x * v[i][K].x + v[i][K].y * v[i][K].y;
#pragma unroll
        for (int i = 0; i < CB; ++i) r[i] = rdiv(P[j0 + i], ph.c13 + ph.c14 * sq[i]);
#pragma unroll
        for (int i = 0; i < CB; ++i) {
          const int j = j0 + i;
          const int li = tid + j * NT;
          const T a = ph.c3 * r[i] - ph.c4;
          const T b = ph.c5 * sq[i] + ph.c6 * r[i];
          C k;
          k.x = a * v[i][K].x + b * v[i][K].y - lu[i].y;
          k.y = a * v[i][K].y - b * v[i][K].x + lu[i].x;
          if (s == 1) acc[j] = k;
          else {
            acc[j].x += wk * k.x;
            acc[j].y += wk * k.y;
          }
          C t;
          if (s < 4) {
            t.x = u[j].x + coef * k.x;
            t.y = u[j].y + coef * k.y;
          } else {
            u[j].x = u[j].x + rk.dt6 * acc[j].x;
            u[j].y = u[j].y + rk.dt6 * acc[j].y;
            t = u[j];
          }
          if (li < len) {
            out[K + li] = t;
            if (left_buf[ob] && li < K) left_buf[ob][seg + K + li] = t;
            if (right_buf[ob] && li >= seg - K) right_buf[ob][li - (seg - K)] = t;
          }
        }
      }
      if (cl > 1) cluster.sync(); else __syncthreads();
    }
  }

  C* __restrict__ Uo = reinterpret_cast<C*>(I.u);
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int li = tid + j * NT;
    if (li < len) Uo[p0 + li] = u[j];
  }
  if (cl > 1) cluster.sync();
}

// Cluster form with temporal blocking: each CTA also evaluates a halo of H = 4K nodes on both
// sides of its segment, so the four stages of a step need only CTA-local barriers; the cluster
// meets once per RK4 step, after every CTA has pushed the H new edge values of its segment into
// its neighbours' state buffers (double-buffered by step parity, so a push never lands in a
// buffer a neighbour is still reading).  Nodes outside [0, n) are never evaluated and stay zero.
template <typename T, int K, int NPT>
__global__ void __launch_bounds__(512) rk4_1d_cluster_tb(const Inst1D* __restrict__ insts, int cl,
                                                         int seg_cap) {
  typedef typename C2<T>::type C;
  constexpr int H = 4 * K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int inst = blockIdx.x / cl;
  const int rank = blockIdx.x % cl;
  const Inst1D& I = insts[inst];
  const int n = I.n;
  const int seg = (n + cl - 1) / cl;
  const int p0 = rank * seg;
  const int len = max(0, min(seg, n - p0));
  const int NT = blockDim.x;
  const int tid = threadIdx.x;
  const int W = seg_cap + 2 * H;
  // buffers: state A[0], A[1] (by step parity), stage buffers B0, B1; element li lives at li + H
  C* A[2] = {reinterpret_cast<C*>(smem_raw) + H, reinterpret_cast<C*>(smem_raw) + W + H};
  C* B0 = reinterpret_cast<C*>(smem_raw) + 2 * W + H;
  C* B1 = reinterpret_cast<C*>(smem_raw) + 3 * W + H;
  cg::cluster_group cluster = cg::this_cluster();
  C* leftA[2] = {nullptr, nullptr};
  C* rightA[2] = {nullptr, nullptr};
  if (rank > 0) {
    leftA[0] = cluster.map_shared_rank(A[0], rank - 1);
    leftA[1] = cluster.map_shared_rank(A[1], rank - 1);
  }
  if (rank < cl - 1) {
    rightA[0] = cluster.map_shared_rank(A[0], rank + 1);
    rightA[1] = cluster.map_shared_rank(A[1], rank + 1);
  }
  C* base = reinterpret_cast<C*>(smem_raw);
  for (int i = tid; i < 4 * W; i += NT) base[i] = mk<T>(0, 0);
  __syncthreads();

  const Params<T>& prm = ParamsOf<T>::get(I);
  const Phys<T> ph = phys_of<T>(prm);
  const RK<T> rk = rk_of<T>(prm);
  const Weights1D<T, K> w = load_w<T, K>(I.op);
  const T h = (T)I.op.h;
  const C* __restrict__ Ug = reinterpret_cast<const C*>(I.u);
  const T* __restrict__ Pg = reinterpret_cast<const T*>(I.P);

  // owned local indices li = tid + j*NT - H, j < NPT, covering [-H, seg + H)
  C u[NPT], acc[NPT];
  T pc[NPT], ir[NPT];
  // double precision: each node's full operator row, built once per launch (see rk4_1d_resident)
  constexpr bool ROWS = sizeof(T) == 8;
  T wrow[ROWS ? NPT : 1][2 * K + 1];
  unsigned indom = 0;
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int li = tid + j * NT - H;
    const int p = p0 + li;
    const bool in = li < seg + H && p >= 0 && p < n;
    indom |= (unsigned)in << j;
    u[j] = in ? Ug[p] : mk<T>(0, 0);
    pc[j] = in ? ph.c12 * Pg[p] : (T)0;
    ir[j] = (in && p >= K) ? (T)1 / ((T)p * h) : (T)0;
    if (ROWS) {
#pragma unroll
      for (int i = 0; i < 2 * K + 1; ++i)
        wrow[ROWS ? j : 0][i] = !in ? (T)0 : (p >= K ? w.w1[i] / ((T)p * h) + w.w2[i] : ParamsOf<T>::near(I.op, p, i));
    }
    acc[j] = mk<T>(0, 0);
    if (in) A[0][li] = u[j];
  }
  __syncthreads();

  auto lap = [&](const C* in, int li, int p, T irv, int j) -> C {
    C lu;
    if (ROWS) {
      T lx = 0, ly = 0;
#pragma unroll
      for (int d = -K; d <= K; ++d) {
        const C v = in[li + d];
        lx += wrow[ROWS ? j : 0][d + K] * v.x;
        ly += wrow[ROWS ? j : 0][d + K] * v.y;
      }
      lu.x = lx;
      lu.y = ly;
    } else if (p >= K) {
      T d2x = 0, d2y = 0, d1x = 0, d1y = 0;
#pragma unroll
      for (int d = -K; d <= K; ++d) {
        const C v = in[li + d];
        d2x += w.w2[d + K] * v.x;
        d2y += w.w2[d + K] * v.y;
        if (d != 0) {
          d1x += w.w1[d + K] * v.x;
          d1y += w.w1[d + K] * v.y;
        }
      }
      lu.x = d2x + irv * d1x;
      lu.y = d2y + irv * d1y;
    } else {
      T lx = 0, ly = 0;
#pragma unroll
      for (int d = -K; d <= K; ++d) {
        const T a = ParamsOf<T>::near(I.op, p, d + K);
        lx += a * in[li + d].x;
        ly += a * in[li + d].y;
      }
      lu.x = lx;
      lu.y = ly;
    }
    return lu;
  };
  auto kval = [&](C v, T pcv, C lu) -> C {
    const T sq = v.x * v.x + v.y * v.y;
    const T r = rdiv(pcv, ph.c13 + ph.c14 * sq);
    const T a = ph.c3 * r - ph.c4;
    const T b = ph.c5 * sq + ph.c6 * r;
    C k;
    k.x = a * v.x + b * v.y - lu.y;
    k.y = a * v.y - b * v.x + lu.x;
    return k;
  };

  const int64_t steps = I.steps;
  for (int64_t step = 0; step < steps; ++step) {
    const int par = (int)(step & 1);
    C* Acur = A[par];
    C* Anext = A[par ^ 1];
    // halo values pushed by the neighbours at the end of the previous step
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
      const int li = tid + j * NT - H;
      if ((indom >> j) & 1u) u[j] = Acur[li];
    }
#pragma unroll 1
    for (int s = 1; s <= 4; ++s) {
      const C* in = s == 1 ? Acur : (s == 3 ? B1 : B0);
      C* out = s == 2 ? B1 : B0;
      const int lo = s < 4 ? -(H - s * K) : 0;
      const int hi = s < 4 ? seg + H - s * K : len;
      const T coef = s == 3 ? rk.dt : rk.half_dt;
      const T wk = (s == 2 || s == 3) ? (T)2 : (T)1;
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
        const int li = tid + j * NT - H;
        if (((indom >> j) & 1u) && li >= lo && li < hi) {
          const int p = p0 + li;
          const C k = kval(in[li], pc[j], lap(in, li, p, ir[j], j));
          if (s == 1) acc[j] = k;
          else {
            acc[j].x += wk * k.x;
            acc[j].y += wk * k.y;
          }
          if (s < 4) {
            out[li] = mk<T>(u[j].x + coef * k.x, u[j].y + coef * k.y);
          } else {
            const C un = mk<T>(u[j].x + rk.dt6 * acc[j].x, u[j].y + rk.dt6 * acc[j].y);
            u[j] = un;
            Anext[li] = un;
            if (leftA[0] && li < H) leftA[par ^ 1][seg + li] = un;
            if (rightA[0] && li >= seg - H) rightA[par ^ 1][li - seg] = un;
          }
        }
      }
      if (s < 4) __syncthreads();
    }
    cluster.sync();
  }

  C* __restrict__ Uo = reinterpret_cast<C*>(I.u);
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int li = tid + j * NT - H;
    if (((indom >> j) & 1u) && li >= 0 && li < len) Uo[p0 + li] = u[j];
  }
  cluster.sync();
}

// One RK4 stage of a 1-D grid held in global memory (see nls_common.cuh for the stage scheme).
template <typename T, int K>
__global__ void __launch_bounds__(256) rk4_1d_stage(int n, int s, const void* __restrict__ src_,
                                                    void* __restrict__ u_, const void* __restrict__ P_,
                                                    void* __restrict__ acc_, void* __restrict__ dst_,
                                                    Params<T> prm, Stencil1D op, T h) {
  typedef typename C2<T>::type C;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const C* __restrict__ src = reinterpret_cast<const C*>(src_);
  C* __restrict__ U = reinterpret_cast<C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  C* __restrict__ acc = reinterpret_cast<C*>(acc_);
  C* __restrict__ dst = reinterpret_cast<C*>(dst_);
  const Phys<T> ph = phys_of<T>(prm);
  const RK<T> rk = rk_of<T>(prm);
  const Weights1D<T, K> w = load_w<T, K>(op);
  // gather the 2K+1 neighbours with zero outside [0, n)
  C v[2 * K + 1];
#pragma unroll
  for (int d = -K; d <= K; ++d) {
    const int q = p + d;
    v[d + K] = (q >= 0 && q < n) ? src[q] : mk<T>(0, 0);
  }
  const T ir = p >= K ? (T)1 / ((T)p * h) : (T)0;
  const C lu = lap1d<T, K>(v, K, p, ir, w, op);
  const C k = rhs<T>(v[K], P[p], lu, ph);
  const C u = U[p];
  if (s == 1) {
    acc[p] = k;
    dst[p] = mk<T>(u.x + rk.half_dt * k.x, u.y + rk.half_dt * k.y);
  } else if (s == 2 || s == 3) {
    C a = acc[p];
    a.x += (T)2 * k.x;
    a.y += (T)2 * k.y;
    acc[p] = a;
    const T c = s == 2 ? rk.half_dt : rk.dt;
    dst[p] = mk<T>(u.x + c * k.x, u.y + c * k.y);
  } else {
    C a = acc[p];
    a.x += k.x;
    a.y += k.y;
    U[p] = mk<T>(u.x + rk.dt6 * a.x, u.y + rk.dt6 * a.y);
  }
}

// v = H(u) for the diagnostics (chemical potential).
template <typename T, int K>
__global__ void __launch_bounds__(256) rhs_1d(int n, const void* __restrict__ u_, const void* __restrict__ P_,
                                              void* __restrict__ v_, Params<T> prm, Stencil1D op, T h) {
  typedef typename C2<T>::type C;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const C* __restrict__ u = reinterpret_cast<const C*>(u_);
  const T* __restrict__ P = reinterpret_cast<const T*>(P_);
  const Phys<T> ph = phys_of<T>(prm);
  const Weights1D<T, K> w = load_w<T, K>(op);
  C v[2 * K + 1];
#pragma unroll
  for (int d = -K; d <= K; ++d) {
    const int q = p + d;
    v[d + K] = (q >= 0 && q < n) ? u[q] : mk<T>(0, 0);
  }
  const T ir = p >= K ? (T)1 / ((T)p * h) : (T)0;
  reinterpret_cast<C*>(v_)[p] = rhs<T>(v[K], P[p], lap1d<T, K>(v, K, p, ir, w, op), ph);
}

// ------------------------------------------------------------------ launchers

template <typename T, int K, int NPT>
static cudaError_t launch_res(const Inst1D* d_insts, int count, int cl, int seg_cap, int nt,
                              cudaStream_t stream, bool prepare_only) {
  // one CTA: per-stage CTA barriers; a cluster: the temporally blocked form (one cluster
  // barrier per step)
  auto kern = cl > 1 ? rk4_1d_cluster_tb<T, K, NPT> : rk4_1d_resident<T, K, NPT>;
  const size_t smem = cl > 1 ? (size_t)4 * (seg_cap + 8 * K) * sizeof(typename C2<T>::type)
                             : (size_t)2 * (seg_cap + 2 * K) * sizeof(typename C2<T>::type);
  // Attributes are raised once, monotonically, so launches inside a stream capture never need
  // to change them (prepare_1d_resident runs before any capture).
  static size_t configured_smem[2] = {0, 0};
  static bool non_portable = false;
  const int ki = cl > 1 ? 1 : 0;
  if (smem > configured_smem[ki]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured_smem[ki] = smem;
  }
  if (cl > 8 && !non_portable) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    non_portable = true;
  }
  if (prepare_only) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(count * cl);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, d_insts, cl, seg_cap);
}

template <typename T, int K>
static cudaError_t launch_res_npt(const Inst1D* d, int count, int cl, int seg_cap, cudaStream_t s,
                                  bool prepare_only) {
  // threads: up to 512; nodes per thread: 1, 2, 4 or 8 (8 only in single precision); the
  // cluster form also owns a halo of 4K nodes on each side
  const int nodes = cl > 1 ? seg_cap + 8 * K : seg_cap;
  int npt = 1;
  while (npt * 512 < nodes) npt *= 2;
  int nt = (nodes + npt - 1) / npt;
  nt = ((nt + 31) / 32) * 32;
  if (nt > 512) nt = 512;
  switch (npt) {
    case 1: return launch_res<T, K, 1>(d, count, cl, seg_cap, nt, s, prepare_only);
    case 2: return launch_res<T, K, 2>(d, count, cl, seg_cap, nt, s, prepare_only);
    case 4: return launch_res<T, K, 4>(d, count, cl, seg_cap, nt, s, prepare_only);
    case 8:
      if (sizeof(T) == 4) return launch_res<T, K, 8>(d, count, cl, seg_cap, nt, s, prepare_only);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

// Complex64 on one CTA per grid: the register-resident kernel, NPT consecutive nodes per thread
// (a power of two >= K, at most 8) on up to 512 threads.  One grid alone takes the smallest NPT
// that fits (most threads: the shortest step); a launch of many grids takes NPT = 8, the fewest
// threads per grid, so that small grids share an SM and each node costs the least SM time (fewer
// halo exchanges and barrier waits per node) -- in a batch the GPU's throughput is what counts.
template <int K>
static cudaError_t launch_reg1d(const Inst1D* d, int count, int seg_cap, cudaStream_t s, bool prepare_only) {
  int npt = 1;
  while (npt < K) npt *= 2;
  while (npt * 512 < seg_cap) npt *= 2;
  if (count > 1) npt = 8;
  if (npt > 8 || npt < K) return cudaErrorInvalidValue;
  int nt = (seg_cap + npt - 1) / npt;
  nt = ((nt + 31) / 32) * 32;
  const size_t smem = (size_t)2 * (nt / 32) * 2 * K * sizeof(float2);
  if (prepare_only) return cudaSuccess;
  switch (npt) {
    case 1: if (K <= 1) { rk4_1d_reg<(K <= 1 ? K : 1), 1><<<count, nt, smem, s>>>(d); return cudaGetLastError(); }
            return cudaErrorInvalidValue;
    case 2: if (K <= 2) { rk4_1d_reg<(K <= 2 ? K : 2), 2><<<count, nt, smem, s>>>(d); return cudaGetLastError(); }
            return cudaErrorInvalidValue;
    case 4: rk4_1d_reg<K, 4><<<count, nt, smem, s>>>(d); return cudaGetLastError();
    case 8: rk4_1d_reg<K, 8><<<count, nt, smem, s>>>(d); return cudaGetLastError();
  }
  return cudaErrorInvalidValue;
}

// Complex64 over a cluster: the register-resident cluster kernel, one segment and its halos per
// CTA (NPT as for one CTA: 8 in a launch of many grids, else the smallest that fits 512 threads).
template <int K>
static cudaError_t launch_reg1d_cl(const Inst1D* d, int count, int cl, int seg_cap, cudaStream_t s,
                                   bool prepare_only) {
  const int nodes = seg_cap + 8 * K;
  int npt = 1;
  while (npt < K) npt *= 2;
  while (npt * 512 < nodes) npt *= 2;
  if (count > 1) npt = 8;
  if (!prepare_only && (npt > 8 || npt < K || npt * 512 < nodes)) return cudaErrorInvalidValue;
  npt = std::min(npt, 8);
  int nt = (nodes + npt - 1) / npt;
  nt = ((nt + 31) / 32) * 32;
  const size_t smem = ((size_t)2 * (nt / 32) * 2 * K + (size_t)2 * 2 * 4 * K) * sizeof(float2);
  auto launch = [&](auto kern) -> cudaError_t {
    static bool non_portable = false;
    if (cl > 8 && !non_portable) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (e != cudaSuccess) return e;
      non_portable = true;
    }
    if (prepare_only) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(count * cl);
    cfg.blockDim = dim3(nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, d, cl);
  };
  if (prepare_only) {
    // a later launch may take any nodes-per-thread form (one grid: the smallest that fits; many
    // grids: 8): prepare them all
    cudaError_t e = cudaSuccess;
    if (K <= 1) e = launch(rk4_1d_reg_cl<(K <= 1 ? K : 1), 1>);
    if (!e && K <= 2) e = launch(rk4_1d_reg_cl<(K <= 2 ? K : 2), 2>);
    if (!e) e = launch(rk4_1d_reg_cl<K, 4>);
    if (!e) e = launch(rk4_1d_reg_cl<K, 8>);
    return e;
  }
  switch (npt) {
    case 1: if (K <= 1) return launch(rk4_1d_reg_cl<(K <= 1 ? K : 1), 1>);
            return cudaErrorInvalidValue;
    case 2: if (K <= 2) return launch(rk4_1d_reg_cl<(K <= 2 ? K : 2), 2>);
            return cudaErrorInvalidValue;
    case 4: return launch(rk4_1d_reg_cl<K, 4>);
    case 8: return launch(rk4_1d_reg_cl<K, 8>);
  }
  return cudaErrorInvalidValue;
}

// Portable cluster sizes only: 16-CTA clusters of this kernel failed to launch inside a batch's
// graph capture (cudaErrorInvalidClusterSize; the profiler reports a maximum potential cluster
// size of 8 for it); they keep the shared-memory cluster kernel.
bool reg1d_cluster_fits(int K, int cl, int seg_cap, int shortest_seg) {
  return cl > 1 && cl <= 8 && shortest_seg >= 4 * K && seg_cap + 8 * K <= 512 * 8;
}

static cudaError_t dispatch_res(int dtype, int K, const Inst1D* d_insts, int count, int cl,
                                int seg_cap, int shortest_seg, cudaStream_t s, bool prepare_only) {
  if (dtype == NLS_C64 && reg1d_cluster_fits(K, cl, seg_cap, shortest_seg)) {
    if (K == 1) return launch_reg1d_cl<1>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 2) return launch_reg1d_cl<2>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 3) return launch_reg1d_cl<3>(d_insts, count, cl, seg_cap, s, prepare_only);
    return cudaErrorInvalidValue;
  }
  if (dtype == NLS_C64 && cl == 1) {
    if (K == 1) return launch_reg1d<1>(d_insts, count, seg_cap, s, prepare_only);
    if (K == 2) return launch_reg1d<2>(d_insts, count, seg_cap, s, prepare_only);
    if (K == 3) return launch_reg1d<3>(d_insts, count, seg_cap, s, prepare_only);
    return cudaErrorInvalidValue;
  }
  if (dtype == NLS_C128) {
    if (K == 1) return launch_res_npt<double, 1>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 2) return launch_res_npt<double, 2>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 3) return launch_res_npt<double, 3>(d_insts, count, cl, seg_cap, s, prepare_only);
  } else {
    if (K == 1) return launch_res_npt<float, 1>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 2) return launch_res_npt<float, 2>(d_insts, count, cl, seg_cap, s, prepare_only);
    if (K == 3) return launch_res_npt<float, 3>(d_insts, count, cl, seg_cap, s, prepare_only);
  }
  return cudaErrorInvalidValue;
}

int resident_1d_seg_limit(int dtype) { return dtype == NLS_C128 ? 2048 : 4096; }

cudaError_t prepare_1d_resident(int dtype, int K, int cl, int seg_cap) {
  if (seg_cap > resident_1d_seg_limit(dtype) || cl < 1 || cl > 16) return cudaErrorInvalidValue;
  cudaError_t e = dispatch_res(dtype, K, nullptr, 0, cl, seg_cap, 0, nullptr, true);
  if (e == cudaSuccess && dtype == NLS_C64 && reg1d_cluster_fits(K, cl, seg_cap, 4 * K))
    e = dispatch_res(dtype, K, nullptr, 0, cl, seg_cap, 4 * K, nullptr, true);
  return e;
}

cudaError_t launch_1d_resident(int dtype, int K, const Inst1D* d_insts, int count, int cl,
                               int seg_cap, int shortest_seg, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if (seg_cap > resident_1d_seg_limit(dtype) || cl < 1 || cl > 16) return cudaErrorInvalidValue;
  return dispatch_res(dtype, K, d_insts, count, cl, seg_cap, shortest_seg, s, false);
}

template <typename T, int K>
static void stage_1d_t(int n, int s, const void* src, void* u, const void* P, void* acc, void* dst,
                       double dt, const PhysD& ph, const Stencil1D& op, cudaStream_t st) {
  rk4_1d_stage<T, K><<<(n + 255) / 256, 256, 0, st>>>(n, s, src, u, P, acc, dst,
                                                      make_params<T>(ph, dt, 0.0, 0.0, 0.0), op, (T)op.h);
}

template <typename T, int K>
static void rhs_1d_t(int n, const void* u, const void* P, void* v, const PhysD& ph, const Stencil1D& op,
                     cudaStream_t st) {
  rhs_1d<T, K><<<(n + 255) / 256, 256, 0, st>>>(n, u, P, v, make_params<T>(ph, 0.0, 0.0, 0.0, 0.0), op, (T)op.h);
}

cudaError_t launch_1d_stage(int dtype, int n, int s, const void* src, void* u, const void* P,
                            void* acc, void* dst, double dt, const PhysD& ph, const Stencil1D& op,
                            cudaStream_t st) {
  const int K = op.K;
  if (dtype == NLS_C128) {
    if (K == 1) stage_1d_t<double, 1>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else if (K == 2) stage_1d_t<double, 2>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else if (K == 3) stage_1d_t<double, 3>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else return cudaErrorInvalidValue;
  } else {
    if (K == 1) stage_1d_t<float, 1>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else if (K == 2) stage_1d_t<float, 2>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else if (K == 3) stage_1d_t<float, 3>(n, s, src, u, P, acc, dst, dt, ph, op, st);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_rhs_1d(int dtype, int n, const void* u, const void* P, void* v, const PhysD& ph,
                          const Stencil1D& op, cudaStream_t st) {
  const int K = op.K;
  if (dtype == NLS_C128) {
    if (K == 1) rhs_1d_t<double, 1>(n, u, P, v, ph, op, st);
    else if (K == 2) rhs_1d_t<double, 2>(n, u, P, v, ph, op, st);
    else if (K == 3) rhs_1d_t<double, 3>(n, u, P, v, ph, op, st);
    else return cudaErrorInvalidValue;
  } else {
    if (K == 1) rhs_1d_t<float, 1>(n, u, P, v, ph, op, st);
    else if (K == 2) rhs_1d_t<float, 2>(n, u, P, v, ph, op, st);
    else if (K == 3) rhs_1d_t<float, 3>(n, u, P, v, ph, op, st);
    else return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace nlsg
