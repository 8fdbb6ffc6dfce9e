// nls_common.cuh -- device-side building blocks shared by every sm_103a kernel of the solver.
//
// The physics is the right-hand side of the reference's `hamiltonian` (nls/nls.f90:621-650,
// 841-870) with the adiabatic reservoir of `revervoir` (nls/nls.f90:570-581):
//     r  = c12 P / (c13 + c14 |u|^2)
//     v  = (c3 r - c4) u + i [ L u - (c5 |u|^2 + c6 r) u ]
// i.e. v_re = a u_re + b u_im - (L u)_im and v_im = a u_im - b u_re + (L u)_re with
// a = c3 r - c4 and b = c5 |u|^2 + c6 r, integrated by the classical RK4 of `runge_kutta`
// (nls/nls.f90:705-734).  c_k is the reference's 1-based coeffs(k).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nls_types.h"

namespace nlsg {

// Programmatic dependent launch: a kernel launched with programmatic stream serialisation may
// start while the kernel before it in the stream is still running.  pdl_wait() blocks until that
// kernel has completed and its memory operations are visible (it returns at once when there is
// no such predecessor), so it comes before anything reads the predecessor's output;
// pdl_trigger() then lets the next kernel's CTAs be scheduled as this one's free their SMs.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// Launch with programmatic stream serialisation (see pdl_wait).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

template <typename T> struct C2;
template <> struct C2<float> { typedef float2 type; };
template <> struct C2<double> { typedef double2 type; };

template <typename T> __device__ __forceinline__ typename C2<T>::type mk(T x, T y) {
  typename C2<T>::type v; v.x = x; v.y = y; return v;
}

// Coefficients of the right-hand side in the working precision.
template <typename T> struct Phys {
  T c3, c4, c5, c6, c12, c13, c14;
};

template <typename T> __host__ __device__ inline Phys<T> phys_from(const PhysD& p) {
  Phys<T> q;
  q.c3 = (T)p.c3; q.c4 = (T)p.c4; q.c5 = (T)p.c5; q.c6 = (T)p.c6;
  q.c12 = (T)p.c12; q.c13 = (T)p.c13; q.c14 = (T)p.c14;
  return q;
}

template <typename T> __device__ __forceinline__ Phys<T> phys_of(const Params<T>& p) {
  Phys<T> q;
  q.c3 = p.c3; q.c4 = p.c4; q.c5 = p.c5; q.c6 = p.c6; q.c12 = p.c12; q.c13 = p.c13; q.c14 = p.c14;
  return q;
}

// Division in the reservoir term.  Double precision: the FP64 pipe runs at a small fraction of
// the FP32 rate on GB300, so the quotient is formed as a * (1/b) with the reciprocal computed by
// the Newton-Raphson iteration y <- y + y (1 - b y) (each step squares the relative error) from an
// FP32 seed (PTX rcp.approx.ftz.f32 of b rounded to float, relative error below about 2^-21 against
// 1/b): one step leaves a relative error below about 2^-42 (2e-13), far inside the plain path's
// 1e-10 parity over tens of thousands of steps, and saves two FP64 FMAs a node-stage against two
// steps (configs 0 and 1: 5.46 -> 5.21 and 24.5 -> 23.4 us per step).  Denominators outside the
// FP32 normal range (and NaN) take the IEEE division.  Single precision (the precision form)
// uses the hardware fast reciprocal-based quotient, within 2 ulp and far inside the form's 1e-4
// error budget.
#ifndef NLSG_RDIV_NEWTON
#define NLSG_RDIV_NEWTON 1
#endif
__device__ __forceinline__ double rdiv(double a, double b) {
  const float bf = (float)b;
  if (!(fabsf(bf) >= 1e-30f && fabsf(bf) <= 1e30f)) return a / b;
  float s;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(bf));
  double y = (double)s;
  y = __fma_rn(y, __fma_rn(-b, y, 1.0), y);
  if (NLSG_RDIV_NEWTON > 1) y = __fma_rn(y, __fma_rn(-b, y, 1.0), y);
  return a * y;
}
__device__ __forceinline__ float rdiv(float a, float b) { return __fdividef(a, b); }

// Right-hand side at one node, given the node value u, pump p and the Laplacian lu.
template <typename T>
__device__ __forceinline__ typename C2<T>::type rhs(typename C2<T>::type u, T p,
                                                    typename C2<T>::type lu, const Phys<T>& ph) {
  T s = u.x * u.x + u.y * u.y;
  T r = rdiv(ph.c12 * p, ph.c13 + ph.c14 * s);
  T a = ph.c3 * r - ph.c4;
  T b = ph.c5 * s + ph.c6 * r;
  typename C2<T>::type v;
  v.x = a * u.x + b * u.y - lu.y;
  v.y = a * u.y - b * u.x + lu.x;
  return v;
}

// RK4 stage constants: the input of stage s+1 is u + kc[s] * k_s, and the update accumulates
// k1 + 2 k2 + 2 k3 + k4 (nls/nls.f90:726-731).
template <typename T> struct RK {
  T half_dt, dt, dt6;
};

template <typename T> __device__ __forceinline__ RK<T> rk_of(const Params<T>& p) {
  RK<T> r;
  r.half_dt = p.half_dt;
  r.dt = p.dt;
  r.dt6 = p.dt6;
  return r;
}

// Weights of the 2-D cross stencil (make_laplacian_2d_o3/o5, nls/nls.f90:297-351) for the
// contiguous axis x and the strided axis y: centre weight plus one weight per distance d.
template <typename T> struct Cross {
  T center, wx[2], wy[2];
};

template <typename T> __host__ __device__ inline Cross<T> cross_from(const Stencil2D& s) {
  Cross<T> c;
  c.center = (T)s.center;
  c.wx[0] = (T)s.w[0]; c.wx[1] = (T)s.w[1];
  c.wy[0] = (T)s.w[0]; c.wy[1] = (T)s.w[1];
  return c;
}

// Packed FP32x2 arithmetic on node pairs or (re, im) pairs (Blackwell FADD2 / FMUL2 / FFMA2).
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// Approximate reciprocal (PTX rcp.approx.ftz.f32, relative error about one unit in the last
// place): the reservoir quotient of the register-resident complex64 kernels.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Warp + block reduction of NV doubles (fixed order, deterministic).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* >= 32*NV */) {
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) smem[warp * NV + i] = v[i];
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = lane < nw ? smem[lane * NV + i] : 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
  }
}

}  // namespace nlsg
