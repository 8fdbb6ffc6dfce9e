// nls_types.h -- plain-old-data descriptors shared by the host runtime and the sm_103a kernels.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define NLSG_HD __host__ __device__
#else
#define NLSG_HD
#endif

namespace nlsg {

// Coefficients of the right-hand side, from the reference's 23-slot vector
// (nls/nls.f90:770-785; c_k = coeffs(k), 1-based).
struct PhysD {
  double c3, c4, c5, c6, c12, c13, c14;
};

// Step constants in the working precision, precomputed on the host: converting from double on the
// device would run on GB300's FP64 pipe, a small fraction of the FP32 rate.
template <typename T>
struct Params {
  T c3, c4, c5, c6, c12, c13, c14;   // coefficient slots 3-6 and 12-14
  T half_dt, dt, dt6;                // dt/2, dt, dt/6
  T wc, w1, w2;                      // 2-D cross-stencil weights (centre, distance 1, distance 2)
};

// 1-D radial operator L = D2 + diag(1/r_p) D1 on r_p = p h (make_laplacian, nls/nls.f90:132-295).
// Rows p >= K use the Toeplitz weights; rows p < K carry the mirror folds at r = 0 and are given
// as full rows.  Index d + K holds the weight of u_{p+d}.
struct Stencil1D {
  int order;          // 3, 5 or 7
  int K;              // (order - 1) / 2
  double h;
  double w2[7];       // second-derivative weights
  double w1[7];       // first-derivative weights (divided by r_p at run time)
  double near[3][7];  // full rows p = 0 .. K-1
  float w2f[7], w1f[7], nearf[3][7];  // the same in single precision
};

// 2-D Cartesian cross stencil (make_laplacian_2d_o3/o5, nls/nls.f90:297-351): the same weights
// along both axes; truncation (zero Dirichlet) outside the n x n grid.
struct Stencil2D {
  int order;          // 3 or 5
  int K;              // 1 or 2
  double center;      // weight of u_p (both axes' central terms together)
  double w[2];        // weight of the neighbours at distance 1 and 2 along either axis
};

// One independent solve inside a batched launch.
struct Inst1D {
  void* u;            // complex state, n nodes, in/out (updated in place)
  const void* P;      // pump, n nodes
  int n;
  int cl;             // CTAs (cluster size) that hold this instance
  int64_t steps;      // RK4 steps this launch applies
  double dt;
  PhysD ph;
  Stencil1D op;
  Params<float> pf;   // step constants (set_params)
  Params<double> pd;
};

// 16-byte aligned and sized, so a kernel can fetch a descriptor into shared memory with one bulk
// copy.
struct alignas(16) Inst2D {
  void* u[2];         // ping-pong complex state buffers, n x n, row-major (x contiguous)
  const void* P;      // pump, n x n
  int n;
  int tiles_x;        // tiles along x for the instance's tile shape
  int parity;         // which of u[0]/u[1] holds the current state before step 0 of the launch
  int64_t steps;      // step j of a launch group applies only while j < steps (0 = idle slot)
  double dt;
  PhysD ph;
  Stencil2D op;
  const void* tmap;   // 3 CUtensorMap (u[0], u[1], P) in global memory for the TMA path, or null
  Params<float> pf;   // step constants (set_params)
  Params<double> pd;
};

template <typename T>
inline Params<T> make_params(const PhysD& ph, double dt, double wc, double w1, double w2) {
  Params<T> p;
  p.c3 = (T)ph.c3; p.c4 = (T)ph.c4; p.c5 = (T)ph.c5; p.c6 = (T)ph.c6;
  p.c12 = (T)ph.c12; p.c13 = (T)ph.c13; p.c14 = (T)ph.c14;
  p.half_dt = (T)(dt * 0.5); p.dt = (T)dt; p.dt6 = (T)(dt / 6.0);
  p.wc = (T)wc; p.w1 = (T)w1; p.w2 = (T)w2;
  return p;
}

// Fill the precomputed constants of a 2-D instance from its ph, dt and op.
inline void set_params(Inst2D& I) {
  I.pf = make_params<float>(I.ph, I.dt, I.op.center, I.op.w[0], I.op.w[1]);
  I.pd = make_params<double>(I.ph, I.dt, I.op.center, I.op.w[0], I.op.w[1]);
}

inline void set_params(Inst1D& I) {
  I.pf = make_params<float>(I.ph, I.dt, 0.0, 0.0, 0.0);
  I.pd = make_params<double>(I.ph, I.dt, 0.0, 0.0, 0.0);
}

template <typename T> struct ParamsOf;
template <> struct ParamsOf<float> {
  static NLSG_HD const Params<float>& get(const Inst2D& I) { return I.pf; }
  static NLSG_HD const Params<float>& get(const Inst1D& I) { return I.pf; }
  static NLSG_HD float w2(const Stencil1D& s, int i) { return s.w2f[i]; }
  static NLSG_HD float w1(const Stencil1D& s, int i) { return s.w1f[i]; }
  static NLSG_HD float near(const Stencil1D& s, int p, int i) { return s.nearf[p][i]; }
};
template <> struct ParamsOf<double> {
  static NLSG_HD const Params<double>& get(const Inst2D& I) { return I.pd; }
  static NLSG_HD const Params<double>& get(const Inst1D& I) { return I.pd; }
  static NLSG_HD double w2(const Stencil1D& s, int i) { return s.w2[i]; }
  static NLSG_HD double w1(const Stencil1D& s, int i) { return s.w1[i]; }
  static NLSG_HD double near(const Stencil1D& s, int p, int i) { return s.near[p][i]; }
};

// One tile of the batched 2-D work list: instance index and tile index inside the instance.
struct TileItem {
  int inst;
  int tile;
};

// One work item of the streaming 2-D step: the strip of 64 columns starting at x0 of instance
// inst, whose columns [ox0, ox1) it writes, over the rows [y0, y1).  Grid sides are below 65536
// (n * n must fit an int).
struct StripItem {
  int inst;
  uint16_t x0, ox0, ox1, y0, y1, pad;
};

}  // namespace nlsg
