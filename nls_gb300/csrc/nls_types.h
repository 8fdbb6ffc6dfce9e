// nls_types.h -- plain-old-data descriptors shared by the host runtime and the sm_103a kernels.
#pragma once

#include <stdint.h>

namespace nlsg {

// Coefficients of the right-hand side, from the reference's 23-slot vector
// (nls/nls.f90:770-785; c_k = coeffs(k), 1-based).
struct PhysD {
  double c3, c4, c5, c6, c12, c13, c14;
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
};

struct Inst2D {
  void* u[2];         // ping-pong complex state buffers, n x n, row-major (x contiguous)
  const void* P;      // pump, n x n
  int n;
  int tiles_x;        // tiles along x for the instance's tile shape
  int parity;         // which of u[0]/u[1] holds the current state before step 0 of the launch
  int64_t steps;      // step j of a launch group applies only while j < steps (0 = idle slot)
  double dt;
  PhysD ph;
  Stencil2D op;
};

// One tile of the batched 2-D work list: instance index and tile index inside the instance.
struct TileItem {
  int inst;
  int tile;
};

}  // namespace nlsg
