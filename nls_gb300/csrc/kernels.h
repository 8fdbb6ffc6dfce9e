// kernels.h -- host-side launchers of the sm_103a kernels (internal to libnls_gb300).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "nls_types.h"

// dtype codes shared with the public C ABI
#ifndef NLS_C128
#define NLS_C128 0
#define NLS_C64 1
#endif

namespace nlsg {

// ---- 1-D
int resident_1d_seg_limit(int dtype);
// Sets the kernel attributes a later launch with these parameters needs (call outside capture).
cudaError_t prepare_1d_resident(int dtype, int K, int cl, int seg_cap);
// shortest_seg: the shortest of the cl segments over the launch's grids (see shortest_segment);
// complex64 clusters take the register-resident cluster kernel when every segment holds at least
// the 4K halo nodes a neighbour needs and a segment with its halos fits one CTA.
cudaError_t launch_1d_resident(int dtype, int K, const Inst1D* d_insts, int count, int cl,
                               int seg_cap, int shortest_seg, cudaStream_t s);
// The last (shortest) of the segments a grid of n nodes is cut into for cl CTAs of ceil(n / cl).
inline int shortest_segment(int n, int cl) {
  const int seg = (n + cl - 1) / cl;
  return n - (cl - 1) * seg;
}
cudaError_t launch_1d_stage(int dtype, int n, int s, const void* src, void* u, const void* P,
                            void* acc, void* dst, double dt, const PhysD& ph, const Stencil1D& op,
                            cudaStream_t st);
cudaError_t launch_rhs_1d(int dtype, int n, const void* u, const void* P, void* v, const PhysD& ph,
                          const Stencil1D& op, cudaStream_t st);

// ---- 2-D
// Fused-step tile shapes (region = tile + halo of 4K on every side).
enum TileShape2D {
  TILE_UNFUSED = 0,   // four stage launches per step, no halo recomputation
  TILE_64x64 = 1,     // region 64 x 64, 512 threads (single precision)
  TILE_128x32 = 2,    // region 128 x 32, 512 threads (single precision)
  TILE_32x32 = 3,     // region 32 x 32, 256 threads (either precision)
  TILE_64x64W = 4,    // region 64 x 64, 1024 threads (single precision)
  TILE_128x32W = 5,   // region 128 x 32, 1024 threads (single precision)
  TILE_64xO64 = 6,    // region 64 x (64 + 8K): output tiles 64 rows high, 512 threads
  TILE_64xO64M = 7,   // the same region with 768 (K = 1) or 640 (K = 2) threads
  // register-resident tiles (rk4_2d_reg, single precision): region 64 wide, warp = row strip
  TILE_R64x80 = 8,    // 16 warps x 5 rows (512 threads)
  TILE_R64x96 = 9,    // 12 warps x 8 rows (384 threads)
  TILE_R64x96S = 10,  // 8 warps x 12 rows (256 threads)
  TILE_R64x64 = 11,   // 16 warps x 4 rows (512 threads)
  TILE_R64x72 = 12,   // 8 warps x 9 rows (256 threads): 64 output rows at order 3
  TILE_R64x72W = 13,  // 12 warps x 6 rows (384 threads)
  TILE_R64x80S = 14,  // 8 warps x 10 rows (256 threads): 64 output rows at order 5
  // streaming wavefront (rk4_2d_stream, single precision): warp = 64-column strip walking down
  // a segment of rows, work items taken from a launch-wide counter
  TILE_STREAM = 15,
};
int tile_region_x(int shape);
int tile_region_y(int shape, int K);
int tile_out_x(int shape, int K);
int tile_out_y(int shape, int K);
bool tile_supported(int shape, int dtype);
// CTAs per SM the fused kernel reaches (for persistent grid sizing)
int fused_2d_blocks_per_sm(int dtype, int K, int shape);
cudaError_t launch_2d_fused(int dtype, int K, int shape, const Inst2D* d_insts,
                            const TileItem* d_items, int n_items, int j_step, int grid,
                            cudaStream_t s);
// TMA path of the fused step (complex64 only): one elected thread per CTA prefetches the next
// tile's state and pump boxes with cp.async.bulk.tensor while the current tile is computed.  A
// bounded wait on those copies that expires sets *wait_flag (the launching context's status word,
// a device int) and the CTA leaves.
bool tma_eligible(int dtype, int n, const void* u0, const void* u1, const void* P);
size_t tma_map_bytes();  // bytes of the 3 tensor maps of one instance (128-byte aligned slot)
int tma_encode_2d(int shape, int K, int n, const void* u0, const void* u1, const void* P, void* out_maps);
int fused_2d_tma_blocks_per_sm(int K, int shape);
cudaError_t launch_2d_fused_tma(int K, int shape, const Inst2D* d_insts, const TileItem* d_items,
                                int n_items, int j_step, int grid, cudaStream_t s, int* wait_flag);
// Test control: arm every tile barrier of the register-tile kernel for this many bytes more than
// its copies deliver (0 = normal operation), on the current device.
cudaError_t tile_tx_extra_set(unsigned bytes);
// Streaming step (TILE_STREAM): CTAs per SM (sets the shared-memory attribute; call outside any
// capture), warps per CTA, and the launch.  counter: two device unsigned ints, zero before the
// first launch; every launch leaves them zero again.
// kinds: which kernel forms a launch runs -- STREAM_EVEN (instances with an even side and 16-byte
// aligned buffers: paired 16-byte copies and stores) and/or STREAM_ODD (per-node copies); each
// form skips the other kind's items, so a group holding both launches both over one item list.
enum { STREAM_EVEN = 1, STREAM_ODD = 2 };
int stream_kind(int n, const void* u0, const void* u1, const void* P);
int stream_2d_blocks_per_sm(int K);
int stream_2d_warps_per_block();
// Device data of one streaming work list: descriptors, items (longest first), the launch's counter
// (3 words: next work index, warps done, epoch = steps published so far), and for launches of
// several steps the dependency lists and one flag per item (zeroed with the counter when the list
// is created) and the context's status word.
struct StreamLaunch {
  const Inst2D* insts;
  const StripItem* items;
  int n_items;
  unsigned* counter;
  const int2* dep_range;
  const int* deps;
  unsigned* flags;
  int* wait_flag;
};
// RK4 steps j0 .. j0 + nsteps - 1 of every item in one launch (nsteps > 1 needs kinds ==
// STREAM_EVEN and the dependency data).
cudaError_t launch_2d_stream(int K, int kinds, const StreamLaunch& L, int j0, int nsteps, int grid, cudaStream_t s);
cudaError_t stream_dep_extra_set(unsigned extra);
// Strip geometry of an n-wide grid (first strip against the left edge, interior strips with a
// 4K halo on both sides, last strip against the right edge), the segment height that minimises
// the estimated makespan of a set of grids over `slots` warps, the items of one instance, and
// the longest-first order the kernel takes them in.
struct StripGeom {
  int x0, ox0, ox1;
};
void stream_strips(int n, int K, std::vector<StripGeom>& out);
int stream_choose_ly(const std::vector<int>& ns, int K, int64_t slots);
// The tallest segment height giving at least items_per_slot items per resident warp, or -1 if
// that needs segments below min_ly rows.
int stream_choose_ly_multi(const std::vector<int>& ns, int K, int64_t slots, double items_per_slot, int min_ly);
void stream_items(int inst, int n, int K, int ly, std::vector<StripItem>& out, int extra_strips = 0);
// The items of a list of grids at segment height ly for `slots` resident warps (see the
// definition: lists just short of one item per warp are topped up to exactly one).
void stream_list_items(const std::vector<int>& ns, int K, int ly, int64_t slots, std::vector<StripItem>& out);
void stream_sort_items(std::vector<StripItem>& items);
// Dependency lists of a sorted item list (ns: grid side by instance): for item k every item of the
// same instance whose written region meets k's read region, or whose read region meets k's written
// region (k itself included); range[k] = {first, count} into deps.
void stream_deps(const std::vector<StripItem>& items, const std::vector<int>& ns, int K, std::vector<int2>& range,
                 std::vector<int>& deps);
cudaError_t launch_2d_stage(int dtype, int n, int s, const void* src, void* u, const void* P,
                            void* acc, void* dst, double dt, const PhysD& ph, const Stencil2D& op,
                            cudaStream_t st);
cudaError_t launch_rhs_2d(int dtype, int n, const void* u, const void* P, void* v, const PhysD& ph,
                          const Stencil2D& op, cudaStream_t st);

// ---- diagnostics (FP64 accumulation, deterministic two-pass reductions)
// Sums over n nodes, written to out[0..]:
//   norm:   out[0] = sum w_i |u_i|^2, out[1] = number of non-finite components
//   mu:     out[0..3] = sum w conj(u) v (re, im), sum w |u|^2 (re), 0
//   relerr: out[0] = sum (|a|^2 - |b|^2)^2, out[1] = sum |b|^4,
//           out[2] = sum (n_a - n_b)^2,     out[3] = sum n_b^2,  n = c12 P / (c13 + c14 |.|^2)
// weight mode: 0 = 1, 1 = radial r_i = i * dx (1-D chemical potential, nls/nls.f90:941-946)
size_t diag_partials_bytes(long long n);
cudaError_t diag_norm(int dtype, long long n, const void* u, int weight_mode, double dx,
                      double* d_partials, double* d_out, cudaStream_t st);
cudaError_t diag_mu(int dtype, long long n, const void* u, const void* v, int weight_mode,
                    double dx, double* d_partials, double* d_out, cudaStream_t st);
// damping: out[0] = sum w_i (c12 P_i / (c13 + c14 |u_i|^2) - 1) |u_i|^2, w_i = 2 pi (i r_step) dx
// (radial) or dx^2
cudaError_t diag_damping(int dtype, long long n, const void* u, const void* P, int radial, double r_step,
                         double dx, double c12, double c13, double c14, double* d_partials, double* d_out,
                         cudaStream_t st);
cudaError_t diag_relerr(int dtype_a, long long n, const void* a, const void* b_c128,
                        const double* P, double c12, double c13, double c14, double* d_partials,
                        double* d_out, cudaStream_t st);

}  // namespace nlsg
