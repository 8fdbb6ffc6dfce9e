// runtime.cu -- host runtime behind the C ABI of include/nls_gb300.h.
//
// Contexts, kernel-path selection, CUDA-graph replay of long step sequences, FP64 diagnostics,
// the batched form (many independent solves advanced by one graph) and the serving pool
// (continuous batching of requests admitted against an HBM budget).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <atomic>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/nls_gb300.h"
#include "kernels.h"
#include "nls_types.h"

#define NLS_API extern "C" __attribute__((visibility("default")))

namespace nlsg {
int host_make_laplacian(int n, int order, double h, double* op);
int host_make_laplacian_2d(int n, int order, double h, double* blocks, int* orders);
int host_stencil_1d(int n, int order, double h, Stencil1D* s);
int host_stencil_2d(int order, double h, Stencil2D* s);
}  // namespace nlsg

using namespace nlsg;

// ------------------------------------------------------------------ context

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct nls_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  static constexpr int kSide = 4;    // side streams for concurrent 1-D groups
  cudaStream_t side[kSide] = {};
  cudaEvent_t side_done[kSide] = {};
  std::string err;
  std::mutex mu;
  int64_t launches = 0;
  DevBuf scratch;   // state ping-pong / stage buffers of single solves
  DevBuf desc;      // instance descriptors and tile lists of single solves
  DevBuf io;        // uploaded inputs of host-buffer calls
  DevBuf diag;      // diagnostics partials and results
  DevBuf diagv;     // H(u) scratch of the device chemical potential
  double* h_diag = nullptr;  // pinned
  // Status word of the bounded tile waits of this context's launches (a device int set by a
  // fused 2-D kernel whose copy wait expired), and its pinned host mirror.
  int* wait_flag = nullptr;
  int* h_wait_flag = nullptr;
};

static int fail(nls_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

static int fail_cuda(nls_ctx* ctx, cudaError_t e, const char* what) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  if (ctx) ctx->err = buf;
  return e == cudaErrorMemoryAllocation ? NLS_ERR_NOMEM : NLS_ERR_CUDA;
}

#define CK(ctx, x)                                       \
  do {                                                   \
    cudaError_t e_ = (x);                                \
    if (e_ != cudaSuccess) return fail_cuda(ctx, e_, #x); \
  } while (0)

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// A bounded wait inside one of this context's tile kernels that expired leaves the context's
// status word set; report it once (then clear it).  Synchronises the context's stream.
static int check_timeout(nls_ctx* ctx) {
  if (cudaMemcpyAsync(ctx->h_wait_flag, ctx->wait_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return fail(ctx, NLS_ERR_CUDA, "reading the tile-wait status word failed");
  if (*ctx->h_wait_flag) {
    *ctx->h_wait_flag = 0;
    cudaMemsetAsync(ctx->wait_flag, 0, sizeof(int), ctx->stream);
    return fail(ctx, NLS_ERR_TIMEOUT, "a tile copy did not arrive within its bounded wait");
  }
  return NLS_OK;
}
static size_t csize(int dtype) { return dtype == NLS_C128 ? 16 : 8; }
static size_t rsize(int dtype) { return dtype == NLS_C128 ? 8 : 4; }

static PhysD phys_of(const double* c) {
  PhysD p;
  p.c3 = c[2]; p.c4 = c[3]; p.c5 = c[4]; p.c6 = c[5];
  p.c12 = c[11]; p.c13 = c[12]; p.c14 = c[13];
  return p;
}

static int check_problem(nls_ctx* ctx, int dtype, const nls_problem* pr) {
  if (!pr) return fail(ctx, NLS_ERR_INVALID, "null problem");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "dtype must be NLS_C128 or NLS_C64");
  if (pr->dim == 1) {
    if (pr->order != 3 && pr->order != 5 && pr->order != 7)
      return fail(ctx, NLS_ERR_ORDER, "1-D order must be 3, 5 or 7");
    if (pr->n < pr->order) return fail(ctx, NLS_ERR_INVALID, "1-D grid needs at least order nodes");
  } else if (pr->dim == 2) {
    if (pr->order != 3 && pr->order != 5)
      return fail(ctx, NLS_ERR_ORDER, "2-D order must be 3 or 5 (the reference's order 7 is undefined)");
    if (pr->n < pr->order) return fail(ctx, NLS_ERR_INVALID, "2-D grid needs at least order nodes per side");
    if ((long long)pr->n * pr->n > (long long)INT_MAX) return fail(ctx, NLS_ERR_INVALID, "2-D grid too large");
  } else {
    return fail(ctx, NLS_ERR_INVALID, "dim must be 1 or 2");
  }
  if (!(pr->dx > 0.0) || !(pr->dt == pr->dt)) return fail(ctx, NLS_ERR_INVALID, "dx must be positive, dt finite");
  return NLS_OK;
}

// ------------------------------------------------------------------ path selection

// 1-D: CTAs per solve for the resident kernel, 0 = unfused stage kernels.
static int choose_cl(int dtype, int n, int K, int variant) {
  const int lim = resident_1d_seg_limit(dtype);
  auto feasible = [&](int cl) {
    if (cl < 1 || cl > 16) return false;
    const int seg = (n + cl - 1) / cl;
    if (cl == 1) return seg <= lim && seg >= 2 * K;
    // the cluster form keeps 4 buffers of seg + 8K nodes and needs segments of at least 4K
    return seg + 8 * K <= lim && seg >= 4 * K;
  };
  if (variant == 0) return 0;
  if (variant > 0) return feasible(variant) ? variant : -1;
  if (dtype == NLS_C128) {
    // FP64 is ALU-bound on GB300: spread the grid over up to 16 SMs of a cluster.
    int cl = std::min(16, std::max(1, n / 64));
    while (cl > 1 && !feasible(cl)) --cl;
    if (feasible(cl)) return cl;
  } else {
    for (int cl = 1; cl <= 16; cl *= 2)
      if (feasible(cl)) return cl;
  }
  return 0;
}

// 2-D: tile shape (TILE_*), 0 = unfused.
static int choose_shape(int dtype, int n, int K, int variant) {
  if (variant >= 0) {
    if (variant == TILE_UNFUSED) return 0;
    if (!tile_supported(variant, dtype)) return -1;
    return variant;
  }
  // complex64: the streaming wavefront (no vertical halo, no CTA barrier); at order 5 it holds 8
  // warps per SM and pays 8 rows of warm-up and drain per segment, so below 2048 per side the
  // register-resident tile is faster (measured on 1024^2: 16 against 20 us per step)
  if (dtype == NLS_C64) return (K == 1 || n >= 2048) ? TILE_STREAM : TILE_R64x96S;
  // complex128 is FP64-bound on GB300: the stage kernels (no halo recomputation) beat the fused
  // tile at every size measured (256^2 .. 1024^2, orders 3 and 5)
  return TILE_UNFUSED;
}

// ------------------------------------------------------------------ graph helpers

// Run `reps` replays of the launch sequence produced by `body` (captured once), then `tail`
// launches directly.  The body must leave every device-side parity where it found it.
template <typename F>
static cudaError_t replay(nls_ctx* ctx, int64_t reps, F&& body) {
  if (reps <= 0) return cudaSuccess;
  if (reps == 1) return body();
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t eb = body();
  e = cudaStreamEndCapture(ctx->stream, &g);
  if (eb != cudaSuccess) { if (g) cudaGraphDestroy(g); return eb; }
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return e;
  for (int64_t r = 0; r < reps && e == cudaSuccess; ++r) e = cudaGraphLaunch(ge, ctx->stream);
  cudaGraphExecDestroy(ge);
  return e;
}

// ------------------------------------------------------------------ single solves

static int solve_1d_dev(nls_ctx* ctx, int dtype, const nls_problem* pr, int64_t iters,
                        const void* P, void* u) {
  Stencil1D op;
  int st = host_stencil_1d(pr->n, pr->order, pr->dx, &op);
  if (st) return fail(ctx, st == 2 ? NLS_ERR_ORDER : NLS_ERR_INVALID, "invalid 1-D operator");
  const PhysD ph = phys_of(pr->coeffs);
  const int n = pr->n;
  const int cl = choose_cl(dtype, n, op.K, pr->variant);
  if (cl < 0) return fail(ctx, NLS_ERR_INVALID, "1-D variant not feasible for this size");
  if (iters <= 0) return NLS_OK;
  if (cl > 0) {
    Inst1D I;
    std::memset(&I, 0, sizeof(I));
    I.u = u; I.P = P; I.n = n; I.cl = cl; I.steps = iters; I.dt = pr->dt; I.ph = ph; I.op = op;
    set_params(I);
    CK(ctx, ctx->desc.ensure(sizeof(Inst1D)));
    CK(ctx, cudaMemcpyAsync(ctx->desc.p, &I, sizeof(I), cudaMemcpyHostToDevice, ctx->stream));
    const int seg = (n + cl - 1) / cl;
    CK(ctx, launch_1d_resident(dtype, op.K, (const Inst1D*)ctx->desc.p, 1, cl, seg, shortest_segment(n, cl),
                               ctx->stream));
    ctx->launches += 1;
    return NLS_OK;
  }
  // unfused: u (state), tA, tB, acc
  const size_t cb = align256((size_t)n * csize(dtype));
  CK(ctx, ctx->scratch.ensure(3 * cb));
  char* base = (char*)ctx->scratch.p;
  void *tA = base, *tB = base + cb, *acc = base + 2 * cb;
  auto one_step = [&]() -> cudaError_t {
    cudaError_t e;
    if ((e = launch_1d_stage(dtype, n, 1, u, u, P, acc, tA, pr->dt, ph, op, ctx->stream))) return e;
    if ((e = launch_1d_stage(dtype, n, 2, tA, u, P, acc, tB, pr->dt, ph, op, ctx->stream))) return e;
    if ((e = launch_1d_stage(dtype, n, 3, tB, u, P, acc, tA, pr->dt, ph, op, ctx->stream))) return e;
    return launch_1d_stage(dtype, n, 4, tA, u, P, acc, nullptr, pr->dt, ph, op, ctx->stream);
  };
  const int S = 16;
  CK(ctx, replay(ctx, iters / S, [&]() -> cudaError_t {
       for (int i = 0; i < S; ++i) { cudaError_t e = one_step(); if (e) return e; }
       return cudaSuccess;
     }));
  for (int64_t i = 0; i < iters % S; ++i) CK(ctx, one_step());
  ctx->launches += 4 * iters;
  return NLS_OK;
}

// Streaming 2-D step (complex64): ping-pong between the caller's buffer and one scratch buffer,
// strip items over segments of the height that balances the grid's work over the GPU's warps.
static int stream_grid(nls_ctx* ctx, int K, int n_items) {
  const int occ = std::max(1, stream_2d_blocks_per_sm(K));
  const int wpb = stream_2d_warps_per_block();
  return std::max(1, std::min(ctx->sm_count * occ, (n_items + wpb - 1) / wpb));
}
static int64_t stream_slots(nls_ctx* ctx, int K) {
  return (int64_t)ctx->sm_count * std::max(1, stream_2d_blocks_per_sm(K)) * stream_2d_warps_per_block();
}

// Steps per launch of a streaming list that runs several steps per launch (bounded so that a
// launch stays well under a second on the largest lists).
static constexpr int kStreamStepsPerLaunch = 512;

// Several steps per launch pay off where a warp finishing an item can take another whose
// dependencies are met: lists of at least 1.5 items per resident warp (the batched mix: 1.9),
// at order 3, whose grids all take the paired form.  Measured: the batched mix 2.04e11 ->
// 2.23e11 node-steps/s; a single 4096^2 grid (one item per warp and step, so each step waits for
// the previous one as at a launch boundary) 2.18e11 -> 1.84e11 at order 3, and at order 5, whose
// nine-row loop body no longer fits the instruction cache once warps drift apart, 1.26e11 ->
// 0.74e11.
static std::atomic<int> g_stream_multi_mode{0};   // test control: 0 automatic, 1 always, 2 never

// Segment height of a streaming list over grids ns: the one-step-per-launch schedule simulation's
// choice, except for the largest lists (below).  (The tallest height giving only 1.5 items per
// warp, so that more lists run several steps per launch, measured worse: 8192^2 2.37e11 ->
// 2.13e11, the batched mix 2.23e11 -> 2.08e11; shorter segments on a 4096^2 grid, 2.21e11 ->
// 2.15e11 at half the height and 2.05e11 at a third.)
static int stream_plan_ly(nls_ctx* ctx, const std::vector<int>& ns, int K) {
  const int64_t slots = stream_slots(ctx, K);
  // Lists large enough for three items per resident warp at segments of 192 rows or more take
  // the tallest such segments and run several steps per launch (the dataflow balances three
  // items per warp; the warm-up and drain of segments that tall cost little): 8192^2 order 3
  // 2.36e11 -> 2.44e11 node-steps/s.
  bool paired = true;
  for (int n : ns) paired = paired && n % 2 == 0;
  if (K == 1 && paired && g_stream_multi_mode.load() != 2) {
    const int ly = stream_choose_ly_multi(ns, K, slots, 3.0, 192);
    if (ly > 0) return ly;
  }
  return stream_choose_ly(ns, K, slots);
}
static bool stream_multi_ok(nls_ctx* ctx, int K, int kinds, int n_items) {
  if (kinds != STREAM_EVEN || n_items <= 0) return false;
  const int mode = g_stream_multi_mode.load();
  if (mode) return mode == 1;
  return K == 1 && 2 * (int64_t)n_items >= 3 * stream_slots(ctx, K);
}

// Device layout of one streaming work list after its descriptors: items, counter (256 B),
// dependency ranges, dependency indices, flags.
struct StreamListLayout {
  size_t items, counter, range, deps, flags, end;
};
static StreamListLayout stream_list_layout(size_t at, size_t n_items, size_t n_deps) {
  StreamListLayout L;
  L.items = at;
  L.counter = L.items + align256(sizeof(StripItem) * std::max<size_t>(1, n_items));
  L.range = L.counter + 256;
  L.deps = L.range + align256(sizeof(int2) * std::max<size_t>(1, n_items));
  L.flags = L.deps + align256(sizeof(int) * std::max<size_t>(1, n_deps));
  L.end = L.flags + align256(sizeof(unsigned) * std::max<size_t>(1, n_items));
  return L;
}

static int solve_2d_stream(nls_ctx* ctx, const nls_problem* pr, const Stencil2D& op, const PhysD& ph,
                           int64_t iters, const void* P, void* u) {
  const int n = pr->n;
  const size_t N = (size_t)n * n;
  const size_t cb = align256(N * csize(NLS_C64));
  CK(ctx, ctx->scratch.ensure(cb));
  Inst2D I;
  std::memset(&I, 0, sizeof(I));
  I.u[0] = u; I.u[1] = ctx->scratch.p; I.P = P; I.n = n; I.tiles_x = 0; I.parity = 0;
  I.steps = INT64_MAX; I.dt = pr->dt; I.ph = ph; I.op = op;
  set_params(I);
  std::vector<StripItem> items;
  stream_list_items({n}, op.K, stream_plan_ly(ctx, {n}, op.K), stream_slots(ctx, op.K), items);
  stream_sort_items(items);
  const int kinds = stream_kind(n, I.u[0], I.u[1], P);
  const int n_items = (int)items.size();
  const bool multi = stream_multi_ok(ctx, op.K, kinds, n_items);
  std::vector<int2> range;
  std::vector<int> deps;
  if (multi) stream_deps(items, {n}, op.K, range, deps);
  const size_t ib = align256(sizeof(Inst2D));
  const StreamListLayout Ly = stream_list_layout(ib, items.size(), deps.size());
  CK(ctx, ctx->desc.ensure(Ly.end));
  char* base = (char*)ctx->desc.p;
  CK(ctx, cudaMemcpyAsync(base, &I, sizeof(I), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + Ly.items, items.data(), sizeof(StripItem) * n_items, cudaMemcpyHostToDevice,
                          ctx->stream));
  CK(ctx, cudaMemsetAsync(base + Ly.counter, 0, 256, ctx->stream));
  StreamLaunch L{(const Inst2D*)base, (const StripItem*)(base + Ly.items), n_items, (unsigned*)(base + Ly.counter),
                 nullptr, nullptr, nullptr, ctx->wait_flag};
  if (multi) {
    CK(ctx, cudaMemcpyAsync(base + Ly.range, range.data(), sizeof(int2) * n_items, cudaMemcpyHostToDevice,
                            ctx->stream));
    CK(ctx, cudaMemcpyAsync(base + Ly.deps, deps.data(), sizeof(int) * deps.size(), cudaMemcpyHostToDevice,
                            ctx->stream));
    CK(ctx, cudaMemsetAsync(base + Ly.flags, 0, sizeof(unsigned) * n_items, ctx->stream));
    L.dep_range = (const int2*)(base + Ly.range);
    L.deps = (const int*)(base + Ly.deps);
    L.flags = (unsigned*)(base + Ly.flags);
  }
  const int grid = stream_grid(ctx, op.K, n_items);
  if (multi) {
    // whole chunks of steps per launch; the state alternates buffers each step
    for (int64_t j = 0; j < iters;) {
      const int s = (int)std::min<int64_t>(kStreamStepsPerLaunch, iters - j);
      CK(ctx, launch_2d_stream(op.K, kinds, L, (int)(j & 1), s, grid, ctx->stream));
      ctx->launches += 1;
      j += s;
    }
  } else {
    const int S = 64;  // even: a replay returns the state to the caller's buffer
    CK(ctx, replay(ctx, iters / S, [&]() -> cudaError_t {
         for (int j = 0; j < S; ++j) {
           cudaError_t e = launch_2d_stream(op.K, kinds, L, j, 1, grid, ctx->stream);
           if (e) return e;
         }
         return cudaSuccess;
       }));
    const int64_t rem = iters % S;
    for (int64_t j = 0; j < rem; ++j) CK(ctx, launch_2d_stream(op.K, kinds, L, (int)j, 1, grid, ctx->stream));
    ctx->launches += iters * ((kinds & STREAM_EVEN ? 1 : 0) + (kinds & STREAM_ODD ? 1 : 0));
  }
  if (iters & 1) CK(ctx, cudaMemcpyAsync(u, ctx->scratch.p, N * csize(NLS_C64), cudaMemcpyDeviceToDevice, ctx->stream));
  return NLS_OK;
}

static int solve_2d_dev(nls_ctx* ctx, int dtype, const nls_problem* pr, int64_t iters,
                        const void* P, void* u) {
  Stencil2D op;
  if (host_stencil_2d(pr->order, pr->dx, &op)) return fail(ctx, NLS_ERR_ORDER, "2-D order must be 3 or 5");
  const PhysD ph = phys_of(pr->coeffs);
  const int n = pr->n;
  const int shape = choose_shape(dtype, n, op.K, pr->variant);
  if (shape < 0) return fail(ctx, NLS_ERR_INVALID, "2-D variant not supported for this precision/order");
  if (iters <= 0) return NLS_OK;
  const size_t N = (size_t)n * n;
  const size_t cb = align256(N * csize(dtype));
  if (shape == TILE_UNFUSED) {
    CK(ctx, ctx->scratch.ensure(3 * cb));
    char* base = (char*)ctx->scratch.p;
    void *tA = base, *tB = base + cb, *acc = base + 2 * cb;
    auto one_step = [&]() -> cudaError_t {
      cudaError_t e;
      if ((e = launch_2d_stage(dtype, n, 1, u, u, P, acc, tA, pr->dt, ph, op, ctx->stream))) return e;
      if ((e = launch_2d_stage(dtype, n, 2, tA, u, P, acc, tB, pr->dt, ph, op, ctx->stream))) return e;
      if ((e = launch_2d_stage(dtype, n, 3, tB, u, P, acc, tA, pr->dt, ph, op, ctx->stream))) return e;
      return launch_2d_stage(dtype, n, 4, tA, u, P, acc, nullptr, pr->dt, ph, op, ctx->stream);
    };
    const int S = 16;
    CK(ctx, replay(ctx, iters / S, [&]() -> cudaError_t {
         for (int i = 0; i < S; ++i) { cudaError_t e = one_step(); if (e) return e; }
         return cudaSuccess;
       }));
    for (int64_t i = 0; i < iters % S; ++i) CK(ctx, one_step());
    ctx->launches += 4 * iters;
    return NLS_OK;
  }
  if (shape == TILE_STREAM) return solve_2d_stream(ctx, pr, op, ph, iters, P, u);
  // fused: ping-pong between the caller's buffer and one scratch buffer
  const int tx = tile_out_x(shape, op.K), ty = tile_out_y(shape, op.K);
  const int tiles_x = (n + tx - 1) / tx, tiles_y = (n + ty - 1) / ty;
  const int n_items = tiles_x * tiles_y;
  CK(ctx, ctx->scratch.ensure(cb));
  Inst2D I;
  std::memset(&I, 0, sizeof(I));
  I.u[0] = u; I.u[1] = ctx->scratch.p; I.P = P; I.n = n; I.tiles_x = tiles_x; I.parity = 0;
  I.steps = INT64_MAX; I.dt = pr->dt; I.ph = ph; I.op = op;
  set_params(I);
  std::vector<TileItem> items(n_items);
  for (int t = 0; t < n_items; ++t) items[t] = TileItem{0, t};
  const size_t ib = align256(sizeof(Inst2D));
  const size_t tb = align256(sizeof(TileItem) * n_items);
  const bool tma = tma_eligible(dtype, n, u, ctx->scratch.p, P);
  CK(ctx, ctx->desc.ensure(ib + tb + (tma ? tma_map_bytes() : 0)));
  Inst2D* dI = (Inst2D*)ctx->desc.p;
  TileItem* dT = (TileItem*)((char*)ctx->desc.p + ib);
  if (tma) {
    alignas(128) unsigned char maps[3 * 128];
    if (tma_encode_2d(shape, op.K, n, u, ctx->scratch.p, P, maps)) return fail(ctx, NLS_ERR_CUDA, "tensor map encoding");
    void* dmaps = (char*)ctx->desc.p + ib + tb;
    CK(ctx, cudaMemcpyAsync(dmaps, maps, tma_map_bytes(), cudaMemcpyHostToDevice, ctx->stream));
    I.tmap = dmaps;
  }
  CK(ctx, cudaMemcpyAsync(dI, &I, sizeof(I), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(dT, items.data(), sizeof(TileItem) * n_items, cudaMemcpyHostToDevice, ctx->stream));
  const int occ = tma ? fused_2d_tma_blocks_per_sm(op.K, shape) : fused_2d_blocks_per_sm(dtype, op.K, shape);
  const int grid = std::max(1, std::min(n_items, ctx->sm_count * std::max(1, occ)));
  auto launch = [&](int j) -> cudaError_t {
    return tma ? launch_2d_fused_tma(op.K, shape, dI, dT, n_items, j, grid, ctx->stream, ctx->wait_flag)
               : launch_2d_fused(dtype, op.K, shape, dI, dT, n_items, j, grid, ctx->stream);
  };
  const int S = 64;  // even: a replay returns the state to the caller's buffer
  CK(ctx, replay(ctx, iters / S, [&]() -> cudaError_t {
       for (int j = 0; j < S; ++j) {
         cudaError_t e = launch(j);
         if (e) return e;
       }
       return cudaSuccess;
     }));
  const int64_t rem = iters % S;
  for (int64_t j = 0; j < rem; ++j) CK(ctx, launch((int)j));
  if (rem & 1) CK(ctx, cudaMemcpyAsync(u, ctx->scratch.p, N * csize(dtype), cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->launches += iters;
  return NLS_OK;
}

static int solve_dev(nls_ctx* ctx, int dtype, const nls_problem* pr, int64_t iters, const void* P, void* u) {
  int st = check_problem(ctx, dtype, pr);
  if (st) return st;
  if (!P || !u) return fail(ctx, NLS_ERR_INVALID, "null device pointer");
  if (iters < 0) return fail(ctx, NLS_ERR_INVALID, "iters must be >= 0");
  CK(ctx, cudaSetDevice(ctx->device));
  return pr->dim == 1 ? solve_1d_dev(ctx, dtype, pr, iters, P, u) : solve_2d_dev(ctx, dtype, pr, iters, P, u);
}

// Host-buffer solve: upload, solve on the device, download.
static int solve_host(nls_ctx* ctx, int dtype, int dim, double dt, double dx, int n, int order,
                      int iters, const double* coeffs, const void* P, const void* u0, void* u) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!coeffs || !P || !u0 || !u) return fail(ctx, NLS_ERR_INVALID, "null host pointer");
  nls_problem pr;
  std::memset(&pr, 0, sizeof(pr));
  pr.dim = dim; pr.n = n; pr.order = order; pr.variant = -1; pr.dt = dt; pr.dx = dx;
  std::memcpy(pr.coeffs, coeffs, sizeof(pr.coeffs));
  int st = check_problem(ctx, dtype, &pr);
  if (st) return st;
  CK(ctx, cudaSetDevice(ctx->device));
  const size_t N = dim == 1 ? (size_t)n : (size_t)n * n;
  const size_t ub = align256(N * csize(dtype)), pb = align256(N * rsize(dtype));
  CK(ctx, ctx->io.ensure(ub + pb));
  void* du = ctx->io.p;
  void* dP = (char*)ctx->io.p + ub;
  CK(ctx, cudaMemcpyAsync(du, u0, N * csize(dtype), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(dP, P, N * rsize(dtype), cudaMemcpyHostToDevice, ctx->stream));
  st = dim == 1 ? solve_1d_dev(ctx, dtype, &pr, iters, dP, du) : solve_2d_dev(ctx, dtype, &pr, iters, dP, du);
  if (st) return st;
  CK(ctx, cudaMemcpyAsync(u, du, N * csize(dtype), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return check_timeout(ctx);
}

// ------------------------------------------------------------------ diagnostics

static int diag_ensure(nls_ctx* ctx) {
  CK(ctx, ctx->diag.ensure(diag_partials_bytes(0) + 64 * sizeof(double)));
  if (!ctx->h_diag) CK(ctx, cudaMallocHost(&ctx->h_diag, 64 * sizeof(double)));
  return NLS_OK;
}

static double* diag_out(nls_ctx* ctx) { return (double*)((char*)ctx->diag.p + diag_partials_bytes(0)); }

// Sums of the chemical potential (nls/nls.f90:921-971) of a device state u: S = sum w conj(u) H(u)
// and M = sum w |u|^2 (w = r_i in 1-D, 1 in 2-D), FP64, with H evaluated with the order-5
// operator like the reference.  v is device scratch of the state's size.  Blocks until done.
static int chem_pot_dev(nls_ctx* ctx, int dtype, int dim, double dx, int n, const double* coeffs,
                        const void* dP, const void* du, void* dv, double* s_re, double* s_im, double* m) {
  const PhysD ph = phys_of(coeffs);
  const size_t N = dim == 1 ? (size_t)n : (size_t)n * n;
  int st = diag_ensure(ctx);
  if (st) return st;
  if (dim == 1) {
    Stencil1D op;
    if (host_stencil_1d(n, 5, dx, &op)) return fail(ctx, NLS_ERR_INVALID, "operator");
    CK(ctx, launch_rhs_1d(dtype, n, du, dP, dv, ph, op, ctx->stream));
  } else {
    Stencil2D op;
    host_stencil_2d(5, dx, &op);
    CK(ctx, launch_rhs_2d(dtype, n, du, dP, dv, ph, op, ctx->stream));
  }
  CK(ctx, diag_mu(dtype, (long long)N, du, dv, dim == 1 ? 1 : 0, dx, (double*)ctx->diag.p, diag_out(ctx), ctx->stream));
  CK(ctx, cudaMemcpyAsync(ctx->h_diag, diag_out(ctx), 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->launches += 3;
  *s_re = ctx->h_diag[0];
  *s_im = ctx->h_diag[1];
  *m = ctx->h_diag[2];
  return NLS_OK;
}

static int chem_pot(nls_ctx* ctx, int dtype, int dim, double dx, int n, const double* coeffs,
                    const void* P, const void* u0, double* s_re, double* s_im, double* m) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!coeffs || !P || !u0) return fail(ctx, NLS_ERR_INVALID, "null host pointer");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  if (n < 5) return fail(ctx, NLS_ERR_INVALID, "chemical potential needs n >= 5 (order-5 operator)");
  CK(ctx, cudaSetDevice(ctx->device));
  const size_t N = dim == 1 ? (size_t)n : (size_t)n * n;
  const size_t ub = align256(N * csize(dtype)), pb = align256(N * rsize(dtype));
  CK(ctx, ctx->io.ensure(2 * ub + pb));
  void* du = ctx->io.p;
  void* dv = (char*)ctx->io.p + ub;
  void* dP = (char*)ctx->io.p + 2 * ub;
  CK(ctx, cudaMemcpyAsync(du, u0, N * csize(dtype), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(dP, P, N * rsize(dtype), cudaMemcpyHostToDevice, ctx->stream));
  return chem_pot_dev(ctx, dtype, dim, dx, n, coeffs, dP, du, dv, s_re, s_im, m);
}

// ------------------------------------------------------------------ arena allocator

class Arena {
 public:
  cudaError_t init(size_t bytes) {
    bytes = align256(bytes);
    cudaError_t e = cudaMalloc(&base_, bytes);
    if (e != cudaSuccess) { base_ = nullptr; return e; }
    size_ = bytes;
    free_.clear();
    free_[0] = bytes;
    used_ = 0;
    return cudaSuccess;
  }
  void destroy() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
    size_ = 0;
    free_.clear();
  }
  // first fit; returns SIZE_MAX if nothing fits
  size_t alloc(size_t bytes) {
    bytes = align256(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const size_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > bytes) free_[off + bytes] = len - bytes;
        used_ += bytes;
        return off;
      }
    }
    return SIZE_MAX;
  }
  void release(size_t off, size_t bytes) {
    bytes = align256(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  char* at(size_t off) const { return base_ + off; }
  size_t used() const { return used_; }
  size_t size() const { return size_; }

 private:
  char* base_ = nullptr;
  size_t size_ = 0;
  size_t used_ = 0;
  std::map<size_t, size_t> free_;
};

// ------------------------------------------------------------------ batched form

// A resident set of independent solves.  Instances are grouped by kernel: 1-D by (K, cluster
// size), 2-D fused by (K, tile shape); 2-D unfused instances step on their own.  One run(steps)
// is one CUDA graph: the 1-D resident launches fork onto an auxiliary stream while the main
// stream issues `steps` fused-step launches per 2-D group.
struct Group1D {
  int K, cl, seg_cap;
  std::vector<int> idx;
  Inst1D* d = nullptr;
};
struct Group2D {
  int K, shape, grid;
  std::vector<int> idx;
  Inst2D* d = nullptr;
  TileItem* items = nullptr;
  int n_items = 0;
  bool tma = false;
  char* maps = nullptr;    // 3 tensor maps per member (TMA path)
  // streaming step (TILE_STREAM): strip items of every member, longest first, the launch-wide
  // item counter, and the dependency lists and flags of launches of several steps
  std::vector<StripItem> sitems_h;
  std::vector<int2> range_h;
  std::vector<int> deps_h;
  StreamLaunch sl{};
  int kinds = 0;           // STREAM_EVEN / STREAM_ODD forms its members need
  bool multi = false;      // several steps per launch
};

struct Member {
  nls_problem pr;
  int kind;        // 1 = 1-D resident, 2 = 2-D fused, 3 = 2-D unfused, 4 = 1-D unfused
  int group;
  size_t N;        // nodes
  char* u[2];
  char* P;
  char* scratch;   // unfused stage buffers (3 complex arrays)
  int parity;
  Stencil1D op1;
  Stencil2D op2;
};

struct nls_batch {
  nls_ctx* ctx;
  int dtype;
  std::vector<Member> m;
  std::vector<Group1D> g1;
  std::vector<Group2D> g2;
  char* mem = nullptr;       // one allocation for states, pumps, descriptors
  size_t mem_bytes = 0;
  int parity = 0;            // common parity of the 2-D fused instances
  std::vector<size_t> poff, soff;  // packed host layout: pump and state byte offsets per instance
  size_t pump_bytes = 0, state_bytes = 0;
  std::map<int64_t, cudaGraphExec_t> graphs;
  std::mutex mu;
};

static int batch_build(nls_batch* b, const nls_problem* probs, int count) {
  nls_ctx* ctx = b->ctx;
  const int dtype = b->dtype;
  b->m.resize(count);
  // layout pass
  size_t off = 0;
  std::map<std::pair<int, int>, int> key1, key2;
  std::vector<size_t> offs(count * 4);
  for (int i = 0; i < count; ++i) {
    Member& M = b->m[i];
    M.pr = probs[i];
    int st = check_problem(ctx, dtype, &M.pr);
    if (st) return st;
    M.parity = 0;
    M.scratch = nullptr;
    if (M.pr.dim == 1) {
      if (host_stencil_1d(M.pr.n, M.pr.order, M.pr.dx, &M.op1)) return fail(ctx, NLS_ERR_INVALID, "1-D operator");
      M.N = M.pr.n;
      const int cl = choose_cl(dtype, M.pr.n, M.op1.K, M.pr.variant);
      if (cl < 0) return fail(ctx, NLS_ERR_INVALID, "1-D variant not feasible");
      M.kind = cl > 0 ? 1 : 4;
      if (M.kind == 1) {
        // group by (K, cluster size, segment size class) so a launch sizes its CTAs to its members
        const int seg = (M.pr.n + cl - 1) / cl;
        int cls = 64;
        while (cls < seg) cls *= 2;
        auto k = std::make_pair(M.op1.K * 1000 + cl, cls);
        if (!key1.count(k)) { key1[k] = (int)b->g1.size(); b->g1.push_back(Group1D{M.op1.K, cl, 0, {}, nullptr}); }
        M.group = key1[k];
        Group1D& G = b->g1[M.group];
        G.idx.push_back(i);
        G.seg_cap = std::max(G.seg_cap, (M.pr.n + cl - 1) / cl);
      }
    } else {
      if (host_stencil_2d(M.pr.order, M.pr.dx, &M.op2)) return fail(ctx, NLS_ERR_ORDER, "2-D operator");
      M.N = (size_t)M.pr.n * M.pr.n;
      const int shape = choose_shape(dtype, M.pr.n, M.op2.K, M.pr.variant);
      if (shape < 0) return fail(ctx, NLS_ERR_INVALID, "2-D variant not supported");
      M.kind = shape > 0 ? 2 : 3;
      if (M.kind == 2) {
        auto k = std::make_pair(M.op2.K, shape);
        if (!key2.count(k)) {
          key2[k] = (int)b->g2.size();
          Group2D G;
          G.K = M.op2.K; G.shape = shape; G.grid = 0;
          b->g2.push_back(G);
        }
        M.group = key2[k];
        b->g2[M.group].idx.push_back(i);
      }
    }
  }
  // states and pumps field by field -- every pump, every state, the second state buffers of the
  // fused 2-D instances, the unfused stage buffers -- each instance padded to 256 bytes, so the pump
  // and state blocks have the packed host layout of nls_batch_set_packed / nls_batch_get_packed
  b->poff.resize(count);
  b->soff.resize(count);
  for (int i = 0; i < count; ++i) {
    offs[4 * i + 2] = off;
    b->poff[i] = off;
    off += align256(b->m[i].N * rsize(dtype));
  }
  b->pump_bytes = off;
  const size_t state_base = off;
  for (int i = 0; i < count; ++i) {
    offs[4 * i + 0] = off;
    b->soff[i] = off - state_base;
    off += align256(b->m[i].N * csize(dtype));
  }
  b->state_bytes = off - state_base;
  for (int i = 0; i < count; ++i)
    if (b->m[i].kind == 2) { offs[4 * i + 1] = off; off += align256(b->m[i].N * csize(dtype)); }
  for (int i = 0; i < count; ++i)
    if (b->m[i].kind == 3 || b->m[i].kind == 4) { offs[4 * i + 3] = off; off += 3 * align256(b->m[i].N * csize(dtype)); }
  // descriptors
  std::vector<size_t> g1off(b->g1.size()), g2off(b->g2.size()), g2items(b->g2.size()), g2maps;
  for (size_t g = 0; g < b->g1.size(); ++g) { g1off[g] = off; off += align256(sizeof(Inst1D) * b->g1[g].idx.size()); }
  for (size_t g = 0; g < b->g2.size(); ++g) {
    Group2D& G = b->g2[g];
    int items = 0;
    size_t item_bytes = 0;
    if (G.shape == TILE_STREAM) {
      std::vector<int> ns;
      for (int i : G.idx) ns.push_back(b->m[i].pr.n);
      const int ly = stream_plan_ly(ctx, ns, G.K);
      G.sitems_h.clear();
      stream_list_items(ns, G.K, ly, stream_slots(ctx, G.K), G.sitems_h);
      stream_sort_items(G.sitems_h);
      stream_deps(G.sitems_h, ns, G.K, G.range_h, G.deps_h);
      items = (int)G.sitems_h.size();
      item_bytes = stream_list_layout(0, G.sitems_h.size(), G.deps_h.size()).end;
    } else {
      for (int i : G.idx) {
        const int tx = tile_out_x(G.shape, G.K), ty = tile_out_y(G.shape, G.K), n = b->m[i].pr.n;
        items += ((n + tx - 1) / tx) * ((n + ty - 1) / ty);
      }
      item_bytes = align256(sizeof(TileItem) * std::max(1, items));
    }
    G.n_items = items;
    g2off[g] = off; off += align256(sizeof(Inst2D) * G.idx.size());
    g2items[g] = off; off += item_bytes;
    g2maps.push_back(off); off += G.shape == TILE_STREAM ? 0 : align256(tma_map_bytes() * G.idx.size());
  }
  b->mem_bytes = std::max<size_t>(off, 256);
  CK(ctx, cudaMalloc(&b->mem, b->mem_bytes));
  CK(ctx, cudaMemsetAsync(b->mem, 0, b->mem_bytes, ctx->stream));
  for (int i = 0; i < count; ++i) {
    Member& M = b->m[i];
    M.u[0] = b->mem + offs[4 * i + 0];
    M.u[1] = M.kind == 2 ? b->mem + offs[4 * i + 1] : M.u[0];
    M.P = b->mem + offs[4 * i + 2];
    if (M.kind == 3 || M.kind == 4) M.scratch = b->mem + offs[4 * i + 3];
  }
  for (size_t g = 0; g < b->g1.size(); ++g) b->g1[g].d = (Inst1D*)(b->mem + g1off[g]);
  for (size_t g = 0; g < b->g2.size(); ++g) {
    Group2D& G = b->g2[g];
    G.d = (Inst2D*)(b->mem + g2off[g]);
    if (G.shape == TILE_STREAM) {
      // items, counter, dependency ranges and lists, flags (counter and flags zeroed with the block)
      const StreamListLayout Ly = stream_list_layout(g2items[g], G.sitems_h.size(), G.deps_h.size());
      G.sl = StreamLaunch{G.d, (const StripItem*)(b->mem + Ly.items), G.n_items, (unsigned*)(b->mem + Ly.counter),
                          (const int2*)(b->mem + Ly.range), (const int*)(b->mem + Ly.deps),
                          (unsigned*)(b->mem + Ly.flags), ctx->wait_flag};
      if (G.n_items) {
        CK(ctx, cudaMemcpyAsync(b->mem + Ly.items, G.sitems_h.data(), sizeof(StripItem) * G.n_items,
                                cudaMemcpyHostToDevice, ctx->stream));
        CK(ctx, cudaMemcpyAsync(b->mem + Ly.range, G.range_h.data(), sizeof(int2) * G.n_items,
                                cudaMemcpyHostToDevice, ctx->stream));
        CK(ctx, cudaMemcpyAsync(b->mem + Ly.deps, G.deps_h.data(), sizeof(int) * G.deps_h.size(),
                                cudaMemcpyHostToDevice, ctx->stream));
      }
      G.tma = false;
      G.grid = stream_grid(ctx, G.K, std::max(1, G.n_items));
      G.kinds = 0;
      for (int i : G.idx) {
        const Member& M = b->m[i];
        G.kinds |= stream_kind(M.pr.n, M.u[0], M.u[1], M.P);
      }
      G.multi = stream_multi_ok(ctx, G.K, G.kinds, G.n_items);
      continue;
    }
    G.items = (TileItem*)(b->mem + g2items[g]);
    std::vector<TileItem> items;
    items.reserve(G.n_items);
    for (size_t k = 0; k < G.idx.size(); ++k) {
      const Member& M = b->m[G.idx[k]];
      const int tx = tile_out_x(G.shape, G.K), ty = tile_out_y(G.shape, G.K), n = M.pr.n;
      const int t = ((n + tx - 1) / tx) * ((n + ty - 1) / ty);
      for (int q = 0; q < t; ++q) items.push_back(TileItem{(int)k, q});
    }
    if (!items.empty())
      CK(ctx, cudaMemcpyAsync(G.items, items.data(), sizeof(TileItem) * items.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    // TMA path when every member qualifies (complex64, n % 4 == 0, 16-byte aligned buffers)
    G.maps = b->mem + g2maps[g];
    G.tma = true;
    for (int i : G.idx) {
      const Member& M = b->m[i];
      G.tma = G.tma && tma_eligible(dtype, M.pr.n, M.u[0], M.u[1], M.P);
    }
    if (G.tma) {
      std::vector<unsigned char> maps(tma_map_bytes() * G.idx.size() + 128);
      unsigned char* hm = (unsigned char*)(((uintptr_t)maps.data() + 127) & ~(uintptr_t)127);
      for (size_t k = 0; k < G.idx.size(); ++k) {
        const Member& M = b->m[G.idx[k]];
        if (tma_encode_2d(G.shape, G.K, M.pr.n, M.u[0], M.u[1], M.P, hm + k * tma_map_bytes()))
          return fail(ctx, NLS_ERR_CUDA, "tensor map encoding");
      }
      CK(ctx, cudaMemcpyAsync(G.maps, hm, tma_map_bytes() * G.idx.size(), cudaMemcpyHostToDevice, ctx->stream));
      CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
    const int occ = G.tma ? fused_2d_tma_blocks_per_sm(G.K, G.shape) : fused_2d_blocks_per_sm(dtype, G.K, G.shape);
    G.grid = std::max(1, std::min(G.n_items, ctx->sm_count * std::max(1, occ)));
  }
  for (auto& G : b->g1) CK(ctx, prepare_1d_resident(dtype, G.K, G.cl, G.seg_cap));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

// Write the descriptors for a run of `steps` steps starting at the batch's current parity.
static int batch_descriptors(nls_batch* b, int64_t steps) {
  nls_ctx* ctx = b->ctx;
  for (auto& G : b->g1) {
    std::vector<Inst1D> h(G.idx.size());
    for (size_t k = 0; k < G.idx.size(); ++k) {
      const Member& M = b->m[G.idx[k]];
      Inst1D& I = h[k];
      std::memset(&I, 0, sizeof(I));
      I.u = M.u[0]; I.P = M.P; I.n = M.pr.n; I.cl = G.cl; I.steps = steps; I.dt = M.pr.dt;
      I.ph = phys_of(M.pr.coeffs); I.op = M.op1;
      set_params(I);
    }
    CK(ctx, cudaMemcpyAsync(G.d, h.data(), sizeof(Inst1D) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  for (auto& G : b->g2) {
    std::vector<Inst2D> h(G.idx.size());
    for (size_t k = 0; k < G.idx.size(); ++k) {
      const Member& M = b->m[G.idx[k]];
      Inst2D& I = h[k];
      std::memset(&I, 0, sizeof(I));
      const int tx = tile_out_x(G.shape, G.K);
      I.u[0] = M.u[0]; I.u[1] = M.u[1]; I.P = M.P; I.n = M.pr.n;
      I.tiles_x = G.shape == TILE_STREAM ? 0 : (M.pr.n + tx - 1) / tx;
      I.parity = M.parity; I.steps = INT64_MAX; I.dt = M.pr.dt;
      I.ph = phys_of(M.pr.coeffs); I.op = M.op2;
      I.tmap = G.tma ? G.maps + k * tma_map_bytes() : nullptr;
      set_params(I);
    }
    CK(ctx, cudaMemcpyAsync(G.d, h.data(), sizeof(Inst2D) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  return NLS_OK;
}

// A streaming group whose members all take the paired form runs many steps per launch.
static bool stream_multi(const Group2D& G) { return G.shape == TILE_STREAM && G.multi; }

static cudaError_t batch_sequence(nls_batch* b, int64_t steps) {
  nls_ctx* ctx = b->ctx;
  const int dtype = b->dtype;
  cudaError_t e;
  const bool fork = !b->g1.empty();
  const int nside = std::min<int>(nls_ctx::kSide, (int)b->g1.size());
  if (fork) {
    // the 1-D groups run concurrently on side streams while the main stream steps the 2-D tiles
    if ((e = cudaEventRecord(ctx->ev_fork, ctx->stream))) return e;
    for (int i = 0; i < nside; ++i)
      if ((e = cudaStreamWaitEvent(ctx->side[i], ctx->ev_fork, 0))) return e;
    for (size_t g = 0; g < b->g1.size(); ++g) {
      auto& G = b->g1[g];
      int shortest = INT32_MAX;
      for (int i : G.idx) shortest = std::min(shortest, shortest_segment(b->m[i].pr.n, G.cl));
      if ((e = launch_1d_resident(dtype, G.K, G.d, (int)G.idx.size(), G.cl, G.seg_cap, shortest,
                                  ctx->side[g % nside])))
        return e;
    }
  }
  // streaming groups whose members all take the paired form: many steps per launch
  for (auto& G : b->g2)
    if (stream_multi(G))
      for (int64_t j = 0; j < steps;) {
        const int s = (int)std::min<int64_t>(kStreamStepsPerLaunch, steps - j);
        if ((e = launch_2d_stream(G.K, G.kinds, G.sl, (int)j, s, G.grid, ctx->stream))) return e;
        j += s;
      }
  for (int64_t j = 0; j < steps; ++j) {
    for (auto& G : b->g2)
      if (!stream_multi(G) &&
          (e = G.shape == TILE_STREAM
                   ? launch_2d_stream(G.K, G.kinds, G.sl, (int)j, 1, G.grid, ctx->stream)
               : G.tma ? launch_2d_fused_tma(G.K, G.shape, G.d, G.items, G.n_items, (int)j, G.grid, ctx->stream,
                                             ctx->wait_flag)
                       : launch_2d_fused(dtype, G.K, G.shape, G.d, G.items, G.n_items, (int)j, G.grid, ctx->stream)))
        return e;
    for (auto& M : b->m) {
      if (M.kind != 3) continue;
      const size_t cb = align256(M.N * csize(dtype));
      void *tA = M.scratch, *tB = M.scratch + cb, *acc = M.scratch + 2 * cb;
      const PhysD ph = phys_of(M.pr.coeffs);
      const int n = M.pr.n;
      void* u = M.u[0];
      if ((e = launch_2d_stage(dtype, n, 1, u, u, M.P, acc, tA, M.pr.dt, ph, M.op2, ctx->stream))) return e;
      if ((e = launch_2d_stage(dtype, n, 2, tA, u, M.P, acc, tB, M.pr.dt, ph, M.op2, ctx->stream))) return e;
      if ((e = launch_2d_stage(dtype, n, 3, tB, u, M.P, acc, tA, M.pr.dt, ph, M.op2, ctx->stream))) return e;
      if ((e = launch_2d_stage(dtype, n, 4, tA, u, M.P, acc, nullptr, M.pr.dt, ph, M.op2, ctx->stream))) return e;
    }
    for (auto& M : b->m) {
      if (M.kind != 4) continue;
      const size_t cb = align256(M.N * csize(dtype));
      void *tA = M.scratch, *tB = M.scratch + cb, *acc = M.scratch + 2 * cb;
      const PhysD ph = phys_of(M.pr.coeffs);
      const int n = M.pr.n;
      void* u = M.u[0];
      if ((e = launch_1d_stage(dtype, n, 1, u, u, M.P, acc, tA, M.pr.dt, ph, M.op1, ctx->stream))) return e;
      if ((e = launch_1d_stage(dtype, n, 2, tA, u, M.P, acc, tB, M.pr.dt, ph, M.op1, ctx->stream))) return e;
      if ((e = launch_1d_stage(dtype, n, 3, tB, u, M.P, acc, tA, M.pr.dt, ph, M.op1, ctx->stream))) return e;
      if ((e = launch_1d_stage(dtype, n, 4, tA, u, M.P, acc, nullptr, M.pr.dt, ph, M.op1, ctx->stream))) return e;
    }
  }
  if (fork) {
    for (int i = 0; i < nside; ++i) {
      if ((e = cudaEventRecord(ctx->side_done[i], ctx->side[i]))) return e;
      if ((e = cudaStreamWaitEvent(ctx->stream, ctx->side_done[i], 0))) return e;
    }
  }
  return cudaSuccess;
}

static int64_t batch_launches(const nls_batch* b, int64_t steps) {
  int64_t l = (int64_t)b->g1.size();
  for (auto& G : b->g2)
    l += stream_multi(G) ? (steps + kStreamStepsPerLaunch - 1) / kStreamStepsPerLaunch
                         : steps * (G.shape == TILE_STREAM && G.kinds == (STREAM_EVEN | STREAM_ODD) ? 2 : 1);
  for (auto& M : b->m) if (M.kind == 3 || M.kind == 4) l += 4 * steps;
  return l;
}

// ------------------------------------------------------------------ serving pool

struct Slot {
  bool used = false, done = false;
  nls_problem pr;
  int64_t tag = 0;
  int64_t remaining = 0;        // steps not yet enqueued in a chunk
  int64_t finish_chunk = -1;    // chunk whose completion finishes the request (all steps enqueued)
  size_t off = 0, bytes = 0;
  size_t N = 0;
  char* u[2] = {nullptr, nullptr};
  char* P = nullptr;
  int parity = 0;               // buffer holding the state after every enqueued step
  int kind = 0;       // 1 = 1-D resident, 2 = 2-D fused
  int K = 0, cl = 0, shape = 0, ntiles = 0, tiles_x = 0;
  Stencil1D op1;
  Stencil2D op2;
  uint64_t finish_seq = 0;
  bool tma = false;
  std::vector<unsigned char> maps;   // 3 tensor maps (host copy), when tma
};

// A chunk enqueued on the context's stream: descriptor buffer `buf` (two, so the next chunk's
// image can be uploaded while the previous chunk runs) and its start/done events.
struct PoolChunk {
  int64_t id;
  int buf;
};

struct nls_pool {
  nls_ctx* ctx;
  int dtype;
  int chunk;
  Arena arena;
  std::vector<Slot> slots;
  uint64_t seq = 0;
  DevBuf d_desc[2];
  std::vector<char> h_desc;
  cudaStream_t copy = nullptr;          // admission uploads and result downloads
  cudaEvent_t ev_upload = nullptr;      // recorded after the latest admission upload
  bool upload_pending = false;          // the next chunk must wait for ev_upload
  cudaEvent_t ev_start[2] = {}, ev_done[2] = {};
  std::deque<PoolChunk> inflight;       // at most two, oldest first
  int64_t next_chunk = 0;
  double busy_ms = 0.0;                 // device time of the completed chunks
  bool waiting = false;                 // a thread is blocked in nls_pool_wait
  std::mutex mu;
};

static size_t pool_bytes(int dtype, const nls_problem& p) {
  const size_t N = p.dim == 1 ? (size_t)p.n : (size_t)p.n * p.n;
  const size_t cb = align256(N * csize(dtype)), pb = align256(N * rsize(dtype));
  return p.dim == 1 ? cb + pb : 2 * cb + pb;
}

// ------------------------------------------------------------------ C ABI

NLS_API int nls_version(int* major, int* minor, int* patch) {
  if (!major || !minor || !patch) return NLS_ERR_INVALID;
  *major = 0; *minor = 2; *patch = 0;
  return NLS_OK;
}

NLS_API int nls_make_laplacian(int n, int order, double h, double* op) {
  if (!op || n < 1) return NLS_ERR_INVALID;
  return host_make_laplacian(n, order, h, op);
}

NLS_API int nls_make_laplacian_2d(int n, int order, double h, double* blocks, int* orders) {
  if (!blocks || !orders || n < 1) return NLS_ERR_INVALID;
  return host_make_laplacian_2d(n, order, h, blocks, orders);
}

static void ctx_release(nls_ctx* ctx) {
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->aux) cudaStreamSynchronize(ctx->aux);
  for (int i = 0; i < nls_ctx::kSide; ++i)
    if (ctx->side[i]) cudaStreamSynchronize(ctx->side[i]);
  ctx->scratch.release();
  ctx->desc.release();
  ctx->io.release();
  ctx->diag.release();
  ctx->diagv.release();
  if (ctx->h_diag) cudaFreeHost(ctx->h_diag);
  if (ctx->wait_flag) cudaFree(ctx->wait_flag);
  if (ctx->h_wait_flag) cudaFreeHost(ctx->h_wait_flag);
  for (int i = 0; i < nls_ctx::kSide; ++i) {
    if (ctx->side_done[i]) cudaEventDestroy(ctx->side_done[i]);
    if (ctx->side[i]) cudaStreamDestroy(ctx->side[i]);
  }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

NLS_API int nls_ctx_create(int device, nls_ctx** out) {
  if (!out) return NLS_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return NLS_ERR_CUDA;
  if (device < 0 || device >= ndev) return NLS_ERR_INVALID;
  nls_ctx* ctx = new nls_ctx();
  ctx->device = device;
  bool ok = cudaSetDevice(device) == cudaSuccess &&
            cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < nls_ctx::kSide; ++i)
    ok = cudaStreamCreateWithFlags(&ctx->side[i], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&ctx->side_done[i], cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaMalloc(&ctx->wait_flag, sizeof(int)) == cudaSuccess &&
       cudaMallocHost(&ctx->h_wait_flag, sizeof(int)) == cudaSuccess &&
       cudaMemset(ctx->wait_flag, 0, sizeof(int)) == cudaSuccess;
  if (ok) *ctx->h_wait_flag = 0;
  if (!ok) {
    ctx_release(ctx);
    return NLS_ERR_CUDA;
  }
  *out = ctx;
  return NLS_OK;
}

NLS_API int nls_ctx_destroy(nls_ctx* ctx) {
  if (!ctx) return NLS_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx_release(ctx);
  return NLS_OK;
}

NLS_API int nls_ctx_stream(nls_ctx* ctx, void** stream) {
  if (!ctx || !stream) return NLS_ERR_INVALID;
  *stream = (void*)ctx->stream;
  return NLS_OK;
}

NLS_API int nls_ctx_synchronize(nls_ctx* ctx) {
  if (!ctx) return NLS_ERR_INVALID;
  CK(ctx, cudaSetDevice(ctx->device));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return check_timeout(ctx);
}

NLS_API const char* nls_last_error(nls_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

NLS_API int64_t nls_ctx_launch_count(nls_ctx* ctx) { return ctx ? ctx->launches : -1; }

NLS_API int nls_solve_1d(nls_ctx* ctx, int dtype, double dt, double dx, int n, int order, int iters,
                         const double* coeffs23, const void* pumping, const void* u0, void* u) {
  return solve_host(ctx, dtype, 1, dt, dx, n, order, iters, coeffs23, pumping, u0, u);
}

NLS_API int nls_solve_2d(nls_ctx* ctx, int dtype, double dt, double dx, int n, int order, int iters,
                         const double* coeffs23, const void* pumping, const void* u0, void* u) {
  return solve_host(ctx, dtype, 2, dt, dx, n, order, iters, coeffs23, pumping, u0, u);
}

NLS_API int nls_solve_device(nls_ctx* ctx, int dtype, const nls_problem* problem, int64_t iters,
                             const void* pumping_dev, void* u_dev) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return solve_dev(ctx, dtype, problem, iters, pumping_dev, u_dev);
}

NLS_API int nls_chemical_potential_1d(nls_ctx* ctx, int dtype, double dx, int n, const double* coeffs23,
                                      const void* pumping, const void* u0, double* mu_re, double* mu_im) {
  if (!mu_re || !mu_im) return fail(ctx, NLS_ERR_INVALID, "null output");
  double sr, si, m;
  int st = chem_pot(ctx, dtype, 1, dx, n, coeffs23, pumping, u0, &sr, &si, &m);
  if (st) return st;
  // mu = i S / M with S = sum r conj(u0) H(u0), M = sum r |u0|^2 (nls/nls.f90:945-947)
  *mu_re = -si / m;
  *mu_im = sr / m;
  return NLS_OK;
}

NLS_API int nls_chemical_potential_2d(nls_ctx* ctx, int dtype, double dx, int n, const double* coeffs23,
                                      const void* pumping, const void* u0, double* mu) {
  if (!mu) return fail(ctx, NLS_ERR_INVALID, "null output");
  double sr, si, m;
  int st = chem_pot(ctx, dtype, 2, dx, n, coeffs23, pumping, u0, &sr, &si, &m);
  if (st) return st;
  *mu = -si / m;  // real part of i S / M (nls/nls.f90:967-970)
  return NLS_OK;
}

NLS_API int nls_chemical_potential_device(nls_ctx* ctx, int dtype, const nls_problem* pr, const void* pumping_dev,
                                          const void* u_dev, double* mu_re, double* mu_im) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!pr || !pumping_dev || !u_dev || !mu_re || !mu_im) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  if ((pr->dim != 1 && pr->dim != 2) || pr->n < 5) return fail(ctx, NLS_ERR_INVALID, "dim 1 or 2 and n >= 5");
  CK(ctx, cudaSetDevice(ctx->device));
  const size_t N = pr->dim == 1 ? (size_t)pr->n : (size_t)pr->n * pr->n;
  CK(ctx, ctx->diagv.ensure(N * csize(dtype)));
  double sr, si, m;
  int st = chem_pot_dev(ctx, dtype, pr->dim, pr->dx, pr->n, pr->coeffs, pumping_dev, u_dev, ctx->diagv.p, &sr, &si, &m);
  if (st) return st;
  *mu_re = -si / m;   // mu = i S / M
  *mu_im = sr / m;
  return NLS_OK;
}

NLS_API int nls_norm_device(nls_ctx* ctx, int dtype, int64_t count, const void* u_dev, double* sum_sq,
                            int64_t* nonfinite) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!u_dev || !sum_sq || count < 0) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  CK(ctx, cudaSetDevice(ctx->device));
  int st = diag_ensure(ctx);
  if (st) return st;
  CK(ctx, diag_norm(dtype, count, u_dev, 0, 0.0, (double*)ctx->diag.p, diag_out(ctx), ctx->stream));
  CK(ctx, cudaMemcpyAsync(ctx->h_diag, diag_out(ctx), 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->launches += 2;
  *sum_sq = ctx->h_diag[0];
  if (nonfinite) *nonfinite = (int64_t)ctx->h_diag[1];
  return ctx->h_diag[1] > 0 ? fail(ctx, NLS_ERR_NONFINITE, "non-finite values in state") : NLS_OK;
}

NLS_API int nls_damping_integral_device(nls_ctx* ctx, int dtype, const nls_problem* pr, const void* pumping_dev,
                                        const void* u_dev, double* integral) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!pr || !pumping_dev || !u_dev || !integral) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  if ((pr->dim != 1 && pr->dim != 2) || pr->n < 1 || !(pr->dx > 0.0)) return fail(ctx, NLS_ERR_INVALID, "dim 1 or 2, n >= 1, dx > 0");
  CK(ctx, cudaSetDevice(ctx->device));
  int st = diag_ensure(ctx);
  if (st) return st;
  const long long N = pr->dim == 1 ? (long long)pr->n : (long long)pr->n * pr->n;
  const double r_step = pr->n > 1 ? (double)pr->n * pr->dx / (double)(pr->n - 1) : 0.0;
  const double* c = pr->coeffs;
  CK(ctx, diag_damping(dtype, N, u_dev, pumping_dev, pr->dim == 1 ? 1 : 0, r_step, pr->dx, c[11], c[12], c[13],
                       (double*)ctx->diag.p, diag_out(ctx), ctx->stream));
  CK(ctx, cudaMemcpyAsync(ctx->h_diag, diag_out(ctx), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->launches += 2;
  *integral = ctx->h_diag[0];
  return NLS_OK;
}

NLS_API int nls_density_error_device(nls_ctx* ctx, int dtype, int64_t count, const void* u_dev,
                                     const void* u_ref_c128_dev, const double* pumping_f64_dev, double c12,
                                     double c13, double c14, double* rel_l2_density, double* rel_l2_reservoir) {
  if (!ctx) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!u_dev || !u_ref_c128_dev || !pumping_f64_dev || !rel_l2_density || !rel_l2_reservoir || count < 0)
    return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  CK(ctx, cudaSetDevice(ctx->device));
  int st = diag_ensure(ctx);
  if (st) return st;
  CK(ctx, diag_relerr(dtype, count, u_dev, u_ref_c128_dev, pumping_f64_dev, c12, c13, c14,
                      (double*)ctx->diag.p, diag_out(ctx), ctx->stream));
  CK(ctx, cudaMemcpyAsync(ctx->h_diag, diag_out(ctx), 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->launches += 2;
  const double* v = ctx->h_diag;
  *rel_l2_density = v[1] > 0 ? std::sqrt(v[0] / v[1]) : std::sqrt(v[0]);
  *rel_l2_reservoir = v[3] > 0 ? std::sqrt(v[2] / v[3]) : std::sqrt(v[2]);
  return NLS_OK;
}

// ---- batch

NLS_API int nls_batch_create(nls_ctx* ctx, int dtype, int count, const nls_problem* problems, nls_batch** out) {
  if (!ctx) return NLS_ERR_INVALID;
  if (!out || !problems || count <= 0) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  *out = nullptr;
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(ctx, cudaSetDevice(ctx->device));
  nls_batch* b = new nls_batch();
  b->ctx = ctx;
  b->dtype = dtype;
  int st = batch_build(b, problems, count);
  if (st) {
    if (b->mem) cudaFree(b->mem);
    delete b;
    return st;
  }
  *out = b;
  return NLS_OK;
}

NLS_API int nls_test_set_tile_tx_extra(int device, unsigned extra_bytes) {
  if (cudaSetDevice(device) != cudaSuccess) return NLS_ERR_CUDA;
  return tile_tx_extra_set(extra_bytes) == cudaSuccess ? NLS_OK : NLS_ERR_CUDA;
}

NLS_API int nls_test_set_stream_steps_per_launch(int mode) {
  if (mode < 0 || mode > 2) return NLS_ERR_INVALID;
  g_stream_multi_mode.store(mode);
  return NLS_OK;
}

NLS_API int nls_test_set_stream_dep_extra(int device, unsigned extra_steps) {
  if (cudaSetDevice(device) != cudaSuccess) return NLS_ERR_CUDA;
  return stream_dep_extra_set(extra_steps) == cudaSuccess ? NLS_OK : NLS_ERR_CUDA;
}

NLS_API int nls_batch_set(nls_batch* b, int index, const void* pumping, const void* u0) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (index < 0 || index >= (int)b->m.size() || !pumping || !u0) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  CK(ctx, cudaSetDevice(ctx->device));
  Member& M = b->m[index];
  CK(ctx, cudaMemcpyAsync(M.P, pumping, M.N * rsize(b->dtype), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(M.u[M.parity], u0, M.N * csize(b->dtype), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_run(nls_batch* b, int64_t steps) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (steps < 0 || steps > INT_MAX) return fail(ctx, NLS_ERR_INVALID, "steps out of range");
  if (steps == 0) return NLS_OK;
  CK(ctx, cudaSetDevice(ctx->device));
  int st = batch_descriptors(b, steps);
  if (st) return st;
  auto it = b->graphs.find(steps);
  if (it == b->graphs.end() && b->graphs.size() >= 8) {
    // keep the cache small: a caller cycling through step counts re-captures instead of growing it
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
  }
  if (it == b->graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t eb = batch_sequence(b, steps);
    cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
    if (eb != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail_cuda(ctx, eb, "batch capture"); }
    CK(ctx, ee);
    cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(ctx, ei);
    it = b->graphs.emplace(steps, ge).first;
  }
  CK(ctx, cudaGraphLaunch(it->second, ctx->stream));
  ctx->launches += batch_launches(b, steps);
  for (auto& M : b->m)
    if (M.kind == 2) M.parity ^= (int)(steps & 1);
  return NLS_OK;
}

NLS_API int nls_batch_get(nls_batch* b, int index, void* u) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (index < 0 || index >= (int)b->m.size() || !u) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  CK(ctx, cudaSetDevice(ctx->device));
  const Member& M = b->m[index];
  CK(ctx, cudaMemcpyAsync(u, M.u[M.parity], M.N * csize(b->dtype), cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_set_many(nls_batch* b, int first, int count, const void* const* pumping,
                               const void* const* u0) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (first < 0 || count < 0 || first > (int)b->m.size() - count || (count && (!pumping || !u0)))
    return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  for (int k = 0; k < count; ++k)
    if (!pumping[k] || !u0[k]) return fail(ctx, NLS_ERR_INVALID, "null host buffer");
  CK(ctx, cudaSetDevice(ctx->device));
  for (int k = 0; k < count; ++k) {
    Member& M = b->m[first + k];
    CK(ctx, cudaMemcpyAsync(M.P, pumping[k], M.N * rsize(b->dtype), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(M.u[M.parity], u0[k], M.N * csize(b->dtype), cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_get_many(nls_batch* b, int first, int count, void* const* u) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (first < 0 || count < 0 || first > (int)b->m.size() - count || (count && !u))
    return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  for (int k = 0; k < count; ++k)
    if (!u[k]) return fail(ctx, NLS_ERR_INVALID, "null host buffer");
  CK(ctx, cudaSetDevice(ctx->device));
  for (int k = 0; k < count; ++k) {
    const Member& M = b->m[first + k];
    CK(ctx, cudaMemcpyAsync(u[k], M.u[M.parity], M.N * csize(b->dtype), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_layout(nls_batch* b, int64_t* pump_offsets, int64_t* state_offsets,
                             int64_t* pump_bytes, int64_t* state_bytes) {
  if (!b) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  for (size_t i = 0; i < b->m.size(); ++i) {
    if (pump_offsets) pump_offsets[i] = (int64_t)b->poff[i];
    if (state_offsets) state_offsets[i] = (int64_t)b->soff[i];
  }
  if (pump_bytes) *pump_bytes = (int64_t)b->pump_bytes;
  if (state_bytes) *state_bytes = (int64_t)b->state_bytes;
  return NLS_OK;
}

namespace {
// Merges copies whose source and destination both continue where the previous one ended: within
// one packed block that are consecutive instances, so a whole batch moves in a few large copies.
struct CopyRun {
  nls_ctx* ctx;
  cudaMemcpyKind kind;
  char* dst = nullptr;
  const char* src = nullptr;
  size_t bytes = 0;
  cudaError_t add(char* d, const char* s, size_t n) {
    if (bytes && d == dst + bytes && s == src + bytes) { bytes += n; return cudaSuccess; }
    cudaError_t e = flush();
    dst = d; src = s; bytes = n;
    return e;
  }
  cudaError_t flush() {
    cudaError_t e = bytes ? cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream) : cudaSuccess;
    bytes = 0;
    return e;
  }
};
}  // namespace

NLS_API int nls_batch_set_packed(nls_batch* b, const void* pumping, const void* u0) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (!pumping || !u0) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  CK(ctx, cudaSetDevice(ctx->device));
  if (b->pump_bytes) CK(ctx, cudaMemcpyAsync(b->mem, pumping, b->pump_bytes, cudaMemcpyHostToDevice, ctx->stream));
  CopyRun run{ctx, cudaMemcpyHostToDevice};
  for (size_t i = 0; i < b->m.size(); ++i) {
    const Member& M = b->m[i];
    CK(ctx, run.add(M.u[M.parity], static_cast<const char*>(u0) + b->soff[i], align256(M.N * csize(b->dtype))));
  }
  CK(ctx, run.flush());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_get_packed(nls_batch* b, void* u) {
  if (!b) return NLS_ERR_INVALID;
  nls_ctx* ctx = b->ctx;
  std::lock_guard<std::mutex> lk(b->mu);
  if (!u) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  CK(ctx, cudaSetDevice(ctx->device));
  CopyRun run{ctx, cudaMemcpyDeviceToHost};
  for (size_t i = 0; i < b->m.size(); ++i) {
    const Member& M = b->m[i];
    CK(ctx, run.add(static_cast<char*>(u) + b->soff[i], M.u[M.parity], align256(M.N * csize(b->dtype))));
  }
  CK(ctx, run.flush());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return NLS_OK;
}

NLS_API int nls_batch_state(nls_batch* b, int index, void** u_dev, const void** pumping_dev) {
  if (!b) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  if (index < 0 || index >= (int)b->m.size()) return fail(b->ctx, NLS_ERR_INVALID, "bad index");
  const Member& M = b->m[index];
  if (u_dev) *u_dev = M.u[M.parity];
  if (pumping_dev) *pumping_dev = M.P;
  return NLS_OK;
}

NLS_API int nls_batch_info(nls_batch* b, int64_t steps, int64_t* launches, int64_t* total_nodes) {
  if (!b) return NLS_ERR_INVALID;
  if (launches) *launches = batch_launches(b, steps);
  if (total_nodes) {
    int64_t t = 0;
    for (auto& M : b->m) t += (int64_t)M.N;
    *total_nodes = t;
  }
  return NLS_OK;
}

NLS_API int nls_batch_destroy(nls_batch* b) {
  if (!b) return NLS_ERR_INVALID;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  if (b->mem) cudaFree(b->mem);
  delete b;
  return NLS_OK;
}

// ---- pool

static void pool_release(nls_pool* p) {
  if (p->copy) cudaStreamSynchronize(p->copy);
  if (p->ctx->stream) cudaStreamSynchronize(p->ctx->stream);
  if (p->ctx->aux) cudaStreamSynchronize(p->ctx->aux);
  for (int b = 0; b < 2; ++b) {
    p->d_desc[b].release();
    if (p->ev_start[b]) cudaEventDestroy(p->ev_start[b]);
    if (p->ev_done[b]) cudaEventDestroy(p->ev_done[b]);
  }
  if (p->ev_upload) cudaEventDestroy(p->ev_upload);
  if (p->copy) cudaStreamDestroy(p->copy);
  p->arena.destroy();
  delete p;
}

NLS_API int nls_pool_create(nls_ctx* ctx, int dtype, size_t budget_bytes, int max_slots, int chunk_steps,
                            nls_pool** out) {
  if (!ctx) return NLS_ERR_INVALID;
  if (!out || max_slots <= 0 || chunk_steps <= 0 || budget_bytes < 4096)
    return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  if (dtype != NLS_C128 && dtype != NLS_C64) return fail(ctx, NLS_ERR_INVALID, "bad dtype");
  *out = nullptr;
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(ctx, cudaSetDevice(ctx->device));
  nls_pool* p = new nls_pool();
  p->ctx = ctx;
  p->dtype = dtype;
  p->chunk = chunk_steps;
  p->slots.resize(max_slots);
  cudaError_t e = p->arena.init(budget_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_upload, cudaEventDisableTiming);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaEventCreate(&p->ev_start[b]);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev_done[b]);
  }
  if (e != cudaSuccess) {
    pool_release(p);
    return fail_cuda(ctx, e, "pool set-up");
  }
  *out = p;
  return NLS_OK;
}

NLS_API int nls_pool_admit(nls_pool* p, const nls_problem* problem, const void* pumping, const void* u0,
                           int64_t steps, int64_t tag, int* slot) {
  if (!p) return NLS_ERR_INVALID;
  nls_ctx* ctx = p->ctx;
  std::lock_guard<std::mutex> lk(p->mu);
  if (!problem || !pumping || !u0 || steps < 0) return fail(ctx, NLS_ERR_INVALID, "bad arguments");
  int st = check_problem(ctx, p->dtype, problem);
  if (st) return st;
  Slot S;
  S.pr = *problem;
  if (S.pr.dim == 1) {
    if (host_stencil_1d(S.pr.n, S.pr.order, S.pr.dx, &S.op1)) return fail(ctx, NLS_ERR_INVALID, "1-D operator");
    S.K = S.op1.K;
    S.cl = choose_cl(p->dtype, S.pr.n, S.K, S.pr.variant > 0 ? S.pr.variant : -1);
    if (S.cl <= 0) return fail(ctx, NLS_ERR_INVALID, "1-D size not servable by the resident kernel");
    S.kind = 1;
    S.N = S.pr.n;
  } else {
    host_stencil_2d(S.pr.order, S.pr.dx, &S.op2);
    S.K = S.op2.K;
    S.shape = choose_shape(p->dtype, S.pr.n, S.K, S.pr.variant > 0 ? S.pr.variant : -1);
    if (S.shape <= 0) S.shape = TILE_32x32;
    if (!tile_supported(S.shape, p->dtype)) return fail(ctx, NLS_ERR_INVALID, "2-D shape not servable");
    S.kind = 2;
    S.N = (size_t)S.pr.n * S.pr.n;
    if (S.shape == TILE_STREAM) {
      S.tiles_x = 0;    // strip items are made per chunk over the pool's current mix
      S.ntiles = 0;
    } else {
      const int tx = tile_out_x(S.shape, S.K), ty = tile_out_y(S.shape, S.K);
      S.tiles_x = (S.pr.n + tx - 1) / tx;
      S.ntiles = S.tiles_x * ((S.pr.n + ty - 1) / ty);
    }
  }
  int free_slot = -1;
  for (size_t i = 0; i < p->slots.size(); ++i)
    if (!p->slots[i].used) { free_slot = (int)i; break; }
  if (free_slot < 0) return fail(ctx, NLS_ERR_BUSY, "no free slot");
  S.bytes = pool_bytes(p->dtype, S.pr);
  S.off = p->arena.alloc(S.bytes);
  if (S.off == SIZE_MAX) return fail(ctx, NLS_ERR_BUSY, "admission budget exhausted");
  CK(ctx, cudaSetDevice(ctx->device));
  const size_t cb = align256(S.N * csize(p->dtype));
  char* base = p->arena.at(S.off);
  S.u[0] = base;
  S.u[1] = S.kind == 2 ? base + cb : base;
  S.P = S.kind == 2 ? base + 2 * cb : base + cb;
  S.used = true;
  S.done = steps == 0;
  S.tag = tag;
  S.remaining = steps;
  S.parity = 0;
  if (S.done) S.finish_seq = ++p->seq;
  if (S.kind == 2 && S.shape != TILE_STREAM && tma_eligible(p->dtype, S.pr.n, S.u[0], S.u[1], S.P)) {
    std::vector<unsigned char> buf(tma_map_bytes() + 128);
    unsigned char* hm = (unsigned char*)(((uintptr_t)buf.data() + 127) & ~(uintptr_t)127);
    if (tma_encode_2d(S.shape, S.K, S.pr.n, S.u[0], S.u[1], S.P, hm) == 0) {
      S.tma = true;
      S.maps.assign(hm, hm + tma_map_bytes());
    }
  }
  // Upload on the pool's copy stream: the chunks running on the context's stream are not waited
  // for (the region is free memory that no chunk in flight touches); the next chunk waits for the
  // upload's event.  Copies from pageable memory return once the bytes are staged.
  cudaError_t e1 = cudaMemcpyAsync(S.P, pumping, S.N * rsize(p->dtype), cudaMemcpyHostToDevice, p->copy);
  cudaError_t e2 = cudaMemcpyAsync(S.u[0], u0, S.N * csize(p->dtype), cudaMemcpyHostToDevice, p->copy);
  cudaError_t e3 = cudaEventRecord(p->ev_upload, p->copy);
  if (e1 || e2 || e3) {
    p->arena.release(S.off, S.bytes);
    return fail_cuda(ctx, e1 ? e1 : (e2 ? e2 : e3), "pool upload");
  }
  p->upload_pending = true;
  p->slots[free_slot] = S;
  if (slot) *slot = free_slot;
  return NLS_OK;
}

// Enqueue the next chunk (every admitted request with steps not yet enqueued advances by up to
// `chunk` steps) if fewer than two chunks are in flight.  Called with p->mu held.
static int pool_launch_locked(nls_pool* p, int* launched) {
  nls_ctx* ctx = p->ctx;
  *launched = 0;
  if (p->inflight.size() >= 2) return NLS_OK;
  CK(ctx, cudaSetDevice(ctx->device));
  const int dtype = p->dtype;
  std::map<std::pair<int, int>, std::vector<int>> g1;
  std::map<std::tuple<int, int, int>, std::vector<int>> g2;   // (K, shape, tma)
  int64_t max_steps = 0;
  for (size_t i = 0; i < p->slots.size(); ++i) {
    const Slot& S = p->slots[i];
    if (!S.used || S.done || S.remaining <= 0) continue;
    if (S.kind == 1) g1[{S.K, S.cl}].push_back((int)i);
    else g2[std::make_tuple(S.K, S.shape, S.tma ? 1 : 0)].push_back((int)i);
    max_steps = std::max<int64_t>(max_steps, std::min<int64_t>(S.remaining, p->chunk));
  }
  if (g1.empty() && g2.empty()) return NLS_OK;
  const int buf = (int)(p->next_chunk & 1);
  // work items of each 2-D group: tiles, or strip items over the group's current mix
  std::vector<std::vector<StripItem>> sitems(g2.size());
  std::vector<std::vector<int2>> sranges(g2.size());
  std::vector<std::vector<int>> sdeps(g2.size());
  {
    size_t gi = 0;
    for (auto& kv : g2) {
      const int K = std::get<0>(kv.first), shape = std::get<1>(kv.first);
      if (shape == TILE_STREAM) {
        std::vector<int> ns;
        for (int i : kv.second) ns.push_back(p->slots[i].pr.n);
        const int ly = stream_plan_ly(ctx, ns, K);
        stream_list_items(ns, K, ly, stream_slots(ctx, K), sitems[gi]);
        stream_sort_items(sitems[gi]);
        stream_deps(sitems[gi], ns, K, sranges[gi], sdeps[gi]);
      }
      ++gi;
    }
  }
  // descriptor image: all groups back to back (a streaming group's item counter and flags are
  // part of the image and upload as zero)
  size_t bytes = 0;
  for (auto& kv : g1) bytes += align256(sizeof(Inst1D) * kv.second.size());
  {
    size_t gi = 0;
    for (auto& kv : g2) {
      if (std::get<1>(kv.first) == TILE_STREAM) {
        bytes += align256(sizeof(Inst2D) * kv.second.size()) +
                 stream_list_layout(0, sitems[gi].size(), sdeps[gi].size()).end;
      } else {
        int items = 0;
        for (int i : kv.second) items += p->slots[i].ntiles;
        bytes += align256(sizeof(Inst2D) * kv.second.size()) + align256(sizeof(TileItem) * items) +
                 align256(tma_map_bytes() * kv.second.size());
      }
      ++gi;
    }
  }
  p->h_desc.assign(bytes, 0);
  CK(ctx, p->d_desc[buf].ensure(bytes));
  char* d = (char*)p->d_desc[buf].p;
  struct L1 { int K, cl, seg, shortest, count; size_t off; };
  struct L2 { int K, shape, n_items, grid; size_t off, off_items; StreamListLayout ly; bool tma; int kinds; };
  std::vector<L1> l1;
  std::vector<L2> l2;
  size_t off = 0;
  for (auto& kv : g1) {
    Inst1D* h = (Inst1D*)(p->h_desc.data() + off);
    int seg = 0, shortest = INT32_MAX;
    for (size_t k = 0; k < kv.second.size(); ++k) {
      const Slot& S = p->slots[kv.second[k]];
      Inst1D& I = h[k];
      I.u = S.u[0]; I.P = S.P; I.n = S.pr.n; I.cl = S.cl;
      I.steps = std::min<int64_t>(S.remaining, p->chunk);
      I.dt = S.pr.dt; I.ph = phys_of(S.pr.coeffs); I.op = S.op1;
      set_params(I);
      seg = std::max(seg, (S.pr.n + S.cl - 1) / S.cl);
      shortest = std::min(shortest, shortest_segment(S.pr.n, S.cl));
    }
    l1.push_back(L1{kv.first.first, kv.first.second, seg, shortest, (int)kv.second.size(), off});
    off += align256(sizeof(Inst1D) * kv.second.size());
  }
  size_t gi = 0;
  for (auto& kv : g2) {
    const int K = std::get<0>(kv.first), shape = std::get<1>(kv.first);
    const bool tma = std::get<2>(kv.first) != 0;
    const bool stream = shape == TILE_STREAM;
    Inst2D* h = (Inst2D*)(p->h_desc.data() + off);
    const size_t ioff = off + align256(sizeof(Inst2D) * kv.second.size());
    int items = 0;
    if (stream) items = (int)sitems[gi].size();
    else for (int i : kv.second) items += p->slots[i].ntiles;
    const StreamListLayout ly = stream_list_layout(ioff, stream ? sitems[gi].size() : 0, stream ? sdeps[gi].size() : 0);
    const size_t moff = stream ? ly.end : ioff + align256(sizeof(TileItem) * items);
    TileItem* it = (TileItem*)(p->h_desc.data() + ioff);
    if (stream && items) {
      std::memcpy(p->h_desc.data() + ly.items, sitems[gi].data(), sizeof(StripItem) * items);
      std::memcpy(p->h_desc.data() + ly.range, sranges[gi].data(), sizeof(int2) * items);
      std::memcpy(p->h_desc.data() + ly.deps, sdeps[gi].data(), sizeof(int) * sdeps[gi].size());
    }
    int q_items = 0, kinds = 0;
    for (size_t k = 0; k < kv.second.size(); ++k) {
      const Slot& S = p->slots[kv.second[k]];
      if (stream) kinds |= stream_kind(S.pr.n, S.u[0], S.u[1], S.P);
      Inst2D& I = h[k];
      I.u[0] = S.u[0]; I.u[1] = S.u[1]; I.P = S.P; I.n = S.pr.n; I.tiles_x = S.tiles_x;
      I.parity = S.parity; I.steps = std::min<int64_t>(S.remaining, p->chunk);
      I.dt = S.pr.dt; I.ph = phys_of(S.pr.coeffs); I.op = S.op2;
      set_params(I);
      if (tma) {
        std::memcpy(p->h_desc.data() + moff + k * tma_map_bytes(), S.maps.data(), tma_map_bytes());
        I.tmap = d + moff + k * tma_map_bytes();
      }
      if (!stream)
        for (int q = 0; q < S.ntiles; ++q) it[q_items++] = TileItem{(int)k, q};
    }
    int grid;
    if (stream) {
      grid = stream_grid(ctx, K, std::max(1, items));
    } else {
      const int occ = tma ? fused_2d_tma_blocks_per_sm(K, shape) : fused_2d_blocks_per_sm(dtype, K, shape);
      grid = std::max(1, std::min(items, ctx->sm_count * std::max(1, occ)));
    }
    l2.push_back(L2{K, shape, items, grid, off, ioff, ly, tma, kinds});
    off = moff + (stream ? 0 : align256(tma_map_bytes() * kv.second.size()));
    ++gi;
  }
  // The previous user of this descriptor buffer is the chunk before the one in flight, already
  // complete; the upload is ordered on the context's stream after the chunk in flight.
  CK(ctx, cudaMemcpyAsync(d, p->h_desc.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
  if (p->upload_pending) {
    CK(ctx, cudaStreamWaitEvent(ctx->stream, p->ev_upload, 0));
    p->upload_pending = false;
  }
  CK(ctx, cudaEventRecord(p->ev_start[buf], ctx->stream));
  if (!l1.empty()) {
    CK(ctx, cudaEventRecord(ctx->ev_fork, ctx->stream));
    CK(ctx, cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0));
    for (auto& L : l1) {
      CK(ctx, launch_1d_resident(dtype, L.K, (const Inst1D*)(d + L.off), L.count, L.cl, L.seg, L.shortest, ctx->aux));
      ctx->launches += 1;
    }
  }
  auto stream_of = [&](const L2& L) {
    return StreamLaunch{(const Inst2D*)(d + L.off), (const StripItem*)(d + L.ly.items), L.n_items,
                        (unsigned*)(d + L.ly.counter), (const int2*)(d + L.ly.range), (const int*)(d + L.ly.deps),
                        (unsigned*)(d + L.ly.flags), ctx->wait_flag};
  };
  auto multi = [&](const L2& L) { return L.shape == TILE_STREAM && stream_multi_ok(ctx, L.K, L.kinds, L.n_items); };
  // streaming groups whose members all take the paired form: the whole chunk in one launch
  for (auto& L : l2)
    if (multi(L))
      for (int64_t j = 0; j < max_steps;) {
        const int s = (int)std::min<int64_t>(kStreamStepsPerLaunch, max_steps - j);
        CK(ctx, launch_2d_stream(L.K, L.kinds, stream_of(L), (int)j, s, L.grid, ctx->stream));
        ctx->launches += 1;
        j += s;
      }
  for (int64_t j = 0; j < max_steps; ++j)
    for (auto& L : l2) {
      if (multi(L)) continue;
      const Inst2D* dI = (const Inst2D*)(d + L.off);
      if (L.shape == TILE_STREAM) {
        CK(ctx, launch_2d_stream(L.K, L.kinds, stream_of(L), (int)j, 1, L.grid, ctx->stream));
      } else {
        const TileItem* dT = (const TileItem*)(d + L.off_items);
        CK(ctx, L.tma ? launch_2d_fused_tma(L.K, L.shape, dI, dT, L.n_items, (int)j, L.grid, ctx->stream,
                                            ctx->wait_flag)
                      : launch_2d_fused(dtype, L.K, L.shape, dI, dT, L.n_items, (int)j, L.grid, ctx->stream));
      }
      ctx->launches += 1;
    }
  if (!l1.empty()) {
    CK(ctx, cudaEventRecord(ctx->ev_join, ctx->aux));
    CK(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  }
  CK(ctx, cudaEventRecord(p->ev_done[buf], ctx->stream));
  const int64_t id = p->next_chunk++;
  for (auto& S : p->slots) {
    if (!S.used || S.done || S.remaining <= 0) continue;
    const int64_t st = std::min<int64_t>(S.remaining, p->chunk);
    S.remaining -= st;
    if (S.kind == 2) S.parity ^= (int)(st & 1);
    if (S.remaining == 0) S.finish_chunk = id;
  }
  p->inflight.push_back(PoolChunk{id, buf});
  *launched = 1;
  return NLS_OK;
}

NLS_API int nls_pool_launch(nls_pool* p, int* launched) {
  if (!p) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(p->mu);
  int l = 0;
  int st = pool_launch_locked(p, &l);
  if (launched) *launched = l;
  return st;
}

NLS_API int nls_pool_wait(nls_pool* p, int* finished) {
  if (!p) return NLS_ERR_INVALID;
  nls_ctx* ctx = p->ctx;
  std::unique_lock<std::mutex> lk(p->mu);
  if (finished) *finished = 0;
  if (p->inflight.empty()) return NLS_OK;
  if (p->waiting) return fail(ctx, NLS_ERR_BUSY, "another thread is waiting on this pool");
  const PoolChunk c = p->inflight.front();
  p->waiting = true;
  lk.unlock();           // admissions, takes and the next launch proceed while the chunk runs
  cudaError_t e = cudaEventSynchronize(p->ev_done[c.buf]);
  lk.lock();
  p->waiting = false;
  if (e != cudaSuccess) return fail_cuda(ctx, e, "waiting for a pool chunk");
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, p->ev_start[c.buf], p->ev_done[c.buf]) == cudaSuccess) p->busy_ms += ms;
  p->inflight.pop_front();
  int done = 0;
  for (auto& S : p->slots) {
    if (!S.used || S.done || S.finish_chunk != c.id) continue;
    S.done = true;
    S.finish_seq = ++p->seq;
    ++done;
  }
  if (finished) *finished = done;
  if (p->inflight.empty()) {
    int st = check_timeout(ctx);   // nothing in flight: reading the status word waits for nothing
    if (st) return st;
  }
  return NLS_OK;
}

NLS_API int nls_pool_ready(nls_pool* p, int* ready) {
  if (!p || !ready) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(p->mu);
  if (p->inflight.empty()) {
    *ready = 1;
    return NLS_OK;
  }
  const cudaError_t e = cudaEventQuery(p->ev_done[p->inflight.front().buf]);
  if (e == cudaErrorNotReady) {
    *ready = 0;
    return NLS_OK;
  }
  if (e != cudaSuccess) return fail_cuda(p->ctx, e, "querying a pool chunk");
  *ready = 1;
  return NLS_OK;
}

NLS_API int nls_pool_step(nls_pool* p, int* finished) {
  if (!p) return NLS_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    int l = 0;
    int st = pool_launch_locked(p, &l);
    if (st) return st;
  }
  return nls_pool_wait(p, finished);
}

NLS_API int nls_pool_take(nls_pool* p, int64_t* tag, void* u, size_t u_bytes) {
  if (!p) return NLS_ERR_INVALID;
  nls_ctx* ctx = p->ctx;
  std::lock_guard<std::mutex> lk(p->mu);
  int best = -1;
  for (size_t i = 0; i < p->slots.size(); ++i) {
    const Slot& S = p->slots[i];
    if (S.used && S.done && (best < 0 || S.finish_seq < p->slots[best].finish_seq)) best = (int)i;
  }
  if (best < 0) return NLS_ERR_NOT_READY;
  Slot& S = p->slots[best];
  const size_t need = S.N * csize(p->dtype);
  if (u) {
    if (u_bytes < need) return fail(ctx, NLS_ERR_INVALID, "output buffer too small");
    CK(ctx, cudaSetDevice(ctx->device));
    // the state is final (its last chunk completed); the copy stream does not wait for the
    // chunks still running on the context's stream
    CK(ctx, cudaMemcpyAsync(u, S.u[S.parity], need, cudaMemcpyDeviceToHost, p->copy));
    CK(ctx, cudaStreamSynchronize(p->copy));
  }
  if (tag) *tag = S.tag;
  p->arena.release(S.off, S.bytes);
  S = Slot();
  return NLS_OK;
}

NLS_API int nls_pool_status(nls_pool* p, int* active, size_t* bytes_in_use) {
  if (!p) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(p->mu);
  int a = 0;
  for (auto& S : p->slots) if (S.used && !S.done) ++a;
  if (active) *active = a;
  if (bytes_in_use) *bytes_in_use = p->arena.used();
  return NLS_OK;
}

NLS_API int nls_pool_info(nls_pool* p, int* in_flight, double* busy_ms) {
  if (!p) return NLS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(p->mu);
  if (in_flight) *in_flight = (int)p->inflight.size();
  if (busy_ms) *busy_ms = p->busy_ms;
  return NLS_OK;
}

NLS_API int nls_pool_destroy(nls_pool* p) {
  if (!p) return NLS_ERR_INVALID;
  cudaSetDevice(p->ctx->device);
  pool_release(p);
  return NLS_OK;
}
