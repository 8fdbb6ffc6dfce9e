// noalloc.cu -- an allocation-free entry point for the 2-D fused RK4 step.
//
// nls_solve_device() keeps a per-context scratch state buffer, descriptor and tile list that it
// obtains with cudaMalloc on first use.  Some callers cannot allow that: a service that reserves
// all of its device memory up front and must never grow it, a host framework whose own caching
// allocator owns the GPU's memory, or a latency-critical loop that cannot afford cudaMalloc /
// cudaFree, which may synchronise the whole device and stall unrelated streams.
// nls_solve_2d_noalloc() serves them: it runs a fused tile kernel of nls_solve_device (for
// complex64 by default the same register-resident tile, rk4_2d_reg; for complex128 the 32x32
// rk4_2d_fused tile, since the stage kernels nls_solve_device uses there need more scratch), but
// its scratch -- the second state buffer of the ping-pong, the instance descriptor and the tile
// list -- lives in one file-scope __device__ array of fixed size, so the call allocates nothing.
#include <cuda.h>

#include <cstring>
#include <mutex>

#include "../../include/nls_gb300.h"
#include "kernels.h"
#include "nls_types.h"

#define NLS_API extern "C" __attribute__((visibility("default")))

namespace nlsg {
int host_stencil_2d(int order, double h, Stencil2D* s);
}
using namespace nlsg;

namespace {

constexpr size_t kStateBytes = (size_t)NLS_NOALLOC_MAX_NODES * 16;  // complex128 worst case
constexpr size_t kDescBytes = 512;                                   // one Inst2D, padded
constexpr size_t kMaxTiles = 16384;                                  // >= tiles of any allowed grid
constexpr size_t kTileBytes = kMaxTiles * sizeof(TileItem);
constexpr size_t kScratchBytes = kStateBytes + kDescBytes + kTileBytes;

// Every GPU that loads the library holds this array until the process exits.  All calls share
// it and it keeps whatever the last call left there.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

static_assert(sizeof(Inst2D) <= kDescBytes, "descriptor slot too small");

// Writes the call's descriptor (passed by value as a kernel parameter) and its tile list
// {0, t} into the scratch array, so that no host memory is read after the call returns.
__global__ void noalloc_setup(Inst2D I, Inst2D* __restrict__ dI, TileItem* __restrict__ items, int n_items) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) *dI = I;
  if (t < n_items) items[t] = TileItem{0, t};
}

// The symbol address is resolved per CUDA context (the array is a module global, instantiated
// once in every context that loads the module), keyed by the current driver context.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

CtxGetCurrentFn ctx_get_current() {
  static std::once_flag once;
  static CtxGetCurrentFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

constexpr int kMaxContexts = 64;
std::mutex g_mu;
CUcontext g_ctx[kMaxContexts] = {};
void* g_addr[kMaxContexts] = {};

// Device address of the scratch array in the current context: resolved with cudaGetSymbolAddress
// the first time a context calls in (which also binds the device's primary context when no
// context is current), then taken from the cache.
cudaError_t scratch_address(char** out) {
  CtxGetCurrentFn get = ctx_get_current();
  if (!get) return cudaErrorNotSupported;
  CUcontext cur = nullptr;
  if (get(&cur) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  std::lock_guard<std::mutex> lk(g_mu);
  auto find = [&](CUcontext c) -> int {
    for (int i = 0; i < kMaxContexts; ++i)
      if (c && g_ctx[i] == c) return i;
    return -1;
  };
  int slot = find(cur);
  if (slot >= 0) {
    *out = (char*)g_addr[slot];
    return cudaSuccess;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  if (!p) return cudaErrorInvalidSymbol;
  if (!cur && (get(&cur) != CUDA_SUCCESS || !cur)) return cudaErrorDeviceUninitialized;
  slot = find(cur);
  for (int i = 0; i < kMaxContexts && slot < 0; ++i)
    if (!g_ctx[i]) slot = i;
  if (slot < 0) slot = (int)(reinterpret_cast<uintptr_t>(cur) % kMaxContexts);  // table full: replace one
  g_ctx[slot] = cur;
  g_addr[slot] = p;
  *out = (char*)p;
  return cudaSuccess;
}

}  // namespace

NLS_API int nls_solve_2d_noalloc(int dtype, const nls_problem* pr, int64_t iters, const void* pumping_dev,
                                 void* u_dev, void* stream) {
  if (!pr || !pumping_dev || !u_dev || iters < 0) return NLS_ERR_INVALID;
  if (dtype != NLS_C128 && dtype != NLS_C64) return NLS_ERR_INVALID;
  if (pr->dim != 2) return NLS_ERR_INVALID;
  if (pr->order != 3 && pr->order != 5) return NLS_ERR_ORDER;
  if (pr->n < pr->order || !(pr->dx > 0.0)) return NLS_ERR_INVALID;
  if ((int64_t)pr->n * pr->n > (int64_t)NLS_NOALLOC_MAX_NODES) return NLS_ERR_TOO_LARGE;
  Stencil2D op;
  if (host_stencil_2d(pr->order, pr->dx, &op)) return NLS_ERR_ORDER;
  // fused tile shape: -1 = the register-resident 64x96 tile (complex64) or the 32x32 tile
  // (complex128); otherwise a fused tile this precision supports (0, the unfused stage kernels,
  // needs three more state-sized buffers and is not offered here)
  int shape = dtype == NLS_C64 ? TILE_R64x96S : TILE_32x32;
  if (pr->variant >= 0) {
    if (pr->variant == 0 || !tile_supported(pr->variant, dtype)) return NLS_ERR_INVALID;
    shape = pr->variant;
  }
  const int n = pr->n;
  const int tx = tile_out_x(shape, op.K), ty = tile_out_y(shape, op.K);
  const int tiles_x = (n + tx - 1) / tx;
  const int n_items = tiles_x * ((n + ty - 1) / ty);
  if ((size_t)n_items > kMaxTiles) return NLS_ERR_TOO_LARGE;
  if (iters == 0) return NLS_OK;

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return NLS_ERR_CUDA;
  char* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return NLS_ERR_CUDA;
  void* state2 = base;
  Inst2D* dI = (Inst2D*)(base + kStateBytes);
  TileItem* dT = (TileItem*)(base + kStateBytes + kDescBytes);
  cudaStream_t st = (cudaStream_t)stream;

  Inst2D I;
  std::memset(&I, 0, sizeof(I));
  I.u[0] = u_dev;
  I.u[1] = state2;
  I.P = pumping_dev;
  I.n = n;
  I.tiles_x = tiles_x;
  I.parity = 0;
  I.steps = INT64_MAX;
  I.dt = pr->dt;
  I.ph.c3 = pr->coeffs[2]; I.ph.c4 = pr->coeffs[3]; I.ph.c5 = pr->coeffs[4]; I.ph.c6 = pr->coeffs[5];
  I.ph.c12 = pr->coeffs[11]; I.ph.c13 = pr->coeffs[12]; I.ph.c14 = pr->coeffs[13];
  I.op = op;
  set_params(I);
  noalloc_setup<<<(n_items + 255) / 256, 256, 0, st>>>(I, dI, dT, n_items);
  if (cudaGetLastError() != cudaSuccess) return NLS_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return NLS_ERR_CUDA;
  const int occ = fused_2d_blocks_per_sm(dtype, op.K, shape);
  const int grid = n_items < sms * (occ > 0 ? occ : 1) ? n_items : sms * (occ > 0 ? occ : 1);
  // The non-TMA form of the tile kernels: every thread loads its own nodes, so no launch of this
  // call waits on a copy barrier and none can time out.
  for (int64_t j = 0; j < iters; ++j) {
    if (launch_2d_fused(dtype, op.K, shape, dI, dT, n_items, (int)(j & 1), grid, st) != cudaSuccess)
      return NLS_ERR_CUDA;
  }
  // After an odd number of steps the state sits in the scratch buffer: bring it home.
  if (iters & 1) {
    const size_t bytes = (size_t)n * n * (dtype == NLS_C128 ? 16 : 8);
    if (cudaMemcpyAsync(u_dev, state2, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return NLS_ERR_CUDA;
  }
  return NLS_OK;
}
