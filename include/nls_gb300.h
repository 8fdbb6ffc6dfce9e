/* nls_gb300.h -- C ABI of the GB300 (sm_103a) solver for the nls time-stepping path.
 *
 * Drop-in boundary.  The reference exposes its native core as the f2py extension module
 * `nls.native` with the Fortran module object `nls` (setup.py:69-79, nls/makefile:49, imported as
 * `from .native import nls` in nls/solver.py:9).  Each entry point below names the reference
 * routine it replaces.  Plain pointers and sizes only; every function returns an int status
 * (NLS_OK = 0) and never aborts.  Host-buffer entry points follow the f2py call shape: inputs are
 * read, a new result is written to the caller's buffer, nothing is retained between calls.
 *
 * Arrays: complex values are interleaved (re, im) pairs (complex128 for NLS_C128, complex64 for
 * NLS_C64); real arrays (pump) are float64 or float32 to match.  2-D fields are n x n with the
 * first Fortran index contiguous, exactly the memory of the reference's Fortran (n, n) arrays.
 * The 23-slot coefficient vector is always float64 and indexed like the reference's coeffs(1..23)
 * shifted to 0-based.
 */
#ifndef NLS_GB300_H
#define NLS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define NLS_OK 0
#define NLS_ERR_INVALID 1     /* bad argument: size, pointer, coefficient vector, dtype */
#define NLS_ERR_ORDER 2       /* unsupported stencil order (1-D: 3, 5, 7; 2-D: 3, 5) */
#define NLS_ERR_CUDA 3        /* CUDA runtime error; nls_last_error() has the text */
#define NLS_ERR_NONFINITE 4   /* NaN or Inf found in a result by the FP64 diagnostics */
#define NLS_ERR_TIMEOUT 5     /* a bounded wait expired */
#define NLS_ERR_NOMEM 6       /* device memory exhausted */
#define NLS_ERR_BUSY 7        /* serving pool: no slot or admission budget for this request now */
#define NLS_ERR_NOT_READY 8   /* serving pool: nothing finished yet */
#define NLS_ERR_TOO_LARGE 9   /* nls_solve_2d_noalloc: grid beyond NLS_NOALLOC_MAX_NODES */

/* ---- precisions -------------------------------------------------------------------------- */
#define NLS_C128 0            /* complex128 state, float64 pump: the plain (drop-in) path */
#define NLS_C64 1             /* complex64 state, float32 pump: the precision form */

typedef struct nls_ctx nls_ctx;
typedef struct nls_batch nls_batch;
typedef struct nls_pool nls_pool;

/* One solve: dim 1 is the radial 1-D model of solve_nls (nls/nls.f90:797-813), dim 2 the
 * Cartesian model of solve_nls_2d (nls/nls.f90:903-919).  variant selects a kernel shape chosen by
 * the autotuner (-1 = built-in choice): 1-D = CTAs per solve (cluster size 1..16; complex64 runs
 * the register-resident kernel on 1 CTA and its cluster form on 2..8 CTAs whenever each segment
 * holds at least 4K nodes; 0 = unfused stage kernels); 2-D = 0 unfused, or a fused tile region (threads): 1 = 64x64 (512),
 * 2 = 128x32 (512), 3 = 32x32 (256), 4 = 64x64 (1024), 5 = 128x32 (1024),
 * 6 = 64 x (64 + 8K) with output tiles exactly 64 rows high (512), 7 = the same region with 768
 * (order 3) or 640 (order 5) threads; register-resident tiles (complex64 only), region 64 wide:
 * 8 = 64x80 (512), 9 = 64x96 (384), 10 = 64x96 (256), 11 = 64x64 (512), 12 = 64x72 (256),
 * 13 = 64x72 (384), 14 = 64x80 (256); 15 = streaming wavefront over 64-column strips (complex64
 * only; the complex64 default except order 5 below 2048 per side; order-3 work lists of at least
 * 1.5 strip items per resident warp run up to 512 RK4 steps per launch). */
typedef struct nls_problem {
  int dim;
  int n;
  int order;
  int variant;
  double dt;
  double dx;
  double coeffs[23];
} nls_problem;

/* version(major, minor, patch) -- nls/nls.f90:29-37 (reports the reference's 0.2.0). */
int nls_version(int* major, int* minor, int* patch);

/* make_laplacian(n, m, h, op) -- nls/nls.f90:278-295.  op: (order, n) column-major band storage,
 * float64.  Host only; needs no GPU. */
int nls_make_laplacian(int n, int order, double h, double* op);

/* make_laplacian_2d(n, m, h, blocks, orders) -- nls/nls.f90:388-403 (orders 3 and 5; the
 * reference's order-7 block array is mis-dimensioned, nls/nls.f90:360).  blocks: (n, 2*order-1)
 * column-major float64; orders: int[order].  Host only. */
int nls_make_laplacian_2d(int n, int order, double h, double* blocks, int* orders);

/* ---- context ----------------------------------------------------------------------------- */
int nls_ctx_create(int device, nls_ctx** out);
int nls_ctx_destroy(nls_ctx* ctx);
/* The context's own (non-blocking) cudaStream_t: every launch and copy of this context is
 * ordered on it, so callers record events on it and order their own work after it. */
int nls_ctx_stream(nls_ctx* ctx, void** stream);
int nls_ctx_synchronize(nls_ctx* ctx);
/* Text of the last failure on this context (empty string if none); valid until the next call. */
const char* nls_last_error(nls_ctx* ctx);
/* Number of kernel launches this context has issued (graph replays count every node). */
int64_t nls_ctx_launch_count(nls_ctx* ctx);

/* ---- single solves ----------------------------------------------------------------------- */
/* u = solve_nls(dt, dx, order, iters, pumping, coeffs, u0, [n]) -- nls/nls.f90:797-813, also
 * solve_nls_1d (:815-827).  Host buffers; blocks until u is written. */
int nls_solve_1d(nls_ctx* ctx, int dtype, double dt, double dx, int n, int order, int iters,
                 const double* coeffs23, const void* pumping, const void* u0, void* u);

/* u = solve_nls_2d(dt, dx, order, iters, pumping, coeffs, u0, [n]) -- nls/nls.f90:903-919. */
int nls_solve_2d(nls_ctx* ctx, int dtype, double dt, double dx, int n, int order, int iters,
                 const double* coeffs23, const void* pumping, const void* u0, void* u);

/* Device-resident form of both: advances the state u_dev in place by iters RK4 steps on the
 * context's stream (no host synchronisation).  pumping_dev and u_dev are device pointers.
 * Replaces the same routines; used for resume (repeated solve(k) from the last state). */
int nls_solve_device(nls_ctx* ctx, int dtype, const nls_problem* problem, int64_t iters,
                     const void* pumping_dev, void* u_dev);

/* mu = chemical_potential_1d(dx, pumping, coeffs, u0, [n]) -- nls/nls.f90:921-948 (complex). */
int nls_chemical_potential_1d(nls_ctx* ctx, int dtype, double dx, int n, const double* coeffs23,
                              const void* pumping, const void* u0, double* mu_re, double* mu_im);

/* mu = chemical_potential_2d(dx, pumping, coeffs, u0, [n]) -- nls/nls.f90:950-971 (real part). */
int nls_chemical_potential_2d(nls_ctx* ctx, int dtype, double dx, int n, const double* coeffs23,
                              const void* pumping, const void* u0, double* mu);

/* ---- FP64 device diagnostics (no reference counterpart: the reference has none) ----------- */
/* Chemical potential of a device-resident state, as chemical_potential_1d/2d (nls/nls.f90:921-971,
 * order-5 operator, radial weight in 1-D) but on device pointers and in FP64: mu = mu_re + i mu_im
 * (the 2-D reference returns mu_re only).  problem supplies dim, n, dx and coeffs.  Blocks. */
int nls_chemical_potential_device(nls_ctx* ctx, int dtype, const nls_problem* problem,
                                  const void* pumping_dev, const void* u_dev, double* mu_re,
                                  double* mu_im);
/* Damping integral of a device state, as Solution.getDampingIntegral (nls/model.py:350-365): the
 * rectangle rule of (n_res - 1) |u|^2 with the reservoir n_res = c12 P / (c13 + c14 |u|^2), weighted
 * by 2 pi r dx on r = linspace(0, n dx, n) in 1-D and by dx^2 in 2-D; FP64.  problem supplies dim,
 * n, dx and coeffs; pumping_dev has the state's precision.  Blocks until done. */
int nls_damping_integral_device(nls_ctx* ctx, int dtype, const nls_problem* problem,
                                const void* pumping_dev, const void* u_dev, double* integral);
/* sum |u|^2 over count nodes and the number of non-finite components; blocks until done. */
int nls_norm_device(nls_ctx* ctx, int dtype, int64_t count, const void* u_dev, double* sum_sq,
                    int64_t* nonfinite);
/* Relative L2 errors of the density |u|^2 and of the reservoir n = c12 P / (c13 + c14 |u|^2)
 * (nls/model.py:376-380) of u_dev against a complex128 reference state; pumping_f64_dev is the
 * float64 pump.  Blocks until done. */
int nls_density_error_device(nls_ctx* ctx, int dtype, int64_t count, const void* u_dev,
                             const void* u_ref_c128_dev, const double* pumping_f64_dev, double c12,
                             double c13, double c14, double* rel_l2_density,
                             double* rel_l2_reservoir);

/* ---- batched form: many independent solves, one graph-captured launch sequence ------------ */
/* Replaces running Model.solve() once per configuration (the reference's benchmark and job farm,
 * benchmark/benchmark.py:21-76, schedulr/workr.py:39-66) with one resident batch on the GPU. */
int nls_batch_create(nls_ctx* ctx, int dtype, int count, const nls_problem* problems,
                     nls_batch** out);
/* Upload instance index's pump and initial state from host buffers (sizes from its problem). */
int nls_batch_set(nls_batch* batch, int index, const void* pumping, const void* u0);
/* Advance every instance by steps RK4 steps (a CUDA graph, replayed from cache). Asynchronous. */
int nls_batch_run(nls_batch* batch, int64_t steps);
/* Copy instance index's current state to a host buffer; blocks until written. */
int nls_batch_get(nls_batch* batch, int index, void* u);
/* The same for count instances first .. first+count-1 (pumping[k], u0[k] / u[k] belong to
 * instance first+k): every copy is queued on the context's stream and the call synchronizes once,
 * instead of once per instance.  Pinned host buffers make the copies asynchronous DMA. */
int nls_batch_set_many(nls_batch* batch, int first, int count, const void* const* pumping,
                       const void* const* u0);
int nls_batch_get_many(nls_batch* batch, int first, int count, void* const* u);
/* Packed host layout of a batch: every pump in one block and every state in another, instance
 * k's at byte offset pump_offsets[k] / state_offsets[k] (instance order, each padded to 256
 * bytes; the arrays hold count entries, any output may be NULL), the blocks pump_bytes and
 * state_bytes long.  The batch keeps its device fields in the same layout, so set_packed and
 * get_packed move the whole batch in a few large copies, one wait each. */
int nls_batch_layout(nls_batch* batch, int64_t* pump_offsets, int64_t* state_offsets,
                     int64_t* pump_bytes, int64_t* state_bytes);
int nls_batch_set_packed(nls_batch* batch, const void* pumping, const void* u0);
int nls_batch_get_packed(nls_batch* batch, void* u);
/* Device pointers of instance index's current state and pump (valid until the next run). */
int nls_batch_state(nls_batch* batch, int index, void** u_dev, const void** pumping_dev);
/* Kernel launches one run(steps) issues, and nodes summed over instances. */
int nls_batch_info(nls_batch* batch, int64_t steps, int64_t* launches, int64_t* total_nodes);
int nls_batch_destroy(nls_batch* batch);

/* ---- serving pool: continuous batching under an HBM budget -------------------------------- */
/* Replaces schedulr's pull queue of independent solves (schedulr/schedulr.py:48-154,
 * schedulr/workr.py:88-102) with in-process admission into a resident, continuously batched
 * set of solves.  budget_bytes bounds the device memory of admitted states and pumps. */
int nls_pool_create(nls_ctx* ctx, int dtype, size_t budget_bytes, int max_slots, int chunk_steps,
                    nls_pool** out);
/* Admit one request.  Its pump and initial state are uploaded from the host buffers on the pool's
 * own copy stream (the buffers may be reused when the call returns); no chunk in flight is waited
 * for, and the next chunk waits for the upload.  NLS_ERR_BUSY if no slot or budget is free now;
 * the caller keeps it queued and retries after a chunk completes. */
int nls_pool_admit(nls_pool* pool, const nls_problem* problem, const void* pumping,
                   const void* u0, int64_t steps, int64_t tag, int* slot);
/* Pipelined operation (no reference counterpart: schedulr's workers run one solve at a time).
 * nls_pool_launch enqueues the next chunk -- every admitted request with steps not yet enqueued
 * advances by up to chunk_steps RK4 steps, each stopping at its own count -- on the context's
 * stream and returns at once (*launched = 1), or does nothing (*launched = 0) when two chunks are
 * already in flight or no request has steps left to enqueue.  nls_pool_wait blocks until the
 * oldest chunk in flight completes (the pool's lock is released meanwhile, so admissions and
 * takes proceed) and reports the requests it finished; with no chunk in flight it returns at
 * once.  nls_pool_ready tells whether the oldest chunk in flight has completed (1 when none is in
 * flight).  Requests finished by a completed chunk are taken while the next chunk runs. */
int nls_pool_launch(nls_pool* pool, int* launched);
int nls_pool_wait(nls_pool* pool, int* finished);
int nls_pool_ready(nls_pool* pool, int* ready);
/* Launch (if fewer than two chunks are in flight) and wait for the oldest chunk:
 * *finished = requests that completed in it. */
int nls_pool_step(nls_pool* pool, int* finished);
/* Take one finished request: its tag and final state (host buffer of its size), copied on the
 * pool's copy stream without waiting for chunks in flight; frees its slot and budget.
 * NLS_ERR_NOT_READY if none is finished. */
int nls_pool_take(nls_pool* pool, int64_t* tag, void* u, size_t u_bytes);
/* Admitted-but-unfinished requests, bytes of budget in use. */
int nls_pool_status(nls_pool* pool, int* active, size_t* bytes_in_use);
/* Chunks in flight and the device time of every completed chunk so far (ms, CUDA events on the
 * context's stream): the pool's GPU-busy time. */
int nls_pool_info(nls_pool* pool, int* in_flight, double* busy_ms);
int nls_pool_destroy(nls_pool* pool);

/* ---- allocation-free 2-D solve ------------------------------------------------------------ */
/* No counterpart in the reference: the reference allocates its work arrays on every call.
 *
 * For callers that must not allocate device memory: services that reserve their whole device
 * budget at start-up and may never grow it, host frameworks whose own caching allocator owns the
 * GPU's memory, and latency-critical loops that cannot pay for cudaMalloc / cudaFree, which can
 * synchronise the device and stall unrelated streams.  The call advances u_dev (n x n, in place)
 * by iters RK4 steps of the 2-D model with a fused tile kernel of nls_solve_device, on the
 * caller's stream (NULL = the legacy default stream), with no cudaMalloc, cudaFree or other
 * allocating call: its scratch (the second state buffer, the descriptor and the tile list) is a
 * fixed file-scope device array of about 4 MiB, which every GPU that loads this library holds
 * until the process exits.  variant: -1 = the register-resident 64x96 tile (complex64) or the
 * 32x32 tile (complex128); otherwise a fused tile variant of nls_problem that the precision
 * supports (variant 0, the unfused stage kernels, and unsupported variants: NLS_ERR_INVALID).
 * The tile kernels run in their plain-load form, which has no copy barrier and so no bounded
 * wait that could expire.  The descriptor and tile list are written into the array by a kernel
 * on the caller's stream; no host memory is read after the call returns.  Limits: dim must be 2
 * and n * n <= NLS_NOALLOC_MAX_NODES (512 x 512), otherwise NLS_ERR_TOO_LARGE.  The first call
 * in a CUDA context resolves the array's device address in that context (cudaGetSymbolAddress,
 * with that context's device current) and caches it per context; make that first call before
 * any stream capture.  Every call shares the one array and it keeps the last call's contents
 * (nothing in it needs to start at zero: the first step overwrites every node it later reads),
 * so calls that overlap on the GPU -- on different streams or threads -- race; serialise them.
 * Returns after enqueueing the work (no host synchronisation). */
#define NLS_NOALLOC_MAX_NODES 262144
int nls_solve_2d_noalloc(int dtype, const nls_problem* problem, int64_t iters,
                         const void* pumping_dev, void* u_dev, void* stream);

/* ---- testing ----------------------------------------------------------------------------- */

/* No counterpart in the reference.  Test control of the failure path of the bounded tile waits:
 * with extra_bytes > 0 every complex64 register-tile launch on `device` (variants 8-14 on grids
 * taking the TMA path) arms its tile barrier for extra_bytes more than its copies deliver, so the
 * barrier never completes, each CTA gives up after its bounded wait (about a second), and the
 * solve returns NLS_ERR_TIMEOUT; 0 restores normal operation.  No fault is raised and the
 * context stays usable.  Not for production use. */
int nls_test_set_tile_tx_extra(int device, unsigned extra_bytes);

/* No counterpart in the reference.  Test control of the failure path of the bounded dependency
 * waits of the streaming 2-D kernel (variant 15) when one launch runs several steps: with
 * extra_steps > 0 every such wait on `device` asks for extra_steps more published steps than
 * will ever exist, so the first waiting warp gives up after its bounded wait (about a second),
 * sets the context's status word, the other warps stop waiting, and the synchronising call
 * returns NLS_ERR_TIMEOUT; 0 restores normal operation.  No fault is raised and the context
 * stays usable.  Not for production use. */
int nls_test_set_stream_dep_extra(int device, unsigned extra_steps);

/* No counterpart in the reference.  Test control of the streaming 2-D kernel's launch schedule
 * for lists set up after the call (single solves, batches, pool chunks): 0 = automatic (several
 * RK4 steps per launch for order-3 lists of at least 1.5 items per resident warp whose grids all
 * take the paired form), 1 = several steps per launch whenever the grids all take the paired form,
 * 2 = one step per launch.  Results are identical either way.  Process-wide; not for production
 * use. */
int nls_test_set_stream_steps_per_launch(int mode);

#ifdef __cplusplus
}
#endif

#endif /* NLS_GB300_H */
