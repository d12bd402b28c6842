/*
 * pasif_gb300.h -- C ABI of the GB300 (sm_103a) engine for PASIf's hot path:
 * batched fixed-step RK4 integration of polynomial first-order systems driven
 * by sampled excitations, and its adjoint.
 *
 * Two layers:
 *   1. pasif_driver_*  -- the drop-in for the reference's pybind11 class
 *      __GpuDriver (src/PASIfgpu.cpp:22-105, src/__GpuDriver.cuh:18-83):
 *      same setters, same getters, same argument meaning.  Each entry point
 *      names the reference method it replaces.
 *   2. pasif_plan_* / pasif_signals_* / pasif_batch_* / pasif_forward --
 *      the native batch interface: many instances sharing one sparsity
 *      pattern, per-instance values, per-instance excitation index.
 *
 * Conventions: every function returns PASIF_OK (0) or an error code and sets
 * a thread-local message (pasif_last_error).  Arrays are plain pointers with
 * explicit sizes, double precision on the interface; the compute precision is
 * a per-plan / per-driver setting.  Unlike the reference, a CUDA failure is
 * reported as a status (the reference prints and calls exit(0),
 * src/helpers.cuh:43-51).  Objects are not thread-safe; use one per thread.
 */
#ifndef PASIF_GB300_H
#define PASIF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PASIF_OK 0
#define PASIF_ERR_INVALID 1     /* bad argument or inconsistent sizes      */
#define PASIF_ERR_CUDA 2        /* CUDA runtime / kernel launch failure    */
#define PASIF_ERR_NVRTC 3       /* specialised kernel could not be built   */
#define PASIF_ERR_MEMORY 4      /* device allocation failed                */
#define PASIF_ERR_STATE 5       /* call order (e.g. solve before set-up)   */
#define PASIF_ERR_LENGTH 6      /* excitation signals of unequal length    */

#define PASIF_FP64 0            /* reference precision (reel = double)     */
#define PASIF_FP32 1            /* reel = float                            */
#define PASIF_FP32_KAHAN 2      /* FP32 stages, compensated state update   */
#define PASIF_FP32_EXT 3        /* FP32 stages; state (and adjoint state)
                                   as double-float pairs; the FP64 values'
                                   FP32 residuals and the exact h/6 applied
                                   once per step: long-horizon precision
                                   mode (pattern-specialised kernels only;
                                   not for serving pools)                  */

#define PASIF_HOST 0            /* pointers are host memory                */
#define PASIF_DEVICE 1          /* pointers are device memory (current GPU) */

#define PASIF_KERNEL_NONE 0
#define PASIF_KERNEL_GENERIC 1      /* pattern-interpreting kernel          */
#define PASIF_KERNEL_SPECIALISED 2  /* NVRTC kernel specialised to pattern  */

#define PASIF_PLAN_GENERIC_ONLY 1   /* plan flag: never specialise          */
#define PASIF_PLAN_NO_LITERALS 2    /* plan flag: specialise to the pattern
                                       only, load every value (one compiled
                                       kernel serves all batches of a plan) */
#define PASIF_PLAN_WARP_SLICED 4    /* plan flag: warp-sliced kernels at any
                                       size (default: from n >= 28 in FP32,
                                       n >= 24 in FP64)                     */
#define PASIF_PLAN_NO_WARP_SLICED 8 /* plan flag: thread per system always  */
#define PASIF_PLAN_FAST 16          /* plan flag: fast thread-per-system
                                       forward kernels (products of the state
                                       shared between terms, the RK sum and
                                       the compensation folded into fmas):
                                       not the oracle's bit-exact operation
                                       order; accuracy as checked against
                                       FP64.  No reference counterpart      */

/* Message of the last failing call on this thread ("" if none). */
const char* pasif_last_error(void);
/* ABI version: major*10000 + minor*100 + patch. */
int pasif_version(void);
/* Number of CUDA devices visible (0 without a driver); never fails. */
int pasif_device_count(void);

/* ======================================================================
 * Layer 1: drop-in __GpuDriver
 * ====================================================================== */
typedef struct pasif_driver pasif_driver;

/* __GpuDriver::__GpuDriver (src/__GpuDriver.cu:25-157, src/PASIfgpu.cpp:26-33).
 * signals[i] points to lengths[i] samples.  Unequal lengths are accepted
 * here and reported by the first solve, as the reference's constructor
 * ignores _loadExcitationsSet's status. */
int pasif_driver_create(pasif_driver** out, const double* const* signals, const long long* lengths,
                        int n_signals, unsigned sample_rate, unsigned numsteps, int d_compute,
                        int d_system, int d_solver, unsigned gpu_id);
/* __GpuDriver::~__GpuDriver (src/__GpuDriver.cu:159-193). */
int pasif_driver_destroy(pasif_driver* d);
/* Compute precision of the solves (PASIF_FP64 default = reel double,
 * src/helpers.cuh:29).  No reference counterpart: the reference fixes it at
 * compile time. */
int pasif_driver_set_precision(pasif_driver* d, int precision);

/* __GpuDriver::_setFwdK / _setBwdK (src/__GpuDriver.cu:199-209, 272-282):
 * CSR of -M^-1 (B+K), shape rows x cols, nnz = indptr[rows]. */
int pasif_driver_set_fwd_k(pasif_driver* d, unsigned rows, unsigned cols, const double* values,
                           const unsigned* indices, const unsigned* indptr, long long nnz);
int pasif_driver_set_bwd_k(pasif_driver* d, unsigned rows, unsigned cols, const double* values,
                           const unsigned* indices, const unsigned* indptr, long long nnz);
/* _setFwdGamma / _setBwdGamma (src/__GpuDriver.cu:211-219, 284-292): 3-D COO,
 * indices[3e..3e+2] = (dest, source, setpoint), src/helpers.cu:277-282. */
int pasif_driver_set_fwd_gamma(pasif_driver* d, const unsigned dims[3], const double* values,
                               const unsigned* indices, long long nnz);
int pasif_driver_set_bwd_gamma(pasif_driver* d, const unsigned dims[3], const double* values,
                               const unsigned* indices, long long nnz);
/* _setFwdLambda / _setBwdLambda (src/__GpuDriver.cu:221-229, 294-302): 4-D COO,
 * (dest, source, setpoint, setpoint), src/helpers.cu:400-406. */
int pasif_driver_set_fwd_lambda(pasif_driver* d, const unsigned dims[4], const double* values,
                                const unsigned* indices, long long nnz);
int pasif_driver_set_bwd_lambda(pasif_driver* d, const unsigned dims[4], const double* values,
                                const unsigned* indices, long long nnz);
/* _setFwdPsi / _setBwdPsi (src/__GpuDriver.cu:231-240, 304-312): 5-D COO. */
int pasif_driver_set_fwd_psi(pasif_driver* d, const unsigned dims[5], const double* values,
                             const unsigned* indices, long long nnz);
int pasif_driver_set_bwd_psi(pasif_driver* d, const unsigned dims[5], const double* values,
                             const unsigned* indices, long long nnz);
/* _setFwdForcePattern / _setBwdForcePattern (src/__GpuDriver.cu:242-246, 314-318):
 * dense pattern; entries with |v| <= DBL_EPSILON are dropped
 * (COOVector, src/helpers.cu:664-682). */
int pasif_driver_set_fwd_force_pattern(pasif_driver* d, const double* pattern, long long n);
int pasif_driver_set_bwd_force_pattern(pasif_driver* d, const double* pattern, long long n);
/* _setFwdInitialConditions / _setBwdInitialConditions (src/__GpuDriver.cu:248-254, 320-326):
 * sets the number of state variables. */
int pasif_driver_set_fwd_initial_conditions(pasif_driver* d, const double* ic, long long n);
int pasif_driver_set_bwd_initial_conditions(pasif_driver* d, const double* ic, long long n);
/* _allocateSystemOnDevice (src/__GpuDriver.cu:256-265): checks sizes,
 * splits the concatenated system into independent blocks, groups blocks of
 * identical pattern and uploads them. */
int pasif_driver_allocate_system(pasif_driver* d);
/* _allocateAdjointOnDevice (src/__GpuDriver.cu:328-337). */
int pasif_driver_allocate_adjoint(pasif_driver* d);

/* _loadExcitationsSet (src/__GpuDriver.cu:343-381): returns PASIF_OK, or
 * PASIF_ERR_LENGTH when the signals differ in length (the reference returns 1). */
int pasif_driver_load_excitations(pasif_driver* d, const double* const* signals, const long long* lengths,
                                  int n_signals, unsigned sample_rate);
/* _setInterpolationMatrix (src/__GpuDriver.cu:383-398): flat matrix of
 * `size` values, rows of `window` weights; only rows 0 and 1 are read
 * (src/kernels.cu:123).  window must be a power of two (the reference's
 * kernel masks with window-1 and silently misbehaves otherwise). */
int pasif_driver_set_interpolation_matrix(pasif_driver* d, const double* matrix, long long size,
                                          unsigned window);
/* _setModulationBuffer (src/__GpuDriver.cu:400-410): stored, never read by
 * any solve (as in the reference). */
int pasif_driver_set_modulation_buffer(pasif_driver* d, const double* buffer, long long n);

/* _getAmplitudes (src/__GpuDriver.cu:416-461): final state of every
 * excitation copy, out[e * n + i].  For the three getters, out == NULL only
 * sets *out_len (nothing is solved); otherwise capacity must hold it. */
int pasif_driver_get_amplitudes(pasif_driver* d, double* out, long long capacity, long long* out_len);
/* _getTrajectory (src/__GpuDriver.cu:463-500): the state after every step t
 * with t % save_steps == 0, laid out [slot][e][i], truncated to
 * floor(n * n_exc * numsteps / save_steps) values like the reference's
 * host vector. */
int pasif_driver_get_trajectory(pasif_driver* d, unsigned save_steps, double* out, long long capacity,
                                long long* out_len);
/* _getGradient (src/__GpuDriver.cu:502-587): final adjoint vector of every
 * excitation copy, out[e * n_adj + i]; afterwards the adjoint initial
 * condition holds that vector (the reference chains it, :743). */
int pasif_driver_get_gradient(pasif_driver* d, unsigned save, double* out, long long capacity,
                              long long* out_len);
/* Kernel used by the last forward solve (PASIF_KERNEL_*). */
int pasif_driver_last_kernel(pasif_driver* d, int* kind);
/* Memory-bounded sweeps: the reference splits its excitation copies into
 * sequential chunks that fit the free device memory
 * (numberOfSimulationToPerform, src/__GpuDriver.cu:420-449, 896-938; its
 * chunks read the wrong excitation offset).  Here every instance (block x
 * signal) keeps its own signal, and a solve whose instances need more device
 * memory than the budget runs as sequential batches of as many instances as
 * fit.  bytes = 0 (default): 90 % of the memory free when the solve starts.
 * A solve in which not even one instance fits returns PASIF_ERR_MEMORY. */
int pasif_driver_set_memory_budget(pasif_driver* d, long long bytes);
/* Sequential batches the last solve of this driver ran (1: all at once). */
int pasif_driver_last_chunks(pasif_driver* d, int* chunks);
/* The split rule itself: instances per sequential batch for n_instances of
 * bytes_per_instance within budget (all when they fit; 0 when none fits). */
int pasif_sweep_chunk(long long n_instances, long long bytes_per_instance, long long budget, long long* per_batch);

/* ======================================================================
 * Layer 2: native batches
 * ====================================================================== */

/* One system pattern.  dQ/dt = K.Q + Gamma:(Q,Qp) + Lambda:(Q,Qp,Qp)
 * + Psi:(Q,Qp,Qp,Qp) + F u(t), index roles as in src/kernels.cu:52,56,61.
 * Instance values: [K (CSR order) | Gamma | Lambda | Psi | F] = P values. */
typedef struct pasif_pattern {
    int n;                       /* state size                               */
    int n_sp;                    /* setpoint size (== n for forward systems) */
    int k_nnz; const int* k_ptr; const int* k_col;   /* CSR, n+1 / k_nnz     */
    int g_nnz; const int* g_idx;                     /* 3 per entry          */
    int l_nnz; const int* l_idx;                     /* 4 per entry          */
    int p_nnz; const int* p_idx;                     /* 5 per entry          */
    int f_nnz; const int* f_idx;                     /* force destinations   */
} pasif_pattern;

typedef struct pasif_reducers {
    int n_max; const int* max_comp; int max_start;   /* max |Q[c]| for steps >= max_start */
    int n_sq;  const int* sq_comp;  int sq_start;    /* h * sum Q[c]^2 for steps >= sq_start */
} pasif_reducers;

typedef struct pasif_plan pasif_plan;
typedef struct pasif_signals pasif_signals;
typedef struct pasif_batch pasif_batch;

/* Plan = pattern + precision (the pattern-specialised kernels are compiled
 * lazily, per batch, by the first solve).  flags: PASIF_PLAN_GENERIC_ONLY,
 * PASIF_PLAN_NO_LITERALS, PASIF_PLAN_WARP_SLICED, PASIF_PLAN_NO_WARP_SLICED. */
int pasif_plan_create(pasif_plan** out, const pasif_pattern* pattern, int precision, int flags);
int pasif_plan_destroy(pasif_plan* p);

/* Excitation table: n_exc signals of len samples (row-major), forcing by
 * sample and hold (window 0, src/kernels.cu:72-89) or window-W linear
 * weights im[2*window] (src/kernels.cu:97-126). memory: where x/im live. */
int pasif_signals_create(pasif_signals** out, const double* x, int n_exc, int len, int window,
                         const double* im, int precision, int memory, void* stream);
int pasif_signals_destroy(pasif_signals* s);
/* Replace the table (same window, weights and precision) in the existing
 * device buffers, grown only when too small: no device allocation, hence no
 * implicit device synchronisation, once they are large enough.  No reference
 * counterpart (serving workers reuse one table object). */
int pasif_signals_update(pasif_signals* s, const double* x, int n_exc, int len, int memory, void* stream);

int pasif_batch_create(pasif_batch** out, pasif_plan* plan, int n_sys);
int pasif_batch_destroy(pasif_batch* b);
/* New instance count for the next pasif_batch_set; device buffers are kept
 * and grown only when too small (a batch reused across requests). */
int pasif_batch_resize(pasif_batch* b, int n_sys);
/* Grow the batch's device buffers to what a forward or exact adjoint of
 * n_sys instances over nsteps steps needs, so later calls up to that size
 * allocate nothing (cudaMalloc/cudaFree synchronise the device). */
int pasif_batch_reserve(pasif_batch* b, int n_sys, int nsteps);
/* Device memory (bytes) the exact adjoint may hold for the whole forward
 * trajectory: (nsteps + 1) * n * n_sys FP32 states, or in FP64 every step's
 * state and three stage inputs, (4 nsteps + 1) * n * n_sys doubles.  Within
 * it the forward kernel writes the trajectory once and the backward sweep
 * reads it; above it the trajectory is recomputed chunk by chunk from
 * checkpoints every ceil(sqrt(nsteps)) steps (about one more forward pass).
 * Results are identical.  Default 16 GiB; 0 always recomputes.  Set it
 * before pasif_batch_reserve. */
int pasif_batch_set_adjoint_storage(pasif_batch* b, long long bytes);
/* values[n_sys][P], x0[n_sys][n], exc_index[n_sys]. */
int pasif_batch_set(pasif_batch* b, const double* values, const double* x0, const int* exc_index,
                    int memory, void* stream);
/* Kernel only: integrate nsteps from step index step0 (inputs resident). */
int pasif_batch_forward(pasif_batch* b, const pasif_signals* s, double h, int step0, int nsteps,
                        const pasif_reducers* red, void* stream);
/* state[n_sys][n], max[n_sys][n_max], sq[n_sys] (any may be NULL). */
int pasif_batch_get(pasif_batch* b, double* state, double* max, double* sq, int memory, void* stream);
/* Exact discrete adjoint of the RK4 map: loss = sum_c g_final[b][c] Q_N[c]
 * + g_sq[b] * (h sum_{s>=sq_start} sum_c Q_{s+1}[c]^2); outputs
 * d_values[n_sys][P] (FP64 accumulation) and d_x0[n_sys][n].  No reference
 * counterpart as such: the reference's adjoint is _getGradient. */
int pasif_batch_adjoint(pasif_batch* b, const pasif_signals* s, double h, int nsteps,
                        const pasif_reducers* red, const double* g_final, const double* g_sq,
                        double* d_values, double* d_x0, int memory, void* stream);
/* Kernel used by the last forward (PASIF_KERNEL_*), registers per thread. */
int pasif_batch_kernel_info(pasif_batch* b, int* kind, int* registers);

/* Compile (without loading; no GPU needed) the pattern-specialised forward
 * kernel that pasif_batch_forward would use for these host values, and copy
 * the compiler's resource report (registers, spills) into log, followed by
 * the generated source after a line "// ---- source ----".  The reducer
 * masks and the forcing window / weights (im[2*window]) select the variant.
 * Diagnostic; no reference counterpart. */
int pasif_plan_jit_report(const pasif_plan* p, const double* values, int n_sys,
                          unsigned long long max_mask, unsigned long long sq_mask,
                          int window, const double* im,
                          char* log, long long capacity, long long* out_len);

/* ======================================================================
 * Serving pools: continuous batching of forward requests (no reference
 * counterpart; the reference solves one configured system set per call).
 * A pool holds `capacity` slots of one pattern class (pattern, precision,
 * forcing window/weights, time step h, reducer components) and a signal
 * arena of `arena_samples` samples.  A request of n_sys systems takes n_sys
 * free slots; each pasif_pool_launch advances every busy slot by up to
 * `chunk` steps from its own step index (one CUDA-graph replay), so requests
 * join and leave between chunks while others run.  Every slot computes what
 * a one-request batch computes, bit for bit.
 * ====================================================================== */
typedef struct pasif_pool pasif_pool;
int pasif_pool_create(pasif_pool** out, const pasif_pattern* pattern, int precision, int window,
                      const double* im, double h, const pasif_reducers* red, int capacity,
                      long long arena_samples, int chunk, int flags);
int pasif_pool_destroy(pasif_pool* p);
/* Host arrays: values[n_sys][P], x0[n_sys][n], exc_index[n_sys],
 * signals[n_exc][len]; integrates nsteps from step 0.  PASIF_ERR_STATE when
 * slots or arena space are short (retry after a harvest); PASIF_ERR_INVALID
 * when the request can never fit (more systems than slots, a table larger
 * than the arena). */
int pasif_pool_admit(pasif_pool* p, int n_sys, const double* values, const double* x0,
                     const int* exc_index, const double* signals, int n_exc, int len, int nsteps,
                     int max_start, int sq_start, int* request_id);
/* One chunk for every busy slot (asynchronous, on the pool's own stream). */
int pasif_pool_launch(pasif_pool* p);
/* Waits for the pool's stream; lists requests whose slots have all finished. */
int pasif_pool_poll(pasif_pool* p, int* finished, int capacity, int* n_finished);
/* Results of a finished request (state[n_sys][n], max[n_sys][n_max],
 * sq[n_sys]; any may be NULL); frees its slots and arena space.
 * PASIF_ERR_STATE (nothing freed) while any of its slots has steps left. */
int pasif_pool_harvest(pasif_pool* p, int request_id, double* state, double* max, double* sq);
int pasif_pool_info(pasif_pool* p, int* free_slots, long long* free_arena, int* active);
/* Compile (no GPU needed) the pool chunk kernel a pool of this plan would
 * use; compiler report then the source after "// ---- source ----". */
int pasif_plan_jit_report_pool(const pasif_plan* p, int window, const double* im, const pasif_reducers* red,
                               char* log, long long capacity, long long* out_len);

/* Same for the pattern-specialised exact-adjoint kernel (sq_mask: components
 * of the sum-of-squares loss).  Diagnostic; no reference counterpart. */
int pasif_plan_jit_report_adjoint(const pasif_plan* p, const double* values, int n_sys,
                                  unsigned long long sq_mask, char* log, long long capacity,
                                  long long* out_len);
/* Kernel used by the last pasif_batch_adjoint (PASIF_KERNEL_*). */
int pasif_batch_adjoint_kernel(pasif_batch* b, int* kind);

/* Measured FMA-pipe throughput of the current GPU in FLOP/s (FMA = 2 FLOP),
 * FP32 (precision != PASIF_FP64) or FP64: the roofline denominator of the
 * FMA-bound RK4 kernels.  Diagnostic; no reference counterpart. */
int pasif_fma_peak(int precision, double* flops_per_second);

/* One-shot forward from host buffers: upload, integrate, download.  The
 * device buffers stay with the library for the next call with the same
 * pattern, precision, forcing window and weights (a repeated call then
 * allocates and frees nothing), until the process exits; concurrent calls
 * from other threads use buffers of their own. */
int pasif_forward(const pasif_pattern* pattern, int precision, int n_sys, const double* values,
                  const double* x0, const int* exc_index, const double* x, int n_exc, int len,
                  int window, const double* im, double h, int step0, int nsteps,
                  const pasif_reducers* red, double* state, double* max, double* sq);

/* Forward solve for callers that cannot allocate device memory (code inside
 * another framework's memory pool or under a fixed memory budget, code that
 * must not trigger the device synchronisation cudaMalloc/cudaFree can cause,
 * applications that reserve all memory up front).  No counterpart in the
 * reference.  FP64, final state only.  Every array except the pattern is a
 * DEVICE pointer: values[n_sys][P], x0[n_sys][n], exc_index[n_sys],
 * signals[n_exc][len], im[2*window] (window 0: sample and hold),
 * state_out[n_sys][n].  Work space: a 32 MiB array owned by the library on
 * every GPU that loads it (until exit); 8*n_sys*(P+7n) + 4*n_sys bytes must
 * fit in 31 MiB and the pattern in 1 MiB, else PASIF_ERR_INVALID.  The first
 * call on a device looks up the array's address (make it before any stream
 * capture).  Calls share the array and keep its last contents: calls whose
 * GPU work overlaps race.  Returns once the work is queued on `stream`; it
 * neither allocates nor waits for the device (the pattern is passed as kernel
 * arguments).  The excitation indices are checked on the device: a system
 * whose index lies outside [0, n_exc) reads no signal, its state_out row is
 * NaN, and pasif_forward_noalloc_status reports it. */
int pasif_forward_noalloc(const pasif_pattern* pattern, int n_sys, const double* values, const double* x0,
                          const int* exc_index, const double* signals, int n_exc, int len, int window,
                          const double* im, double h, int step0, int nsteps, double* state_out, void* stream);
/* Status of the last pasif_forward_noalloc call on the current device, read
 * from the library's array after waiting for `stream` (pass the stream of
 * that call): *n_bad = systems with an out-of-range excitation index,
 * *first_bad = the lowest of them (n_sys when none; may be NULL).  No
 * counterpart in the reference. */
int pasif_forward_noalloc_status(int* n_bad, int* first_bad, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PASIF_GB300_H */
