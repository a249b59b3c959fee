/*
 * fgpu.h -- C-ABI of the GB300 GPR log-likelihood engine.
 *
 * Drop-in for the likelihood evaluation that FEREBUS-v7's particle swarm runs
 * once per particle: kernel matrix K(theta) + nugget, Cholesky, log-det,
 * alpha = K^-1 (y - mu), marginal or concentrated log-likelihood.
 *
 * Conventions (ISO_C_BINDING compatible: plain pointers and scalars only)
 *  - Arrays are FP64 and column-major exactly as Fortran stores them:
 *    X(N, d) is DataSet%x%data (src/csv.f90:37-177, src/data/data_input.f90:34).
 *  - theta is the reference's raw parameter vector: kernel parameters in
 *    kernel-tree order (src/kernels/kernel_module.f90:235-245) followed, when
 *    optimise_noise is set, by the LINEAR noise value (src/model/gpr/gpr.f90:191-202).
 *    The engine applies exp(theta) (rbf, rbf-cyclic), exp(-theta)^2 (periodic),
 *    exp(-theta) (linear) and the identity (constant) itself.
 *  - Return value: 0 on success, < 0 on an argument / CUDA / allocation error
 *    (fgpu_last_error() has the message).  A non-positive-definite K is NOT
 *    an error: the call returns 0 and sets info > 0 to the 1-based column of
 *    the first non-positive pivot, as LAPACK dpotrf does
 *    (src/model/gpr/likelihood.f90:130-159); the host maps info != 0 to
 *    IterResult%success = .false. (src/optimiser/iter_result.f90:92-101).
 *  - No entry point aborts the process.
 */
#ifndef FGPU_H
#define FGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel-spec opcodes.  kspec is the postfix flattening of the kernel
 * expression tree built by the reference's KernelInterpreter
 * (src/interpreter/kernel_interpreter.f90:43-69, ast.f90:173-271):
 * a leaf is {op, n_active, dim_1 .. dim_n} with 1-based feature indices
 * (TOML active_dimensions), an operator is {op}.  A constant leaf is
 * {FGPU_CONSTANT, 0} and owns one parameter. */
#define FGPU_RBF 1
#define FGPU_PERIODIC 2
#define FGPU_RBF_CYCLIC 3
#define FGPU_LINEAR 4
#define FGPU_CONSTANT 5
#define FGPU_SUM 10
#define FGPU_PROD 11

#define FGPU_MARGINAL 0
#define FGPU_CONCENTRATED 1

/* Error codes (negative return values). */
#define FGPU_OK 0
#define FGPU_EINVAL (-1)
#define FGPU_ECUDA (-2)
#define FGPU_ENOMEM (-3)
#define FGPU_ENODEV (-4)
#define FGPU_ETIMEOUT (-5)

typedef struct fgpu_ctx fgpu_ctx;     /* one training set on one device */
typedef struct fgpu_plan fgpu_plan;   /* a fixed batch of problems, graph-captured */

/* Create a context for one training set.  Replaces the per-GPR set-up of
 * GaussianProcessRegressor%init (src/model/gpr/gpr.f90:124-183) and the
 * distance-tensor precompute (src/kernels/distance_matrix.f90:48-62,
 * called at app/main.f90:108).  X, y and mu are copied to the device once;
 * mu is the cached mean vector (gpr.f90:171) and is ignored (may be NULL)
 * for the concentrated likelihood.  Create it once per training set, not
 * once per particle. */
int fgpu_create(fgpu_ctx** ctx, int N, int d, const double* X, const double* y,
                const double* mu, const int* kspec, int nkspec, int likelihood,
                double noise, int optimise_noise);

/* Number of entries theta must hold (GaussianProcessRegressor%nparams, gpr.f90:248-256). */
int fgpu_nparams(const fgpu_ctx* ctx);

/* Trailing-update arithmetic of the Cholesky for contexts created after the
 * call (process-wide default; returns the previous setting):
 *   FGPU_TRAILING_TCGEN05 (default): 128-wide panels; the O(N^3) update runs
 *     on the tensor cores as exact integer products of 7 fp16 digit planes
 *     per FP64 value, accumulated exactly in int64;
 *   FGPU_TRAILING_FP64: 64-wide panels, FP64 mma.sync on the FP64 pipe.
 * Diagonal blocks, panel solves and the right-hand-side rows are FP64 in
 * both.  The environment variable FGPU_TRAILING=fp64 selects FP64 at load.
 * No counterpart in the reference (which calls LAPACK dpotrf). */
#define FGPU_TRAILING_FP64 0
#define FGPU_TRAILING_TCGEN05 1
int fgpu_set_trailing_update(int mode);

/* Kernel-matrix build for contexts created after the call (process-wide
 * default; returns the previous setting): FGPU_BUILD_TC (default) forms the
 * exact distances on the tensor cores where the kernel allows it (leaves
 * rbf / periodic / linear / constant, at most two rbf-or-periodic leaves);
 * FGPU_BUILD_FP64 keeps the FP64 dot-product build.  The environment
 * variable FGPU_BUILD=fp64 selects FP64 at load.  Both give the likelihood
 * to the parity tolerance; the autotuner picks between them per shape.  No
 * counterpart in the reference. */
#define FGPU_BUILD_FP64 0
#define FGPU_BUILD_TC 1
int fgpu_set_build_mode(int mode);

/* Plain drop-in: one particle per call.  Replaces
 * GaussianProcessRegressor%log_likelihood (src/model/gpr/gpr.f90:291-307) ->
 * compute_R (gpr.f90:185-189) + Likelihood%ll (src/model/gpr/likelihood.f90:161-253).
 * alpha (length N, may be NULL) receives K^-1 (y - mu) (the [weights] of the
 * model file, likelihood.f90:255-264).  Thread-safe: concurrent calls on one
 * context each take their own stream and workspace from the context's pool. */
int fgpu_loglik(fgpu_ctx* ctx, const double* theta, int ntheta, double* ll, int* info,
                double* alpha);

/* Batched: nprob problems (any mix of contexts -- atoms, properties, particles;
 * ragged N and d) evaluated as one graph-captured pass.  Replaces the OpenMP
 * particle loop of global_swarm_update (src/optimiser/pso/pso.f90:419-452)
 * and init_pso (pso.f90:294-308).  theta[p] points at problem p's raw
 * parameters.  The plan for a given context list is built on first use and
 * cached. */
int fgpu_loglik_batch(fgpu_ctx* const* ctxs, int nprob, const double* const* theta,
                      double* ll, int* info);

/* Log-likelihood and its gradient d logL / d theta (including the noise
 * parameter when optimise_noise is set) by the FP64 adjoint
 * 1/2 tr((alpha alpha^T / s - K^-1) dK/dtheta), s = 1 (marginal) or sigma^2
 * (concentrated).  The factor is the evaluation's own (on a tensor-core
 * context the same factor, log-likelihood and alpha as fgpu_loglik), K^-1
 * comes from it in FP64, and dK is recomputed tile by tile.  The reference
 * has no analytic likelihood gradient (negative_log_likelihood,
 * gpr.f90:258-289, accepts but ignores gradient=.true.); this is the
 * optional gradient polish.  dll_dtheta has fgpu_nparams(ctx) entries. */
int fgpu_grad(fgpu_ctx* ctx, const double* theta, int ntheta, double* ll,
              double* dll_dtheta, int* info);

/* Device-resident batch plan (inputs and outputs stay in HBM).  theta_dev is
 * nprob x ldtheta doubles on the device; ll_dev / info_dev are device arrays of
 * nprob entries.  stream is a cudaStream_t (NULL = the plan's own stream).
 * A plan holds at most 65535 problems, 32767 on tensor-core contexts.
 * A plan owns one set of workspaces: its runs must not overlap on the GPU
 * (fgpu_plan_run_device calls on different streams, or one on a stream other
 * than the plan's followed by fgpu_plan_run, race unless the caller orders
 * them); fgpu_plan_run returns after its run has finished.
 * Used by the throughput benchmark and by hosts that keep the swarm on the GPU.
 * A plan whose problems' workspaces exceed the device-memory budget (the
 * free memory less a reserve, or FGPU_PLAN_MEM_BUDGET_MB) runs them in waves
 * that share one workspace arena, still as one graph replay per run; a single
 * problem larger than the budget is FGPU_ENOMEM.  After fgpu_plan_run_device,
 * info_dev[p] < 0 means -1: a bounded device wait gave up (fgpu_plan_run
 * returns FGPU_ETIMEOUT for it), -2: a panel value broke its row-scale bound
 * (fgpu_plan_run returns FGPU_ECUDA); ll_dev[p] is then NaN.  No counterpart
 * in the reference (its particles are evaluated one per OpenMP thread,
 * src/optimiser/pso/pso.f90:419-452). */
int fgpu_plan_create(fgpu_plan** plan, fgpu_ctx* const* ctxs, int nprob, int ldtheta);
int fgpu_plan_run_device(fgpu_plan* plan, const double* theta_dev, double* ll_dev,
                         int* info_dev, void* stream);
int fgpu_plan_run(fgpu_plan* plan, const double* theta_host, double* ll_host,
                  int* info_host);
void fgpu_plan_destroy(fgpu_plan* plan);

/* The waves a plan runs in and the bytes of its shared workspace arena. */
int fgpu_plan_waves(const fgpu_plan* plan, int* nwaves, long long* arena_bytes);

/* Host-only: the wave partition fgpu_plan_create applies to problems of
 * the given workspace sizes under `budget` bytes (wave_of[i] receives
 * problem i's wave).  Touches no device; for checking the partition rule. */
int fgpu_plan_partition(const long long* bytes, int n, long long budget, int* wave_of, int* nwaves);

/* Frees a context, its workers, its adjoint workspace and the plans
 * fgpu_loglik_batch cached for it.  Call it only after every call that uses
 * the context has returned and every plan built over it (fgpu_plan_create)
 * has been destroyed or will not run again: those plans read the context's
 * training data on the device. */
void fgpu_destroy(fgpu_ctx* ctx);

/* One evaluation that allocates no device memory.  No counterpart in the
 * reference: it exists for hosts that may not call cudaMalloc when they need
 * a likelihood (device memory owned by an OpenACC runtime's data regions, or
 * by a pool that forbids side allocations).  Inputs (X(N,d) column-major, y,
 * mu, theta: theta holds the kernel parameters and, with optimise_noise, the
 * linear noise value last) and outputs (ll, info: one value each) are DEVICE
 * pointers; kspec is host memory.  All intermediates live in one fixed
 * static device array (about 9.5 MB per device, held until the process
 * exits), so N <= FGPU_NOALLOC_MAX_N and the kernel spec may need at most
 * FGPU_NOALLOC_MAX_PLANES feature planes (one per rbf dim, two per periodic
 * dim); larger inputs are rejected with FGPU_EINVAL before any device work.
 * The work, including the copy of the call's descriptors (passed as kernel
 * arguments, no host staging buffer), is enqueued on `stream` (a
 * cudaStream_t, NULL = legacy default) and the call returns without waiting
 * for it; read ll/info after synchronising with the stream.  *info_dev is 0,
 * a LAPACK-style pivot column > 0 (non-positive-definite K, ll NaN), or
 * negative: -1 a bounded device wait gave up (what other entry points report
 * as FGPU_ETIMEOUT), -2 a panel value broke its row-scale bound (FGPU_ECUDA).
 * The first call on a device resolves the array's address
 * (cudaGetSymbolAddress) -- make it before any stream capture.  Every call
 * shares the array and finds the previous call's contents there: calls
 * that overlap on the GPU race and must be serialised by the caller. */
#define FGPU_NOALLOC_MAX_N 1024
#define FGPU_NOALLOC_MAX_PLANES 64
int fgpu_loglik_noalloc(int N, int d, const double* X_dev, const double* y_dev, const double* mu_dev,
                        const int* kspec, int nkspec, int likelihood, double noise, int optimise_noise,
                        const double* theta_dev, double* ll_dev, int* info_dev, void* stream);

/* Stage timing for roofline accounting.  When enabled, the plan's graph is
 * re-captured with CUDA event nodes around every launch (enable = 1) or
 * around the trailing-update launches only (enable = 2, which leaves the
 * rest of the graph as it runs unprofiled); after a run,
 * fgpu_plan_stage_times fills ms[k] with the summed device time of stage k
 * during the LAST replay and count[k] with its launches (k: 0 build,
 * 1 diagonal factor, 2 panel solve, 3 trailing update, 4 likelihood
 * epilogue, 5 panel conversion, 6 digit split, 7 right-hand-side rows,
 * 8 quarter-panel coupling).
 * Diagnostic only; the reference has no counterpart. */
#define FGPU_NSTAGES 9
int fgpu_plan_set_profiling(fgpu_plan* plan, int enable);
int fgpu_plan_stage_times(fgpu_plan* plan, double* ms, int* count);

/* The device exponential every kernel-matrix entry goes through (a
 * fixed-point evaluation on the integer pipes), applied to n host values:
 * y[i] = exp(x[i]).  Diagnostic only, for checking it against the host libm;
 * synchronous.  The reference has no counterpart. */
int fgpu_diag_exp(const double* x, double* y, int n);

/* The kernel-matrix build's form of that exponential, for exact integer
 * arguments of one scale: y[i] = exp(-E[i] 2^e), e in -128..-1.
 * Diagnostic only, synchronous.  The reference has no counterpart. */
int fgpu_diag_exp_fixed(const unsigned long long* E, int e, double* y, int n);

/* The kernels' bounded mbarrier wait, alone: one warp waits with `polls`
 * polls (1 .. 2^22) on a barrier that nothing arrives on (arrive = 0), or
 * that it completed itself first (arrive = 1).  Returns FGPU_ETIMEOUT when
 * the wait gave up -- through the same status word and host mapping as an
 * evaluation -- and FGPU_OK otherwise; nothing asynchronous is in flight,
 * and the device stays usable.  Diagnostic only, synchronous; the reference
 * has no counterpart. */
int fgpu_diag_wait(int polls, int arrive);

/* Thread-local message for the last failing call on this thread. */
const char* fgpu_last_error(void);

/* Engine version string and the number of kernel launches the last call on
 * this thread enqueued (graph replays count their nodes). */
const char* fgpu_version(void);
long long fgpu_last_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* FGPU_H */
