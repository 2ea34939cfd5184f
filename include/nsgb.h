/*
 * nsgb.h -- C ABI of the GB300 (sm_103a) single-device Chorin-projection solver.
 *
 * Each entry point replaces one operation of the reference JAX solver
 * (helmhlotz/ns_solver_jax_differential_distributed, file NS_solver.py); the
 * comment above it names the reference symbol and lines it stands in for.
 *
 * Conventions
 *  - Fields are float32, C-contiguous, caller-owned DEVICE pointers.  A vector
 *    field is (2, N, N): component 0 = u_x, 1 = u_y; axis 1 = x (rows, index i),
 *    axis 2 = y (contiguous, index j) -- the reference's layout
 *    (NS_solver.py:116, 676-679).
 *  - N is a power of two, 16 <= N <= NSGB_MAX_N (8192).
 *  - Fields read by the step kernels (u, u0) must be 16-byte aligned (the
 *    kernels load them as float4 groups); a misaligned pointer is rejected
 *    with NSGB_ERR_INVALID_ARG.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  All calls are
 *    asynchronous with respect to the host unless stated otherwise.
 *  - Every call returns an int status (NSGB_OK = 0); on failure the
 *    thread-local nsgb_last_error() string says why.  No C++ exception crosses
 *    this boundary.
 *  - `theta` is a device pointer to theta_len float32 values: [A, B] (the
 *    reference's forcing parameters, NS_solver.py:623) or [A, B, nu], in which
 *    case theta[2] replaces the viscosity.
 *  - Workspace buffers are caller-owned device memory of at least the size
 *    the matching *_workspace_bytes() query returns.  A plan owns only its
 *    constant tables (twiddles, squared wavenumbers).
 */
#ifndef NSGB_H
#define NSGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSGB_OK 0
#define NSGB_ERR_INVALID_ARG 1
#define NSGB_ERR_UNSUPPORTED_N 2
#define NSGB_ERR_CUDA 3
#define NSGB_ERR_OOM 4
#define NSGB_ERR_WORKSPACE 5
#define NSGB_ERR_NONFINITE 6
#define NSGB_ERR_BOUNDS 7    /* bounds-checking build: a kernel accessed memory outside the valid ranges */

#define NSGB_MAX_N 8192 /* largest grid a plan accepts */

#define NSGB_SCHEME_CENTRAL 0 /* CentralAdvection, NS_solver.py:468-477 */
#define NSGB_SCHEME_UPWIND 1  /* UpwindAdvection,  NS_solver.py:480-488 */

typedef struct nsgb_plan nsgb_plan;

/* Physical and time parameters of one solve: the reference's Phys (nu, mu0,
 * sigma0, C; NS_solver.py:99-101), Time.dt (NS_solver.py:108-110), the grid
 * length L (NS_solver.py:112-117) and the advection scheme name. */
typedef struct nsgb_phys {
  double L;
  double nu;
  double dt;
  double mu0;
  double sigma0;
  double C;
  int scheme; /* NSGB_SCHEME_* */
} nsgb_phys;

/* Library version (major*10000 + minor*100 + patch). */
int nsgb_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* nsgb_last_error(void);

/* Create the constant tables of one grid size on the current device: the
 * FFT twiddles and the squared wavenumbers k = 2*pi*fftfreq(N, dx) of
 * SpectralPoissonSolver.__init__ (NS_solver.py:517-521).  A plan is immutable
 * after set-up and may be shared by streams. */
int nsgb_plan_create(int N, double L, nsgb_plan** plan);
int nsgb_plan_destroy(nsgb_plan* plan);

/* No counterpart in the reference (launch tuning).  Launch shapes used by
 * the plan's kernels: the stencil shape -- a tile of tw x th cells (tw <= 128)
 * of the tiled kernel, or for tw >= 256 a band of min(tw, N) columns by th
 * rows of the row-streaming kernel -- then rows per CTA of the row FFTs and
 * k-rows per CTA of the column FFT.  0 keeps the current value.  Chosen by
 * the autotuner; results do not depend on them. */
int nsgb_plan_set_tiles(nsgb_plan* plan, int tw, int th, int rows_per_cta, int cols_per_cta);
int nsgb_plan_get_tiles(const nsgb_plan* plan, int out[4]);

/* No counterpart in the reference (launch tuning).  Stockham radix (16 or 8)
 * of the row passes and of the column pass of the FFT-Poisson solve; 0 keeps
 * the current value.  Radix 8 carries a transform on twice as many threads
 * with half the registers each.  Results agree to FFT rounding. */
int nsgb_plan_set_fft_radix(nsgb_plan* plan, int radix_rows, int radix_cols);
int nsgb_plan_get_fft_radix(const nsgb_plan* plan, int out[2]);

/* No counterpart in the reference (launch tuning).  Shape of the adjoint
 * stencil in nsgb_rollout_grad: a tile of tw x th cells of the tiled kernel
 * (tw <= 128, tw <= N, th <= N), or for tw >= 256 a band of min(tw, N)
 * columns (tw a power of two <= 1024) by th rows of the row-streaming kernel;
 * 0 keeps the current value.  lambda and dJ/du0 have the same bits for every
 * shape; the theta sensitivities are summed per CTA, so they agree to
 * rounding across shapes (and are reproducible for a fixed shape). */
int nsgb_plan_set_adjoint_tiles(nsgb_plan* plan, int tw, int th);
int nsgb_plan_get_adjoint_tiles(const nsgb_plan* plan, int out[2]);

/* No counterpart in the reference (launch choice).  rows > 0 makes
 * nsgb_rollout run each step after the first as two kernels instead of four:
 * a fused row kernel -- the inverse row FFT of the solved spectrum into p in
 * shared memory, the stencil of SingleCoreNSSolver.step (NS_solver.py:727-730,
 * ChorinProjector.step :671-697, with the projection of the previous step)
 * and the forward row FFT of its div(u*)/dt -- then the column FFT with the
 * Poisson multiplier (SpectralPoissonSolver.__call__, :523-527), so neither p
 * nor the right-hand side is written to device memory between the kernels.
 * Bands of `rows` rows (even); clusters of N/2048 CTAs split each row when N
 * > 2048.  rows < 0 picks the band height that fits all clusters on the GPU
 * in one wave; 0 restores the four-kernel step.  N in {1024, 2048, 4096}
 * (NSGB_ERR_UNSUPPORTED_N otherwise).  The results are those of the
 * four-kernel step with the row-streaming stencil of the same band (width
 * min(N, 2048), `rows` rows) and radix-16 row transforms, bit for bit. */
int nsgb_plan_set_fused(nsgb_plan* plan, int rows);
int nsgb_plan_get_fused(const nsgb_plan* plan, int* rows);

/* Bytes of workspace for nsgb_poisson / nsgb_projector_step / nsgb_step. */
size_t nsgb_poisson_workspace_bytes(const nsgb_plan* plan);
size_t nsgb_step_workspace_bytes(const nsgb_plan* plan);
/* Bytes of workspace for nsgb_rollout over `steps` steps. */
size_t nsgb_rollout_workspace_bytes(const nsgb_plan* plan, int steps);
/* Bytes of workspace for nsgb_rollout_grad with checkpoints every `every` steps. */
size_t nsgb_rollout_grad_workspace_bytes(const nsgb_plan* plan, int steps, int every);

/* PeriodicDifferentialOps.grad (NS_solver.py:243-247): central gradient.
 * f: (N,N); gx, gy: (N,N). */
int nsgb_grad(const nsgb_plan* plan, const float* f, float* gx, float* gy, void* stream);

/* PeriodicDifferentialOps.laplacian (NS_solver.py:249-255): 5-point Laplacian. */
int nsgb_laplacian(const nsgb_plan* plan, const float* f, float* out, void* stream);

/* DifferentialOps.divergence / divergence_vec (NS_solver.py:206-218):
 * u: (2,N,N) -> out: (N,N). */
int nsgb_divergence(const nsgb_plan* plan, const float* u, float* out, void* stream);

/* AdvectionScheme.advect (NS_solver.py:453-488): -(u.grad) field with the
 * central gradient (CentralAdvection, :474-477) or first-order upwind
 * differences (PeriodicDifferentialOps.upwind_advect, :257-265). */
int nsgb_advect(const nsgb_plan* plan, int scheme, const float* field, const float* ux,
                const float* uy, float* out, void* stream);

/* SpectralPoissonSolver.__call__ (NS_solver.py:523-527): p = Re ifft2(
 * -fft2(rhs) * inv_k2) with p_hat[0,0] = 0, i.e. lap(p) = rhs.  Hand-written
 * R2C / C2R FFTs; `workspace` holds the half spectrum. */
int nsgb_poisson(const nsgb_plan* plan, const float* rhs, float* p, void* workspace,
                 size_t workspace_bytes, void* stream);

/* GaussianForcingField.__call__ (NS_solver.py:637-640): writes the (2,N,N)
 * force field at time t (fy = 0). */
int nsgb_forcing(const nsgb_plan* plan, const nsgb_phys* phys, const float* theta, int theta_len,
                 float t, float* f_out, void* stream);

/* ChorinProjector.step (NS_solver.py:671-697) with an explicit force field
 * f (2,N,N): u* = u + dt(nu lap u + adv(u) + f); p = poisson(div(u*)/dt);
 * u_out = u* - dt grad p.  nu, dt, scheme are taken from `phys`. */
int nsgb_projector_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u,
                        const float* f, float* u_out, void* workspace, size_t workspace_bytes,
                        void* stream);

/* SingleCoreNSSolver.step (NS_solver.py:727-730): one step with the Gaussian
 * forcing at time t. */
int nsgb_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u, const float* theta,
              int theta_len, float t, float* u_out, void* workspace, size_t workspace_bytes,
              void* stream);

/* SingleCoreNSSolver.rollout (NS_solver.py:732-750): `steps` steps from u0 with
 * t = i*dt, accumulating J += dt * sum(u*f) * dx^2 on the state before each
 * step.  Writes u_final (2,N,N) and *J (one float, device).  The projection of
 * each step is fused into the next step's stencil; steps are replayed as
 * CUDA-graph chunks when use_graph != 0. */
int nsgb_rollout(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                 int theta_len, int steps, float* u_final, float* J, void* workspace,
                 size_t workspace_bytes, int use_graph, void* stream);

/* Phases of nsgb_rollout_grad. */
#define NSGB_GRAD_FORWARD 1  /* rollout with checkpoints, J, u_final */
#define NSGB_GRAD_BACKWARD 2 /* adjoint sweep: dJ/dtheta (and dJ/du0) */

/* jax.grad of the rollout objective (SingleCoreNSSolver.jit_gradient,
 * NS_solver.py:725, generalised to a given u0): hand-written discrete adjoint
 * of the whole step with checkpoints of the state every `every` steps and
 * recomputation of each segment during the backward sweep.
 * `phases` selects NSGB_GRAD_FORWARD and/or NSGB_GRAD_BACKWARD; a backward
 * call must follow a forward call with the same arguments and workspace
 * (the checkpoints live in the workspace).  The forward phase writes *J and,
 * if non-NULL, u_final; the backward phase writes dJdtheta[theta_len] and, if
 * non-NULL, dJdu0 (2,N,N).  A call repeated with the same arguments (pointers,
 * sizes, physics, launch shapes) is captured as one CUDA graph on its second
 * use and replayed after that, with the same results; inside a caller's own
 * stream capture the work is recorded eagerly.  Workspace:
 * nsgb_rollout_grad_workspace_bytes(plan, steps, every) (it depends on the
 * plan's adjoint shape). */
int nsgb_rollout_grad(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0,
                      const float* theta, int theta_len, int steps, int every, int phases,
                      float* J, float* u_final, float* dJdtheta, float* dJdu0, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Bounds checking (no counterpart in the reference).  The library built with
 * NSGB_CHECK_BOUNDS (libnsgb_checked.so) checks every global-memory access of
 * its kernels against the device ranges it knows to be valid: its plans'
 * tables, its static scratch, and the ranges registered here.  An access
 * outside all of them is skipped (a load yields zero) and counted, and the
 * entry point that launched it waits for its stream and returns
 * NSGB_ERR_BOUNDS with the first bad address, its size and the source line of
 * the access, instead of faulting.  In the normal build these calls do
 * nothing and return NSGB_OK; nsgb_bounds_checking() tells the builds apart
 * (1 when checking).  Registered ranges are [base, base + bytes).  The
 * checked build keeps one table of ranges per process and loads it into the
 * current device whenever it changes: use it with one device. */
int nsgb_bounds_checking(void);
int nsgb_bounds_register(const void* base, size_t bytes);
int nsgb_bounds_unregister(const void* base);
int nsgb_bounds_clear(void);

/* One gradient solve of a batch advanced by nsgb_grad_batch_advance. */
typedef struct nsgb_grad_member {
  const nsgb_plan* plan; /* plan of this solve's N and L; its launch shapes must not
                            change while the solve is in progress */
  nsgb_phys phys;
  const float* u0;       /* (2,N,N) device */
  const float* theta;    /* device, theta_len entries */
  int theta_len;
  int steps, every;      /* rollout length and checkpoint interval */
  float* J;              /* one float, device; written when the forward phase ends */
  float* u_final;        /* (2,N,N) device or NULL; written with J */
  float* dJdtheta;       /* device, theta_len entries; written when the solve completes */
  float* dJdu0;          /* (2,N,N) device or NULL; written when the solve completes */
  void* state;           /* device state kept between calls:
                            nsgb_rollout_grad_workspace_bytes(plan, steps, every) bytes,
                            256-byte aligned */
  int done_ops;          /* operations of its schedule already done (0: not started) */
} nsgb_grad_member;

/* Operations in the schedule of one gradient solve (0 on invalid arguments):
 * `steps` forward steps, then per checkpoint segment (last first) its
 * recomputed steps and its `steps`-many adjoint steps in total. */
int nsgb_grad_ops(int steps, int every);

/* Bytes of workspace for nsgb_grad_batch_advance of `count` solves by up to
 * `ops` operations (the argument tables of the call). */
size_t nsgb_grad_batch_workspace_bytes(int count, int ops);

/* Batched, continuously batchable form of nsgb_rollout_grad (both phases;
 * jax.grad of the rollout objective, NS_solver.py:725): every member performs
 * min(ops, nsgb_grad_ops(steps, every) - done_ops) further operations of its
 * schedule, the members in lock-step.  At each step, the stencils of the
 * forward and recomputed steps of all members with the same plan and scheme
 * are ONE batched launch, their adjoint stencils another, and all their
 * FFT-Poisson solves one batched launch per pass; groups of different plans
 * run side by side on internal streams joined back into `stream`.  Each
 * member's J, u_final,
 * dJdtheta and dJdu0 equal those of nsgb_rollout_grad with the same
 * arguments bit for bit, however its work is split into calls and whatever
 * else is in the batch.  The caller advances done_ops itself.  Uploads its
 * argument tables from host memory, so it refuses a capturing stream. */
int nsgb_grad_batch_advance(const nsgb_grad_member* members, int count, int ops, void* workspace,
                            size_t workspace_bytes, void* stream);

/* One member of an ensemble of independent solves (see nsgb_ensemble_advance). */
typedef struct nsgb_member {
  const nsgb_plan* plan; /* plan of this member's N and L (tiles as tuned) */
  nsgb_phys phys;
  const float* u0;       /* (2,N,N) device; read when done_steps == 0 */
  const float* theta;    /* device, theta_len entries */
  int theta_len;
  float* u_final;        /* (2,N,N) device; written when the member finishes */
  float* J;              /* one float, device; written when the member finishes */
  void* state;           /* device state kept between calls, at least
                            nsgb_rollout_workspace_bytes(plan, total_steps) bytes,
                            256-byte aligned; NULL: carved from the call's workspace */
  int total_steps;       /* steps of the whole solve */
  int done_steps;        /* steps already taken (0: start from u0) */
} nsgb_member;

/* Bytes of workspace for nsgb_ensemble_advance / nsgb_ensemble_rollout (the
 * member table plus the state of every member whose `state` is NULL). */
size_t nsgb_ensemble_workspace_bytes(const nsgb_member* members, int count);

/* Ensemble form of SingleCoreNSSolver.rollout (NS_solver.py:732-750), used for
 * batching and continuous batching: every member takes min(steps, total_steps
 * - done_steps) further steps from its saved state; members that reach
 * total_steps get u_final and J written.  Members with the same plan, scheme,
 * progress parity and step count form a group, and each stage of a step is
 * ONE batched launch per group (the member index is a grid dimension); the
 * groups run side by side on internal streams that start after the work
 * already on `stream` and that `stream` waits for.  The results equal one
 * nsgb_rollout per member bit for bit.  The caller advances done_steps
 * itself.  It uploads the member table from host memory, so it refuses a
 * capturing stream (as does nsgb_ensemble_rollout, which captures its step
 * chunks itself). */
int nsgb_ensemble_advance(const nsgb_member* members, int count, int steps, void* workspace,
                          size_t workspace_bytes, void* stream);

/* One-shot ensemble: all members start from u0 (done_steps ignored) and run
 * total_steps (equal for all members).  Chunks of `chunk` steps (even; 0 =
 * direct launches) are replayed as ONE CUDA graph per chunk in which the
 * groups run as parallel branches; `workspace` must stay the same between
 * calls for the cached graph to be reused. */
int nsgb_ensemble_rollout(const nsgb_member* members, int count, int chunk, void* workspace,
                          size_t workspace_bytes, void* stream);

/* The ensemble of nsgb_ensemble_rollout (members start from u0 and run equal
 * total_steps) advanced in ONE persistent cooperative launch: its CTAs walk a
 * work list per stage -- the 64 x 16 stencil tiles of every member, then the
 * blocks of the forward row, column and inverse row transforms -- with a
 * bounded grid-wide barrier between stages, for every step.  Members' fields
 * equal their solo rollouts with radix-16 transforms bit for bit; the
 * objective partials follow that tiling, so J agrees to rounding.  N a
 * power of two in [64, 4096] (NSGB_ERR_UNSUPPORTED_N otherwise).  If a CTA
 * waits at a barrier beyond the launch's bound, the launch stops and every J
 * is NaN.  Refuses a capturing stream (it uploads its tables from host
 * memory).  Workspace: nsgb_ensemble_persistent_workspace_bytes (0 on invalid
 * members). */
size_t nsgb_ensemble_persistent_workspace_bytes(const nsgb_member* members, int count);
int nsgb_ensemble_persistent(const nsgb_member* members, int count, void* workspace, size_t workspace_bytes,
                             void* stream);

/* Measurement helper (no counterpart in the reference): runs the four kernels
 * of one rollout step from state u0 `reps` times each on `stream`, each launch
 * bracketed by CUDA events, and writes the mean device time per launch in
 * milliseconds: out_ms[0] fused stencil, [1] row FFT forward, [2] column FFT
 * with the Poisson multiplier, [3] row FFT inverse.  With the fused row
 * kernel (nsgb_plan_set_fused) a step has two kernels: out_ms[0] the fused
 * row kernel, [1] the column FFT, [2] and [3] zero.  When flush != NULL,
 * flush_bytes of it are overwritten before every timed launch (outside the
 * events) so each launch starts with a cold L2.  Synchronises the stream.
 * Workspace: nsgb_rollout_workspace_bytes(plan, 1). */
int nsgb_time_stages(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0,
                     const float* theta, int theta_len, int reps, void* flush,
                     size_t flush_bytes, void* workspace, size_t workspace_bytes, float* out_ms,
                     void* stream);

/* Measurement helper (no counterpart in the reference): runs `steps` solver
 * steps from state u0 back to back on `stream`, as a rollout does, with a
 * CUDA event between consecutive kernels, and writes the mean device time per
 * launch of the four step kernels in milliseconds (out_ms as for
 * nsgb_time_stages): the durations the kernels have inside the pipelined
 * rollout, L2 shared between them.  Synchronises the stream.  Workspace:
 * nsgb_rollout_workspace_bytes(plan, steps). */
int nsgb_time_step_pipeline(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0,
                            const float* theta, int theta_len, int steps, void* workspace,
                            size_t workspace_bytes, float* out_ms, void* stream);

/* Optimisers of ParameterOptimizationStudy (studies.py:879-884): optax
 * 0.2.4's sgd, adam and rmsprop, whose update rules nsgb_optim.cu restates. */
#define NSGB_OPT_SGD 0
#define NSGB_OPT_ADAM 1
#define NSGB_OPT_RMSPROP 2

typedef struct nsgb_optimizer {
  int kind;             /* NSGB_OPT_* */
  double learning_rate;
  double b1, b2;        /* adam moment decays (optax defaults 0.9, 0.999) */
  double eps;           /* adam: added to sqrt(v_hat); rmsprop: inside the sqrt (1e-8) */
  double eps_root;      /* adam: inside the sqrt (0) */
  double decay;         /* rmsprop second-moment decay (0.9) */
} nsgb_optimizer;

/* Workspace of nsgb_optimize: the gradient workspace of (steps, every) plus
 * the parameters, gradient, optimiser moments and two state fields.  0 on an
 * invalid argument. */
size_t nsgb_optimize_workspace_bytes(const nsgb_plan* plan, int steps, int every, int theta_len);

/* ParameterOptimizationStudy._run_single_optimizer (studies.py:890-934) on
 * the device: from theta0, `iters` optimiser steps theta_{k+1} = theta_k +
 * update(dJ/dtheta(theta_k)), the gradient by the discrete adjoint of a
 * `steps`-step rollout (nsgb_rollout_grad, checkpoints every `every` steps)
 * from u0, or from the zero state when u0 is NULL (objective / jit_gradient,
 * NS_solver.py:724-725, 752-756).  Writes objectives[k] = J(theta_k) for
 * k = 0..iters and parameters[k * theta_len ...] = theta_k (device arrays of
 * iters + 1 and (iters + 1) * theta_len floats).  Every launch is ordered on
 * `stream`; the host never waits.  theta_len 2 ([A, B]) or 3 ([A, B, nu]). */
int nsgb_optimize(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta0,
                  int theta_len, int steps, int every, const nsgb_optimizer* opt, int iters, float* objectives,
                  float* parameters, void* workspace, size_t workspace_bytes, void* stream);

/* Largest N accepted by nsgb_poisson_noalloc. */
#define NSGB_NOALLOC_MAX_N 1024

/* No counterpart in the reference.  The spectral Poisson solve of
 * nsgb_poisson (lap(p) = rhs, same kernels, same results) for callers that
 * cannot allocate device memory when they solve: code confined to a fixed
 * device-memory budget it cannot grow, loops in which a cudaMalloc (which may
 * synchronise the device) is unacceptable, and plain C FFI hosts that cannot
 * own a plan and a workspace.  It needs no plan and no workspace: its scratch
 * (the half spectrum and the constant tables) is a file-scope static device
 * array for N <= NSGB_NOALLOC_MAX_N, about 4.2 MB held on every GPU that loads
 * the library until the process exits; larger N is rejected with
 * NSGB_ERR_UNSUPPORTED_N.  It calls no cudaMalloc or cudaFree.  The first call
 * on a device resolves the arrays' device addresses (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture.
 * Those addresses are cached per device ordinal, i.e. for the runtime's
 * primary context (the one torch uses); do not reuse them across a
 * cudaDeviceReset or from a context the caller created itself.  A call whose
 * stream is capturing returns NSGB_ERR_INVALID_ARG and enqueues nothing: its
 * table uploads read shared host buffers that a later call may refill before
 * a graph replay would read them.
 * All calls share the arrays, which keep the last call's contents: calls
 * whose work overlaps on the GPU (other streams or host threads) race and
 * must be serialised by the caller.  rhs and p are (N,N) float32 device
 * fields on the current device. */
int nsgb_poisson_noalloc(int N, double L, const float* rhs, float* p, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NSGB_H */
