// Internal interfaces between the kernel translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "nsgb_common.cuh"

namespace nsgb {

// ------------------------------------------------------------------ FFT --
struct FftLaunch {
  const float* rhs = nullptr;  // rows forward input (nullptr: skip the pass)
  float2* spec = nullptr;      // transposed half spectrum, (N/2 + 1) x N complex
  bool do_cols = true;         // column transform + Poisson multiplier
  float* p = nullptr;          // rows inverse output (nullptr: skip the pass)
  const float2* tw = nullptr;  // per-pass twiddle tables (nsgb_fft.cuh)
  const float* k2 = nullptr;   // squared wavenumbers, N entries
  float scale = 0.f;           // 1 / (2 N^2)
  int rows_per_cta = 8;        // even, power of two
  int cols_per_cta = 2;        // power of two
  int radix_rows = 16;         // Stockham radix of the row passes (16 or 8)
  int radix_cols = 16;         // ... and of the column pass
};
cudaError_t poisson_fft(int N, const FftLaunch& L, cudaStream_t st);
size_t fft_rows_smem_bytes(int N, int rows_per_cta);
size_t fft_cols_smem_bytes(int N, int cols_per_cta);

// --------------------------------------------------------------- stencil --
enum StencilMode : int {
  MODE_ROLLOUT = 0,  // Gaussian forcing computed per row, J partial per block
  MODE_FIELD = 1,    // explicit (2,N,N) force field, no J
};

struct StencilArgs {
  const float* us = nullptr;     // (2,N,N) u* of the pending projection (or u if p == nullptr)
  const float* p = nullptr;      // (N,N) pressure of the pending projection, or nullptr
  const float* f = nullptr;      // (2,N,N) force field (MODE_FIELD)
  float* us_out = nullptr;       // (2,N,N) next u*
  float* rhs = nullptr;          // (N,N) div(u*)/dt
  float* u_out = nullptr;        // optional (2,N,N): the projected state u^n
  float* jpart = nullptr;        // per-block partial sums of u_x * f_x, [step][nblk]
  int jpart_rows = 0;            // rows allocated in jpart (a store beyond is skipped)
  const float* theta = nullptr;  // device theta
  int theta_len = 2;
  const int* step_ctr = nullptr;  // device step base (nullptr: 0); step = base + step_fixed
  int step_fixed = 0;
  int t_from_step = 1;  // t = float(step) * dt (rollout) or t_fixed (single step)
  float t_fixed = 0.f;
  int scheme = 0;
  int tw = 64, th = 16;  // tile shape, or row-streaming band (tw >= NSGB_ROWS_MIN_W)
  StepConsts c;
};
cudaError_t launch_stencil(const StencilArgs& a, int mode, cudaStream_t st);
int stencil_nblocks(int N, int tw, int th);
bool stencil_tile_supported(int tw, int th);
// Launch shapes with tw >= NSGB_ROWS_MIN_W select the row-streaming kernel:
// bands of min(tw, N) columns (a power of two <= NSGB_ROWS_MAX_W) by th rows.
constexpr int NSGB_ROWS_MIN_W = 256;
constexpr int NSGB_ROWS_MAX_W = 2048;
bool stencil_rows_mode(int tw);
bool stencil_rows_supported(int N, int tw, int th);
// Tile of the tiled kernel for N (the adjoint and explicit-force steps use it
// when the forward stencil streams rows).
void tile_kernel_default(int N, int& tw, int& th);

// ---------------------------------------------------- fused row kernel --
// One rollout step's row work in one launch (nsgb_fused.cu): inverse row FFT
// of spec_in into p (on chip), the fused stencil (a.us -> a.us_out, objective
// partial; a.th = rows per band, a.tw unused) and the forward row FFT of its
// rhs into spec_out.  The column pass (k_cols) then runs on spec_out.
struct FusedArgs {
  StencilArgs a;
  const float2* spec_in = nullptr;  // half spectrum after the previous step's column pass
  float2* spec_out = nullptr;       // half spectrum of this step's rhs (row transforms only)
  const float2* tw = nullptr;       // the plan's radix-16 twiddle tables
};
bool fused_supported(int N);
int fused_cluster(int N);               // CTAs per cluster (= N / band width)
int fused_nblocks(int N, int th);       // CTAs per launch (the objective partials per step)
cudaError_t launch_fused_rows(const FusedArgs& f, cudaStream_t st);
// Band height whose clusters all fit on the GPU at once (one CTA per SM).
cudaError_t fused_default_rows(int N, int& rows);

// ------------------------------------------------------------- ensembles --
// Device-resident description of one member of an ensemble advanced by
// batched launches (blockIdx.z / blockIdx.y = member).
struct FftPtrs {
  const float* rhs;
  float2* spec;
  float* p;
};
struct SolveDev {
  StencilArgs st[3];  // 0: first step (u0 -> A), 1: A -> B, 2: B -> A
  FftPtrs fft;
  float* u_final;
  float* J;
  double* jsteps;
  double jscale;
  int* ctr;
  int ctr_init;  // progress of the member when the call started
};
cudaError_t launch_stencil_batch(const SolveDev* solves, int count, int variant, int step_off, int scheme, int N,
                                 int tw, int th, cudaStream_t st);
cudaError_t launch_project_batch(const SolveDev* solves, int count, int variant, int N, cudaStream_t st);
cudaError_t launch_jreduce_batch(const SolveDev* solves, int count, int nblk, int steps, cudaStream_t st);
// add: *ctr += value; otherwise *ctr = ctr_init + value (per member)
cudaError_t launch_counter_batch(const SolveDev* solves, int count, int value, bool add, cudaStream_t st);
cudaError_t poisson_fft_batch(int N, const FftLaunch& L, const SolveDev* solves, int count, cudaStream_t st);

// ------------------------------------------------- persistent ensemble --
// One cooperative launch for all steps of an ensemble (nsgb_ens_persistent.cu).
struct PersMember {
  const float2* tw;  // the member's plan twiddles (radix-16 tables first)
  const float* k2;
  float scale;       // 1 / (2 N^2)
  int N;
};
struct PersWork {
  const SolveDev* dev;     // members, in table order
  const PersMember* pm;
  const int* first[4];     // per stage (stencil, rows fwd, cols, rows inv): first item of each member, count + 1
  int items[4];            // per stage: total items
  int count, steps, done;  // members; steps of the launch; steps done before it
  unsigned* bar;           // barrier words: arrivals, generation, abort (zeroed before the launch)
  unsigned poll_limit;     // polls of a waiting CTA before it gives up
};
bool pers_supported(int N);        // N a power of two in [64, 4096]
void pers_tile(int N, int& tw, int& th);  // stencil tile of the persistent launch
size_t pers_smem_bytes(int N);     // dynamic shared memory the items of N need
void pers_items(int N, int out[4]);
cudaError_t launch_ensemble_persistent(const PersWork& w, size_t smem, int sms, int* grid_out, cudaStream_t st);
// J of every member non-finite when the launch gave up at a barrier
cudaError_t launch_ensemble_poison(const unsigned* bar, const SolveDev* dev, int count, cudaStream_t st);

// u_out = us - dt * grad(p)  (NS_solver.py:696-697)
cudaError_t launch_project(const float* us, const float* p, float* u_out, const StepConsts& c,
                           cudaStream_t st);
// Sum the per-block partials of each step in a fixed order and accumulate J.
cudaError_t launch_jreduce(const float* jpart, int nblk, int steps, double* jsteps, float* J,
                           double jscale, cudaStream_t st);
// *step_ctr = value (add = false) or *step_ctr += value (add = true)
cudaError_t launch_step_counter(int* step_ctr, int value, bool add, cudaStream_t st);

// Single operators of PeriodicDifferentialOps / AdvectionScheme.
cudaError_t launch_grad(const float* f, float* gx, float* gy, const StepConsts& c, cudaStream_t st);
cudaError_t launch_laplacian(const float* f, float* out, const StepConsts& c, cudaStream_t st);
cudaError_t launch_divergence(const float* u, float* out, const StepConsts& c, cudaStream_t st);
cudaError_t launch_advect(int scheme, const float* fld, const float* ux, const float* uy, float* out,
                          const StepConsts& c, cudaStream_t st);
cudaError_t launch_forcing_field(const float* theta, int theta_len, float t, float* f,
                                 const StepConsts& c, cudaStream_t st);

// ---------------------------------------------------------------- adjoint --
struct AdjointArgs {
  const float* lam = nullptr;    // (2,N,N) lambda_{s+1} (before projection), or nullptr (zero)
  const float* p = nullptr;      // (N,N) pressure of the pending adjoint projection, or nullptr
  const float* u = nullptr;      // (2,N,N) forward state u_s
  float* lam_out = nullptr;      // (2,N,N) lambda_s
  float* rhs = nullptr;          // (N,N) div(lambda_s)/dt
  double* gpart = nullptr;       // per-block partial theta sensitivities, [step][nblk][3]
  const float* theta = nullptr;
  int theta_len = 2;
  int step = 0;                  // forward step index s (forcing time t = s*dt)
  int gslot = 0;                 // row of gpart to write
  int scheme = 0;
  int tw = 64, th = 16;
  StepConsts c;
};
cudaError_t launch_adjoint_stencil(const AdjointArgs& a, cudaStream_t st);
// The adjoint step of `count` solves in one launch (blockIdx.z = solve): tab
// is a device table of their arguments; shape gives the launch shape, scheme
// and N, which all entries share.  Each solve's results are those of its own
// launch_adjoint_stencil.
cudaError_t launch_adjoint_batch(const AdjointArgs& shape, const AdjointArgs* tab, int count, cudaStream_t st);
// Adjoint shapes with tw >= NSGB_ROWS_MIN_W select the row-streaming adjoint
// kernel: bands of min(tw, N) columns (a power of two <= NSGB_ADJ_ROWS_MAX_W;
// its five input rings bound the band) by th rows.
constexpr int NSGB_ADJ_ROWS_MAX_W = 1024;
bool adjoint_rows_supported(int N, int tw, int th);
// rowsum: nrows x 3 doubles of scratch
cudaError_t launch_greduce(const double* gpart, int nblk, int nrows, double* rowsum, double* gacc,
                           cudaStream_t st);
cudaError_t launch_gfinal(const double* gacc, int theta_len, float* dJ, cudaStream_t st);

// ------------------------------------------------------------- optimiser --
// Constants of one optimiser update, float32 as the library rounds them;
// bc1/bc2 = 1 - b^t for the step count t of the launch.
struct OptimizerRule {
  int kind;
  float lr, b1, b2, one_minus_b1, one_minus_b2, bc1, bc2, eps, eps_root, decay, one_minus_decay;
};
cudaError_t launch_optimizer_update(const OptimizerRule& r, float* theta, const float* grad, float* mu, float* nu,
                                    float* theta_copy, int n, cudaStream_t st);

// Record the message nsgb_last_error() returns on this host thread.
void set_last_error(const char* msg);

// Raise `kernel`'s dynamic shared-memory limit to everything the current
// device allows beside its static shared memory.  Done once per (kernel,
// device) under a lock, and never lowered afterwards, so launches of the same
// kernel with different sizes from several host threads cannot race on the
// limit.
cudaError_t raise_smem_limit(const void* kernel);
// Bounds-checking build: a device range of the library's own (plan tables,
// static scratch) that kernels may access; no-op otherwise.
int bounds_add_library_range(const void* p, size_t bytes);
int bounds_remove_library_range(const void* p);
// The status an entry point returns after enqueueing its work: NSGB_OK, or
// in the bounds-checking build NSGB_ERR_BOUNDS when a kernel of the call
// accessed memory outside the valid ranges (it waits for the stream).
int finish_call(cudaStream_t st);
template <class K>
inline cudaError_t raise_smem_limit(K* kernel) {
  return raise_smem_limit(reinterpret_cast<const void*>(kernel));
}

}  // namespace nsgb
