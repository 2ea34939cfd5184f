// Fused stencil kernel of the Chorin step and the single operators of
// PeriodicDifferentialOps / AdvectionScheme.
//
// k_stencil processes one TH x TW tile of the grid per CTA (blockDim 32 x 8).
// It stages the pending pressure p with a 3-cell halo and the pending u* with
// a 2-cell halo in shared memory (periodic wrap by index masking), then
//   1. finishes the previous step's projection  u^n = u* - dt grad p
//      (NS_solver.py:696-697) on the tile + 2-cell halo,
//   2. accumulates the objective partial  sum u^n_x f_x  (NS_solver.py:746),
//   3. forms u*^{n+1} = u^n + dt (nu lap u^n + adv(u^n) + f)  on the tile +
//      1-cell halo (NS_solver.py:685-689, 249-265, 474-477),
//   4. writes u*^{n+1} and rhs = div(u*^{n+1}) / dt for the tile
//      (NS_solver.py:692-693, 206-210).
// The elementwise arithmetic keeps the reference's operation order with
// explicitly rounded intrinsics (no FMA contraction), so it rounds exactly
// like the reference's float32 array expressions.
#include "nsgb_internal.h"

namespace nsgb {

// 5-point Laplacian at centre o of a tile with row pitch W (NS_solver.py:249-255).
__device__ __forceinline__ float lap5(const float* s, int o, int W, const StepConsts& c) {
  const float f = s[o];
  const float left = s[o - W], right = s[o + W], up = s[o + 1], down = s[o - 1];
  return divc(fsub(fadd(fadd(fadd(left, right), up), down), fmul(4.0f, f)), c.dx2, c.rdx2);
}

// -(u . grad) field at centre o (NS_solver.py:474-477 central, :257-265 upwind).
template <int SCHEME>
__device__ __forceinline__ float adv5(const float* s, int o, int W, float ux, float uy,
                                      const StepConsts& c) {
  const float f = s[o];
  const float left = s[o - W], right = s[o + W], up = s[o + 1], down = s[o - 1];
  if (SCHEME == NSGB_SCHEME_CENTRAL) {
    const float gx = divc(fsub(right, left), c.h2, c.rh2);
    const float gy = divc(fsub(up, down), c.h2, c.rh2);
    return -fadd(fmul(ux, gx), fmul(uy, gy));
  } else {
    const float dfx = divc(ux >= 0.0f ? fsub(f, left) : fsub(right, f), c.h1, c.rh1);
    const float dfy = divc(uy >= 0.0f ? fsub(f, down) : fsub(up, f), c.h1, c.rh1);
    return -fadd(fmul(ux, dfx), fmul(uy, dfy));
  }
}

template <int SCHEME, int MODE, int TW, int TH>
__device__ __forceinline__ void stencil_body(const StencilArgs& a, int step_off = 0) {
  extern __shared__ float sm[];
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const int j0 = blockIdx.x * TW, i0 = blockIdx.y * TH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * 32 + tx;
  constexpr int PW = TW + 6, PH = TH + 6;
  constexpr int UW = TW + 4, UH = TH + 4;
  constexpr int SW = TW + 2, SH = TH + 2;
  float* sP = sm;
  float* sUx = sP + PH * PW;
  float* sUy = sUx + UH * UW;
  float* sSx = sUy + UH * UW;
  float* sSy = sSx + SH * SW;
  float* sF = sSy + SH * SW;
  float* sRed = sF + SH;

  int step = 0;
  float t = a.t_fixed;
  if (MODE == MODE_ROLLOUT) {
    step = (a.step_ctr ? *a.step_ctr : 0) + a.step_fixed + step_off;
    if (a.t_from_step) t = fmul((float)step, c.dt);
  }
  const float nu = (a.theta != nullptr && a.theta_len == 3) ? __ldg(a.theta + 2) : c.nu;

  // Tile loads: compile-time trip counts, so every load of a thread is in
  // flight before the first shared-memory store.
  const bool has_p = a.p != nullptr;
  if (has_p) {
    const float* __restrict__ pp = a.p;
    forflat<PH, PW>(tid, [&](int r, int cc) {
      sP[r * PW + cc] = __ldg(pp + (size_t)((i0 - 3 + r) & M) * N + ((j0 - 3 + cc) & M));
    });
  }
  {
    const float* __restrict__ us = a.us;
    forflat<UH, UW>(tid, [&](int r, int cc) {
      const size_t g = (size_t)((i0 - 2 + r) & M) * N + ((j0 - 2 + cc) & M);
      sUx[r * UW + cc] = __ldg(us + g);
      sUy[r * UW + cc] = __ldg(us + NN + g);
    });
  }
  if (MODE == MODE_ROLLOUT) {
    if (tid < SH) {
      const ForcingRow fr = forcing_time(__ldg(a.theta), __ldg(a.theta + 1), t, c);
      sF[tid] = forcing_fx((i0 - 1 + tid) & M, fr, c);
    }
  }
  __syncthreads();

  // 1. pending projection u^n = u* - dt * grad p
  if (has_p) {
    forflat<UH, UW>(tid, [&](int r, int cc) {
      const int op = (r + 1) * PW + (cc + 1);
      const float px = divc(fsub(sP[op + PW], sP[op - PW]), c.h2, c.rh2);
      const float py = divc(fsub(sP[op + 1], sP[op - 1]), c.h2, c.rh2);
      const int ou = r * UW + cc;
      sUx[ou] = fsub(sUx[ou], fmul(c.dt, px));
      sUy[ou] = fsub(sUy[ou], fmul(c.dt, py));
    });
    __syncthreads();
  }

  // 2. objective partial on the state before the step; optional state output
  float jacc = 0.0f;
  forflat<TH, TW>(tid, [&](int r, int cc) {
    const int ou = (r + 2) * UW + (cc + 2);
    if (MODE == MODE_ROLLOUT) jacc += sUx[ou] * sF[r + 1];
    if (a.u_out) {
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      a.u_out[g] = sUx[ou];
      a.u_out[NN + g] = sUy[ou];
    }
  });

  // 3. u*^{n+1} on the tile + 1 halo
  forflat<SH, SW>(tid, [&](int r, int cc) {
    const int o = (r + 1) * UW + (cc + 1);
    const float ux = sUx[o], uy = sUy[o];
    const float lapx = lap5(sUx, o, UW, c), lapy = lap5(sUy, o, UW, c);
    const float advx = adv5<SCHEME>(sUx, o, UW, ux, uy, c);
    const float advy = adv5<SCHEME>(sUy, o, UW, ux, uy, c);
    float fx, fy;
    if (MODE == MODE_ROLLOUT) {
      fx = sF[r];
      fy = 0.0f;
    } else {
      const size_t g = (size_t)((i0 - 1 + r) & M) * N + ((j0 - 1 + cc) & M);
      fx = __ldg(a.f + g);
      fy = __ldg(a.f + NN + g);
    }
    sSx[r * SW + cc] = fadd(ux, fmul(c.dt, fadd(fadd(fmul(nu, lapx), advx), fx)));
    sSy[r * SW + cc] = fadd(uy, fmul(c.dt, fadd(fadd(fmul(nu, lapy), advy), fy)));
  });
  __syncthreads();

  // 4. write u*^{n+1} and div(u*^{n+1}) / dt
  {
    float* __restrict__ uso = a.us_out;
    float* __restrict__ rhs = a.rhs;
    forflat<TH, TW>(tid, [&](int r, int cc) {
      const int o = (r + 1) * SW + (cc + 1);
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      uso[g] = sSx[o];
      uso[NN + g] = sSy[o];
      const float gx = divc(fsub(sSx[o + SW], sSx[o - SW]), c.h2, c.rh2);
      const float gy = divc(fsub(sSy[o + 1], sSy[o - 1]), c.h2, c.rh2);
      rhs[g] = divc(fadd(gx, gy), c.dt, c.rdt);
    });
  }

  if (MODE == MODE_ROLLOUT) {
    jacc = warp_sum(jacc);
    if (tx == 0) sRed[ty] = jacc;
    __syncthreads();
    if (ty == 0) {
      float v = (tx < 8) ? sRed[tx] : 0.0f;
      v = warp_sum(v);
      if (tx == 0 && (unsigned)step < (unsigned)a.jpart_rows) {
        const int nblk = gridDim.x * gridDim.y;
        a.jpart[(size_t)step * nblk + blockIdx.y * gridDim.x + blockIdx.x] = v;
      }
    }
  }
}

template <int SCHEME, int MODE, int TW, int TH>
__global__ void __launch_bounds__(256) k_stencil(const StencilArgs a) {
  stencil_body<SCHEME, MODE, TW, TH>(a);
}

// Ensemble variant: blockIdx.z selects the solve, `variant` its argument set.
template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_stencil_batch(const SolveDev* __restrict__ solves, int variant,
                                                      int step_off) {
  stencil_body<SCHEME, MODE_ROLLOUT, TW, TH>(solves[blockIdx.z].st[variant], step_off);
}

int stencil_nblocks(int N, int tw, int th) { return (N / tw) * (N / th); }

bool stencil_tile_supported(int tw, int th) {
#define NSGB_TILE_OK(W, H) if (tw == W && th == H) return true;
  NSGB_STENCIL_TILES(NSGB_TILE_OK)
#undef NSGB_TILE_OK
  return false;
}

static size_t stencil_smem(int tw, int th) {
  const size_t f = (size_t)(th + 6) * (tw + 6) + 2 * (size_t)(th + 4) * (tw + 4) +
                   2 * (size_t)(th + 2) * (tw + 2) + (th + 2) + 32;
  return f * sizeof(float);
}

template <int SCHEME, int MODE, int TW, int TH>
static cudaError_t launch_stencil_t(const StencilArgs& a, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_stencil<SCHEME, MODE, TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         160 * 1024);
    configured = true;
  }
  const dim3 grid(a.c.N / TW, a.c.N / TH);
  k_stencil<SCHEME, MODE, TW, TH><<<grid, dim3(32, 8), stencil_smem(TW, TH), st>>>(a);
  return cudaGetLastError();
}

template <int SCHEME, int TW, int TH>
static cudaError_t launch_stencil_batch_t(const SolveDev* solves, int count, int variant, int step_off, int N,
                                          cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_stencil_batch<SCHEME, TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         160 * 1024);
    configured = true;
  }
  const dim3 grid(N / TW, N / TH, count);
  k_stencil_batch<SCHEME, TW, TH><<<grid, dim3(32, 8), stencil_smem(TW, TH), st>>>(solves, variant, step_off);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_stencil_batch_s(const SolveDev* solves, int count, int variant, int step_off, int N,
                                          int tw, int th, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (tw == W && th == H) return launch_stencil_batch_t<SCHEME, W, H>(solves, count, variant, step_off, N, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_stencil_batch(const SolveDev* solves, int count, int variant, int step_off, int scheme, int N,
                                 int tw, int th, cudaStream_t st) {
  return scheme == NSGB_SCHEME_CENTRAL
             ? launch_stencil_batch_s<NSGB_SCHEME_CENTRAL>(solves, count, variant, step_off, N, tw, th, st)
             : launch_stencil_batch_s<NSGB_SCHEME_UPWIND>(solves, count, variant, step_off, N, tw, th, st);
}

template <int SCHEME, int MODE>
static cudaError_t launch_stencil_s(const StencilArgs& a, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (a.tw == W && a.th == H) return launch_stencil_t<SCHEME, MODE, W, H>(a, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_stencil(const StencilArgs& a, int mode, cudaStream_t st) {
  if (a.scheme == NSGB_SCHEME_CENTRAL) {
    return mode == MODE_ROLLOUT ? launch_stencil_s<NSGB_SCHEME_CENTRAL, MODE_ROLLOUT>(a, st)
                                : launch_stencil_s<NSGB_SCHEME_CENTRAL, MODE_FIELD>(a, st);
  }
  return mode == MODE_ROLLOUT ? launch_stencil_s<NSGB_SCHEME_UPWIND, MODE_ROLLOUT>(a, st)
                              : launch_stencil_s<NSGB_SCHEME_UPWIND, MODE_FIELD>(a, st);
}

// ------------------------------------------------------------ projection --
__global__ void k_project(const float* __restrict__ us, const float* __restrict__ p,
                          float* __restrict__ u, const StepConsts c) {
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  const int i = (int)(g >> c.logN), j = (int)(g & M);
  const float px = divc(fsub(__ldg(p + (size_t)((i + 1) & M) * N + j),
                             __ldg(p + (size_t)((i - 1) & M) * N + j)), c.h2, c.rh2);
  const float py = divc(fsub(__ldg(p + (size_t)i * N + ((j + 1) & M)),
                             __ldg(p + (size_t)i * N + ((j - 1) & M))), c.h2, c.rh2);
  u[g] = fsub(__ldg(us + g), fmul(c.dt, px));
  u[NN + g] = fsub(__ldg(us + NN + g), fmul(c.dt, py));
}

cudaError_t launch_project(const float* us, const float* p, float* u_out, const StepConsts& c,
                           cudaStream_t st) {
  const size_t NN = (size_t)c.N * c.N;
  k_project<<<(unsigned)((NN + 255) / 256), 256, 0, st>>>(us, p, u_out, c);
  return cudaGetLastError();
}

__global__ void k_project_batch(const SolveDev* __restrict__ solves, int variant) {
  const SolveDev& d = solves[blockIdx.y];
  const StencilArgs& a = d.st[variant];
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  const int i = (int)(g >> c.logN), j = (int)(g & M);
  const float* p = a.p;
  const float px = divc(fsub(__ldg(p + (size_t)((i + 1) & M) * N + j),
                             __ldg(p + (size_t)((i - 1) & M) * N + j)), c.h2, c.rh2);
  const float py = divc(fsub(__ldg(p + (size_t)i * N + ((j + 1) & M)),
                             __ldg(p + (size_t)i * N + ((j - 1) & M))), c.h2, c.rh2);
  d.u_final[g] = fsub(__ldg(a.us + g), fmul(c.dt, px));
  d.u_final[NN + g] = fsub(__ldg(a.us + NN + g), fmul(c.dt, py));
}

// Projection of the final state of every solve: `variant` names the argument
// set whose (us, p) hold the pending u* and pressure.
cudaError_t launch_project_batch(const SolveDev* solves, int count, int variant, int N, cudaStream_t st) {
  const size_t NN = (size_t)N * N;
  k_project_batch<<<dim3((unsigned)((NN + 255) / 256), count), 256, 0, st>>>(solves, variant);
  return cudaGetLastError();
}

// ----------------------------------------------------------- J reduction --
// One CTA per step: fixed-order sum of that step's block partials.
__global__ void k_jreduce(const float* __restrict__ jpart, int nblk, double* __restrict__ jsteps) {
  __shared__ double red[256];
  const float* row = jpart + (size_t)blockIdx.x * nblk;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += (double)row[b];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) jsteps[blockIdx.x] = red[0];
}

__global__ void k_jfinal(const double* __restrict__ jsteps, int steps, double jscale,
                         float* __restrict__ J) {
  double acc = 0.0;
  for (int s = 0; s < steps; ++s) acc += jsteps[s] * jscale;
  *J = (float)acc;
}

cudaError_t launch_jreduce(const float* jpart, int nblk, int steps, double* jsteps, float* J,
                           double jscale, cudaStream_t st) {
  if (steps > 0) k_jreduce<<<steps, 256, 0, st>>>(jpart, nblk, jsteps);
  k_jfinal<<<1, 1, 0, st>>>(jsteps, steps, jscale, J);
  return cudaGetLastError();
}

__global__ void k_jreduce_batch(const SolveDev* __restrict__ solves, int nblk) {
  __shared__ double red[256];
  const SolveDev& d = solves[blockIdx.y];
  const float* row = d.st[1].jpart + (size_t)blockIdx.x * nblk;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += (double)row[b];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) d.jsteps[blockIdx.x] = red[0];
}

__global__ void k_jfinal_batch(const SolveDev* __restrict__ solves, int count, int steps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const SolveDev& d = solves[k];
  double acc = 0.0;
  for (int s = 0; s < steps; ++s) acc += d.jsteps[s] * d.jscale;
  *d.J = (float)acc;
}

cudaError_t launch_jreduce_batch(const SolveDev* solves, int count, int nblk, int steps, cudaStream_t st) {
  if (steps > 0) k_jreduce_batch<<<dim3(steps, count), 256, 0, st>>>(solves, nblk);
  k_jfinal_batch<<<(count + 127) / 128, 128, 0, st>>>(solves, count, steps);
  return cudaGetLastError();
}

__global__ void k_counter_batch(const SolveDev* __restrict__ solves, int count, int value, int add) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  int* ctr = solves[k].ctr;
  *ctr = add ? *ctr + value : solves[k].ctr_init + value;
}

cudaError_t launch_counter_batch(const SolveDev* solves, int count, int value, bool add, cudaStream_t st) {
  k_counter_batch<<<(count + 127) / 128, 128, 0, st>>>(solves, count, value, add ? 1 : 0);
  return cudaGetLastError();
}

__global__ void k_step_counter(int* ctr, int value, int add) { *ctr = add ? *ctr + value : value; }
cudaError_t launch_step_counter(int* step_ctr, int value, bool add, cudaStream_t st) {
  k_step_counter<<<1, 1, 0, st>>>(step_ctr, value, add ? 1 : 0);
  return cudaGetLastError();
}

// ------------------------------------------------------- single operators --
__device__ __forceinline__ void ij_of(size_t g, const StepConsts& c, int& i, int& j) {
  i = (int)(g >> c.logN);
  j = (int)(g & (c.N - 1));
}

__global__ void k_grad(const float* __restrict__ f, float* __restrict__ gx, float* __restrict__ gy,
                       const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  gx[g] = divc(fsub(f[(size_t)((i + 1) & M) * N + j], f[(size_t)((i - 1) & M) * N + j]), c.h2, c.rh2);
  gy[g] = divc(fsub(f[(size_t)i * N + ((j + 1) & M)], f[(size_t)i * N + ((j - 1) & M)]), c.h2, c.rh2);
}

__global__ void k_laplacian(const float* __restrict__ f, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float left = f[(size_t)((i - 1) & M) * N + j], right = f[(size_t)((i + 1) & M) * N + j];
  const float up = f[(size_t)i * N + ((j + 1) & M)], down = f[(size_t)i * N + ((j - 1) & M)];
  out[g] = divc(fsub(fadd(fadd(fadd(left, right), up), down), fmul(4.0f, f[g])), c.dx2, c.rdx2);
}

__global__ void k_divergence(const float* __restrict__ u, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float* uy = u + NN;
  const float gx = divc(fsub(u[(size_t)((i + 1) & M) * N + j], u[(size_t)((i - 1) & M) * N + j]), c.h2, c.rh2);
  const float gy = divc(fsub(uy[(size_t)i * N + ((j + 1) & M)], uy[(size_t)i * N + ((j - 1) & M)]), c.h2, c.rh2);
  out[g] = fadd(gx, gy);
}

template <int SCHEME>
__global__ void k_advect(const float* __restrict__ fld, const float* __restrict__ ux,
                         const float* __restrict__ uy, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float f = fld[g];
  const float left = fld[(size_t)((i - 1) & M) * N + j], right = fld[(size_t)((i + 1) & M) * N + j];
  const float up = fld[(size_t)i * N + ((j + 1) & M)], down = fld[(size_t)i * N + ((j - 1) & M)];
  const float vx = ux[g], vy = uy[g];
  if (SCHEME == NSGB_SCHEME_CENTRAL) {
    const float gx = divc(fsub(right, left), c.h2, c.rh2);
    const float gy = divc(fsub(up, down), c.h2, c.rh2);
    out[g] = -fadd(fmul(vx, gx), fmul(vy, gy));
  } else {
    const float dfx = divc(vx >= 0.0f ? fsub(f, left) : fsub(right, f), c.h1, c.rh1);
    const float dfy = divc(vy >= 0.0f ? fsub(f, down) : fsub(up, f), c.h1, c.rh1);
    out[g] = -fadd(fmul(vx, dfx), fmul(vy, dfy));
  }
}

__global__ void k_forcing_field(const float* __restrict__ theta, float t, float* __restrict__ f,
                                const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const ForcingRow fr = forcing_time(__ldg(theta), __ldg(theta + 1), t, c);
  f[g] = forcing_fx(i, fr, c);
  f[NN + g] = 0.0f;
}

static unsigned nb(const StepConsts& c) { return (unsigned)(((size_t)c.N * c.N + 255) / 256); }

cudaError_t launch_grad(const float* f, float* gx, float* gy, const StepConsts& c, cudaStream_t st) {
  k_grad<<<nb(c), 256, 0, st>>>(f, gx, gy, c);
  return cudaGetLastError();
}
cudaError_t launch_laplacian(const float* f, float* out, const StepConsts& c, cudaStream_t st) {
  k_laplacian<<<nb(c), 256, 0, st>>>(f, out, c);
  return cudaGetLastError();
}
cudaError_t launch_divergence(const float* u, float* out, const StepConsts& c, cudaStream_t st) {
  k_divergence<<<nb(c), 256, 0, st>>>(u, out, c);
  return cudaGetLastError();
}
cudaError_t launch_advect(int scheme, const float* fld, const float* ux, const float* uy, float* out,
                          const StepConsts& c, cudaStream_t st) {
  if (scheme == NSGB_SCHEME_CENTRAL)
    k_advect<NSGB_SCHEME_CENTRAL><<<nb(c), 256, 0, st>>>(fld, ux, uy, out, c);
  else
    k_advect<NSGB_SCHEME_UPWIND><<<nb(c), 256, 0, st>>>(fld, ux, uy, out, c);
  return cudaGetLastError();
}
cudaError_t launch_forcing_field(const float* theta, int theta_len, float t, float* f,
                                 const StepConsts& c, cudaStream_t st) {
  (void)theta_len;
  k_forcing_field<<<nb(c), 256, 0, st>>>(theta, t, f, c);
  return cudaGetLastError();
}

}  // namespace nsgb
