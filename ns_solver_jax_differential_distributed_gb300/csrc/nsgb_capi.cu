// C ABI of the GB300 Chorin-projection solver (declarations in include/nsgb.h).
//
// The host side owns no field memory: callers pass device pointers and a
// workspace of the size the *_workspace_bytes queries return.  A plan holds
// the per-N constant tables and the launch shapes, and caches instantiated
// CUDA graphs of rollout chunks.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "nsgb_internal.h"

using namespace nsgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(NSGB_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define NSGB_CUDA(call)                                  \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}
size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

struct GraphEntry {
  const void* ws = nullptr;
  const float* theta = nullptr;
  int theta_len = 0;
  int chunk = 0;
  StepConsts c{};
  int scheme = 0;
  int tiles[4] = {0, 0, 0, 0};
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

struct nsgb_plan {
  int N = 0, logN = 0;
  double L = 1.0;
  int device = 0;
  float2* tw = nullptr;
  float* k2 = nullptr;
  int tile_w = 64, tile_h = 16, rows_per_cta = 8, cols_per_cta = 2;
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  std::vector<GraphEntry> graphs;
  std::mutex mu;
};

namespace {

void default_tiles(int N, int out[4]) {
  const int T = N / (N < 16 ? N : 16);
  out[0] = N < 64 ? N : 64;
  out[1] = N < 16 ? N : 16;
  int rows;
  if (N >= 2048) rows = 8;
  else if (N >= 512) rows = 2;
  else if (N >= 128) rows = 4;
  else rows = 8;
  if (rows > N) rows = N;
  out[2] = rows;
  int kb = 512 / T;
  if (kb < 1) kb = 1;
  if (N >= 512 && N <= 1024) kb = 2;
  if (kb > N / 2) kb = N / 2;
  out[3] = kb;
}

int check_tiles(int N, int tw, int th, int rows, int cols) {
  const int T = N / (N < 16 ? N : 16);
  if (!is_pow2(tw) || tw < 16 || tw > 128 || tw > N)
    return fail(NSGB_ERR_INVALID_ARG, "stencil tile width %d must be a power of two in [16, min(128, N)]", tw);
  if (!is_pow2(th) || th < 2 || th > 32 || th > N)
    return fail(NSGB_ERR_INVALID_ARG, "stencil tile height %d must be a power of two in [2, min(32, N)]", th);
  if (!is_pow2(rows) || rows < 2 || rows > N || (rows / 2) * T > 1024 ||
      fft_rows_smem_bytes(N, rows) > 200 * 1024)
    return fail(NSGB_ERR_INVALID_ARG, "rows_per_cta %d invalid for N=%d", rows, N);
  if (!is_pow2(cols) || cols > N / 2 || cols * T > 512 || fft_cols_smem_bytes(N, cols) > 200 * 1024)
    return fail(NSGB_ERR_INVALID_ARG, "cols_per_cta %d invalid for N=%d", cols, N);
  return NSGB_OK;
}

int check_plan(const nsgb_plan* plan) {
  if (!plan) return fail(NSGB_ERR_INVALID_ARG, "plan is NULL");
  return NSGB_OK;
}

int check_phys(const nsgb_phys* ph) {
  if (!ph) return fail(NSGB_ERR_INVALID_ARG, "phys is NULL");
  if (!(std::isfinite(ph->dt) && ph->dt > 0)) return fail(NSGB_ERR_INVALID_ARG, "dt must be positive and finite");
  if (!std::isfinite(ph->nu)) return fail(NSGB_ERR_INVALID_ARG, "nu must be finite");
  if (!(std::isfinite(ph->L) && ph->L > 0)) return fail(NSGB_ERR_INVALID_ARG, "L must be positive and finite");
  if (ph->scheme != NSGB_SCHEME_CENTRAL && ph->scheme != NSGB_SCHEME_UPWIND)
    return fail(NSGB_ERR_INVALID_ARG, "unknown advection scheme %d", ph->scheme);
  return NSGB_OK;
}

// Constants as float32, the way the reference's Python scalars enter its
// float32 expressions (dx, 2*dx and dx**2 are computed in double first).
StepConsts make_consts(const nsgb_plan* plan, const nsgb_phys* ph) {
  StepConsts c{};
  const double dx = plan->L / plan->N;
  c.N = plan->N;
  c.logN = plan->logN;
  c.L = (float)plan->L;
  c.h1 = (float)dx;
  c.h2 = (float)(2 * dx);
  c.dx2 = (float)(dx * dx);
  c.dt = ph ? (float)ph->dt : 1.0f;
  c.nu = ph ? (float)ph->nu : 0.0f;
  c.mu0 = ph ? (float)ph->mu0 : 0.5f;
  c.sigma0 = ph ? (float)ph->sigma0 : 0.1f;
  c.C = ph ? (float)ph->C : 1.0f;
  c.jscale = ph ? (float)(ph->dt * dx * dx) : 0.0f;
  return c;
}

FftLaunch fft_launch(const nsgb_plan* plan, const float* rhs, void* spec, float* p) {
  FftLaunch L;
  L.rhs = rhs;
  L.spec = (float2*)spec;
  L.do_cols = true;
  L.p = p;
  L.tw = plan->tw;
  L.k2 = plan->k2;
  L.scale = (float)(1.0 / (2.0 * (double)plan->N * (double)plan->N));
  L.rows_per_cta = plan->rows_per_cta;
  L.cols_per_cta = plan->cols_per_cta;
  return L;
}

StencilArgs stencil_args(const nsgb_plan* plan, const nsgb_phys* ph) {
  StencilArgs a;
  a.c = make_consts(plan, ph);
  a.scheme = ph ? ph->scheme : 0;
  a.tw = plan->tile_w;
  a.th = plan->tile_h;
  return a;
}

// Workspace carving helper.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base((char*)b) {}
  template <class T>
  T* take(size_t count) {
    T* p = base ? (T*)(base + off) : nullptr;
    off += align_up(count * sizeof(T));
    return p;
  }
};

struct RolloutWs {
  float *usA, *usB, *p, *rhs, *spec, *jpart;
  double* jsteps;
  int* ctr;
  size_t bytes;
};

RolloutWs carve_rollout(const nsgb_plan* plan, int steps, void* ws) {
  const size_t NN = (size_t)plan->N * plan->N;
  const int nblk = stencil_nblocks(plan->N, plan->tile_w, plan->tile_h);
  Carver cv(ws);
  RolloutWs w;
  w.usA = cv.take<float>(2 * NN);
  w.usB = cv.take<float>(2 * NN);
  w.p = cv.take<float>(NN);
  w.rhs = cv.take<float>(NN);
  w.spec = cv.take<float>(NN);
  w.jpart = cv.take<float>((size_t)(steps > 0 ? steps : 1) * nblk);
  w.jsteps = cv.take<double>(steps > 0 ? steps : 1);
  w.ctr = cv.take<int>(1);
  w.bytes = cv.off;
  return w;
}

struct GradWs {
  RolloutWs f;
  float *ckpt, *ustore, *lamA, *lamB, *padj, *gpart;
  double* gacc;
  size_t bytes;
};

GradWs carve_grad(const nsgb_plan* plan, int steps, int every, void* ws) {
  const size_t NN = (size_t)plan->N * plan->N;
  const int nblk = stencil_nblocks(plan->N, plan->tile_w, plan->tile_h);
  GradWs g;
  g.f = carve_rollout(plan, steps, ws);
  Carver cv(ws);
  cv.off = g.f.bytes;
  const int ncp = (steps + every - 1) / every;
  g.ckpt = cv.take<float>((size_t)(ncp > 0 ? ncp : 1) * 2 * NN);
  g.ustore = cv.take<float>((size_t)every * 2 * NN);
  g.lamA = cv.take<float>(2 * NN);
  g.lamB = cv.take<float>(2 * NN);
  g.padj = cv.take<float>(NN);
  g.gpart = cv.take<float>((size_t)every * nblk * 3);
  g.gacc = cv.take<double>(4);
  g.bytes = cv.off;
  return g;
}

int check_ws(void* ws, size_t have, size_t need) {
  if (!ws) return fail(NSGB_ERR_WORKSPACE, "workspace is NULL (need %zu bytes)", need);
  if (have < need) return fail(NSGB_ERR_WORKSPACE, "workspace too small: %zu < %zu bytes", have, need);
  if (((uintptr_t)ws & 255) != 0) return fail(NSGB_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  return NSGB_OK;
}

int check_theta(const float* theta, int theta_len) {
  if (!theta) return fail(NSGB_ERR_INVALID_ARG, "theta is NULL");
  if (theta_len != 2 && theta_len != 3)
    return fail(NSGB_ERR_INVALID_ARG, "theta must have 2 or 3 entries, got %d", theta_len);
  return NSGB_OK;
}

// One forward step of a rollout: stencil (with the pending projection) then
// the FFT-Poisson solve of its rhs into p.
cudaError_t rollout_step(const nsgb_plan* plan, StencilArgs a, const float* us_in, const float* p_in,
                         float* us_out, const RolloutWs& w, int step_fixed, const int* ctr,
                         float* u_out, bool do_fft, cudaStream_t st) {
  a.us = us_in;
  a.p = p_in;
  a.us_out = us_out;
  a.rhs = w.rhs;
  a.u_out = u_out;
  a.jpart = w.jpart;
  a.step_ctr = ctr;
  a.step_fixed = step_fixed;
  a.t_from_step = 1;
  cudaError_t e = launch_stencil(a, MODE_ROLLOUT, st);
  if (e != cudaSuccess || !do_fft) return e;
  return poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, w.p), st);
}

}  // namespace

// ============================================================== C ABI ====
extern "C" {

int nsgb_version(void) { return 10000; }

const char* nsgb_last_error(void) { return g_last_error.c_str(); }

int nsgb_plan_create(int N, double L, nsgb_plan** out) {
  if (!out) return fail(NSGB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!is_pow2(N) || N < 16 || N > 4096)
    return fail(NSGB_ERR_UNSUPPORTED_N, "N=%d unsupported: power of two in [16, 4096] required", N);
  if (!(std::isfinite(L) && L > 0)) return fail(NSGB_ERR_INVALID_ARG, "L must be positive and finite");
  nsgb_plan* p = new nsgb_plan();
  p->N = N;
  p->logN = ilog2(N);
  p->L = L;
  cudaGetDevice(&p->device);
  int t[4];
  default_tiles(N, t);
  p->tile_w = t[0];
  p->tile_h = t[1];
  p->rows_per_cta = t[2];
  p->cols_per_cta = t[3];

  std::vector<float2> tw(N);
  for (int m = 0; m < N; ++m) {
    const double ang = -2.0 * M_PI * (double)m / (double)N;
    tw[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  // k = 2 pi fftfreq(N, dx) in float32 as NS_solver.py:518-519 evaluates it:
  // (m / float32(dx*N)) * 2 * float32(pi), then squared in float32.
  std::vector<float> k2(N);
  const double dx = L / N;
  const float dn = (float)(dx * N);
  for (int m = 0; m < N; ++m) {
    const int mm = m < N / 2 ? m : m - N;
    volatile float k = (float)mm / dn;
    k = k * 2.0f;
    k = k * (float)M_PI;
    volatile float kk = k * k;
    k2[m] = kk;
  }
  cudaError_t e = cudaMalloc(&p->tw, N * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&p->k2, N * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(p->tw, tw.data(), N * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->k2, k2.data(), N * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->tw);
    cudaFree(p->k2);
    delete p;
    return fail(e == cudaErrorMemoryAllocation ? NSGB_ERR_OOM : NSGB_ERR_CUDA, "plan set-up: %s",
                cudaGetErrorString(e));
  }
  *out = p;
  return NSGB_OK;
}

int nsgb_plan_destroy(nsgb_plan* plan) {
  if (!plan) return NSGB_OK;
  for (auto& g : plan->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (plan->graph_stream) cudaStreamDestroy(plan->graph_stream);
  if (plan->ev_in) cudaEventDestroy(plan->ev_in);
  if (plan->ev_out) cudaEventDestroy(plan->ev_out);
  cudaFree(plan->tw);
  cudaFree(plan->k2);
  delete plan;
  return NSGB_OK;
}

int nsgb_plan_set_tiles(nsgb_plan* plan, int tw, int th, int rows, int cols) {
  if (int r = check_plan(plan)) return r;
  tw = tw ? tw : plan->tile_w;
  th = th ? th : plan->tile_h;
  rows = rows ? rows : plan->rows_per_cta;
  cols = cols ? cols : plan->cols_per_cta;
  if (int r = check_tiles(plan->N, tw, th, rows, cols)) return r;
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->tile_w = tw;
  plan->tile_h = th;
  plan->rows_per_cta = rows;
  plan->cols_per_cta = cols;
  return NSGB_OK;
}

int nsgb_plan_get_tiles(const nsgb_plan* plan, int out[4]) {
  if (int r = check_plan(plan)) return r;
  if (!out) return fail(NSGB_ERR_INVALID_ARG, "out is NULL");
  out[0] = plan->tile_w;
  out[1] = plan->tile_h;
  out[2] = plan->rows_per_cta;
  out[3] = plan->cols_per_cta;
  return NSGB_OK;
}

size_t nsgb_poisson_workspace_bytes(const nsgb_plan* plan) {
  return plan ? align_up((size_t)plan->N * plan->N * sizeof(float)) : 0;
}

size_t nsgb_step_workspace_bytes(const nsgb_plan* plan) {
  return plan ? carve_rollout(plan, 1, nullptr).bytes : 0;
}

size_t nsgb_rollout_workspace_bytes(const nsgb_plan* plan, int steps) {
  return plan ? carve_rollout(plan, steps, nullptr).bytes : 0;
}

size_t nsgb_rollout_grad_workspace_bytes(const nsgb_plan* plan, int steps, int every) {
  if (!plan || every <= 0) return 0;
  return carve_grad(plan, steps, every, nullptr).bytes;
}

int nsgb_grad(const nsgb_plan* plan, const float* f, float* gx, float* gy, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!f || !gx || !gy) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_grad(f, gx, gy, make_consts(plan, nullptr), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_laplacian(const nsgb_plan* plan, const float* f, float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!f || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_laplacian(f, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_divergence(const nsgb_plan* plan, const float* u, float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!u || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_divergence(u, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_advect(const nsgb_plan* plan, int scheme, const float* field, const float* ux, const float* uy,
                float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (scheme != NSGB_SCHEME_CENTRAL && scheme != NSGB_SCHEME_UPWIND)
    return fail(NSGB_ERR_INVALID_ARG, "unknown advection scheme %d", scheme);
  if (!field || !ux || !uy || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_advect(scheme, field, ux, uy, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_poisson(const nsgb_plan* plan, const float* rhs, float* p, void* workspace, size_t ws_bytes,
                 void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!rhs || !p) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (int r = check_ws(workspace, ws_bytes, nsgb_poisson_workspace_bytes(plan))) return r;
  NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, rhs, workspace, p), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_forcing(const nsgb_plan* plan, const nsgb_phys* phys, const float* theta, int theta_len, float t,
                 float* f_out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!f_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_forcing_field(theta, theta_len, t, f_out, make_consts(plan, phys), (cudaStream_t)stream));
  return NSGB_OK;
}

int nsgb_projector_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u, const float* f,
                        float* u_out, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (!u || !f || !u_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  RolloutWs w = carve_rollout(plan, 1, nullptr);
  if (int r = check_ws(workspace, ws_bytes, w.bytes)) return r;
  w = carve_rollout(plan, 1, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  StencilArgs a = stencil_args(plan, phys);
  a.us = u;
  a.p = nullptr;
  a.f = f;
  a.us_out = w.usA;
  a.rhs = w.rhs;
  a.t_from_step = 0;
  NSGB_CUDA(launch_stencil(a, MODE_FIELD, st));
  NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, w.p), st));
  NSGB_CUDA(launch_project(w.usA, w.p, u_out, a.c, st));
  return NSGB_OK;
}

int nsgb_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u, const float* theta, int theta_len,
              float t, float* u_out, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u || !u_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  RolloutWs w = carve_rollout(plan, 1, nullptr);
  if (int r = check_ws(workspace, ws_bytes, w.bytes)) return r;
  w = carve_rollout(plan, 1, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  StencilArgs a = stencil_args(plan, phys);
  a.us = u;
  a.p = nullptr;
  a.us_out = w.usA;
  a.rhs = w.rhs;
  a.jpart = w.jpart;
  a.theta = theta;
  a.theta_len = theta_len;
  a.step_fixed = 0;
  a.t_from_step = 0;
  a.t_fixed = t;
  NSGB_CUDA(launch_stencil(a, MODE_ROLLOUT, st));
  NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, w.p), st));
  NSGB_CUDA(launch_project(w.usA, w.p, u_out, a.c, st));
  return NSGB_OK;
}

int nsgb_rollout(const nsgb_plan* plan_c, const nsgb_phys* phys, const float* u0, const float* theta,
                 int theta_len, int steps, float* u_final, float* J, void* workspace, size_t ws_bytes,
                 int use_graph, void* stream) {
  nsgb_plan* plan = const_cast<nsgb_plan*>(plan_c);
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u0 || !u_final || !J) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (steps < 0) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 0");
  const size_t need = carve_rollout(plan, steps, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  RolloutWs w = carve_rollout(plan, steps, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t NN = (size_t)plan->N * plan->N;
  StencilArgs a = stencil_args(plan, phys);
  a.theta = theta;
  a.theta_len = theta_len;
  const int nblk = stencil_nblocks(plan->N, a.tw, a.th);

  if (steps == 0) {
    NSGB_CUDA(cudaMemcpyAsync(u_final, u0, 2 * NN * sizeof(float), cudaMemcpyDeviceToDevice, st));
    NSGB_CUDA(launch_jreduce(w.jpart, nblk, 0, w.jsteps, J, 0.0, st));
    return NSGB_OK;
  }

  // step 0 reads u0 directly; later steps ping-pong usA <-> usB.
  NSGB_CUDA(rollout_step(plan, a, u0, nullptr, w.usA, w, 0, nullptr, nullptr, true, st));
  int s = 1;
  const float* cur = w.usA;
  const int K = 16;  // steps per graph chunk (even: a chunk starts and ends in usA)
  if (use_graph && steps - 1 >= 2 * K) {
    std::lock_guard<std::mutex> lk(plan->mu);
    GraphEntry* ge = nullptr;
    for (auto& g : plan->graphs) {
      if (g.ws == workspace && g.theta == theta && g.theta_len == theta_len && g.chunk == K &&
          g.scheme == a.scheme && std::memcmp(&g.c, &a.c, sizeof(StepConsts)) == 0 &&
          g.tiles[0] == plan->tile_w && g.tiles[1] == plan->tile_h && g.tiles[2] == plan->rows_per_cta &&
          g.tiles[3] == plan->cols_per_cta) {
        ge = &g;
        break;
      }
    }
    if (!plan->graph_stream) {
      NSGB_CUDA(cudaStreamCreateWithFlags(&plan->graph_stream, cudaStreamNonBlocking));
      NSGB_CUDA(cudaEventCreateWithFlags(&plan->ev_in, cudaEventDisableTiming));
      NSGB_CUDA(cudaEventCreateWithFlags(&plan->ev_out, cudaEventDisableTiming));
    }
    if (!ge) {
      if (plan->graphs.size() >= 8) {
        cudaGraphExecDestroy(plan->graphs.front().exec);
        plan->graphs.erase(plan->graphs.begin());
      }
      cudaGraph_t graph;
      cudaStream_t gs = plan->graph_stream;
      NSGB_CUDA(cudaStreamBeginCapture(gs, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = cudaSuccess;
      for (int k = 0; k < K && ce == cudaSuccess; ++k) {
        const float* in = (k % 2 == 0) ? w.usA : w.usB;
        float* out = (k % 2 == 0) ? w.usB : w.usA;
        ce = rollout_step(plan, a, in, w.p, out, w, k, w.ctr, nullptr, true, gs);
      }
      if (ce == cudaSuccess) ce = launch_step_counter(w.ctr, K, true, gs);
      cudaError_t ee = cudaStreamEndCapture(gs, &graph);
      if (ce != cudaSuccess) return cuda_fail(ce, "rollout graph capture");
      if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
      GraphEntry g;
      g.ws = workspace;
      g.theta = theta;
      g.theta_len = theta_len;
      g.chunk = K;
      g.c = a.c;
      g.scheme = a.scheme;
      g.tiles[0] = plan->tile_w;
      g.tiles[1] = plan->tile_h;
      g.tiles[2] = plan->rows_per_cta;
      g.tiles[3] = plan->cols_per_cta;
      cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
      plan->graphs.push_back(g);
      ge = &plan->graphs.back();
    }
    // The chunk graph reads its first step index from w.ctr and advances it
    // by K in its last node, so one instantiated graph serves every chunk.
    NSGB_CUDA(cudaEventRecord(plan->ev_in, st));
    NSGB_CUDA(cudaStreamWaitEvent(plan->graph_stream, plan->ev_in, 0));
    NSGB_CUDA(launch_step_counter(w.ctr, s, false, plan->graph_stream));
    while (steps - s >= K) {
      NSGB_CUDA(cudaGraphLaunch(ge->exec, plan->graph_stream));
      s += K;
    }
    NSGB_CUDA(cudaEventRecord(plan->ev_out, plan->graph_stream));
    NSGB_CUDA(cudaStreamWaitEvent(st, plan->ev_out, 0));
    cur = w.usA;
  }
  for (; s < steps; ++s) {
    const float* in = cur;
    float* out = (in == w.usA) ? w.usB : w.usA;
    NSGB_CUDA(rollout_step(plan, a, in, w.p, out, w, s, nullptr, nullptr, true, st));
    cur = out;
  }
  NSGB_CUDA(launch_project(cur, w.p, u_final, a.c, st));
  NSGB_CUDA(launch_jreduce(w.jpart, nblk, steps, w.jsteps, J, (double)phys->dt * (plan->L / plan->N) *
                                                                  (plan->L / plan->N), st));
  return NSGB_OK;
}

int nsgb_rollout_grad(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                      int theta_len, int steps, int every, int phases, float* J, float* u_final,
                      float* dJdtheta, float* dJdu0, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u0) return fail(NSGB_ERR_INVALID_ARG, "u0 is NULL");
  if (steps < 1) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 1");
  if (every < 1) return fail(NSGB_ERR_INVALID_ARG, "checkpoint interval must be >= 1");
  if (phases < 1 || phases > 3) return fail(NSGB_ERR_INVALID_ARG, "phases must be 1, 2 or 3");
  if ((phases & NSGB_GRAD_FORWARD) && !J) return fail(NSGB_ERR_INVALID_ARG, "J is NULL");
  if ((phases & NSGB_GRAD_BACKWARD) && !dJdtheta) return fail(NSGB_ERR_INVALID_ARG, "dJdtheta is NULL");
  const size_t need = carve_grad(plan, steps, every, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  GradWs g = carve_grad(plan, steps, every, workspace);
  const RolloutWs& w = g.f;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t NN = (size_t)plan->N * plan->N;
  StencilArgs a = stencil_args(plan, phys);
  a.theta = theta;
  a.theta_len = theta_len;
  const int nblk = stencil_nblocks(plan->N, a.tw, a.th);
  const double dx = plan->L / plan->N;

  if (phases & NSGB_GRAD_FORWARD) {
    // Forward rollout: checkpoint u_s every `every` steps, objective, u_final.
    const float* cur = u0;
    const float* curp = nullptr;
    for (int s = 0; s < steps; ++s) {
      float* out = (s % 2 == 0) ? w.usA : w.usB;
      float* ck = (s % every == 0) ? g.ckpt + (size_t)(s / every) * 2 * NN : nullptr;
      NSGB_CUDA(rollout_step(plan, a, cur, curp, out, w, s, nullptr, ck, true, st));
      cur = out;
      curp = w.p;
    }
    if (u_final) NSGB_CUDA(launch_project(cur, w.p, u_final, a.c, st));
    NSGB_CUDA(launch_jreduce(w.jpart, nblk, steps, w.jsteps, J, (double)phys->dt * dx * dx, st));
  }
  if (!(phases & NSGB_GRAD_BACKWARD)) return NSGB_OK;

  // Backward: segments in reverse; recompute each segment's states from its
  // checkpoint, then run the adjoint steps backwards through them.
  NSGB_CUDA(cudaMemsetAsync(g.gacc, 0, 4 * sizeof(double), st));
  AdjointArgs b;
  b.c = a.c;
  b.scheme = a.scheme;
  b.tw = a.tw;
  b.th = a.th;
  b.theta = theta;
  b.theta_len = theta_len;
  b.gpart = g.gpart;
  b.rhs = w.rhs;
  const float* lam = nullptr;  // lambda_S = 0
  bool have_padj = false;
  const int nseg = (steps + every - 1) / every;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * every, s1 = std::min(steps, s0 + every);
    const float* rc = g.ckpt + (size_t)seg * 2 * NN;
    const float* rp = nullptr;
    for (int s = s0; s < s1; ++s) {
      float* out = ((s - s0) % 2 == 0) ? w.usA : w.usB;
      NSGB_CUDA(rollout_step(plan, a, rc, rp, out, w, s, nullptr, g.ustore + (size_t)(s - s0) * 2 * NN,
                             s + 1 < s1, st));
      rc = out;
      rp = w.p;
    }
    for (int s = s1 - 1; s >= s0; --s) {
      float* lam_out = (s == 0 && dJdu0) ? dJdu0 : ((lam == g.lamA) ? g.lamB : g.lamA);
      b.lam = lam;
      b.p = have_padj ? g.padj : nullptr;
      b.u = g.ustore + (size_t)(s - s0) * 2 * NN;
      b.lam_out = lam_out;
      b.step = s;
      b.gslot = s - s0;
      NSGB_CUDA(launch_adjoint_stencil(b, st));
      if (s > 0) {
        NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, g.padj), st));
        have_padj = true;
      }
      lam = lam_out;
    }
    NSGB_CUDA(launch_greduce(g.gpart, nblk, s1 - s0, g.gacc, st));
  }
  NSGB_CUDA(launch_gfinal(g.gacc, theta_len, dJdtheta, st));
  return NSGB_OK;
}

}  // extern "C"
