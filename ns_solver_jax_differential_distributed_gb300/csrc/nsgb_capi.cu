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
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "nsgb_fft.cuh"
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
// Transposed half spectrum: N/2 + 1 rows of N complex values.
size_t spec_floats(int N) { return (size_t)(N / 2 + 1) * N * 2; }

struct GraphEntry {
  const void* ws = nullptr;
  int steps = 0;
  const float* theta = nullptr;
  int theta_len = 0;
  int chunk = 0;
  StepConsts c{};
  int scheme = 0;
  int tiles[7] = {0, 0, 0, 0, 0, 0, 0};
  cudaGraphExec_t exec = nullptr;
};

// Everything a gradient call's enqueued work depends on (pointers are read at
// replay, so a graph of the call replays it for the same arguments).
struct GradKey {
  const void* ws;
  const float *u0, *theta;
  float *J, *u_final, *dJdtheta, *dJdu0;
  int theta_len, steps, every, phases, scheme;
  int tiles[8];
  StepConsts c;
};
// compared with memcmp: no padding bytes
static_assert(sizeof(GradKey) == 7 * sizeof(void*) + 13 * sizeof(int) + sizeof(StepConsts), "GradKey padding");

}  // namespace

struct nsgb_plan {
  int N = 0, logN = 0;
  double L = 1.0;
  int device = 0;
  float2* tw = nullptr;
  float* k2 = nullptr;
  int tile_w = 64, tile_h = 16, rows_per_cta = 8, cols_per_cta = 2;
  int adj_w = 64, adj_h = 16;  // tiled-kernel shape of the adjoint stencil
  int radix_rows = 16, radix_cols = 16;  // Stockham radix of the FFT passes
  int fused_rows = 0;  // row band of the fused row kernel (0: the four-kernel step)
  cudaStream_t graph_stream = nullptr;  // private stream graphs are captured on
  std::vector<GraphEntry> graphs;
  // gradient calls: the last call's arguments, and graphs of calls repeated
  // with identical arguments
  GradKey last_grad{};
  std::vector<std::pair<GradKey, cudaGraphExec_t>> grad_graphs;
  std::mutex mu;
};

namespace {

// Launch shapes measured best on GB300 by the autotuner (see autotune.py);
// the autotuner refines them per process.
void default_tiles(int N, int out[4]) {
  tile_kernel_default(N, out[0], out[1]);
  int rows = N >= 1024 ? 4 : (N >= 256 ? 8 : 16);
  if (rows > N) rows = N;
  out[2] = rows;
  int kb = N >= 1024 ? 1 : 4;
  if (kb > N / 2) kb = N / 2;
  out[3] = kb;
}

int check_tiles(int N, int tw, int th, int rows, int cols, int radix_rows, int radix_cols) {
  const int Tr = N / (N < radix_rows ? N : radix_rows);
  const int Tc = N / (N < radix_cols ? N : radix_cols);
  if (stencil_rows_mode(tw)) {
    if (!stencil_rows_supported(N, tw, th))
      return fail(NSGB_ERR_INVALID_ARG,
                  "row-streaming stencil needs a power-of-two band width in [%d, %d] and 1 <= rows <= N "
                  "(got %dx%d, N=%d)", NSGB_ROWS_MIN_W, NSGB_ROWS_MAX_W, tw, th, N);
  } else if (!stencil_tile_supported(tw, th) || tw > N || th > N) {
    return fail(NSGB_ERR_INVALID_ARG, "stencil tile %dx%d is not an instantiated shape for N=%d", tw, th, N);
  }
  if (!is_pow2(rows) || rows < 2 || rows > N || (rows / 2) * Tr > 1024 ||
      fft_rows_smem_bytes(N, rows) > 200 * 1024)
    return fail(NSGB_ERR_INVALID_ARG, "rows_per_cta %d invalid for N=%d (radix %d)", rows, N, radix_rows);
  if (!is_pow2(cols) || cols > N / 2 || cols * Tc > 512 || fft_cols_smem_bytes(N, cols) > 200 * 1024)
    return fail(NSGB_ERR_INVALID_ARG, "cols_per_cta %d invalid for N=%d (radix %d)", cols, N, radix_cols);
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

// Correctly rounded float reciprocal of d: the float nearest 1/d, chosen among
// the neighbours of float(1/d) by the exact (double) residual |r*d - 1|.
float recip_rn(float d) {
  float r = (float)(1.0 / (double)d);
  float best = r;
  double err = std::fabs((double)r * (double)d - 1.0);
  for (float c : {std::nextafter(r, -INFINITY), std::nextafter(r, INFINITY)}) {
    const double e = std::fabs((double)c * (double)d - 1.0);
    if (e < err) {
      err = e;
      best = c;
    }
  }
  return best;
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
  c.rh1 = recip_rn(c.h1);
  c.rh2 = recip_rn(c.h2);
  c.rdx2 = recip_rn(c.dx2);
  c.rdt = recip_rn(c.dt);
  c.cP = (float)((double)c.dt / c.h2);
  c.cD = (float)(1.0 / ((double)c.h2 * c.dt));
  c.cAc = (float)((double)c.dt / c.h2);
  c.cAu = (float)((double)c.dt / c.h1);
  c.dtdx2 = (float)((double)c.dt / c.dx2);
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
  L.radix_rows = plan->radix_rows;
  L.radix_cols = plan->radix_cols;
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
  float *usA, *usB, *p, *rhs, *spec, *spec2, *jpart;
  double* jsteps;
  int* ctr;
  int steps;  // rows of jpart
  size_t bytes;
};

// Objective partials per step of a rollout: one per CTA of its stencil
// launches (the fused row kernel's grid when the plan uses it).
int rollout_nblk(const nsgb_plan* plan) {
  return plan->fused_rows > 0 ? fused_nblocks(plan->N, plan->fused_rows)
                              : stencil_nblocks(plan->N, plan->tile_w, plan->tile_h);
}

RolloutWs carve_rollout(const nsgb_plan* plan, int steps, void* ws) {
  const size_t NN = (size_t)plan->N * plan->N;
  // rows of partials wide enough for either grid: every caller indexes them
  // with the block count of the kernels it launches
  const int nblk = std::max(stencil_nblocks(plan->N, plan->tile_w, plan->tile_h),
                            plan->fused_rows > 0 ? fused_nblocks(plan->N, plan->fused_rows) : 0);
  Carver cv(ws);
  RolloutWs w;
  // Buffers that captured graphs reference come first, at offsets that do
  // not depend on `steps`.
  w.ctr = cv.take<int>(1);
  w.usA = cv.take<float>(2 * NN);
  w.usB = cv.take<float>(2 * NN);
  w.p = cv.take<float>(NN);
  w.rhs = cv.take<float>(NN);
  w.spec = cv.take<float>(spec_floats(plan->N));
  w.spec2 = cv.take<float>(spec_floats(plan->N));
  w.jpart = cv.take<float>((size_t)(steps > 0 ? steps : 1) * nblk);
  w.jsteps = cv.take<double>(steps > 0 ? steps : 1);
  w.steps = steps > 0 ? steps : 1;
  w.bytes = cv.off;
  return w;
}

struct GradWs {
  RolloutWs f;
  float *ckpt, *ustore, *lamA, *lamB, *padj;
  double *gpart, *growsum, *gacc;
  size_t bytes;
};

// Rows of per-block theta partials (one row per adjoint step) reduced into
// the double accumulator by one launch: the summation order is the same for
// every checkpoint interval.
constexpr int kGradRows = 64;

GradWs carve_grad(const nsgb_plan* plan, int steps, int every, void* ws) {
  const size_t NN = (size_t)plan->N * plan->N;
  const int nblk = stencil_nblocks(plan->N, plan->adj_w, plan->adj_h);  // adjoint blocks
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
  g.gpart = cv.take<double>((size_t)kGradRows * nblk * 3);
  g.growsum = cv.take<double>((size_t)kGradRows * 3);
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

// The stencil kernels read fields as aligned float4 groups.
int check_field(const float* f, const char* name) {
  if (!f) return fail(NSGB_ERR_INVALID_ARG, "%s is NULL", name);
  if (((uintptr_t)f & 15) != 0) return fail(NSGB_ERR_INVALID_ARG, "%s must be 16-byte aligned", name);
  return NSGB_OK;
}

// Calls that upload their argument tables from host memory that does not
// outlive them refuse a capturing stream: a captured copy would read that
// memory again at every replay.
int refuse_capture(cudaStream_t st, const char* fn) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
  if (cap != cudaStreamCaptureStatusNone)
    return fail(NSGB_ERR_INVALID_ARG, "%s does not run on a capturing stream (it uploads tables from host memory)", fn);
  return NSGB_OK;
}

int check_theta(const float* theta, int theta_len) {
  if (!theta) return fail(NSGB_ERR_INVALID_ARG, "theta is NULL");
  if (theta_len != 2 && theta_len != 3)
    return fail(NSGB_ERR_INVALID_ARG, "theta must have 2 or 3 entries, got %d", theta_len);
  return NSGB_OK;
}


// ------------------------------------------------------------- ensembles --
// Variant of the argument set that performs step s of a member (see SolveDev).
inline int variant_of(int s) { return s == 0 ? 0 : ((s & 1) ? 1 : 2); }

struct EnsGroup {
  const nsgb_plan* plan;
  int scheme;
  int first, count;  // range in the member table
  int done, todo;    // progress of the group's first member (parity shared)
};

struct EnsLayout {
  size_t tab_off = 0, fin_off = 0, bytes = 0;
  std::vector<size_t> state_off;  // per member: offset of a carved state, or SIZE_MAX
};

EnsLayout ensemble_layout(const nsgb_member* m, int count) {
  EnsLayout L;
  size_t off = 0;
  L.tab_off = off;
  off += align_up(sizeof(SolveDev) * (size_t)count);
  L.fin_off = off;
  off += align_up(sizeof(SolveDev) * (size_t)count);
  L.state_off.assign(count, (size_t)-1);
  for (int k = 0; k < count; ++k) {
    if (m[k].state) continue;
    L.state_off[k] = off;
    off += align_up(carve_rollout(m[k].plan, m[k].total_steps, nullptr).bytes);
  }
  L.bytes = off;
  return L;
}

SolveDev make_solvedev(const nsgb_member& m, void* state) {
  RolloutWs w = carve_rollout(m.plan, m.total_steps, state);
  StencilArgs a = stencil_args(m.plan, &m.phys);
  a.theta = m.theta;
  a.theta_len = m.theta_len;
  a.jpart = w.jpart;
  a.jpart_rows = w.steps;
  a.rhs = w.rhs;
  a.step_ctr = w.ctr;
  a.step_fixed = 0;
  a.t_from_step = 1;
  SolveDev d;
  d.st[0] = a;
  d.st[0].us = m.u0;
  d.st[0].p = nullptr;
  d.st[0].us_out = w.usA;
  d.st[1] = a;
  d.st[1].us = w.usA;
  d.st[1].p = w.p;
  d.st[1].us_out = w.usB;
  d.st[2] = a;
  d.st[2].us = w.usB;
  d.st[2].p = w.p;
  d.st[2].us_out = w.usA;
  d.fft = {w.rhs, (float2*)w.spec, w.p};
  d.u_final = m.u_final;
  d.J = m.J;
  d.jsteps = w.jsteps;
  const double dx = m.plan->L / m.plan->N;
  d.jscale = m.phys.dt * dx * dx;
  d.ctr = w.ctr;
  d.ctr_init = m.done_steps;
  return d;
}

int check_members(const nsgb_member* members, int count, bool need_state_size) {
  if (!members || count <= 0) return fail(NSGB_ERR_INVALID_ARG, "empty ensemble");
  for (int i = 0; i < count; ++i) {
    const nsgb_member& m = members[i];
    if (!m.plan) return fail(NSGB_ERR_INVALID_ARG, "member %d: plan is NULL", i);
    if (int r = check_phys(&m.phys)) return r;
    if (std::fabs(m.phys.L - m.plan->L) > 1e-12 * m.plan->L)
      return fail(NSGB_ERR_INVALID_ARG, "member %d: phys.L differs from its plan's L", i);
    if (int r = check_theta(m.theta, m.theta_len)) return r;
    if (!m.u0 || !m.u_final || !m.J) return fail(NSGB_ERR_INVALID_ARG, "member %d: NULL pointer", i);
    if (int r = check_field(m.u0, "member u0")) return r;
    if (m.total_steps < 1) return fail(NSGB_ERR_INVALID_ARG, "member %d: total_steps must be >= 1", i);
    if (m.done_steps < 0 || m.done_steps > m.total_steps)
      return fail(NSGB_ERR_INVALID_ARG, "member %d: done_steps out of range", i);
    if (m.state && ((uintptr_t)m.state & 255))
      return fail(NSGB_ERR_WORKSPACE, "member %d: state must be 256-byte aligned", i);
  }
  (void)need_state_size;
  return NSGB_OK;
}

struct EnsGraph {
  const void* ws;
  int count, chunk;
  uint64_t sig;
  cudaGraphExec_t exec;
};
std::mutex g_ens_mu;
std::vector<EnsGraph> g_ens_graphs;
// Streams and events an ensemble chunk graph is captured with, per device
// (the capture stream and up to 8 branch streams; the fork event and one join
// event per branch).  Replays run on the caller's stream.
struct EnsPool {
  cudaStream_t s[9] = {};
  cudaEvent_t e[9] = {};
};
std::map<int, EnsPool> g_ens_pools;

// The pool of the current device, creating what is missing (a failed creation
// leaves the rest for the next call to retry).
int ens_pool(EnsPool*& out) {
  int dev = 0;
  NSGB_CUDA(cudaGetDevice(&dev));
  EnsPool& p = g_ens_pools[dev];
  for (auto& x : p.s)
    if (!x) NSGB_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  for (auto& x : p.e)
    if (!x) NSGB_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
  out = &p;
  return NSGB_OK;
}

// Eager fork/join of independent groups of batched launches: the groups'
// kernels go to branch streams that start after the caller's stream's work so
// far and that the caller's stream waits for at the join, so groups of
// different N overlap on the device.  One pool per device; the lock is held
// while a call enqueues (the events are reused).
class Branches {
 public:
  static constexpr int kMax = 8;
  // Forks n (1..kMax) branches off st; with n == 1 everything stays on st.
  // The branch count is set only once the pool exists, so a failure while
  // creating it leaves a one-branch object whose destructor joins nothing.
  int open(cudaStream_t st, int n) {
    st_ = st;
    n = std::max(1, std::min(n, kMax));
    if (n == 1) return NSGB_OK;
    int dev = 0;
    NSGB_CUDA(cudaGetDevice(&dev));
    lk_ = std::unique_lock<std::mutex>(mu());
    Pool& p = pools()[dev];
    if (!p.ready) {
      for (auto& x : p.s)
        if (!x) NSGB_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
      if (!p.fork) NSGB_CUDA(cudaEventCreateWithFlags(&p.fork, cudaEventDisableTiming));
      for (auto& x : p.join)
        if (!x) NSGB_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
      p.ready = true;
    }
    pool_ = &p;
    NSGB_CUDA(cudaEventRecord(p.fork, st));
    n_ = n;  // from here on the destructor joins every branch
    for (int b = 0; b < n_; ++b) NSGB_CUDA(cudaStreamWaitEvent(p.s[b], p.fork, 0));
    return NSGB_OK;
  }
  cudaStream_t stream(int group) const { return n_ == 1 ? st_ : pool_->s[group % n_]; }
  std::vector<cudaStream_t> streams() const {
    std::vector<cudaStream_t> v;
    for (int b = 0; b < n_; ++b) v.push_back(stream(b));
    return v;
  }
  int close() {
    if (n_ == 1) return NSGB_OK;
    for (int b = 0; b < n_; ++b) {
      NSGB_CUDA(cudaEventRecord(pool_->join[b], pool_->s[b]));
      NSGB_CUDA(cudaStreamWaitEvent(st_, pool_->join[b], 0));
    }
    n_ = 1;
    lk_ = std::unique_lock<std::mutex>();
    return NSGB_OK;
  }
  // A call that returns early with an error still joins what it enqueued, so
  // later work on the caller's stream never overtakes it.
  ~Branches() {
    if (n_ == 1 || !pool_) return;
    for (int b = 0; b < n_; ++b)
      if (cudaEventRecord(pool_->join[b], pool_->s[b]) == cudaSuccess) cudaStreamWaitEvent(st_, pool_->join[b], 0);
  }

 private:
  struct Pool {
    bool ready = false;
    cudaStream_t s[kMax] = {};
    cudaEvent_t fork = nullptr, join[kMax] = {};
  };
  static std::mutex& mu() {
    static std::mutex m;
    return m;
  }
  static std::map<int, Pool>& pools() {
    static std::map<int, Pool> p;
    return p;
  }
  cudaStream_t st_ = nullptr;
  int n_ = 1;
  Pool* pool_ = nullptr;
  std::unique_lock<std::mutex> lk_;
};

uint64_t fnv(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char* c = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

// One solver step (step `done + k`) of each group, on the group's stream.
cudaError_t ensemble_step(const std::vector<EnsGroup>& groups, const SolveDev* dev, int k,
                          const std::vector<cudaStream_t>& gs) {
  for (size_t g = 0; g < groups.size(); ++g) {
    const EnsGroup& G = groups[g];
    if (k >= G.todo) continue;
    const SolveDev* d = dev + G.first;
    cudaStream_t st = gs[g % gs.size()];
    cudaError_t e = launch_stencil_batch(d, G.count, variant_of(G.done + k), k, G.scheme, G.plan->N,
                                         G.plan->tile_w, G.plan->tile_h, st);
    if (e != cudaSuccess) return e;
    e = poisson_fft_batch(G.plan->N, fft_launch(G.plan, nullptr, nullptr, nullptr), d, G.count, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Sort members into groups; fills `order` (table position -> member index).
std::vector<EnsGroup> make_groups(const nsgb_member* m, int count, int steps, std::vector<int>& order) {
  auto todo = [&](int i) { return std::min(steps, m[i].total_steps - m[i].done_steps); };
  auto dk = [&](int i) { return m[i].done_steps == 0 ? 2 : (m[i].done_steps & 1); };
  order.resize(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (m[a].plan->N != m[b].plan->N) return m[a].plan->N < m[b].plan->N;
    if (m[a].plan != m[b].plan) return m[a].plan < m[b].plan;
    if (m[a].phys.scheme != m[b].phys.scheme) return m[a].phys.scheme < m[b].phys.scheme;
    if (dk(a) != dk(b)) return dk(a) < dk(b);
    return todo(a) < todo(b);
  });
  std::vector<EnsGroup> groups;
  for (int k = 0; k < count; ++k) {
    const int i = order[k];
    const nsgb_member& x = m[i];
    bool same = !groups.empty();
    if (same) {
      const nsgb_member& y = m[order[groups.back().first]];
      same = y.plan == x.plan && y.phys.scheme == x.phys.scheme && dk(order[groups.back().first]) == dk(i) &&
             groups.back().todo == todo(i);
    }
    if (!same) groups.push_back({x.plan, x.phys.scheme, k, 0, x.done_steps, todo(i)});
    groups.back().count++;
  }
  return groups;
}

// Final projection and objective of the members that finish in this call.
// persistent: the objective partials follow the persistent launch's tiling
// instead of the plans' stencil shapes.
cudaError_t ensemble_finalize(const nsgb_member* m, const std::vector<int>& order, const std::vector<SolveDev>& tab,
                              int steps, SolveDev* fin_dev, cudaStream_t st, bool persistent = false) {
  std::vector<int> fin;
  for (size_t k = 0; k < order.size(); ++k) {
    const nsgb_member& x = m[order[k]];
    if (x.done_steps + std::min(steps, x.total_steps - x.done_steps) == x.total_steps) fin.push_back((int)k);
  }
  if (fin.empty()) return cudaSuccess;
  std::stable_sort(fin.begin(), fin.end(), [&](int a, int b) {
    const nsgb_member &x = m[order[a]], &y = m[order[b]];
    if (x.plan != y.plan) return x.plan < y.plan;
    if (variant_of(x.total_steps) != variant_of(y.total_steps))
      return variant_of(x.total_steps) < variant_of(y.total_steps);
    return x.total_steps < y.total_steps;
  });
  std::vector<SolveDev> ft(fin.size());
  for (size_t k = 0; k < fin.size(); ++k) ft[k] = tab[fin[k]];
  cudaError_t e = cudaMemcpyAsync(fin_dev, ft.data(), sizeof(SolveDev) * ft.size(), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  size_t a = 0;
  while (a < fin.size()) {
    const nsgb_member& x = m[order[fin[a]]];
    size_t b = a + 1;
    while (b < fin.size()) {
      const nsgb_member& y = m[order[fin[b]]];
      if (y.plan != x.plan || variant_of(y.total_steps) != variant_of(x.total_steps) ||
          y.total_steps != x.total_steps)
        break;
      ++b;
    }
    const int n = (int)(b - a);
    e = launch_project_batch(fin_dev + a, n, variant_of(x.total_steps), x.plan->N, st);
    int tw = x.plan->tile_w, th = x.plan->tile_h;
    if (persistent) pers_tile(x.plan->N, tw, th);
    if (e == cudaSuccess) e = launch_jreduce_batch(fin_dev + a, n, stencil_nblocks(x.plan->N, tw, th), x.total_steps, st);
    if (e != cudaSuccess) return e;
    a = b;
  }
  return cudaSuccess;
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
  a.jpart_rows = w.steps;
  a.step_ctr = ctr;
  a.step_fixed = step_fixed;
  a.t_from_step = 1;
  cudaError_t e = launch_stencil(a, MODE_ROLLOUT, st);
  if (e != cudaSuccess || !do_fft) return e;
  return poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, w.p), st);
}

// Band width of the fused row kernel: whole rows up to 2048 columns, else
// 2048-column slices (one CTA of a cluster each).
int fused_width(int N) { return N / fused_cluster(N); }

// The row passes that bracket a fused rollout (the first step's forward rows,
// the last step's inverse rows) use radix 16 like the fused kernel, so every
// transform of the rollout rounds the same way.
FftLaunch fused_fft_launch(const nsgb_plan* plan, const float* rhs, void* spec, float* p) {
  FftLaunch L = fft_launch(plan, rhs, spec, p);
  L.radix_rows = 16;
  return L;
}

// One forward step in the fused form: the fused row kernel (inverse row FFT
// of spec_in into p on chip, the stencil with the pending projection, forward
// row FFT of its rhs into spec_out), then the column pass on spec_out.
cudaError_t fused_step(const nsgb_plan* plan, const StencilArgs& a, const float* us_in, const float* spec_in,
                       float* us_out, float* spec_out, const RolloutWs& w, int step_fixed, const int* ctr,
                       cudaStream_t st) {
  FusedArgs f;
  f.a = a;
  f.a.us = us_in;
  f.a.p = nullptr;
  f.a.us_out = us_out;
  f.a.rhs = nullptr;
  f.a.u_out = nullptr;
  f.a.jpart = w.jpart;
  f.a.jpart_rows = w.steps;
  f.a.step_ctr = ctr;
  f.a.step_fixed = step_fixed;
  f.a.t_from_step = 1;
  f.a.th = plan->fused_rows;
  f.spec_in = (const float2*)spec_in;
  f.spec_out = (float2*)spec_out;
  f.tw = plan->tw;  // radix-16 tables first
  cudaError_t e = launch_fused_rows(f, st);
  if (e != cudaSuccess) return e;
  return poisson_fft(plan->N, fused_fft_launch(plan, nullptr, spec_out, nullptr), st);
}

}  // namespace

void nsgb::set_last_error(const char* msg) { g_last_error = msg; }

// ------------------------------------------------------ bounds checking --
// The bounds-checking build keeps the valid device ranges -- the library's
// own (plan tables, the no-allocation scratch) and the caller's
// (nsgb_bounds_register) -- and uploads them to every translation unit's
// table whenever they change, after the device has finished the work that
// reads the old table.  Every entry point that enqueues work ends with
// finish_call: it waits for its stream and turns recorded out-of-range
// accesses into NSGB_ERR_BOUNDS.
#ifdef NSGB_CHECK_BOUNDS
namespace nsgb {
cudaError_t bounds_upload_stencil(const bounds::Table& t);
cudaError_t bounds_upload_fft(const bounds::Table& t);
cudaError_t bounds_upload_adjoint(const bounds::Table& t);
cudaError_t bounds_upload_fused(const bounds::Table& t);
cudaError_t bounds_upload_optim(const bounds::Table& t);
cudaError_t bounds_upload_persistent(const bounds::Table& t);
}  // namespace nsgb
namespace {
std::mutex g_bounds_mu;
std::vector<std::pair<unsigned long long, unsigned long long>> g_bounds_lib, g_bounds_caller;
unsigned long long* g_bounds_report = nullptr;

int bounds_upload_locked() {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "bounds table update");
  if (!g_bounds_report) {
    if ((e = cudaMalloc(&g_bounds_report, 4 * sizeof(unsigned long long))) != cudaSuccess)
      return cuda_fail(e, "bounds report");
    if ((e = cudaMemset(g_bounds_report, 0, 4 * sizeof(unsigned long long))) != cudaSuccess)
      return cuda_fail(e, "bounds report");
  }
  bounds::Table t{};
  for (const auto* v : {&g_bounds_lib, &g_bounds_caller})
    for (const auto& r : *v) {
      if (t.n == bounds::kMaxRanges) return fail(NSGB_ERR_INVALID_ARG, "more than %d checked ranges", bounds::kMaxRanges);
      t.lo[t.n] = r.first;
      t.hi[t.n] = r.second;
      ++t.n;
    }
  t.report = g_bounds_report;
  for (auto up : {bounds_upload_stencil, bounds_upload_fft, bounds_upload_adjoint, bounds_upload_fused,
                  bounds_upload_optim, bounds_upload_persistent})
    if ((e = up(t)) != cudaSuccess) return cuda_fail(e, "bounds table upload");
  return NSGB_OK;
}

int bounds_add(std::vector<std::pair<unsigned long long, unsigned long long>>& v, const void* p, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_bounds_mu);
  const unsigned long long a = (unsigned long long)p;
  v.emplace_back(a, a + bytes);
  return bounds_upload_locked();
}
int bounds_remove(std::vector<std::pair<unsigned long long, unsigned long long>>& v, const void* p) {
  std::lock_guard<std::mutex> lk(g_bounds_mu);
  const unsigned long long a = (unsigned long long)p;
  for (size_t k = 0; k < v.size(); ++k)
    if (v[k].first == a) {
      v.erase(v.begin() + k);
      return bounds_upload_locked();
    }
  return NSGB_OK;
}
}  // namespace
#endif

int nsgb::bounds_add_library_range(const void* p, size_t bytes) {
#ifdef NSGB_CHECK_BOUNDS
  return bounds_add(g_bounds_lib, p, bytes);
#else
  (void)p;
  (void)bytes;
  return NSGB_OK;
#endif
}

int nsgb::bounds_remove_library_range(const void* p) {
#ifdef NSGB_CHECK_BOUNDS
  return bounds_remove(g_bounds_lib, p);
#else
  (void)p;
  return NSGB_OK;
#endif
}

int nsgb::finish_call(cudaStream_t st) {
#ifdef NSGB_CHECK_BOUNDS
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
  if (cap != cudaStreamCaptureStatusNone) return NSGB_OK;  // checked when the graph is launched eagerly
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "bounds check: stream");
  unsigned long long r[4] = {0, 0, 0, 0};
  std::lock_guard<std::mutex> lk(g_bounds_mu);
  if (!g_bounds_report) return NSGB_OK;
  if ((e = cudaMemcpy(r, g_bounds_report, sizeof r, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail(e, "bounds report");
  if (r[0] == 0) return NSGB_OK;
  if ((e = cudaMemset(g_bounds_report, 0, sizeof r)) != cudaSuccess) return cuda_fail(e, "bounds report");
  return fail(NSGB_ERR_BOUNDS,
              "out-of-range device access: %llu access(es) outside the valid ranges, the first at address 0x%llx "
              "(%llu bytes) from translation unit %llu, source line %llu",
              r[0], r[1], r[3], r[2] / 100000ull, r[2] % 100000ull);
#else
  (void)st;
  return NSGB_OK;
#endif
}

cudaError_t nsgb::raise_smem_limit(const void* kernel) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, cudaError_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(kernel, dev);
  const auto it = done.find(key);
  if (it != done.end()) return it->second;
  int optin = 0;
  cudaFuncAttributes fa;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) done[key] = e;  // failures are retried on the next launch
  return e;
}

// ============================================================== C ABI ====
extern "C" {

int nsgb_version(void) { return 10000; }

const char* nsgb_last_error(void) { return g_last_error.c_str(); }

int nsgb_bounds_checking(void) {
#ifdef NSGB_CHECK_BOUNDS
  return 1;
#else
  return 0;
#endif
}

int nsgb_bounds_register(const void* base, size_t bytes) {
  if (!base || bytes == 0) return fail(NSGB_ERR_INVALID_ARG, "bounds range is empty");
#ifdef NSGB_CHECK_BOUNDS
  return bounds_add(g_bounds_caller, base, bytes);
#else
  return NSGB_OK;
#endif
}

int nsgb_bounds_unregister(const void* base) {
#ifdef NSGB_CHECK_BOUNDS
  return bounds_remove(g_bounds_caller, base);
#else
  (void)base;
  return NSGB_OK;
#endif
}

int nsgb_bounds_clear(void) {
#ifdef NSGB_CHECK_BOUNDS
  std::lock_guard<std::mutex> lk(g_bounds_mu);
  g_bounds_caller.clear();
  return bounds_upload_locked();
#else
  return NSGB_OK;
#endif
}

int nsgb_plan_create(int N, double L, nsgb_plan** out) {
  if (!out) return fail(NSGB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!is_pow2(N) || N < 16 || N > NSGB_MAX_N)
    return fail(NSGB_ERR_UNSUPPORTED_N, "N=%d unsupported: power of two in [16, %d] required", N, NSGB_MAX_N);
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
  tile_kernel_default(N, p->adj_w, p->adj_h);
  if (N >= 1024) {
    // the row-streaming adjoint: bands of 1024 columns, rows for about two
    // CTAs per SM (measured faster than the tiles from N = 1024 on)
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    const int col_bands = N / NSGB_ADJ_ROWS_MAX_W;
    const int row_bands = (2 * sms + col_bands - 1) / col_bands;
    p->adj_w = NSGB_ADJ_ROWS_MAX_W;
    p->adj_h = std::max(8, (N + row_bands - 1) / row_bands);
  }
  p->rows_per_cta = t[2];
  p->cols_per_cta = t[3];

  // Per-pass twiddle tables of the Stockham FFT, radix 16 then radix 8
  // (layout in nsgb_fft.cuh).
  const int ntw = nsgb::fft::tw_total(N);
  std::vector<float2> tw(ntw);
  nsgb::fft::host_twiddles(N, tw.data());
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
  cudaError_t e = cudaMalloc(&p->tw, ntw * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&p->k2, N * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(p->tw, tw.data(), ntw * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->k2, k2.data(), N * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->tw);
    cudaFree(p->k2);
    delete p;
    return fail(e == cudaErrorMemoryAllocation ? NSGB_ERR_OOM : NSGB_ERR_CUDA, "plan set-up: %s",
                cudaGetErrorString(e));
  }
  if (int r = bounds_add_library_range(p->tw, ntw * sizeof(float2))) return r;
  if (int r = bounds_add_library_range(p->k2, N * sizeof(float))) return r;
  *out = p;
  return NSGB_OK;
}

int nsgb_plan_destroy(nsgb_plan* plan) {
  if (!plan) return NSGB_OK;
  for (auto& g : plan->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  for (auto& g : plan->grad_graphs) cudaGraphExecDestroy(g.second);
  if (plan->graph_stream) cudaStreamDestroy(plan->graph_stream);
  bounds_remove_library_range(plan->tw);
  bounds_remove_library_range(plan->k2);
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
  if (int r = check_tiles(plan->N, tw, th, rows, cols, plan->radix_rows, plan->radix_cols)) return r;
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->tile_w = tw;
  plan->tile_h = th;
  if (!stencil_rows_mode(tw)) {
    plan->adj_w = tw;
    plan->adj_h = th;
  }
  plan->rows_per_cta = rows;
  plan->cols_per_cta = cols;
  return NSGB_OK;
}

int nsgb_plan_set_fft_radix(nsgb_plan* plan, int radix_rows, int radix_cols) {
  if (int r = check_plan(plan)) return r;
  radix_rows = radix_rows ? radix_rows : plan->radix_rows;
  radix_cols = radix_cols ? radix_cols : plan->radix_cols;
  if ((radix_rows != 8 && radix_rows != 16) || (radix_cols != 8 && radix_cols != 16))
    return fail(NSGB_ERR_INVALID_ARG, "FFT radix must be 8 or 16 (got %d, %d)", radix_rows, radix_cols);
  if (int r = check_tiles(plan->N, plan->tile_w, plan->tile_h, plan->rows_per_cta, plan->cols_per_cta,
                          radix_rows, radix_cols))
    return r;
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->radix_rows = radix_rows;
  plan->radix_cols = radix_cols;
  return NSGB_OK;
}

int nsgb_plan_get_fft_radix(const nsgb_plan* plan, int out[2]) {
  if (int r = check_plan(plan)) return r;
  if (!out) return fail(NSGB_ERR_INVALID_ARG, "out is NULL");
  out[0] = plan->radix_rows;
  out[1] = plan->radix_cols;
  return NSGB_OK;
}

int nsgb_plan_set_adjoint_tiles(nsgb_plan* plan, int tw, int th) {
  if (int r = check_plan(plan)) return r;
  tw = tw ? tw : plan->adj_w;
  th = th ? th : plan->adj_h;
  if (stencil_rows_mode(tw) ? !adjoint_rows_supported(plan->N, tw, th)
                            : (!stencil_tile_supported(tw, th) || tw > plan->N || th > plan->N))
    return fail(NSGB_ERR_INVALID_ARG,
                "adjoint shape %dx%d invalid for N=%d: a tiled-kernel shape, or a row band of power-of-two "
                "width in [%d, %d] and 1 <= rows <= N", tw, th, plan->N, NSGB_ROWS_MIN_W, NSGB_ADJ_ROWS_MAX_W);
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->adj_w = tw;
  plan->adj_h = th;
  return NSGB_OK;
}

int nsgb_plan_get_adjoint_tiles(const nsgb_plan* plan, int out[2]) {
  if (int r = check_plan(plan)) return r;
  if (!out) return fail(NSGB_ERR_INVALID_ARG, "out is NULL");
  out[0] = plan->adj_w;
  out[1] = plan->adj_h;
  return NSGB_OK;
}

int nsgb_plan_set_fused(nsgb_plan* plan, int rows) {
  if (int r = check_plan(plan)) return r;
  if (rows == 0) {
    std::lock_guard<std::mutex> lk(plan->mu);
    plan->fused_rows = 0;
    return NSGB_OK;
  }
  if (!fused_supported(plan->N))
    return fail(NSGB_ERR_UNSUPPORTED_N, "the fused row kernel supports N in {1024, 2048, 4096} (N=%d)", plan->N);
  if (rows < 0) {
    const cudaError_t e = fused_default_rows(plan->N, rows);
    if (e != cudaSuccess) return cuda_fail(e, "fused kernel occupancy");
  }
  if (rows < 2 || (rows & 1) || rows > plan->N)
    return fail(NSGB_ERR_INVALID_ARG, "fused row band must be even and in [2, N] (got %d)", rows);
  if (!stencil_rows_supported(plan->N, fused_width(plan->N), rows))
    return fail(NSGB_ERR_INVALID_ARG, "fused row band %d not supported for N=%d", rows, plan->N);
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->fused_rows = rows;
  return NSGB_OK;
}

int nsgb_plan_get_fused(const nsgb_plan* plan, int* rows) {
  if (int r = check_plan(plan)) return r;
  if (!rows) return fail(NSGB_ERR_INVALID_ARG, "rows is NULL");
  *rows = plan->fused_rows;
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
  return plan ? align_up(spec_floats(plan->N) * sizeof(float)) : 0;
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
  return finish_call((cudaStream_t)stream);
}

int nsgb_laplacian(const nsgb_plan* plan, const float* f, float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!f || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_laplacian(f, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return finish_call((cudaStream_t)stream);
}

int nsgb_divergence(const nsgb_plan* plan, const float* u, float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!u || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_divergence(u, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return finish_call((cudaStream_t)stream);
}

int nsgb_advect(const nsgb_plan* plan, int scheme, const float* field, const float* ux, const float* uy,
                float* out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (scheme != NSGB_SCHEME_CENTRAL && scheme != NSGB_SCHEME_UPWIND)
    return fail(NSGB_ERR_INVALID_ARG, "unknown advection scheme %d", scheme);
  if (!field || !ux || !uy || !out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_advect(scheme, field, ux, uy, out, make_consts(plan, nullptr), (cudaStream_t)stream));
  return finish_call((cudaStream_t)stream);
}

int nsgb_poisson(const nsgb_plan* plan, const float* rhs, float* p, void* workspace, size_t ws_bytes,
                 void* stream) {
  if (int r = check_plan(plan)) return r;
  if (!rhs || !p) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (int r = check_ws(workspace, ws_bytes, nsgb_poisson_workspace_bytes(plan))) return r;
  NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, rhs, workspace, p), (cudaStream_t)stream));
  return finish_call((cudaStream_t)stream);
}

int nsgb_forcing(const nsgb_plan* plan, const nsgb_phys* phys, const float* theta, int theta_len, float t,
                 float* f_out, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!f_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  NSGB_CUDA(launch_forcing_field(theta, theta_len, t, f_out, make_consts(plan, phys), (cudaStream_t)stream));
  return finish_call((cudaStream_t)stream);
}

int nsgb_projector_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u, const float* f,
                        float* u_out, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (!u || !f || !u_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (int r = check_field(u, "u")) return r;
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
  return finish_call(st);
}

int nsgb_step(const nsgb_plan* plan, const nsgb_phys* phys, const float* u, const float* theta, int theta_len,
              float t, float* u_out, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u || !u_out) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (int r = check_field(u, "u")) return r;
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
  a.jpart_rows = w.steps;
  a.theta = theta;
  a.theta_len = theta_len;
  a.step_fixed = 0;
  a.t_from_step = 0;
  a.t_fixed = t;
  NSGB_CUDA(launch_stencil(a, MODE_ROLLOUT, st));
  NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, w.p), st));
  NSGB_CUDA(launch_project(w.usA, w.p, u_out, a.c, st));
  return finish_call(st);
}

int nsgb_rollout(const nsgb_plan* plan_c, const nsgb_phys* phys, const float* u0, const float* theta,
                 int theta_len, int steps, float* u_final, float* J, void* workspace, size_t ws_bytes,
                 int use_graph, void* stream) {
  nsgb_plan* plan = const_cast<nsgb_plan*>(plan_c);
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u0 || !u_final || !J) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  if (int r = check_field(u0, "u0")) return r;
  if (steps < 0) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 0");
  const size_t need = carve_rollout(plan, steps, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  RolloutWs w = carve_rollout(plan, steps, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t NN = (size_t)plan->N * plan->N;
  StencilArgs a = stencil_args(plan, phys);
  a.theta = theta;
  a.theta_len = theta_len;
  // fused form: the first step's stencil uses the fused kernel's bands, so
  // all steps write the same grid of objective partials
  const bool fused = plan->fused_rows > 0;
  if (fused) {
    a.tw = fused_width(plan->N);
    a.th = plan->fused_rows;
  }
  const int nblk = stencil_nblocks(plan->N, a.tw, a.th);

  if (steps == 0) {
    NSGB_CUDA(cudaMemcpyAsync(u_final, u0, 2 * NN * sizeof(float), cudaMemcpyDeviceToDevice, st));
    NSGB_CUDA(launch_jreduce(w.jpart, nblk, 0, w.jsteps, J, 0.0, st));
    return finish_call(st);
  }

  // step 0 reads u0 directly; later steps ping-pong usA <-> usB (and, fused,
  // the half spectrum spec <-> spec2).
  NSGB_CUDA(rollout_step(plan, a, u0, nullptr, w.usA, w, 0, nullptr, nullptr, !fused, st));
  if (fused) NSGB_CUDA(poisson_fft(plan->N, fused_fft_launch(plan, w.rhs, w.spec, nullptr), st));
  int s = 1;
  const float* cur = w.usA;
  const float* spec_cur = w.spec;
  const int K = 16;  // steps per graph chunk (even: a chunk starts and ends in usA)
  if (use_graph && steps - 1 >= 2 * K) {
    std::lock_guard<std::mutex> lk(plan->mu);
    GraphEntry* ge = nullptr;
    for (auto& g : plan->graphs) {
      if (g.ws == workspace && g.steps == steps && g.theta == theta && g.theta_len == theta_len && g.chunk == K &&
          g.scheme == a.scheme && std::memcmp(&g.c, &a.c, sizeof(StepConsts)) == 0 &&
          g.tiles[0] == plan->tile_w && g.tiles[1] == plan->tile_h && g.tiles[2] == plan->rows_per_cta &&
          g.tiles[3] == plan->cols_per_cta && g.tiles[4] == plan->radix_rows &&
          g.tiles[5] == plan->radix_cols && g.tiles[6] == plan->fused_rows) {
        ge = &g;
        break;
      }
    }
    if (!plan->graph_stream) NSGB_CUDA(cudaStreamCreateWithFlags(&plan->graph_stream, cudaStreamNonBlocking));
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
        if (fused)
          ce = fused_step(plan, a, in, (k % 2 == 0) ? w.spec : w.spec2, out, (k % 2 == 0) ? w.spec2 : w.spec, w,
                          k, w.ctr, gs);
        else
          ce = rollout_step(plan, a, in, w.p, out, w, k, w.ctr, nullptr, true, gs);
      }
      if (ce == cudaSuccess) ce = launch_step_counter(w.ctr, K, true, gs);
      cudaError_t ee = cudaStreamEndCapture(gs, &graph);
      if (ce != cudaSuccess) return cuda_fail(ce, "rollout graph capture");
      if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
      GraphEntry g;
      g.ws = workspace;
      g.steps = steps;
      g.theta = theta;
      g.theta_len = theta_len;
      g.chunk = K;
      g.c = a.c;
      g.scheme = a.scheme;
      g.tiles[0] = plan->tile_w;
      g.tiles[1] = plan->tile_h;
      g.tiles[2] = plan->rows_per_cta;
      g.tiles[3] = plan->cols_per_cta;
      g.tiles[4] = plan->radix_rows;
      g.tiles[5] = plan->radix_cols;
      g.tiles[6] = plan->fused_rows;
      cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
      plan->graphs.push_back(g);
      ge = &plan->graphs.back();
    }
    // The chunk graph reads its first step index from w.ctr and advances it
    // by K in its last node, so one instantiated graph serves every chunk.
    // Graphs are captured on the plan's private stream and replayed on the
    // caller's, so callers on different streams overlap on the device.
    NSGB_CUDA(launch_step_counter(w.ctr, s, false, st));
    while (steps - s >= K) {
      NSGB_CUDA(cudaGraphLaunch(ge->exec, st));
      s += K;
    }
    cur = w.usA;
    spec_cur = w.spec;
  }
  for (; s < steps; ++s) {
    const float* in = cur;
    float* out = (in == w.usA) ? w.usB : w.usA;
    if (fused) {
      float* spec_next = (spec_cur == w.spec) ? w.spec2 : w.spec;
      NSGB_CUDA(fused_step(plan, a, in, spec_cur, out, spec_next, w, s, nullptr, st));
      spec_cur = spec_next;
    } else {
      NSGB_CUDA(rollout_step(plan, a, in, w.p, out, w, s, nullptr, nullptr, true, st));
    }
    cur = out;
  }
  if (fused) {  // p of the last step from its spectrum
    FftLaunch L = fused_fft_launch(plan, nullptr, (void*)spec_cur, w.p);
    L.do_cols = false;
    NSGB_CUDA(poisson_fft(plan->N, L, st));
  }
  NSGB_CUDA(launch_project(cur, w.p, u_final, a.c, st));
  NSGB_CUDA(launch_jreduce(w.jpart, nblk, steps, w.jsteps, J, (double)phys->dt * (plan->L / plan->N) *
                                                                  (plan->L / plan->N), st));
  return finish_call(st);
}

}  // extern "C"

namespace {
// The work of one gradient call (validated arguments), enqueued on st.
int grad_enqueue(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                 int theta_len, int steps, int every, int phases, float* J, float* u_final, float* dJdtheta,
                 float* dJdu0, void* workspace, cudaStream_t st) {
  GradWs g = carve_grad(plan, steps, every, workspace);
  const RolloutWs& w = g.f;
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
  b.tw = plan->adj_w;
  b.th = plan->adj_h;
  const int adj_nblk = stencil_nblocks(plan->N, b.tw, b.th);
  b.theta = theta;
  b.theta_len = theta_len;
  b.gpart = g.gpart;
  b.rhs = w.rhs;
  const float* lam = nullptr;  // lambda_S = 0
  bool have_padj = false;
  const int nseg = (steps + every - 1) / every;
  int grow = 0;  // rows of gpart holding partials not yet reduced
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * every, s1 = std::min(steps, s0 + every);
    const float* rc = g.ckpt + (size_t)seg * 2 * NN;
    const float* rp = nullptr;
    // a one-step segment's state is its checkpoint: nothing to recompute
    const bool stored = (s1 - s0 == 1);
    for (int s = s0; s < s1 && !stored; ++s) {
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
      b.u = stored ? g.ckpt + (size_t)seg * 2 * NN : g.ustore + (size_t)(s - s0) * 2 * NN;
      b.lam_out = lam_out;
      b.step = s;
      b.gslot = grow;
      NSGB_CUDA(launch_adjoint_stencil(b, st));
      if (++grow == kGradRows) {
        NSGB_CUDA(launch_greduce(g.gpart, adj_nblk, grow, g.growsum, g.gacc, st));
        grow = 0;
      }
      if (s > 0) {
        NSGB_CUDA(poisson_fft(plan->N, fft_launch(plan, w.rhs, w.spec, g.padj), st));
        have_padj = true;
      }
      lam = lam_out;
    }
  }
  NSGB_CUDA(launch_greduce(g.gpart, adj_nblk, grow, g.growsum, g.gacc, st));
  NSGB_CUDA(launch_gfinal(g.gacc, theta_len, dJdtheta, st));
  return NSGB_OK;
}
}  // namespace

extern "C" {

int nsgb_rollout_grad(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                      int theta_len, int steps, int every, int phases, float* J, float* u_final,
                      float* dJdtheta, float* dJdu0, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (int r = check_field(u0, "u0")) return r;
  if (steps < 1) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 1");
  if (every < 1) return fail(NSGB_ERR_INVALID_ARG, "checkpoint interval must be >= 1");
  if (phases < 1 || phases > 3) return fail(NSGB_ERR_INVALID_ARG, "phases must be 1, 2 or 3");
  if ((phases & NSGB_GRAD_FORWARD) && !J) return fail(NSGB_ERR_INVALID_ARG, "J is NULL");
  if ((phases & NSGB_GRAD_BACKWARD) && !dJdtheta) return fail(NSGB_ERR_INVALID_ARG, "dJdtheta is NULL");
  const size_t need = carve_grad(plan, steps, every, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  nsgb_plan* pl = const_cast<nsgb_plan*>(plan);
  // Inside a caller's stream capture the work is simply recorded.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  NSGB_CUDA(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return grad_enqueue(plan, phys, u0, theta, theta_len, steps, every, phases, J, u_final, dJdtheta, dJdu0,
                        workspace, st);  // (a capture is checked when it runs)
  GradKey key;
  std::memset(&key, 0, sizeof key);
  key.ws = workspace;
  key.u0 = u0;
  key.theta = theta;
  key.J = J;
  key.u_final = u_final;
  key.dJdtheta = dJdtheta;
  key.dJdu0 = dJdu0;
  key.theta_len = theta_len;
  key.steps = steps;
  key.every = every;
  key.phases = phases;
  key.scheme = phys->scheme;
  {
    StencilArgs a = stencil_args(plan, phys);
    key.c = a.c;
  }
  std::unique_lock<std::mutex> lk(pl->mu);
  const int t8[8] = {pl->tile_w, pl->tile_h, pl->rows_per_cta, pl->cols_per_cta,
                     pl->radix_rows, pl->radix_cols, pl->adj_w, pl->adj_h};
  std::memcpy(key.tiles, t8, sizeof t8);
  cudaGraphExec_t exec = nullptr;
  for (auto& e : pl->grad_graphs)
    if (std::memcmp(&e.first, &key, sizeof key) == 0) exec = e.second;
  if (!exec) {
    // A call is captured as a graph the second time it is made with the same
    // arguments (an optimisation loop, repeated timing); one-off calls run
    // eagerly, without the capture's host cost.
    const bool repeat = std::memcmp(&pl->last_grad, &key, sizeof key) == 0;
    std::memcpy(&pl->last_grad, &key, sizeof key);
    if (!repeat) {
      lk.unlock();
      const int r = grad_enqueue(plan, phys, u0, theta, theta_len, steps, every, phases, J, u_final, dJdtheta,
                                 dJdu0, workspace, st);
      return r ? r : finish_call(st);
    }
    if (!pl->graph_stream) NSGB_CUDA(cudaStreamCreateWithFlags(&pl->graph_stream, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    NSGB_CUDA(cudaStreamBeginCapture(pl->graph_stream, cudaStreamCaptureModeThreadLocal));
    const int r = grad_enqueue(plan, phys, u0, theta, theta_len, steps, every, phases, J, u_final, dJdtheta,
                               dJdu0, workspace, pl->graph_stream);
    const cudaError_t ee = cudaStreamEndCapture(pl->graph_stream, &graph);
    if (r != NSGB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return r;
    }
    if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture (gradient)");
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate (gradient)");
    if (pl->grad_graphs.size() >= 4) {
      cudaGraphExecDestroy(pl->grad_graphs.front().second);
      pl->grad_graphs.erase(pl->grad_graphs.begin());
    }
    pl->grad_graphs.emplace_back(key, exec);
  }
  // captured on the plan's private stream, replayed on the caller's
  NSGB_CUDA(cudaGraphLaunch(exec, st));
  return finish_call(st);
}

}  // extern "C"

// --------------------------------------------------- batched gradients --
namespace {
enum { GOP_FWD = 0, GOP_REC = 1, GOP_ADJ = 2 };
// One operation of a gradient solve: a forward step (with its checkpoint), a
// recomputed step of checkpoint segment [s0, s1), or an adjoint step.
struct GradOp {
  int kind;
  int s;        // step index
  int seg, s0, s1;
};
inline int grad_seg_ops(int len) { return len == 1 ? 1 : 2 * len; }

// The operations in the order grad_enqueue issues them: `steps` forward steps,
// then per checkpoint segment, last first, its recomputed steps (none for a
// one-step segment, whose state is its checkpoint) and its adjoint steps.
int grad_ops_total(int steps, int every) {
  const int nseg = (steps + every - 1) / every;
  const int last = steps - (nseg - 1) * every;
  return steps + grad_seg_ops(last) + (nseg - 1) * grad_seg_ops(every);
}

GradOp grad_op(int steps, int every, int k) {
  GradOp o{};
  if (k < steps) {
    o.kind = GOP_FWD;
    o.s = k;
    return o;
  }
  int r = k - steps;
  const int nseg = (steps + every - 1) / every;
  const int last = steps - (nseg - 1) * every;
  if (r < grad_seg_ops(last)) {
    o.seg = nseg - 1;
  } else {
    r -= grad_seg_ops(last);
    const int q = r / grad_seg_ops(every);
    r -= q * grad_seg_ops(every);
    o.seg = nseg - 2 - q;
  }
  o.s0 = o.seg * every;
  o.s1 = std::min(steps, o.s0 + every);
  const int len = o.s1 - o.s0;
  if (len > 1 && r < len) {
    o.kind = GOP_REC;
    o.s = o.s0 + r;
  } else {
    o.kind = GOP_ADJ;
    o.s = o.s1 - 1 - (r - (len > 1 ? len : 0));
  }
  return o;
}

int check_grad_members(const nsgb_grad_member* m, int count) {
  if (!m || count <= 0) return fail(NSGB_ERR_INVALID_ARG, "empty gradient batch");
  for (int i = 0; i < count; ++i) {
    const nsgb_grad_member& x = m[i];
    if (!x.plan) return fail(NSGB_ERR_INVALID_ARG, "member %d: plan is NULL", i);
    if (int r = check_phys(&x.phys)) return r;
    if (std::fabs(x.phys.L - x.plan->L) > 1e-12 * x.plan->L)
      return fail(NSGB_ERR_INVALID_ARG, "member %d: phys.L differs from its plan's L", i);
    if (int r = check_theta(x.theta, x.theta_len)) return r;
    if (int r = check_field(x.u0, "member u0")) return r;
    if (!x.J || !x.dJdtheta) return fail(NSGB_ERR_INVALID_ARG, "member %d: J or dJdtheta is NULL", i);
    if (x.steps < 1 || x.every < 1)
      return fail(NSGB_ERR_INVALID_ARG, "member %d: steps and every must be >= 1", i);
    if (!x.state || ((uintptr_t)x.state & 255))
      return fail(NSGB_ERR_WORKSPACE, "member %d: state must be non-NULL and 256-byte aligned", i);
    if (x.done_ops < 0 || x.done_ops > grad_ops_total(x.steps, x.every))
      return fail(NSGB_ERR_INVALID_ARG, "member %d: done_ops out of range", i);
  }
  std::vector<const void*> states(count);
  for (int i = 0; i < count; ++i) states[i] = m[i].state;
  std::sort(states.begin(), states.end(), std::less<const void*>());
  for (int i = 1; i < count; ++i)
    if (states[i] == states[i - 1]) return fail(NSGB_ERR_INVALID_ARG, "two members share one state");
  return NSGB_OK;
}

// Work of one tick, enqueued after the tick's tables are on the device.
struct GradAction {
  enum Kind { GACC_ZERO, FWD, ADJ, GREDUCE, FFT, FWD_DONE, ADJ_DONE } kind;
  int group;           // plan group (its branch stream)
  int member;          // GACC_ZERO, GREDUCE, FWD_DONE, ADJ_DONE
  const nsgb_plan* plan;
  int scheme;
  size_t off;          // FWD, ADJ, FFT: table offset in the upload
  int count;
  AdjointArgs shape;   // ADJ: launch shape
  const float* cur;    // FWD_DONE: the last step's u*
};

// Per-member view of its state (the layout of nsgb_rollout_grad).
struct GradMemberCtx {
  GradWs g;
  StencilArgs a;
  AdjointArgs b;
  int nblk, adj_nblk;
  size_t NN;
};

GradMemberCtx grad_member_ctx(const nsgb_grad_member& m) {
  GradMemberCtx c;
  c.g = carve_grad(m.plan, m.steps, m.every, m.state);
  c.NN = (size_t)m.plan->N * m.plan->N;
  c.a = stencil_args(m.plan, &m.phys);
  c.a.theta = m.theta;
  c.a.theta_len = m.theta_len;
  c.nblk = stencil_nblocks(m.plan->N, c.a.tw, c.a.th);
  c.b = AdjointArgs();
  c.b.c = c.a.c;
  c.b.scheme = c.a.scheme;
  c.b.tw = m.plan->adj_w;
  c.b.th = m.plan->adj_h;
  c.b.theta = m.theta;
  c.b.theta_len = m.theta_len;
  c.b.gpart = c.g.gpart;
  c.b.rhs = c.g.f.rhs;
  c.adj_nblk = stencil_nblocks(m.plan->N, c.b.tw, c.b.th);
  return c;
}

// Arguments of forward or recomputed step o (rollout_step's, with the
// checkpoint or the stored state as u_out).
StencilArgs grad_fwd_args(const nsgb_grad_member& m, const GradMemberCtx& c, const GradOp& o, bool& fft,
                          const float*& out_us) {
  const RolloutWs& w = c.g.f;
  StencilArgs x = c.a;
  const int s = o.s;
  if (o.kind == GOP_FWD) {
    x.us = s == 0 ? m.u0 : (((s - 1) % 2 == 0) ? w.usA : w.usB);
    x.p = s == 0 ? nullptr : w.p;
    x.us_out = (s % 2 == 0) ? w.usA : w.usB;
    x.u_out = (s % m.every == 0) ? c.g.ckpt + (size_t)(s / m.every) * 2 * c.NN : nullptr;
    fft = true;
  } else {
    const int r = s - o.s0;
    x.us = r == 0 ? c.g.ckpt + (size_t)o.seg * 2 * c.NN : (((r - 1) % 2 == 0) ? w.usA : w.usB);
    x.p = r == 0 ? nullptr : w.p;
    x.us_out = (r % 2 == 0) ? w.usA : w.usB;
    x.u_out = c.g.ustore + (size_t)r * 2 * c.NN;
    fft = s + 1 < o.s1;
  }
  x.rhs = w.rhs;
  x.jpart = w.jpart;
  x.jpart_rows = w.steps;
  x.step_ctr = nullptr;
  x.step_fixed = s;
  x.t_from_step = 1;
  out_us = x.us_out;
  return x;
}

// Arguments of adjoint step o (grad_enqueue's lambda ping-pong: the adjoint
// step b = steps - 1 - s writes lamA for even b, lamB for odd b).
AdjointArgs grad_adj_args(const nsgb_grad_member& m, const GradMemberCtx& c, const GradOp& o) {
  AdjointArgs x = c.b;
  const int s = o.s, b = m.steps - 1 - s;
  x.lam = b == 0 ? nullptr : (((b - 1) % 2 == 0) ? c.g.lamA : c.g.lamB);
  x.p = b >= 1 ? c.g.padj : nullptr;
  x.u = (o.s1 - o.s0 == 1) ? c.g.ckpt + (size_t)o.seg * 2 * c.NN : c.g.ustore + (size_t)(s - o.s0) * 2 * c.NN;
  x.lam_out = (s == 0 && m.dJdu0) ? m.dJdu0 : ((b % 2 == 0) ? c.g.lamA : c.g.lamB);
  x.step = s;
  x.gslot = b % kGradRows;
  return x;
}

// Appends a device table (entries contiguous, sizeof(T) apart, as the
// batched kernels index them) at a 16-byte aligned offset.
template <class T>
size_t put_table(std::vector<unsigned char>& buf, const std::vector<T>& v) {
  const size_t off = (buf.size() + 15) & ~(size_t)15;
  buf.resize(off + sizeof(T) * v.size());
  std::memcpy(buf.data() + off, v.data(), sizeof(T) * v.size());
  return off;
}
}  // namespace

extern "C" {

int nsgb_grad_ops(int steps, int every) {
  if (steps < 1 || every < 1) return 0;
  return grad_ops_total(steps, every);
}

size_t nsgb_grad_batch_workspace_bytes(int count, int ops) {
  if (count < 1 || ops < 1) return 0;
  return (size_t)ops * count * (2 * sizeof(SolveDev) + sizeof(AdjointArgs) + 5 * 16) + 256;
}

int nsgb_grad_batch_advance(const nsgb_grad_member* members, int count, int ops, void* workspace,
                            size_t ws_bytes, void* stream) {
  if (int r = check_grad_members(members, count)) return r;
  if (ops < 0) return fail(NSGB_ERR_INVALID_ARG, "ops must be >= 0");
  if (ops == 0) return NSGB_OK;
  if (int r = check_ws(workspace, ws_bytes, nsgb_grad_batch_workspace_bytes(count, ops))) return r;
  cudaStream_t st = (cudaStream_t)stream;
  if (int r = refuse_capture(st, "nsgb_grad_batch_advance")) return r;

  std::vector<GradMemberCtx> ctx;
  ctx.reserve(count);
  std::vector<int> todo(count);
  int maxtodo = 0;
  for (int i = 0; i < count; ++i) {
    ctx.push_back(grad_member_ctx(members[i]));
    todo[i] = std::min(ops, grad_ops_total(members[i].steps, members[i].every) - members[i].done_ops);
    maxtodo = std::max(maxtodo, todo[i]);
  }
  // Members grouped by plan (one launch shape and transform per group).
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return std::less<const nsgb_plan*>()(members[x].plan, members[y].plan); });

  std::vector<unsigned char> buf;
  buf.reserve(nsgb_grad_batch_workspace_bytes(count, std::min(ops, maxtodo)));
  std::vector<GradAction> acts;
  int ngroups = 0;
  for (int k = 0; k < maxtodo; ++k) {
    int gi = 0;  // plan group index: the same for a plan in every tick
    for (int g0 = 0; g0 < count; ++gi) {
      const nsgb_plan* plan = members[order[g0]].plan;
      int g1 = g0;
      while (g1 < count && members[order[g1]].plan == plan) ++g1;
      std::vector<SolveDev> fwd[2], fft;
      std::vector<AdjointArgs> adj[2];
      std::vector<GradAction> mid, post;
      const size_t first_act = acts.size();
      for (int q = g0; q < g1; ++q) {
        const int i = order[q];
        if (k >= todo[i]) continue;
        const nsgb_grad_member& m = members[i];
        const GradMemberCtx& c = ctx[i];
        const GradOp o = grad_op(m.steps, m.every, m.done_ops + k);
        const int sch = m.phys.scheme == NSGB_SCHEME_CENTRAL ? 0 : 1;
        if (m.done_ops + k == m.steps) {
          GradAction z{};
          z.kind = GradAction::GACC_ZERO;
          z.member = i;
          acts.push_back(z);
        }
        if (o.kind != GOP_ADJ) {
          bool do_fft = false;
          const float* out_us = nullptr;
          SolveDev d{};
          d.st[0] = grad_fwd_args(m, c, o, do_fft, out_us);
          fwd[sch].push_back(d);
          if (do_fft) {
            SolveDev f{};
            f.fft = {c.g.f.rhs, (float2*)c.g.f.spec, c.g.f.p};
            fft.push_back(f);
          }
          if (o.kind == GOP_FWD && o.s == m.steps - 1) {
            GradAction z{};
            z.kind = GradAction::FWD_DONE;
            z.member = i;
            z.cur = out_us;
            post.push_back(z);
          }
        } else {
          adj[sch].push_back(grad_adj_args(m, c, o));
          const int b = m.steps - 1 - o.s;
          if (b % kGradRows == kGradRows - 1) {
            GradAction z{};
            z.kind = GradAction::GREDUCE;
            z.member = i;
            mid.push_back(z);
          }
          if (o.s > 0) {
            SolveDev f{};
            f.fft = {c.g.f.rhs, (float2*)c.g.f.spec, c.g.padj};
            fft.push_back(f);
          } else {
            GradAction z{};
            z.kind = GradAction::ADJ_DONE;
            z.member = i;
            post.push_back(z);
          }
        }
      }
      for (int sch = 0; sch < 2; ++sch) {
        if (fwd[sch].empty()) continue;
        GradAction z{};
        z.kind = GradAction::FWD;
        z.plan = plan;
        z.scheme = fwd[sch][0].st[0].scheme;
        z.off = put_table(buf, fwd[sch]);
        z.count = (int)fwd[sch].size();
        acts.push_back(z);
      }
      for (int sch = 0; sch < 2; ++sch) {
        if (adj[sch].empty()) continue;
        GradAction z{};
        z.kind = GradAction::ADJ;
        z.plan = plan;
        z.shape = adj[sch][0];
        z.off = put_table(buf, adj[sch]);
        z.count = (int)adj[sch].size();
        acts.push_back(z);
      }
      acts.insert(acts.end(), mid.begin(), mid.end());
      if (!fft.empty()) {
        GradAction z{};
        z.kind = GradAction::FFT;
        z.plan = plan;
        z.off = put_table(buf, fft);
        z.count = (int)fft.size();
        acts.push_back(z);
      }
      acts.insert(acts.end(), post.begin(), post.end());
      for (size_t a = first_act; a < acts.size(); ++a) acts[a].group = gi;
      g0 = g1;
    }
    ngroups = gi;
  }
  if (buf.size() > ws_bytes) return fail(NSGB_ERR_WORKSPACE, "gradient batch tables exceed the workspace");
  char* dev = (char*)workspace;
  if (!buf.empty()) NSGB_CUDA(cudaMemcpyAsync(dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, st));
  Branches br;  // the plan groups run side by side
  if (int r = br.open(st, ngroups)) return r;
  for (const GradAction& z : acts) {
    cudaStream_t st = br.stream(z.group);
    switch (z.kind) {
      case GradAction::GACC_ZERO:
        NSGB_CUDA(cudaMemsetAsync(ctx[z.member].g.gacc, 0, 4 * sizeof(double), st));
        break;
      case GradAction::FWD:
        NSGB_CUDA(launch_stencil_batch((const SolveDev*)(dev + z.off), z.count, 0, 0, z.scheme, z.plan->N,
                                       z.plan->tile_w, z.plan->tile_h, st));
        break;
      case GradAction::ADJ:
        NSGB_CUDA(launch_adjoint_batch(z.shape, (const AdjointArgs*)(dev + z.off), z.count, st));
        break;
      case GradAction::GREDUCE: {
        const GradMemberCtx& c = ctx[z.member];
        NSGB_CUDA(launch_greduce(c.g.gpart, c.adj_nblk, kGradRows, c.g.growsum, c.g.gacc, st));
        break;
      }
      case GradAction::FFT:
        NSGB_CUDA(poisson_fft_batch(z.plan->N, fft_launch(z.plan, nullptr, nullptr, nullptr),
                                    (const SolveDev*)(dev + z.off), z.count, st));
        break;
      case GradAction::FWD_DONE: {
        const nsgb_grad_member& m = members[z.member];
        const GradMemberCtx& c = ctx[z.member];
        if (m.u_final) NSGB_CUDA(launch_project(z.cur, c.g.f.p, m.u_final, c.a.c, st));
        const double dx = m.plan->L / m.plan->N;
        NSGB_CUDA(launch_jreduce(c.g.f.jpart, c.nblk, m.steps, c.g.f.jsteps, m.J, (double)m.phys.dt * dx * dx, st));
        break;
      }
      case GradAction::ADJ_DONE: {
        const nsgb_grad_member& m = members[z.member];
        const GradMemberCtx& c = ctx[z.member];
        NSGB_CUDA(launch_greduce(c.g.gpart, c.adj_nblk, m.steps % kGradRows, c.g.growsum, c.g.gacc, st));
        NSGB_CUDA(launch_gfinal(c.g.gacc, m.theta_len, m.dJdtheta, st));
        break;
      }
    }
  }
  if (int r = br.close()) return r;
  return finish_call(st);
}

// ----------------------------------------------------------- optimiser --
namespace {
struct OptWs {
  GradWs g;
  float *theta, *grad, *mu, *nu, *J, *zero_u, *u_final;
  size_t bytes;
};

OptWs carve_opt(const nsgb_plan* plan, int steps, int every, void* ws) {
  const size_t NN = (size_t)plan->N * plan->N;
  OptWs o;
  o.g = carve_grad(plan, steps, every, ws);
  Carver cv(ws);
  cv.off = o.g.bytes;
  o.theta = cv.take<float>(4);
  o.grad = cv.take<float>(4);
  o.mu = cv.take<float>(4);
  o.nu = cv.take<float>(4);
  o.J = cv.take<float>(4);
  o.zero_u = cv.take<float>(2 * NN);
  o.u_final = cv.take<float>(2 * NN);
  o.bytes = cv.off;
  return o;
}

OptimizerRule optimizer_rule(const nsgb_optimizer& o, int count) {
  OptimizerRule r{};
  r.kind = o.kind;
  r.lr = (float)o.learning_rate;
  r.b1 = (float)o.b1;
  r.b2 = (float)o.b2;
  r.one_minus_b1 = (float)(1.0 - o.b1);
  r.one_minus_b2 = (float)(1.0 - o.b2);
  r.bc1 = (float)(1.0 - std::pow(o.b1, (double)count));
  r.bc2 = (float)(1.0 - std::pow(o.b2, (double)count));
  r.eps = (float)o.eps;
  r.eps_root = (float)o.eps_root;
  r.decay = (float)o.decay;
  r.one_minus_decay = (float)(1.0 - o.decay);
  return r;
}
}  // namespace

size_t nsgb_optimize_workspace_bytes(const nsgb_plan* plan, int steps, int every, int theta_len) {
  if (!plan || steps < 1 || every < 1 || (theta_len != 2 && theta_len != 3)) return 0;
  return carve_opt(plan, steps, every, nullptr).bytes;
}

int nsgb_optimize(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta0,
                  int theta_len, int steps, int every, const nsgb_optimizer* opt, int iters, float* objectives,
                  float* parameters, void* workspace, size_t ws_bytes, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta0, theta_len)) return r;
  if (u0)
    if (int r = check_field(u0, "u0")) return r;
  if (!opt) return fail(NSGB_ERR_INVALID_ARG, "optimizer is NULL");
  if (opt->kind != NSGB_OPT_SGD && opt->kind != NSGB_OPT_ADAM && opt->kind != NSGB_OPT_RMSPROP)
    return fail(NSGB_ERR_INVALID_ARG, "unknown optimizer kind %d", opt->kind);
  if (!(std::isfinite(opt->learning_rate) && std::isfinite(opt->b1) && std::isfinite(opt->b2) &&
        std::isfinite(opt->eps) && std::isfinite(opt->eps_root) && std::isfinite(opt->decay)))
    return fail(NSGB_ERR_INVALID_ARG, "optimizer hyper-parameters must be finite");
  if (steps < 1) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 1");
  if (every < 1) return fail(NSGB_ERR_INVALID_ARG, "checkpoint interval must be >= 1");
  if (iters < 0) return fail(NSGB_ERR_INVALID_ARG, "iters must be >= 0");
  if (!objectives || !parameters) return fail(NSGB_ERR_INVALID_ARG, "NULL history pointer");
  const size_t need = carve_opt(plan, steps, every, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  OptWs o = carve_opt(plan, steps, every, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t NN = (size_t)plan->N * plan->N;
  const size_t tb = (size_t)theta_len * sizeof(float);
  NSGB_CUDA(cudaMemcpyAsync(o.theta, theta0, tb, cudaMemcpyDeviceToDevice, st));
  NSGB_CUDA(cudaMemcpyAsync(parameters, theta0, tb, cudaMemcpyDeviceToDevice, st));
  NSGB_CUDA(cudaMemsetAsync(o.mu, 0, 4 * sizeof(float), st));
  NSGB_CUDA(cudaMemsetAsync(o.nu, 0, 4 * sizeof(float), st));
  if (!u0) {
    NSGB_CUDA(cudaMemsetAsync(o.zero_u, 0, 2 * NN * sizeof(float), st));
    u0 = o.zero_u;
  }
  const size_t grad_bytes = o.g.bytes;
  for (int k = 0; k < iters; ++k) {
    // the same arguments every iteration (J into a fixed slot), so from the
    // second iteration on the gradient replays as one graph
    if (int r = nsgb_rollout_grad(plan, phys, u0, o.theta, theta_len, steps, every,
                                  NSGB_GRAD_FORWARD | NSGB_GRAD_BACKWARD, o.J, nullptr, o.grad, nullptr, workspace,
                                  grad_bytes, stream))
      return r;
    NSGB_CUDA(cudaMemcpyAsync(objectives + k, o.J, sizeof(float), cudaMemcpyDeviceToDevice, st));
    NSGB_CUDA(launch_optimizer_update(optimizer_rule(*opt, k + 1), o.theta, o.grad, o.mu, o.nu,
                                      parameters + (size_t)(k + 1) * theta_len, theta_len, st));
  }
  // objective at the last parameters (the study evaluates it after each update)
  return nsgb_rollout(plan, phys, u0, o.theta, theta_len, steps, o.u_final, objectives + iters, workspace,
                      grad_bytes, 0, stream);
}

size_t nsgb_ensemble_workspace_bytes(const nsgb_member* members, int count) {
  if (!members || count <= 0) return 0;
  for (int i = 0; i < count; ++i)
    if (!members[i].plan || members[i].total_steps < 1) return 0;
  return ensemble_layout(members, count).bytes;
}

int nsgb_ensemble_advance(const nsgb_member* members, int count, int steps, void* workspace, size_t ws_bytes,
                          void* stream) {
  if (int r = check_members(members, count, true)) return r;
  if (steps < 0) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 0");
  EnsLayout L = ensemble_layout(members, count);
  if (int r = check_ws(workspace, ws_bytes, L.bytes)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  if (int r = refuse_capture(st, "nsgb_ensemble_advance")) return r;
  char* base = (char*)workspace;
  SolveDev* dev = (SolveDev*)(base + L.tab_off);
  std::vector<int> order;
  std::vector<EnsGroup> groups = make_groups(members, count, steps, order);
  std::vector<SolveDev> tab(count);
  int maxtodo = 0;
  for (int k = 0; k < count; ++k) {
    const int i = order[k];
    void* state = members[i].state ? members[i].state : (void*)(base + L.state_off[i]);
    tab[k] = make_solvedev(members[i], state);
  }
  for (const EnsGroup& G : groups) maxtodo = std::max(maxtodo, G.todo);
  NSGB_CUDA(cudaMemcpyAsync(dev, tab.data(), sizeof(SolveDev) * count, cudaMemcpyHostToDevice, st));
  NSGB_CUDA(launch_counter_batch(dev, count, 0, false, st));  // counters = done_steps
  Branches br;  // the groups run side by side
  if (int r = br.open(st, (int)groups.size())) return r;
  const std::vector<cudaStream_t> gs = br.streams();
  for (int k = 0; k < maxtodo; ++k) NSGB_CUDA(ensemble_step(groups, dev, k, gs));
  if (int r = br.close()) return r;
  NSGB_CUDA(ensemble_finalize(members, order, tab, steps, (SolveDev*)(base + L.fin_off), st));
  return finish_call(st);
}

int nsgb_ensemble_rollout(const nsgb_member* members_in, int count, int chunk, void* workspace, size_t ws_bytes,
                          void* stream) {
  if (int r = check_members(members_in, count, true)) return r;
  if (chunk < 0 || (chunk % 2) != 0) return fail(NSGB_ERR_INVALID_ARG, "chunk must be even and >= 0");
  const int steps = members_in[0].total_steps;
  for (int i = 1; i < count; ++i)
    if (members_in[i].total_steps != steps)
      return fail(NSGB_ERR_INVALID_ARG, "nsgb_ensemble_rollout needs equal total_steps (use advance)");
  std::vector<nsgb_member> members(members_in, members_in + count);
  for (auto& m : members) m.done_steps = 0;
  EnsLayout L = ensemble_layout(members.data(), count);
  if (int r = check_ws(workspace, ws_bytes, L.bytes)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  if (int r = refuse_capture(st, "nsgb_ensemble_rollout")) return r;
  char* base = (char*)workspace;
  SolveDev* dev = (SolveDev*)(base + L.tab_off);
  std::vector<int> order;
  std::vector<EnsGroup> groups = make_groups(members.data(), count, steps, order);
  std::vector<SolveDev> tab(count);
  for (int k = 0; k < count; ++k) {
    const int i = order[k];
    void* state = members[i].state ? members[i].state : (void*)(base + L.state_off[i]);
    tab[k] = make_solvedev(members[i], state);
  }
  NSGB_CUDA(cudaMemcpyAsync(dev, tab.data(), sizeof(SolveDev) * count, cudaMemcpyHostToDevice, st));
  NSGB_CUDA(launch_counter_batch(dev, count, 0, false, st));
  std::vector<cudaStream_t> one{st};
  // step 0 reads u0; then counters = 1 and the groups are at odd parity.
  NSGB_CUDA(ensemble_step(groups, dev, 0, one));
  NSGB_CUDA(launch_counter_batch(dev, count, 1, true, st));
  for (auto& G : groups) {
    G.done = 1;
    G.todo = steps - 1;
  }
  int s = 1;
  if (chunk > 0 && steps - 1 >= chunk) {
    std::lock_guard<std::mutex> lk(g_ens_mu);
    const uint64_t sig = fnv(tab.data(), sizeof(SolveDev) * count);
    EnsGraph* eg = nullptr;
    for (auto& g : g_ens_graphs)
      if (g.ws == workspace && g.count == count && g.chunk == chunk && g.sig == sig) eg = &g;
    const int nbr = (int)std::min<size_t>(groups.size(), 8);
    if (!eg) {
      EnsPool* pool = nullptr;
      if (int r = ens_pool(pool)) return r;
      cudaStream_t cs = pool->s[0];
      if (g_ens_graphs.size() >= 8) {
        cudaGraphExecDestroy(g_ens_graphs.front().exec);
        g_ens_graphs.erase(g_ens_graphs.begin());
      }
      std::vector<cudaStream_t> br(pool->s + 1, pool->s + 1 + nbr);
      std::vector<EnsGroup> cg = groups;
      for (auto& G : cg) G.todo = chunk;
      cudaGraph_t graph;
      NSGB_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = cudaEventRecord(pool->e[0], cs);
      for (int b = 0; b < nbr && ce == cudaSuccess; ++b) ce = cudaStreamWaitEvent(br[b], pool->e[0], 0);
      for (int k = 0; k < chunk && ce == cudaSuccess; ++k) ce = ensemble_step(cg, dev, k, br);
      for (int b = 0; b < nbr && ce == cudaSuccess; ++b) {
        ce = cudaEventRecord(pool->e[1 + b], br[b]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(cs, pool->e[1 + b], 0);
      }
      if (ce == cudaSuccess) ce = launch_counter_batch(dev, count, chunk, true, cs);
      cudaError_t ee = cudaStreamEndCapture(cs, &graph);
      if (ce != cudaSuccess) return cuda_fail(ce, "ensemble graph capture");
      if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
      EnsGraph g{workspace, count, chunk, sig, nullptr};
      cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
      g_ens_graphs.push_back(g);
      eg = &g_ens_graphs.back();
    }
    // captured on the pool's streams, replayed on the caller's, so ensembles
    // on different streams overlap on the device
    while (steps - s >= chunk) {
      NSGB_CUDA(cudaGraphLaunch(eg->exec, st));
      s += chunk;
    }
  }
  // remaining steps: the chunks kept the parity (chunk is even)
  for (auto& G : groups) {
    G.done = s;
    G.todo = steps - s;
  }
  for (int k = 0; k < steps - s; ++k) NSGB_CUDA(ensemble_step(groups, dev, k, one));
  NSGB_CUDA(ensemble_finalize(members.data(), order, tab, steps, (SolveDev*)(base + L.fin_off), st));
  return finish_call(st);
}

}  // extern "C"

namespace {
// Workspace of nsgb_ensemble_persistent: the ensemble layout, then the member
// constants, the stage item tables, the barrier words and, per member, the
// objective partials of the persistent launch's tiling.
struct PersLayout {
  EnsLayout ens;
  size_t pm_off = 0, first_off = 0, bar_off = 0, bytes = 0;
  std::vector<size_t> jpart_off;
};

PersLayout pers_layout(const nsgb_member* m, int count) {
  PersLayout P;
  P.ens = ensemble_layout(m, count);
  size_t off = P.ens.bytes;
  P.pm_off = off;
  off += align_up(sizeof(PersMember) * (size_t)count);
  P.first_off = off;
  off += align_up(sizeof(int) * 4 * (size_t)(count + 1));
  P.bar_off = off;
  off += align_up(4 * sizeof(unsigned));
  P.jpart_off.resize(count);
  for (int k = 0; k < count; ++k) {
    P.jpart_off[k] = off;
    int tw, th;
    pers_tile(m[k].plan->N, tw, th);
    off += align_up(sizeof(float) * (size_t)m[k].total_steps * stencil_nblocks(m[k].plan->N, tw, th));
  }
  P.bytes = off;
  return P;
}
}  // namespace

extern "C" {

size_t nsgb_ensemble_persistent_workspace_bytes(const nsgb_member* members, int count) {
  if (!members || count <= 0) return 0;
  for (int i = 0; i < count; ++i)
    if (!members[i].plan || members[i].total_steps < 1 || !pers_supported(members[i].plan->N)) return 0;
  return pers_layout(members, count).bytes;
}

int nsgb_ensemble_persistent(const nsgb_member* members_in, int count, void* workspace, size_t ws_bytes,
                             void* stream) {
  if (int r = check_members(members_in, count, true)) return r;
  const int steps = members_in[0].total_steps;
  for (int i = 0; i < count; ++i) {
    if (members_in[i].total_steps != steps)
      return fail(NSGB_ERR_INVALID_ARG, "nsgb_ensemble_persistent needs equal total_steps");
    if (!pers_supported(members_in[i].plan->N))
      return fail(NSGB_ERR_UNSUPPORTED_N, "member %d: N=%d outside the persistent launch's 64..4096", i,
                  members_in[i].plan->N);
  }
  std::vector<nsgb_member> members(members_in, members_in + count);
  for (auto& m : members) m.done_steps = 0;
  const PersLayout P = pers_layout(members.data(), count);
  if (int r = check_ws(workspace, ws_bytes, P.bytes)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  if (int r = refuse_capture(st, "nsgb_ensemble_persistent")) return r;
  char* base = (char*)workspace;
  SolveDev* dev = (SolveDev*)(base + P.ens.tab_off);
  std::vector<int> order;
  (void)make_groups(members.data(), count, steps, order);
  // largest members first: their items lead every stage's work list, so the
  // list ends with short items and the CTAs finish a stage close together
  std::reverse(order.begin(), order.end());
  std::vector<SolveDev> tab(count);
  std::vector<PersMember> pm(count);
  std::vector<int> first(4 * (size_t)(count + 1), 0);
  size_t smem = 0;
  for (int k = 0; k < count; ++k) {
    const int i = order[k];
    const nsgb_member& x = members[i];
    void* state = x.state ? x.state : (void*)(base + P.ens.state_off[i]);
    tab[k] = make_solvedev(x, state);
    float* jp = (float*)(base + P.jpart_off[i]);
    for (auto& a : tab[k].st) {
      a.jpart = jp;
      a.jpart_rows = steps;
    }
    const int N = x.plan->N;
    pm[k] = {x.plan->tw, x.plan->k2, (float)(1.0 / (2.0 * (double)N * (double)N)), N};
    int it[4];
    pers_items(N, it);
    for (int s = 0; s < 4; ++s) first[(size_t)s * (count + 1) + k + 1] = first[(size_t)s * (count + 1) + k] + it[s];
    smem = std::max(smem, pers_smem_bytes(N));
  }
  NSGB_CUDA(cudaMemcpyAsync(dev, tab.data(), sizeof(SolveDev) * count, cudaMemcpyHostToDevice, st));
  NSGB_CUDA(cudaMemcpyAsync(base + P.pm_off, pm.data(), sizeof(PersMember) * count, cudaMemcpyHostToDevice, st));
  NSGB_CUDA(cudaMemcpyAsync(base + P.first_off, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice,
                            st));
  unsigned* bar = (unsigned*)(base + P.bar_off);
  NSGB_CUDA(cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), st));
  NSGB_CUDA(launch_counter_batch(dev, count, 0, false, st));  // step counters = 0
  PersWork w;
  w.dev = dev;
  w.pm = (const PersMember*)(base + P.pm_off);
  for (int s = 0; s < 4; ++s) {
    w.first[s] = (const int*)(base + P.first_off) + (size_t)s * (count + 1);
    w.items[s] = first[(size_t)s * (count + 1) + count];
  }
  w.count = count;
  w.steps = steps;
  w.done = 0;
  w.bar = bar;
  w.poll_limit = 1u << 22;
  int dev_id = 0, sms = 152;
  NSGB_CUDA(cudaGetDevice(&dev_id));
  NSGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  NSGB_CUDA(launch_ensemble_persistent(w, smem, sms, nullptr, st));
  NSGB_CUDA(ensemble_finalize(members.data(), order, tab, steps, (SolveDev*)(base + P.ens.fin_off), st, true));
  NSGB_CUDA(launch_ensemble_poison(bar, dev, count, st));
  return finish_call(st);
}

int nsgb_time_stages(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                     int theta_len, int reps, void* flush, size_t flush_bytes, void* workspace,
                     size_t ws_bytes, float* out_ms, void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u0 || !out_ms) return fail(NSGB_ERR_INVALID_ARG, "NULL pointer");
  if (int r = check_field(u0, "u0")) return r;
  if (reps < 1) return fail(NSGB_ERR_INVALID_ARG, "reps must be >= 1");
  const size_t need = carve_rollout(plan, 1, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  RolloutWs w = carve_rollout(plan, 1, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  StencilArgs a = stencil_args(plan, phys);
  a.theta = theta;
  a.theta_len = theta_len;
  const bool fused = plan->fused_rows > 0;
  if (fused) {
    a.tw = fused_width(plan->N);
    a.th = plan->fused_rows;
  }
  // Steady state: one step from u0 leaves u* in usA and p pending (fused:
  // the solved spectrum in spec).
  NSGB_CUDA(rollout_step(plan, a, u0, nullptr, w.usA, w, 0, nullptr, nullptr, !fused, st));
  if (fused) NSGB_CUDA(poisson_fft(plan->N, fused_fft_launch(plan, w.rhs, w.spec, nullptr), st));
  cudaEvent_t e0, e1;
  NSGB_CUDA(cudaEventCreate(&e0));
  if (cudaError_t ce = cudaEventCreate(&e1)) {
    cudaEventDestroy(e0);
    return cuda_fail(ce, "cudaEventCreate");
  }
  double tot[4] = {0, 0, 0, 0};
  cudaError_t err = cudaSuccess;
  for (int stage = 0; stage < 4 && err == cudaSuccess; ++stage) {
    for (int r = 0; r < reps && err == cudaSuccess; ++r) {
      if (flush && flush_bytes) err = cudaMemsetAsync(flush, r & 0xff, flush_bytes, st);
      if (err == cudaSuccess) err = cudaEventRecord(e0, st);
      if (err != cudaSuccess) break;
      if (fused) {
        // stage 0: the fused row kernel; stage 1: the column pass; 2, 3: none
        if (stage == 0) {
          FusedArgs f;
          f.a = a;
          f.a.us = w.usA;
          f.a.us_out = w.usB;
          f.a.jpart = w.jpart;
          f.a.jpart_rows = w.steps;
          f.a.step_fixed = 0;
          f.spec_in = (const float2*)w.spec;
          f.spec_out = (float2*)w.spec2;
          f.tw = plan->tw;
          err = launch_fused_rows(f, st);
        } else if (stage == 1) {
          err = poisson_fft(plan->N, fused_fft_launch(plan, nullptr, w.spec2, nullptr), st);
        }
      } else if (stage == 0) {
        StencilArgs b = a;
        b.us = w.usA;
        b.p = w.p;
        b.us_out = w.usB;
        b.rhs = w.rhs;
        b.jpart = w.jpart;
        b.jpart_rows = w.steps;
        b.step_fixed = 0;
        err = launch_stencil(b, MODE_ROLLOUT, st);
      } else {
        FftLaunch L = fft_launch(plan, w.rhs, w.spec, w.p);
        if (stage != 1) L.rhs = nullptr;
        L.do_cols = (stage == 2);
        if (stage != 3) L.p = nullptr;
        err = poisson_fft(plan->N, L, st);
      }
      if (err == cudaSuccess) err = cudaEventRecord(e1, st);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      tot[stage] += ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return cuda_fail(err, "nsgb_time_stages");
  for (int k = 0; k < 4; ++k) out_ms[k] = (float)(tot[k] / reps);
  return finish_call(st);
}

int nsgb_time_step_pipeline(const nsgb_plan* plan, const nsgb_phys* phys, const float* u0, const float* theta,
                            int theta_len, int steps, void* workspace, size_t ws_bytes, float* out_ms,
                            void* stream) {
  if (int r = check_plan(plan)) return r;
  if (int r = check_phys(phys)) return r;
  if (int r = check_theta(theta, theta_len)) return r;
  if (!u0 || !out_ms) return fail(NSGB_ERR_INVALID_ARG, "NULL pointer");
  if (int r = check_field(u0, "u0")) return r;
  if (steps < 1) return fail(NSGB_ERR_INVALID_ARG, "steps must be >= 1");
  const size_t need = carve_rollout(plan, steps + 1, nullptr).bytes;
  if (int r = check_ws(workspace, ws_bytes, need)) return r;
  RolloutWs w = carve_rollout(plan, steps + 1, workspace);
  cudaStream_t st = (cudaStream_t)stream;
  StencilArgs a = stencil_args(plan, phys);
  a.theta = theta;
  a.theta_len = theta_len;
  const bool fused = plan->fused_rows > 0;
  if (fused) {
    a.tw = fused_width(plan->N);
    a.th = plan->fused_rows;
  }
  // first step from u0 (p not yet pending), then `steps` timed steps
  NSGB_CUDA(rollout_step(plan, a, u0, nullptr, w.usA, w, 0, nullptr, nullptr, !fused, st));
  if (fused) NSGB_CUDA(poisson_fft(plan->N, fused_fft_launch(plan, w.rhs, w.spec, nullptr), st));
  const float* spec_cur = w.spec;
  std::vector<cudaEvent_t> ev((size_t)steps * 4 + 1, nullptr);
  cudaError_t err = cudaSuccess;
  for (auto& e : ev)
    if (err == cudaSuccess) err = cudaEventCreate(&e);
  const float* cur = w.usA;
  for (int s = 0; s < steps && err == cudaSuccess; ++s) {
    float* out = (cur == w.usA) ? w.usB : w.usA;
    StencilArgs b = a;
    b.us = cur;
    b.p = w.p;
    b.us_out = out;
    b.rhs = w.rhs;
    b.jpart = w.jpart;
    b.jpart_rows = w.steps;
    b.step_fixed = s + 1;
    if (s == 0) err = cudaEventRecord(ev[0], st);
    if (fused) {
      // stages: the fused row kernel, the column pass (two empty stages)
      float* spec_next = (spec_cur == w.spec) ? w.spec2 : w.spec;
      FusedArgs f;
      f.a = b;
      f.a.p = nullptr;
      f.a.rhs = nullptr;
      f.spec_in = (const float2*)spec_cur;
      f.spec_out = (float2*)spec_next;
      f.tw = plan->tw;
      if (err == cudaSuccess) err = launch_fused_rows(f, st);
      if (err == cudaSuccess) err = cudaEventRecord(ev[(size_t)s * 4 + 1], st);
      if (err == cudaSuccess) err = poisson_fft(plan->N, fused_fft_launch(plan, nullptr, spec_next, nullptr), st);
      for (int stage = 2; stage <= 4 && err == cudaSuccess; ++stage)
        err = cudaEventRecord(ev[(size_t)s * 4 + stage], st);
      spec_cur = spec_next;
      cur = out;
      continue;
    }
    if (err == cudaSuccess) err = launch_stencil(b, MODE_ROLLOUT, st);
    for (int stage = 1; stage <= 4 && err == cudaSuccess; ++stage) {
      err = cudaEventRecord(ev[(size_t)s * 4 + stage], st);
      if (err != cudaSuccess || stage == 4) break;
      FftLaunch L = fft_launch(plan, w.rhs, w.spec, w.p);
      if (stage != 1) L.rhs = nullptr;
      L.do_cols = (stage == 2);
      if (stage != 3) L.p = nullptr;
      err = poisson_fft(plan->N, L, st);
    }
    cur = out;
  }
  double tot[4] = {0, 0, 0, 0};
  if (err == cudaSuccess) err = cudaEventSynchronize(ev.back());
  for (int s = 0; s < steps && err == cudaSuccess; ++s)
    for (int k = 0; k < 4 && err == cudaSuccess; ++k) {
      float ms = 0.f;
      err = cudaEventElapsedTime(&ms, ev[(size_t)s * 4 + k], ev[(size_t)s * 4 + k + 1]);
      tot[k] += ms;
    }
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (err != cudaSuccess) return cuda_fail(err, "nsgb_time_step_pipeline");
  for (int k = 0; k < 4; ++k) out_ms[k] = (float)(tot[k] / steps);
  return finish_call(st);
}

}  // extern "C"
