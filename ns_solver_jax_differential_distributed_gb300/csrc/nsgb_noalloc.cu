// nsgb_poisson_noalloc: the spectral Poisson solve without any device
// allocation by the library or the caller beyond the input and output fields.
//
// Who needs it: callers that cannot allocate device memory when they solve --
// code that runs inside a fixed device-memory budget owned by an arena or
// pool it cannot grow, latency-critical loops in which a cudaMalloc (which may
// synchronise the device) is not acceptable, and hosts reaching the library
// through a plain C FFI that have no way to own a plan and a workspace.
//
// How: the half spectrum and the constant tables live in file-scope
// `static __device__` arrays sized for N <= NSGB_NOALLOC_MAX_N (about 4.2 MB
// per GPU that loads the library, held until the process exits).  Host code
// cannot use those array names as device addresses, so the first call on each
// device, with that device current, asks cudaGetSymbolAddress for them and
// caches the addresses; that first call should come before any stream
// capture.  The cache is keyed by device ordinal and so assumes the runtime's
// primary context on that device (the context torch and the runtime API use);
// a caller that resets the device or runs in a context of its own creation
// must not share the cached addresses.  A call on a capturing stream is
// refused with NSGB_ERR_INVALID_ARG and enqueues nothing.  Every call uploads
// the twiddle and wavenumber tables for its
// (N, L) from a static host buffer with cudaMemcpyToSymbolAsync and runs the
// same three FFT kernels as nsgb_poisson.  Nothing needs clearing: the
// forward row pass writes every spectrum entry before the column pass reads it.
//
// All calls share the arrays: two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on them, and the
// arrays keep the last call's contents.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "nsgb_fft.cuh"
#include "nsgb_internal.h"

namespace {

constexpr int kMaxN = NSGB_NOALLOC_MAX_N;
constexpr int kMaxTw = nsgb::fft::tw_total(kMaxN);

static __device__ __align__(256) float2 g_noalloc_spec[(kMaxN / 2 + 1) * kMaxN];
static __device__ __align__(256) float2 g_noalloc_tw[kMaxTw];
static __device__ __align__(256) float g_noalloc_k2[kMaxN];

struct DevicePtrs {
  bool ready = false;
  float2* spec = nullptr;
  float2* tw = nullptr;
  float* k2 = nullptr;
};
constexpr int kMaxDevices = 64;
DevicePtrs g_dev[kMaxDevices];
std::mutex g_mu;                 // guards g_dev and the host staging tables
float2 g_host_tw[kMaxTw];        // host staging of the per-call tables
float g_host_k2[kMaxN];

// Failures are reported through nsgb_last_error(), like every other entry point.
int fail(int code, const char* fmt, ...) {
  char buf[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  nsgb::set_last_error(buf);
  return code;
}

// Twiddles of the Stockham passes and squared wavenumbers, laid out and
// rounded exactly as a plan of the same (N, L) holds them.
void fill_tables(int N, double L) {
  nsgb::fft::host_twiddles(N, g_host_tw);
  const double dx = L / N;
  const float dn = (float)(dx * N);
  for (int m = 0; m < N; ++m) {
    const int mm = m < N / 2 ? m : m - N;
    volatile float k = (float)mm / dn;
    k = k * 2.0f;
    k = k * (float)M_PI;
    volatile float kk = k * k;
    g_host_k2[m] = kk;
  }
}

}  // namespace

extern "C" int nsgb_poisson_noalloc(int N, double L, const float* rhs, float* p, void* stream) {
  if (N < 16 || (N & (N - 1)) != 0)
    return fail(NSGB_ERR_UNSUPPORTED_N, "N=%d unsupported: power of two >= 16 required", N);
  if (N > kMaxN)
    return fail(NSGB_ERR_UNSUPPORTED_N,
                "N=%d exceeds the static scratch of nsgb_poisson_noalloc (N <= %d); use nsgb_poisson",
                N, kMaxN);
  if (!(std::isfinite(L) && L > 0)) return fail(NSGB_ERR_INVALID_ARG, "L must be positive and finite");
  if (!rhs || !p) return fail(NSGB_ERR_INVALID_ARG, "NULL field pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(NSGB_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(NSGB_ERR_INVALID_ARG, "device %d out of range", dev);
  cudaStream_t st = (cudaStream_t)stream;
  // A captured table upload would become a graph node that reads the shared
  // host staging tables at replay time, after later calls may have refilled
  // them for another (N, L): refuse instead of recording it.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(st, &cap)) != cudaSuccess)
    return fail(NSGB_ERR_CUDA, "cudaStreamIsCapturing: %s", cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(NSGB_ERR_INVALID_ARG,
                "nsgb_poisson_noalloc does not run on a capturing stream (its table uploads read shared "
                "host buffers); call nsgb_poisson with a plan inside captures");

  std::lock_guard<std::mutex> lk(g_mu);
  DevicePtrs& d = g_dev[dev];
  if (!d.ready) {  // once per device, with that device current
    void* a = nullptr;
    if ((e = cudaGetSymbolAddress(&a, g_noalloc_spec)) != cudaSuccess)
      return fail(NSGB_ERR_CUDA, "cudaGetSymbolAddress(spec): %s", cudaGetErrorString(e));
    d.spec = (float2*)a;
    if ((e = cudaGetSymbolAddress(&a, g_noalloc_tw)) != cudaSuccess)
      return fail(NSGB_ERR_CUDA, "cudaGetSymbolAddress(tw): %s", cudaGetErrorString(e));
    d.tw = (float2*)a;
    if ((e = cudaGetSymbolAddress(&a, g_noalloc_k2)) != cudaSuccess)
      return fail(NSGB_ERR_CUDA, "cudaGetSymbolAddress(k2): %s", cudaGetErrorString(e));
    d.k2 = (float*)a;
    int r = nsgb::bounds_add_library_range(d.spec, sizeof g_noalloc_spec);
    if (!r) r = nsgb::bounds_add_library_range(d.tw, sizeof g_noalloc_tw);
    if (!r) r = nsgb::bounds_add_library_range(d.k2, sizeof g_noalloc_k2);
    if (r) return r;
    d.ready = true;
  }
  fill_tables(N, L);
  // From pageable host memory these copies return once the data is staged,
  // so the static host tables may be refilled by the next call.
  e = cudaMemcpyToSymbolAsync(g_noalloc_tw, g_host_tw, sizeof(float2) * nsgb::fft::tw_total(N), 0,
                              cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(g_noalloc_k2, g_host_k2, sizeof(float) * N, 0, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail(NSGB_ERR_CUDA, "table upload: %s", cudaGetErrorString(e));

  nsgb::FftLaunch Lc;
  Lc.rhs = rhs;
  Lc.spec = d.spec;
  Lc.do_cols = true;
  Lc.p = p;
  Lc.tw = d.tw;
  Lc.k2 = d.k2;
  Lc.scale = (float)(1.0 / (2.0 * (double)N * (double)N));
  Lc.rows_per_cta = N >= 1024 ? 4 : 8;
  Lc.cols_per_cta = 1;
  e = nsgb::poisson_fft(N, Lc, st);
  if (e != cudaSuccess) return fail(NSGB_ERR_CUDA, "poisson kernels: %s", cudaGetErrorString(e));
  return nsgb::finish_call(st);
}
