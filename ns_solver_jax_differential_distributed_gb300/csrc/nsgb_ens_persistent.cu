// Persistent ensemble kernel: every step of every member of an ensemble of
// uneven grid sizes in ONE cooperative launch.  The CTAs walk a work list per
// stage -- the stencil tiles of all members, then their forward row-transform
// blocks, column blocks and inverse row-transform blocks -- and meet at a
// grid-wide barrier between stages.  Each work item runs the same body as the
// stage's own kernel (tiled stencil 64 x 16, radix-16 transforms), so a
// member's fields equal those of its solo rollout with radix-16 transforms bit
// for bit; its objective partials follow the 64 x 16 tiling.
//
// Loads of fields other CTAs wrote during the launch go through L2 only
// (__ldcg): the non-coherent read-only path and L1 could return lines of an
// earlier step.  The barrier is bounded: a CTA that waits longer than the
// launch's poll limit raises the abort word, every CTA leaves at its next
// barrier, and the host turns the abort into non-finite objectives.
#include "nsgb_fft_bodies.cuh"
#include "nsgb_stencil_body.cuh"

namespace nsgb {
namespace pers {

constexpr int kThreads = 256;  // blockDim (32, 8): the tiled stencil's CTA
constexpr int kTW = 64, kTH = 16;  // stencil tile

__host__ __device__ inline int fft_T(int N) { return N / 16; }
// Row pairs of one forward/inverse row item, and spectrum rows of one column
// item, for a 256-thread CTA.
__host__ __device__ inline int rows_P(int N) { return kThreads / fft_T(N) < N / 2 ? kThreads / fft_T(N) : N / 2; }
__host__ __device__ inline int cols_KB(int N) { return kThreads / fft_T(N); }

// Member whose items [first[m], first[m+1]) contain item `it` (first[0] = 0).
__device__ __forceinline__ int member_of(const int* __restrict__ first, int count, int it) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(first + mid) <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Grid-wide barrier over gridDim.x CTAs; false once any CTA gave up waiting.
// bar[0]: arrivals, bar[1]: generation, bar[2]: abort.
__device__ bool grid_barrier(unsigned* bar, unsigned limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    volatile unsigned* vb = bar;
    int good = 1;
    const unsigned gen = vb[1];
    __threadfence();  // this CTA's stores before its arrival
    if (atomicAdd(&bar[0], 1u) + 1u == gridDim.x) {
      bar[0] = 0u;
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      for (unsigned i = 0; vb[1] == gen; ++i) {
        if (vb[2] != 0u || i >= limit) {
          atomicExch(&bar[2], 1u);
          good = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();  // the other CTAs' stores before this CTA's next loads
    ok = good && vb[2] == 0u;
  }
  __syncthreads();
  return ok != 0;
}

template <int N>
__device__ __forceinline__ void rows_fwd_item(const FftPtrs& f, const PersMember& pm, int tid, int u) {
  rows_fwd_body<N, 16, true>(f.rhs, f.spec, pm.tw, tid % fft_T(N), tid / fft_T(N), rows_P(N), u);
}
template <int N>
__device__ __forceinline__ void cols_item(const FftPtrs& f, const PersMember& pm, int tid, int u) {
  cols_body<N, 16, true>(f.spec, pm.tw, pm.k2, pm.scale, tid % fft_T(N), tid / fft_T(N), cols_KB(N), u);
}
template <int N>
__device__ __forceinline__ void rows_inv_item(const FftPtrs& f, const PersMember& pm, int tid, int u) {
  rows_inv_body<N, 16, true>(f.spec, f.p, pm.tw, tid % fft_T(N), tid / fft_T(N), rows_P(N), u);
}

#define NSGB_PERS_SIZES(X) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

// Bounded to 80 registers for three CTAs per SM (the union of the stage bodies
// would otherwise take about 200 and leave one).
__global__ void __launch_bounds__(kThreads, 3) k_ensemble_persistent(const PersWork w) {
  const int tid = threadIdx.y * 32 + threadIdx.x;
  for (int k = 0; k < w.steps; ++k) {
    const int s = w.done + k;
    const int variant = s == 0 ? 0 : ((s & 1) ? 1 : 2);
    // 1. fused stencil of every member, tile by tile (64 x 16 tiles)
    for (int it = blockIdx.x; it < w.items[0]; it += gridDim.x) {
      const int m = member_of(w.first[0], w.count, it);
      const int u = it - __ldg(w.first[0] + m);
      const StencilArgs& a = w.dev[m].st[variant];
      const int gx = a.c.N / kTW, gy = a.c.N / kTH;
      if (a.scheme == NSGB_SCHEME_CENTRAL)
        stencil_body<NSGB_SCHEME_CENTRAL, MODE_ROLLOUT, kTW, kTH, true>(a, k, u % gx, u / gx, gx, gy);
      else
        stencil_body<NSGB_SCHEME_UPWIND, MODE_ROLLOUT, kTW, kTH, true>(a, k, u % gx, u / gx, gx, gy);
      __syncthreads();
    }
    if (!grid_barrier(w.bar, w.poll_limit)) return;
    // 2.-4. the three FFT-Poisson passes
    for (int stage = 1; stage <= 3; ++stage) {
      for (int it = blockIdx.x; it < w.items[stage]; it += gridDim.x) {
        const int m = member_of(w.first[stage], w.count, it);
        const int u = it - __ldg(w.first[stage] + m);
        const FftPtrs f = w.dev[m].fft;
        const PersMember pm = w.pm[m];
        switch (pm.N) {
#define NSGB_PERS_CASE(NN)                                   \
  case NN:                                                   \
    if (stage == 1) rows_fwd_item<NN>(f, pm, tid, u);        \
    else if (stage == 2) cols_item<NN>(f, pm, tid, u);       \
    else rows_inv_item<NN>(f, pm, tid, u);                   \
    break;
          NSGB_PERS_SIZES(NSGB_PERS_CASE)
#undef NSGB_PERS_CASE
          default:
            break;
        }
        __syncthreads();
      }
      if (!grid_barrier(w.bar, w.poll_limit)) return;
    }
  }
}

// After the members' final projection and objective: non-finite objectives
// when the launch gave up at a barrier.
__global__ void k_ensemble_poison(const unsigned* __restrict__ bar, const SolveDev* __restrict__ dev, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count && bar[2] != 0u) gst(dev[k].J, __int_as_float(0x7fc00000));
}

}  // namespace pers

// Host side ------------------------------------------------------------------
void pers_tile(int N, int& tw, int& th) {
  (void)N;
  tw = pers::kTW;
  th = pers::kTH;
}

size_t pers_smem_bytes(int N) {
  const size_t stencil = sizeof(float) * StencilSmem<pers::kTW, pers::kTH>::FLOATS;
  const int T = pers::fft_T(N);
  const size_t stride = sizeof(float2) * (size_t)(fft::padlen(N) + 2);
  const size_t rows = (size_t)(pers::kThreads / T) * stride;  // the extra threads' buffers too
  const size_t cols = (size_t)pers::cols_KB(N) * stride;
  return std::max(stencil, std::max(rows, cols));
}

void pers_items(int N, int out[4]) {
  const int T = pers::fft_T(N);
  int tw, th;
  pers_tile(N, tw, th);
  out[0] = (N / tw) * (N / th);
  out[1] = out[3] = N / (2 * pers::rows_P(N));
  const int KB = pers::kThreads / T;
  out[2] = (N / 2 + 1 + KB - 1) / KB;
}

bool pers_supported(int N) { return N >= 64 && N <= 4096 && (N & (N - 1)) == 0; }

cudaError_t launch_ensemble_persistent(const PersWork& w, size_t smem, int sms, int* grid_out, cudaStream_t st) {
  cudaError_t e = raise_smem_limit(pers::k_ensemble_persistent);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pers::k_ensemble_persistent, pers::kThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int most = std::max(w.items[0], std::max(w.items[1], std::max(w.items[2], w.items[3])));
  const int grid = std::max(1, std::min(per_sm * sms, most));
  if (grid_out) *grid_out = grid;
  PersWork arg = w;
  void* args[] = {&arg};
  return cudaLaunchCooperativeKernel((const void*)pers::k_ensemble_persistent, dim3(grid), dim3(32, 8), args, smem,
                                     st);
}

cudaError_t launch_ensemble_poison(const unsigned* bar, const SolveDev* dev, int count, cudaStream_t st) {
  pers::k_ensemble_poison<<<(count + 127) / 128, 128, 0, st>>>(bar, dev, count);
  return cudaGetLastError();
}

NSGB_BOUNDS_UNIT(persistent, 6)

}  // namespace nsgb
