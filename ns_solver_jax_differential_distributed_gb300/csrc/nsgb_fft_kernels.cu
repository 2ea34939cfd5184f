// FFT-Poisson kernels: the hand-written replacement of SpectralPoissonSolver
// (NS_solver.py:507-527).
//
// The real N x N right-hand side is transformed in two passes:
//   rows (along y, contiguous): two real rows a, b are packed as a + i b, one
//     complex length-N FFT gives both half spectra X_a[k], X_b[k], k=0..N/2.
//     The half spectrum is stored transposed, spec[k][i] (k = 0..N/2, i
//     contiguous): N/2 + 1 rows of N complex values.
//   columns (along x): each spec[k] row is transformed, multiplied by
//     -1/|k|^2 (0 at k = 0; NS_solver.py:521, 525-526), transformed back and
//     written in place.  Every ky column has its own row -- in particular the
//     DC and Nyquist columns are never packed together -- so a field that is
//     constant along y keeps exactly zero spectrum at ky != 0, as the
//     reference's C2C transforms do (its zero-state runs stay exactly
//     y-independent, which the upwind study at the diffusive stability limit
//     relies on).
//   rows again: the inverse two-for-one C2R transform writes p.
// All scale factors (the 1/2 of the two-for-one split and the 1/N^2 of ifft2)
// are powers of two folded into the spectral multiplier, so they round
// exactly.
#include "nsgb_fft.cuh"
#include "nsgb_internal.h"

namespace nsgb {

using fft::ept;
using fft::pad;
using fft::padlen;

// Per-transform exchange buffer stride in float2 (padded length plus a small
// skew so the buffers of different transforms start in different banks).
template <int N>
__host__ __device__ constexpr int pair_stride() {
  return padlen(N) + 2;
}

// ---------------------------------------------------------------- rows fwd --
// blockDim = (T, P): P row pairs per CTA, rows [blockIdx.x * 2P, +2P).
template <int N, int E>
__device__ __forceinline__ void rows_fwd_body(const float* __restrict__ rhs, float2* __restrict__ spec,
                                              const float2* __restrict__ tw) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  const int j = threadIdx.x, pp = threadIdx.y, P = blockDim.y;
  float2* sb = smem2 + pp * pair_stride<N>();
  const int RB = 2 * P;
  const int i0 = blockIdx.x * RB;
  const float* ra = rhs + (size_t)(i0 + 2 * pp) * N;
  const float* rb = ra + N;

  // Row data is read once: evict-first loads keep the twiddle tables in L1.
  float2 a[E];
#pragma unroll
  for (int s = 0; s < E; ++s) a[s] = make_float2(gldcs(ra + j + s * T), gldcs(rb + j + s * T));
  fft::block_fft<N, false, E>(a, sb, j, tw);
  __syncthreads();
  fft::store_strided<T, E>(a, sb, j);
  __syncthreads();

  const int tid = threadIdx.y * T + threadIdx.x;
  const int nth = T * P;
  const int lp = __ffs(P) - 1;  // P is a power of two
  // Element e = k * P + q (row pair q of the CTA, frequency k) for e = tid,
  // tid + nth, ...: both rows of a pair come from one read of Z[k] and
  // Z[N-k] and leave in one 16-byte store; a warp's stores cover whole
  // 32-byte sectors when P >= 2.
  // 2 X_a[k] = Z[k] + conj(Z[N-k]);  2 X_b[k] = -i (Z[k] - conj(Z[N-k]))
  for (int e = tid; e < P * (H + 1); e += nth) {
    const int q = e & (P - 1);
    const int k = e >> lp;
    const float2* pb = smem2 + q * pair_stride<N>();
    const float2 zk = pb[pad(k)], wk = pb[pad((N - k) & (N - 1))];
    gst(reinterpret_cast<float4*>(spec + (size_t)k * N + i0 + 2 * q),
        make_float4(zk.x + wk.x, zk.y - wk.y, zk.y + wk.y, wk.x - zk.x));
  }
}

// ----------------------------------------------------------------- columns --
// Spectral multiplier  -1/(kx^2 + ky^2) * scale, 0 where the sum is 0.
__device__ __forceinline__ float poisson_mult(float k2x, float k2y, float scale) {
  const float den = k2x + k2y;
  // __frcp_rn is the correctly rounded 1/den, the same float as 1.0f / den
  const float inv = (den == 0.0f) ? 0.0f : __frcp_rn(den);
  return -inv * scale;
}

// blockDim = (T, KB): KB spectrum rows per CTA, rows [blockIdx.x * KB, +KB).
template <int N, int E>
__device__ __forceinline__ void cols_body(float2* __restrict__ spec, const float2* __restrict__ tw,
                                          const float* __restrict__ k2, float scale) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  const int j = threadIdx.x, y = threadIdx.y;
  float2* sb = smem2 + y * pair_stride<N>();
  // N/2 + 1 rows; the last CTA may hold rows past N/2, which recompute row
  // N/2 and do not store.
  const int kreq = blockIdx.x * blockDim.y + y;
  const int ky = kreq < H ? kreq : H;
  float2* row = spec + (size_t)ky * N;

  float2 a[E];
#pragma unroll
  for (int s = 0; s < E; ++s) a[s] = gldcs(row + j + s * T);
  fft::block_fft<N, false, E>(a, sb, j, tw);

  const float k2y = gldg(k2 + ky);
#pragma unroll
  for (int s = 0; s < E; ++s) {
    const float g = poisson_mult(gldg(k2 + j + s * T), k2y, scale);
    a[s] = make_float2(a[s].x * g, a[s].y * g);
  }
  fft::block_fft<N, true, E>(a, sb, j, tw);
  __syncthreads();  // rows clamped to N/2 were loaded by other threads
  if (kreq <= H) {
#pragma unroll
    for (int s = 0; s < E; ++s) gst(row + j + s * T, a[s]);
  }
}

// ---------------------------------------------------------------- rows inv --
template <int N, int E>
__device__ __forceinline__ void rows_inv_body(const float2* __restrict__ spec, float* __restrict__ p,
                                              const float2* __restrict__ tw) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  const int j = threadIdx.x, pp = threadIdx.y, P = blockDim.y;
  const int RB = 2 * P;
  const int i0 = blockIdx.x * RB;
  const int tid = threadIdx.y * T + threadIdx.x;
  const int nth = T * P;

  // Stage Z[m] = X_a[m] + i X_b[m] of each row pair (m > N/2 from the
  // conjugate symmetry of the two real rows: Z[N-k] = conj(X_a[k]) + i
  // conj(X_b[k])) straight into the pair's exchange buffer: element e = k * P
  // + q reads X_a[k], X_b[k] of pair q as one 16-byte load (a warp covers
  // whole 32-byte sectors when P >= 2) and writes Z[k] and Z[N-k].  DC and
  // Nyquist of a real row are real: their imaginary parts (rounding noise of
  // the column pass) are dropped, as Re(ifft2) drops them.  The loads are
  // issued in batches of 8 before their shared-memory stores, so their
  // latencies overlap.
  const int tot = P * (H + 1);
  const int lp = __ffs(P) - 1;  // P is a power of two
  auto stage = [&](int e, float4 v) {
    const int q = e & (P - 1);
    const int k = e >> lp;
    float2* pb = smem2 + q * pair_stride<N>();
    if (k == 0 || k == H) {
      pb[pad(k)] = make_float2(v.x, v.z);
    } else {
      pb[pad(k)] = make_float2(v.x - v.w, v.y + v.z);
      pb[pad(N - k)] = make_float2(v.x + v.w, v.z - v.y);
    }
  };
  auto src = [&](int e) {
    return reinterpret_cast<const float4*>(spec + (size_t)(e >> lp) * N + i0 + 2 * (e & (P - 1)));
  };
  {
    int e = tid;
    for (; e + 7 * nth < tot; e += 8 * nth) {
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = gldcs(src(e + u * nth));
#pragma unroll
      for (int u = 0; u < 8; ++u) stage(e + u * nth, v[u]);
    }
    for (; e < tot; e += nth) stage(e, gldcs(src(e)));
  }
  __syncthreads();

  float2* sb = smem2 + pp * pair_stride<N>();
  float2 a[E];
  fft::load_strided<T, E>(a, sb, j);
  __syncthreads();
  fft::block_fft<N, true, E>(a, sb, j, tw);
  float* ra = p + (size_t)(i0 + 2 * pp) * N;
  float* rb = ra + N;
#pragma unroll
  for (int s = 0; s < E; ++s) {
    gst(ra + j + s * T, a[s].x);
    gst(rb + j + s * T, a[s].y);
  }
}

// ---------------------------------------------------------------- kernels --
// Radix 16 keeps about 64 registers per thread; radix 8 about 40, so its
// column kernel is bounded for three 512-thread CTAs per SM.
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_fwd(const float* __restrict__ rhs, float2* __restrict__ spec,
                                                   const float2* __restrict__ tw) {
  rows_fwd_body<N, E>(rhs, spec, tw);
}
template <int N, int E>
__global__ void __launch_bounds__(512, E == 8 ? 3 : 2) k_cols(float2* __restrict__ spec,
                                                              const float2* __restrict__ tw,
                                                              const float* __restrict__ k2, float scale) {
  cols_body<N, E>(spec, tw, k2, scale);
}
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_inv(const float2* __restrict__ spec, float* __restrict__ p,
                                                   const float2* __restrict__ tw) {
  rows_inv_body<N, E>(spec, p, tw);
}
// Ensemble variants: blockIdx.y selects the member.
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_fwd_b(const SolveDev* __restrict__ sv,
                                                     const float2* __restrict__ tw) {
  const FftPtrs f = sv[blockIdx.y].fft;
  rows_fwd_body<N, E>(f.rhs, f.spec, tw);
}
template <int N, int E>
__global__ void __launch_bounds__(512, E == 8 ? 3 : 2) k_cols_b(const SolveDev* __restrict__ sv,
                                                                const float2* __restrict__ tw,
                                                                const float* __restrict__ k2, float scale) {
  cols_body<N, E>(sv[blockIdx.y].fft.spec, tw, k2, scale);
}
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_inv_b(const SolveDev* __restrict__ sv,
                                                     const float2* __restrict__ tw) {
  const FftPtrs f = sv[blockIdx.y].fft;
  rows_inv_body<N, E>(f.spec, f.p, tw);
}

// ------------------------------------------------------------- launchers --
template <int N, int E>
static const float2* radix_tables(const FftLaunch& L) {
  return L.tw + (E == 8 ? fft::tw8_offset(N) : 0);
}


template <int N, int E>
static cudaError_t stage_rows_fwd(const FftLaunch& L, const SolveDev* sv, int count, cudaStream_t st) {
  constexpr int T = N / E;
  const int P = L.rows_per_cta / 2;
  const size_t smem = (size_t)P * pair_stride<N>() * sizeof(float2);
  if (smem > 48 * 1024) {
    const cudaError_t e = raise_smem_limit(sv ? (const void*)k_rows_fwd_b<N, E> : (const void*)k_rows_fwd<N, E>);
    if (e != cudaSuccess) return e;
  }
  if (sv)
    k_rows_fwd_b<N, E><<<dim3(N / (2 * P), count), dim3(T, P), smem, st>>>(sv, radix_tables<N, E>(L));
  else
    k_rows_fwd<N, E><<<N / (2 * P), dim3(T, P), smem, st>>>(L.rhs, L.spec, radix_tables<N, E>(L));
  return cudaGetLastError();
}

template <int N, int E>
static cudaError_t stage_cols(const FftLaunch& L, const SolveDev* sv, int count, cudaStream_t st) {
  constexpr int T = N / E;
  const int KB = L.cols_per_cta;
  const size_t smem = (size_t)KB * pair_stride<N>() * sizeof(float2);
  if (smem > 48 * 1024) {
    const cudaError_t e = raise_smem_limit(sv ? (const void*)k_cols_b<N, E> : (const void*)k_cols<N, E>);
    if (e != cudaSuccess) return e;
  }
  if (sv)
    k_cols_b<N, E><<<dim3((N / 2) / KB + 1, count), dim3(T, KB), smem, st>>>(sv, radix_tables<N, E>(L), L.k2,
                                                                            L.scale);
  else
    k_cols<N, E><<<(N / 2) / KB + 1, dim3(T, KB), smem, st>>>(L.spec, radix_tables<N, E>(L), L.k2, L.scale);
  return cudaGetLastError();
}

template <int N, int E>
static cudaError_t stage_rows_inv(const FftLaunch& L, const SolveDev* sv, int count, cudaStream_t st) {
  constexpr int T = N / E;
  const int P = L.rows_per_cta / 2;
  const size_t smem = (size_t)P * pair_stride<N>() * sizeof(float2);
  if (smem > 48 * 1024) {
    const cudaError_t e = raise_smem_limit(sv ? (const void*)k_rows_inv_b<N, E> : (const void*)k_rows_inv<N, E>);
    if (e != cudaSuccess) return e;
  }
  if (sv)
    k_rows_inv_b<N, E><<<dim3(N / (2 * P), count), dim3(T, P), smem, st>>>(sv, radix_tables<N, E>(L));
  else
    k_rows_inv<N, E><<<N / (2 * P), dim3(T, P), smem, st>>>(L.spec, L.p, radix_tables<N, E>(L));
  return cudaGetLastError();
}

template <int N>
static cudaError_t launch_poisson_fft(const FftLaunch& L, const SolveDev* sv, int count, cudaStream_t st) {
  const bool r8 = L.radix_rows == 8, c8 = L.radix_cols == 8;
  cudaError_t e = cudaSuccess;
  if (sv || L.rhs) e = r8 ? stage_rows_fwd<N, 8>(L, sv, count, st) : stage_rows_fwd<N, fft::ept(N)>(L, sv, count, st);
  if (e == cudaSuccess && (sv || L.do_cols))
    e = c8 ? stage_cols<N, 8>(L, sv, count, st) : stage_cols<N, fft::ept(N)>(L, sv, count, st);
  if (e == cudaSuccess && (sv || L.p))
    e = r8 ? stage_rows_inv<N, 8>(L, sv, count, st) : stage_rows_inv<N, fft::ept(N)>(L, sv, count, st);
  return e;
}

size_t fft_rows_smem_bytes(int N, int rows_per_cta) {
  return (size_t)(rows_per_cta / 2) * (padlen(N) + 2) * sizeof(float2);
}
size_t fft_cols_smem_bytes(int N, int cols_per_cta) {
  return (size_t)cols_per_cta * (padlen(N) + 2) * sizeof(float2);
}

static cudaError_t dispatch(int N, const FftLaunch& L, const SolveDev* sv, int count, cudaStream_t st) {
  switch (N) {
    case 16: return launch_poisson_fft<16>(L, sv, count, st);
    case 32: return launch_poisson_fft<32>(L, sv, count, st);
    case 64: return launch_poisson_fft<64>(L, sv, count, st);
    case 128: return launch_poisson_fft<128>(L, sv, count, st);
    case 256: return launch_poisson_fft<256>(L, sv, count, st);
    case 512: return launch_poisson_fft<512>(L, sv, count, st);
    case 1024: return launch_poisson_fft<1024>(L, sv, count, st);
    case 2048: return launch_poisson_fft<2048>(L, sv, count, st);
    case 4096: return launch_poisson_fft<4096>(L, sv, count, st);
    case 8192: return launch_poisson_fft<8192>(L, sv, count, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t poisson_fft(int N, const FftLaunch& L, cudaStream_t st) { return dispatch(N, L, nullptr, 0, st); }

cudaError_t poisson_fft_batch(int N, const FftLaunch& L, const SolveDev* solves, int count, cudaStream_t st) {
  return dispatch(N, L, solves, count, st);
}

NSGB_BOUNDS_UNIT(fft, 2)

}  // namespace nsgb
