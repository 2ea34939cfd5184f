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
#include "nsgb_fft_bodies.cuh"

namespace nsgb {

// ---------------------------------------------------------------- kernels --
// Radix 16 keeps about 64 registers per thread; radix 8 about 40, so its
// column kernel is bounded for three 512-thread CTAs per SM.
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_fwd(const float* __restrict__ rhs, float2* __restrict__ spec,
                                                   const float2* __restrict__ tw) {
  rows_fwd_body<N, E>(rhs, spec, tw, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
}
template <int N, int E>
__global__ void __launch_bounds__(512, E == 8 ? 3 : 2) k_cols(float2* __restrict__ spec,
                                                              const float2* __restrict__ tw,
                                                              const float* __restrict__ k2, float scale) {
  cols_body<N, E>(spec, tw, k2, scale, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
}
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_inv(const float2* __restrict__ spec, float* __restrict__ p,
                                                   const float2* __restrict__ tw) {
  rows_inv_body<N, E>(spec, p, tw, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
}
// Ensemble variants: blockIdx.y selects the member.
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_fwd_b(const SolveDev* __restrict__ sv,
                                                     const float2* __restrict__ tw) {
  const FftPtrs f = sv[blockIdx.y].fft;
  rows_fwd_body<N, E>(f.rhs, f.spec, tw, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
}
template <int N, int E>
__global__ void __launch_bounds__(512, E == 8 ? 3 : 2) k_cols_b(const SolveDev* __restrict__ sv,
                                                                const float2* __restrict__ tw,
                                                                const float* __restrict__ k2, float scale) {
  cols_body<N, E>(sv[blockIdx.y].fft.spec, tw, k2, scale, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
}
template <int N, int E>
__global__ void __launch_bounds__(1024) k_rows_inv_b(const SolveDev* __restrict__ sv,
                                                     const float2* __restrict__ tw) {
  const FftPtrs f = sv[blockIdx.y].fft;
  rows_inv_body<N, E>(f.spec, f.p, tw, threadIdx.x, threadIdx.y, blockDim.y, blockIdx.x);
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
