// Bodies of the FFT-Poisson passes (two-for-one row transforms, column
// transform with the Poisson multiplier), shared by the pass kernels
// (nsgb_fft_kernels.cu) and the persistent ensemble kernel
// (nsgb_ens_persistent.cu).
#pragma once

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
// Transform thread j of row pair pp of a CTA carrying P row pairs, rows
// [bx * 2P, +2P) (blockDim = (T, P): j = threadIdx.x, pp = threadIdx.y).  A
// persistent kernel passes more threads than pairs: those with pp >= P
// transform a copy of the last pair in their own buffer and store nothing,
// so every thread reaches the transform's barriers.  COH: L2-only loads of
// data other CTAs of the same launch wrote.
template <int N, int E, bool COH = false>
__device__ __forceinline__ void rows_fwd_body(const float* __restrict__ rhs, float2* __restrict__ spec,
                                              const float2* __restrict__ tw, int j, int pp, int P, int bx) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  float2* sb = smem2 + pp * pair_stride<N>();
  const int RB = 2 * P;
  const int i0 = bx * RB;
  // (only a persistent kernel, COH, has threads beyond its P pairs)
  const float* ra = rhs + (size_t)(i0 + 2 * ((COH && pp >= P) ? P - 1 : pp)) * N;
  const float* rb = ra + N;

  // Row data is read once: evict-first loads keep the twiddle tables in L1.
  float2 a[E];
#pragma unroll
  for (int s = 0; s < E; ++s)
    a[s] = make_float2(gldstream<COH>(ra + j + s * T), gldstream<COH>(rb + j + s * T));
  fft::block_fft<N, false, E>(a, sb, j, tw);
  __syncthreads();
  fft::store_strided<T, E>(a, sb, j);
  __syncthreads();

  const int tid = pp * T + j;  // >= nth for the extra threads of a persistent CTA
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

// Transform thread j of spectrum row y of a CTA carrying KB rows, rows
// [bx * KB, +KB) (blockDim = (T, KB): j = threadIdx.x, y = threadIdx.y).
template <int N, int E, bool COH = false>
__device__ __forceinline__ void cols_body(float2* __restrict__ spec, const float2* __restrict__ tw,
                                          const float* __restrict__ k2, float scale, int j, int y, int KB,
                                          int bx) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  float2* sb = smem2 + y * pair_stride<N>();
  // N/2 + 1 rows; the last CTA may hold rows past N/2, which recompute row
  // N/2 and do not store.
  const int kreq = bx * KB + y;
  const int ky = kreq < H ? kreq : H;
  float2* row = spec + (size_t)ky * N;

  float2 a[E];
#pragma unroll
  for (int s = 0; s < E; ++s) a[s] = gldstream<COH>(row + j + s * T);
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
// Thread layout as for rows_fwd_body; the extra threads of a persistent CTA
// (pp >= P) transform their own buffer and store nothing.
template <int N, int E, bool COH = false>
__device__ __forceinline__ void rows_inv_body(const float2* __restrict__ spec, float* __restrict__ p,
                                              const float2* __restrict__ tw, int j, int pp, int P, int bx) {
  constexpr int T = N / E;
  constexpr int H = N / 2;
  extern __shared__ float2 smem2[];
  const int RB = 2 * P;
  const int i0 = bx * RB;
  const int tid = pp * T + j;  // >= nth for the extra threads of a persistent CTA
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
      for (int u = 0; u < 8; ++u) v[u] = gldstream<COH>(src(e + u * nth));
#pragma unroll
      for (int u = 0; u < 8; ++u) stage(e + u * nth, v[u]);
    }
    for (; e < tot; e += nth) stage(e, gldstream<COH>(src(e)));
  }
  __syncthreads();

  float2* sb = smem2 + pp * pair_stride<N>();
  float2 a[E];
  fft::load_strided<T, E>(a, sb, j);
  __syncthreads();
  fft::block_fft<N, true, E>(a, sb, j, tw);
  if (COH && pp >= P) return;
  float* ra = p + (size_t)(i0 + 2 * pp) * N;
  float* rb = ra + N;
#pragma unroll
  for (int s = 0; s < E; ++s) {
    gst(ra + j + s * T, a[s].x);
    gst(rb + j + s * T, a[s].y);
  }
}

}  // namespace nsgb
