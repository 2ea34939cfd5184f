// Block-level FFT building blocks for power-of-two lengths 16..4096.
//
// A transform of length N is carried by T = N/E threads, each holding E
// complex values in registers (E = 16 or 8, at most N).  Thread j holds elements j + s*T
// (s = 0..E-1) on entry and X[j + s*T] on exit, so the first pass reads and
// the last pass writes "natural" strided positions; rows stored contiguously
// in global memory are therefore loaded and stored fully coalesced.
//
// The transform is the radix-E Stockham autosort algorithm (a final pass of
// smaller radix when log2(N) is not a multiple of log2(E)).  Radix 8 needs
// half the registers per thread of radix 16 for the same arithmetic, so twice
// as many threads (and warps) carry a transform.  Between passes the values
// are exchanged through shared memory as float2, padded by one element every
// 16 (index i -> i + i/16), which keeps the 64-bit pass writes and reads
// bank-conflict free within each half warp.  Twiddles come from per-pass tables computed on
// the host in double precision and rounded to float: the pass with stride NS
// and radix RP stores W_{NS*RP}^{bm*r} at [r*NS + bm], so the twiddle loads of
// a warp (consecutive bm) are contiguous.  A plan holds the radix-16 tables
// followed by the radix-8 tables (host_twiddles).
#pragma once

#include <cmath>

#include "nsgb_common.cuh"

namespace nsgb {
namespace fft {

__host__ __device__ constexpr int ept(int N) { return N < 16 ? N : 16; }
__host__ __device__ constexpr int padlen(int N) { return N + N / 16 + 4; }
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }

template <int R>
__device__ __forceinline__ constexpr int bitrev(int k) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (k & 1);
    k >>= 1;
  }
  return r;
}

// cos / sin of 2*pi*m/16 for m = 0..7
__device__ __forceinline__ float c16(int m) {
  switch (m) {
    case 0: return 1.0f;
    case 1: return 0.923879532511286756f;
    case 2: return 0.707106781186547524f;
    case 3: return 0.382683432365089772f;
    case 4: return 0.0f;
    case 5: return -0.382683432365089772f;
    case 6: return -0.707106781186547524f;
    default: return -0.923879532511286756f;
  }
}
__device__ __forceinline__ float s16(int m) {
  switch (m) {
    case 0: return 0.0f;
    case 1: return 0.382683432365089772f;
    case 2: return 0.707106781186547524f;
    case 3: return 0.923879532511286756f;
    case 4: return 1.0f;
    case 5: return 0.923879532511286756f;
    case 6: return 0.707106781186547524f;
    default: return 0.382683432365089772f;
  }
}

// d * exp(-+ 2 pi i m / 16): forward uses the minus sign.
template <bool INV>
__device__ __forceinline__ float2 rot16(float2 d, int m) {
  if (m == 0) return d;
  if (m == 4) return INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  const float c = c16(m);
  const float s = INV ? s16(m) : -s16(m);
  return make_float2(d.x * c - d.y * s, d.x * s + d.y * c);
}

// In-register DFT of size R (2, 4, 8 or 16): natural order in and out.
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
#pragma unroll
  for (int len = R; len >= 2; len >>= 1) {
    const int half = len >> 1;
#pragma unroll
    for (int s = 0; s < R; s += len) {
#pragma unroll
      for (int t = 0; t < half; ++t) {
        const float2 u = a[s + t];
        const float2 v = a[s + t + half];
        a[s + t] = cadd(u, v);
        a[s + t + half] = rot16<INV>(csub(u, v), t * (16 / len));
      }
    }
  }
  float2 b[R];
#pragma unroll
  for (int k = 0; k < R; ++k) b[k] = a[bitrev<R>(k)];
#pragma unroll
  for (int k = 0; k < R; ++k) a[k] = b[k];
}

// Offset (in complex entries) of the twiddle table of the pass with stride
// NS in the radix-R tables: the passes before it all have radix R and stride
// R, R^2, ...
template <int R>
__host__ __device__ constexpr int tw_offset(int NS) {
  int off = 0;
  for (int ns = R; ns < NS; ns *= R) off += R * ns;
  return off;
}
// Twiddle entries of the radix-R tables for length N.
template <int R>
__host__ __device__ constexpr int tw_entries(int N) {
  int off = 0;
  for (int ns = R; ns < N; ns *= R) off += ((N / ns >= R) ? R : N / ns) * ns;
  return off > 0 ? off : 1;
}
// Entries of a plan's table (radix 16, then radix 8) and the radix-8 offset.
__host__ __device__ constexpr int tw_total(int N) { return tw_entries<16>(N) + tw_entries<8>(N); }
__host__ __device__ constexpr int tw8_offset(int N) { return tw_entries<16>(N); }

// Fill a plan's twiddle table (tw_total(N) entries): per pass with stride ns
// and radix rp, W_{ns*rp}^{bm*r} at [off + r*ns + bm], in double then rounded.
inline void host_twiddles(int N, float2* out) {
  for (int i = 0; i < tw_total(N); ++i) out[i] = make_float2(1.f, 0.f);
  for (int R = 16, base = 0; R >= 8; base += tw_entries<16>(N), R /= 2) {
    for (int ns = R, off = base; ns < N; off += (N / ns >= R ? R : N / ns) * ns, ns *= R) {
      const int rp = N / ns >= R ? R : N / ns;
      for (int r = 1; r < rp; ++r)
        for (int bm = 0; bm < ns; ++bm) {
          const double ang = -2.0 * M_PI * (double)bm * r / ((double)ns * rp);
          out[off + r * ns + bm] = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
    }
  }
}

// a[s] = buffer[pad(j + s*T)], s = 0..E-1 (and the store of the same
// positions): with T a multiple of 16 the padded positions are pad(j) plus
// constants.
template <int T, int E>
__device__ __forceinline__ void load_strided(float2 (&a)[E], const float2* __restrict__ sb, int j) {
  if constexpr (T % 16 == 0) {
    const float2* src = sb + pad(j);
#pragma unroll
    for (int s = 0; s < E; ++s) a[s] = src[s * (T + T / 16)];
  } else {
#pragma unroll
    for (int s = 0; s < E; ++s) a[s] = sb[pad(j + s * T)];
  }
}
template <int T, int E>
__device__ __forceinline__ void store_strided(const float2 (&a)[E], float2* __restrict__ sb, int j) {
  if constexpr (T % 16 == 0) {
    float2* dst = sb + pad(j);
#pragma unroll
    for (int s = 0; s < E; ++s) dst[s * (T + T / 16)] = a[s];
  } else {
#pragma unroll
    for (int s = 0; s < E; ++s) sb[pad(j + s * T)] = a[s];
  }
}

// Barrier of the threads that carry one transform: the whole CTA (BAR = 0)
// or the NT threads of a warp group using hardware barrier BAR (kernels in
// which other warps run other work at the same time).
template <int BAR, int NT>
__device__ __forceinline__ void group_sync() {
  if constexpr (BAR == 0) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NT) : "memory");
  }
}

// One Stockham pass (stride NS) and, recursively, the remaining passes.
template <int N, int NS, bool INV, int E, int BAR = 0>
__device__ __forceinline__ void pass(float2 (&a)[E], float2* __restrict__ sb, int j,
                                     const float2* __restrict__ tw) {
  static_assert(E == 16 || E == 8 || E == N, "radix");
  constexpr int T = N / E;
  constexpr int REM = N / NS;
  constexpr int RP = REM >= E ? E : REM;
  constexpr int Q = E / RP;
  constexpr bool LAST = (NS * RP == N);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = j + q * T;
    float2 x[RP];
#pragma unroll
    for (int r = 0; r < RP; ++r) x[r] = a[q + r * Q];
    if constexpr (NS > 1 && RP == 16) {
      // W^r for r = 1..15 from the table's W^1, W^2, W^4, W^8 and at most two
      // complex products each (a few ulps), so a radix-16 pass issues 4
      // twiddle loads instead of 15
      const int bm = b & (NS - 1);
      const float2* __restrict__ tp = tw + tw_offset<E>(NS) + bm;
      float2 w1 = gldg(tp + NS), w2 = gldg(tp + 2 * NS), w4 = gldg(tp + 4 * NS), w8 = gldg(tp + 8 * NS);
      if (INV) {
        w1.y = -w1.y;
        w2.y = -w2.y;
        w4.y = -w4.y;
        w8.y = -w8.y;
      }
      const float2 w3 = cmul(w2, w1), w12 = cmul(w8, w4);
      x[1] = cmul(x[1], w1);
      x[2] = cmul(x[2], w2);
      x[3] = cmul(x[3], w3);
      x[4] = cmul(x[4], w4);
      x[5] = cmul(x[5], cmul(w4, w1));
      x[6] = cmul(x[6], cmul(w4, w2));
      x[7] = cmul(x[7], cmul(w4, w3));
      x[8] = cmul(x[8], w8);
      x[9] = cmul(x[9], cmul(w8, w1));
      x[10] = cmul(x[10], cmul(w8, w2));
      x[11] = cmul(x[11], cmul(w8, w3));
      x[12] = cmul(x[12], w12);
      x[13] = cmul(x[13], cmul(w12, w1));
      x[14] = cmul(x[14], cmul(w12, w2));
      x[15] = cmul(x[15], cmul(w12, w3));
    } else if constexpr (NS > 1) {
      const int bm = b & (NS - 1);
      const float2* __restrict__ tp = tw + tw_offset<E>(NS) + bm;
#pragma unroll
      for (int r = 1; r < RP; ++r) {
        float2 w = gldg(tp + r * NS);
        if (INV) w.y = -w.y;
        x[r] = cmul(x[r], w);
      }
    }
    dft<RP, INV>(x);
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < RP; ++r) a[q + r * Q] = x[r];
    } else {
      const int base = (b / NS) * (NS * RP) + (b & (NS - 1));
      if constexpr (NS == 1 || NS % 16 == 0) {
        // base + r stays inside one 16-entry block (NS = 1) or r * NS is a
        // multiple of 16: the padded positions are pad(base) plus constants
        float2* dst = sb + pad(base);
#pragma unroll
        for (int r = 0; r < RP; ++r) dst[r * (NS + NS / 16)] = x[r];
      } else {
#pragma unroll
        for (int r = 0; r < RP; ++r) sb[pad(base + r * NS)] = x[r];
      }
    }
  }
  if constexpr (!LAST) {
    group_sync<BAR, T>();
    load_strided<T, E>(a, sb, j);
    group_sync<BAR, T>();
    pass<N, NS * RP, INV, E, BAR>(a, sb, j, tw);
  }
}

// Full FFT of length N (unnormalised; INV uses exp(+2 pi i ...)) in radix E,
// with `tw` the radix-E tables.  Every thread of the CTA (BAR = 0), or of the
// N/E-thread warp group synchronised by barrier BAR, must call it: it
// synchronises those threads between passes.  On return the exchange buffer
// is free for reuse without a further barrier only after their next
// synchronisation.
template <int N, bool INV, int E, int BAR = 0>
__device__ __forceinline__ void block_fft(float2 (&a)[E], float2* sb, int j, const float2* __restrict__ tw) {
  pass<N, 1, INV, E, BAR>(a, sb, j, tw);
}

}  // namespace fft
}  // namespace nsgb
