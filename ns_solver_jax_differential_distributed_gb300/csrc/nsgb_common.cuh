// Common device helpers for the GB300 Chorin-projection solver.
//
// Arithmetic that mirrors the reference's elementwise expressions is written
// with explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn, ...) so the
// compiler cannot contract it into FMAs: the stencils then round exactly like
// the reference's float32 array expressions (NS_solver.py:243-265, 687-697).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nsgb.h"

namespace nsgb {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// x / d rounded to nearest, for a divisor d whose correctly rounded
// reciprocal rd = RN(1/d) is precomputed: q = RN(x*rd) is within one ulp of
// x/d, the remainder x - q*d is exact in one FMA, and RN(q + r*rd) = RN(x/d)
// (Markstein's theorem, binary floating point, normal range).  Three
// instructions instead of a full IEEE division; the stencil tests compare the
// results bit for bit with NumPy's divisions.  (A -0 numerator gives +0, an
// infinite one NaN.)
__device__ __forceinline__ float divc(float x, float d, float rd) {
  const float q = __fmul_rn(x, rd);
  const float r = __fmaf_rn(-q, d, x);
  return __fmaf_rn(r, rd, q);
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// Constants of one solve, computed on the host in double precision and rounded
// to float32 the way the reference's weakly typed Python scalars are.
struct StepConsts {
  int N, logN;
  float L;      // grid length, float32 (grid x = L * (i/N))
  float h1;     // float32(dx)        upwind divisor   (NS_solver.py:261)
  float h2;     // float32(2*dx)      central divisor  (NS_solver.py:245)
  float dx2;    // float32(dx**2)     Laplacian divisor (NS_solver.py:255)
  float dt;     // float32(dt)
  float nu;     // float32(nu) (used when theta has 2 entries)
  float mu0, sigma0, C;
  float jscale; // dt * dx**2 in double, applied at the reduction
  // correctly rounded reciprocals of the divisors (for divc)
  float rh1, rh2, rdx2, rdt;
};

// Gaussian forcing fx at row i for time t (NS_solver.py:621-627):
//   mu = mu0 + sin(2 pi A t); sig = sigma0 + cos(2 pi B t)^2;
//   d = (x - mu) - round_half_even(x - mu); fx = C exp(-(d d) / (2 sig sig)).
struct ForcingRow {
  float mu, sig, twosig2;
};

__device__ __forceinline__ ForcingRow forcing_time(float A, float B, float t, const StepConsts& c) {
  const float twopi = 6.28318548202514648f;  // float32(2*pi)
  ForcingRow f;
  f.mu = fadd(c.mu0, sinf(fmul(fmul(twopi, A), t)));
  float cb = cosf(fmul(fmul(twopi, B), t));
  f.sig = fadd(c.sigma0, fmul(cb, cb));
  f.twosig2 = fmul(fmul(2.0f, f.sig), f.sig);
  return f;
}

__device__ __forceinline__ float grid_x(int i, const StepConsts& c) {
  // jnp.linspace(0, L, N, endpoint=False) = L * (i / N) in float32; exact
  // quotient for power-of-two N.
  return fmul(c.L, fdiv((float)i, (float)c.N));
}

__device__ __forceinline__ float forcing_fx(int i, const ForcingRow& f, const StepConsts& c) {
  float r = fsub(grid_x(i, c), f.mu);
  float d = fsub(r, rintf(r));
  return fmul(c.C, expf(fdiv(-fmul(d, d), f.twosig2)));
}

// Derivatives of fx with respect to mu and sigma (for the adjoint):
//   dfx/dmu = fx * d / sig^2,  dfx/dsig = fx * d^2 / sig^3.
__device__ __forceinline__ void forcing_fx_grad(int i, const ForcingRow& f, const StepConsts& c,
                                                float& fx, float& dmu, float& dsig) {
  float r = fsub(grid_x(i, c), f.mu);
  float d = fsub(r, rintf(r));
  fx = fmul(c.C, expf(fdiv(-fmul(d, d), f.twosig2)));
  float s2 = f.sig * f.sig;
  dmu = fx * d / s2;
  dsig = fx * d * d / (s2 * f.sig);
}

// Visit the cells (r, cc) of an H x W tile with a 32 x 8 thread block; the
// trip counts are compile-time, so the loop unrolls completely.
template <int H, int W, class F>
__device__ __forceinline__ void for2d(int tx, int ty, F&& f) {
#pragma unroll
  for (int r0 = 0; r0 < H; r0 += 8) {
#pragma unroll
    for (int c0 = 0; c0 < W; c0 += 32) {
      const int r = r0 + ty, cc = c0 + tx;
      if ((H % 8 == 0 || r < H) && (W % 32 == 0 || cc < W)) f(r, cc);
    }
  }
}

// Visit the cells (r, cc) of an H x W tile with the 256 threads of a block,
// flattened row-major so every lane has work (rows wider than a warp would
// otherwise leave most lanes idle in their last sweep); trip counts are
// compile-time, so the loop unrolls and W is a constant divisor.
template <int H, int W, class F>
__device__ __forceinline__ void forflat(int tid, F&& f) {
  constexpr int TOT = H * W;
#pragma unroll
  for (int e0 = 0; e0 < TOT; e0 += 256) {
    const int e = e0 + tid;
    if (TOT % 256 == 0 || e < TOT) {
      const int r = e / W;
      f(r, e - r * W);
    }
  }
}

// Stencil tile shapes (width x height) the kernels are instantiated for.
#define NSGB_STENCIL_TILES(X) X(16, 8) X(16, 16) X(32, 8) X(32, 16) X(64, 8) X(64, 16) X(128, 8)

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace nsgb
