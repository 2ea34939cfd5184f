// Common device helpers for the GB300 Chorin-projection solver.
//
// Arithmetic that mirrors the reference's elementwise expressions is written
// with explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn, ...) so the
// compiler cannot contract it into FMAs: the single-operator stencils then
// round exactly like the reference's float32 array expressions
// (NS_solver.py:243-265).  The fused step uses the folded forms below.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nsgb.h"

namespace nsgb {

// ------------------------------------------------------ bounds checking --
// Every global-memory access of the kernels goes through the accessors below.
// In the bounds-checking build (compiled with NSGB_CHECK_BOUNDS) each access
// is checked against the device ranges the library knows to be valid (the
// plans' tables, the no-allocation scratch, and the ranges the caller
// registered with nsgb_bounds_register); an access outside all of them is
// skipped (a load yields zero) and recorded, and the entry point returns
// NSGB_ERR_BOUNDS instead of faulting.  In the normal build the accessors are
// the plain accesses.
namespace bounds {
constexpr int kMaxRanges = 96;
struct Table {
  int n;
  int unit;                                  // translation unit of this copy (reported with the line)
  unsigned long long lo[kMaxRanges];         // [lo, hi) byte ranges
  unsigned long long hi[kMaxRanges];
  unsigned long long* report;                // device: count, first address, unit*100000+line, bytes
};
}  // namespace bounds

#ifdef NSGB_CHECK_BOUNDS
// One copy per translation unit, set by that unit's bounds_upload_<unit>.
static __constant__ bounds::Table g_bounds;

__device__ __noinline__ static void bounds_record(unsigned long long a, unsigned bytes, int line) {
  unsigned long long* r = g_bounds.report;
  if (!r) return;
  if (atomicAdd(r, 1ull) == 0ull) {
    r[1] = a;
    r[2] = (unsigned long long)g_bounds.unit * 100000ull + (unsigned long long)line;
    r[3] = bytes;
  }
}
__device__ __forceinline__ bool bounds_ok(const void* p, unsigned bytes, int line) {
  const unsigned long long a = (unsigned long long)p;
  for (int k = 0; k < g_bounds.n; ++k)
    if (a >= g_bounds.lo[k] && a + bytes <= g_bounds.hi[k]) return true;
  bounds_record(a, bytes, line);
  return false;
}
// Defines the host function that uploads a table to this unit's copy.
#define NSGB_BOUNDS_UNIT(name, id)                                                   \
  cudaError_t bounds_upload_##name(const bounds::Table& t) {                         \
    bounds::Table u = t;                                                              \
    u.unit = (id);                                                                    \
    return cudaMemcpyToSymbol(g_bounds, &u, sizeof u);                                \
  }
#else
__device__ __forceinline__ bool bounds_ok(const void*, unsigned, int) { return true; }
#define NSGB_BOUNDS_UNIT(name, id)
#endif

// Plain load / store.
template <class T>
__device__ __forceinline__ T gld(const T* p, int line = __builtin_LINE()) {
  return bounds_ok(p, sizeof(T), line) ? *p : T{};
}
template <class T>
__device__ __forceinline__ void gst(T* p, T v, int line = __builtin_LINE()) {
  if (bounds_ok(p, sizeof(T), line)) *p = v;
}
// Read-only-path load (__ldg), streaming load and store (__ldcs, __stcs).
template <class T>
__device__ __forceinline__ T gldg(const T* p, int line = __builtin_LINE()) {
  return bounds_ok(p, sizeof(T), line) ? __ldg(p) : T{};
}
template <class T>
__device__ __forceinline__ T gldcs(const T* p, int line = __builtin_LINE()) {
  return bounds_ok(p, sizeof(T), line) ? __ldcs(p) : T{};
}
template <class T>
__device__ __forceinline__ void gstcs(T* p, T v, int line = __builtin_LINE()) {
  if (bounds_ok(p, sizeof(T), line)) __stcs(p, v);
}
// L2-only load (__ldcg): for data other CTAs of the same launch wrote before
// a grid-wide barrier (the non-coherent and L1 paths may hold stale lines).
template <class T>
__device__ __forceinline__ T gldcg(const T* p, int line = __builtin_LINE()) {
  return bounds_ok(p, sizeof(T), line) ? __ldcg(p) : T{};
}
// Streamed load of a field: evict-first (__ldcs) in kernels whose inputs were
// written by earlier launches, L2-only (__ldcg) in a persistent kernel
// (COH) whose inputs other CTAs wrote during the launch.
template <bool COH, class T>
__device__ __forceinline__ T gldstream(const T* p, int line = __builtin_LINE()) {
  if constexpr (COH) {
    return gldcg(p, line);
  } else {
    return gldcs(p, line);
  }
}
// Read-only-path load (__ldg) of a field, or L2-only in a persistent kernel.
template <bool COH, class T>
__device__ __forceinline__ T gldfield(const T* p, int line = __builtin_LINE()) {
  if constexpr (COH) {
    return gldcg(p, line);
  } else {
    return gldg(p, line);
  }
}
// float4 views of float arrays (16-byte aligned offsets).
__device__ __forceinline__ float4 gldg4(const float* p, int line = __builtin_LINE()) {
  return gldg(reinterpret_cast<const float4*>(p), line);
}
__device__ __forceinline__ float4 gld4(const float* p, int line = __builtin_LINE()) {
  return gld(reinterpret_cast<const float4*>(p), line);
}
__device__ __forceinline__ void gst4(float* p, float4 v, int line = __builtin_LINE()) {
  gst(reinterpret_cast<float4*>(p), v, line);
}

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
  // coefficients of the fused step (each rounded once from double):
  float cP;     // dt / h2          projection     u = u* - cP (p(i+1) - p(i-1))
  float cD;     // 1 / (h2 dt)      rhs = cD (dx-difference + dy-difference)
  float cAc;    // dt / h2          central advection
  float cAu;    // dt / h1          upwind advection
  float dtdx2;  // dt / dx^2        (times nu: the diffusion coefficient)
};

// ------------------------------------------------------- fused-step cells --
// The per-cell arithmetic of the fused Chorin step (NS_solver.py:685-697):
// the reference's expressions with their constant divisions folded into the
// coefficients above and explicit FMAs, so a cell costs about half the
// instructions of the operator-by-operator form.  Every op is an explicitly
// rounded intrinsic, so each kernel that uses these helpers produces the same
// bits; against the reference's own rounding order the results differ by a
// few ulps per step.

// u = u* - dt dp/dh from the two neighbours of the projected direction.
__device__ __forceinline__ float fused_proj(float us, float p_plus, float p_minus, float cP) {
  return __fmaf_rn(-cP, __fsub_rn(p_plus, p_minus), us);
}

// u*next = u + dt (nu lap u + adv(u) + f) for one velocity component:
// o centre, l/r its i-1/i+1 neighbours, dn/up its j-1/j+1 neighbours, (ux, uy)
// the velocity at the cell, cL = dt nu / dx^2, cF = dt f.
template <int SCHEME>
__device__ __forceinline__ float fused_ustar(float o, float l, float r, float up, float dn, float ux, float uy,
                                             float cL, float cF, const StepConsts& c) {
  const float lap = __fmaf_rn(-4.0f, o, __fadd_rn(__fadd_rn(l, r), __fadd_rn(up, dn)));
  float a, cA;
  if (SCHEME == NSGB_SCHEME_CENTRAL) {
    a = __fmaf_rn(ux, __fsub_rn(r, l), __fmul_rn(uy, __fsub_rn(up, dn)));
    cA = c.cAc;
  } else {
    const float gx = ux >= 0.0f ? __fsub_rn(o, l) : __fsub_rn(r, o);
    const float gy = uy >= 0.0f ? __fsub_rn(o, dn) : __fsub_rn(up, o);
    a = __fmaf_rn(ux, gx, __fmul_rn(uy, gy));
    cA = c.cAu;
  }
  return __fadd_rn(o, __fmaf_rn(-cA, a, __fmaf_rn(cL, lap, cF)));
}

// rhs = div(u*)/dt from the i-neighbours of u*_x and the j-neighbours of u*_y.
__device__ __forceinline__ float fused_rhs(float xp, float xm, float yp, float ym, float cD) {
  return __fmul_rn(__fadd_rn(__fsub_rn(xp, xm), __fsub_rn(yp, ym)), cD);
}

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

// A double-float value hi + lo (|lo| <= ulp(hi)/2): about 48 significant bits
// from float operations, which run at the full FP32 rate where FP64 runs at a
// small fraction of it.
struct DFloat {
  float hi, lo;
};

// hi + lo of a + b: Knuth's TwoSum of the high parts (an error-free
// transformation, so the result does not depend on the operand order), the
// low parts added to its error, renormalised by Dekker's FastTwoSum.
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  const float t = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
  const float hi = __fadd_rn(s, t);
  return {hi, __fsub_rn(t, __fsub_rn(hi, s))};
}

__device__ __forceinline__ DFloat warp_sum_df(DFloat v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const DFloat w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}

}  // namespace nsgb
