// Building blocks of the row-streaming stencil kernels (the forward step in
// nsgb_stencil.cu, the adjoint step in nsgb_adjoint.cu).
//
// A CTA owns a band of W columns (W = N: whole rows, the periodic wrap stays
// inside the CTA; W < N: one extra group of four halo columns on each side,
// computed but not stored) and marches down a range of rows.  Thread g owns
// the four consecutive columns of group g.  Input rows arrive in
// shared-memory rings, each ring row holding the band plus four columns on
// each side (and four pad floats at both ends), by per-thread asynchronous
// 16-byte copies.
#pragma once

#include <stdint.h>

#include "nsgb_common.cuh"

namespace nsgb {
namespace rows {

__host__ __device__ inline int band_width(int N, int tw) { return tw < N ? tw : N; }
__host__ __device__ inline int groups(int N, int W) { return W == N ? N / 4 : W / 4 + 2; }
__host__ __device__ inline int threads(int N, int W) { return (groups(N, W) + 31) / 32 * 32; }
// ring row: 4 pad floats, the W + 8 columns from j0 - 4 (W < N) or from -4
// (W = N, wrapped copies at both ends), 4 pad floats
__host__ __device__ inline int ring_stride(int W) { return W + 16; }

// Input rows are read once: their copies carry an L2 evict-first policy, so
// they do not push the FFT passes' fields out of L2.
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void cp16(float* dst_smem, const float* src, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst_smem)),
               "l"(src), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

__device__ __forceinline__ void st4(float* __restrict__ base, size_t off, const float (&v)[4]) {
  *reinterpret_cast<float4*>(base + off) = make_float4(v[0], v[1], v[2], v[3]);
}
// Evict-first store, for fields read only after the FFT passes (u*next), so
// they do not push the passes' inputs out of L2.
__device__ __forceinline__ void st4_stream(float* __restrict__ base, size_t off, const float (&v)[4]) {
  __stcs(reinterpret_cast<float4*>(base + off), make_float4(v[0], v[1], v[2], v[3]));
}
__device__ __forceinline__ void ld4s(const float* s, float (&o)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(s);
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}

// Copy one band row (W + 8 columns, or the wrapped row when W = N) of `field`
// into a ring row: thread g copies its group's four columns, and for W = N
// the first and last threads also copy the wrapped neighbours.
__device__ __forceinline__ void copy_row(float* ring_row, const float* __restrict__ field, int row, int N, int M,
                                         bool wrap, bool active, int tid, int G, int bi, int col, uint64_t pol) {
  const float* src = field + (size_t)(row & M) * N;
  if (active) cp16(ring_row + bi, src + col, pol);
  if (wrap && tid == 0) cp16(ring_row + 4, src + N - 4, pol);
  if (wrap && tid == G - 1) cp16(ring_row + N + 8, src, pol);
}

}  // namespace rows
}  // namespace nsgb
