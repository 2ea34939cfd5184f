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
__device__ __forceinline__ void cp16(float* dst_smem, const float* src, uint64_t pol, int line = __builtin_LINE()) {
  if (!bounds_ok(src, 16, line)) return;
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

// ---- bulk copies: one thread moves whole row segments with the copy engine
// (cp.async.bulk, completion counted in bytes on an mbarrier); every wait on
// an mbarrier is bounded.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count) : "memory");
}
// make initialised mbarriers visible to the copy engine
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mb, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)), "r"(bytes) : "memory");
}
// `bytes` (a multiple of 16, both addresses 16-byte aligned) from global src
// to this CTA's shared dst; completes `bytes` transactions on mb.
__device__ __forceinline__ void bulk_g2s(float* dst, const float* src, unsigned bytes, uint64_t* mb, uint64_t pol,
                                         int line = __builtin_LINE()) {
  if (!bounds_ok(src, bytes, line)) return;  // the mbarrier's wait then runs out (bounded)
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mb)), "l"(pol)
      : "memory");
}
// Wait for the phase of parity `parity` of mb to complete, polling at most
// `limit` times; false if it did not.
__device__ __forceinline__ bool mbar_wait(uint64_t* mb, unsigned parity, unsigned limit) {
  const uint32_t a = smem_u32(mb);
  for (unsigned i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Segments of one band row as bulk copies: ring offset, source column and
// length in floats; the W + 8 columns from j0 - 4 (W < N), or the row with
// four wrapped columns at each end (W = N), split where the periodic wrap
// falls.  All offsets and lengths are multiples of four floats (16 bytes).
struct RowPieces {
  int n;
  int dst[3], col[3], len[3];
};
__device__ __forceinline__ RowPieces row_pieces(int N, int W, int j0) {
  RowPieces r;
  if (W == N) {
    r.n = 3;
    r.dst[0] = 4, r.col[0] = N - 4, r.len[0] = 4;
    r.dst[1] = 8, r.col[1] = 0, r.len[1] = N;
    r.dst[2] = N + 8, r.col[2] = 0, r.len[2] = 4;
  } else if (j0 == 0) {
    r.n = 2;
    r.dst[0] = 4, r.col[0] = N - 4, r.len[0] = 4;
    r.dst[1] = 8, r.col[1] = 0, r.len[1] = W + 4;
  } else if (j0 + W == N) {
    r.n = 2;
    r.dst[0] = 4, r.col[0] = j0 - 4, r.len[0] = W + 4;
    r.dst[1] = W + 8, r.col[1] = 0, r.len[1] = 4;
  } else {
    r.n = 1;
    r.dst[0] = 4, r.col[0] = j0 - 4, r.len[0] = W + 8;
  }
  return r;
}

__device__ __forceinline__ void st4(float* __restrict__ base, size_t off, const float (&v)[4],
                                    int line = __builtin_LINE()) {
  gst4(base + off, make_float4(v[0], v[1], v[2], v[3]), line);
}
// Evict-first store, for fields read only after the FFT passes (u*next), so
// they do not push the passes' inputs out of L2.
__device__ __forceinline__ void st4_stream(float* __restrict__ base, size_t off, const float (&v)[4],
                                           int line = __builtin_LINE()) {
  gstcs(reinterpret_cast<float4*>(base + off), make_float4(v[0], v[1], v[2], v[3]), line);
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
                                         bool wrap, bool active, int tid, int G, int bi, int col, uint64_t pol,
                                         int line = __builtin_LINE()) {
  const float* src = field + (size_t)(row & M) * N;
  if (active) cp16(ring_row + bi, src + col, pol, line);
  if (wrap && tid == 0) cp16(ring_row + 4, src + N - 4, pol, line);
  if (wrap && tid == G - 1) cp16(ring_row + N + 8, src, pol, line);
}

}  // namespace rows
}  // namespace nsgb
