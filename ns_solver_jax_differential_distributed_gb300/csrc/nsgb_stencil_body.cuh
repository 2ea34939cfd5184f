// The tiled form of the fused Chorin step (one TH x TW tile per CTA of 32 x 8
// threads), shared by k_stencil / k_stencil_batch (nsgb_stencil.cu) and the
// persistent ensemble kernel (nsgb_ens_persistent.cu).
#pragma once

#include "nsgb_internal.h"

namespace nsgb {

// Shared-memory layout of one TW x TH tile (TW a multiple of 4, TH even).
// Tiles are fetched from HBM as aligned float4 groups covering columns
// j0-4 .. j0+TW+3 (a 16-byte-aligned superset of the halos); each field
// component has its own plane, so a warp's accesses along a row are
// consecutive words.
template <int TW, int TH>
struct StencilSmem {
  static constexpr int G = TW / 4 + 2;        // float4 groups per tile row
  static constexpr int W4 = 4 * G;            // = TW + 8 columns, from j0 - 4
  static constexpr int PH = TH + 6, UH = TH + 4, SH = TH + 2, SW = TW + 2;
  static constexpr int P_OFF = 0;                     // PH x W4
  static constexpr int UX_OFF = P_OFF + PH * W4;      // UH x W4
  static constexpr int UY_OFF = UX_OFF + UH * W4;     // UH x W4
  static constexpr int SX_OFF = UY_OFF + UH * W4;     // SH x SW
  static constexpr int SY_OFF = SX_OFF + SH * SW;     // SH x SW
  static constexpr int F_OFF = SY_OFF + SH * SW;      // SH forcing rows
  static constexpr int R_OFF = F_OFF + SH + 2;        // 8 partial sums
  static constexpr int FLOATS = R_OFF + 8;
};

// Tile (bx, by) of a gx x gy tiling (the objective partial's slot); COH:
// L2-only loads of fields other CTAs of the same launch wrote.
template <int SCHEME, int MODE, int TW, int TH, bool COH = false>
__device__ __forceinline__ void stencil_body(const StencilArgs& a, int step_off, int bx, int by, int gx, int gy) {
  using L = StencilSmem<TW, TH>;
  constexpr int G = L::G, W4 = L::W4, PH = L::PH, UH = L::UH, SH = L::SH, SW = L::SW;
  static_assert(TH % 2 == 0, "the u* phase works on pairs of rows");
  extern __shared__ __align__(16) float sm[];
  float* sP = sm + L::P_OFF;
  float* sUx = sm + L::UX_OFF;
  float* sUy = sm + L::UY_OFF;
  float* sSx = sm + L::SX_OFF;
  float* sSy = sm + L::SY_OFF;
  float* sF = sm + L::F_OFF;
  float* sRed = sm + L::R_OFF;
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const int j0 = bx * TW, i0 = by * TH;
  const int tid = threadIdx.y * 32 + threadIdx.x;

  int step = 0;
  float t = a.t_fixed;
  if (MODE == MODE_ROLLOUT) {
    step = (a.step_ctr ? gld(a.step_ctr) : 0) + a.step_fixed + step_off;
    if (a.t_from_step) t = fmul((float)step, c.dt);
  }
  const float nu = (a.theta != nullptr && a.theta_len == 3) ? gldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);

  // Tile loads: aligned float4 groups (a group never straddles the periodic
  // wrap because N and the group start are multiples of 4).
  const bool has_p = a.p != nullptr;
  if (has_p) {
    const float* __restrict__ pp = a.p;
    forflat<PH, G>(tid, [&](int r, int q) {
      const float4 v = gldfield<COH>(reinterpret_cast<const float4*>(pp + (size_t)((i0 - 3 + r) & M) * N +
                                                                     ((j0 - 4 + 4 * q) & M)));
      *reinterpret_cast<float4*>(sP + r * W4 + 4 * q) = v;
    });
  }
  {
    const float* __restrict__ us = a.us;
    forflat<UH, G>(tid, [&](int r, int q) {
      const size_t g = (size_t)((i0 - 2 + r) & M) * N + ((j0 - 4 + 4 * q) & M);
      *reinterpret_cast<float4*>(sUx + r * W4 + 4 * q) = gldfield<COH>(reinterpret_cast<const float4*>(us + g));
      *reinterpret_cast<float4*>(sUy + r * W4 + 4 * q) =
          gldfield<COH>(reinterpret_cast<const float4*>(us + NN + g));
    });
  }
  if (MODE == MODE_ROLLOUT && tid < SH) {
    const ForcingRow fr = forcing_time(gldg(a.theta), gldg(a.theta + 1), t, c);
    sF[tid] = forcing_fx((i0 - 1 + tid) & M, fr, c);
  }
  __syncthreads();

  // 1. pending projection u^n = u* - dt grad p on rows i0-2 .. i0+TH+1 and
  //    columns j0-2 .. j0+TW+1 (plane columns 2 .. TW+5)
  if (has_p) {
    forflat<UH, TW + 4>(tid, [&](int r, int cc) {
      const int col = cc + 2;
      const float* P0 = sP + (r + 1) * W4 + col;  // p at (i0-2+r, j0-2+cc)
      const int o = r * W4 + col;
      sUx[o] = fused_proj(sUx[o], P0[W4], P0[-W4], c.cP);
      sUy[o] = fused_proj(sUy[o], P0[1], P0[-1], c.cP);
    });
    __syncthreads();
  }

  // 2. objective partial on the state before the step; optional state output
  float jacc = 0.0f;
  forflat<TH, TW>(tid, [&](int r, int cc) {
    const int o = (r + 2) * W4 + cc + 4;
    if (MODE == MODE_ROLLOUT) jacc += sUx[o] * sF[r + 1];
    if (a.u_out) {
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      gst(a.u_out + g, sUx[o]);
      gst(a.u_out + NN + g, sUy[o]);
    }
  });

  // 3. u*^{n+1} on rows i0-1 .. i0+TH and columns j0-1 .. j0+TW, two
  //    vertically adjacent cells per thread (rows 2h and 2h+1 of the S tile)
  //    sharing their column loads
  forflat<SH / 2, SW>(tid, [&](int h, int cc) {
    const int r = 2 * h;
    const int o = (r + 1) * W4 + cc + 3;  // U cell of S cell (r, cc)
    float x[4], y[4];                     // U rows r .. r+3 at the cell's column
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      x[k] = sUx[o + (k - 1) * W4];
      y[k] = sUy[o + (k - 1) * W4];
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int ok = o + k * W4;
      const float ox = x[k + 1], oy = y[k + 1];
      const float lx = x[k], rx = x[k + 2], ux_ = sUx[ok + 1], dx_ = sUx[ok - 1];
      const float ly = y[k], ry = y[k + 2], uy_ = sUy[ok + 1], dy_ = sUy[ok - 1];
      float fx, fy;
      if (MODE == MODE_ROLLOUT) {
        fx = sF[r + k];
        fy = 0.0f;
      } else {
        const size_t g = (size_t)((i0 - 1 + r + k) & M) * N + ((j0 - 1 + cc) & M);
        fx = gldg(a.f + g);
        fy = gldg(a.f + NN + g);
      }
      const int so = (r + k) * SW + cc;
      sSx[so] = fused_ustar<SCHEME>(ox, lx, rx, ux_, dx_, ox, oy, cL, fmul(c.dt, fx), c);
      sSy[so] = fused_ustar<SCHEME>(oy, ly, ry, uy_, dy_, ox, oy, cL, fmul(c.dt, fy), c);
    }
  });
  __syncthreads();

  // 4. write u*^{n+1} and div(u*^{n+1}) / dt for the tile
  {
    float* __restrict__ uso = a.us_out;
    float* __restrict__ rhs = a.rhs;
    forflat<TH, TW>(tid, [&](int r, int cc) {
      const int o = (r + 1) * SW + cc + 1;
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      gst(uso + g, sSx[o]);
      gst(uso + NN + g, sSy[o]);
      gst(rhs + g, fused_rhs(sSx[o + SW], sSx[o - SW], sSy[o + 1], sSy[o - 1], c.cD));
    });
  }

  if (MODE == MODE_ROLLOUT) {
    const int tx = threadIdx.x, ty = threadIdx.y;
    jacc = warp_sum(jacc);
    if (tx == 0) sRed[ty] = jacc;
    __syncthreads();
    if (ty == 0) {
      float v = (tx < 8) ? sRed[tx] : 0.0f;
      v = warp_sum(v);
      if (tx == 0 && (unsigned)step < (unsigned)a.jpart_rows) {
        const int nblk = gx * gy;
        gst(a.jpart + (size_t)step * nblk + by * gx + bx, v);
      }
    }
  }
}

}  // namespace nsgb
