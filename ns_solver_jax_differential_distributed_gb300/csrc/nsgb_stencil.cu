// Fused stencil kernel of the Chorin step and the single operators of
// PeriodicDifferentialOps / AdvectionScheme.
//
// k_stencil processes one TH x TW tile of the grid per CTA (blockDim 32 x 8).
// It stages the pending pressure p with a 3-cell halo and the pending u* with
// a 2-cell halo in shared memory (periodic wrap by index masking), then
//   1. finishes the previous step's projection  u^n = u* - dt grad p
//      (NS_solver.py:696-697) on the tile + 2-cell halo,
//   2. accumulates the objective partial  sum u^n_x f_x  (NS_solver.py:746),
//   3. forms u*^{n+1} = u^n + dt (nu lap u^n + adv(u^n) + f)  on the tile +
//      1-cell halo (NS_solver.py:685-689, 249-265, 474-477),
//   4. writes u*^{n+1} and rhs = div(u*^{n+1}) / dt for the tile
//      (NS_solver.py:692-693, 206-210).
// The fused step evaluates each cell with the folded-coefficient FMA forms of
// nsgb_common.cuh (fused_proj / fused_ustar / fused_rhs); the single-operator
// kernels at the end of the file keep the reference's operation order with
// explicitly rounded intrinsics, so they round exactly like the reference's
// float32 array expressions.
#include "nsgb_internal.h"
#include "nsgb_rows.cuh"
#include "nsgb_stencil_body.cuh"

namespace nsgb {

template <int SCHEME, int MODE, int TW, int TH>
__global__ void __launch_bounds__(256) k_stencil(const StencilArgs a) {
  stencil_body<SCHEME, MODE, TW, TH>(a, 0, blockIdx.x, blockIdx.y, gridDim.x, gridDim.y);
}

// Ensemble variant: blockIdx.z selects the solve, `variant` its argument set.
template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_stencil_batch(const SolveDev* __restrict__ solves, int variant,
                                                      int step_off) {
  stencil_body<SCHEME, MODE_ROLLOUT, TW, TH>(solves[blockIdx.z].st[variant], step_off, blockIdx.x, blockIdx.y,
                                             gridDim.x, gridDim.y);
}

// ------------------------------------------------------- row streaming --
// k_stencil_rows: the same step as k_stencil (MODE_ROLLOUT), computed by
// threads that march down the grid instead of working on 2-D tiles.
//
// A CTA owns the rows [r0, r0 + RH) of a band of W columns (W = N: whole
// rows, the periodic wrap stays inside the CTA; W < N: one extra group of
// four halo columns on each side, computed but not stored).  Thread g owns the
// four consecutive columns of group g and at iteration t
//   - finishes the projection of row t:  u(t) = u*(t) - dt grad p, from p rows
//     t-1, t, t+1,
//   - forms u*next(t-1) from u(t-2), u(t-1), u(t) (registers) and the edge
//     values of u(t-1) of the neighbouring groups,
//   - writes u*next(t-2) and rhs(t-2) = div(u*next)/dt, and adds the row's
//     objective partial u_x(t-2) f_x.
// The input rows (p and u*) arrive in shared-memory rings kAhead rows ahead,
// so the loads of later rows overlap the arithmetic without holding
// registers; p neighbours come straight from the ring.  The copies are either
// per-thread 16-byte asynchronous copies (each thread its own columns) or,
// with BULK, a few bulk copies of whole row segments issued by one thread
// through the copy engine, counted on an mbarrier per group of rows: thread 0
// waits for the next group before the iteration's barrier, bounded; if a
// wait runs out the CTA stops marching, drains its copies in flight and
// writes a NaN objective partial, so the call's J comes out non-finite.  Computed values that other groups need (the first and last
// column of a group of u and u*next_y) pass through small edge arrays,
// double-buffered by iteration parity; one barrier per iteration orders
// both.  The i-neighbours of computed rows never leave registers.
namespace rows {

constexpr int F_UX = 0, F_UY = 1, F_SY = 2;  // exchanged fields
constexpr int kAhead = 3;                    // rows copied ahead of use
constexpr int kPRing = 8;                    // p rows t-1 .. t+1+kAhead (power of two)
constexpr int kURing = 4;                    // u* rows t .. t+kAhead (power of two)
constexpr int kMbSlots = 4;                  // mbarriers of row groups in flight (power of two)
static_assert(kPRing >= kAhead + 3 && kURing >= kAhead + 1 && kMbSlots >= kAhead + 1, "ring depth");

constexpr unsigned kWaitLimit = 1u << 22;  // mbarrier polls before a CTA gives up
// Row copies by the copy engine (BULK) or per thread.  Measured at N=4096
// (band 2048 x 54, in the pipelined step): 84.3 us per launch with bulk
// copies at prefetch depth 3 or 5, 72.6 us with per-thread copies -- thread
// 0's issuing and polling lies on every iteration's barrier -- so the kernels
// use per-thread copies; both give the same bits.
constexpr bool kBulkRows = false;

// shared memory: rings, edges [2 slots][3 fields][2 sides][G], forcing rows,
// 32 partial sums, then (8-byte aligned) kMbSlots + 1 mbarriers
inline size_t floats_before_mbar(int N, int W, int RH) {
  const size_t f = (size_t)(kPRing + 2 * kURing) * ring_stride(W) + (size_t)12 * groups(N, W) + RH + 2 + 32;
  return (f + 1) & ~(size_t)1;
}
inline size_t smem_bytes(int N, int W, int RH) {
  return sizeof(float) * floats_before_mbar(N, W, RH) + (kMbSlots + 1) * sizeof(uint64_t);
}

}  // namespace rows

template <int SCHEME, bool BULK>
__device__ __forceinline__ void stencil_rows_body(const StencilArgs& a, int step_off) {
  using namespace rows;
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const int W = band_width(N, a.tw);
  const bool wrap = (W == N);
  const int G = groups(N, W);
  const int RH = a.th;
  const int r0 = blockIdx.y * RH;
  const int r1 = min(r0 + RH, N);
  const int j0 = blockIdx.x * W;
  const int tid = threadIdx.x;
  const bool active = tid < G;
  const int g = active ? tid : G - 1;  // idle lanes shadow the last group
  const int col = wrap ? 4 * g : ((j0 - 4 + 4 * g) & M);
  const bool store = active && (wrap || (g >= 1 && g <= G - 2));
  const int gl = g == 0 ? (wrap ? G - 1 : 0) : g - 1;
  const int gr = g == G - 1 ? (wrap ? 0 : G - 1) : g + 1;
  const int RS = ring_stride(W);
  const int bi = 4 + 4 * g + (wrap ? 4 : 0);  // the group's first column in a ring row

  extern __shared__ __align__(16) float sm[];
  float* sP = sm;                              // [kPRing][RS]
  float* sUX = sP + kPRing * RS;               // [kURing][RS]
  float* sUY = sUX + kURing * RS;              // [kURing][RS]
  float* sE = sUY + kURing * RS;               // [slot][field][side][G]
  float* sF = sE + 12 * G;                     // f_x of rows r0-1 .. r1
  float* sRed = sF + RH + 2;                   // per-warp partial sums
  auto edge = [&](int slot, int f, int side) { return sE + ((slot * 3 + f) * 2 + side) * G; };
  // mbarriers (BULK): [0, kMbSlots) the groups of iterations t (p row t+1,
  // u* row t) by (t - r0 + 2) mod kMbSlots, [kMbSlots] the prologue's p rows
  // r0-3, r0-2
  uint64_t* sMb = reinterpret_cast<uint64_t*>(sm + (((kPRing + 2 * kURing) * (size_t)RS + (size_t)12 * G + RH + 2 + 32 + 1) & ~(size_t)1));

  int step = (a.step_ctr ? gld(a.step_ctr) : 0) + a.step_fixed + step_off;
  const float t_now = a.t_from_step ? fmul((float)step, c.dt) : a.t_fixed;
  const float nu = (a.theta != nullptr && a.theta_len == 3) ? gldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);
  {
    const ForcingRow fr = forcing_time(gldg(a.theta), gldg(a.theta + 1), t_now, c);
    for (int k = tid; k < r1 - r0 + 2; k += blockDim.x) sF[k] = forcing_fx((r0 - 1 + k) & M, fr, c);
  }

  const bool has_p = a.p != nullptr;
  const float* __restrict__ pp = a.p;
  const float* __restrict__ usx_g = a.us;
  const float* __restrict__ usy_g = a.us + NN;
  // one copy group: p row `pr` (if do_p) and u* row `ur` (if do_u)
  const uint64_t pol = evict_first_policy();
  const RowPieces pcs = row_pieces(N, W, j0);
  const unsigned row_bytes = 4u * (unsigned)(W + 8);
  auto issue_bulk = [&](int pr, bool do_p, int ur, bool do_u, uint64_t* mb) {  // thread 0
    const bool cp_p = do_p && has_p;
    mbar_expect_tx(mb, row_bytes * ((cp_p ? 1u : 0u) + (do_u ? 2u : 0u)));
    for (int k = 0; k < pcs.n; ++k) {
      const unsigned nb = 4u * (unsigned)pcs.len[k];
      if (cp_p) bulk_g2s(sP + (pr & (kPRing - 1)) * RS + pcs.dst[k], pp + (size_t)(pr & M) * N + pcs.col[k], nb, mb, pol);
      if (do_u) {
        const size_t o = (size_t)(ur & M) * N + pcs.col[k];
        const int d = (ur & (kURing - 1)) * RS + pcs.dst[k];
        bulk_g2s(sUX + d, usx_g + o, nb, mb, pol);
        bulk_g2s(sUY + d, usy_g + o, nb, mb, pol);
      }
    }
  };
  auto issue = [=](int pr, bool do_p, int ur, bool do_u) {
    if (do_p && has_p) {
      float* dst = sP + (pr & (kPRing - 1)) * RS;
      const float* src = pp + (size_t)(pr & M) * N;
      if (active) cp16(dst + bi, src + col, pol);
      if (wrap && tid == 0) cp16(dst + 4, src + N - 4, pol);
      if (wrap && tid == G - 1) cp16(dst + N + 8, src, pol);
    }
    if (do_u && active) {
      const int slot = (ur & (kURing - 1)) * RS + bi;
      const size_t o = (size_t)(ur & M) * N + col;
      cp16(sUX + slot, usx_g + o, pol);
      cp16(sUY + slot, usy_g + o, pol);
    }
    cp_commit();
  };
  // prologue: p rows r0-3, r0-2, then the groups of iterations r0-2-kAhead ..
  // r0-3 (p rows r0-1 .., u* rows r0-2 ..); wait for those of iteration r0-2
  auto mb_of = [&](int t) { return sMb + ((t - r0 + 2) & (kMbSlots - 1)); };  // group of iteration t
  auto par_of = [&](int t) { return (unsigned)(((t - r0 + 2) / kMbSlots) & 1); };
  uint64_t* mb_pro = sMb + kMbSlots;
  int issued = min(r0 - 2 + kAhead - 1, r1 + 1);  // last iteration whose group was issued (BULK)
  int waited = r0 - 2;               // last iteration whose group was waited for (BULK)
  bool late = false;  // thread 0: a wait ran out (BULK)
  if constexpr (BULK) {
    if (tid == 0) {
      for (int k = 0; k <= kMbSlots; ++k) mbar_init(sMb + k, 1);
      mbar_init_fence();
      // the prologue's two p rows share one mbarrier
      mbar_expect_tx(mb_pro, has_p ? 2u * row_bytes : 0u);
      if (has_p)
        for (int r = r0 - 3; r <= r0 - 2; ++r)
          for (int k = 0; k < pcs.n; ++k)
            bulk_g2s(sP + (r & (kPRing - 1)) * RS + pcs.dst[k], pp + (size_t)(r & M) * N + pcs.col[k],
                     4u * (unsigned)pcs.len[k], mb_pro, pol);
      for (int t = r0 - 2; t <= issued; ++t) issue_bulk(t + 1, true, t, true, mb_of(t));
      late = !mbar_wait(mb_pro, 0, kWaitLimit) || !mbar_wait(mb_of(r0 - 2), 0, kWaitLimit);
    }
  } else {
    issue(r0 - 3, true, 0, false);
    issue(r0 - 2, true, 0, false);
#pragma unroll
    for (int k = kAhead; k >= 1; --k) issue(r0 - 1 - k + kAhead, true, r0 - 2 - k + kAhead, true);
    cp_wait<kAhead - 1>();
  }
  // the barrier also tells every thread whether thread 0 gave up waiting
  bool aborted = __syncthreads_or(late) != 0;

  // registers entering iteration t: u rows t-1, t-2; u*next x rows t-3, t-2
  // and y row t-2
  float u1x[4] = {0, 0, 0, 0}, u1y[4] = {0, 0, 0, 0}, u2x[4] = {0, 0, 0, 0}, u2y[4] = {0, 0, 0, 0};
  float sx3[4] = {0, 0, 0, 0}, sx2[4] = {0, 0, 0, 0}, sy2[4] = {0, 0, 0, 0};
  float jacc = 0.0f;
  float* __restrict__ uso_x = a.us_out;
  float* __restrict__ uso_y = a.us_out + NN;
  float* __restrict__ rhs_g = a.rhs;
#pragma unroll 1
  for (int t = r0 - 2; t <= r1 + 1 && !aborted; ++t) {
    const int rs = (t - 1) & 1, ws = t & 1;
    if constexpr (BULK) {
      // rows beyond the band's last iteration are never read: not copied
      if (tid == 0 && t + kAhead <= r1 + 1) {
        issue_bulk(t + 1 + kAhead, true, t + kAhead, true, mb_of(t + kAhead));
        issued = t + kAhead;
      }
    } else {
      issue(t + 1 + kAhead, true, t + kAhead, true);
    }

    // u(t): projection of row t
    float ux[4], uy[4];
    {
      const float* ur = sUX + (t & (kURing - 1)) * RS + bi;
      ld4s(ur, ux);
      ld4s(sUY + (t & (kURing - 1)) * RS + bi, uy);
    }
    if (has_p) {
      float pm[4], pn[4], q[4];
      ld4s(sP + ((t - 1) & (kPRing - 1)) * RS + bi, pm);
      ld4s(sP + ((t + 1) & (kPRing - 1)) * RS + bi, pn);
      const float* pc = sP + (t & (kPRing - 1)) * RS + bi;
      ld4s(pc, q);
      const float P[6] = {pc[-1], q[0], q[1], q[2], q[3], pc[4]};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ux[k] = fused_proj(ux[k], pn[k], pm[k], c.cP);
        uy[k] = fused_proj(uy[k], P[k + 2], P[k], c.cP);
      }
    }

    // u*next(t-1)
    float sx1[4] = {0, 0, 0, 0}, sy1[4] = {0, 0, 0, 0};
    if (t >= r0) {
      const float X[6] = {edge(rs, F_UX, 1)[gl], u1x[0], u1x[1], u1x[2], u1x[3], edge(rs, F_UX, 0)[gr]};
      const float Y[6] = {edge(rs, F_UY, 1)[gl], u1y[0], u1y[1], u1y[2], u1y[3], edge(rs, F_UY, 0)[gr]};
      const float cFx = fmul(c.dt, sF[t - r0]), cFy = fmul(c.dt, 0.0f);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float ox = X[k + 1], oy = Y[k + 1];
        sx1[k] = fused_ustar<SCHEME>(ox, u2x[k], ux[k], X[k + 2], X[k], ox, oy, cL, cFx, c);
        sy1[k] = fused_ustar<SCHEME>(oy, u2y[k], uy[k], Y[k + 2], Y[k], ox, oy, cL, cFy, c);
      }
    }

    // u*next(t-2), rhs(t-2), objective partial and state of row t-2
    if (t >= r0 + 2) {
      const float Y2[6] = {edge(rs, F_SY, 1)[gl], sy2[0], sy2[1], sy2[2], sy2[3], edge(rs, F_SY, 0)[gr]};
      float rh[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) rh[k] = fused_rhs(sx1[k], sx3[k], Y2[k + 2], Y2[k], c.cD);
      if (store) {
        const size_t o = (size_t)((t - 2) & M) * N + col;
        st4_stream(uso_x, o, sx2);
        st4_stream(uso_y, o, sy2);
        st4(rhs_g, o, rh);
        if (a.u_out) {
          st4(a.u_out, o, u2x);
          st4(a.u_out + NN, o, u2y);
        }
        const float fj = sF[t - r0 - 1];
#pragma unroll
        for (int k = 0; k < 4; ++k) jacc += u2x[k] * fj;
      }
    }

    // edge values for the next iteration: u(t), u*next_y(t-1)
    if (active) {
      edge(ws, F_UX, 0)[g] = ux[0];
      edge(ws, F_UX, 1)[g] = ux[3];
      edge(ws, F_UY, 0)[g] = uy[0];
      edge(ws, F_UY, 1)[g] = uy[3];
      edge(ws, F_SY, 0)[g] = sy1[0];
      edge(ws, F_SY, 1)[g] = sy1[3];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      u2x[k] = u1x[k];
      u2y[k] = u1y[k];
      u1x[k] = ux[k];
      u1y[k] = uy[k];
      sx3[k] = sx2[k];
      sx2[k] = sx1[k];
      sy2[k] = sy1[k];
    }
    if constexpr (BULK) {
      if (tid == 0 && t + 1 <= r1 + 1) {  // the rows of iteration t+1 have landed
        late = !mbar_wait(mb_of(t + 1), par_of(t + 1), kWaitLimit);
        waited = t + 1;
      }
      aborted = __syncthreads_or(late) != 0;
    } else {
      cp_wait<kAhead - 1>();  // the rows of iteration t+1 have landed
      __syncthreads();
    }
  }
  if constexpr (BULK) {
    // no copy may still be writing into this CTA's shared memory when it
    // exits: wait (bounded again) for every group not yet seen complete
    if (tid == 0) {
      if (aborted) (void)mbar_wait(mb_pro, 0, kWaitLimit);
      for (int t = aborted ? waited : waited + 1; t <= issued; ++t) (void)mbar_wait(mb_of(t), par_of(t), kWaitLimit);
    }
  } else {
    cp_wait<0>();
  }

  // objective partial of the CTA
  jacc = warp_sum(jacc);
  const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  if (lane == 0) sRed[warp] = jacc;
  __syncthreads();
  if (warp == 0) {
    float v = lane < nwarps ? sRed[lane] : 0.0f;
    v = warp_sum(v);
    if (aborted) v = __int_as_float(0x7fc00000);  // NaN: the step did not complete
    if (lane == 0 && (unsigned)step < (unsigned)a.jpart_rows) {
      const int nblk = gridDim.x * gridDim.y;
      gst(a.jpart + (size_t)step * nblk + blockIdx.y * gridDim.x + blockIdx.x, v);
    }
  }
}

template <int SCHEME>
__global__ void __launch_bounds__(544, 1) k_stencil_rows(const StencilArgs a) {
  stencil_rows_body<SCHEME, rows::kBulkRows>(a, 0);
}

template <int SCHEME>
__global__ void __launch_bounds__(544, 1) k_stencil_rows_batch(const SolveDev* __restrict__ solves, int variant,
                                                              int step_off) {
  stencil_rows_body<SCHEME, rows::kBulkRows>(solves[blockIdx.z].st[variant], step_off);
}

bool stencil_rows_mode(int tw) { return tw >= NSGB_ROWS_MIN_W; }

bool stencil_rows_supported(int N, int tw, int th) {
  if (!stencil_rows_mode(tw) || (tw & (tw - 1)) != 0 || tw > NSGB_ROWS_MAX_W) return false;
  return th >= 1 && th <= N;
}

// Launch shape of a row-streaming kernel: grid (bands of columns, bands of
// rows, count), one thread per column group.
template <class K>
static cudaError_t rows_config(K kernel, int N, int tw, int th, unsigned count, dim3& grid, dim3& block,
                               size_t& smem) {
  const int W = rows::band_width(N, tw);
  smem = rows::smem_bytes(N, W, th);
  if (smem > 48 * 1024) {
    const cudaError_t e = raise_smem_limit(kernel);
    if (e != cudaSuccess) return e;
  }
  grid = dim3(N / W, (N + th - 1) / th, count);
  block = dim3(rows::threads(N, W));
  return cudaSuccess;
}

template <int SCHEME>
static cudaError_t launch_stencil_rows(const StencilArgs& a, cudaStream_t st) {
  dim3 grid, block;
  size_t smem;
  cudaError_t e = rows_config(k_stencil_rows<SCHEME>, a.c.N, a.tw, a.th, 1, grid, block, smem);
  if (e != cudaSuccess) return e;
  k_stencil_rows<SCHEME><<<grid, block, smem, st>>>(a);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_stencil_rows_batch(const SolveDev* solves, int count, int variant, int step_off, int N,
                                             int tw, int th, cudaStream_t st) {
  dim3 grid, block;
  size_t smem;
  cudaError_t e = rows_config(k_stencil_rows_batch<SCHEME>, N, tw, th, (unsigned)count, grid, block, smem);
  if (e != cudaSuccess) return e;
  k_stencil_rows_batch<SCHEME><<<grid, block, smem, st>>>(solves, variant, step_off);
  return cudaGetLastError();
}

int stencil_nblocks(int N, int tw, int th) {
  if (stencil_rows_mode(tw)) return (N / rows::band_width(N, tw)) * ((N + th - 1) / th);
  return (N / tw) * (N / th);
}

bool stencil_tile_supported(int tw, int th) {
#define NSGB_TILE_OK(W, H) if (tw == W && th == H) return true;
  NSGB_STENCIL_TILES(NSGB_TILE_OK)
#undef NSGB_TILE_OK
  return false;
}

template <int TW, int TH>
static constexpr size_t stencil_smem() {
  return StencilSmem<TW, TH>::FLOATS * sizeof(float);
}

template <int SCHEME, int MODE, int TW, int TH>
static cudaError_t launch_stencil_t(const StencilArgs& a, cudaStream_t st) {
  const cudaError_t e = raise_smem_limit(k_stencil<SCHEME, MODE, TW, TH>);
  if (e != cudaSuccess) return e;
  const dim3 grid(a.c.N / TW, a.c.N / TH);
  k_stencil<SCHEME, MODE, TW, TH><<<grid, dim3(32, 8), stencil_smem<TW, TH>(), st>>>(a);
  return cudaGetLastError();
}

template <int SCHEME, int TW, int TH>
static cudaError_t launch_stencil_batch_t(const SolveDev* solves, int count, int variant, int step_off, int N,
                                          cudaStream_t st) {
  const cudaError_t e = raise_smem_limit(k_stencil_batch<SCHEME, TW, TH>);
  if (e != cudaSuccess) return e;
  const dim3 grid(N / TW, N / TH, count);
  k_stencil_batch<SCHEME, TW, TH><<<grid, dim3(32, 8), stencil_smem<TW, TH>(), st>>>(solves, variant,
                                                                                   step_off);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_stencil_batch_s(const SolveDev* solves, int count, int variant, int step_off, int N,
                                          int tw, int th, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (tw == W && th == H) return launch_stencil_batch_t<SCHEME, W, H>(solves, count, variant, step_off, N, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_stencil_batch(const SolveDev* solves, int count, int variant, int step_off, int scheme, int N,
                                 int tw, int th, cudaStream_t st) {
  if (stencil_rows_mode(tw))
    return scheme == NSGB_SCHEME_CENTRAL
               ? launch_stencil_rows_batch<NSGB_SCHEME_CENTRAL>(solves, count, variant, step_off, N, tw, th, st)
               : launch_stencil_rows_batch<NSGB_SCHEME_UPWIND>(solves, count, variant, step_off, N, tw, th, st);
  return scheme == NSGB_SCHEME_CENTRAL
             ? launch_stencil_batch_s<NSGB_SCHEME_CENTRAL>(solves, count, variant, step_off, N, tw, th, st)
             : launch_stencil_batch_s<NSGB_SCHEME_UPWIND>(solves, count, variant, step_off, N, tw, th, st);
}

template <int SCHEME, int MODE>
static cudaError_t launch_stencil_s(const StencilArgs& a, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (a.tw == W && a.th == H) return launch_stencil_t<SCHEME, MODE, W, H>(a, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

void tile_kernel_default(int N, int& tw, int& th) {
  tw = N < 64 ? N : (N <= 512 ? 32 : 64);
  th = N < 16 ? N : (N >= 1024 ? 16 : 8);
}

cudaError_t launch_stencil(const StencilArgs& a, int mode, cudaStream_t st) {
  if (stencil_rows_mode(a.tw)) {
    if (mode == MODE_ROLLOUT)
      return a.scheme == NSGB_SCHEME_CENTRAL ? launch_stencil_rows<NSGB_SCHEME_CENTRAL>(a, st)
                                             : launch_stencil_rows<NSGB_SCHEME_UPWIND>(a, st);
    // explicit force fields: the tiled kernel
    StencilArgs b = a;
    tile_kernel_default(a.c.N, b.tw, b.th);
    return launch_stencil(b, mode, st);
  }
  if (a.scheme == NSGB_SCHEME_CENTRAL) {
    return mode == MODE_ROLLOUT ? launch_stencil_s<NSGB_SCHEME_CENTRAL, MODE_ROLLOUT>(a, st)
                                : launch_stencil_s<NSGB_SCHEME_CENTRAL, MODE_FIELD>(a, st);
  }
  return mode == MODE_ROLLOUT ? launch_stencil_s<NSGB_SCHEME_UPWIND, MODE_ROLLOUT>(a, st)
                              : launch_stencil_s<NSGB_SCHEME_UPWIND, MODE_FIELD>(a, st);
}

// ------------------------------------------------------------ projection --
__global__ void k_project(const float* __restrict__ us, const float* __restrict__ p,
                          float* __restrict__ u, const StepConsts c) {
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  const int i = (int)(g >> c.logN), j = (int)(g & M);
  gst(u + g, fused_proj(gldg(us + g), gldg(p + (size_t)((i + 1) & M) * N + j),
                        gldg(p + (size_t)((i - 1) & M) * N + j), c.cP));
  gst(u + NN + g, fused_proj(gldg(us + NN + g), gldg(p + (size_t)i * N + ((j + 1) & M)),
                             gldg(p + (size_t)i * N + ((j - 1) & M)), c.cP));
}

cudaError_t launch_project(const float* us, const float* p, float* u_out, const StepConsts& c,
                           cudaStream_t st) {
  const size_t NN = (size_t)c.N * c.N;
  k_project<<<(unsigned)((NN + 255) / 256), 256, 0, st>>>(us, p, u_out, c);
  return cudaGetLastError();
}

__global__ void k_project_batch(const SolveDev* __restrict__ solves, int variant) {
  const SolveDev& d = solves[blockIdx.y];
  const StencilArgs& a = d.st[variant];
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  const int i = (int)(g >> c.logN), j = (int)(g & M);
  const float* p = a.p;
  gst(d.u_final + g, fused_proj(gldg(a.us + g), gldg(p + (size_t)((i + 1) & M) * N + j),
                                gldg(p + (size_t)((i - 1) & M) * N + j), c.cP));
  gst(d.u_final + NN + g, fused_proj(gldg(a.us + NN + g), gldg(p + (size_t)i * N + ((j + 1) & M)),
                                     gldg(p + (size_t)i * N + ((j - 1) & M)), c.cP));
}

// Projection of the final state of every solve: `variant` names the argument
// set whose (us, p) hold the pending u* and pressure.
cudaError_t launch_project_batch(const SolveDev* solves, int count, int variant, int N, cudaStream_t st) {
  const size_t NN = (size_t)N * N;
  k_project_batch<<<dim3((unsigned)((NN + 255) / 256), count), 256, 0, st>>>(solves, variant);
  return cudaGetLastError();
}

// ----------------------------------------------------------- J reduction --
// One CTA per step: fixed-order sum of that step's block partials.
__global__ void k_jreduce(const float* __restrict__ jpart, int nblk, double* __restrict__ jsteps) {
  __shared__ double red[256];
  const float* row = jpart + (size_t)blockIdx.x * nblk;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += (double)gld(row + b);
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) gst(jsteps + blockIdx.x, red[0]);
}

__global__ void k_jfinal(const double* __restrict__ jsteps, int steps, double jscale,
                         float* __restrict__ J) {
  double acc = 0.0;
  for (int s = 0; s < steps; ++s) acc += gld(jsteps + s) * jscale;
  gst(J, (float)acc);
}

cudaError_t launch_jreduce(const float* jpart, int nblk, int steps, double* jsteps, float* J,
                           double jscale, cudaStream_t st) {
  if (steps > 0) k_jreduce<<<steps, 256, 0, st>>>(jpart, nblk, jsteps);
  k_jfinal<<<1, 1, 0, st>>>(jsteps, steps, jscale, J);
  return cudaGetLastError();
}

__global__ void k_jreduce_batch(const SolveDev* __restrict__ solves, int nblk) {
  __shared__ double red[256];
  const SolveDev& d = solves[blockIdx.y];
  const float* row = d.st[1].jpart + (size_t)blockIdx.x * nblk;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += (double)gld(row + b);
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) gst(d.jsteps + blockIdx.x, red[0]);
}

__global__ void k_jfinal_batch(const SolveDev* __restrict__ solves, int count, int steps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const SolveDev& d = solves[k];
  double acc = 0.0;
  for (int s = 0; s < steps; ++s) acc += gld(d.jsteps + s) * d.jscale;
  gst(d.J, (float)acc);
}

cudaError_t launch_jreduce_batch(const SolveDev* solves, int count, int nblk, int steps, cudaStream_t st) {
  if (steps > 0) k_jreduce_batch<<<dim3(steps, count), 256, 0, st>>>(solves, nblk);
  k_jfinal_batch<<<(count + 127) / 128, 128, 0, st>>>(solves, count, steps);
  return cudaGetLastError();
}

__global__ void k_counter_batch(const SolveDev* __restrict__ solves, int count, int value, int add) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  int* ctr = solves[k].ctr;
  gst(ctr, add ? gld(ctr) + value : solves[k].ctr_init + value);
}

cudaError_t launch_counter_batch(const SolveDev* solves, int count, int value, bool add, cudaStream_t st) {
  k_counter_batch<<<(count + 127) / 128, 128, 0, st>>>(solves, count, value, add ? 1 : 0);
  return cudaGetLastError();
}

__global__ void k_step_counter(int* ctr, int value, int add) { gst(ctr, add ? gld(ctr) + value : value); }
cudaError_t launch_step_counter(int* step_ctr, int value, bool add, cudaStream_t st) {
  k_step_counter<<<1, 1, 0, st>>>(step_ctr, value, add ? 1 : 0);
  return cudaGetLastError();
}

// ------------------------------------------------------- single operators --
__device__ __forceinline__ void ij_of(size_t g, const StepConsts& c, int& i, int& j) {
  i = (int)(g >> c.logN);
  j = (int)(g & (c.N - 1));
}

__global__ void k_grad(const float* __restrict__ f, float* __restrict__ gx, float* __restrict__ gy,
                       const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  gst(gx + g, divc(fsub(gld(f + (size_t)((i + 1) & M) * N + j), gld(f + (size_t)((i - 1) & M) * N + j)), c.h2, c.rh2));
  gst(gy + g, divc(fsub(gld(f + (size_t)i * N + ((j + 1) & M)), gld(f + (size_t)i * N + ((j - 1) & M))), c.h2, c.rh2));
}

__global__ void k_laplacian(const float* __restrict__ f, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float left = gld(f + (size_t)((i - 1) & M) * N + j), right = gld(f + (size_t)((i + 1) & M) * N + j);
  const float up = gld(f + (size_t)i * N + ((j + 1) & M)), down = gld(f + (size_t)i * N + ((j - 1) & M));
  gst(out + g, divc(fsub(fadd(fadd(fadd(left, right), up), down), fmul(4.0f, gld(f + g))), c.dx2, c.rdx2));
}

__global__ void k_divergence(const float* __restrict__ u, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float* uy = u + NN;
  const float gx = divc(fsub(gld(u + (size_t)((i + 1) & M) * N + j), gld(u + (size_t)((i - 1) & M) * N + j)), c.h2, c.rh2);
  const float gy = divc(fsub(gld(uy + (size_t)i * N + ((j + 1) & M)), gld(uy + (size_t)i * N + ((j - 1) & M))), c.h2, c.rh2);
  gst(out + g, fadd(gx, gy));
}

template <int SCHEME>
__global__ void k_advect(const float* __restrict__ fld, const float* __restrict__ ux,
                         const float* __restrict__ uy, float* __restrict__ out, const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const int N = c.N, M = N - 1;
  const float f = gld(fld + g);
  const float left = gld(fld + (size_t)((i - 1) & M) * N + j), right = gld(fld + (size_t)((i + 1) & M) * N + j);
  const float up = gld(fld + (size_t)i * N + ((j + 1) & M)), down = gld(fld + (size_t)i * N + ((j - 1) & M));
  const float vx = gld(ux + g), vy = gld(uy + g);
  if (SCHEME == NSGB_SCHEME_CENTRAL) {
    const float gx = divc(fsub(right, left), c.h2, c.rh2);
    const float gy = divc(fsub(up, down), c.h2, c.rh2);
    gst(out + g, -fadd(fmul(vx, gx), fmul(vy, gy)));
  } else {
    const float dfx = divc(vx >= 0.0f ? fsub(f, left) : fsub(right, f), c.h1, c.rh1);
    const float dfy = divc(vy >= 0.0f ? fsub(f, down) : fsub(up, f), c.h1, c.rh1);
    gst(out + g, -fadd(fmul(vx, dfx), fmul(vy, dfy)));
  }
}

__global__ void k_forcing_field(const float* __restrict__ theta, float t, float* __restrict__ f,
                                const StepConsts c) {
  const size_t NN = (size_t)c.N * c.N;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= NN) return;
  int i, j;
  ij_of(g, c, i, j);
  const ForcingRow fr = forcing_time(gldg(theta), gldg(theta + 1), t, c);
  gst(f + g, forcing_fx(i, fr, c));
  gst(f + NN + g, 0.0f);
}

static unsigned nb(const StepConsts& c) { return (unsigned)(((size_t)c.N * c.N + 255) / 256); }

cudaError_t launch_grad(const float* f, float* gx, float* gy, const StepConsts& c, cudaStream_t st) {
  k_grad<<<nb(c), 256, 0, st>>>(f, gx, gy, c);
  return cudaGetLastError();
}
cudaError_t launch_laplacian(const float* f, float* out, const StepConsts& c, cudaStream_t st) {
  k_laplacian<<<nb(c), 256, 0, st>>>(f, out, c);
  return cudaGetLastError();
}
cudaError_t launch_divergence(const float* u, float* out, const StepConsts& c, cudaStream_t st) {
  k_divergence<<<nb(c), 256, 0, st>>>(u, out, c);
  return cudaGetLastError();
}
cudaError_t launch_advect(int scheme, const float* fld, const float* ux, const float* uy, float* out,
                          const StepConsts& c, cudaStream_t st) {
  if (scheme == NSGB_SCHEME_CENTRAL)
    k_advect<NSGB_SCHEME_CENTRAL><<<nb(c), 256, 0, st>>>(fld, ux, uy, out, c);
  else
    k_advect<NSGB_SCHEME_UPWIND><<<nb(c), 256, 0, st>>>(fld, ux, uy, out, c);
  return cudaGetLastError();
}
cudaError_t launch_forcing_field(const float* theta, int theta_len, float t, float* f,
                                 const StepConsts& c, cudaStream_t st) {
  (void)theta_len;
  k_forcing_field<<<nb(c), 256, 0, st>>>(theta, t, f, c);
  return cudaGetLastError();
}

NSGB_BOUNDS_UNIT(stencil, 1)

}  // namespace nsgb
