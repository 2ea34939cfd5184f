// k_fused_rows: one rollout step's row work in a single kernel -- the inverse
// row FFT that turns the Poisson-solved half spectrum into p, the fused Chorin
// stencil (projection of the previous step, objective partial, u*next and
// div(u*next)/dt), and the forward row FFT of that right-hand side -- so that
// neither p nor rhs is ever written to HBM.  The column FFT (k_cols, with the
// -1/|k|^2 multiplier) runs between two launches of this kernel.  Together
// they replace SpectralPoissonSolver.__call__ (NS_solver.py:523-527), the
// projection grad(p) (NS_solver.py:692-697) and the stencil work of
// ChorinProjector.step (NS_solver.py:671-689).
//
// Layout.  A cluster of C = N / W CTAs (W = min(N, 2048) columns each) owns a
// band of rows [r0, r1); CTA c owns columns [c W, (c+1) W).  Each CTA runs two
// roles in separate warps:
//   * stencil warps (one thread per group of four columns, plus one halo group
//     on each side when W < N): the row-streaming step of k_stencil_rows, with
//     p read from a shared-memory ring that the FFT warps fill and rhs written
//     into the forward-FFT staging buffer of the CTA that transforms its row
//     pair; the neighbouring groups' edge values travel by warp shuffles (and
//     through shared memory across warps);
//   * FFT warps (N/16 threads per transform, radix-16 Stockham): the inverse
//     two-for-one C2R transform of p row pairs and the forward two-for-one R2C
//     transform of rhs row pairs.  Row pairs are dealt round-robin to the CTAs
//     of the cluster; a transform's output columns go straight into the p
//     rings of the CTAs that own them (distributed shared memory) and its
//     input rhs rows arrive from all CTAs the same way.  When C = 1 two FFT
//     groups run the inverse and forward transforms side by side.
// The stencil marches two rows per period; one cluster-wide barrier per
// period publishes that period's p pair and rhs rows.  p rows r0-4 .. r1+3 are
// produced (the stencil needs three rows of halo; pairs start on even rows so
// a pair's spectrum entries share 32-byte sectors), and every row pair is
// transformed by exactly the arithmetic of k_rows_inv / k_rows_fwd, so the
// step gives the same bits as the four-kernel step.
//
// Barriers: CTA barrier 0 and the cluster barrier are executed by every
// thread the same number of times (one after the prologue, one per period);
// barrier 1 synchronises the stencil warps between the two rows of a period,
// barriers 2 and 3 the FFT groups between their passes.  There are no spin
// waits.
#include "nsgb_fft.cuh"
#include "nsgb_internal.h"
#include "nsgb_rows.cuh"

namespace nsgb {
namespace fused {

constexpr int kMaxW = 2048;  // columns per CTA
constexpr int kAhead = 3;    // u* rows copied ahead of use
constexpr int kPRing = 8;    // p rows: pairs k .. k+2 in use, pair k+3 being written
constexpr int kURing = 4;    // u* rows t .. t+kAhead
constexpr int kE = 16;       // radix of the row transforms

template <int N>
struct Shape {
  static constexpr int W = N < kMaxW ? N : kMaxW;
  static constexpr int C = N / W;                       // CTAs per cluster
  static constexpr bool WRAP = (C == 1);                // whole rows: periodic wrap inside the CTA
  static constexpr int G = WRAP ? W / 4 : W / 4 + 2;    // column groups of the stencil
  static constexpr int ST = (G + 31) / 32 * 32;         // stencil threads
  static constexpr int NWS = ST / 32;
  static constexpr int FT = N / kE;                     // threads of one transform
  static constexpr int NG = WRAP ? 2 : 1;               // FFT groups
  static constexpr int THREADS = ST + NG * FT;
  static constexpr int RS = W + 16;                     // ring row: 4 pad, W + 8 columns, 4 pad
  static constexpr int NSLOT = WRAP ? 2 : 1;            // rhs staging buffers
  static constexpr int XB = 2 * (fft::padlen(N) + 2);   // floats of one transform buffer
  static constexpr int P_OFF = 0;
  static constexpr int UX_OFF = P_OFF + kPRing * RS;
  static constexpr int UY_OFF = UX_OFF + kURing * RS;
  static constexpr int STG_OFF = UY_OFF + kURing * RS;
  static constexpr int INV_OFF = STG_OFF + NSLOT * XB;
  static constexpr int EDGE_OFF = INV_OFF + XB;          // [2 slots][3 fields][2 sides][NWS]
  static constexpr int RED_OFF = EDGE_OFF + 12 * NWS;    // 32 partial sums
  static constexpr int F_OFF = RED_OFF + 32;             // f_x of rows r0-1 .. r1
  static_assert(C <= 2, "clusters of one or two CTAs");
  static_assert(THREADS <= 1024, "block size");
  static_assert(XB % 4 == 0 && RS % 4 == 0 && (12 * NWS) % 4 == 0, "16-byte aligned sections");
  static_assert(W % FT == 0, "an FFT thread's output columns s*FT + j belong to CTA s*FT/W");
};

template <int N>
__host__ __device__ constexpr size_t smem_bytes(int rows) {
  return sizeof(float) * ((size_t)Shape<N>::F_OFF + rows + 2);
}

__device__ __forceinline__ unsigned cta_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

template <int C>
__device__ __forceinline__ void cluster_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
}

// Stores into the dynamic shared memory of any CTA of the cluster (offsets in
// floats from its start; every CTA has the same layout).
template <int C>
struct ClusterSmem {
  float* local;
  uint32_t base0, base1;
  __device__ __forceinline__ void init(float* sm) {
    local = sm;
    if constexpr (C > 1) {
      const uint32_t a = (uint32_t)__cvta_generic_to_shared(sm);
      asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(base0) : "r"(a));
      asm volatile("mapa.shared::cluster.u32 %0, %1, 1;" : "=r"(base1) : "r"(a));
    }
  }
  __device__ __forceinline__ void st(unsigned rank, int off, float v) const {
    if constexpr (C == 1) {
      local[off] = v;
    } else {
      const uint32_t a = (rank ? base1 : base0) + 4u * (uint32_t)off;
      asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
    }
  }
  __device__ __forceinline__ void st4(unsigned rank, int off, float x, float y, float z, float w) const {
    if constexpr (C == 1) {
      *reinterpret_cast<float4*>(local + off) = make_float4(x, y, z, w);
    } else {
      const uint32_t a = (rank ? base1 : base0) + 4u * (uint32_t)off;
      asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(x), "f"(y), "f"(z), "f"(w)
                   : "memory");
    }
  }
};

// Inverse two-for-one transform of p rows i, i+1 (i even, possibly negative:
// taken mod N) from the Poisson-solved half spectrum, its columns written into
// the p rings of the cluster (and the halo columns of the neighbouring CTAs).
// The spectrum entries are combined exactly as k_rows_inv combines them.
template <int N, int C>
__device__ __forceinline__ void inverse_pair(const float2* __restrict__ spec, int i, float2* xb,
                                             const float2* __restrict__ tw, int j, const ClusterSmem<C>& cs) {
  using S = Shape<N>;
  constexpr int T = S::FT, H = N / 2, W = S::W, RS = S::RS, U = H / T;
  using fft::pad;
  const int ir = i & (N - 1);
  float4 v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) v[u] = gldg(reinterpret_cast<const float4*>(spec + (size_t)(j + u * T) * N + ir));
  float4 vh = make_float4(0.f, 0.f, 0.f, 0.f);
  if (j == 0) vh = gldg(reinterpret_cast<const float4*>(spec + (size_t)H * N + ir));
  // X_a[k] = (x, y), X_b[k] = (z, w):  Z[k] = X_a + i X_b,  Z[N-k] = conj(X_a) + i conj(X_b);
  // DC and Nyquist keep only the real parts (as Re(ifft2) drops the rest)
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k = j + u * T;
    const float4 x = v[u];
    if (k == 0) {
      xb[pad(0)] = make_float2(x.x, x.z);
    } else {
      xb[pad(k)] = make_float2(x.x - x.w, x.y + x.z);
      xb[pad(N - k)] = make_float2(x.x + x.w, x.z - x.y);
    }
  }
  if (j == 0) xb[pad(H)] = make_float2(vh.x, vh.z);
  fft::group_sync<2, T>();
  float2 a[kE];
  fft::load_strided<T, kE>(a, xb, j);
  fft::group_sync<2, T>();
  fft::block_fft<N, true, kE, 2>(a, xb, j, tw);
  // thread j holds columns j + s T: real parts are row i, imaginary parts row i + 1
  const int ra = S::P_OFF + (i & (kPRing - 1)) * RS, rb = S::P_OFF + ((i + 1) & (kPRing - 1)) * RS;
#pragma unroll
  for (int s = 0; s < kE; ++s) {
    const int blk = (s * T) & (W - 1);
    const unsigned tgt = (unsigned)((s * T) / W);
    const int m = blk + j;  // column within CTA tgt
    cs.st(tgt, ra + 8 + m, a[s].x);
    cs.st(tgt, rb + 8 + m, a[s].y);
    if (blk == 0 && j < 4) {  // right halo of the CTA on the left (periodic)
      const unsigned nb = (tgt + C - 1) % C;
      cs.st(nb, ra + W + 8 + m, a[s].x);
      cs.st(nb, rb + W + 8 + m, a[s].y);
    }
    if (blk == W - T && j >= T - 4) {  // left halo of the CTA on the right (periodic)
      const unsigned nb = (tgt + 1) % C;
      cs.st(nb, ra + m - (W - 8), a[s].x);
      cs.st(nb, rb + m - (W - 8), a[s].y);
    }
  }
}

// Forward two-for-one transform of the rhs rows i, i+1 staged (unpadded,
// z[n] = rhs_i[n] + i rhs_{i+1}[n]) in `stg`, which then serves as the
// exchange buffer; the half spectra are split and stored transposed exactly
// as k_rows_fwd stores them.
template <int N, int BAR>
__device__ __forceinline__ void forward_pair(float2* stg, float2* __restrict__ spec, int i,
                                             const float2* __restrict__ tw, int j) {
  constexpr int T = N / kE, H = N / 2;
  using fft::pad;
  float2 a[kE];
#pragma unroll
  for (int s = 0; s < kE; ++s) a[s] = stg[j + s * T];
  fft::group_sync<BAR, T>();
  fft::block_fft<N, false, kE, BAR>(a, stg, j, tw);
  fft::group_sync<BAR, T>();
  fft::store_strided<T, kE>(a, stg, j);
  fft::group_sync<BAR, T>();
  // 2 X_i[k] = Z[k] + conj(Z[N-k]);  2 X_{i+1}[k] = -i (Z[k] - conj(Z[N-k]))
  for (int k = j; k <= H; k += T) {
    const float2 zk = stg[pad(k)], wk = stg[pad((N - k) & (N - 1))];
    gst(reinterpret_cast<float4*>(spec + (size_t)k * N + i),
        make_float4(zk.x + wk.x, zk.y - wk.y, zk.y + wk.y, wk.x - zk.x));
  }
}

}  // namespace fused

template <int SCHEME, int N>
__device__ __forceinline__ void fused_rows_body(const FusedArgs& fa) {
  using namespace fused;
  using namespace rows;
  using S = Shape<N>;
  constexpr int W = S::W, C = S::C, G = S::G, ST = S::ST, NWS = S::NWS, FT = S::FT, RS = S::RS, XB = S::XB;
  constexpr bool WRAP = S::WRAP;
  constexpr int M = N - 1;
  constexpr size_t NN = (size_t)N * N;
  const StencilArgs& a = fa.a;
  const StepConsts& c = a.c;
  const int RH = a.th;
  const int r0 = blockIdx.y * RH;
  const int r1 = min(r0 + RH, N);
  const int NK = (r1 - r0 + 4) / 2;  // periods (two stencil rows each)
  const int NQ = NK + 2;             // inverse pairs: p rows r0-4 .. r1+3
  const int NF = (r1 - r0) / 2;      // forward pairs: rhs rows r0 .. r1-1
  const unsigned rank = (C > 1) ? cta_rank() : 0u;
  const int tid = threadIdx.x;
  const bool is_st = tid < ST;  // warps 0 .. ST/32-1: stencil; the rest: FFT groups

  extern __shared__ __align__(16) float sm[];
  ClusterSmem<C> cs;
  cs.init(sm);
  // every CTA of the cluster is running before any of them writes into
  // another's shared memory
  if constexpr (C > 1) cluster_barrier<C>();
  float* sP = sm + S::P_OFF;
  float* sUX = sm + S::UX_OFF;
  float* sUY = sm + S::UY_OFF;
  float* sE = sm + S::EDGE_OFF;
  float* sRed = sm + S::RED_OFF;
  float* sF = sm + S::F_OFF;

  const int step = (a.step_ctr ? gld(a.step_ctr) : 0) + a.step_fixed;
  const float t_now = a.t_from_step ? fmul((float)step, c.dt) : a.t_fixed;
  const float nu = (a.theta != nullptr && a.theta_len == 3) ? gldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);

  // ---- stencil role state
  const int lane = tid & 31, warp = tid >> 5;
  const bool active = tid < G;
  const int g = active ? tid : G - 1;  // idle lanes shadow the last group
  const int j0 = (int)rank * W;
  const int col = WRAP ? 4 * g : ((j0 - 4 + 4 * g) & M);
  const bool store = active && (WRAP || (g >= 1 && g <= G - 2));
  const int bi = WRAP ? 8 + 4 * g : 4 + 4 * g;  // the group's first column in a ring row
  const int wl = warp > 0 ? warp - 1 : (WRAP ? NWS - 1 : 0);
  const int wr = warp < NWS - 1 ? warp + 1 : (WRAP ? 0 : NWS - 1);
  auto eb = [&](int slot, int f, int side, int w) -> float& { return sE[((slot * 3 + f) * 2 + side) * NWS + w]; };
  const float* __restrict__ usx_g = a.us;
  const float* __restrict__ usy_g = a.us + NN;
  float* __restrict__ uso_x = a.us_out;
  float* __restrict__ uso_y = a.us_out + NN;
  const uint64_t pol = evict_first_policy();
  auto issue_u = [&](int ur) {
    if (active) {
      const int slot = (ur & (kURing - 1)) * RS + bi;
      const size_t o = (size_t)(ur & M) * N + col;
      cp16(sUX + slot, usx_g + o, pol);
      cp16(sUY + slot, usy_g + o, pol);
    }
    cp_commit();
  };
  // registers entering iteration t: u rows t-1, t-2; u*next x rows t-3, t-2
  // and y row t-2; rhs of the even row of the pending pair
  float u1x[4] = {0, 0, 0, 0}, u1y[4] = {0, 0, 0, 0}, u2x[4] = {0, 0, 0, 0}, u2y[4] = {0, 0, 0, 0};
  float sx3[4] = {0, 0, 0, 0}, sx2[4] = {0, 0, 0, 0}, sy2[4] = {0, 0, 0, 0}, rhe[4] = {0, 0, 0, 0};
  float jacc = 0.0f;

  auto iterate = [&](int t, int h, int k) {
    const int rs = (t - 1) & 1, ws = t & 1;
    issue_u(t + kAhead);
    // u(t): projection of row t
    float ux[4], uy[4];
    ld4s(sUX + (t & (kURing - 1)) * RS + bi, ux);
    ld4s(sUY + (t & (kURing - 1)) * RS + bi, uy);
    {
      float pm[4], pn[4], q[4];
      ld4s(sP + ((t - 1) & (kPRing - 1)) * RS + bi, pm);
      ld4s(sP + ((t + 1) & (kPRing - 1)) * RS + bi, pn);
      const float* pc = sP + (t & (kPRing - 1)) * RS + bi;
      ld4s(pc, q);
      const float P[6] = {pc[-1], q[0], q[1], q[2], q[3], pc[4]};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        ux[kk] = fused_proj(ux[kk], pn[kk], pm[kk], c.cP);
        uy[kk] = fused_proj(uy[kk], P[kk + 2], P[kk], c.cP);
      }
    }
    // edge values of the neighbouring groups: u(t-1) and u*next_y(t-2)
    constexpr unsigned FULL = 0xffffffffu;
    float lx = __shfl_up_sync(FULL, u1x[3], 1), rx = __shfl_down_sync(FULL, u1x[0], 1);
    float ly = __shfl_up_sync(FULL, u1y[3], 1), ry = __shfl_down_sync(FULL, u1y[0], 1);
    float l2 = __shfl_up_sync(FULL, sy2[3], 1), r2 = __shfl_down_sync(FULL, sy2[0], 1);
    if (lane == 0) {
      lx = eb(rs, 0, 1, wl);
      ly = eb(rs, 1, 1, wl);
      l2 = eb(rs, 2, 1, wl);
    }
    if (lane == 31) {
      rx = eb(rs, 0, 0, wr);
      ry = eb(rs, 1, 0, wr);
      r2 = eb(rs, 2, 0, wr);
    }
    // u*next(t-1)
    float sx1[4] = {0, 0, 0, 0}, sy1[4] = {0, 0, 0, 0};
    if (t >= r0) {
      const float X[6] = {lx, u1x[0], u1x[1], u1x[2], u1x[3], rx};
      const float Y[6] = {ly, u1y[0], u1y[1], u1y[2], u1y[3], ry};
      const float cFx = fmul(c.dt, sF[t - r0]), cFy = fmul(c.dt, 0.0f);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float ox = X[kk + 1], oy = Y[kk + 1];
        sx1[kk] = fused_ustar<SCHEME>(ox, u2x[kk], ux[kk], X[kk + 2], X[kk], ox, oy, cL, cFx, c);
        sy1[kk] = fused_ustar<SCHEME>(oy, u2y[kk], uy[kk], Y[kk + 2], Y[kk], ox, oy, cL, cFy, c);
      }
    }
    // u*next(t-2), rhs(t-2) into the staging of its pair, objective partial
    if (t >= r0 + 2) {
      const float Y2[6] = {l2, sy2[0], sy2[1], sy2[2], sy2[3], r2};
      float rh[4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) rh[kk] = fused_rhs(sx1[kk], sx3[kk], Y2[kk + 2], Y2[kk], c.cD);
      if (store) {
        const size_t o = (size_t)((t - 2) & M) * N + col;
        st4_stream(uso_x, o, sx2);
        st4_stream(uso_y, o, sy2);
        const float fj = sF[t - r0 - 1];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) jacc += u2x[kk] * fj;
        if (h == 0) {
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) rhe[kk] = rh[kk];
        } else {
          // pair f = k - 2 (rows r0 + 2f, r0 + 2f + 1) is transformed by CTA (f + 1) mod C
          const int f = k - 2;
          const unsigned own = (unsigned)((f + 1) % C);
          const int off = S::STG_OFF + ((f / C) % S::NSLOT) * XB + 2 * col;
          cs.st4(own, off, rhe[0], rh[0], rhe[1], rh[1]);
          cs.st4(own, off + 4, rhe[2], rh[2], rhe[3], rh[3]);
        }
      }
    }
    // boundary values for the neighbouring warps in the next iteration
    if (lane == 31) {
      eb(ws, 0, 1, warp) = ux[3];
      eb(ws, 1, 1, warp) = uy[3];
      eb(ws, 2, 1, warp) = sy1[3];
    }
    if (lane == 0) {
      eb(ws, 0, 0, warp) = ux[0];
      eb(ws, 1, 0, warp) = uy[0];
      eb(ws, 2, 0, warp) = sy1[0];
    }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      u2x[kk] = u1x[kk];
      u2y[kk] = u1y[kk];
      u1x[kk] = ux[kk];
      u1y[kk] = uy[kk];
      sx3[kk] = sx2[kk];
      sx2[kk] = sx1[kk];
      sy2[kk] = sy1[kk];
    }
    cp_wait<kAhead - 1>();  // the u* rows of iteration t+1 have landed
  };

  // ---- FFT role
  auto fft_role = [&]() {
    const int ft = tid - ST;
    const int grp = ft / FT;  // C == 1: group 0 inverse, group 1 forward
    const int jf = ft - grp * FT;
    float2* xinv = reinterpret_cast<float2*>(sm + S::INV_OFF);
    const float2* __restrict__ tw = fa.tw;
    constexpr int BARF = (C == 1) ? 3 : 2;
    auto inverse = [&](int q) { inverse_pair<N, C>(fa.spec_in, r0 - 4 + 2 * q, xinv, tw, jf, cs); };
    auto forward = [&](int f) {
      float2* stg = reinterpret_cast<float2*>(sm + S::STG_OFF + ((f / C) % S::NSLOT) * XB);
      forward_pair<N, BARF>(stg, fa.spec_out, r0 + 2 * f, tw, jf);
    };
    // prologue: p pairs 0, 1, 2
    if (grp == 0)
      for (int q = 0; q < 3; ++q)
        if (q % C == (int)rank) inverse(q);
    cluster_barrier<C>();
    // period k: inverse pair k + 3 and forward pair k - 3
#pragma unroll 1
    for (int k = 0; k < NK; ++k) {
      if (C == 1) {
        if (grp == 0) {
          if (k + 3 < NQ) inverse(k + 3);
        } else if (k >= 3) {
          forward(k - 3);
        }
      } else {
        if (k + 3 < NQ && (k + 3) % C == (int)rank) inverse(k + 3);
        if (k >= 3 && (k - 2) % C == (int)rank) forward(k - 3);
      }
      cluster_barrier<C>();
    }
    // epilogue: the last rhs pair (its rows were written in the last period)
    if (C == 1 ? grp == 1 : (NF % C == (int)rank)) forward(NF - 1);
  };

  if (!is_st) {
    fft_role();
    return;
  }

  // ---- stencil role: prologue (forcing rows, the first u* rows)
  {
    const ForcingRow fr = forcing_time(gldg(a.theta), gldg(a.theta + 1), t_now, c);
    for (int k = tid; k < r1 - r0 + 2; k += ST) sF[k] = forcing_fx((r0 - 1 + k) & M, fr, c);
    for (int k = tid; k < 12 * NWS; k += ST) sE[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < kAhead; ++k) issue_u(r0 - 2 + k);
    cp_wait<kAhead - 1>();
  }
  cluster_barrier<C>();
  // periods: stencil rows t0 and t0 + 1
#pragma unroll 1
  for (int k = 0; k < NK; ++k) {
    const int t0 = r0 - 2 + 2 * k;
    iterate(t0, 0, k);
    fft::group_sync<1, ST>();
    iterate(t0 + 1, 1, k);
    cluster_barrier<C>();
  }
  // objective partial of the CTA
  cp_wait<0>();
  jacc = warp_sum(jacc);
  if (lane == 0) sRed[warp] = jacc;
  fft::group_sync<1, ST>();
  if (warp == 0) {
    float v = lane < NWS ? sRed[lane] : 0.0f;
    v = warp_sum(v);
    if (lane == 0 && (unsigned)step < (unsigned)a.jpart_rows) {
      const int nblk = gridDim.x * gridDim.y;
      gst(a.jpart + (size_t)step * nblk + blockIdx.y * gridDim.x + blockIdx.x, v);
    }
  }
}

template <int SCHEME, int N>
__global__ void __cluster_dims__(fused::Shape<N>::C, 1, 1) __launch_bounds__(fused::Shape<N>::THREADS, 1)
    k_fused_rows(const FusedArgs fa) {
  fused_rows_body<SCHEME, N>(fa);
}

bool fused_supported(int N) { return N == 1024 || N == 2048 || N == 4096; }

int fused_cluster(int N) { return N > fused::kMaxW ? N / fused::kMaxW : 1; }

int fused_nblocks(int N, int th) { return fused_cluster(N) * ((N + th - 1) / th); }

template <int SCHEME, int N>
static cudaError_t launch_fused_n(const FusedArgs& f, cudaStream_t st) {
  using S = fused::Shape<N>;
  const size_t smem = fused::smem_bytes<N>(f.a.th);
  cudaError_t e = raise_smem_limit(k_fused_rows<SCHEME, N>);
  if (e != cudaSuccess) return e;
  const dim3 grid(S::C, (N + f.a.th - 1) / f.a.th);
  k_fused_rows<SCHEME, N><<<grid, S::THREADS, smem, st>>>(f);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_fused_s(int N, const FusedArgs& f, cudaStream_t st) {
  switch (N) {
    case 1024: return launch_fused_n<SCHEME, 1024>(f, st);
    case 2048: return launch_fused_n<SCHEME, 2048>(f, st);
    case 4096: return launch_fused_n<SCHEME, 4096>(f, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fused_rows(const FusedArgs& f, cudaStream_t st) {
  if (f.a.th < 2 || (f.a.th & 1) || f.a.th > f.a.c.N) return cudaErrorInvalidValue;
  return f.a.scheme == NSGB_SCHEME_UPWIND ? launch_fused_s<NSGB_SCHEME_UPWIND>(f.a.c.N, f, st)
                                          : launch_fused_s<NSGB_SCHEME_CENTRAL>(f.a.c.N, f, st);
}

// Row bands per launch that fit the GPU's co-resident clusters in one wave
// (the kernel holds one CTA per SM): the smallest even band height whose band
// count does not exceed the number of clusters that can be active at once.
template <int N>
static cudaError_t max_clusters_n(int& out) {
  using S = fused::Shape<N>;
  cudaError_t e = raise_smem_limit(k_fused_rows<NSGB_SCHEME_CENTRAL, N>);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S::C, 64);
  cfg.blockDim = dim3(S::THREADS);
  cfg.dynamicSmemBytes = fused::smem_bytes<N>(64);
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = S::C;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(&out, k_fused_rows<NSGB_SCHEME_CENTRAL, N>, &cfg);
}

cudaError_t fused_default_rows(int N, int& rows) {
  int maxc = 0;
  cudaError_t e = cudaErrorInvalidValue;
  switch (N) {
    case 1024: e = max_clusters_n<1024>(maxc); break;
    case 2048: e = max_clusters_n<2048>(maxc); break;
    case 4096: e = max_clusters_n<4096>(maxc); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  if (maxc < 1) return cudaErrorInvalidConfiguration;
  rows = 2 * ((N + 2 * maxc - 1) / (2 * maxc));
  if (rows < 2) rows = 2;
  return cudaSuccess;
}

NSGB_BOUNDS_UNIT(fused, 4)

}  // namespace nsgb
