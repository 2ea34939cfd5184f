// Discrete adjoint of one Chorin step (the reverse-mode derivative that
// jax.grad takes of SingleCoreNSSolver.objective, NS_solver.py:725, 742-756).
//
// Forward step s (exact arithmetic):  v = u + dt (nu L u + A(u) + f_s),
// u_{s+1} = Pr v with Pr = I - G P^-1 D, and J += jscale <u_x, f_x>,
// jscale = dt dx^2.  With periodic central differences G^T = -D and the
// spectral inverse Laplacian symmetric, so Pr^T = Pr and the adjoint recursion
// (lambda_S = 0) is
//   mu_s      = Pr lambda_{s+1}
//   lambda_s  = mu_s + dt (nu L mu_s + A'(u_s)^T mu_s) + jscale (f_x, 0)
//   dJ/dA,B  += sum_cells (jscale u_x + dt mu_x) dfx/dA,B
//   dJ/dnu   += dt <mu_s, L u_s>
// A'(u)^T for central advection A_c = -(u_x Gx u_c + u_y Gy u_c):
//   (A'^T mu)_x = -(mu_x Gx u_x + mu_y Gx u_y) + Gx(mu_x u_x) + Gy(mu_x u_y)
//   (A'^T mu)_y = -(mu_x Gy u_x + mu_y Gy u_y) + Gx(mu_y u_x) + Gy(mu_y u_y)
// and for upwind differences (masks m = [u >= 0] held fixed, as the
// derivative of jnp.where is taken):
//   (A'^T mu)_c = -(mu_x DX u_c... ) terms as below, with the transposed
//   one-sided operator (DX^m)^T w (i) = [(2m_i - 1) w_i - m_{i+1} w_{i+1}
//   + (1 - m_{i-1}) w_{i-1}] / dx.
// The projection Pr lambda_{s+1} reuses the forward machinery: the previous
// adjoint kernel wrote rhs = div(lambda_{s+1}) / dt, the FFT kernels solved for
// p, and this kernel applies mu = lambda - dt grad p on its tile.  The cell
// arithmetic uses the folded coefficients of the fused forward step (dt/h,
// dt nu/dx^2, 1/(h dt)) and FMAs; the theta sensitivities are summed in float
// over a thread's few cells and in double from there on.
#include "nsgb_internal.h"
#include "nsgb_rows.cuh"

namespace nsgb {

// Shared-memory planes of one TW x TH tile: p with a 3-cell halo, u and
// lambda with a 2-cell halo, all fetched as aligned float4 groups from column
// j0 - 4 (pitch W4 = TW + 8), then lambda_s on the tile + 1 halo (pitch SW).
template <int TW, int TH>
struct AdjointSmem {
  static constexpr int G = TW / 4 + 2;
  static constexpr int W4 = 4 * G;
  static constexpr int PH = TH + 6, UH = TH + 4, SH = TH + 2, SW = TW + 2;
  static constexpr int P_OFF = 0;
  static constexpr int UX_OFF = P_OFF + PH * W4;
  static constexpr int UY_OFF = UX_OFF + UH * W4;
  static constexpr int MX_OFF = UY_OFF + UH * W4;
  static constexpr int MY_OFF = MX_OFF + UH * W4;
  static constexpr int LX_OFF = MY_OFF + UH * W4;
  static constexpr int LY_OFF = LX_OFF + SH * SW;
  static constexpr int F_OFF = LY_OFF + SH * SW;  // fx for the SH rows
  static constexpr int DA_OFF = F_OFF + SH;        // dfx/dA, dfx/dB for the TH rows
  static constexpr int DB_OFF = DA_OFF + TH;
  static constexpr int RED_OFF = (DB_OFF + TH + 1) & ~1;  // 3 x 8 double-floats
  static constexpr size_t BYTES = (size_t)RED_OFF * sizeof(float) + 24 * sizeof(DFloat);
};

// lambda_s of one cell from mu and u at the cell (o) and its four
// neighbours n = (i+1, j), s = (i-1, j), e = (i, j+1), w = (i, j-1);
// fterm = jscale * f_x(i).  Both adjoint kernels use it, so they give the same
// bits.
struct AdjNbr {
  float o, n, s, e, w;
};
template <int SCHEME>
__device__ __forceinline__ void adjoint_cell(const AdjNbr& Mx, const AdjNbr& My, const AdjNbr& Ux, const AdjNbr& Uy,
                                             float cL, float cA, float fterm, float& lx, float& ly) {
  const float mx = Mx.o, my = My.o;
  const float lmx = fmaf(-4.0f, mx, (Mx.s + Mx.n) + (Mx.e + Mx.w));
  const float lmy = fmaf(-4.0f, my, (My.s + My.n) + (My.e + My.w));
  // at = h (A'(u)^T mu): the difference quotients' 1/h is folded into cA
  float atx, aty;
  if (SCHEME == NSGB_SCHEME_CENTRAL) {
    const float gxux = Ux.n - Ux.s, gxuy = Uy.n - Uy.s;
    const float gyux = Ux.e - Ux.w, gyuy = Uy.e - Uy.w;
    atx = -fmaf(mx, gxux, my * gxuy) + (fmaf(Mx.n, Ux.n, -Mx.s * Ux.s) + fmaf(Mx.e, Uy.e, -Mx.w * Uy.w));
    aty = -fmaf(mx, gyux, my * gyuy) + (fmaf(My.n, Ux.n, -My.s * Ux.s) + fmaf(My.e, Uy.e, -My.w * Uy.w));
  } else {
    const float uxo = Ux.o, uyo = Uy.o;
    const bool mxo = uxo >= 0.f, myo = uyo >= 0.f;
    // one-sided differences of u at o (the forward's dfx, dfy)
    const float dxux = mxo ? uxo - Ux.s : Ux.n - uxo;
    const float dxuy = mxo ? uyo - Uy.s : Uy.n - uyo;
    const float dyux = myo ? uxo - Ux.w : Ux.e - uxo;
    const float dyuy = myo ? uyo - Uy.w : Uy.e - uyo;
    atx = -fmaf(mx, dxux, my * dxuy);
    aty = -fmaf(mx, dyux, my * dyuy);
    // transposed one-sided operators applied to mu_c u_x (x) and mu_c u_y (y)
    const bool mxn = Ux.n >= 0.f, mxs = Ux.s >= 0.f;
    const bool mye = Uy.e >= 0.f, myw = Uy.w >= 0.f;
    auto dxt = [&](const AdjNbr& mu) {
      return (mxo ? mu.o * uxo : -mu.o * uxo) - (mxn ? mu.n * Ux.n : 0.f) + (mxs ? 0.f : mu.s * Ux.s);
    };
    auto dyt = [&](const AdjNbr& mu) {
      return (myo ? mu.o * uyo : -mu.o * uyo) - (mye ? mu.e * Uy.e : 0.f) + (myw ? 0.f : mu.w * Uy.w);
    };
    atx -= dxt(Mx) + dyt(Mx);
    aty -= dxt(My) + dyt(My);
  }
  lx = mx + fmaf(cL, lmx, fmaf(cA, atx, fterm));
  ly = my + fmaf(cL, lmy, cA * aty);
}

// dfx/dA and dfx/dB of row i at time t (the forcing's sensitivities to theta).
__device__ __forceinline__ void forcing_theta_grad(int i, const ForcingRow& fr, float A, float B, float t,
                                                   const StepConsts& c, float& dA, float& dB) {
  float fx, dmu, dsig;
  forcing_fx_grad(i, fr, c, fx, dmu, dsig);
  const float twopi = 6.28318548202514648f;
  const float argA = fmul(fmul(twopi, A), t);
  const float argB = fmul(fmul(twopi, B), t);
  const float cb = cosf(argB);
  // d mu/dA = cos(2 pi A t) 2 pi t ;  d sig/dB = -2 cos sin (2 pi B t) 2 pi t
  dA = dmu * (cosf(argA) * twopi * t);
  dB = dsig * (-2.0f * cb * sinf(argB) * twopi * t);
}

template <int SCHEME, int TW, int TH>
__device__ __forceinline__ void adjoint_body(const AdjointArgs& a) {
  using Lay = AdjointSmem<TW, TH>;
  constexpr int G = Lay::G, W4 = Lay::W4, PH = Lay::PH, UH = Lay::UH, SH = Lay::SH, SW = Lay::SW;
  extern __shared__ __align__(16) float sm[];
  float* sP = sm + Lay::P_OFF;
  float* sUx = sm + Lay::UX_OFF;
  float* sUy = sm + Lay::UY_OFF;
  float* sMx = sm + Lay::MX_OFF;
  float* sMy = sm + Lay::MY_OFF;
  float* sLx = sm + Lay::LX_OFF;
  float* sLy = sm + Lay::LY_OFF;
  float* sF = sm + Lay::F_OFF;
  float* sDA = sm + Lay::DA_OFF;
  float* sDB = sm + Lay::DB_OFF;
  DFloat* sRed = reinterpret_cast<DFloat*>(sm + Lay::RED_OFF);
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const int j0 = blockIdx.x * TW, i0 = blockIdx.y * TH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * 32 + tx;

  const float dt = c.dt;
  const float jscale = c.jscale;  // float32(dt * dx^2) = dJ/du_x / f_x
  const float nu = (a.theta_len == 3) ? gldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);                              // dt nu / dx^2
  const float cA = SCHEME == NSGB_SCHEME_CENTRAL ? c.cAc : c.cAu;  // dt / h
  const float t = fmul((float)a.step, dt);
  const float A = gldg(a.theta), B = gldg(a.theta + 1);

  const bool has_lam = a.lam != nullptr;
  const bool has_p = a.p != nullptr;
  // aligned float4 tile loads (a group never straddles the periodic wrap)
  if (has_p) {
    const float* __restrict__ pp = a.p;
    forflat<PH, G>(tid, [&](int r, int q) {
      const float4 v = gldg4(pp + (size_t)((i0 - 3 + r) & M) * N + ((j0 - 4 + 4 * q) & M));
      *reinterpret_cast<float4*>(sP + r * W4 + 4 * q) = v;
    });
  }
  {
    const float* __restrict__ u = a.u;
    const float* __restrict__ lam = a.lam;
    forflat<UH, G>(tid, [&](int r, int q) {
      const size_t g = (size_t)((i0 - 2 + r) & M) * N + ((j0 - 4 + 4 * q) & M);
      const int o = r * W4 + 4 * q;
      *reinterpret_cast<float4*>(sUx + o) = gldg4(u + g);
      *reinterpret_cast<float4*>(sUy + o) = gldg4(u + NN + g);
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(sMx + o) = has_lam ? gldg4(lam + g) : z;
      *reinterpret_cast<float4*>(sMy + o) = has_lam ? gldg4(lam + NN + g) : z;
    });
  }
  {
    const ForcingRow fr = forcing_time(A, B, t, c);
    if (tid < SH) {
      sF[tid] = forcing_fx((i0 - 1 + tid) & M, fr, c);
    } else if (tid >= 64 && tid < 64 + TH) {
      const int r = tid - 64;
      forcing_theta_grad((i0 + r) & M, fr, A, B, t, c, sDA[r], sDB[r]);
    }
  }
  __syncthreads();

  // mu = lambda - dt grad p on rows i0-2 .. i0+TH+1, columns j0-2 .. j0+TW+1
  if (has_p) {
    forflat<UH, TW + 4>(tid, [&](int r, int cc) {
      const int col = cc + 2;
      const float* P0 = sP + (r + 1) * W4 + col;
      const int o = r * W4 + col;
      sMx[o] = fused_proj(sMx[o], P0[W4], P0[-W4], c.cP);
      sMy[o] = fused_proj(sMy[o], P0[1], P0[-1], c.cP);
    });
    __syncthreads();
  }

  // theta sensitivities of the interior cells: float over a thread's few
  // cells, double-float across the block's threads, double across blocks and
  // steps (the nu term is a small difference of large contributions)
  float fA = 0.f, fB = 0.f, fN = 0.f;
  forflat<TH, TW>(tid, [&](int r, int cc) {
    const int o = (r + 2) * W4 + (cc + 4);
    const float w = fmaf(jscale, sUx[o], dt * sMx[o]);
    fA = fmaf(w, sDA[r], fA);
    fB = fmaf(w, sDB[r], fB);
    // Laplacian sums from neighbour differences: for a smooth field each
    // difference of close values is exact, so the small sum keeps its digits
    // (summing the neighbours first would cancel about two of them)
    const float ox = sUx[o], oy = sUy[o];
    const float lux = ((sUx[o - W4] - ox) + (sUx[o + W4] - ox)) + ((sUx[o + 1] - ox) + (sUx[o - 1] - ox));
    const float luy = ((sUy[o - W4] - oy) + (sUy[o + W4] - oy)) + ((sUy[o + 1] - oy) + (sUy[o - 1] - oy));
    fN = fmaf(sMx[o], lux, fmaf(sMy[o], luy, fN));
  });

  // lambda_s on rows i0-1 .. i0+TH, columns j0-1 .. j0+TW
  forflat<SH, SW>(tid, [&](int r, int cc) {
    const int o = (r + 1) * W4 + (cc + 3);
    const int n = o + W4, s = o - W4, e = o + 1, w = o - 1;  // i+1, i-1, j+1, j-1
    const AdjNbr Mx = {sMx[o], sMx[n], sMx[s], sMx[e], sMx[w]};
    const AdjNbr My = {sMy[o], sMy[n], sMy[s], sMy[e], sMy[w]};
    const AdjNbr Ux = {sUx[o], sUx[n], sUx[s], sUx[e], sUx[w]};
    const AdjNbr Uy = {sUy[o], sUy[n], sUy[s], sUy[e], sUy[w]};
    adjoint_cell<SCHEME>(Mx, My, Ux, Uy, cL, cA, jscale * sF[r], sLx[r * SW + cc], sLy[r * SW + cc]);
  });
  __syncthreads();

  {
    float* __restrict__ lo = a.lam_out;
    float* __restrict__ rhs = a.rhs;
    forflat<TH, TW>(tid, [&](int r, int cc) {
      const int o = (r + 1) * SW + (cc + 1);
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      gst(lo + g, sLx[o]);
      gst(lo + NN + g, sLy[o]);
      gst(rhs + g, fused_rhs(sLx[o + SW], sLx[o - SW], sLy[o + 1], sLy[o - 1], c.cD));
    });
  }

  const DFloat gA = warp_sum_df({fA, 0.f});
  const DFloat gB = warp_sum_df({fB, 0.f});
  const DFloat gN = warp_sum_df({fN, 0.f});
  if (tx == 0) {
    sRed[ty] = gA;
    sRed[8 + ty] = gB;
    sRed[16 + ty] = gN;
  }
  __syncthreads();
  if (ty == 0) {
    const DFloat z = {0.f, 0.f};
    const DFloat v0 = warp_sum_df(tx < 8 ? sRed[tx] : z);
    const DFloat v1 = warp_sum_df(tx < 8 ? sRed[8 + tx] : z);
    const DFloat v2 = warp_sum_df(tx < 8 ? sRed[16 + tx] : z);
    if (tx == 0) {
      const int nblk = gridDim.x * gridDim.y;
      double* gp = a.gpart + ((size_t)a.gslot * nblk + blockIdx.y * gridDim.x + blockIdx.x) * 3;
      gst(gp, (double)v0.hi + (double)v0.lo);
      gst(gp + 1, (double)v1.hi + (double)v1.lo);
      // the nu partial carries the Laplacian's 1/dx^2 and the step's dt
      gst(gp + 2, ((double)v2.hi + (double)v2.lo) * ((double)dt * (double)c.rdx2));
    }
  }
}

template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_adjoint(const AdjointArgs a) {
  adjoint_body<SCHEME, TW, TH>(a);
}
// Batched form: blockIdx.z selects the solve's arguments.
template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_adjoint_b(const AdjointArgs* __restrict__ tab) {
  adjoint_body<SCHEME, TW, TH>(tab[blockIdx.z]);
}

// a: the shape, scheme and N of the launch; tab (device, count entries) or
// nullptr for the single launch with a itself.
template <int SCHEME, int TW, int TH>
static cudaError_t launch_adjoint_t(const AdjointArgs& a, const AdjointArgs* tab, int count, cudaStream_t st) {
  const cudaError_t e = tab ? raise_smem_limit(k_adjoint_b<SCHEME, TW, TH>) : raise_smem_limit(k_adjoint<SCHEME, TW, TH>);
  if (e != cudaSuccess) return e;
  const dim3 grid(a.c.N / TW, a.c.N / TH, tab ? count : 1);
  if (tab)
    k_adjoint_b<SCHEME, TW, TH><<<grid, dim3(32, 8), AdjointSmem<TW, TH>::BYTES, st>>>(tab);
  else
    k_adjoint<SCHEME, TW, TH><<<grid, dim3(32, 8), AdjointSmem<TW, TH>::BYTES, st>>>(a);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_adjoint_s(const AdjointArgs& a, const AdjointArgs* tab, int count, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (a.tw == W && a.th == H) return launch_adjoint_t<SCHEME, W, H>(a, tab, count, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

// ------------------------------------------------------ row-streaming --
// The adjoint step marched down row bands, as the forward row kernel does
// (nsgb_rows.cuh): thread g owns four columns and at iteration t
//   - forms mu(t) = lambda_{s+1}(t) - dt grad p from p rows t-1, t, t+1,
//   - forms lambda_s(t-1) from mu rows t-2, t-1, t (registers), the edge
//     values of mu(t-1) of the neighbouring groups and u rows t-2 .. t (ring),
//     and adds the theta partials of row t-1,
//   - writes lambda_s(t-2) and rhs(t-2) = div(lambda_s)/dt.
// p, lambda_{s+1} and u_s stream through shared-memory rings by asynchronous
// copies kAhead rows ahead; the cells use the tiled kernel's arithmetic
// (adjoint_cell), so lambda_s and rhs have the same bits.
namespace adjrows {
constexpr int F_MX = 0, F_MY = 1, F_LY = 2;  // exchanged fields
constexpr int kAhead = 3;                    // rows copied ahead of use
constexpr int kPRing = 8;                    // p rows t-1 .. t+1+kAhead
constexpr int kLRing = 4;                    // lambda rows t .. t+kAhead
constexpr int kURing = 8;                    // u rows t-2 .. t+kAhead
static_assert(kPRing >= kAhead + 3 && kLRing >= kAhead + 1 && kURing >= kAhead + 3, "ring depth");
constexpr int kMaxWarps = 32;
// rings, edges [2 slots][3 fields][2 sides][G], f_x of RH + 2 rows, dfx/dA and
// dfx/dB of RH rows, per-warp double-float partials
inline size_t smem_bytes(int N, int W, int RH) {
  return sizeof(float) * ((size_t)(kPRing + 2 * kLRing + 2 * kURing) * rows::ring_stride(W) +
                          (size_t)12 * rows::groups(N, W) + (RH + 2) + 2 * RH) +
         sizeof(DFloat) * 3 * kMaxWarps;
}
}  // namespace adjrows

template <int SCHEME>
__device__ __forceinline__ void adjoint_rows_body(const AdjointArgs& a) {
  using namespace rows;
  using adjrows::kAhead;
  using adjrows::kLRing;
  using adjrows::kPRing;
  using adjrows::kURing;
  using adjrows::F_LY;
  using adjrows::F_MX;
  using adjrows::F_MY;
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
  float* sP = sm;                   // [kPRing][RS]
  float* sLX = sP + kPRing * RS;    // [kLRing][RS]
  float* sLY = sLX + kLRing * RS;   // [kLRing][RS]
  float* sUX = sLY + kLRing * RS;   // [kURing][RS]
  float* sUY = sUX + kURing * RS;   // [kURing][RS]
  float* sE = sUY + kURing * RS;    // [slot][field][side][G]
  float* sF = sE + 12 * G;          // f_x of rows r0-1 .. r1
  float* sDA = sF + RH + 2;         // dfx/dA of rows r0 .. r1-1
  float* sDB = sDA + RH;            // dfx/dB
  DFloat* sRed = reinterpret_cast<DFloat*>(sDB + RH);  // [3][kMaxWarps]
  auto edge = [&](int slot, int f, int side) { return sE + ((slot * 3 + f) * 2 + side) * G; };

  const float dt = c.dt;
  const float jscale = c.jscale;
  const float nu = (a.theta_len == 3) ? gldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);
  const float cA = SCHEME == NSGB_SCHEME_CENTRAL ? c.cAc : c.cAu;
  const float tf = fmul((float)a.step, dt);
  const float A = gldg(a.theta), B = gldg(a.theta + 1);
  {
    const ForcingRow fr = forcing_time(A, B, tf, c);
    for (int k = tid; k < r1 - r0 + 2; k += blockDim.x) sF[k] = forcing_fx((r0 - 1 + k) & M, fr, c);
    for (int k = tid; k < r1 - r0; k += blockDim.x) forcing_theta_grad((r0 + k) & M, fr, A, B, tf, c, sDA[k], sDB[k]);
  }

  const bool has_p = a.p != nullptr;
  const bool has_lam = a.lam != nullptr;
  const uint64_t pol = evict_first_policy();
  // one copy group: p row `pr` (if do_p), lambda and u rows `lr` (if do_lu)
  auto issue = [&](int pr, bool do_p, int lr, bool do_lu) {
    if (do_p && has_p) copy_row(sP + (pr & (kPRing - 1)) * RS, a.p, pr, N, M, wrap, active, tid, G, bi, col, pol);
    if (do_lu) {
      if (has_lam && active) {  // only the group's own columns of lambda are read
        const size_t o = (size_t)(lr & M) * N + col;
        cp16(sLX + (lr & (kLRing - 1)) * RS + bi, a.lam + o, pol);
        cp16(sLY + (lr & (kLRing - 1)) * RS + bi, a.lam + NN + o, pol);
      }
      copy_row(sUX + (lr & (kURing - 1)) * RS, a.u, lr, N, M, wrap, active, tid, G, bi, col, pol);
      copy_row(sUY + (lr & (kURing - 1)) * RS, a.u + NN, lr, N, M, wrap, active, tid, G, bi, col, pol);
    }
    cp_commit();
  };
  // prologue: p rows r0-3, r0-2, then the groups of iterations r0-2-kAhead ..
  // r0-3 (p rows r0-1 .., lambda and u rows r0-2 ..); wait for those of
  // iteration r0-2
  issue(r0 - 3, true, 0, false);
  issue(r0 - 2, true, 0, false);
#pragma unroll
  for (int k = kAhead; k >= 1; --k) issue(r0 - 1 - k + kAhead, true, r0 - 2 - k + kAhead, true);
  cp_wait<kAhead - 1>();
  __syncthreads();

  // registers entering iteration t: mu rows t-1, t-2; lambda_s x rows t-3,
  // t-2 and y row t-2
  float m1x[4] = {0, 0, 0, 0}, m1y[4] = {0, 0, 0, 0}, m2x[4] = {0, 0, 0, 0}, m2y[4] = {0, 0, 0, 0};
  float lx3[4] = {0, 0, 0, 0}, lx2[4] = {0, 0, 0, 0}, ly2[4] = {0, 0, 0, 0};
  // theta partials: float over a row's four cells, double-float over rows
  DFloat gA = {0.f, 0.f}, gB = {0.f, 0.f}, gN = {0.f, 0.f};
  float* __restrict__ lo_x = a.lam_out;
  float* __restrict__ lo_y = a.lam_out + NN;
  float* __restrict__ rhs_g = a.rhs;
#pragma unroll 1
  for (int t = r0 - 2; t <= r1 + 1; ++t) {
    const int rs = (t - 1) & 1, ws = t & 1;
    issue(t + 1 + kAhead, true, t + kAhead, true);

    // mu(t) = lambda(t) - dt grad p
    float mx[4] = {0, 0, 0, 0}, my[4] = {0, 0, 0, 0};
    if (has_lam) {
      ld4s(sLX + (t & (kLRing - 1)) * RS + bi, mx);
      ld4s(sLY + (t & (kLRing - 1)) * RS + bi, my);
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
        mx[k] = fused_proj(mx[k], pn[k], pm[k], c.cP);
        my[k] = fused_proj(my[k], P[k + 2], P[k], c.cP);
      }
    }

    // lambda_s(t-1) and the theta partials of row t-1
    float lx1[4] = {0, 0, 0, 0}, ly1[4] = {0, 0, 0, 0};
    if (t >= r0) {
      const float* ucx = sUX + ((t - 1) & (kURing - 1)) * RS + bi;
      const float* ucy = sUY + ((t - 1) & (kURing - 1)) * RS + bi;
      float cx[4], cy[4], nx[4], ny[4], sx[4], sy[4];
      ld4s(ucx, cx);
      ld4s(ucy, cy);
      ld4s(sUX + (t & (kURing - 1)) * RS + bi, nx);
      ld4s(sUY + (t & (kURing - 1)) * RS + bi, ny);
      ld4s(sUX + ((t - 2) & (kURing - 1)) * RS + bi, sx);
      ld4s(sUY + ((t - 2) & (kURing - 1)) * RS + bi, sy);
      const float UX[6] = {ucx[-1], cx[0], cx[1], cx[2], cx[3], ucx[4]};
      const float UY[6] = {ucy[-1], cy[0], cy[1], cy[2], cy[3], ucy[4]};
      const float MX[6] = {edge(rs, F_MX, 1)[gl], m1x[0], m1x[1], m1x[2], m1x[3], edge(rs, F_MX, 0)[gr]};
      const float MY[6] = {edge(rs, F_MY, 1)[gl], m1y[0], m1y[1], m1y[2], m1y[3], edge(rs, F_MY, 0)[gr]};
      const float fterm = jscale * sF[t - r0];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const AdjNbr Mx = {MX[k + 1], mx[k], m2x[k], MX[k + 2], MX[k]};
        const AdjNbr My = {MY[k + 1], my[k], m2y[k], MY[k + 2], MY[k]};
        const AdjNbr Ux = {UX[k + 1], nx[k], sx[k], UX[k + 2], UX[k]};
        const AdjNbr Uy = {UY[k + 1], ny[k], sy[k], UY[k + 2], UY[k]};
        adjoint_cell<SCHEME>(Mx, My, Ux, Uy, cL, cA, fterm, lx1[k], ly1[k]);
      }
      if (store && t - 1 >= r0 && t - 1 < r1) {
        const float dA = sDA[t - 1 - r0], dB = sDB[t - 1 - r0];
        float fA = 0.f, fB = 0.f, fN = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float ox = UX[k + 1], oy = UY[k + 1];
          const float w = fmaf(jscale, ox, dt * MX[k + 1]);
          fA = fmaf(w, dA, fA);
          fB = fmaf(w, dB, fB);
          // Laplacian sums from neighbour differences (the tiled kernel's order)
          const float lux = ((sx[k] - ox) + (nx[k] - ox)) + ((UX[k + 2] - ox) + (UX[k] - ox));
          const float luy = ((sy[k] - oy) + (ny[k] - oy)) + ((UY[k + 2] - oy) + (UY[k] - oy));
          fN = fmaf(MX[k + 1], lux, fmaf(MY[k + 1], luy, fN));
        }
        gA = df_add(gA, {fA, 0.f});
        gB = df_add(gB, {fB, 0.f});
        gN = df_add(gN, {fN, 0.f});
      }
    }

    // lambda_s(t-2) and rhs(t-2)
    if (t >= r0 + 2 && store) {
      const float Y2[6] = {edge(rs, F_LY, 1)[gl], ly2[0], ly2[1], ly2[2], ly2[3], edge(rs, F_LY, 0)[gr]};
      float rh[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) rh[k] = fused_rhs(lx1[k], lx3[k], Y2[k + 2], Y2[k], c.cD);
      const size_t o = (size_t)((t - 2) & M) * N + col;
      st4_stream(lo_x, o, lx2);
      st4_stream(lo_y, o, ly2);
      st4(rhs_g, o, rh);
    }

    // edge values for the next iteration: mu(t), lambda_s y(t-1)
    if (active) {
      edge(ws, F_MX, 0)[g] = mx[0];
      edge(ws, F_MX, 1)[g] = mx[3];
      edge(ws, F_MY, 0)[g] = my[0];
      edge(ws, F_MY, 1)[g] = my[3];
      edge(ws, F_LY, 0)[g] = ly1[0];
      edge(ws, F_LY, 1)[g] = ly1[3];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      m2x[k] = m1x[k];
      m2y[k] = m1y[k];
      m1x[k] = mx[k];
      m1y[k] = my[k];
      lx3[k] = lx2[k];
      lx2[k] = lx1[k];
      ly2[k] = ly1[k];
    }
    cp_wait<kAhead - 1>();  // the rows of iteration t+1 have landed
    __syncthreads();
  }
  cp_wait<0>();

  // theta partials of the CTA: double-float across threads
  gA = warp_sum_df(gA);
  gB = warp_sum_df(gB);
  gN = warp_sum_df(gN);
  const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  if (lane == 0) {
    sRed[warp] = gA;
    sRed[adjrows::kMaxWarps + warp] = gB;
    sRed[2 * adjrows::kMaxWarps + warp] = gN;
  }
  __syncthreads();
  if (warp == 0) {
    const DFloat z = {0.f, 0.f};
    const DFloat v0 = warp_sum_df(lane < nwarps ? sRed[lane] : z);
    const DFloat v1 = warp_sum_df(lane < nwarps ? sRed[adjrows::kMaxWarps + lane] : z);
    const DFloat v2 = warp_sum_df(lane < nwarps ? sRed[2 * adjrows::kMaxWarps + lane] : z);
    if (lane == 0) {
      const int nblk = gridDim.x * gridDim.y;
      double* gp = a.gpart + ((size_t)a.gslot * nblk + blockIdx.y * gridDim.x + blockIdx.x) * 3;
      gst(gp, (double)v0.hi + (double)v0.lo);
      gst(gp + 1, (double)v1.hi + (double)v1.lo);
      gst(gp + 2, ((double)v2.hi + (double)v2.lo) * ((double)dt * (double)c.rdx2));
    }
  }
}

template <int SCHEME>
__global__ void __launch_bounds__(NSGB_ADJ_ROWS_MAX_W / 4 + 32) k_adjoint_rows(const AdjointArgs a) {
  adjoint_rows_body<SCHEME>(a);
}
template <int SCHEME>
__global__ void __launch_bounds__(NSGB_ADJ_ROWS_MAX_W / 4 + 32) k_adjoint_rows_b(const AdjointArgs* __restrict__ tab) {
  adjoint_rows_body<SCHEME>(tab[blockIdx.z]);
}

bool adjoint_rows_supported(int N, int tw, int th) {
  if (!stencil_rows_mode(tw) || (tw & (tw - 1)) != 0 || tw > NSGB_ADJ_ROWS_MAX_W) return false;
  return th >= 1 && th <= N && adjrows::smem_bytes(N, rows::band_width(N, tw), th) <= 227 * 1024;
}

template <int SCHEME>
static cudaError_t launch_adjoint_rows(const AdjointArgs& a, const AdjointArgs* tab, int count, cudaStream_t st) {
  const int N = a.c.N;
  const int W = rows::band_width(N, a.tw);
  const size_t smem = adjrows::smem_bytes(N, W, a.th);
  if (smem > 48 * 1024) {
    const cudaError_t e = tab ? raise_smem_limit(k_adjoint_rows_b<SCHEME>) : raise_smem_limit(k_adjoint_rows<SCHEME>);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid(N / W, (N + a.th - 1) / a.th, tab ? count : 1);
  if (tab)
    k_adjoint_rows_b<SCHEME><<<grid, rows::threads(N, W), smem, st>>>(tab);
  else
    k_adjoint_rows<SCHEME><<<grid, rows::threads(N, W), smem, st>>>(a);
  return cudaGetLastError();
}

static cudaError_t launch_adjoint_any(const AdjointArgs& a, const AdjointArgs* tab, int count, cudaStream_t st) {
  if (stencil_rows_mode(a.tw))
    return a.scheme == NSGB_SCHEME_CENTRAL ? launch_adjoint_rows<NSGB_SCHEME_CENTRAL>(a, tab, count, st)
                                           : launch_adjoint_rows<NSGB_SCHEME_UPWIND>(a, tab, count, st);
  return a.scheme == NSGB_SCHEME_CENTRAL ? launch_adjoint_s<NSGB_SCHEME_CENTRAL>(a, tab, count, st)
                                         : launch_adjoint_s<NSGB_SCHEME_UPWIND>(a, tab, count, st);
}

cudaError_t launch_adjoint_stencil(const AdjointArgs& a, cudaStream_t st) {
  return launch_adjoint_any(a, nullptr, 1, st);
}

cudaError_t launch_adjoint_batch(const AdjointArgs& shape, const AdjointArgs* tab, int count, cudaStream_t st) {
  if (!tab || count < 1) return cudaErrorInvalidValue;
  return launch_adjoint_any(shape, tab, count, st);
}

// Fixed-order reduction of nrows x nblk x 3 partials into gacc[3] (double):
// one CTA per row sums the row's blocks by a fixed tree, then one thread adds
// the row sums to gacc in row order.
__global__ void k_greduce_rows(const double* __restrict__ gpart, int nblk, double* __restrict__ rowsum) {
  __shared__ double red[3][256];
  const double* base = gpart + (size_t)blockIdx.x * nblk * 3;
  double v0 = 0, v1 = 0, v2 = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    v0 += gld(base + 3 * b);
    v1 += gld(base + 3 * b + 1);
    v2 += gld(base + 3 * b + 2);
  }
  red[0][threadIdx.x] = v0;
  red[1][threadIdx.x] = v1;
  red[2][threadIdx.x] = v2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
      red[2][threadIdx.x] += red[2][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x < 3) gst(rowsum + 3 * blockIdx.x + threadIdx.x, red[threadIdx.x][0]);
}

__global__ void k_greduce_acc(const double* __restrict__ rowsum, int nrows, double* __restrict__ gacc) {
  if (threadIdx.x >= 3) return;
  double g = gld(gacc + threadIdx.x);
  for (int row = 0; row < nrows; ++row) g += gld(rowsum + 3 * row + threadIdx.x);
  gst(gacc + threadIdx.x, g);
}

cudaError_t launch_greduce(const double* gpart, int nblk, int nrows, double* rowsum, double* gacc,
                           cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_greduce_rows<<<nrows, 256, 0, st>>>(gpart, nblk, rowsum);
  k_greduce_acc<<<1, 32, 0, st>>>(rowsum, nrows, gacc);
  return cudaGetLastError();
}

__global__ void k_gfinal(const double* __restrict__ gacc, int theta_len, float* __restrict__ dJ) {
  for (int k = 0; k < theta_len; ++k) gst(dJ + k, (float)gld(gacc + k));
}

cudaError_t launch_gfinal(const double* gacc, int theta_len, float* dJ, cudaStream_t st) {
  k_gfinal<<<1, 1, 0, st>>>(gacc, theta_len, dJ);
  return cudaGetLastError();
}

NSGB_BOUNDS_UNIT(adjoint, 3)

}  // namespace nsgb
