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

template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_adjoint(const AdjointArgs a) {
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
  const float nu = (a.theta_len == 3) ? __ldg(a.theta + 2) : c.nu;
  const float cL = fmul(c.dtdx2, nu);                              // dt nu / dx^2
  const float cA = SCHEME == NSGB_SCHEME_CENTRAL ? c.cAc : c.cAu;  // dt / h
  const float t = fmul((float)a.step, dt);
  const float A = __ldg(a.theta), B = __ldg(a.theta + 1);

  const bool has_lam = a.lam != nullptr;
  const bool has_p = a.p != nullptr;
  // aligned float4 tile loads (a group never straddles the periodic wrap)
  if (has_p) {
    const float* __restrict__ pp = a.p;
    forflat<PH, G>(tid, [&](int r, int q) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(
          pp + (size_t)((i0 - 3 + r) & M) * N + ((j0 - 4 + 4 * q) & M)));
      *reinterpret_cast<float4*>(sP + r * W4 + 4 * q) = v;
    });
  }
  {
    const float* __restrict__ u = a.u;
    const float* __restrict__ lam = a.lam;
    forflat<UH, G>(tid, [&](int r, int q) {
      const size_t g = (size_t)((i0 - 2 + r) & M) * N + ((j0 - 4 + 4 * q) & M);
      const int o = r * W4 + 4 * q;
      *reinterpret_cast<float4*>(sUx + o) = __ldg(reinterpret_cast<const float4*>(u + g));
      *reinterpret_cast<float4*>(sUy + o) = __ldg(reinterpret_cast<const float4*>(u + NN + g));
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(sMx + o) = has_lam ? __ldg(reinterpret_cast<const float4*>(lam + g)) : z;
      *reinterpret_cast<float4*>(sMy + o) = has_lam ? __ldg(reinterpret_cast<const float4*>(lam + NN + g)) : z;
    });
  }
  {
    const ForcingRow fr = forcing_time(A, B, t, c);
    if (tid < SH) {
      sF[tid] = forcing_fx((i0 - 1 + tid) & M, fr, c);
    } else if (tid >= 64 && tid < 64 + TH) {
      const int r = tid - 64;
      float fx, dmu, dsig;
      forcing_fx_grad((i0 + r) & M, fr, c, fx, dmu, dsig);
      const float twopi = 6.28318548202514648f;
      const float argA = fmul(fmul(twopi, A), t);
      const float argB = fmul(fmul(twopi, B), t);
      const float cb = cosf(argB);
      // d mu/dA = cos(2 pi A t) 2 pi t ;  d sig/dB = -2 cos sin (2 pi B t) 2 pi t
      sDA[r] = dmu * (cosf(argA) * twopi * t);
      sDB[r] = dsig * (-2.0f * cb * sinf(argB) * twopi * t);
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
    const float mx = sMx[o], my = sMy[o];
    const float lmx = fmaf(-4.0f, mx, (sMx[s] + sMx[n]) + (sMx[e] + sMx[w]));
    const float lmy = fmaf(-4.0f, my, (sMy[s] + sMy[n]) + (sMy[e] + sMy[w]));
    // at = h (A'(u)^T mu): the difference quotients' 1/h is folded into cA
    float atx, aty;
    if (SCHEME == NSGB_SCHEME_CENTRAL) {
      const float gxux = sUx[n] - sUx[s], gxuy = sUy[n] - sUy[s];
      const float gyux = sUx[e] - sUx[w], gyuy = sUy[e] - sUy[w];
      atx = -fmaf(mx, gxux, my * gxuy) +
            (fmaf(sMx[n], sUx[n], -sMx[s] * sUx[s]) + fmaf(sMx[e], sUy[e], -sMx[w] * sUy[w]));
      aty = -fmaf(mx, gyux, my * gyuy) +
            (fmaf(sMy[n], sUx[n], -sMy[s] * sUx[s]) + fmaf(sMy[e], sUy[e], -sMy[w] * sUy[w]));
    } else {
      const float uxo = sUx[o], uyo = sUy[o];
      const bool mxo = uxo >= 0.f, myo = uyo >= 0.f;
      // one-sided differences of u at o (the forward's dfx, dfy)
      const float dxux = mxo ? uxo - sUx[s] : sUx[n] - uxo;
      const float dxuy = mxo ? uyo - sUy[s] : sUy[n] - uyo;
      const float dyux = myo ? uxo - sUx[w] : sUx[e] - uxo;
      const float dyuy = myo ? uyo - sUy[w] : sUy[e] - uyo;
      atx = -fmaf(mx, dxux, my * dxuy);
      aty = -fmaf(mx, dyux, my * dyuy);
      // transposed one-sided operators applied to mu_c u_x (x) and mu_c u_y (y)
      const bool mxn = sUx[n] >= 0.f, mxs = sUx[s] >= 0.f;
      const bool mye = sUy[e] >= 0.f, myw = sUy[w] >= 0.f;
      auto dxt = [&](const float* mu) {
        return (mxo ? mu[o] * uxo : -mu[o] * uxo) - (mxn ? mu[n] * sUx[n] : 0.f) +
               (mxs ? 0.f : mu[s] * sUx[s]);
      };
      auto dyt = [&](const float* mu) {
        return (myo ? mu[o] * uyo : -mu[o] * uyo) - (mye ? mu[e] * sUy[e] : 0.f) +
               (myw ? 0.f : mu[w] * sUy[w]);
      };
      atx -= dxt(sMx) + dyt(sMx);
      aty -= dxt(sMy) + dyt(sMy);
    }
    sLx[r * SW + cc] = mx + fmaf(cL, lmx, fmaf(cA, atx, jscale * sF[r]));
    sLy[r * SW + cc] = my + fmaf(cL, lmy, cA * aty);
  });
  __syncthreads();

  {
    float* __restrict__ lo = a.lam_out;
    float* __restrict__ rhs = a.rhs;
    forflat<TH, TW>(tid, [&](int r, int cc) {
      const int o = (r + 1) * SW + (cc + 1);
      const size_t g = (size_t)(i0 + r) * N + (j0 + cc);
      lo[g] = sLx[o];
      lo[NN + g] = sLy[o];
      rhs[g] = fused_rhs(sLx[o + SW], sLx[o - SW], sLy[o + 1], sLy[o - 1], c.cD);
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
      gp[0] = (double)v0.hi + (double)v0.lo;
      gp[1] = (double)v1.hi + (double)v1.lo;
      // the nu partial carries the Laplacian's 1/dx^2 and the step's dt
      gp[2] = ((double)v2.hi + (double)v2.lo) * ((double)dt * (double)c.rdx2);
    }
  }
}

template <int SCHEME, int TW, int TH>
static cudaError_t launch_adjoint_t(const AdjointArgs& a, cudaStream_t st) {
  const cudaError_t e = raise_smem_limit(k_adjoint<SCHEME, TW, TH>);
  if (e != cudaSuccess) return e;
  const dim3 grid(a.c.N / TW, a.c.N / TH);
  k_adjoint<SCHEME, TW, TH><<<grid, dim3(32, 8), AdjointSmem<TW, TH>::BYTES, st>>>(a);
  return cudaGetLastError();
}

template <int SCHEME>
static cudaError_t launch_adjoint_s(const AdjointArgs& a, cudaStream_t st) {
#define NSGB_TILE_CASE(W, H) \
  if (a.tw == W && a.th == H) return launch_adjoint_t<SCHEME, W, H>(a, st);
  NSGB_STENCIL_TILES(NSGB_TILE_CASE)
#undef NSGB_TILE_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_adjoint_stencil(const AdjointArgs& a, cudaStream_t st) {
  return a.scheme == NSGB_SCHEME_CENTRAL ? launch_adjoint_s<NSGB_SCHEME_CENTRAL>(a, st)
                                         : launch_adjoint_s<NSGB_SCHEME_UPWIND>(a, st);
}

// Fixed-order reduction of nrows x nblk x 3 partials into gacc[3] (double):
// one CTA per row sums the row's blocks by a fixed tree, then one thread adds
// the row sums to gacc in row order.
__global__ void k_greduce_rows(const double* __restrict__ gpart, int nblk, double* __restrict__ rowsum) {
  __shared__ double red[3][256];
  const double* base = gpart + (size_t)blockIdx.x * nblk * 3;
  double v0 = 0, v1 = 0, v2 = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    v0 += base[3 * b];
    v1 += base[3 * b + 1];
    v2 += base[3 * b + 2];
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
  if (threadIdx.x < 3) rowsum[3 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_greduce_acc(const double* __restrict__ rowsum, int nrows, double* __restrict__ gacc) {
  if (threadIdx.x >= 3) return;
  double g = gacc[threadIdx.x];
  for (int row = 0; row < nrows; ++row) g += rowsum[3 * row + threadIdx.x];
  gacc[threadIdx.x] = g;
}

cudaError_t launch_greduce(const double* gpart, int nblk, int nrows, double* rowsum, double* gacc,
                           cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_greduce_rows<<<nrows, 256, 0, st>>>(gpart, nblk, rowsum);
  k_greduce_acc<<<1, 32, 0, st>>>(rowsum, nrows, gacc);
  return cudaGetLastError();
}

__global__ void k_gfinal(const double* __restrict__ gacc, int theta_len, float* __restrict__ dJ) {
  for (int k = 0; k < theta_len; ++k) dJ[k] = (float)gacc[k];
}

cudaError_t launch_gfinal(const double* gacc, int theta_len, float* dJ, cudaStream_t st) {
  k_gfinal<<<1, 1, 0, st>>>(gacc, theta_len, dJ);
  return cudaGetLastError();
}

}  // namespace nsgb
