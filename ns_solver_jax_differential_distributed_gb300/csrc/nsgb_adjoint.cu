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
// p, and this kernel applies mu = lambda - dt grad p on its tile.
#include "nsgb_internal.h"

namespace nsgb {

template <int SCHEME, int TW, int TH>
__global__ void __launch_bounds__(256) k_adjoint(const AdjointArgs a) {
  extern __shared__ float sm[];
  const StepConsts& c = a.c;
  const int N = c.N, M = N - 1;
  const size_t NN = (size_t)N * N;
  const int j0 = blockIdx.x * TW, i0 = blockIdx.y * TH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * 32 + tx;
  constexpr int PW = TW + 6, PH = TH + 6;
  constexpr int UW = TW + 4, UH = TH + 4;
  constexpr int SW = TW + 2, SH = TH + 2;
  float* sP = sm;
  float* sMx = sP + PH * PW;
  float* sMy = sMx + UH * UW;
  float* sUx = sMy + UH * UW;
  float* sUy = sUx + UH * UW;
  float* sLx = sUy + UH * UW;
  float* sLy = sLx + SH * SW;
  float* sF = sLy + SH * SW;   // fx for the SH rows of the lambda tile
  float* sDA = sF + SH;        // dfx/dA for the TH interior rows
  float* sDB = sDA + TH;       // dfx/dB
  double* sRed = reinterpret_cast<double*>(sDB + TH + ((TH & 1) ? 1 : 0));  // 3 x 8 doubles

  const float dt = c.dt;
  const float jscale = c.jscale;  // float32(dt * dx^2) = dJ/du_x / f_x
  const float nu = (a.theta_len == 3) ? __ldg(a.theta + 2) : c.nu;
  const float t = fmul((float)a.step, dt);
  const float A = __ldg(a.theta), B = __ldg(a.theta + 1);

  const bool has_lam = a.lam != nullptr;
  const bool has_p = a.p != nullptr;
  if (has_p) {
    const float* __restrict__ pp = a.p;
    forflat<PH, PW>(tid, [&](int r, int cc) {
      sP[r * PW + cc] = __ldg(pp + (size_t)((i0 - 3 + r) & M) * N + ((j0 - 3 + cc) & M));
    });
  }
  {
    const float* __restrict__ u = a.u;
    const float* __restrict__ lam = a.lam;
    forflat<UH, UW>(tid, [&](int r, int cc) {
      const size_t g = (size_t)((i0 - 2 + r) & M) * N + ((j0 - 2 + cc) & M);
      const int o = r * UW + cc;
      sUx[o] = __ldg(u + g);
      sUy[o] = __ldg(u + NN + g);
      sMx[o] = has_lam ? __ldg(lam + g) : 0.0f;
      sMy[o] = has_lam ? __ldg(lam + NN + g) : 0.0f;
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

  if (has_p) {  // mu = lambda - dt grad p
    forflat<UH, UW>(tid, [&](int r, int cc) {
      const int op = (r + 1) * PW + (cc + 1);
      const float px = fdiv(fsub(sP[op + PW], sP[op - PW]), c.h2);
      const float py = fdiv(fsub(sP[op + 1], sP[op - 1]), c.h2);
      const int o = r * UW + cc;
      sMx[o] = fsub(sMx[o], fmul(dt, px));
      sMy[o] = fsub(sMy[o], fmul(dt, py));
    });
    __syncthreads();
  }

  // theta sensitivities on the interior cells, accumulated in double: the
  // nu term is a small difference of large contributions
  double gA = 0.0, gB = 0.0, gN = 0.0;
  forflat<TH, TW>(tid, [&](int r, int cc) {
    const int o = (r + 2) * UW + (cc + 2);
    const float w = jscale * sUx[o] + dt * sMx[o];
    gA += (double)(w * sDA[r]);
    gB += (double)(w * sDB[r]);
    const float lux = (sUx[o - UW] + sUx[o + UW] + sUx[o + 1] + sUx[o - 1] - 4.0f * sUx[o]) / c.dx2;
    const float luy = (sUy[o - UW] + sUy[o + UW] + sUy[o + 1] + sUy[o - 1] - 4.0f * sUy[o]) / c.dx2;
    gN += (double)dt * ((double)sMx[o] * lux + (double)sMy[o] * luy);
  });

  // lambda_s on the tile + 1 halo
  const float inv_h2 = 1.0f / c.h2;
  const float inv_h1 = 1.0f / c.h1;
  forflat<SH, SW>(tid, [&](int r, int cc) {
    const int o = (r + 1) * UW + (cc + 1);
    const int n = o + UW, s = o - UW, e = o + 1, w = o - 1;  // i+1, i-1, j+1, j-1
    const float mx = sMx[o], my = sMy[o];
    const float lmx = (sMx[s] + sMx[n] + sMx[e] + sMx[w] - 4.0f * mx) / c.dx2;
    const float lmy = (sMy[s] + sMy[n] + sMy[e] + sMy[w] - 4.0f * my) / c.dx2;
    float atx, aty;
    if (SCHEME == NSGB_SCHEME_CENTRAL) {
      const float gxux = (sUx[n] - sUx[s]) * inv_h2, gxuy = (sUy[n] - sUy[s]) * inv_h2;
      const float gyux = (sUx[e] - sUx[w]) * inv_h2, gyuy = (sUy[e] - sUy[w]) * inv_h2;
      atx = -(mx * gxux + my * gxuy) + (sMx[n] * sUx[n] - sMx[s] * sUx[s]) * inv_h2 +
            (sMx[e] * sUy[e] - sMx[w] * sUy[w]) * inv_h2;
      aty = -(mx * gyux + my * gyuy) + (sMy[n] * sUx[n] - sMy[s] * sUx[s]) * inv_h2 +
            (sMy[e] * sUy[e] - sMy[w] * sUy[w]) * inv_h2;
    } else {
      const float uxo = sUx[o], uyo = sUy[o];
      const bool mxo = uxo >= 0.f, myo = uyo >= 0.f;
      // one-sided differences of u at o (the forward's dfx, dfy)
      const float dxux = (mxo ? uxo - sUx[s] : sUx[n] - uxo) * inv_h1;
      const float dxuy = (mxo ? uyo - sUy[s] : sUy[n] - uyo) * inv_h1;
      const float dyux = (myo ? uxo - sUx[w] : sUx[e] - uxo) * inv_h1;
      const float dyuy = (myo ? uyo - sUy[w] : sUy[e] - uyo) * inv_h1;
      atx = -(mx * dxux + my * dxuy);
      aty = -(mx * dyux + my * dyuy);
      // transposed one-sided operators applied to w = mu_c u_x (x) and mu_c u_y (y)
      const bool mxn = sUx[n] >= 0.f, mxs = sUx[s] >= 0.f;
      const bool mye = sUy[e] >= 0.f, myw = sUy[w] >= 0.f;
      auto dxt = [&](const float* mu) {
        return ((mxo ? mu[o] * uxo : -mu[o] * uxo) - (mxn ? mu[n] * sUx[n] : 0.f) +
                (mxs ? 0.f : mu[s] * sUx[s])) * inv_h1;
      };
      auto dyt = [&](const float* mu) {
        return ((myo ? mu[o] * uyo : -mu[o] * uyo) - (mye ? mu[e] * sUy[e] : 0.f) +
                (myw ? 0.f : mu[w] * sUy[w])) * inv_h1;
      };
      atx -= dxt(sMx) + dyt(sMx);
      aty -= dxt(sMy) + dyt(sMy);
    }
    sLx[r * SW + cc] = mx + dt * (nu * lmx + atx) + jscale * sF[r];
    sLy[r * SW + cc] = my + dt * (nu * lmy + aty);
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
      const float gx = fdiv(fsub(sLx[o + SW], sLx[o - SW]), c.h2);
      const float gy = fdiv(fsub(sLy[o + 1], sLy[o - 1]), c.h2);
      rhs[g] = fdiv(fadd(gx, gy), dt);
    });
  }

  gA = warp_sum_d(gA);
  gB = warp_sum_d(gB);
  gN = warp_sum_d(gN);
  if (tx == 0) {
    sRed[ty] = gA;
    sRed[8 + ty] = gB;
    sRed[16 + ty] = gN;
  }
  __syncthreads();
  if (ty == 0) {
    double v0 = (tx < 8) ? sRed[tx] : 0.0;
    double v1 = (tx < 8) ? sRed[8 + tx] : 0.0;
    double v2 = (tx < 8) ? sRed[16 + tx] : 0.0;
    v0 = warp_sum_d(v0);
    v1 = warp_sum_d(v1);
    v2 = warp_sum_d(v2);
    if (tx == 0) {
      const int nblk = gridDim.x * gridDim.y;
      double* gp = a.gpart + ((size_t)a.gslot * nblk + blockIdx.y * gridDim.x + blockIdx.x) * 3;
      gp[0] = v0;
      gp[1] = v1;
      gp[2] = v2;
    }
  }
}

static size_t adjoint_smem(int tw, int th) {
  // floats of the tiles and forcing rows, then 24 doubles (8-byte aligned)
  const size_t f = (size_t)(th + 6) * (tw + 6) + 4 * (size_t)(th + 4) * (tw + 4) +
                   2 * (size_t)(th + 2) * (tw + 2) + (th + 2) + 2 * th + 2;
  return f * sizeof(float) + 24 * sizeof(double) + 8;
}

template <int SCHEME, int TW, int TH>
static cudaError_t launch_adjoint_t(const AdjointArgs& a, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_adjoint<SCHEME, TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    configured = true;
  }
  const dim3 grid(a.c.N / TW, a.c.N / TH);
  k_adjoint<SCHEME, TW, TH><<<grid, dim3(32, 8), adjoint_smem(TW, TH), st>>>(a);
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

// Fixed-order reduction of nrows x nblk x 3 partials into gacc[3] (double).
__global__ void k_greduce(const double* __restrict__ gpart, int nblk, int nrows,
                          double* __restrict__ gacc) {
  __shared__ double red[3][256];
  for (int row = 0; row < nrows; ++row) {
    const double* base = gpart + (size_t)row * nblk * 3;
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
    if (threadIdx.x == 0) {
      gacc[0] += red[0][0];
      gacc[1] += red[1][0];
      gacc[2] += red[2][0];
    }
    __syncthreads();
  }
}

cudaError_t launch_greduce(const double* gpart, int nblk, int nrows, double* gacc, cudaStream_t st) {
  if (nrows > 0) k_greduce<<<1, 256, 0, st>>>(gpart, nblk, nrows, gacc);
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
