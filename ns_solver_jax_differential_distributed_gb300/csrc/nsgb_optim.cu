// Optimiser updates of the parameter study (studies.py:864-934), on the
// device: the reference drives jit_gradient with optax 0.2.4's adam, sgd and
// rmsprop (studies.py:879-884) and applies the updates with
// optax.apply_updates (studies.py:900).  This kernel restates those published
// update rules in float32, in the library's evaluation order:
//   sgd:     u = g * (-lr)
//   adam:    m = (1-b1) g + b1 m;  v = (1-b2) g^2 + b2 v;
//            u = (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t) + eps_root) + eps) * (-lr)
//   rmsprop: v = (1-decay) g^2 + decay v;  u = g * rsqrt(v + eps) * (-lr)
//   theta = theta + u
// Each step runs as one tiny launch on the stream of the gradient it
// follows, so an optimisation loop never waits for the host.
#include "nsgb_internal.h"

namespace nsgb {

__global__ void k_optimizer_update(OptimizerRule r, float* __restrict__ theta,
                                   const float* __restrict__ grad, float* __restrict__ mu,
                                   float* __restrict__ nu, float* __restrict__ theta_copy, int n) {
  const int k = threadIdx.x;
  if (k >= n) return;
  const float g = gld(grad + k);
  float u;
  if (r.kind == NSGB_OPT_SGD) {
    u = __fmul_rn(g, -r.lr);
  } else if (r.kind == NSGB_OPT_ADAM) {
    const float m = __fadd_rn(__fmul_rn(r.one_minus_b1, g), __fmul_rn(r.b1, gld(mu + k)));
    const float v = __fadd_rn(__fmul_rn(r.one_minus_b2, __fmul_rn(g, g)), __fmul_rn(r.b2, gld(nu + k)));
    gst(mu + k, m);
    gst(nu + k, v);
    const float m_hat = __fdiv_rn(m, r.bc1);
    const float v_hat = __fdiv_rn(v, r.bc2);
    u = __fmul_rn(__fdiv_rn(m_hat, __fadd_rn(__fsqrt_rn(__fadd_rn(v_hat, r.eps_root)), r.eps)), -r.lr);
  } else {
    const float v = __fadd_rn(__fmul_rn(r.one_minus_decay, __fmul_rn(g, g)), __fmul_rn(r.decay, gld(nu + k)));
    gst(nu + k, v);
    u = __fmul_rn(__fmul_rn(g, rsqrtf(__fadd_rn(v, r.eps))), -r.lr);
  }
  const float t = __fadd_rn(gld(theta + k), u);
  gst(theta + k, t);
  if (theta_copy) gst(theta_copy + k, t);
}

cudaError_t launch_optimizer_update(const OptimizerRule& r, float* theta, const float* grad, float* mu,
                                    float* nu, float* theta_copy, int n, cudaStream_t st) {
  k_optimizer_update<<<1, 32, 0, st>>>(r, theta, grad, mu, nu, theta_copy, n);
  return cudaGetLastError();
}

NSGB_BOUNDS_UNIT(optim, 5)

}  // namespace nsgb
