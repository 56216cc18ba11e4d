// wotg_coef.cuh — per-epsilon coefficients of the Sinkhorn updates, shared by
// the single-problem driver (host) and the batched driver (device).
#pragma once

#include <math.h>
#include <stdint.h>

namespace wotg {

struct Coef {
  double eps, inv_eps;
  double alpha1, alpha2;
  double inv_l1e, inv_l2e;  // 1/(lambda + eps)
  double lambda1, lambda2;
  double logI, logJ, logq, q;
  double kappa;             // cost_scale / eps
  float kappa2;             // cost_scale / eps * log2(e), rounded towards zero
  float kappa2_lo;          // the remainder (> 0), so kappa2 + kappa2_lo carries ~48 bits
  // log(tau) -/+ 1e-9: the absorption test max exp(la) > tau is decided from la
  // alone outside this band (set by the single-problem driver; by default the
  // band is the whole line, i.e. exp is always formed)
  double ltau_lo, ltau_hi;
};

// The reference's exponents alpha1 = lambda1 / (lambda1 + eps) and
// alpha2 = lambda2 / (lambda2 + eps) (optimal_transport.py:119-121 / :201-203)
// and the constants the log-domain updates need.
__host__ __device__ inline Coef make_coef(double eps, double lambda1, double lambda2, double cost_scale, int64_t I,
                                          int64_t J, double q) {
  Coef c;
  c.eps = eps;
  c.inv_eps = 1.0 / eps;
  c.alpha1 = lambda1 / (lambda1 + eps);
  c.alpha2 = lambda2 / (lambda2 + eps);
  c.inv_l1e = 1.0 / (lambda1 + eps);
  c.inv_l2e = 1.0 / (lambda2 + eps);
  c.lambda1 = lambda1;
  c.lambda2 = lambda2;
  c.logI = log((double)I);
  c.logJ = log((double)J);
  c.q = q;
  c.logq = log(q);
  c.kappa = cost_scale / eps;
  // kappa2 = hi + lo with lo > 0: hi the FP32 value at or below the FP64 one, lo
  // the FP32 remainder (a tiny positive value when hi is exact), so that
  // -hi * inf - lo * inf of a +inf padding cost entry is -inf, never NaN
  const double k2 = cost_scale / eps * 1.4426950408889634074;
  float hi = (float)k2;
  if ((double)hi > k2) hi = nextafterf(hi, 0.f);
  float lo = (float)(k2 - (double)hi);
  if (!(lo > 0.f)) lo = 1e-30f;
  c.kappa2 = hi;
  c.kappa2_lo = lo;
  c.ltau_lo = -INFINITY;
  c.ltau_hi = INFINITY;
  return c;
}

}  // namespace wotg
