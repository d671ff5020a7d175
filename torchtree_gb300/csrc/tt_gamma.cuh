// Quantiles of the Gamma(shape a, rate 1) distribution and their derivative
// with respect to the shape, in FP64, on the host and the device.
//
// The discretised Gamma site model takes the category rates at the
// quantiles (2k+1)/(2K), divided by their mean (the same construction as
// torchtree's discretised Weibull model, site_model.py:173-195).  With the
// Gamma(a, rate a) distribution the quantile is x/a, where x solves
// P(a, x) = q for the regularised lower incomplete gamma function
//
//   P(a, x) = gamma(a, x) / Gamma(a),
//   gamma(a, x) = x^a e^-x S0,   S0 = sum_n x^n / (a (a+1) ... (a+n))
//
// (the power series of Abramowitz & Stegun 6.5.29; every term is positive).
// The root is found by Halley's method on f(x) = P(a, x) - q with
// f'(x) = x^(a-1) e^-x / Gamma(a) and f''/f' = (a-1)/x - 1, from the
// starting points of Numerical Recipes (Press et al., 3rd ed., section 6.2.1:
// Abramowitz & Stegun 26.2.23 with the Wilson-Hilferty transform for a > 1,
// the small-x power law for a <= 1).
//
// The shape derivative is analytic.  Differentiating the series term by term,
// d S0 / da = -S1 with S1 = sum_n T_n H_n, T_n = x^n / (a (a+1) ... (a+n))
// and H_n = sum_(j<=n) 1/(a+j), so
//
//   dP/da = x^a e^-x / Gamma(a) * (S0 (ln x - psi(a)) - S1),
//   dx/da = -(dP/da) / (dP/dx) = -x (S0 (ln x - psi(a)) - S1),
//
// with psi the digamma function (recurrence psi(a) = psi(a+1) - 1/a up to
// a >= 10, then the asymptotic series of Abramowitz & Stegun 6.3.18).
#pragma once

#include <math.h>

namespace tt {

#ifdef __CUDACC__
#define TT_HD __host__ __device__
#else
#define TT_HD
#endif

// digamma for a > 0
TT_HD inline double digamma_pos(double a) {
  double acc = 0.0;
  while (a < 10.0) {
    acc -= 1.0 / a;
    a += 1.0;
  }
  const double r = 1.0 / a, r2 = r * r;
  // ln a - 1/(2a) - sum_k B_2k / (2k a^2k), k = 1..6
  const double series =
      r2 * (1.0 / 12.0 - r2 * (1.0 / 120.0 - r2 * (1.0 / 252.0 - r2 * (1.0 / 240.0 - r2 * (1.0 / 132.0 -
                                                                                          r2 * (691.0 / 32760.0))))));
  return acc + log(a) - 0.5 * r - series;
}

// log(x^a e^-x / Gamma(a)).  For a >= 10 the large terms a ln x, x and
// ln Gamma(a) nearly cancel; with x = a (1 + t) and Stirling's series for
// ln Gamma (Abramowitz & Stegun 6.1.41) it is
//   ln(a / 2 pi) / 2 - c(a) + a (ln(1 + t) - t),
// c(a) = 1/(12a) - 1/(360a^3) + 1/(1260a^5) - 1/(1680a^7) + 1/(1188a^9) - ...
TT_HD inline double gamma_log_scale(double a, double x, double lga) {
  if (a < 10.0) return a * log(x) - x - lga;
  const double r = 1.0 / a, r2 = r * r;
  const double c = r * (1.0 / 12.0 - r2 * (1.0 / 360.0 - r2 * (1.0 / 1260.0 - r2 * (1.0 / 1680.0 -
                                                                                 r2 * (1.0 / 1188.0)))));
  const double t = (x - a) / a;
  return 0.5 * log(a / 6.283185307179586) - c + a * (log1p(t) - t);
}

// The series at (a, x), scaled to P: p = P(a, x) = sum_n p_n with
// p_n = scale T_n, z = sum_n p_n H_n = scale S1, and scale = x^a e^-x / Gamma(a)
// (the terms stay below 1, so nothing overflows for large a and x).
// False if the series did not converge.
TT_HD inline bool gamma_p_series(double a, double x, double lga, double &p, double &z, double &scale) {
  scale = exp(gamma_log_scale(a, x, lga));
  double term = scale / a, h = 1.0 / a;
  p = term;
  z = term * h;
  for (int n = 1; n < 200000; ++n) {
    term *= x / (a + n);
    h += 1.0 / (a + n);
    p += term;
    z += term * h;
    if (term <= p * 1e-17 && term * h <= z * 1e-17) return true;
  }
  return false;
}

// x with P(a, x) = q and dx/da; false for invalid input or no convergence
TT_HD inline bool gamma_quantile(double a, double q, double &x_out, double &dxda_out) {
  if (!(a > 0.0) || !(q > 0.0) || !(q < 1.0) || !isfinite(a)) return false;
  const double lga = lgamma(a);
  // starting point (Numerical Recipes 6.2.1)
  double x;
  if (a > 1.0) {
    const double pp = q < 0.5 ? q : 1.0 - q;
    const double t = sqrt(-2.0 * log(pp));
    double zq = (2.30753 + t * 0.27061) / (1.0 + t * (0.99229 + t * 0.04481)) - t;
    if (q < 0.5) zq = -zq;
    const double w = 1.0 - 1.0 / (9.0 * a) - zq / (3.0 * sqrt(a));
    x = fmax(1e-3, a * w * w * w);
  } else {
    const double t = 1.0 - a * (0.253 + a * 0.12);
    x = q < t ? pow(q / t, 1.0 / a) : 1.0 - log(1.0 - (q - t) / (1.0 - t));
  }
  double p = 0.0, z = 0.0, scale = 0.0, delta = 0.0;
  for (int it = 0; it < 100; ++it) {
    if (!(x > 0.0)) x = 1e-300;
    if (!gamma_p_series(a, x, lga, p, z, scale)) return false;
    const double dfdx = scale / x;  // x^(a-1) e^-x / Gamma(a)
    if (!(dfdx > 0.0) || !isfinite(dfdx)) return false;
    const double u = (p - q) / dfdx;
    const double step = u / (1.0 - 0.5 * fmin(1.0, u * ((a - 1.0) / x - 1.0)));
    double xn = x - step;
    if (xn <= 0.0) xn = 0.5 * x;
    delta = fabs(xn - x);
    x = xn;
    if (delta <= 4e-16 * x) break;
  }
  if (!(delta <= 1e-13 * x)) return false;
  if (!gamma_p_series(a, x, lga, p, z, scale)) return false;
  x_out = x;
  dxda_out = -x * (p * (log(x) - digamma_pos(a)) - z) / scale;
  return true;
}

}  // namespace tt
