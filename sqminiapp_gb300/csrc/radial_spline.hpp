// radial_spline.hpp -- cubic spline of radial pseudopotential tables.
//
// End conditions and arithmetic of the reference (getYD_gen / tridiag_gen / SplineEvaluate,
// src/lsdft_tools.cc:15-151): the not-a-knot spline, with the per-interval cubic
// coefficients precomputed once and the interval found by binary search.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <vector>

namespace sq {

// Cubic spline with the reference's end conditions, coefficients precomputed per interval.
class RadialSpline {
 public:
  RadialSpline() = default;
  RadialSpline(const std::vector<double> &x, const std::vector<double> &y) : x_(x) {
    const int n = (int)x.size();
    if (n < 3) throw std::runtime_error("spline needs >= 3 points");
    std::vector<double> A(n), B(n), C(n), D(n);
    double h0 = x[1] - x[0], h1 = x[2] - x[1];
    double r0 = (y[1] - y[0]) / h0, r1 = (y[2] - y[1]) / h1;
    B[0] = h1 * (h0 + h1);
    C[0] = (h0 + h1) * (h0 + h1);
    D[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
    int i = 1;
    for (; i < n - 1; i++) {
      h0 = x[i] - x[i - 1];
      h1 = x[i + 1] - x[i];
      r0 = (y[i] - y[i - 1]) / h0;
      r1 = (y[i + 1] - y[i]) / h1;
      A[i] = h1;
      B[i] = 2 * (h0 + h1);
      C[i] = h0;
      D[i] = 3 * (r0 * h1 + r1 * h0);
    }
    A[i] = (h0 + h1) * (h0 + h1);
    B[i] = h0 * (h0 + h1);
    D[i] = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
    // Gaussian elimination of the tridiagonal system for the derivatives
    std::vector<double> F(n);
    double b = B[0];
    D[0] /= b;
    for (int k = 1; k < n; k++) {
      F[k] = C[k - 1] / b;
      b = B[k] - A[k] * F[k];
      if (b == 0) throw std::runtime_error("singular spline system");
      D[k] = (D[k] - D[k - 1] * A[k]) / b;
    }
    for (int k = n - 2; k >= 0; k--) D[k] -= D[k + 1] * F[k + 1];
    coef_.resize(4 * (size_t)(n - 1));
    for (int k = 0; k < n - 1; k++) {
      double dx = 1.0 / (x[k + 1] - x[k]);
      double dy = (y[k + 1] - y[k]) * dx;
      coef_[4 * k + 0] = y[k];
      coef_[4 * k + 1] = D[k];
      coef_[4 * k + 2] = dx * (3.0 * dy - 2.0 * D[k] - D[k + 1]);
      coef_[4 * k + 3] = dx * dx * (-2.0 * dy + D[k] + D[k + 1]);
    }
  }
  // interval: largest k with x[k] <= p (k = n-2 at the right end)
  int interval(double p) const {
    if (p < x_.front() || p > x_.back()) throw std::runtime_error("radius outside the psd grid");
    int k = (int)(std::upper_bound(x_.begin(), x_.end(), p) - x_.begin()) - 1;
    return std::min(k, (int)x_.size() - 2);
  }
  double eval_in(int k, double p) const {
    const double *c = &coef_[4 * (size_t)k];
    double t = p - x_[k];
    return ((c[3] * t + c[2]) * t + c[1]) * t + c[0];
  }
  double operator()(double p) const { return eval_in(interval(p), p); }
  const std::vector<double> &knots() const { return x_; }

 private:
  std::vector<double> x_, coef_;
};


}  // namespace sq
