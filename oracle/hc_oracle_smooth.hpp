// hc_oracle_smooth.hpp -- residual smoothing of the reference's legacy 1D path.
//
// TEST INFRASTRUCTURE ONLY (see hc_oracle.hpp).  Restates, in the order the reference
// writes it, OLD.fieldOperations/centralImplicitSmoothing.ipp:2-60 (centralImplicit-
// Smoothing: four weighted-Jacobi sweeps, omega 2/3, of (1 - beta delta^2) r1 = r0 with
// beta = (alpha^2 - 1)/4, the result times alpha) and centralExplicitSmoothing.ipp:5-39
// (centralExplicitSmoothing: r1 = r0 + gamma delta^2 r0 written as face differences,
// gamma = ((1 + 4 beta)/alpha - 1)/4).  The line's end treatment is the reference's
// GridControls1D::boundaryCondition character: 'p' periodic, 'a' one-neighbour
// normalisation, anything else unscaled ends.  The reference's own headers for these
// functions (array1D/array1D.h, types.h) are absent from its tree, so they are not
// compiled; the restatement is pinned by the closed-form Fourier amplification of both
// iterations on periodic sinusoids (tests/test_oracle_smooth.py).
#pragma once

#include <cstddef>
#include <vector>

namespace hco {

inline void smooth_implicit_1d(const double* r0, double* r1, size_t n, double alpha, char bc) {
  std::vector<double> wrk(r0, r0 + n), t(n);
  const double beta = 0.25 * (alpha * alpha - 1.);
  const double omega = 2. / 3.;
  for (int j = 0; j < 4; ++j) {
    for (size_t i = 0; i < n; ++i) t[i] = r0[i];
    for (size_t i = 0; i + 1 < n; ++i) {
      t[i] += beta * wrk[i + 1];
      t[i + 1] += beta * wrk[i];
    }
    for (size_t i = 1; i + 1 < n; ++i) t[i] *= 1. / (1. + 2. * beta);
    if (bc == 'p') {
      t[0] += beta * wrk[n - 1];
      t[n - 1] += beta * wrk[0];
      t[0] *= 1. / (1. + 2. * beta);
      t[n - 1] *= 1. / (1. + 2. * beta);
    } else if (bc == 'a') {
      t[0] *= 1. / (1. + 1. * beta);
      t[n - 1] *= 1. / (1. + 1. * beta);
    }
    for (size_t i = 0; i < n; ++i) wrk[i] = (1. - omega) * wrk[i] + omega * t[i];
  }
  for (size_t i = 0; i < n; ++i) r1[i] = wrk[i] * alpha;
}

inline void smooth_explicit_1d(const double* r0, double* r1, size_t n, double alpha, char bc) {
  const double beta = 0.25 * (alpha * alpha - 1.);
  const double gamma = 0.25 * ((1. + 4. * beta) / alpha - 1.);
  for (size_t i = 0; i < n; ++i) r1[i] = r0[i];
  for (size_t i = 1; i < n; ++i) {
    const double dr = gamma * (r0[i] - r0[i - 1]);
    r1[i - 1] -= dr;
    r1[i] += dr;
  }
  if (bc == 'p') {
    const double dr = gamma * (r0[0] - r0[n - 1]);
    r1[n - 1] -= dr;
    r1[0] += dr;
  }
}

}  // namespace hco
