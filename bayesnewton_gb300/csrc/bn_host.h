// Host-only helpers shared by the engine and the C-ABI unit: Gauss-Hermite rule
// and the Matern SDE blocks.
#pragma once
#include <algorithm>
#include <cmath>

#include "../../include/bnx.h"

namespace bn {

// Gauss-Hermite nodes/weights (physicists' Hermite, weight exp(-x^2)) by Newton
// iteration on the three-term recurrence with the standard asymptotic starting
// guesses (Golub-Welsch would give the same nodes).  Returned scaled as the
// reference uses them: x * sqrt(2), w / sqrt(pi) (bayesnewton/cubature.py:76-84).
inline void gauss_hermite(int n, double* x, double* w) {
  const double pim4 = 0.7511255444649425;  // pi^(-1/4)
  int m = (n + 1) / 2;
  double z = 0, z1, pp = 0;
  for (int i = 0; i < m; ++i) {
    if (i == 0) z = std::sqrt(double(2 * n + 1)) - 1.85575 * std::pow(double(2 * n + 1), -0.16667);
    else if (i == 1) z -= 1.14 * std::pow(double(n), 0.426) / z;
    else if (i == 2) z = 1.86 * z - 0.86 * x[0];
    else if (i == 3) z = 1.91 * z - 0.91 * x[1];
    else z = 2.0 * z - x[i - 2];
    for (int it = 0; it < 100; ++it) {
      double p1 = pim4, p2 = 0.0;
      for (int j = 0; j < n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = z * std::sqrt(2.0 / (j + 1)) * p2 - std::sqrt(double(j) / (j + 1)) * p3;
      }
      pp = std::sqrt(2.0 * n) * p2;
      z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) <= 1e-15) break;
    }
    x[i] = z;
    x[n - 1 - i] = -z;
    w[i] = 2.0 / (pp * pp);
    w[n - 1 - i] = w[i];
  }
  // ascending order as numpy.polynomial.hermite.hermgauss returns them
  for (int i = 0; i < n / 2; ++i) {
    std::swap(x[i], x[n - 1 - i]);
    std::swap(w[i], w[n - 1 - i]);
  }
  const double s2 = std::sqrt(2.0), ispi = 1.0 / std::sqrt(M_PI);
  for (int i = 0; i < n; ++i) {
    x[i] *= s2;
    w[i] *= ispi;
  }
}

inline bool matern_blocks(int kind, int size, double var, double ell, double* F, double* Pinf) {
  // F and Pinf of one Matern component (kernels.py:139-145, 191-200, 249-265, 319-338)
  for (int i = 0; i < size * size; ++i) F[i] = Pinf[i] = 0.0;
  if (kind == BN_KIND_MATERN12 && size == 1) {
    F[0] = -1.0 / ell;
    Pinf[0] = var;
  } else if (kind == BN_KIND_MATERN32 && size == 2) {
    const double lam = std::sqrt(3.0) / ell;
    F[1] = 1.0;
    F[2] = -lam * lam;
    F[3] = -2.0 * lam;
    Pinf[0] = var;
    Pinf[3] = 3.0 * var / (ell * ell);
  } else if (kind == BN_KIND_MATERN52 && size == 3) {
    const double lam = std::sqrt(5.0) / ell;
    F[1] = 1.0;
    F[5] = 1.0;
    F[6] = -lam * lam * lam;
    F[7] = -3.0 * lam * lam;
    F[8] = -3.0 * lam;
    const double kappa = 5.0 / 3.0 * var / (ell * ell);
    Pinf[0] = var;
    Pinf[2] = -kappa;
    Pinf[4] = kappa;
    Pinf[6] = -kappa;
    Pinf[8] = 25.0 * var / std::pow(ell, 4.0);
  } else if (kind == BN_KIND_MATERN72 && size == 4) {
    const double lam = std::sqrt(7.0) / ell;
    F[1] = F[6] = F[11] = 1.0;
    F[12] = -std::pow(lam, 4.0);
    F[13] = -4.0 * std::pow(lam, 3.0);
    F[14] = -6.0 * lam * lam;
    F[15] = -4.0 * lam;
    const double kappa = 7.0 / 5.0 * var / (ell * ell);
    const double kappa2 = 9.8 * var / std::pow(ell, 4.0);
    Pinf[0] = var;
    Pinf[2] = -kappa;
    Pinf[5] = kappa;
    Pinf[7] = -kappa2;
    Pinf[8] = -kappa;
    Pinf[10] = kappa2;
    Pinf[13] = -kappa2;
    Pinf[15] = 343.0 * var / std::pow(ell, 6.0);
  } else {
    return false;
  }
  return true;
}

inline double matern_lam(int kind, double ell) {
  switch (kind) {
    case BN_KIND_MATERN12: return 1.0 / ell;
    case BN_KIND_MATERN32: return std::sqrt(3.0) / ell;
    case BN_KIND_MATERN52: return std::sqrt(5.0) / ell;
    case BN_KIND_MATERN72: return std::sqrt(7.0) / ell;
    default: return 0.0;
  }
}

}  // namespace bn
