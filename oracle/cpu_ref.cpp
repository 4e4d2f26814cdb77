// oracle/cpu_ref.cpp -- TEST INFRASTRUCTURE: a float64 C++ restatement of the
// reference's sequential Markov-GP inference step, used (1) as the oracle for
// GPU parity at sizes the numpy oracle is too slow for and (2) as the timed CPU
// baseline of bench.py (kind "port").  Nothing in the product links it.
//
// One step = the VI site update from the expectations at the current posterior
// (inference.py:21-39, 65-90, 170-195), the sequential Kalman filter with its log
// marginal (ops.py:154-180, utils.py:376-396), the sequential RTS smoother on the
// shifted dt (ops.py:288-311, basemodels.py:689-706), then the site expectations
// and energy at the new posterior (inference.py:197-222, basemodels.py:708-741).
// The filter / smoother recursions run on one thread, as jax.lax.scan does on a
// CPU; the per-site expectations run on `threads` OpenMP threads (the reference
// vmaps them).
//
// Priors: Sum / Independent stacks of Matern12/32/52/72 (kernels.py:123-382,
// 1499-1663).  Likelihoods: Gaussian (closed form), Bernoulli logit / probit
// (20-point GH, score form of cubature.py:198-246), Poisson exp (closed form),
// heteroscedastic exp / softplus (2-D GH, likelihoods.py:613-664).
#include <omp.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr double kLog2Pi = 1.8378770664093453;
constexpr int MAXD = 8;

struct Prior {
  int nc, combine, D, P;
  int kind[8], size[8], off[8];
  double var[8], ell[8];
  double Pinf[MAXD][MAXD];
  double H[2][MAXD];
};

struct Lik {
  int kind, ncub;
  double variance;
  double x[32], w[32];
};

void hermgauss_scaled(int n, double* x, double* w) {
  // Newton iteration on the orthonormal Hermite recurrence (as the library does)
  const double pim4 = 0.7511255444649425;
  int m = (n + 1) / 2;
  double z = 0, z1, pp = 0;
  std::vector<double> xx(n), ww(n);
  for (int i = 0; i < m; ++i) {
    if (i == 0) z = std::sqrt(double(2 * n + 1)) - 1.85575 * std::pow(double(2 * n + 1), -0.16667);
    else if (i == 1) z -= 1.14 * std::pow(double(n), 0.426) / z;
    else if (i == 2) z = 1.86 * z - 0.86 * xx[0];
    else if (i == 3) z = 1.91 * z - 0.91 * xx[1];
    else z = 2.0 * z - xx[i - 2];
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
    xx[i] = z;
    xx[n - 1 - i] = -z;
    ww[i] = 2.0 / (pp * pp);
    ww[n - 1 - i] = ww[i];
  }
  for (int i = 0; i < n; ++i) {
    x[i] = std::sqrt(2.0) * xx[n - 1 - i];
    w[i] = ww[n - 1 - i] / std::sqrt(M_PI);
  }
}

void transition(const Prior& pr, double dt, double A[MAXD][MAXD]) {
  for (int i = 0; i < pr.D; ++i)
    for (int j = 0; j < pr.D; ++j) A[i][j] = 0.0;
  for (int c = 0; c < pr.nc; ++c) {
    const int o = pr.off[c];
    const double ell = pr.ell[c];
    if (pr.kind[c] == 1) {
      A[o][o] = std::exp(-dt / ell);
    } else if (pr.kind[c] == 2) {
      const double lam = std::sqrt(3.0) / ell, e = std::exp(-dt * lam);
      A[o][o] = e * (dt * lam + 1.0);
      A[o][o + 1] = e * dt;
      A[o + 1][o] = -e * dt * lam * lam;
      A[o + 1][o + 1] = e * (1.0 - dt * lam);
    } else if (pr.kind[c] == 3) {
      const double lam = std::sqrt(5.0) / ell, tl = dt * lam, e = std::exp(-tl);
      const double M[3][3] = {{lam * (0.5 * tl + 1.0), tl + 1.0, 0.5 * dt},
                              {-0.5 * tl * lam * lam, lam * (1.0 - tl), 1.0 - 0.5 * tl},
                              {lam * lam * lam * (0.5 * tl - 1.0), lam * lam * (tl - 3), lam * (0.5 * tl - 2.0)}};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[o + i][o + j] = e * (dt * M[i][j] + (i == j));
    } else {
      const double lam = std::sqrt(7.0) / ell, l2 = lam * lam, l3 = l2 * lam, tl = dt * lam, tl2 = tl * tl;
      const double e = std::exp(-tl);
      const double M[4][4] = {
          {lam * (1.0 + 0.5 * tl + tl2 / 6.0), 1.0 + tl + 0.5 * tl2, 0.5 * dt * (1.0 + tl), dt * dt / 6},
          {-tl2 * l2 / 6.0, lam * (1.0 + 0.5 * tl - 0.5 * tl2), 1.0 + tl - 0.5 * tl2, dt * (0.5 - tl / 6.0)},
          {l3 * tl * (tl / 6.0 - 0.5), tl * l2 * (0.5 * tl - 2.0), lam * (1.0 - 2.5 * tl + 0.5 * tl2),
           1.0 - tl + tl2 / 6.0},
          {l2 * l2 * (tl - 1.0 - tl2 / 6.0), l3 * (3.5 * tl - 4.0 - 0.5 * tl2), l2 * (4.0 * tl - 6.0 - 0.5 * tl2),
           lam * (1.5 * tl - 3.0 - tl2 / 6.0)}};
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) A[o + i][o + j] = e * (dt * M[i][j] + (i == j));
    }
  }
}

bool chol(int n, double M[MAXD][MAXD], double L[MAXD][MAXD]) {
  for (int j = 0; j < n; ++j) {
    double s = M[j][j];
    for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
    if (!(s > 0)) return false;
    L[j][j] = std::sqrt(s);
    for (int i = j + 1; i < n; ++i) {
      double t = M[i][j];
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / L[j][j];
    }
    for (int i = 0; i < j; ++i) L[i][j] = 0.0;
  }
  return true;
}

// X <- M^-1 X (ncol columns) given the Cholesky factor of M
void chol_solve(int n, const double L[MAXD][MAXD], double X[MAXD][MAXD], int ncol) {
  for (int c = 0; c < ncol; ++c) {
    for (int i = 0; i < n; ++i) {
      double t = X[i][c];
      for (int k = 0; k < i; ++k) t -= L[i][k] * X[k][c];
      X[i][c] = t / L[i][i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double t = X[i][c];
      for (int k = i + 1; k < n; ++k) t -= L[k][i] * X[k][c];
      X[i][c] = t / L[i][i];
    }
  }
}

inline double sp(double z) { return std::max(z, 0.0) + std::log1p(std::exp(-std::fabs(z))); }

double loglik1(const Lik& lk, double y, double f) {
  if (lk.kind == 1) return -0.5 * std::log(2 * M_PI * lk.variance) - 0.5 * (y - f) * (y - f) / lk.variance;
  if (lk.kind == 2) return y == 1.0 ? -sp(-f) : -sp(f);
  if (lk.kind == 3) {
    const double j = 1e-3, p = 0.5 * std::erfc(-(y == 1.0 ? f : -f) / std::sqrt(2.0)) * (1 - 2 * j) + j;
    return std::log(p);
  }
  const double mu = std::exp(f);
  return y * f - mu - std::lgamma(y + 1.0);
}

// VE of one scalar site -> E, dE, d2E (closed forms or score-form GH)
void ve1(const Lik& lk, double y, double m, double v, double& E, double& g, double& h) {
  if (lk.kind == 1) {
    E = -0.5 * std::log(2 * M_PI) - 0.5 * std::log(lk.variance) - 0.5 * ((y - m) * (y - m) + v) / lk.variance;
    g = (y - m) / lk.variance;
    h = -1.0 / lk.variance;
    return;
  }
  if (lk.kind == 4) {
    const double emc = std::exp(m + v / 2);
    E = y * m - emc - std::lgamma(y + 1.0);
    g = y - emc;
    h = -emc;
    return;
  }
  const double sv = std::sqrt(v);
  double e = 0, a = 0, b = 0;
  for (int i = 0; i < lk.ncub; ++i) {
    const double wl = lk.w[i] * loglik1(lk, y, sv * lk.x[i] + m);
    e += wl;
    a += wl * lk.x[i];
    b += wl * (lk.x[i] * lk.x[i] - 1.0);
  }
  E = e;
  g = a / sv;
  h = b / v;
}

void hetero_point(int kind, double y, double f1, double f2, double& l, double g[2], double h[3]) {
  double s, ds, d2s;
  if (kind == 5) {
    s = ds = d2s = std::exp(f2);
  } else {
    s = sp(f2);
    ds = 1.0 / (1.0 + std::exp(-f2));
    d2s = ds * (1 - ds);
  }
  const double r = y - f1, is2 = 1.0 / (s * s);
  l = -0.5 * std::log(2 * M_PI * s * s) - 0.5 * r * r * is2;
  g[0] = r * is2;
  g[1] = -ds / s + r * r * ds / (s * s * s);
  h[0] = -is2;
  h[1] = -2.0 * r * ds / (s * s * s);
  h[2] = -(d2s * s - ds * ds) * is2 + r * r * (d2s / (s * s * s) - 3.0 * ds * ds * is2 * is2);
}

void ve2(const Lik& lk, double y, const double m[2], const double V[3], double& E, double g[2], double H[3]) {
  const double L11 = std::sqrt(V[0]), L21 = V[1] / L11, L22 = std::sqrt(std::max(V[2] - L21 * L21, 0.0));
  E = 0;
  g[0] = g[1] = H[0] = H[1] = H[2] = 0;
  for (int i = 0; i < lk.ncub; ++i)
    for (int j = 0; j < lk.ncub; ++j) {
      const double w = lk.w[i] * lk.w[j];
      double l, gg[2], hh[3];
      hetero_point(lk.kind, y, L11 * lk.x[i] + m[0], L21 * lk.x[i] + L22 * lk.x[j] + m[1], l, gg, hh);
      E += w * l;
      g[0] += w * gg[0];
      g[1] += w * gg[1];
      H[0] += w * hh[0];
      H[1] += w * hh[1];
      H[2] += w * hh[2];
    }
}

}  // namespace

extern "C" {

// prior: nc components (kind 1..4 = Matern12..72, size = kind), combine 0 = Sum,
// 1 = Independent; lik kind: 1 Gaussian, 2 logit, 3 probit, 4 Poisson, 5/6
// heteroscedastic exp / softplus.  Arrays as in include/bnx.h (float64):
// dt [N], y [N], nat1 [N,P], nat2 [N,P,P], pm [N,P], pv [N,P,P], grad [N,P],
// hess [N,P,P], lin [N,P].  newton = 1 performs the site update first (from
// grad/hess/lin), 0 only recomputes the posterior.  result: energy, log marginal,
// sum1, sum2.  Returns 0, or -1 on bad arguments.
int cpuref_step(int64_t N, int nc, int combine, const int* kind, const double* var, const double* ell, int lik_kind,
                double lik_var, int ncub, int newton, double lr, const double* dt, const double* y, double* nat1,
                double* nat2, double* pm, double* pv, double* grad, double* hess, double* lin, int threads,
                double* result) {
  Prior pr;
  std::memset(&pr, 0, sizeof(pr));
  if (nc < 1 || nc > 8 || N < 1) return -1;
  pr.nc = nc;
  pr.combine = combine;
  int off = 0;
  for (int c = 0; c < nc; ++c) {
    if (kind[c] < 1 || kind[c] > 4) return -1;
    pr.kind[c] = kind[c];
    pr.size[c] = kind[c];
    pr.off[c] = off;
    pr.var[c] = var[c];
    pr.ell[c] = ell[c];
    const double v = var[c], l = ell[c];
    double (*Pi)[MAXD] = pr.Pinf;
    const int o = off;
    if (kind[c] == 1) {
      Pi[o][o] = v;
    } else if (kind[c] == 2) {
      Pi[o][o] = v;
      Pi[o + 1][o + 1] = 3.0 * v / (l * l);
    } else if (kind[c] == 3) {
      const double k = 5.0 / 3.0 * v / (l * l);
      Pi[o][o] = v;
      Pi[o][o + 2] = Pi[o + 2][o] = -k;
      Pi[o + 1][o + 1] = k;
      Pi[o + 2][o + 2] = 25.0 * v / std::pow(l, 4.0);
    } else {
      const double k = 7.0 / 5.0 * v / (l * l), k2 = 9.8 * v / std::pow(l, 4.0);
      Pi[o][o] = v;
      Pi[o][o + 2] = Pi[o + 2][o] = -k;
      Pi[o + 1][o + 1] = k;
      Pi[o + 1][o + 3] = Pi[o + 3][o + 1] = -k2;
      Pi[o + 2][o + 2] = k2;
      Pi[o + 3][o + 3] = 343.0 * v / std::pow(l, 6.0);
    }
    off += kind[c];
  }
  if (off > MAXD) return -1;
  pr.D = off;
  pr.P = combine ? nc : 1;
  if (pr.P > 2) return -1;
  for (int c = 0; c < nc; ++c) pr.H[combine ? c : 0][pr.off[c]] = 1.0;
  const int D = pr.D, P = pr.P;
  Lik lk;
  lk.kind = lik_kind;
  lk.variance = lik_var;
  lk.ncub = ncub > 0 ? ncub : 20;
  hermgauss_scaled(lk.ncub, lk.x, lk.w);
  if (threads > 0) omp_set_num_threads(threads);

  // 1. site update (newton_update + damping, inference.py:21-39, 83-86)
  if (newton) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < N; ++k) {
      for (int p = 0; p < P; ++p) {
        double hm = 0.0;
        double hrow[2];
        for (int q = 0; q < P; ++q) {
          const double hv = hess[(k * P + p) * P + q];
          hrow[q] = std::isnan(hv) ? -1e-6 : hv;
          hm += hrow[q] * lin[k * P + q];
        }
        const double gp = std::isnan(grad[k * P + p]) ? hm : grad[k * P + p];
        nat1[k * P + p] = (1 - lr) * nat1[k * P + p] + lr * (gp - hm);
        for (int q = 0; q < P; ++q) nat2[(k * P + p) * P + q] = (1 - lr) * nat2[(k * P + p) * P + q] + lr * (-hrow[q]);
      }
    }
  }
  // site mean / covariance
  std::vector<double> sy(N * P), sR(N * P * P);
  for (int64_t k = 0; k < N; ++k) {
    if (P == 1) {
      sR[k] = 1.0 / nat2[k];
      sy[k] = nat1[k] * sR[k];
    } else {
      const double* n2 = nat2 + k * 4;
      const double det = n2[0] * n2[3] - n2[1] * n2[2];
      sR[k * 4 + 0] = n2[3] / det;
      sR[k * 4 + 3] = n2[0] / det;
      sR[k * 4 + 1] = -n2[1] / det;
      sR[k * 4 + 2] = -n2[2] / det;
      sy[k * 2 + 0] = sR[k * 4 + 0] * nat1[k * 2] + sR[k * 4 + 1] * nat1[k * 2 + 1];
      sy[k * 2 + 1] = sR[k * 4 + 2] * nat1[k * 2] + sR[k * 4 + 3] * nat1[k * 2 + 1];
    }
  }
  // 2. sequential Kalman filter (ops.py:154-180)
  std::vector<double> fm(N * D), fP(N * D * D);
  double m[MAXD] = {0}, Pm[MAXD][MAXD];
  std::memcpy(Pm, pr.Pinf, sizeof(Pm));
  double ll = 0.0;
  double A[MAXD][MAXD], X[MAXD][MAXD], Pp[MAXD][MAXD], mp[MAXD];
  for (int64_t k = 0; k < N; ++k) {
    transition(pr, k == 0 ? 0.0 : dt[k], A);
    if (k == 0)
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) A[i][j] = (i == j);
    for (int i = 0; i < D; ++i) {
      mp[i] = 0;
      for (int j = 0; j < D; ++j) mp[i] += A[i][j] * m[j];
    }
    // Pp = A (P - Pinf) A^T + Pinf
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        double t = 0;
        for (int q = 0; q < D; ++q) t += A[i][q] * (Pm[q][j] - pr.Pinf[q][j]);
        X[i][j] = t;
      }
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        double t = pr.Pinf[i][j];
        for (int q = 0; q < D; ++q) t += X[i][q] * A[j][q];
        Pp[i][j] = t;
      }
    double HP[2][MAXD], S[2][2], r[2], Si[2][2];
    for (int p = 0; p < P; ++p) {
      double hm = 0;
      for (int j = 0; j < D; ++j) {
        double t = 0;
        for (int i = 0; i < D; ++i) t += pr.H[p][i] * Pp[i][j];
        HP[p][j] = t;
        hm += pr.H[p][j] * mp[j];
      }
      r[p] = sy[k * P + p] - hm;
    }
    for (int p = 0; p < P; ++p)
      for (int q = 0; q < P; ++q) {
        double t = sR[(k * P + p) * P + q];
        for (int j = 0; j < D; ++j) t += HP[p][j] * pr.H[q][j];
        S[p][q] = t;
      }
    double ldet;
    if (P == 1) {
      Si[0][0] = 1.0 / S[0][0];
      ldet = std::log(S[0][0]);
    } else {
      const double det = S[0][0] * S[1][1] - S[0][1] * S[1][0];
      Si[0][0] = S[1][1] / det;
      Si[1][1] = S[0][0] / det;
      Si[0][1] = -S[0][1] / det;
      Si[1][0] = -S[1][0] / det;
      ldet = std::log(det);
    }
    // masked log marginal: missing observations (NaN y) contribute 0 (single latent)
    const bool masked = (P == 1) && std::isnan(y[k]);
    if (!masked) {
      double q = 0;
      for (int p = 0; p < P; ++p)
        for (int qq = 0; qq < P; ++qq) q += r[p] * Si[p][qq] * r[qq];
      ll += -0.5 * (q + P * kLog2Pi + ldet);
    }
    double SiHP[2][MAXD];
    for (int p = 0; p < P; ++p)
      for (int j = 0; j < D; ++j) {
        double t = 0;
        for (int q = 0; q < P; ++q) t += Si[p][q] * HP[q][j];
        SiHP[p][j] = t;
      }
    for (int i = 0; i < D; ++i) {
      double t = mp[i];
      for (int p = 0; p < P; ++p) {
        double sr = 0;
        for (int q = 0; q < P; ++q) sr += Si[p][q] * r[q];
        t += HP[p][i] * sr;
      }
      m[i] = t;
      for (int j = 0; j < D; ++j) {
        double u = Pp[i][j];
        for (int p = 0; p < P; ++p) u -= HP[p][i] * SiHP[p][j];
        Pm[i][j] = u;
      }
    }
    for (int i = 0; i < D; ++i) {
      fm[k * D + i] = m[i];
      for (int j = 0; j < D; ++j) fP[(k * D + i) * D + j] = Pm[i][j];
    }
  }
  // 3. sequential RTS smoother on the shifted dt (ops.py:288-311)
  double sm[MAXD], sP[MAXD][MAXD];
  for (int i = 0; i < D; ++i) {
    sm[i] = fm[(N - 1) * D + i];
    for (int j = 0; j < D; ++j) sP[i][j] = fP[((N - 1) * D + i) * D + j];
  }
  for (int64_t k = N - 1; k >= 0; --k) {
    double Fm[MAXD], FP[MAXD][MAXD];
    for (int i = 0; i < D; ++i) {
      Fm[i] = fm[k * D + i];
      for (int j = 0; j < D; ++j) FP[i][j] = fP[(k * D + i) * D + j];
    }
    if (k < N - 1) {
      transition(pr, dt[k + 1], A);
      double AF[MAXD][MAXD], L[MAXD][MAXD], Gt[MAXD][MAXD];
      for (int i = 0; i < D; ++i) {
        mp[i] = 0;
        for (int j = 0; j < D; ++j) {
          mp[i] += A[i][j] * Fm[j];
          double t = 0;
          for (int q = 0; q < D; ++q) t += A[i][q] * FP[q][j];
          AF[i][j] = t;
        }
      }
      // Pp = A fP A^T + Q,  Q = Pinf - A Pinf A^T  (ops.py:149-151, 294-296)
      double APi[MAXD][MAXD];
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          double t = 0;
          for (int q = 0; q < D; ++q) t += A[i][q] * pr.Pinf[q][j];
          APi[i][j] = AF[i][j] - t;
        }
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          double t = pr.Pinf[i][j];
          for (int q = 0; q < D; ++q) t += APi[i][q] * A[j][q];
          Pp[i][j] = t;
        }
      chol(D, Pp, L);
      std::memcpy(Gt, AF, sizeof(Gt));
      chol_solve(D, L, Gt, D);  // Gt = Pp^-1 A fP = G^T
      double dm[MAXD], Dp[MAXD][MAXD], nm[MAXD], nP[MAXD][MAXD];
      for (int i = 0; i < D; ++i) {
        dm[i] = sm[i] - mp[i];
        for (int j = 0; j < D; ++j) Dp[i][j] = sP[i][j] - Pp[i][j];
      }
      for (int i = 0; i < D; ++i) {
        double t = Fm[i];
        for (int j = 0; j < D; ++j) t += Gt[j][i] * dm[j];
        nm[i] = t;
      }
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          double t = 0;
          for (int q = 0; q < D; ++q) t += Gt[q][i] * Dp[q][j];
          X[i][j] = t;
        }
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          double t = FP[i][j];
          for (int q = 0; q < D; ++q) t += X[i][q] * Gt[q][j];
          nP[i][j] = t;
        }
      std::memcpy(sm, nm, sizeof(sm));
      std::memcpy(sP, nP, sizeof(sP));
    }
    for (int p = 0; p < P; ++p) {
      double t = 0;
      for (int j = 0; j < D; ++j) t += pr.H[p][j] * sm[j];
      pm[k * P + p] = t;
      for (int q = 0; q < P; ++q) {
        double u = 0;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) u += pr.H[p][i] * sP[i][j] * pr.H[q][j];
        pv[(k * P + p) * P + q] = u;
      }
    }
  }
  // 4. site expectations at the new posterior and the energy terms
  double s1 = 0.0, s2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s1, s2)
  for (int64_t k = 0; k < N; ++k) {
    if (P == 1) {
      const bool masked = std::isnan(y[k]);
      double E, g, h;
      ve1(lk, masked ? pm[k] : y[k], pm[k], pv[k], E, g, h);
      if (masked) {
        g = h = NAN;
      } else {
        s1 += E;
        const double r = sy[k] - pm[k];
        s2 += -0.5 * std::log(2 * M_PI * sR[k]) - 0.5 * (r * r + pv[k]) / sR[k];
      }
      grad[k] = g;
      hess[k] = (-h < 0) ? -1e-2 : h;
      lin[k] = pm[k];
    } else {
      double E, g[2], H[3];
      const double mm[2] = {pm[k * 2], pm[k * 2 + 1]};
      const double V[3] = {pv[k * 4], 0.5 * (pv[k * 4 + 1] + pv[k * 4 + 2]), pv[k * 4 + 3]};
      ve2(lk, y[k], mm, V, E, g, H);
      s1 += E;
      const double* R = &sR[k * 4];
      const double det = R[0] * R[3] - R[1] * R[2];
      const double Si[4] = {R[3] / det, -R[1] / det, -R[2] / det, R[0] / det};
      const double r0 = sy[k * 2] - mm[0], r1 = sy[k * 2 + 1] - mm[1];
      const double q = r0 * (Si[0] * r0 + Si[1] * r1) + r1 * (Si[2] * r0 + Si[3] * r1);
      const double tr = Si[0] * pv[k * 4] + Si[1] * pv[k * 4 + 2] + Si[2] * pv[k * 4 + 1] + Si[3] * pv[k * 4 + 3];
      s2 += -0.5 * (q + 2 * kLog2Pi + std::log(det)) - 0.5 * tr;
      grad[k * 2] = g[0];
      grad[k * 2 + 1] = g[1];
      hess[k * 4] = (-H[0] < 0) ? -1e-2 : H[0];
      hess[k * 4 + 1] = hess[k * 4 + 2] = 0.0;
      hess[k * 4 + 3] = (-H[2] < 0) ? -1e-2 : H[2];
      lin[k * 2] = mm[0];
      lin[k * 2 + 1] = mm[1];
    }
  }
  result[0] = -(s1 - (s2 - ll));
  result[1] = ll;
  result[2] = s1;
  result[3] = s2;
  return 0;
}

int cpuref_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
