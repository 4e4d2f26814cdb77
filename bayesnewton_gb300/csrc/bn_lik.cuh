// Per-site likelihood arithmetic on the device.
//
// Single-latent sites (P = 1):
//   Gaussian      closed-form VE and moment match (bayesnewton/likelihoods.py:727-780)
//   Poisson(exp)  closed-form VE (likelihoods.py:979-1008), GH moment match
//   Bernoulli     logit or probit link (likelihoods.py:806-860), GH cubature.
//                 The expected log density E = sum_i w_i log p(y | sqrt(v) x_i + m)
//                 is the reference's (cubature.py:198-246).  Its mean derivatives
//                 are the reference's score-function sums when score_form is set,
//                 else sum_i w_i d/df log p and sum_i w_i d2/df2 log p at the same
//                 nodes: the expectations of the derivatives, equal to the score
//                 sums for the exact integral and within ~1e-6 of them under the
//                 20-point rule for the logit link, without the score form's float32
//                 cancellation (~eps |log p| / v for a small posterior variance v).
//                 The probit link, whose jitter makes log p non-smooth so that the
//                 two 20-point sums differ by up to 1e-2, and float64 runs use the
//                 score form (chosen by the host).
// Two-latent sites (P = 2): HeteroscedasticNoise, N(y | f1, link(f2)^2), 2-D GH with
//   the per-node gradient and Hessian of log p (likelihoods.py:613-664, 1244-1281).
//
// Log densities of the Bernoulli link use log sigma(f) = -softplus(-f) and
// log(1 - sigma(f)) = -softplus(f), the same values as the reference's
// log(where(y == 1, sigma, 1 - sigma)) without its cancellation for large |f|.
#pragma once
#include "bn_small.cuh"
#include "../../include/bnx.h"

namespace bn {

template <typename T>
struct LikParams {
  int kind;
  int method;
  int ncub;
  int ensure_psd;
  int score_form;   // 1: the reference's score-function derivative sums
  T variance;
  T binsize;
  T power;
  T log_binsize;
  T cub_x[BN_MAX_CUB];  // sqrt(2) * Hermite nodes
  T cub_w[BN_MAX_CUB];  // Hermite weights / sqrt(pi)
};

// The likelihood of one site: kind and Gaussian noise variance.  Normally the
// model's (lp.kind, lp.variance); a model of many series gives each series its own.
template <typename T>
struct SiteLik {
  int kind;
  T variance;
};
template <typename T> __device__ __forceinline__ SiteLik<T> site_lik(const LikParams<T>& lp) {
  return SiteLik<T>{lp.kind, lp.variance};
}

constexpr double kLog2Pi = 1.8378770664093453;
constexpr double kInv2Pi = 0.15915494309189535;

// Transcendentals: hardware approximations in float32 (ex2/lg2 based, absolute
// error ~1e-7 on the log scale), the correctly rounded library versions in float64.
__device__ __forceinline__ float fexp(float x) { return __expf(x); }
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ float flog(float x) { return __logf(x); }
__device__ __forceinline__ double flog(double x) { return log(x); }
__device__ __forceinline__ float flog1p(float x) { return __logf(1.0f + x); }
__device__ __forceinline__ double flog1p(double x) { return log1p(x); }

template <typename T> __device__ __forceinline__ T softplus(T x) {
  const T ax = x < T(0) ? -x : x;
  return (x > T(0) ? x : T(0)) + flog1p(fexp(-ax));
}
template <typename T> __device__ __forceinline__ T sigmoid(T x) { return bn_rcp(T(1) + fexp(-x)); }

__device__ __forceinline__ float bn_normcdf(float x) { return normcdff(x); }
__device__ __forceinline__ double bn_normcdf(double x) { return normcdf(x); }

// log p(y|f) and its first two f-derivatives for single-latent likelihoods;
// KIND = 0 dispatches on sl.kind at run time.
template <int KIND, typename T>
__device__ __forceinline__ void loglik1k(const LikParams<T>& lp, SiteLik<T> sl, T y, T f, T& l, T& d1, T& d2) {
  switch (KIND == 0 ? sl.kind : KIND) {
    case BN_LIK_GAUSSIAN: {
      const T iv = T(1) / sl.variance;
      const T r = y - f;
      l = T(-0.5) * (T(kLog2Pi) + log(sl.variance)) - T(0.5) * r * r * iv;
      d1 = r * iv;
      d2 = -iv;
      break;
    }
    case BN_LIK_BERNOULLI_LOGIT: {
      // one exponential serves sigma(f) and both softplus branches
      const T e = fexp(-bn_abs(f));
      const T r = bn_rcp(T(1) + e);
      const T lg = flog1p(e);
      const bool one = (y == T(1));
      const bool pos = f >= T(0);
      const T s = pos ? r : e * r;        // sigma(f)
      const T sc = pos ? e * r : r;       // 1 - sigma(f)
      const T z = one ? -f : f;           // log p = -softplus(z)
      l = -((z > T(0) ? z : T(0)) + lg);
      d1 = one ? sc : -s;
      d2 = -s * sc;
      break;
    }
    case BN_LIK_BERNOULLI_PROBIT: {
      const T j = T(1e-3);
      const bool one = (y == T(1));
      const T sgn = one ? T(1) : T(-1);
      const T p = bn_normcdf(sgn * f) * (T(1) - T(2) * j) + j;  // P(y | f)
      const T phi = exp(T(-0.5) * f * f) * T(0.3989422804014327) * (T(1) - T(2) * j);
      const T a = sgn * phi / p;                                   // d log p
      l = log(p);
      d1 = a;
      d2 = sgn * (-f * phi) / p - a * a;
      break;
    }
    case BN_LIK_POISSON_EXP:
    default: {
      const T mu = fexp(f) * lp.binsize;
      l = y * (f + lp.log_binsize) - mu - lgamma(y + T(1));
      d1 = y - mu;
      d2 = -mu;
      break;
    }
  }
}

template <typename T>
__device__ __forceinline__ void loglik1(const LikParams<T>& lp, SiteLik<T> sl, T y, T f, T& l, T& d1, T& d2) {
  loglik1k<0>(lp, sl, y, f, l, d1, d2);
}
template <typename T>
__device__ __forceinline__ void loglik1(const LikParams<T>& lp, T y, T f, T& l, T& d1, T& d2) {
  loglik1k<0>(lp, site_lik(lp), y, f, l, d1, d2);
}

// Cubature sums of one scalar site for likelihood KIND with NC nodes (NC = 0:
// the runtime count).  A compile-time NC unrolls the node loop so that the
// transcendentals of different nodes overlap.
template <int KIND, int NC, typename T>
__device__ __forceinline__ void ve1_gh(const LikParams<T>& lp, SiteLik<T> sl, T y, T m, T v, T& E, T& dE, T& d2E) {
  const T sv = sqrt(v);
  T e = T(0), a = T(0), b = T(0);
  if (lp.score_form) {
    // Score-function sums of cubature.py:198-246.  log p is taken relative to its
    // value at the mean, c: sum_i w_i x_i = sum_i w_i (x_i^2 - 1) = 0 for the GH
    // rule, so the derivative sums are unchanged while the float32 cancellation
    // shrinks from |log p| to |log p - c|.
    T c, c1, c2;
    loglik1k<KIND>(lp, sl, y, m, c, c1, c2);
    auto node = [&](int i) {
      const T x = lp.cub_x[i];
      const T w = lp.cub_w[i];
      T l, d1, d2;
      loglik1k<KIND>(lp, sl, y, fma(sv, x, m), l, d1, d2);
      e = fma(w, l, e);
      const T wl = w * (l - c);
      a = fma(wl, x, a);
      b = fma(wl, x * x - T(1), b);
    };
    if constexpr (NC > 0) {
#pragma unroll
      for (int i = 0; i < NC; ++i) node(i);
    } else {
      for (int i = 0; i < lp.ncub; ++i) node(i);
    }
    E = e;
    dE = a / sv;
    d2E = b / v;
  } else {
    auto node = [&](int i) {
      const T w = lp.cub_w[i];
      T l, d1, d2;
      loglik1k<KIND>(lp, sl, y, fma(sv, lp.cub_x[i], m), l, d1, d2);
      e = fma(w, l, e);
      a = fma(w, d1, a);
      b = fma(w, d2, b);
    };
    if constexpr (NC > 0) {
#pragma unroll
      for (int i = 0; i < NC; ++i) node(i);
    } else {
      for (int i = 0; i < lp.ncub; ++i) node(i);
    }
    E = e;
    dE = a;
    d2E = b;
  }
}

// Derivative-form cubature of the Bernoulli-logit site with NC nodes.  With
// t = -f for y = 1 and t = f for y = 0:  log p = -softplus(t),
// d/df log p = -s sigma(t) (s = -1 for y = 1, +1 for y = 0) and
// d2/df2 log p = -sigma(t) (1 - sigma(t)); one exponential, one reciprocal and one
// logarithm per node serve all three.
template <int NC, typename T>
__device__ __forceinline__ void ve1_logit(const LikParams<T>& lp, T y, T m, T v, T& E, T& dE, T& d2E) {
  const T sv = sqrt(v);
  const T flip = (y == T(1)) ? T(-1) : T(1);
  const T sf = flip * sv, mf = flip * m;
  T e = T(0), a = T(0), b = T(0);
  auto node = [&](int i) {
    const T w = lp.cub_w[i];
    const T t = fma(sf, lp.cub_x[i], mf);
    const T ex = fexp(-bn_abs(t));
    const T den = T(1) + ex;
    const T r = bn_rcp(den);
    const T sg = t >= T(0) ? r : ex * r;                 // sigma(t)
    const T sp = (t > T(0) ? t : T(0)) + flog(den);     // softplus(t)
    e = fma(-w, sp, e);
    a = fma(w, sg, a);
    b = fma(w, fma(sg, sg, -sg), b);
  };
  if constexpr (NC > 0) {
#pragma unroll
    for (int i = 0; i < NC; ++i) node(i);
  } else {
    for (int i = 0; i < lp.ncub; ++i) node(i);
  }
  E = e;
  dE = -flip * a;
  d2E = b;
}

// Variational expectation of one scalar site: E_q log p, dE/dm, d2E/dm2.
template <typename T>
__device__ __forceinline__ void ve1(const LikParams<T>& lp, SiteLik<T> sl, T y, T m, T v, T& E, T& dE, T& d2E) {
  if (sl.kind == BN_LIK_GAUSSIAN) {
    const T iv = T(1) / sl.variance;
    const T r = y - m;
    // the library log: log(variance) is the same in every site of a series, so
    // the hardware approximation's error would not average out over its sites
    E = T(-0.5) * (T(kLog2Pi) + log(sl.variance)) - T(0.5) * (r * r + v) * iv;
    dE = r * iv;
    d2E = -iv;
    return;
  }
  if (sl.kind == BN_LIK_POISSON_EXP) {
    // the library exp (one per site): the approximation's relative error grows
    // with |m + v/2| and would weigh on large counts' rates
    const T emc = lp.binsize * exp(m + T(0.5) * v);
    E = y * lp.log_binsize + y * m - emc - lgamma(y + T(1));
    dE = y - emc;
    d2E = -emc;
    return;
  }
  if (sl.kind == BN_LIK_BERNOULLI_LOGIT) {
    if (!lp.score_form) {
      if (lp.ncub == 20) ve1_logit<20>(lp, y, m, v, E, dE, d2E);
      else ve1_logit<0>(lp, y, m, v, E, dE, d2E);
    } else if (lp.ncub == 20) {
      ve1_gh<BN_LIK_BERNOULLI_LOGIT, 20>(lp, sl, y, m, v, E, dE, d2E);
    } else {
      ve1_gh<BN_LIK_BERNOULLI_LOGIT, 0>(lp, sl, y, m, v, E, dE, d2E);
    }
  } else {
    ve1_gh<0, 0>(lp, sl, y, m, v, E, dE, d2E);
  }
}
template <typename T>
__device__ __forceinline__ void ve1(const LikParams<T>& lp, T y, T m, T v, T& E, T& dE, T& d2E) {
  ve1(lp, site_lik(lp), y, m, v, E, dE, d2E);
}

// EP moment matching of one scalar site at the cavity (m, v) with power a
// (cubature.py:310-371; Gaussian in closed form, likelihoods.py:755-780).
template <typename T>
__device__ __forceinline__ void mm1(const LikParams<T>& lp, T y, T m, T v, T& lZ, T& dlZ, T& d2lZ) {
  const T pw = lp.power;
  if (lp.kind == BN_LIK_GAUSSIAN) {
    const T s = lp.variance / pw + v;
    const T r = y - m;
    lZ = T(-0.5) * (r * r / s + T(kLog2Pi) + log(s));
    dlZ = r / s;
    d2lZ = -T(1) / s;
    // pep constant (utils.py:431-446) for a scalar site
    lZ += T(0.5) * ((T(1) - pw) * T(kLog2Pi) - log(pw)) + T(0.5) * (T(1) - pw) * log(lp.variance);
    return;
  }
  const T sv = sqrt(v);
  T Z = T(0), Z1 = T(0), Z2 = T(0);
  for (int i = 0; i < lp.ncub; ++i) {
    const T x = lp.cub_x[i];
    T l, d1, d2;
    loglik1(lp, y, fma(sv, x, m), l, d1, d2);
    const T wl = lp.cub_w[i] * fexp(pw * l);
    Z += wl;
    Z1 = fma(wl, x, Z1);
    Z2 = fma(wl, x * x - T(1), Z2);
  }
  const T Zc = Z > T(1e-8) ? Z : T(1e-8);
  lZ = flog(Zc);
  dlZ = (Z1 / sv) / Zc;
  d2lZ = -dlZ * dlZ + (Z2 / v) / Zc;
}

// Conditional moments E[y|f], Var[y|f] of the single-latent likelihoods
// (likelihoods.py:719-725, 854-860, 952-959) and dE[y|f]/df.
template <typename T>
__device__ __forceinline__ void cond_moments(const LikParams<T>& lp, T f, T& ey, T& vy, T& dey) {
  if (lp.kind == BN_LIK_GAUSSIAN) {
    ey = f;
    vy = lp.variance;
    dey = T(1);
  } else if (lp.kind == BN_LIK_POISSON_EXP) {
    ey = fexp(f) * lp.binsize;
    vy = ey;
    dey = ey;
  } else if (lp.kind == BN_LIK_BERNOULLI_LOGIT) {
    ey = sigmoid(f);
    vy = ey - ey * ey;
    dey = vy;
  } else {  // probit, with the reference's jitter 1e-3 (likelihoods.py:826-827)
    ey = bn_normcdf(f) * T(1 - 2e-3) + T(1e-3);
    vy = ey - ey * ey;
    dey = fexp(T(-0.5) * f * f) * T(0.3989422804014327 * (1 - 2e-3));
  }
}
template <typename T>
__device__ __forceinline__ void cond_moments(const LikParams<T>& lp, T f, T& ey, T& vy) {
  T d;
  cond_moments(lp, f, ey, vy, d);
}

// Statistical linear regression of one scalar site at N(m, v) (cubature.py:374-430):
// mu = E[E[y|f]], omega = S - C^2 / v with S = E[(E[y|f] - mu)^2 + Var[y|f]] and
// C = E[(f - m)(E[y|f] - mu)], and dmu/dm = E[dE[y|f]/df] (the derivative of the
// cubature sum in m, whose nodes move with m).  The sums are taken about E[y|f=m] so
// that S and C keep their digits in float32 when E[y|f] hardly varies over the nodes.
template <typename T>
__device__ __forceinline__ void slr1(const LikParams<T>& lp, T m, T v, T& mu, T& omega, T& dmu) {
  const T sv = sqrt(v);
  T h0, v0, d0;
  cond_moments(lp, m, h0, v0, d0);
  T s0 = T(0), s1 = T(0), s2 = T(0), sx = T(0), sd = T(0);
  for (int i = 0; i < lp.ncub; ++i) {
    const T x = lp.cub_x[i], w = lp.cub_w[i];
    T ey, vy, dey;
    cond_moments(lp, fma(sv, x, m), ey, vy, dey);
    const T d = ey - h0;
    s0 = fma(w, d, s0);
    s1 = fma(w, d * d, s1);
    s2 = fma(w, vy, s2);
    sx = fma(w, x * d, sx);
    sd = fma(w, dey, sd);
  }
  mu = h0 + s0;
  // S = sum w d^2 - (sum w d)^2 + sum w Var;  C = sv sum w x d, so C^2 / v = (sum w x d)^2
  omega = s1 - s0 * s0 + s2 - sx * sx;
  dmu = sd;
}

// ---------------------------------------------------------------- two latents
template <typename T>
__device__ __forceinline__ void hetero_link(int kind, T f2, T& s, T& ds, T& d2s) {
  if (kind == BN_LIK_HETERO_EXP) {
    s = fexp(f2);
    ds = s;
    d2s = s;
  } else {
    s = softplus(f2);
    ds = sigmoid(f2);
    d2s = ds * (T(1) - ds);
  }
}

// log p, gradient g[2] and Hessian (h11, h12, h22) of N(y | f1, link(f2)^2)
template <typename T>
__device__ __forceinline__ void hetero_point(int kind, T y, T f1, T f2, T& l, T (&g)[2], T (&h)[3]) {
  const T r = y - f1;
  if (kind == BN_LIK_HETERO_EXP) {
    const T is2 = fexp(T(-2) * f2);
    const T r2 = r * r * is2;
    l = T(-0.5) * T(kLog2Pi) - f2 - T(0.5) * r2;
    g[0] = r * is2;
    g[1] = r2 - T(1);
    h[0] = -is2;
    h[1] = T(-2) * r * is2;
    h[2] = T(-2) * r2;
  } else {
    T s, ds, d2s;
    hetero_link(kind, f2, s, ds, d2s);
    const T is = bn_rcp(s);
    const T is2 = is * is;
    l = T(-0.5) * T(kLog2Pi) - flog(s) - T(0.5) * r * r * is2;
    g[0] = r * is2;
    g[1] = -ds * is + r * r * ds * is2 * is;
    h[0] = -is2;
    h[1] = T(-2) * r * ds * is2 * is;
    h[2] = -(d2s * s - ds * ds) * is2 + r * r * (d2s * is2 * is - T(3) * ds * ds * is2 * is2);
  }
}

// 2-D GH variational expectation: m[2], V (v11, v12, v22) -> E, g[2], H (h11,h12,h22)
template <typename T>
__device__ __forceinline__ void ve2(const LikParams<T>& lp, T y, const T (&m)[2], const T (&V)[3], T& E,
                                    T (&g)[2], T (&H)[3]) {
  const T L11 = sqrt(V[0]);
  const T L21 = V[1] / L11;
  const T t = V[2] - L21 * L21;
  const T L22 = sqrt(t > T(0) ? t : T(0));
  T e = T(0), g0 = T(0), g1 = T(0), h0 = T(0), h1 = T(0), h2 = T(0);
  for (int i = 0; i < lp.ncub; ++i) {
    const T xi = lp.cub_x[i], wi = lp.cub_w[i];
    const T f1 = fma(L11, xi, m[0]);
    const T f2b = fma(L21, xi, m[1]);
    T ei = T(0), a0 = T(0), a1 = T(0), b0 = T(0), b1 = T(0), b2 = T(0);
    for (int j = 0; j < lp.ncub; ++j) {
      const T wj = lp.cub_w[j];
      T l, gg[2], hh[3];
      hetero_point(lp.kind, y, f1, fma(L22, lp.cub_x[j], f2b), l, gg, hh);
      ei = fma(wj, l, ei);
      a0 = fma(wj, gg[0], a0);
      a1 = fma(wj, gg[1], a1);
      b0 = fma(wj, hh[0], b0);
      b1 = fma(wj, hh[1], b1);
      b2 = fma(wj, hh[2], b2);
    }
    e = fma(wi, ei, e);
    g0 = fma(wi, a0, g0);
    g1 = fma(wi, a1, g1);
    h0 = fma(wi, b0, h0);
    h1 = fma(wi, b1, h1);
    h2 = fma(wi, b2, h2);
  }
  E = e;
  g[0] = g0;
  g[1] = g1;
  H[0] = h0;
  H[1] = h1;
  H[2] = h2;
}

// The 2-D Gauss-Hermite sums of ve2 over the outer nodes i = i0, i0 + di, ...
// only (a share of the 400 nodes, for several lanes working on one site; the
// shares' sums add up to ve2's).
template <typename T>
__device__ __forceinline__ void ve2_part(const LikParams<T>& lp, T y, const T (&m)[2], const T (&V)[3], int i0, int di,
                                         T (&acc)[6]) {
  const T L11 = sqrt(V[0]);
  const T L21 = V[1] / L11;
  const T t = V[2] - L21 * L21;
  const T L22 = sqrt(t > T(0) ? t : T(0));
#pragma unroll
  for (int q = 0; q < 6; ++q) acc[q] = T(0);
  for (int i = i0; i < lp.ncub; i += di) {
    const T xi = lp.cub_x[i], wi = lp.cub_w[i];
    const T f1 = fma(L11, xi, m[0]);
    const T f2b = fma(L21, xi, m[1]);
    T s[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (int j = 0; j < lp.ncub; ++j) {
      const T wj = lp.cub_w[j];
      T l, gg[2], hh[3];
      hetero_point(lp.kind, y, f1, fma(L22, lp.cub_x[j], f2b), l, gg, hh);
      s[0] = fma(wj, l, s[0]);
      s[1] = fma(wj, gg[0], s[1]);
      s[2] = fma(wj, gg[1], s[2]);
      s[3] = fma(wj, hh[0], s[3]);
      s[4] = fma(wj, hh[1], s[4]);
      s[5] = fma(wj, hh[2], s[5]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] = fma(wi, s[q], acc[q]);
  }
}

// ---------------------------------------------------------------- site algebra
// ensure_diagonal_positive_precision applied to -H, returned as H (utils.py:89-96):
// keep the diagonal where -H_ii >= 0 (NaN kept), else -1e-2; off-diagonals dropped.
template <typename T> __device__ __forceinline__ T psd_diag(T h) { return (-h < T(0)) ? T(-1e-2) : h; }

}  // namespace bn
