// Gradient of the variational energy with respect to the hyperparameters.
//
// The reference differentiates VariationalInference.energy (bayesnewton/
// inference.py:197-222) with objax.GradValues (README.md:58-66).  Its posterior
// marginals are state variables, constant under that derivative, so the energy
// depends on the hyperparameters in two places only:
//   - the filter log marginal of the pseudo-observations inside compute_kl
//     (basemodels.py:708-741), log Z(theta), through the prior; and
//   - E_q[log p(y | f)] through the likelihood's own parameters (Gaussian noise
//     variance, likelihoods.py:727-753).
// d energy / d theta = -d log Z / d theta - sum_n d E_q[log p(y_n | f_n)] / d theta.
// The Newton, EP and PL energies have the same log Z term (their compute_kl /
// lZ_post, inference.py:130-154, 286-325, 371-428); their likelihood terms are
// log p(y | m) and (1 / a) lZ at the cavity.
//
// d log Z / d theta is taken with Fisher's identity: the expected gradient of the
// prior's log density, log N(x_0 | 0, Pinf) + sum_k log N(x_k | A_k x_{k-1}, Q_k),
// under the smoothing distribution of the pseudo-observations.  With the filtered
// (m, P) at k-1, pm = A m, pP = A P A^T + Q, the smoothed mean / covariance mu_k,
// S_k and the smoother gain G_{k-1}, the expectations reduce to (per step k >= 1)
//   1/2 tr(dQ B_k) + tr(dA C_k),
//   B_k = pP^-1 [(S_k - pP) + d d^T] pP^-1,   C_k = [G_{k-1} (S_k - pP) + mu_{k-1} d^T] pP^-1,
//   d = mu_k - pm,
// (the first state: A = 0, Q = Pinf, pP = Pinf).  These forms come from writing
// x_k - A x_{k-1} through the smoother's backward conditional; they contain no Q^-1,
// so short and zero time gaps (Q -> 0) are as well conditioned as the filter.  Each
// step is independent: one thread per step in the model's dtype, block sums in
// float64.
//
// dA / d lengthscale is exact: the closed-form Matern transition evaluated on dual
// numbers.  Pinf of a Matern block has entries proportional to lengthscale^-(i+j),
// so d Pinf_ij / d lengthscale = -(i + j) Pinf_ij / lengthscale, and Pinf and Q are
// proportional to the variance.
//
// Exactness: log Z of the reference leaves the log density of masked (missing)
// pseudo-observations out of its sum while the filter still conditions on them
// (ops.py:154-180); Fisher's identity gives the gradient of the unmasked log Z.
// The two differ by the masked terms' dependence on theta, each weighted by the
// site precision of a missing observation (1e-6), which is below the float64
// tolerance of the parity tests for the missing fractions they use.
#pragma once
#include "bn_ssm.cuh"

namespace bn {

// Forward-mode dual number (value, derivative).  Its operators live in their own
// namespace, found by argument-dependent lookup, so that they do not hide the
// float / double exp and fma for the rest of bn.
namespace ad {
template <typename R>
struct Dual {
  R v, d;
  __device__ __forceinline__ Dual() : v(R(0)), d(R(0)) {}
  __device__ __forceinline__ Dual(R x) : v(x), d(R(0)) {}
  __device__ __forceinline__ Dual(R x, R dx) : v(x), d(dx) {}
};
template <typename R>
__device__ __forceinline__ Dual<R> operator+(Dual<R> a, Dual<R> b) { return Dual<R>(a.v + b.v, a.d + b.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> a, Dual<R> b) { return Dual<R>(a.v - b.v, a.d - b.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> a) { return Dual<R>(-a.v, -a.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator*(Dual<R> a, Dual<R> b) {
  return Dual<R>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <typename R>
__device__ __forceinline__ Dual<R> operator/(Dual<R> a, Dual<R> b) {
  const R r = R(1) / b.v;
  return Dual<R>(a.v * r, (a.d - a.v * r * b.d) * r);
}
template <typename R>
__device__ __forceinline__ Dual<R> exp(Dual<R> a) {
  const R e = ::exp(a.v);
  return Dual<R>(e, e * a.d);
}
template <typename R>
__device__ __forceinline__ Dual<R> fma(Dual<R> a, Dual<R> b, Dual<R> c) { return a * b + c; }
}  // namespace ad
using ad::Dual;

constexpr int kGradMax = 2 * BN_MAX_COMPONENTS + 1;

template <typename R, int D, int P>
struct GradArgs {
  SSM<R, D, P> ssm;
  double var[BN_MAX_COMPONENTS];
  double ell[BN_MAX_COMPONENTS];
  int64_t n;
  int obs_dim;
  int lik_gauss;    // 1: add the Gaussian noise-variance term
  int method;       // BN_METHOD_*: which energy's likelihood term
  double lik_var;
  double power;     // EP power (PL: 1)
  const void* dt;   // [n] model dtype, dt[0] unused (the first state is the prior)
  const void* fm;   // [n, D] filtered means
  const void* fP;   // [n, D, D]
  const void* sm;   // [n, D] smoothed means
  const void* sP;   // [n, D, D]
  const void* G;    // [n, D, D] smoother gains (G_k maps k+1 to k)
  const void* y;    // [n, obs_dim]
  const void* pm;   // [n, P] stored posterior marginals (the likelihood term)
  const void* pv;   // [n, P, P]
  const void* nat1; // [n, P] sites (the EP / PL cavity)
  const void* nat2; // [n, P, P]
  double* acc;      // [kGradMax]: d log Z / d (var_c, ell_c) ..., then sum d E_q log p / d lik_var
};

template <typename T, int D>
__device__ __forceinline__ void gload(const void* p, int64_t k, T (&M)[D][D]) {
  const T* q = static_cast<const T*>(p) + (size_t)k * D * D;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M[i][j] = q[i * D + j];
}
template <typename T, int D>
__device__ __forceinline__ void gload(const void* p, int64_t k, T (&v)[D]) {
  const T* q = static_cast<const T*>(p) + (size_t)k * D;
#pragma unroll
  for (int i = 0; i < D; ++i) v[i] = q[i];
}

// Per-component contributions 1/2 tr(dQ B) + tr(dA C) of one step.  head: the first
// state (A = 0, Q = Pinf).
template <typename L, int c, typename R, int D, int P>
__device__ __forceinline__ void grad_comp(const GradArgs<R, D, P>& g, bool head, R dt, const R (&A)[D][D],
                                          const R (&B)[D][D], const R (&C)[D][D], R (&out)[kGradMax]) {
  if constexpr (c < L::NC) {
    constexpr int o = L::off(c);
    constexpr int s = L::size(c);
    const R sig2 = R(g.var[c]), ell = R(g.ell[c]);
    const R(&Pi)[D][D] = g.ssm.Pinf;
    // dPinf / d ell
    R dPl[s][s];
#pragma unroll
    for (int i = 0; i < s; ++i)
#pragma unroll
      for (int j = 0; j < s; ++j) dPl[i][j] = -R(i + j) / ell * Pi[o + i][o + j];
    R tv = R(0), tl = R(0);
    if (head) {
      // dQ = dPinf, no transition
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) {
          tv = fma(Pi[o + i][o + j] / sig2, B[o + j][o + i], tv);
          tl = fma(dPl[i][j], B[o + j][o + i], tl);
        }
      out[2 * c] += R(0.5) * tv;
      out[2 * c + 1] += R(0.5) * tl;
    } else {
      // dA / d lam on dual numbers, then d lam / d ell = -lam / ell
      Dual<R> Ad[s][s];
      const R lam = g.ssm.lam[c];
      matern_transition<s>(Dual<R>(lam, R(1)), Dual<R>(dt), Ad);
      R dA[s][s], AP[s][s], AdP[s][s];
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) dA[i][j] = Ad[i][j].d * (-lam / ell);
      // A Pinf and A dPinf on the block
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) {
          R a = R(0), b = R(0);
#pragma unroll
          for (int k = 0; k < s; ++k) {
            a = fma(A[o + i][o + k], Pi[o + k][o + j], a);
            b = fma(A[o + i][o + k], dPl[k][j], b);
          }
          AP[i][j] = a;
          AdP[i][j] = b;
        }
      // Q = Pinf - A Pinf A^T (dQ / d var = Q / var);
      // dQ / d ell = dPl - dA Pinf A^T - A dPl A^T - A Pinf dA^T
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) {
          R q = Pi[o + i][o + j], d = dPl[i][j];
#pragma unroll
          for (int k = 0; k < s; ++k) {
            q = fma(-AP[i][k], A[o + j][o + k], q);
            d = fma(-dA[i][k], AP[j][k], d);
            d = fma(-AdP[i][k], A[o + j][o + k], d);
            d = fma(-AP[i][k], dA[j][k], d);
          }
          tv = fma(R(0.5) * q / sig2, B[o + j][o + i], tv);
          tl = fma(R(0.5) * d, B[o + j][o + i], tl);
        }
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) tl = fma(dA[i][j], C[o + j][o + i], tl);
      out[2 * c] += tv;
      out[2 * c + 1] += tl;
    }
    grad_comp<L, c + 1>(g, head, dt, A, B, C, out);
  }
}

template <typename T, typename L, int P>
__global__ void __launch_bounds__(128) grad_kernel(GradArgs<T, L::D, P> g) {
  // per-step algebra in the model's dtype (the forms above are well conditioned),
  // a handful of steps per thread summed in it, block sums in float64
  constexpr int D = L::D;
  constexpr int NG = 2 * L::NC + 1;
  using R = T;
  __shared__ double red[NG][4];
  R out[kGradMax];
#pragma unroll
  for (int i = 0; i < kGradMax; ++i) out[i] = R(0);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < g.n; k += stride) {
    const bool head = k == 0;
    R A[D][D], pP[D][D], S[D][D], pm[D], mu[D];
    R dt = R(0);
    gload<T, D>(g.sm, k, mu);
    gload<T, D>(g.sP, k, S);
    if (head) {
      set_zero(A);
      copy(pP, g.ssm.Pinf);
      set_zero(pm);
    } else {
      dt = static_cast<const T*>(g.dt)[k];
      transition<L>(g.ssm, dt, A);
      R fm[D], X[D][D], AP[D][D];
      gload<T, D>(g.fm, k - 1, fm);
      gload<T, D>(g.fP, k - 1, X);
      mv_blk<L>(pm, A, fm);
      mm_blk<L>(AP, A, X);
      R Q[D][D];
      process_noise<L>(Q, A, g.ssm.Pinf);
      mmt_blk_sym_add<L>(pP, AP, A, Q);
    }
    // W1 = S - pP, dd = mu - pm
    R W1[D][D], dd[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      dd[i] = mu[i] - pm[i];
#pragma unroll
      for (int j = 0; j < D; ++j) W1[i][j] = S[i][j] - pP[i][j];
    }
    // Y = pP^-1
    R Y[D][D];
    cholesky(pP);
    set_identity(Y);
    chol_solve(pP, Y);
    // B = Y (W1 + dd dd^T) Y
    R B[D][D], C[D][D], Z[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) S[i][j] = W1[i][j] + dd[i] * dd[j];
    mm(Z, Y, S);
    mm(B, Z, Y);
    if (head) {
      set_zero(C);
    } else {
      // C = (G_{k-1} W1 + mu_{k-1} dd^T) Y
      R Gm[D][D], mu0[D];
      gload<T, D>(g.G, k - 1, Gm);
      gload<T, D>(g.sm, k - 1, mu0);
      mm(Z, Gm, W1);
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) Z[i][j] = fma(mu0[i], dd[j], Z[i][j]);
      mm(C, Z, Y);
    }
    grad_comp<L, 0>(g, head, dt, A, B, C, out);
    if (P == 1 && g.lik_gauss) {
      const T yk = static_cast<const T*>(g.y)[k * g.obs_dim];
      if (yk == yk) {
        const R m = static_cast<const T*>(g.pm)[k];
        const R v = static_cast<const T*>(g.pv)[k];
        const R s2 = R(g.lik_var);
        R lt;
        if (g.method == BN_METHOD_VI) {
          // d E_q log N(y | f, s2) / d s2
          const R r = R(yk) - m;
          lt = R(-0.5) / s2 + R(0.5) * (r * r + v) / (s2 * s2);
        } else if (g.method == BN_METHOD_NEWTON) {
          // d log N(y | m, s2) / d s2
          const R r = R(yk) - m;
          lt = R(-0.5) / s2 + R(0.5) * r * r / (s2 * s2);
        } else {
          // EP / PL: (1 / a) d lZ / d s2 with lZ = log N(y | cm, s2 / a + cv) + the
          // power-EP constant 1/2 (1 - a) log s2 (utils.py:431-446), at the cavity
          // (compute_cavity, utils.py:534-541, jitter 1e-8)
          const R a = R(g.power);
          const R n1 = static_cast<const T*>(g.nat1)[k];
          const R n2 = static_cast<const T*>(g.nat2)[k];
          const R pn2 = R(1) / (v + R(1e-8));
          const R cv = R(1) / (pn2 - a * n2);
          const R cm = cv * (pn2 * m - a * n1);
          const R sv = s2 / a + cv;
          const R r = R(yk) - cm;
          lt = ((R(-0.5) / sv + R(0.5) * r * r / (sv * sv)) / a + R(0.5) * (R(1) - a) / s2) / a;
        }
        out[NG - 1] += lt;
      }
    }
  }
  // block sums
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < NG; ++q) {
    double v = double(out[q]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (l == 0) red[q][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < NG) {
    const double v = red[threadIdx.x][0] + red[threadIdx.x][1] + red[threadIdx.x][2] + red[threadIdx.x][3];
    atomicAdd(&g.acc[threadIdx.x], v);
  }
}

}  // namespace bn
