// State-space prior on the device: A(dt) per component, Pinf and H.
//
// The prior is a block-diagonal stack of components (a single kernel, a Sum or an
// Independent stack; bayesnewton/kernels.py:1499-1663).  The block sizes are a
// compile-time Layout so that every register index is static and products with A
// (and with the block-diagonal Pinf) skip the zero blocks.
//
// Each component's transition is the reference's closed form when one exists
// (Matern12/32/52/72, kernels.py:158-165, 216-224, 273-286, 344-365; a Matern block
// is recognised by its size 1/2/3/4) and otherwise the generic A = expm(F dt) of
// kernels.py:63-67, evaluated by scaling and squaring of a degree-12 Taylor
// polynomial (Moler & Van Loan, "Nineteen dubious ways to compute the exponential
// of a matrix", method 3).
#pragma once
#include <type_traits>

#include "bn_layout.h"
#include "bn_small.cuh"

namespace bn {

template <typename T, int D, int P>
struct SSM {
  int ncomp;
  int kind[BN_MAX_COMPONENTS];
  T lam[BN_MAX_COMPONENTS];  // sqrt(2 nu) / lengthscale (1/lengthscale for Matern12)
  T var[BN_MAX_COMPONENTS];  // component variances (Matern blocks)
  T Pinf[D][D];
  T H[P][D];
  T F[D][D];                 // feedback matrix; read only for BN_KIND_FEEDBACK blocks
  T hph[P];                  // prior marginal variances diag(H Pinf H^T)
};

// ------------------------------------------------------------- measurement model
// On a layout of several blocks (one per prior component) H observes the first
// state of each block: summed into the single output of a Sum (P = 1), one output
// per block of an Independent stack (P = number of blocks) -- the construction of
// kernels.py:1588-1663.  That H is known at compile time, so its products cost
// additions only.  Single-block layouts (one Matern, or a prior run on the dense
// layout, whose H is the model's) read H from the model.
template <typename L, int P>
struct HLayout {
  static constexpr bool kStatic = L::NC >= 2 && (P == 1 || P == L::NC) && L::D <= 8 && P <= 8;
  // bit 8 p + i set when H[p][i] = 1 (a compile-time constant, so that a test of
  // it with the unrolled loop indices folds away)
  static constexpr unsigned long long bits() {
    unsigned long long b = 0;
    for (int c = 0; c < L::NC; ++c) b |= 1ull << ((P == 1 ? 0 : c) * 8 + L::off(c));
    return b;
  }
  static constexpr unsigned long long kBits = bits();
};

// s + H[p][i] x
template <typename L, int P, typename T, int D, int Q>
__device__ __forceinline__ T hacc(const SSM<T, D, Q>& m, int p, int i, T x, T s) {
  if constexpr (HLayout<L, P>::kStatic) {
    return ((HLayout<L, P>::kBits >> (p * 8 + i)) & 1ull) ? s + x : s;
  } else {
    return fma(m.H[p][i], x, s);
  }
}

// ------------------------------------------------------------- block products
// O = A X for block-diagonal A
template <typename L, typename T, int D>
BN_HD void mm_blk(T (&O)[D][D], const T (&A)[D][D], const T (&X)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = L::lo(i); k < L::hi(i); ++k) s = fma(A[i][k], X[k][j], s);
      O[i][j] = s;
    }
}

// o = A v for block-diagonal A
template <typename L, typename T, int D>
BN_HD void mv_blk(T (&o)[D], const T (&A)[D][D], const T (&v)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = T(0);
#pragma unroll
    for (int k = L::lo(i); k < L::hi(i); ++k) s = fma(A[i][k], v[k], s);
    o[i] = s;
  }
}

// O = X A^T + Z (symmetric result), A block-diagonal
template <typename L, typename T, int D>
BN_HD void mmt_blk_sym_add(T (&O)[D][D], const T (&X)[D][D], const T (&A)[D][D], const T (&Z)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Z[i][j];
#pragma unroll
      for (int k = L::lo(j); k < L::hi(j); ++k) s = fma(X[i][k], A[j][k], s);
      O[i][j] = s;
      O[j][i] = s;
    }
}

// Q = Pinf - A Pinf A^T, block-diagonal (Pinf and A share the layout)
template <typename L, typename T, int D>
BN_HD void process_noise(T (&Q)[D][D], const T (&A)[D][D], const T (&Pinf)[D][D]) {
  T X[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
      if (L::lo(i) == L::lo(j)) {
#pragma unroll
        for (int k = L::lo(i); k < L::hi(i); ++k) s = fma(A[i][k], Pinf[k][j], s);
      }
      X[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Pinf[i][j];
      if (L::lo(i) == L::lo(j)) {
#pragma unroll
        for (int k = L::lo(j); k < L::hi(j); ++k) s = fma(-X[i][k], A[j][k], s);
      } else {
        s = T(0);
      }
      Q[i][j] = s;
      Q[j][i] = s;
    }
}

// Q = Pinf - A Pinf A^T on the block [o, o+S)
template <int S, int o, typename T, int D>
BN_HD void process_noise_block(const T (&A)[D][D], const T (&Pinf)[D][D], T (&Q)[D][D]) {
  T X[S][S];
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = 0; j < S; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < S; ++k) s = fma(A[o + i][o + k], Pinf[o + k][o + j], s);
      X[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = i; j < S; ++j) {
      T s = Pinf[o + i][o + j];
#pragma unroll
      for (int k = 0; k < S; ++k) s = fma(-X[i][k], A[o + j][o + k], s);
      Q[o + i][o + j] = s;
      Q[o + j][o + i] = s;
    }
}

// ------------------------------------------------------------- transitions
// Degree-12 Taylor expm with scaling and squaring for the block [O, O+S).
template <typename T, int D, int O, int S>
__device__ __forceinline__ void expm_block(const T (&F)[D][D], T dt, T (&A)[D][D]) {
  T X[S][S], R[S][S], Tm[S][S];
  T nrm = T(0);
#pragma unroll
  for (int i = 0; i < S; ++i) {
    T row = T(0);
#pragma unroll
    for (int j = 0; j < S; ++j) {
      X[i][j] = F[O + i][O + j] * dt;
      row += bn_abs(X[i][j]);
    }
    nrm = row > nrm ? row : nrm;
  }
  int sq = 0;
  while (nrm > T(0.5) && sq < 60) {
    nrm *= T(0.5);
    ++sq;
  }
  const T sc = ldexp(T(1), -sq);
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = 0; j < S; ++j) X[i][j] *= sc;
  set_identity(R);
#pragma unroll
  for (int k = 12; k >= 1; --k) {
    mm(Tm, X, R);
    const T ik = T(1) / T(k);
#pragma unroll
    for (int i = 0; i < S; ++i)
#pragma unroll
      for (int j = 0; j < S; ++j) R[i][j] = fma(Tm[i][j], ik, (i == j ? T(1) : T(0)));
  }
  for (int q = 0; q < sq; ++q) {
    mm(Tm, R, R);
    copy(R, Tm);
  }
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = 0; j < S; ++j) A[O + i][O + j] = R[i][j];
}

// Closed-form transition of one Matern block of size S (1/2/3/4: Matern12/32/52/72)
// with lam = sqrt(2 nu) / lengthscale.  Generic in T so that it also runs on dual
// numbers (the lengthscale derivative of the energy).
template <int S, typename T>
BN_HD void matern_transition(T lam, T dt, T (&B)[S][S]) {
  if constexpr (S == 1) {
    B[0][0] = exp(-dt * lam);
  } else if constexpr (S == 2) {
    const T e = exp(-dt * lam);
    const T tl = dt * lam;
    B[0][0] = e * (tl + T(1));
    B[0][1] = e * dt;
    B[1][0] = -e * dt * lam * lam;
    B[1][1] = e * (T(1) - tl);
  } else if constexpr (S == 3) {
    const T tl = dt * lam;
    const T e = exp(-tl);
    const T l2 = lam * lam, l3 = l2 * lam;
    B[0][0] = e * (dt * lam * (T(0.5) * tl + T(1)) + T(1));
    B[0][1] = e * (dt * (tl + T(1)));
    B[0][2] = e * (dt * T(0.5) * dt);
    B[1][0] = e * (dt * (T(-0.5) * tl * l2));
    B[1][1] = e * (dt * lam * (T(1) - tl) + T(1));
    B[1][2] = e * (dt * (T(1) - T(0.5) * tl));
    B[2][0] = e * (dt * l3 * (T(0.5) * tl - T(1)));
    B[2][1] = e * (dt * l2 * (tl - T(3)));
    B[2][2] = e * (dt * lam * (T(0.5) * tl - T(2)) + T(1));
  } else if constexpr (S == 4) {
    const T l2 = lam * lam, l3 = l2 * lam, l4 = l2 * l2;
    const T tl = dt * lam;
    const T tl2 = tl * tl;
    const T e = exp(-tl);
    const T s6 = T(1) / T(6);
    T M[4][4];
    M[0][0] = lam * (T(1) + T(0.5) * tl + tl2 * s6);
    M[0][1] = T(1) + tl + T(0.5) * tl2;
    M[0][2] = T(0.5) * dt * (T(1) + tl);
    M[0][3] = dt * dt * s6;
    M[1][0] = -tl2 * l2 * s6;
    M[1][1] = lam * (T(1) + T(0.5) * tl - T(0.5) * tl2);
    M[1][2] = T(1) + tl - T(0.5) * tl2;
    M[1][3] = dt * (T(0.5) - tl * s6);
    M[2][0] = l3 * tl * (tl * s6 - T(0.5));
    M[2][1] = tl * l2 * (T(0.5) * tl - T(2));
    M[2][2] = lam * (T(1) - T(2.5) * tl + T(0.5) * tl2);
    M[2][3] = T(1) - tl + tl2 * s6;
    M[3][0] = l4 * (tl - T(1) - tl2 * s6);
    M[3][1] = l3 * (T(3.5) * tl - T(4) - T(0.5) * tl2);
    M[3][2] = l2 * (T(4) * tl - T(6) - T(0.5) * tl2);
    M[3][3] = lam * (T(1.5) * tl - T(3) - tl2 * s6);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) B[i][j] = e * fma(dt, M[i][j], (i == j ? T(1) : T(0)));
  }
}

template <typename L, int c, typename T, int D, int P>
__device__ __forceinline__ void transition_comp(const SSM<T, D, P>& m, T dt, T (&A)[D][D]) {
  if constexpr (c < L::NC) {
    constexpr int o = L::off(c);
    constexpr int s = L::size(c);
    if (m.kind[c] == BN_KIND_FEEDBACK || s > 4) {
      expm_block<T, D, o, s>(m.F, dt, A);
    } else if constexpr (s <= 4) {
      T B[s][s];
      matern_transition<s>(m.lam[c], dt, B);
#pragma unroll
      for (int i = 0; i < s; ++i)
#pragma unroll
        for (int j = 0; j < s; ++j) A[o + i][o + j] = B[i][j];
    }
    transition_comp<L, c + 1>(m, dt, A);
  }
}

// A = blockdiag_c A_c(dt)
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void transition(const SSM<T, D, P>& m, T dt, T (&A)[D][D]) {
  set_zero(A);
  transition_comp<L, 0>(m, dt, A);
}

// ------------------------------------------------------------- process noise
// Q = Pinf - A Pinf^T of one Matern block without the cancellation of that form.
//
// With the state scaled by diag(lam^i), a Matern block of size S has feedback
// lam F~ (F~ the companion matrix of (s + 1)^S), stationary covariance var P~ and
// transition e^{-x} Pi(x) at x = lam dt, where Pi(x) = sum_{k<S} N^k x^k / k! and
// N = F~ + I is nilpotent.  Writing P~ = e^{-2x} e^{2x} P~ gives
//   Q_ij = var lam^(i+j) e^{-2x} [ sum_{n<=2S-2} c_ij,n x^n
//                                  + 2^(2S-1) P~_ij x^(2S-1) phi_(2S-1)(2x) ],
//   c_n = 2^n P~ / n! - sum_{a+b=n} N^a P~ (N^b)^T / (a! b!),
//   phi_k(z) = sum_{j>=0} z^j / (j+k)!  (a series of positive terms),
// in which the terms below each entry's leading power of x are exactly zero, so
// an entry of order x^5 keeps its relative precision when Pinf - A Pinf A^T in
// float32 would keep none of it.  The c_n are exact rationals (tabulated below);
// the form is used for x < 2 (phi_k by its Taylor series, z < 4); beyond that the
// direct form loses less than two digits and is used instead.
constexpr double qc_matern(int S, int n, int i, int j) {
  // entries (i <= j) of c_n for S = 1..4; zero elsewhere
  if (j < i) { const int t = i; i = j; j = t; }
  if (S == 2) {
    if (n == 1 && i == 1 && j == 1) return 4.0;
    if (n == 2 && i == 0 && j == 1) return 2.0;
  } else if (S == 3) {
    if (n == 1 && i == 2 && j == 2) return 16.0 / 3.0;
    if (n == 2) return (i == 1 && j == 2) ? 8.0 / 3.0 : (i == 2 && j == 2) ? -16.0 / 3.0 : 0.0;
    if (n == 3) {
      if (i == 0 && j == 2) return 8.0 / 9.0;
      if (i == 1 && j == 1) return 16.0 / 9.0;
      if (i == 1 && j == 2) return -8.0 / 3.0;
      if (i == 2 && j == 2) return 16.0 / 3.0;
    }
    if (n == 4) {
      if (i == 0 && j == 1) return 2.0 / 3.0;
      if (i == 0 && j == 2) return -8.0 / 9.0;
      if (i == 1 && j == 1) return -4.0 / 9.0;
      if (i == 1 && j == 2) return 2.0 / 3.0;
    }
  } else if (S == 4) {
    if (n == 1 && i == 3 && j == 3) return 32.0 / 5.0;
    if (n == 2) return (i == 2 && j == 3) ? 16.0 / 5.0 : (i == 3 && j == 3) ? -64.0 / 5.0 : 0.0;
    if (n == 3) {
      if (i == 1 && j == 3) return 16.0 / 15.0;
      if (i == 2 && j == 2) return 32.0 / 15.0;
      if (i == 2 && j == 3) return -32.0 / 5.0;
      if (i == 3 && j == 3) return 256.0 / 15.0;
    }
    if (n == 4) {
      if (i == 0 && j == 3) return 4.0 / 15.0;
      if (i == 1 && j == 2) return 4.0 / 5.0;
      if (i == 1 && j == 3) return -32.0 / 15.0;
      if (i == 2 && j == 2) return -32.0 / 15.0;
      if (i == 2 && j == 3) return 64.0 / 15.0;
      if (i == 3 && j == 3) return -32.0 / 5.0;
    }
    if (n == 5) {
      if (i == 0 && j == 2) return 16.0 / 75.0;
      if (i == 0 && j == 3) return -8.0 / 15.0;
      if (i == 1 && j == 1) return 8.0 / 25.0;
      if (i == 1 && j == 2) return -8.0 / 15.0;
      if (i == 1 && j == 3) return 56.0 / 75.0;
      if (i == 2 && j == 2) return 64.0 / 75.0;
      if (i == 2 && j == 3) return -16.0 / 15.0;
      if (i == 3 && j == 3) return 8.0 / 5.0;
    }
    if (n == 6) {
      if (i == 0 && j == 1) return 4.0 / 45.0;
      if (i == 0 && j == 2) return -8.0 / 75.0;
      if (i == 0 && j == 3) return 4.0 / 45.0;
      if (i == 1 && j == 1) return -16.0 / 225.0;
      if (i == 1 && j == 2) return 4.0 / 45.0;
      if (i == 1 && j == 3) return -8.0 / 75.0;
      if (i == 2 && j == 2) return -16.0 / 225.0;
      if (i == 2 && j == 3) return 4.0 / 45.0;
    }
  }
  return 0.0;
}

// P~_ij of a Matern block of size S (the stationary covariance at var = lam = 1)
constexpr double pinf_matern(int S, int i, int j) {
  if (j < i) { const int t = i; i = j; j = t; }
  if (i == j) return (S == 3 && i == 1) ? 1.0 / 3.0 : (S == 4 && (i == 1 || i == 2)) ? 1.0 / 5.0 : 1.0;
  if (S == 3 && i == 0 && j == 2) return -1.0 / 3.0;
  if (S == 4 && j == i + 2) return -1.0 / 5.0;
  return 0.0;
}

constexpr double inv_factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= double(i);
  return 1.0 / f;
}

// phi_K(z) = sum_{j>=0} z^j / (j+K)! for 0 <= z < 4: 9 terms for z < 0.5 and 18
// otherwise (relative truncation error below 1e-7 for every K >= 1 either way)
template <int K, int NT, typename T>
BN_HD T phi_terms(T z) {
  T s = T(inv_factorial(NT - 1 + K));
#pragma unroll
  for (int j = NT - 2; j >= 0; --j) s = fma(s, z, T(inv_factorial(j + K)));
  return s;
}
template <int K, typename T>
BN_HD T phi_series(T z) {
  if (z < T(0.5)) return phi_terms<K, 9>(z);
  return phi_terms<K, 18>(z);
}

// Q block [o, o+S) of a Matern component (A's block must already be in A).
template <int S, int o, typename T, int D>
BN_HD void matern_noise(T var, T lam, T dt, const T (&A)[D][D], const T (&Pinf)[D][D], T (&Q)[D][D]) {
  const T x = lam * dt;
  if (x < T(2)) {
    constexpr int K = 2 * S - 1;
    const T e = exp(-x);
    const T ph = phi_series<K>(T(2) * x);
    T xk = x;
#pragma unroll
    for (int k = 1; k < K; ++k) xk *= x;
    T lp[2 * S - 1];
    lp[0] = var;
#pragma unroll
    for (int k = 1; k < 2 * S - 1; ++k) lp[k] = lp[k - 1] * lam;
    const T sc = e * e;
#pragma unroll
    for (int i = 0; i < S; ++i)
#pragma unroll
      for (int j = i; j < S; ++j) {
        T p = T(0);
#pragma unroll
        for (int n = 2 * S - 2; n >= 0; --n)
          p = (qc_matern(S, n, i, j) != 0.0) ? fma(p, x, T(qc_matern(S, n, i, j))) : p * x;
        if (pinf_matern(S, i, j) != 0.0) p = fma(T(pinf_matern(S, i, j) * double(1 << K)) * xk, ph, p);
        const T q = lp[i + j] * sc * p;
        Q[o + i][o + j] = q;
        Q[o + j][o + i] = q;
      }
  } else {
    process_noise_block<S, o>(A, Pinf, Q);
  }
}

// Transition and process noise of one Matern block of size S in T arithmetic,
// from (variance, lam): the kernels' own formulas, callable on the host too.
template <int S, typename T>
BN_HD void matern_block_aq(T var, T lam, T dt, T (&A)[S][S], T (&Q)[S][S]) {
  T Pinf[S][S];
  T lp[2 * S - 1];
  lp[0] = var;
  for (int k = 1; k < 2 * S - 1; ++k) lp[k] = lp[k - 1] * lam;
  for (int i = 0; i < S; ++i)
    for (int j = 0; j < S; ++j) Pinf[i][j] = lp[i + j] * T(pinf_matern(S, i, j));
  matern_transition<S>(lam, dt, A);
  matern_noise<S, 0>(var, lam, dt, A, Pinf, Q);
}

template <typename L, int c, typename T, int D, int P>
__device__ __forceinline__ void noise_comp(const SSM<T, D, P>& m, T dt, const T (&A)[D][D], T (&Q)[D][D]) {
  if constexpr (c < L::NC) {
    constexpr int o = L::off(c);
    constexpr int s = L::size(c);
    if constexpr (s <= 4) {
      if (m.kind[c] == BN_KIND_FEEDBACK) {
        process_noise_block<s, o>(A, m.Pinf, Q);
      } else {
        matern_noise<s, o>(m.var[c], m.lam[c], dt, A, m.Pinf, Q);
      }
    } else {
      process_noise_block<s, o>(A, m.Pinf, Q);
    }
    noise_comp<L, c + 1>(m, dt, A, Q);
  }
}

// Transition A(dt) and process noise Q(dt) of every block.  float32 Matern blocks
// take Q from the cancellation-free form above; float64 keeps the reference's
// Q = Pinf - A Pinf A^T (ops.py:149-151), exact to its own rounding.
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void transition_noise(const SSM<T, D, P>& m, T dt, T (&A)[D][D], T (&Q)[D][D]) {
  transition<L>(m, dt, A);
  if constexpr (std::is_same<T, float>::value) {
    set_zero(Q);
    noise_comp<L, 0>(m, dt, A, Q);
  } else {
    process_noise<L>(Q, A, m.Pinf);
  }
}

}  // namespace bn
