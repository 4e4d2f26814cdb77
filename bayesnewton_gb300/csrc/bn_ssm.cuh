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
#include "bn_layout.h"
#include "bn_small.cuh"

namespace bn {

template <typename T, int D, int P>
struct SSM {
  int ncomp;
  int kind[BN_MAX_COMPONENTS];
  T lam[BN_MAX_COMPONENTS];  // sqrt(2 nu) / lengthscale (1/lengthscale for Matern12)
  T Pinf[D][D];
  T H[P][D];
  T F[D][D];                 // feedback matrix; read only for BN_KIND_FEEDBACK blocks
  T hph[P];                  // prior marginal variances diag(H Pinf H^T)
};

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
__device__ __forceinline__ void matern_transition(T lam, T dt, T (&B)[S][S]) {
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

}  // namespace bn
