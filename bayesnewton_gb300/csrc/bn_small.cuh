// Small dense linear algebra held in registers, and the associative-scan element
// algebra of the Kalman filter and RTS smoother.
//
// Every routine is fully unrolled over compile-time sizes so matrices stay in
// registers.  Symmetric matrices are kept as full D x D arrays and symmetrised
// where a product is mathematically symmetric.
//
// Element conventions (Sarkka & Garcia-Fernandez 2021, "Temporal parallelization
// of Bayesian smoothers"; the reference restates them in bayesnewton/ops.py:183-229
// and :314-335):
//   filter element  (A, b, C, J, eta):  p(x_k | x_{s-1}, y_{s..k}) = N(A x_{s-1} + b, C)
//                                       p(y_{s..k} | x_{s-1}) ~ exp(-x'Jx/2 + eta'x)
//   smoother element (E, g, L):         p(x_k | x_{k+1}, y_{1..N}) = N(E x_{k+1} + g, L)
// The filter combine is written with W = (I + C1 J2)^-1 instead of the reference's
// inv(C1) (ops.py:208-209), so singular C1 (dt = 0, empty chunks) is handled.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define BN_HD __host__ __device__ __forceinline__

namespace bn {

template <typename T> BN_HD T bn_abs(T x) { return x < T(0) ? -x : x; }

// Reciprocal and reciprocal square root: hardware approximations in float32
// (relative error ~1 ulp), correctly rounded division / sqrt in float64.
__device__ __forceinline__ float bn_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double bn_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float bn_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double bn_rsqrt(double x) { return 1.0 / sqrt(x); }

// ---------------------------------------------------------------- matrices
template <typename T, int D>
BN_HD void set_identity(T (&M)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M[i][j] = (i == j) ? T(1) : T(0);
}

template <typename T, int D>
BN_HD void set_zero(T (&M)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M[i][j] = T(0);
}

template <typename T, int D>
BN_HD void set_zero(T (&v)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) v[i] = T(0);
}

template <typename T, int D>
BN_HD void copy(T (&O)[D][D], const T (&M)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) O[i][j] = M[i][j];
}

template <typename T, int D>
BN_HD void copy(T (&o)[D], const T (&v)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) o[i] = v[i];
}

// O = X Y
template <typename T, int D>
BN_HD void mm(T (&O)[D][D], const T (&X)[D][D], const T (&Y)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = X[i][0] * Y[0][j];
#pragma unroll
      for (int k = 1; k < D; ++k) s = fma(X[i][k], Y[k][j], s);
      O[i][j] = s;
    }
}

// O = X^T Y
template <typename T, int D>
BN_HD void mtm(T (&O)[D][D], const T (&X)[D][D], const T (&Y)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = X[0][i] * Y[0][j];
#pragma unroll
      for (int k = 1; k < D; ++k) s = fma(X[k][i], Y[k][j], s);
      O[i][j] = s;
    }
}

// O = X Y^T + Z, computed as a symmetric result (upper triangle mirrored).  Used
// only where X Y^T is symmetric in exact arithmetic.
template <typename T, int D>
BN_HD void mmt_sym_add(T (&O)[D][D], const T (&X)[D][D], const T (&Y)[D][D], const T (&Z)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Z[i][j];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[i][k], Y[j][k], s);
      O[i][j] = s;
      O[j][i] = s;
    }
}

// O = X^T Y + Z, symmetric result (X^T Y symmetric in exact arithmetic).
template <typename T, int D>
BN_HD void mtm_sym_add(T (&O)[D][D], const T (&X)[D][D], const T (&Y)[D][D], const T (&Z)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Z[i][j];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[k][i], Y[k][j], s);
      O[i][j] = s;
      O[j][i] = s;
    }
}

// o = X v
template <typename T, int D>
BN_HD void mv(T (&o)[D], const T (&X)[D][D], const T (&v)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = X[i][0] * v[0];
#pragma unroll
    for (int k = 1; k < D; ++k) s = fma(X[i][k], v[k], s);
    o[i] = s;
  }
}

// o = X v + a
template <typename T, int D>
BN_HD void mv_add(T (&o)[D], const T (&X)[D][D], const T (&v)[D], const T (&a)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = a[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(X[i][k], v[k], s);
    o[i] = s;
  }
}

// o = X^T v + a
template <typename T, int D>
BN_HD void mtv_add(T (&o)[D], const T (&X)[D][D], const T (&v)[D], const T (&a)[D]) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = a[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(X[k][i], v[k], s);
    o[i] = s;
  }
}

// Inverse by Gauss-Jordan elimination with partial pivoting.  Row exchanges are
// done with predicated swaps so every index stays compile-time (no local memory).
// M is overwritten.  Returns false when a pivot is exactly zero.
template <typename T, int D>
__device__ __forceinline__ bool inverse_gj(T (&M)[D][D], T (&X)[D][D]) {
  set_identity(X);
  bool ok = true;
#pragma unroll
  for (int k = 0; k < D; ++k) {
#pragma unroll
    for (int r = k + 1; r < D; ++r) {
      const bool sw = bn_abs(M[r][k]) > bn_abs(M[k][k]);
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const T a = M[k][c], bb = M[r][c];
        M[k][c] = sw ? bb : a;
        M[r][c] = sw ? a : bb;
        const T x = X[k][c], y = X[r][c];
        X[k][c] = sw ? y : x;
        X[r][c] = sw ? x : y;
      }
    }
    const T piv = M[k][k];
    ok = ok && (piv != T(0));
    const T ip = bn_rcp(piv);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      M[k][c] *= ip;
      X[k][c] *= ip;
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      if (r == k) continue;
      const T f = M[r][k];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        M[r][c] = fma(-f, M[k][c], M[r][c]);
        X[r][c] = fma(-f, X[k][c], X[r][c]);
      }
    }
  }
  return ok;
}

// In-place lower Cholesky factor of a symmetric positive-definite matrix; the
// diagonal holds the reciprocals of the factor's diagonal (what the solves use).
// Returns false when a pivot is not positive (the factor is then not usable).
template <typename T, int D>
__device__ __forceinline__ bool cholesky(T (&M)[D][D]) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    T s = M[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) s = fma(-M[j][k], M[j][k], s);
    ok = ok && (s > T(0));
    const T id = bn_rsqrt(s > T(0) ? s : T(1e-30));
    M[j][j] = id;
#pragma unroll
    for (int i = j + 1; i < D; ++i) {
      T t = M[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) t = fma(-M[i][k], M[j][k], t);
      M[i][j] = t * id;
    }
#pragma unroll
    for (int i = 0; i < j; ++i) M[i][j] = T(0);
  }
  return ok;
}

// X <- (L L^T)^-1 X for the factor from cholesky() (reciprocal diagonal).
template <typename T, int D>
__device__ __forceinline__ void chol_solve(const T (&L)[D][D], T (&X)[D][D]) {
#pragma unroll
  for (int c = 0; c < D; ++c) {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      T t = X[i][c];
#pragma unroll
      for (int k = 0; k < i; ++k) t = fma(-L[i][k], X[k][c], t);
      X[i][c] = t * L[i][i];
    }
#pragma unroll
    for (int i = D - 1; i >= 0; --i) {
      T t = X[i][c];
#pragma unroll
      for (int k = i + 1; k < D; ++k) t = fma(-L[k][i], X[k][c], t);
      X[i][c] = t * L[i][i];
    }
  }
}

// ---------------------------------------------------------------- elements
template <typename T, int D>
struct FElem {
  T A[D][D];
  T b[D];
  T C[D][D];
  T J[D][D];
  T eta[D];
};

template <typename T, int D>
struct SElem {
  T E[D][D];
  T g[D];
  T L[D][D];
};

template <typename T, int D>
struct State {
  T m[D];
  T P[D][D];
};

template <typename T, int D>
BN_HD void felem_identity(FElem<T, D>& e) {
  set_identity(e.A);
  set_zero(e.b);
  set_zero(e.C);
  set_zero(e.J);
  set_zero(e.eta);
}

template <typename T, int D>
BN_HD void selem_identity(SElem<T, D>& e) {
  set_identity(e.E);
  set_zero(e.g);
  set_zero(e.L);
}

// r = e1 (earlier) (+) e2 (later).  Returns false if I + C1 J2 was singular.
//   W   = (I + C1 J2)^-1
//   A   = A2 W A1
//   b   = A2 W (b1 + C1 eta2) + b2
//   C   = A2 W C1 A2^T + C2
//   eta = (W A1)^T (eta2 - J2 b1) + eta1
//   J   = (W A1)^T J2 A1 + J1
template <typename T, int D>
__device__ __forceinline__ bool fcombine(const FElem<T, D>& e1, const FElem<T, D>& e2, FElem<T, D>& r) {
  T M[D][D], W[D][D], X[D][D], Y[D][D];
  mm(M, e1.C, e2.J);
#pragma unroll
  for (int i = 0; i < D; ++i) M[i][i] += T(1);
  const bool ok = inverse_gj(M, W);
  mm(X, e2.A, W);            // A2 W
  // b
  T t[D], u[D];
  mv_add(t, e1.C, e2.eta, e1.b);
  mv_add(r.b, X, t, e2.b);
  // C
  mm(Y, X, e1.C);            // A2 W C1
  mmt_sym_add(r.C, Y, e2.A, e2.C);
  // A
  mm(r.A, X, e1.A);
  // eta, J
  mm(X, W, e1.A);            // W A1
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = e2.eta[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(-e2.J[i][k], e1.b[k], s);
    u[i] = s;
  }
  mtv_add(r.eta, X, u, e1.eta);
  mm(Y, e2.J, e1.A);         // J2 A1
  mtm_sym_add(r.J, X, Y, e1.J);
  return ok;
}

// Filtered state s (a prefix whose A is 0) followed by element e:
//   W = (I + P J)^-1, m' = A W (m + P eta) + b, P' = A W P A^T + C
template <typename T, int D>
__device__ __forceinline__ bool state_fcombine(const State<T, D>& s, const FElem<T, D>& e, State<T, D>& r) {
  T M[D][D], W[D][D], X[D][D], Y[D][D];
  mm(M, s.P, e.J);
#pragma unroll
  for (int i = 0; i < D; ++i) M[i][i] += T(1);
  const bool ok = inverse_gj(M, W);
  mm(X, e.A, W);
  T t[D];
  mv_add(t, s.P, e.eta, s.m);
  mv_add(r.m, X, t, e.b);
  mm(Y, X, s.P);
  mmt_sym_add(r.P, Y, e.A, e.C);
  return ok;
}

// r = e (earlier) o l (later): E = E_e E_l, g = E_e g_l + g_e, L = E_e L_l E_e^T + L_e
template <typename T, int D>
BN_HD void scompose(const SElem<T, D>& e, const SElem<T, D>& l, SElem<T, D>& r) {
  T Y[D][D];
  mv_add(r.g, e.E, l.g, e.g);
  mm(Y, e.E, l.L);
  mmt_sym_add(r.L, Y, e.E, e.L);
  mm(r.E, e.E, l.E);
}

// Smoothed state at time k from element k and the smoothed state at k+1.
template <typename T, int D>
BN_HD void selem_apply(const SElem<T, D>& e, const State<T, D>& s, State<T, D>& r) {
  T Y[D][D];
  mv_add(r.m, e.E, s.m, e.g);
  mm(Y, e.E, s.P);
  mmt_sym_add(r.P, Y, e.E, e.L);
}

}  // namespace bn
