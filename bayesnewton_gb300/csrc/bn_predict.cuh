// Prediction at new times and the predictive densities.
//
//   conditional_kernel   the state at each test time given the smoothed states of
//                        its two neighbouring training times (bayesnewton/utils.py
//                        temporal_conditional :123-138, predict_from_state :99-118,
//                        compute_conditional_statistics :172-213)
//   log_density_kernel   log p(y*) = log E_N(f|m,v)[p(y*|f)] per test point and the
//                        sum / count behind the NLPD (likelihoods.py:385-388 ->
//                        cubature.py:249-276; Gaussian closed form :784-800;
//                        basemodels.py:177-193)
//   predict_y_kernel     data-space mean and variance (likelihoods.py:493-506 ->
//                        cubature.py:438-465; Gaussian :802-803)
//
// One thread per test point.  The conditional statistics are computed in float64
// whatever the model's dtype: Q_fwd = Pinf - A Pinf A^T cancels for short gaps and
// enters through Q_mp^-1, so float32 would lose most of its digits there; a test
// point costs a few thousand float64 FLOPs and two exponentials per prior block.
// Times stay float64 end to end (a test time is located among the training times
// by binary search in float64, as numpy.searchsorted does).
#pragma once
#include "bn_lik.cuh"
#include "bn_ssm.cuh"

namespace bn {

template <int D, int P>
struct CondArgs {
  SSM<double, D, P> ssm;
  int64_t n, nt;
  const double* x;    // [n] sorted training times
  const double* xt;   // [nt] test times (any order)
  const void* mean;   // [n, D] smoothed means (model dtype)
  const void* cov;    // [n, D, D] smoothed covariances
  const void* gain;   // [n, D, D] smoother gains
  void* out_m;        // [nt, R]
  void* out_P;        // [nt, R, R]
  int* status;
};

// Conditional statistics of one test time, block by block of the prior (every
// matrix below is block-diagonal): with A_f = A(t - x_k0), A_b = A(x_k1 - t),
//   Q_mp = Q_b + A_b Q_f A_b^T + 1e-8 I,  W = Q_f A_b^T Q_mp^-1,
//   M1 = A_f - W A_b A_f,  Tc = Q_f - W A_b Q_f,
// so that the state is N(M1 m0 + W m1, [M1 W] S [M1 W]^T + Tc) for the joint
// smoothed posterior S of the two neighbours.  A missing neighbour (before the
// first / after the last training time) is the reference's dummy state at -/+1e10,
// whose transition is exactly zero: A_f = 0 (resp. A_b = 0) and Q = Pinf.
template <typename L, int D, int P>
__device__ __forceinline__ bool cond_stats(const SSM<double, D, P>& m, bool ldum, bool rdum, double dtf, double dtb,
                                           double (&M1)[D][D], double (&W)[D][D], double (&Tc)[D][D]) {
  double Af[D][D], Ab[D][D], Qf[D][D], X[D][D], Qmp[D][D];
  if (ldum) set_zero(Af);
  else transition<L>(m, dtf, Af);
  if (rdum) set_zero(Ab);
  else transition<L>(m, dtb, Ab);
  process_noise<L>(Qf, Af, m.Pinf);
  process_noise<L>(Qmp, Ab, m.Pinf);  // Q_b
  mm_blk<L>(X, Ab, Qf);               // A_b Q_f
  mmt_blk_sym_add<L>(Qmp, X, Ab, Qmp);
#pragma unroll
  for (int i = 0; i < D; ++i) Qmp[i][i] += 1e-8;
  const bool ok = cholesky(Qmp);
  // V = Q_mp^-1 A_b (held in W until the transpose below)
  double V[D][D];
  copy(V, Ab);
  chol_solve(Qmp, V);
  // W = Q_f V^T
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
      if (L::lo(i) == L::lo(j)) {
#pragma unroll
        for (int k = L::lo(j); k < L::hi(j); ++k) s = fma(Qf[i][k], V[j][k], s);
      }
      W[i][j] = s;
    }
  // Tc = Q_f - W (A_b Q_f)
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = Qf[i][j];
      if (L::lo(i) == L::lo(j)) {
#pragma unroll
        for (int k = L::lo(j); k < L::hi(j); ++k) s = fma(-W[i][k], X[k][j], s);
      }
      Tc[i][j] = s;
    }
  // M1 = A_f - W (A_b A_f)
  mm_blk<L>(X, Ab, Af);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = Af[i][j];
      if (L::lo(i) == L::lo(j)) {
#pragma unroll
        for (int k = L::lo(j); k < L::hi(j); ++k) s = fma(-W[i][k], X[k][j], s);
      }
      M1[i][j] = s;
    }
  return ok;
}

template <typename T, int D>
__device__ __forceinline__ void load_mat(const T* p, double (&M)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M[i][j] = double(p[i * D + j]);
}

// R = P: outputs projected by H ([nt, P], [nt, P, P]); R = D: full states.
template <typename T, typename L, int P, int R>
__global__ void __launch_bounds__(128) conditional_kernel(CondArgs<L::D, P> c) {
  constexpr int D = L::D;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c.nt) return;
  const double t = c.xt[j];
  // number of training times below t (numpy.searchsorted, side='left')
  int64_t lo = 0, hi = c.n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (c.x[mid] < t) lo = mid + 1;
    else hi = mid;
  }
  const bool ldum = lo == 0, rdum = lo == c.n;
  const int64_t k0 = lo - 1, k1 = lo;
  const double dtf = ldum ? 0.0 : t - c.x[k0];
  const double dtb = rdum ? 0.0 : c.x[k1] - t;
  double U1[R][D], U2[R][D], HT[R][R];
  {
    double M1[D][D], W[D][D], Tc[D][D];
    if (!cond_stats<L>(c.ssm, ldum, rdum, dtf, dtb, M1, W, Tc)) atomicOr(c.status, BN_STATUS_NONPD);
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        if constexpr (R == D) {
          U1[r][k] = M1[r][k];
          U2[r][k] = W[r][k];
        } else {
          double s1 = 0.0, s2 = 0.0;
#pragma unroll
          for (int q = L::lo(k); q < L::hi(k); ++q) {
            s1 = fma(c.ssm.H[r][q], M1[q][k], s1);
            s2 = fma(c.ssm.H[r][q], W[q][k], s2);
          }
          U1[r][k] = s1;
          U2[r][k] = s2;
        }
      }
    // HT = Hsel Tc Hsel^T
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int s = 0; s < R; ++s) {
        if constexpr (R == D) {
          HT[r][s] = Tc[r][s];
        } else {
          double acc = 0.0;
#pragma unroll
          for (int a = 0; a < D; ++a) {
            double u = 0.0;
#pragma unroll
            for (int b = L::lo(a); b < L::hi(a); ++b) u = fma(Tc[a][b], c.ssm.H[s][b], u);
            acc = fma(c.ssm.H[r][a], u, acc);
          }
          HT[r][s] = acc;
        }
      }
  }
  const T* mean = static_cast<const T*>(c.mean);
  const T* cov = static_cast<const T*>(c.cov);
  const T* gain = static_cast<const T*>(c.gain);
  double om[R], oP[R][R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    om[r] = 0.0;
#pragma unroll
    for (int s = 0; s < R; ++s) oP[r][s] = HT[r][s];
  }
  if (!ldum) {
    // left neighbour: U1 m0 and U1 P0 U1^T
    double S[D][D];
    load_mat<T, D>(cov + (size_t)k0 * D * D, S);
#pragma unroll
    for (int r = 0; r < R; ++r) {
#pragma unroll
      for (int k = 0; k < D; ++k) om[r] = fma(U1[r][k], double(mean[k0 * D + k]), om[r]);
      double u[D];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < D; ++b) s = fma(S[a][b], U1[r][b], s);
        u[a] = s;
      }
#pragma unroll
      for (int q = 0; q < R; ++q) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) s = fma(U1[q][a], u[a], s);
        oP[q][r] += s;
      }
    }
  }
  if (!rdum) {
    // right neighbour: U2 m1; with Y = U1 G0 + U2 (the cross covariance is
    // G0 P1), U1 C U2^T + U2 C^T U1^T + U2 P1 U2^T = Y P1 Y^T - U1 G0 P1 G0^T U1^T;
    // written without that difference as Z P1 U2^T + U2 P1 Z^T + U2 P1 U2^T, Z = U1 G0
    double S[D][D], Z[R][D];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int k = 0; k < D; ++k) Z[r][k] = 0.0;
    if (!ldum) {
      load_mat<T, D>(gain + (size_t)k0 * D * D, S);
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < D; ++k) {
          double s = 0.0;
#pragma unroll
          for (int a = 0; a < D; ++a) s = fma(U1[r][a], S[a][k], s);
          Z[r][k] = s;
        }
    }
    load_mat<T, D>(cov + (size_t)k1 * D * D, S);
#pragma unroll
    for (int r = 0; r < R; ++r) {
#pragma unroll
      for (int k = 0; k < D; ++k) om[r] = fma(U2[r][k], double(mean[k1 * D + k]), om[r]);
      // v = P1 U2[r]^T
      double v[D];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < D; ++b) s = fma(S[a][b], U2[r][b], s);
        v[a] = s;
      }
#pragma unroll
      for (int q = 0; q < R; ++q) {
        double zu = 0.0, uu = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          zu = fma(Z[q][a], v[a], zu);
          uu = fma(U2[q][a], v[a], uu);
        }
        oP[q][r] += zu + uu;
        oP[r][q] += zu;
      }
    }
  }
  T* out_m = static_cast<T*>(c.out_m);
  T* out_P = static_cast<T*>(c.out_P);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    out_m[j * R + r] = T(om[r]);
#pragma unroll
    for (int s = 0; s < R; ++s) out_P[(j * R + r) * R + s] = T(0.5 * (oP[r][s] + oP[s][r]));
  }
}

// log p(y | m, v) by the likelihood's predictive rule (power 1), NaN for a
// missing y; the block sums of the finite values and their count go to acc[0..1].
template <typename T>
__global__ void __launch_bounds__(256) log_density_kernel(LikParams<T> lp, int64_t n, const T* y, const T* m,
                                                          const T* v, T* out, double* acc) {
  __shared__ double red[2][8];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0, c = 0.0;
  if (i < n) {
    const T yi = y[i];
    T lZ = T(NAN);
    if (yi == yi) {  // not NaN
      T d1, d2;
      mm1(lp, yi, m[i], v[i], lZ, d1, d2);
      s = double(lZ);
      c = 1.0;
    }
    if (out) out[i] = lZ;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s;
    red[1][w] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ts = 0.0, tc = 0.0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) {
      ts += red[0][k];
      tc += red[1][k];
    }
    atomicAdd(&acc[0], ts);
    atomicAdd(&acc[1], tc);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) predict_y_kernel(LikParams<T> lp, int64_t n, const T* m, const T* v, T* my,
                                                        T* vy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T mi = m[i], vi = v[i];
  if (lp.kind == BN_LIK_GAUSSIAN) {
    my[i] = mi;
    vy[i] = vi + lp.variance;
    return;
  }
  const T sv = sqrt(vi);
  T e1 = T(0), e2 = T(0);
  for (int q = 0; q < lp.ncub; ++q) {
    T ey, v2;
    cond_moments(lp, fma(sv, lp.cub_x[q], mi), ey, v2);
    e1 = fma(lp.cub_w[q], ey, e1);
    e2 = fma(lp.cub_w[q], v2 + ey * ey, e2);
  }
  my[i] = e1;
  vy[i] = e2 - e1 * e1;
}

}  // namespace bn
