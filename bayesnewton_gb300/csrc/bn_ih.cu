// Infinite-horizon Markov GP: the steady-state filter and smoother of
// bayesnewton's InfiniteHorizonGaussianProcess (basemodels.py:1257-1308) for
// equidistant time steps, with the site updates of the temporal model.
//
// Filter (ops.py:796-955): the Riccati recursion X <- A (X - K H X) A^T + Q,
// K = X H^T (H X H^T + R)^-1, run for dare_iters steps from a warm start (the
// previous call's solution, Pinf at first) with the tied noise R = mean(nat2)^-1
// (basemodels.py:1277-1292) gives Pdare; the filtered means then follow the affine
// recursion m_n = (A - K_n H A) m_{n-1} + K_n y_n from m = 0, with the tied gain
// K (homoscedastic: Gaussian likelihood, no missing data) or the per-site gain
// K_n = Pdare H^T (H Pdare H^T + R_n)^-1 (heteroscedastic), and the log marginal
// sum_n log N(y_n | H A m_{n-1}, S_n) over the observed sites.  The filtered
// covariance is the constant cov = Pdare - K H Pdare.
// Smoother (ops.py:957-1068): gain G = cov A^T Pdare^-1, Qdare = cov - G Pdare G^T,
// the Lyapunov recursion X <- G X G^T + Qdare from its own warm start gives the
// constant smoothed covariance; the means follow sm_n = G sm_{n+1} + (m_n - G A m_n)
// backwards from sm_N = m_{N-1}.
//
// Both mean recursions are affine, x_n = B_n x_{n-1} + v_n, so they run as one
// chunked scan: ih_reduce composes each thread's chunk of steps into (B, v) and
// scans a block's chunks in shared memory, ih_blocks walks the block aggregates
// from the initial state (one thread: only vectors are carried), ih_rerun replays
// each chunk from its exact entering state and emits the outputs.  The filter emits
// the means and the log marginal terms, the smoother the posterior marginals
// (H sm_n, H X H^T); a site-parallel kernel then takes the site expectations and
// energy sums of the temporal model's site tail.  Single-latent sites (P = 1).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>

#include "bn_engine.cuh"
#include "bn_host.h"

namespace bn {
namespace ih {

constexpr int kT = 128;  // threads per block of the chunk kernels
constexpr int kL = 32;   // steps per thread

// Constants of one call, float64 (written by the single-thread Riccati kernels).
template <int D>
struct Const {
  double A[D][D], H[D], HA[D];
  double Pdare[D][D], cov[D][D], PH[D], hPh, R, S, K[D], AKHA[D][D];
  double G[D][D], GA[D][D], X[D][D], covh;
  double hph;  // H Pinf H^T (float32 site clamp)
};

template <typename T, int D>
struct Elem {
  T B[D][D];
  T v[D];
};

template <typename T, int D>
__device__ __forceinline__ void elem_identity(Elem<T, D>& e) {
  set_identity(e.B);
  set_zero(e.v);
}
// first x then y: (By Bx, By vx + vy)
template <typename T, int D>
__device__ __forceinline__ void elem_then(const Elem<T, D>& x, const Elem<T, D>& y, Elem<T, D>& r) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = y.v[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(y.B[i][k], x.v[k], s);
    r.v[i] = s;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T t = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) t = fma(y.B[i][k], x.B[k][j], t);
      r.B[i][j] = t;
    }
  }
}

template <typename T, int D>
struct Args {
  const Const<D>* c;
  int64_t n;
  int nblocks;
  int hetero;
  int method;
  const T* y;      // [n] observations (NaN = missing)
  T* nat1;         // [n] sites
  T* nat2;
  T* fm;           // [n, D] filtered means (filter output, smoother input)
  T* post_mean;    // [n] posterior marginals
  T* post_var;
  T* grad;         // [n] site expectations at the posterior
  T* hess;
  T* lin;
  T* pref;         // [nblocks * kT] per-thread exclusive prefixes, field-major
  T* agg;          // [nblocks] block aggregates
  T* sin;          // [nblocks, D] states entering each block
  double* acc;     // accumulators (below)
  int* status;
  LikParams<T> lik;
  T lr;
};
// accumulator slots
enum { A_NAT2 = 0, A_LL = 1, A_S1 = 2, A_S2 = 3, A_D1 = 4, A_D2 = 5, A_N = 6 };

template <typename T, int D>
constexpr int elem_words() {
  return D * D + D;
}

template <typename T, int D>
__device__ __forceinline__ void store_elem(T* base, int64_t idx, int64_t stride, const Elem<T, D>& e) {
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) base[(size_t)(f++) * stride + idx] = e.B[i][j];
#pragma unroll
  for (int i = 0; i < D; ++i) base[(size_t)(f++) * stride + idx] = e.v[i];
}
template <typename T, int D>
__device__ __forceinline__ void load_elem(const T* base, int64_t idx, int64_t stride, Elem<T, D>& e) {
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) e.B[i][j] = base[(size_t)(f++) * stride + idx];
#pragma unroll
  for (int i = 0; i < D; ++i) e.v[i] = base[(size_t)(f++) * stride + idx];
}

// Site of step n as a pseudo observation (y = nat1 / nat2, R = 1 / nat2).
template <typename T, int D>
__device__ __forceinline__ void pseudo(const Args<T, D>& a, int64_t n, T& py, T& pr) {
  const T n2 = a.nat2[n];
  pr = T(1) / n2;
  py = a.nat1[n] * pr;
}

// Forward element of step n: B = A - K_n H A, v = K_n y_n.
template <typename T, int D>
__device__ __forceinline__ void filter_elem(const Args<T, D>& a, int64_t n, Elem<T, D>& e, T& S, T& py) {
  const Const<D>& c = *a.c;
  T pr;
  pseudo(a, n, py, pr);
  S = a.hetero ? T(c.hPh) + pr : T(c.S);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const T k = a.hetero ? T(c.PH[i]) / S : T(c.K[i]);
    e.v[i] = k * py;
#pragma unroll
    for (int j = 0; j < D; ++j) e.B[i][j] = a.hetero ? fma(-k, T(c.HA[j]), T(c.A[i][j])) : T(c.AKHA[i][j]);
  }
}

// Backward element of step n: B = G, v = m_n - G A m_n.  The recursion starts
// from sm_N = m_{N-1}, so the gain applies at the last step too, as in the
// reference (ops.py:978-993, 1003-1015).
template <typename T, int D>
__device__ __forceinline__ void smoother_elem(const Args<T, D>& a, int64_t n, Elem<T, D>& e) {
  const Const<D>& c = *a.c;
  T m[D];
#pragma unroll
  for (int i = 0; i < D; ++i) m[i] = a.fm[n * D + i];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = m[i];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      s = fma(-T(c.GA[i][k]), m[k], s);
      e.B[i][k] = T(c.G[i][k]);
    }
    e.v[i] = s;
  }
}

template <int TPB>
__device__ __forceinline__ void block_atomic(double v, double* red, double* dst) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < TPB / 32; ++w) s += red[w];
    atomicAdd(dst, s);
  }
  __syncthreads();
}

// ---------------------------------------------------------------- site update
// Damped Newton update of every site from the expectations cached at the
// posterior (inference.py:21-39, 83-86) and the update sizes.
template <typename T, int D>
__global__ void __launch_bounds__(256) site_update_kernel(Args<T, D> a) {
  __shared__ double red[8];
  double d1 = 0.0, d2 = 0.0;
  const T hph[1] = {T(a.c->hph)};
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += (int64_t)gridDim.x * blockDim.x) {
    const T g[1] = {a.grad[n]}, h[1][1] = {{a.hess[n]}}, m[1] = {a.lin[n]};
    const T o1[1] = {a.nat1[n]}, o2[1][1] = {{a.nat2[n]}};
    T n1[1], n2[1][1], e1, e2;
    site_nat_update<T, 1>(a.lr, hph, g, h, m, o1, o2, n1, n2, e1, e2, a.status);
    a.nat1[n] = n1[0];
    a.nat2[n] = n2[0][0];
    d1 += double(e1);
    d2 += double(e2);
  }
  block_atomic<256>(d1, red, a.acc + A_D1);
  block_atomic<256>(d2, red, a.acc + A_D2);
}

template <typename T, int D>
__global__ void __launch_bounds__(256) tied_kernel(Args<T, D> a) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += (int64_t)gridDim.x * blockDim.x)
    s += double(a.nat2[n]);
  block_atomic<256>(s, red, a.acc + A_NAT2);
}

// ---------------------------------------------------------------- Riccati
template <int D>
__device__ __forceinline__ void mat_mul(double (&O)[D][D], const double (&X)[D][D], const double (&Y)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[i][k], Y[k][j], s);
      O[i][j] = s;
    }
}
// O = X Y^T
template <int D>
__device__ __forceinline__ void mat_mul_t(double (&O)[D][D], const double (&X)[D][D], const double (&Y)[D][D]) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[i][k], Y[j][k], s);
      O[i][j] = s;
    }
}

// Warp-cooperative products on shared D x D arrays (entries over lanes):
// O = X Y (TY: O = X Y^T), then O += Z when Z is given.
template <int D, bool TY, typename R>
__device__ __forceinline__ void warp_mm(R (*O)[D], const R (*X)[D], const R (*Y)[D], const R (*Z)[D]) {
  for (int e = threadIdx.x; e < D * D; e += 32) {
    const int i = e / D, j = e % D;
    R s = Z ? Z[i][j] : R(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(X[i][k], TY ? Y[j][k] : Y[k][j], s);
    O[i][j] = s;
  }
  __syncwarp();
}

// Filter constants: the DARE from the warm start X0 (updated in place), then S,
// K, A - K H A and the filtered covariance (ops.py:796-821, 903-935).  One warp:
// the recursion's products run over the lanes.
template <typename L, typename R, int D, int P>
__global__ void __launch_bounds__(32) dare_filter_kernel(SSM<double, D, P> m, double dt, int iters, double* X0,
                                                         Const<D>* c, const double* acc, int64_t n) {
  // the recursion in the model's dtype R (float64 runs at 1/64 rate here), the
  // constants derived from its result in float64
  __shared__ R sA[D][D], sQ[D][D], sX[D][D], sT[D][D], sHX[D], sH[D];
  const int lane = threadIdx.x;
  if (lane == 0) {
    double A[D][D], Q[D][D];
    transition<L>(m, dt, A);
    process_noise<L>(Q, A, m.Pinf);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      sH[i] = R(m.H[0][i]);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        sA[i][j] = R(A[i][j]);
        sQ[i][j] = R(Q[i][j]);
      }
    }
  }
  for (int e = lane; e < D * D; e += 32) sX[e / D][e % D] = R(X0[e]);
  __syncwarp();
  const double Rt = double(n) / acc[A_NAT2];  // inv(mean(nat2))
  const R Rr = R(Rt);
  for (int it = 0; it < iters; ++it) {
    // HX, s = HX H^T + R, T = X - HX^T HX / s, X = A T A^T + Q
    if (lane < D) {
      R t = R(0);
#pragma unroll
      for (int k = 0; k < D; ++k) t = fma(sH[k], sX[k][lane], t);
      sHX[lane] = t;
    }
    __syncwarp();
    R sv = Rr;
#pragma unroll
    for (int j = 0; j < D; ++j) sv = fma(sHX[j], sH[j], sv);
    for (int e = lane; e < D * D; e += 32) {
      const int i = e / D, j = e % D;
      sT[i][j] = sX[i][j] - sHX[i] / sv * sHX[j];
    }
    __syncwarp();
    warp_mm<D, false, R>(sX, sA, sT, nullptr);  // A T
    warp_mm<D, true, R>(sT, sX, sA, sQ);         // (A T) A^T + Q
    for (int e = lane; e < D * D; e += 32) sX[e / D][e % D] = sT[e / D][e % D];
    __syncwarp();
  }
  for (int e = lane; e < D * D; e += 32) X0[e] = double(sX[e / D][e % D]);
  if (lane != 0) return;
  double X[D][D], A[D][D], H[D];
  transition<L>(m, dt, A);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    H[i] = m.H[0][i];
#pragma unroll
    for (int j = 0; j < D; ++j) X[i][j] = double(sX[i][j]);
  }
  double PH[D], hPh = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) t = fma(X[i][k], H[k], t);
    PH[i] = t;
  }
#pragma unroll
  for (int i = 0; i < D; ++i) hPh = fma(H[i], PH[i], hPh);
  const double S = hPh + Rt;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    c->H[i] = H[i];
    c->PH[i] = PH[i];
    c->K[i] = PH[i] / S;
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) t = fma(H[k], A[k][i], t);
    c->HA[i] = t;
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      c->A[i][j] = A[i][j];
      c->Pdare[i][j] = X[i][j];
      c->AKHA[i][j] = A[i][j] - c->K[i] * c->HA[j];
      c->cov[i][j] = X[i][j] - c->K[i] * PH[j];  // K H Pdare = K (Pdare H^T)^T
    }
  c->hPh = hPh;
  c->R = Rt;
  c->S = S;
  c->hph = m.hph[0];
}

// Smoother constants: G = cov A^T Pdare^-1, Qdare = cov - G Pdare G^T, the
// Lyapunov recursion from its warm start (ops.py:957-976, 1037-1068).  One warp.
template <typename R, int D>
__global__ void __launch_bounds__(32) dare_smoother_kernel(int iters, double* X0, Const<D>* c) {
  __shared__ R sG[D][D], sQ[D][D], sX[D][D], sT[D][D];
  const int lane = threadIdx.x;
  if (lane == 0) {
    double L[D][D], G[D][D], T1[D][D], Qd[D][D];
    // G^T = Pdare^-1 (A cov^T) = Pdare^-1 A cov
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) L[i][j] = c->Pdare[i][j];
    cholesky(L);
    mat_mul(T1, c->A, c->cov);
    chol_solve(L, T1);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) G[i][j] = T1[j][i];
    mat_mul(T1, G, c->Pdare);
    mat_mul_t(Qd, T1, G);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        sG[i][j] = R(G[i][j]);
        sQ[i][j] = R(c->cov[i][j] - Qd[i][j]);
      }
  }
  for (int e = lane; e < D * D; e += 32) sX[e / D][e % D] = R(X0[e]);
  __syncwarp();
  for (int it = 0; it < iters; ++it) {
    warp_mm<D, false, R>(sT, sG, sX, nullptr);  // G X
    warp_mm<D, true, R>(sX, sT, sG, sQ);        // (G X) G^T + Qdare
  }
  for (int e = lane; e < D * D; e += 32) X0[e] = double(sX[e / D][e % D]);
  if (lane != 0) return;
  double covh = 0.0, G[D][D], T1[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      G[i][j] = double(sG[i][j]);
      c->X[i][j] = double(sX[i][j]);
      c->G[i][j] = G[i][j];
      covh = fma(c->H[i] * double(sX[i][j]), c->H[j], covh);
    }
  mat_mul(T1, G, c->A);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) c->GA[i][j] = T1[i][j];
  c->covh = covh;
}

// ---------------------------------------------------------------- affine scan
// REV: the smoother's backward recursion (chunks and threads in reverse order).
template <typename T, int D, bool REV>
__device__ __forceinline__ void step_elem(const Args<T, D>& a, int64_t n, Elem<T, D>& e) {
  if constexpr (REV) {
    smoother_elem(a, n, e);
  } else {
    T S, py;
    filter_elem(a, n, e, S, py);
  }
}

template <typename T, int D, bool REV>
__global__ void __launch_bounds__(kT) reduce_kernel(Args<T, D> a) {
  __shared__ Elem<T, D> sm[kT];
  const int tid = threadIdx.x;
  const int64_t g = (int64_t)blockIdx.x * kT + tid;
  const int64_t s = g * kL;
  const int64_t e = s + kL < a.n ? s + kL : a.n;
  Elem<T, D> agg, t;
  elem_identity(agg);
  if constexpr (REV) {
    for (int64_t n = e - 1; n >= s; --n) {
      Elem<T, D> x;
      step_elem<T, D, REV>(a, n, x);
      elem_then(agg, x, t);
      agg = t;
    }
  } else {
    for (int64_t n = s; n < e; ++n) {
      Elem<T, D> x;
      step_elem<T, D, REV>(a, n, x);
      elem_then(agg, x, t);
      agg = t;
    }
  }
  // inclusive scan over the block's chunks in time order (REV: from the last thread)
  const int pos = REV ? kT - 1 - tid : tid;
  sm[pos] = agg;
  __syncthreads();
  for (int off = 1; off < kT; off <<= 1) {
    Elem<T, D> r;
    const bool act = pos >= off;
    if (act) elem_then(sm[pos - off], sm[pos], r);
    __syncthreads();
    if (act) sm[pos] = r;
    __syncthreads();
  }
  Elem<T, D> ex;
  if (pos == 0) elem_identity(ex);
  else ex = sm[pos - 1];
  store_elem(a.pref, g, (int64_t)a.nblocks * kT, ex);
  if (pos == kT - 1) store_elem(a.agg, blockIdx.x, a.nblocks, sm[pos]);
}

// The state entering each block, from the initial state (the filter: 0; the
// smoother: sm_N = m_{N-1}).  The block aggregates are staged through shared
// memory a tile at a time by all threads, and one thread walks them.
template <typename T, int D, bool REV>
__global__ void __launch_bounds__(256) blocks_kernel(Args<T, D> a) {
  constexpr int W = D * D + D;
  // aggregates per tile: at most 256 and 40 KB of static shared memory
  constexpr int TILE = 40960 / int(W * sizeof(T)) < 256 ? 40960 / int(W * sizeof(T)) : 256;
  __shared__ T tile[TILE * W];
  T st[D];  // the walking state, in thread 0's registers
#pragma unroll
  for (int d = 0; d < D; ++d) st[d] = REV ? a.fm[(a.n - 1) * D + d] : T(0);
  for (int t0 = 0; t0 < a.nblocks; t0 += TILE) {
    const int cnt = a.nblocks - t0 < TILE ? a.nblocks - t0 : TILE;
    __syncthreads();
    // tile slot i holds the i-th block in walking order
    for (int e = threadIdx.x; e < cnt * W; e += blockDim.x) {
      const int i = e / W, f = e % W;
      const int b = REV ? a.nblocks - 1 - (t0 + i) : t0 + i;
      tile[i * W + f] = a.agg[(size_t)f * a.nblocks + b];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < cnt; ++i) {
        const int b = REV ? a.nblocks - 1 - (t0 + i) : t0 + i;
        const T* x = tile + i * W;
        T nx[D];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          a.sin[b * D + r] = st[r];
          T v = x[D * D + r];
#pragma unroll
          for (int k = 0; k < D; ++k) v = fma(x[r * D + k], st[k], v);
          nx[r] = v;
        }
#pragma unroll
        for (int r = 0; r < D; ++r) st[r] = nx[r];
      }
    }
  }
}

// Replay each chunk from its entering state.  Filter: means and log marginal.
// Smoother: posterior marginals, site expectations, energy sums.
template <typename T, typename Lay, bool REV>
__global__ void __launch_bounds__(kT) rerun_kernel(Args<T, Lay::D> a) {
  constexpr int D = Lay::D;
  __shared__ double red[kT / 32];
  const int tid = threadIdx.x;
  const int64_t g = (int64_t)blockIdx.x * kT + tid;
  const int64_t s = g * kL;
  const int64_t e = s + kL < a.n ? s + kL : a.n;
  Elem<T, D> ex;
  load_elem(a.pref, g, (int64_t)a.nblocks * kT, ex);
  T st[D];
#pragma unroll
  for (int r = 0; r < D; ++r) {
    T v = ex.v[r];
#pragma unroll
    for (int k = 0; k < D; ++k) v = fma(ex.B[r][k], a.sin[blockIdx.x * D + k], v);
    st[r] = v;
  }
  const Const<D>& c = *a.c;
  KSum<T> ll, s1, s2;
  if constexpr (!REV) {
    for (int64_t n = s; n < e; ++n) {
      Elem<T, D> x;
      T S, py;
      filter_elem(a, n, x, S, py);
      // log N(y_n | H A m_{n-1}, S_n) over observed sites
      if (!bn_isnan(a.y[n])) {
        T mu = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) mu = fma(T(c.HA[k]), st[k], mu);
        const T r = py - mu;
        ll.add(T(-0.5) * (r * r / S + T(kLog2Pi) + log(S)));
      }
      T nx[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        T v = x.v[r];
#pragma unroll
        for (int k = 0; k < D; ++k) v = fma(x.B[r][k], st[k], v);
        nx[r] = v;
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        st[r] = nx[r];
        a.fm[n * D + r] = nx[r];
      }
    }
    block_atomic<kT>(ll.get(), red, a.acc + A_LL);
  } else {
    const T pv = T(c.covh);
    for (int64_t n = e - 1; n >= s; --n) {
      Elem<T, D> x;
      smoother_elem(a, n, x);
      T nx[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        T v = x.v[r];
#pragma unroll
        for (int k = 0; k < D; ++k) v = fma(x.B[r][k], st[k], v);
        nx[r] = v;
      }
      T f = T(0);
#pragma unroll
      for (int r = 0; r < D; ++r) {
        st[r] = nx[r];
        f = fma(T(c.H[r]), nx[r], f);
      }
      a.post_mean[n] = f;
      a.post_var[n] = pv;
    }
  }
}

// Site expectations at the posterior marginals and the energy sums: the temporal
// model's site tail (compiled for the method), one thread per site.
template <typename T, typename Lay, int MODE>
__global__ void __launch_bounds__(256) tail_kernel(Args<T, Lay::D> a) {
  constexpr int D = Lay::D;
  __shared__ double red[8];
  ScanArgs<T, D, 1> sa;
  memset(&sa, 0, sizeof(sa));
  sa.grad = a.grad;
  sa.hess = a.hess;
  sa.lin = a.lin;
  sa.status = a.status;
  const SiteLik<T> sl = site_lik(a.lik);
  const T pv[1][1] = {{T(a.c->covh)}};
  KSum<T> s1, s2;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.n; n += (int64_t)gridDim.x * blockDim.x) {
    const T pm[1] = {a.post_mean[n]};
    const T sn1[1] = {a.nat1[n]}, sn2[1][1] = {{a.nat2[n]}};
    site_tail<T, D, 1, MODE>(sa, a.lik, sl, n, pm, pv, a.y[n], sn1, sn2, s1, s2);
  }
  block_atomic<256>(s1.get(), red, a.acc + A_S1);
  block_atomic<256>(s2.get(), red, a.acc + A_S2);
}

// ---------------------------------------------------------------- host engine
struct Base {
  virtual ~Base() {}
  virtual int set_prior(const bn_prior_desc* d) = 0;
  virtual int set_lik(const bn_lik_desc* d) = 0;
  virtual int update_posterior(cudaStream_t st, double dt, int hetero, const void* y, const bn_site_state& s) = 0;
  virtual int site_update(cudaStream_t st, double lr, const bn_site_state& s) = 0;
  virtual int log_lik(cudaStream_t st, double dt, int hetero, const void* y, const bn_site_state& s) = 0;
  virtual int result(cudaStream_t st, double* out, int32_t* status) = 0;
  virtual int dare_state(cudaStream_t st, double* filter, double* smoother) = 0;
  int state_dim = 0;
};

template <typename T, typename Lay>
struct Engine : Base {
  static constexpr int D = Lay::D;
  int64_t n = 0;
  int nblocks = 0, iters = 20;
  SSM<double, D, 1> ssm;
  LikParams<T> lik;
  void* pool = nullptr;
  T *fm = nullptr, *pref = nullptr, *agg = nullptr, *sin = nullptr;
  double *acc = nullptr, *warm_f = nullptr, *warm_s = nullptr;
  Const<D>* cst = nullptr;
  int* status = nullptr;

  ~Engine() override {
    if (pool) cudaFree(pool);
  }

  int init(int64_t num, int dare_iters) {
    n = num;
    iters = dare_iters;
    state_dim = D;
    const int64_t chunks = (n + kL - 1) / kL;
    nblocks = int((chunks + kT - 1) / kT);
    const size_t w = size_t(elem_words<T, D>());
    const size_t sizes[4] = {size_t(n) * D, size_t(nblocks) * kT * w, size_t(nblocks) * w, size_t(nblocks) * D};
    size_t tot = 0;
    for (size_t s : sizes) tot += (s * sizeof(T) + 255) / 256 * 256;
    const size_t dbl = (size_t(A_N) + 2 * D * D) * sizeof(double);
    tot += (dbl + 255) / 256 * 256 + (sizeof(Const<D>) + 255) / 256 * 256 + 256;
    BN_CUDA_TRY(cudaMalloc(&pool, tot));
    BN_CUDA_TRY(cudaMemset(pool, 0, tot));
    char* p = static_cast<char*>(pool);
    T** ptrs[4] = {&fm, &pref, &agg, &sin};
    for (int i = 0; i < 4; ++i) {
      *ptrs[i] = reinterpret_cast<T*>(p);
      p += (sizes[i] * sizeof(T) + 255) / 256 * 256;
    }
    acc = reinterpret_cast<double*>(p);
    warm_f = acc + A_N;
    warm_s = warm_f + D * D;
    p += (dbl + 255) / 256 * 256;
    cst = reinterpret_cast<Const<D>*>(p);
    p += (sizeof(Const<D>) + 255) / 256 * 256;
    status = reinterpret_cast<int*>(p);
    return BN_OK;
  }

  bool warm = false;
  int set_prior(const bn_prior_desc* d) override {
    const int e = build_ssm<double, D, 1>(d, false, ssm);
    if (e != BN_OK) return e;
    // the Riccati recursions start from the first prior's Pinf (basemodels.py:1272-1275)
    // and keep their warm starts across later hyperparameter changes, as there
    if (warm) return BN_OK;
    warm = true;
    double h[2 * D * D];
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) h[i * D + j] = h[D * D + i * D + j] = ssm.Pinf[i][j];
    BN_CUDA_TRY(cudaMemcpy(warm_f, h, sizeof(h), cudaMemcpyHostToDevice));
    return BN_OK;
  }
  int set_lik(const bn_lik_desc* d) override {
    if (d->kind == BN_LIK_HETERO_EXP || d->kind == BN_LIK_HETERO_SOFTPLUS) return BN_ERR_UNSUPPORTED;
    return build_lik<T>(d, lik);
  }

  Args<T, D> args(const void* y, const bn_site_state& s) const {
    Args<T, D> a;
    std::memset(&a, 0, sizeof(a));
    a.c = cst;
    a.n = n;
    a.nblocks = nblocks;
    a.method = lik.method;
    a.y = static_cast<const T*>(y);
    a.nat1 = static_cast<T*>(s.nat1);
    a.nat2 = static_cast<T*>(s.nat2);
    a.fm = fm;
    a.post_mean = static_cast<T*>(s.post_mean);
    a.post_var = static_cast<T*>(s.post_var);
    a.grad = static_cast<T*>(s.grad);
    a.hess = static_cast<T*>(s.hess);
    a.lin = static_cast<T*>(s.lin);
    a.pref = pref;
    a.agg = agg;
    a.sin = sin;
    a.acc = acc;
    a.status = status;
    a.lik = lik;
    return a;
  }

  int filter(cudaStream_t st, double dt, Args<T, D>& a) {
    BN_CUDA_TRY(cudaMemsetAsync(acc + A_NAT2, 0, 2 * sizeof(double), st));  // nat2 sum, log marginal
    tied_kernel<T, D><<<152 * 4, 256, 0, st>>>(a);
    dare_filter_kernel<Lay, T, D, 1><<<1, 32, 0, st>>>(ssm, dt, iters, warm_f, cst, acc, n);
    reduce_kernel<T, D, false><<<nblocks, kT, 0, st>>>(a);
    blocks_kernel<T, D, false><<<1, 256, 0, st>>>(a);
    rerun_kernel<T, Lay, false><<<nblocks, kT, 0, st>>>(a);
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int update_posterior(cudaStream_t st, double dt, int hetero, const void* y, const bn_site_state& s) override {
    Args<T, D> a = args(y, s);
    a.hetero = hetero;
    BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    BN_CUDA_TRY(cudaMemsetAsync(acc + A_S1, 0, 2 * sizeof(double), st));
    int e = filter(st, dt, a);
    if (e != BN_OK) return e;
    dare_smoother_kernel<T, D><<<1, 32, 0, st>>>(iters, warm_s, cst);
    reduce_kernel<T, D, true><<<nblocks, kT, 0, st>>>(a);
    blocks_kernel<T, D, true><<<1, 256, 0, st>>>(a);
    rerun_kernel<T, Lay, true><<<nblocks, kT, 0, st>>>(a);
    int64_t nb = (n + 255) / 256;
    if (nb > 152 * 8) nb = 152 * 8;
    if (lik.method == BN_METHOD_VI) tail_kernel<T, Lay, 0><<<unsigned(nb), 256, 0, st>>>(a);
    else if (lik.method == BN_METHOD_NEWTON) tail_kernel<T, Lay, 1><<<unsigned(nb), 256, 0, st>>>(a);
    else tail_kernel<T, Lay, 2><<<unsigned(nb), 256, 0, st>>>(a);
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int site_update(cudaStream_t st, double lr, const bn_site_state& s) override {
    Args<T, D> a = args(nullptr, s);
    a.lr = T(lr);
    BN_CUDA_TRY(cudaMemsetAsync(acc + A_D1, 0, 2 * sizeof(double), st));
    int64_t nb = (n + 255) / 256;
    if (nb > 152 * 4) nb = 152 * 4;
    site_update_kernel<T, D><<<unsigned(nb), 256, 0, st>>>(a);
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int log_lik(cudaStream_t st, double dt, int hetero, const void* y, const bn_site_state& s) override {
    Args<T, D> a = args(y, s);
    a.hetero = hetero;
    return filter(st, dt, a);
  }

  int result(cudaStream_t st, double* out, int32_t* stat) override {
    double h[A_N];
    int s = 0;
    BN_CUDA_TRY(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaMemcpyAsync(&s, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < BN_NRESULT; ++i) out[i] = 0.0;
    const double ll = h[A_LL], s1 = h[A_S1], s2 = h[A_S2];
    out[BN_RES_LOGLIK] = ll;
    out[BN_RES_SUM1] = s1;
    out[BN_RES_SUM2] = s2;
    out[BN_RES_DIFF1] = h[A_D1];
    out[BN_RES_DIFF2] = h[A_D2];
    out[BN_RES_ENERGY] = (lik.method == BN_METHOD_EP || lik.method == BN_METHOD_PL)
                             ? -(ll + (s1 - s2) / double(lik.power))
                             : -(s1 - (s2 - ll));
    if (stat) *stat = s;
    return BN_OK;
  }

  int dare_state(cudaStream_t st, double* f, double* s) override {
    if (f) BN_CUDA_TRY(cudaMemcpyAsync(f, warm_f, D * D * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (s) BN_CUDA_TRY(cudaMemcpyAsync(s, warm_s, D * D * sizeof(double), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaStreamSynchronize(st));
    return BN_OK;
  }
};

template <typename T, typename Lay>
Base* make(int64_t n, int iters, int* err) {
  auto* e = new (std::nothrow) Engine<T, Lay>();
  if (!e) {
    *err = BN_ERR_ARG;
    return nullptr;
  }
  *err = e->init(n, iters);
  if (*err != BN_OK) {
    delete e;
    return nullptr;
  }
  return e;
}

template <int... Bs>
bool sizes_are(const bn_prior_desc* d) {
  constexpr int s[] = {Bs...};
  if (d->num_components != int(sizeof...(Bs))) return false;
  for (int c = 0; c < int(sizeof...(Bs)); ++c)
    if (d->size[c] != s[c] || d->kind[c] == BN_KIND_FEEDBACK) return false;
  return true;
}

Base* dispatch(const bn_prior_desc* d, int dtype, int64_t n, int iters, int* err) {
  if (d->combine != BN_COMBINE_SUM && d->num_components != 1) {
    *err = BN_ERR_UNSUPPORTED;
    return nullptr;
  }
#define BN_IH_TRY(T, ...)                                                                          \
  if (dtype == (sizeof(T) == 4 ? BN_DTYPE_F32 : BN_DTYPE_F64) && sizes_are<__VA_ARGS__>(d))        \
    return make<T, Layout<__VA_ARGS__>>(n, iters, err);
  BN_IH_TRY(float, 1)
  BN_IH_TRY(float, 2)
  BN_IH_TRY(float, 3)
  BN_IH_TRY(float, 4)
  BN_IH_TRY(float, 3, 2)
  BN_IH_TRY(double, 1)
  BN_IH_TRY(double, 2)
  BN_IH_TRY(double, 3)
  BN_IH_TRY(double, 3, 2)
#undef BN_IH_TRY
  *err = BN_ERR_UNSUPPORTED;
  return nullptr;
}

}  // namespace ih
}  // namespace bn

struct bn_ih_model {
  bn::ih::Base* eng;
};

extern "C" {

int bn_ih_create(const bn_prior_desc* prior, const bn_lik_desc* lik, int64_t num_data, int32_t dtype,
                 int32_t dare_iters, bn_ih_model** out) {
  if (!prior || !lik || !out || num_data < 1 || dare_iters < 0) return BN_ERR_ARG;
  if (prior->num_components < 1 || prior->num_components > BN_MAX_COMPONENTS) return BN_ERR_ARG;
  int err = BN_OK;
  bn::ih::Base* e = bn::ih::dispatch(prior, dtype, num_data, dare_iters, &err);
  if (!e) return err;
  if ((err = e->set_prior(prior)) != BN_OK || (err = e->set_lik(lik)) != BN_OK) {
    delete e;
    return err;
  }
  auto* m = new (std::nothrow) bn_ih_model;
  if (!m) {
    delete e;
    return BN_ERR_ARG;
  }
  m->eng = e;
  *out = m;
  return BN_OK;
}

int bn_ih_destroy(bn_ih_model* m) {
  if (!m) return BN_ERR_ARG;
  delete m->eng;
  delete m;
  return BN_OK;
}

int bn_ih_set_prior(bn_ih_model* m, const bn_prior_desc* prior) {
  if (!m || !prior) return BN_ERR_ARG;
  return m->eng->set_prior(prior);
}

int bn_ih_set_likelihood(bn_ih_model* m, const bn_lik_desc* lik) {
  if (!m || !lik) return BN_ERR_ARG;
  return m->eng->set_lik(lik);
}

int bn_ih_update_posterior(bn_ih_model* m, void* stream, double dt, int32_t heteroscedastic, const void* y,
                           const bn_site_state* s) {
  if (!m || !s || !y || !s->nat1 || !s->nat2 || !s->post_mean || !s->post_var || !s->grad || !s->hess || !s->lin)
    return BN_ERR_ARG;
  return m->eng->update_posterior(static_cast<cudaStream_t>(stream), dt, heteroscedastic, y, *s);
}

int bn_ih_site_update(bn_ih_model* m, void* stream, double lr, const bn_site_state* s) {
  if (!m || !s || !s->nat1 || !s->nat2 || !s->grad || !s->hess || !s->lin) return BN_ERR_ARG;
  return m->eng->site_update(static_cast<cudaStream_t>(stream), lr, *s);
}

int bn_ih_log_lik(bn_ih_model* m, void* stream, double dt, int32_t heteroscedastic, const void* y,
                  const bn_site_state* s) {
  if (!m || !s || !y || !s->nat1 || !s->nat2) return BN_ERR_ARG;
  return m->eng->log_lik(static_cast<cudaStream_t>(stream), dt, heteroscedastic, y, *s);
}

int bn_ih_result(bn_ih_model* m, void* stream, double* out, int32_t* status) {
  if (!m || !out) return BN_ERR_ARG;
  return m->eng->result(static_cast<cudaStream_t>(stream), out, status);
}

int bn_ih_dare_state(bn_ih_model* m, void* stream, double* filter, double* smoother) {
  if (!m) return BN_ERR_ARG;
  return m->eng->dare_state(static_cast<cudaStream_t>(stream), filter, smoother);
}

}  // extern "C"
