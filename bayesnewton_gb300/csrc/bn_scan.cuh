// Chunked associative-scan Kalman filter and RTS smoother for small state
// dimensions (D <= 8), with the Newton site update and the site expectations /
// energy fused into the first and last passes.
//
// Work decomposition (one long series of N steps):
//   thread g of block b owns the chunk of steps [g L, g L + L);
//   F1  filter_reduce   : site update (fused step), chunk filter element by a
//                         sequential "conditioned on x_{s-1}" Kalman pass, block
//                         Kogge-Stone scan in shared memory -> per-thread exclusive
//                         prefix element and the block aggregate;
//   F2  filter_blocks   : one CTA scans the block aggregates -> filtered state
//                         entering each block;
//   F3  filter_rerun    : each thread enters its chunk with the exact filtered state,
//                         reruns the Kalman filter (writes filtered states, log
//                         marginal), composes its chunk smoother element on the fly,
//                         and a block reverse scan gives smoother suffixes;
//   S2  smoother_blocks : one CTA reverse-scans the smoother block aggregates;
//   S3  smoother_rerun  : each thread reruns the RTS smoother over its chunk from
//                         the exact smoothed state after it, writes the posterior
//                         marginals and evaluates the site tail (expectations,
//                         next Newton derivatives, energy partials).
// No kernel waits on another block: the cross-block dependency is carried by the
// kernel boundaries F1 -> F2 -> F3 -> S2 -> S3.
//
// The arithmetic is the reference's (bayesnewton/ops.py:154-380,
// basemodels.py:689-741, inference.py:21-222) reorganised into chunks.
#pragma once
#include <limits>
#include <type_traits>

#include "bn_lik.cuh"
#include "bn_small.cuh"
#include "bn_ssm.cuh"

namespace bn {

enum SiteMode { SITE_GIVEN = 0, SITE_NAT = 1, SITE_NEWTON = 2 };
enum StoreMode { STORE_INTERNAL = 0, STORE_REF = 1, STORE_NONE = 2, STORE_SEQ = 3, STORE_ELEM = 4 };

template <typename T, int D, int P>
struct ScanArgs {
  int64_t N;
  int L;
  int nblocks;
  int shift_dt;      // smoother: 1 = A_k uses dt[k+1] (model path), 0 = dt[k] (ops API)
  int return_predict;
  int return_full;   // ops smoother: write full states instead of H-projections
  int obs_dim;
  SSM<T, D, P> ssm;
  LikParams<T> lik;
  T lr;
  // inputs
  const T* dt;             // [N]
  const T* y;              // [N, obs_dim] observations (NaN = missing)
  const uint8_t* mask;     // [N, P] (ops filter) or null
  const T* site_y;         // [N, P]    ops-level sites
  const T* site_R;         // [N, P, P]
  const T* in_m;           // ops smoother: filter means [N, D]
  const T* in_P;           // ops smoother: filter covs  [N, D, D]
  // model state
  T* nat1;                 // [N, P]
  T* nat2;                 // [N, P, P] (full, symmetric)
  T* grad;                 // [N, P]     cached site derivatives
  T* hess;                 // [N, P, P]
  T* lin;                  // [N, P]     linearisation point of the cached derivatives
  T* post_mean;            // [N, P]
  T* post_var;             // [N, P, P]
  // ops-level outputs
  T* out_m;                // [N, D] or [N, P]
  T* out_P;                // [N, D, D] or [N, P, P]
  T* out_G;                // [N, D, D] gains (or null)
  // workspace
  T* fx;                   // per-thread exclusive filter prefix  [nblocks][FE][TPB]
  T* fagg;                 // [nblocks][FE]
  T* fin;                  // [nblocks][ST]
  T* fst;                  // filtered states, internal layout
  T* sx;                   // per-thread exclusive smoother suffix [nblocks][SE][TPB]
  T* sagg;                 // [nblocks][SE]
  T* sin;                  // [nblocks][ST]
  int staged;              // 1: F1 may stage its per-step streams with cp.async (16-B aligned)
  // batched series (BATCH kernels): series of each step and per-series parameters
  const int* sid;          // [N] series index of each step (non-decreasing)
  const T* ser_var;        // [S][ncomp] component variances
  const T* ser_ell;        // [S][ncomp] component lengthscales
  const int* ser_lik;      // [S] likelihood kind
  const T* ser_likvar;     // [S] Gaussian noise variance
  T* ll_step;              // [N] per-step log-marginal term (for per-series energies)
  const T* ser_gauss;      // [S][4] Gaussian series: var and 1 / var, each as a (head, tail) pair
                           // of T whose sum is the float64 value
  double* ser_energy;      // [S] per-series energy
  const T* ext;             // [N][6] site expectations (E, g1, g2, h11, h12, h22) of two-latent
                           // sites computed outside the tail (the learned surrogate), or null
  // time segments of one long series (one segment per rank; see bn_segment_step)
  const T* seg_left;       // filtered state entering the segment (State, flat) or null: prior
  const T* seg_right;      // smoothed state of the next segment's first step (State) or null
  T* seg_total_f;          // out: the segment's filter element total (FElem) or null
  T* seg_total_s;          // out: the segment's smoother element total (SElem) or null
  int seg_continue;        // the first step continues the previous segment (not a series start)
  int seg_more;            // another segment follows: the last step gets a full RTS element
  T dt_next;               // time step to the next segment's first step
  double* part;            // [nblocks][BN_NPART]
  double* tpart;           // [ntail_blocks][2] partial sums of the site-tail kernel
  int ntail_blocks;
  unsigned* counter;       // [2] last-block counters
  double* result;          // [BN_NRESULT]
  int* status;
};

template <typename T, int D>
struct Sz {
  static constexpr int FE = sizeof(FElem<T, D>) / sizeof(T);
  static constexpr int SE = sizeof(SElem<T, D>) / sizeof(T);
  static constexpr int ST = sizeof(State<T, D>) / sizeof(T);
  static constexpr int REC = D + D * (D + 1) / 2;  // filtered record: m, packed P
  static constexpr int RECE = D * D + D + D * (D + 1) / 2;  // smoother element: E, g, packed L
};

template <typename T> __device__ __forceinline__ bool bn_isnan(T x) { return x != x; }

// ------------------------------------------------------------ flat element I/O
template <typename T, typename E>
__device__ __forceinline__ void store_interleaved(T* base, const E& e, int tid, int tpb) {
  const T* s = reinterpret_cast<const T*>(&e);
  constexpr int n = sizeof(E) / sizeof(T);
#pragma unroll
  for (int f = 0; f < n; ++f) base[(size_t)f * tpb + tid] = s[f];
}

template <typename T, typename E>
__device__ __forceinline__ void load_interleaved(E& e, const T* base, int tid, int tpb) {
  T* d = reinterpret_cast<T*>(&e);
  constexpr int n = sizeof(E) / sizeof(T);
#pragma unroll
  for (int f = 0; f < n; ++f) d[f] = base[(size_t)f * tpb + tid];
}

template <typename T, typename E>
__device__ __forceinline__ void store_flat(T* dst, const E& e) {
  const T* s = reinterpret_cast<const T*>(&e);
  constexpr int n = sizeof(E) / sizeof(T);
#pragma unroll
  for (int f = 0; f < n; ++f) dst[f] = s[f];
}

template <typename T, typename E>
__device__ __forceinline__ void load_flat(E& e, const T* src) {
  T* d = reinterpret_cast<T*>(&e);
  constexpr int n = sizeof(E) / sizeof(T);
#pragma unroll
  for (int f = 0; f < n; ++f) d[f] = src[f];
}

// ------------------------------------------------------------ small P algebra
template <typename T, int P>
__device__ __forceinline__ bool inv_small(const T (&S)[P][P], T (&Si)[P][P], T& logdet) {
  if constexpr (P == 1) {
    Si[0][0] = T(1) / S[0][0];
    logdet = log(S[0][0]);
    return S[0][0] > T(0);
  } else {
    const T det = S[0][0] * S[1][1] - S[0][1] * S[1][0];
    const T id = T(1) / det;
    Si[0][0] = S[1][1] * id;
    Si[1][1] = S[0][0] * id;
    Si[0][1] = -S[0][1] * id;
    Si[1][0] = -S[1][0] * id;
    logdet = log(det);
    return det > T(0) && S[0][0] > T(0);
  }
}

// Gaussian log density of residual r under covariance S with masked components
// dropped (a masked component contributes exactly 0, utils.py:376-396).
template <typename T, int P>
__device__ __forceinline__ T masked_logpdf(const T (&r)[P], const T (&S)[P][P], const bool (&mk)[P]) {
  if constexpr (P == 1) {
    if (mk[0]) return T(0);
    return T(-0.5) * (r[0] * r[0] / S[0][0] + T(kLog2Pi) + log(S[0][0]));
  } else {
    if (mk[0] && mk[1]) return T(0);
    if (mk[0]) return T(-0.5) * (r[1] * r[1] / S[1][1] + T(kLog2Pi) + log(S[1][1]));
    if (mk[1]) return T(-0.5) * (r[0] * r[0] / S[0][0] + T(kLog2Pi) + log(S[0][0]));
    T Si[2][2], ld;
    inv_small<T, 2>(S, Si, ld);
    const T q = r[0] * (Si[0][0] * r[0] + Si[0][1] * r[1]) + r[1] * (Si[1][0] * r[0] + Si[1][1] * r[1]);
    return T(-0.5) * (q + T(2) * T(kLog2Pi) + ld);
  }
}

// Kahan-compensated accumulation in T, promoted to double at block level.
template <typename T>
struct KSum {
  T s = T(0), c = T(0);
  __device__ __forceinline__ void add(T x) {
    const T yv = x - c;
    const T t = s + yv;
    c = (t - s) - yv;
    s = t;
  }
  __device__ __forceinline__ double get() const { return double(s) - double(c); }
};

// ------------------------------------------------------------ model pieces
// Transition into step k.  A series starts from its stationary prior: A = 0
// there (so Q = Pinf), which also makes the previous step's smoother element
// (0, m, P) and its filter element independent of anything before the start.
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void step_transition(const SSM<T, D, P>& m, bool head, T dtk, T (&A)[D][D], T (&Q)[D][D]) {
  if (head) {
    set_zero(A);
    copy(Q, m.Pinf);
  } else {
    transition_noise<L>(m, dtk, A, Q);
  }
}

// Prior of each step.  FixedModel: one series, the kernel-parameter prior.
template <typename L, typename T, int P>
struct FixedModel {
  const SSM<T, L::D, P>& ss;
  int cont;  // the series started before step 0 (a continuing time segment)
  __device__ __forceinline__ const SSM<T, L::D, P>& at(int64_t k, bool& head) {
    head = (k == 0) && !cont;
    return ss;
  }
};

// Matern rate and stationary covariance of each component from per-series
// (variance, lengthscale) (kernels.py:139-145, 191-200, 249-265, 319-338).
template <typename L, int c, typename T, int D, int P>
__device__ __forceinline__ void set_series_params(SSM<T, D, P>& ss, const T* var, const T* ell) {
  if constexpr (c < L::NC) {
    constexpr int o = L::off(c);
    constexpr int sz = L::size(c);
    const T v = var[c], l = ell[c];
    const T il2 = T(1) / (l * l);
    ss.var[c] = v;
    if constexpr (sz == 1) {
      ss.lam[c] = T(1) / l;
      ss.Pinf[o][o] = v;
    } else if constexpr (sz == 2) {
      ss.lam[c] = sqrt(T(3)) / l;
      ss.Pinf[o][o] = v;
      ss.Pinf[o + 1][o + 1] = T(3) * v * il2;
    } else if constexpr (sz == 3) {
      const T kp = T(5) / T(3) * v * il2;
      ss.lam[c] = sqrt(T(5)) / l;
      ss.Pinf[o][o] = v;
      ss.Pinf[o][o + 2] = ss.Pinf[o + 2][o] = -kp;
      ss.Pinf[o + 1][o + 1] = kp;
      ss.Pinf[o + 2][o + 2] = T(25) * v * il2 * il2;
    } else if constexpr (sz == 4) {
      const T kp = T(7) / T(5) * v * il2, k2 = T(9.8) * v * il2 * il2;
      ss.lam[c] = sqrt(T(7)) / l;
      ss.Pinf[o][o] = v;
      ss.Pinf[o][o + 2] = ss.Pinf[o + 2][o] = -kp;
      ss.Pinf[o + 1][o + 1] = kp;
      ss.Pinf[o + 1][o + 3] = ss.Pinf[o + 3][o + 1] = -k2;
      ss.Pinf[o + 2][o + 2] = k2;
      ss.Pinf[o + 3][o + 3] = T(343) * v * il2 * il2 * il2;
    }
    if constexpr (c == 0) ss.hph[0] = v;  // single component: H = e_0
    set_series_params<L, c + 1>(ss, var, ell);
  }
}

// SeriesModel: many series concatenated; each step's prior is its series'.
template <typename L, typename T, int P>
struct SeriesModel {
  SSM<T, L::D, P> ss;
  const int* sid;
  const T* var;
  const T* ell;
  int cur, prev;
  __device__ __forceinline__ SeriesModel(const ScanArgs<T, L::D, P>& a, int64_t first)
      : ss(a.ssm), sid(a.sid), var(a.ser_var), ell(a.ser_ell), cur(-1) {
    // threads past the data (first >= N) construct one but never call at()
    prev = (first > 0 && first <= a.N) ? sid[first - 1] : -1;
  }
  __device__ __forceinline__ const SSM<T, L::D, P>& at(int64_t k, bool& head) {
    const int s = sid[k];
    head = (s != prev);
    prev = s;
    if (s != cur) {
      cur = s;
      set_series_params<L, 0>(ss, var + (size_t)s * L::NC, ell + (size_t)s * L::NC);
    }
    return ss;
  }
};

// Observation mask of step k for the filter log marginal.
template <typename T, int D, int P, int SITE>
__device__ __forceinline__ void step_mask(const ScanArgs<T, D, P>& a, int64_t k, bool (&mk)[P]) {
#pragma unroll
  for (int p = 0; p < P; ++p) mk[p] = false;
  if constexpr (SITE == SITE_GIVEN) {
    if (a.mask) {
#pragma unroll
      for (int p = 0; p < P; ++p) mk[p] = a.mask[k * P + p] != 0;
    }
  } else {
    // mask_pseudo_y = isnan(Y) for single-latent sites; none for multi-latent ones
    if (a.obs_dim == P) {
#pragma unroll
      for (int p = 0; p < P; ++p) mk[p] = bn_isnan(a.y[k * P + p]);
    }
  }
}

// Pseudo-observation (site mean y, site covariance R) of step k.
template <typename T, int D, int P, int SITE>
__device__ __forceinline__ void step_site(const ScanArgs<T, D, P>& a, int64_t k, T (&y)[P], T (&R)[P][P]) {
  if constexpr (SITE == SITE_GIVEN) {
#pragma unroll
    for (int p = 0; p < P; ++p) {
      y[p] = a.site_y[k * P + p];
#pragma unroll
      for (int q = 0; q < P; ++q) R[p][q] = a.site_R[(k * P + p) * P + q];
    }
  } else {
    T n1[P], n2[P][P], ld;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      n1[p] = a.nat1[k * P + p];
#pragma unroll
      for (int q = 0; q < P; ++q) n2[p][q] = a.nat2[(k * P + p) * P + q];
    }
    inv_small<T, P>(n2, R, ld);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) s = fma(R[p][q], n1[q], s);
      y[p] = s;
    }
  }
}

// Fused Newton site update of step k from the cached derivatives
// (newton_update + damping, inference.py:21-39, :75-86).  Returns |d nat1|, |d nat2|.
// New site natural parameters from the cached expectations (gradient g and
// Hessian h at the linearisation point m) and the old ones (o1, o2), damped by lr:
// nat1 = (1 - lr) o1 + lr (g - h m), nat2 = (1 - lr) o2 - lr h (the site update
// of inference.py:65-90).  A NaN derivative (a masked site) counts as g = h m,
// h = -1e-6.  Range guard: a site whose new parameters are not finite (e.g. a
// Poisson rate exp(m + v/2) beyond the type's range at a far overshooting mean)
// keeps its old parameters (BN_STATUS_SITE_KEPT); in float32 a site whose
// precision exceeds 1e6 times the prior precision hph^-1 is scaled back to that
// bound with its mean unchanged (BN_STATUS_SITE_CLAMPED), since the filter's
// covariance update P = Pp - Pp H^T S^-1 H Pp loses all digits of such a site's
// variance in float32 and can turn indefinite.
template <typename T, int P>
__device__ __forceinline__ void site_nat_update(T lr, const T (&hph)[P], const T (&gi)[P], const T (&hi)[P][P],
                                                const T (&m)[P], const T (&o1)[P], const T (&o2)[P][P], T (&n1)[P],
                                                T (&n2)[P][P], T& dn1, T& dn2, int* status) {
  T h[P][P];
#pragma unroll
  for (int p = 0; p < P; ++p)
#pragma unroll
    for (int q = 0; q < P; ++q) h[p][q] = bn_isnan(hi[p][q]) ? T(-1e-6) : hi[p][q];
  dn1 = T(0);
  dn2 = T(0);
  bool fin = true;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T hm = T(0);
#pragma unroll
    for (int q = 0; q < P; ++q) hm = fma(h[p][q], m[q], hm);
    const T gp = bn_isnan(gi[p]) ? hm : gi[p];
    const T nn = gp - hm;
    dn1 += bn_abs(nn - o1[p]);
    n1[p] = (T(1) - lr) * o1[p] + lr * nn;
    fin = fin && bn_abs(n1[p]) <= std::numeric_limits<T>::max();
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const T mm2 = -h[p][q];
      dn2 += bn_abs(mm2 - o2[p][q]);
      n2[p][q] = (T(1) - lr) * o2[p][q] + lr * mm2;
      fin = fin && bn_abs(n2[p][q]) <= std::numeric_limits<T>::max();
    }
  }
  if (!fin) {
    dn1 = T(0);
    dn2 = T(0);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      n1[p] = o1[p];
#pragma unroll
      for (int q = 0; q < P; ++q) n2[p][q] = o2[p][q];
    }
    atomicOr(status, BN_STATUS_SITE_KEPT);
  } else if constexpr (std::is_same<T, float>::value) {
    T sc = T(0);
#pragma unroll
    for (int p = 0; p < P; ++p) sc = fmaxf(sc, n2[p][p] * hph[p]);
    if (sc > T(1e6)) {
      const T f = T(1e6) / sc;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        n1[p] *= f;
#pragma unroll
        for (int q = 0; q < P; ++q) n2[p][q] *= f;
      }
      atomicOr(status, BN_STATUS_SITE_CLAMPED);
    }
  }
}

// Site update of step k in place (sequential form).
template <typename T, int D, int P>
__device__ __forceinline__ void site_newton_update(const ScanArgs<T, D, P>& a, int64_t k, T& dn1, T& dn2) {
  T g[P], h[P][P], m[P], o1[P], o2[P][P], n1[P], n2[P][P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    g[p] = a.grad[k * P + p];
    m[p] = a.lin[k * P + p];
    o1[p] = a.nat1[k * P + p];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      h[p][q] = a.hess[(k * P + p) * P + q];
      o2[p][q] = a.nat2[(k * P + p) * P + q];
    }
  }
  site_nat_update<T, P>(a.lr, a.ssm.hph, g, h, m, o1, o2, n1, n2, dn1, dn2, a.status);
#pragma unroll
  for (int p = 0; p < P; ++p) {
    a.nat1[k * P + p] = n1[p];
#pragma unroll
    for (int q = 0; q < P; ++q) a.nat2[(k * P + p) * P + q] = n2[p][q];
  }
}

// ------------------------------------------------------------ per-step inputs
// Loaded one step ahead in the chunk loops so that the loads of step k+1 are in
// flight while step k computes.
template <typename T, int P>
struct NewtonIn {
  T dt;
  T g[P], m[P], o1[P];
  T h[P][P], o2[P][P];
};

template <typename T, int D, int P>
__device__ __forceinline__ void load_newton(const ScanArgs<T, D, P>& a, int64_t k, NewtonIn<T, P>& x) {
  x.dt = a.dt[k];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    x.g[p] = a.grad[k * P + p];
    x.m[p] = a.lin[k * P + p];
    x.o1[p] = a.nat1[k * P + p];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      x.h[p][q] = a.hess[(k * P + p) * P + q];
      x.o2[p][q] = a.nat2[(k * P + p) * P + q];
    }
  }
}

// Newton update of one site from prefetched inputs: writes the new natural
// parameters and returns the pseudo-observation (y, R) they define.
template <typename T, int D, int P>
__device__ __forceinline__ void newton_site(const ScanArgs<T, D, P>& a, const T (&hph)[P], int64_t k,
                                            const NewtonIn<T, P>& x, T (&y)[P], T (&R)[P][P], T& dn1, T& dn2) {
  T n1[P], n2[P][P], ld;
  site_nat_update<T, P>(a.lr, hph, x.g, x.h, x.m, x.o1, x.o2, n1, n2, dn1, dn2, a.status);
#pragma unroll
  for (int p = 0; p < P; ++p) {
    a.nat1[k * P + p] = n1[p];
#pragma unroll
    for (int q = 0; q < P; ++q) a.nat2[(k * P + p) * P + q] = n2[p][q];
  }
  inv_small<T, P>(n2, R, ld);
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < P; ++q) t = fma(R[p][q], n1[q], t);
    y[p] = t;
  }
}

template <typename T, int P>
struct SiteIn {
  T dt;
  T n1[P], yo[P];
  T n2[P][P];
};

template <typename T, int D, int P, int SITE>
__device__ __forceinline__ void load_site_in(const ScanArgs<T, D, P>& a, int64_t k, SiteIn<T, P>& x) {
  x.dt = a.dt[k];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    if constexpr (SITE == SITE_GIVEN) {
      x.n1[p] = a.site_y[k * P + p];
      x.yo[p] = a.mask ? T(a.mask[k * P + p]) : T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) x.n2[p][q] = a.site_R[(k * P + p) * P + q];
    } else {
      x.n1[p] = a.nat1[k * P + p];
      x.yo[p] = (a.obs_dim == P) ? a.y[k * P + p] : T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) x.n2[p][q] = a.nat2[(k * P + p) * P + q];
    }
  }
}

// Pseudo-observation and log-marginal mask of a prefetched step.
template <typename T, int P, int SITE>
__device__ __forceinline__ void site_of(const SiteIn<T, P>& x, T (&y)[P], T (&R)[P][P], bool (&mk)[P]) {
  if constexpr (SITE == SITE_GIVEN) {
#pragma unroll
    for (int p = 0; p < P; ++p) {
      y[p] = x.n1[p];
      mk[p] = x.yo[p] != T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) R[p][q] = x.n2[p][q];
    }
  } else {
    T ld;
    inv_small<T, P>(x.n2, R, ld);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T t = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) t = fma(R[p][q], x.n1[q], t);
      y[p] = t;
      mk[p] = bn_isnan(x.yo[p]);
    }
  }
}

// One step of the chunk filter element: Kalman step conditioned on a known x_{s-1}.
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void felem_step(const SSM<T, D, P>& m, const T (&A)[D][D], const T (&Q)[D][D],
                                           const T (&y)[P], const T (&R)[P][P], FElem<T, D>& e) {
  T X[D][D], Cp[D][D];
  // predict: M <- A M, b <- A b, C <- A C A^T + Q
  mm_blk<L>(X, A, e.A);
  copy(e.A, X);
  T bp[D];
  mv_blk<L>(bp, A, e.b);
  mm_blk<L>(X, A, e.C);
  mmt_blk_sym_add<L>(Cp, X, A, Q);
  // innovation
  T HM[P][D], HC[P][D], Hb[P], S[P][P], Si[P][P], ld;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T hb = T(0);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s1 = T(0), s2 = T(0);
#pragma unroll
      for (int i = 0; i < D; ++i) {
        s1 = hacc<L, P>(m, p, i, e.A[i][j], s1);
        s2 = hacc<L, P>(m, p, i, Cp[i][j], s2);
      }
      HM[p][j] = s1;
      HC[p][j] = s2;
      hb = hacc<L, P>(m, p, j, bp[j], hb);
    }
    Hb[p] = hb;
  }
#pragma unroll
  for (int p = 0; p < P; ++p)
#pragma unroll
    for (int q = 0; q < P; ++q) {
      T s = R[p][q];
#pragma unroll
      for (int j = 0; j < D; ++j) s = hacc<L, P>(m, q, j, HC[p][j], s);
      S[p][q] = s;
    }
  inv_small<T, P>(S, Si, ld);
  T r[P], SiHM[P][D], SiHC[P][D], Sir[P];
#pragma unroll
  for (int p = 0; p < P; ++p) r[p] = y[p] - Hb[p];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < P; ++q) t = fma(Si[p][q], r[q], t);
    Sir[p] = t;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s1 = T(0), s2 = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) {
        s1 = fma(Si[p][q], HM[q][j], s1);
        s2 = fma(Si[p][q], HC[q][j], s2);
      }
      SiHM[p][j] = s1;
      SiHC[p][j] = s2;
    }
  }
  // information about x_{s-1}
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = e.eta[i];
#pragma unroll
    for (int p = 0; p < P; ++p) t = fma(HM[p][i], Sir[p], t);
    e.eta[i] = t;
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = e.J[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(HM[p][i], SiHM[p][j], s);
      e.J[i][j] = s;
      e.J[j][i] = s;
    }
  }
  // update: K = HC^T Si (K[i][p] = SiHC[p][i])
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = bp[i];
#pragma unroll
    for (int p = 0; p < P; ++p) t = fma(SiHC[p][i], r[p], t);
    e.b[i] = t;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = e.A[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-SiHC[p][i], HM[p][j], s);
      e.A[i][j] = s;
    }
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Cp[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-SiHC[p][i], HC[p][j], s);
      e.C[i][j] = s;
      e.C[j][i] = s;
    }
  }
}

// Predict the filtered state (m, P) at k-1 to k: mp = A m, Pp = A P A^T + Q
// (ops.py:149-170).  Returns the prediction and A P (the cross term the smoother
// gain needs).
template <typename L, typename T, int D>
__device__ __forceinline__ void predict(const T (&A)[D][D], const T (&Q)[D][D], const T (&m)[D], const T (&Pm)[D][D],
                                        T (&mp)[D], T (&Pp)[D][D], T (&AP)[D][D]) {
  mv_blk<L>(mp, A, m);
  mm_blk<L>(AP, A, Pm);
  mmt_blk_sym_add<L>(Pp, AP, A, Q);
}

// Smoother element of step k from its filtered state (fm, fP) and the prediction
// to k+1 (mp, Pp, AP = A fP):  G = fP A^T Pp^-1, g = fm - G mp, L = fP - G A fP.
// Returns false if Pp was not positive definite.
template <typename T, int D>
__device__ __forceinline__ bool smoother_element(const T (&fm)[D], const T (&fP)[D][D], const T (&mp)[D],
                                                 const T (&Pp)[D][D], const T (&AP)[D][D], SElem<T, D>& e) {
  T Lc[D][D], Gt[D][D];
  copy(Lc, Pp);
  const bool ok = cholesky(Lc);
  copy(Gt, AP);
  chol_solve(Lc, Gt);   // Gt = Pp^-1 A fP = G^T
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = fm[i];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      e.E[i][j] = Gt[j][i];
      t = fma(-Gt[j][i], mp[j], t);
    }
    e.g[i] = t;
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = fP[i][j];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(-Gt[k][i], AP[k][j], s);
      e.L[i][j] = s;
      e.L[j][i] = s;
    }
  return ok;
}

// Kalman update of the prediction (mp, Pp) with pseudo-observation (y, R).
// Writes the filtered state and the innovation quantities for the log marginal.
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void kf_update(const SSM<T, D, P>& mdl, const T (&mp)[D], const T (&Pp)[D][D], const T (&y)[P],
                                          const T (&R)[P][P], T (&m)[D], T (&Pm)[D][D], T (&r)[P], T (&S)[P][P]) {
  T HP[P][D], Si[P][P], SiHP[P][D], ld;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T hm = T(0);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int i = 0; i < D; ++i) s = hacc<L, P>(mdl, p, i, Pp[i][j], s);
      HP[p][j] = s;
      hm = hacc<L, P>(mdl, p, j, mp[j], hm);
    }
    r[p] = y[p] - hm;
  }
#pragma unroll
  for (int p = 0; p < P; ++p)
#pragma unroll
    for (int q = 0; q < P; ++q) {
      T s = R[p][q];
#pragma unroll
      for (int j = 0; j < D; ++j) s = hacc<L, P>(mdl, q, j, HP[p][j], s);
      S[p][q] = s;
    }
  inv_small<T, P>(S, Si, ld);
  T Sir[P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < P; ++q) t = fma(Si[p][q], r[q], t);
    Sir[p] = t;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) s = fma(Si[p][q], HP[q][j], s);
      SiHP[p][j] = s;
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = mp[i];
#pragma unroll
    for (int p = 0; p < P; ++p) t = fma(HP[p][i], Sir[p], t);
    m[i] = t;
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Pp[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-HP[p][i], SiHP[p][j], s);
      Pm[i][j] = s;
      Pm[j][i] = s;
    }
  }
}

// Kalman update that also returns H Pp and S^-1 (the fixed-point smoother of the
// chunk aggregate reuses them).
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void kf_update_x(const SSM<T, D, P>& mdl, const T (&mp)[D], const T (&Pp)[D][D], const T (&y)[P],
                                            const T (&R)[P][P], T (&m)[D], T (&Pm)[D][D], T (&r)[P], T (&S)[P][P],
                                            T (&HP)[P][D], T (&Si)[P][P]) {
  T SiHP[P][D], ld;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T hm = T(0);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int i = 0; i < D; ++i) s = hacc<L, P>(mdl, p, i, Pp[i][j], s);
      HP[p][j] = s;
      hm = hacc<L, P>(mdl, p, j, mp[j], hm);
    }
    r[p] = y[p] - hm;
  }
#pragma unroll
  for (int p = 0; p < P; ++p)
#pragma unroll
    for (int q = 0; q < P; ++q) {
      T s = R[p][q];
#pragma unroll
      for (int j = 0; j < D; ++j) s = hacc<L, P>(mdl, q, j, HP[p][j], s);
      S[p][q] = s;
    }
  inv_small<T, P>(S, Si, ld);
  T Sir[P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < P; ++q) t = fma(Si[p][q], r[q], t);
    Sir[p] = t;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) s = fma(Si[p][q], HP[q][j], s);
      SiHP[p][j] = s;
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = mp[i];
#pragma unroll
    for (int p = 0; p < P; ++p) t = fma(HP[p][i], Sir[p], t);
    m[i] = t;
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Pp[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-HP[p][i], SiHP[p][j], s);
      Pm[i][j] = s;
      Pm[j][i] = s;
    }
  }
}

// Fixed-point smoother of the chunk's first state x_s, advanced by one Kalman
// step k > s: with X = Cov(x_s, x_{k-1} | y_{s..k-1}) predicted to X A_k^T and
// c = X^- H^T,  mu += c S^-1 r,  Sig -= c S^-1 c^T,  X = X^- - c S^-1 H Pp.
// At the chunk end the aggregate of the RTS elements over [s, e) follows from the
// joint Gaussian of (x_s, x_e): E = C Pp_e^-1, g = mu - E mp_e, L = Sig - E C^T
// with C = X A_e^T -- the same (E, g, L) as composing the per-step elements.
template <typename L, typename T, int D, int P>
__device__ __forceinline__ void fixed_point_step(const SSM<T, D, P>& mdl, const T (&A)[D][D], const T (&r)[P],
                                                 const T (&Si)[P][P], const T (&HP)[P][D], T (&mu)[D], T (&Sig)[D][D],
                                                 T (&X)[D][D]) {
  T Xm[D][D];
  // Xm = X A^T  (A block-diagonal)
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int q = L::lo(j); q < L::hi(j); ++q) s = fma(X[i][q], A[j][q], s);
      Xm[i][j] = s;
    }
  T c[D][P], cS[D][P];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T s = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) s = hacc<L, P>(mdl, p, j, Xm[i][j], s);
      c[i][p] = s;
    }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) s = fma(c[i][q], Si[q][p], s);
      cS[i][p] = s;
    }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T t = mu[i];
#pragma unroll
    for (int p = 0; p < P; ++p) t = fma(cS[i][p], r[p], t);
    mu[i] = t;
#pragma unroll
    for (int j = i; j < D; ++j) {
      T s = Sig[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-cS[i][p], c[j][p], s);
      Sig[i][j] = s;
      Sig[j][i] = s;
    }
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = Xm[i][j];
#pragma unroll
      for (int p = 0; p < P; ++p) s = fma(-cS[i][p], HP[p][j], s);
      X[i][j] = s;
    }
  }
}

// ------------------------------------------------------------ filtered-state records
// Internal layout: warp-interleaved records so a warp's 32 lanes touch one
// contiguous 32-word line per field: ((warp * L + kk) * REC + f) * 32 + lane.
template <typename T, int D, int RECSZ = Sz<T, D>::REC>
__device__ __forceinline__ size_t rec_index(int64_t g, int kk, int L, int f) {
  const int64_t w = g >> 5;
  const int lane = int(g & 31);
  return ((size_t)(w * L + kk) * RECSZ + f) * 32 + lane;
}

// Smoother element of one step in the same warp-interleaved order.
template <typename T, int D>
__device__ __forceinline__ void store_elem(T* base, int64_t g, int kk, int L, const SElem<T, D>& e) {
  constexpr int R = Sz<T, D>::RECE;
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) base[rec_index<T, D, R>(g, kk, L, f++)] = e.E[i][j];
#pragma unroll
  for (int i = 0; i < D; ++i) base[rec_index<T, D, R>(g, kk, L, f++)] = e.g[i];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) base[rec_index<T, D, R>(g, kk, L, f++)] = e.L[i][j];
}

template <typename T, int D>
__device__ __forceinline__ void load_elem(const T* base, int64_t g, int kk, int L, SElem<T, D>& e) {
  constexpr int R = Sz<T, D>::RECE;
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) e.E[i][j] = base[rec_index<T, D, R>(g, kk, L, f++)];
#pragma unroll
  for (int i = 0; i < D; ++i) e.g[i] = base[rec_index<T, D, R>(g, kk, L, f++)];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      const T v = base[rec_index<T, D, R>(g, kk, L, f++)];
      e.L[i][j] = v;
      e.L[j][i] = v;
    }
}

template <typename T, int D>
__device__ __forceinline__ void store_rec(T* base, int64_t g, int kk, int L, const T (&m)[D], const T (&Pm)[D][D]) {
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) base[rec_index<T, D>(g, kk, L, f++)] = m[i];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) base[rec_index<T, D>(g, kk, L, f++)] = Pm[i][j];
}

template <typename T, int D>
__device__ __forceinline__ void load_rec(const T* base, int64_t g, int kk, int L, T (&m)[D], T (&Pm)[D][D]) {
  int f = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) m[i] = base[rec_index<T, D>(g, kk, L, f++)];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      const T v = base[rec_index<T, D>(g, kk, L, f++)];
      Pm[i][j] = v;
      Pm[j][i] = v;
    }
}

// ------------------------------------------------------------ block scans
template <typename T, int D, int TPB>
__device__ __forceinline__ void block_scan_filter(FElem<T, D>* sm, int tid, int* status) {
  for (int off = 1; off < TPB; off <<= 1) {
    FElem<T, D> r;
    const bool act = tid >= off;
    bool ok = true;
    if (act) ok = fcombine(sm[tid - off], sm[tid], r);
    __syncthreads();
    if (act) sm[tid] = r;
    if (!ok) atomicOr(status, BN_STATUS_SINGULAR);
    __syncthreads();
  }
}

template <typename T, int D, int TPB>
__device__ __forceinline__ void block_rscan_smoother(SElem<T, D>* sm, int tid) {
  for (int off = 1; off < TPB; off <<= 1) {
    SElem<T, D> r;
    const bool act = tid + off < TPB;
    if (act) scompose(sm[tid], sm[tid + off], r);
    __syncthreads();
    if (act) sm[tid] = r;
    __syncthreads();
  }
}

// Block sum of per-thread doubles into part[blk * BN_NPART + slot].
template <int TPB>
__device__ __forceinline__ void block_sum_store(double v, double* red, double* dst, int tid) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < TPB / 32; ++w) s += red[w];
    *dst = s;
  }
  __syncthreads();
}

// Column sums of per-block partials (row stride `stride`) by all threads of the
// block that finished last; every thread gets the sums.  Loads go to L2 (__ldcg):
// the rows were written by other blocks.
template <int TPB, int NQ>
__device__ __forceinline__ void sum_partials(const double* part, int stride, int nb, const int (&cols)[NQ],
                                             double (&out)[NQ], double* red, int tid) {
  double v[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = 0.0;
  for (int b = tid; b < nb; b += TPB) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] += __ldcg(part + (size_t)b * stride + cols[q]);
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = x;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < TPB / 32; ++w) t += red[w];
    out[q] = t;
  }
  __syncthreads();
}

// ------------------------------------------------------------ cp.async staging
// F1's per-step input streams (dt, g, h, lin, nat1, nat2 for one scalar site) are
// staged through shared memory in sub-tiles of kSub steps, double buffered: each
// thread copies its own 32-byte slice of each stream with two 16-byte cp.async
// (zero-filled past N), so the loads of sub-tile j+1 overlap the work on j.  Slot
// v of thread t is stored at 16-byte position v ^ ((t >> 2) & 1), which keeps the
// 128-bit reads of a quarter warp on distinct banks.
constexpr int kSub = 8;
constexpr int kNStream = 6;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int bytes) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// buffer layout: [stage][stream][thread][2 x float4]
template <int TPB>
__device__ __forceinline__ float4* stage_slot(float* buf, int stage, int stream, int tid, int v) {
  return reinterpret_cast<float4*>(buf) + ((size_t(stage) * kNStream + stream) * TPB + tid) * 2 + (v ^ ((tid >> 2) & 1));
}

template <int TPB, typename Args>
__device__ __forceinline__ void stage_issue(const Args& a, float* buf, int stage, int tid, int64_t k0) {
  const float* src[kNStream] = {a.dt, a.grad, a.hess, a.lin, a.nat1, a.nat2};
#pragma unroll
  for (int st = 0; st < kNStream; ++st)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int64_t i0 = k0 + 4 * v;
      const int64_t left = a.N - i0;
      const int bytes = left >= 4 ? 16 : (left > 0 ? int(left) * 4 : 0);
      cp_async16(stage_slot<TPB>(buf, stage, st, tid, v), bytes > 0 ? src[st] + i0 : src[st], bytes);
    }
}

// ============================================================ F1
template <typename T, typename L, int P, int SITE, int TPB, bool BATCH = false>
__global__ void __launch_bounds__(TPB) filter_reduce_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FElem<T, D>* sm = reinterpret_cast<FElem<T, D>*>(smem_raw);
  __shared__ double red[TPB / 32];
  const int tid = threadIdx.x;
  const int blk = blockIdx.x;
  const int64_t g = (int64_t)blk * TPB + tid;
  const int64_t s = g * a.L;
  const int64_t e = s + a.L < a.N ? s + a.L : a.N;
  FElem<T, D> E;
  felem_identity(E);
  KSum<T> d1, d2;
  constexpr bool kStageable = std::is_same<T, float>::value && P == 1 && SITE == SITE_NEWTON && !BATCH;
  if (kStageable && a.staged) {
    if constexpr (kStageable) {
      float* buf = reinterpret_cast<float*>(smem_raw);
      const int nsub = (a.L + kSub - 1) / kSub;
      stage_issue<TPB>(a, buf, 0, tid, s);
      cp_async_commit();
      if (nsub > 1) stage_issue<TPB>(a, buf, 1, tid, s + kSub);
      cp_async_commit();
      for (int j = 0; j < nsub; ++j) {
        cp_async_wait<1>();
        const int stg = j & 1;
        // one copy of the step's code (not unrolled over the sub-tile) keeps the
        // kernel small for the instruction cache
#pragma unroll 1
        for (int h4 = 0; h4 < 2; ++h4) {
          float4 q[kNStream];
#pragma unroll
          for (int st = 0; st < kNStream; ++st) q[st] = *stage_slot<TPB>(buf, stg, st, tid, h4);
#pragma unroll 1
          for (int i = 0; i < 4; ++i) {
            const int64_t k = s + int64_t(j) * kSub + 4 * h4 + i;
            if (k < e) {
              auto pick = [&](const float4& f) { return i == 0 ? f.x : (i == 1 ? f.y : (i == 2 ? f.z : f.w)); };
              NewtonIn<T, P> x;
              x.dt = pick(q[0]);
              x.g[0] = pick(q[1]);
              x.h[0][0] = pick(q[2]);
              x.m[0] = pick(q[3]);
              x.o1[0] = pick(q[4]);
              x.o2[0][0] = pick(q[5]);
              T y[P], R[P][P], A[D][D], x1, x2;
              newton_site(a, a.ssm.hph, k, x, y, R, x1, x2);
              d1.add(x1);
              d2.add(x2);
              T Q[D][D];
              step_transition<L>(a.ssm, k == 0 && !a.seg_continue, x.dt, A, Q);
              felem_step<L>(a.ssm, A, Q, y, R, E);
            }
          }
        }
        if (j + 2 < nsub) stage_issue<TPB>(a, buf, stg, tid, s + int64_t(j + 2) * kSub);
        cp_async_commit();
      }
      cp_async_wait<0>();
      __syncthreads();  // the block scan reuses the staging buffer
    }
  } else {
    auto chunk = [&](auto& mdl) {
      if constexpr (SITE == SITE_NEWTON) {
        NewtonIn<T, P> cur, nxt;
        if (s < e) load_newton(a, s, cur);
        for (int64_t k = s; k < e; ++k) {
          if (k + 1 < e) load_newton(a, k + 1, nxt);
          T y[P], R[P][P], A[D][D], x1, x2;
          bool head;
          const auto& ss = mdl.at(k, head);
          newton_site(a, ss.hph, k, cur, y, R, x1, x2);
          d1.add(x1);
          d2.add(x2);
          T Q[D][D];
          step_transition<L>(ss, head, cur.dt, A, Q);
          felem_step<L>(ss, A, Q, y, R, E);
          cur = nxt;
        }
      } else {
        SiteIn<T, P> cur, nxt;
        if (s < e) load_site_in<T, D, P, SITE>(a, s, cur);
        for (int64_t k = s; k < e; ++k) {
          if (k + 1 < e) load_site_in<T, D, P, SITE>(a, k + 1, nxt);
          T y[P], R[P][P], A[D][D];
          bool mk[P];
          site_of<T, P, SITE>(cur, y, R, mk);
          bool head;
          const auto& ss = mdl.at(k, head);
          T Q[D][D];
          step_transition<L>(ss, head, cur.dt, A, Q);
          felem_step<L>(ss, A, Q, y, R, E);
          cur = nxt;
        }
      }
    };
    if constexpr (BATCH) {
      SeriesModel<L, T, P> mdl(a, s);
      chunk(mdl);
    } else {
      FixedModel<L, T, P> mdl{a.ssm, a.seg_continue};
      chunk(mdl);
    }
  }
  sm[tid] = E;
  __syncthreads();
  block_scan_filter<T, D, TPB>(sm, tid, a.status);
  // per-thread exclusive prefix (slot 0 is never read)
  if (tid > 0) store_interleaved(a.fx + (size_t)blk * Sz<T, D>::FE * TPB, sm[tid - 1], tid, TPB);
  if (tid == TPB - 1) store_flat(a.fagg + (size_t)blk * Sz<T, D>::FE, sm[tid]);
  if constexpr (SITE == SITE_NEWTON) {
    block_sum_store<TPB>(d1.get(), red, a.part + (size_t)blk * BN_NPART + 3, tid);
    block_sum_store<TPB>(d2.get(), red, a.part + (size_t)blk * BN_NPART + 4, tid);
  } else if (tid == 0) {
    a.part[(size_t)blk * BN_NPART + 3] = 0.0;
    a.part[(size_t)blk * BN_NPART + 4] = 0.0;
  }
}

// ============================================================ F2
// One CTA: thread t owns block aggregates [t*per, (t+1)*per).
template <typename T, typename L, int P, int TPB>
__global__ void __launch_bounds__(TPB) filter_blocks_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FElem<T, D>* sm = reinterpret_cast<FElem<T, D>*>(smem_raw);
  const int tid = threadIdx.x;
  const int nb = a.nblocks;
  const int per = (nb + TPB - 1) / TPB;
  const int j0 = tid * per;
  const int j1 = j0 + per < nb ? j0 + per : nb;
  FElem<T, D> R;
  bool ok = true;
  if (j0 < j1) {
    load_flat(R, a.fagg + (size_t)j0 * Sz<T, D>::FE);
    for (int j = j0 + 1; j < j1; ++j) {
      FElem<T, D> x, r;
      load_flat(x, a.fagg + (size_t)j * Sz<T, D>::FE);
      ok = fcombine(R, x, r) && ok;
      R = r;
    }
  } else {
    felem_identity(R);
  }
  sm[tid] = R;
  __syncthreads();
  block_scan_filter<T, D, TPB>(sm, tid, a.status);
  if (a.seg_total_f && tid == TPB - 1) store_flat(a.seg_total_f, sm[tid]);
  // state entering aggregate j0: stationary prior (0, Pinf) -- or the state handed
  // over by the previous time segment -- then the exclusive prefix
  State<T, D> st;
  if (a.seg_left) {
    load_flat(st, a.seg_left);
  } else {
    set_zero(st.m);
    copy(st.P, a.ssm.Pinf);
  }
  if (tid > 0 && j0 < nb) {
    State<T, D> t2;
    ok = state_fcombine(st, sm[tid - 1], t2) && ok;
    st = t2;
  }
  for (int j = j0; j < j1; ++j) {
    store_flat(a.fin + (size_t)j * Sz<T, D>::ST, st);
    if (j + 1 < j1) {
      FElem<T, D> x;
      State<T, D> t2;
      load_flat(x, a.fagg + (size_t)j * Sz<T, D>::FE);
      ok = state_fcombine(st, x, t2) && ok;
      st = t2;
    }
  }
  if (!ok) atomicOr(a.status, BN_STATUS_SINGULAR);
}

// ============================================================ F3
// SITE: SITE_GIVEN (ops API) or SITE_NAT (model path).  STORE: where filtered
// states go.  SMOOTH: build smoother chunk elements (model path: shifted dt).
template <typename T, typename L, int P, int SITE, int STORE, bool SMOOTH, int TPB, bool BATCH = false>
__global__ void __launch_bounds__(TPB) filter_rerun_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SElem<T, D>* sm = reinterpret_cast<SElem<T, D>*>(smem_raw);
  __shared__ double red[TPB / 32];
  const int tid = threadIdx.x;
  const int blk = blockIdx.x;
  const int64_t g = (int64_t)blk * TPB + tid;
  const int64_t s = g * a.L;
  const int64_t e = s + a.L < a.N ? s + a.L : a.N;
  bool ok = true;
  State<T, D> st;
  load_flat(st, a.fin + (size_t)blk * Sz<T, D>::ST);
  if (tid > 0 && s < a.N) {
    FElem<T, D> x;
    State<T, D> t2;
    load_interleaved(x, a.fx + (size_t)blk * Sz<T, D>::FE * TPB, tid, TPB);
    ok = state_fcombine(st, x, t2) && ok;
    st = t2;
  }
  KSum<T> ll;
  SElem<T, D> Z;
  selem_identity(Z);
  T mp[D], Pp[D][D], AP[D][D], A[D][D];
  // fixed-point smoother of x_s (chunk aggregate of the RTS elements)
  T fmu[D], fSig[D][D], fX[D][D];
  auto chunk = [&](auto& mdl) {
  SiteIn<T, P> cur, nxt;
  if (s < e) load_site_in<T, D, P, SITE>(a, s, cur);
#pragma unroll 1
  for (int64_t k = s; k < e; ++k) {
    if (k + 1 < e) load_site_in<T, D, P, SITE>(a, k + 1, nxt);
    bool head;
    const auto& ss = mdl.at(k, head);
    {
      T Q[D][D];
      step_transition<L>(ss, head, cur.dt, A, Q);
      predict<L>(A, Q, st.m, st.P, mp, Pp, AP);
    }
    if constexpr (SMOOTH) {
      if (k > s && STORE == STORE_ELEM) {
        SElem<T, D> el;
        ok = smoother_element(st.m, st.P, mp, Pp, AP, el) && ok;
        store_elem<T, D>(a.fst, g, int(k - 1 - s), a.L, el);
      }
    }
    T y[P], R[P][P], rr[P], S[P][P], HP[P][D], Si[P][P];
    bool mk[P];
    site_of<T, P, SITE>(cur, y, R, mk);
    kf_update_x<L>(ss, mp, Pp, y, R, st.m, st.P, rr, S, HP, Si);
    const T llk = masked_logpdf<T, P>(rr, S, mk);
    ll.add(llk);
    if constexpr (BATCH) a.ll_step[k] = llk;
    if constexpr (SMOOTH) {
      if (k == s) {
        copy(fmu, st.m);
        copy(fSig, st.P);
        copy(fX, st.P);
      } else {
        fixed_point_step<L>(ss, A, rr, Si, HP, fmu, fSig, fX);
      }
    }
    if constexpr (STORE == STORE_INTERNAL) {
      store_rec<T, D>(a.fst, g, int(k - s), a.L, st.m, st.P);
    } else if constexpr (STORE == STORE_REF) {
      const T(&om)[D] = a.return_predict ? mp : st.m;
      const T(&oP)[D][D] = a.return_predict ? Pp : st.P;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        a.out_m[k * D + i] = om[i];
#pragma unroll
        for (int j = 0; j < D; ++j) a.out_P[(k * D + i) * D + j] = oP[i][j];
      }
    }
    cur = nxt;
  }
  if constexpr (SMOOTH) {
    if (e > s) {
      SElem<T, D> el;
      if (e < a.N || a.seg_more) {
        // the step after the chunk: inside the data, or the next segment's first step
        bool head;
        const auto& ss = mdl.at(e < a.N ? e : e - 1, head);
        if (e >= a.N) head = false;
        T Q[D][D];
        step_transition<L>(ss, head, e < a.N ? a.dt[e] : a.dt_next, A, Q);
        predict<L>(A, Q, st.m, st.P, mp, Pp, AP);
        if constexpr (STORE == STORE_ELEM) {
          ok = smoother_element(st.m, st.P, mp, Pp, AP, el) && ok;
          store_elem<T, D>(a.fst, g, int(e - 1 - s), a.L, el);
        }
        // aggregate: C = X A_e^T, E = C Pp^-1, g = mu - E mp, L = Sig - E C^T
        T C[D][D], Lc[D][D], Et[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T t = T(0);
#pragma unroll
            for (int q = L::lo(j); q < L::hi(j); ++q) t = fma(fX[i][q], A[j][q], t);
            C[i][j] = t;
          }
        copy(Lc, Pp);
        ok = cholesky(Lc) && ok;
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) Et[i][j] = C[j][i];
        chol_solve(Lc, Et);  // Et = Pp^-1 C^T = E^T
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T t = fmu[i];
#pragma unroll
          for (int j = 0; j < D; ++j) {
            Z.E[i][j] = Et[j][i];
            t = fma(-Et[j][i], mp[j], t);
          }
          Z.g[i] = t;
        }
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = i; j < D; ++j) {
            T t = fSig[i][j];
#pragma unroll
            for (int q = 0; q < D; ++q) t = fma(-Et[q][i], C[j][q], t);
            Z.L[i][j] = t;
            Z.L[j][i] = t;
          }
      } else {
        // the series' last step: element (0, m, P); the aggregate is x_s given all data
        set_zero(el.E);
        copy(el.g, st.m);
        copy(el.L, st.P);
        if constexpr (STORE == STORE_ELEM) store_elem<T, D>(a.fst, g, int(e - 1 - s), a.L, el);
        set_zero(Z.E);
        copy(Z.g, fmu);
        copy(Z.L, fSig);
      }
    }
    }
  };
  if constexpr (BATCH) {
    SeriesModel<L, T, P> mdl(a, s);
    chunk(mdl);
  } else {
    FixedModel<L, T, P> mdl{a.ssm, a.seg_continue};
    chunk(mdl);
  }
  if constexpr (SMOOTH) {
    sm[tid] = Z;
    __syncthreads();
    block_rscan_smoother<T, D, TPB>(sm, tid);
    if (tid < TPB - 1) store_interleaved(a.sx + (size_t)blk * Sz<T, D>::SE * TPB, sm[tid + 1], tid, TPB);
    if (tid == 0) store_flat(a.sagg + (size_t)blk * Sz<T, D>::SE, sm[0]);
  }
  if (!ok) atomicOr(a.status, BN_STATUS_NONPD);
  block_sum_store<TPB>(ll.get(), red, a.part + (size_t)blk * BN_NPART + 0, tid);
  if constexpr (STORE == STORE_REF) {
    // ops API: the last block sums the log marginal
    __shared__ bool last;
    if (tid == 0) {
      __threadfence();
      last = atomicAdd(&a.counter[0], 1u) == unsigned(a.nblocks - 1);
    }
    __syncthreads();
    if (last) {
      __threadfence();
      const int cols[1] = {0};
      double t[1];
      sum_partials<TPB, 1>(a.part, BN_NPART, a.nblocks, cols, t, red, tid);
      if (tid == 0) {
        a.result[BN_RES_LOGLIK] = t[0];
        a.counter[0] = 0u;
      }
    }
  }
}

// ============================================================ S1 (ops API)
// Smoother chunk elements from given filter means / covariances (ops.py:314-325).
template <typename T, typename L, int P, int TPB>
__global__ void __launch_bounds__(TPB) smoother_reduce_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SElem<T, D>* sm = reinterpret_cast<SElem<T, D>*>(smem_raw);
  const int tid = threadIdx.x;
  const int blk = blockIdx.x;
  const int64_t g = (int64_t)blk * TPB + tid;
  const int64_t s = g * a.L;
  const int64_t e = s + a.L < a.N ? s + a.L : a.N;
  bool ok = true;
  SElem<T, D> Z;
  selem_identity(Z);
  for (int64_t k = s; k < e; ++k) {
    T fm[D], fP[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      fm[i] = a.in_m[k * D + i];
#pragma unroll
      for (int j = 0; j < D; ++j) fP[i][j] = a.in_P[(k * D + i) * D + j];
    }
    SElem<T, D> el, r;
    if (k == a.N - 1) {
      set_zero(el.E);
      copy(el.g, fm);
      copy(el.L, fP);
    } else {
      T A[D][D], mp[D], Pp[D][D], AP[D][D];
      // transition from k to k+1: dt[k+1] when the caller passed the model's dt
      // (shift_dt), dt[k] in the ops API
      T Q[D][D];
      transition_noise<L>(a.ssm, a.shift_dt ? a.dt[k + 1] : a.dt[k], A, Q);
      predict<L>(A, Q, fm, fP, mp, Pp, AP);
      ok = smoother_element(fm, fP, mp, Pp, AP, el) && ok;
    }
    scompose(Z, el, r);
    Z = r;
  }
  sm[tid] = Z;
  __syncthreads();
  block_rscan_smoother<T, D, TPB>(sm, tid);
  if (tid < TPB - 1) store_interleaved(a.sx + (size_t)blk * Sz<T, D>::SE * TPB, sm[tid + 1], tid, TPB);
  if (tid == 0) store_flat(a.sagg + (size_t)blk * Sz<T, D>::SE, sm[0]);
  if (!ok) atomicOr(a.status, BN_STATUS_NONPD);
}

// ============================================================ S2
template <typename T, typename L, int P, int TPB>
__global__ void __launch_bounds__(TPB) smoother_blocks_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SElem<T, D>* sm = reinterpret_cast<SElem<T, D>*>(smem_raw);
  const int tid = threadIdx.x;
  const int nb = a.nblocks;
  const int per = (nb + TPB - 1) / TPB;
  const int j0 = tid * per;
  const int j1 = j0 + per < nb ? j0 + per : nb;
  SElem<T, D> R;
  if (j1 > j0) {
    load_flat(R, a.sagg + (size_t)(j1 - 1) * Sz<T, D>::SE);
    for (int j = j1 - 2; j >= j0; --j) {
      SElem<T, D> x, r;
      load_flat(x, a.sagg + (size_t)j * Sz<T, D>::SE);
      scompose(x, R, r);
      R = r;
    }
  } else {
    selem_identity(R);
  }
  sm[tid] = R;
  __syncthreads();
  block_rscan_smoother<T, D, TPB>(sm, tid);
  if (a.seg_total_s && tid == 0) store_flat(a.seg_total_s, sm[0]);
  // smoothed state entering (from the right) the last aggregate of this thread:
  // the next time segment's first smoothed state, else zero (the series' last
  // element has E = 0)
  State<T, D> st;
  if (a.seg_right) {
    load_flat(st, a.seg_right);
  } else {
    set_zero(st.m);
    set_zero(st.P);
  }
  if (tid < TPB - 1 && j1 > j0) {
    State<T, D> t2;
    selem_apply(sm[tid + 1], st, t2);
    st = t2;
  }
  for (int j = j1 - 1; j >= j0; --j) {
    store_flat(a.sin + (size_t)j * Sz<T, D>::ST, st);
    if (j > j0) {
      SElem<T, D> x;
      State<T, D> t2;
      load_flat(x, a.sagg + (size_t)j * Sz<T, D>::SE);
      selem_apply(x, st, t2);
      st = t2;
    }
  }
}

// ============================================================ site tail
// Expectations at the new posterior marginal (pm, pv) of step k: caches the next
// Newton derivatives and accumulates the two energy sums.
//   VI     s1 = E_q log p(y|f)                       s2 = E_q log N(site | f)
//   Newton s1 = log p(y | f = pm)                    s2 = E_q log N(site | f)
//   EP     s1 = log E_cav p(y|f)^a (lel)             s2 = lel_pseudo (basemodels.py:241-262)
//   PL     the EP sums at power 1; sites from statistical linear regression
// MODE: -1 reads the method at run time; 0 (VI), 1 (Newton), 2 (EP / PL) compile
// only that method's code (a smaller kernel for the instruction cache).
template <typename T, int D, int P, int MODE = -1>
__device__ __forceinline__ void site_tail(const ScanArgs<T, D, P>& a, const LikParams<T>& lp, SiteLik<T> sl, int64_t k,
                                          const T (&pm)[P], const T (&pv)[P][P], T yo, const T (&sn1)[P],
                                          const T (&sn2)[P][P], KSum<T>& s1, KSum<T>& s2) {
  T mu[P], Sg[P][P];
  {
    T ld;
    inv_small<T, P>(sn2, Sg, ld);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T t = T(0);
#pragma unroll
      for (int q = 0; q < P; ++q) t = fma(Sg[p][q], sn1[q], t);
      mu[p] = t;
    }
  }
  if constexpr (P == 1) {
    const bool masked = bn_isnan(yo);
    const T yv = masked ? pm[0] : yo;
    T g, h, lm;
    const bool eppl = MODE < 0 ? (lp.method == BN_METHOD_EP || lp.method == BN_METHOD_PL) : MODE == 2;
    const bool vi = MODE < 0 ? lp.method == BN_METHOD_VI : MODE == 0;
    if (eppl) {
      const T n1 = sn1[0], n2 = sn2[0][0];
      const T pn2 = T(1) / (pv[0][0] + T(1e-8));
      const T cv = T(1) / (pn2 - lp.power * n2);
      const T cm = cv * (pn2 * pm[0] - lp.power * n1);
      T lZ, dlZ, d2lZ;
      mm1(lp, masked ? cm : yo, cm, cv, lZ, dlZ, d2lZ);
      const T cp = T(1) / cv;
      const T sc = cp / (d2lZ + cp) / lp.power;
      g = masked ? T(NAN) : sc * dlZ;
      h = masked ? T(NAN) : sc * d2lZ;
      lm = cm;
      if (!masked) {
        s1.add(lZ);
        const T sv = Sg[0][0] / lp.power + cv;
        const T r = mu[0] - cm;
        s2.add(T(-0.5) * (r * r / sv + T(kLog2Pi) + log(sv)) + T(0.5) * ((T(1) - lp.power) * T(kLog2Pi) - log(lp.power)) +
               T(0.5) * (T(1) - lp.power) * log(Sg[0][0]));
      }
      if (lp.method == BN_METHOD_PL) {
        // posterior linearisation (inference.py:339-369): the EP energy above at power
        // 1 (:371-428), sites from the SLR at the posterior marginal; a missing y has
        // residual 0 and omega 1e6
        T smu, om, dmu;
        slr1(lp, pm[0], pv[0][0], smu, om, dmu);
        const T res = masked ? T(0) : yo - smu;
        if (masked) om = T(1e6);
        g = dmu * res / om;
        h = -dmu * dmu / om;
        lm = pm[0];
      }
    } else {
      T E;
      if (vi) {
        ve1(lp, sl, yv, pm[0], pv[0][0], E, g, h);
      } else {
        loglik1(lp, sl, yv, pm[0], E, g, h);
      }
      lm = pm[0];
      if (masked) {
        g = T(NAN);
        h = T(NAN);
      } else {
        s1.add(E);
        const T r = mu[0] - pm[0];
        s2.add(T(-0.5) * (T(kLog2Pi) + log(Sg[0][0])) - T(0.5) * (r * r + pv[0][0]) / Sg[0][0]);
      }
    }
    a.grad[k] = g;
    a.hess[k] = lp.ensure_psd ? psd_diag(h) : h;
    a.lin[k] = lm;
  } else {
    // two latents (multi-latent likelihood, no masking)
    T E, g[2], H[3];
    if (a.ext && lp.method == BN_METHOD_VI) {
      const T* x = a.ext + k * 6;
      E = x[0];
      g[0] = x[1];
      g[1] = x[2];
      H[0] = x[3];
      H[1] = x[4];
      H[2] = x[5];
    } else if (lp.method == BN_METHOD_NEWTON) {
      hetero_point(lp.kind, yo, pm[0], pm[1], E, g, H);
    } else {
      const T m2[2] = {pm[0], pm[1]};
      const T V[3] = {pv[0][0], T(0.5) * (pv[0][1] + pv[1][0]), pv[1][1]};
      ve2(lp, yo, m2, V, E, g, H);
    }
    s1.add(E);
    // E_q log N(mu | f, Sg) = log N(mu | pm, Sg) - tr(Sg^-1 pv) / 2
    T Si[2][2], ld;
    inv_small<T, 2>(Sg, Si, ld);
    const T r0 = mu[0] - pm[0], r1 = mu[1] - pm[1];
    const T q = r0 * (Si[0][0] * r0 + Si[0][1] * r1) + r1 * (Si[1][0] * r0 + Si[1][1] * r1);
    const T tr = Si[0][0] * pv[0][0] + Si[0][1] * pv[1][0] + Si[1][0] * pv[0][1] + Si[1][1] * pv[1][1];
    s2.add(T(-0.5) * (q + T(2) * T(kLog2Pi) + ld) - T(0.5) * tr);
    a.grad[k * 2 + 0] = g[0];
    a.grad[k * 2 + 1] = g[1];
    if (lp.ensure_psd) {
      a.hess[k * 4 + 0] = psd_diag(H[0]);
      a.hess[k * 4 + 1] = T(0);
      a.hess[k * 4 + 2] = T(0);
      a.hess[k * 4 + 3] = psd_diag(H[2]);
    } else {
      a.hess[k * 4 + 0] = H[0];
      a.hess[k * 4 + 1] = H[1];
      a.hess[k * 4 + 2] = H[1];
      a.hess[k * 4 + 3] = H[2];
    }
    a.lin[k * 2 + 0] = pm[0];
    a.lin[k * 2 + 1] = pm[1];
  }
}

// Per-step inputs of the smoother rerun, prefetched one step ahead.
template <typename T, int D, int P>
struct SmIn {
  T fm[D];
  T fP[D][D];
  T dt;
  T yo;
  T n1[P];
  T n2[P][P];
};

template <typename T, int D, int P, int LOAD, bool TAIL>
__device__ __forceinline__ void load_sm(const ScanArgs<T, D, P>& a, int64_t g, int64_t k, int64_t s, SmIn<T, D, P>& x) {
  if constexpr (LOAD == STORE_INTERNAL) {
    load_rec<T, D>(a.fst, g, int(k - s), a.L, x.fm, x.fP);
  } else if constexpr (LOAD == STORE_SEQ) {
    constexpr int REC = Sz<T, D>::REC;
    int f = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) x.fm[i] = a.fst[k * REC + f++];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = i; j < D; ++j) {
        const T v = a.fst[k * REC + f++];
        x.fP[i][j] = v;
        x.fP[j][i] = v;
      }
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      x.fm[i] = a.in_m[k * D + i];
#pragma unroll
      for (int j = 0; j < D; ++j) x.fP[i][j] = a.in_P[(k * D + i) * D + j];
    }
  }
  // transition from k to k+1: dt[k+1] on the model path, dt[k] in the ops API
  x.dt = a.shift_dt ? (k + 1 < a.N ? a.dt[k + 1] : T(0)) : a.dt[k];
  if constexpr (TAIL) {
    x.yo = a.y[k * a.obs_dim];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      x.n1[p] = a.nat1[k * P + p];
#pragma unroll
      for (int q = 0; q < P; ++q) x.n2[p][q] = a.nat2[(k * P + p) * P + q];
    }
  }
}

// ============================================================ S3
// LOAD: STORE_INTERNAL (model path, fused tail) or STORE_REF (ops API).
template <typename T, typename L, int P, int LOAD, bool TAIL, int TPB>
__global__ void __launch_bounds__(TPB) smoother_rerun_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  __shared__ double red[TPB / 32];
  __shared__ bool last;
  const int tid = threadIdx.x;
  const int blk = blockIdx.x;
  const int64_t g = (int64_t)blk * TPB + tid;
  const int64_t s = g * a.L;
  const int64_t e = s + a.L < a.N ? s + a.L : a.N;
  bool ok = true;
  State<T, D> st;
  load_flat(st, a.sin + (size_t)blk * Sz<T, D>::ST);
  if (tid < TPB - 1 && s < a.N) {
    SElem<T, D> x;
    State<T, D> t2;
    load_interleaved(x, a.sx + (size_t)blk * Sz<T, D>::SE * TPB, tid, TPB);
    selem_apply(x, st, t2);
    st = t2;
  }
  KSum<T> s1, s2;
  if constexpr (LOAD == STORE_ELEM) {
    // sm_k = E_k sm_{k+1} + g_k,  sP_k = E_k sP_{k+1} E_k^T + L_k  (elements stored by F3)
    SElem<T, D> ce, ne;
    T cyo = T(0), nyo = T(0), cn1[P], cn2[P][P], nn1[P], nn2[P][P];
    auto load_tail = [&](int64_t k, T& yo, T (&n1)[P], T (&n2)[P][P]) {
      if constexpr (TAIL) {
        yo = a.y[k * a.obs_dim];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          n1[p] = a.nat1[k * P + p];
#pragma unroll
          for (int q = 0; q < P; ++q) n2[p][q] = a.nat2[(k * P + p) * P + q];
        }
      }
    };
    if (e > s) {
      load_elem<T, D>(a.fst, g, int(e - 1 - s), a.L, ce);
      load_tail(e - 1, cyo, cn1, cn2);
    }
#pragma unroll 1
    for (int64_t k = e - 1; k >= s; --k) {
      if (k - 1 >= s) {
        load_elem<T, D>(a.fst, g, int(k - 1 - s), a.L, ne);
        load_tail(k - 1, nyo, nn1, nn2);
      }
      State<T, D> t2;
      selem_apply(ce, st, t2);
      st = t2;
      T pm[P], pv[P][P], HP[P][D];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        T t = T(0);
#pragma unroll
        for (int j = 0; j < D; ++j) {
          t = hacc<L, P>(a.ssm, p, j, st.m[j], t);
          T u = T(0);
#pragma unroll
          for (int i = 0; i < D; ++i) u = hacc<L, P>(a.ssm, p, i, st.P[i][j], u);
          HP[p][j] = u;
        }
        pm[p] = t;
      }
#pragma unroll
      for (int p = 0; p < P; ++p)
#pragma unroll
        for (int q = 0; q < P; ++q) {
          T t = T(0);
#pragma unroll
          for (int j = 0; j < D; ++j) t = hacc<L, P>(a.ssm, q, j, HP[p][j], t);
          pv[p][q] = t;
        }
#pragma unroll
      for (int p = 0; p < P; ++p) {
        a.post_mean[k * P + p] = pm[p];
#pragma unroll
        for (int q = 0; q < P; ++q) a.post_var[(k * P + p) * P + q] = pv[p][q];
      }
      if constexpr (TAIL) site_tail<T, D, P>(a, a.lik, site_lik(a.lik), k, pm, pv, cyo, cn1, cn2, s1, s2);
      ce = ne;
      cyo = nyo;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        cn1[p] = nn1[p];
#pragma unroll
        for (int q = 0; q < P; ++q) cn2[p][q] = nn2[p][q];
      }
    }
  } else {
  SmIn<T, D, P> cur, nxt;
  if (e > s) load_sm<T, D, P, LOAD, TAIL>(a, g, e - 1, s, cur);
  for (int64_t k = e - 1; k >= s; --k) {
    if (k - 1 >= s) load_sm<T, D, P, LOAD, TAIL>(a, g, k - 1, s, nxt);
    const T(&fm)[D] = cur.fm;
    const T(&fP)[D][D] = cur.fP;
    const bool lastk = (k == a.N - 1);
    T Gt[D][D];
    if (lastk && LOAD == STORE_INTERNAL) {
      copy(st.m, fm);
      copy(st.P, fP);
    } else {
      T A[D][D], mp[D], Pp[D][D], AP[D][D], Lc[D][D];
      T Q[D][D];
      transition_noise<L>(a.ssm, cur.dt, A, Q);
      predict<L>(A, Q, fm, fP, mp, Pp, AP);
      copy(Lc, Pp);
      ok = cholesky(Lc) && ok;
      copy(Gt, AP);
      chol_solve(Lc, Gt);
      if (lastk) {
        copy(st.m, fm);
        copy(st.P, fP);
      } else {
        // sm = fm + G (sm_next - mp);  sP = fP + G (sP_next - Pp) G^T
        T dm[D], Dp[D][D], X[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          dm[i] = st.m[i] - mp[i];
#pragma unroll
          for (int j = 0; j < D; ++j) Dp[i][j] = st.P[i][j] - Pp[i][j];
        }
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T t = fm[i];
#pragma unroll
          for (int j = 0; j < D; ++j) t = fma(Gt[j][i], dm[j], t);
          st.m[i] = t;
        }
        mtm(X, Gt, Dp);   // G (sP - Pp)
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = i; j < D; ++j) {
            T t = fP[i][j];
#pragma unroll
            for (int q = 0; q < D; ++q) t = fma(X[i][q], Gt[q][j], t);
            st.P[i][j] = t;
            st.P[j][i] = t;
          }
      }
      if constexpr (LOAD == STORE_REF) {
        if (a.out_G) {
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) a.out_G[(k * D + i) * D + j] = Gt[j][i];
        }
      }
    }
    // posterior marginal H sm, H sP H^T
    T pm[P], pv[P][P], HP[P][D];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T t = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        t = hacc<L, P>(a.ssm, p, j, st.m[j], t);
        T u = T(0);
#pragma unroll
        for (int i = 0; i < D; ++i) u = hacc<L, P>(a.ssm, p, i, st.P[i][j], u);
        HP[p][j] = u;
      }
      pm[p] = t;
    }
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int q = 0; q < P; ++q) {
        T t = T(0);
#pragma unroll
        for (int j = 0; j < D; ++j) t = hacc<L, P>(a.ssm, q, j, HP[p][j], t);
        pv[p][q] = t;
      }
    if constexpr (LOAD == STORE_REF) {
      if (a.return_full) {
#pragma unroll
        for (int i = 0; i < D; ++i) {
          a.out_m[k * D + i] = st.m[i];
#pragma unroll
          for (int j = 0; j < D; ++j) a.out_P[(k * D + i) * D + j] = st.P[i][j];
        }
      } else {
#pragma unroll
        for (int p = 0; p < P; ++p) {
          a.out_m[k * P + p] = pm[p];
#pragma unroll
          for (int q = 0; q < P; ++q) a.out_P[(k * P + p) * P + q] = pv[p][q];
        }
      }
    } else {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        a.post_mean[k * P + p] = pm[p];
#pragma unroll
        for (int q = 0; q < P; ++q) a.post_var[(k * P + p) * P + q] = pv[p][q];
      }
      if constexpr (TAIL) site_tail<T, D, P>(a, a.lik, site_lik(a.lik), k, pm, pv, cur.yo, cur.n1, cur.n2, s1, s2);
    }
    cur = nxt;
  }
  }
  if (!ok) atomicOr(a.status, BN_STATUS_NONPD);
  if constexpr (TAIL) {
    block_sum_store<TPB>(s1.get(), red, a.part + (size_t)blk * BN_NPART + 1, tid);
    block_sum_store<TPB>(s2.get(), red, a.part + (size_t)blk * BN_NPART + 2, tid);
    if (tid == 0) {
      __threadfence();
      last = atomicAdd(&a.counter[1], 1u) == unsigned(a.nblocks - 1);
    }
    __syncthreads();
    if (last) {
      __threadfence();
      const int cols[5] = {0, 1, 2, 3, 4};
      double t[5];
      sum_partials<TPB, 5>(a.part, BN_NPART, a.nblocks, cols, t, red, tid);
      if (tid == 0) {
        const double ll = t[0], s1t = t[1], s2t = t[2];
        a.result[BN_RES_LOGLIK] = ll;
        a.result[BN_RES_SUM1] = s1t;
        a.result[BN_RES_SUM2] = s2t;
        a.result[BN_RES_DIFF1] = t[3];
        a.result[BN_RES_DIFF2] = t[4];
        if (a.lik.method == BN_METHOD_EP || a.lik.method == BN_METHOD_PL) {
          a.result[BN_RES_ENERGY] = -(ll + (s1t - s2t) / double(a.lik.power));
        } else {
          a.result[BN_RES_ENERGY] = -(s1t - (s2t - ll));
        }
        a.counter[1] = 0u;
      }
    }
  }
}

// ============================================================ site tail (separate)
// One thread per site: the expectations at the new posterior marginal written by
// the smoother rerun, the next Newton derivatives and the two energy sums; the
// last block finalises the energy from these sums and the filter's log marginal.
// Running it apart from the sequential smoother recursion gives the cubature the
// whole GPU (one thread per site instead of one per chunk).
// Error-free sum: s + e == a + b exactly (Knuth's TwoSum; no products, so no
// FMA contraction can change it).
template <typename T>
__device__ __forceinline__ void two_sum(T a, T b, T& s, T& e) {
  s = a + b;
  const T bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Sum of the compensated pairs (v, c) over the lanes of a warp that share key
// (keys non-decreasing along the lanes); the last lane of each run gets the
// run's total as a pair, the others partial sums.  The pair keeps the float
// sum's rounding, so a series whose per-site energy terms of order one cancel
// to a small total keeps the digits of that total.
template <typename T>
__device__ __forceinline__ void warp_segment_sum(T& v, T& c, int key, bool& tail) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T u = __shfl_up_sync(0xffffffffu, v, d);
    const T uc = __shfl_up_sync(0xffffffffu, c, d);
    const int ku = __shfl_up_sync(0xffffffffu, key, d);
    if (lane >= d && ku == key) {
      T s, e;
      two_sum(v, u, s, e);
      v = s;
      c += uc + e;
    }
  }
  const int kn = __shfl_down_sync(0xffffffffu, key, 1);
  tail = (lane == 31) || (kn != key);
}

template <typename T, typename L, int P, int TPB, int SPT, bool BATCH = false, int MODE = -1>
__global__ void __launch_bounds__(TPB) site_tail_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  __shared__ double red[TPB / 32];
  __shared__ bool last;
  const int tid = threadIdx.x;
  // SPT sites per thread, strided by TPB so each pass is coalesced; the float
  // (compensated) sums keep the double-precision reduction -- slow on this GPU --
  // to one per SPT sites
  KSum<T> s1, s2;
  // not unrolled: one copy of the site code keeps the kernel small for the
  // instruction cache
#pragma unroll 1
  for (int j = 0; j < SPT; ++j) {
    const int64_t k = ((int64_t)blockIdx.x * SPT + j) * TPB + tid;
    int key = -1;
    T contrib = T(0), contrib_c = T(0);
    if (k < a.N) {
      T pm[P], pv[P][P], n1[P], n2[P][P];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        pm[p] = a.post_mean[k * P + p];
        n1[p] = a.nat1[k * P + p];
#pragma unroll
        for (int q = 0; q < P; ++q) {
          pv[p][q] = a.post_var[(k * P + p) * P + q];
          n2[p][q] = a.nat2[(k * P + p) * P + q];
        }
      }
      if constexpr (BATCH) {
        // this site's series: its likelihood, and its energy term
        // -(s1 - s2 + log-marginal term) (VI / Newton; EP is not batched)
        key = a.sid[k];
        const SiteLik<T> sl{a.ser_lik[key], a.ser_likvar[key]};
        KSum<T> t1, t2;
        site_tail<T, D, P>(a, a.lik, sl, k, pm, pv, a.y[k * a.obs_dim], n1, n2, t1, t2);
        s1.add(t1.s);
        s2.add(t2.s);
        const T yk = a.y[k * a.obs_dim];
        if (sl.kind == BN_LIK_GAUSSIAN && !bn_isnan(yk)) {
          // An observed Gaussian site.  With t1 = -0.5 (log 2 pi + log var) - u / (2 var)
          // (u = (y - m)^2, + v for VI) and t2 = -0.5 (log 2 pi - log n2) - q n2 / 2
          // (site precision n2, site mean mu, q = (mu - m)^2 + v), the term is
          //   -(t1 - t2 + ll) = 0.5 log(var n2) + u / (2 var) - q n2 / 2 - ll.
          // var and n2 are the same at every site of the series (the Gaussian site
          // update gives every site the same precision), so float32 rounding of
          // log var, log n2 or 1 / var would repeat at every site and grow linearly
          // over the series against a net energy that is a small fraction of the
          // terms.  Here log 2 pi cancels exactly, log(var n2) = log1p(var n2 - 1)
          // is taken from var as a float64 (head, tail) pair, and u / var is an
          // exact product with 1 / var as a pair; the float32 log 2 pi inside ll
          // (3.1e-8 below log 2 pi, one -0.5 log 2 pi per observed site) is
          // corrected by its known rounding error.
          const T* gk = a.ser_gauss + (size_t)key * 4;  // var (head, tail), 1 / var (head, tail)
          const T n2v = n2[0][0];
          const T r = yk - pm[0];
          const T u = a.lik.method == BN_METHOD_NEWTON ? r * r : fma(r, r, pv[0][0]);
          const T dmu = n1[0] / n2v - pm[0];
          const T qn = fma(dmu, dmu, pv[0][0]) * n2v;
          const T lg = T(0.5) * log1p(fma(gk[0], n2v, T(-1)) + gk[1] * n2v);
          const T ph = u * gk[2];
          const T pl = fma(u, gk[2], -ph) + u * gk[3];
          T s_1, s_2, s_3, e1, e2, e3;
          two_sum(T(0.5) * ph, T(-0.5) * qn, s_1, e1);
          two_sum(s_1, -a.ll_step[k], s_2, e2);
          two_sum(s_2, lg, s_3, e3);
          contrib = s_3;
          contrib_c = e1 + e2 + e3 + T(0.5) * pl + T(0.5 * (kLog2Pi - double(T(kLog2Pi))));
        } else {
          // -(t1 - t2 + ll) as an exact pair (contrib + contrib_c)
          T u, e1, e2;
          two_sum(t1.s, -t2.s, u, e1);
          two_sum(u, a.ll_step[k], contrib, e2);
          contrib = -contrib;
          contrib_c = -(e1 + e2 - t1.c + t2.c);
        }
      } else {
        site_tail<T, D, P, MODE>(a, a.lik, site_lik(a.lik), k, pm, pv, a.y[k * a.obs_dim], n1, n2, s1, s2);
      }
    }
    if constexpr (BATCH) {
      bool tail;
      warp_segment_sum(contrib, contrib_c, key, tail);
      if (tail && key >= 0) atomicAdd(a.ser_energy + key, double(contrib) + double(contrib_c));
    }
  }
  block_sum_store<TPB>(s1.get(), red, a.tpart + (size_t)blockIdx.x * 2 + 0, tid);
  block_sum_store<TPB>(s2.get(), red, a.tpart + (size_t)blockIdx.x * 2 + 1, tid);
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(&a.counter[1], 1u) == unsigned(a.ntail_blocks - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const int c3[3] = {0, 3, 4};
    const int c2[2] = {0, 1};
    double f[3], t[2];
    sum_partials<TPB, 3>(a.part, BN_NPART, a.nblocks, c3, f, red, tid);
    sum_partials<TPB, 2>(a.tpart, 2, a.ntail_blocks, c2, t, red, tid);
    if (tid != 0) return;
    const double ll = f[0], d1 = f[1], d2 = f[2], s1t = t[0], s2t = t[1];
    a.result[BN_RES_LOGLIK] = ll;
    a.result[BN_RES_SUM1] = s1t;
    a.result[BN_RES_SUM2] = s2t;
    a.result[BN_RES_DIFF1] = d1;
    a.result[BN_RES_DIFF2] = d2;
    a.result[BN_RES_ENERGY] =
        (a.lik.method == BN_METHOD_EP || a.lik.method == BN_METHOD_PL) ? -(ll + (s1t - s2t) / double(a.lik.power))
                                                                         : -(s1t - (s2t - ll));
    a.counter[1] = 0u;
  }
}

// ============================================================ sequential forms
// parallel=False: one thread walks the whole series (ops.py:154-180, 288-311).
// Filtered states go to fst as packed records [N][REC] (STORE_SEQ) or to the
// ops-level outputs (STORE_REF).
template <typename T, typename L, int P, int SITE, int STORE>
__global__ void seq_filter_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  constexpr int REC = Sz<T, D>::REC;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  State<T, D> st;
  set_zero(st.m);
  copy(st.P, a.ssm.Pinf);
  KSum<T> ll, d1, d2;
  T mp[D], Pp[D][D], AP[D][D], A[D][D];
  for (int64_t k = 0; k < a.N; ++k) {
    if constexpr (SITE == SITE_NEWTON) {
      T x1, x2;
      site_newton_update(a, k, x1, x2);
      d1.add(x1);
      d2.add(x2);
    }
    constexpr int SM = (SITE == SITE_GIVEN ? SITE_GIVEN : SITE_NAT);
    T Q[D][D];
    step_transition<L>(a.ssm, k == 0, a.dt[k], A, Q);
    predict<L>(A, Q, st.m, st.P, mp, Pp, AP);
    T y[P], R[P][P], rr[P], S[P][P];
    bool mk[P];
    step_site<T, D, P, SM>(a, k, y, R);
    step_mask<T, D, P, SM>(a, k, mk);
    kf_update<L>(a.ssm, mp, Pp, y, R, st.m, st.P, rr, S);
    ll.add(masked_logpdf<T, P>(rr, S, mk));
    if constexpr (STORE == STORE_SEQ) {
      int f = 0;
#pragma unroll
      for (int i = 0; i < D; ++i) a.fst[k * REC + f++] = st.m[i];
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = i; j < D; ++j) a.fst[k * REC + f++] = st.P[i][j];
    } else if constexpr (STORE == STORE_REF) {
      const T(&om)[D] = a.return_predict ? mp : st.m;
      const T(&oP)[D][D] = a.return_predict ? Pp : st.P;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        a.out_m[k * D + i] = om[i];
#pragma unroll
        for (int j = 0; j < D; ++j) a.out_P[(k * D + i) * D + j] = oP[i][j];
      }
    }
  }
  a.result[BN_RES_LOGLIK] = ll.get();
  a.result[BN_RES_DIFF1] = d1.get();
  a.result[BN_RES_DIFF2] = d2.get();
}

template <typename T, typename L, int P, int LOAD, bool TAIL>
__global__ void seq_smoother_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  bool ok = true;
  State<T, D> st;
  KSum<T> s1, s2;
  SmIn<T, D, P> cur, nxt;
  load_sm<T, D, P, LOAD, TAIL>(a, 0, a.N - 1, 0, cur);
  for (int64_t k = a.N - 1; k >= 0; --k) {
    if (k > 0) load_sm<T, D, P, LOAD, TAIL>(a, 0, k - 1, 0, nxt);
    const T(&fm)[D] = cur.fm;
    const T(&fP)[D][D] = cur.fP;
    const bool lastk = (k == a.N - 1);
    T Gt[D][D];
    if (lastk && LOAD == STORE_SEQ) {
      copy(st.m, fm);
      copy(st.P, fP);
    } else {
      T A[D][D], mp[D], Pp[D][D], AP[D][D], Lc[D][D];
      T Q[D][D];
      transition_noise<L>(a.ssm, cur.dt, A, Q);
      predict<L>(A, Q, fm, fP, mp, Pp, AP);
      copy(Lc, Pp);
      ok = cholesky(Lc) && ok;
      copy(Gt, AP);
      chol_solve(Lc, Gt);
      if (lastk) {
        copy(st.m, fm);
        copy(st.P, fP);
      } else {
        T dm[D], Dp[D][D], X[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          dm[i] = st.m[i] - mp[i];
#pragma unroll
          for (int j = 0; j < D; ++j) Dp[i][j] = st.P[i][j] - Pp[i][j];
        }
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T t = fm[i];
#pragma unroll
          for (int j = 0; j < D; ++j) t = fma(Gt[j][i], dm[j], t);
          st.m[i] = t;
        }
        mtm(X, Gt, Dp);
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = i; j < D; ++j) {
            T t = fP[i][j];
#pragma unroll
            for (int q = 0; q < D; ++q) t = fma(X[i][q], Gt[q][j], t);
            st.P[i][j] = t;
            st.P[j][i] = t;
          }
      }
      if constexpr (LOAD == STORE_REF) {
        if (a.out_G) {
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) a.out_G[(k * D + i) * D + j] = Gt[j][i];
        }
      }
    }
    T pm[P], pv[P][P], HP[P][D];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      T t = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        t = hacc<L, P>(a.ssm, p, j, st.m[j], t);
        T u = T(0);
#pragma unroll
        for (int i = 0; i < D; ++i) u = hacc<L, P>(a.ssm, p, i, st.P[i][j], u);
        HP[p][j] = u;
      }
      pm[p] = t;
    }
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int q = 0; q < P; ++q) {
        T t = T(0);
#pragma unroll
        for (int j = 0; j < D; ++j) t = hacc<L, P>(a.ssm, q, j, HP[p][j], t);
        pv[p][q] = t;
      }
    if constexpr (LOAD == STORE_REF) {
      if (a.return_full) {
#pragma unroll
        for (int i = 0; i < D; ++i) {
          a.out_m[k * D + i] = st.m[i];
#pragma unroll
          for (int j = 0; j < D; ++j) a.out_P[(k * D + i) * D + j] = st.P[i][j];
        }
      } else {
#pragma unroll
        for (int p = 0; p < P; ++p) {
          a.out_m[k * P + p] = pm[p];
#pragma unroll
          for (int q = 0; q < P; ++q) a.out_P[(k * P + p) * P + q] = pv[p][q];
        }
      }
    } else {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        a.post_mean[k * P + p] = pm[p];
#pragma unroll
        for (int q = 0; q < P; ++q) a.post_var[(k * P + p) * P + q] = pv[p][q];
      }
      if constexpr (TAIL) site_tail<T, D, P>(a, a.lik, site_lik(a.lik), k, pm, pv, cur.yo, cur.n1, cur.n2, s1, s2);
    }
    cur = nxt;
  }
  if (!ok) atomicOr(a.status, BN_STATUS_NONPD);
  if constexpr (TAIL) {
    const double ll = a.result[BN_RES_LOGLIK];
    const double s1t = s1.get(), s2t = s2.get();
    a.result[BN_RES_SUM1] = s1t;
    a.result[BN_RES_SUM2] = s2t;
    if (a.lik.method == BN_METHOD_EP || a.lik.method == BN_METHOD_PL) {
      a.result[BN_RES_ENERGY] = -(ll + (s1t - s2t) / double(a.lik.power));
    } else {
      a.result[BN_RES_ENERGY] = -(s1t - (s2t - ll));
    }
  }
}

}  // namespace bn
