// C ABI of libbnx.so (declared in include/bnx.h).  Dispatches a prior to the
// compiled configuration of its dtype, block layout and site dimension.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include <new>
#include <type_traits>

#include "bn_dense.cuh"
#include "bn_host.h"
#include "bn_layout.h"
#include "bn_ssm.cuh"

struct bn_model {
  bn::EngineBase* eng;
  bn_prior_desc prior;
  bn_lik_desc lik;
  int dtype;
};

namespace bn {
// explicit instantiations are generated per configuration by the build (one unit each)
#define BN_DECL(T, P, ...) extern template EngineBase* make_engine<T, Layout<__VA_ARGS__>, P>(int64_t, int, int, bool, int*);
BN_CONFIGS_F32(BN_DECL)
BN_CONFIGS_F64(BN_DECL)
#undef BN_DECL

namespace {

template <int... Bs>
bool sizes_match(const bn_prior_desc* d) {
  constexpr int s[] = {Bs...};
  if (d->num_components != int(sizeof...(Bs))) return false;
  for (int c = 0; c < int(sizeof...(Bs)); ++c)
    if (d->size[c] != s[c]) return false;
  return true;
}

template <int... Bs>
constexpr int layout_d() {
  return (0 + ... + Bs);
}

template <int... Bs>
constexpr int layout_nc() {
  return int(sizeof...(Bs));
}

// Exact layout first; otherwise the single-block layout of the same D (expm path).
EngineBase* dispatch(const bn_prior_desc* d, int P, int dtype, int64_t n, int obs, int spt, int* err) {
  int D = 0;
  for (int c = 0; c < d->num_components; ++c) D += d->size[c];
#define BN_TRY_EXACT(T, PP, ...)                                                                   \
  if (dtype == (sizeof(T) == 4 ? BN_DTYPE_F32 : BN_DTYPE_F64) && P == PP && sizes_match<__VA_ARGS__>(d)) \
    return make_engine<T, Layout<__VA_ARGS__>, PP>(n, obs, spt, false, err);
  BN_CONFIGS_F32(BN_TRY_EXACT)
  BN_CONFIGS_F64(BN_TRY_EXACT)
#undef BN_TRY_EXACT
#define BN_TRY_DENSE(T, PP, ...)                                                                        \
  if (dtype == (sizeof(T) == 4 ? BN_DTYPE_F32 : BN_DTYPE_F64) && P == PP && layout_nc<__VA_ARGS__>() == 1 && \
      layout_d<__VA_ARGS__>() == D)                                                                   \
    return make_engine<T, Layout<__VA_ARGS__>, PP>(n, obs, spt, true, err);
  BN_CONFIGS_F32(BN_TRY_DENSE)
  BN_CONFIGS_F64(BN_TRY_DENSE)
#undef BN_TRY_DENSE
  *err = BN_ERR_UNSUPPORTED;
  return nullptr;
}

int site_dim_of(const bn_prior_desc* d) {
  return d->combine == BN_COMBINE_INDEPENDENT ? d->num_components : 1;
}

}  // namespace
}  // namespace bn

extern "C" {

static bool prior_ok(const bn_prior_desc* d) {
  if (d->num_components < 1 || d->num_components > BN_MAX_COMPONENTS) return false;
  if (d->combine != BN_COMBINE_SUM && d->combine != BN_COMBINE_INDEPENDENT) return false;
  int D = 0;
  for (int c = 0; c < d->num_components; ++c) {
    if (d->size[c] < 1) return false;
    if (d->kind[c] < BN_KIND_MATERN12 || d->kind[c] > BN_KIND_FEEDBACK) return false;
    if (d->kind[c] != BN_KIND_FEEDBACK && (d->size[c] != d->kind[c] || !(d->lengthscale[c] > 0.0))) return false;
    D += d->size[c];
  }
  return D <= BN_MAX_STATE;
}

int bn_model_create(const bn_prior_desc* prior, const bn_lik_desc* lik, int64_t num_data, int32_t obs_dim,
                    int32_t dtype, int32_t steps_per_thread, bn_model** out) {
  if (!prior || !lik || !out || num_data < 1 || obs_dim < 1 || steps_per_thread < 0) return BN_ERR_ARG;
  if (dtype != BN_DTYPE_F32 && dtype != BN_DTYPE_F64) return BN_ERR_ARG;
  if (!prior_ok(prior)) return BN_ERR_ARG;
  *out = nullptr;
  int err = BN_OK;
  bn::EngineBase* e = bn::dispatch(prior, bn::site_dim_of(prior), dtype, num_data, obs_dim, steps_per_thread, &err);
  if (!e) return err;
  if ((err = e->set_prior(prior)) != BN_OK || (err = e->set_lik(lik)) != BN_OK) {
    delete e;
    return err;
  }
  bn_model* m = new (std::nothrow) bn_model;
  if (!m) {
    delete e;
    return BN_ERR_ARG;
  }
  m->eng = e;
  m->prior = *prior;
  m->lik = *lik;
  m->dtype = dtype;
  *out = m;
  return BN_OK;
}

int bn_model_destroy(bn_model* m) {
  if (!m) return BN_ERR_ARG;
  delete m->eng;
  delete m;
  return BN_OK;
}

int bn_model_set_prior(bn_model* m, const bn_prior_desc* prior) {
  if (!m || !prior || !prior_ok(prior)) return BN_ERR_ARG;
  int D = 0;
  for (int c = 0; c < prior->num_components; ++c) D += prior->size[c];
  if (D != m->eng->state_dim || bn::site_dim_of(prior) != m->eng->site_dim) return BN_ERR_ARG;
  const int err = m->eng->set_prior(prior);
  if (err == BN_OK) m->prior = *prior;
  return err;
}

int bn_model_set_likelihood(bn_model* m, const bn_lik_desc* lik) {
  if (!m || !lik) return BN_ERR_ARG;
  const int err = m->eng->set_lik(lik);
  if (err == BN_OK) m->lik = *lik;
  return err;
}

int bn_model_info(const bn_model* m, int32_t* state_dim, int32_t* site_dim, int32_t* steps_per_thread,
                  int32_t* num_blocks) {
  if (!m) return BN_ERR_ARG;
  if (state_dim) *state_dim = m->eng->state_dim;
  if (site_dim) *site_dim = m->eng->site_dim;
  if (steps_per_thread) *steps_per_thread = m->eng->spt;
  if (num_blocks) *num_blocks = m->eng->nblocks;
  return BN_OK;
}

static bool state_ok(const bn_site_state* s) {
  return s && s->nat1 && s->nat2 && s->post_mean && s->post_var && s->grad && s->hess && s->lin;
}

int bn_update_posterior(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                        const bn_site_state* s) {
  if (!m || !dt || !y || !state_ok(s)) return BN_ERR_ARG;
  return m->eng->update_posterior(static_cast<cudaStream_t>(stream), parallel, dt, y, *s);
}

int bn_newton_step(bn_model* m, void* stream, int32_t parallel, double lr, const void* dt, const void* y,
                   const bn_site_state* s) {
  if (!m || !dt || !y || !state_ok(s)) return BN_ERR_ARG;
  return m->eng->newton_step(static_cast<cudaStream_t>(stream), parallel, lr, dt, y, *s);
}

int bn_model_result(bn_model* m, void* stream, double* out, int32_t* status) {
  if (!m) return BN_ERR_ARG;
  return m->eng->result(static_cast<cudaStream_t>(stream), out, status);
}

int bn_kalman_filter(bn_model* m, void* stream, int32_t parallel, int32_t return_predict, const void* dt,
                     const void* site_y, const void* site_cov, const uint8_t* mask, void* means, void* covs) {
  if (!m || !dt || !site_y || !site_cov || !means || !covs) return BN_ERR_ARG;
  return m->eng->kalman_filter(static_cast<cudaStream_t>(stream), parallel, return_predict, dt, site_y, site_cov, mask,
                               means, covs);
}

int bn_rts_smoother(bn_model* m, void* stream, int32_t parallel, int32_t return_full, const void* dt,
                    const void* filter_mean, const void* filter_cov, void* means, void* covs, void* gains) {
  if (!m || !dt || !filter_mean || !filter_cov || !means || !covs) return BN_ERR_ARG;
  return m->eng->rts_smoother(static_cast<cudaStream_t>(stream), parallel, return_full, dt, filter_mean, filter_cov,
                              means, covs, gains);
}

int bn_temporal_conditional(bn_model* m, void* stream, const double* x, int64_t num_test, const double* x_test,
                            const void* mean, const void* cov, const void* gains, int32_t return_full,
                            void* test_mean, void* test_cov) {
  if (!m || num_test < 0) return BN_ERR_ARG;
  if (num_test == 0) return BN_OK;
  if (!x || !x_test || !mean || !cov || !gains || !test_mean || !test_cov) return BN_ERR_ARG;
  return m->eng->temporal_conditional(static_cast<cudaStream_t>(stream), x, num_test, x_test, mean, cov, gains,
                                      return_full, test_mean, test_cov);
}

int bn_model_predict(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                     const bn_site_state* s, const double* x, int64_t num_test, const double* x_test, void* test_mean,
                     void* test_cov) {
  if (!m || !s || num_test < 0) return BN_ERR_ARG;
  if (!dt || !y || !s->nat1 || !s->nat2 || !x) return BN_ERR_ARG;
  if (num_test > 0 && (!x_test || !test_mean || !test_cov)) return BN_ERR_ARG;
  return m->eng->predict(static_cast<cudaStream_t>(stream), parallel, dt, y, *s, x, num_test, x_test, test_mean,
                         test_cov);
}

int bn_model_log_density(bn_model* m, void* stream, int64_t n, const void* y, const void* mean, const void* var,
                         void* out, double* sum_count) {
  if (!m || n < 0) return BN_ERR_ARG;
  if (n > 0 && (!y || !mean || !var)) return BN_ERR_ARG;
  return m->eng->log_density(static_cast<cudaStream_t>(stream), n, y, mean, var, out, sum_count);
}

int bn_model_predict_y(bn_model* m, void* stream, int64_t n, const void* mean, const void* var, void* mean_y,
                       void* var_y) {
  if (!m || n < 0) return BN_ERR_ARG;
  if (n > 0 && (!mean || !var || !mean_y || !var_y)) return BN_ERR_ARG;
  return m->eng->predict_y(static_cast<cudaStream_t>(stream), n, mean, var, mean_y, var_y);
}

int bn_model_energy_grad(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                         const bn_site_state* s, double* grad, double* log_z) {
  if (!m || !s || !dt || !y || !grad || !s->nat1 || !s->nat2 || !s->post_mean || !s->post_var) return BN_ERR_ARG;
  return m->eng->energy_grad(static_cast<cudaStream_t>(stream), parallel, dt, y, *s, grad, log_z);
}

int bn_model_set_series(bn_model* m, int64_t num_series, const int64_t* offsets, const double* variance,
                        const double* lengthscale, const int32_t* lik_kind, const double* lik_variance) {
  if (!m) return BN_ERR_ARG;
  return m->eng->set_series(num_series, offsets, variance, lengthscale, lik_kind, lik_variance);
}

int bn_model_series_energy(bn_model* m, void* stream, double* out) {
  if (!m || !out) return BN_ERR_ARG;
  return m->eng->series_energy(static_cast<cudaStream_t>(stream), out);
}

// Batched product C_i = alpha op(A_i) op(B_i) + beta C0_i on the tensor cores
// (3xTF32) or the CUDA cores, for tests of the two paths (device float32 arrays,
// batch stride M K / K N / M N).
int bn_dense_gemm(void* stream, int32_t tensor_cores, int32_t batch, int32_t ta, int32_t tb, int32_t M, int32_t N,
                  int32_t K, float alpha, const float* A, const float* B, float beta, const float* C0, float* C) {
  if (batch < 1 || M < 1 || N < 1 || K < 1 || !A || !B || !C) return BN_ERR_ARG;
  using bn::dense::BRef;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BRef a(const_cast<float*>(A), int64_t(M) * K), b(const_cast<float*>(B), int64_t(K) * N),
      c0(const_cast<float*>(C0), int64_t(M) * N), c(C, int64_t(M) * N);
  if (tensor_cores) {
    if (!bn::dense::tc_attr_all()) return BN_ERR_CUDA;
    if (!bn::dense::tc_gemm(st, batch, ta != 0, tb != 0, M, N, K, alpha, a, b, beta, c0, c, 0)) return BN_ERR_ARG;
    int err = 0;
    if (cudaGetLastError() != cudaSuccess) return BN_ERR_CUDA;
    if (cudaMemcpyFromSymbolAsync(&err, bn::dense::g_tc_gemm_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return BN_ERR_CUDA;
    return err ? BN_ERR_CUDA : BN_OK;
  }
  dim3 grid((N + bn::dense::kGT - 1) / bn::dense::kGT, (M + bn::dense::kGT - 1) / bn::dense::kGT, batch);
  if (!ta && !tb) bn::dense::bgemm_kernel<false, false><<<grid, 256, 0, st>>>(M, N, K, alpha, a, b, beta, c0, c, 0);
  else if (ta && !tb) bn::dense::bgemm_kernel<true, false><<<grid, 256, 0, st>>>(M, N, K, alpha, a, b, beta, c0, c, 0);
  else if (!ta && tb) bn::dense::bgemm_kernel<false, true><<<grid, 256, 0, st>>>(M, N, K, alpha, a, b, beta, c0, c, 0);
  else bn::dense::bgemm_kernel<true, true><<<grid, 256, 0, st>>>(M, N, K, alpha, a, b, beta, c0, c, 0);
  return cudaGetLastError() == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}

// Batched in-place inverse with partial pivoting (device float32, contiguous n x n
// matrices): engine 0 the shared-memory Gauss-Jordan, 1 the register-resident one
// (n <= 200), 2 the register-resident one with the diagonal pivots in order (for
// symmetric positive definite matrices); logdet (device, may be null) gets sum log|pivot| per matrix, *status
// (device, may be null) is or-ed with 1 when a pivot is zero.
int bn_dense_inverse(void* stream, int32_t engine, int32_t batch, int32_t n, float* A, double* logdet,
                     int32_t* status) {
  if (batch < 1 || n < 1 || !A || engine < 0 || engine > 2) return BN_ERR_ARG;
  if (engine >= 1 && n > bn::dense::kGjMax) return BN_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (engine == 0 && cudaFuncSetAttribute(bn::dense::binv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          int(bn::dense::inv_smem(n))) != cudaSuccess)
    return BN_ERR_CUDA;
  const cudaError_t e = bn::dense::binv(st, batch, n, bn::dense::BRef(A, int64_t(n) * n), logdet, 1, 0, status, 1,
                                        engine == 0 ? 0 : 1, engine == 2);
  return e == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}

int bn_model_set_surrogate(bn_model* m, bn_mlp* h, int32_t spot, double tol) {
  if (!m || spot < 0 || !(tol > 0.0)) return BN_ERR_ARG;
  return m->eng->set_surrogate(h, spot, tol);
}

int bn_model_set_segment(bn_model* m, int32_t continue_left, int32_t more_right, double dt_next) {
  if (!m) return BN_ERR_ARG;
  return m->eng->set_segment(continue_left, more_right, dt_next);
}

int bn_model_element_sizes(bn_model* m, int32_t* filter_words, int32_t* smoother_words, int32_t* state_words) {
  if (!m) return BN_ERR_ARG;
  int fe = 0, se = 0, stw = 0;
  m->eng->element_sizes(&fe, &se, &stw);
  if (filter_words) *filter_words = fe;
  if (smoother_words) *smoother_words = se;
  if (state_words) *state_words = stw;
  return BN_OK;
}

int bn_segment_step(bn_model* m, void* stream, int32_t phase, int32_t newton, double lr, const void* dt,
                    const void* y, const bn_site_state* s, const double* boundary, double* total) {
  if (!m || !dt || !y || !state_ok(s) || phase < 0 || phase > 2) return BN_ERR_ARG;
  if (phase < 2 && !total) return BN_ERR_ARG;
  return m->eng->segment_step(static_cast<cudaStream_t>(stream), phase, newton != 0, lr, dt, y, *s, boundary,
                              total);
}

namespace {
// X = A^-1 B for a d x d A (Gaussian elimination with partial pivoting; false if singular)
bool host_solve(int d, std::vector<double> A, std::vector<double>& B, int nrhs) {
  for (int k = 0; k < d; ++k) {
    int p = k;
    for (int i = k + 1; i < d; ++i)
      if (std::fabs(A[size_t(i) * d + k]) > std::fabs(A[size_t(p) * d + k])) p = i;
    if (!(std::fabs(A[size_t(p) * d + k]) > 0.0)) return false;
    if (p != k) {
      for (int j = 0; j < d; ++j) std::swap(A[size_t(k) * d + j], A[size_t(p) * d + j]);
      for (int j = 0; j < nrhs; ++j) std::swap(B[size_t(k) * nrhs + j], B[size_t(p) * nrhs + j]);
    }
    for (int i = k + 1; i < d; ++i) {
      const double f = A[size_t(i) * d + k] / A[size_t(k) * d + k];
      for (int j = k; j < d; ++j) A[size_t(i) * d + j] -= f * A[size_t(k) * d + j];
      for (int j = 0; j < nrhs; ++j) B[size_t(i) * nrhs + j] -= f * B[size_t(k) * nrhs + j];
    }
  }
  for (int i = d - 1; i >= 0; --i)
    for (int j = 0; j < nrhs; ++j) {
      double v = B[size_t(i) * nrhs + j];
      for (int k = i + 1; k < d; ++k) v -= A[size_t(i) * d + k] * B[size_t(k) * nrhs + j];
      B[size_t(i) * nrhs + j] = v / A[size_t(i) * d + i];
    }
  return true;
}
}  // namespace

// Filtered state (m, P) followed by a filter element (A, b, C, J, eta) (flat, the
// layout bn_segment_step exchanges): W = (I + P J)^-1, m' = A W (m + P eta) + b,
// P' = A W P A^T + C.  Host float64; state_in = null starts from the element alone
// (a segment that begins the series).
int bn_segment_filter_state(int32_t d, const double* state_in, const double* elem, double* state_out) {
  if (d < 1 || !elem || !state_out) return BN_ERR_ARG;
  const size_t dd = size_t(d) * d;
  const double* A = elem;
  const double* b = A + dd;
  const double* C = b + d;
  const double* J = C + dd;
  const double* eta = J + dd;
  std::vector<double> m(d, 0.0), P(dd, 0.0);
  if (state_in) {
    std::copy(state_in, state_in + d, m.begin());
    std::copy(state_in + d, state_in + d + dd, P.begin());
  }
  // W^T = (I + J P)^-1 since (I + P J)^T = I + J P; X = A W = (W^T A^T)^T
  std::vector<double> M(dd), AT(dd);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double v = (i == j) ? 1.0 : 0.0;
      for (int k = 0; k < d; ++k) v += J[size_t(i) * d + k] * P[size_t(k) * d + j];
      M[size_t(i) * d + j] = v;
      AT[size_t(i) * d + j] = A[size_t(j) * d + i];
    }
  if (!host_solve(d, M, AT, d)) return BN_ERR_ARG;  // AT := W^T A^T = X^T
  std::vector<double> t(d);
  for (int i = 0; i < d; ++i) {
    double v = m[i];
    for (int k = 0; k < d; ++k) v += P[size_t(i) * d + k] * eta[k];
    t[i] = v;
  }
  for (int i = 0; i < d; ++i) {
    double v = b[i];
    for (int k = 0; k < d; ++k) v += AT[size_t(k) * d + i] * t[k];
    state_out[i] = v;
  }
  // P' = X P A^T + C
  std::vector<double> Y(dd);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double v = 0.0;
      for (int k = 0; k < d; ++k) v += AT[size_t(k) * d + i] * P[size_t(k) * d + j];
      Y[size_t(i) * d + j] = v;
    }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double v = C[size_t(i) * d + j];
      for (int k = 0; k < d; ++k) v += Y[size_t(i) * d + k] * A[size_t(j) * d + k];
      state_out[d + size_t(i) * d + j] = v;
    }
  return BN_OK;
}

// Smoother element (E, g, L) applied to the smoothed state (m, P) that follows it:
// m' = E m + g, P' = E P E^T + L.  state_in = null: the state is zero (the
// element then has E = 0, the series' last segment).
int bn_segment_smoother_state(int32_t d, const double* elem, const double* state_in, double* state_out) {
  if (d < 1 || !elem || !state_out) return BN_ERR_ARG;
  const size_t dd = size_t(d) * d;
  const double* E = elem;
  const double* g = E + dd;
  const double* L = g + d;
  std::vector<double> m(d, 0.0), P(dd, 0.0), Y(dd);
  if (state_in) {
    std::copy(state_in, state_in + d, m.begin());
    std::copy(state_in + d, state_in + d + dd, P.begin());
  }
  for (int i = 0; i < d; ++i) {
    double v = g[i];
    for (int k = 0; k < d; ++k) v += E[size_t(i) * d + k] * m[k];
    state_out[i] = v;
  }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double v = 0.0;
      for (int k = 0; k < d; ++k) v += E[size_t(i) * d + k] * P[size_t(k) * d + j];
      Y[size_t(i) * d + j] = v;
    }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double v = L[size_t(i) * d + j];
      for (int k = 0; k < d; ++k) v += Y[size_t(i) * d + k] * E[size_t(j) * d + k];
      state_out[d + size_t(i) * d + j] = v;
    }
  return BN_OK;
}

int bn_model_set_profiling(bn_model* m, int32_t on) {
  if (!m) return BN_ERR_ARG;
  return m->eng->set_profiling(on);
}

int bn_model_kernel_times(bn_model* m, float* ms, int32_t n) {
  if (!m || !ms || n < 1) return BN_ERR_ARG;
  return m->eng->kernel_times(ms, n);
}

// Bounded-wait probe (failure detection without a GPU fault): one thread waits on
// an mbarrier phase that nothing completes, with the poll limit the caller gives,
// and must give up (status[0] = 1); it then completes the phase with its own
// arrive and waits again, which must succeed (status[1] = 1).  The kernel always
// returns, so the context stays usable; the tensor-core kernels' waits use the
// same bounded poll loop with their own limit.
namespace {
constexpr uint32_t kProbeMaxPolls = 1u << 20;

__global__ void bounded_wait_probe_kernel(uint32_t polls, int32_t* status) {
  __shared__ __align__(8) unsigned long long mbar_s;
  const uint32_t mbar = uint32_t(__cvta_generic_to_shared(&mbar_s));
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const bool never = bn::tc::wait_phase_for(mbar, 0, polls);
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(mbar) : "memory");
  const bool done = bn::tc::wait_phase_for(mbar, 0, polls);
  status[0] = never ? 0 : 1;
  status[1] = done ? 1 : 0;
}
}  // namespace

int bn_bounded_wait_probe(void* stream, uint32_t polls, int32_t* status) {
  if (!status || polls < 1 || polls > kProbeMaxPolls) return BN_ERR_ARG;
  bounded_wait_probe_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(polls, status);
  return cudaGetLastError() == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}

int bn_matern_process_noise(int32_t size, double variance, double lengthscale, double dt, float* a, float* q) {
  if (size < 1 || size > 4 || !(variance > 0.0) || !(lengthscale > 0.0) || !(dt >= 0.0) || !a || !q)
    return BN_ERR_ARG;
  const float var = float(variance), lam = float(std::sqrt(double(2 * size - 1)) / lengthscale), t = float(dt);
  auto run = [&](auto tag) {
    constexpr int S = decltype(tag)::value;
    float A[S][S], Q[S][S];
    bn::matern_block_aq<S>(var, lam, t, A, Q);
    for (int i = 0; i < S; ++i)
      for (int j = 0; j < S; ++j) {
        a[i * S + j] = A[i][j];
        q[i * S + j] = Q[i][j];
      }
  };
  switch (size) {
    case 1: run(std::integral_constant<int, 1>{}); break;
    case 2: run(std::integral_constant<int, 2>{}); break;
    case 3: run(std::integral_constant<int, 3>{}); break;
    default: run(std::integral_constant<int, 4>{}); break;
  }
  return BN_OK;
}

int bn_gauss_hermite(int32_t n, double* x, double* w) {
  if (n < 1 || n > BN_MAX_CUB || !x || !w) return BN_ERR_ARG;
  bn::gauss_hermite(n, x, w);
  return BN_OK;
}

const char* bn_build_info(void) {
  return "libbnx: Markov-GP inference step for sm_103a (chunked associative-scan Kalman filter / RTS smoother)";
}

}  // extern "C"
