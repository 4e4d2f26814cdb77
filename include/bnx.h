/*
 * bnx.h -- C ABI of the GB300 Markov-GP inference step (libbnx.so).
 *
 * Plain pointers and sizes only.  Every array argument is a DEVICE pointer to a
 * contiguous row-major buffer of the model's dtype (float32 or float64), owned by
 * the caller.  Every entry point takes a cudaStream_t (passed as void*; NULL =
 * the legacy default stream) and enqueues work on it; results that are scalars
 * are read back with bn_model_result().
 *
 * Return codes: BN_OK (0) or a negative BN_ERR_*.  Numerical conditions found on
 * the device (a covariance that failed its Cholesky, a singular scan combine) are
 * reported as BN_STATUS_* bits by bn_model_result(); they do not abort the step,
 * matching the reference, which lets such cases run on as NaN.
 *
 * Reference interfaces replaced (bayesnewton 1.3.4):
 *   bn_kalman_filter      <- bayesnewton/ops.py:256-285  kalman_filter(dt, kernel, y, noise_cov,
 *                                                         mask, parallel, return_predict)
 *   bn_rts_smoother       <- bayesnewton/ops.py:357-380  rauch_tung_striebel_smoother(dt, kernel,
 *                                                         filter_mean, filter_cov, return_full, parallel)
 *   bn_update_posterior   <- bayesnewton/basemodels.py:689-706 MarkovGaussianProcess.update_posterior
 *                            (+ the site expectations and energy terms of inference.py:197-222)
 *   bn_newton_step        <- bayesnewton/inference.py:65-90 InferenceMixin.inference(lr) for the
 *                            VariationalInference / Newton / ExpectationPropagation mixins
 *                            (inference.py:99-325) on a MarkovGaussianProcess, followed by the
 *                            energy of inference.py:197-222 (VI), :130-154 (Newton), :286-325 (EP)
 *   bn_model_result       <- the scalar returns of the above (energy, log marginal, diffs)
 *   bn_model_create / set_prior / set_likelihood
 *                         <- the model constructors of bayesnewton/models.py:118-132, 216-231,
 *                            297-299 and the kernels / likelihoods they hold
 *                            (kernels.py:123-382, 1499-1663; likelihoods.py:684-1008, 1244-1281)
 */
#ifndef BNX_H
#define BNX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BN_MAX_COMPONENTS 8
#define BN_MAX_STATE 8
#define BN_MAX_CUB 32

/* prior components */
#define BN_KIND_MATERN12 1
#define BN_KIND_MATERN32 2
#define BN_KIND_MATERN52 3
#define BN_KIND_MATERN72 4
#define BN_KIND_FEEDBACK 5 /* generic: A = expm(F dt), F and Pinf given */

#define BN_COMBINE_SUM 0         /* H = [H_1, H_2, ...]          (kernels.py:1624-1663) */
#define BN_COMBINE_INDEPENDENT 1 /* H = block_diag(H_1, H_2 ...) (kernels.py:1499-1616) */

/* likelihoods */
#define BN_LIK_GAUSSIAN 1
#define BN_LIK_BERNOULLI_LOGIT 2
#define BN_LIK_BERNOULLI_PROBIT 3
#define BN_LIK_POISSON_EXP 4
#define BN_LIK_HETERO_EXP 5
#define BN_LIK_HETERO_SOFTPLUS 6

/* site-update methods */
#define BN_METHOD_VI 0
#define BN_METHOD_NEWTON 1
#define BN_METHOD_EP 2
#define BN_METHOD_PL 3 /* posterior linearisation (statistical linear regression sites, EP energy) */

#define BN_DTYPE_F32 0
#define BN_DTYPE_F64 1

/* return codes */
#define BN_OK 0
#define BN_ERR_ARG (-1)
#define BN_ERR_UNSUPPORTED (-2)
#define BN_ERR_CUDA (-3)
#define BN_ERR_SCRATCH (-4) /* bn_kalman_filter_noalloc: the call needs more than its fixed scratch */

/* device status bits */
#define BN_STATUS_NONPD 1    /* a predicted covariance failed its Cholesky */
#define BN_STATUS_SINGULAR 2 /* a scan combine met a singular I + C J */
#define BN_STATUS_SITE_KEPT 4    /* a site update was not finite; that site kept its old parameters */
#define BN_STATUS_SITE_CLAMPED 8 /* float32: a site precision above 1e6 x the prior precision was
                                  * scaled back to that bound (its mean unchanged) */

/* bn_model_result slots */
#define BN_RES_ENERGY 0
#define BN_RES_LOGLIK 1
#define BN_RES_SUM1 2  /* VI: sum E_q log p(y|f); Newton: sum log p(y|m); EP: sum lel   */
#define BN_RES_SUM2 3  /* VI/Newton: sum E_q log N(site|f); EP: sum lel_pseudo        */
#define BN_RES_DIFF1 4 /* sum |nat1_new - nat1_old| over sites (undamped, as the reference) */
#define BN_RES_DIFF2 5 /* sum |nat2_new - nat2_old|                                       */
#define BN_RES_SURR_PSD 6  /* learned sites: sites sent back to cubature, -h11 or -h22 not positive */
#define BN_RES_SURR_SPOT 7 /* learned sites: spot-checked sites off by more than tol           */
#define BN_NRESULT 8
#define BN_NPART 8

typedef struct bn_prior_desc {
  int32_t num_components;
  int32_t combine;                         /* BN_COMBINE_* */
  int32_t kind[BN_MAX_COMPONENTS];         /* BN_KIND_* */
  int32_t size[BN_MAX_COMPONENTS];         /* state size of each component */
  double variance[BN_MAX_COMPONENTS];
  double lengthscale[BN_MAX_COMPONENTS];
  double feedback[BN_MAX_STATE * BN_MAX_STATE]; /* D x D, read for BN_KIND_FEEDBACK blocks */
  double pinf[BN_MAX_STATE * BN_MAX_STATE];     /* D x D, read for BN_KIND_FEEDBACK blocks */
} bn_prior_desc;

typedef struct bn_lik_desc {
  int32_t kind;       /* BN_LIK_* */
  int32_t method;     /* BN_METHOD_* */
  int32_t num_cub;    /* Gauss-Hermite points per latent (reference default 20) */
  int32_t ensure_psd; /* 1 = the reference default */
  int32_t score_form; /* 1 = score-function derivative sums of cubature.py:198-246 */
  double variance;    /* Gaussian noise variance */
  double binsize;     /* Poisson bin size */
  double power;       /* EP power */
} bn_lik_desc;

typedef struct bn_model bn_model;
typedef struct bn_mlp bn_mlp;

/* Caller-owned per-site state of a model (device pointers, model dtype). */
typedef struct bn_site_state {
  void* nat1;      /* [N, P]    site natural parameters nat1 = Sigma^-1 mu (in/out)          */
  void* nat2;      /* [N, P, P] site precision Sigma^-1 (in/out)                              */
  void* post_mean; /* [N, P]    posterior marginal means (out)                                */
  void* post_var;  /* [N, P, P] posterior marginal covariances (out)                          */
  void* grad;      /* [N, P]    site expectation derivatives at the posterior (out; read by
                                bn_newton_step)                                               */
  void* hess;      /* [N, P, P] second derivatives, after the reference's PSD fix when asked  */
  void* lin;       /* [N, P]    point they were taken at (posterior mean; EP: cavity mean)    */
} bn_site_state;

/* Create a model for one series of num_data sorted time points.  obs_dim is the
 * number of observation columns (1 for every likelihood here).  steps_per_thread
 * picks the scan chunk length (0 = automatic).  Allocates all device workspace;
 * nothing later allocates. */
int bn_model_create(const bn_prior_desc* prior, const bn_lik_desc* lik, int64_t num_data, int32_t obs_dim,
                    int32_t dtype, int32_t steps_per_thread, bn_model** out);
int bn_model_destroy(bn_model* m);
int bn_model_set_prior(bn_model* m, const bn_prior_desc* prior);
int bn_model_set_likelihood(bn_model* m, const bn_lik_desc* lik);
/* state dimension, site (latent) dimension, chunk length, blocks per scan */
int bn_model_info(const bn_model* m, int32_t* state_dim, int32_t* site_dim, int32_t* steps_per_thread,
                  int32_t* num_blocks);

/* Posterior from the current sites: filter + smoother, then the site expectations
 * at the new posterior (grad / hess / lin, read by the next bn_newton_step) and
 * the energy terms.  dt [N] (dt[0] is ignored: the first state is the stationary
 * prior), y [N, obs_dim] with NaN = missing.  parallel = 0 runs the sequential
 * filter/smoother on one thread; 1 the chunked associative scan. */
int bn_update_posterior(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                        const bn_site_state* s);

/* One damped Newton step of the sites from grad / hess / lin (the expectations at
 * the current posterior), then the posterior, the expectations and the energy at
 * the new sites.  nat1 / nat2 are updated in place. */
int bn_newton_step(bn_model* m, void* stream, int32_t parallel, double lr, const void* dt, const void* y,
                   const bn_site_state* s);

/* Many independent series in one model (no counterpart in the reference, which
 * builds one model per series): the model's num_data time points are
 * num_series series concatenated, series i occupying [offsets[i], offsets[i+1])
 * (host array, offsets[0] = 0, offsets[num_series] = num_data), each sorted in
 * time.  Series i has its own prior hyperparameters (variance[i], lengthscale[i];
 * single-component Matern priors) and likelihood (lik_kind[i] =
 * BN_LIK_GAUSSIAN / POISSON_EXP / BERNOULLI_*, Gaussian noise lik_variance[i]);
 * the model's likelihood descriptor supplies the method (VI or Newton) and the
 * cubature.  dt[offsets[i]] is ignored: every series starts from its stationary
 * prior.  After this call bn_update_posterior / bn_newton_step (parallel = 1)
 * run all series in one pass; BN_RES_ENERGY is the sum over series.  Allocates
 * the per-series tables (set-up, not on the step path). */
int bn_model_set_series(bn_model* m, int64_t num_series, const int64_t* offsets, const double* variance,
                        const double* lengthscale, const int32_t* lik_kind, const double* lik_variance);
/* Energy of each series after the last step (num_series doubles, host); synchronises. */
int bn_model_series_energy(bn_model* m, void* stream, double* out);

/* ---------------------------------------------------------------------------
 * Learned site expectations (no counterpart in the reference): a 6-64-64-64-6
 * tanh MLP that maps a two-latent site's (y, m1, m2, v11, v12, v22) to
 * (E, g1, g2, h11, h12, h22) of E_q log p(y|f) for the HeteroscedasticNoise
 * likelihood, in place of its 2-D Gauss-Hermite cubature (likelihoods.py:613-664).
 * Parameters: W1[64][6] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[6][64] b4[6]
 * (bn_mlp_num_params floats); standardisation: in mean[6], in sd[6], out mean[6],
 * out sd[6].  Array arguments are device float32 unless noted.
 * ------------------------------------------------------------------------- */
int bn_mlp_create(int32_t lik_kind, bn_mlp** out); /* BN_LIK_HETERO_EXP / _SOFTPLUS */
void bn_mlp_destroy(bn_mlp* h);
int32_t bn_mlp_num_params(void);
int bn_mlp_set_params(bn_mlp* h, const float* params /* host or null */, const float* norm /* host [24] or null */);
int bn_mlp_get_params(bn_mlp* h, float* params /* host or null */, float* norm /* host [24] or null */);
/* raw sites [n][6] -> standardised features xn [n][6]; with tn / traw, targets
 * from ncub x ncub Gauss-Hermite cubature, standardised and raw */
int bn_mlp_prepare(bn_mlp* h, void* stream, int32_t n, int32_t ncub, const float* raw, float* xn, float* tn,
                   float* traw);
/* the learned site pass on marginals pm [n][2], pv [n][2][2], y [n] -> ext [n][6]
 * (E, g1, g2, h11, h12, h22) with the model step's checks (cubature of ncub^2
 * points for reverted sites); tensor_cores: 1 = tcgen05 pass, 0 = CUDA cores;
 * counts (host [2]) = sites reverted for precision / by the spot check */
int bn_mlp_sites(bn_mlp* h, void* stream, int64_t n, const float* pm, const float* pv, const float* y, int32_t ncub,
                 int32_t spot, double tol, int32_t tensor_cores, float* ext, uint32_t* counts);
/* network outputs (standardised) for standardised features */
int bn_mlp_forward(bn_mlp* h, void* stream, int32_t n, const float* xn, float* out);
/* mean squared error over all outputs and its gradient (host grad[num_params]) */
int bn_mlp_loss_grad(bn_mlp* h, void* stream, int32_t n, const float* xn, const float* tn, double* loss, float* grad);
/* Adam on random mini-batches; *loss = the last mini-batch's loss */
int bn_mlp_train(bn_mlp* h, void* stream, int32_t n, const float* xn, const float* tn, int32_t steps, int32_t bsz,
                 float lr, uint32_t seed, double* loss);
/* use the network for the model's two-latent VI sites (h = null: back to cubature);
 * every spot-th site is also integrated by cubature and reverts to it when the
 * derivatives differ by more than tol (relative); sites whose predicted diagonal
 * precision (-h11, -h22) is not positive always revert.  Counts go to result
 * slots BN_RES_SURR_PSD / _SPOT. */
int bn_model_set_surrogate(bn_model* m, bn_mlp* h, int32_t spot, double tol);

/* Batched product C_i = alpha op(A_i) op(B_i) + beta C0_i (device float32,
 * contiguous row-major matrices, batch strides M K, K N, M N; op = transpose when
 * ta / tb): tensor_cores = 1 runs the TMA-fed tcgen05 3xTF32 kernel, which needs
 * each operand's contiguous extent (K for A, N for B untransposed; M, K
 * transposed) to be a multiple of 4 and returns BN_ERR_ARG otherwise; 0 runs the
 * CUDA-core tiles, any shape (the kernels behind the spatio-temporal path; no
 * reference counterpart). */
int bn_dense_gemm(void* stream, int32_t tensor_cores, int32_t batch, int32_t ta, int32_t tb, int32_t M, int32_t N,
                  int32_t K, float alpha, const float* A, const float* B, float beta, const float* C0, float* C);

/* Batched in-place inverse with partial pivoting (device float32, contiguous
 * row-major n x n matrices, batch stride n n): engine 0 runs the shared-memory
 * Gauss-Jordan kernel, 1 the register-resident one (n <= 200; the one the
 * spatio-temporal filter combine uses), 2 the register-resident one with the
 * diagonal pivots taken in order, for symmetric positive definite matrices (the
 * spatio-temporal smoother gains); logdet (device, may be null) receives
 * sum log|pivot| per matrix and *status (device, may be null) is or-ed with 1 when
 * a pivot is zero (the kernels behind the spatio-temporal path; no reference
 * counterpart). */
int bn_dense_inverse(void* stream, int32_t engine, int32_t batch, int32_t n, float* A, double* logdet,
                     int32_t* status);

/* ---------------------------------------------------------------------------
 * Time segments (no counterpart in the reference): one long series split into
 * G consecutive segments, one per rank or per GPU, each a bn_model over its own
 * points.  A step runs in three phases with two small exchanges in between:
 *   phase 0: site update + local filter scan; total = the segment's filter
 *            element (bn_model_element_sizes: filter_words doubles)
 *   [gather the G filter totals; the state entering segment g is the fold
 *    bn_segment_filter_state over totals 0..g-1, starting from null]
 *   phase 1: boundary = that state (null for g = 0); filter, RTS elements; total
 *            = the segment's smoother element (smoother_words doubles)
 *   [gather the smoother totals; the smoothed state at the first step of segment
 *    g+1 is the fold bn_segment_smoother_state over totals G-1..g+1, from null]
 *   phase 2: boundary = that state (null for the last segment); smoother, site
 *            expectations, energy terms; bn_model_result then holds this
 *            segment's sums (energy, log marginal, ... add up across segments).
 * bn_model_set_segment marks a segment that continues an earlier one
 * (continue_left: its dt[0] is the step from the previous segment's last point)
 * and one that is followed by another (more_right, with dt_next the step to the
 * next segment's first point).  Totals and boundaries are host float64 arrays
 * in the flat element layouts: filter (A[d][d], b[d], C[d][d], J[d][d], eta[d]),
 * smoother (E[d][d], g[d], L[d][d]), state (m[d], P[d][d]).
 * ------------------------------------------------------------------------- */
int bn_model_set_segment(bn_model* m, int32_t continue_left, int32_t more_right, double dt_next);
int bn_model_element_sizes(bn_model* m, int32_t* filter_words, int32_t* smoother_words, int32_t* state_words);
int bn_segment_step(bn_model* m, void* stream, int32_t phase, int32_t newton, double lr, const void* dt,
                    const void* y, const bn_site_state* s, const double* boundary, double* total);
/* host-only folds of the exchanged totals (float64; no GPU) */
int bn_segment_filter_state(int32_t d, const double* state_in, const double* elem, double* state_out);
int bn_segment_smoother_state(int32_t d, const double* elem, const double* state_in, double* state_out);

/* ---------------------------------------------------------------------------
 * Spatio-temporal models (sparse in space): bayesnewton's MarkovVariationalGP
 * with a SpatioTemporalKernel (kernels.py:385-586) -- the temporal Matern prior
 * of each of M spatial inducing inputs z, the spatial kernel's conditional
 * f(t, R) | u(t) ~ N(B u(t), C) with the 'Full' conditional covariance, VI sites
 * in data space.  Inputs: dt [Nt] (time steps, dt[0] = 0), y [Nt, Nr] and the
 * spatial inputs R [Nt, Nr, spatial_dim] (device, float32, kept by the model);
 * the site state arrays (bn_site_state) are [Nt * Nr] scalars and post_mean /
 * post_var receive the data-space marginals of f.  Float32 only.
 * ------------------------------------------------------------------------- */
typedef struct bn_st_desc {
  int32_t temporal_kind;        /* BN_KIND_MATERN12 / 32 / 52 */
  double temporal_variance;
  double temporal_lengthscale;
  int32_t spatial_kind;         /* BN_KIND_MATERN12 / 32 / 52 */
  double spatial_variance;
  double spatial_lengthscale;
  int32_t num_inducing;         /* M, state dimension M x (temporal state size) <= 216 */
  int32_t spatial_dim;          /* 1 .. 3 */
  const double* z;              /* host [M, spatial_dim], read at create / set_prior */
  int32_t conditional;          /* 0: 'Full' or 'FIC' (the same diagonal, all VI reads); 1: 'DTC' (C = 0) */
} bn_st_desc;

typedef struct bn_st_model bn_st_model;

/* replaces the model construction of models.py:118-132 with a SpatioTemporalKernel */
int bn_st_create(const bn_st_desc* prior, const bn_lik_desc* lik, int64_t num_time, int32_t num_space,
                 const void* spatial_inputs, bn_st_model** out);
void bn_st_destroy(bn_st_model* m);
int bn_st_set_prior(bn_st_model* m, const bn_st_desc* prior);
int bn_st_set_likelihood(bn_st_model* m, const bn_lik_desc* lik);
/* MarkovGaussianProcess.update_posterior (basemodels.py:689-706) in its
 * spatio-temporal case, plus the site expectations and energy terms */
int bn_st_update_posterior(bn_st_model* m, void* stream, const void* dt, const void* y, const bn_site_state* s);
/* InferenceMixin.inference (inference.py:65-90), VI, plus the energy */
int bn_st_newton_step(bn_st_model* m, void* stream, double lr, const void* dt, const void* y,
                      const bn_site_state* s);
int bn_st_result(bn_st_model* m, void* stream, double* out, int32_t* status);
/* posterior_mean [Nt, M] and posterior_variance [Nt, M, M] (device) of the last step */
int bn_st_latent_posterior(bn_st_model* m, void* stream, void* mean, void* cov);
/* Prediction of f at test times and spatial inputs (MarkovGaussianProcess.predict,
 * basemodels.py:766-816, spatio-temporal case), from the smoother state of the
 * last step: x [Nt] sorted training times and x_test [num_test] (float64,
 * device), spatial_test [num_test, num_space_test, D] (float32, device); mean and
 * var [num_test, num_space_test] (float32, device): the marginals of f(t*, r*)
 * with the spatial conditional of kernels.py:486-505 (predict=True).  Keeps a
 * workspace of the model (Nt (d + 2 d^2) words plus the test outputs). */
int bn_st_predict(bn_st_model* m, void* stream, const double* x, int64_t num_test, const double* x_test,
                  int32_t num_space_test, const void* spatial_test, void* mean, void* var);
int bn_st_set_profiling(bn_st_model* m, int32_t on);
/* device time of the last profiled step (ms) */
int bn_st_step_time(bn_st_model* m, float* ms);

/* Copy the scalar results of the last step (BN_NRESULT doubles) and the status
 * bits to the host; synchronises the stream. */
int bn_model_result(bn_model* m, void* stream, double* out, int32_t* status);

/* ops-level Kalman filter:  dt [N], site_y [N, P], site_cov [N, P, P],
 * mask [N, P] (uint8, may be NULL) -> means [N, D], covs [N, D, D]; the log
 * marginal goes to result slot BN_RES_LOGLIK. */
int bn_kalman_filter(bn_model* m, void* stream, int32_t parallel, int32_t return_predict, const void* dt,
                     const void* site_y, const void* site_cov, const uint8_t* mask, void* means, void* covs);

/* ops-level RTS smoother:  dt [N] (already shifted: A_k = A(dt[k]) maps k to k+1),
 * filter_mean [N, D], filter_cov [N, D, D] -> means [N, P] / covs [N, P, P]
 * (or [N, D] / [N, D, D] when return_full), gains [N, D, D] (may be NULL). */
int bn_rts_smoother(bn_model* m, void* stream, int32_t parallel, int32_t return_full, const void* dt,
                    const void* filter_mean, const void* filter_cov, void* means, void* covs, void* gains);

/* ops-level prediction from smoothed states: the state at each test time given
 * the smoothed posterior of its two neighbouring training times.  Replaces
 * bayesnewton/utils.py temporal_conditional (:123-138) with predict_from_state
 * (:99-118) and compute_conditional_statistics (:172-213).  x [N] sorted training
 * times and x_test [num_test] (any order), float64 device arrays; mean [N, D],
 * cov [N, D, D], gains [N, D, D] from bn_rts_smoother(return_full = 1) on the
 * shifted dt.  Outputs test_mean [num_test, P] and test_cov [num_test, P, P]
 * projected by H, or [num_test, D] / [num_test, D, D] when return_full.  Test
 * times before the first / after the last training time use the reference's dummy
 * edge states (prior mean 0, covariance Pinf).  Computed in float64 whatever the
 * model's dtype.  A failed Cholesky of Q_mp sets BN_STATUS_NONPD. */
int bn_temporal_conditional(bn_model* m, void* stream, const double* x, int64_t num_test, const double* x_test,
                            const void* mean, const void* cov, const void* gains, int32_t return_full,
                            void* test_mean, void* test_cov);

/* Model-level prediction of f at test times (MarkovGaussianProcess.predict,
 * basemodels.py:766-816, temporal case): filter from the sites in s, smoother
 * with gains into a workspace of the model (5 N D^2 words, allocated by the first
 * call and kept), then bn_temporal_conditional.  x: the model's sorted training
 * times (float64, device).  Outputs [num_test, P] and [num_test, P, P].  Leaves
 * the last step's results and status as they were. */
int bn_model_predict(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                     const bn_site_state* s, const double* x, int64_t num_test, const double* x_test, void* test_mean,
                     void* test_cov);

/* log p(y* | data) = log E_N(f | mean, var)[p(y* | f)] per point, by the
 * likelihood's predictive rule: closed form for Gaussian (likelihoods.py:784-800),
 * Gauss-Hermite with the sum floored at 1e-8 otherwise (likelihoods.py:385-388,
 * cubature.py:249-276).  out [n] (may be NULL) gets NaN where y is NaN; sum_count
 * (host, may be NULL) gets the sum of the finite values and their count, so that
 * the reference's negative_log_predictive_density (basemodels.py:177-193) is
 * -sum / count; a non-NULL sum_count synchronises the stream.  Single-latent
 * likelihoods only (BN_ERR_UNSUPPORTED otherwise). */
int bn_model_log_density(bn_model* m, void* stream, int64_t n, const void* y, const void* mean, const void* var,
                         void* out, double* sum_count);

/* Data-space predictive mean and variance from f's (likelihood.predict,
 * likelihoods.py:493-506 -> cubature.py:438-465 with the conditional moments
 * :854-860 / :952-959; Gaussian: (mean, var + noise), :802-803).  Single-latent
 * likelihoods only. */
int bn_model_predict_y(bn_model* m, void* stream, int64_t n, const void* mean, const void* var, void* mean_y,
                       void* var_y);

/* Gradient of the variational energy (VariationalInference.energy,
 * bayesnewton/inference.py:197-222) with respect to the hyperparameters, as the
 * reference's objax.GradValues(model.energy) gives it (README.md:58-66; checked by
 * tests/test_gp_vs_markovgp_reg.py:77-118): the sites and the stored posterior
 * marginals in s are constants, so the kernel gradient is -d log Z / d theta of the
 * filter log marginal of the pseudo-observations (Fisher's identity over the
 * smoothed states of a filter + smoother pass at the current prior) and the
 * likelihood gradient is -sum_n d E_q[log p(y_n | f_n)] / d theta.  grad (host,
 * 2 C + 1 doubles for C prior components): d/d variance_c, d/d lengthscale_c for
 * each component in order, then d/d the Gaussian noise variance (0 for likelihoods
 * without a parameter).  Derivatives are with respect to the parameters
 * themselves; the reference's softplus-transformed variables need the factor
 * 1 - exp(-theta).  log_z (host, may be NULL) gets log Z.  The Newton, EP and PL
 * energies (inference.py:130-154, 286-325, 371-428) share the log Z term; their
 * likelihood terms are log p(y | m) and (1 / power) lZ at the cavity.  Matern
 * components on their closed-form layouts, one series; synchronises the stream.
 * Uses the prediction workspace of bn_model_predict. */
int bn_model_energy_grad(bn_model* m, void* stream, int32_t parallel, const void* dt, const void* y,
                         const bn_site_state* s, double* grad, double* log_z);

/* ---------------------------------------------------------------- infinite horizon
 * InfiniteHorizonGaussianProcess (bayesnewton/basemodels.py:1257-1308) on
 * equidistant times, single-latent sites: the steady-state Kalman filter and RTS
 * smoother of ops.py:796-1068 (kalman_filter_infinite_horizon,
 * rauch_tung_striebel_smoother_infinite_horizon, dare, rts_dare) with the
 * reference's warm-started Riccati recursions (dare_iters steps per call from the
 * previous call's solution, Pinf at first), the tied noise mean(nat2)^-1 and the
 * per-site gains of the heteroscedastic case.  Priors: one Matern component or
 * Sum(Matern52, Matern32).  The host drives the reference's call sequence:
 * InferenceMixin.inference = update_posterior, site_update, update_posterior;
 * VariationalInference.energy = log_lik (a fresh filter, advancing its Riccati
 * warm start) with the sums of the last update_posterior. */
typedef struct bn_ih_model bn_ih_model;
int bn_ih_create(const bn_prior_desc* prior, const bn_lik_desc* lik, int64_t num_data, int32_t dtype,
                 int32_t dare_iters, bn_ih_model** out);
int bn_ih_destroy(bn_ih_model* m);
int bn_ih_set_prior(bn_ih_model* m, const bn_prior_desc* prior); /* keeps the Riccati warm starts */
int bn_ih_set_likelihood(bn_ih_model* m, const bn_lik_desc* lik);
/* filter + smoother from the sites in s (dt: the constant step); writes the
 * posterior marginals, the site expectations at them and the energy sums */
int bn_ih_update_posterior(bn_ih_model* m, void* stream, double dt, int32_t heteroscedastic, const void* y,
                           const bn_site_state* s);
/* damped Newton update of the sites from the expectations cached by the last
 * bn_ih_update_posterior (inference.py:21-39, 83-86) */
int bn_ih_site_update(bn_ih_model* m, void* stream, double lr, const bn_site_state* s);
/* the filter alone: the log marginal of the pseudo-observations (compute_log_lik) */
int bn_ih_log_lik(bn_ih_model* m, void* stream, double dt, int32_t heteroscedastic, const void* y,
                  const bn_site_state* s);
/* BN_NRESULT doubles as bn_model_result (energy from the latest log marginal and
 * the last update_posterior's sums); synchronises the stream */
int bn_ih_result(bn_ih_model* m, void* stream, double* out, int32_t* status);
/* the Riccati warm starts (D x D each, host, may be NULL); synchronises */
int bn_ih_dare_state(bn_ih_model* m, void* stream, double* filter, double* smoother);

/* The parallel Kalman filter of bn_kalman_filter for callers that cannot
 * allocate device memory (a framework that owns all allocations through its own
 * arena, a real-time loop that may not allocate after start-up): it needs no
 * bn_model and allocates nothing.  No counterpart in the reference, which has no
 * allocation-free entry point.  float32 only; priors: a single Matern12/32/52/72,
 * or the sum of exactly two components Matern52 + Matern32 given in that order
 * (combine = BN_COMBINE_SUM; any other sum, including Matern32 + Matern52,
 * returns BN_ERR_UNSUPPORTED).  Same arrays as bn_kalman_filter; the log marginal
 * is written to log_lik (one double in device memory, may be NULL) and the scan's
 * BN_STATUS_* bits of this call (e.g. BN_STATUS_SINGULAR) to status (one int32 in
 * device memory, may be NULL), both on `stream` when the call's kernels end.
 * Scratch is a fixed 16 MiB array in the library's device memory, held by every
 * GPU that loads the library until exit; long series run with longer chunks per
 * thread to fit it, and a call that still needs more (about N > 4.8e7 for state
 * dim 5) returns BN_ERR_SCRATCH and launches nothing.  The first call on each
 * device looks up that array's address: make it before any stream capture, and do
 * not use the entry point across a device reset (the address is kept per device
 * for the life of the process).  All calls on a device share the array, so calls
 * that overlap on the GPU race and must be serialised by the caller. */
int bn_kalman_filter_noalloc(const bn_prior_desc* prior, int64_t num_data, void* stream, int32_t return_predict,
                             const void* dt, const void* site_y, const void* site_cov, const uint8_t* mask,
                             void* means, void* covs, double* log_lik, int32_t* status);

/* Diagnostics: while on, each parallel step records CUDA events between its
 * kernels on the caller's stream (the step then runs without its CUDA graph). */
int bn_model_set_profiling(bn_model* m, int32_t on);
/* Durations (ms) of the kernels of the last profiled step, in launch order:
 * filter_reduce, filter_blocks, filter_rerun, smoother_blocks, smoother_rerun,
 * site_tail (0 when the tail runs inside smoother_rerun).  Waits for that step. */
int bn_model_kernel_times(bn_model* m, float* ms, int32_t n);

/* Failure-detection probe (no counterpart in the reference, whose JAX code has
 * no device waits): launches one thread on `stream` that waits on an mbarrier
 * phase nothing completes, giving up after `polls` polls (status[0] = 1 when it
 * gave up), then completes the phase itself and waits again (status[1] = 1 when
 * that wait succeeded).  status: two int32 in device memory, written when the
 * kernel ends; polls in [1, 2^20], else BN_ERR_ARG before any launch.  The
 * tensor-core kernels bound their mbarrier waits the same way and report a wait
 * that gave up through their error flag instead of hanging. */
int bn_bounded_wait_probe(void* stream, uint32_t polls, int32_t* status);

/* The float32 transition A(dt) and process noise Q(dt) = Pinf - A Pinf A^T
 * (ops.py:149-151) of one Matern block of `size` 1..4 (Matern12/32/52/72, kernels.py:
 * 123-382), written row-major to a and q (size x size floats, host memory), computed
 * exactly as the float32 kernels compute them: Q without the cancellation of the
 * Pinf - A Pinf A^T form for lam dt < 2.  Host-only; needs no GPU. */
int bn_matern_process_noise(int32_t size, double variance, double lengthscale, double dt, float* a, float* q);

/* The Gauss-Hermite rule the site kernels use: n nodes x and weights w (host
 * memory), already scaled by sqrt(2) and 1/sqrt(pi) as bayesnewton/cubature.py:76-84
 * scales numpy's hermgauss.  Host-only; needs no GPU. */
int bn_gauss_hermite(int32_t n, double* x, double* w);

/* Library build information: a static string. */
const char* bn_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* BNX_H */
