// Compile-time block layout of the state and the type-erased engine interface.
// Kept free of device code so the C-ABI translation unit instantiates no kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bnx.h"

namespace bn {

// Block-diagonal layout of the state: one block per prior component.
template <int... Bs>
struct Layout {
  static constexpr int NC = sizeof...(Bs);
  static constexpr int D = (0 + ... + Bs);
  __host__ __device__ static constexpr int size(int c) {
    constexpr int s[] = {Bs...};
    return s[c];
  }
  __host__ __device__ static constexpr int off(int c) {
    int o = 0;
    for (int i = 0; i < c; ++i) o += size(i);
    return o;
  }
  __host__ __device__ static constexpr int comp_of(int i) {
    int c = 0;
    while (c + 1 < NC && off(c + 1) <= i) ++c;
    return c;
  }
  __host__ __device__ static constexpr int lo(int i) { return off(comp_of(i)); }
  __host__ __device__ static constexpr int hi(int i) { return off(comp_of(i)) + size(comp_of(i)); }
};

struct EngineBase {
  virtual ~EngineBase() {}
  virtual int set_prior(const bn_prior_desc* d) = 0;
  virtual int set_lik(const bn_lik_desc* d) = 0;
  virtual int update_posterior(cudaStream_t st, int parallel, const void* dt, const void* y,
                               const bn_site_state& s) = 0;
  virtual int newton_step(cudaStream_t st, int parallel, double lr, const void* dt, const void* y,
                          const bn_site_state& s) = 0;
  virtual int kalman_filter(cudaStream_t st, int parallel, int return_predict, const void* dt, const void* sy,
                            const void* sR, const uint8_t* mask, void* om, void* oP) = 0;
  virtual int rts_smoother(cudaStream_t st, int parallel, int return_full, const void* dt, const void* fm,
                           const void* fP, void* om, void* oP, void* oG) = 0;
  virtual int result(cudaStream_t st, double* out, int32_t* status) = 0;
  virtual int set_profiling(int on) = 0;
  virtual int set_series(int64_t nseries, const int64_t* offsets, const double* var, const double* ell,
                         const int32_t* lik_kind, const double* lik_var) = 0;
  virtual int series_energy(cudaStream_t st, double* out) = 0;
  virtual int set_segment(int continue_left, int more_right, double dt_next) = 0;
  virtual int segment_step(cudaStream_t st, int phase, bool newton, double lr, const void* dt, const void* y,
                           const bn_site_state& s, const double* boundary, double* total) = 0;
  virtual void element_sizes(int* fe, int* se, int* stw) = 0;
  virtual int set_surrogate(bn_mlp* h, int spot, double tol) = 0;
  virtual int temporal_conditional(cudaStream_t st, const double* x, int64_t nt, const double* xt, const void* sm,
                                   const void* sP, const void* G, int full, void* om, void* oP) = 0;
  virtual int predict(cudaStream_t st, int parallel, const void* dt, const void* y, const bn_site_state& s,
                      const double* x, int64_t nt, const double* xt, void* om, void* oP) = 0;
  virtual int log_density(cudaStream_t st, int64_t n, const void* y, const void* m, const void* v, void* out,
                          double* sum_count) = 0;
  virtual int predict_y(cudaStream_t st, int64_t n, const void* m, const void* v, void* my, void* vy) = 0;
  virtual int energy_grad(cudaStream_t st, int parallel, const void* dt, const void* y, const bn_site_state& s,
                          double* out, double* log_z) = 0;
  int64_t num_series = 0;
  virtual int kernel_times(float* ms, int n) = 0;
  int state_dim = 0, site_dim = 0, spt = 0, nblocks = 0, obs_dim = 1;
  int64_t num_data = 0;
};

// Defined in bn_engine.cuh, explicitly instantiated in the bn_inst_*.cu units.
template <typename T, typename Lay, int P>
EngineBase* make_engine(int64_t n, int obs, int spt, bool dense, int* err);

// Compiled configurations: X(T, P, block sizes...).  Priors whose block sizes are
// not listed run on the single-block ("dense") layout of the same D and P, with
// every block's transition taken by the generic expm path.
#define BN_CONFIGS_F32(X)                                                                             \
  X(float, 1, 1) X(float, 1, 2) X(float, 1, 3) X(float, 1, 4) X(float, 1, 3, 2) X(float, 1, 2, 2)    \
  X(float, 1, 5) X(float, 1, 6) X(float, 1, 7) X(float, 1, 8)                                         \
  X(float, 2, 1, 1) X(float, 2, 2, 2) X(float, 2, 3, 3) X(float, 2, 6)
#define BN_CONFIGS_F64(X)                                                                             \
  X(double, 1, 1) X(double, 1, 2) X(double, 1, 3) X(double, 1, 3, 2) X(double, 1, 5)                  \
  X(double, 2, 2, 2) X(double, 2, 3, 3)

}  // namespace bn
