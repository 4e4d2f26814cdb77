// Host side of one compiled configuration (dtype T, block layout L, site dim P):
// owns the device workspace of a model and enqueues the kernel sequences.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <type_traits>
#include <vector>
#include <cstring>

#include "bn_host.h"
#include "bn_cscan.cuh"
#include "bn_grad.cuh"
#include "bn_mlp.h"
#include "bn_predict.cuh"
#include "bn_scan.cuh"

namespace bn {

constexpr int kTPB = 128;   // threads per block of the chunked scans
constexpr int kCtaPerSM = 2; // chunk kernels' CTAs per SM the chunk length aims at
constexpr int kTPB2 = 256;  // threads of the single-CTA block-aggregate scans (one aggregate each up to 256;
                            // 128 when 256 elements would not fit in shared memory)
constexpr int kTPBT = 256;  // threads per block of the site-tail kernel
constexpr int kSPTT = 4;    // sites per thread of the site-tail kernel


// Fill the device prior.  When `dense` is set every block is handled by the
// generic expm path (the layout is then a single D-block).
template <typename T, int D, int P>
int build_ssm(const bn_prior_desc* d, bool dense, SSM<T, D, P>& s) {
  std::memset(&s, 0, sizeof(s));
  int off = 0;
  double F[D][D] = {}, Pi[D][D] = {};
  const int nc = d->num_components;
  if (nc < 1 || nc > BN_MAX_COMPONENTS) return BN_ERR_ARG;
  int offs[BN_MAX_COMPONENTS];
  for (int c = 0; c < nc; ++c) {
    const int sz = d->size[c];
    if (sz < 1 || off + sz > D) return BN_ERR_ARG;
    offs[c] = off;
    if (d->kind[c] == BN_KIND_FEEDBACK) {
      for (int i = 0; i < sz; ++i)
        for (int j = 0; j < sz; ++j) {
          F[off + i][off + j] = d->feedback[(off + i) * BN_MAX_STATE + off + j];
          Pi[off + i][off + j] = d->pinf[(off + i) * BN_MAX_STATE + off + j];
        }
    } else {
      double f[16], p[16];
      if (!matern_blocks(d->kind[c], sz, d->variance[c], d->lengthscale[c], f, p)) return BN_ERR_ARG;
      for (int i = 0; i < sz; ++i)
        for (int j = 0; j < sz; ++j) {
          F[off + i][off + j] = f[i * sz + j];
          Pi[off + i][off + j] = p[i * sz + j];
        }
    }
    off += sz;
  }
  if (off != D) return BN_ERR_ARG;
  if (dense) {
    s.ncomp = 1;
    s.kind[0] = BN_KIND_FEEDBACK;
  } else {
    s.ncomp = nc;
    for (int c = 0; c < nc; ++c) {
      s.kind[c] = d->kind[c];
      s.lam[c] = T(matern_lam(d->kind[c], d->lengthscale[c]));
      s.var[c] = T(d->variance[c]);
    }
  }
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) {
      s.F[i][j] = T(F[i][j]);
      s.Pinf[i][j] = T(Pi[i][j]);
    }
  if (d->combine == BN_COMBINE_SUM) {
    if (P != 1) return BN_ERR_ARG;
    for (int c = 0; c < nc; ++c) s.H[0][offs[c]] = T(1);
  } else {
    if (P != nc) return BN_ERR_ARG;
    for (int c = 0; c < nc; ++c) s.H[c][offs[c]] = T(1);
  }
  for (int p = 0; p < P; ++p) {
    double v = 0.0;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) v += double(s.H[p][i]) * Pi[i][j] * double(s.H[p][j]);
    s.hph[p] = T(v);
  }
  return BN_OK;
}

template <typename T>
int build_lik(const bn_lik_desc* d, LikParams<T>& l) {
  std::memset(&l, 0, sizeof(l));
  l.kind = d->kind;
  l.method = d->method;
  l.ncub = d->num_cub > 0 ? d->num_cub : 20;
  if (l.ncub > BN_MAX_CUB) return BN_ERR_ARG;
  l.ensure_psd = d->ensure_psd;
  l.score_form = d->score_form;
  l.variance = T(d->variance);
  l.binsize = T(d->binsize > 0 ? d->binsize : 1.0);
  l.log_binsize = T(std::log(d->binsize > 0 ? d->binsize : 1.0));
  l.power = T(d->power > 0 ? d->power : 1.0);
  double x[BN_MAX_CUB], w[BN_MAX_CUB];
  gauss_hermite(l.ncub, x, w);
  for (int i = 0; i < l.ncub; ++i) {
    l.cub_x[i] = T(x[i]);
    l.cub_w[i] = T(w[i]);
  }
  return BN_OK;
}

#define BN_CUDA_TRY(x)                     \
  do {                                     \
    if ((x) != cudaSuccess) return BN_ERR_CUDA; \
  } while (0)

template <typename T, typename Lay, int P>
struct Engine : EngineBase {
  static constexpr int DD = Lay::D;
  static constexpr int TPB2 = (kTPB2 * sizeof(FElem<T, DD>) <= 200 * 1024) ? kTPB2 : kTPB2 / 2;
  using A = ScanArgs<T, DD, P>;
  using Z = Sz<T, DD>;
  bool dense = false;
  SSM<T, DD, P> ssm;
  SSM<double, DD, P> ssm64;  // the same prior in float64, for prediction and gradients
  int comp_kind[BN_MAX_COMPONENTS] = {};
  double comp_var[BN_MAX_COMPONENTS] = {}, comp_ell[BN_MAX_COMPONENTS] = {};
  double lik_var64 = 0.0;
  LikParams<T> lik;
  // workspace
  T *fx = nullptr, *fagg = nullptr, *fin = nullptr, *fst = nullptr;
  T *sx = nullptr, *sagg = nullptr, *sin = nullptr;
  double *part = nullptr, *res = nullptr, *tpart = nullptr;
  int ntail = 1;
  bool split_tail = true;
  // single series: hand the filtered states (m, packed P: 20 words at state dim 5)
  // from F3 to S3 and let S3 recompute each step's gain, instead of storing the
  // 45-word RTS elements (E, g, L).  The records fit the L2 between the two
  // passes, F3 drops its per-step Cholesky and solve, and S3, which waited on
  // memory, gets the arithmetic.  The element hand-off stays for many series and
  // time segments (BN_STORE_REC=0 selects it everywhere).
  bool store_rec = true;
  unsigned* counter = nullptr;
  int* status = nullptr;
  void* pool = nullptr;
  // CUDA graph of the parallel step, replayed while its launch parameters hold
  struct GraphKey {
    int newton = -1;
    double lr = 0.0;
    const void* p[9] = {};
    unsigned version = 0;
    bool operator==(const GraphKey& o) const {
      if (newton != o.newton || lr != o.lr || version != o.version) return false;
      for (int i = 0; i < 9; ++i)
        if (p[i] != o.p[i]) return false;
      return true;
    }
  };
  GraphKey gkey;
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t cap_stream = nullptr;
  unsigned version = 1;
  bool use_graph = true;
  // per-kernel timing (diagnostics): events between the step's kernels
  bool profiling = false;
  cudaEvent_t ev[7] = {};

  // batched series
  bool batch = false;
  void* bpool = nullptr;
  int* d_sid = nullptr;
  int* d_ser_lik = nullptr;
  T *d_ser_var = nullptr, *d_ser_ell = nullptr, *d_ser_likvar = nullptr, *d_ll_step = nullptr;
  T* d_ser_gauss = nullptr;
  double* d_ser_energy = nullptr;
  static constexpr bool kBatchable = (P == 1 && Lay::NC == 1 && Lay::D <= 4);

  // prediction workspace (allocated by the first prediction): filtered and
  // smoothed states and smoother gains of every step, and its own result / status
  // words so that a prediction leaves the last step's results in place
  void* pred_buf = nullptr;
  T *p_fm = nullptr, *p_fP = nullptr, *p_sm = nullptr, *p_sP = nullptr, *p_G = nullptr;
  double* p_res = nullptr;
  int* p_status = nullptr;

  ~Engine() override {
    if (pred_buf) cudaFree(pred_buf);
    if (surr_buf) cudaFree(surr_buf);
    if (seg_buf) cudaFree(seg_buf);
    if (bpool) cudaFree(bpool);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (pool) cudaFree(pool);
  }

  int init(int64_t n, int obs, int spt, bool dense_) {
    dense = dense_;
    num_data = n;
    state_dim = DD;
    site_dim = P;
    obs_dim = obs;
    if (spt <= 0) {
      // aim at 2 resident blocks per SM of the 152 on a GB300: the shortest chunk
      // (a multiple of 4 steps, for F1's 16-byte staged loads) that needs at most
      // 2 x 152 blocks, up to 64 steps
      const double per = double(n) / (152.0 * double(kCtaPerSM) * kTPB);
      int l = 4 * int(std::ceil(per / 4.0));
      spt = l < 4 ? 4 : (l > 64 ? 64 : l);
    }
    this->spt = spt;
    const char* ng = std::getenv("BN_NO_GRAPH");
    use_graph = !(ng && ng[0] == '1');
    const char* ft = std::getenv("BN_FUSED_TAIL");
    split_tail = !(ft && ft[0] == '1');
    const char* sr = std::getenv("BN_STORE_REC");
    store_rec = !(sr && sr[0] == '0');
    const int64_t nchunks = (n + spt - 1) / spt;
    nblocks = int((nchunks + kTPB - 1) / kTPB);
    if (nblocks < 1) nblocks = 1;
    const size_t nb = size_t(nblocks);
    const size_t rec = std::max(nb * kTPB * size_t(spt) * size_t(Z::RECE), size_t(n) * Z::REC);
    size_t sizes[] = {nb * Z::FE * kTPB, nb * Z::FE, nb * Z::ST, rec, nb * Z::SE * kTPB, nb * Z::SE, nb * Z::ST};
    size_t tot = 0;
    for (size_t s : sizes) tot += ((s * sizeof(T) + 255) / 256) * 256;
    ntail = int((n + kTPBT * kSPTT - 1) / (kTPBT * kSPTT));
    const size_t dbl = ((nb * BN_NPART + BN_NRESULT + size_t(ntail) * 2) * sizeof(double) + 255) / 256 * 256;
    tot += dbl + 256;
    BN_CUDA_TRY(cudaMalloc(&pool, tot));
    BN_CUDA_TRY(cudaMemset(pool, 0, tot));
    char* p = static_cast<char*>(pool);
    T** ptrs[] = {&fx, &fagg, &fin, &fst, &sx, &sagg, &sin};
    for (int i = 0; i < 7; ++i) {
      *ptrs[i] = reinterpret_cast<T*>(p);
      p += ((sizes[i] * sizeof(T) + 255) / 256) * 256;
    }
    part = reinterpret_cast<double*>(p);
    res = part + nb * BN_NPART;
    tpart = res + BN_NRESULT;
    p += dbl;
    counter = reinterpret_cast<unsigned*>(p);
    status = reinterpret_cast<int*>(p + 16);
    // dynamic shared memory beyond 48 KB needs an opt-in per kernel
    const int fsm = f1_smem();
    const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_reduce_kernel<T, Lay, P, SITE_NEWTON, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_reduce_kernel<T, Lay, P, SITE_NAT, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_reduce_kernel<T, Lay, P, SITE_GIVEN, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_blocks_kernel<T, Lay, P, TPB2>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, TPB2 * int(sizeof(FElem<T, DD>))));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_ELEM, true, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, ssm_b));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_INTERNAL, true, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, ssm_b));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_rerun_kernel<T, Lay, P, SITE_GIVEN, STORE_REF, false, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, ssm_b));
    BN_CUDA_TRY(cudaFuncSetAttribute(smoother_reduce_kernel<T, Lay, P, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, ssm_b));
    BN_CUDA_TRY(cudaFuncSetAttribute(smoother_blocks_kernel<T, Lay, P, TPB2>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, TPB2 * int(sizeof(SElem<T, DD>))));
    setup_cluster_scans();
    return BN_OK;
  }

  int set_prior(const bn_prior_desc* d) override {
    ++version;
    for (int c = 0; c < d->num_components && c < BN_MAX_COMPONENTS; ++c) {
      comp_kind[c] = d->kind[c];
      comp_var[c] = d->variance[c];
      comp_ell[c] = d->lengthscale[c];
    }
    const int e = build_ssm<double, DD, P>(d, dense, ssm64);
    if (e != BN_OK) return e;
    return build_ssm<T, DD, P>(d, dense, ssm);
  }
  int set_lik(const bn_lik_desc* d) override {
    if (d->method < BN_METHOD_VI || d->method > BN_METHOD_PL) return BN_ERR_ARG;
    // posterior linearisation: single-latent sites (the reference's multi-latent SLR is its own method)
    if (d->method == BN_METHOD_PL && P != 1) return BN_ERR_UNSUPPORTED;
    ++version;
    lik_var64 = d->variance;
    return build_lik<T>(d, lik);
  }

  A args() const {
    A a;
    std::memset(&a, 0, sizeof(a));
    a.N = num_data;
    a.L = spt;
    a.nblocks = nblocks;
    a.obs_dim = obs_dim;
    a.ssm = ssm;
    a.lik = lik;
    a.fx = fx;
    a.fagg = fagg;
    a.fin = fin;
    a.fst = fst;
    a.sx = sx;
    a.sagg = sagg;
    a.sin = sin;
    a.part = part;
    a.tpart = tpart;
    a.sid = d_sid;
    a.ser_var = d_ser_var;
    a.ser_ell = d_ser_ell;
    a.ser_lik = d_ser_lik;
    a.ser_likvar = d_ser_likvar;
    a.ll_step = d_ll_step;
    a.ser_gauss = d_ser_gauss;
    a.ser_energy = d_ser_energy;
    a.ext = surr ? static_cast<const T*>(surr_buf) : nullptr;
    a.ntail_blocks = ntail;
    a.counter = counter;
    a.result = res;
    a.status = status;
    return a;
  }

  int posterior_pass(cudaStream_t st, int parallel, bool newton, double lr, const void* dt, const void* y,
                     const bn_site_state& ss) {
    A a = args();
    a.lr = T(lr);
    a.dt = static_cast<const T*>(dt);
    a.y = static_cast<const T*>(y);
    a.nat1 = static_cast<T*>(ss.nat1);
    a.nat2 = static_cast<T*>(ss.nat2);
    a.post_mean = static_cast<T*>(ss.post_mean);
    a.post_var = static_cast<T*>(ss.post_var);
    a.grad = static_cast<T*>(ss.grad);
    a.hess = static_cast<T*>(ss.hess);
    a.lin = static_cast<T*>(ss.lin);
    a.shift_dt = 1;
    {
      const void* ps[6] = {dt, ss.grad, ss.hess, ss.lin, ss.nat1, ss.nat2};
      // 16-byte copies of four steps: every chunk must start on a multiple of 4 steps
      bool al = std::is_same<T, float>::value && P == 1 && spt % 4 == 0;
      for (const void* q : ps) al = al && (reinterpret_cast<uintptr_t>(q) % 16 == 0);
      a.staged = al ? 1 : 0;
    }
    if (!parallel && batch) return BN_ERR_UNSUPPORTED;
    if (!parallel) {
      BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
      if (newton) seq_filter_kernel<T, Lay, P, SITE_NEWTON, STORE_SEQ><<<1, 1, 0, st>>>(a);
      else seq_filter_kernel<T, Lay, P, SITE_NAT, STORE_SEQ><<<1, 1, 0, st>>>(a);
      seq_smoother_kernel<T, Lay, P, STORE_SEQ, true><<<1, 1, 0, st>>>(a);
      BN_CUDA_TRY(cudaGetLastError());
      return BN_OK;
    }
    if (!use_graph || profiling) return enqueue_step(st, a, newton);
    GraphKey key;
    key.newton = newton ? 1 : 0;
    key.lr = newton ? lr : 0.0;
    const void* ps[9] = {dt, y, ss.nat1, ss.nat2, ss.post_mean, ss.post_var, ss.grad, ss.hess, ss.lin};
    for (int i = 0; i < 9; ++i) key.p[i] = ps[i];
    key.version = version;
    if (!gexec || !(key == gkey)) {
      if (gexec) {
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
      }
      if (!cap_stream) BN_CUDA_TRY(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
      BN_CUDA_TRY(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
      const int err = enqueue_step(cap_stream, a, newton);
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(cap_stream, &graph);
      if (err != BN_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return BN_ERR_CUDA;
      }
      const cudaError_t ie = cudaGraphInstantiate(&gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        gexec = nullptr;
        return BN_ERR_CUDA;
      }
      gkey = key;
    }
    BN_CUDA_TRY(cudaGraphLaunch(gexec, st));
    return BN_OK;
  }

  // status reset + F1 -> F2 -> F3 -> S2 -> S3 on one stream (events between the
  // kernels when profiling)
  int enqueue_step(cudaStream_t st, const A& a, bool newton) {
    if constexpr (kBatchable) {
      if (batch) return enqueue_step_batch(st, a, newton);
    }
    BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    const int fsm = f1_smem();
    const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
    auto mark = [&](int i) {
      if (profiling) cudaEventRecord(ev[i], st);
    };
    mark(0);
    if (newton) filter_reduce_kernel<T, Lay, P, SITE_NEWTON, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
    else filter_reduce_kernel<T, Lay, P, SITE_NAT, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
    mark(1);
    launch_filter_blocks(st, a);
    mark(2);
    const bool rec = store_rec && (split_tail || surr) && !a.seg_more && !a.seg_right && !a.seg_continue &&
                     !a.seg_left;
    if (rec) filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_INTERNAL, true, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
    else filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_ELEM, true, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
    mark(3);
    launch_smoother_blocks(st, a);
    mark(4);
    if (split_tail || surr) {
      if (rec) smoother_rerun_kernel<T, Lay, P, STORE_INTERNAL, false, kTPB><<<nblocks, kTPB, 0, st>>>(a);
      else smoother_rerun_kernel<T, Lay, P, STORE_ELEM, false, kTPB><<<nblocks, kTPB, 0, st>>>(a);
      mark(5);
      if constexpr (std::is_same<T, float>::value && P == 2) {
        if (surr) {
          BN_CUDA_TRY(cudaMemsetAsync(surr_counters(), 0, 2 * sizeof(unsigned), st));
          const int e = mlp_site_expectations(surr, st, num_data, a.post_mean, a.post_var, a.y, lik, surr_spot,
                                              surr_tol, surr_ext(), surr_counters(),
                                              reinterpret_cast<unsigned*>(static_cast<char*>(surr_buf) +
                                                                          size_t(num_data) * 6 * sizeof(float) + 256));
          if (e != BN_OK) return e;
        }
      }
      launch_tail(st, a);
      mark(6);
    } else {
      smoother_rerun_kernel<T, Lay, P, STORE_ELEM, true, kTPB><<<nblocks, kTPB, 0, st>>>(a);
      mark(5);
    }
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  // the site tail compiled for the model's method (single-latent sites)
  void launch_tail(cudaStream_t st, const A& a) {
    if constexpr (P == 1) {
      if (lik.method == BN_METHOD_VI) {
        site_tail_kernel<T, Lay, P, kTPBT, kSPTT, false, 0><<<ntail, kTPBT, 0, st>>>(a);
        return;
      }
      if (lik.method == BN_METHOD_NEWTON) {
        site_tail_kernel<T, Lay, P, kTPBT, kSPTT, false, 1><<<ntail, kTPBT, 0, st>>>(a);
        return;
      }
      site_tail_kernel<T, Lay, P, kTPBT, kSPTT, false, 2><<<ntail, kTPBT, 0, st>>>(a);
    } else {
      site_tail_kernel<T, Lay, P, kTPBT, kSPTT><<<ntail, kTPBT, 0, st>>>(a);
    }
  }

  // scans of the block aggregates: on a cluster of cl_size CTAs, one warp per
  // element (bn_cscan.cuh), or on one CTA, one aggregate per thread up to kTPB2
  static constexpr int kWPC = 16;  // warps per CTA of the cluster scans
  int cl_size = 0;
  static int cl_smem_f() { return kWPC * int(sizeof(WarpSlot<T, FElem<T, DD>, DD>)); }
  static int cl_smem_s() { return kWPC * int(sizeof(WarpSlot<T, SElem<T, DD>, DD>)); }
  template <typename K>
  static cudaError_t cl_launch(K kernel, int cl, int smem, cudaStream_t st, const A& a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cl, 1, 1);
    cfg.blockDim = dim3(kWPC * 32, 1, 1);
    cfg.dynamicSmemBytes = size_t(smem);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
  }
  // the largest cluster (16, else 8 CTAs) that can be resident; 0 when neither
  // (the single-CTA scans are used then)
  void setup_cluster_scans() {
    cl_size = 0;
    const char* cs = std::getenv("BN_CLUSTER_SCAN");
    if (cs && cs[0] == '0') return;
    auto kf = filter_blocks_cluster_kernel<T, Lay, P, kWPC>;
    auto ks = smoother_blocks_cluster_kernel<T, Lay, P, kWPC>;
    if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, cl_smem_f()) != cudaSuccess ||
        cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, cl_smem_s()) != cudaSuccess ||
        cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(ks, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    for (int cl : {16, 8}) {
      bool fits = true;
      for (int which = 0; which < 2; ++which) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cl, 1, 1);
        cfg.blockDim = dim3(kWPC * 32, 1, 1);
        cfg.dynamicSmemBytes = size_t(which ? cl_smem_s() : cl_smem_f());
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cl;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const cudaError_t e = which ? cudaOccupancyMaxActiveClusters(&n, ks, &cfg)
                                    : cudaOccupancyMaxActiveClusters(&n, kf, &cfg);
        if (e != cudaSuccess || n < 1) {
          cudaGetLastError();
          fits = false;
        }
      }
      if (fits) {
        cl_size = cl;
        return;
      }
    }
  }
  void launch_filter_blocks(cudaStream_t st, const A& a) {
    if (cl_size) {
      cl_launch(filter_blocks_cluster_kernel<T, Lay, P, kWPC>, cl_size, cl_smem_f(), st, a);
      return;
    }
    filter_blocks_kernel<T, Lay, P, TPB2><<<1, TPB2, TPB2 * int(sizeof(FElem<T, DD>)), st>>>(a);
  }
  void launch_smoother_blocks(cudaStream_t st, const A& a) {
    if (cl_size) {
      cl_launch(smoother_blocks_cluster_kernel<T, Lay, P, kWPC>, cl_size, cl_smem_s(), st, a);
      return;
    }
    smoother_blocks_kernel<T, Lay, P, TPB2><<<1, TPB2, TPB2 * int(sizeof(SElem<T, DD>)), st>>>(a);
  }

  // F1's dynamic shared memory: the block scan's elements, or the cp.async staging
  // buffers of its six input streams when larger
  static int f1_smem() {
    const int scan = kTPB * int(sizeof(FElem<T, DD>));
    const int stage = 2 * kNStream * kTPB * kSub * int(sizeof(float));
    return scan > stage ? scan : stage;
  }

  // many series concatenated: series-aware filter passes and site tail
  int enqueue_step_batch(cudaStream_t st, const A& a, bool newton) {
    if constexpr (kBatchable) {
      BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
      BN_CUDA_TRY(cudaMemsetAsync(d_ser_energy, 0, size_t(num_series) * sizeof(double), st));
      // the series-aware F1 does not stage its inputs: shared memory for the block scan only
      const int fsm = kTPB * int(sizeof(FElem<T, DD>));
      const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
      auto mark = [&](int i) {
        if (profiling) cudaEventRecord(ev[i], st);
      };
      mark(0);
      if (newton) filter_reduce_kernel<T, Lay, P, SITE_NEWTON, kTPB, true><<<nblocks, kTPB, fsm, st>>>(a);
      else filter_reduce_kernel<T, Lay, P, SITE_NAT, kTPB, true><<<nblocks, kTPB, fsm, st>>>(a);
      mark(1);
      launch_filter_blocks(st, a);
      mark(2);
      filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_ELEM, true, kTPB, true><<<nblocks, kTPB, ssm_b, st>>>(a);
      mark(3);
      launch_smoother_blocks(st, a);
      mark(4);
      smoother_rerun_kernel<T, Lay, P, STORE_ELEM, false, kTPB><<<nblocks, kTPB, 0, st>>>(a);
      mark(5);
      site_tail_kernel<T, Lay, P, kTPBT, kSPTT, true><<<ntail, kTPBT, 0, st>>>(a);
      mark(6);
      BN_CUDA_TRY(cudaGetLastError());
      return BN_OK;
    } else {
      return BN_ERR_UNSUPPORTED;
    }
  }

  int set_series(int64_t ns, const int64_t* off, const double* var, const double* ell, const int32_t* lk,
                 const double* lv) override {
    if constexpr (!kBatchable) {
      return BN_ERR_UNSUPPORTED;
    } else {
      if (ns < 1 || !off || !var || !ell || !lk || !lv || off[0] != 0 || off[ns] != num_data) return BN_ERR_ARG;
      if (lik.method == BN_METHOD_EP || lik.method == BN_METHOD_PL || ssm.kind[0] == BN_KIND_FEEDBACK)
        return BN_ERR_UNSUPPORTED;
      for (int64_t i = 0; i < ns; ++i) {
        if (off[i + 1] <= off[i]) return BN_ERR_ARG;
        if (!(ell[i] > 0.0) || !(var[i] > 0.0)) return BN_ERR_ARG;
        if (lk[i] != BN_LIK_GAUSSIAN && lk[i] != BN_LIK_POISSON_EXP && lk[i] != BN_LIK_BERNOULLI_LOGIT &&
            lk[i] != BN_LIK_BERNOULLI_PROBIT)
          return BN_ERR_ARG;
      }
      if (bpool) {
        cudaFree(bpool);
        bpool = nullptr;
      }
      const size_t n = size_t(num_data), S = size_t(ns);
      size_t sz[] = {n * sizeof(int), S * sizeof(int), S * sizeof(T), S * sizeof(T), S * sizeof(T), n * sizeof(T),
                     S * sizeof(double), 4 * S * sizeof(T)};
      size_t tot = 0;
      for (size_t b : sz) tot += (b + 255) / 256 * 256;
      BN_CUDA_TRY(cudaMalloc(&bpool, tot));
      char* p = static_cast<char*>(bpool);
      void** ptrs[] = {(void**)&d_sid, (void**)&d_ser_lik, (void**)&d_ser_var, (void**)&d_ser_ell,
                       (void**)&d_ser_likvar, (void**)&d_ll_step, (void**)&d_ser_energy, (void**)&d_ser_gauss};
      for (int i = 0; i < 8; ++i) {
        *ptrs[i] = p;
        p += (sz[i] + 255) / 256 * 256;
      }
      std::vector<int> sid(n);
      for (int64_t i = 0; i < ns; ++i)
        for (int64_t k = off[i]; k < off[i + 1]; ++k) sid[k] = int(i);
      std::vector<T> hv(S), he(S), hl(S), hg(4 * S);
      auto split = [](double x, T* o) {
        o[0] = T(x);
        o[1] = T(x - double(o[0]));
      };
      for (size_t i = 0; i < S; ++i) {
        hv[i] = T(var[i]);
        he[i] = T(ell[i]);
        hl[i] = T(lv[i]);
        // Gaussian series: var and 1 / var in float64, each split into a (head, tail) pair
        split(lv[i] > 0.0 ? lv[i] : 1.0, &hg[4 * i]);
        split(1.0 / (lv[i] > 0.0 ? lv[i] : 1.0), &hg[4 * i + 2]);
      }
      BN_CUDA_TRY(cudaMemcpy(d_sid, sid.data(), n * sizeof(int), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemcpy(d_ser_lik, lk, S * sizeof(int), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemcpy(d_ser_var, hv.data(), S * sizeof(T), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemcpy(d_ser_ell, he.data(), S * sizeof(T), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemcpy(d_ser_likvar, hl.data(), S * sizeof(T), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemcpy(d_ser_gauss, hg.data(), 4 * S * sizeof(T), cudaMemcpyHostToDevice));
      BN_CUDA_TRY(cudaMemset(d_ser_energy, 0, S * sizeof(double)));
      num_series = ns;
      batch = true;
      ++version;
      return BN_OK;
    }
  }

  int series_energy(cudaStream_t st, double* out) override {
    if (!batch || !out) return BN_ERR_ARG;
    BN_CUDA_TRY(cudaMemcpyAsync(out, d_ser_energy, size_t(num_series) * sizeof(double), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaStreamSynchronize(st));
    return BN_OK;
  }

  // ------------------------------------------------------------ learned sites
  bn_mlp* surr = nullptr;
  int surr_spot = 64;
  float surr_tol = 0.05f;
  void* surr_buf = nullptr;  // ext [N][6] floats, then 2 counters

  int set_surrogate(bn_mlp* h, int spot, double tol) override {
    if constexpr (!(std::is_same<T, float>::value && P == 2)) {
      return BN_ERR_UNSUPPORTED;
    } else {
      if (h && lik.kind != BN_LIK_HETERO_EXP && lik.kind != BN_LIK_HETERO_SOFTPLUS) return BN_ERR_UNSUPPORTED;
      if (h && lik.method != BN_METHOD_VI) return BN_ERR_UNSUPPORTED;
      if (h && !surr_buf)
        BN_CUDA_TRY(cudaMalloc(&surr_buf, size_t(num_data) * 6 * sizeof(float) + 256 +
                                              2 * (size_t(num_data) + 1) * sizeof(unsigned)));
      surr = h;
      surr_spot = spot;
      surr_tol = float(tol);
      ++version;
      return BN_OK;
    }
  }
  float* surr_ext() const { return static_cast<float*>(surr_buf); }
  unsigned* surr_counters() const {
    return reinterpret_cast<unsigned*>(static_cast<char*>(surr_buf) + size_t(num_data) * 6 * sizeof(float));
  }

  // ------------------------------------------------------------ time segments
  int seg_continue = 0, seg_more = 0;
  T seg_dt_next = T(0);
  void* seg_buf = nullptr;  // left state, right state, filter total, smoother total

  int set_segment(int continue_left, int more_right, double dt_next) override {
    if (batch) return BN_ERR_UNSUPPORTED;
    seg_continue = continue_left ? 1 : 0;
    seg_more = more_right ? 1 : 0;
    seg_dt_next = T(dt_next);
    ++version;
    if (!seg_buf) {
      const size_t words = size_t(2 * Z::ST + Z::FE + Z::SE);
      BN_CUDA_TRY(cudaMalloc(&seg_buf, words * sizeof(T)));
    }
    return BN_OK;
  }

  void element_sizes(int* fe, int* se, int* stw) override {
    if (fe) *fe = Z::FE;
    if (se) *se = Z::SE;
    if (stw) *stw = Z::ST;
  }

  // One phase of a step on a time segment (parallel form, no graph):
  //   0: site update + chunk filter elements; total filter element -> total (FE words)
  //   1: boundary = filtered state entering the segment (ST words, or null for
  //      the first segment); filter, RTS elements; total smoother element -> total (SE)
  //   2: boundary = smoothed state of the next segment's first step (or null for
  //      the last segment); smoother, site expectations, energy terms (bn_model_result)
  int segment_step(cudaStream_t st, int phase, bool newton, double lr, const void* dt, const void* y,
                   const bn_site_state& ss, const double* boundary, double* total) override {
    if (!seg_buf) return BN_ERR_ARG;
    A a = args();
    a.lr = T(lr);
    a.dt = static_cast<const T*>(dt);
    a.y = static_cast<const T*>(y);
    a.nat1 = static_cast<T*>(ss.nat1);
    a.nat2 = static_cast<T*>(ss.nat2);
    a.post_mean = static_cast<T*>(ss.post_mean);
    a.post_var = static_cast<T*>(ss.post_var);
    a.grad = static_cast<T*>(ss.grad);
    a.hess = static_cast<T*>(ss.hess);
    a.lin = static_cast<T*>(ss.lin);
    a.shift_dt = 1;
    a.staged = 0;
    a.seg_continue = seg_continue;
    a.seg_more = seg_more;
    a.dt_next = seg_dt_next;
    T* lbuf = static_cast<T*>(seg_buf);
    T* rbuf = lbuf + Z::ST;
    T* ftot = rbuf + Z::ST;
    T* stot = ftot + Z::FE;
    const int fsm = f1_smem();
    const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
    auto upload = [&](T* dst, int words) -> int {
      std::vector<T> h(static_cast<size_t>(words));
      for (int i = 0; i < words; ++i) h[i] = T(boundary[i]);
      BN_CUDA_TRY(cudaMemcpyAsync(dst, h.data(), size_t(words) * sizeof(T), cudaMemcpyHostToDevice, st));
      BN_CUDA_TRY(cudaStreamSynchronize(st));
      return BN_OK;
    };
    auto download = [&](const T* src, int words) -> int {
      std::vector<T> h(static_cast<size_t>(words));
      BN_CUDA_TRY(cudaMemcpyAsync(h.data(), src, size_t(words) * sizeof(T), cudaMemcpyDeviceToHost, st));
      BN_CUDA_TRY(cudaStreamSynchronize(st));
      for (int i = 0; i < words; ++i) total[i] = double(h[i]);
      return BN_OK;
    };
    if (phase == 0) {
      BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
      if (newton) filter_reduce_kernel<T, Lay, P, SITE_NEWTON, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
      else filter_reduce_kernel<T, Lay, P, SITE_NAT, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
      a.seg_total_f = ftot;
      launch_filter_blocks(st, a);
      BN_CUDA_TRY(cudaGetLastError());
      return total ? download(ftot, Z::FE) : BN_OK;
    }
    if (phase == 1) {
      if (boundary) {
        const int e = upload(lbuf, Z::ST);
        if (e != BN_OK) return e;
        a.seg_left = lbuf;
      }
      launch_filter_blocks(st, a);
      filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_ELEM, true, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
      a.seg_total_s = stot;
      launch_smoother_blocks(st, a);
      BN_CUDA_TRY(cudaGetLastError());
      return total ? download(stot, Z::SE) : BN_OK;
    }
    if (phase == 2) {
      if (boundary) {
        const int e = upload(rbuf, Z::ST);
        if (e != BN_OK) return e;
        a.seg_right = rbuf;
      }
      launch_smoother_blocks(st, a);
      smoother_rerun_kernel<T, Lay, P, STORE_ELEM, false, kTPB><<<nblocks, kTPB, 0, st>>>(a);
      launch_tail(st, a);
      BN_CUDA_TRY(cudaGetLastError());
      return BN_OK;
    }
    return BN_ERR_ARG;
  }

  int set_profiling(int on) override {
    if (on && !ev[0])
      for (auto& e : ev) BN_CUDA_TRY(cudaEventCreate(&e));
    profiling = on != 0;
    return BN_OK;
  }

  int kernel_times(float* ms, int n) override {
    if (!ev[0]) return BN_ERR_ARG;
    const int nk = (split_tail || batch) ? 6 : 5;
    BN_CUDA_TRY(cudaEventSynchronize(ev[nk]));
    for (int i = 0; i < n && i < 6; ++i) {
      if (i < nk) BN_CUDA_TRY(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
      else ms[i] = 0.0f;
    }
    return BN_OK;
  }

  int update_posterior(cudaStream_t st, int parallel, const void* dt, const void* y,
                       const bn_site_state& ss) override {
    return posterior_pass(st, parallel, false, 1.0, dt, y, ss);
  }

  int newton_step(cudaStream_t st, int parallel, double lr, const void* dt, const void* y,
                  const bn_site_state& ss) override {
    return posterior_pass(st, parallel, true, lr, dt, y, ss);
  }

  int kalman_filter(cudaStream_t st, int parallel, int return_predict, const void* dt, const void* sy, const void* sR,
                    const uint8_t* mask, void* om, void* oP) override {
    A a = args();
    a.dt = static_cast<const T*>(dt);
    a.site_y = static_cast<const T*>(sy);
    a.site_R = static_cast<const T*>(sR);
    a.mask = mask;
    a.out_m = static_cast<T*>(om);
    a.out_P = static_cast<T*>(oP);
    a.return_predict = return_predict;
    BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    if (!parallel) {
      seq_filter_kernel<T, Lay, P, SITE_GIVEN, STORE_REF><<<1, 1, 0, st>>>(a);
    } else {
      const int fsm = kTPB * int(sizeof(FElem<T, DD>));
      const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
      filter_reduce_kernel<T, Lay, P, SITE_GIVEN, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
      launch_filter_blocks(st, a);
      filter_rerun_kernel<T, Lay, P, SITE_GIVEN, STORE_REF, false, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
    }
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int rts_smoother(cudaStream_t st, int parallel, int return_full, const void* dt, const void* fm, const void* fP,
                   void* om, void* oP, void* oG) override {
    A a = args();
    a.dt = static_cast<const T*>(dt);
    a.in_m = static_cast<const T*>(fm);
    a.in_P = static_cast<const T*>(fP);
    a.out_m = static_cast<T*>(om);
    a.out_P = static_cast<T*>(oP);
    a.out_G = static_cast<T*>(oG);
    a.return_full = return_full;
    a.shift_dt = 0;
    BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    if (!parallel) {
      seq_smoother_kernel<T, Lay, P, STORE_REF, false><<<1, 1, 0, st>>>(a);
    } else {
      const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
      smoother_reduce_kernel<T, Lay, P, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
      launch_smoother_blocks(st, a);
      smoother_rerun_kernel<T, Lay, P, STORE_REF, false, kTPB><<<nblocks, kTPB, 0, st>>>(a);
    }
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  // ---------------------------------------------------------------- prediction
  int conditional(cudaStream_t st, int64_t nt, const double* x, const double* xt, const void* sm, const void* sP,
                  const void* G, void* om, void* oP, int full, int* stat) {
    if (nt <= 0) return BN_OK;
    CondArgs<DD, P> c;
    std::memset(&c, 0, sizeof(c));
    c.ssm = ssm64;
    c.n = num_data;
    c.nt = nt;
    c.x = x;
    c.xt = xt;
    c.mean = sm;
    c.cov = sP;
    c.gain = G;
    c.out_m = om;
    c.out_P = oP;
    c.status = stat;
    const int64_t nb = (nt + 127) / 128;
    if (nb > 0x7fffffff) return BN_ERR_ARG;
    if (full) conditional_kernel<T, Lay, P, DD><<<unsigned(nb), 128, 0, st>>>(c);
    else conditional_kernel<T, Lay, P, P><<<unsigned(nb), 128, 0, st>>>(c);
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int temporal_conditional(cudaStream_t st, const double* x, int64_t nt, const double* xt, const void* sm,
                           const void* sP, const void* G, int full, void* om, void* oP) override {
    BN_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    return conditional(st, nt, x, xt, sm, sP, G, om, oP, full, status);
  }

  int ensure_pred() {
    if (pred_buf) return BN_OK;
    const size_t n = size_t(num_data);
    const size_t words[5] = {n * DD, n * DD * DD, n * DD, n * DD * DD, n * DD * DD};
    size_t tot = 0;
    for (size_t w : words) tot += (w * sizeof(T) + 255) / 256 * 256;
    tot += 256 + 256;
    BN_CUDA_TRY(cudaMalloc(&pred_buf, tot));
    char* p = static_cast<char*>(pred_buf);
    T** ptrs[5] = {&p_fm, &p_fP, &p_sm, &p_sP, &p_G};
    for (int i = 0; i < 5; ++i) {
      *ptrs[i] = reinterpret_cast<T*>(p);
      p += (words[i] * sizeof(T) + 255) / 256 * 256;
    }
    p_res = reinterpret_cast<double*>(p);
    p_status = reinterpret_cast<int*>(p + 256);
    const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
    BN_CUDA_TRY(cudaFuncSetAttribute(filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_REF, false, kTPB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, ssm_b));
    return BN_OK;
  }

  // filtered states, smoothed states and gains of the current sites into the
  // prediction workspace (the reference's predict, basemodels.py:780-795)
  int smooth_full(cudaStream_t st, int parallel, const void* dt, const void* y, const bn_site_state& ss) {
    const int e = ensure_pred();
    if (e != BN_OK) return e;
    BN_CUDA_TRY(cudaMemsetAsync(p_status, 0, sizeof(int), st));
    A a = args();
    a.result = p_res;
    a.status = p_status;
    a.dt = static_cast<const T*>(dt);
    a.y = static_cast<const T*>(y);
    a.nat1 = static_cast<T*>(ss.nat1);
    a.nat2 = static_cast<T*>(ss.nat2);
    a.out_m = p_fm;
    a.out_P = p_fP;
    a.return_predict = 0;
    A b = args();
    b.result = p_res;
    b.status = p_status;
    b.dt = static_cast<const T*>(dt);
    b.in_m = p_fm;
    b.in_P = p_fP;
    b.out_m = p_sm;
    b.out_P = p_sP;
    b.out_G = p_G;
    b.return_full = 1;
    b.shift_dt = 1;
    if (!parallel) {
      seq_filter_kernel<T, Lay, P, SITE_NAT, STORE_REF><<<1, 1, 0, st>>>(a);
      seq_smoother_kernel<T, Lay, P, STORE_REF, false><<<1, 1, 0, st>>>(b);
    } else {
      const int fsm = f1_smem();
      const int ssm_b = kTPB * int(sizeof(SElem<T, DD>));
      filter_reduce_kernel<T, Lay, P, SITE_NAT, kTPB><<<nblocks, kTPB, fsm, st>>>(a);
      launch_filter_blocks(st, a);
      filter_rerun_kernel<T, Lay, P, SITE_NAT, STORE_REF, false, kTPB><<<nblocks, kTPB, ssm_b, st>>>(a);
      smoother_reduce_kernel<T, Lay, P, kTPB><<<nblocks, kTPB, ssm_b, st>>>(b);
      launch_smoother_blocks(st, b);
      smoother_rerun_kernel<T, Lay, P, STORE_REF, false, kTPB><<<nblocks, kTPB, 0, st>>>(b);
    }
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  // basemodels.py:766-816 (temporal case): filter from the current sites, full
  // smoother with gains, then the conditional at the test times
  int predict(cudaStream_t st, int parallel, const void* dt, const void* y, const bn_site_state& ss,
              const double* x, int64_t nt, const double* xt, void* om, void* oP) override {
    if (batch) return BN_ERR_UNSUPPORTED;
    const int e = smooth_full(st, parallel, dt, y, ss);
    if (e != BN_OK) return e;
    return conditional(st, nt, x, xt, p_sm, p_sP, p_G, om, oP, 0, p_status);
  }

  // d energy / d (variance_c, lengthscale_c, ..., likelihood variance) of the VI
  // energy (bn_grad.cuh); out (host) gets 2 NC + 1 values and log_z the filter log
  // marginal of the pseudo-observations at the current hyperparameters
  int energy_grad(cudaStream_t st, int parallel, const void* dt, const void* y, const bn_site_state& ss,
                  double* out, double* log_z) override {
    if (batch || dense) return BN_ERR_UNSUPPORTED;
    for (int c = 0; c < Lay::NC; ++c)
      if (comp_kind[c] == BN_KIND_FEEDBACK) return BN_ERR_UNSUPPORTED;
    int e = smooth_full(st, parallel, dt, y, ss);
    if (e != BN_OK) return e;
    double* acc = p_res + BN_NRESULT;
    BN_CUDA_TRY(cudaMemsetAsync(acc, 0, kGradMax * sizeof(double), st));
    GradArgs<T, DD, P> g;
    std::memset(&g, 0, sizeof(g));
    g.ssm = ssm;
    for (int c = 0; c < Lay::NC; ++c) {
      g.var[c] = comp_var[c];
      g.ell[c] = comp_ell[c];
    }
    g.n = num_data;
    g.obs_dim = obs_dim;
    g.lik_gauss = (P == 1 && lik.kind == BN_LIK_GAUSSIAN) ? 1 : 0;
    g.method = lik.method;
    g.lik_var = lik_var64;
    g.power = double(lik.power);
    g.nat1 = ss.nat1;
    g.nat2 = ss.nat2;
    g.dt = dt;
    g.fm = p_fm;
    g.fP = p_fP;
    g.sm = p_sm;
    g.sP = p_sP;
    g.G = p_G;
    g.y = y;
    g.pm = ss.post_mean;
    g.pv = ss.post_var;
    g.acc = acc;
    int64_t nb = (num_data + 127) / 128;
    if (nb > 152 * 16) nb = 152 * 16;
    grad_kernel<T, Lay, P><<<unsigned(nb), 128, 0, st>>>(g);
    BN_CUDA_TRY(cudaGetLastError());
    double h[kGradMax + 1];
    BN_CUDA_TRY(cudaMemcpyAsync(h, acc, kGradMax * sizeof(double), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaMemcpyAsync(h + kGradMax, p_res + BN_RES_LOGLIK, sizeof(double), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaStreamSynchronize(st));
    const int nc = Lay::NC;
    for (int c = 0; c < 2 * nc; ++c) out[c] = -h[c];
    out[2 * nc] = -h[2 * nc];
    if (log_z) *log_z = h[kGradMax];
    return BN_OK;
  }

  // log predictive density per point (out may be null) and, in sum_count (host),
  // the sum of its finite values and their count
  int log_density(cudaStream_t st, int64_t n, const void* y, const void* m, const void* v, void* out,
                  double* sum_count) override {
    if (P != 1 || lik.kind == BN_LIK_HETERO_EXP || lik.kind == BN_LIK_HETERO_SOFTPLUS) return BN_ERR_UNSUPPORTED;
    const int e = ensure_pred();
    if (e != BN_OK) return e;
    double* acc = p_res + BN_NRESULT;
    BN_CUDA_TRY(cudaMemsetAsync(acc, 0, 2 * sizeof(double), st));
    LikParams<T> lp = lik;
    lp.power = T(1);
    if (n > 0) {
      const int64_t nb = (n + 255) / 256;
      if (nb > 0x7fffffff) return BN_ERR_ARG;
      log_density_kernel<T><<<unsigned(nb), 256, 0, st>>>(lp, n, static_cast<const T*>(y), static_cast<const T*>(m),
                                                          static_cast<const T*>(v), static_cast<T*>(out), acc);
      BN_CUDA_TRY(cudaGetLastError());
    }
    if (sum_count) {
      BN_CUDA_TRY(cudaMemcpyAsync(sum_count, acc, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
      BN_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return BN_OK;
  }

  int predict_y(cudaStream_t st, int64_t n, const void* m, const void* v, void* my, void* vy) override {
    if (P != 1 || lik.kind == BN_LIK_HETERO_EXP || lik.kind == BN_LIK_HETERO_SOFTPLUS) return BN_ERR_UNSUPPORTED;
    if (n <= 0) return BN_OK;
    const int64_t nb = (n + 255) / 256;
    if (nb > 0x7fffffff) return BN_ERR_ARG;
    predict_y_kernel<T><<<unsigned(nb), 256, 0, st>>>(lik, n, static_cast<const T*>(m), static_cast<const T*>(v),
                                                      static_cast<T*>(my), static_cast<T*>(vy));
    BN_CUDA_TRY(cudaGetLastError());
    return BN_OK;
  }

  int result(cudaStream_t st, double* out, int32_t* stat) override {
    if (out) BN_CUDA_TRY(cudaMemcpyAsync(out, res, BN_NRESULT * sizeof(double), cudaMemcpyDeviceToHost, st));
    int s = 0;
    unsigned cnt[2] = {0u, 0u};
    BN_CUDA_TRY(cudaMemcpyAsync(&s, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (surr) BN_CUDA_TRY(cudaMemcpyAsync(cnt, surr_counters(), sizeof(cnt), cudaMemcpyDeviceToHost, st));
    BN_CUDA_TRY(cudaStreamSynchronize(st));
    if (stat) *stat = s;
    if (out) {
      out[BN_RES_SURR_PSD] = double(cnt[0]);
      out[BN_RES_SURR_SPOT] = double(cnt[1]);
    }
    return BN_OK;
  }
};

template <typename T, typename Lay, int P>
EngineBase* make_engine(int64_t n, int obs, int spt, bool dense, int* err) {
  auto* e = new Engine<T, Lay, P>();
  *err = e->init(n, obs, spt, dense);
  if (*err != BN_OK) {
    delete e;
    return nullptr;
  }
  return e;
}

}  // namespace bn
