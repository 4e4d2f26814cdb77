// bn_kalman_filter_noalloc: the parallel (associative-scan) Kalman filter of
// bn_kalman_filter for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden --
// a host framework that owns every device allocation through its own arena and
// forbids a plugin from calling the CUDA allocator, a real-time loop that must not
// allocate after start-up, or a caller inside a region where allocation would
// synchronise the device.  Such callers cannot create a bn_model (which allocates
// its workspace), so this entry point takes the prior directly and keeps its
// scratch in one fixed array in the library's device memory.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes (16 MiB):
// every GPU that loads the library holds it until the process exits.  The caller
// still passes the inputs and the outputs.  Long series use longer chunks per
// thread so that the scan workspace fits; a call that does not fit even with
// kMaxChunk steps per thread (about N > 4.8e7 at state dim 5) is rejected with
// BN_ERR_SCRATCH before anything is launched.
//
// Per-device set-up: the first call on each device (with that device current)
// looks up the array's device address with cudaGetSymbolAddress; make that first
// call before any stream capture.  Every call on a device shares the one array:
// calls whose work overlaps on the GPU (different streams, or host threads that
// do not order their streams) race on it and must be serialised by the caller.
// The array keeps the previous call's contents; the parts that must start at zero
// (the last-block counter and the status word) are cleared by each call.
//
// The address looked up at set-up belongs to the device's current context: after
// cudaDeviceReset (or any teardown of the primary context) it is stale, so the
// entry point must not be used across a device reset in the same process.
//
// Numerical conditions the scan meets (BN_STATUS_* bits, e.g. a singular combine)
// are copied to the caller's optional status word at the end of each call.
#include <cuda_runtime.h>

#include <mutex>

#include "bn_engine.cuh"

namespace bn {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
constexpr int kMaxDevices = 64;
constexpr int kTPBn = 128;     // threads per block, as in the model path
constexpr int kMaxChunk = 1024;  // longest chunk (time steps per thread) it will use

__device__ __align__(256) static unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on first use).
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BN_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return BN_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return BN_OK;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

template <typename Lay>
int filter_noalloc(const bn_prior_desc* prior, int64_t N, cudaStream_t st, int return_predict, const float* dt,
                   const float* sy, const float* sR, const uint8_t* mask, float* om, float* oP, double* log_lik,
                   int32_t* status) {
  using T = float;
  constexpr int D = Lay::D;
  using Z = Sz<T, D>;
  // chunk length as the model path picks it, lengthened (fewer blocks, less
  // scratch) until the scan workspace fits the fixed array
  const double per = double(N) / (152.0 * 2.0 * kTPBn);
  int L = 4;
  while (L < 64 && L < per) L <<= 1;
  size_t nb = 0, b_fx = 0, b_fagg = 0, b_fin = 0, b_part = 0, need = 0;
  const size_t b_res = align256(BN_NRESULT * sizeof(double));
  const size_t b_ctl = 256;  // counters [2] + status
  for (;; L <<= 1) {
    const int64_t nchunks = (N + L - 1) / L;
    const int64_t nb64 = (nchunks + kTPBn - 1) / kTPBn;
    nb = size_t(nb64 < 1 ? 1 : nb64);
    b_fx = align256(nb * Z::FE * kTPBn * sizeof(T));
    b_fagg = align256(nb * Z::FE * sizeof(T));
    b_fin = align256(nb * Z::ST * sizeof(T));
    b_part = align256(nb * BN_NPART * sizeof(double));
    need = b_fx + b_fagg + b_fin + b_part + b_res + b_ctl;
    if (need <= kNoAllocScratchBytes) break;
    if (L >= kMaxChunk) return BN_ERR_SCRATCH;
  }
  void* base = nullptr;
  int err = scratch_address(&base);
  if (err != BN_OK) return err;
  char* p = static_cast<char*>(base);
  ScanArgs<T, D, 1> a;
  std::memset(&a, 0, sizeof(a));
  if ((err = build_ssm<T, D, 1>(prior, false, a.ssm)) != BN_OK) return err;
  a.N = N;
  a.L = L;
  a.nblocks = int(nb);
  a.obs_dim = 1;
  a.return_predict = return_predict;
  a.dt = dt;
  a.site_y = sy;
  a.site_R = sR;
  a.mask = mask;
  a.out_m = om;
  a.out_P = oP;
  a.fx = reinterpret_cast<T*>(p);
  p += b_fx;
  a.fagg = reinterpret_cast<T*>(p);
  p += b_fagg;
  a.fin = reinterpret_cast<T*>(p);
  p += b_fin;
  a.part = reinterpret_cast<double*>(p);
  p += b_part;
  a.result = reinterpret_cast<double*>(p);
  p += b_res;
  a.counter = reinterpret_cast<unsigned*>(p);
  a.status = reinterpret_cast<int*>(p + 16);
  // the last-block counter and the status word must start at zero
  if (cudaMemsetAsync(p, 0, b_ctl, st) != cudaSuccess) return BN_ERR_CUDA;
  const int fsm = kTPBn * int(sizeof(FElem<T, D>));
  const int ssm_b = kTPBn * int(sizeof(SElem<T, D>));
  filter_reduce_kernel<T, Lay, 1, SITE_GIVEN, kTPBn><<<int(nb), kTPBn, fsm, st>>>(a);
  filter_blocks_kernel<T, Lay, 1, kTPBn><<<1, kTPBn, fsm, st>>>(a);
  filter_rerun_kernel<T, Lay, 1, SITE_GIVEN, STORE_REF, false, kTPBn><<<int(nb), kTPBn, ssm_b, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return BN_ERR_CUDA;
  if (log_lik &&
      cudaMemcpyAsync(log_lik, a.result + BN_RES_LOGLIK, sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return BN_ERR_CUDA;
  if (status && cudaMemcpyAsync(status, a.status, sizeof(int32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return BN_ERR_CUDA;
  return BN_OK;
}

template <int... Bs>
bool layout_is(const bn_prior_desc* d) {
  constexpr int s[] = {Bs...};
  if (d->num_components != int(sizeof...(Bs))) return false;
  for (int c = 0; c < int(sizeof...(Bs)); ++c)
    if (d->size[c] != s[c] || d->kind[c] == BN_KIND_FEEDBACK) return false;
  return true;
}

}  // namespace
}  // namespace bn

extern "C" int bn_kalman_filter_noalloc(const bn_prior_desc* prior, int64_t num_data, void* stream,
                                        int32_t return_predict, const void* dt, const void* site_y,
                                        const void* site_cov, const uint8_t* mask, void* means, void* covs,
                                        double* log_lik, int32_t* status) {
  using namespace bn;
  if (!prior || num_data < 1 || !dt || !site_y || !site_cov || !means || !covs) return BN_ERR_ARG;
  if (prior->combine != BN_COMBINE_SUM) return BN_ERR_UNSUPPORTED;
  for (int c = 0; c < prior->num_components && c < BN_MAX_COMPONENTS; ++c)
    if (!(prior->lengthscale[c] > 0.0) || prior->kind[c] != prior->size[c]) return BN_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float* d = static_cast<const float*>(dt);
  const float* y = static_cast<const float*>(site_y);
  const float* R = static_cast<const float*>(site_cov);
  float* m = static_cast<float*>(means);
  float* P = static_cast<float*>(covs);
  if (layout_is<1>(prior)) return filter_noalloc<Layout<1>>(prior, num_data, st, return_predict, d, y, R, mask, m, P, log_lik, status);
  if (layout_is<2>(prior)) return filter_noalloc<Layout<2>>(prior, num_data, st, return_predict, d, y, R, mask, m, P, log_lik, status);
  if (layout_is<3>(prior)) return filter_noalloc<Layout<3>>(prior, num_data, st, return_predict, d, y, R, mask, m, P, log_lik, status);
  if (layout_is<4>(prior)) return filter_noalloc<Layout<4>>(prior, num_data, st, return_predict, d, y, R, mask, m, P, log_lik, status);
  if (layout_is<3, 2>(prior))
    return filter_noalloc<Layout<3, 2>>(prior, num_data, st, return_predict, d, y, R, mask, m, P, log_lik, status);
  return BN_ERR_UNSUPPORTED;
}
