// bn_xla.cc: XLA custom-call shim for the ops-level Kalman filter (jax 0.4.14's
// status-returning custom-call ABI, which needs no XLA headers).  A JAX maintainer
// builds it next to libbnx.so and registers bn_xla_kalman_filter as the
// "bn_kalman_filter" custom-call target:
//   g++ -O2 -shared -fPIC integration/bn_xla.cc -Iinclude -Lbayesnewton_gb300 -lbnx -o libbn_xla.so
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include "bnx.h"

struct XlaCustomCallStatus;                     // provided by jaxlib
extern "C" void XlaCustomCallStatusSetFailure(XlaCustomCallStatus*, const char*, size_t);

// backend_config: the prior, the series length and the flags, packed by the Python side
struct BnXlaFilterCfg { bn_prior_desc prior; int64_t num_data; int32_t dtype, parallel, return_predict; };

// one bn_model per (prior, length, dtype): created on first use, workspace kept
static bn_model* model_for(const BnXlaFilterCfg& c) {
  static std::mutex mu;
  static std::map<std::tuple<std::string, int64_t, int32_t>, bn_model*> cache;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_tuple(std::string((const char*)&c.prior, sizeof c.prior), c.num_data, c.dtype);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  bn_lik_desc lik{};                            // unused by the ops-level filter
  bn_model* m = nullptr;
  if (bn_model_create(&c.prior, &lik, c.num_data, 1, c.dtype, 0, &m) != BN_OK) return nullptr;
  return cache[key] = m;
}

// operands: dt [N], y [N,P,1], noise_cov [N,P,P], mask [N,P] (uint8)
// results:  means [N,D,1], covs [N,D,D]
extern "C" void bn_xla_kalman_filter(void* stream, void** buffers, const char* opaque, size_t len,
                                     XlaCustomCallStatus* status) {
  BnXlaFilterCfg c;
  if (len != sizeof c) { XlaCustomCallStatusSetFailure(status, "bad config", 10); return; }
  std::memcpy(&c, opaque, sizeof c);
  bn_model* m = model_for(c);
  int rc = m ? bn_kalman_filter(m, stream, c.parallel, c.return_predict, buffers[0], buffers[1],
                                buffers[2], (const uint8_t*)buffers[3], buffers[4], buffers[5])
             : BN_ERR_ARG;
  if (rc != BN_OK) XlaCustomCallStatusSetFailure(status, "bn_kalman_filter failed", 23);
}
