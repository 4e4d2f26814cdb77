// Learned site expectations for the two-latent (heteroscedastic) likelihood: a
// small MLP maps a site's (y, marginal mean, marginal covariance) to
// (E, dE/dm, d2E/dm2) of E_q log p(y | f), standing in for the 2-D Gauss-Hermite
// cubature (likelihoods.py:613-664 with cubature.py:198-246).  Training pairs come
// from high-order cubature on the device, and the network is trained here by
// hand-written forward / backward / Adam kernels.  In a model step the network's
// outputs replace the cubature except where a check fails: a site whose predicted
// diagonal precision -h11, -h22 is not positive, or a spot-checked site (every
// `spot`-th) whose prediction is off by more than `tol`, reverts to cubature
// (counted in BN_RES_SURR_*).
//
// Network: 6 -> 64 -> 64 -> 64 -> 6, tanh hidden units, float32.  Features of a
// site (y, m1, m2, v11, v12, v22), with l = link(m2) the noise scale at the mean:
//   f = [(y - m1) / l, log(v11 / l^2), v12 / sqrt(v11 v22), log v22, m2, m1], standardised;
// outputs with the noise scale divided out:
//   t = [E + log l, g1 l, g2, h11 l^2, h12 l, h22], standardised.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bn_dense.cuh"
#include "bn_tc.cuh"
#include "bn_engine.cuh"
#include "bn_mlp.h"

namespace bn {
namespace mlp {

constexpr int kIn = 6, kH = 64, kOut = 6;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kH * kH, kW4 = kB3 + kH, kB4 = kW4 + kOut * kH, kNParam = kB4 + kOut;
constexpr int kNorm = 4 * 6;  // in mean, in sd, out mean, out sd
constexpr int kTPB = 128;

struct Norm {
  float in_mu[kIn], in_sd[kIn], out_mu[kOut], out_sd[kOut];
};

__device__ __forceinline__ float link_of(int kind, float f2) {
  if (kind == BN_LIK_HETERO_EXP) return __expf(f2);
  return f2 > 20.f ? f2 : __logf(1.f + __expf(f2));
}

// raw site -> standardised features.  In units of the noise scale l = link(m2)
// the site is (z = (y - m1) / l, v11 / l^2, corr(f1, f2), v22): for the exp link
// the scaled expectations below depend on these alone.
__device__ __forceinline__ void features(const Norm& nz, int kind, float y, float m1, float m2, float v11, float v12,
                                         float v22, float (&x)[kIn]) {
  const float a = fmaxf(v11, 1e-30f), c = fmaxf(v22, 1e-30f);
  const float l = link_of(kind, m2);
  const float f[kIn] = {(y - m1) / l, __logf(a / (l * l)), v12 * rsqrtf(a * c), __logf(c), m2, m1};
#pragma unroll
  for (int i = 0; i < kIn; ++i) x[i] = (f[i] - nz.in_mu[i]) / nz.in_sd[i];
}

// raw expectations -> standardised targets, and back: the noise scale divided
// out, [E + log l, g1 l, g2, h11 l^2, h12 l, h22] (dimensionless)
__device__ __forceinline__ void scale_targets(const Norm& nz, int kind, float m2, const float (&r)[kOut],
                                              float (&t)[kOut]) {
  const float l = link_of(kind, m2);
  const float s[kOut] = {r[0] + __logf(l), r[1] * l, r[2], r[3] * l * l, r[4] * l, r[5]};
#pragma unroll
  for (int i = 0; i < kOut; ++i) t[i] = (s[i] - nz.out_mu[i]) / nz.out_sd[i];
}
__device__ __forceinline__ void unscale_targets(const Norm& nz, int kind, float m2, const float (&o)[kOut],
                                                float (&r)[kOut]) {
  const float l = link_of(kind, m2);
  const float il = 1.f / l;
  float s[kOut];
#pragma unroll
  for (int i = 0; i < kOut; ++i) s[i] = fmaf(o[i], nz.out_sd[i], nz.out_mu[i]);
  r[0] = s[0] - __logf(l);
  r[1] = s[1] * il;
  r[2] = s[2];
  r[3] = s[3] * il * il;
  r[4] = s[4] * il;
  r[5] = s[5];
}

// tanh for the inference passes: the hardware approximation (tanh.approx.f32,
// ~2^-11 relative), well inside the network's own error against the cubature;
// training keeps the library tanhf
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// weights into shared memory (kNParam floats)
__device__ __forceinline__ void load_params(float* w, const float* params) {
  for (int i = threadIdx.x; i < kNParam; i += blockDim.x) w[i] = params[i];
  __syncthreads();
}

// forward pass of one sample from standardised features (KEEP: library tanhf,
// for the checked forward_kernel; else the hardware tanh of the site pass)
template <bool KEEP>
__device__ __forceinline__ void forward(const float* w, const float (&x)[kIn], float (&h1)[kH], float (&h2)[kH],
                                        float (&h3)[kH], float (&o)[kOut]) {
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    float s = w[kB1 + j];
#pragma unroll
    for (int i = 0; i < kIn; ++i) s = fmaf(w[kW1 + j * kIn + i], x[i], s);
    h1[j] = KEEP ? tanhf(s) : tanh_fast(s);
  }
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    float s = w[kB2 + j];
#pragma unroll
    for (int i = 0; i < kH; i += 4) {
      const float4 q = *reinterpret_cast<const float4*>(w + kW2 + j * kH + i);
      s = fmaf(q.x, h1[i], s);
      s = fmaf(q.y, h1[i + 1], s);
      s = fmaf(q.z, h1[i + 2], s);
      s = fmaf(q.w, h1[i + 3], s);
    }
    h2[j] = KEEP ? tanhf(s) : tanh_fast(s);
  }
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    float s = w[kB3 + j];
#pragma unroll
    for (int i = 0; i < kH; i += 4) {
      const float4 q = *reinterpret_cast<const float4*>(w + kW3 + j * kH + i);
      s = fmaf(q.x, h2[i], s);
      s = fmaf(q.y, h2[i + 1], s);
      s = fmaf(q.z, h2[i + 2], s);
      s = fmaf(q.w, h2[i + 3], s);
    }
    h3[j] = KEEP ? tanhf(s) : tanh_fast(s);
  }
#pragma unroll
  for (int j = 0; j < kOut; ++j) {
    float s = w[kB4 + j];
#pragma unroll
    for (int i = 0; i < kH; i += 4) {
      const float4 q = *reinterpret_cast<const float4*>(w + kW4 + j * kH + i);
      s = fmaf(q.x, h3[i], s);
      s = fmaf(q.y, h3[i + 1], s);
      s = fmaf(q.z, h3[i + 2], s);
      s = fmaf(q.w, h3[i + 3], s);
    }
    o[j] = s;
  }
}

// Batched inference on standardised features: xn [n][6] -> out [n][6].
__global__ void __launch_bounds__(kTPB) forward_kernel(int n, const float* params, const float* xn, float* out) {
  extern __shared__ __align__(16) float w[];
  load_params(w, params);
  const int i = blockIdx.x * kTPB + threadIdx.x;
  if (i >= n) return;
  float x[kIn], h1[kH], h2[kH], h3[kH], o[kOut];
#pragma unroll
  for (int q = 0; q < kIn; ++q) x[q] = xn[int64_t(i) * kIn + q];
  forward<true>(w, x, h1, h2, h3, o);
#pragma unroll
  for (int q = 0; q < kOut; ++q) out[int64_t(i) * kOut + q] = o[q];
}

// Training runs the network as batched products over the whole mini-batch
// (bn_dense bgemm) with elementwise bias / activation kernels in between:
//   H1 = tanh(X W1^T + b1), H2 = tanh(H1 W2^T + b2), H3 = tanh(H2 W3^T + b3),
//   O = H3 W4^T + b4, loss = sum (O - T)^2 / (n kOut),
//   D4 = 2 (O - T) / (n kOut), D3 = (D4 W4) . (1 - H3^2), D2 = (D3 W3) . (1 - H2^2),
//   D1 = (D2 W2) . (1 - H1^2), dW_l = D_l^T H_{l-1}, db_l = column sums of D_l.
__global__ void bias_act_kernel(int64_t n, int wdt, const float* b, float* X, int act) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n * wdt; e += int64_t(gridDim.x) * blockDim.x) {
    const float v = X[e] + b[int(e % wdt)];
    X[e] = act ? tanhf(v) : v;
  }
}

__global__ void dact_kernel(int64_t len, const float* H, float* D) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < len; e += int64_t(gridDim.x) * blockDim.x)
    D[e] *= (1.f - H[e] * H[e]);
}

__global__ void __launch_bounds__(256) out_delta_kernel(int n, const float* O, const float* T, float* D4,
                                                        double* loss_part) {
  __shared__ double red[8];
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double l = 0.0;
  if (e < int64_t(n) * kOut) {
    const float r = O[e] - T[e];
    l = double(r) * r;
    D4[e] = (2.f / (float(n) * kOut)) * r;
  }
  block_sum_store<256>(l, red, loss_part + blockIdx.x, threadIdx.x);
}

// grad[p] = sum over chunk partials (the weight-gradient products ran per chunk)
__global__ void reduce_chunks_kernel(int nchunk, int len, const float* part, float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= len) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; ++c) s += part[int64_t(c) * len + p];
  out[p] = s;
}

// bias gradients: column sums of the deltas, D [n][w] -> out [w]
__global__ void colsum_kernel(int n, int wdt, const float* D, float* out) {
  __shared__ float red[256];
  const int c = blockIdx.x;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += D[int64_t(i) * wdt + c];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

__global__ void adam_kernel(int np, float* p, const float* g, float* m1, float* m2, float lr, float b1, float b2,
                            float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// random mini-batch gather: idx from a counter-based hash of (step, slot)
__global__ void gather_batch_kernel(int n, int bsz, unsigned step, unsigned seed, const float* X, const float* T,
                                    float* xb, float* tb) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= bsz) return;
  unsigned h = seed ^ (step * 0x9E3779B9u) ^ (unsigned(s) * 0x85EBCA6Bu);
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  const int i = int(h % unsigned(n));
#pragma unroll
  for (int q = 0; q < kIn; ++q) xb[int64_t(s) * kIn + q] = X[int64_t(i) * kIn + q];
#pragma unroll
  for (int q = 0; q < kOut; ++q) tb[int64_t(s) * kOut + q] = T[int64_t(i) * kOut + q];
}

// raw sites (y, m1, m2, v11, v12, v22) -> standardised features and, from
// high-order cubature, standardised targets
__global__ void prepare_kernel(int n, Norm nz, int kind, LikParams<float> lp, const float* raw, float* xn, float* tn,
                               float* traw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = raw + int64_t(i) * 6;
  float x[kIn];
  features(nz, kind, r[0], r[1], r[2], r[3], r[4], r[5], x);
#pragma unroll
  for (int q = 0; q < kIn; ++q) xn[int64_t(i) * kIn + q] = x[q];
  if (tn || traw) {
    float E, g[2], H[3];
    const float m[2] = {r[1], r[2]};
    const float V[3] = {r[3], r[4], r[5]};
    ve2(lp, r[0], m, V, E, g, H);
    const float e[kOut] = {E, g[0], g[1], H[0], H[1], H[2]};
    if (traw)
#pragma unroll
      for (int q = 0; q < kOut; ++q) traw[int64_t(i) * kOut + q] = e[q];
    if (tn) {
      float t[kOut];
      scale_targets(nz, kind, r[2], e, t);
#pragma unroll
      for (int q = 0; q < kOut; ++q) tn[int64_t(i) * kOut + q] = t[q];
    }
  }
}

// Learned expectations of each site at its marginal.  One thread per site, the
// weights in shared memory.  Sites that fail a check -- predicted diagonal
// precision -h11 or -h22 not positive, or (every `spot`-th site) a prediction
// off the cubature by more than `tol` -- are appended to a list (list[0] = count)
// for the cubature pass, so that no warp of this kernel waits on a 400-point
// cubature.  Spot checks are themselves a short list.
__global__ void __launch_bounds__(kTPB) site_kernel(int64_t n, const float* params, Norm nz, int kind,
                                                    const float* pm, const float* pv, const float* y, int spot,
                                                    float* ext, unsigned* counters, unsigned* redo, unsigned* chk) {
  extern __shared__ __align__(16) float w[];
  load_params(w, params);
  const int64_t k = int64_t(blockIdx.x) * kTPB + threadIdx.x;
  if (k >= n) return;
  const float m1 = pm[k * 2], m2 = pm[k * 2 + 1];
  const float v11 = pv[k * 4], v12 = 0.5f * (pv[k * 4 + 1] + pv[k * 4 + 2]), v22 = pv[k * 4 + 3];
  float x[kIn], h1[kH], h2[kH], h3[kH], o[kOut], r[kOut];
  features(nz, kind, y[k], m1, m2, v11, v12, v22, x);
  forward<false>(w, x, h1, h2, h3, o);
  unscale_targets(nz, kind, m2, o, r);
  // the site precision it becomes must be positive: -h11 > 0 and -h22 > 0 (the
  // model keeps the diagonal, ensure_diagonal_positive_precision, utils.py:89-96)
  bool bad = !(r[3] < 0.f && r[5] < 0.f);
#pragma unroll
  for (int q = 0; q < kOut; ++q) bad = bad || !(fabsf(r[q]) < 3e38f);
#pragma unroll
  for (int q = 0; q < kOut; ++q) ext[k * kOut + q] = r[q];
  if (bad) {
    atomicAdd(&counters[0], 1u);
    const unsigned slot = atomicAdd(&redo[0], 1u);
    redo[1 + slot] = unsigned(k);
  } else if (spot > 0 && (k % spot) == 0) {
    const unsigned slot = atomicAdd(&chk[0], 1u);
    chk[1 + slot] = unsigned(k);
  }
}

// Cubature for the listed sites: `redo` sites take it outright; `chk` sites are
// compared with the prediction and take it when off by more than tol.  Four lanes
// share a site (each a quarter of the 400 nodes, summed by shuffles), so the few
// listed sites keep four times as many threads busy.
constexpr int kCubLanes = 4;
__global__ void __launch_bounds__(128) site_cubature_kernel(LikParams<float> lp, const float* pm, const float* pv,
                                                            const float* y, float tol, float* ext,
                                                            unsigned* counters, const unsigned* redo,
                                                            const unsigned* chk) {
  const unsigned nr = redo[0], nc = chk[0];
  const int sub = threadIdx.x & (kCubLanes - 1);
  const unsigned g0 = (blockIdx.x * blockDim.x + threadIdx.x) / kCubLanes;
  const unsigned gstride = gridDim.x * blockDim.x / kCubLanes;
  // every lane of a group runs the same number of iterations (the shuffles below)
  for (unsigned i = g0; i < ((nr + nc + gstride - 1) / gstride) * gstride; i += gstride) {
    const bool live = i < nr + nc;
    const bool is_chk = i >= nr;
    const int64_t k = !live ? 0 : (is_chk ? chk[1 + (i - nr)] : redo[1 + i]);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (live) {
      const float m[2] = {pm[k * 2], pm[k * 2 + 1]};
      const float V[3] = {pv[k * 4], 0.5f * (pv[k * 4 + 1] + pv[k * 4 + 2]), pv[k * 4 + 3]};
      ve2_part(lp, y[k], m, V, sub, kCubLanes, acc);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q)
#pragma unroll
      for (int o = 1; o < kCubLanes; o <<= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o, kCubLanes);
    if (!live || sub != 0) continue;
    const float* c = acc;  // E, g1, g2, h11, h12, h22
    float* r = ext + k * kOut;
    bool take = !is_chk;
    if (is_chk) {
      // relative error of the derivatives against their own scale
      const float sg = fabsf(c[1]) + fabsf(c[2]) + 1e-6f, sh = fabsf(c[3]) + fabsf(c[5]) + 1e-6f;
      const float eg = (fabsf(r[1] - c[1]) + fabsf(r[2] - c[2])) / sg;
      const float eh = (fabsf(r[3] - c[3]) + fabsf(r[4] - c[4]) + fabsf(r[5] - c[5])) / sh;
      if (eg > tol || eh > tol) {
        atomicAdd(&counters[1], 1u);
        take = true;
      }
    }
    if (take)
#pragma unroll
      for (int q = 0; q < kOut; ++q) r[q] = c[q];
  }
}

// ------------------------------------------------------------ tensor-core pass
// The same network on the 5th-generation tensor cores (tcgen05, TF32 operands,
// float32 accumulators in tensor memory).  A persistent CTA of 128 threads owns
// 128-site tiles: thread i builds row i of the features, each layer is one chain
// of tcgen05.mma (M = 128, N = 64 (16 for the output), K = 8 per instruction)
// issued by one thread, the accumulator is read back with tcgen05.ld (warp w reads
// TMEM lanes 32w..32w+31 = rows 32w..), and bias + tanh are applied on the way
// into the next layer's operand tile.  Operands sit in shared memory in the
// canonical K-major, non-swizzled layout: 8-row x 16-byte core matrices, LBO =
// 128 B between core matrices along K, SBO between 8-row groups.
namespace tc {
constexpr int kRows = 128;
constexpr int kK1 = 8;                        // layer-1 K (6 features, zero padded)
constexpr int kN4 = 16;                       // output N (6 outputs, zero padded)
constexpr int kSBO1 = (kK1 / 4) * 128;        // 256 B
constexpr int kSBOH = (kH / 4) * 128;         // 2048 B
constexpr int kOffAH = 0;                     // 128 x 64 hidden-layer operand
// the 128 x 8 layer-1 operand shares the hidden operand's first 4 KB: layer 1's
// MMA has completed before its epilogue writes the hidden operand, and a tile's
// features are written after the previous tile's last MMA completed (this keeps
// three CTAs within an SM's shared memory)
constexpr int kOffA1 = kOffAH;
constexpr int kOffW1 = kOffAH + kRows * kH * 4;    // 64 x 8
constexpr int kOffW2 = kOffW1 + kH * kK1 * 4;      // 64 x 64
constexpr int kOffW3 = kOffW2 + kH * kH * 4;
constexpr int kOffW4 = kOffW3 + kH * kH * 4;       // 16 x 64
constexpr int kOffB = kOffW4 + kN4 * kH * 4;       // biases: 64 + 64 + 64 + 16 floats
constexpr int kSmem = kOffB + (3 * kH + kN4) * 4;
constexpr int kCols = 64;                     // TMEM columns (the 128 x 64 accumulator)

}  // namespace tc

__global__ void __launch_bounds__(128, 3) site_kernel_tc(int64_t n, const float* params, Norm nz, int kind,
                                                      const float* pm, const float* pv, const float* y, int spot,
                                                      float* ext, unsigned* counters, unsigned* redo,
                                                      unsigned* chk, int* err) {
  using namespace tc;
  using namespace ::bn::tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t taddr_s;
  __shared__ __align__(8) uint64_t mbar_s;
  const int tid = threadIdx.x, warp = tid >> 5;
  float* bias = reinterpret_cast<float*>(sm + kOffB);
  // weights into the operand layouts (B operands are the weight rows: N x K, K-major)
  for (int e = tid; e < kH * kK1; e += 128) {
    const int r = e / kK1, k = e % kK1;
    *reinterpret_cast<float*>(sm + kOffW1 + off_k(r, k, kSBO1)) = k < kIn ? params[kW1 + r * kIn + k] : 0.f;
  }
  for (int e = tid; e < kH * kH; e += 128) {
    const int r = e / kH, k = e % kH;
    *reinterpret_cast<float*>(sm + kOffW2 + off_k(r, k, kSBOH)) = params[kW2 + e];
    *reinterpret_cast<float*>(sm + kOffW3 + off_k(r, k, kSBOH)) = params[kW3 + e];
  }
  for (int e = tid; e < kN4 * kH; e += 128) {
    const int r = e / kH, k = e % kH;
    *reinterpret_cast<float*>(sm + kOffW4 + off_k(r, k, kSBOH)) = r < kOut ? params[kW4 + r * kH + k] : 0.f;
  }
  for (int e = tid; e < 3 * kH + kN4; e += 128) {
    float v;
    if (e < kH) v = params[kB1 + e];
    else if (e < 2 * kH) v = params[kB2 + e - kH];
    else if (e < 3 * kH) v = params[kB3 + e - 2 * kH];
    else v = (e - 3 * kH) < kOut ? params[kB4 + e - 3 * kH] : 0.f;
    bias[e] = v;
  }
  const uint32_t base = uint32_t(__cvta_generic_to_shared(sm));
  const uint32_t mbar = uint32_t(__cvta_generic_to_shared(&mbar_s));
  if (warp == 0) {
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(&taddr_s));
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = taddr_s;
  const uint32_t lane_base = tmem + (uint32_t(warp * 32) << 16);
  uint32_t parity = 0;
  bool ok = true;
  const int64_t ntiles = (n + kRows - 1) / kRows;
  for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int64_t k = t * kRows + tid;
    const bool live = k < n;
    float m1 = 0.f, m2 = 0.f, v11 = 1.f, v12 = 0.f, v22 = 1.f, yo = 0.f;
    if (live) {
      m1 = pm[k * 2];
      m2 = pm[k * 2 + 1];
      v11 = pv[k * 4];
      v12 = 0.5f * (pv[k * 4 + 1] + pv[k * 4 + 2]);
      v22 = pv[k * 4 + 3];
      yo = y[k];
    }
    float x[kIn];
    features(nz, kind, yo, m1, m2, v11, v12, v22, x);
#pragma unroll
    for (int q = 0; q < kK1; q += 4)
      *reinterpret_cast<float4*>(sm + kOffA1 + off_k(tid, q, kSBO1)) =
          make_float4((q < kIn && live) ? x[q] : 0.f, (q + 1 < kIn && live) ? x[q + 1] : 0.f,
                      (q + 2 < kIn && live) ? x[q + 2] : 0.f, (q + 3 < kIn && live) ? x[q + 3] : 0.f);
    float o[kOut];
    // four layers: (A operand, its SBO, K, weights, N, bias offset)
#pragma unroll 1
    for (int layer = 0; layer < 4 && ok; ++layer) {
      fence_async_smem();
      fence_before();
      __syncthreads();
      fence_after();
      const int K = layer == 0 ? kK1 : kH;
      const int N = layer == 3 ? kN4 : kH;
      const uint32_t a0 = base + (layer == 0 ? kOffA1 : kOffAH);
      const uint32_t asbo = layer == 0 ? kSBO1 : kSBOH;
      const uint32_t b0 = base + (layer == 0 ? kOffW1 : layer == 1 ? kOffW2 : layer == 2 ? kOffW3 : kOffW4);
      if (tid == 0) {
        const uint32_t id = idesc_tf32(N);
        for (int j = 0; j < K / 8; ++j)
          mma_tf32(tmem, sdesc(a0 + j * 256, 128, asbo), sdesc(b0 + j * 256, 128, asbo), id, j > 0 ? 1u : 0u);
        commit(mbar);
      }
      // one thread polls the mbarrier; the barrier hands its verdict to the CTA
      ok = __syncthreads_and(tid == 0 ? (wait_phase(mbar, parity) ? 1 : 0) : 1) != 0;
      parity ^= 1u;
      fence_after();
      if (!ok) break;
      if (layer < 3) {
        const float* bl = bias + layer * kH;
        // the whole 64-column row of this thread's TMEM lane in one wait, then
        // bias + tanh four columns at a time into one 16-byte store (four
        // consecutive K of a core-matrix row: a quarter warp's stores cover 128
        // contiguous bytes, no bank conflict)
        float v[kH];
#pragma unroll
        for (int c = 0; c < kH; c += 16) ld16(lane_base + uint32_t(c), *reinterpret_cast<float(*)[16]>(v + c));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int c = 0; c < kH; c += 4) {
          const float4 q = make_float4(tanh_fast(v[c] + bl[c]), tanh_fast(v[c + 1] + bl[c + 1]),
                                       tanh_fast(v[c + 2] + bl[c + 2]), tanh_fast(v[c + 3] + bl[c + 3]));
          *reinterpret_cast<float4*>(sm + kOffAH + off_k(tid, c, kSBOH)) = q;
        }
      } else {
        float v[16];
        ld16(lane_base, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int i = 0; i < kOut; ++i) o[i] = v[i] + bias[3 * kH + i];
      }
    }
    if (!ok) break;
    if (live) {
      float r[kOut];
      unscale_targets(nz, kind, m2, o, r);
      bool bad = !(r[3] < 0.f && r[5] < 0.f);
#pragma unroll
      for (int q = 0; q < kOut; ++q) bad = bad || !(fabsf(r[q]) < 3e38f);
#pragma unroll
      for (int q = 0; q < kOut; ++q) ext[k * kOut + q] = r[q];
      if (bad) {
        atomicAdd(&counters[0], 1u);
        const unsigned slot = atomicAdd(&redo[0], 1u);
        redo[1 + slot] = unsigned(k);
      } else if (spot > 0 && (k % spot) == 0) {
        const unsigned slot = atomicAdd(&chk[0], 1u);
        chk[1 + slot] = unsigned(k);
      }
    }
  }
  if (!ok && tid == 0) atomicOr(err, 1);
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols));
}

}  // namespace mlp
}  // namespace bn

// ============================================================ handle + C ABI
struct bn_mlp {
  float* params = nullptr;  // device [kNParam]
  int* err = nullptr;       // device flag: a tensor-core wait gave up
  bool use_tc = true;       // site pass on tcgen05 (else the CUDA-core kernel)
  float *adam1 = nullptr, *adam2 = nullptr, *grad = nullptr;
  bn::mlp::Norm norm;
  int kind = BN_LIK_HETERO_EXP;
  unsigned adam_t = 0;
  // training scratch (grown on demand)
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
};

namespace bn {
int mlp_site_expectations(bn_mlp* h, cudaStream_t st, int64_t n, const float* pm, const float* pv, const float* y,
                          const LikParams<float>& lp, int spot, float tol, float* ext, unsigned* counters,
                          unsigned* lists) {
  constexpr int tpb = bn::mlp::kTPB;
  unsigned* redo = lists;
  unsigned* chk = lists + (n + 1);
  if (cudaMemsetAsync(redo, 0, sizeof(unsigned), st) != cudaSuccess ||
      cudaMemsetAsync(chk, 0, sizeof(unsigned), st) != cudaSuccess)
    return BN_ERR_CUDA;
  if (h->use_tc) {
    // persistent tensor-core pass: three CTAs per SM of the 152 (75 KB of shared
    // memory each), so that one CTA's tanh epilogue overlaps the others' MMAs
    const int64_t tiles = (n + bn::mlp::tc::kRows - 1) / bn::mlp::tc::kRows;
    const unsigned grid = unsigned(tiles < 456 ? tiles : 456);
    bn::mlp::site_kernel_tc<<<grid, 128, bn::mlp::tc::kSmem, st>>>(n, h->params, h->norm, h->kind, pm, pv, y, spot,
                                                                    ext, counters, redo, chk, h->err);
  } else {
    bn::mlp::site_kernel<<<unsigned((n + tpb - 1) / tpb), tpb, bn::mlp::kNParam * 4, st>>>(
        n, h->params, h->norm, h->kind, pm, pv, y, spot, ext, counters, redo, chk);
  }
  // the listed sites are a small fraction: a grid sized for ~1/8 of the sites,
  // four lanes each
  const unsigned nb = unsigned((n / 8 * bn::mlp::kCubLanes + 127) / 128) + 1;
  bn::mlp::site_cubature_kernel<<<nb, 128, 0, st>>>(lp, pm, pv, y, tol, ext, counters, redo, chk);
  return cudaGetLastError() == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}
}  // namespace bn

namespace {
using namespace bn::mlp;

int ensure_scratch(bn_mlp* h, size_t bytes) {
  if (h->scratch_bytes >= bytes) return BN_OK;
  if (h->scratch) cudaFree(h->scratch);
  h->scratch = nullptr;
  h->scratch_bytes = 0;
  if (cudaMalloc(&h->scratch, bytes) != cudaSuccess) return BN_ERR_CUDA;
  h->scratch_bytes = bytes;
  return BN_OK;
}

// gradients of the loss on (xn, tn) [n] into h->grad; loss into *loss (host)
int loss_grad(bn_mlp* h, cudaStream_t st, int n, const float* xn, const float* tn, double* loss) {
  constexpr int kChunk = 512;
  const int nchunk = (n + kChunk - 1) / kChunk;
  const int nlb = int((int64_t(n) * kOut + 255) / 256);
  const size_t act = size_t(n) * kH;
  const size_t need = (6 * act + 2 * size_t(n) * kOut) * sizeof(float) + size_t(nchunk) * kH * kH * sizeof(float) +
                      size_t(nlb) * sizeof(double) + 1024;
  int e = ensure_scratch(h, need);
  if (e != BN_OK) return e;
  float* p = static_cast<float*>(h->scratch);
  float *H1 = p, *H2 = H1 + act, *H3 = H2 + act, *D1 = H3 + act, *D2 = D1 + act, *D3 = D2 + act;
  float* O = D3 + act;
  float* D4 = O + size_t(n) * kOut;
  float* part = D4 + size_t(n) * kOut;
  double* lp = reinterpret_cast<double*>(part + size_t(nchunk) * kH * kH);
  using bn::dense::BRef;
  auto B1 = [](float* q) { return BRef(q, 0); };
  float* W = h->params;
  auto ew = [&](int64_t len) { return int((len + 255) / 256 > 1024 ? 1024 : (len + 255) / 256); };
  // forward
  bn::dense::bgemm(st, 1, false, true, n, kH, kIn, 1.f, B1(const_cast<float*>(xn)), B1(W + kW1), 0.f, BRef(), B1(H1));
  bias_act_kernel<<<ew(act), 256, 0, st>>>(n, kH, W + kB1, H1, 1);
  bn::dense::bgemm(st, 1, false, true, n, kH, kH, 1.f, B1(H1), B1(W + kW2), 0.f, BRef(), B1(H2));
  bias_act_kernel<<<ew(act), 256, 0, st>>>(n, kH, W + kB2, H2, 1);
  bn::dense::bgemm(st, 1, false, true, n, kH, kH, 1.f, B1(H2), B1(W + kW3), 0.f, BRef(), B1(H3));
  bias_act_kernel<<<ew(act), 256, 0, st>>>(n, kH, W + kB3, H3, 1);
  bn::dense::bgemm(st, 1, false, true, n, kOut, kH, 1.f, B1(H3), B1(W + kW4), 0.f, BRef(), B1(O));
  bias_act_kernel<<<ew(int64_t(n) * kOut), 256, 0, st>>>(n, kOut, W + kB4, O, 0);
  // backward
  out_delta_kernel<<<nlb, 256, 0, st>>>(n, O, tn, D4, lp);
  bn::dense::bgemm(st, 1, false, false, n, kH, kOut, 1.f, B1(D4), B1(W + kW4), 0.f, BRef(), B1(D3));
  dact_kernel<<<ew(act), 256, 0, st>>>(int64_t(act), H3, D3);
  bn::dense::bgemm(st, 1, false, false, n, kH, kH, 1.f, B1(D3), B1(W + kW3), 0.f, BRef(), B1(D2));
  dact_kernel<<<ew(act), 256, 0, st>>>(int64_t(act), H2, D2);
  bn::dense::bgemm(st, 1, false, false, n, kH, kH, 1.f, B1(D2), B1(W + kW2), 0.f, BRef(), B1(D1));
  dact_kernel<<<ew(act), 256, 0, st>>>(int64_t(act), H1, D1);
  // weight gradients dW = D^T A over chunks of samples (split-K), then summed
  auto wgrad = [&](const float* D, int dw, const float* A, int aw, float* out) {
    const int kc = kChunk;
    const int full = n / kc;
    if (full > 0)
      bn::dense::bgemm(st, full, true, false, dw, aw, kc, 1.f, BRef(const_cast<float*>(D), int64_t(kc) * dw),
                       BRef(const_cast<float*>(A), int64_t(kc) * aw), 0.f, BRef(), BRef(part, int64_t(dw) * aw));
    int nch = full;
    if (n % kc) {
      bn::dense::bgemm(st, 1, true, false, dw, aw, n % kc, 1.f,
                       BRef(const_cast<float*>(D) + int64_t(full) * kc * dw, 0),
                       BRef(const_cast<float*>(A) + int64_t(full) * kc * aw, 0), 0.f, BRef(),
                       BRef(part + int64_t(full) * dw * aw, 0));
      ++nch;
    }
    reduce_chunks_kernel<<<(dw * aw + 255) / 256, 256, 0, st>>>(nch, dw * aw, part, out);
  };
  float* g = h->grad;
  wgrad(D1, kH, xn, kIn, g + kW1);
  wgrad(D2, kH, H1, kH, g + kW2);
  wgrad(D3, kH, H2, kH, g + kW3);
  wgrad(D4, kOut, H3, kH, g + kW4);
  colsum_kernel<<<kH, 256, 0, st>>>(n, kH, D1, g + kB1);
  colsum_kernel<<<kH, 256, 0, st>>>(n, kH, D2, g + kB2);
  colsum_kernel<<<kH, 256, 0, st>>>(n, kH, D3, g + kB3);
  colsum_kernel<<<kOut, 256, 0, st>>>(n, kOut, D4, g + kB4);
  if (cudaGetLastError() != cudaSuccess) return BN_ERR_CUDA;
  if (loss) {
    std::vector<double> hl(nlb);
    if (cudaMemcpyAsync(hl.data(), lp, nlb * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return BN_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BN_ERR_CUDA;
    double s = 0.0;
    for (double v : hl) s += v;
    *loss = s / (double(n) * kOut);
  }
  return BN_OK;
}

bool norm_ok(const float* nz) {
  for (int i = 0; i < kNorm; ++i)
    if (!std::isfinite(nz[i])) return false;
  for (int i = 0; i < 6; ++i)
    if (!(nz[6 + i] > 0.f) || !(nz[18 + i] > 0.f)) return false;
  return true;
}
}  // namespace

extern "C" {

int bn_mlp_create(int32_t lik_kind, bn_mlp** out) {
  if (!out || (lik_kind != BN_LIK_HETERO_EXP && lik_kind != BN_LIK_HETERO_SOFTPLUS)) return BN_ERR_ARG;
  auto* h = new bn_mlp;
  h->kind = lik_kind;
  for (int i = 0; i < 6; ++i) {
    h->norm.in_mu[i] = h->norm.out_mu[i] = 0.f;
    h->norm.in_sd[i] = h->norm.out_sd[i] = 1.f;
  }
  const size_t b = kNParam * sizeof(float);
  const char* cc = std::getenv("BN_MLP_CUDACORE");
  h->use_tc = !(cc && cc[0] == '1');
  if (cudaMalloc(&h->err, sizeof(int)) != cudaSuccess || cudaMemset(h->err, 0, sizeof(int)) != cudaSuccess ||
      cudaFuncSetAttribute(site_kernel_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::kSmem) != cudaSuccess) {
    delete h;
    return BN_ERR_CUDA;
  }
  if (cudaMalloc(&h->params, b) != cudaSuccess || cudaMalloc(&h->adam1, b) != cudaSuccess ||
      cudaMalloc(&h->adam2, b) != cudaSuccess || cudaMalloc(&h->grad, b) != cudaSuccess ||
      cudaMemset(h->adam1, 0, b) != cudaSuccess || cudaMemset(h->adam2, 0, b) != cudaSuccess ||
      cudaMemset(h->params, 0, b) != cudaSuccess) {
    cudaFree(h->params);
    cudaFree(h->adam1);
    cudaFree(h->adam2);
    cudaFree(h->grad);
    delete h;
    return BN_ERR_CUDA;
  }
  *out = h;
  return BN_OK;
}

void bn_mlp_destroy(bn_mlp* h) {
  if (!h) return;
  cudaFree(h->err);
  cudaFree(h->params);
  cudaFree(h->adam1);
  cudaFree(h->adam2);
  cudaFree(h->grad);
  if (h->scratch) cudaFree(h->scratch);
  delete h;
}

int32_t bn_mlp_num_params(void) { return kNParam; }

int bn_mlp_set_params(bn_mlp* h, const float* params, const float* norm) {
  if (!h || (!params && !norm)) return BN_ERR_ARG;
  if (norm) {
    if (!norm_ok(norm)) return BN_ERR_ARG;
    std::memcpy(h->norm.in_mu, norm, 6 * 4);
    std::memcpy(h->norm.in_sd, norm + 6, 6 * 4);
    std::memcpy(h->norm.out_mu, norm + 12, 6 * 4);
    std::memcpy(h->norm.out_sd, norm + 18, 6 * 4);
  }
  if (params) {
    if (cudaMemcpy(h->params, params, kNParam * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
      return BN_ERR_CUDA;
    cudaMemset(h->adam1, 0, kNParam * sizeof(float));
    cudaMemset(h->adam2, 0, kNParam * sizeof(float));
    h->adam_t = 0;
  }
  return BN_OK;
}

int bn_mlp_get_params(bn_mlp* h, float* params, float* norm) {
  if (!h) return BN_ERR_ARG;
  if (params && cudaMemcpy(params, h->params, kNParam * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return BN_ERR_CUDA;
  if (norm) {
    std::memcpy(norm, h->norm.in_mu, 6 * 4);
    std::memcpy(norm + 6, h->norm.in_sd, 6 * 4);
    std::memcpy(norm + 12, h->norm.out_mu, 6 * 4);
    std::memcpy(norm + 18, h->norm.out_sd, 6 * 4);
  }
  return BN_OK;
}

// raw sites [n][6] (y, m1, m2, v11, v12, v22) -> standardised features xn [n][6]
// and, when requested, cubature targets (ncub^2 points): standardised tn [n][6]
// and raw traw [n][6] (E, g1, g2, h11, h12, h22).  Device pointers.
int bn_mlp_prepare(bn_mlp* h, void* stream, int32_t n, int32_t ncub, const float* raw, float* xn, float* tn,
                   float* traw) {
  if (!h || n < 1 || !raw || !xn || ncub < 2 || ncub > BN_MAX_CUB) return BN_ERR_ARG;
  bn_lik_desc d;
  std::memset(&d, 0, sizeof(d));
  d.kind = h->kind;
  d.num_cub = ncub;
  bn::LikParams<float> lp;
  if (bn::build_lik<float>(&d, lp) != BN_OK) return BN_ERR_ARG;
  prepare_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(n, h->norm, h->kind, lp, raw, xn,
                                                                                 tn, traw);
  return cudaGetLastError() == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}

// The learned site pass on raw marginals (pm [n][2], pv [n][2][2], y [n]) ->
// ext [n][6], with the model step's checks and cubature pass (ncub x ncub GH);
// counts [2] (host) = sites reverted for precision / by the spot check.
// tensor_cores: 1 tcgen05 pass, 0 CUDA-core pass.
int bn_mlp_sites(bn_mlp* h, void* stream, int64_t n, const float* pm, const float* pv, const float* y, int32_t ncub,
                 int32_t spot, double tol, int32_t tensor_cores, float* ext, uint32_t* counts) {
  if (!h || n < 1 || !pm || !pv || !y || !ext || ncub < 2 || ncub > BN_MAX_CUB) return BN_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  bn_lik_desc d;
  std::memset(&d, 0, sizeof(d));
  d.kind = h->kind;
  d.num_cub = ncub;
  bn::LikParams<float> lp;
  if (bn::build_lik<float>(&d, lp) != BN_OK) return BN_ERR_ARG;
  unsigned* buf = nullptr;
  if (cudaMalloc(&buf, (2 + 2 * (size_t(n) + 1)) * sizeof(unsigned)) != cudaSuccess) return BN_ERR_CUDA;
  cudaMemsetAsync(buf, 0, 2 * sizeof(unsigned), st);
  const bool keep = h->use_tc;
  h->use_tc = tensor_cores != 0;
  int e = bn::mlp_site_expectations(h, st, n, pm, pv, y, lp, spot, float(tol), ext, buf, buf + 2);
  h->use_tc = keep;
  unsigned c[2] = {0u, 0u};
  int werr = 0;
  if (e == BN_OK && (cudaMemcpyAsync(c, buf, sizeof(c), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                     cudaMemcpyAsync(&werr, h->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                     cudaStreamSynchronize(st) != cudaSuccess))
    e = BN_ERR_CUDA;
  cudaFree(buf);
  if (counts) {
    counts[0] = c[0];
    counts[1] = c[1];
  }
  if (e == BN_OK && werr) e = BN_ERR_CUDA;
  return e;
}

int bn_mlp_forward(bn_mlp* h, void* stream, int32_t n, const float* xn, float* out) {
  if (!h || n < 1 || !xn || !out) return BN_ERR_ARG;
  forward_kernel<<<(n + kTPB - 1) / kTPB, kTPB, kNParam * 4, static_cast<cudaStream_t>(stream)>>>(n, h->params, xn,
                                                                                                out);
  return cudaGetLastError() == cudaSuccess ? BN_OK : BN_ERR_CUDA;
}

// loss and its gradient (host grad[kNParam]) on standardised (xn, tn), device pointers
int bn_mlp_loss_grad(bn_mlp* h, void* stream, int32_t n, const float* xn, const float* tn, double* loss,
                     float* grad) {
  if (!h || n < 1 || !xn || !tn) return BN_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int e = loss_grad(h, st, n, xn, tn, loss);
  if (e != BN_OK) return e;
  if (grad) {
    if (cudaMemcpyAsync(grad, h->grad, kNParam * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return BN_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BN_ERR_CUDA;
  }
  return BN_OK;
}

// Adam on random mini-batches of (xn, tn) [n]: `steps` updates of batch `bsz`;
// *loss = the loss of the last mini-batch.
int bn_mlp_train(bn_mlp* h, void* stream, int32_t n, const float* xn, const float* tn, int32_t steps, int32_t bsz,
                 float lr, uint32_t seed, double* loss) {
  if (!h || n < 1 || !xn || !tn || steps < 1 || bsz < 1) return BN_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float *xb = nullptr, *tb = nullptr;
  if (cudaMalloc(&xb, size_t(bsz) * kIn * 4) != cudaSuccess) return BN_ERR_CUDA;
  if (cudaMalloc(&tb, size_t(bsz) * kOut * 4) != cudaSuccess) {
    cudaFree(xb);
    return BN_ERR_CUDA;
  }
  int err = BN_OK;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int s = 0; s < steps && err == BN_OK; ++s) {
    gather_batch_kernel<<<(bsz + 255) / 256, 256, 0, st>>>(n, bsz, unsigned(s), seed, xn, tn, xb, tb);
    err = loss_grad(h, st, bsz, xb, tb, s == steps - 1 ? loss : nullptr);
    if (err != BN_OK) break;
    ++h->adam_t;
    const float c1 = 1.f - std::pow(b1, float(h->adam_t)), c2 = 1.f - std::pow(b2, float(h->adam_t));
    adam_kernel<<<(kNParam + 255) / 256, 256, 0, st>>>(kNParam, h->params, h->grad, h->adam1, h->adam2, lr, b1, b2,
                                                       c1, c2, 1e-8f);
    if (cudaGetLastError() != cudaSuccess) err = BN_ERR_CUDA;
  }
  cudaStreamSynchronize(st);
  cudaFree(xb);
  cudaFree(tb);
  return err;
}

}  // extern "C"
