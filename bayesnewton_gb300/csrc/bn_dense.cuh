// Batched dense linear algebra for the spatio-temporal path (state dimension
// d = M x S in the hundreds): every routine runs one independent problem per
// batch index, with operands addressed as base + (mul * i + add) * stride so
// that the scan levels can pair elements (i -> 2i+1, 2i+3 ...) without copies.
// Matrices are row-major, contiguous (leading dimension = column count).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdlib>

#include "bn_tc.cuh"

namespace bn {
namespace dense {

// Operand i of a batched call: p + (mul * i + add) * stride.
struct BRef {
  float* p;
  int64_t stride, mul, add;
  __host__ __device__ BRef() : p(nullptr), stride(0), mul(0), add(0) {}
  __host__ __device__ BRef(float* p_, int64_t s, int64_t m = 1, int64_t a = 0) : p(p_), stride(s), mul(m), add(a) {}
  __device__ __forceinline__ float* at(int i) const { return p + (mul * int64_t(i) + add) * stride; }
};

// ---------------------------------------------------------------- GEMM
// C_i = alpha op(A_i) op(B_i) + beta C0_i (+ I when add_identity), C_i M x N,
// op(A) M x K, op(B) K x N.  C0 may be the same storage as C (each output
// element reads only its own C0 entry).  64 x 64 tiles, 16-deep k slices, 256
// threads with a 4 x 4 register tile each, float32 FMA accumulation.
constexpr int kGT = 64, kGK = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) bgemm_kernel(int M, int N, int K, float alpha, BRef A, BRef B, float beta,
                                                    BRef C0, BRef C, int add_identity) {
  __shared__ float As[kGK][kGT + 4];
  __shared__ float Bs[kGK][kGT + 4];
  const int bi = blockIdx.z;
  const float* a = A.at(bi);
  const float* b = B.at(bi);
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kGK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;  // 1024 elements of each 64 x 16 slice
      if (!TA) {
        const int kk = e & 15, mm = e >> 4;
        const int gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < M && gk < K) ? a[int64_t(gm) * K + gk] : 0.f;
      } else {
        const int mm = e & 63, kk = e >> 6;
        const int gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < M && gk < K) ? a[int64_t(gk) * M + gm] : 0.f;
      }
      if (!TB) {
        const int nn = e & 63, kk = e >> 6;
        const int gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < N && gk < K) ? b[int64_t(gk) * N + gn] : 0.f;
      } else {
        const int kk = e & 15, nn = e >> 4;
        const int gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < N && gk < K) ? b[int64_t(gn) * K + gk] : 0.f;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      float av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* c = C.at(bi);
  const float* c0 = beta != 0.f ? C0.at(bi) : nullptr;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = alpha * acc[i][j];
      if (c0) v = fmaf(beta, c0[int64_t(gm) * N + gn], v);
      if (add_identity && gm == gn) v += 1.f;
      c[int64_t(gm) * N + gn] = v;
    }
  }
}

// ---------------------------------------------------------------- tensor-core GEMM
// The same batched product on the tcgen05 tensor cores in 3xTF32: each operand is
// split into a TF32 head and its float32 remainder, x = hi + lo, and
// A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi (float32-level accuracy), accumulated
// in float32 in tensor memory.  A CTA of 128 threads owns a 128 x 64 tile of C;
// K runs in 32-deep stages, double-buffered in shared memory (the hi / lo parts of
// both operands in the canonical K-major layout, op(A) and op(B) transposed on the
// way in), one thread issuing 3 x 4 MMAs (M = 128, N = 64, K = 8) per stage and
// committing them to the stage's mbarrier, so that the next stage loads while the
// tensor cores work.  The epilogue reads the accumulator back with tcgen05.ld (warp
// w: rows 32w..32w+31) and applies alpha, beta C0 and the identity.
constexpr int kTM = 128, kTN = 64, kTK = 32;
constexpr int kTSBO = (kTK / 4) * 128;                      // 1024 B between 8-row groups
constexpr int kTAh = 0, kTAl = kTM * kTK * 4, kTBh = 2 * kTM * kTK * 4, kTBl = kTBh + kTN * kTK * 4;
constexpr int kTStage = kTBl + kTN * kTK * 4;               // 48 KB
constexpr int kTSmem = 2 * kTStage;

static __device__ int g_tc_gemm_err;

// Loads of one stage: the operand chunk of 4 consecutive elements along the
// contiguous dimension of its global layout (K for A, N for B when not
// transposed) as one 16-byte load when VEC (rows a multiple of 4 long, 16-byte
// aligned base), split into TF32 head and remainder, stored at the K-major offsets.
// Internal linkage (here and in the launch helpers below): the dynamic
// shared-memory opt-in is an attribute of one translation unit's kernel, so each
// unit that launches the kernel owns its instantiation and sets it itself.
template <bool TA, bool TB, bool VEC>
static __global__ void __launch_bounds__(256) tc_bgemm_kernel(int M, int N, int K, float alpha, BRef A, BRef B, float beta,
                                                       BRef C0, BRef C, int add_identity) {
  using namespace ::bn::tc;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t taddr_s;
  __shared__ __align__(8) uint64_t mbar_s[2];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int bi = blockIdx.z;
  const float* a = A.at(bi);
  const float* b = B.at(bi);
  const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
  const uint32_t base = uint32_t(__cvta_generic_to_shared(tsm));
  const uint32_t mb0 = uint32_t(__cvta_generic_to_shared(&mbar_s[0]));
  const uint32_t mb1 = uint32_t(__cvta_generic_to_shared(&mbar_s[1]));
  if (warp == 0) {
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(&taddr_s));
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(dst));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  auto put = [&](unsigned char* p, int hi_off, int lo_off, int r, int k, float v) {
    const float h = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    const uint32_t o = off_k(r, k, kTSBO);
    *reinterpret_cast<float*>(p + hi_off + o) = h;
    *reinterpret_cast<float*>(p + lo_off + o) = v - h;
  };
  auto put4 = [&](unsigned char* p, int hi_off, int lo_off, int r, int k, const float (&v)[4]) {
    float h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      h[i] = __uint_as_float(__float_as_uint(v[i]) & 0xFFFFE000u);
      l[i] = v[i] - h[i];
    }
    const uint32_t o = off_k(r, k, kTSBO);  // 16 contiguous bytes: one core-matrix row
    *reinterpret_cast<float4*>(p + hi_off + o) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4*>(p + lo_off + o) = make_float4(l[0], l[1], l[2], l[3]);
  };
  // One stage is fetched from global memory into registers (issued before the wait
  // for the MMAs that still read the destination buffer, so the loads overlap it)
  // and then split into TF32 heads and remainders in shared memory.
  constexpr int kCA = kTM * kTK / 4 / 256, kCB = kTN * kTK / 4 / 256;  // float4 chunks per thread
  float va[kCA][4], vb[kCB][4];
  auto fetch = [&](int kt) {
    const int k0 = kt * kTK;
#pragma unroll
    for (int i = 0; i < kCA; ++i) {
      const int c = tid + 256 * i;
#pragma unroll
      for (int q = 0; q < 4; ++q) va[i][q] = 0.f;
      if (!TA) {
        const int r = c >> 3, kk = (c & 7) * 4;  // 8 chunks per row
        const int gm = m0 + r, gk = k0 + kk;
        if (gm < M) {
          if (VEC && gk + 3 < K) {
            const float4 q = *reinterpret_cast<const float4*>(a + int64_t(gm) * K + gk);
            va[i][0] = q.x, va[i][1] = q.y, va[i][2] = q.z, va[i][3] = q.w;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (gk + q < K) va[i][q] = a[int64_t(gm) * K + gk + q];
          }
        }
      } else {
        const int kk = c >> 5, r = (c & 31) * 4;  // 32 chunks of 4 m per k
        const int gm = m0 + r, gk = k0 + kk;
        if (gk < K) {
          if (VEC && gm + 3 < M) {
            const float4 q = *reinterpret_cast<const float4*>(a + int64_t(gk) * M + gm);
            va[i][0] = q.x, va[i][1] = q.y, va[i][2] = q.z, va[i][3] = q.w;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (gm + q < M) va[i][q] = a[int64_t(gk) * M + gm + q];
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < kCB; ++i) {
      const int c = tid + 256 * i;
#pragma unroll
      for (int q = 0; q < 4; ++q) vb[i][q] = 0.f;
      if (!TB) {
        const int kk = c >> 4, n = (c & 15) * 4;  // 16 chunks of 4 n per k
        const int gn = n0 + n, gk = k0 + kk;
        if (gk < K) {
          if (VEC && gn + 3 < N) {
            const float4 q = *reinterpret_cast<const float4*>(b + int64_t(gk) * N + gn);
            vb[i][0] = q.x, vb[i][1] = q.y, vb[i][2] = q.z, vb[i][3] = q.w;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (gn + q < N) vb[i][q] = b[int64_t(gk) * N + gn + q];
          }
        }
      } else {
        const int n = c >> 3, kk = (c & 7) * 4;
        const int gn = n0 + n, gk = k0 + kk;
        if (gn < N) {
          if (VEC && gk + 3 < K) {
            const float4 q = *reinterpret_cast<const float4*>(b + int64_t(gn) * K + gk);
            vb[i][0] = q.x, vb[i][1] = q.y, vb[i][2] = q.z, vb[i][3] = q.w;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (gk + q < K) vb[i][q] = b[int64_t(gn) * K + gk + q];
          }
        }
      }
    }
  };
  auto stash = [&](int s) {
    unsigned char* p = tsm + s * kTStage;
#pragma unroll
    for (int i = 0; i < kCA; ++i) {
      const int c = tid + 256 * i;
      if (!TA) {
        put4(p, kTAh, kTAl, c >> 3, (c & 7) * 4, va[i]);
      } else {
        const int kk = c >> 5, r = (c & 31) * 4;
#pragma unroll
        for (int q = 0; q < 4; ++q) put(p, kTAh, kTAl, r + q, kk, va[i][q]);
      }
    }
#pragma unroll
    for (int i = 0; i < kCB; ++i) {
      const int c = tid + 256 * i;
      if (!TB) {
        const int kk = c >> 4, n = (c & 15) * 4;
#pragma unroll
        for (int q = 0; q < 4; ++q) put(p, kTBh, kTBl, n + q, kk, vb[i][q]);
      } else {
        put4(p, kTBh, kTBl, c >> 3, (c & 7) * 4, vb[i]);
      }
    }
  };
  // one thread polls an mbarrier (bounded), the block learns the outcome at the barrier
  auto block_wait = [&](uint32_t mb, uint32_t ph) {
    int w = 1;
    if (tid == 0) w = wait_phase(mb, ph) ? 1 : 0;
    return __syncthreads_and(w) != 0;
  };
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = taddr_s;
  const int nk = (K + kTK - 1) / kTK;
  uint32_t ph0 = 0u, ph1 = 0u;
  bool ok = true;
  fetch(0);
  stash(0);
  for (int kt = 0; kt < nk && ok; ++kt) {
    const int s = kt & 1;
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
      const uint32_t sb = base + uint32_t(s * kTStage);
      const uint32_t id = idesc_tf32(kTN);
#pragma unroll
      for (int j = 0; j < kTK / 8; ++j) {
        const uint32_t ah = sb + kTAh + j * 256, al = sb + kTAl + j * 256;
        const uint32_t bh = sb + kTBh + j * 256, bl = sb + kTBl + j * 256;
        mma_tf32(tmem, sdesc(ah, 128, kTSBO), sdesc(bh, 128, kTSBO), id, (kt > 0 || j > 0) ? 1u : 0u);
        mma_tf32(tmem, sdesc(ah, 128, kTSBO), sdesc(bl, 128, kTSBO), id, 1u);
        mma_tf32(tmem, sdesc(al, 128, kTSBO), sdesc(bh, 128, kTSBO), id, 1u);
      }
      commit(s ? mb1 : mb0);
    }
    if (kt + 1 < nk) {
      fetch(kt + 1);
      // buffer s ^ 1 was read by the MMAs of stage kt - 1: wait for them first
      if (kt >= 1) {
        if (s == 0) {
          ok = block_wait(mb1, ph1);
          ph1 ^= 1u;
        } else {
          ok = block_wait(mb0, ph0);
          ph0 ^= 1u;
        }
      }
      if (ok) stash(s ^ 1);
    }
  }
  // the last one or two stages' commits are still outstanding
  if (ok && nk >= 2) {
    if (((nk - 2) & 1) == 0) {
      ok = block_wait(mb0, ph0);
      ph0 ^= 1u;
    } else {
      ok = block_wait(mb1, ph1);
      ph1 ^= 1u;
    }
  }
  if (ok) ok = block_wait((nk - 1) & 1 ? mb1 : mb0, (nk - 1) & 1 ? ph1 : ph0);
  fence_after();
  if (ok) {
    // accumulator -> shared tile (the stage buffers are free now) -> coalesced rows.
    // Warps w and w + 4 share TMEM lanes 32 (w % 4) ..: columns 0-31 and 32-63; the
    // tile's row pitch of 65 floats keeps a warp's 32 rows on 32 banks.
    float* tile = reinterpret_cast<float*>(tsm);
    const int lw = warp & 3, half = warp >> 2;
    const int r = lw * 32 + (tid & 31);
    const uint32_t lane_base = tmem + (uint32_t(lw * 32) << 16);
#pragma unroll
    for (int cc = half * 32; cc < half * 32 + 32; cc += 16) {
      float v[16];
      ld16(lane_base + uint32_t(cc), v);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int i = 0; i < 16; ++i) tile[r * (kTN + 1) + cc + i] = v[i];
    }
    __syncthreads();
    float* c = C.at(bi);
    const float* c0 = beta != 0.f ? C0.at(bi) : nullptr;
    for (int e = tid; e < kTM * kTN; e += 256) {
      const int rr = e / kTN, col = e % kTN;
      const int gm = m0 + rr, gn = n0 + col;
      if (gm < M && gn < N) {
        float x = alpha * tile[rr * (kTN + 1) + col];
        if (c0) x = fmaf(beta, c0[int64_t(gm) * N + gn], x);
        if (add_identity && gm == gn) x += 1.f;
        c[int64_t(gm) * N + gn] = x;
      }
    }
  } else if (tid == 0) {
    atomicOr(&g_tc_gemm_err, 1);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// 16-byte vector loads apply when both operands' rows are whole float4s on
// 16-byte aligned bases (every batch element's too)
static inline bool tc_vec_ok(bool ta, bool tb, int M, int N, int K, const BRef& A, const BRef& B) {
  const bool al = (reinterpret_cast<uintptr_t>(A.p) % 16 == 0) && (reinterpret_cast<uintptr_t>(B.p) % 16 == 0) &&
                  A.stride % 4 == 0 && B.stride % 4 == 0;
  const int la = ta ? M : K, lb = tb ? K : N;
  return al && la % 4 == 0 && lb % 4 == 0;
}

template <bool TA, bool TB>
static inline void tc_launch(cudaStream_t st, dim3 g, bool vec, int M, int N, int K, float alpha, BRef A, BRef B, float beta,
                      BRef C0, BRef C, int ai) {
  if (vec) tc_bgemm_kernel<TA, TB, true><<<g, 256, kTSmem, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
  else tc_bgemm_kernel<TA, TB, false><<<g, 256, kTSmem, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
}

template <bool TA, bool TB>
static inline bool tc_attr() {
  return cudaFuncSetAttribute(tc_bgemm_kernel<TA, TB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTSmem) ==
             cudaSuccess &&
         cudaFuncSetAttribute(tc_bgemm_kernel<TA, TB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTSmem) ==
             cudaSuccess;
}

static inline void tc_gemm(cudaStream_t st, int batch, bool ta, bool tb, int M, int N, int K, float alpha, BRef A, BRef B,
                    float beta, BRef C0, BRef C, int ai) {
  dim3 g((N + kTN - 1) / kTN, (M + kTM - 1) / kTM, batch);
  const bool vec = tc_vec_ok(ta, tb, M, N, K, A, B);
  if (!ta && !tb) tc_launch<false, false>(st, g, vec, M, N, K, alpha, A, B, beta, C0, C, ai);
  else if (ta && !tb) tc_launch<true, false>(st, g, vec, M, N, K, alpha, A, B, beta, C0, C, ai);
  else if (!ta && tb) tc_launch<false, true>(st, g, vec, M, N, K, alpha, A, B, beta, C0, C, ai);
  else tc_launch<true, true>(st, g, vec, M, N, K, alpha, A, B, beta, C0, C, ai);
}

static inline bool tc_attr_all() { return tc_attr<false, false>() && tc_attr<true, false>() && tc_attr<false, true>() && tc_attr<true, true>(); }

// The tensor-core path is opt-in (BN_TC_GEMM=1): with the operand split and the
// K-major staging done by the CTA's own threads it runs the spatio-temporal step
// at 167 ms against 125 ms on the CUDA-core tiles (the per-element staging, not
// the tensor cores, is its bottleneck); TMA staging is the next step for it.
static inline bool tc_gemm_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("BN_TC_GEMM");
    if (!(e && e[0] == '1')) return false;
    return tc_attr_all();
  }();
  return on;
}

inline void bgemm(cudaStream_t st, int batch, bool ta, bool tb, int M, int N, int K, float alpha, BRef A, BRef B,
                  float beta, BRef C0, BRef C, bool add_identity = false) {
  if (batch <= 0) return;
  const int ai = add_identity ? 1 : 0;
  if (M >= 96 && N >= 32 && K >= 32 && tc_gemm_enabled()) {
    tc_gemm(st, batch, ta, tb, M, N, K, alpha, A, B, beta, C0, C, ai);
    return;
  }
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, batch);
  if (!ta && !tb) bgemm_kernel<false, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
  else if (ta && !tb) bgemm_kernel<true, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
  else if (!ta && tb) bgemm_kernel<false, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
  else bgemm_kernel<true, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, B, beta, C0, C, ai);
}

// ---------------------------------------------------------------- GEMV
// y_i = alpha op(A_i) x_i + beta y0_i (+ z_i), A_i R x C (op(A) = A^T when TA).
template <bool TA>
__global__ void __launch_bounds__(256) bgemv_kernel(int R, int Cc, float alpha, BRef A, BRef x, float beta, BRef y0,
                                                    BRef z, BRef y) {
  const int bi = blockIdx.x;
  const float* a = A.at(bi);
  const float* xv = x.at(bi);
  const float* y0v = beta != 0.f ? y0.at(bi) : nullptr;
  const float* zv = z.p ? z.at(bi) : nullptr;
  float* yv = y.at(bi);
  if (!TA) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = w; i < R; i += 8) {
      float s = 0.f;
      for (int j = lane; j < Cc; j += 32) s = fmaf(a[int64_t(i) * Cc + j], xv[j], s);
#pragma unroll
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) {
        float v = alpha * s;
        if (y0v) v = fmaf(beta, y0v[i], v);
        if (zv) v += zv[i];
        yv[i] = v;
      }
    }
  } else {
    for (int j = threadIdx.x; j < Cc; j += blockDim.x) {
      float s = 0.f;
      for (int i = 0; i < R; ++i) s = fmaf(a[int64_t(i) * Cc + j], xv[i], s);
      float v = alpha * s;
      if (y0v) v = fmaf(beta, y0v[j], v);
      if (zv) v += zv[j];
      yv[j] = v;
    }
  }
}

// y may alias y0 or z only when each output reads its own index (always true here).
inline void bgemv(cudaStream_t st, int batch, bool ta, int R, int Cc, float alpha, BRef A, BRef x, float beta, BRef y0,
                  BRef z, BRef y) {
  if (batch <= 0) return;
  if (ta) bgemv_kernel<true><<<batch, 256, 0, st>>>(R, Cc, alpha, A, x, beta, y0, z, y);
  else bgemv_kernel<false><<<batch, 256, 0, st>>>(R, Cc, alpha, A, x, beta, y0, z, y);
}

// ---------------------------------------------------------------- inverse
// In-place inverse of each n x n matrix (n <= kInvMax) by Gauss-Jordan elimination
// with partial pivoting, the matrix held in shared memory; logdet_i = log|det A_i|
// (double).  A zero pivot sets *status |= flag and leaves the matrix undefined.
constexpr int kInvMax = 216;
constexpr int kInvThreads = 1024;

inline size_t inv_smem(int n) { return size_t(n) * n * sizeof(float) + size_t(n) * (sizeof(float) + sizeof(int)) + 64; }

static __global__ void __launch_bounds__(kInvThreads) binv_kernel(int n, BRef A, double* logdet, int64_t ld_mul,
                                                           int64_t ld_add, int* status, int flag) {
  extern __shared__ __align__(16) unsigned char inv_raw[];
  float* a = reinterpret_cast<float*>(inv_raw);
  float* col = a + n * n;
  int* perm = reinterpret_cast<int*>(col + n);
  __shared__ float red_v[32];
  __shared__ int red_i[32];
  __shared__ double ld_acc;
  __shared__ int bad;
  const int bi = blockIdx.x;
  float* g = A.at(bi);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < n * n; e += nt) a[e] = g[e];
  if (tid == 0) {
    ld_acc = 0.0;
    bad = 0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot search in column k, rows k..n-1
    float best = -1.f;
    int bidx = k;
    for (int i = k + tid; i < n; i += nt) {
      const float v = fabsf(a[i * n + k]);
      if (v > best) {
        best = v;
        bidx = i;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      if (ov > best || (ov == best && oi < bidx)) {
        best = ov;
        bidx = oi;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = best;
      red_i[tid >> 5] = bidx;
    }
    __syncthreads();
    if (tid < 32) {
      const int nw = nt >> 5;
      best = tid < nw ? red_v[tid] : -1.f;
      bidx = tid < nw ? red_i[tid] : k;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
          best = ov;
          bidx = oi;
        }
      }
      if (tid == 0) {
        perm[k] = bidx;
        if (!(best > 0.f)) bad = 1;
      }
    }
    __syncthreads();
    const int p = perm[k];
    if (p != k)
      for (int j = tid; j < n; j += nt) {
        const float t = a[k * n + j];
        a[k * n + j] = a[p * n + j];
        a[p * n + j] = t;
      }
    __syncthreads();
    const float piv = a[k * n + k];
    const float ip = 1.f / piv;
    // float log (double-precision transcendentals run at 1/64 rate here and would
    // sit on every column's critical path), summed in double
    if (logdet && tid == 0) ld_acc += double(logf(fabsf(piv)));
    // column k (the multipliers) before the row updates overwrite it
    for (int i = tid; i < n; i += nt) col[i] = a[i * n + k];
    __syncthreads();
    for (int j = tid; j < n; j += nt) a[k * n + j] = (j == k ? 1.f : a[k * n + j]) * ip;
    __syncthreads();
    // rows by warps, columns by lanes (no index division, conflict-free rows)
    {
      const int lane = tid & 31, nw = nt >> 5;
      for (int i = tid >> 5; i < n; i += nw) {
        if (i == k) continue;
        const float f = col[i];
        float* ai = a + i * n;
        const float* ak = a + k * n;
        for (int j = lane; j < n; j += 32) ai[j] = (j == k ? 0.f : ai[j]) - f * ak[j];
      }
    }
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = n - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = tid; i < n; i += nt) {
        const float t = a[i * n + k];
        a[i * n + k] = a[i * n + p];
        a[i * n + p] = t;
      }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) g[e] = a[e];
  if (tid == 0) {
    if (logdet) logdet[ld_mul * bi + ld_add] = ld_acc;
    if (bad && status) atomicOr(status, flag);
  }
}

inline cudaError_t binv(cudaStream_t st, int batch, int n, BRef A, double* logdet, int64_t ld_mul, int64_t ld_add,
                        int* status, int flag) {
  if (batch <= 0) return cudaSuccess;
  binv_kernel<<<batch, kInvThreads, inv_smem(n), st>>>(n, A, logdet, ld_mul, ld_add, status, flag);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- Cholesky
// In-place lower Cholesky factor of each SPD n x n matrix (n <= kInvMax), held
// in shared memory; the strict upper triangle is zeroed; logdet_i = log|A_i| =
// 2 sum log L_kk (double).  A non-positive pivot sets *status |= flag and is
// replaced by a tiny positive value so that the factor stays finite.
static __global__ void __launch_bounds__(kInvThreads) bchol_kernel(int n, BRef A, double* logdet, int* status, int flag) {
  extern __shared__ __align__(16) unsigned char chol_raw[];
  float* a = reinterpret_cast<float*>(chol_raw);
  float* colk = a + n * n;
  __shared__ double ld_acc;
  __shared__ int bad;
  const int bi = blockIdx.x;
  float* g = A.at(bi);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < n * n; e += nt) a[e] = g[e];
  if (tid == 0) {
    ld_acc = 0.0;
    bad = 0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      float p = a[k * n + k];
      if (!(p > 0.f)) {
        bad = 1;
        p = 1e-30f;
      }
      const float l = sqrtf(p);
      a[k * n + k] = l;
      if (logdet) ld_acc += 2.0 * double(logf(l));
    }
    __syncthreads();
    const float il = 1.f / a[k * n + k];
    for (int i = k + 1 + tid; i < n; i += nt) {
      const float v = a[i * n + k] * il;
      a[i * n + k] = v;
      colk[i] = v;
    }
    __syncthreads();
    // trailing update of the lower triangle (rows i > k by warps, columns
    // k < j <= i by lanes), the column k read from its copy
    {
      const int lane = tid & 31, nw = nt >> 5;
      for (int i = k + 1 + (tid >> 5); i < n; i += nw) {
        const float lik = colk[i];
        float* ai = a + i * n;
        for (int j = k + 1 + lane; j <= i; j += 32) ai[j] = fmaf(-lik, colk[j], ai[j]);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    g[e] = j > i ? 0.f : a[e];
  }
  if (tid == 0) {
    if (logdet) logdet[bi] = ld_acc;
    if (bad && status) atomicOr(status, flag);
  }
}

inline void bchol(cudaStream_t st, int batch, int n, BRef A, double* logdet, int* status, int flag) {
  if (batch <= 0) return;
  bchol_kernel<<<batch, kInvThreads, size_t(n) * (n + 1) * sizeof(float), st>>>(n, A, logdet, status, flag);
}

// In-place inverse of each lower-triangular n x n L (n <= kInvMax) in shared
// memory, row by row: X[i][j] = -(sum_{j<=k<i} L[i][k] X[k][j]) / L[i][i] for j < i
// and 1 / L[i][i] on the diagonal.  Rows < i already hold X; row i of L is copied
// out before it is overwritten.  Warps take columns j, lanes split k.
static __global__ void __launch_bounds__(kInvThreads) btrinv_kernel(int n, BRef A) {
  extern __shared__ __align__(16) unsigned char tri_raw[];
  float* x = reinterpret_cast<float*>(tri_raw);
  float* row = x + n * n;
  const int bi = blockIdx.x;
  float* g = A.at(bi);
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, nw = nt >> 5;
  for (int e = tid; e < n * n; e += nt) x[e] = g[e];
  __syncthreads();
  for (int i = 0; i < n; ++i) {
    for (int k = tid; k <= i; k += nt) row[k] = x[i * n + k];
    __syncthreads();
    const float inv = 1.f / row[i];
    for (int j = tid >> 5; j < i; j += nw) {
      float s = 0.f;
      for (int k = j + lane; k < i; k += 32) s = fmaf(row[k], x[k * n + j], s);
#pragma unroll
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) x[i * n + j] = -s * inv;
    }
    if (tid == 0) x[i * n + i] = inv;
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    g[e] = j > i ? 0.f : x[e];
  }
}

inline void btrinv(cudaStream_t st, int batch, int n, BRef A) {
  if (batch <= 0) return;
  btrinv_kernel<<<batch, kInvThreads, size_t(n) * (n + 1) * sizeof(float), st>>>(n, A);
}

// Triangular solves with a lower factor L (n x n): X = L^-1 B (forward) or, with
// trans_l, X = L^-T B (backward); B is n x nc (or nc x n read transposed when
// trans_b); X is n x nc (or written transposed, nc x n, when trans_x).  L sits in
// shared memory; each thread solves whole columns.  X must not alias B unless
// neither is transposed.
static __global__ void __launch_bounds__(256) btrsm_kernel(int n, int nc, BRef L, BRef B, BRef X, int trans_l, int trans_b,
                                                    int trans_x) {
  extern __shared__ __align__(16) unsigned char trsm_raw[];
  float* l = reinterpret_cast<float*>(trsm_raw);
  const int bi = blockIdx.x;
  const float* lg = L.at(bi);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) l[e] = lg[e];
  __syncthreads();
  const float* b = B.at(bi);
  float* x = X.at(bi);
  for (int j = blockIdx.y * blockDim.x + threadIdx.x; j < nc; j += gridDim.y * blockDim.x) {
    auto bin = [&](int i) { return trans_b ? b[int64_t(j) * n + i] : b[int64_t(i) * nc + j]; };
    auto xo = [&](int i) -> float& { return trans_x ? x[int64_t(j) * n + i] : x[int64_t(i) * nc + j]; };
    if (!trans_l) {
      for (int i = 0; i < n; ++i) {
        float s = bin(i);
        for (int k = 0; k < i; ++k) s = fmaf(-l[i * n + k], xo(k), s);
        xo(i) = s / l[i * n + i];
      }
    } else {
      for (int i = n - 1; i >= 0; --i) {
        float s = bin(i);
        for (int k = i + 1; k < n; ++k) s = fmaf(-l[k * n + i], xo(k), s);
        xo(i) = s / l[i * n + i];
      }
    }
  }
}

inline void btrsm(cudaStream_t st, int batch, int n, int nc, BRef L, BRef B, BRef X, bool trans_l, bool trans_b,
                  bool trans_x) {
  if (batch <= 0) return;
  const int gy = (nc + 255) / 256;
  btrsm_kernel<<<dim3(batch, gy), 256, size_t(n) * n * sizeof(float), st>>>(n, nc, L, B, X, trans_l ? 1 : 0,
                                                                          trans_b ? 1 : 0, trans_x ? 1 : 0);
}

// ---------------------------------------------------------------- copies
static __global__ void bcopy_kernel(int64_t len, BRef src, BRef dst) {
  const float* s = src.at(blockIdx.y);
  float* d = dst.at(blockIdx.y);
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < len; e += int64_t(gridDim.x) * blockDim.x)
    d[e] = s[e];
}
inline void bcopy(cudaStream_t st, int batch, int64_t len, BRef src, BRef dst) {
  if (batch <= 0) return;
  int gx = int((len + 255) / 256);
  if (gx > 64) gx = 64;
  bcopy_kernel<<<dim3(gx, batch), 256, 0, st>>>(len, src, dst);
}

// identity element of the filter scan: A = I, b = C = J = eta = 0 (or E = I, g = L = 0)
static __global__ void bidentity_kernel(int d, BRef I, BRef Z1, BRef Z2, BRef v1, BRef v2) {
  const int bi = blockIdx.y;
  float* ip = I.at(bi);
  float* z1 = Z1.p ? Z1.at(bi) : nullptr;
  float* z2 = Z2.p ? Z2.at(bi) : nullptr;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d * d; e += gridDim.x * blockDim.x) {
    ip[e] = (e / d == e % d) ? 1.f : 0.f;
    if (z1) z1[e] = 0.f;
    if (z2) z2[e] = 0.f;
  }
  float* a = v1.p ? v1.at(bi) : nullptr;
  float* b = v2.p ? v2.at(bi) : nullptr;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d; e += gridDim.x * blockDim.x) {
    if (a) a[e] = 0.f;
    if (b) b[e] = 0.f;
  }
}

}  // namespace dense
}  // namespace bn
