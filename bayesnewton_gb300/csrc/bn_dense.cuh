// Batched dense linear algebra for the spatio-temporal path (state dimension
// d = M x S in the hundreds): every routine runs one independent problem per
// batch index, with operands addressed as base + (mul * i + add) * stride so
// that the scan levels can pair elements (i -> 2i+1, 2i+3 ...) without copies.
// Matrices are row-major, contiguous (leading dimension = column count).
#pragma once
#include <cuda.h>
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
  // the tile's C0 values are loaded before any store (C0 may be C itself, so a load
  // could not move past an earlier store on its own)
  float cv[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      cv[i][j] = (c0 && gm < M && gn < N) ? c0[int64_t(gm) * N + gn] : 0.f;
    }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = alpha * acc[i][j];
      if (c0) v = fmaf(beta, cv[i][j], v);
      if (add_identity && gm == gn) v += 1.f;
      c[int64_t(gm) * N + gn] = v;
    }
  }
}

// ---------------------------------------------------------------- tensor-core GEMM
// The same batched product on the tcgen05 tensor cores in 3xTF32: each operand is
// split into its nearest TF32 value and the nearest TF32 value of the remainder,
// x ~ hi + lo (|x - hi - lo| <= 2^-22 |x|), and
// A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi (float32-level accuracy), accumulated in
// float32 in tensor memory.
//
// A persistent CTA per SM walks the 128 x BN tiles of C (batch, row tile, column
// tile; neighbouring CTAs share A and B blocks in L2; BN below) with four warp roles
// around mbarrier rings:
//   warp 16, one lane TMA producer: per 32-deep K stage, cp.async.bulk.tensor loads
//                     of op(A) (128 x 32) and op(B) (BN x 32) into a raw ring with
//                     the 128-byte swizzle; K-major operands arrive as one box of
//                     32 K x rows, M/N-major ones (a transposed A, an untransposed
//                     B) as 32 x 32 boxes;
//   warps 8-15        split: thread (warp w, lane l) takes row 32 (w % 4) + l of
//                     op(A), K columns 16 ((w - 8) / 4) .. + 15, and stores their
//                     hi / lo parts into tensor memory
//                     (tcgen05.st: the MMAs read A from there, which keeps A's
//                     three reads per slice off the shared-memory port); op(B) goes
//                     to the hi / lo halves of a double-buffered set in the
//                     canonical K-major 128-byte-swizzled layout (8-row groups
//                     1024 B apart), elementwise from K-major raw data, through
//                     4 x 4 register transposes from M/N-major (lane pattern chosen
//                     so that the reads and the writes of every 8 lanes hit 8
//                     distinct 16-byte bank groups);
//   warp 17, one lane MMA issuer: 3 MMAs (M = 128, N = BN, K = 8, A in tensor
//                     memory) per 8-deep slice into one of two accumulators,
//                     committed to the set's mbarrier (which frees the set and its
//                     A columns) and, after a tile's last stage, to the
//                     accumulator's;
//   warps 0-7         epilogue: warps w and w + 4 read accumulator rows 32 w..
//                     32 w + 31 (lane quarter w), alternate 32-column chunks ->
//                     a per-warp 32 x 32 staging tile -> alpha acc + beta C0 (+ I)
//                     stored a row segment of 128 B at a time (C0 read 16 rows at a
//                     time), while the tensor cores run the next tile in the other
//                     accumulator.
// Tensor memory (512 columns): see Cfg (accumulators and the A hi / lo pairs).
// Every wait is bounded: a wait that runs out raises the CTA's abort flag (the
// other roles see it and leave their loops) and the error flag the host reads.
namespace tg {
constexpr int kBM = 128, kBK = 32;
constexpr int kStage = 32 * 33 * 4;                       // epilogue staging per warp
constexpr int kThreads = 576;                             // 8 epilogue, 8 split, TMA, MMA warps
constexpr int kSplit = 256;                               // split threads
constexpr uint32_t kBytesKMajorA = kBM * 128, kBytesMNMajorA = 4 * 32 * 128;
// Column tile BN = 112 (two accumulators at columns 0 / 128, two A sets at 256 + 64 h,
// a 4-slot raw ring) or BN = 208 (one column tile for N <= 208: every A block is
// loaded and split once instead of twice; accumulators at 0 / 224, one A set at
// 448, which the split refills once the previous stage's MMAs are done; a 2-slot
// raw ring of 44 KB slots).  The MMA N is BN.
template <int BN>
struct Cfg {
  static constexpr int kBN = BN;
  static constexpr int kNBoxB = (BN + 31) / 32;                   // 32-row boxes of an M/N-major B
  static constexpr int kRaw = BN > 128 ? 2 : 4;                   // raw ring slots
  static constexpr int kRawA = 16384, kRawB = kNBoxB * 4096, kRawSlot = kRawA + kRawB;
  static constexpr int kHiB = BN * 128;
  static constexpr int kSet = 2 * kHiB;                           // hi B, lo B
  static constexpr int kOffSet = kRaw * kRawSlot;
  static constexpr int kOffStage = kOffSet + 2 * kSet;
  static constexpr int kSmem = kOffStage + 8 * kStage + 1024;     // + 1024 B for the base alignment
  static constexpr int kAccCols = BN > 128 ? 224 : 128;           // accumulator b at column kAccCols b
  static constexpr int kASets = BN > 128 ? 1 : 2;
  static constexpr int kACol = 2 * kAccCols;                      // A of set h: hi at kACol + 64 h, lo + 32
  static constexpr uint32_t kBytesKMajorB = BN * 128, kBytesMNMajorB = kNBoxB * 4096;
  static_assert(kSmem <= 232448, "shared memory");
  static_assert(kACol + 64 * kASets <= 512, "tensor memory");
};
}  // namespace tg

static __device__ int g_tc_gemm_err;

// K-major operand in the 128-byte swizzle: rows of 128 B (32 float32 of K), 8-row
// groups 1024 B apart; the start address steps by 32 B per 8-deep K slice
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  return uint64_t((saddr >> 4) & 0x3FFF) | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) |
         (uint64_t(2) << 61);
}

__device__ __forceinline__ bool tg_try(uint32_t mb, uint32_t par) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(mb), "r"(par)
      : "memory");
  return done != 0;
}

// bounded wait that also gives up once another role has raised the abort flag
__device__ __forceinline__ bool tg_wait(uint32_t mb, uint32_t par, volatile int* abort_flag) {
  for (unsigned it = 0; it < ::bn::tc::kWaitLimit; ++it) {
    if (tg_try(mb, par)) return true;
    if ((it & 63) == 63) {
      if (*abort_flag) return false;
      __nanosleep(32);
    }
  }
  *abort_flag = 1;
  atomicOr(&g_tc_gemm_err, 1);
  return false;
}

__device__ __forceinline__ void tg_arrive(uint32_t mb) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mb) : "memory");
}

__device__ __forceinline__ void tg_expect(uint32_t mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tg_load(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t mb) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mb)
      : "memory");
}

// nearest TF32 value (ties away from zero): add half a unit of the 10-bit
// mantissa's last place, then clear the 13 low bits
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void tg_pair(float x, float& h, float& l) {
  h = tf32_rn(x);
  l = tf32_rn(x - h);
}

__device__ __forceinline__ void tg_pair4(float4 v, float4& h, float4& l) {
  tg_pair(v.x, h.x, l.x);
  tg_pair(v.y, h.y, l.y);
  tg_pair(v.z, h.z, l.z);
  tg_pair(v.w, h.w, l.w);
}

// 16 consecutive tensor-memory columns of the warp's 32 lanes
__device__ __forceinline__ void tg_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
      "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
      : "memory");
}

// op(A) row r, K columns 16 kh .. 16 kh + 15 of the raw slot (K-major: half of one
// 128-byte swizzled row; M-major: column r of box r / 32) -> hi / lo in tensor
// memory (the calling warp's 32 lanes)
template <bool TA>
__device__ __forceinline__ void tg_split_a(const unsigned char* raw, int r, int kh, uint32_t t_hi, uint32_t t_lo) {
  float h[16], l[16];
  if (!TA) {
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const int c = 4 * kh + cc;
      const float4 v = *reinterpret_cast<const float4*>(raw + r * 128 + ((c ^ (r & 7)) << 4));
      tg_pair(v.x, h[4 * cc], l[4 * cc]);
      tg_pair(v.y, h[4 * cc + 1], l[4 * cc + 1]);
      tg_pair(v.z, h[4 * cc + 2], l[4 * cc + 2]);
      tg_pair(v.w, h[4 * cc + 3], l[4 * cc + 3]);
    }
  } else {
    const unsigned char* box = raw + (r >> 5) * 4096;
    const int ml = r & 31;
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const int k = 16 * kh + kk;
      const float v = *reinterpret_cast<const float*>(box + k * 128 + (((ml >> 2) ^ (k & 7)) << 4) + (ml & 3) * 4);
      tg_pair(v, h[kk], l[kk]);
    }
  }
  tg_st16(t_hi, h);
  tg_st16(t_lo, l);
}

constexpr int kSplitStride = tg::kSplit;

// raw K-major rows -> hi / lo at the same (swizzled) offsets
__device__ __forceinline__ void tg_split_k(const unsigned char* raw, unsigned char* hi, unsigned char* lo, int bytes,
                                           int t) {
#pragma unroll 4
  for (int o = t * 16; o < bytes; o += kSplitStride * 16) {
    float4 h, l;
    tg_pair4(*reinterpret_cast<const float4*>(raw + o), h, l);
    *reinterpret_cast<float4*>(hi + o) = h;
    *reinterpret_cast<float4*>(lo + o) = l;
  }
}

// raw M/N-major boxes (box j: 32 K rows x 32 M/N, 128-byte swizzle) -> hi / lo rows
// n = 32 j + 4 c + p (K-major): thread block (j, k chunk a, M/N chunk c) with
// a = c ^ d, so that for fixed (j, d) eight lanes cover c = 0..7
__device__ __forceinline__ void tg_split_t(const unsigned char* raw, unsigned char* hi, unsigned char* lo, int rows,
                                           int nbox, int t) {
  for (int blk = t; blk < 64 * nbox; blk += kSplitStride) {
    const int j = blk >> 6, d = (blk >> 3) & 7, c = blk & 7, a = c ^ d;
    if (32 * j + 4 * c >= rows) continue;
    float4 r[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = 4 * a + q;
      r[q] = *reinterpret_cast<const float4*>(raw + j * 4096 + k * 128 + ((c ^ (k & 7)) << 4));
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int n = 32 * j + 4 * c + p;
      const float4 v = p == 0   ? make_float4(r[0].x, r[1].x, r[2].x, r[3].x)
                       : p == 1 ? make_float4(r[0].y, r[1].y, r[2].y, r[3].y)
                       : p == 2 ? make_float4(r[0].z, r[1].z, r[2].z, r[3].z)
                                : make_float4(r[0].w, r[1].w, r[2].w, r[3].w);
      float4 h, l;
      tg_pair4(v, h, l);
      const int o = n * 128 + ((a ^ (n & 7)) << 4);
      *reinterpret_cast<float4*>(hi + o) = h;
      *reinterpret_cast<float4*>(lo + o) = l;
    }
  }
}

// Internal linkage (here and in the launch helpers below): the dynamic
// shared-memory opt-in is an attribute of one translation unit's kernel, so each
// unit that launches the kernel owns its instantiation and sets it itself.
// QF: instead of C, out_i[r] = alpha a_r^T op(B_i) a_r for each row a_r of A_i
// (N = K, one column tile): the epilogue thread that holds accumulator row r dots
// it with row r of A (read through QA) and writes one value (C.at(i)[r]).
template <bool TA, bool TB, bool QF = false, int BN = 112>
static __global__ void __launch_bounds__(tg::kThreads, 1)
    tc_bgemm_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int M, int N,
                    int K, int batch, float alpha, float beta, BRef C0, BRef C, int add_identity, BRef QA = BRef()) {
  using namespace ::bn::tc;
  using namespace tg;
  using G = Cfg<BN>;
  constexpr int kBN = BN, kRaw = G::kRaw, kRawA = G::kRawA, kRawSlot = G::kRawSlot, kHiB = G::kHiB, kSet = G::kSet;
  constexpr int kOffSet = G::kOffSet, kOffStage = G::kOffStage, kAccCols = G::kAccCols, kACol = G::kACol;
  constexpr int kASets = G::kASets, kNBoxB = G::kNBoxB;
  extern __shared__ unsigned char tg_dsm[];
  __shared__ __align__(8) uint64_t bars[2 * kRaw + 8];
  __shared__ uint32_t taddr_s;
  __shared__ int abort_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sraw = uint32_t(__cvta_generic_to_shared(tg_dsm));
  const uint32_t base = (sraw + 1023u) & ~1023u;
  unsigned char* gbase = tg_dsm + (base - sraw);
  const uint32_t b0 = uint32_t(__cvta_generic_to_shared(&bars[0]));
  // raw_full[r] = bars[r], raw_empty[r] = bars[kRaw + r], set_full[h] = bars[2 kRaw + h],
  // set_empty[h] = bars[2 kRaw + 2 + h], acc_full[b] = bars[2 kRaw + 4 + b],
  // acc_empty[b] = bars[2 kRaw + 6 + b]
  auto bar = [&](int i) { return b0 + 8u * uint32_t(i); };
  volatile int* abort_flag = &abort_s;
  if (tid == 0) {
    for (int r = 0; r < kRaw; ++r) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(r)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(kRaw + r)), "r"(kSplit));
    }
    for (int h = 0; h < 2; ++h) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(2 * kRaw + h)), "r"(kSplit));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(2 * kRaw + 2 + h)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(2 * kRaw + 4 + h)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 256;" ::"r"(bar(2 * kRaw + 6 + h)));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_s = 0;
  }
  if (warp == 17) {
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(&taddr_s));
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(dst));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = taddr_s;
  const int nM = (M + kBM - 1) / kBM, nN = (N + kBN - 1) / kBN, nk = (K + kBK - 1) / kBK;
  const int tiles = batch * nM * nN;
  auto decode = [&](int t, int& b, int& m0, int& n0) {
    const int nt = t % nN, r = t / nN;
    m0 = (r % nM) * kBM, n0 = nt * kBN, b = r / nM;
  };
  if (warp == 16) {
    if (lane == 0) {
      // ---- TMA producer
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
      const uint32_t bytes = (TA ? kBytesMNMajorA : kBytesKMajorA) + (TB ? G::kBytesKMajorB : G::kBytesMNMajorB);
      int it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        int b, m0, n0;
        decode(t, b, m0, n0);
        for (int kt = 0; kt < nk; ++kt, ++it) {
          const int r = it % kRaw;
          if (!(ok = tg_wait(bar(kRaw + r), ((it / kRaw) & 1) ^ 1, abort_flag))) break;
          const uint32_t full = bar(r), dst = base + uint32_t(r * kRawSlot);
          tg_expect(full, bytes);
          const int k0 = kt * kBK;
          if (!TA) {
            tg_load(dst, &map_a, k0, m0, b, full);
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) tg_load(dst + j * 4096, &map_a, m0 + 32 * j, k0, b, full);
          }
          if (TB) {
            tg_load(dst + kRawA, &map_b, k0, n0, b, full);
          } else {
#pragma unroll
            for (int j = 0; j < kNBoxB; ++j) tg_load(dst + kRawA + j * 4096, &map_b, n0 + 32 * j, k0, b, full);
          }
        }
      }
      // copies still in flight land before the CTA may leave (bounded)
      for (int q = 1; q <= kRaw && q <= it; ++q) {
        const int i = it - q;
        wait_phase_for(bar(i % kRaw), (i / kRaw) & 1, 1u << 20);
      }
    }
  } else if (warp == 17) {
    if (lane == 0) {
      // ---- MMA issuer
      const uint32_t id = idesc_tf32(kBN);
      int it = 0, tl = 0;
      bool ok = true;
      uint32_t last_mb = 0, last_ph = 0;
      for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++tl) {
        const int ab = tl & 1;
        if (!(ok = tg_wait(bar(2 * kRaw + 6 + ab), ((tl >> 1) & 1) ^ 1, abort_flag))) break;
        fence_after();
        const uint32_t d = tmem + uint32_t(ab * kAccCols);
        for (int kt = 0; kt < nk; ++kt, ++it) {
          const int h = it & 1;
          if (!(ok = tg_wait(bar(2 * kRaw + h), (it >> 1) & 1, abort_flag))) break;
          fence_after();
          const uint32_t sb = base + uint32_t(kOffSet + h * kSet);
          const uint32_t ta_hi = tmem + uint32_t(kACol + (kASets == 2 ? 64 * h : 0)), ta_lo = ta_hi + 32u;
          const int rem = K - kt * kBK, nj = rem >= kBK ? 4 : (rem + 7) / 8;
          for (int j = 0; j < nj; ++j) {
            const uint64_t bh = sdesc_sw128(sb + j * 32), bl = sdesc_sw128(sb + kHiB + j * 32);
            mma_tf32_ta(d, ta_hi + 8u * j, bh, id, (kt > 0 || j > 0) ? 1u : 0u);
            mma_tf32_ta(d, ta_hi + 8u * j, bl, id, 1u);
            mma_tf32_ta(d, ta_lo + 8u * j, bh, id, 1u);
          }
          commit(bar(2 * kRaw + 2 + h));
          last_mb = bar(2 * kRaw + 2 + h), last_ph = (it >> 1) & 1;
        }
        if (!ok) break;
        commit(bar(2 * kRaw + 4 + ab));
      }
      // the tensor cores finish their queue before tensor memory is released (bounded)
      if (last_mb) wait_phase_for(last_mb, last_ph, 1u << 20);
    }
  } else if (warp >= 8 && warp < 16) {
    // ---- split: raw slot -> A hi / lo in tensor memory, B hi / lo in the set
    const int st = tid - 256, ra = 32 * (warp & 3) + lane, kh = (warp - 8) >> 2;  // op(A) row, K half
    const uint32_t lane_off = uint32_t((warp & 3) * 32) << 16;
    int it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
      for (int kt = 0; kt < nk; ++kt, ++it) {
        const int r = it % kRaw, h = it & 1;
        if (!(ok = tg_wait(bar(r), (it / kRaw) & 1, abort_flag))) break;
        if (!(ok = tg_wait(bar(2 * kRaw + 2 + h), ((it >> 1) & 1) ^ 1, abort_flag))) break;
        fence_after();
        const unsigned char* raw = gbase + r * kRawSlot;
        unsigned char* set = gbase + kOffSet + h * kSet;
        if (TB) tg_split_k(raw + kRawA, set, set + kHiB, kHiB, st);
        else tg_split_t(raw + kRawA, set, set + kHiB, kBN, kNBoxB, st);
        // one A set: the previous stage's MMAs have to be done with it
        if (kASets == 1 && it > 0 && !(ok = tg_wait(bar(2 * kRaw + 2 + ((it - 1) & 1)), ((it - 1) >> 1) & 1, abort_flag)))
          break;
        fence_after();
        const uint32_t ta_hi = tmem + lane_off + uint32_t(kACol + (kASets == 2 ? 64 * h : 0) + 16 * kh);
        tg_split_a<TA>(raw, ra, kh, ta_hi, ta_hi + 32u);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        fence_async_smem();
        fence_before();
        tg_arrive(bar(kRaw + r));
        tg_arrive(bar(2 * kRaw + h));
      }
    }
  } else {
    // ---- epilogue: tensor memory -> alpha acc + beta C0 (+ I) -> C; warps w and w + 4
    // share lane quarter w (rows 32 w..) and take alternate 32-column chunks
    const int lq = warp & 3, eh = warp >> 2;
    float* stg = reinterpret_cast<float*>(gbase + kOffStage + warp * kStage);
    int tl = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++tl) {
      const int ab = tl & 1;
      if (!tg_wait(bar(2 * kRaw + 4 + ab), (tl >> 1) & 1, abort_flag)) break;
      fence_after();
      int b, m0, n0;
      decode(t, b, m0, n0);
      const uint32_t la = tmem + uint32_t(ab * kAccCols) + (uint32_t(lq * 32) << 16);
      if (QF && eh) {  // the row dots stay with warps 0-3
        tg_arrive(bar(2 * kRaw + 6 + ab));
        continue;
      }
      if (QF) {
        const int gm = m0 + lq * 32 + lane;
        const float* arow = QA.at(b) + int64_t(gm < M ? gm : 0) * K;
        float dot = 0.f;
#pragma unroll
        for (int cc = 0; cc < kBN; cc += 16) {
          float v[16];
          ld16(la + uint32_t(cc), v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (cc + 16 >= kBN) {  // the accumulator is free for the tile after next
            fence_before();
            tg_arrive(bar(2 * kRaw + 6 + ab));
          }
          if (gm < M) {
#pragma unroll
            for (int j = 0; j < 16; j += 4) {
              if (cc + j < N) {  // N is a multiple of 4 (TMA rows of whole 16-byte units)
                const float4 x = *reinterpret_cast<const float4*>(arow + cc + j);
                dot = fmaf(v[j], x.x, fmaf(v[j + 1], x.y, fmaf(v[j + 2], x.z, fmaf(v[j + 3], x.w, dot))));
              }
            }
          }
        }
        if (gm < M) C.at(b)[gm] = alpha * dot;
        continue;
      }
      // 32-column chunks: tensor memory -> registers -> the warp's staging tile
      // (pitch 33: the row writes and the column reads each hit 32 banks) -> 128-byte
      // row segments
      float* cb = C.at(b);
      const float* c0b = beta != 0.f ? C0.at(b) : nullptr;
      const int rows = M - (m0 + lq * 32) < 32 ? M - (m0 + lq * 32) : 32;
      if (32 * eh >= kBN) {  // no chunk for this warp
        tg_arrive(bar(2 * kRaw + 6 + ab));
        continue;
      }
#pragma unroll
      for (int cc = 32 * eh; cc < kBN; cc += 64) {
        float v[32];
        ld16(la + uint32_t(cc), *reinterpret_cast<float(*)[16]>(&v[0]));
        if (cc + 16 < kBN) ld16(la + uint32_t(cc + 16), *reinterpret_cast<float(*)[16]>(&v[16]));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (cc + 64 >= kBN) {  // this warp's last chunk: the accumulator is free for the tile after next
          fence_before();
          tg_arrive(bar(2 * kRaw + 6 + ab));
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (cc + j < kBN) stg[lane * 33 + j] = v[j];
        __syncwarp();
        const int gn = n0 + cc + lane;
        if (cc + lane < kBN && gn < N) {
          if (!c0b) {
            for (int rr = 0; rr < rows; ++rr) {
              const int gm = m0 + lq * 32 + rr;
              float x = alpha * stg[rr * 33 + lane];
              if (add_identity && gm == gn) x += 1.f;
              cb[int64_t(gm) * N + gn] = x;
            }
          } else {
            // sixteen rows at a time: their C0 loads are issued together (C0 may be C
            // itself, so a load cannot move past an earlier row's store on its own)
            for (int rb = 0; rb < rows; rb += 16) {
              float cv[16];
#pragma unroll
              for (int u = 0; u < 16; ++u)
                cv[u] = rb + u < rows ? c0b[int64_t(m0 + lq * 32 + rb + u) * N + gn] : 0.f;
#pragma unroll
              for (int u = 0; u < 16; ++u) {
                const int rr = rb + u;
                if (rr < rows) {
                  const int gm = m0 + lq * 32 + rr;
                  float x = fmaf(beta, cv[u], alpha * stg[rr * 33 + lane]);
                  if (add_identity && gm == gn) x += 1.f;
                  cb[int64_t(gm) * N + gn] = x;
                }
              }
            }
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 17) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}

typedef CUresult (*TgEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static inline TgEncodeFn tg_encoder() {
  static const TgEncodeFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return TgEncodeFn(nullptr);
    return reinterpret_cast<TgEncodeFn>(p);
  }();
  return fn;
}

// float32 tensor {inner, rows, batch} (row pitch inner, batch pitch bstride
// elements), boxes of 32 x box_rows x 1 with the 128-byte swizzle, zero fill
static inline bool tg_map(CUtensorMap* m, const float* p, int64_t inner, int64_t rows, int64_t batch, int64_t bstride,
                          int box_rows) {
  const TgEncodeFn enc = tg_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {cuuint64_t(inner), cuuint64_t(rows), cuuint64_t(batch)};
  const cuuint64_t strides[2] = {cuuint64_t(inner) * 4, cuuint64_t(bstride) * 4};
  const cuuint32_t box[3] = {32u, cuuint32_t(box_rows), 1u};
  const cuuint32_t es[3] = {1u, 1u, 1u};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(p), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool TA, bool TB, int BN>
static inline bool tc_attr() {
  return cudaFuncSetAttribute(tc_bgemm_kernel<TA, TB, false, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              tg::Cfg<BN>::kSmem) == cudaSuccess;
}

template <int BN>
static inline bool tc_attr_bn() {
  return tc_attr<false, false, BN>() && tc_attr<true, false, BN>() && tc_attr<false, true, BN>() &&
         tc_attr<true, true, BN>();
}

static inline bool tc_attr_all() {
  static const bool ok = tc_attr_bn<112>() && tc_attr_bn<208>() && tg_encoder() != nullptr;
  return ok;
}

// column tile: 208 (one tile) for 112 < N <= 208 and beyond, 112 up to N = 112
static inline int tg_bn(int N) { return N > 112 ? 208 : 112; }

static inline int tg_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

static inline bool tg_aligned(const float* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Launches the tensor-core product when the operands suit the TMA boxes: rows of
// whole 16-byte units (the contiguous extent a multiple of 4), 16-byte aligned
// bases, and batch pitches at least one matrix apart in 16-byte units.  false:
// nothing launched (the caller takes the CUDA-core tiles).
static inline bool tc_gemm(cudaStream_t st, int batch, bool ta, bool tb, int M, int N, int K, float alpha, BRef A,
                           BRef B, float beta, BRef C0, BRef C, int ai) {
  if (!tc_attr_all()) return false;
  const int64_t ia = ta ? M : K, ra = ta ? K : M, ib = tb ? K : N, rb = tb ? N : K;
  if (ia % 4 || ib % 4) return false;
  const float* pa = A.p + A.add * A.stride;
  const float* pb = B.p + B.add * B.stride;
  int64_t sa = A.mul * A.stride, sb = B.mul * B.stride;
  if (batch == 1) sa = ia * ra, sb = ib * rb;
  if (!tg_aligned(pa) || !tg_aligned(pb) || sa < ia * ra || sb < ib * rb || sa % 4 || sb % 4) return false;
  CUtensorMap ma, mb;
  const int bn = tg_bn(N);
  if (!tg_map(&ma, pa, ia, ra, batch, sa, ta ? 32 : tg::kBM)) return false;
  if (!tg_map(&mb, pb, ib, rb, batch, sb, tb ? bn : 32)) return false;
  const int64_t tiles = int64_t(batch) * ((M + tg::kBM - 1) / tg::kBM) * ((N + bn - 1) / bn);
  if (tiles > (int64_t(1) << 30)) return false;
  const unsigned grid = unsigned(tiles < tg_sms() ? tiles : tg_sms());
#define BN_TG_LAUNCH(TA_, TB_, BN_)                                                                      \
  tc_bgemm_kernel<TA_, TB_, false, BN_><<<grid, tg::kThreads, tg::Cfg<BN_>::kSmem, st>>>(ma, mb, M, N, K, batch, \
                                                                                        alpha, beta, C0, C, ai)
  if (bn == 208) {
    if (!ta && !tb) BN_TG_LAUNCH(false, false, 208);
    else if (ta && !tb) BN_TG_LAUNCH(true, false, 208);
    else if (!ta && tb) BN_TG_LAUNCH(false, true, 208);
    else BN_TG_LAUNCH(true, true, 208);
  } else {
    if (!ta && !tb) BN_TG_LAUNCH(false, false, 112);
    else if (ta && !tb) BN_TG_LAUNCH(true, false, 112);
    else if (!ta && tb) BN_TG_LAUNCH(false, true, 112);
    else BN_TG_LAUNCH(true, true, 112);
  }
#undef BN_TG_LAUNCH
  return true;
}

// Row quadratic forms out_i[r] = alpha a_r^T B_i^T a_r (A_i M x K row-major, B_i
// K x K stored as K-major rows, i.e. op(B) = B^T; for a symmetric B_i this is
// a_r^T B_i a_r) on the tensor cores; false: nothing launched (K above one column
// tile, or operands the TMA boxes do not suit).
static inline bool tc_rowquad(cudaStream_t st, int batch, int M, int K, float alpha, BRef A, BRef B, BRef out) {
  if (!tc_attr_all() || K > 112 || K % 4) return false;
  static const bool attr = cudaFuncSetAttribute(tc_bgemm_kernel<false, true, true, 112>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                tg::Cfg<112>::kSmem) == cudaSuccess;
  if (!attr) return false;
  const float* pa = A.p + A.add * A.stride;
  const float* pb = B.p + B.add * B.stride;
  int64_t sa = A.mul * A.stride, sb = B.mul * B.stride;
  if (batch == 1) sa = int64_t(K) * M, sb = int64_t(K) * K;
  if (!tg_aligned(pa) || !tg_aligned(pb) || sa < int64_t(K) * M || sb < int64_t(K) * K || sa % 4 || sb % 4)
    return false;
  CUtensorMap ma, mb;
  if (!tg_map(&ma, pa, K, M, batch, sa, tg::kBM)) return false;
  if (!tg_map(&mb, pb, K, K, batch, sb, 112)) return false;
  const int64_t tiles = int64_t(batch) * ((M + tg::kBM - 1) / tg::kBM);
  if (tiles > (int64_t(1) << 30)) return false;
  const unsigned grid = unsigned(tiles < tg_sms() ? tiles : tg_sms());
  tc_bgemm_kernel<false, true, true, 112><<<grid, tg::kThreads, tg::Cfg<112>::kSmem, st>>>(ma, mb, M, K, K, batch,
                                                                                          alpha, 0.f, BRef(), out, 0, A);
  return true;
}

// The tensor-core path is the default (BN_TC_GEMM=0 keeps every product on the
// CUDA-core tiles).
static inline bool tc_gemm_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("BN_TC_GEMM");
    if (e && e[0] == '0') return false;
    return tc_attr_all();
  }();
  return on;
}

static inline void bgemm(cudaStream_t st, int batch, bool ta, bool tb, int M, int N, int K, float alpha, BRef A,
                         BRef B, float beta, BRef C0, BRef C, bool add_identity = false) {
  if (batch <= 0) return;
  const int ai = add_identity ? 1 : 0;
  // below a full wave of 128 x 112 tiles the CUDA-core tiles finish sooner (their
  // 64 x 64 tiles spread one product over more CTAs)
  const int64_t tiles = int64_t(batch) * ((M + tg::kBM - 1) / tg::kBM) * ((N + 111) / 112);
  if (M >= 64 && N >= 32 && K >= 32 && tc_gemm_enabled() && tiles >= tg_sms() &&
      tc_gemm(st, batch, ta, tb, M, N, K, alpha, A, B, beta, C0, C, ai))
    return;
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
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // four chains: the column's loads overlap
      int i = 0;
      for (; i + 3 < R; i += 4) {
        s0 = fmaf(a[int64_t(i) * Cc + j], xv[i], s0);
        s1 = fmaf(a[int64_t(i + 1) * Cc + j], xv[i + 1], s1);
        s2 = fmaf(a[int64_t(i + 2) * Cc + j], xv[i + 2], s2);
        s3 = fmaf(a[int64_t(i + 3) * Cc + j], xv[i + 3], s3);
      }
      for (; i < R; ++i) s0 = fmaf(a[int64_t(i) * Cc + j], xv[i], s0);
      const float s = (s0 + s1) + (s2 + s3);
      float v = alpha * s;
      if (y0v) v = fmaf(beta, y0v[j], v);
      if (zv) v += zv[j];
      yv[j] = v;
    }
  }
}

// Two independent products of the form above in one launch (job blockIdx.y), each
// with its own transpose flag.
struct GemvJob {
  int ta, R, Cc;
  float alpha, beta;
  BRef A, x, y0, z, y;
};

static __global__ void __launch_bounds__(256) bgemv_jobs_kernel(GemvJob j0, GemvJob j1) {
  const GemvJob& jb = blockIdx.y == 0 ? j0 : j1;
  const int bi = blockIdx.x, R = jb.R, Cc = jb.Cc;
  const float* a = jb.A.at(bi);
  const float* xv = jb.x.at(bi);
  const float* y0v = jb.beta != 0.f ? jb.y0.at(bi) : nullptr;
  const float* zv = jb.z.p ? jb.z.at(bi) : nullptr;
  float* yv = jb.y.at(bi);
  if (!jb.ta) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = w; i < R; i += 8) {
      float sum = 0.f;
      for (int j = lane; j < Cc; j += 32) sum = fmaf(a[int64_t(i) * Cc + j], xv[j], sum);
#pragma unroll
      for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) {
        float v = jb.alpha * sum;
        if (y0v) v = fmaf(jb.beta, y0v[i], v);
        if (zv) v += zv[i];
        yv[i] = v;
      }
    }
  } else {
    for (int j = threadIdx.x; j < Cc; j += blockDim.x) {
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // four chains: the column's loads overlap
      int i = 0;
      for (; i + 3 < R; i += 4) {
        s0 = fmaf(a[int64_t(i) * Cc + j], xv[i], s0);
        s1 = fmaf(a[int64_t(i + 1) * Cc + j], xv[i + 1], s1);
        s2 = fmaf(a[int64_t(i + 2) * Cc + j], xv[i + 2], s2);
        s3 = fmaf(a[int64_t(i + 3) * Cc + j], xv[i + 3], s3);
      }
      for (; i < R; ++i) s0 = fmaf(a[int64_t(i) * Cc + j], xv[i], s0);
      const float sum = (s0 + s1) + (s2 + s3);
      float v = jb.alpha * sum;
      if (y0v) v = fmaf(jb.beta, y0v[j], v);
      if (zv) v += zv[j];
      yv[j] = v;
    }
  }
}

static inline void bgemv_jobs(cudaStream_t st, int batch, const GemvJob& j0, const GemvJob& j1) {
  if (batch <= 0) return;
  bgemv_jobs_kernel<<<dim3(batch, 2), 256, 0, st>>>(j0, j1);
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

// The same inverse with the matrix in registers, by blocks of 4 pivots (block
// Gauss-Jordan).  Tile thread t of ceil(n / 7) x ceil(n / 8) <= 725 holds rows
// 7g..7g+6 x columns 8h..8h+7 of row group g = t % G and column group h = t / G
// (G row groups); one more warp (the panel warp) holds no tile.  Rows are never
// exchanged: pivot k takes the unused row p_k with the largest |a_ik| (|value|
// compared by its bit pattern, a total order with NaN above infinity; smallest row
// on ties, as the row-exchanging form above).  Block b covers columns 4b..4b+3
// (half b % 2 of column group b / 2):
//   panel  the threads of that column group copy the 4 columns (all rows) into a
//          panel buffer; after a block barrier the panel warp alone loads the panel
//          into registers (lane l: rows l, l + 32, ...) and runs the 4 pivots
//          warp-synchronously (candidates and the pivot row by shuffles, no
//          barrier), which leaves in panel column s the column p_s of the block's
//          transform T (the product of the 4 elementary Gauss-Jordan steps);
//   bulk   after one block barrier every tile column x takes x + G x_P with
//          G = T[:, P] - I[:, P] from the panel buffer and x_P the block's pivot rows
//          as they were before the block, read from a shared-memory mirror of the
//          unused rows (a pivot row is never read again once used, so writing the
//          mirror back after the update races with no read of this block); the
//          panel's own columns then take the panel buffer's values.
// Letting the panel of block b + 1 start while the other warps finish block b (a
// named barrier among the panel's warps) gained nothing: the panel warp then shares
// its scheduler with them, and its pivot chain (about 3,000 cycles per pivot,
// dependent shuffles and selects) is the bound either way.  With B = P A (row k of
// B = row p_k of A) the
// storage ends as B^-1 with row r at p_r, so inv(A)[pinv[i]][p_j] = S[i][j]; the
// result is unpermuted through shared memory and written back row by row.
constexpr int kGjRB = 7, kGjCB = 8, kGjMax = 200;
constexpr int kGjTileWarps = 23, kGjPanelWarp = kGjTileWarps, kGjThreads = 32 * (kGjTileWarps + 1);
constexpr int kGjPW = 4, kGjPP = 5;        // panel width, panel row pitch (odd: no bank conflicts)
constexpr int kGjLR = (kGjMax + 31) / 32;  // panel rows per lane
static_assert(((kGjMax + kGjRB - 1) / kGjRB) * ((kGjMax + kGjCB - 1) / kGjCB) <= 32 * kGjTileWarps, "tiles");

inline int gj_pitch(int n) { return kGjCB * ((n + kGjCB - 1) / kGjCB) + 4; }

// SPD: symmetric positive definite input, pivots taken in order on the diagonal (no
// search; Gauss-Jordan without pivoting is stable for such matrices).
template <bool SPD = false>
static __global__ void __launch_bounds__(kGjThreads, 1) binv_reg_kernel(int n, BRef A, double* logdet,
                                                                        int64_t ld_mul, int64_t ld_add, int* status,
                                                                        int flag) {
  extern __shared__ __align__(16) float gj_mir[];  // n x pitch; the unpermuted result at the end
  __shared__ float pan[2][kGjMax * kGjPP];
  __shared__ int pid[2][kGjPW];
  __shared__ float pvs[kGjPW];
  __shared__ int perm[kGjMax], pinv[kGjMax];
  __shared__ unsigned char uflag[kGjMax];
  __shared__ double ld_acc;
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nrg = (n + kGjRB - 1) / kGjRB, ncg = (n + kGjCB - 1) / kGjCB, pitch = kGjCB * ncg + 4;
  const int nblk = (n + kGjPW - 1) / kGjPW;
  if (tid == 0) {
    ld_acc = 0.0;
    bad = 0;
  }
  for (int i = tid; i < n; i += blockDim.x) {
    pinv[i] = -1;
    uflag[i] = 0;
  }
  if (warp == kGjPanelWarp) {
    // ---------------------------------------------------------------- panel warp
    __syncthreads();  // initialisation and the first mirror
    for (int b = 0; b < nblk; ++b) {
      const int bp = b & 1;
      const int nv = n - kGjPW * b < kGjPW ? n - kGjPW * b : kGjPW;
      float* pb = pan[bp];
      __syncthreads();  // the panel's columns are in the buffer; the tile warps wait
      float pr[kGjLR][kGjPW];
      unsigned um = 0;  // bit m: row lane + 32 m used (or past n)
#pragma unroll
      for (int m = 0; m < kGjLR; ++m) {
        const int i = lane + 32 * m;
        const bool in = i < n;
        if (!in || uflag[i]) um |= 1u << m;
#pragma unroll
        for (int c = 0; c < kGjPW; ++c) pr[m][c] = in ? pb[i * kGjPP + c] : 0.f;
      }
#pragma unroll 1
      for (int s = 0; s < nv; ++s) {
        // column s of the lane's rows (selects: no register indexing by s)
        float col[kGjLR];
#pragma unroll
        for (int m = 0; m < kGjLR; ++m)
          col[m] = s == 0 ? pr[m][0] : (s == 1 ? pr[m][1] : (s == 2 ? pr[m][2] : pr[m][3]));
        // the lane's best unused row (key: |value|'s bit pattern; rows in ascending
        // order, so the first of equal keys wins), then two warp reductions: the
        // largest key, and the smallest row among the lanes that hold it
        unsigned rmin = unsigned(kGjPW * b + s);  // SPD: the diagonal, in order
        if (!SPD) {
          unsigned key = 0u, row = 0xffffffffu;
#pragma unroll
          for (int m = 0; m < kGjLR; ++m) {
            const unsigned kk = __float_as_uint(fabsf(col[m]));
            if (!((um >> m) & 1u) && (row == 0xffffffffu || kk > key)) key = kk, row = unsigned(lane + 32 * m);
          }
          const unsigned kmax = __reduce_max_sync(0xffffffffu, row != 0xffffffffu ? key : 0u);
          rmin = __reduce_min_sync(0xffffffffu, row != 0xffffffffu && key == kmax ? row : 0xffffffffu);
        }
        const int p = rmin < unsigned(n) ? int(rmin) : 0;  // an unused row is always offered
        const int lp = p & 31, mp = p >> 5;
        // the pivot row from the lane that holds it, then scaled
        float praw[kGjPW];
#pragma unroll
        for (int c = 0; c < kGjPW; ++c) {
          static_assert(kGjLR == 7, "a 3-level select tree over 7 row slots");
          // row slot mp (< 7) of this lane by a 3-level select tree on mp's bits
          const float t01 = (mp & 1) ? pr[1][c] : pr[0][c];
          const float t23 = (mp & 1) ? pr[3][c] : pr[2][c];
          const float t45 = (mp & 1) ? pr[5][c] : pr[4][c];
          const float t67 = pr[6][c];
          const float t03 = (mp & 2) ? t23 : t01, t47 = (mp & 2) ? t67 : t45;
          praw[c] = __shfl_sync(0xffffffffu, (mp & 4) ? t47 : t03, lp);
        }
        const float pv = rmin < unsigned(n) ? (s == 0 ? praw[0] : (s == 1 ? praw[1] : (s == 2 ? praw[2] : praw[3])))
                                            : 0.f;
        const float ip = __frcp_rn(pv);  // correctly rounded, as 1 / pv
        float prow[kGjPW];
#pragma unroll
        for (int c = 0; c < kGjPW; ++c) prow[c] = (c == s ? 1.f : praw[c]) * ip;
#pragma unroll
        for (int m = 0; m < kGjLR; ++m) {
          const bool piv = m == mp && lane == lp;
#pragma unroll
          for (int c = 0; c < kGjPW; ++c) pr[m][c] = piv ? prow[c] : fmaf(-col[m], prow[c], c == s ? 0.f : pr[m][c]);
        }
        if (lane == lp) um |= 1u << mp;
        if (lane == 0) {
          pid[bp][s] = p;
          pvs[s] = pv;
        }
      }
      // the block's bookkeeping, off the pivot chain
      __syncwarp();
      if (lane == 0) {
        for (int s = 0; s < nv; ++s) {
          const int p = pid[bp][s], k = kGjPW * b + s;
          const float pv = pvs[s];
          if (pinv[p] >= 0) bad = 1;  // a row taken twice (cannot happen); its output rows stay unwritten
          uflag[p] = 1;
          perm[k] = p;
          pinv[p] = k;
          if (logdet) ld_acc += double(logf(fabsf(pv)));
          if (!(fabsf(pv) > 0.f)) bad = 1;
        }
      }
#pragma unroll
      for (int m = 0; m < kGjLR; ++m) {
        const int i = lane + 32 * m;
        if (i < n) {
#pragma unroll
          for (int c = 0; c < kGjPW; ++c) pb[i * kGjPP + c] = pr[m][c];
        }
      }
      __syncthreads();  // the block's panel and pivots are published
    }
    __syncthreads();  // the unpermuted result
    __syncthreads();
  } else {
    // ---------------------------------------------------------------- tile threads
    const bool active = tid < nrg * ncg;
    const int cg = active ? tid / nrg : -1, rg = active ? tid % nrg : -1;
    const int r0 = (active ? rg : 0) * kGjRB, c0 = (active ? cg : 0) * kGjCB;
    float a[kGjRB][kGjCB];
    unsigned used = 0;  // bit r: row r0 + r is a pivot row already (or past n)
    {
      const float* g = A.at(blockIdx.x);
#pragma unroll
      for (int r = 0; r < kGjRB; ++r) {
        const int i = r0 + r;
        if (i >= n) used |= 1u << r;
#pragma unroll
        for (int c = 0; c < kGjCB; ++c) {
          const int j = c0 + c;
          a[r][c] = (active && i < n && j < n) ? g[int64_t(i) * n + j] : 0.f;
        }
      }
    }
    // the thread's unused rows -> mirror
#define BN_GJ_MIRROR()                                                                          \
  if (active) {                                                                                 \
    _Pragma("unroll") for (int r = 0; r < kGjRB; ++r) if (!((used >> r) & 1u)) {               \
      float* m = gj_mir + (r0 + r) * pitch + c0;                                                \
      *reinterpret_cast<float4*>(m) = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);          \
      *reinterpret_cast<float4*>(m + 4) = make_float4(a[r][4], a[r][5], a[r][6], a[r][7]);      \
    }                                                                                           \
  }
    BN_GJ_MIRROR();
    __syncthreads();  // initialisation and the first mirror
    for (int b = 0; b < nblk; ++b) {
      const int bp = b & 1, pc = b >> 1, half = b & 1;
      const int nv = n - kGjPW * b < kGjPW ? n - kGjPW * b : kGjPW;
      float* pb = pan[bp];
      if (cg == pc) {
#pragma unroll
        for (int r = 0; r < kGjRB; ++r)
          if (r0 + r < n) {
#pragma unroll
            for (int c = 0; c < kGjPW; ++c) pb[(r0 + r) * kGjPP + c] = half ? a[r][kGjPW + c] : a[r][c];
          }
      }
      __syncthreads();  // the panel's columns are in the buffer
      __syncthreads();  // the panel warp has published the block
#pragma unroll
      for (int s = 0; s < kGjPW; ++s) {
        const int q = s < nv ? pid[bp][s] : -1;
        if (q >= 0 && q / kGjRB == rg) used |= 1u << (q % kGjRB);
      }
      if (active) {
        for (int s = 0; s < nv; ++s) {
          const int q = pid[bp][s];
          const float* xp = gj_mir + q * pitch + c0;
          const float4 x0 = *reinterpret_cast<const float4*>(xp);
          const float4 x1 = *reinterpret_cast<const float4*>(xp + 4);
          const float xv[kGjCB] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
          for (int r = 0; r < kGjRB; ++r) {
            const int i = r0 + r;
            const float gv = (i < n ? pb[i * kGjPP + s] : 0.f) - (i == q ? 1.f : 0.f);
#pragma unroll
            for (int c = 0; c < kGjCB; ++c) a[r][c] = fmaf(gv, xv[c], a[r][c]);
          }
        }
        if (cg == pc) {
#pragma unroll
          for (int r = 0; r < kGjRB; ++r)
            if (r0 + r < n) {
#pragma unroll
              for (int c = 0; c < kGjPW; ++c) {
                const float v = pb[(r0 + r) * kGjPP + c];
                if (half) a[r][kGjPW + c] = v;
                else a[r][c] = v;
              }
            }
        }
      }
      BN_GJ_MIRROR();
    }
#undef BN_GJ_MIRROR
    __syncthreads();  // every tile has its last update; the mirror is free
    if (active) {
#pragma unroll
      for (int r = 0; r < kGjRB; ++r) {
        const int i = r0 + r;
        const int oi = i < n ? pinv[i] : -1;
        if (oi >= 0 && oi < n) {
#pragma unroll
          for (int c = 0; c < kGjCB; ++c) {
            const int j = c0 + c;
            const int oj = j < n ? perm[j] : -1;
            if (oj >= 0 && oj < n) gj_mir[oi * n + oj] = a[r][c];
          }
        }
      }
    }
    __syncthreads();
  }
  float* g = A.at(blockIdx.x);
  for (int e = tid; e < n * n; e += blockDim.x) g[e] = gj_mir[e];
  if (tid == 0) {
    if (logdet) logdet[ld_mul * blockIdx.x + ld_add] = ld_acc;
    if (bad && status) atomicOr(status, flag);
  }
}

static inline bool binv_reg_ok(int n) {
  if (n > kGjMax) return false;
  static const bool attr =
      cudaFuncSetAttribute(binv_reg_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kGjMax * gj_pitch(kGjMax) * int(sizeof(float))) == cudaSuccess &&
      cudaFuncSetAttribute(binv_reg_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kGjMax * gj_pitch(kGjMax) * int(sizeof(float))) == cudaSuccess;
  return attr;
}

// engine: 0 = shared-memory Gauss-Jordan (binv_kernel), 1 = register-resident
// (binv_reg_kernel, n <= 200), -1 = the register-resident one where it applies;
// spd: the register-resident kernel takes the diagonal pivots in order
static inline cudaError_t binv(cudaStream_t st, int batch, int n, BRef A, double* logdet, int64_t ld_mul,
                               int64_t ld_add, int* status, int flag, int engine = -1, bool spd = false) {
  if (batch <= 0) return cudaSuccess;
  if (engine != 0 && binv_reg_ok(n)) {
    const size_t sm = size_t(n) * gj_pitch(n) * sizeof(float);
    if (spd) binv_reg_kernel<true><<<batch, kGjThreads, sm, st>>>(n, A, logdet, ld_mul, ld_add, status, flag);
    else binv_reg_kernel<false><<<batch, kGjThreads, sm, st>>>(n, A, logdet, ld_mul, ld_add, status, flag);
  } else {
    if (engine == 1) return cudaErrorInvalidValue;
    binv_kernel<<<batch, kInvThreads, inv_smem(n), st>>>(n, A, logdet, ld_mul, ld_add, status, flag);
  }
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

// Triangular solves with a lower factor L (n x n): X = L^-1 B (forward) or, with
// trans_l, X = L^-T B (backward); B is n x nc (or nc x n read transposed when
// trans_b); X is n x nc (or written transposed, nc x n, when trans_x).  L sits in
// shared memory; each thread solves whole columns.  X must not alias B unless
// neither is transposed.
static __global__ void __launch_bounds__(256) btrsm_kernel(int n, int nc, BRef L, BRef B, BRef X, int trans_l, int trans_b,
                                                    int trans_x) {
  extern __shared__ __align__(16) unsigned char trsm_raw[];
  float* l = reinterpret_cast<float*>(trsm_raw);
  float* xs = l + n * n;  // this block's columns of X: xs[i * blockDim.x + thread]
  const int bi = blockIdx.x, tj = threadIdx.x, nb = blockDim.x;
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
        float s0 = bin(i), s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int k = 0;
        for (; k + 3 < i; k += 4) {
          s0 = fmaf(-l[i * n + k], xs[k * nb + tj], s0);
          s1 = fmaf(-l[i * n + k + 1], xs[(k + 1) * nb + tj], s1);
          s2 = fmaf(-l[i * n + k + 2], xs[(k + 2) * nb + tj], s2);
          s3 = fmaf(-l[i * n + k + 3], xs[(k + 3) * nb + tj], s3);
        }
        for (; k < i; ++k) s0 = fmaf(-l[i * n + k], xs[k * nb + tj], s0);
        const float v = ((s0 + s1) + (s2 + s3)) / l[i * n + i];
        xs[i * nb + tj] = v;
        xo(i) = v;
      }
    } else {
      for (int i = n - 1; i >= 0; --i) {
        float s0 = bin(i), s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int k = i + 1;
        for (; k + 3 < n; k += 4) {
          s0 = fmaf(-l[k * n + i], xs[k * nb + tj], s0);
          s1 = fmaf(-l[(k + 1) * n + i], xs[(k + 1) * nb + tj], s1);
          s2 = fmaf(-l[(k + 2) * n + i], xs[(k + 2) * nb + tj], s2);
          s3 = fmaf(-l[(k + 3) * n + i], xs[(k + 3) * nb + tj], s3);
        }
        for (; k < n; ++k) s0 = fmaf(-l[k * n + i], xs[k * nb + tj], s0);
        const float v = ((s0 + s1) + (s2 + s3)) / l[i * n + i];
        xs[i * nb + tj] = v;
        xo(i) = v;
      }
    }
  }
}

// block width for nc right-hand sides, and the shared memory it takes (L, then the
// block's columns of X)
inline int btrsm_threads(int nc) { return nc >= 128 ? 128 : (nc + 31) / 32 * 32; }
inline size_t btrsm_smem(int n, int nc) { return (size_t(n) * n + size_t(n) * btrsm_threads(nc)) * sizeof(float); }

inline void btrsm(cudaStream_t st, int batch, int n, int nc, BRef L, BRef B, BRef X, bool trans_l, bool trans_b,
                  bool trans_x) {
  if (batch <= 0) return;
  const int nt = btrsm_threads(nc);
  dim3 grid(batch, (nc + nt - 1) / nt);
  btrsm_kernel<<<grid, nt, btrsm_smem(n, nc), st>>>(n, nc, L, B, X, trans_l ? 1 : 0, trans_b ? 1 : 0,
                                                    trans_x ? 1 : 0);
}

// ---------------------------------------------------------------- copies
static __global__ void bcopy_kernel(int64_t len, BRef src, BRef dst) {
  const float* s = src.at(blockIdx.y);
  float* d = dst.at(blockIdx.y);
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < len; e += int64_t(gridDim.x) * blockDim.x)
    d[e] = s[e];
}
// Up to kCopyJobs batched copies (job z: dst_z.at(i)[e] = src_z.at(i)[e], e < len_z)
// in one launch; 16-byte moves when every length and address allows.
constexpr int kCopyJobs = 5;
struct CopyJobs {
  int64_t len[kCopyJobs];
  BRef src[kCopyJobs], dst[kCopyJobs];
};

template <bool V4>
static __global__ void bcopy_jobs_kernel(CopyJobs js) {
  const int z = blockIdx.z;
  const float* s = js.src[z].at(blockIdx.y);
  float* d = js.dst[z].at(blockIdx.y);
  const int64_t len = js.len[z];
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  if (V4) {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < len / 4; e += stride)
      reinterpret_cast<float4*>(d)[e] = reinterpret_cast<const float4*>(s)[e];
  } else {
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < len; e += stride) d[e] = s[e];
  }
}

static inline void bcopy_jobs(cudaStream_t st, int batch, int njobs, const CopyJobs& js) {
  if (batch <= 0 || njobs <= 0) return;
  int64_t mx = 0;
  bool v4 = true;
  for (int z = 0; z < njobs; ++z) {
    mx = js.len[z] > mx ? js.len[z] : mx;
    const auto al = [](const BRef& r) {
      return (reinterpret_cast<uintptr_t>(r.p) % 16 == 0) && (r.stride % 4 == 0);
    };
    v4 = v4 && js.len[z] % 4 == 0 && al(js.src[z]) && al(js.dst[z]);
  }
  int gx = int(((v4 ? mx / 4 : mx) + 255) / 256);
  gx = gx < 1 ? 1 : (gx > 64 ? 64 : gx);
  if (v4) bcopy_jobs_kernel<true><<<dim3(gx, batch, njobs), 256, 0, st>>>(js);
  else bcopy_jobs_kernel<false><<<dim3(gx, batch, njobs), 256, 0, st>>>(js);
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
