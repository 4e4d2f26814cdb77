// Scans of the block aggregates (F2 / S2) spread over one thread-block cluster,
// one warp per element.
//
// F1 leaves one filter element per block of chunks (a few hundred at N = 1e6); the
// filtered state entering each block is the stationary prior combined with the
// exclusive prefix of those aggregates (ops.py:203-219 restated with
// W = (I + C1 J2)^-1).  A scan of n elements takes log2(n) dependent combines, so
// what matters is the latency of one combine: here each combine is one warp's
// work, its lanes spread over the entries of the D x D products (operands in
// shared memory, read as broadcasts along rows and coalesced along columns), and
// the Kogge-Stone levels run over CL CTAs of one cluster that read each other's
// elements through distributed shared memory, with a cluster barrier between
// levels.  S2 is the same for the smoother elements (E, g, L) in reverse order
// (ops.py:328-335).
//
// Every thread executes the same sequence of cluster barriers (no early exit),
// and the last barrier keeps every CTA's shared memory alive until no other CTA
// reads it.
#pragma once
#include "bn_scan.cuh"

namespace bn {

// ------------------------------------------------------------ cluster primitives
__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  __syncwarp();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// value at the same shared-memory offset as `p` in CTA `rank` of the cluster
__device__ __forceinline__ float cl_load(const float* p, unsigned rank) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
  unsigned ra;
  asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  float v;
  asm("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(ra));
  return v;
}
__device__ __forceinline__ double cl_load(const double* p, unsigned rank) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(p));
  unsigned ra;
  asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  double v;
  asm("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra));
  return v;
}

// ------------------------------------------------------------ warp algebra
// D x D row-major matrices and D-vectors in shared memory; lane l owns entries
// l, l + 32, ...  Every routine ends with __syncwarp() so its result is visible
// to the whole warp.
template <typename T, int D>
struct WarpOps {
  static constexpr int DD = D * D;
  // O = X Y
  static __device__ __forceinline__ void mm(T* O, const T* X, const T* Y, int lane) {
    for (int e = lane; e < DD; e += 32) {
      const int i = e / D, j = e - (e / D) * D;
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[i * D + k], Y[k * D + j], s);
      O[e] = s;
    }
    __syncwarp();
  }
  // O = X^T Y
  static __device__ __forceinline__ void mtm(T* O, const T* X, const T* Y, int lane) {
    for (int e = lane; e < DD; e += 32) {
      const int i = e / D, j = e - (e / D) * D;
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[k * D + i], Y[k * D + j], s);
      O[e] = s;
    }
    __syncwarp();
  }
  // O = X Y^T + Z, symmetric (entry (i, j) computed as (min, max): exactly mirrored)
  static __device__ __forceinline__ void mmt_sym_add(T* O, const T* X, const T* Y, const T* Z, int lane) {
    for (int e = lane; e < DD; e += 32) {
      int i = e / D, j = e - (e / D) * D;
      if (i > j) {
        const int t = i;
        i = j;
        j = t;
      }
      T s = Z[i * D + j];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[i * D + k], Y[j * D + k], s);
      O[e] = s;
    }
    __syncwarp();
  }
  // O = X^T Y + Z, symmetric
  static __device__ __forceinline__ void mtm_sym_add(T* O, const T* X, const T* Y, const T* Z, int lane) {
    for (int e = lane; e < DD; e += 32) {
      int i = e / D, j = e - (e / D) * D;
      if (i > j) {
        const int t = i;
        i = j;
        j = t;
      }
      T s = Z[i * D + j];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[k * D + i], Y[k * D + j], s);
      O[e] = s;
    }
    __syncwarp();
  }
  // o = X v + a
  static __device__ __forceinline__ void mv_add(T* o, const T* X, const T* v, const T* a, int lane) {
    if (lane < D) {
      T s = a[lane];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[lane * D + k], v[k], s);
      o[lane] = s;
    }
    __syncwarp();
  }
  // o = X^T v + a
  static __device__ __forceinline__ void mtv_add(T* o, const T* X, const T* v, const T* a, int lane) {
    if (lane < D) {
      T s = a[lane];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(X[k * D + lane], v[k], s);
      o[lane] = s;
    }
    __syncwarp();
  }
  // o = a - X v
  static __device__ __forceinline__ void sub_mv(T* o, const T* a, const T* X, const T* v, int lane) {
    if (lane < D) {
      T s = a[lane];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(-X[lane * D + k], v[k], s);
      o[lane] = s;
    }
    __syncwarp();
  }
  // W = M^-1 by Gauss-Jordan elimination with partial pivoting (M overwritten).
  // Returns false (on every lane) when a pivot is exactly zero.
  static __device__ __forceinline__ bool inverse(T* M, T* W, int lane) {
    for (int e = lane; e < DD; e += 32) W[e] = (e / D == e - (e / D) * D) ? T(1) : T(0);
    __syncwarp();
    bool ok = true;
    for (int k = 0; k < D; ++k) {
      // pivot row: the largest |M[r][k]|, r >= k
      int p = k;
      if (lane == 0) {
        T best = bn_abs(M[k * D + k]);
        for (int r = k + 1; r < D; ++r) {
          const T v = bn_abs(M[r * D + k]);
          if (v > best) {
            best = v;
            p = r;
          }
        }
      }
      p = __shfl_sync(0xffffffffu, p, 0);
      if (p != k) {
        if (lane < D) {
          const T a = M[k * D + lane], b = M[p * D + lane];
          M[k * D + lane] = b;
          M[p * D + lane] = a;
        } else if (lane < 2 * D) {
          const int c = lane - D;
          const T a = W[k * D + c], b = W[p * D + c];
          W[k * D + c] = b;
          W[p * D + c] = a;
        }
        __syncwarp();
      }
      const T piv = M[k * D + k];
      ok = ok && (piv != T(0));
      const T ip = T(1) / piv;
      // read phase: new values of every entry of M and W, then write
      T nv[(2 * DD + 31) / 32];
      int q = 0;
      for (int e = lane; e < 2 * DD; e += 32, ++q) {
        const bool isw = e >= DD;
        const int f = isw ? e - DD : e;
        const int r = f / D, c = f - (f / D) * D;
        const T* S = isw ? W : M;
        const T rk = S[k * D + c] * ip;  // normalised pivot row
        nv[q] = (r == k) ? rk : fma(-M[r * D + k], rk, S[f]);
      }
      __syncwarp();
      q = 0;
      for (int e = lane; e < 2 * DD; e += 32, ++q) {
        if (e >= DD) W[e - DD] = nv[q];
        else M[e] = nv[q];
      }
      __syncwarp();
    }
    return ok;
  }
};

// The same algebra with the matrices in registers, for D * D <= 32: lane l holds
// entry (l / D, l % D) of each D x D matrix and entry l (< D) of each vector,
// and the operands of a product come from the other lanes by shuffles, so a
// combine needs no shared-memory round trip or warp barrier between its steps.
template <typename T, int D>
struct RegOps {
  static __device__ __forceinline__ T sh(T v, int src) { return __shfl_sync(0xffffffffu, v, src); }
  // (X Y)[i][j]
  static __device__ __forceinline__ T mm(T x, T y, int i, int j) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(sh(x, i * D + k), sh(y, k * D + j), s);
    return s;
  }
  // (X Y^T)[a][b] + Z[a][b] and (X^T Y)[a][b] + Z[a][b] at (a, b) = (min, max)(i, j):
  // both mirror entries from the same arithmetic
  static __device__ __forceinline__ T mmt_sym_add(T x, T y, T z, int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    T s = sh(z, a * D + b);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(sh(x, a * D + k), sh(y, b * D + k), s);
    return s;
  }
  static __device__ __forceinline__ T mtm_sym_add(T x, T y, T z, int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    T s = sh(z, a * D + b);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(sh(x, k * D + a), sh(y, k * D + b), s);
    return s;
  }
  // (X v)[l] and (X^T v)[l] for lanes l < D
  static __device__ __forceinline__ T mv(T x, T v, int lane) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(sh(x, lane * D + k), sh(v, k), s);
    return s;
  }
  static __device__ __forceinline__ T mtv(T x, T v, int lane) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(sh(x, k * D + lane), sh(v, k), s);
    return s;
  }
  // W = M^-1 by Gauss-Jordan elimination with partial pivoting; the pivot row
  // is the largest |M[r][k]| (r >= k, ties to the lower row) by one warp max
  // reduction.  Returns false when a pivot is exactly zero.
  static __device__ __forceinline__ bool inverse(T& m, T& w, int lane, int i, int j) {
    w = (i == j && lane < D * D) ? T(1) : T(0);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const T cv = sh(m, lane * D + k);  // M[lane][k] on lanes < D
      unsigned key = 0u;
      if (lane >= k && lane < D) key = (__float_as_uint(float(bn_abs(cv))) & ~7u) | unsigned(7 - lane);
      const int p = 7 - int(__reduce_max_sync(0xffffffffu, key) & 7u);
      const int src = (i == k) ? p * D + j : ((i == p) ? k * D + j : lane);
      m = sh(m, src);
      w = sh(w, src);
      const T piv = sh(m, k * D + k);
      ok = ok && (piv != T(0));
      const T ip = T(1) / piv;
      const T mkj = sh(m, k * D + j) * ip, wkj = sh(w, k * D + j) * ip, mik = sh(m, i * D + k);
      if (i == k) {
        m = mkj;
        w = wkj;
      } else {
        m = fma(-mik, mkj, m);
        w = fma(-mik, wkj, w);
      }
    }
    return ok;
  }
};

template <typename T, int D>
__device__ __forceinline__ bool warp_fcombine_reg(const FElem<T, D>& e1, const FElem<T, D>& e2, FElem<T, D>& r,
                                                  int lane) {
  using R = RegOps<T, D>;
  constexpr int DD = D * D;
  const int i = lane / D, j = lane - (lane / D) * D;
  const bool in = lane < DD, vl = lane < D;
  const int le = in ? lane : 0, lv = vl ? lane : 0;
  const T a1 = (&e1.A[0][0])[le], c1 = (&e1.C[0][0])[le], j1 = (&e1.J[0][0])[le];
  const T a2 = (&e2.A[0][0])[le], c2 = (&e2.C[0][0])[le], j2 = (&e2.J[0][0])[le];
  const T b1 = e1.b[lv], eta1 = e1.eta[lv], b2 = e2.b[lv], eta2 = e2.eta[lv];
  T m = R::mm(c1, j2, i, j) + ((i == j) ? T(1) : T(0));  // I + C1 J2
  T w;
  const bool ok = R::inverse(m, w, lane, i, j);
  const T x = R::mm(a2, w, i, j);                        // A2 W
  const T t = R::mv(c1, eta2, lane) + b1;                // C1 eta2 + b1
  const T rb = R::mv(x, t, lane) + b2;                   // A2 W (b1 + C1 eta2) + b2
  const T y = R::mm(x, c1, i, j);                        // A2 W C1
  const T rc = R::mmt_sym_add(y, a2, c2, i, j);          // + C2
  const T ra = R::mm(x, a1, i, j);                       // A2 W A1
  const T x2 = R::mm(w, a1, i, j);                       // W A1
  const T u = eta2 - R::mv(j2, b1, lane);                // eta2 - J2 b1
  const T reta = R::mtv(x2, u, lane) + eta1;             // (W A1)^T u + eta1
  const T y2 = R::mm(j2, a1, i, j);                      // J2 A1
  const T rj = R::mtm_sym_add(x2, y2, j1, i, j);         // (W A1)^T J2 A1 + J1
  if (in) {
    (&r.A[0][0])[lane] = ra;
    (&r.C[0][0])[lane] = rc;
    (&r.J[0][0])[lane] = rj;
  }
  if (vl) {
    r.b[lane] = rb;
    r.eta[lane] = reta;
  }
  __syncwarp();
  return ok;
}

template <typename T, int D>
__device__ __forceinline__ void warp_scompose_reg(const SElem<T, D>& e, const SElem<T, D>& l, SElem<T, D>& r,
                                                  int lane) {
  using R = RegOps<T, D>;
  constexpr int DD = D * D;
  const int i = lane / D, j = lane - (lane / D) * D;
  const bool in = lane < DD, vl = lane < D;
  const int le = in ? lane : 0, lv = vl ? lane : 0;
  const T E = (&e.E[0][0])[le], Le = (&e.L[0][0])[le], El = (&l.E[0][0])[le], Ll = (&l.L[0][0])[le];
  const T ge = e.g[lv], gl = l.g[lv];
  const T rg = R::mv(E, gl, lane) + ge;
  const T y = R::mm(E, Ll, i, j);
  const T rl = R::mmt_sym_add(y, E, Le, i, j);
  const T re = R::mm(E, El, i, j);
  if (in) {
    (&r.E[0][0])[lane] = re;
    (&r.L[0][0])[lane] = rl;
  }
  if (vl) r.g[lane] = rg;
  __syncwarp();
}

// Scratch of one warp's combine: four D x D matrices and two vectors.
template <typename T, int D>
struct WarpScratch {
  T M[D * D], W[D * D], X[D * D], Y[D * D];
  T t[D], u[D];
};

// r = e1 (earlier) (+) e2 (later), the algebra of fcombine (bn_small.cuh) on one
// warp.  r may alias neither input.
template <typename T, int D>
__device__ __forceinline__ bool warp_fcombine(const FElem<T, D>& e1, const FElem<T, D>& e2, FElem<T, D>& r,
                                              WarpScratch<T, D>& s, int lane) {
  if constexpr (D * D <= 32) return warp_fcombine_reg(e1, e2, r, lane);
  using O = WarpOps<T, D>;
  const T* A1 = &e1.A[0][0];
  const T* C1 = &e1.C[0][0];
  const T* J1 = &e1.J[0][0];
  const T* A2 = &e2.A[0][0];
  const T* C2 = &e2.C[0][0];
  const T* J2 = &e2.J[0][0];
  O::mm(s.M, C1, J2, lane);
  if (lane < D) s.M[lane * D + lane] += T(1);
  __syncwarp();
  const bool ok = O::inverse(s.M, s.W, lane);
  O::mm(s.X, A2, s.W, lane);                          // A2 W
  O::mv_add(s.t, C1, e2.eta, e1.b, lane);             // C1 eta2 + b1
  O::mv_add(r.b, s.X, s.t, e2.b, lane);               // A2 W (b1 + C1 eta2) + b2
  O::mm(s.Y, s.X, C1, lane);                          // A2 W C1
  O::mmt_sym_add(&r.C[0][0], s.Y, A2, C2, lane);      // + C2
  O::mm(&r.A[0][0], s.X, A1, lane);                   // A2 W A1
  O::mm(s.X, s.W, A1, lane);                          // W A1
  O::sub_mv(s.u, e2.eta, J2, e1.b, lane);             // eta2 - J2 b1
  O::mtv_add(r.eta, s.X, s.u, e1.eta, lane);          // (W A1)^T u + eta1
  O::mm(s.Y, J2, A1, lane);                           // J2 A1
  O::mtm_sym_add(&r.J[0][0], s.X, s.Y, J1, lane);     // (W A1)^T J2 A1 + J1
  return ok;
}

// r = e (earlier) o l (later) for smoother elements (scompose on one warp).
template <typename T, int D>
__device__ __forceinline__ void warp_scompose(const SElem<T, D>& e, const SElem<T, D>& l, SElem<T, D>& r,
                                              WarpScratch<T, D>& s, int lane) {
  if constexpr (D * D <= 32) {
    warp_scompose_reg(e, l, r, lane);
    return;
  }
  using O = WarpOps<T, D>;
  const T* E = &e.E[0][0];
  O::mv_add(r.g, E, l.g, e.g, lane);
  O::mm(s.Y, E, &l.L[0][0], lane);
  O::mmt_sym_add(&r.L[0][0], s.Y, E, &e.L[0][0], lane);
  O::mm(&r.E[0][0], E, &l.E[0][0], lane);
}

// copy an element between shared-memory slots of one warp
template <typename T, typename E>
__device__ __forceinline__ void warp_copy(E& dst, const E& src, int lane) {
  constexpr int n = sizeof(E) / sizeof(T);
  T* d = reinterpret_cast<T*>(&dst);
  const T* s = reinterpret_cast<const T*>(&src);
  for (int f = lane; f < n; f += 32) d[f] = s[f];
  __syncwarp();
}
// copy an element from the same slot layout in another CTA of the cluster
// (all of a lane's remote loads are issued before any is stored: the loads are
// ordered against other CTAs' writes by the cluster barriers around them)
template <typename T, typename E>
__device__ __forceinline__ void warp_copy_remote(E& dst, const E& src, unsigned rank, int lane) {
  constexpr int n = sizeof(E) / sizeof(T);
  constexpr int q = (n + 31) / 32;
  T* d = reinterpret_cast<T*>(&dst);
  const T* s = reinterpret_cast<const T*>(&src);
  T v[q];
#pragma unroll
  for (int r = 0; r < q; ++r) {
    const int f = lane + 32 * r;
    v[r] = f < n ? cl_load(s + f, rank) : T(0);
  }
#pragma unroll
  for (int r = 0; r < q; ++r) {
    const int f = lane + 32 * r;
    if (f < n) d[f] = v[r];
  }
  __syncwarp();
}
template <typename T, typename E>
__device__ __forceinline__ void warp_load_global(E& dst, const T* src, int lane) {
  constexpr int n = sizeof(E) / sizeof(T);
  T* d = reinterpret_cast<T*>(&dst);
  for (int f = lane; f < n; f += 32) d[f] = __ldcg(src + f);
  __syncwarp();
}
template <typename T, typename E>
__device__ __forceinline__ void warp_store_global(T* dst, const E& src, int lane) {
  constexpr int n = sizeof(E) / sizeof(T);
  const T* s = reinterpret_cast<const T*>(&src);
  for (int f = lane; f < n; f += 32) dst[f] = s[f];
}
// Shared memory of one warp of the cluster scans: its element in two buffers
// (level l reads buf[l % 2] of other warps and writes buf[(l + 1) % 2] of its
// own, so one cluster barrier per level orders every read before the write that
// replaces it), a copy of the partner's element and scratch.
template <typename T, typename E, int D>
struct WarpSlot {
  E buf[2], other;
  WarpScratch<T, D> s;
};

// ============================================================ F2 on a cluster
// CL CTAs x WPC warps; warp w (cluster-wide index) owns aggregates
// [w per, (w + 1) per), per = ceil(nblocks / (CL WPC)), and the scan runs over
// the NA = ceil(nblocks / per) warps that own some.  Writes the filtered state
// entering every aggregate (fin) and, for a time segment, the total element.
template <typename T, typename L, int P, int WPC>
__global__ void __launch_bounds__(WPC * 32, 1) filter_blocks_cluster_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  using E = FElem<T, D>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSlot<T, E, D>* slots = reinterpret_cast<WarpSlot<T, E, D>*>(smem_raw);
  const int lane = threadIdx.x & 31;
  const int wl = threadIdx.x >> 5;
  const unsigned rank = cl_rank();
  const int TW = int(gridDim.x) * WPC;  // the grid is one cluster
  const int w = int(rank) * WPC + wl;
  WarpSlot<T, E, D>& S = slots[wl];
  const int nb = a.nblocks;
  const int per = (nb + TW - 1) / TW;
  const int NA = (nb + per - 1) / per;
  const int j0 = w * per;
  const int j1 = j0 + per < nb ? j0 + per : nb;
  bool ok = true;
  // fold this warp's aggregates into buf[0]
  if (w < NA) {
    warp_load_global<T>(S.buf[0], a.fagg + (size_t)j0 * Sz<T, D>::FE, lane);
    for (int j = j0 + 1; j < j1; ++j) {
      warp_load_global<T>(S.other, a.fagg + (size_t)j * Sz<T, D>::FE, lane);
      ok = warp_fcombine(S.buf[0], S.other, S.buf[1], S.s, lane) && ok;
      warp_copy<T>(S.buf[0], S.buf[1], lane);
    }
  }
  cl_sync();
  // Kogge-Stone over the NA warp elements: x(w) <- x(w - off) (+) x(w)
  int cur = 0;
  for (int off = 1; off < NA; off <<= 1) {
    if (w < NA) {
      if (w >= off) {
        const int src = w - off;
        warp_copy_remote<T>(S.other, slots[src % WPC].buf[cur], unsigned(src / WPC), lane);
        ok = warp_fcombine(S.other, S.buf[cur], S.buf[cur ^ 1], S.s, lane) && ok;
      } else {
        warp_copy<T>(S.buf[cur ^ 1], S.buf[cur], lane);
      }
    }
    cur ^= 1;
    cl_sync();
  }
  if (a.seg_total_f && w == NA - 1) warp_store_global<T>(a.seg_total_f, S.buf[cur], lane);
  // state entering aggregate j0: the stationary prior (or the state handed over
  // by the previous time segment), then the exclusive prefix (inclusive of w - 1)
  if (w < NA && w > 0) warp_copy_remote<T>(S.other, slots[(w - 1) % WPC].buf[cur], unsigned((w - 1) / WPC), lane);
  cl_sync();  // the last reads of other CTAs' shared memory
  if (w < NA) {
    // the state as an element with A = 0, J = 0, eta = 0, b = m, C = P: a state
    // followed by an element is then the element combine (its b and C)
    E* st = &S.buf[cur ^ 1];
    E* nx = &S.buf[cur];
    {
      T* p = reinterpret_cast<T*>(st);
      for (int f = lane; f < int(sizeof(E) / sizeof(T)); f += 32) p[f] = T(0);
      __syncwarp();
      if (lane < D) st->b[lane] = a.seg_left ? a.seg_left[lane] : T(0);
      for (int f = lane; f < D * D; f += 32)
        (&st->C[0][0])[f] = a.seg_left ? a.seg_left[D + f] : (&a.ssm.Pinf[0][0])[f];
      __syncwarp();
    }
    if (w > 0) {
      ok = warp_fcombine(*st, S.other, *nx, S.s, lane) && ok;
      E* t = st;
      st = nx;
      nx = t;
    }
    for (int j = j0; j < j1; ++j) {
      T* dst = a.fin + (size_t)j * Sz<T, D>::ST;  // State: m [D], P [D][D]
      if (lane < D) dst[lane] = st->b[lane];
      for (int f = lane; f < D * D; f += 32) dst[D + f] = (&st->C[0][0])[f];
      if (j + 1 < j1) {
        warp_load_global<T>(S.other, a.fagg + (size_t)j * Sz<T, D>::FE, lane);
        ok = warp_fcombine(*st, S.other, *nx, S.s, lane) && ok;
        E* t = st;
        st = nx;
        nx = t;
      }
    }
  }
  if (!ok && lane == 0) atomicOr(a.status, BN_STATUS_SINGULAR);
}

// ============================================================ S2 on a cluster
// Reverse scan of the smoother aggregates; writes the smoothed state after every
// aggregate (sin) and, for a time segment, the total element.
template <typename T, typename L, int P, int WPC>
__global__ void __launch_bounds__(WPC * 32, 1) smoother_blocks_cluster_kernel(ScanArgs<T, L::D, P> a) {
  constexpr int D = L::D;
  using E = SElem<T, D>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSlot<T, E, D>* slots = reinterpret_cast<WarpSlot<T, E, D>*>(smem_raw);
  const int lane = threadIdx.x & 31;
  const int wl = threadIdx.x >> 5;
  const unsigned rank = cl_rank();
  const int TW = int(gridDim.x) * WPC;
  const int w = int(rank) * WPC + wl;
  WarpSlot<T, E, D>& S = slots[wl];
  const int nb = a.nblocks;
  const int per = (nb + TW - 1) / TW;
  const int NA = (nb + per - 1) / per;
  const int j0 = w * per;
  const int j1 = j0 + per < nb ? j0 + per : nb;
  if (w < NA) {
    warp_load_global<T>(S.buf[0], a.sagg + (size_t)(j1 - 1) * Sz<T, D>::SE, lane);
    for (int j = j1 - 2; j >= j0; --j) {
      warp_load_global<T>(S.other, a.sagg + (size_t)j * Sz<T, D>::SE, lane);
      warp_scompose(S.other, S.buf[0], S.buf[1], S.s, lane);
      warp_copy<T>(S.buf[0], S.buf[1], lane);
    }
  }
  cl_sync();
  // reverse Kogge-Stone: x(w) <- x(w) o x(w + off)
  int cur = 0;
  for (int off = 1; off < NA; off <<= 1) {
    if (w < NA) {
      if (w + off < NA) {
        const int src = w + off;
        warp_copy_remote<T>(S.other, slots[src % WPC].buf[cur], unsigned(src / WPC), lane);
        warp_scompose(S.buf[cur], S.other, S.buf[cur ^ 1], S.s, lane);
      } else {
        warp_copy<T>(S.buf[cur ^ 1], S.buf[cur], lane);
      }
    }
    cur ^= 1;
    cl_sync();
  }
  if (a.seg_total_s && w == 0) warp_store_global<T>(a.seg_total_s, S.buf[cur], lane);
  if (w + 1 < NA) warp_copy_remote<T>(S.other, slots[(w + 1) % WPC].buf[cur], unsigned((w + 1) / WPC), lane);
  cl_sync();
  if (w < NA) {
    // smoothed state after the last aggregate of this warp: the next time
    // segment's first smoothed state, else zero (the series' last element has
    // E = 0), held as an element with E = 0, g = m, L = P so that an aggregate
    // applied to it is the element composition (its g and L)
    E* st = &S.buf[cur ^ 1];
    E* nx = &S.buf[cur];
    {
      T* p = reinterpret_cast<T*>(st);
      for (int f = lane; f < int(sizeof(E) / sizeof(T)); f += 32) p[f] = T(0);
      __syncwarp();
      if (a.seg_right) {
        if (lane < D) st->g[lane] = a.seg_right[lane];
        for (int f = lane; f < D * D; f += 32) (&st->L[0][0])[f] = a.seg_right[D + f];
      }
      __syncwarp();
    }
    if (w + 1 < NA) {
      warp_scompose(S.other, *st, *nx, S.s, lane);
      E* t = st;
      st = nx;
      nx = t;
    }
    for (int j = j1 - 1; j >= j0; --j) {
      T* dst = a.sin + (size_t)j * Sz<T, D>::ST;
      if (lane < D) dst[lane] = st->g[lane];
      for (int f = lane; f < D * D; f += 32) dst[D + f] = (&st->L[0][0])[f];
      if (j > j0) {
        warp_load_global<T>(S.other, a.sagg + (size_t)j * Sz<T, D>::SE, lane);
        warp_scompose(S.other, *st, *nx, S.s, lane);
        E* t = st;
        st = nx;
        nx = t;
      }
    }
  }
}

}  // namespace bn
