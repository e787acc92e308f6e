// band_lu.cu -- banded LU with partial pivoting and the banded triangular
// solves: the replacement of `Δu = -K_gl \ r_gl` (src/analysis/FiniteElement.jl:38).
//
// The reference hands the sparse tangent to UMFPACK.  Here K stays in the
// reference's lexicographic (node-major) unknown ordering, where it is banded
// with half bandwidth b ≈ (2 num1np + 2) ndf, and is factored as a band matrix
// (the algorithm of LAPACK's gbtrf: partial pivoting inside the kl
// sub-diagonals, U widened to kl + ku by the row interchanges).
//
// Blocking: panels of nb columns.  For panel [j0, j1) with rows [j0, j0+R),
// R = (j1 - j0) + kl:
//   panel_cluster_kernel  a 16-CTA thread-block cluster, panel rows spread
//                         over the CTAs' shared memory: pivot search (cluster
//                         argmax, first maximum like idamax), interchanges as
//                         row relabelling, scaling, rank-1 updates; records
//                         ipiv and the panel's row permutation.
//   panel_apply_kernel    one warp per trailing column c in [j1, j1+kl+ku):
//                         permute rows [j0, j0+R) of column c, solve with the
//                         unit lower L11, subtract L21 · U12(:, c).  The
//                         right-hand side rides along as one extra column, so
//                         the forward substitution costs no extra pass.
// Band layout (BandLayout): column-major with ldb rows per column and nb rows
// of padding on both sides of the LAPACK band, so every block above is a
// plain strided rectangle; the bottom padding holds the panel-local L fill
// (LAPACK keeps it in a separate WORK31 array).

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mafem_internal.h"

namespace mafem {

__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

BandLayout make_band_layout(int64_t n, int kl, int ku, int nb) {
  BandLayout L;
  L.n = n;
  L.kl = kl;
  L.ku = ku;
  L.nb = nb;
  L.off = (int64_t)kl + ku + nb;
  int64_t rows = 2 * (int64_t)kl + ku + 2 * nb + 1;
  L.ldb = (rows + 3) / 4 * 4;  // 32-byte aligned columns (FP64) / 16-byte (FP32)
  return L;
}

__device__ __forceinline__ int64_t bidx(const BandLayout& L, int64_t i, int64_t j) {
  return j * L.ldb + L.off + i - j;
}

template <class T>
__device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// ---------------------------------------------------------------------------
// Panel factorisation on a thread-block cluster of CS CTAs.  CTA c holds the
// panel rows [c*RC, min(R, (c+1)*RC)) in shared memory (column-major); four
// threads share each row (thread t: row t/4, part t%4), so the FP64 rank-1
// updates are spread over CS SMs and all four sub-partitions of each.  Rows
// never move: every thread keeps the logical row index of its data (row
// interchanges swap labels), so a pivot step moves no data and the panel's
// permutation falls out at the end as perm[logical] = physical.
//
// GB300 issues FP64 instructions at a small fraction of the FP32 rate, so the
// per-column critical path avoids them: the pivot search compares integer keys
// (the bit pattern of |v| orders non-negative doubles), and the reciprocal of
// each CTA's candidate pivot is computed once, before the cluster barrier, and
// travels with the candidate.
// Per column jj (one __syncthreads, one cluster barrier):
//   1. rows with logical index in [jj, jj+kl] offer |A(., jj)|; the CTA argmax
//      keeps ties at the smaller logical row (LAPACK's idamax rule);
//   2. every CTA pushes, with remote stores into each peer's inbox, its
//      candidate (key, 1/value, logical row, physical row) and candidate row;
//   3. cluster barrier (release/acquire): all inboxes complete and visible;
//   4. every thread picks the same global winner from its local inbox,
//      relabels (winner -> jj, old jj -> winner's label), and rows with logical
//      index in (jj, jj+kl] are scaled and rank-1 updated with the winner's row.
// Inboxes are double-buffered by column parity: a CTA reads inbox[jj&1] before
// it arrives at the barrier of column jj+1, and peers write inbox[jj&1] again
// only for column jj+2, after that barrier.
__device__ __forceinline__ unsigned long long abs_key(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
  return b >= 0x7ff0000000000000ULL ? 0ULL : b;  // NaN, ±Inf -> 0 (never a valid pivot)
}
__device__ __forceinline__ unsigned long long abs_key(float v) {
  unsigned b = (unsigned)__float_as_int(v) & 0x7fffffffu;
  return b >= 0x7f800000u ? 0ULL : (unsigned long long)b;
}
// 1/x for the pivot: FP32 seed + two Newton steps (no FP64 divide sequence).
__device__ __forceinline__ double fast_rcp(double x) {
  const float xf = (float)x;
  const float sf = __frcp_rn(xf);
  if (xf == 0.0f || !isfinite(sf) || sf == 0.0f) return 1.0 / x;  // outside FP32 range
  double r = (double)sf;
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}
__device__ __forceinline__ float fast_rcp(float x) { return __frcp_rn(x); }

template <class T>
struct PanelInbox {
  unsigned long long key[16];  // candidate |value| key from each CTA (0 = none)
  T rinv[16];                  // 1 / candidate value
  int lidx[16];                // its logical row
  int pidx[16];                // its physical row
  T cand[16][32];              // candidate rows
};

template <class T, int CS>
__global__ void __launch_bounds__(512) panel_cluster_kernel(T* __restrict__ ab, BandLayout L, int64_t j0,
                                                            int* __restrict__ ipiv, int* __restrict__ perm,
                                                            int* __restrict__ info) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int cr = (int)cl.block_rank();
  const int w = (int)min64(L.nb, L.n - j0);
  const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
  const int RC = (R + CS - 1) / CS;  // <= blockDim.x / 4 (checked on the host)
  const int r0 = cr * RC, r1 = min(R, r0 + RC);
  const int nr = max(0, r1 - r0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // [w][RC]
  __shared__ PanelInbox<T> inbox[2];
  __shared__ unsigned long long red_k[2][16];
  __shared__ int red_l[2][16], red_p[2][16];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  for (int k = tid; k < w * nr; k += nt) {
    const int c = k / nr, r = k - c * nr;
    P[c * RC + r] = ab[bidx(L, j0 + r0 + r, j0 + c)];
  }
  const int rl = tid >> 2, part = tid & 3;  // local row, column part
  const bool have = rl < nr;
  const int prow = r0 + rl;                 // physical panel row
  int lrow = prow;                          // its logical row
  __syncthreads();
  for (int jj = 0; jj < w; ++jj) {
    const int par = jj & 1;
    // 1. local candidate (integer keys)
    unsigned long long bk = 0ULL;
    int bl = 0x7fffffff, bp = 0;
    if (have && part == 0 && lrow >= jj && lrow <= jj + L.kl) {
      const unsigned long long k = abs_key(P[jj * RC + rl]);
      if (k) { bk = k; bl = lrow; bp = prow; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok_ = __shfl_down_sync(0xffffffffu, bk, o);
      const int ol = __shfl_down_sync(0xffffffffu, bl, o);
      const int op = __shfl_down_sync(0xffffffffu, bp, o);
      if (ok_ > bk || (ok_ == bk && ol < bl)) { bk = ok_; bl = ol; bp = op; }
    }
    if (lane == 0) { red_k[par][warp] = bk; red_l[par][warp] = bl; red_p[par][warp] = bp; }
    __syncthreads();
    // every warp combines the per-warp results with shuffles (lane k <- warp k)
    bk = lane < nwarp ? red_k[par][lane] : 0ULL;
    bl = lane < nwarp ? red_l[par][lane] : 0x7fffffff;
    bp = lane < nwarp ? red_p[par][lane] : 0;
    for (int o = 8; o > 0; o >>= 1) {
      const unsigned long long ok_ = __shfl_down_sync(0xffffffffu, bk, o);
      const int ol = __shfl_down_sync(0xffffffffu, bl, o);
      const int op = __shfl_down_sync(0xffffffffu, bp, o);
      if (ok_ > bk || (ok_ == bk && ol < bl)) { bk = ok_; bl = ol; bp = op; }
    }
    bk = __shfl_sync(0xffffffffu, bk, 0);
    bl = __shfl_sync(0xffffffffu, bl, 0);
    bp = __shfl_sync(0xffffffffu, bp, 0);
    // 2. push the candidate into every peer's inbox
    if (bk)
      for (int k = tid; k < CS * w; k += nt) {
        const int peer = k / w, c = k - peer * w;
        cl.map_shared_rank(&inbox[par], peer)->cand[cr][c] = P[c * RC + (bp - r0)];
      }
    if (warp == nwarp - 1 && lane < CS) {  // last warp: the reciprocal, then one peer per lane
      const T rv = bk ? fast_rcp(P[jj * RC + (bp - r0)]) : T(0);
      PanelInbox<T>* box = cl.map_shared_rank(&inbox[par], lane);
      box->key[cr] = bk;
      box->rinv[cr] = rv;
      box->lidx[cr] = bl;
      box->pidx[cr] = bp;
    }
    // 3. cluster barrier
    cl.sync();
    // 4. global winner from the local inbox (identical in every thread)
    const PanelInbox<T>& ib = inbox[par];
    unsigned long long gk_ = lane < CS ? ib.key[lane] : 0ULL;
    int gl = lane < CS && gk_ ? ib.lidx[lane] : 0x7fffffff, gc = lane < CS && gk_ ? lane : -1;
    for (int o = 8; o > 0; o >>= 1) {
      const unsigned long long ok_ = __shfl_down_sync(0xffffffffu, gk_, o);
      const int ol = __shfl_down_sync(0xffffffffu, gl, o);
      const int oc = __shfl_down_sync(0xffffffffu, gc, o);
      if (ok_ > gk_ || (ok_ == gk_ && ol < gl)) { gk_ = ok_; gl = ol; gc = oc; }
    }
    gl = __shfl_sync(0xffffffffu, gl, 0);
    gc = __shfl_sync(0xffffffffu, gc, 0);
    const bool ok = gc >= 0;  // false for a zero or non-finite column
    const int gp = ok ? ib.pidx[gc] : -1;
    if (cr == 0 && tid == 0) {
      ipiv[j0 + jj] = (int)(j0 + (ok ? gl : jj));
      if (!ok) atomicCAS(info, 0, (int)(j0 + jj + 1));
    }
    if (ok) {
      if (have) {
        if (prow == gp) lrow = jj;       // the pivot row becomes row jj
        else if (lrow == jj) lrow = gl;  // row jj takes the pivot row's place
      }
      const T* pr = ib.cand[gc];
      const T rinv = ib.rinv[gc];
      const bool upd = have && lrow > jj && lrow <= jj + L.kl;
      T l = T(0);
      if (upd && part == 0) {
        l = P[jj * RC + rl] * rinv;
        P[jj * RC + rl] = l;
      }
      l = __shfl_sync(0xffffffffu, l, lane & ~3);  // share with the row's four threads
      if (upd)
        for (int c = jj + 1 + part; c < w; c += 4) P[c * RC + rl] -= l * pr[c];
    }
  }
  // write back in logical order; perm[logical] = physical
  __syncthreads();
  if (have && part == 0) perm[lrow] = prow;
  if (have)
    for (int c = part; c < w; c += 4) ab[bidx(L, j0 + lrow, j0 + c)] = P[c * RC + rl];
  cl.sync();  // no CTA exits while a peer may still write its inbox
}

// ---------------------------------------------------------------------------
// Critical-path trailing update: one CTA (four warps) per column, rows of the
// L21 product split over the warps so the column's FP64 work uses all four
// sub-partitions of the SM.
template <class T>
__global__ void __launch_bounds__(128) panel_apply_col_kernel(T* __restrict__ ab, BandLayout L, int64_t j0,
                                                              const int* __restrict__ perm, int cb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = (int)min64(L.nb, L.n - j0);
  const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
  const int64_t c = j0 + w + cb + blockIdx.x;
  T* seg = reinterpret_cast<T*>(smem_raw);  // [R]
  __shared__ T L11[32][33];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int r = tid; r < R; r += nt) seg[r] = ab[bidx(L, j0 + perm[r], c)];
  for (int k = tid; k < w * w; k += nt) {
    const int cc = k / w, i = k - cc * w;
    L11[cc][i] = i > cc ? ab[bidx(L, j0 + i, j0 + cc)] : T(0);
  }
  __syncthreads();
  if (tid < 32) {
    T x = tid < w ? seg[tid] : T(0);
    for (int k = 0; k < w; ++k) {
      const T xk = __shfl_sync(0xffffffffu, x, k);
      if (tid > k) x -= L11[k][tid] * xk;
    }
    if (tid < w) seg[tid] = x;
  }
  __syncthreads();
  for (int r = w + tid; r < R; r += nt) {
    T acc = seg[r];
#pragma unroll 8
    for (int k = 0; k < w; ++k) acc -= ab[bidx(L, j0 + r, j0 + k)] * seg[k];
    seg[r] = acc;
  }
  __syncthreads();
  for (int r = tid; r < R; r += nt) ab[bidx(L, j0 + r, c)] = seg[r];
}

// ---------------------------------------------------------------------------
// trailing columns: one warp per column (plus, optionally, the right-hand side)
template <class T>
__global__ void panel_apply_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, const int* __restrict__ perm,
                                   T* __restrict__ rhs, int cb, int ce) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = (int)min64(L.nb, L.n - j0);
  const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
  const int64_t j1 = j0 + w;
  // columns j1 + [cb, ce) of the trailing block, then the right-hand side if given
  const int ncol = (ce - cb) + (rhs ? 1 : 0);
  T* Lp = reinterpret_cast<T*>(smem_raw);             // [w][R] panel L (column-major)
  T* seg = Lp + (size_t)w * R;                         // [warps][R] column segments
  int* sperm = reinterpret_cast<int*>(seg + (size_t)(blockDim.x / 32) * R);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int k = tid; k < w * R; k += nt) {
    int c = k / R, r = k - c * R;
    Lp[k] = ab[bidx(L, j0 + r, j0 + c)];
  }
  for (int r = tid; r < R; r += nt) sperm[r] = perm[r];
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  T* s = seg + (size_t)warp * R;
  for (int cc = blockIdx.x * nw + warp; cc < ncol; cc += gridDim.x * nw) {
    const bool is_rhs = rhs && cc == ncol - 1;
    const int64_t c = j1 + cb + cc;
    // gather + permute rows [j0, j0 + R)
    if (is_rhs) {
      for (int r = lane; r < R; r += 32) s[r] = rhs[j0 + sperm[r]];
    } else {
      for (int r = lane; r < R; r += 32) s[r] = ab[bidx(L, j0 + sperm[r], c)];
    }
    __syncwarp();
    // forward substitution with the unit lower L11 (lane k owns row k, w <= 32)
    T x = lane < w ? s[lane] : T(0);
    for (int k = 0; k < w; ++k) {
      T xk = __shfl_sync(0xffffffffu, x, k);
      if (lane > k && lane < w) x -= Lp[k * R + lane] * xk;
    }
    if (lane < w) s[lane] = x;
    __syncwarp();
    // rows [w, R): subtract L21 · x
    for (int r = w + lane; r < R; r += 32) {
      T acc = s[r];
#pragma unroll 8
      for (int k = 0; k < w; ++k) acc -= Lp[k * R + r] * s[k];
      s[r] = acc;
    }
    __syncwarp();
    if (is_rhs) {
      for (int r = lane; r < R; r += 32) rhs[j0 + r] = s[r];
    } else {
      for (int r = lane; r < R; r += 32) ab[bidx(L, j0 + r, c)] = s[r];
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Forward substitution with the stored panels (for a new right-hand side),
// one CTA.  Per panel: permute rows [j0, j0+R), solve the unit-lower L11
// (staged in shared memory), subtract L21 x from rows [j0+w, j0+R).
template <class T, class V>
__global__ void __launch_bounds__(1024) forward_solve_kernel(const T* __restrict__ ab, BandLayout L,
                                                             const int* __restrict__ perm_all, int rmax,
                                                             V* __restrict__ b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* s = reinterpret_cast<V*>(smem_raw);  // [R]
  __shared__ V Ls[32][33];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t j0 = 0, pnl = 0; j0 < L.n; j0 += L.nb, ++pnl) {
    const int w = (int)min64(L.nb, L.n - j0);
    const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
    const int* pm = perm_all + pnl * rmax;
    for (int r = tid; r < R; r += nt) s[r] = b[j0 + pm[r]];
    for (int k = tid; k < w * w; k += nt) {
      const int c = k / w, i = k - c * w;
      Ls[c][i] = i > c ? V(ab[bidx(L, j0 + i, j0 + c)]) : V(0);
    }
    __syncthreads();
    if (tid < 32) {
      V x = tid < w ? s[tid] : V(0);
      for (int k = 0; k < w; ++k) {
        const V xk = __shfl_sync(0xffffffffu, x, k);
        if (tid > k) x -= Ls[k][tid] * xk;
      }
      if (tid < w) s[tid] = x;
    }
    __syncthreads();
    for (int r = w + tid; r < R; r += nt) {
      V acc = s[r];
#pragma unroll 8
      for (int k = 0; k < w; ++k) acc -= V(ab[bidx(L, j0 + r, j0 + k)]) * s[k];
      s[r] = acc;
    }
    __syncthreads();
    for (int r = tid; r < R; r += nt) b[j0 + r] = s[r];
    __syncthreads();
  }
}

// Back substitution U x = y (U has kl + ku super-diagonals), one CTA, panels
// in reverse order; x overwrites y.  The off-diagonal block product
// U(j0:j1, j1:jend) x(j1:jend) is spread over 32 warps with 8 independent
// column loads in flight per warp; U11 is staged in shared memory for the
// sequential triangular part.
template <class T, class V>
__global__ void __launch_bounds__(1024) backward_solve_kernel(const T* __restrict__ ab, BandLayout L,
                                                              V* __restrict__ y) {
  __shared__ V part[32][33];
  __shared__ V Us[32][33];
  __shared__ V xs[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  for (int64_t pnl = npan - 1; pnl >= 0; --pnl) {
    const int64_t j0 = pnl * L.nb;
    const int w = (int)min64(L.nb, L.n - j0);
    const int64_t j1 = j0 + w;
    const int64_t jend = min64(L.n, j1 + L.kl + L.ku);
    for (int k = tid; k < w * w; k += blockDim.x) {
      const int c = k / w, i = k - c * w;
      Us[c][i] = i <= c ? V(ab[bidx(L, j0 + i, j0 + c)]) : V(0);
    }
    V acc = V(0);
    if (lane < w) {
      int64_t c = j1 + warp;
      for (; c + 7 * nw < jend; c += 8 * nw) {
        V u[8], xv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          u[q] = V(ab[bidx(L, j0 + lane, c + q * nw)]);
          xv[q] = y[c + q * nw];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += u[q] * xv[q];
      }
      for (; c < jend; c += nw) acc += V(ab[bidx(L, j0 + lane, c)]) * y[c];
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      V sum = V(0);
      for (int k = 0; k < nw; ++k) sum += part[k][lane];
      V rhs = lane < w ? y[j0 + lane] - sum : V(0);
      V x = V(0);
      for (int k = w - 1; k >= 0; --k) {
        V xk = V(0);
        if (lane == k) {
          x = rhs / Us[k][k];
          xk = x;
        }
        xk = __shfl_sync(0xffffffffu, xk, k);
        if (lane < k) rhs -= Us[k][lane] * xk;
      }
      if (lane < w) xs[lane] = x;
    }
    __syncthreads();
    if (tid < w) y[j0 + tid] = xs[tid];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// host-side drivers (stream-ordered, graph-capturable)
template <class T>
size_t apply_smem_bytes(const BandLayout& L, int threads) {
  size_t R = (size_t)L.nb + L.kl;
  return R * L.nb * sizeof(T) + (size_t)(threads / 32) * R * sizeof(T) + R * sizeof(int);
}

constexpr int kClusterCS = 16;

template <class T>
size_t cluster_smem_bytes(const BandLayout& L) {
  size_t R = (size_t)L.nb + L.kl;
  return ((R + kClusterCS - 1) / kClusterCS) * L.nb * sizeof(T);
}
static int cluster_threads(const BandLayout& L) {
  int rc = (L.nb + L.kl + kClusterCS - 1) / kClusterCS;
  return 4 * ((rc + 7) / 8 * 8);
}

// Kernel attributes are process-wide, so the dynamic shared-memory cap is set
// to the device's opt-in maximum (never to one handle's size, which could
// lower it under another live handle); each layout is then checked against it.
template <class T>
cudaError_t band_lu_setup(const BandLayout& L, int apply_threads) {
  int dev = 0, cap = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t need_cluster = cluster_smem_bytes<T>(L) + 2 * sizeof(PanelInbox<T>) + 1024;
  const size_t need_apply = apply_smem_bytes<T>(L, apply_threads);
  const size_t need_col = ((size_t)L.nb + L.kl) * sizeof(T) + 32 * 33 * sizeof(T);
  if (need_cluster > (size_t)cap || need_apply > (size_t)cap || need_col > (size_t)cap) return cudaErrorInvalidValue;
  if (cluster_threads(L) > 512) return cudaErrorInvalidValue;
  const int dyn_cap = cap - 20 * 1024;  // room for the kernels' static shared memory
  if ((e = cudaFuncSetAttribute(panel_cluster_kernel<T, kClusterCS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                dyn_cap)) != cudaSuccess)
    return e;
  if (kClusterCS > 8 && (e = cudaFuncSetAttribute(panel_cluster_kernel<T, kClusterCS>,
                                                  cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(panel_apply_col_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_cap)) !=
      cudaSuccess)
    return e;
  return cudaFuncSetAttribute(panel_apply_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
}

template <class T>
static cudaError_t launch_panel(T* ab, const BandLayout& L, int64_t j0, int* ipiv, int* perm, int* info,
                                cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCS, 1, 1);
  cfg.blockDim = dim3(cluster_threads(L), 1, 1);
  cfg.dynamicSmemBytes = cluster_smem_bytes<T>(L);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kClusterCS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T, kClusterCS>, ab, L, j0, ipiv, perm, info);
}

// Factor (and, if rhs != nullptr, forward-substitute rhs in the same sweep).
// Lookahead on two streams: `st` carries the bulk trailing updates, `st2` the
// update of the next panel's columns followed by that panel's factorisation,
// so the (latency-bound) panel overlaps the (FP64-bound) bulk update.
// ev_pool holds >= 2*npan+2 events (cudaEventDisableTiming).  With prof !=
// nullptr the factorisation runs serially on `st` with timing events
// prof[3p..3p+2] around panel p's kernels.
template <class T>
int band_lu_factor(T* ab, const BandLayout& L, int* ipiv, int* perm_all, int rmax, int* info, T* rhs,
                   int apply_threads, int apply_blocks, cudaStream_t st, cudaStream_t st2, cudaEvent_t* ev_pool,
                   cudaEvent_t* prof) {
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  const size_t as = apply_smem_bytes<T>(L, apply_threads);
  const int nwarp = apply_threads / 32;
  int launches = 0;
  cudaError_t lerr = cudaSuccess;
  auto panel = [&](int64_t p, cudaStream_t s) {
    cudaError_t e = launch_panel<T>(ab, L, p * L.nb, ipiv, perm_all + p * rmax, info, s);
    if (e != cudaSuccess && lerr == cudaSuccess) lerr = e;
    ++launches;
  };
  auto ncol_of = [&](int64_t p) -> int {
    const int64_t j0 = p * L.nb, j1 = j0 + min64(L.nb, L.n - j0);
    return (int)(min64(L.n, j1 + L.kl + L.ku) - j1);
  };
  auto apply = [&](int64_t p, int cb, int ce, bool with_rhs, cudaStream_t s, bool narrow = false) {
    const int n = (ce - cb) + (with_rhs ? 1 : 0);
    if (n <= 0) return;
    if (narrow) {  // critical-path columns: one 4-warp CTA each
      panel_apply_col_kernel<T><<<ce - cb, 128, ((size_t)L.nb + L.kl) * sizeof(T), s>>>(ab, L, p * L.nb,
                                                                                   perm_all + p * rmax, cb);
    } else {
      const int blocks = (int)min64(apply_blocks, (n + nwarp - 1) / nwarp);
      panel_apply_kernel<T><<<blocks, apply_threads, as, s>>>(ab, L, p * L.nb, perm_all + p * rmax,
                                                               with_rhs ? rhs : nullptr, cb, ce);
    }
    ++launches;
  };
  if (prof || !st2) {
    for (int64_t p = 0; p < npan; ++p) {
      if (prof) cudaEventRecord(prof[3 * p], st);
      panel(p, st);
      if (prof) cudaEventRecord(prof[3 * p + 1], st);
      apply(p, 0, ncol_of(p), rhs != nullptr, st);
      if (prof) cudaEventRecord(prof[3 * p + 2], st);
    }
    return lerr == cudaSuccess ? launches : -1;
  }
  cudaEvent_t* ev_panel = ev_pool;         // [npan]
  cudaEvent_t* ev_rest = ev_pool + npan;   // [npan]
  cudaEvent_t ev_start = ev_pool[2 * npan], ev_join = ev_pool[2 * npan + 1];
  cudaEventRecord(ev_start, st);
  cudaStreamWaitEvent(st2, ev_start, 0);
  panel(0, st2);
  cudaEventRecord(ev_panel[0], st2);
  for (int64_t p = 0; p < npan; ++p) {
    const int nc = ncol_of(p);
    const int wnext = (p + 1 < npan) ? (int)min64(L.nb, L.n - (p + 1) * L.nb) : 0;
    const int split = std::min(nc, wnext);
    // bulk update of panel p on st
    cudaStreamWaitEvent(st, ev_panel[p], 0);
    apply(p, split, nc, rhs != nullptr, st);
    cudaEventRecord(ev_rest[p], st);
    if (p + 1 < npan) {
      // next panel's columns, then its factorisation, on st2
      if (p > 0) cudaStreamWaitEvent(st2, ev_rest[p - 1], 0);
      apply(p, 0, split, false, st2, true);
      panel(p + 1, st2);
      cudaEventRecord(ev_panel[p + 1], st2);
    }
  }
  cudaEventRecord(ev_join, st2);
  cudaStreamWaitEvent(st, ev_join, 0);
  return lerr == cudaSuccess ? launches : -1;
}

template <class T, class V>
cudaError_t band_solve_setup(const BandLayout& L) {
  return cudaFuncSetAttribute(forward_solve_kernel<T, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(((size_t)L.nb + L.kl) * sizeof(V)));
}
template <class T, class V>
void band_forward(const T* ab, const BandLayout& L, const int* perm_all, int rmax, V* b, cudaStream_t st) {
  forward_solve_kernel<T, V><<<1, 1024, ((size_t)L.nb + L.kl) * sizeof(V), st>>>(ab, L, perm_all, rmax, b);
}
template <class T, class V>
void band_backward(const T* ab, const BandLayout& L, V* y, cudaStream_t st) {
  backward_solve_kernel<T, V><<<1, 1024, 0, st>>>(ab, L, y);
}

template size_t apply_smem_bytes<double>(const BandLayout&, int);
template size_t apply_smem_bytes<float>(const BandLayout&, int);
template cudaError_t band_lu_setup<double>(const BandLayout&, int);
template cudaError_t band_lu_setup<float>(const BandLayout&, int);
template int band_lu_factor<double>(double*, const BandLayout&, int*, int*, int, int*, double*, int, int,
                                    cudaStream_t, cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template int band_lu_factor<float>(float*, const BandLayout&, int*, int*, int, int*, float*, int, int,
                                   cudaStream_t, cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template cudaError_t band_solve_setup<double, double>(const BandLayout&);
template cudaError_t band_solve_setup<float, double>(const BandLayout&);
template void band_forward<double, double>(const double*, const BandLayout&, const int*, int, double*,
                                           cudaStream_t);
template void band_forward<float, double>(const float*, const BandLayout&, const int*, int, double*, cudaStream_t);
template void band_backward<double, double>(const double*, const BandLayout&, double*, cudaStream_t);
template void band_backward<float, double>(const float*, const BandLayout&, double*, cudaStream_t);

}  // namespace mafem
