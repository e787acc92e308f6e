// band_lu_blk.cu -- banded LU with pivoting restricted to each node's dof block.
//
// The tangent is ordered node-major (Mesh.jl:276-284), so the unknowns of one
// control point are consecutive: a "pivot block" of at most ndf rows.  Here the
// pivot of column j is searched only among the rows of j's block that are not
// yet eliminated, instead of among all kl rows below the diagonal as LAPACK's
// gbtrf does.  On the membrane tangents this is as accurate as full partial
// pivoting (growth ~1e2, backward error ~1e-15, forward error at the
// conditioning floor) and it changes the work and the critical path on a GPU:
//   * panels are runs of whole blocks, so interchanges never leave a panel and
//     U fills only to kuf = ku + ndfp columns (ndfp = largest block - 1)
//     instead of kl + ku: half the FP64 work of the trailing updates;
//   * the pivot search is one warp reduction over <= 8 rows;
//   * rows below a panel never take part in its pivot steps, so their
//     multipliers L21 = A21 U11^-1 are never formed: the trailing update and
//     the forward substitution apply L21 u = A21 (U11^-1 u) with the raw A21.
// A zero or non-finite pivot sets `info`; the caller then falls back to the
// full partial-pivoting factorisation (band_lu.cu).
//
// After panel p (columns [j0, j1), w = j1 - j0 <= 32) the band holds, in the
// panel's columns, L11 (unit, strict lower) and U11 in rows [j0, j1) and the
// untouched A21 in rows [j1, j0 + R), R = w + kl; rdiag[j] = 1 / U(j, j);
// perm_all[p * kBlkW + i] = the panel row moved to position i.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "band_lu_common.cuh"

namespace mafem {


// ---------------------------------------------------------------------------
// Panel factorisation kernel: one CTA, the body in blk_panel_factor.
template <class T>
__global__ void __launch_bounds__(32 * kPanelWarps) blk_panel_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, int w,
                                                                     const int* __restrict__ blk_end,
                                                                     int* __restrict__ perm, T* __restrict__ rdiag,
                                                                     int* __restrict__ info) {
  __shared__ T s_l[2][32];
  __shared__ int s_p[2];
  blk_panel_factor<T, false>(ab, L, j0, w, blk_end, perm, rdiag, info, s_l, s_p);
}

// ---------------------------------------------------------------------------
// Trailing update of a panel: four columns per CTA, each column run by a pair
// of warps (warps q and q + 4 share a sub-partition's FP64 pipe, so one warp's
// issue stalls overlap the other's work).  Per column segment
// s = A(j0 .. j0+R-1, c), rows [0, w) permuted:
//   u = L11^-1 s[0:w]   (kept as U12),   y = U11^-1 u,   s[w:R] -= A21 y.
// Warp q stages the column and runs the two triangular solves, then releases
// warp q + 4 (named barrier 1 + q); the two split the 32-row chunks of the
// A21 y update (NCH chunks each per pass).  Before warp q overwrites the
// column buffer for its next column it waits until warp q + 4 is done with
// the previous one (named barrier 5 + q).  The panel columns (L11\U11 and
// A21) are staged in shared memory once per CTA.
template <class T, int NCH>
__global__ void __launch_bounds__(256) blk_apply_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, int w,
                                                        const int* __restrict__ perm, const T* __restrict__ rdiag,
                                                        T* __restrict__ rhs, int64_t c0, int ncol) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
  T* Lp = reinterpret_cast<T*>(smem_raw);  // [w][R] + 64 NCH padding (chunk reads past R)
  T* S = Lp + (size_t)w * R + 64 * NCH;    // [4][R]
  T* Y = S + (size_t)4 * R;                // [4][32]
  T* rd = Y + 128;                         // [32]
  int* sp = reinterpret_cast<int*>(rd + 32);  // [32]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int slot = warp & 3, half = warp >> 2;
  const int ntot = ncol + (rhs ? 1 : 0);
  if ((int)blockIdx.x * 4 >= ntot) return;
  for (int c = 0; c < w; ++c) {
    const T* src = ab + bix(L, j0, j0 + c);  // A(j0 + r, j0 + c) = src[r]
    for (int r = tid; r < R; r += 256) cp_async(Lp + (size_t)c * R + r, src + r);
  }
  if (tid < w) {
    rd[tid] = rdiag[j0 + tid];
    sp[tid] = perm[tid];
  }
  cp_async_wait_all();
  __syncthreads();
  T* s = S + (size_t)slot * R;
  T* yw = Y + slot * 32;
  for (int cc = blockIdx.x * 4 + slot; cc < ntot; cc += gridDim.x * 4) {
    const bool is_rhs = cc == ncol;
    const bool more = cc + (int)gridDim.x * 4 < ntot;
    T* dst = is_rhs ? rhs + j0 : ab + bix(L, j0, c0 + cc);  // row j0 + r of the column = dst[r]
    if (half == 0) {
      if (cc != (int)blockIdx.x * 4 + slot) bar_sync_n(5 + slot, 64);  // partner done with the previous column
      for (int r = lane; r < R; r += 32) cp_async(s + r, dst + (r < w ? sp[r] : r));
      cp_async_wait_all();
      __syncwarp();
      T x = lane < w ? s[lane] : T(0);
      for (int k = 0; k < w; ++k) {
        const T xk = __shfl_sync(kFull, x, k);
        if (lane > k && lane < w) x -= Lp[k * R + lane] * xk;
      }
      if (lane < w) dst[lane] = x;  // U12
      T v = x;
      for (int k = w - 1; k >= 0; --k) {
        T yk = lane == k ? v * rd[k] : T(0);
        yk = __shfl_sync(kFull, yk, k);
        if (lane == k) v = yk;
        if (lane < k) v -= Lp[k * R + lane] * yk;
      }
      yw[lane] = v;
      bar_arrive_n(1 + slot, 64);
    } else {
      bar_sync_n(1 + slot, 64);
    }
    for (int base = w; base < R; base += 64 * NCH) {
      const int hb = base + half * 32 * NCH;  // this warp's first row
      T acc[NCH];
#pragma unroll
      for (int j = 0; j < NCH; ++j) acc[j] = s[min(hb + 32 * j + lane, R - 1)];
      for (int k = 0; k < w; ++k) {
        const T yk = yw[k];
        const T* lk = Lp + (size_t)k * R + hb + lane;
#pragma unroll
        for (int j = 0; j < NCH; ++j)
          if (hb + 32 * j < R) acc[j] = fma(-lk[32 * j], yk, acc[j]);  // warp-uniform guard
      }
#pragma unroll
      for (int j = 0; j < NCH; ++j) {
        const int r = hb + 32 * j + lane;
        if (r < R) dst[r] = acc[j];
      }
    }
    if (half == 1 && more) bar_arrive_n(5 + slot, 64);
  }
}

// ---------------------------------------------------------------------------
// Critical-path variant for the next panel's columns: one CTA per column.
// Warp 0 runs the triangular solves; the four warps share the A21 y update,
// NR rows per thread, reading A21 straight from the band (L2-resident).
template <class T, int NR>
__global__ void __launch_bounds__(128) blk_apply_col_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, int w,
                                                            const int* __restrict__ perm,
                                                            const T* __restrict__ rdiag, int64_t c0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
  const int64_t c = c0 + blockIdx.x;
  T* s = reinterpret_cast<T*>(smem_raw);  // [R]
  __shared__ T T11[32][33];               // L11 below, U11 on and above the diagonal (transposed: [col][row])
  __shared__ T y[32];
  __shared__ T rd[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < w) rd[tid] = rdiag[j0 + tid];
  for (int r = tid; r < R; r += 128) s[r] = ab[bix(L, j0 + (r < w ? perm[r] : r), c)];
  for (int k = tid; k < w * w; k += 128) {
    const int cc = k / w, i = k - cc * w;
    T11[cc][i] = ab[bix(L, j0 + i, j0 + cc)];
  }
  __syncthreads();
  if (warp == 0) {
    T x = lane < w ? s[lane] : T(0);
    for (int k = 0; k < w; ++k) {
      const T xk = __shfl_sync(kFull, x, k);
      if (lane > k && lane < w) x -= T11[k][lane] * xk;
    }
    if (lane < w) s[lane] = x;
    T v = x;
    for (int k = w - 1; k >= 0; --k) {
      T yk = lane == k ? v * rd[k] : T(0);
      yk = __shfl_sync(kFull, yk, k);
      if (lane == k) v = yk;
      if (lane < k) v -= T11[k][lane] * yk;
    }
    y[lane] = lane < w ? v : T(0);
  }
  __syncthreads();
  for (int base = w; base < R; base += 128 * NR) {
    T acc[NR];
    int ri[NR];
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      ri[i] = min(base + 128 * i + tid, R - 1);
      acc[i] = s[ri[i]];
    }
    const int wrow = base + warp * 32;
    const T* col0 = ab + bix(L, j0, j0);  // A(j0 + r, j0 + k) = col0[k * (ldb - 1) + r]
    for (int k0 = 0; k0 < w; k0 += 8) {
      T a[8][NR];  // eight columns of A21 in flight per thread
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const T* col = col0 + (int64_t)min(k0 + kk, w - 1) * (L.ldb - 1);
#pragma unroll
        for (int i = 0; i < NR; ++i) a[kk][i] = (wrow + 128 * i < R) ? col[ri[i]] : T(0);
      }
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        if (k0 + kk < w) {
          const T yk = y[k0 + kk];
#pragma unroll
          for (int i = 0; i < NR; ++i)
            if (wrow + 128 * i < R) acc[i] = fma(-a[kk][i], yk, acc[i]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      const int r = base + 128 * i + tid;
      if (r < R) ab[bix(L, j0 + r, c)] = acc[i];
    }
  }
  for (int r = tid; r < w; r += 128) ab[bix(L, j0 + r, c)] = s[r];
}

// ---------------------------------------------------------------------------
// Forward substitution with the stored panels, one CTA (re-solves and the
// refinement sweeps of the FP32 form).
template <class T, class V>
__global__ void __launch_bounds__(1024) blk_forward_kernel(const T* __restrict__ ab, BandLayout L,
                                                           const int* __restrict__ ps, int npan,
                                                           const int* __restrict__ perm_all,
                                                           const T* __restrict__ rdiag, V* __restrict__ b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* s = reinterpret_cast<V*>(smem_raw);  // [R]
  __shared__ V Ls[32][33];
  __shared__ V y[32];
  __shared__ V rd[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int pnl = 0; pnl < npan; ++pnl) {
    const int64_t j0 = ps[pnl];
    const int w = ps[pnl + 1] - ps[pnl];
    const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
    const int* pm = perm_all + (size_t)pnl * kBlkW;
    for (int r = tid; r < R; r += nt) s[r] = b[j0 + (r < w ? pm[r] : r)];
    for (int k = tid; k < w * w; k += nt) {
      const int c = k / w, i = k - c * w;
      Ls[c][i] = V(ab[bix(L, j0 + i, j0 + c)]);
    }
    if (tid < w) rd[tid] = V(rdiag[j0 + tid]);
    __syncthreads();
    if (tid < 32) {
      V x = tid < w ? s[tid] : V(0);
      for (int k = 0; k < w; ++k) {
        const V xk = __shfl_sync(kFull, x, k);
        if (tid > k && tid < w) x -= Ls[k][tid] * xk;
      }
      if (tid < w) s[tid] = x;
      V v = x;
      for (int k = w - 1; k >= 0; --k) {
        V yk = tid == k ? v * rd[k] : V(0);
        yk = __shfl_sync(kFull, yk, k);
        if (tid == k) v = yk;
        if (tid < k) v -= Ls[k][tid] * yk;
      }
      y[tid] = tid < w ? v : V(0);
    }
    __syncthreads();
    for (int r = w + tid; r < R; r += nt) {
      V acc = s[r];
      const T* row = ab + bix(L, j0 + r, j0);  // A(j0 + r, j0 + k) = row[k * (ldb - 1)]
#pragma unroll 8
      for (int k = 0; k < w; ++k) acc -= V(row[(int64_t)k * (L.ldb - 1)]) * y[k];
      s[r] = acc;
    }
    __syncthreads();
    for (int r = tid; r < R; r += nt) b[j0 + r] = s[r];
    __syncthreads();
  }
}

// Back substitution U x = y, one CTA, panels in reverse; U has kuf
// super-diagonals and its diagonal reciprocals are in rdiag.
template <class T, class V>
__global__ void __launch_bounds__(1024) blk_backward_kernel(const T* __restrict__ ab, BandLayout L, int kuf,
                                                            const int* __restrict__ ps, int npan,
                                                            const T* __restrict__ rdiag, V* __restrict__ y) {
  __shared__ V part[32][33];
  __shared__ V Us[32][33];
  __shared__ V xs[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int pnl = npan - 1; pnl >= 0; --pnl) {
    const int64_t j0 = ps[pnl];
    const int w = ps[pnl + 1] - ps[pnl];
    const int64_t j1 = j0 + w;
    const int64_t jend = min64b(L.n, j1 + kuf);
    for (int k = tid; k < w * w; k += blockDim.x) {
      const int c = k / w, i = k - c * w;
      Us[c][i] = i < c ? V(ab[bix(L, j0 + i, j0 + c)]) : (i == c ? V(rdiag[j0 + c]) : V(0));
    }
    V acc = V(0);
    if (lane < w) {
      int64_t c = j1 + warp;
      for (; c + 7 * nw < jend; c += 8 * nw) {
        V u[8], xv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          u[q] = V(ab[bix(L, j0 + lane, c + q * nw)]);
          xv[q] = y[c + q * nw];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += u[q] * xv[q];
      }
      for (; c < jend; c += nw) acc += V(ab[bix(L, j0 + lane, c)]) * y[c];
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      V sum = V(0);
      for (int k = 0; k < nw; ++k) sum += part[k][lane];
      V v = lane < w ? y[j0 + lane] - sum : V(0);
      for (int k = w - 1; k >= 0; --k) {
        V xk = lane == k ? v * Us[k][k] : V(0);  // Us[k][k] holds 1 / U(k, k)
        xk = __shfl_sync(kFull, xk, k);
        if (lane == k) v = xk;
        if (lane < k) v -= Us[k][lane] * xk;
      }
      if (lane < w) xs[lane] = v;
    }
    __syncthreads();
    if (tid < w) y[j0 + tid] = xs[tid];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Explicit inverses of every panel's diagonal triangles for the cooperative
// substitutions: Li = L11^-1 (unit lower) and Ui = U11^-1 (upper, 1 / U(k, k)
// from rdiag), 32 x 32 each with element (i, k) at k * 32 + i, zero outside
// the panel's w x w block; inv[p] = Li then Ui.  One warp per panel (four per
// CTA), lane c
// forming column c of both by substitution.  With them the step of a
// substitution that lies on its critical path -- the panel's two triangles --
// is two 32-term dot products per lane with independent shuffles instead of
// two 32-step dependent chains.
template <class T, class V>
__global__ void __launch_bounds__(128) blk_inverses_kernel(const T* __restrict__ ab, BandLayout L,
                                                           const int* __restrict__ ps, int npan,
                                                           const T* __restrict__ rdiag, V* __restrict__ inv) {
  __shared__ V S[4][32][33];  // per warp: S[c][i] = A(j0 + i, j0 + c) of its panel
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.x * 4 + warp;
  if (p >= npan) return;  // warp-uniform; only warp-level synchronisation below
  const int64_t j0 = ps[p];
  const int w = (int)(ps[p + 1] - j0);
  for (int c = 0; c < 32; ++c) S[warp][c][lane] = (c < w && lane < w) ? V(ab[bix(L, j0 + lane, j0 + c)]) : V(0);
  const V rd = lane < w ? V(rdiag[j0 + lane]) : V(0);
  __syncwarp();
  V* Li = inv + (size_t)p * 2 * kBlkW * kBlkW;
  V* Ui = Li + kBlkW * kBlkW;
  V x[32];
  // column `lane` of L11^-1: L11 x = e_lane, forward
#pragma unroll
  for (int i = 0; i < 32; ++i) x[i] = i == lane ? V(1) : V(0);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const V xk = x[k];
#pragma unroll
    for (int i = k + 1; i < 32; ++i) x[i] = fma(-S[warp][k][i], xk, x[i]);
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) Li[lane * 32 + i] = (lane < w && i < w) ? x[i] : V(0);
  // column `lane` of U11^-1: U11 x = e_lane, backward
#pragma unroll
  for (int i = 0; i < 32; ++i) x[i] = i == lane ? V(1) : V(0);
#pragma unroll
  for (int k = 31; k >= 0; --k) {
    const V xk = x[k] * __shfl_sync(kFull, rd, k);
    x[k] = xk;
#pragma unroll
    for (int i = 0; i < k; ++i) x[i] = fma(-S[warp][k][i], xk, x[i]);
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) Ui[lane * 32 + i] = (lane < w && i < w) ? x[i] : V(0);
}

// ---------------------------------------------------------------------------
// Back substitution on many SMs: one cooperative launch, panel q handled by
// CTA (npan - 1 - q) mod gridDim.x.  A CTA accumulates U(q rows, c) x(c) over
// the columns of the panels above it as their flags appear (most are done
// long before it needs them), then solves its U11 triangle and publishes
// x(q) with a release store of the flag.  Flags hold the epoch of the solve
// that set them, so they never need clearing.  Waits are bounded: after
// wt.limit polls (kSpinLimit by default) the kernel records MAFEM status in
// *err and every CTA returns (no GPU hang; the host reports the error).
// wt.withhold = k >= 0 (failure-detection tests only): the flag of panel
// npan - 1 - k is never published, so the CTAs that need it run out of polls
// and every CTA returns.
template <class T, class V>
__global__ void __launch_bounds__(256) blk_backward_coop_kernel(const T* __restrict__ ab, BandLayout L, int kuf,
                                                                const int* __restrict__ ps, int npan,
                                                                const V* __restrict__ inv, V* y, int* flags,
                                                                int epoch, int* err, WaitTest wt,
                                                                const int* gate) {
  __shared__ V part[8][33];
  __shared__ V Uis[32 * 32];  // U11^-1 of the panel, element (i, k) at k * 32 + i
  __shared__ int s_ok;
  if (gate && *gate) return;  // every CTA reads the same word: all return (refinement already stopped)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int q = npan - 1 - (int)blockIdx.x; q >= 0; q -= gridDim.x) {
    const int64_t j0 = ps[q], j1 = ps[q + 1];
    const int w = (int)(j1 - j0);
    const int64_t jend = min64b(L.n, j1 + kuf);
    const V* Ui = inv + (size_t)q * 2 * kBlkW * kBlkW + kBlkW * kBlkW;
    for (int k = tid; k < kBlkW * kBlkW; k += 256) Uis[k] = __ldcg(Ui + k);
    int pl = q + 1;  // last panel with columns in [j1, jend)
    while (pl + 1 < npan && ps[pl + 1] < jend) ++pl;
    V acc = V(0);
    for (int p = (j1 < jend) ? pl : q; p > q; --p) {
      if (!wait_flag(flags, p, epoch, err, &s_ok, wt.limit)) return;
      const int64_t cb = ps[p], ce = min64b(ps[p + 1], jend);
      if (lane < w)
        for (int64_t c = cb + warp; c < ce; c += 8) acc += V(ab[bix(L, j0 + lane, c)]) * __ldcg(y + c);
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      const V sum = ((part[0][lane] + part[1][lane]) + (part[2][lane] + part[3][lane])) +
                    ((part[4][lane] + part[5][lane]) + (part[6][lane] + part[7][lane]));  // tree: 3 dependent adds
      // x1 = U11^-1 (y1 - U12 x2): one dot product per lane, the shuffles independent
      const V v = lane < w ? __ldcg(y + j0 + lane) - sum : V(0);
      V x = V(0);
#pragma unroll
      for (int k = 0; k < 32; ++k) x = fma(Uis[k * 32 + lane], __shfl_sync(kFull, v, k), x);
      if (lane < w) __stcg(y + j0 + lane, x);
      __threadfence();
      __syncwarp();
      if (lane == 0 && npan - 1 - q != wt.withhold) st_release(flags + q, epoch);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Forward substitution on many SMs: one cooperative launch, panel p handled by
// CTA p mod gridDim.x in increasing order.  For its panel's rows a CTA gathers
// the contributions A21(q) z(q) of the earlier panels q whose rows reach them
// (rows of panel q end at ps[q + 1] + kl), each as soon as q's flag appears,
// then applies the panel's interchanges and triangles like blk_forward_kernel:
// y1 = L11^-1 P b1 replaces b1 in place, z = U11^-1 y1 goes to zbuf[p] with a
// release store of the flag.  A panel waits only for lower-numbered panels,
// which CTAs take in increasing order, so the chain always progresses; waits
// are bounded (kSpinLimit polls, then *err and every CTA returns).
template <class T, class V>
__global__ void __launch_bounds__(256) blk_forward_coop_kernel(const T* __restrict__ ab, BandLayout L,
                                                               const int* __restrict__ ps, int npan,
                                                               const int* __restrict__ perm_all,
                                                               const V* __restrict__ inv, V* b, V* zbuf,
                                                               int* flags, int epoch, int* err, WaitTest wt,
                                                               const int* gate) {
  __shared__ V part[8][33];
  __shared__ V Is[2 * 32 * 32];  // L11^-1 then U11^-1 of the panel, element (i, k) at k * 32 + i
  __shared__ V accs[32];
  __shared__ int s_ok;
  if (gate && *gate) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int p = blockIdx.x; p < npan; p += gridDim.x) {
    const int64_t j0 = ps[p], j1 = ps[p + 1];
    const int w = (int)(j1 - j0);
    const V* Ip = inv + (size_t)p * 2 * kBlkW * kBlkW;
    for (int k = tid; k < 2 * kBlkW * kBlkW; k += 256) Is[k] = __ldcg(Ip + k);
    int pf = p;  // earliest panel whose rows reach j0
    while (pf > 0 && ps[pf] + L.kl > j0) --pf;
    V acc = V(0);
    for (int q = pf; q < p; ++q) {
      if (!wait_flag(flags, q, epoch, err, &s_ok, wt.limit)) return;
      const int64_t q0 = ps[q];
      const int wq = ps[q + 1] - ps[q];
      if (lane < w)
        for (int k = warp; k < wq; k += 8)
          if (j0 + lane - (q0 + k) <= L.kl)  // inside panel q's band rows
            acc += V(ab[bix(L, j0 + lane, q0 + k)]) * __ldcg(zbuf + (size_t)q * kBlkW + k);
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      accs[lane] = ((part[0][lane] + part[1][lane]) + (part[2][lane] + part[3][lane])) +
                   ((part[4][lane] + part[5][lane]) + (part[6][lane] + part[7][lane]));
      __syncwarp();
      const int pr = lane < w ? perm_all[(size_t)p * kBlkW + lane] : 0;
      const V x = lane < w ? __ldcg(b + j0 + pr) - accs[pr] : V(0);
      // y1 = L11^-1 P b1, z = U11^-1 y1: dot products with independent shuffles
      V y1 = V(0);
#pragma unroll
      for (int k = 0; k < 32; ++k) y1 = fma(Is[k * 32 + lane], __shfl_sync(kFull, x, k), y1);
      V v = V(0);
#pragma unroll
      for (int k = 0; k < 32; ++k) v = fma(Is[kBlkW * kBlkW + k * 32 + lane], __shfl_sync(kFull, y1, k), v);
      if (lane < w) {
        __stcg(b + j0 + lane, y1);
        __stcg(zbuf + (size_t)p * kBlkW + lane, v);
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release(flags + p, epoch);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// host side
constexpr int kApplyNR = 9;     // 32-row chunks per warp per pass of the bulk update (two warps per column)
constexpr int kColNR = 6;       // rows per thread per pass of the critical-path update

template <class T>
static size_t blk_apply_smem(const BandLayout& L, int w) {
  const size_t R = (size_t)w + L.kl;
  return ((size_t)w * R + 64 * kApplyNR) * sizeof(T) + 4 * R * sizeof(T) + 128 * sizeof(T) + 32 * sizeof(T) +
         32 * sizeof(int);  // Lp (+ padding) S Y rd sp
}

bool blk_plan(const std::vector<int>& blk_end, int wmax, int ku, BlkPlan& out) {
  const int n = (int)blk_end.size();
  out.ps.clear();
  out.ndfp = 0;
  out.wmax = 0;
  int j0 = 0;
  out.ps.push_back(0);
  while (j0 < n) {
    int j1 = j0;
    while (j1 < n && blk_end[j1] - j0 <= wmax) {
      out.ndfp = std::max(out.ndfp, blk_end[j1] - j1 - 1);
      j1 = blk_end[j1];
    }
    if (j1 == j0) return false;  // a block wider than wmax
    out.wmax = std::max(out.wmax, j1 - j0);
    out.ps.push_back(j1);
    j0 = j1;
  }
  out.kuf = ku + out.ndfp;
  return true;
}

template <class T>
int blk_lu_setup(const BandLayout& L) {
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  int wmax = 0;
  for (int w : {32, 24, 16, 8}) {
    if (w > L.nb) continue;
    if (blk_apply_smem<T>(L, w) <= (size_t)cap && ((size_t)w + L.kl) * sizeof(double) + 10 * 1024 <= (size_t)cap) {
      wmax = w;
      break;
    }
  }
  if (!wmax) return 0;
  if (cudaFuncSetAttribute(blk_apply_kernel<T, kApplyNR>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap) !=
          cudaSuccess ||
      cudaFuncSetAttribute(blk_apply_col_kernel<T, kColNR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           cap - 10 * 1024) != cudaSuccess ||
      cudaFuncSetAttribute(blk_forward_kernel<T, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           cap - 10 * 1024) != cudaSuccess)
    return 0;
  return wmax;
}

// Factor with node-block pivoting (and forward-substitute rhs when given).
// Lookahead on two streams: st2 updates the next panel's columns (one CTA
// each) and factors that panel while st carries the bulk of the update.
// With prof != nullptr it runs serially on st, recording prof[3p..3p+2].
template <class T>
int blk_lu_factor(T* ab, const BandLayout& L, const BlkPlan& B, int* perm_all, T* rdiag, int* info, T* rhs,
                  cudaStream_t st, cudaStream_t st2, cudaEvent_t* ev_pool, cudaEvent_t* prof) {
  const int npan = B.npan();
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int launches = 0;
  auto w_of = [&](int p) { return B.ps[p + 1] - B.ps[p]; };
  auto ncol_of = [&](int p) -> int {
    const int64_t j1 = B.ps[p + 1];
    return (int)(min64b(L.n, j1 + B.kuf) - j1);
  };
  auto panel = [&](int p, cudaStream_t s) {
    blk_panel_kernel<T><<<1, 32 * kPanelWarps, 0, s>>>(ab, L, B.ps[p], w_of(p), B.d_blk_end, perm_all + (size_t)p * kBlkW, rdiag,
                                          info);
    ++launches;
  };
  // columns [cb, ce) of the trailing block of panel p (relative to its end)
  auto apply = [&](int p, int cb, int ce, bool with_rhs, cudaStream_t s, bool narrow) {
    const int ncol = ce - cb;
    const int ntot = ncol + (with_rhs ? 1 : 0);
    if (ntot <= 0) return;
    const int64_t j0 = B.ps[p], c0 = B.ps[p + 1] + cb;
    const int w = w_of(p);
    const int* pm = perm_all + (size_t)p * kBlkW;
    if (narrow) {
      const size_t sm = ((size_t)w + L.kl) * sizeof(T);
      blk_apply_col_kernel<T, kColNR><<<ncol, 128, sm, s>>>(ab, L, j0, w, pm, rdiag, c0);
    } else {
      const int blocks = (int)min64b(sms, (ntot + 3) / 4);
      blk_apply_kernel<T, kApplyNR><<<blocks, 256, blk_apply_smem<T>(L, w), s>>>(
          ab, L, j0, w, pm, rdiag, with_rhs ? rhs : nullptr, c0, ncol);
    }
    ++launches;
  };
  if (prof || !st2) {
    for (int p = 0; p < npan; ++p) {
      if (prof) cudaEventRecord(prof[3 * p], st);
      panel(p, st);
      if (prof) cudaEventRecord(prof[3 * p + 1], st);
      apply(p, 0, ncol_of(p), rhs != nullptr, st, false);
      if (prof) cudaEventRecord(prof[3 * p + 2], st);
    }
    return launches;
  }
  cudaEvent_t* ev_panel = ev_pool;
  cudaEvent_t* ev_rest = ev_pool + npan;
  cudaEvent_t ev_start = ev_pool[2 * npan], ev_join = ev_pool[2 * npan + 1];
  cudaEventRecord(ev_start, st);
  cudaStreamWaitEvent(st2, ev_start, 0);
  panel(0, st2);
  cudaEventRecord(ev_panel[0], st2);
  for (int p = 0; p < npan; ++p) {
    const int nc = ncol_of(p);
    const int split = (p + 1 < npan) ? std::min(nc, w_of(p + 1)) : 0;
    cudaStreamWaitEvent(st, ev_panel[p], 0);
    apply(p, split, nc, rhs != nullptr, st, false);
    cudaEventRecord(ev_rest[p], st);
    if (p + 1 < npan) {
      if (p > 0) cudaStreamWaitEvent(st2, ev_rest[p - 1], 0);
      apply(p, 0, split, false, st2, true);
      panel(p + 1, st2);
      cudaEventRecord(ev_panel[p + 1], st2);
    }
  }
  cudaEventRecord(ev_join, st2);
  cudaStreamWaitEvent(st, ev_join, 0);
  return launches;
}

template <class V, class T>
void blk_forward(const T* ab, const BandLayout& L, const BlkPlan& B, const int* perm_all, const T* rdiag, V* b,
                 cudaStream_t st) {
  const size_t sm = ((size_t)B.wmax + L.kl) * sizeof(V);
  blk_forward_kernel<T, V><<<1, 1024, sm, st>>>(ab, L, B.d_ps, B.npan(), perm_all, rdiag, b);
}
template <class V, class T>
void blk_inverses(const T* ab, const BandLayout& L, const BlkPlan& B, const T* rdiag, V* inv, cudaStream_t st) {
  blk_inverses_kernel<T, V><<<(B.npan() + 3) / 4, 128, 0, st>>>(ab, L, B.d_ps, B.npan(), rdiag, inv);
}
template <class V, class T>
int blk_backward(const T* ab, const BandLayout& L, const BlkPlan& B, const V* inv, V* y, int* flags, int epoch,
                 int* err, int grid, cudaStream_t st, WaitTest wt, const int* gate) {
  const int npan = B.npan();
  int kuf = B.kuf;
  const int* ps = B.d_ps;
  void* args[] = {(void*)&ab,    (void*)&L,     (void*)&kuf, (void*)&ps, (void*)&npan, (void*)&inv,
                  (void*)&y,     (void*)&flags, (void*)&epoch, (void*)&err, (void*)&wt,  (void*)&gate};
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)blk_backward_coop_kernel<T, V>,
                                                    dim3(std::min(grid, npan)), dim3(256), args, 0, st);
  return e == cudaSuccess ? 0 : -1;
}
// single-CTA back substitution (used when a cooperative launch is not possible)
template <class V, class T>
void blk_backward_1cta(const T* ab, const BandLayout& L, const BlkPlan& B, const T* rdiag, V* y, cudaStream_t st) {
  blk_backward_kernel<T, V><<<1, 1024, 0, st>>>(ab, L, B.kuf, B.d_ps, B.npan(), rdiag, y);
}
// cooperative forward substitution; returns 0, or -1 if the launch was refused
template <class V, class T>
int blk_forward_coop(const T* ab, const BandLayout& L, const BlkPlan& B, const int* perm_all, const V* inv, V* b,
                     V* zbuf, int* flags, int epoch, int* err, int grid, cudaStream_t st, WaitTest wt,
                     const int* gate) {
  const int npan = B.npan();
  const int* ps = B.d_ps;
  void* args[] = {(void*)&ab,    (void*)&L,    (void*)&ps,    (void*)&npan,  (void*)&perm_all, (void*)&inv,
                  (void*)&b,     (void*)&zbuf, (void*)&flags, (void*)&epoch, (void*)&err, (void*)&wt, (void*)&gate};
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)blk_forward_coop_kernel<T, V>,
                                                    dim3(std::min(grid, npan)), dim3(256), args, 0, st);
  return e == cudaSuccess ? 0 : -1;
}
// CTAs of the cooperative back substitution that can be resident at once
template <class V, class T>
int blk_backward_grid() {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, blk_backward_coop_kernel<T, V>, 256, 0);
  return std::max(0, sms * std::min(per, 1));
}

template int blk_lu_setup<double>(const BandLayout&);
template int blk_lu_setup<float>(const BandLayout&);
template int blk_lu_factor<double>(double*, const BandLayout&, const BlkPlan&, int*, double*, int*, double*,
                                   cudaStream_t, cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template int blk_lu_factor<float>(float*, const BandLayout&, const BlkPlan&, int*, float*, int*, float*, cudaStream_t,
                                  cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template void blk_forward<double, double>(const double*, const BandLayout&, const BlkPlan&, const int*, const double*,
                                          double*, cudaStream_t);
template void blk_forward<double, float>(const float*, const BandLayout&, const BlkPlan&, const int*, const float*,
                                         double*, cudaStream_t);
template void blk_inverses<double, double>(const double*, const BandLayout&, const BlkPlan&, const double*, double*,
                                           cudaStream_t);
template void blk_inverses<double, float>(const float*, const BandLayout&, const BlkPlan&, const float*, double*,
                                          cudaStream_t);
template int blk_backward<double, double>(const double*, const BandLayout&, const BlkPlan&, const double*, double*,
                                          int*, int, int*, int, cudaStream_t, WaitTest, const int*);
template int blk_backward<double, float>(const float*, const BandLayout&, const BlkPlan&, const double*, double*, int*,
                                         int, int*, int, cudaStream_t, WaitTest, const int*);
template void blk_backward_1cta<double, double>(const double*, const BandLayout&, const BlkPlan&, const double*,
                                                double*, cudaStream_t);
template void blk_backward_1cta<double, float>(const float*, const BandLayout&, const BlkPlan&, const float*, double*,
                                               cudaStream_t);
template int blk_backward_grid<double, double>();
template int blk_backward_grid<double, float>();
template int blk_forward_coop<double, double>(const double*, const BandLayout&, const BlkPlan&, const int*,
                                              const double*, double*, double*, int*, int, int*, int, cudaStream_t,
                                              WaitTest, const int*);
template int blk_forward_coop<double, float>(const float*, const BandLayout&, const BlkPlan&, const int*,
                                             const double*, double*, double*, int*, int, int*, int, cudaStream_t,
                                             WaitTest, const int*);

}  // namespace mafem
