// band_lu_blk.cu -- banded LU with pivoting restricted to each node's dof block.
//
// The tangent is ordered node-major (Mesh.jl:276-284), so the unknowns of one
// control point are consecutive: a "pivot block" of at most ndf rows.  Here the
// pivot of column j is searched only among the rows of j's block that are not
// yet eliminated (rows j .. blk_end[j]-1), instead of among all kl rows below
// the diagonal as LAPACK's gbtrf does.  On the membrane tangents this is as
// accurate as full partial pivoting (growth ~1e2, backward error ~1e-15,
// forward error at the conditioning floor) and it changes the work and the
// critical path on a GPU completely:
//   * interchanges stay inside a block, so U fills only to ku + ndfp columns
//     (ndfp = max block size - 1) instead of kl + ku: half the FP64 work of the
//     trailing updates;
//   * the pivot search is a warp shuffle over <= 8 rows -- no panel-wide
//     reduction per column;
//   * rows below the panel's diagonal block never take part in a pivot step,
//     so their multipliers need not be formed: the trailing update applies
//     L21 u = A21 (U11^-1 u) per column, with the raw panel rows A21.
// A zero or non-finite pivot inside a block sets `info`; the caller then falls
// back to the full partial-pivoting factorisation (band_lu.cu).
//
// Panel p covers columns [j0, j1), w = j1 - j0 <= nb, with
//   diagonal block rows [j0, j0 + Rd), Rd = w + ndfp (it holds every row a
//   pivot of the panel can come from), and all affected rows [j0, j0 + R),
//   R = w + kl + ndfp.
// After the panel kernel the band holds, in the panel's columns: L11 (strict
// lower) and U11 (upper) in rows [j0, j1); explicit multipliers Lx in rows
// [j1, j0+Rd); the raw A21 in rows [j0+Rd, j0+R).  rdiag[j] = 1 / U(j, j).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mafem_internal.h"

namespace mafem {

namespace {
__host__ __device__ __forceinline__ int64_t min64b(int64_t a, int64_t b) { return a < b ? a : b; }
__device__ __forceinline__ int64_t bix(const BandLayout& L, int64_t i, int64_t j) { return j * L.ldb + L.off + i - j; }
__device__ __forceinline__ unsigned long long akey(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
  return b > 0x7ff0000000000000ULL ? 0ULL : b;  // NaN -> 0
}
__device__ __forceinline__ unsigned long long akey(float v) {
  unsigned b = (unsigned)__float_as_int(v) & 0x7fffffffu;
  return b > 0x7f800000u ? 0ULL : (unsigned long long)b;
}
// 1/x: FP32 seed + two Newton steps (GB300 issues FP64 slowly; a divide is a long sequence)
__device__ __forceinline__ double rcp_fast(double x) {
  const float xf = (float)x;
  const float sf = __frcp_rn(xf);
  if (xf == 0.0f || !isfinite(sf) || sf == 0.0f) return 1.0 / x;
  double r = (double)sf;
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}
__device__ __forceinline__ float rcp_fast(float x) { return __frcp_rn(x); }
constexpr int kMaxRd = 40;  // nb (32) + ndfp (<= 7), rounded up
}  // namespace

// ---------------------------------------------------------------------------
// Diagonal-block factorisation of one panel: one CTA, block in shared memory.
template <class T>
__global__ void __launch_bounds__(128) blk_panel_kernel(T* __restrict__ ab, BandLayout L, int ndfp, int64_t j0,
                                                        const int* __restrict__ blk_end, int* __restrict__ ipiv,
                                                        int* __restrict__ perm, T* __restrict__ rdiag,
                                                        int* __restrict__ info) {
  __shared__ T D[32 * kMaxRd];  // column-major [c][r], stride Rd
  __shared__ int s_perm[kMaxRd];
  __shared__ int s_p;
  __shared__ T s_rinv;
  const int w = (int)min64b(L.nb, L.n - j0);
  const int Rd = (int)min64b(L.n - j0, (int64_t)w + ndfp);
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  for (int k = tid; k < w * Rd; k += nt) {
    const int c = k / Rd, r = k - c * Rd;
    D[c * Rd + r] = ab[bix(L, j0 + r, j0 + c)];
  }
  for (int r = tid; r < Rd; r += nt) s_perm[r] = r;
  __syncthreads();
  for (int jj = 0; jj < w; ++jj) {
    if (tid < 32) {
      const int bend = min(Rd, blk_end[j0 + jj] - (int)j0);  // rows jj .. bend-1 are candidates
      unsigned long long k = 0ULL;
      int idx = 0x7fffffff;
      if (jj + lane < bend) {
        k = akey(D[jj * Rd + jj + lane]);
        idx = jj + lane;
      }
      for (int o = 4; o > 0; o >>= 1) {  // blocks have <= 8 rows
        const unsigned long long ok = __shfl_down_sync(0xffffffffu, k, o);
        const int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ok > k || (ok == k && oi < idx)) { k = ok; idx = oi; }
      }
      k = __shfl_sync(0xffffffffu, k, 0);
      idx = __shfl_sync(0xffffffffu, idx, 0);
      const int p = (k != 0ULL) ? idx : jj;  // zero / NaN block: keep the diagonal, flag it
      if (p != jj && lane < w) {
        const T t = D[lane * Rd + jj];
        D[lane * Rd + jj] = D[lane * Rd + p];
        D[lane * Rd + p] = t;
      }
      __syncwarp();
      if (lane == 0) {
        if (p != jj) {
          const int t = s_perm[jj];
          s_perm[jj] = s_perm[p];
          s_perm[p] = t;
        }
        const T piv = D[jj * Rd + jj];
        const T rv = (k != 0ULL) ? rcp_fast(piv) : T(0);
        s_rinv = rv;
        s_p = p;
        ipiv[j0 + jj] = (int)(j0 + p);
        rdiag[j0 + jj] = rv;
        if (k == 0ULL) atomicCAS(info, 0, (int)(j0 + jj + 1));
      }
    }
    __syncthreads();
    const T rinv = s_rinv;
    for (int r = jj + 1 + tid; r < Rd; r += nt) D[jj * Rd + r] *= rinv;
    __syncthreads();
    const int nr = Rd - jj - 1, ncl = w - jj - 1;
    for (int k = tid; k < nr * ncl; k += nt) {
      const int c = jj + 1 + k / nr, r = jj + 1 + k % nr;
      D[c * Rd + r] -= D[jj * Rd + r] * D[c * Rd + jj];
    }
    __syncthreads();
  }
  for (int k = tid; k < w * Rd; k += nt) {
    const int c = k / Rd, r = k - c * Rd;
    ab[bix(L, j0 + r, j0 + c)] = D[c * Rd + r];
  }
  for (int r = tid; r < Rd; r += nt) perm[r] = s_perm[r];
}

// ---------------------------------------------------------------------------
// Trailing update of panel p: one warp per column c in j1 + [cb, ce) (plus the
// right-hand side if given).  For the column segment s = A(j0 .. j0+R-1, c):
//   permute rows [0, Rd); solve L11 (unit lower) on rows [0, w) -> u (U12);
//   y = U11^-1 u (back substitution with rdiag);
//   rows [w, Rd) -= Lx u;  rows [Rd, R) -= A21 y.
// NW warps per CTA; the panel columns are staged in shared memory once per CTA.
template <class T, int NW>
__global__ void __launch_bounds__(NW * 32) blk_apply_kernel(T* __restrict__ ab, BandLayout L, int ndfp, int64_t j0,
                                                            const int* __restrict__ perm,
                                                            const T* __restrict__ rdiag, T* __restrict__ rhs, int cb,
                                                            int ce) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = (int)min64b(L.nb, L.n - j0);
  const int Rd = (int)min64b(L.n - j0, (int64_t)w + ndfp);
  const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl + ndfp);
  const int64_t j1 = j0 + w;
  const int ncol = (ce - cb) + (rhs ? 1 : 0);
  T* Lp = reinterpret_cast<T*>(smem_raw);      // [w][R]
  T* seg = Lp + (size_t)w * R;                 // [NW][R]
  T* yb = seg + (size_t)NW * R;                // [NW][32]
  T* rd = yb + NW * 32;                        // [32]
  int* sperm = reinterpret_cast<int*>(rd + 32);  // [kMaxRd]
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int k = tid; k < w * R; k += nt) {
    const int c = k / R, r = k - c * R;
    Lp[k] = ab[bix(L, j0 + r, j0 + c)];
  }
  for (int k = tid; k < w; k += nt) rd[k] = rdiag[j0 + k];
  for (int r = tid; r < Rd; r += nt) sperm[r] = perm[r];
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  T* s = seg + (size_t)warp * R;
  T* y = yb + warp * 32;
  for (int cc = blockIdx.x * NW + warp; cc < ncol; cc += gridDim.x * NW) {
    const bool is_rhs = rhs && cc == ncol - 1;
    const int64_t c = j1 + cb + cc;
    if (is_rhs) {
      for (int r = lane; r < R; r += 32) s[r] = rhs[j0 + (r < Rd ? sperm[r] : r)];
    } else {
      for (int r = lane; r < R; r += 32) s[r] = ab[bix(L, j0 + (r < Rd ? sperm[r] : r), c)];
    }
    __syncwarp();
    // u = L11^-1 s[0:w]  (lane k owns row k)
    T x = lane < w ? s[lane] : T(0);
    for (int k = 0; k < w; ++k) {
      const T xk = __shfl_sync(0xffffffffu, x, k);
      if (lane > k && lane < w) x -= Lp[k * R + lane] * xk;
    }
    if (lane < w) s[lane] = x;
    // y = U11^-1 u
    T v = x;
    for (int k = w - 1; k >= 0; --k) {
      T yk = lane == k ? v * rd[k] : T(0);
      yk = __shfl_sync(0xffffffffu, yk, k);
      if (lane == k) v = yk;
      if (lane < k) v -= Lp[k * R + lane] * yk;
    }
    if (lane < w) y[lane] = v;
    __syncwarp();
    for (int r = w + lane; r < R; r += 32) {
      const T* coef = r < Rd ? s : y;
      T acc = s[r];
#pragma unroll 8
      for (int k = 0; k < w; ++k) acc -= Lp[k * R + r] * coef[k];
      s[r] = acc;
    }
    __syncwarp();
    if (is_rhs) {
      for (int r = lane; r < R; r += 32) rhs[j0 + r] = s[r];
    } else {
      for (int r = lane; r < R; r += 32) ab[bix(L, j0 + r, c)] = s[r];
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Critical-path variant: one 4-warp CTA per column of the next panel.  Warp 0
// runs the two triangular solves; all four warps share the row update, so the
// column's FP64 work uses the SM's four sub-partitions.
template <class T>
__global__ void __launch_bounds__(128) blk_apply_col_kernel(T* __restrict__ ab, BandLayout L, int ndfp, int64_t j0,
                                                            const int* __restrict__ perm,
                                                            const T* __restrict__ rdiag, int cb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = (int)min64b(L.nb, L.n - j0);
  const int Rd = (int)min64b(L.n - j0, (int64_t)w + ndfp);
  const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl + ndfp);
  const int64_t c = j0 + w + cb + blockIdx.x;
  T* s = reinterpret_cast<T*>(smem_raw);  // [R]
  __shared__ T T11[32][33];               // L11 below, U11 above the diagonal
  __shared__ T y[32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  for (int r = tid; r < R; r += nt) s[r] = ab[bix(L, j0 + (r < Rd ? perm[r] : r), c)];
  for (int k = tid; k < w * w; k += nt) {
    const int cc = k / w, i = k - cc * w;
    T11[cc][i] = ab[bix(L, j0 + i, j0 + cc)];
  }
  __syncthreads();
  if (tid < 32) {
    T x = lane < w ? s[lane] : T(0);
    for (int k = 0; k < w; ++k) {
      const T xk = __shfl_sync(0xffffffffu, x, k);
      if (lane > k && lane < w) x -= T11[k][lane] * xk;
    }
    if (lane < w) s[lane] = x;
    T v = x;
    for (int k = w - 1; k >= 0; --k) {
      T yk = lane == k ? v * rdiag[j0 + k] : T(0);
      yk = __shfl_sync(0xffffffffu, yk, k);
      if (lane == k) v = yk;
      if (lane < k) v -= T11[k][lane] * yk;
    }
    if (lane < w) y[lane] = v;
  }
  __syncthreads();
  for (int r = w + tid; r < R; r += nt) {
    const T* coef = r < Rd ? s : y;
    T acc = s[r];
#pragma unroll 8
    for (int k = 0; k < w; ++k) acc -= ab[bix(L, j0 + r, j0 + k)] * coef[k];
    s[r] = acc;
  }
  __syncthreads();
  for (int r = tid; r < R; r += nt) ab[bix(L, j0 + r, c)] = s[r];
}

// ---------------------------------------------------------------------------
// Forward substitution with the stored panels, one CTA (re-solves and the
// refinement sweeps of the FP32 form).
template <class T, class V>
__global__ void __launch_bounds__(1024) blk_forward_kernel(const T* __restrict__ ab, BandLayout L, int ndfp,
                                                           const int* __restrict__ perm_all, int rmax,
                                                           const T* __restrict__ rdiag, V* __restrict__ b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* s = reinterpret_cast<V*>(smem_raw);  // [R]
  __shared__ V Ls[32][33];
  __shared__ V y[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t j0 = 0, pnl = 0; j0 < L.n; j0 += L.nb, ++pnl) {
    const int w = (int)min64b(L.nb, L.n - j0);
    const int Rd = (int)min64b(L.n - j0, (int64_t)w + ndfp);
    const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl + ndfp);
    const int* pm = perm_all + pnl * rmax;
    for (int r = tid; r < R; r += nt) s[r] = b[j0 + (r < Rd ? pm[r] : r)];
    for (int k = tid; k < w * w; k += nt) {
      const int c = k / w, i = k - c * w;
      Ls[c][i] = V(ab[bix(L, j0 + i, j0 + c)]);  // L11 below, U11 on and above the diagonal
    }
    __syncthreads();
    if (tid < 32) {
      V x = tid < w ? s[tid] : V(0);
      for (int k = 0; k < w; ++k) {
        const V xk = __shfl_sync(0xffffffffu, x, k);
        if (tid > k && tid < w) x -= Ls[k][tid] * xk;
      }
      if (tid < w) s[tid] = x;
      V v = x;
      for (int k = w - 1; k >= 0; --k) {
        V yk = tid == k ? v * V(rdiag[j0 + k]) : V(0);
        yk = __shfl_sync(0xffffffffu, yk, k);
        if (tid == k) v = yk;
        if (tid < k) v -= Ls[k][tid] * yk;
      }
      if (tid < w) y[tid] = v;
    }
    __syncthreads();
    for (int r = w + tid; r < R; r += nt) {
      const V* coef = r < Rd ? s : y;
      V acc = s[r];
#pragma unroll 8
      for (int k = 0; k < w; ++k) acc -= V(ab[bix(L, j0 + r, j0 + k)]) * coef[k];
      s[r] = acc;
    }
    __syncthreads();
    for (int r = tid; r < R; r += nt) b[j0 + r] = s[r];
    __syncthreads();
  }
}

// Back substitution U x = y, one CTA, panels in reverse; U has ku + ndfp
// super-diagonals and its diagonal reciprocals are in rdiag.
template <class T, class V>
__global__ void __launch_bounds__(1024) blk_backward_kernel(const T* __restrict__ ab, BandLayout L, int kuf,
                                                            const T* __restrict__ rdiag, V* __restrict__ y) {
  __shared__ V part[32][33];
  __shared__ V Us[32][33];
  __shared__ V xs[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  for (int64_t pnl = npan - 1; pnl >= 0; --pnl) {
    const int64_t j0 = pnl * L.nb;
    const int w = (int)min64b(L.nb, L.n - j0);
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
        xk = __shfl_sync(0xffffffffu, xk, k);
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
// host drivers
template <class T>
static size_t blk_apply_smem(const BandLayout& L, int ndfp, int nw) {
  const size_t R = (size_t)L.nb + L.kl + ndfp;
  return R * L.nb * sizeof(T) + (size_t)nw * R * sizeof(T) + (size_t)nw * 32 * sizeof(T) + 32 * sizeof(T) +
         kMaxRd * sizeof(int);
}
static size_t blk_fwd_smem(const BandLayout& L, int ndfp, size_t vsize) {
  return ((size_t)L.nb + L.kl + ndfp) * vsize;
}

template <class T>
cudaError_t blk_lu_setup(const BandLayout& L, int ndfp) {
  int dev = 0, cap = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
  if (L.nb > 32 || L.nb + ndfp > kMaxRd) return cudaErrorInvalidValue;
  if (blk_apply_smem<T>(L, ndfp, 4) > (size_t)cap || blk_fwd_smem(L, ndfp, sizeof(double)) + 9 * 1024 > (size_t)cap)
    return cudaErrorInvalidValue;
  if ((e = cudaFuncSetAttribute(blk_apply_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap)) !=
      cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(blk_apply_col_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                cap - 10 * 1024)) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(blk_forward_kernel<T, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              cap - 10 * 1024);
}

// Factor with node-block pivoting (and forward-substitute rhs when given).
// Lookahead on two streams as in band_lu_factor: st2 updates the next panel's
// columns (one 1-warp CTA each) and factors that panel, st carries the bulk.
template <class T>
int blk_lu_factor(T* ab, const BandLayout& L, int ndfp, const int* blk_end, int* ipiv, int* perm_all, int rmax,
                  T* rdiag, int* info, T* rhs, cudaStream_t st, cudaStream_t st2, cudaEvent_t* ev_pool,
                  cudaEvent_t* prof) {
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  const int kuf = L.ku + ndfp;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t as4 = blk_apply_smem<T>(L, ndfp, 4);
  int launches = 0;
  auto ncol_of = [&](int64_t p) -> int {
    const int64_t j1 = p * L.nb + min64b(L.nb, L.n - p * L.nb);
    return (int)(min64b(L.n, j1 + kuf) - j1);
  };
  auto panel = [&](int64_t p, cudaStream_t s) {
    blk_panel_kernel<T><<<1, 128, 0, s>>>(ab, L, ndfp, p * L.nb, blk_end, ipiv, perm_all + p * rmax, rdiag, info);
    ++launches;
  };
  auto apply = [&](int64_t p, int cb, int ce, bool with_rhs, cudaStream_t s, bool narrow) {
    const int n = (ce - cb) + (with_rhs ? 1 : 0);
    if (n <= 0) return;
    if (narrow) {
      blk_apply_col_kernel<T><<<ce - cb, 128, ((size_t)L.nb + L.kl + ndfp) * sizeof(T), s>>>(
          ab, L, ndfp, p * L.nb, perm_all + p * rmax, rdiag, cb);
    } else {
      const int blocks = (int)min64b(sms, (n + 3) / 4);
      blk_apply_kernel<T, 4><<<blocks, 128, as4, s>>>(ab, L, ndfp, p * L.nb, perm_all + p * rmax, rdiag,
                                                      with_rhs ? rhs : nullptr, cb, ce);
    }
    ++launches;
  };
  if (prof || !st2) {
    for (int64_t p = 0; p < npan; ++p) {
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
  for (int64_t p = 0; p < npan; ++p) {
    const int nc = ncol_of(p);
    const int wnext = (p + 1 < npan) ? (int)min64b(L.nb, L.n - (p + 1) * L.nb) : 0;
    const int split = std::min(nc, wnext);
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
void blk_forward(const T* ab, const BandLayout& L, int ndfp, const int* perm_all, int rmax, const T* rdiag, V* b,
                 cudaStream_t st) {
  blk_forward_kernel<T, V><<<1, 1024, blk_fwd_smem(L, ndfp, sizeof(V)), st>>>(ab, L, ndfp, perm_all, rmax, rdiag, b);
}
template <class V, class T>
void blk_backward(const T* ab, const BandLayout& L, int ndfp, const T* rdiag, V* y, cudaStream_t st) {
  blk_backward_kernel<T, V><<<1, 1024, 0, st>>>(ab, L, L.ku + ndfp, rdiag, y);
}

template cudaError_t blk_lu_setup<double>(const BandLayout&, int);
template cudaError_t blk_lu_setup<float>(const BandLayout&, int);
template int blk_lu_factor<double>(double*, const BandLayout&, int, const int*, int*, int*, int, double*, int*, double*,
                                   cudaStream_t, cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template int blk_lu_factor<float>(float*, const BandLayout&, int, const int*, int*, int*, int, float*, int*, float*,
                                  cudaStream_t, cudaStream_t, cudaEvent_t*, cudaEvent_t*);
template void blk_forward<double, double>(const double*, const BandLayout&, int, const int*, int, const double*, double*,
                                          cudaStream_t);
template void blk_forward<double, float>(const float*, const BandLayout&, int, const int*, int, const float*, double*,
                                         cudaStream_t);
template void blk_backward<double, double>(const double*, const BandLayout&, int, const double*, double*, cudaStream_t);
template void blk_backward<double, float>(const float*, const BandLayout&, int, const float*, double*, cudaStream_t);

}  // namespace mafem
