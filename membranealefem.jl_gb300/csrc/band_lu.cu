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
//   panel_factor_kernel   one CTA, panel resident in shared memory: pivot
//                         search (block argmax, first maximum like idamax),
//                         row interchanges across the whole panel, scaling,
//                         rank-1 updates; records ipiv and the panel's row
//                         permutation.
//   panel_apply_kernel    one warp per trailing column c in [j1, j1+kl+ku):
//                         permute rows [j0, j0+R) of column c, solve with the
//                         unit lower L11, subtract L21 · U12(:, c).  The
//                         right-hand side rides along as one extra column, so
//                         the forward substitution costs no extra pass.
// Band layout (BandLayout): column-major with ldb rows per column and nb rows
// of padding on both sides of the LAPACK band, so every block above is a
// plain strided rectangle; the bottom padding holds the panel-local L fill
// (LAPACK keeps it in a separate WORK31 array).

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
// panel factorisation: one CTA; P[c * R + r] holds A(j0 + r, j0 + c)
template <class T>
__global__ void panel_factor_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, int* __restrict__ ipiv,
                                    int* __restrict__ perm, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);
  const int w = (int)min64(L.nb, L.n - j0);
  const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
  __shared__ T red_v[32];
  __shared__ int red_i[32];
  __shared__ int s_p;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int k = tid; k < w * R; k += nt) {
    int c = k / R, r = k - c * R;
    P[k] = ab[bidx(L, j0 + r, j0 + c)];
  }
  __syncthreads();
  for (int jj = 0; jj < w; ++jj) {
    const int rend = min(R, jj + L.kl + 1);
    // argmax |P[jj][r]| over r in [jj, rend), ties -> smallest r
    T bv = T(-1);
    int bi = 0x7fffffff;
    for (int r = jj + tid; r < rend; r += nt) {
      T v = tabs(P[jj * R + r]);
      if (v > bv) { bv = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, bv, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if ((tid & 31) == 0) { red_v[tid >> 5] = bv; red_i[tid >> 5] = bi; }
    __syncthreads();
    if (tid < 32) {
      int nw = (nt + 31) >> 5;
      bv = tid < nw ? red_v[tid] : T(-1);
      bi = tid < nw ? red_i[tid] : 0x7fffffff;
      for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffffu, bv, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
      }
      if (tid == 0) {
        s_p = bi;
        ipiv[j0 + jj] = (int)(j0 + bi);
        if (!(bv > T(0))) atomicCAS(info, 0, (int)(j0 + jj + 1));
      }
    }
    __syncthreads();
    const int p = s_p;
    const T piv = P[jj * R + p];
    if (piv != T(0)) {
      if (p != jj)
        for (int c = tid; c < w; c += nt) {
          T t = P[c * R + jj];
          P[c * R + jj] = P[c * R + p];
          P[c * R + p] = t;
        }
      __syncthreads();
      const T rinv = T(1) / P[jj * R + jj];
      for (int r = jj + 1 + tid; r < rend; r += nt) {
        T l = P[jj * R + r] * rinv;
        P[jj * R + r] = l;
        for (int c = jj + 1; c < w; ++c) P[c * R + r] -= l * P[c * R + jj];
      }
    }
    __syncthreads();
  }
  for (int k = tid; k < w * R; k += nt) {
    int c = k / R, r = k - c * R;
    ab[bidx(L, j0 + r, j0 + c)] = P[k];
  }
  if (tid == 0) {
    // row permutation of the panel: position r receives original row perm[r]
    int* pm = perm;
    for (int r = 0; r < R; ++r) pm[r] = r;
    for (int jj = 0; jj < w; ++jj) {
      int q = ipiv[j0 + jj] - (int)j0;
      int t = pm[jj];
      pm[jj] = pm[q];
      pm[q] = t;
    }
  }
}

// ---------------------------------------------------------------------------
// trailing columns: one warp per column (plus, optionally, the right-hand side)
template <class T>
__global__ void panel_apply_kernel(T* __restrict__ ab, BandLayout L, int64_t j0, const int* __restrict__ perm,
                                   T* __restrict__ rhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = (int)min64(L.nb, L.n - j0);
  const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
  const int64_t j1 = j0 + w;
  const int64_t jend = min64(L.n, j1 + L.kl + L.ku);
  const int ncol = (int)(jend - j1) + (rhs ? 1 : 0);
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
    const int64_t c = j1 + cc;
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
// Forward substitution with the stored panels (for a new right-hand side).
template <class T, class V>
__global__ void forward_solve_kernel(const T* __restrict__ ab, BandLayout L, const int* __restrict__ perm_all,
                                     int rmax, V* __restrict__ b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* s = reinterpret_cast<V*>(smem_raw);  // [R]
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t j0 = 0, pnl = 0; j0 < L.n; j0 += L.nb, ++pnl) {
    const int w = (int)min64(L.nb, L.n - j0);
    const int R = (int)min64(L.n - j0, (int64_t)w + L.kl);
    const int* pm = perm_all + pnl * rmax;
    for (int r = tid; r < R; r += nt) s[r] = b[j0 + pm[r]];
    __syncthreads();
    if (tid < 32) {
      V x = tid < w ? s[tid] : V(0);
      for (int k = 0; k < w; ++k) {
        V xk = __shfl_sync(0xffffffffu, x, k);
        if (tid > k && tid < w) x -= V(ab[bidx(L, j0 + tid, j0 + k)]) * xk;
      }
      if (tid < w) s[tid] = x;
    }
    __syncthreads();
    for (int r = w + tid; r < R; r += nt) {
      V acc = s[r];
      for (int k = 0; k < w; ++k) acc -= V(ab[bidx(L, j0 + r, j0 + k)]) * s[k];
      s[r] = acc;
    }
    __syncthreads();
    for (int r = tid; r < R; r += nt) b[j0 + r] = s[r];
    __syncthreads();
  }
}

// Back substitution U x = y (U has kl + ku super-diagonals), one CTA, panels
// in reverse order; x overwrites y.
template <class T, class V>
__global__ void backward_solve_kernel(const T* __restrict__ ab, BandLayout L, V* __restrict__ y) {
  __shared__ V part[32][33];
  __shared__ V xs[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  for (int64_t pnl = npan - 1; pnl >= 0; --pnl) {
    const int64_t j0 = pnl * L.nb;
    const int w = (int)min64(L.nb, L.n - j0);
    const int64_t j1 = j0 + w;
    const int64_t jend = min64(L.n, j1 + L.kl + L.ku);
    // part[warp][lane] = sum over this warp's columns of U(j0 + lane, c) x[c]
    V acc = V(0);
    if (lane < w)
      for (int64_t c = j1 + warp; c < jend; c += nw) acc += V(ab[bidx(L, j0 + lane, c)]) * y[c];
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      V sum = V(0);
      for (int k = 0; k < nw; ++k) sum += part[k][lane];
      V rhs = lane < w ? y[j0 + lane] - sum : V(0);
      // upper-triangular solve of U11, lane k owns row k
      V x = V(0);
      for (int k = w - 1; k >= 0; --k) {
        V xk = V(0);
        if (lane == k) {
          x = rhs / V(ab[bidx(L, j0 + k, j0 + k)]);
          xk = x;
        }
        xk = __shfl_sync(0xffffffffu, xk, k);
        if (lane < k) rhs -= V(ab[bidx(L, j0 + lane, j0 + k)]) * xk;
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
size_t panel_smem_bytes(const BandLayout& L) {
  return (size_t)L.nb * ((size_t)L.nb + L.kl) * sizeof(T);
}
template <class T>
size_t apply_smem_bytes(const BandLayout& L, int threads) {
  size_t R = (size_t)L.nb + L.kl;
  return R * L.nb * sizeof(T) + (size_t)(threads / 32) * R * sizeof(T) + R * sizeof(int);
}

template <class T>
cudaError_t band_lu_setup(const BandLayout& L, int apply_threads) {
  cudaError_t e = cudaFuncSetAttribute(panel_factor_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)panel_smem_bytes<T>(L));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(panel_apply_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)apply_smem_bytes<T>(L, apply_threads));
}

// Factor (and, if rhs != nullptr, forward-substitute rhs in the same sweep).
template <class T>
int band_lu_factor(T* ab, const BandLayout& L, int* ipiv, int* perm_all, int rmax, int* info, T* rhs,
                   int apply_threads, int apply_blocks, cudaStream_t st, cudaEvent_t* ev) {
  const int64_t npan = (L.n + L.nb - 1) / L.nb;
  const size_t ps = panel_smem_bytes<T>(L), as = apply_smem_bytes<T>(L, apply_threads);
  int launches = 0;
  for (int64_t p = 0; p < npan; ++p) {
    const int64_t j0 = p * L.nb;
    if (ev) cudaEventRecord(ev[3 * p], st);
    panel_factor_kernel<T><<<1, 512, ps, st>>>(ab, L, j0, ipiv, perm_all + p * rmax, info);
    ++launches;
    if (ev) cudaEventRecord(ev[3 * p + 1], st);
    const int64_t j1 = j0 + min64(L.nb, L.n - j0);
    const int64_t ncol = min64(L.n, j1 + L.kl + L.ku) - j1 + (rhs ? 1 : 0);
    if (ncol > 0) {
      int nwarp = apply_threads / 32;
      int blocks = (int)min64(apply_blocks, (ncol + nwarp - 1) / nwarp);
      panel_apply_kernel<T><<<blocks, apply_threads, as, st>>>(ab, L, j0, perm_all + p * rmax, rhs);
      ++launches;
    }
    if (ev) cudaEventRecord(ev[3 * p + 2], st);
  }
  return launches;
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

template size_t panel_smem_bytes<double>(const BandLayout&);
template size_t panel_smem_bytes<float>(const BandLayout&);
template size_t apply_smem_bytes<double>(const BandLayout&, int);
template size_t apply_smem_bytes<float>(const BandLayout&, int);
template cudaError_t band_lu_setup<double>(const BandLayout&, int);
template cudaError_t band_lu_setup<float>(const BandLayout&, int);
template int band_lu_factor<double>(double*, const BandLayout&, int*, int*, int, int*, double*, int, int,
                                    cudaStream_t, cudaEvent_t*);
template int band_lu_factor<float>(float*, const BandLayout&, int*, int*, int, int*, float*, int, int,
                                   cudaStream_t, cudaEvent_t*);
template cudaError_t band_solve_setup<double, double>(const BandLayout&);
template cudaError_t band_solve_setup<float, double>(const BandLayout&);
template void band_forward<double, double>(const double*, const BandLayout&, const int*, int, double*,
                                           cudaStream_t);
template void band_forward<float, double>(const float*, const BandLayout&, const int*, int, double*, cudaStream_t);
template void band_backward<double, double>(const double*, const BandLayout&, double*, cudaStream_t);
template void band_backward<float, double>(const float*, const BandLayout&, double*, cudaStream_t);

}  // namespace mafem
