// band_lu_common.cuh -- device helpers shared by the node-block pivoted LU
// kernels (band_lu_blk.cu: one launch per panel step; band_lu_persist.cu: one
// persistent cooperative launch per factorisation).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mafem_internal.h"

namespace mafem {

namespace {
constexpr unsigned kFull = 0xffffffffu;
constexpr int kPanelWarps = 8;
__host__ __device__ __forceinline__ int64_t min64b(int64_t a, int64_t b) { return a < b ? a : b; }
__device__ __forceinline__ int64_t bix(const BandLayout& L, int64_t i, int64_t j) { return j * L.ldb + L.off + i - j; }

// pivot key: |v| ordered as an unsigned integer (top 32 bits of a double);
// zero, subnormal, NaN and Inf map to 0 (no usable pivot)
__device__ __forceinline__ unsigned pkey(double v) {
  const unsigned hi = (unsigned)__double2hiint(v) & 0x7fffffffu;
  return (hi >= 0x7ff00000u || hi < 0x00100000u) ? 0u : hi;
}
__device__ __forceinline__ unsigned pkey(float v) {
  const unsigned b = __float_as_uint(v) & 0x7fffffffu;
  return b >= 0x7f800000u ? 0u : b;
}

// Reciprocal of a pivot in two parts, 1/d = r0 (1 + t): r0 is the hardware's
// approximate FP64 reciprocal (rcp.approx.ftz.f64, a special-function-unit
// op; |1 - d r0| < 2^-19.9 measured over 2^26 seeded inputs on GB300),
// e = 1 - d r0 and t = e + e^2, so r0 (1 + t) = (1 - e^3) / d with
// |e^3| < 2^-59 -- two Newton-Raphson corrections folded into one factor.
// x / d is then fma(x r0, t, x r0).  On GB300 every FP64 instruction (and
// every f64<->f32 conversion) occupies a sub-partition's FP64 pipe for ~64
// cycles, so this takes three pipe slots where a divide takes a long sequence.
// Pivots are normal numbers here (pkey rejects the rest), which the ftz form
// requires.
__device__ __forceinline__ void recip2(double d, double& r0, double& t) {
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(d));
  const double e = fma(-d, r0, 1.0);
  t = fma(e, e, e);
}
__device__ __forceinline__ void recip2(float d, float& r0, float& t) {
  r0 = __frcp_rn(d);
  t = 0.0f;
}
template <class T>
__device__ __forceinline__ T mul_recip(T x, T r0, T t) {
  const T a = x * r0;
  return fma(a, t, a);
}

// asynchronous global -> shared copies (sm_80+ cp.async): every copy of a
// staging loop is in flight at once instead of one L2 round trip per element
template <class T>
__device__ __forceinline__ void cp_async(T* smem, const T* gmem) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(s), "l"(gmem), "n"(sizeof(T)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's most recent cp.async groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// --- TMA bulk copies (cp.async.bulk, sm_90+) completed through an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of transactions for the current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy; both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// order this thread's earlier generic-proxy shared-memory accesses before later async-proxy (TMA) ones
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// the same for global memory: written by ordinary stores, read by TMA (here or, after a flag hand-over, on another SM)
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void bar_sync_n(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void bar_arrive_n(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
}  // namespace

namespace {
template <bool CG, class T>
__device__ __forceinline__ T ldx(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}

constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// thread 0 waits for flags[p] == epoch; returns false (all threads) after
// `limit` polls (kSpinLimit when limit <= 0) or when another CTA has set *err
__device__ __forceinline__ bool wait_flag(const int* flags, int p, int epoch, int* err, int* s_ok, int limit = 0) {
  if (threadIdx.x == 0) {
    const int lim = limit > 0 ? limit : kSpinLimit;
    int ok = 1;
    for (int it = 0; ld_acquire(flags + p) != epoch; ++it) {
      if (it > lim || *(volatile int*)err) {
        atomicCAS(err, 0, 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

}  // namespace

// One pivot step of the panel, run by the warp that owns column k: pick the
// pivot among the block's rows not yet eliminated, form the multipliers,
// publish them (shared memory + named-barrier arrive) and record the pivot.
// Returns the column's final value for this lane: the multiplier below the
// pivot, the U entry (or the pivot itself) otherwise.
template <class T>
__device__ __forceinline__ T blk_pivot_step(int k, T col, int w, int lane, int bend, unsigned E, int64_t j0,
                                            T (*s_l)[32], int* s_p, int* perm, T* rdiag, int* info, int& op,
                                            T& ol, int nthreads) {
  const int bk = __shfl_sync(kFull, bend, k);  // the block of position k ends at row bk
  const bool cand = lane < bk && !((E >> lane) & 1u);
  const unsigned key = cand ? pkey(col) : 0u;
  const unsigned mx = __reduce_max_sync(kFull, key);
  const unsigned bal = __ballot_sync(kFull, cand && key == mx);
  const int p = __ffs(bal) - 1;  // the candidates are never empty
  const T piv = __shfl_sync(kFull, col, p);
  T r0, t;
  recip2(piv, r0, t);
  const bool act = lane < w && lane != p && !((E >> lane) & 1u);
  const T l = act ? mul_recip(col, r0, t) : T(0);
  s_l[k & 1][lane] = l;
  if (lane == 0) s_p[k & 1] = p;
  bar_arrive_n(1 + (k & 1), nthreads);
  if (lane == 0) {
    perm[k] = p;
    rdiag[j0 + k] = fma(r0, t, r0);
    if (mx == 0u) atomicCAS(info, 0, (int)(j0 + k + 1));
  }
  op = p;
  ol = l;
  return act ? l : col;
}

// ---------------------------------------------------------------------------
// Panel factorisation by one CTA of 8 warps (two per sub-partition, so one
// warp's FP64 issue stalls overlap the other's work), the w x w diagonal block
// in registers.  Warp q owns columns q, q + 8, ...; lane i holds panel row i (its
// original position).  Rows are never moved during the factorisation: a row
// is marked eliminated at the step that picks it and written to that position
// at the end.  Step k: the owner of column k finds the pivot (largest |v| among
// the block's rows not yet eliminated), forms the multipliers of column k,
// publishes the pivot row index and the multipliers in shared memory and
// arrives at a named barrier; the other warps wait on it, and every warp
// updates its own columns.  The owner of column k + 1 updates that column
// first and publishes step k + 1 before finishing its other columns, so the
// next pivot step overlaps the rest of step k.  Named barriers 1 and 2
// alternate between steps; the shared buffers are double-buffered by the same
// parity.
// CG: read the block with L2-only loads (it was written by other CTAs of the
// same kernel).  NW warps (4: one per sub-partition, so the pivot chain's FP64
// operations never queue behind a partner warp's).  Uses named barriers 1 and
// 2 and must be called by exactly the CTA's warps 0 .. NW-1.
template <class T, bool CG, int NW = kPanelWarps>
__device__ __forceinline__ void blk_panel_factor(T* __restrict__ ab, const BandLayout& L, int64_t j0, int w,
                                                 const int* __restrict__ blk_end, int* __restrict__ perm,
                                                 T* __restrict__ rdiag, int* __restrict__ info, T (*s_l)[32],
                                                 int* s_p) {
  const int tid = threadIdx.x, lane = tid & 31, q = tid >> 5;
  const int bend = lane < w ? (int)(blk_end[j0 + lane] - j0) : 0;
  constexpr int NCOL = 32 / NW;
  T v[NCOL];
#pragma unroll
  for (int m = 0; m < NCOL; ++m) {
    const int c = q + NW * m;
    v[m] = (c < w && lane < w) ? ldx<CG>(ab + bix(L, j0 + lane, j0 + c)) : T(0);
  }
  unsigned E = 0u;  // eliminated rows
  int mypos = 0;
  int op = 0;
  T ol = T(0);  // the step this warp published last: pivot row, multiplier of this lane's row

  if (q == 0) v[0] = blk_pivot_step(0, v[0], w, lane, bend, E, j0, s_l, s_p, perm, rdiag, info, op, ol, 32 * NW);
  for (int k = 0; k < w; ++k) {
    int p;
    T l;
    if (q == k % NW) {
      p = op;
      l = ol;
    } else {
      bar_sync_n(1 + (k & 1), 32 * NW);
      p = s_p[k & 1];
      l = s_l[k & 1][lane];
    }
    E |= 1u << p;
    if (lane == p) mypos = k;
#pragma unroll
    for (int m = 0; m < NCOL; ++m) {
      const int c = q + NW * m;
      if (c > k && c < w) {  // warp-uniform
        const T u = __shfl_sync(kFull, v[m], p);
        v[m] = fma(-l, u, v[m]);  // l == 0 on eliminated rows
        if (c == k + 1) v[m] = blk_pivot_step(k + 1, v[m], w, lane, bend, E, j0, s_l, s_p, perm, rdiag, info, op, ol, 32 * NW);
      }
    }
  }
#pragma unroll
  for (int m = 0; m < NCOL; ++m) {
    const int c = q + NW * m;
    if (c < w && lane < w) ab[bix(L, j0 + mypos, j0 + c)] = v[m];
  }
}


// Variant of blk_panel_factor with the block in shared memory (P[c][r],
// 32 x 33): a warp visits its columns with a run-time index, so the pivot
// step is one call site instead of one per register slot (smaller code, no
// per-slot branches); the column of the next pivot is still updated first.
template <class T, bool CG, int NW = kPanelWarps>
__device__ __forceinline__ void blk_panel_factor_smem(T* __restrict__ ab, const BandLayout& L, int64_t j0, int w,
                                                      const int* __restrict__ blk_end, int* __restrict__ perm,
                                                      T* __restrict__ rdiag, int* __restrict__ info, T (*s_l)[32],
                                                      int* s_p, T (*P)[33]) {
  const int tid = threadIdx.x, lane = tid & 31, q = tid >> 5;
  const int bend = lane < w ? (int)(blk_end[j0 + lane] - j0) : 0;
  for (int c = q; c < w; c += NW) P[c][lane] = lane < w ? ldx<CG>(ab + bix(L, j0 + lane, j0 + c)) : T(0);
  __syncwarp();
  unsigned E = 0u;
  int mypos = 0, op = 0;
  T ol = T(0);
  if (q == 0) P[0][lane] = blk_pivot_step(0, P[0][lane], w, lane, bend, E, j0, s_l, s_p, perm, rdiag, info, op, ol,
                                          32 * NW);
  for (int k = 0; k < w; ++k) {
    int p;
    T l;
    if (q == k % NW) {
      p = op;
      l = ol;
    } else {
      bar_sync_n(1 + (k & 1), 32 * NW);
      p = s_p[k & 1];
      l = s_l[k & 1][lane];
    }
    E |= 1u << p;
    if (lane == p) mypos = k;
    // my columns > k, the next pivot's first
    for (int c = k + 1 + (((q - (k + 1)) % NW) + NW) % NW; c < w; c += NW) {
      const T u = P[c][p];
      T v = fma(-l, u, P[c][lane]);  // l == 0 on eliminated rows
      if (c == k + 1) v = blk_pivot_step(k + 1, v, w, lane, bend, E, j0, s_l, s_p, perm, rdiag, info, op, ol, 32 * NW);
      __syncwarp();
      P[c][lane] = v;
      __syncwarp();
    }
  }
  for (int c = q; c < w; c += NW)
    if (lane < w) ab[bix(L, j0 + mypos, j0 + c)] = P[c][lane];
}

}  // namespace mafem
