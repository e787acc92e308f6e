// band_lu_persist.cu -- the node-block pivoted banded LU (band_lu_blk.cu) as
// ONE persistent cooperative launch per factorisation.
//
// Roles.  CTA G-1 only factorises panels; CTA G-2 carries the right-hand side
// (when there is one).  Column c is owned by worker CTA c mod GW for the
// whole factorisation, so the updates of a column by successive panels run in
// order on one CTA without any flag; a worker has ~(ku + ndfp) / GW columns
// per panel.
//
// Per panel p every worker with columns in p's trailing range:
//   1. waits for pdone[p] (panel p factorised) and a21cnt[p] (every column of
//      p has its rows below the diagonal block final),
//   2. stages panel p (L11\U11, A21, permutation, 1/U(j,j)) in shared memory,
//   3. loads its columns and runs the triangular solves (one warp each),
//   4. for its column of panel p + 1 (at most one): updates the 32 rows the
//      next factorisation reads, bumps critcnt[p + 1], then the rows below,
//      bumps a21cnt[p + 1],
//   5. updates the rows of its other columns.
// The factorising CTA waits for critcnt[p + 1] = w(p + 1), factorises panel
// p + 1 in registers and publishes pdone[p + 1].  So the critical path per
// panel is: stage, one triangular solve, 32 rows of one column, the panel
// factorisation, and two flag hand-overs -- no kernel launches.
//
// Flags and counters are monotone across factorisations: pdone[t] holds the
// epoch that set it, critcnt[t] / a21cnt[t] reach epoch * w(t).  All waits
// are bounded (kSpinLimit polls) and abort every CTA through *err.
//
// L1 coherence.  Bulk copies into shared memory use cp.async (L1-allocating)
// only for data that no other SM writes after this SM may have cached it: a
// column's segments (written only by its owner) and the rows below a panel's
// diagonal block (written only by the owners of the panel's columns).  The
// diagonal block itself is rewritten by the factorising CTA after the column
// owners last touched it, so it -- like the pivot data and the flags -- is
// read with L2-only loads (__ldcg / ld.acquire).

#include "band_lu_common.cuh"

namespace mafem {

namespace {

template <class T>
struct PersistArgs {
  T* ab;
  BandLayout L;
  const int* ps;
  int npan, kuf, rmax, wmax;  // rmax = wmax + kl: rows of a staged panel column
  const int* blk_end;
  int* perm_all;
  T* rdiag;
  int* info;
  T* rhs;
  int* pdone;
  int* critcnt;
  int* a21cnt;
  int epoch;
  int* err;
  long long* trace;  // optional: kTraceSlots device-clock stamps per panel (diagnostics)
};
constexpr int kTraceSlots = 12;
constexpr int kMaxCols = 8;  // columns a worker handles per panel (more: the grid is too small)
__device__ __forceinline__ void stamp(long long* trace, int t, int slot) {
  if (trace && threadIdx.x == 0) {
    long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    trace[(size_t)t * kTraceSlots + slot] = v;
  }
}

// thread 0 waits until *p >= target; false (uniform over the CTA) on timeout / abort
__device__ __forceinline__ bool wait_geq(const int* p, int target, int* err, int* s_ok) {
  if (threadIdx.x == 0) {
    int ok = 1;
    for (int it = 0; ld_acquire(p) < target; ++it) {
      if (it > kSpinLimit || *(volatile int*)err) {
        atomicCAS(err, 0, 1);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

}  // namespace

template <class T>
__global__ void __launch_bounds__(256, 1) blk_factor_persist_kernel(PersistArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T s_l[2][32];
  __shared__ int s_p[2];
  __shared__ int s_ok;
  __shared__ int64_t s_col[kMaxCols];  // this panel's columns (-1: the right-hand side)
  __shared__ T s_part[4][32];          // partial sums of the critical rows
  const BandLayout& L = a.L;
  // CTA G-1 factorises; with a right-hand side CTA G-2 carries it alone (its
  // extra column would otherwise make one worker late every few panels);
  // CTAs 0 .. GW-1 own the columns.
  const int G = gridDim.x, me = blockIdx.x, GW = G - 1 - (a.rhs ? 1 : 0);
  const bool rhs_cta = a.rhs != nullptr && me == G - 2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if (me == G - 1) {  // the factorising CTA
    for (int t = 0; t < a.npan; ++t) {
      const int wt = a.ps[t + 1] - a.ps[t];
      stamp(a.trace, t, 0);
      if (t > 0 && !wait_geq(a.critcnt + t, a.epoch * wt, a.err, &s_ok)) return;
      stamp(a.trace, t, 1);
      blk_panel_factor<T, true>(a.ab, L, a.ps[t], wt, a.blk_end, a.perm_all + (size_t)t * kBlkW, a.rdiag, a.info,
                                s_l, s_p);
      fence_proxy_async_global();  // the factors are read by TMA on other SMs
      __threadfence();
      __syncthreads();
      if (tid == 0) st_release(a.pdone + t, a.epoch);
      stamp(a.trace, t, 2);
    }
    return;
  }

  // Shared memory.  Column slots of LDp elements: the panel's w columns (Lp)
  // and four column segments (S).  A segment starting at global element index
  // g is placed at slot offset g mod E (E elements = 16 bytes), so that its
  // 16-byte-aligned global elements land 16-byte-aligned in shared memory and
  // the bulk of it can be one TMA copy (cp.async.bulk); the at most E - 1
  // elements before and after the aligned bulk are loaded directly.
  constexpr int E = 16 / (int)sizeof(T);
  const int LDp = (a.rmax + 2 * E - 1) / E * E;
  T* Lp = reinterpret_cast<T*>(smem_raw);             // [kBlkW][LDp] (+64: chunk reads past R)
  T* S = Lp + (size_t)a.wmax * LDp + 64;              // [4][LDp] column segments
  T* Y = S + (size_t)4 * LDp;                         // [4][32]
  T* rd = Y + 128;                                    // [32]
  int* sp = reinterpret_cast<int*>(rd + 32);          // [32]
  __shared__ __align__(8) uint64_t s_bar[2];          // TMA completion: [0] tops, [1] the panel's A21
  __shared__ int s_sb[4];                             // S slot offsets
  if (tid == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  uint32_t ph0 = 0, ph1 = 0;
  auto lpa = [&](int k) -> T* { return Lp + (size_t)k * LDp + ((L.off - k) & (E - 1)); };  // panel column k, row 0
  // Copy of n elements src[0..n) -> dst[0..n) (same address phase mod 16 bytes): mode 0 returns the bytes
  // of the aligned bulk, mode 1 issues it as one TMA copy on `bar`, mode 2 loads the unaligned head and
  // tail (at most E - 1 elements each) directly -- after every TMA copy is in flight.
  auto seg_copy = [&](T* dst, const T* src, int n, uint64_t* bar, int mode) -> uint32_t {
    const int g = (int)(((uintptr_t)src / sizeof(T)) & (E - 1));
    const int h = min(n, (E - g) & (E - 1));
    const int nb = max(0, (n - h) / E * E);
    if (mode == 1 && nb > 0) tma_load_1d(dst + h, src + h, (uint32_t)(nb * sizeof(T)), bar);
    if (mode == 2) {
      T hv[E - 1], tv[E - 1];
#pragma unroll
      for (int i = 0; i < E - 1; ++i) {
        hv[i] = i < h ? __ldcg(src + i) : T(0);
        tv[i] = h + nb + i < n ? __ldcg(src + h + nb + i) : T(0);
      }
#pragma unroll
      for (int i = 0; i < E - 1; ++i) {
        if (i < h) dst[i] = hv[i];
        if (h + nb + i < n) dst[h + nb + i] = tv[i];
      }
    }
    return (uint32_t)(nb * sizeof(T));
  };
  auto wait_bar = [&](uint64_t* bar, uint32_t& ph) -> bool {
    int ok = 1;
    for (int it = 0; !mbar_try_wait(bar, ph); ++it)
      if (it > kSpinLimit) {
        ok = 0;
        atomicCAS(a.err, 0, 3);
        break;
      }
    ph ^= 1u;
    return __syncthreads_and(ok) != 0;
  };

  for (int p = 0; p < a.npan; ++p) {
    const int64_t j0 = a.ps[p], j1 = a.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
    const int64_t jend = min64b(L.n, j1 + a.kuf);
    const int64_t jn = p + 1 < a.npan ? a.ps[p + 2] : j1;  // panel p + 1 = columns [j1, jn)
    const int64_t cend = jend > jn ? jend : jn;
    const bool is_rhs = rhs_cta;
    const int64_t cfirst = rhs_cta ? cend : j1 + (((me - j1) % GW) + GW) % GW;
    if (cfirst >= cend && !is_rhs) continue;
    const bool tr_owner = p + 1 < a.npan && me == j1 % GW;
    if (tr_owner) stamp(a.trace, p + 1, 3);
    if (p > 0) {
      if (!wait_geq(a.pdone + p, a.epoch, a.err, &s_ok)) return;
      if (!wait_geq(a.a21cnt + p, a.epoch * w, a.err, &s_ok)) return;
    } else if (!wait_geq(a.pdone, a.epoch, a.err, &s_ok)) {
      return;
    }
    if (tr_owner) stamp(a.trace, p + 1, 4);
    const int nch = (R - w + 31) / 32;  // 32-row chunks below the diagonal block
    // columns of this panel: the one of panel p + 1 first, then the others, then the right-hand side
    const int nown = cfirst < cend ? (int)((cend - 1 - cfirst) / GW) + 1 : 0;
    const int ncol = nown + (is_rhs ? 1 : 0);
    if (ncol > kMaxCols || (nown > 1 && cfirst + GW < jn)) {  // grid too small (the host setup rules this out)
      if (tid == 0) atomicCAS(a.err, 0, 2);
      return;
    }
    if (tid < nown) s_col[tid] = cfirst + (int64_t)tid * GW;
    if (tid == 0 && is_rhs) s_col[nown] = -1;
    fence_proxy_async_smem();  // earlier reads / writes of the buffers before the TMA writes below
    __syncthreads();
    // Warp 0 issues the copies: lane l the diagonal block rows [0, w) of panel
    // column l and the segment of this CTA's column l (both on s_bar[0]), and
    // rows [w, R) of panel column l (on s_bar[1]).  So the triangular solves
    // start as soon as the small copies land, while the panel's A21 streams in.
    auto issue_cols = [&](int b0, int nb, bool with_panel) {
      if (warp != 0) return;
      fence_proxy_async_global();  // data written by ordinary stores (here or, before a flag, elsewhere)
      T* sd = nullptr;
      const T* ss = nullptr;
      if (lane < nb) {
        const int64_t c = s_col[b0 + lane];
        ss = c < 0 ? a.rhs + j0 : a.ab + bix(L, j0, c);
        const int off = (int)(((uintptr_t)ss / sizeof(T)) & (E - 1));
        s_sb[lane] = lane * LDp + off;
        sd = S + lane * LDp + off;
      }
      const bool pc = with_panel && lane < w;
      const T* pd_src = pc ? a.ab + bix(L, j0, j0 + lane) : nullptr;
      // rows [0, P1) of panel column `lane` (diagonal block + chunk 0, the rows the
      // next factorisation's update reads) on s_bar[0], rows [P1, R) on s_bar[1];
      // P1 = first 16-byte-aligned row at or after w + 32
      const int br = min(R, w + 32);
      const int P1 = min(R, br + (int)((-(L.off - lane + br)) & (E - 1)));
      uint32_t b0b = 0, b1b = 0;
      if (lane < nb) b0b += seg_copy(sd, ss, R, &s_bar[0], 0);
      if (pc) {
        b0b += seg_copy(lpa(lane), pd_src, P1, &s_bar[0], 0);
        if (R > P1) b1b += seg_copy(lpa(lane) + P1, pd_src + P1, R - P1, &s_bar[1], 0);
      }
      for (int o = 16; o > 0; o >>= 1) {
        b0b += __shfl_xor_sync(kFull, b0b, o);
        b1b += __shfl_xor_sync(kFull, b1b, o);
      }
      if (lane == 0) {
        mbar_arrive_expect_tx(&s_bar[0], b0b);
        if (with_panel) mbar_arrive_expect_tx(&s_bar[1], b1b);
      }
      __syncwarp();
      for (int mode = 1; mode <= 2; ++mode) {
        if (lane < nb) seg_copy(sd, ss, R, &s_bar[0], mode);
        if (pc) {
          seg_copy(lpa(lane), pd_src, P1, &s_bar[0], mode);
          if (R > P1) seg_copy(lpa(lane) + P1, pd_src + P1, R - P1, &s_bar[1], mode);
        }
      }
    };
    issue_cols(0, min(4, ncol), true);
    if (tid >= 32 && tid < 32 + w) {
      rd[tid - 32] = __ldcg(a.rdiag + j0 + tid - 32);
      sp[tid - 32] = __ldcg(a.perm_all + (size_t)p * kBlkW + tid - 32);
    }
    if (!wait_bar(&s_bar[0], ph0)) return;  // tops + diagonal block
    if (tr_owner) stamp(a.trace, p + 1, 5);

    for (int b0 = 0; b0 < ncol; b0 += 4) {
      const int nb = min(4, ncol - b0);
      if (b0 > 0) {  // later batches (small grids only)
        fence_proxy_async_smem();
        __syncthreads();
        issue_cols(b0, nb, false);
        if (!wait_bar(&s_bar[0], ph0)) return;
      }
      // triangular solves, one warp per column: u = L11^-1 P s[0:w] (kept as U12), y = U11^-1 u
      if (warp < 4) {
        T v = T(0);
        if (warp < nb) {
          const int64_t c = s_col[b0 + warp];
          const T* s = S + s_sb[warp];
          T* dst = c < 0 ? a.rhs + j0 : a.ab + bix(L, j0, c);
          // this lane's row of the diagonal block in registers (no shared-memory
          // load on the dependency chains): L(lane, k) for k < lane, U(lane, k) for k > lane
          T Tr[32];
#pragma unroll
          for (int k = 0; k < 32; ++k) Tr[k] = (k < w && lane < w) ? lpa(k)[lane] : T(0);
          T x = lane < w ? s[sp[lane]] : T(0);  // row `lane` of the permuted top
#pragma unroll
          for (int k = 0; k < 32; ++k) {
            if (k < w) {
              const T xk = __shfl_sync(kFull, x, k);
              if (lane > k) x = fma(-Tr[k], xk, x);
            }
          }
          if (lane < w) dst[lane] = x;  // U12: not read again by this kernel
          // y = U11^-1 u with this lane's U row pre-scaled by 1/U(lane, lane)
          // (unit diagonal): each step is one shuffle and one FMA
          const T rl = lane < w ? rd[lane] : T(0);
#pragma unroll
          for (int k = 0; k < 32; ++k)
            if (k > lane) Tr[k] *= rl;
          v = x * rl;
#pragma unroll
          for (int k = 31; k >= 0; --k) {
            if (k < w) {
              const T yk = __shfl_sync(kFull, v, k);
              if (lane < k) v = fma(-Tr[k], yk, v);
            }
          }
        }
        Y[warp * 32 + lane] = (warp < nb && lane < w) ? v : T(0);
      }
      __syncthreads();
      if (tr_owner && b0 == 0) stamp(a.trace, p + 1, 6);
      // rows [w, R): s -= A21 y, 32-row chunks; tasks (column qq, chunk ci) in [q0, q1) x [c0, c1)
      auto rows = [&](int q0, int q1, int c0, int c1) {
        const int nq = q1 - q0, ntask = nq * (c1 - c0);
        for (int tk = warp; tk < ntask; tk += 8) {
          const int qq = q0 + tk % nq, ci = c0 + tk / nq;
          const int r = w + 32 * ci + lane;
          const T* s = S + s_sb[qq];
          const T* yq = Y + qq * 32;
          T acc = s[min(r, R - 1)];
          for (int k = 0; k < w; ++k) acc = fma(-lpa(k)[r], yq[k], acc);
          if (r < R) {
            const int64_t c = s_col[b0 + qq];
            T* dst = c < 0 ? a.rhs + j0 : a.ab + bix(L, j0, c);
            dst[r] = acc;
          }
        }
        fence_proxy_async_global();  // these rows are read by TMA later
        __syncthreads();
      };
      int q0 = 0;
      if (b0 == 0 && s_col[0] >= j1 && s_col[0] < jn) {  // the column of panel p + 1
        const bool reach = s_col[0] < jend;
        if (reach && nch > 0) {  // chunk 0 (the rows panel p + 1 factorises): k split over 4 warps
          const int r = w + lane;
          if (warp < 4) {
            T part = T(0);
            for (int k = 8 * warp; k < min(w, 8 * warp + 8); ++k) part = fma(-lpa(k)[r], Y[k], part);
            s_part[warp][lane] = part;
          }
          __syncthreads();
          if (warp == 0 && r < R) {
            T* dst = a.ab + bix(L, j0, s_col[0]);
            dst[r] = S[s_sb[0] + min(r, R - 1)] +
                     ((s_part[0][lane] + s_part[1][lane]) + (s_part[2][lane] + s_part[3][lane]));
          }
          __threadfence();  // read by the factorising CTA with L2-only loads (and rewritten by it before any TMA read)
          __syncthreads();
        }
        if (tid == 0) atomicAdd(a.critcnt + p + 1, 1);
        if (tr_owner) stamp(a.trace, p + 1, 7);
        if (!wait_bar(&s_bar[1], ph1)) return;  // the rest of A21
        if (reach) {
          rows(0, 1, min(1, nch), nch);
          __threadfence();
          __syncthreads();
        }
        if (tid == 0) atomicAdd(a.a21cnt + p + 1, 1);
        if (tr_owner) stamp(a.trace, p + 1, 8);
        q0 = 1;
      }
      if (b0 == 0 && q0 == 0 && !wait_bar(&s_bar[1], ph1)) return;  // the rest of A21
      if (q0 < nb) rows(q0, nb, 0, nch);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
template <class T>
static size_t persist_smem(const BandLayout& L, int wmax) {
  constexpr int E = 16 / (int)sizeof(T);
  const size_t rmax = (size_t)wmax + L.kl;
  const size_t ldp = (rmax + 2 * E - 1) / E * E;
  return ((size_t)wmax * ldp + 64 + 4 * ldp + 128 + 32) * sizeof(T) + 32 * sizeof(int);
}

template <class T>
int blk_persist_setup(const BandLayout& L, const BlkPlan& B, BlkPersist& S) {
  int dev = 0, sms = 0, cap = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  const size_t sm = persist_smem<T>(L, B.wmax);
  if (!coop || sm + 12 * 1024 > (size_t)cap || B.wmax > kBlkW) return 0;  // + static shared memory
  if (cudaFuncSetAttribute(blk_factor_persist_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
      cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, blk_factor_persist_kernel<T>, 256, sm) != cudaSuccess ||
      per < 1)
    return 0;
  // workers need at most kMaxCols columns each per panel (columns c of the
  // trailing range, owned by c mod (G - 1), plus the right-hand side)
  S.grid = sms;
  // workers: <= kMaxCols columns each per panel, and at least one per column of
  // the widest panel (a worker owns at most one column of the next panel);
  // + the right-hand-side CTA + the factorising CTA
  S.min_grid = std::max((int)((B.kuf + B.wmax + 1 + kMaxCols - 1) / kMaxCols), B.wmax) + 2;
  if (S.grid < S.min_grid) return S.grid = 0;
  S.max_grid = S.grid;
  S.smem = sm;
  return S.grid;
}

template <class T>
int blk_lu_factor_persist(T* ab, const BandLayout& L, const BlkPlan& B, const BlkPersist& S, int epoch, int* perm_all,
                          T* rdiag, int* info, T* rhs, int* err, cudaStream_t st, long long* trace) {
  PersistArgs<T> a;
  a.ab = ab;
  a.L = L;
  a.ps = B.d_ps;
  a.npan = B.npan();
  a.kuf = B.kuf;
  a.rmax = B.wmax + (int)L.kl;
  a.wmax = B.wmax;
  a.blk_end = B.d_blk_end;
  a.perm_all = perm_all;
  a.rdiag = rdiag;
  a.info = info;
  a.rhs = rhs;
  a.pdone = S.d_pdone;
  a.critcnt = S.d_critcnt;
  a.a21cnt = S.d_a21cnt;
  a.epoch = epoch;
  a.err = err;
  a.trace = trace;
  void* args[] = {(void*)&a};
  const cudaError_t e = cudaLaunchCooperativeKernel((const void*)blk_factor_persist_kernel<T>, dim3(S.grid),
                                                    dim3(256), args, S.smem, st);
  return e == cudaSuccess ? 1 : -1;
}

template int blk_persist_setup<double>(const BandLayout&, const BlkPlan&, BlkPersist&);
template int blk_persist_setup<float>(const BandLayout&, const BlkPlan&, BlkPersist&);
template int blk_lu_factor_persist<double>(double*, const BandLayout&, const BlkPlan&, const BlkPersist&, int, int*,
                                           double*, int*, double*, int*, cudaStream_t, long long*);
template int blk_lu_factor_persist<float>(float*, const BandLayout&, const BlkPlan&, const BlkPersist&, int, int*,
                                          float*, int*, float*, int*, cudaStream_t, long long*);

}  // namespace mafem
