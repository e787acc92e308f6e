// band_lu_patch.cu -- many patches' FP32 linear solves in two launches.
//
// The batched FP32 form solves K Δu = -r for every patch of a batch with one
// CTA per patch: `patch_factor_kernel` factors each patch's FP32 band with
// node-block pivoting (the same factors as band_lu_blk.cu: L11\U11 with the
// panel's rows permuted, U12 = L11^-1 P A12, raw A21, rdiag = 1/U(j,j),
// perm_all[p * 32 + i]), and `patch_refine_kernel` runs the FP32 triangular
// solves and FP64 iterative refinement x += LU^-1 (r - A0 x) until the last
// correction is at most tol |x| -- the role of `K_gl \ r_gl` (FiniteElement.jl:38).
// A single patch's LU is a chain of dependent panels; across a batch the
// chains are independent, so one CTA per patch keeps every SM busy without
// any inter-CTA synchronisation (the multi-CTA persistent kernel spends most
// of its SM time waiting on the chain, which pays only for one patch alone).
//
// Per panel (columns [j0, j1), w <= 32 wide, R = w + kl rows) the CTA
//   1. factors the w x w diagonal block (blk_panel_factor, warps 0..7),
//   2. stages the panel columns (L11\U11 and A21) in shared memory and forms
//      Li = L11^-1 and Ui = U11^-1 explicitly (one warp each, lane = column),
//      Mi = Ui Li, and stores Li, Ui for the solves,
//   3. for the kuf trailing columns, in chunks of 512: U12 = Li P A12 and
//      Y = Mi P A12 (one thread per column, the column in registers, the
//      inverses' rows as shared-memory broadcasts), then A22 -= A21 Y: each thread owns one
//      row and 32 columns in registers, A21 from shared memory, Y as float4
//      broadcasts, the band read and written once, coalesced along columns.
// The explicit inverses turn the triangular solves of step 3 and of the
// substitutions into small matrix products; the refinement absorbs their
// rounding.

#include <cuda_runtime.h>

#include <cstdint>

#include "band_lu_common.cuh"
#include "tcgen05.cuh"

namespace mafem {

constexpr int kPT = 512;   // threads per CTA of the factorisation (16 warps)
constexpr int kRT = 768;   // threads per CTA of the refinement (24 warps)
constexpr int kNCH = 256;  // trailing columns per chunk at most (the MMA's N <= 256)
constexpr int kMT = 128;   // rows of A22 per tensor-core tile (the MMA's M)
constexpr int kIS = 36;    // shared-memory row stride of the 32 x 32 inverses (16-byte rows)
// Y (the MMA's B operand, K-major core matrices): element (k, c) of a chunk at
// float (k / 4) * 4 kNCH + 4 c + k % 4, hi and lo parts in two such arrays
constexpr uint32_t kYPlane = 16u * kNCH;                // bytes between k-quads (the LBO of B)
constexpr uint32_t kYBytes = 8u * kYPlane;              // one of Yh / Yl: 32 KB
constexpr uint32_t kATile = 8u * kMT * 16u;             // one of A21h / A21l per M tile: 16 KB
constexpr uint32_t kChunkBytes = 2 * kYBytes + 4 * kATile;  // Yh, Yl and two (A21h, A21l) tile buffers: 128 KB
constexpr uint32_t kTmemCols = 2 * kNCH;                // two FP32 accumulators of 128 x 256
// A factorisation CTA asks for at least this much dynamic shared memory, so no
// two of them share an SM and its Tensor Memory (each allocates all 512 columns).
constexpr size_t kExclusiveSmem = 116 * 1024;

// panel column stride in shared memory: >= 32 + kl, == 8 mod 32 (conflict-free column staging)
__host__ __device__ inline int patch_rp(int kl) { return ((kBlkW + kl + 23) & ~31) + 8; }
__host__ __device__ inline size_t patch_region0(int kl) {
  const size_t lp = sizeof(float) * (size_t)kBlkW * patch_rp(kl);
  const size_t r = lp > kChunkBytes ? lp : kChunkBytes;
  return (r + 1023) & ~(size_t)1023;
}

size_t patch_factor_smem(int kl) {
  const size_t s = patch_region0(kl) + sizeof(float) * 3 * (size_t)kBlkW * kIS;
  return s > kExclusiveSmem ? s : kExclusiveSmem;
}
// Rows of the split-A21 buffer per part (hi, lo): the most rows below a panel's
// diagonal block (kl), rounded up to whole M tiles.
int patch_a21_rows(int kl) { return (kl + kMT - 1) / kMT * kMT; }

// x = hi + lo with hi, lo TF32 (round to nearest): the 3xTF32 split
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  unsigned h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  const float r = x - __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  hi = __uint_as_float(h);
  lo = __uint_as_float(l);
}
size_t patch_refine_smem(int64_t n) { return sizeof(float) * (size_t)n; }

__device__ __forceinline__ void stamp(long long* tr, int slot) {
  if (tr && threadIdx.x == 0) {
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    tr[slot] = (long long)v;
  }
}

// all threads of every CTA of the cluster; orders each CTA's prior memory
// accesses (global included) before the others' later ones
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Bounded wait on an mbarrier phase: after kMbarPolls polls the wait gives up
// and records 1 in *err (the patch's wait-ran-out word); once that word is
// set every later wait gives up at its first poll, so the kernel runs to its
// end quickly, and the host reports the failure.
constexpr int kMbarPolls = 1 << 20;
__device__ __forceinline__ void mbar_wait_bounded(uint64_t* bar, uint32_t& ph, int* err) {
  for (int it = 0; !mbar_try_wait(bar, ph); ++it)
    if (it > kMbarPolls || *(volatile int*)err) {
      atomicExch(err, 1);
      break;
    }
  ph ^= 1u;
}

// trace (J.trace, optional): per panel 6 globaltimer stamps -- [0] start,
// [1] diagonal block factored, [2] panel staged, inverses formed and A21 split,
// [3] U12 / Y of the first chunk, [4] its trailing update, [5] panel done
//
// NR = 2: a patch on a cluster of two CTAs (launched with cluster dims (2,1,1)).
// Rank 0 factors the diagonal block; both ranks stage the panel, form the
// inverses and split half of A21 each; rank r updates the trailing chunks
// r, r + 2, ... .  A column moves from rank 1's chunks to rank 0's as the
// panels advance, so every band read goes to L2 (ld.global.cg) and each panel
// ends at a cluster barrier; the factored block is published by another after
// the panel factorisation.  Both ranks run the same panel loop, so every
// barrier is reached by all threads of both CTAs.
//
// The trailing update A22 -= A21 Y runs on the fifth-generation tensor cores:
// per 128-row tile of A22, 3 x 4 tcgen05.mma of kind::tf32 (the 3xTF32 split
// a b ~ al bh + ah bl + ah bh over K = 32 in steps of 8) accumulate A21 Y in
// Tensor Memory; the A21 tiles come by TMA (a 3-D tensor map over the patch's
// split-A21 buffer, written once per panel) into two shared-memory buffers, so
// the copy of tile t + 2 and the MMAs of tile t + 1 run while all 16 warps read
// tile t's accumulators back (tcgen05.ld) and write A22 - A21 Y to the band.
template <int NR>
__global__ void __launch_bounds__(kPT, 1) patch_factor_kernel(const PatchJob* __restrict__ jobs,
                                                             const int* __restrict__ order) {
  constexpr bool CG = NR > 1;
  const int rank = (int)(blockIdx.x % NR);
  const PatchJob& J = jobs[order[blockIdx.x / NR]];
  const BandLayout L = J.L;
  float* __restrict__ ab = J.band;
  const int Rp = patch_rp(L.kl);
  extern __shared__ __align__(1024) unsigned char smem_fac[];
  // region 0: the panel's columns while the panel is staged, then the chunk buffers
  float* Lp = reinterpret_cast<float*>(smem_fac);  // [32][Rp]: A(j0 + r, j0 + c) at Lp[c * Rp + r]
  float* Yh = reinterpret_cast<float*>(smem_fac);  // [8][kNCH][4]
  float* Yl = reinterpret_cast<float*>(smem_fac + kYBytes);
  unsigned char* Abuf = smem_fac + 2 * kYBytes;  // [2][A21h tile | A21l tile]
  float* Li = reinterpret_cast<float*>(smem_fac + patch_region0(L.kl));  // [32][kIS]
  float* Ui = Li + kBlkW * kIS;
  float* Mi = Ui + kBlkW * kIS;
  __shared__ float s_l[2][32];
  __shared__ int s_p[2];
  __shared__ int sp[32];
  __shared__ float rd[32];
  __shared__ __align__(8) uint64_t bar_tma[2], bar_mma[2];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t ldm = L.ldb - 1;  // A(i, j + 1) - A(i, j) in the band array
  const int nrp = J.a21_rows;     // rows per part of the split-A21 buffer
  int* err = J.info + 1;

  if (tid == 0) {
    mbar_init(&bar_tma[0], 1);
    mbar_init(&bar_tma[1], 1);
    mbar_init(&bar_mma[0], 1);
    mbar_init(&bar_mma[1], 1);
    mbar_init_fence();
  }
  if (warp == 0) {
    tc::tmem_alloc(&s_tmem, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = s_tmem;
  uint32_t ph_tma[2] = {0u, 0u}, ph_mma[2] = {0u, 0u};  // phases (thread 0 uses ph_tma)

  for (int p = 0; p < J.npan; ++p) {
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
    const int C = (int)(min64b(L.n, j1 + J.kuf) - j1);
    int* perm = J.perm + (size_t)p * kBlkW;
    long long* tr = J.trace ? J.trace + (size_t)p * 6 : nullptr;
    stamp(tr, 0);

    // 1. the diagonal block
    if (rank == 0 && warp < kPanelWarps)
      blk_panel_factor<float, CG>(ab, L, j0, w, J.blk_end, perm, J.rdiag, J.info, s_l, s_p);
    __syncthreads();
    if (NR > 1) cluster_sync();
    stamp(tr, 1);

    // 2. panel columns (all copies in flight at once), then the inverses of
    //    L11 and U11 by column, each lane's column in registers
    for (int c = 0; c < w; ++c) {
      const float* src = ab + bix(L, j0, j0 + c);
      if (CG) {
        for (int r = tid; r < R; r += kPT) Lp[c * Rp + r] = __ldcg(src + r);
      } else {
        for (int r = tid; r < R; r += kPT) cp_async(Lp + c * Rp + r, src + r);
      }
    }
    if (tid < kBlkW) {
      sp[tid] = tid < w ? ldx<CG>(perm + tid) : 0;
      rd[tid] = tid < w ? ldx<CG>(J.rdiag + j0 + tid) : 0.0f;
    }
    if (!CG) cp_async_wait_all();
    __syncthreads();
    if (warp < 2) {
      float x[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) x[i] = i == lane ? 1.0f : 0.0f;
      if (warp == 0) {  // L11 X = I (unit lower), forward by columns of L
#pragma unroll
        for (int k = 0; k < 32; ++k)
          if (k < w) {
            const float xk = x[k];
#pragma unroll
            for (int i = k + 1; i < 32; ++i)
              if (i < w) x[i] = fmaf(-Lp[k * Rp + i], xk, x[i]);
          }
      } else {  // U11 X = I, backward by columns of U
#pragma unroll
        for (int k = 31; k >= 0; --k)
          if (k < w) {
            x[k] *= rd[k];
            const float xk = x[k];
#pragma unroll
            for (int i = 0; i < k; ++i) x[i] = fmaf(-Lp[k * Rp + i], xk, x[i]);
          }
      }
      float* X = warp == 0 ? Li : Ui;
#pragma unroll
      for (int i = 0; i < 32; ++i) X[i * kIS + lane] = (lane < w && i < w) ? x[i] : 0.0f;
    } else {
      // A21 (rows w .. R-1 of the panel) split into TF32 hi / lo parts, written
      // to the patch's split-A21 buffer as 8 k-quad planes [k/4][row][k%4]
      // (hi rows 0 .. nrp-1, lo rows nrp .. 2 nrp-1), rows past the panel and
      // columns k >= w zero; each rank of a cluster writes its share of the rows
      const int nr = R - w;
      const int nrt = (nr + kMT - 1) / kMT * kMT;
      const int rlo = rank * (nrt / NR), rhi = rank + 1 == NR ? nrt : (rank + 1) * (nrt / NR);
      for (int idx = tid - 64; idx < (rhi - rlo) * 8; idx += kPT - 64) {
        const int r = rlo + idx % (rhi - rlo), kq = idx / (rhi - rlo);
        float4 h, l;
        float* hv = &h.x;
        float* lv = &l.x;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int k = 4 * kq + e;
          const float v = (r < nr && k < w) ? Lp[k * Rp + w + r] : 0.0f;
          split_tf32(v, hv[e], lv[e]);
        }
        float4* plane = reinterpret_cast<float4*>(J.a21) + (size_t)kq * 2 * nrp;
        plane[r] = h;
        plane[nrp + r] = l;
      }
      fence_proxy_async_global();  // read by TMA (this CTA or, after the cluster barrier, the other)
    }
    __syncthreads();
    float* inv = J.inv + (size_t)p * 2 * kBlkW * kBlkW;  // Li then Ui, 32 x 32, column-major
    for (int idx = tid; idx < kBlkW * kBlkW; idx += kPT) {
      const int i = idx >> 5, c = idx & 31;
      float s = 0.0f;
      for (int k = max(i, c); k < w; ++k) s = fmaf(Ui[i * kIS + k], Li[k * kIS + c], s);
      Mi[i * kIS + c] = s;
      if (rank == 0) {  // stored transposed: element (i, c) at c * 32 + i
        inv[c * kBlkW + i] = Li[i * kIS + c];
        inv[kBlkW * kBlkW + c * kBlkW + i] = Ui[i * kIS + c];
      }
    }
    __syncthreads();
    if (NR > 1) cluster_sync();  // both halves of the split A21 written (and Lp no longer read)
    stamp(tr, 2);

    // 3. trailing columns [j1, j1 + C) in chunks of nch <= kNCH, balanced over the ranks
    const int nr = R - w;
    const int ntile = (nr + kMT - 1) / kMT;
    const int cpr = (C + NR * kNCH - 1) / (NR * kNCH);  // chunks per rank
    const int nch = C > 0 ? ((C + NR * cpr - 1) / (NR * cpr) + 15) & ~15 : kNCH;
    bool first = true;
    for (int cb = rank * nch; cb < C; cb += NR * nch) {
      const int nc = min(nch, C - cb);
      const int ncp = (nc + 15) & ~15;  // the MMA's N
      // U12 = Li P A12 and Y = Mi P A12: one thread per column, the column in
      // registers; Y goes to Yh / Yl split into TF32 parts (zero beyond nc)
      for (int c = tid; c < ncp; c += kPT) {
        const int64_t col = j1 + cb + c;
        float* dst = ab + bix(L, j0, col);  // A(j0 + r, col) = dst[r]
        float a[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) a[k] = (c < nc && k < w) ? ldx<CG>(dst + sp[k]) : 0.0f;
#pragma unroll 2
        for (int r = 0; r < 32; ++r) {
          float u = 0.0f, y = 0.0f;
          if (r < w) {  // block-uniform
            const float4* l4 = reinterpret_cast<const float4*>(Li + r * kIS);
            const float4* m4 = reinterpret_cast<const float4*>(Mi + r * kIS);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const float4 l = l4[k], m = m4[k];
              u = fmaf(l.x, a[4 * k], u);
              u = fmaf(l.y, a[4 * k + 1], u);
              u = fmaf(l.z, a[4 * k + 2], u);
              u = fmaf(l.w, a[4 * k + 3], u);
              y = fmaf(m.x, a[4 * k], y);
              y = fmaf(m.y, a[4 * k + 1], y);
              y = fmaf(m.z, a[4 * k + 2], y);
              y = fmaf(m.w, a[4 * k + 3], y);
            }
            if (c < nc) dst[r] = u;  // U12
          }
          float yh, yl;
          split_tf32(y, yh, yl);  // rows r >= w: 0
          const int o = (r >> 2) * (4 * kNCH) + 4 * c + (r & 3);
          Yh[o] = yh;
          Yl[o] = yl;
        }
      }
      fence_proxy_async_smem();  // Yh / Yl are read by the tensor cores
      __syncthreads();
      if (first) stamp(tr, 3);

      // A22 -= A21 Y, 128 rows at a time
      const uint32_t idesc = tc::idesc_tf32(kMT, ncp);
      const uint32_t yh = tc::saddr(Yh), yl = tc::saddr(Yl), a0 = tc::saddr(Abuf);
      const int ksteps = (w + 7) >> 3;
      auto tma_tile = [&](int t) {  // thread 0: tile t's A21h and A21l into buffer t & 1
        const int b = t & 1;
        mbar_arrive_expect_tx(&bar_tma[b], 2 * kATile);
        tc::tma_load_3d(Abuf + b * 2 * kATile, &J.a21_map, 0, t * kMT, 0, &bar_tma[b]);
        tc::tma_load_3d(Abuf + b * 2 * kATile + kATile, &J.a21_map, 0, nrp + t * kMT, 0, &bar_tma[b]);
      };
      auto mma_tile = [&](int t) {  // thread 0: tile t's products into accumulator t & 1
        const int b = t & 1;
        mbar_wait_bounded(&bar_tma[b], ph_tma[b], err);
        tc::fence_after();
        const uint32_t ah = a0 + b * 2 * kATile, al = ah + kATile, d = tmem + b * kNCH;
        for (int s = 0; s < ksteps; ++s) {  // k = 8 s .. 8 s + 7: k-quads 2 s and 2 s + 1
          const uint64_t dah = tc::smem_desc(ah + 2 * s * (kMT * 16), kMT * 16, 128);
          const uint64_t dal = tc::smem_desc(al + 2 * s * (kMT * 16), kMT * 16, 128);
          const uint64_t dbh = tc::smem_desc(yh + 2 * s * kYPlane, kYPlane, 128);
          const uint64_t dbl = tc::smem_desc(yl + 2 * s * kYPlane, kYPlane, 128);
          tc::mma_tf32(d, dal, dbh, idesc, s > 0 ? 1u : 0u);
          tc::mma_tf32(d, dah, dbl, idesc, 1u);
          tc::mma_tf32(d, dah, dbh, idesc, 1u);
        }
        tc::commit(&bar_mma[b]);
      };
      if (tid == 0 && ntile > 0) {
        tma_tile(0);
        if (ntile > 1) tma_tile(1);
        mma_tile(0);
      }
      // epilogue roles: warp w reads lanes 32 (w % 4) .. + 31 (its rows) of
      // column group w / 4 (a quarter of the chunk, in multiples of 8 columns)
      const int q = warp & 3, grp = warp >> 2;
      const int cpg = ((ncp >> 2) + 7) & ~7;
      const int cs = min(ncp, grp * cpg), ce = min(ncp, cs + cpg);
      for (int t = 0; t < ntile; ++t) {
        const int b = t & 1;
        mbar_wait_bounded(&bar_mma[b], ph_mma[b], err);  // tile t's products are in Tensor Memory
        if (tid == 0) {
          if (t + 2 < ntile) tma_tile(t + 2);  // buffer b is free: tile t's MMAs have completed
          if (t + 1 < ntile) mma_tile(t + 1);  // into the other accumulator, read back at t - 1
        }
        tc::fence_after();
        const int row = w + t * kMT + 32 * q + lane;  // panel row of this thread
        const bool live = row < R;
        float* pa = ab + bix(L, j0 + (live ? row : 0), j1 + cb);  // + c * ldm: A(j0 + row, j1 + cb + c)
        const uint32_t dt = tmem + ((uint32_t)(32 * q) << 16) + b * kNCH;
        for (int c0 = cs; c0 < ce; c0 += 16) {
          float d0[8], d1[8];
          tc::ld8(dt + c0, d0);
          if (c0 + 8 < ce) tc::ld8(dt + c0 + 8, d1);
          tc::wait_ld();
          float v[16];
#pragma unroll
          for (int k = 0; k < 16; ++k) v[k] = (live && c0 + k < ce && c0 + k < nc) ? ldx<CG>(pa + (int64_t)(c0 + k) * ldm) : 0.0f;
#pragma unroll
          for (int k = 0; k < 16; ++k)
            if (live && c0 + k < ce && c0 + k < nc) pa[(int64_t)(c0 + k) * ldm] = v[k] - (k < 8 ? d0[k] : d1[k - 8]);
        }
        tc::fence_before();
        __syncthreads();  // accumulator b is read before the MMAs of tile t + 2 overwrite it
      }
      if (first) stamp(tr, 4);
      first = false;
    }
    if (NR > 1) cluster_sync();
    stamp(tr, 5);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------------------
// Solve + refinement, one CTA per patch.  The FP32 working vector lives in
// shared memory; x and the FP64 residual in global memory.

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int q = 0; q < kRT / 32; ++q) s += red[q];  // same order in every thread
  return s;
}

// 16-byte global -> shared copy, L2 only (16-byte aligned addresses)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}

constexpr int kTraceSweeps = 32;  // sweeps the refinement trace records
constexpr int kFwdRows = 1;       // A21 rows per thread (warps 1..31) whose loads run ahead
constexpr int kBwdCols = 24;      // U12 columns per warp whose loads run ahead

// v <- (L U)^-1 v with the stored factors and inverses.  Every panel step
// waits for one round trip at most: the next panel's inverses are copied into
// a second shared buffer while the current panel is processed, and each
// thread loads its next A21 rows (forward) or U12 columns (backward) into
// registers as soon as it has used the current ones.
// inv_s: 2 x (2 x 32 x 32) floats of shared memory, 16-byte aligned.
// prof (trace mode, optional): thread 0 and thread 32 add the globaltimer
// time of each phase -- [0..3] thread 0 forward: wait + barrier, warp-0 work,
// barrier, row update; [4..7] thread 32 the same; [8..11] thread 0 backward:
// partial sums + prefetch, wait + barrier, warp-0 work, barrier; [12..15] thread 32
__device__ __forceinline__ long long gtime() {
  unsigned long long v;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
  return (long long)v;
}
__device__ void patch_lu_solve(const PatchJob& J, float* v, float* bz, float (*part)[33], float* inv_s,
                               long long* prof) {
  const bool pt = prof && (threadIdx.x == 0 || threadIdx.x == 32);
  const int po = threadIdx.x == 32 ? 4 : 0;
  long long tk = pt ? gtime() : 0;
  auto lap = [&](int slot) {
    if (pt) {
      const long long t1 = gtime();
      prof[slot] += t1 - tk;
      tk = t1;
    }
  };
  const BandLayout L = J.L;
  const float* __restrict__ ab = J.band;
  const int64_t ldm = L.ldb - 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int npan = J.npan;
  constexpr int kInv = 2 * kBlkW * kBlkW;  // floats per panel: Li then Ui, column-major
  auto inv_copy = [&](int p, int buf) {  // 512 threads x 16 bytes = one panel's Li and Ui
    if (p >= 0 && p < npan && tid < kInv / 4)
      cp_async16(inv_s + buf * kInv + tid * 4, J.inv + (size_t)p * kInv + tid * 4);
    cp_async_commit();
  };
  // ---- forward: per panel y1 = Li P b1, z = Ui y1, b2 -= A21 z
  const int rt = tid - 32;  // row slot of warps 1..15
  float t[kFwdRows][32];
  auto fwd_load = [&](int p) {  // this thread's A21 rows of panel p
    if (rt < 0 || p >= npan) return;
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int64_t rend = j0 + min64b(L.n - j0, (int64_t)w + L.kl);
#pragma unroll
    for (int q = 0; q < kFwdRows; ++q) {
      const int64_t i = j1 + rt + (int64_t)q * (kRT - 32);
      const float* a = ab + bix(L, i, j0);
#pragma unroll
      for (int k = 0; k < 32; ++k) t[q][k] = (i < rend && k < w) ? a[k * ldm] : 0.0f;
    }
  };
  inv_copy(0, 0);
  fwd_load(0);
  int pnext = warp == 0 && lane < J.ps[1] - J.ps[0] ? J.perm[lane] : 0;  // panel 0's permutation
  for (int p = 0; p < npan; ++p) {
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int64_t rend = j0 + min64b(L.n - j0, (int64_t)w + L.kl);
    inv_copy(p + 1, (p + 1) & 1);
    cp_async_wait_group<1>();  // this panel's inverses (this thread's part)
    __syncthreads();
    lap(po + 0);
    const float* Li = inv_s + (p & 1) * kInv;
    const float* Ui = Li + kBlkW * kBlkW;
    if (warp == 0) {
      const int pm = pnext;
      if (p + 1 < npan && lane < J.ps[p + 2] - j1) pnext = J.perm[(size_t)(p + 1) * kBlkW + lane];
      const float b = lane < w ? v[j0 + pm] : 0.0f;
      float y = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) y = fmaf(Li[k * 32 + lane], __shfl_sync(kFull, b, k), y);
      float z = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) z = fmaf(Ui[k * 32 + lane], __shfl_sync(kFull, y, k), z);
      if (lane < w) v[j0 + lane] = y;
      bz[lane] = lane < w ? z : 0.0f;
    }
    lap(po + 1);
    __syncthreads();
    lap(po + 2);
    if (rt >= 0) {
#pragma unroll
      for (int q = 0; q < kFwdRows; ++q) {
        const int64_t i = j1 + rt + (int64_t)q * (kRT - 32);
        if (i < rend) {
          float sacc = 0.0f;
#pragma unroll
          for (int k = 0; k < 32; ++k) sacc = fmaf(t[q][k], bz[k], sacc);
          v[i] -= sacc;
        }
      }
      // rows beyond kFwdRows slots (very wide bands): loaded on the spot
      for (int64_t i = j1 + rt + (int64_t)kFwdRows * (kRT - 32); i < rend; i += kRT - 32) {
        const float* a = ab + bix(L, i, j0);
        float sacc = 0.0f;
        for (int k = 0; k < w; ++k) sacc = fmaf(a[k * ldm], bz[k], sacc);
        v[i] -= sacc;
      }
      fwd_load(p + 1);
    }
    lap(po + 3);
  }
  cp_async_wait_group<0>();
  __syncthreads();
  tk = pt ? gtime() : 0;
  // ---- backward: per panel x1 = Ui (y1 - U12 x2)
  float u[kBwdCols];
  auto bwd_load = [&](int p) {  // this lane's row of U12 in this warp's columns, panel p
    if (p < 0) return;
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int C = (int)(min64b(L.n, j1 + J.kuf) - j1);
    const float* ur = ab + bix(L, j0 + lane, j1);  // U(j0 + lane, j1 + c) = ur[c * ldm]
#pragma unroll
    for (int m = 0; m < kBwdCols; ++m) {
      const int c = warp + m * (kRT / 32);
      u[m] = (lane < w && c < C) ? ur[(int64_t)c * ldm] : 0.0f;
    }
  };
  inv_copy(npan - 1, (npan - 1) & 1);
  bwd_load(npan - 1);
  for (int p = npan - 1; p >= 0; --p) {
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int C = (int)(min64b(L.n, j1 + J.kuf) - j1);
    inv_copy(p - 1, (p - 1) & 1);
    float acc = 0.0f;
#pragma unroll
    for (int m = 0; m < kBwdCols; ++m) {
      const int c = warp + m * (kRT / 32);
      if (c < C) acc = fmaf(u[m], v[j1 + c], acc);
    }
    if (lane < w) {  // columns beyond kBwdCols slots (very wide bands): loaded on the spot
      const float* ur = ab + bix(L, j0 + lane, j1);
      for (int c = warp + kBwdCols * (kRT / 32); c < C; c += kRT / 32) acc = fmaf(ur[(int64_t)c * ldm], v[j1 + c], acc);
    }
    part[warp][lane] = acc;
    bwd_load(p - 1);
    lap(8 + po);
    cp_async_wait_group<1>();  // this panel's inverses
    __syncthreads();
    lap(9 + po);
    if (warp == 0) {
      const float* Ui = inv_s + (p & 1) * kInv + kBlkW * kBlkW;
      float sum = 0.0f;
      for (int q = 0; q < kRT / 32; ++q) sum += part[q][lane];
      const float tv = lane < w ? v[j0 + lane] - sum : 0.0f;
      float x = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) x = fmaf(Ui[k * 32 + lane], __shfl_sync(kFull, tv, k), x);
      if (lane < w) v[j0 + lane] = x;
    }
    lap(10 + po);
    __syncthreads();
    lap(11 + po);
  }
  cp_async_wait_group<0>();
  __syncthreads();
}

// One column run [j0, j1) of a warp's double-float row sums (see patch_residual).
__device__ __forceinline__ void residual_run(const float* a, int64_t ldm, const float2* xs, int64_t j0, int64_t j1,
                                             float& sh, float& sl) {
  int64_t j = j0;
  for (; j + 8 <= j1; j += 8) {
    float av[8];
    float2 xv[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {  // all loads in flight
      av[m] = a[(j + m) * ldm];
      xv[m] = xs[j + m];
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      // explicit roundings: a contraction of p into t would break TwoSum
      const float p = __fmul_rn(av[m], xv[m].x);
      const float e = fmaf(av[m], xv[m].y, fmaf(av[m], xv[m].x, -p));
      const float t = __fadd_rn(sh, p);
      const float z = __fsub_rn(t, sh);
      sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
      sh = t;
    }
  }
  for (; j < j1; ++j) {
    const float av = a[j * ldm];
    const float2 xv = xs[j];
    const float p = __fmul_rn(av, xv.x);
    const float e = fmaf(av, xv.y, fmaf(av, xv.x, -p));
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
    sh = t;
  }
}

// res = rhs - A0 x (A0: the unfactored FP32 band); returns |res|.  The
// products are formed on the FP32 pipe in double-float arithmetic: x = xh + xl
// (two floats, split once per sweep), a xh = p + e exactly (FMA), and the row
// sum kept as an unevaluated float pair (Knuth's TwoSum for the high part);
// the pair's error (~2^-44 of the row's term magnitudes) is far below the
// refinement tolerance, at a sixth of the cost of FP64 FMAs on this GPU.
// A warp takes 32 rows and walks, in increasing order, only the columns their
// control points couple to: an unknown of control point (s1, s2) couples only
// to the unknowns of points (s1 +- 2, s2 +- 2) (biquadratic elements).  The
// rows' points run from (s1a, s2a) to (s1b, s2b) in lexicographic order, so
// grid row g is coupled to points [s1a - 2, W) through the points of grid row
// s2a (if |g - s2a| <= 2), to [0, s1b + 2] through those of grid row s2b (if
// |g - s2b| <= 2), and to the whole grid row through any grid row between
// them: at most two runs per grid row.  The columns skipped hold stored
// zeros, whose products leave the pair unchanged: the sums equal a walk of
// the whole band window.
__device__ double patch_residual(const PatchJob& J, const float2* xs, double* red) {
  const BandLayout L = J.L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ldm = L.ldb - 1;
  double ss = 0.0;
  // With nb >= 32 every (i, j) of the band window [rb - ku, rb + 32 + kl) lies
  // inside the band's storage, where the entries outside the band are stored
  // zeros, so A0(i, j) = a[j * ldm + lane] with a at row rb of column 0 needs
  // no guard but i < n; the runs are clipped to that window.
  for (int64_t rb = (int64_t)warp * 32; rb < L.n; rb += kRT) {
    const int64_t i = rb + lane;
    const bool live = i < L.n;
    const int64_t jlo = rb - L.ku > 0 ? rb - L.ku : 0;
    const int64_t jhi = min64b(L.n, rb + 32 + L.kl);
    const float* a = J.band0 + L.off + (live ? i : rb);  // + j * ldm: A0(i, j)
    float sh = 0.0f, sl = 0.0f;
    if (J.node_first) {
      const int W = J.num1np, H = J.num2np;
      const int na = J.unk_node[rb], nb = J.unk_node[min64b(rb + 31, L.n - 1)];
      const int s1a = na % W, s2a = na / W, s1b = nb % W, s2b = nb / W;
      for (int g = max(s2a - 2, 0); g <= min(s2b + 2, H - 1); ++g) {
        // the runs [c0, c1] (and [d0, d1] after it) of grid row g, in points
        int c0 = 0, c1 = -1, d0 = 0, d1 = -1;
        const bool fa = abs(g - s2a) <= 2, fb = abs(g - s2b) <= 2;
        const bool fm = s2b - s2a >= 2 && g >= s2a - 1 && g <= s2b + 1;  // a grid row strictly between
        if (s2a == s2b) {
          c0 = max(s1a - 2, 0);
          c1 = min(s1b + 2, W - 1);
        } else if (fm || (fa && fb && s1b + 3 >= s1a - 2)) {
          c1 = W - 1;
        } else {
          if (fb) c1 = min(s1b + 2, W - 1);  // [0, s1b + 2] comes first
          if (fa) {
            d0 = max(s1a - 2, 0);
            d1 = W - 1;
          }
        }
        for (int r = 0; r < 2; ++r) {
          const int e0 = r ? d0 : c0, e1 = r ? d1 : c1;
          if (e1 < e0) continue;
          const int64_t j0 = max((int64_t)J.node_first[g * W + e0], jlo);
          const int64_t j1 = min64b((int64_t)J.node_first[g * W + e1 + 1], jhi);
          if (j0 < j1) residual_run(a, ldm, xs, j0, j1, sh, sl);
        }
      }
    } else {
      residual_run(a, ldm, xs, jlo, jhi, sh, sl);
    }
    if (live) {
      const double r = J.rhs[i] - ((double)sh + (double)sl);
      J.res[i] = r;
      ss = fma(r, r, ss);
    }
  }
  return sqrt(block_sum(ss, red));
}

__global__ void __launch_bounds__(kRT, 1) patch_refine_kernel(const PatchJob* __restrict__ jobs,
                                                             const int* __restrict__ order, int max_sweeps,
                                                             double tol) {
  const PatchJob& J = jobs[order[blockIdx.x]];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* v = reinterpret_cast<float*>(smem_raw);  // [n]
  __shared__ float bz[32];  // zero beyond the panel width
  __shared__ float part[kRT / 32][33];
  __shared__ __align__(16) float inv_s[2 * 2 * kBlkW * kBlkW];  // double-buffered panel inverses
  __shared__ double red[kRT / 32];
  const int tid = threadIdx.x;
  const int64_t n = J.L.n;
  int* stat = J.stat;  // [0] status, [1] sweeps
  float2* xs = J.xs;   // x split into two floats
  if (J.info[1] != 0 || J.info[0] != 0) {  // a bounded wait ran out, or a node block had no usable pivot
    if (tid == 0) {
      stat[0] = J.info[1] != 0 ? MAFEM_ERR_CUDA : MAFEM_ZERO_PIVOT;
      stat[1] = 0;
    }
    return;
  }
  double ss = 0.0;
  for (int64_t i = tid; i < n; i += kRT) {
    const double r = J.rhs[i];
    J.res[i] = r;
    J.x[i] = 0.0;
    ss = fma(r, r, ss);
  }
  const double r0 = sqrt(block_sum(ss, red));
  // trace: per sweep 4 stamps after J.trace's 6 per panel -- [0] sweep start,
  // [1] substitutions done, [2] x updated and norms formed, [3] residual done
  long long* tr = J.trace ? J.trace + (size_t)J.npan * 6 : nullptr;
  // Stop when the error left in x is small against x.  After sweep k that
  // error is about the next correction, rho |d_k| with rho = |d_k| / |d_k-1|
  // the sweeps' contraction: stop once rho |d_k| <= tol |x| while the sweeps
  // contract (rho <= 1/2), or once |d_k| <= tol |x| itself.  A bound on the
  // forward error of x whatever the conditioning, where a residual test would
  // accept a large error in x on an ill-conditioned tangent; the residual
  // after the final sweep is never needed.
  int status = MAFEM_OK, sweeps = 0;
  double rn = r0, prev_dn = INFINITY;
  if (r0 > 0.0) {
    status = MAFEM_REFINE_STALLED;
    for (int k = 0; k < max_sweeps; ++k) {
      long long* trk = tr && k < kTraceSweeps ? tr + 4 * k : nullptr;
      stamp(trk, 0);
      const double sc = 1.0 / rn;
      for (int64_t i = tid; i < n; i += kRT) v[i] = (float)(J.res[i] * sc);
      __syncthreads();
      patch_lu_solve(J, v, bz, part, inv_s, tr && k == 0 ? tr + 4 * kTraceSweeps : nullptr);
      stamp(trk, 1);
      double dd = 0.0, xx = 0.0;
      for (int64_t i = tid; i < n; i += kRT) {
        const double d = rn * (double)v[i];
        const double x = J.x[i] + d;
        J.x[i] = x;
        const float xh = (float)x;
        xs[i] = make_float2(xh, (float)(x - (double)xh));
        dd = fma(d, d, dd);
        xx = fma(x, x, xx);
      }
      const double dn = sqrt(block_sum(dd, red));
      const double xn = sqrt(block_sum(xx, red));
      stamp(trk, 2);
      sweeps = k + 1;
      if (!isfinite(dn) || !isfinite(xn)) {
        status = MAFEM_NAN_DETECTED;
        break;
      }
      const double rho = dn / prev_dn;  // 0 after the first sweep (prev_dn infinite)
      if (dn <= tol * xn || (k >= 1 && rho <= 0.5 && rho * dn <= tol * xn)) {
        status = MAFEM_OK;
        break;
      }
      rn = patch_residual(J, xs, red);  // block_sum orders the x / xs writes before it
      stamp(trk, 3);
      if (tr && tid == 0 && k < kTraceSweeps)  // trace: the residual after each sweep, relative to |r0|
        tr[4 * kTraceSweeps + 16 + k] = __double_as_longlong(rn / r0);
      if (!isfinite(rn)) {
        status = MAFEM_NAN_DETECTED;
        break;
      }
      // A residual at FP64 level (<= min(tol, 1e-10) |r0|) also ends the solve:
      // on large, stiff tangents the relative correction has a rounding floor
      // (about 1e-9 on the 64 x 64 patch) that a tight tol would never reach.
      if (rn <= fmin(tol, 1e-10) * r0) {
        status = MAFEM_OK;
        break;
      }
      if (k >= 3 && dn > 0.5 * prev_dn) {  // no longer contracting
        // at the rounding floor (the correction a small part of x) the
        // solution is as accurate as the factors allow: accept it
        if (dn <= 1e-8 * xn) status = MAFEM_OK;
        break;
      }
      prev_dn = dn;
    }
  }
  if (tid == 0) {
    stat[0] = status;
    stat[1] = sweeps;
  }
}

int patch_chunk_cols() { return kNCH; }

// The split-A21 buffer as a 3-D tensor (k % 4, row, k / 4) of FP32 with strides
// 16 bytes (rows) and 2 a21_rows x 16 bytes (k-quad planes); one 4 x 128 x 8 box
// is one M tile in the MMA's K-major core-matrix layout (k-quad planes 2 KB
// apart, rows 16 bytes apart).
bool patch_a21_map(PatchJob& J) {
  using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = reinterpret_cast<EncodeFn>(fn);
  }
  const cuuint64_t dims[3] = {4, (cuuint64_t)2 * J.a21_rows, 8};
  const cuuint64_t strides[2] = {16, (cuuint64_t)2 * J.a21_rows * 16};
  const cuuint32_t box[3] = {4, (cuuint32_t)kMT, 8};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(&J.a21_map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, J.a21, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int patch_solve_setup() {
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const int dyn = cap - 20 * 1024;  // room for the kernels' static shared memory (refine: ~19 KB)
  if (cudaFuncSetAttribute(patch_factor_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_factor_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_factor_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
    return 0;
  return dyn;
}

int patch_cluster_ctas(int kuf) { return kuf > 2 * kNCH ? 4 : kuf > kNCH ? 2 : 1; }

static cudaError_t launch_factor(const PatchJob* d_jobs, const int* d_order, int njobs, int nr, size_t smem,
                                 cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (nr == 1) {
    patch_factor_kernel<1><<<njobs, kPT, smem, st>>>(d_jobs, d_order);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nr * njobs));
  cfg.blockDim = dim3(kPT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)nr;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return nr == 4 ? cudaLaunchKernelEx(&cfg, patch_factor_kernel<4>, d_jobs, d_order)
                 : cudaLaunchKernelEx(&cfg, patch_factor_kernel<2>, d_jobs, d_order);
}

cudaError_t patch_solve_stage(const PatchJob* d_jobs, const int* d_order, int njobs, int nr, size_t smem_factor,
                              size_t smem_refine, int max_sweeps, double tol, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (smem_factor) {
    const cudaError_t e = launch_factor(d_jobs, d_order, njobs, nr, smem_factor, st);
    if (e != cudaSuccess) return e;
  }
  if (smem_refine) patch_refine_kernel<<<njobs, kRT, smem_refine, st>>>(d_jobs, d_order, max_sweeps, tol);
  return cudaGetLastError();
}

// ---- autotuning: the factorisation's time per cluster size -------------------------
// A synthetic band of the job's shape: entries of the band uniform in [-1, 1)
// (a hash of i and j), the diagonal kl + ku + 2 (diagonally dominant, so every
// node block keeps its own pivots), the pivoting fill rows zero.  The
// factorisation's time does not depend on the values.
__global__ void patch_fill_synthetic_kernel(const PatchJob* __restrict__ jobs, const int* __restrict__ order) {
  const PatchJob& J = jobs[order[0]];
  const BandLayout L = J.L;
  const int64_t total = L.ldb * L.n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / L.ldb, i = j + (idx - j * L.ldb) - L.off;
    float v = 0.0f;
    if (i >= 0 && i < L.n && i - j <= L.kl && j - i <= L.ku) {
      uint32_t h = (uint32_t)i * 73856093u ^ (uint32_t)j * 19349663u;
      h ^= h >> 13;
      h *= 0x5bd1e995u;
      h ^= h >> 15;
      v = i == j ? (float)(L.kl + L.ku + 2) : (float)(h & 0xffffu) * (1.0f / 32768.0f) - 1.0f;
    }
    J.band[idx] = v;
  }
}

cudaError_t patch_time_factor(const PatchJob* d_jobs, const int* d_order1, int nr, size_t smem, cudaStream_t st,
                              float* ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // the second run is timed
    patch_fill_synthetic_kernel<<<1024, 256, 0, st>>>(d_jobs, d_order1);
    e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) e = launch_factor(d_jobs, d_order1, 1, nr, smem, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return e;
}

int patch_solve_launches(int n4, int n2, int njobs) {
  const int groups = (n4 > 0) + (n2 > 0) + (njobs - n4 - n2 > 0);
  return groups + (groups > 1 ? 2 : 1);  // the factor launches and one refinement per stream
}

cudaError_t patch_solve(const PatchJob* d_jobs, const int* d_order, int n4, int n2, int njobs, size_t smem_factor,
                        size_t smem_refine, int max_sweeps, double tol, cudaStream_t st, cudaStream_t st2,
                        cudaEvent_t ev_fork, cudaEvent_t ev_join) {
  if (njobs <= 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  // the groups in launch order: four-CTA clusters, two-CTA clusters, single
  // CTAs; the first non-empty group on st, the others one after the other on
  // st2 beside it (their chains are the shorter ones).  Each stream refines its
  // own patches as soon as their factors are done, so the refinement of one
  // group overlaps the factorisations of the other.
  const int cnt[3] = {n4, n2, njobs - n4 - n2}, nrs[3] = {4, 2, 1};
  int first = 0;
  while (first < 3 && cnt[first] == 0) ++first;
  const bool fork = cnt[first] < njobs;
  if (fork) {
    e = cudaEventRecord(ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, ev_fork, 0);
  }
  int off = 0;
  for (int g = 0; g < 3 && e == cudaSuccess; ++g) {
    if (cnt[g] == 0) continue;
    e = launch_factor(d_jobs, d_order + off, cnt[g], nrs[g], smem_factor, g == first ? st : st2);
    off += cnt[g];
    if (g == first && e == cudaSuccess) {
      patch_refine_kernel<<<cnt[g], kRT, smem_refine, st>>>(d_jobs, d_order, max_sweeps, tol);
      e = cudaGetLastError();
    }
  }
  if (fork && e == cudaSuccess) {
    patch_refine_kernel<<<njobs - cnt[first], kRT, smem_refine, st2>>>(d_jobs, d_order + cnt[first], max_sweeps,
                                                                        tol);
    e = cudaGetLastError();
  }
  if (fork && e == cudaSuccess) e = cudaEventRecord(ev_join, st2);
  if (fork && e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_join, 0);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace mafem
