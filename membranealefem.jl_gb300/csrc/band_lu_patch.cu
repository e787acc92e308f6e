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

namespace mafem {

constexpr int kPT = 512;   // threads per CTA of the factorisation (16 warps)
constexpr int kRT = 768;   // threads per CTA of the refinement (24 warps)
constexpr int kPCH = 288;      // trailing columns per chunk (a 32 x 32 patch's ~550 in two)
constexpr int kYS = kPCH + 8;  // row stride of Y (uint2 hi/lo pairs) in shared memory
constexpr int kIS = 36;    // shared-memory row stride of the 32 x 32 inverses (16-byte rows)

// panel column stride in shared memory: >= 32 + kl, == 8 mod 32 (conflict-free MMA fragments)
__host__ __device__ inline int patch_rp(int kl) { return ((kBlkW + kl + 23) & ~31) + 8; }

size_t patch_factor_smem(int kl) {
  return sizeof(float) * ((size_t)kBlkW * patch_rp(kl) + 2 * (size_t)kBlkW * kYS + 3 * (size_t)kBlkW * kIS);
}

// D += A B on the tensor cores: A 16 x 8 (row), B 8 x 8 (col), TF32 in, FP32 accumulate
__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
// x = hi + lo with hi, lo TF32 (round to nearest): the 3xTF32 split
__device__ __forceinline__ void split_tf32(float x, unsigned& hi, unsigned& lo) {
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
  const float r = x - __uint_as_float(hi);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
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

// trace (J.trace, optional): per panel 6 globaltimer stamps -- [0] start,
// [1] diagonal block factored, [2] panel staged and inverses formed,
// [3] U12 / Y of the first chunk, [4] its trailing update, [5] panel done
//
// NR = 2: a patch on a cluster of two CTAs (launched with cluster dims (2,1,1)).
// Rank 0 factors the diagonal block; both ranks stage the panel and form the
// inverses; rank r updates the trailing chunks r, r + 2, ... .  A column moves
// from rank 1's chunks to rank 0's as the panels advance, so every band read
// goes to L2 (ld.global.cg) and each panel ends at a cluster barrier; the
// factored block is published by another after the panel factorisation.  Both
// ranks run the same panel loop, so every barrier is reached by all threads of
// both CTAs.
template <int NR>
__global__ void __launch_bounds__(kPT, 1) patch_factor_kernel(const PatchJob* __restrict__ jobs,
                                                             const int* __restrict__ order) {
  constexpr bool CG = NR > 1;
  const int rank = (int)(blockIdx.x % NR);
  const PatchJob& J = jobs[order[blockIdx.x / NR]];
  const BandLayout L = J.L;
  float* __restrict__ ab = J.band;
  const int Rp = patch_rp(L.kl);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* Lp = reinterpret_cast<float*>(smem_raw);  // [32][Rp]: A(j0 + r, j0 + c) at Lp[c * Rp + r]
  uint2* Ys = reinterpret_cast<uint2*>(Lp + (size_t)kBlkW * Rp);  // [32][kYS]: Y = Mi P A12 split hi/lo (TF32)
  float* Li = reinterpret_cast<float*>(Ys + kBlkW * kYS);          // [32][kIS]
  float* Ui = Li + kBlkW * kIS;
  float* Mi = Ui + kBlkW * kIS;
  __shared__ float s_l[2][32];
  __shared__ int s_p[2];
  __shared__ int sp[32];
  __shared__ float rd[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t ldm = L.ldb - 1;  // A(i, j + 1) - A(i, j) in the band array

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
    stamp(tr, 2);

    // 3. trailing columns [j1, j1 + C) in chunks of kPCH
    const int nr = R - w;
    for (int cb = rank * kPCH; cb < C; cb += NR * kPCH) {
      const int nc = min(kPCH, C - cb);
      // U12 = Li P A12 and Y = Mi P A12: one thread per column, the column in registers
      for (int c = tid; c < nc; c += kPT) {
        const int64_t col = j1 + cb + c;
        float* dst = ab + bix(L, j0, col);  // A(j0 + r, col) = dst[r]
        float a[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) a[k] = k < w ? ldx<CG>(dst + sp[k]) : 0.0f;
#pragma unroll 2
        for (int r = 0; r < 32; ++r) {
          if (r < w) {  // block-uniform
            const float4* l4 = reinterpret_cast<const float4*>(Li + r * kIS);
            const float4* m4 = reinterpret_cast<const float4*>(Mi + r * kIS);
            float u = 0.0f, y = 0.0f;
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
            dst[r] = u;  // U12
            uint2 yy;
            split_tf32(y, yy.x, yy.y);
            Ys[r * kYS + c] = yy;
          }
        }
      }
      __syncthreads();
      if (cb == 0) stamp(tr, 3);
      // A22 -= A21 Y on the tensor cores, 3xTF32 (a b ~ ah bh + ah bl + al bh:
      // FP32-level accuracy).  A warp task is a 16-row strip of A22 over half
      // of the chunk's column tiles: the strip's A21 fragments (negated, so the
      // MMAs accumulate A22 - A21 Y) are split once into registers; Y comes
      // pre-split from shared memory; the next column tile's A22 values are
      // loaded while the current tile's MMAs run.  Fragment layouts
      // (m16n8k8, g = lane / 4, t = lane % 4): A a0 (g, t), a1 (g + 8, t),
      // a2 (g, t + 4), a3 (g + 8, t + 4); B b0 (t, g), b1 (t + 4, g);
      // C c0 (g, 2t), c1 (g, 2t + 1), c2 (g + 8, 2t), c3 (g + 8, 2t + 1).
      {
        const int g = lane >> 2, t4 = lane & 3;
        const int nrs = (nr + 15) >> 4, nct = (nc + 31) >> 5;
        const int nhalf = nct > 1 ? 2 : 1;
        const int ksteps = (w + 7) >> 3;
        for (int task = warp; task < nrs * nhalf; task += kPT / 32) {
          const int rs = task / nhalf, hf = task - rs * nhalf;
          const int ct0 = hf * ((nct + 1) >> 1), ct1 = hf + 1 == nhalf ? nct : (nct + 1) >> 1;
          const int r0 = w + rs * 16;
          const int ra = r0 + g, rb = r0 + g + 8;
          const bool oka = ra < R, okb = rb < R;
          unsigned ah[4][4], al[4][4];
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const int k0 = ks * 8 + t4, k1 = k0 + 4;
            const int ca = min(ra, R - 1), cbr = min(rb, R - 1);
            const float x0 = k0 < w ? -Lp[k0 * Rp + ca] : 0.0f;
            const float x1 = k0 < w ? -Lp[k0 * Rp + cbr] : 0.0f;
            const float x2 = k1 < w ? -Lp[k1 * Rp + ca] : 0.0f;
            const float x3 = k1 < w ? -Lp[k1 * Rp + cbr] : 0.0f;
            split_tf32(x0, ah[ks][0], al[ks][0]);
            split_tf32(x1, ah[ks][1], al[ks][1]);
            split_tf32(x2, ah[ks][2], al[ks][2]);
            split_tf32(x3, ah[ks][3], al[ks][3]);
          }
          // rows ra / rb of the chunk's first column: A(j0 + r, j1 + cb) = row pointer
          float* pa = ab + bix(L, j0 + ra, j1 + cb);
          float* pb = ab + bix(L, j0 + rb, j1 + cb);
          auto load_c = [&](int ct, float (&c)[4][4]) {
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
              const int cc = ct * 32 + nt * 8 + 2 * t4;
              const bool c0k = cc < nc, c1k = cc + 1 < nc;
              c[nt][0] = oka && c0k ? ldx<CG>(pa + (int64_t)cc * ldm) : 0.0f;
              c[nt][1] = oka && c1k ? ldx<CG>(pa + (int64_t)(cc + 1) * ldm) : 0.0f;
              c[nt][2] = okb && c0k ? ldx<CG>(pb + (int64_t)cc * ldm) : 0.0f;
              c[nt][3] = okb && c1k ? ldx<CG>(pb + (int64_t)(cc + 1) * ldm) : 0.0f;
            }
          };
          float acc[4][4], nxt[4][4];
          if (ct0 < ct1) load_c(ct0, nxt);
          for (int ct = ct0; ct < ct1; ++ct) {
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
              for (int e = 0; e < 4; ++e) acc[nt][e] = nxt[nt][e];
            if (ct + 1 < ct1) load_c(ct + 1, nxt);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              if (ks >= ksteps) break;  // warp-uniform; the unrolled index keeps ah / al in registers
              const int k0 = ks * 8 + t4;
#pragma unroll
              for (int nt = 0; nt < 4; ++nt) {
                const int c = ct * 32 + nt * 8 + g;
                // rows k >= w of Y are stale shared memory: mask them (0 * NaN would not vanish)
                const uint2 y0 = k0 < w ? Ys[k0 * kYS + c] : make_uint2(0u, 0u);
                const uint2 y1 = k0 + 4 < w ? Ys[(k0 + 4) * kYS + c] : make_uint2(0u, 0u);
                const unsigned bh[2] = {y0.x, y1.x}, bl[2] = {y0.y, y1.y};
                mma_tf32(acc[nt], al[ks], bh);
                mma_tf32(acc[nt], ah[ks], bl);
                mma_tf32(acc[nt], ah[ks], bh);
              }
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
              const int cc = ct * 32 + nt * 8 + 2 * t4;
              const bool c0k = cc < nc, c1k = cc + 1 < nc;
              if (oka && c0k) pa[(int64_t)cc * ldm] = acc[nt][0];
              if (oka && c1k) pa[(int64_t)(cc + 1) * ldm] = acc[nt][1];
              if (okb && c0k) pb[(int64_t)cc * ldm] = acc[nt][2];
              if (okb && c1k) pb[(int64_t)(cc + 1) * ldm] = acc[nt][3];
            }
          }
        }
      }
      __syncthreads();
      if (cb == 0) stamp(tr, 4);
    }
    if (NR > 1) cluster_sync();
    stamp(tr, 5);
  }
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

// res = rhs - A0 x (A0: the unfactored FP32 band); returns |res|.  The
// products are formed on the FP32 pipe in double-float arithmetic: x = xh + xl
// (two floats, split once per sweep), a xh = p + e exactly (FMA), and the row
// sum kept as an unevaluated float pair (Knuth's TwoSum for the high part);
// the pair's error (~2^-44 of the row's term magnitudes) is far below the
// refinement tolerance, at a sixth of the cost of FP64 FMAs on this GPU.
__device__ double patch_residual(const PatchJob& J, const float2* xs, double* red) {
  const BandLayout L = J.L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ldm = L.ldb - 1;
  double ss = 0.0;
  // A warp takes 32 rows and walks the columns j of their band window; with
  // nb >= 32 every (i, j) it visits lies inside the band's storage, where the
  // entries outside the band are stored zeros, so A0(i, j) = a[j * ldm + lane]
  // with a at row rb of column 0 needs no guard but i < n.
  for (int64_t rb = (int64_t)warp * 32; rb < L.n; rb += kRT) {
    const int64_t i = rb + lane;
    const bool live = i < L.n;
    const int64_t jlo = rb - L.ku > 0 ? rb - L.ku : 0;
    const int64_t jhi = min64b(L.n, rb + 32 + L.kl);
    const float* a = J.band0 + L.off + (live ? i : rb);  // + j * ldm: A0(i, j)
    float sh = 0.0f, sl = 0.0f;
    int64_t j = jlo;
    for (; j + 8 <= jhi; j += 8) {
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
    for (; j < jhi; ++j) {
      const float av = a[j * ldm];
      const float2 xv = xs[j];
      const float p = __fmul_rn(av, xv.x);
      const float e = fmaf(av, xv.y, fmaf(av, xv.x, -p));
      const float t = __fadd_rn(sh, p);
      const float z = __fsub_rn(t, sh);
      sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
      sh = t;
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
  if (J.info[0] != 0) {  // a node block without a usable pivot
    if (tid == 0) {
      stat[0] = MAFEM_ZERO_PIVOT;
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
  // Stop when the last correction is small against x: |d| <= tol |x| bounds
  // the forward error of x (about rho |d| with rho < 1 the sweep's
  // contraction) whatever the conditioning, where a residual test would
  // accept a large error in x on an ill-conditioned tangent.  The residual
  // after the final sweep is then never needed.
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
      if (dn <= tol * xn) {
        status = MAFEM_OK;
        break;
      }
      if (k >= 3 && dn > 0.5 * prev_dn) break;  // stalled
      prev_dn = dn;
      rn = patch_residual(J, xs, red);  // block_sum orders the x / xs writes before it
      stamp(trk, 3);
      if (!isfinite(rn)) {
        status = MAFEM_NAN_DETECTED;
        break;
      }
      if (rn == 0.0) {
        status = MAFEM_OK;
        break;
      }
    }
  }
  if (tid == 0) {
    stat[0] = status;
    stat[1] = sweeps;
  }
}

int patch_chunk_cols() { return kPCH; }

int patch_solve_setup() {
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const int dyn = cap - 20 * 1024;  // room for the kernels' static shared memory (refine: ~19 KB)
  if (cudaFuncSetAttribute(patch_factor_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_factor_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
    return 0;
  return dyn;
}

static cudaError_t launch_factor(const PatchJob* d_jobs, const int* d_order, int njobs, int nr, size_t smem,
                                 cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  if (nr == 1) {
    patch_factor_kernel<1><<<njobs, kPT, smem, st>>>(d_jobs, d_order);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(2 * njobs));
  cfg.blockDim = dim3(kPT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, patch_factor_kernel<2>, d_jobs, d_order);
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

cudaError_t patch_solve(const PatchJob* d_jobs, const int* d_order, int nbig, int njobs, size_t smem_factor,
                        size_t smem_refine, int max_sweeps, double tol, cudaStream_t st, cudaStream_t st2,
                        cudaEvent_t ev_fork, cudaEvent_t ev_join) {
  if (njobs <= 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  const int nsmall = njobs - nbig;
  if (nsmall > 0 && nbig > 0) {  // the single-CTA patches beside the clusters, on the second stream
    e = cudaEventRecord(ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, ev_fork, 0);
    if (e == cudaSuccess) e = launch_factor(d_jobs, d_order, nbig, 2, smem_factor, st);
    if (e == cudaSuccess) e = launch_factor(d_jobs, d_order + nbig, nsmall, 1, smem_factor, st2);
    if (e == cudaSuccess) e = cudaEventRecord(ev_join, st2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_join, 0);
  } else {
    e = launch_factor(d_jobs, d_order, njobs, nbig > 0 ? 2 : 1, smem_factor, st);
  }
  if (e != cudaSuccess) return e;
  patch_refine_kernel<<<njobs, kRT, smem_refine, st>>>(d_jobs, d_order, max_sweeps, tol);
  return cudaGetLastError();
}

}  // namespace mafem
