// band_lu_patch.cu -- many patches' FP32 linear solves in two launches.
//
// The batched FP32 form solves K Δu = -r for every patch of a batch with one
// CTA per patch: `patch_factor_kernel` factors each patch's FP32 band with
// node-block pivoting (the same factors as band_lu_blk.cu: L11\U11 with the
// panel's rows permuted, U12 = L11^-1 P A12, raw A21, rdiag = 1/U(j,j),
// perm_all[p * 32 + i]), and `patch_refine_kernel` runs the FP32 triangular
// solves and FP64 iterative refinement x += LU^-1 (r - A0 x) until
// |r - A0 x| <= tol |r| -- the role of `K_gl \ r_gl` (FiniteElement.jl:38).
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

constexpr int kPT = 512;   // threads per CTA (16 warps)
constexpr int kPCH = 512;  // trailing columns per chunk: one thread per column for U12 and Y
constexpr int kIS = 36;    // shared-memory row stride of the 32 x 32 inverses (16-byte rows)

__host__ __device__ inline int patch_rp(int kl) { return (kBlkW + kl + 3) & ~3; }

size_t patch_factor_smem(int kl) {
  return sizeof(float) * ((size_t)kBlkW * patch_rp(kl) + (size_t)kBlkW * kPCH + 3 * (size_t)kBlkW * kIS);
}
size_t patch_refine_smem(int64_t n) { return sizeof(float) * (size_t)n; }

__global__ void __launch_bounds__(kPT, 1) patch_factor_kernel(const PatchJob* __restrict__ jobs,
                                                             const int* __restrict__ order) {
  const PatchJob& J = jobs[order[blockIdx.x]];
  const BandLayout L = J.L;
  float* __restrict__ ab = J.band;
  const int Rp = patch_rp(L.kl);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* Lp = reinterpret_cast<float*>(smem_raw);  // [32][Rp]: A(j0 + r, j0 + c) at Lp[c * Rp + r]
  float* Ys = Lp + (size_t)kBlkW * Rp;              // [32][kPCH]: Y = Mi P A12 (row k at Ys + k * kPCH)
  float* Li = Ys + kBlkW * kPCH;                    // [32][kIS]
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

    // 1. the diagonal block
    if (warp < kPanelWarps) blk_panel_factor<float, false>(ab, L, j0, w, J.blk_end, perm, J.rdiag, J.info, s_l, s_p);
    __syncthreads();

    // 2. panel columns (all copies in flight at once), then the inverses of
    //    L11 and U11 by column, each lane's column in registers
    for (int c = 0; c < w; ++c) {
      const float* src = ab + bix(L, j0, j0 + c);
      for (int r = tid; r < R; r += kPT) cp_async(Lp + c * Rp + r, src + r);
    }
    if (tid < kBlkW) {
      sp[tid] = tid < w ? perm[tid] : 0;
      rd[tid] = tid < w ? J.rdiag[j0 + tid] : 0.0f;
    }
    cp_async_wait_all();
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
    float* inv = J.inv + (size_t)p * 2 * kBlkW * kBlkW;  // Li then Ui, row-major 32 x 32
    for (int idx = tid; idx < kBlkW * kBlkW; idx += kPT) {
      const int i = idx >> 5, c = idx & 31;
      float s = 0.0f;
      for (int k = max(i, c); k < w; ++k) s = fmaf(Ui[i * kIS + k], Li[k * kIS + c], s);
      Mi[i * kIS + c] = s;
      inv[idx] = Li[i * kIS + c];
      inv[kBlkW * kBlkW + idx] = Ui[i * kIS + c];
    }
    __syncthreads();

    // 3. trailing columns [j1, j1 + C) in chunks of kPCH
    const int nr = R - w;
    for (int cb = 0; cb < C; cb += kPCH) {
      const int nc = min(kPCH, C - cb);
      // U12 = Li P A12 and Y = Mi P A12: one thread per column, the column in registers
      if (tid < nc) {
        const int64_t col = j1 + cb + tid;
        float* dst = ab + bix(L, j0, col);  // A(j0 + r, col) = dst[r]
        float a[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) a[k] = k < w ? dst[sp[k]] : 0.0f;
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
            Ys[r * kPCH + tid] = y;
          }
        }
      }
      __syncthreads();
      // A22 -= A21 Y: warp tasks of 128 rows x 16 columns; lane owns rows
      // lane + 32 q (q < 4), so every load and store instruction of the warp
      // covers 32 consecutive rows of one column; per k: 4 A21 values and 4
      // float4 broadcasts of Y for 64 FMAs
      const int nrb = (nr + 127) >> 7, ncb = (nc + 15) >> 4;
      for (int t = warp; t < nrb * ncb; t += kPT / 32) {
        const int rb = t / ncb, c0 = (t - rb * ncb) * 16;
        const int i0 = w + rb * 128 + lane;
        float acc[4][16];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = i0 + 32 * q;
          const float* a0 = ab + bix(L, j0 + i, j1 + cb + c0);
#pragma unroll
          for (int m = 0; m < 16; ++m) acc[q][m] = (i < R && c0 + m < nc) ? a0[m * ldm] : 0.0f;
        }
        for (int k = 0; k < w; ++k) {
          float a[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) a[q] = Lp[k * Rp + min(i0 + 32 * q, R - 1)];
          const float4* y4 = reinterpret_cast<const float4*>(Ys + k * kPCH + c0);
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            const float4 y = y4[m];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              acc[q][4 * m + 0] = fmaf(-a[q], y.x, acc[q][4 * m + 0]);
              acc[q][4 * m + 1] = fmaf(-a[q], y.y, acc[q][4 * m + 1]);
              acc[q][4 * m + 2] = fmaf(-a[q], y.z, acc[q][4 * m + 2]);
              acc[q][4 * m + 3] = fmaf(-a[q], y.w, acc[q][4 * m + 3]);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = i0 + 32 * q;
          float* a0 = ab + bix(L, j0 + i, j1 + cb + c0);
#pragma unroll
          for (int m = 0; m < 16; ++m)
            if (i < R && c0 + m < nc) a0[m * ldm] = acc[q][m];
        }
      }
      __syncthreads();
    }
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
  for (int q = 0; q < kPT / 32; ++q) s += red[q];  // same order in every thread
  return s;
}

// row `lane` of a 32 x 32 row-major matrix in global memory, as registers
__device__ __forceinline__ void load_row32(const float* m, int lane, float r[32]) {
  const float4* q = reinterpret_cast<const float4*>(m + lane * 32);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float4 t = q[k];
    r[4 * k] = t.x;
    r[4 * k + 1] = t.y;
    r[4 * k + 2] = t.z;
    r[4 * k + 3] = t.w;
  }
}

// v <- (L U)^-1 v with the stored factors and inverses
__device__ void patch_lu_solve(const PatchJob& J, float* v, float* bz, float (*part)[33]) {
  const BandLayout L = J.L;
  const float* __restrict__ ab = J.band;
  const int64_t ldm = L.ldb - 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // forward: per panel y1 = Li P b1, z = Ui y1, b2 -= A21 z
  for (int p = 0; p < J.npan; ++p) {
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int R = (int)min64b(L.n - j0, (int64_t)w + L.kl);
    if (warp == 0) {
      const float* inv = J.inv + (size_t)p * 2 * kBlkW * kBlkW;
      float li[32], ui[32];
      load_row32(inv, lane, li);
      load_row32(inv + kBlkW * kBlkW, lane, ui);
      const float b = lane < w ? v[j0 + J.perm[(size_t)p * kBlkW + lane]] : 0.0f;
      float y = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) y = fmaf(li[k], __shfl_sync(kFull, b, k), y);
      float z = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) z = fmaf(ui[k], __shfl_sync(kFull, y, k), z);
      if (lane < w) v[j0 + lane] = y;
      bz[lane] = lane < w ? z : 0.0f;
    }
    __syncthreads();
    for (int64_t i = j1 + tid; i < j0 + R; i += kPT) {
      const float* a = ab + bix(L, i, j0);
      float t[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) t[k] = k < w ? a[k * ldm] : 0.0f;  // all loads in flight
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) s = fmaf(t[k], bz[k], s);
      v[i] -= s;
    }
    __syncthreads();
  }
  // backward: per panel x1 = Ui (y1 - U12 x2)
  for (int p = J.npan - 1; p >= 0; --p) {
    const int64_t j0 = J.ps[p], j1 = J.ps[p + 1];
    const int w = (int)(j1 - j0);
    const int C = (int)(min64b(L.n, j1 + J.kuf) - j1);
    float acc = 0.0f;
    if (lane < w) {
      const float* u = ab + bix(L, j0 + lane, j1);  // U(j0 + lane, j1 + c) = u[c * ldm]
      for (int c = warp; c < C; c += 8 * (kPT / 32)) {
        float t[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const int cc = c + m * (kPT / 32);
          t[m] = cc < C ? u[(int64_t)cc * ldm] * v[j1 + cc] : 0.0f;
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) acc += t[m];
      }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
      float ui[32];
      load_row32(J.inv + (size_t)p * 2 * kBlkW * kBlkW + kBlkW * kBlkW, lane, ui);
      float s = 0.0f;
      for (int q = 0; q < kPT / 32; ++q) s += part[q][lane];
      const float t = lane < w ? v[j0 + lane] - s : 0.0f;
      float x = 0.0f;
#pragma unroll
      for (int k = 0; k < 32; ++k) x = fmaf(ui[k], __shfl_sync(kFull, t, k), x);
      if (lane < w) v[j0 + lane] = x;
    }
    __syncthreads();
  }
}

// res = rhs - A0 x (A0: the unfactored FP32 band); returns |res|.  The
// products are formed on the FP32 pipe in double-float arithmetic: x = xh + xl
// (two floats, split once per sweep), a xh = p + e exactly (FMA), and the row
// sum kept as an unevaluated float pair (Knuth's TwoSum for the high part);
// the pair's error (~2^-44 of the row's term magnitudes) is far below the
// refinement tolerance, at a sixth of the cost of FP64 FMAs on this GPU.
__device__ double patch_residual(const PatchJob& J, const float2* xs, double* red) {
  const BandLayout L = J.L;
  const float* __restrict__ a0 = J.band0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double ss = 0.0;
  for (int64_t rb = (int64_t)warp * 32; rb < L.n; rb += kPT) {
    const int64_t i = rb + lane;
    const int64_t jlo = rb - L.ku > 0 ? rb - L.ku : 0;
    const int64_t jhi = min64b(L.n, rb + 32 + L.kl);
    float sh = 0.0f, sl = 0.0f;
    if (i < L.n)
      for (int64_t jb = jlo; jb < jhi; jb += 8) {
        float av[8];
        float2 xv[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {  // all loads in flight
          const int64_t j = jb + m;
          const bool in = j < jhi && i - j <= L.kl && j - i <= L.ku;
          av[m] = in ? a0[bix(L, i, j)] : 0.0f;
          xv[m] = in ? xs[j] : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const float a = av[m];
          const float2 x = xv[m];
          // explicit roundings: a contraction of p into t would break TwoSum
          const float p = __fmul_rn(a, x.x);
          const float e = fmaf(a, x.y, fmaf(a, x.x, -p));
          const float t = __fadd_rn(sh, p);
          const float z = __fsub_rn(t, sh);
          sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
          sh = t;
        }
      }
    if (i < L.n) {
      const double r = J.rhs[i] - ((double)sh + (double)sl);
      J.res[i] = r;
      ss = fma(r, r, ss);
    }
  }
  return sqrt(block_sum(ss, red));
}

__global__ void __launch_bounds__(kPT, 1) patch_refine_kernel(const PatchJob* __restrict__ jobs,
                                                             const int* __restrict__ order, int max_sweeps,
                                                             double tol) {
  const PatchJob& J = jobs[order[blockIdx.x]];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* v = reinterpret_cast<float*>(smem_raw);  // [n]
  __shared__ float bz[32];  // zero beyond the panel width
  __shared__ float part[kPT / 32][33];
  __shared__ double red[kPT / 32];
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
  for (int64_t i = tid; i < n; i += kPT) {
    const double r = J.rhs[i];
    J.res[i] = r;
    J.x[i] = 0.0;
    ss = fma(r, r, ss);
  }
  const double r0 = sqrt(block_sum(ss, red));
  int status = MAFEM_OK, sweeps = 0;
  double rn = r0, prev = r0;
  if (r0 > 0.0) {
    status = MAFEM_REFINE_STALLED;
    for (int k = 0; k < max_sweeps; ++k) {
      const double sc = 1.0 / rn;
      for (int64_t i = tid; i < n; i += kPT) v[i] = (float)(J.res[i] * sc);
      __syncthreads();
      patch_lu_solve(J, v, bz, part);
      for (int64_t i = tid; i < n; i += kPT) {
        const double x = fma(rn, (double)v[i], J.x[i]);
        J.x[i] = x;
        const float xh = (float)x;
        xs[i] = make_float2(xh, (float)(x - (double)xh));
      }
      __syncthreads();
      rn = patch_residual(J, xs, red);
      sweeps = k + 1;
      if (!isfinite(rn)) {
        status = MAFEM_NAN_DETECTED;
        break;
      }
      if (rn <= tol * r0) {
        status = MAFEM_OK;
        break;
      }
      if (k >= 3 && rn > 0.5 * prev) break;  // stalled
      prev = rn;
    }
  }
  if (tid == 0) {
    stat[0] = status;
    stat[1] = sweeps;
  }
}

int patch_solve_setup() {
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const int dyn = cap - 12 * 1024;  // room for the kernels' static shared memory
  if (cudaFuncSetAttribute(patch_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(patch_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
    return 0;
  return dyn;
}

cudaError_t patch_solve(const PatchJob* d_jobs, const int* d_order, int njobs, size_t smem_factor, size_t smem_refine,
                        int max_sweeps, double tol, cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  patch_factor_kernel<<<njobs, kPT, smem_factor, st>>>(d_jobs, d_order);
  patch_refine_kernel<<<njobs, kPT, smem_refine, st>>>(d_jobs, d_order, max_sweeps, tol);
  return cudaGetLastError();
}

}  // namespace mafem
