// assemble.cu -- scatter of element blocks into the global residual and banded
// tangent (FiniteElement.jl:128-136, 186-194), the Newton update
// (FiniteElement.jl:40-48), update_xms! (FiniteElement.jl:408-423), and the
// FP64 refinement residual of the FP32 solve.
//
// The reference scatters with LM into per-thread sparse matrices and sums them.
// Here the scatter is inverted into a gather over the tensor-product
// connectivity: element (e1, e2) owns nodes (e1..e1+2) x (e2..e2+2)
// (Mesh.jl:582-589), so a band entry (i, j) receives contributions only from
// the <= 3x3 elements that contain both node(i) and node(j), and each output
// is produced by exactly one thread -- no atomics, deterministic sums.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "batch_common.cuh"
#include "mafem_internal.h"

namespace mafem {

__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

// One thread per stored entry of band column j; entries outside the element
// stencil (structural zeros, pivoting-fill rows, padding) are written as zero,
// so the band needs no separate clearing pass.
// Band entry (row j + s - off, column j): the sum of the <= 3 x 3 element
// contributions, zero outside the element stencil.
template <class T>
__device__ __forceinline__ T band_entry(const DevPatch& P, int ndf, int nq, const BandLayout& L,
                                        const T* __restrict__ K_el, int64_t j, int s1J, int s2J, int dj, int64_t s) {
  const int64_t i = j + s - L.off;
  T val = T(0);
  if (i >= 0 && i < L.n && i - j >= -L.ku && i - j <= L.kl) {
    const int NI = P.unk_node[i], di = P.unk_dof[i];
    const int s1I = NI % P.num1np, s2I = NI / P.num1np;
    if (abs(s1I - s1J) <= 2 && abs(s2I - s2J) <= 2) {
      const int e1lo = max(max(s1I, s1J) - 2, 0), e1hi = min(min(s1I, s1J), P.num1el - 1);
      const int e2lo = max(max(s2I, s2J) - 2, 0), e2hi = min(min(s2I, s2J), P.num2el - 1);
      for (int e2 = e2lo; e2 <= e2hi; ++e2)
        for (int e1 = e1lo; e1 <= e1hi; ++e1) {
          const int e = e1 + P.num1el * e2;
          const int a = (s1I - e1) + 3 * (s2I - e2), b = (s1J - e1) + 3 * (s2J - e2);
          val += K_el[(size_t)e * nq * nq + (size_t)(b * ndf + dj) * nq + a * ndf + di];
        }
    }
  }
  return val;
}

// One thread per stored entry of band column j; entries outside the element
// stencil (structural zeros, pivoting-fill rows, padding) are written as zero,
// so the band needs no separate clearing pass.
template <class T>
__global__ void band_gather_kernel(DevPatch P, int ndf, int nq, BandLayout L, const T* __restrict__ K_el,
                                   T* __restrict__ ab, T* __restrict__ ab2) {
  for (int64_t j = blockIdx.y; j < L.n; j += gridDim.y) {
    const int NJ = P.unk_node[j], dj = P.unk_dof[j];
    const int s1J = NJ % P.num1np, s2J = NJ / P.num1np;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < L.ldb;
         s += (int64_t)gridDim.x * blockDim.x) {
      const T val = band_entry<T>(P, ndf, nq, L, K_el, j, s1J, s2J, dj, s);
      ab[j * L.ldb + s] = val;
      if (ab2) ab2[j * L.ldb + s] = val;  // the unfactored copy the refinement multiplies by
    }
  }
}

// r[i] = Σ_e r_el[e][(a, di)] over the elements containing node(i) (FiniteElement.jl:131)
__global__ void resid_gather_kernel(DevPatch P, int ndf, int nq, const double* __restrict__ r_el,
                                    double* __restrict__ r) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.nmdf; i += (int64_t)gridDim.x * blockDim.x) {
    const int NI = P.unk_node[i], di = P.unk_dof[i];
    const int s1 = NI % P.num1np, s2 = NI / P.num1np;
    double acc = 0.0;
    for (int e2 = max(s2 - 2, 0); e2 <= min(s2, P.num2el - 1); ++e2)
      for (int e1 = max(s1 - 2, 0); e1 <= min(s1, P.num1el - 1); ++e1) {
        const int e = e1 + P.num1el * e2;
        const int a = (s1 - e1) + 3 * (s2 - e2);
        acc += r_el[(size_t)e * nq + a * ndf + di];
      }
    r[i] = acc;
  }
}

// update_xms! (FiniteElement.jl:408-423) used as the predictor (Analysis.jl:70):
// xms[:, j] += dt * cps[:, m_motion_order[j]]
__global__ void predictor_kernel(DevPatch P, PhysParams pp, double dt) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < 3LL * P.numnp;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / P.numnp), node = (int)(k - (int64_t)j * P.numnp);
    const int d = pp.mmo[j];
    if (d >= 0) P.xms[k] += dt * P.cps[(size_t)d * P.numnp + node];
  }
}

// Newton update (FiniteElement.jl:41-46): Δu = -x, Δcps[ID_inv] = Δu, cps += Δcps,
// xms[:, j] += dt Δcps[:, m_motion_order[j]]; per-block partial sums of Δu² and r².
// skip, skip2: when either word is nonzero (the factorisation found no usable
// pivot, the batched solve failed, or a bounded wait ran out) the state is left
// unchanged and only r² is summed (so a non-finite residual still shows); the
// host redoes the iteration or reports the failure.
__device__ __forceinline__ void newton_update_body(const DevPatch& P, const PhysParams& pp, double dt,
                                                   const double* __restrict__ x, const double* __restrict__ r,
                                                   double* __restrict__ part, bool hold, int blk, int nblk) {
  __shared__ double s_du[32], s_r[32];
  double du2 = 0.0, r2 = 0.0;
  for (int64_t q = blk * (int64_t)blockDim.x + threadIdx.x; q < P.nmdf; q += (int64_t)nblk * blockDim.x) {
    r2 += r[q] * r[q];
    if (hold) continue;
    const double du = -x[q];
    const int node = P.unk_node[q], d = P.unk_dof[q];
    P.cps[(size_t)d * P.numnp + node] += du;
    for (int j = 0; j < 3; ++j)
      if (pp.mmo[j] == d) P.xms[(size_t)j * P.numnp + node] += dt * du;
    du2 += du * du;
  }
  for (int o = 16; o > 0; o >>= 1) {
    du2 += __shfl_down_sync(0xffffffffu, du2, o);
    r2 += __shfl_down_sync(0xffffffffu, r2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_du[threadIdx.x >> 5] = du2;
    s_r[threadIdx.x >> 5] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += s_du[k];
      b += s_r[k];
    }
    part[2 * blk] = a;
    part[2 * blk + 1] = b;
  }
}

__global__ void newton_update_kernel(DevPatch P, PhysParams pp, double dt, const double* __restrict__ x,
                                     const double* __restrict__ r, double* __restrict__ part,
                                     const int* __restrict__ skip, const int* __restrict__ skip2,
                                     const int* __restrict__ skip3) {
  const bool hold = (skip && *skip) || (skip2 && *skip2) || (skip3 && *skip3);
  newton_update_body(P, pp, dt, x, r, part, hold, blockIdx.x, gridDim.x);
}

// Fixed-order final reduction: out[0] = ‖Δu‖₂ / nmdf (the Newton ε,
// FiniteElement.jl:48), out[1] = ‖r‖₂, out[2] = 1 if either is not finite.
__global__ void newton_norm_kernel(const double* __restrict__ part, int nblk, int64_t nmdf, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < nblk; ++k) {
      a += part[2 * k];
      b += part[2 * k + 1];
    }
    out[0] = sqrt(a) / (double)nmdf;
    out[1] = sqrt(b);
    out[2] = (isfinite(a) && isfinite(b)) ? 0.0 : 1.0;
  }
}

// Refinement residual res = r - A0 x in FP64 arithmetic, A0 = the unfactored
// band (any storage type).  A warp owns 32 consecutive rows and walks the
// columns of its band window, so every load of A0 is a coalesced 32-row
// column segment.
template <class T>
__global__ void band_residual_kernel(const T* __restrict__ a0, BandLayout L, const double* __restrict__ x,
                                     const double* __restrict__ r, double* __restrict__ res,
                                     double* __restrict__ part, const int* __restrict__ gate) {
  __shared__ double s_p[32];
  if (gate && *gate) return;  // the refinement has already stopped
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  double nrm = 0.0;
  for (int64_t wi = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); wi * 32 < L.n; wi += nwarps) {
    const int64_t i0 = wi * 32, i = i0 + lane;
    const int64_t jlo = max64(0, i0 - L.kl), jhi = min64(L.n - 1, i0 + 31 + L.ku);
    double acc = 0.0;
    for (int64_t j = jlo; j <= jhi; ++j) {
      const double xj = x[j];
      if (i < L.n && i - j >= -L.ku && i - j <= L.kl) acc += (double)a0[j * L.ldb + L.off + i - j] * xj;
    }
    if (i < L.n) {
      const double v = r[i] - acc;
      res[i] = v;
      nrm += v * v;
    }
  }
  for (int o = 16; o > 0; o >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, o);
  if (lane == 0) s_p[threadIdx.x >> 5] = nrm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) a += s_p[k];
    part[blockIdx.x] = a;
  }
}
__global__ void sqrt_sum_kernel(const double* __restrict__ part, int n, double* __restrict__ out,
                                const int* __restrict__ gate) {
  if (gate && *gate) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0;
    for (int k = 0; k < n; ++k) a += part[k];
    *out = sqrt(a);
  }
}
__global__ void axpy_kernel(int64_t n, const double* __restrict__ dx, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += dx[i];
}

// x += dx with the partial sums of |dx|^2 and |x|^2 per block (part[2 b], part[2 b + 1])
__global__ void axpy_norms_kernel(int64_t n, const double* __restrict__ dx, double* __restrict__ x,
                                  double* __restrict__ part, const int* __restrict__ gate) {
  if (gate && *gate) return;
  double dd = 0.0, xx = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = dx[i];
    const double v = x[i] + d;
    x[i] = v;
    dd = fma(d, d, dd);
    xx = fma(v, v, xx);
  }
  __shared__ double s[2][8];
  for (int o = 16; o > 0; o >>= 1) {
    dd += __shfl_xor_sync(0xffffffffu, dd, o);
    xx += __shfl_xor_sync(0xffffffffu, xx, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s[0][threadIdx.x >> 5] = dd;
    s[1][threadIdx.x >> 5] = xx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; ++w) {
      a += s[0][w];
      b += s[1][w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}
// out[0] = |dx|, out[1] = |x| from the block partial sums, in a fixed order
__global__ void sqrt_pair_kernel(const double* __restrict__ part, int nblk, double* __restrict__ out,
                                 const int* __restrict__ gate) {
  if (gate && *gate) return;
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblk; ++k) {
      a += part[2 * k];
      b += part[2 * k + 1];
    }
    out[0] = sqrt(a);
    out[1] = sqrt(b);
  }
}

// ---- batched kernels of a Newton round: every patch of the round in one launch ----------
// Each patch gets exactly the CTAs (and the same CTA-to-work map) its own
// launch would use: the gathers, the update and the norms sum in the same
// order as the per-patch kernels.

// Both bands of the FP32 form, kGatherCols columns per CTA.
__global__ void __launch_bounds__(256, 4) batch_gather_kernel(const AsmJob* __restrict__ jobs,
                                                           const AsmItem* __restrict__ items,
                                                           const int* __restrict__ off, int m) {
  __shared__ int s_k;
  const int k = batch_item(off, m, &s_k);
  const AsmJob& J = jobs[items[k].job];
  const BandLayout L = J.L;
  const int ndf = J.pp.ndf, nq = J.pp.nq;
  const int64_t j0 = (int64_t)(off[0] + (int)blockIdx.x - off[k]) * kGatherCols;
  for (int64_t j = j0; j < min64(j0 + kGatherCols, L.n); ++j) {
    const int NJ = J.P.unk_node[j], dj = J.P.unk_dof[j];
    const int s1J = NJ % J.P.num1np, s2J = NJ / J.P.num1np;
    for (int64_t s = threadIdx.x; s < L.ldb; s += blockDim.x) {
      const float val = band_entry<float>(J.P, ndf, nq, L, J.K_el, j, s1J, s2J, dj, s);
      J.band[j * L.ldb + s] = val;
      J.band0[j * L.ldb + s] = val;
    }
  }
}

// The residual, 256 unknowns per CTA; the patch's first CTA also zeroes its
// info words for the round's solve.
__global__ void __launch_bounds__(256) batch_rgather_kernel(const AsmJob* __restrict__ jobs,
                                                            const AsmItem* __restrict__ items,
                                                            const int* __restrict__ off, int m) {
  __shared__ int s_k;
  const int k = batch_item(off, m, &s_k);
  const AsmJob& J = jobs[items[k].job];
  const int blk = off[0] + (int)blockIdx.x - off[k];
  if (blk == 0 && threadIdx.x < 4) J.info[threadIdx.x] = 0;
  const int64_t i = (int64_t)blk * blockDim.x + threadIdx.x;
  if (i >= J.P.nmdf) return;
  const int ndf = J.pp.ndf, nq = J.pp.nq;
  const int NI = J.P.unk_node[i], di = J.P.unk_dof[i];
  const int s1 = NI % J.P.num1np, s2 = NI / J.P.num1np;
  double acc = 0.0;
  for (int e2 = max(s2 - 2, 0); e2 <= min(s2, J.P.num2el - 1); ++e2)
    for (int e1 = max(s1 - 2, 0); e1 <= min(s1, J.P.num1el - 1); ++e1) {
      const int e = e1 + J.P.num1el * e2;
      const int a = (s1 - e1) + 3 * (s2 - e2);
      acc += J.r_el[(size_t)e * nq + a * ndf + di];
    }
  J.r[i] = acc;
}

// Newton update of every patch; a patch whose solve failed (status or
// wait-ran-out word set) keeps its state.
__global__ void __launch_bounds__(256) batch_update_kernel(const AsmJob* __restrict__ jobs,
                                                           const AsmItem* __restrict__ items,
                                                           const int* __restrict__ off, int m) {
  __shared__ int s_k;
  const int k = batch_item(off, m, &s_k);
  const AsmItem it = items[k];
  const AsmJob& J = jobs[it.job];
  const bool hold = J.info[2] != 0 || J.info[1] != 0;
  newton_update_body(J.P, J.pp, it.dt, J.x, J.r, J.part, hold, off[0] + (int)blockIdx.x - off[k], off[k + 1] - off[k]);
}

// The fixed-order norms of newton_norm_kernel, one CTA per patch, copied with
// the info words into outs[k] for the host.
__global__ void batch_norm_kernel(const AsmJob* __restrict__ jobs, const AsmItem* __restrict__ items,
                                  const int* __restrict__ off, int m, AsmOut* __restrict__ outs) {
  const int k = blockIdx.x;
  if (k >= m || threadIdx.x != 0) return;
  const AsmJob& J = jobs[items[k].job];
  const int nblk = off[k + 1] - off[k];
  double a = 0, b = 0;
  for (int t = 0; t < nblk; ++t) {
    a += J.part[2 * t];
    b += J.part[2 * t + 1];
  }
  AsmOut o;
  o.out[0] = sqrt(a) / (double)J.P.nmdf;
  o.out[1] = sqrt(b);
  o.out[2] = (isfinite(a) && isfinite(b)) ? 0.0 : 1.0;
  for (int t = 0; t < 3; ++t) J.out[t] = o.out[t];
  for (int t = 0; t < 4; ++t) o.info[t] = J.info[t];
  outs[k] = o;
}

// The scaled inhomogeneous Dirichlet values of the patches that start a time
// step (mafem_set_dirichlet_scale's edit of the state).
__global__ void __launch_bounds__(256) batch_dirichlet_kernel(const AsmJob* __restrict__ jobs,
                                                              const AsmItem* __restrict__ items,
                                                              const int* __restrict__ off, int m) {
  __shared__ int s_k;
  const int k = batch_item(off, m, &s_k);
  const AsmItem it = items[k];
  const AsmJob& J = jobs[it.job];
  const int idx = (off[0] + (int)blockIdx.x - off[k]) * blockDim.x + threadIdx.x;
  if ((it.start & kStartDirichlet) && idx < J.n_dir) J.P.cps[J.dir_idx[idx]] = it.dscale * J.dir_val[idx];
}

// update_xms! as the predictor of every patch (Analysis.jl:70).
__global__ void __launch_bounds__(256) batch_predictor_kernel(const AsmJob* __restrict__ jobs,
                                                              const AsmItem* __restrict__ items,
                                                              const int* __restrict__ off, int m) {
  __shared__ int s_k;
  const int k = batch_item(off, m, &s_k);
  const AsmItem it = items[k];
  const AsmJob& J = jobs[it.job];
  const int64_t idx = (int64_t)(off[0] + (int)blockIdx.x - off[k]) * blockDim.x + threadIdx.x;
  if (!(it.start & kStartPredict) || idx >= 3LL * J.P.numnp) return;
  const int j = (int)(idx / J.P.numnp), node = (int)(idx - (int64_t)j * J.P.numnp);
  const int d = J.pp.mmo[j];
  if (d >= 0) J.P.xms[idx] += it.dt * J.P.cps[(size_t)d * J.P.numnp + node];
}

// ---- launchers -------------------------------------------------------------------
void launch_batch_gather(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, cudaStream_t st) {
  if (ctas > 0) batch_gather_kernel<<<ctas, 256, 0, st>>>(jobs, items, off, m);
}
void launch_batch_rgather(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, cudaStream_t st) {
  if (ctas > 0) batch_rgather_kernel<<<ctas, 256, 0, st>>>(jobs, items, off, m);
}
void launch_batch_update(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, AsmOut* outs,
                         cudaStream_t st) {
  if (ctas <= 0) return;
  batch_update_kernel<<<ctas, 256, 0, st>>>(jobs, items, off, m);
  batch_norm_kernel<<<m, 32, 0, st>>>(jobs, items, off, m, outs);
}
void launch_batch_predictor(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                            cudaStream_t st) {
  if (ctas > 0) batch_predictor_kernel<<<ctas, 256, 0, st>>>(jobs, items, off, m);
}
void launch_batch_dirichlet(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                            cudaStream_t st) {
  if (ctas > 0) batch_dirichlet_kernel<<<ctas, 256, 0, st>>>(jobs, items, off, m);
}
template <class T>
void launch_band_gather(const DevPatch& P, int ndf, int nq, const BandLayout& L, const T* K_el, T* ab,
                        cudaStream_t st, T* ab2) {
  dim3 grid((unsigned)((L.ldb + 255) / 256), (unsigned)min64(L.n, 65535));
  band_gather_kernel<T><<<grid, 256, 0, st>>>(P, ndf, nq, L, K_el, ab, ab2);
}
void launch_resid_gather(const DevPatch& P, int ndf, int nq, const double* r_el, double* r, cudaStream_t st) {
  const int blocks = (int)min64(1024, (P.nmdf + 255) / 256);
  resid_gather_kernel<<<blocks, 256, 0, st>>>(P, ndf, nq, r_el, r);
}
// cps[idx[k]] = s * val[k]: the inhomogeneous Dirichlet entries of the state, scaled
__global__ void dirichlet_scale_kernel(double* __restrict__ cps, const int* __restrict__ idx,
                                       const double* __restrict__ val, int n, double s) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) cps[idx[k]] = s * val[k];
}
void launch_dirichlet_scale(double* cps, const int* idx, const double* val, int n, double s, cudaStream_t st) {
  if (n > 0) dirichlet_scale_kernel<<<(n + 255) / 256, 256, 0, st>>>(cps, idx, val, n, s);
}
void launch_predictor(const DevPatch& P, const PhysParams& pp, double dt, cudaStream_t st) {
  const int blocks = (int)min64(1024, (3LL * P.numnp + 255) / 256);
  predictor_kernel<<<blocks, 256, 0, st>>>(P, pp, dt);
}
int newton_update_blocks(int64_t nmdf) { return (int)min64(256, (nmdf + 255) / 256); }
void launch_newton_update(const DevPatch& P, const PhysParams& pp, double dt, const double* x, const double* r,
                          double* part, double* out, cudaStream_t st, const int* skip, const int* skip2,
                          const int* skip3) {
  const int blocks = newton_update_blocks(P.nmdf);
  newton_update_kernel<<<blocks, 256, 0, st>>>(P, pp, dt, x, r, part, skip, skip2, skip3);
  newton_norm_kernel<<<1, 32, 0, st>>>(part, blocks, P.nmdf, out);
}
int band_residual_blocks(int64_t n) { return (int)min64(304, (n + 255) / 256); }
template <class T>
void launch_band_residual(const T* a0, const BandLayout& L, const double* x, const double* r, double* res,
                          double* part, double* out, cudaStream_t st, const int* gate) {
  const int blocks = band_residual_blocks(L.n);
  band_residual_kernel<T><<<blocks, 256, 0, st>>>(a0, L, x, r, res, part, gate);
  sqrt_sum_kernel<<<1, 32, 0, st>>>(part, blocks, out, gate);
}
void launch_axpy_norms(int64_t n, const double* dx, double* x, double* part, double* out, cudaStream_t st,
                       const int* gate) {
  const int blocks = (int)min64(1024, (n + 255) / 256);  // part holds 2048 doubles
  axpy_norms_kernel<<<blocks, 256, 0, st>>>(n, dx, x, part, gate);
  sqrt_pair_kernel<<<1, 32, 0, st>>>(part, blocks, out, gate);
}

// ---- device-side stopping test of one handle's iterative refinement ----------------
// st[0] done, st[1] sweeps, st[2] status; nrm[0] |r0|, nrm[1] the previous
// residual norm.  rn: the residual norm after the sweep (band_residual's out).
__global__ void refine_init_kernel(const double* __restrict__ r0, int* __restrict__ st, double* __restrict__ nrm) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double v = *r0;
    nrm[0] = v;
    nrm[1] = v;
    st[1] = 0;
    st[2] = MAFEM_OK;
    st[0] = (v > 0.0) ? 0 : 1;  // a zero right-hand side: x = 0, nothing to refine
    if (!(v == v) || v > 1.7976931348623157e308) {  // NaN or Inf
      st[0] = 1;
      st[2] = MAFEM_NAN_DETECTED;
    }
  }
}
// After each sweep: stop on |r| <= tol |r0| (MAFEM_OK), a non-finite norm
// (MAFEM_NAN_DETECTED), a stall -- |r| > |r_prev| / 2 after the fourth sweep --
// or max_sweeps (MAFEM_REFINE_STALLED, or MAFEM_OK when the last correction is
// at most 1e-8 |x|: the residual has reached its rounding floor, which in a
// late Newton iteration, where |r0| is itself tiny, lies above tol |r0|).
__global__ void refine_check_kernel(const double* __restrict__ rn, const double* __restrict__ dxn, int* __restrict__ st,
                                    double* __restrict__ nrm, double tol, int max_sweeps) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || st[0]) return;
  const double r = *rn, d = dxn[0], xv = dxn[1];
  // (refine_init_kernel clears st[0..2]; st[3] is written by refine_seal_kernel)
  const int k = st[1] + 1;
  st[1] = k;
  if (!isfinite(r) || !isfinite(d) || !isfinite(xv)) {
    st[2] = MAFEM_NAN_DETECTED;
    st[0] = 1;
  } else if (r <= tol * nrm[0]) {
    st[0] = 1;
  } else if ((k >= 4 && r > 0.5 * nrm[1]) || k >= max_sweeps) {
    // no longer contracting: at the rounding floor (the last correction a
    // small part of x) the solution is as accurate as the factors allow
    st[2] = (d <= 1e-8 * xv) ? MAFEM_OK : MAFEM_REFINE_STALLED;
    st[0] = 1;
  }
  nrm[1] = r;
}
__global__ void copy_gated_kernel(int64_t n, const double* __restrict__ src, double* __restrict__ dst,
                                  const int* __restrict__ gate) {
  if (gate && *gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
void launch_refine_init(const double* r0, int* st, double* nrm, cudaStream_t s) {
  refine_init_kernel<<<1, 32, 0, s>>>(r0, st, nrm);
}
void launch_refine_check(const double* rn, const double* dxn, int* st, double* nrm, double tol, int max_sweeps,
                         cudaStream_t s) {
  refine_check_kernel<<<1, 32, 0, s>>>(rn, dxn, st, nrm, tol, max_sweeps);
}
// st[3] = 1 unless the refinement has stopped with MAFEM_OK (the Newton update's skip word)
__global__ void refine_seal_kernel(int* __restrict__ st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) st[3] = (st[0] && st[2] == MAFEM_OK) ? 0 : 1;
}
void launch_refine_seal(int* st, cudaStream_t s) { refine_seal_kernel<<<1, 32, 0, s>>>(st); }
void launch_copy_gated(int64_t n, const double* src, double* dst, const int* gate, cudaStream_t s) {
  const int blocks = (int)min64(304, (n + 255) / 256);
  copy_gated_kernel<<<blocks, 256, 0, s>>>(n, src, dst, gate);
}
void launch_axpy(int64_t n, const double* dx, double* x, cudaStream_t st) {
  const int blocks = (int)min64(1024, (n + 255) / 256);
  axpy_kernel<<<blocks, 256, 0, st>>>(n, dx, x);
}

template void launch_band_gather<double>(const DevPatch&, int, int, const BandLayout&, const double*, double*,
                                         cudaStream_t, double*);
template void launch_band_gather<float>(const DevPatch&, int, int, const BandLayout&, const float*, float*,
                                        cudaStream_t, float*);
template void launch_band_residual<double>(const double*, const BandLayout&, const double*, const double*, double*,
                                           double*, double*, cudaStream_t, const int*);
template void launch_band_residual<float>(const float*, const BandLayout&, const double*, const double*, double*,
                                          double*, double*, cudaStream_t, const int*);

}  // namespace mafem
