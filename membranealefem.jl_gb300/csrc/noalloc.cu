// noalloc.cu -- banded LU factor + solve that allocates no device memory.
//
// Who needs this: callers whose device memory is owned by their own allocator
// and who therefore must not call cudaMalloc behind its back -- for example a
// Julia host using CUDA.jl, whose memory pool tracks every device byte to
// decide when to collect garbage (an allocation it cannot see can push it
// into an out-of-memory error), or a step loop that must not stall, since
// cudaMalloc and cudaFree synchronise the device.  Such a caller already has
// its matrix, right-hand side and result in device memory; this entry point
// works on those buffers and keeps its own scratch (the padded band the
// factorisation works in, the panel permutations, the pivot flag) in one
// statically sized array that is part of the library's device image.
//
// Properties a caller must know:
//  - The scratch is a file-scope device array of kNoAllocScratchBytes bytes.
//    Every GPU that loads the library holds it until the process exits.
//  - All calls share it.  Calls whose work overlaps on the GPU (different
//    streams or host threads without ordering between them) race on it; order
//    them on one stream or serialise them.
//  - It keeps whatever the previous call left.  Every call rewrites the whole
//    padded band (zeros outside the caller's band) and clears the pivot flag
//    before use, so nothing stale is read.
//  - Every call looks up the array's device address on the current device
//    (cudaGetSymbolAddress, which allocates nothing), so a device or context
//    reset between calls cannot leave a stale address behind.
//  - Systems whose working set does not fit are rejected with MAFEM_ERR_ARG.
//  - A zero, infinite or NaN pivot gives MAFEM_ZERO_PIVOT; a non-finite entry
//    of x (a NaN or Inf in the band that never became a pivot) gives
//    MAFEM_NAN_DETECTED.

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "mafem.h"
#include "mafem_internal.h"

namespace mafem {

constexpr size_t kNoAllocScratchBytes = 32u << 20;  // 32 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Sets *flag when x holds a NaN or an infinity.
__global__ void nonfinite_kernel(const double* __restrict__ x, int64_t n, int* __restrict__ flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(x[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

// LAPACK band (A(i,j) at band[j*ldab + kl+ku+i-j]) -> the factorisation's padded
// layout; every stored entry of every column is written (zero outside the band).
__global__ void lapack_to_padded_kernel(const double* __restrict__ band, int64_t ldab, BandLayout L,
                                        double* __restrict__ ab) {
  for (int64_t j = blockIdx.y; j < L.n; j += gridDim.y)
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < L.ldb;
         s += (int64_t)gridDim.x * blockDim.x) {
      const int64_t i = j + s - L.off;
      double v = 0.0;
      if (i >= 0 && i < L.n && i - j >= -L.ku && i - j <= L.kl) v = band[j * ldab + L.kl + L.ku + i - j];
      ab[j * L.ldb + s] = v;
    }
}

int pick_nb(int kl) {
  for (int nb : {32, 16, 8}) {
    const size_t R = (size_t)nb + kl;
    if (R * nb * 8 + 8 * R * 8 + R * 4 <= 220 * 1024) return nb;
  }
  return 0;
}

}  // namespace
}  // namespace mafem

using namespace mafem;

/* See include/mafem.h. */
extern "C" int mafem_band_solve_noalloc(const double* band_dev, int64_t n, int64_t kl, int64_t ku, int64_t ldab,
                                        const double* rhs_dev, double* x_dev, void* stream) {
  if (!band_dev || !rhs_dev || !x_dev || n < 1 || kl < 0 || ku < 0 || ldab < 2 * kl + ku + 1 || kl != ku) {
    set_global_error("mafem_band_solve_noalloc: bad arguments (kl must equal ku, ldab >= 2kl+ku+1)");
    return MAFEM_ERR_ARG;
  }
  if (kl > 4096 || n > ((int64_t)1 << 40)) {  // before any narrowing: far beyond what the scratch holds
    set_global_error("mafem_band_solve_noalloc: half bandwidth or size too large");
    return MAFEM_ERR_ARG;
  }
  const int nb = pick_nb((int)kl);
  if (!nb) {
    set_global_error("mafem_band_solve_noalloc: half bandwidth too large");
    return MAFEM_ERR_ARG;
  }
  const BandLayout L = make_band_layout(n, (int)kl, (int)ku, nb);
  const int64_t npan = (n + nb - 1) / nb, rmax = nb + kl;
  // scratch layout: padded band | panel permutations | pivots | info
  const size_t band_bytes = (size_t)L.ldb * n * sizeof(double);
  const size_t perm_off = (band_bytes + 255) / 256 * 256;
  const size_t perm_bytes = (size_t)npan * rmax * sizeof(int);
  const size_t ipiv_off = (perm_off + perm_bytes + 255) / 256 * 256;
  const size_t info_off = (ipiv_off + (size_t)n * sizeof(int) + 255) / 256 * 256;
  const size_t need = info_off + 256;  // info[0]: zero-pivot column, info[1]: non-finite x
  if (need > kNoAllocScratchBytes) {
    set_global_error("mafem_band_solve_noalloc: needs " + std::to_string(need) + " bytes of scratch, the limit is " +
                     std::to_string(kNoAllocScratchBytes) + " (reduce n or the bandwidth, or use mafem_solve)");
    return MAFEM_ERR_ARG;
  }
  // the array's address on the current device, looked up on every call
  void* base = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
  if (e != cudaSuccess || !base) {
    set_global_error(std::string("mafem_band_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  // dynamic shared-memory limits depend on kl; set them for this size (no allocation)
  e = band_lu_setup<double>(L, 256);
  if (e != cudaSuccess) {
    set_global_error(std::string("mafem_band_solve_noalloc: kernel set-up: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned char* sb = reinterpret_cast<unsigned char*>(base);
  double* ab = reinterpret_cast<double*>(sb);
  int* perm = reinterpret_cast<int*>(sb + perm_off);
  int* ipiv = reinterpret_cast<int*>(sb + ipiv_off);
  int* info = reinterpret_cast<int*>(sb + info_off);
  dim3 grid((unsigned)((L.ldb + 255) / 256), (unsigned)(n < 65535 ? n : 65535));
  lapack_to_padded_kernel<<<grid, 256, 0, st>>>(band_dev, ldab, L, ab);
  if ((e = cudaMemsetAsync(info, 0, 2 * sizeof(int), st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(x_dev, rhs_dev, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st)) != cudaSuccess) {
    set_global_error(std::string("mafem_band_solve_noalloc: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  // factorisation with the right-hand side riding along (forward substitution),
  // on the caller's stream only, then the back substitution
  if (band_lu_factor<double>(ab, L, ipiv, perm, (int)rmax, info, x_dev, 256, 152, st, nullptr, nullptr, nullptr) < 0) {
    set_global_error(std::string("mafem_band_solve_noalloc: launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    return MAFEM_ERR_CUDA;
  }
  band_backward<double, double>(ab, L, x_dev, st);
  nonfinite_kernel<<<(unsigned)(n < 152 * 256 ? (n + 255) / 256 : 152), 256, 0, st>>>(x_dev, n, info + 1);
  int h_info[2] = {0, 0};
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(h_info, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    set_global_error(std::string("mafem_band_solve_noalloc: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  if (h_info[0]) {
    set_global_error("mafem_band_solve_noalloc: zero or non-finite pivot in column " + std::to_string(h_info[0]));
    return MAFEM_ZERO_PIVOT;
  }
  if (h_info[1]) {
    set_global_error("mafem_band_solve_noalloc: the solution holds a NaN or an infinity");
    return MAFEM_NAN_DETECTED;
  }
  return MAFEM_OK;
}
