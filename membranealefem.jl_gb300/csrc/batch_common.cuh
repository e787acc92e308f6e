// batch_common.cuh -- CTA-to-patch lookup of the batched kernels of a Newton
// round (elem.cu, assemble.cu).
#pragma once

#include "mafem_internal.h"

namespace mafem {

// The item whose CTA range holds CTA b: the count of items k with
// off[k + 1] <= b (off is non-decreasing; empty items are skipped).  Called by
// all 32 lanes of one warp; every lane gets the result.
__device__ __forceinline__ int batch_item_of(const int* __restrict__ off, int m, int b) {
  const int lane = threadIdx.x & 31;
  int cnt = 0;
  for (int k = lane; k < m; k += 32) cnt += off[k + 1] <= b;
  return __reduce_add_sync(0xffffffffu, cnt);
}

// The round item of this CTA (b = off[0] + blockIdx.x), found by warp 0 and
// shared through *s_k; ends with a barrier.
__device__ __forceinline__ int batch_item(const int* __restrict__ off, int m, int* s_k) {
  if (threadIdx.x < 32) {
    const int k = batch_item_of(off, m, off[0] + (int)blockIdx.x);
    if (threadIdx.x == 0) *s_k = k;
  }
  __syncthreads();
  return *s_k;
}

// Copies `bytes` (a multiple of 8) from global to shared memory, all threads.
__device__ __forceinline__ void batch_copy(void* dst, const void* src, int bytes) {
  const unsigned long long* s = static_cast<const unsigned long long*>(src);
  unsigned long long* d = static_cast<unsigned long long*>(dst);
  for (int k = threadIdx.x; k < bytes / 8; k += blockDim.x) d[k] = s[k];
}

}  // namespace mafem
