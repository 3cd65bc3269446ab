// Deterministic block reductions (fixed tree order, no atomics).  Together
// with a fixed grid size they make every global reduction of the library
// bit-reproducible run to run; they stand in for the reference's serial sums
// plus MPI_Reduce/MPI_Bcast (tensor0.cpp:364-509).
#pragma once

namespace tpm {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Sum over the block; result valid in thread 0.  `sh` holds >= 32 entries.
// All threads of the block must call it.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = lane < nw ? sh[lane] : T(0);
    r = warp_sum(r);
  }
  return r;
}

template <typename T>
__device__ __forceinline__ T block_max(T v, T *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = lane < nw ? sh[lane] : T(0);
    r = warp_max(r);
  }
  return r;
}

// regions of tpm_ctx::partials (kRedBlocks doubles each)
enum { kPartQ = 0, kPartRhs = 1, kPartRu = 2 /* 3 regions */, kPartErr = 5, kPartDiv = 6,
       kPartTke2 = 7, kPartRegions = 8 };

}  // namespace tpm
