// Tile loads by the tensor memory accelerator (TMA) for the z-marching
// kernels: a tensor map (CUtensorMap, built on the host by
// cuTensorMapEncodeTiled) describes an FP64 field as a 3-D array
// [nz'][ny][nx]; one thread issues cp.async.bulk.tensor copies of boxes of it
// into shared memory, and the block waits on an mbarrier that counts the
// bytes landing.  A kernel prefetches the next plane's boxes while it
// computes on the current one.
//
// Rules the callers keep: every box lands at a 128-byte aligned shared
// address; a box's x extent times 8 bytes is a multiple of 16 and its x start
// an even element index; a slot is only refilled after a __syncthreads that
// follows the last read of it, then fence.proxy.async orders those generic
// reads before the copy.  Every wait is bounded: after kTmaSpinLimit polls the
// wait gives up and reports it, and the kernel records the timeout for the
// host (TPM_ERR_TIMEOUT) instead of hanging.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tpm {

// polls of an mbarrier before a wait gives up (with the 64 ns back-off each,
// about a quarter of a second: orders of magnitude beyond any copy of these
// tiles)
constexpr unsigned kTmaSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// makes the initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// waits for the phase of `bar` with the given parity to complete; false if
// it did not within kTmaSpinLimit polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  for (unsigned n = 0; n < kTmaSpinLimit; ++n) {
    if (mbar_test(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}

// generic-proxy accesses of shared memory before this fence are ordered
// before later async-proxy (TMA) accesses
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// box of `map` at element coordinates (x, y, z) into shared memory at dst,
// completing `bytes` on bar
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// box of `map` at (x, y, z) from shared memory at src, in the bulk group of
// this thread (elements out of the array's range are not written)
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int x, int y,
                                             int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// the bulk stores of this thread have read their shared-memory sources
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Host: a tensor map of an FP64 array [nz][ny][nx] (x fastest) with boxes of
// bx x by x 1 elements, out-of-range elements read as zero.  Returns false if
// the driver refuses it.
bool make_tensor_map_f64(CUtensorMap *map, const double *base, int nx, int ny, long long nz,
                         int bx, int by);
// Host: a tensor map of 8-byte elements [nz][ny][nx] whose rows are `pitch`
// elements apart (pitch >= nx, pitch * 8 a multiple of 16), boxes bx x by x bz.
bool make_tensor_map_8b(CUtensorMap *map, const void *base, int nx, int ny, int nz, int pitch,
                        int bx, int by, int bz);

}  // namespace tpm
