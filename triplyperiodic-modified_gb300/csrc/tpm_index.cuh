// Division of cell and row indices by a grid extent without an integer
// divide.  A 64-bit quotient or remainder by a run-time value is a long
// instruction sequence on the GPU; the kernels that turn a flat index
// c = (k*Ny + j)*Nx + i back into (i, j, k) use a multiply-high by a
// precomputed reciprocal instead.  Every index is below 2^31 (context
// creation rejects larger boxes).
//
// With m = floor((2^64 - 1) / d) + 1, floor(a m / 2^64) = floor(a / d) for
// every 32-bit a: m = 2^64/d + delta with 0 <= delta <= 1, so
// a m / 2^64 = a/d + a delta / 2^64, and a delta / 2^64 < 1/d because
// a d < 2^64; the fraction of a/d is at most (d - 1)/d, so the floor holds.
#pragma once

#include <cuda_runtime.h>

namespace tpm {

// the reciprocal of d >= 1 for udiv (0 encodes d = 1)
inline unsigned long long udiv_magic(unsigned d) { return d <= 1u ? 0ull : ~0ull / d + 1ull; }

#if defined(__CUDACC__) || defined(TPM_HOST_CHECK)
// floor(a / d) for m = udiv_magic(d): the high 64 bits of the 96-bit product
// a m from two 32 x 32 products (a m_hi + hi32(a m_lo) < 2^64, no carry out)
__device__ __forceinline__ unsigned udiv(unsigned a, unsigned long long m) {
  if (m == 0ull) return a;
  const unsigned long long t =
      (unsigned long long)a * (unsigned)(m >> 32) + __umulhi(a, (unsigned)m);
  return (unsigned)(t >> 32);
}
#endif

}  // namespace tpm
