// Pressure projection: poisson::FFT / poisson::CCP_FFT (poisson.cpp:391-462)
// as hand-written pencil FFTs in shared memory.
//
// One Richardson iteration is five kernels over a half-complex spectrum
// [Nz][Ny][Nx/2+1] (the reference transforms a full complex box whose input
// is real, poisson.cpp:423-431; a real-to-complex transform is the same
// transform at half the traffic):
//   1. x-pass: residual r = cc*(div(C grad P) - RHS) of a block of x-rows,
//      computed on the fly, packed as Nx/2 complex points, FFT, real-to-
//      complex post-processing, written to the spectrum;
//   2. y-pass forward;
//   3. z-pass: forward FFT, divide by the modified wave number
//      mwn = (2/dx^2)(1-cos kx dx) + ... except the zero mode
//      (poisson.cpp:438-451), inverse FFT - all in shared memory;
//   4. y-pass inverse;
//   5. x-pass inverse: complex-to-real, dp = -x/N^3 (poisson.cpp:460),
//      P += dp and a per-block max|dp| (poisson.cpp:405-407).
// FFTs are mixed-radix (4, 2, 3, 5) Stockham auto-sort with twiddles from a
// host table (cos/sin of 2 pi m/n).  Butterflies use explicit FMAs; the
// residual and the update keep the reference's operation order.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "tpm_internal.cuh"
#include "tpm_ff.cuh"
#include "tpm_reduce.cuh"
#include "tpm_tma.cuh"

namespace tpm {
namespace {

constexpr int kFftThreads = 256;
constexpr int kFftSmemPoints = 2048;  // complex points per ping-pong buffer
constexpr int kMaxPens = 32;           // pencils per block at most (pens_for, autotune)

template <typename T2>
struct Cx;
template <>
struct Cx<double2> {
  using T = double;
  static __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
  static __device__ __forceinline__ double fma_(double a, double b, double c) {
    return __fma_rn(a, b, c);
  }
  static __device__ __forceinline__ double2 tw(const FftPlan &p, int e) { return p.tw64[e]; }
};
template <>
struct Cx<float2> {
  using T = float;
  static __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
  static __device__ __forceinline__ float fma_(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
  }
  static __device__ __forceinline__ float2 tw(const FftPlan &p, int e) { return p.tw32[e]; }
};

// (a) * (w or conj(w))
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 w, int sign) {
  using C = Cx<T2>;
  typename C::T wi = sign < 0 ? w.y : -w.y;
  return C::mk(C::fma_(a.x, w.x, -a.y * wi), C::fma_(a.x, wi, a.y * w.x));
}

// i / d by one multiply-high with m = ceil(2^32 / d), exact for 0 <= i < 2^16
// and 2 <= d < 2^16 (the error i*(m - 2^32/d)/2^32 < 2^-16 < 1/d cannot carry
// the quotient past an integer); m = 0 stands for d = 1.  Every index of the
// pencil passes is below 2^13.
unsigned fdiv_magic(int d) { return d <= 1 ? 0u : 0xFFFFFFFFu / (unsigned)d + 1u; }
__device__ __forceinline__ int fdiv(int i, unsigned m) {
  return m ? (int)__umulhi((unsigned)i, m) : i;
}

// DFT4 in place: V_u = sum_t v_t W^(t u), W = exp(sign 2 pi i / 4)
template <typename T2>
__device__ __forceinline__ void dft4(T2 *v, int sign) {
  using C = Cx<T2>;
  T2 a = C::mk(v[0].x + v[2].x, v[0].y + v[2].y);
  T2 b = C::mk(v[0].x - v[2].x, v[0].y - v[2].y);
  T2 c = C::mk(v[1].x + v[3].x, v[1].y + v[3].y);
  T2 d = C::mk(v[1].x - v[3].x, v[1].y - v[3].y);
  T2 j = sign < 0 ? C::mk(d.y, -d.x) : C::mk(-d.y, d.x);  // d * (sign i)
  v[0] = C::mk(a.x + c.x, a.y + c.y);
  v[2] = C::mk(a.x - c.x, a.y - c.y);
  v[1] = C::mk(b.x + j.x, b.y + j.y);
  v[3] = C::mk(b.x - j.x, b.y - j.y);
}

template <typename T2>
__device__ __forceinline__ void dft8(T2 *v, int sign);
template <typename T2>
__device__ __forceinline__ void dft16(T2 *v, int sign);

// V_u = sum_t v_t W^(t u), W = exp(sign 2 pi i / R), in place
template <typename T2>
__device__ __forceinline__ void dft_small(T2 *v, int R, int sign) {
  using C = Cx<T2>;
  using T = typename C::T;
  if (R == 16) {
    dft16(v, sign);
  } else if (R == 8) {
    dft8(v, sign);
  } else if (R == 2) {
    T2 a = v[0], b = v[1];
    v[0] = C::mk(a.x + b.x, a.y + b.y);
    v[1] = C::mk(a.x - b.x, a.y - b.y);
  } else if (R == 4) {
    dft4(v, sign);
  } else if (R == 3) {
    const T s3 = (T)0.86602540378443864676;
    T s = sign < 0 ? -s3 : s3;
    T2 sm = C::mk(v[1].x + v[2].x, v[1].y + v[2].y);
    T2 df = C::mk(v[1].x - v[2].x, v[1].y - v[2].y);
    T2 m = C::mk(C::fma_((T)-0.5, sm.x, v[0].x), C::fma_((T)-0.5, sm.y, v[0].y));
    v[0] = C::mk(v[0].x + sm.x, v[0].y + sm.y);
    v[1] = C::mk(C::fma_(-s, df.y, m.x), C::fma_(s, df.x, m.y));
    v[2] = C::mk(C::fma_(s, df.y, m.x), C::fma_(-s, df.x, m.y));
  } else {  // R == 5
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
    T sa = sign < 0 ? -s1 : s1, sb = sign < 0 ? -s2 : s2;
    T2 t1 = C::mk(v[1].x + v[4].x, v[1].y + v[4].y), t2 = C::mk(v[2].x + v[3].x, v[2].y + v[3].y);
    T2 d1 = C::mk(v[1].x - v[4].x, v[1].y - v[4].y), d2 = C::mk(v[2].x - v[3].x, v[2].y - v[3].y);
    T2 x0 = v[0];
    T2 p1 = C::mk(C::fma_(c2, t2.x, C::fma_(c1, t1.x, x0.x)), C::fma_(c2, t2.y, C::fma_(c1, t1.y, x0.y)));
    T2 p2 = C::mk(C::fma_(c1, t2.x, C::fma_(c2, t1.x, x0.x)), C::fma_(c1, t2.y, C::fma_(c2, t1.y, x0.y)));
    T2 q1 = C::mk(C::fma_(sb, d2.x, sa * d1.x), C::fma_(sb, d2.y, sa * d1.y));
    T2 q2 = C::mk(C::fma_(-sa, d2.x, sb * d1.x), C::fma_(-sa, d2.y, sb * d1.y));
    v[0] = C::mk(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
    v[1] = C::mk(p1.x - q1.y, p1.y + q1.x);
    v[4] = C::mk(p1.x + q1.y, p1.y - q1.x);
    v[2] = C::mk(p2.x - q2.y, p2.y + q2.x);
    v[3] = C::mk(p2.x + q2.y, p2.y - q2.x);
  }
}

// a * (wr + i wi) for a constant twiddle
template <typename T2>
__device__ __forceinline__ T2 cmulc(T2 a, typename Cx<T2>::T wr, typename Cx<T2>::T wi) {
  using C = Cx<T2>;
  return C::mk(C::fma_(a.x, wr, -a.y * wi), C::fma_(a.x, wi, a.y * wr));
}

// Radix 8 as 4 x 2 (Cooley-Tukey, N = N1 N2 with n = 2 n1 + n2 and
// k = k1 + 4 k2): DFT4 over the even and the odd elements, the odd ones times
// W8^k1, then one DFT2 per k1.
template <typename T2>
__device__ __forceinline__ void dft8(T2 *v, int sign) {
  using C = Cx<T2>;
  using T = typename C::T;
  const T r = (T)0.70710678118654752440, s = sign < 0 ? (T)-1 : (T)1;
  T2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e, sign);
  dft4(o, sign);
  o[1] = cmulc(o[1], r, s * r);
  o[2] = C::mk(-s * o[2].y, s * o[2].x);
  o[3] = cmulc(o[3], -r, s * r);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = C::mk(e[k].x + o[k].x, e[k].y + o[k].y);
    v[k + 4] = C::mk(e[k].x - o[k].x, e[k].y - o[k].y);
  }
}

// Radix 16 as 4 x 4 (n = 4 n1 + n2, k = k1 + 4 k2): four DFT4 over n1,
// the twiddles W16^(n2 k1), four DFT4 over n2; all in registers.
template <typename T2>
__device__ __forceinline__ void dft16(T2 *v, int sign) {
  using C = Cx<T2>;
  using T = typename C::T;
  const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
  const T r = (T)0.70710678118654752440, s = sign < 0 ? (T)-1 : (T)1;
  T2 y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    T2 t[4] = {v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]};
    dft4(t, sign);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = t[k1];
  }
  y[1][1] = cmulc(y[1][1], c1, s * s1);        // W^1
  y[1][2] = cmulc(y[1][2], r, s * r);          // W^2
  y[1][3] = cmulc(y[1][3], s1, s * c1);        // W^3
  y[2][1] = cmulc(y[2][1], r, s * r);          // W^2
  y[2][2] = C::mk(-s * y[2][2].y, s * y[2][2].x);  // W^4 = sign i
  y[2][3] = cmulc(y[2][3], -r, s * r);         // W^6
  y[3][1] = cmulc(y[3][1], s1, s * c1);        // W^3
  y[3][2] = cmulc(y[3][2], -r, s * r);         // W^6
  y[3][3] = cmulc(y[3][3], -c1, -s * s1);      // W^9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    T2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft4(t, sign);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

// One Stockham stage of radix R:  for i in [0, n/R): k = i mod p,
//   v_t = a[i + t n/R] * w^(k t n/(p R)),  V = DFT_R(v),
//   b[(i/p) p R + k + u p] = V_u.
// npen = 2^lq pencils; pm is the division magic of p (fdiv_magic).
template <int R, typename T2>
__device__ __forceinline__ void stockham_stage(const T2 *__restrict__ a, T2 *__restrict__ b,
                                               int lq, const FftPlan &pl, int p, unsigned pm,
                                               int sign, const T2 *__restrict__ tws) {
  const int n = pl.n;
  const int m = n / R;
  const int step = n / (p * R);
  const int npen = 1 << lq;
  const int total = m << lq;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int q = idx & (npen - 1);
    const int i = idx >> lq;
    const int ip = fdiv(i, pm);  // i / p
    const int k = i - ip * p;
    T2 v[R];
    v[0] = a[i * npen + q];
    if (p == 1) {  // first stage: every twiddle is w^0 = 1
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = a[(i + t * m) * npen + q];
    } else {
#pragma unroll
      for (int t = 1; t < R; ++t)
        v[t] = cmul(a[(i + t * m) * npen + q],
                    tws ? tws[k * t * step] : Cx<T2>::tw(pl, k * t * step), sign);
    }
    dft_small(v, R, sign);
    const int j = ip * p * R + k;
    if (sizeof(T2) == sizeof(float2) && p == 1 && (R & (R - 1)) == 0 && npen >= 4 && npen <= 8) {
      // first stage: the lanes of a warp hold 32 / npen consecutive i, whose
      // outputs u sit R * npen elements apart, all on the same banks when
      // written in the same order; lanes with odd i (and, at 4 pencils, with
      // i = 2, 3 mod 4) write their outputs in a swapped order, so that one
      // store instruction covers both halves of the banks
      const int sw = i & (npen == 8 ? 1 : 3);
#pragma unroll
      for (int u = 0; u < R; ++u) {
        T2 w = (sw & 1) ? v[u ^ 1] : v[u];
        if (npen == 4) {
          const T2 w2 = (sw & 1) ? v[u ^ 3] : v[u ^ 2];
          w = (sw & 2) ? w2 : w;
        }
        b[(j + (u ^ sw) * p) * npen + q] = w;
      }
    } else {
#pragma unroll
      for (int u = 0; u < R; ++u) b[(j + u * p) * npen + q] = v[u];
    }
  }
}

// Batched Stockham FFT in shared memory.  Element t of pencil q lives at
// a[t*npen + q]; consecutive threads take consecutive pencils; npen is a power
// of two.  Returns the buffer (a or b) that holds the result.  Ends with
// __syncthreads().
template <typename T2>
__device__ T2 *smem_fft(T2 *a, T2 *b, int npen, const FftPlan &pl, int sign,
                        const T2 *tws = nullptr) {
  const int lq = __ffs(npen) - 1;
  int p = 1;
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.radix[s];
    const unsigned pm = pl.pmag[s];
    if constexpr (sizeof(T2) == sizeof(float2)) {  // radices 16 and 8: FP32 plans only
      if (R == 16) {
        stockham_stage<16>(a, b, lq, pl, p, pm, sign, tws);
        goto staged;
      }
      if (R == 8) {
        stockham_stage<8>(a, b, lq, pl, p, pm, sign, tws);
        goto staged;
      }
    }
    switch (R) {
      case 4: stockham_stage<4>(a, b, lq, pl, p, pm, sign, tws); break;
      case 2: stockham_stage<2>(a, b, lq, pl, p, pm, sign, tws); break;
      case 3: stockham_stage<3>(a, b, lq, pl, p, pm, sign, tws); break;
      default: stockham_stage<5>(a, b, lq, pl, p, pm, sign, tws); break;
    }
  staged:
    __syncthreads();
    T2 *t = a;
    a = b;
    b = t;
    p *= R;
  }
  return a;
}

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

// Real-to-complex post-processing of npen x-rows held as Nx/2-point complex
// transforms z (row q at stride npen): X[k] = Fe[k] + W^k Fo[k], k <= Nx/2,
// stored to the half spectrum.
template <typename T2>
__device__ __forceinline__ void r2c_store(const Grid &g, const T2 *z, int npen, const FftPlan &pl,
                                          long long row0, long long nrows,
                                          const T2 *__restrict__ r2c_tw, T2 *__restrict__ spec) {
  using T = typename Cx<T2>::T;
  const int nxh = g.nxh, M = pl.n;
  for (int idx = threadIdx.x; idx < npen * nxh; idx += blockDim.x) {
    const int q = fdiv(idx, pl.nhmag), kx = idx - q * nxh;
    const long long row = row0 + q;
    if (row >= nrows) continue;
    T2 Z = z[(kx == M ? 0 : kx) * npen + q];
    T2 Zc = z[(kx == 0 ? 0 : M - kx) * npen + q];
    Zc.y = -Zc.y;
    T fer = (Z.x + Zc.x) * (T)0.5, fei = (Z.y + Zc.y) * (T)0.5;
    T dr = Z.x - Zc.x, di = Z.y - Zc.y;
    T for_ = di * (T)0.5, foi = -dr * (T)0.5;  // (Z - Zc) / (2i)
    T2 w = r2c_tw[kx];
    T xr = Cx<T2>::fma_(w.x, for_, Cx<T2>::fma_(-w.y, foi, fer));
    T xi = Cx<T2>::fma_(w.x, foi, Cx<T2>::fma_(w.y, for_, fei));
    spec[row * g.sxh + kx] = Cx<T2>::mk(xr, xi);
  }
}

// ------------------------------------------------- 1. residual + R2C along x
// poisson.cpp:399-404 (residual) and the first third of fft_3d (:431).
template <typename T2>
__global__ void k_xfwd_resid(Grid g, FftPlan pl, const T2 *__restrict__ r2c_tw,
                             const double *__restrict__ P, const double *__restrict__ Cf,
                             const double *__restrict__ cc, const double *__restrict__ RHS,
                             const DevScalars *__restrict__ s, T2 *__restrict__ spec, int npen) {
  if (s->skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using T = typename Cx<T2>::T;
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  const int M = pl.n;  // nx/2
  T2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  const double mean = s->mean_rhs;
  const double *Cx_ = Cf, *Cy_ = Cf + g.n, *Cz_ = Cf + 2 * g.n;
  // residual, written interleaved as z[m] = r[2m] + i r[2m+1]
  for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
    const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
    const long long row = row0 + q;
    double r = 0;
    if (row < nrows) {
      int j, k;
      row_jk(g, row, j, k);
      const long long c = at(g, i, j, k);
      const int ip = wrap_p(i, g.nx), im = wrap_m(i, g.nx);
      const int jp = wrap_p(j, g.ny), jm = wrap_m(j, g.ny);
      const int kp = wrap_p(k, g.nz), km = wrap_m(k, g.nz);
      const long long cxp = at(g, ip, j, k), cyp = at(g, i, jp, k), czp = at(g, i, j, kp);
      const double pc = P[c];
      // dummy = grad_C2F(P) * C at the low and high faces
      double gx_hi = (P[cxp] - pc) * g.inv_dx * Cx_[cxp];
      double gx_lo = (pc - P[at(g, im, j, k)]) * g.inv_dx * Cx_[c];
      double gy_hi = (P[cyp] - pc) * g.inv_dy * Cy_[cyp];
      double gy_lo = (pc - P[at(g, i, jm, k)]) * g.inv_dy * Cy_[c];
      double gz_hi = (P[czp] - pc) * g.inv_dz * Cz_[czp];
      double gz_lo = (pc - P[at(g, i, j, km)]) * g.inv_dz * Cz_[c];
      double rn = (gx_hi - gx_lo) * g.inv_dx + (gy_hi - gy_lo) * g.inv_dy + (gz_hi - gz_lo) * g.inv_dz;
      rn -= (RHS[c] - mean);
      rn *= cc[c];
      r = rn;
    }
    T *slot = reinterpret_cast<T *>(&a[(i >> 1) * npen + q]);
    slot[i & 1] = (T)r;
  }
  __syncthreads();
  T2 *z = smem_fft(a, b, npen, pl, -1);
  r2c_store(g, z, npen, pl, row0, nrows, r2c_tw, spec);
}

// Mixed path: the x-pass of one step of iterative refinement.  Iterations 0
// and 1 of a solve form the residual of P itself, div(C grad P) - (RHS -
// mean), from FP64 face differences P_nb - P (exact to rounding for the close
// values of neighbouring cells, and the kernel's only FP64 operations: seven
// per cell against the seventeen of an FP64 residual), each split into a
// float-float pair (tpm_ff.cuh), multiplied by Cs2 = C/d^2 and summed as
// pairs on the FP32 pipe.  Iteration 0 then corrects P directly; iteration 1
// stores its residual as R0 and starts a correction sum dP (a float-float
// pair per cell), and iteration k >= 2 forms R0 + div(C grad dP) with no FP64
// operation (correction form; P += dP once when the loop ends,
// k_refine_finish).  After the first correction dP is about 1e-6 of P, so
// the pair carries it and the rounding noise of the correction form, which
// scales with dP, lies far below that of an FP64 residual of P; R0's own
// rounding, made once, only shifts the fixed point (by about 1e-14 of P).
// The residual times cc is rounded to FP32 for the correction's FFT solve.
__global__ void k_xfwd_resid_refine(Grid g, FftPlan pl, const float2 *__restrict__ r2c_tw,
                                    const double *__restrict__ P, const float2 *__restrict__ dP,
                                    const float2 *__restrict__ Cs2, const float *__restrict__ cc32,
                                    const double *__restrict__ RHS,
                                    const DevScalars *__restrict__ s, float2 *__restrict__ R0,
                                    float2 *__restrict__ spec, int npen) {
  if (s->skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *a = reinterpret_cast<float2 *>(smem_raw);
  const int M = pl.n;  // nx/2
  float2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  const int it = s->it;
  const int nd = s->warm ? 1 : 2;  // direct iterations of this solve
  const bool direct = it < nd;
  const double mean = s->mean_rhs;
  const float2 *Cx_ = Cs2, *Cy_ = Cs2 + g.n, *Cz_ = Cs2 + 2 * g.n;
  // per pencil: its first cell and the offsets of its y and z neighbours
  // (wrapped), once per block instead of once per element
  __shared__ int rbase[kMaxPens], rym[kMaxPens], ryp[kMaxPens], rzm[kMaxPens], rzp[kMaxPens];
  for (int q = threadIdx.x; q < npen; q += blockDim.x) {
    const long long row = row0 + q;
    if (row < nrows) {
      int j, k;
      row_jk(g, row, j, k);
      const int nxy = g.nx * g.ny;
      rbase[q] = (int)at(g, 0, j, k);
      rym[q] = j == 0 ? (g.ny - 1) * g.nx : -g.nx;
      ryp[q] = j == g.ny - 1 ? -(g.ny - 1) * g.nx : g.nx;
      rzm[q] = k == 0 ? (g.nz - 1) * nxy : -nxy;
      rzp[q] = k == g.nz - 1 ? -(g.nz - 1) * nxy : nxy;
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
    const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
    const long long row = row0 + q;
    float r = 0.f;
    if (row < nrows) {
      const int c = rbase[q] + i;
      const int cxm = i == 0 ? c + g.nx - 1 : c - 1, cxp = i == g.nx - 1 ? c - g.nx + 1 : c + 1;
      const int cym = c + rym[q], cyp = c + ryp[q], czm = c + rzm[q], czp = c + rzp[q];
      float2 acc;
      if (direct) {
        acc = ff_from_double(mean - RHS[c]);
        const double pc = P[c];
        acc = ff_add(acc, ff_mul(Cx_[c], ff_from_double(P[cxm] - pc)));
        acc = ff_add(acc, ff_mul(Cx_[cxp], ff_from_double(P[cxp] - pc)));
        acc = ff_add(acc, ff_mul(Cy_[c], ff_from_double(P[cym] - pc)));
        acc = ff_add(acc, ff_mul(Cy_[cyp], ff_from_double(P[cyp] - pc)));
        acc = ff_add(acc, ff_mul(Cz_[c], ff_from_double(P[czm] - pc)));
        acc = ff_add(acc, ff_mul(Cz_[czp], ff_from_double(P[czp] - pc)));
        if (it == nd - 1) R0[c] = acc;
      } else {
        // (after the rebase dP is ~1e-6 of P: the one-TwoSum difference's
        // error, 2^-46 |dP|, lies near 1e-22 of P)
        acc = R0[c];
        const float2 dc = dP[c];
        acc = ff_add(acc, ff_mul(Cx_[c], ff_sub_sloppy(dP[cxm], dc)));
        acc = ff_add(acc, ff_mul(Cx_[cxp], ff_sub_sloppy(dP[cxp], dc)));
        acc = ff_add(acc, ff_mul(Cy_[c], ff_sub_sloppy(dP[cym], dc)));
        acc = ff_add(acc, ff_mul(Cy_[cyp], ff_sub_sloppy(dP[cyp], dc)));
        acc = ff_add(acc, ff_mul(Cz_[c], ff_sub_sloppy(dP[czm], dc)));
        acc = ff_add(acc, ff_mul(Cz_[czp], ff_sub_sloppy(dP[czp], dc)));
      }
      r = (acc.x + acc.y) * cc32[c];
    }
    float *slot = reinterpret_cast<float *>(&a[(i >> 1) * npen + q]);
    slot[i & 1] = r;
  }
  __syncthreads();
  float2 *z = smem_fft(a, b, npen, pl, -1);
  r2c_store(g, z, npen, pl, row0, nrows, r2c_tw, spec);
}

// Pencil tile load a[idx] = src(q, t) for idx = t*npen + q < total (npen =
// 2^lq): kBatch independent global loads in flight per thread before their
// shared-memory stores (a plain loop waits one L2 round trip per element).
template <int kBatch, typename T2, typename F>
__device__ __forceinline__ void tile_load(T2 *a, int total, int lq, F &&src) {
  for (int base = threadIdx.x; base < total; base += kBatch * blockDim.x) {
    T2 v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int idx = base + u * blockDim.x;
      v[u] = idx < total ? src(idx & ((1 << lq) - 1), idx >> lq) : Cx<T2>::mk(0, 0);
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx < total) a[idx] = v[u];
    }
  }
}

// ------------------------------------------------------- 2./4. y pencils
template <typename T2>
__global__ void k_fft_y(Grid g, FftPlan pl, T2 *__restrict__ spec, int npen, int sign,
                        const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lq = __ffs(npen) - 1;  // npen is a power of two
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  T2 *b = a + pl.n * npen;
  const int tiles = (g.nxh + npen - 1) / npen;
  const int kz = blockIdx.x / tiles, kx0 = (blockIdx.x % tiles) * npen;
  const long long base = (long long)kz * g.ny * g.sxh;
  tile_load<8>(a, npen * g.ny, lq, [&](int q, int ky) {
    return (kx0 + q < g.nxh) ? spec[base + (long long)ky * g.sxh + kx0 + q] : Cx<T2>::mk(0, 0);
  });
  __syncthreads();
  T2 *r = smem_fft(a, b, npen, pl, sign);
  for (int idx = threadIdx.x; idx < npen * g.ny; idx += blockDim.x) {
    const int q = idx & (npen - 1), ky = idx >> lq;
    if (kx0 + q < g.nxh) spec[base + (long long)ky * g.sxh + kx0 + q] = r[ky * npen + q];
  }
}

// 1/(ax[kx] + ay[ky] + az[kz]): FP64 on the FP64 path, FP32 for the mixed
// path's correction solve
template <typename T>
__device__ __forceinline__ T inv_mwn_at(const double *ax, const double *ay, const double *az,
                                        int kx, int ky, int kz);
template <>
__device__ __forceinline__ double inv_mwn_at<double>(const double *ax, const double *ay,
                                                     const double *az, int kx, int ky, int kz) {
  return 1.0 / (ax[kx] + ay[ky] + az[kz]);
}
template <>
__device__ __forceinline__ float inv_mwn_at<float>(const double *ax, const double *ay,
                                                   const double *az, int kx, int ky, int kz) {
  return 1.0f / ((float)ax[kx] + (float)ay[ky] + (float)az[kz]);
}

// the table of those reciprocals over the half spectrum (1 at the zero mode,
// which the solve leaves alone), built once per context
template <typename T>
__global__ void k_inv_mwn(Grid g, const double *__restrict__ ax, const double *__restrict__ ay,
                          const double *__restrict__ az, T *__restrict__ tab) {
  const long long total = (long long)g.nxh * g.ny * g.nz;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
       m += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(m % g.nxh);
    const long long r = m / g.nxh;
    const int ky = (int)(r % g.ny), kz = (int)(r / g.ny);
    tab[m] = (kx + ky + kz) > 0 ? inv_mwn_at<T>(ax, ay, az, kx, ky, kz) : (T)1;
  }
}

// ------------------------------------------- 3. z pencils + wave-number solve
template <typename T2>
__global__ void k_fft_z_solve(Grid g, FftPlan pl, T2 *__restrict__ spec, const double *__restrict__ ax,
                              const double *__restrict__ ay, const double *__restrict__ az,
                              const typename Cx<T2>::T *__restrict__ inv_mwn, int npen,
                              const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lq = __ffs(npen) - 1;  // npen is a power of two
  using T = typename Cx<T2>::T;
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  T2 *b = a + pl.n * npen;
  const int tiles = (g.nxh + npen - 1) / npen;
  const int ky = blockIdx.x / tiles, kx0 = (blockIdx.x % tiles) * npen;
  const long long plane = (long long)g.ny * g.sxh;
  const long long base = (long long)ky * g.sxh + kx0;
  const int tot = npen * g.nz;
  // the first kInvPre reciprocals of each thread's modes, loaded before the
  // pencils so that their latency hides behind the loads and the forward FFT
  constexpr int kInvPre = 8;
  T invr[kInvPre];
  if (inv_mwn) {
#pragma unroll
    for (int u = 0; u < kInvPre; ++u) {
      const int idx = threadIdx.x + u * (int)blockDim.x;
      const int q = idx & (npen - 1), kz = idx >> lq;
      invr[u] = (idx < tot && kx0 + q < g.nxh)
                    ? inv_mwn[((long long)kz * g.ny + ky) * g.nxh + kx0 + q]
                    : T(0);
    }
  }
  tile_load<8>(a, tot, lq, [&](int q, int kz) {
    return (kx0 + q < g.nxh) ? spec[base + kz * plane + q] : Cx<T2>::mk(0, 0);
  });
  __syncthreads();
  T2 *r = smem_fft(a, b, npen, pl, -1);
  T2 *other = (r == a) ? b : a;
  // divide by the modified wave number except the zero mode (poisson.cpp:442-449)
  int from = threadIdx.x;
  if (inv_mwn) {
#pragma unroll
    for (int u = 0; u < kInvPre; ++u) {
      const int idx = threadIdx.x + u * (int)blockDim.x;
      const int q = idx & (npen - 1), kz = idx >> lq;
      const int kx = kx0 + q;
      if (idx < tot && kx < g.nxh && (kx + ky + kz) > 0) {
        T2 v = r[kz * npen + q];
        v.y = v.y * invr[u];
        v.x = v.x * invr[u];
        r[kz * npen + q] = v;
      }
    }
    from += kInvPre * (int)blockDim.x;
  }
#pragma unroll 4
  for (int idx = from; idx < tot; idx += blockDim.x) {
    const int q = idx & (npen - 1), kz = idx >> lq;
    const int kx = kx0 + q;
    if (kx < g.nxh && (kx + ky + kz) > 0) {
      T2 v = r[kz * npen + q];
      // the reciprocal from the per-mode table (k_inv_mwn, same expression)
      // when there is one
      const T inv = inv_mwn ? inv_mwn[((long long)kz * g.ny + ky) * g.nxh + kx]
                            : inv_mwn_at<T>(ax, ay, az, kx, ky, kz);
      v.y = v.y * inv;
      v.x = v.x * inv;
      r[kz * npen + q] = v;
    }
  }
  __syncthreads();
  T2 *o = smem_fft(r, other, npen, pl, +1);
  for (int idx = threadIdx.x; idx < npen * g.nz; idx += blockDim.x) {
    const int q = idx & (npen - 1), kz = idx >> lq;
    if (kx0 + q < g.nxh) spec[base + kz * plane + q] = o[kz * npen + q];
  }
}

// ------------------------------------- 2.-4. y and z passes fed by the TMA
// Mixed path, pencils of at most 256 points: the y pass and the z pass (with
// the wave-number divide between its forward and inverse transforms) on tiles
// of 8 pencils moved by the tensor memory accelerator.  The blocks are
// persistent: each walks its share of the tiles, and while it transforms one
// tile the next one's box is already being loaded (cp.async.bulk.tensor into
// the other of two tile buffers, completion counted on that buffer's
// mbarrier); the result box goes back by a bulk tensor store that runs while
// the next tile is waited for.  A tile lands as [points][8 pencils], exactly
// the layout the Stockham stages read.  The bulk store skips the elements past
// the half spectrum's Nx/2 + 1 columns, so the last, partial tile needs no
// special case, and the spectrum's rows are padded to an even number of
// float2 so that a row is a 16-byte multiple, as a tensor map requires.
// Every wait is bounded (a timeout is recorded for the host).
constexpr int kTmaPens = 8;

// bytes of one tile buffer of n points, rounded to the 128-byte alignment a
// TMA box destination needs
__host__ __device__ __forceinline__ int tma_tile_bytes(int n) {
  return (n * kTmaPens * (int)sizeof(float2) + 127) & ~127;
}

// dynamic shared memory of k_fft_yz_tma: two tile buffers, the scratch
// buffer, the n twiddles (an eighth of a tile, 128-byte rounded) and two
// mbarriers; with one tile per block (ring = 1) a single tile buffer
__host__ __device__ __forceinline__ size_t tma_yz_smem(int n, int ring = 2) {
  return (ring + 1) * (size_t)tma_tile_bytes(n) + tma_tile_bytes(n) / kTmaPens + 16;
}

// z pass of a 256-point plan (two radix-16 stages), kFused: the forward
// transform's second stage leaves thread (i, q) < 128 holding modes
// kz = i + 16 u (u < 16) of pencil q, exactly the elements the inverse
// transform's first stage gives that thread.  So the second forward stage,
// the divide and the first inverse stage run in its registers, with no
// shared-memory round trip and no barrier between them; the arithmetic is
// the unfused path's, operation for operation.
template <bool kZ, bool kFused = false>
__global__ void __launch_bounds__(256, 4)
k_fft_yz_tma(Grid g, FftPlan pl, const __grid_constant__ CUtensorMap map, int sign,
             const float *__restrict__ inv_mwn, const int *__restrict__ skip,
             DevScalars *__restrict__ s, int ntiles, int ring) {
  if (skip && *skip) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tb = tma_tile_bytes(pl.n);
  // ring = 2: persistent blocks, the next tile loading into the other buffer;
  // ring = 1: one tile per block (the grid covers the tiles), one buffer
  auto buf = [&](int slot) { return reinterpret_cast<float2 *>(sm + slot * tb); };
  float2 *scratch = reinterpret_cast<float2 *>(sm + ring * tb);
  float2 *tw = reinterpret_cast<float2 *>(sm + (ring + 1) * tb);  // the plan's twiddles
  uint64_t *bar =
      reinterpret_cast<uint64_t *>(sm + (ring + 1) * tb + tma_tile_bytes(pl.n) / kTmaPens);
  constexpr int lq = 3;  // log2(kTmaPens)
  const int tiles = (g.nxh + kTmaPens - 1) / kTmaPens;
  const unsigned bytes = (unsigned)(pl.n * kTmaPens * sizeof(float2));
  const int tot = kTmaPens * pl.n;
  if ((smem_u32(sm) & 127u) || (ring == 1 && (int)gridDim.x < ntiles)) {
    // never issue a box to a misaligned address, nor to a buffer in use
    if (threadIdx.x == 0) s->timeout = 1;
    return;
  }
  // box coordinates of tile t: y pass (kx0, 0, kz), z pass (kx0, ky, 0)
  auto coords = [&](int t, int &x, int &y, int &z) {
    const int outer = t / tiles;
    x = (t - outer * tiles) * kTmaPens;
    y = kZ ? outer : 0;
    z = kZ ? 0 : outer;
  };
  auto load = [&](int t, int slot) {
    int x, y, z;
    coords(t, x, y, z);
    mbar_arrive_expect_tx(&bar[slot], bytes);
    tma_load_3d(buf(slot), &map, &bar[slot], x, y, z);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    if ((int)blockIdx.x < ntiles) load(blockIdx.x, 0);
  }
  // the plan's twiddles in shared memory (copied while the first tile loads:
  // the stages then read them without an L1 round trip)
  for (int m = threadIdx.x; m < pl.n; m += blockDim.x) tw[m] = pl.tw32[m];
  const float2 *tws = tw;
  __syncthreads();
  // a transform ends in its input buffer after an even number of Stockham
  // stages (the z pass runs two transforms of the same plan): then the store
  // of a tile reads only that tile's buffer, which the load two tiles later
  // refills, and only the thread that issues both waits for the store; else
  // (a y pass with an odd number of stages) the store reads the scratch buffer
  // the next transform writes, and the block waits for it
  const bool store_from_scratch = kFused || (!kZ && (pl.nst & 1));
  static_assert(kZ || !kFused, "only the z pass fuses its transforms");
  bool ok = true;
  int it = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
    const int slot = it & 1;
    if (threadIdx.x == 0) bulk_wait_read_all();  // the last store has read its buffer
    if (store_from_scratch) __syncthreads();
    if (threadIdx.x == 0 && t + (int)gridDim.x < ntiles) load(t + gridDim.x, slot ^ 1);
    int x, y, z;
    coords(t, x, y, z);
    // z pass: the reciprocals of this thread's modes (the table of
    // k_inv_mwn), loaded while the tile is in flight
    constexpr int kInv = kFused ? 16 : 8;  // tot <= 8 * 256 = 8 * blockDim.x
    float invr[kInv];
    if constexpr (kFused) {  // thread (i, q) < 128: modes kz = i + 16 u of pencil q
      const int kx = x + (threadIdx.x & 7), i = threadIdx.x >> 3;
#pragma unroll
      for (int u = 0; u < kInv; ++u)
        invr[u] = (threadIdx.x < 128 && kx < g.nxh)
                      ? inv_mwn[((long long)(i + 16 * u) * g.ny + y) * g.nxh + kx]
                      : 0.f;
    } else if constexpr (kZ) {
#pragma unroll
      for (int u = 0; u < kInv; ++u) {
        const int idx = threadIdx.x + u * (int)blockDim.x;
        const int q = idx & (kTmaPens - 1), kz = idx >> lq;
        invr[u] = (idx < tot && x + q < g.nxh)
                      ? inv_mwn[((long long)kz * g.ny + y) * g.nxh + x + q]
                      : 0.f;
      }
    }
    ok = mbar_wait(&bar[slot], (unsigned)(it >> 1) & 1u);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    float2 *r;
    if constexpr (kFused) {
      stockham_stage<16>(buf(slot), scratch, lq, pl, 1, pl.pmag[0], -1, tws);
      __syncthreads();
      if (threadIdx.x < 128) {
        const int i = threadIdx.x >> 3, q = threadIdx.x & 7, kx = x + q;
        float2 v[16];
        v[0] = scratch[i * kTmaPens + q];
#pragma unroll
        for (int t = 1; t < 16; ++t)
          v[t] = cmul(scratch[(i + 16 * t) * kTmaPens + q], tws ? tws[i * t] : pl.tw32[i * t], -1);
        dft16(v, -1);
        // divide by the modified wave number except the zero mode (poisson.cpp:442-449)
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          if (kx < g.nxh && (kx + y + i + 16 * u) > 0) {
            v[u].y = v[u].y * invr[u];
            v[u].x = v[u].x * invr[u];
          }
        }
        dft16(v, +1);
        // (odd i in swapped order: a store instruction covers both bank
        // halves, as in the first Stockham stage)
#pragma unroll
        for (int u = 0; u < 16; ++u)
          buf(slot)[(16 * i + (u ^ (i & 1))) * kTmaPens + q] = (i & 1) ? v[u ^ 1] : v[u];
      }
      __syncthreads();
      stockham_stage<16>(buf(slot), scratch, lq, pl, 16, pl.pmag[1], +1, tws);
      __syncthreads();
      r = scratch;
    } else {
      r = smem_fft(buf(slot), scratch, kTmaPens, pl, kZ ? -1 : sign, tws);
    }
    if constexpr (kZ && !kFused) {
      float2 *other = (r == scratch) ? buf(slot) : scratch;
      // divide by the modified wave number except the zero mode (poisson.cpp:442-449)
#pragma unroll
      for (int u = 0; u < kInv; ++u) {
        const int idx = threadIdx.x + u * (int)blockDim.x;
        const int q = idx & (kTmaPens - 1), kz = idx >> lq;
        const int kx = x + q;
        if (idx < tot && kx < g.nxh && (kx + y + kz) > 0) {
          float2 v = r[kz * kTmaPens + q];
          v.y = v.y * invr[u];
          v.x = v.x * invr[u];
          r[kz * kTmaPens + q] = v;
        }
      }
      __syncthreads();
      r = smem_fft(r, other, kTmaPens, pl, +1, tws);
    }
    fence_proxy_async();  // the transform's shared-memory writes, before the bulk store reads them
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store_3d(&map, r, x, y, z);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) {
    if (!ok) {
      s->timeout = 1;
      // let the loads still in flight land (bounded) before the block's
      // shared memory is released
      mbar_wait(&bar[it & 1], (unsigned)(it >> 1) & 1u);
      if (ring == 2) mbar_wait(&bar[(it + 1) & 1], (unsigned)((it + 1) >> 1) & 1u);
    }
    bulk_wait_read_all();
  }
}

// A block's max|dp| (>= 0): into the iteration's accumulator by an atomic
// maximum on the bits (non-negative doubles order as their bit patterns, and
// a maximum does not depend on the order the blocks arrive in), or into the
// block's partial slot when there is no accumulator
__device__ __forceinline__ void put_block_max(double v, double *partials,
                                              unsigned long long *err_acc) {
  if (err_acc)
    atomicMax(err_acc, (unsigned long long)__double_as_longlong(v));
  else
    partials[blockIdx.x] = v;
}

// ------------------------------------------- 5. C2R along x + P update
template <typename T2>
__global__ void k_xinv_update(Grid g, FftPlan pl, const T2 *__restrict__ r2c_tw,
                              const T2 *__restrict__ spec, double *__restrict__ P,
                              double *__restrict__ partials, int npen,
                              const int *__restrict__ skip, float2 *__restrict__ dP,
                              const int *__restrict__ it, const int *__restrict__ warm,
                              double inv_tot, unsigned long long *__restrict__ err_acc) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double sh[32];
  __shared__ float shf[32];
  using T = typename Cx<T2>::T;
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  const int M = pl.n;
  T2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  const int sxh = g.sxh;
  // Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) W^-k, k < M;
  // kB elements' loads in flight per thread before their stores
  constexpr int kB = 4;
  for (int base = threadIdx.x; base < npen * M; base += kB * blockDim.x) {
    T2 X[kB], Y[kB], W[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int idx = base + u * blockDim.x;
      const int q = fdiv(idx, pl.nmag), kx = idx - q * M;
      const long long row = row0 + q;
      const bool ok = idx < npen * M && row < nrows;
      X[u] = ok ? spec[row * sxh + kx] : Cx<T2>::mk(0, 0);
      Y[u] = ok ? spec[row * sxh + (M - kx)] : Cx<T2>::mk(0, 0);
      W[u] = ok ? r2c_tw[kx] : Cx<T2>::mk(0, 0);  // exp(-2 pi i k / nx); use its conjugate
    }
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx >= npen * M) break;
      const int q = fdiv(idx, pl.nmag), kx = idx - q * M;
      const T2 Xv = X[u], w = W[u];
      const T yr = Y[u].x, yi = -Y[u].y;
      T fer = Xv.x + yr, fei = Xv.y + yi;
      T dr = Xv.x - yr, di = Xv.y - yi;
      T for_ = Cx<T2>::fma_(dr, w.x, di * w.y);
      T foi = Cx<T2>::fma_(di, w.x, -dr * w.y);
      a[kx * npen + q] = Cx<T2>::mk(fer - foi, fei + for_);  // Fe + i Fo (0 past the rows)
    }
  }
  __syncthreads();
  T2 *z = smem_fft(a, b, npen, pl, +1);
  // inv_tot = 1/(Nx Ny Nz) from the host (an FP64 division per thread would
  // cost about as much as the update itself on this FP64 pipe)
  double mx = 0;
  if (sizeof(T) == sizeof(float)) {
    // mixed path: the correction dp = -x/N^3, formed in FP32, goes to P at
    // iteration 0 of a cold solve (converted exactly, one FP64 operation per
    // cell), starts the solve's float-float correction sum dP at the last
    // direct iteration (0 warm, 1 cold) and joins it after (P += dP in
    // k_refine_finish).  max|x| in FP32 (exact: the maximum picks one x,
    // scaled once below).
    const int itv = *it;
    const int nd = *warm ? 1 : 2;  // direct iterations of this solve
    const float inv_tot_f = 1.0f / (float)((long long)g.nx * g.ny * g.nz);
    float mxf = 0.f;
    // kB elements per thread at a time: their P or dP loads in flight together
    for (int base = threadIdx.x; base < npen * g.nx; base += kB * blockDim.x) {
      float2 old[kB];
      double pold[kB];
#pragma unroll
      for (int u = 0; u < kB; ++u) {
        const int idx = base + u * blockDim.x;
        const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
        const long long row = row0 + q;
        const bool ok = idx < npen * g.nx && row < nrows;
        const long long c = row * g.nx + i;
        old[u] = ok && itv >= nd ? dP[c] : make_float2(0.f, 0.f);
        pold[u] = ok && itv < nd - 1 ? P[c] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kB; ++u) {
        const int idx = base + u * blockDim.x;
        const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
        const long long row = row0 + q;
        if (idx >= npen * g.nx || row >= nrows) continue;
        const T *zz = reinterpret_cast<const T *>(&z[(i >> 1) * npen + q]);
        const float xf = (float)zz[i & 1];
        const long long c = row * g.nx + i;
        const float dp = -(xf * inv_tot_f);
        if (itv < nd - 1)
          P[c] = pold[u] + ff_f2d(dp);
        else
          dP[c] = itv == nd - 1 ? make_float2(dp, 0.f) : ff_add_f(old[u], dp);
        const float ax = fabsf(xf);
        mxf = ax > mxf ? ax : mxf;
      }
    }
    // the block maximum in FP32 too (FP64 compares issue on the FP64 pipe);
    // one conversion and one product per block
    const float bm = block_max(mxf, shf);
    if (threadIdx.x == 0) put_block_max(ff_f2d(bm) * inv_tot, partials, err_acc);
    return;
  } else {
    for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
      const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
      const long long row = row0 + q;
      if (row >= nrows) continue;
      const T *zz = reinterpret_cast<const T *>(&z[(i >> 1) * npen + q]);
      double x = (double)zz[i & 1];
      double dp = -(x * inv_tot);  // poisson.cpp:460, (-1)*re/N^3
      const long long c = row * g.nx + i;
      P[c] += dp;
      double ad = fabs(dp);
      mx = ad > mx ? ad : mx;
    }
  }
  double bm = block_max(mx, sh);
  if (threadIdx.x == 0) put_block_max(bm, partials, err_acc);
}

// max|dp| of the iteration (poisson.cpp:407) and the loop test of
// poisson.cpp:397 for iterations run from a graph: with a conditional handle
// (loop_max > 0) the enclosing while node repeats while it < max_it and
// max|dp| > epsilon; without one, a satisfied test turns the remaining
// unrolled iterations into no-ops (skip).  `it` counts up by one per
// iteration, so the loop ends after at most loop_max bodies.
__global__ void k_finish_max(const double *__restrict__ partials, int nparts, DevScalars *s,
                             double eps_ctl, cudaGraphConditionalHandle loop, int loop_max,
                             unsigned long long *__restrict__ err_acc) {
  if (loop_max == 0 && s->skip) return;
  __shared__ double sh[32];
  double m;
  if (err_acc) {  // the blocks' atomic maximum; cleared for the next iteration
    m = __longlong_as_double((long long)*err_acc);
  } else {
    double v = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v = partials[b] > v ? partials[b] : v;
    m = block_max(v, sh);
  }
  if (threadIdx.x == 0) {
    if (err_acc) *err_acc = 0ull;
    s->err = m;
    s->it += 1;
    s->it_sum += 1;
    // poisson.cpp:397: while (i < Iteration && error > epsilon) - for every
    // epsilon, so with epsilon = 0 a solve stops once max|dp| is exactly 0
    // (a NaN error stops it too); callers that never stop pass a negative one
    const bool more = m > eps_ctl;
    if (loop_max > 0)
      cudaGraphSetConditional(loop, (s->it < loop_max && more) ? 1u : 0u);
    else if (!more)
      s->skip = 1;
  }
}

// End of a mixed refinement loop that started the correction sum (at least
// as many iterations as the solve's direct ones ran): P += dP
__global__ void k_refine_finish(Grid g, const float2 *__restrict__ dP,
                                const DevScalars *__restrict__ s, double *__restrict__ P) {
  if (s->it < (s->warm ? 1 : 2)) return;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const float2 d = dP[c];
    P[c] = (P[c] + ff_f2d(d.x)) + ff_f2d(d.y);
  }
}

// pencils per block: two ping-pong buffers of 32 KB each, a power of two
int pens_for(int n, int elem_bytes = 16) {
  int cap = (kFftSmemPoints * 16 / elem_bytes) / n;
  if (cap > 32) cap = 32;
  int p = 1;
  while (2 * p <= cap) p *= 2;
  return p;
}


// Radices of an n-point plan: 4, 2, 3, 5 (the FP64 passes); with big, 16 and
// 8 first (the FP32 passes: half the shared-memory stages of radix 4, each
// butterfly in registers)
void factorize(int n, FftPlan &pl, bool big = false) {
  pl.n = n;
  pl.nst = 0;
  int m = n;
  while (big && m % 16 == 0) { pl.radix[pl.nst++] = 16; m /= 16; }
  while (big && m % 8 == 0) { pl.radix[pl.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { pl.radix[pl.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { pl.radix[pl.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { pl.radix[pl.nst++] = 3; m /= 3; }
  while (m % 5 == 0) { pl.radix[pl.nst++] = 5; m /= 5; }
  if (m != 1) throw std::string("grid size must factor into 2, 3 and 5");
  int p = 1;
  for (int st = 0; st < pl.nst; ++st) {
    pl.pmag[st] = fdiv_magic(p);
    p *= pl.radix[st];
  }
  pl.nmag = fdiv_magic(n);
  pl.n2mag = fdiv_magic(2 * n);
  pl.nhmag = fdiv_magic(n + 1);
}

}  // namespace

// modified wave number tables, evaluated with the host libm exactly as
// poisson.cpp:433-447 writes them:  a_x[i] = (2/dx^2)*(1-cos(kk_i*dx)) with
// kk_i = ((i<nx/2)?i:i-nx)*2pi/Lx.
static void mwn_table(int n, double L, double d, std::vector<double> &t, int count) {
  double TWO_PI(2 * 3.141592653589793);
  double two_pi_over_L = TWO_PI / L;
  double d2 = 2. / (d * d);
  t.resize(count);
  for (int i = 0; i < count; ++i) {
    double kk = ((i < n / 2) ? i : i - n) * two_pi_over_L;
    t[i] = (d2) * (1 - cos(kk * d));
  }
}

void fft_plans_create(tpm_ctx *c) {
  const Grid &g = c->g;
  if (g.nx % 2) throw std::string("Nx must be even (real-to-complex x pass)");
  factorize(g.nx / 2, c->fx);
  factorize(g.ny, c->fy);
  factorize(g.nz, c->fz);
  c->pen[0] = pens_for(c->fx.n);
  c->pen[1] = pens_for(c->fy.n);
  c->pen[2] = pens_for(c->fz.n);
  // twiddles: one block of [n] double2 + [n] float2 per plan, plus the r2c table
  auto table = [](int n, std::vector<double2> &d, std::vector<float2> &f) {
    d.resize(n);
    f.resize(n);
    for (int m = 0; m < n; ++m) {
      double a = 2.0 * 3.14159265358979323846 * (double)m / (double)n;
      d[m] = make_double2(cos(a), -sin(a));
      f[m] = make_float2((float)d[m].x, (float)d[m].y);
    }
  };
  std::vector<double2> dx_, dy_, dz_, dr;
  std::vector<float2> fx_, fy_, fz_, fr;
  table(c->fx.n, dx_, fx_);
  table(c->fy.n, dy_, fy_);
  table(c->fz.n, dz_, fz_);
  table(g.nx, dr, fr);  // r2c post-processing uses W^k, k <= nx/2
  std::vector<double> ax, ay, az;
  mwn_table(g.nx, g.Lx, g.dx, ax, g.nxh);
  mwn_table(g.ny, g.Ly, g.dy, ay, g.ny);
  mwn_table(g.nz, g.Lz, g.dz, az, g.nz);
  size_t n64 = dx_.size() + dy_.size() + dz_.size() + dr.size();
  size_t bytes = n64 * (sizeof(double2) + sizeof(float2)) + (ax.size() + ay.size() + az.size()) * 8;
  char *mem = nullptr;
  TPM_CUDA_TRY(cudaMalloc(&mem, bytes + 256));
  c->fft_mem = mem;
  double2 *d64 = reinterpret_cast<double2 *>(mem);
  float2 *d32 = reinterpret_cast<float2 *>(d64 + n64);
  double *tabs = reinterpret_cast<double *>(d32 + n64);
  size_t o = 0;
  auto put = [&](std::vector<double2> &d, std::vector<float2> &f, FftPlan *pl) -> size_t {
    TPM_CUDA_TRY(cudaMemcpy(d64 + o, d.data(), d.size() * sizeof(double2), cudaMemcpyHostToDevice));
    TPM_CUDA_TRY(cudaMemcpy(d32 + o, f.data(), f.size() * sizeof(float2), cudaMemcpyHostToDevice));
    if (pl) {
      pl->tw64 = d64 + o;
      pl->tw32 = d32 + o;
    }
    size_t at0 = o;
    o += d.size();
    return at0;
  };
  put(dx_, fx_, &c->fx);
  put(dy_, fy_, &c->fy);
  put(dz_, fz_, &c->fz);
  // the FP32 plans: the same tables, radices 16 and 8 first
  c->fx32 = c->fx;
  c->fy32 = c->fy;
  c->fz32 = c->fz;
  factorize(c->fx.n, c->fx32, true);
  factorize(c->fy.n, c->fy32, true);
  factorize(c->fz.n, c->fz32, true);
  size_t r0 = put(dr, fr, nullptr);
  c->r2c64 = d64 + r0;
  c->r2c32 = d32 + r0;
  c->ax = tabs;
  c->ay = tabs + ax.size();
  c->az = tabs + ax.size() + ay.size();
  TPM_CUDA_TRY(cudaMemcpy(c->ax, ax.data(), ax.size() * 8, cudaMemcpyHostToDevice));
  TPM_CUDA_TRY(cudaMemcpy(c->ay, ay.data(), ay.size() * 8, cudaMemcpyHostToDevice));
  TPM_CUDA_TRY(cudaMemcpy(c->az, az.data(), az.size() * 8, cudaMemcpyHostToDevice));
  {  // per-mode reciprocals of the wave-number sum for the z-pass solve
    const long long nmodes = (long long)g.nxh * g.ny * g.nz;
    const int blocks = (int)std::min<long long>((nmodes + 255) / 256, 4096);
    if (c->p.precision == TPM_PREC_MIXED) {
      float *t = dalloc<float>(c, nmodes);
      k_inv_mwn<float><<<blocks, 256, 0, c->stream>>>(g, c->ax, c->ay, c->az, t);
      c->inv_mwn = t;
    } else {
      double *t = dalloc<double>(c, nmodes);
      k_inv_mwn<double><<<blocks, 256, 0, c->stream>>>(g, c->ax, c->ay, c->az, t);
      c->inv_mwn = t;
    }
    TPM_CUDA_TRY(cudaGetLastError());
  }
  // dynamic shared memory above 48 KB
  int smem64 = 2 * kFftSmemPoints * (int)sizeof(double2);
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_xfwd_resid<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_fft_y<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_fft_z_solve<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_xinv_update<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_xfwd_resid_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_fft_y<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_fft_z_solve<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_xinv_update<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  // the Richardson loop's spectrum: FP64 rows of Nx/2 + 1 double2; on the
  // mixed path rows of an even number of float2 (the buffer holds double2
  // rows, so the padded float2 rows fit), and where the pencils of the y and z
  // passes fit one TMA box (at most 256 points) the tile maps of those passes
  c->spec_pitch = g.nxh;
  c->tma_fft = false;
  if (c->p.precision == TPM_PREC_MIXED) {
    c->spec_pitch = g.nxh + (g.nxh & 1);
    if (g.ny <= 256 && g.nz <= 256 &&
        make_tensor_map_8b(&c->fft_map_y, c->spec, g.nxh, g.ny, g.nz, c->spec_pitch, kTmaPens,
                           g.ny, 1) &&
        make_tensor_map_8b(&c->fft_map_z, c->spec, g.nxh, g.ny, g.nz, c->spec_pitch, kTmaPens, 1,
                           g.nz)) {
      // persistent blocks: as many as stay resident (SMs x blocks per SM)
      const int ns[3] = {c->fy32.n, c->fz32.n, c->fz32.n};
      const void *kern[3] = {reinterpret_cast<const void *>(k_fft_yz_tma<false>),
                             reinterpret_cast<const void *>(k_fft_yz_tma<true>),
                             reinterpret_cast<const void *>(k_fft_yz_tma<true, true>)};
      bool fits = true;
      for (int d = 0; d < 3; ++d) {
        // (the attribute belongs to the kernel, not to this context: it is set
        // to the largest pencil the pass takes, so that contexts of different
        // grids in one process never lower it below another's launches)
        const int smem = (int)tma_yz_smem(ns[d]);
        TPM_CUDA_TRY(cudaFuncSetAttribute(kern[d], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)tma_yz_smem(256)));
        int per_sm = 0;
        TPM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern[d], 256, smem));
        if (d < 2) c->tma_fft_blocks[d] = per_sm * (c->sms > 0 ? c->sms : 1);
        fits = fits && per_sm > 0;
      }
      c->tma_fft = fits;
      c->tma_y = c->tma_z = fits;
    }
  }
}

// One Richardson iteration of poisson::FFT (poisson.cpp:397-409).  Inputs:
// P, c->Cface, c->cc, c->RHS and dsc->mean_rhs.  Output: P updated and
// dsc->err = max|dp|.  T2 is the type of the constant-coefficient FFT solve:
// double2 on the FP64 path (FP64 residual and update); float2 on the mixed
// path, where each iteration is one step of iterative refinement: float-float
// residual (c->Cs2, c->cc32) from FP64 face differences of P, FP32
// correction, then from the third iteration on the correction form (c->R0
// and the float-float correction sum c->dP) with P += dP once the loop ends
// (refine_finish).
template <typename T2>
static void poisson_iteration_t(tpm_ctx *c, double eps_ctl, const LoopCtl *loop) {
  Grid g = c->g;
  g.sxh = c->spec_pitch;  // the loop's spectrum rows (padded on the mixed path)
  constexpr bool f32 = sizeof(T2) == sizeof(float2);
  const FftPlan &plx = f32 ? c->fx32 : c->fx, &ply = f32 ? c->fy32 : c->fy,
                &plz = f32 ? c->fz32 : c->fz;
  const long long nrows = (long long)g.ny * g.nz;
  T2 *spec = reinterpret_cast<T2 *>(c->spec);
  const T2 *r2c = sizeof(T2) == sizeof(double2) ? reinterpret_cast<const T2 *>(c->r2c64)
                                                : reinterpret_cast<const T2 *>(c->r2c32);
  const int *skip = &c->dsc->skip;
  const int npx = c->pen[0], npy = c->pen[1], npz = c->pen[2];
  const int tx = c->fthreads[0], ty = c->fthreads[1], tz = c->fthreads[2];
  const int xblocks = (int)((nrows + npx - 1) / npx);
  {
    size_t smem = 2 * (size_t)npx * plx.n * sizeof(T2);
    if constexpr (sizeof(T2) == sizeof(float2))
      TPM_LAUNCH(c, "fft_x_fwd_resid", k_xfwd_resid_refine, xblocks, tx, smem, g, plx, r2c,
                 c->P, c->dP, c->Cs2, c->cc32, c->RHS, c->dsc, c->R0, spec, npx);
    else
      TPM_LAUNCH(c, "fft_x_fwd_resid", k_xfwd_resid<T2>, xblocks, tx, smem, g, plx, r2c,
                 c->P, c->Cface, c->cc, c->RHS, c->dsc, spec, npx);
  }
  const int tma_tiles = (g.nxh + kTmaPens - 1) / kTmaPens;
  auto y_pass = [&](int sign) {
    if (f32 && c->tma_y) {
      const int ntiles = g.nz * tma_tiles;
      // one tile per block, 128 threads (a stage's items): more blocks resident
      // than persistent 256-thread blocks with two tile buffers
      TPM_LAUNCH(c, "fft_y", k_fft_yz_tma<false>, ntiles, 128, tma_yz_smem(ply.n, 1), g, ply,
                 c->fft_map_y, sign, static_cast<const float *>(nullptr), skip, c->dsc, ntiles,
                 1);
      return;
    }
    int blocks = g.nz * ((g.nxh + npy - 1) / npy);
    size_t smem = 2 * (size_t)npy * ply.n * sizeof(T2);
    TPM_LAUNCH(c, "fft_y", k_fft_y<T2>, blocks, ty, smem, g, ply, spec, npy, sign, skip);
  };
  y_pass(-1);
  if (f32 && c->tma_z) {
    const int ntiles = g.ny * tma_tiles;
    // (one tile per block: the z pass's two transforms give its blocks enough
    // work between loads, and its tiles load while other blocks compute;
    // persistent blocks measured the same, 1.05 ms per 256^3 step; 128
    // threads, one per item of a stage, where the divide allows)
    if (plz.nst == 2 && plz.radix[0] == 16 && plz.radix[1] == 16)
      TPM_LAUNCH(c, "fft_z_solve", (k_fft_yz_tma<true, true>), ntiles, 128,
                 tma_yz_smem(plz.n, 1), g, plz, c->fft_map_z, -1,
                 static_cast<const float *>(c->inv_mwn), skip, c->dsc, ntiles, 1);
    else  // (its divide preloads 8 modes per thread: 256 threads)
      TPM_LAUNCH(c, "fft_z_solve", k_fft_yz_tma<true>, ntiles, 256,
                 tma_yz_smem(plz.n, 1), g, plz, c->fft_map_z, -1,
                 static_cast<const float *>(c->inv_mwn), skip, c->dsc, ntiles, 1);
  } else {
    int blocks = g.ny * ((g.nxh + npz - 1) / npz);
    size_t smem = 2 * (size_t)npz * plz.n * sizeof(T2);
    TPM_LAUNCH(c, "fft_z_solve", k_fft_z_solve<T2>, blocks, tz, smem, g, plz, spec,
               c->ax, c->ay, c->az, static_cast<const typename Cx<T2>::T *>(c->inv_mwn), npz, skip);
  }
  y_pass(+1);
  {
    size_t smem = 2 * (size_t)npx * plx.n * sizeof(T2);
    double *parts = c->err_parts;
    TPM_LAUNCH(c, "fft_x_inv_update", k_xinv_update<T2>, xblocks, tx, smem, g, plx,
               r2c, spec, c->P, parts, npx, skip, c->dP, &c->dsc->it, &c->dsc->warm,
               1.0 / (double)((long long)g.nx * g.ny * g.nz), &c->dsc->err_acc);
    TPM_LAUNCH(c, "finish_max", k_finish_max, 1, 32, 0, parts, xblocks, c->dsc, eps_ctl,
               loop ? loop->handle : cudaGraphConditionalHandle{}, loop ? loop->max_it : 0,
               &c->dsc->err_acc);
  }
}

// the following solves of the step start from this one's P: warm
__global__ void k_mark_warm(DevScalars *s) { s->warm = 1; }

__global__ void k_loop_begin(DevScalars *s) {
  s->skip = 0;
  s->it = 0;
  s->err = 100;
}

void poisson_loop_begin(tpm_ctx *c) {
  TPM_LAUNCH(c, "poisson_begin", k_loop_begin, 1, 1, 0, c->dsc);
}

void refine_finish(tpm_ctx *c) {
  TPM_LAUNCH(c, "refine_finish", k_refine_finish, cell_blocks(c->g), 256, 0, c->g, c->dP,
             c->dsc, c->P);
  TPM_LAUNCH(c, "refine_finish", k_mark_warm, 1, 1, 0, c->dsc);
}

void poisson_iteration(tpm_ctx *c, double eps_ctl, const LoopCtl *loop) {
  if (c->p.precision == TPM_PREC_MIXED)
    poisson_iteration_t<float2>(c, eps_ctl, loop);
  else
    poisson_iteration_t<double2>(c, eps_ctl, loop);
}

int pens_default(int n, int elem_bytes) { return pens_for(n, elem_bytes); }
int pens_max(int n, int elem_bytes) {
  return pens_for(n, elem_bytes);  // both buffers within the 64 KB set per kernel
}

}  // namespace tpm

namespace tpm {

// ---------------------------------------------------------- energy spectrum
// Forward 3-D transform of one real face-velocity component with the same
// pencil passes (no residual, no solve), then |X/N^3|^2/2 per half-spectrum
// mode, doubled for 0 < kx < Nx/2 (their conjugates are not stored), summed
// over the three components into emode[(kz*Ny + ky)*(Nx/2+1) + kx].
namespace {

__global__ void k_spec_xfwd(Grid g, FftPlan pl, const double2 *__restrict__ r2c_tw,
                            const double *__restrict__ f, double2 *__restrict__ spec, int npen) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *a = reinterpret_cast<double2 *>(smem_raw);
  const int M = pl.n;
  double2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
    const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
    const long long row = row0 + q;
    double *slot = reinterpret_cast<double *>(&a[(i >> 1) * npen + q]);
    slot[i & 1] = row < nrows ? f[row * g.nx + i] : 0.0;
  }
  __syncthreads();
  double2 *z = smem_fft(a, b, npen, pl, -1);
  r2c_store(g, z, npen, pl, row0, nrows, r2c_tw, spec);
}

__global__ void k_spec_z_energy(Grid g, FftPlan pl, const double2 *__restrict__ spec,
                                double *__restrict__ emode, int npen, int accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lq = __ffs(npen) - 1;  // npen is a power of two
  double2 *a = reinterpret_cast<double2 *>(smem_raw);
  double2 *b = a + pl.n * npen;
  const int tiles = (g.nxh + npen - 1) / npen;
  const int ky = blockIdx.x / tiles, kx0 = (blockIdx.x % tiles) * npen;
  const long long plane = (long long)g.ny * g.nxh;
  const long long base = (long long)ky * g.nxh + kx0;
  for (int idx = threadIdx.x; idx < npen * g.nz; idx += blockDim.x) {
    const int q = idx & (npen - 1), kz = idx >> lq;
    a[kz * npen + q] = (kx0 + q < g.nxh) ? spec[base + kz * plane + q] : make_double2(0, 0);
  }
  __syncthreads();
  const double2 *r = smem_fft(a, b, npen, pl, -1);
  const double inv_tot = 1.0 / ((double)g.nx * (double)g.ny * (double)g.nz);
  for (int idx = threadIdx.x; idx < npen * g.nz; idx += blockDim.x) {
    const int q = idx & (npen - 1), kz = idx >> lq;
    const int kx = kx0 + q;
    if (kx >= g.nxh) continue;
    const double2 v = r[kz * npen + q];
    const double ur = v.x * inv_tot, ui = v.y * inv_tot;
    const double w = (kx == 0 || 2 * kx == g.nx) ? 0.5 : 1.0;
    const double e = w * (ur * ur + ui * ui);
    const long long m = base + kz * plane + q;
    emode[m] = accumulate ? emode[m] + e : e;
  }
}

}  // namespace

void spectrum_mode_energy(tpm_ctx *c, const double *U3, double2 *spec, double *emode) {
  const Grid &g = c->g;
  const long long nrows = (long long)g.ny * g.nz;
  for (int d = 0; d < 3; ++d) {
    {
      int npen = pens_for(c->fx.n);
      int blocks = (int)((nrows + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * c->fx.n * sizeof(double2);
      TPM_LAUNCH(c, "spec_x", k_spec_xfwd, blocks, kFftThreads, smem, g, c->fx, c->r2c64,
                 U3 + d * g.n, spec, npen);
    }
    {
      int npen = pens_for(c->fy.n);
      int blocks = g.nz * ((g.nxh + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * c->fy.n * sizeof(double2);
      TPM_LAUNCH(c, "spec_y", k_fft_y<double2>, blocks, kFftThreads, smem, g, c->fy, spec, npen,
                 -1, nullptr);
    }
    {
      int npen = pens_for(c->fz.n);
      int blocks = g.ny * ((g.nxh + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * c->fz.n * sizeof(double2);
      TPM_LAUNCH(c, "spec_z_energy", k_spec_z_energy, blocks, kFftThreads, smem, g, c->fz, spec,
                 emode, npen, d > 0);
    }
  }
}

// ------------------------------------------------ FFT preconditioner (PCG)
// z = M^-1 r with M^-1 = S (-Lap_h)^-1 S, S = diag(sc): the Richardson loop's
// preconditioner (poisson.cpp:393-394 scale by -1/I_F2C(C), then the
// constant-coefficient spectral solve) in its symmetric form, sc = 1/sqrt(C_c)
// at the cell centres, so that it can precondition conjugate gradients.
// x-pass forward of sc*r, y forward, z forward + divide by the modified wave
// number + z inverse, y inverse, x-pass inverse storing z = sc*x/N^3 with
// per-block partials of r.z.
namespace {

template <typename T2>
__global__ void k_pc_xfwd(Grid g, FftPlan pl, const T2 *__restrict__ r2c_tw,
                          const double *__restrict__ r, const double *__restrict__ sc,
                          T2 *__restrict__ spec, int npen, const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using T = typename Cx<T2>::T;
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  const int M = pl.n;
  T2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
    const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
    const long long row = row0 + q;
    T *slot = reinterpret_cast<T *>(&a[(i >> 1) * npen + q]);
    const long long c = row * g.nx + i;
    slot[i & 1] = row < nrows ? (T)(r[c] * sc[c]) : (T)0;
  }
  __syncthreads();
  T2 *z = smem_fft(a, b, npen, pl, -1);
  r2c_store(g, z, npen, pl, row0, nrows, r2c_tw, spec);
}

template <typename T2>
__global__ void k_pc_xinv(Grid g, FftPlan pl, const T2 *__restrict__ r2c_tw,
                          const T2 *__restrict__ spec, const double *__restrict__ r,
                          const double *__restrict__ sc, double *__restrict__ zout,
                          double *__restrict__ partials, int npen, const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double sh[32];
  using T = typename Cx<T2>::T;
  T2 *a = reinterpret_cast<T2 *>(smem_raw);
  const int M = pl.n;
  T2 *b = a + M * npen;
  const long long nrows = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * npen;
  for (int idx = threadIdx.x; idx < npen * M; idx += blockDim.x) {
    const int q = fdiv(idx, pl.nmag), kx = idx - q * M;
    const long long row = row0 + q;
    T2 Z = Cx<T2>::mk(0, 0);
    if (row < nrows) {
      T2 X = spec[row * g.sxh + kx];
      T2 Y = spec[row * g.sxh + (M - kx)];
      Y.y = -Y.y;
      T fer = X.x + Y.x, fei = X.y + Y.y;
      T dr = X.x - Y.x, di = X.y - Y.y;
      T2 w = r2c_tw[kx];
      T for_ = Cx<T2>::fma_(dr, w.x, di * w.y);
      T foi = Cx<T2>::fma_(di, w.x, -dr * w.y);
      Z = Cx<T2>::mk(fer - foi, fei + for_);
    }
    a[kx * npen + q] = Z;
  }
  __syncthreads();
  T2 *zz = smem_fft(a, b, npen, pl, +1);
  const double inv_tot = 1.0 / (double)(g.nx * g.ny * g.nz);
  double acc = 0;
  for (int idx = threadIdx.x; idx < npen * g.nx; idx += blockDim.x) {
    const int q = fdiv(idx, pl.n2mag), i = idx - q * g.nx;
    const long long row = row0 + q;
    if (row >= nrows) continue;
    const T *v = reinterpret_cast<const T *>(&zz[(i >> 1) * npen + q]);
    const long long c = row * g.nx + i;
    const double zc = ((double)v[i & 1] * inv_tot) * sc[c];
    zout[c] = zc;
    acc += r[c] * zc;
  }
  double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bs;
}

template <typename T2>
void precondition_t(tpm_ctx *c, const double *r, const double *sc, double *z, double *parts,
                    const int *skip) {
  const Grid &g = c->g;
  constexpr bool f32 = sizeof(T2) == sizeof(float2);
  const FftPlan &plx = f32 ? c->fx32 : c->fx, &ply = f32 ? c->fy32 : c->fy,
                &plz = f32 ? c->fz32 : c->fz;
  const long long nrows = (long long)g.ny * g.nz;
  T2 *spec = reinterpret_cast<T2 *>(c->spec);
  const T2 *r2c = sizeof(T2) == sizeof(double2) ? reinterpret_cast<const T2 *>(c->r2c64)
                                                : reinterpret_cast<const T2 *>(c->r2c32);
  const int npx = c->pen[0], npy = c->pen[1], npz = c->pen[2];
  const int tx = c->fthreads[0], ty = c->fthreads[1], tz = c->fthreads[2];
  const int xblocks = (int)((nrows + npx - 1) / npx);
  const size_t sx = 2 * (size_t)npx * plx.n * sizeof(T2);
  const size_t sy = 2 * (size_t)npy * ply.n * sizeof(T2);
  const size_t sz = 2 * (size_t)npz * plz.n * sizeof(T2);
  TPM_LAUNCH(c, "pcg_fft_x_fwd", k_pc_xfwd<T2>, xblocks, tx, sx, g, plx, r2c, r, sc,
             spec, npx, skip);
  TPM_LAUNCH(c, "pcg_fft_y", k_fft_y<T2>, g.nz * ((g.nxh + npy - 1) / npy), ty, sy, g,
             ply, spec, npy, -1, skip);
  TPM_LAUNCH(c, "pcg_fft_z_solve", k_fft_z_solve<T2>, g.ny * ((g.nxh + npz - 1) / npz),
             tz, sz, g, plz, spec, c->ax, c->ay, c->az,
             static_cast<const typename Cx<T2>::T *>(c->inv_mwn), npz, skip);
  TPM_LAUNCH(c, "pcg_fft_y", k_fft_y<T2>, g.nz * ((g.nxh + npy - 1) / npy), ty, sy, g,
             ply, spec, npy, +1, skip);
  TPM_LAUNCH(c, "pcg_fft_x_inv", k_pc_xinv<T2>, xblocks, tx, sx, g, plx, r2c, spec, r,
             sc, z, parts, npx, skip);
}

}  // namespace

int fft_precondition(tpm_ctx *c, const double *r, const double *sc, double *z, double *parts,
                     const int *skip) {
  if (c->p.precision == TPM_PREC_MIXED)
    precondition_t<float2>(c, r, sc, z, parts, skip);
  else
    precondition_t<double2>(c, r, sc, z, parts, skip);
  return (int)(((long long)c->g.ny * c->g.nz + c->pen[0] - 1) / c->pen[0]);
}

void precondition_setup() {
  const int smem64 = 2 * kFftSmemPoints * (int)sizeof(double2);
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_pc_xfwd<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_pc_xfwd<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_pc_xinv<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_pc_xinv<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
}

void spectrum_kernels_setup() {
  const int smem64 = 2 * kFftSmemPoints * (int)sizeof(double2);
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_spec_xfwd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_spec_z_energy, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64));
}
}  // namespace tpm

// ===========================================================================
// Allocation-free Poisson solve (tpm_poisson_solve_noalloc, include/tpm.h).
//
// Some callers cannot allocate device memory at all: a plug-in that only
// receives buffers from its host application, or a runtime whose memory pool
// owns the device and forbids side allocations.  This entry point runs the
// same kernels as tpm_poisson_solve, but every byte of scratch it needs
// (spectrum, centre coefficients, partial maxima, twiddle and wave-number
// tables, device scalars) lives in the fixed array below, which each GPU that
// loads the library holds until the process exits.  The caller passes device
// pointers for the inputs and the output only.  The call synchronises its
// stream (the small tables are copied from host staging), so it cannot run
// while that stream is being captured into a CUDA graph; it refuses to.
// ===========================================================================
namespace tpm {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)TPM_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kStaticScratchBytes];

// Host state shared by every calling thread, guarded by g_noalloc_mutex: the
// device address of g_noalloc_scratch per device (looked up once, with that
// device current) and the staging arrays of the small tables (fixed size: no
// host allocation either).  The lock is held from the first write of the
// staging arrays until the stream has finished copying them.
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};
double2 g_tab_host[4 * 2048 + 8];
double g_mwn_host[2048 + 2048 + 2048 + 8];

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

__global__ void k_center_coeff_noalloc(Grid g, const double *__restrict__ Cf, double *__restrict__ cc) {
  const double OneThird = 1. / 3.;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const long long cxp = at(g, wrap_p(i, g.nx), j, k), cyp = at(g, i, wrap_p(j, g.ny), k),
                    czp = at(g, i, j, wrap_p(k, g.nz));
    double m = OneThird * ((Cf[c] + Cf[cxp]) * 0.5 + (Cf[g.n + c] + Cf[g.n + cyp]) * 0.5 +
                           (Cf[2 * g.n + c] + Cf[2 * g.n + czp]) * 0.5);
    cc[c] = -1. / m;
  }
}

// device address of this device's scratch array, resolved on first use
int noalloc_scratch(int dev, unsigned char **out) {
  if (!g_noalloc_ptr[dev]) {
    // the host-side name g_noalloc_scratch is only a stand-in: the kernels
    // need the address cudaGetSymbolAddress gives for the current device
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return TPM_ERR_CUDA;
    int smem64 = 2 * kFftSmemPoints * (int)sizeof(double2);
    if (cudaFuncSetAttribute(k_xfwd_resid<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_y<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_z_solve<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64) != cudaSuccess ||
        cudaFuncSetAttribute(k_xinv_update<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem64) != cudaSuccess)
      return TPM_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
  return TPM_OK;
}

}  // namespace
}  // namespace tpm

extern "C" int tpm_poisson_solve_noalloc(int Nx, int Ny, int Nz, double Lx, double Ly, double Lz,
                                         const double *C3, double *P, const double *RHS,
                                         int max_iterations, double epsilon, void *stream,
                                         int *iterations_out, double *error_out) {
  using namespace tpm;
  auto ok = [](int n) {
    if (n < 1) return false;
    for (int f : {2, 3, 5})
      while (n % f == 0) n /= f;
    return n == 1;
  };
  if (!C3 || !P || !RHS || max_iterations < 0) return TPM_ERR_ARG;
  if (!ok(Nx) || !ok(Ny) || !ok(Nz) || (Nx % 2) || Nx < 4 || Ny < 2 || Nz < 2 ||
      Nx / 2 > 2048 || Ny > 2048 || Nz > 2048 || !(Lx > 0) || !(Ly > 0) || !(Lz > 0))
    return TPM_ERR_ARG;
  Grid g;
  g.nx = Nx; g.ny = Ny; g.nz = Nz; g.nxh = Nx / 2 + 1; g.sxh = g.nxh;
  g.n = (long long)Nx * Ny * Nz;
  g.mx = tpm::udiv_magic((unsigned)Nx); g.my = tpm::udiv_magic((unsigned)Ny);
  g.Lx = Lx; g.Ly = Ly; g.Lz = Lz;
  g.dx = Lx / Nx; g.dy = Ly / Ny; g.dz = Lz / Nz;
  g.inv_dx = 1. / g.dx; g.inv_dy = 1. / g.dy; g.inv_dz = 1. / g.dz;
  g.inv_dx2 = 1. / (g.dx * g.dx); g.inv_dy2 = 1. / (g.dy * g.dy); g.inv_dz2 = 1. / (g.dz * g.dz);
  g.idx = g.inv_dx; g.idy = g.inv_dy; g.idz = g.inv_dz;
  g.xh = Nx * g.dx; g.yh = Ny * g.dy; g.zh = Nz * g.dz;
  const long long nrows = (long long)Ny * Nz;
  const int npx = pens_for(Nx / 2);
  const int xblocks = (int)((nrows + npx - 1) / npx);
  const int ntab = Nx / 2 + Ny + Nz + Nx;
  // scratch layout
  const size_t o_sc = 0;
  const size_t o_spec = o_sc + align256(sizeof(DevScalars));
  const size_t o_cc = o_spec + align256((size_t)g.nxh * Ny * Nz * sizeof(double2));
  const size_t o_err = o_cc + align256((size_t)g.n * sizeof(double));
  const size_t o_tab = o_err + align256((size_t)xblocks * sizeof(double));
  const size_t o_mwn = o_tab + align256((size_t)ntab * sizeof(double2));
  const size_t need = o_mwn + align256((size_t)(g.nxh + Ny + Nz) * sizeof(double));
  if (need > kStaticScratchBytes) return TPM_ERR_ARG;  // grid too large for the fixed scratch

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return TPM_ERR_CUDA;
  if (cap != cudaStreamCaptureStatusNone) return TPM_ERR_STATE;  // it synchronises the stream
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TPM_ERR_CUDA;

  FftPlan fx, fy, fz;
  try {
    factorize(Nx / 2, fx);
    factorize(Ny, fy);
    factorize(Nz, fz);
  } catch (const std::string &) {
    return TPM_ERR_ARG;
  }
  unsigned char *base = nullptr;
  DevScalars *dsc;
  double *cc, *errp, *mwn;
  double2 *spec, *tab;
  const double2 *r2c;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    const int rc = noalloc_scratch(dev, &base);
    if (rc != TPM_OK) return rc;
    dsc = reinterpret_cast<DevScalars *>(base + o_sc);
    spec = reinterpret_cast<double2 *>(base + o_spec);
    cc = reinterpret_cast<double *>(base + o_cc);
    errp = reinterpret_cast<double *>(base + o_err);
    tab = reinterpret_cast<double2 *>(base + o_tab);
    mwn = reinterpret_cast<double *>(base + o_mwn);
    // plans and tables (twiddles exp(-2 pi i m/n); wave numbers as in
    // poisson.cpp:433-447)
    int off = 0;
    auto put_tw = [&](int n) {
      for (int m = 0; m < n; ++m) {
        double a = 2.0 * 3.14159265358979323846 * (double)m / (double)n;
        g_tab_host[off + m] = make_double2(cos(a), -sin(a));
      }
      int at0 = off;
      off += n;
      return at0;
    };
    fx.tw64 = tab + put_tw(Nx / 2);
    fy.tw64 = tab + put_tw(Ny);
    fz.tw64 = tab + put_tw(Nz);
    r2c = tab + put_tw(Nx);
    fx.tw32 = fy.tw32 = fz.tw32 = nullptr;
    auto put_mwn = [](int n, double L, double d, double *t, int count) {
      double TWO_PI(2 * 3.141592653589793);
      double two_pi_over_L = TWO_PI / L;
      double d2 = 2. / (d * d);
      for (int i = 0; i < count; ++i) {
        double kk = ((i < n / 2) ? i : i - n) * two_pi_over_L;
        t[i] = (d2) * (1 - cos(kk * d));
      }
    };
    put_mwn(Nx, Lx, g.dx, g_mwn_host, g.nxh);
    put_mwn(Ny, Ly, g.dy, g_mwn_host + g.nxh, Ny);
    put_mwn(Nz, Lz, g.dz, g_mwn_host + g.nxh + Ny, Nz);
    if (cudaMemcpyAsync(tab, g_tab_host, sizeof(double2) * ntab, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(mwn, g_mwn_host, sizeof(double) * (g.nxh + Ny + Nz), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(dsc, 0, sizeof(DevScalars), st) != cudaSuccess)  // mean_rhs = 0: RHS used as given
      return TPM_ERR_CUDA;
    // the copies read the staging arrays: finish them before another call
    // may rewrite them
    if (cudaStreamSynchronize(st) != cudaSuccess) return TPM_ERR_CUDA;
  }
  const double *ax = mwn, *ay = mwn + g.nxh, *az = mwn + g.nxh + Ny;

  int cb = (int)((g.n + 255) / 256);
  if (cb > kRedBlocks) cb = kRedBlocks;
  k_center_coeff_noalloc<<<cb, 256, 0, st>>>(g, C3, cc);
  k_loop_begin<<<1, 1, 0, st>>>(dsc);  // skip = it = 0, err = 100
  const int *skip = &dsc->skip;
  // poisson.cpp:395-410: while (i < Iteration && error > epsilon).  The device
  // applies the test after every iteration and turns the remaining ones into
  // no-ops once it fails (with epsilon <= 0: when max|dp| is exactly 0); with
  // epsilon > 0 the host also reads max|dp| to stop launching.
  int launched = 0;
  double error = 100;
  while ((launched < max_iterations) && (error > epsilon)) {
    {
      size_t smem = 2 * (size_t)npx * fx.n * sizeof(double2);
      k_xfwd_resid<double2><<<xblocks, kFftThreads, smem, st>>>(g, fx, r2c, P, C3, cc, RHS, dsc, spec, npx);
    }
    {
      int npen = pens_for(fy.n);
      int blocks = Nz * ((g.nxh + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * fy.n * sizeof(double2);
      k_fft_y<double2><<<blocks, kFftThreads, smem, st>>>(g, fy, spec, npen, -1, skip);
    }
    {
      int npen = pens_for(fz.n);
      int blocks = Ny * ((g.nxh + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * fz.n * sizeof(double2);
      k_fft_z_solve<double2><<<blocks, kFftThreads, smem, st>>>(g, fz, spec, ax, ay, az, nullptr, npen,
                                                                 skip);
    }
    {
      int npen = pens_for(fy.n);
      int blocks = Nz * ((g.nxh + npen - 1) / npen);
      size_t smem = 2 * (size_t)npen * fy.n * sizeof(double2);
      k_fft_y<double2><<<blocks, kFftThreads, smem, st>>>(g, fy, spec, npen, +1, skip);
    }
    {
      size_t smem = 2 * (size_t)npx * fx.n * sizeof(double2);
      k_xinv_update<double2><<<xblocks, kFftThreads, smem, st>>>(g, fx, r2c, spec, P, errp, npx,
                                                                 skip, nullptr, nullptr, nullptr,
                                                                 1.0 / (double)((long long)Nx * Ny * Nz),
                                                                 nullptr);
      k_finish_max<<<1, 256, 0, st>>>(errp, xblocks, dsc, epsilon, cudaGraphConditionalHandle{}, 0,
                                      nullptr);
    }
    if (cudaGetLastError() != cudaSuccess) return TPM_ERR_CUDA;
    launched++;
    if (epsilon > 0) {
      if (cudaMemcpyAsync(&error, &dsc->err, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return TPM_ERR_CUDA;
    }
  }
  int it = 0;
  double err = 0;
  if (cudaMemcpyAsync(&it, &dsc->it, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&err, &dsc->err, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return TPM_ERR_CUDA;
  if (iterations_out) *iterations_out = it;
  if (error_out) *error_out = err;
  return TPM_OK;
}
