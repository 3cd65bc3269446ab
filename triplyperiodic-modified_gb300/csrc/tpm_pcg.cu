// Pressure solve by preconditioned conjugate gradients (Solver = 2).
//
// The reference offers HYPRE Krylov solvers besides the FFT-preconditioned
// Richardson loop (poisson.cpp:117-388; Solver 2 is PCG with a two-norm
// relative stopping test ||r||/||b|| < epsilon and at most Iteration
// iterations, poisson.cpp:214-245).  Here the same operator
// div(C grad P) = RHS (7-point, face coefficients C = 1/Rho_face) is solved by
// PCG preconditioned by the Richardson loop's own approximate inverse in
// symmetric form, M^-1 = S (-Lap_h)^-1 S with S = diag(1/sqrt(C_c)) and C_c the
// centre-averaged coefficient (poisson.cpp:393-394), applied with the same
// pencil FFTs.  For strongly heated flows, where the
// density ratio and with it the Richardson contraction factor grow, CG needs
// about the square root of the iterations.  Vectors and reductions are FP64;
// on the mixed path the preconditioner's FFTs are FP32.
//
// Per iteration: p = z + beta p; q = A p (A = -div(C grad .)) with p.q;
// alpha; P += alpha p, r -= alpha q with r.r; z = M^-1 r with r.z; beta and
// the stopping test.  Every reduction is a fixed-order tree over per-block
// partials, so a solve is bit-reproducible.
#include <cmath>

#include "tpm_internal.cuh"
#include "tpm_reduce.cuh"

namespace tpm {
namespace {

constexpr int kThreadsPcg = 256;

// device scalars of the iteration
enum { PC_RHO = 0, PC_PQ, PC_ALPHA, PC_BETA, PC_RR, PC_BB, PC_ERR, PC_COUNT };

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

// div(C grad f) at cell c with the operation order of the Richardson
// residual (poisson.cpp:399-401); kScaled: Cf holds C/d^2 per component.
template <bool kScaled>
__device__ __forceinline__ double lap_c(const Grid &g, const double *__restrict__ f,
                                        const double *__restrict__ Cf, long long c) {
  int i, j, k;
  cell_ijk(g, c, i, j, k);
  const double *Cx = Cf, *Cy = Cf + g.n, *Cz = Cf + 2 * g.n;
  const long long xp = at(g, wrap_p(i, g.nx), j, k), xm = at(g, wrap_m(i, g.nx), j, k);
  const long long yp = at(g, i, wrap_p(j, g.ny), k), ym = at(g, i, wrap_m(j, g.ny), k);
  const long long zp = at(g, i, j, wrap_p(k, g.nz)), zm = at(g, i, j, wrap_m(k, g.nz));
  const double fc = f[c];
  if (kScaled)
    return (Cx[xp] * (f[xp] - fc) - Cx[c] * (fc - f[xm])) +
           (Cy[yp] * (f[yp] - fc) - Cy[c] * (fc - f[ym])) +
           (Cz[zp] * (f[zp] - fc) - Cz[c] * (fc - f[zm]));
  const double gx_hi = (f[xp] - fc) * g.inv_dx * Cx[xp], gx_lo = (fc - f[xm]) * g.inv_dx * Cx[c];
  const double gy_hi = (f[yp] - fc) * g.inv_dy * Cy[yp], gy_lo = (fc - f[ym]) * g.inv_dy * Cy[c];
  const double gz_hi = (f[zp] - fc) * g.inv_dz * Cz[zp], gz_lo = (fc - f[zm]) * g.inv_dz * Cz[c];
  return (gx_hi - gx_lo) * g.inv_dx + (gy_hi - gy_lo) * g.inv_dy + (gz_hi - gz_lo) * g.inv_dz;
}

// r = b - A P = div(C grad P) - (RHS - mean(RHS)); partials of r.r and b.b;
// the preconditioner scale sc = sqrt(-cc) = 1/sqrt(I_F2C(C)) once per solve
template <bool kScaled>
__global__ void k_pcg_residual(Grid g, const double *__restrict__ P, const double *__restrict__ Cf,
                               const double *__restrict__ RHS, const DevScalars *__restrict__ s,
                               const double *__restrict__ cc, double *__restrict__ scale,
                               double *__restrict__ r, double *__restrict__ parts_rr,
                               double *__restrict__ parts_bb) {
  __shared__ double sh[32];
  const double mean = s->mean_rhs;
  double rr = 0, bb = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const double b = RHS[c] - mean;
    const double rc = lap_c<kScaled>(g, P, Cf, c) - b;
    r[c] = rc;
    scale[c] = sqrt(-cc[c]);
    rr += rc * rc;
    bb += b * b;
  }
  double v = block_sum(rr, sh);
  if (threadIdx.x == 0) parts_rr[blockIdx.x] = v;
  v = block_sum(bb, sh);
  if (threadIdx.x == 0) parts_bb[blockIdx.x] = v;
}

__device__ double sum_parts(const double *__restrict__ parts, int n, double *sh) {
  double v = 0;
  for (int b = threadIdx.x; b < n; b += blockDim.x) v += parts[b];
  return block_sum(v, sh);
}

// after the first preconditioning: rho = r.z, b.b, the relative residual,
// and whether the loop runs at all (poisson.cpp:214-245's HYPRE PCG stops on
// ||r||_2 / ||b||_2 < epsilon)
__global__ void k_pcg_init(const double *__restrict__ parts_rz, int n_rz,
                           const double *__restrict__ parts_rr, const double *__restrict__ parts_bb,
                           int n_c, double *__restrict__ sc, DevScalars *__restrict__ s, double eps) {
  __shared__ double sh[32];
  const double rz = sum_parts(parts_rz, n_rz, sh);
  __syncthreads();
  const double rr = sum_parts(parts_rr, n_c, sh);
  __syncthreads();
  const double bb = sum_parts(parts_bb, n_c, sh);
  if (threadIdx.x == 0) {
    sc[PC_RHO] = rz;
    sc[PC_BETA] = 0.0;
    sc[PC_RR] = rr;
    sc[PC_BB] = bb;
    const double rel = bb > 0 ? sqrt(rr) / sqrt(bb) : 0.0;
    sc[PC_ERR] = rel;
    s->err = rel;
    const bool more = bb > 0 && !(eps > 0 && !(rel > eps));
    s->skip = more ? 0 : 1;  // a captured loop then runs one no-op body and stops
  }
}

// p = z + beta p
__global__ void k_pcg_p(long long n, const double *__restrict__ z, double *__restrict__ p,
                        const double *__restrict__ sc, const int *__restrict__ skip) {
  if (*skip) return;
  const double beta = sc[PC_BETA];
  if (beta == 0.0) {  // first iteration: p = z (p holds the previous solve)
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
      p[c] = z[c];
    return;
  }
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x)
    p[c] = z[c] + beta * p[c];
}

// q = A p = -div(C grad p); partials of p.q
template <bool kScaled>
__global__ void k_pcg_matvec(Grid g, const double *__restrict__ p, const double *__restrict__ Cf,
                             double *__restrict__ q, double *__restrict__ parts,
                             const int *__restrict__ skip) {
  if (*skip) return;
  __shared__ double sh[32];
  double acc = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const double qc = -lap_c<kScaled>(g, p, Cf, c);
    q[c] = qc;
    acc += p[c] * qc;
  }
  double v = block_sum(acc, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = v;
}

__global__ void k_pcg_alpha(const double *__restrict__ parts, int n, double *__restrict__ sc,
                            const int *__restrict__ skip) {
  if (*skip) return;
  __shared__ double sh[32];
  const double pq = sum_parts(parts, n, sh);
  if (threadIdx.x == 0) {
    sc[PC_PQ] = pq;
    sc[PC_ALPHA] = pq != 0 ? sc[PC_RHO] / pq : 0.0;
  }
}

// P += alpha p, r -= alpha q; partials of r.r
__global__ void k_pcg_update(long long n, double *__restrict__ P, double *__restrict__ r,
                             const double *__restrict__ p, const double *__restrict__ q,
                             const double *__restrict__ sc, double *__restrict__ parts_rr,
                             const int *__restrict__ skip) {
  if (*skip) return;
  __shared__ double sh[32];
  const double alpha = sc[PC_ALPHA];
  double rr = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    P[c] += alpha * p[c];
    const double rc = r[c] - alpha * q[c];
    r[c] = rc;
    rr += rc * rc;
  }
  double v = block_sum(rr, sh);
  if (threadIdx.x == 0) parts_rr[blockIdx.x] = v;
}

// beta = r.z / rho, the stopping test, the iteration count
__global__ void k_pcg_finish(const double *__restrict__ parts_rz, int n_rz,
                             const double *__restrict__ parts_rr, int n_c, double *__restrict__ sc,
                             DevScalars *__restrict__ s, double eps,
                             cudaGraphConditionalHandle loop, int loop_max) {
  if (s->skip) {  // converged before this body (set-up or previous iteration)
    if (loop_max > 0 && threadIdx.x == 0) cudaGraphSetConditional(loop, 0u);
    return;
  }
  __shared__ double sh[32];
  const double rz = sum_parts(parts_rz, n_rz, sh);
  __syncthreads();
  const double rr = sum_parts(parts_rr, n_c, sh);
  if (threadIdx.x == 0) {
    const double rho = sc[PC_RHO];
    sc[PC_BETA] = rho != 0 ? rz / rho : 0.0;
    sc[PC_RHO] = rz;
    sc[PC_RR] = rr;
    const double rel = sc[PC_BB] > 0 ? sqrt(rr) / sqrt(sc[PC_BB]) : 0.0;
    sc[PC_ERR] = rel;
    s->err = rel;
    s->it += 1;
    s->it_sum += 1;
    const bool more = !(eps > 0 && !(rel > eps));
    if (loop_max > 0)
      cudaGraphSetConditional(loop, (s->it < loop_max && more) ? 1u : 0u);
    else if (!more)
      s->skip = 1;
  }
}

int cblocks(const Grid &g) {
  long long b = (g.n + kThreadsPcg - 1) / kThreadsPcg;
  return (int)(b < kRedBlocks ? b : kRedBlocks);
}

}  // namespace

// Buffers of the solver; called by tpm_create (never inside a graph capture).
void pcg_alloc(tpm_ctx *c) {
  if (c->pcg_r) return;
  const size_t n = (size_t)c->g.n;
  c->pcg_r = dalloc<double>(c, n);
  c->pcg_z = dalloc<double>(c, n);
  c->pcg_p = dalloc<double>(c, n);
  c->pcg_q = dalloc<double>(c, n);
  c->pcg_s = dalloc<double>(c, n);
  c->pcg_sc = dalloc<double>(c, PC_COUNT);
  const size_t np = 4 * (size_t)kRedBlocks + (size_t)c->g.ny * c->g.nz;
  c->pcg_parts = dalloc<double>(c, np);
  for (double *v : {c->pcg_r, c->pcg_z, c->pcg_p, c->pcg_q, c->pcg_s})
    TPM_CUDA_TRY(cudaMemsetAsync(v, 0, sizeof(double) * n, c->stream));
  TPM_CUDA_TRY(cudaMemsetAsync(c->pcg_sc, 0, sizeof(double) * PC_COUNT, c->stream));
  TPM_CUDA_TRY(cudaMemsetAsync(c->pcg_parts, 0, sizeof(double) * np, c->stream));
  precondition_setup();
}

// One PCG iteration (everything after the set-up); `loop` when captured.
static void pcg_iteration(tpm_ctx *c, double eps, const LoopCtl *loop) {
  const Grid &g = c->g;
  const bool scaled = c->p.precision == TPM_PREC_MIXED;
  const double *Cf = scaled ? c->Cs : c->Cface;
  const int nb = cblocks(g);
  const int *skip = &c->dsc->skip;
  double *pq = c->pcg_parts, *prr = pq + kRedBlocks, *prz = prr + 3 * kRedBlocks;
  TPM_LAUNCH(c, "pcg_p", k_pcg_p, nb, kThreadsPcg, 0, g.n, c->pcg_z, c->pcg_p, c->pcg_sc, skip);
  if (scaled)
    TPM_LAUNCH(c, "pcg_matvec", k_pcg_matvec<true>, nb, kThreadsPcg, 0, g, c->pcg_p, Cf, c->pcg_q,
               pq, skip);
  else
    TPM_LAUNCH(c, "pcg_matvec", k_pcg_matvec<false>, nb, kThreadsPcg, 0, g, c->pcg_p, Cf, c->pcg_q,
               pq, skip);
  TPM_LAUNCH(c, "pcg_alpha", k_pcg_alpha, 1, kThreadsPcg, 0, pq, nb, c->pcg_sc, skip);
  TPM_LAUNCH(c, "pcg_update", k_pcg_update, nb, kThreadsPcg, 0, g.n, c->P, c->pcg_r, c->pcg_p,
             c->pcg_q, c->pcg_sc, prr, skip);
  const int nrz = fft_precondition(c, c->pcg_r, c->pcg_s, c->pcg_z, prz, skip);
  TPM_LAUNCH(c, "pcg_finish", k_pcg_finish, 1, kThreadsPcg, 0, prz, nrz, prr, nb, c->pcg_sc,
             c->dsc, eps, loop ? loop->handle : cudaGraphConditionalHandle{}, loop ? loop->max_it : 0);
}

// Set-up of a solve: r = b - A P, z = M^-1 r, rho = r.z, the initial test.
void pcg_setup(tpm_ctx *c, double eps, const LoopCtl *loop) {
  if (!c->pcg_r) throw std::string("PCG buffers not allocated (Solver != 2 at create)");
  const Grid &g = c->g;
  const bool scaled = c->p.precision == TPM_PREC_MIXED;
  const double *Cf = scaled ? c->Cs : c->Cface;
  const int nb = cblocks(g);
  double *prr = c->pcg_parts + kRedBlocks, *pbb = c->pcg_parts,
         *prz = c->pcg_parts + 3 * kRedBlocks;
  if (scaled)
    TPM_LAUNCH(c, "pcg_residual", k_pcg_residual<true>, nb, kThreadsPcg, 0, g, c->P, Cf, c->RHS,
               c->dsc, c->cc, c->pcg_s, c->pcg_r, prr, pbb);
  else
    TPM_LAUNCH(c, "pcg_residual", k_pcg_residual<false>, nb, kThreadsPcg, 0, g, c->P, Cf, c->RHS,
               c->dsc, c->cc, c->pcg_s, c->pcg_r, prr, pbb);
  const int nrz = fft_precondition(c, c->pcg_r, c->pcg_s, c->pcg_z, prz, nullptr);
  TPM_LAUNCH(c, "pcg_init", k_pcg_init, 1, kThreadsPcg, 0, prz, nrz, prr, pbb, nb, c->pcg_sc,
             c->dsc, eps);
  (void)loop;
}

void pcg_step(tpm_ctx *c, double eps, const LoopCtl *loop) { pcg_iteration(c, eps, loop); }

}  // namespace tpm
