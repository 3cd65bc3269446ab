// Discrete adjoint of the RK4 step (tpm_adjoint_run).
//
// Regime: the adjoint workload's physics - two-way momentum coupling, linear
// forcing, no particle heating (I0 = 0), no cooling, no gravity, uniform
// density.  There the density stays uniform to the Poisson tolerance, so a
// step is the reference's incompressible update (simulation.cpp:60-91,
// grid.cpp:776-900, particle.cpp:314-520) and its adjoint treats Rho_face and
// the Poisson coefficient as the constants of the forward run.  The adjoint is
// the exact transpose of that discrete map, stage by stage:
//   * projection: RU_new'' = (I - Q) RU_new', RU_np1'' = RU_np1' - (b/a) Q RU_new',
//     Q = G Lap^-1 D symmetric, so lam_new' = lam_new - Q (lam_new + (b/a) lam_np1)
//     with Lap^-1 by the pencil FFTs of the pressure solve;
//   * right-hand side (grid.cpp:776-814): (mu/3) G D and mu Lap are symmetric;
//     the convective term conv_d = sum_a D_a(I_a U_d * I_d RU_a) transposes to
//     gathers of D_a^T, I_a^T (D^T = -G, I_C2F^T = I_F2C);
//   * particles: velocity interpolation and force deposition are each other's
//     transposes (particle.cpp:340-360, 494-520); their position derivatives
//     are the slopes of the linear weights;
//   * RK4 bookkeeping, including the step-boundary detail that the next step's
//     first stage reads RU_int = RU_np1 before make_mean_U0 (grid.cpp:893,
//     simulation.cpp:80).
// Forward states are recomputed per segment from checkpoints taken every K
// steps, so the trajectory memory is 4K stage records.  The objective is
// J = w_tke * 0.5 * sum_d mean(RU_d^2 / Rho_face_d) + w_cvar * var(C) at the
// final step boundary, C the cloud-in-cell concentration of the final particle
// positions (particle.cpp:522-555 weights).  Gradients: dJ/dRU(0) projected on
// discretely divergence-free fields, dJ/dA, and dJ/dtau_p for a uniform shift
// of the Stokes time.  Scatter-adds use FP64 atomics, so gradients are
// reproducible to rounding, not bit for bit.
#include <cmath>
#include <vector>

#include "tpm_internal.cuh"
#include "tpm_reduce.cuh"

namespace tpm {
namespace {

constexpr int kAT = 256;
constexpr double kPreA[4] = {0.5, 0.5, 1., 1. / 6.};          // grid.cpp:18-21
constexpr double kPostA[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

struct Ix {
  int i, j, k;
};

__device__ __forceinline__ Ix ix_of(const Grid &g, long long c) {
  Ix r;
  cell_ijk(g, c, r.i, r.j, r.k);
  return r;
}

// index of cell q shifted by s in direction d (periodic)
__device__ __forceinline__ long long sh(const Grid &g, Ix q, int d, int s) {
  if (d == 0) return at(g, wrap_any(q.i + s, g.nx), q.j, q.k);
  if (d == 1) return at(g, q.i, wrap_any(q.j + s, g.ny), q.k);
  return at(g, q.i, q.j, wrap_any(q.k + s, g.nz));
}

__device__ __forceinline__ Ix shq(const Grid &g, Ix q, int d, int s) {
  if (d == 0) q.i = wrap_any(q.i + s, g.nx);
  else if (d == 1) q.j = wrap_any(q.j + s, g.ny);
  else q.k = wrap_any(q.k + s, g.nz);
  return q;
}

__device__ __forceinline__ double inv_h(const Grid &g, int d) {
  return d == 0 ? g.inv_dx : d == 1 ? g.inv_dy : g.inv_dz;
}

// Rho_face_d at cell q: I_C2F(Rho) = (Rho[q] + Rho[q - e_d]) * 0.5
__device__ __forceinline__ double rface(const Grid &g, const double *Rho, Ix q, int d) {
  return (Rho[at(g, q.i, q.j, q.k)] + Rho[sh(g, q, d, -1)]) * 0.5;
}

// D(lam) at cell q: sum_a (lam_a[q + e_a] - lam_a[q]) / h_a
__device__ __forceinline__ double divl(const Grid &g, const double *L, Ix q) {
  const long long c = at(g, q.i, q.j, q.k);
  double s = 0;
  for (int a = 0; a < 3; ++a) s += (L[a * g.n + sh(g, q, a, 1)] - L[a * g.n + c]) * inv_h(g, a);
  return s;
}

// ------------------------------------------------------------- objective
// lam_RU = w * RU / Rho_face / n and partial sums of 0.5 RU^2 / Rho_face
__global__ void k_obj_tke(Grid g, const double *__restrict__ RU, const double *__restrict__ Rho,
                          double w, double *__restrict__ lam, double *__restrict__ parts) {
  __shared__ double sh_[32];
  double acc = 0;
  const double inv_n = 1.0 / (double)g.n;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const Ix q = ix_of(g, c);
    for (int d = 0; d < 3; ++d) {
      const double rf = rface(g, Rho, q, d), ru = RU[d * g.n + c];
      lam[d * g.n + c] = w * ru / rf * inv_n;
      acc += 0.5 * ru * ru / rf;
    }
  }
  double v = block_sum(acc, sh_);
  if (threadIdx.x == 0) parts[blockIdx.x] = v;
}

struct Cic {
  long long c[8];
  double l[3];
};

// part2gas_concentration's round indexing (particle.cpp:522-555)
__device__ __forceinline__ Cic cic(const Grid &g, double x, double y, double z) {
  Cic r;
  const int ii = (int)round(x * g.idx), jj = (int)round(y * g.idy), kk = (int)round(z * g.idz);
  r.l[0] = x * g.idx - ii + 0.5;
  r.l[1] = y * g.idy - jj + 0.5;
  r.l[2] = z * g.idz - kk + 0.5;
  const int i1 = wrap_any(ii, g.nx), i0 = wrap_any(ii - 1, g.nx);
  const int j1 = wrap_any(jj, g.ny), j0 = wrap_any(jj - 1, g.ny);
  const int k1 = wrap_any(kk, g.nz), k0 = wrap_any(kk - 1, g.nz);
  int m = 0;
  for (int a = 1; a >= 0; --a)
    for (int b = 1; b >= 0; --b)
      for (int cc = 1; cc >= 0; --cc) r.c[m++] = at(g, a ? i1 : i0, b ? j1 : j0, cc ? k1 : k0);
  return r;
}

__global__ void k_conc(Grid g, int64_t np, const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, double *__restrict__ C) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const Cic w = cic(g, x[p], y[p], z[p]);
    int m = 0;
    for (int a = 1; a >= 0; --a)
      for (int b = 1; b >= 0; --b)
        for (int cc = 1; cc >= 0; --cc) {
          const double wx = a ? w.l[0] : 1 - w.l[0], wy = b ? w.l[1] : 1 - w.l[1],
                       wz = cc ? w.l[2] : 1 - w.l[2];
          atomicAdd(&C[w.c[m++]], wx * wy * wz);
        }
  }
}

__global__ void k_sum2(long long n, const double *__restrict__ C, double *__restrict__ parts) {
  __shared__ double sh_[32];
  double s = 0, s2 = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    s += C[c];
    s2 += C[c] * C[c];
  }
  double v = block_sum(s, sh_);
  if (threadIdx.x == 0) parts[blockIdx.x] = v;
  v = block_sum(s2, sh_);
  if (threadIdx.x == 0) parts[kRedBlocks + blockIdx.x] = v;
}

// lam_X = w dvar/dx: var = mean(C^2) - mean(C)^2, dvar/dC = 2 (C - mean)/n
__global__ void k_obj_cvar(Grid g, int64_t np, const double *__restrict__ x,
                           const double *__restrict__ y, const double *__restrict__ z,
                           const double *__restrict__ C, double meanC, double w,
                           double *__restrict__ lx, double *__restrict__ ly, double *__restrict__ lz) {
  const double idn[3] = {g.idx, g.idy, g.idz};
  const double inv_n = 1.0 / (double)g.n;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const Cic q = cic(g, x[p], y[p], z[p]);
    double gx = 0, gy = 0, gz = 0;
    int m = 0;
    for (int a = 1; a >= 0; --a)
      for (int b = 1; b >= 0; --b)
        for (int cc = 1; cc >= 0; --cc) {
          const double dC = w * (2.0 * C[q.c[m++]] * inv_n - 2.0 * meanC * inv_n);
          const double wx = a ? q.l[0] : 1 - q.l[0], wy = b ? q.l[1] : 1 - q.l[1],
                       wz = cc ? q.l[2] : 1 - q.l[2];
          gx += dC * (a ? 1 : -1) * idn[0] * wy * wz;
          gy += dC * wx * (b ? 1 : -1) * idn[1] * wz;
          gz += dC * wx * wy * (cc ? 1 : -1) * idn[2];
        }
    lx[p] = gx;
    ly[p] = gy;
    lz[p] = gz;
  }
}

// ---------------------------------------------------------- bookkeeping
__global__ void k_comp_sums(Grid g, const double *__restrict__ L, double *__restrict__ parts) {
  __shared__ double sh_[32];
  for (int d = 0; d < 3; ++d) {
    double s = 0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
         c += (long long)gridDim.x * blockDim.x)
      s += L[d * g.n + c];
    double v = block_sum(s, sh_);
    if (threadIdx.x == 0) parts[d * kRedBlocks + blockIdx.x] = v;
    __syncthreads();
  }
}

__global__ void k_finish_sums(const double *__restrict__ parts, int nparts, int nsets,
                              double scale, double *__restrict__ out) {
  __shared__ double sh_[32];
  for (int d = 0; d < nsets; ++d) {
    double v = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += parts[d * kRedBlocks + b];
    double s = block_sum(v, sh_);
    if (threadIdx.x == 0) out[d] = s * scale;
    __syncthreads();
  }
}

// end of step (make_mean_U0 and TimeAdvance): lam_np1 = M(lam_RU) + lam_RUint0
__global__ void k_end_gas(long long n3, long long n, const double *__restrict__ lam_RU,
                          const double *__restrict__ means, const double *__restrict__ lam_int0,
                          double *__restrict__ lam_np1) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n3;
       c += (long long)gridDim.x * blockDim.x)
    lam_np1[c] = lam_RU[c] - means[c / n] + lam_int0[c];
}

// y = a + b (elementwise)
__global__ void k_add(long long m, const double *__restrict__ a, const double *__restrict__ b,
                      double *__restrict__ y) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < m;
       c += (long long)gridDim.x * blockDim.x)
    y[c] = a[c] + b[c];
}

// ----------------------------------------------------------- projection
// f = D(lam_new + r lam_np1)
__global__ void k_div_comb(Grid g, const double *__restrict__ A, const double *__restrict__ B,
                           double r, double *__restrict__ f) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const Ix q = ix_of(g, c);
    double s = 0;
    for (int a = 0; a < 3; ++a) {
      const long long cp = sh(g, q, a, 1);
      const double hi = A[a * g.n + cp] + (B ? r * B[a * g.n + cp] : 0.0);
      const double lo = A[a * g.n + c] + (B ? r * B[a * g.n + c] : 0.0);
      s += (hi - lo) * inv_h(g, a);
    }
    f[c] = s;
  }
}

// out = lam - G phi with phi = Lap^-1 f = -z, z = (-Lap)^-1 f:  out = lam + G z
__global__ void k_sub_grad(Grid g, const double *__restrict__ lam, const double *__restrict__ z,
                           double *__restrict__ out) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const Ix q = ix_of(g, c);
    for (int d = 0; d < 3; ++d)
      out[d * g.n + c] = lam[d * g.n + c] + (z[c] - z[sh(g, q, d, -1)]) * inv_h(g, d);
  }
}

// stage bookkeeping of the gas (s < 3): lam_RHS = b lam_np1 + a lam_newp,
// lam_RUb += lam_newp;  s == 3: lam_RHS = b lam_np1
__global__ void k_stage_gas(long long n3, const double *__restrict__ lam_np1,
                            const double *__restrict__ lam_newp, double a, double b, int last,
                            double *__restrict__ lam_RHS, double *__restrict__ lam_RUb) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n3;
       c += (long long)gridDim.x * blockDim.x) {
    if (last) {
      lam_RHS[c] = b * lam_np1[c];
    } else {
      lam_RHS[c] = b * lam_np1[c] + a * lam_newp[c];
      lam_RUb[c] += lam_newp[c];
    }
  }
}

// --------------------------------------------------------------- particles
struct PAdj {
  const double *X[3], *V[3];   // int set of the stage
  double *lXnew[3], *lVnew[3]; // in: adjoint of x_new / u_new; out: of x_int / u_int
  const double *lXnp1[3], *lVnp1[3];
  double *lXb[3], *lVb[3];
  const double *tau;
  double iTp, tau0, a, b, mpV;
  int last, twc;
};

// One stage of the particle adjoint (update_position, update_velocity,
// gas2part_velocity, part2gas_velocity); scatters lam_ug into lamU and adds
// to dJ/dtau.
__global__ void k_adj_particles(Grid g, int64_t np, PAdj s, const double *__restrict__ RU,
                                const double *__restrict__ Rho, const double *__restrict__ lam_RHS,
                                double *__restrict__ lamU, double *__restrict__ gtau) {
  __shared__ double sh_[32];
  const double idn[3] = {g.idx, g.idy, g.idz};
  double acc_tau = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int t[3];
    double xl[3];
    for (int d = 0; d < 3; ++d) {
      const double xs = s.X[d][p] * idn[d];
      t[d] = (int)xs;
      xl[d] = xs - (int)xs;
    }
    Ix lo;
    lo.i = wrap_any(t[0], g.nx);
    lo.j = wrap_any(t[1], g.ny);
    lo.k = wrap_any(t[2], g.nz);
    const long long clo = at(g, lo.i, lo.j, lo.k);
    const double it = s.tau ? 1.0 / s.tau[p] : s.iTp;
    const double tp = s.tau ? s.tau[p] : s.tau0;
    for (int d = 0; d < 3; ++d) {
      const long long chi = sh(g, lo, d, 1);
      const Ix qhi = shq(g, lo, d, 1);
      const double Uhi = RU[d * g.n + chi] / rface(g, Rho, qhi, d);
      const double Ulo = RU[d * g.n + clo] / rface(g, Rho, lo, d);
      const double ug = xl[d] * Uhi + (1 - xl[d]) * Ulo;
      const double V = s.V[d][p];
      const double RHSu = (ug - V) * it;
      // RK bookkeeping (update_position uses u_int; update_velocity RHSu)
      double lVint, lRHSu;
      const double lXnew = s.lXnew[d][p], lVnew = s.lVnew[d][p];
      if (s.last) {
        lVint = s.b * s.lXnp1[d][p];
        lRHSu = s.b * s.lVnp1[d][p];
      } else {
        s.lXb[d][p] += lXnew;
        s.lVb[d][p] += lVnew;
        lVint = s.a * lXnew + s.b * s.lXnp1[d][p];
        lRHSu = s.a * lVnew + s.b * s.lVnp1[d][p];
      }
      double lXint = 0;
      if (s.twc) {  // F_p = deposit(RHSu at x_int), RHS += -(mp/Vcell) F_p
        const double Fhi = -s.mpV * lam_RHS[d * g.n + chi], Flo = -s.mpV * lam_RHS[d * g.n + clo];
        lRHSu += xl[d] * Fhi + (1 - xl[d]) * Flo;
        lXint += RHSu * idn[d] * (Fhi - Flo);
      }
      const double lug = it * lRHSu;
      lVint -= it * lRHSu;
      acc_tau += lRHSu * (-(ug - V) / (tp * tp));
      atomicAdd(&lamU[d * g.n + chi], xl[d] * lug);
      atomicAdd(&lamU[d * g.n + clo], (1 - xl[d]) * lug);
      lXint += lug * idn[d] * (Uhi - Ulo);
      s.lXnew[d][p] = lXint;
      s.lVnew[d][p] = lVint;
    }
  }
  double v = block_sum(acc_tau, sh_);
  if (threadIdx.x == 0) atomicAdd(gtau, v);
}

// ------------------------------------------------------------------ gas RHS
// lam_RUint = (lamU_visc + lamU_conv + lamU_part) / Rho_face + lamRU_conv + A lam;
// partial sums of <lam, RU_int> for dJ/dA
__global__ void k_adj_rhs(Grid g, const double *__restrict__ lam, const double *__restrict__ RU,
                          const double *__restrict__ Rho, const double *__restrict__ lamUp,
                          double mu, double A, double *__restrict__ out,
                          double *__restrict__ parts) {
  __shared__ double sh_[32];
  double accA = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    const Ix q = ix_of(g, c);
    double lamU[3], lamR[3] = {0, 0, 0};
    // viscous: (mu/3) G D lam + mu Lap lam_d
    const double dl0 = divl(g, lam, q);
    for (int d = 0; d < 3; ++d) {
      const Ix qm = shq(g, q, d, -1);
      const double gd = (dl0 - divl(g, lam, qm)) * inv_h(g, d);
      const double *L = lam + d * g.n;
      const double lc = L[c];
      double lap = 0;
      for (int a = 0; a < 3; ++a)
        lap += (L[sh(g, q, a, 1)] - 2 * lc + L[sh(g, q, a, -1)]) * (inv_h(g, a) * inv_h(g, a));
      lamU[d] = (mu / 3.0) * gd + mu * lap;
    }
    // convective: m_{d,a}[r] = (lam_d[r] - lam_d[r - e_a]) / h_a
    //   lamU_d[c] += sum_a 0.5 (m_{d,a}[c] I_d(RU_a)[c] + m_{d,a}[c+e_a] I_d(RU_a)[c+e_a])
    //   lamRU_a[c] += sum_d 0.5 (m_{d,a}[c] I_a(U_d)[c] + m_{d,a}[c+e_d] I_a(U_d)[c+e_d])
    for (int d = 0; d < 3; ++d) {
      const double *L = lam + d * g.n;
      for (int a = 0; a < 3; ++a) {
        const double *Ra = RU + a * g.n;
        const double ia = inv_h(g, a);
        // at c
        const double m_c = (L[c] - L[sh(g, q, a, -1)]) * ia;
        const Ix qa = shq(g, q, a, 1);
        const long long ca = at(g, qa.i, qa.j, qa.k);
        const double m_ca = (L[ca] - L[c]) * ia;
        const double IdRa_c = (Ra[c] + Ra[sh(g, q, d, -1)]) * 0.5;
        const double IdRa_ca = (Ra[ca] + Ra[sh(g, qa, d, -1)]) * 0.5;
        lamU[d] += 0.5 * (m_c * IdRa_c + m_ca * IdRa_ca);
        // lamRU_a: needs m_{d,a} at c and c + e_d, I_a(U_d) there
        const Ix qd = shq(g, q, d, 1);
        const long long cd = at(g, qd.i, qd.j, qd.k);
        const double m_cd = (L[cd] - L[sh(g, qd, a, -1)]) * ia;
        const double *Rd = RU + d * g.n;
        const double Ud_c = Rd[c] / rface(g, Rho, q, d);
        const Ix qam = shq(g, q, a, -1);
        const long long cam = at(g, qam.i, qam.j, qam.k);
        const double Ud_cam = Rd[cam] / rface(g, Rho, qam, d);
        const Ix qdam = shq(g, qd, a, -1);
        const long long cdam = at(g, qdam.i, qdam.j, qdam.k);
        const double Ud_cd = Rd[cd] / rface(g, Rho, qd, d);
        const double Ud_cdam = Rd[cdam] / rface(g, Rho, qdam, d);
        const double IaUd_c = (Ud_c + Ud_cam) * 0.5;
        const double IaUd_cd = (Ud_cd + Ud_cdam) * 0.5;
        lamR[a] += 0.5 * (m_c * IaUd_c + m_cd * IaUd_cd);
      }
    }
    for (int d = 0; d < 3; ++d) {
      const double ld = lam[d * g.n + c];
      const double rf = rface(g, Rho, q, d);
      out[d * g.n + c] = (lamU[d] + lamUp[d * g.n + c]) / rf + lamR[d] + A * ld;
      accA += ld * RU[d * g.n + c];
    }
  }
  double v = block_sum(accA, sh_);
  if (threadIdx.x == 0) parts[blockIdx.x] = v;
}

int blocks_for(long long m) {
  long long b = (m + kAT - 1) / kAT;
  return (int)(b < kRedBlocks ? b : kRedBlocks);
}

// ------------------------------------------------------------ host side
struct Checkpoint {
  double *RU, *RU_int, *Rho, *P, *Q, *rhs_t, *pq[7];
  DevScalars ds;
  double T_cur;
  int64_t step;
};

struct Adj {
  tpm_ctx *c;
  long long n, n3;
  int64_t np;
  // trajectory: per stage RU_int (3n), Rho_int (n), X (3np), V (3np)
  std::vector<double *> tr_RU, tr_Rho, tr_P;
  // adjoint state
  double *lRU, *lRUint0, *lnp1, *lnew, *lnewp, *lRUb, *lRHS, *lUp;
  double *f, *z, *ones, *parts, *red;
  double *lX[3], *lV[3], *lXint0[3], *lVint0[3], *lXnp1[3], *lVnp1[3], *lXnew[3], *lVnew[3],
      *lXb[3], *lVb[3];
  double *gscal;  // [0] dJ/dtau
  std::vector<Checkpoint> cps;
  std::vector<void *> mem;  // freed when the call returns (or throws)
  ~Adj() {
    if (c && c->stream) cudaStreamSynchronize(c->stream);
    for (void *p : mem) cudaFree(p);
  }
  double *alloc(size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(double) * (count ? count : 1)) != cudaSuccess) {
      cudaGetLastError();
      throw std::make_pair(TPM_ERR_NOMEM, std::string("adjoint scratch allocation failed"));
    }
    mem.push_back(p);
    return static_cast<double *>(p);
  }
};

// Lap^-1 projection transpose: out = lam_new - G Lap^-1 D (lam_new + r lam_np1)
void proj_T(Adj &A, const double *lam_new, const double *lam_np1, double r, double *out) {
  tpm_ctx *c = A.c;
  const Grid &g = c->g;
  TPM_LAUNCH(c, "adj_div", k_div_comb, blocks_for(g.n), kAT, 0, g, lam_new, lam_np1, r, A.f);
  fft_precondition(c, A.f, A.ones, A.z, A.parts, nullptr);
  TPM_LAUNCH(c, "adj_grad", k_sub_grad, blocks_for(g.n), kAT, 0, g, lam_new, A.z, out);
}

void save_cp(Adj &A, Checkpoint &k) {
  tpm_ctx *c = A.c;
  auto cp = [&](double *dst, const double *src, size_t m) {
    TPM_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * m, cudaMemcpyDeviceToDevice, c->stream));
  };
  cp(k.RU, c->RU, A.n3);
  cp(k.RU_int, c->RU_int, A.n3);
  cp(k.Rho, c->Rho, A.n);
  cp(k.P, c->P, A.n);
  cp(k.Q, c->Q, A.n);
  if (A.np) {
    cp(k.rhs_t, c->rhs_t, A.np);
    for (int q = 0; q < 7; ++q) cp(k.pq[q], c->pq[0][q], A.np);
  }
  TPM_CUDA_TRY(cudaMemcpyAsync(&k.ds, c->dsc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  k.T_cur = c->T_cur;
  k.step = c->num_timestep;
}

void load_cp(Adj &A, const Checkpoint &k) {
  tpm_ctx *c = A.c;
  auto cp = [&](double *dst, const double *src, size_t m) {
    TPM_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * m, cudaMemcpyDeviceToDevice, c->stream));
  };
  cp(c->RU, k.RU, A.n3);
  cp(c->RU_int, k.RU_int, A.n3);
  cp(c->Rho, k.Rho, A.n);
  cp(c->P, k.P, A.n);
  cp(c->Q, k.Q, A.n);
  if (A.np) {
    cp(c->rhs_t, k.rhs_t, A.np);
    for (int q = 0; q < 7; ++q) cp(c->pq[0][q], k.pq[q], A.np);
  }
  TPM_CUDA_TRY(cudaMemcpyAsync(c->dsc, &k.ds, sizeof(DevScalars), cudaMemcpyHostToDevice, c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->T_cur = k.T_cur;
  c->num_timestep = k.step;
  const bool stepped = c->stepped;
  resume_device(c);
  c->stepped = stepped;
}

// one forward step, recording the four stage inputs into slot `rec`
void record_step(Adj &A, int rec, std::vector<double> &A_of_step) {
  tpm_ctx *c = A.c;
  step_param_update(c);
  A_of_step.push_back(c->A);
  for (int s = 0; s < 4; ++s) {
    const int slot = rec * 4 + s;
    TPM_CUDA_TRY(cudaMemcpyAsync(A.tr_RU[slot], c->RU_int, sizeof(double) * A.n3,
                                 cudaMemcpyDeviceToDevice, c->stream));
    TPM_CUDA_TRY(cudaMemcpyAsync(A.tr_Rho[slot], c->Rho_int, sizeof(double) * A.n,
                                 cudaMemcpyDeviceToDevice, c->stream));
    for (int q = 0; q < 6 && A.np; ++q)
      TPM_CUDA_TRY(cudaMemcpyAsync(A.tr_P[slot] + q * A.np, c->pq[1][q], sizeof(double) * A.np,
                                   cudaMemcpyDeviceToDevice, c->stream));
    step_substep(c, s);
  }
  step_end(c);
}

// backward through one recorded step; appends each stage's <lam_RHS, RU_int>
// (its part of dJ/dA) to gA
void backward_step(Adj &A, int rec, double Astep, std::vector<double> &gA) {
  tpm_ctx *c = A.c;
  const Grid &g = c->g;
  const double dt = c->p.dt;
  const int nbc = blocks_for(g.n), nb3 = blocks_for(A.n3), nbp = blocks_for(A.np > 0 ? A.np : 1);
  // end of step: lam_np1 = M(lam_RU) + lam_RUint0; particles np1 = base + int0
  TPM_LAUNCH(c, "adj_means", k_comp_sums, nbc, kAT, 0, g, A.lRU, A.red);
  TPM_LAUNCH(c, "adj_finish", k_finish_sums, 1, kAT, 0, A.red, nbc, 3, 1.0 / (double)g.n,
             A.red + 3 * kRedBlocks);
  TPM_LAUNCH(c, "adj_end", k_end_gas, nb3, kAT, 0, A.n3, g.n, A.lRU, A.red + 3 * kRedBlocks,
             A.lRUint0, A.lnp1);
  for (int d = 0; d < 3 && A.np; ++d) {
    TPM_LAUNCH(c, "adj_add", k_add, nbp, kAT, 0, A.np, A.lX[d], A.lXint0[d], A.lXnp1[d]);
    TPM_LAUNCH(c, "adj_add", k_add, nbp, kAT, 0, A.np, A.lV[d], A.lVint0[d], A.lVnp1[d]);
    TPM_CUDA_TRY(cudaMemsetAsync(A.lXnew[d], 0, sizeof(double) * A.np, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(A.lVnew[d], 0, sizeof(double) * A.np, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(A.lXb[d], 0, sizeof(double) * A.np, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(A.lVb[d], 0, sizeof(double) * A.np, c->stream));
  }
  TPM_CUDA_TRY(cudaMemsetAsync(A.lnew, 0, sizeof(double) * A.n3, c->stream));
  TPM_CUDA_TRY(cudaMemsetAsync(A.lRUb, 0, sizeof(double) * A.n3, c->stream));
  for (int s = 3; s >= 0; --s) {
    const int slot = rec * 4 + s;
    const double a = dt * kPreA[s], b = dt * kPostA[s];
    if (s == 3) {
      proj_T(A, A.lnp1, nullptr, 0.0, A.lnewp);  // RU_new = RU_np1 at the last stage
      std::swap(A.lnp1, A.lnewp);
    } else {
      proj_T(A, A.lnew, A.lnp1, b / a, A.lnewp);
    }
    TPM_LAUNCH(c, "adj_stage", k_stage_gas, nb3, kAT, 0, A.n3, A.lnp1, A.lnewp, a, b, s == 3,
               A.lRHS, A.lRUb);
    TPM_CUDA_TRY(cudaMemsetAsync(A.lUp, 0, sizeof(double) * A.n3, c->stream));
    if (A.np) {
      PAdj pa;
      for (int d = 0; d < 3; ++d) {
        pa.X[d] = A.tr_P[slot] + d * A.np;
        pa.V[d] = A.tr_P[slot] + (3 + d) * A.np;
        pa.lXnew[d] = A.lXnew[d];
        pa.lVnew[d] = A.lVnew[d];
        pa.lXnp1[d] = A.lXnp1[d];
        pa.lVnp1[d] = A.lVnp1[d];
        pa.lXb[d] = A.lXb[d];
        pa.lVb[d] = A.lVb[d];
      }
      pa.tau = c->tau;
      pa.iTp = c->Tp != 0 ? 1.0 / c->Tp : 0.0;
      pa.tau0 = c->Tp;
      pa.a = a;
      pa.b = b;
      pa.mpV = c->mp / c->Vcell;
      pa.last = s == 3;
      pa.twc = c->p.TWC;
      TPM_LAUNCH(c, "adj_particles", k_adj_particles, nbp, kAT, 0, g, A.np, pa, A.tr_RU[slot],
                 A.tr_Rho[slot], A.lRHS, A.lUp, A.gscal);
    }
    TPM_LAUNCH(c, "adj_rhs", k_adj_rhs, nbc, kAT, 0, g, A.lRHS, A.tr_RU[slot], A.tr_Rho[slot],
               A.lUp, c->p.Mu0, Astep, A.lnew, A.red);
    TPM_LAUNCH(c, "adj_finish", k_finish_sums, 1, kAT, 0, A.red, nbc, 1, 1.0,
               A.red + 3 * kRedBlocks);
    double ga = 0;
    TPM_CUDA_TRY(cudaMemcpyAsync(&ga, A.red + 3 * kRedBlocks, sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    gA.push_back(ga);
  }
  // stage 0's int inputs are this step's RU_int0 / particle int0; its np1
  // inputs are the base state
  std::swap(A.lRUint0, A.lnew);
  TPM_LAUNCH(c, "adj_add", k_add, nb3, kAT, 0, A.n3, A.lRUb, A.lnp1, A.lRU);
  for (int d = 0; d < 3 && A.np; ++d) {
    std::swap(A.lXint0[d], A.lXnew[d]);
    std::swap(A.lVint0[d], A.lVnew[d]);
    TPM_LAUNCH(c, "adj_add", k_add, nbp, kAT, 0, A.np, A.lXb[d], A.lXnp1[d], A.lX[d]);
    TPM_LAUNCH(c, "adj_add", k_add, nbp, kAT, 0, A.np, A.lVb[d], A.lVnp1[d], A.lV[d]);
  }
}

}  // namespace
}  // namespace tpm

using namespace tpm;

extern "C" int tpm_adjoint_run(tpm_ctx *c, int nsteps, int checkpoint_every, double w_tke,
                               double w_cvar, double *J_out, double *dJ_dRU0, double *dJ_dA,
                               double *dJ_dtau) {
  return guarded(c, [&]() -> int {
    if (!c->initialized || c->stepped || !c->np1_is_base)
      return fail(c, TPM_ERR_STATE, "the adjoint starts right after tpm_initialize / tpm_resume");
    if (c->p.precision != TPM_PREC_FP64)
      return fail(c, TPM_ERR_UNSUPPORTED, "the adjoint runs on the FP64 path");
    if (c->p.I01 != 0 || c->p.I02 != 0 || c->p.cooling || c->p.solve_for_scalar ||
        c->p.gx1 != 0 || c->p.gy1 != 0 || c->p.gz1 != 0 || c->p.gx2 != 0 || c->p.gy2 != 0 ||
        c->p.gz2 != 0)
      return fail(c, TPM_ERR_UNSUPPORTED,
                  "the adjoint covers the unheated, uncooled, gravity-free uniform-density regime");
    if (nsteps < 1 || checkpoint_every < 1) return fail(c, TPM_ERR_ARG, "nsteps, checkpoint_every >= 1");
    const Grid &g = c->g;
    Adj A;
    A.c = c;
    A.lRU = nullptr;
    A.n = g.n;
    A.n3 = 3 * g.n;
    A.np = c->np;
    const int K = checkpoint_every < nsteps ? checkpoint_every : nsteps;
    // buffers (allocated per call; freed with the context)
    for (int i = 0; i < 4 * K; ++i) {
      A.tr_RU.push_back(A.alloc(A.n3));
      A.tr_Rho.push_back(A.alloc(A.n));
      A.tr_P.push_back(A.alloc(6 * (size_t)(A.np ? A.np : 1)));
    }
    for (double **p : {&A.lRU, &A.lRUint0, &A.lnp1, &A.lnew, &A.lnewp, &A.lRUb, &A.lRHS, &A.lUp})
      *p = A.alloc(A.n3);
    A.f = A.alloc(A.n);
    A.z = A.alloc(A.n);
    A.ones = A.alloc(A.n);
    A.parts = A.alloc((size_t)g.ny * g.nz + kRedBlocks);
    A.red = A.alloc(4 * (size_t)kRedBlocks + 8);
    A.gscal = A.alloc(4);
    const size_t npa = A.np ? A.np : 1;
    for (int d = 0; d < 3; ++d)
      for (double **p : {&A.lX[d], &A.lV[d], &A.lXint0[d], &A.lVint0[d], &A.lXnp1[d], &A.lVnp1[d],
                         &A.lXnew[d], &A.lVnew[d], &A.lXb[d], &A.lVb[d]}) {
        *p = A.alloc(npa);
        TPM_CUDA_TRY(cudaMemsetAsync(*p, 0, sizeof(double) * npa, c->stream));
      }
    {
      std::vector<double> ones((size_t)A.n, 1.0);
      TPM_CUDA_TRY(cudaMemcpy(A.ones, ones.data(), sizeof(double) * A.n, cudaMemcpyHostToDevice));
    }
    precondition_setup();
    TPM_CUDA_TRY(cudaMemsetAsync(A.gscal, 0, sizeof(double) * 4, c->stream));
    const bool prof = c->prof_on;
    c->prof_on = false;
    // ---- forward with checkpoints every K steps
    const int ncp = (nsteps + K - 1) / K;
    A.cps.resize(ncp);
    for (int k = 0; k < ncp; ++k) {
      Checkpoint &cp = A.cps[k];
      cp.RU = A.alloc(A.n3);
      cp.RU_int = A.alloc(A.n3);
      cp.Rho = A.alloc(A.n);
      cp.P = A.alloc(A.n);
      cp.Q = A.alloc(A.n);
      cp.rhs_t = A.alloc(npa);
      for (int q = 0; q < 7; ++q) cp.pq[q] = A.alloc(npa);
    }
    for (int st = 0; st < nsteps; ++st) {
      if (st % K == 0) save_cp(A, A.cps[st / K]);
      step_param_update(c);
      step_body(c);
    }
    // final state: objective and its gradient
    Checkpoint fin;
    fin.RU = A.alloc(A.n3);
    fin.RU_int = A.alloc(A.n3);
    fin.Rho = A.alloc(A.n);
    fin.P = A.alloc(A.n);
    fin.Q = A.alloc(A.n);
    fin.rhs_t = A.alloc(npa);
    for (int q = 0; q < 7; ++q) fin.pq[q] = A.alloc(npa);
    save_cp(A, fin);
    const bool fin_stepped = c->stepped;
    const int nbc = blocks_for(g.n);
    TPM_LAUNCH(c, "adj_obj_tke", k_obj_tke, nbc, kAT, 0, g, c->RU, c->Rho, w_tke, A.lRU, A.red);
    TPM_LAUNCH(c, "adj_finish", k_finish_sums, 1, kAT, 0, A.red, nbc, 1, 1.0 / (double)g.n,
               A.red + 3 * kRedBlocks);
    double tke = 0;
    TPM_CUDA_TRY(cudaMemcpyAsync(&tke, A.red + 3 * kRedBlocks, sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    double var = 0;
    if (A.np) {
      double *C = A.f;
      TPM_CUDA_TRY(cudaMemsetAsync(C, 0, sizeof(double) * A.n, c->stream));
      const int nbp = blocks_for(A.np);
      TPM_LAUNCH(c, "adj_conc", k_conc, nbp, kAT, 0, g, A.np, c->pq[0][0], c->pq[0][1],
                 c->pq[0][2], C);
      TPM_LAUNCH(c, "adj_sum2", k_sum2, nbc, kAT, 0, A.n, C, A.red);
      TPM_LAUNCH(c, "adj_finish", k_finish_sums, 1, kAT, 0, A.red, nbc, 2, 1.0 / (double)g.n,
                 A.red + 3 * kRedBlocks);
      double m[2];
      TPM_CUDA_TRY(cudaMemcpyAsync(m, A.red + 3 * kRedBlocks, 2 * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->stream));
      TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
      var = m[1] - m[0] * m[0];
      TPM_LAUNCH(c, "adj_obj_cvar", k_obj_cvar, nbp, kAT, 0, g, A.np, c->pq[0][0], c->pq[0][1],
                 c->pq[0][2], C, m[0], w_cvar, A.lX[0], A.lX[1], A.lX[2]);
    }
    const double J = w_tke * tke + w_cvar * var;
    TPM_CUDA_TRY(cudaMemsetAsync(A.lRUint0, 0, sizeof(double) * A.n3, c->stream));
    // ---- backward, segment by segment
    double gA = 0;
    for (int k = ncp - 1; k >= 0; --k) {
      load_cp(A, A.cps[k]);
      const int s0 = k * K, s1 = (s0 + K < nsteps) ? s0 + K : nsteps;
      std::vector<double> Asteps;
      for (int st = s0; st < s1; ++st) record_step(A, st - s0, Asteps);
      for (int st = s1 - 1; st >= s0; --st) {
        std::vector<double> parts;
        backward_step(A, st - s0, Asteps[st - s0], parts);
        for (double v : parts) gA += v;
      }
    }
    // t = 0: RU_int = RU (grid.cpp:461-472); project on divergence-free fields
    TPM_LAUNCH(c, "adj_add", k_add, blocks_for(A.n3), kAT, 0, A.n3, A.lRU, A.lRUint0, A.lnp1);
    proj_T(A, A.lnp1, nullptr, 0.0, A.lnewp);
    if (dJ_dRU0)
      TPM_CUDA_TRY(cudaMemcpyAsync(dJ_dRU0, A.lnewp, sizeof(double) * A.n3, cudaMemcpyDeviceToHost,
                                   c->stream));
    double gs[4];
    TPM_CUDA_TRY(cudaMemcpyAsync(gs, A.gscal, sizeof(gs), cudaMemcpyDeviceToHost, c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    // leave the context at the final state
    load_cp(A, fin);
    c->stepped = fin_stepped;
    c->prof_on = prof;
    if (J_out) *J_out = J;
    if (dJ_dA) *dJ_dA = gA;
    if (dJ_dtau) *dJ_dtau = gs[0];
    return TPM_OK;
  });
}
