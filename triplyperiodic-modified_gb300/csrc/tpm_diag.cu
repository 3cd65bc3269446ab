// Diagnostics of the step-boundary state, on the device:
//
//  * tpm_statistics: the scalars of grid::Statistics (grid.cpp:902-940) plus
//    the particle-concentration variance (tensor0::var, tensor0.cpp:516-519),
//    the rms velocity and the dissipation rate 2 nu <S_ij S_ij>;
//  * tpm_spectrum: the shell-summed energy spectrum of the face velocity,
//    through the pencil FFT passes of the pressure solve;
//  * tpm_rdf: the particle radial distribution function from a cell list.
//
// Every floating-point reduction is a fixed tree over a fixed number of
// blocks (no floating-point atomics), so each result is bit-reproducible; the
// pair counts of the RDF are integers.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "tpm_internal.cuh"

using tpm::Grid;

namespace tpm {
namespace {

constexpr int kDiagThreads = 256;
constexpr int kDiagBlocks = 1024;  // fixed: partial sums in a fixed order

// statistics slots (per-block partials, then the finished values)
enum Slot {
  S_RHO_SUM, S_RHO_MAX, S_RHO_MIN,
  S_C_SUM, S_C_MAX, S_C_MIN, S_C_SQ,
  S_TG_SUM,
  S_TKE_U, S_TKE_V, S_TKE_W,
  S_UMAX_X, S_UMAX_Y, S_UMAX_Z,
  S_USQ, S_SS, S_PS_SQ,
  S_VP_MAX, S_TP_MAX, S_TP_SUM,
  S_COUNT
};
enum { OP_SUM = 0, OP_MAX = 1, OP_MIN = 2 };

__host__ __device__ constexpr int slot_op(int s) {
  return (s == S_RHO_MAX || s == S_C_MAX || s == S_UMAX_X || s == S_UMAX_Y || s == S_UMAX_Z ||
          s == S_VP_MAX || s == S_TP_MAX)
             ? OP_MAX
             : (s == S_RHO_MIN || s == S_C_MIN) ? OP_MIN : OP_SUM;
}

__device__ __forceinline__ double op_apply(int op, double a, double b) {
  return op == OP_SUM ? a + b : op == OP_MAX ? (b > a ? b : a) : (b < a ? b : a);
}

__device__ __forceinline__ double op_identity(int op) {
  return op == OP_SUM ? 0.0 : op == OP_MAX ? -INFINITY : INFINITY;
}

// block reduction with the operation's identity in the unused lanes; result
// valid in thread 0; every thread of the block calls it
__device__ double block_reduce(int op, double v, double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op_apply(op, v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = op_identity(op);
  if (w == 0) {
    r = lane < nw ? sh[lane] : op_identity(op);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = op_apply(op, r, __shfl_down_sync(0xffffffffu, r, o));
  }
  return r;
}

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

// U = RU / I_C2F(Rho), the velocity grid::Statistics forms from RU_np1 and
// Rho_face (grid.cpp:917; tensor0.cpp:137-141 and the C2F mean
// (f[i] + f[i-1]) * 0.5 of tensor0.cpp:268-362)
__global__ void k_diag_velocity(Grid g, const double *__restrict__ RU,
                                const double *__restrict__ Rho, double *__restrict__ U) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const double r = Rho[c];
    U[c] = RU[c] / ((r + Rho[at(g, wrap_m(i, g.nx), j, k)]) * 0.5);
    U[g.n + c] = RU[g.n + c] / ((r + Rho[at(g, i, wrap_m(j, g.ny), k)]) * 0.5);
    U[2 * g.n + c] = RU[2 * g.n + c] / ((r + Rho[at(g, i, j, wrap_m(k, g.nz))]) * 0.5);
  }
}

// One pass over the cells: field sums, extrema, the grid::Statistics kinetic
// energies U_d*RU_d (grid.cpp:924-928), P0/R/Rho (grid.cpp:939), and the
// strain rate of the face velocity.  S_dd = dU_d/dd at the cell centre;
// S_xy = (du/dy + dv/dx)/2 on the z-directed edge through face corners
// (i, j), and likewise S_xz, S_yz: each of N^3 cells owns one edge of each
// kind, so S:S = S_xx^2 + S_yy^2 + S_zz^2 + 2 (S_xy^2 + S_xz^2 + S_yz^2)
// summed over cells is the volume integral.
__global__ void __launch_bounds__(kDiagThreads)
k_diag_cells(Grid g, const double *__restrict__ Rho, const double *__restrict__ C,
             const double *__restrict__ RU, const double *__restrict__ U,
             const double *__restrict__ PS, double a_tg, double *__restrict__ parts) {
  __shared__ double sh[32];
  double v[S_VP_MAX];
#pragma unroll
  for (int s = 0; s < S_VP_MAX; ++s) v[s] = op_identity(slot_op(s));
  const double *u = U, *vv = U + g.n, *w = U + 2 * g.n;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const double r = Rho[c];
    v[S_RHO_SUM] += r;
    v[S_RHO_MAX] = r > v[S_RHO_MAX] ? r : v[S_RHO_MAX];
    v[S_RHO_MIN] = r < v[S_RHO_MIN] ? r : v[S_RHO_MIN];
    const double cv = C[c];
    v[S_C_SUM] += cv;
    v[S_C_MAX] = cv > v[S_C_MAX] ? cv : v[S_C_MAX];
    v[S_C_MIN] = cv < v[S_C_MIN] ? cv : v[S_C_MIN];
    v[S_C_SQ] += cv * cv;
    v[S_TG_SUM] += a_tg / r;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double ud = U[d * g.n + c];
      v[S_TKE_U + d] += ud * RU[d * g.n + c];
      v[S_UMAX_X + d] = ud > v[S_UMAX_X + d] ? ud : v[S_UMAX_X + d];
      v[S_USQ] += ud * ud;
    }
    const int ip = wrap_p(i, g.nx), im = wrap_m(i, g.nx);
    const int jp = wrap_p(j, g.ny), jm = wrap_m(j, g.ny);
    const int kp = wrap_p(k, g.nz), km = wrap_m(k, g.nz);
    const double sxx = (u[at(g, ip, j, k)] - u[c]) * g.inv_dx;
    const double syy = (vv[at(g, i, jp, k)] - vv[c]) * g.inv_dy;
    const double szz = (w[at(g, i, j, kp)] - w[c]) * g.inv_dz;
    const double sxy = 0.5 * ((u[c] - u[at(g, i, jm, k)]) * g.inv_dy + (vv[c] - vv[at(g, im, j, k)]) * g.inv_dx);
    const double sxz = 0.5 * ((u[c] - u[at(g, i, j, km)]) * g.inv_dz + (w[c] - w[at(g, im, j, k)]) * g.inv_dx);
    const double syz = 0.5 * ((vv[c] - vv[at(g, i, j, km)]) * g.inv_dz + (w[c] - w[at(g, i, jm, k)]) * g.inv_dy);
    v[S_SS] += sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz);
    if (PS) v[S_PS_SQ] += PS[c] * PS[c];
  }
#pragma unroll
  for (int s = 0; s < S_VP_MAX; ++s) {
    const double b = block_reduce(slot_op(s), v[s], sh);
    if (threadIdx.x == 0) parts[s * kDiagBlocks + blockIdx.x] = b;
  }
}

// particle maxima and the temperature sum (particle.cpp:668-715)
__global__ void __launch_bounds__(kDiagThreads)
k_diag_particles(int64_t np, const double *__restrict__ up, const double *__restrict__ Tp,
                 double *__restrict__ parts) {
  __shared__ double sh[32];
  double vmax = -INFINITY, tmax = -INFINITY, tsum = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double a = up[p], t = Tp[p];
    vmax = a > vmax ? a : vmax;
    tmax = t > tmax ? t : tmax;
    tsum += t;
  }
  double b = block_reduce(OP_MAX, vmax, sh);
  if (threadIdx.x == 0) parts[S_VP_MAX * kDiagBlocks + blockIdx.x] = b;
  b = block_reduce(OP_MAX, tmax, sh);
  if (threadIdx.x == 0) parts[S_TP_MAX * kDiagBlocks + blockIdx.x] = b;
  b = block_reduce(OP_SUM, tsum, sh);
  if (threadIdx.x == 0) parts[S_TP_SUM * kDiagBlocks + blockIdx.x] = b;
}

__global__ void k_diag_finish(const double *__restrict__ parts, int cell_blocks,
                              int part_blocks, double *__restrict__ out) {
  __shared__ double sh[32];
  for (int s = 0; s < S_COUNT; ++s) {
    const int op = slot_op(s);
    const int nb = s >= S_VP_MAX ? part_blocks : cell_blocks;
    double v = op_identity(op);
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v = op_apply(op, v, parts[s * kDiagBlocks + b]);
    const double r = block_reduce(op, v, sh);
    if (threadIdx.x == 0) out[s] = r;
  }
}

// sum of the mode energies of each shell, in the fixed order of the mode list
__global__ void k_shell_sum(const double *__restrict__ emode, const int32_t *__restrict__ modes,
                            const int32_t *__restrict__ start, double *__restrict__ E) {
  __shared__ double sh[32];
  const int s = blockIdx.x;
  double v = 0;
  for (int m = start[s] + threadIdx.x; m < start[s + 1]; m += blockDim.x) v += emode[modes[m]];
  const double r = block_reduce(OP_SUM, v, sh);
  if (threadIdx.x == 0) E[s] = r;
}

// ----------------------------------------------------------------- RDF
struct RdfGrid {
  int mx, my, mz;
  double sx, sy, sz;  // cells per unit length
  double Lx, Ly, Lz, hx, hy, hz;
};

__device__ __forceinline__ int rdf_coord(double x, double s, int m) {
  int c = (int)(x * s);
  return c < 0 ? 0 : (c >= m ? m - 1 : c);
}

__device__ __forceinline__ int rdf_cell(const RdfGrid &r, double x, double y, double z) {
  return (rdf_coord(z, r.sz, r.mz) * r.my + rdf_coord(y, r.sy, r.my)) * r.mx + rdf_coord(x, r.sx, r.mx);
}

__global__ void k_rdf_count(RdfGrid r, int64_t np, const double *__restrict__ x,
                            const double *__restrict__ y, const double *__restrict__ z,
                            int32_t *__restrict__ counts) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&counts[rdf_cell(r, x[p], y[p], z[p])], 1);
}

// exclusive scan of ncell counts by one block: thread t owns one contiguous
// chunk (a diagnostic-sized array of at most 128^3 cells)
__global__ void k_rdf_scan(const int32_t *__restrict__ counts, long long ncell,
                           int32_t *__restrict__ start) {
  __shared__ long long sh[1024];
  const long long chunk = (ncell + blockDim.x - 1) / blockDim.x;
  const long long b = threadIdx.x * chunk, e = b + chunk < ncell ? b + chunk : ncell;
  long long s = 0;
  for (long long i = b; i < e; ++i) s += counts[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      long long v = sh[t];
      sh[t] = run;
      run += v;
    }
    start[ncell] = (int32_t)run;
  }
  __syncthreads();
  long long run = sh[threadIdx.x];
  for (long long i = b; i < e; ++i) {
    start[i] = (int32_t)run;
    run += counts[i];
  }
}

__global__ void k_rdf_scatter(RdfGrid r, int64_t np, const double *__restrict__ x,
                              const double *__restrict__ y, const double *__restrict__ z,
                              const int32_t *__restrict__ start, int32_t *__restrict__ fill,
                              double *__restrict__ pos) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double px = x[p], py = y[p], pz = z[p];
    const int cell = rdf_cell(r, px, py, pz);
    const int64_t at_ = start[cell] + atomicAdd(&fill[cell], 1);
    pos[at_] = px;
    pos[np + at_] = py;
    pos[2 * np + at_] = pz;
  }
}

__device__ __forceinline__ double min_image(double d, double L, double h) {
  if (d > h) return d - L;
  if (d < -h) return d + L;
  return d;
}

// Pairs (a, b), a < b in cell order, with minimum-image distance below r_max:
// each unordered pair once, whatever order the scatter left within a cell.
__global__ void __launch_bounds__(kDiagThreads)
k_rdf_pairs(RdfGrid r, int64_t np, const double *__restrict__ pos,
            const int32_t *__restrict__ start, double r_max2, double dr, int nbins,
            unsigned long long *__restrict__ hist) {
  extern __shared__ unsigned long long sh_hist[];
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh_hist[b] = 0;
  __syncthreads();
  const double *X = pos, *Y = pos + np, *Z = pos + 2 * np;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < np;
       a += (int64_t)gridDim.x * blockDim.x) {
    const double xa = X[a], ya = Y[a], za = Z[a];
    const int cx = rdf_coord(xa, r.sx, r.mx), cy = rdf_coord(ya, r.sy, r.my),
              cz = rdf_coord(za, r.sz, r.mz);
    for (int dz = -1; dz <= 1; ++dz) {
      const int nz = wrap_any(cz + dz, r.mz);
      for (int dy = -1; dy <= 1; ++dy) {
        const int ny = wrap_any(cy + dy, r.my);
        for (int dx = -1; dx <= 1; ++dx) {
          const int cell = (nz * r.my + ny) * r.mx + wrap_any(cx + dx, r.mx);
          int64_t b = start[cell], e = start[cell + 1];
          if (b <= a) b = a + 1;
          for (; b < e; ++b) {
            const double ddx = min_image(X[b] - xa, r.Lx, r.hx);
            const double ddy = min_image(Y[b] - ya, r.Ly, r.hy);
            const double ddz = min_image(Z[b] - za, r.Lz, r.hz);
            const double r2 = ddx * ddx + ddy * ddy + ddz * ddz;
            if (r2 < r_max2) {
              const int bin = (int)(sqrt(r2) / dr);
              if (bin < nbins) atomicAdd(&sh_hist[bin], 1ull);
            }
          }
        }
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    if (sh_hist[b]) atomicAdd(&hist[b], sh_hist[b]);
}

int diag_blocks(long long n) {
  long long b = (n + kDiagThreads - 1) / kDiagThreads;
  return (int)(b < 1 ? 1 : (b < kDiagBlocks ? b : kDiagBlocks));
}

void ensure_diag(tpm_ctx *c) {
  if (c->diag_u) return;
  c->diag_u = dalloc<double>(c, 3 * (size_t)c->g.n);
  c->diag_parts = dalloc<double>(c, (size_t)S_COUNT * kDiagBlocks);
  c->diag_out = dalloc<double>(c, S_COUNT + 64);
}

// Shells: nint(|k|/dk), |k| from the signed integer wave numbers of each
// half-spectrum mode; the mode list groups modes by shell in index order.
void ensure_spectrum(tpm_ctx *c) {
  if (c->diag_modes) return;
  const Grid &g = c->g;
  const double kx0 = 2.0 * kPi / g.Lx, ky0 = 2.0 * kPi / g.Ly, kz0 = 2.0 * kPi / g.Lz;
  double dk = kx0 < ky0 ? kx0 : ky0;
  dk = kz0 < dk ? kz0 : dk;
  const long long nm = (long long)g.nz * g.ny * g.nxh;
  std::vector<int32_t> shell(nm);
  int nshell = 0;
  for (int kz = 0; kz < g.nz; ++kz)
    for (int ky = 0; ky < g.ny; ++ky)
      for (int kx = 0; kx < g.nxh; ++kx) {
        const double a = kx * kx0;
        const double b = (ky <= g.ny / 2 ? ky : ky - g.ny) * ky0;
        const double d = (kz <= g.nz / 2 ? kz : kz - g.nz) * kz0;
        const double km = std::sqrt(a * a + b * b + d * d);
        const int s = (int)std::floor(km / dk + 0.5);
        shell[((long long)kz * g.ny + ky) * g.nxh + kx] = s;
        nshell = s + 1 > nshell ? s + 1 : nshell;
      }
  std::vector<int32_t> start(nshell + 1, 0), modes(nm);
  for (long long m = 0; m < nm; ++m) start[shell[m] + 1]++;
  for (int s = 0; s < nshell; ++s) start[s + 1] += start[s];
  std::vector<int32_t> fill(start.begin(), start.end() - 1);
  for (long long m = 0; m < nm; ++m) modes[fill[shell[m]]++] = (int32_t)m;
  c->diag_modes = dalloc<int32_t>(c, nm);
  c->diag_shell_start = dalloc<int32_t>(c, nshell + 1);
  c->diag_spec = dalloc<double2>(c, nm);
  c->diag_emode = dalloc<double>(c, nm);
  TPM_CUDA_TRY(cudaMemcpy(c->diag_modes, modes.data(), nm * sizeof(int32_t), cudaMemcpyHostToDevice));
  TPM_CUDA_TRY(cudaMemcpy(c->diag_shell_start, start.data(), (nshell + 1) * sizeof(int32_t),
                          cudaMemcpyHostToDevice));
  c->diag_nshell = nshell;
  c->diag_dk = dk;
  spectrum_kernels_setup();
}

void launch_velocity(tpm_ctx *c) {
  TPM_LAUNCH(c, "diag_velocity", k_diag_velocity, diag_blocks(c->g.n), kDiagThreads, 0, c->g,
             c->RU, c->Rho, c->diag_u);
}

int check_boundary(tpm_ctx *c) {
  if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize or tpm_resume has not run");
  if (!c->np1_is_base) return fail(c, TPM_ERR_STATE, "diagnostics are defined at a step boundary");
  return TPM_OK;
}

}  // namespace
}  // namespace tpm

using namespace tpm;

extern "C" {

int tpm_statistics(tpm_ctx *c, tpm_stats *out) {
  return guarded(c, [&]() -> int {
    if (!out) return fail(c, TPM_ERR_ARG, "null output");
    if (int rc = check_boundary(c)) return rc;
    ensure_diag(c);
    const Grid &g = c->g;
    launch_velocity(c);
    DevScalars ds;
    TPM_CUDA_TRY(cudaMemcpyAsync(&ds, c->dsc, sizeof(ds), cudaMemcpyDeviceToHost, c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const double a_tg = ds.P0 / c->R;  // P0/param_->R() (grid.cpp:939)
    const int cb = diag_blocks(g.n), pb = diag_blocks(c->np);
    TPM_LAUNCH(c, "diag_cells", k_diag_cells, cb, kDiagThreads, 0, g, c->Rho, c->C, c->RU,
               c->diag_u, c->PS, a_tg, c->diag_parts);
    if (c->np > 0)
      TPM_LAUNCH(c, "diag_particles", k_diag_particles, pb, kDiagThreads, 0, c->np, c->pq[0][3],
                 c->pq[0][6], c->diag_parts);
    TPM_LAUNCH(c, "diag_finish", k_diag_finish, 1, kDiagThreads, 0, c->diag_parts, cb,
               c->np > 0 ? pb : 0, c->diag_out);
    double v[S_COUNT];
    TPM_CUDA_TRY(cudaMemcpyAsync(v, c->diag_out, sizeof(v), cudaMemcpyDeviceToHost, c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const double n = (double)g.n;
    tpm_stats s = {};
    s.T_cur = c->T_cur;
    s.num_timestep = c->num_timestep;
    s.Rho_mean = v[S_RHO_SUM] / n;
    s.Rho_max = v[S_RHO_MAX];
    s.Rho_min = v[S_RHO_MIN];
    s.C_mean = v[S_C_SUM] / n;
    s.C_max = v[S_C_MAX];
    s.C_min = v[S_C_MIN];
    s.TKE_U = v[S_TKE_U] / n;
    s.TKE_V = v[S_TKE_V] / n;
    s.TKE_W = v[S_TKE_W] / n;
    s.TKE = s.TKE_U + s.TKE_V + s.TKE_W;
    // tensor1::max_cfl (tensor1.cpp:365-373) and tensor1::max (:327-335)
    const double dt = c->p.dt;
    double cfl = v[S_UMAX_X] * dt / g.dx, cy = v[S_UMAX_Y] * dt / g.dy, cz = v[S_UMAX_Z] * dt / g.dz;
    cfl = (cy > cfl) ? cy : cfl;
    cfl = (cz > cfl) ? cz : cfl;
    s.Gas_CFL_Max = cfl;
    double um = v[S_UMAX_X];
    um = (v[S_UMAX_Y] > um) ? v[S_UMAX_Y] : um;
    um = (v[S_UMAX_Z] > um) ? v[S_UMAX_Z] : um;
    s.u_max = um;
    s.Gas_Max_Diff_CFL = dt / (g.dx * g.dx * s.Rho_min / c->p.Mu0) * 6.;  // grid.cpp:934
    // particle::max returns -1e9 for an empty set (particle.cpp:671)
    s.Vp_max = c->np > 0 ? v[S_VP_MAX] : -1e9;
    s.Tp_max = c->np > 0 ? v[S_TP_MAX] : -1e9;
    s.Tp_mean = c->np > 0 ? v[S_TP_SUM] / (double)c->np : 0.0;
    s.Tg_mean = v[S_TG_SUM] / n;
    s.P0 = ds.P0;
    s.TKE2 = c->stepped ? ds.tke2 : 0.0;
    s.HT_mean = c->stepped ? ds.mean_Q : 0.0;
    s.num_iteration = c->stepped ? ds.it : 0;
    s.C_var = v[S_C_SQ] / n - s.C_mean * s.C_mean;  // tensor0::var
    s.u_rms = std::sqrt(v[S_USQ] / n / 3.0);
    s.dissipation = 2.0 * (c->p.Mu0 / c->p.Rho0) * (v[S_SS] / n);
    s.Passive_Scalar_mean = c->PS ? v[S_PS_SQ] / n : 0.0;  // tensor0::mean_squares
    *out = s;
    return TPM_OK;
  });
}

int tpm_spectrum_shells(tpm_ctx *c, int *nshells, double *dk) {
  return guarded(c, [&]() -> int {
    ensure_spectrum(c);
    if (nshells) *nshells = c->diag_nshell;
    if (dk) *dk = c->diag_dk;
    return TPM_OK;
  });
}

int tpm_spectrum(tpm_ctx *c, double *E, int nshells) {
  return guarded(c, [&]() -> int {
    if (!E) return fail(c, TPM_ERR_ARG, "null output");
    if (int rc = check_boundary(c)) return rc;
    ensure_diag(c);
    ensure_spectrum(c);
    if (nshells < c->diag_nshell)
      return fail(c, TPM_ERR_ARG, "nshells below tpm_spectrum_shells (" +
                                      std::to_string(c->diag_nshell) + ")");
    launch_velocity(c);
    spectrum_mode_energy(c, c->diag_u, c->diag_spec, c->diag_emode);
    // per-shell sums land in the statistics partials (S_COUNT * kDiagBlocks doubles,
    // more than the ~0.87 max(N) shells of any supported grid)
    double *dev = c->diag_parts;
    TPM_LAUNCH(c, "shell_sum", k_shell_sum, c->diag_nshell, kDiagThreads, 0, c->diag_emode,
               c->diag_modes, c->diag_shell_start, dev);
    TPM_CUDA_TRY(cudaMemcpyAsync(E, dev, sizeof(double) * c->diag_nshell, cudaMemcpyDeviceToHost,
                                 c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int s = c->diag_nshell; s < nshells; ++s) E[s] = 0;
    return TPM_OK;
  });
}

int tpm_rdf(tpm_ctx *c, double r_max, int nbins, unsigned long long *pairs, double *gr) {
  return guarded(c, [&]() -> int {
    if (!pairs) return fail(c, TPM_ERR_ARG, "null output");
    if (nbins < 1 || nbins > 4096) return fail(c, TPM_ERR_ARG, "nbins must be in [1, 4096]");
    if (!(r_max > 0)) return fail(c, TPM_ERR_ARG, "r_max must be positive");
    if (int rc = check_boundary(c)) return rc;
    const Grid &g = c->g;
    RdfGrid r;
    int *m[3] = {&r.mx, &r.my, &r.mz};
    const double L[3] = {g.Lx, g.Ly, g.Lz};
    for (int d = 0; d < 3; ++d) {
      // cells no smaller than r_max, at most 128 per direction, at least 3
      int k = (int)std::floor(L[d] / r_max + 1e-9);  // L/(L/3) may round below 3
      while (k > 1 && L[d] / k < r_max) --k;
      if (k > 128) k = 128;
      if (k < 3) return fail(c, TPM_ERR_ARG, "r_max must be at most min(L)/3");
      *m[d] = k;
    }
    r.sx = r.mx / g.Lx;
    r.sy = r.my / g.Ly;
    r.sz = r.mz / g.Lz;
    r.Lx = g.Lx; r.Ly = g.Ly; r.Lz = g.Lz;
    r.hx = 0.5 * g.Lx; r.hy = 0.5 * g.Ly; r.hz = 0.5 * g.Lz;
    const long long ncell = (long long)r.mx * r.my * r.mz;
    for (int b = 0; b < nbins; ++b) pairs[b] = 0;
    if (c->np >= 2) {
      if (ncell > c->rdf_cells_cap) {
        c->rdf_counts = dalloc<int32_t>(c, ncell + 1);
        c->rdf_start = dalloc<int32_t>(c, ncell + 1);
        c->rdf_fill = dalloc<int32_t>(c, ncell + 1);
        c->rdf_cells_cap = ncell;
      }
      if (!c->rdf_pos) c->rdf_pos = dalloc<double>(c, 3 * (size_t)c->np);
      if (nbins > c->rdf_bins_cap) {
        c->rdf_hist = dalloc<unsigned long long>(c, nbins);
        c->rdf_bins_cap = nbins;
      }
      const int pb = diag_blocks(c->np);
      TPM_CUDA_TRY(cudaMemsetAsync(c->rdf_counts, 0, sizeof(int32_t) * ncell, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->rdf_fill, 0, sizeof(int32_t) * ncell, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->rdf_hist, 0, sizeof(unsigned long long) * nbins, c->stream));
      const double *x = c->pq[0][0], *y = c->pq[0][1], *z = c->pq[0][2];
      TPM_LAUNCH(c, "rdf_count", k_rdf_count, pb, kDiagThreads, 0, r, c->np, x, y, z,
                 c->rdf_counts);
      TPM_LAUNCH(c, "rdf_scan", k_rdf_scan, 1, 1024, 0, c->rdf_counts, ncell, c->rdf_start);
      TPM_LAUNCH(c, "rdf_scatter", k_rdf_scatter, pb, kDiagThreads, 0, r, c->np, x, y, z,
                 c->rdf_start, c->rdf_fill, c->rdf_pos);
      const int qb = (int)((c->np + kDiagThreads - 1) / kDiagThreads);
      TPM_LAUNCH(c, "rdf_pairs", k_rdf_pairs, qb, kDiagThreads,
                 sizeof(unsigned long long) * nbins, r, c->np, c->rdf_pos, c->rdf_start,
                 r_max * r_max, r_max / nbins, nbins, c->rdf_hist);
      TPM_CUDA_TRY(cudaMemcpyAsync(pairs, c->rdf_hist, sizeof(unsigned long long) * nbins,
                                   cudaMemcpyDeviceToHost, c->stream));
      TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    if (gr) {
      const double np = (double)c->np, dr = r_max / nbins;
      const double npair = np * (np - 1.0) * 0.5, vol = g.Lx * g.Ly * g.Lz;
      for (int b = 0; b < nbins; ++b) {
        const double shell = (4.0 / 3.0) * kPi * (std::pow((b + 1) * dr, 3) - std::pow(b * dr, 3));
        const double ideal = npair * shell / vol;
        gr[b] = ideal > 0 ? (double)pairs[b] / ideal : 0.0;
      }
    }
    return TPM_OK;
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 FMA throughput of the current device (the roof of the FP64 path,
// whose kernels are bound by the FP64 pipe rather than by HBM): every thread
// runs eight independent chains of dependent FMAs, so the pipe never waits
// on a result; 2 flops per FMA.
namespace tpm {
__global__ void k_fp64_fma_peak(double *__restrict__ sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = (threadIdx.x + 32 * j) * 1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  if (s == -1.0) sink[blockIdx.x] = s;  // never true for these inputs: keeps the chains live
}
}  // namespace tpm

extern "C" int tpm_measure_fp64_peak(double *tflops) {
  if (!tflops) return TPM_ERR_ARG;
  *tflops = 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return TPM_ERR_CUDA;
  const int threads = 256, blocks = sms * 8, iters = 8192;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = TPM_OK;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = TPM_ERR_CUDA;
  } else {
    double best = 0;
    for (int r = 0; r < 4 && rc == TPM_OK; ++r) {  // the first launch warms up
      tpm::k_fp64_fma_peak<<<blocks, threads, 0, st>>>(nullptr, iters, 0.9999999, 1e-9);
      if (cudaEventRecord(e0, st) != cudaSuccess) rc = TPM_ERR_CUDA;
      tpm::k_fp64_fma_peak<<<blocks, threads, 0, st>>>(nullptr, iters, 0.9999999, 1e-9);
      float ms = 0;
      if (rc != TPM_OK || cudaEventRecord(e1, st) != cudaSuccess ||
          cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        rc = TPM_ERR_CUDA;
      else if (r > 0 && ms > 0)
        best = std::max(best, 2.0 * 8.0 * iters * (double)threads * blocks / (ms * 1e-3) / 1e12);
    }
    *tflops = best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return rc;
}
