// Grid-side kernels of the FP64 RK4 substep.
//
// Each kernel fuses a run of the reference's whole-field sweeps
// (tensor0/tensor1 operators, grid.cpp:608-863) into one pass over the box.
// Halo exchange becomes periodic index wrap.  Every expression keeps the
// reference's floating-point operation order and the library is compiled
// with --fmad=false, so apart from reductions and the FFT the results are
// the reference's to the last bit.
#include <cudaTypedefs.h>

#include <map>
#include <mutex>
#include <utility>

#include "tpm_internal.cuh"
#include "tpm_ff.cuh"
#include "tpm_reduce.cuh"
#include "tpm_tma.cuh"

namespace tpm {
namespace {

constexpr int kThreads = 256;

struct Cell {
  int i, j, k;
  long long c;
};

__device__ __forceinline__ Cell cell_of(const Grid &g, long long c) {
  Cell r;
  r.c = c;
  cell_ijk(g, c, r.i, r.j, r.k);
  return r;
}

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

// ---------------------------------------------------------------- P0 update
// grid::Update_P0, grid.cpp:816-830, with mean(RHS_Part_Temp) finished from
// the heat deposit's per-block partial sums.
__global__ void k_p0_update(const double *__restrict__ partials, int nparts, DevScalars *s,
                            long long ntot, int cooling, double R, double Cv, double Cp,
                            double Vcell, double dtpo, double dtpr, int stage, int np1_is_base) {
  __shared__ double sh[kThreads];
  double v = 0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += partials[b];
  double sum = block_sum(v, sh);
  if (threadIdx.x == 0) {
    double mean_energy_transferred = sum / (double)ntot;
    double dP0_dt = cooling ? 0.0 : -R / Cv * mean_energy_transferred / Vcell;
    double np1 = np1_is_base ? s->P0 : s->P0_np1;
    np1 += dtpo * dP0_dt;
    s->P0_np1 = np1;
    s->P0_new = (stage != 3) ? s->P0 + dtpr * dP0_dt : np1;
    s->T_scale = s->P0_new / R;
    s->coef_div = -R / (Cp * s->P0_new * Vcell);
    s->mean_Q = mean_energy_transferred;
  }
}

// ---------------------------------------------------------------- density
// grid::Update_Rho, grid.cpp:608-614, plus the two centre fields the rest of
// the substep needs: 1/Rho_new (grid.cpp:834) and T = (P0_new/R)/Rho_new
// (grid.cpp:882).
__global__ void k_rho_update(Grid g, const double *__restrict__ RUi, const double *__restrict__ Rho,
                             const double *__restrict__ np1_in, double *__restrict__ Rho_np1,
                             double *__restrict__ Rho_new, double *__restrict__ inv_rho,
                             double *__restrict__ Tgas, const DevScalars *__restrict__ s,
                             double a_np1, double b_new, int stage) {
  const double *RUx = RUi, *RUy = RUi + g.n, *RUz = RUi + 2 * g.n;
  const double T_scale = s->T_scale;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    double D = (RUx[at(g, wrap_p(q.i, g.nx), q.j, q.k)] - RUx[c]) * g.inv_dx +
               (RUy[at(g, q.i, wrap_p(q.j, g.ny), q.k)] - RUy[c]) * g.inv_dy +
               (RUz[at(g, q.i, q.j, wrap_p(q.k, g.nz))] - RUz[c]) * g.inv_dz;
    double np1 = np1_in[c] + a_np1 * D;
    double nw = (stage != 3) ? 1 * Rho[c] + b_new * D : np1;
    Rho_np1[c] = np1;
    Rho_new[c] = nw;
    inv_rho[c] = 1. / nw;
    Tgas[c] = T_scale / nw;
  }
}

// ------------------------------------------------------------ face velocity
// U = RU_int / Rho_face with Rho_face = I_C2F(Rho_int) (grid.cpp:868,843).
__global__ void k_face_velocity(Grid g, const double *__restrict__ RUi,
                                const double *__restrict__ Rho_int, double *__restrict__ U) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    double r = Rho_int[c];
    U[c] = RUi[c] / ((r + Rho_int[at(g, wrap_m(q.i, g.nx), q.j, q.k)]) * 0.5);
    U[g.n + c] = RUi[g.n + c] / ((r + Rho_int[at(g, q.i, wrap_m(q.j, g.ny), q.k)]) * 0.5);
    U[2 * g.n + c] = RUi[2 * g.n + c] / ((r + Rho_int[at(g, q.i, q.j, wrap_m(q.k, g.nz))]) * 0.5);
  }
}

// ------------------------------------------------------- momentum RHS + RK
struct RhsArgs {
  double a_fp;   // -mp/Vcell
  double b_gd;   // Mu0/3.
  double c_lap;  // Mu0
  double A, Rho0, g[3];
  double dtpo, dtpr;
  int stage, has_g;
  // the same coefficients and 1/d, 1/d^2 rounded to FP32 on the host, for
  // the FP32 stencil (no per-thread FP64 conversions)
  float f_a_fp, f_b_gd, f_c_lap, f_A, f_Rho0, f_g[3], f_inv_d[3], f_inv_d2[3];
};

// offsets of the neighbour in direction e (0,1,2) at +1 / -1, wrapped
struct Nbr {
  long long p[3], m[3];
};
__device__ __forceinline__ Nbr nbr_of(const Grid &g, const Cell &q) {
  Nbr r;
  r.p[0] = at(g, wrap_p(q.i, g.nx), q.j, q.k);
  r.m[0] = at(g, wrap_m(q.i, g.nx), q.j, q.k);
  r.p[1] = at(g, q.i, wrap_p(q.j, g.ny), q.k);
  r.m[1] = at(g, q.i, wrap_m(q.j, g.ny), q.k);
  r.p[2] = at(g, q.i, q.j, wrap_p(q.k, g.nz));
  r.m[2] = at(g, q.i, q.j, wrap_m(q.k, g.nz));
  return r;
}

// grid::Update_RU_WOP (grid.cpp:776-814) on the mixed path: the right-hand
// side in FP32 from FP32 copies of U, RU_int and F_p, the RK combinations
// RU_np1 += dt*post*RHS, RU_new = RU + dt*pre*RHS in FP64 (FMAs).  Per cell
// and component d: grad_C2F(div U) (tensor1.cpp:259-270, tensor0.cpp:249-256)
// times Mu0/3, Del2(U_d) (tensor0.cpp:258-265) times Mu0, -mp/Vcell F_p, the
// convection Div_F2C of the fluxes P_{d,e} = I_e,C2F(U_d) I_d,C2F(RU_e)
// (grid.cpp:785-801), the forcing A RU_int (grid.cpp:803) and the body force
// (Rho_face - Rho0) g (grid.cpp:805-809), each in the reference's operation
// order.  A block owns a kZX x kZY column of cells and walks zlen planes up
// in z; the FP32 copies of U and RU_int live in a ring of three
// shared-memory planes (z - 1, z, z + 1) with a one-cell halo in x and y, so
// each value is loaded from global memory once per column instead of once
// per stencil use.
constexpr int kZX = 32, kZY = 8;  // column tile; the z chunk is zm_zlen planes

// The FP32 momentum right-hand side of one cell, all three components, from
// its stencil values V(f, dx, dy, dz) (f 0-2 the face velocity U, 3-5 RU_int,
// at the offset (dx, dy, dz) from the cell) and its F_p: per component d
// (grid.cpp:785-803) -mp/Vcell F_p + Mu0/3 grad_C2F(div U) + Mu0 Del2(U_d)
// - Div_F2C(P_{d,e}) + A RU_int, the fluxes P_{d,e} = I_e(U_d) I_d(RU_e), in
// the reference's operation order (the body force is the caller's).
template <typename VF>
__device__ __forceinline__ void momentum_rhs(const VF &V, const float fp[3], const float inv_d[3],
                                             const float inv_d2[3], float a_fp, float b_gd,
                                             float c_lap, float A_, float rhs[3]) {
  auto divU = [&](int ox, int oy, int oz) -> float {
    return (V(0, ox + 1, oy, oz) - V(0, ox, oy, oz)) * inv_d[0] +
           (V(1, ox, oy + 1, oz) - V(1, ox, oy, oz)) * inv_d[1] +
           (V(2, ox, oy, oz + 1) - V(2, ox, oy, oz)) * inv_d[2];
  };
  const float div_c = divU(0, 0, 0);
  const float div_m[3] = {divU(-1, 0, 0), divU(0, -1, 0), divU(0, 0, -1)};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float gd = (div_c - div_m[d]) * inv_d[d];
    const float ud = V(d, 0, 0, 0);
    const float lap = (V(d, 1, 0, 0) - 2 * ud + V(d, -1, 0, 0)) * inv_d2[0] +
                      (V(d, 0, 1, 0) - 2 * ud + V(d, 0, -1, 0)) * inv_d2[1] +
                      (V(d, 0, 0, 1) - 2 * ud + V(d, 0, 0, -1)) * inv_d2[2];
    float r = a_fp * fp[d] + b_gd * gd + c_lap * lap;
    // flux P_{d,e} at (ox, oy, oz): I_e(U_d) * I_d(RU_e)
    auto flux = [&](int e, int ox, int oy, int oz) -> float {
      const int ex = e == 0, ey = e == 1, ez = e == 2;
      const int dx = d == 0, dy = d == 1, dz = d == 2;
      const float iu = (V(d, ox, oy, oz) + V(d, ox - ex, oy - ey, oz - ez)) * 0.5f;
      const float ir = (V(3 + e, ox, oy, oz) + V(3 + e, ox - dx, oy - dy, oz - dz)) * 0.5f;
      return iu * ir;
    };
    float t[3];
#pragma unroll
    for (int e = 0; e < 3; ++e)
      t[e] = (flux(e, e == 0, e == 1, e == 2) - flux(e, 0, 0, 0)) * inv_d[e];
    const float conv = t[0] + t[1] + t[2];
    r -= conv;
    r += A_ * V(3 + d, 0, 0, 0);
    rhs[d] = r;
  }
}
constexpr int kZPX = kZX + 2, kZPY = kZY + 2, kZPlane = kZPX * kZPY;

__global__ void __launch_bounds__(kZX * kZY, 4)
k_rhs_momentum_zm(Grid g, const float *__restrict__ U, const float *__restrict__ RUi,
                  const float *__restrict__ Fp, const double *__restrict__ Rho_int,
                  const double *__restrict__ RU, const double *__restrict__ np1_in,
                  double *__restrict__ RU_np1, double *__restrict__ RU_new, RhsArgs a,
                  int zlen) {
  // [slot][field][plane]: fields 0-2 U, 3-5 RU_int
  __shared__ float sp[3][6][kZPlane];
  const int tx = threadIdx.x % kZX, ty = threadIdx.x / kZX;
  const int tilesx = (g.nx + kZX - 1) / kZX, tilesy = (g.ny + kZY - 1) / kZY;
  const int bx = blockIdx.x % tilesx, by = (blockIdx.x / tilesx) % tilesy;
  const int bz = blockIdx.x / (tilesx * tilesy);
  const int i0 = bx * kZX, j0 = by * kZY, k0 = bz * zlen;
  const int k1 = min(k0 + zlen, g.nz);
  const int i = i0 + tx, j = j0 + ty;
  const bool live = i < g.nx && j < g.ny;
  const float inv_d[3] = {a.f_inv_d[0], a.f_inv_d[1], a.f_inv_d[2]};
  const float inv_d2[3] = {a.f_inv_d2[0], a.f_inv_d2[1], a.f_inv_d2[2]};
  const float a_fp = a.f_a_fp, b_gd = a.f_b_gd, c_lap = a.f_c_lap, A_ = a.f_A, Rho0 = a.f_Rho0;
  const float gv[3] = {a.f_g[0], a.f_g[1], a.f_g[2]};
  // plane kk (any integer, wrapped) of the six fields: a thread's share of the
  // 34 x 10 halo plane (at most two elements) is fetched into registers, then
  // stored into a ring slot; the fetch of plane k + 2 is issued before plane k
  // is computed, so its loads are in flight during the stencil
  constexpr int kPer = (kZPlane + kZX * kZY - 1) / (kZX * kZY);
  float pre[kPer][6];
  auto fetch_plane = [&](int kk) {
    kk %= g.nz;
    if (kk < 0) kk += g.nz;
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int e = threadIdx.x + u * kZX * kZY;
      if (e < kZPlane) {
        const int hy = e / kZPX, hx = e - hy * kZPX;
        int ii = i0 - 1 + hx, jj = j0 - 1 + hy;  // one cell of halo: one wrap at most
        ii = ii < 0 ? ii + g.nx : (ii >= g.nx ? ii - g.nx : ii);
        jj = jj < 0 ? jj + g.ny : (jj >= g.ny ? jj - g.ny : jj);
        const long long c = at(g, ii, jj, kk);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          pre[u][f] = U[f * g.n + c];
          pre[u][3 + f] = RUi[f * g.n + c];
        }
      }
    }
  };
  auto store_plane = [&](int slot) {
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int e = threadIdx.x + u * kZX * kZY;
      if (e < kZPlane) {
#pragma unroll
        for (int f = 0; f < 6; ++f) sp[slot][f][e] = pre[u][f];
      }
    }
  };
  fetch_plane(k0 - 1);
  store_plane(0);
  fetch_plane(k0);
  store_plane(1);
  fetch_plane(k0 + 1);
  int sm = 0, s0 = 1;  // ring slots of planes k - 1 and k
  for (int k = k0; k < k1; ++k) {
    const int sp1 = 3 - sm - s0;  // slot of plane k + 1
    store_plane(sp1);
    __syncthreads();
    if (k + 1 < k1) fetch_plane(k + 2);
    if (live) {
      const int slot_of[3] = {sm, s0, sp1};
      // value of field f at the offset (dx, dy, dz) from the cell
      auto V = [&](int f, int dx, int dy, int dz) -> float {
        return sp[slot_of[dz + 1]][f][(ty + 1 + dy) * kZPX + tx + 1 + dx];
      };
      const long long c = at(g, i, j, k);
      const long long cm[3] = {at(g, wrap_m(i, g.nx), j, k), at(g, i, wrap_m(j, g.ny), k),
                               at(g, i, j, wrap_m(k, g.nz))};
      // the cell's own inputs, loaded ahead of the stencil arithmetic
      float fp[3];
      double in_np1[3], in_ru[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        fp[d] = Fp[d * g.n + c];
        in_np1[d] = np1_in[d * g.n + c];
        in_ru[d] = a.stage != 3 ? RU[d * g.n + c] : 0.0;
      }
      float rhs[3];
      momentum_rhs(V, fp, inv_d, inv_d2, a_fp, b_gd, c_lap, A_, rhs);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (a.has_g) {
          const float rf = (ff_cast<float>(Rho_int[c]) + ff_cast<float>(Rho_int[cm[d]])) * 0.5f;
          rhs[d] += (rf - Rho0) * gv[d];
        }
        const double r64 = ff_widen(rhs[d]);
        const double np1 = fma(a.dtpo, r64, in_np1[d]);
        RU_np1[d * g.n + c] = np1;
        RU_new[d * g.n + c] = (a.stage != 3) ? fma(a.dtpr, r64, in_ru[d]) : np1;
      }
    }
    __syncthreads();  // plane k - 1's slot takes plane k + 2 next
    sm = s0;
    s0 = sp1;
  }
}

// grid::Update_RU_WOP (grid.cpp:776-814) on the FP64 path, every operation
// the reference's (the terms of k_rhs_momentum_zm, in FP64 with separate
// multiplies and adds).  One block owns a TX x TY x TZ tile; U and RU_int of
// the tile plus a one-cell halo are staged in shared memory, the divergence
// of U and the nine convective fluxes P_{d,e} are evaluated once per cell of
// the tile (a per-cell form re-evaluates them 4x and 2x), then each thread
// assembles its cell.
constexpr int kTX = 32, kTY = 4, kTZ = 2;
constexpr int kBX = kTX + 2, kBY = kTY + 2, kBZ = kTZ + 2;  // staged box
constexpr int kFX = kTX + 1, kFY = kTY + 1, kFZ = kTZ + 1;  // divergence / flux boxes
constexpr int kBox = kBX * kBY * kBZ, kFBox = kFX * kFY * kFZ;

template <typename TC>
constexpr size_t rhs_tiled_smem() {
  return sizeof(TC) * (6 * (size_t)kBox + (size_t)kFBox + 9 * (size_t)kFBox);
}

template <typename TC, typename TIn>
__global__ void __launch_bounds__(kTX * kTY * kTZ)
k_rhs_momentum_tiled(Grid g, const TIn *__restrict__ U, const TIn *__restrict__ RUi,
                     const TIn *__restrict__ Fp, const double *__restrict__ Rho_int,
                     const double *__restrict__ RU, const double *__restrict__ np1_in,
                     double *__restrict__ RU_np1, double *__restrict__ RU_new, RhsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TC *sU = reinterpret_cast<TC *>(smem_raw);  // [3][kBox]
  TC *sR = sU + 3 * kBox;                      // [3][kBox]
  TC *sD = sR + 3 * kBox;                      // [kFBox] divergence, box coords 0..T
  TC *sP = sD + kFBox;                         // [9][kFBox] fluxes, box coords 1..T+1
  const int tilesx = (g.nx + kTX - 1) / kTX, tilesy = (g.ny + kTY - 1) / kTY;
  const int bx = blockIdx.x % tilesx, by = (blockIdx.x / tilesx) % tilesy,
            bz = blockIdx.x / (tilesx * tilesy);
  const int i0 = bx * kTX, j0 = by * kTY, k0 = bz * kTZ;
  const int t = threadIdx.x;
  const TC inv_d[3] = {(TC)g.inv_dx, (TC)g.inv_dy, (TC)g.inv_dz};
  const TC inv_d2[3] = {(TC)g.inv_dx2, (TC)g.inv_dy2, (TC)g.inv_dz2};
  // ---- stage U and RU_int with a one-cell periodic halo
  for (int b = t; b < kBox; b += blockDim.x) {
    const int xb = b % kBX, yb = (b / kBX) % kBY, zb = b / (kBX * kBY);
    const int i = wrap_any(i0 + xb - 1, g.nx), j = wrap_any(j0 + yb - 1, g.ny),
              k = wrap_any(k0 + zb - 1, g.nz);
    const long long c = at(g, i, j, k);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      sU[d * kBox + b] = (TC)U[d * g.n + c];
      sR[d * kBox + b] = (TC)RUi[d * g.n + c];
    }
  }
  __syncthreads();
  auto B = [](int x, int y, int z) { return (z * kBY + y) * kBX + x; };
  // ---- divergence of U at box cells 0..T (tile-relative -1..T-1)
  for (int f = t; f < kFBox; f += blockDim.x) {
    const int x = f % kFX, y = (f / kFX) % kFY, z = f / (kFX * kFY);
    const int b = B(x, y, z);
    sD[f] = (sU[b + 1] - sU[b]) * inv_d[0] + (sU[kBox + b + kBX] - sU[kBox + b]) * inv_d[1] +
            (sU[2 * kBox + b + kBX * kBY] - sU[2 * kBox + b]) * inv_d[2];
  }
  // ---- convective fluxes P_{d,e} = I_e(U_d) * I_d(RU_e) at box cells 1..T+1
  const int off[3] = {1, kBX, kBX * kBY};
  for (int f = t; f < 9 * kFBox; f += blockDim.x) {
    const int de = f / kFBox, r = f % kFBox;
    const int d = de / 3, e = de % 3;
    const int x = r % kFX + 1, y = (r / kFX) % kFY + 1, z = r / (kFX * kFY) + 1;
    const int b = B(x, y, z);
    const TC iu = (sU[d * kBox + b] + sU[d * kBox + b - off[e]]) * (TC)0.5;
    const TC ir = (sR[e * kBox + b] + sR[e * kBox + b - off[d]]) * (TC)0.5;
    sP[f] = iu * ir;
  }
  __syncthreads();
  // ---- assemble each cell of the tile
  const int rx = t % kTX, ry = (t / kTX) % kTY, rz = t / (kTX * kTY);
  const int i = i0 + rx, j = j0 + ry, k = k0 + rz;
  if (i >= g.nx || j >= g.ny || k >= g.nz) return;
  const long long c = at(g, i, j, k);
  const int b = B(rx + 1, ry + 1, rz + 1);
  const int fb = (rz + 1) * kFX * kFY + (ry + 1) * kFX + (rx + 1);  // divergence index of the cell
  const int fp = rz * kFX * kFY + ry * kFX + rx;                    // flux index of the cell
  const int foff[3] = {1, kFX, kFX * kFY};
  const TC div_c = sD[fb];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const TC *Ud = sU + d * kBox;
    TC gd = (div_c - sD[fb - foff[d]]) * inv_d[d];
    TC ud = Ud[b];
    TC lap = (Ud[b + off[0]] - 2 * ud + Ud[b - off[0]]) * inv_d2[0] +
             (Ud[b + off[1]] - 2 * ud + Ud[b - off[1]]) * inv_d2[1] +
             (Ud[b + off[2]] - 2 * ud + Ud[b - off[2]]) * inv_d2[2];
    TC rhs = (TC)a.a_fp * (TC)Fp[d * g.n + c] + (TC)a.b_gd * gd + (TC)a.c_lap * lap;
    TC tt[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const TC *Pde = sP + (d * 3 + e) * kFBox;
      tt[e] = (Pde[fp + foff[e]] - Pde[fp]) * inv_d[e];
    }
    rhs -= tt[0] + tt[1] + tt[2];
    rhs += (TC)a.A * sR[d * kBox + b];
    if (a.has_g) {
      const long long cm = d == 0 ? at(g, wrap_m(i, g.nx), j, k)
                           : d == 1 ? at(g, i, wrap_m(j, g.ny), k)
                                    : at(g, i, j, wrap_m(k, g.nz));
      TC rf = ((TC)Rho_int[c] + (TC)Rho_int[cm]) * (TC)0.5;
      rhs += (rf - (TC)a.Rho0) * (TC)a.g[d];
    }
    const double r64 = (double)rhs;
    double np1 = np1_in[d * g.n + c] + a.dtpo * r64;
    RU_np1[d * g.n + c] = np1;
    RU_new[d * g.n + c] = (a.stage != 3) ? 1 * RU[d * g.n + c] + a.dtpr * r64 : np1;
  }
}

// ---------------------------------------------------- Poisson right side
// grid::Compute_Div_U_new (grid.cpp:832-839), grid::Compute_RHS_Pois
// (grid.cpp:841-849) and the coefficient set-up of grid::Solve_Poisson /
// poisson::FFT (grid.cpp:853, poisson.cpp:393-394).  The mean of RHS_Pois is
// reduced per block; it is subtracted where RHS_Pois is read.
struct PoisArgs {
  double kCp;        // k/Cp
  double inv_dtpre;  // 1./(dt*pre)
  int cooling, store_div;
};

// FP64 path, split in two passes so that each face's two divisions are done
// once instead of once per adjacent cell (an FP64 division is ~10 FP64-pipe
// operations; the kernel is FP64-pipe bound):
//   k_poisson_faces: Rho_face = I_C2F(Rho_new), C = 1/Rho_face (Cface) and
//                    U = RU_new/Rho_face on the three lower faces of each cell;
//   k_poisson_rhs2:  divergence constraint, RHS_Pois and the centre coefficient
//                    from those face values.
// Every value is formed by the reference's operations in its order, and each
// face value is the same whichever adjacent cell asks for it.
__global__ void k_poisson_faces(Grid g, const double *__restrict__ Rho_new,
                                const double *__restrict__ RUn, double *__restrict__ Cface,
                                double *__restrict__ Uf) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    const double r = Rho_new[c];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double rf = (r + Rho_new[nb.m[d]]) * 0.5;
      Cface[d * g.n + c] = 1. / rf;
      Uf[d * g.n + c] = RUn[d * g.n + c] / rf;
    }
  }
}

__global__ void k_poisson_rhs2(Grid g, const double *__restrict__ inv_rho,
                               const double *__restrict__ Q, const double *__restrict__ Uf,
                               const double *__restrict__ Cface, const DevScalars *__restrict__ s,
                               double *__restrict__ RHS, double *__restrict__ divg,
                               double *__restrict__ cc, double *__restrict__ partials,
                               double *__restrict__ tke_parts, PoisArgs a) {
  __shared__ double sh[kThreads];
  const double coef = s->coef_div, meanQ = s->mean_Q;
  const double OneThird = 1. / 3.;
  double acc = 0, usq = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    double ir = inv_rho[c];
    double lap = (inv_rho[nb.p[0]] - 2 * ir + inv_rho[nb.m[0]]) * g.inv_dx2 +
                 (inv_rho[nb.p[1]] - 2 * ir + inv_rho[nb.m[1]]) * g.inv_dy2 +
                 (inv_rho[nb.p[2]] - 2 * ir + inv_rho[nb.m[2]]) * g.inv_dz2;
    double Qc = a.cooling ? Q[c] - meanQ : Q[c];
    double dv = a.kCp * lap + coef * Qc;
    if (a.store_div) divg[c] = dv;
    double t[3];
    double csum = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double u_lo = Uf[d * g.n + c], u_hi = Uf[d * g.n + nb.p[d]];
      t[d] = (u_hi - u_lo) * (d == 0 ? g.inv_dx : d == 1 ? g.inv_dy : g.inv_dz);
      if (tke_parts) usq += u_lo * u_lo;
      const double half = (Cface[d * g.n + c] + Cface[d * g.n + nb.p[d]]) * 0.5;
      csum = d == 0 ? half : csum + half;
    }
    double rhs = t[0] + t[1] + t[2];
    rhs -= dv;
    rhs *= a.inv_dtpre;
    RHS[c] = rhs;
    acc += rhs;
    double m = OneThird * csum;
    cc[c] = -1. / m;
  }
  double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bs;
  if (tke_parts) {
    double bu = block_sum(usq, sh);
    if (threadIdx.x == 0) tke_parts[blockIdx.x] = bu;
  }
}

// ------------------------------------------------ mixed-path variants
// k_rho_update of the mixed path: the same FP64 update of the density state
// (Rho_np1, Rho_new by FMAs), with the divergence of RU_int and the
// reciprocal 1/Rho_new formed as float-float pairs on the FP32 pipe (each
// within 2^-45 of its value).  1/Rho_new is stored as its pair (inv_rho2, in
// the FP64 path's inv_rho buffer): its one reader, the mixed Poisson
// right-hand side, works in pairs.  FP64 operations per cell: four, against
// twelve in FP64 arithmetic.
__global__ void k_rho_update_mixed(Grid g, const double *__restrict__ RUi,
                                   const double *__restrict__ Rho, const double *__restrict__ np1_in,
                                   double *__restrict__ Rho_np1, double *__restrict__ Rho_new,
                                   float2 *__restrict__ inv_rho2, double *__restrict__ Tgas,
                                   const DevScalars *__restrict__ s, double a_np1, double b_new,
                                   int stage) {
  const double *RUx = RUi, *RUy = RUi + g.n, *RUz = RUi + 2 * g.n;
  const double T_scale = s->T_scale;
  const float2 inv_d[3] = {ff_from_double(g.inv_dx), ff_from_double(g.inv_dy),
                           ff_from_double(g.inv_dz)};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    float2 D = ff_mul(ff_sub(ff_from_double(RUx[at(g, wrap_p(q.i, g.nx), q.j, q.k)]),
                             ff_from_double(RUx[c])),
                      inv_d[0]);
    D = ff_add(D, ff_mul(ff_sub(ff_from_double(RUy[at(g, q.i, wrap_p(q.j, g.ny), q.k)]),
                                ff_from_double(RUy[c])),
                         inv_d[1]));
    D = ff_add(D, ff_mul(ff_sub(ff_from_double(RUz[at(g, q.i, q.j, wrap_p(q.k, g.nz))]),
                                ff_from_double(RUz[c])),
                         inv_d[2]));
    const double Dd = ff_to_double(D);
    double np1 = fma(a_np1, Dd, np1_in[c]);
    double nw = (stage != 3) ? fma(b_new, Dd, Rho[c]) : np1;
    Rho_np1[c] = np1;
    Rho_new[c] = nw;
    const float2 ir = ff_rcp(ff_from_double(nw));
    if (inv_rho2) inv_rho2[c] = ir;  // (the TMA Poisson pass forms it from Rho_new itself)
    Tgas[c] = T_scale * ff_to_double(ir);
  }
}

// Face coefficients of the mixed path, C = 1/Rho_face(Rho_new) on the three
// lower faces of each cell (each face once), as float-float pairs on the FP32
// pipe: 2 / (Rho + Rho_m) from the pair sum of the two densities (within
// 2^-45; an FP32 C would perturb the divergence constraint at 1e-7, which the
// nearly divergence-free right-hand side amplifies in P).  C is stored as a
// double (one FP64 addition per face) and, times 1/d^2, as the pair (Cs2)
// that feeds the refinement's residual; for the PCG operator only also as a
// double C/d^2 (Cs, else null).
__global__ void k_face_coeff_mixed(Grid g, const double *__restrict__ Rho_new,
                                   double *__restrict__ Cface, float2 *__restrict__ Cs2,
                                   double *__restrict__ Cs) {
  const double inv_d2[3] = {g.inv_dx2, g.inv_dy2, g.inv_dz2};
  const float2 inv_d2f[3] = {ff_from_double(g.inv_dx2), ff_from_double(g.inv_dy2),
                             ff_from_double(g.inv_dz2)};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    const float2 r = ff_from_double(Rho_new[c]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float2 h = ff_rcp(ff_add(r, ff_from_double(Rho_new[nb.m[d]])));
      const float2 C = make_float2(2.f * h.x, 2.f * h.y);
      const double clo = ff_to_double(C);
      Cface[d * g.n + c] = clo;
      Cs2[d * g.n + c] = ff_norm(ff_mul(C, inv_d2f[d]));
      if (Cs) Cs[d * g.n + c] = clo * inv_d2[d];
    }
  }
}

// k_poisson_rhs of the mixed path, in float-float pairs (tpm_ff.cuh) on the
// FP32 pipe: every FP64 input is split into a pair by integer operations,
// and the thermal divergence dv = (k/Cp) lap(1/rho) + coef (Q - mean Q) and
// div(RU C) - dv are formed and summed as pairs (the neighbour differences of
// 1/rho and of the face fluxes through the exact-difference subtraction; each
// face's flux is the same pair for both of its cells, so the fluxes still
// telescope).  The pairs carry about 2^-47 of each flux, which leaves the
// projection a divergence error near 1e-12, under the 1e-10 the mixed path
// keeps.  The last factor, 1/(dt pre), is an FP64 product: a right-hand side
// rebuilt from a pair has a fixed pattern in its low bits, which would bias
// the rounding when the refinement splits mean - RHS into pairs again and
// leave its residual a nonzero mean that the iteration cannot remove.  FP64
// operations per cell: four (three more for the kinetic energy sum of the
// last stage) against about twenty-four for the same sums in FP64.  The
// preconditioner scale cc is FP32 (it sets the rate of the Richardson
// iteration, not its fixed point).
// The kernel is z-marching: a block owns a kZX x kZY column of cells and
// walks zlen planes up in z.  Each face's flux pair RU C (and the
// high part of C, for the preconditioner scale) is formed once into shared
// memory and read by the two cells it separates (a per-cell form would form
// every face twice, and split RU and C into pairs twice); the x and y faces
// of the current plane and the z faces of it and the plane above (a ring of
// two) are held.  The mean's partial sums take one slot per block in
// `partials`.
__global__ void __launch_bounds__(kZX * kZY)
k_poisson_rhs_zm(Grid g, const float2 *__restrict__ inv_rho2, const double *__restrict__ Q,
                 const double *__restrict__ RUn, const double *__restrict__ Cface,
                 const DevScalars *__restrict__ s, double *__restrict__ RHS,
                 double *__restrict__ divg, float *__restrict__ cc32, double *__restrict__ cc,
                 double *__restrict__ partials, double *__restrict__ tke_parts, PoisArgs a,
                 int zlen) {
  constexpr int kNX = (kZX + 1) * kZY, kNY = kZX * (kZY + 1), kNZ = kZX * kZY;
  __shared__ float2 fx[kNX], fy[kNY], fz[2][kNZ];  // face fluxes: x, y of plane k; z ring
  __shared__ float cx[kNX], cy[kNY], cz[2][kNZ];  // high parts of the face C
  __shared__ double sh[32];
  const int tx = threadIdx.x % kZX, ty = threadIdx.x / kZX;
  const int tilesx = (g.nx + kZX - 1) / kZX, tilesy = (g.ny + kZY - 1) / kZY;
  const int bx = blockIdx.x % tilesx, by = (blockIdx.x / tilesx) % tilesy;
  const int bz = blockIdx.x / (tilesx * tilesy);
  const int i0 = bx * kZX, j0 = by * kZY, k0 = bz * zlen;
  const int k1 = min(k0 + zlen, g.nz);
  const int i = i0 + tx, j = j0 + ty;
  const bool live = i < g.nx && j < g.ny;
  const float2 coef = ff_from_double(s->coef_div), meanQ = ff_from_double(s->mean_Q);
  const float2 kCp = ff_from_double(a.kCp);
  const float2 inv_d2[3] = {ff_from_double(g.inv_dx2), ff_from_double(g.inv_dy2),
                            ff_from_double(g.inv_dz2)};
  const float2 inv_d[3] = {ff_from_double(g.inv_dx), ff_from_double(g.inv_dy),
                           ff_from_double(g.inv_dz)};
  auto wrapx = [&](int v) { return v >= g.nx ? v - g.nx : v; };
  auto wrapy = [&](int v) { return v >= g.ny ? v - g.ny : v; };
  // the flux pair and C's high part of face d of cell (ii, jj, kk) (wrapped)
  auto face = [&](int d, int ii, int jj, int kk, float2 &u, float &ch) {
    const long long c = at(g, ii, jj, kk);
    const float2 cp = ff_from_double(Cface[d * g.n + c]);
    u = ff_norm(ff_mul(ff_from_double(RUn[d * g.n + c]), cp));
    ch = cp.x;
  };
  // z faces of plane kk into ring slot `slot`
  auto zfaces = [&](int kk, int slot) {
    if (kk >= g.nz) kk -= g.nz;
    for (int e = threadIdx.x; e < kNZ; e += kZX * kZY) {
      const int ey = e / kZX, ex = e - ey * kZX;
      if (i0 + ex < g.nx && j0 + ey < g.ny) face(2, i0 + ex, j0 + ey, kk, fz[slot][e], cz[slot][e]);
    }
  };
  double acc = 0, usq = 0;
  zfaces(k0, 0);
  int zs = 0;
  for (int k = k0; k < k1; ++k) {
    // x faces (i0 .. i0 + kZX) and y faces (j0 .. j0 + kZY) of plane k, z faces of k + 1
    for (int e = threadIdx.x; e < kNX; e += kZX * kZY) {
      const int ey = e / (kZX + 1), ex = e - ey * (kZX + 1);
      if (i0 + ex <= g.nx && j0 + ey < g.ny) face(0, wrapx(i0 + ex), j0 + ey, k, fx[e], cx[e]);
    }
    for (int e = threadIdx.x; e < kNY; e += kZX * kZY) {
      const int ey = e / kZX, ex = e - ey * kZX;
      if (i0 + ex < g.nx && j0 + ey <= g.ny) face(1, i0 + ex, wrapy(j0 + ey), k, fy[e], cy[e]);
    }
    zfaces(k + 1, zs ^ 1);
    __syncthreads();
    if (live) {
      const long long c = at(g, i, j, k);
      const long long pn[3] = {at(g, wrap_p(i, g.nx), j, k), at(g, i, wrap_p(j, g.ny), k),
                               at(g, i, j, wrap_p(k, g.nz))};
      const long long mn[3] = {at(g, wrap_m(i, g.nx), j, k), at(g, i, wrap_m(j, g.ny), k),
                               at(g, i, j, wrap_m(k, g.nz))};
      const float2 ir = inv_rho2[c];
      float2 lap = make_float2(0.f, 0.f);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float2 sec = ff_add(ff_sub(inv_rho2[pn[d]], ir), ff_sub(inv_rho2[mn[d]], ir));
        lap = ff_add(lap, ff_mul(sec, inv_d2[d]));
      }
      float2 Qc = ff_from_double(Q[c]);
      if (a.cooling) Qc = ff_sub(Qc, meanQ);
      const float2 dv = ff_add(ff_mul(kCp, lap), ff_mul(coef, Qc));
      divg[c] = ff_to_double(dv);
      float2 divu = make_float2(-dv.x, -dv.y);
      float msum = 0.f;
      const int ex = ty * (kZX + 1) + tx, ey = ty * kZX + tx, ez = ty * kZX + tx;
      const float2 ulo[3] = {fx[ex], fy[ey], fz[zs][ez]};
      const float2 uhi[3] = {fx[ex + 1], fy[ey + kZX], fz[zs ^ 1][ez]};
      const float clo[3] = {cx[ex], cy[ey], cz[zs][ez]};
      const float chi[3] = {cx[ex + 1], cy[ey + kZX], cz[zs ^ 1][ez]};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        divu = ff_add(divu, ff_mul(ff_sub(uhi[d], ulo[d]), inv_d[d]));
        msum += (clo[d] + chi[d]) * 0.5f;
        if (tke_parts) {
          const double ul = ff_f2d(ulo[d].x);
          usq = fma(ul, ul, usq);
        }
      }
      const double rhs = ff_to_double(divu) * a.inv_dtpre;
      RHS[c] = rhs;
      acc += rhs;
      const float ccf = -3.0f / msum;
      cc32[c] = ccf;
      if (cc) cc[c] = ff_f2d(ccf);  // the PCG operator's copy
    }
    __syncthreads();  // the faces of plane k are rewritten next
    zs ^= 1;
  }
  double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bs;
  if (tke_parts) {
    double bu = block_sum(usq, sh);
    if (threadIdx.x == 0) tke_parts[blockIdx.x] = bu;
  }
}

// ---------------------------------------------------------------------------
// Mixed path, Solver 0, grids of whole 32 x 8 column tiles: the face
// coefficients (what k_face_coeff_mixed forms from Rho_new) and the Poisson
// right-hand side (k_poisson_rhs_zm) in one z-marching pass whose tiles the
// TMA brings in.  Per plane a block needs Rho_new with a one-cell halo (1/Rho
// for the Laplacian of the thermal divergence, 2/(Rho + Rho_m) for the face
// coefficients), RU_new on its faces and Q: one thread issues the boxes of
// the next plane (cp.async.bulk.tensor, tpm_tma.cuh) into a ring of shared-
// memory slots while the block computes on the current one, so the pass
// waits on no global load.  It reads 40 B per cell (Rho_new, RU_new 3, Q) and
// writes 44 B (RHS, divergence, cc, C/d^2 pairs 3) where the two passes it
// replaces moved 140 B (1/Rho pairs written by the density update and read
// back, C as a double written and read back).  The arithmetic is the
// float-float arithmetic of those kernels: C = 2 rcp(Rho + Rho_m) and 1/Rho as
// pairs, each face's flux RU C formed once and read by its two cells; the
// differences of neighbouring pairs (fluxes, 1/Rho) take one TwoSum on the
// high parts (ff_sub_sloppy, within 2^-46 of the operands: about 1e-12 of the
// divergence, a hundredth of the 1e-10 the projection is held to).
namespace {

struct PrSmem {
  // raw FP64 tiles landed by TMA (byte offsets; every box 128-byte aligned)
  static constexpr int kRhoSlot = (32 + 256 + 32 + 16 + 16) * 8;  // ylo row | 8 rows | yhi row | xlo 8x2 | xhi 8x2
  static constexpr int kRhoMain = 256, kRhoYhi = 2304, kRhoXlo = 2560, kRhoXhi = 2688;
  static constexpr int kRuxSlot = (256 + 16) * 8;  // 8 rows | xhi 8x2
  static constexpr int kRuySlot = (256 + 32) * 8;  // 8 rows | yhi row
  static constexpr int kTile = 256 * 8;            // 8 rows of 32
  static constexpr int oRho = 0;                   // 3 planes
  static constexpr int oRux = oRho + 3 * kRhoSlot;  // 2 planes
  static constexpr int oRuy = oRux + 2 * kRuxSlot;  // 2 planes
  static constexpr int oRuz = oRuy + 2 * kRuySlot;  // 2 planes
  static constexpr int oQ = oRuz + 2 * kTile;       // 2 planes
  // Rho_new and 1/Rho_new as pairs, [10][34] per plane (rows j0-1 .. j0+8,
  // columns i0-1 .. i0+32): Rho of 2 planes, 1/Rho of 3
  static constexpr int kPairPlane = 10 * 34 * 8;
  static constexpr int oRp = oQ + 2 * kTile;
  static constexpr int oIr = oRp + 2 * kPairPlane;
  // flux pairs of the x faces [8][33] and y faces [9][32] of the plane, and
  // the high parts of their C
  static constexpr int oFx = oIr + 3 * kPairPlane;
  static constexpr int oFy = oFx + 264 * 8;
  static constexpr int oCx = oFy + 288 * 8;
  static constexpr int oCy = oCx + 264 * 4;
  static constexpr int oBar = oCy + 288 * 4;  // 2 mbarriers
  static constexpr int oRed = oBar + 16;      // 32 doubles for the block sums
  static constexpr int kBytes = oRed + 32 * 8;
  static constexpr unsigned kStageBytes = kRhoSlot + kRuxSlot + kRuySlot + 2 * kTile;
  static constexpr unsigned kPrologueBytes = 2 * kRhoSlot + kTile;
};
static_assert(PrSmem::oRux % 128 == 0 && PrSmem::oRuy % 128 == 0 && PrSmem::oRuz % 128 == 0 &&
                  PrSmem::oQ % 128 == 0 && PrSmem::kRhoSlot % 128 == 0 &&
                  PrSmem::kRuxSlot % 128 == 0 && PrSmem::kRuySlot % 128 == 0 &&
                  PrSmem::oBar % 8 == 0,
              "TMA destinations must stay 128-byte aligned");

// the tensor maps of one launch: Rho_new and RU_new (as [3 nz][ny][nx]) with
// boxes 32 x 8 (a tile), 32 x 1 (a halo row), 2 x 8 (a halo column pair), Q
// with tile boxes
struct PrMaps {
  CUtensorMap rho_t, rho_r, rho_c, ru_t, ru_r, ru_c, q_t;
};

// C = 1/Rho_face = 2 / (Rho_a + Rho_b) and the flux RU C, as pairs
__device__ __forceinline__ void pr_face(float2 ra, float2 rb, double ru, float2 &flux, float2 &C) {
  const float2 h = ff_rcp(ff_add(ra, rb));
  C = make_float2(2.f * h.x, 2.f * h.y);
  flux = ff_norm(ff_mul(ff_from_double(ru), C));
}

// Thread (tx, ty) owns the cell column (i0 + tx, j0 + ty): it converts that
// cell of each plane to pairs, forms the cell's lower x, y and z faces (the z
// faces of the column stay in its registers from one plane to the next), and
// the right-hand side of the cell; threads 0-79 also convert the tile's halo,
// threads 0-7 form the x faces at i0 + 32 and threads 32-63 the y faces at
// j0 + 8.
__global__ void __launch_bounds__(kZX * kZY)
k_poisson_rhs_tma(Grid g, const __grid_constant__ PrMaps m, DevScalars *__restrict__ s,
                  double *__restrict__ RHS, double *__restrict__ divg, float *__restrict__ cc32,
                  float2 *__restrict__ Cs2, double *__restrict__ partials,
                  double *__restrict__ tke_parts, PoisArgs a, int zlen) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, tx = tid % kZX, ty = tid / kZX;
  const int tilesx = g.nx / kZX, tilesy = g.ny / kZY;
  const int bx = blockIdx.x % tilesx, by = (blockIdx.x / tilesx) % tilesy;
  const int bz = blockIdx.x / (tilesx * tilesy);
  const int i0 = bx * kZX, j0 = by * kZY, k0 = bz * zlen;
  const int k1 = min(k0 + zlen, g.nz);
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + PrSmem::oBar);
  double *red = reinterpret_cast<double *>(sm + PrSmem::oRed);
  if (smem_u32(sm) & 127u) {  // the layout's alignment rests on this: never issue a misaligned box
    if (tid == 0) s->timeout = 1;
    return;
  }
  auto rho_raw = [&](int kk) {
    return sm + PrSmem::oRho + ((kk + 3) % 3) * PrSmem::kRhoSlot;
  };
  auto rux_slot = [&](int kk) { return sm + PrSmem::oRux + (kk & 1) * PrSmem::kRuxSlot; };
  auto ruy_slot = [&](int kk) { return sm + PrSmem::oRuy + (kk & 1) * PrSmem::kRuySlot; };
  auto ruz_slot = [&](int kk) { return sm + PrSmem::oRuz + (kk & 1) * PrSmem::kTile; };
  auto q_slot = [&](int kk) { return sm + PrSmem::oQ + (kk & 1) * PrSmem::kTile; };
  auto rp_plane = [&](int kk) {
    return reinterpret_cast<float2 *>(sm + PrSmem::oRp + ((kk + 2) & 1) * PrSmem::kPairPlane);
  };
  auto ir_plane = [&](int kk) {
    return reinterpret_cast<float2 *>(sm + PrSmem::oIr + ((kk + 3) % 3) * PrSmem::kPairPlane);
  };
  float2 *fx = reinterpret_cast<float2 *>(sm + PrSmem::oFx);
  float2 *fy = reinterpret_cast<float2 *>(sm + PrSmem::oFy);
  float *cxh = reinterpret_cast<float *>(sm + PrSmem::oCx);
  float *cyh = reinterpret_cast<float *>(sm + PrSmem::oCy);
  const int jlo = j0 == 0 ? g.ny - 1 : j0 - 1, jhi = j0 + kZY == g.ny ? 0 : j0 + kZY;
  const int ilo = i0 == 0 ? g.nx - 2 : i0 - 2, ihi = i0 + kZX == g.nx ? 0 : i0 + kZX;
  auto wz = [&](int kk) { return kk < 0 ? kk + g.nz : (kk >= g.nz ? kk - g.nz : kk); };
  // the boxes of Rho_new plane kk (with its halo) into its raw slot
  auto load_rho = [&](int kk, uint64_t *b) {
    unsigned char *d = rho_raw(kk);
    const int z = wz(kk);
    tma_load_3d(d + PrSmem::kRhoMain, &m.rho_t, b, i0, j0, z);
    tma_load_3d(d, &m.rho_r, b, i0, jlo, z);
    tma_load_3d(d + PrSmem::kRhoYhi, &m.rho_r, b, i0, jhi, z);
    tma_load_3d(d + PrSmem::kRhoXlo, &m.rho_c, b, ilo, j0, z);
    tma_load_3d(d + PrSmem::kRhoXhi, &m.rho_c, b, ihi, j0, z);
  };
  // stage kk: Rho plane kk + 1, RU_new x and y faces and Q of plane kk, the z
  // faces of plane kk + 1
  auto load_stage = [&](int kk, uint64_t *b) {
    mbar_arrive_expect_tx(b, PrSmem::kStageBytes);
    load_rho(kk + 1, b);
    tma_load_3d(rux_slot(kk), &m.ru_t, b, i0, j0, kk);
    tma_load_3d(rux_slot(kk) + 2048, &m.ru_c, b, ihi, j0, kk);
    tma_load_3d(ruy_slot(kk), &m.ru_t, b, i0, j0, g.nz + kk);
    tma_load_3d(ruy_slot(kk) + 2048, &m.ru_r, b, i0, jhi, g.nz + kk);
    tma_load_3d(ruz_slot(kk + 1), &m.ru_t, b, i0, j0, 2 * g.nz + wz(kk + 1));
    tma_load_3d(q_slot(kk), &m.q_t, b, i0, j0, kk);
  };
  // waits for stage r (the prologue is stage 0, plane kk is stage kk - k0 + 1)
  bool ok = true;
  auto wait_stage = [&](int r) {
    if (!mbar_wait(&bar[r & 1], (unsigned)(r >> 1) & 1u)) {
      ok = false;
      s->timeout = 1;
    }
  };
  // this thread's part of the halo of a plane: raw index and pair index
  int h_raw = -1, h_at = 0;
  if (tid < 32) {
    h_raw = tid;  // row j0 - 1
    h_at = tid + 1;
  } else if (tid < 64) {
    h_raw = 288 + tid - 32;  // row j0 + 8
    h_at = 9 * 34 + tid - 32 + 1;
  } else if (tid < 72) {
    h_raw = 320 + 2 * (tid - 64) + 1;  // column i0 - 1: the second of the pair
    h_at = (tid - 64 + 1) * 34;
  } else if (tid < 80) {
    h_raw = 336 + 2 * (tid - 72);  // column i0 + 32: the first of the pair
    h_at = (tid - 72 + 1) * 34 + 33;
  }
  const int own = (ty + 1) * 34 + tx + 1;  // the owned cell in a pair plane
  // Rho and 1/Rho pairs of plane kk (the owned cell and the halo part)
  auto convert = [&](int kk) {
    const double *d = reinterpret_cast<const double *>(rho_raw(kk));
    float2 *rp = rp_plane(kk), *ir = ir_plane(kk);
    const float2 v = ff_from_double(d[32 + tid]);
    rp[own] = v;
    ir[own] = ff_rcp(v);
    if (h_raw >= 0) {
      const float2 w = ff_from_double(d[h_raw]);
      rp[h_at] = w;
      ir[h_at] = ff_rcp(w);
    }
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    tma_prefetch_map(&m.rho_t);
    tma_prefetch_map(&m.ru_t);
  }
  __syncthreads();
  if (tid == 0) {  // prologue: Rho planes k0 - 1, k0 and the z faces of plane k0; then stage k0
    mbar_arrive_expect_tx(&bar[0], PrSmem::kPrologueBytes);
    load_rho(k0 - 1, &bar[0]);
    load_rho(k0, &bar[0]);
    tma_load_3d(ruz_slot(k0), &m.ru_t, &bar[0], i0, j0, 2 * g.nz + k0);
    load_stage(k0, &bar[1]);
  }
  const float2 coef = ff_from_double(s->coef_div), meanQ = ff_from_double(s->mean_Q);
  const float2 kCp = ff_from_double(a.kCp);
  const float2 inv_d2[3] = {ff_from_double(g.inv_dx2), ff_from_double(g.inv_dy2),
                            ff_from_double(g.inv_dz2)};
  const float2 inv_d[3] = {ff_from_double(g.inv_dx), ff_from_double(g.inv_dy),
                           ff_from_double(g.inv_dz)};
  double acc = 0, usq = 0;
  int issued = 1;  // stages issued so far: the prologue (0) and stage 1
  float2 fz_lo = make_float2(0.f, 0.f), cz_lo = fz_lo;  // the column's lower z face
  wait_stage(0);
  ok = __syncthreads_and(ok) != 0;  // every thread takes the same branch
  if (ok) {
    convert(k0 - 1);
    convert(k0);
    pr_face(rp_plane(k0)[own], rp_plane(k0 - 1)[own],
            reinterpret_cast<const double *>(ruz_slot(k0))[tid], fz_lo, cz_lo);
  }
  __syncthreads();
  for (int k = k0; k < k1 && ok; ++k) {
    const int r = k - k0 + 1;
    if (k + 1 < k1) {
      if (tid == 0) {
        fence_proxy_async();  // the reads of the slots being refilled came before
        load_stage(k + 1, &bar[(r + 1) & 1]);
      }
      issued = r + 1;
    }
    wait_stage(r);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    convert(k + 1);
    // faces: lower x, y of the owned cell in plane k, lower z of plane k + 1
    const float2 *rk = rp_plane(k);
    float2 cx_lo, cy_lo, fz_hi, cz_hi;
    {
      float2 f;
      pr_face(rk[own], rk[own - 1], reinterpret_cast<const double *>(rux_slot(k))[tid], f, cx_lo);
      fx[ty * 33 + tx] = f;
      cxh[ty * 33 + tx] = cx_lo.x;
      pr_face(rk[own], rk[own - 34], reinterpret_cast<const double *>(ruy_slot(k))[tid], f, cy_lo);
      fy[tid] = f;
      cyh[tid] = cy_lo.x;
      pr_face(rp_plane(k + 1)[own], rk[own],
              reinterpret_cast<const double *>(ruz_slot(k + 1))[tid], fz_hi, cz_hi);
      float2 C;
      if (tid < 8) {  // x face at i0 + 32 of row tid
        const int o = (tid + 1) * 34 + 33;
        pr_face(rk[o], rk[o - 1], reinterpret_cast<const double *>(rux_slot(k))[256 + 2 * tid],
                f, C);
        fx[tid * 33 + 32] = f;
        cxh[tid * 33 + 32] = C.x;
      } else if (tid >= 32 && tid < 64) {  // y face at j0 + 8 of column tid - 32
        const int o = 9 * 34 + tid - 32 + 1;
        pr_face(rk[o], rk[o - 34], reinterpret_cast<const double *>(ruy_slot(k))[256 + tid - 32],
                f, C);
        fy[256 + tid - 32] = f;
        cyh[256 + tid - 32] = C.x;
      }
    }
    __syncthreads();
    {
      const int i = i0 + tx, j = j0 + ty;
      const long long c = at(g, i, j, k);
      const float2 *irk = ir_plane(k);
      const float2 ir = irk[own];
      const float2 pn[3] = {irk[own + 1], irk[own + 34], ir_plane(k + 1)[own]};
      const float2 mn[3] = {irk[own - 1], irk[own - 34], ir_plane(k - 1)[own]};
      float2 lap = make_float2(0.f, 0.f);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float2 sec = ff_add(ff_sub_sloppy(pn[d], ir), ff_sub_sloppy(mn[d], ir));
        lap = ff_add(lap, ff_mul(sec, inv_d2[d]));
      }
      float2 Qc = ff_from_double(reinterpret_cast<const double *>(q_slot(k))[tid]);
      if (a.cooling) Qc = ff_sub(Qc, meanQ);
      const float2 dv = ff_add(ff_mul(kCp, lap), ff_mul(coef, Qc));
      if (a.store_div) divg[c] = ff_to_double(dv);
      float2 divu = make_float2(-dv.x, -dv.y);
      const int ex = ty * (kZX + 1) + tx;
      const float2 ulo[3] = {fx[ex], fy[tid], fz_lo};
      const float2 uhi[3] = {fx[ex + 1], fy[tid + kZX], fz_hi};
      const float2 clo[3] = {cx_lo, cy_lo, cz_lo};
      const float chi[3] = {cxh[ex + 1], cyh[tid + kZX], cz_hi.x};
      float msum = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        divu = ff_add(divu, ff_mul(ff_sub_sloppy(uhi[d], ulo[d]), inv_d[d]));
        msum += (clo[d].x + chi[d]) * 0.5f;
        if (tke_parts) {
          const double ul = ff_f2d(ulo[d].x);
          usq = fma(ul, ul, usq);
        }
        Cs2[d * g.n + c] = ff_norm(ff_mul(clo[d], inv_d2[d]));
      }
      const double rhs = ff_to_double(divu) * a.inv_dtpre;
      RHS[c] = rhs;
      acc += rhs;
      cc32[c] = -3.0f / msum;
    }
    fz_lo = fz_hi;
    cz_lo = cz_hi;
    __syncthreads();  // the slots, pair planes and faces of plane k are refilled next
  }
  if (!ok && tid == 0) {
    // a wait gave up: let the copies of the last two stages issued land
    // (again bounded) before the block's shared memory is released
    for (int r = issued > 0 ? issued - 1 : 0; r <= issued; ++r)
      mbar_wait(&bar[r & 1], (unsigned)(r >> 1) & 1u);
  }
  __syncthreads();
  double bs = block_sum(acc, red);
  if (tid == 0) partials[blockIdx.x] = bs;
  if (tke_parts) {
    double bu = block_sum(usq, red);
    if (tid == 0) tke_parts[blockIdx.x] = bu;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Mixed path, grids of whole 32 x 8 column tiles: grid::Update_Rho
// (grid.cpp:608-614) and the face velocity U = RU_int / Rho_face(Rho_int)
// that Update_Particle forms first (grid.cpp:868) in one z-marching pass fed
// by the TMA.  Both read RU_int: the two kernels this replaces
// (k_rho_update_mixed, k_face_velocity_mixed) read it twice (in FP64 and as
// its FP32 copy, which equals its truncation ff_hi) and gather the
// neighbours of every cell with scattered loads.  Per plane k a block needs
// RU_int's x component with the column pair at i0 + 32, its y component with
// the row at j0 + 8, its z component of plane k + 1 (plane k's stays in the
// thread's registers), and Rho_int with the row at j0 - 1 and the column pair
// at i0 - 2 (plane k - 1's stays in registers); Rho and the RK input of
// Rho_np1 are plain coalesced loads issued before the wait.  One thread
// issues the next plane's boxes into the other of two slots while the block
// computes.  The arithmetic is the two kernels' except for the differences
// of neighbouring RU_int pairs, which take one TwoSum on the high parts
// (ff_sub_sloppy: within 2^-46 of the operands, about 1e-15 of Rho per
// stage, far below the FP32 parts of the mixed step) instead of two.
namespace {

struct RfSmem {
  // one slot (bytes; every box 128-byte aligned): RU_int x tile [8][32] |
  // x column pair [8][2] at i0 + 32 | y tile | y row [32] at j0 + 8 | z tile of
  // plane k + 1 | Rho_int row [32] at j0 - 1 | Rho_int tile | column pair
  // [8][2] at i0 - 2
  static constexpr int kRuxXhi = 2048;
  static constexpr int kRuy = kRuxXhi + 128;
  static constexpr int kRuyYhi = kRuy + 2048;
  static constexpr int kRuz = kRuyYhi + 256;
  static constexpr int kRhoYlo = kRuz + 2048;
  static constexpr int kRho = kRhoYlo + 256;
  static constexpr int kRhoXlo = kRho + 2048;
  static constexpr int kSlot = kRhoXlo + 128;  // the bytes of one stage's boxes
  static constexpr int oBar = 2 * kSlot;
  static constexpr int kBytes = oBar + 16;
};
static_assert(RfSmem::kRuy % 128 == 0 && RfSmem::kRuyYhi % 128 == 0 && RfSmem::kRuz % 128 == 0 &&
                  RfSmem::kRhoYlo % 128 == 0 && RfSmem::kRho % 128 == 0 &&
                  RfSmem::kRhoXlo % 128 == 0 && RfSmem::kSlot % 128 == 0,
              "TMA destinations must stay 128-byte aligned");

// RU_int (as [3 nz][ny][nx]) and Rho_int: tile, row and column-pair boxes
struct RfMaps {
  CUtensorMap ru_t, ru_r, ru_c, rho_t, rho_r, rho_c;
};

__global__ void __launch_bounds__(kZX * kZY)
k_rho_face_tma(Grid g, const __grid_constant__ RfMaps m, DevScalars *__restrict__ s,
               const double *__restrict__ RUi, const double *__restrict__ Rho_int,
               const double *__restrict__ Rho, const double *__restrict__ np1_in,
               double *__restrict__ Rho_np1, double *__restrict__ Rho_new,
               double *__restrict__ Tgas, float *__restrict__ U, double a_np1, double b_new,
               int stage, int zlen) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, tx = tid % kZX, ty = tid / kZX;
  const int tilesx = g.nx / kZX, tilesy = g.ny / kZY;
  const int bx = blockIdx.x % tilesx, by = (blockIdx.x / tilesx) % tilesy;
  const int bz = blockIdx.x / (tilesx * tilesy);
  const int i0 = bx * kZX, j0 = by * kZY, k0 = bz * zlen;
  const int nplanes = min(k0 + zlen, g.nz) - k0;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + RfSmem::oBar);
  if (smem_u32(sm) & 127u) {  // never issue a box to a misaligned address
    if (tid == 0) s->timeout = 1;
    return;
  }
  const int jlo = j0 == 0 ? g.ny - 1 : j0 - 1, jhi = j0 + kZY == g.ny ? 0 : j0 + kZY;
  const int ilo = i0 == 0 ? g.nx - 2 : i0 - 2, ihi = i0 + kZX == g.nx ? 0 : i0 + kZX;
  auto slot = [&](int r) { return sm + (r & 1) * RfSmem::kSlot; };
  // the boxes of plane k0 + r into slot r & 1, counted on bar[r & 1]
  auto load_stage = [&](int r) {
    uint64_t *b = &bar[r & 1];
    unsigned char *d = slot(r);
    const int k = k0 + r, kp = k + 1 == g.nz ? 0 : k + 1;
    mbar_arrive_expect_tx(b, RfSmem::kSlot);
    tma_load_3d(d, &m.ru_t, b, i0, j0, k);
    tma_load_3d(d + RfSmem::kRuxXhi, &m.ru_c, b, ihi, j0, k);
    tma_load_3d(d + RfSmem::kRuy, &m.ru_t, b, i0, j0, g.nz + k);
    tma_load_3d(d + RfSmem::kRuyYhi, &m.ru_r, b, i0, jhi, g.nz + k);
    tma_load_3d(d + RfSmem::kRuz, &m.ru_t, b, i0, j0, 2 * g.nz + kp);
    tma_load_3d(d + RfSmem::kRhoYlo, &m.rho_r, b, i0, jlo, k);
    tma_load_3d(d + RfSmem::kRho, &m.rho_t, b, i0, j0, k);
    tma_load_3d(d + RfSmem::kRhoXlo, &m.rho_c, b, ilo, j0, k);
  };
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
    tma_prefetch_map(&m.ru_t);
    tma_prefetch_map(&m.rho_t);
  }
  __syncthreads();
  if (tid == 0 && nplanes > 0) load_stage(0);
  const int i = i0 + tx, j = j0 + ty;
  // the column's RU_int z component at plane k0 (as its pair) and Rho_int at
  // plane k0 - 1 (truncated): carried from one plane to the next
  float2 pz_c = ff_from_double(nplanes > 0 ? RUi[2 * g.n + at(g, i, j, k0)] : 0.0);
  float rho_zm = ff_hi(nplanes > 0 ? Rho_int[at(g, i, j, k0 == 0 ? g.nz - 1 : k0 - 1)] : 0.0);
  const double T_scale = s->T_scale;
  const float2 inv_d[3] = {ff_from_double(g.inv_dx), ff_from_double(g.inv_dy),
                           ff_from_double(g.inv_dz)};
  bool ok = true;
  int issued = 0;  // the last stage issued
  for (int r = 0; r < nplanes; ++r) {
    const int k = k0 + r;
    if (r + 1 < nplanes) {
      if (tid == 0) {
        fence_proxy_async();  // the reads of the slot being refilled came before
        load_stage(r + 1);
      }
      issued = r + 1;
    }
    const long long c = at(g, i, j, k);
    const double rho_b = Rho[c], np1_b = np1_in[c];
    ok = mbar_wait(&bar[r & 1], (unsigned)(r >> 1) & 1u);
    if (!ok) s->timeout = 1;
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    const unsigned char *d = slot(r);
    const double *rux = reinterpret_cast<const double *>(d);
    const double *ruy = reinterpret_cast<const double *>(d + RfSmem::kRuy);
    const double *rho = reinterpret_cast<const double *>(d + RfSmem::kRho);
    const double rux_c = rux[tid];
    const double rux_p =
        tx < kZX - 1 ? rux[tid + 1] : reinterpret_cast<const double *>(d + RfSmem::kRuxXhi)[2 * ty];
    const double ruy_c = ruy[tid];
    const double ruy_p =
        ty < kZY - 1 ? ruy[tid + kZX] : reinterpret_cast<const double *>(d + RfSmem::kRuyYhi)[tx];
    const float2 pz_p = ff_from_double(reinterpret_cast<const double *>(d + RfSmem::kRuz)[tid]);
    // Update_Rho: the divergence of RU_int as a pair, the FP64 state update
    const float2 px_c = ff_from_double(rux_c), py_c = ff_from_double(ruy_c);
    float2 D = ff_mul(ff_sub_sloppy(ff_from_double(rux_p), px_c), inv_d[0]);
    D = ff_add(D, ff_mul(ff_sub_sloppy(ff_from_double(ruy_p), py_c), inv_d[1]));
    D = ff_add(D, ff_mul(ff_sub_sloppy(pz_p, pz_c), inv_d[2]));
    const double Dd = ff_to_double(D);
    const double np1 = fma(a_np1, Dd, np1_b);
    const double nw = (stage != 3) ? fma(b_new, Dd, rho_b) : np1;
    Rho_np1[c] = np1;
    Rho_new[c] = nw;
    Tgas[c] = T_scale * ff_to_double(ff_rcp(ff_from_double(nw)));
    // the face velocity in FP32 from the truncated RU_int (the high parts of
    // its pairs) and Rho_int
    const double rho_xm =
        tx > 0 ? rho[tid - 1] : reinterpret_cast<const double *>(d + RfSmem::kRhoXlo)[2 * ty + 1];
    const double rho_ym =
        ty > 0 ? rho[tid - kZX] : reinterpret_cast<const double *>(d + RfSmem::kRhoYlo)[tx];
    const float rf = ff_hi(rho[tid]);
    U[c] = px_c.x / ((rf + ff_hi(rho_xm)) * 0.5f);
    U[g.n + c] = py_c.x / ((rf + ff_hi(rho_ym)) * 0.5f);
    U[2 * g.n + c] = pz_c.x / ((rf + rho_zm) * 0.5f);
    pz_c = pz_p;
    rho_zm = rf;
    __syncthreads();  // slot r & 1 is refilled by stage r + 2
  }
  if (!ok && tid == 0) {
    // a wait gave up: let the copies issued land (again bounded) before the
    // block's shared memory is released
    for (int r = issued > 0 ? issued - 1 : 0; r <= issued; ++r)
      mbar_wait(&bar[r & 1], (unsigned)(r >> 1) & 1u);
  }
}

}  // namespace

// face velocity of the mixed path: only the FP32 stencil and the particle
// gather read it, so it is formed in FP32
__global__ void k_face_velocity_mixed(Grid g, const float *__restrict__ RUi32,
                                      const double *__restrict__ Rho_int, float *__restrict__ U) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    // the face density in FP32 (it only divides the FP32 momentum copy)
    const float r = ff_hi(Rho_int[c]);
    U[c] = RUi32[c] / ((r + ff_hi(Rho_int[at(g, wrap_m(q.i, g.nx), q.j, q.k)])) * 0.5f);
    U[g.n + c] = RUi32[g.n + c] / ((r + ff_hi(Rho_int[at(g, q.i, wrap_m(q.j, g.ny), q.k)])) * 0.5f);
    U[2 * g.n + c] =
        RUi32[2 * g.n + c] / ((r + ff_hi(Rho_int[at(g, q.i, q.j, wrap_m(q.k, g.nz))])) * 0.5f);
  }
}

// FP32 copies of FP64 fields for the mixed path's stencils (truncated, by
// integer operations)
__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = ff_hi(a[i]);
}

__global__ void k_to_double(const float *__restrict__ a, double *__restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// mean of a field from per-block partial sums, stored at *out
__global__ void k_finish_mean(const double *__restrict__ partials, int nparts, long long ntot,
                              double *out) {
  __shared__ double sh[kThreads];
  double v = 0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += partials[b];
  double sum = block_sum(v, sh);
  if (threadIdx.x == 0) *out = sum / (double)ntot;
}

// -------------------------------------------------------- passive scalar
// grid::Update_Passive_Scalar (grid.cpp:743-772) at one cell: with U the face
// velocity RU_int/Rho_face (TU: FP32 copy on the mixed path),
//   RHS = D_M Del2(PS_int) + (-1) div_F2C(U * PS_face) + source,
// source = S1 - mean(S1) (S1_type 0, scalar_source.h) or (-1) Ix_F2C(U.x);
//   PS_np1 += (dt*post) RHS,  PS_new = 1*PS + (dt*pre) RHS  (stage 3: PS_np1).
struct PsArgs {
  double D_M, dtpo, dtpr;
  int stage, s1_type;
};

template <typename TU>
__global__ void k_passive_scalar(Grid g, const TU *__restrict__ U, const double *__restrict__ PSf,
                                 const double *__restrict__ PSi, const double *__restrict__ PS,
                                 const double *__restrict__ PSnp1_in, double *__restrict__ PSnp1,
                                 double *__restrict__ PSnew, const double *__restrict__ S1,
                                 PsArgs a) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    const TU *Ux = U, *Uy = U + g.n, *Uz = U + 2 * g.n;
    const double *Fx = PSf, *Fy = PSf + g.n, *Fz = PSf + 2 * g.n;
    // dummy = U * PS_face; div_F2C(dummy) (tensor0.cpp:249-256)
    const double conv = ((double)Ux[nb.p[0]] * Fx[nb.p[0]] - (double)Ux[c] * Fx[c]) * g.inv_dx +
                        ((double)Uy[nb.p[1]] * Fy[nb.p[1]] - (double)Uy[c] * Fy[c]) * g.inv_dy +
                        ((double)Uz[nb.p[2]] * Fz[nb.p[2]] - (double)Uz[c] * Fz[c]) * g.inv_dz;
    const double pc = PSi[c];
    const double lap = (PSi[nb.p[0]] - 2 * pc + PSi[nb.m[0]]) * g.inv_dx2 +
                       (PSi[nb.p[1]] - 2 * pc + PSi[nb.m[1]]) * g.inv_dy2 +
                       (PSi[nb.p[2]] - 2 * pc + PSi[nb.m[2]]) * g.inv_dz2;
    double rhs = a.D_M * lap + -1 * conv;
    if (a.s1_type == 0)
      rhs += S1[c];
    else
      rhs += -1 * (((double)Ux[c] + (double)Ux[nb.p[0]]) * 0.5);
    const double np1 = PSnp1_in[c] + a.dtpo * rhs;
    PSnp1[c] = np1;
    PSnew[c] = a.stage != 3 ? 1 * PS[c] + a.dtpr * rhs : np1;
  }
}

// Passive_Scalar_face = I_C2F(src) (tensor1.cpp:278-283, tensor0.cpp:283-296)
__global__ void k_ps_face(Grid g, const double *__restrict__ src, double *__restrict__ F) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    const double v = src[c];
    F[c] = (v + src[nb.m[0]]) * 0.5;
    F[g.n + c] = (v + src[nb.m[1]]) * 0.5;
    F[2 * g.n + c] = (v + src[nb.m[2]]) * 0.5;
  }
}

// ---------------------------------------------------------- projection
// grid::Update_RU_WP, grid.cpp:857-863.  At the last stage (kSum) the
// per-component sums of RU_np1 for make_mean_U0 (simulation.cpp:80) are
// reduced too.  kFma (mixed path): the updates as FMAs
template <bool kFma, bool kSum>
__global__ void k_project(Grid g, const double *__restrict__ P, double *__restrict__ RU_np1,
                          double *__restrict__ RU_new, double a_np1, double b_new, int stage,
                          double *__restrict__ partials, float *__restrict__ RUn32) {
  __shared__ double sh[kThreads];
  double acc[3] = {0, 0, 0};
  const double inv_d[3] = {g.inv_dx, g.inv_dy, g.inv_dz};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    double pc = P[c];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      // mixed path: the pressure difference times the folded constants
      // a/d, b/d (one FP64 product fewer per face; no bitwise parity there)
      const double dp = pc - P[nb.m[d]];
      const double G = kFma ? dp : dp * inv_d[d];
      const double ca = kFma ? a_np1 * inv_d[d] : a_np1, cb = kFma ? b_new * inv_d[d] : b_new;
      double np1 = kFma ? fma(ca, G, RU_np1[d * g.n + c]) : RU_np1[d * g.n + c] + ca * G;
      RU_np1[d * g.n + c] = np1;
      const double nw = (stage != 3) ? (kFma ? fma(cb, G, RU_new[d * g.n + c])
                                             : RU_new[d * g.n + c] + cb * G)
                                     : np1;
      RU_new[d * g.n + c] = nw;
      if (RUn32) RUn32[d * g.n + c] = ff_hi(nw);
      if (kSum) acc[d] += np1;
    }
  }
  if (kSum) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double bs = block_sum(acc[d], sh);
      if (threadIdx.x == 0) partials[d * kRedBlocks + blockIdx.x] = bs;
    }
  }
}

__global__ void k_finish_means3(const double *__restrict__ partials, int nparts, long long ntot,
                                DevScalars *s) {
  __shared__ double sh[kThreads];
  for (int d = 0; d < 3; ++d) {
    double v = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += partials[d * kRedBlocks + b];
    double sum = block_sum(v, sh);
    if (threadIdx.x == 0) s->mean_ru[d] = sum / (double)ntot;
    __syncthreads();
  }
}

// Post-projection divergence residual of the mixed path:
// res = div_F2C(RU_new * C) - divergence - dt*pre*mean(RHS_Pois), with
// C = 1/Rho_face(Rho_new).  A converged projection gives res = 0
// (grid.cpp:841-863): div u_new = divergence + dt*pre*mean.  Formed to FP64
// accuracy in float-float pairs on the FP32 pipe: the face
// coefficients of this stage are the pairs C/d^2 the Poisson right-hand side
// pass wrote (Cs2, formed from this stage's Rho_new), so
// div(RU C) = sum_d d (RU_p Cs2_p - RU_c Cs2_c); each flux pair carries about
// 2^-46 of its value, far below the 1e-10 the residual is held to.  Two FP64
// operations per cell (the constraint and its mean offset) instead of the
// FP64 fluxes.
__global__ void k_div_residual(Grid g, const double *__restrict__ RUn,
                               const float2 *__restrict__ Cs2,
                               const double *__restrict__ divg, const DevScalars *__restrict__ s,
                               double dtpre, double *__restrict__ partials) {
  __shared__ double sh[kThreads];
  const double off = dtpre * s->mean_rhs;
  const float2 dd[3] = {ff_from_double(g.dx), ff_from_double(g.dy), ff_from_double(g.dz)};
  double mx = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    float2 dv = ff_from_double(-(divg[c] + off));
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double *R = RUn + d * g.n;
      const float2 *C = Cs2 + d * g.n;
      const float2 fp = ff_mul(ff_from_double(R[nb.p[d]]), C[nb.p[d]]);
      const float2 fc = ff_mul(ff_from_double(R[c]), C[c]);
      dv = ff_add(dv, ff_mul(ff_sub(ff_norm(fp), ff_norm(fc)), dd[d]));
    }
    const double r = fabs(ff_to_double(dv));
    mx = r > mx ? r : mx;
  }
  double b = block_max(mx, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

__global__ void k_finish_max_div(const double *__restrict__ partials, int nparts, DevScalars *s) {
  __shared__ double sh[kThreads];
  double v = 0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) v = partials[b] > v ? partials[b] : v;
  double m = block_max(v, sh);
  if (threadIdx.x == 0) s->max_div = m;
}

// tensor0::make_mean_U0 per component (tensor0.cpp:389-394) and
// grid::TimeAdvance RU = RU_np1 (grid.cpp:599): the result goes to RU.
__global__ void k_mean_reset(Grid g, const double *__restrict__ RU_np1, double *__restrict__ RU,
                             const DevScalars *__restrict__ s, double r0, double r1, double r2) {
  const double m[3] = {s->mean_ru[0], s->mean_ru[1], s->mean_ru[2]};
  const double a[3] = {r0, r1, r2};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double v = RU_np1[d * g.n + c];
      v -= m[d];
      v += a[d];
      RU[d * g.n + c] = v;
    }
  }
}

// grid::Initialize (grid.cpp:474): nothing to store on the device beyond the
// copies done by the host; kept for the operator-level Poisson entry point:
// center_coeff = -1/I_F2C(C) for a caller-supplied C (poisson.cpp:393-394).
// Cs_d = C_d / d^2 for caller-supplied face coefficients (operator-level
// solve), as a double and a float-float pair, and cc in FP32
__global__ void k_scale_faces(Grid g, const double *__restrict__ Cf, const double *__restrict__ cc,
                              double *__restrict__ Cs, float2 *__restrict__ Cs2,
                              float *__restrict__ cc32) {
  const double inv_d2[3] = {g.inv_dx2, g.inv_dy2, g.inv_dz2};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double cs = Cf[d * g.n + c] * inv_d2[d];
      Cs[d * g.n + c] = cs;
      Cs2[d * g.n + c] = ff_from_double(cs);
    }
    cc32[c] = (float)cc[c];
  }
}

__global__ void k_center_coeff(Grid g, const double *__restrict__ Cf, double *__restrict__ cc) {
  const double OneThird = 1. / 3.;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    Cell q = cell_of(g, c);
    Nbr nb = nbr_of(g, q);
    double m = OneThird * ((Cf[c] + Cf[nb.p[0]]) * 0.5 + (Cf[g.n + c] + Cf[g.n + nb.p[1]]) * 0.5 +
                           (Cf[2 * g.n + c] + Cf[2 * g.n + nb.p[2]]) * 0.5);
    cc[c] = -1. / m;
  }
}

}  // namespace

int cell_blocks(const Grid &g) {
  long long b = (g.n + kThreads - 1) / kThreads;
  return (int)(b < kRedBlocks ? b : kRedBlocks);
}

int wave_blocks(tpm_ctx *c, const void *kernel, int threads, long long items, bool reduces) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> occ;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = occ.find({kernel, threads});
    if (it != occ.end()) {
      per_sm = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) !=
              cudaSuccess ||
          per_sm < 1)
        per_sm = 1;
      occ[{kernel, threads}] = per_sm;
    }
  }
  const long long sms = c->sms > 0 ? c->sms : 1;
  long long b = sms * per_sm;
  if (reduces && b > kRedBlocks) b = sms <= kRedBlocks ? (kRedBlocks / sms) * sms : kRedBlocks;
  const long long need = (items + threads - 1) / threads;
  if (need < b) b = need > 0 ? need : 1;
  return (int)b;
}

// blocks of the z-marching kernels (column tiles x z chunks)
// planes per z chunk: 16 where the grid gives four blocks per SM with them,
// fewer (at least 4) on small grids so that every SM still gets work
int zm_zlen(const tpm_ctx *c) {
  const Grid &g = c->g;
  const long long cols = (long long)((g.nx + kZX - 1) / kZX) * ((g.ny + kZY - 1) / kZY);
  const long long want = 4LL * (c->sms > 0 ? c->sms : 1);  // blocks
  long long z = cols * g.nz / want;
  z = z > 16 ? 16 : (z < 4 ? 4 : z);
  return (int)z;
}

int zm_blocks(const tpm_ctx *c) {
  const Grid &g = c->g;
  const int z = zm_zlen(c);
  return ((g.nx + kZX - 1) / kZX) * ((g.ny + kZY - 1) / kZY) * ((g.nz + z - 1) / z);
}

namespace {
// wave_blocks for a cell kernel of this file (kThreads per block unless
// given)
template <typename K>
int cell_waves(tpm_ctx *c, K *kernel, bool reduces, int threads = kThreads) {
  return wave_blocks(c, reinterpret_cast<const void *>(kernel), threads, c->g.n, reduces);
}

}  // namespace

static const double kPre[4] = {0.5, 0.5, 1., 1. / 6.};          // grid.cpp:18-21
static const double kPost[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};  // grid.cpp:22-25

void launch_p0_update(tpm_ctx *c, int s) {
  TPM_LAUNCH(c, "p0_update", k_p0_update, 1, kThreads, 0, c->partials + kPartQ * kRedBlocks, c->q_parts, c->dsc, c->g.n,
             c->p.cooling, c->R, c->p.Cv, c->p.Cp, c->Vcell, c->p.dt * kPost[s],
             c->p.dt * kPre[s], s, (int)c->np1_is_base);
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  return encode;
}

bool encode_3d_8b(CUtensorMap *map, const void *base, long long nx, long long ny, long long nz,
                  long long pitch, int bx, int by, int bz) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)pitch * 8, (cuuint64_t)pitch * ny * 8};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(base), dims, strides,
                box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

bool make_tensor_map_f64(CUtensorMap *map, const double *base, int nx, int ny, long long nz,
                         int bx, int by) {
  return encode_3d_8b(map, base, nx, ny, nz, nx, bx, by, 1);
}

bool make_tensor_map_8b(CUtensorMap *map, const void *base, int nx, int ny, int nz, int pitch,
                        int bx, int by, int bz) {
  return encode_3d_8b(map, base, nx, ny, nz, pitch, bx, by, bz);
}

// the tensor maps of a device array, built on first use (host work only)
const TmaField &tma_field(tpm_ctx *c, const double *base, long long layers) {
  for (const TmaField &f : c->tma_fields)
    if (f.base == base && f.layers == layers) return f;
  TmaField f;
  f.base = base;
  f.layers = layers;
  const Grid &g = c->g;
  if (!make_tensor_map_f64(&f.tile, base, g.nx, g.ny, layers, kZX, kZY) ||
      !make_tensor_map_f64(&f.row, base, g.nx, g.ny, layers, kZX, 1) ||
      !make_tensor_map_f64(&f.col, base, g.nx, g.ny, layers, 2, kZY))
    throw std::string("the driver refused a TMA tensor map");
  c->tma_fields.push_back(f);
  return c->tma_fields.back();
}

void launch_rho_update(tpm_ctx *c, int s, bool np1_in_base) {
  if (c->p.precision == TPM_PREC_MIXED && c->tma_rhs) {  // with the face velocity
    RfMaps m;
    const TmaField &R = tma_field(c, c->RU_int, 3LL * c->g.nz);
    m.ru_t = R.tile;
    m.ru_r = R.row;
    m.ru_c = R.col;
    const TmaField &D = tma_field(c, c->Rho_int, c->g.nz);
    m.rho_t = D.tile;
    m.rho_r = D.row;
    m.rho_c = D.col;
    TPM_LAUNCH(c, "rho_update", k_rho_face_tma, zm_blocks(c), kZX * kZY, RfSmem::kBytes, c->g, m,
               c->dsc, c->RU_int, c->Rho_int, c->Rho, np1_in_base ? c->Rho : c->Rho_np1,
               c->Rho_np1, c->Rho_new, c->Tgas, c->U32, -(c->p.dt * kPost[s]),
               -c->p.dt * kPre[s], s, zm_zlen(c));
    return;
  }
  if (c->p.precision == TPM_PREC_MIXED) {
    TPM_LAUNCH(c, "rho_update", k_rho_update_mixed, cell_waves(c, k_rho_update_mixed, false),
               kThreads, 0, c->g,
               c->RU_int, c->Rho, np1_in_base ? c->Rho : c->Rho_np1, c->Rho_np1, c->Rho_new,
               c->tma_rhs ? nullptr : reinterpret_cast<float2 *>(c->inv_rho), c->Tgas, c->dsc,
               -(c->p.dt * kPost[s]), -c->p.dt * kPre[s], s);
    return;
  }
  TPM_LAUNCH(c, "rho_update", k_rho_update, cell_waves(c, k_rho_update, false), kThreads, 0,
             c->g, c->RU_int,
             c->Rho, np1_in_base ? c->Rho : c->Rho_np1, c->Rho_np1, c->Rho_new, c->inv_rho,
             c->Tgas, c->dsc, -(c->p.dt * kPost[s]), -c->p.dt * kPre[s], s);
}

bool face_velocity_in_rho_pass(const tpm_ctx *c) {
  return c->p.precision == TPM_PREC_MIXED && c->tma_rhs;
}

void launch_face_velocity(tpm_ctx *c) {
  if (face_velocity_in_rho_pass(c)) return;  // k_rho_face_tma formed it
  if (c->p.precision == TPM_PREC_MIXED) {
    TPM_LAUNCH(c, "face_velocity", k_face_velocity_mixed,
               cell_waves(c, k_face_velocity_mixed, false), kThreads, 0, c->g,
               c->RUi32, c->Rho_int, c->U32);
    return;
  }
  TPM_LAUNCH(c, "face_velocity", k_face_velocity, cell_waves(c, k_face_velocity, false),
             kThreads, 0, c->g,
             c->RU_int, c->Rho_int, c->U);
}

void launch_rhs_momentum(tpm_ctx *c, int s, bool np1_in_base) {
  RhsArgs a;
  a.a_fp = -c->mp / c->Vcell;
  a.b_gd = c->p.Mu0 / 3.;
  a.c_lap = c->p.Mu0;
  a.A = c->A;
  a.Rho0 = c->p.Rho0;
  a.g[0] = c->gx;
  a.g[1] = c->gy;
  a.g[2] = c->gz;
  a.has_g = (c->gx != 0 || c->gy != 0 || c->gz != 0);
  a.dtpo = c->p.dt * kPost[s];
  a.dtpr = c->p.dt * kPre[s];
  a.stage = s;
  a.f_a_fp = (float)a.a_fp; a.f_b_gd = (float)a.b_gd; a.f_c_lap = (float)a.c_lap;
  a.f_A = (float)a.A; a.f_Rho0 = (float)a.Rho0;
  const double inv_d[3] = {c->g.inv_dx, c->g.inv_dy, c->g.inv_dz};
  const double inv_d2[3] = {c->g.inv_dx2, c->g.inv_dy2, c->g.inv_dz2};
  for (int d = 0; d < 3; ++d) {
    a.f_g[d] = (float)a.g[d];
    a.f_inv_d[d] = (float)inv_d[d];
    a.f_inv_d2[d] = (float)inv_d2[d];
  }
  const int tiles = ((c->g.nx + kTX - 1) / kTX) * ((c->g.ny + kTY - 1) / kTY) *
                    ((c->g.nz + kTZ - 1) / kTZ);
  // FP32: the cached per-cell form is faster (6.1 ms tiled vs 4.2 ms per 256^3
  // step); FP64: the tiled form saves FP64 issue slots (28.7 vs 31.5 ms).
  if (c->p.precision == TPM_PREC_MIXED)
    TPM_LAUNCH(c, "rhs_momentum", k_rhs_momentum_zm, zm_blocks(c), kZX * kZY, 0, c->g, c->U32,
               c->RUi32, c->Fp32, c->Rho_int, c->RU, np1_in_base ? c->RU : c->RU_np1,
               c->RU_np1, c->RU_new, a, zm_zlen(c));
  else
    TPM_LAUNCH(c, "rhs_momentum", (k_rhs_momentum_tiled<double, double>), tiles,
               kTX * kTY * kTZ, rhs_tiled_smem<double>(), c->g, c->U, c->RU_int, c->Fp,
               c->Rho_int, c->RU, np1_in_base ? c->RU : c->RU_np1, c->RU_np1, c->RU_new, a);
}

void launch_face_coeff(tpm_ctx *c) {
  if (c->p.precision != TPM_PREC_MIXED || c->tma_rhs) return;  // (formed by the TMA pass)
  TPM_LAUNCH(c, "face_coeff", k_face_coeff_mixed, cell_waves(c, k_face_coeff_mixed, false),
             kThreads, 0, c->g, c->Rho_new, c->Cface, c->Cs2,
             c->p.Solver == 2 ? c->Cs : nullptr);
}

void launch_poisson_rhs(tpm_ctx *c, int s, bool store_div) {
  PoisArgs a;
  a.kCp = c->p.k / c->p.Cp;
  a.inv_dtpre = (1. / (c->p.dt * kPre[s]));
  a.cooling = c->p.cooling;
  a.store_div = store_div;
  const bool mixed = c->p.precision == TPM_PREC_MIXED;
  const int nzm = zm_blocks(c);
  const int nb = mixed ? nzm : cell_waves(c, k_poisson_rhs2, true);
  double *rhs_parts = mixed ? c->zm_parts : c->partials + kPartRhs * kRedBlocks;
  double *tke_parts =
      s == 3 ? (mixed ? c->zm_parts + nzm : c->partials + kPartTke2 * kRedBlocks) : nullptr;
  if (mixed && c->tma_rhs) {
    PrMaps m;
    const TmaField &R = tma_field(c, c->Rho_new, c->g.nz);
    m.rho_t = R.tile;
    m.rho_r = R.row;
    m.rho_c = R.col;
    const TmaField &U = tma_field(c, c->RU_new, 3LL * c->g.nz);
    m.ru_t = U.tile;
    m.ru_r = U.row;
    m.ru_c = U.col;
    m.q_t = tma_field(c, c->Q, c->g.nz).tile;
    TPM_LAUNCH(c, "poisson_rhs", k_poisson_rhs_tma, nzm, kZX * kZY, PrSmem::kBytes, c->g, m,
               c->dsc, c->RHS, c->divg, c->cc32, c->Cs2, rhs_parts, tke_parts, a, zm_zlen(c));
  } else if (mixed) {
    // (C and Cs2 come from launch_face_coeff, run beside the particle stage)
    const bool pcg = c->p.Solver == 2;
    TPM_LAUNCH(c, "poisson_rhs", k_poisson_rhs_zm, nzm, kZX * kZY, 0, c->g,
               reinterpret_cast<const float2 *>(c->inv_rho), c->Q,
               c->RU_new, c->Cface, c->dsc, c->RHS, c->divg, c->cc32, pcg ? c->cc : nullptr,
               rhs_parts, tke_parts, a, zm_zlen(c));
  } else {
    // c->U (the face velocity of RU_int) is dead after the momentum RHS; it
    // holds RU_new/Rho_face here
    TPM_LAUNCH(c, "poisson_faces", k_poisson_faces, cell_waves(c, k_poisson_faces, false),
               kThreads, 0, c->g, c->Rho_new, c->RU_new, c->Cface, c->U);
    TPM_LAUNCH(c, "poisson_rhs", k_poisson_rhs2, nb, kThreads, 0, c->g, c->inv_rho, c->Q, c->U,
               c->Cface, c->dsc, c->RHS, c->divg, c->cc, c->partials + kPartRhs * kRedBlocks,
               tke_parts, a);
  }
  TPM_LAUNCH(c, "finish_mean", k_finish_mean, 1, kThreads, 0, rhs_parts, nb, c->g.n,
             &c->dsc->mean_rhs);
  if (tke_parts)
    TPM_LAUNCH(c, "finish_mean", k_finish_mean, 1, kThreads, 0, tke_parts, nb, c->g.n,
               &c->dsc->tke2);
}

void launch_project(tpm_ctx *c, int s) {
  const bool mixed = c->p.precision == TPM_PREC_MIXED;
  auto kern = mixed ? (s == 3 ? k_project<true, true> : k_project<true, false>)
                    : (s == 3 ? k_project<false, true> : k_project<false, false>);
  const int nb = cell_waves(c, kern, true);
  TPM_LAUNCH(c, "project", kern, nb, kThreads, 0, c->g, c->P, c->RU_np1, c->RU_new,
             -(c->p.dt * kPost[s]), -(c->p.dt * kPre[s]), s,
             c->partials + kPartRu * kRedBlocks, mixed ? c->RUn32 : nullptr);
  if (s == 3)
    TPM_LAUNCH(c, "finish_means3", k_finish_means3, 1, kThreads, 0,
               c->partials + kPartRu * kRedBlocks, nb, c->g.n,
               c->dsc);
}

void launch_passive_scalar(tpm_ctx *c, int s, bool np1_in_base) {
  PsArgs a;
  a.D_M = c->p.D_M;
  a.dtpo = c->p.dt * kPost[s];
  a.dtpr = c->p.dt * kPre[s];
  a.stage = s;
  a.s1_type = c->p.S1_type;
  const double *np1_in = np1_in_base ? c->PS : c->PS_np1;
  if (c->p.precision == TPM_PREC_MIXED)
    TPM_LAUNCH(c, "passive_scalar", k_passive_scalar<float>,
               cell_waves(c, k_passive_scalar<float>, false), kThreads, 0,
               c->g, c->U32, c->PS_face, c->PS_int, c->PS, np1_in, c->PS_np1, c->PS_new, c->S1,
               a);
  else
    TPM_LAUNCH(c, "passive_scalar", k_passive_scalar<double>,
               cell_waves(c, k_passive_scalar<double>, false), kThreads, 0,
               c->g, c->U, c->PS_face, c->PS_int, c->PS, np1_in, c->PS_np1, c->PS_new, c->S1, a);
  launch_passive_scalar_face(c, c->PS_new);
}

void launch_passive_scalar_face(tpm_ctx *c, const double *src) {
  TPM_LAUNCH(c, "passive_scalar_face", k_ps_face, cell_waves(c, k_ps_face, false), kThreads, 0,
             c->g, src,
             c->PS_face);
}

void launch_div_residual(tpm_ctx *c, int s, const double *RUn) {
  const int nb = cell_waves(c, k_div_residual, true);
  TPM_LAUNCH(c, "div_residual", k_div_residual, nb, kThreads, 0, c->g, RUn, c->Cs2,
             c->divg, c->dsc, c->p.dt * kPre[s], c->partials + kPartDiv * kRedBlocks);
  TPM_LAUNCH(c, "finish_max_div", k_finish_max_div, 1, kThreads, 0,
             c->partials + kPartDiv * kRedBlocks, nb, c->dsc);
}

void launch_to_float(tpm_ctx *c, const double *src, float *dst, long long n) {
  TPM_LAUNCH(c, "to_float", k_to_float, cell_blocks(c->g), kThreads, 0, src, dst, n);
}

void launch_to_double(tpm_ctx *c, const float *src, double *dst, long long n) {
  TPM_LAUNCH(c, "to_double", k_to_double, cell_blocks(c->g), kThreads, 0, src, dst, n);
}

void rhs_kernels_setup(tpm_ctx *c) {
  TPM_CUDA_TRY(cudaFuncSetAttribute(k_rhs_momentum_tiled<double, double>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)rhs_tiled_smem<double>()));
  // the TMA Poisson pass of the mixed path where the grid is whole 32 x 8
  // column tiles and the pressure solver is Richardson's; its tensor maps for
  // both buffers Rho_new and RU_new take turns in, and Q
  c->tma_rhs = false;
  if (c->p.precision == TPM_PREC_MIXED && c->p.Solver == 0 && c->g.nx % kZX == 0 &&
      c->g.ny % kZY == 0) {
    TPM_CUDA_TRY(cudaFuncSetAttribute(k_poisson_rhs_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      PrSmem::kBytes));
    try {
      for (const double *b : {c->Rho_new, c->Rho_int, c->Q}) tma_field(c, b, c->g.nz);
      for (const double *b : {c->RU_new, c->RU_int}) tma_field(c, b, 3LL * c->g.nz);
      c->tma_rhs = true;
    } catch (const std::string &) {
      c->tma_fields.clear();  // the driver has no TMA maps for us: the two-pass form
    }
  }
  // the occupancy of every wave-sized kernel, queried here once (not while a
  // step is being captured into a graph)
  cell_waves(c, k_rho_update_mixed, false);
  cell_waves(c, k_rho_update, false);
  cell_waves(c, k_face_velocity_mixed, false);
  cell_waves(c, k_face_velocity, false);
  cell_waves(c, k_poisson_rhs2, true);
  cell_waves(c, k_face_coeff_mixed, false);
  cell_waves(c, k_poisson_faces, false);
  cell_waves(c, k_project<true, true>, true);
  cell_waves(c, k_project<true, false>, true);
  cell_waves(c, k_project<false, true>, true);
  cell_waves(c, k_project<false, false>, true);
  cell_waves(c, k_passive_scalar<float>, false);
  cell_waves(c, k_passive_scalar<double>, false);
  cell_waves(c, k_ps_face, false);
  cell_waves(c, k_div_residual, true);
  cell_waves(c, k_mean_reset, false);
}

void launch_mean_reset(tpm_ctx *c) {
  TPM_LAUNCH(c, "mean_reset", k_mean_reset, cell_waves(c, k_mean_reset, false), kThreads, 0,
             c->g, c->RU_np1,
             c->RU, c->dsc, c->p.U0 * c->p.Rho0, c->p.V0 * c->p.Rho0, c->p.W0 * c->p.Rho0);
}

void launch_center_coeff_from_C(tpm_ctx *c) {
  TPM_LAUNCH(c, "center_coeff", k_center_coeff, cell_blocks(c->g), kThreads, 0, c->g, c->Cface,
             c->cc);
  if (c->p.precision == TPM_PREC_MIXED)  // the mixed residual reads C/d^2
    TPM_LAUNCH(c, "face_coeff_scaled", k_scale_faces, cell_blocks(c->g), kThreads, 0, c->g,
               c->Cface, c->cc, c->Cs, c->Cs2, c->cc32);
}

}  // namespace tpm
