// Lagrangian particle stage of the RK4 substep (grid::Update_Particle,
// grid.cpp:865-888) on the GPU.
//
//  * k_push: one thread per particle does the whole per-particle chain of the
//    reference - face-linear gas velocity at x_int (particle.cpp:340-360),
//    position / velocity / temperature RK updates (:314-338, :362-399,
//    :477-492), the periodic wrap that replaces migration (:58-104,
//    :150-250), the trilinear gas temperature at x_new and the heat
//    exchange rate (:430-474) - and emits each particle's deposit payload
//    and its cell key.
//  * deposits (part2gas_velocity :494-520, part2gas_concentration :522-555,
//    part2gas_Temp_new :620-654) are deterministic: particles are counting-
//    sorted by cell (ties ordered by particle index), then every target cell
//    gathers the contributions of the particles in its neighbouring cells in
//    a fixed order.  No floating-point atomics, so the sources are bit-
//    reproducible run to run; they differ from the reference's particle-order
//    sums only by FP64 reassociation.
#include <utility>

#include "tpm_internal.cuh"
#include "tpm_ff.cuh"
#include "tpm_reduce.cuh"

namespace tpm {
namespace {

constexpr int kThreads = 256;

// flat index in 32-bit arithmetic (every box has fewer than 2^31 cells)
__device__ __forceinline__ long long at(const Grid &g, int i, int j, int k) {
  return (long long)((k * g.ny + j) * g.nx + i);
}

struct PushArgs {
  double dtpo, dtpr;       // dt*post, dt*pre
  double iTp;              // 1/Tp (particle.cpp:365)
  double gp[3];            // ParticleGravity*g (particle.cpp:376-378)
  double alpha;            // particle.cpp:481
  double iS;               // 1/(mp*Cvp), particle.cpp:483
  double iTth;             // Nu*pi*Dp*k, particle.cpp:470
  int stage, twc, has_tau;
  int has_gp;              // any gp[d] nonzero
};

struct PState {
  const double *b[7];  // base (x is written back when wrapped)
  double *bx[3];
  const double *in[7];  // int
  const double *np1_in[7];
  double *np1[7];
  double *nw[7];
};

// a warp's keys (lanes in `live`) counted into their cells, one atomic per
// distinct key (the counting sort's histogram; in cell order neighbouring
// lanes share a cell)
__device__ __forceinline__ void count_keys(unsigned live, bool mine, int32_t key,
                                           int32_t *__restrict__ counts) {
  if (mine) {
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(live, key);
    if (lane == __ffs(peers) - 1) atomicAdd(&counts[key], __popc(peers));
  }
}

// TU: element type of the face velocity (FP32 copy on the mixed path);
// TP: type of the momentum-deposit payload.  cnt_t / cnt_r (when not null,
// cleared): the per-cell counts of key_t / key_r, the two counting sorts'
// histograms, formed here instead of by a pass over the keys.  A warp walks
// the particles together (uniform trip count) for the counting.
template <typename TU, typename TP>
__global__ void __launch_bounds__(kThreads, sizeof(TU) == sizeof(float) ? 4 : 3)
k_push(Grid g, PState ps, PushArgs a, int64_t np, const TU *__restrict__ U,
                       const double *__restrict__ RUi, const double *__restrict__ Rhoi,
                       const double *__restrict__ Tgas, double *__restrict__ rhs_t,
                       const double *__restrict__ tau, int32_t *__restrict__ key_t,
                       TP *__restrict__ pay_t, int32_t *__restrict__ key_r,
                       TP *__restrict__ pay_r, int32_t *__restrict__ cnt_t,
                       int32_t *__restrict__ cnt_r) {
  const int lane_ = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane_; base < np;
       base += (int64_t)gridDim.x * blockDim.x) {
  const int64_t p = base + lane_;
  const unsigned live = __ballot_sync(0xffffffffu, p < np);
  int32_t kt = 0, kr = 0;
  if (p < np) {
    constexpr bool kMixed = sizeof(TU) == sizeof(float);
    const double xi = ps.in[0][p], yi = ps.in[1][p], zi = ps.in[2][p];
    const double ui = ps.in[3][p], vi = ps.in[4][p], wi = ps.in[5][p];
    // ---- gas2part_velocity at x_int (particle.cpp:340-360) ----
    int tx, ty, tz;
    double xl = 0, yl = 0, zl = 0;     // FP64 path: fractions in FP64
    float2 fx, fy, fz;                 // mixed path: the same fractions as pairs
    if constexpr (kMixed) {
      // trunc(x/d) and its fraction from the bits of the FP64 product (the
      // same cell as the FP64 route, no FP64-pipe conversions)
      ff_int_frac2(xi * g.idx, tx, fx);
      ff_int_frac2(yi * g.idy, ty, fy);
      ff_int_frac2(zi * g.idz, tz, fz);
    } else {
      tx = (int)(xi * g.idx);
      ty = (int)(yi * g.idy);
      tz = (int)(zi * g.idz);
      xl = (xi * g.idx - ((int)(xi * g.idx)));
      yl = (yi * g.idy - ((int)(yi * g.idy)));
      zl = (zi * g.idz - ((int)(zi * g.idz)));
    }
    const int i0 = wrap_any(tx, g.nx), j0 = wrap_any(ty, g.ny), k0 = wrap_any(tz, g.nz);
    const long long c0 = at(g, i0, j0, k0);
    double ug = 0, vg = 0, wg = 0;  // FP64 path
    float2 gq[3];                   // mixed path: the gas velocity as pairs
    if constexpr (!kMixed) {
      ug = xl * (double)U[at(g, wrap_p(i0, g.nx), j0, k0)] + (1 - xl) * (double)U[c0];
      vg = yl * (double)U[g.n + at(g, i0, wrap_p(j0, g.ny), k0)] + (1 - yl) * (double)U[g.n + c0];
      wg = zl * (double)U[2 * g.n + at(g, i0, j0, wrap_p(k0, g.nz))] +
           (1 - zl) * (double)U[2 * g.n + c0];
    } else {
      // mixed path: the face velocity RU_int / I_C2F(Rho_int) at the particle's
      // two faces of each component, and the interpolation between them, in
      // float-float pairs from the FP64 state (within ~2^-44 of the FP64
      // route).  An FP32 face velocity would put ~1e-7 into every particle's
      // gas velocity, and the reference's interpolation is nearest-cell across
      // the transverse faces (particle.cpp:340-360): a particle whose position
      // then drifts across a face takes another cell's velocity.
      const long long cxp = at(g, wrap_p(i0, g.nx), j0, k0), cxm = at(g, wrap_m(i0, g.nx), j0, k0);
      const long long cyp = at(g, i0, wrap_p(j0, g.ny), k0), cym = at(g, i0, wrap_m(j0, g.ny), k0);
      const long long czp = at(g, i0, j0, wrap_p(k0, g.nz)), czm = at(g, i0, j0, wrap_m(k0, g.nz));
      const float2 r0 = ff_from_double(Rhoi[c0]);
      // RU / ((Rho_a + Rho_b) / 2) = 2 RU / (Rho_a + Rho_b)
      auto uface = [&](double ru, const float2 &ra, double rb) {
        const float2 q = ff_mul(ff_from_double(ru), ff_rcp(ff_add(ra, ff_from_double(rb))));
        return ff_norm(make_float2(2.f * q.x, 2.f * q.y));
      };
      auto lerp = [&](const float2 &f, const float2 &u0, const float2 &u1) {
        return ff_add(u0, ff_mul(f, ff_sub(u1, u0)));
      };
      const float2 rxp = ff_from_double(Rhoi[cxp]), ryp = ff_from_double(Rhoi[cyp]),
                   rzp = ff_from_double(Rhoi[czp]);
      gq[0] = lerp(fx, uface(RUi[c0], r0, Rhoi[cxm]), uface(RUi[cxp], rxp, Rhoi[c0]));
      gq[1] = lerp(fy, uface(RUi[g.n + c0], r0, Rhoi[cym]), uface(RUi[g.n + cyp], ryp, Rhoi[c0]));
      gq[2] = lerp(fz, uface(RUi[2 * g.n + c0], r0, Rhoi[czm]),
                   uface(RUi[2 * g.n + czp], rzp, Rhoi[c0]));
    }
    // ---- update_position (particle.cpp:314-338) ----
    // (the mixed path, TU = float, accumulates with FMAs; the FP64 path keeps
    // the reference's separate multiply and add)
    constexpr bool kFma = sizeof(TU) == sizeof(float);
    double xn[3], xp[3], xb[3];
    const double uint_[3] = {ui, vi, wi};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      xb[d] = ps.b[d][p];
      xp[d] = kFma ? fma(a.dtpo, uint_[d], ps.np1_in[d][p]) : ps.np1_in[d][p] + a.dtpo * uint_[d];
      xn[d] = (a.stage != 3) ? (kFma ? fma(a.dtpr, uint_[d], xb[d]) : xb[d] + a.dtpr * uint_[d])
                             : xp[d];
    }
    // ---- update_velocity (particle.cpp:362-399) ----
    const double iTp = a.has_tau ? 1. / tau[p] : a.iTp;
    // RHS_u = (u_gas - u_int) / Tp; the mixed path forms it in pairs (within
    // ~2^-44 of the FP64 value: the drag of a relaxing particle, a difference
    // of close velocities, keeps its relative accuracy) with one FP64
    // operation per component instead of four; rh: its FP32 value for the
    // deposit payload
    double rhs[3];
    float rh[3];
    if constexpr (kMixed) {
      const float2 it2 = ff_from_double(iTp);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float2 r = ff_mul(ff_sub_sloppy(gq[d], ff_from_double(uint_[d])), it2);
        rh[d] = r.x;
        rhs[d] = ff_to_double(r);
      }
    } else {
      rhs[0] = (ug - ui) * iTp;
      rhs[1] = (vg - vi) * iTp;
      rhs[2] = (wg - wi) * iTp;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double f = (!kMixed || a.has_gp) ? rhs[d] + a.gp[d] : rhs[d];
      double np1 = kFma ? fma(a.dtpo, f, ps.np1_in[3 + d][p]) : ps.np1_in[3 + d][p] + a.dtpo * f;
      ps.np1[3 + d][p] = np1;
      ps.nw[3 + d][p] = (a.stage != 3) ? (kFma ? fma(a.dtpr, f, ps.b[3 + d][p])
                                               : ps.b[3 + d][p] + a.dtpr * f)
                                       : np1;
    }
    // ---- update_Temp with the previous heat rate (particle.cpp:477-492) ----
    const double rt_old = rhs_t[p];
    const double Tnp1 = ps.np1_in[6][p] + a.dtpo * a.iS * (rt_old + a.alpha);
    const double Tnew = (a.stage != 3) ? ps.b[6][p] + a.dtpr * a.iS * (rt_old + a.alpha) : Tnp1;
    ps.np1[6][p] = Tnp1;
    ps.nw[6][p] = Tnew;
    // ---- part2gas_velocity payload at x_int (particle.cpp:494-520) ----
    if (a.twc) {
      key_t[p] = (int32_t)c0;
      kt = (int32_t)c0;
      if (kFma) {  // FP32 payload (mixed path): FP32 products of truncated copies
        const float xf = fx.x, yf = fy.x, zf = fz.x;
        const float r0 = rh[0], r1 = rh[1], r2 = rh[2];
        pay_t[0 * np + p] = (TP)((1 - xf) * r0);
        pay_t[1 * np + p] = (TP)(xf * r0);
        pay_t[2 * np + p] = (TP)((1 - yf) * r1);
        pay_t[3 * np + p] = (TP)(yf * r1);
        pay_t[4 * np + p] = (TP)((1 - zf) * r2);
        pay_t[5 * np + p] = (TP)(zf * r2);
      } else {
        pay_t[0 * np + p] = (TP)((1 - xl) * rhs[0]);
        pay_t[1 * np + p] = (TP)(xl * rhs[0]);
        pay_t[2 * np + p] = (TP)((1 - yl) * rhs[1]);
        pay_t[3 * np + p] = (TP)(yl * rhs[1]);
        pay_t[4 * np + p] = (TP)((1 - zl) * rhs[2]);
        pay_t[5 * np + p] = (TP)(zl * rhs[2]);
      }
    }
    // ---- Send_Recv on one rank = periodic wrap (particle.cpp:58-104, 150-250) ----
    const double L[3] = {g.Lx, g.Ly, g.Lz};
    const double hi[3] = {g.xh, g.yh, g.zh};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      // mixed path: the two tests on the bit patterns (integer compares; for
      // hi > 0, x > hi iff the signed patterns compare so, and x < 0 iff the
      // sign is set on a nonzero magnitude)
      const long long bx_ = __double_as_longlong(xn[d]);
      const bool out = kMixed ? (bx_ > __double_as_longlong(hi[d]) ||
                                 (unsigned long long)bx_ > 0x8000000000000000ull)
                              : (xn[d] > hi[d] || xn[d] < 0);
      if (out) {
        if (xn[d] > L[d]) {
          xn[d] -= L[d];
          xb[d] -= L[d];
          xp[d] -= L[d];
          ps.bx[d][p] = xb[d];
        } else if (xn[d] < 0) {
          xn[d] += L[d];
          xb[d] += L[d];
          xp[d] += L[d];
          ps.bx[d][p] = xb[d];
        }
      }
      ps.np1[d][p] = xp[d];
      ps.nw[d][p] = xn[d];
    }
    // ---- gas2part_Temp_new + Compute_RHS_Temp_new at x_new (particle.cpp:430-474) ----
    int ri, rj, rk;
    double x_l, y_l, z_l;
    float xl_f[3] = {0, 0, 0};  // mixed: the fractions in FP32
    if constexpr (kMixed) {
      // round(x/d) (half away from zero) and x/d - round + 1/2 from the bits
      // of the FP64 product
      const double u[3] = {xn[0] * g.idx, xn[1] * g.idy, xn[2] * g.idz};
      int r[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        int ip;
        float fr;
        bool up;
        ff_int_frac(u[d], ip, fr, up);
        const bool neg = __double_as_longlong(u[d]) < 0;  // sign bit, no FP64 compare
        r[d] = ip + (up ? (neg ? -1 : 1) : 0);
        xl_f[d] = fr + 0.5f + (up ? (neg ? 1.f : -1.f) : 0.f);
      }
      ri = r[0]; rj = r[1]; rk = r[2];
      x_l = ff_f2d(xl_f[0]);
      y_l = ff_f2d(xl_f[1]);
      z_l = ff_f2d(xl_f[2]);
    } else {
      ri = (int)(round(xn[0] * g.idx));
      rj = (int)(round(xn[1] * g.idy));
      rk = (int)(round(xn[2] * g.idz));
      x_l = xn[0] * g.idx - ri + 0.5;
      y_l = xn[1] * g.idy - rj + 0.5;
      z_l = xn[2] * g.idz - rk + 0.5;
    }
    const int i1 = wrap_any(ri, g.nx), im = wrap_any(ri - 1, g.nx);
    const int j1 = wrap_any(rj, g.ny), jm = wrap_any(rj - 1, g.ny);
    const int k1 = wrap_any(rk, g.nz), km = wrap_any(rk - 1, g.nz);
    double rt;
    if (sizeof(TU) == sizeof(double)) {
      const double Tg = x_l * y_l * z_l * Tgas[at(g, i1, j1, k1)] +
                        (1 - x_l) * y_l * z_l * Tgas[at(g, im, j1, k1)] +
                        x_l * (1 - y_l) * z_l * Tgas[at(g, i1, jm, k1)] +
                        x_l * y_l * (1 - z_l) * Tgas[at(g, i1, j1, km)] +
                        (1 - x_l) * (1 - y_l) * z_l * Tgas[at(g, im, jm, k1)] +
                        (1 - x_l) * y_l * (1 - z_l) * Tgas[at(g, im, j1, km)] +
                        x_l * (y_l - 1) * (z_l - 1) * Tgas[at(g, i1, jm, km)] +
                        (1 - x_l) * (1 - y_l) * (1 - z_l) * Tgas[at(g, im, jm, km)];
      rt = (Tg - Tnew) * a.iTth;
    } else {
      // mixed path: Tg - T_new = sum_k w_k (T_k - T_new) (the weights sum to
      // one); the differences are FP64, the small weighted sum FP32, so the
      // heat rate - a difference of nearly equal temperatures - keeps its
      // relative accuracy
      // (the differences from split pairs: the high parts of two close
      // temperatures subtract exactly, the low parts add their remainder)
      const float xf = xl_f[0], yf = xl_f[1], zf = xl_f[2];
      const float2 tn = ff_from_double(Tnew);
      auto dT = [&](long long cell) {
        const float2 t = ff_from_double(Tgas[cell]);
        return (t.x - tn.x) + (t.y - tn.y);
      };
      const float d0 = dT(at(g, i1, j1, k1));
      const float d1 = dT(at(g, im, j1, k1));
      const float d2 = dT(at(g, i1, jm, k1));
      const float d3 = dT(at(g, i1, j1, km));
      const float d4 = dT(at(g, im, jm, k1));
      const float d5 = dT(at(g, im, j1, km));
      const float d6 = dT(at(g, i1, jm, km));
      const float d7 = dT(at(g, im, jm, km));
      const float sum = xf * yf * zf * d0 + (1 - xf) * yf * zf * d1 + xf * (1 - yf) * zf * d2 +
                        xf * yf * (1 - zf) * d3 + (1 - xf) * (1 - yf) * zf * d4 +
                        (1 - xf) * yf * (1 - zf) * d5 + xf * (1 - yf) * (1 - zf) * d6 +
                        (1 - xf) * (1 - yf) * (1 - zf) * d7;
      rt = ff_f2d(sum) * a.iTth;
    }
    rhs_t[p] = rt;
    kr = (int32_t)at(g, i1, j1, k1);
    key_r[p] = kr;
    if constexpr (kMixed) {  // the FP32 values the mixed deposit uses (x_l is one exactly)
      pay_r[0 * np + p] = ff_hi(x_l);
      pay_r[1 * np + p] = ff_hi(y_l);
      pay_r[2 * np + p] = ff_hi(z_l);
      pay_r[3 * np + p] = ff_hi(rt);
    } else {
      pay_r[0 * np + p] = x_l;
      pay_r[1 * np + p] = y_l;
      pay_r[2 * np + p] = z_l;
      pay_r[3 * np + p] = rt;
    }
  }
  if (cnt_t) count_keys(live, p < np, kt, cnt_t);
  if (cnt_r) count_keys(live, p < np, kr, cnt_r);
  }
}

// round-indexed key and payload of the given particle set (used at
// initialisation, at x_int: grid.cpp:481-484); TP float for the mixed
// deposit (the FP64 values truncated, as that deposit reads them)
template <typename TP>
__global__ void k_cic_payload(Grid g, const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ z, const double *__restrict__ Tp,
                              const double *__restrict__ Tgas, double iTth, int64_t np,
                              double *__restrict__ rhs_t, int32_t *__restrict__ key_r,
                              TP *__restrict__ pay_r, int compute_rhs) {
  auto put = [&](int f, int64_t p, double v) { pay_r[f * np + p] = ff_cast<TP>(v); };
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double xx = x[p], yy = y[p], zz = z[p];
    const int ri = (int)(round(xx * g.idx)), rj = (int)(round(yy * g.idy)),
              rk = (int)(round(zz * g.idz));
    const double x_l = xx * g.idx - ri + 0.5;
    const double y_l = yy * g.idy - rj + 0.5;
    const double z_l = zz * g.idz - rk + 0.5;
    const int i1 = wrap_any(ri, g.nx), im = wrap_any(ri - 1, g.nx);
    const int j1 = wrap_any(rj, g.ny), jm = wrap_any(rj - 1, g.ny);
    const int k1 = wrap_any(rk, g.nz), km = wrap_any(rk - 1, g.nz);
    key_r[p] = (int32_t)at(g, i1, j1, k1);
    put(0, p, x_l);
    put(1, p, y_l);
    put(2, p, z_l);
    if (!compute_rhs) {  // heat rate given (continuation of a run)
      put(3, p, rhs_t[p]);
      continue;
    }
    // gas2part_Temp_int + Compute_RHS_Temp_int (particle.cpp:402-466)
    const double Tg = x_l * y_l * z_l * Tgas[at(g, i1, j1, k1)] +
                      (1 - x_l) * y_l * z_l * Tgas[at(g, im, j1, k1)] +
                      x_l * (1 - y_l) * z_l * Tgas[at(g, i1, jm, k1)] +
                      x_l * y_l * (1 - z_l) * Tgas[at(g, i1, j1, km)] +
                      (1 - x_l) * (1 - y_l) * z_l * Tgas[at(g, im, jm, k1)] +
                      (1 - x_l) * y_l * (1 - z_l) * Tgas[at(g, im, j1, km)] +
                      x_l * (y_l - 1) * (z_l - 1) * Tgas[at(g, i1, jm, km)] +
                      (1 - x_l) * (1 - y_l) * (1 - z_l) * Tgas[at(g, im, jm, km)];
    const double rt = (Tg - Tp[p]) * iTth;
    rhs_t[p] = rt;
    put(3, p, rt);
  }
}

// block partial sums of a centre field (mean for grid::Update_P0)
__global__ void k_partial_sums(long long n, const double *__restrict__ f,
                               double *__restrict__ partials) {
  __shared__ double sh[32];
  double acc = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x)
    acc += f[c];
  double b = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

__global__ void k_fill_tgas(long long n, const double *__restrict__ Rho, double T_scale,
                            double *__restrict__ Tgas) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x)
    Tgas[c] = T_scale / Rho[c];
}

// ------------------------------------------------------------ counting sort
// The counting sort's atomics are aggregated per warp over equal keys: with
// the particles in cell order (mixed path) neighbouring lanes share a cell,
// and one atomic per cell and warp replaces up to 32 on the same address.
// The warp walks the particles together (uniform trip count) so that the
// match covers exactly the lanes holding a particle.
__global__ void k_hist(const int32_t *__restrict__ key, int64_t np, int32_t *__restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < np;
       base += stride) {
    const int64_t p = base + lane;
    const unsigned live = __ballot_sync(0xffffffffu, p < np);
    if (p < np) {
      const int32_t k = key[p];
      const unsigned peers = __match_any_sync(live, k);
      if (lane == __ffs(peers) - 1) atomicAdd(&counts[k], __popc(peers));
    }
  }
}

constexpr int kScanThreads = 512;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

// exclusive scan, phase 1: per-chunk totals
__global__ void k_scan_reduce(const int32_t *__restrict__ counts, long long n,
                              int32_t *__restrict__ chunk_sums) {
  __shared__ int32_t sh[32];
  long long base = (long long)blockIdx.x * kScanChunk + threadIdx.x * kScanPer;
  int32_t s = 0;
#pragma unroll
  for (int e = 0; e < kScanPer; ++e)
    if (base + e < n) s += counts[base + e];
  int32_t t = block_sum(s, sh);
  if (threadIdx.x == 0) chunk_sums[blockIdx.x] = t;
}

// phase 2: one block turns chunk totals into chunk offsets (exclusive)
__global__ void k_scan_chunks(int32_t *__restrict__ chunk_sums, int nchunks) {
  __shared__ int32_t carry;
  __shared__ int32_t sh[kScanThreads];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nchunks; b0 += kScanThreads) {
    int i = b0 + threadIdx.x;
    int32_t v = i < nchunks ? chunk_sums[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {  // Hillis-Steele inclusive
      int32_t w = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += w;
      __syncthreads();
    }
    int32_t incl = sh[threadIdx.x];
    if (i < nchunks) chunk_sums[i] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry += incl;
    __syncthreads();
  }
}

// phase 3: starts[c] = offset + exclusive scan within the chunk; counts
// are cleared so the scatter can reuse them as cursors.  Each thread takes 8
// consecutive counts (two 16-byte loads where the chunk is whole), the block
// scans its threads' sums with warp shuffles and one pass over the 16 warp
// totals.
__global__ void k_scan_apply(int32_t *__restrict__ counts, long long n,
                             const int32_t *__restrict__ chunk_off, int32_t *__restrict__ starts,
                             int32_t total) {
  static_assert(kScanPer == 8 && kScanThreads % 32 == 0, "two int4 per thread");
  __shared__ int32_t wsum[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanChunk + threadIdx.x * kScanPer;
  const bool whole = base + kScanPer <= n;
  int32_t v[kScanPer];
  if (whole) {
    const int4 a = *reinterpret_cast<const int4 *>(counts + base);
    const int4 b = *reinterpret_cast<const int4 *>(counts + base + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int e = 0; e < kScanPer; ++e) v[e] = (base + e < n) ? counts[base + e] : 0;
  }
  int32_t s = 0;
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) s += v[e];
  // inclusive scan of the thread sums within the warp, then over the warps
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t w = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += w;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int32_t t = lane < kScanThreads / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t w = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += w;
    }
    if (lane < kScanThreads / 32) wsum[lane] = t;  // inclusive warp prefixes
  }
  __syncthreads();
  int32_t run = chunk_off[blockIdx.x] + (warp ? wsum[warp - 1] : 0) + incl - s;
  int32_t out[kScanPer];
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) {
    out[e] = run;
    run += v[e];
  }
  if (whole) {
    *reinterpret_cast<int4 *>(starts + base) = make_int4(out[0], out[1], out[2], out[3]);
    *reinterpret_cast<int4 *>(starts + base + 4) = make_int4(out[4], out[5], out[6], out[7]);
    *reinterpret_cast<int4 *>(counts + base) = make_int4(0, 0, 0, 0);
    *reinterpret_cast<int4 *>(counts + base + 4) = make_int4(0, 0, 0, 0);
  } else {
#pragma unroll
    for (int e = 0; e < kScanPer; ++e)
      if (base + e < n) {
        starts[base + e] = out[e];
        counts[base + e] = 0;
      }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) starts[n] = total;
}

// Lanes of a warp with equal keys take consecutive slots in lane order, that
// is in particle order; only a cell whose particles arrive from more than one
// warp (a group smaller than the cell's count) can end up out of order, and
// only such cells are flagged for k_segsort.  A group that is the whole cell
// (the usual case for particles kept in cell order) starts at the cell's
// first slot without touching its cursor (the cursors are cleared before
// every histogram).
__global__ void k_scatter(const int32_t *__restrict__ key, int64_t np,
                          const int32_t *__restrict__ starts, int32_t *__restrict__ cursor,
                          int32_t *__restrict__ perm, unsigned char *__restrict__ unsorted) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; base < np;
       base += stride) {
    const int64_t p = base + lane;
    const unsigned live = __ballot_sync(0xffffffffu, p < np);
    if (p < np) {
      const int32_t k = key[p];
      const unsigned peers = __match_any_sync(live, k);
      const int leader = __ffs(peers) - 1;
      int32_t first = 0;
      if (lane == leader && __popc(peers) != starts[k + 1] - starts[k]) {
        first = atomicAdd(&cursor[k], __popc(peers));
        unsorted[k] = 1;
      }
      first = __shfl_sync(live, first, leader);
      const int32_t slot = starts[k] + first + __popc(peers & ((1u << lane) - 1u));
      perm[slot] = (int32_t)p;
    }
  }
}

// order each flagged cell's particles by index (and clear its flag): the
// deposit sums become independent of the scatter's atomic order.  Insertion
// sort for the usual few particles
// per cell, an in-place heap sort (O(m log m), bounded) up to kSortMaxRun;
// a cell beyond that (a diverging run crowding its particles) is left in
// arrival order and flagged, so that no cell costs a thread more than
// ~kSortMaxRun log2(kSortMaxRun) steps.
constexpr int32_t kSortMaxRun = 65536;

__device__ __forceinline__ void sift_down(int32_t *a, int32_t root, int32_t end) {
  while (true) {
    int32_t child = 2 * root + 1;
    if (child >= end) return;
    if (child + 1 < end && a[child] < a[child + 1]) ++child;
    if (!(a[root] < a[child])) return;
    const int32_t t = a[root];
    a[root] = a[child];
    a[child] = t;
    root = child;
  }
}

__device__ void sort_cell(int32_t s, int32_t e, int32_t *__restrict__ perm,
                          int *__restrict__ crowded) {
  const int32_t m = e - s;
  if (m <= 32) {
    for (int32_t a = s + 1; a < e; ++a) {
      int32_t v = perm[a];
      int32_t b = a - 1;
      while (b >= s && perm[b] > v) {
        perm[b + 1] = perm[b];
        --b;
      }
      perm[b + 1] = v;
    }
  } else if (m <= kSortMaxRun) {
    int32_t *a = perm + s;
    for (int32_t i = m / 2 - 1; i >= 0; --i) sift_down(a, i, m);
    for (int32_t end = m - 1; end > 0; --end) {
      const int32_t t = a[0];
      a[0] = a[end];
      a[end] = t;
      sift_down(a, 0, end);
    }
  } else {
    *crowded = 1;
  }
}

// One thread per 16 flags (the flag array is padded to a multiple of 16
// bytes, the padding zero): most words are all zero, so the pass is one
// 16-byte load per thread and iteration.
__global__ void k_segsort(long long nwords, const int32_t *__restrict__ starts,
                          int32_t *__restrict__ perm, uint4 *__restrict__ unsorted,
                          int *__restrict__ crowded) {
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nwords;
       w += (long long)gridDim.x * blockDim.x) {
    const uint4 f = unsorted[w];
    if ((f.x | f.y | f.z | f.w) == 0u) continue;
    unsorted[w] = make_uint4(0u, 0u, 0u, 0u);
    const unsigned word[4] = {f.x, f.y, f.z, f.w};
    for (int q = 0; q < 4; ++q)
      for (int b = 0; b < 4; ++b)
        if ((word[q] >> (8 * b)) & 0xffu) {
          const long long c = w * 16 + q * 4 + b;
          sort_cell(starts[c], starts[c + 1], perm, crowded);
        }
  }
}

template <typename T>
__global__ void k_gather_payload(int64_t np, int nf, const int32_t *__restrict__ perm,
                                 const T *__restrict__ pay, T *__restrict__ sorted) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x) {
    int32_t p = perm[s];
    for (int f = 0; f < nf; ++f) sorted[f * np + s] = pay[f * np + p];
  }
}

// ------------------------------------------------------------------ deposits
// part2gas_velocity (particle.cpp:494-520) + cumulative ghost fold: face d of
// cell c collects the upper weight of the particles in cell c - e_d and the
// lower weight of those in cell c.
template <typename TP, typename TO>
__global__ void k_dep_momentum(Grid g, const int32_t *__restrict__ starts,
                               const TP *__restrict__ pay, int64_t np, TO *__restrict__ Fp) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const long long m[3] = {at(g, wrap_m(i, g.nx), j, k), at(g, i, wrap_m(j, g.ny), k),
                            at(g, i, j, wrap_m(k, g.nz))};
    const int32_t s0 = starts[c], e0 = starts[c + 1];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      TP acc = 0;
      const int32_t s1 = starts[m[d]], e1 = starts[m[d] + 1];
      for (int32_t s = s1; s < e1; ++s) acc += pay[(2 * d + 1) * np + s];
      for (int32_t s = s0; s < e0; ++s) acc += pay[(2 * d) * np + s];
      Fp[d * g.n + c] = (TO)acc;
    }
  }
}

// part2gas_concentration (particle.cpp:522-555) and part2gas_Temp_* (:582-654):
// ((fx*fy)*fz)*rhs with fx = xl for the centre at the round cell and 1-xl for
// the one below (the operation order of particle.cpp:545-552, :605-612,
// :643-650).
// Both linear-stencil deposits of one sorted particle set in one pass: the
// heat rate (weights x RHS_T) for this substep and the concentration
// (weights) that the next substep deposits at the same positions (its x_int
// is this x_new).  Weights are built per sorted slot from the unsorted
// payload; the sums keep the order of k_dep_sum8.
template <typename TW>
__global__ void k_cic_weights2(int64_t np, const int32_t *__restrict__ perm,
                               const double *__restrict__ pay, TW *__restrict__ wq,
                               TW *__restrict__ wc) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = perm[s];
    // (FP64 -> FP32 by integer operations on the mixed path: ff_cast)
    const TW xl = ff_cast<TW>(pay[p]), yl = ff_cast<TW>(pay[np + p]), zl = ff_cast<TW>(pay[2 * np + p]);
    const TW r = ff_cast<TW>(pay[3 * np + p]);
    const TW fx[2] = {xl, 1 - xl}, fy[2] = {yl, 1 - yl}, fz[2] = {zl, 1 - zl};
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const TW fxy = fx[dx] * fy[dy];
#pragma unroll
        for (int dz = 0; dz < 2; ++dz) {
          const size_t o = (size_t)((dz * 2 + dy) * 2 + dx) * np + s;
          const TW v = fxy * fz[dz];
          wc[o] = v;
          wq[o] = v * r;
        }
      }
  }
}

template <typename TW>
__global__ void k_dep_sum8x2(Grid g, const int32_t *__restrict__ starts, const TW *__restrict__ wq,
                             const TW *__restrict__ wc, int64_t np, double *__restrict__ Q,
                             double *__restrict__ C, double *__restrict__ partials) {
  __shared__ double sh[32];
  double bsum = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    TW aq = 0, ac = 0;
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
          const long long r = at(g, dx ? wrap_p(i, g.nx) : i, dy ? wrap_p(j, g.ny) : j,
                                 dz ? wrap_p(k, g.nz) : k);
          const size_t o = (size_t)((dz * 2 + dy) * 2 + dx) * np;
          const int32_t s0 = starts[r], e0 = starts[r + 1];
          for (int32_t s = s0; s < e0; ++s) {
            aq += wq[o + s];
            ac += wc[o + s];
          }
        }
    const double qd = ff_widen(aq);
    Q[c] = qd;
    C[c] = ff_widen(ac);
    bsum += qd;
  }
  double b = block_sum(bsum, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// Mixed path, the same deposit in two passes without the per-particle corner
// weights.  Pass 1, per source cell r (the round-indexed cell of its
// particles): every particle's eight corner weights
// ((fx[dx] fy[dy]) fz[dz], the operation order of k_cic_weights2) and their
// products with its heat rate are summed over the cell's particles in slot
// order into 8 + 8 corner sums of r.  Pass 2, per target cell c: the corner
// sums of the 8 cells r = c + (dx, dy, dz) in corner order.  Deterministic;
// the sums associate per corner first.
__global__ void k_dep_corners(Grid g, const int32_t *__restrict__ starts,
                              const int32_t *__restrict__ perm, const float *__restrict__ pay,
                              int64_t np, float *__restrict__ sums) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.n;
       r += (long long)gridDim.x * blockDim.x) {
    float sq[8], sc[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) sq[o] = sc[o] = 0.f;
    const int32_t s0 = starts[r], e0 = starts[r + 1];
    for (int32_t s = s0; s < e0; ++s) {
      const int32_t p = perm[s];
      const float xl = pay[p], yl = pay[np + p], zl = pay[2 * np + p];
      const float rt = pay[3 * np + p];
      const float fx[2] = {xl, 1 - xl}, fy[2] = {yl, 1 - yl}, fz[2] = {zl, 1 - zl};
#pragma unroll
      for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
          const float fxy = fx[dx] * fy[dy];
#pragma unroll
          for (int dz = 0; dz < 2; ++dz) {
            const int o = (dz * 2 + dy) * 2 + dx;
            const float v = fxy * fz[dz];
            sc[o] += v;
            sq[o] += v * rt;
          }
        }
    }
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      sums[(size_t)o * g.n + r] = sq[o];
      sums[(size_t)(8 + o) * g.n + r] = sc[o];
    }
  }
}

__global__ void k_dep_gather8(Grid g, const float *__restrict__ sums, double *__restrict__ Q,
                              double *__restrict__ C, double *__restrict__ partials) {
  __shared__ double sh[32];
  double bsum = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    float aq = 0.f, ac = 0.f;
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx) {
          const long long r = at(g, dx ? wrap_p(i, g.nx) : i, dy ? wrap_p(j, g.ny) : j,
                                 dz ? wrap_p(k, g.nz) : k);
          const int o = (dz * 2 + dy) * 2 + dx;
          aq += sums[(size_t)o * g.n + r];
          ac += sums[(size_t)(8 + o) * g.n + r];
        }
    const double qd = ff_f2d(aq);
    Q[c] = qd;
    C[c] = ff_f2d(ac);
    bsum += qd;
  }
  double b = block_sum(bsum, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// Mixed path, the two-way momentum deposit in two passes without the sorted
// payload copy.  Pass 1, per source cell r (the cell of its particles at
// x_int): the six payload components (lower and upper weight times the
// momentum source, per axis) summed over the cell's particles in slot order.
// Pass 2, per face: face d of cell c takes the upper sum of cell c - e_d plus
// the lower sum of cell c (the order of k_dep_momentum).
__global__ void k_dep_mom_cells(Grid g, const int32_t *__restrict__ starts,
                                const int32_t *__restrict__ perm, const float *__restrict__ pay,
                                int64_t np, float *__restrict__ sums) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.n;
       r += (long long)gridDim.x * blockDim.x) {
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int32_t s0 = starts[r], e0 = starts[r + 1];
    for (int32_t s = s0; s < e0; ++s) {
      const int32_t p = perm[s];
#pragma unroll
      for (int f = 0; f < 6; ++f) acc[f] += pay[f * np + p];
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) sums[(size_t)f * g.n + r] = acc[f];
  }
}

__global__ void k_dep_mom_faces(Grid g, const float *__restrict__ sums, float *__restrict__ Fp) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const long long m[3] = {at(g, wrap_m(i, g.nx), j, k), at(g, i, wrap_m(j, g.ny), k),
                            at(g, i, j, wrap_m(k, g.nz))};
#pragma unroll
    for (int d = 0; d < 3; ++d)
      Fp[d * g.n + c] = sums[(size_t)(2 * d + 1) * g.n + m[d]] + sums[(size_t)(2 * d) * g.n + c];
  }
}

// The two mixed deposits in one z-marching pass each over whole 32 x 8 cell
// tiles (the sums of a plane of source cells kept in shared memory instead of
// written to and read back from HBM: 64 B + 64 B per cell for the heat and
// concentration corners, 24 B + 24 B for the momentum), with the arithmetic
// of the two-pass kernels above in the same order, so the same bits.  A block
// takes work items (tile, chunk of kDepZ planes) blockIdx.x, + gridDim.x, ...;
// the grid is at most one resident wave and kRedBlocks blocks (the heat
// deposit's per-block sums of Q feed the P0 update).  Every source cell of a
// plane (the tile and its halo) has its own thread, which walks its column of
// source cells down the chunk with the loads of the next plane's cell range
// and first particle in flight while the current plane is summed (the chain
// starts -> perm -> payload would otherwise be paid in full at every plane).
constexpr int kDX = 32, kDY = 8, kDepZ = 16, kDepThreads = 320;

// A thread's column of source cells: the index range [s0, e0) of plane m's
// cell and its first particle p0, with plane m + 1's range and first particle
// and plane m + 2's range in flight.
struct SrcColumn {
  int32_t s0 = 0, e0 = 0, p0 = 0, s1 = 0, e1 = 0, p1 = 0, s2 = 0, e2 = 0;
  __device__ __forceinline__ void range(const int32_t *__restrict__ starts, long long r,
                                        int32_t &a, int32_t &b) {
    a = starts[r];
    b = starts[r + 1];
  }
};

// the 8 + 8 corner sums of a source cell (particles [s0, e0), the first p0)
// in slot order (k_dep_corners)
__device__ __forceinline__ void corner_sums(const int32_t *__restrict__ perm,
                                            const float *__restrict__ pay, int64_t np, int32_t s0,
                                            int32_t e0, int32_t p0, float sq[8], float sc[8]) {
#pragma unroll
  for (int o = 0; o < 8; ++o) sq[o] = sc[o] = 0.f;
  for (int32_t s = s0; s < e0; ++s) {
    const int32_t p = s == s0 ? p0 : perm[s];
    const float xl = pay[p], yl = pay[np + p], zl = pay[2 * np + p];
    const float rt = pay[3 * np + p];
    const float fx[2] = {xl, 1 - xl}, fy[2] = {yl, 1 - yl}, fz[2] = {zl, 1 - zl};
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const float fxy = fx[dx] * fy[dy];
#pragma unroll
        for (int dz = 0; dz < 2; ++dz) {
          const int o = (dz * 2 + dy) * 2 + dx;
          const float v = fxy * fz[dz];
          sc[o] += v;
          sq[o] += v * rt;
        }
      }
  }
}

// Heat rate and concentration (k_dep_corners + k_dep_gather8): target cell
// (i, j, k) adds the corners o = dz*4 + dy*2 + dx of source cells (i + dx,
// j + dy, k + dz), o = 0..3 when source plane k is formed and 4..7 when plane
// k + 1 is.  Threads 0-255 own the tile's cells (sources and targets),
// threads 256-296 the sources of its upper x column and y row.
__global__ void __launch_bounds__(kDepThreads)
k_dep_heat_zm(Grid g, const int32_t *__restrict__ starts, const int32_t *__restrict__ perm,
              const float *__restrict__ pay, int64_t np, double *__restrict__ Q,
              double *__restrict__ C, double *__restrict__ partials) {
  __shared__ float S[16][kDY + 1][kDX + 1];
  __shared__ double sh[32];
  const int tid = threadIdx.x, tx = tid % kDX, ty = tid / kDX;
  const bool tgt = tid < kDX * kDY, src = tid < kDX * kDY + kDY + kDX + 1;
  // this thread's source cell in the tile's (kDX + 1) x (kDY + 1) plane
  const int h = tid - kDX * kDY;
  const int sx = tgt ? tx : (h < kDY ? kDX : h - kDY), sy = tgt ? ty : (h < kDY ? h : kDY);
  const int tilesx = g.nx / kDX, tilesy = g.ny / kDY, chunks = (g.nz + kDepZ - 1) / kDepZ;
  const int items = tilesx * tilesy * chunks;
  double bsum = 0;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int bx = w % tilesx, by = (w / tilesx) % tilesy, bz = w / (tilesx * tilesy);
    const int i0 = bx * kDX, j0 = by * kDY, k0 = bz * kDepZ, k1 = min(k0 + kDepZ, g.nz);
    const int is = i0 + sx == g.nx ? 0 : i0 + sx, js = j0 + sy == g.ny ? 0 : j0 + sy;
    auto cell = [&](int m) { return at(g, is, js, m >= g.nz ? m - g.nz : m); };
    SrcColumn q;
    if (src) {
      q.range(starts, cell(k0), q.s0, q.e0);
      if (k0 + 1 <= k1) q.range(starts, cell(k0 + 1), q.s1, q.e1);
      if (q.s0 < q.e0) q.p0 = perm[q.s0];
    }
    float aq = 0.f, ac = 0.f;
    for (int m = k0; m <= k1; ++m) {
      if (src) {  // in flight: plane m + 1's first particle, plane m + 2's range
        q.p1 = q.s1 < q.e1 ? perm[q.s1] : 0;
        q.s2 = q.e2 = 0;
        if (m + 2 <= k1) q.range(starts, cell(m + 2), q.s2, q.e2);
        float sq[8], sc[8];
        corner_sums(perm, pay, np, q.s0, q.e0, q.p0, sq, sc);
#pragma unroll
        for (int o = 0; o < 8; ++o) {
          S[o][sy][sx] = sq[o];
          S[8 + o][sy][sx] = sc[o];
        }
      }
      __syncthreads();
      if (tgt && m > k0) {  // target plane m - 1: the corners of source plane m (dz = 1)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
          for (int dx = 0; dx < 2; ++dx) {
            const int o = (2 + dy) * 2 + dx;
            aq += S[o][ty + dy][tx + dx];
            ac += S[8 + o][ty + dy][tx + dx];
          }
        const long long c = at(g, i0 + tx, j0 + ty, m - 1);
        const double qd = ff_f2d(aq);
        Q[c] = qd;
        C[c] = ff_f2d(ac);
        bsum += qd;
      }
      if (tgt && m < k1) {  // target plane m: the corners of source plane m (dz = 0)
        aq = 0.f;
        ac = 0.f;
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
          for (int dx = 0; dx < 2; ++dx) {
            const int o = dy * 2 + dx;
            aq += S[o][ty + dy][tx + dx];
            ac += S[8 + o][ty + dy][tx + dx];
          }
      }
      q.s0 = q.s1; q.e0 = q.e1; q.p0 = q.p1; q.s1 = q.s2; q.e1 = q.e2;
      __syncthreads();  // (the plane's sums are rewritten next)
    }
  }
  const double b = block_sum(bsum, sh);
  if (tid == 0) partials[blockIdx.x] = b;
}

// Two-way momentum source on the faces (k_dep_mom_cells + k_dep_mom_faces):
// face d of cell c takes the upper sum of cell c - e_d plus the lower sum of
// cell c.  Threads 0-255 own the tile's cells; threads 256-263 form the upper
// x sums of the column below the tile in x and threads 264-295 the upper y
// sums of the row below it in y, through shared memory; the upper z sum of a
// thread's own cell stays in a register for the plane above.  The walk starts
// one plane below the chunk (that plane's upper z sums).
__global__ void __launch_bounds__(kDepThreads)
k_dep_mom_zm(Grid g, const int32_t *__restrict__ starts, const int32_t *__restrict__ perm,
             const float *__restrict__ pay, int64_t np, float *__restrict__ Fp) {
  __shared__ float hxs[kDY][kDX + 1], hys[kDY + 1][kDX];
  const int tid = threadIdx.x, tx = tid % kDX, ty = tid / kDX;
  const bool own = tid < kDX * kDY, src = tid < kDX * kDY + kDY + kDX;
  const int h = tid - kDX * kDY;
  const int tilesx = g.nx / kDX, tilesy = g.ny / kDY, chunks = (g.nz + kDepZ - 1) / kDepZ;
  const int items = tilesx * tilesy * chunks;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int bx = w % tilesx, by = (w / tilesx) % tilesy, bz = w / (tilesx * tilesy);
    const int i0 = bx * kDX, j0 = by * kDY, k0 = bz * kDepZ, k1 = min(k0 + kDepZ, g.nz);
    const int il = i0 == 0 ? g.nx - 1 : i0 - 1, jl = j0 == 0 ? g.ny - 1 : j0 - 1;
    const int is = own ? i0 + tx : (h < kDY ? il : i0 + h - kDY);
    const int js = own ? j0 + ty : (h < kDY ? j0 + h : jl);
    const int f1 = h < kDY ? 1 : 3;  // the one sum a halo cell gives
    auto cell = [&](int m) { return at(g, is, js, m < 0 ? m + g.nz : m); };
    SrcColumn q;
    if (src) {
      q.range(starts, cell(k0 - 1), q.s0, q.e0);
      q.range(starts, cell(k0), q.s1, q.e1);
      if (q.s0 < q.e0) q.p0 = perm[q.s0];
    }
    float hz = 0.f;
    for (int m = k0 - 1; m < k1; ++m) {
      float acc[6];
#pragma unroll
      for (int f = 0; f < 6; ++f) acc[f] = 0.f;
      if (src) {
        q.p1 = q.s1 < q.e1 ? perm[q.s1] : 0;
        q.s2 = q.e2 = 0;
        if (m + 2 < k1) q.range(starts, cell(m + 2), q.s2, q.e2);
        if (own) {
          for (int32_t s = q.s0; s < q.e0; ++s) {
            const int32_t p = s == q.s0 ? q.p0 : perm[s];
#pragma unroll
            for (int f = 0; f < 6; ++f) acc[f] += pay[f * np + p];
          }
        } else {
          float a1 = 0.f;
          for (int32_t s = q.s0; s < q.e0; ++s) a1 += pay[f1 * np + (s == q.s0 ? q.p0 : perm[s])];
          acc[f1] = a1;
        }
      }
      q.s0 = q.s1; q.e0 = q.e1; q.p0 = q.p1; q.s1 = q.s2; q.e1 = q.e2;
      if (m < k0) {  // the plane below the chunk: its upper z sums only
        hz = acc[5];
        continue;
      }
      if (own) {
        hxs[ty][tx + 1] = acc[1];
        hys[ty + 1][tx] = acc[3];
      } else if (src) {
        if (h < kDY)
          hxs[h][0] = acc[1];
        else
          hys[0][h - kDY] = acc[3];
      }
      __syncthreads();
      if (own) {
        const long long c = at(g, i0 + tx, j0 + ty, m);
        Fp[c] = hxs[ty][tx] + acc[0];
        Fp[g.n + c] = hys[ty][tx] + acc[2];
        Fp[2 * g.n + c] = hz + acc[4];
        hz = acc[5];
      }
      __syncthreads();  // (the plane's sums are rewritten next)
    }
  }
}

// the fused deposits run on whole tiles with at most kRedBlocks blocks
static bool dep_fused(const tpm_ctx *c) {
  return c->g.nx % kDX == 0 && c->g.ny % kDY == 0 && c->dep_fused;
}
static int dep_blocks(tpm_ctx *c, const void *kernel) {
  const long long items = (long long)(c->g.nx / kDX) * (c->g.ny / kDY) *
                          ((c->g.nz + kDepZ - 1) / kDepZ);
  const int b = wave_blocks(c, kernel, kDepThreads, items * kDepThreads, true);
  return b < 1 ? 1 : b;
}

// wave_blocks for a cell kernel of this file (kThreads per block)
template <typename K>
int cell_waves(tpm_ctx *c, K *kernel, bool reduces) {
  return wave_blocks(c, reinterpret_cast<const void *>(kernel), kThreads, c->g.n, reduces);
}

int pblocks(int64_t np) {
  int64_t b = (np + kThreads - 1) / kThreads;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

// sort `key` into perm / starts (deterministic cell-major, index-minor order)
// with the momentum deposit's scratch set (mom) or the heat deposit's
void sort_by_cell(tpm_ctx *c, const int32_t *key, int32_t *perm, int32_t *starts, bool mom) {
  const long long n = c->g.n;
  int32_t *counts = mom ? c->counts_t : c->counts;
  int32_t *scan_blocks = mom ? c->scan_blocks_t : c->scan_blocks;
  unsigned char *unsorted = mom ? c->unsorted_t : c->unsorted;
  bool &counted = mom ? c->counted_t : c->counted_r;
  if (!counted) {  // (after a push the histogram is already there)
    TPM_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int32_t) * n, c->stream));
    TPM_LAUNCH(c, "sort_hist", k_hist, pblocks(c->np), kThreads, 0, key, c->np, counts);
  }
  counted = false;
  const int nchunks = (int)((n + kScanChunk - 1) / kScanChunk);
  TPM_LAUNCH(c, "sort_scan_reduce", k_scan_reduce, nchunks, kScanThreads, 0, counts, n,
             scan_blocks);
  TPM_LAUNCH(c, "sort_scan_chunks", k_scan_chunks, 1, kScanThreads, 0, scan_blocks, nchunks);
  TPM_LAUNCH(c, "sort_scan_apply", k_scan_apply, nchunks, kScanThreads, 0, counts, n,
             scan_blocks, starts, (int32_t)c->np);
  TPM_LAUNCH(c, "sort_scatter", k_scatter, pblocks(c->np), kThreads, 0, key, c->np, starts,
             counts, perm, unsorted);
  const long long nwords = (n + 15) / 16;
  TPM_LAUNCH(c, "sort_segsort", k_segsort,
             wave_blocks(c, reinterpret_cast<const void *>(k_segsort), kThreads, nwords, false),
             kThreads, 0, nwords, starts, perm, reinterpret_cast<uint4 *>(unsorted),
             &c->dsc->crowded);
}

__global__ void k_iota(int32_t *__restrict__ a, int64_t np) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x)
    a[p] = (int32_t)p;
}

struct ReorderArgs {
  const double *src[7];
  double *d0[7], *d1[7];
  const double *rhs_t, *tau;
  double *rhs_t2, *tau2;
  const int32_t *flag, *pid;
  int32_t *flag2, *pid2;
};

// slot s of the new order takes particle perm[s] of the old one (both copies
// of the base set, the heat rate, the flag, the caller index, the Stokes time)
__global__ void k_reorder(int64_t np, const int32_t *__restrict__ perm, ReorderArgs a) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = perm[s];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      const double v = a.src[q][p];
      a.d0[q][s] = v;
      a.d1[q][s] = v;
    }
    a.rhs_t2[s] = a.rhs_t[p];
    a.flag2[s] = a.flag[p];
    a.pid2[s] = a.pid[p];
    if (a.tau) a.tau2[s] = a.tau[p];
  }
}

// storage slot s <- caller element pid[s], and back
template <typename T>
__global__ void k_from_caller(int64_t np, const int32_t *__restrict__ pid, const T *__restrict__ in,
                              T *__restrict__ out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x)
    out[s] = in[pid[s]];
}
template <typename T>
__global__ void k_to_caller(int64_t np, const int32_t *__restrict__ pid, const T *__restrict__ in,
                            T *__restrict__ out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x)
    out[pid[s]] = in[s];
}

// slot[i]: the storage slot of the caller's particle i (pid inverted)
__global__ void k_slot_of(int64_t np, const int32_t *__restrict__ pid, int32_t *__restrict__ slot) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < np;
       s += (int64_t)gridDim.x * blockDim.x)
    slot[pid[s]] = (int32_t)s;
}

PState pstate(tpm_ctx *c, bool np1_in_base) {
  PState s;
  for (int q = 0; q < 7; ++q) {
    s.b[q] = c->pq[0][q];
    s.in[q] = c->pq[1][q];
    s.np1_in[q] = np1_in_base ? c->pq[0][q] : c->pq[3][q];
    s.np1[q] = c->pq[3][q];
    s.nw[q] = c->pq[2][q];
  }
  for (int d = 0; d < 3; ++d) s.bx[d] = c->pq[0][d];
  return s;
}

}  // namespace

static const double kPre[4] = {0.5, 0.5, 1., 1. / 6.};
static const double kPost[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};

void launch_particle_push(tpm_ctx *c, int s, bool np1_in_base) {
  if (c->np == 0) return;
  PushArgs a;
  a.dtpo = c->p.dt * kPost[s];
  a.dtpr = c->p.dt * kPre[s];
  a.iTp = (c->Tp != 0) ? 1. / c->Tp : 0.0;
  const double pg = (double)(c->p.ParticleGravity != 0);
  a.gp[0] = pg * c->gx;
  a.gp[1] = pg * c->gy;
  a.gp[2] = pg * c->gz;
  a.alpha = 0.25 * c->p.epsilonp * kPi * c->p.Dp * c->p.Dp * c->I0;
  a.iS = 1. / (c->mp * c->p.Cvp);
  a.iTth = c->p.Nu * kPi * c->p.Dp * c->p.k;
  a.stage = s;
  a.twc = c->p.TWC;
  a.has_tau = c->tau != nullptr;
  a.has_gp = a.gp[0] != 0 || a.gp[1] != 0 || a.gp[2] != 0;
  // the two sorts' histograms (the momentum deposit's only with two-way
  // coupling) are counted by the push
  const long long n = c->g.n;
  TPM_CUDA_TRY(cudaMemsetAsync(c->counts, 0, sizeof(int32_t) * n, c->stream));
  if (a.twc) TPM_CUDA_TRY(cudaMemsetAsync(c->counts_t, 0, sizeof(int32_t) * n, c->stream));
  int32_t *cnt_t = a.twc ? c->counts_t : nullptr;
  c->counted_t = a.twc != 0;
  c->counted_r = true;
  if (c->p.precision == TPM_PREC_MIXED)
    TPM_LAUNCH(c, "particle_push", (k_push<float, float>), pblocks(c->np), kThreads, 0, c->g,
               pstate(c, np1_in_base), a, c->np, static_cast<const float *>(nullptr), c->RU_int,
               c->Rho_int, c->Tgas, c->rhs_t, c->tau, c->key_t,
               reinterpret_cast<float *>(c->pay_t), c->key_r,
               reinterpret_cast<float *>(c->pay_r), cnt_t, c->counts);
  else
    TPM_LAUNCH(c, "particle_push", (k_push<double, double>), pblocks(c->np), kThreads, 0, c->g,
               pstate(c, np1_in_base), a, c->np, c->U, nullptr, nullptr, c->Tgas, c->rhs_t, c->tau, c->key_t,
               c->pay_t, c->key_r, c->pay_r, cnt_t, c->counts);
}

// two-way momentum source at x_int (grid.cpp:877)
void particle_deposit_momentum(tpm_ctx *c) {
  const bool mixed = c->p.precision == TPM_PREC_MIXED;
  if (c->np == 0 || !c->p.TWC) {
    if (mixed)
      TPM_CUDA_TRY(cudaMemsetAsync(c->Fp32, 0, sizeof(float) * 3 * c->g.n, c->stream));
    else
      TPM_CUDA_TRY(cudaMemsetAsync(c->Fp, 0, sizeof(double) * 3 * c->g.n, c->stream));
    return;
  }
  sort_by_cell(c, c->key_t, c->perm_t, c->starts_t, true);
  if (mixed && dep_fused(c)) {
    TPM_LAUNCH(c, "deposit_momentum", k_dep_mom_zm,
               dep_blocks(c, reinterpret_cast<const void *>(k_dep_mom_zm)), kDepThreads, 0, c->g,
               c->starts_t, c->perm_t, reinterpret_cast<const float *>(c->pay_t), c->np, c->Fp32);
  } else if (mixed) {
    // (its own scratch: it runs beside the heat deposit)
    TPM_LAUNCH(c, "deposit_momentum_cells", k_dep_mom_cells,
               cell_waves(c, k_dep_mom_cells, false), kThreads, 0,
               c->g, c->starts_t, c->perm_t, reinterpret_cast<const float *>(c->pay_t), c->np,
               c->mom_sums);
    TPM_LAUNCH(c, "deposit_momentum", k_dep_mom_faces, cell_waves(c, k_dep_mom_faces, false),
               kThreads, 0, c->g,
               c->mom_sums, c->Fp32);
  } else {
    TPM_LAUNCH(c, "payload_gather_t", k_gather_payload<double>, pblocks(c->np), kThreads, 0, c->np,
               6, c->perm_t, c->pay_t, c->pay_t_s);
    TPM_LAUNCH(c, "deposit_momentum", (k_dep_momentum<double, double>),
               cell_waves(c, k_dep_momentum<double, double>, false),
               kThreads, 0, c->g, c->starts_t, c->pay_t_s, c->np, c->Fp);
  }
}

// concentration at x_int (grid.cpp:876): the previous substep's heat deposit
// (or the initial one) already summed it at these positions
void particle_deposit_concentration(tpm_ctx *c) {
  if (c->np == 0) {
    TPM_CUDA_TRY(cudaMemsetAsync(c->C, 0, sizeof(double) * c->g.n, c->stream));
    return;
  }
  std::swap(c->C, c->C_next);
}

// sort the round-indexed keys in c->key_r and deposit the heat rate into Q
// and the concentration of these positions into C_next
static void heat_deposit(tpm_ctx *c) {
  const bool mixed = c->p.precision == TPM_PREC_MIXED;
  const bool fused = mixed && dep_fused(c);
  const int nb = fused ? dep_blocks(c, reinterpret_cast<const void *>(k_dep_heat_zm))
                 : mixed ? cell_waves(c, k_dep_gather8, true)
                         : cell_waves(c, k_dep_sum8x2<double>, true);
  sort_by_cell(c, c->key_r, c->perm_r[0], c->starts_r[0], false);
  double *parts = c->partials + kPartQ * kRedBlocks;
  if (fused) {
    TPM_LAUNCH(c, "deposit_heat_conc", k_dep_heat_zm, nb, kDepThreads, 0, c->g, c->starts_r[0],
               c->perm_r[0], reinterpret_cast<const float *>(c->pay_r), c->np, c->Q, c->C_next,
               parts);
  } else if (mixed) {
    TPM_LAUNCH(c, "deposit_corner_sums", k_dep_corners, cell_waves(c, k_dep_corners, false),
               kThreads, 0, c->g, c->starts_r[0], c->perm_r[0],
               reinterpret_cast<const float *>(c->pay_r), c->np, c->corner_sums);
    TPM_LAUNCH(c, "deposit_heat_conc", k_dep_gather8, nb, kThreads, 0, c->g, c->corner_sums,
               c->Q, c->C_next, parts);
  } else {
    double *wq = c->w8, *wc = wq + 8 * (size_t)c->np;
    TPM_LAUNCH(c, "cic_weights", k_cic_weights2<double>, pblocks(c->np), kThreads, 0, c->np,
               c->perm_r[0], c->pay_r, wq, wc);
    TPM_LAUNCH(c, "deposit_heat_conc", k_dep_sum8x2<double>, nb, kThreads, 0, c->g,
               c->starts_r[0], wq, wc, c->np, c->Q, c->C_next, parts);
  }
  c->q_parts = nb;
}

// part2gas_Temp_new at x_new (grid.cpp:886)
void particle_heat(tpm_ctx *c) {
  if (c->np == 0) {
    TPM_CUDA_TRY(cudaMemsetAsync(c->Q, 0, sizeof(double) * c->g.n, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(c->partials + kPartQ * kRedBlocks, 0, sizeof(double) * kRedBlocks,
                                 c->stream));
    return;
  }
  heat_deposit(c);
}

// key and heat payload of the x_int set (FP32 payload for the mixed deposit)
static void launch_cic_payload(tpm_ctx *c, double iTth, int compute_rhs) {
  if (c->p.precision == TPM_PREC_MIXED)
    TPM_LAUNCH(c, "cic_payload", k_cic_payload<float>, pblocks(c->np), kThreads, 0, c->g,
               c->pq[1][0], c->pq[1][1], c->pq[1][2], c->pq[1][6], c->Tgas, iTth, c->np,
               c->rhs_t, c->key_r, reinterpret_cast<float *>(c->pay_r), compute_rhs);
  else
    TPM_LAUNCH(c, "cic_payload", k_cic_payload<double>, pblocks(c->np), kThreads, 0, c->g,
               c->pq[1][0], c->pq[1][1], c->pq[1][2], c->pq[1][6], c->Tgas, iTth, c->np,
               c->rhs_t, c->key_r, c->pay_r, compute_rhs);
}

// grid::Initialize tail (grid.cpp:481-484): T = (P0_int/R)/Rho_int, heat rate
// at x_int and its deposit, plus the concentration at x_int for stage 0.
void particle_init_heat(tpm_ctx *c) {
  TPM_LAUNCH(c, "fill_tgas", k_fill_tgas, cell_blocks(c->g), kThreads, 0, c->g.n, c->Rho_int,
             c->hsc->P0_int / c->R, c->Tgas);
  if (c->np == 0) {
    TPM_CUDA_TRY(cudaMemsetAsync(c->Q, 0, sizeof(double) * c->g.n, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(c->partials + kPartQ * kRedBlocks, 0, sizeof(double) * kRedBlocks,
                                 c->stream));
    return;
  }
  double iTth = c->p.Nu * kPi * c->p.Dp * c->p.k;
  launch_cic_payload(c, iTth, 1);
  heat_deposit(c);
}

void particle_kernels_setup(tpm_ctx *c) {
  // the occupancy of every wave-sized kernel, queried once at creation (not
  // while a step is being captured into a graph)
  cell_waves(c, k_segsort, false);
  cell_waves(c, k_dep_mom_cells, false);
  cell_waves(c, k_dep_mom_faces, false);
  cell_waves(c, k_dep_momentum<double, double>, false);
  cell_waves(c, k_dep_gather8, true);
  cell_waves(c, k_dep_sum8x2<double>, true);
  cell_waves(c, k_dep_corners, false);
  dep_blocks(c, reinterpret_cast<const void *>(k_dep_heat_zm));
  dep_blocks(c, reinterpret_cast<const void *>(k_dep_mom_zm));
}

// Continuation from a caller-held state: the given heat rates at x_int give
// back the caller's RHS_Part_Temp (same sums, same order) and the
// concentration for the first substep.
void particle_resume(tpm_ctx *c) {
  int nb = cell_blocks(c->g);
  if (c->np == 0) {
    TPM_LAUNCH(c, "partial_sums", k_partial_sums, nb, kThreads, 0, c->g.n, c->Q,
               c->partials + kPartQ * kRedBlocks);
    c->q_parts = nb;
    return;
  }
  launch_cic_payload(c, 0.0, 0);
  heat_deposit(c);
}

void particle_reorder(tpm_ctx *c) {
  if (!c->reorder || c->np == 0 || !c->np1_is_base) return;
  ReorderArgs a;
  for (int q = 0; q < 7; ++q) {
    a.src[q] = c->pq[0][q];
    a.d0[q] = c->pq[3][q];
    a.d1[q] = c->pq[2][q];
  }
  a.rhs_t = c->rhs_t; a.rhs_t2 = c->rhs_t2;
  a.tau = c->tau; a.tau2 = c->tau2;
  a.flag = c->flag; a.flag2 = c->flag2;
  a.pid = c->pid; a.pid2 = c->pid2;
  TPM_LAUNCH(c, "particle_reorder", k_reorder, pblocks(c->np), kThreads, 0, c->np, c->perm_r[0],
             a);
  // the small arrays go back in place; the base set and its int copy take the
  // two filled buffers, so that over a step the buffer pointers still only
  // alternate between two states (two captured graphs)
  TPM_CUDA_TRY(cudaMemcpyAsync(c->rhs_t, c->rhs_t2, sizeof(double) * c->np,
                               cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(c->flag, c->flag2, sizeof(int32_t) * c->np,
                               cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(c->pid, c->pid2, sizeof(int32_t) * c->np,
                               cudaMemcpyDeviceToDevice, c->stream));
  if (c->tau)
    TPM_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(c->tau), c->tau2, sizeof(double) * c->np,
                                 cudaMemcpyDeviceToDevice, c->stream));
  for (int q = 0; q < 7; ++q) {
    std::swap(c->pq[0][q], c->pq[3][q]);
    std::swap(c->pq[1][q], c->pq[2][q]);
  }
}

void particles_reorder_init(tpm_ctx *c) {
  if (c->reorder && c->np)
    TPM_LAUNCH(c, "pid_init", k_iota, pblocks(c->np), kThreads, 0, c->pid, c->np);
}

void particles_from_host(tpm_ctx *c, void *dev, const void *host, int elem) {
  if (c->np == 0) return;
  const size_t bytes = (size_t)elem * c->np;
  if (!c->reorder) {
    TPM_CUDA_TRY(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, c->stream));
    return;
  }
  TPM_CUDA_TRY(cudaMemcpyAsync(c->pstage, host, bytes, cudaMemcpyHostToDevice, c->stream));
  if (elem == 8)
    TPM_LAUNCH(c, "from_caller", k_from_caller<double>, pblocks(c->np), kThreads, 0, c->np, c->pid,
               c->pstage, static_cast<double *>(dev));
  else
    TPM_LAUNCH(c, "from_caller", k_from_caller<int32_t>, pblocks(c->np), kThreads, 0, c->np, c->pid,
               reinterpret_cast<const int32_t *>(c->pstage), static_cast<int32_t *>(dev));
}

void particle_state_copy_in(tpm_ctx *c, const double *const *part, const double *rhs_t) {
  if (c->np == 0) return;
  const size_t bytes = sizeof(double) * c->np;
  for (int k = 0; k < kStateArrays; ++k) {
    const double *h = k < 7 ? part[k] : rhs_t;
    double *d = c->reorder ? c->pstage + (size_t)k * c->np : (k < 7 ? c->pq[0][k] : c->rhs_t);
    TPM_CUDA_TRY(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream));
  }
}

// The permutations between the staging slots and storage are gathers, one
// array per pass: the 64 MB source of an 8M-particle array stays in L2 while
// its random reads land, where one pass over all eight arrays (or scattered
// 8-byte stores, each rewriting a partial sector) goes to DRAM for each.
void particle_state_stage_in(tpm_ctx *c) {
  if (c->np == 0 || !c->reorder) return;
  for (int k = 0; k < kStateArrays; ++k)
    TPM_LAUNCH(c, "state_from_caller", k_from_caller<double>, pblocks(c->np), kThreads, 0, c->np,
               c->pid, c->pstage + (size_t)k * c->np, k < 7 ? c->pq[0][k] : c->rhs_t);
}

void particle_state_from_host(tpm_ctx *c, const double *const *part, const double *rhs_t) {
  particle_state_copy_in(c, part, rhs_t);
  particle_state_stage_in(c);
}

void particle_state_index(tpm_ctx *c) {
  if (c->np == 0 || !c->reorder) return;
  TPM_LAUNCH(c, "slot_of", k_slot_of, pblocks(c->np), kThreads, 0, c->np, c->pid, c->slot);
}

void particle_state_stage_out(tpm_ctx *c, double *const *src, const double *rhs_t) {
  if (c->np == 0 || !c->reorder) return;
  for (int k = 0; k < kStateArrays; ++k)  // (slot[i] = s with pid[s] = i: a gather too)
    TPM_LAUNCH(c, "state_to_caller", k_from_caller<double>, pblocks(c->np), kThreads, 0, c->np,
               c->slot, k < 7 ? src[k] : rhs_t, c->pstage + (size_t)k * c->np);
}

void particle_state_copy_out(tpm_ctx *c, double *const *part, double *rhs_t,
                             double *const *src, const double *rhs_t_dev) {
  if (c->np == 0) return;
  const size_t bytes = sizeof(double) * c->np;
  for (int k = 0; k < kStateArrays; ++k) {
    double *h = k < 7 ? part[k] : rhs_t;
    const double *d = c->reorder ? c->pstage + (size_t)k * c->np : (k < 7 ? src[k] : rhs_t_dev);
    TPM_CUDA_TRY(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream));
  }
}

void particles_to_host(tpm_ctx *c, void *host, const void *dev, int elem) {
  if (c->np == 0) return;
  const size_t bytes = (size_t)elem * c->np;
  if (!c->reorder) {
    TPM_CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    return;
  }
  if (elem == 8)
    TPM_LAUNCH(c, "to_caller", k_to_caller<double>, pblocks(c->np), kThreads, 0, c->np, c->pid,
               static_cast<const double *>(dev), c->pstage);
  else
    TPM_LAUNCH(c, "to_caller", k_to_caller<int32_t>, pblocks(c->np), kThreads, 0, c->np, c->pid,
               static_cast<const int32_t *>(dev), reinterpret_cast<int32_t *>(c->pstage));
  // the next transfer reuses pstage: it is enqueued after this copy on the stream
  TPM_CUDA_TRY(cudaMemcpyAsync(host, c->pstage, bytes, cudaMemcpyDeviceToHost, c->stream));
}

void particle_zero_fields(tpm_ctx *c) {
  TPM_CUDA_TRY(cudaMemsetAsync(c->Fp, 0, sizeof(double) * 3 * c->g.n, c->stream));
  if (c->Fp32) TPM_CUDA_TRY(cudaMemsetAsync(c->Fp32, 0, sizeof(float) * 3 * c->g.n, c->stream));
  TPM_CUDA_TRY(cudaMemsetAsync(c->C, 0, sizeof(double) * c->g.n, c->stream));
}

}  // namespace tpm
