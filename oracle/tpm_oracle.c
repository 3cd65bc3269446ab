/*
 * CPU ORACLE - TEST INFRASTRUCTURE ONLY (see tpm_oracle.h).
 *
 * Plain-C restatement of the reference's RK4 substep.  Fields are unghosted,
 * x-fastest, index c = (k*Ny + j)*Nx + i; a neighbour at i-1 / i+1 wraps
 * periodically, which is what the reference's ghost layers plus
 * communicator::SEND_RECV_BLOCKING (communicator.cpp:157-258) amount to on one
 * rank.  Deposits land on wrapped indices, which is what
 * SEND_RECV_BLOCKING_CUM (communicator.cpp:277-366) folds them into.
 * Every expression keeps the reference's evaluation order; the comments cite
 * the line each one restates.  Build with -ffp-contract=off.
 */
#include "tpm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "offt.h"

#define REF_PI 3.141592653589793 /* params.h:5 */

typedef struct { double *x, *y, *z; } vec3;

/* particle quantity q in copy s: base, int, new, np1 (particle.h:61-113) */
enum { QX, QY, QZ, QU, QV, QW, QT, NQ };

struct orc {
  tpm_params p;
  int nx, ny, nz;
  long n;
  double dx, dy, dz, idx, idy, idz, inv_dx, inv_dy, inv_dz, inv_dx2, inv_dy2, inv_dz2;
  double R, Tp, mp, Vcell, xh, yh, zh;
  /* grid state (grid.h:57-98) */
  vec3 RU, RU_int, RU_new, RU_np1, RHS_RU, U, Rho_face, dummy, dummy2;
  vec3 Fp; /* copy of the part2gas_velocity deposit, for inspection */
  double *Rho, *Rho_int, *Rho_new, *Rho_np1, *RHS_Rho, *P, *C, *T, *divergence, *RHS_Pois,
      *RHS_Part_Temp;
  /* poisson scratch (poisson.h:61-62) */
  double *center_coeff, *RHS_new;
  vec3 pdummy;
  double *fft;
  /* particles */
  long np;
  double *q[4][NQ];
  double *RHS_u, *RHS_v, *RHS_w, *RHS_T, *ug, *vg, *wg, *Tg, *tau;
  int32_t *flag;
  /* scalars */
  double P0, P0_int, P0_new, P0_np1, T_cur, dP0_dt;
  int64_t num_timestep;
  int Iteration, n_it, total_it;
  double A, gx, gy, gz, I0, last_err;
  double met;  /* mean_energy_transferred of the last Update_P0 (grid.cpp:818) */
  /* passive scalar (grid.h:64-70), allocated with solve_for_scalar */
  double *PS, *PS_int, *PS_new, *PS_np1, *RHS_PS, *S1;
  vec3 PS_face, ps_tmp;
  int stepped; /* a full step has run since orc_initialize */
};

static const double RK4_pre[4] = {0.5, 0.5, 1., 1. / 6.};   /* grid.cpp:18-21 */
static const double RK4_post[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.}; /* grid.cpp:22-25 */

static double *alloc(long n) { return (double *)calloc((size_t)n, sizeof(double)); }
static vec3 valloc(long n) { vec3 v = {alloc(n), alloc(n), alloc(n)}; return v; }
static void vfree(vec3 v) { free(v.x); free(v.y); free(v.z); }

#define IDX(o, i, j, k) (((long)(k) * (o)->ny + (j)) * (o)->nx + (i))
static inline int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }

/* ------------------------------------------------------------------ create */
orc *orc_create(const tpm_params *p, int64_t np) {
  orc *o = (orc *)calloc(1, sizeof(orc));
  o->p = *p;
  o->nx = p->Nx; o->ny = p->Ny; o->nz = p->Nz;
  o->n = (long)o->nx * o->ny * o->nz;
  /* gridsize.cpp:25-27 */
  o->dx = p->Lx / o->nx; o->dy = p->Ly / o->ny; o->dz = p->Lz / o->nz;
  /* tensor0.cpp:17-22 (tensor0 ctor) */
  o->inv_dx = 1. / o->dx; o->inv_dy = 1. / o->dy; o->inv_dz = 1. / o->dz;
  o->inv_dx2 = 1. / (o->dx * o->dx); o->inv_dy2 = 1. / (o->dy * o->dy);
  o->inv_dz2 = 1. / (o->dz * o->dz);
  /* particle.cpp:19-21 */
  o->idx = 1. / o->dx; o->idy = 1. / o->dy; o->idz = 1. / o->dz;
  /* gridsize.cpp:72-77: upper bounds of the local box (one rank: whole box) */
  o->xh = o->nx * o->dx; o->yh = o->ny * o->dy; o->zh = o->nz * o->dz;
  /* params.cpp:70-73 */
  o->R = p->Cp - p->Cv;
  o->Tp = p->Rhop * p->Dp * p->Dp / (18 * p->Mu0);
  o->mp = p->Rhop * REF_PI * p->Dp * p->Dp * p->Dp / 6.;
  o->Vcell = o->dx * o->dy * o->dz; /* gridsize.h:43 */
  long n = o->n;
  o->RU = valloc(n); o->RU_int = valloc(n); o->RU_new = valloc(n); o->RU_np1 = valloc(n);
  o->RHS_RU = valloc(n); o->U = valloc(n); o->Rho_face = valloc(n); o->Fp = valloc(n);
  o->dummy = valloc(n); o->dummy2 = valloc(n); o->pdummy = valloc(n);
  o->Rho = alloc(n); o->Rho_int = alloc(n); o->Rho_new = alloc(n); o->Rho_np1 = alloc(n);
  o->RHS_Rho = alloc(n); o->P = alloc(n); o->C = alloc(n); o->T = alloc(n);
  o->divergence = alloc(n); o->RHS_Pois = alloc(n); o->RHS_Part_Temp = alloc(n);
  o->center_coeff = alloc(n); o->RHS_new = alloc(n);
  o->fft = alloc(2 * n);
  o->np = np;
  for (int s = 0; s < 4; ++s)
    for (int q = 0; q < NQ; ++q) o->q[s][q] = alloc(np > 0 ? np : 1);
  o->RHS_u = alloc(np + 1); o->RHS_v = alloc(np + 1); o->RHS_w = alloc(np + 1);
  o->RHS_T = alloc(np + 1); o->ug = alloc(np + 1); o->vg = alloc(np + 1);
  o->wg = alloc(np + 1); o->Tg = alloc(np + 1);
  o->flag = (int32_t *)calloc((size_t)np + 1, sizeof(int32_t));
  /* params.cpp:75-82 initial parameter set */
  o->Iteration = p->Iteration1; o->A = p->A1;
  o->gx = p->gx1; o->gy = p->gy1; o->gz = p->gz1; o->I0 = p->I01;
  o->P0 = p->Rho0 * p->T0 * o->R; /* params.cpp:71 */
  if (p->solve_for_scalar) {
    o->PS = alloc(n); o->PS_int = alloc(n); o->PS_new = alloc(n); o->PS_np1 = alloc(n);
    o->RHS_PS = alloc(n); o->S1 = alloc(n);
    o->PS_face = valloc(n); o->ps_tmp = valloc(n);
  }
  return o;
}

void orc_destroy(orc *o) {
  if (!o) return;
  vec3 *vs[] = {&o->RU, &o->RU_int, &o->RU_new, &o->RU_np1, &o->RHS_RU, &o->U, &o->Rho_face, &o->Fp,
                &o->dummy, &o->dummy2, &o->pdummy};
  for (size_t i = 0; i < sizeof(vs) / sizeof(vs[0]); ++i) vfree(*vs[i]);
  if (o->PS) {
    vfree(o->PS_face); vfree(o->ps_tmp);
    free(o->PS); free(o->PS_int); free(o->PS_new); free(o->PS_np1); free(o->RHS_PS); free(o->S1);
  }
  double *ss[] = {o->Rho, o->Rho_int, o->Rho_new, o->Rho_np1, o->RHS_Rho, o->P, o->C, o->T,
                  o->divergence, o->RHS_Pois, o->RHS_Part_Temp, o->center_coeff, o->RHS_new,
                  o->fft, o->RHS_u, o->RHS_v, o->RHS_w, o->RHS_T, o->ug, o->vg, o->wg, o->Tg,
                  o->tau};
  for (size_t i = 0; i < sizeof(ss) / sizeof(ss[0]); ++i) free(ss[i]);
  for (int s = 0; s < 4; ++s)
    for (int q = 0; q < NQ; ++q) free(o->q[s][q]);
  free(o->flag);
  free(o);
}

/* ------------------------------------------------ field algebra (tensor0/1) */
/* Equal_Div_F2C, tensor0.cpp:249-256 with ddx/ddy/ddz_F2C, tensor0.cpp:204-217 */
static void div_f2c(orc *o, vec3 T, double *out) {
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        long c = IDX(o, i, j, k);
        double a = (T.x[IDX(o, wrap(i + 1, o->nx), j, k)] - T.x[c]) * o->inv_dx;
        double b = (T.y[IDX(o, i, wrap(j + 1, o->ny), k)] - T.y[c]) * o->inv_dy;
        double d = (T.z[IDX(o, i, j, wrap(k + 1, o->nz))] - T.z[c]) * o->inv_dz;
        out[c] = a + b + d;
      }
}

/* Equal_Grad_C2F, tensor1.cpp:259-270 with ddx/ddy/ddz_C2F, tensor0.cpp:219-232 */
static void grad_c2f(orc *o, const double *f, vec3 out) {
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        long c = IDX(o, i, j, k);
        out.x[c] = (f[c] - f[IDX(o, wrap(i - 1, o->nx), j, k)]) * o->inv_dx;
        out.y[c] = (f[c] - f[IDX(o, i, wrap(j - 1, o->ny), k)]) * o->inv_dy;
        out.z[c] = (f[c] - f[IDX(o, i, j, wrap(k - 1, o->nz))]) * o->inv_dz;
      }
}

/* Equal_Del2, tensor0.cpp:258-265 with d2dx2/d2dy2/d2dz2, tensor0.cpp:234-247 */
static void del2(orc *o, const double *f, double *out) {
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        long c = IDX(o, i, j, k);
        double a = (f[IDX(o, wrap(i + 1, o->nx), j, k)] - 2 * f[c] +
                    f[IDX(o, wrap(i - 1, o->nx), j, k)]) * o->inv_dx2;
        double b = (f[IDX(o, i, wrap(j + 1, o->ny), k)] - 2 * f[c] +
                    f[IDX(o, i, wrap(j - 1, o->ny), k)]) * o->inv_dy2;
        double d = (f[IDX(o, i, j, wrap(k + 1, o->nz))] - 2 * f[c] +
                    f[IDX(o, i, j, wrap(k - 1, o->nz))]) * o->inv_dz2;
        out[c] = a + b + d;
      }
}

/* Equal_I{x,y,z}_C2F, tensor0.cpp:283-324 with I{x,y,z}_C2F :283-296:
 * out[c] = (f[c] + f[c - e_dir]) * 0.5 */
static void interp_c2f(orc *o, const double *f, double *out, int dir) {
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        long c = IDX(o, i, j, k);
        long m = dir == 0 ? IDX(o, wrap(i - 1, o->nx), j, k)
                 : dir == 1 ? IDX(o, i, wrap(j - 1, o->ny), k)
                            : IDX(o, i, j, wrap(k - 1, o->nz));
        out[c] = (f[c] + f[m]) * 0.5;
      }
}

/* tensor1::Equal_I_C2F, tensor1.cpp:278-283 */
static void interp_c2f_vec(orc *o, const double *f, vec3 out) {
  interp_c2f(o, f, out.x, 0);
  interp_c2f(o, f, out.y, 1);
  interp_c2f(o, f, out.z, 2);
}

/* tensor0::Equal_I_F2C, tensor0.cpp:354-362 with I{x,y,z}_F2C :268-281 */
static void interp_f2c_mean(orc *o, vec3 T, double *out) {
  double OneThird = 1. / 3.;
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        long c = IDX(o, i, j, k);
        double a = (T.x[c] + T.x[IDX(o, wrap(i + 1, o->nx), j, k)]) * 0.5;
        double b = (T.y[c] + T.y[IDX(o, i, wrap(j + 1, o->ny), k)]) * 0.5;
        double d = (T.z[c] + T.z[IDX(o, i, j, wrap(k + 1, o->nz))]) * 0.5;
        out[c] = OneThird * (a + b + d);
      }
}

/* tensor0::sum / mean, tensor0.cpp:364-381: serial sum over i, then j, then k
 * innermost; mean divides by size_tot. */
static double field_mean(orc *o, const double *f) {
  double s = 0;
  for (int i = 0; i < o->nx; ++i)
    for (int j = 0; j < o->ny; ++j)
      for (int k = 0; k < o->nz; ++k) s += f[IDX(o, i, j, k)];
  return s / (double)(o->nx * o->ny * o->nz);
}

/* tensor0::max_abs, tensor0.cpp:466-477 */
static double field_max_abs(orc *o, const double *f) {
  double m = fabs(f[0]);
  for (int i = 0; i < o->nx; ++i)
    for (int j = 0; j < o->ny; ++j)
      for (int k = 0; k < o->nz; ++k) {
        double a = fabs(f[IDX(o, i, j, k)]);
        if (a > m) m = a;
      }
  return m;
}

/* ------------------------------------------------------------- particles */
/* particle.cpp:106-119 x2i (truncation) with il=0; the array index wraps */
static inline int trunc_idx(double x, double id) { return (int)(x * id); }
/* particle.cpp:121-134 x2i_round (round half away from zero) */
static inline int round_idx(double x, double id) { return (int)(round(x * id)); }

/* gas2part_velocity, particle.cpp:340-360: 1-D linear along each face normal */
static void gas2part_velocity(orc *o, vec3 u) {
  double *x = o->q[1][QX], *y = o->q[1][QY], *z = o->q[1][QZ];
  for (long p = 0; p < o->np; ++p) {
    int ii = trunc_idx(x[p], o->idx), jj = trunc_idx(y[p], o->idy), kk = trunc_idx(z[p], o->idz);
    double xl = (x[p] * o->idx - ((int)(x[p] * o->idx)));
    double yl = (y[p] * o->idy - ((int)(y[p] * o->idy)));
    double zl = (z[p] * o->idz - ((int)(z[p] * o->idz)));
    int i0 = wrap(ii, o->nx), j0 = wrap(jj, o->ny), k0 = wrap(kk, o->nz);
    o->ug[p] = xl * u.x[IDX(o, wrap(ii + 1, o->nx), j0, k0)] + (1 - xl) * u.x[IDX(o, i0, j0, k0)];
    o->vg[p] = yl * u.y[IDX(o, i0, wrap(jj + 1, o->ny), k0)] + (1 - yl) * u.y[IDX(o, i0, j0, k0)];
    o->wg[p] = zl * u.z[IDX(o, i0, j0, wrap(kk + 1, o->nz))] + (1 - zl) * u.z[IDX(o, i0, j0, k0)];
  }
}

/* update_position, particle.cpp:314-338 */
static void update_position(orc *o, int s, double pre, double post) {
  double dt = o->p.dt;
  for (int d = 0; d < 3; ++d) {
    double *np1 = o->q[3][QX + d], *nw = o->q[2][QX + d], *b = o->q[0][QX + d];
    double *ui = o->q[1][QU + d];
    for (long p = 0; p < o->np; ++p) np1[p] += dt * post * ui[p];
    if (s != 3)
      for (long p = 0; p < o->np; ++p) nw[p] = b[p] + dt * pre * ui[p];
    else
      for (long p = 0; p < o->np; ++p) nw[p] = np1[p];
  }
}

/* update_velocity, particle.cpp:362-399 (optionally with a per-particle
 * relaxation time: an extension, the reference has one global Tp) */
static void update_velocity(orc *o, int s, double pre, double post) {
  double iTp = 0;
  if (o->Tp != 0) iTp = 1. / o->Tp;
  double *gs[3] = {o->ug, o->vg, o->wg};
  double *rhs[3] = {o->RHS_u, o->RHS_v, o->RHS_w};
  for (int d = 0; d < 3; ++d) {
    double *ui = o->q[1][QU + d];
    for (long p = 0; p < o->np; ++p) {
      double it = o->tau ? 1. / o->tau[p] : iTp;
      rhs[d][p] = (gs[d][p] - ui[p]) * it;
    }
  }
  double dt = o->p.dt;
  double g[3] = {o->p.ParticleGravity * o->gx, o->p.ParticleGravity * o->gy,
                 o->p.ParticleGravity * o->gz};
  for (int d = 0; d < 3; ++d) {
    double *np1 = o->q[3][QU + d], *nw = o->q[2][QU + d], *b = o->q[0][QU + d];
    for (long p = 0; p < o->np; ++p) np1[p] += dt * post * (rhs[d][p] + g[d]);
    if (s != 3)
      for (long p = 0; p < o->np; ++p) nw[p] = b[p] + dt * pre * (rhs[d][p] + g[d]);
    else
      for (long p = 0; p < o->np; ++p) nw[p] = np1[p];
  }
}

/* update_Temp, particle.cpp:477-492 */
static void update_temp(orc *o, int s, double pre, double post) {
  double alpha = 0.25 * o->p.epsilonp * REF_PI * o->p.Dp * o->p.Dp * o->I0;
  double dt = o->p.dt;
  double iS = 1. / (o->mp * o->p.Cvp);
  double *np1 = o->q[3][QT], *nw = o->q[2][QT], *b = o->q[0][QT];
  for (long p = 0; p < o->np; ++p) np1[p] += dt * post * iS * (o->RHS_T[p] + alpha);
  if (s != 3)
    for (long p = 0; p < o->np; ++p) nw[p] = b[p] + dt * pre * iS * (o->RHS_T[p] + alpha);
  else
    for (long p = 0; p < o->np; ++p) nw[p] = np1[p];
}

/* cell-centre stencil of the round-indexed linear weights used by
 * part2gas_concentration (particle.cpp:522-555), gas2part_Temp_* (:402-456)
 * and part2gas_Temp_* (:582-654) */
typedef struct { long c[8]; double xl, yl, zl; } cic;
static inline cic cic_of(orc *o, double x, double y, double z) {
  cic r;
  int ii = round_idx(x, o->idx), jj = round_idx(y, o->idy), kk = round_idx(z, o->idz);
  r.xl = x * o->idx - ii + 0.5;
  r.yl = y * o->idy - jj + 0.5;
  r.zl = z * o->idz - kk + 0.5;
  int i1 = wrap(ii, o->nx), i0 = wrap(ii - 1, o->nx);
  int j1 = wrap(jj, o->ny), j0 = wrap(jj - 1, o->ny);
  int k1 = wrap(kk, o->nz), k0 = wrap(kk - 1, o->nz);
  /* order of the reference's eight terms */
  r.c[0] = IDX(o, i1, j1, k1);
  r.c[1] = IDX(o, i0, j1, k1);
  r.c[2] = IDX(o, i1, j0, k1);
  r.c[3] = IDX(o, i1, j1, k0);
  r.c[4] = IDX(o, i0, j0, k1);
  r.c[5] = IDX(o, i0, j1, k0);
  r.c[6] = IDX(o, i1, j0, k0);
  r.c[7] = IDX(o, i0, j0, k0);
  return r;
}

/* gas2part_Temp_int / _new, particle.cpp:402-456 (set 1 = x_int, 2 = x_new) */
static void gas2part_temp(orc *o, int set, const double *T) {
  double *x = o->q[set][QX], *y = o->q[set][QY], *z = o->q[set][QZ];
  for (long p = 0; p < o->np; ++p) {
    cic w = cic_of(o, x[p], y[p], z[p]);
    double xl = w.xl, yl = w.yl, zl = w.zl;
    o->Tg[p] = xl * yl * zl * T[w.c[0]] +
               (1 - xl) * yl * zl * T[w.c[1]] + xl * (1 - yl) * zl * T[w.c[2]] +
               xl * yl * (1 - zl) * T[w.c[3]] +
               (1 - xl) * (1 - yl) * zl * T[w.c[4]] + (1 - xl) * yl * (1 - zl) * T[w.c[5]] +
               xl * (yl - 1) * (zl - 1) * T[w.c[6]] +
               (1 - xl) * (1 - yl) * (1 - zl) * T[w.c[7]];
  }
}

/* Compute_RHS_Temp_int / _new, particle.cpp:460-474 */
static void compute_rhs_temp(orc *o, int set) {
  double iTth = o->p.Nu * REF_PI * o->p.Dp * o->p.k;
  double *Tp = o->q[set][QT];
  for (long p = 0; p < o->np; ++p) o->RHS_T[p] = (o->Tg[p] - Tp[p]) * iTth;
}

/* part2gas_Temp_int / _new, particle.cpp:582-654 */
static void part2gas_temp(orc *o, int set, double *A) {
  memset(A, 0, sizeof(double) * (size_t)o->n);
  double *x = o->q[set][QX], *y = o->q[set][QY], *z = o->q[set][QZ];
  for (long p = 0; p < o->np; ++p) {
    cic w = cic_of(o, x[p], y[p], z[p]);
    double xl = w.xl, yl = w.yl, zl = w.zl, r = o->RHS_T[p];
    A[w.c[0]] += xl * yl * zl * r;
    A[w.c[1]] += (1 - xl) * yl * zl * r;
    A[w.c[2]] += xl * (1 - yl) * zl * r;
    A[w.c[3]] += xl * yl * (1 - zl) * r;
    A[w.c[4]] += (1 - xl) * (1 - yl) * zl * r;
    A[w.c[5]] += (1 - xl) * yl * (1 - zl) * r;
    A[w.c[6]] += xl * (1 - yl) * (1 - zl) * r;
    A[w.c[7]] += (1 - xl) * (1 - yl) * (1 - zl) * r;
  }
}

/* part2gas_concentration, particle.cpp:522-555 (at x_int) */
static void part2gas_concentration(orc *o, double *A) {
  memset(A, 0, sizeof(double) * (size_t)o->n);
  double *x = o->q[1][QX], *y = o->q[1][QY], *z = o->q[1][QZ];
  for (long p = 0; p < o->np; ++p) {
    cic w = cic_of(o, x[p], y[p], z[p]);
    double xl = w.xl, yl = w.yl, zl = w.zl;
    A[w.c[0]] += (xl * yl * zl);
    A[w.c[1]] += (1 - xl) * yl * zl;
    A[w.c[2]] += xl * (1 - yl) * zl;
    A[w.c[3]] += xl * yl * (1 - zl);
    A[w.c[4]] += (1 - xl) * (1 - yl) * zl;
    A[w.c[5]] += (1 - xl) * yl * (1 - zl);
    A[w.c[6]] += xl * (1 - yl) * (1 - zl);
    A[w.c[7]] += (1 - xl) * (1 - yl) * (1 - zl);
  }
}

/* part2gas_velocity, particle.cpp:494-520 (at x_int; transpose of
 * gas2part_velocity) */
static void part2gas_velocity(orc *o, vec3 A) {
  memset(A.x, 0, sizeof(double) * (size_t)o->n);
  memset(A.y, 0, sizeof(double) * (size_t)o->n);
  memset(A.z, 0, sizeof(double) * (size_t)o->n);
  double *x = o->q[1][QX], *y = o->q[1][QY], *z = o->q[1][QZ];
  for (long p = 0; p < o->np; ++p) {
    int ii = trunc_idx(x[p], o->idx), jj = trunc_idx(y[p], o->idy), kk = trunc_idx(z[p], o->idz);
    double xl = (x[p] * o->idx - ((int)(x[p] * o->idx)));
    double yl = (y[p] * o->idy - ((int)(y[p] * o->idy)));
    double zl = (z[p] * o->idz - ((int)(z[p] * o->idz)));
    int i0 = wrap(ii, o->nx), j0 = wrap(jj, o->ny), k0 = wrap(kk, o->nz);
    A.x[IDX(o, wrap(ii + 1, o->nx), j0, k0)] += xl * o->RHS_u[p];
    A.x[IDX(o, i0, j0, k0)] += (1 - xl) * o->RHS_u[p];
    A.y[IDX(o, i0, wrap(jj + 1, o->ny), k0)] += yl * o->RHS_v[p];
    A.y[IDX(o, i0, j0, k0)] += (1 - yl) * o->RHS_v[p];
    A.z[IDX(o, i0, j0, wrap(kk + 1, o->nz))] += zl * o->RHS_w[p];
    A.z[IDX(o, i0, j0, k0)] += (1 - zl) * o->RHS_w[p];
  }
}

/* Send_Recv on one rank (particle.cpp:841-846 -> SortValidX/Y/Z :150-250 ->
 * MODE_Lx/y/z :58-104): a particle whose x_new leaves [xl, xh] is wrapped by
 * MODE_L, which shifts x_new, x and x_np1 (not x_int) by L. */
static void wrap_particles(orc *o) {
  double L[3] = {o->p.Lx, o->p.Ly, o->p.Lz};
  double hi[3] = {o->xh, o->yh, o->zh};
  for (int d = 0; d < 3; ++d) {
    double *nw = o->q[2][QX + d], *b = o->q[0][QX + d], *np1 = o->q[3][QX + d];
    for (long p = 0; p < o->np; ++p) {
      if (nw[p] > hi[d] || nw[p] < 0) {
        if (nw[p] > L[d]) { nw[p] -= L[d]; b[p] -= L[d]; np1[p] -= L[d]; }
        else if (nw[p] < 0) { nw[p] += L[d]; b[p] += L[d]; np1[p] += L[d]; }
      }
    }
  }
}

/* ---------------------------------------------------------- Poisson (FFT) */
/* poisson::CCP_FFT, poisson.cpp:413-462 */
static void ccp_fft(orc *o, const double *rhs, double *out) {
  double TWO_PI = (2 * 3.141592653589793);
  double Two_PI_Over_Lx = TWO_PI / o->p.Lx;
  double Two_PI_Over_Ly = TWO_PI / o->p.Ly;
  double Two_PI_Over_Lz = TWO_PI / o->p.Lz;
  int nx = o->nx, ny = o->ny, nz = o->nz;
  for (long c = 0; c < o->n; ++c) { o->fft[2 * c] = rhs[c]; o->fft[2 * c + 1] = 0; }
  offt_3d(o->fft, nx, ny, nz, -1);
  double dx2 = 2. / (o->dx * o->dx), dy2 = 2. / (o->dy * o->dy), dz2 = 2. / (o->dz * o->dz);
  long count = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (i + j + k > 0) {
          double ii = ((i < nx / 2) ? i : i - nx) * Two_PI_Over_Lx;
          double jj = ((j < ny / 2) ? j : j - ny) * Two_PI_Over_Ly;
          double kk = ((k < nz / 2) ? k : k - nz) * Two_PI_Over_Lz;
          double mwn = ((dx2) * (1 - cos(ii * o->dx)) + (dy2) * (1 - cos(jj * o->dy)) +
                        (dz2) * (1 - cos(kk * o->dz)));
          o->fft[2 * count + 1] /= mwn;
          o->fft[2 * count] /= mwn;
        }
        count++;
      }
  offt_3d(o->fft, nx, ny, nz, +1);
  double tot = (double)(nx * ny * nz);
  for (long c = 0; c < o->n; ++c) out[c] = (-1) * o->fft[2 * c] / (tot);
}

/* poisson::FFT, poisson.cpp:391-411 */
static int poisson_fft(orc *o, vec3 C, double *P, const double *RHS, int max_it, double eps,
                       double *err_out) {
  interp_f2c_mean(o, C, o->center_coeff);
  for (long c = 0; c < o->n; ++c) o->center_coeff[c] = -1. / o->center_coeff[c];
  int it = 0;
  double error = 100;
  while ((it < max_it) && (error > eps)) {
    grad_c2f(o, P, o->pdummy);
    for (long c = 0; c < o->n; ++c) {
      o->pdummy.x[c] *= C.x[c];
      o->pdummy.y[c] *= C.y[c];
      o->pdummy.z[c] *= C.z[c];
    }
    div_f2c(o, o->pdummy, o->RHS_new);
    for (long c = 0; c < o->n; ++c) o->RHS_new[c] -= RHS[c];
    for (long c = 0; c < o->n; ++c) o->RHS_new[c] *= o->center_coeff[c];
    ccp_fft(o, o->RHS_new, o->pdummy.x);
    for (long c = 0; c < o->n; ++c) P[c] += o->pdummy.x[c];
    error = field_max_abs(o, o->pdummy.x);
    it++;
  }
  if (err_out) *err_out = error;
  return it;
}

int orc_poisson_solve(orc *o, const double *C3, double *P, const double *RHS, int max_it,
                      double eps, double *err_out) {
  vec3 C = {(double *)C3, (double *)C3 + o->n, (double *)C3 + 2 * o->n};
  return poisson_fft(o, C, P, RHS, max_it, eps, err_out);
}

static void vcopy(orc *o, vec3 dst, vec3 src);

/* --------------------------------------------------------- grid operators */
/* grid::Update_Rho, grid.cpp:608-614 */
static void update_rho(orc *o, int s) {
  double dt = o->p.dt;
  div_f2c(o, o->RU_int, o->RHS_Rho);
  double a = -(dt * RK4_post[s]);
  for (long c = 0; c < o->n; ++c) o->Rho_np1[c] += a * o->RHS_Rho[c];
  if (s != 3) {
    double b = -dt * RK4_pre[s];
    for (long c = 0; c < o->n; ++c) o->Rho_new[c] = 1 * o->Rho[c] + b * o->RHS_Rho[c];
  } else {
    memcpy(o->Rho_new, o->Rho_np1, sizeof(double) * (size_t)o->n);
  }
}

/* grid::Update_P0, grid.cpp:816-830 */
static void update_p0(orc *o, int s) {
  double mean_energy_transferred = field_mean(o, o->RHS_Part_Temp);
  o->met = mean_energy_transferred;
  if (o->p.cooling)
    o->dP0_dt = 0;
  else
    o->dP0_dt = -o->R / o->p.Cv * mean_energy_transferred / o->Vcell;
  o->P0_np1 += o->p.dt * RK4_post[s] * o->dP0_dt;
  if (s != 3)
    o->P0_new = o->P0 + o->p.dt * RK4_pre[s] * o->dP0_dt;
  else
    o->P0_new = o->P0_np1;
}

static void vdivide(orc *o, vec3 a, vec3 b, vec3 out) {
  for (long c = 0; c < o->n; ++c) {
    out.x[c] = a.x[c] / b.x[c];
    out.y[c] = a.y[c] / b.y[c];
    out.z[c] = a.z[c] / b.z[c];
  }
}

/* grid::Update_Particle, grid.cpp:865-888 (called at simulation.cpp:64 when
 * the particle stage is enabled) */
static void update_particle(orc *o, int s) {
  vdivide(o, o->RU_int, o->Rho_face, o->U);
  gas2part_velocity(o, o->U);
  update_position(o, s, RK4_pre[s], RK4_post[s]);
  update_velocity(o, s, RK4_pre[s], RK4_post[s]);
  update_temp(o, s, RK4_pre[s], RK4_post[s]);
  part2gas_concentration(o, o->C);
  if (o->p.TWC)
    part2gas_velocity(o, o->RHS_RU);
  else {
    memset(o->RHS_RU.x, 0, sizeof(double) * (size_t)o->n);
    memset(o->RHS_RU.y, 0, sizeof(double) * (size_t)o->n);
    memset(o->RHS_RU.z, 0, sizeof(double) * (size_t)o->n);
  }
  vcopy(o, o->Fp, o->RHS_RU);
  wrap_particles(o);
  double a = o->P0_new / o->R;
  for (long c = 0; c < o->n; ++c) o->T[c] = a / o->Rho_new[c];
  gas2part_temp(o, 2, o->T);
  compute_rhs_temp(o, 2);
  part2gas_temp(o, 2, o->RHS_Part_Temp);
}

/* convective term of one momentum component (grid.cpp:785-801):
 * dummy = I_C2F(U_d); dummy2 = I_d,C2F(RU_int); dummy *= dummy2;
 * out = Div_F2C(dummy) */
static void convection(orc *o, const double *Ud, int d, double *out) {
  interp_c2f_vec(o, Ud, o->dummy);
  interp_c2f(o, o->RU_int.x, o->dummy2.x, d);
  interp_c2f(o, o->RU_int.y, o->dummy2.y, d);
  interp_c2f(o, o->RU_int.z, o->dummy2.z, d);
  for (long c = 0; c < o->n; ++c) {
    o->dummy.x[c] *= o->dummy2.x[c];
    o->dummy.y[c] *= o->dummy2.y[c];
    o->dummy.z[c] *= o->dummy2.z[c];
  }
  div_f2c(o, o->dummy, out);
}

/* grid::Update_RU_WOP, grid.cpp:776-814 */
static void update_ru_wop(orc *o, int s) {
  long n = o->n;
  div_f2c(o, o->U, o->divergence);
  grad_c2f(o, o->divergence, o->dummy2);
  del2(o, o->U.x, o->dummy.x);
  del2(o, o->U.y, o->dummy.y);
  del2(o, o->U.z, o->dummy.z);
  double a = -o->mp / o->Vcell, b = o->p.Mu0 / 3., cc = o->p.Mu0;
  for (long c = 0; c < n; ++c) {
    o->RHS_RU.x[c] = a * o->RHS_RU.x[c] + b * o->dummy2.x[c] + cc * o->dummy.x[c];
    o->RHS_RU.y[c] = a * o->RHS_RU.y[c] + b * o->dummy2.y[c] + cc * o->dummy.y[c];
    o->RHS_RU.z[c] = a * o->RHS_RU.z[c] + b * o->dummy2.z[c] + cc * o->dummy.z[c];
  }
  double *rhs[3] = {o->RHS_RU.x, o->RHS_RU.y, o->RHS_RU.z};
  double *Ud[3] = {o->U.x, o->U.y, o->U.z};
  double *conv = o->RHS_Rho; /* scratch: RHS_Rho is dead until the next Update_Rho */
  for (int d = 0; d < 3; ++d) {
    convection(o, Ud[d], d, conv);
    for (long c = 0; c < n; ++c) rhs[d][c] -= conv[c];
  }
  for (long c = 0; c < n; ++c) {
    o->RHS_RU.x[c] += o->A * o->RU_int.x[c];
    o->RHS_RU.y[c] += o->A * o->RU_int.y[c];
    o->RHS_RU.z[c] += o->A * o->RU_int.z[c];
  }
  for (long c = 0; c < n; ++c) {
    o->Rho_face.x[c] -= o->p.Rho0;
    o->Rho_face.y[c] -= o->p.Rho0;
    o->Rho_face.z[c] -= o->p.Rho0;
  }
  for (long c = 0; c < n; ++c) {
    o->RHS_RU.x[c] += o->Rho_face.x[c] * o->gx;
    o->RHS_RU.y[c] += o->Rho_face.y[c] * o->gy;
    o->RHS_RU.z[c] += o->Rho_face.z[c] * o->gz;
  }
  double dt = o->p.dt;
  double po = dt * RK4_post[s];
  for (long c = 0; c < n; ++c) {
    o->RU_np1.x[c] += po * o->RHS_RU.x[c];
    o->RU_np1.y[c] += po * o->RHS_RU.y[c];
    o->RU_np1.z[c] += po * o->RHS_RU.z[c];
  }
  if (s != 3) {
    double pr = dt * RK4_pre[s];
    for (long c = 0; c < n; ++c) {
      o->RU_new.x[c] = 1 * o->RU.x[c] + pr * o->RHS_RU.x[c];
      o->RU_new.y[c] = 1 * o->RU.y[c] + pr * o->RHS_RU.y[c];
      o->RU_new.z[c] = 1 * o->RU.z[c] + pr * o->RHS_RU.z[c];
    }
  } else {
    memcpy(o->RU_new.x, o->RU_np1.x, sizeof(double) * (size_t)n);
    memcpy(o->RU_new.y, o->RU_np1.y, sizeof(double) * (size_t)n);
    memcpy(o->RU_new.z, o->RU_np1.z, sizeof(double) * (size_t)n);
  }
}

/* grid::Compute_Div_U_new, grid.cpp:832-839 */
static void compute_div_u_new(orc *o) {
  long n = o->n;
  for (long c = 0; c < n; ++c) o->dummy.x[c] = 1. / o->Rho_new[c];
  del2(o, o->dummy.x, o->dummy.y);
  memcpy(o->dummy.z, o->RHS_Part_Temp, sizeof(double) * (size_t)n);
  if (o->p.cooling) {
    double m = field_mean(o, o->dummy.z);
    for (long c = 0; c < n; ++c) o->dummy.z[c] -= m;
  }
  double a = o->p.k / o->p.Cp;
  double b = -o->R / (o->p.Cp * o->P0_new * o->Vcell);
  for (long c = 0; c < n; ++c) o->divergence[c] = a * o->dummy.y[c] + b * o->dummy.z[c];
}

/* grid::Compute_RHS_Pois, grid.cpp:841-849 */
static void compute_rhs_pois(orc *o, int s) {
  long n = o->n;
  interp_c2f_vec(o, o->Rho_new, o->Rho_face);
  vdivide(o, o->RU_new, o->Rho_face, o->U);
  div_f2c(o, o->U, o->RHS_Pois);
  for (long c = 0; c < n; ++c) o->RHS_Pois[c] -= o->divergence[c];
  double f = (1. / (o->p.dt * RK4_pre[s]));
  for (long c = 0; c < n; ++c) o->RHS_Pois[c] *= f;
  double m = field_mean(o, o->RHS_Pois);
  for (long c = 0; c < n; ++c) o->RHS_Pois[c] -= m;
}

/* grid::Solve_Poisson, grid.cpp:851-855 */
static void solve_poisson(orc *o) {
  long n = o->n;
  for (long c = 0; c < n; ++c) {
    o->dummy.x[c] = 1. / o->Rho_face.x[c];
    o->dummy.y[c] = 1. / o->Rho_face.y[c];
    o->dummy.z[c] = 1. / o->Rho_face.z[c];
  }
  o->n_it = poisson_fft(o, o->dummy, o->P, o->RHS_Pois, o->Iteration, o->p.epsilon, &o->last_err);
  o->total_it += o->n_it;
}

/* grid::Update_RU_WP, grid.cpp:857-863 */
static void update_ru_wp(orc *o, int s) {
  long n = o->n;
  grad_c2f(o, o->P, o->dummy);
  double a = -(o->p.dt * RK4_post[s]);
  for (long c = 0; c < n; ++c) {
    o->RU_np1.x[c] += a * o->dummy.x[c];
    o->RU_np1.y[c] += a * o->dummy.y[c];
    o->RU_np1.z[c] += a * o->dummy.z[c];
  }
  if (s != 3) {
    double b = -(o->p.dt * RK4_pre[s]);
    for (long c = 0; c < n; ++c) {
      o->RU_new.x[c] += b * o->dummy.x[c];
      o->RU_new.y[c] += b * o->dummy.y[c];
      o->RU_new.z[c] += b * o->dummy.z[c];
    }
  } else {
    memcpy(o->RU_new.x, o->RU_np1.x, sizeof(double) * (size_t)n);
    memcpy(o->RU_new.y, o->RU_np1.y, sizeof(double) * (size_t)n);
    memcpy(o->RU_new.z, o->RU_np1.z, sizeof(double) * (size_t)n);
  }
}

static void vcopy(orc *o, vec3 dst, vec3 src) {
  memcpy(dst.x, src.x, sizeof(double) * (size_t)o->n);
  memcpy(dst.y, src.y, sizeof(double) * (size_t)o->n);
  memcpy(dst.z, src.z, sizeof(double) * (size_t)o->n);
}
static void pcopy(orc *o, int dst, int src) {
  for (int q = 0; q < NQ; ++q) memcpy(o->q[dst][q], o->q[src][q], sizeof(double) * (size_t)o->np);
}

/* grid::TimeAdvance_RK4, grid.cpp:890-900 */
static void time_advance_rk4(orc *o) {
  memcpy(o->Rho_int, o->Rho_new, sizeof(double) * (size_t)o->n);
  vcopy(o, o->RU_int, o->RU_new);
  o->P0_int = o->P0_new;
  pcopy(o, 1, 2);
  if (o->PS) memcpy(o->PS_int, o->PS_new, sizeof(double) * (size_t)o->n); /* grid.cpp:897 */
}

/* PARAM.update, params.cpp:80-86 */
static void param_update(orc *o) {
  if (o->T_cur > o->p.threshold) {
    o->Iteration = o->p.Iteration2;
    o->A = o->p.A2;
    o->gx = o->p.gx2; o->gy = o->p.gy2; o->gz = o->p.gz2;
    o->I0 = o->p.I02;
  }
}

/* grid::C_Source (grid.cpp:718-741) with scalar_source.h's Scalar_Source
 * (A*cos(k*x), A = k = 1), called with (X, Y, X, T) */
static void c_source(orc *o) {
  for (int k = 0; k < o->nz; ++k)
    for (int j = 0; j < o->ny; ++j)
      for (int i = 0; i < o->nx; ++i) {
        const double X = o->dx / 2. + i * o->dx;
        const double A = 1., kk = 1.;
        o->S1[IDX(o, i, j, k)] = A * cos(kk * X);
      }
}

/* grid::Update_Passive_Scalar, grid.cpp:743-772 */
static void update_passive_scalar(orc *o, int s) {
  const long n = o->n;
  vdivide(o, o->RU_int, o->Rho_face, o->U); /* U = RU_int / Rho_face */
  vec3 d = o->ps_tmp;                       /* dummy = U * Passive_Scalar_face */
  for (long c = 0; c < n; ++c) {
    d.x[c] = o->U.x[c] * o->PS_face.x[c];
    d.y[c] = o->U.y[c] * o->PS_face.y[c];
    d.z[c] = o->U.z[c] * o->PS_face.z[c];
  }
  double *conv = o->RHS_new; /* dummy2.x: poisson scratch, dead here */
  div_f2c(o, d, conv);
  double *diff = o->center_coeff; /* dummy2.y */
  del2(o, o->PS_int, diff);
  c_source(o);
  for (long c = 0; c < n; ++c) o->RHS_PS[c] = o->p.D_M * diff[c] + -1 * conv[c];
  if (!o->p.S1_type) {
    double m = field_mean(o, o->S1);
    for (long c = 0; c < n; ++c) o->S1[c] -= m;
    for (long c = 0; c < n; ++c) o->RHS_PS[c] += o->S1[c];
  } else {
    for (int i = 0; i < o->nx; ++i) /* dummy.x = Ix_F2C(U.x) (tensor0.cpp:268-271) */
      for (int j = 0; j < o->ny; ++j)
        for (int k = 0; k < o->nz; ++k)
          d.x[IDX(o, i, j, k)] = (o->U.x[IDX(o, i, j, k)] + o->U.x[IDX(o, wrap(i + 1, o->nx), j, k)]) * 0.5;
    for (long c = 0; c < n; ++c) o->RHS_PS[c] += -1 * d.x[c];
  }
  const double a = o->p.dt * RK4_post[s];
  for (long c = 0; c < n; ++c) o->PS_np1[c] += a * o->RHS_PS[c];
  if (s != 3) {
    const double b = o->p.dt * RK4_pre[s];
    for (long c = 0; c < n; ++c) o->PS_new[c] = 1 * o->PS[c] + b * o->RHS_PS[c];
  } else {
    memcpy(o->PS_new, o->PS_np1, sizeof(double) * (size_t)n);
  }
  interp_c2f_vec(o, o->PS_new, o->PS_face);
}

void orc_substep(orc *o, int s, int with_particles) {
  update_rho(o, s);
  update_p0(o, s);
  if (with_particles) update_particle(o, s);
  if (o->PS) update_passive_scalar(o, s);
  update_ru_wop(o, s);
  compute_div_u_new(o);
  compute_rhs_pois(o, s);
  solve_poisson(o);
  update_ru_wp(o, s);
  time_advance_rk4(o);
}

/* simulation.cpp:80 (tensor1::make_mean_U0, tensor1.cpp:320-325 ->
 * tensor0.cpp:389-394) and grid::TimeAdvance, grid.cpp:595-606 */
void orc_end_step(orc *o) {
  double RhoU[3] = {o->p.U0 * o->p.Rho0, o->p.V0 * o->p.Rho0, o->p.W0 * o->p.Rho0};
  double *f[3] = {o->RU_np1.x, o->RU_np1.y, o->RU_np1.z};
  for (int d = 0; d < 3; ++d) {
    double m = field_mean(o, f[d]);
    for (long c = 0; c < o->n; ++c) f[d][c] -= m;
    for (long c = 0; c < o->n; ++c) f[d][c] += RhoU[d];
  }
  memcpy(o->Rho, o->Rho_np1, sizeof(double) * (size_t)o->n);
  if (o->PS) memcpy(o->PS, o->PS_np1, sizeof(double) * (size_t)o->n); /* grid.cpp:598 */
  vcopy(o, o->RU, o->RU_np1);
  o->P0 = o->P0_np1;
  pcopy(o, 0, 3);
  o->T_cur += o->p.dt;
  o->num_timestep++;
  o->stepped = 1;
}

void orc_step(orc *o, int with_particles) {
  param_update(o);
  for (int s = 0; s < 4; ++s) orc_substep(o, s, with_particles);
  orc_end_step(o);
}

/* grid::Initialize tail, grid.cpp:461-484 */
void orc_initialize(orc *o) {
  o->stepped = 0;
  if (o->PS) { /* grid.cpp:465-476 */
    memcpy(o->PS_int, o->PS, sizeof(double) * (size_t)o->n);
    memcpy(o->PS_np1, o->PS, sizeof(double) * (size_t)o->n);
    interp_c2f_vec(o, o->PS, o->PS_face);
  }
  vcopy(o, o->RU_int, o->RU);
  vcopy(o, o->RU_np1, o->RU);
  memcpy(o->Rho_int, o->Rho, sizeof(double) * (size_t)o->n);
  memcpy(o->Rho_np1, o->Rho, sizeof(double) * (size_t)o->n);
  o->P0_int = o->P0;
  o->P0_np1 = o->P0;
  interp_c2f_vec(o, o->Rho, o->Rho_face);
  pcopy(o, 1, 0);
  pcopy(o, 3, 0);
  double a = o->P0_int / o->R;
  for (long c = 0; c < o->n; ++c) o->T[c] = a / o->Rho_int[c];
  gas2part_temp(o, 1, o->T);
  compute_rhs_temp(o, 1);
  part2gas_temp(o, 1, o->RHS_Part_Temp);
}

/* ------------------------------------------------------------- accessors */
static double *field_ptr(orc *o, int f, int *nvec) {
  *nvec = 1;
  vec3 *v = NULL;
  switch (f) {
    case TPM_FIELD_RU: v = &o->RU; break;
    case TPM_FIELD_RU_INT: v = &o->RU_int; break;
    case TPM_FIELD_RU_NEW: v = &o->RU_new; break;
    case TPM_FIELD_RU_NP1: v = &o->RU_np1; break;
    case TPM_FIELD_FP: v = &o->Fp; break;
    case TPM_FIELD_RHO: return o->Rho;
    case TPM_FIELD_RHO_INT: return o->Rho_int;
    case TPM_FIELD_RHO_NEW: return o->Rho_new;
    case TPM_FIELD_RHO_NP1: return o->Rho_np1;
    case TPM_FIELD_P: return o->P;
    case TPM_FIELD_C: return o->C;
    case TPM_FIELD_Q: return o->RHS_Part_Temp;
    case TPM_FIELD_RHS_POIS: return o->RHS_Pois;
    case TPM_FIELD_DIVERGENCE: return o->divergence;
    case TPM_FIELD_PASSIVE_SCALAR: return o->PS;
    default: return NULL;
  }
  *nvec = 3;
  return (double *)v;
}

void orc_set_field(orc *o, int f, const double *src) {
  int nv;
  double *p = field_ptr(o, f, &nv);
  if (!p) return;
  if (nv == 1) { memcpy(p, src, sizeof(double) * (size_t)o->n); return; }
  vec3 *v = (vec3 *)p;
  memcpy(v->x, src, sizeof(double) * (size_t)o->n);
  memcpy(v->y, src + o->n, sizeof(double) * (size_t)o->n);
  memcpy(v->z, src + 2 * o->n, sizeof(double) * (size_t)o->n);
}

void orc_get_field(orc *o, int f, double *dst) {
  int nv;
  double *p = field_ptr(o, f, &nv);
  if (!p) return;
  if (nv == 1) { memcpy(dst, p, sizeof(double) * (size_t)o->n); return; }
  vec3 *v = (vec3 *)p;
  memcpy(dst, v->x, sizeof(double) * (size_t)o->n);
  memcpy(dst + o->n, v->y, sizeof(double) * (size_t)o->n);
  memcpy(dst + 2 * o->n, v->z, sizeof(double) * (size_t)o->n);
}

void orc_set_particles(orc *o, int set, const double *x, const double *y, const double *z,
                       const double *u, const double *v, const double *w, const double *T,
                       const int32_t *flag) {
  const double *src[NQ] = {x, y, z, u, v, w, T};
  for (int q = 0; q < NQ; ++q)
    if (src[q]) memcpy(o->q[set][q], src[q], sizeof(double) * (size_t)o->np);
  if (flag) memcpy(o->flag, flag, sizeof(int32_t) * (size_t)o->np);
}

void orc_get_particles(orc *o, int set, double *x, double *y, double *z, double *u, double *v,
                       double *w, double *T, int32_t *flag) {
  double *dst[NQ] = {x, y, z, u, v, w, T};
  for (int q = 0; q < NQ; ++q)
    if (dst[q]) memcpy(dst[q], o->q[set][q], sizeof(double) * (size_t)o->np);
  if (flag) memcpy(flag, o->flag, sizeof(int32_t) * (size_t)o->np);
}

void orc_get_particle_rhs_t(orc *o, double *rhs_t) {
  memcpy(rhs_t, o->RHS_T, sizeof(double) * (size_t)o->np);
}

void orc_set_particle_tau(orc *o, const double *tau) {
  free(o->tau);
  o->tau = NULL;
  if (tau) {
    o->tau = alloc(o->np);
    memcpy(o->tau, tau, sizeof(double) * (size_t)o->np);
  }
}

void orc_set_scalars(orc *o, double P0, double T_cur, int64_t num_timestep) {
  o->P0 = P0;
  o->T_cur = T_cur;
  o->num_timestep = num_timestep;
}

void orc_get_scalars(orc *o, tpm_scalars *s) {
  memset(s, 0, sizeof(*s));
  s->P0 = o->P0; s->P0_int = o->P0_int; s->P0_new = o->P0_new; s->P0_np1 = o->P0_np1;
  s->T_cur = o->T_cur; s->num_timestep = o->num_timestep;
  s->last_poisson_iterations = o->n_it;
  s->total_poisson_iterations = o->total_it;
  s->last_poisson_error = o->last_err;
  s->max_abs_div = -1;
}

/* ------------------------------------------------------------ statistics */
/* tensor0::max / min (tensor0.cpp:453-491): serial scan from the first
 * interior element */
static double field_max(orc *o, const double *f) {
  double m = f[0];
  for (int i = 0; i < o->nx; ++i)
    for (int j = 0; j < o->ny; ++j)
      for (int k = 0; k < o->nz; ++k)
        if (f[IDX(o, i, j, k)] > m) m = f[IDX(o, i, j, k)];
  return m;
}
static double field_min(orc *o, const double *f) {
  double m = f[0];
  for (int i = 0; i < o->nx; ++i)
    for (int j = 0; j < o->ny; ++j)
      for (int k = 0; k < o->nz; ++k)
        if (f[IDX(o, i, j, k)] < m) m = f[IDX(o, i, j, k)];
  return m;
}
/* tensor0::sum_squares (tensor0.cpp:493-504) */
static double field_sum_squares(orc *o, const double *f) {
  double s = 0;
  for (int i = 0; i < o->nx; ++i)
    for (int j = 0; j < o->ny; ++j)
      for (int k = 0; k < o->nz; ++k) s += f[IDX(o, i, j, k)] * f[IDX(o, i, j, k)];
  return s;
}
/* particle::max (particle.cpp:668-684), -1e9 for an empty set */
static double part_max(orc *o, const double *v) {
  if (o->np == 0) return -1e9;
  double m = v[0];
  for (long i = 1; i < o->np; ++i)
    if (v[i] > m) m = v[i];
  return m;
}

/* grid::Statistics (grid.cpp:902-940) on the step-boundary state, without
 * touching the solver state (the reference overwrites U and dummy; with the
 * particle stage on, U is recomputed before its next use, grid.cpp:868).
 * The last three members are extensions: C variance (tensor0::var,
 * tensor0.cpp:516-519), rms velocity, and 2 nu <S:S> with the strain rate of
 * the face velocity from the staggered differences. */
void orc_statistics(orc *o, tpm_stats *s) {
  const long n = o->n;
  const double size_tot = (double)(o->nx * o->ny * o->nz);
  memset(s, 0, sizeof(*s));
  s->T_cur = o->T_cur;
  s->num_timestep = o->num_timestep;
  s->Rho_mean = field_mean(o, o->Rho);
  s->Rho_max = field_max(o, o->Rho);
  s->Rho_min = field_min(o, o->Rho);
  s->C_max = field_max(o, o->C);
  s->C_min = field_min(o, o->C);
  s->C_mean = field_mean(o, o->C);
  /* TKE2 = U.mean_squares() (tensor1.cpp:351-359) of U as the last stage
   * left it (RU_new/Rho_face before projection, grid.cpp:844) */
  s->TKE2 = o->stepped ? (field_sum_squares(o, o->U.x) + field_sum_squares(o, o->U.y) +
                          field_sum_squares(o, o->U.z)) / size_tot
                       : 0.0;
  vec3 V = valloc(n);
  vdivide(o, o->RU_np1, o->Rho_face, V); /* U.Equal_Divide(RU_np1, Rho_face) */
  double mx = field_max(o, V.x) * o->p.dt / o->dx; /* tensor1::max_cfl */
  double my = field_max(o, V.y) * o->p.dt / o->dy;
  double mz = field_max(o, V.z) * o->p.dt / o->dz;
  mx = (my > mx) ? my : mx;
  mx = (mz > mx) ? mz : mx;
  s->Gas_CFL_Max = mx;
  double ux = field_max(o, V.x), uy = field_max(o, V.y), uz = field_max(o, V.z); /* tensor1::max */
  ux = (uy > ux) ? uy : ux;
  ux = (uz > ux) ? uz : ux;
  s->u_max = ux;
  s->Vp_max = part_max(o, o->q[0][QU]);
  s->Tp_max = part_max(o, o->q[0][QT]);
  /* extensions on the same velocity */
  s->u_rms = sqrt((field_sum_squares(o, V.x) + field_sum_squares(o, V.y) +
                   field_sum_squares(o, V.z)) / size_tot / 3.0);
  {
    double ss = 0;
    for (int i = 0; i < o->nx; ++i)
      for (int j = 0; j < o->ny; ++j)
        for (int k = 0; k < o->nz; ++k) {
          const long c = IDX(o, i, j, k);
          const int ip = wrap(i + 1, o->nx), im = wrap(i - 1, o->nx);
          const int jp = wrap(j + 1, o->ny), jm = wrap(j - 1, o->ny);
          const int kp = wrap(k + 1, o->nz), km = wrap(k - 1, o->nz);
          const double sxx = (V.x[IDX(o, ip, j, k)] - V.x[c]) * o->inv_dx;
          const double syy = (V.y[IDX(o, i, jp, k)] - V.y[c]) * o->inv_dy;
          const double szz = (V.z[IDX(o, i, j, kp)] - V.z[c]) * o->inv_dz;
          const double sxy = 0.5 * ((V.x[c] - V.x[IDX(o, i, jm, k)]) * o->inv_dy +
                                    (V.y[c] - V.y[IDX(o, im, j, k)]) * o->inv_dx);
          const double sxz = 0.5 * ((V.x[c] - V.x[IDX(o, i, j, km)]) * o->inv_dz +
                                    (V.z[c] - V.z[IDX(o, im, j, k)]) * o->inv_dx);
          const double syz = 0.5 * ((V.y[c] - V.y[IDX(o, i, j, km)]) * o->inv_dz +
                                    (V.z[c] - V.z[IDX(o, i, jm, k)]) * o->inv_dy);
          ss += sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz);
        }
    s->dissipation = 2.0 * (o->p.Mu0 / o->p.Rho0) * (ss / size_tot);
  }
  for (long c = 0; c < n; ++c) { /* U *= RU_np1 */
    V.x[c] *= o->RU_np1.x[c];
    V.y[c] *= o->RU_np1.y[c];
    V.z[c] *= o->RU_np1.z[c];
  }
  s->TKE_U = field_mean(o, V.x);
  s->TKE_V = field_mean(o, V.y);
  s->TKE_W = field_mean(o, V.z);
  s->TKE = s->TKE_U + s->TKE_V + s->TKE_W;
  s->Gas_Max_Diff_CFL = o->p.dt / (o->dx * o->dx * s->Rho_min / o->p.Mu0) * 6.;
  { /* particle::mean (particle.cpp:700-715) */
    double sum = 0;
    for (long i = 0; i < o->np; ++i) sum += o->q[0][QT][i];
    s->Tp_mean = o->np > 0 ? sum / (double)o->np : 0.0;
  }
  s->HT_mean = o->stepped ? o->met : 0.0;
  { /* dummy.x.Equal_Divide(P0/R, Rho); Tg_mean = dummy.x.mean() */
    const double a = o->P0 / o->R;
    for (long c = 0; c < n; ++c) V.x[c] = a / o->Rho[c];
    s->Tg_mean = field_mean(o, V.x);
  }
  s->P0 = o->P0;
  s->num_iteration = o->stepped ? o->n_it : 0;
  s->C_var = field_sum_squares(o, o->C) / size_tot - s->C_mean * s->C_mean;
  s->Passive_Scalar_mean = o->PS ? field_sum_squares(o, o->PS) / size_tot : 0.0; /* grid.cpp:913 */
  vfree(V);
}

/* Unordered particle pairs by minimum-image distance, all pairs i < j
 * (the O(Np^2) definition the cell-list count on the GPU must equal). */
void orc_rdf_pairs(const double *x, const double *y, const double *z, int64_t np, double Lx,
                   double Ly, double Lz, double r_max, int nbins, uint64_t *pairs) {
  const double hx = 0.5 * Lx, hy = 0.5 * Ly, hz = 0.5 * Lz, r2max = r_max * r_max;
  const double dr = r_max / nbins;
  for (int b = 0; b < nbins; ++b) pairs[b] = 0;
  for (int64_t i = 0; i < np; ++i)
    for (int64_t j = i + 1; j < np; ++j) {
      double dx = x[j] - x[i], dy = y[j] - y[i], dz = z[j] - z[i];
      if (dx > hx) dx -= Lx; else if (dx < -hx) dx += Lx;
      if (dy > hy) dy -= Ly; else if (dy < -hy) dy += Ly;
      if (dz > hz) dz -= Lz; else if (dz < -hz) dz += Lz;
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < r2max) {
        const int b = (int)(sqrt(r2) / dr);
        if (b < nbins) pairs[b]++;
      }
    }
}
