/*
 * tpm.h - C ABI of the GB300-native RK4 substep of the triply-periodic,
 * low-Mach, particle-laden turbulence solver (libtpm.so).
 *
 * The library replaces the reference's per-operator C++ classes on the hot
 * path: grid's substep sequence (grid.cpp:595-900), the field algebra of
 * tensor0/tensor1 (tensor0.cpp, tensor1.cpp), the Lagrangian particle stage
 * (particle.cpp:58-654) and the FFT pressure projection (poisson.cpp:391-462).
 * One context owns one periodic box resident on one GPU; the reference's MPI
 * halo exchange and particle migration (communicator.cpp:157-373,
 * particle.cpp:150-297,772-846) become periodic index wrap inside the kernels.
 *
 * Conventions
 *  - Every call returns an int status (TPM_OK = 0, negative on error) and
 *    never exits or traps; tpm_last_error() describes the last failure.
 *  - Fields cross the boundary in the reference's file layout
 *    (communicator.cpp:114-155): unghosted global FP64 arrays, C order
 *    [Nz][Ny][Nx] (x fastest); a vector field (tensor1) is the x, y and z
 *    blocks back to back (3*Nx*Ny*Nz doubles).
 *  - Particles cross as SoA host arrays of length np, like the restart files
 *    Restart_Part_{x,y,z,u,v,w,T}.bin (FP64) and Restart_Part_flag.bin (int32)
 *    (particle.cpp:939-989).
 *  - A context is used from one host thread at a time.  Work is queued on
 *    the context's CUDA stream; downloads synchronise.
 */
#ifndef TPM_H
#define TPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TPM_ABI_VERSION 1

/* ---- status codes (the reference has none: void + std::cout + exit(1)) ---- */
enum {
  TPM_OK = 0,
  TPM_ERR_ARG = -1,         /* bad argument / size / id */
  TPM_ERR_CUDA = -2,        /* a CUDA runtime error */
  TPM_ERR_TIMEOUT = -3,     /* a bounded device wait ran out */
  TPM_ERR_NONFINITE = -4,   /* NaN/Inf detected in the state */
  TPM_ERR_UNSUPPORTED = -5, /* option outside the ported path */
  TPM_ERR_STATE = -6,       /* call out of order (e.g. step before initialize) */
  TPM_ERR_NOMEM = -7        /* device allocation failed */
};

/* ---- arithmetic of the substep ---- */
enum {
  TPM_PREC_FP64 = 0,  /* plain FP64 path, parity with the reference */
  TPM_PREC_MIXED = 1  /* FP32 stencils/FFT/particles, FP64 state, means and
                         one FP64 defect-correction projection */
};

/*
 * Run parameters: the fields of the reference's parameter deck
 * (params.h:9-59, read in the token order of params.cpp:23-63) that the
 * substep uses.  Derived constants are computed inside exactly as
 * params.cpp:70-77 does: R=Cp-Cv, P0=Rho0*T0*R, Tp=Rhop*Dp*Dp/(18*Mu0),
 * mp=Rhop*pi*Dp^3/6, N0=(int)(np0*Lx*Ly*Lz).  The "...1"/"...2" pairs switch
 * at T_cur > threshold (params.cpp:80-86).
 */
typedef struct tpm_params {
  int32_t Nx, Ny, Nz;       /* global grid, each a product of 2,3,5; Nx even */
  int32_t precision;        /* TPM_PREC_* */
  double Lx, Ly, Lz;        /* box size */
  double dt, threshold;
  int32_t cooling;          /* params.cpp:35 */
  int32_t Iteration1, Iteration2;
  int32_t TWC;              /* two-way momentum coupling */
  double epsilon;           /* Poisson stop criterion on max|dp| */
  int32_t ParticleGravity;
  int32_t elongated_box;    /* must be 0 (outside the ported path) */
  int32_t solve_for_scalar; /* passive scalar transport (grid.cpp:743-772) */
  int32_t solve_for_vector; /* must be 0 */
  double A1, A2;            /* linear forcing coefficient */
  double Rho0;
  double U0, V0, W0;        /* mean momentum target per component / Rho0 */
  double T0;
  double Mu0, k;            /* viscosity, conductivity */
  double gx1, gy1, gz1, gx2, gy2, gz2;
  double Cp, Cv;
  double np0;               /* particle number density */
  double Dp, Rhop, Cvp, epsilonp, Nu;
  double I01, I02;          /* radiative intensity */
  double D_M;               /* passive-scalar diffusivity (params.h:51) */
  int32_t S1_type;          /* passive-scalar source (params.h:53): 0 = cos(x) source with
                               its mean removed, else -u (mean gradient along x) */
  int32_t Solver;           /* pressure solver (params.h, deck token Solver): 0 = FFT-
                               preconditioned Richardson, stop on max|dp| <= epsilon
                               (poisson.cpp:391-411); 2 = conjugate gradients, stop on
                               ||r||_2/||b||_2 < epsilon as the reference's PCG does
                               (poisson.cpp:214-245), preconditioned here by the
                               constant-coefficient FFT solve instead of BoomerAMG */
} tpm_params;

/* Field identifiers for upload/download.  Vector fields are 3*N doubles. */
enum {
  TPM_FIELD_RU = 0,      /* grid.h:57  rho*u on faces (vector)                 */
  TPM_FIELD_RU_INT,      /* grid.h:58  stage value (vector)                    */
  TPM_FIELD_RU_NEW,      /* grid.h:59  next stage value (vector)               */
  TPM_FIELD_RU_NP1,      /* grid.h:60  next step accumulator (vector)          */
  TPM_FIELD_RHO,         /* grid.h:85  density at centres                      */
  TPM_FIELD_RHO_INT,
  TPM_FIELD_RHO_NEW,
  TPM_FIELD_RHO_NP1,
  TPM_FIELD_P,           /* grid.h:72  hydrodynamic pressure                   */
  TPM_FIELD_C,           /* grid.h:78  particle concentration                  */
  TPM_FIELD_Q,           /* grid.h:98  RHS_Part_Temp, particle heat per cell   */
  TPM_FIELD_FP,          /* part2gas_velocity output: two-way momentum source
                            before the -mp/Vcell factor (vector)               */
  TPM_FIELD_RHS_POIS,    /* grid.h:76  Poisson right-hand side (mean removed)  */
  TPM_FIELD_DIVERGENCE,  /* grid.h:97  thermodynamic divergence constraint     */
  TPM_FIELD_PASSIVE_SCALAR, /* grid.h:66 Passive_Scalar (solve_for_scalar only)  */
  TPM_FIELD_COUNT
};

/* Particle copies (particle.h:61-113). */
enum { TPM_PSET_BASE = 0, TPM_PSET_INT = 1, TPM_PSET_NEW = 2, TPM_PSET_NP1 = 3 };

typedef struct tpm_scalars {
  double P0, P0_int, P0_new, P0_np1; /* grid.h:100-103 */
  double T_cur;                      /* grid.h:106 */
  int64_t num_timestep;              /* grid.h:107 */
  int32_t last_poisson_iterations;   /* poisson.h:74 num_iteration_ */
  int32_t total_poisson_iterations;  /* sum over all solves since create */
  double last_poisson_error;         /* max|dp| of the last iteration */
  double max_abs_div;                /* FP64 post-projection max|div u - divergence|
                                        of the last stage (mixed path only; else -1).
                                        At a step boundary it is evaluated on the first
                                        read after the step (not inside the step); after
                                        a field upload or an operator-level solve it
                                        keeps the last evaluated value */
} tpm_scalars;

typedef struct tpm_ctx tpm_ctx;

int tpm_abi_version(void);

/* Create a context for one box with np particles on the current CUDA device.
 * Rejects options outside the ported path (HYPRE solvers other than the PCG
 * stand-in, passive vector, elongated box) with TPM_ERR_UNSUPPORTED. */
int tpm_create(const tpm_params *params, int64_t np, tpm_ctx **out);
int tpm_destroy(tpm_ctx *ctx);
const char *tpm_last_error(const tpm_ctx *ctx);

/* Fields (reference file layout, see above). */
int tpm_upload_field(tpm_ctx *ctx, int field, const double *host);
int tpm_download_field(tpm_ctx *ctx, int field, double *host);

/* Particles: any pointer may be NULL to skip that quantity (flag too). */
int tpm_upload_particles(tpm_ctx *ctx, int set, const double *x, const double *y,
                         const double *z, const double *u, const double *v, const double *w,
                         const double *T, const int32_t *flag);
int tpm_download_particles(tpm_ctx *ctx, int set, double *x, double *y, double *z, double *u,
                           double *v, double *w, double *T, int32_t *flag);
/* particle.h:113 RHS_T (heat exchange rate, W) */
int tpm_download_particle_rhs_t(tpm_ctx *ctx, double *rhs_t);
int tpm_upload_particle_rhs_t(tpm_ctx *ctx, const double *rhs_t);
/* Optional per-particle momentum relaxation time (extension: the reference has
 * one global Tp, particle.cpp:365).  NULL restores the global Tp. */
int tpm_set_particle_tau(tpm_ctx *ctx, const double *tau);

/* Thermodynamic pressure, time and step counter (Restart_numbers.dat,
 * grid.cpp:232-236). */
int tpm_set_scalars(tpm_ctx *ctx, double P0, double T_cur, int64_t num_timestep);
int tpm_get_scalars(tpm_ctx *ctx, tpm_scalars *out);

/* The step-boundary state in one call each way (one stream synchronisation
 * for the copies): tpm_load_state uploads RU, RU_INT, RHO, P, the base
 * particle set (part[0..6] = x, y, z, u, v, w, T) and its heat rates, sets
 * the scalars and resumes (what tpm_upload_field / tpm_upload_particles /
 * tpm_upload_particle_rhs_t / tpm_set_scalars / tpm_resume do one by one);
 * tpm_save_state downloads the same arrays and the scalars.  The heat deposit
 * Q is rebuilt from the heat rates, and particle ids do not change, so neither
 * is part of it.  A run saved and loaded at every step continues bit for bit. */
int tpm_load_state(tpm_ctx *ctx, const double *RU, const double *RU_int, const double *Rho,
                   const double *P, const double *const *part, const double *rhs_t, double P0,
                   double T_cur, int64_t num_timestep);
int tpm_save_state(tpm_ctx *ctx, double *RU, double *RU_int, double *Rho, double *P,
                   double *const *part, double *rhs_t, tpm_scalars *scalars);

/* tpm_load_state, one tpm_step and tpm_save_state in one call, with the same
 * results bit for bit, the host transfers overlapping the step: the particle
 * state goes up first, then Rho and RU_int while the resume's particle work
 * runs, then RU and P while the first stage's head and particle deposits run;
 * the particles, their heat rates and Rho come down during the last stage's
 * pressure solve, and P, RU_int and RU each as soon as it is final.  The
 * inputs and outputs may be the same arrays (pinned host memory gives the
 * link's full rate).  Steps from a CUDA graph per piece when
 * TPM_OPT_CUDA_GRAPH is on.  (Not in the reference: its state is host memory
 * throughout.) */
int tpm_step_state(tpm_ctx *ctx, const double *RU, const double *RU_int, const double *Rho,
                   const double *P, const double *const *part, const double *rhs_t, double P0,
                   double T_cur, int64_t num_timestep, double *RU_out, double *RU_int_out,
                   double *Rho_out, double *P_out, double *const *part_out, double *rhs_t_out,
                   tpm_scalars *scalars);

/* Restart files in the reference's format, the set its Initial=1 branch reads
 * (grid.cpp:221-238, particle.cpp:939-989): Restart_RU.bin, Restart_Rho.bin,
 * Restart_P.bin (raw FP64, [Nz][Ny][Nx], RU as x,y,z blocks),
 * Restart_Part_{x,y,z,u,v,w,T}.bin (FP64), Restart_Part_flag.bin (int32) and
 * Restart_numbers.dat ("P0 T_cur num_timestep").  tpm_write_restart writes the
 * current base state; tpm_read_restart uploads one, after which tpm_initialize
 * does what the reference does after reading it. */
int tpm_write_restart(tpm_ctx *ctx, const char *dir);
int tpm_read_restart(tpm_ctx *ctx, const char *dir);
/* The dumps of grid::Store / particle::Store_All (grid.cpp:525-592,
 * particle.cpp:848-897) at the current step n: RU_<n>.bin, Rho_<n>.bin, P_<n>.bin,
 * Part_{x,y,z,u,v,w,T,flag}_<n>.bin and numbers_<n>.dat. */
int tpm_store(tpm_ctx *ctx, const char *dir);

/* grid::Initialize tail (grid.cpp:461-484): stage copies, face density and
 * the initial particle heat coupling.  Call after uploading RU, Rho, P,
 * particles and scalars. */
int tpm_initialize(tpm_ctx *ctx);

/* Continue from a step-boundary state held by the caller: after uploading
 * RU, RU_INT, RHO, P and Q (RHS_Part_Temp), the base particle set, the
 * particle heat rates and the scalars, this restores the derived device state
 * (stage copies, deposit sort) so the next tpm_step continues the run exactly
 * where tpm_download_* took it.  (The reference's own restart, grid.cpp:221-238
 * + :461-484, recomputes RU_int and RHS_Part_Temp instead and so does not
 * continue a run bit for bit; tpm_initialize reproduces that.) */
int tpm_resume(tpm_ctx *ctx);

/* One RK4 substep (simulation.cpp:62-77 with Update_Particle enabled):
 * Update_Rho, Update_P0, Update_Particle, Update_RU_WOP, Compute_Div_U_new,
 * Compute_RHS_Pois, Solve_Poisson, Update_RU_WP, TimeAdvance_RK4. */
int tpm_substep(tpm_ctx *ctx, int rk_stage);
/* End of a time step (simulation.cpp:80,91): RU_np1.make_mean_U0, TimeAdvance. */
int tpm_end_step(tpm_ctx *ctx);

/*
 * The reference's grid methods one by one, for a time loop kept in the shape
 * of simulation.cpp:58-91 (include/tpm_grid.hpp wraps them in a C++ class
 * with the reference's names).  Each queues the kernels of one method for RK4
 * stage rk_stage (grid::RK4_count) on the context's stream.  They must come
 * in the reference loop's order - Update_Rho and Update_P0 (either order),
 * Update_Particle, Update_Passive_Scalar (solve_for_scalar only),
 * Update_RU_WOP, Compute_Div_U_new, Compute_RHS_Pois, Solve_Poisson,
 * Update_RU_WP, TimeAdvance_RK4, and after the fourth stage
 * RU_np1.make_mean_U0 and TimeAdvance - with rk_stage the stage the context
 * is at; a call out of that order returns TPM_ERR_STATE and queues nothing.
 * The sequence gives the same bits as tpm_substep / tpm_end_step (which run
 * independent kernels of a stage side by side on a second stream).  Where
 * the GPU path fuses two methods into one pass, the first records its turn
 * and the second queues the pass: the divergence constraint of
 * Compute_Div_U_new is formed by Compute_RHS_Pois's pass, and the gas
 * temperature Update_Particle reads is formed by the density pass, which
 * therefore queues Update_P0's kernel first when Update_P0 has not run yet
 * (P0 does not depend on the density, grid.cpp:816-830).
 */
int tpm_param_update(tpm_ctx *ctx);                 /* PARAM.update(T_cur), params.cpp:80-86 */
int tpm_update_rho(tpm_ctx *ctx, int rk_stage);      /* grid::Update_Rho, grid.cpp:608-614 */
int tpm_update_p0(tpm_ctx *ctx, int rk_stage);       /* grid::Update_P0, grid.cpp:816-830 */
int tpm_update_particle(tpm_ctx *ctx, int rk_stage); /* grid::Update_Particle, grid.cpp:865-888 */
int tpm_update_passive_scalar(tpm_ctx *ctx, int rk_stage); /* grid.cpp:743-772 */
int tpm_update_ru_wop(tpm_ctx *ctx, int rk_stage);   /* grid::Update_RU_WOP, grid.cpp:776-814 */
int tpm_compute_div_u_new(tpm_ctx *ctx, int rk_stage); /* grid.cpp:832-839 */
int tpm_compute_rhs_pois(tpm_ctx *ctx, int rk_stage);  /* grid.cpp:841-849 */
int tpm_solve_poisson(tpm_ctx *ctx, int rk_stage);   /* grid::Solve_Poisson, grid.cpp:851-855 */
int tpm_update_ru_wp(tpm_ctx *ctx, int rk_stage);    /* grid::Update_RU_WP, grid.cpp:857-863 */
int tpm_time_advance_rk4(tpm_ctx *ctx, int rk_stage); /* grid::TimeAdvance_RK4, grid.cpp:890-900 */
int tpm_make_mean_u0(tpm_ctx *ctx);  /* RU_np1.make_mean_U0 (simulation.cpp:80, tensor1.cpp:320-325) */
int tpm_time_advance(tpm_ctx *ctx);  /* grid::TimeAdvance, grid.cpp:595-606 */
/* PARAM.update(T_cur) + 4 substeps + end of step (simulation.cpp:58-91). */
int tpm_step(tpm_ctx *ctx);
int tpm_run(tpm_ctx *ctx, int nsteps);
int tpm_sync(tpm_ctx *ctx);
/* The context's CUDA stream (cudaStream_t), e.g. to record timing events. */
void *tpm_stream(tpm_ctx *ctx);

/* poisson::Solve with Solver==0 (poisson.h:79, poisson.cpp:391-462) on host
 * buffers: div(C grad P) = RHS by Richardson iteration preconditioned with
 * the FFT constant-coefficient solve.  C is a vector field (3N), P holds the
 * initial guess and receives the result.  Uses the context's grid. */
int tpm_poisson_solve(tpm_ctx *ctx, const double *C3, double *P, const double *RHS,
                      int max_iterations, double epsilon, int *iterations_out,
                      double *error_out);

/*
 * Poisson solve that allocates nothing.  This entry point has no counterpart
 * in the reference.  It is for callers that cannot call cudaMalloc: plug-ins
 * handed device buffers by a host application that owns all device memory,
 * or runtimes whose memory pool forbids side allocations.  It solves the same
 * problem as tpm_poisson_solve (the reference's poisson::Solve with
 * Solver==0, stopping as poisson.cpp:397 does: while iterations <
 * max_iterations and max|dp| > epsilon) on DEVICE pointers: C3 (3 face
 * blocks), P (initial guess in, solution out) and RHS, for an Nx*Ny*Nz box of
 * size Lx*Ly*Lz, on `stream` (a cudaStream_t; NULL = legacy default stream).
 * It needs no context and never calls cudaMalloc, cudaFree or any allocating
 * routine: its scratch is one file-scope device array of
 * TPM_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * process exit, which bounds the grid to roughly 100^3 cells; larger grids
 * return TPM_ERR_ARG.  The first call on a device looks up the array's
 * device address and sets kernel attributes.  Each call synchronises
 * `stream` (once, and once per iteration when epsilon > 0, to test the
 * stopping rule), so `stream` must not be capturing a CUDA graph: the call
 * then returns TPM_ERR_STATE and does nothing.  All calls on one GPU share
 * its array: calls that overlap on that GPU (other streams, other host
 * threads) race and must be serialised by the caller; calls on different
 * GPUs may run concurrently.  With max_iterations = 0 it reports error 100,
 * the reference's initial error.
 */
#define TPM_NOALLOC_SCRATCH_BYTES (16u << 20)
int tpm_poisson_solve_noalloc(int Nx, int Ny, int Nz, double Lx, double Ly, double Lz,
                              const double *C3, double *P, const double *RHS,
                              int max_iterations, double epsilon, void *stream,
                              int *iterations_out, double *error_out);

/* Options (tpm_set_option). */
enum {
  TPM_OPT_STORE_DIVERGENCE = 1, /* keep the divergence constraint field for download
                                   (grid.h:97); off by default to save bandwidth */
  TPM_OPT_DIV_RESIDUAL_EVERY_STAGE = 2, /* mixed path: evaluate the FP64 post-projection
                                          divergence residual after every stage, not
                                          only after the last one of each step */
  TPM_OPT_CUDA_GRAPH = 3 /* tpm_step/tpm_run replay each step from a CUDA graph
                            captured on first use (one per distinct host state:
                            the step-copy pointer swaps alternate, so two); the
                            Poisson stopping test then runs on the device.
                            Results are bit-identical to eager stepping.  Not used
                            while profiling is on. */,
  TPM_OPT_FFT_TMA = 4, /* mixed path: the y and z pencil passes take tiles of 8
                         pencils moved by the TMA (1; the default where every
                         pencil has at most 256 points) or plain tiles (0).
                         tpm_autotune may turn either pass's TMA tiles off on a
                         grid where plain tiles are faster.  Results do not
                         depend on it.  (Not in the reference.) */
  TPM_OPT_FUSED_DEPOSITS = 5 /* mixed path on grids of whole 32 x 8 column tiles:
                                the heat/concentration and the momentum deposits
                                each in one z-marching pass with the source
                                cells' sums in shared memory (1, the default) or
                                in two passes through HBM (0).  The same bits.
                                (Not in the reference.) */
};
int tpm_set_option(tpm_ctx *ctx, int option, int value);

/* ---------------------------------------------------------------- diagnostics
 * Statistics of the current step-boundary state, computed on the device.  The
 * first block is grid::Statistics (grid.cpp:902-940), which the reference calls
 * after each step (simulation.cpp:92) and writes to <Stat_dir>/<name>.dat; the
 * names in the comments are those files.  Quantities of the last RK4 stage
 * (TKE2, HT_mean, num_iteration) are those of the step just taken; before the
 * first step they are 0.  The second block is not in the reference. */
typedef struct tpm_stats {
  double T_cur;
  int64_t num_timestep;
  double Rho_mean, Rho_max, Rho_min;  /* Rho_Mean, Rho_Max, Rho_Min */
  double C_mean, C_max, C_min;        /* C_Mean, C_Max, C_Min */
  double TKE2;                 /* RU: U.mean_squares() of the stage-3 velocity
                                  RU_new/Rho_face before projection (grid.cpp:911) */
  double TKE_U, TKE_V, TKE_W;  /* TKE_U/V/W: mean(RU_d/Rho_face_d * RU_d) */
  double TKE;                  /* TKE_U + TKE_V + TKE_W (twice the kinetic energy) */
  double Gas_CFL_Max;          /* Max_CFL_U: max_d max(U_d) dt/d_d, signed max */
  double Gas_Max_Diff_CFL;     /* dt/(dx^2 Rho_min/Mu0)*6 */
  double u_max;                /* max over components of max(U_d) */
  double Vp_max, Tp_max;       /* max of particle u and T (-1e9 with no particles) */
  double Tp_mean;              /* Tp: mean particle temperature */
  double HT_mean;              /* HT: mean(RHS_Part_Temp) used by the stage-3 P0 update */
  double Tg_mean;              /* Tg: mean(P0/R/Rho) */
  double P0;                   /* P0 */
  int32_t num_iteration;       /* Num_Iteration: Poisson iterations of the last solve */
  int32_t reserved;
  /* not computed by the reference */
  double C_var;                /* mean(C^2) - mean(C)^2, particle concentration variance */
  double u_rms;                /* sqrt(mean(u^2+v^2+w^2)/3), u = RU/I_C2F(Rho) */
  double dissipation;          /* 2 (Mu0/Rho0) <S_ij S_ij>, strain rate from the face
                                  velocity with the staggered differences */
  double Passive_Scalar_mean;  /* Passive_Scalar_mean: mean of the squared scalar
                                  (grid.cpp:913); 0 without solve_for_scalar */
} tpm_stats;
int tpm_statistics(tpm_ctx *ctx, tpm_stats *out);

/* Energy spectrum of the face velocity u = RU/I_C2F(Rho): E[s] is the sum of
 * |u_hat(k)|^2/2 (u_hat = DFT/(Nx Ny Nz), all three components) over wave
 * vectors with nint(|k|/dk) = s, dk = min_d 2 pi/L_d, so sum_s E[s] =
 * mean(u^2+v^2+w^2)/2.  tpm_spectrum_shells gives the number of shells and
 * dk; tpm_spectrum needs nshells at least that number. */
int tpm_spectrum_shells(tpm_ctx *ctx, int *nshells, double *dk);
int tpm_spectrum(tpm_ctx *ctx, double *E, int nshells);

/* Radial distribution function of the base particle positions: pairs[b] is
 * the number of unordered pairs with minimum-image distance r in
 * [b dr, (b+1) dr), dr = r_max/nbins; g[b] (optional) is pairs[b] divided by
 * its ideal-gas expectation Np(Np-1)/2 * (4/3)pi((b+1)^3-b^3)dr^3/(Lx Ly Lz).
 * r_max must be at most min_d L_d/3. */
int tpm_rdf(tpm_ctx *ctx, double r_max, int nbins, unsigned long long *pairs, double *g);

/* Discrete adjoint of nsteps RK4 steps from the current state (right after
 * tpm_initialize or tpm_resume), for the unheated, uncooled, gravity-free
 * uniform-density regime (FP64 path; other settings return
 * TPM_ERR_UNSUPPORTED).  Objective at the final step boundary:
 *   J = w_tke * 0.5 * sum_d mean(RU_d^2 / Rho_face_d) + w_cvar * var(C),
 * C the cloud-in-cell concentration of the final particle positions
 * (particle.cpp:522-555 weights).  Outputs (each optional): J; dJ/dRU(0)
 * (3*N doubles on the host, projected on discretely divergence-free fields);
 * dJ/dA (forcing coefficient A1 = A2); dJ/dtau_p (uniform shift of the Stokes
 * time).  Forward states are recomputed from checkpoints taken every
 * checkpoint_every steps.  Returns with the context at the final state, as
 * after tpm_run(ctx, nsteps).  Not in the reference. */
int tpm_adjoint_run(tpm_ctx *ctx, int nsteps, int checkpoint_every, double w_tke, double w_cvar,
                    double *J, double *dJ_dRU0, double *dJ_dA, double *dJ_dtau);

/* Picks the pencils per block and the threads per block of each FFT pass
 * (x, y, z) of the pressure solve by timing Poisson iterations on the
 * context's grid; results do not depend on the choice (each pencil is
 * transformed independently).  The state is kept: P and the device scalars
 * are restored afterwards.  pens_out (6 ints, optional) receives the pencils
 * of the x, y, z passes, then their threads per block. */
int tpm_autotune(tpm_ctx *ctx, int *pens_out);

/* Sets the FFT tiles that tpm_autotune would pick, e.g. ones it picked before
 * for the same grid: tiles[0..2] the pencils per block of the x, y, z passes
 * (powers of two, at most what the passes' shared memory holds), tiles[3..5]
 * their threads per block (multiples of 32, 32..1024).  Results do not depend
 * on the tiles.  TPM_ERR_ARG for values out of range.  Not in the reference. */
int tpm_set_fft_tiles(tpm_ctx *ctx, const int *tiles);

/* ---------------------------------------------------------------- ensembles
 * A batch owns nboxes independent contexts (grids and particle counts may
 * differ; all on the current device).  tpm_batch_run advances every box by
 * nsteps: with use_graph, each step of all boxes is one CUDA graph launch
 * (captured once per distinct state) whose per-box kernel chains run
 * concurrently on the boxes' streams; without, the boxes step one after
 * another, eagerly.  Boxes are loaded, initialised and read through the
 * tpm_ctx API on tpm_batch_box(b, i).  Not in the reference, which runs one
 * box per MPI job. */
typedef struct tpm_batch tpm_batch;
int tpm_batch_create(const tpm_params *params, const int64_t *np, int nboxes, tpm_batch **out);
int tpm_batch_destroy(tpm_batch *b);
const char *tpm_batch_last_error(const tpm_batch *b);
tpm_ctx *tpm_batch_box(tpm_batch *b, int i);
int tpm_batch_autotune(tpm_batch *b);  /* tpm_autotune once per distinct grid shape */
int tpm_batch_run(tpm_batch *b, int nsteps, int use_graph);
int tpm_batch_sync(tpm_batch *b);

/* The FP64 FMA throughput of the current device in TFLOP/s (2 flops per FMA),
 * measured by a kernel of independent FMA chains: the roof of the FP64 path,
 * whose kernels are bound by the FP64 pipe (GB300 issues FP64 at a small
 * fraction of its FP32 rate) rather than by HBM.  For the bench; not in the
 * reference. */
int tpm_measure_fp64_peak(double *tflops);

/* Per-kernel timing with CUDA events on the context stream (for the bench). */
int tpm_profile_enable(tpm_ctx *ctx, int on);
/* Fills names (NUL separated, up to cap bytes), launches and total ms per
 * kernel; returns the number of kernels (or a negative status). */
int tpm_profile_report(tpm_ctx *ctx, char *names, int cap, int *launches, double *total_ms,
                       int max_kernels);
int tpm_profile_reset(tpm_ctx *ctx);
/* Number of kernel launches issued by this context since create.  A graph
 * replay counts the kernels it holds; the body of a captured Poisson loop (a
 * conditional while node, 6 kernels) is counted once per solve although the
 * device runs it once per iteration. */
int64_t tpm_launch_count(const tpm_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* TPM_H */
