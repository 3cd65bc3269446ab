/*
 * CPU ORACLE - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solver's RK4 substep (grid.cpp,
 * tensor0.cpp, tensor1.cpp, particle.cpp, poisson.cpp) used as the checker
 * for the GPU library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it; the GPU library never links or calls it.
 *
 * It works on unghosted periodic arrays (index wrap replaces the reference's
 * ghost layers and halo exchange) and keeps the reference's floating-point
 * operation order, so it reproduces the reference build bit for bit except
 * where the reference's particle array order (changed by its migration
 * swap-remove, particle.cpp:150-297) alters deposition summation order.
 * It is pinned against the reference's own sources compiled here
 * (oracle/Makefile `ref`) by tests/test_oracle_pin.py.
 */
#ifndef TPM_ORACLE_H
#define TPM_ORACLE_H

#include <stdint.h>

#include "tpm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

orc *orc_create(const tpm_params *p, int64_t np);
void orc_destroy(orc *o);

void orc_set_field(orc *o, int field, const double *src);
void orc_get_field(orc *o, int field, double *dst);
void orc_set_particles(orc *o, int set, const double *x, const double *y, const double *z,
                       const double *u, const double *v, const double *w, const double *T,
                       const int32_t *flag);
void orc_get_particles(orc *o, int set, double *x, double *y, double *z, double *u, double *v,
                       double *w, double *T, int32_t *flag);
void orc_get_particle_rhs_t(orc *o, double *rhs_t);
void orc_set_particle_tau(orc *o, const double *tau);
void orc_set_scalars(orc *o, double P0, double T_cur, int64_t num_timestep);
void orc_get_scalars(orc *o, tpm_scalars *s);

void orc_initialize(orc *o);
/* with_particles = 0 reproduces the shipped loop (simulation.cpp:64 commented) */
void orc_substep(orc *o, int rk_stage, int with_particles);
void orc_end_step(orc *o);
void orc_step(orc *o, int with_particles);

/* grid::Statistics (grid.cpp:902-940) plus the extensions of tpm_stats. */
void orc_statistics(orc *o, tpm_stats *s);
/* O(Np^2) pair histogram by minimum-image distance (tpm_rdf's definition). */
void orc_rdf_pairs(const double *x, const double *y, const double *z, int64_t np, double Lx,
                   double Ly, double Lz, double r_max, int nbins, uint64_t *pairs);

/* poisson::Solve (Solver==0) on caller buffers; returns iterations. */
int orc_poisson_solve(orc *o, const double *C3, double *P, const double *RHS, int max_it,
                      double eps, double *err_out);

#ifdef __cplusplus
}
#endif
#endif
