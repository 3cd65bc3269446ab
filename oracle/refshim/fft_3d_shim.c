/* fft_3d stand-in (test infrastructure): single-rank implementation of the
 * Sandia fft_3d interface the reference calls (fft_3d.h:173-177, used at
 * poisson.cpp:87,431,453), on top of the oracle FFT in ../offt.c.
 *   - one rank owns the whole box, so the remaps are identities;
 *   - data are x-fastest [nslow][nmid][nfast] complex doubles (FFT_DATA);
 *   - scaled = 0 (as the reference requests) means no normalisation;
 *   - isign = 1 -> forward exp(-i...), isign = -1 -> backward.  The reference
 *     divides by a real, even symbol and keeps the real part, so the sign
 *     convention does not affect its result. */
#include <stdlib.h>

#include "mpi.h"
#define FFT_NONE 1
#include "fft_3d.h"
#include "../offt.h"

struct remap_plan_3d { int unused; };

struct fft_plan_3d *fft_3d_create_plan(MPI_Comm comm, int nfast, int nmid, int nslow,
                                       int in_ilo, int in_ihi, int in_jlo, int in_jhi,
                                       int in_klo, int in_khi, int out_ilo, int out_ihi,
                                       int out_jlo, int out_jhi, int out_klo, int out_khi,
                                       int scaled, int permute, int *nbuf) {
  (void)comm; (void)in_ilo; (void)in_ihi; (void)in_jlo; (void)in_jhi; (void)in_klo;
  (void)in_khi; (void)out_ilo; (void)out_ihi; (void)out_jlo; (void)out_jhi; (void)out_klo;
  (void)out_khi; (void)permute;
  struct fft_plan_3d *p = (struct fft_plan_3d *)calloc(1, sizeof(struct fft_plan_3d));
  p->length1 = nfast;
  p->length2 = nmid;
  p->length3 = nslow;
  p->scaled = scaled;
  *nbuf = nfast * nmid * nslow;
  return p;
}

void fft_3d(FFT_DATA *in, FFT_DATA *out, int isign, struct fft_plan_3d *plan) {
  long n = (long)plan->length1 * plan->length2 * plan->length3;
  if (out != in)
    for (long i = 0; i < n; ++i) out[i] = in[i];
  offt_3d((double *)out, plan->length1, plan->length2, plan->length3, isign == 1 ? -1 : 1);
  if (plan->scaled)
    for (long i = 0; i < n; ++i) { out[i].re /= (double)n; out[i].im /= (double)n; }
}

void fft_3d_destroy_plan(struct fft_plan_3d *plan) { free(plan); }
