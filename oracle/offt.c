/* Oracle FFT (TEST INFRASTRUCTURE ONLY).  See offt.h for what it restates. */
#include "offt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OFFT_PI 3.14159265358979323846

struct offt_plan {
  int n;
  int nstages;
  int radix[40];
  double *tw;      /* tw[2m], tw[2m+1] = cos, -sin of 2*pi*m/n (forward) */
  double *work;    /* 2 ping-pong buffers of n complex */
};

offt_plan *offt_plan_create(int n) {
  if (n < 1) return NULL;
  offt_plan *p = (offt_plan *)calloc(1, sizeof(offt_plan));
  int m = n;
  while (m % 4 == 0) { p->radix[p->nstages++] = 4; m /= 4; }
  while (m % 2 == 0) { p->radix[p->nstages++] = 2; m /= 2; }
  while (m % 3 == 0) { p->radix[p->nstages++] = 3; m /= 3; }
  while (m % 5 == 0) { p->radix[p->nstages++] = 5; m /= 5; }
  if (m != 1) { free(p); return NULL; }
  p->n = n;
  p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    double a = 2.0 * OFFT_PI * (double)k / (double)n;
    p->tw[2 * k] = cos(a);
    p->tw[2 * k + 1] = -sin(a);
  }
  p->work = (double *)malloc(sizeof(double) * 4 * (size_t)n);
  return p;
}

void offt_plan_destroy(offt_plan *p) {
  if (!p) return;
  free(p->tw);
  free(p->work);
  free(p);
}

/* One Stockham stage of radix R:  for i in [0, n/R): k = i mod p,
 *   v_t = a[i + t n/R] * w^(k t n/(p R)),  V = DFT_R(v),
 *   b[(i/p) p R + k + u p] = V_u. */
static void stage(const double *a, double *b, int n, int R, int p, const double *tw, int sign) {
  const int m = n / R;
  const int step = n / (p * R);
  const double s3 = 0.86602540378443864676;  /* sin(pi/3) */
  const double c5a = 0.30901699437494742410, c5b = -0.80901699437494742410; /* cos 2pi/5, 4pi/5 */
  const double s5a = 0.95105651629515357212, s5b = 0.58778525229247312917;  /* sin 2pi/5, 4pi/5 */
  for (int i = 0; i < m; ++i) {
    int k = i % p;
    double vr[5], vi[5];
    for (int t = 0; t < R; ++t) {
      double xr = a[2 * (i + t * m)], xi = a[2 * (i + t * m) + 1];
      int e = (k * t * step) % n;
      double wr = tw[2 * e], wi = sign < 0 ? tw[2 * e + 1] : -tw[2 * e + 1];
      vr[t] = xr * wr - xi * wi;
      vi[t] = xr * wi + xi * wr;
    }
    double Vr[5], Vi[5];
    if (R == 2) {
      Vr[0] = vr[0] + vr[1]; Vi[0] = vi[0] + vi[1];
      Vr[1] = vr[0] - vr[1]; Vi[1] = vi[0] - vi[1];
    } else if (R == 4) {
      double ar = vr[0] + vr[2], ai = vi[0] + vi[2];
      double br = vr[0] - vr[2], bi = vi[0] - vi[2];
      double cr = vr[1] + vr[3], ci = vi[1] + vi[3];
      double dr = vr[1] - vr[3], di = vi[1] - vi[3];
      /* multiply d by sign*i */
      double jr = sign < 0 ? di : -di, ji = sign < 0 ? -dr : dr;
      Vr[0] = ar + cr; Vi[0] = ai + ci;
      Vr[2] = ar - cr; Vi[2] = ai - ci;
      Vr[1] = br + jr; Vi[1] = bi + ji;
      Vr[3] = br - jr; Vi[3] = bi - ji;
    } else if (R == 3) {
      double sr = vr[1] + vr[2], si = vi[1] + vi[2];
      double dr = vr[1] - vr[2], di = vi[1] - vi[2];
      double mr = vr[0] - 0.5 * sr, mi = vi[0] - 0.5 * si;
      double s = sign < 0 ? -s3 : s3;  /* imaginary part of w^1 */
      Vr[0] = vr[0] + sr; Vi[0] = vi[0] + si;
      Vr[1] = mr - s * di; Vi[1] = mi + s * dr;
      Vr[2] = mr + s * di; Vi[2] = mi - s * dr;
    } else { /* R == 5 */
      double sa = sign < 0 ? -s5a : s5a, sb = sign < 0 ? -s5b : s5b;
      double t1r = vr[1] + vr[4], t1i = vi[1] + vi[4];
      double t2r = vr[2] + vr[3], t2i = vi[2] + vi[3];
      double d1r = vr[1] - vr[4], d1i = vi[1] - vi[4];
      double d2r = vr[2] - vr[3], d2i = vi[2] - vi[3];
      Vr[0] = vr[0] + t1r + t2r; Vi[0] = vi[0] + t1i + t2i;
      double p1r = vr[0] + c5a * t1r + c5b * t2r, p1i = vi[0] + c5a * t1i + c5b * t2i;
      double p2r = vr[0] + c5b * t1r + c5a * t2r, p2i = vi[0] + c5b * t1i + c5a * t2i;
      double q1r = sa * d1r + sb * d2r, q1i = sa * d1i + sb * d2i;
      double q2r = sb * d1r - sa * d2r, q2i = sb * d1i - sa * d2i;
      Vr[1] = p1r - q1i; Vi[1] = p1i + q1r;
      Vr[4] = p1r + q1i; Vi[4] = p1i - q1r;
      Vr[2] = p2r - q2i; Vi[2] = p2i + q2r;
      Vr[3] = p2r + q2i; Vi[3] = p2i - q2r;
    }
    int j = (i / p) * p * R + k;
    for (int u = 0; u < R; ++u) {
      b[2 * (j + u * p)] = Vr[u];
      b[2 * (j + u * p) + 1] = Vi[u];
    }
  }
}

static void fft_one(offt_plan *pl, double *x, int sign) {
  int n = pl->n;
  double *a = pl->work, *b = pl->work + 2 * n;
  memcpy(a, x, sizeof(double) * 2 * (size_t)n);
  int p = 1;
  for (int s = 0; s < pl->nstages; ++s) {
    stage(a, b, n, pl->radix[s], p, pl->tw, sign);
    p *= pl->radix[s];
    double *t = a; a = b; b = t;
  }
  memcpy(x, a, sizeof(double) * 2 * (size_t)n);
}

void offt_many(offt_plan *p, double *data, long count, long seq_stride, long elem_stride,
               int sign) {
  int n = p->n;
  double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  for (long s = 0; s < count; ++s) {
    double *base = data + 2 * s * seq_stride;
    for (int t = 0; t < n; ++t) {
      tmp[2 * t] = base[2 * t * elem_stride];
      tmp[2 * t + 1] = base[2 * t * elem_stride + 1];
    }
    fft_one(p, tmp, sign);
    for (int t = 0; t < n; ++t) {
      base[2 * t * elem_stride] = tmp[2 * t];
      base[2 * t * elem_stride + 1] = tmp[2 * t + 1];
    }
  }
  free(tmp);
}

void offt_3d(double *data, int nx, int ny, int nz, int sign) {
  offt_plan *px = offt_plan_create(nx), *py = offt_plan_create(ny), *pz = offt_plan_create(nz);
  long nxy = (long)nx * ny;
  /* x: contiguous rows */
  offt_many(px, data, (long)ny * nz, nx, 1, sign);
  /* y: for each z-plane, nx sequences with element stride nx */
  for (int k = 0; k < nz; ++k) offt_many(py, data + 2 * (long)k * nxy, nx, 1, nx, sign);
  /* z: nxy sequences with element stride nxy */
  offt_many(pz, data, nxy, 1, nxy, sign);
  offt_plan_destroy(px);
  offt_plan_destroy(py);
  offt_plan_destroy(pz);
}
