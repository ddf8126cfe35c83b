/*****************************************************************************
 *
 *  fftw_dft.c  (test infrastructure: part of the oracle, never shipped)
 *
 *  A plain implementation of the FFTW3 calls declared in fftw3.h: the 3-d
 *  complex DFT as three passes of direct 1-d DFTs along z, y and x.  Each
 *  1-d DFT of length n uses a table of the n twiddles exp(sign 2 pi i m/n),
 *  m = 0..n-1, each computed once with sin/cos in double from the reduced
 *  angle (j*k mod n), and accumulates in double.  Cost O(N (n0+n1+n2)): a
 *  few seconds at 128^3, which is all the reference's length_from_sk needs.
 *
 *****************************************************************************/

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

struct fftw_plan_s {
  int n[3];
  int sign;
  fftw_complex * in;
  fftw_complex * out;
};

void * fftw_malloc(size_t n) {
  return malloc(n);
}

void fftw_free(void * p) {
  free(p);
}

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex * in,
			   fftw_complex * out, int sign, unsigned flags) {
  (void) flags;
  if (n0 < 1 || n1 < 1 || n2 < 1 || in == NULL || out == NULL) return NULL;
  if (sign != FFTW_FORWARD && sign != FFTW_BACKWARD) return NULL;
  fftw_plan p = (fftw_plan) malloc(sizeof(struct fftw_plan_s));
  if (p == NULL) return NULL;
  p->n[0] = n0;
  p->n[1] = n1;
  p->n[2] = n2;
  p->sign = sign;
  p->in = in;
  p->out = out;
  return p;
}

/* In place 1-d DFTs of length n along one axis: the lines start at
 * base(l) and have element stride `stride` (in complex values). */
static void dft_lines(double * a, int n, long nlines, long stride,
		      long (*base)(long l, const int * n3), const int * n3,
		      int sign) {
  const double two_pi = 6.283185307179586476925286766559;
  double * tw = (double *) malloc(2*sizeof(double)*n);
  if (tw == NULL) abort();
  for (int m = 0; m < n; m++) {
    double t = two_pi*(double) m/(double) n;
    tw[2*m + 0] = cos(t);
    tw[2*m + 1] = sign*sin(t);
  }
  #pragma omp parallel
  {
    double * tmp = (double *) malloc(2*sizeof(double)*n);
    if (tmp == NULL) abort();
    #pragma omp for schedule(static)
    for (long l = 0; l < nlines; l++) {
      double * x = a + 2*base(l, n3);
      for (int k = 0; k < n; k++) {
	double re = 0.0, im = 0.0;
	for (int j = 0; j < n; j++) {
	  int m = (int) (((long) j*k) % n);
	  double xr = x[2*j*stride], xi = x[2*j*stride + 1];
	  re += xr*tw[2*m] - xi*tw[2*m + 1];
	  im += xr*tw[2*m + 1] + xi*tw[2*m];
	}
	tmp[2*k] = re;
	tmp[2*k + 1] = im;
      }
      for (int k = 0; k < n; k++) {
	x[2*k*stride] = tmp[2*k];
	x[2*k*stride + 1] = tmp[2*k + 1];
      }
    }
    free(tmp);
  }
  free(tw);
}

/* line l of each pass: z lines run over (i, j); y lines over (i, k);
 * x lines over (j, k) of the row-major n0 x n1 x n2 array */
static long base_z(long l, const int * n) { return l*n[2]; }
static long base_y(long l, const int * n) {
  long i = l/n[2], k = l % n[2];
  return i*n[1]*n[2] + k;
}
static long base_x(long l, const int * n) { return l; }

void fftw_execute(const fftw_plan p) {
  if (p == NULL) return;
  const int * n = p->n;
  long ntot = (long) n[0]*n[1]*n[2];
  double * a = (double *) p->out;
  if (p->out != p->in) memcpy(p->out, p->in, sizeof(fftw_complex)*ntot);
  dft_lines(a, n[2], (long) n[0]*n[1], 1, base_z, n, p->sign);
  dft_lines(a, n[1], (long) n[0]*n[2], n[2], base_y, n, p->sign);
  dft_lines(a, n[0], (long) n[1]*n[2], (long) n[1]*n[2], base_x, n, p->sign);
}

void fftw_destroy_plan(fftw_plan p) {
  free(p);
}
