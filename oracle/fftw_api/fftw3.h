/*****************************************************************************
 *
 *  fftw3.h  (test infrastructure: part of the oracle, never shipped)
 *
 *  The five calls of the FFTW3 interface that util/length_from_sk.c of the
 *  reference uses (fftw_malloc, fftw_plan_dft_3d, fftw_execute, fftw_free,
 *  fftw_destroy_plan; util/length_from_sk.c:111-185), so that the
 *  reference's own program compiles unmodified where FFTW3 is not
 *  installed.  The transform behind them is a plain complex DFT in double
 *  precision (fftw_dft.c), with FFTW's definitions: for FFTW_FORWARD
 *  (sign -1), out[k] = sum_j in[j] exp(-2 pi i j.k / n) over a row-major
 *  n0 x n1 x n2 array, unnormalised.
 *
 *  Names, types and constants follow FFTW3's published API (fftw3.h of
 *  FFTW 3.x): fftw_complex is double[2], plans are opaque pointers.
 *
 *****************************************************************************/

#ifndef ORACLE_FFTW3_API_H
#define ORACLE_FFTW3_API_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s * fftw_plan;

#define FFTW_FORWARD  (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE  (0U)
#define FFTW_ESTIMATE (1U << 6)

void * fftw_malloc(size_t n);
void fftw_free(void * p);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex * in,
			   fftw_complex * out, int sign, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);

#ifdef __cplusplus
}
#endif

#endif
