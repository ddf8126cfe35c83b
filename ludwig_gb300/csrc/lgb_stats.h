/*****************************************************************************
 *
 *  lgb_stats.h
 *
 *  Device reductions (FP64, compensated).  Each needs a device scratch
 *  array of LGBK_RED_SCRATCH doubles for the per-block partials and the
 *  final words.
 *
 *****************************************************************************/

#ifndef LGB_STATS_H
#define LGB_STATS_H

#include "lgb_kernels.h"

#define LGBK_RED_BLOCKS  1024
#define LGBK_RED_REC     14                 /* 3*4 Klein words + min + max */
#define LGBK_RED_SCRATCH (LGBK_RED_BLOCKS*LGBK_RED_REC + 16)

#ifdef __cplusplus
extern "C" {
#endif

/* out = {sum, sum of squares, min, max} of n = nsites values */
int lgbk_field_stats(const lgbk_dims_t * d, int prec, const void * a,
		     double * scratch, double out_host[4], void * stream);
/* ncol (1 or 3; 3 in FP64 only) columns a[j*nsites + i] summed over the
 * sites with status 0 (all sites for status NULL): out = {sum_0 ..
 * sum_{ncol-1}, min of column 0, max of column 0} */
int lgbk_masked_cols(const lgbk_dims_t * d, int prec, int ncol, const void * a,
		     const uint8_t * status, double * scratch,
		     double * out_host, void * stream);
/* out = {sum f, sum f c_x, sum f c_y, sum f c_z, min, max of site sums};
 * for shifted storage the sums are of f - w rho0 */
int lgbk_dist_moments(const lgbk_dims_t * d, int prec, const void * f,
		      double scale, double * scratch, double out_host[6],
		      void * stream);
/* out = {total free energy, min, max} */
/* the same from stored FP64 gradients (grad: 3 x nsites) */
int lgbk_symm_fed_total_grad(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			     const double * phi, const double * grad,
			     double * scratch, double out_host[3],
			     void * stream);
int lgbk_symm_fed_total(const lgbk_dims_t * d, int prec,
			const lgbk_symm_t * fe, const void * phi,
			double * scratch, double out_host[3], void * stream);

#ifdef __cplusplus
}
#endif

#endif
