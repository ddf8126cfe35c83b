/*****************************************************************************
 *
 *  lgb_sk.h
 *
 *  Structure factor and domain length (diagnostic between steps).
 *
 *****************************************************************************/

#ifndef LGB_SK_H
#define LGB_SK_H

#include <stddef.h>
#include "lgb_kernels.h"

#define LGBK_SK_NBIN 128
#define LGBK_SK_NMAX 1024

#ifdef __cplusplus
extern "C" {
#endif

/* Sum of |phi(k)|^2 and counts per |k| bin over the half space k_z >= 0;
 * work: lgbk_structure_factor_work_bytes(d) bytes of device memory. */
int lgbk_structure_factor(const lgbk_dims_t * d, int prec, const void * phi,
			  int faithful, void * work, double * sk_host,
			  double * nk_host, void * stream);
size_t lgbk_structure_factor_work_bytes(const lgbk_dims_t * d);

#ifdef __cplusplus
}
#endif

#endif
