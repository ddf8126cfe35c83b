/*****************************************************************************
 *
 *  lgb_coarse.h
 *
 *  Fine -> coarse (x2) restriction of FP32 binary-fluid states
 *  (lgb_coarse.cu).
 *
 *****************************************************************************/

#ifndef LGB_COARSE_H
#define LGB_COARSE_H

#include "lgb_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Full state: coarse f (the reference's f, not pending), phi, u, rho */
int lgbk_restrict_state(const lgbk_dims_t * df, const lgbk_dims_t * dc,
			const float * ff, int pending, const float * phif,
			const float * uf, double rho0, double su, double sneq,
			float * fc, float * phic, float * uc, float * rhoc,
			void * stream);

/* Fields only: out5 = [phi, u (x su), rho] on the coarse lattice */
int lgbk_restrict_fields(const lgbk_dims_t * df, const lgbk_dims_t * dc,
			 const float * phif, const float * uf,
			 const float * rhof, double su, float * out5,
			 void * stream);

#ifdef __cplusplus
}
#endif

#endif
