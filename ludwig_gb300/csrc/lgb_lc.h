/*****************************************************************************
 *
 *  lgb_lc.h
 *
 *  Launchers of the liquid-crystal kernels (thin C ABI, as lgb_kernels.h).
 *  Q: 5 components (XX, XY, XZ, YY, YZ) x nsites; grad 15 x nsites
 *  ([n][ia]); delsq 5 x nsites; flux: fw, fe, fy, fz of 5 x nsites each.
 *
 *****************************************************************************/

#ifndef LGB_LC_H
#define LGB_LC_H

#include "lgb_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters as used by the kernels (src/blue_phase.h:50-75): epsilon
 * already divided by 12 pi, rredshift = 1/redshift. */
typedef struct lgbk_lc_s {
  double a0, q0, gamma, kappa0, kappa1, xi, redshift, rredshift, epsilon;
  double e0[3];
  double coswt;
} lgbk_lc_t;

/* Arguments of the two-kernel LC step (k_lc_fields, k_lc_update) */
typedef struct lgbk_lc_step_args_s {
  const void * f_in;  void * f_out;
  const void * q_in;  void * q_out;
  const void * u_in;  void * u_out;
  void * rho_out;
  const void * pth;   const void * h;       /* written by k_lc_fields */
  const uint8_t * status;
  double xi, gamma_rot, rho0, fscale;
  lgbk_collide_t cp;
} lgbk_lc_step_args_t;

/* One LC step: fields (P, H into a->pth, a->h) then the update */
int lgbk_lc_step(const lgbk_dims_t * d, int prec, const lgbk_lc_t * p,
		 const lgbk_lc_step_args_t * a, void * stream);
int lgbk_lc_step_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		     const lgbk_lc_step_args_t * a, void * stream);

int lgbk_lc_stress_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		       const double * q, const double * grad,
		       const double * delsq, double * pth, void * stream);
int lgbk_lc_h_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		  const double * q, const double * grad, const double * delsq,
		  double * h, void * stream);
int lgbk_lc_fed_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		    const double * q, const double * grad, double * fed,
		    void * stream);
int lgbk_be_update_f64(const lgbk_dims_t * d, double xi, double gamma_rot,
		       const uint8_t * status, const double * u,
		       const double * flux, const double * h, double * q,
		       void * stream);

#ifdef __cplusplus
}
#endif

#endif
