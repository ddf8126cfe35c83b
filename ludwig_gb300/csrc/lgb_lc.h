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

/* The same in float, for the reduced-precision kernels (GB300's FP64
 * pipe is slow: no double -> float conversions per site) */
typedef struct lgbk_lc_f_s {
  float a0, q0, gamma, kappa0, kappa1, xi, redshift, rredshift, epsilon;
  float e0[3];
  float coswt;
} lgbk_lc_f_t;

/* float copies of the step scalars (lgbk_lc_step_args_t.fp) */
enum lgbk_lc_fp_index {LGBK_LCF_XI, LGBK_LCF_GAMMA_ROT, LGBK_LCF_RHO0,
		       LGBK_LCF_FSCALE, LGBK_LCF_RFSCALE, LGBK_LCF_FX,
		       LGBK_LCF_FY, LGBK_LCF_FZ, LGBK_LCF_RTAU_SHEAR,
		       LGBK_LCF_RTAU_BULK, LGBK_LCF_N};

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
  float fp[LGBK_LCF_N];                     /* filled by lgbk_lc_args_pack */
  int sites;          /* float forms: 2 for the two-site collision
			 kernel, otherwise one site per thread */
} lgbk_lc_step_args_t;

static inline void lgbk_lc_args_pack(lgbk_lc_step_args_t * a) {
  a->fp[LGBK_LCF_XI] = (float) a->xi;
  a->fp[LGBK_LCF_GAMMA_ROT] = (float) a->gamma_rot;
  a->fp[LGBK_LCF_RHO0] = (float) a->rho0;
  a->fp[LGBK_LCF_FSCALE] = (float) a->fscale;
  a->fp[LGBK_LCF_RFSCALE] = (float) (1.0/a->fscale);
  a->fp[LGBK_LCF_FX] = (float) a->cp.force_global[0];
  a->fp[LGBK_LCF_FY] = (float) a->cp.force_global[1];
  a->fp[LGBK_LCF_FZ] = (float) a->cp.force_global[2];
  a->fp[LGBK_LCF_RTAU_SHEAR] = (float) a->cp.rtau_shear;
  a->fp[LGBK_LCF_RTAU_BULK] = (float) a->cp.rtau_bulk;
}

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
/* out: 3 x nsites = fed, bulk part, gradient part (blue_phase_fbg) */
int lgbk_lc_fbg_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		    const double * q, const double * grad, double * out,
		    void * stream);
int lgbk_be_update_f64(const lgbk_dims_t * d, double xi, double gamma_rot,
		       const uint8_t * status, const double * u,
		       const double * flux, const double * h, double * q,
		       void * stream);

#ifdef __cplusplus
}
#endif

#endif
