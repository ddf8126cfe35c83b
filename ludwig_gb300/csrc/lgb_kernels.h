/*****************************************************************************
 *
 *  lgb_kernels.h
 *
 *  Thin C ABI between the host-side C library (ludwig_gb.c) and the CUDA
 *  kernels (lgb_*.cu).  Plain pointers to device memory, sizes, parameter
 *  structs and a cudaStream_t passed as void *.  Every launcher returns 0
 *  or a cudaError_t value from the launch.
 *
 *  Device layout of every lattice array: interior sites only (periodic
 *  boundaries are applied by index wrap inside the kernels), one
 *  contiguous plane per component, z fastest:
 *      a[((n*nx + x)*ny + y)*nz + z]
 *
 *****************************************************************************/

#ifndef LGB_KERNELS_H
#define LGB_KERNELS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGB_NVEL 19

typedef struct lgbk_dims_s {
  int nx, ny, nz;
  long long nsites;
} lgbk_dims_t;

/* The fused steps index sites with 32-bit unsigned integers: a lattice
 * (or ensemble box) holds fewer sites than this.  At the smallest storage
 * (108 B per site, FP16) 2^32 sites would need 464 GB. */
#define LGBK_MAX_SITES (1LL << 32)

typedef struct lgbk_symm_s {
  double a, b, kappa;
} lgbk_symm_t;

typedef struct lgbk_collide_s {
  double rtau_shear;
  double rtau_bulk;
  double rtau_ghost[LGB_NVEL];
  double force_global[3];
  int ghosts_zero;               /* 1 if every ghost rtau is exactly 1 */
} lgbk_collide_t;

/* Precision / storage of the fused step */
enum lgbk_prec {
  LGBK_PREC_FP64 = 0,            /* double, reference-exact */
  LGBK_PREC_FP32 = 1,            /* float arithmetic, f stored as f - w rho0 */
  LGBK_PREC_FP16 = 2             /* as FP32, f - w rho0 stored as scaled half */
};

/* Reference-semantics FP64 kernels (one per reference kernel) */
int lgbk_grad7_f64(const lgbk_dims_t * d, int nf, const double * field,
		   double * grad, double * delsq, void * stream);
int lgbk_grad27_f64(const lgbk_dims_t * d, int nf, const double * field,
		    double * grad, double * delsq, void * stream);
int lgbk_symm_stress_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			 const double * phi, const double * grad,
			 const double * delsq, double * pth, void * stream);
int lgbk_symm_mu_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
		     const double * phi, const double * delsq, double * mu,
		     void * stream);
int lgbk_force_div_f64(const lgbk_dims_t * d, const double * pth,
		       double * force, void * stream);
int lgbk_advect_f64(const lgbk_dims_t * d, int order, int nf,
		    const double * field, const double * u, double * fw,
		    double * fe, double * fy, double * fz, void * stream);
int lgbk_advect_upwind_f64(const lgbk_dims_t * d, int nf,
			   const double * field, const double * u,
			   double * fw, double * fe, double * fy, double * fz,
			   void * stream);
int lgbk_ch_flux_mu_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			double mobility, const double * phi,
			const double * delsq, double * fw, double * fe_,
			double * fy, double * fz, void * stream);
int lgbk_flux_no_normal_f64(const lgbk_dims_t * d, int nf,
			    const uint8_t * status, double * fw, double * fe,
			    double * fy, double * fz, void * stream);
int lgbk_ch_update_f64(const lgbk_dims_t * d, const double * fw,
		       const double * fe, const double * fy, const double * fz,
		       double * phi, void * stream);
int lgbk_collide_f64(const lgbk_dims_t * d, const lgbk_collide_t * cp,
		     const uint8_t * status, double * f, const double * force,
		     double * rho, double * u, void * stream);
/* the same after a pending propagation: populations pulled from fpost
 * (post-collision values), results to fout (a second array) */
int lgbk_collide_pull_f64(const lgbk_dims_t * d, const lgbk_collide_t * cp,
			  const uint8_t * status, const double * fpost,
			  double * fout, const double * force, double * rho,
			  double * u, void * stream);
/* dir = +1: fprime_p(x) = f_p(x - c_p) (propagation); dir = -1: inverse */
int lgbk_propagate_f64(const lgbk_dims_t * d, int dir, const double * f,
		       double * fprime, void * stream);
int lgbk_fill_f64(double * a, long long n, double v, void * stream);

/* Fused binary-fluid step (one kernel per step).
 * Input f is the post-collision state of the previous step (its streamed
 * image is the reference's f); output likewise.  force_out may be NULL. */
/* Scalar parameters of the fused step, as doubles (pd) and as floats (pf)
 * so that reduced-precision kernels use them without conversions */
enum lgbk_param_index {
  LGBK_P_RTAU_SHEAR, LGBK_P_RTAU_BULK, LGBK_P_FX, LGBK_P_FY, LGBK_P_FZ,
  LGBK_P_MOBILITY, LGBK_P_RHO0, LGBK_P_FSCALE, LGBK_P_RFSCALE,
  LGBK_P_A, LGBK_P_B, LGBK_P_KAPPA, LGBK_NPARAM
};

typedef struct lgbk_binary_args_s {
  const void * f_in;   void * f_out;
  const void * phi_in; void * phi_out;
  const void * u_in;   void * u_out;
  void * rho_out;
  void * force_out;
  const uint8_t * status;
  double mobility;
  double rho0;
  double fscale;       /* FP16 storage: stored = (f - w rho0)*fscale */
  lgbk_symm_t fe;
  lgbk_collide_t cp;
  double pd[LGBK_NPARAM];
  float pf[LGBK_NPARAM];
} lgbk_binary_args_t;

/* Fill pd/pf from the other members */
static inline void lgbk_binary_args_pack(lgbk_binary_args_t * a) {
  a->pd[LGBK_P_RTAU_SHEAR] = a->cp.rtau_shear;
  a->pd[LGBK_P_RTAU_BULK] = a->cp.rtau_bulk;
  a->pd[LGBK_P_FX] = a->cp.force_global[0];
  a->pd[LGBK_P_FY] = a->cp.force_global[1];
  a->pd[LGBK_P_FZ] = a->cp.force_global[2];
  a->pd[LGBK_P_MOBILITY] = a->mobility;
  a->pd[LGBK_P_RHO0] = a->rho0;
  a->pd[LGBK_P_FSCALE] = a->fscale;
  a->pd[LGBK_P_RFSCALE] = 1.0/a->fscale;
  a->pd[LGBK_P_A] = a->fe.a;
  a->pd[LGBK_P_B] = a->fe.b;
  a->pd[LGBK_P_KAPPA] = a->fe.kappa;
  for (int i = 0; i < LGBK_NPARAM; i++) a->pf[i] = (float) a->pd[i];
}

/* A box of an ensemble: its lattice, its step arguments, and whether it
 * is still stepped (0 once quarantined). */
typedef struct lgbk_box_s {
  lgbk_dims_t d;
  lgbk_binary_args_t a;
  int active;
} lgbk_box_t;

/* One step of every active box: items[k] = (box, item within the box),
 * built for tile height ty and xchunk by lgbk_ensemble_items(); CTAs take
 * the items in list order from the counters sched_dev[0..1] (two ints,
 * zero before the first step; each launch leaves them zero). */
int lgbk_ensemble_step(int prec, const lgbk_box_t * boxes_dev,
		       const void * items_dev, int nitems, int xchunk, int ty,
		       int minb, int has_map, int sites, int * sched_dev,
		       void * stream);
/* Number of work items of one box (and fill items if non-NULL, host) */
int lgbk_ensemble_items(const lgbk_dims_t * d, int box, int xchunk, int ty,
			int * items);

/* sites = 2: two sites per thread in packed FP32x2 (float forms without a
 * status map); otherwise one */
int lgbk_binary_step(const lgbk_dims_t * d, int prec,
		     const lgbk_binary_args_t * a, int xchunk, int ty, int minb,
		     int sites, void * stream);

/* FP16 storage: largest stored magnitude (dev_word: one device word of
 * scratch) and rescaling of n stored values by factor */
int lgbk_half_absmax(long long n, const void * a, unsigned int * dev_word,
		     float * host_max, void * stream);
int lgbk_half_scale(long long n, void * a, float factor, void * stream);

/* Conversions between FP64 canonical state and reduced storage */
int lgbk_f64_to_store(const lgbk_dims_t * d, int prec, int ncomp,
		      double shift_rho0, double scale, const double * src,
		      void * dst, void * stream);
int lgbk_store_to_f64(const lgbk_dims_t * d, int prec, int ncomp,
		      double shift_rho0, double scale, const void * src,
		      double * dst, void * stream);
/* Streaming of reduced-precision distributions (dir as above) */
int lgbk_propagate_store(const lgbk_dims_t * d, int prec, int dir,
			 const void * f, void * fprime, void * stream);

/* Two-distribution binary fluid (lgb_lb2.cu); pull = 1 when the stored
 * arrays hold post-collision values awaiting streaming */
int lgbk_phi_from_g_f64(const lgbk_dims_t * d, int pull, const double * g,
			double * phi, void * stream);
int lgbk_g_from_phi_f64(const lgbk_dims_t * d, const double * phi,
			double * g, void * stream);
int lgbk_collide_binary_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			    const lgbk_collide_t * cp, double mobility,
			    int pull, const double * f_in, const double * g_in,
			    const double * phi, const double * grad,
			    const double * delsq, double * f_out,
			    double * g_out, double * u_out, void * stream);


#ifdef __cplusplus
}
#endif

#endif
