/*****************************************************************************
 *
 *  ludwig_oracle.h
 *
 *  TEST INFRASTRUCTURE ONLY.  A plain-C CPU restatement of the reference's
 *  (Ludwig v0.23) lattice-Boltzmann time step for the symmetric binary
 *  fluid and the cholesteric liquid crystal.  It is the checker for the
 *  CUDA path: only tests/, __graft_entry__.smoke() and bench.py's
 *  cpu_baseline / reference legs load it.  The product never calls it.
 *
 *  Parity: pinned bit-for-bit against the reference's own serial build
 *  (oracle/ref.mk + oracle/ref_shim.c) on the same seeded inputs; see
 *  tests/test_oracle_golden.py and tests/golden/.
 *
 *  Layout of every array: interior sites only, periodic, component-major
 *  with z fastest:  a[((n*Lx + x)*Ly + y)*Lz + z].
 *
 *****************************************************************************/

#ifndef LUDWIG_ORACLE_H
#define LUDWIG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {ORC_NVEL = 19};

typedef struct orc_symm_param_s {
  double a;                 /* A */
  double b;                 /* B */
  double kappa;             /* kappa */
} orc_symm_param_t;

typedef struct orc_collide_param_s {
  double rtau_shear;
  double rtau_bulk;
  double rtau_ghost[ORC_NVEL];
  double force_global[3];
} orc_collide_param_t;

/* Model tables (rational values rounded once), src/lb_d3q19.{h,c} */
const int8_t * orc_cv(void);             /* [19][3] */
const double * orc_wv(void);             /* [19]    */
const double * orc_ma(void);             /* [19][19] mode matrix */
const double * orc_mi(void);             /* [19][19] inverse     */

/* Relaxation times, src/collision.c:1163-1246 (M10 scheme) */
void orc_collide_param_m10(double eta_shear, double eta_bulk, double rho0,
			   orc_collide_param_t * p);

/* Initial conditions */
void orc_spinodal_init(const int L[3], int seed, double phi0, double amp,
		       double * phi);
void orc_lb_init_rest(const int L[3], double rho0, double * f);

/* Hot-path functions */
void orc_grad_7pt(const int L[3], int nf, const double * field,
		  double * grad, double * delsq);
void orc_grad_27pt(const int L[3], int nf, const double * field,
		   double * grad, double * delsq);
void orc_symm_mu(const int L[3], const orc_symm_param_t * fe,
		 const double * phi, const double * delsq, double * mu);
void orc_symm_stress(const int L[3], const orc_symm_param_t * fe,
		     const double * phi, const double * grad,
		     const double * delsq, double * pth);
void orc_force_divergence(const int L[3], const double * pth, double * force);
void orc_advect_upwind(const int L[3], int nf, const double * field,
		       const double * u, double * fw, double * fe,
		       double * fy, double * fz);
void orc_advect_2nd(const int L[3], int nf, const double * field,
		    const double * u, double * fw, double * fe,
		    double * fy, double * fz);
void orc_advect_3rd(const int L[3], int nf, const double * field,
		    const double * u, double * fw, double * fe,
		    double * fy, double * fz);
void orc_advection_order_set(int n);
void orc_gradient_stencil_set(int n);
void orc_ch_flux_mu(const int L[3], const orc_symm_param_t * fe,
		    double mobility, const double * phi, const double * delsq,
		    double * fw, double * fe_, double * fy, double * fz);
void orc_flux_no_normal(const int L[3], int nf, const uint8_t * status,
			double * fw, double * fe, double * fy, double * fz);
void orc_ch_update(const int L[3], const double * fw, const double * fe,
		   const double * fy, const double * fz, double * phi);
void orc_collide_mrt(const int L[3], const orc_collide_param_t * p,
		     const uint8_t * status, double * f, const double * force,
		     double * rho, double * u);
void orc_propagate(const int L[3], const double * f, double * fprime);

/* Full step, src/ludwig.c:528-860, symmetric FD Cahn-Hilliard.
 * work must hold 13*nsites doubles. */
void orc_binary_step(const int L[3], const orc_symm_param_t * fe,
		     double mobility, const orc_collide_param_t * cp,
		     const uint8_t * status,
		     double * f, double * fscratch, double * phi, double * u,
		     double * rho, double * force, double * work, int nsteps);

/* Statistics, src/util_sum.c:30-175, src/phi_stats.c:211-270 */
/* Two-distribution binary fluid (symmetric_lb) */
void orc_phi_from_g(const int L[3], const double * g, double * phi);
void orc_collide_binary(const int L[3], const orc_symm_param_t * fe,
			const orc_collide_param_t * cp, double mobility,
			double * f, double * g, const double * phi,
			const double * grad, const double * delsq, double * u);
void orc_lb2_step(const int L[3], const orc_symm_param_t * fe,
		  double mobility, const orc_collide_param_t * cp,
		  double * f, double * g, double * scratch, double * phi,
		  double * u, double * work, int nsteps);

typedef struct orc_klein_s { double sum; double cs; double ccs; } orc_klein_t;
void orc_klein_add(orc_klein_t * k, double v);
double orc_klein_total(const orc_klein_t * k);
void orc_field_stats(const int L[3], const double * q, double out[5]);
double orc_symm_fed_total(const int L[3], const orc_symm_param_t * fe,
			  const double * phi, const double * grad);

/* Cholesteric liquid crystal (Landau-de Gennes), src/blue_phase.h:50-75.
 * Q is stored as its 5 independent components XX, XY, XZ, YY, YZ;
 * gradients as grad[(3*n + ia)*N + i], delsq[n*N + i]. */
typedef struct orc_lc_param_s {
  double a0;
  double q0;
  double gamma;
  double kappa0;
  double kappa1;
  double xi;
  double redshift;
  double rredshift;
  double epsilon;            /* already divided by 12 pi */
  double e0[3];
  double coswt;
  double amplitude0;
} orc_lc_param_t;

void orc_lc_mol_field(const int L[3], const orc_lc_param_t * p,
		      const double * q, const double * grad,
		      const double * delsq, double * h);
void orc_lc_stress(const int L[3], const orc_lc_param_t * p,
		   const double * q, const double * grad,
		   const double * delsq, double * pth);
void orc_lc_fed(const int L[3], const orc_lc_param_t * p, const double * q,
		const double * grad, double * fed);
/* Beris-Edwards update of q (src/blue_phase_beris_edwards.c:266-289,
 * :538-840) given u and upwind fluxes computed here; work >= 20 N. */
void orc_beris_edw_update(const int L[3], const orc_lc_param_t * p,
			  double gamma_rot, const uint8_t * status,
			  const double * u, const double * grad,
			  const double * delsq, double * q, double * work);
/* Full LC step as src/ludwig.c:528-860; work >= 40 N doubles. */
void orc_lc_step(const int L[3], const orc_lc_param_t * p, double gamma_rot,
		 const orc_collide_param_t * cp, const uint8_t * status,
		 double * f, double * fscratch, double * q, double * u,
		 double * rho, double * force, double * work, int nsteps);
/* Blue phase I (O8M) initial condition, src/blue_phase_init.c:59-132,
 * no rotation */
void orc_lc_init_o8m(const int L[3], const orc_lc_param_t * p, double * q);

#ifdef __cplusplus
}
#endif

#endif
