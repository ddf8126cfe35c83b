/*****************************************************************************
 *
 *  ludwig_gb.h
 *
 *  C ABI of libludwig_gb.so: the lattice-Boltzmann time step of Ludwig
 *  (symmetric binary fluid and cholesteric liquid crystal) on one GB300.
 *
 *  The hot-path entry points keep the names, argument lists and meaning of
 *  the reference functions they replace (cited per declaration as
 *  path:line within the reference tree), and the structures a caller fills
 *  or reads (option structures, parameter structures, the free-energy
 *  object fe_t and its function table fe_vt_t) have the reference's
 *  members in the reference's order, so that code compiled against the
 *  reference's headers and code compiled against this one agree on every
 *  offset.  Objects are opaque handles that own device memory; data stay
 *  resident on the device between calls.
 *
 *  Site indices passed to the free-energy function table and to the
 *  per-site field accessors are the reference's cs_index() numbering
 *  (src/coords.c:617): halo sites included, index = xs*(nhalo + ic - 1) +
 *  ys*(nhalo + jc - 1) + (nhalo + kc - 1) with ic = 1 .. Lx (halo sites
 *  1 - nhalo .. Lx + nhalo) and strides zs = 1, ys = Lz + 2 nhalo,
 *  xs = (Ly + 2 nhalo) ys; a halo site is the periodic image of the
 *  interior site it copies.  Host arrays of the *_to_host / *_from_host
 *  functions hold the interior sites only, component-major, z fastest,
 *      a[((n*Lx + x)*Ly + y)*Lz + z],   x, y, z = 0 .. L-1;
 *  the ludwig_gb_*_to_host_cs functions write the reference's own host
 *  layout (all cs_index sites, in its AOS or SOA data model).
 *  Every function returns 0 on success or a LUDWIG_GB_E* code, with a
 *  message from ludwig_gb_last_error().  Nothing traps on the device.
 *  Calls are synchronous: results are complete when a call returns.
 *
 *  Types not supported on this path (noise with kT > 0, viscosity models,
 *  walls, Lees-Edwards planes, colloids) are accepted as NULL only.
 *
 *****************************************************************************/

#ifndef LUDWIG_GB_H
#define LUDWIG_GB_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes */
enum {
  LUDWIG_GB_OK       = 0,
  LUDWIG_GB_EINVAL   = 1,    /* invalid argument or unsupported option */
  LUDWIG_GB_ENOMEM   = 2,    /* device or host allocation failed */
  LUDWIG_GB_ECUDA    = 3,    /* CUDA runtime error */
  LUDWIG_GB_ESTATE   = 4,    /* object in the wrong state for this call */
  LUDWIG_GB_ETIMEOUT = 5,    /* a bounded device wait ran out */
  LUDWIG_GB_ENOTFINITE = 6,  /* NaN or Inf detected in a reduction */
  LUDWIG_GB_EIO      = 7     /* a snapshot file could not be written/read */
};

const char * ludwig_gb_last_error(void);
const char * ludwig_gb_version(void);

/* Arithmetic and storage of a state */
typedef enum ludwig_gb_prec_e {
  LUDWIG_GB_FP64 = 0,        /* double; the drop-in, reference-exact */
  LUDWIG_GB_FP32 = 1,        /* float; f stored as f - w_p rho0 */
  LUDWIG_GB_FP16 = 2         /* float arithmetic; (f - w_p rho0)*scale as
				half, the scale derived from the range */
} ludwig_gb_prec_t;

/* Opaque objects (names as in the reference) */
typedef struct pe_s pe_t;
typedef struct cs_s cs_t;
typedef struct physics_s physics_t;
typedef struct lb_data_s lb_t;
typedef struct field_s field_t;
typedef struct field_grad_s field_grad_t;
typedef struct hydro_s hydro_t;
typedef struct map_s map_t;
typedef struct fe_s fe_t;
typedef struct fe_symm_s fe_symm_t;
typedef struct fe_lc_s fe_lc_t;
typedef struct pth_s pth_t;
typedef struct phi_ch_s phi_ch_t;
typedef struct beris_edw_s beris_edw_t;
typedef struct noise_s noise_t;              /* NULL only */
typedef struct visc_s visc_t;                /* NULL only */
typedef struct wall_s wall_t;                /* NULL only */
typedef struct lees_edw_s lees_edw_t;        /* NULL only */
typedef struct colloids_info_s colloids_info_t;  /* NULL only */

/*---------------------------------------------------------------------------
 * Parallel environment (one process, one GPU): src/pe.h:26-27
 *-------------------------------------------------------------------------*/
int pe_create(int device, pe_t ** ppe);
int pe_free(pe_t * pe);

/*---------------------------------------------------------------------------
 * Coordinate system: src/coords.h:73-84.  Periodic in all directions.
 * nhalo is recorded for layout conversions; device arrays hold no halo.
 *-------------------------------------------------------------------------*/
int cs_create(pe_t * pe, cs_t ** pcs);
int cs_free(cs_t * cs);
int cs_ntotal_set(cs_t * cs, const int ntotal[3]);
int cs_nhalo_set(cs_t * cs, int nhalo);
int cs_init(cs_t * cs);
int cs_nlocal(cs_t * cs, int nlocal[3]);
/* src/coords.h:98-107: the site numbering of the free-energy slots and of
 * the ludwig_gb_*_cs functions */
int cs_ntotal(cs_t * cs, int ntotal[3]);
int cs_nhalo(cs_t * cs, int * nhalo);
int cs_nsites(cs_t * cs, int * nsites);
int cs_strides(cs_t * cs, int * xs, int * ys, int * zs);
int cs_nall(cs_t * cs, int nall[3]);
int cs_index(cs_t * cs, int ic, int jc, int kc);
int cs_index_to_ijk(cs_t * cs, int index, int coords[3]);

/*---------------------------------------------------------------------------
 * Physical parameters: src/physics.h:20-37.  As in the reference, the most
 * recently created object is the one the collision and Cahn-Hilliard
 * stages read (physics_ref, src/physics.c:76).
 *-------------------------------------------------------------------------*/
int physics_create(pe_t * pe, physics_t ** phys);
int physics_free(physics_t * phys);
int physics_rho0_set(physics_t * phys, double rho0);
int physics_eta_shear_set(physics_t * phys, double eta);
int physics_eta_bulk_set(physics_t * phys, double zeta);
int physics_mobility_set(physics_t * phys, double mobility);
int physics_fbody_set(physics_t * phys, const double f[3]);
int physics_ref(physics_t ** ref);
/* Frequency of the external electric field (src/physics.h:30,47): with a
 * frequency f the LC free energy's field carries the phase
 * coswt = cos(2 pi f t) at the current time t, evaluated before every use
 * of its parameters (fe_lc_param_commit, src/blue_phase.c:210-226) */
int physics_e0_frequency_set(physics_t * phys, double e0_frequency);
int physics_e0_frequency(physics_t * phys, double * e0_frequency);
/* Time step control, src/physics.c:600-668: a run of nstep steps from
 * nstart; next_step advances the counter (positive while steps remain),
 * time is t_start + t_current - 1 in lattice units */
int physics_control_init_time(physics_t * phys, int nstart, int nstep);
int physics_control_next_step(physics_t * phys);
int physics_control_timestep(physics_t * phys);
int physics_control_time(physics_t * phys, double * t);

/*---------------------------------------------------------------------------
 * Distributions: src/lb_data.h:30-47,162-171 (D3Q19, ndist = 1)
 *-------------------------------------------------------------------------*/
/* I/O options carried by the option structures, src/io_options.h:25-62
 * and src/io_info_args.h:33-38 (the snapshot functions below read
 * iorformat; the rest is accepted and recorded) */
enum io_mode_enum {IO_MODE_INVALID, IO_MODE_MPIIO};
enum io_record_format_enum {IO_RECORD_INVALID, IO_RECORD_ASCII,
			    IO_RECORD_BINARY};
enum io_metadata_version_enum {IO_METADATA_INVALID, IO_METADATA_SINGLE_V1,
			       IO_METADATA_MULTI_V1, IO_METADATA_V2};
typedef enum io_mode_enum             io_mode_enum_t;
typedef enum io_record_format_enum    io_record_format_enum_t;
typedef enum io_metadata_version_enum io_metadata_version_enum_t;

typedef struct io_options_s {
  io_mode_enum_t             mode;
  io_record_format_enum_t    iorformat;
  io_metadata_version_enum_t metadata_version;
  int                        report;
  int                        asynchronous;
  int                        compression_levl;
  int                        iogrid[3];
} io_options_t;

typedef struct io_info_args_s {
  io_options_t input;
  io_options_t output;
  int grid[3];
  int iofreq;
} io_info_args_t;

/* src/io_options.c, src/io_info_args.c: MPIIO, binary, single-file V1,
 * grid 1 1 1 */
io_options_t io_options_default(void);
io_info_args_t io_info_args_default(void);

/*---------------------------------------------------------------------------
 * Distributions: src/lb_data.h:162-171, src/lb_data_options.h:20-47
 * (D3Q19, ndist = 1 or 2)
 *-------------------------------------------------------------------------*/
typedef enum lb_relaxation_enum {LB_RELAXATION_M10, LB_RELAXATION_BGK,
				 LB_RELAXATION_TRT} lb_relaxation_enum_t;
typedef enum lb_halo_enum {LB_HALO_FULL = 1, LB_HALO_REDUCED = 2}
  lb_halo_enum_t;

typedef struct lb_data_options_s {
  int ndim;                      /* 3 */
  int nvel;                      /* 19 */
  int ndist;                     /* 1, or 2 (symmetric_lb) */
  lb_relaxation_enum_t nrelax;   /* default M10 */
  lb_halo_enum_t halo;           /* recorded (the halo is implicit) */
  int reportimbalance;           /* recorded */
  int usefirsttouch;             /* recorded */
  io_info_args_t iodata;         /* record formats of the snapshot files */
} lb_data_options_t;

lb_data_options_t lb_data_options_default(void);
lb_data_options_t lb_data_options_ndim_nvel_ndist(int ndim, int nvel,
						  int ndist);
/* Objects created by the reference-named functions are FP64 (the
 * drop-in).  The reduced-precision forms are created here; fp16_scale is
 * the FP16 storage scale of f - w_p rho0 (0: the default). */
int lb_data_create(pe_t * pe, cs_t * cs, const lb_data_options_t * opts,
		   lb_t ** lb);
int ludwig_gb_lb_data_create(pe_t * pe, cs_t * cs,
			     const lb_data_options_t * opts, int precision,
			     double fp16_scale, lb_t ** lb);
int lb_free(lb_t * lb);
int lb_init_rest_f(lb_t * lb, double rho0);                /* lb_data.c:659 */
int lb_halo(lb_t * lb);                                     /* lb_data.c:754 */
int lb_f_to_host(lb_t * lb, double * f);       /* 19 x nsites, reference f */
int lb_f_from_host(lb_t * lb, const double * f);
/* ndist = 2 (symmetric_lb): the order-parameter distribution g */
int lb_g_to_host(lb_t * lb, double * g);       /* 19 x nsites, reference g */
int lb_g_from_host(lb_t * lb, const double * g);
/* src/phi_lb_coupler.h: phi = sum_p g_p; g_0 = phi, other g_p = 0 */
int phi_lb_to_field(field_t * phi, lb_t * lb);
int phi_lb_from_field(field_t * phi, lb_t * lb);
/* nsteps of the main loop with ndist = 2 (src/ludwig.c:528-860):
 * phi_lb_to_field, field_grad_compute, binary lb_collide
 * (src/collision.c:604-1013), lb_propagation.  FP64, bit-exact. */
int ludwig_gb_lb2_step(lb_t * lb, field_t * phi, hydro_t * hydro, fe_t * fe,
		       int nsteps);

/* src/collision.h:27, src/collision.c:143 */
int lb_collide(lb_t * lb, hydro_t * hydro, map_t * map, noise_t * noise,
	       fe_t * fe, visc_t * visc);
/* src/propagation.h:21, src/propagation.c:43 */
int lb_propagation(lb_t * lb);

/*---------------------------------------------------------------------------
 * Fields: src/field.h:97-119, src/field_options.h
 *-------------------------------------------------------------------------*/
typedef enum field_halo_enum {FIELD_HALO_HOST, FIELD_HALO_TARGET,
			      FIELD_HALO_OPENMP} field_halo_enum_t;

typedef struct field_options_s {
  int ndata;                     /* components: 1 (phi) or 5 (Q) */
  int nhcomm;                    /* halo width requested (recorded) */
  field_halo_enum_t haloscheme;  /* recorded */
  int haloverbose;               /* recorded */
  int usefirsttouch;             /* recorded */
  io_info_args_t iodata;         /* record formats of the snapshot files */
} field_options_t;

field_options_t field_options_default(void);
field_options_t field_options_ndata_nhalo(int ndata, int nhalo);
int field_create(pe_t * pe, cs_t * cs, lees_edw_t * le, const char * name,
		 const field_options_t * opts, field_t ** pobj);
/* field_create with the precision of the state it belongs to (FP64; FP32
 * and FP16 states keep their fields in float) */
int ludwig_gb_field_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
			   const char * name, const field_options_t * opts,
			   int precision, field_t ** pobj);
int field_free(field_t * obj);
int field_nf(field_t * obj, int * nf);
int field_halo(field_t * obj);                              /* field.c:371 */
int field_to_host(field_t * obj, double * data);
int field_from_host(field_t * obj, const double * data);
/* Per-site values at a cs_index() site, src/field.h:109-120 (one small
 * device copy per call: for host code that visits a few sites) */
int field_scalar(field_t * obj, int index, double * phi);
int field_scalar_set(field_t * obj, int index, double phi);
int field_vector(field_t * obj, int index, double p[3]);
int field_vector_set(field_t * obj, int index, const double p[3]);
int field_tensor(field_t * obj, int index, double q[3][3]);
int field_tensor_set(field_t * obj, int index, double q[3][3]);
int field_scalar_array(field_t * obj, int index, double * array);
int field_scalar_array_set(field_t * obj, int index, const double * array);
int field_phi_init_spinodal(field_t * phi, int seed, double phi0, double amp);
/* Spinodal patches of +-1, src/field_phi_init.c:537 */
int field_phi_init_spinodal_patches(field_t * phi, int seed, int patch,
				    double volminus1);
/* src/field_phi_init.c:38: phi = phistar tanh((r - radius)/xi) about the
 * box centre */
int field_phi_init_drop(field_t * phi, double xi, double radius,
			double phistar, int is_centred);
                                                    /* field_phi_init.c:484 */

/*---------------------------------------------------------------------------
 * Gradients: src/field_grad.h:44-50 (3d_7pt_fluid stencil)
 *-------------------------------------------------------------------------*/
int field_grad_create(pe_t * pe, field_t * f, int level, field_grad_t ** p);
void field_grad_free(field_grad_t * obj);
/* src/field_grad.c:319 -> src/gradient_3d_7pt_fluid.c:231 */
int field_grad_compute(field_grad_t * obj);
/* The stencil of field_grad_compute: 7 (default, 3d_7pt_fluid) or 27
 * (3d_27pt_fluid, src/gradient_3d_27pt_fluid.c); the reference selects it
 * with field_grad_set(fg, grad_3d_27pt_fluid_d2, NULL).  The fused steps
 * use 7 points and reject 27. */
int field_grad_stencil_set(field_grad_t * fg, int npoints);
/* src/advection.c:82: order of the advective fluxes of phi_cahn_hilliard
 * and beris_edw_update (1 upwind, default; 2 centred; 3 upwind-biased);
 * the fused steps use 1 and reject the others */
int advection_order_set(int n);
/* grad: 3*nf x nsites ([n][ia]), delsq: nf x nsites */
int field_grad_to_host(field_grad_t * obj, double * grad, double * delsq);

/*---------------------------------------------------------------------------
 * Hydrodynamic fields: src/hydro.h:28-61
 *-------------------------------------------------------------------------*/
typedef struct hydro_options_s {
  int nhcomm;                    /* halo width (recorded) */
  field_options_t rho;           /* density (its iodata: file "rho") */
  field_options_t u;             /* velocity (its iodata: file "vel") */
  field_options_t force;
  field_options_t eta;           /* viscosity field: unused */
} hydro_options_t;

hydro_options_t hydro_options_default(void);
hydro_options_t hydro_options_nhalo(int nhalo);
int hydro_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		 const hydro_options_t * opts, hydro_t ** pobj);
/* hydro_create with the precision of the state it belongs to (FP64; FP32
 * and FP16 states keep rho, u and the force in float) */
int ludwig_gb_hydro_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
			   const hydro_options_t * opts, int precision,
			   hydro_t ** pobj);
int hydro_free(hydro_t * obj);
int hydro_f_zero(hydro_t * obj, const double fzero[3]);    /* hydro.c:244 */
int hydro_u_zero(hydro_t * obj, const double uzero[3]);    /* hydro.c:217 */
int hydro_u_halo(hydro_t * obj);                            /* hydro.c:185 */
int hydro_to_host(hydro_t * obj, double * rho, double * u, double * force);
int hydro_from_host(hydro_t * obj, const double * rho, const double * u,
		    const double * force);

/*---------------------------------------------------------------------------
 * The reference's host layout (what lb_memcpy / field_memcpy /
 * hydro_memcpy leave in its host arrays, src/lb_data.h:144,
 * src/field.c:329, src/hydro.c:306-331): every cs_index() site, halo sites
 * holding the periodic images (as after lb_halo / field_halo), component
 * k of K at
 *     DATA_MODEL_AOS (the reference's default CPU build):  a[K*index + k]
 *     DATA_MODEL_SOA (built with ADDR_SOA, its GPU builds): a[nsites*k + index]
 * with nsites from cs_nsites().  Components: lb k = n*19 + p (n the
 * distribution), fields k = n, hydro u and force k = ia, rho K = 1.  The
 * reduced-precision forms are converted to double.  The _from_ functions
 * read the interior sites only.  (src/memory.h:151-170, data_model_enum)
 *-------------------------------------------------------------------------*/
typedef enum data_model_enum_type {DATA_MODEL_AOS, DATA_MODEL_SOA,
				   DATA_MODEL_AOSOA} data_model_enum_t;

int ludwig_gb_lb_to_host_cs(lb_t * lb, int data_model, double * f);
int ludwig_gb_lb_from_host_cs(lb_t * lb, int data_model, const double * f);
int ludwig_gb_field_to_host_cs(field_t * obj, int data_model, double * data);
int ludwig_gb_field_from_host_cs(field_t * obj, int data_model,
				 const double * data);
/* any of rho, u, force may be NULL */
int ludwig_gb_hydro_to_host_cs(hydro_t * obj, int data_model, double * rho,
			       double * u, double * force);

/*---------------------------------------------------------------------------
 * Site status map: src/map.h:26-63 (MAP_FLUID = 0)
 *-------------------------------------------------------------------------*/
enum map_status {MAP_FLUID, MAP_BOUNDARY, MAP_COLLOID, MAP_STATUS_MAX};

/* src/map_options.h:21-26 */
typedef struct map_options_s {
  int ndata;                     /* 0 only (no per-site data) */
  int is_porous_media;           /* 0 only */
  const char * filestub;         /* recorded */
  io_info_args_t iodata;         /* recorded */
} map_options_t;

map_options_t map_options_default(void);
map_options_t map_options_ndata(int ndata);
/* src/map.h:51-53 (every site starts as MAP_FLUID) */
int map_create(pe_t * pe, cs_t * cs, const map_options_t * options,
	       map_t ** map);
int map_free(map_t ** map);
/* status of every interior site (uint8, site order as the host arrays) */
int map_status_from_host(map_t * obj, const uint8_t * status);

/*---------------------------------------------------------------------------
 * Free energy: the fe_t interface of src/free_energy.h:27-76, member for
 * member.  The slots take cs_index() site indices (halo sites are the
 * periodic images); the vectorised (_v) slots have NSIMDVL = 1, as the
 * reference's default build.  Implemented: FE_SYMMETRIC (free, target,
 * fed, mu, stress, str_symm, stress_v, str_symm_v) and FE_LC (free,
 * target, fed, stress, str_symm, str_anti, htensor and the four _v
 * slots); the other slots are NULL, as in the reference's tables
 * (src/symmetric.c:46-61, src/blue_phase.c:35-50).  Each slot call reads
 * the few values it needs from the device: a per-site host interface, as
 * in the reference's host tables.
 *-------------------------------------------------------------------------*/
#ifndef NSIMDVL
#define NSIMDVL 1
#endif

enum fe_id_enum {FE_NULL,
		 FE_SYMMETRIC,
		 FE_BRAZOVSKII,
		 FE_SURFACTANT,
		 FE_POLAR,
		 FE_LC,
		 FE_ELECTRO,
		 FE_ELECTRO_SYMMETRIC,
		 FE_LC_DROPLET,
		 FE_TERNARY};
typedef enum fe_id_enum fe_id_enum_t;

typedef struct fe_vt_s fe_vt_t;

typedef int (* fe_free_ft)(fe_t * fe);
typedef int (* fe_id_ft)(fe_t * fe);
typedef int (* fe_target_ft)(fe_t * fe, fe_t ** target);
typedef int (* fe_fed_ft)(fe_t * fe, int index, double * fed);
typedef int (* fe_mu_ft)(fe_t * fe, int index, double * mu);
typedef int (* fe_str_ft)(fe_t * fe, int index, double s[3][3]);
typedef int (* fe_mu_solv_ft)(fe_t * fe, int index, int k, double * mu);
typedef int (* fe_hvector_ft)(fe_t * fe, int index, double h[3]);
typedef int (* fe_htensor_ft)(fe_t * fe, int index, double h[3][3]);
typedef void (* fe_htensor_v_ft)(fe_t * fe, int index,
				 double h[3][3][NSIMDVL]);
typedef void (* fe_stress_v_ft)(fe_t * fe, int index,
				double s[3][3][NSIMDVL]);

struct fe_vt_s {
  fe_free_ft free;              /* destructor */
  fe_target_ft target;          /* the object itself (no device copy) */
  fe_fed_ft fed;                /* free energy density */
  fe_mu_ft mu;                  /* chemical potential */
  fe_mu_solv_ft mu_solv;        /* NULL */
  fe_str_ft stress;             /* chemical stress (total) */
  fe_str_ft str_symm;           /* symmetric part */
  fe_str_ft str_anti;           /* antisymmetric part */
  fe_hvector_ft hvector;        /* NULL */
  fe_htensor_ft htensor;        /* molecular field */
  fe_htensor_v_ft htensor_v;
  fe_stress_v_ft stress_v;
  fe_stress_v_ft str_symm_v;
  fe_stress_v_ft str_anti_v;
};

struct fe_s {
  fe_vt_t * func;
  int id;                       /* enum fe_id_enum */
  int use_stress_relaxation;    /* 0 only */
};

/* src/symmetric.h:38-51 */
typedef struct fe_symm_param_s {
  double a;
  double b;
  double kappa;
  double c;
  double h;
} fe_symm_param_t;

int fe_symm_create(pe_t * pe, cs_t * cs, field_t * phi, field_grad_t * dphi,
		   fe_symm_t ** p);
int fe_symm_free(fe_symm_t * fe);
int fe_symm_param_set(fe_symm_t * fe, fe_symm_param_t values);
int fe_symm_param(fe_symm_t * fe, fe_symm_param_t * values);

/* Cholesteric liquid crystal: src/blue_phase.h:51-74 (Q as 5 components
 * XX, XY, XZ, YY, YZ of a field with ndata = 5); anchoring:
 * src/lc_anchoring.h:20-35 (no walls or colloids here: recorded only) */
typedef enum lc_anchoring_enum {
  LC_ANCHORING_NONE = 0,
  LC_ANCHORING_PLANAR,
  LC_ANCHORING_NORMAL,
  LC_ANCHORING_FIXED,
  LC_ANCHORING_INVALID
} lc_anchoring_enum_t;

typedef struct lc_anchoring_param_s {
  lc_anchoring_enum_t type;
  double w1;
  double w2;
  double nfix[3];
} lc_anchoring_param_t;

typedef struct fe_lc_param_s {
  double a0;
  double q0;
  double gamma;
  double kappa0;
  double kappa1;
  double xi;                  /* flow aligning parameter */
  double zeta0, zeta1, zeta2; /* active stress: 0 only */
  double redshift;
  double rredshift;           /* set by fe_lc_param_set */
  double epsilon;             /* dielectric anisotropy (scaled by 1/12pi) */
  double amplitude0;          /* initial amplitude */
  double e0[3];               /* external electric field */
  double coswt;               /* field phase (1 for a static field) */
  int is_redshift_updated;    /* 0 only */
  int is_active;              /* 0 only */
  lc_anchoring_param_t coll;  /* colloid anchoring: unused */
  lc_anchoring_param_t wall;  /* wall anchoring: unused */
} fe_lc_param_t;

int fe_lc_create(pe_t * pe, cs_t * cs, lees_edw_t * le, field_t * q,
		 field_grad_t * dq, fe_lc_t ** p);      /* blue_phase.c:78 */
int fe_lc_free(fe_lc_t * fe);
/* blue_phase.c:241: epsilon is divided by 12 pi, rredshift = 1/redshift */
int fe_lc_param_set(fe_lc_t * fe, const fe_lc_param_t * values);
int fe_lc_param(fe_lc_t * fe, fe_lc_param_t * values);
/* Blue phase I initial condition, src/blue_phase_init.c:59; euler_angles
 * (degrees, Z-X-Z; NULL for none) rotate the structure about the centre */
int blue_phase_O8M_init(cs_t * cs, fe_lc_param_t * param, field_t * q,
			const double euler_angles[3]);
/* Blue phase II, src/blue_phase_init.c:155 (Euler angles as above) */
int blue_phase_O2_init(cs_t * cs, fe_lc_param_t * param, field_t * q,
		       const double euler_angles[3]);
/* Cholesteric helix along X, Y or Z (0, 1, 2), src/blue_phase_init.c:763 */
int blue_phase_twist_init(cs_t * cs, fe_lc_param_t * param, field_t * q,
			  int helical_axis);
/* Random directors (amplitude 0.01) in the box rmin..rmax (1-based,
 * inclusive), src/blue_phase_init.c:1279 */
int blue_phase_random_q_rectangle(cs_t * cs, fe_lc_param_t * param,
				  field_t * q, int rmin[3], int rmax[3]);
/* Random uniaxial directors (seed 13), src/blue_phase_init.c:1170 */
int blue_phase_random_q_init(cs_t * cs, fe_lc_param_t * param, field_t * q);
/* Uniform uniaxial nematic along n, src/blue_phase_init.c:836 */
int blue_phase_nematic_init(cs_t * cs, fe_lc_param_t * param, field_t * q,
			    const double n[3]);

/* Beris-Edwards: src/blue_phase_beris_edwards.h:28-49 */
#define NQAB 5
typedef struct beris_edw_param_s {
  double xi;                  /* effective aspect ratio */
  double gamma;               /* rotational diffusion constant Gamma */
  int noise;                  /* 0 only */
  double var;
  double tmatrix[3][3][NQAB]; /* noise basis: unused (noise off) */
} beris_edw_param_t;

int beris_edw_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		     beris_edw_t ** pobj);
int beris_edw_free(beris_edw_t * be);
int beris_edw_param_set(beris_edw_t * be, beris_edw_param_t * values);
/* src/blue_phase_beris_edwards.c:266 */
int beris_edw_update(beris_edw_t * be, fe_t * fe, field_t * fq,
		     field_grad_t * fq_grad, hydro_t * hydro,
		     colloids_info_t * cinfo, map_t * map, noise_t * noise);
/* molecular field of the last update: 5 x nsites */
int beris_edw_h_to_host(beris_edw_t * be, double * h);

/* Fused GB300 step of the cholesteric: nsteps iterations of the main loop
 * of src/ludwig.c:528-860 (the physics object's step counter advanced,
 * q gradients, molecular field and chiral stress, stress-divergence force,
 * Beris-Edwards update with upwind fluxes, collision, streaming) in two
 * kernel launches per step; a time-dependent field's phase is taken at
 * each step's time.  FP64 objects
 * give the results of the functions above called one by one; FP32 objects
 * (lb, q, hydro) run the same step in float arithmetic. */
int ludwig_gb_lc_step(lb_t * lb, field_t * q, hydro_t * hydro, map_t * map,
		      fe_t * fe, beris_edw_t * be, int nsteps);
/* device time (ms) of nsteps LC steps, CUDA events on the library stream */
int ludwig_gb_time_lc(lb_t * lb, field_t * q, hydro_t * hydro, map_t * map,
		      fe_t * fe, beris_edw_t * be, int nsteps, double * ms);

/*---------------------------------------------------------------------------
 * Force from the free energy: src/phi_force_stress.h:36-39,
 * src/phi_force.h:24 (stress divergence, fluid only)
 *-------------------------------------------------------------------------*/
enum {FE_FORCE_METHOD_NO_FORCE = 0, FE_FORCE_METHOD_STRESS_DIVERGENCE = 1};
int pth_create(pe_t * pe, cs_t * cs, int method, pth_t ** pth);
int pth_free(pth_t * pth);
int pth_stress_compute(pth_t * pth, fe_t * fe);   /* phi_force_stress.c:171 */
int pth_to_host(pth_t * pth, double * str);        /* 9 x nsites */
int phi_force_calculation(pe_t * pe, cs_t * cs, lees_edw_t * le,
			  wall_t * wall, pth_t * pth, fe_t * fe, map_t * map,
			  field_t * phi, hydro_t * hydro);

/*---------------------------------------------------------------------------
 * Cahn-Hilliard finite-difference update: src/phi_cahn_hilliard.h:35-56
 *-------------------------------------------------------------------------*/
typedef struct phi_ch_info_s {
  int conserve;                  /* 0 only */
  int noise;                     /* 0 only */
} phi_ch_info_t;

int phi_ch_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		  const phi_ch_info_t * info, phi_ch_t ** pch);
int phi_ch_free(phi_ch_t * pch);
int phi_cahn_hilliard(phi_ch_t * pch, fe_t * fe, field_t * phi,
		      hydro_t * hydro, map_t * map, noise_t * noise);

/*---------------------------------------------------------------------------
 * Fused GB300 step.  One call performs nsteps iterations of the main loop
 * of src/ludwig.c:528-860 for the symmetric binary fluid (field gradients,
 * stress-divergence force, Cahn-Hilliard update, collision, streaming),
 * one kernel launch per step, replayed from a CUDA graph.  For FP64
 * objects the results equal those of calling the functions above one by
 * one.  hydro's force is not stored by the fused step.
 *-------------------------------------------------------------------------*/
int ludwig_gb_binary_step(lb_t * lb, field_t * phi, hydro_t * hydro,
			  map_t * map, fe_t * fe, int nsteps);
/* FP16 storage keeps f - w_p rho0 times a power-of-two scale derived from
 * the field's range: the largest deviation maps into [2^10, 2^11), room to
 * grow 32-fold before half precision's largest value.  The scale is derived when f
 * is set from the host (lb_f_from_host), again every 256 steps of
 * ludwig_gb_binary_step, and on this call, which requantises the stored
 * values (scale: the new value, may be NULL; no-op for FP32 and FP64). */
int ludwig_gb_lb_fp16_rescale(lb_t * lb, double * scale);
/* As ludwig_gb_binary_step without synchronising (and without the FP16
 * rescaling): the steps are queued on the library's stream;
 * ludwig_gb_sync() waits for them. */
int ludwig_gb_binary_step_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				map_t * map, fe_t * fe, int nsteps);
int ludwig_gb_sync(void);
/* The CUDA stream (cudaStream_t) every launch of the library uses. */
void * ludwig_gb_stream(void);
/* Tuning of the fused kernel: planes per x chunk (0, the default: an equal
 * share of the (tile, plane) pairs per resident CTA), tile height (4, 8,
 * 16) and resident CTAs per SM for tile height 8 (2..4; 0 = default). */
int ludwig_gb_tune_set(int xchunk, int tile_y, int min_blocks);
/* Sites per thread of the float forms of the fused steps: 2 (two rows of
 * the tile per thread, packed FP32x2 arithmetic, the pulled populations of
 * the next plane loaded while the current one is computed; the tile then
 * has tile_y rows in tile_y/2 thread rows), 1, or 0 (the default: the
 * faster form of each on GB300: 2 for the binary fluid with FP16 storage,
 * 1 for it in FP32; for the cholesteric, one site a thread with the
 * force + collision kernel reading the stress neighbours through L1,
 * where 1 asks for the one that streams stress planes through a
 * shared-memory ring).  A status map with solid sites always uses the
 * one-site ring forms. */
int ludwig_gb_tune_sites(int sites_per_thread);

/*---------------------------------------------------------------------------
 * State transfer in the storage format of the objects' precision, for
 * callers that keep the state in host memory between steps.  Elements:
 * f 19*nsites (FP64: double; FP32: float f - w_p rho0; FP16: half
 * (f - w_p rho0)*scale), phi nsites and u 3*nsites (double or float).
 * f is the carried post-collision state of the fused step.  The copies are
 * queued on the library's stream (use pinned host memory for speed).
 *-------------------------------------------------------------------------*/
int ludwig_gb_state_bytes(lb_t * lb, size_t * f_bytes, size_t * phi_bytes,
			  size_t * u_bytes);
int ludwig_gb_state_to_host_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				  void * f, void * phi_h, void * u);
int ludwig_gb_state_from_host_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				    const void * f, const void * phi_h,
				    const void * u);
/* Page-locked host memory */
int ludwig_gb_host_alloc(size_t bytes, void ** p);
int ludwig_gb_host_free(void * p);

/* Device time (CUDA events on the library's stream) of nsteps fused steps,
 * and of nsteps end-to-end steps: state in from host buffers, one fused
 * step, state (and rho) back to host buffers. */
int ludwig_gb_time_binary(lb_t * lb, field_t * phi, hydro_t * hydro,
			  map_t * map, fe_t * fe, int nsteps, double * ms);
int ludwig_gb_time_binary_e2e(lb_t * lb, field_t * phi, hydro_t * hydro,
			      map_t * map, fe_t * fe, int nsteps, void * f_h,
			      void * phi_h, void * u_h, void * rho_h,
			      double * ms);
/* The same with the copies of consecutive steps overlapped: every step
 * uploads the same host input (in_*), takes one fused step and downloads
 * the result (out_*: f, phi, u, rho); two device buffer sets alternate and
 * the upload of step k+1 runs while the download of step k does.  All
 * host buffers pinned (ludwig_gb_host_alloc).  On return the objects hold
 * the input state. */
int ludwig_gb_time_binary_e2e_overlap(lb_t * lb, field_t * phi,
				      hydro_t * hydro, map_t * map, fe_t * fe,
				      int nsteps, const void * in_f,
				      const void * in_phi, const void * in_u,
				      void * out_f, void * out_phi,
				      void * out_u, void * out_rho,
				      double * ms);

/*---------------------------------------------------------------------------
 * Statistics (FP64 accumulation, compensated), src/phi_stats.c:91-140,
 * src/stats_distribution.c:55-120, src/stats_free_energy.c:38
 *-------------------------------------------------------------------------*/
/* out = {total, mean, variance, min, max} of component n */
int stats_field_q(field_t * field, int n, double out[5]);
/* out = {total mass, momentum x, y, z} from the distributions */
int stats_distribution(lb_t * lb, double out[4]);
/* total symmetric free energy (bulk + gradient) */
int stats_free_energy_symm(fe_symm_t * fe, double * total);
/* LC total free energy (fe_lc_fed summed, src/stats_free_energy.c:38);
 * FP64 fields, after field_grad_compute() of the q gradients */
int stats_free_energy_lc(fe_lc_t * fe, double * total);
/* The numbers fe_lc_stats_info prints (src/fe_lc_stats.c:55-150), without
 * walls or colloids: out = {f, v, f/v, f_bulk/v, f_grad/v, redshift} over
 * the fluid sites of map (all sites for NULL); after field_grad_compute()
 * of the q gradients */
int ludwig_gb_fe_lc_stats_info(fe_lc_t * fe, map_t * map, double out[6]);
/* The numbers stats_velocity_minmax prints (src/stats_velocity.c:54-125):
 * out = {min u_x, u_y, u_z, max u_x, u_y, u_z, volume flux x, y, z} over
 * the fluid sites of map (all sites for NULL); min starts at FLT_MAX, max
 * at FLT_MIN */
int ludwig_gb_stats_velocity_minmax(hydro_t * hydro, map_t * map,
				    double out[9]);

/*---------------------------------------------------------------------------
 * Ensembles: many independent periodic binary-fluid boxes of any sizes and
 * parameters advanced together, one kernel launch per step for all boxes
 * (replayed from a CUDA graph).  No counterpart in the reference, which
 * runs one system per job; each box follows the same step as
 * ludwig_gb_binary_step.
 *-------------------------------------------------------------------------*/
typedef struct ludwig_gb_ensemble_s ludwig_gb_ensemble_t;

typedef struct ludwig_gb_box_param_s {
  int ntotal[3];
  double rho0;
  double eta;                 /* shear viscosity */
  double eta_bulk;            /* bulk viscosity (<= 0: eta) */
  double a, b, kappa;         /* symmetric free energy */
  double mobility;
  int seed;                   /* spinodal initial condition */
  double phi0, noise;
} ludwig_gb_box_param_t;

int ludwig_gb_ensemble_create(int nbox, const ludwig_gb_box_param_t * p,
			      int precision, ludwig_gb_ensemble_t ** pens);
int ludwig_gb_ensemble_free(ludwig_gb_ensemble_t * ens);
int ludwig_gb_ensemble_step(ludwig_gb_ensemble_t * ens, int nsteps);
/* device time of nsteps (CUDA events on the library stream) */
int ludwig_gb_ensemble_time(ludwig_gb_ensemble_t * ens, int nsteps,
			    double * ms);
int ludwig_gb_ensemble_tune_set(ludwig_gb_ensemble_t * ens, int xchunk,
				int tile_y, int min_blocks);
/* Time each candidate tiling for trial_steps on a copy of the state and
 * keep the fastest; the state itself is left unchanged. */
int ludwig_gb_ensemble_autotune(ludwig_gb_ensemble_t * ens, int trial_steps,
				int best[3], double * ms_best);
/* reference f (19 x n), phi (n), u (3 x n), rho (n) of one box; any NULL */
int ludwig_gb_ensemble_box_get(ludwig_gb_ensemble_t * ens, int box,
			       double * f, double * phi, double * u,
			       double * rho);
int ludwig_gb_ensemble_box_set_phi(ludwig_gb_ensemble_t * ens, int box,
				   const double * phi);
/* Boxes whose mass or total phi is no longer finite are quarantined: they
 * are not stepped any more; the others continue unchanged. */
int ludwig_gb_ensemble_check(ludwig_gb_ensemble_t * ens, int * nactive);
int ludwig_gb_ensemble_box_active(ludwig_gb_ensemble_t * ens, int box,
				  int * active);
/* lattice sites of the active boxes */
int ludwig_gb_ensemble_sites(ludwig_gb_ensemble_t * ens, long long * n);

/* Domain length from the spherically averaged structure factor of a
 * scalar field (util/length_from_sk.c:88-190): L = 2 pi sum S dk /
 * sum k S dk over 128 bins.  faithful = 1 keeps the reference's
 * wavevector for i > N/2 (dk*i - pi); faithful = 0 uses dk*i - 2 pi.
 * sk and nk (128 doubles each, may be NULL) receive the binned sums. */
int ludwig_gb_length_from_sk(field_t * phi, int faithful, double * length,
			     double * sk, double * nk);

/* Field statistics that allocate nothing.  No counterpart in the
 * reference.  For callers that cannot allocate device memory themselves
 * (their device memory belongs to another allocator or runtime, or the call
 * sits in a loop that must not pay the implicit synchronisation of
 * cudaMalloc): d_data is the caller's device array of ncomp x nsites
 * doubles (component-major), out the caller's host array of 5*ncomp
 * doubles, per component {total, mean, variance, min, max} as
 * stats_field_q computes them, but over every site of d_data (there is no
 * status map; stats_field_q skips solid sites).  stream is a cudaStream_t
 * (NULL: the default stream).
 * Partial sums go to a static device array sized for at most
 * LUDWIG_GB_NOALLOC_MAX_NCOMP components; larger ncomp is rejected with
 * LUDWIG_GB_EINVAL.  The first call on each device looks up that array's
 * device address, so make it before any stream capture.  Calls that overlap
 * on the GPU share the array and race: order them (e.g. one stream). */
#define LUDWIG_GB_NOALLOC_MAX_NCOMP 5
int ludwig_gb_field_stats_noalloc(const double * d_data, long long nsites,
				  int ncomp, double * out, void * stream);

/*****************************************************************************
 *
 *  Learned corrector of a 2x-coarsened binary fluid.  No counterpart in the
 *  reference.  A 4-layer 3x3x3 convolutional network (32 channels, GELU;
 *  inputs phi, u, rho; outputs corrections of phi and u) runs on the coarse
 *  lattice after each coarse step.  Forward and backward passes are
 *  tensor-core implicit GEMMs (BF16 operands, FP32 accumulation); the
 *  parameters are FP32 and trained with Adam on the GPU.
 *
 *  Coarse extents: nz in {32, 64} or a multiple of 128, and ny a multiple
 *  of 128/nz when nz < 128.  Device arrays are component-major float:
 *  in5 = [phi, u_x, u_y, u_z, rho] x nsites, t4/out4 = 4 x nsites
 *  (normalised corrections: d phi / out_scale[0], d u_a / out_scale[1+a]).
 *
 *****************************************************************************/

typedef struct ludwig_gb_cnn_s ludwig_gb_cnn_t;

int ludwig_gb_cnn_create(const int ncoarse[3], unsigned long long seed,
			 ludwig_gb_cnn_t ** cnn);
int ludwig_gb_cnn_free(ludwig_gb_cnn_t * cnn);
/* number of float parameters: 4 x (27*32*32 weights + 32 biases) */
int ludwig_gb_cnn_nparams(void);
int ludwig_gb_cnn_params_get(ludwig_gb_cnn_t * cnn, float * host);
/* replaces the parameters and restarts the optimiser */
int ludwig_gb_cnn_params_set(ludwig_gb_cnn_t * cnn, const float * host);
/* gradients of the last loss_grad / train_step (host, nparams floats) */
int ludwig_gb_cnn_grads_get(ludwig_gb_cnn_t * cnn, float * host);
/* features = (in5 - in_off) * in_scale; corrections = out4 * out_scale */
int ludwig_gb_cnn_scales_set(ludwig_gb_cnn_t * cnn, const float in_off[5],
			     const float in_scale[5],
			     const float out_scale[4]);
int ludwig_gb_cnn_scales_get(ludwig_gb_cnn_t * cnn, float in_off[5],
			     float in_scale[5], float out_scale[4]);
int ludwig_gb_cnn_forward(ludwig_gb_cnn_t * cnn, const float * d_in5,
			  float * d_out4);
/* n forward passes issued back to back on the library's stream (inputs
 * and outputs: n device pointers each); the error word of the tensor-core
 * kernels is read once, after the last */
int ludwig_gb_cnn_forward_n(ludwig_gb_cnn_t * cnn, int n,
			    const float * const * d_in5,
			    float * const * d_out4);
/* loss = (1/N) sum over sites and 4 outputs of (out4 - t4)^2 and its
 * gradient (no update) */
int ludwig_gb_cnn_loss_grad(ludwig_gb_cnn_t * cnn, const float * d_in5,
			    const float * d_t4, double * loss);
/* one Adam step (beta 0.9, 0.999, eps 1e-8) on one pair */
int ludwig_gb_cnn_train_step(ludwig_gb_cnn_t * cnn, const float * d_in5,
			     const float * d_t4, double lr, double * loss);
int ludwig_gb_cnn_train_steps(ludwig_gb_cnn_t * cnn, int nsteps,
			      const float * const * d_in5,
			      const float * const * d_t4, double lr,
			      double * losses);
/* apply the network to a coarse FP32 state in place: phi, u, and f
 * shifted by w_p rho 3 c_p . du (momentum changed by rho du) */
int ludwig_gb_cnn_correct(ludwig_gb_cnn_t * cnn, lb_t * lb, field_t * phi,
			  hydro_t * hydro);
/* Where nz is a multiple of 128 the convolutions reuse neighbour lines:
 * mode 1 stores a line as 4 unswizzled planes of 8 channels, mode 2 as
 * 64-byte-swizzled rows, mode 3 (nz = 128; mode 1 otherwise) as mode 1
 * with the three z taps of a line in one tensor-core MMA, mode 4 (nz =
 * 128; mode 1 otherwise) as mode 3 with the last layer's three y taps in
 * its MMAs as well (one MMA per x neighbour line), mode 5 (nz = 128; mode
 * 1 otherwise) as mode 4 on 64-byte-swizzled lines; mode 0: one TMA box
 * per tap (any supported extents).  Default: 5 where nz = 128, else 1 */
int ludwig_gb_cnn_line_reuse(ludwig_gb_cnn_t * cnn, int mode);
/* Failure detection of the tensor-core kernels: runs one device wait that
 * nothing satisfies; returns LUDWIG_GB_ETIMEOUT once the bounded wait has
 * given up and the kernel has returned (the context stays usable), with
 * the kernel's duration in *seconds */
int ludwig_gb_selftest_bounded_wait(double * seconds);
/* one convolution / weight gradient on given fp32 device arrays
 * (operands rounded to bf16), for checks of the kernels themselves:
 * flip = 0: out[s][n] = b[n] + sum_t sum_c a[s+e_t][c] w[t][n][c];
 * flip = 1: out[s][c] = sum_t sum_n a[s-e_t][n] w[t][n][c];
 * wgrad:    dw[t][n][c] = sum_s g[s-e_t][n] a[s][c]. */
int ludwig_gb_cnn_conv3(ludwig_gb_cnn_t * cnn, const float * d_a,
			const float * d_w, const float * d_b, int flip,
			float * d_out);
int ludwig_gb_cnn_wgrad3(ludwig_gb_cnn_t * cnn, const float * d_g,
			 const float * d_a, float * d_dw);

/* Fine (2n) -> coarse (n) FP32 state: phi and rho averaged, velocities
 * x 2, non-equilibrium stress x 4 (diffusive scaling dx x 2, dt x 4);
 * coarse f rebuilt from its moments. */
int ludwig_gb_coarse_restrict(lb_t * lb_fine, field_t * phi_fine,
			      hydro_t * hydro_fine, lb_t * lb_coarse,
			      field_t * phi_coarse, hydro_t * hydro_coarse);
/* restricted fields of a fine FP32 state into d_out5 (coarse extents nc) */
int ludwig_gb_fields_restrict(field_t * phi_fine, hydro_t * hydro_fine,
			      lb_t * lb_fine, float * d_out5, const int nc[3]);
/* [phi, u, rho] of an FP32 state into d_out5 */
int ludwig_gb_fields_pack(field_t * phi, hydro_t * hydro, lb_t * lb,
			  float * d_out5);
/* Make phys the physics object the step functions read (the reference
 * keeps one per process, src/physics.c:76; two systems with different
 * mobilities take turns). */
int ludwig_gb_physics_use(physics_t * phys);

/*---------------------------------------------------------------------------
 * Snapshot (restart) files in the reference's format: one file per object
 * in the current directory, single rank, as lb_io_write/lb_io_read
 * (src/lb_data.c:1716-1830) and field_io_write/field_io_read
 * (src/field.c:1633-1737) write and read them:
 *   data      "<stub>-%9.9d.001-001" (stub "dist" or the field's name):
 *             the sites in x, y, z order (z fastest), one record each:
 *             binary, ndist*19 (or nf) native doubles; or ascii, " %22.15e"
 *             per value with a newline after each velocity's ndist values
 *             (lb) or after the nf values (field);
 *   metadata  "<stub>-metadata.001-001" (JSON, written with the first data
 *             file of the object).
 * Reduced-precision objects are written as the doubles of the reference's
 * f and read back into their own precision.
 *-------------------------------------------------------------------------*/
typedef struct io_event_s io_event_t;       /* accepted; may be NULL */
/* record formats of input and output (default binary), the
 * lb_data_options_t / field_options_t iodata.input/output.iorformat */
int lb_io_record_format_set(lb_t * lb, int iorformat_in, int iorformat_out);
int field_io_record_format_set(field_t * field, int iorformat_in,
			       int iorformat_out);
int lb_io_write(lb_t * lb, int timestep, io_event_t * event);
int lb_io_read(lb_t * lb, int timestep, io_event_t * event);
int field_io_write(field_t * field, int timestep, io_event_t * event);
int field_io_read(field_t * field, int timestep, io_event_t * event);
/* hydro_io_write / hydro_io_read (src/hydro.c:941-967): the fields "rho"
 * (1 value a site) and "vel" (3) in the field format */
int hydro_io_record_format_set(hydro_t * hydro, int iorformat_in,
			       int iorformat_out);
int hydro_io_write(hydro_t * hydro, int timestep, io_event_t * event);
int hydro_io_read(hydro_t * hydro, int timestep, io_event_t * event);

#ifdef __cplusplus
}
#endif

#endif
