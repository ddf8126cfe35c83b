/*****************************************************************************
 *
 *  ludwig_gb.c
 *
 *  Host side of libludwig_gb.so, in C: the objects and entry points of
 *  include/ludwig_gb.h on top of the kernel launchers of lgb_kernels.h.
 *
 *  State of the distributions.  The reference keeps f and, after
 *  lb_collide, overwrites it with post-collision values which
 *  lb_propagation then streams.  Here an lb_t carries a flag "pending":
 *  when set, the stored array holds post-collision values and the
 *  reference's f is their streamed image.  lb_propagation only sets the
 *  flag (streaming is folded into the next pull); the fused step keeps it
 *  set; any call that needs the reference's f materialises the stream
 *  first.  All of this is exact: streaming is a permutation.
 *
 *****************************************************************************/

#include <assert.h>
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "ludwig_gb.h"
#include "lgb_kernels.h"
#include "lgb_stats.h"
#include "lgb_lc.h"
#include "lgb_sk.h"
#include "lgb_internal.h"

#define NVEL LGB_NVEL

/*****************************************************************************
 *  Errors
 *****************************************************************************/

static __thread char last_error_[512] = "";

static int err_set(int code, const char * fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(last_error_, sizeof(last_error_), fmt, ap);
  va_end(ap);
  return code;
}

static int cuda_check(int rc, const char * where) {
  if (rc != 0) {
    return err_set(LUDWIG_GB_ECUDA, "%s: %s", where,
		   cudaGetErrorString((cudaError_t) rc));
  }
  return LUDWIG_GB_OK;
}

#define CK(call, where) do { int rc_ = (int) (call); \
    if (rc_) return cuda_check(rc_, where); } while (0)

const char * ludwig_gb_last_error(void) { return last_error_; }
const char * ludwig_gb_version(void) { return "ludwig-gb300 0.1"; }

/*****************************************************************************
 *  Library stream and scratch
 *****************************************************************************/

static cudaStream_t stream_ = NULL;
static double * red_scratch_ = NULL;
static int tune_xchunk_ = 0;         /* 0: balanced shares of the planes */
static int tune_ty_ = 8;
static int tune_minb_ = 3;
#define LGB_FP16_RESCALE_STEPS 256
static int tune_sites_ = 0;          /* sites per thread, float forms;
					0: two for FP16 storage, one for FP32 */
static int advection_order_ = 1;

/* src/advection.c:82: order of the advective fluxes of the per-function
 * Cahn-Hilliard and Beris-Edwards steps: 1 (upwind, the default), 2 or 3.
 * The fused steps use order 1 and reject the others. */
int advection_order_set(int n) {
  if (n < 1 || n > 3) return err_set(LUDWIG_GB_EINVAL, "advection order "
				     "1, 2 or 3");
  advection_order_ = n;
  return LUDWIG_GB_OK;
}

static int lib_init(void) {
  if (stream_ == NULL) {
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking),
       "cudaStreamCreate");
  }
  return LUDWIG_GB_OK;
}

static int red_scratch(double ** p) {
  if (red_scratch_ == NULL) {
    CK(cudaMalloc((void **) &red_scratch_, LGBK_RED_SCRATCH*sizeof(double)),
       "cudaMalloc(scratch)");
  }
  *p = red_scratch_;
  return LUDWIG_GB_OK;
}

void * ludwig_gb_stream(void) {
  if (lib_init()) return NULL;
  return (void *) stream_;
}

int ludwig_gb_sync(void) {
  if (lib_init()) return LUDWIG_GB_ECUDA;
  CK(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
  return LUDWIG_GB_OK;
}

int ludwig_gb_tune_set(int xchunk, int tile_y, int min_blocks) {
  if (xchunk < 0 || (tile_y != 4 && tile_y != 8 && tile_y != 16) ||
      min_blocks < 0 || min_blocks > 4) {
    return err_set(LUDWIG_GB_EINVAL, "tune: xchunk >= 0 (0: balanced "
		   "shares), tile_y in {4,8,16}, min_blocks in 0..4");
  }
  tune_xchunk_ = xchunk;
  tune_ty_ = tile_y;
  tune_minb_ = min_blocks;
  return LUDWIG_GB_OK;
}

int ludwig_gb_tune_sites(int sites_per_thread) {
  if (sites_per_thread < 0 || sites_per_thread > 2) {
    return err_set(LUDWIG_GB_EINVAL, "tune_sites: 0 (by form), 1 or 2");
  }
  tune_sites_ = sites_per_thread;
  return LUDWIG_GB_OK;
}

static size_t prec_size(int prec) {
  return (prec == LUDWIG_GB_FP64) ? 8 : ((prec == LUDWIG_GB_FP32) ? 4 : 2);
}

/* phi, u and rho are float in both reduced-precision forms */
static size_t field_size(int prec) { return (prec == LUDWIG_GB_FP64) ? 8 : 4; }
static int field_kprec(int prec) {
  return (prec == LUDWIG_GB_FP64) ? LGBK_PREC_FP64 : LGBK_PREC_FP32;
}

static int dev_alloc(void ** p, size_t bytes, const char * what) {
  *p = NULL;
  if (bytes == 0) return LUDWIG_GB_OK;
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    *p = NULL;
    return err_set(LUDWIG_GB_ENOMEM, "cudaMalloc(%s, %zu bytes) failed",
		   what, bytes);
  }
  return LUDWIG_GB_OK;
}

static void dev_free(void * p) { if (p) cudaFree(p); }

/*****************************************************************************
 *  pe_t, cs_t, physics_t
 *****************************************************************************/

struct pe_s { int device; };

int pe_create(int device, pe_t ** ppe) {
  if (ppe == NULL) return err_set(LUDWIG_GB_EINVAL, "pe_create: NULL");
  CK(cudaSetDevice(device), "cudaSetDevice");
  pe_t * pe = (pe_t *) calloc(1, sizeof(pe_t));
  if (pe == NULL) return err_set(LUDWIG_GB_ENOMEM, "pe_create");
  pe->device = device;
  *ppe = pe;
  return lib_init();
}

int pe_free(pe_t * pe) { free(pe); return LUDWIG_GB_OK; }

struct cs_s {
  int ntotal[3];
  int nhalo;
  int initialised;
  lgbk_dims_t d;
};

int cs_create(pe_t * pe, cs_t ** pcs) {
  (void) pe;
  if (pcs == NULL) return err_set(LUDWIG_GB_EINVAL, "cs_create: NULL");
  cs_t * cs = (cs_t *) calloc(1, sizeof(cs_t));
  if (cs == NULL) return err_set(LUDWIG_GB_ENOMEM, "cs_create");
  cs->ntotal[0] = cs->ntotal[1] = cs->ntotal[2] = 64;   /* src/coords.c */
  cs->nhalo = 1;
  *pcs = cs;
  return LUDWIG_GB_OK;
}

int cs_free(cs_t * cs) { free(cs); return LUDWIG_GB_OK; }

int cs_ntotal_set(cs_t * cs, const int ntotal[3]) {
  if (cs == NULL || ntotal == NULL) return err_set(LUDWIG_GB_EINVAL, "cs");
  if (cs->initialised) return err_set(LUDWIG_GB_ESTATE, "cs initialised");
  for (int i = 0; i < 3; i++) {
    if (ntotal[i] < 2) {
      return err_set(LUDWIG_GB_EINVAL, "cs_ntotal_set: every extent >= 2");
    }
    cs->ntotal[i] = ntotal[i];
  }
  return LUDWIG_GB_OK;
}

int cs_nhalo_set(cs_t * cs, int nhalo) {
  if (cs == NULL || nhalo < 0) return err_set(LUDWIG_GB_EINVAL, "nhalo");
  if (cs->initialised) return err_set(LUDWIG_GB_ESTATE, "cs initialised");
  cs->nhalo = nhalo;
  return LUDWIG_GB_OK;
}

int cs_init(cs_t * cs) {
  if (cs == NULL) return err_set(LUDWIG_GB_EINVAL, "cs_init: NULL");
  cs->d.nx = cs->ntotal[0];
  cs->d.ny = cs->ntotal[1];
  cs->d.nz = cs->ntotal[2];
  cs->d.nsites = (long long) cs->d.nx*cs->d.ny*cs->d.nz;
  if (cs->d.nsites >= LGBK_MAX_SITES) {
    return err_set(LUDWIG_GB_EINVAL, "cs_init: %lld sites; the lattice "
		   "must hold fewer than 2^32", cs->d.nsites);
  }
  cs->initialised = 1;
  return LUDWIG_GB_OK;
}

int cs_nlocal(cs_t * cs, int nlocal[3]) {
  if (cs == NULL || !cs->initialised) {
    return err_set(LUDWIG_GB_ESTATE, "cs not initialised");
  }
  nlocal[0] = cs->d.nx; nlocal[1] = cs->d.ny; nlocal[2] = cs->d.nz;
  return LUDWIG_GB_OK;
}

int cs_ntotal(cs_t * cs, int ntotal[3]) {
  if (cs == NULL || ntotal == NULL) return err_set(LUDWIG_GB_EINVAL, "cs");
  for (int i = 0; i < 3; i++) ntotal[i] = cs->ntotal[i];
  return LUDWIG_GB_OK;
}

int cs_nhalo(cs_t * cs, int * nhalo) {
  if (cs == NULL || nhalo == NULL) return err_set(LUDWIG_GB_EINVAL, "cs");
  *nhalo = cs->nhalo;
  return LUDWIG_GB_OK;
}

/* Extents with the halo, src/coords.c (cs_nall) */
int cs_nall(cs_t * cs, int nall[3]) {
  if (cs == NULL || nall == NULL) return err_set(LUDWIG_GB_EINVAL, "cs");
  for (int i = 0; i < 3; i++) nall[i] = cs->ntotal[i] + 2*cs->nhalo;
  return LUDWIG_GB_OK;
}

int cs_nsites(cs_t * cs, int * nsites) {
  int n[3];
  int rc = cs_nall(cs, n);
  if (rc) return rc;
  if (nsites == NULL) return err_set(LUDWIG_GB_EINVAL, "cs_nsites");
  *nsites = n[0]*n[1]*n[2];
  return LUDWIG_GB_OK;
}

int cs_strides(cs_t * cs, int * xs, int * ys, int * zs) {
  int n[3];
  int rc = cs_nall(cs, n);
  if (rc) return rc;
  *xs = n[1]*n[2];
  *ys = n[2];
  *zs = 1;
  return LUDWIG_GB_OK;
}

/* src/coords.c:617-631: ic, jc, kc from 1 - nhalo to L + nhalo */
int cs_index(cs_t * cs, int ic, int jc, int kc) {
  int xs = 0, ys = 0, zs = 0;
  if (cs_strides(cs, &xs, &ys, &zs)) return -1;
  return xs*(cs->nhalo + ic - 1) + ys*(cs->nhalo + jc - 1)
    + zs*(cs->nhalo + kc - 1);
}

/* src/coords.c:790-801 */
int cs_index_to_ijk(cs_t * cs, int index, int coords[3]) {
  int xs = 0, ys = 0, zs = 0;
  int rc = cs_strides(cs, &xs, &ys, &zs);
  if (rc) return rc;
  coords[0] = (1 - cs->nhalo) + index/xs;
  coords[1] = (1 - cs->nhalo) + (index % xs)/ys;
  coords[2] = (1 - cs->nhalo) + index % ys;
  return LUDWIG_GB_OK;
}

/* Interior site (0-based, ((x*Ly + y)*Lz + z)) of a cs_index() site: halo
 * sites are the periodic images of the interior sites they copy.  -1 if
 * the index is not a site of the lattice with its halo. */
static long long cs_interior(const cs_t * cs, int index) {
  const int h = cs->nhalo;
  const int ny = cs->ntotal[1] + 2*h, nz = cs->ntotal[2] + 2*h;
  const long long nall = (long long) (cs->ntotal[0] + 2*h)*ny*nz;
  if (index < 0 || index >= nall) return -1;
  int c[3] = {index/(ny*nz), (index % (ny*nz))/nz, index % nz};
  for (int a = 0; a < 3; a++) {
    int n = cs->ntotal[a];
    c[a] = ((c[a] - h) % n + n) % n;
  }
  return ((long long) c[0]*cs->ntotal[1] + c[1])*cs->ntotal[2] + c[2];
}

struct physics_s {
  double rho0;
  double eta_shear;
  double eta_bulk;
  double mobility;
  double fbody[3];
  double e0_frequency;          /* frequency of the external electric field */
  int t_start;                  /* time step control, src/physics.c:600-668 */
  int nsteps;
  int t_current;
};

static physics_t * phys_ref_ = NULL;

int physics_create(pe_t * pe, physics_t ** phys) {
  (void) pe;
  if (phys == NULL) return err_set(LUDWIG_GB_EINVAL, "physics_create");
  physics_t * p = (physics_t *) calloc(1, sizeof(physics_t));
  if (p == NULL) return err_set(LUDWIG_GB_ENOMEM, "physics_create");
  /* Defaults of src/physics.c:108-111 */
  p->eta_shear = 1.0/6.0;
  p->eta_bulk = 1.0/6.0;
  p->rho0 = 1.0;
  phys_ref_ = p;
  *phys = p;
  return LUDWIG_GB_OK;
}

int physics_free(physics_t * phys) {
  if (phys == phys_ref_) phys_ref_ = NULL;
  free(phys);
  return LUDWIG_GB_OK;
}

int physics_ref(physics_t ** ref) { *ref = phys_ref_; return LUDWIG_GB_OK; }

int physics_e0_frequency_set(physics_t * p, double f) {
  if (p == NULL) return err_set(LUDWIG_GB_EINVAL, "physics");
  p->e0_frequency = f;
  return LUDWIG_GB_OK;
}

int physics_e0_frequency(physics_t * p, double * f) {
  if (p == NULL || f == NULL) return err_set(LUDWIG_GB_EINVAL, "physics");
  *f = p->e0_frequency;
  return LUDWIG_GB_OK;
}

/* src/physics.c:658-668 */
int physics_control_init_time(physics_t * p, int nstart, int nstep) {
  if (p == NULL) return err_set(LUDWIG_GB_EINVAL, "physics");
  p->t_start = nstart;
  p->nsteps = nstep;
  p->t_current = nstart;
  return LUDWIG_GB_OK;
}

/* src/physics.c:641-647: advance the step counter; positive while steps
 * of the run remain */
int physics_control_next_step(physics_t * p) {
  if (p == NULL) return 0;
  p->t_current += 1;
  return p->t_start + p->nsteps - p->t_current + 1;
}

int physics_control_timestep(physics_t * p) {
  return (p == NULL) ? 0 : p->t_current;
}

/* src/physics.c:622-630: the time in lattice units, 1.0 in the first
 * iteration of a run started at 0 */
int physics_control_time(physics_t * p, double * t) {
  if (p == NULL || t == NULL) return err_set(LUDWIG_GB_EINVAL, "physics");
  *t = 1.0*(p->t_start + p->t_current - 1.0);
  return LUDWIG_GB_OK;
}
int physics_rho0_set(physics_t * p, double v) { p->rho0 = v; return 0; }
int physics_eta_shear_set(physics_t * p, double v) { p->eta_shear = v; return 0; }
int physics_eta_bulk_set(physics_t * p, double v) { p->eta_bulk = v; return 0; }
int physics_mobility_set(physics_t * p, double v) { p->mobility = v; return 0; }
int physics_fbody_set(physics_t * p, const double f[3]) {
  for (int i = 0; i < 3; i++) p->fbody[i] = f[i];
  return 0;
}

static int phys_get(physics_t ** p) {
  if (phys_ref_ == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "no physics_t: call physics_create()");
  }
  *p = phys_ref_;
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  lb_t
 *****************************************************************************/

struct lb_data_s {
  cs_t * cs;
  int prec;
  lb_relaxation_enum_t nrelax;
  double fscale;                /* FP16 storage: f - w_p rho0 scaled by it */
  int fp16_since;               /* steps since the scale was last derived */
  double rho0;                 /* shift of the reduced-precision storage */
  void * f;
  void * fprime;
  int pending;                 /* stored values await streaming */
  int ndist;                   /* 1, or 2 with the order parameter in g */
  void * g;                    /* ndist = 2: g and its second buffer */
  void * gprime;
  lgb_io_state_t io;           /* snapshot files */
};

/* src/io_options.c:26-40, src/io_info_args.c:28-35 */
io_options_t io_options_default(void) {
  io_options_t o = {IO_MODE_MPIIO, IO_RECORD_BINARY, IO_METADATA_V2, 0, 0, 0,
		    {1, 1, 1}};
  return o;
}

io_info_args_t io_info_args_default(void) {
  io_info_args_t a;
  a.input = io_options_default();
  a.output = io_options_default();
  a.grid[0] = a.grid[1] = a.grid[2] = 1;
  a.iofreq = 0;
  return a;
}

/* record format of a side of iodata (binary unless ascii is asked for) */
static int io_format_of(const io_options_t * o) {
  return (o->iorformat == IO_RECORD_ASCII) ? IO_RECORD_ASCII
    : IO_RECORD_BINARY;
}

/* src/lb_data_options.c:28-57 */
lb_data_options_t lb_data_options_default(void) {
  lb_data_options_t o;
  memset(&o, 0, sizeof(o));
  o.ndim = 3;
  o.nvel = 19;
  o.ndist = 1;
  o.nrelax = LB_RELAXATION_M10;
  o.halo = LB_HALO_FULL;
  o.reportimbalance = 0;
  o.usefirsttouch = 0;
  o.iodata = io_info_args_default();
  return o;
}

lb_data_options_t lb_data_options_ndim_nvel_ndist(int ndim, int nvel,
						  int ndist) {
  lb_data_options_t o = lb_data_options_default();
  o.ndim = ndim;
  o.nvel = nvel;
  o.ndist = ndist;
  return o;
}

int lb_data_create(pe_t * pe, cs_t * cs, const lb_data_options_t * opts,
		   lb_t ** plb) {
  return ludwig_gb_lb_data_create(pe, cs, opts, LUDWIG_GB_FP64, 0.0, plb);
}

int ludwig_gb_lb_data_create(pe_t * pe, cs_t * cs,
			     const lb_data_options_t * opts, int precision,
			     double fp16_scale, lb_t ** plb) {
  (void) pe;
  lb_data_options_t o = opts ? *opts : lb_data_options_default();
  if (cs == NULL || !cs->initialised || plb == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "lb_data_create: cs not initialised");
  }
  if (o.ndim != 3 || o.nvel != 19 || (o.ndist != 1 && o.ndist != 2)) {
    return err_set(LUDWIG_GB_EINVAL, "lb_data_create: D3Q19, ndist 1 or 2");
  }
  if (o.ndist == 2 && precision != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "lb_data_create: ndist 2 is FP64");
  }
  if (precision < LUDWIG_GB_FP64 || precision > LUDWIG_GB_FP16) {
    return err_set(LUDWIG_GB_EINVAL, "lb_data_create: precision");
  }
  if (o.nrelax < LB_RELAXATION_M10 || o.nrelax > LB_RELAXATION_TRT) {
    return err_set(LUDWIG_GB_EINVAL, "lb_data_create: nrelax");
  }
  int rc = lib_init();
  if (rc) return rc;

  lb_t * lb = (lb_t *) calloc(1, sizeof(lb_t));
  if (lb == NULL) return err_set(LUDWIG_GB_ENOMEM, "lb_data_create");
  lb->cs = cs;
  lb->prec = precision;
  lb->nrelax = o.nrelax;
  lb->fscale = (fp16_scale > 0.0) ? fp16_scale : 1024.0;
  lb->io.fmt_in = io_format_of(&o.iodata.input);
  lb->io.fmt_out = io_format_of(&o.iodata.output);
  lb->rho0 = phys_ref_ ? phys_ref_->rho0 : 1.0;

  size_t bytes = NVEL*(size_t) cs->d.nsites*prec_size(lb->prec);
  lb->ndist = o.ndist;
  if ((rc = dev_alloc(&lb->f, bytes, "f")) ||
      (rc = dev_alloc(&lb->fprime, bytes, "fprime"))) {
    lb_free(lb);
    return rc;
  }
  if (lb->ndist == 2) {
    if ((rc = dev_alloc(&lb->g, bytes, "g")) ||
	(rc = dev_alloc(&lb->gprime, bytes, "gprime"))) {
      lb_free(lb);
      return rc;
    }
    if (cudaMemsetAsync(lb->g, 0, bytes, stream_) != cudaSuccess) {
      lb_free(lb);
      return err_set(LUDWIG_GB_ECUDA, "lb_data_create: memset g");
    }
  }
  *plb = lb;
  return lb_init_rest_f(lb, lb->rho0);
}

int lb_free(lb_t * lb) {
  if (lb) {
    dev_free(lb->f);
    dev_free(lb->fprime);
    dev_free(lb->g);
    dev_free(lb->gprime);
    free(lb);
  }
  return LUDWIG_GB_OK;
}

static void lb_swap(lb_t * lb) {
  void * t = lb->f; lb->f = lb->fprime; lb->fprime = t;
}

static void lb_swap_g(lb_t * lb) {
  void * t = lb->g; lb->g = lb->gprime; lb->gprime = t;
}

/* Make the stored arrays hold the reference's f (and g) (apply pending
 * streaming) */
static int lb_materialise(lb_t * lb) {
  if (!lb->pending) return LUDWIG_GB_OK;
  CK(lgbk_propagate_store(&lb->cs->d, lb->prec, +1, lb->f, lb->fprime,
			  stream_), "propagate");
  lb_swap(lb);
  if (lb->ndist == 2) {
    CK(lgbk_propagate_store(&lb->cs->d, lb->prec, +1, lb->g, lb->gprime,
			    stream_), "propagate g");
    lb_swap_g(lb);
  }
  lb->pending = 0;
  return LUDWIG_GB_OK;
}

/* Make the stored arrays hold post-collision values (pending = 1) */
static int lb_unstream(lb_t * lb) {
  if (lb->pending) return LUDWIG_GB_OK;
  CK(lgbk_propagate_store(&lb->cs->d, lb->prec, -1, lb->f, lb->fprime,
			  stream_), "unstream");
  lb_swap(lb);
  if (lb->ndist == 2) {
    CK(lgbk_propagate_store(&lb->cs->d, lb->prec, -1, lb->g, lb->gprime,
			    stream_), "unstream g");
    lb_swap_g(lb);
  }
  lb->pending = 1;
  return LUDWIG_GB_OK;
}

/* src/lb_data.c:659-680 and :809-834 with u = 0: f_p = rho0 w_p */
int lb_init_rest_f(lb_t * lb, double rho0) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "lb_init_rest_f");
  const lgbk_dims_t * d = &lb->cs->d;
  double * tmp = NULL;
  int rc = dev_alloc((void **) &tmp, NVEL*(size_t) d->nsites*sizeof(double),
		     "init");
  if (rc) return rc;
  for (int p = 0; p < NVEL; p++) {
    static const int w36[NVEL] = {12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1,
				  1, 1, 2, 1, 1};
    double w = (double) w36[p]/36.0;
    rc = lgbk_fill_f64(tmp + p*d->nsites, d->nsites, rho0*w*1.0, stream_);
    if (rc) break;
  }
  if (rc == 0) {
    rc = lgbk_f64_to_store(d, lb->prec, NVEL, lb->rho0, lb->fscale, tmp,
			   lb->f, stream_);
  }
  if (rc == 0) rc = cudaStreamSynchronize(stream_);
  dev_free(tmp);
  lb->pending = 0;
  return cuda_check(rc, "lb_init_rest_f");
}

int lb_halo(lb_t * lb) {
  /* Periodic images are read in place by every kernel. */
  return (lb == NULL) ? err_set(LUDWIG_GB_EINVAL, "lb_halo") : LUDWIG_GB_OK;
}

int lb_f_to_host(lb_t * lb, double * fh) {
  if (lb == NULL || fh == NULL) return err_set(LUDWIG_GB_EINVAL, "lb_f");
  const lgbk_dims_t * d = &lb->cs->d;
  const void * src = lb->f;
  size_t n = NVEL*(size_t) d->nsites;
  if (lb->pending) {
    CK(lgbk_propagate_store(d, lb->prec, +1, lb->f, lb->fprime, stream_),
       "propagate");
    src = lb->fprime;
  }
  if (lb->prec == LUDWIG_GB_FP64) {
    CK(cudaMemcpyAsync(fh, src, n*sizeof(double), cudaMemcpyDeviceToHost,
		       stream_), "lb_f_to_host");
  }
  else {
    double * tmp = NULL;
    int rc = dev_alloc((void **) &tmp, n*sizeof(double), "convert");
    if (rc) return rc;
    rc = lgbk_store_to_f64(d, lb->prec, NVEL, lb->rho0, lb->fscale, src, tmp,
			   stream_);
    if (rc == 0) rc = cudaMemcpyAsync(fh, tmp, n*sizeof(double),
				      cudaMemcpyDeviceToHost, stream_);
    if (rc == 0) rc = cudaStreamSynchronize(stream_);
    dev_free(tmp);
    return cuda_check(rc, "lb_f_to_host");
  }
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* FP16 storage scale for deviations of magnitude up to maxdev: the power of
 * two that maps maxdev into [2^10, 2^11) (room for the deviations to grow
 * 32-fold before half precision's largest value, 65504, between two
 * derivations; the relative precision of half does not depend on the
 * scale, which only keeps the values out of the subnormal range), between
 * 1 and 2^24; 0 if maxdev is zero (keep the scale) */
static double fp16_scale_for(double maxdev) {
  if (!(maxdev > 0.0) || !isfinite(maxdev)) return 0.0;
  int e = 0;
  (void) frexp(2048.0/maxdev, &e);             /* 2048/maxdev in [2^(e-1), 2^e) */
  double sc = ldexp(1.0, e - 1);
  if (sc < 1.0) sc = 1.0;
  if (sc > 16777216.0) sc = 16777216.0;
  return sc;
}

int lb_f_from_host(lb_t * lb, const double * fh) {
  if (lb == NULL || fh == NULL) return err_set(LUDWIG_GB_EINVAL, "lb_f");
  if (lb->ndist == 2) {
    int rc0 = lb_materialise(lb);        /* g keeps its streamed values */
    if (rc0) return rc0;
  }
  const lgbk_dims_t * d = &lb->cs->d;
  size_t n = NVEL*(size_t) d->nsites;
  if (lb->prec == LUDWIG_GB_FP64) {
    CK(cudaMemcpyAsync(lb->f, fh, n*sizeof(double), cudaMemcpyHostToDevice,
		       stream_), "lb_f_from_host");
  }
  else {
    if (lb->prec == LUDWIG_GB_FP16) {
      /* the storage scale from the range of the deviations handed over */
      static const int w36[NVEL] = {12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2,
				    1, 1, 1, 2, 1, 1};
      double m = 0.0;
      for (int p = 0; p < NVEL; p++) {
	const double w = lb->rho0*((double) w36[p]/36.0);
	const double * fp = fh + (size_t) p*d->nsites;
	for (long long i = 0; i < d->nsites; i++) {
	  m = fmax(m, fabs(fp[i] - w));
	}
      }
      double sc = fp16_scale_for(m);
      if (sc > 0.0) lb->fscale = sc;
      lb->fp16_since = 0;
    }
    double * tmp = NULL;
    int rc = dev_alloc((void **) &tmp, n*sizeof(double), "convert");
    if (rc) return rc;
    rc = cudaMemcpyAsync(tmp, fh, n*sizeof(double), cudaMemcpyHostToDevice,
			 stream_);
    if (rc == 0) rc = lgbk_f64_to_store(d, lb->prec, NVEL, lb->rho0,
					lb->fscale, tmp, lb->f, stream_);
    if (rc == 0) rc = cudaStreamSynchronize(stream_);
    dev_free(tmp);
    if (rc) return cuda_check(rc, "lb_f_from_host");
  }
  CK(cudaStreamSynchronize(stream_), "sync");
  lb->pending = 0;
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  field_t, field_grad_t
 *****************************************************************************/

struct field_s {
  cs_t * cs;
  int nf;
  int nhcomm;
  int prec;
  char name[32];
  void * data;
  void * data2;                /* second buffer for the fused step */
  lgb_io_state_t io;           /* snapshot files */
};

/* src/field_options.c:27-52 */
field_options_t field_options_default(void) {
  field_options_t o;
  memset(&o, 0, sizeof(o));
  o.ndata = 1;
  o.nhcomm = 0;
  o.haloscheme = FIELD_HALO_TARGET;
  o.haloverbose = 0;
  o.usefirsttouch = 0;
  o.iodata = io_info_args_default();
  return o;
}

field_options_t field_options_ndata_nhalo(int ndata, int nhalo) {
  field_options_t o = field_options_default();
  o.ndata = ndata;
  o.nhcomm = nhalo;
  return o;
}

int field_create(pe_t * pe, cs_t * cs, lees_edw_t * le, const char * name,
		 const field_options_t * opts, field_t ** pobj) {
  return ludwig_gb_field_create(pe, cs, le, name, opts, LUDWIG_GB_FP64, pobj);
}

int ludwig_gb_field_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
			   const char * name, const field_options_t * opts,
			   int precision, field_t ** pobj) {
  (void) pe;
  if (le != NULL) return err_set(LUDWIG_GB_EINVAL, "Lees-Edwards planes");
  if (cs == NULL || !cs->initialised || opts == NULL || pobj == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "field_create");
  }
  if (opts->ndata < 1 || opts->ndata > 5) {
    return err_set(LUDWIG_GB_EINVAL, "field_create: ndata in 1..5");
  }
  if (precision < LUDWIG_GB_FP64 || precision > LUDWIG_GB_FP16) {
    return err_set(LUDWIG_GB_EINVAL, "field_create: precision");
  }
  int rc = lib_init();
  if (rc) return rc;
  field_t * f = (field_t *) calloc(1, sizeof(field_t));
  if (f == NULL) return err_set(LUDWIG_GB_ENOMEM, "field_create");
  f->cs = cs;
  f->nf = opts->ndata;
  f->nhcomm = opts->nhcomm;
  f->prec = precision;
  f->io.fmt_in = io_format_of(&opts->iodata.input);
  f->io.fmt_out = io_format_of(&opts->iodata.output);
  snprintf(f->name, sizeof(f->name), "%s", name ? name : "field");
  size_t bytes = (size_t) f->nf*cs->d.nsites*field_size(f->prec);
  if ((rc = dev_alloc(&f->data, bytes, "field")) ||
      (rc = dev_alloc(&f->data2, bytes, "field2"))) {
    field_free(f);
    return rc;
  }
  CK(cudaMemsetAsync(f->data, 0, bytes, stream_), "memset");
  CK(cudaStreamSynchronize(stream_), "sync");
  *pobj = f;
  return LUDWIG_GB_OK;
}

int field_free(field_t * f) {
  if (f) { dev_free(f->data); dev_free(f->data2); free(f); }
  return LUDWIG_GB_OK;
}

int field_nf(field_t * f, int * nf) { *nf = f->nf; return LUDWIG_GB_OK; }

int field_halo(field_t * f) {
  return (f == NULL) ? err_set(LUDWIG_GB_EINVAL, "field_halo") : LUDWIG_GB_OK;
}

static int copy_to_host(int prec, long long n, const void * src, double * dst) {
  if (prec == LUDWIG_GB_FP64) {
    CK(cudaMemcpyAsync(dst, src, n*sizeof(double), cudaMemcpyDeviceToHost,
		       stream_), "to_host");
    CK(cudaStreamSynchronize(stream_), "sync");
    return LUDWIG_GB_OK;
  }
  float * tmp = (float *) malloc(n*sizeof(float));
  if (tmp == NULL) return err_set(LUDWIG_GB_ENOMEM, "to_host");
  int rc = cudaMemcpyAsync(tmp, src, n*sizeof(float), cudaMemcpyDeviceToHost,
			   stream_);
  if (rc == 0) rc = cudaStreamSynchronize(stream_);
  for (long long i = 0; rc == 0 && i < n; i++) dst[i] = tmp[i];
  free(tmp);
  return cuda_check(rc, "to_host");
}

static int copy_from_host(int prec, long long n, const double * src,
			  void * dst) {
  if (prec == LUDWIG_GB_FP64) {
    CK(cudaMemcpyAsync(dst, src, n*sizeof(double), cudaMemcpyHostToDevice,
		       stream_), "from_host");
    CK(cudaStreamSynchronize(stream_), "sync");
    return LUDWIG_GB_OK;
  }
  float * tmp = (float *) malloc(n*sizeof(float));
  if (tmp == NULL) return err_set(LUDWIG_GB_ENOMEM, "from_host");
  for (long long i = 0; i < n; i++) tmp[i] = (float) src[i];
  int rc = cudaMemcpyAsync(dst, tmp, n*sizeof(float), cudaMemcpyHostToDevice,
			   stream_);
  if (rc == 0) rc = cudaStreamSynchronize(stream_);
  free(tmp);
  return cuda_check(rc, "from_host");
}

int field_to_host(field_t * f, double * data) {
  if (f == NULL || data == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  return copy_to_host(f->prec, f->nf*f->cs->d.nsites, f->data, data);
}

int field_from_host(field_t * f, const double * data) {
  if (f == NULL || data == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  return copy_from_host(f->prec, f->nf*f->cs->d.nsites, data, f->data);
}

/* KISS99-type generator of src/noise.h:96-112 and the per-site seeding of
 * src/noise.c:278-340; spinodal phi = phi0 + amp (r - 1/2),
 * src/field_phi_init.c:484-518.  Global coordinates are 1-based. */

static unsigned int kiss(unsigned int s[4]) {
  unsigned int b;
  s[0] = 69069u*s[0] + 1234567u;
  b = s[1] ^ (s[1] << 17);
  b ^= (b >> 13);
  s[1] = b ^ (b << 5);
  s[2] = 36969u*(s[2] & 0xffffu) + (s[2] >> 16);
  s[3] = 18000u*(s[3] & 0xffffu) + (s[3] >> 16);
  b = (s[2] << 16) + s[3];
  return (s[1] + (s[0] ^ b));
}

/* src/field_phi_init.c:38-82: a drop phi(r) = phistar tanh((r - radius)/xi)
 * about the centre of the box (is_centred adds Lmin = 0.5, as the
 * reference's corrected form); sites at integer positions 1..L. */
int field_phi_init_drop(field_t * phi, double xi, double radius,
			double phistar, int is_centred) {
  if (phi == NULL || phi->nf != 1 || !(xi > 0.0)) {
    return err_set(LUDWIG_GB_EINVAL, "field_phi_init_drop");
  }
  const lgbk_dims_t * d = &phi->cs->d;
  double * h = (double *) malloc((size_t) d->nsites*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "field_phi_init_drop");
  const double lmin = 0.5;
  const double rxi0 = 1.0/xi;
  double centre[3];
  const int n[3] = {d->nx, d->ny, d->nz};
  for (int a = 0; a < 3; a++) centre[a] = is_centred*lmin + 0.5*n[a];
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	double pos[3] = {1.0*(x + 1) - centre[0], 1.0*(y + 1) - centre[1],
			 1.0*(z + 1) - centre[2]};
	double r = sqrt(pos[0]*pos[0] + pos[1]*pos[1] + pos[2]*pos[2]);
	h[((size_t) x*d->ny + y)*d->nz + z] = phistar*tanh(rxi0*(r - radius));
      }
    }
  }
  int rc = field_from_host(phi, h);
  free(h);
  return rc;
}

/* The first n uniform draws of the per-site generator of site (x, y, z)
 * (0-based), src/noise.c:278-340 and noise_uniform_double_reap
 * (src/noise.c:437): each draw advances the site's state */
static void site_uniforms(unsigned int seed0, int x, int y, int z, int n,
			  double * out) {
  unsigned int sl[4], st[4];
  sl[0] = seed0 + (unsigned int) (x + 1);
  sl[1] = 12953u + (unsigned int) (y + 1);
  sl[2] = 712357u + (unsigned int) (z + 1);
  sl[3] = 22383979u;
  for (int k = 0; k < 4; k++) st[k] = kiss(sl);
  for (int k = 0; k < n; k++) out[k] = (1.0/UINT_MAX)*kiss(st);
}

static double site_uniform(unsigned int seed0, int x, int y, int z) {
  double r;
  site_uniforms(seed0, x, y, z, 1, &r);
  return r;
}

int field_phi_init_spinodal(field_t * phi, int seed, double phi0, double amp) {
  if (phi == NULL || phi->nf != 1) {
    return err_set(LUDWIG_GB_EINVAL, "field_phi_init_spinodal: scalar field");
  }
  const lgbk_dims_t * d = &phi->cs->d;
  double * h = (double *) malloc(d->nsites*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "spinodal");
  unsigned int seed0 = (seed > 1) ? (unsigned int) seed : 13u;
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	double ran = site_uniform(seed0, x, y, z);
	h[((long long) x*d->ny + y)*d->nz + z] = phi0 + amp*(ran - 0.5);
      }
    }
  }
  int rc = field_from_host(phi, h);
  free(h);
  return rc;
}

/* Spinodal patches, src/field_phi_init.c:537-590: cubes of patch^3 sites
 * (cut at the upper edges) of phi = -1 where the draw of the cube's first
 * site is below volminus1, +1 elsewhere */
int field_phi_init_spinodal_patches(field_t * phi, int seed, int patch,
				    double volminus1) {
  if (phi == NULL || phi->nf != 1 || patch < 1) {
    return err_set(LUDWIG_GB_EINVAL, "field_phi_init_spinodal_patches");
  }
  const lgbk_dims_t * d = &phi->cs->d;
  double * h = (double *) malloc(d->nsites*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "patches");
  unsigned int seed0 = (seed > 1) ? (unsigned int) seed : 13u;
  for (int x = 0; x < d->nx; x += patch) {
    for (int y = 0; y < d->ny; y += patch) {
      for (int z = 0; z < d->nz; z += patch) {
	const double phi1 = (site_uniform(seed0, x, y, z) < volminus1)
	  ? -1.0 : 1.0;
	for (int ip = x; ip < x + patch && ip < d->nx; ip++)
	  for (int jp = y; jp < y + patch && jp < d->ny; jp++)
	    for (int kp = z; kp < z + patch && kp < d->nz; kp++)
	      h[((long long) ip*d->ny + jp)*d->nz + kp] = phi1;
      }
    }
  }
  int rc = field_from_host(phi, h);
  free(h);
  return rc;
}

struct field_grad_s {
  field_t * field;
  int level;
  int stencil;                 /* 7 (3d_7pt_fluid) or 27 (3d_27pt_fluid) */
  double * grad;
  double * delsq;
};

int field_grad_create(pe_t * pe, field_t * f, int level, field_grad_t ** p) {
  (void) pe;
  if (f == NULL || p == NULL || level < 1) {
    return err_set(LUDWIG_GB_EINVAL, "field_grad_create");
  }
  field_grad_t * g = (field_grad_t *) calloc(1, sizeof(field_grad_t));
  if (g == NULL) return err_set(LUDWIG_GB_ENOMEM, "field_grad_create");
  g->field = f;
  g->level = level;
  g->stencil = 7;
  *p = g;
  return LUDWIG_GB_OK;
}

void field_grad_free(field_grad_t * g) {
  if (g) { dev_free(g->grad); dev_free(g->delsq); free(g); }
}

static int grad_alloc(field_grad_t * g) {
  if (g->grad) return LUDWIG_GB_OK;
  size_t n = (size_t) g->field->nf*g->field->cs->d.nsites;
  int rc = dev_alloc((void **) &g->grad, 3*n*sizeof(double), "grad");
  if (rc == 0) rc = dev_alloc((void **) &g->delsq, n*sizeof(double), "delsq");
  return rc;
}

/* The reference selects the stencil with field_grad_set(fg,
 * grad_3d_7pt_fluid_d2 | grad_3d_27pt_fluid_d2, NULL) (src/field_grad.c);
 * here by its number of points. */
int field_grad_stencil_set(field_grad_t * g, int npoints) {
  if (g == NULL || (npoints != 7 && npoints != 27)) {
    return err_set(LUDWIG_GB_EINVAL, "field_grad_stencil_set: 7 or 27");
  }
  g->stencil = npoints;
  return LUDWIG_GB_OK;
}

static int grad_launch(field_grad_t * g) {
  if (g->stencil == 27) {
    return lgbk_grad27_f64(&g->field->cs->d, g->field->nf,
			   (const double *) g->field->data, g->grad, g->delsq,
			   stream_);
  }
  return lgbk_grad7_f64(&g->field->cs->d, g->field->nf,
			(const double *) g->field->data, g->grad, g->delsq,
			stream_);
}

int field_grad_compute(field_grad_t * g) {
  if (g == NULL) return err_set(LUDWIG_GB_EINVAL, "field_grad_compute");
  if (g->field->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "field_grad_compute: FP64 fields only");
  }
  int rc = grad_alloc(g);
  if (rc) return rc;
  CK(grad_launch(g), "field_grad_compute");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int field_grad_to_host(field_grad_t * g, double * grad, double * delsq) {
  if (g == NULL || g->grad == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "field_grad_to_host: not computed");
  }
  long long n = (long long) g->field->nf*g->field->cs->d.nsites;
  int rc = LUDWIG_GB_OK;
  if (grad) rc = copy_to_host(LUDWIG_GB_FP64, 3*n, g->grad, grad);
  if (rc == 0 && delsq) rc = copy_to_host(LUDWIG_GB_FP64, n, g->delsq, delsq);
  return rc;
}

/*****************************************************************************
 *  hydro_t, map_t
 *****************************************************************************/

struct hydro_s {
  cs_t * cs;
  int prec;
  void * rho;
  void * u;
  void * u2;
  void * force;
  lgb_io_state_t io_rho;       /* snapshot files "rho" and "vel" */
  lgb_io_state_t io_vel;
};

/* src/hydro_options.c:32-72 */
hydro_options_t hydro_options_nhalo(int nhalo) {
  hydro_options_t o;
  memset(&o, 0, sizeof(o));
  o.nhcomm = nhalo;
  o.rho = field_options_ndata_nhalo(1, nhalo);
  o.u = field_options_ndata_nhalo(3, nhalo);
  o.force = field_options_ndata_nhalo(3, nhalo);
  o.eta = field_options_ndata_nhalo(1, nhalo);
  return o;
}

hydro_options_t hydro_options_default(void) {
  return hydro_options_nhalo(1);
}

int hydro_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		 const hydro_options_t * opts, hydro_t ** pobj) {
  return ludwig_gb_hydro_create(pe, cs, le, opts, LUDWIG_GB_FP64, pobj);
}

int ludwig_gb_hydro_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
			   const hydro_options_t * opts, int precision,
			   hydro_t ** pobj) {
  (void) pe;
  if (le != NULL) return err_set(LUDWIG_GB_EINVAL, "Lees-Edwards planes");
  if (cs == NULL || !cs->initialised || pobj == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "hydro_create");
  }
  if (precision < LUDWIG_GB_FP64 || precision > LUDWIG_GB_FP16) {
    return err_set(LUDWIG_GB_EINVAL, "hydro_create: precision");
  }
  hydro_options_t o = opts ? *opts : hydro_options_default();
  int rc = lib_init();
  if (rc) return rc;
  hydro_t * h = (hydro_t *) calloc(1, sizeof(hydro_t));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "hydro_create");
  h->cs = cs;
  h->prec = precision;
  h->io_rho.fmt_in = io_format_of(&o.rho.iodata.input);
  h->io_rho.fmt_out = io_format_of(&o.rho.iodata.output);
  h->io_vel.fmt_in = io_format_of(&o.u.iodata.input);
  h->io_vel.fmt_out = io_format_of(&o.u.iodata.output);
  size_t n = (size_t) cs->d.nsites, es = field_size(h->prec);
  if ((rc = dev_alloc(&h->rho, n*es, "rho")) ||
      (rc = dev_alloc(&h->u, 3*n*es, "u")) ||
      (rc = dev_alloc(&h->u2, 3*n*es, "u2")) ||
      (rc = dev_alloc(&h->force, 3*n*es, "force"))) {
    hydro_free(h);
    return rc;
  }
  CK(cudaMemsetAsync(h->u, 0, 3*n*es, stream_), "memset");
  CK(cudaMemsetAsync(h->force, 0, 3*n*es, stream_), "memset");
  CK(cudaMemsetAsync(h->rho, 0, n*es, stream_), "memset");
  CK(cudaStreamSynchronize(stream_), "sync");
  *pobj = h;
  return LUDWIG_GB_OK;
}

int hydro_free(hydro_t * h) {
  if (h) {
    dev_free(h->rho); dev_free(h->u); dev_free(h->u2); dev_free(h->force);
    free(h);
  }
  return LUDWIG_GB_OK;
}

static int fill3(hydro_t * h, void * a, const double v[3]) {
  long long n = h->cs->d.nsites;
  if (h->prec != LUDWIG_GB_FP64) {
    if (v[0] == 0.0 && v[1] == 0.0 && v[2] == 0.0) {
      CK(cudaMemsetAsync(a, 0, 3*n*sizeof(float), stream_), "memset");
      CK(cudaStreamSynchronize(stream_), "sync");
      return LUDWIG_GB_OK;
    }
    return err_set(LUDWIG_GB_EINVAL, "non-zero fill of a float field");
  }
  for (int i = 0; i < 3; i++) {
    CK(lgbk_fill_f64((double *) a + i*n, n, v[i], stream_), "fill");
  }
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int hydro_f_zero(hydro_t * h, const double fzero[3]) {
  if (h == NULL || fzero == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro");
  return fill3(h, h->force, fzero);
}

int hydro_u_zero(hydro_t * h, const double uzero[3]) {
  if (h == NULL || uzero == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro");
  return fill3(h, h->u, uzero);
}

int hydro_u_halo(hydro_t * h) {
  return (h == NULL) ? err_set(LUDWIG_GB_EINVAL, "hydro") : LUDWIG_GB_OK;
}

int hydro_to_host(hydro_t * h, double * rho, double * u, double * force) {
  if (h == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro_to_host");
  long long n = h->cs->d.nsites;
  int rc = LUDWIG_GB_OK;
  if (rho) rc = copy_to_host(h->prec, n, h->rho, rho);
  if (rc == 0 && u) rc = copy_to_host(h->prec, 3*n, h->u, u);
  if (rc == 0 && force) rc = copy_to_host(h->prec, 3*n, h->force, force);
  return rc;
}

int hydro_from_host(hydro_t * h, const double * rho, const double * u,
		    const double * force) {
  if (h == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro_from_host");
  long long n = h->cs->d.nsites;
  int rc = LUDWIG_GB_OK;
  if (rho) rc = copy_from_host(h->prec, n, rho, h->rho);
  if (rc == 0 && u) rc = copy_from_host(h->prec, 3*n, u, h->u);
  if (rc == 0 && force) rc = copy_from_host(h->prec, 3*n, force, h->force);
  return rc;
}

struct map_s {
  cs_t * cs;
  uint8_t * status;
  int all_fluid;
  long long nfluid;
};

/* src/map_options.c:26-52 */
map_options_t map_options_default(void) {
  map_options_t o;
  memset(&o, 0, sizeof(o));
  o.ndata = 0;
  o.is_porous_media = 0;
  o.filestub = "map";
  o.iodata = io_info_args_default();
  return o;
}

map_options_t map_options_ndata(int ndata) {
  map_options_t o = map_options_default();
  o.ndata = ndata;
  return o;
}

int map_create(pe_t * pe, cs_t * cs, const map_options_t * options,
	       map_t ** pobj) {
  (void) pe;
  if (cs == NULL || !cs->initialised || pobj == NULL || options == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "map_create");
  }
  if (options->ndata != 0 || options->is_porous_media != 0) {
    return err_set(LUDWIG_GB_EINVAL, "map_create: ndata 0 and no porous "
		   "media only");
  }
  int rc = lib_init();
  if (rc) return rc;
  map_t * m = (map_t *) calloc(1, sizeof(map_t));
  if (m == NULL) return err_set(LUDWIG_GB_ENOMEM, "map_create");
  m->cs = cs;
  m->all_fluid = 1;
  m->nfluid = cs->d.nsites;
  if ((rc = dev_alloc((void **) &m->status, (size_t) cs->d.nsites, "map"))) {
    free(m);
    return rc;
  }
  CK(cudaMemsetAsync(m->status, 0, (size_t) cs->d.nsites, stream_), "memset");
  CK(cudaStreamSynchronize(stream_), "sync");
  *pobj = m;
  return LUDWIG_GB_OK;
}

/* src/map.h:53: frees *map and sets it to NULL */
int map_free(map_t ** pm) {
  if (pm && *pm) {
    dev_free((*pm)->status);
    free(*pm);
    *pm = NULL;
  }
  return LUDWIG_GB_OK;
}

int map_status_from_host(map_t * m, const uint8_t * status) {
  if (m == NULL || status == NULL) return err_set(LUDWIG_GB_EINVAL, "map");
  long long n = m->cs->d.nsites;
  long long nfluid = 0;
  for (long long i = 0; i < n; i++) {
    if (status[i] >= MAP_STATUS_MAX) {
      return err_set(LUDWIG_GB_EINVAL, "map status value out of range");
    }
    if (status[i] == MAP_FLUID) nfluid += 1;
  }
  m->nfluid = nfluid;
  m->all_fluid = (nfluid == n);
  CK(cudaMemcpyAsync(m->status, status, (size_t) n, cudaMemcpyHostToDevice,
		     stream_), "map");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* Device status pointer, or NULL when every site is fluid */
static const uint8_t * map_dev(map_t * m) {
  return (m == NULL || m->all_fluid) ? NULL : m->status;
}

/*****************************************************************************
 *  Symmetric free energy (fe_t interface)
 *****************************************************************************/

struct fe_symm_s {
  fe_t super;
  fe_symm_param_t param;
  field_t * phi;
  field_grad_t * dphi;
};

static int site_get(field_t * f, int n, int index, double * v) {
  if (index < 0 || index >= f->cs->d.nsites) {
    return err_set(LUDWIG_GB_EINVAL, "site index out of range");
  }
  const char * base = (const char *) f->data
    + ((size_t) n*f->cs->d.nsites + index)*field_size(f->prec);
  if (f->prec == LUDWIG_GB_FP64) {
    CK(cudaMemcpy(v, base, sizeof(double), cudaMemcpyDeviceToHost), "site");
  }
  else {
    float t;
    CK(cudaMemcpy(&t, base, sizeof(float), cudaMemcpyDeviceToHost), "site");
    *v = t;
  }
  return LUDWIG_GB_OK;
}

static int grad_site(field_grad_t * g, int index, double gr[3], double * dsq) {
  if (g->grad == NULL) return err_set(LUDWIG_GB_ESTATE, "gradients not computed");
  size_t N = (size_t) g->field->cs->d.nsites;
  for (int ia = 0; ia < 3; ia++) {
    CK(cudaMemcpy(gr + ia, g->grad + ia*N + index, sizeof(double),
		  cudaMemcpyDeviceToHost), "grad");
  }
  if (dsq) {
    CK(cudaMemcpy(dsq, g->delsq + index, sizeof(double),
		  cudaMemcpyDeviceToHost), "delsq");
  }
  return LUDWIG_GB_OK;
}

/* The slots of the function tables take cs_index() sites (halo sites are
 * periodic images); the device arrays hold the interior sites. */
static int slot_site(const field_t * f, int index, int * i) {
  long long k = cs_interior(f->cs, index);
  if (k < 0) {
    return err_set(LUDWIG_GB_EINVAL, "free energy: index %d is not a "
		   "cs_index() site", index);
  }
  *i = (int) k;
  return LUDWIG_GB_OK;
}

/* src/symmetric.c:285-300 */
static int symm_fed(fe_t * base, int index, double * fed) {
  fe_symm_t * fe = (fe_symm_t *) base;
  double phi, g[3];
  int i = 0;
  int rc = slot_site(fe->phi, index, &i);
  if (rc == 0) rc = site_get(fe->phi, 0, i, &phi);
  if (rc == 0) rc = grad_site(fe->dphi, i, g, NULL);
  if (rc) return rc;
  *fed = (0.5*fe->param.a + 0.25*fe->param.b*phi*phi)*phi*phi
    + 0.5*fe->param.kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
  return LUDWIG_GB_OK;
}

/* src/symmetric.c:308-320 */
static int symm_mu(fe_t * base, int index, double * mu) {
  fe_symm_t * fe = (fe_symm_t *) base;
  double phi, g[3], dsq;
  int i = 0;
  int rc = slot_site(fe->phi, index, &i);
  if (rc == 0) rc = site_get(fe->phi, 0, i, &phi);
  if (rc == 0) rc = grad_site(fe->dphi, i, g, &dsq);
  if (rc) return rc;
  *mu = fe->param.a*phi + fe->param.b*phi*phi*phi - fe->param.kappa*dsq;
  return LUDWIG_GB_OK;
}

/* src/symmetric.c:334-365 */
static int symm_str(fe_t * base, int index, double s[3][3]) {
  fe_symm_t * fe = (fe_symm_t *) base;
  double phi, g[3], dsq;
  int i = 0;
  int rc = slot_site(fe->phi, index, &i);
  if (rc == 0) rc = site_get(fe->phi, 0, i, &phi);
  if (rc == 0) rc = grad_site(fe->dphi, i, g, &dsq);
  if (rc) return rc;
  double kappa = fe->param.kappa;
  double p0 = 0.5*fe->param.a*phi*phi + 0.75*fe->param.b*phi*phi*phi*phi
    - kappa*phi*dsq - 0.5*kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double dab = (ia == ib);
      s[ia][ib] = p0*dab + kappa*g[ia]*g[ib];
    }
  }
  return LUDWIG_GB_OK;
}

/* src/symmetric.c:372-400: the stress at the NSIMDVL (= 1) sites from
 * index.  The slot type returns nothing: a failure leaves s untouched and
 * the message in ludwig_gb_last_error(). */
static void symm_str_v(fe_t * base, int index, double s[3][3][NSIMDVL]) {
  double t[3][3];
  if (symm_str(base, index, t)) return;
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) s[ia][ib][0] = t[ia][ib];
}

static int symm_free(fe_t * base) { return fe_symm_free((fe_symm_t *) base); }
static int symm_target(fe_t * base, fe_t ** t) { *t = base; return 0; }

/* src/symmetric.c:46-61, slot for slot */
static fe_vt_t fe_symm_vt_ = {
  symm_free,               /* free */
  symm_target,             /* target */
  symm_fed,                /* fed */
  symm_mu,                 /* mu */
  NULL,                    /* mu_solv */
  symm_str,                /* stress */
  symm_str,                /* str_symm */
  NULL,                    /* str_anti */
  NULL,                    /* hvector */
  NULL,                    /* htensor */
  NULL,                    /* htensor_v */
  symm_str_v,              /* stress_v */
  symm_str_v,              /* str_symm_v */
  NULL                     /* str_anti_v */
};

int fe_symm_create(pe_t * pe, cs_t * cs, field_t * phi, field_grad_t * dphi,
		   fe_symm_t ** p) {
  (void) pe; (void) cs;
  if (phi == NULL || dphi == NULL || p == NULL || phi->nf != 1) {
    return err_set(LUDWIG_GB_EINVAL, "fe_symm_create");
  }
  fe_symm_t * fe = (fe_symm_t *) calloc(1, sizeof(fe_symm_t));
  if (fe == NULL) return err_set(LUDWIG_GB_ENOMEM, "fe_symm_create");
  fe->super.id = FE_SYMMETRIC;
  fe->super.func = &fe_symm_vt_;
  fe->super.use_stress_relaxation = 0;
  /* Defaults of src/symmetric.c:40-42 */
  fe->param.a = -0.003125;
  fe->param.b = +0.003125;
  fe->param.kappa = +0.002;
  fe->phi = phi;
  fe->dphi = dphi;
  *p = fe;
  return LUDWIG_GB_OK;
}

int fe_symm_free(fe_symm_t * fe) { free(fe); return LUDWIG_GB_OK; }

int fe_symm_param_set(fe_symm_t * fe, fe_symm_param_t values) {
  if (fe == NULL) return err_set(LUDWIG_GB_EINVAL, "fe_symm_param_set");
  fe->param = values;
  return LUDWIG_GB_OK;
}

int fe_symm_param(fe_symm_t * fe, fe_symm_param_t * values) {
  *values = fe->param;
  return LUDWIG_GB_OK;
}

static int fe_symm_get(fe_t * fe, fe_symm_t ** s) {
  if (fe == NULL || fe->id != FE_SYMMETRIC) {
    return err_set(LUDWIG_GB_EINVAL, "symmetric free energy required");
  }
  *s = (fe_symm_t *) fe;
  return LUDWIG_GB_OK;
}


/*****************************************************************************
 *  Force: pth_t and phi_force_calculation
 *****************************************************************************/

struct pth_s {
  cs_t * cs;
  int method;
  double * str;
};

int pth_create(pe_t * pe, cs_t * cs, int method, pth_t ** p) {
  (void) pe;
  if (cs == NULL || p == NULL ||
      (method != FE_FORCE_METHOD_NO_FORCE &&
       method != FE_FORCE_METHOD_STRESS_DIVERGENCE)) {
    return err_set(LUDWIG_GB_EINVAL, "pth_create: no_force or "
		   "stress_divergence");
  }
  pth_t * pth = (pth_t *) calloc(1, sizeof(pth_t));
  if (pth == NULL) return err_set(LUDWIG_GB_ENOMEM, "pth_create");
  pth->cs = cs;
  pth->method = method;
  *p = pth;
  return LUDWIG_GB_OK;
}

int pth_free(pth_t * pth) {
  if (pth) { dev_free(pth->str); free(pth); }
  return LUDWIG_GB_OK;
}

static int lc_stress_compute(pth_t * pth, fe_lc_t * fe);
static int collide_param(lb_t * lb, lgbk_collide_t * cp);

int pth_stress_compute(pth_t * pth, fe_t * fe) {
  if (pth == NULL || fe == NULL) return err_set(LUDWIG_GB_EINVAL, "pth");
  if (pth->str == NULL) {
    int rc = dev_alloc((void **) &pth->str, 9*(size_t) pth->cs->d.nsites
		       *sizeof(double), "pth");
    if (rc) return rc;
  }
  if (fe->id == FE_LC) return lc_stress_compute(pth, (fe_lc_t *) fe);

  fe_symm_t * s = NULL;
  int rc = fe_symm_get(fe, &s);
  if (rc) return rc;
  if (s->phi->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "pth_stress_compute: FP64 only");
  }
  rc = grad_alloc(s->dphi);
  if (rc) return rc;
  lgbk_symm_t sp = {s->param.a, s->param.b, s->param.kappa};
  CK(lgbk_symm_stress_f64(&pth->cs->d, &sp, (const double *) s->phi->data,
			  s->dphi->grad, s->dphi->delsq, pth->str, stream_),
     "stress");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int pth_to_host(pth_t * pth, double * str) {
  if (pth == NULL || pth->str == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "pth_to_host: stress not computed");
  }
  return copy_to_host(LUDWIG_GB_FP64, 9*pth->cs->d.nsites, pth->str, str);
}

/* src/phi_force.c:74-140, stress divergence, fluid only */
int phi_force_calculation(pe_t * pe, cs_t * cs, lees_edw_t * le,
			  wall_t * wall, pth_t * pth, fe_t * fe, map_t * map,
			  field_t * phi, hydro_t * hydro) {
  (void) pe; (void) cs; (void) map; (void) phi;
  if (pth == NULL) return err_set(LUDWIG_GB_EINVAL, "pth NULL");
  if (le != NULL || wall != NULL) {
    return err_set(LUDWIG_GB_EINVAL, "walls and Lees-Edwards not supported");
  }
  if (hydro == NULL) return LUDWIG_GB_OK;
  if (pth->method == FE_FORCE_METHOD_NO_FORCE) return LUDWIG_GB_OK;
  if (hydro->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "phi_force_calculation: FP64 only");
  }
  int rc = pth_stress_compute(pth, fe);
  if (rc) return rc;
  CK(lgbk_force_div_f64(&pth->cs->d, pth->str, (double *) hydro->force,
			stream_), "force");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Cholesteric liquid crystal: fe_lc_t, Beris-Edwards
 *****************************************************************************/

struct fe_lc_s {
  fe_t super;
  fe_lc_param_t param;
  field_t * q;
  field_grad_t * dq;
};

/* The phase of a time-dependent electric field, as fe_lc_param_commit
 * (src/blue_phase.c:210-226) sets it before every use of the parameters:
 * coswt = cos(2 pi f t) at the physics object's current time; a static
 * field (frequency zero) keeps the parameter block's value. */
static void lc_commit_field(fe_lc_t * fe) {
  if (phys_ref_ == NULL || phys_ref_->e0_frequency == 0.0) return;
  const double pi = 4.0*atan(1.0);
  double t = 0.0;
  physics_control_time(phys_ref_, &t);
  fe->param.coswt = cos(2.0*pi*phys_ref_->e0_frequency*t);
}

static void lc_kparam(fe_lc_t * fe, lgbk_lc_t * k) {
  lc_commit_field(fe);
  memset(k, 0, sizeof(*k));
  k->a0 = fe->param.a0;
  k->q0 = fe->param.q0;
  k->gamma = fe->param.gamma;
  k->kappa0 = fe->param.kappa0;
  k->kappa1 = fe->param.kappa1;
  k->xi = fe->param.xi;
  k->redshift = fe->param.redshift;
  k->rredshift = fe->param.rredshift;
  k->epsilon = fe->param.epsilon;
  for (int i = 0; i < 3; i++) k->e0[i] = fe->param.e0[i];
  k->coswt = fe->param.coswt;
}

static int lc_ready(fe_lc_t * fe) {
  if (fe->q->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "liquid crystal: FP64 fields only");
  }
  if (fe->dq->grad == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "liquid crystal: call "
		   "field_grad_compute() on the q gradients first");
  }
  return LUDWIG_GB_OK;
}

static int lc_stress_compute(pth_t * pth, fe_lc_t * fe) {
  int rc = lc_ready(fe);
  if (rc) return rc;
  lgbk_lc_t k;
  lc_kparam(fe, &k);
  CK(lgbk_lc_stress_f64(&pth->cs->d, &k, (const double *) fe->q->data,
			fe->dq->grad, fe->dq->delsq, pth->str, stream_),
     "lc_stress");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* Per-site vtable entries: evaluate on the lattice, return one site. */
static int lc_site_eval(fe_lc_t * fe, int index, int what, double * out) {
  const lgbk_dims_t * d = &fe->q->cs->d;
  double * tmp = NULL;
  int ncomp = (what == 0) ? 1 : ((what == 1) ? 9 : 5);
  int rc = lc_ready(fe);
  if (rc) return rc;
  int i = 0;
  if ((rc = slot_site(fe->q, index, &i))) return rc;
  rc = dev_alloc((void **) &tmp, (size_t) ncomp*d->nsites*sizeof(double),
		 "lc_site");
  if (rc) return rc;
  lgbk_lc_t k;
  lc_kparam(fe, &k);
  const double * q = (const double *) fe->q->data;
  if (what == 0) rc = lgbk_lc_fed_f64(d, &k, q, fe->dq->grad, tmp, stream_);
  if (what == 1) rc = lgbk_lc_stress_f64(d, &k, q, fe->dq->grad,
					 fe->dq->delsq, tmp, stream_);
  if (what == 2) rc = lgbk_lc_h_f64(d, &k, q, fe->dq->grad, fe->dq->delsq,
				    tmp, stream_);
  if (rc == 0) rc = cudaStreamSynchronize(stream_);
  for (int n = 0; rc == 0 && n < ncomp; n++) {
    rc = cudaMemcpy(out + n, tmp + (size_t) n*d->nsites + i,
		    sizeof(double), cudaMemcpyDeviceToHost);
  }
  dev_free(tmp);
  return cuda_check(rc, "lc_site_eval");
}

/* Total free energy of the LC (src/stats_free_energy.c:38-90 with
 * fe_lc_fed): FP64 Klein-compensated sum of the density over the sites.
 * Needs field_grad_compute() on the q gradients first. */
int stats_free_energy_lc(fe_lc_t * fe, double * total) {
  if (fe == NULL || total == NULL) return err_set(LUDWIG_GB_EINVAL, "stats");
  int rc = lc_ready(fe);
  if (rc) return rc;
  const lgbk_dims_t * d = &fe->q->cs->d;
  double * tmp = NULL, * scr = NULL, r[4];
  if ((rc = red_scratch(&scr))) return rc;
  rc = dev_alloc((void **) &tmp, (size_t) d->nsites*sizeof(double), "fed");
  if (rc) return rc;
  lgbk_lc_t k;
  lc_kparam(fe, &k);
  rc = lgbk_lc_fed_f64(d, &k, (const double *) fe->q->data, fe->dq->grad,
		       tmp, stream_);
  if (rc == 0) rc = lgbk_field_stats(d, LGBK_PREC_FP64, tmp, scr, r, stream_);
  dev_free(tmp);
  if (rc) return cuda_check(rc, "stats_free_energy_lc");
  *total = r[0];
  return LUDWIG_GB_OK;
}

/* The statistics fe_lc_stats_info prints without walls or colloids
 * (src/fe_lc_stats.c:55-150): out = {f, v, f/v, f_bulk/v, f_grad/v,
 * redshift}, sums over the fluid sites of the map (all sites for map
 * NULL).  Needs field_grad_compute() on the q gradients first. */
int ludwig_gb_fe_lc_stats_info(fe_lc_t * fe, map_t * map, double out[6]) {
  if (fe == NULL || out == NULL) return err_set(LUDWIG_GB_EINVAL, "stats");
  int rc = lc_ready(fe);
  if (rc) return rc;
  const lgbk_dims_t * d = &fe->q->cs->d;
  if (map && map->cs->d.nsites != d->nsites) {
    return err_set(LUDWIG_GB_EINVAL, "fe_lc_stats_info: map size");
  }
  double * tmp = NULL, * scr = NULL, r[5];
  if ((rc = red_scratch(&scr))) return rc;
  rc = dev_alloc((void **) &tmp, (size_t) 3*d->nsites*sizeof(double), "fbg");
  if (rc) return rc;
  lgbk_lc_t k;
  lc_kparam(fe, &k);
  const uint8_t * st = (map && !map->all_fluid) ? map->status : NULL;
  rc = lgbk_lc_fbg_f64(d, &k, (const double *) fe->q->data, fe->dq->grad,
		       tmp, stream_);
  if (rc == 0) rc = lgbk_masked_cols(d, LGBK_PREC_FP64, 3, tmp, st, scr, r,
				     stream_);
  dev_free(tmp);
  if (rc) return cuda_check(rc, "fe_lc_stats_info");
  double v = (double) (map ? map->nfluid : d->nsites);
  out[0] = r[0];
  out[1] = v;
  out[2] = r[0]/v;
  out[3] = r[1]/v;
  out[4] = r[2]/v;
  out[5] = fe->param.redshift;
  return LUDWIG_GB_OK;
}

static int lc_fed(fe_t * base, int index, double * fed) {
  return lc_site_eval((fe_lc_t *) base, index, 0, fed);
}

static int lc_stress(fe_t * base, int index, double s[3][3]) {
  return lc_site_eval((fe_lc_t *) base, index, 1, &s[0][0]);
}

static int lc_htensor(fe_t * base, int index, double h[3][3]) {
  double h5[5];
  int rc = lc_site_eval((fe_lc_t *) base, index, 2, h5);
  if (rc) return rc;
  h[0][0] = h5[0]; h[0][1] = h5[1]; h[0][2] = h5[2];
  h[1][0] = h5[1]; h[1][1] = h5[3]; h[1][2] = h5[4];
  h[2][0] = h5[2]; h[2][1] = h5[4]; h[2][2] = 0.0 - h5[0] - h5[3];
  return LUDWIG_GB_OK;
}

/* The antisymmetric piece of the stress, -(Q_ac H_bc - H_ac Q_bc) summed
 * over c (src/blue_phase.c:780-812), from Q and H at the site */
static int lc_qh(fe_t * base, int index, double q[3][3], double h[3][3]) {
  fe_lc_t * fe = (fe_lc_t *) base;
  int rc = field_tensor(fe->q, index, q);
  if (rc == 0) rc = lc_htensor(base, index, h);
  return rc;
}

static int lc_str_anti(fe_t * base, int index, double s[3][3]) {
  double q[3][3], h[3][3];
  int rc = lc_qh(base, index, q, h);
  if (rc) return rc;
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      s[ia][ib] = 0.0;
      for (int ic = 0; ic < 3; ic++) {
	s[ia][ib] -= (q[ia][ic]*h[ib][ic] - h[ia][ic]*q[ib][ic]);
      }
    }
  }
  return LUDWIG_GB_OK;
}

/* The stress with its antisymmetric piece taken out
 * (src/blue_phase.c:729-770) */
static int lc_str_symm(fe_t * base, int index, double s[3][3]) {
  double q[3][3], h[3][3];
  int rc = lc_stress(base, index, s);
  if (rc == 0) rc = lc_qh(base, index, q, h);
  if (rc) return rc;
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      for (int ic = 0; ic < 3; ic++) {
	s[ia][ib] += q[ia][ic]*h[ib][ic] - h[ia][ic]*q[ib][ic];
      }
    }
  }
  return LUDWIG_GB_OK;
}

/* Vectorised slots at NSIMDVL = 1 (src/blue_phase.c:1669-2279): the site
 * index; a failure leaves the output untouched, message in
 * ludwig_gb_last_error() */
static void lc_htensor_v(fe_t * base, int index, double h[3][3][NSIMDVL]) {
  double t[3][3];
  if (lc_htensor(base, index, t)) return;
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) h[ia][ib][0] = t[ia][ib];
}

static void lc_stress_v(fe_t * base, int index, double s[3][3][NSIMDVL]) {
  double t[3][3];
  if (lc_stress(base, index, t)) return;
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) s[ia][ib][0] = t[ia][ib];
}

static void lc_str_symm_v(fe_t * base, int index, double s[3][3][NSIMDVL]) {
  double t[3][3];
  if (lc_str_symm(base, index, t)) return;
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) s[ia][ib][0] = t[ia][ib];
}

static void lc_str_anti_v(fe_t * base, int index, double s[3][3][NSIMDVL]) {
  double t[3][3];
  if (lc_str_anti(base, index, t)) return;
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) s[ia][ib][0] = t[ia][ib];
}

static int lc_free(fe_t * base) { return fe_lc_free((fe_lc_t *) base); }
static int lc_target(fe_t * base, fe_t ** t) { *t = base; return 0; }

/* src/blue_phase.c:35-50, slot for slot */
static fe_vt_t fe_lc_vt_ = {
  lc_free,                 /* free */
  lc_target,               /* target */
  lc_fed,                  /* fed */
  NULL,                    /* mu */
  NULL,                    /* mu_solv */
  lc_stress,               /* stress */
  lc_str_symm,             /* str_symm */
  lc_str_anti,             /* str_anti */
  NULL,                    /* hvector */
  lc_htensor,              /* htensor */
  lc_htensor_v,            /* htensor_v */
  lc_stress_v,             /* stress_v */
  lc_str_symm_v,           /* str_symm_v */
  lc_str_anti_v            /* str_anti_v */
};

int fe_lc_create(pe_t * pe, cs_t * cs, lees_edw_t * le, field_t * q,
		 field_grad_t * dq, fe_lc_t ** p) {
  (void) pe; (void) cs;
  if (le != NULL) return err_set(LUDWIG_GB_EINVAL, "Lees-Edwards planes");
  if (q == NULL || dq == NULL || p == NULL || q->nf != 5) {
    return err_set(LUDWIG_GB_EINVAL, "fe_lc_create: q must have 5 components");
  }
  fe_lc_t * fe = (fe_lc_t *) calloc(1, sizeof(fe_lc_t));
  if (fe == NULL) return err_set(LUDWIG_GB_ENOMEM, "fe_lc_create");
  fe->super.id = FE_LC;
  fe->super.func = &fe_lc_vt_;
  fe->q = q;
  fe->dq = dq;
  fe->param.redshift = 1.0;
  fe->param.rredshift = 1.0;
  fe->param.coswt = 1.0;
  *p = fe;
  return LUDWIG_GB_OK;
}

int fe_lc_free(fe_lc_t * fe) { free(fe); return LUDWIG_GB_OK; }

int fe_lc_param_set(fe_lc_t * fe, const fe_lc_param_t * values) {
  const double pi = 3.1415926535897932385;
  if (fe == NULL || values == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "fe_lc_param_set");
  }
  if (values->is_active || values->is_redshift_updated ||
      values->zeta0 != 0.0 || values->zeta1 != 0.0 || values->zeta2 != 0.0) {
    return err_set(LUDWIG_GB_EINVAL, "fe_lc: active stress and dynamic "
		   "redshift are not supported");
  }
  if (values->redshift == 0.0) {
    return err_set(LUDWIG_GB_EINVAL, "fe_lc: redshift must be non-zero");
  }
  fe->param = *values;
  fe->param.epsilon *= (1.0/(12.0*pi));
  fe->param.rredshift = 1.0/fe->param.redshift;
  return LUDWIG_GB_OK;
}

int fe_lc_param(fe_lc_t * fe, fe_lc_param_t * values) {
  if (fe == NULL || values == NULL) return err_set(LUDWIG_GB_EINVAL, "fe_lc");
  *values = fe->param;
  return LUDWIG_GB_OK;
}

/* src/blue_phase_init.c:59-132 without rotation; global coordinates are
 * 1-based */
/* Euler rotation (Z, X, Z) of the blue-phase initial conditions,
 * src/blue_phase_init.c:1358-1445: angles in degrees, applied with a
 * minus sign (a clockwise rotation of the argument turns Q
 * counterclockwise); r' = M2 M1 M0 r summed in the reference's order. */
typedef struct euler_rot_s { double m[3][3][3]; } euler_rot_t;

static void rot_axis(double M[3][3], int dim, double alpha) {
  const double c = cos(alpha), s = sin(alpha);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) M[i][j] = 0.0;
  if (dim == 0) {
    M[0][0] = 1.0; M[1][1] = c; M[1][2] = -s; M[2][1] = s; M[2][2] = c;
  }
  else if (dim == 1) {
    M[0][0] = c; M[0][2] = -s; M[1][1] = 1.0; M[2][0] = s; M[2][2] = c;
  }
  else {
    M[0][0] = c; M[0][1] = -s; M[1][0] = s; M[1][1] = c; M[2][2] = 1.0;
  }
}

static void euler_rot_create(const double deg[3], euler_rot_t * rot) {
  const double pi = 3.1415926535897932385;
  const int axis[3] = {2, 0, 2};
  for (int k = 0; k < 3; k++) {
    const double a = deg ? -1.0*pi*deg[k]/180.0 : 0.0;
    rot_axis(rot->m[k], axis[k], a);
  }
}

static void euler_rotate(const euler_rot_t * rot, double r[3]) {
  const double r0[3] = {r[0], r[1], r[2]};
  for (int k = 0; k < 3; k++) {
    double t = 0.0;
    for (int l = 0; l < 3; l++)
      for (int m = 0; m < 3; m++)
	for (int n = 0; n < 3; n++)
	  t += rot->m[2][k][l]*rot->m[1][l][m]*rot->m[0][m][n]*r0[n];
    r[k] = t;
  }
}

int blue_phase_O8M_init(cs_t * cs, fe_lc_param_t * param, field_t * fq,
			const double euler_angles[3]) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_O8M_init");
  }
  euler_rot_t rot;
  euler_rot_create(euler_angles, &rot);
  const lgbk_dims_t * d = &cs->d;
  const long long N = d->nsites;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "o8m");
  const double root2 = sqrt(2.0);
  const double q0 = param->q0, a = param->amplitude0;
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	long long i = ((long long) x*d->ny + y)*d->nz + z;
	double r[3];
	r[0] = (double) (x + 1) - 0.5*d->nx;
	r[1] = (double) (y + 1) - 0.5*d->ny;
	r[2] = (double) (z + 1) - 0.5*d->nz;
	euler_rotate(&rot, r);
	r[0] += 0.5*d->nx; r[1] += 0.5*d->ny; r[2] += 0.5*d->nz;
	double cosx = cos(root2*q0*r[0]), sinx = sin(root2*q0*r[0]);
	double cosy = cos(root2*q0*r[1]), siny = sin(root2*q0*r[1]);
	double cosz = cos(root2*q0*r[2]), sinz = sin(root2*q0*r[2]);
	h[0*N + i] = a*(-2.0*cosy*sinz + sinx*cosz + cosx*siny);
	h[1*N + i] = a*(root2*cosy*cosz + root2*sinx*sinz - sinx*cosy);
	h[2*N + i] = a*(root2*cosx*cosy + root2*sinz*siny - cosx*sinz);
	h[3*N + i] = a*(-2.0*sinx*cosz + siny*cosx + cosy*sinz);
	h[4*N + i] = a*(root2*cosz*cosx + root2*siny*sinx - siny*cosz);
      }
    }
  }
  int rc = field_from_host(fq, h);
  free(h);
  return rc;
}

/* Blue phase II, src/blue_phase_init.c:155-235 */
int blue_phase_O2_init(cs_t * cs, fe_lc_param_t * param, field_t * fq,
		       const double euler_angles[3]) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_O2_init");
  }
  euler_rot_t rot;
  euler_rot_create(euler_angles, &rot);
  const lgbk_dims_t * d = &cs->d;
  const long long N = d->nsites;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "o2");
  const double q0 = param->q0, a = param->amplitude0;
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	long long i = ((long long) x*d->ny + y)*d->nz + z;
	double r[3];
	r[0] = (double) (x + 1) - 0.5*d->nx;
	r[1] = (double) (y + 1) - 0.5*d->ny;
	r[2] = (double) (z + 1) - 0.5*d->nz;
	euler_rotate(&rot, r);
	r[0] += 0.5*d->nx; r[1] += 0.5*d->ny; r[2] += 0.5*d->nz;
	double cosx = cos(2.0*q0*r[0]), sinx = sin(2.0*q0*r[0]);
	double cosy = cos(2.0*q0*r[1]), siny = sin(2.0*q0*r[1]);
	double cosz = cos(2.0*q0*r[2]), sinz = sin(2.0*q0*r[2]);
	h[0*N + i] = a*(cosz - cosy);
	h[1*N + i] = a*sinz;
	h[2*N + i] = a*siny;
	h[3*N + i] = a*(cosx - cosz);
	h[4*N + i] = a*sinx;
      }
    }
  }
  int rc = field_from_host(fq, h);
  free(h);
  return rc;
}

/* Uniform uniaxial nematic along n (normalised here),
 * src/blue_phase_init.c:836-872 with fe_lc_q_uniaxial,
 * src/blue_phase.c:1406: Q_ab = (A/2)(3 n_a n_b - d_ab) */
int blue_phase_nematic_init(cs_t * cs, fe_lc_param_t * param, field_t * fq,
			    const double n[3]) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5 || n == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_nematic_init");
  }
  const double mod = sqrt(n[0]*n[0] + n[1]*n[1] + n[2]*n[2]);
  if (!(mod > 0.0)) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_nematic_init: |n| = 0");
  }
  double nh[3], q[3][3];
  for (int a = 0; a < 3; a++) nh[a] = n[a]/mod;
  for (int a = 0; a < 3; a++) {
    for (int b = 0; b < 3; b++) {
      q[a][b] = 0.5*param->amplitude0*(3.0*nh[a]*nh[b] - (double) (a == b));
    }
  }
  const double q5[5] = {q[0][0], q[0][1], q[0][2], q[1][1], q[1][2]};
  const long long N = cs->d.nsites;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "nematic");
  for (int c = 0; c < 5; c++) {
    for (long long i = 0; i < N; i++) h[c*N + i] = q5[c];
  }
  int rc = field_from_host(fq, h);
  free(h);
  return rc;
}

/* Random uniaxial directors, src/blue_phase_init.c:1170-1212 (seed 13,
 * two draws per site: azimuth 2 pi (1/2 - r1), polar acos(2 r2 - 1)) */
int blue_phase_random_q_init(cs_t * cs, fe_lc_param_t * param, field_t * fq) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_random_q_init");
  }
  const double pi = 3.1415926535897932385;
  const lgbk_dims_t * d = &cs->d;
  const long long N = d->nsites;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "random_q");
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	const long long i = ((long long) x*d->ny + y)*d->nz + z;
	double r[2], n[3], q[3][3];
	site_uniforms(13u, x, y, z, 2, r);
	const double phase1 = 2.0*pi*(0.5 - r[0]);
	const double phase2 = acos(2.0*r[1] - 1.0);
	n[0] = cos(phase1)*sin(phase2);
	n[1] = sin(phase1)*sin(phase2);
	n[2] = cos(phase2);
	for (int a = 0; a < 3; a++) {
	  for (int b = 0; b < 3; b++) {
	    q[a][b] = 0.5*param->amplitude0*(3.0*n[a]*n[b] - (double) (a == b));
	  }
	}
	h[0*N + i] = q[0][0]; h[1*N + i] = q[0][1]; h[2*N + i] = q[0][2];
	h[3*N + i] = q[1][1]; h[4*N + i] = q[1][2];
      }
    }
  }
  int rc = field_from_host(fq, h);
  free(h);
  return rc;
}

/* Cholesteric helix along axis 0, 1, 2 (X, Y, Z), src/blue_phase_init.c:
 * 763-825: n = (0, cos q0 x, sin q0 x), (cos q0 y, 0, -sin q0 y) or
 * (cos q0 z, sin q0 z, 0) with 1-based coordinates; Q uniaxial along n */
int blue_phase_twist_init(cs_t * cs, fe_lc_param_t * param, field_t * fq,
			  int helical_axis) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5 ||
      helical_axis < 0 || helical_axis > 2) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_twist_init");
  }
  const lgbk_dims_t * d = &cs->d;
  const long long N = d->nsites;
  const double q0 = param->q0;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "twist");
  for (int x = 0; x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	const long long i = ((long long) x*d->ny + y)*d->nz + z;
	double n[3] = {0.0, 0.0, 0.0}, q[3][3];
	if (helical_axis == 0) {
	  n[1] = cos(q0*(x + 1)); n[2] = sin(q0*(x + 1));
	}
	else if (helical_axis == 1) {
	  n[0] = cos(q0*(y + 1)); n[2] = -sin(q0*(y + 1));
	}
	else {
	  n[0] = cos(q0*(z + 1)); n[1] = sin(q0*(z + 1));
	}
	for (int a = 0; a < 3; a++) {
	  for (int b = 0; b < 3; b++) {
	    q[a][b] = 0.5*param->amplitude0*(3.0*n[a]*n[b] - (double) (a == b));
	  }
	}
	h[0*N + i] = q[0][0]; h[1*N + i] = q[0][1]; h[2*N + i] = q[0][2];
	h[3*N + i] = q[1][1]; h[4*N + i] = q[1][2];
      }
    }
  }
  int rc = field_from_host(fq, h);
  free(h);
  return rc;
}

/* Random uniaxial directors of amplitude 0.01 superposed (replacing Q) on
 * the sites of the box rmin..rmax (1-based, inclusive),
 * src/blue_phase_init.c:1279-1345 (seed 13, as the random initial
 * condition) */
int blue_phase_random_q_rectangle(cs_t * cs, fe_lc_param_t * param,
				  field_t * fq, int rmin[3], int rmax[3]) {
  if (cs == NULL || param == NULL || fq == NULL || fq->nf != 5 ||
      rmin == NULL || rmax == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "blue_phase_random_q_rectangle");
  }
  const double pi = 3.1415926535897932385;
  const double a0 = 0.01;
  const lgbk_dims_t * d = &cs->d;
  const long long N = d->nsites;
  double * h = (double *) malloc(5*(size_t) N*sizeof(double));
  if (h == NULL) return err_set(LUDWIG_GB_ENOMEM, "random_q_rectangle");
  int rc = field_to_host(fq, h);
  for (int x = 0; rc == 0 && x < d->nx; x++) {
    for (int y = 0; y < d->ny; y++) {
      for (int z = 0; z < d->nz; z++) {
	if (x + 1 < rmin[0] || x + 1 > rmax[0] || y + 1 < rmin[1] ||
	    y + 1 > rmax[1] || z + 1 < rmin[2] || z + 1 > rmax[2]) continue;
	const long long i = ((long long) x*d->ny + y)*d->nz + z;
	double r[2], n[3], q[3][3];
	site_uniforms(13u, x, y, z, 2, r);
	const double phase1 = 2.0*pi*(0.5 - r[0]);
	const double phase2 = acos(2.0*r[1] - 1.0);
	n[0] = cos(phase1)*sin(phase2);
	n[1] = sin(phase1)*sin(phase2);
	n[2] = cos(phase2);
	for (int a = 0; a < 3; a++) {
	  for (int b = 0; b < 3; b++) {
	    q[a][b] = 0.5*a0*(3.0*n[a]*n[b] - (double) (a == b));
	  }
	}
	h[0*N + i] = q[0][0]; h[1*N + i] = q[0][1]; h[2*N + i] = q[0][2];
	h[3*N + i] = q[1][1]; h[4*N + i] = q[1][2];
      }
    }
  }
  if (rc == 0) rc = field_from_host(fq, h);
  free(h);
  return rc;
}

struct beris_edw_s {
  cs_t * cs;
  beris_edw_param_t param;
  double * flux;               /* fw, fe, fy, fz: 4 x 5 x nsites */
  double * h;                  /* 5 x nsites */
};

int beris_edw_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		     beris_edw_t ** pobj) {
  (void) pe;
  if (le != NULL) return err_set(LUDWIG_GB_EINVAL, "Lees-Edwards planes");
  if (cs == NULL || !cs->initialised || pobj == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "beris_edw_create");
  }
  beris_edw_t * be = (beris_edw_t *) calloc(1, sizeof(beris_edw_t));
  if (be == NULL) return err_set(LUDWIG_GB_ENOMEM, "beris_edw_create");
  be->cs = cs;
  size_t N = (size_t) cs->d.nsites;
  int rc;
  if ((rc = dev_alloc((void **) &be->flux, 20*N*sizeof(double), "flux")) ||
      (rc = dev_alloc((void **) &be->h, 5*N*sizeof(double), "h"))) {
    beris_edw_free(be);
    return rc;
  }
  *pobj = be;
  return LUDWIG_GB_OK;
}

int beris_edw_free(beris_edw_t * be) {
  if (be) { dev_free(be->flux); dev_free(be->h); free(be); }
  return LUDWIG_GB_OK;
}

int beris_edw_param_set(beris_edw_t * be, beris_edw_param_t * values) {
  if (be == NULL || values == NULL) return err_set(LUDWIG_GB_EINVAL, "be");
  if (values->noise) {
    return err_set(LUDWIG_GB_EINVAL, "beris_edw: noise not supported");
  }
  be->param = *values;
  return LUDWIG_GB_OK;
}

/* src/blue_phase_beris_edwards.c:266-289 */
int beris_edw_update(beris_edw_t * be, fe_t * fe, field_t * fq,
		     field_grad_t * fq_grad, hydro_t * hydro,
		     colloids_info_t * cinfo, map_t * map, noise_t * noise) {
  if (be == NULL || fe == NULL || fq == NULL || fq_grad == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "beris_edw_update");
  }
  if (fe->id != FE_LC) return err_set(LUDWIG_GB_EINVAL, "fe_lc required");
  if (cinfo != NULL || noise != NULL) {
    return err_set(LUDWIG_GB_EINVAL, "colloids/noise not supported");
  }
  fe_lc_t * lc = (fe_lc_t *) fe;
  int rc = lc_ready(lc);
  if (rc) return rc;
  if (hydro && hydro->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "beris_edw_update: FP64 hydro only");
  }
  const lgbk_dims_t * d = &be->cs->d;
  const long long N5 = 5*d->nsites;
  if (hydro) {
    double * fw = be->flux, * fe_ = fw + N5, * fy = fw + 2*N5;
    double * fz = fw + 3*N5;
    CK(lgbk_advect_f64(d, advection_order_, 5, (const double *) fq->data,
			      (const double *) hydro->u, fw, fe_, fy, fz,
			      stream_), "advect");
    CK(lgbk_flux_no_normal_f64(d, 5, map_dev(map), fw, fe_, fy, fz, stream_),
       "no_flux");
  }
  lgbk_lc_t k;
  lc_kparam(lc, &k);
  CK(lgbk_lc_h_f64(d, &k, (const double *) fq->data, fq_grad->grad,
		   fq_grad->delsq, be->h, stream_), "h");
  CK(lgbk_be_update_f64(d, be->param.xi, be->param.gamma, map_dev(map),
			hydro ? (const double *) hydro->u : NULL,
			hydro ? be->flux : NULL, be->h, (double *) fq->data,
			stream_), "be_update");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

static int lc_step_async(lb_t * lb, field_t * q, hydro_t * hydro,
			 map_t * map, fe_t * fe, beris_edw_t * be, int nsteps);

int ludwig_gb_lc_step(lb_t * lb, field_t * q, hydro_t * hydro, map_t * map,
		      fe_t * fe, beris_edw_t * be, int nsteps) {
  int rc = lc_step_async(lb, q, hydro, map, fe, be, nsteps);
  if (rc) return rc;
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* Device time of nsteps LC steps (CUDA events on the library stream) */
int ludwig_gb_time_lc(lb_t * lb, field_t * q, hydro_t * hydro, map_t * map,
		      fe_t * fe, beris_edw_t * be, int nsteps, double * ms) {
  cudaEvent_t e0, e1;
  int rc;
  if (ms == NULL) return err_set(LUDWIG_GB_EINVAL, "time_lc");
  if ((rc = lc_step_async(lb, q, hydro, map, fe, be, 0))) return rc;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  CK(cudaEventRecord(e0, stream_), "record");
  rc = lc_step_async(lb, q, hydro, map, fe, be, nsteps);
  if (rc == 0) rc = cuda_check(cudaEventRecord(e1, stream_), "record");
  if (rc == 0) rc = cuda_check(cudaEventSynchronize(e1), "sync");
  if (rc == 0) {
    float t = 0.0f;
    rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

static int lc_step_async(lb_t * lb, field_t * q, hydro_t * hydro,
			 map_t * map, fe_t * fe, beris_edw_t * be, int nsteps) {
  if (lb == NULL || q == NULL || hydro == NULL || fe == NULL || be == NULL ||
      nsteps < 0 || q->nf != 5) {
    return err_set(LUDWIG_GB_EINVAL, "ludwig_gb_lc_step");
  }
  if (fe->id != FE_LC) return err_set(LUDWIG_GB_EINVAL, "fe_lc required");
  int fp = (lb->prec == LUDWIG_GB_FP64);
  if (fp != (q->prec == LUDWIG_GB_FP64) ||
      fp != (hydro->prec == LUDWIG_GB_FP64)) {
    return err_set(LUDWIG_GB_EINVAL, "lc_step: lb, q and hydro must be all "
		   "FP64 or all reduced precision");
  }
  fe_lc_t * lc = (fe_lc_t *) fe;
  if (lc->dq && lc->dq->stencil != 7) {
    return err_set(LUDWIG_GB_EINVAL, "lc_step: the fused step uses "
		   "7-point gradients");
  }
  if (advection_order_ != 1) {
    return err_set(LUDWIG_GB_EINVAL, "lc_step: the fused step uses "
		   "first-order advection");
  }
  lgbk_lc_t k;
  lc_kparam(lc, &k);
  lgbk_lc_step_args_t a;
  memset(&a, 0, sizeof(a));
  int rc = collide_param(lb, &a.cp);
  if (rc) return rc;
  if (!a.cp.ghosts_zero) {
    return err_set(LUDWIG_GB_EINVAL, "lc_step: M10 relaxation only");
  }
  if ((rc = lb_unstream(lb))) return rc;
  const size_t N = (size_t) lb->cs->d.nsites;
  const size_t es = field_size(q->prec);
  a.status = map_dev(map);
  a.xi = be->param.xi;
  a.gamma_rot = be->param.gamma;
  a.rho0 = lb->rho0;
  a.fscale = lb->fscale;
  a.sites = tune_sites_;
  a.rho_out = hydro->rho;
  a.pth = be->flux;                                /* 9 N elements */
  a.h = (const char *) be->flux + 9*N*es;          /* 5 N elements */
  lgbk_lc_args_pack(&a);
  for (int n = 0; n < nsteps; n++) {
    /* one iteration of the main loop: the step counter first
     * (src/ludwig.c:528), then a time-dependent field's phase at the new
     * time (fe_lc_param_commit, src/blue_phase.c:210) */
    if (phys_ref_ != NULL) physics_control_next_step(phys_ref_);
    if (phys_ref_ != NULL && phys_ref_->e0_frequency != 0.0) {
      lc_kparam(lc, &k);
    }
    a.f_in = lb->f;   a.f_out = lb->fprime;
    a.q_in = q->data; a.q_out = q->data2;
    a.u_in = hydro->u; a.u_out = hydro->u2;
    CK(lgbk_lc_step(&lb->cs->d, lb->prec, &k, &a, stream_), "lc_step");
    lb_swap(lb);
    void * t = q->data; q->data = q->data2; q->data2 = t;
    t = hydro->u; hydro->u = hydro->u2; hydro->u2 = t;
  }
  return LUDWIG_GB_OK;
}

int beris_edw_h_to_host(beris_edw_t * be, double * h) {
  if (be == NULL || h == NULL) return err_set(LUDWIG_GB_EINVAL, "be_h");
  return copy_to_host(LUDWIG_GB_FP64, 5*be->cs->d.nsites, be->h, h);
}

/*****************************************************************************
 *  Cahn-Hilliard
 *****************************************************************************/

struct phi_ch_s {
  cs_t * cs;
  phi_ch_info_t info;
  double * flux;               /* fw, fe, fy, fz */
};

int phi_ch_create(pe_t * pe, cs_t * cs, lees_edw_t * le,
		  const phi_ch_info_t * info, phi_ch_t ** pch) {
  (void) pe;
  if (le != NULL) return err_set(LUDWIG_GB_EINVAL, "Lees-Edwards planes");
  if (cs == NULL || pch == NULL) return err_set(LUDWIG_GB_EINVAL, "phi_ch");
  if (info && (info->conserve != 0 || info->noise != 0)) {
    return err_set(LUDWIG_GB_EINVAL, "phi_ch: conserve 0, noise 0 only");
  }
  phi_ch_t * p = (phi_ch_t *) calloc(1, sizeof(phi_ch_t));
  if (p == NULL) return err_set(LUDWIG_GB_ENOMEM, "phi_ch_create");
  p->cs = cs;
  if (info) p->info = *info;
  *pch = p;
  return LUDWIG_GB_OK;
}

int phi_ch_free(phi_ch_t * p) {
  if (p) { dev_free(p->flux); free(p); }
  return LUDWIG_GB_OK;
}

/* src/phi_cahn_hilliard.c:213-288 */
int phi_cahn_hilliard(phi_ch_t * pch, fe_t * fe, field_t * phi,
		      hydro_t * hydro, map_t * map, noise_t * noise) {
  fe_symm_t * s = NULL;
  int rc = fe_symm_get(fe, &s);
  if (rc) return rc;
  if (pch == NULL || phi == NULL || phi->nf != 1) {
    return err_set(LUDWIG_GB_EINVAL, "phi_cahn_hilliard");
  }
  if (noise != NULL) return err_set(LUDWIG_GB_EINVAL, "noise not supported");
  if (phi->prec != LUDWIG_GB_FP64 || (hydro && hydro->prec != LUDWIG_GB_FP64)) {
    return err_set(LUDWIG_GB_EINVAL, "phi_cahn_hilliard: FP64 only");
  }
  physics_t * ph = NULL;
  if ((rc = phys_get(&ph))) return rc;

  const lgbk_dims_t * d = &phi->cs->d;
  size_t N = (size_t) d->nsites;
  if (pch->flux == NULL) {
    rc = dev_alloc((void **) &pch->flux, 4*N*sizeof(double), "flux");
    if (rc) return rc;
  }
  /* mu uses the gradients last computed by field_grad_compute(), as the
   * reference's fe_symm_mu reads fe->dphi (src/symmetric.c:308-320) */
  if (s->dphi->delsq == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "phi_cahn_hilliard: call "
		   "field_grad_compute() first");
  }

  double * fw = pch->flux, * fe_ = fw + N, * fy = fw + 2*N, * fz = fw + 3*N;
  if (hydro) {
    CK(lgbk_advect_f64(d, advection_order_, 1, (const double *) phi->data,
			      (const double *) hydro->u, fw, fe_, fy, fz,
			      stream_), "advect");
  }
  else {
    CK(cudaMemsetAsync(pch->flux, 0, 4*N*sizeof(double), stream_), "zero");
  }
  lgbk_symm_t sp = {s->param.a, s->param.b, s->param.kappa};
  CK(lgbk_ch_flux_mu_f64(d, &sp, ph->mobility, (const double *) phi->data,
			 s->dphi->delsq, fw, fe_, fy, fz, stream_), "flux_mu");
  CK(lgbk_flux_no_normal_f64(d, 1, map_dev(map), fw, fe_, fy, fz, stream_),
     "no_flux");
  CK(lgbk_ch_update_f64(d, fw, fe_, fy, fz, (double *) phi->data, stream_),
     "update");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Collision and propagation
 *****************************************************************************/

/* src/collision.c:1163-1246, src/collision.c:1906-1958 */
static int collide_param(lb_t * lb, lgbk_collide_t * cp) {
  physics_t * ph = NULL;
  int rc = phys_get(&ph);
  if (rc) return rc;
  const double cs2 = (1.0/3.0);
  double rho0 = ph->rho0;
  double rtau_shear = 1.0/(0.5 + ph->eta_shear / (rho0*cs2));
  double rtau_bulk = 1.0/(0.5 + ph->eta_bulk / (rho0*cs2));
  memset(cp, 0, sizeof(*cp));
  cp->rtau_shear = rtau_shear;
  cp->rtau_bulk = rtau_bulk;
  for (int p = 0; p < NVEL; p++) cp->rtau_ghost[p] = 1.0;
  if (lb->nrelax == LB_RELAXATION_BGK) {
    cp->rtau_bulk = rtau_shear;
    for (int p = 0; p < NVEL; p++) cp->rtau_ghost[p] = rtau_shear;
  }
  if (lb->nrelax == LB_RELAXATION_TRT) {
    double tau = ph->eta_shear / (rho0*cs2);
    double rtau = 0.5 + 2.0*tau/(tau + 3.0/8.0);
    if (rtau > 2.0) rtau = 2.0;
    cp->rtau_ghost[10] = rtau_shear;
    cp->rtau_ghost[14] = rtau_shear;
    cp->rtau_ghost[18] = rtau_shear;
    cp->rtau_ghost[11] = cp->rtau_ghost[12] = cp->rtau_ghost[13] = rtau;
    cp->rtau_ghost[15] = cp->rtau_ghost[16] = cp->rtau_ghost[17] = rtau;
  }
  cp->ghosts_zero = 1;
  for (int p = 10; p < NVEL; p++) {
    if (cp->rtau_ghost[p] != 1.0) cp->ghosts_zero = 0;
  }
  for (int i = 0; i < 3; i++) cp->force_global[i] = ph->fbody[i];
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Two-distribution binary fluid (symmetric_lb, ndist = 2)
 *****************************************************************************/

/* lb_collision_binary (src/collision.c:604-1013): needs the symmetric free
 * energy and the gradients of phi (field_grad_compute) of this step.  The
 * reference applies it at every site (no status test); so does this. */
static int lb_collide_binary(lb_t * lb, hydro_t * hydro, map_t * map,
			     fe_t * fe, const lgbk_collide_t * cp) {
  (void) map;
  fe_symm_t * s = NULL;
  physics_t * ph = NULL;
  int rc = fe_symm_get(fe, &s);
  if (rc == 0) rc = phys_get(&ph);
  if (rc) return rc;
  if (s->dphi == NULL || s->dphi->grad == NULL) {
    return err_set(LUDWIG_GB_ESTATE, "binary collision: call "
		   "field_grad_compute() on phi first");
  }
  if (s->phi->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "binary collision: FP64 phi");
  }
  lgbk_symm_t sp = {s->param.a, s->param.b, s->param.kappa};
  CK(lgbk_collide_binary_f64(&lb->cs->d, &sp, cp, ph->mobility, lb->pending,
			     (const double *) lb->f, (const double *) lb->g,
			     (const double *) s->phi->data, s->dphi->grad,
			     s->dphi->delsq, (double *) lb->fprime,
			     (double *) lb->gprime, (double *) hydro->u,
			     stream_), "collide binary");
  lb_swap(lb);
  lb_swap_g(lb);
  lb->pending = 0;                 /* the stored arrays are post-collision */
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* src/phi_lb_coupler.c:49: phi = sum_p g_p */
int phi_lb_to_field(field_t * phi, lb_t * lb) {
  if (phi == NULL || lb == NULL || lb->ndist != 2 || phi->nf != 1 ||
      phi->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "phi_lb_to_field: ndist 2, FP64 phi");
  }
  CK(lgbk_phi_from_g_f64(&lb->cs->d, lb->pending, (const double *) lb->g,
			 (double *) phi->data, stream_), "phi_from_g");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* src/phi_lb_coupler.c:107: g_0 = phi, the other g_p = 0 */
int phi_lb_from_field(field_t * phi, lb_t * lb) {
  if (phi == NULL || lb == NULL || lb->ndist != 2 || phi->nf != 1 ||
      phi->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "phi_lb_from_field: ndist 2, FP64 phi");
  }
  int rc = lb_materialise(lb);
  if (rc) return rc;
  CK(lgbk_g_from_phi_f64(&lb->cs->d, (const double *) phi->data,
			 (double *) lb->g, stream_), "g_from_phi");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* The reference's g (19 x nsites) */
int lb_g_to_host(lb_t * lb, double * gh) {
  if (lb == NULL || gh == NULL || lb->ndist != 2) {
    return err_set(LUDWIG_GB_EINVAL, "lb_g_to_host: ndist 2");
  }
  int rc = lb_materialise(lb);
  if (rc) return rc;
  CK(cudaMemcpyAsync(gh, lb->g, NVEL*(size_t) lb->cs->d.nsites*sizeof(double),
		     cudaMemcpyDeviceToHost, stream_), "lb_g_to_host");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int lb_g_from_host(lb_t * lb, const double * gh) {
  if (lb == NULL || gh == NULL || lb->ndist != 2) {
    return err_set(LUDWIG_GB_EINVAL, "lb_g_from_host: ndist 2");
  }
  int rc = lb_materialise(lb);
  if (rc) return rc;
  CK(cudaMemcpyAsync(lb->g, gh, NVEL*(size_t) lb->cs->d.nsites*sizeof(double),
		     cudaMemcpyHostToDevice, stream_), "lb_g_from_host");
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/* nsteps of the main loop with ndist = 2 (src/ludwig.c:528-860):
 * phi_lb_to_field, field_grad_compute, lb_collide (binary), lb_propagation;
 * three kernels per step, streaming folded into the next pull. */
int ludwig_gb_lb2_step(lb_t * lb, field_t * phi, hydro_t * hydro, fe_t * fe,
		       int nsteps) {
  fe_symm_t * s = NULL;
  physics_t * ph = NULL;
  int rc = fe_symm_get(fe, &s);
  if (rc == 0) rc = phys_get(&ph);
  if (rc) return rc;
  if (lb == NULL || phi == NULL || hydro == NULL || lb->ndist != 2 ||
      s->phi != phi || s->dphi == NULL || nsteps < 0) {
    return err_set(LUDWIG_GB_EINVAL, "lb2_step: ndist 2 lb, phi of fe");
  }
  lgbk_collide_t cp;
  if ((rc = collide_param(lb, &cp))) return rc;
  if ((rc = grad_alloc(s->dphi))) return rc;
  lgbk_symm_t sp = {s->param.a, s->param.b, s->param.kappa};
  const lgbk_dims_t * d = &lb->cs->d;
  for (int n = 0; n < nsteps; n++) {
    CK(lgbk_phi_from_g_f64(d, lb->pending, (const double *) lb->g,
			   (double *) phi->data, stream_), "phi_from_g");
    CK(grad_launch(s->dphi), "field_grad_compute");
    CK(lgbk_collide_binary_f64(d, &sp, &cp, ph->mobility, lb->pending,
			       (const double *) lb->f, (const double *) lb->g,
			       (const double *) phi->data, s->dphi->grad,
			       s->dphi->delsq, (double *) lb->fprime,
			       (double *) lb->gprime, (double *) hydro->u,
			       stream_), "collide binary");
    lb_swap(lb);
    lb_swap_g(lb);
    lb->pending = 1;                    /* lb_propagation */
  }
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int lb_collide(lb_t * lb, hydro_t * hydro, map_t * map, noise_t * noise,
	       fe_t * fe, visc_t * visc) {
  (void) fe;
  if (hydro == NULL) return LUDWIG_GB_OK;
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "lb_collide: lb NULL");
  if (noise != NULL || visc != NULL) {
    return err_set(LUDWIG_GB_EINVAL, "lb_collide: noise/visc not supported");
  }
  if (lb->prec != LUDWIG_GB_FP64 || hydro->prec != LUDWIG_GB_FP64) {
    return err_set(LUDWIG_GB_EINVAL, "lb_collide: FP64 objects only");
  }
  lgbk_collide_t cp;
  int rc = collide_param(lb, &cp);
  if (rc) return rc;
  if (lb->ndist == 2) return lb_collide_binary(lb, hydro, map, fe, &cp);
  if (lb->pending) {
    /* streaming still pending: pull and collide in one pass, into f' */
    CK(lgbk_collide_pull_f64(&lb->cs->d, &cp, map_dev(map),
			     (const double *) lb->f, (double *) lb->fprime,
			     (const double *) hydro->force,
			     (double *) hydro->rho, (double *) hydro->u,
			     stream_), "collide");
    lb_swap(lb);
    lb->pending = 0;
  }
  else {
    CK(lgbk_collide_f64(&lb->cs->d, &cp, map_dev(map), (double *) lb->f,
			(const double *) hydro->force, (double *) hydro->rho,
			(double *) hydro->u, stream_), "collide");
  }
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int lb_propagation(lb_t * lb) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "lb_propagation");
  int rc = lb_materialise(lb);
  if (rc) return rc;
  lb->pending = 1;
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Fused step with CUDA-graph replay
 *****************************************************************************/

typedef struct graph_cache_s {
  lgbk_binary_args_t args;     /* arguments of the first step of the pair */
  int prec;
  int xchunk, ty, minb, sites;
  lgbk_dims_t d;
  cudaGraphExec_t exec;
  int valid;
} graph_cache_t;

static graph_cache_t gcache_[2];

static int binary_args(lb_t * lb, field_t * phi, hydro_t * hydro,
		       map_t * map, fe_t * fe, lgbk_binary_args_t * a) {
  fe_symm_t * s = NULL;
  physics_t * ph = NULL;
  int rc = fe_symm_get(fe, &s);
  if (rc == 0) rc = phys_get(&ph);
  if (rc) return rc;
  if (lb == NULL || phi == NULL || hydro == NULL || phi->nf != 1) {
    return err_set(LUDWIG_GB_EINVAL, "binary_step: lb, phi, hydro required");
  }
  int fp = (lb->prec == LUDWIG_GB_FP64);
  if (fp != (phi->prec == LUDWIG_GB_FP64) ||
      fp != (hydro->prec == LUDWIG_GB_FP64)) {
    return err_set(LUDWIG_GB_EINVAL, "binary_step: lb, phi and hydro must "
		   "be all FP64 or all reduced precision");
  }
  if (lb->cs->d.nsites != phi->cs->d.nsites ||
      lb->cs->d.nsites != hydro->cs->d.nsites) {
    return err_set(LUDWIG_GB_EINVAL, "binary_step: lattice mismatch");
  }
  if (s->dphi && s->dphi->stencil != 7) {
    return err_set(LUDWIG_GB_EINVAL, "binary_step: the fused step uses "
		   "7-point gradients (call the per-function path for 27)");
  }
  if (advection_order_ != 1) {
    return err_set(LUDWIG_GB_EINVAL, "binary_step: the fused step uses "
		   "first-order advection");
  }
  memset(a, 0, sizeof(*a));
  if ((rc = collide_param(lb, &a->cp))) return rc;
  if (lb->prec != LUDWIG_GB_FP64 && !a->cp.ghosts_zero) {
    return err_set(LUDWIG_GB_EINVAL, "reduced precision: M10 only");
  }
  a->f_in = lb->f;       a->f_out = lb->fprime;
  a->phi_in = phi->data; a->phi_out = phi->data2;
  a->u_in = hydro->u;    a->u_out = hydro->u2;
  a->rho_out = hydro->rho;
  a->force_out = NULL;
  a->status = map_dev(map);
  a->mobility = ph->mobility;
  a->rho0 = lb->rho0;
  a->fscale = lb->fscale;
  a->fe.a = s->param.a; a->fe.b = s->param.b; a->fe.kappa = s->param.kappa;
  lgbk_binary_args_pack(a);
  return LUDWIG_GB_OK;
}

static void binary_swap(lb_t * lb, field_t * phi, hydro_t * hydro) {
  void * t;
  lb_swap(lb);
  t = phi->data; phi->data = phi->data2; phi->data2 = t;
  t = hydro->u; hydro->u = hydro->u2; hydro->u2 = t;
}

static int pair_graph(const lgbk_binary_args_t * a, int prec,
		      const lgbk_dims_t * d, cudaGraphExec_t * exec) {
  graph_cache_t * slot = NULL;
  for (int i = 0; i < 2; i++) {
    graph_cache_t * g = gcache_ + i;
    if (g->valid && g->prec == prec && g->xchunk == tune_xchunk_ &&
	g->ty == tune_ty_ && g->minb == tune_minb_ &&
	g->sites == tune_sites_ &&
	memcmp(&g->d, d, sizeof(*d)) == 0 &&
	memcmp(&g->args, a, sizeof(*a)) == 0) {
      *exec = g->exec;
      return LUDWIG_GB_OK;
    }
  }
  /* replace the older slot */
  slot = gcache_[0].valid ? (gcache_[1].valid ? gcache_ : gcache_ + 1)
                          : gcache_;
  if (slot->valid) {
    cudaGraphExecDestroy(slot->exec);
    slot->valid = 0;
  }
  lgbk_binary_args_t b = *a;
  b.f_in = a->f_out;     b.f_out = (void *) a->f_in;
  b.phi_in = a->phi_out; b.phi_out = (void *) a->phi_in;
  b.u_in = a->u_out;     b.u_out = (void *) a->u_in;

  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed),
     "BeginCapture");
  int rc1 = lgbk_binary_step(d, prec, a, tune_xchunk_, tune_ty_, tune_minb_, tune_sites_, stream_);
  int rc2 = lgbk_binary_step(d, prec, &b, tune_xchunk_, tune_ty_, tune_minb_, tune_sites_, stream_);
  int rc3 = cudaStreamEndCapture(stream_, &graph);
  if (rc1 || rc2 || rc3) {
    return cuda_check(rc1 ? rc1 : (rc2 ? rc2 : rc3), "graph capture");
  }
  int rc = cudaGraphInstantiate(&slot->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (rc) return cuda_check(rc, "cudaGraphInstantiate");
  slot->args = *a;
  slot->prec = prec;
  slot->d = *d;
  slot->xchunk = tune_xchunk_;
  slot->ty = tune_ty_;
  slot->minb = tune_minb_;
  slot->sites = tune_sites_;
  slot->valid = 1;
  *exec = slot->exec;
  return LUDWIG_GB_OK;
}

int ludwig_gb_binary_step_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				map_t * map, fe_t * fe, int nsteps) {
  lgbk_binary_args_t a;
  int rc;
  if (nsteps < 0) return err_set(LUDWIG_GB_EINVAL, "nsteps < 0");
  if ((rc = binary_args(lb, phi, hydro, map, fe, &a))) return rc;
  if ((rc = lb_unstream(lb))) return rc;
  a.f_in = lb->f;
  a.f_out = lb->fprime;

  const lgbk_dims_t * d = &lb->cs->d;
  int npair = nsteps/2;
  if (npair > 0) {
    cudaGraphExec_t exec = NULL;
    if ((rc = pair_graph(&a, lb->prec, d, &exec))) return rc;
    for (int k = 0; k < npair; k++) {
      CK(cudaGraphLaunch(exec, stream_), "cudaGraphLaunch");
    }
  }
  if (nsteps % 2) {
    CK(lgbk_binary_step(d, lb->prec, &a, tune_xchunk_, tune_ty_, tune_minb_, tune_sites_,
			 stream_),
       "binary_step");
    binary_swap(lb, phi, hydro);
  }
  return LUDWIG_GB_OK;
}

/* Derive the FP16 storage scale of lb from the range of its stored
 * deviations and requantise them (a power-of-two factor: exact unless a
 * value leaves half precision's range).  No-op for other precisions. */
int ludwig_gb_lb_fp16_rescale(lb_t * lb, double * scale) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "fp16_rescale: lb NULL");
  if (lb->prec != LUDWIG_GB_FP16) {
    if (scale) *scale = 1.0;
    return LUDWIG_GB_OK;
  }
  const long long n = NVEL*lb->cs->d.nsites;
  unsigned int * word = NULL;
  int rc = dev_alloc((void **) &word, sizeof(unsigned int), "absmax");
  if (rc) return rc;
  float mstored = 0.0f;
  rc = lgbk_half_absmax(n, lb->f, word, &mstored, stream_);
  dev_free(word);
  if (rc) return cuda_check(rc, "fp16_rescale");
  if (!isfinite(mstored)) {
    return err_set(LUDWIG_GB_ENOTFINITE, "fp16_rescale: stored values not "
		   "finite");
  }
  const double sc = fp16_scale_for((double) mstored/lb->fscale);
  if (sc > 0.0 && sc != lb->fscale) {
    CK(lgbk_half_scale(n, lb->f, (float) (sc/lb->fscale), stream_),
       "fp16_rescale");
    CK(cudaStreamSynchronize(stream_), "sync");
    lb->fscale = sc;
  }
  lb->fp16_since = 0;
  if (scale) *scale = lb->fscale;
  return LUDWIG_GB_OK;
}

int ludwig_gb_binary_step(lb_t * lb, field_t * phi, hydro_t * hydro,
			  map_t * map, fe_t * fe, int nsteps) {
  if (lb != NULL && lb->prec == LUDWIG_GB_FP16 && nsteps > 0) {
    /* FP16 storage: the scale is derived again from the range every
     * LGB_FP16_RESCALE_STEPS steps */
    while (nsteps > 0) {
      int k = LGB_FP16_RESCALE_STEPS - lb->fp16_since;
      if (k > nsteps) k = nsteps;
      int rc = ludwig_gb_binary_step_async(lb, phi, hydro, map, fe, k);
      if (rc) return rc;
      nsteps -= k;
      lb->fp16_since += k;
      if (lb->fp16_since >= LGB_FP16_RESCALE_STEPS) {
	if ((rc = ludwig_gb_lb_fp16_rescale(lb, NULL))) return rc;
      }
    }
    return ludwig_gb_sync();
  }
  int rc = ludwig_gb_binary_step_async(lb, phi, hydro, map, fe, nsteps);
  if (rc) return rc;
  return ludwig_gb_sync();
}

/*****************************************************************************
 *  Statistics
 *****************************************************************************/

int stats_field_q(field_t * field, int n, double out[5]) {
  if (field == NULL || n < 0 || n >= field->nf || out == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "stats_field_q");
  }
  double * scr = NULL, r[4];
  int rc = red_scratch(&scr);
  if (rc) return rc;
  const lgbk_dims_t * d = &field->cs->d;
  const char * a = (const char *) field->data
    + (size_t) n*d->nsites*field_size(field->prec);
  CK(lgbk_field_stats(d, field_kprec(field->prec), a, scr, r, stream_),
     "field_stats");
  double vol = (double) d->nsites;
  double rvol = 1.0/vol;
  out[0] = r[0];
  out[1] = rvol*r[0];
  out[2] = rvol*r[1] - out[1]*out[1];
  out[3] = r[2];
  out[4] = r[3];
  if (!isfinite(r[0]) || !isfinite(r[1])) {
    return err_set(LUDWIG_GB_ENOTFINITE, "stats_field_q: NaN or Inf");
  }
  return LUDWIG_GB_OK;
}

/* Velocity statistics, src/stats_velocity.c:54-125: out = {min u_x, u_y,
 * u_z, max u_x, u_y, u_z, volume flux (sum u) x, y, z} over the fluid
 * sites of the map (all sites for map NULL).  As there, the minimum
 * starts from FLT_MAX and the maximum from FLT_MIN (the smallest positive
 * float), so a component that is negative everywhere reports FLT_MIN as
 * its maximum. */
int ludwig_gb_stats_velocity_minmax(hydro_t * hydro, map_t * map,
				    double out[9]) {
  if (hydro == NULL || out == NULL) return err_set(LUDWIG_GB_EINVAL, "stats");
  const lgbk_dims_t * d = &hydro->cs->d;
  if (map && map->cs->d.nsites != d->nsites) {
    return err_set(LUDWIG_GB_EINVAL, "stats_velocity_minmax: map size");
  }
  double * scr = NULL, r[3];
  int rc = red_scratch(&scr);
  if (rc) return rc;
  const uint8_t * st = (map && !map->all_fluid) ? map->status : NULL;
  for (int a = 0; a < 3; a++) {
    const char * u = (const char *) hydro->u
      + (size_t) a*d->nsites*field_size(hydro->prec);
    CK(lgbk_masked_cols(d, field_kprec(hydro->prec), 1, u, st, scr, r,
			stream_), "stats_velocity");
    out[a] = fmin((double) FLT_MAX, r[1]);
    out[3 + a] = fmax((double) FLT_MIN, r[2]);
    out[6 + a] = r[0];
  }
  return LUDWIG_GB_OK;
}

int stats_distribution(lb_t * lb, double out[4]) {
  if (lb == NULL || out == NULL) return err_set(LUDWIG_GB_EINVAL, "stats");
  double * scr = NULL, r[6];
  int rc = red_scratch(&scr);
  if (rc) return rc;
  const lgbk_dims_t * d = &lb->cs->d;
  /* Streaming only permutes values: the sums are the same either way. */
  CK(lgbk_dist_moments(d, lb->prec, lb->f, lb->fscale, scr, r, stream_),
     "dist_moments");
  out[0] = r[0];
  if (lb->prec != LUDWIG_GB_FP64) out[0] += lb->rho0*(double) d->nsites;
  out[1] = r[1]; out[2] = r[2]; out[3] = r[3];
  if (!isfinite(out[0])) {
    return err_set(LUDWIG_GB_ENOTFINITE, "stats_distribution: NaN or Inf");
  }
  return LUDWIG_GB_OK;
}

int stats_free_energy_symm(fe_symm_t * fe, double * total) {
  if (fe == NULL || total == NULL) return err_set(LUDWIG_GB_EINVAL, "stats");
  double * scr = NULL, r[3];
  int rc = red_scratch(&scr);
  if (rc) return rc;
  lgbk_symm_t sp = {fe->param.a, fe->param.b, fe->param.kappa};
  if (fe->dphi && fe->dphi->stencil != 7) {
    /* the stored gradients of the last field_grad_compute, as the
     * reference's fe_symm_fed (src/symmetric.c:285) reads them */
    if (fe->dphi->grad == NULL || fe->phi->prec != LUDWIG_GB_FP64) {
      return err_set(LUDWIG_GB_ESTATE, "stats_free_energy_symm: call "
		     "field_grad_compute() first");
    }
    CK(lgbk_symm_fed_total_grad(&fe->phi->cs->d, &sp,
				(const double *) fe->phi->data,
				fe->dphi->grad, scr, r, stream_), "fed");
  }
  else {
    CK(lgbk_symm_fed_total(&fe->phi->cs->d, field_kprec(fe->phi->prec), &sp,
			   fe->phi->data, scr, r, stream_), "fed");
  }
  *total = r[0];
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Raw state transfer, pinned memory, timing
 *****************************************************************************/

int ludwig_gb_state_bytes(lb_t * lb, size_t * fb, size_t * pb, size_t * ub) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "state_bytes");
  size_t n = (size_t) lb->cs->d.nsites;
  if (fb) *fb = NVEL*n*prec_size(lb->prec);
  if (pb) *pb = n*field_size(lb->prec);
  if (ub) *ub = 3*n*field_size(lb->prec);
  return LUDWIG_GB_OK;
}

int ludwig_gb_state_to_host_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				  void * f, void * ph, void * u) {
  size_t fb, pb, ub;
  if (lb == NULL || phi == NULL || hydro == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "state_to_host");
  }
  ludwig_gb_state_bytes(lb, &fb, &pb, &ub);
  int rc = lb_unstream(lb);
  if (rc) return rc;
  if (f)  CK(cudaMemcpyAsync(f, lb->f, fb, cudaMemcpyDeviceToHost, stream_),
	     "f");
  if (ph) CK(cudaMemcpyAsync(ph, phi->data, pb, cudaMemcpyDeviceToHost,
			     stream_), "phi");
  if (u)  CK(cudaMemcpyAsync(u, hydro->u, ub, cudaMemcpyDeviceToHost,
			     stream_), "u");
  return LUDWIG_GB_OK;
}

int ludwig_gb_state_from_host_async(lb_t * lb, field_t * phi, hydro_t * hydro,
				    const void * f, const void * ph,
				    const void * u) {
  size_t fb, pb, ub;
  if (lb == NULL || phi == NULL || hydro == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "state_from_host");
  }
  ludwig_gb_state_bytes(lb, &fb, &pb, &ub);
  if (f) {
    CK(cudaMemcpyAsync(lb->f, f, fb, cudaMemcpyHostToDevice, stream_), "f");
    lb->pending = 1;
  }
  if (ph) CK(cudaMemcpyAsync(phi->data, ph, pb, cudaMemcpyHostToDevice,
			     stream_), "phi");
  if (u)  CK(cudaMemcpyAsync(hydro->u, u, ub, cudaMemcpyHostToDevice,
			     stream_), "u");
  return LUDWIG_GB_OK;
}

int ludwig_gb_host_alloc(size_t bytes, void ** p) {
  if (p == NULL) return err_set(LUDWIG_GB_EINVAL, "host_alloc");
  if (cudaMallocHost(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return err_set(LUDWIG_GB_ENOMEM, "cudaMallocHost(%zu)", bytes);
  }
  return LUDWIG_GB_OK;
}

int ludwig_gb_host_free(void * p) {
  if (p) cudaFreeHost(p);
  return LUDWIG_GB_OK;
}

int ludwig_gb_time_binary(lb_t * lb, field_t * phi, hydro_t * hydro,
			  map_t * map, fe_t * fe, int nsteps, double * ms) {
  cudaEvent_t e0, e1;
  int rc;
  /* settle the state and the graph outside the timed region */
  if ((rc = lb_unstream(lb))) return rc;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  CK(cudaEventRecord(e0, stream_), "record");
  rc = ludwig_gb_binary_step_async(lb, phi, hydro, map, fe, nsteps);
  if (rc == 0) rc = cuda_check(cudaEventRecord(e1, stream_), "record");
  if (rc == 0) rc = cuda_check(cudaEventSynchronize(e1), "sync");
  if (rc == 0) {
    float t = 0.0f;
    rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int ludwig_gb_time_binary_e2e(lb_t * lb, field_t * phi, hydro_t * hydro,
			      map_t * map, fe_t * fe, int nsteps, void * f_h,
			      void * phi_h, void * u_h, void * rho_h,
			      double * ms) {
  cudaEvent_t e0, e1;
  int rc = 0;
  size_t pb = 0;
  ludwig_gb_state_bytes(lb, NULL, &pb, NULL);
  if ((rc = lb_unstream(lb))) return rc;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  CK(cudaEventRecord(e0, stream_), "record");
  for (int k = 0; rc == 0 && k < nsteps; k++) {
    rc = ludwig_gb_state_from_host_async(lb, phi, hydro, f_h, phi_h, u_h);
    if (rc == 0) rc = ludwig_gb_binary_step_async(lb, phi, hydro, map, fe, 1);
    if (rc == 0) rc = ludwig_gb_state_to_host_async(lb, phi, hydro, f_h,
						     phi_h, u_h);
    if (rc == 0 && rho_h) {
      rc = cuda_check(cudaMemcpyAsync(rho_h, hydro->rho, pb,
				      cudaMemcpyDeviceToHost, stream_), "rho");
    }
  }
  if (rc == 0) rc = cuda_check(cudaEventRecord(e1, stream_), "record");
  if (rc == 0) rc = cuda_check(cudaEventSynchronize(e1), "sync");
  if (rc == 0) {
    float t = 0.0f;
    rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

/* End to end with the copies of consecutive steps overlapped: every step
 * copies the same host input (in_*: stored f, phi, u) to the device, takes
 * one fused step and copies the result (out_*: f, phi, u, rho) back.  Two
 * device buffer sets alternate between steps, and three streams (host to
 * device, step, device to host) let the upload of step k+1 run while the
 * download of step k does.  On return the objects hold the input state. */
int ludwig_gb_time_binary_e2e_overlap(lb_t * lb, field_t * phi,
				      hydro_t * hydro, map_t * map, fe_t * fe,
				      int nsteps, const void * in_f,
				      const void * in_phi, const void * in_u,
				      void * out_f, void * out_phi,
				      void * out_u, void * out_rho,
				      double * ms) {
  if (ms == NULL || nsteps < 1 || in_f == NULL || in_phi == NULL ||
      in_u == NULL || out_f == NULL || out_phi == NULL || out_u == NULL ||
      out_rho == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "time_binary_e2e_overlap");
  }
  lgbk_binary_args_t a[2];
  int rc = binary_args(lb, phi, hydro, map, fe, &a[0]);
  if (rc) return rc;
  if ((rc = lb_unstream(lb))) return rc;
  a[0].f_in = lb->f;       a[0].f_out = lb->fprime;
  a[0].phi_in = phi->data; a[0].phi_out = phi->data2;
  a[0].u_in = hydro->u;    a[0].u_out = hydro->u2;
  a[0].rho_out = hydro->rho;
  size_t fb, pb, ub;
  ludwig_gb_state_bytes(lb, &fb, &pb, &ub);
  const size_t sz[7] = {fb, fb, pb, pb, ub, ub, pb};
  void * b[7] = {NULL};
  for (int k = 0; rc == 0 && k < 7; k++) rc = dev_alloc(b + k, sz[k], "e2e");
  a[1] = a[0];
  a[1].f_in = b[0];   a[1].f_out = b[1];
  a[1].phi_in = b[2]; a[1].phi_out = b[3];
  a[1].u_in = b[4];   a[1].u_out = b[5];
  a[1].rho_out = b[6];
  const lgbk_dims_t * d = &lb->cs->d;
  cudaStream_t st[3] = {NULL, NULL, NULL};
  cudaEvent_t ev[3][2], e0 = NULL, e1 = NULL;
  memset(ev, 0, sizeof(ev));
  for (int i = 0; rc == 0 && i < 3; i++) {
    rc = cuda_check(cudaStreamCreateWithFlags(st + i, cudaStreamNonBlocking),
		    "stream");
    for (int x = 0; rc == 0 && x < 2; x++) {
      rc = cuda_check(cudaEventCreateWithFlags(&ev[i][x],
					       cudaEventDisableTiming), "event");
    }
  }
  if (rc == 0) rc = cuda_check(cudaEventCreate(&e0), "event");
  if (rc == 0) rc = cuda_check(cudaEventCreate(&e1), "event");
  /* start after everything queued on the library stream */
  if (rc == 0) rc = cuda_check(cudaStreamSynchronize(stream_), "sync");
  if (rc == 0) rc = cuda_check(cudaEventRecord(e0, st[0]), "record");
  for (int k = 0; rc == 0 && k < nsteps; k++) {
    const int x = k & 1;
    const lgbk_binary_args_t * ax = a + x;
    /* upload: buffer set x is free once its previous download is done */
    if (k >= 2) rc = cuda_check(cudaStreamWaitEvent(st[0], ev[2][x], 0),
				"wait");
    if (rc == 0) rc = cudaMemcpyAsync((void *) ax->f_in, in_f, fb,
				      cudaMemcpyHostToDevice, st[0]);
    if (rc == 0) rc = cudaMemcpyAsync((void *) ax->phi_in, in_phi, pb,
				      cudaMemcpyHostToDevice, st[0]);
    if (rc == 0) rc = cudaMemcpyAsync((void *) ax->u_in, in_u, ub,
				      cudaMemcpyHostToDevice, st[0]);
    if (rc == 0) rc = cudaEventRecord(ev[0][x], st[0]);
    /* step */
    if (rc == 0) rc = cudaStreamWaitEvent(st[1], ev[0][x], 0);
    if (rc == 0) rc = lgbk_binary_step(d, lb->prec, ax, tune_xchunk_, tune_ty_,
				       tune_minb_, tune_sites_, st[1]);
    if (rc == 0) rc = cudaEventRecord(ev[1][x], st[1]);
    /* download */
    if (rc == 0) rc = cudaStreamWaitEvent(st[2], ev[1][x], 0);
    if (rc == 0) rc = cudaMemcpyAsync(out_f, ax->f_out, fb,
				      cudaMemcpyDeviceToHost, st[2]);
    if (rc == 0) rc = cudaMemcpyAsync(out_phi, ax->phi_out, pb,
				      cudaMemcpyDeviceToHost, st[2]);
    if (rc == 0) rc = cudaMemcpyAsync(out_u, ax->u_out, ub,
				      cudaMemcpyDeviceToHost, st[2]);
    if (rc == 0) rc = cudaMemcpyAsync(out_rho, ax->rho_out, pb,
				      cudaMemcpyDeviceToHost, st[2]);
    if (rc == 0) rc = cudaEventRecord(ev[2][x], st[2]);
    if (rc) rc = cuda_check(rc, "e2e_overlap");
  }
  if (rc == 0) rc = cuda_check(cudaEventRecord(e1, st[2]), "record");
  if (rc == 0) rc = cuda_check(cudaEventSynchronize(e1), "sync");
  if (rc == 0) {
    float t = 0.0f;
    rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
  }
  for (int i = 0; i < 3; i++) {
    if (st[i]) cudaStreamSynchronize(st[i]);
  }
  for (int i = 0; i < 3; i++) {
    for (int x = 0; x < 2; x++) if (ev[i][x]) cudaEventDestroy(ev[i][x]);
    if (st[i]) cudaStreamDestroy(st[i]);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  for (int k = 0; k < 7; k++) dev_free(b[k]);
  /* set 0 holds the uploaded input: f in the stored, unstreamed form */
  lb->pending = 1;
  return rc;
}

/*****************************************************************************
 *  Domain length from the structure factor
 *****************************************************************************/

int ludwig_gb_length_from_sk(field_t * phi, int faithful, double * length,
			     double * sk, double * nk) {
  if (phi == NULL || phi->nf != 1 || length == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "length_from_sk: scalar field");
  }
  const lgbk_dims_t * d = &phi->cs->d;
  if (d->nx > LGBK_SK_NMAX || d->ny > LGBK_SK_NMAX || d->nz > LGBK_SK_NMAX) {
    return err_set(LUDWIG_GB_EINVAL, "length_from_sk: extent > %d",
		   LGBK_SK_NMAX);
  }
  void * work = NULL;
  double skh[LGBK_SK_NBIN], nkh[LGBK_SK_NBIN];
  int rc = dev_alloc(&work, lgbk_structure_factor_work_bytes(d), "sk");
  if (rc) return rc;
  rc = lgbk_structure_factor(d, field_kprec(phi->prec), phi->data, faithful,
			     work, skh, nkh, stream_);
  dev_free(work);
  if (rc) return cuda_check(rc, "structure_factor");

  /* quadrature of the binned S(k), util/length_from_sk.c:170-185 */
  const double pi = 3.14159265358979323846;
  const double dk = sqrt(3.0)*pi/LGBK_SK_NBIN;
  double sum1 = 0.0, sum2 = 0.0;
  for (int k = 0; k < LGBK_SK_NBIN; k++) {
    double sbar = (nkh[k] != 0.0) ? skh[k]/nkh[k] : 0.0;
    double kk = (k + 0.5)*dk;
    sum1 += dk*sbar;
    sum2 += kk*dk*sbar;
  }
  *length = 2.0*pi*sum1/sum2;
  if (sk) memcpy(sk, skh, sizeof(skh));
  if (nk) memcpy(nk, nkh, sizeof(nkh));
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Ensembles of independent boxes
 *****************************************************************************/

struct ludwig_gb_ensemble_s {
  int nbox;
  int prec;
  ludwig_gb_box_param_t * param;
  long long * off;             /* first site of each box */
  long long ntot;
  int * active;
  void * f[2];                 /* 19 x ntot each (storage type) */
  void * phi[2];               /* ntot */
  void * u[2];                 /* 3 x ntot */
  void * rho;                  /* ntot */
  lgbk_box_t * boxes_h[2];     /* arrangement k: reads buffer k */
  lgbk_box_t * boxes_d[2];
  int * items_d;               /* (box, item) pairs, longest items first */
  int nitems;
  int * sched_d;               /* work counters of the ensemble kernels */
  int xchunk, ty, minb;
  int parity;                  /* buffers read by the next step */
  cudaGraphExec_t pair[2];
  int pair_valid[2];
};

static void ens_graph_reset(ludwig_gb_ensemble_t * e) {
  for (int k = 0; k < 2; k++) {
    if (e->pair_valid[k]) cudaGraphExecDestroy(e->pair[k]);
    e->pair_valid[k] = 0;
  }
}

/* Work of an item: its planes plus the two of the pipeline's start */
static int ens_item_cost(const lgbk_dims_t * d, int xchunk, int ty, int k) {
  const int ntz = (d->nz + 31)/32, nty = (d->ny + ty - 1)/ty;
  const int x0 = (k/(ntz*nty))*xchunk;
  const int xl = (d->nx - x0 < xchunk) ? d->nx - x0 : xchunk;
  return xl + 2;
}

typedef struct { int cost, pos, box, item; } ens_item_t;

static int ens_item_cmp(const void * a, const void * b) {
  const ens_item_t * p = (const ens_item_t *) a;
  const ens_item_t * q = (const ens_item_t *) b;
  if (p->cost != q->cost) return (p->cost > q->cost) ? -1 : 1;
  return (p->pos < q->pos) ? -1 : (p->pos > q->pos);
}

static int ens_items(ludwig_gb_ensemble_t * e) {
  int n = 0;
  for (int b = 0; b < e->nbox; b++) {
    lgbk_dims_t d = e->boxes_h[0][b].d;
    n += lgbk_ensemble_items(&d, b, e->xchunk, e->ty, NULL);
  }
  int * h = (int *) malloc(2*(size_t) n*sizeof(int));
  ens_item_t * t = (ens_item_t *) malloc((size_t) n*sizeof(ens_item_t));
  if (h == NULL || t == NULL) {
    free(h);
    free(t);
    return err_set(LUDWIG_GB_ENOMEM, "ensemble items");
  }
  int k = 0;
  for (int b = 0; b < e->nbox; b++) {
    lgbk_dims_t d = e->boxes_h[0][b].d;
    k += lgbk_ensemble_items(&d, b, e->xchunk, e->ty, h + 2*k);
  }
  /* longest items first (list order otherwise kept): the CTAs take them
   * from a counter, so the short items fill in at the end */
  for (int i = 0; i < n; i++) {
    const lgbk_dims_t * d = &e->boxes_h[0][h[2*i]].d;
    t[i].cost = ens_item_cost(d, e->xchunk, e->ty, h[2*i + 1]);
    t[i].pos = i;
    t[i].box = h[2*i];
    t[i].item = h[2*i + 1];
  }
  qsort(t, (size_t) n, sizeof(ens_item_t), ens_item_cmp);
  for (int i = 0; i < n; i++) {
    h[2*i] = t[i].box;
    h[2*i + 1] = t[i].item;
  }
  free(t);
  dev_free(e->items_d);
  e->items_d = NULL;
  int rc = dev_alloc((void **) &e->items_d, 2*(size_t) n*sizeof(int),
		     "items");
  if (rc == 0) {
    rc = cuda_check(cudaMemcpy(e->items_d, h, 2*(size_t) n*sizeof(int),
			       cudaMemcpyHostToDevice), "items");
  }
  free(h);
  e->nitems = n;
  ens_graph_reset(e);
  return rc;
}

static int ens_upload_boxes(ludwig_gb_ensemble_t * e) {
  for (int k = 0; k < 2; k++) {
    for (int b = 0; b < e->nbox; b++) e->boxes_h[k][b].active = e->active[b];
    CK(cudaMemcpy(e->boxes_d[k], e->boxes_h[k], e->nbox*sizeof(lgbk_box_t),
		  cudaMemcpyHostToDevice), "boxes");
  }
  ens_graph_reset(e);
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_free(ludwig_gb_ensemble_t * e) {
  if (e == NULL) return LUDWIG_GB_OK;
  ens_graph_reset(e);
  for (int k = 0; k < 2; k++) {
    dev_free(e->f[k]); dev_free(e->phi[k]); dev_free(e->u[k]);
    dev_free(e->boxes_d[k]);
    free(e->boxes_h[k]);
  }
  dev_free(e->rho);
  dev_free(e->items_d);
  dev_free(e->sched_d);
  free(e->param); free(e->off); free(e->active);
  free(e);
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_create(int nbox, const ludwig_gb_box_param_t * p,
			      int precision, ludwig_gb_ensemble_t ** pens) {
  if (nbox < 1 || p == NULL || pens == NULL ||
      precision < LUDWIG_GB_FP64 || precision > LUDWIG_GB_FP16) {
    return err_set(LUDWIG_GB_EINVAL, "ensemble_create");
  }
  int rc = lib_init();
  if (rc) return rc;
  ludwig_gb_ensemble_t * e =
    (ludwig_gb_ensemble_t *) calloc(1, sizeof(ludwig_gb_ensemble_t));
  if (e == NULL) return err_set(LUDWIG_GB_ENOMEM, "ensemble");
  e->nbox = nbox;
  e->prec = precision;
  e->xchunk = 16; e->ty = 8; e->minb = (precision == LUDWIG_GB_FP64) ? 0 : 3;
  e->param = (ludwig_gb_box_param_t *) malloc(nbox*sizeof(*p));
  e->off = (long long *) calloc(nbox + 1, sizeof(long long));
  e->active = (int *) malloc(nbox*sizeof(int));
  for (int k = 0; k < 2; k++) {
    e->boxes_h[k] = (lgbk_box_t *) calloc(nbox, sizeof(lgbk_box_t));
  }
  if (!e->param || !e->off || !e->active || !e->boxes_h[0] ||
      !e->boxes_h[1]) {
    ludwig_gb_ensemble_free(e);
    return err_set(LUDWIG_GB_ENOMEM, "ensemble");
  }
  memcpy(e->param, p, nbox*sizeof(*p));
  for (int b = 0; b < nbox; b++) {
    for (int i = 0; i < 3; i++) {
      if (p[b].ntotal[i] < 2) {
	ludwig_gb_ensemble_free(e);
	return err_set(LUDWIG_GB_EINVAL, "ensemble: box %d extent < 2", b);
      }
    }
    long long nb = (long long) p[b].ntotal[0]*p[b].ntotal[1]*p[b].ntotal[2];
    if (nb >= LGBK_MAX_SITES) {
      ludwig_gb_ensemble_free(e);
      return err_set(LUDWIG_GB_EINVAL, "ensemble: box %d has 2^32 sites "
		     "or more", b);
    }
    e->off[b + 1] = e->off[b] + nb;
    e->active[b] = 1;
  }
  e->ntot = e->off[nbox];

  const size_t es = prec_size(precision), fs = field_size(precision);
  const size_t n = (size_t) e->ntot;
  for (int k = 0; k < 2 && rc == 0; k++) {
    if ((rc = dev_alloc(&e->f[k], NVEL*n*es, "ens f")) == 0 &&
	(rc = dev_alloc(&e->phi[k], n*fs, "ens phi")) == 0 &&
	(rc = dev_alloc(&e->u[k], 3*n*fs, "ens u")) == 0) {
      rc = dev_alloc((void **) &e->boxes_d[k], nbox*sizeof(lgbk_box_t),
		     "boxes");
    }
  }
  if (rc == 0) rc = dev_alloc(&e->rho, n*fs, "ens rho");
  if (rc) { ludwig_gb_ensemble_free(e); return rc; }

  /* Box descriptors (arrangement 0 reads buffer 0, writes buffer 1) */
  for (int b = 0; b < nbox && rc == 0; b++) {
    const ludwig_gb_box_param_t * q = p + b;
    lgbk_dims_t d = {q->ntotal[0], q->ntotal[1], q->ntotal[2],
		     (long long) q->ntotal[0]*q->ntotal[1]*q->ntotal[2]};
    const double cs2 = (1.0/3.0);
    double eta_bulk = (q->eta_bulk > 0.0) ? q->eta_bulk : q->eta;
    lgbk_binary_args_t a;
    memset(&a, 0, sizeof(a));
    a.cp.rtau_shear = 1.0/(0.5 + q->eta / (q->rho0*cs2));
    a.cp.rtau_bulk = 1.0/(0.5 + eta_bulk / (q->rho0*cs2));
    for (int m = 0; m < NVEL; m++) a.cp.rtau_ghost[m] = 1.0;
    a.cp.ghosts_zero = 1;
    a.mobility = q->mobility;
    a.rho0 = q->rho0;
    a.fscale = 1024.0;
    a.fe.a = q->a; a.fe.b = q->b; a.fe.kappa = q->kappa;
    lgbk_binary_args_pack(&a);
    a.status = NULL;
    a.force_out = NULL;
    a.rho_out = (char *) e->rho + e->off[b]*fs;
    for (int k = 0; k < 2; k++) {
      lgbk_binary_args_t ak = a;
      int in = k, out = 1 - k;
      ak.f_in = (char *) e->f[in] + NVEL*e->off[b]*es;
      ak.f_out = (char *) e->f[out] + NVEL*e->off[b]*es;
      ak.phi_in = (char *) e->phi[in] + e->off[b]*fs;
      ak.phi_out = (char *) e->phi[out] + e->off[b]*fs;
      ak.u_in = (char *) e->u[in] + 3*e->off[b]*fs;
      ak.u_out = (char *) e->u[out] + 3*e->off[b]*fs;
      e->boxes_h[k][b].d = d;
      e->boxes_h[k][b].a = ak;
      e->boxes_h[k][b].active = 1;
    }
  }

  /* Initial state: rest distributions (shift removed), spinodal phi, u = 0
   * (the f buffers are post-collision values; a uniform state streams to
   * itself) */
  for (int b = 0; b < nbox && rc == 0; b++) {
    const ludwig_gb_box_param_t * q = p + b;
    lgbk_dims_t d = e->boxes_h[0][b].d;
    double * tmp = NULL;
    rc = dev_alloc((void **) &tmp, NVEL*(size_t) d.nsites*sizeof(double),
		   "init");
    for (int m = 0; rc == 0 && m < NVEL; m++) {
      static const int w36[NVEL] = {12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2,
				    1, 1, 1, 2, 1, 1};
      rc = lgbk_fill_f64(tmp + m*d.nsites, d.nsites,
			 q->rho0*((double) w36[m]/36.0)*1.0, stream_);
    }
    if (rc == 0) {
      rc = lgbk_f64_to_store(&d, precision, NVEL, q->rho0, 1024.0, tmp,
			     (char *) e->f[0] + NVEL*e->off[b]*es, stream_);
    }
    if (rc == 0) rc = cudaStreamSynchronize(stream_);
    dev_free(tmp);
    if (rc) { rc = cuda_check(rc, "ensemble init"); break; }
  }
  if (rc == 0) {
    rc = cuda_check(cudaMemset(e->u[0], 0, 3*n*fs), "u");
    if (rc == 0) rc = cuda_check(cudaMemset(e->rho, 0, n*fs), "rho");
  }
  for (int b = 0; b < nbox && rc == 0; b++) {
    const ludwig_gb_box_param_t * q = p + b;
    lgbk_dims_t d = e->boxes_h[0][b].d;
    double * h = (double *) malloc(d.nsites*sizeof(double));
    if (h == NULL) { rc = err_set(LUDWIG_GB_ENOMEM, "init"); break; }
    unsigned int seed0 = (q->seed > 1) ? (unsigned int) q->seed : 13u;
    for (int x = 0; x < d.nx; x++) {
      for (int y = 0; y < d.ny; y++) {
	for (int z = 0; z < d.nz; z++) {
	  unsigned int sl[4], st[4];
	  sl[0] = seed0 + (unsigned int) (x + 1);
	  sl[1] = 12953u + (unsigned int) (y + 1);
	  sl[2] = 712357u + (unsigned int) (z + 1);
	  sl[3] = 22383979u;
	  for (int k = 0; k < 4; k++) st[k] = kiss(sl);
	  double ran = (1.0/UINT_MAX)*kiss(st);
	  h[((long long) x*d.ny + y)*d.nz + z] = q->phi0 + q->noise*(ran - 0.5);
	}
      }
    }
    rc = copy_from_host(precision, d.nsites, h,
			(char *) e->phi[0] + e->off[b]*fs);
    free(h);
  }
  if (rc == 0) rc = ens_items(e);
  if (rc == 0) rc = ens_upload_boxes(e);
  if (rc == 0) rc = dev_alloc((void **) &e->sched_d, 2*sizeof(int), "sched");
  if (rc == 0) {
    rc = cuda_check(cudaMemset(e->sched_d, 0, 2*sizeof(int)), "sched");
  }
  if (rc) { ludwig_gb_ensemble_free(e); return rc; }
  e->parity = 0;
  *pens = e;
  return LUDWIG_GB_OK;
}

static int ens_launch(ludwig_gb_ensemble_t * e, int k) {
  return lgbk_ensemble_step(e->prec, e->boxes_d[k], e->items_d, e->nitems,
			    e->xchunk, e->ty, e->minb, 0, tune_sites_,
			    e->sched_d, stream_);
}

static int ens_step_async(ludwig_gb_ensemble_t * e, int nsteps) {
  int npair = nsteps/2;
  if (npair > 0) {
    int k = e->parity;
    if (!e->pair_valid[k]) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed),
	 "capture");
      int rc1 = ens_launch(e, k);
      int rc2 = ens_launch(e, 1 - k);
      int rc3 = cudaStreamEndCapture(stream_, &g);
      if (rc1 || rc2 || rc3) {
	return cuda_check(rc1 ? rc1 : (rc2 ? rc2 : rc3), "ensemble capture");
      }
      int rc = cudaGraphInstantiate(&e->pair[k], g, 0);
      cudaGraphDestroy(g);
      if (rc) return cuda_check(rc, "instantiate");
      e->pair_valid[k] = 1;
    }
    for (int i = 0; i < npair; i++) {
      CK(cudaGraphLaunch(e->pair[k], stream_), "graph launch");
    }
  }
  if (nsteps % 2) {
    CK(ens_launch(e, e->parity), "ensemble step");
    e->parity = 1 - e->parity;
  }
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_step(ludwig_gb_ensemble_t * e, int nsteps) {
  if (e == NULL || nsteps < 0) return err_set(LUDWIG_GB_EINVAL, "ens step");
  int rc = ens_step_async(e, nsteps);
  if (rc) return rc;
  CK(cudaStreamSynchronize(stream_), "sync");
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_time(ludwig_gb_ensemble_t * e, int nsteps,
			    double * ms) {
  cudaEvent_t e0, e1;
  if (e == NULL || ms == NULL) return err_set(LUDWIG_GB_EINVAL, "ens time");
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  CK(cudaEventRecord(e0, stream_), "record");
  int rc = ens_step_async(e, nsteps);
  if (rc == 0) rc = cuda_check(cudaEventRecord(e1, stream_), "record");
  if (rc == 0) rc = cuda_check(cudaEventSynchronize(e1), "sync");
  if (rc == 0) {
    float t = 0.0f;
    rc = cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int ludwig_gb_ensemble_tune_set(ludwig_gb_ensemble_t * e, int xchunk,
				int tile_y, int min_blocks) {
  if (e == NULL || xchunk < 1 || (tile_y != 4 && tile_y != 8 &&
				   tile_y != 16)) {
    return err_set(LUDWIG_GB_EINVAL, "ensemble tune");
  }
  if (e->prec == LUDWIG_GB_FP64) tile_y = 8;     /* one FP64 form */
  e->xchunk = xchunk;
  e->ty = tile_y;
  e->minb = min_blocks;
  return ens_items(e);
}

int ludwig_gb_ensemble_autotune(ludwig_gb_ensemble_t * e, int trial_steps,
				int best[3], double * ms_best) {
  static const int cand[][3] = {{16, 4, 0}, {32, 4, 0}, {8, 4, 0},
				{16, 8, 4}, {32, 8, 4}, {16, 8, 3},
				{32, 8, 3}, {64, 8, 3}, {96, 8, 3},
				{32, 16, 2}};
  const int ncand = (int) (sizeof(cand)/sizeof(cand[0]));
  if (e == NULL || trial_steps < 2) {
    return err_set(LUDWIG_GB_EINVAL, "autotune: trial_steps >= 2");
  }
  /* save the state: the trials advance a copy of it */
  const size_t es = prec_size(e->prec), fs = field_size(e->prec);
  const size_t n = (size_t) e->ntot;
  const int k = e->parity;
  void * sf = NULL, * sp = NULL, * su = NULL;
  int rc = dev_alloc(&sf, NVEL*n*es, "save f");
  if (rc == 0) rc = dev_alloc(&sp, n*fs, "save phi");
  if (rc == 0) rc = dev_alloc(&su, 3*n*fs, "save u");
  if (rc == 0) rc = cuda_check(cudaMemcpy(sf, e->f[k], NVEL*n*es,
					  cudaMemcpyDeviceToDevice), "save");
  if (rc == 0) rc = cuda_check(cudaMemcpy(sp, e->phi[k], n*fs,
					  cudaMemcpyDeviceToDevice), "save");
  if (rc == 0) rc = cuda_check(cudaMemcpy(su, e->u[k], 3*n*fs,
					  cudaMemcpyDeviceToDevice), "save");
  int bi = -1;
  double bt = 1.0e300;
  for (int c = 0; rc == 0 && c < ncand; c++) {
    if (e->prec == LUDWIG_GB_FP64 && cand[c][1] != 8) continue;
    rc = ludwig_gb_ensemble_tune_set(e, cand[c][0], cand[c][1], cand[c][2]);
    double ms = 0.0;
    if (rc == 0) rc = ludwig_gb_ensemble_step(e, 2);        /* warm-up */
    if (rc == 0) rc = ludwig_gb_ensemble_time(e, trial_steps, &ms);
    if (rc == 0 && ms < bt) { bt = ms; bi = c; }
  }
  /* restore */
  if (e->parity != k) e->parity = k;
  if (rc == 0) rc = cuda_check(cudaMemcpy(e->f[k], sf, NVEL*n*es,
					  cudaMemcpyDeviceToDevice), "restore");
  if (rc == 0) rc = cuda_check(cudaMemcpy(e->phi[k], sp, n*fs,
					  cudaMemcpyDeviceToDevice), "restore");
  if (rc == 0) rc = cuda_check(cudaMemcpy(e->u[k], su, 3*n*fs,
					  cudaMemcpyDeviceToDevice), "restore");
  dev_free(sf); dev_free(sp); dev_free(su);
  if (rc == 0 && bi >= 0) {
    rc = ludwig_gb_ensemble_tune_set(e, cand[bi][0], cand[bi][1],
				     cand[bi][2]);
    if (best) { best[0] = cand[bi][0]; best[1] = cand[bi][1];
      best[2] = cand[bi][2]; }
    if (ms_best) *ms_best = bt/trial_steps;
  }
  return rc;
}

int ludwig_gb_ensemble_box_get(ludwig_gb_ensemble_t * e, int box, double * f,
			       double * phi, double * u, double * rho) {
  if (e == NULL || box < 0 || box >= e->nbox) {
    return err_set(LUDWIG_GB_EINVAL, "ensemble box");
  }
  const size_t es = prec_size(e->prec), fs = field_size(e->prec);
  const int k = e->parity;
  lgbk_dims_t d = e->boxes_h[0][box].d;
  int rc = LUDWIG_GB_OK;
  if (f) {
    /* stored values are post-collision: stream them (into the spare
     * buffer, free between steps), then convert */
    void * src = (char *) e->f[k] + NVEL*e->off[box]*es;
    void * dst = (char *) e->f[1 - k] + NVEL*e->off[box]*es;
    double * tmp = NULL;
    rc = cuda_check(lgbk_propagate_store(&d, e->prec, +1, src, dst, stream_),
		    "propagate");
    if (rc == 0) rc = dev_alloc((void **) &tmp,
				NVEL*(size_t) d.nsites*sizeof(double), "tmp");
    if (rc == 0) {
      rc = cuda_check(lgbk_store_to_f64(&d, e->prec, NVEL,
					e->param[box].rho0, 1024.0, dst, tmp,
					stream_), "convert");
    }
    if (rc == 0) rc = cuda_check(cudaMemcpyAsync(f, tmp, NVEL*d.nsites
						 *sizeof(double),
						 cudaMemcpyDeviceToHost,
						 stream_), "f");
    if (rc == 0) rc = cuda_check(cudaStreamSynchronize(stream_), "sync");
    dev_free(tmp);
  }
  if (rc == 0 && phi) {
    rc = copy_to_host(e->prec, d.nsites,
		      (char *) e->phi[k] + e->off[box]*fs, phi);
  }
  if (rc == 0 && u) {
    rc = copy_to_host(e->prec, 3*d.nsites,
		      (char *) e->u[k] + 3*e->off[box]*fs, u);
  }
  if (rc == 0 && rho) {
    rc = copy_to_host(e->prec, d.nsites, (char *) e->rho + e->off[box]*fs,
		      rho);
  }
  return rc;
}

int ludwig_gb_ensemble_box_set_phi(ludwig_gb_ensemble_t * e, int box,
				   const double * phi) {
  if (e == NULL || box < 0 || box >= e->nbox || phi == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "ensemble box");
  }
  const size_t fs = field_size(e->prec);
  lgbk_dims_t d = e->boxes_h[0][box].d;
  return copy_from_host(e->prec, d.nsites,
			phi, (char *) e->phi[e->parity] + e->off[box]*fs);
}

int ludwig_gb_ensemble_check(ludwig_gb_ensemble_t * e, int * nactive) {
  if (e == NULL) return err_set(LUDWIG_GB_EINVAL, "ensemble check");
  double * scr = NULL;
  int rc = red_scratch(&scr);
  if (rc) return rc;
  const size_t es = prec_size(e->prec), fs = field_size(e->prec);
  const int k = e->parity;
  int changed = 0, na = 0;
  for (int b = 0; b < e->nbox; b++) {
    if (!e->active[b]) continue;
    lgbk_dims_t d = e->boxes_h[0][b].d;
    double m[6], q[4];
    CK(lgbk_dist_moments(&d, e->prec, (char *) e->f[k] + NVEL*e->off[b]*es,
			 1024.0, scr, m, stream_), "moments");
    CK(lgbk_field_stats(&d, field_kprec(e->prec),
			(char *) e->phi[k] + e->off[b]*fs, scr, q, stream_),
       "stats");
    if (!isfinite(m[0]) || !isfinite(q[0]) || !isfinite(q[1])) {
      e->active[b] = 0;
      changed = 1;
    }
    else {
      na++;
    }
  }
  if (changed && (rc = ens_upload_boxes(e))) return rc;
  if (nactive) *nactive = na;
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_box_active(ludwig_gb_ensemble_t * e, int box,
				  int * active) {
  if (e == NULL || box < 0 || box >= e->nbox || active == NULL) {
    return err_set(LUDWIG_GB_EINVAL, "ensemble box");
  }
  *active = e->active[box];
  return LUDWIG_GB_OK;
}

int ludwig_gb_ensemble_sites(ludwig_gb_ensemble_t * e, long long * n) {
  if (e == NULL || n == NULL) return err_set(LUDWIG_GB_EINVAL, "sites");
  long long t = 0;
  for (int b = 0; b < e->nbox; b++) {
    if (e->active[b]) t += e->off[b + 1] - e->off[b];
  }
  *n = t;
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Private views for the corrector (lgb_internal.h)
 *****************************************************************************/

int lgb_internal_binary_view(lb_t * lb, field_t * phi, hydro_t * hydro,
			     int layout, lgb_view_t * v) {
  if (lb == NULL || phi == NULL || hydro == NULL || v == NULL ||
      phi->nf != 1) {
    return err_set(LUDWIG_GB_EINVAL, "binary view: lb, phi, hydro");
  }
  if (lb->cs->d.nsites != phi->cs->d.nsites ||
      lb->cs->d.nsites != hydro->cs->d.nsites) {
    return err_set(LUDWIG_GB_EINVAL, "binary view: lattice mismatch");
  }
  int rc = LUDWIG_GB_OK;
  if (layout == 1) rc = lb_unstream(lb);
  else if (layout == 0) rc = lb_materialise(lb);
  if (rc) return rc;
  v->d = lb->cs->d;
  v->prec = lb->prec;
  v->pending = lb->pending;
  v->f = lb->f;
  v->phi = phi->data;
  v->u = hydro->u;
  v->rho = hydro->rho;
  v->rho0 = lb->rho0;
  v->stream = (void *) stream_;
  return LUDWIG_GB_OK;
}

int lgb_internal_lb_set_pending(lb_t * lb, int pending) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "lb");
  lb->pending = pending ? 1 : 0;
  return LUDWIG_GB_OK;
}

int lgb_internal_lb_io(lb_t * lb, int ntotal[3], int * ndist,
		       lgb_io_state_t ** io) {
  if (lb == NULL) return err_set(LUDWIG_GB_EINVAL, "lb");
  for (int a = 0; a < 3; a++) ntotal[a] = lb->cs->ntotal[a];
  *ndist = lb->ndist;
  *io = &lb->io;
  if (lb->io.fmt_in == 0) lb->io.fmt_in = IO_RECORD_BINARY;
  if (lb->io.fmt_out == 0) lb->io.fmt_out = IO_RECORD_BINARY;
  return LUDWIG_GB_OK;
}

int lgb_internal_field_io(field_t * f, int ntotal[3], int * nf,
			  const char ** name, lgb_io_state_t ** io) {
  if (f == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  for (int a = 0; a < 3; a++) ntotal[a] = f->cs->ntotal[a];
  *nf = f->nf;
  *name = f->name;
  *io = &f->io;
  if (f->io.fmt_in == 0) f->io.fmt_in = IO_RECORD_BINARY;
  if (f->io.fmt_out == 0) f->io.fmt_out = IO_RECORD_BINARY;
  return LUDWIG_GB_OK;
}

int lgb_internal_hydro_io(hydro_t * h, int ntotal[3], lgb_io_state_t ** rho,
			  lgb_io_state_t ** vel) {
  if (h == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro");
  for (int a = 0; a < 3; a++) ntotal[a] = h->cs->ntotal[a];
  lgb_io_state_t * s[2] = {&h->io_rho, &h->io_vel};
  for (int k = 0; k < 2; k++) {
    if (s[k]->fmt_in == 0) s[k]->fmt_in = IO_RECORD_BINARY;
    if (s[k]->fmt_out == 0) s[k]->fmt_out = IO_RECORD_BINARY;
  }
  *rho = s[0];
  *vel = s[1];
  return LUDWIG_GB_OK;
}

/*****************************************************************************
 *  Per-site field values at cs_index() sites (src/field.c field_scalar,
 *  field_vector, field_tensor, field_scalar_array and their _set forms)
 *****************************************************************************/

/* Read (write = 0) or write count components n0 .. n0+count-1 of the
 * interior site behind cs_index() site index */
static int field_site_rw(field_t * f, int index, int n0, int count,
			 double * v, int write) {
  if (f == NULL || v == NULL) return err_set(LUDWIG_GB_EINVAL, "field site");
  if (n0 + count > f->nf) {
    return err_set(LUDWIG_GB_EINVAL, "field site: %d components asked of "
		   "a field of %d", n0 + count, f->nf);
  }
  long long i = cs_interior(f->cs, index);
  if (i < 0) return err_set(LUDWIG_GB_EINVAL, "field site: index %d is not "
			    "a cs_index() site", index);
  const size_t N = (size_t) f->cs->d.nsites, es = field_size(f->prec);
  for (int k = 0; k < count; k++) {
    char * a = (char *) f->data + ((size_t) (n0 + k)*N + (size_t) i)*es;
    if (f->prec == LUDWIG_GB_FP64) {
      if (write) CK(cudaMemcpy(a, v + k, 8, cudaMemcpyHostToDevice), "site");
      else CK(cudaMemcpy(v + k, a, 8, cudaMemcpyDeviceToHost), "site");
    }
    else {
      float t = (float) v[k];
      if (write) CK(cudaMemcpy(a, &t, 4, cudaMemcpyHostToDevice), "site");
      else {
	CK(cudaMemcpy(&t, a, 4, cudaMemcpyDeviceToHost), "site");
	v[k] = t;
      }
    }
  }
  return LUDWIG_GB_OK;
}

int field_scalar(field_t * f, int index, double * phi) {
  return field_site_rw(f, index, 0, 1, phi, 0);
}

int field_scalar_set(field_t * f, int index, double phi) {
  return field_site_rw(f, index, 0, 1, &phi, 1);
}

int field_vector(field_t * f, int index, double p[3]) {
  if (f && f->nf != 3) return err_set(LUDWIG_GB_EINVAL, "field_vector: nf 3");
  return field_site_rw(f, index, 0, 3, p, 0);
}

int field_vector_set(field_t * f, int index, const double p[3]) {
  if (f && f->nf != 3) return err_set(LUDWIG_GB_EINVAL, "field_vector: nf 3");
  double v[3] = {p[0], p[1], p[2]};
  return field_site_rw(f, index, 0, 3, v, 1);
}

/* Q from the 5 stored components XX, XY, XZ, YY, YZ (src/field.c) */
int field_tensor(field_t * f, int index, double q[3][3]) {
  if (f && f->nf != 5) return err_set(LUDWIG_GB_EINVAL, "field_tensor: nf 5");
  double v[5];
  int rc = field_site_rw(f, index, 0, 5, v, 0);
  if (rc) return rc;
  q[0][0] = v[0]; q[0][1] = v[1]; q[0][2] = v[2];
  q[1][0] = q[0][1]; q[1][1] = v[3]; q[1][2] = v[4];
  q[2][0] = q[0][2]; q[2][1] = q[1][2]; q[2][2] = 0.0 - q[0][0] - q[1][1];
  return LUDWIG_GB_OK;
}

int field_tensor_set(field_t * f, int index, double q[3][3]) {
  if (f && f->nf != 5) return err_set(LUDWIG_GB_EINVAL, "field_tensor: nf 5");
  double v[5] = {q[0][0], q[0][1], q[0][2], q[1][1], q[1][2]};
  return field_site_rw(f, index, 0, 5, v, 1);
}

int field_scalar_array(field_t * f, int index, double * array) {
  return field_site_rw(f, index, 0, f ? f->nf : 0, array, 0);
}

int field_scalar_array_set(field_t * f, int index, const double * array) {
  double v[5];
  if (f == NULL || array == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  for (int k = 0; k < f->nf; k++) v[k] = array[k];
  return field_site_rw(f, index, 0, f->nf, v, 1);
}

/*****************************************************************************
 *  The reference's host layout: every cs_index() site, halo sites holding
 *  the periodic images, AOS (a[K*index + k]) or SOA (a[nsites*k + index])
 *  (src/memory.h:151-170, src/lb_data.h:144)
 *****************************************************************************/

/* out[layout(index, k)] = in[k][interior(index)] over all cs_index() sites
 * (to = 1), or in the other direction over the interior sites (to = 0) */
static int host_layout(const cs_t * cs, int model, int K, double * in,
		       double * out, int to) {
  if (model != DATA_MODEL_AOS && model != DATA_MODEL_SOA) {
    return err_set(LUDWIG_GB_EINVAL, "data model: DATA_MODEL_AOS or "
		   "DATA_MODEL_SOA");
  }
  const int h = cs->nhalo;
  const int nall[3] = {cs->ntotal[0] + 2*h, cs->ntotal[1] + 2*h,
		       cs->ntotal[2] + 2*h};
  const long long nsites = (long long) nall[0]*nall[1]*nall[2];
  const long long N = cs->d.nsites;
  for (int x = 0; x < nall[0]; x++) {
    int ix = ((x - h) % cs->ntotal[0] + cs->ntotal[0]) % cs->ntotal[0];
    for (int y = 0; y < nall[1]; y++) {
      int iy = ((y - h) % cs->ntotal[1] + cs->ntotal[1]) % cs->ntotal[1];
      for (int z = 0; z < nall[2]; z++) {
	int iz = ((z - h) % cs->ntotal[2] + cs->ntotal[2]) % cs->ntotal[2];
	int interior = (x >= h && x < h + cs->ntotal[0] && y >= h &&
			y < h + cs->ntotal[1] && z >= h &&
			z < h + cs->ntotal[2]);
	if (!to && !interior) continue;
	long long index = ((long long) x*nall[1] + y)*nall[2] + z;
	long long i = ((long long) ix*cs->ntotal[1] + iy)*cs->ntotal[2] + iz;
	for (int k = 0; k < K; k++) {
	  long long a = (model == DATA_MODEL_AOS) ? K*index + k
	    : nsites*k + index;
	  if (to) out[a] = in[k*N + i];
	  else in[k*N + i] = out[a];
	}
      }
    }
  }
  return LUDWIG_GB_OK;
}

static int host_tmp(long long n, double ** p) {
  *p = (double *) malloc((size_t) n*sizeof(double));
  return (*p == NULL) ? err_set(LUDWIG_GB_ENOMEM, "host buffer")
    : LUDWIG_GB_OK;
}

int ludwig_gb_lb_to_host_cs(lb_t * lb, int model, double * f) {
  if (lb == NULL || f == NULL) return err_set(LUDWIG_GB_EINVAL, "lb");
  const long long N = lb->cs->d.nsites;
  double * t = NULL;
  int rc = host_tmp(NVEL*lb->ndist*N, &t);
  if (rc == 0) rc = lb_f_to_host(lb, t);
  if (rc == 0 && lb->ndist == 2) rc = lb_g_to_host(lb, t + NVEL*N);
  if (rc == 0) rc = host_layout(lb->cs, model, NVEL*lb->ndist, t, f, 1);
  free(t);
  return rc;
}

int ludwig_gb_lb_from_host_cs(lb_t * lb, int model, const double * f) {
  if (lb == NULL || f == NULL) return err_set(LUDWIG_GB_EINVAL, "lb");
  const long long N = lb->cs->d.nsites;
  double * t = NULL;
  int rc = host_tmp(NVEL*lb->ndist*N, &t);
  if (rc == 0) rc = host_layout(lb->cs, model, NVEL*lb->ndist, t,
				(double *) f, 0);
  if (rc == 0) rc = lb_f_from_host(lb, t);
  if (rc == 0 && lb->ndist == 2) rc = lb_g_from_host(lb, t + NVEL*N);
  free(t);
  return rc;
}

int ludwig_gb_field_to_host_cs(field_t * obj, int model, double * data) {
  if (obj == NULL || data == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  double * t = NULL;
  int rc = host_tmp(obj->nf*obj->cs->d.nsites, &t);
  if (rc == 0) rc = field_to_host(obj, t);
  if (rc == 0) rc = host_layout(obj->cs, model, obj->nf, t, data, 1);
  free(t);
  return rc;
}

int ludwig_gb_field_from_host_cs(field_t * obj, int model,
				 const double * data) {
  if (obj == NULL || data == NULL) return err_set(LUDWIG_GB_EINVAL, "field");
  double * t = NULL;
  int rc = host_tmp(obj->nf*obj->cs->d.nsites, &t);
  if (rc == 0) rc = host_layout(obj->cs, model, obj->nf, t, (double *) data,
				0);
  if (rc == 0) rc = field_from_host(obj, t);
  free(t);
  return rc;
}

int ludwig_gb_hydro_to_host_cs(hydro_t * obj, int model, double * rho,
			       double * u, double * force) {
  if (obj == NULL) return err_set(LUDWIG_GB_EINVAL, "hydro");
  const long long N = obj->cs->d.nsites;
  double * t = NULL;
  int rc = host_tmp(7*N, &t);
  if (rc == 0) rc = hydro_to_host(obj, t, t + N, t + 4*N);
  if (rc == 0 && rho) rc = host_layout(obj->cs, model, 1, t, rho, 1);
  if (rc == 0 && u) rc = host_layout(obj->cs, model, 3, t + N, u, 1);
  if (rc == 0 && force) rc = host_layout(obj->cs, model, 3, t + 4*N, force,
					 1);
  free(t);
  return rc;
}

int lgb_internal_err(int code, const char * what) {
  return err_set(code, "%s", what);
}

int lgb_internal_cuda(int cuda_rc, const char * where) {
  return cuda_check(cuda_rc, where);
}

/* Make p the physics object the step functions read (the reference keeps
 * one per process; two systems with different mobilities take turns). */
int ludwig_gb_physics_use(physics_t * p) {
  if (p == NULL) return err_set(LUDWIG_GB_EINVAL, "physics_use: NULL");
  phys_ref_ = p;
  return LUDWIG_GB_OK;
}
