/*****************************************************************************
 *
 *  ref_shim.c
 *
 *  Test infrastructure only.  A small driver linked against the
 *  reference (Ludwig v0.23, built from its own sources by oracle/ref.mk)
 *  that runs the reference's own hot-path functions on given inputs and
 *  writes the results as raw little-endian doubles.  It pins the oracle
 *  restatement (oracle/ludwig_oracle.c) and generates the golden fixtures
 *  under tests/golden/.  Nothing in the product links against it.
 *
 *  File layout of every array: interior sites only, component-major,
 *  z fastest:  a[(n*Lx + x)*Ly + y)*Lz + z]  with x,y,z 0-based.
 *
 *  Usage (key=value arguments):
 *    ref_shim mode=run    size=X,Y,Z steps=N A= B= K= M= eta= seed= noise=
 *                         [grad=7|27] [order=1|2|3]
 *                         phi0= out=PREFIX
 *    ref_shim mode=collide  size=.. eta= in=PREFIX out=PREFIX
 *    ref_shim mode=propagate size=.. in=PREFIX out=PREFIX
 *    ref_shim mode=grad     size=.. in=PREFIX out=PREFIX       (nf from file)
 *    ref_shim mode=force    size=.. A= B= K= in=PREFIX out=PREFIX
 *    ref_shim mode=ch       size=.. A= B= K= M= in=PREFIX out=PREFIX
 *    ref_shim mode=step     size=.. A= B= K= M= eta= steps= in=PREFIX out=PREFIX
 *    ref_shim mode=lb2      ndist=2 size=.. steps=N A= B= K= M= eta= seed=
 *                           (symmetric_lb: two distributions)
 *    ref_shim mode=collide2 ndist=2 size=.. in=PREFIX out=PREFIX
 *    ref_shim mode=lc       size=.. steps= a0= gamma= kappa0= kappa1= pitch= xi=
 *                           Gamma= redshift= amplitude= eta= out=PREFIX
 *    ref_shim mode=lc_fields size=.. (lc parameters) in=PREFIX out=PREFIX
 *    ref_shim mode=lc_be    size=.. (lc parameters) in=PREFIX out=PREFIX
 *    ref_shim mode=lc_step  size=.. (lc parameters) steps= in=PREFIX out=PREFIX
 *    ref_shim mode=io_write size=.. ndist=1|2 nf=1|5 fmt=binary|ascii
 *                           step=N in=PREFIX dir=DIR [hydro=1]
 *                           (lb_io_write, field_io_write and, with
 *                           hydro=1, hydro_io_write into DIR)
 *    ref_shim mode=io_read  size=.. ndist= nf= fmt= step=N dir=DIR out=PREFIX
 *                           (lb_io_read and field_io_read from DIR)
 *  Any mode accepts status=FILE (uint8 per site, canonical order; 0 fluid).
 *
 *  The call sequence of mode=run/step follows src/ludwig.c:528-860 for
 *  the symmetric free energy with finite-difference Cahn-Hilliard.
 *
 *****************************************************************************/

#include <assert.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "pe.h"
#include "coords.h"
#include "physics.h"
#include "leesedwards.h"
#include "field.h"
#include "field_grad.h"
#include "gradient_3d_7pt_fluid.h"
#include "gradient_3d_27pt_fluid.h"
#include "symmetric.h"
#include "phi_force.h"
#include "phi_force_stress.h"
#include "phi_cahn_hilliard.h"
#include "hydro.h"
#include "map.h"
#include "lb_data.h"
#include "collision.h"
#include "propagation.h"
#include "field_phi_init.h"
#include "util_sum.h"
#include "wall.h"
#include "blue_phase.h"
#include "blue_phase_init.h"
#include "blue_phase_beris_edwards.h"
#include "colloids.h"
#include "phi_lb_coupler.h"
#include "advection.h"
#include "io_event.h"
#include <unistd.h>

static const char * arg(int argc, char ** argv, const char * key,
			const char * def) {
  size_t n = strlen(key);
  for (int i = 1; i < argc; i++) {
    if (strncmp(argv[i], key, n) == 0 && argv[i][n] == '=') return argv[i]+n+1;
  }
  return def;
}

static double argd(int argc, char ** argv, const char * key, double def) {
  const char * s = arg(argc, argv, key, NULL);
  return s ? atof(s) : def;
}

static int L[3];

static size_t nint(void) { return (size_t) L[0]*L[1]*L[2]; }
static size_t canon(int n, int x, int y, int z) {
  return (((size_t) n*L[0] + x)*L[1] + y)*L[2] + z;
}

static double * readf(const char * prefix, const char * name, size_t n) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_%s.bin", prefix, name);
  FILE * fp = fopen(path, "rb");
  if (fp == NULL) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  double * a = malloc(n*sizeof(double));
  if (fread(a, sizeof(double), n, fp) != n) {
    fprintf(stderr, "short read %s\n", path); exit(2);
  }
  fclose(fp);
  return a;
}

static void writef(const char * prefix, const char * name, const double * a,
		   size_t n) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_%s.bin", prefix, name);
  FILE * fp = fopen(path, "wb");
  if (fp == NULL) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  fwrite(a, sizeof(double), n, fp);
  fclose(fp);
}

/* Field <-> canonical copies (interior only) */

static void field_get(cs_t * cs, field_t * f, double * out) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int n = 0; n < f->nf; n++)
	out[canon(n,x,y,z)] = f->data[addr_rank1(f->nsites, f->nf, index, n)];
    }
}

static void field_put(cs_t * cs, field_t * f, const double * in) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int n = 0; n < f->nf; n++)
	f->data[addr_rank1(f->nsites, f->nf, index, n)] = in[canon(n,x,y,z)];
    }
}

static void lb_get(cs_t * cs, lb_t * lb, double * out) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int p = 0; p < NVEL; p++)
	out[canon(p,x,y,z)] = lb->f[LB_ADDR(lb->nsite, lb->ndist, NVEL,
					     index, 0, p)];
    }
}

static void lb_put(cs_t * cs, lb_t * lb, const double * in) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int p = 0; p < NVEL; p++)
	lb->f[LB_ADDR(lb->nsite, lb->ndist, NVEL, index, 0, p)]
	  = in[canon(p,x,y,z)];
    }
}

typedef struct sys_s {
  pe_t * pe;
  cs_t * cs;
  physics_t * phys;
  lees_edw_t * le;
  field_t * phi;
  field_grad_t * dphi;
  fe_symm_t * fe;
  phi_ch_t * pch;
  pth_t * pth;
  hydro_t * hydro;
  map_t * map;
  lb_t * lb;
  wall_t * wall;
} sys_t;

static void sys_create(int argc, char ** argv, sys_t * s) {

  memset(s, 0, sizeof(*s));
  pe_create(MPI_COMM_WORLD, PE_QUIET, &s->pe);
  cs_create(s->pe, &s->cs);
  cs_nhalo_set(s->cs, 2);
  cs_ntotal_set(s->cs, L);
  cs_init(s->cs);

  physics_create(s->pe, &s->phys);
  {
    double eta = argd(argc, argv, "eta", 0.1);
    physics_eta_shear_set(s->phys, eta);
    physics_eta_bulk_set(s->phys, argd(argc, argv, "eta_bulk", eta));
    physics_mobility_set(s->phys, argd(argc, argv, "M", 0.3));
  }

  {
    lees_edw_options_t opts = {0};
    lees_edw_create(s->pe, s->cs, &opts, &s->le);
  }
  {
    field_options_t opts = field_options_ndata_nhalo(1, 2);
    field_create(s->pe, s->cs, s->le, "phi", &opts, &s->phi);
    field_grad_create(s->pe, s->phi, 2, &s->dphi);
    if (atoi(arg(argc, argv, "grad", "7")) == 27) {
      field_grad_set(s->dphi, grad_3d_27pt_fluid_d2, NULL);
    }
    else {
      field_grad_set(s->dphi, grad_3d_7pt_fluid_d2, NULL);
    }
  }
  advection_order_set(atoi(arg(argc, argv, "order", "1")));
  {
    fe_symm_param_t p = {0};
    p.a     = argd(argc, argv, "A", -0.0625);
    p.b     = argd(argc, argv, "B", +0.0625);
    p.kappa = argd(argc, argv, "K", 0.04);
    fe_symm_create(s->pe, s->cs, s->phi, s->dphi, &s->fe);
    fe_symm_param_set(s->fe, p);
  }
  {
    phi_ch_info_t info = {.conserve = 0, .noise = 0};
    phi_ch_create(s->pe, s->cs, s->le, &info, &s->pch);
  }
  pth_create(s->pe, s->cs, FE_FORCE_METHOD_STRESS_DIVERGENCE, &s->pth);
  {
    hydro_options_t opts = hydro_options_default();
    hydro_create(s->pe, s->cs, s->le, &opts, &s->hydro);
  }
  {
    map_options_t opts = map_options_default();
    map_create(s->pe, s->cs, &opts, &s->map);
  }
  {
    lb_data_options_t opts = lb_data_options_default();
    opts.ndist = atoi(arg(argc, argv, "ndist", "1"));
    lb_data_create(s->pe, s->cs, &opts, &s->lb);
    lb_init_rest_f(s->lb, 1.0);
  }
  wall_create(s->pe, s->cs, s->map, s->lb, &s->wall);

  /* Optional site status (uint8, canonical order), e.g. solid sites */
  {
    const char * sp = arg(argc, argv, "status", NULL);
    if (sp) {
      FILE * fp = fopen(sp, "rb");
      unsigned char * st = malloc(nint());
      if (fp == NULL || fread(st, 1, nint(), fp) != nint()) {
	fprintf(stderr, "cannot read status %s\n", sp); exit(2);
      }
      fclose(fp);
      for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
	for (int z = 0; z < L[2]; z++) {
	  map_status_set(s->map, cs_index(s->cs, x+1, y+1, z+1),
			 st[canon(0,x,y,z)]);
	}
      map_halo(s->map);
      free(st);
    }
  }
}

/* One time step as src/ludwig.c:528-860 (symmetric, FD CH, no colloids). */

static void sys_step(sys_t * s) {
  double zero[3] = {0.0, 0.0, 0.0};
  physics_control_next_step(s->phys);
  hydro_f_zero(s->hydro, zero);
  field_halo(s->phi);
  field_grad_compute(s->dphi);
  phi_force_calculation(s->pe, s->cs, s->le, s->wall, s->pth,
			(fe_t *) s->fe, s->map, s->phi, s->hydro);
  phi_cahn_hilliard(s->pch, (fe_t *) s->fe, s->phi, s->hydro, s->map, NULL);
  hydro_u_zero(s->hydro, zero);
  lb_collide(s->lb, s->hydro, s->map, NULL, (fe_t *) s->fe, NULL);
  lb_halo(s->lb);
  lb_propagation(s->lb);
}

/* One time step of the two-distribution binary fluid (symmetric_lb):
 * src/ludwig.c:528-860 with ndist = 2 (phi from g, gradients, no order
 * parameter dynamics outside the collision). */

static void sys_step_lb2(sys_t * s) {
  double zero[3] = {0.0, 0.0, 0.0};
  physics_control_next_step(s->phys);
  hydro_f_zero(s->hydro, zero);
  phi_lb_to_field(s->phi, s->lb);
  field_halo(s->phi);
  field_grad_compute(s->dphi);
  hydro_u_zero(s->hydro, zero);
  lb_collide(s->lb, s->hydro, s->map, NULL, (fe_t *) s->fe, NULL);
  lb_halo(s->lb);
  lb_propagation(s->lb);
}

static void lb_get_dist(cs_t * cs, lb_t * lb, int nd, double * out) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int p = 0; p < NVEL; p++)
	out[canon(p,x,y,z)] = lb->f[LB_ADDR(lb->nsite, lb->ndist, NVEL,
					     index, nd, p)];
    }
}

static void lb_put_dist(cs_t * cs, lb_t * lb, int nd, const double * in) {
  for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
    for (int z = 0; z < L[2]; z++) {
      int index = cs_index(cs, x+1, y+1, z+1);
      for (int p = 0; p < NVEL; p++)
	lb->f[LB_ADDR(lb->nsite, lb->ndist, NVEL, index, nd, p)]
	  = in[canon(p,x,y,z)];
    }
}

static void sys_dump(sys_t * s, const char * out) {
  size_t n = nint();
  double * a = malloc(NVEL*n*sizeof(double));
  field_get(s->cs, s->phi, a);           writef(out, "phi", a, n);
  field_get(s->cs, s->hydro->u, a);      writef(out, "u", a, 3*n);
  field_get(s->cs, s->hydro->rho, a);    writef(out, "rho", a, n);
  field_get(s->cs, s->hydro->force, a);  writef(out, "force", a, 3*n);
  lb_get(s->cs, s->lb, a);               writef(out, "f", a, NVEL*n);
  if (s->lb->ndist == 2) {
    lb_get_dist(s->cs, s->lb, 1, a);     writef(out, "g", a, NVEL*n);
  }
  free(a);
}


/*****************************************************************************
 *
 *  Cholesteric liquid crystal: src/ludwig.c:1598-1660 set-up and the main
 *  loop order of src/ludwig.c:528-860 (no colloids, walls or planes).
 *
 *****************************************************************************/

typedef struct lcsys_s {
  sys_t b;                    /* pe, cs, physics, le, hydro, map, lb, wall */
  field_t * q;
  field_grad_t * dq;
  fe_lc_t * fe;
  beris_edw_t * be;
  pth_t * pth;
  colloids_info_t * cinfo;
} lcsys_t;

static void lcsys_create(int argc, char ** argv, lcsys_t * s) {
  sys_create(argc, argv, &s->b);
  {
    field_options_t opts = field_options_ndata_nhalo(NQAB, 2);
    field_create(s->b.pe, s->b.cs, s->b.le, "q", &opts, &s->q);
    field_grad_create(s->b.pe, s->q, 2, &s->dq);
    field_grad_set(s->dq, grad_3d_7pt_fluid_d2, NULL);
  }
  fe_lc_create(s->b.pe, s->b.cs, s->b.le, s->q, s->dq, &s->fe);
  {
    fe_lc_param_t p = {0};
    const double pi = 4.0*atan(1.0);
    p.a0 = argd(argc, argv, "a0", 0.01);
    p.gamma = argd(argc, argv, "gamma", 3.0);
    p.kappa0 = argd(argc, argv, "kappa0", 0.01);
    p.kappa1 = argd(argc, argv, "kappa1", 0.01);
    p.q0 = 2.0*pi/argd(argc, argv, "pitch", 32.0);
    p.xi = argd(argc, argv, "xi", 0.7);
    p.redshift = argd(argc, argv, "redshift", 1.0);
    p.amplitude0 = argd(argc, argv, "amplitude", -0.2);
    fe_lc_param_set(s->fe, &p);
  }
  beris_edw_create(s->b.pe, s->b.cs, s->b.le, &s->be);
  {
    beris_edw_param_t bp = {0};
    bp.xi = argd(argc, argv, "xi", 0.7);
    bp.gamma = argd(argc, argv, "Gamma", 0.5);
    beris_edw_param_set(s->be, &bp);
  }
  pth_create(s->b.pe, s->b.cs, FE_FORCE_METHOD_STRESS_DIVERGENCE, &s->pth);
  {
    int ncell[3] = {2, 2, 2};
    colloids_info_create(s->b.pe, s->b.cs, ncell, &s->cinfo);
    colloids_info_map_init(s->cinfo);
  }
}

static void lcsys_step(lcsys_t * s) {
  double zero[3] = {0.0, 0.0, 0.0};
  physics_control_next_step(s->b.phys);
  hydro_f_zero(s->b.hydro, zero);
  field_halo(s->q);
  field_grad_compute(s->dq);
  fe_lc_redshift_compute(s->b.cs, s->fe);
  phi_force_calculation(s->b.pe, s->b.cs, s->b.le, s->b.wall, s->pth,
			(fe_t *) s->fe, s->b.map, s->q, s->b.hydro);
  hydro_u_halo(s->b.hydro);
  beris_edw_update(s->be, (fe_t *) s->fe, s->q, s->dq, s->b.hydro, s->cinfo,
		   s->b.map, NULL);
  hydro_u_zero(s->b.hydro, zero);
  lb_collide(s->b.lb, s->b.hydro, s->b.map, NULL, (fe_t *) s->fe, NULL);
  lb_halo(s->b.lb);
  lb_propagation(s->b.lb);
}

static int lc_main(int argc, char ** argv, const char * mode) {
  lcsys_t s;
  const char * in   = arg(argc, argv, "in", NULL);
  const char * out  = arg(argc, argv, "out", "ref");
  size_t n = nint();
  double * a = malloc(NVEL*n*sizeof(double));

  lcsys_create(argc, argv, &s);

  if (strcmp(mode, "lc") == 0) {
    double angles[3] = {0.0, 0.0, 0.0};
    fe_lc_param_t p;
    int steps = atoi(arg(argc, argv, "steps", "1"));
    fe_lc_param(s.fe, &p);
    blue_phase_O8M_init(s.b.cs, &p, s.q, angles);
    field_get(s.b.cs, s.q, a);
    writef(out, "q0", a, NQAB*n);
    for (int k = 0; k < steps; k++) lcsys_step(&s);
    sys_dump(&s.b, out);
    field_get(s.b.cs, s.q, a);
    writef(out, "q", a, NQAB*n);
  }
  else if (strcmp(mode, "lc_fields") == 0) {
    /* molecular field, stress and free energy density of a given q */
    double * q = readf(in, "q", NQAB*n);
    field_put(s.b.cs, s.q, q);
    field_halo(s.q);
    field_grad_compute(s.dq);
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(s.b.cs, x+1, y+1, z+1);
	double h[3][3], st[3][3], fed;
	fe_lc_mol_field(s.fe, index, h);
	fe_lc_stress(s.fe, index, st);
	fe_lc_fed(s.fe, index, &fed);
	a[canon(0,x,y,z)] = h[0][0]; a[canon(1,x,y,z)] = h[0][1];
	a[canon(2,x,y,z)] = h[0][2]; a[canon(3,x,y,z)] = h[1][1];
	a[canon(4,x,y,z)] = h[1][2];
	for (int ia = 0; ia < 3; ia++) for (int ib = 0; ib < 3; ib++)
	  a[canon(5 + 3*ia + ib,x,y,z)] = st[ia][ib];
	a[canon(14,x,y,z)] = fed;
      }
    writef(out, "h", a, 5*n);
    writef(out, "stress", a + 5*n, 9*n);
    writef(out, "fed", a + 14*n, n);
  }
  else if (strcmp(mode, "lc_be") == 0) {
    double * q = readf(in, "q", NQAB*n);
    double * u = readf(in, "u", 3*n);
    field_put(s.b.cs, s.q, q);
    field_put(s.b.cs, s.b.hydro->u, u);
    field_halo(s.q);
    field_grad_compute(s.dq);
    hydro_u_halo(s.b.hydro);
    beris_edw_update(s.be, (fe_t *) s.fe, s.q, s.dq, s.b.hydro, s.cinfo,
		     s.b.map, NULL);
    field_get(s.b.cs, s.q, a);
    writef(out, "q", a, NQAB*n);
  }
  else if (strcmp(mode, "lc_step") == 0) {
    double * q = readf(in, "q", NQAB*n);
    double * u = readf(in, "u", 3*n);
    double * f = readf(in, "f", NVEL*n);
    int steps = atoi(arg(argc, argv, "steps", "1"));
    field_put(s.b.cs, s.q, q);
    field_put(s.b.cs, s.b.hydro->u, u);
    lb_put(s.b.cs, s.b.lb, f);
    for (int k = 0; k < steps; k++) lcsys_step(&s);
    sys_dump(&s.b, out);
    field_get(s.b.cs, s.q, a);
    writef(out, "q", a, NQAB*n);
  }
  free(a);
  MPI_Finalize();
  return 0;
}

/* Snapshot files through the reference's own I/O (src/lb_data.c:1716-1830,
 * src/field.c:1633-1737): one file per object, single rank. */
static int io_main(int argc, char ** argv, const char * mode) {
  const int ndist = atoi(arg(argc, argv, "ndist", "1"));
  const int nf = atoi(arg(argc, argv, "nf", "1"));
  const int step = atoi(arg(argc, argv, "step", "0"));
  const char * dir = arg(argc, argv, "dir", ".");
  const io_record_format_enum_t fmt =
    strcmp(arg(argc, argv, "fmt", "binary"), "ascii") == 0
    ? IO_RECORD_ASCII : IO_RECORD_BINARY;
  pe_t * pe = NULL;
  cs_t * cs = NULL;
  lb_t * lb = NULL;
  field_t * fld = NULL;
  pe_create(MPI_COMM_WORLD, PE_QUIET, &pe);
  cs_create(pe, &cs);
  cs_nhalo_set(cs, 2);
  cs_ntotal_set(cs, L);
  cs_init(cs);
  {
    lb_data_options_t opts = lb_data_options_default();
    opts.ndist = ndist;
    opts.iodata.input.iorformat = fmt;
    opts.iodata.output.iorformat = fmt;
    lb_data_create(pe, cs, &opts, &lb);
  }
  {
    field_options_t opts = field_options_ndata_nhalo(nf, 2);
    opts.iodata.input.iorformat = fmt;
    opts.iodata.output.iorformat = fmt;
    field_create(pe, cs, NULL, (nf == 5) ? "q" : "phi", &opts, &fld);
  }
  hydro_t * hydro = NULL;
  if (atoi(arg(argc, argv, "hydro", "0"))) {
    hydro_options_t opts = hydro_options_default();
    opts.rho.iodata.input.iorformat = fmt;
    opts.rho.iodata.output.iorformat = fmt;
    opts.u.iodata.input.iorformat = fmt;
    opts.u.iodata.output.iorformat = fmt;
    hydro_create(pe, cs, NULL, &opts, &hydro);
  }
  const size_t n = nint();
  io_event_t event = {0};
  if (strcmp(mode, "io_write") == 0 && hydro) {
    const char * in = arg(argc, argv, "in", NULL);
    double * rho = readf(in, "rho", n);
    double * u = readf(in, "u", 3*n);
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(cs, x+1, y+1, z+1);
	field_t * fr = hydro->rho, * fu = hydro->u;
	fr->data[addr_rank1(fr->nsites, 1, index, 0)] = rho[canon(0,x,y,z)];
	for (int a = 0; a < 3; a++)
	  fu->data[addr_rank1(fu->nsites, 3, index, a)] = u[canon(a,x,y,z)];
      }
    hydro_memcpy(hydro, tdpMemcpyHostToDevice);
  }
  if (strcmp(mode, "io_write") == 0) {
    const char * in = arg(argc, argv, "in", NULL);
    double * f = readf(in, "f", (size_t) ndist*NVEL*n);
    double * q = readf(in, "phi", (size_t) nf*n);
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(cs, x+1, y+1, z+1);
	for (int d = 0; d < ndist; d++) for (int p = 0; p < NVEL; p++)
	  lb->f[LB_ADDR(lb->nsite, ndist, NVEL, index, d, p)]
	    = f[canon(d*NVEL + p, x, y, z)];
	for (int c = 0; c < nf; c++)
	  fld->data[addr_rank1(fld->nsites, nf, index, c)] = q[canon(c,x,y,z)];
      }
    lb_memcpy(lb, tdpMemcpyHostToDevice);
    field_memcpy(fld, tdpMemcpyHostToDevice);
    if (chdir(dir) != 0) return 2;
    if (lb_io_write(lb, step, &event)) return 3;
    if (field_io_write(fld, step, &event)) return 3;
    if (hydro && hydro_io_write(hydro, step, &event)) return 3;
  }
  else {
    const char * out = arg(argc, argv, "out", "ref");
    char cwd[1024];
    if (getcwd(cwd, sizeof(cwd)) == NULL || chdir(dir) != 0) return 2;
    if (lb_io_read(lb, step, &event)) return 3;
    if (field_io_read(fld, step, &event)) return 3;
    if (chdir(cwd) != 0) return 2;
    double * f = malloc((size_t) ndist*NVEL*n*sizeof(double));
    double * q = malloc((size_t) nf*n*sizeof(double));
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(cs, x+1, y+1, z+1);
	for (int d = 0; d < ndist; d++) for (int p = 0; p < NVEL; p++)
	  f[canon(d*NVEL + p, x, y, z)]
	    = lb->f[LB_ADDR(lb->nsite, ndist, NVEL, index, d, p)];
	for (int c = 0; c < nf; c++)
	  q[canon(c,x,y,z)] = fld->data[addr_rank1(fld->nsites, nf, index, c)];
      }
    writef(out, "f", f, (size_t) ndist*NVEL*n);
    writef(out, "phi", q, (size_t) nf*n);
  }
  MPI_Finalize();
  return 0;
}

int main(int argc, char ** argv) {

  const char * mode = arg(argc, argv, "mode", "run");
  const char * in   = arg(argc, argv, "in", NULL);
  const char * out  = arg(argc, argv, "out", "ref");
  sys_t s;

  MPI_Init(&argc, &argv);

  if (sscanf(arg(argc, argv, "size", "8,8,8"), "%d,%d,%d",
	     L, L+1, L+2) != 3) return 2;

  if (strncmp(mode, "lc", 2) == 0) return lc_main(argc, argv, mode);
  if (strncmp(mode, "io_", 3) == 0) return io_main(argc, argv, mode);

  sys_create(argc, argv, &s);

  if (strcmp(mode, "run") == 0) {
    int seed = atoi(arg(argc, argv, "seed", "13"));
    double amp = argd(argc, argv, "noise", 0.02);
    double phi0 = argd(argc, argv, "phi0", 0.0);
    int steps = atoi(arg(argc, argv, "steps", "1"));
    field_phi_init_spinodal(s.phi, seed, phi0, amp);
    if (atoi(arg(argc, argv, "dump0", "0"))) {
      char p0[1024];
      snprintf(p0, sizeof(p0), "%s0", out);
      sys_dump(&s, p0);
    }
    for (int n = 0; n < steps; n++) sys_step(&s);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "lb2") == 0) {
    /* symmetric_lb: spinodal phi moved into g (src/phi_lb_coupler.c:107),
     * then the main loop with ndist = 2 */
    int seed = atoi(arg(argc, argv, "seed", "13"));
    double amp = argd(argc, argv, "noise", 0.02);
    double phi0 = argd(argc, argv, "phi0", 0.0);
    int steps = atoi(arg(argc, argv, "steps", "1"));
    if (s.lb->ndist != 2) { fprintf(stderr, "lb2 needs ndist=2\n"); return 2; }
    field_phi_init_spinodal(s.phi, seed, phi0, amp);
    phi_lb_from_field(s.phi, s.lb);
    for (int n = 0; n < steps; n++) sys_step_lb2(&s);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "collide2") == 0) {
    /* one binary collision (lb_collision_binary) on given f, g, phi
     * (gradients from phi) */
    size_t n = nint();
    double * f = readf(in, "f", NVEL*n);
    double * g = readf(in, "g", NVEL*n);
    double * phi = readf(in, "phi", n);
    if (s.lb->ndist != 2) { fprintf(stderr, "collide2 needs ndist=2\n");
      return 2; }
    lb_put_dist(s.cs, s.lb, 0, f);
    lb_put_dist(s.cs, s.lb, 1, g);
    field_put(s.cs, s.phi, phi);
    field_halo(s.phi);
    field_grad_compute(s.dphi);
    lb_collide(s.lb, s.hydro, s.map, NULL, (fe_t *) s.fe, NULL);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "step") == 0) {
    size_t n = nint();
    double * phi = readf(in, "phi", n);
    double * u   = readf(in, "u", 3*n);
    double * f   = readf(in, "f", NVEL*n);
    int steps = atoi(arg(argc, argv, "steps", "1"));
    field_put(s.cs, s.phi, phi);
    field_put(s.cs, s.hydro->u, u);
    lb_put(s.cs, s.lb, f);
    for (int k = 0; k < steps; k++) sys_step(&s);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "collide") == 0) {
    size_t n = nint();
    double * f = readf(in, "f", NVEL*n);
    double * force = readf(in, "force", 3*n);
    lb_put(s.cs, s.lb, f);
    field_put(s.cs, s.hydro->force, force);
    lb_collide(s.lb, s.hydro, s.map, NULL, (fe_t *) s.fe, NULL);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "propagate") == 0) {
    size_t n = nint();
    double * f = readf(in, "f", NVEL*n);
    lb_put(s.cs, s.lb, f);
    lb_halo(s.lb);
    lb_propagation(s.lb);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "grad27") == 0) {
    /* field_grad_compute with grad_3d_27pt_fluid_d2 */
    int nf = atoi(arg(argc, argv, "nf", "1"));
    size_t n = nint();
    field_t * fld = NULL;
    field_grad_t * fg = NULL;
    field_options_t opts = field_options_ndata_nhalo(nf, 2);
    field_create(s.pe, s.cs, s.le, "f27", &opts, &fld);
    field_grad_create(s.pe, fld, 2, &fg);
    field_grad_set(fg, grad_3d_27pt_fluid_d2, NULL);
    double * a = readf(in, "phi", nf*n);
    field_put(s.cs, fld, a);
    field_halo(fld);
    field_grad_compute(fg);
    double * g = malloc(3*nf*n*sizeof(double));
    double * dl = malloc(nf*n*sizeof(double));
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(s.cs, x+1, y+1, z+1);
	for (int k = 0; k < nf; k++) {
	  for (int ia = 0; ia < 3; ia++) {
	    g[canon(3*k + ia, x, y, z)] =
	      fg->grad[addr_rank2(fg->nsite, nf, 3, index, k, ia)];
	  }
	  dl[canon(k, x, y, z)] = fg->delsq[addr_rank1(fg->nsite, nf, index, k)];
	}
      }
    writef(out, "grad", g, 3*nf*n);
    writef(out, "delsq", dl, nf*n);
  }
  else if (strcmp(mode, "grad") == 0) {
    size_t n = nint();
    double * phi = readf(in, "phi", n);
    double * g = malloc(3*n*sizeof(double));
    double * d = malloc(n*sizeof(double));
    field_put(s.cs, s.phi, phi);
    field_halo(s.phi);
    field_grad_compute(s.dphi);
    for (int x = 0; x < L[0]; x++) for (int y = 0; y < L[1]; y++)
      for (int z = 0; z < L[2]; z++) {
	int index = cs_index(s.cs, x+1, y+1, z+1);
	for (int ia = 0; ia < 3; ia++)
	  g[canon(ia,x,y,z)] = s.dphi->grad[addr_rank2(s.dphi->nsite, 1, 3,
						       index, 0, ia)];
	d[canon(0,x,y,z)] = s.dphi->delsq[addr_rank1(s.dphi->nsite, 1,
						    index, 0)];
      }
    writef(out, "grad", g, 3*n);
    writef(out, "delsq", d, n);
  }
  else if (strcmp(mode, "force") == 0) {
    size_t n = nint();
    double zero[3] = {0.0, 0.0, 0.0};
    double * phi = readf(in, "phi", n);
    field_put(s.cs, s.phi, phi);
    hydro_f_zero(s.hydro, zero);
    field_halo(s.phi);
    field_grad_compute(s.dphi);
    phi_force_calculation(s.pe, s.cs, s.le, s.wall, s.pth, (fe_t *) s.fe,
			  s.map, s.phi, s.hydro);
    sys_dump(&s, out);
  }
  else if (strcmp(mode, "ch") == 0) {
    size_t n = nint();
    double * phi = readf(in, "phi", n);
    double * u   = readf(in, "u", 3*n);
    field_put(s.cs, s.phi, phi);
    field_put(s.cs, s.hydro->u, u);
    field_halo(s.phi);
    field_grad_compute(s.dphi);
    phi_cahn_hilliard(s.pch, (fe_t *) s.fe, s.phi, s.hydro, s.map, NULL);
    sys_dump(&s, out);
  }
  else {
    fprintf(stderr, "unknown mode %s\n", mode);
    return 2;
  }

  MPI_Finalize();
  return 0;
}
