/*****************************************************************************
 *
 *  ludwig_loop.c  (test program)
 *
 *  A C host that drives libludwig_gb.so through include/ludwig_gb.h the
 *  way the reference's main loop (src/ludwig.c:528-860) drives its own
 *  functions: objects built from the reference's option structures, one
 *  call per reference function per step, and free-energy values read
 *  through the function table fe->func with cs_index() site numbers, as
 *  src/stats_free_energy.c:60-90 does.  It writes what it computed as raw
 *  doubles, <prefix>_<name>.bin, for tests/test_c_host_gpu.py to compare
 *  with the fixtures the reference made.
 *
 *    ludwig_loop binary   <prefix>            8x6x4, spinodal seed 8361235,
 *                                             10 steps
 *    ludwig_loop lc       <prefix> <q0 file>  8x8x8 blue phase I from q0
 *                                             (reference AOS host layout,
 *                                             nhalo 2), 3 steps
 *    ludwig_loop lc_sites <prefix> <q file>   6x5x4: fed, stress,
 *                                             str_symm, str_anti, htensor
 *                                             and the _v slots at every
 *                                             site through fe->func
 *
 *  Exit status 0 on success; a failing call prints ludwig_gb_last_error().
 *
 *****************************************************************************/

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ludwig_gb.h"

/* The layout facts the drop-in depends on, for an LP64 target: the same
 * numbers as the reference's src/free_energy.h gives */
_Static_assert(offsetof(struct fe_s, func) == 0, "fe_s.func first");
_Static_assert(offsetof(struct fe_s, id) == sizeof(void *), "fe_s.id");
_Static_assert(offsetof(fe_vt_t, stress) == 5*sizeof(void *), "stress slot");
_Static_assert(offsetof(fe_vt_t, htensor) == 9*sizeof(void *), "htensor");
_Static_assert(offsetof(fe_vt_t, str_anti_v) == 13*sizeof(void *), "last");
_Static_assert(sizeof(fe_vt_t) == 14*sizeof(void *), "14 slots");
_Static_assert(FE_LC == 5 && FE_SYMMETRIC == 1, "fe_id_enum values");
_Static_assert(NSIMDVL == 1, "vector length of the _v slots");

#define CHECK(call) do {						\
    int rc_ = (call);							\
    if (rc_ != 0) {							\
      fprintf(stderr, "%s:%d: %s returned %d: %s\n", __FILE__, __LINE__, \
	      #call, rc_, ludwig_gb_last_error());			\
      exit(1);								\
    }									\
  } while (0)

static const char * prefix_ = NULL;

static void write_array(const char * name, const double * a, size_t n) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_%s.bin", prefix_, name);
  FILE * fp = fopen(path, "wb");
  if (fp == NULL || fwrite(a, sizeof(double), n, fp) != n) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(1);
  }
  fclose(fp);
}

static double * read_array(const char * path, size_t n) {
  double * a = (double *) malloc(n*sizeof(double));
  FILE * fp = fopen(path, "rb");
  if (a == NULL || fp == NULL || fread(a, sizeof(double), n, fp) != n) {
    fprintf(stderr, "cannot read %s\n", path);
    exit(1);
  }
  fclose(fp);
  return a;
}

static double * alloc(size_t n) {
  double * a = (double *) calloc(n, sizeof(double));
  if (a == NULL) exit(2);
  return a;
}

static cs_t * lattice(pe_t * pe, int nx, int ny, int nz) {
  cs_t * cs = NULL;
  const int ntotal[3] = {nx, ny, nz};
  CHECK(cs_create(pe, &cs));
  CHECK(cs_ntotal_set(cs, ntotal));
  CHECK(cs_nhalo_set(cs, 2));
  CHECK(cs_init(cs));
  return cs;
}

/* The state of the step, interior layout */
static void write_state(cs_t * cs, lb_t * lb, hydro_t * hydro) {
  int n[3];
  CHECK(cs_nlocal(cs, n));
  size_t N = (size_t) n[0]*n[1]*n[2];
  double * f = alloc(19*N), * rho = alloc(N), * u = alloc(3*N);
  double * force = alloc(3*N);
  CHECK(lb_f_to_host(lb, f));
  CHECK(hydro_to_host(hydro, rho, u, force));
  write_array("f", f, 19*N);
  write_array("rho", rho, N);
  write_array("u", u, 3*N);
  write_array("force", force, 3*N);
  free(f); free(rho); free(u); free(force);
}

/*****************************************************************************
 *  Symmetric binary fluid: 8x6x4, config 1's parameters, 10 steps
 *****************************************************************************/

static int run_binary(void) {
  pe_t * pe = NULL;
  physics_t * phys = NULL;
  lb_t * lb = NULL;
  field_t * phi = NULL;
  field_grad_t * dphi = NULL;
  hydro_t * hydro = NULL;
  map_t * map = NULL;
  fe_symm_t * fe = NULL;
  pth_t * pth = NULL;
  phi_ch_t * pch = NULL;
  const double zero[3] = {0.0, 0.0, 0.0};

  CHECK(pe_create(0, &pe));
  cs_t * cs = lattice(pe, 8, 6, 4);
  CHECK(physics_create(pe, &phys));
  CHECK(physics_eta_shear_set(phys, 0.1));
  CHECK(physics_eta_bulk_set(phys, 0.1));
  CHECK(physics_mobility_set(phys, 0.3));

  lb_data_options_t lbo = lb_data_options_default();
  CHECK(lb_data_create(pe, cs, &lbo, &lb));
  CHECK(lb_init_rest_f(lb, 1.0));
  field_options_t fo = field_options_ndata_nhalo(1, 2);
  CHECK(field_create(pe, cs, NULL, "phi", &fo, &phi));
  CHECK(field_grad_create(pe, phi, 2, &dphi));
  hydro_options_t ho = hydro_options_default();
  CHECK(hydro_create(pe, cs, NULL, &ho, &hydro));
  map_options_t mo = map_options_default();
  CHECK(map_create(pe, cs, &mo, &map));
  CHECK(fe_symm_create(pe, cs, phi, dphi, &fe));
  fe_symm_param_t fp = {-0.0625, 0.0625, 0.04, 0.0, 0.0};
  CHECK(fe_symm_param_set(fe, fp));
  CHECK(pth_create(pe, cs, FE_FORCE_METHOD_STRESS_DIVERGENCE, &pth));
  phi_ch_info_t info = {0, 0};
  CHECK(phi_ch_create(pe, cs, NULL, &info, &pch));
  CHECK(field_phi_init_spinodal(phi, 8361235, 0.0, 0.02));

  fe_t * base = (fe_t *) fe;
  if (base->id != FE_SYMMETRIC || base->func->fed == NULL ||
      base->func->htensor != NULL) {
    fprintf(stderr, "symmetric function table\n");
    return 1;
  }

  for (int step = 1; step <= 10; step++) {
    CHECK(hydro_f_zero(hydro, zero));
    CHECK(field_halo(phi));
    CHECK(field_grad_compute(dphi));
    CHECK(phi_force_calculation(pe, cs, NULL, NULL, pth, base, map, phi,
				hydro));
    CHECK(hydro_u_halo(hydro));
    CHECK(phi_cahn_hilliard(pch, base, phi, hydro, map, NULL));
    CHECK(hydro_u_zero(hydro, zero));
    CHECK(lb_collide(lb, hydro, map, NULL, base, NULL));
    CHECK(lb_halo(lb));
    CHECK(lb_propagation(lb));
  }

  int n[3], nsites = 0, nhalo = 0;
  CHECK(cs_nlocal(cs, n));
  CHECK(cs_nsites(cs, &nsites));
  CHECK(cs_nhalo(cs, &nhalo));
  size_t N = (size_t) n[0]*n[1]*n[2];
  double * phih = alloc(N);
  CHECK(field_to_host(phi, phih));
  write_array("phi", phih, N);
  write_state(cs, lb, hydro);

  /* The reference's host layout: phi (AOS) and f (SOA) at every
   * cs_index() site */
  double * phics = alloc((size_t) nsites);
  double * fcs = alloc(19*(size_t) nsites);
  CHECK(ludwig_gb_field_to_host_cs(phi, DATA_MODEL_AOS, phics));
  CHECK(ludwig_gb_lb_to_host_cs(lb, DATA_MODEL_SOA, fcs));
  write_array("phi_cs_aos", phics, (size_t) nsites);
  write_array("f_cs_soa", fcs, 19*(size_t) nsites);

  /* Free energy through the function table at cs_index() sites, as
   * src/stats_free_energy.c:60-90, against the device total; and the
   * per-site mu and stress at every site with its halo */
  CHECK(field_grad_compute(dphi));
  double fsum = 0.0, total = 0.0;
  double * mu = alloc((size_t) nsites), * fed = alloc((size_t) nsites);
  double * str = alloc(9*(size_t) nsites), * strv = alloc(9*(size_t) nsites);
  for (int ic = 1 - nhalo; ic <= n[0] + nhalo; ic++) {
    for (int jc = 1 - nhalo; jc <= n[1] + nhalo; jc++) {
      for (int kc = 1 - nhalo; kc <= n[2] + nhalo; kc++) {
	int index = cs_index(cs, ic, jc, kc);
	double s[3][3], sv[3][3][NSIMDVL];
	CHECK(base->func->fed(base, index, fed + index));
	CHECK(base->func->mu(base, index, mu + index));
	CHECK(base->func->stress(base, index, s));
	base->func->stress_v(base, index, sv);
	for (int a = 0; a < 3; a++) {
	  for (int b = 0; b < 3; b++) {
	    str[9*(size_t) index + 3*a + b] = s[a][b];
	    strv[9*(size_t) index + 3*a + b] = sv[a][b][0];
	  }
	}
	if (ic >= 1 && ic <= n[0] && jc >= 1 && jc <= n[1] && kc >= 1 &&
	    kc <= n[2]) fsum += fed[index];
      }
    }
  }
  CHECK(stats_free_energy_symm(fe, &total));
  double pair[2] = {fsum, total};
  write_array("fed_total", pair, 2);
  write_array("fed_cs", fed, (size_t) nsites);
  write_array("mu_cs", mu, (size_t) nsites);
  write_array("stress_cs", str, 9*(size_t) nsites);
  write_array("stress_v_cs", strv, 9*(size_t) nsites);
  double * dg = alloc(3*N), * dd = alloc(N);
  CHECK(field_grad_to_host(dphi, dg, dd));
  write_array("grad", dg, 3*N);
  write_array("delsq", dd, N);

  free(phih); free(phics); free(fcs); free(mu); free(fed); free(str);
  free(strv); free(dg); free(dd);
  CHECK(phi_ch_free(pch));
  CHECK(pth_free(pth));
  CHECK(fe_symm_free(fe));
  CHECK(map_free(&map));
  if (map != NULL) return 1;
  CHECK(hydro_free(hydro));
  field_grad_free(dphi);
  CHECK(field_free(phi));
  CHECK(lb_free(lb));
  CHECK(physics_free(phys));
  CHECK(cs_free(cs));
  CHECK(pe_free(pe));
  return 0;
}

/*****************************************************************************
 *  Cholesteric liquid crystal
 *****************************************************************************/

typedef struct lc_sys_s {
  pe_t * pe;
  cs_t * cs;
  physics_t * phys;
  lb_t * lb;
  field_t * q;
  field_grad_t * dq;
  hydro_t * hydro;
  map_t * map;
  fe_lc_t * fe;
  beris_edw_t * be;
  pth_t * pth;
} lc_sys_t;

static void lc_create(lc_sys_t * s, int nx, int ny, int nz,
		      const char * qfile) {
  memset(s, 0, sizeof(*s));
  CHECK(pe_create(0, &s->pe));
  s->cs = lattice(s->pe, nx, ny, nz);
  CHECK(physics_create(s->pe, &s->phys));
  CHECK(physics_eta_shear_set(s->phys, 0.5));
  CHECK(physics_eta_bulk_set(s->phys, 0.5));
  lb_data_options_t lbo = lb_data_options_default();
  CHECK(lb_data_create(s->pe, s->cs, &lbo, &s->lb));
  CHECK(lb_init_rest_f(s->lb, 1.0));
  field_options_t fo = field_options_ndata_nhalo(5, 2);
  CHECK(field_create(s->pe, s->cs, NULL, "q", &fo, &s->q));
  CHECK(field_grad_create(s->pe, s->q, 2, &s->dq));
  hydro_options_t ho = hydro_options_default();
  CHECK(hydro_create(s->pe, s->cs, NULL, &ho, &s->hydro));
  map_options_t mo = map_options_default();
  CHECK(map_create(s->pe, s->cs, &mo, &s->map));
  CHECK(fe_lc_create(s->pe, s->cs, NULL, s->q, s->dq, &s->fe));
  fe_lc_param_t p;
  memset(&p, 0, sizeof(p));
  p.a0 = 0.01; p.gamma = 3.0; p.kappa0 = 0.01; p.kappa1 = 0.01;
  p.q0 = 2.0*(4.0*atan(1.0))/32.0;
  p.xi = 0.7; p.redshift = 1.0; p.amplitude0 = -0.2; p.coswt = 1.0;
  CHECK(fe_lc_param_set(s->fe, &p));
  CHECK(beris_edw_create(s->pe, s->cs, NULL, &s->be));
  beris_edw_param_t bp;
  memset(&bp, 0, sizeof(bp));
  bp.xi = 0.7; bp.gamma = 0.5;
  CHECK(beris_edw_param_set(s->be, &bp));
  CHECK(pth_create(s->pe, s->cs, FE_FORCE_METHOD_STRESS_DIVERGENCE, &s->pth));

  /* Q in the reference's AOS host layout, all cs_index() sites */
  int nsites = 0;
  CHECK(cs_nsites(s->cs, &nsites));
  double * q = read_array(qfile, 5*(size_t) nsites);
  CHECK(ludwig_gb_field_from_host_cs(s->q, DATA_MODEL_AOS, q));
  free(q);
}

static void lc_destroy(lc_sys_t * s) {
  CHECK(pth_free(s->pth));
  CHECK(beris_edw_free(s->be));
  CHECK(fe_lc_free(s->fe));
  CHECK(map_free(&s->map));
  CHECK(hydro_free(s->hydro));
  field_grad_free(s->dq);
  CHECK(field_free(s->q));
  CHECK(lb_free(s->lb));
  CHECK(physics_free(s->phys));
  CHECK(cs_free(s->cs));
  CHECK(pe_free(s->pe));
}

static int run_lc(const char * qfile) {
  lc_sys_t s;
  const double zero[3] = {0.0, 0.0, 0.0};
  lc_create(&s, 8, 8, 8, qfile);
  fe_t * base = (fe_t *) s.fe;
  if (base->id != FE_LC || base->func->htensor == NULL ||
      base->func->mu != NULL) {
    fprintf(stderr, "LC function table\n");
    return 1;
  }
  for (int step = 1; step <= 3; step++) {
    CHECK(hydro_f_zero(s.hydro, zero));
    CHECK(field_halo(s.q));
    CHECK(field_grad_compute(s.dq));
    CHECK(phi_force_calculation(s.pe, s.cs, NULL, NULL, s.pth, base, s.map,
				s.q, s.hydro));
    CHECK(hydro_u_halo(s.hydro));
    CHECK(beris_edw_update(s.be, base, s.q, s.dq, s.hydro, NULL, s.map,
			   NULL));
    CHECK(hydro_u_zero(s.hydro, zero));
    CHECK(lb_collide(s.lb, s.hydro, s.map, NULL, base, NULL));
    CHECK(lb_halo(s.lb));
    CHECK(lb_propagation(s.lb));
  }
  size_t N = 8*8*8;
  double * q = alloc(5*N);
  CHECK(field_to_host(s.q, q));
  write_array("q", q, 5*N);
  write_state(s.cs, s.lb, s.hydro);
  free(q);
  lc_destroy(&s);
  return 0;
}

static int run_lc_sites(const char * qfile) {
  lc_sys_t s;
  lc_create(&s, 6, 5, 4, qfile);
  fe_t * base = (fe_t *) s.fe;
  int n[3], nsites = 0;
  CHECK(cs_nlocal(s.cs, n));
  CHECK(cs_nsites(s.cs, &nsites));
  CHECK(field_grad_compute(s.dq));
  size_t N = (size_t) n[0]*n[1]*n[2];
  double * fed = alloc(N), * h = alloc(9*N), * hv = alloc(9*N);
  double * st = alloc(9*N), * sy = alloc(9*N), * an = alloc(9*N);
  double * stv = alloc(9*N), * syv = alloc(9*N), * anv = alloc(9*N);
  /* interior sites in x, y, z order, through cs_index() */
  size_t k = 0;
  for (int ic = 1; ic <= n[0]; ic++) {
    for (int jc = 1; jc <= n[1]; jc++) {
      for (int kc = 1; kc <= n[2]; kc++, k++) {
	int index = cs_index(s.cs, ic, jc, kc);
	double a[3][3], b[3][3], c[3][3], d[3][3];
	double av[3][3][NSIMDVL], bv[3][3][NSIMDVL], cv[3][3][NSIMDVL];
	double dv[3][3][NSIMDVL];
	CHECK(base->func->fed(base, index, fed + k));
	CHECK(base->func->stress(base, index, a));
	CHECK(base->func->str_symm(base, index, b));
	CHECK(base->func->str_anti(base, index, c));
	CHECK(base->func->htensor(base, index, d));
	base->func->stress_v(base, index, av);
	base->func->str_symm_v(base, index, bv);
	base->func->str_anti_v(base, index, cv);
	base->func->htensor_v(base, index, dv);
	for (int i = 0; i < 3; i++) {
	  for (int j = 0; j < 3; j++) {
	    st[9*k + 3*i + j] = a[i][j];
	    sy[9*k + 3*i + j] = b[i][j];
	    an[9*k + 3*i + j] = c[i][j];
	    h[9*k + 3*i + j] = d[i][j];
	    stv[9*k + 3*i + j] = av[i][j][0];
	    syv[9*k + 3*i + j] = bv[i][j][0];
	    anv[9*k + 3*i + j] = cv[i][j][0];
	    hv[9*k + 3*i + j] = dv[i][j][0];
	  }
	}
      }
    }
  }
  write_array("fed", fed, N);
  write_array("stress", st, 9*N);
  write_array("str_symm", sy, 9*N);
  write_array("str_anti", an, 9*N);
  write_array("htensor", h, 9*N);
  write_array("stress_v", stv, 9*N);
  write_array("str_symm_v", syv, 9*N);
  write_array("str_anti_v", anv, 9*N);
  write_array("htensor_v", hv, 9*N);
  free(fed); free(h); free(hv); free(st); free(sy); free(an); free(stv);
  free(syv); free(anv);
  lc_destroy(&s);
  return 0;
}

int main(int argc, char ** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s binary|lc|lc_sites <prefix> [q file]\n",
	    argv[0]);
    return 2;
  }
  prefix_ = argv[2];
  if (strcmp(argv[1], "binary") == 0) return run_binary();
  if (strcmp(argv[1], "lc") == 0 && argc > 3) return run_lc(argv[3]);
  if (strcmp(argv[1], "lc_sites") == 0 && argc > 3) {
    return run_lc_sites(argv[3]);
  }
  fprintf(stderr, "unknown mode %s\n", argv[1]);
  return 2;
}
