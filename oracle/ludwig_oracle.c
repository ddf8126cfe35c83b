/*****************************************************************************
 *
 *  ludwig_oracle.c
 *
 *  TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 *  A CPU restatement, in plain C with OpenMP, of the reference's
 *  lattice-Boltzmann time step for the symmetric binary fluid
 *  (Ludwig v0.23).  Each function cites the reference code it follows and
 *  keeps that code's floating-point operation order, so that results agree
 *  bit for bit with the reference's own serial build when both are
 *  compiled without multiply-add contraction (-ffp-contract=off).
 *
 *  The reference stores fields with a halo of width 2 that is refreshed by
 *  a periodic halo swap before each stencil.  With one domain, every halo
 *  value is the periodic image of an interior value, and every quantity
 *  the reference computes "on the interior plus one halo layer" equals the
 *  value at that image site.  The restatement therefore works on the
 *  interior only and wraps indices periodically, which gives identical
 *  numbers on the interior.
 *
 *****************************************************************************/

#include <assert.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ludwig_oracle.h"

#define NVEL ORC_NVEL

/*****************************************************************************
 *
 *  Model tables.
 *
 *  Velocity set and weights: src/lb_d3q19.h:26-38.
 *  Mode matrix ma (rho, j, S_ab, chi1, jchi1, chi2, jchi2, chi3):
 *  src/lb_d3q19.c:107-153.  Inverse mi_pm = w_p na_m ma_mp with
 *  na_m = 1 / sum_p w_p ma_mp^2: src/lb_d3q19.c:75-82, src/lb_model.c.
 *  The reference's unrolled transforms (src/collision.c:1990-2850) hold the
 *  same rational entries rounded once to double; here they are derived
 *  exactly in integer arithmetic and rounded once.
 *
 *****************************************************************************/

static const int8_t cv_[NVEL][3] = {
  { 0,  0,  0},
  { 1,  1,  0}, { 1,  0,  1}, { 1,  0,  0},
  { 1,  0, -1}, { 1, -1,  0}, { 0,  1,  1},
  { 0,  1,  0}, { 0,  1, -1}, { 0,  0,  1},
  { 0,  0, -1}, { 0, -1,  1}, { 0, -1,  0},
  { 0, -1, -1}, {-1,  1,  0}, {-1,  0,  1},
  {-1,  0,  0}, {-1,  0, -1}, {-1, -1,  0}};

/* weights as numerator over 36 */
static const int w36_[NVEL] = {12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1,
			       1, 2, 1, 1};

static double wv_[NVEL];
static double ma_[NVEL][NVEL];
static double mi_[NVEL][NVEL];
static int tables_ready_ = 0;

typedef struct { long long n; long long d; } rat_t;

static long long gcdll(long long a, long long b) {
  if (a < 0) a = -a;
  if (b < 0) b = -b;
  while (b) { long long t = a % b; a = b; b = t; }
  return a ? a : 1;
}

static rat_t rat(long long n, long long d) {
  long long g = gcdll(n, d);
  rat_t r = {n/g, d/g};
  if (r.d < 0) { r.n = -r.n; r.d = -r.d; }
  return r;
}
static rat_t rmul(rat_t a, rat_t b) { return rat(a.n*b.n, a.d*b.d); }
static rat_t radd(rat_t a, rat_t b) { return rat(a.n*b.d + b.n*a.d, a.d*b.d); }
static double rdbl(rat_t a) { return (double) a.n / (double) a.d; }

/* Mode m of velocity p as an exact rational (src/lb_d3q19.c:121-151) */

static rat_t mode_entry(int m, int p) {
  long long cx = cv_[p][0], cy = cv_[p][1], cz = cv_[p][2];
  long long c2 = cx*cx + cy*cy + cz*cz;
  long long chi1 = (2*c2 - 3)*(3*cz*cz - c2);
  long long chi2 = (2*c2 - 3)*(cy*cy - cx*cx);
  long long chi3 = 3*c2*c2 - 6*c2 + 1;
  switch (m) {
  case  0: return rat(1, 1);
  case  1: return rat(cx, 1);
  case  2: return rat(cy, 1);
  case  3: return rat(cz, 1);
  case  4: return rat(3*cx*cx - 1, 3);
  case  5: return rat(cx*cy, 1);
  case  6: return rat(cx*cz, 1);
  case  7: return rat(3*cy*cy - 1, 3);
  case  8: return rat(cy*cz, 1);
  case  9: return rat(3*cz*cz - 1, 3);
  case 10: return rat(chi1, 1);
  case 11: return rat(chi1*cx, 1);
  case 12: return rat(chi1*cy, 1);
  case 13: return rat(chi1*cz, 1);
  case 14: return rat(chi2, 1);
  case 15: return rat(chi2*cx, 1);
  case 16: return rat(chi2*cy, 1);
  case 17: return rat(chi2*cz, 1);
  default: return rat(chi3, 1);
  }
}

static void tables_init(void) {

  if (tables_ready_) return;

  for (int p = 0; p < NVEL; p++) wv_[p] = (double) w36_[p] / 36.0;

  for (int m = 0; m < NVEL; m++) {
    rat_t norm = rat(0, 1);
    for (int p = 0; p < NVEL; p++) {
      rat_t e = mode_entry(m, p);
      ma_[m][p] = rdbl(e);
      norm = radd(norm, rmul(rat(w36_[p], 36), rmul(e, e)));
    }
    {
      rat_t na = rat(norm.d, norm.n);
      for (int p = 0; p < NVEL; p++) {
	rat_t e = rmul(rmul(rat(w36_[p], 36), na), mode_entry(m, p));
	mi_[p][m] = rdbl(e);
      }
    }
  }
  tables_ready_ = 1;
}

const int8_t * orc_cv(void) { return &cv_[0][0]; }
const double * orc_wv(void) { tables_init(); return wv_; }
const double * orc_ma(void) { tables_init(); return &ma_[0][0]; }
const double * orc_mi(void) { tables_init(); return &mi_[0][0]; }

/*****************************************************************************
 *
 *  Indexing helpers (periodic wrap of the interior).
 *
 *****************************************************************************/

static inline int wrap(int i, int n) {
  i %= n;
  return (i < 0) ? i + n : i;
}

static inline size_t site(const int L[3], int x, int y, int z) {
  return ((size_t) wrap(x, L[0])*L[1] + wrap(y, L[1]))*L[2] + wrap(z, L[2]);
}

static inline size_t nsites(const int L[3]) {
  return (size_t) L[0]*L[1]*L[2];
}

/*****************************************************************************
 *
 *  orc_collide_param_m10
 *
 *  src/collision.c:1163-1200 (relaxation times, M10 scheme) with
 *  cs2 = 1/3; ghost modes relax with rtau = 1.
 *
 *****************************************************************************/

void orc_collide_param_m10(double eta_shear, double eta_bulk, double rho0,
			   orc_collide_param_t * p) {
  const double cs2 = (1.0/3.0);
  memset(p, 0, sizeof(*p));
  p->rtau_shear = 1.0/(0.5 + eta_shear / (rho0*cs2));
  p->rtau_bulk  = 1.0/(0.5 + eta_bulk / (rho0*cs2));
  for (int m = 0; m < NVEL; m++) p->rtau_ghost[m] = 1.0;
}

/*****************************************************************************
 *
 *  KISS99-type generator: src/noise.h:96-112 (ns_uniform), per-site seeding
 *  src/noise.c:278-340, reap src/noise.c:437-454; spinodal initial
 *  condition src/field_phi_init.c:484-518.
 *
 *****************************************************************************/

static inline unsigned int kiss_next(unsigned int s[4]) {
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

/* One draw of the generator (ns_uniform, src/noise.h:96-112) on state s */
unsigned int orc_kiss_next(unsigned int s[4]) { return kiss_next(s); }

void orc_spinodal_init(const int L[3], int seed, double phi0, double amp,
		       double * phi) {

  unsigned int seed0 = (seed > 1) ? (unsigned int) seed : 13u;

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	unsigned int sl[4], st[4];
	sl[0] = seed0 + (unsigned int) (x + 1);
	sl[1] = 12953u + (unsigned int) (y + 1);
	sl[2] = 712357u + (unsigned int) (z + 1);
	sl[3] = 22383979u;
	st[0] = kiss_next(sl);
	st[1] = kiss_next(sl);
	st[2] = kiss_next(sl);
	st[3] = kiss_next(sl);
	{
	  unsigned int iu = kiss_next(st);
	  double ran = (1.0/UINT_MAX)*iu;
	  phi[site(L, x, y, z)] = phi0 + amp*(ran - 0.5);
	}
      }
    }
  }
}

/* src/lb_data.c:659-680, 809-834 with u = 0: f_p = rho0 w_p */

void orc_lb_init_rest(const int L[3], double rho0, double * f) {
  size_t n = nsites(L);
  tables_init();
  for (int p = 0; p < NVEL; p++) {
    double fp = rho0*wv_[p]*1.0;
    for (size_t i = 0; i < n; i++) f[p*n + i] = fp;
  }
}

/*****************************************************************************
 *
 *  orc_grad_7pt
 *
 *  src/gradient_3d_7pt_fluid.c:231-306: centred first differences and the
 *  7-point Laplacian (sum of six neighbours in x+, x-, y+, y-, z+, z-
 *  order, minus 6 phi).  grad[(n*3 + ia)*N + i], delsq[n*N + i].
 *
 *****************************************************************************/

void orc_grad_7pt(const int L[3], int nf, const double * field,
		  double * grad, double * delsq) {
  size_t N = nsites(L);

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	size_t xp = site(L, x+1, y, z), xm = site(L, x-1, y, z);
	size_t yp = site(L, x, y+1, z), ym = site(L, x, y-1, z);
	size_t zp = site(L, x, y, z+1), zm = site(L, x, y, z-1);
	for (int n = 0; n < nf; n++) {
	  const double * fn = field + n*N;
	  grad[(3*n + 0)*N + i] = 0.5*(fn[xp] - fn[xm]);
	  grad[(3*n + 1)*N + i] = 0.5*(fn[yp] - fn[ym]);
	  grad[(3*n + 2)*N + i] = 0.5*(fn[zp] - fn[zm]);
	  delsq[n*N + i] = fn[xp] + fn[xm] + fn[yp] + fn[ym] + fn[zp] + fn[zm]
	    - 6.0*fn[i];
	}
      }
    }
  }
}

/*****************************************************************************
 *
 *  Symmetric free energy, src/symmetric.c:285-400.
 *
 *  mu   = A phi + B phi^3 - kappa delsq                       (:308-320)
 *  P_ab = p0 delta_ab + kappa d_a phi d_b phi                 (:372-400)
 *  p0   = 1/2 A phi^2 + 3/4 B phi^4 - kappa phi delsq - 1/2 kappa |grad|^2
 *
 *****************************************************************************/

/*****************************************************************************
 *
 *  orc_grad_27pt
 *
 *  src/gradient_3d_27pt_fluid.c:219-362 (grad_3d_27pt_kernel, del^2):
 *  each gradient component is (0.5/9) times the sum over the nine
 *  neighbour pairs of the +1 and -1 planes, in the reference's order, and
 *  del^2 is (1/9)(sum of the 26 neighbours - 26 phi).
 *
 *****************************************************************************/

void orc_grad_27pt(const int L[3], int nf, const double * field,
		   double * grad, double * delsq) {
  size_t N = nsites(L);
  const double r9 = (1.0/9.0);
  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	for (int n = 0; n < nf; n++) {
	  const double * fn = field + (size_t) n*N;
#define F(dx, dy, dz) fn[site(L, x + (dx), y + (dy), z + (dz))]
	  double sx = 0.0, sy = 0.0, sz = 0.0, sl = 0.0;
	  int first = 1;
	  for (int a = -1; a <= 1; a++) {
	    for (int b = -1; b <= 1; b++) {
	      if (first) sx = +F(1, a, b);
	      else sx = sx + F(1, a, b);
	      sx = sx - F(-1, a, b);
	      first = 0;
	    }
	  }
	  first = 1;
	  for (int a = -1; a <= 1; a++) {
	    for (int b = -1; b <= 1; b++) {
	      if (first) sy = +F(a, 1, b);
	      else sy = sy + F(a, 1, b);
	      sy = sy - F(a, -1, b);
	      first = 0;
	    }
	  }
	  first = 1;
	  for (int a = -1; a <= 1; a++) {
	    for (int b = -1; b <= 1; b++) {
	      if (first) sz = +F(a, b, 1);
	      else sz = sz + F(a, b, 1);
	      sz = sz - F(a, b, -1);
	      first = 0;
	    }
	  }
	  first = 1;
	  for (int a = -1; a <= 1; a++) {
	    for (int b = -1; b <= 1; b++) {
	      for (int c = -1; c <= 1; c++) {
		if (a == 0 && b == 0 && c == 0) continue;
		if (first) sl = +F(a, b, c);
		else sl = sl + F(a, b, c);
		first = 0;
	      }
	    }
	  }
	  sl = sl - 26.0*F(0, 0, 0);
#undef F
	  grad[(3*n + 0)*N + i] = 0.5*r9*sx;
	  grad[(3*n + 1)*N + i] = 0.5*r9*sy;
	  grad[(3*n + 2)*N + i] = 0.5*r9*sz;
	  delsq[n*N + i] = r9*sl;
	}
      }
    }
  }
}

static inline double symm_mu_site(const orc_symm_param_t * fe, double phi,
				  double delsq) {
  return fe->a*phi + fe->b*phi*phi*phi - fe->kappa*delsq;
}

void orc_symm_mu(const int L[3], const orc_symm_param_t * fe,
		 const double * phi, const double * delsq, double * mu) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) mu[i] = symm_mu_site(fe, phi[i], delsq[i]);
}

void orc_symm_stress(const int L[3], const orc_symm_param_t * fe,
		     const double * phi, const double * grad,
		     const double * delsq, double * pth) {
  size_t N = nsites(L);
  const double a = fe->a, b = fe->b, kappa = fe->kappa;

  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double g[3] = {grad[i], grad[N + i], grad[2*N + i]};
    double ph = phi[i];
    double d = delsq[i];
    double p0 = 0.5*a*ph*ph + 0.75*b*ph*ph*ph*ph - kappa*ph*d
      - 0.5*kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
    for (int ia = 0; ia < 3; ia++) {
      for (int ib = 0; ib < 3; ib++) {
	double dab = (ia == ib);
	pth[(3*ia + ib)*N + i] = p0*dab + kappa*g[ia]*g[ib];
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_force_divergence
 *
 *  src/phi_force_colloid.c:315-467 (pth_force_fluid_kernel_v):
 *  F_a = -1/2 (P_ax(x+1) + P_ax) + 1/2 (P_ax(x-1) + P_ax)
 *        -1/2 (P_ay(y+1) + P_ay) + 1/2 (P_ay(y-1) + P_ay)
 *        -1/2 (P_az(z+1) + P_az) + 1/2 (P_az(z-1) + P_az)
 *  accumulated in that order and added to force (which the caller zeroes,
 *  as hydro_f_zero does at src/ludwig.c:535).
 *
 *****************************************************************************/

void orc_force_divergence(const int L[3], const double * pth, double * force) {
  size_t N = nsites(L);

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	size_t nb[6] = {site(L, x+1, y, z), site(L, x-1, y, z),
			site(L, x, y+1, z), site(L, x, y-1, z),
			site(L, x, y, z+1), site(L, x, y, z-1)};
	double fa[3];
	for (int ia = 0; ia < 3; ia++) {
	  const double * px = pth + (3*ia + 0)*N;
	  const double * py = pth + (3*ia + 1)*N;
	  const double * pz = pth + (3*ia + 2)*N;
	  fa[ia]  = -0.5*(px[nb[0]] + px[i]);
	  fa[ia] +=  0.5*(px[nb[1]] + px[i]);
	  fa[ia] -=  0.5*(py[nb[2]] + py[i]);
	  fa[ia] +=  0.5*(py[nb[3]] + py[i]);
	  fa[ia] -=  0.5*(pz[nb[4]] + pz[i]);
	  fa[ia] +=  0.5*(pz[nb[5]] + pz[i]);
	}
	for (int ia = 0; ia < 3; ia++) force[ia*N + i] += fa[ia]*1;
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_advect_upwind
 *
 *  First-order upwind face fluxes, src/advection.c:538-629:
 *  fw (x-1/2): u = 1/2 (u_x(x) + u_x(x-1)); upwind x-1 if u > 0
 *  fe (x+1/2): u = 1/2 (u_x(x) + u_x(x+1)); upwind x+1 if u < 0
 *  fy (y+1/2), fz (z+1/2) as fe.
 *
 *****************************************************************************/

void orc_advect_upwind(const int L[3], int nf, const double * field,
		       const double * u, double * fw, double * fe,
		       double * fy, double * fz) {
  size_t N = nsites(L);

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i0 = site(L, x, y, z);
	size_t i1, idx;
	double uf;

	i1 = site(L, x-1, y, z);
	uf = 0.5*(u[i0] + u[i1]);
	idx = (uf > 0.0) ? i1 : i0;
	for (int n = 0; n < nf; n++) fw[n*N + i0] = uf*field[n*N + idx];

	i1 = site(L, x+1, y, z);
	uf = 0.5*(u[i0] + u[i1]);
	idx = (uf < 0.0) ? i1 : i0;
	for (int n = 0; n < nf; n++) fe[n*N + i0] = uf*field[n*N + idx];

	i1 = site(L, x, y+1, z);
	uf = 0.5*(u[N + i0] + u[N + i1]);
	idx = (uf < 0.0) ? i1 : i0;
	for (int n = 0; n < nf; n++) fy[n*N + i0] = uf*field[n*N + idx];

	i1 = site(L, x, y, z+1);
	uf = 0.5*(u[2*N + i0] + u[2*N + i1]);
	idx = (uf < 0.0) ? i1 : i0;
	for (int n = 0; n < nf; n++) fz[n*N + i0] = uf*field[n*N + idx];
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_advect_2nd: centred fluxes, src/advection.c:770-900
 *  (advection_2nd_kernel_v): face velocity 0.5 (u0 + u1), flux
 *  ((0.5 (u0 + u1)) 1) 0.5 (phi_a + phi_b), west face (phi(x-1) + phi(x)),
 *  the others (phi(x) + phi(x+1)).
 *
 *  orc_advect_3rd: three-point upwind-biased fluxes, src/advection.c:
 *  946-1135 (advection_le_3rd_kernel_v): u_face = (0.5 1)(u0 + u1),
 *  flux = u_face (a1 fd1 + a2 fd2 + a3 fd3) with a1 = -0.213933,
 *  a2 = 0.927865, a3 = 0.286067 and fd1..3 the values two sites upwind,
 *  one upwind and one downwind of the face.
 *
 *****************************************************************************/

void orc_advect_2nd(const int L[3], int nf, const double * field,
		    const double * u, double * fw, double * fe,
		    double * fy, double * fz) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i0 = site(L, x, y, z), i1;
	const double mask = 1.0;
	i1 = site(L, x-1, y, z);
	for (int n = 0; n < nf; n++) {
	  fw[n*N + i0] = 0.5*(u[i0] + u[i1])*mask*0.5
	    *(field[n*N + i1] + field[n*N + i0]);
	}
	i1 = site(L, x+1, y, z);
	for (int n = 0; n < nf; n++) {
	  fe[n*N + i0] = 0.5*(u[i0] + u[i1])*mask*0.5
	    *(field[n*N + i0] + field[n*N + i1]);
	}
	i1 = site(L, x, y+1, z);
	for (int n = 0; n < nf; n++) {
	  fy[n*N + i0] = 0.5*(u[N + i0] + u[N + i1])*mask*0.5
	    *(field[n*N + i0] + field[n*N + i1]);
	}
	i1 = site(L, x, y, z+1);
	for (int n = 0; n < nf; n++) {
	  fz[n*N + i0] = 0.5*(u[2*N + i0] + u[2*N + i1])*mask*0.5
	    *(field[n*N + i0] + field[n*N + i1]);
	}
      }
    }
  }
}

void orc_advect_3rd(const int L[3], int nf, const double * field,
		    const double * u, double * fw, double * fe,
		    double * fy, double * fz) {
  size_t N = nsites(L);
  const double a1 = -0.213933;
  const double a2 =  0.927865;
  const double a3 =  0.286067;
  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	const size_t i0 = site(L, x, y, z);
	const double mask = 1.0;
	/* x: m2 = x-2, m1 = x-1, p1 = x+1, p2 = x+2 */
	{
	  const size_t m2 = site(L, x-2, y, z), m1 = site(L, x-1, y, z);
	  const size_t p1 = site(L, x+1, y, z), p2 = site(L, x+2, y, z);
	  double uf = 0.5*mask*(u[i0] + u[m1]);
	  for (int n = 0; n < nf; n++) {
	    const double * f = field + n*N;
	    double d1, d2, d3;
	    if (uf > 0.0) { d1 = f[m2]; d2 = f[m1]; d3 = f[i0]; }
	    else          { d1 = f[p1]; d2 = f[i0]; d3 = f[m1]; }
	    fw[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
	  }
	  uf = 0.5*mask*(u[i0] + u[p1]);
	  for (int n = 0; n < nf; n++) {
	    const double * f = field + n*N;
	    double d1, d2, d3;
	    if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
	    else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
	    fe[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
	  }
	}
	/* y face between y and y+1 */
	{
	  const size_t m1 = site(L, x, y-1, z), p1 = site(L, x, y+1, z);
	  const size_t p2 = site(L, x, y+2, z);
	  double uf = 0.5*mask*(u[N + i0] + u[N + p1]);
	  for (int n = 0; n < nf; n++) {
	    const double * f = field + n*N;
	    double d1, d2, d3;
	    if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
	    else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
	    fy[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
	  }
	}
	/* z face between z and z+1 */
	{
	  const size_t m1 = site(L, x, y, z-1), p1 = site(L, x, y, z+1);
	  const size_t p2 = site(L, x, y, z+2);
	  double uf = 0.5*mask*(u[2*N + i0] + u[2*N + p1]);
	  for (int n = 0; n < nf; n++) {
	    const double * f = field + n*N;
	    double d1, d2, d3;
	    if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
	    else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
	    fz[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
	  }
	}
      }
    }
  }
}

/* Advection order of the Cahn-Hilliard step (src/advection.c:82,
 * advection_order_set): 1 (default), 2 or 3 */
static int adv_order_ = 1;
void orc_advection_order_set(int n) { adv_order_ = n; }

/* Gradient stencil of the binary step: 7 (default) or 27 points */
static int grad_stencil_ = 7;
void orc_gradient_stencil_set(int n) { grad_stencil_ = n; }

static void advect_order(const int L[3], int nf, const double * field,
			 const double * u, double * fw, double * fe,
			 double * fy, double * fz) {
  if (adv_order_ == 2) orc_advect_2nd(L, nf, field, u, fw, fe, fy, fz);
  else if (adv_order_ == 3) orc_advect_3rd(L, nf, field, u, fw, fe, fy, fz);
  else orc_advect_upwind(L, nf, field, u, fw, fe, fy, fz);
}

/*****************************************************************************
 *
 *  orc_ch_flux_mu
 *
 *  Diffusive fluxes, src/phi_cahn_hilliard.c:350-404:
 *  fw -= M (mu0 - mu(x-1)); fe -= M (mu(x+1) - mu0);
 *  fy -= M (mu(y+1) - mu0); fz -= M (mu(z+1) - mu0).
 *
 *****************************************************************************/

void orc_ch_flux_mu(const int L[3], const orc_symm_param_t * fe,
		    double mobility, const double * phi, const double * delsq,
		    double * fw, double * fe_, double * fy, double * fz) {
  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i0 = site(L, x, y, z);
	size_t i1;
	double mu0 = symm_mu_site(fe, phi[i0], delsq[i0]);
	double mu1;

	i1 = site(L, x-1, y, z);
	mu1 = symm_mu_site(fe, phi[i1], delsq[i1]);
	fw[i0] -= mobility*(mu0 - mu1);

	i1 = site(L, x+1, y, z);
	mu1 = symm_mu_site(fe, phi[i1], delsq[i1]);
	fe_[i0] -= mobility*(mu1 - mu0);

	i1 = site(L, x, y+1, z);
	mu1 = symm_mu_site(fe, phi[i1], delsq[i1]);
	fy[i0] -= mobility*(mu1 - mu0);

	i1 = site(L, x, y, z+1);
	mu1 = symm_mu_site(fe, phi[i1], delsq[i1]);
	fz[i0] -= mobility*(mu1 - mu0);
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_flux_no_normal
 *
 *  src/advection_bcs.c:80-140: every face flux is multiplied by
 *  (site is fluid)*(neighbour across that face is fluid).
 *
 *****************************************************************************/

void orc_flux_no_normal(const int L[3], int nf, const uint8_t * status,
			double * fw, double * fe, double * fy, double * fz) {
  size_t N = nsites(L);
  if (status == NULL) return;

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	double mask  = (status[i] == 0);
	double maskw = (status[site(L, x-1, y, z)] == 0);
	double maske = (status[site(L, x+1, y, z)] == 0);
	double masky = (status[site(L, x, y+1, z)] == 0);
	double maskz = (status[site(L, x, y, z+1)] == 0);
	for (int n = 0; n < nf; n++) {
	  fw[n*N + i] *= mask*maskw;
	  fe[n*N + i] *= mask*maske;
	  fy[n*N + i] *= mask*masky;
	  fz[n*N + i] *= mask*maskz;
	}
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_ch_update
 *
 *  Forward Euler, src/phi_cahn_hilliard.c:1018-1049:
 *  phi -= (fe - fw + fy - fy(y-1) + fz - fz(z-1))   (wz = 1 in 3d)
 *
 *****************************************************************************/

void orc_ch_update(const int L[3], const double * fw, const double * fe,
		   const double * fy, const double * fz, double * phi) {
  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	const double wz = 1.0;
	phi[i] -= (+ fe[i] - fw[i]
		   + fy[i] - fy[site(L, x, y-1, z)]
		   + wz*fz[i] - wz*fz[site(L, x, y, z-1)]);
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_collide_mrt
 *
 *  M10 collision with body force, src/collision.c:253-593
 *  (lb_collision_mrt1_site), no fluctuations, no viscosity model, no
 *  stress relaxation.  Mode transforms as src/collision.c:1990 and :2401
 *  (terms with an exact zero coefficient add nothing and are omitted:
 *  a running sum that starts at +0.0 is never -0.0 under round-to-nearest,
 *  so adding +/-0.0 leaves it unchanged).
 *
 *  f is updated in place; rho and u are written at fluid sites only
 *  (the chunk of one site is "full" exactly when the site is fluid).
 *
 *****************************************************************************/

static void collide_site_sth(const orc_collide_param_t * p,
			     double fs[NVEL], const double force[3],
			     const double sth[3][3], double * prho,
			     double u[3]);

static void collide_site(const orc_collide_param_t * p, double fs[NVEL],
			 const double force[3], double * prho, double u[3]) {
  collide_site_sth(p, fs, force, NULL, prho, u);
}

/* As collide_site; with sth the equilibrium stress includes the
 * thermodynamic stress (src/collision.c:706-1013, lb_collision_mrt2_site):
 * seq = rho u u + sth. */
static void collide_site_sth(const orc_collide_param_t * p,
			     double fs[NVEL], const double force[3],
			     const double sth[3][3], double * prho,
			     double u[3]) {

  double mode[NVEL];
  double s[3][3], seq[3][3];
  double rho, rrho, tr_s, tr_seq;
  const double rdim = (1.0/3.0);
  const double rtau = p->rtau_shear;
  const double rtau_bulk = p->rtau_bulk;

  /* f -> modes */
  for (int m = 0; m < NVEL; m++) {
    double acc = 0.0;
    for (int q = 0; q < NVEL; q++) {
      if (ma_[m][q] != 0.0) acc += fs[q]*ma_[m][q];
    }
    mode[m] = acc;
  }

  rho = mode[0];
  for (int ia = 0; ia < 3; ia++) u[ia] = mode[1 + ia];
  {
    int m = 0;
    for (int ia = 0; ia < 3; ia++) {
      for (int ib = ia; ib < 3; ib++) {
	s[ia][ib] = mode[4 + m];
	m++;
      }
    }
    for (int ia = 1; ia < 3; ia++) {
      for (int ib = 0; ib < ia; ib++) s[ia][ib] = s[ib][ia];
    }
  }

  rrho = 1.0/rho;
  for (int ia = 0; ia < 3; ia++) u[ia] = rrho*(u[ia] + 0.5*force[ia]);

  tr_s = 0.0;
  tr_seq = 0.0;
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      seq[ia][ib] = rho*u[ia]*u[ib];
      if (sth) seq[ia][ib] = rho*u[ia]*u[ib] + sth[ia][ib];
    }
    tr_s   += s[ia][ia];
    tr_seq += seq[ia][ia];
  }

  for (int ia = 0; ia < 3; ia++) {
    s[ia][ia]   -= rdim*tr_s;
    seq[ia][ia] -= rdim*tr_seq;
  }

  tr_s = tr_s - rtau_bulk*(tr_s - tr_seq);

  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double dab = (ia == ib);
      s[ia][ib] -= rtau*(s[ia][ib] - seq[ia][ib]);
      s[ia][ib] += dab*rdim*tr_s;
      s[ia][ib] += (2.0 - rtau)*(u[ia]*force[ib] + force[ia]*u[ib]);
    }
  }

  for (int ia = 0; ia < 3; ia++) mode[1 + ia] += force[ia];
  {
    int m = 0;
    for (int ia = 0; ia < 3; ia++) {
      for (int ib = ia; ib < 3; ib++) {
	mode[4 + m] = s[ia][ib] + 0.0;
	m++;
      }
    }
  }

  for (int m = 10; m < NVEL; m++) {
    mode[m] = mode[m] - p->rtau_ghost[m]*(mode[m] - 0.0) + 0.0;
  }

  /* modes -> f */
  for (int q = 0; q < NVEL; q++) {
    double acc = 0.0;
    for (int m = 0; m < NVEL; m++) {
      if (mi_[q][m] != 0.0) acc += mi_[q][m]*mode[m];
    }
    fs[q] = acc;
  }

  *prho = rho;
}

void orc_collide_mrt(const int L[3], const orc_collide_param_t * p,
		     const uint8_t * status, double * f, const double * force,
		     double * rho, double * u) {
  size_t N = nsites(L);
  tables_init();

  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double fs[NVEL], fa[3], uu[3], r;
    for (int q = 0; q < NVEL; q++) fs[q] = f[q*N + i];
    for (int ia = 0; ia < 3; ia++) {
      fa[ia] = p->force_global[ia] + (force ? force[ia*N + i] : 0.0);
    }
    collide_site(p, fs, fa, &r, uu);
    if (status == NULL || status[i] == 0) {
      for (int q = 0; q < NVEL; q++) f[q*N + i] = fs[q];
      rho[i] = r;
      for (int ia = 0; ia < 3; ia++) u[ia*N + i] = uu[ia];
    }
  }
}

/*****************************************************************************
 *
 *  orc_propagate
 *
 *  Pull streaming, src/propagation.c:153-197:
 *  fprime_p(x) = f_p(x - c_p).
 *
 *****************************************************************************/

void orc_propagate(const int L[3], const double * f, double * fprime) {
  size_t N = nsites(L);

  #pragma omp parallel for
  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	for (int q = 0; q < NVEL; q++) {
	  fprime[q*N + i] = f[q*N + site(L, x - cv_[q][0], y - cv_[q][1],
					 z - cv_[q][2])];
	}
      }
    }
  }
}

/*****************************************************************************
 *
 *  orc_binary_step
 *
 *  The main-loop order of src/ludwig.c:528-860 for the symmetric free
 *  energy with the finite-difference Cahn-Hilliard solver, no colloids,
 *  no walls, no Lees-Edwards planes:
 *    hydro_f_zero; field_halo(phi); field_grad_compute;
 *    phi_force_calculation (stress divergence);
 *    phi_cahn_hilliard (u halo, upwind advection, mu fluxes, no-flux
 *    mask, forward step);
 *    hydro_u_zero; lb_collide; lb_halo; lb_propagation.
 *
 *  f and fscratch are swapped in place (the result is always in f).
 *  work holds 13 N doubles: grad 3, delsq 1, pth 9 (fluxes reuse pth).
 *
 *****************************************************************************/

void orc_binary_step(const int L[3], const orc_symm_param_t * fe,
		     double mobility, const orc_collide_param_t * cp,
		     const uint8_t * status,
		     double * f, double * fscratch, double * phi, double * u,
		     double * rho, double * force, double * work, int nsteps) {
  size_t N = nsites(L);
  double * grad = work;
  double * delsq = work + 3*N;
  double * pth = work + 4*N;

  tables_init();

  for (int step = 0; step < nsteps; step++) {

    memset(force, 0, 3*N*sizeof(double));
    if (grad_stencil_ == 27) orc_grad_27pt(L, 1, phi, grad, delsq);
    else orc_grad_7pt(L, 1, phi, grad, delsq);
    orc_symm_stress(L, fe, phi, grad, delsq, pth);
    orc_force_divergence(L, pth, force);

    {
      double * fw = pth, * fe_ = pth + N, * fy = pth + 2*N, * fz = pth + 3*N;
      advect_order(L, 1, phi, u, fw, fe_, fy, fz);
      orc_ch_flux_mu(L, fe, mobility, phi, delsq, fw, fe_, fy, fz);
      orc_flux_no_normal(L, 1, status, fw, fe_, fy, fz);
      orc_ch_update(L, fw, fe_, fy, fz, phi);
    }

    memset(u, 0, 3*N*sizeof(double));
    orc_collide_mrt(L, cp, status, f, force, rho, u);
    orc_propagate(L, f, fscratch);
    memcpy(f, fscratch, NVEL*N*sizeof(double));
  }
}

/*****************************************************************************
 *
 *  Two-distribution binary fluid (symmetric_lb), ndist = 2.
 *
 *  orc_phi_from_g: phi = sum_p g_p in order p (src/phi_lb_coupler.c:72-93).
 *
 *  orc_collide_binary: src/collision.c:706-1013 (lb_collision_mrt2_site)
 *  for one step at every site: f relaxes as the single-fluid collision
 *  with the chemical stress (src/symmetric.c:372, fe_symm_str_v) in the
 *  equilibrium stress; then the order-parameter distribution is rebuilt
 *  from phi, jphi (relaxed toward phi u at rate rtau2 = 2/(1 + 2 M),
 *  src/collision.c:1951) and sphi = phi u u + mu delta, with the sums of
 *  d3q19_mode2f_phi (src/collision.c:2849-): for each p, jdotc adds the
 *  jphi components with c_pa != 0 and sphidotq the sphi entries with
 *  c_pa c_pb - delta_ab/3 != 0 in row-major order; then
 *  g_p = w_p (3 jdotc + 4.5 sphidotq) (+ phi for p = 0).
 *
 *  u is written at every site (no rho: the binary collision does not
 *  store it).
 *
 *****************************************************************************/

void orc_phi_from_g(const int L[3], const double * g, double * phi) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double phi0 = 0.0;
    for (int q = 0; q < NVEL; q++) phi0 += g[q*N + i];
    phi[i] = phi0;
  }
}

void orc_collide_binary(const int L[3], const orc_symm_param_t * fe,
			const orc_collide_param_t * cp, double mobility,
			double * f, double * g, const double * phi,
			const double * grad, const double * delsq, double * u) {
  size_t N = nsites(L);
  const double rtau2 = 2.0/(1.0 + 2.0*mobility);
  const double r3 = (1.0/3.0);
  const double q_diag[2] = {-(1.0/3.0), (2.0/3.0)};   /* c_a^2 = 0, 1 */
  tables_init();

  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double fs[NVEL], fa[3], uu[3], r, sth[3][3];
    const double ph = phi[i];
    const double gr[3] = {grad[i], grad[N + i], grad[2*N + i]};
    const double d = delsq[i];

    /* chemical stress, src/symmetric.c:372-400 */
    {
      const double p0 = 0.5*fe->a*ph*ph + 0.75*fe->b*ph*ph*ph*ph
	- fe->kappa*ph*d - 0.5*fe->kappa*(gr[0]*gr[0] + gr[1]*gr[1]
					 + gr[2]*gr[2]);
      for (int ia = 0; ia < 3; ia++) {
	for (int ib = 0; ib < 3; ib++) {
	  const double dab = (ia == ib);
	  sth[ia][ib] = p0*dab + fe->kappa*gr[ia]*gr[ib];
	}
      }
    }

    for (int q = 0; q < NVEL; q++) fs[q] = f[q*N + i];
    for (int ia = 0; ia < 3; ia++) fa[ia] = cp->force_global[ia] + 0.0;
    collide_site_sth(cp, fs, fa, (const double (*)[3]) sth, &r, uu);
    for (int q = 0; q < NVEL; q++) f[q*N + i] = fs[q];
    for (int ia = 0; ia < 3; ia++) u[ia*N + i] = uu[ia];

    /* order parameter distribution */
    const double mu = symm_mu_site(fe, ph, d);
    double jphi[3] = {0.0, 0.0, 0.0};
    for (int q = 1; q < NVEL; q++) {
      for (int ia = 0; ia < 3; ia++) {
	if (cv_[q][ia]) jphi[ia] += cv_[q][ia]*g[q*N + i];
      }
    }
    double sphi[3][3];
    for (int ia = 0; ia < 3; ia++) {
      for (int ib = 0; ib < 3; ib++) {
	const double dab = (ia == ib);
	sphi[ia][ib] = ph*uu[ia]*uu[ib] + mu*dab;
      }
      jphi[ia] = jphi[ia] - rtau2*(jphi[ia] - ph*uu[ia]);
    }
    (void) r3;
    for (int q = 0; q < NVEL; q++) {
      double jdotc = 0.0, sphidotq = 0.0;
      for (int ia = 0; ia < 3; ia++) {
	if (cv_[q][ia] > 0) jdotc += jphi[ia];
	if (cv_[q][ia] < 0) jdotc -= jphi[ia];
      }
      for (int ia = 0; ia < 3; ia++) {
	for (int ib = 0; ib < 3; ib++) {
	  double qab;
	  if (ia == ib) qab = q_diag[cv_[q][ia] != 0];
	  else qab = (double) (cv_[q][ia]*cv_[q][ib]);
	  if (qab != 0.0) sphidotq += sphi[ia][ib]*qab;
	}
      }
      double gq = wv_[q]*(jdotc*3.0 + sphidotq*4.5);
      if (q == 0) gq = wv_[q]*(jdotc*3.0 + sphidotq*4.5) + ph;
      g[q*N + i] = gq;
    }
  }
}

/* The main loop of src/ludwig.c:528-860 with ndist = 2: phi from g,
 * gradients, binary collision, propagation of f and g.  The results are
 * in f, g, phi (phi of the last step's start) and u.  work: 4 N doubles;
 * scratch: 19 N doubles. */
void orc_lb2_step(const int L[3], const orc_symm_param_t * fe,
		  double mobility, const orc_collide_param_t * cp,
		  double * f, double * g, double * scratch, double * phi,
		  double * u, double * work, int nsteps) {
  size_t N = nsites(L);
  double * grad = work;
  double * delsq = work + 3*N;
  tables_init();
  for (int step = 0; step < nsteps; step++) {
    orc_phi_from_g(L, g, phi);
    orc_grad_7pt(L, 1, phi, grad, delsq);
    orc_collide_binary(L, fe, cp, mobility, f, g, phi, grad, delsq, u);
    orc_propagate(L, f, scratch);
    memcpy(f, scratch, NVEL*N*sizeof(double));
    orc_propagate(L, g, scratch);
    memcpy(g, scratch, NVEL*N*sizeof(double));
  }
}

/*****************************************************************************
 *
 *  Compensated sums, src/util_sum.c:30-140, and field statistics in the
 *  order of src/phi_stats.c:211-270 for one thread (serial sweep).
 *
 *****************************************************************************/

void orc_klein_add(orc_klein_t * k, double val) {
  volatile double c;
  volatile double cc;
  volatile double t = k->sum + val;

  if (fabs(k->sum) >= fabs(val)) {
    c = (k->sum - t) + val;
  }
  else {
    c = (val - t) + k->sum;
  }
  k->sum = t;
  t = k->cs + c;
  if (fabs(k->cs) >= fabs(c)) {
    cc = (k->cs - t) + c;
  }
  else {
    cc = (c - t) + k->cs;
  }
  k->cs = t;
  k->ccs = k->ccs + cc;
}

double orc_klein_total(const orc_klein_t * k) {
  return k->sum + k->cs + k->ccs;
}

/* out = {total, mean, variance, min, max} (src/phi_stats.c:116-123) */

void orc_field_stats(const int L[3], const double * q, double out[5]) {
  size_t N = nsites(L);
  orc_klein_t k = {0.0, 0.0, 0.0};
  double qvar = 0.0, qmin = +1.0e300, qmax = -1.0e300, vol = 0.0;

  for (size_t i = 0; i < N; i++) {
    orc_klein_add(&k, q[i]);
    qvar += q[i]*q[i];
    qmin = (q[i] < qmin) ? q[i] : qmin;
    qmax = (q[i] > qmax) ? q[i] : qmax;
    vol += 1.0;
  }
  {
    double qsum = orc_klein_total(&k);
    double rvol = 1.0/vol;
    double qbar = rvol*qsum;
    out[0] = qsum;
    out[1] = qbar;
    out[2] = rvol*qvar - qbar*qbar;
    out[3] = qmin;
    out[4] = qmax;
  }
}

/* Free energy density src/symmetric.c:285-300, summed with a Klein sum */

double orc_symm_fed_total(const int L[3], const orc_symm_param_t * fe,
			  const double * phi, const double * grad) {
  size_t N = nsites(L);
  orc_klein_t k = {0.0, 0.0, 0.0};
  for (size_t i = 0; i < N; i++) {
    double g0 = grad[i], g1 = grad[N + i], g2 = grad[2*N + i];
    double ph = phi[i];
    double fed = (0.5*fe->a + 0.25*fe->b*ph*ph)*ph*ph
      + 0.5*fe->kappa*(g0*g0 + g1*g1 + g2*g2);
    orc_klein_add(&k, fed);
  }
  return orc_klein_total(&k);
}

/*****************************************************************************
 *
 *  Cholesteric liquid crystal (Landau-de Gennes free energy).
 *
 *  The per-site formulas follow the loop forms of the reference:
 *  molecular field src/blue_phase.c:1016-1110 (fe_lc_compute_h),
 *  free-energy density :309-400 (fe_lc_compute_fed), chiral stress
 *  :827-930 (fe_lc_compute_stress, with its final minus sign).  The
 *  reference's device build evaluates the same expressions through
 *  unrolled forms (:2094-2450), so the two agree to rounding.
 *
 *****************************************************************************/

enum {NQAB = 5};

static const int lc_e_[3][3][3] = {
  {{0, 0, 0}, {0, 0, 1}, {0, -1, 0}},
  {{0, 0, -1}, {0, 0, 0}, {1, 0, 0}},
  {{0, 1, 0}, {-1, 0, 0}, {0, 0, 0}}};

static void lc_expand(const double * a, size_t N, size_t i, double t[3][3]) {
  t[0][0] = a[0*N + i];
  t[0][1] = a[1*N + i];
  t[0][2] = a[2*N + i];
  t[1][0] = t[0][1];
  t[1][1] = a[3*N + i];
  t[1][2] = a[4*N + i];
  t[2][0] = t[0][2];
  t[2][1] = t[1][2];
  t[2][2] = 0.0 - t[0][0] - t[1][1];
}

/* dq[ia][b][c] = d_ia Q_bc from grad[(3*n + ia)] of the 5 components */
static void lc_expand_grad(const double * g, size_t N, size_t i,
			   double dq[3][3][3]) {
  for (int ia = 0; ia < 3; ia++) {
    dq[ia][0][0] = g[(3*0 + ia)*N + i];
    dq[ia][0][1] = g[(3*1 + ia)*N + i];
    dq[ia][0][2] = g[(3*2 + ia)*N + i];
    dq[ia][1][0] = dq[ia][0][1];
    dq[ia][1][1] = g[(3*3 + ia)*N + i];
    dq[ia][1][2] = g[(3*4 + ia)*N + i];
    dq[ia][2][0] = dq[ia][0][2];
    dq[ia][2][1] = dq[ia][1][2];
    dq[ia][2][2] = 0.0 - dq[ia][0][0] - dq[ia][1][1];
  }
}

static void lc_h_site(const orc_lc_param_t * p, double q[3][3],
		      double dq[3][3][3], double dsq[3][3], double h[3][3]) {
  const double r3 = (1.0/3.0);
  const double gamma = p->gamma;
  double q0 = p->q0*p->rredshift;
  double kappa0 = p->kappa0*p->redshift*p->redshift;
  double kappa1 = p->kappa1*p->redshift*p->redshift;
  double q2 = 0.0, eq = 0.0, e2 = 0.0;

  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) q2 += q[ia][ib]*q[ia][ib];

  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double sum = 0.0;
      double dab = (ia == ib);
      for (int ic = 0; ic < 3; ic++) sum += q[ia][ic]*q[ib][ic];
      h[ia][ib] = -p->a0*(1.0 - r3*gamma)*q[ia][ib]
	+ p->a0*gamma*(sum - r3*q2*dab)
	- p->a0*gamma*q2*q[ia][ib];
    }
  }

  for (int ib = 0; ib < 3; ib++)
    for (int ic = 0; ic < 3; ic++)
      for (int ia = 0; ia < 3; ia++) eq += lc_e_[ib][ic][ia]*dq[ib][ic][ia];

  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double sum = 0.0;
      double dab = (ia == ib);
      for (int ic = 0; ic < 3; ic++) {
	for (int id = 0; id < 3; id++) {
	  sum += (lc_e_[ia][ic][id]*dq[ic][ib][id]
		  + lc_e_[ib][ic][id]*dq[ic][ia][id]);
	}
      }
      h[ia][ib] += kappa0*dsq[ia][ib]
	- 2.0*kappa1*q0*sum + 4.0*r3*kappa1*q0*eq*dab
	- 4.0*kappa1*q0*q0*q[ia][ib];
    }
  }

  for (int ia = 0; ia < 3; ia++) {
    double ea = p->e0[ia]*p->coswt;
    e2 += ea*ea;
  }
  for (int ia = 0; ia < 3; ia++) {
    double ea = p->e0[ia]*p->coswt;
    for (int ib = 0; ib < 3; ib++) {
      double eb = p->e0[ib]*p->coswt;
      double dab = (ia == ib);
      h[ia][ib] += p->epsilon*(ea*eb - r3*dab*e2);
    }
  }
}

static double lc_fed_site(const orc_lc_param_t * p, double q[3][3],
			  double dq[3][3][3]) {
  const double r3 = 1.0/3.0;
  const double gamma = p->gamma;
  double q0 = p->q0*p->rredshift;
  double kappa0 = p->kappa0*p->redshift*p->redshift;
  double kappa1 = p->kappa1*p->redshift*p->redshift;
  double q2 = 0.0, q3 = 0.0, dq0 = 0.0, dq1 = 0.0, efield = 0.0;

  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) q2 += q[ia][ib]*q[ia][ib];
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++)
      for (int ic = 0; ic < 3; ic++) q3 += q[ia][ib]*q[ib][ic]*q[ia][ic];
  for (int ia = 0; ia < 3; ia++) {
    double sum = 0.0;
    for (int ib = 0; ib < 3; ib++) sum += dq[ib][ia][ib];
    dq0 += sum*sum;
  }
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double sum = 0.0;
      for (int ic = 0; ic < 3; ic++)
	for (int id = 0; id < 3; id++) sum += lc_e_[ia][ic][id]*dq[ic][ib][id];
      sum += 2.0*q0*q[ia][ib];
      dq1 += sum*sum;
    }
  }
  for (int ia = 0; ia < 3; ia++) {
    double ea = p->e0[ia]*p->coswt;
    for (int ib = 0; ib < 3; ib++) {
      double eb = p->e0[ib]*p->coswt;
      efield += ea*q[ia][ib]*eb;
    }
  }
  return 0.5*p->a0*(1.0 - r3*gamma)*q2 - r3*p->a0*gamma*q3
    + 0.25*p->a0*gamma*q2*q2 + 0.5*kappa0*dq0 + 0.5*kappa1*dq1
    - p->epsilon*efield;
}

static void lc_stress_site(const orc_lc_param_t * p, double q[3][3],
			   double dq[3][3][3], double h[3][3],
			   double sth[3][3]) {
  const double r3 = (1.0/3.0);
  double q0 = p->q0*p->rredshift;
  double kappa0 = p->kappa0*p->redshift*p->redshift;
  double kappa1 = p->kappa1*p->redshift*p->redshift;
  double p0 = 0.0 - lc_fed_site(p, q, dq);
  double qh = 0.0;

  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) qh += q[ia][ib]*h[ia][ib];

  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      double dab = (ia == ib);
      sth[ia][ib] = -p0*dab + 2.0*p->xi*(q[ia][ib] + r3*dab)*qh;
    }
  }
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      for (int ic = 0; ic < 3; ic++) {
	double dbc = (ib == ic), dac = (ia == ic);
	sth[ia][ib] += -p->xi*h[ia][ic]*(q[ib][ic] + r3*dbc)
	  -p->xi*(q[ia][ic] + r3*dac)*h[ib][ic];
      }
    }
  }
  for (int ia = 0; ia < 3; ia++) {
    for (int ib = 0; ib < 3; ib++) {
      for (int ic = 0; ic < 3; ic++) {
	for (int id = 0; id < 3; id++) {
	  sth[ia][ib] += - kappa0*dq[ia][ib][ic]*dq[id][ic][id]
	    - kappa1*dq[ia][ic][id]*dq[ib][ic][id]
	    + kappa1*dq[ia][ic][id]*dq[ic][ib][id];
	  for (int ie = 0; ie < 3; ie++) {
	    sth[ia][ib] += -2.0*kappa1*q0*dq[ia][ic][id]*lc_e_[ib][ic][ie]
	      *q[id][ie];
	  }
	}
      }
    }
  }
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++)
      for (int ic = 0; ic < 3; ic++)
	sth[ia][ib] += q[ia][ic]*h[ib][ic] - h[ia][ic]*q[ib][ic];

  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) sth[ia][ib] = -sth[ia][ib];
}

void orc_lc_mol_field(const int L[3], const orc_lc_param_t * p,
		      const double * q, const double * grad,
		      const double * delsq, double * h) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double qs[3][3], dq[3][3][3], dsq[3][3], hs[3][3];
    lc_expand(q, N, i, qs);
    lc_expand_grad(grad, N, i, dq);
    lc_expand(delsq, N, i, dsq);
    lc_h_site(p, qs, dq, dsq, hs);
    h[0*N + i] = hs[0][0]; h[1*N + i] = hs[0][1]; h[2*N + i] = hs[0][2];
    h[3*N + i] = hs[1][1]; h[4*N + i] = hs[1][2];
  }
}

void orc_lc_stress(const int L[3], const orc_lc_param_t * p,
		   const double * q, const double * grad,
		   const double * delsq, double * pth) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double qs[3][3], dq[3][3][3], dsq[3][3], hs[3][3], s[3][3];
    lc_expand(q, N, i, qs);
    lc_expand_grad(grad, N, i, dq);
    lc_expand(delsq, N, i, dsq);
    lc_h_site(p, qs, dq, dsq, hs);
    lc_stress_site(p, qs, dq, hs, s);
    for (int ia = 0; ia < 3; ia++)
      for (int ib = 0; ib < 3; ib++) pth[(3*ia + ib)*N + i] = s[ia][ib];
  }
}

void orc_lc_fed(const int L[3], const orc_lc_param_t * p, const double * q,
		const double * grad, double * fed) {
  size_t N = nsites(L);
  #pragma omp parallel for
  for (size_t i = 0; i < N; i++) {
    double qs[3][3], dq[3][3][3];
    lc_expand(q, N, i, qs);
    lc_expand_grad(grad, N, i, dq);
    fed[i] = lc_fed_site(p, qs, dq);
  }
}

/*****************************************************************************
 *
 *  orc_beris_edw_update
 *
 *  src/blue_phase_beris_edwards.c:266-289 (driver): upwind advective
 *  fluxes of the 5 components (src/advection.c:538-629), no-normal-flux
 *  mask, molecular field, then the site update of :538-840:
 *    W_ab = d_b u_a (centred), made traceless; D, Omega its symmetric and
 *    antisymmetric parts;
 *    S = -2 xi (Q + I/3) tr(QW) + (xi D + Omega)(Q + I/3)
 *        + (Q + I/3)(xi D - Omega);
 *    Q += S + Gamma H - div(flux)   (dt = 1, no noise)
 *  at fluid sites.  u may be NULL (no hydrodynamics).
 *
 *****************************************************************************/

void orc_beris_edw_update(const int L[3], const orc_lc_param_t * p,
			  double gamma_rot, const uint8_t * status,
			  const double * u, const double * grad,
			  const double * delsq, double * q, double * work) {
  size_t N = nsites(L);
  double * fw = work, * fe = work + 5*N, * fy = work + 10*N;
  double * fz = work + 15*N;
  double * h = work + 20*N;                     /* 5 N */

  if (u) {
    orc_advect_upwind(L, NQAB, q, u, fw, fe, fy, fz);
    orc_flux_no_normal(L, NQAB, status, fw, fe, fy, fz);
  }
  orc_lc_mol_field(L, p, q, grad, delsq, h);

  {
    double * qn = work + 25*N;                   /* 5 N */
    const double r3 = (1.0/3.0);
    const double dt = 1.0;

    #pragma omp parallel for
    for (int x = 0; x < L[0]; x++) {
      for (int y = 0; y < L[1]; y++) {
	for (int z = 0; z < L[2]; z++) {
	  size_t i = site(L, x, y, z);
	  double qs[3][3], w[3][3] = {{0}}, d[3][3], om[3][3], s[3][3] = {{0}};
	  lc_expand(q, N, i, qs);
	  int fluid = (status == NULL || status[i] == 0);

	  if (u) {
	    size_t im = site(L, x-1, y, z), ip = site(L, x+1, y, z);
	    double tr, trace_qw = 0.0;
	    if (fluid) {
	      for (int ia = 0; ia < 3; ia++)
		w[ia][0] = 0.5*(u[ia*N + ip] - u[ia*N + im]);
	    }
	    im = site(L, x, y-1, z); ip = site(L, x, y+1, z);
	    for (int ia = 0; ia < 3; ia++)
	      w[ia][1] = 0.5*(u[ia*N + ip] - u[ia*N + im]);
	    im = site(L, x, y, z-1); ip = site(L, x, y, z+1);
	    for (int ia = 0; ia < 3; ia++)
	      w[ia][2] = 0.5*(u[ia*N + ip] - u[ia*N + im]);

	    tr = r3*(w[0][0] + w[1][1] + w[2][2]);
	    w[0][0] -= tr; w[1][1] -= tr; w[2][2] -= tr;

	    for (int ia = 0; ia < 3; ia++) {
	      for (int ib = 0; ib < 3; ib++) {
		trace_qw += qs[ia][ib]*w[ib][ia];
		d[ia][ib]  = 0.5*(w[ia][ib] + w[ib][ia]);
		om[ia][ib] = 0.5*(w[ia][ib] - w[ib][ia]);
	      }
	    }
	    for (int ia = 0; ia < 3; ia++) {
	      for (int ib = 0; ib < 3; ib++) {
		double dab = (ia == ib);
		s[ia][ib] = -2.0*p->xi*(qs[ia][ib] + r3*dab)*trace_qw;
		for (int id = 0; id < 3; id++) {
		  double ddb = (id == ib), dad = (ia == id);
		  s[ia][ib] += (p->xi*d[ia][id] + om[ia][id])
		    *(qs[id][ib] + r3*ddb)
		    + (qs[ia][id] + r3*dad)*(p->xi*d[id][ib] - om[id][ib]);
		}
	      }
	    }
	  }

	  {
	    static const int ca[NQAB] = {0, 0, 0, 1, 1};
	    static const int cb[NQAB] = {0, 1, 2, 1, 2};
	    size_t ij = site(L, x, y-1, z), ik = site(L, x, y, z-1);
	    for (int n = 0; n < NQAB; n++) {
	      double v = qs[ca[n]][cb[n]];
	      if (fluid) {
		/* zero fluxes without hydrodynamics */
		double fen = u ? fe[n*N + i] : 0.0, fwn = u ? fw[n*N + i] : 0.0;
		double fyn = u ? fy[n*N + i] : 0.0, fyj = u ? fy[n*N + ij] : 0.0;
		double fzn = u ? fz[n*N + i] : 0.0, fzk = u ? fz[n*N + ik] : 0.0;
		v += dt*(s[ca[n]][cb[n]] + 0.0 + gamma_rot*h[n*N + i]
			 - fen + fwn - fyn + fyj - fzn + fzk);
	      }
	      qn[n*N + i] = v;
	    }
	  }
	}
      }
    }
    memcpy(q, qn, 5*N*sizeof(double));
  }
}

/*****************************************************************************
 *
 *  orc_lc_step
 *
 *  src/ludwig.c:528-860 for the cholesteric (no colloids, walls or
 *  planes): q halo, q gradients, stress divergence force, u halo,
 *  Beris-Edwards update, u zero, collision, halo, propagation.
 *  work >= 45 N doubles.
 *
 *****************************************************************************/

void orc_lc_step(const int L[3], const orc_lc_param_t * p, double gamma_rot,
		 const orc_collide_param_t * cp, const uint8_t * status,
		 double * f, double * fscratch, double * q, double * u,
		 double * rho, double * force, double * work, int nsteps) {
  size_t N = nsites(L);
  double * grad = work;                 /* 15 N */
  double * delsq = work + 15*N;         /*  5 N */
  double * pth = work + 20*N;           /*  9 N; reused by the update */
  double * bew = work + 20*N;           /* 30 N for the update */

  tables_init();

  for (int step = 0; step < nsteps; step++) {
    memset(force, 0, 3*N*sizeof(double));
    orc_grad_7pt(L, NQAB, q, grad, delsq);
    orc_lc_stress(L, p, q, grad, delsq, pth);
    orc_force_divergence(L, pth, force);
    orc_beris_edw_update(L, p, gamma_rot, status, u, grad, delsq, q, bew);
    memset(u, 0, 3*N*sizeof(double));
    orc_collide_mrt(L, cp, status, f, force, rho, u);
    orc_propagate(L, f, fscratch);
    memcpy(f, fscratch, NVEL*N*sizeof(double));
  }
}

/* src/blue_phase_init.c:59-132 without rotation; global coordinates are
 * 1-based */

void orc_lc_init_o8m(const int L[3], const orc_lc_param_t * p, double * q) {
  size_t N = nsites(L);
  const double root2 = sqrt(2.0);
  const double q0 = p->q0, a = p->amplitude0;

  for (int x = 0; x < L[0]; x++) {
    for (int y = 0; y < L[1]; y++) {
      for (int z = 0; z < L[2]; z++) {
	size_t i = site(L, x, y, z);
	double r[3];
	r[0] = (double) (x + 1) - 0.5*L[0];
	r[1] = (double) (y + 1) - 0.5*L[1];
	r[2] = (double) (z + 1) - 0.5*L[2];
	r[0] += 0.5*L[0]; r[1] += 0.5*L[1]; r[2] += 0.5*L[2];
	double cosx = cos(root2*q0*r[0]), sinx = sin(root2*q0*r[0]);
	double cosy = cos(root2*q0*r[1]), siny = sin(root2*q0*r[1]);
	double cosz = cos(root2*q0*r[2]), sinz = sin(root2*q0*r[2]);
	q[0*N + i] = a*(-2.0*cosy*sinz + sinx*cosz + cosx*siny);
	q[1*N + i] = a*(root2*cosy*cosz + root2*sinx*sinz - sinx*cosy);
	q[2*N + i] = a*(root2*cosx*cosy + root2*sinz*siny - cosx*sinz);
	q[3*N + i] = a*(-2.0*sinx*cosz + siny*cosx + cosy*sinz);
	q[4*N + i] = a*(root2*cosz*cosx + root2*siny*sinx - siny*cosz);
      }
    }
  }
}
