/*****************************************************************************
 *
 *  lgb_coarse.cu
 *
 *  Restriction of a binary-fluid state from a fine lattice to the lattice
 *  coarsened by 2 in every direction, in the units of the coarse lattice.
 *  Diffusive scaling (dx x 2, dt x 4): lengths / 2, velocities x 2, strain
 *  rates x 4.  Per coarse site the 8 fine sites are averaged:
 *
 *    phi_c = <phi>,  rho_c = <rho>,  u_c = s_u <u>               (s_u = 2)
 *    j_c   = s_u <j>,
 *    Pi_c  = rho_c/3 I + j_c j_c / rho_c + s_neq (<Pi> - <rho>/3 I - <j><j>/<rho>)
 *                                                                 (s_neq = 4)
 *
 *  and the coarse distributions are rebuilt from (rho_c, j_c, Pi_c) with
 *  the second-order Hermite form (ghost modes zero):
 *
 *    f_p = w_p [rho + 3 c_p.j + 9/2 (c_p c_p - I/3) : (Pi - rho/3 I)].
 *
 *  Fine f may be stored post-collision with streaming pending (the fused
 *  step's form): then f_p(x) is read as stored_p(x - c_p).  Both lattices
 *  hold FP32 deviations f - w_p rho0.
 *
 *****************************************************************************/

#include "lgb_common.cuh"
#include "lgb_coarse.h"

__global__ void k_restrict_state(lgbk_dims_t df, lgbk_dims_t dc,
				 const float * __restrict__ ff, int pending,
				 const float * __restrict__ phif,
				 const float * __restrict__ uf,
				 float rho0, float su, float sneq,
				 float * __restrict__ fc,
				 float * __restrict__ phic,
				 float * __restrict__ uc,
				 float * __restrict__ rhoc) {
  const long long sc = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (sc >= dc.nsites) return;
  const int zc = (int) (sc % dc.nz);
  const long long r = sc / dc.nz;
  const int yc = (int) (r % dc.ny);
  const int xc = (int) (r / dc.ny);
  const long long Nf = df.nsites, Nc = dc.nsites;

  double drho = 0.0, phi = 0.0;
  double j[3] = {0.0, 0.0, 0.0}, uu[3] = {0.0, 0.0, 0.0};
  double pi[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};

  for (int k = 0; k < 8; k++) {
    const int x = 2*xc + (k >> 2), y = 2*yc + ((k >> 1) & 1), z = 2*zc + (k & 1);
    const long long s = lgb_site(df, x, y, z);
    phi += (double) phif[s];
    for (int a = 0; a < 3; a++) uu[a] += (double) uf[a*Nf + s];
    for (int p = 0; p < LGB_NVEL; p++) {
      const int cx = lgb_cv_c[p][0], cy = lgb_cv_c[p][1], cz = lgb_cv_c[p][2];
      long long src = s;
      if (pending) src = lgb_site_w(df, x - cx, y - cy, z - cz);
      const double v = (double) ff[p*Nf + src];
      const int c[3] = {cx, cy, cz};
      drho += v;
      for (int a = 0; a < 3; a++) {
	j[a] += c[a]*v;
	for (int b = 0; b < 3; b++) pi[a][b] += c[a]*c[b]*v;
      }
    }
  }
  const double r8 = 0.125;
  drho *= r8; phi *= r8;
  for (int a = 0; a < 3; a++) {
    j[a] *= r8; uu[a] *= r8;
    for (int b = 0; b < 3; b++) pi[a][b] *= r8;
  }
  /* Fine averages: rho = rho0 + drho; the deviation's second moment
   * lacks the rest part rho0/3 I, which cancels in Pi - rho/3 I. */
  const double rho = (double) rho0 + drho;
  double pneq[3][3];
  for (int a = 0; a < 3; a++) {
    for (int b = 0; b < 3; b++) {
      const double pfull = pi[a][b] + ((a == b) ? (double) rho0/3.0 : 0.0);
      pneq[a][b] = pfull - ((a == b) ? rho/3.0 : 0.0) - j[a]*j[b]/rho;
    }
  }
  double jc[3], pdev[3][3];
  for (int a = 0; a < 3; a++) jc[a] = (double) su*j[a];
  for (int a = 0; a < 3; a++) {
    for (int b = 0; b < 3; b++) {
      pdev[a][b] = jc[a]*jc[b]/rho + (double) sneq*pneq[a][b];
    }
  }
  for (int p = 0; p < LGB_NVEL; p++) {
    const int c[3] = {lgb_cv_c[p][0], lgb_cv_c[p][1], lgb_cv_c[p][2]};
    const double w = lgb_w(p);
    double cj = 0.0, cpc = 0.0;
    for (int a = 0; a < 3; a++) {
      cj += c[a]*jc[a];
      for (int b = 0; b < 3; b++) {
	cpc += (c[a]*c[b] - ((a == b) ? 1.0/3.0 : 0.0))*pdev[a][b];
      }
    }
    fc[p*Nc + sc] = (float) (w*(drho + 3.0*cj + 4.5*cpc));
  }
  phic[sc] = (float) phi;
  for (int a = 0; a < 3; a++) uc[a*Nc + sc] = (float) ((double) su*uu[a]);
  rhoc[sc] = (float) rho;
}

/* Fields only: out5 = [phi, u_x, u_y, u_z, rho] of the coarse lattice */
__global__ void k_restrict_fields(lgbk_dims_t df, lgbk_dims_t dc,
				  const float * __restrict__ phif,
				  const float * __restrict__ uf,
				  const float * __restrict__ rhof, float su,
				  float * __restrict__ out5) {
  const long long sc = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (sc >= dc.nsites) return;
  const int zc = (int) (sc % dc.nz);
  const long long r = sc / dc.nz;
  const int yc = (int) (r % dc.ny);
  const int xc = (int) (r / dc.ny);
  const long long Nf = df.nsites, Nc = dc.nsites;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = 0; k < 8; k++) {
    const long long s = lgb_site(df, 2*xc + (k >> 2), 2*yc + ((k >> 1) & 1),
				 2*zc + (k & 1));
    acc[0] += (double) phif[s];
    for (int a = 0; a < 3; a++) acc[1 + a] += (double) uf[a*Nf + s];
    acc[4] += (double) rhof[s];
  }
  out5[sc] = (float) (0.125*acc[0]);
  for (int a = 0; a < 3; a++) {
    out5[(1 + a)*Nc + sc] = (float) ((double) su*0.125*acc[1 + a]);
  }
  out5[4*Nc + sc] = (float) (0.125*acc[4]);
}

static int check_dims(const lgbk_dims_t * df, const lgbk_dims_t * dc) {
  return (df->nx == 2*dc->nx && df->ny == 2*dc->ny && df->nz == 2*dc->nz)
    ? 0 : (int) cudaErrorInvalidValue;
}

extern "C" int lgbk_restrict_state(const lgbk_dims_t * df,
				   const lgbk_dims_t * dc, const float * ff,
				   int pending, const float * phif,
				   const float * uf, double rho0, double su,
				   double sneq, float * fc, float * phic,
				   float * uc, float * rhoc, void * stream) {
  int rc = check_dims(df, dc);
  if (rc) return rc;
  k_restrict_state<<<(unsigned int) ((dc->nsites + 127)/128), 128, 0,
    (cudaStream_t) stream>>>(*df, *dc, ff, pending, phif, uf, (float) rho0,
			     (float) su, (float) sneq, fc, phic, uc, rhoc);
  return (int) cudaGetLastError();
}

extern "C" int lgbk_restrict_fields(const lgbk_dims_t * df,
				    const lgbk_dims_t * dc, const float * phif,
				    const float * uf, const float * rhof,
				    double su, float * out5, void * stream) {
  int rc = check_dims(df, dc);
  if (rc) return rc;
  k_restrict_fields<<<(unsigned int) ((dc->nsites + 255)/256), 256, 0,
    (cudaStream_t) stream>>>(*df, *dc, phif, uf, rhof, (float) su, out5);
  return (int) cudaGetLastError();
}
