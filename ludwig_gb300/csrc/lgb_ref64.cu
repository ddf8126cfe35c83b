/*****************************************************************************
 *
 *  lgb_ref64.cu
 *
 *  FP64 kernels with the reference's per-function semantics, one launch per
 *  reference kernel.  They back the drop-in C API (lb_collide,
 *  lb_propagation, field_grad_compute, phi_force_calculation,
 *  phi_cahn_hilliard) when those are called one by one from a host main
 *  loop.  Each thread handles one site; consecutive threads run along z so
 *  that every component plane is read and written with coalesced accesses.
 *
 *  Compiled with --fmad=false: results equal the reference's serial build
 *  bit for bit (operation order as cited per kernel).
 *
 *****************************************************************************/

#include "lgb_common.cuh"

#define LGB_TPB 256

static inline dim3 grid_for(long long n) {
  return dim3((unsigned int) ((n + LGB_TPB - 1)/LGB_TPB));
}

__device__ __forceinline__ void site_xyz(const lgbk_dims_t & d, long long i,
					 int & x, int & y, int & z) {
  z = (int) (i % d.nz);
  long long r = i / d.nz;
  y = (int) (r % d.ny);
  x = (int) (r / d.ny);
}

/* src/gradient_3d_7pt_fluid.c:231-306 */

__global__ void k_grad7(lgbk_dims_t d, int nf, const double * __restrict__ fld,
			double * __restrict__ grad,
			double * __restrict__ delsq) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const long long N = d.nsites;
  long long xp = lgb_site_w(d, x+1, y, z), xm = lgb_site_w(d, x-1, y, z);
  long long yp = lgb_site_w(d, x, y+1, z), ym = lgb_site_w(d, x, y-1, z);
  long long zp = lgb_site_w(d, x, y, z+1), zm = lgb_site_w(d, x, y, z-1);
  for (int n = 0; n < nf; n++) {
    const double * fn = fld + n*N;
    grad[(3*n + 0)*N + i] = 0.5*(fn[xp] - fn[xm]);
    grad[(3*n + 1)*N + i] = 0.5*(fn[yp] - fn[ym]);
    grad[(3*n + 2)*N + i] = 0.5*(fn[zp] - fn[zm]);
    delsq[n*N + i] = fn[xp] + fn[xm] + fn[yp] + fn[ym] + fn[zp] + fn[zm]
      - 6.0*fn[i];
  }
}

/* src/symmetric.c:372-400 (fe_symm_str_v) */

__global__ void k_symm_stress(lgbk_dims_t d, lgbk_symm_t fe,
			      const double * __restrict__ phi,
			      const double * __restrict__ grad,
			      const double * __restrict__ delsq,
			      double * __restrict__ pth) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double g[3] = {grad[i], grad[N + i], grad[2*N + i]};
  double p0 = lgb_symm_p0<double>(fe, phi[i], delsq[i], g);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      double dab = (ia == ib);
      pth[(3*ia + ib)*N + i] = p0*dab + fe.kappa*g[ia]*g[ib];
    }
  }
}

/* src/symmetric.c:308-320 */

__global__ void k_symm_mu(lgbk_dims_t d, lgbk_symm_t fe,
			  const double * __restrict__ phi,
			  const double * __restrict__ delsq,
			  double * __restrict__ mu) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  mu[i] = lgb_symm_mu<double>(fe, phi[i], delsq[i]);
}

/* src/phi_force_colloid.c:315-467 (pth_force_fluid_kernel_v) */

__global__ void k_force_div(lgbk_dims_t d, const double * __restrict__ pth,
			    double * __restrict__ force) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const long long N = d.nsites;
  const long long nb[6] = {lgb_site_w(d, x+1, y, z), lgb_site_w(d, x-1, y, z),
			   lgb_site_w(d, x, y+1, z), lgb_site_w(d, x, y-1, z),
			   lgb_site_w(d, x, y, z+1), lgb_site_w(d, x, y, z-1)};
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const double * px = pth + (3*ia + 0)*N;
    const double * py = pth + (3*ia + 1)*N;
    const double * pz = pth + (3*ia + 2)*N;
    double fa;
    fa  = -0.5*(px[nb[0]] + px[i]);
    fa +=  0.5*(px[nb[1]] + px[i]);
    fa -=  0.5*(py[nb[2]] + py[i]);
    fa +=  0.5*(py[nb[3]] + py[i]);
    fa -=  0.5*(pz[nb[4]] + pz[i]);
    fa +=  0.5*(pz[nb[5]] + pz[i]);
    force[ia*N + i] += fa*1.0;
  }
}

/* src/advection.c:538-629 (advection_le_1st_kernel, no planes) */

__global__ void k_advect_upwind(lgbk_dims_t d, int nf,
				const double * __restrict__ fld,
				const double * __restrict__ u,
				double * __restrict__ fw,
				double * __restrict__ fe,
				double * __restrict__ fy,
				double * __restrict__ fz) {
  long long i0 = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i0 >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i0, x, y, z);
  const long long N = d.nsites;
  long long i1, idx;
  double uf;

  i1 = lgb_site_w(d, x-1, y, z);
  uf = 0.5*(u[i0] + u[i1]);
  idx = (uf > 0.0) ? i1 : i0;
  for (int n = 0; n < nf; n++) fw[n*N + i0] = uf*fld[n*N + idx];

  i1 = lgb_site_w(d, x+1, y, z);
  uf = 0.5*(u[i0] + u[i1]);
  idx = (uf < 0.0) ? i1 : i0;
  for (int n = 0; n < nf; n++) fe[n*N + i0] = uf*fld[n*N + idx];

  i1 = lgb_site_w(d, x, y+1, z);
  uf = 0.5*(u[N + i0] + u[N + i1]);
  idx = (uf < 0.0) ? i1 : i0;
  for (int n = 0; n < nf; n++) fy[n*N + i0] = uf*fld[n*N + idx];

  i1 = lgb_site_w(d, x, y, z+1);
  uf = 0.5*(u[2*N + i0] + u[2*N + i1]);
  idx = (uf < 0.0) ? i1 : i0;
  for (int n = 0; n < nf; n++) fz[n*N + i0] = uf*fld[n*N + idx];
}

/* src/phi_cahn_hilliard.c:350-404 (phi_ch_flux_mu1_kernel) */

__global__ void k_ch_flux_mu(lgbk_dims_t d, lgbk_symm_t fe, double mobility,
			     const double * __restrict__ phi,
			     const double * __restrict__ delsq,
			     double * __restrict__ fw,
			     double * __restrict__ fe_,
			     double * __restrict__ fy,
			     double * __restrict__ fz) {
  long long i0 = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i0 >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i0, x, y, z);
  long long i1;
  double mu0 = lgb_symm_mu<double>(fe, phi[i0], delsq[i0]);
  double mu1;

  i1 = lgb_site_w(d, x-1, y, z);
  mu1 = lgb_symm_mu<double>(fe, phi[i1], delsq[i1]);
  fw[i0] -= mobility*(mu0 - mu1);

  i1 = lgb_site_w(d, x+1, y, z);
  mu1 = lgb_symm_mu<double>(fe, phi[i1], delsq[i1]);
  fe_[i0] -= mobility*(mu1 - mu0);

  i1 = lgb_site_w(d, x, y+1, z);
  mu1 = lgb_symm_mu<double>(fe, phi[i1], delsq[i1]);
  fy[i0] -= mobility*(mu1 - mu0);

  i1 = lgb_site_w(d, x, y, z+1);
  mu1 = lgb_symm_mu<double>(fe, phi[i1], delsq[i1]);
  fz[i0] -= mobility*(mu1 - mu0);
}

/* src/advection_bcs.c:80-140 (advection_bcs_no_flux_kernel_v) */

__global__ void k_flux_no_normal(lgbk_dims_t d, int nf,
				 const uint8_t * __restrict__ st,
				 double * __restrict__ fw,
				 double * __restrict__ fe,
				 double * __restrict__ fy,
				 double * __restrict__ fz) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const long long N = d.nsites;
  double mask  = (st[i] == 0);
  double maskw = (st[lgb_site_w(d, x-1, y, z)] == 0);
  double maske = (st[lgb_site_w(d, x+1, y, z)] == 0);
  double masky = (st[lgb_site_w(d, x, y+1, z)] == 0);
  double maskz = (st[lgb_site_w(d, x, y, z+1)] == 0);
  for (int n = 0; n < nf; n++) {
    fw[n*N + i] *= mask*maskw;
    fe[n*N + i] *= mask*maske;
    fy[n*N + i] *= mask*masky;
    fz[n*N + i] *= mask*maskz;
  }
}

/* src/phi_cahn_hilliard.c:1018-1049 (phi_ch_ufs_kernel), wz = 1 */

__global__ void k_ch_update(lgbk_dims_t d, const double * __restrict__ fw,
			    const double * __restrict__ fe,
			    const double * __restrict__ fy,
			    const double * __restrict__ fz,
			    double * __restrict__ phi) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const double wz = 1.0;
  phi[i] -= (+ fe[i] - fw[i]
	     + fy[i] - fy[lgb_site_w(d, x, y-1, z)]
	     + wz*fz[i] - wz*fz[lgb_site_w(d, x, y, z-1)]);
}

/* src/collision.c:221-593 (lb_collision_mrt1 / _site).  With PULL the
 * input holds post-collision values whose streaming is still pending: each
 * population is pulled from its upstream site (the permutation of
 * src/propagation.c:153-197) and the result goes to a second array, so
 * that lb_propagation followed by lb_collide reads and writes f once.
 * Solid sites keep their (streamed) populations. */

template <bool GZERO, bool PULL>
__global__ void k_collide(lgbk_dims_t d, lgbk_collide_t cp,
			  const uint8_t * __restrict__ st,
			  const double * fin, double * fout,
			  const double * __restrict__ force,
			  double * __restrict__ rho, double * __restrict__ u) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double fs[LGB_NVEL], fa[3], uu[3], r;
  if (PULL) {
    int x, y, z;
    site_xyz(d, i, x, y, z);
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) {
      long long j = lgb_site_w(d, x - lgb_cv_c[p][0], y - lgb_cv_c[p][1],
			       z - lgb_cv_c[p][2]);
      fs[p] = fin[p*N + j];
    }
  }
  else {
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) fs[p] = fin[p*N + i];
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    fa[ia] = cp.force_global[ia] + (force ? force[ia*N + i] : 0.0);
  }
  const bool fluid = (st == NULL || st[i] == 0);
  if (PULL && !fluid) {
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) fout[p*N + i] = fs[p];
    return;
  }
  lgb_collide_site<double, true, false, GZERO>(cp, 0.0, fs, fa, r, uu);
  if (fluid) {
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) fout[p*N + i] = fs[p];
    rho[i] = r;
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) u[ia*N + i] = uu[ia];
  }
}

/* src/propagation.c:153-197 (pull); dir = -1 gives the inverse shift. */

__global__ void k_propagate(lgbk_dims_t d, int dir,
			    const double * __restrict__ f,
			    double * __restrict__ fp) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const long long N = d.nsites;
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) {
    long long j = lgb_site_w(d, x - dir*lgb_cv_c[p][0], y - dir*lgb_cv_c[p][1],
			     z - dir*lgb_cv_c[p][2]);
    fp[p*N + i] = f[p*N + j];
  }
}

__global__ void k_fill(double * a, long long n, double v) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

/* 2nd-order (centred) advective fluxes, src/advection.c:770-900, in the
 * reference's operation order (the face mask is 1 on a periodic box) */
__global__ void k_advect_2nd(lgbk_dims_t d, int nf,
			     const double * __restrict__ fld,
			     const double * __restrict__ u,
			     double * __restrict__ fw, double * __restrict__ fe,
			     double * __restrict__ fy, double * __restrict__ fz) {
  long long i0 = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i0 >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i0, x, y, z);
  const long long N = d.nsites;
  const double mask = 1.0;
  long long i1 = lgb_site_w(d, x-1, y, z);
  for (int n = 0; n < nf; n++) {
    fw[n*N + i0] = 0.5*(u[i0] + u[i1])*mask*0.5*(fld[n*N + i1] + fld[n*N + i0]);
  }
  i1 = lgb_site_w(d, x+1, y, z);
  for (int n = 0; n < nf; n++) {
    fe[n*N + i0] = 0.5*(u[i0] + u[i1])*mask*0.5*(fld[n*N + i0] + fld[n*N + i1]);
  }
  i1 = lgb_site_w(d, x, y+1, z);
  for (int n = 0; n < nf; n++) {
    fy[n*N + i0] = 0.5*(u[N + i0] + u[N + i1])*mask*0.5
      *(fld[n*N + i0] + fld[n*N + i1]);
  }
  i1 = lgb_site_w(d, x, y, z+1);
  for (int n = 0; n < nf; n++) {
    fz[n*N + i0] = 0.5*(u[2*N + i0] + u[2*N + i1])*mask*0.5
      *(fld[n*N + i0] + fld[n*N + i1]);
  }
}

/* 3rd-order upwind-biased fluxes, src/advection.c:946-1135: the face value
 * a1 f(two upwind) + a2 f(upwind) + a3 f(downwind) */
__global__ void k_advect_3rd(lgbk_dims_t d, int nf,
			     const double * __restrict__ fld,
			     const double * __restrict__ u,
			     double * __restrict__ fw, double * __restrict__ fe,
			     double * __restrict__ fy, double * __restrict__ fz) {
  long long i0 = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i0 >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i0, x, y, z);
  const long long N = d.nsites;
  const double a1 = -0.213933, a2 = 0.927865, a3 = 0.286067;
  const double mask = 1.0;
  {
    const long long m2 = lgb_site_w(d, x-2, y, z), m1 = lgb_site_w(d, x-1, y, z);
    const long long p1 = lgb_site_w(d, x+1, y, z), p2 = lgb_site_w(d, x+2, y, z);
    double uf = 0.5*mask*(u[i0] + u[m1]);
    for (int n = 0; n < nf; n++) {
      const double * f = fld + n*N;
      double d1, d2, d3;
      if (uf > 0.0) { d1 = f[m2]; d2 = f[m1]; d3 = f[i0]; }
      else          { d1 = f[p1]; d2 = f[i0]; d3 = f[m1]; }
      fw[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
    }
    uf = 0.5*mask*(u[i0] + u[p1]);
    for (int n = 0; n < nf; n++) {
      const double * f = fld + n*N;
      double d1, d2, d3;
      if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
      else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
      fe[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
    }
  }
  {
    const long long m1 = lgb_site_w(d, x, y-1, z), p1 = lgb_site_w(d, x, y+1, z);
    const long long p2 = lgb_site_w(d, x, y+2, z);
    const double uf = 0.5*mask*(u[N + i0] + u[N + p1]);
    for (int n = 0; n < nf; n++) {
      const double * f = fld + n*N;
      double d1, d2, d3;
      if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
      else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
      fy[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
    }
  }
  {
    const long long m1 = lgb_site_w(d, x, y, z-1), p1 = lgb_site_w(d, x, y, z+1);
    const long long p2 = lgb_site_w(d, x, y, z+2);
    const double uf = 0.5*mask*(u[2*N + i0] + u[2*N + p1]);
    for (int n = 0; n < nf; n++) {
      const double * f = fld + n*N;
      double d1, d2, d3;
      if (uf < 0.0) { d1 = f[p2]; d2 = f[p1]; d3 = f[i0]; }
      else          { d1 = f[m1]; d2 = f[i0]; d3 = f[p1]; }
      fz[n*N + i0] = uf*(a1*d1 + a2*d2 + a3*d3);
    }
  }
}

/*****************************************************************************
 *
 *  Launchers
 *
 *****************************************************************************/

#define LAUNCH_RET return (int) cudaGetLastError()

extern "C" {

/* 27-point gradient and Laplacian (src/gradient_3d_27pt_fluid.c:219-362):
 * (0.5/9) times the sum over the nine neighbour pairs of the +1 / -1
 * planes, and (1/9)(sum of the 26 neighbours - 26 f), in the reference's
 * order of terms. */
__global__ void k_grad27(lgbk_dims_t d, int nf, const double * __restrict__ fld,
			 double * __restrict__ grad,
			 double * __restrict__ delsq) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int x, y, z;
  site_xyz(d, i, x, y, z);
  const long long N = d.nsites;
  const double r9 = (1.0/9.0);
  long long nb[3][3][3];
  #pragma unroll
  for (int a = 0; a < 3; a++)
    #pragma unroll
    for (int b = 0; b < 3; b++)
      #pragma unroll
      for (int c = 0; c < 3; c++)
	nb[a][b][c] = lgb_site_w(d, x + a - 1, y + b - 1, z + c - 1);
  for (int n = 0; n < nf; n++) {
    const double * fn = fld + n*N;
    double sx = 0.0, sy = 0.0, sz = 0.0, sl = 0.0;
    #pragma unroll
    for (int a = 0; a < 3; a++) {
      #pragma unroll
      for (int b = 0; b < 3; b++) {
	if (a == 0 && b == 0) sx = +fn[nb[2][a][b]];
	else sx = sx + fn[nb[2][a][b]];
	sx = sx - fn[nb[0][a][b]];
	if (a == 0 && b == 0) sy = +fn[nb[a][2][b]];
	else sy = sy + fn[nb[a][2][b]];
	sy = sy - fn[nb[a][0][b]];
	if (a == 0 && b == 0) sz = +fn[nb[a][b][2]];
	else sz = sz + fn[nb[a][b][2]];
	sz = sz - fn[nb[a][b][0]];
      }
    }
    bool first = true;
    #pragma unroll
    for (int a = 0; a < 3; a++) {
      #pragma unroll
      for (int b = 0; b < 3; b++) {
	#pragma unroll
	for (int c = 0; c < 3; c++) {
	  if (a == 1 && b == 1 && c == 1) continue;
	  if (first) sl = +fn[nb[a][b][c]];
	  else sl = sl + fn[nb[a][b][c]];
	  first = false;
	}
      }
    }
    sl = sl - 26.0*fn[i];
    grad[(3*n + 0)*N + i] = 0.5*r9*sx;
    grad[(3*n + 1)*N + i] = 0.5*r9*sy;
    grad[(3*n + 2)*N + i] = 0.5*r9*sz;
    delsq[n*N + i] = r9*sl;
  }
}

int lgbk_grad27_f64(const lgbk_dims_t * d, int nf, const double * field,
		    double * grad, double * delsq, void * stream) {
  k_grad27<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, nf, field, grad, delsq);
  return (int) cudaGetLastError();
}

int lgbk_grad7_f64(const lgbk_dims_t * d, int nf, const double * field,
		   double * grad, double * delsq, void * stream) {
  k_grad7<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, nf, field, grad, delsq);
  LAUNCH_RET;
}

int lgbk_symm_stress_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			 const double * phi, const double * grad,
			 const double * delsq, double * pth, void * stream) {
  k_symm_stress<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, *fe, phi, grad, delsq, pth);
  LAUNCH_RET;
}

int lgbk_symm_mu_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
		     const double * phi, const double * delsq, double * mu,
		     void * stream) {
  k_symm_mu<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, *fe, phi, delsq, mu);
  LAUNCH_RET;
}

int lgbk_force_div_f64(const lgbk_dims_t * d, const double * pth,
		       double * force, void * stream) {
  k_force_div<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, pth, force);
  LAUNCH_RET;
}

/* order 1 (upwind), 2 (centred) or 3 (upwind-biased) */
int lgbk_advect_f64(const lgbk_dims_t * d, int order, int nf,
		    const double * field, const double * u, double * fw,
		    double * fe, double * fy, double * fz, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (order == 2) {
    k_advect_2nd<<<grid_for(d->nsites), LGB_TPB, 0, s>>>(*d, nf, field, u,
							 fw, fe, fy, fz);
  }
  else if (order == 3) {
    k_advect_3rd<<<grid_for(d->nsites), LGB_TPB, 0, s>>>(*d, nf, field, u,
							 fw, fe, fy, fz);
  }
  else {
    k_advect_upwind<<<grid_for(d->nsites), LGB_TPB, 0, s>>>(*d, nf, field, u,
							    fw, fe, fy, fz);
  }
  LAUNCH_RET;
}

int lgbk_advect_upwind_f64(const lgbk_dims_t * d, int nf,
			   const double * field, const double * u,
			   double * fw, double * fe, double * fy, double * fz,
			   void * stream) {
  k_advect_upwind<<<grid_for(d->nsites), LGB_TPB, 0,
    (cudaStream_t) stream>>>(*d, nf, field, u, fw, fe, fy, fz);
  LAUNCH_RET;
}

int lgbk_ch_flux_mu_f64(const lgbk_dims_t * d, const lgbk_symm_t * fe,
			double mobility, const double * phi,
			const double * delsq, double * fw, double * fe_,
			double * fy, double * fz, void * stream) {
  k_ch_flux_mu<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, *fe, mobility, phi, delsq, fw, fe_, fy, fz);
  LAUNCH_RET;
}

int lgbk_flux_no_normal_f64(const lgbk_dims_t * d, int nf,
			    const uint8_t * status, double * fw, double * fe,
			    double * fy, double * fz, void * stream) {
  if (status == NULL) return 0;
  k_flux_no_normal<<<grid_for(d->nsites), LGB_TPB, 0,
    (cudaStream_t) stream>>>(*d, nf, status, fw, fe, fy, fz);
  LAUNCH_RET;
}

int lgbk_ch_update_f64(const lgbk_dims_t * d, const double * fw,
		       const double * fe, const double * fy, const double * fz,
		       double * phi, void * stream) {
  k_ch_update<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, fw, fe, fy, fz, phi);
  LAUNCH_RET;
}

int lgbk_collide_f64(const lgbk_dims_t * d, const lgbk_collide_t * cp,
		     const uint8_t * status, double * f, const double * force,
		     double * rho, double * u, void * stream) {
  if (cp->ghosts_zero) {
    k_collide<true, false><<<grid_for(d->nsites), LGB_TPB, 0,
      (cudaStream_t) stream>>>(*d, *cp, status, f, f, force, rho, u);
  }
  else {
    k_collide<false, false><<<grid_for(d->nsites), LGB_TPB, 0,
      (cudaStream_t) stream>>>(*d, *cp, status, f, f, force, rho, u);
  }
  LAUNCH_RET;
}

int lgbk_collide_pull_f64(const lgbk_dims_t * d, const lgbk_collide_t * cp,
			  const uint8_t * status, const double * fpost,
			  double * fout, const double * force, double * rho,
			  double * u, void * stream) {
  if (cp->ghosts_zero) {
    k_collide<true, true><<<grid_for(d->nsites), LGB_TPB, 0,
      (cudaStream_t) stream>>>(*d, *cp, status, fpost, fout, force, rho, u);
  }
  else {
    k_collide<false, true><<<grid_for(d->nsites), LGB_TPB, 0,
      (cudaStream_t) stream>>>(*d, *cp, status, fpost, fout, force, rho, u);
  }
  LAUNCH_RET;
}

int lgbk_propagate_f64(const lgbk_dims_t * d, int dir, const double * f,
		       double * fprime, void * stream) {
  k_propagate<<<grid_for(d->nsites), LGB_TPB, 0, (cudaStream_t) stream>>>(
    *d, dir, f, fprime);
  LAUNCH_RET;
}

int lgbk_fill_f64(double * a, long long n, double v, void * stream) {
  if (n <= 0) return 0;
  k_fill<<<grid_for(n), LGB_TPB, 0, (cudaStream_t) stream>>>(a, n, v);
  LAUNCH_RET;
}

}
