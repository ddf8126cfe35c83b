/*****************************************************************************
 *
 *  lgb_lb2.cu
 *
 *  The two-distribution binary fluid (symmetric_lb, ndist = 2) in FP64,
 *  compiled with --fmad=false and in the reference's operation order:
 *
 *    k_phi_from_g      phi = sum_p g_p (src/phi_lb_coupler.c:72-93); with
 *                      pending streaming the g_p are pulled, g_p(x - c_p)
 *    k_collide_binary  lb_collision_mrt2_site (src/collision.c:706-1013):
 *                      f relaxes with the chemical stress in the equilibrium
 *                      stress; g is rebuilt from phi, jphi (relaxed at
 *                      rtau2) and sphi = phi u u + mu delta with the sums of
 *                      d3q19_mode2f_phi (src/collision.c:2849-); pulls f and
 *                      g when streaming is pending, writes the
 *                      post-collision values to the other buffers
 *    k_g_from_phi      g_0 = phi, g_p = 0 (src/phi_lb_coupler.c:107-135)
 *
 *****************************************************************************/

#include "lgb_common.cuh"
#include "lgb_kernels.h"

#define TPB 128

static dim3 gridn(long long n) {
  return dim3((unsigned int) ((n + TPB - 1)/TPB));
}

template <bool PULL>
__global__ void k_phi_from_g(lgbk_dims_t d, const double * __restrict__ g,
			     double * __restrict__ phi) {
  const long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const int z = (int) (i % d.nz);
  const long long r = i / d.nz;
  const int y = (int) (r % d.ny);
  const int x = (int) (r / d.ny);
  double phi0 = 0.0;
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) {
    const long long j = PULL ? lgb_site_w(d, x - lgb_cv_c[p][0],
					  y - lgb_cv_c[p][1],
					  z - lgb_cv_c[p][2]) : i;
    phi0 += g[p*d.nsites + j];
  }
  phi[i] = phi0;
}

__global__ void k_g_from_phi(lgbk_dims_t d, const double * __restrict__ phi,
			     double * __restrict__ g) {
  const long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  g[i] = phi[i];
  #pragma unroll
  for (int p = 1; p < LGB_NVEL; p++) g[p*d.nsites + i] = 0.0;
}

template <bool PULL, bool GZERO>
__global__ void k_collide_binary(lgbk_dims_t d, lgbk_symm_t fe,
				 lgbk_collide_t cp, double rtau2,
				 const double * __restrict__ f_in,
				 const double * __restrict__ g_in,
				 const double * __restrict__ phi,
				 const double * __restrict__ grad,
				 const double * __restrict__ delsq,
				 double * __restrict__ f_out,
				 double * __restrict__ g_out,
				 double * __restrict__ u_out) {
  const long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  const int z = (int) (i % d.nz);
  const long long r = i / d.nz;
  const int y = (int) (r % d.ny);
  const int x = (int) (r / d.ny);

  long long src[LGB_NVEL];
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) {
    src[p] = PULL ? lgb_site_w(d, x - lgb_cv_c[p][0], y - lgb_cv_c[p][1],
			       z - lgb_cv_c[p][2]) : i;
  }

  const double ph = phi[i];
  const double gr[3] = {grad[i], grad[N + i], grad[2*N + i]};
  const double dl = delsq[i];

  /* chemical stress (src/symmetric.c:372-400) */
  double sth[3][3];
  {
    const double g2[3] = {gr[0], gr[1], gr[2]};
    const double p0 = lgb_symm_p0<double>(fe, ph, dl, g2);
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      #pragma unroll
      for (int ib = 0; ib < 3; ib++) {
	const double dab = (ia == ib);
	sth[ia][ib] = p0*dab + fe.kappa*gr[ia]*gr[ib];
      }
    }
  }

  double fs[LGB_NVEL];
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) fs[p] = f_in[p*N + src[p]];
  double force[3], rho, u[3];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) force[ia] = cp.force_global[ia] + 0.0;
  lgb_collide_site_sth<double, true, false, GZERO>(
    cp.rtau_shear, cp.rtau_bulk, cp.rtau_ghost, 1.0, fs, force,
    (const double (*)[3]) sth, rho, u);
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) f_out[p*N + i] = fs[p];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) u_out[ia*N + i] = u[ia];

  /* order parameter distribution */
  const double mu = lgb_symm_mu<double>(fe, ph, dl);
  double jphi[3] = {0.0, 0.0, 0.0};
  #pragma unroll
  for (int p = 1; p < LGB_NVEL; p++) {
    const double gp = g_in[p*N + src[p]];
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      if (lgb_cv_c[p][ia]) jphi[ia] += lgb_cv_c[p][ia]*gp;
    }
  }
  double sphi[3][3];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      const double dab = (ia == ib);
      sphi[ia][ib] = ph*u[ia]*u[ib] + mu*dab;
    }
    jphi[ia] = jphi[ia] - rtau2*(jphi[ia] - ph*u[ia]);
  }
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) {
    double jdotc = 0.0, sphidotq = 0.0;
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      if (lgb_cv_c[p][ia] > 0) jdotc += jphi[ia];
      if (lgb_cv_c[p][ia] < 0) jdotc -= jphi[ia];
    }
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      #pragma unroll
      for (int ib = 0; ib < 3; ib++) {
	double qab;
	if (ia == ib) qab = lgb_cv_c[p][ia] ? (2.0/3.0) : -(1.0/3.0);
	else qab = (double) (lgb_cv_c[p][ia]*lgb_cv_c[p][ib]);
	if (qab != 0.0) sphidotq += sphi[ia][ib]*qab;
      }
    }
    double gq = lgb_w(p)*(jdotc*3.0 + sphidotq*4.5);
    if (p == 0) gq = gq + ph;
    g_out[p*N + i] = gq;
  }
}

extern "C" int lgbk_phi_from_g_f64(const lgbk_dims_t * d, int pull,
				   const double * g, double * phi,
				   void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (pull) k_phi_from_g<true><<<gridn(d->nsites), TPB, 0, s>>>(*d, g, phi);
  else      k_phi_from_g<false><<<gridn(d->nsites), TPB, 0, s>>>(*d, g, phi);
  return (int) cudaGetLastError();
}

extern "C" int lgbk_g_from_phi_f64(const lgbk_dims_t * d, const double * phi,
				   double * g, void * stream) {
  k_g_from_phi<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(*d, phi,
								     g);
  return (int) cudaGetLastError();
}

extern "C" int lgbk_collide_binary_f64(const lgbk_dims_t * d,
				       const lgbk_symm_t * fe,
				       const lgbk_collide_t * cp,
				       double mobility, int pull,
				       const double * f_in, const double * g_in,
				       const double * phi, const double * grad,
				       const double * delsq, double * f_out,
				       double * g_out, double * u_out,
				       void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  const double rtau2 = 2.0/(1.0 + 2.0*mobility);
  const dim3 gr = gridn(d->nsites);
#define LGB_CB(P, G) k_collide_binary<P, G><<<gr, TPB, 0, s>>>(*d, *fe, *cp, \
    rtau2, f_in, g_in, phi, grad, delsq, f_out, g_out, u_out)
  if (pull) { if (cp->ghosts_zero) LGB_CB(true, true); else LGB_CB(true, false); }
  else      { if (cp->ghosts_zero) LGB_CB(false, true); else LGB_CB(false, false); }
#undef LGB_CB
  return (int) cudaGetLastError();
}
