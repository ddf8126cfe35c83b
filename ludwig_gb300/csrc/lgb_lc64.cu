/*****************************************************************************
 *
 *  lgb_lc64.cu
 *
 *  FP64 kernels of the cholesteric liquid crystal with the reference's
 *  per-function semantics (compiled with --fmad=false):
 *    k_lc_stress : H and the chiral stress on every site (pth_kernel_v with
 *                  fe_lc_stress_v, src/phi_force_stress.c:256)
 *    k_lc_h      : H on every site (beris_edw_h_kernel_v,
 *                  src/blue_phase_beris_edwards.c:942)
 *    k_be_update : the Beris-Edwards site update (beris_edw_kernel_v,
 *                  src/blue_phase_beris_edwards.c:538-840), in place
 *    k_lc_fed    : free-energy density (fe_lc_fed, src/blue_phase.c:284)
 *
 *****************************************************************************/

#include "lgb_lc.cuh"
#include "lgb_lc.h"

#define TPB 128

static dim3 gridn(long long n) {
  return dim3((unsigned int) ((n + TPB - 1)/TPB));
}

__global__ void k_lc_stress(lgbk_dims_t d, lgbk_lc_t p,
			    const double * __restrict__ q,
			    const double * __restrict__ grad,
			    const double * __restrict__ delsq,
			    double * __restrict__ pth) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double qs[3][3], dq[3][3][3], dsq[3][3], h[3][3], s[3][3];
  lc_expand(q, N, i, qs);
  lc_expand_grad(grad, N, i, dq);
  lc_expand(delsq, N, i, dsq);
  lc_h_site<double>(p, qs, dq, dsq, h);
  lc_stress_site<double>(p, qs, dq, h, s);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) pth[(3*ia + ib)*N + i] = s[ia][ib];
}

__global__ void k_lc_h(lgbk_dims_t d, lgbk_lc_t p,
		       const double * __restrict__ q,
		       const double * __restrict__ grad,
		       const double * __restrict__ delsq,
		       double * __restrict__ h5) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double qs[3][3], dq[3][3][3], dsq[3][3], h[3][3];
  lc_expand(q, N, i, qs);
  lc_expand_grad(grad, N, i, dq);
  lc_expand(delsq, N, i, dsq);
  lc_h_site<double>(p, qs, dq, dsq, h);
  h5[0*N + i] = h[0][0]; h5[1*N + i] = h[0][1]; h5[2*N + i] = h[0][2];
  h5[3*N + i] = h[1][1]; h5[4*N + i] = h[1][2];
}

__global__ void k_lc_fed(lgbk_dims_t d, lgbk_lc_t p,
			 const double * __restrict__ q,
			 const double * __restrict__ grad,
			 double * __restrict__ fed) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double qs[3][3], dq[3][3][3];
  lc_expand(q, N, i, qs);
  lc_expand_grad(grad, N, i, dq);
  fed[i] = lc_fed_site<double>(p, qs, dq);
}

/* fed, bulk and gradient parts in three columns (the statistics of
 * fe_lc_stats_info, src/fe_lc_stats.c:55-150) */
__global__ void k_lc_fbg(lgbk_dims_t d, lgbk_lc_t p,
			 const double * __restrict__ q,
			 const double * __restrict__ grad,
			 double * __restrict__ out) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  double qs[3][3], dq[3][3][3], fb, fg;
  lc_expand(q, N, i, qs);
  lc_expand_grad(grad, N, i, dq);
  out[i] = lc_fed_site<double>(p, qs, dq);
  lc_fbg_site<double>(p, qs, dq, fb, fg);
  out[N + i] = fb;
  out[2*N + i] = fg;
}

/* u and the fluxes may be NULL (no hydrodynamics: zero fluxes, no S) */
__global__ void k_be_update(lgbk_dims_t d, double xi, double gamma_rot,
			    const uint8_t * __restrict__ st,
			    const double * __restrict__ u,
			    const double * __restrict__ fw,
			    const double * __restrict__ fe,
			    const double * __restrict__ fy,
			    const double * __restrict__ fz,
			    const double * __restrict__ h5,
			    double * __restrict__ q) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  if (st && st[i] != 0) return;                       /* fluid sites only */

  const long long N = d.nsites;
  const double r3 = (1.0/3.0);
  const double dt = 1.0;
  int z = (int) (i % d.nz);
  long long r = i / d.nz;
  int y = (int) (r % d.ny);
  int x = (int) (r / d.ny);

  double qs[3][3], s[3][3];
  lc_expand(q, N, i, qs);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) s[ia][ib] = 0.0;

  if (u) {
    double w[3][3], dd[3][3], om[3][3];
    long long im, ip;
    im = lgb_site_w(d, x-1, y, z); ip = lgb_site_w(d, x+1, y, z);
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) w[ia][0] = 0.5*(u[ia*N + ip] - u[ia*N + im]);
    im = lgb_site_w(d, x, y-1, z); ip = lgb_site_w(d, x, y+1, z);
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) w[ia][1] = 0.5*(u[ia*N + ip] - u[ia*N + im]);
    im = lgb_site_w(d, x, y, z-1); ip = lgb_site_w(d, x, y, z+1);
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) w[ia][2] = 0.5*(u[ia*N + ip] - u[ia*N + im]);

    double tr = r3*(w[0][0] + w[1][1] + w[2][2]);
    w[0][0] -= tr; w[1][1] -= tr; w[2][2] -= tr;

    double trace_qw = 0.0;
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      #pragma unroll
      for (int ib = 0; ib < 3; ib++) {
	trace_qw += qs[ia][ib]*w[ib][ia];
	dd[ia][ib] = 0.5*(w[ia][ib] + w[ib][ia]);
	om[ia][ib] = 0.5*(w[ia][ib] - w[ib][ia]);
      }
    }
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      #pragma unroll
      for (int ib = 0; ib < 3; ib++) {
	const double dab = (ia == ib);
	s[ia][ib] = -2.0*xi*(qs[ia][ib] + r3*dab)*trace_qw;
	#pragma unroll
	for (int id = 0; id < 3; id++) {
	  const double ddb = (id == ib), dad = (ia == id);
	  s[ia][ib] += (xi*dd[ia][id] + om[ia][id])*(qs[id][ib] + r3*ddb)
	    + (qs[ia][id] + r3*dad)*(xi*dd[id][ib] - om[id][ib]);
	}
      }
    }
  }

  const long long ij = lgb_site_w(d, x, y-1, z), ik = lgb_site_w(d, x, y, z-1);
  const int ca[5] = {0, 0, 0, 1, 1};
  const int cb[5] = {0, 1, 2, 1, 2};
  #pragma unroll
  for (int n = 0; n < 5; n++) {
    const double fen = u ? fe[n*N + i] : 0.0, fwn = u ? fw[n*N + i] : 0.0;
    const double fyn = u ? fy[n*N + i] : 0.0, fyj = u ? fy[n*N + ij] : 0.0;
    const double fzn = u ? fz[n*N + i] : 0.0, fzk = u ? fz[n*N + ik] : 0.0;
    double v = qs[ca[n]][cb[n]];
    v += dt*(s[ca[n]][cb[n]] + 0.0 + gamma_rot*h5[n*N + i]
	     - fen + fwn - fyn + fyj - fzn + fzk);
    q[n*N + i] = v;
  }
}

extern "C" {

int lgbk_lc_stress_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		       const double * q, const double * grad,
		       const double * delsq, double * pth, void * stream) {
  k_lc_stress<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(
    *d, *p, q, grad, delsq, pth);
  return (int) cudaGetLastError();
}

int lgbk_lc_h_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		  const double * q, const double * grad, const double * delsq,
		  double * h, void * stream) {
  k_lc_h<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(
    *d, *p, q, grad, delsq, h);
  return (int) cudaGetLastError();
}

int lgbk_lc_fed_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		    const double * q, const double * grad, double * fed,
		    void * stream) {
  k_lc_fed<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(
    *d, *p, q, grad, fed);
  return (int) cudaGetLastError();
}

int lgbk_lc_fbg_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
		    const double * q, const double * grad, double * out,
		    void * stream) {
  k_lc_fbg<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(
    *d, *p, q, grad, out);
  return (int) cudaGetLastError();
}

int lgbk_be_update_f64(const lgbk_dims_t * d, double xi, double gamma_rot,
		       const uint8_t * status, const double * u,
		       const double * flux, const double * h, double * q,
		       void * stream) {
  const long long N5 = 5*d->nsites;
  const double * fw = flux, * fe = flux ? flux + N5 : NULL;
  const double * fy = flux ? flux + 2*N5 : NULL;
  const double * fz = flux ? flux + 3*N5 : NULL;
  k_be_update<<<gridn(d->nsites), TPB, 0, (cudaStream_t) stream>>>(
    *d, xi, gamma_rot, status, u, fw, fe, fy, fz, h, q);
  return (int) cudaGetLastError();
}

}

extern "C" int lgbk_lc_step_f64(const lgbk_dims_t * d, const lgbk_lc_t * p,
				const lgbk_lc_step_args_t * a, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  k_lc_fields<double, lgbk_lc_t><<<gridn(d->nsites), TPB, 0, s>>>(
    *d, *p, (const double *) a->q_in, (double *) a->pth, (double *) a->h);
  if (a->status) {
    k_lc_update<double, double, true, false, true>
      <<<gridn(d->nsites), TPB, 0, s>>>(*d, *a);
  }
  else {
    k_lc_update<double, double, true, false, false>
      <<<gridn(d->nsites), TPB, 0, s>>>(*d, *a);
  }
  return (int) cudaGetLastError();
}
