/*****************************************************************************
 *
 *  lgb_lc32.cu
 *
 *  Reduced-precision LC step (float arithmetic; distributions stored as
 *  f - w_p rho0 in float or scaled half) and the precision dispatch.
 *
 *****************************************************************************/

#include "lgb_lc.cuh"

#define TPB 128

static dim3 gridn(long long n) {
  return dim3((unsigned int) ((n + TPB - 1)/TPB));
}

template <typename S>
static int lc_step32(const lgbk_dims_t * d, const lgbk_lc_t * p,
		     const lgbk_lc_step_args_t * a, cudaStream_t s) {
  lgbk_lc_f_t pf;
  pf.a0 = (float) p->a0; pf.q0 = (float) p->q0; pf.gamma = (float) p->gamma;
  pf.kappa0 = (float) p->kappa0; pf.kappa1 = (float) p->kappa1;
  pf.xi = (float) p->xi; pf.redshift = (float) p->redshift;
  pf.rredshift = (float) p->rredshift; pf.epsilon = (float) p->epsilon;
  for (int i = 0; i < 3; i++) pf.e0[i] = (float) p->e0[i];
  pf.coswt = (float) p->coswt;
  k_lc_fields<float, lgbk_lc_f_t><<<gridn(d->nsites), TPB, 0, s>>>(
    *d, pf, (const float *) a->q_in, (float *) a->pth, (float *) a->h);
  if (a->status) {
    k_lc_update<float, S, false, true, true>
      <<<gridn(d->nsites), TPB, 0, s>>>(*d, *a);
  }
  else {
    k_lc_update<float, S, false, true, false>
      <<<gridn(d->nsites), TPB, 0, s>>>(*d, *a);
  }
  return (int) cudaGetLastError();
}

extern "C" int lgbk_lc_step(const lgbk_dims_t * d, int prec,
			    const lgbk_lc_t * p, const lgbk_lc_step_args_t * a,
			    void * stream) {
  if (!a->cp.ghosts_zero) return (int) cudaErrorInvalidValue;
  switch (prec) {
  case LGBK_PREC_FP64: return lgbk_lc_step_f64(d, p, a, stream);
  case LGBK_PREC_FP32: return lc_step32<float>(d, p, a, (cudaStream_t) stream);
  case LGBK_PREC_FP16: return lc_step32<__half>(d, p, a, (cudaStream_t) stream);
  default: return (int) cudaErrorInvalidValue;
  }
}
