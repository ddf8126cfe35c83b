/*****************************************************************************
 *
 *  lgb_lc32.cu
 *
 *  Reduced-precision LC step (float arithmetic; distributions stored as
 *  f - w_p rho0 in float or scaled half) and the precision dispatch.
 *
 *****************************************************************************/

#include "lgb_lc32.cuh"
#include "lgb_lc32_2.cuh"

/* Tile of the force + collision kernel on a plane ring (status maps, and
 * all-fluid lattices on request) and resident CTAs per SM */
#define LC32_TY 8
#define LC32_MINB 2

template <typename S, bool HAS_MAP>
static int launch_collide(const lgbk_dims_t * d, const lgbk_lc_step_args_t * a,
			  cudaStream_t s) {
  auto kern = k_lc32_collide<S, HAS_MAP, LC32_TY, LC32_MINB>;
  const size_t smem = LcCollideSmem<LC32_TY>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*LC32_TY, smem);
  if (occ < 1) occ = 1;
  const int ntz = (d->nz + 31)/32, nty = (d->ny + LC32_TY - 1)/LC32_TY;
  long long grid = (long long) nsm*occ;
  /* about 1.5 items per CTA (16 planes at 128^3: 0.170 ms per LC step,
   * against 0.177 ms with 13-plane chunks) */
  const int xchunk = lgbk_auto_xchunk(0, d->nx, ntz*nty, grid, 3);
  const long long items = (long long) ntz*nty*((d->nx + xchunk - 1)/xchunk);
  if (grid > items) grid = items;
  kern<<<(unsigned int) grid, dim3(32, LC32_TY), smem, s>>>(*d, *a, xchunk);
  return (int) cudaGetLastError();
}

/* Force + collision without a plane ring (all-fluid lattices, the
 * default): blocks of 32 x LC32_DTY sites, a cap of LC32_DMINB blocks'
 * registers (56 used).  LC step at 128^3: 0.1445 ms against 0.162 with
 * the ring kernel; 32 x 2, 32 x 4 with caps 4 and 8, 32 x 8 within 1 %. */
#define LC32_DTY 4
#define LC32_DMINB 4

template <typename S>
static int launch_collide_direct(const lgbk_dims_t * d,
				 const lgbk_lc_step_args_t * a,
				 cudaStream_t s) {
  const dim3 grid((unsigned int) (((d->nz + 31)/32)
				  *((d->ny + LC32_DTY - 1)/LC32_DTY)),
		  (unsigned int) d->nx);
  k_lc32_collide_direct<S, LC32_DTY, LC32_DMINB><<<grid, dim3(32, LC32_DTY),
    0, s>>>(*d, *a);
  return (int) cudaGetLastError();
}

/* The same with two sites per thread (tiles of 2 TYT rows) */
template <typename S, int TYT, int MINB>
static int launch_collide2(const lgbk_dims_t * d,
			   const lgbk_lc_step_args_t * a, cudaStream_t s) {
  auto kern = k_lc32_collide2<S, TYT, MINB>;
  const size_t smem = LcCollideSmem<2*TYT>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TYT, smem);
  if (occ < 1) occ = 1;
  const int ntz = (d->nz + 31)/32, nty = (d->ny + 2*TYT - 1)/(2*TYT);
  long long grid = (long long) nsm*occ;
  const int xchunk = lgbk_auto_xchunk(0, d->nx, ntz*nty, grid, 3);
  const long long items = (long long) ntz*nty*((d->nx + xchunk - 1)/xchunk);
  if (grid > items) grid = items;
  kern<<<(unsigned int) grid, dim3(32, TYT), smem, s>>>(*d, *a, xchunk);
  return (int) cudaGetLastError();
}

/* Fields + Beris-Edwards with two sites per thread (tiles of 2 LC32_F2Y
 * rows, LC32_F2MINB blocks per SM; 168 registers and a few spilled).
 * Measured LC step at 128^3 with this kernel and the one-site collision:
 * (F2Y, blocks/SM) (2, 5) 0.1725 ms, (2, 4) 0.179 (238 registers, no
 * spills), (1, 8) 0.178, (4, 2) 0.179, against 0.160 with the one-site
 * kernel: the pair's registers cut the resident warps from 20 to 8-10 per
 * SM, which costs more latency hiding than the packed arithmetic saves. */
#define LC32_F2Y 2
#define LC32_F2MINB 5

static int launch_fields2(const lgbk_dims_t * d, const lgbk_lc_f_t * pf,
			  const lgbk_lc_step_args_t * a, cudaStream_t s) {
  const dim3 grid((unsigned int) (((d->nz + 31)/32)
				  *((d->ny + 2*LC32_F2Y - 1)/(2*LC32_F2Y))),
		  (unsigned int) d->nx);
  k_lc32_fields_be2<LC32_F2Y, LC32_F2MINB><<<grid, dim3(32, LC32_F2Y), 0, s>>>(
    *d, *pf, *a);
  return (int) cudaGetLastError();
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
  const dim3 fgrid((unsigned int) (((d->nz + 31)/32)
				   *((d->ny + LC32_FY - 1)/LC32_FY)),
		    (unsigned int) d->nx);
  const dim3 fblock(32, LC32_FY);
  cudaError_t err = cudaSuccess;
  if (a->status) {
    k_lc32_fields_be<true><<<fgrid, fblock, 0, s>>>(*d, pf, *a);
    err = cudaGetLastError();
  }
  else if (a->sites == 2) {
    err = (cudaError_t) launch_fields2(d, &pf, a, s);
  }
  else {
    k_lc32_fields_be<false><<<fgrid, fblock, 0, s>>>(*d, pf, *a);
    err = cudaGetLastError();
  }
  if (err != cudaSuccess) return (int) err;
  if (a->status) return launch_collide<S, true>(d, a, s);
  /* two sites per thread only when asked for: at 128^3 the one-site
   * kernels are the faster (0.161 against 0.171 ms per LC step with the
   * two-site collision, FP32); sites = 1 asks for the ring kernel */
  if (a->sites == 2) return launch_collide2<S, 4, 3>(d, a, s);
  if (a->sites == 1) return launch_collide<S, false>(d, a, s);
  return launch_collide_direct<S>(d, a, s);
}

extern "C" int lgbk_lc_step(const lgbk_dims_t * d, int prec,
			    const lgbk_lc_t * p, const lgbk_lc_step_args_t * a,
			    void * stream) {
  if (!a->cp.ghosts_zero) return (int) cudaErrorInvalidValue;
  if (d->nsites >= LGBK_MAX_SITES) return (int) cudaErrorInvalidValue;
  switch (prec) {
  case LGBK_PREC_FP64: return lgbk_lc_step_f64(d, p, a, stream);
  case LGBK_PREC_FP32: return lc_step32<float>(d, p, a, (cudaStream_t) stream);
  case LGBK_PREC_FP16: return lc_step32<__half>(d, p, a, (cudaStream_t) stream);
  default: return (int) cudaErrorInvalidValue;
  }
}
