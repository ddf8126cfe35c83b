/*****************************************************************************
 *
 *  lgb_fused32.cu
 *
 *  Reduced-precision forms of the fused binary-fluid step:
 *    FP32: float arithmetic; distributions stored as f - w_p rho0 (float)
 *    FP16: float arithmetic; (f - w_p rho0)*scale stored as half
 *  phi, u and rho are float in both.  Also the conversions between the
 *  FP64 canonical arrays and these storage forms, and streaming of stored
 *  distributions.
 *
 *****************************************************************************/

#include <cstring>

#include "lgb_fused.cuh"
#include "lgb_fused2.cuh"

extern "C" int lgbk_binary_step_f64(const lgbk_dims_t * d,
				    const lgbk_binary_args_t * a, int xchunk,
				    int ty, void * stream);
extern "C" int lgbk_ensemble_step_f64(const lgbk_box_t * boxes,
				      const void * items, int nitems,
				      int xchunk, int has_map, int * sched,
				      void * stream);

template <typename S, bool HAS_MAP, int TY, int MINB>
static int launch32(const lgbk_dims_t * d, const lgbk_binary_args_t * a,
		    int xchunk, cudaStream_t stream) {
  auto kern = k_binary_fused<float, S, false, true, true, HAS_MAP, TY, MINB>;
  size_t smem = FusedSmem<float, TY>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;

  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TY, smem);
  if (occ < 1) occ = 1;

  int ntz = (d->nz + 31)/32, nty = (d->ny + TY - 1)/TY;
  long long grid = (long long) nsm*occ;
  xchunk = lgbk_auto_xchunk(xchunk, d->nx, ntz*nty, grid);
  long long items = (long long) ntz*nty*((d->nx + xchunk - 1)/xchunk);
  if (grid > items) grid = items;

  kern<<<(unsigned int) grid, dim3(32, TY), smem, stream>>>(*d, *a, xchunk);
  return (int) cudaGetLastError();
}

/* Two sites per thread (packed FP32x2): TYT x 32 threads, tiles of 2 TYT
 * rows, MINB resident CTAs per SM */
template <typename S, int TYT, int MINB>
static int launch32_two(const lgbk_dims_t * d, const lgbk_binary_args_t * a,
			int xchunk, cudaStream_t stream) {
  auto kern = k_binary_fused2<S, TYT, MINB>;
  size_t smem = FusedSmem<float, 2*TYT>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;

  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TYT, smem);
  if (occ < 1) occ = 1;

  int ntz = (d->nz + 31)/32, nty = (d->ny + 2*TYT - 1)/(2*TYT);
  long long grid = (long long) nsm*occ;
  xchunk = lgbk_auto_xchunk(xchunk, d->nx, ntz*nty, grid);
  long long items = (long long) ntz*nty*((d->nx + xchunk - 1)/xchunk);
  if (grid > items) grid = items;

  kern<<<(unsigned int) grid, dim3(32, TYT), smem, stream>>>(*d, *a, xchunk);
  return (int) cudaGetLastError();
}

/* Tile height and resident CTAs per SM (register cap 65536/(32*TY*MINB)):
 * (8,4) and (16,2) and (4,8) cap at 64 registers, (8,3) at 85, (8,2) at 128.
 * minb = 0 picks the default for the tile height. */
template <typename S>
static int dispatch32(const lgbk_dims_t * d, const lgbk_binary_args_t * a,
		      int xchunk, int ty, int minb, int sites,
		      cudaStream_t s) {
  const bool m = (a->status != NULL);
  if (sites == 2 && !m) {
    /* tile rows 8 (4 thread rows) or 16 (8 thread rows) */
    if (ty == 16) return launch32_two<S, 8, 2>(d, a, xchunk, s);
    if (minb == 2) return launch32_two<S, 4, 2>(d, a, xchunk, s);
    if (minb == 4) return launch32_two<S, 4, 4>(d, a, xchunk, s);
    return launch32_two<S, 4, 3>(d, a, xchunk, s);
  }
  if (ty == 4) {
    return m ? launch32<S, true, 4, 8>(d, a, xchunk, s)
             : launch32<S, false, 4, 8>(d, a, xchunk, s);
  }
  if (ty == 16) {
    return m ? launch32<S, true, 16, 2>(d, a, xchunk, s)
             : launch32<S, false, 16, 2>(d, a, xchunk, s);
  }
  if (minb == 2) {
    return m ? launch32<S, true, 8, 2>(d, a, xchunk, s)
             : launch32<S, false, 8, 2>(d, a, xchunk, s);
  }
  if (minb == 3) {
    return m ? launch32<S, true, 8, 3>(d, a, xchunk, s)
             : launch32<S, false, 8, 3>(d, a, xchunk, s);
  }
  return m ? launch32<S, true, 8, 4>(d, a, xchunk, s)
           : launch32<S, false, 8, 4>(d, a, xchunk, s);
}

extern "C" int lgbk_binary_step(const lgbk_dims_t * d, int prec,
				const lgbk_binary_args_t * a, int xchunk,
				int ty, int minb, int sites, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (ty <= 0) ty = 8;
  if (d->nsites >= LGBK_MAX_SITES) return (int) cudaErrorInvalidValue;
  switch (prec) {
  case LGBK_PREC_FP64:
    return lgbk_binary_step_f64(d, a, xchunk, ty, stream);
  case LGBK_PREC_FP32:
    if (!a->cp.ghosts_zero) return (int) cudaErrorInvalidValue;
    return dispatch32<float>(d, a, xchunk, ty, minb, (sites == 2) ? 2 : 1,
			     s);
  case LGBK_PREC_FP16:
    if (!a->cp.ghosts_zero) return (int) cudaErrorInvalidValue;
    return dispatch32<__half>(d, a, xchunk, ty, minb, (sites == 1) ? 1 : 2,
			      s);
  default:
    return (int) cudaErrorInvalidValue;
  }
}

/*****************************************************************************
 *
 *  Ensembles of boxes (one launch for all boxes)
 *
 *****************************************************************************/

template <typename S, bool HAS_MAP, int TY, int MINB>
static int launch_ens32(const lgbk_box_t * boxes, const void * items,
			int nitems, int xchunk, int * sched,
			cudaStream_t stream) {
  auto kern = k_binary_ensemble<float, S, false, true, true, HAS_MAP, TY,
				MINB>;
  size_t smem = FusedSmem<float, TY>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TY, smem);
  if (occ < 1) occ = 1;
  long long grid = (long long) nsm*occ;
  if (grid > nitems) grid = nitems;
  if (grid < 1) return 0;
  kern<<<(unsigned int) grid, dim3(32, TY), smem, stream>>>(
    boxes, (const int2 *) items, nitems, xchunk, sched);
  return (int) cudaGetLastError();
}

template <typename S, int TYT, int MINB>
static int launch_ens32_two(const lgbk_box_t * boxes, const void * items,
			    int nitems, int xchunk, int * sched,
			    cudaStream_t stream) {
  auto kern = k_binary_ensemble2<S, TYT, MINB>;
  size_t smem = FusedSmem<float, 2*TYT>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TYT, smem);
  if (occ < 1) occ = 1;
  long long grid = (long long) nsm*occ;
  if (grid > nitems) grid = nitems;
  if (grid < 1) return 0;
  kern<<<(unsigned int) grid, dim3(32, TYT), smem, stream>>>(
    boxes, (const int2 *) items, nitems, xchunk, sched);
  return (int) cudaGetLastError();
}

/* tile rows ty: 8 and 16 with two sites per thread (sites = 2, no map),
 * otherwise one */
template <typename S>
static int dispatch_ens32(const lgbk_box_t * b, const void * it, int n,
			  int xchunk, int ty, int minb, int m, int sites,
			  int * q, cudaStream_t s) {
  if (sites == 2 && !m && ty == 16) {
    return launch_ens32_two<S, 8, 2>(b, it, n, xchunk, q, s);
  }
  if (sites == 2 && !m && ty == 8) {
    if (minb == 4) return launch_ens32_two<S, 4, 4>(b, it, n, xchunk, q, s);
    if (minb == 2) return launch_ens32_two<S, 4, 2>(b, it, n, xchunk, q, s);
    return launch_ens32_two<S, 4, 3>(b, it, n, xchunk, q, s);
  }
  if (ty == 4) {
    return m ? launch_ens32<S, true, 4, 8>(b, it, n, xchunk, q, s)
             : launch_ens32<S, false, 4, 8>(b, it, n, xchunk, q, s);
  }
  if (ty == 16) {
    return m ? launch_ens32<S, true, 16, 2>(b, it, n, xchunk, q, s)
             : launch_ens32<S, false, 16, 2>(b, it, n, xchunk, q, s);
  }
  if (minb == 3) {
    return m ? launch_ens32<S, true, 8, 3>(b, it, n, xchunk, q, s)
             : launch_ens32<S, false, 8, 3>(b, it, n, xchunk, q, s);
  }
  return m ? launch_ens32<S, true, 8, 4>(b, it, n, xchunk, q, s)
           : launch_ens32<S, false, 8, 4>(b, it, n, xchunk, q, s);
}

extern "C" int lgbk_ensemble_step(int prec, const lgbk_box_t * boxes,
				  const void * items, int nitems, int xchunk,
				  int ty, int minb, int has_map, int sites,
				  int * sched, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  switch (prec) {
  case LGBK_PREC_FP64:
    return lgbk_ensemble_step_f64(boxes, items, nitems, xchunk, has_map,
				  sched, stream);
  case LGBK_PREC_FP32:
    return dispatch_ens32<float>(boxes, items, nitems, xchunk, ty, minb,
				 has_map, (sites == 2) ? 2 : 1, sched, s);
  case LGBK_PREC_FP16:
    return dispatch_ens32<__half>(boxes, items, nitems, xchunk, ty, minb,
				  has_map, (sites == 1) ? 1 : 2, sched, s);
  default:
    return (int) cudaErrorInvalidValue;
  }
}

extern "C" int lgbk_ensemble_items(const lgbk_dims_t * d, int box,
				   int xchunk, int ty, int * items) {
  int ntz = (d->nz + 31)/32, nty = (d->ny + ty - 1)/ty;
  int ncx = (d->nx + xchunk - 1)/xchunk;
  int n = ntz*nty*ncx;
  if (items) {
    for (int k = 0; k < n; k++) { items[2*k] = box; items[2*k + 1] = k; }
  }
  return n;
}

/*****************************************************************************
 *
 *  Conversions.  For distributions (ncomp == 19) the shift w_p rho0 is
 *  removed on the way in and restored on the way out; other fields are
 *  converted as they are (shift_rho0 ignored).
 *
 *****************************************************************************/

template <typename S>
__global__ void k_to_store(long long nsites, int ncomp, double rho0,
			   double scale, const double * __restrict__ src,
			   S * __restrict__ dst) {
  /* component p = blockIdx.y: no division to find it */
  const long long k = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (k >= nsites) return;
  const int p = (int) blockIdx.y;
  const long long i = (long long) p*nsites + k;
  double v = src[i];
  if (ncomp == LGB_NVEL) v -= lgb_w(p)*rho0;
  FStore<S, double>::st(dst + i, v, scale);
}

template <typename S>
__global__ void k_from_store(long long nsites, int ncomp, double rho0,
			     double scale, const S * __restrict__ src,
			     double * __restrict__ dst) {
  const long long k = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (k >= nsites) return;
  const int p = (int) blockIdx.y;
  const long long i = (long long) p*nsites + k;
  double v = FStore<S, double>::ld(src + i, 1.0/scale);
  if (ncomp == LGB_NVEL) v += lgb_w(p)*rho0;
  dst[i] = v;
}

template <typename S>
__global__ void k_propagate_store(lgbk_dims_t d, int dir,
				  const S * __restrict__ f,
				  S * __restrict__ fp) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  int z = (int) (i % d.nz);
  long long r = i / d.nz;
  int y = (int) (r % d.ny);
  int x = (int) (r / d.ny);
  const long long N = d.nsites;
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) {
    long long j = lgb_site_w(d, x - dir*lgb_cv_c[p][0], y - dir*lgb_cv_c[p][1],
			     z - dir*lgb_cv_c[p][2]);
    fp[p*N + i] = f[p*N + j];
  }
}

static dim3 g256(long long n) { return dim3((unsigned int) ((n + 255)/256)); }
/* blocks of 256 sites x one component each */
static dim3 g256c(long long nsites, int ncomp) {
  return dim3((unsigned int) ((nsites + 255)/256), (unsigned int) ncomp);
}

extern "C" int lgbk_f64_to_store(const lgbk_dims_t * d, int prec, int ncomp,
				 double shift_rho0, double scale,
				 const double * src, void * dst, void * stream) {
  long long n = d->nsites*ncomp;
  cudaStream_t s = (cudaStream_t) stream;
  if (prec == LGBK_PREC_FP64) {
    return (int) cudaMemcpyAsync(dst, src, n*sizeof(double),
				 cudaMemcpyDeviceToDevice, s);
  }
  if (prec == LGBK_PREC_FP16 && ncomp == LGB_NVEL) {
    k_to_store<__half><<<g256c(d->nsites, ncomp), 256, 0, s>>>(d->nsites, ncomp, shift_rho0,
					       scale, src, (__half *) dst);
  }
  else {
    k_to_store<float><<<g256c(d->nsites, ncomp), 256, 0, s>>>(d->nsites, ncomp, shift_rho0,
					      1.0, src, (float *) dst);
  }
  return (int) cudaGetLastError();
}

extern "C" int lgbk_store_to_f64(const lgbk_dims_t * d, int prec, int ncomp,
				 double shift_rho0, double scale,
				 const void * src, double * dst, void * stream) {
  long long n = d->nsites*ncomp;
  cudaStream_t s = (cudaStream_t) stream;
  if (prec == LGBK_PREC_FP64) {
    return (int) cudaMemcpyAsync(dst, src, n*sizeof(double),
				 cudaMemcpyDeviceToDevice, s);
  }
  if (prec == LGBK_PREC_FP16 && ncomp == LGB_NVEL) {
    k_from_store<__half><<<g256c(d->nsites, ncomp), 256, 0, s>>>(d->nsites, ncomp,
						 shift_rho0, scale,
						 (const __half *) src, dst);
  }
  else {
    k_from_store<float><<<g256c(d->nsites, ncomp), 256, 0, s>>>(d->nsites, ncomp, shift_rho0,
						1.0, (const float *) src, dst);
  }
  return (int) cudaGetLastError();
}

extern "C" int lgbk_propagate_store(const lgbk_dims_t * d, int prec, int dir,
				    const void * f, void * fprime,
				    void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  switch (prec) {
  case LGBK_PREC_FP64:
    return lgbk_propagate_f64(d, dir, (const double *) f, (double *) fprime,
			      stream);
  case LGBK_PREC_FP32:
    k_propagate_store<float><<<g256(d->nsites), 256, 0, s>>>(
      *d, dir, (const float *) f, (float *) fprime);
    break;
  default:
    k_propagate_store<__half><<<g256(d->nsites), 256, 0, s>>>(
      *d, dir, (const __half *) f, (__half *) fprime);
  }
  return (int) cudaGetLastError();
}

/*****************************************************************************
 *
 *  FP16 storage scale: the largest stored magnitude, and a rescaling of the
 *  stored values by a power of two (exact unless a value leaves the range
 *  of half precision).
 *
 *****************************************************************************/

__global__ void k_half_absmax(long long n, const __half * __restrict__ a,
			      unsigned int * __restrict__ out) {
  float m = 0.0f;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < n;
       i += (long long) gridDim.x*blockDim.x) {
    m = fmaxf(m, fabsf(__half2float(a[i])));
  }
  #pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
  }
  /* non-negative floats order as their bit patterns */
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void k_half_scale(long long n, __half * __restrict__ a,
			     float factor) {
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < n;
       i += (long long) gridDim.x*blockDim.x) {
    a[i] = __float2half_rn(__half2float(a[i])*factor);
  }
}

extern "C" int lgbk_half_absmax(long long n, const void * a,
				unsigned int * dev_word, float * host_max,
				void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  cudaError_t err = cudaMemsetAsync(dev_word, 0, sizeof(unsigned int), s);
  if (err != cudaSuccess) return (int) err;
  k_half_absmax<<<1024, 256, 0, s>>>(n, (const __half *) a, dev_word);
  err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  unsigned int w = 0;
  err = cudaMemcpyAsync(&w, dev_word, sizeof(w), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return (int) err;
  memcpy(host_max, &w, sizeof(float));
  return 0;
}

extern "C" int lgbk_half_scale(long long n, void * a, float factor,
			       void * stream) {
  k_half_scale<<<1024, 256, 0, (cudaStream_t) stream>>>(n, (__half *) a,
							factor);
  return (int) cudaGetLastError();
}
