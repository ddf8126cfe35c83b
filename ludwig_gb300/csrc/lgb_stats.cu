/*****************************************************************************
 *
 *  lgb_stats.cu
 *
 *  Global sums on the device in FP64 with doubly compensated (Klein)
 *  accumulation: field totals/variance/min/max (src/phi_stats.c:211-270),
 *  distribution mass and momentum (src/stats_distribution.c:125-260) and
 *  the symmetric free-energy total (src/stats_free_energy.c:38).
 *
 *  Two passes, both deterministic: a fixed grid of LGBK_RED_BLOCKS blocks
 *  writes per-block partials to a scratch array, then one block combines
 *  them in a fixed order.  Each thread first sums its own sites (at most
 *  ceil(n / 262144) of them, a grid-stride loop) in plain FP64 -- the
 *  compensated sum costs a dozen FP64 operations a term, and FP64 is the
 *  scarce pipe of this GPU -- then the per-thread sums are combined with
 *  Klein's doubly compensated sum through warp shuffles, shared memory
 *  and the final block, in a fixed tree order.  The rounding error is that
 *  of at most 512 FP64 additions per thread at 512^3, far below the
 *  relative 1e-13 the conservation checks resolve.
 *
 *****************************************************************************/

#include <atomic>
#include <cstdio>

#include "lgb_fused.cuh"
#include "lgb_internal.h"
#include "lgb_stats.h"
#include "ludwig_gb.h"

/* Klein doubly compensated sum, src/util_sum.c:91-120 */
struct Klein {
  double sum, cs, ccs;
  __device__ __forceinline__ void zero() { sum = cs = ccs = 0.0; }
  __device__ __forceinline__ void add(double v) {
    double t = sum + v;
    double c = (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
    sum = t;
    t = cs + c;
    double cc = (fabs(cs) >= fabs(c)) ? (cs - t) + c : (c - t) + cs;
    cs = t;
    ccs = ccs + cc;
  }
  __device__ __forceinline__ void add(const Klein & o) {
    add(o.sum); add(o.cs); add(o.ccs);
  }
  __device__ __forceinline__ double total() const { return sum + cs + ccs; }
};

__device__ __forceinline__ Klein shfl_down(const Klein & k, int off) {
  Klein r;
  r.sum = __shfl_down_sync(0xffffffffu, k.sum, off);
  r.cs  = __shfl_down_sync(0xffffffffu, k.cs, off);
  r.ccs = __shfl_down_sync(0xffffffffu, k.ccs, off);
  return r;
}

/* Reduce NK Klein sums + min/max over a block; thread 0 gets the result */
template <int NK>
__device__ void block_reduce(Klein k[NK], double & vmin, double & vmax) {
  __shared__ Klein sk[32][NK];
  __shared__ double smin[32], smax[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  #pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    #pragma unroll
    for (int j = 0; j < NK; j++) {
      Klein o = shfl_down(k[j], off);
      if (lane < off) k[j].add(o);
    }
    double omin = __shfl_down_sync(0xffffffffu, vmin, off);
    double omax = __shfl_down_sync(0xffffffffu, vmax, off);
    if (lane < off) { vmin = fmin(vmin, omin); vmax = fmax(vmax, omax); }
  }
  if (lane == 0) {
    #pragma unroll
    for (int j = 0; j < NK; j++) sk[warp][j] = k[j];
    smin[warp] = vmin; smax[warp] = vmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; w++) {
      #pragma unroll
      for (int j = 0; j < NK; j++) k[j].add(sk[w][j]);
      vmin = fmin(vmin, smin[w]);
      vmax = fmax(vmax, smax[w]);
    }
  }
}

/* Partial record per block: NK*3 Klein words, then min, max */

template <int NK>
__device__ void write_partial(double * part, const Klein k[NK], double vmin,
			      double vmax) {
  double * p = part + (size_t) blockIdx.x*(3*NK + 2);
  #pragma unroll
  for (int j = 0; j < NK; j++) {
    p[3*j] = k[j].sum; p[3*j + 1] = k[j].cs; p[3*j + 2] = k[j].ccs;
  }
  p[3*NK] = vmin;
  p[3*NK + 1] = vmax;
}

/* One block of RED_FINAL threads: thread t combines the partial records
 * t, t + RED_FINAL, ... in that order, then the block combines the
 * threads' sums (block_reduce, fixed tree order). */
#define RED_FINAL 256

template <int NK>
__global__ void __launch_bounds__(RED_FINAL)
k_final(const double * __restrict__ part, int nblocks,
	double * __restrict__ out) {
  Klein k[NK];
  #pragma unroll
  for (int j = 0; j < NK; j++) k[j].zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double * p = part + (size_t) b*(3*NK + 2);
    #pragma unroll
    for (int j = 0; j < NK; j++) {
      Klein o;
      o.sum = p[3*j]; o.cs = p[3*j + 1]; o.ccs = p[3*j + 2];
      k[j].add(o);
    }
    vmin = fmin(vmin, p[3*NK]);
    vmax = fmax(vmax, p[3*NK + 1]);
  }
  block_reduce<NK>(k, vmin, vmax);
  if (threadIdx.x == 0) {
    #pragma unroll
    for (int j = 0; j < NK; j++) out[j] = k[j].total();
    out[NK] = vmin;
    out[NK + 1] = vmax;
  }
}

/* A thread's own sums: plain FP64 over its sites, folded into Klein sums
 * once at the end */
template <int NK>
struct Plain {
  double v[NK];
  __device__ __forceinline__ void zero() {
    #pragma unroll
    for (int j = 0; j < NK; j++) v[j] = 0.0;
  }
  __device__ __forceinline__ void to(Klein k[NK]) const {
    #pragma unroll
    for (int j = 0; j < NK; j++) { k[j].zero(); k[j].add(v[j]); }
  }
};

template <typename T>
__device__ __forceinline__ double ldv(const T * p) { return (double) *p; }

/* Field component: sum, sum of squares, min, max */
template <typename T>
__global__ void k_field_stats(long long n, const T * __restrict__ a,
			      double * __restrict__ part) {
  Plain<2> t;
  Klein k[2];
  t.zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < n;
       i += (long long) gridDim.x*blockDim.x) {
    double v = ldv(a + i);
    t.v[0] += v;
    t.v[1] += v*v;
    vmin = fmin(vmin, v);
    vmax = fmax(vmax, v);
  }
  t.to(k);
  block_reduce<2>(k, vmin, vmax);
  if (threadIdx.x == 0) write_partial<2>(part, k, vmin, vmax);
}

/* NK columns a[j*n + i] summed over the sites whose status is fluid (all
 * sites when st is NULL); min and max of column 0 over the same sites */
template <typename T, int NK>
__global__ void k_masked_cols(long long n, const T * __restrict__ a,
			      const uint8_t * __restrict__ st,
			      double * __restrict__ part) {
  Plain<NK> t;
  Klein k[NK];
  t.zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < n;
       i += (long long) gridDim.x*blockDim.x) {
    if (st && st[i] != 0) continue;
    #pragma unroll
    for (int j = 0; j < NK; j++) t.v[j] += ldv(a + j*n + i);
    double v = ldv(a + i);
    vmin = fmin(vmin, v);
    vmax = fmax(vmax, v);
  }
  t.to(k);
  block_reduce<NK>(k, vmin, vmax);
  if (threadIdx.x == 0) write_partial<NK>(part, k, vmin, vmax);
}

/* Distribution moments: mass and momentum of stored (possibly shifted) f */
template <typename S>
__global__ void k_dist_moments(long long n, const S * __restrict__ f,
			       double rscale, double * __restrict__ part) {
  Plain<4> t;
  Klein k[4];
  t.zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < n;
       i += (long long) gridDim.x*blockDim.x) {
    double fp[LGB_NVEL];
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) {
      fp[p] = FStore<S, double>::ld(f + p*n + i, rscale);
    }
    double m = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) {
      m += fp[p];
      jx += lgb_cv_c[p][0]*fp[p];
      jy += lgb_cv_c[p][1]*fp[p];
      jz += lgb_cv_c[p][2]*fp[p];
    }
    t.v[0] += m; t.v[1] += jx; t.v[2] += jy; t.v[3] += jz;
    vmin = fmin(vmin, m);
    vmax = fmax(vmax, m);
  }
  t.to(k);
  block_reduce<4>(k, vmin, vmax);
  if (threadIdx.x == 0) write_partial<4>(part, k, vmin, vmax);
}

/* Symmetric free energy density (src/symmetric.c:285-300) */
template <typename T>
__global__ void k_symm_fed(lgbk_dims_t d, lgbk_symm_t fe,
			   const T * __restrict__ phi,
			   double * __restrict__ part) {
  Plain<1> t;
  Klein k[1];
  t.zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
       i < d.nsites; i += (long long) gridDim.x*blockDim.x) {
    int z = (int) (i % d.nz);
    long long r = i / d.nz;
    int y = (int) (r % d.ny);
    int x = (int) (r / d.ny);
    double g[3];
    g[0] = 0.5*(ldv(phi + lgb_site_w(d, x+1, y, z))
		- ldv(phi + lgb_site_w(d, x-1, y, z)));
    g[1] = 0.5*(ldv(phi + lgb_site_w(d, x, y+1, z))
		- ldv(phi + lgb_site_w(d, x, y-1, z)));
    g[2] = 0.5*(ldv(phi + lgb_site_w(d, x, y, z+1))
		- ldv(phi + lgb_site_w(d, x, y, z-1)));
    double p = ldv(phi + i);
    double fed = (0.5*fe.a + 0.25*fe.b*p*p)*p*p
      + 0.5*fe.kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
    t.v[0] += fed;
    vmin = fmin(vmin, fed);
    vmax = fmax(vmax, fed);
  }
  t.to(k);
  block_reduce<1>(k, vmin, vmax);
  if (threadIdx.x == 0) write_partial<1>(part, k, vmin, vmax);
}

/* As k_symm_fed with stored gradients (any stencil): FP64 fields */
__global__ void k_symm_fed_g(lgbk_dims_t d, lgbk_symm_t fe,
			     const double * __restrict__ phi,
			     const double * __restrict__ grad,
			     double * __restrict__ part) {
  Plain<1> t;
  Klein k[1];
  t.zero();
  double vmin = +INFINITY, vmax = -INFINITY;
  const long long N = d.nsites;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
       i < N; i += (long long) gridDim.x*blockDim.x) {
    const double g[3] = {grad[i], grad[N + i], grad[2*N + i]};
    const double p = phi[i];
    double fed = (0.5*fe.a + 0.25*fe.b*p*p)*p*p
      + 0.5*fe.kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
    t.v[0] += fed;
    vmin = fmin(vmin, fed);
    vmax = fmax(vmax, fed);
  }
  t.to(k);
  block_reduce<1>(k, vmin, vmax);
  if (threadIdx.x == 0) write_partial<1>(part, k, vmin, vmax);
}

#define RED_TPB 256

static int finish(int nk, double * scratch, double * out_host,
		  cudaStream_t s) {
  double * out = scratch + (size_t) LGBK_RED_BLOCKS*LGBK_RED_REC;
  switch (nk) {
  case 1: k_final<1><<<1, RED_FINAL, 0, s>>>(scratch, LGBK_RED_BLOCKS, out); break;
  case 2: k_final<2><<<1, RED_FINAL, 0, s>>>(scratch, LGBK_RED_BLOCKS, out); break;
  case 3: k_final<3><<<1, RED_FINAL, 0, s>>>(scratch, LGBK_RED_BLOCKS, out); break;
  default: k_final<4><<<1, RED_FINAL, 0, s>>>(scratch, LGBK_RED_BLOCKS, out); break;
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  err = cudaMemcpyAsync(out_host, out, (nk + 2)*sizeof(double),
			cudaMemcpyDeviceToHost, s);
  if (err != cudaSuccess) return (int) err;
  return (int) cudaStreamSynchronize(s);
}

extern "C" int lgbk_field_stats(const lgbk_dims_t * d, int prec,
				const void * a, double * scratch,
				double out_host[4], void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (prec == LGBK_PREC_FP64) {
    k_field_stats<double><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      d->nsites, (const double *) a, scratch);
  }
  else {
    k_field_stats<float><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      d->nsites, (const float *) a, scratch);
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  return finish(2, scratch, out_host, s);
}

extern "C" int lgbk_masked_cols(const lgbk_dims_t * d, int prec, int ncol,
				const void * a, const uint8_t * status,
				double * scratch, double * out_host,
				void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  const long long n = d->nsites;
  if (ncol == 1 && prec == LGBK_PREC_FP64) {
    k_masked_cols<double, 1><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      n, (const double *) a, status, scratch);
  }
  else if (ncol == 1) {
    k_masked_cols<float, 1><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      n, (const float *) a, status, scratch);
  }
  else if (ncol == 3 && prec == LGBK_PREC_FP64) {
    k_masked_cols<double, 3><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      n, (const double *) a, status, scratch);
  }
  else {
    return (int) cudaErrorInvalidValue;
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  return finish(ncol, scratch, out_host, s);
}

extern "C" int lgbk_dist_moments(const lgbk_dims_t * d, int prec,
				 const void * f, double scale, double * scratch,
				 double out_host[6], void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (prec == LGBK_PREC_FP64) {
    k_dist_moments<double><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      d->nsites, (const double *) f, 1.0, scratch);
  }
  else if (prec == LGBK_PREC_FP32) {
    k_dist_moments<float><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      d->nsites, (const float *) f, 1.0, scratch);
  }
  else {
    k_dist_moments<__half><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      d->nsites, (const __half *) f, 1.0/scale, scratch);
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  return finish(4, scratch, out_host, s);
}

extern "C" int lgbk_symm_fed_total_grad(const lgbk_dims_t * d,
					const lgbk_symm_t * fe,
					const double * phi,
					const double * grad, double * scratch,
					double out_host[3], void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  k_symm_fed_g<<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(*d, *fe, phi, grad,
						   scratch);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  return finish(1, scratch, out_host, s);
}

extern "C" int lgbk_symm_fed_total(const lgbk_dims_t * d, int prec,
				   const lgbk_symm_t * fe, const void * phi,
				   double * scratch, double out_host[3],
				   void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (prec == LGBK_PREC_FP64) {
    k_symm_fed<double><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      *d, *fe, (const double *) phi, scratch);
  }
  else {
    k_symm_fed<float><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      *d, *fe, (const float *) phi, scratch);
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  return finish(1, scratch, out_host, s);
}

/*****************************************************************************
 *
 *  Field statistics without allocation.
 *
 *  For callers that cannot allocate device memory themselves: code that
 *  runs where cudaMalloc is not allowed or not wanted, for example a host
 *  application whose device memory is owned by another allocator or
 *  runtime, or a time-critical loop that must not pay the implicit device
 *  synchronisation of cudaMalloc/cudaFree.  They pass a device pointer to
 *  their own data and a host array for the result; the per-block partial
 *  sums go to the static array below instead of a buffer the library
 *  allocates.
 *
 *  The array is a file-scope __device__ variable: every GPU that loads the
 *  library holds it (NOALLOC_MAX_NCOMP*NOALLOC_SLOT doubles, 328 KB) until
 *  the process exits.  Host code cannot use the name of a __device__
 *  variable as a device address (on the host it names a stand-in object),
 *  so the device address is looked up with cudaGetSymbolAddress once per
 *  device, with that device current, on the first call made on it.  That
 *  first call should therefore come before any stream capture.  The
 *  per-device addresses are cached in atomics, so first calls from several
 *  host threads at once are well defined (they store the same address).
 *
 *  All calls share the one array and it keeps whatever the last call left
 *  there: each call writes every partial record it later reads, so nothing
 *  has to be cleared first.  Calls whose work overlaps on the GPU (several
 *  host threads, or several streams) race on the array; the caller must
 *  order them, for instance by using one stream.
 *
 *  Every site of d_data is counted: there is no status map, unlike
 *  stats_field_q, which skips solid sites.
 *
 *****************************************************************************/

#define NOALLOC_REC (3*2 + 2)                       /* k_field_stats NK = 2 */
#define NOALLOC_SLOT (LGBK_RED_BLOCKS*NOALLOC_REC + 16)
#define NOALLOC_MAX_NCOMP 5
#define NOALLOC_DEVICES 64

static __device__ __align__(256) double
  lgb_noalloc_scratch[NOALLOC_MAX_NCOMP*NOALLOC_SLOT];

static std::atomic<double *> noalloc_addr_[NOALLOC_DEVICES];

static int noalloc_cuda(cudaError_t err, const char * where) {
  char msg[256];
  snprintf(msg, sizeof(msg), "ludwig_gb_field_stats_noalloc: %s: %s", where,
	   cudaGetErrorString(err));
  return lgb_internal_err(LUDWIG_GB_ECUDA, msg);
}

extern "C" int ludwig_gb_field_stats_noalloc(const double * d_data,
					     long long nsites, int ncomp,
					     double * out, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  int dev = 0;
  double raw[NOALLOC_MAX_NCOMP][4];

  static_assert(NOALLOC_MAX_NCOMP == LUDWIG_GB_NOALLOC_MAX_NCOMP,
		"static scratch sized for the documented maximum");

  /* More components than the static array holds partials for */
  if (ncomp < 1 || ncomp > NOALLOC_MAX_NCOMP) {
    char msg[160];
    snprintf(msg, sizeof(msg), "ludwig_gb_field_stats_noalloc: ncomp = %d; "
	     "the static scratch holds 1 to %d components", ncomp,
	     NOALLOC_MAX_NCOMP);
    return lgb_internal_err(LUDWIG_GB_EINVAL, msg);
  }
  if (d_data == NULL || out == NULL || nsites <= 0) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "ludwig_gb_field_stats_noalloc:"
			    " NULL data or result, or nsites <= 0");
  }

  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return noalloc_cuda(err, "cudaGetDevice");
  if (dev < 0 || dev >= NOALLOC_DEVICES) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "ludwig_gb_field_stats_noalloc:"
			    " device ordinal beyond the address cache (64)");
  }
  double * base = noalloc_addr_[dev].load(std::memory_order_acquire);
  if (base == NULL) {
    /* once per device, with that device current */
    void * p = NULL;
    err = cudaGetSymbolAddress(&p, lgb_noalloc_scratch);
    if (err != cudaSuccess) return noalloc_cuda(err, "cudaGetSymbolAddress");
    if (p == NULL) {
      return lgb_internal_err(LUDWIG_GB_ECUDA, "ludwig_gb_field_stats_noalloc:"
			      " cudaGetSymbolAddress returned NULL");
    }
    base = (double *) p;
    noalloc_addr_[dev].store(base, std::memory_order_release);
  }

  for (int n = 0; n < ncomp; n++) {
    double * part = base + (size_t) n*NOALLOC_SLOT;
    double * fin = part + (size_t) LGBK_RED_BLOCKS*NOALLOC_REC;
    k_field_stats<double><<<LGBK_RED_BLOCKS, RED_TPB, 0, s>>>(
      nsites, d_data + (size_t) n*nsites, part);
    k_final<2><<<1, RED_FINAL, 0, s>>>(part, LGBK_RED_BLOCKS, fin);
    err = cudaGetLastError();
    if (err != cudaSuccess) return noalloc_cuda(err, "kernel launch");
    err = cudaMemcpyAsync(raw[n], fin, 4*sizeof(double),
			  cudaMemcpyDeviceToHost, s);
    if (err != cudaSuccess) return noalloc_cuda(err, "cudaMemcpyAsync");
  }
  err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return noalloc_cuda(err, "cudaStreamSynchronize");

  for (int n = 0; n < ncomp; n++) {
    double rvol = 1.0/(double) nsites;
    double mean = rvol*raw[n][0];
    out[5*n + 0] = raw[n][0];
    out[5*n + 1] = mean;
    out[5*n + 2] = rvol*raw[n][1] - mean*mean;
    out[5*n + 3] = raw[n][2];
    out[5*n + 4] = raw[n][3];
  }
  return LUDWIG_GB_OK;
}
