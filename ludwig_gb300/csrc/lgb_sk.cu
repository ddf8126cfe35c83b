/*****************************************************************************
 *
 *  lgb_sk.cu
 *
 *  Spherically averaged structure factor S(|k|) of a scalar field and the
 *  domain length L = 2 pi sum S dk / sum k S dk (util/length_from_sk.c:
 *  88-190).  The 3-d transform is three passes of 1-d transforms (one
 *  line per CTA, twiddles from a table; radix-2 FFT for power-of-two
 *  lengths, the direct sum otherwise), in FP64; this is a diagnostic
 *  computed between steps, not part of the step.
 *
 *  Binning follows the reference: half space k_z in [0, N/2], 128 bins of
 *  width sqrt(3) pi / 128.  With faithful = 1 the bin of each wavevector
 *  is the one the reference's program computes: its wavevector for i > N/2
 *  is dk*i - pi (util/length_from_sk.c:138, which subtracts pi rather than
 *  2 pi), and it forms the wavevectors and |k| in FP32 (a bin edge decided
 *  in FP64 instead moves whole shells of a lamellar pattern to the next
 *  bin).  faithful = 0 uses dk*i - 2 pi in FP64.  An index of 128 (only
 *  possible at the corner |k| = sqrt(3) pi, where the reference would
 *  write one past its arrays) falls in the last bin; at 128^3 the FP32
 *  corner rounds into bin 127 in the reference too.  The sums are FP64
 *  (the reference sums in FP32).
 *
 *****************************************************************************/

#include "lgb_common.cuh"
#include "lgb_sk.h"

/* One 1-d DFT along axis `axis` for every line: out[k] = sum_n in[n] w^kn,
 * w = exp(-2 pi i / n).  in/out: complex double2 arrays in the canonical
 * site order.  One CTA per line; the line is staged in shared memory.
 * A power-of-two length is transformed by the radix-2 Cooley-Tukey FFT
 * (the line loaded in bit-reversed order, log2 n stages of butterflies
 * with the twiddles w^(j n/m) of the table); other lengths by the direct
 * sum. */
__global__ void k_dft_axis(lgbk_dims_t d, int axis,
			   const double2 * __restrict__ in,
			   double2 * __restrict__ out,
			   const double2 * __restrict__ tw) {
  extern __shared__ double2 line[];
  const int n = (axis == 0) ? d.nx : ((axis == 1) ? d.ny : d.nz);
  const long long stride = (axis == 0) ? (long long) d.ny*d.nz
    : ((axis == 1) ? d.nz : 1);
  /* line index -> base site */
  long long li = blockIdx.x;
  long long base;
  if (axis == 2) base = li*d.nz;
  else if (axis == 1) {
    long long x = li / d.nz, z = li % d.nz;
    base = x*(long long) d.ny*d.nz + z;
  }
  else base = li;                        /* x-lines: li = y*nz + z */

  if (n > 1 && (n & (n - 1)) == 0) {
    int lg = 0;
    while ((1 << lg) < n) lg++;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int r = (int) (__brev((unsigned int) i) >> (32 - lg));
      line[r] = in[base + i*stride];
    }
    __syncthreads();
    for (int half = 1; half < n; half *= 2) {
      const int step = n/(2*half);       /* twiddle index stride */
      for (int b = threadIdx.x; b < n/2; b += blockDim.x) {
	const int j = b % half;
	const int i0 = (b / half)*2*half + j;
	const int i1 = i0 + half;
	const double2 w = tw[j*step];
	const double2 v = line[i1];
	const double2 t = make_double2(v.x*w.x - v.y*w.y, v.x*w.y + v.y*w.x);
	const double2 u = line[i0];
	line[i0] = make_double2(u.x + t.x, u.y + t.y);
	line[i1] = make_double2(u.x - t.x, u.y - t.y);
      }
      __syncthreads();
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      out[base + k*stride] = line[k];
    }
    return;
  }

  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    line[i] = in[base + i*stride];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double re = 0.0, im = 0.0;
    int idx = 0;
    for (int j = 0; j < n; j++) {
      const double2 w = tw[idx];
      const double2 v = line[j];
      re += v.x*w.x - v.y*w.y;
      im += v.x*w.y + v.y*w.x;
      idx += k;
      if (idx >= n) idx -= n;
    }
    out[base + k*stride] = make_double2(re, im);
  }
}

template <typename T>
__global__ void k_to_complex(long long n, const T * __restrict__ a,
			     double2 * __restrict__ c) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i < n) c[i] = make_double2((double) a[i], 0.0);
}

/* Bin of the wavevector (ii, j, k) as util/length_from_sk.c:126-166
 * computes it: the wavevectors, their squares, sums and |k| in FP32, one
 * rounding per operation (the _rn intrinsics keep the compiler from
 * contracting them into fused multiply-adds), kmax = float(pi), dk =
 * float(2 kmax / nx) for every axis (the program assumes a cube), k -= kmax
 * for indices above n/2, and the bin floor(|k| 128 / (sqrt(3) kmax)) in
 * double. */
__device__ int bin_reference(const lgbk_dims_t & d, int ii, int j, int k) {
  const float kmax = 3.14159265358979323846f;
  const float dk = __double2float_rn(__ddiv_rn(2.0*(double) kmax,
					       (double) d.nx));
  float kx = __fmul_rn(dk, (float) ii);
  if (ii > d.nx/2) kx = __fsub_rn(kx, kmax);
  float ky = __fmul_rn(dk, (float) j);
  if (j > d.ny/2) ky = __fsub_rn(ky, kmax);
  float kz = __fmul_rn(dk, (float) k);
  float s = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)),
		      __fmul_rn(kz, kz));
  float kmod = __double2float_rn(__dsqrt_rn((double) s));
  double r = __ddiv_rn(__dmul_rn((double) kmod, (double) LGBK_SK_NBIN),
		       __dmul_rn(__dsqrt_rn(3.0), (double) kmax));
  return (int) floor(r);
}

/* Bin with the wavevector 2 pi i / n - 2 pi for i > n/2, in FP64, one
 * rounding per operation in the order ((kx kx + ky ky) + kz kz): diagonal
 * wavevectors (m, m, m) of a cube whose side is a multiple of 128 lie
 * exactly on bin edges, so a fused multiply-add would move them. */
__device__ int bin_corrected(const lgbk_dims_t & d, int ii, int j, int k) {
  const double pi = 3.14159265358979323846;
  const double twopi = 2.0*pi;
  double kx = __ddiv_rn(__dmul_rn(twopi, (double) ii), (double) d.nx);
  if (ii > d.nx/2) kx = __dsub_rn(kx, twopi);
  double ky = __ddiv_rn(__dmul_rn(twopi, (double) j), (double) d.ny);
  if (j > d.ny/2) ky = __dsub_rn(ky, twopi);
  double kz = __ddiv_rn(__dmul_rn(twopi, (double) k), (double) d.nz);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)),
		       __dmul_rn(kz, kz));
  double kmod = __dsqrt_rn(s);
  return (int) floor(__ddiv_rn(__dmul_rn(kmod, (double) LGBK_SK_NBIN),
			       __dmul_rn(__dsqrt_rn(3.0), pi)));
}

/* Bins of the half-space wavevectors: each CTA sums its sites into
 * shared-memory bins, then adds those to the global bins (one atomic per
 * bin and CTA instead of one per site) */
__global__ void k_bin_sk(lgbk_dims_t d, int faithful,
			 const double2 * __restrict__ c,
			 double * __restrict__ sk, double * __restrict__ nk) {
  __shared__ double ssk[LGBK_SK_NBIN], snk[LGBK_SK_NBIN];
  for (int b = threadIdx.x; b < LGBK_SK_NBIN; b += blockDim.x) {
    ssk[b] = 0.0;
    snk[b] = 0.0;
  }
  __syncthreads();
  const int nzh = d.nz/2 + 1;
  const long long nh = (long long) d.nx*d.ny*nzh;
  for (long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x; i < nh;
       i += (long long) gridDim.x*blockDim.x) {
    const int k = (int) (i % nzh);
    const long long r = i / nzh;
    const int j = (int) (r % d.ny);
    const int ii = (int) (r / d.ny);
    int n = faithful ? bin_reference(d, ii, j, k)
      : bin_corrected(d, ii, j, k);
    if (n >= LGBK_SK_NBIN) n = LGBK_SK_NBIN - 1;
    const double2 v = c[((long long) ii*d.ny + j)*d.nz + k];
    atomicAdd(ssk + n, v.x*v.x + v.y*v.y);
    atomicAdd(snk + n, 1.0);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < LGBK_SK_NBIN; b += blockDim.x) {
    if (snk[b] != 0.0) {
      atomicAdd(sk + b, ssk[b]);
      atomicAdd(nk + b, snk[b]);
    }
  }
}

extern "C" int lgbk_structure_factor(const lgbk_dims_t * d, int prec,
				     const void * phi, int faithful,
				     void * work, double * sk_host,
				     double * nk_host, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  const long long N = d->nsites;
  double2 * a = (double2 *) work;
  double2 * b = a + N;
  double2 * tw = b + N;                  /* up to 3 tables of n entries */
  double * bins = (double *) (tw + (d->nx + d->ny + d->nz));
  const int nmax = (d->nx > d->ny) ? ((d->nx > d->nz) ? d->nx : d->nz)
    : ((d->ny > d->nz) ? d->ny : d->nz);
  if (nmax > LGBK_SK_NMAX) return (int) cudaErrorInvalidValue;

  /* twiddle tables exp(-2 pi i m / n), computed on the host in double */
  double2 twh[3*LGBK_SK_NMAX];
  const int ns[3] = {d->nx, d->ny, d->nz};
  int off[3] = {0, d->nx, d->nx + d->ny};
  for (int ax = 0; ax < 3; ax++) {
    for (int m = 0; m < ns[ax]; m++) {
      double ang = -2.0*3.14159265358979323846*(double) m/ns[ax];
      twh[off[ax] + m] = make_double2(cos(ang), sin(ang));
    }
  }
  cudaError_t err = cudaMemcpyAsync(tw, twh, (d->nx + d->ny + d->nz)
				    *sizeof(double2), cudaMemcpyHostToDevice, s);
  if (err != cudaSuccess) return (int) err;

  dim3 g((unsigned int) ((N + 255)/256));
  if (prec == LGBK_PREC_FP64) {
    k_to_complex<double><<<g, 256, 0, s>>>(N, (const double *) phi, a);
  }
  else {
    k_to_complex<float><<<g, 256, 0, s>>>(N, (const float *) phi, a);
  }
  /* z lines, then y lines, then x lines */
  k_dft_axis<<<(unsigned int) (N/d->nz), 128, d->nz*sizeof(double2), s>>>(
    *d, 2, a, b, tw + off[2]);
  k_dft_axis<<<(unsigned int) (N/d->ny), 128, d->ny*sizeof(double2), s>>>(
    *d, 1, b, a, tw + off[1]);
  k_dft_axis<<<(unsigned int) (N/d->nx), 128, d->nx*sizeof(double2), s>>>(
    *d, 0, a, b, tw + off[0]);
  err = cudaMemsetAsync(bins, 0, 2*LGBK_SK_NBIN*sizeof(double), s);
  if (err != cudaSuccess) return (int) err;
  long long nh = (long long) d->nx*d->ny*(d->nz/2 + 1);
  long long nb = (nh + 255)/256;
  if (nb > 1024) nb = 1024;
  k_bin_sk<<<(unsigned int) nb, 256, 0, s>>>(
    *d, faithful, b, bins, bins + LGBK_SK_NBIN);
  err = cudaGetLastError();
  if (err != cudaSuccess) return (int) err;
  err = cudaMemcpyAsync(sk_host, bins, LGBK_SK_NBIN*sizeof(double),
			cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) {
    err = cudaMemcpyAsync(nk_host, bins + LGBK_SK_NBIN,
			  LGBK_SK_NBIN*sizeof(double), cudaMemcpyDeviceToHost,
			  s);
  }
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  return (int) err;
}

extern "C" size_t lgbk_structure_factor_work_bytes(const lgbk_dims_t * d) {
  return (size_t) (2*d->nsites + d->nx + d->ny + d->nz)*sizeof(double2)
    + 2*LGBK_SK_NBIN*sizeof(double);
}
