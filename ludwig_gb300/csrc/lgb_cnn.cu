/*****************************************************************************
 *
 *  lgb_cnn.cu
 *
 *  Kernels of the learned corrector (a 4-layer 3x3x3 convolutional network
 *  with 32 channels on the coarse lattice).
 *
 *  k_conv3_tc: the convolution as an implicit GEMM,
 *      D[m][n] = sum_t sum_c A_t[m][c] W[t][n][c],   m = 128 sites of a tile,
 *  with M = 128, N = 32, K = 27 taps x 32 channels.  Per tap the A operand
 *  is the tile's neighbour rows (a TMA box of contiguous padded rows, K-major,
 *  64-byte swizzle); the weights of all 27 taps stay in shared memory.
 *  Warp roles: warp 0 issues TMA, warp 1 issues tcgen05.mma into one of two
 *  TMEM accumulators, warps 2-9 drain the other accumulator (tcgen05.ld,
 *  two warps per TMEM lane quarter, 16 columns each) and run the epilogue
 *  (bias, GELU, GELU', bf16 rows).  The backward-data pass
 *  is the same kernel with flipped, transposed weights.
 *
 *  k_wgrad_tc: the weight gradient
 *      dW[t][n][c] = sum_s G[s - e_t][n] X[s][c]
 *  with K = sites: four taps are stacked along M (M = 4 taps x 32 = 128,
 *  N = 32), both operands MN-major (channels contiguous, sites strided), so
 *  shifted taps are again plain TMA boxes of rows.  Seven tap groups
 *  accumulate in 7 x 32 TMEM columns over all tiles of a CTA; each CTA then
 *  writes its partial sums and a second kernel adds them in a fixed order.
 *
 *  Every wait is bounded (lgb_tc.cuh); on a timeout the kernel raises the
 *  error word, waits for its own copies and MMAs in flight, frees its tensor
 *  memory and returns.
 *
 *****************************************************************************/

#include <cuda_bf16.h>
#include <cuda.h>

#include "lgb_tc.cuh"
#include "lgb_cnn.h"

#define CNN_C      LGBK_CNN_C
#define CNN_NTAP   LGBK_CNN_NTAP
#define ROWB       64                    /* bytes per padded row */
#define TILEB      8192                  /* 128 rows */
#define WTAPB      2048                  /* 32 rows of weights per tap */

#define CONV_STAGES  12
#define CONV_THREADS 320               /* TMA, MMA, 8 epilogue warps */
#define CONV_EPI_THREADS 256
#define CONV_TMEM_COLS 64
#define CONV_SMEM (1024 + CNN_NTAP*WTAPB + CONV_STAGES*TILEB + 256)

#define WG_XSTAGES 2
#define WG_ASTAGES 6
#define WG_GROUPS  7                     /* ceil(27/4) */
#define WG_ASTAGEB (4*TILEB)
#define WG_THREADS 192
#define WG_TMEM_COLS 256
#define WG_SMEM (1024 + WG_XSTAGES*TILEB + WG_ASTAGES*WG_ASTAGEB + 256)

/*****************************************************************************
 *  Geometry
 *****************************************************************************/

extern "C" int lgbk_cnn_geom(int nx, int ny, int nz, lgbk_cnn_geom_t * g) {
  if (nx < 2 || ny < 2 || nz < 2) return 1;
  int bz, lpt;
  if (nz == 32 || nz == 64) { bz = nz; lpt = LGBK_CNN_TILE/nz; }
  else if (nz % LGBK_CNN_TILE == 0) { bz = LGBK_CNN_TILE; lpt = 1; }
  else return 1;
  if (ny % lpt) return 1;
  g->nx = nx; g->ny = ny; g->nz = nz;
  g->bz = bz; g->lpt = lpt;
  g->nsites = (long long) nx*ny*nz;
  g->rows = (long long) (nx + 2)*(ny + 2)*(nz + 2);
  long long nt = g->nsites/LGBK_CNN_TILE;
  if (nt > 0x7fffffffLL || g->rows > 0x7fffffffLL) return 1;
  g->ntiles = (int) nt;
  return 0;
}

static int num_sms(void) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm > 0 ? nsm : 1;
}

extern "C" int lgbk_cnn_conv_blocks(const lgbk_cnn_geom_t * g) {
  int n = num_sms();
  return (g->ntiles < n) ? g->ntiles : n;
}

extern "C" int lgbk_cnn_wgrad_blocks(const lgbk_cnn_geom_t * g) {
  int n = num_sms();
  return (g->ntiles < n) ? g->ntiles : n;
}

__device__ __forceinline__ int prow(const lgbk_cnn_geom_t & g, int x, int y,
				    int z) {
  return ((x + 1)*(g.ny + 2) + (y + 1))*(g.nz + 2) + (z + 1);
}

__device__ __forceinline__ void tile_decode(const lgbk_cnn_geom_t & g,
					    int tile, int & x, int & y0,
					    int & z0) {
  const int nzc = g.nz/g.bz;
  const int zc = tile % nzc;
  const int r = tile / nzc;
  const int nyg = g.ny/g.lpt;
  y0 = (r % nyg)*g.lpt;
  x = r / nyg;
  z0 = zc*g.bz;
}

__device__ __forceinline__ void tap_offsets(int t, int & dx, int & dy,
					    int & dz) {
  dx = t/9 - 1; dy = (t/3) % 3 - 1; dz = t % 3 - 1;
}

/* Bounded wait that ignores the abort flag: used to drain copies and MMAs
 * already in flight before the CTA exits. */
__device__ __forceinline__ bool tc_drain_wait(uint32_t bar, uint32_t parity,
					      int * err) {
  volatile int never = 0;
  return tc_mbar_wait(bar, parity, &never, err);
}

/* GELU in the tanh form of Hendrycks and Gimpel (2016),
 * 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3), evaluated as
 * z sigma(2u) = z / (1 + exp(-2u)): one fast exponential and one fast
 * division per value, and no cancellation where z < 0.  2u is held above
 * -80 so that the divisor stays finite (the value there is below 1e-33
 * in magnitude either way). */
#define GELU_K0 1.5957691216057308f          /* 2 sqrt(2/pi) */
#define GELU_K1 0.044715f

__device__ __forceinline__ float gelu_f(float z) {
  const float v = fmaxf(GELU_K0*z*fmaf(GELU_K1*z, z, 1.0f), -80.0f);
  return __fdividef(z, 1.0f + __expf(-v));
}

/* GELU(z) and its slope d/dz z sigma(2u) = s + z s (1 - s) d(2u)/dz,
 * s = sigma(2u), from one exponential: the forward pass of training keeps
 * the slope for the backward pass */
__device__ __forceinline__ float gelu_and_slope(float z, float & d) {
  const float v = fmaxf(GELU_K0*z*fmaf(GELU_K1*z, z, 1.0f), -80.0f);
  const float e = 1.0f + __expf(-v);
  const float s = __fdividef(1.0f, e);
  const float dv = GELU_K0*fmaf(3.0f*GELU_K1*z, z, 1.0f);
  d = fmaf(z*s*(1.0f - s), dv, s);
  return __fdividef(z, e);                /* as gelu_f */
}

__device__ __forceinline__ void store_row_bf16(uint8_t * dst,
					       const float v[32]) {
  uint4 * d4 = (uint4 *) dst;
  #pragma unroll
  for (int q = 0; q < 4; q++) {
    uint32_t w[4];
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      __nv_bfloat162 h = __floats2bfloat162_rn(v[8*q + 2*k],
					       v[8*q + 2*k + 1]);
      w[k] = *(uint32_t *) &h;
    }
    d4[q] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__device__ __forceinline__ void load_row_bf16(const uint8_t * src,
					      float v[32]) {
  const uint4 * s4 = (const uint4 *) src;
  #pragma unroll
  for (int q = 0; q < 4; q++) {
    uint4 u = s4[q];
    uint32_t w[4] = {u.x, u.y, u.z, u.w};
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      __nv_bfloat162 h = *(__nv_bfloat162 *) &w[k];
      float2 f = __bfloat1622float2(h);
      v[8*q + 2*k] = f.x;
      v[8*q + 2*k + 1] = f.y;
    }
  }
}

__device__ __forceinline__ void store_half_row_bf16(uint8_t * dst,
						    const float v[16]) {
  uint4 * d4 = (uint4 *) dst;
  #pragma unroll
  for (int q = 0; q < 2; q++) {
    uint32_t w[4];
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      __nv_bfloat162 h = __floats2bfloat162_rn(v[8*q + 2*k],
					       v[8*q + 2*k + 1]);
      w[k] = *(uint32_t *) &h;
    }
    d4[q] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

/* 16 values -> 16 BF16 (two 16-byte words) */
__device__ __forceinline__ void pack_half_row_bf16(const float v[16],
						   uint4 w[2]) {
  #pragma unroll
  for (int q = 0; q < 2; q++) {
    uint32_t u[4];
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      __nv_bfloat162 h = __floats2bfloat162_rn(v[8*q + 2*k],
					       v[8*q + 2*k + 1]);
      u[k] = *(uint32_t *) &h;
    }
    w[q] = make_uint4(u[0], u[1], u[2], u[3]);
  }
}

/* Bytes [off, off + nw*16) of site (x, y, z)'s padded row and of every
 * periodic image of it in the halo (a site on a face of the lattice has
 * up to seven), so that no separate halo pass is needed */
template <int NW>
__device__ __forceinline__ void store_row_images(const lgbk_cnn_geom_t & g,
						 uint8_t * base, int x, int y,
						 int z, int off,
						 const uint4 * w) {
  const int xb = (x == 0) ? g.nx + 1 : ((x == g.nx - 1) ? 0 : -1);
  const int yb = (y == 0) ? g.ny + 1 : ((y == g.ny - 1) ? 0 : -1);
  const int zb = (z == 0) ? g.nz + 1 : ((z == g.nz - 1) ? 0 : -1);
  #pragma unroll
  for (int k = 0; k < 8; k++) {
    const int xp = (k & 1) ? xb : x + 1;
    const int yp = (k & 2) ? yb : y + 1;
    const int zp = (k & 4) ? zb : z + 1;
    if (xp < 0 || yp < 0 || zp < 0) continue;
    uint4 * d = (uint4 *) (base + (long long) ((xp*(g.ny + 2) + yp)
					       *(g.nz + 2) + zp)*ROWB + off);
    #pragma unroll
    for (int j = 0; j < NW; j++) d[j] = w[j];
  }
}

__device__ __forceinline__ void load_half_row_bf16(const uint8_t * src,
						   float v[16]) {
  const uint4 * s4 = (const uint4 *) src;
  #pragma unroll
  for (int q = 0; q < 2; q++) {
    uint4 u = s4[q];
    uint32_t w[4] = {u.x, u.y, u.z, u.w};
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      __nv_bfloat162 h = *(__nv_bfloat162 *) &w[k];
      float2 f = __bfloat1622float2(h);
      v[8*q + 2*k] = f.x;
      v[8*q + 2*k + 1] = f.y;
    }
  }
}

/*****************************************************************************
 *  k_conv3_tc
 *****************************************************************************/

struct ConvP {
  lgbk_cnn_geom_t g;
  const float * bias;
  const uint8_t * zprev;
  uint8_t * zout;
  uint8_t * pout;
  float * outf;
  int * err;
  int khn;                    /* K halves of 16 input channels: 1 or 2 */
  int nb;                     /* weight rows per tap in shared memory: 32,
				 or 16 for the last layer's 4 outputs in
				 the three-tap line form */
};

/* Epilogue of channels c0 .. c0+15 of one output site (x, y, z) from 16
 * accumulator columns */
/* The backward-data epilogue of channels c0 .. c0+15 with the stored
 * slopes GELU'(z) already loaded (two 16-byte pieces of the row) */
__device__ __forceinline__ void conv_epilogue_bwd(const ConvP & p, int x,
						  int y, int z, int c0,
						  const uint32_t r[16],
						  const uint4 zq[2]) {
  const lgbk_cnn_geom_t & g = p.g;
  float v[16];
  #pragma unroll
  for (int q = 0; q < 2; q++) {
    const uint32_t w[4] = {zq[q].x, zq[q].y, zq[q].z, zq[q].w};
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      const float2 f = __bfloat1622float2(*(const __nv_bfloat162 *) &w[k]);
      v[8*q + 2*k] = __uint_as_float(r[8*q + 2*k])*f.x;
      v[8*q + 2*k + 1] = __uint_as_float(r[8*q + 2*k + 1])*f.y;
    }
  }
  /* with the periodic images: the three-tap line form writes the halo */
  uint4 w[2];
  pack_half_row_bf16(v, w);
  store_row_images<2>(g, p.pout, x, y, z, 2*c0, w);
}

template <int MODE, bool IMG = false>
__device__ __forceinline__ void conv_epilogue(const ConvP & p,
					      const float bias[16], int x,
					      int y, int z, int c0,
					      const uint32_t r[16]) {
  const lgbk_cnn_geom_t & g = p.g;
  const long long s = ((long long) x*g.ny + y)*g.nz + z;
  float v[16];
  #pragma unroll
  for (int n = 0; n < 16; n++) v[n] = __uint_as_float(r[n]);

  if (MODE == LGBK_CNN_FWD_GELU) {
    #pragma unroll
    for (int n = 0; n < 16; n++) v[n] += bias[n];
    if (p.zout) {
      /* training: the slopes GELU'(z), kept for the backward pass */
      float d[16];
      #pragma unroll
      for (int n = 0; n < 16; n++) v[n] = gelu_and_slope(v[n], d[n]);
      store_half_row_bf16(p.zout + s*ROWB + 2*c0, d);
    }
    else {
      #pragma unroll
      for (int n = 0; n < 16; n++) v[n] = gelu_f(v[n]);
    }
    if (IMG) {
      uint4 w[2];
      pack_half_row_bf16(v, w);
      store_row_images<2>(g, p.pout, x, y, z, 2*c0, w);
    }
    else {
      store_half_row_bf16(p.pout + (long long) prow(g, x, y, z)*ROWB + 2*c0,
			  v);
    }
  }
  else if (MODE == LGBK_CNN_FWD_OUT) {
    if (c0 == 0) {
      #pragma unroll
      for (int c = 0; c < LGBK_CNN_NOUT; c++) {
	p.outf[c*g.nsites + s] = v[c] + bias[c];
      }
    }
  }
  else if (MODE == LGBK_CNN_BWD_GELU) {
    /* the slopes GELU'(z) the forward pass kept */
    float zp[16];
    load_half_row_bf16(p.zprev + s*ROWB + 2*c0, zp);
    #pragma unroll
    for (int n = 0; n < 16; n++) v[n] *= zp[n];
    store_half_row_bf16(p.pout + (long long) prow(g, x, y, z)*ROWB + 2*c0, v);
  }
  else {
    float4 * o = (float4 *) (p.outf + s*CNN_C + c0);
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      o[k] = make_float4(v[4*k] + bias[4*k], v[4*k + 1] + bias[4*k + 1],
			 v[4*k + 2] + bias[4*k + 2],
			 v[4*k + 3] + bias[4*k + 3]);
    }
  }
}

template <int MODE>
__global__ void __launch_bounds__(CONV_THREADS, 1)
k_conv3_tc(const __grid_constant__ CUtensorMap tm_in,
	   const __grid_constant__ CUtensorMap tm_w, const ConvP p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc_smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t * sgen = smem_raw + (sbase - raw);

  const uint32_t sW = sbase;
  const uint32_t sA = sW + CNN_NTAP*WTAPB;
  const uint32_t sBar = sA + CONV_STAGES*TILEB;
  const uint32_t bFull = sBar;
  const uint32_t bEmpty = sBar + 8*CONV_STAGES;
  const uint32_t bW = sBar + 16*CONV_STAGES;
  const uint32_t bTFull = bW + 8;
  const uint32_t bTEmpty = bW + 24;
  const uint32_t bDone = bW + 40;
  uint32_t * tslot = (uint32_t *) (sgen + (bW + 48 - sbase));
  volatile int * abort_flag = (volatile int *) (sgen + (bW + 52 - sbase));

  const int warp = threadIdx.x/32;
  const int lane = threadIdx.x % 32;
  const lgbk_cnn_geom_t & g = p.g;

  if (threadIdx.x == 0) {
    for (int s = 0; s < CONV_STAGES; s++) {
      tc_mbar_init(bFull + 8*s, 1);
      tc_mbar_init(bEmpty + 8*s, 1);
    }
    tc_mbar_init(bW, 1);
    tc_mbar_init(bTFull, 1);
    tc_mbar_init(bTFull + 8, 1);
    tc_mbar_init(bTEmpty, CONV_EPI_THREADS);
    tc_mbar_init(bTEmpty + 8, CONV_EPI_THREADS);
    tc_mbar_init(bDone, 1);
    *abort_flag = 0;
    tc_fence_barrier_init();
  }
  if (warp == 1) tc_tmem_alloc(tc_smem_u32(tslot), CONV_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    /* TMA producer */
    tc_prefetch_map(&tm_in);
    tc_prefetch_map(&tm_w);
    tc_mbar_arrive_tx(bW, CNN_NTAP*WTAPB);
    for (int t = 0; t < CNN_NTAP; t++) {
      tc_tma_load_2d(sW + t*WTAPB, &tm_w, bW, 0, t*CNN_C);
    }
    int stage = 0;
    uint32_t phase = 0;
    uint32_t fills[CONV_STAGES];
    for (int s = 0; s < CONV_STAGES; s++) fills[s] = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile < g.ntiles; tile += gridDim.x) {
      int x, y0, z0;
      tile_decode(g, tile, x, y0, z0);
      for (int t = 0; t < CNN_NTAP; t++) {
	if (!tc_mbar_wait(bEmpty + 8*stage, phase ^ 1u, abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	int dx, dy, dz;
	tap_offsets(t, dx, dy, dz);
	tc_mbar_arrive_tx(bFull + 8*stage, TILEB);
	for (int l = 0; l < g.lpt; l++) {
	  const int row = prow(g, x + dx, y0 + l + dy, z0 + dz);
	  tc_tma_load_2d(sA + stage*TILEB + l*g.bz*ROWB, &tm_in,
			 bFull + 8*stage, 0, row);
	}
	fills[stage] += 1;
	if (++stage == CONV_STAGES) { stage = 0; phase ^= 1u; }
      }
    }
    /* drain: every copy issued has landed before the CTA may exit */
    tc_drain_wait(bW, 0, p.err);
    for (int s = 0; s < CONV_STAGES; s++) {
      if (fills[s]) tc_drain_wait(bFull + 8*s, (fills[s] - 1u) & 1u, p.err);
    }
  }
  else if (warp == 1 && lane == 0) {
    /* MMA issuer */
    constexpr uint32_t idesc = tc_idesc_bf16(128, CNN_C, 0, 0);
    bool ok = tc_mbar_wait(bW, 0, abort_flag, p.err);
    int stage = 0;
    uint32_t phase = 0;
    int i = 0;
    for (int tile = blockIdx.x; ok && tile < g.ntiles; tile += gridDim.x) {
      const int acc = i & 1;
      const uint32_t ap = (uint32_t) (i >> 1) & 1u;
      if (!tc_mbar_wait(bTEmpty + 8*acc, ap ^ 1u, abort_flag, p.err)) break;
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t) (acc*CNN_C);
      for (int t = 0; t < CNN_NTAP; t++) {
	if (!tc_mbar_wait(bFull + 8*stage, phase, abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	tc_fence_after();
	#pragma unroll
	for (int kh = 0; kh < 2; kh++) {
	  if (kh >= p.khn) break;
	  const uint64_t ad = tc_sdesc(sA + stage*TILEB + kh*32, 16, 512,
				       LGB_TC_SWIZZLE_64B);
	  const uint64_t bd = tc_sdesc(sW + t*WTAPB + kh*32, 16, 512,
				       LGB_TC_SWIZZLE_64B);
	  tc_mma_bf16(d, ad, bd, idesc, (uint32_t) ((t | kh) != 0));
	}
	tc_commit(bEmpty + 8*stage);
	if (++stage == CONV_STAGES) { stage = 0; phase ^= 1u; }
      }
      if (!ok) break;
      tc_commit(bTFull + 8*acc);
      i++;
    }
    tc_commit(bDone);
    tc_drain_wait(bDone, 0, p.err);
  }
  else if (warp >= 2) {
    /* epilogue: warp w reads TMEM lanes 32*(w % 4) .. +31 */
    /* warp w reads TMEM lanes 32*(w % 4) .. +31, columns c0 .. c0+15 */
    const int q = warp & 3;
    const int m = q*32 + lane;
    const int c0 = 16*((warp - 2) >> 2);
    float bias[16];
    #pragma unroll
    for (int n = 0; n < 16; n++) bias[n] = p.bias ? p.bias[c0 + n] : 0.0f;
    int i = 0;
    for (int tile = blockIdx.x; tile < g.ntiles; tile += gridDim.x) {
      const int acc = i & 1;
      const uint32_t ap = (uint32_t) (i >> 1) & 1u;
      bool okw = tc_mbar_wait(bTFull + 8*acc, ap, abort_flag, p.err);
      if (!__all_sync(0xffffffffu, okw)) break;
      tc_fence_after();
      uint32_t r[16];
      tc_tmem_ld16(tmem + (uint32_t) (acc*CNN_C + c0)
		   + ((uint32_t) (q*32) << 16), r);
      tc_fence_before();
      tc_mbar_arrive(bTEmpty + 8*acc);

      int x, y0, z0;
      tile_decode(g, tile, x, y0, z0);
      conv_epilogue<MODE>(p, bias, x, y0 + m / g.bz, z0 + (m % g.bz), c0,
			  r);
      i++;
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tc_tmem_dealloc(tmem, CONV_TMEM_COLS);
  }
}

/*****************************************************************************
 *  k_conv3_line: the same convolution for nz a multiple of 128, reusing
 *  neighbour lines.  A CTA walks a run of up to LN_YRUN tiles along y at
 *  fixed (x, z-chunk); a tile needs the 9 lines (x+dx, y+dy) of 130 rows
 *  (z0-1 .. z0+128), of which the next tile shares 6, so each tile loads
 *  only the 3 lines at y+1 (9 at the start of a run).  The three lines of
 *  one y (dx = -1, 0, 1) fill one of LN_NY ring slots in load order; a
 *  slot is refilled once the MMAs of the last tile that reads it have
 *  completed, so loads run up to LN_NY - 3 tiles ahead of the MMAs.  The A
 *  operand is stored without swizzle, as four planes of 8 channels x 130
 *  rows (16 bytes per row), so the three z taps of a line are the same
 *  planes at row offsets 0, 1, 2: start address + 16 bytes per row.
 *  L2 -> shared traffic per tile drops from 27 boxes of 128 rows to 3
 *  lines of 130 rows.
 *****************************************************************************/

#define LN_ROWS   130
#define LN_CHUNK  2176                  /* >= 130 x 16, 128-byte aligned */
#define LN_SLOT   (4*LN_CHUNK)
#define LN_NY     6                     /* y-line slots of the ring */
#define LN_NSLOT  (3*LN_NY)             /* 3 dx x LN_NY y-lines */
#define LN_YRUN   16
#define LN_TXLINE (4*LN_ROWS*16)        /* bytes of one line (4 planes) */
#define LN_XCH   4096                  /* boundary-row exchange (CYC) */
#define LN_OUTL  (3*LGBK_CNN_TILE*16)      /* FOLD: three output lines */
#define LN_SMEM (1024 + CNN_NTAP*WTAPB + LN_NSLOT*LN_SLOT + 256 + LN_XCH \
		 + LN_OUTL)

__device__ __forceinline__ void line_item(const lgbk_cnn_geom_t & g, int it,
					  int & x, int & z0, int & ya,
					  int & yb) {
  const int nzc = g.nz/LGBK_CNN_TILE;
  const int nyc = (g.ny + LN_YRUN - 1)/LN_YRUN;
  const int zc = it % nzc;
  const int r = it / nzc;
  const int yc = r % nyc;
  x = r / nyc;
  z0 = zc*LGBK_CNN_TILE;
  ya = yc*LN_YRUN;
  yb = min(g.ny, ya + LN_YRUN);
}

__host__ __device__ __forceinline__ int line_items(const lgbk_cnn_geom_t & g) {
  return g.nx*(g.nz/LGBK_CNN_TILE)*((g.ny + LN_YRUN - 1)/LN_YRUN);
}

/* 16-byte shared-memory store and load (32-bit shared addresses) */
__device__ __forceinline__ void lds_st4(uint32_t a, const uint32_t v[4]) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};"
	       :: "r"(a), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3])
	       : "memory");
}
__device__ __forceinline__ void lds_ld4(uint32_t a, uint32_t v[4]) {
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];"
	       : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
	       : "r"(a) : "memory");
}

/* SWZ = 0: a line is 4 unswizzled planes (8 channels x 130 rows, 16 bytes
 * a row; TMA box 8 x 130 each), z taps at +16 bytes per row.
 * SWZ = 1: a line is 130 rows of 64 bytes with the 64-byte swizzle (one
 * TMA box 32 x 130), z taps at +64 bytes per row; this relies on the
 * swizzle being a function of the absolute shared-memory address, which
 * the checks against the one-box-per-tap kernel establish.
 *
 * CYC = 1 (nz = 128: a line is the whole periodic z extent): the three z
 * taps of a line share one MMA of N = 96, A = the line's 128 interior rows
 * and B = the three taps' weights (consecutive in shared memory), so the
 * A tile is read once per line instead of three times.  The accumulator
 * holds D_dz[r] = sum over the lines of x(r) W_dz in columns 32 (dz + 1)
 * .. + 31, and the output is out(r) = D_-1[r - 1] + D_0[r] + D_+1[r + 1]
 * with r - 1, r + 1 taken modulo 128: the epilogue moves the two shifted
 * terms one TMEM lane with warp shuffles, and across the four warps of a
 * group through shared memory (16-byte accesses, an mbarrier per group
 * and buffer, bounded waits).  The two groups of four epilogue warps take
 * alternate tiles (the accumulator parity), each warp both channel
 * halves, and write the periodic images of the rows they store (no halo
 * pass).  Sums in another order than the one-box-per-tap kernel: equal to
 * FP32 rounding, not bit for bit.
 *
 * The ring also runs on 64-byte-swizzled lines (SWZ = 1: one TMA box a
 * line instead of four boxes of 16-byte rows), the default form. */
/* FOLD = 1 (the last layer, 4 outputs, with CYC): the y taps go into N
 * as well.  Each step takes one new y-line (x-1, x, x+1 at y') and issues
 * one MMA per dx and K half with B = the 48 rows [dz][dy][4 outputs] (12
 * of each 16 used; weights rearranged by k_cnn_wfold, nine 16-row blocks
 * (dx, dz)), so that a tile costs 6 MMAs instead of 18.  The accumulator
 * then holds, per dz, the contributions of line y' to the output lines
 * y' + 1 (dy = -1), y' and y' - 1; the epilogue combines the dz taps as in
 * the three-tap form and adds the three dy parts into three running output
 * lines in shared memory, writing line y' - 1 once line y' has been
 * added; the two groups of epilogue warps take alternate steps, and each
 * step adds its parts after the previous one's (a token per step
 * parity), so that every line is summed in step order.  A run of output lines ya .. yb - 1 takes the lines ya - 1 .. yb:
 * the same lines, in the same order, as the other forms load. */
template <int MODE, int SWZ, int CYC, int FOLD>
__global__ void __launch_bounds__(CONV_THREADS, 1)
k_conv3_line(const __grid_constant__ CUtensorMap tm_line,
	     const __grid_constant__ CUtensorMap tm_w, const ConvP p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc_smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t * sgen = smem_raw + (sbase - raw);

  const uint32_t sW = sbase;
  const uint32_t sL = sW + CNN_NTAP*WTAPB;
  const uint32_t sBar = sL + LN_NSLOT*LN_SLOT;
  const uint32_t bFull = sBar;                 /* LN_NY, per ring slot */
  const uint32_t bRel = sBar + 8*LN_NY;        /* LN_NY, per ring slot */
  const uint32_t bW = sBar + 16*LN_NY;
  const uint32_t bTFull = bW + 8;
  const uint32_t bTEmpty = bW + 24;
  const uint32_t bFin = bW + 40;
  uint32_t * tslot = (uint32_t *) (sgen + (bW + 48 - sbase));
  volatile int * abort_flag = (volatile int *) (sgen + (bW + 52 - sbase));
  const uint32_t bX = bW + 56;                 /* 4: [channel half][parity] */
  const uint32_t bTok = bW + 88;               /* FOLD: 2, [step parity] */
  const uint32_t sXch = sBar + 256;            /* [half][parity][quarter] */
  const uint32_t sOut = sXch + LN_XCH;         /* FOLD: [3][128][4] floats */
  /* accumulator columns per tile and TMEM columns allocated */
  /* accumulator columns per tile (three taps of nb outputs each in the
   * three-tap form) and TMEM columns allocated */
  const int nbk = CYC ? p.nb : CNN_C;
  /* the two groups of epilogue warps take alternate tiles (three-tap
   * form, not folded) */
  constexpr bool ALT = CYC && !FOLD;
  const uint32_t NACC = CYC ? 3u*(uint32_t) nbk : (uint32_t) CNN_C;
  constexpr uint32_t TCOLS = CYC ? 256 : CONV_TMEM_COLS;

  const int warp = threadIdx.x/32;
  const int lane = threadIdx.x % 32;
  const lgbk_cnn_geom_t & g = p.g;
  const int nitems = line_items(g);

  if (threadIdx.x == 0) {
    for (int k = 0; k < LN_NY; k++) {
      tc_mbar_init(bFull + 8*k, 1);
      tc_mbar_init(bRel + 8*k, 1);
    }
    for (int k = 0; k < 4; k++) tc_mbar_init(bX + 8*k, 8);
    tc_mbar_init(bTok, 128);
    tc_mbar_init(bTok + 8, 128);
    tc_mbar_init(bW, 1);
    tc_mbar_init(bTFull, 1);
    tc_mbar_init(bTFull + 8, 1);
    /* ALT: one group of four epilogue warps releases each accumulator */
    tc_mbar_init(bTEmpty, (ALT || FOLD) ? 128 : CONV_EPI_THREADS);
    tc_mbar_init(bTEmpty + 8, (ALT || FOLD) ? 128 : CONV_EPI_THREADS);
    tc_mbar_init(bFin, 1);
    *abort_flag = 0;
    tc_fence_barrier_init();
  }
  if (warp == 1) tc_tmem_alloc(tc_smem_u32(tslot), TCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    tc_prefetch_map(&tm_line);
    tc_prefetch_map(&tm_w);
    /* the first nb output rows of every tap's weights (FOLD: of the
     * nine (dx, dz) blocks) */
    const uint32_t wtap = (uint32_t) (CYC ? p.nb : CNN_C)*ROWB;
    constexpr int NTW = FOLD ? 9 : CNN_NTAP;
    tc_mbar_arrive_tx(bW, NTW*wtap);
    for (int t = 0; t < NTW; t++) {
      tc_tma_load_2d(sW + t*wtap, &tm_w, bW, 0, t*CNN_C);
    }
    /* y-lines are numbered in load order (sq); line sq fills ring slot
     * sq % LN_NY, after line sq - LN_NY has been released */
    uint32_t sq = 0;
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; ok && y < yb; y++) {
	const bool first = (y == ya);
	const int nl = first ? 3 : 1;
	for (int li = 0; li < nl; li++, sq++) {
	  const int yy = first ? (y - 1 + li) : (y + 1);
	  const uint32_t r = sq % LN_NY;
	  if (sq >= LN_NY &&
	      !tc_mbar_wait(bRel + 8*r, (sq/LN_NY - 1u) & 1u, abort_flag,
			    p.err)) {
	    ok = false;
	    break;
	  }
	  const uint32_t bar = bFull + 8*r;
	  tc_mbar_arrive_tx(bar, 3*LN_TXLINE);
	  for (int dxi = 0; dxi < 3; dxi++) {
	    const uint32_t dst = sL + (uint32_t) (dxi*LN_NY + r)*LN_SLOT;
	    const int row = prow(g, x + dxi - 1, yy, z0 - 1);
	    if (SWZ) {
	      tc_tma_load_2d(dst, &tm_line, bar, 0, row);
	    }
	    else {
	      for (int c = 0; c < 4; c++) {
		tc_tma_load_2d(dst + c*LN_CHUNK, &tm_line, bar, 8*c, row);
	      }
	    }
	  }
	}
      }
    }
    tc_drain_wait(bW, 0, p.err);
    /* the last fill of every slot used (earlier fills were consumed before
     * their slot was refilled) */
    for (uint32_t r = 0; r < LN_NY && r < sq; r++) {
      const uint32_t nfill = (sq - r + LN_NY - 1)/LN_NY;
      tc_drain_wait(bFull + 8*r, (nfill - 1u) & 1u, p.err);
    }
  }
  else if (warp == 1 && lane == 0) {
    const uint32_t idesc = tc_idesc_bf16(128, (int) NACC, 0, 0);
    /* descriptors of the first ring slot and of the first tap's weights */
    const uint64_t ad0 = SWZ
      ? tc_sdesc(sL, 16, 512, LGB_TC_SWIZZLE_64B)
      : tc_sdesc(sL, LN_CHUNK, 128, 0u);
    const uint64_t bd0 = tc_sdesc(sW, 16, 512, LGB_TC_SWIZZLE_64B);
    const uint32_t alo0 = (uint32_t) ad0, ahi = (uint32_t) (ad0 >> 32);
    const uint32_t blo0 = (uint32_t) bd0, bhi = (uint32_t) (bd0 >> 32);
    bool ok = tc_mbar_wait(bW, 0, abort_flag, p.err);
    uint32_t sq = 0;                   /* y-lines consumed, as loaded */
    int i = 0;
    for (int it = blockIdx.x; ok && FOLD && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      /* one step per y-line ya - 1 .. yb, as loaded */
      for (int y = ya - 1; y <= yb; y++, i++, sq++) {
	const int acc = i & 1;
	if (!tc_mbar_wait(bTEmpty + 8*acc, ((uint32_t) (i >> 1) & 1u) ^ 1u,
			  abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	const uint32_t r = sq % LN_NY;
	if (!tc_mbar_wait(bFull + 8*r, (sq/LN_NY) & 1u, abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	tc_fence_after();
	constexpr uint32_t DXS = LN_NY*LN_SLOT >> 4;
	constexpr uint32_t DZS = (SWZ ? ROWB : 16) >> 4;
	constexpr uint32_t KHA = (SWZ ? 32 : 2*LN_CHUNK) >> 4;
	constexpr uint32_t KHB = 32 >> 4;
	const uint32_t a0 = alo0 + r*(LN_SLOT >> 4) + DZS;
	const uint32_t d = tmem + (uint32_t) acc*NACC;
	#pragma unroll
	for (int dxi = 0; dxi < 3; dxi++) {
	  #pragma unroll
	  for (int kh = 0; kh < 2; kh++) {
	    if (kh >= p.khn) break;
	    tc_mma_bf16_w(d, a0 + (uint32_t) dxi*DXS + kh*KHA, ahi,
			  blo0 + (uint32_t) (3*dxi*nbk*ROWB >> 4) + kh*KHB,
			  bhi, idesc, (uint32_t) ((dxi | kh) != 0));
	  }
	}
	/* no later step reads this line */
	tc_commit(bRel + 8*r);
	tc_commit(bTFull + 8*acc);
      }
    }
    for (int it = blockIdx.x; ok && !FOLD && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; y < yb; y++, i++) {
	const int acc = i & 1;
	const bool first = (y == ya), last = (y == yb - 1);
	if (!tc_mbar_wait(bTEmpty + 8*acc, ((uint32_t) (i >> 1) & 1u) ^ 1u,
			  abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	for (int li = 0; ok && li < (first ? 3 : 1); li++, sq++) {
	  ok = tc_mbar_wait(bFull + 8*(sq % LN_NY), (sq/LN_NY) & 1u,
			    abort_flag, p.err);
	}
	if (!ok) break;
	tc_fence_after();
	/* low descriptor words of the lines y-1, y, y+1 at dx = -1 (ring
	 * slots of the three y-lines); dx steps by LN_NY slots, z taps and
	 * K halves by fixed byte offsets: one addition per MMA operand */
	const uint32_t rr[3] = {(sq - 3u) % LN_NY, (sq - 2u) % LN_NY,
				(sq - 1u) % LN_NY};
	const uint32_t aln[3] = {alo0 + rr[0]*(LN_SLOT >> 4),
				 alo0 + rr[1]*(LN_SLOT >> 4),
				 alo0 + rr[2]*(LN_SLOT >> 4)};
	constexpr uint32_t DXS = LN_NY*LN_SLOT >> 4;
	constexpr uint32_t DZS = (SWZ ? ROWB : 16) >> 4;
	constexpr uint32_t KHA = (SWZ ? 32 : 2*LN_CHUNK) >> 4;
	constexpr uint32_t KHB = 32 >> 4;
	const uint32_t d = tmem + (uint32_t) acc*NACC;
	if (CYC) {
	  /* one MMA per line (dx, dy) and K half: the three z taps' weights
	   * (taps 3 ln .. 3 ln + 2) as N = 96, A = rows z0 .. z0 + 127 */
	  #pragma unroll
	  for (int ln = 0; ln < 9; ln++) {
	    const uint32_t a = aln[ln % 3] + (uint32_t) (ln/3)*DXS + DZS;
	    #pragma unroll
	    for (int kh = 0; kh < 2; kh++) {
	      if (kh >= p.khn) break;
	      tc_mma_bf16_w(d, a + kh*KHA, ahi,
			    blo0 + (uint32_t) (3*ln*nbk*ROWB >> 4) + kh*KHB,
			    bhi, idesc, (uint32_t) ((ln | kh) != 0));
	    }
	  }
	}
	else {
	  #pragma unroll
	  for (int t = 0; t < CNN_NTAP; t++) {
	    const int dxi = t/9, dyi = (t/3) % 3, dzi = t % 3;
	    const uint32_t a = aln[dyi] + (uint32_t) dxi*DXS + dzi*DZS;
	    #pragma unroll
	    for (int kh = 0; kh < 2; kh++) {
	      if (kh >= p.khn) break;
	      tc_mma_bf16_w(d, a + kh*KHA, ahi, blo0 + (t*WTAPB >> 4)
			    + kh*KHB, bhi, idesc, (uint32_t) ((t | kh) != 0));
	    }
	  }
	}
	/* the next tile of the run does not read line y-1; after the last
	 * tile of a run none of the three is read again */
	tc_commit(bRel + 8*rr[0]);
	if (last) {
	  tc_commit(bRel + 8*rr[1]);
	  tc_commit(bRel + 8*rr[2]);
	}
	tc_commit(bTFull + 8*acc);
      }
    }
    tc_commit(bFin);
    tc_drain_wait(bFin, 0, p.err);
  }
  else if (ALT && warp >= 2) {
    /* Warps 2-5 take the even tiles (accumulator 0), warps 6-9 the odd
     * ones, so that two tiles' epilogues overlap; warp w reads TMEM lanes
     * 32 (w % 4) .. + 31 and both channel halves (one where the layer has
     * 16 weight rows a tap).  The shifted terms of the interior rows are
     * added before the edge rows' exchange completes. */
    const int grp = (warp - 2) >> 2;
    const int q = warp & 3;
    const int m = q*32 + lane;
    const bool two = (nbk > 16);
    float bias[32];
    #pragma unroll
    for (int n = 0; n < 32; n++) bias[n] = p.bias ? p.bias[n] : 0.0f;
    int i = 0;
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; y < yb; y++, i++) {
	if ((i & 1) != grp) continue;
	const int acc = grp;
	/* backward: this site's stored slopes GELU'(z), loaded before the
	 * accumulator is waited for */
	uint4 zq[4];
	if (MODE == LGBK_CNN_BWD_GELU) {
	  const long long sq = ((long long) x*g.ny + y)*g.nz + z0 + m;
	  const uint4 * zr = (const uint4 *) (p.zprev + sq*ROWB);
	  zq[0] = zr[0];
	  zq[1] = zr[1];
	  if (two) {
	    zq[2] = zr[2];
	    zq[3] = zr[3];
	  }
	}
	bool okw = tc_mbar_wait(bTFull + 8*acc, (uint32_t) (i >> 1) & 1u,
				abort_flag, p.err);
	if (!__all_sync(0xffffffffu, okw)) { ok = false; break; }
	tc_fence_after();
	const uint32_t ta = tmem + (uint32_t) acc*NACC
	  + ((uint32_t) (q*32) << 16);
	uint32_t rm0[16], r0[16], rp0[16], rm1[16], r1[16], rp1[16];
	tc_tmem_ld16_async(ta, rm0);                 /* D_-1 */
	tc_tmem_ld16_async(ta + nbk, r0);            /* D_0 */
	tc_tmem_ld16_async(ta + 2*nbk, rp0);         /* D_+1 */
	if (two) {
	  tc_tmem_ld16_async(ta + 16, rm1);
	  tc_tmem_ld16_async(ta + nbk + 16, r1);
	  tc_tmem_ld16_async(ta + 2*nbk + 16, rp1);
	}
	tc_tmem_wait_ld16x3(rm0, r0, rp0);
	if (two) tc_tmem_wait_ld16x3(rm1, r1, rp1);
	tc_fence_before();
	tc_mbar_arrive(bTEmpty + 8*acc);
	/* edge rows: slot [group][buffer][quarter] of 256 bytes, lane 31's
	 * D_-1 (bytes 0-127, both halves) and lane 0's D_+1 (128-255); a
	 * group's consecutive tiles alternate between two buffers */
	const int xb = grp*2 + ((i >> 1) & 1);
	const uint32_t sx = sXch + (uint32_t) (xb*4)*256u;
	if (lane == 31) {
	  #pragma unroll
	  for (int k = 0; k < 4; k++) {
	    lds_st4(sx + (uint32_t) q*256u + 16u*k, rm0 + 4*k);
	    if (two) lds_st4(sx + (uint32_t) q*256u + 64u + 16u*k, rm1 + 4*k);
	  }
	  tc_mbar_arrive(bX + 8*xb);
	}
	if (lane == 0) {
	  #pragma unroll
	  for (int k = 0; k < 4; k++) {
	    lds_st4(sx + (uint32_t) q*256u + 128u + 16u*k, rp0 + 4*k);
	    if (two) lds_st4(sx + (uint32_t) q*256u + 192u + 16u*k, rp1 + 4*k);
	  }
	  tc_mbar_arrive(bX + 8*xb);
	}
	/* out(r) = D_-1[r - 1] + D_0[r] + D_+1[r + 1]: within the warp by
	 * shuffles; lane 0's D_-1 and lane 31's D_+1 term come next */
	#pragma unroll
	for (int n = 0; n < 16; n++) {
	  float dm = __shfl_up_sync(0xffffffffu, __uint_as_float(rm0[n]), 1);
	  float dp = __shfl_down_sync(0xffffffffu, __uint_as_float(rp0[n]), 1);
	  if (lane == 0) dm = 0.0f;
	  if (lane == 31) dp = 0.0f;
	  r0[n] = __float_as_uint((__uint_as_float(r0[n]) + dm) + dp);
	}
	if (two) {
	  #pragma unroll
	  for (int n = 0; n < 16; n++) {
	    float dm = __shfl_up_sync(0xffffffffu, __uint_as_float(rm1[n]), 1);
	    float dp = __shfl_down_sync(0xffffffffu, __uint_as_float(rp1[n]),
					1);
	    if (lane == 0) dm = 0.0f;
	    if (lane == 31) dp = 0.0f;
	    r1[n] = __float_as_uint((__uint_as_float(r1[n]) + dm) + dp);
	  }
	}
	const bool okx = tc_mbar_wait(bX + 8*xb, (uint32_t) (i >> 2) & 1u,
				      abort_flag, p.err);
	if (!__all_sync(0xffffffffu, okx)) { ok = false; break; }
	if (lane == 0 || lane == 31) {
	  /* lane 0: row 32 q - 1's D_-1; lane 31: row 32 q + 32's D_+1 */
	  const uint32_t src = (lane == 0)
	    ? sx + (uint32_t) ((q + 3) & 3)*256u
	    : sx + (uint32_t) ((q + 1) & 3)*256u + 128u;
	  uint32_t ev[16];
	  #pragma unroll
	  for (int k = 0; k < 4; k++) lds_ld4(src + 16u*k, ev + 4*k);
	  #pragma unroll
	  for (int n = 0; n < 16; n++) {
	    r0[n] = __float_as_uint(__uint_as_float(r0[n])
				    + __uint_as_float(ev[n]));
	  }
	  if (two) {
	    #pragma unroll
	    for (int k = 0; k < 4; k++) lds_ld4(src + 64u + 16u*k, ev + 4*k);
	    #pragma unroll
	    for (int n = 0; n < 16; n++) {
	      r1[n] = __float_as_uint(__uint_as_float(r1[n])
				      + __uint_as_float(ev[n]));
	    }
	  }
	}
	if (MODE == LGBK_CNN_BWD_GELU) {
	  conv_epilogue_bwd(p, x, y, z0 + m, 0, r0, zq);
	  if (two) conv_epilogue_bwd(p, x, y, z0 + m, 16, r1, zq + 2);
	}
	else {
	  /* padded rows with their periodic images (no halo pass) */
	  conv_epilogue<MODE, true>(p, bias, x, y, z0 + m, 0, r0);
	  if (two) {
	    conv_epilogue<MODE, true>(p, bias + 16, x, y, z0 + m, 16, r1);
	  }
	}
      }
    }
  }
  else if (FOLD && warp >= 2) {
    /* The two groups of four warps take alternate steps (y-lines).  A
     * step's three y parts go into three running output lines in shared
     * memory (this thread's row of each), after the previous step's parts
     * (a token per step parity, 128 arrivals), so that every line is
     * summed in step order; the line a step completes is written out and
     * its slot cleared for the line three further on. */
    const int grp = (warp - 2) >> 2;
    const int q = warp & 3;
    const int m = q*32 + lane;
    float bias4[LGBK_CNN_NOUT];
    #pragma unroll
    for (int c = 0; c < LGBK_CNN_NOUT; c++) bias4[c] = p.bias ? p.bias[c] : 0.0f;
    auto line_slot = [&](int ln) {
      return sOut + (uint32_t) (((ln % 3) + 3) % 3)*(LGBK_CNN_TILE*16)
	+ (uint32_t) m*16u;
    };
    if (grp == 0) {
      /* the lines start cleared (by the group of step 0; the other group
       * first touches them after step 0's token) */
      const uint32_t zero[4] = {0u, 0u, 0u, 0u};
      #pragma unroll
      for (int k = 0; k < 3; k++) lds_st4(line_slot(k), zero);
    }
    int i = 0;
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya - 1; y <= yb; y++, i++) {
	if ((i & 1) != grp) continue;
	const int acc = grp;
	bool okw = tc_mbar_wait(bTFull + 8*acc, (uint32_t) (i >> 1) & 1u,
				abort_flag, p.err);
	if (!__all_sync(0xffffffffu, okw)) { ok = false; break; }
	tc_fence_after();
	const uint32_t ta = tmem + (uint32_t) acc*NACC
	  + ((uint32_t) (q*32) << 16);
	uint32_t rm[16], r[16], rp[16];
	tc_tmem_ld16_async(ta, rm);                  /* D_-1 */
	tc_tmem_ld16_async(ta + nbk, r);             /* D_0 */
	tc_tmem_ld16_async(ta + 2*nbk, rp);          /* D_+1 */
	tc_tmem_wait_ld16x3(rm, r, rp);
	tc_fence_before();
	tc_mbar_arrive(bTEmpty + 8*acc);
	/* edge rows: slot [group][buffer][quarter] of 128 bytes, lane 31's
	 * D_-1 (0-63) and lane 0's D_+1 (64-127) */
	const int xb = grp*2 + ((i >> 1) & 1);
	const uint32_t sx = sXch + (uint32_t) (xb*4)*128u;
	if (lane == 31) {
	  #pragma unroll
	  for (int k = 0; k < 4; k++) {
	    lds_st4(sx + (uint32_t) q*128u + 16u*k, rm + 4*k);
	  }
	  tc_mbar_arrive(bX + 8*xb);
	}
	if (lane == 0) {
	  #pragma unroll
	  for (int k = 0; k < 4; k++) {
	    lds_st4(sx + (uint32_t) q*128u + 64u + 16u*k, rp + 4*k);
	  }
	  tc_mbar_arrive(bX + 8*xb);
	}
	#pragma unroll
	for (int n = 0; n < 12; n++) {
	  float dm = __shfl_up_sync(0xffffffffu, __uint_as_float(rm[n]), 1);
	  float dp = __shfl_down_sync(0xffffffffu, __uint_as_float(rp[n]), 1);
	  if (lane == 0) dm = 0.0f;
	  if (lane == 31) dp = 0.0f;
	  r[n] = __float_as_uint((__uint_as_float(r[n]) + dm) + dp);
	}
	const bool okx = tc_mbar_wait(bX + 8*xb, (uint32_t) (i >> 2) & 1u,
				      abort_flag, p.err);
	if (!__all_sync(0xffffffffu, okx)) { ok = false; break; }
	if (lane == 0 || lane == 31) {
	  /* lane 0: row 32 q - 1's D_-1; lane 31: row 32 q + 32's D_+1 */
	  const uint32_t src = (lane == 0)
	    ? sx + (uint32_t) ((q + 3) & 3)*128u
	    : sx + (uint32_t) ((q + 1) & 3)*128u + 64u;
	  uint32_t ev[16];
	  #pragma unroll
	  for (int k = 0; k < 4; k++) lds_ld4(src + 16u*k, ev + 4*k);
	  #pragma unroll
	  for (int n = 0; n < 12; n++) {
	    r[n] = __float_as_uint(__uint_as_float(r[n])
				   + __uint_as_float(ev[n]));
	  }
	}
	/* the previous step's parts are in */
	if (i > 0) {
	  const bool okt = tc_mbar_wait(bTok + 8*((i - 1) & 1),
					(uint32_t) ((i - 1) >> 1) & 1u,
					abort_flag, p.err);
	  if (!__all_sync(0xffffffffu, okt)) { ok = false; break; }
	}
	/* column 4 dyi + c: the part of output line y + 1 - dyi */
	#pragma unroll
	for (int dyi = 0; dyi < 3; dyi++) {
	  const uint32_t a = line_slot(y + 1 - dyi);
	  uint32_t v[4];
	  lds_ld4(a, v);
	  #pragma unroll
	  for (int c = 0; c < LGBK_CNN_NOUT; c++) {
	    v[c] = __float_as_uint(__uint_as_float(v[c])
				   + __uint_as_float(r[4*dyi + c]));
	  }
	  if (dyi < 2) lds_st4(a, v);
	  else if (y - 1 >= ya) {
	    /* line y - 1 is complete */
	    const long long sy = ((long long) x*g.ny + (y - 1))*g.nz + z0 + m;
	    #pragma unroll
	    for (int c = 0; c < LGBK_CNN_NOUT; c++) {
	      p.outf[c*g.nsites + sy] = __uint_as_float(v[c]) + bias4[c];
	    }
	  }
	}
	{
	  /* clear the completed line's slot; after the run's last step the
	   * two lines past the run as well */
	  const uint32_t zero[4] = {0u, 0u, 0u, 0u};
	  lds_st4(line_slot(y - 1), zero);
	  if (y == yb) {
	    lds_st4(line_slot(y), zero);
	    lds_st4(line_slot(y + 1), zero);
	  }
	}
	tc_mbar_arrive(bTok + 8*(i & 1));
      }
    }
  }
  else if (!FOLD && warp >= 2) {
    /* warp w reads TMEM lanes 32*(w % 4) .. +31, columns c0 .. c0+15 */
    const int q = warp & 3;
    const int m = q*32 + lane;
    const int c0 = 16*((warp - 2) >> 2);
    float bias[16];
    #pragma unroll
    for (int n = 0; n < 16; n++) bias[n] = p.bias ? p.bias[c0 + n] : 0.0f;
    int i = 0;
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; y < yb; y++, i++) {
	const int acc = i & 1;
	bool okw = tc_mbar_wait(bTFull + 8*acc, (uint32_t) (i >> 1) & 1u,
				abort_flag, p.err);
	if (!__all_sync(0xffffffffu, okw)) { ok = false; break; }
	tc_fence_after();
	uint32_t r[16];
	const uint32_t ta = tmem + (uint32_t) acc*NACC + (uint32_t) c0
	  + ((uint32_t) (q*32) << 16);
	if (CYC && c0 >= nbk) {
	  /* no accumulator columns for this channel half */
	  tc_fence_before();
	  tc_mbar_arrive(bTEmpty + 8*acc);
	  continue;
	}
	if (CYC) {
	  uint32_t rm[16], rp[16];
	  tc_tmem_ld16_async(ta, rm);                /* D_-1, this row */
	  tc_tmem_ld16_async(ta + nbk, r);           /* D_0 */
	  tc_tmem_ld16_async(ta + 2*nbk, rp);        /* D_+1 */
	  tc_tmem_wait_ld16x3(rm, r, rp);
	  tc_fence_before();
	  tc_mbar_arrive(bTEmpty + 8*acc);
	  /* rows 32 q - 1 and 32 q + 32 belong to the neighbouring warps
	   * of this channel half: publish this warp's edge rows */
	  /* 16-byte shared-memory accesses only: the tensor core's operand
	   * reads keep the shared-memory banks busy, and each access waits
	   * its turn (four-byte accesses here cost more than the MMAs) */
	  const int grp = (warp - 2) >> 2;
	  const int xb = grp*2 + (i & 1);
	  const uint32_t sx = sXch + (uint32_t) (xb*4)*128u;
	  /* lanes 31 and 0 each publish and arrive (8 arrivals a phase):
	   * slot q holds lane 31's D_-1 (bytes 0-63), lane 0's D_+1 (64-127) */
	  if (lane == 31) {
	    #pragma unroll
	    for (int k = 0; k < 4; k++) {
	      lds_st4(sx + (uint32_t) q*128u + 16u*k, rm + 4*k);
	    }
	    tc_mbar_arrive(bX + 8*xb);
	  }
	  if (lane == 0) {
	    #pragma unroll
	    for (int k = 0; k < 4; k++) {
	      lds_st4(sx + (uint32_t) q*128u + 64u + 16u*k, rp + 4*k);
	    }
	    tc_mbar_arrive(bX + 8*xb);
	  }
	  /* the interior rows' shifted terms while the exchange completes */
	  #pragma unroll
	  for (int n = 0; n < 16; n++) {
	    float dm = __shfl_up_sync(0xffffffffu, __uint_as_float(rm[n]), 1);
	    float dp = __shfl_down_sync(0xffffffffu, __uint_as_float(rp[n]), 1);
	    if (lane == 0) dm = 0.0f;
	    if (lane == 31) dp = 0.0f;
	    r[n] = __float_as_uint((__uint_as_float(r[n]) + dm) + dp);
	  }
	  const bool okx = tc_mbar_wait(bX + 8*xb, (uint32_t) (i >> 1) & 1u,
					abort_flag, p.err);
	  if (!__all_sync(0xffffffffu, okx)) { ok = false; break; }
	  /* lane 0: row 32 q - 1's D_-1; lane 31: row 32 q + 32's D_+1 */
	  if (lane == 0 || lane == 31) {
	    uint32_t ev[16];
	    const uint32_t src = (lane == 0)
	      ? sx + (uint32_t) ((q + 3) & 3)*128u
	      : sx + (uint32_t) ((q + 1) & 3)*128u + 64u;
	    #pragma unroll
	    for (int k = 0; k < 4; k++) lds_ld4(src + 16u*k, ev + 4*k);
	    #pragma unroll
	    for (int n = 0; n < 16; n++) {
	      r[n] = __float_as_uint(__uint_as_float(r[n])
				     + __uint_as_float(ev[n]));
	    }
	  }
	}
	else {
	  tc_tmem_ld16(ta, r);
	  tc_fence_before();
	  tc_mbar_arrive(bTEmpty + 8*acc);
	}
	conv_epilogue<MODE>(p, bias, x, y, z0 + m, c0, r);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tc_tmem_dealloc(tmem, TCOLS);
  }
}

template <int MODE, int SWZ, int CYC, int FOLD = 0>
static cudaError_t launch_line(const lgbk_cnn_geom_t * g,
			       const CUtensorMap & ml, const CUtensorMap & mw,
			       const ConvP & p, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_conv3_line<MODE, SWZ, CYC, FOLD>,
    cudaFuncAttributeMaxDynamicSharedMemorySize, LN_SMEM);
  if (e != cudaSuccess) return e;
  int grid = line_items(*g);
  const int nsm = num_sms();
  if (grid > nsm) grid = nsm;
  k_conv3_line<MODE, SWZ, CYC, FOLD><<<grid, CONV_THREADS, LN_SMEM, s>>>(
    ml, mw, p);
  return cudaSuccess;
}

template <int MODE>
static cudaError_t launch_conv(const lgbk_cnn_geom_t * g, const CUtensorMap & mi,
			       const CUtensorMap * ml, int line_kind,
			       const CUtensorMap & mw, const ConvP & p,
			       cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (ml) {
    if (line_kind == 4 || line_kind == 6) {
      /* y taps folded into N: the last layer only; 6 on swizzled lines */
      if (MODE != LGBK_CNN_FWD_OUT || g->nz != LGBK_CNN_TILE ||
	  p.nb != 16) {
	return cudaErrorInvalidValue;
      }
      if constexpr (MODE == LGBK_CNN_FWD_OUT) {
	e = (line_kind == 6) ? launch_line<MODE, 1, 1, 1>(g, *ml, mw, p, s)
	                     : launch_line<MODE, 0, 1, 1>(g, *ml, mw, p, s);
      }
    }
    else if (line_kind == 3) {
      if (g->nz != LGBK_CNN_TILE) return cudaErrorInvalidValue;
      e = launch_line<MODE, 0, 1>(g, *ml, mw, p, s);
    }
    else if (line_kind == 5) {
      /* the three-tap form on 64-byte-swizzled lines (one box a line) */
      if (g->nz != LGBK_CNN_TILE) return cudaErrorInvalidValue;
      e = launch_line<MODE, 1, 1>(g, *ml, mw, p, s);
    }
    else if (line_kind == 2) {
      e = launch_line<MODE, 1, 0>(g, *ml, mw, p, s);
    }
    else {
      e = launch_line<MODE, 0, 0>(g, *ml, mw, p, s);
    }
    if (e != cudaSuccess) return e;
  }
  else {
    e = cudaFuncSetAttribute(k_conv3_tc<MODE>,
			     cudaFuncAttributeMaxDynamicSharedMemorySize,
			     CONV_SMEM);
    if (e != cudaSuccess) return e;
    k_conv3_tc<MODE><<<lgbk_cnn_conv_blocks(g), CONV_THREADS, CONV_SMEM, s>>>(
      mi, mw, p);
  }
  return cudaGetLastError();
}

extern "C" int lgbk_cnn_conv(const lgbk_cnn_geom_t * g, int mode, int kin, int wrows,
			     const void * tm_in, const void * tm_line,
			     int line_kind, const void * tm_w, const float * bias,
			     const void * zprev, void * zout, void * pout,
			     float * outf, int * err, void * stream) {
  ConvP p;
  p.g = *g;
  p.bias = bias;
  p.zprev = (const uint8_t *) zprev;
  p.zout = (uint8_t *) zout;
  p.pout = (uint8_t *) pout;
  p.outf = outf;
  p.err = err;
  if (kin != 16 && kin != CNN_C) return (int) cudaErrorInvalidValue;
  p.khn = kin/16;
  p.nb = wrows;
  const CUtensorMap mi = *(const CUtensorMap *) tm_in;
  const CUtensorMap mw = *(const CUtensorMap *) tm_w;
  const CUtensorMap * ml = NULL;
  CUtensorMap mlv;
  if (tm_line && g->bz == LGBK_CNN_TILE && g->lpt == 1) {
    mlv = *(const CUtensorMap *) tm_line;
    ml = &mlv;
  }
  /* 16 weight rows per tap (tm_w boxes of 16 rows): only where the
   * three-tap line form runs */
  if (wrows != CNN_C &&
      !(wrows == 16 && ml && line_kind >= 3 && line_kind <= 6 &&
	g->nz == LGBK_CNN_TILE)) {
    return (int) cudaErrorInvalidValue;
  }
  if ((line_kind == 4 || line_kind == 6) &&
      (wrows != 16 || mode != LGBK_CNN_FWD_OUT)) {
    return (int) cudaErrorInvalidValue;
  }
  cudaStream_t s = (cudaStream_t) stream;
  cudaError_t e;
  switch (mode) {
  case LGBK_CNN_FWD_GELU:
    e = launch_conv<LGBK_CNN_FWD_GELU>(g, mi, ml, line_kind, mw, p, s); break;
  case LGBK_CNN_FWD_OUT:
    e = launch_conv<LGBK_CNN_FWD_OUT>(g, mi, ml, line_kind, mw, p, s); break;
  case LGBK_CNN_BWD_GELU:
    e = launch_conv<LGBK_CNN_BWD_GELU>(g, mi, ml, line_kind, mw, p, s); break;
  case LGBK_CNN_RAW:
    e = launch_conv<LGBK_CNN_RAW>(g, mi, ml, line_kind, mw, p, s); break;
  default:
    return (int) cudaErrorInvalidValue;
  }
  return (int) e;
}

/*****************************************************************************
 *  k_wgrad_tc
 *****************************************************************************/

struct WgP {
  lgbk_cnn_geom_t g;
  float * part;
  int * err;
};

__global__ void __launch_bounds__(WG_THREADS, 1)
k_wgrad_tc(const __grid_constant__ CUtensorMap tm_g,
	   const __grid_constant__ CUtensorMap tm_x, const WgP p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc_smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t * sgen = smem_raw + (sbase - raw);

  const uint32_t sX = sbase;
  const uint32_t sA = sX + WG_XSTAGES*TILEB;
  const uint32_t sBar = sA + WG_ASTAGES*WG_ASTAGEB;
  const uint32_t bXFull = sBar;
  const uint32_t bXEmpty = sBar + 8*WG_XSTAGES;
  const uint32_t bAFull = sBar + 16*WG_XSTAGES;
  const uint32_t bAEmpty = bAFull + 8*WG_ASTAGES;
  const uint32_t bDone = bAEmpty + 8*WG_ASTAGES;
  uint32_t * tslot = (uint32_t *) (sgen + (bDone + 8 - sbase));
  volatile int * abort_flag = (volatile int *) (sgen + (bDone + 12 - sbase));

  const int warp = threadIdx.x/32;
  const int lane = threadIdx.x % 32;
  const lgbk_cnn_geom_t & g = p.g;

  if (threadIdx.x == 0) {
    for (int s = 0; s < WG_XSTAGES; s++) {
      tc_mbar_init(bXFull + 8*s, 1);
      tc_mbar_init(bXEmpty + 8*s, 1);
    }
    for (int s = 0; s < WG_ASTAGES; s++) {
      tc_mbar_init(bAFull + 8*s, 1);
      tc_mbar_init(bAEmpty + 8*s, 1);
    }
    tc_mbar_init(bDone, 1);
    *abort_flag = 0;
    tc_fence_barrier_init();
  }
  if (warp == 1) tc_tmem_alloc(tc_smem_u32(tslot), WG_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    tc_prefetch_map(&tm_g);
    tc_prefetch_map(&tm_x);
    int xs = 0, as = 0;
    uint32_t xph = 0, aph = 0;
    uint32_t xfills[WG_XSTAGES], afills[WG_ASTAGES];
    for (int k = 0; k < WG_XSTAGES; k++) xfills[k] = 0;
    for (int k = 0; k < WG_ASTAGES; k++) afills[k] = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile < g.ntiles; tile += gridDim.x) {
      int x, y0, z0;
      tile_decode(g, tile, x, y0, z0);
      if (!tc_mbar_wait(bXEmpty + 8*xs, xph ^ 1u, abort_flag, p.err)) break;
      tc_mbar_arrive_tx(bXFull + 8*xs, TILEB);
      for (int l = 0; l < g.lpt; l++) {
	tc_tma_load_2d(sX + xs*TILEB + l*g.bz*ROWB, &tm_x, bXFull + 8*xs, 0,
		       prow(g, x, y0 + l, z0));
      }
      xfills[xs] += 1;
      if (++xs == WG_XSTAGES) { xs = 0; xph ^= 1u; }
      for (int grp = 0; grp < WG_GROUPS; grp++) {
	if (!tc_mbar_wait(bAEmpty + 8*as, aph ^ 1u, abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	tc_mbar_arrive_tx(bAFull + 8*as, WG_ASTAGEB);
	for (int j = 0; j < 4; j++) {
	  int t = 4*grp + j;
	  if (t > CNN_NTAP - 1) t = CNN_NTAP - 1;   /* padding block, unused */
	  int dx, dy, dz;
	  tap_offsets(t, dx, dy, dz);
	  for (int l = 0; l < g.lpt; l++) {
	    tc_tma_load_2d(sA + as*WG_ASTAGEB + j*TILEB + l*g.bz*ROWB, &tm_g,
			   bAFull + 8*as, 0, prow(g, x - dx, y0 + l - dy,
						  z0 - dz));
	  }
	}
	afills[as] += 1;
	if (++as == WG_ASTAGES) { as = 0; aph ^= 1u; }
      }
    }
    for (int s = 0; s < WG_XSTAGES; s++) {
      if (xfills[s]) tc_drain_wait(bXFull + 8*s, (xfills[s] - 1u) & 1u, p.err);
    }
    for (int s = 0; s < WG_ASTAGES; s++) {
      if (afills[s]) tc_drain_wait(bAFull + 8*s, (afills[s] - 1u) & 1u, p.err);
    }
  }
  else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = tc_idesc_bf16(128, CNN_C, 1, 1);
    int xs = 0, as = 0;
    uint32_t xph = 0, aph = 0;
    int i = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile < g.ntiles; tile += gridDim.x) {
      if (!tc_mbar_wait(bXFull + 8*xs, xph, abort_flag, p.err)) break;
      tc_fence_after();
      for (int grp = 0; grp < WG_GROUPS; grp++) {
	if (!tc_mbar_wait(bAFull + 8*as, aph, abort_flag, p.err)) {
	  ok = false;
	  break;
	}
	tc_fence_after();
	#pragma unroll
	for (int k = 0; k < LGBK_CNN_TILE/16; k++) {
	  const uint64_t ad = tc_sdesc(sA + as*WG_ASTAGEB + k*1024, TILEB, 512,
				       LGB_TC_SWIZZLE_64B);
	  const uint64_t bd = tc_sdesc(sX + xs*TILEB + k*1024, TILEB, 512,
				       LGB_TC_SWIZZLE_64B);
	  tc_mma_bf16(tmem + (uint32_t) (grp*CNN_C), ad, bd, idesc,
		      (uint32_t) ((i | k) != 0));
	}
	tc_commit(bAEmpty + 8*as);
	if (++as == WG_ASTAGES) { as = 0; aph ^= 1u; }
      }
      if (!ok) break;
      tc_commit(bXEmpty + 8*xs);
      if (++xs == WG_XSTAGES) { xs = 0; xph ^= 1u; }
      i++;
    }
    tc_commit(bDone);
    tc_drain_wait(bDone, 0, p.err);
  }
  else if (warp >= 2) {
    const int q = warp & 3;
    bool okw = tc_mbar_wait(bDone, 0, abort_flag, p.err);
    if (__all_sync(0xffffffffu, okw)) {
      tc_fence_after();
      for (int grp = 0; grp < WG_GROUPS; grp++) {
	uint32_t r[32];
	tc_tmem_ld32(tmem + (uint32_t) (grp*CNN_C) + ((uint32_t) (q*32) << 16),
		     r);
	const int t = 4*grp + q;
	if (t < CNN_NTAP) {
	  float4 * o = (float4 *) (p.part + (((long long) blockIdx.x*CNN_NTAP
					      + t)*CNN_C + lane)*CNN_C);
	  #pragma unroll
	  for (int k = 0; k < 8; k++) {
	    o[k] = make_float4(__uint_as_float(r[4*k]),
			       __uint_as_float(r[4*k + 1]),
			       __uint_as_float(r[4*k + 2]),
			       __uint_as_float(r[4*k + 3]));
	  }
	}
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tc_tmem_dealloc(tmem, WG_TMEM_COLS);
  }
}

/* dw[k] = sum over blocks of part[b][k], fixed order */
/* dw[k] = sum over the nblk per-CTA partials, in a fixed order: a block
 * of 32 x 8 threads takes 32 consecutive k; thread (k, j) adds the
 * partials b = j, j + 8, ... (eight chains of loads in flight per k), and
 * thread (k, 0) then adds the eight chain sums in order j = 0 .. 7.  FP32
 * sums (chains of about 20 values, then 8): in FP64 this kernel was bound
 * by the FP64 pipe, a small fraction of the FP32 one on this part. */
__global__ void k_wgrad_reduce(const float * __restrict__ part, int nblk,
			       float * __restrict__ dw) {
  __shared__ float red[8][32];
  const int k = blockIdx.x*32 + threadIdx.x;
  const int j = threadIdx.y;
  float s = 0.0f;
  if (k < LGBK_CNN_WL) {
    /* eight loads in flight, added in the order b = j, j + 8, ... */
    for (int b0 = j; b0 < nblk; b0 += 64) {
      float v[8];
      #pragma unroll
      for (int u = 0; u < 8; u++) {
	const int b = b0 + 8*u;
	v[u] = (b < nblk) ? part[(long long) b*LGBK_CNN_WL + k] : 0.0f;
      }
      #pragma unroll
      for (int u = 0; u < 8; u++) s += v[u];
    }
  }
  red[j][threadIdx.x] = s;
  __syncthreads();
  if (j == 0 && k < LGBK_CNN_WL) {
    float t = 0.0f;
    #pragma unroll
    for (int q = 0; q < 8; q++) t += red[q][threadIdx.x];
    dw[k] = t;
  }
}

/*****************************************************************************
 *  k_wgrad_line: the weight gradient for nz a multiple of 128, reusing
 *  gradient lines as k_conv3_line reuses activation lines.
 *
 *  dW[t][co][ci] = sum_s g(s - e_t)[co] x(s)[ci].  A CTA walks runs of
 *  tiles along y (128 sites in z at fixed x, y); per tile the x rows are
 *  one box (B: N = 32 input channels, K = sites), and the gradient is read
 *  from the 9 lines (x - dx, y - dy) of 130 rows held in a ring (three
 *  new lines per tile, 64-byte swizzled rows).  One MMA takes, as its
 *  M = 128 rows, the three dx lines of one (dy, dz) side by side (the dx
 *  banks of the ring are a constant stride apart: the leading byte offset
 *  of an MN-major operand) plus a fourth bank that holds no data (its
 *  accumulator rows are not read), with the z shift as a start offset of
 *  1 - dz rows in the swizzled lines.  9 (dy, dz) groups x 8 K steps per
 *  tile; the accumulators (9 x 32 TMEM columns) hold the CTA's sums over
 *  all its tiles and are written once at the end.
 *****************************************************************************/

#define WL_NY      5                    /* y-line slots per dx bank */
#define WL_XST     2                    /* x-row tile stages */
#define WL_BANK    (WL_NY*LN_SLOT)      /* bytes per dx bank */
#define WL_THREADS 192
#define WL_TMEM_COLS 512
#define WL_SMEM (1024 + 4*WL_BANK + WL_XST*LN_SLOT + 256)

template <int DUMMY>
__global__ void __launch_bounds__(WL_THREADS, 1)
k_wgrad_line(const __grid_constant__ CUtensorMap tm_gline,
	     const __grid_constant__ CUtensorMap tm_xline, const WgP p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc_smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t * sgen = smem_raw + (sbase - raw);

  const uint32_t sL = sbase;                    /* 4 dx banks (the 4th empty) */
  const uint32_t sX = sL + 4*WL_BANK;
  const uint32_t sBar = sX + WL_XST*LN_SLOT;
  const uint32_t bFull = sBar;                  /* WL_NY */
  const uint32_t bRel = sBar + 8*WL_NY;         /* WL_NY */
  const uint32_t bXFull = sBar + 16*WL_NY;      /* WL_XST */
  const uint32_t bXEmpty = bXFull + 8*WL_XST;   /* WL_XST */
  const uint32_t bDone = bXEmpty + 8*WL_XST;
  uint32_t * tslot = (uint32_t *) (sgen + (bDone + 8 - sbase));
  volatile int * abort_flag = (volatile int *) (sgen + (bDone + 12 - sbase));

  const int warp = threadIdx.x/32;
  const int lane = threadIdx.x % 32;
  const lgbk_cnn_geom_t & g = p.g;
  const int nitems = line_items(g);

  if (threadIdx.x == 0) {
    for (int k = 0; k < WL_NY; k++) {
      tc_mbar_init(bFull + 8*k, 1);
      tc_mbar_init(bRel + 8*k, 1);
    }
    for (int k = 0; k < WL_XST; k++) {
      tc_mbar_init(bXFull + 8*k, 1);
      tc_mbar_init(bXEmpty + 8*k, 1);
    }
    tc_mbar_init(bDone, 1);
    *abort_flag = 0;
    tc_fence_barrier_init();
  }
  if (warp == 1) tc_tmem_alloc(tc_smem_u32(tslot), WL_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    tc_prefetch_map(&tm_gline);
    tc_prefetch_map(&tm_xline);
    uint32_t sq = 0, nx = 0;           /* gradient lines and x tiles loaded */
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; ok && y < yb; y++) {
	/* the x line of the tile: rows z0 - 1 .. z0 + 128 */
	const uint32_t xs = nx % WL_XST;
	if (nx >= WL_XST &&
	    !tc_mbar_wait(bXEmpty + 8*xs, (nx/WL_XST - 1u) & 1u, abort_flag,
			  p.err)) {
	  ok = false;
	  break;
	}
	tc_mbar_arrive_tx(bXFull + 8*xs, LN_ROWS*ROWB);
	tc_tma_load_2d(sX + xs*LN_SLOT, &tm_xline, bXFull + 8*xs, 0,
		       prow(g, x, y, z0 - 1));
	nx++;
	/* gradient lines y - 1 .. y + 1 (a new run) or y + 1 */
	const bool first = (y == ya);
	for (int li = 0; li < (first ? 3 : 1); li++, sq++) {
	  const int yy = first ? (y - 1 + li) : (y + 1);
	  const uint32_t r = sq % WL_NY;
	  if (sq >= WL_NY &&
	      !tc_mbar_wait(bRel + 8*r, (sq/WL_NY - 1u) & 1u, abort_flag,
			    p.err)) {
	    ok = false;
	    break;
	  }
	  tc_mbar_arrive_tx(bFull + 8*r, 3*LN_ROWS*ROWB);
	  for (int dxi = 0; dxi < 3; dxi++) {
	    tc_tma_load_2d(sL + (uint32_t) dxi*WL_BANK + r*LN_SLOT, &tm_gline,
			   bFull + 8*r, 0, prow(g, x + dxi - 1, yy, z0 - 1));
	  }
	}
      }
    }
    for (uint32_t k = 0; k < WL_XST && k < nx; k++) {
      const uint32_t nf = (nx - k + WL_XST - 1)/WL_XST;
      tc_drain_wait(bXFull + 8*k, (nf - 1u) & 1u, p.err);
    }
    for (uint32_t k = 0; k < WL_NY && k < sq; k++) {
      const uint32_t nf = (sq - k + WL_NY - 1)/WL_NY;
      tc_drain_wait(bFull + 8*k, (nf - 1u) & 1u, p.err);
    }
  }
  else if (warp == 1 && lane == 0) {
    /* N = 96: the x line's rows from z0 - 1 + dzi for dzi = 0, 1, 2, as
     * three 32-channel atoms of the MN-major operand one row (64 bytes,
     * the leading byte offset) apart */
    constexpr uint32_t idesc = tc_idesc_bf16(128, 3*CNN_C, 1, 1);
    const uint64_t ad0 = tc_sdesc(sL, WL_BANK, 512, LGB_TC_SWIZZLE_64B);
    const uint64_t bd0 = tc_sdesc(sX, ROWB, 512, LGB_TC_SWIZZLE_64B);
    const uint32_t alo0 = (uint32_t) ad0, ahi = (uint32_t) (ad0 >> 32);
    const uint32_t blo0 = (uint32_t) bd0, bhi = (uint32_t) (bd0 >> 32);
    uint32_t sq = 0, nx = 0;
    bool ok = true;
    for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
      int x, z0, ya, yb;
      line_item(g, it, x, z0, ya, yb);
      for (int y = ya; y < yb; y++) {
	const bool first = (y == ya), last = (y == yb - 1);
	const uint32_t xs = nx % WL_XST;
	ok = tc_mbar_wait(bXFull + 8*xs, (nx/WL_XST) & 1u, abort_flag, p.err);
	for (int li = 0; ok && li < (first ? 3 : 1); li++, sq++) {
	  ok = tc_mbar_wait(bFull + 8*(sq % WL_NY), (sq/WL_NY) & 1u,
			    abort_flag, p.err);
	}
	if (!ok) break;
	tc_fence_after();
	/* ring slots of the lines y - 1, y, y + 1 (dy = 1, 0, -1) */
	const uint32_t rr[3] = {(sq - 3u) % WL_NY, (sq - 2u) % WL_NY,
				(sq - 1u) % WL_NY};
	const uint32_t bx = blo0 + xs*(LN_SLOT >> 4);
	#pragma unroll
	for (int j = 0; j < 3; j++) {
	  /* gradient rows z0 .. z0 + 127 (line row 1 on) */
	  const uint32_t a = alo0 + rr[j]*(LN_SLOT >> 4) + (ROWB >> 4);
	  const uint32_t d = tmem + (uint32_t) (j*3*CNN_C);
	  #pragma unroll
	  for (int k = 0; k < LGBK_CNN_TILE/16; k++) {
	    tc_mma_bf16_w(d, a + k*(1024 >> 4), ahi, bx + k*(1024 >> 4), bhi,
			  idesc, (uint32_t) ((nx | k) != 0));
	  }
	}
	tc_commit(bXEmpty + 8*xs);
	nx++;
	tc_commit(bRel + 8*rr[0]);
	if (last) {
	  tc_commit(bRel + 8*rr[1]);
	  tc_commit(bRel + 8*rr[2]);
	}
      }
    }
    tc_commit(bDone);
    tc_drain_wait(bDone, 0, p.err);
  }
  else if (warp >= 2) {
    /* warp w reads TMEM lanes 32 q .. (q = w % 4): bank q = dx 1 - q */
    const int q = warp & 3;
    bool okw = tc_mbar_wait(bDone, 0, abort_flag, p.err);
    if (__all_sync(0xffffffffu, okw) && q < 3) {
      tc_fence_after();
      for (int j = 0; j < 3; j++) {
	for (int dzi = 0; dzi < 3; dzi++) {
	  uint32_t r[32];
	  tc_tmem_ld32(tmem + (uint32_t) ((3*j + dzi)*CNN_C)
		       + ((uint32_t) (q*32) << 16), r);
	  /* columns 96 j + 32 dzi: gradient rows z, x rows z - 1 + dzi */
	  /* dx = 1 - q, dy = 1 - j, dz = dzi - 1 */
	  const int t = (2 - q)*9 + (2 - j)*3 + dzi;
	  float4 * o = (float4 *) (p.part + (((long long) blockIdx.x*CNN_NTAP
					      + t)*CNN_C + lane)*CNN_C);
	  #pragma unroll
	  for (int k = 0; k < 8; k++) {
	    o[k] = make_float4(__uint_as_float(r[4*k]),
			       __uint_as_float(r[4*k + 1]),
			       __uint_as_float(r[4*k + 2]),
			       __uint_as_float(r[4*k + 3]));
	  }
	}
      }
    }
    else if (q == 3) {
      /* the fourth bank's rows hold no tap; the TMEM loads above are
       * warp-collective per quarter, so this warp has nothing to do */
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tc_tmem_dealloc(tmem, WL_TMEM_COLS);
  }
}

extern "C" int lgbk_cnn_wgrad(const lgbk_cnn_geom_t * g, const void * tm_g,
			      const void * tm_gline, const void * tm_x,
			      const void * tm_xline, float * part, float * dw,
			      int * err, void * stream) {
  WgP p;
  p.g = *g;
  p.part = part;
  p.err = err;
  const CUtensorMap mx = *(const CUtensorMap *) tm_x;
  cudaStream_t s = (cudaStream_t) stream;
  int grid = lgbk_cnn_wgrad_blocks(g);
  cudaError_t e;
  if (tm_gline && tm_xline && g->bz == LGBK_CNN_TILE && g->lpt == 1) {
    const CUtensorMap ml = *(const CUtensorMap *) tm_gline;
    const CUtensorMap mxl = *(const CUtensorMap *) tm_xline;
    const int items = line_items(*g);
    if (grid > items) grid = items;
    e = cudaFuncSetAttribute(k_wgrad_line<0>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, WL_SMEM);
    if (e != cudaSuccess) return (int) e;
    k_wgrad_line<0><<<grid, WL_THREADS, WL_SMEM, s>>>(ml, mxl, p);
  }
  else {
    const CUtensorMap mg = *(const CUtensorMap *) tm_g;
    e = cudaFuncSetAttribute(k_wgrad_tc,
      cudaFuncAttributeMaxDynamicSharedMemorySize, WG_SMEM);
    if (e != cudaSuccess) return (int) e;
    k_wgrad_tc<<<grid, WG_THREADS, WG_SMEM, s>>>(mg, mx, p);
  }
  k_wgrad_reduce<<<(LGBK_CNN_WL + 31)/32, dim3(32, 8), 0, s>>>(part, grid,
								 dw);
  return (int) cudaGetLastError();
}

/*****************************************************************************
 *  Self-test of the bounded waits: one thread waits on an mbarrier that
 *  nothing arrives on.  The wait gives up after LGB_TC_WAIT_CYCLES, raises
 *  the error word and returns, so the context stays usable (the failure
 *  path every tensor-core kernel takes when a copy or an MMA never
 *  completes).
 *****************************************************************************/

__global__ void k_wait_selftest(int * err) {
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int abort_word;
  if (threadIdx.x == 0) {
    tc_mbar_init(tc_smem_u32(&bar), 1);
    abort_word = 0;
    tc_fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    (void) tc_mbar_wait(tc_smem_u32(&bar), 0u, (volatile int *) &abort_word,
			err);
  }
}

extern "C" int lgbk_wait_selftest(int * err, void * stream) {
  k_wait_selftest<<<1, 32, 0, (cudaStream_t) stream>>>(err);
  return (int) cudaGetLastError();
}

/*****************************************************************************
 *  Elementwise kernels
 *****************************************************************************/

/* Periodic images of the padded rows: only the halo rows are visited, as
 * three disjoint sets (the two x faces whole; the two y faces for interior
 * x; the two z faces for interior x and y), 4 threads (16 bytes each) per
 * row; each image is copied from its interior source row. */
__global__ void k_cnn_halo(lgbk_cnn_geom_t g, uint4 * __restrict__ p) {
  /* 32-bit arithmetic: the padded rows number below 2^31, their halo
   * rows far fewer */
  const unsigned i = blockIdx.x*blockDim.x + threadIdx.x;
  const unsigned Z = (unsigned) g.nz + 2u, Y = (unsigned) g.ny + 2u;
  const unsigned nx = (unsigned) g.nx, ny = (unsigned) g.ny;
  const unsigned nxf = 2u*Y*Z, nyf = 2u*nx*Z, nzf = 2u*nx*ny;
  const unsigned h = i >> 2;
  const int q = (int) (i & 3u);
  int xp, yp, zp;
  if (h < nxf) {
    const unsigned r = h / Z;
    zp = (int) (h - r*Z);
    const unsigned f = r / Y;
    yp = (int) (r - f*Y);
    xp = f ? g.nx + 1 : 0;
  }
  else if (h < nxf + nyf) {
    const unsigned k = h - nxf;
    const unsigned r = k / Z;
    zp = (int) (k - r*Z);
    const unsigned f = r / nx;
    xp = 1 + (int) (r - f*nx);
    yp = f ? g.ny + 1 : 0;
  }
  else if (h < nxf + nyf + nzf) {
    const unsigned k = h - nxf - nyf;
    const unsigned r = k / ny;
    yp = 1 + (int) (k - r*ny);
    const unsigned f = r / nx;
    xp = 1 + (int) (r - f*nx);
    zp = f ? g.nz + 1 : 0;
  }
  else {
    return;
  }
  /* the interior source of each image: one period in from the face */
  const int x = (xp == 0) ? g.nx - 1 : ((xp == g.nx + 1) ? 0 : xp - 1);
  const int y = (yp == 0) ? g.ny - 1 : ((yp == g.ny + 1) ? 0 : yp - 1);
  const int z = (zp == 0) ? g.nz - 1 : ((zp == g.nz + 1) ? 0 : zp - 1);
  const long long row = ((long long) xp*Y + yp)*Z + zp;
  const long long src = ((long long) (x + 1)*Y + (y + 1))*Z + (z + 1);
  p[row*4 + q] = p[src*4 + q];
}

extern "C" int lgbk_cnn_halo(const lgbk_cnn_geom_t * g, void * p,
			     void * stream) {
  const long long Z = g->nz + 2, Y = g->ny + 2;
  const long long n = 4*(2*Y*Z + 2LL*g->nx*Z + 2LL*g->nx*g->ny);
  if (n >= 0xffffffffLL) return (int) cudaErrorInvalidValue;
  k_cnn_halo<<<(unsigned int) ((n + 255)/256), 256, 0,
    (cudaStream_t) stream>>>(*g, (uint4 *) p);
  return (int) cudaGetLastError();
}

struct FeatP {
  float off[5];
  float scale[5];
};

/* full = 0: channels 0..15 only (channels 16..31 of the rows are zero
 * already, and only the first layer, which reads 16, uses them) */
__global__ void k_cnn_features(lgbk_cnn_geom_t g, const float * __restrict__ phi,
			       const float * __restrict__ u,
			       const float * __restrict__ rho, FeatP fp,
			       uint8_t * __restrict__ p0, int full) {
  /* 32-bit site index and decoding (the padded rows, and so the sites,
   * number below 2^31) */
  const unsigned s = blockIdx.x*blockDim.x + threadIdx.x;
  if (s >= (unsigned) g.nsites) return;
  const unsigned r = s / (unsigned) g.nz;
  const int z = (int) (s - r*(unsigned) g.nz);
  const int x = (int) (r / (unsigned) g.ny);
  const int y = (int) (r - (unsigned) x*(unsigned) g.ny);
  const size_t N = (size_t) g.nsites;
  float v[32];
  #pragma unroll
  for (int c = 0; c < 32; c++) v[c] = 0.0f;
  v[0] = __fmul_rn(__fsub_rn(phi[s], fp.off[0]), fp.scale[0]);
  v[1] = __fmul_rn(__fsub_rn(u[s], fp.off[1]), fp.scale[1]);
  v[2] = __fmul_rn(__fsub_rn(u[N + s], fp.off[2]), fp.scale[2]);
  v[3] = __fmul_rn(__fsub_rn(u[2*N + s], fp.off[3]), fp.scale[3]);
  v[4] = __fmul_rn(__fsub_rn(rho[s], fp.off[4]), fp.scale[4]);
  /* the row and its periodic images (no halo pass) */
  uint4 w[4];
  pack_half_row_bf16(v, w);
  if (full) {
    pack_half_row_bf16(v + 16, w + 2);
    store_row_images<4>(g, p0, x, y, z, 0, w);
  }
  else {
    store_row_images<2>(g, p0, x, y, z, 0, w);
  }
}

extern "C" int lgbk_cnn_features(const lgbk_cnn_geom_t * g, const float * phi,
				 const float * u, const float * rho,
				 const float off[5], const float scale[5],
				 void * p0, int full, void * stream) {
  FeatP fp;
  for (int c = 0; c < 5; c++) { fp.off[c] = off[c]; fp.scale[c] = scale[c]; }
  cudaStream_t s = (cudaStream_t) stream;
  k_cnn_features<<<(unsigned int) ((g->nsites + 255)/256), 256, 0, s>>>(
    *g, phi, u, rho, fp, (uint8_t *) p0, full);
  return (int) cudaGetLastError();
}

/* fp32 rows [s][32] -> padded bf16 rows (interior), then halo */
__global__ void k_cnn_pack(lgbk_cnn_geom_t g, const float * __restrict__ src,
			   uint8_t * __restrict__ p) {
  /* 32-bit site index and decoding (the padded rows, and so the sites,
   * number below 2^31) */
  const unsigned s = blockIdx.x*blockDim.x + threadIdx.x;
  if (s >= (unsigned) g.nsites) return;
  const unsigned r = s / (unsigned) g.nz;
  const int z = (int) (s - r*(unsigned) g.nz);
  const int x = (int) (r / (unsigned) g.ny);
  const int y = (int) (r - (unsigned) x*(unsigned) g.ny);
  float v[32];
  #pragma unroll
  for (int c = 0; c < 32; c++) v[c] = src[(size_t) s*32 + c];
  store_row_bf16(p + (long long) prow(g, x, y, z)*ROWB, v);
}

extern "C" int lgbk_cnn_pack_rows(const lgbk_cnn_geom_t * g, const float * src,
				  void * p, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  k_cnn_pack<<<(unsigned int) ((g->nsites + 255)/256), 256, 0, s>>>(
    *g, src, (uint8_t *) p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int) e;
  return lgbk_cnn_halo(g, p, stream);
}

/* dL/dz_4 = 2 (out - t)/N on channels 0..3 (bf16 rows), block partial
 * sums of (out - t)^2 */
__global__ void k_cnn_loss_grad(lgbk_cnn_geom_t g, const float * __restrict__ out4,
				const float * __restrict__ t4,
				uint8_t * __restrict__ pg,
				double * __restrict__ part) {
  __shared__ double red[256];
  const long long N = g.nsites;
  const float rn2 = (float) (2.0/(double) N);
  /* per-thread sums of a few sites' squares in FP32 (the FP64 pipe is a
   * small fraction of the FP32 one here), block sums in FP64 */
  float acc = 0.0f;
  for (long long s = (long long) blockIdx.x*blockDim.x + threadIdx.x; s < N;
       s += (long long) gridDim.x*blockDim.x) {
    const unsigned su = (unsigned) s;             /* sites < 2^31 */
    const unsigned r = su / (unsigned) g.nz;
    const int z = (int) (su - r*(unsigned) g.nz);
    const int x = (int) (r / (unsigned) g.ny);
    const int y = (int) (r - (unsigned) x*(unsigned) g.ny);
    /* channels 0..3; 4..7 zero in the same 16 bytes; 8..31 of these
     * rows are zero from the buffer's creation and nothing else writes
     * this buffer */
    float v[4];
    #pragma unroll
    for (int c = 0; c < LGBK_CNN_NOUT; c++) {
      const float d = out4[c*N + s] - t4[c*N + s];
      acc = fmaf(d, d, acc);
      v[c] = rn2*d;
    }
    const __nv_bfloat162 h0 = __floats2bfloat162_rn(v[0], v[1]);
    const __nv_bfloat162 h1 = __floats2bfloat162_rn(v[2], v[3]);
    const uint4 w = make_uint4(*(const uint32_t *) &h0,
			       *(const uint32_t *) &h1, 0u, 0u);
    store_row_images<1>(g, pg, x, y, z, 0, &w);   /* no halo pass */
  }
  red[threadIdx.x] = (double) acc;
  __syncthreads();
  for (int w = blockDim.x/2; w > 0; w /= 2) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

/* 256 threads: thread j adds part[j], part[j + 256], ...; a fixed
 * pairwise tree then adds the 256 sums */
__global__ void k_cnn_loss_final(const double * __restrict__ part, int n,
				 double rn, double * __restrict__ loss) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w /= 2) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0]*rn;
}

extern "C" int lgbk_cnn_loss_grad(const lgbk_cnn_geom_t * g, const float * out4,
				  const float * t4, void * pg, double * part,
				  double * loss, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  k_cnn_loss_grad<<<LGBK_CNN_RED_BLOCKS, 256, 0, s>>>(*g, out4, t4,
						       (uint8_t *) pg, part);
  k_cnn_loss_final<<<1, 256, 0, s>>>(part, LGBK_CNN_RED_BLOCKS,
				    1.0/(double) g->nsites, loss);
  return (int) cudaGetLastError();
}

/* Bias gradient: per-block channel sums of the interior rows.  Block b
 * takes the z-lines b, b + G, ... (G blocks); a line's interior rows are
 * contiguous, 4 x 16 bytes a row, and thread t reads the 16-byte pieces
 * t, t + 256, ... of it, always channel group t % 4 (8 channels); two
 * lines' loads are issued before either is summed. */
__global__ void k_cnn_bias_part(lgbk_cnn_geom_t g, const uint8_t * __restrict__ pg,
				float * __restrict__ part) {
  __shared__ float red[256][9];
  const int cg = threadIdx.x & 3;
  float acc[8];
  #pragma unroll
  for (int k = 0; k < 8; k++) acc[k] = 0.0f;
  const int nlines = g.nx*g.ny;
  const int npiece = 4*g.nz;                    /* 16-byte pieces a line */
  auto add = [&](const uint4 & u) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      const float2 f = __bfloat1622float2(*(const __nv_bfloat162 *) &w[k]);
      acc[2*k] += f.x;
      acc[2*k + 1] += f.y;
    }
  };
  for (int l0 = blockIdx.x; l0 < nlines; l0 += 2*gridDim.x) {
    const int l1 = l0 + gridDim.x;
    const uint4 * a0 = (const uint4 *) (pg + (long long) prow(g, l0/g.ny,
							       l0 % g.ny, 0)*ROWB);
    const uint4 * a1 = (l1 < nlines)
      ? (const uint4 *) (pg + (long long) prow(g, l1/g.ny, l1 % g.ny, 0)*ROWB)
      : a0;
    for (int j = threadIdx.x; j < npiece; j += 2*256) {
      const bool two = (j + 256 < npiece);
      uint4 u00 = a0[j], u10 = a1[j];
      uint4 u01 = two ? a0[j + 256] : make_uint4(0u, 0u, 0u, 0u);
      uint4 u11 = two ? a1[j + 256] : make_uint4(0u, 0u, 0u, 0u);
      add(u00);
      add(u01);
      if (l1 < nlines) {
	add(u10);
	add(u11);
      }
    }
  }
  #pragma unroll
  for (int k = 0; k < 8; k++) red[threadIdx.x][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < 32) {
    const int c = threadIdx.x;             /* channel: group c/8, entry c%8 */
    float sum = 0.0f;
    for (int t = c/8; t < 256; t += 4) sum += red[t][c % 8];
    part[blockIdx.x*32 + c] = sum;
  }
}

/* 32 x 32 threads: thread (c, j) sums the partials b = j, j + 32, ... of
 * channel c, then thread (c, 0) adds the 32 sums in order j = 0 .. 31
 * (FP32 throughout: a single block of FP64 additions bounded this step) */
__global__ void k_cnn_bias_final(const float * __restrict__ part, int nblk,
				 float * __restrict__ db) {
  __shared__ float red[32][33];
  const int c = threadIdx.x, j = threadIdx.y;
  float s = 0.0f;
  /* eight loads in flight, added in the order b = j, j + 32, ... */
  for (int b0 = j; b0 < nblk; b0 += 256) {
    float v[8];
    #pragma unroll
    for (int u = 0; u < 8; u++) {
      const int b = b0 + 32*u;
      v[u] = (b < nblk) ? part[b*32 + c] : 0.0f;
    }
    #pragma unroll
    for (int u = 0; u < 8; u++) s += v[u];
  }
  red[j][c] = s;
  __syncthreads();
  if (j == 0) {
    float t = 0.0f;
    for (int k = 0; k < 32; k++) t += red[k][c];
    db[c] = t;
  }
}

extern "C" int lgbk_cnn_bias_grad(const lgbk_cnn_geom_t * g, const void * pg,
				  double * part, float * db, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  /* float partials in the first half of the scratch */
  float * pf = (float *) part;
  k_cnn_bias_part<<<LGBK_CNN_RED_BLOCKS, 256, 0, s>>>(*g, (const uint8_t *) pg,
						       pf);
  k_cnn_bias_final<<<1, dim3(32, 32), 0, s>>>(pf, LGBK_CNN_RED_BLOCKS, db);
  return (int) cudaGetLastError();
}

__global__ void k_cnn_adam(float * __restrict__ w, float * __restrict__ m,
			   float * __restrict__ v, const float * __restrict__ gr,
			   long long n, float lr, float b1, float b2, float eps,
			   float bc1, float bc2) {
  const long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = gr[i];
  const float mi = b1*m[i] + (1.0f - b1)*gi;
  const float vi = b2*v[i] + (1.0f - b2)*gi*gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi/bc1;
  const float vh = vi/bc2;
  w[i] -= lr*mh/(sqrtf(vh) + eps);
}

extern "C" int lgbk_cnn_adam(float * w, float * m, float * v,
			     const float * grad, long long n, float lr,
			     float beta1, float beta2, float eps, int step,
			     void * stream) {
  const float bc1 = (float) (1.0 - pow((double) beta1, (double) step));
  const float bc2 = (float) (1.0 - pow((double) beta2, (double) step));
  k_cnn_adam<<<(unsigned int) ((n + 255)/256), 256, 0, (cudaStream_t) stream>>>(
    w, m, v, grad, n, lr, beta1, beta2, eps, bc1, bc2);
  return (int) cudaGetLastError();
}

__global__ void k_cnn_wprep(const float * __restrict__ w,
			    __nv_bfloat16 * __restrict__ wf,
			    __nv_bfloat16 * __restrict__ wt) {
  const int k = blockIdx.x*blockDim.x + threadIdx.x;
  if (k >= LGBK_CNN_WL) return;
  const int c = k % 32;
  const int n = (k/32) % 32;
  const int t = k/1024;
  const __nv_bfloat16 h = __float2bfloat16_rn(w[k]);
  wf[k] = h;
  if (wt) wt[((CNN_NTAP - 1 - t)*32 + c)*32 + n] = h;
}

extern "C" int lgbk_cnn_wprep(const float * w, void * wf, void * wt,
			      void * stream) {
  k_cnn_wprep<<<(LGBK_CNN_WL + 255)/256, 256, 0, (cudaStream_t) stream>>>(
    w, (__nv_bfloat16 *) wf, (__nv_bfloat16 *) wt);
  return (int) cudaGetLastError();
}

/* The last layer's weights for the folded form: block b = 3 dxi + dzi
 * (32-row stride, 16 rows loaded), row 4 dyi + c = tap (dxi, dyi, dzi),
 * output c; rows 12..15 zero */
__global__ void k_cnn_wfold(const __nv_bfloat16 * __restrict__ wf,
			    __nv_bfloat16 * __restrict__ wfold) {
  const int k = blockIdx.x*blockDim.x + threadIdx.x;
  if (k >= 9*32*32) return;
  const int ci = k % 32;
  const int row = (k/32) % 32;
  const int b = k/1024;
  const int dxi = b/3, dzi = b % 3;
  __nv_bfloat16 h = __float2bfloat16_rn(0.0f);
  if (row < 3*LGBK_CNN_NOUT) {
    const int dyi = row/LGBK_CNN_NOUT, c = row % LGBK_CNN_NOUT;
    const int t = 9*dxi + 3*dyi + dzi;
    h = wf[(t*32 + c)*32 + ci];
  }
  wfold[k] = h;
}

extern "C" int lgbk_cnn_wfold(const void * wf, void * wfold, void * stream) {
  k_cnn_wfold<<<(9*32*32 + 255)/256, 256, 0, (cudaStream_t) stream>>>(
    (const __nv_bfloat16 *) wf, (__nv_bfloat16 *) wfold);
  return (int) cudaGetLastError();
}

/* Correction of the coarse state: phi, u and the momentum of f */
struct ApplyP {
  float os[4];
};

__global__ void k_cnn_apply(lgbk_cnn_geom_t g, const float * __restrict__ out4,
			    ApplyP ap, float * __restrict__ phi,
			    float * __restrict__ u, float * __restrict__ f,
			    const float * __restrict__ rho) {
  const long long s = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  const long long N = g.nsites;
  if (s >= N) return;
  phi[s] += ap.os[0]*out4[s];
  const float du[3] = {ap.os[1]*out4[N + s], ap.os[2]*out4[2*N + s],
		       ap.os[3]*out4[3*N + s]};
  u[s] += du[0];
  u[N + s] += du[1];
  u[2*N + s] += du[2];
  if (f) {
    const float r3 = 3.0f*rho[s];
    const int8_t cv[19][3] = {{0, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 0, 0},
			      {1, 0, -1}, {1, -1, 0}, {0, 1, 1}, {0, 1, 0},
			      {0, 1, -1}, {0, 0, 1}, {0, 0, -1}, {0, -1, 1},
			      {0, -1, 0}, {0, -1, -1}, {-1, 1, 0}, {-1, 0, 1},
			      {-1, 0, 0}, {-1, 0, -1}, {-1, -1, 0}};
    const int w36[19] = {12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 2,
			 1, 1};
    #pragma unroll
    for (int q = 1; q < 19; q++) {
      const float cu = cv[q][0]*du[0] + cv[q][1]*du[1] + cv[q][2]*du[2];
      f[q*N + s] += (w36[q]*(1.0f/36.0f))*r3*cu;
    }
  }
}

extern "C" int lgbk_cnn_apply(const lgbk_cnn_geom_t * g, const float * out4,
			      const float os[4], float * phi, float * u,
			      float * f, const float * rho, void * stream) {
  ApplyP ap;
  for (int c = 0; c < 4; c++) ap.os[c] = os[c];
  k_cnn_apply<<<(unsigned int) ((g->nsites + 255)/256), 256, 0,
    (cudaStream_t) stream>>>(*g, out4, ap, phi, u, f, rho);
  return (int) cudaGetLastError();
}
