/*****************************************************************************
 *
 *  ludwig_gb_cnn.c
 *
 *  Host side of the learned corrector: a 4-layer 3x3x3 convolutional
 *  network (32 channels, GELU) that corrects phi and u of a binary fluid
 *  run on a lattice coarsened by 2, after every coarse step.  Training and
 *  inference run on the GPU through the tensor-core kernels of lgb_cnn.cu;
 *  this file owns the parameters, the activation buffers, their TMA tensor
 *  maps and the order of the passes.  The reference has no counterpart.
 *
 *  Parameters (FP32 master copy, Adam moments beside it), per layer l:
 *  W_l [27 taps][32 out][32 in] then b_l [32].  Layer 1 reads 5 real input
 *  channels (phi, u, rho after an affine normalisation), layer 4 writes 4
 *  real outputs (the normalised corrections of phi and u); the padding
 *  channels start at zero and receive zero gradients.
 *
 *****************************************************************************/

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime_api.h>

#include "ludwig_gb.h"
#include "lgb_cnn.h"
#include "lgb_coarse.h"
#include "lgb_internal.h"

#define NL   LGBK_CNN_NLAYER
#define PL   LGBK_CNN_PL
#define WL   LGBK_CNN_WL

struct ludwig_gb_cnn_s {
  CUtensorMap tm_act[NL];      /* padded activations a_0 .. a_3 */
  CUtensorMap tm_g[NL + 1];    /* padded dL/dz_1 .. dL/dz_4 (index 1..4) */
  CUtensorMap tm_wf[NL];       /* bf16 weights, forward order */
  CUtensorMap tm_wf16;         /* the last layer's, 16 rows a tap */
  CUtensorMap tm_wfold;        /* ... rearranged for the folded form */
  CUtensorMap tm_wt[NL];       /* bf16 weights, flipped and transposed */
  CUtensorMap tm_actl[NL];     /* the same buffers as 8 x 130 line boxes */
  CUtensorMap tm_gl[NL + 1];
  CUtensorMap tm_acts[NL];     /* ... and as swizzled 32 x 130 line boxes */
  CUtensorMap tm_gs[NL + 1];
  lgbk_cnn_geom_t g;
  int line_ok;                 /* nz a multiple of 128: line-reuse kernel */
  int line_on;
  int act0_dirty;              /* act[0] channels 16..31 may be nonzero */
  float * params;              /* [NL][PL] */
  float * grads;
  float * adam_m;
  float * adam_v;
  void * wf[NL];
  void * wt[NL];
  void * wfold;                /* bf16 [9][32][32] */
  void * act[NL];
  void * zpre[NL];             /* bf16 [N][32] GELU'(z), index 1..3 */
  void * gpad[NL + 1];         /* index 1..4 */
  float * out4;                /* [4][N] */
  float * part;                /* wgrad partial sums */
  double * red;                /* reduction scratch */
  double * loss_dev;
  int * err_dev;
  float in_off[5], in_scale[5], out_scale[4];
  int step;                    /* Adam steps taken */
  int wprep_valid;
};

static PFN_cuTensorMapEncodeTiled_v12000 encode_ = NULL;

static int ck(int cuda_rc, const char * where) {
  return cuda_rc ? lgb_internal_cuda(cuda_rc, where) : LUDWIG_GB_OK;
}

static cudaStream_t lib_stream(void) {
  return (cudaStream_t) ludwig_gb_stream();
}

static int get_encoder(void) {
  if (encode_) return LUDWIG_GB_OK;
  void * fn = NULL;
  enum cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled",
						   &fn, 12000,
						   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == NULL) {
    return lgb_internal_err(LUDWIG_GB_ECUDA,
			    "cuTensorMapEncodeTiled entry point not found");
  }
  encode_ = (PFN_cuTensorMapEncodeTiled_v12000) fn;
  return LUDWIG_GB_OK;
}

/* 2-d map over rows of 32 bf16 channels (64 bytes), box 32 x box_rows,
 * 64-byte swizzle (the layout the tcgen05 descriptors expect) */
static int map_rows(CUtensorMap * m, void * base, long long rows,
		    int box_rows) {
  cuuint64_t dims[2] = {32, (cuuint64_t) rows};
  cuuint64_t strides[1] = {64};
  cuuint32_t box[2] = {32, (cuuint32_t) box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims,
		       strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
		       CU_TENSOR_MAP_SWIZZLE_64B,
		       CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
		       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    return lgb_internal_err(LUDWIG_GB_ECUDA, "cuTensorMapEncodeTiled failed");
  }
  return LUDWIG_GB_OK;
}

/* The same rows as boxes of 8 channels x 130 rows without swizzle (one
 * plane of a line for the line-reuse convolution) */
static int map_lines(CUtensorMap * m, void * base, long long rows,
		     int swizzled) {
  cuuint64_t dims[2] = {32, (cuuint64_t) rows};
  cuuint64_t strides[1] = {64};
  cuuint32_t box[2] = {swizzled ? 32u : 8u, 130};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims,
		       strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
		       swizzled ? CU_TENSOR_MAP_SWIZZLE_64B
		                : CU_TENSOR_MAP_SWIZZLE_NONE,
		       CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
		       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    return lgb_internal_err(LUDWIG_GB_ECUDA, "cuTensorMapEncodeTiled failed");
  }
  return LUDWIG_GB_OK;
}

static int dalloc(void ** p, size_t bytes) {
  *p = NULL;
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    *p = NULL;
    return lgb_internal_err(LUDWIG_GB_ENOMEM, "cudaMalloc (corrector)");
  }
  return LUDWIG_GB_OK;
}

/* splitmix64 -> uniform in [-1, 1) */
static double urand(uint64_t * s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30))*0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27))*0x94D049BB133111EBull;
  z ^= (z >> 31);
  return 2.0*((double) (z >> 11)*(1.0/9007199254740992.0)) - 1.0;
}

int ludwig_gb_cnn_nparams(void) { return NL*PL; }

/* Deterministic initial parameters: uniform with variance 2/fan_in on the
 * real channels (last layer x 0.1), zero on padding and biases. */
static void init_params(uint64_t seed, float * h) {
  uint64_t s = seed ? seed : 1;
  memset(h, 0, sizeof(float)*NL*PL);
  for (int l = 0; l < NL; l++) {
    const int cin = (l == 0) ? LGBK_CNN_NIN : LGBK_CNN_C;
    const int cout = (l == NL - 1) ? LGBK_CNN_NOUT : LGBK_CNN_C;
    const double fan = 27.0*cin;
    double bound = sqrt(3.0)*sqrt(2.0/fan);
    if (l == NL - 1) bound *= 0.1;
    for (int t = 0; t < LGBK_CNN_NTAP; t++) {
      for (int n = 0; n < LGBK_CNN_C; n++) {
	for (int c = 0; c < LGBK_CNN_C; c++) {
	  double v = bound*urand(&s);
	  if (n < cout && c < cin) h[l*PL + (t*32 + n)*32 + c] = (float) v;
	}
      }
    }
  }
}

int ludwig_gb_cnn_free(ludwig_gb_cnn_t * m) {
  if (m == NULL) return LUDWIG_GB_OK;
  cudaFree(m->params); cudaFree(m->grads);
  cudaFree(m->adam_m); cudaFree(m->adam_v);
  for (int l = 0; l < NL; l++) {
    cudaFree(m->wf[l]); cudaFree(m->wt[l]);
    cudaFree(m->act[l]); cudaFree(m->zpre[l]);
  }
  for (int l = 0; l <= NL; l++) cudaFree(m->gpad[l]);
  cudaFree(m->wfold);
  cudaFree(m->out4); cudaFree(m->part); cudaFree(m->red);
  cudaFree(m->loss_dev); cudaFree(m->err_dev);
  free(m);
  return LUDWIG_GB_OK;
}

static int wprep(ludwig_gb_cnn_t * m) {
  cudaStream_t s = lib_stream();
  for (int l = 0; l < NL; l++) {
    int rc = lgbk_cnn_wprep(m->params + l*PL, m->wf[l], m->wt[l], s);
    if (rc) return ck(rc, "cnn wprep");
  }
  int rc = lgbk_cnn_wfold(m->wf[NL - 1], m->wfold, s);
  if (rc) return ck(rc, "cnn wfold");
  m->wprep_valid = 1;
  return LUDWIG_GB_OK;
}

int ludwig_gb_cnn_create(const int n[3], unsigned long long seed,
			 ludwig_gb_cnn_t ** pm) {
  if (n == NULL || pm == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_create: NULL");
  }
  lgbk_cnn_geom_t g;
  if (lgbk_cnn_geom(n[0], n[1], n[2], &g)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_create: extents "
			    "(nz in {32, 64} or a multiple of 128, ny a "
			    "multiple of 128/nz)");
  }
  if (ludwig_gb_stream() == NULL) {
    return lgb_internal_err(LUDWIG_GB_ECUDA, "cnn_create: no stream");
  }
  int rc = get_encoder();
  if (rc) return rc;

  ludwig_gb_cnn_t * m = NULL;
  if (posix_memalign((void **) &m, 128, sizeof(*m)) || m == NULL) {
    return lgb_internal_err(LUDWIG_GB_ENOMEM, "cnn_create");
  }
  memset(m, 0, sizeof(*m));
  m->g = g;
  const size_t N = (size_t) g.nsites;
  const size_t prow = (size_t) g.rows*64;
  const size_t nblk = (size_t) lgbk_cnn_wgrad_blocks(&g);

  rc = dalloc((void **) &m->params, sizeof(float)*NL*PL);
  if (!rc) rc = dalloc((void **) &m->grads, sizeof(float)*NL*PL);
  if (!rc) rc = dalloc((void **) &m->adam_m, sizeof(float)*NL*PL);
  if (!rc) rc = dalloc((void **) &m->adam_v, sizeof(float)*NL*PL);
  for (int l = 0; l < NL && !rc; l++) {
    rc = dalloc(&m->wf[l], 2*WL);
    if (!rc) rc = dalloc(&m->wt[l], 2*WL);
    if (!rc) rc = dalloc(&m->act[l], prow);
    if (!rc && l > 0) rc = dalloc(&m->zpre[l], N*64);
  }
  for (int l = 1; l <= NL && !rc; l++) rc = dalloc(&m->gpad[l], prow);
  if (!rc) rc = dalloc(&m->wfold, 2*9*32*32);
  if (!rc) rc = dalloc((void **) &m->out4, sizeof(float)*4*N);
  if (!rc) rc = dalloc((void **) &m->part, sizeof(float)*nblk*WL);
  if (!rc) rc = dalloc((void **) &m->red,
		       sizeof(double)*LGBK_CNN_RED_BLOCKS*32);
  if (!rc) rc = dalloc((void **) &m->loss_dev, sizeof(double));
  if (!rc) rc = dalloc((void **) &m->err_dev, sizeof(int));
  if (rc) { ludwig_gb_cnn_free(m); return rc; }

  for (int l = 0; l < NL && !rc; l++) {
    rc = map_rows(&m->tm_act[l], m->act[l], g.rows, g.bz);
    if (!rc) rc = map_rows(&m->tm_wf[l], m->wf[l], LGBK_CNN_NTAP*32, 32);
    if (!rc) rc = map_rows(&m->tm_wt[l], m->wt[l], LGBK_CNN_NTAP*32, 32);
  }
  if (!rc) rc = map_rows(&m->tm_wf16, m->wf[NL - 1], LGBK_CNN_NTAP*32, 16);
  if (!rc) rc = map_rows(&m->tm_wfold, m->wfold, 9*32, 16);
  for (int l = 1; l <= NL && !rc; l++) {
    rc = map_rows(&m->tm_g[l], m->gpad[l], g.rows, g.bz);
  }
  m->line_ok = (g.bz == LGBK_CNN_TILE && g.lpt == 1);
  /* default: three z taps per MMA where a line is the whole z extent,
   * the last layer's y taps folded into its MMAs too, on swizzled lines
   * (one TMA box a line instead of four of 16-byte rows): 0.547 ms per
   * forward pass at 128^3 against 0.562 on planes and 0.907 with one tap
   * per MMA; planes otherwise */
  m->line_on = m->line_ok ? ((g.nz == LGBK_CNN_TILE) ? 5 : 1) : 0;
  for (int l = 0; l < NL && !rc && m->line_ok; l++) {
    rc = map_lines(&m->tm_actl[l], m->act[l], g.rows, 0);
    if (!rc) rc = map_lines(&m->tm_acts[l], m->act[l], g.rows, 1);
  }
  for (int l = 1; l <= NL && !rc && m->line_ok; l++) {
    rc = map_lines(&m->tm_gl[l], m->gpad[l], g.rows, 0);
    if (!rc) rc = map_lines(&m->tm_gs[l], m->gpad[l], g.rows, 1);
  }
  if (rc) { ludwig_gb_cnn_free(m); return rc; }

  cudaStream_t s = lib_stream();
  /* Halo rows and padding channels are always written before they are
   * read; zero everything once so that no buffer holds stale bits. */
  for (int l = 0; l < NL && !rc; l++) {
    rc = ck(cudaMemsetAsync(m->act[l], 0, prow, s), "memset");
  }
  for (int l = 1; l <= NL && !rc; l++) {
    rc = ck(cudaMemsetAsync(m->gpad[l], 0, prow, s), "memset");
  }
  if (!rc) rc = ck(cudaMemsetAsync(m->adam_m, 0, sizeof(float)*NL*PL, s),
		   "memset");
  if (!rc) rc = ck(cudaMemsetAsync(m->adam_v, 0, sizeof(float)*NL*PL, s),
		   "memset");
  if (!rc) rc = ck(cudaMemsetAsync(m->err_dev, 0, sizeof(int), s), "memset");

  float * h = (float *) malloc(sizeof(float)*NL*PL);
  if (h == NULL) rc = lgb_internal_err(LUDWIG_GB_ENOMEM, "cnn_create");
  if (!rc) {
    init_params(seed, h);
    rc = ck(cudaMemcpyAsync(m->params, h, sizeof(float)*NL*PL,
			    cudaMemcpyHostToDevice, s), "params");
    if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  }
  free(h);
  for (int c = 0; c < 5; c++) { m->in_off[c] = 0.0f; m->in_scale[c] = 1.0f; }
  m->in_off[4] = 1.0f;
  for (int c = 0; c < 4; c++) m->out_scale[c] = 1.0f;
  if (!rc) rc = wprep(m);
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  if (rc) { ludwig_gb_cnn_free(m); return rc; }
  *pm = m;
  return LUDWIG_GB_OK;
}

int ludwig_gb_cnn_scales_set(ludwig_gb_cnn_t * m, const float in_off[5],
			     const float in_scale[5],
			     const float out_scale[4]) {
  if (m == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn");
  for (int c = 0; c < 5; c++) {
    if (in_off) m->in_off[c] = in_off[c];
    if (in_scale) m->in_scale[c] = in_scale[c];
  }
  for (int c = 0; c < 4; c++) if (out_scale) m->out_scale[c] = out_scale[c];
  return LUDWIG_GB_OK;
}

int ludwig_gb_cnn_scales_get(ludwig_gb_cnn_t * m, float in_off[5],
			     float in_scale[5], float out_scale[4]) {
  if (m == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn");
  for (int c = 0; c < 5; c++) { in_off[c] = m->in_off[c];
    in_scale[c] = m->in_scale[c]; }
  for (int c = 0; c < 4; c++) out_scale[c] = m->out_scale[c];
  return LUDWIG_GB_OK;
}

int ludwig_gb_cnn_params_get(ludwig_gb_cnn_t * m, float * h) {
  if (m == NULL || h == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn");
  cudaStream_t s = lib_stream();
  int rc = ck(cudaMemcpyAsync(h, m->params, sizeof(float)*NL*PL,
			      cudaMemcpyDeviceToHost, s), "params_get");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

/* Replaces the parameters and restarts Adam */
int ludwig_gb_cnn_params_set(ludwig_gb_cnn_t * m, const float * h) {
  if (m == NULL || h == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn");
  cudaStream_t s = lib_stream();
  int rc = ck(cudaMemcpyAsync(m->params, h, sizeof(float)*NL*PL,
			      cudaMemcpyHostToDevice, s), "params_set");
  if (!rc) rc = ck(cudaMemsetAsync(m->adam_m, 0, sizeof(float)*NL*PL, s), "m");
  if (!rc) rc = ck(cudaMemsetAsync(m->adam_v, 0, sizeof(float)*NL*PL, s), "v");
  m->step = 0;
  if (!rc) rc = wprep(m);
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

int ludwig_gb_cnn_grads_get(ludwig_gb_cnn_t * m, float * h) {
  if (m == NULL || h == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn");
  cudaStream_t s = lib_stream();
  int rc = ck(cudaMemcpyAsync(h, m->grads, sizeof(float)*NL*PL,
			      cudaMemcpyDeviceToHost, s), "grads_get");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

/* line map for activation layer l (act = 1) or gradient l (act = 0) in
 * the line form kind: swizzled rows for 2 and 5, planes otherwise */
static const void * lmapk(ludwig_gb_cnn_t * m, int act, int l, int kind) {
  if (!kind) return NULL;
  if (kind == 2 || kind == 5 || kind == 6) {
    return act ? &m->tm_acts[l] : &m->tm_gs[l];
  }
  return act ? &m->tm_actl[l] : &m->tm_gl[l];
}

/* 1: the line-reuse convolution where the extents allow it; 2: the same
 * with swizzled line boxes; 3: the same with the three z taps of a line
 * in one MMA where nz = 128; 4: as 3, and the last layer with the y taps
 * folded into the MMA as well; 5: as 4 on swizzled lines (3, 4 and 5 fall
 * back to 1 where nz != 128; the default is 5 where nz = 128, else 1);
 * 0: one box per tap */
int ludwig_gb_cnn_line_reuse(ludwig_gb_cnn_t * m, int mode) {
  if (m == NULL || mode < 0 || mode > 5) {
    return lgb_internal_err(LUDWIG_GB_EINVAL,
			    "cnn_line_reuse: 0 .. 5");
  }
  if (mode >= 3 && m->g.nz != LGBK_CNN_TILE) mode = 1;
  m->line_on = m->line_ok ? mode : 0;
  return LUDWIG_GB_OK;
}

/* the line form of the hidden layers and of every backward convolution */
static int lkind(const ludwig_gb_cnn_t * m) {
  return (m->line_on == 4) ? 3 : m->line_on;
}
/* mode 5: mode 4 on swizzled lines (one TMA box a line) */

static const void * lmap(ludwig_gb_cnn_t * m, int act, int l) {
  return lmapk(m, act, l, lkind(m));
}

/* the three-tap line forms write the periodic images of the padded rows
 * themselves (no halo pass after their convolutions) */
static int writes_images(const ludwig_gb_cnn_t * m) {
  const int k = lkind(m);
  return k == 3 || k == 5;
}

static int check_err(ludwig_gb_cnn_t * m) {
  cudaStream_t s = lib_stream();
  int herr = 0;
  int rc = ck(cudaMemcpyAsync(&herr, m->err_dev, sizeof(int),
			      cudaMemcpyDeviceToHost, s), "err");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  if (rc) return rc;
  if (herr) {
    cudaMemsetAsync(m->err_dev, 0, sizeof(int), s);
    cudaStreamSynchronize(s);
    return lgb_internal_err(LUDWIG_GB_ETIMEOUT, "corrector kernel: a "
			    "bounded wait ran out (tensor-core pipeline)");
  }
  return LUDWIG_GB_OK;
}

/* Input channels a layer's convolution reads: the first layer's input
 * rows hold the LGBK_CNN_NIN features and zeros */
static int kin_of(int l) {
  return (l == 0 && LGBK_CNN_NIN <= 16) ? 16 : LGBK_CNN_C;
}

/* a_0 from [phi, u, rho] pointers, then the four layers -> out (m->out4
 * when NULL); the slopes GELU'(z) of the hidden layers (for the backward
 * pass) are stored only when train */
static int forward(ludwig_gb_cnn_t * m, const float * phi, const float * u,
		   const float * rho, int train, float * out) {
  cudaStream_t s = lib_stream();
  const lgbk_cnn_geom_t * g = &m->g;
  /* the first layer reads channels 0..15; 16..31 stay zero unless a
   * direct convolution call packed other data into act[0] */
  int rc = lgbk_cnn_features(g, phi, u, rho, m->in_off, m->in_scale,
			     m->act[0], m->act0_dirty, s);
  m->act0_dirty = 0;
  if (rc) return ck(rc, "cnn features");
  for (int l = 0; l < NL; l++) {
    const float * b = m->params + l*PL + WL;
    if (l < NL - 1) {
      rc = lgbk_cnn_conv(g, LGBK_CNN_FWD_GELU, kin_of(l), LGBK_CNN_C,
			 &m->tm_act[l],
			 lmap(m, 1, l), lkind(m), &m->tm_wf[l], b, NULL,
			 train ? m->zpre[l + 1] : NULL, m->act[l + 1], NULL,
			 m->err_dev, s);
      if (!rc && !writes_images(m)) rc = lgbk_cnn_halo(g, m->act[l + 1], s);
    }
    else {
      /* the 4 outputs: 16 weight rows a tap where the three-tap form
       * runs; the folded blocks in the folded form */
      const int w16 = (m->line_on >= 3);
      const int fold = (m->line_on == 4 || m->line_on == 5);
      const int kl = fold ? ((m->line_on == 5) ? 6 : 4) : m->line_on;
      const CUtensorMap * tw = fold ? &m->tm_wfold
	: (w16 ? &m->tm_wf16 : &m->tm_wf[l]);
      rc = lgbk_cnn_conv(g, LGBK_CNN_FWD_OUT, kin_of(l),
			 w16 ? 16 : LGBK_CNN_C, &m->tm_act[l],
			 lmapk(m, 1, l, kl), kl, tw, b, NULL, NULL,
			 NULL, out ? out : m->out4, m->err_dev, s);
    }
    if (rc) return ck(rc, "cnn conv");
  }
  return LUDWIG_GB_OK;
}

/* Loss and gradients into m->grads (no update) */
static int backward(ludwig_gb_cnn_t * m, const float * t4) {
  cudaStream_t s = lib_stream();
  const lgbk_cnn_geom_t * g = &m->g;
  int rc = lgbk_cnn_loss_grad(g, m->out4, t4, m->gpad[NL], m->red,
			      m->loss_dev, s);
  if (rc) return ck(rc, "cnn loss");
  for (int l = NL - 1; l >= 0; l--) {
    /* dL/dz_{l+1} is in gpad[l+1]; the layer input is act[l] */
    rc = lgbk_cnn_wgrad(g, &m->tm_g[l + 1],
			m->line_on ? &m->tm_gs[l + 1] : NULL, &m->tm_act[l],
			m->line_on ? &m->tm_acts[l] : NULL,
			m->part, m->grads + l*PL, m->err_dev, s);
    if (!rc) rc = lgbk_cnn_bias_grad(g, m->gpad[l + 1], m->red,
				     m->grads + l*PL + WL, s);
    if (rc) return ck(rc, "cnn wgrad");
    if (l == 0) break;
    rc = lgbk_cnn_conv(g, LGBK_CNN_BWD_GELU, LGBK_CNN_C, LGBK_CNN_C,
		       &m->tm_g[l + 1],
		       lmap(m, 0, l + 1), lkind(m), &m->tm_wt[l], NULL, m->zpre[l],
		       NULL, m->gpad[l], NULL, m->err_dev, s);
    if (!rc && !writes_images(m)) rc = lgbk_cnn_halo(g, m->gpad[l], s);
    if (rc) return ck(rc, "cnn conv (backward)");
  }
  return LUDWIG_GB_OK;
}

static int read_loss(ludwig_gb_cnn_t * m, double * loss) {
  cudaStream_t s = lib_stream();
  double h = 0.0;
  int rc = ck(cudaMemcpyAsync(&h, m->loss_dev, sizeof(double),
			      cudaMemcpyDeviceToHost, s), "loss");
  if (!rc) rc = check_err(m);
  if (!rc && loss) *loss = h;
  return rc;
}

int ludwig_gb_cnn_forward(ludwig_gb_cnn_t * m, const float * in5,
			  float * out4) {
  if (m == NULL || in5 == NULL || out4 == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_forward");
  }
  const size_t N = (size_t) m->g.nsites;
  int rc = forward(m, in5, in5 + N, in5 + 4*N, 0, out4);
  if (!rc) rc = check_err(m);
  return rc;
}

int ludwig_gb_cnn_forward_n(ludwig_gb_cnn_t * m, int n,
			    const float * const * in5,
			    float * const * out4) {
  if (m == NULL || n < 0 || (n > 0 && (in5 == NULL || out4 == NULL))) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_forward_n");
  }
  const size_t N = (size_t) m->g.nsites;
  for (int k = 0; k < n; k++) {
    if (in5[k] == NULL || out4[k] == NULL) {
      return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_forward_n: pointer");
    }
    int rc = forward(m, in5[k], in5[k] + N, in5[k] + 4*N, 0, out4[k]);
    if (rc) return rc;
  }
  return check_err(m);
}

int ludwig_gb_cnn_loss_grad(ludwig_gb_cnn_t * m, const float * in5,
			    const float * t4, double * loss) {
  if (m == NULL || in5 == NULL || t4 == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_loss_grad");
  }
  const size_t N = (size_t) m->g.nsites;
  int rc = forward(m, in5, in5 + N, in5 + 4*N, 1, NULL);
  if (!rc) rc = backward(m, t4);
  if (!rc) rc = read_loss(m, loss);
  return rc;
}

static int adam(ludwig_gb_cnn_t * m, double lr) {
  cudaStream_t s = lib_stream();
  m->step += 1;
  int rc = lgbk_cnn_adam(m->params, m->adam_m, m->adam_v, m->grads,
			 (long long) NL*PL, (float) lr, 0.9f, 0.999f, 1e-8f,
			 m->step, s);
  if (rc) return ck(rc, "cnn adam");
  return wprep(m);
}

int ludwig_gb_cnn_train_step(ludwig_gb_cnn_t * m, const float * in5,
			     const float * t4, double lr, double * loss) {
  if (m == NULL || in5 == NULL || t4 == NULL || !(lr > 0.0)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_train_step");
  }
  const size_t N = (size_t) m->g.nsites;
  int rc = forward(m, in5, in5 + N, in5 + 4*N, 1, NULL);
  if (!rc) rc = backward(m, t4);
  if (!rc) rc = adam(m, lr);
  if (!rc) rc = read_loss(m, loss);
  return rc;
}

/* Several steps without reading the loss in between (losses: nsteps) */
int ludwig_gb_cnn_train_steps(ludwig_gb_cnn_t * m, int nsteps,
			      const float * const * in5,
			      const float * const * t4, double lr,
			      double * losses) {
  if (m == NULL || nsteps < 0 || in5 == NULL || t4 == NULL || !(lr > 0.0)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_train_steps");
  }
  const size_t N = (size_t) m->g.nsites;
  for (int k = 0; k < nsteps; k++) {
    int rc = forward(m, in5[k], in5[k] + N, in5[k] + 4*N, 1, NULL);
    if (!rc) rc = backward(m, t4[k]);
    if (!rc) rc = adam(m, lr);
    if (!rc && losses) rc = read_loss(m, losses + k);
    if (rc) return rc;
  }
  return check_err(m);
}

/* Corrects a coarse FP32 state in place: phi, u and the momentum of f */
int ludwig_gb_cnn_correct(ludwig_gb_cnn_t * m, lb_t * lb, field_t * phi,
			  hydro_t * hydro) {
  if (m == NULL) return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_correct");
  lgb_view_t v;
  int rc = lgb_internal_binary_view(lb, phi, hydro, -1, &v);
  if (rc) return rc;
  if (v.prec != LUDWIG_GB_FP32) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_correct: FP32 state");
  }
  if (v.d.nx != m->g.nx || v.d.ny != m->g.ny || v.d.nz != m->g.nz) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_correct: extents");
  }
  const size_t N = (size_t) m->g.nsites;
  rc = forward(m, (const float *) v.phi, (const float *) v.u,
	       (const float *) v.rho, 0, NULL);
  if (rc) return rc;
  rc = lgbk_cnn_apply(&m->g, m->out4, m->out_scale, (float *) v.phi,
		      (float *) v.u, (float *) v.f, (const float *) v.rho,
		      lib_stream());
  (void) N;
  if (rc) return ck(rc, "cnn apply");
  return check_err(m);
}

/*****************************************************************************
 *  Fine -> coarse restriction and field packing
 *****************************************************************************/

int ludwig_gb_coarse_restrict(lb_t * lbf, field_t * phif, hydro_t * hf,
			      lb_t * lbc, field_t * phic, hydro_t * hc) {
  lgb_view_t vf, vc;
  int rc = lgb_internal_binary_view(lbf, phif, hf, -1, &vf);
  if (!rc) rc = lgb_internal_binary_view(lbc, phic, hc, -1, &vc);
  if (rc) return rc;
  if (vf.prec != LUDWIG_GB_FP32 || vc.prec != LUDWIG_GB_FP32) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "coarse_restrict: FP32 states");
  }
  if (vf.rho0 != vc.rho0) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "coarse_restrict: rho0");
  }
  rc = lgbk_restrict_state(&vf.d, &vc.d, (const float *) vf.f, vf.pending,
			   (const float *) vf.phi, (const float *) vf.u,
			   vf.rho0, 2.0, 4.0, (float *) vc.f, (float *) vc.phi,
			   (float *) vc.u, (float *) vc.rho, vf.stream);
  if (rc) return ck(rc, "coarse_restrict (extents must be 2x)");
  rc = lgb_internal_lb_set_pending(lbc, 0);
  if (!rc) rc = ck(cudaStreamSynchronize((cudaStream_t) vf.stream), "sync");
  return rc;
}

int ludwig_gb_fields_restrict(field_t * phif, hydro_t * hf, lb_t * lbf,
			      float * out5, const int nc[3]) {
  lgb_view_t vf;
  int rc = lgb_internal_binary_view(lbf, phif, hf, -1, &vf);
  if (rc) return rc;
  if (vf.prec != LUDWIG_GB_FP32 || out5 == NULL || nc == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "fields_restrict");
  }
  lgbk_dims_t dc = {nc[0], nc[1], nc[2], (long long) nc[0]*nc[1]*nc[2]};
  rc = lgbk_restrict_fields(&vf.d, &dc, (const float *) vf.phi,
			    (const float *) vf.u, (const float *) vf.rho, 2.0,
			    out5, vf.stream);
  if (rc) return ck(rc, "fields_restrict (extents must be 2x)");
  return ck(cudaStreamSynchronize((cudaStream_t) vf.stream), "sync");
}

int ludwig_gb_fields_pack(field_t * phi, hydro_t * hydro, lb_t * lb,
			  float * out5) {
  lgb_view_t v;
  int rc = lgb_internal_binary_view(lb, phi, hydro, -1, &v);
  if (rc) return rc;
  if (v.prec != LUDWIG_GB_FP32 || out5 == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "fields_pack");
  }
  const size_t N = (size_t) v.d.nsites;
  cudaStream_t s = (cudaStream_t) v.stream;
  rc = ck(cudaMemcpyAsync(out5, v.phi, 4*N, cudaMemcpyDeviceToDevice, s),
	  "pack");
  if (!rc) rc = ck(cudaMemcpyAsync(out5 + N, v.u, 12*N,
				   cudaMemcpyDeviceToDevice, s), "pack");
  if (!rc) rc = ck(cudaMemcpyAsync(out5 + 4*N, v.rho, 4*N,
				   cudaMemcpyDeviceToDevice, s), "pack");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

/*****************************************************************************
 *  Single-kernel entry points (for kernel-level checks)
 *****************************************************************************/

/* out[s][n] = b[n] + sum_t sum_c a[s + e_t][c] w[t][n][c]   (flip = 0)
 * out[s][c] = sum_t sum_n a[s - e_t][n] w[t][n][c]          (flip = 1)
 * a, w, b, out: device fp32; a and w are rounded to bf16 first. */
int ludwig_gb_cnn_conv3(ludwig_gb_cnn_t * m, const float * a, const float * w,
			const float * b, int flip, float * out) {
  if (m == NULL || a == NULL || w == NULL || out == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_conv3");
  }
  cudaStream_t s = lib_stream();
  int rc = lgbk_cnn_pack_rows(&m->g, a, m->act[0], s);
  m->act0_dirty = 1;
  if (!rc) rc = lgbk_cnn_wprep(w, m->wf[0], m->wt[0], s);
  if (!rc) rc = lgbk_cnn_conv(&m->g, LGBK_CNN_RAW, LGBK_CNN_C, LGBK_CNN_C,
			      &m->tm_act[0],
			      lmap(m, 1, 0), lkind(m),
			      flip ? &m->tm_wt[0] : &m->tm_wf[0],
			      flip ? NULL : b, NULL, NULL, NULL, out,
			      m->err_dev, s);
  m->wprep_valid = 0;
  if (rc) return ck(rc, "cnn_conv3");
  rc = check_err(m);
  if (!rc) rc = wprep(m);            /* restore layer 0 weights */
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

/* dw[t][n][c] = sum_s gr[s - e_t][n] a[s][c]; device fp32 in, bf16-rounded */
int ludwig_gb_cnn_wgrad3(ludwig_gb_cnn_t * m, const float * gr,
			 const float * a, float * dw) {
  if (m == NULL || gr == NULL || a == NULL || dw == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "cnn_wgrad3");
  }
  cudaStream_t s = lib_stream();
  int rc = lgbk_cnn_pack_rows(&m->g, a, m->act[0], s);
  m->act0_dirty = 1;
  if (!rc) rc = lgbk_cnn_pack_rows(&m->g, gr, m->gpad[1], s);
  if (!rc) rc = lgbk_cnn_wgrad(&m->g, &m->tm_g[1],
			       m->line_on ? &m->tm_gs[1] : NULL, &m->tm_act[0],
			       m->line_on ? &m->tm_acts[0] : NULL,
			       m->part, dw, m->err_dev, s);
  if (rc) return ck(rc, "cnn_wgrad3");
  rc = check_err(m);
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  return rc;
}

/* Runs one device wait that nothing satisfies and reports how the bounded
 * wait ended: LUDWIG_GB_ETIMEOUT (the expected outcome) once the kernel
 * has given up, raised its error word and returned; *seconds: the time
 * the kernel took. */
int ludwig_gb_selftest_bounded_wait(double * seconds) {
  if (seconds == NULL) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "selftest_bounded_wait");
  }
  cudaStream_t s = lib_stream();
  int * err = NULL;
  if (cudaMalloc((void **) &err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return lgb_internal_err(LUDWIG_GB_ENOMEM, "selftest_bounded_wait");
  }
  cudaEvent_t e0, e1;
  int herr = 0;
  int rc = ck(cudaEventCreate(&e0), "event");
  if (!rc) rc = ck(cudaEventCreate(&e1), "event");
  if (!rc) rc = ck(cudaMemsetAsync(err, 0, sizeof(int), s), "memset");
  if (!rc) rc = ck(cudaEventRecord(e0, s), "record");
  if (!rc) rc = ck(lgbk_wait_selftest(err, s), "selftest kernel");
  if (!rc) rc = ck(cudaEventRecord(e1, s), "record");
  if (!rc) rc = ck(cudaMemcpyAsync(&herr, err, sizeof(int),
				   cudaMemcpyDeviceToHost, s), "err");
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  if (!rc) {
    float ms = 0.0f;
    rc = ck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
    *seconds = 1e-3*ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(err);
  if (rc) return rc;
  if (herr) {
    return lgb_internal_err(LUDWIG_GB_ETIMEOUT, "selftest: the bounded "
			    "wait ran out as intended");
  }
  return LUDWIG_GB_OK;
}
