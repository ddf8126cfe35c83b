/*****************************************************************************
 *
 *  lgb_cnn.h
 *
 *  Launchers of the learned corrector's kernels (lgb_cnn.cu): the 3x3x3
 *  convolution as an implicit GEMM on the tensor cores (tcgen05, BF16
 *  operands, FP32 accumulation in tensor memory), its weight gradient,
 *  and the elementwise pieces around them.
 *
 *  Activations live in "padded rows": one 64-byte row of 32 bf16 channels
 *  per site of the (nx+2) x (ny+2) x (nz+2) box that carries a one-site
 *  periodic halo, row index ((x+1)(ny+2) + (y+1))(nz+2) + (z+1).  A tile of
 *  128 output sites is lpt lines of bz consecutive z sites, so every tap of
 *  the stencil reads lpt runs of contiguous rows: one TMA box each.
 *
 *****************************************************************************/

#ifndef LGB_CNN_H
#define LGB_CNN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGBK_CNN_C      32          /* channels of every layer (padded) */
#define LGBK_CNN_NTAP   27
#define LGBK_CNN_NIN    5           /* phi, u_x, u_y, u_z, rho */
#define LGBK_CNN_NOUT   4           /* d phi, d u_x, d u_y, d u_z */
#define LGBK_CNN_NLAYER 4
#define LGBK_CNN_WL     (LGBK_CNN_NTAP*LGBK_CNN_C*LGBK_CNN_C)
#define LGBK_CNN_PL     (LGBK_CNN_WL + LGBK_CNN_C)   /* params per layer */
#define LGBK_CNN_TILE   128
#define LGBK_CNN_RED_BLOCKS 1024

typedef struct lgbk_cnn_geom_s {
  int nx, ny, nz;
  int bz;                     /* z sites per line of a tile */
  int lpt;                    /* lines per tile (128 = lpt*bz) */
  int ntiles;
  long long nsites;
  long long rows;             /* padded rows */
} lgbk_cnn_geom_t;

enum lgbk_cnn_mode {
  LGBK_CNN_FWD_GELU = 0,      /* z = acc + b: GELU(z) -> pout, GELU'(z) ->
				 zout (bf16; when zout is not NULL) */
  LGBK_CNN_FWD_OUT  = 1,      /* acc + b, channels 0..3 -> outf[c][s] fp32 */
  LGBK_CNN_BWD_GELU = 2,      /* acc * zprev (the stored GELU'(z)) -> pout */
  LGBK_CNN_RAW      = 3       /* acc + b (b may be NULL) -> outf[s][32] fp32 */
};

/* 0, or nonzero if the extents cannot be tiled (nz in {32, 64} or a
 * multiple of 128; ny a multiple of 128/nz when nz < 128) */
int lgbk_cnn_geom(int nx, int ny, int nz, lgbk_cnn_geom_t * g);

int lgbk_cnn_conv_blocks(const lgbk_cnn_geom_t * g);
int lgbk_cnn_wgrad_blocks(const lgbk_cnn_geom_t * g);

/* tm_in, tm_line, tm_w: host pointers to CUtensorMap objects (passed by
 * value).  tm_in: rows, box 32 x bz, 64-byte swizzle; tm_w: weights, box
 * 32 x 32, 64-byte swizzle; tm_line (may be NULL; nz a multiple of 128):
 * line_kind 1: rows, box 8 x 130, no swizzle; line_kind 2: rows, box
 * 32 x 130, 64-byte swizzle (line-reuse kernel); line_kind 3 (nz = 128):
 * the kind-1 map, three z taps per MMA; line_kind 5: the same on the
 * kind-2 map; line_kind 4 / 6 (nz = 128, mode LGBK_CNN_FWD_OUT, tm_w the
 * folded weights of lgbk_cnn_wfold): the kind-1 / kind-2 map, the y taps
 * folded into the MMAs as well.  With line_kind 3 or 5 the modes
 * LGBK_CNN_FWD_GELU and LGBK_CNN_BWD_GELU also write the periodic images
 * of the rows they write (no lgbk_cnn_halo pass after them). */
/* kin: input channels read, 32 or 16 (the first layer: channels 16..31 of
 * its input rows are zero, so their products are left out); wrows: weight
 * rows (output channels) per tap in tm_w's boxes, 32, or 16 for the last
 * layer's 4 outputs where a three-tap line form runs (line_kind 3 .. 6,
 * nz = 128) */
int lgbk_cnn_conv(const lgbk_cnn_geom_t * g, int mode, int kin, int wrows,
		  const void * tm_in,
		  const void * tm_line, int line_kind, const void * tm_w,
		  const float * bias,
		  const void * zprev, void * zout, void * pout, float * outf,
		  int * err, void * stream);

/* dW[t][n][c] = sum_s g[s - e_t][n] x[s][c]; part: wgrad_blocks*27*1024
 * floats of scratch; dw: 27*1024 floats.  tm_gline, tm_xline (may be
 * NULL): the gradient's and the input's line maps (box 32 x 130, 64-byte
 * swizzle); both given and nz a multiple of 128, the line-reuse kernel
 * runs. */
int lgbk_cnn_wgrad(const lgbk_cnn_geom_t * g, const void * tm_g,
		   const void * tm_gline, const void * tm_x,
		   const void * tm_xline, float * part, float * dw, int * err,
		   void * stream);

int lgbk_cnn_halo(const lgbk_cnn_geom_t * g, void * p, void * stream);

/* channel c < 5: (src[c][s] - off[c]) * scale[c]; others 0 (full = 0:
 * channels 5..15 only, 16..31 left as they are); the periodic images in
 * the halo written with the rows */
int lgbk_cnn_features(const lgbk_cnn_geom_t * g, const float * phi,
		      const float * u, const float * rho, const float off[5],
		      const float scale[5], void * p0, int full,
		      void * stream);

/* Loss (1/N) sum (out - t)^2 over 4 channels and dL/dz_4 (bf16, padded,
 * the periodic images written with the rows; channels 8..31 of pg must be
 * zero and stay so); part: LGBK_CNN_RED_BLOCKS doubles; loss: 1 double */
int lgbk_cnn_loss_grad(const lgbk_cnn_geom_t * g, const float * out4,
		       const float * t4, void * pg, double * part,
		       double * loss, void * stream);

/* db[n] = sum_s g[s][n]; part: LGBK_CNN_RED_BLOCKS*32 doubles */
int lgbk_cnn_bias_grad(const lgbk_cnn_geom_t * g, const void * pg,
		       double * part, float * db, void * stream);

/* Adam on n parameters (step >= 1) */
int lgbk_cnn_adam(float * w, float * m, float * v, const float * grad,
		  long long n, float lr, float beta1, float beta2, float eps,
		  int step, void * stream);

/* Master weights [27][32][32] fp32 -> bf16 forward copy (same order) and
 * the flipped, transposed copy wt[26 - t][c][n] = w[t][n][c] */
int lgbk_cnn_wprep(const float * w, void * wf, void * wt, void * stream);
/* The last layer's bf16 weights (wf, [27][32][32]) rearranged for the
 * folded line form (line_kind 4): wfold [9][32][32], block 3 dxi + dzi,
 * row 4 dyi + c */
int lgbk_cnn_wfold(const void * wf, void * wfold, void * stream);

/* phi += os0 out0; du = os out1..3; u += du; f_p += 3 w_p rho c_p.du
 * (FP32 deviation storage of f) */
int lgbk_cnn_apply(const lgbk_cnn_geom_t * g, const float * out4,
		   const float os[4], float * phi, float * u, float * f,
		   const float * rho, void * stream);

/* fp32 [s][32] <-> padded bf16 rows (tests of single kernels) */
int lgbk_cnn_pack_rows(const lgbk_cnn_geom_t * g, const float * src,
		       void * p, void * stream);

/* One bounded wait that runs out (nothing arrives): raises *err */
int lgbk_wait_selftest(int * err, void * stream);

#ifdef __cplusplus
}
#endif

#endif
