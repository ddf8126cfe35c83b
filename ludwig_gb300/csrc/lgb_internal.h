/*****************************************************************************
 *
 *  lgb_internal.h
 *
 *  Private interface between the two host translation units of
 *  libludwig_gb.so: ludwig_gb.c (the reference-facing objects) gives
 *  ludwig_gb_cnn.c (the learned corrector) device views of a binary-fluid
 *  state, and ludwig_gb_io.c (snapshot files) the objects' sizes and I/O
 *  state.  Not installed, not part of the C ABI.
 *
 *****************************************************************************/

#ifndef LGB_INTERNAL_H
#define LGB_INTERNAL_H

#include "ludwig_gb.h"
#include "lgb_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgb_view_s {
  lgbk_dims_t d;
  int prec;                   /* LUDWIG_GB_FP64 / FP32 / FP16 */
  int pending;                /* f holds post-collision values */
  void * f;                   /* stored distributions [19][nsites] */
  void * phi;                 /* [nsites] */
  void * u;                   /* [3][nsites] */
  void * rho;                 /* [nsites] */
  double rho0;                /* shift of the reduced-precision storage */
  void * stream;
} lgb_view_t;

/* layout: 1 = post-collision (pending streaming), 0 = the reference's f,
 * -1 = as stored */
int lgb_internal_binary_view(lb_t * lb, field_t * phi, hydro_t * hydro,
			     int layout, lgb_view_t * v);

/* Declare that the stored f now holds the reference's f (pending = 0) */
int lgb_internal_lb_set_pending(lb_t * lb, int pending);

/* Snapshot I/O state of an lb_t or a field_t: record formats of input and
 * output (IO_RECORD_ASCII / IO_RECORD_BINARY) and whether the metadata
 * file has been written */
typedef struct lgb_io_state_s {
  int fmt_in;
  int fmt_out;
  int meta_written;
} lgb_io_state_t;

int lgb_internal_lb_io(lb_t * lb, int ntotal[3], int * ndist,
		       lgb_io_state_t ** io);
int lgb_internal_field_io(field_t * f, int ntotal[3], int * nf,
			  const char ** name, lgb_io_state_t ** io);
int lgb_internal_hydro_io(hydro_t * h, int ntotal[3], lgb_io_state_t ** rho,
			  lgb_io_state_t ** vel);

int lgb_internal_err(int code, const char * what);     /* LUDWIG_GB_* code */
int lgb_internal_cuda(int cuda_rc, const char * where); /* cudaError_t -> ECUDA */

#ifdef __cplusplus
}
#endif

#endif
