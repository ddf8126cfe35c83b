/*****************************************************************************
 *
 *  cnn_oracle.c
 *
 *  Test infrastructure only: a plain-C, double-precision restatement of
 *  the learned corrector's network (forward, loss and backward), against
 *  which the tensor-core kernels are checked.  The reference has no such
 *  network, so nothing here pins to the reference: the restatement is
 *  checked by central finite differences of its own loss instead.
 *
 *  Network (the corrector of a 2x-coarsened binary fluid):
 *    a0 = features (5 real channels, zero-padded to 32)
 *    z_l = b_l + sum_t sum_c a_{l-1}(s + e_t)[c] W_l[t][n][c]   (3^3 taps)
 *    a_l = GELU(z_l) (tanh form), l = 1, 2, 3;   output = z_4 channels 0..3
 *  Periodic neighbours; tap t = (dx+1)*9 + (dy+1)*3 + (dz+1).
 *  Loss = (1/N) sum_s sum_{c<4} (z_4[c](s) - target[c](s))^2.
 *
 *  With emulate = 1 every quantity the device stores in bf16 is rounded
 *  to bf16 (round to nearest even) at the same point: weights, features,
 *  activations a_l, the slopes GELU'(z_l) that the forward pass keeps for
 *  the backward pass (evaluated at the unrounded z_l), and the gradients
 *  dL/dz_l.  The output z_4 and the loss stay unrounded (the device keeps
 *  them in fp32).
 *
 *****************************************************************************/

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_CNN_C      32
#define ORC_CNN_NTAP   27
#define ORC_CNN_NIN    5
#define ORC_CNN_NOUT   4
#define ORC_CNN_NLAYER 4
#define ORC_CNN_WL     (ORC_CNN_NTAP*ORC_CNN_C*ORC_CNN_C)

/* float -> bf16 -> float, round to nearest even (finite inputs) */
static double bf16r(double v) {
  float f = (float) v;
  uint32_t u;
  memcpy(&u, &f, 4);
  uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  u &= 0xffff0000u;
  memcpy(&f, &u, 4);
  return (double) f;
}

static double rnd(int emulate, double v) { return emulate ? bf16r(v) : v; }

/* GELU, tanh form (Hendrycks and Gimpel 2016):
 * 0.5 z (1 + tanh(u)) = z sigma(2u), u = sqrt(2/pi) (z + 0.044715 z^3) */
static double gelu_v(double z) {
  const double k0 = 2.0*sqrt(2.0/3.14159265358979323846);
  return k0*z*(1.0 + 0.044715*z*z);
}

static double gelu(double z) { return z/(1.0 + exp(-gelu_v(z))); }

static double gelu_d(double z) {
  const double k0 = 2.0*sqrt(2.0/3.14159265358979323846);
  const double s = 1.0/(1.0 + exp(-gelu_v(z)));
  return s + z*s*(1.0 - s)*k0*(1.0 + 3.0*0.044715*z*z);
}

static long long nbr(const int n[3], long long s, int t, int sign) {
  int z = (int) (s % n[2]);
  long long r = s / n[2];
  int y = (int) (r % n[1]);
  int x = (int) (r / n[1]);
  int dx = t/9 - 1, dy = (t/3) % 3 - 1, dz = t % 3 - 1;
  x = (x + sign*dx + n[0]) % n[0];
  y = (y + sign*dy + n[1]) % n[1];
  z = (z + sign*dz + n[2]) % n[2];
  return ((long long) x*n[1] + y)*n[2] + z;
}

/* z[s][n] = b[n] + sum_t sum_c a[s + e_t][c] w[t][n][c] */
static void conv_fwd(const int n[3], const double * a, const double * w,
		     const double * b, double * z) {
  const long long N = (long long) n[0]*n[1]*n[2];
  #pragma omp parallel for schedule(static)
  for (long long s = 0; s < N; s++) {
    double acc[ORC_CNN_C];
    for (int o = 0; o < ORC_CNN_C; o++) acc[o] = 0.0;
    for (int t = 0; t < ORC_CNN_NTAP; t++) {
      const double * an = a + nbr(n, s, t, +1)*ORC_CNN_C;
      const double * wt = w + (long long) t*ORC_CNN_C*ORC_CNN_C;
      for (int o = 0; o < ORC_CNN_C; o++) {
	double v = 0.0;
	for (int c = 0; c < ORC_CNN_C; c++) v += an[c]*wt[o*ORC_CNN_C + c];
	acc[o] += v;
      }
    }
    for (int o = 0; o < ORC_CNN_C; o++) z[s*ORC_CNN_C + o] = b[o] + acc[o];
  }
}

/* da[s][c] = sum_t sum_o g[s - e_t][o] w[t][o][c] */
static void conv_bwd_data(const int n[3], const double * g, const double * w,
			  double * da) {
  const long long N = (long long) n[0]*n[1]*n[2];
  #pragma omp parallel for schedule(static)
  for (long long s = 0; s < N; s++) {
    double acc[ORC_CNN_C];
    for (int c = 0; c < ORC_CNN_C; c++) acc[c] = 0.0;
    for (int t = 0; t < ORC_CNN_NTAP; t++) {
      const double * gn = g + nbr(n, s, t, -1)*ORC_CNN_C;
      const double * wt = w + (long long) t*ORC_CNN_C*ORC_CNN_C;
      for (int o = 0; o < ORC_CNN_C; o++) {
	for (int c = 0; c < ORC_CNN_C; c++) acc[c] += gn[o]*wt[o*ORC_CNN_C + c];
      }
    }
    for (int c = 0; c < ORC_CNN_C; c++) da[s*ORC_CNN_C + c] = acc[c];
  }
}

/* dw[t][o][c] = sum_s g[s - e_t][o] a[s][c];  db[o] = sum_s g[s][o] */
static void conv_wgrad(const int n[3], const double * g, const double * a,
		       double * dw, double * db) {
  const long long N = (long long) n[0]*n[1]*n[2];
  #pragma omp parallel for schedule(static)
  for (int t = 0; t < ORC_CNN_NTAP; t++) {
    double * dwt = dw + (long long) t*ORC_CNN_C*ORC_CNN_C;
    for (int k = 0; k < ORC_CNN_C*ORC_CNN_C; k++) dwt[k] = 0.0;
    for (long long s = 0; s < N; s++) {
      const double * gn = g + nbr(n, s, t, -1)*ORC_CNN_C;
      const double * as = a + s*ORC_CNN_C;
      for (int o = 0; o < ORC_CNN_C; o++) {
	if (gn[o] == 0.0) continue;
	for (int c = 0; c < ORC_CNN_C; c++) dwt[o*ORC_CNN_C + c] += gn[o]*as[c];
      }
    }
  }
  for (int o = 0; o < ORC_CNN_C; o++) db[o] = 0.0;
  for (long long s = 0; s < N; s++) {
    for (int o = 0; o < ORC_CNN_C; o++) db[o] += g[s*ORC_CNN_C + o];
  }
}

/* Features: channel c < 5 = in[c][s] * scale[c]; the rest zero. */
static void features(const int n[3], int emulate, const float * in5,
		     const float * scale, double * a0) {
  const long long N = (long long) n[0]*n[1]*n[2];
  for (long long s = 0; s < N; s++) {
    for (int c = 0; c < ORC_CNN_C; c++) {
      double v = 0.0;
      if (c < ORC_CNN_NIN) v = (double) ((float) in5[c*N + s]*scale[c]);
      a0[s*ORC_CNN_C + c] = rnd(emulate, v);
    }
  }
}

/* Runs the network; optionally keeps the activations and the slopes
 * GELU'(z) of the hidden layers.
 * W: [4][27][32][32] float; b: [4][32] float; out4: [4][N] double. */
static int cnn_forward_keep(const int n[3], int emulate, const float * in5,
			    const float * scale, const float * W,
			    const float * b, double * out4, double ** act,
			    double ** pre) {
  const long long N = (long long) n[0]*n[1]*n[2];
  const long long NC = N*ORC_CNN_C;
  double * w = (double *) malloc(sizeof(double)*ORC_CNN_WL);
  double * bb = (double *) malloc(sizeof(double)*ORC_CNN_C);
  double * z = (double *) malloc(sizeof(double)*NC);
  if (!w || !bb || !z) { free(w); free(bb); free(z); return -1; }

  features(n, emulate, in5, scale, act[0]);
  for (int l = 0; l < ORC_CNN_NLAYER; l++) {
    for (long long k = 0; k < ORC_CNN_WL; k++) {
      w[k] = rnd(emulate, (double) W[l*ORC_CNN_WL + k]);
    }
    for (int o = 0; o < ORC_CNN_C; o++) bb[o] = (double) b[l*ORC_CNN_C + o];
    conv_fwd(n, act[l], w, bb, z);
    if (emulate) {
      for (long long k = 0; k < NC; k++) z[k] = (double) (float) z[k];
    }
    if (l < ORC_CNN_NLAYER - 1) {
      for (long long k = 0; k < NC; k++) {
	pre[l + 1][k] = rnd(emulate, gelu_d(z[k]));
	act[l + 1][k] = rnd(emulate, gelu(z[k]));
      }
    }
    else {
      for (long long s = 0; s < N; s++) {
	for (int c = 0; c < ORC_CNN_NOUT; c++) {
	  out4[c*N + s] = z[s*ORC_CNN_C + c];
	}
      }
    }
  }
  free(w); free(bb); free(z);
  return 0;
}

static int alloc_set(double ** v, int count, long long n) {
  for (int i = 0; i < count; i++) v[i] = NULL;
  for (int i = 0; i < count; i++) {
    v[i] = (double *) calloc((size_t) n, sizeof(double));
    if (v[i] == NULL) return -1;
  }
  return 0;
}

static void free_set(double ** v, int count) {
  for (int i = 0; i < count; i++) free(v[i]);
}

int orc_cnn_forward(const int n[3], int emulate, const float * in5,
		    const float * scale, const float * W, const float * b,
		    double * out4) {
  const long long NC = (long long) n[0]*n[1]*n[2]*ORC_CNN_C;
  double * act[ORC_CNN_NLAYER], * pre[ORC_CNN_NLAYER];
  int rc = alloc_set(act, ORC_CNN_NLAYER, NC);
  if (rc == 0) rc = alloc_set(pre, ORC_CNN_NLAYER, NC);
  if (rc == 0) rc = cnn_forward_keep(n, emulate, in5, scale, W, b, out4, act,
				     pre);
  free_set(act, ORC_CNN_NLAYER);
  free_set(pre, ORC_CNN_NLAYER);
  return rc;
}

/* Loss and its gradients dW [4][27][32][32], db [4][32] (double). */
int orc_cnn_loss_grad(const int n[3], int emulate, const float * in5,
		      const float * scale, const float * target4,
		      const float * W, const float * b, double * loss,
		      double * dW, double * db) {
  const long long N = (long long) n[0]*n[1]*n[2];
  const long long NC = N*ORC_CNN_C;
  double * act[ORC_CNN_NLAYER], * pre[ORC_CNN_NLAYER];
  double * g = NULL, * ga = NULL, * out4 = NULL, * w = NULL;
  int rc = alloc_set(act, ORC_CNN_NLAYER, NC);
  if (rc == 0) rc = alloc_set(pre, ORC_CNN_NLAYER, NC);
  g = (double *) calloc((size_t) NC, sizeof(double));
  ga = (double *) calloc((size_t) NC, sizeof(double));
  out4 = (double *) calloc((size_t) (ORC_CNN_NOUT*N), sizeof(double));
  w = (double *) malloc(sizeof(double)*ORC_CNN_WL);
  if (rc || !g || !ga || !out4 || !w) { rc = -1; goto done; }

  rc = cnn_forward_keep(n, emulate, in5, scale, W, b, out4, act, pre);
  if (rc) goto done;

  /* loss and dL/dz_4 */
  double sum = 0.0;
  for (long long s = 0; s < N; s++) {
    for (int c = 0; c < ORC_CNN_C; c++) {
      double gv = 0.0;
      if (c < ORC_CNN_NOUT) {
	double d = out4[c*N + s] - (double) target4[c*N + s];
	sum += d*d;
	gv = 2.0*d/(double) N;
      }
      g[s*ORC_CNN_C + c] = rnd(emulate, gv);
    }
  }
  *loss = sum/(double) N;

  for (int l = ORC_CNN_NLAYER - 1; l >= 0; l--) {
    conv_wgrad(n, g, act[l], dW + (long long) l*ORC_CNN_WL,
	       db + l*ORC_CNN_C);
    if (l == 0) break;
    for (long long k = 0; k < ORC_CNN_WL; k++) {
      w[k] = rnd(emulate, (double) W[l*ORC_CNN_WL + k]);
    }
    conv_bwd_data(n, g, w, ga);
    for (long long k = 0; k < NC; k++) {
      double v = ga[k];
      if (emulate) v = (double) (float) v;
      g[k] = rnd(emulate, v*pre[l][k]);
    }
  }

 done:
  free_set(act, ORC_CNN_NLAYER);
  free_set(pre, ORC_CNN_NLAYER);
  free(g); free(ga); free(out4); free(w);
  return rc;
}

/* Single-layer forms for kernel-level checks.
 * a: [N][32] (already the operand values), w: [27][32][32] */
int orc_conv3_fwd(const int n[3], const double * a, const double * w,
		  const double * b, double * z) {
  conv_fwd(n, a, w, b, z);
  return 0;
}

int orc_conv3_bwd_data(const int n[3], const double * g, const double * w,
		       double * da) {
  conv_bwd_data(n, g, w, da);
  return 0;
}

int orc_conv3_wgrad(const int n[3], const double * g, const double * a,
		    double * dw, double * db) {
  conv_wgrad(n, g, a, dw, db);
  return 0;
}

double orc_bf16_round(double v) { return bf16r(v); }
