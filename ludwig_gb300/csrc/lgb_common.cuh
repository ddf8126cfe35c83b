/*****************************************************************************
 *
 *  lgb_common.cuh
 *
 *  Device helpers shared by the kernels: lattice indexing with periodic
 *  wrap, the D3Q19 velocity set, and the per-site collision and free-energy
 *  arithmetic.  The FP64 translation units are compiled with --fmad=false
 *  so that every multiply and add rounds separately, as in the reference's
 *  serial build; the same source instantiated with float (and fmad on)
 *  serves the reduced-precision paths.
 *
 *****************************************************************************/

#ifndef LGB_COMMON_CUH
#define LGB_COMMON_CUH

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "lgb_kernels.h"
#include "lgb_d3q19.h"

#define LGB_HD __host__ __device__ __forceinline__

/* Velocity set as compile-time tables usable in unrolled device loops */
__device__ __constant__ static const int8_t lgb_cv_c[LGB_NVEL][3] =
  LGB_D3Q19_CV;

template <int P> struct Cv;
#define LGB_CV_ROW(p, x, y, z) \
  template <> struct Cv<p> { static constexpr int X = x, Y = y, Z = z; };
LGB_CV_ROW( 0,  0,  0,  0)
LGB_CV_ROW( 1,  1,  1,  0)
LGB_CV_ROW( 2,  1,  0,  1)
LGB_CV_ROW( 3,  1,  0,  0)
LGB_CV_ROW( 4,  1,  0, -1)
LGB_CV_ROW( 5,  1, -1,  0)
LGB_CV_ROW( 6,  0,  1,  1)
LGB_CV_ROW( 7,  0,  1,  0)
LGB_CV_ROW( 8,  0,  1, -1)
LGB_CV_ROW( 9,  0,  0,  1)
LGB_CV_ROW(10,  0,  0, -1)
LGB_CV_ROW(11,  0, -1,  1)
LGB_CV_ROW(12,  0, -1,  0)
LGB_CV_ROW(13,  0, -1, -1)
LGB_CV_ROW(14, -1,  1,  0)
LGB_CV_ROW(15, -1,  0,  1)
LGB_CV_ROW(16, -1,  0,  0)
LGB_CV_ROW(17, -1,  0, -1)
LGB_CV_ROW(18, -1, -1,  0)
#undef LGB_CV_ROW

/* Weights w_p = W36_p / 36 */
LGB_HD double lgb_w(int p) {
  const int w36[LGB_NVEL] = LGB_D3Q19_W36;
  return (double) w36[p] / 36.0;
}

/* Periodic wrap for |offset| <= n (n >= 2 is required of every lattice) */
LGB_HD int lgb_wrap(int i, int n) {
  return (i < 0) ? i + n : ((i >= n) ? i - n : i);
}

LGB_HD long long lgb_site(const lgbk_dims_t & d, int x, int y, int z) {
  return ((long long) x*d.ny + y)*d.nz + z;
}

LGB_HD long long lgb_site_w(const lgbk_dims_t & d, int x, int y, int z) {
  return lgb_site(d, lgb_wrap(x, d.nx), lgb_wrap(y, d.ny), lgb_wrap(z, d.nz));
}

/* Compile-time unroll helper */
template <int N> struct Unroll {
  template <typename Fn> __device__ __forceinline__ static void run(Fn && fn) {
    Unroll<N - 1>::run(fn);
    fn(std::integral_constant<int, N - 1>());
  }
};
template <> struct Unroll<0> {
  template <typename Fn> __device__ __forceinline__ static void run(Fn &&) {}
};

/*****************************************************************************
 *
 *  Symmetric free energy, src/symmetric.c:308-400, per site.
 *
 *****************************************************************************/

template <typename T>
__device__ __forceinline__ T lgb_symm_mu(T a, T b, T kappa, T phi, T delsq) {
  return a*phi + b*phi*phi*phi - kappa*delsq;
}

template <typename T>
__device__ __forceinline__ T lgb_symm_mu(const lgbk_symm_t & fe, T phi,
					 T delsq) {
  return lgb_symm_mu<T>((T) fe.a, (T) fe.b, (T) fe.kappa, phi, delsq);
}

/* p0 of P_ab = p0 delta_ab + kappa g_a g_b (src/symmetric.c:386-391) */
template <typename T>
__device__ __forceinline__ T lgb_symm_p0(T a, T b, T kappa, T phi, T delsq,
					 const T g[3]) {
  return T(0.5)*a*phi*phi + T(0.75)*b*phi*phi*phi*phi - kappa*phi*delsq
    - T(0.5)*kappa*(g[0]*g[0] + g[1]*g[1] + g[2]*g[2]);
}

template <typename T>
__device__ __forceinline__ T lgb_symm_p0(const lgbk_symm_t & fe, T phi,
					 T delsq, const T g[3]) {
  return lgb_symm_p0<T>((T) fe.a, (T) fe.b, (T) fe.kappa, phi, delsq, g);
}

/* Sum of populations fs[p0..18] as h + l with h exact (error-free
 * splitting, as in Rump, Ogita and Oishi's AccSum): for |x| < 8 and
 * C = 1.5*2^4, fl(x + C) - C is x rounded to a multiple of ulp(C) = 2^-19
 * (FP32), exactly, and x minus it is exact too.  The rounded parts then
 * add without error while the partial sums stay below 2^24 ulp(C) = 32;
 * only the remainders (|r| <= 2^-20) are summed with rounding. */
template <typename T, int P0>
__device__ __forceinline__ void lgb_mass_split(const T fs[LGB_NVEL], T & h,
					       T & l) {
  const T C = T(24.0);
  h = T(0.0); l = T(0.0);
  #pragma unroll
  for (int p = P0; p < LGB_NVEL; p++) {
    const T a = fs[p] + C;
    const T hx = a - C;
    h += hx;
    l += fs[p] - hx;
  }
}

/* The same on pairs of populations with the packed FP32x2 operations */
template <int P0>
__device__ __forceinline__ void lgb_mass_split2(const float fs[LGB_NVEL],
						float & h, float & l) {
  const float2 c2 = make_float2(24.0f, 24.0f);
  const float2 m1 = make_float2(-1.0f, -1.0f);
  float2 h2 = make_float2(0.0f, 0.0f), l2 = h2;
  #pragma unroll
  for (int p = 1; p < LGB_NVEL; p += 2) {
    const float2 x = make_float2(fs[p], fs[p + 1]);
    const float2 a = __fadd2_rn(x, c2);
    const float2 hx = __ffma2_rn(c2, m1, a);         /* a - C, exact */
    const float2 lx = __ffma2_rn(hx, m1, x);         /* x - hx, exact */
    h2 = __fadd2_rn(h2, hx);
    l2 = __fadd2_rn(l2, lx);
  }
  h = h2.x + h2.y;
  l = l2.x + l2.y;
  if (P0 == 0) {
    const float a = fs[0] + 24.0f;
    const float hx = a - 24.0f;
    h += hx;
    l += fs[0] - hx;
  }
}

template <typename T, int P0>
__device__ __forceinline__ void lgb_mass(const T fs[LGB_NVEL], T & h, T & l) {
  lgb_mass_split<T, P0>(fs, h, l);
}

template <>
__device__ __forceinline__ void lgb_mass<float, 0>(const float fs[LGB_NVEL],
						   float & h, float & l) {
  lgb_mass_split2<0>(fs, h, l);
}
template <>
__device__ __forceinline__ void lgb_mass<float, 1>(const float fs[LGB_NVEL],
						   float & h, float & l) {
  lgb_mass_split2<1>(fs, h, l);
}

/*****************************************************************************
 *
 *  lgb_collide_site
 *
 *  M10 collision with body force (src/collision.c:253-593), for one site,
 *  on f given as SHIFTED (f - w rho0 when SHIFT, else f itself).
 *  The reference operation order is kept (FP64 exactness); the SEQ flag
 *  selects the reference-order transforms, else the factorised ones.
 *
 *  On exit fs holds post-collision (shifted) populations; rho and u are
 *  the density and velocity the reference stores (src/collision.c:557-590).
 *
 *****************************************************************************/

template <typename T, bool SEQ, bool SHIFT, bool GZERO>
__device__ __forceinline__ void lgb_collide_site_sth(T rtau, T rtau_bulk,
						     const double * rtau_ghost,
						     T rho0, T fs[LGB_NVEL],
						     const T force[3],
						     const T (*sth)[3],
						     T & rho_out, T u[3]);

template <typename T, bool SEQ, bool SHIFT, bool GZERO>
__device__ __forceinline__ void lgb_collide_site(T rtau, T rtau_bulk,
						 const double * rtau_ghost,
						 T rho0, T fs[LGB_NVEL],
						 const T force[3], T & rho_out,
						 T u[3]) {
  lgb_collide_site_sth<T, SEQ, SHIFT, GZERO>(rtau, rtau_bulk, rtau_ghost,
					     rho0, fs, force, nullptr,
					     rho_out, u);
}

/* As lgb_collide_site; a non-null sth adds the thermodynamic stress to the
 * equilibrium stress, seq = rho u u + sth (the two-distribution binary
 * collision, src/collision.c:706-1013). */
template <typename T, bool SEQ, bool SHIFT, bool GZERO>
__device__ __forceinline__ void lgb_collide_site_sth(T rtau, T rtau_bulk,
						     const double * rtau_ghost,
						     T rho0, T fs[LGB_NVEL],
						     const T force[3],
						     const T (*sth)[3],
						     T & rho_out, T u[3]) {
  T mode[LGB_NVEL];
  constexpr int NM = GZERO ? 10 : LGB_NVEL;

  /* Reduced precision: the mass of the incoming populations as an
   * unevaluated sum hi + lo, hi exact (error-free splitting) */
  T mass_hi = T(0.0), mass_lo = T(0.0);
  if (!SEQ) lgb_mass<T, 0>(fs, mass_hi, mass_lo);

  if (SEQ) d3q19_f2mode_seq<T, NM>(fs, mode);
  else     d3q19_f2mode_fast<T, NM>(fs, mode);

  const T rdim = T(1.0/3.0);

  /* density: mode 0 is rho (or rho - rho0 for shifted populations) */
  const T rho = SHIFT ? (rho0 + mode[0]) : mode[0];

  T s[3][3];
  s[0][0] = mode[4]; s[0][1] = mode[5]; s[0][2] = mode[6];
  s[1][1] = mode[7]; s[1][2] = mode[8]; s[2][2] = mode[9];
  s[1][0] = s[0][1]; s[2][0] = s[0][2]; s[2][1] = s[1][2];

  const T rrho = T(1.0)/rho;
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) u[ia] = rrho*(mode[1 + ia] + T(0.5)*force[ia]);

  T seq[3][3];
  T tr_s = T(0.0), tr_seq = T(0.0);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      if (sth) seq[ia][ib] = rho*u[ia]*u[ib] + sth[ia][ib];
      else     seq[ia][ib] = rho*u[ia]*u[ib];
    }
    tr_s   += s[ia][ia];
    tr_seq += seq[ia][ia];
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    s[ia][ia]   -= rdim*tr_s;
    seq[ia][ia] -= rdim*tr_seq;
  }
  tr_s = tr_s - rtau_bulk*(tr_s - tr_seq);

  /* Only the upper triangle feeds the modes (src/collision.c:510-520). */
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = ia; ib < 3; ib++) {
      T sab = s[ia][ib];
      sab -= rtau*(sab - seq[ia][ib]);
      if (ia == ib) sab += T(1.0)*rdim*tr_s;
      sab += (T(2.0) - rtau)*(u[ia]*force[ib] + force[ia]*u[ib]);
      s[ia][ib] = sab;
    }
  }

  #pragma unroll
  for (int ia = 0; ia < 3; ia++) mode[1 + ia] += force[ia];
  mode[4] = s[0][0]; mode[5] = s[0][1]; mode[6] = s[0][2];
  mode[7] = s[1][1]; mode[8] = s[1][2]; mode[9] = s[2][2];

  if (!GZERO) {
    #pragma unroll
    for (int m = 10; m < LGB_NVEL; m++) {
      mode[m] = mode[m] - ((T) rtau_ghost[m])*(mode[m] - T(0.0));
    }
  }

  if (SEQ) d3q19_mode2f_seq<T, NM>(mode, fs);
  else     d3q19_mode2f_fast<T, NM>(mode, fs);

  if (!SEQ) {
    /* Reduced precision: the rounded mode -> f coefficients do not sum
     * exactly to the conserved moments, and the stress modes (which carry
     * rho u u, always positive) then leak mass with one sign every step.
     * Rebuild the rest population from the incoming mass instead, with
     * error-free (split) sums on both sides, so that the populations' sum
     * equals the incoming sum up to one rounding of the rest population
     * and the rounding of the small remainders. */
    T h, l;
    lgb_mass<T, 1>(fs, h, l);
    fs[0] = (mass_hi - h) + (mass_lo - l);
  }

  rho_out = rho;
}

/* As above with the relaxation times of a parameter block */
template <typename T, bool SEQ, bool SHIFT, bool GZERO>
__device__ __forceinline__ void lgb_collide_site(const lgbk_collide_t & cp,
						 T rho0, T fs[LGB_NVEL],
						 const T force[3], T & rho_out,
						 T u[3]) {
  lgb_collide_site<T, SEQ, SHIFT, GZERO>((T) cp.rtau_shear,
					 (T) cp.rtau_bulk, cp.rtau_ghost,
					 rho0, fs, force, rho_out, u);
}

#endif
