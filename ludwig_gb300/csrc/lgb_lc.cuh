/*****************************************************************************
 *
 *  lgb_lc.cuh
 *
 *  Cholesteric liquid crystal (Landau-de Gennes free energy) per site:
 *  molecular field H_ab (src/blue_phase.c:1016-1110), free-energy density
 *  (:309-400), chiral stress including the antisymmetric part (:827-930,
 *  with its final minus sign) and the Beris-Edwards site update
 *  (src/blue_phase_beris_edwards.c:538-840).  The loops follow the
 *  reference's loop forms, term by term, except that products by a zero
 *  Levi-Civita or Kronecker entry are not formed (adding a zero to a sum
 *  leaves its value unchanged; only the sign of an exact zero can
 *  differ); compiled for FP64 with --fmad=false they give the same values
 *  as the oracle's restatement.
 *
 *  Q is stored as its 5 independent components XX, XY, XZ, YY, YZ
 *  (Q_zz = -Q_xx - Q_yy); gradients as grad[(3*n + ia)*N], delsq[n*N].
 *
 *****************************************************************************/

#ifndef LGB_LC_CUH
#define LGB_LC_CUH

#include "lgb_common.cuh"
#include "lgb_lc.h"
#include "lgb_vf2.cuh"

/* Levi-Civita symbol as a compile-time value */
LGB_HD constexpr int lgb_eps(int a, int b, int c) {
  return ((a - b)*(b - c)*(c - a))/2;
}

template <typename T>
__device__ __forceinline__ void lc_expand(const T * a, long long N,
					  long long i, T t[3][3]) {
  t[0][0] = a[0*N + i];
  t[0][1] = a[1*N + i];
  t[0][2] = a[2*N + i];
  t[1][0] = t[0][1];
  t[1][1] = a[3*N + i];
  t[1][2] = a[4*N + i];
  t[2][0] = t[0][2];
  t[2][1] = t[1][2];
  t[2][2] = T(0.0) - t[0][0] - t[1][1];
}

template <typename T>
__device__ __forceinline__ void lc_expand_grad(const T * g, long long N,
					       long long i, T dq[3][3][3]) {
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    dq[ia][0][0] = g[(3*0 + ia)*N + i];
    dq[ia][0][1] = g[(3*1 + ia)*N + i];
    dq[ia][0][2] = g[(3*2 + ia)*N + i];
    dq[ia][1][0] = dq[ia][0][1];
    dq[ia][1][1] = g[(3*3 + ia)*N + i];
    dq[ia][1][2] = g[(3*4 + ia)*N + i];
    dq[ia][2][0] = dq[ia][0][2];
    dq[ia][2][1] = dq[ia][1][2];
    dq[ia][2][2] = T(0.0) - dq[ia][0][0] - dq[ia][1][1];
  }
}

template <typename T, typename P>
__device__ __forceinline__ void lc_h_site(const P & p, T q[3][3],
					  T dq[3][3][3], T dsq[3][3],
					  T h[3][3]) {
  const T r3 = T(1.0/3.0);
  const T gamma = (T) p.gamma, a0 = (T) p.a0;
  const T q0 = (T) p.q0*(T) p.rredshift;
  const T kappa0 = (T) p.kappa0*(T) p.redshift*(T) p.redshift;
  const T kappa1 = (T) p.kappa1*(T) p.redshift*(T) p.redshift;
  T q2 = T(0.0), eq = T(0.0), e2 = T(0.0);

  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) q2 += q[ia][ib]*q[ia][ib];

  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      T sum = T(0.0);
      const T dab = (T) (ia == ib);
      #pragma unroll
      for (int ic = 0; ic < 3; ic++) sum += q[ia][ic]*q[ib][ic];
      h[ia][ib] = -a0*(T(1.0) - r3*gamma)*q[ia][ib]
	+ a0*gamma*((ia == ib) ? (sum - r3*q2*dab) : sum)
	- a0*gamma*q2*q[ia][ib];
    }
  }

  #pragma unroll
  for (int ib = 0; ib < 3; ib++)
    #pragma unroll
    for (int ic = 0; ic < 3; ic++)
      #pragma unroll
      for (int ia = 0; ia < 3; ia++)
	if (lgb_eps(ib, ic, ia) != 0)
	  eq += ((T) lgb_eps(ib, ic, ia))*dq[ib][ic][ia];

  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      T sum = T(0.0);
      const T dab = (T) (ia == ib);
      #pragma unroll
      for (int ic = 0; ic < 3; ic++) {
	#pragma unroll
	for (int id = 0; id < 3; id++) {
	  const int e1 = lgb_eps(ia, ic, id), e2 = lgb_eps(ib, ic, id);
	  if (e1 != 0 && e2 != 0) {
	    sum += (((T) e1)*dq[ic][ib][id] + ((T) e2)*dq[ic][ia][id]);
	  }
	  else if (e1 != 0) {
	    sum += ((T) e1)*dq[ic][ib][id];
	  }
	  else if (e2 != 0) {
	    sum += ((T) e2)*dq[ic][ia][id];
	  }
	}
      }
      if (ia == ib) {
	h[ia][ib] += kappa0*dsq[ia][ib]
	  - T(2.0)*kappa1*q0*sum + T(4.0)*r3*kappa1*q0*eq*dab
	  - T(4.0)*kappa1*q0*q0*q[ia][ib];
      }
      else {
	h[ia][ib] += kappa0*dsq[ia][ib]
	  - T(2.0)*kappa1*q0*sum
	  - T(4.0)*kappa1*q0*q0*q[ia][ib];
      }
    }
  }

  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const T ea = (T) p.e0[ia]*(T) p.coswt;
    e2 += ea*ea;
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const T ea = (T) p.e0[ia]*(T) p.coswt;
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      const T eb = (T) p.e0[ib]*(T) p.coswt;
      const T dab = (T) (ia == ib);
      h[ia][ib] += (T) p.epsilon*(ea*eb - r3*dab*e2);
    }
  }
}

/* The invariants of the free energy: q2 = Q_ab Q_ab, q3 = Q_ab Q_bc Q_ca,
 * dq0 = (d_b Q_ab)^2, dq1 = (e_acd d_c Q_db + 2 q0 Q_ab)^2, in the order of
 * src/blue_phase.c:284-340 (the same order as blue_phase_fbg,
 * src/fe_lc_stats.c:721-806, for a symmetric Q) */
template <typename T, typename P>
__device__ __forceinline__ void lc_invariants(const P & p, T q[3][3],
					      T dq[3][3][3], T & q2, T & q3,
					      T & dq0, T & dq1) {
  const T q0 = (T) p.q0*(T) p.rredshift;
  q2 = T(0.0); q3 = T(0.0); dq0 = T(0.0); dq1 = T(0.0);

  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) q2 += q[ia][ib]*q[ia][ib];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++)
      #pragma unroll
      for (int ic = 0; ic < 3; ic++) q3 += q[ia][ib]*q[ib][ic]*q[ia][ic];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    T sum = T(0.0);
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) sum += dq[ib][ia][ib];
    dq0 += sum*sum;
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      T sum = T(0.0);
      #pragma unroll
      for (int ic = 0; ic < 3; ic++)
	#pragma unroll
	for (int id = 0; id < 3; id++)
	  if (lgb_eps(ia, ic, id) != 0)
	    sum += ((T) lgb_eps(ia, ic, id))*dq[ic][ib][id];
      sum += T(2.0)*q0*q[ia][ib];
      dq1 += sum*sum;
    }
  }
}

template <typename T, typename P>
__device__ __forceinline__ T lc_fed_site(const P & p, T q[3][3],
					 T dq[3][3][3]) {
  const T r3 = T(1.0/3.0);
  const T gamma = (T) p.gamma, a0 = (T) p.a0;
  const T kappa0 = (T) p.kappa0*(T) p.redshift*(T) p.redshift;
  const T kappa1 = (T) p.kappa1*(T) p.redshift*(T) p.redshift;
  T q2, q3, dq0, dq1, efield = T(0.0);
  lc_invariants<T>(p, q, dq, q2, q3, dq0, dq1);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const T ea = (T) p.e0[ia]*(T) p.coswt;
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      const T eb = (T) p.e0[ib]*(T) p.coswt;
      efield += ea*q[ia][ib]*eb;
    }
  }
  return T(0.5)*a0*(T(1.0) - r3*gamma)*q2 - r3*a0*gamma*q3
    + T(0.25)*a0*gamma*q2*q2 + T(0.5)*kappa0*dq0 + T(0.5)*kappa1*dq1
    - (T) p.epsilon*efield;
}

/* Bulk and gradient parts of the free-energy density, blue_phase_fbg
 * (src/fe_lc_stats.c:721-806): no electric-field term */
template <typename T, typename P>
__device__ __forceinline__ void lc_fbg_site(const P & p, T q[3][3],
					    T dq[3][3][3], T & fbulk,
					    T & fgrad) {
  const T r3 = T(1.0/3.0);
  const T gamma = (T) p.gamma, a0 = (T) p.a0;
  const T kappa0 = (T) p.kappa0*(T) p.redshift*(T) p.redshift;
  const T kappa1 = (T) p.kappa1*(T) p.redshift*(T) p.redshift;
  T q2, q3, dq0, dq1;
  lc_invariants<T>(p, q, dq, q2, q3, dq0, dq1);
  fbulk = T(0.5)*a0*(T(1.0) - r3*gamma)*q2;
  fbulk = fbulk - r3*a0*gamma*q3;
  fbulk = fbulk + T(0.25)*a0*gamma*q2*q2;
  fgrad = T(0.5)*kappa0*dq0;
  fgrad = fgrad + T(0.5)*kappa1*dq1;
}

template <typename T, typename P>
__device__ __forceinline__ void lc_stress_site(const P & p,
					       T q[3][3], T dq[3][3][3],
					       T h[3][3], T sth[3][3]) {
  const T r3 = T(1.0/3.0);
  const T xi = (T) p.xi;
  const T q0 = (T) p.q0*(T) p.rredshift;
  const T kappa0 = (T) p.kappa0*(T) p.redshift*(T) p.redshift;
  const T kappa1 = (T) p.kappa1*(T) p.redshift*(T) p.redshift;
  const T p0 = T(0.0) - lc_fed_site<T>(p, q, dq);
  T qh = T(0.0);

  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) qh += q[ia][ib]*h[ia][ib];

  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      const T dab = (T) (ia == ib);
      if (ia == ib) sth[ia][ib] = -p0*dab + T(2.0)*xi*(q[ia][ib] + r3*dab)*qh;
      else          sth[ia][ib] = T(2.0)*xi*q[ia][ib]*qh;
    }
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      #pragma unroll
      for (int ic = 0; ic < 3; ic++) {
	const T dbc = (T) (ib == ic), dac = (T) (ia == ic);
	const T qbc = (ib == ic) ? (q[ib][ic] + r3*dbc) : q[ib][ic];
	const T qac = (ia == ic) ? (q[ia][ic] + r3*dac) : q[ia][ic];
	sth[ia][ib] += -xi*h[ia][ic]*qbc - xi*qac*h[ib][ic];
      }
    }
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      #pragma unroll
      for (int ic = 0; ic < 3; ic++) {
	#pragma unroll
	for (int id = 0; id < 3; id++) {
	  sth[ia][ib] += - kappa0*dq[ia][ib][ic]*dq[id][ic][id]
	    - kappa1*dq[ia][ic][id]*dq[ib][ic][id]
	    + kappa1*dq[ia][ic][id]*dq[ic][ib][id];
	  #pragma unroll
	  for (int ie = 0; ie < 3; ie++) {
	    if (lgb_eps(ib, ic, ie) != 0) {
	      sth[ia][ib] += -T(2.0)*kappa1*q0*dq[ia][ic][id]
		*((T) lgb_eps(ib, ic, ie))*q[id][ie];
	    }
	  }
	}
      }
    }
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++)
      #pragma unroll
      for (int ic = 0; ic < 3; ic++)
	sth[ia][ib] += q[ia][ic]*h[ib][ic] - h[ia][ic]*q[ib][ic];

  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) sth[ia][ib] = -sth[ia][ib];
}

/*****************************************************************************
 *
 *  Reduced-operation forms for the float path (any summation order is
 *  allowed there).  The reference's loops above carry every Levi-Civita
 *  and Kronecker product, zeros included (a product by a zero constant
 *  cannot be dropped under IEEE rules); written with the intermediates
 *  below, the same quantities take about a third of the operations:
 *
 *    R_ab  = e_acd d_c Q_bd         (curl of Q; tr R is the pseudoscalar)
 *    QQ_ab = Q_ac Q_bc              (q3 = QQ_ab Q_ab)
 *    v_c   = d_d Q_cd               (dq0 = v.v; the kappa0 stress term)
 *    M_ab  = H_ac Qt_cb, Qt = Q + I/3  (the xi terms and [Q, H])
 *    G_ab  = d_a Q_cd d_b Q_cd,  X_ab = d_a Q_cd d_c Q_bd
 *    C_ab  = e_bce d_a Q_cd Q_de    (from the off-diagonal of dQ_a . Q)
 *
 *  H (src/blue_phase.c:1016-1110):
 *    H = c1 Q + a0 gamma (QQ - q2/3 I) + kappa0 d2Q
 *        - 2 kappa1 q0 (R + R^T) + (4/3) kappa1 q0 tr R I + eps (E E - E^2/3 I)
 *    c1 = -a0 (1 - gamma/3) - a0 gamma q2 - 4 kappa1 q0^2
 *  stress (src/blue_phase.c:827-930), before its final sign:
 *    f I + 2 xi Qt (Q:H) - xi (M + M^T) - kappa0 K + kappa1 (X - G)
 *        - 2 kappa1 q0 C + (M^T - M),   K_ab = d_a Q_bc v_c,
 *    X - G = d_a Q_cd (d_c Q_bd - d_b Q_cd) over c != b
 *
 *****************************************************************************/

template <typename T>
struct LcFastT {
  T q[3][3], dq[3][3][3];
  T R[3][3], QQ[3][3], v[3];
  T q2, fed;
};
using LcFast = LcFastT<float>;

/* a*b + c: fused for float (fmaf), one packed FMA for a pair of sites */
__device__ __forceinline__ float lc_fma(float a, float b, float c) {
  return fmaf(a, b, c);
}
__device__ __forceinline__ vf2 lc_fma(const vf2 & a, const vf2 & b,
				      const vf2 & c) {
  return a*b + c;
}

template <typename T>
__device__ __forceinline__ void lc_fast_prepare(LcFastT<T> & w) {
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) {
      /* R_ab = sum_{c,d} e_acd dq[c][b][d]: two terms */
      const int c = (a + 1) % 3, d = (a + 2) % 3;
      w.R[a][b] = w.dq[c][b][d] - w.dq[d][b][c];
    }
  }
  T q2(0.0f);
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) q2 = lc_fma(w.q[a][b], w.q[a][b], q2);
  }
  w.q2 = q2;
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = a; b < 3; b++) {
      T t(0.0f);
      #pragma unroll
      for (int c = 0; c < 3; c++) t = lc_fma(w.q[a][c], w.q[b][c], t);
      w.QQ[a][b] = t;
      w.QQ[b][a] = t;
    }
  }
  #pragma unroll
  for (int c = 0; c < 3; c++) {
    w.v[c] = w.dq[0][c][0] + w.dq[1][c][1] + w.dq[2][c][2];
  }
}

/* Free-energy density (src/blue_phase.c:309-400) */
template <typename T, typename P>
__device__ __forceinline__ T lc_fast_fed(const P & p, const LcFastT<T> & w) {
  const float r3 = 1.0f/3.0f;
  const float gamma = (float) p.gamma, a0 = (float) p.a0;
  const float q0 = (float) p.q0*(float) p.rredshift;
  const float rs2 = (float) p.redshift*(float) p.redshift;
  const float kappa0 = (float) p.kappa0*rs2, kappa1 = (float) p.kappa1*rs2;
  T q3(0.0f), dq1(0.0f), efield(0.0f);
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) {
      q3 = lc_fma(w.QQ[a][b], w.q[a][b], q3);
      const T t = lc_fma(T(2.0f*q0), w.q[a][b], w.R[a][b]);
      dq1 = lc_fma(t, t, dq1);
    }
  }
  const T dq0 = w.v[0]*w.v[0] + w.v[1]*w.v[1] + w.v[2]*w.v[2];
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) {
      efield += (float) p.e0[a]*w.q[a][b]*(float) p.e0[b];
    }
  }
  efield *= (float) p.coswt*(float) p.coswt;
  return 0.5f*a0*(1.0f - r3*gamma)*w.q2 - r3*a0*gamma*q3
    + 0.25f*a0*gamma*w.q2*w.q2 + 0.5f*kappa0*dq0 + 0.5f*kappa1*dq1
    - (float) p.epsilon*efield;
}

/* Molecular field H (symmetric, traceless) */
template <typename T, typename P>
__device__ __forceinline__ void lc_fast_h(const P & p, const LcFastT<T> & w,
					  const T dsq[3][3], T h[3][3]) {
  const float r3 = 1.0f/3.0f;
  const float gamma = (float) p.gamma, a0 = (float) p.a0;
  const float q0 = (float) p.q0*(float) p.rredshift;
  const float rs2 = (float) p.redshift*(float) p.redshift;
  const float kappa0 = (float) p.kappa0*rs2, kappa1 = (float) p.kappa1*rs2;
  const T c1 = -a0*(1.0f - r3*gamma) - a0*gamma*w.q2
    - 4.0f*kappa1*q0*q0;
  const float ag = a0*gamma;
  const float k2 = -2.0f*kappa1*q0;
  const T eq = w.R[0][0] + w.R[1][1] + w.R[2][2];
  float e[3], e2 = 0.0f;
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    e[a] = (float) p.e0[a]*(float) p.coswt;
    e2 += e[a]*e[a];
  }
  const T diag = -r3*ag*w.q2 + 4.0f*r3*kappa1*q0*eq
    - (float) p.epsilon*r3*e2;
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = a; b < 3; b++) {
      T t = c1*w.q[a][b] + ag*w.QQ[a][b] + kappa0*dsq[a][b]
	+ k2*(w.R[a][b] + w.R[b][a]) + (float) p.epsilon*e[a]*e[b];
      if (a == b) t += diag;
      h[a][b] = t;
      h[b][a] = t;
    }
  }
}

/* Chiral stress including the antisymmetric part, with the final sign */
template <typename T, typename P>
__device__ __forceinline__ void lc_fast_stress(const P & p,
					       const LcFastT<T> & w,
					       const T h[3][3], T sth[3][3]) {
  const float r3 = 1.0f/3.0f;
  const float xi = (float) p.xi;
  const float q0 = (float) p.q0*(float) p.rredshift;
  const float rs2 = (float) p.redshift*(float) p.redshift;
  const float kappa0 = (float) p.kappa0*rs2, kappa1 = (float) p.kappa1*rs2;
  const T fed = w.fed;
  T qh(0.0f);
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) qh = lc_fma(w.q[a][b], h[a][b], qh);
  }
  /* M = H Qt */
  T M[3][3];
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) {
      T t = r3*h[a][b];
      #pragma unroll
      for (int c = 0; c < 3; c++) t = lc_fma(h[a][c], w.q[c][b], t);
      M[a][b] = t;
    }
  }
  /* off-diagonal of dQ_a . Q for the chiral term */
  T C[3][3];
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    T Pm[3][3];
    #pragma unroll
    for (int c = 0; c < 3; c++) {
      #pragma unroll
      for (int e = 0; e < 3; e++) {
	if (c == e) continue;
	T t(0.0f);
	#pragma unroll
	for (int d = 0; d < 3; d++) t = lc_fma(w.dq[a][c][d], w.q[d][e], t);
	Pm[c][e] = t;
      }
    }
    C[a][0] = Pm[1][2] - Pm[2][1];
    C[a][1] = Pm[2][0] - Pm[0][2];
    C[a][2] = Pm[0][1] - Pm[1][0];
  }
  /* X - G = d_a Q_cd (d_c Q_bd - d_b Q_cd): the bracket is antisymmetric
   * in (c, b) and vanishes for c = b */
  T Dm[3][3][3];
  #pragma unroll
  for (int c = 0; c < 3; c++) {
    #pragma unroll
    for (int b = c + 1; b < 3; b++) {
      #pragma unroll
      for (int d = 0; d < 3; d++) {
	const T t = w.dq[c][b][d] - w.dq[b][c][d];
	Dm[c][b][d] = t;
	Dm[b][c][d] = -t;
      }
    }
  }
  #pragma unroll
  for (int a = 0; a < 3; a++) {
    #pragma unroll
    for (int b = 0; b < 3; b++) {
      T XG(0.0f), K(0.0f);
      #pragma unroll
      for (int c = 0; c < 3; c++) {
	K = lc_fma(w.dq[a][b][c], w.v[c], K);
	if (c == b) continue;
	#pragma unroll
	for (int d = 0; d < 3; d++) XG = lc_fma(w.dq[a][c][d], Dm[c][b][d], XG);
      }
      const T qt = w.q[a][b] + ((a == b) ? r3 : 0.0f);
      T t = 2.0f*xi*qt*qh - xi*(M[a][b] + M[b][a]) - kappa0*K
	+ kappa1*XG - 2.0f*kappa1*q0*C[a][b]
	+ (M[b][a] - M[a][b]);
      if (a == b) t += fed;
      sth[a][b] = -t;
    }
  }
}

/* H, free energy and stress of one site (or a pair) from Q and its
 * gradients */
template <typename T, typename P>
__device__ __forceinline__ void lc_fast_site(const P & p, LcFastT<T> & w,
					     const T dsq[3][3],
					     T h[3][3], T sth[3][3]) {
  lc_fast_prepare(w);
  w.fed = lc_fast_fed(p, w);
  lc_fast_h(p, w, dsq, h);
  lc_fast_stress(p, w, h, sth);
}

#endif

#ifndef LGB_LC_STEP_KERNELS
#define LGB_LC_STEP_KERNELS

#include "lgb_fused.cuh"

/*****************************************************************************
 *
 *  Two-kernel LC step (src/ludwig.c:528-860 for the cholesteric):
 *
 *  k_lc_fields : Q gradients (7-point, src/gradient_3d_7pt_fluid.c:231) on
 *                the fly, then H (5) and the chiral stress P (9) per site.
 *  k_lc_update : stress-divergence force (src/phi_force_colloid.c:315),
 *                upwind Q fluxes (src/advection.c:538) with the no-flux mask,
 *                Beris-Edwards update (src/blue_phase_beris_edwards.c:538),
 *                pulled populations and the M10 collision with the force.
 *                Q and u are double-buffered (neighbours read old values).
 *
 *  Same arithmetic, in the same order, as the per-function kernels (the
 *  FP64 step; the float step is lgb_lc32.cuh).
 *
 *****************************************************************************/

template <typename T, typename P>
__global__ void k_lc_fields(lgbk_dims_t d, P p,
			    const T * __restrict__ q, T * __restrict__ pth,
			    T * __restrict__ h5) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  int z = (int) (i % d.nz);
  long long r = i / d.nz;
  int y = (int) (r % d.ny);
  int x = (int) (r / d.ny);
  const long long xp = lgb_site_w(d, x+1, y, z), xm = lgb_site_w(d, x-1, y, z);
  const long long yp = lgb_site_w(d, x, y+1, z), ym = lgb_site_w(d, x, y-1, z);
  const long long zp = lgb_site_w(d, x, y, z+1), zm = lgb_site_w(d, x, y, z-1);

  T g[15], dl[5];
  #pragma unroll
  for (int n = 0; n < 5; n++) {
    const T * fn = q + n*N;
    g[3*n + 0] = T(0.5)*(fn[xp] - fn[xm]);
    g[3*n + 1] = T(0.5)*(fn[yp] - fn[ym]);
    g[3*n + 2] = T(0.5)*(fn[zp] - fn[zm]);
    dl[n] = fn[xp] + fn[xm] + fn[yp] + fn[ym] + fn[zp] + fn[zm]
      - T(6.0)*fn[i];
  }
  T qs[3][3], dq[3][3][3], dsq[3][3], hs[3][3], s[3][3];
  lc_expand(q, N, i, qs);
  lc_expand_grad(g, 1, 0, dq);
  lc_expand(dl, 1, 0, dsq);
  lc_h_site<T>(p, qs, dq, dsq, hs);
  lc_stress_site<T>(p, qs, dq, hs, s);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) pth[(3*ia + ib)*N + i] = s[ia][ib];
  h5[0*N + i] = hs[0][0]; h5[1*N + i] = hs[0][1]; h5[2*N + i] = hs[0][2];
  h5[3*N + i] = hs[1][1]; h5[4*N + i] = hs[1][2];
}


/* Step scalars: the doubles themselves for FP64, their float copies
 * otherwise */
template <typename T> struct LcPar;
template <> struct LcPar<double> {
  static __device__ __forceinline__ double get(const lgbk_lc_step_args_t & a,
					       int i) {
    switch (i) {
    case LGBK_LCF_XI: return a.xi;
    case LGBK_LCF_GAMMA_ROT: return a.gamma_rot;
    case LGBK_LCF_RHO0: return a.rho0;
    case LGBK_LCF_FSCALE: return a.fscale;
    case LGBK_LCF_RFSCALE: return 1.0/a.fscale;
    case LGBK_LCF_FX: return a.cp.force_global[0];
    case LGBK_LCF_FY: return a.cp.force_global[1];
    case LGBK_LCF_FZ: return a.cp.force_global[2];
    case LGBK_LCF_RTAU_SHEAR: return a.cp.rtau_shear;
    default: return a.cp.rtau_bulk;
    }
  }
};
template <> struct LcPar<float> {
  static __device__ __forceinline__ float get(const lgbk_lc_step_args_t & a,
					      int i) { return a.fp[i]; }
};

template <typename T, typename S, bool SEQ, bool SHIFT, bool HAS_MAP>
__global__ void k_lc_update(lgbk_dims_t d, lgbk_lc_step_args_t a) {
  long long i = (long long) blockIdx.x*blockDim.x + threadIdx.x;
  if (i >= d.nsites) return;
  const long long N = d.nsites;
  const T r3 = T(1.0/3.0);
  const T dt = T(1.0);
  const T xi = LcPar<T>::get(a, LGBK_LCF_XI);
  const T gamma_rot = LcPar<T>::get(a, LGBK_LCF_GAMMA_ROT);
  const T rho0 = LcPar<T>::get(a, LGBK_LCF_RHO0);
  const T fscale = LcPar<T>::get(a, LGBK_LCF_FSCALE);
  const T rfscale = T(1.0)/fscale;
  int z = (int) (i % d.nz);
  long long r = i / d.nz;
  int y = (int) (r % d.ny);
  int x = (int) (r / d.ny);
  const long long nb[6] = {lgb_site_w(d, x+1, y, z), lgb_site_w(d, x-1, y, z),
			   lgb_site_w(d, x, y+1, z), lgb_site_w(d, x, y-1, z),
			   lgb_site_w(d, x, y, z+1), lgb_site_w(d, x, y, z-1)};
  const T * __restrict__ pth = (const T *) a.pth;
  const T * __restrict__ h5 = (const T *) a.h;
  const T * __restrict__ q = (const T *) a.q_in;
  const T * __restrict__ u = (const T *) a.u_in;
  const uint8_t * __restrict__ st = a.status;

  /* pulled populations first (their latency overlaps the rest) */
  T fs[LGB_NVEL];
  {
    const S * __restrict__ fin = (const S *) a.f_in;
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) {
      long long j = lgb_site_w(d, x - lgb_cv_c[p][0], y - lgb_cv_c[p][1],
			       z - lgb_cv_c[p][2]);
      fs[p] = FStore<S, T>::ld(fin + p*N + j, rfscale);
    }
  }

  /* force: src/phi_force_colloid.c:352-455 */
  T force[3];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const T * px = pth + (3*ia + 0)*N;
    const T * py = pth + (3*ia + 1)*N;
    const T * pz = pth + (3*ia + 2)*N;
    T fa;
    fa  = -T(0.5)*(px[nb[0]] + px[i]);
    fa +=  T(0.5)*(px[nb[1]] + px[i]);
    fa -=  T(0.5)*(py[nb[2]] + py[i]);
    fa +=  T(0.5)*(py[nb[3]] + py[i]);
    fa -=  T(0.5)*(pz[nb[4]] + pz[i]);
    fa +=  T(0.5)*(pz[nb[5]] + pz[i]);
    force[ia] = fa;
  }

  const bool fluid = !HAS_MAP || st[i] == 0;
  T qs[3][3];
  lc_expand(q, N, i, qs);

  /* Beris-Edwards update of the 5 components */
  if (fluid) {
    T s[3][3];
    {
      T w[3][3], dd[3][3], om[3][3];
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	w[ia][0] = T(0.5)*(u[ia*N + nb[0]] - u[ia*N + nb[1]]);
	w[ia][1] = T(0.5)*(u[ia*N + nb[2]] - u[ia*N + nb[3]]);
	w[ia][2] = T(0.5)*(u[ia*N + nb[4]] - u[ia*N + nb[5]]);
      }
      T tr = r3*(w[0][0] + w[1][1] + w[2][2]);
      w[0][0] -= tr; w[1][1] -= tr; w[2][2] -= tr;
      T trace_qw = T(0.0);
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	#pragma unroll
	for (int ib = 0; ib < 3; ib++) {
	  trace_qw += qs[ia][ib]*w[ib][ia];
	  dd[ia][ib] = T(0.5)*(w[ia][ib] + w[ib][ia]);
	  om[ia][ib] = T(0.5)*(w[ia][ib] - w[ib][ia]);
	}
      }
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	#pragma unroll
	for (int ib = 0; ib < 3; ib++) {
	  const T dab = (T) (ia == ib);
	  s[ia][ib] = -T(2.0)*xi*(qs[ia][ib] + r3*dab)*trace_qw;
	  #pragma unroll
	  for (int id = 0; id < 3; id++) {
	    const T ddb = (T) (id == ib), dad = (T) (ia == id);
	    s[ia][ib] += (xi*dd[ia][id] + om[ia][id])*(qs[id][ib] + r3*ddb)
	      + (qs[ia][id] + r3*dad)*(xi*dd[id][ib] - om[id][ib]);
	  }
	}
      }
    }

    /* upwind fluxes (src/advection.c:538-629) of every component at the
     * faces of this site: fw, fe, fy, fz here; fy, fz of y-1 and z-1 */
    T mw = T(1.0), me = T(1.0), my = T(1.0), mz = T(1.0), mym = T(1.0),
      mzm = T(1.0);
    if (HAS_MAP) {
      mw = (T) (st[nb[1]] == 0); me = (T) (st[nb[0]] == 0);
      my = (T) (st[nb[2]] == 0); mz = (T) (st[nb[4]] == 0);
      mym = (T) (st[nb[3]] == 0); mzm = (T) (st[nb[5]] == 0);
    }
    const T ux0 = u[i], uy0 = u[N + i], uz0 = u[2*N + i];
    const T uw = T(0.5)*(ux0 + u[nb[1]]);
    const T ue = T(0.5)*(ux0 + u[nb[0]]);
    const T uyp = T(0.5)*(uy0 + u[N + nb[2]]);
    const T uzp = T(0.5)*(uz0 + u[2*N + nb[4]]);
    const T uym = T(0.5)*(u[N + nb[3]] + uy0);
    const T uzm = T(0.5)*(u[2*N + nb[5]] + uz0);
    const long long iw = (uw > T(0.0)) ? nb[1] : i;
    const long long ie = (ue < T(0.0)) ? nb[0] : i;
    const long long iy = (uyp < T(0.0)) ? nb[2] : i;
    const long long iz = (uzp < T(0.0)) ? nb[4] : i;
    const long long iym = (uym < T(0.0)) ? i : nb[3];
    const long long izm = (uzm < T(0.0)) ? i : nb[5];

    const int ca[5] = {0, 0, 0, 1, 1};
    const int cb[5] = {0, 1, 2, 1, 2};
    T * __restrict__ qo = (T *) a.q_out;
    #pragma unroll
    for (int n = 0; n < 5; n++) {
      const T * qn = q + n*N;
      T fw = uw*qn[iw], fe = ue*qn[ie], fy = uyp*qn[iy], fz = uzp*qn[iz];
      T fyj = uym*qn[iym], fzk = uzm*qn[izm];
      if (HAS_MAP) {
	fw *= T(1.0)*mw; fe *= T(1.0)*me; fy *= T(1.0)*my; fz *= T(1.0)*mz;
	fyj *= mym*T(1.0); fzk *= mzm*T(1.0);
      }
      T v = qs[ca[n]][cb[n]];
      v += dt*(s[ca[n]][cb[n]] + T(0.0) + gamma_rot*h5[n*N + i]
	       - fe + fw - fy + fyj - fz + fzk);
      qo[n*N + i] = v;
    }
  }
  else {
    T * __restrict__ qo = (T *) a.q_out;
    #pragma unroll
    for (int n = 0; n < 5; n++) qo[n*N + i] = q[n*N + i];
  }

  /* collision with the force: global + (zeroed, then added) */
  T ftot[3];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    ftot[ia] = LcPar<T>::get(a, LGBK_LCF_FX + ia) + (T(0.0) + force[ia]*T(1.0));
  }
  T rho, uu[3];
  T * __restrict__ uo = (T *) a.u_out;
  if (fluid) {
    lgb_collide_site<T, SEQ, SHIFT, true>(
      LcPar<T>::get(a, LGBK_LCF_RTAU_SHEAR),
      LcPar<T>::get(a, LGBK_LCF_RTAU_BULK), a.cp.rtau_ghost, rho0, fs, ftot,
      rho, uu);
    ((T *) a.rho_out)[i] = rho;
  }
  else {
    uu[0] = uu[1] = uu[2] = T(0.0);
  }
  S * __restrict__ fo = (S *) a.f_out;
  #pragma unroll
  for (int p = 0; p < LGB_NVEL; p++) FStore<S, T>::st(fo + p*N + i, fs[p], fscale);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) uo[ia*N + i] = uu[ia];
}

#endif
