/*****************************************************************************
 *
 *  lgb_fused2.cuh
 *
 *  The reduced-precision fused binary-fluid step with two sites per thread:
 *  a thread owns the sites (x, y, z) and (x, y + 1, z) of two neighbouring
 *  rows of the tile and computes both in packed FP32x2 arithmetic (vf2).
 *  The step is the one of lgb_fused.cuh (src/ludwig.c:528-860 for the
 *  symmetric binary fluid): 7-point gradient, stress and chemical
 *  potential in rolling shared-memory planes, force as half central
 *  differences of the stress, upwind + chemical-potential Cahn-Hilliard
 *  fluxes, forward-Euler phi update, pulled populations and the M10
 *  collision with the force.
 *
 *  The one-site kernel issues about 950 (FP32) to 1050 (FP16 storage)
 *  instructions per site and is issue bound; here the arithmetic of the two
 *  sites shares each instruction, and the per-thread index work, loop
 *  control and barriers are shared by two sites.
 *
 *  Tile: 2 TYT rows (y) x 32 (z), TYT x 32 threads; thread (ty, tz) owns
 *  rows 2 ty and 2 ty + 1 at column tz.  Shared memory as FusedSmem with
 *  TY = 2 TYT rows.  The halo ring of the stress/chemical-potential plane
 *  is computed one site per thread by the first NB threads (scalar).
 *
 *  No status map (all-fluid lattices); the one-site kernel serves maps.
 *
 *****************************************************************************/

#ifndef LGB_FUSED2_CUH
#define LGB_FUSED2_CUH

#include "lgb_fused.cuh"
#include "lgb_vf2.cuh"

/* Per-lane typed load/store of the stored distributions */
template <typename S> struct FStore2 {
  static __device__ __forceinline__ float ld(const S * p, float rs) {
    return FStore<S, float>::ld(p, rs);
  }
  static __device__ __forceinline__ void st(S * p, float v, float s) {
    FStore<S, float>::st(p, v, s);
  }
};

/* Stress P_ab (upper triangle and diagonal) and mu of one site from the
 * phi stencil (V = sf1 for the halo ring, vf2 for a thread's two sites:
 * the same roundings, so that a site's values do not depend on whether it
 * is a halo site of one tile or an own site of the next) */
template <typename V>
__device__ __forceinline__ void lgb_d_values(V pa, V pb, V kappa, V c,
					     V xp, V xm, V yp, V ym, V zp,
					     V zm, V out[10]) {
  V g[3];
  g[0] = V(0.5)*(xp - xm);
  g[1] = V(0.5)*(yp - ym);
  g[2] = V(0.5)*(zp - zm);
  const V delsq = xp + xm + yp + ym + zp + zm - V(6.0)*c;
  const V p0 = lgb_symm_p0<V>(pa, pb, kappa, c, delsq, g);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      if (ia == ib) out[3*ia + ib] = p0 + kappa*g[ia]*g[ib];
      else out[3*ia + ib] = kappa*g[ia]*g[ib];
    }
  }
  out[9] = lgb_symm_mu<V>(pa, pb, kappa, c, delsq);
}

template <typename S, int TYT>
__device__ __forceinline__ void
binary_item2(const lgbk_dims_t & d, const lgbk_binary_args_t & a, int itz,
	     int ity, int x0, int xe, unsigned char * smem_raw) {

  constexpr int TY = 2*TYT;                           /* rows of the tile */
  using SM = FusedSmem<float, TY>;
  constexpr int TZ = SM::TZ;
  constexpr int PZ = SM::PZ, DZ = SM::DZ;
  constexpr int NPHI = SM::NPHI, ND = SM::ND;
  constexpr int NTHR = TYT*TZ;
  constexpr int KPHI = (NPHI + NTHR - 1)/NTHR;
  constexpr int KD = (ND + NTHR - 1)/NTHR;
  constexpr int NB = ND - TY*TZ;                      /* halo ring sites */
  static_assert(NB <= NTHR, "one halo ring site per thread at most");

  float * sphi = reinterpret_cast<float *>(smem_raw);   /* [4][NPHI] */
  float * sD = sphi + 4*NPHI;                           /* [2][10][ND] */
  float * su0 = sD + 2*SM::NDC*ND;                      /* [2][3][ND] */

  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty*TZ + tz;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;

  const float * __restrict__ phi_in = (const float *) a.phi_in;
  float * __restrict__ phi_out = (float *) a.phi_out;
  const float * __restrict__ u_in = (const float *) a.u_in;
  float * __restrict__ u_out = (float *) a.u_out;
  float * __restrict__ rho_out = (float *) a.rho_out;
  float * __restrict__ force_out = (float *) a.force_out;
  const S * __restrict__ f_in = (const S *) a.f_in;
  S * __restrict__ f_out = (S *) a.f_out;

  const float mobility_s = a.pf[LGBK_P_MOBILITY];
  const float rho0 = a.pf[LGBK_P_RHO0];
  const float fscale = a.pf[LGBK_P_FSCALE];
  const float rfscale = a.pf[LGBK_P_RFSCALE];
  const float pa_s = a.pf[LGBK_P_A];
  const float pb_s = a.pf[LGBK_P_B];
  const float kappa_s = a.pf[LGBK_P_KAPPA];
  const vf2 mobility(mobility_s), pa(pa_s), pb(pb_s), kappa(kappa_s);

  /* own sites in the D/u planes (rows 2 ty + 1, 2 ty + 2 with the halo)
   * and in the phi planes (rows 2 ty + 2, 2 ty + 3) */
  const int cA = (2*ty + 1)*DZ + (tz + 1), cB = cA + DZ;
  const int pA = (2*ty + 2)*PZ + (tz + 2), pB = pA + PZ;

  const int z0 = itz*TZ, y0 = ity*TY;

  int phoff[KPHI], uoff[KD];
  #pragma unroll
  for (int j = 0; j < KPHI; j++) {
    int k = tid + j*NTHR;
    int ly = k / PZ - 2, lz = k % PZ - 2;
    phoff[j] = (k < NPHI) ? lgb_wrap_far(y0 + ly, d.ny)*d.nz
      + lgb_wrap_far(z0 + lz, d.nz) : -1;
  }
  #pragma unroll
  for (int j = 0; j < KD; j++) {
    int k = tid + j*NTHR;
    int ly = k / DZ - 1, lz = k % DZ - 1;
    uoff[j] = (k < ND) ? lgb_wrap_far(y0 + ly, d.ny)*d.nz
      + lgb_wrap_far(z0 + lz, d.nz) : -1;
  }

  auto pslot = [&](int x) { return (x - x0 + 4) & 3; };
  auto dslot = [&](int x) { return (x - x0 + 2) & 1; };
  auto uslot = [&](int x) { return su0 + ((x - x0 + 2) & 1)*3*ND; };

  auto load_phi = [&](int x) {
    const float * src = phi_in + (long long) lgb_wrap_far(x, d.nx)*NP;
    float * dst = sphi + pslot(x)*NPHI;
    #pragma unroll
    for (int j = 0; j < KPHI; j++) {
      if (phoff[j] >= 0) {
	__pipeline_memcpy_async(dst + tid + j*NTHR, src + phoff[j],
				sizeof(float));
      }
    }
  };

  auto load_u = [&](int x) {
    const float * src = u_in + (long long) lgb_wrap_far(x, d.nx)*NP;
    float * dst = uslot(x);
    #pragma unroll
    for (int j = 0; j < KD; j++) {
      if (uoff[j] >= 0) {
	const int k = tid + j*NTHR;
	__pipeline_memcpy_async(dst + k, src + uoff[j], sizeof(float));
	__pipeline_memcpy_async(dst + ND + k, src + N + uoff[j],
				sizeof(float));
	__pipeline_memcpy_async(dst + 2*ND + k, src + 2*N + uoff[j],
				sizeof(float));
      }
    }
  };

  /* halo ring site of this thread (scalar), or -1 */
  int hring = -1;
  if (tid < NB) {
    if (tid < DZ) hring = tid;                                 /* row 0 */
    else if (tid < 2*DZ) hring = (TY + 1)*DZ + (tid - DZ);     /* last row */
    else if (tid < 2*DZ + TY) hring = (1 + tid - 2*DZ)*DZ;     /* column 0 */
    else hring = (1 + tid - 2*DZ - TY)*DZ + DZ - 1;            /* last col */
  }

  /* D of plane x: the two own sites (packed) and the ring site (scalar) */
  auto compute_D = [&](int x) {
    const float * pc = sphi + pslot(x)*NPHI;
    const float * pp = sphi + pslot(x + 1)*NPHI;
    const float * pm = sphi + pslot(x - 1)*NPHI;
    float * D = sD + dslot(x)*SM::NDC*ND;
    {
      const vf2 c(pc[pA], pc[pB]);
      const vf2 xp(pp[pA], pp[pB]), xm(pm[pA], pm[pB]);
      const vf2 yp(pc[pB], pc[pB + PZ]), ym(pc[pA - PZ], pc[pA]);
      const vf2 zp(pc[pA + 1], pc[pB + 1]), zm(pc[pA - 1], pc[pB - 1]);
      vf2 out[10];
      lgb_d_values<vf2>(pa, pb, kappa, c, xp, xm, yp, ym, zp, zm, out);
      #pragma unroll
      for (int k = 0; k < 10; k++) {
	if (k == 3 || k == 6 || k == 7) continue;       /* lower triangle */
	D[k*ND + cA] = out[k].v.x;
	D[k*ND + cB] = out[k].v.y;
      }
    }
    if (hring >= 0) {
      const int ly = hring / DZ, lz = hring % DZ;
      const int q = (ly + 1)*PZ + (lz + 1);
      sf1 out[10];
      lgb_d_values<sf1>(sf1(pa_s), sf1(pb_s), sf1(kappa_s), sf1(pc[q]),
			sf1(pp[q]), sf1(pm[q]), sf1(pc[q + PZ]),
			sf1(pc[q - PZ]), sf1(pc[q + 1]), sf1(pc[q - 1]), out);
      #pragma unroll
      for (int k = 0; k < 10; k++) {
	if (k == 3 || k == 6 || k == 7) continue;
	D[k*ND + hring] = out[k].v;
      }
    }
  };
  /* P_ab with a > b is P_ba: the stored upper triangle */
  auto pidx = [](int ia, int ib) { return (ia <= ib) ? 3*ia + ib : 3*ib + ia; };

  const int yA = y0 + 2*ty, zg = z0 + tz;
  const bool actA = (yA < d.ny) && (zg < d.nz);
  const bool actB = (yA + 1 < d.ny) && (zg < d.nz);
  const int yAw = actA ? yA : 0, yBw = actB ? yA + 1 : yAw, zgw = actA ? zg : 0;

  /* pull-source offsets in y and z, per site (fixed per item) */
  const int oypA = (yAw == 0) ? (d.ny - 1)*d.nz : -d.nz;
  const int oymA = (yAw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
  const int oypB = (yBw == 0) ? (d.ny - 1)*d.nz : -d.nz;
  const int oymB = (yBw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
  const int ozp = (zgw == 0) ? d.nz - 1 : -1;
  const int ozm = (zgw == d.nz - 1) ? -(d.nz - 1) : 1;
  const int syzA = yAw*d.nz + zgw, syzB = yBw*d.nz + zgw;

  /* ---- prologue ---- */
  load_phi(x0 - 2);
  load_phi(x0 - 1);
  load_phi(x0);
  load_phi(x0 + 1);
  __pipeline_commit();
  __pipeline_wait_prior(0);
  __syncthreads();
  compute_D(x0 - 1);
  __syncthreads();

  /* the x0 - 1 column values the first plane needs: P_ax, mu, phi, u_x
   * (their ring slots are reused before that plane reads them) */
  vf2 prevP[3], prev_fe(0.0f), prev_mu, prev_phi, prev_ux;
  {
    const float * D = sD + dslot(x0 - 1)*SM::NDC*ND;
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      const int k = pidx(ia, 0);
      prevP[ia] = vf2(D[k*ND + cA], D[k*ND + cB]);
    }
    prev_mu = vf2(D[9*ND + cA], D[9*ND + cB]);
    const float * pm = sphi + pslot(x0 - 1)*NPHI;
    prev_phi = vf2(pm[pA], pm[pB]);
    const long long xm = (long long) lgb_wrap_far(x0 - 1, d.nx)*NP;
    prev_ux = vf2(u_in[xm + syzA], u_in[xm + syzB]);
  }
  compute_D(x0);
  load_phi(x0 + 2);
  load_u(x0);
  __pipeline_commit();

  const vf2 half(0.5f), zero(0.0f);

  /* Pulled populations f_p(x - c_p) of both sites, as stored (raw); the
   * loads of plane x + 1 are issued before plane x is computed, so that
   * they are in flight through the whole of its arithmetic. */
  S fr[LGB_NVEL][2];
  auto issue_pull = [&](int x) {
    const unsigned xs = (unsigned) x*NP;
    const unsigned sA = xs + syzA, sB = xs + syzB;
    const unsigned oxp = (x == 0) ? (unsigned) (d.nx - 1)*NP : 0u - NP;
    const unsigned oxm = (x == d.nx - 1) ? 0u - (unsigned) (d.nx - 1)*NP
      : (unsigned) NP;
    Unroll<LGB_NVEL>::run([&](auto P) {
      constexpr int p = decltype(P)::value;
      unsigned offx = 0, offz = 0;
      if (Cv<p>::X == +1) offx = oxp;
      if (Cv<p>::X == -1) offx = oxm;
      if (Cv<p>::Z == +1) offz = (unsigned) ozp;
      if (Cv<p>::Z == -1) offz = (unsigned) ozm;
      unsigned offA = offx + offz, offB = offx + offz;
      if (Cv<p>::Y == +1) { offA += (unsigned) oypA; offB += (unsigned) oypB; }
      if (Cv<p>::Y == -1) { offA += (unsigned) oymA; offB += (unsigned) oymB; }
      const S * fp = f_in + p*N;
      fr[p][0] = fp[sA + offA];
      fr[p][1] = fp[sB + offB];
    });
  };
  issue_pull(x0);

  for (int x = x0; x < xe; x++) {
    const unsigned xs = (unsigned) x*NP;
    const unsigned sA = xs + syzA, sB = xs + syzB;
    const unsigned oxm = (x == d.nx - 1) ? 0u - (unsigned) (d.nx - 1)*NP
      : (unsigned) NP;

    vf2 fs[LGB_NVEL];
    #pragma unroll
    for (int p = 0; p < LGB_NVEL; p++) {
      fs[p] = vf2(FStore<S, float>::ld(&fr[p][0], rfscale),
		  FStore<S, float>::ld(&fr[p][1], rfscale));
    }
    if (x + 1 < xe) issue_pull(x + 1);

    __pipeline_wait_prior(0);
    __syncthreads();
    if (x + 1 < xe) {
      load_phi(x + 3);
      load_u(x + 1);
    }
    __pipeline_commit();
    compute_D(x + 1);

    const float * Dc = sD + dslot(x)*SM::NDC*ND;
    const float * Dn = sD + dslot(x + 1)*SM::NDC*ND;
    const float * pc = sphi + pslot(x)*NPHI;
    const float * pn = sphi + pslot(x + 1)*NPHI;
    const float * su = uslot(x);

    /* Force: minus the divergence of the face stresses; the own-site
     * halves cancel: 0.5 (P(x-1) - P(x+1)) summed over the axes */
    vf2 force[3];
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      const int kx = pidx(ia, 0), ky = pidx(ia, 1), kz = pidx(ia, 2);
      const vf2 pxc(Dc[kx*ND + cA], Dc[kx*ND + cB]);
      const vf2 pxn(Dn[kx*ND + cA], Dn[kx*ND + cB]);
      const vf2 pym(Dc[ky*ND + cA - DZ], Dc[ky*ND + cA]);
      const vf2 pyp(Dc[ky*ND + cB], Dc[ky*ND + cB + DZ]);
      const vf2 pzm(Dc[kz*ND + cA - 1], Dc[kz*ND + cB - 1]);
      const vf2 pzp(Dc[kz*ND + cA + 1], Dc[kz*ND + cB + 1]);
      force[ia] = half*((prevP[ia] - pxn) + (pym - pyp) + (pzm - pzp));
      prevP[ia] = pxc;
    }

    /* Cahn-Hilliard fluxes (upwind advective + chemical potential) */
    const vf2 phic(pc[pA], pc[pB]);
    const vf2 muc(Dc[9*ND + cA], Dc[9*ND + cB]);
    const vf2 uxc(su[cA], su[cB]);
    const vf2 uyc(su[ND + cA], su[ND + cB]);
    const vf2 uzc(su[2*ND + cA], su[2*ND + cB]);
    vf2 fw;
    if (x > x0) {
      fw = prev_fe;            /* the x-1 site's east face is this west face */
    }
    else {
      const vf2 uf = half*(uxc + prev_ux);
      fw = uf*sel_gt0(uf, prev_phi, phic);
      fw -= mobility*(muc - prev_mu);
    }
    vf2 fe, fy, fym, fz, fzm;
    {
      const vf2 uxp(u_in[sA + oxm], u_in[sB + oxm]);
      const vf2 phip(pn[pA], pn[pB]);
      const vf2 mup(Dn[9*ND + cA], Dn[9*ND + cB]);
      const vf2 uf = half*(uxc + uxp);
      fe = uf*sel_lt0(uf, phip, phic);
      fe -= mobility*(mup - muc);
    }
    {
      const vf2 uyn(su[ND + cB], su[ND + cB + DZ]);
      const vf2 phin(pc[pB], pc[pB + PZ]);
      const vf2 mun(Dc[9*ND + cB], Dc[9*ND + cB + DZ]);
      const vf2 uf = half*(uyc + uyn);
      fy = uf*sel_lt0(uf, phin, phic);
      fy -= mobility*(mun - muc);
    }
    {
      const vf2 uyn(su[ND + cA - DZ], su[ND + cA]);
      const vf2 phin(pc[pA - PZ], pc[pA]);
      const vf2 mun(Dc[9*ND + cA - DZ], Dc[9*ND + cA]);
      const vf2 uf = half*(uyn + uyc);
      fym = uf*sel_lt0(uf, phic, phin);
      fym -= mobility*(muc - mun);
    }
    {
      const vf2 uzn(su[2*ND + cA + 1], su[2*ND + cB + 1]);
      const vf2 phin(pc[pA + 1], pc[pB + 1]);
      const vf2 mun(Dc[9*ND + cA + 1], Dc[9*ND + cB + 1]);
      const vf2 uf = half*(uzc + uzn);
      fz = uf*sel_lt0(uf, phin, phic);
      fz -= mobility*(mun - muc);
    }
    {
      const vf2 uzn(su[2*ND + cA - 1], su[2*ND + cB - 1]);
      const vf2 phin(pc[pA - 1], pc[pB - 1]);
      const vf2 mun(Dc[9*ND + cA - 1], Dc[9*ND + cB - 1]);
      const vf2 uf = half*(uzn + uzc);
      fzm = uf*sel_lt0(uf, phic, phin);
      fzm -= mobility*(muc - mun);
    }
    const vf2 phinew = phic - (fe - fw + fy - fym + fz - fzm);
    prev_fe = fe;

    vf2 ftot[3];
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      ftot[ia] = vf2(a.pf[LGBK_P_FX + ia]) + force[ia];
    }

    vf2 rho, uu[3];
    lgb_collide_site<vf2, false, true, true>(
      vf2(a.pf[LGBK_P_RTAU_SHEAR]), vf2(a.pf[LGBK_P_RTAU_BULK]),
      a.cp.rtau_ghost, vf2(rho0), fs, ftot, rho, uu);

    if (actA) {
      phi_out[sA] = phinew.v.x;
      rho_out[sA] = rho.v.x;
      #pragma unroll
      for (int p = 0; p < LGB_NVEL; p++) {
	FStore2<S>::st(f_out + p*N + sA, fs[p].v.x, fscale);
      }
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) (u_out + ia*N)[sA] = uu[ia].v.x;
      if (force_out) {
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) (force_out + ia*N)[sA] = force[ia].v.x;
      }
    }
    if (actB) {
      phi_out[sB] = phinew.v.y;
      rho_out[sB] = rho.v.y;
      #pragma unroll
      for (int p = 0; p < LGB_NVEL; p++) {
	FStore2<S>::st(f_out + p*N + sB, fs[p].v.y, fscale);
      }
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) (u_out + ia*N)[sB] = uu[ia].v.y;
      if (force_out) {
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) (force_out + ia*N)[sB] = force[ia].v.y;
      }
    }
  }
  __pipeline_wait_prior(0);
  __syncthreads();
}

template <typename S, int TYT, int MINB>
__global__ void __launch_bounds__(32*TYT, MINB)
k_binary_fused2(lgbk_dims_t d, lgbk_binary_args_t a, int xchunk) {
  extern __shared__ unsigned char smem_raw[];
  constexpr int TY = 2*TYT;
  const int ntz = (d.nz + 31)/32;
  const int nty = (d.ny + TY - 1)/TY;
  const int ncx = (d.nx + xchunk - 1)/xchunk;
  const int nitems = ntz*nty*ncx;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int itz = item % ntz;
    const int ity = (item / ntz) % nty;
    const int x0 = (item / (ntz*nty))*xchunk;
    binary_item2<S, TYT>(d, a, itz, ity, x0, min(x0 + xchunk, d.nx),
			 smem_raw);
  }
}

/* Ensembles: as k_binary_ensemble with two sites per thread */
template <typename S, int TYT, int MINB>
__global__ void __launch_bounds__(32*TYT, MINB)
k_binary_ensemble2(const lgbk_box_t * __restrict__ boxes,
		   const int2 * __restrict__ items, int nitems, int xchunk,
		   int * __restrict__ sched) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ lgbk_box_t sb;
  __shared__ int2 sit;
  constexpr int TY = 2*TYT;
  for (;;) {
    __syncthreads();                 /* the last item is done with sb, sit */
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      sit = lgbk_sched_next(sched, items, nitems);
      if (sit.x >= 0) sb = boxes[sit.x];
    }
    __syncthreads();
    const int2 it = sit;
    if (it.x < 0) break;
    if (!sb.active) continue;
    const int ntz = (sb.d.nz + 31)/32;
    const int nty = (sb.d.ny + TY - 1)/TY;
    const int itz = it.y % ntz;
    const int ity = (it.y / ntz) % nty;
    const int x0 = (it.y / (ntz*nty))*xchunk;
    binary_item2<S, TYT>(sb.d, sb.a, itz, ity, x0,
			 min(x0 + xchunk, sb.d.nx), smem_raw);
  }
  lgbk_sched_retire(sched);
}

#endif
