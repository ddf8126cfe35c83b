/*****************************************************************************
 *
 *  lgb_lc32_2.cuh
 *
 *  The two kernels of the float LC step (lgb_lc32.cuh) with two sites per
 *  thread: thread (ty, tz) owns the sites of rows 2 ty and 2 ty + 1 of a
 *  2 TYT x 32 (y, z) tile at column tz and computes both in packed FP32x2
 *  arithmetic (vf2).
 *
 *  k_lc32_fields_be2: Q gradients, H, the chiral stress P and the
 *  Beris-Edwards update of the pair (the site functions of k_lc32_fields_be
 *  on vf2).  Of the y neighbours, the lower site's y + 1 is the upper
 *  site and the upper site's y - 1 the lower, so a pair loads 12 values of
 *  each field where two single sites load 14.
 *
 *  k_lc32_collide2: the force + collision kernel; the pulled populations
 *  of plane x + 1 are loaded while plane x is computed.
 *
 *  Same data flow as the one-site kernel: planes of the chiral stress P
 *  (9 components, tile + 1 halo) stream into a 3-slot shared-memory ring
 *  one plane ahead with cp.async; the force is minus the divergence of the
 *  face values 0.5 (P(s) + P(s + e)) (src/phi_force_colloid.c:315-467),
 *  whose own-site halves cancel; then the M10 collision with the force
 *  (src/collision.c:253-593).  No status map (all-fluid lattices); the
 *  one-site kernel serves maps.
 *
 *****************************************************************************/

#ifndef LGB_LC32_2_CUH
#define LGB_LC32_2_CUH

#include "lgb_lc32.cuh"
#include "lgb_vf2.cuh"

template <int TYT, int MINB>
__global__ void __launch_bounds__(32*TYT, MINB)
k_lc32_fields_be2(lgbk_dims_t d, lgbk_lc_f_t p, lgbk_lc_step_args_t a) {
  const int ntz = (d.nz + 31)/32;
  const int z = (blockIdx.x % ntz)*32 + threadIdx.x;
  const int yA = (blockIdx.x / ntz)*(2*TYT) + 2*threadIdx.y;
  const int x = blockIdx.y;
  if (z >= d.nz || yA >= d.ny) return;
  /* the upper site is row yA + 1, or row 0 when yA is the last row: then
   * it is computed (in bounds) and not stored */
  const bool actB = yA + 1 < d.ny;
  const int yB = actB ? yA + 1 : 0;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;
  const unsigned iA = (unsigned) x*NP + yA*d.nz + z;
  const unsigned iB = (unsigned) x*NP + yB*d.nz + z;
  /* neighbour offsets (modulo 2^32) shared by the two sites: x and z */
  const unsigned xw = (unsigned) (d.nx - 1)*NP;
  const unsigned oxp = (x == d.nx - 1) ? 0u - xw : (unsigned) NP;
  const unsigned oxm = (x == 0) ? xw : 0u - (unsigned) NP;
  const unsigned ozp = (z == d.nz - 1) ? 0u - (unsigned) (d.nz - 1) : 1u;
  const unsigned ozm = (z == 0) ? (unsigned) (d.nz - 1) : 0u - 1u;
  /* the lower site's y - 1 and the upper site's y + 1 */
  const unsigned iAym = (yA == 0) ? iA + (unsigned) (d.ny - 1)*d.nz
    : iA - (unsigned) d.nz;
  const unsigned iByp = (yB == d.ny - 1) ? iB - (unsigned) (d.ny - 1)*d.nz
    : iB + (unsigned) d.nz;
  const float * __restrict__ q = (const float *) a.q_in;
  const float * __restrict__ u = (const float *) a.u_in;
  float * __restrict__ qo = (float *) a.q_out;
  float * __restrict__ pth = (float *) a.pth;

  /* neighbour order: 0 x+1, 1 x-1, 2 y+1, 3 y-1, 4 z+1, 5 z-1 */
  auto load = [&](const float * f, vf2 & c, vf2 nbr[6]) {
    const float a0 = f[iA], b0 = f[iB];
    c = vf2(a0, b0);
    nbr[0] = vf2(f[iA + oxp], f[iB + oxp]);
    nbr[1] = vf2(f[iA + oxm], f[iB + oxm]);
    nbr[2] = vf2(b0, f[iByp]);
    nbr[3] = vf2(f[iAym], a0);
    nbr[4] = vf2(f[iA + ozp], f[iB + ozp]);
    nbr[5] = vf2(f[iA + ozm], f[iB + ozm]);
  };
  vf2 qc[5], qn[5][6];
  #pragma unroll
  for (int n = 0; n < 5; n++) load(q + n*N, qc[n], qn[n]);
  vf2 uc[3], un[3][6];
  #pragma unroll
  for (int c = 0; c < 3; c++) load(u + c*N, uc[c], un[c]);

  LcFastT<vf2> w;
  vf2 h[3][3], sth[3][3];
  lc32_fields_site(p, qc, qn, w, h, sth);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) {
      float * pc = pth + (3*ia + ib)*N;
      pc[iA] = sth[ia][ib].v.x;
      if (actB) pc[iB] = sth[ia][ib].v.y;
    }
  }
  const vf2 msk[6] = {vf2(1.0f), vf2(1.0f), vf2(1.0f), vf2(1.0f), vf2(1.0f),
		      vf2(1.0f)};
  vf2 qnew[5];
  lc32_be_site<vf2, false>(a.fp[LGBK_LCF_XI], a.fp[LGBK_LCF_GAMMA_ROT], w,
			   h, qc, qn, uc, un, msk, qnew);
  #pragma unroll
  for (int n = 0; n < 5; n++) {
    float * qn_out = qo + n*N;
    qn_out[iA] = qnew[n].v.x;
    if (actB) qn_out[iB] = qnew[n].v.y;
  }
}

template <typename S, int TYT, int MINB>
__global__ void __launch_bounds__(32*TYT, MINB)
k_lc32_collide2(lgbk_dims_t d, lgbk_lc_step_args_t a, int xchunk) {
  extern __shared__ unsigned char smem_raw[];
  constexpr int TY = 2*TYT;
  using SM = LcCollideSmem<TY>;
  constexpr int TZ = SM::TZ, DZ = SM::RZ, ND = SM::ND, Z0 = SM::Z0;
  constexpr int DY = SM::DY;
  constexpr int NTHR = 32*TYT;
  static_assert(DY*10 <= NTHR, "one copy task per thread");
  float * sP = reinterpret_cast<float *>(smem_raw);        /* [3][9][ND] */

  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty*TZ + tz;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;
  const float * __restrict__ pth = (const float *) a.pth;
  const S * __restrict__ f_in = (const S *) a.f_in;
  S * __restrict__ f_out = (S *) a.f_out;
  float * __restrict__ u_out = (float *) a.u_out;
  float * __restrict__ rho_out = (float *) a.rho_out;
  const float fscale = a.fp[LGBK_LCF_FSCALE];
  const float rfscale = a.fp[LGBK_LCF_RFSCALE];
  const vf2 rho0(a.fp[LGBK_LCF_RHO0]);
  const vf2 rtau(a.fp[LGBK_LCF_RTAU_SHEAR]), rtau_bulk(a.fp[LGBK_LCF_RTAU_BULK]);
  const vf2 half(0.5f);
  /* own sites in the P planes: rows 2 ty + 1 and 2 ty + 2 with the halo */
  const int cA = (2*ty + 1)*DZ + (tz + Z0), cB = cA + DZ;
  const bool vec = (d.nz % 4) == 0;

  const int ntz = (d.nz + TZ - 1)/TZ;
  const int nty = (d.ny + TY - 1)/TY;
  const int ncx = (d.nx + xchunk - 1)/xchunk;
  const int nitems = ntz*nty*ncx;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int itz = item % ntz;
    const int ity = (item / ntz) % nty;
    const int x0 = (item / (ntz*nty))*xchunk;
    const int xe = min(x0 + xchunk, d.nx);
    const int z0 = itz*TZ, y0 = ity*TY;

    /* copy tasks: thread (row r, part t) copies one 16-byte chunk of the
     * row interior (t < 8) or one z-halo float (t = 8, 9) of every plane */
    const bool full = vec && (z0 + TZ <= d.nz);
    const bool copier = tid < DY*10;
    int csrc = 0, cdst = 0, ct = 0;
    if (copier) {
      const int r = tid / 10;
      ct = tid % 10;
      const int lz = (ct < 8) ? 4*ct : ((ct == 8) ? -1 : TZ);
      csrc = lgb_wrap_far(y0 + r - 1, d.ny)*d.nz;
      if (ct >= 8 || full) csrc += lgb_wrap_far(z0 + lz, d.nz);
      cdst = r*DZ + Z0 + lz;
    }
    auto slot = [&](int xx) { return sP + ((xx - x0 + 3) % 3)*9*ND; };
    auto load_P = [&](int xx) {
      if (!copier) return;
      const float * src = pth + (long long) lgb_wrap_far(xx, d.nx)*NP + csrc;
      float * dst = slot(xx) + cdst;
      #pragma unroll
      for (int c = 0; c < 9; c++) {
	const float * sc = src + (long long) c*N;
	float * dc = dst + c*ND;
	if (ct >= 8) {
	  __pipeline_memcpy_async(dc, sc, sizeof(float));
	}
	else if (full) {
	  __pipeline_memcpy_async(dc, sc, 16);
	}
	else {
	  #pragma unroll
	  for (int e = 0; e < 4; e++) {
	    const int z = lgb_wrap_far(z0 + 4*ct + e, d.nz);
	    __pipeline_memcpy_async(dc + e, sc + z, sizeof(float));
	  }
	}
      }
    };

    const int yA = y0 + 2*ty, zg = z0 + tz;
    const bool actA = (yA < d.ny) && (zg < d.nz);
    const bool actB = (yA + 1 < d.ny) && (zg < d.nz);
    const int yAw = actA ? yA : 0, yBw = actB ? yA + 1 : yAw;
    const int zgw = actA ? zg : 0;
    const int oypA = (yAw == 0) ? (d.ny - 1)*d.nz : -d.nz;
    const int oymA = (yAw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
    const int oypB = (yBw == 0) ? (d.ny - 1)*d.nz : -d.nz;
    const int oymB = (yBw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
    const int ozp = (zgw == 0) ? d.nz - 1 : -1;
    const int ozm = (zgw == d.nz - 1) ? -(d.nz - 1) : 1;
    const int syzA = yAw*d.nz + zgw, syzB = yBw*d.nz + zgw;

    /* P_ax of x0 - 1 at the two sites */
    vf2 prevP[3];
    {
      const long long sm1 = (long long) lgb_wrap_far(x0 - 1, d.nx)*NP;
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	prevP[ia] = vf2(pth[(3*ia)*N + sm1 + syzA], pth[(3*ia)*N + sm1 + syzB]);
      }
    }

    /* pulled populations f_p(x - c_p) of both sites, as stored */
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

    __syncthreads();                 /* ring free (previous item done) */
    load_P(x0);
    load_P(x0 + 1);
    __pipeline_commit();
    issue_pull(x0);

    for (int x = x0; x < xe; x++) {
      const unsigned xs = (unsigned) x*NP;
      const unsigned sA = xs + syzA, sB = xs + syzB;

      vf2 fs[LGB_NVEL];
      #pragma unroll
      for (int p = 0; p < LGB_NVEL; p++) {
	fs[p] = vf2(FStore<S, float>::ld(&fr[p][0], rfscale),
		    FStore<S, float>::ld(&fr[p][1], rfscale));
      }
      if (x + 1 < xe) issue_pull(x + 1);

      /* planes x and x + 1 have landed; the slot of x - 1 is free */
      __pipeline_wait_prior(0);
      __syncthreads();
      if (x + 2 <= xe) load_P(x + 2);
      __pipeline_commit();

      const float * Pc = slot(x);
      const float * Pn = slot(x + 1);
      vf2 ftot[3];
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	const float * Px = Pc + (3*ia + 0)*ND;
	const float * Py = Pc + (3*ia + 1)*ND;
	const float * Pz = Pc + (3*ia + 2)*ND;
	const vf2 pxc(Px[cA], Px[cB]);
	const vf2 pxn(Pn[(3*ia)*ND + cA], Pn[(3*ia)*ND + cB]);
	const vf2 pym(Py[cA - DZ], Py[cA]), pyp(Py[cB], Py[cB + DZ]);
	const vf2 pzm(Pz[cA - 1], Pz[cB - 1]), pzp(Pz[cA + 1], Pz[cB + 1]);
	const vf2 force = half*((prevP[ia] - pxn) + (pym - pyp)
				+ (pzm - pzp));
	prevP[ia] = pxc;
	ftot[ia] = vf2(a.fp[LGBK_LCF_FX + ia]) + force;
      }

      vf2 rho, uu[3];
      lgb_collide_site<vf2, false, true, true>(rtau, rtau_bulk,
					       a.cp.rtau_ghost, rho0, fs,
					       ftot, rho, uu);
      if (actA) {
	rho_out[sA] = rho.v.x;
	#pragma unroll
	for (int p = 0; p < LGB_NVEL; p++) {
	  FStore<S, float>::st(f_out + p*N + sA, fs[p].v.x, fscale);
	}
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) u_out[ia*N + sA] = uu[ia].v.x;
      }
      if (actB) {
	rho_out[sB] = rho.v.y;
	#pragma unroll
	for (int p = 0; p < LGB_NVEL; p++) {
	  FStore<S, float>::st(f_out + p*N + sB, fs[p].v.y, fscale);
	}
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) u_out[ia*N + sB] = uu[ia].v.y;
      }
    }
    __pipeline_wait_prior(0);
  }
}

#endif
