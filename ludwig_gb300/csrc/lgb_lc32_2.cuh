/*****************************************************************************
 *
 *  lgb_lc32_2.cuh
 *
 *  The force + collision kernel of the float LC step (k_lc32_collide in
 *  lgb_lc32.cuh) with two sites per thread: thread (ty, tz) owns the sites
 *  of rows 2 ty and 2 ty + 1 of a 2 TYT x 32 (y, z) tile at column tz and
 *  computes both in packed FP32x2 arithmetic (vf2).  The pulled
 *  populations of plane x + 1 are loaded while plane x is computed.
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
