/*****************************************************************************
 *
 *  lgb_lc32.cuh
 *
 *  The float LC step in two kernels, split so that each array crosses HBM
 *  once per step:
 *
 *  k_lc32_fields_be : per site, from Q and u of the previous step: the
 *                     7-point Q gradients (src/gradient_3d_7pt_fluid.c:231),
 *                     the molecular field H and the chiral stress P
 *                     (src/blue_phase.c:827-1110, reduced-operation forms of
 *                     lgb_lc.cuh), then the Beris-Edwards update with the
 *                     upwind fluxes and the no-flux mask
 *                     (src/blue_phase_beris_edwards.c:538-840,
 *                     src/advection.c:538, src/advection_bcs.c:42).
 *                     Reads Q (5) and u (3), writes Q (5) and P (9); H
 *                     stays in registers.
 *  k_lc32_collide   : stress-divergence force (src/phi_force_colloid.c:315)
 *                     from P, the pulled populations and the M10 collision
 *                     with the force.  A CTA owns a TY x 32 (y, z) tile and
 *                     marches along x; planes of P (tile + 1 halo) stream
 *                     into a 3-slot shared-memory ring one plane ahead with
 *                     cp.async, so every P value is read from HBM once.
 *
 *  The reference applies the force of step n to the collision after the
 *  Beris-Edwards update of step n; both use Q of step n only, so splitting
 *  the work this way keeps the reference's data dependences.
 *
 *****************************************************************************/

#ifndef LGB_LC32_CUH
#define LGB_LC32_CUH

#include "lgb_lc.cuh"

/* Launch shape of k_lc32_fields_be: blocks of 32 (z) x LC32_FY (y) sites,
 * grid (z tiles * y tiles, nx), LC32_FMINB blocks per SM (a cap of 102
 * registers, no spills).  Measured LC step at 128^3 (FY, blocks/SM):
 * (4, 4) 0.169 ms, (4, 5) 0.162, (4, 6) 0.171 (spills), (2, 10) 0.162,
 * (8, 2) 0.173. */
#define LC32_FY 2
#define LC32_FMINB 10

/* lane-wise c = (u > 0) ? a : b for one site or a pair */
__device__ __forceinline__ float lc_sel_gt0(float u, float a, float b) {
  return (u > 0.0f) ? a : b;
}
__device__ __forceinline__ vf2 lc_sel_gt0(const vf2 & u, const vf2 & a,
					  const vf2 & b) {
  return sel_gt0(u, a, b);
}
__device__ __forceinline__ float lc_sel_lt0(float u, float a, float b) {
  return (u < 0.0f) ? a : b;
}
__device__ __forceinline__ vf2 lc_sel_lt0(const vf2 & u, const vf2 & a,
					  const vf2 & b) {
  return sel_lt0(u, a, b);
}

/* H and the chiral stress P of a site (T = float) or of a pair of sites
 * (T = vf2) from Q at the site and its six neighbours (0 x+1, 1 x-1,
 * 2 y+1, 3 y-1, 4 z+1, 5 z-1); w keeps Q for the update */
template <typename T, typename P>
__device__ __forceinline__ void lc32_fields_site(const P & p, const T qc[5],
						 const T qn[5][6],
						 LcFastT<T> & w, T h[3][3],
						 T sth[3][3]) {
  T dsq[3][3];
  {
    T g[15], dl[5];
    #pragma unroll
    for (int n = 0; n < 5; n++) {
      g[3*n + 0] = 0.5f*(qn[n][0] - qn[n][1]);
      g[3*n + 1] = 0.5f*(qn[n][2] - qn[n][3]);
      g[3*n + 2] = 0.5f*(qn[n][4] - qn[n][5]);
      dl[n] = qn[n][0] + qn[n][1] + qn[n][2] + qn[n][3] + qn[n][4]
	+ qn[n][5] - 6.0f*qc[n];
    }
    lc_expand(qc, 1, 0, w.q);
    lc_expand_grad(g, 1, 0, w.dq);
    lc_expand(dl, 1, 0, dsq);
  }
  lc_fast_site(p, w, dsq, h, sth);
}

/* Beris-Edwards update of a site or a pair: S = -2 xi Qt (Q:W) + A Qt +
 * (A Qt)^T with A = xi D + Omega, the upwind fluxes of Q with the face
 * velocities, and the no-flux mask m (neighbour order as above; used only
 * with HAS_MAP) */
template <typename T, bool HAS_MAP>
__device__ __forceinline__ void lc32_be_site(float xi, float gamma_rot,
					     const LcFastT<T> & w,
					     const T h[3][3], const T qc[5],
					     const T qn[5][6], const T uc[3],
					     const T un[3][6], const T m[6],
					     T qo[5]) {
  const float r3 = 1.0f/3.0f;
  T s5[5];
  {
    T wv[3][3];
    #pragma unroll
    for (int c = 0; c < 3; c++) {
      wv[c][0] = 0.5f*(un[c][0] - un[c][1]);
      wv[c][1] = 0.5f*(un[c][2] - un[c][3]);
      wv[c][2] = 0.5f*(un[c][4] - un[c][5]);
    }
    const T tr = r3*(wv[0][0] + wv[1][1] + wv[2][2]);
    wv[0][0] -= tr; wv[1][1] -= tr; wv[2][2] -= tr;
    T tqw(0.0f), A[3][3], qt[3][3];
    #pragma unroll
    for (int ia = 0; ia < 3; ia++) {
      #pragma unroll
      for (int ib = 0; ib < 3; ib++) {
	tqw += w.q[ia][ib]*wv[ib][ia];
	A[ia][ib] = 0.5f*(xi*(wv[ia][ib] + wv[ib][ia])
			  + (wv[ia][ib] - wv[ib][ia]));
	qt[ia][ib] = w.q[ia][ib] + ((ia == ib) ? r3 : 0.0f);
      }
    }
    auto aq = [&](int ia, int ib) -> T {
      return A[ia][0]*qt[0][ib] + A[ia][1]*qt[1][ib] + A[ia][2]*qt[2][ib];
    };
    const T m2 = -2.0f*xi*tqw;
    s5[0] = m2*qt[0][0] + 2.0f*aq(0, 0);
    s5[1] = m2*qt[0][1] + aq(0, 1) + aq(1, 0);
    s5[2] = m2*qt[0][2] + aq(0, 2) + aq(2, 0);
    s5[3] = m2*qt[1][1] + 2.0f*aq(1, 1);
    s5[4] = m2*qt[1][2] + aq(1, 2) + aq(2, 1);
  }

  /* upwind face velocities, masked by the no-flux condition */
  const T uw = 0.5f*(uc[0] + un[0][1]);
  const T ue = 0.5f*(uc[0] + un[0][0]);
  const T uyp = 0.5f*(uc[1] + un[1][2]);
  const T uym = 0.5f*(un[1][3] + uc[1]);
  const T uzp = 0.5f*(uc[2] + un[2][4]);
  const T uzm = 0.5f*(un[2][5] + uc[2]);
  const T muw = HAS_MAP ? T(m[1]*uw) : uw;
  const T mue = HAS_MAP ? T(m[0]*ue) : ue;
  const T muyp = HAS_MAP ? T(m[2]*uyp) : uyp;
  const T muzp = HAS_MAP ? T(m[4]*uzp) : uzp;
  const T muym = HAS_MAP ? T(m[3]*uym) : uym;
  const T muzm = HAS_MAP ? T(m[5]*uzm) : uzm;
  const T hv[5] = {h[0][0], h[0][1], h[0][2], h[1][1], h[1][2]};
  #pragma unroll
  for (int n = 0; n < 5; n++) {
    const auto fw = muw*lc_sel_gt0(uw, qn[n][1], qc[n]);
    const auto fe = mue*lc_sel_lt0(ue, qn[n][0], qc[n]);
    const auto fy = muyp*lc_sel_lt0(uyp, qn[n][2], qc[n]);
    const auto fz = muzp*lc_sel_lt0(uzp, qn[n][4], qc[n]);
    const auto fyj = muym*lc_sel_lt0(uym, qc[n], qn[n][3]);
    const auto fzk = muzm*lc_sel_lt0(uzm, qc[n], qn[n][5]);
    qo[n] = qc[n] + (s5[n] + gamma_rot*hv[n] - fe + fw - fy + fyj
		     - fz + fzk);
  }
}

template <bool HAS_MAP>
__global__ void __launch_bounds__(32*LC32_FY, LC32_FMINB)
k_lc32_fields_be(lgbk_dims_t d, lgbk_lc_f_t p, lgbk_lc_step_args_t a) {
  const int ntz = (d.nz + 31)/32;
  const int z = (blockIdx.x % ntz)*32 + threadIdx.x;
  const int y = (blockIdx.x / ntz)*LC32_FY + threadIdx.y;
  const int x = blockIdx.y;
  if (z >= d.nz || y >= d.ny) return;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;
  /* 32-bit unsigned site indices (the host refuses 2^32 sites or more);
   * pointers are formed from per-component bases */
  const unsigned i = (unsigned) x*NP + y*d.nz + z;
  /* neighbours: 0 x+1, 1 x-1, 2 y+1, 3 y-1, 4 z+1, 5 z-1 */
  const unsigned xw = (unsigned) (d.nx - 1)*NP;   /* x wrap, modulo 2^32 */
  const unsigned nb[6] = {
    (x == d.nx - 1) ? i - xw : i + NP,
    (x == 0) ? i + xw : i - NP,
    i + ((y == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz),
    i + ((y == 0) ? (d.ny - 1)*d.nz : -d.nz),
    i + ((z == d.nz - 1) ? -(d.nz - 1) : 1),
    i + ((z == 0) ? d.nz - 1 : -1)};
  const float * __restrict__ q = (const float *) a.q_in;
  const float * __restrict__ u = (const float *) a.u_in;
  const uint8_t * __restrict__ st = a.status;
  float * __restrict__ qo = (float *) a.q_out;
  float * __restrict__ pth = (float *) a.pth;

  /* Q at the site and its six neighbours, all five components */
  float qc[5], qn[5][6];
  #pragma unroll
  for (int n = 0; n < 5; n++) {
    const float * fn = q + n*N;
    qc[n] = fn[i];
    #pragma unroll
    for (int k = 0; k < 6; k++) qn[n][k] = fn[nb[k]];
  }
  float uc[3], un[3][6];
  #pragma unroll
  for (int c = 0; c < 3; c++) {
    const float * fu = u + c*N;
    uc[c] = fu[i];
    #pragma unroll
    for (int k = 0; k < 6; k++) un[c][k] = fu[nb[k]];
  }

  /* H and P */
  LcFast w;
  float h[3][3], sth[3][3];
  lc32_fields_site(p, qc, qn, w, h, sth);
  #pragma unroll
  for (int ia = 0; ia < 3; ia++)
    #pragma unroll
    for (int ib = 0; ib < 3; ib++) (pth + (3*ia + ib)*N)[i] = sth[ia][ib];

  const bool fluid = !HAS_MAP || st[i] == 0;
  if (!fluid) {
    #pragma unroll
    for (int n = 0; n < 5; n++) (qo + n*N)[i] = qc[n];
    return;
  }

  float msk[6] = {1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.0f};
  if (HAS_MAP) {
    #pragma unroll
    for (int k = 0; k < 6; k++) msk[k] = (float) (st[nb[k]] == 0);
  }
  float qnew[5];
  lc32_be_site<float, HAS_MAP>(a.fp[LGBK_LCF_XI], a.fp[LGBK_LCF_GAMMA_ROT],
			       w, h, qc, qn, uc, un, msk, qnew);
  #pragma unroll
  for (int n = 0; n < 5; n++) (qo + n*N)[i] = qnew[n];
}

/* Force + collision without a plane ring (all-fluid lattices): one site
 * per thread on a (z tiles x y tiles, nx) grid; the stress neighbours
 * come through L1 like the fields kernel's Q neighbours, so that no
 * barrier separates the planes. */
template <typename S, int TY, int MINB>
__global__ void __launch_bounds__(32*TY, MINB)
k_lc32_collide_direct(lgbk_dims_t d, lgbk_lc_step_args_t a) {
  const int ntz = (d.nz + 31)/32;
  const int z = (blockIdx.x % ntz)*32 + threadIdx.x;
  const int y = (blockIdx.x / ntz)*TY + threadIdx.y;
  const int x = blockIdx.y;
  if (z >= d.nz || y >= d.ny) return;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;
  const unsigned s0 = (unsigned) x*NP + y*d.nz + z;
  const unsigned xw = (unsigned) (d.nx - 1)*NP;
  /* neighbours: x+1, x-1, y+1, y-1, z+1, z-1 */
  const unsigned sxp = (x == d.nx - 1) ? s0 - xw : s0 + NP;
  const unsigned sxm = (x == 0) ? s0 + xw : s0 - NP;
  const unsigned syp = s0 + ((y == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz);
  const unsigned sym = s0 + ((y == 0) ? (d.ny - 1)*d.nz : -d.nz);
  const unsigned szp = s0 + ((z == d.nz - 1) ? -(d.nz - 1) : 1);
  const unsigned szm = s0 + ((z == 0) ? d.nz - 1 : -1);
  const float * __restrict__ pth = (const float *) a.pth;
  const S * __restrict__ f_in = (const S *) a.f_in;
  S * __restrict__ f_out = (S *) a.f_out;
  float * __restrict__ u_out = (float *) a.u_out;
  float * __restrict__ rho_out = (float *) a.rho_out;
  const float rho0 = a.fp[LGBK_LCF_RHO0];
  const float fscale = a.fp[LGBK_LCF_FSCALE];
  const float rfscale = a.fp[LGBK_LCF_RFSCALE];

  /* pulled populations f_p(x - c_p) */
  const int oxp = (x == 0) ? (d.nx - 1)*NP : -NP;
  const int oxm = (x == d.nx - 1) ? -(d.nx - 1)*NP : NP;
  const int oyp = (y == 0) ? (d.ny - 1)*d.nz : -d.nz;
  const int oym = (y == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
  const int ozp = (z == 0) ? d.nz - 1 : -1;
  const int ozm = (z == d.nz - 1) ? -(d.nz - 1) : 1;
  float fs[LGB_NVEL];
  const S * fb = f_in + s0;
  Unroll<LGB_NVEL>::run([&](auto P) {
    constexpr int pp = decltype(P)::value;
    int off = 0;
    if (Cv<pp>::X == +1) off += oxp;
    if (Cv<pp>::X == -1) off += oxm;
    if (Cv<pp>::Y == +1) off += oyp;
    if (Cv<pp>::Y == -1) off += oym;
    if (Cv<pp>::Z == +1) off += ozp;
    if (Cv<pp>::Z == -1) off += ozm;
    fs[pp] = FStore<S, float>::ld(fb + pp*N + off, rfscale);
  });

  /* minus the divergence of the face values 0.5 (P(s) + P(s + e)); the
   * own-site halves cancel */
  float ftot[3];
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) {
    const float * Px = pth + (3*ia + 0)*N;
    const float * Py = pth + (3*ia + 1)*N;
    const float * Pz = pth + (3*ia + 2)*N;
    const float force = 0.5f*((Px[sxm] - Px[sxp]) + (Py[sym] - Py[syp])
			      + (Pz[szm] - Pz[szp]));
    ftot[ia] = a.fp[LGBK_LCF_FX + ia] + force;
  }
  float rho, uu[3];
  lgb_collide_site<float, false, true, true>(
    a.fp[LGBK_LCF_RTAU_SHEAR], a.fp[LGBK_LCF_RTAU_BULK],
    a.cp.rtau_ghost, rho0, fs, ftot, rho, uu);
  rho_out[s0] = rho;
  S * ob = f_out + s0;
  #pragma unroll
  for (int pp = 0; pp < LGB_NVEL; pp++) {
    FStore<S, float>::st(ob + pp*N, fs[pp], fscale);
  }
  #pragma unroll
  for (int ia = 0; ia < 3; ia++) u_out[ia*N + s0] = uu[ia];
}

/* A plane of P in shared memory: 9 components x (TY + 2) rows of RZ
 * floats; the 32 interior z values of a row start at float 4 (16-byte
 * aligned, so that they arrive as 16-byte copies), the z halo sits at
 * floats 3 and 36 */
template <int TY>
struct LcCollideSmem {
  static constexpr int TZ = 32;
  static constexpr int DY = TY + 2, RZ = 40, Z0 = 4;
  static constexpr int ND = DY*RZ;
  static constexpr size_t bytes() { return sizeof(float)*3*9*ND; }
};

template <typename S, bool HAS_MAP, int TY, int MINB>
__global__ void __launch_bounds__(32*TY, MINB)
k_lc32_collide(lgbk_dims_t d, lgbk_lc_step_args_t a, int xchunk) {
  extern __shared__ unsigned char smem_raw[];
  using SM = LcCollideSmem<TY>;
  constexpr int TZ = SM::TZ, DZ = SM::RZ, ND = SM::ND, Z0 = SM::Z0;
  constexpr int DY = SM::DY;
  static_assert(DY*10 <= TY*TZ, "one copy task per thread");
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
  const uint8_t * __restrict__ st = a.status;
  const float rho0 = a.fp[LGBK_LCF_RHO0];
  const float fscale = a.fp[LGBK_LCF_FSCALE];
  const float rfscale = a.fp[LGBK_LCF_RFSCALE];
  const int cidx = (ty + 1)*DZ + (tz + Z0);
  /* 16-byte copies need 16-byte aligned rows: nz a multiple of 4 */
  const bool vec = (d.nz % 4) == 0;

  const int ntz = (d.nz + TZ - 1)/TZ;
  const int nty = (d.ny + TY - 1)/TY;

  /* work items (tile, chunk of xchunk planes), z tiles fastest so that
   * neighbouring CTAs stream neighbouring rows of the same planes */
  const int ncx = (d.nx + xchunk - 1)/xchunk;
  const int nitems = ntz*nty*ncx;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int itz = item % ntz;
    const int ity = (item / ntz) % nty;
    const int x0 = (item / (ntz*nty))*xchunk;
    const int xe = min(x0 + xchunk, d.nx);
    const int z0 = itz*TZ, y0 = ity*TY;

    /* Copy tasks: the first DY*10 threads each own one (row r, part t)
     * of the tile -- t < 8 a 16-byte chunk of the row interior, t = 8, 9
     * the z-halo floats -- and copy it for the 9 components of every
     * plane; source and destination offsets are fixed for the item. */
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
	  __pipeline_memcpy_async(dc, sc, sizeof(float));      /* z halo */
	}
	else if (full) {
	  __pipeline_memcpy_async(dc, sc, 16);
	}
	else {
	  /* a chunk of a partial tile, element by element (positions past
	   * the lattice edge take their periodic images); sc is the row */
	  #pragma unroll
	  for (int e = 0; e < 4; e++) {
	    const int z = lgb_wrap_far(z0 + 4*ct + e, d.nz);
	    __pipeline_memcpy_async(dc + e, sc + z, sizeof(float));
	  }
	}
      }
    };

    const int yg = y0 + ty, zg = z0 + tz;
    const bool active = (yg < d.ny) && (zg < d.nz);
    const int ygw = active ? yg : 0, zgw = active ? zg : 0;
    const int oyp = (ygw == 0) ? (d.ny - 1)*d.nz : -d.nz;
    const int oym = (ygw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
    const int ozp = (zgw == 0) ? d.nz - 1 : -1;
    const int ozm = (zgw == d.nz - 1) ? -(d.nz - 1) : 1;
    const int syz = ygw*d.nz + zgw;

    /* P_ax of x0 - 1 at this column; planes x0 and x0 + 1 in the ring */
    float prevP[3];
    {
      const long long sm1 = (long long) lgb_wrap_far(x0 - 1, d.nx)*NP + syz;
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) prevP[ia] = pth[(3*ia)*N + sm1];
    }
    __syncthreads();                 /* ring free (previous item done) */
    load_P(x0);
    load_P(x0 + 1);
    __pipeline_commit();

    for (int x = x0; x < xe; x++) {
      const long long s0 = (long long) x*NP + syz;
      const int oxp = (x == 0) ? (d.nx - 1)*NP : -NP;
      const int oxm = (x == d.nx - 1) ? -(d.nx - 1)*NP : NP;

      float fs[LGB_NVEL];
      if (active) {
	const S * fb = f_in + s0;
	Unroll<LGB_NVEL>::run([&](auto P) {
	  constexpr int pp = decltype(P)::value;
	  int off = 0;
	  if (Cv<pp>::X == +1) off += oxp;
	  if (Cv<pp>::X == -1) off += oxm;
	  if (Cv<pp>::Y == +1) off += oyp;
	  if (Cv<pp>::Y == -1) off += oym;
	  if (Cv<pp>::Z == +1) off += ozp;
	  if (Cv<pp>::Z == -1) off += ozm;
	  fs[pp] = FStore<S, float>::ld(fb + pp*N + off, rfscale);
	});
      }

      /* planes x and x + 1 have landed; the slot of x - 1 is free */
      __pipeline_wait_prior(0);
      __syncthreads();
      if (x + 2 < xe + 1) load_P(x + 2);
      __pipeline_commit();

      if (active) {
	const float * Pc = slot(x);
	const float * Pn = slot(x + 1);
	float force[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  const float * Px = Pc + (3*ia + 0)*ND;
	  const float * Py = Pc + (3*ia + 1)*ND;
	  const float * Pz = Pc + (3*ia + 2)*ND;
	  const float pxc = Px[cidx];
	  /* minus the divergence of the face values 0.5 (P(s) + P(s + e));
	   * the own-site halves cancel */
	  force[ia] = 0.5f*((prevP[ia] - Pn[(3*ia)*ND + cidx])
			    + (Py[cidx - DZ] - Py[cidx + DZ])
			    + (Pz[cidx - 1] - Pz[cidx + 1]));
	  prevP[ia] = pxc;
	}
	const bool fluid = !HAS_MAP || st[s0] == 0;
	float ftot[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  ftot[ia] = a.fp[LGBK_LCF_FX + ia] + force[ia];
	}
	float rho, uu[3];
	if (fluid) {
	  lgb_collide_site<float, false, true, true>(
	    a.fp[LGBK_LCF_RTAU_SHEAR], a.fp[LGBK_LCF_RTAU_BULK],
	    a.cp.rtau_ghost, rho0, fs, ftot, rho, uu);
	  rho_out[s0] = rho;
	}
	else {
	  uu[0] = uu[1] = uu[2] = 0.0f;
	}
	S * ob = f_out + s0;
	#pragma unroll
	for (int pp = 0; pp < LGB_NVEL; pp++) {
	  FStore<S, float>::st(ob + pp*N, fs[pp], fscale);
	}
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) u_out[ia*N + s0] = uu[ia];
      }
    }
    __pipeline_wait_prior(0);
  }
}

#endif
