/*****************************************************************************
 *
 *  lgb_fused.cuh
 *
 *  One kernel per time step of the symmetric binary fluid: the whole of
 *  src/ludwig.c:528-860 for this model (7-point gradient, stress, stress
 *  divergence force, upwind advection + chemical-potential fluxes,
 *  forward-Euler phi update, M10 collision with the force, streaming).
 *
 *  Data flow (per site, per step):
 *    reads  f (19, pulled from the neighbours: streaming is fused into the
 *           load), phi (1), u from the previous collision (3)
 *    writes f (19, post-collision), phi (1), u (3), rho (1)
 *  No gradient, stress, force or flux array is stored: they live in
 *  registers and in shared memory.
 *
 *  Stored-state convention: the f array holds post-collision populations;
 *  the reference's f at the start of a step is its streamed image.
 *
 *  Blocking: a CTA owns a TY x 32 (y, z) tile and marches along x over a
 *  chunk of planes.  Shared memory holds rolling planes:
 *    phi   : 3 planes (x, x+1, x+2), tile + 2 halo
 *    D     : 2 planes (x, x+1), tile + 1 halo: P_ab (9) and mu
 *    u     : plane x, tile + 1 halo
 *  The x-1 values each thread needs (P_ax, mu, phi, u_x at its own column)
 *  are carried in registers from the previous plane.
 *
 *  Work items (tile, x-chunk) are distributed over a grid sized to the
 *  number of resident CTAs (persistent-style loop), z tiles fastest.
 *
 *****************************************************************************/

#ifndef LGB_FUSED_CUH
#define LGB_FUSED_CUH

#include "lgb_common.cuh"
#include <cuda_pipeline.h>

/* Storage of distributions */

template <typename S, typename T> struct FStore {
  static __device__ __forceinline__ T ld(const S * p, T) { return (T) *p; }
  static __device__ __forceinline__ void st(S * p, T v, T) { *p = (S) v; }
};

template <typename T> struct FStore<__half, T> {
  static __device__ __forceinline__ T ld(const __half * p, T rscale) {
    return (T) __half2float(*p)*rscale;
  }
  static __device__ __forceinline__ void st(__half * p, T v, T scale) {
    *p = __float2half_rn((float) (v*scale));
  }
};

__device__ __forceinline__ int lgb_mod(int i, int n) {
  int r = i % n;
  return (r < 0) ? r + n : r;
}

/* Typed access to the parameter block */
template <typename T> struct KP;
template <> struct KP<float> {
  static __device__ __forceinline__ float get(const lgbk_binary_args_t & a,
					      int i) { return a.pf[i]; }
};
template <> struct KP<double> {
  static __device__ __forceinline__ double get(const lgbk_binary_args_t & a,
					       int i) { return a.pd[i]; }
};

template <typename T, int TY>
struct FusedSmem {
  static constexpr int TZ = 32;
  static constexpr int PY = TY + 4, PZ = TZ + 4;     /* phi plane */
  static constexpr int DY = TY + 2, DZ = TZ + 2;     /* D and u planes */
  static constexpr int NPHI = PY*PZ;
  static constexpr int ND = DY*DZ;
  static constexpr int NDC = 10;                     /* P (9) + mu */
  static constexpr size_t bytes() {
    return sizeof(T)*(4*NPHI + 2*NDC*ND + 2*3*ND);
  }
};

/* Planes per work item when none is asked for (xchunk <= 0): long runs
 * amortise each item's prologue (the halo planes before the first site),
 * but there must be work items enough for about `items` per resident CTA
 * (in halves: 4 = two items): ncx = ceil(items grid / tiles) chunks, of 8
 * to 64 planes.  Measured at 256^3 (256 tiles, 456 CTAs, two items): 16
 * planes 27.6, 32 planes 28.2, 64 planes 28.4 G site updates/s. */
static inline int lgbk_auto_xchunk(int xchunk, int nx, int tiles,
				   long long grid, int half_items = 4) {
  if (xchunk > 0) return xchunk;
  long long ncx = (half_items*grid + 2*tiles - 1)/(2*tiles);
  if (ncx < 1) ncx = 1;
  int c = (int) ((nx + ncx - 1)/ncx);
  if (c > 64) c = 64;
  if (c < 8) c = 8;
  return c;
}

/* Wrap a coordinate that may lie up to one tile outside [0, n) */
__device__ __forceinline__ int lgb_wrap_far(int i, int n) {
  if (i < 0) i += n;
  while (i >= n) i -= n;
  return i;
}

/* One work item: the TY x 32 tile (ity, itz) of box d, planes
 * [x0, xe).  Called by every thread of the CTA;
 * smem_raw holds FusedSmem<T, TY>::bytes(). */
template <typename T, typename S, bool SEQ, bool SHIFT, bool GZERO,
	  bool HAS_MAP, int TY>
__device__ __forceinline__ void
binary_item(const lgbk_dims_t & d, const lgbk_binary_args_t & a, int itz,
	    int ity, int x0, int xe, unsigned char * smem_raw) {

  using SM = FusedSmem<T, TY>;
  constexpr int TZ = SM::TZ;
  constexpr int PZ = SM::PZ, DZ = SM::DZ;
  constexpr int NPHI = SM::NPHI, ND = SM::ND;
  constexpr int NTHR = TY*TZ;
  constexpr int KPHI = (NPHI + NTHR - 1)/NTHR;      /* phi halo loads/thread */
  constexpr int KD = (ND + NTHR - 1)/NTHR;          /* D sites / u loads */

  T * sphi = reinterpret_cast<T *>(smem_raw);          /* [4][NPHI] */
  T * sD = sphi + 4*NPHI;                              /* [2][10][ND] */
  T * su0 = sD + 2*SM::NDC*ND;                         /* [2][3][ND] */

  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty*TZ + tz;
  const long long N = d.nsites;
  const int NP = d.ny*d.nz;                            /* sites per x plane */

  const T * __restrict__ phi_in = (const T *) a.phi_in;
  T * __restrict__ phi_out = (T *) a.phi_out;
  const T * __restrict__ u_in = (const T *) a.u_in;
  T * __restrict__ u_out = (T *) a.u_out;
  T * __restrict__ rho_out = (T *) a.rho_out;
  T * __restrict__ force_out = (T *) a.force_out;
  const S * __restrict__ f_in = (const S *) a.f_in;
  S * __restrict__ f_out = (S *) a.f_out;
  const uint8_t * __restrict__ st = a.status;

  const T mobility = KP<T>::get(a, LGBK_P_MOBILITY);
  const T rho0 = KP<T>::get(a, LGBK_P_RHO0);
  const T fscale = KP<T>::get(a, LGBK_P_FSCALE);
  const T rfscale = KP<T>::get(a, LGBK_P_RFSCALE);
  const T pa = KP<T>::get(a, LGBK_P_A);
  const T pb = KP<T>::get(a, LGBK_P_B);
  const T kappa = KP<T>::get(a, LGBK_P_KAPPA);
  /* Reduced-precision forms (float): free of the reference's operation
   * order, so cancelling terms and additions of zero are left out */
  constexpr bool RED = (sizeof(T) == 4);

  const int cidx = (ty + 1)*DZ + (tz + 1);       /* own site in D/u */
  const int pidx = (ty + 2)*PZ + (tz + 2);       /* own site in phi */

  {
    const int z0 = itz*TZ, y0 = ity*TY;

    /* In-plane offsets (wrapped) of the halo elements this thread loads;
     * fixed for the whole item, so no index arithmetic per plane. */
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

    /* Ring slots (x >= x0 - 2): phi 4 planes, D 2 planes, u 2 planes.
     * Halo planes are copied asynchronously one plane ahead (cp.async):
     * phi(x+3) and u(x+1) stream in while plane x is processed. */
    auto pslot = [&](int x) { return (x - x0 + 4) & 3; };
    auto dslot = [&](int x) { return (x - x0 + 2) & 1; };
    auto uslot = [&](int x) { return su0 + ((x - x0 + 2) & 1)*3*ND; };

    auto load_phi = [&](int x) {
      const T * src = phi_in + (long long) lgb_wrap_far(x, d.nx)*NP;
      T * dst = sphi + pslot(x)*NPHI;
      #pragma unroll
      for (int j = 0; j < KPHI; j++) {
	if (phoff[j] >= 0) {
	  __pipeline_memcpy_async(dst + tid + j*NTHR, src + phoff[j],
				  sizeof(T));
	}
      }
    };

    auto load_u = [&](int x) {
      const T * src = u_in + (long long) lgb_wrap_far(x, d.nx)*NP;
      T * dst = uslot(x);
      #pragma unroll
      for (int j = 0; j < KD; j++) {
	if (uoff[j] >= 0) {
	  const int k = tid + j*NTHR;
	  __pipeline_memcpy_async(dst + k, src + uoff[j], sizeof(T));
	  __pipeline_memcpy_async(dst + ND + k, src + N + uoff[j], sizeof(T));
	  __pipeline_memcpy_async(dst + 2*ND + k, src + 2*N + uoff[j],
				  sizeof(T));
	}
      }
    };

    /* Gradient, stress and chemical potential of plane x at the site k of
     * the tile + 1 (halo-1 coordinates + 1: ly = k / DZ, lz = k % DZ) */
    auto d_site = [&](int x, int k) {
      const T * pc = sphi + pslot(x)*NPHI;
      const T * pp = sphi + pslot(x + 1)*NPHI;
      const T * pm = sphi + pslot(x - 1)*NPHI;
      T * D = sD + dslot(x)*SM::NDC*ND;
      const int ly = k / DZ, lz = k % DZ;
      const int q = (ly + 1)*PZ + (lz + 1);    /* same site in phi plane */
      T c = pc[q];
      T xp = pp[q], xm = pm[q];
      T yp = pc[q + PZ], ym = pc[q - PZ];
      T zp = pc[q + 1], zm = pc[q - 1];
      T g[3];
      g[0] = T(0.5)*(xp - xm);
      g[1] = T(0.5)*(yp - ym);
      g[2] = T(0.5)*(zp - zm);
      T delsq = xp + xm + yp + ym + zp + zm - T(6.0)*c;
      T p0 = lgb_symm_p0<T>(pa, pb, kappa, c, delsq, g);
      T p0z = RED ? T(0.0) : p0*T(0.0);
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) {
	#pragma unroll
	for (int ib = 0; ib < 3; ib++) {
	  if (RED && ia != ib) D[(3*ia + ib)*ND + k] = kappa*g[ia]*g[ib];
	  else D[(3*ia + ib)*ND + k] = ((ia == ib) ? p0 : p0z)
		 + kappa*g[ia]*g[ib];
	}
      }
      D[9*ND + k] = lgb_symm_mu<T>(pa, pb, kappa, c, delsq);
    };
    /* The whole tile + 1 of plane x: every thread its own site, the first
     * NB threads one site of the halo ring each.  A thread therefore
     * writes D at its own site itself, and may read it back without a
     * barrier. */
    constexpr int NB = ND - NTHR;                 /* 2 DZ + 2 TY ring sites */
    int hring = -1;
    if (tid < NB) {
      if (tid < DZ) hring = tid;                            /* row 0 */
      else if (tid < 2*DZ) hring = (TY + 1)*DZ + (tid - DZ); /* last row */
      else if (tid < 2*DZ + TY) hring = (1 + tid - 2*DZ)*DZ;  /* column 0 */
      else hring = (1 + tid - 2*DZ - TY)*DZ + DZ - 1;          /* last col */
    }
    auto compute_D = [&](int x) {
      d_site(x, cidx);
      if (hring >= 0) d_site(x, hring);
    };

    const int yg = y0 + ty, zg = z0 + tz;
    const bool active = (yg < d.ny) && (zg < d.nz);
    const int ygw = active ? yg : 0, zgw = active ? zg : 0;

    /* Wrapped offsets of the pull sources in y and z (fixed per item):
     * a population with c_y = +1 comes from y - 1, etc. */
    const int oyp = (ygw == 0) ? (d.ny - 1)*d.nz : -d.nz;
    const int oym = (ygw == d.ny - 1) ? -(d.ny - 1)*d.nz : d.nz;
    const int ozp = (zgw == 0) ? d.nz - 1 : -1;
    const int ozm = (zgw == d.nz - 1) ? -(d.nz - 1) : 1;
    const int syz = ygw*d.nz + zgw;

    /* ---- prologue: D(x0-1), D(x0) and the x0-1 column registers ---- */

    load_phi(x0 - 2);
    load_phi(x0 - 1);
    load_phi(x0);
    load_phi(x0 + 1);
    __pipeline_commit();
    __pipeline_wait_prior(0);
    __syncthreads();
    compute_D(x0 - 1);
    __syncthreads();

    T prevP[3], prev_mu, prev_phi, prev_ux, prev_fe = T(0.0);
    {
      const T * D = sD + dslot(x0 - 1)*SM::NDC*ND;
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) prevP[ia] = D[(3*ia)*ND + cidx];
      prev_mu = D[9*ND + cidx];
      prev_phi = sphi[pslot(x0 - 1)*NPHI + pidx];
      prev_ux = u_in[(long long) lgb_wrap_far(x0 - 1, d.nx)*NP + syz];
    }
    compute_D(x0);
    load_phi(x0 + 2);
    load_u(x0);
    __pipeline_commit();

    /* ---- march along x ---- */

    for (int x = x0; x < xe; x++) {

      /* site index: 32-bit unsigned (the host refuses lattices of 2^32
       * sites or more), pointers formed from per-component bases */
      const unsigned s0 = (unsigned) x*NP + syz;
      /* x offsets of the pull sources, modulo 2^32 */
      const unsigned oxp = (x == 0) ? (unsigned) (d.nx - 1)*NP : 0u - NP;
      const unsigned oxm = (x == d.nx - 1) ? 0u - (unsigned) (d.nx - 1)*NP
	: (unsigned) NP;

      /* Pulled populations f_p(x - c_p): issued first, consumed after the
       * stencil phase, so their latency overlaps it. */
      T fs[LGB_NVEL];
      if (active) {
	Unroll<LGB_NVEL>::run([&](auto P) {
	  constexpr int p = decltype(P)::value;
	  unsigned off = 0;
	  if (Cv<p>::X == +1) off += oxp;
	  if (Cv<p>::X == -1) off += oxm;
	  if (Cv<p>::Y == +1) off += oyp;
	  if (Cv<p>::Y == -1) off += oym;
	  if (Cv<p>::Z == +1) off += ozp;
	  if (Cv<p>::Z == -1) off += ozm;
	  const S * fp = f_in + p*N;
	  fs[p] = FStore<S, T>::ld(fp + (s0 + off), rfscale);
	});
      }

      /* phi(x+2) and u(x) have landed; stream phi(x+3) and u(x+1) into
       * the slots of phi(x-1) and u(x-1), free since the last barrier */
      __pipeline_wait_prior(0);
      __syncthreads();
      if (x + 1 < xe) {
	load_phi(x + 3);
	load_u(x + 1);
      }
      __pipeline_commit();
      /* D(x+1): each thread's own site is its own work (read back below
       * without a barrier); the neighbours' values of D(x+1) are read only
       * in the next plane, after its barrier */
      compute_D(x + 1);

      if (active) {
	const T * Dc = sD + dslot(x)*SM::NDC*ND;
	const T * Dn = sD + dslot(x + 1)*SM::NDC*ND;
	const T * pc = sphi + pslot(x)*NPHI;
	const T * pn = sphi + pslot(x + 1)*NPHI;
	const T * su = uslot(x);

	/* Force: src/phi_force_colloid.c:352-455 */
	T force[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  const T * Px = Dc + (3*ia + 0)*ND;
	  const T * Py = Dc + (3*ia + 1)*ND;
	  const T * Pz = Dc + (3*ia + 2)*ND;
	  T pxc = Px[cidx];
	  T fa;
	  if (RED) {
	    /* the face values' own-site halves cancel */
	    fa = T(0.5)*((prevP[ia] - Dn[(3*ia)*ND + cidx])
			 + (Py[cidx - DZ] - Py[cidx + DZ])
			 + (Pz[cidx - 1] - Pz[cidx + 1]));
	  }
	  else {
	    fa  = -T(0.5)*(Dn[(3*ia)*ND + cidx] + pxc);
	    fa +=  T(0.5)*(prevP[ia] + pxc);
	    fa -=  T(0.5)*(Py[cidx + DZ] + Py[cidx]);
	    fa +=  T(0.5)*(Py[cidx - DZ] + Py[cidx]);
	    fa -=  T(0.5)*(Pz[cidx + 1] + Pz[cidx]);
	    fa +=  T(0.5)*(Pz[cidx - 1] + Pz[cidx]);
	  }
	  force[ia] = fa;
	  prevP[ia] = pxc;
	}

	/* Cahn-Hilliard fluxes: src/advection.c:538-629,
	 * src/phi_cahn_hilliard.c:350-404, src/advection_bcs.c:80-140 */
	const T phic = pc[pidx];
	const T muc = Dc[9*ND + cidx];
	const T uxc = su[cidx], uyc = su[ND + cidx], uzc = su[2*ND + cidx];
	T fw, fe, fy, fym, fz, fzm;
	if (RED && x > x0) {
	  fw = prev_fe;      /* the x-1 site's east face is this west face */
	}
	else {
	  T uf = T(0.5)*(uxc + prev_ux);
	  fw = uf*((uf > T(0.0)) ? prev_phi : phic);
	  fw -= mobility*(muc - prev_mu);
	}
	{
	  const T uxp = u_in[s0 + oxm];
	  const T phip = pn[pidx];
	  const T mup = Dn[9*ND + cidx];
	  T uf = T(0.5)*(uxc + uxp);
	  fe = uf*((uf < T(0.0)) ? phip : phic);
	  fe -= mobility*(mup - muc);
	}
	{
	  T uf = T(0.5)*(uyc + su[ND + cidx + DZ]);
	  fy = uf*((uf < T(0.0)) ? pc[pidx + PZ] : phic);
	  fy -= mobility*(Dc[9*ND + cidx + DZ] - muc);
	}
	{
	  T uf = T(0.5)*(su[ND + cidx - DZ] + uyc);
	  fym = uf*((uf < T(0.0)) ? phic : pc[pidx - PZ]);
	  fym -= mobility*(muc - Dc[9*ND + cidx - DZ]);
	}
	{
	  T uf = T(0.5)*(uzc + su[2*ND + cidx + 1]);
	  fz = uf*((uf < T(0.0)) ? pc[pidx + 1] : phic);
	  fz -= mobility*(Dc[9*ND + cidx + 1] - muc);
	}
	{
	  T uf = T(0.5)*(su[2*ND + cidx - 1] + uzc);
	  fzm = uf*((uf < T(0.0)) ? phic : pc[pidx - 1]);
	  fzm -= mobility*(muc - Dc[9*ND + cidx - 1]);
	}

	bool fluid = true;
	if (HAS_MAP) {
	  /* pull offsets double as neighbour offsets: x-1 is s0 + oxp, etc. */
	  const T m0 = (T) (st[s0] == 0);
	  const T mym = (T) (st[s0 + oyp] == 0), mzm = (T) (st[s0 + ozp] == 0);
	  fw  *= m0*((T) (st[s0 + oxp] == 0));
	  fe  *= m0*((T) (st[s0 + oxm] == 0));
	  fy  *= m0*((T) (st[s0 + oym] == 0));
	  fz  *= m0*((T) (st[s0 + ozm] == 0));
	  fym *= mym*m0;
	  fzm *= mzm*m0;
	  fluid = (st[s0] == 0);
	}

	/* src/phi_cahn_hilliard.c:1040-1045 with wz = 1 */
	phi_out[s0] = phic - (+ fe - fw + fy - fym + fz - fzm);
	prev_fe = fe;

	prev_ux = uxc;
	prev_mu = muc;
	prev_phi = phic;

	/* Collision: force = global + (hydro force zeroed, then added) */
	T ftot[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  if (RED) ftot[ia] = KP<T>::get(a, LGBK_P_FX + ia) + force[ia];
	  else     ftot[ia] = KP<T>::get(a, LGBK_P_FX + ia)
		     + (T(0.0) + force[ia]*T(1.0));
	}
	if (force_out) {
	  #pragma unroll
	  for (int ia = 0; ia < 3; ia++) (force_out + ia*N)[s0] = force[ia];
	}

	T rho, uu[3];
	if (fluid) {
	  lgb_collide_site<T, SEQ, SHIFT, GZERO>(
	    KP<T>::get(a, LGBK_P_RTAU_SHEAR), KP<T>::get(a, LGBK_P_RTAU_BULK),
	    a.cp.rtau_ghost, rho0, fs, ftot, rho, uu);
	  rho_out[s0] = rho;
	}
	else {
	  uu[0] = uu[1] = uu[2] = T(0.0);
	}
	#pragma unroll
	for (int p = 0; p < LGB_NVEL; p++) {
	  FStore<S, T>::st(f_out + p*N + s0, fs[p], fscale);
	}
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) (u_out + ia*N)[s0] = uu[ia];
      }
    }
    __pipeline_wait_prior(0);
    __syncthreads();
  }
}

template <typename T, typename S, bool SEQ, bool SHIFT, bool GZERO,
	  bool HAS_MAP, int TY, int MINB>
__global__ void __launch_bounds__(32*TY, MINB)
k_binary_fused(lgbk_dims_t d, lgbk_binary_args_t a, int xchunk) {
  extern __shared__ unsigned char smem_raw[];
  const int ntz = (d.nz + 31)/32;
  const int nty = (d.ny + TY - 1)/TY;
  /* chunks of xchunk planes of a tile, dealt round the grid with the z
   * tiles fastest, so that CTAs with neighbouring indices stream
   * neighbouring rows of the same planes (DRAM page locality) */
  const int ncx = (d.nx + xchunk - 1)/xchunk;
  const int nitems = ntz*nty*ncx;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int itz = item % ntz;
    const int ity = (item / ntz) % nty;
    const int x0 = (item / (ntz*nty))*xchunk;
    binary_item<T, S, SEQ, SHIFT, GZERO, HAS_MAP, TY>(
      d, a, itz, ity, x0, min(x0 + xchunk, d.nx), smem_raw);
  }
}

/* Work items of the ensemble kernels are taken from a counter (sched[0])
 * in list order, the host having sorted the list longest first, so that
 * the short items of small boxes fill in behind the long ones.  After its
 * last fetch each CTA counts itself out (sched[1]); the last one resets
 * both counters for the next launch, which the stream orders after this
 * one. */
__device__ __forceinline__ int2 lgbk_sched_next(int * sched,
						const int2 * items,
						int nitems) {
  const int k = atomicAdd(sched, 1);
  return (k < nitems) ? items[k] : make_int2(-1, 0);
}

__device__ __forceinline__ void lgbk_sched_retire(int * sched) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    if (atomicAdd(sched + 1, 1) == (int) gridDim.x - 1) {
      __threadfence();
      atomicExch(sched, 0);
      atomicExch(sched + 1, 0);
    }
  }
}

/* Ensemble of independent boxes: box descriptors and a flat list of
 * (box, local item) pairs; one launch covers every box.  Boxes marked
 * inactive (quarantined) are skipped. */
template <typename T, typename S, bool SEQ, bool SHIFT, bool GZERO,
	  bool HAS_MAP, int TY, int MINB>
__global__ void __launch_bounds__(32*TY, MINB)
k_binary_ensemble(const lgbk_box_t * __restrict__ boxes,
		  const int2 * __restrict__ items, int nitems, int xchunk,
		  int * __restrict__ sched) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ lgbk_box_t sb;
  __shared__ int2 sit;
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
    binary_item<T, S, SEQ, SHIFT, GZERO, HAS_MAP, TY>(
      sb.d, sb.a, itz, ity, x0, min(x0 + xchunk, sb.d.nx), smem_raw);
  }
  lgbk_sched_retire(sched);
}

#endif
