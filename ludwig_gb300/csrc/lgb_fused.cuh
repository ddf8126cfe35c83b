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
 *  number of resident CTAs (persistent-style loop).
 *
 *****************************************************************************/

#ifndef LGB_FUSED_CUH
#define LGB_FUSED_CUH

#include "lgb_common.cuh"

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

template <typename T, int TY>
struct FusedSmem {
  static constexpr int TZ = 32;
  static constexpr int PY = TY + 4, PZ = TZ + 4;     /* phi plane */
  static constexpr int DY = TY + 2, DZ = TZ + 2;     /* D and u planes */
  static constexpr int NPHI = PY*PZ;
  static constexpr int ND = DY*DZ;
  static constexpr int NDC = 10;                     /* P (9) + mu */
  static constexpr size_t bytes() {
    return sizeof(T)*(3*NPHI + 2*NDC*ND + 3*ND);
  }
};

template <typename T, typename S, bool SEQ, bool SHIFT, bool GZERO,
	  bool HAS_MAP, int TY, int MINB>
__global__ void __launch_bounds__(32*TY, MINB)
k_binary_fused(lgbk_dims_t d, lgbk_binary_args_t a, int xchunk) {

  using SM = FusedSmem<T, TY>;
  constexpr int TZ = SM::TZ;
  constexpr int PZ = SM::PZ, DZ = SM::DZ;
  constexpr int NPHI = SM::NPHI, ND = SM::ND;

  extern __shared__ unsigned char smem_raw[];
  T * sphi = reinterpret_cast<T *>(smem_raw);          /* [3][NPHI] */
  T * sD = sphi + 3*NPHI;                              /* [2][10][ND] */
  T * su = sD + 2*SM::NDC*ND;                          /* [3][ND] */

  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty*TZ + tz;
  const int nthr = TY*TZ;
  const long long N = d.nsites;
  const long long NP = (long long) d.ny*d.nz;          /* sites per x plane */

  const int ntz = (d.nz + TZ - 1)/TZ;
  const int nty = (d.ny + TY - 1)/TY;
  const int ncx = (d.nx + xchunk - 1)/xchunk;
  const int nitems = ntz*nty*ncx;

  const T * __restrict__ phi_in = (const T *) a.phi_in;
  T * __restrict__ phi_out = (T *) a.phi_out;
  const T * __restrict__ u_in = (const T *) a.u_in;
  T * __restrict__ u_out = (T *) a.u_out;
  T * __restrict__ rho_out = (T *) a.rho_out;
  T * __restrict__ force_out = (T *) a.force_out;
  const S * __restrict__ f_in = (const S *) a.f_in;
  S * __restrict__ f_out = (S *) a.f_out;
  const uint8_t * __restrict__ st = a.status;

  const T mobility = (T) a.mobility;
  const T rho0 = (T) a.rho0;
  const T fscale = (T) a.fscale;
  const T rfscale = T(1.0)/fscale;
  const T kappa = (T) a.fe.kappa;

  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {

    const int itz = item % ntz;
    const int ity = (item / ntz) % nty;
    const int icx = item / (ntz*nty);
    const int z0 = itz*TZ, y0 = ity*TY, x0 = icx*xchunk;
    const int xe = min(x0 + xchunk, d.nx);

    /* Ring slot of plane x: phi ring of 3, D ring of 2 (x >= x0 - 2) */
    auto pslot = [&](int x) { return (x - x0 + 3) % 3; };
    auto dslot = [&](int x) { return (x - x0 + 2) & 1; };

    auto load_phi = [&](int x) {
      const int xw = lgb_mod(x, d.nx);
      T * dst = sphi + pslot(x)*NPHI;
      for (int k = tid; k < NPHI; k += nthr) {
	int ly = k / PZ - 2, lz = k % PZ - 2;
	int yw = lgb_mod(y0 + ly, d.ny), zw = lgb_mod(z0 + lz, d.nz);
	dst[k] = phi_in[(long long) xw*NP + (long long) yw*d.nz + zw];
      }
    };

    auto load_u = [&](int x) {
      const int xw = lgb_mod(x, d.nx);
      for (int k = tid; k < ND; k += nthr) {
	int ly = k / DZ - 1, lz = k % DZ - 1;
	int yw = lgb_mod(y0 + ly, d.ny), zw = lgb_mod(z0 + lz, d.nz);
	long long s = (long long) xw*NP + (long long) yw*d.nz + zw;
	su[k]        = u_in[s];
	su[ND + k]   = u_in[N + s];
	su[2*ND + k] = u_in[2*N + s];
      }
    };

    /* Gradient, stress and chemical potential of plane x on tile + 1 */
    auto compute_D = [&](int x) {
      const T * pc = sphi + pslot(x)*NPHI;
      const T * pp = sphi + pslot(x + 1)*NPHI;
      const T * pm = sphi + pslot(x - 1)*NPHI;
      T * D = sD + dslot(x)*SM::NDC*ND;
      for (int k = tid; k < ND; k += nthr) {
	int ly = k / DZ, lz = k % DZ;          /* halo-1 coordinates + 1 */
	int q = (ly + 1)*PZ + (lz + 1);        /* same site in phi plane */
	T c = pc[q];
	T xp = pp[q], xm = pm[q];
	T yp = pc[q + PZ], ym = pc[q - PZ];
	T zp = pc[q + 1], zm = pc[q - 1];
	T g[3];
	g[0] = T(0.5)*(xp - xm);
	g[1] = T(0.5)*(yp - ym);
	g[2] = T(0.5)*(zp - zm);
	T delsq = xp + xm + yp + ym + zp + zm - T(6.0)*c;
	T p0 = lgb_symm_p0<T>(a.fe, c, delsq, g);
	T p0z = p0*T(0.0);
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  #pragma unroll
	  for (int ib = 0; ib < 3; ib++) {
	    D[(3*ia + ib)*ND + k] = ((ia == ib) ? p0 : p0z) + kappa*g[ia]*g[ib];
	  }
	}
	D[9*ND + k] = lgb_symm_mu<T>(a.fe, c, delsq);
      }
    };

    /* ---- prologue: D(x0-1), D(x0) and the x0-1 column registers ---- */

    load_phi(x0 - 2);
    load_phi(x0 - 1);
    load_phi(x0);
    __syncthreads();
    compute_D(x0 - 1);
    __syncthreads();

    const int cidx = (ty + 1)*DZ + (tz + 1);       /* own site in D/u */
    const int pidx = (ty + 2)*PZ + (tz + 2);       /* own site in phi */
    const int yg = y0 + ty, zg = z0 + tz;
    const bool active = (yg < d.ny) && (zg < d.nz);
    const int ygw = active ? yg : 0, zgw = active ? zg : 0;

    T prevP[3], prev_mu, prev_phi, prev_ux;
    {
      const T * D = sD + dslot(x0 - 1)*SM::NDC*ND;
      #pragma unroll
      for (int ia = 0; ia < 3; ia++) prevP[ia] = D[(3*ia)*ND + cidx];
      prev_mu = D[9*ND + cidx];
      prev_phi = sphi[pslot(x0 - 1)*NPHI + pidx];
      prev_ux = u_in[(long long) lgb_mod(x0 - 1, d.nx)*NP
		     + (long long) ygw*d.nz + zgw];
    }
    __syncthreads();
    load_phi(x0 + 1);
    __syncthreads();
    compute_D(x0);
    __syncthreads();

    /* ---- march along x ---- */

    for (int x = x0; x < xe; x++) {

      load_phi(x + 2);
      load_u(x);
      __syncthreads();
      compute_D(x + 1);
      __syncthreads();

      if (active) {
	const long long s0 = (long long) x*NP + (long long) yg*d.nz + zg;

	/* Pulled populations f_p(x - c_p): issue the loads first */
	T fs[LGB_NVEL];
	Unroll<LGB_NVEL>::run([&](auto P) {
	  constexpr int p = decltype(P)::value;
	  int xs = x - Cv<p>::X, ys = yg - Cv<p>::Y, zs = zg - Cv<p>::Z;
	  if (Cv<p>::X != 0) xs = lgb_wrap(xs, d.nx);
	  if (Cv<p>::Y != 0) ys = lgb_wrap(ys, d.ny);
	  if (Cv<p>::Z != 0) zs = lgb_wrap(zs, d.nz);
	  long long j = (long long) xs*NP + (long long) ys*d.nz + zs;
	  fs[p] = FStore<S, T>::ld(f_in + p*N + j, rfscale);
	});

	const T * Dc = sD + dslot(x)*SM::NDC*ND;
	const T * Dn = sD + dslot(x + 1)*SM::NDC*ND;
	const T * pc = sphi + pslot(x)*NPHI;
	const T * pn = sphi + pslot(x + 1)*NPHI;

	/* Force: src/phi_force_colloid.c:352-455 */
	T force[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  const T * Px = Dc + (3*ia + 0)*ND;
	  const T * Py = Dc + (3*ia + 1)*ND;
	  const T * Pz = Dc + (3*ia + 2)*ND;
	  T pxc = Px[cidx];
	  T fa;
	  fa  = -T(0.5)*(Dn[(3*ia)*ND + cidx] + pxc);
	  fa +=  T(0.5)*(prevP[ia] + pxc);
	  fa -=  T(0.5)*(Py[cidx + DZ] + Py[cidx]);
	  fa +=  T(0.5)*(Py[cidx - DZ] + Py[cidx]);
	  fa -=  T(0.5)*(Pz[cidx + 1] + Pz[cidx]);
	  fa +=  T(0.5)*(Pz[cidx - 1] + Pz[cidx]);
	  force[ia] = fa;
	  prevP[ia] = pxc;
	}

	/* Cahn-Hilliard fluxes: src/advection.c:538-629,
	 * src/phi_cahn_hilliard.c:350-404, src/advection_bcs.c:80-140 */
	const T phic = pc[pidx];
	const T muc = Dc[9*ND + cidx];
	const T uxc = su[cidx], uyc = su[ND + cidx], uzc = su[2*ND + cidx];
	T fw, fe, fy, fym, fz, fzm;
	{
	  T uf = T(0.5)*(uxc + prev_ux);
	  fw = uf*((uf > T(0.0)) ? prev_phi : phic);
	  fw -= mobility*(muc - prev_mu);
	}
	{
	  const T uxp = u_in[(long long) lgb_wrap(x + 1, d.nx)*NP
			     + (long long) yg*d.nz + zg];
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
	  auto fl = [&](int xx, int yy, int zz) -> T {
	    long long j = (long long) lgb_wrap(xx, d.nx)*NP
	      + (long long) lgb_wrap(yy, d.ny)*d.nz + lgb_wrap(zz, d.nz);
	    return (T) (st[j] == 0);
	  };
	  T m0 = fl(x, yg, zg);
	  T mym = fl(x, yg - 1, zg), mzm = fl(x, yg, zg - 1);
	  fw  *= m0*fl(x - 1, yg, zg);
	  fe  *= m0*fl(x + 1, yg, zg);
	  fy  *= m0*fl(x, yg + 1, zg);
	  fz  *= m0*fl(x, yg, zg + 1);
	  fym *= mym*m0;
	  fzm *= mzm*m0;
	  fluid = (st[s0] == 0);
	}

	/* src/phi_cahn_hilliard.c:1040-1045 with wz = 1 */
	phi_out[s0] = phic - (+ fe - fw + fy - fym + fz - fzm);

	prev_ux = uxc;
	prev_mu = muc;
	prev_phi = phic;

	/* Collision: force = global + (hydro force zeroed, then added) */
	T ftot[3];
	#pragma unroll
	for (int ia = 0; ia < 3; ia++) {
	  ftot[ia] = ((T) a.cp.force_global[ia]) + (T(0.0) + force[ia]*T(1.0));
	}
	if (force_out) {
	  #pragma unroll
	  for (int ia = 0; ia < 3; ia++) force_out[ia*N + s0] = force[ia];
	}

	T rho, uu[3];
	if (fluid) {
	  lgb_collide_site<T, SEQ, SHIFT, GZERO>(a.cp, rho0, fs, ftot, rho, uu);
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
	for (int ia = 0; ia < 3; ia++) u_out[ia*N + s0] = uu[ia];
      }
      __syncthreads();
    }
    __syncthreads();
  }
}

#endif
