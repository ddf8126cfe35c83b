/*****************************************************************************
 *
 *  lgb_fused64.cu
 *
 *  FP64 instantiation of the fused binary-fluid step (compiled with
 *  --fmad=false; reference operation order; bit-exact).
 *
 *****************************************************************************/

#include "lgb_fused.cuh"

template <bool GZERO, bool HAS_MAP>
static int launch64(const lgbk_dims_t * d, const lgbk_binary_args_t * a,
		    int xchunk, int ty, cudaStream_t stream) {
  constexpr int TY = 8;
  (void) ty;
  auto kern = k_binary_fused<double, double, true, false, GZERO, HAS_MAP,
			     TY, 2>;
  size_t smem = FusedSmem<double, TY>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;

  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TY, smem);
  if (occ < 1) occ = 1;

  int ntz = (d->nz + 31)/32, nty = (d->ny + TY - 1)/TY;
  long long grid = (long long) nsm*occ;
  xchunk = lgbk_auto_xchunk(xchunk, d->nx, ntz*nty, grid);
  long long items = (long long) ntz*nty*((d->nx + xchunk - 1)/xchunk);
  if (grid > items) grid = items;

  kern<<<(unsigned int) grid, dim3(32, TY), smem, stream>>>(*d, *a, xchunk);
  return (int) cudaGetLastError();
}

extern "C" int lgbk_binary_step_f64(const lgbk_dims_t * d,
				    const lgbk_binary_args_t * a, int xchunk,
				    int ty, void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  if (a->cp.ghosts_zero) {
    return a->status ? launch64<true, true>(d, a, xchunk, ty, s)
                     : launch64<true, false>(d, a, xchunk, ty, s);
  }
  return a->status ? launch64<false, true>(d, a, xchunk, ty, s)
                   : launch64<false, false>(d, a, xchunk, ty, s);
}

/* Ensembles in FP64 (tile 8 x 32, 2 CTAs per SM) */
template <bool HAS_MAP>
static int launch_ens64(const lgbk_box_t * boxes, const void * items,
			int nitems, int xchunk, int * sched,
			cudaStream_t stream) {
  constexpr int TY = 8;
  auto kern = k_binary_ensemble<double, double, true, false, true, HAS_MAP,
				TY, 2>;
  size_t smem = FusedSmem<double, TY>::bytes();
  cudaError_t err = cudaFuncSetAttribute(kern,
    cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (err != cudaSuccess) return (int) err;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32*TY, smem);
  if (occ < 1) occ = 1;
  long long grid = (long long) nsm*occ;
  if (grid > nitems) grid = nitems;
  if (grid < 1) return 0;
  kern<<<(unsigned int) grid, dim3(32, TY), smem, stream>>>(
    boxes, (const int2 *) items, nitems, xchunk, sched);
  return (int) cudaGetLastError();
}

/* Requires every box to relax its ghost modes with rtau = 1 (M10). */
extern "C" int lgbk_ensemble_step_f64(const lgbk_box_t * boxes,
				      const void * items, int nitems,
				      int xchunk, int has_map, int * sched,
				      void * stream) {
  cudaStream_t s = (cudaStream_t) stream;
  return has_map ? launch_ens64<true>(boxes, items, nitems, xchunk, sched, s)
                 : launch_ens64<false>(boxes, items, nitems, xchunk, sched,
				       s);
}
