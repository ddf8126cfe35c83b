/*****************************************************************************
 *
 *  lgb_tc.cuh
 *
 *  Inline-PTX building blocks of the tensor-core kernels (sm_103a):
 *  mbarriers with bounded waits, TMA tile loads, tensor-memory allocation,
 *  tcgen05.mma (kind::f16, BF16 operands, FP32 accumulate), commit and
 *  tcgen05.ld, and the shared-memory matrix descriptors.
 *
 *  Every wait is bounded by a clock budget; a wait that runs out sets the
 *  CTA's abort flag and a global error word and returns false, so that no
 *  kernel here can spin for ever.
 *
 *****************************************************************************/

#ifndef LGB_TC_CUH
#define LGB_TC_CUH

#include <cuda_runtime.h>
#include <stdint.h>

/* About one second at the GB300 SM clock */
#define LGB_TC_WAIT_CYCLES (2000000000LL)

/* Error codes written to the global error word */
#define LGB_TC_ERR_TIMEOUT 1

__device__ __forceinline__ uint32_t tc_smem_u32(const void * p) {
  return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tc_mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
	       :: "r"(bar), "r"(count) : "memory");
}

/* Make barrier initialisation visible to the async proxy (TMA, tcgen05) */
__device__ __forceinline__ void tc_fence_barrier_init(void) {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_mbar_arrive_tx(uint32_t bar,
						  uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
	       :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tc_mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];"
	       :: "r"(bar) : "memory");
}

__device__ __forceinline__ bool tc_mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile("{\n\t.reg .pred p;\n\t"
	       "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	       "selp.b32 %0, 1, 0, p;\n\t}"
	       : "=r"(done) : "r"(bar), "r"(parity) : "memory");
  return done != 0;
}

/* Bounded wait for the phase of the given parity to complete.  Gives up
 * when the CTA's abort flag is raised or the clock budget runs out. */
__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, uint32_t parity,
					     volatile int * abort_flag,
					     int * err) {
  long long t0 = clock64();
  for (uint32_t it = 0;; it++) {
    if (tc_mbar_try(bar, parity)) return true;
    if ((it & 63u) == 63u) {
      if (*abort_flag) return false;
      if (clock64() - t0 > LGB_TC_WAIT_CYCLES) {
	*abort_flag = 1;
	atomicExch(err, LGB_TC_ERR_TIMEOUT);
	return false;
      }
    }
  }
}

/* 2-d TMA tile load into shared memory, completion on an mbarrier.
 * c0 is the innermost (channel) coordinate and is always 0 here. */
__device__ __forceinline__ void tc_tma_load_2d(uint32_t dst, const void * map,
					       uint32_t bar, int c0, int c1) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile"
	       ".mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
	       :: "r"(dst), "l"(map), "r"(bar), "r"(c0), "r"(c1) : "memory");
}

__device__ __forceinline__ void tc_prefetch_map(const void * map) {
  asm volatile("prefetch.tensormap [%0];" :: "l"(map) : "memory");
}

/* Tensor memory: whole-warp allocation of ncols columns (power of 2,
 * >= 32); the base address is written to shared memory at dst. */
__device__ __forceinline__ void tc_tmem_alloc(uint32_t dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32"
	       " [%0], %1;" :: "r"(dst), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;"
	       ::: "memory");
}

__device__ __forceinline__ void tc_tmem_dealloc(uint32_t taddr,
						uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
	       :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before(void) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after(void) {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* D[tmem] (+)= A[smem] * B[smem], one thread issues */
__device__ __forceinline__ void tc_mma_bf16(uint32_t d, uint64_t adesc,
					    uint64_t bdesc, uint32_t idesc,
					    uint32_t accumulate) {
  asm volatile("{\n\t.reg .pred p;\n\t"
	       "setp.ne.b32 p, %4, 0;\n\t"
	       "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
	       :: "r"(d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
	       : "memory");
}

/* The same with each descriptor as two 32-bit words (low: start address
 * and leading byte offset; high: stride byte offset, version, layout), so
 * that a loop can step a descriptor's start address with one integer
 * addition of (byte offset >> 4) to the low word (the address field cannot
 * carry out: shared-memory addresses are below 2^18) */
__device__ __forceinline__ void tc_mma_bf16_w(uint32_t d, uint32_t alo,
					      uint32_t ahi, uint32_t blo,
					      uint32_t bhi, uint32_t idesc,
					      uint32_t accumulate) {
  asm volatile("{\n\t.reg .pred p;\n\t.reg .b64 ad, bd;\n\t"
	       "mov.b64 ad, {%1, %2};\n\t"
	       "mov.b64 bd, {%3, %4};\n\t"
	       "setp.ne.b32 p, %6, 0;\n\t"
	       "tcgen05.mma.cta_group::1.kind::f16 [%0], ad, bd, %5, p;\n\t}"
	       :: "r"(d), "r"(alo), "r"(ahi), "r"(blo), "r"(bhi), "r"(idesc),
		  "r"(accumulate)
	       : "memory");
}

/* Arrive on an mbarrier once every earlier tcgen05 op of this thread has
 * completed (frees the shared-memory operands, publishes the TMEM result) */
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one"
	       ".shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

/* 32 lanes x 32 consecutive 32-bit columns: thread i of the warp gets
 * lane (base lane + i), columns col .. col+31. */
__device__ __forceinline__ void tc_tmem_ld32(uint32_t taddr, uint32_t r[32]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
	       "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
	       "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, "
	       "%26, %27, %28, %29, %30, %31}, [%32];"
	       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
		 "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
		 "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
		 "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
		 "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
		 "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
		 "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
		 "=r"(r[30]), "=r"(r[31])
	       : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* 32 lanes x 16 consecutive 32-bit columns */
__device__ __forceinline__ void tc_tmem_ld16(uint32_t taddr, uint32_t r[16]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
	       "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
	       "%14, %15}, [%16];"
	       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
		 "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
		 "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
		 "=r"(r[14]), "=r"(r[15])
	       : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* The same without the wait: the registers are valid only after
 * tc_tmem_wait_ld16x3 on them */
__device__ __forceinline__ void tc_tmem_ld16_async(uint32_t taddr,
						   uint32_t r[16]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
	       "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
	       "%14, %15}, [%16];"
	       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
		 "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
		 "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
		 "=r"(r[14]), "=r"(r[15])
	       : "r"(taddr) : "memory");
}

/* Wait for the TMEM loads in flight; the registers of three x16 loads are
 * operands, so that no use of them moves above the wait */
__device__ __forceinline__ void tc_tmem_wait_ld16x3(uint32_t a[16],
						    uint32_t b[16],
						    uint32_t c[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
	       : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]),
		 "+r"(a[5]), "+r"(a[6]), "+r"(a[7]), "+r"(a[8]), "+r"(a[9]),
		 "+r"(a[10]), "+r"(a[11]), "+r"(a[12]), "+r"(a[13]),
		 "+r"(a[14]), "+r"(a[15]),
		 "+r"(b[0]), "+r"(b[1]), "+r"(b[2]), "+r"(b[3]), "+r"(b[4]),
		 "+r"(b[5]), "+r"(b[6]), "+r"(b[7]), "+r"(b[8]), "+r"(b[9]),
		 "+r"(b[10]), "+r"(b[11]), "+r"(b[12]), "+r"(b[13]),
		 "+r"(b[14]), "+r"(b[15]),
		 "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3]), "+r"(c[4]),
		 "+r"(c[5]), "+r"(c[6]), "+r"(c[7]), "+r"(c[8]), "+r"(c[9]),
		 "+r"(c[10]), "+r"(c[11]), "+r"(c[12]), "+r"(c[13]),
		 "+r"(c[14]), "+r"(c[15])
	       :: "memory");
}

/* Shared-memory matrix descriptor (tcgen05): start, leading and stride
 * byte offsets in 16-byte units, descriptor version 1, layout type in
 * bits 61-63 (4 = 64-byte swizzle). */
#define LGB_TC_SWIZZLE_64B 4u

__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo,
					     uint32_t sbo, uint32_t layout) {
  uint64_t d = 0;
  d |= (uint64_t) ((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t) 1u << 46;
  d |= (uint64_t) (layout & 7u) << 61;
  return d;
}

/* Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B,
 * a_mn / b_mn = 1 for MN-major operands, shape M x N. */
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int m, int n, int a_mn,
						     int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) a_mn << 15)
    | ((uint32_t) b_mn << 16) | ((uint32_t) (n >> 3) << 17)
    | ((uint32_t) (m >> 4) << 24);
}

#endif
