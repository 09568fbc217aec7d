// Blackwell (sm_103a) tensor-core primitives in inline PTX: TMEM allocation, tcgen05.mma (kind::f16,
// BF16 operands, FP32 accumulator in TMEM), commit to an mbarrier, TMEM loads, and the shared-memory
// matrix / instruction descriptors.
//
// Operand layout used throughout (SWIZZLE_NONE): a "core matrix" is 8 rows x 16 bytes (8 bf16) stored
// as 128 contiguous bytes, row r at +16*r.
//   K-major operand (rows = M or N, 8 consecutive K elements per 16-byte row):
//     element (row, k) at  (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2
//   MN-major operand (8 consecutive M/N elements per 16-byte row, one row per k):
//     element (row, k) at  (row / 8) * SBO + (k / 8) * LBO + (k % 8) * 16 + (row % 8) * 2
// i.e. in both cases SBO steps between 8-row groups along M/N and LBO between 8-element groups along K.
// Start addresses need only 16-byte alignment, and LBO may be smaller than a core matrix (LBO = 16
// makes the second K group the first one shifted by one row).
// Every wait on an mbarrier is bounded; on expiry the caller records an error and returns.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace swgpu
{
namespace tc05
{

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05 "matrix descriptor"): start address, leading and stride
// byte offsets (all >> 4, 14 bits), descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t make_sdesc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes)
{
	uint64_t d = 0;
	d |= uint64_t((saddr >> 4) & 0x3FFF);
	d |= uint64_t((lbo_bytes >> 4) & 0x3FFF) << 16;
	d |= uint64_t((sbo_bytes >> 4) & 0x3FFF) << 32;
	d |= uint64_t(1) << 46;
	return d;
}

// Instruction descriptor of tcgen05.mma.kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), A / B major-ness (bit 15 / 16: 0 = K-major, 1 = MN-major), N >> 3 at
// bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t make_idesc_bf16(uint32_t m, uint32_t n, uint32_t a_mn_major, uint32_t b_mn_major)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | (a_mn_major << 15) | (b_mn_major << 16) | ((n >> 3) << 17) |
		((m >> 4) << 24);
}

// ---- TMEM ----

// Warp-wide: allocate ncols (power of two, >= 32) TMEM columns; the base address is written to
// *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
				 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Make generic-proxy shared-memory stores visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA ----

// D[tmem] (+)= A * B^T, M x N x 16, one thread issues.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
		"l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
		: "memory");
}

// Arrive on the mbarrier once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
				 : "memory");
}

// ---- mbarrier ----

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity)
{
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
		: "=r"(ok)
		: "r"(smem_addr(mbar)), "r"(parity)
		: "memory");
	return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(mbar)) : "memory");
}
// Bounded wait: true when the phase completed, false after max_polls unsuccessful polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity, uint32_t max_polls)
{
	for (uint32_t i = 0; i < max_polls; ++i)
		if (mbar_try_wait(mbar, parity)) return true;
	return false;
}

// ---- bulk copies (TMA, untiled) ----

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Global -> shared copy of `bytes` (multiple of 16; both addresses 16-byte aligned), completing as
// transaction bytes on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* mbar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
					 smem_addr(dst_smem)),
		"l"(src_gmem), "r"(bytes), "r"(smem_addr(mbar))
				 : "memory");
}

// Tiled 4-D TMA load of one box of the tensor map (a __grid_constant__ kernel parameter) at coordinates
// (c0 innermost .. c3) into shared memory, completing as transaction bytes on the mbarrier.
__device__ __forceinline__ void tma_load_4d(void* dst_smem, const void* tmap, int c0, int c1, int c2, int c3, uint64_t* mbar)
{
	asm volatile(
		"cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
			smem_addr(dst_smem)),
		"l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(mbar))
		: "memory");
}

// ---- TMEM -> registers ----

// 32 lanes x 32 bits, 8 consecutive columns: thread t of the warp gets lane (quadrant*32 + t),
// columns col..col+7 of taddr.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
	uint32_t r[8];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
				 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
				 : "r"(taddr)
				 : "memory");
	for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 32 bits, 8 consecutive columns of zeros (thread t writes lane quadrant*32 + t).
__device__ __forceinline__ void tmem_zero8(uint32_t taddr)
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr), "r"(0u)
				 : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

} // namespace tc05
} // namespace swgpu
