// Device-side arithmetic shared by the GB300 kernels.
//
// Every kernel is compiled with --fmad=false and IEEE division/sqrt so that each a*b+c is two
// correctly rounded operations, which is the reference's generic fast_math semantics
// (src/square_wheel/fast_math.rs:376-384, 736-740). Float->int conversions use PTX cvt.rzi,
// which truncates and saturates (NaN -> 0), matching the reference's to_int_unchecked on aarch64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/swgpu.h"

namespace swgpu
{

constexpr float MIN_POSITIVE_VALUE = 1.0f / float(1 << 30);

// Programmatic dependent launch between the frame's kernels: a kernel launched with
// launch_dependent() may start while its predecessor in the stream is still running and must call
// pdl_wait() before it reads anything the predecessor writes (it waits for the predecessor grid to
// complete and its memory to be visible; a no-op without such a predecessor). pdl_trigger() tells the
// runtime that the successor may be scheduled (each CTA calls it once its work is done).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
	Args&&... args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

__device__ __forceinline__ float inv_fast(float x) { return __fdiv_rn(1.0f, x); }
__device__ __forceinline__ float inv_sqrt_fast(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
// f32_mul_add, generic: two roundings.
__device__ __forceinline__ float mad2(float x, float y, float z) { return __fadd_rn(__fmul_rn(x, y), z); }

struct V3
{
	float x, y, z;
};
__device__ __forceinline__ V3 mkv3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3add(V3 a, V3 b) { return mkv3(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)); }
__device__ __forceinline__ V3 v3sub(V3 a, V3 b) { return mkv3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)); }
__device__ __forceinline__ V3 v3scale(V3 a, float s) { return mkv3(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)); }
__device__ __forceinline__ float v3dot(V3 a, V3 b) { return mad2(a.x, b.x, mad2(a.y, b.y, fmul(a.z, b.z))); }
__device__ __forceinline__ V3 v3sma(V3 a, float s, V3 b) { return mkv3(mad2(a.x, s, b.x), mad2(a.y, s, b.y), mad2(a.z, s, b.z)); }

// Four-lane colour in the reference's lane order (0 = B, 1 = G, 2 = R, 3 = A).
struct CV
{
	float b, g, r, a;
};
__device__ __forceinline__ CV cv_zero() { return CV{0.0f, 0.0f, 0.0f, 0.0f}; }
__device__ __forceinline__ CV cv_rgb(const float c[3], float alpha) { return CV{c[2], c[1], c[0], alpha}; }
__device__ __forceinline__ CV cv_sma(CV a, float s, CV b)
{
	return CV{mad2(a.b, s, b.b), mad2(a.g, s, b.g), mad2(a.r, s, b.r), mad2(a.a, s, b.a)};
}
__device__ __forceinline__ CV cv_scale(CV a, float s) { return CV{fmul(a.b, s), fmul(a.g, s), fmul(a.r, s), fmul(a.a, s)}; }
__device__ __forceinline__ CV cv_mul(CV a, CV b) { return CV{fmul(a.b, b.b), fmul(a.g, b.g), fmul(a.r, b.r), fmul(a.a, b.a)}; }
__device__ __forceinline__ CV cv_add(CV a, CV b) { return CV{fadd(a.b, b.b), fadd(a.g, b.g), fadd(a.r, b.r), fadd(a.a, b.a)}; }

__device__ __forceinline__ CV cv_from_c32(uint32_t c)
{
	return CV{float(c & 0xFFu), float((c >> 8) & 0xFFu), float((c >> 16) & 0xFFu), float(c >> 24)};
}
__device__ __forceinline__ CV cv_from_c64(uint64_t c)
{
	return CV{float(uint32_t(c) & 0xFFFFu), float(uint32_t(c >> 16) & 0xFFFFu), float(uint32_t(c >> 32) & 0xFFFFu),
		float(uint32_t(c >> 48))};
}
// ColorVec -> Color32/64: min(255/65535) then truncating, saturating conversion (fminf(NaN, m) = m).
__device__ __forceinline__ uint32_t f2u_rz(float x) { return __float2uint_rz(x); }
__device__ __forceinline__ uint32_t cv_to_c32(CV c)
{
	return f2u_rz(fminf(c.b, 255.0f)) | (f2u_rz(fminf(c.g, 255.0f)) << 8) | (f2u_rz(fminf(c.r, 255.0f)) << 16) |
		(f2u_rz(fminf(c.a, 255.0f)) << 24);
}
__device__ __forceinline__ uint64_t cv_to_c64(CV c)
{
	return uint64_t(f2u_rz(fminf(c.b, 65535.0f))) | (uint64_t(f2u_rz(fminf(c.g, 65535.0f))) << 16) |
		(uint64_t(f2u_rz(fminf(c.r, 65535.0f))) << 32) | (uint64_t(f2u_rz(fminf(c.a, 65535.0f))) << 48);
}

// Integer four-lane colour (ColorVecI) with wrapping arithmetic.
struct CI
{
	int32_t v[4];
};
__device__ __forceinline__ CI ci_from_c32(uint32_t c)
{
	return CI{{int32_t(c & 0xFFu), int32_t((c >> 8) & 0xFFu), int32_t((c >> 16) & 0xFFu), int32_t(c >> 24)}};
}
__device__ __forceinline__ CI ci_from_c64(uint64_t c)
{
	return CI{{int32_t(uint32_t(c) & 0xFFFFu), int32_t(uint32_t(c >> 16) & 0xFFFFu), int32_t(uint32_t(c >> 32) & 0xFFFFu),
		int32_t(uint32_t(c >> 48))}};
}
// ColorVecI -> Color32: (v as u32).min(255); -> Color64: (v as u64).min(65535) (negative -> max).
__device__ __forceinline__ uint32_t ci_to_c32(const CI& c)
{
	uint32_t r = 0;
#pragma unroll
	for (int i = 0; i < 4; ++i) r |= min(uint32_t(c.v[i]), 255u) << (i * 8);
	return r;
}
__device__ __forceinline__ uint64_t ci_to_c64(const CI& c)
{
	uint64_t r = 0;
#pragma unroll
	for (int i = 0; i < 4; ++i) r |= uint64_t(min(uint32_t(c.v[i]), 65535u)) << (i * 16);
	return r;
}
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
__device__ __forceinline__ int32_t wsub(int32_t a, int32_t b) { return int32_t(uint32_t(a) - uint32_t(b)); }

// Pixel-format traits (AbstractColor for Color32 / Color64).
struct PixC32
{
	typedef uint32_t T;
	static constexpr uint32_t FORMAT = SW_PIXEL_C32;
	__device__ static T from_cv(CV c) { return cv_to_c32(c); }
	__device__ static CI to_ci(T c) { return ci_from_c32(c); }
	__device__ static T from_ci(const CI& c) { return ci_to_c32(c); }
	__device__ static T average(T a, T b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); }
	__device__ static T saturated_sum(T a, T b) { return __vaddus4(a, b); }
	__device__ static int32_t get_alpha(T c) { return int32_t(c >> 24); }
	__device__ static bool test_alpha(T c) { return (c & 0xFF000000u) > 0x7F000000u; }
};
struct PixC64
{
	typedef uint64_t T;
	static constexpr uint32_t FORMAT = SW_PIXEL_C64;
	__device__ static T from_cv(CV c) { return cv_to_c64(c); }
	__device__ static CI to_ci(T c) { return ci_from_c64(c); }
	__device__ static T from_ci(const CI& c) { return ci_to_c64(c); }
	__device__ static T average(T a, T b) { return (((a ^ b) & 0xFFFEFFFEFFFEFFFEull) >> 1) + (a & b); }
	__device__ static T saturated_sum(T a, T b)
	{
		uint32_t lo = __vaddus2(uint32_t(a), uint32_t(b));
		uint32_t hi = __vaddus2(uint32_t(a >> 32), uint32_t(b >> 32));
		return uint64_t(lo) | (uint64_t(hi) << 32);
	}
	__device__ static int32_t get_alpha(T c) { return int32_t(c >> 48); }
	__device__ static bool test_alpha(T c) { return (c & 0xFFFF000000000000ull) > 0x007F000000000000ull; }
};

template <class P>
__device__ __forceinline__ typename P::T alpha_blend(typename P::T dst, typename P::T src)
{
	const int32_t alpha = P::get_alpha(src);
	const CI d = P::to_ci(dst), s = P::to_ci(src);
	CI r;
#pragma unroll
	for (int i = 0; i < 4; ++i) r.v[i] = wadd(wmul(d.v[i], wsub(255, alpha)), wmul(s.v[i], alpha)) >> 8;
	return P::from_ci(r);
}

} // namespace swgpu
