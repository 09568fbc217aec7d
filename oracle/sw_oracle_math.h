// Test infrastructure: CPU restatement of the reference's arithmetic primitives, used only as the
// checker for the GPU path (tests, smoke check and the CPU baseline leg of the benchmark).
//
// Semantics are the reference's generic (non-SSE) fast_math implementation, which is what the
// reference compiles to on aarch64 and on any target without SSE4.1:
//   inv_fast(x) = 1/x, inv_sqrt_fast(x) = 1/sqrt(x)          src/square_wheel/fast_math.rs:376-384
//   f32_mul_add(x,y,z) = x*y + z (two roundings)              src/square_wheel/fast_math.rs:736-740
//   ColorVec -> Color32/64 truncates after min(255/65535)     src/square_wheel/fast_math.rs:472-498
//   ColorVecI -> Color32/64 clamps (v as u32).min(255)        src/square_wheel/fast_math.rs:650-668
// The library must be compiled with -ffp-contract=off so the compiler never fuses a*b+c.
#pragma once

#include <cmath>
#include <cstdint>

namespace sworacle
{

constexpr float MIN_POSITIVE_VALUE = 1.0f / float(1 << 30); // fast_math.rs:744

inline float inv_fast(float x) { return 1.0f / x; }
inline float inv_sqrt_fast(float x) { return 1.0f / std::sqrt(x); }
inline float f32_mul_add(float x, float y, float z) { return x * y + z; }
// Rust f32::max / f32::min: NaN operand yields the other operand.
inline float fmaxr(float a, float b) { return std::fmax(a, b); }
inline float fminr(float a, float b) { return std::fmin(a, b); }

// f32 -> integer conversions as the reference's targets perform them for `to_int_unchecked` and
// saturating `as`: truncation toward zero, clamped to the destination range, NaN -> 0.
inline uint32_t f2u32(float x)
{
	if (!(x > 0.0f)) return 0u;
	if (x >= 4294967296.0f) return 0xFFFFFFFFu;
	return uint32_t(x);
}
inline uint64_t f2u64(float x)
{
	if (!(x > 0.0f)) return 0u;
	if (x >= 18446744073709551616.0f) return ~uint64_t(0);
	return uint64_t(x);
}
inline int32_t f2i32(float x)
{
	if (x != x) return 0;
	if (x >= 2147483648.0f) return INT32_MAX;
	if (x <= -2147483648.0f) return INT32_MIN;
	return int32_t(x);
}
inline int64_t f2i64(float x)
{
	if (x != x) return 0;
	if (x >= 9223372036854775808.0f) return INT64_MAX;
	if (x <= -9223372036854775808.0f) return INT64_MIN;
	return int64_t(x);
}

// Wrapping integer arithmetic (Rust release builds wrap on overflow).
inline int32_t wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
inline int32_t wsub(int32_t a, int32_t b) { return int32_t(uint32_t(a) - uint32_t(b)); }
inline int32_t wmul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
inline int64_t wadd64(int64_t a, int64_t b) { return int64_t(uint64_t(a) + uint64_t(b)); }
inline int64_t wmul64(int64_t a, int64_t b) { return int64_t(uint64_t(a) * uint64_t(b)); }

struct Vec3
{
	float x, y, z;
};
inline Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
inline Vec3 operator+(Vec3 a, Vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec3 operator-(Vec3 a, Vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec3 operator*(Vec3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
// vec3_dot, fast_math.rs:780-783: x*x' + (y*y' + z*z')
inline float vec3_dot(Vec3 a, Vec3 b) { return f32_mul_add(a.x, b.x, f32_mul_add(a.y, b.y, a.z * b.z)); }
inline float vec3_len2(Vec3 v) { return vec3_dot(v, v); }
// vec3_scalar_mul_add, fast_math.rs:786-793
inline Vec3 vec3_scalar_mul_add(Vec3 a, float s, Vec3 b)
{
	return v3(f32_mul_add(a.x, s, b.x), f32_mul_add(a.y, s, b.y), f32_mul_add(a.z, s, b.z));
}

// ColorVec, generic impl (fast_math.rs:441-584). Lane 0 = B, 1 = G, 2 = R, 3 = A.
struct ColorVec
{
	float v[4];
};
inline ColorVec cv_zero() { return ColorVec{{0.0f, 0.0f, 0.0f, 0.0f}}; }
inline ColorVec cv_from_c32(uint32_t c)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = float((c >> (i * 8)) & 0xFFu);
	return r;
}
inline ColorVec cv_from_c64(uint64_t c)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = float(uint32_t((c >> (i * 16)) & 0xFFFFu));
	return r;
}
inline uint32_t cv_to_c32(const ColorVec& c)
{
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i) r |= f2u32(fminr(c.v[i], 255.0f)) << (i * 8);
	return r;
}
inline uint64_t cv_to_c64(const ColorVec& c)
{
	uint64_t r = 0;
	for (int i = 0; i < 4; ++i) r |= f2u64(fminr(c.v[i], 65535.0f)) << (i * 16);
	return r;
}
// from_color_f32x3 (with zero / with one): [c2, c1, c0, 0|1]
inline ColorVec cv_from_f32x3(const float c[3]) { return ColorVec{{c[2], c[1], c[0], 0.0f}}; }
inline ColorVec cv_from_f32x3_one(const float c[3]) { return ColorVec{{c[2], c[1], c[0], 1.0f}}; }
inline ColorVec cv_add(const ColorVec& a, const ColorVec& b)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] + b.v[i];
	return r;
}
inline ColorVec cv_mul(const ColorVec& a, const ColorVec& b)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * b.v[i];
	return r;
}
inline ColorVec cv_scalar_mul(const ColorVec& a, float s)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * s;
	return r;
}
inline ColorVec cv_mul_scalar_add(const ColorVec& a, float s, const ColorVec& b)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = f32_mul_add(a.v[i], s, b.v[i]);
	return r;
}
inline ColorVec cv_mul_add(const ColorVec& a, const ColorVec& b, const ColorVec& c)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = f32_mul_add(a.v[i], b.v[i], c.v[i]);
	return r;
}
inline ColorVec cv_div(const ColorVec& a, const ColorVec& b)
{
	ColorVec r;
	for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] / b.v[i];
	return r;
}

// ColorVecI, generic impl (fast_math.rs:594-724).
struct ColorVecI
{
	int32_t v[4];
};
inline ColorVecI ci_zero() { return ColorVecI{{0, 0, 0, 0}}; }
inline ColorVecI ci_from_c32(uint32_t c)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = int32_t((c >> (i * 8)) & 0xFFu);
	return r;
}
inline ColorVecI ci_from_c64(uint64_t c)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = int32_t((c >> (i * 16)) & 0xFFFFu);
	return r;
}
inline uint32_t ci_to_c32(const ColorVecI& c)
{
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i)
	{
		uint32_t u = uint32_t(c.v[i]);
		r |= (u < 255u ? u : 255u) << (i * 8);
	}
	return r;
}
inline uint64_t ci_to_c64(const ColorVecI& c)
{
	uint64_t r = 0;
	for (int i = 0; i < 4; ++i)
	{
		uint64_t u = uint64_t(int64_t(c.v[i])); // i32 as u64 sign-extends
		r |= (u < 65535u ? u : 65535u) << (i * 16);
	}
	return r;
}
// ColorVecI::from_color_f32x3: [c2 as i32, c1 as i32, c0 as i32, 0]
inline ColorVecI ci_from_f32x3(const float c[3]) { return ColorVecI{{f2i32(c[2]), f2i32(c[1]), f2i32(c[0]), 0}}; }
inline ColorVecI ci_add(const ColorVecI& a, const ColorVecI& b)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = wadd(a.v[i], b.v[i]);
	return r;
}
inline ColorVecI ci_mul(const ColorVecI& a, const ColorVecI& b)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = wmul(a.v[i], b.v[i]);
	return r;
}
inline ColorVecI ci_mul_scalar(const ColorVecI& a, int32_t s)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = wmul(a.v[i], s);
	return r;
}
inline ColorVecI ci_shr(const ColorVecI& a, int n)
{
	ColorVecI r;
	for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] >> n;
	return r;
}
inline ColorVec ci_to_cv(const ColorVecI& a)
{
	return ColorVec{{float(a.v[0]), float(a.v[1]), float(a.v[2]), float(a.v[3])}};
}

// Pixel-type traits for the two AbstractColor instantiations (abstract_color.rs:181-299, color.rs).
struct C32
{
	typedef uint32_t T;
	static ColorVec to_vec(T c) { return cv_from_c32(c); }
	static T from_vec(const ColorVec& c) { return cv_to_c32(c); }
	static ColorVecI to_veci(T c) { return ci_from_c32(c); }
	static T from_veci(const ColorVecI& c) { return ci_to_c32(c); }
	// Color32::get_average, color.rs:46-49 (generic color32_average)
	static T average(T a, T b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); }
	static T saturated_sum(T a, T b)
	{
		T r = 0;
		for (int i = 0; i < 4; ++i)
		{
			uint32_t s = ((a >> (i * 8)) & 0xFFu) + ((b >> (i * 8)) & 0xFFu);
			r |= (s < 0xFFu ? s : 0xFFu) << (i * 8);
		}
		return r;
	}
	static int32_t get_alpha(T c) { return int32_t(c >> 24); }
	static bool test_alpha(T c) { return (c & 0xFF000000u) > 0x7F000000u; }
};

struct C64
{
	typedef uint64_t T;
	static ColorVec to_vec(T c) { return cv_from_c64(c); }
	static T from_vec(const ColorVec& c) { return cv_to_c64(c); }
	static ColorVecI to_veci(T c) { return ci_from_c64(c); }
	static T from_veci(const ColorVecI& c) { return ci_to_c64(c); }
	static T average(T a, T b) { return (((a ^ b) & 0xFFFEFFFEFFFEFFFEull) >> 1) + (a & b); }
	static T saturated_sum(T a, T b)
	{
		T r = 0;
		for (int i = 0; i < 4; ++i)
		{
			uint64_t s = ((a >> (i * 16)) & 0xFFFFu) + ((b >> (i * 16)) & 0xFFFFu);
			r |= (s < 0xFFFFu ? s : 0xFFFFu) << (i * 16);
		}
		return r;
	}
	static int32_t get_alpha(T c) { return int32_t(c >> 48); }
	static bool test_alpha(T c) { return (c & 0xFFFF000000000000ull) > 0x007F000000000000ull; }
};

// AbstractColor::alpha_blend, abstract_color.rs:198-208 / 258-268
template <class P>
inline typename P::T alpha_blend(typename P::T dst, typename P::T src)
{
	int32_t alpha = P::get_alpha(src);
	return P::from_veci(
		ci_shr(ci_add(ci_mul_scalar(P::to_veci(dst), wsub(255, alpha)), ci_mul_scalar(P::to_veci(src), alpha)), 8));
}

} // namespace sworacle
