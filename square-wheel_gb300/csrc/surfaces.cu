// Surface builder for the GB300 path: every visible polygon surface of a frame in one persistent
// launch.
//
// Replaces build_polygons_surfaces' per-polygon work (src/square_wheel/partial_renderer.rs:1682-1831):
// build_surface_impl_6_static_params (src/square_wheel/surfaces.rs:433-852) followed by the emissive
// layer mix_surface_with_texture (src/square_wheel/surfaces.rs:903-971), fused in one pass.
//
// Work decomposition: the frame's surfaces form one flat texel index space (prefix sums of surface
// areas, in descriptor order). A grid of (#SMs x resident blocks) threads strides over it, so surfaces
// from 4x4 to 512x512 texels share one launch without tail effects. Each warp owns 32 consecutive
// texels: lane 0 finds the first texel's surface by binary search over the prefix array, every lane
// then steps forward to its own surface (at most a few steps, only across tiny surfaces). Each thread
// rebuilds the reference's row-interpolated lightmap line entries it needs (the two vertical mixes of
// the line buffer and the horizontal mix, in the reference's operation order), evaluates lighting and
// stores its texel. Neighbouring threads read neighbouring TextureElements and share lightmap elements,
// so texture reads and surface writes are coalesced and lightmap reads are L1 broadcasts.
#include "sw_kernels.cuh"

#include <cmath>

namespace swgpu
{

namespace
{

const float NORMAL_UNPACK_SCALE = 1.0f / 127.0f;
constexpr float PI_F = 3.14159265358979323846f;
// Specular lobe constants, src/square_wheel/surfaces.rs:1108-1110 (f32 constant arithmetic).
constexpr float SPEC_A = 2.0f * PI_F / 2.645751311f;
constexpr float SPEC_B = PI_F * 2.645751311f / 2.0f;
constexpr float DIELECTRIC_ZERO_REFLECTIVITY = 0.04f;
constexpr float DIELECTRIC_AVERAGE_REFLECTIVITY = DIELECTRIC_ZERO_REFLECTIVITY * 3.0f;
constexpr float METAL_AVERAGE_SCHLICK_FACTOR = 0.5f;

__device__ __forceinline__ float specular_intensity(float angle_cos, float inv_roughness)
{
	float x = fmul(fsub(angle_cos, 1.0f), inv_roughness);
	return fmul(inv_fast(mad2(fmul(x, x), SPEC_B, SPEC_A)), inv_roughness);
}
__device__ __forceinline__ float fresnel_factor_base(float c)
{
	float omc = fmaxf(fsub(1.0f, c), 0.0f);
	float omc2 = fmul(omc, omc);
	return fmul(fmul(omc2, omc2), omc);
}
__device__ __forceinline__ float specular_k(int spec, float f, float roughness)
{
	if (spec == 1)
	{
		float fresnel = mad2(f, 1.0f - DIELECTRIC_ZERO_REFLECTIVITY, DIELECTRIC_ZERO_REFLECTIVITY);
		return mad2(fresnel, fsub(1.0f, roughness), fmul(DIELECTRIC_AVERAGE_REFLECTIVITY, roughness));
	}
	return mad2(f, fsub(1.0f, roughness), fmul(METAL_AVERAGE_SCHLICK_FACTOR, roughness));
}

struct Lm
{
	float amb[3];
	V3 dir;
	float dev;
	float col[3];
};

template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lm_load(const SurfaceKernelArgs& a, uint64_t index)
{
	Lm e;
	if (DIRECTIONAL)
	{
		// 40-byte element, 8-byte aligned: five 64-bit read-only loads.
		const float2* p = reinterpret_cast<const float2*>(a.directional_lightmaps + index);
		const float2 q0 = __ldg(p + 0), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3), q4 = __ldg(p + 4);
		e.amb[0] = q0.x;
		e.amb[1] = q0.y;
		e.amb[2] = q1.x;
		e.dir = mkv3(q1.y, q2.x, q2.y);
		e.dev = q3.x;
		e.col[0] = q3.y;
		e.col[1] = q4.x;
		e.col[2] = q4.y;
	}
	else
	{
		const float* p = a.lightmaps + index * 3;
		e.amb[0] = __ldg(p + 0);
		e.amb[1] = __ldg(p + 1);
		e.amb[2] = __ldg(p + 2);
	}
	return e;
}

// LightmapElementOps::mix(a, b, ratio) = a*ratio + b*(1-ratio), surfaces.rs:996-1071
template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lm_mix(const Lm& a, const Lm& b, float ratio)
{
	const float omr = fsub(1.0f, ratio);
	Lm r;
#pragma unroll
	for (int i = 0; i < 3; ++i) r.amb[i] = mad2(a.amb[i], ratio, fmul(b.amb[i], omr));
	if (DIRECTIONAL)
	{
		r.dir = mkv3(mad2(a.dir.x, ratio, fmul(b.dir.x, omr)), mad2(a.dir.y, ratio, fmul(b.dir.y, omr)),
			mad2(a.dir.z, ratio, fmul(b.dir.z, omr)));
		r.dev = mad2(a.dev, ratio, fmul(b.dev, omr));
#pragma unroll
		for (int i = 0; i < 3; ++i) r.col[i] = mad2(a.col[i], ratio, fmul(b.col[i], omr));
	}
	return r;
}

__device__ __forceinline__ uint32_t wrap(int32_t a, uint32_t b)
{
	int32_t r = a % int32_t(b);
	return uint32_t(r < 0 ? r + int32_t(b) : r);
}
// rem_euclid by a texture side: a mask for powers of two (mask != ~0u), else the remainder
__device__ __forceinline__ uint32_t wrap_side(int32_t a, uint32_t b, uint32_t mask)
{
	return mask != ~0u ? uint32_t(a) & mask : wrap(a, b);
}
// n / d and n % d: the float estimate of the quotient (truncated product with the rounded reciprocal) is
// within one of it while the quotient stays below 2^22 (a surface's row), then corrected exactly
__device__ __forceinline__ void div_row(uint32_t n, uint32_t d, float inv_d, uint32_t& q, uint32_t& r)
{
	int32_t qi = int32_t(__fmul_rz(float(n), inv_d));
	int32_t ri = int32_t(n) - qi * int32_t(d);
	if (ri < 0)
	{
		--qi;
		ri += int32_t(d);
	}
	else if (ri >= int32_t(d))
	{
		++qi;
		ri -= int32_t(d);
	}
	q = uint32_t(qi);
	r = uint32_t(ri);
}

// cube_shadow_map_side_fetch (light.rs:235-258): 1 in light, 0 in shadow.
__device__ __forceinline__ float cube_side_fetch(const unsigned long long* side, uint32_t size, float x, float y, float z)
{
	const float ONE_MINUS_EPS = 1.0f - 1.0f / 65536.0f;
	const float size_f = float(size);
	const float depth = inv_fast(fmaxf(z, MIN_POSITIVE_VALUE));
	const float half_depth = fmul(0.5f, depth);
	const float u_f = fmul(fminf(fmaxf(fadd(fmul(x, half_depth), 0.5f), 0.0f), ONE_MINUS_EPS), size_f);
	const float v_f = fmul(fminf(fmaxf(fadd(fmul(y, half_depth), 0.5f), 0.0f), ONE_MINUS_EPS), size_f);
	const uint32_t u = __float2uint_rz(u_f), v = __float2uint_rz(v_f); // in [0, size)
	return depth >= __uint_as_float(uint32_t(__ldg(side + u + v * size))) ? 1.0f : 0.0f; // the texel's f32 bits
}

// projector_shadow_map_fetch (light.rs:261-294): 0 behind the projector or outside its map.
__device__ __forceinline__ float projector_fetch(const SurfaceKernelArgs& a, const SwLightShadow& m, V3 vec)
{
	const float z = v3dot(mkv3(m.basis_z[0], m.basis_z[1], m.basis_z[2]), vec);
	if (z <= 0.0f) return 0.0f;
	const float depth = inv_fast(z);
	const float half_depth = fmul(0.5f, depth);
	const float size_f = float(m.size);
	const float u_f = fmul(mad2(v3dot(mkv3(m.basis_x[0], m.basis_x[1], m.basis_x[2]), vec), half_depth, 0.5f), size_f);
	const float v_f = fmul(mad2(v3dot(mkv3(m.basis_y[0], m.basis_y[1], m.basis_y[2]), vec), half_depth, 0.5f), size_f);
	if (u_f < 0.0f || v_f < 0.0f || u_f >= size_f || v_f >= size_f) return 0.0f;
	const uint32_t u = __float2uint_rz(u_f), v = __float2uint_rz(v_f); // in [0, size)
	return depth >= __uint_as_float(uint32_t(__ldg(a.shadow_texels + m.offset + u + v * m.size))) ? 1.0f : 0.0f;
}

// get_light_shadow_factor / cube_shadow_map_fetch (light.rs:185-233) for `to_light` = light - point.
__device__ __forceinline__ float light_shadow_factor(const SurfaceKernelArgs& a, uint32_t light, V3 to_light)
{
	if (!a.shadows || light >= a.num_shadows) return 1.0f;
	const SwLightShadow m = a.shadows[light];
	if (m.kind == SW_SHADOW_PROJECTOR) return projector_fetch(a, m, to_light);
	if (m.kind != SW_SHADOW_CUBE) return 1.0f;
	const uint64_t side_texels = uint64_t(m.size) * m.size;
	const unsigned long long* maps = a.shadow_texels + m.offset;
	const float ax = fabsf(to_light.x), ay = fabsf(to_light.y), az = fabsf(to_light.z);
	if (ax >= ay && ax >= az)
		return to_light.x >= 0.0f ? cube_side_fetch(maps + 1 * side_texels, m.size, -to_light.y, to_light.z, ax)
								  : cube_side_fetch(maps + 0 * side_texels, m.size, to_light.y, to_light.z, ax);
	if (ay >= ax && ay >= az)
		return to_light.y >= 0.0f ? cube_side_fetch(maps + 3 * side_texels, m.size, to_light.x, to_light.z, ay)
								  : cube_side_fetch(maps + 2 * side_texels, m.size, -to_light.x, to_light.z, ay);
	return to_light.z >= 0.0f ? cube_side_fetch(maps + 5 * side_texels, m.size, -to_light.x, to_light.y, az)
							  : cube_side_fetch(maps + 4 * side_texels, m.size, -to_light.x, -to_light.y, az);
}

// The line buffer of the reference's row loop (surfaces.rs:477-502) for one thread's run of texels: the
// entries line_lightmap[lu] and [lu + 1] of texel row v (the vertical mixes of lightmap rows lv and
// lv + 1 at ratio kv), kept while the run stays in that row and column and shifted by one when it
// steps into the next lightmap column, as the reference's row buffer holds them.
template <bool DIRECTIONAL>
struct LineCache
{
	uint32_t si = 0xFFFFFFFFu, v = 0, lu = 0;
	Lm line0, line1;
};

template <bool DIRECTIONAL>
__device__ __forceinline__ void line_entries(const SurfaceKernelArgs& a, const SurfaceGpu& s, uint32_t si, uint32_t v,
	uint32_t lv, uint32_t lu, float kv, LineCache<DIRECTIONAL>& c)
{
	if (c.si == si && c.v == v && c.lu == lu) return;
	const uint64_t row0 = uint64_t(s.lm_offset) + uint64_t(lv) * s.lm_width;
	const uint64_t row1 = row0 + s.lm_width;
	if (c.si == si && c.v == v && c.lu + 1 == lu)
		c.line0 = c.line1;
	else
		c.line0 = lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu), lm_load<DIRECTIONAL>(a, row0 + lu), kv);
	c.line1 = lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu + 1), lm_load<DIRECTIONAL>(a, row0 + lu + 1), kv);
	c.si = si;
	c.v = v;
	c.lu = lu;
}

// The texel's lightmap element (surfaces.rs:504-513): the horizontal mix of its two line entries.
template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lightmap_sample(const SurfaceKernelArgs& a, const SurfaceGpu& s, uint32_t si, uint32_t u,
	uint32_t v, LineCache<DIRECTIONAL>& c)
{
	const uint32_t log2 = s.lm_log2;
	const uint32_t mask = (1u << log2) - 1u;
	const uint32_t base_v = v + s.lm_shift1;
	const float kv = mad2(float(base_v & mask), s.inv_scale, s.k_shift);
	const uint32_t base_u = u + s.lm_shift0;
	const float ku = mad2(float(base_u & mask), s.inv_scale, s.k_shift);
	line_entries<DIRECTIONAL>(a, s, si, v, base_v >> log2, base_u >> log2, kv, c);
	return lm_mix<DIRECTIONAL>(c.line1, c.line0, ku);
}

// The same element for a single texel: both line entries built for it alone.
template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lightmap_sample_once(const SurfaceKernelArgs& a, const SurfaceGpu& s, uint32_t u, uint32_t v)
{
	const uint32_t log2 = s.lm_log2;
	const uint32_t mask = (1u << log2) - 1u;
	const uint32_t base_v = v + s.lm_shift1;
	const float kv = mad2(float(base_v & mask), s.inv_scale, s.k_shift);
	const uint32_t base_u = u + s.lm_shift0;
	const uint32_t lu = base_u >> log2;
	const float ku = mad2(float(base_u & mask), s.inv_scale, s.k_shift);
	const uint64_t row0 = uint64_t(s.lm_offset) + uint64_t(base_v >> log2) * s.lm_width;
	const uint64_t row1 = row0 + s.lm_width;
	const Lm line0 = lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu), lm_load<DIRECTIONAL>(a, row0 + lu), kv);
	const Lm line1 = lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu + 1), lm_load<DIRECTIONAL>(a, row0 + lu + 1), kv);
	return lm_mix<DIRECTIONAL>(line1, line0, ku);
}

// Lighting of one texel (surfaces.rs:515-842) with its lightmap element `l` (when the surface has a
// lightmap); returns the ColorVec before conversion.
template <bool DIRECTIONAL>
__device__ __forceinline__ CV shade_texel(const SurfaceKernelArgs& a, const SurfaceGpu& s, uint64_t texel, uint32_t u,
	uint32_t v, V3 cam, const Lm& l)
{
	const uint32_t tex_flags = s.flags & 7u;
	const bool use_normal_map = (tex_flags & SW_TEX_HAS_NORMAL_MAP) != 0;
	const int spec = (tex_flags & SW_TEX_HAS_NON_ONE_ROUGHNESS) ? ((tex_flags & SW_TEX_IS_METAL) ? 2 : 1) : 0;

	const V3 u_vec = mkv3(s.u[0], s.u[1], s.u[2]);
	const V3 v_vec = mkv3(s.v[0], s.v[1], s.v[2]);
	const V3 bnormal = mkv3(s.normal[0], s.normal[1], s.normal[2]);
	const V3 pos = v3sma(u_vec, float(u), v3sma(v_vec, float(v), mkv3(s.start_pos[0], s.start_pos[1], s.start_pos[2])));

	V3 tn = mkv3(0.0f, 0.0f, 1.0f);
	float rough = 0.0f;
	const int32_t packed = int32_t(uint32_t(texel >> 32));
	if (use_normal_map)
	{
		tn = mkv3(fmul(float(int32_t(uint32_t(packed) << 24) >> 24), NORMAL_UNPACK_SCALE),
			fmul(float(int32_t(uint32_t(packed) << 16) >> 24), NORMAL_UNPACK_SCALE),
			fmul(float(int32_t(uint32_t(packed) << 8) >> 24), NORMAL_UNPACK_SCALE));
		rough = fmul(float(packed >> 24), NORMAL_UNPACK_SCALE);
	}
	else if (spec != 0)
		rough = fmul(float(packed >> 24), NORMAL_UNPACK_SCALE);

	CV albedo = cv_zero(); // total_light_albedo_modulated
	CV direct = cv_zero(); // total_light_direct
	if (s.flags & SW_SG_LIGHTMAP)
	{
		if (spec == 0)
		{
			albedo = cv_rgb(l.amb, 1.0f);
			if (DIRECTIONAL)
			{
				float dot = use_normal_map ? fmaxf(v3dot(l.dir, tn), 0.0f) : l.dir.z;
				albedo = cv_sma(cv_rgb(l.col, 0.0f), dot, albedo);
			}
		}
		else
		{
			const V3 u_norm = mkv3(s.u_norm[0], s.u_norm[1], s.u_norm[2]);
			const V3 v_norm = mkv3(s.v_norm[0], s.v_norm[1], s.v_norm[2]);
			const V3 normal = use_normal_map ? tn : mkv3(0.0f, 0.0f, 1.0f);
			const V3 to_cam = v3sub(cam, pos);
			const V3 to_cam_ts = mkv3(v3dot(to_cam, u_norm), v3dot(to_cam, v_norm), v3dot(to_cam, bnormal));
			const float ndot = v3dot(to_cam_ts, normal);
			const V3 refl = v3sub(v3scale(normal, fmul(2.0f, ndot)), to_cam_ts);
			const float refl_len2 = fmaxf(v3dot(refl, refl), MIN_POSITIVE_VALUE);
			const float angle_cos = fmaxf(fmul(ndot, inv_sqrt_fast(refl_len2)), 0.0f);
			const float sk = specular_k(spec, fresnel_factor_base(angle_cos), rough);
			const float omsk = fsub(1.0f, sk);
			const CV constant = cv_rgb(l.amb, 0.0f);
			albedo = cv_scale(constant, omsk);
			direct = cv_scale(constant, sk);
			albedo.a = 1.0f;
			if (DIRECTIONAL)
			{
				const float dir_len2 = v3dot(l.dir, l.dir);
				const float dir_len = fmul(dir_len2, inv_sqrt_fast(dir_len2));
				const float rl_cos = fmul(v3dot(refl, l.dir), inv_sqrt_fast(fmul(refl_len2, dir_len2)));
				const float inv_rc = fmaxf(inv_fast(fadd(rough, l.dev)), 0.75f);
				const float si = specular_intensity(rl_cos, inv_rc);
				const CV dcol = cv_rgb(l.col, 0.0f);
				if (spec == 1)
				{
					const float di = fmaxf(v3dot(l.dir, tn), 0.0f);
					albedo = cv_sma(dcol, fmul(di, omsk), albedo);
					direct = cv_sma(dcol, fmul(fmul(si, sk), dir_len), direct);
				}
				else
				{
					const float sf = fmul(si, dir_len);
					albedo = cv_sma(dcol, fmul(omsk, sf), albedo);
					direct = cv_sma(dcol, fmul(sk, sf), direct);
				}
			}
		}
	}

	if (s.num_lights > 0)
	{
		V3 normal = bnormal;
		if (use_normal_map)
		{
			const V3 u_norm = mkv3(s.u_norm[0], s.u_norm[1], s.u_norm[2]);
			const V3 v_norm = mkv3(s.v_norm[0], s.v_norm[1], s.v_norm[2]);
			normal = mkv3(mad2(tn.x, u_norm.x, mad2(tn.y, v_norm.x, fmul(tn.z, bnormal.x))),
				mad2(tn.x, u_norm.y, mad2(tn.y, v_norm.y, fmul(tn.z, bnormal.y))),
				mad2(tn.x, u_norm.z, mad2(tn.y, v_norm.z, fmul(tn.z, bnormal.z))));
		}
		V3 refl = mkv3(0.0f, 0.0f, 0.0f);
		float refl_len2 = MIN_POSITIVE_VALUE;
		float sk = 0.0f, inv_rough = 0.0f;
		if (spec != 0)
		{
			const V3 to_cam = v3sub(cam, pos);
			const float ndot = v3dot(to_cam, normal);
			refl = v3sub(v3scale(normal, fmul(2.0f, ndot)), to_cam);
			refl_len2 = fmaxf(v3dot(refl, refl), MIN_POSITIVE_VALUE);
			const float angle_cos = fmaxf(fmul(ndot, inv_sqrt_fast(refl_len2)), 0.0f);
			sk = specular_k(spec, fresnel_factor_base(angle_cos), rough);
			inv_rough = inv_fast(rough);
		}
		for (uint32_t li = 0; li < s.num_lights; ++li)
		{
			const SwLight& L = a.lights[s.lights[li]];
			const V3 to_light = v3sub(mkv3(L.position[0], L.position[1], L.position[2]), pos);
			const float tl_len2 = fmaxf(v3dot(to_light, to_light), MIN_POSITIVE_VALUE);
			const float sdf = fmul(light_shadow_factor(a, s.lights[li], to_light), fmaxf(fsub(inv_fast(tl_len2), L.inv_square_radius), 0.0f));
			float di = 0.0f;
			if (spec != 2) di = fmaxf(fmul(v3dot(normal, to_light), inv_sqrt_fast(tl_len2)), 0.0f);
			float si = 0.0f;
			if (spec != 0)
				si = specular_intensity(fmul(v3dot(refl, to_light), inv_sqrt_fast(fmul(refl_len2, tl_len2))), inv_rough);
			const CV lc = cv_rgb(L.color, 0.0f);
			if (spec == 0)
				albedo = cv_sma(lc, fmul(di, sdf), albedo);
			else if (spec == 1)
			{
				albedo = cv_sma(lc, fmul(fmul(di, fsub(1.0f, sk)), sdf), albedo);
				direct = cv_sma(lc, fmul(fmul(si, sk), sdf), direct);
			}
			else
			{
				const float sisdf = fmul(si, sdf);
				albedo = cv_sma(lc, fmul(fsub(1.0f, sk), sisdf), albedo);
				direct = cv_sma(lc, fmul(sk, sisdf), direct);
			}
		}
	}

	CV result = cv_mul(cv_from_c32(uint32_t(texel)), albedo);
	if (spec != 0) result = cv_sma(direct, 255.0f, result);
	return result;
}

template <class P>
__device__ __forceinline__ typename P::T emissive_mix(const SurfaceKernelArgs& a, const SurfaceGpu& s, uint32_t u,
	uint32_t v, typename P::T dst, bool additive)
{
	const uint32_t sv = wrap_side(s.tc1 + int32_t(v), s.em_h, s.em_mask[1]);
	const uint32_t su = wrap_side(s.tc0 + int32_t(u), s.em_w, s.em_mask[0]);
	const uint32_t texel = __ldg(a.emissive_pixels + s.em_offset + uint64_t(sv) * s.em_w + su);
	const CI t = ci_from_c32(texel);
	CI m{{wmul(t.v[0], s.em_light[0]) >> 8, wmul(t.v[1], s.em_light[1]) >> 8, wmul(t.v[2], s.em_light[2]) >> 8, 0}};
	if (!additive) return P::from_ci(m);
	const CI d = P::to_ci(dst);
#pragma unroll
	for (int i = 0; i < 4; ++i) m.v[i] = wadd(m.v[i], d.v[i]);
	return P::from_ci(m);
}

// K consecutive texels of the flat texel space per thread (a warp owns 32 * K): the thread's surface is
// found once (lane 0's binary search for the warp, then forward steps), its later texels step along the
// row and into following surfaces, and its line-buffer entries carry from texel to texel. K = 1 runs
// four blocks per SM (64 registers, a few bytes spilled): the kernel issues ~600 instructions per
// texel of exact, unfused f32 shading and integer indexing, and more resident warps hide their latency
// better than fewer, longer threads (K = 4 and its shared line entries measured no faster).
template <class P, bool DIRECTIONAL, int K>
__global__ void __launch_bounds__(256, K == 1 ? 4 : 2) surf_build_kernel(SurfaceKernelArgs a)
{
	typedef typename P::T T;
	T* arena = static_cast<T*>(a.arena);
	const uint64_t total = a.counts ? a.counts->total_texels : a.total_work;
	const V3 cam = a.cam_pos_dev ? mkv3(a.cam_pos_dev[0], a.cam_pos_dev[1], a.cam_pos_dev[2])
								 : mkv3(a.cam_pos[0], a.cam_pos[1], a.cam_pos[2]);
	const uint32_t num_surfaces = a.counts ? a.counts->num_surfaces : a.num_surfaces;
	const uint64_t stride = uint64_t(gridDim.x) * blockDim.x * K;
	const uint32_t lane = threadIdx.x & 31u;
	const uint64_t warp_first = (uint64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u)) * K;
	for (uint64_t wbase = a.work_begin + warp_first; wbase < total; wbase += stride)
	{
		const uint64_t t0 = wbase + uint64_t(lane) * K;
		// Surface of the warp's first texel (binary search by lane 0), then forward steps per lane.
		uint32_t s0 = 0;
		if (lane == 0)
		{
			uint32_t lo = 0, hi = num_surfaces; // prefix[lo] <= wbase < prefix[hi]
			while (hi - lo > 1)
			{
				const uint32_t mid = (lo + hi) >> 1;
				if (__ldg(a.work_prefix + mid) <= wbase)
					lo = mid;
				else
					hi = mid;
			}
			s0 = lo;
		}
		uint32_t si = __shfl_sync(0xFFFFFFFFu, s0, 0);
		if (t0 >= total) continue;
		uint64_t next = __ldg(a.work_prefix + si + 1);
		while (next <= t0)
		{
			++si;
			next = __ldg(a.work_prefix + si + 1);
		}
		uint32_t local = uint32_t(t0 - __ldg(a.work_prefix + si));
		uint32_t width = a.surfaces[si].width;
		uint32_t v, u;
		div_row(local, width, a.surfaces[si].inv_width, v, u);
		[[maybe_unused]] LineCache<DIRECTIONAL> cache;
#pragma unroll 1
		for (int k = 0; k < K; ++k)
		{
			if (k > 0)
			{
				const uint64_t t = t0 + uint64_t(k);
				if (t >= total) break;
				if (t >= next)
				{
					// the next surface with texels: its first texel
					do
					{
						++si;
						next = __ldg(a.work_prefix + si + 1);
					} while (next <= t);
					width = a.surfaces[si].width;
					local = 0;
					u = 0;
					v = 0;
				}
				else
				{
					++local;
					if (++u == width)
					{
						u = 0;
						++v;
					}
				}
			}
			const SurfaceGpu& s = a.surfaces[si];
			T out = T(0);
			const bool diffuse_layer = (s.flags & SW_SG_DIFFUSE) != 0;
			if (diffuse_layer)
			{
				const uint32_t sv = wrap_side(s.tc1 + int32_t(v), s.tex_h, s.tex_mask[1]);
				const uint32_t su = wrap_side(s.tc0 + int32_t(u), s.tex_w, s.tex_mask[0]);
				const uint64_t texel =
					__ldg(reinterpret_cast<const unsigned long long*>(a.texels) + s.tex_offset + uint64_t(sv) * s.tex_w + su);
				Lm l;
				if (s.flags & SW_SG_LIGHTMAP)
				{
					if constexpr (K == 1)
						l = lightmap_sample_once<DIRECTIONAL>(a, s, u, v);
					else
						l = lightmap_sample<DIRECTIONAL>(a, s, si, u, v, cache);
				}
				out = P::from_cv(shade_texel<DIRECTIONAL>(a, s, texel, u, v, cam, l));
			}
			if (s.flags & SW_SG_EMISSIVE) out = emissive_mix<P>(a, s, u, v, out, diffuse_layer);
			arena[s.out_offset + local] = out;
		}
	}
	pdl_trigger(); // the tile pass may be scheduled (it waits for this grid before reading the arena)
}

} // namespace

int launch_surface_build(const SurfaceKernelArgs& args, uint32_t pixel_format, int num_sms, int blocks_per_sm, cudaStream_t stream,
	uint64_t work_hint, uint32_t texels_per_thread)
{
	const uint64_t work = args.counts ? work_hint : args.total_work - args.work_begin;
	if (work == 0 && !args.counts) return 0;
	const int threads = 256;
	// texels per thread: as tuned (by default 1: the shading arithmetic, not the lightmap mixes, bounds the
	// kernel, and carrying line entries over 4 texels measured no faster)
	const int k = texels_per_thread == 4 ? 4 : 1;
	uint64_t blocks_needed = (work + uint64_t(threads) * k - 1) / (uint64_t(threads) * k);
	if (args.counts && blocks_needed < uint64_t(num_sms)) blocks_needed = uint64_t(num_sms);
	// At most blocks_per_sm blocks per SM (several waves of resident blocks): small frames get one
	// texel per thread (latency hidden by parallelism), large batches stride.
	uint64_t blocks_max = uint64_t(num_sms) * uint64_t(blocks_per_sm);
	unsigned blocks = unsigned(blocks_needed < blocks_max ? blocks_needed : blocks_max);
	const bool c64 = pixel_format == SW_PIXEL_C64;
	if (k == 4)
	{
		if (c64)
			args.directional ? surf_build_kernel<PixC64, true, 4><<<blocks, threads, 0, stream>>>(args)
							 : surf_build_kernel<PixC64, false, 4><<<blocks, threads, 0, stream>>>(args);
		else
			args.directional ? surf_build_kernel<PixC32, true, 4><<<blocks, threads, 0, stream>>>(args)
							 : surf_build_kernel<PixC32, false, 4><<<blocks, threads, 0, stream>>>(args);
	}
	else if (c64)
		args.directional ? surf_build_kernel<PixC64, true, 1><<<blocks, threads, 0, stream>>>(args)
						 : surf_build_kernel<PixC64, false, 1><<<blocks, threads, 0, stream>>>(args);
	else
		args.directional ? surf_build_kernel<PixC32, true, 1><<<blocks, threads, 0, stream>>>(args)
						 : surf_build_kernel<PixC32, false, 1><<<blocks, threads, 0, stream>>>(args);
	return int(cudaGetLastError());
}

} // namespace swgpu
