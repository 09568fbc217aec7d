// Test infrastructure (oracle): CPU restatement of the reference's surface builder.
//
// Follows src/square_wheel/surfaces.rs:433-852 (build_surface_impl_6_static_params, all template
// parameter combinations as runtime switches), :903-971 (mix_surface_with_texture_impl),
// :973-1086 (lightmap element mixing), :1088-1154 (specular helpers), and the per-polygon driver
// src/square_wheel/partial_renderer.rs:1682-1831. Texture texel unpacking follows
// src/square_wheel/textures.rs:41-61.
//
// Deviation kept on purpose: the reference keeps one lightmap line in a fixed 19-element buffer
// (surfaces.rs:465-467, MAX_LIGHTMAP_SIZE + 2); maps whose lightmaps are wider than that (the batched
// surface workload with surfaces up to 512 texels) would overrun it, so the line buffer here is sized
// by the lightmap width. The arithmetic is unchanged.
#include "sw_oracle.h"
#include "sw_oracle_math.h"

#include <atomic>
#include <thread>
#include <vector>

namespace sworacle
{

namespace
{

const float NORMAL_UNPACK_SCALE = 1.0f / 127.0f; // textures.rs:46-49, 64-65

struct TexelUnpacked
{
	uint32_t diffuse;
	int32_t packed;
};

// PackedNormalRoughness::unpack, textures.rs:41-56 with upack_bytes_into_f32x4 (fast_math.rs:430-438)
inline void unpack_normal_roughness(int32_t b, Vec3& n, float& roughness)
{
	float r[4];
	for (int i = 0; i < 4; ++i)
	{
		int32_t shifted = int32_t(uint32_t(b) << (24 - i * 8)) >> 24;
		r[i] = float(shifted) * NORMAL_UNPACK_SCALE;
	}
	n = v3(r[0], r[1], r[2]);
	roughness = r[3];
}
inline float unpack_roughness(int32_t b) { return float(b >> 24) * NORMAL_UNPACK_SCALE; } // textures.rs:58-61

const float SQRT_7 = 2.645751311f;
const float PI_F = 3.14159265358979323846f;
const float SPEC_A = 2.0f * PI_F / SQRT_7; // surfaces.rs:1109
const float SPEC_B = PI_F * SQRT_7 / 2.0f; // surfaces.rs:1110
const float DIELECTRIC_ZERO_REFLECTIVITY = 0.04f;
const float DIELECTRIC_AVERAGE_REFLECTIVITY = DIELECTRIC_ZERO_REFLECTIVITY * 3.0f;
const float METAL_AVERAGE_SCHLICK_FACTOR = 0.5f;

// surfaces.rs:1088-1114 (the "new formula" branch is the one compiled)
inline float get_specular_intensity(float angle_cos, float inv_roughness)
{
	float x = (angle_cos - 1.0f) * inv_roughness;
	return inv_fast(f32_mul_add(x * x, SPEC_B, SPEC_A)) * inv_roughness;
}
// surfaces.rs:1116-1123
inline float get_fresnel_factor_base(float c)
{
	float omc = fmaxr(1.0f - c, 0.0f);
	float omc2 = omc * omc;
	return omc2 * omc2 * omc;
}
// surfaces.rs:1125-1141
inline float get_specular_k_dielectric(float f, float roughness)
{
	float fresnel = f32_mul_add(f, 1.0f - DIELECTRIC_ZERO_REFLECTIVITY, DIELECTRIC_ZERO_REFLECTIVITY);
	return f32_mul_add(fresnel, 1.0f - roughness, DIELECTRIC_AVERAGE_REFLECTIVITY * roughness);
}
// surfaces.rs:1143-1150
inline float get_specular_k_metal(float f, float roughness)
{
	return f32_mul_add(f, 1.0f - roughness, METAL_AVERAGE_SCHLICK_FACTOR * roughness);
}

enum
{
	SPEC_NONE = 0,
	SPEC_DIELECTRIC = 1,
	SPEC_METAL = 2
};

// Directional lightmap element (bsp_map_compact.rs:144-156); the simple element uses ambient only.
struct LmElem
{
	float ambient[3];
	Vec3 dir;
	float deviation;
	float color[3];
};

// LightmapElementOps::mix for both kinds (surfaces.rs:996-1004, 1022-1071): a*ratio + b*(1-ratio)
inline LmElem lm_mix(const LmElem& a, const LmElem& b, float ratio, bool directional)
{
	float omr = 1.0f - ratio;
	LmElem r;
	for (int i = 0; i < 3; ++i) r.ambient[i] = f32_mul_add(a.ambient[i], ratio, b.ambient[i] * omr);
	if (directional)
	{
		r.dir = v3(f32_mul_add(a.dir.x, ratio, b.dir.x * omr), f32_mul_add(a.dir.y, ratio, b.dir.y * omr),
			f32_mul_add(a.dir.z, ratio, b.dir.z * omr));
		r.deviation = f32_mul_add(a.deviation, ratio, b.deviation * omr);
		for (int i = 0; i < 3; ++i) r.color[i] = f32_mul_add(a.color[i], ratio, b.color[i] * omr);
	}
	else
	{
		r.dir = v3(0, 0, 0);
		r.deviation = 0;
		r.color[0] = r.color[1] = r.color[2] = 0;
	}
	return r;
}

inline LmElem lm_load(const SwCreateInfo* d, bool directional, uint64_t index)
{
	LmElem e;
	if (directional)
	{
		const SwDirectionalLightmapElement& s = d->directional_lightmaps[index];
		for (int i = 0; i < 3; ++i)
		{
			e.ambient[i] = s.ambient_light[i];
			e.color[i] = s.directional_light_color[i];
		}
		e.dir = v3(s.light_direction_vector_scaled[0], s.light_direction_vector_scaled[1],
			s.light_direction_vector_scaled[2]);
		e.deviation = s.directional_light_deviation;
	}
	else
	{
		for (int i = 0; i < 3; ++i)
		{
			e.ambient[i] = d->lightmaps[index * 3 + i];
			e.color[i] = 0;
		}
		e.dir = v3(0, 0, 0);
		e.deviation = 0;
	}
	return e;
}

inline int32_t rem_euclid(int32_t a, int32_t b)
{
	int32_t r = a % b;
	return r < 0 ? r + b : r;
}

// The frame's shadow maps (NULL shadows: every light unshadowed).
struct Shadows
{
	const SwLightShadow* shadows;
	uint32_t num;
	const float* texels;
	uint64_t num_texels;
};

// cube_shadow_map_side_fetch, light.rs:235-258. Returns 1 if in light, 0 if in shadow.
float cube_shadow_map_side_fetch(const float* side, uint32_t size, Vec3 vec)
{
	const float ONE_MINUS_EPS = 1.0f - 1.0f / 65536.0f;
	const float cubemap_size_f = float(size);
	const float depth = inv_fast(fmaxr(vec.z, MIN_POSITIVE_VALUE));
	const float half_depth = 0.5f * depth;
	const float u_f = fminr(fmaxr(f32_mul_add(vec.x, half_depth, 0.5f), 0.0f), ONE_MINUS_EPS) * cubemap_size_f;
	const float v_f = fminr(fmaxr(f32_mul_add(vec.y, half_depth, 0.5f), 0.0f), ONE_MINUS_EPS) * cubemap_size_f;
	const uint32_t u = uint32_t(u_f), v = uint32_t(v_f); // in [0, size): to_int_unchecked is a truncation
	const float value = side[u + v * size];
	return depth >= value ? 1.0f : 0.0f;
}

// projector_shadow_map_fetch, light.rs:261-294: 0 behind the projector or outside its map.
float projector_shadow_map_fetch(const SwLightShadow& m, const float* data, Vec3 vec)
{
	const Vec3 bx = v3(m.basis_x[0], m.basis_x[1], m.basis_x[2]);
	const Vec3 by = v3(m.basis_y[0], m.basis_y[1], m.basis_y[2]);
	const Vec3 bz = v3(m.basis_z[0], m.basis_z[1], m.basis_z[2]);
	const float z = vec3_dot(bz, vec);
	if (z <= 0.0f) return 0.0f;
	const float depth = inv_fast(z);
	const float half_depth = 0.5f * depth;
	const float size_f = float(m.size);
	const float u_f = f32_mul_add(vec3_dot(bx, vec), half_depth, 0.5f) * size_f;
	const float v_f = f32_mul_add(vec3_dot(by, vec), half_depth, 0.5f) * size_f;
	if (u_f < 0.0f || v_f < 0.0f || u_f >= size_f || v_f >= size_f) return 0.0f;
	const uint32_t u = uint32_t(u_f), v = uint32_t(v_f); // in [0, size): to_int_unchecked is a truncation
	return depth >= data[u + v * m.size] ? 1.0f : 0.0f;
}

// get_light_shadow_factor / cube_shadow_map_fetch, light.rs:185-233 (`vec` = light position - point).
float light_shadow_factor(const Shadows& sh, uint32_t light, Vec3 vec)
{
	if (sh.shadows && light < sh.num && sh.shadows[light].kind == SW_SHADOW_PROJECTOR)
		return projector_shadow_map_fetch(sh.shadows[light], sh.texels + sh.shadows[light].offset, vec);
	if (!sh.shadows || light >= sh.num || sh.shadows[light].kind != SW_SHADOW_CUBE) return 1.0f; // ShadowMap::None
	const SwLightShadow& m = sh.shadows[light];
	const uint64_t side_texels = uint64_t(m.size) * m.size;
	auto side = [&](uint32_t i) { return sh.texels + m.offset + i * side_texels; };
	const Vec3 a = v3(std::fabs(vec.x), std::fabs(vec.y), std::fabs(vec.z));
	if (a.x >= a.y && a.x >= a.z)
	{
		if (vec.x >= 0.0f) return cube_shadow_map_side_fetch(side(1), m.size, v3(-vec.y, vec.z, a.x));
		return cube_shadow_map_side_fetch(side(0), m.size, v3(vec.y, vec.z, a.x));
	}
	if (a.y >= a.x && a.y >= a.z)
	{
		if (vec.y >= 0.0f) return cube_shadow_map_side_fetch(side(3), m.size, v3(vec.x, vec.z, a.y));
		return cube_shadow_map_side_fetch(side(2), m.size, v3(-vec.x, vec.z, a.y));
	}
	if (vec.z >= 0.0f) return cube_shadow_map_side_fetch(side(5), m.size, v3(-vec.x, vec.y, a.z));
	return cube_shadow_map_side_fetch(side(4), m.size, v3(-vec.x, -vec.y, a.z));
}

template <class P>
void build_surface(const SwCreateInfo* data, const SwSurfaceDesc& s, const SwLight* lights, const Shadows& shadows,
	Vec3 cam_pos, bool use_directional, typename P::T* out)
{
	typedef typename P::T T;
	const SwTextureMip& tex = data->texture_mips[s.texture_mip];
	const uint64_t* tex_texels = data->texels + tex.offset;
	const bool use_normal_map = (tex.flags & SW_TEX_HAS_NORMAL_MAP) != 0;
	int spec = SPEC_NONE; // surfaces.rs:354-422
	if (tex.flags & SW_TEX_HAS_NON_ONE_ROUGHNESS) spec = (tex.flags & SW_TEX_IS_METAL) ? SPEC_METAL : SPEC_DIELECTRIC;

	const bool has_lightmap = s.lightmap_offset != SW_NO_LIGHTMAP; // surfaces.rs:140 (empty lightmap slice)
	const bool directional = use_directional;
	const uint32_t scale_log2 = s.lightmap_scale_log2;
	const bool use_dynamic_lights = s.num_lights > 0;

	const Vec3 u_vec = v3(s.basis_u[0], s.basis_u[1], s.basis_u[2]);
	const Vec3 v_vec = v3(s.basis_v[0], s.basis_v[1], s.basis_v[2]);
	const Vec3 basis_start = v3(s.basis_start[0], s.basis_start[1], s.basis_start[2]);
	const Vec3 basis_normal = v3(s.basis_normal[0], s.basis_normal[1], s.basis_normal[2]);

	// surfaces.rs:456-471
	const Vec3 start_pos = basis_start + u_vec * (float(s.tc_start[0]) + 0.5f) + v_vec * (float(s.tc_start[1]) + 0.5f);
	const Vec3 u_vec_normalized = u_vec * inv_sqrt_fast(fmaxr(vec3_len2(u_vec), MIN_POSITIVE_VALUE));
	const Vec3 v_vec_normalized = v_vec * inv_sqrt_fast(fmaxr(vec3_len2(v_vec), MIN_POSITIVE_VALUE));

	std::vector<LmElem> line_lightmap(has_lightmap ? s.lightmap_size[0] + 2 : 1);
	const float lightmap_scale_f = float(1u << (has_lightmap ? scale_log2 : 0));
	const float inv_lightmap_scale_f = 1.0f / lightmap_scale_f;
	const float k_shift = 0.5f * inv_lightmap_scale_f;
	const uint32_t lightmap_fetch_mask = (1u << (has_lightmap ? scale_log2 : 0)) - 1u;

	const int32_t tex_w = int32_t(tex.width), tex_h = int32_t(tex.height);

	for (uint32_t dst_v = 0; dst_v < s.size[1]; ++dst_v)
	{
		if (has_lightmap) // surfaces.rs:477-502
		{
			uint32_t lightmap_base_v = dst_v + s.lightmap_tc_shift[1];
			uint32_t lightmap_v = lightmap_base_v >> scale_log2;
			float k = f32_mul_add(float(lightmap_base_v & lightmap_fetch_mask), inv_lightmap_scale_f, k_shift);
			uint64_t base = uint64_t(s.lightmap_offset) + uint64_t(lightmap_v) * s.lightmap_size[0];
			for (uint32_t i = 0; i < s.lightmap_size[0]; ++i)
			{
				LmElem l0 = lm_load(data, directional, base + i);
				LmElem l1 = lm_load(data, directional, base + s.lightmap_size[0] + i);
				line_lightmap[i] = lm_mix(l1, l0, k, directional);
			}
		}

		T* dst_line = out + uint64_t(dst_v) * s.size[0];
		int32_t src_v = rem_euclid(s.tc_start[1] + int32_t(dst_v), tex_h);
		const uint64_t* src_line = tex_texels + uint64_t(src_v) * tex.width;
		int32_t src_u = rem_euclid(s.tc_start[0], tex_w);
		const Vec3 start_pos_v = vec3_scalar_mul_add(v_vec, float(dst_v), start_pos);
		for (uint32_t dst_u = 0; dst_u < s.size[0]; ++dst_u)
		{
			const Vec3 pos = vec3_scalar_mul_add(u_vec, float(dst_u), start_pos_v);
			const uint64_t texel = src_line[src_u];
			const uint32_t diffuse = uint32_t(texel);
			const int32_t packed = int32_t(uint32_t(texel >> 32));

			Vec3 texel_normal = v3(0.0f, 0.0f, 1.0f);
			float texel_roughness = 0.0f;
			if (use_normal_map)
				unpack_normal_roughness(packed, texel_normal, texel_roughness);
			else if (spec != SPEC_NONE)
				texel_roughness = unpack_roughness(packed);

			ColorVec total_light_albedo_modulated = cv_zero();
			ColorVec total_light_direct = cv_zero();
			if (has_lightmap) // surfaces.rs:536-679
			{
				uint32_t lightmap_base_u = dst_u + s.lightmap_tc_shift[0];
				uint32_t lightmap_u = lightmap_base_u >> scale_log2;
				const LmElem& l0 = line_lightmap[lightmap_u];
				const LmElem& l1 = line_lightmap[lightmap_u + 1];
				float k = f32_mul_add(float(lightmap_base_u & lightmap_fetch_mask), inv_lightmap_scale_f, k_shift);
				LmElem l_mixed = lm_mix(l1, l0, k, directional);

				if (spec == SPEC_NONE)
				{
					total_light_albedo_modulated = cv_from_f32x3_one(l_mixed.ambient);
					if (directional)
					{
						float dot = use_normal_map ? fmaxr(vec3_dot(l_mixed.dir, texel_normal), 0.0f) : l_mixed.dir.z;
						total_light_albedo_modulated =
							cv_mul_scalar_add(cv_from_f32x3(l_mixed.color), dot, total_light_albedo_modulated);
					}
				}
				else
				{
					Vec3 normal = use_normal_map ? texel_normal : v3(0.0f, 0.0f, 1.0f);
					Vec3 vec_to_camera = cam_pos - pos;
					Vec3 vec_to_camera_texture_space = v3(vec3_dot(vec_to_camera, u_vec_normalized),
						vec3_dot(vec_to_camera, v_vec_normalized), vec3_dot(vec_to_camera, basis_normal));
					float vec_to_camera_normal_dot = vec3_dot(vec_to_camera_texture_space, normal);
					Vec3 vec_to_camera_reflected = normal * (2.0f * vec_to_camera_normal_dot) - vec_to_camera_texture_space;
					float vec_to_camera_len2 = fmaxr(vec3_len2(vec_to_camera_reflected), MIN_POSITIVE_VALUE);
					float angle_cos = fmaxr(vec_to_camera_normal_dot * inv_sqrt_fast(vec_to_camera_len2), 0.0f);
					float fresnel_factor_base = get_fresnel_factor_base(angle_cos);
					float specular_k = spec == SPEC_DIELECTRIC ? get_specular_k_dielectric(fresnel_factor_base, texel_roughness)
																										 : get_specular_k_metal(fresnel_factor_base, texel_roughness);
					float one_minus_specular_k = 1.0f - specular_k;
					ColorVec constant_component = cv_from_f32x3(l_mixed.ambient);
					total_light_albedo_modulated = cv_scalar_mul(constant_component, one_minus_specular_k);
					total_light_direct = cv_scalar_mul(constant_component, specular_k);
					total_light_albedo_modulated.v[3] = 1.0f;

					if (directional)
					{
						float direction_vec_len2 = vec3_len2(l_mixed.dir);
						float direction_vec_len = direction_vec_len2 * inv_sqrt_fast(direction_vec_len2);
						float reflected_light_angle_cos = vec3_dot(vec_to_camera_reflected, l_mixed.dir) *
							inv_sqrt_fast(vec_to_camera_len2 * direction_vec_len2);
						float inv_roughness_corrected = fmaxr(inv_fast(texel_roughness + l_mixed.deviation), 0.75f);
						float specular_intensity = get_specular_intensity(reflected_light_angle_cos, inv_roughness_corrected);
						ColorVec dir_color = cv_from_f32x3(l_mixed.color);
						if (spec == SPEC_DIELECTRIC)
						{
							float diffuse_intensity = fmaxr(vec3_dot(l_mixed.dir, texel_normal), 0.0f);
							float light_intensity_diffuse = diffuse_intensity * one_minus_specular_k;
							total_light_albedo_modulated =
								cv_mul_scalar_add(dir_color, light_intensity_diffuse, total_light_albedo_modulated);
							float light_intensity_specular = specular_intensity * specular_k * direction_vec_len;
							total_light_direct = cv_mul_scalar_add(dir_color, light_intensity_specular, total_light_direct);
						}
						else
						{
							float scale_factor = specular_intensity * direction_vec_len;
							float light_intensity_modulated = one_minus_specular_k * scale_factor;
							total_light_albedo_modulated =
								cv_mul_scalar_add(dir_color, light_intensity_modulated, total_light_albedo_modulated);
							float light_intensity_direct = specular_k * scale_factor;
							total_light_direct = cv_mul_scalar_add(dir_color, light_intensity_direct, total_light_direct);
						}
					}
				}
			}

			if (use_dynamic_lights) // surfaces.rs:681-831
			{
				Vec3 normal = basis_normal;
				if (use_normal_map)
					normal = v3(f32_mul_add(texel_normal.x, u_vec_normalized.x,
									f32_mul_add(texel_normal.y, v_vec_normalized.x, texel_normal.z * basis_normal.x)),
						f32_mul_add(texel_normal.x, u_vec_normalized.y,
							f32_mul_add(texel_normal.y, v_vec_normalized.y, texel_normal.z * basis_normal.y)),
						f32_mul_add(texel_normal.x, u_vec_normalized.z,
							f32_mul_add(texel_normal.y, v_vec_normalized.z, texel_normal.z * basis_normal.z)));

				Vec3 vec_to_camera_reflected = v3(0, 0, 0);
				float vec_to_camera_len2 = MIN_POSITIVE_VALUE;
				float specular_k = 0.0f;
				float inv_roughness = 0.0f;
				if (spec != SPEC_NONE)
				{
					Vec3 vec_to_camera = cam_pos - pos;
					float vec_to_camera_normal_dot = vec3_dot(vec_to_camera, normal);
					vec_to_camera_reflected = normal * (2.0f * vec_to_camera_normal_dot) - vec_to_camera;
					vec_to_camera_len2 = fmaxr(vec3_len2(vec_to_camera_reflected), MIN_POSITIVE_VALUE);
					float angle_cos = fmaxr(vec_to_camera_normal_dot * inv_sqrt_fast(vec_to_camera_len2), 0.0f);
					float fresnel_factor_base = get_fresnel_factor_base(angle_cos);
					specular_k = spec == SPEC_DIELECTRIC ? get_specular_k_dielectric(fresnel_factor_base, texel_roughness)
																							: get_specular_k_metal(fresnel_factor_base, texel_roughness);
					inv_roughness = inv_fast(texel_roughness);
				}

				for (uint32_t li = 0; li < s.num_lights; ++li)
				{
					const SwLight& light = lights[s.lights[li]];
					Vec3 vec_to_light = v3(light.position[0], light.position[1], light.position[2]) - pos;
					const float shadow_factor = light_shadow_factor(shadows, s.lights[li], vec_to_light); // light.rs:185-194
					float vec_to_light_len2 = fmaxr(vec3_len2(vec_to_light), MIN_POSITIVE_VALUE);
					float distance_factor = fmaxr(inv_fast(vec_to_light_len2) - light.inv_square_radius, 0.0f);
					float shadow_distance_factor = shadow_factor * distance_factor;
					float diffuse_intensity = 0.0f;
					if (spec != SPEC_METAL)
						diffuse_intensity = fmaxr(vec3_dot(normal, vec_to_light) * inv_sqrt_fast(vec_to_light_len2), 0.0f);
					float specular_intensity = 0.0f;
					if (spec != SPEC_NONE)
					{
						float c = vec3_dot(vec_to_camera_reflected, vec_to_light) *
							inv_sqrt_fast(vec_to_camera_len2 * vec_to_light_len2);
						specular_intensity = get_specular_intensity(c, inv_roughness);
					}
					ColorVec light_color = cv_from_f32x3(light.color);
					if (spec == SPEC_NONE)
					{
						total_light_albedo_modulated = cv_mul_scalar_add(
							light_color, diffuse_intensity * shadow_distance_factor, total_light_albedo_modulated);
					}
					else if (spec == SPEC_DIELECTRIC)
					{
						float light_intensity_diffuse = diffuse_intensity * (1.0f - specular_k) * shadow_distance_factor;
						total_light_albedo_modulated =
							cv_mul_scalar_add(light_color, light_intensity_diffuse, total_light_albedo_modulated);
						float light_intensity_specular = specular_intensity * specular_k * shadow_distance_factor;
						total_light_direct = cv_mul_scalar_add(light_color, light_intensity_specular, total_light_direct);
					}
					else
					{
						float sisdf = specular_intensity * shadow_distance_factor;
						float light_intensity_modulated = (1.0f - specular_k) * sisdf;
						total_light_albedo_modulated =
							cv_mul_scalar_add(light_color, light_intensity_modulated, total_light_albedo_modulated);
						float light_intensity_direct = specular_k * sisdf;
						total_light_direct = cv_mul_scalar_add(light_color, light_intensity_direct, total_light_direct);
					}
				}
			}

			// surfaces.rs:833-842
			ColorVec result_color = cv_mul(cv_from_c32(diffuse), total_light_albedo_modulated);
			if (spec != SPEC_NONE) result_color = cv_mul_scalar_add(total_light_direct, 255.0f, result_color);
			dst_line[dst_u] = P::from_vec(result_color);

			src_u += 1;
			if (src_u == tex_w) src_u = 0;
		}
	}
}

// mix_surface_with_texture_impl, surfaces.rs:903-971
template <class P>
void mix_surface_with_texture(const SwCreateInfo* data, const SwSurfaceDesc& s, uint32_t blend, typename P::T* out)
{
	typedef typename P::T T;
	const SwEmissiveMip& em = data->emissive_mips[s.emissive_mip];
	const uint32_t* pixels = data->emissive_pixels + em.offset;
	const float light_scale = float(1 << 8);
	const float light_scaled[3] = {
		s.emissive_light[0] * light_scale, s.emissive_light[1] * light_scale, s.emissive_light[2] * light_scale};
	const ColorVecI light_vec = ci_from_f32x3(light_scaled);
	const int32_t w = int32_t(em.width), h = int32_t(em.height);
	for (uint32_t dst_v = 0; dst_v < s.size[1]; ++dst_v)
	{
		T* dst_line = out + uint64_t(dst_v) * s.size[0];
		int32_t src_v = rem_euclid(s.tc_start[1] + int32_t(dst_v), h);
		const uint32_t* src_line = pixels + uint64_t(src_v) * em.width;
		int32_t src_u = rem_euclid(s.tc_start[0], w);
		for (uint32_t x = 0; x < s.size[0]; ++x)
		{
			uint32_t texel = src_line[src_u];
			ColorVecI modulated = ci_shr(ci_mul(ci_from_c32(texel), light_vec), 8);
			T& dst = dst_line[x];
			switch (blend)
			{
			case SW_BLEND_NONE: dst = P::from_veci(modulated); break;
			case SW_BLEND_AVERAGE: dst = P::from_veci(ci_shr(ci_add(modulated, P::to_veci(dst)), 1)); break;
			case SW_BLEND_ADDITIVE: dst = P::from_veci(ci_add(modulated, P::to_veci(dst))); break;
			case SW_BLEND_ALPHA_TEST:
				if (C32::test_alpha(texel)) dst = P::from_veci(modulated);
				break;
			case SW_BLEND_ALPHA_BLEND:
			{
				int32_t alpha = C32::get_alpha(texel);
				dst = P::from_veci(
					ci_shr(ci_add(ci_mul_scalar(modulated, alpha), ci_mul_scalar(P::to_veci(dst), wsub(255, alpha))), 8));
				break;
			}
			}
			src_u += 1;
			if (src_u == w) src_u = 0;
		}
	}
}

template <class P>
void build_one(const SwCreateInfo* data, const SwSurfaceDesc& s, const SwLight* lights, const Shadows& shadows,
	Vec3 cam_pos, bool use_directional, void* arena)
{
	typename P::T* out = static_cast<typename P::T*>(arena) + s.out_offset;
	const bool diffuse_layer = (s.flags & SW_SURF_DIFFUSE_LAYER) != 0;
	if (diffuse_layer) build_surface<P>(data, s, lights, shadows, cam_pos, use_directional, out);
	if (s.emissive_mip != SW_NO_EMISSIVE)
		mix_surface_with_texture<P>(data, s, diffuse_layer ? SW_BLEND_ADDITIVE : SW_BLEND_NONE, out);
}

} // namespace

} // namespace sworacle

using namespace sworacle;

extern "C" int orc_build_surfaces(const SwCreateInfo* data, const SwSurfaceDesc* surfaces, uint32_t num_surfaces,
	const SwLight* lights, uint32_t num_lights, const SwLightShadow* shadows, const float* shadow_texels,
	uint64_t shadow_texel_count, const SwFrameParams* frame, void* arena, uint64_t arena_texels, uint32_t num_threads)
{
	if (!data || !frame || (!surfaces && num_surfaces) || (!arena && num_surfaces)) return SW_ERR_INVALID_ARGUMENT;
	const Shadows sh{shadows, shadows ? num_lights : 0u, shadow_texels, shadow_texel_count};
	for (uint32_t l = 0; l < sh.num; ++l)
		if (shadows[l].kind == SW_SHADOW_CUBE &&
			(shadows[l].size == 0 || !shadow_texels || shadows[l].offset + 6 * uint64_t(shadows[l].size) * shadows[l].size > shadow_texel_count))
			return SW_ERR_INVALID_ARGUMENT;
	for (uint32_t i = 0; i < num_surfaces; ++i)
	{
		const SwSurfaceDesc& s = surfaces[i];
		if (s.texture_mip >= data->num_texture_mips) return SW_ERR_INVALID_ARGUMENT;
		if (s.emissive_mip != SW_NO_EMISSIVE && s.emissive_mip >= data->num_emissive_mips) return SW_ERR_INVALID_ARGUMENT;
		if (s.out_offset + uint64_t(s.size[0]) * s.size[1] > arena_texels) return SW_ERR_INVALID_ARGUMENT;
		if (s.num_lights > SW_MAX_POLYGON_LIGHTS) return SW_ERR_INVALID_ARGUMENT;
		for (uint32_t l = 0; l < s.num_lights; ++l)
			if (s.lights[l] >= num_lights) return SW_ERR_INVALID_ARGUMENT;
		if (s.lightmap_offset != SW_NO_LIGHTMAP && s.lightmap_scale_log2 > 4) return SW_ERR_INVALID_ARGUMENT;
	}
	const Vec3 cam = v3(frame->cam_pos[0], frame->cam_pos[1], frame->cam_pos[2]);
	const bool dir = frame->use_directional_lightmaps != 0;
	auto work = [&](uint32_t i) {
		if (frame->pixel_format == SW_PIXEL_C64)
			build_one<C64>(data, surfaces[i], lights, sh, cam, dir, arena);
		else
			build_one<C32>(data, surfaces[i], lights, sh, cam, dir, arena);
	};
	if (num_threads <= 1)
	{
		for (uint32_t i = 0; i < num_surfaces; ++i) work(i);
	}
	else
	{
		std::atomic<uint32_t> next(0);
		std::vector<std::thread> pool;
		for (uint32_t t = 0; t < num_threads; ++t)
			pool.emplace_back([&]() {
				for (;;)
				{
					uint32_t i = next.fetch_add(1);
					if (i >= num_surfaces) break;
					work(i);
				}
			});
		for (auto& th : pool) th.join();
	}
	return SW_OK;
}
