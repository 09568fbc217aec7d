// Per-polygon steps of the renderer's frame preparation, shared by the host (frame.cpp, g++ with
// -ffp-contract=off) and the GPU-side preparation (csrc/prep.cu, nvcc with --fmad=false, IEEE division
// and square root). Every function is one expression sequence with the reference's operation order, so
// both compilers round every operation identically and the two paths produce the same bits.
//
// Restated here:
//   clip_3d_polygon_by_z_plane, clip_2d_polygon (src/common/clipping.rs:4-51, 115-175),
//   project_and_clip_polygon, affine / line-z interpolation tests, calculate_mip
//   (src/square_wheel/renderer_utils.rs:10-242),
//   prepare_polygon_surface (src/square_wheel/partial_renderer.rs:1464-1638),
//   the per-surface half of build_polygons_surfaces (:1682-1819) with polygon_is_affected_by_light
//   (:3877-3985), and draw_polygon's projection and mode selection (:4011-4142).
#pragma once

#include <stdint.h>

#include "../../include/swgpu.h"
#include "hmath.h"

namespace swhost
{

constexpr uint32_t PREP_MAX_VERTICES = SW_MAX_POLYGON_VERTICES; // renderer_utils.rs:4
constexpr float PREP_Z_NEAR = 1.0f;                             // renderer_utils.rs:7
constexpr float PREP_TC_ERROR_THRESHOLD = 0.75f;                // renderer_utils.rs:199
constexpr uint32_t PREP_MAX_MIP = 4;
constexpr uint32_t PREP_LIGHTMAP_SCALE_LOG2 = 4;
constexpr uint32_t PREP_NUM_MIPS = 5;

struct DepthEquation
{
	float d_inv_z_dx, d_inv_z_dy, k;
	SWH_HD float sample(Vec2 p) const { return d_inv_z_dx * p.x + d_inv_z_dy * p.y + k; }
};
struct TexCoordEquation
{
	float d_tc_dx[2], d_tc_dy[2], k[2];
};

// f32 -> integer `as` casts: truncating, saturating, NaN -> 0.
SWH_HD inline int32_t as_i32(float x)
{
	if (x != x) return 0;
	if (x >= 2147483648.0f) return INT32_MAX;
	if (x <= -2147483648.0f) return INT32_MIN;
	return int32_t(x);
}

// f32::log2 rounded to nearest: evaluated in double precision and rounded once, on both sides. The
// only consumers are ceil() decisions (mip level, z scale), which depend on the correctly rounded value.
SWH_HD inline float log2_rn(float x) { return float(log2(double(x))); }

// exp2 of an integer-valued (or infinite / NaN) float, as f32::exp2 gives it: exact.
SWH_HD inline float exp2_int(float e)
{
	if (e != e) return e;
	if (e < -150.0f) return 0.0f;
	if (e > 128.0f) return ldexpf(1.0f, 128); // +inf
	return ldexpf(1.0f, int(e));
}

// clip_3d_polygon_by_z_plane, clipping.rs:4-51
SWH_HD inline Vec3 line_z_intersection(Vec3 v0, Vec3 v1, float z)
{
	const float dist0 = v0.z - z, dist1 = v1.z - z, dist_sum = v1.z - v0.z;
	const float k0 = dist0 / dist_sum, k1 = dist1 / dist_sum;
	return v0 * k1 - v1 * k0;
}
SWH_HD inline uint32_t clip_3d_polygon_by_z_plane(const Vec3* polygon, uint32_t n, float z_dist, Vec3* out, uint32_t out_cap)
{
	if (n == 0) return 0;
	const Vec3* prev_v = &polygon[n - 1];
	uint32_t count = 0;
	for (uint32_t i = 0; i < n; ++i)
	{
		const Vec3& v = polygon[i];
		if (v.z > z_dist)
		{
			if (prev_v->z < z_dist)
			{
				out[count++] = line_z_intersection(*prev_v, v, z_dist);
				if (count == out_cap) break;
			}
			out[count++] = v;
			if (count == out_cap) break;
		}
		else if (v.z == z_dist)
		{
			out[count++] = v;
			if (count == out_cap) break;
		}
		else if (prev_v->z > z_dist)
		{
			out[count++] = line_z_intersection(*prev_v, v, z_dist);
			if (count == out_cap) break;
		}
		prev_v = &v;
	}
	return count;
}

// clip_2d_polygon, clipping.rs:115-175
SWH_HD inline Vec2 line_line_intersection(Vec2 v0, Vec2 v1, Vec3 line)
{
	const float dist0 = dot(v0, v2(line.x, line.y)) - line.z;
	const float dist1 = dot(v1, v2(line.x, line.y)) - line.z;
	const float dist_sum = dist1 - dist0;
	const float k0 = dist0 / dist_sum, k1 = dist1 / dist_sum;
	return v0 * k1 - v1 * k0;
}
SWH_HD inline uint32_t clip_2d_polygon(const Vec2* polygon, uint32_t n, Vec3 line, Vec2* out, uint32_t out_cap)
{
	const Vec2* prev_v = &polygon[n - 1];
	float prev_dist = dot(*prev_v, v2(line.x, line.y)) - line.z;
	uint32_t count = 0;
	for (uint32_t i = 0; i < n; ++i)
	{
		const Vec2& v = polygon[i];
		const float dist = dot(v, v2(line.x, line.y)) - line.z;
		if (dist > 0.0f)
		{
			if (prev_dist < 0.0f)
			{
				out[count++] = line_line_intersection(*prev_v, v, line);
				if (count == out_cap) break;
			}
			out[count++] = v;
			if (count == out_cap) break;
		}
		else if (dist == 0.0f)
		{
			out[count++] = v;
			if (count == out_cap) break;
		}
		else if (prev_dist > 0.0f)
		{
			out[count++] = line_line_intersection(*prev_v, v, line);
			if (count == out_cap) break;
		}
		prev_v = &v;
		prev_dist = dist;
	}
	return count;
}

// project_and_clip_polygon, renderer_utils.rs:10-58
SWH_HD inline uint32_t project_and_clip_polygon(const Vec3 clip_planes[8], const Vec3* vertices_transformed, uint32_t n, Vec2* out)
{
	uint32_t count = n < PREP_MAX_VERTICES ? n : PREP_MAX_VERTICES;
	Vec3 z_clipped[PREP_MAX_VERTICES];
	count = clip_3d_polygon_by_z_plane(vertices_transformed, count, PREP_Z_NEAR, z_clipped, PREP_MAX_VERTICES);
	if (count < 3) return count;
	for (uint32_t i = 0; i < count; ++i) out[i] = v2(z_clipped[i].x, z_clipped[i].y) / z_clipped[i].z;
	Vec2 temp[PREP_MAX_VERTICES];
	for (uint32_t i = 0; i < 4; ++i)
	{
		count = clip_2d_polygon(out, count, clip_planes[i * 2], temp, PREP_MAX_VERTICES);
		if (count < 3) return count;
		count = clip_2d_polygon(temp, count, clip_planes[i * 2 + 1], out, PREP_MAX_VERTICES);
		if (count < 3) return count;
	}
	return count;
}

// affine_texture_coordinates_interpolation_may_be_used, renderer_utils.rs:60-132
SWH_HD inline bool affine_may_be_used(const DepthEquation& de, const TexCoordEquation& te, Vec2 min_p, Vec2 max_p)
{
	const Vec2 edge = max_p - min_p;
	const float edge_square_len = dot(edge, edge);
	if (edge_square_len == 0.0f) return true;
	const float edge_len = sqrtf(edge_square_len);
	const Vec2 edge_vec_normalized = edge / edge_len;
	const float inv_z_clamp = 1.0f / float(1 << 20);
	const float min_point_inv_z = fmaxf(de.sample(min_p), inv_z_clamp);
	const float a = dot(v2(de.d_inv_z_dx, de.d_inv_z_dy), edge_vec_normalized);
	const float b = min_point_inv_z;
	if (fabsf(a) < 1.0e-10f) return true;
	const float b_div_a = b / a;
	const float max_diff_point = sqrtf((0.0f + b_div_a) * (edge_len + b_div_a)) - b_div_a;
	const float max_diff_point_inv_z = a * max_diff_point + b;
	for (int i = 0; i < 2; ++i)
	{
		const float min_point_tc = te.d_tc_dx[i] * min_p.x + te.d_tc_dy[i] * min_p.y + te.k[i];
		const float max_point_tc = te.d_tc_dx[i] * max_p.x + te.d_tc_dy[i] * max_p.y + te.k[i];
		const float tc_a = dot(v2(te.d_tc_dx[i], te.d_tc_dy[i]), edge_vec_normalized);
		const float tc_b = min_point_tc;
		const float min_point_tc_z_mul = min_point_tc / min_point_inv_z;
		const float max_point_tc_z_mul = max_point_tc / fmaxf(de.sample(max_p), inv_z_clamp);
		const float real = (tc_a * max_diff_point + tc_b) / max_diff_point_inv_z;
		const float approx =
			min_point_tc_z_mul + (max_point_tc_z_mul - min_point_tc_z_mul) * (max_diff_point - 0.0f) / (edge_len - 0.0f);
		if (fabsf(real - approx) > PREP_TC_ERROR_THRESHOLD) return false;
	}
	return true;
}

// line_z_corrected_texture_coordinates_interpolation_may_be_used, renderer_utils.rs:134-197
SWH_HD inline bool line_z_may_be_used(const DepthEquation& de, const TexCoordEquation& te, Vec2 max_p, float min_x, float max_x)
{
	if (max_x - min_x < 1.0f) return true;
	const float a = de.d_inv_z_dx;
	const float b = de.d_inv_z_dy * max_p.y + de.k;
	if (fabsf(a) < 1.0e-10f) return true;
	const float b_div_a = b / a;
	const float max_diff_x = sqrtf((min_x + b_div_a) * (max_x + b_div_a)) - b_div_a;
	const float max_diff_point_inv_z = a * max_diff_x + b;
	const float inv_z_at_min_x = a * min_x + b;
	const float inv_z_at_max_x = a * max_x + b;
	const float almost_zero = 1e-20f;
	if (inv_z_at_min_x <= almost_zero || inv_z_at_max_x <= almost_zero || max_diff_point_inv_z <= almost_zero) return false;
	for (int i = 0; i < 2; ++i)
	{
		const float ta = te.d_tc_dx[i];
		const float tb = te.d_tc_dy[i] * max_p.y + te.k[i];
		const float tc_at_min_x = (ta * min_x + tb) / inv_z_at_min_x;
		const float tc_at_max_x = (ta * max_x + tb) / inv_z_at_max_x;
		const float real = (ta * max_diff_x + tb) / max_diff_point_inv_z;
		const float approx = tc_at_min_x + (tc_at_max_x - tc_at_min_x) * (max_diff_x - min_x) / (max_x - min_x);
		if (fabsf(real - approx) > PREP_TC_ERROR_THRESHOLD) return false;
	}
	return true;
}

// calculate_mip, renderer_utils.rs:201-242
SWH_HD inline uint32_t calculate_mip(const Vec2* points, uint32_t n, const DepthEquation& de, const TexCoordEquation& te, float mip_bias)
{
	Vec2 mip_point = points[0];
	float mip_point_inv_z = 0.0f;
	for (uint32_t i = 0; i < n; ++i)
	{
		const float inv_z = de.sample(points[i]);
		if (inv_z > mip_point_inv_z)
		{
			mip_point_inv_z = inv_z;
			mip_point = points[i];
		}
	}
	const float z_2 = 1.0f / (mip_point_inv_z * mip_point_inv_z);
	const float z_4 = z_2 * z_2;
	float d_tc_2[2];
	for (int i = 0; i < 2; ++i)
	{
		const float d_tc_dx = te.d_tc_dx[i] * (de.k + de.d_inv_z_dy * mip_point.y) - (te.k[i] + te.d_tc_dy[i] * mip_point.y) * de.d_inv_z_dx;
		const float d_tc_dy = te.d_tc_dy[i] * (de.k + de.d_inv_z_dx * mip_point.x) - (te.k[i] + te.d_tc_dx[i] * mip_point.x) * de.d_inv_z_dy;
		d_tc_2[i] = (d_tc_dx * d_tc_dx + d_tc_dy * d_tc_dy) * z_4;
	}
	const float max_d_tc_2 = fmaxf(d_tc_2[0], d_tc_2[1]);
	const float mip_f = log2_rn(max_d_tc_2) * 0.5f + mip_bias;
	const int32_t m = as_i32(ceilf(mip_f));
	return uint32_t(m < 0 ? 0 : (m > int32_t(PREP_MAX_MIP) ? int32_t(PREP_MAX_MIP) : m));
}

// cgmath Matrix3::invert (cofactor form), then transpose; used by polygon_is_affected_by_light.
struct Mat3
{
	Vec3 c[3];
};
SWH_HD inline bool mat3_invert_transpose(Vec3 a, Vec3 b, Vec3 c, Mat3& out)
{
	const float det = dot(a, cross(b, c));
	if (det == 0.0f) return false;
	// inverse rows are cross products / det; transposed -> columns.
	out.c[0] = cross(b, c) / det;
	out.c[1] = cross(c, a) / det;
	out.c[2] = cross(a, b) / det;
	return true;
}

SWH_HD inline Vec3 poly_vec3(const float* f) { return v3(f[0], f[1], f[2]); }

// polygon_is_affected_by_light, partial_renderer.rs:3877-3985; `shadow` (may be null) is the light's
// shadow map: a projector's cone is tested against the polygon's texture-coordinate rectangle corners.
SWH_HD inline bool polygon_is_affected_by_light(const SwMapPolygon& polygon, const SwLight& light,
	const SwLightShadow* shadow = nullptr)
{
	const Vec3 lp = v3(light.position[0], light.position[1], light.position[2]);
	const Vec3 bu = poly_vec3(polygon.basis_u), bv = poly_vec3(polygon.basis_v), bn = poly_vec3(polygon.basis_normal);
	const Vec3 vec = lp - poly_vec3(polygon.basis_start);
	const float signed_distance = dot(vec, bn);
	if (signed_distance <= 0.0f) return false;
	const float square_radius = light.radius * light.radius - signed_distance * signed_distance;
	if (square_radius <= 0.0f) return false;
	if (shadow && shadow->kind == SW_SHADOW_PROJECTOR)
	{
		// the light pyramid's five planes against the (approximate) polygon corners (:3901-3944)
		const Vec3 start = poly_vec3(polygon.basis_start);
		const Vec3 u0 = bu * float(polygon.tex_coord_min[0]), u1 = bu * float(polygon.tex_coord_max[0]);
		const Vec3 v0 = bv * float(polygon.tex_coord_min[1]), v1 = bv * float(polygon.tex_coord_max[1]);
		const Vec3 corners[4] = {start + u0 + v0, start + u0 + v1, start + u1 + v0, start + u1 + v1};
		const Vec3 bx = poly_vec3(shadow->basis_x), by = poly_vec3(shadow->basis_y), bz = poly_vec3(shadow->basis_z);
		const Vec3 plane_vecs[5] = {bz, bz - bx, bz + bx, bz - by, bz + by};
		for (int k = 0; k < 5; ++k)
		{
			const float dist = dot(plane_vecs[k], lp);
			int front = 0;
			for (int c = 0; c < 4; ++c)
				if (dot(plane_vecs[k], corners[c]) >= dist) ++front;
			if (front >= 4) return false;
		}
		return true;
	}
	Mat3 m;
	if (!mat3_invert_transpose(bu, bv, bn, m)) return false;
	const float tc0 = dot(vec, m.c[0]), tc1 = dot(vec, m.c[1]);
	const float radius = sqrtf(square_radius);
	const float u_radius = radius * (1.0f / sqrtf(magnitude2(bu)));
	const float v_radius = radius * (1.0f / sqrtf(magnitude2(bv)));
	if (tc0 + u_radius < float(polygon.tex_coord_min[0]) || tc1 + v_radius < float(polygon.tex_coord_min[1]) ||
		tc0 - u_radius > float(polygon.tex_coord_max[0]) || tc1 - v_radius > float(polygon.tex_coord_max[1]))
		return false;
	return true;
}

// Result of prepare_polygon_surface for a polygon with a surface.
struct SurfacePrep
{
	DepthEquation depth;
	TexCoordEquation tc; // scaled for the mip and shifted to the surface's tc_min
	uint32_t size[2];
	uint32_t mip;
	int32_t tc_min[2];
};

enum PrepResult
{
	PREP_HIDDEN = 0,  // back-facing, not drawn, or clipped away
	PREP_SURFACE = 1, // visible: `out` holds the surface
	PREP_SKY = 2,     // visible sky polygon: v2d[0..count) is its projection
};

// DepthRenderer::draw_polygon::<false> + draw_depth_polygon (depth_renderer.rs:199-287), the part before
// the clipping: shadow-casting opaque polygons facing the side camera (materials_shadow_table, :20-38),
// and their depth equation (DepthEquation::from_transformed_plane_equation) with the constant and slope
// bias added and the whole scaled by 1 - 1/1024. False: the polygon draws nothing.
SWH_HD inline bool depth_map_equation(const SwMapPolygon& p, const Mat4& planes_matrix, float eq[3])
{
	if (!(p.flags & SW_POLY_SHADOW) || p.blending_mode != SW_BLEND_NONE) return false;
	const Vec4 pt = planes_matrix * extend(poly_vec3(p.plane), -p.plane[3]);
	if (pt.w <= 0.0f) return false;
	const float pw = -pt.w;
	const float d_inv_z_dx = pt.x / pw, d_inv_z_dy = pt.y / pw;
	const float DEPTH_BIAS_CONST = -1.0f / float(1 << 20), DEPTH_BIAS_SLOPE = -1.0f;
	const float DEPTH_EQUATION_SCALE = 1.0f - 1.0f / 1024.0f;
	eq[0] = DEPTH_EQUATION_SCALE * d_inv_z_dx;
	eq[1] = DEPTH_EQUATION_SCALE * d_inv_z_dy;
	eq[2] = DEPTH_EQUATION_SCALE * (pt.z / pw + DEPTH_BIAS_CONST + DEPTH_BIAS_SLOPE * (fabsf(d_inv_z_dx) + fabsf(d_inv_z_dy)));
	return true;
}

// prepare_polygon_surface, partial_renderer.rs:1464-1638. Transforms the polygon's first
// min(num_vertices, PREP_MAX_VERTICES) vertices into vt (the ones project_and_clip_polygon reads) and
// returns the projected, clipped polygon in v2d / *count.
SWH_HD inline PrepResult prepare_polygon_surface(const SwMapPolygon& p, const Vec3* map_vertices, const Mat4& view_matrix,
	const Mat4& planes_matrix, const Vec3 clip_planes[8], float mip_bias, Vec3* vt, Vec2* v2d, uint32_t* count_out, SurfacePrep& out)
{
	*count_out = 0;
	const Vec4 plane_transformed = planes_matrix * extend(poly_vec3(p.plane), -p.plane[3]);
	if (plane_transformed.w <= 0.0f) return PREP_HIDDEN;
	if (!(p.flags & SW_POLY_DRAW)) return PREP_HIDDEN;
	const uint32_t nv = p.num_vertices < PREP_MAX_VERTICES ? p.num_vertices : PREP_MAX_VERTICES;
	for (uint32_t i = 0; i < nv; ++i) vt[i] = view_transform(view_matrix, map_vertices[p.first_vertex + i]);
	const uint32_t count = project_and_clip_polygon(clip_planes, vt, nv, v2d);
	*count_out = count;
	if (count < 3) return PREP_HIDDEN;
	if (p.flags & SW_POLY_SKY) return PREP_SKY; // the sky bounds are collected by the caller (:1510-1528)

	// DepthEquation::from_transformed_plane_equation, equations.rs:23-31
	const float pw = -plane_transformed.w;
	const DepthEquation de{plane_transformed.x / pw, plane_transformed.y / pw, plane_transformed.z / pw};
	// tc equations, partial_renderer.rs:1536-1544, equations.rs:55-74
	const Vec4 tb[2] = {planes_matrix * extend(poly_vec3(p.tex_coord_equation[0]), p.tex_coord_equation[0][3]),
		planes_matrix * extend(poly_vec3(p.tex_coord_equation[1]), p.tex_coord_equation[1][3])};
	TexCoordEquation te;
	for (int i = 0; i < 2; ++i)
	{
		te.d_tc_dx[i] = tb[i].x + tb[i].w * de.d_inv_z_dx;
		te.d_tc_dy[i] = tb[i].y + tb[i].w * de.d_inv_z_dy;
		te.k[i] = tb[i].z + tb[i].w * de.k;
	}
	const uint32_t mip = calculate_mip(v2d, count, de, te, mip_bias);
	const float mip_scale = 1.0f / float(1u << mip);
	TexCoordEquation ts;
	for (int i = 0; i < 2; ++i)
	{
		ts.d_tc_dx[i] = te.d_tc_dx[i] * mip_scale;
		ts.d_tc_dy[i] = te.d_tc_dy[i] * mip_scale;
		ts.k[i] = te.k[i] * mip_scale;
	}
	const float inf = float(1 << 29);
	const float max_z = float(1 << 16);
	float tc_min[2] = {inf, inf}, tc_max[2] = {-inf, -inf};
	for (uint32_t k = 0; k < count; ++k)
	{
		const float inv_z = fmaxf(de.sample(v2d[k]), 1.0f / max_z);
		const float z = 1.0f / inv_z;
		for (int i = 0; i < 2; ++i)
		{
			const float tc = z * (ts.d_tc_dx[i] * v2d[k].x + ts.d_tc_dy[i] * v2d[k].y + ts.k[i]);
			if (tc < tc_min[i]) tc_min[i] = tc;
			if (tc > tc_max[i]) tc_max[i] = tc;
		}
	}
	for (int i = 0; i < 2; ++i)
	{
		const float eps = 1.0f / 32.0f;
		tc_min[i] += eps;
		tc_max[i] -= eps;
		const int32_t round_mask = ~int32_t((1u << PREP_LIGHTMAP_SCALE_LOG2) - 1);
		const int32_t min_down = (p.tex_coord_min[i] & round_mask) >> mip;
		const int32_t max_up = ((p.tex_coord_max[i] + int32_t(1u << PREP_LIGHTMAP_SCALE_LOG2) - 1) & round_mask) >> mip;
		int32_t tmin = as_i32(floorf(fmaxf(tc_min[i], -inf)));
		if (tmin < min_down) tmin = min_down;
		int32_t tmax = as_i32(ceilf(fminf(tc_max[i], inf)));
		if (tmax > max_up) tmax = max_up;
		if (tmin >= tmax)
		{
			if (tmin > max_up - 1) tmin = max_up - 1;
			tmax = tmin + 1;
		}
		out.tc_min[i] = tmin;
		out.size[i] = uint32_t(tmax - tmin);
	}
	out.depth = de;
	out.tc = ts;
	out.mip = mip;
	for (int i = 0; i < 2; ++i)
	{
		const float tmf = float(out.tc_min[i]);
		out.tc.d_tc_dx[i] -= tmf * de.d_inv_z_dx;
		out.tc.d_tc_dy[i] -= tmf * de.d_inv_z_dy;
		out.tc.k[i] -= tmf * de.k;
	}
	return PREP_SURFACE;
}

// Largest surface (texels) prepare_polygon_surface can give the polygon: per axis the mip-0 span of its
// lightmap-aligned tc bounds (at least 1). Capacity bound for the GPU-side preparation.
SWH_HD inline uint64_t max_surface_texels(const SwMapPolygon& p)
{
	uint64_t area = 1;
	for (int i = 0; i < 2; ++i)
	{
		const int64_t lo = int64_t(p.tex_coord_min[i] & ~int32_t(15));
		const int64_t hi = int64_t((p.tex_coord_max[i] + 15) & ~int32_t(15));
		area *= uint64_t(hi - lo > 1 ? hi - lo : 1);
	}
	return area;
}

// The descriptor half of build_polygons_surfaces for one surface (partial_renderer.rs:1682-1819), without
// its light list. `directional`: directional lightmaps in use; `simple_lightmaps`: the map has simple ones.
// `shift`: get_texture_shift of the polygon's material (texels of mip 0), applied >> mip
// (partial_renderer.rs:1687-1693); `texture`: the material's current animation frame (get_texture).
// `mf`: the polygon's material this frame (texture, scrolling shift, flags and emissive layer of the
// current animation frame), or NULL for the polygon's own material, unshifted.
SWH_HD inline void make_surface_desc(const SwMapPolygon& p, const SurfacePrep& sp, uint64_t out_offset, bool directional,
	bool simple_lightmaps, const SwMaterialFrame* mf, SwSurfaceDesc& d)
{
	d = SwSurfaceDesc{};
	const int32_t shift_mip[2] = {mf ? mf->shift[0] >> sp.mip : 0, mf ? mf->shift[1] >> sp.mip : 0};
	const uint32_t texture = mf ? mf->texture : p.texture, flags = mf ? mf->flags : p.flags;
	const uint32_t emissive_texture = mf ? mf->emissive_texture : p.emissive_texture;
	const float* emissive_light = mf ? mf->emissive_light : p.emissive_light;
	d.size[0] = sp.size[0];
	d.size[1] = sp.size[1];
	d.tc_start[0] = sp.tc_min[0] + shift_mip[0];
	d.tc_start[1] = sp.tc_min[1] + shift_mip[1];
	d.out_offset = out_offset;
	d.emissive_mip = SW_NO_EMISSIVE;
	if (flags & SW_POLY_DIFFUSE_LAYER)
	{
		d.flags = SW_SURF_DIFFUSE_LAYER;
		// get_basis_vecs_for_mip + texture shift correction (surfaces.rs:49-63, partial_renderer.rs:1736-1740)
		Vec3 bu = poly_vec3(p.basis_u), bv = poly_vec3(p.basis_v);
		if (sp.mip != 0)
		{
			const float scale = float(1u << sp.mip);
			bu = bu * scale;
			bv = bv * scale;
		}
		const Vec3 start = poly_vec3(p.basis_start) - (float(shift_mip[0]) * bu + float(shift_mip[1]) * bv);
		const Vec3 bn = poly_vec3(p.basis_normal);
		d.basis_u[0] = bu.x, d.basis_u[1] = bu.y, d.basis_u[2] = bu.z;
		d.basis_v[0] = bv.x, d.basis_v[1] = bv.y, d.basis_v[2] = bv.z;
		d.basis_start[0] = start.x, d.basis_start[1] = start.y, d.basis_start[2] = start.z;
		d.basis_normal[0] = bn.x, d.basis_normal[1] = bn.y, d.basis_normal[2] = bn.z;
		d.texture_mip = texture * PREP_NUM_MIPS + sp.mip;
		for (int i = 0; i < 2; ++i)
		{
			const int32_t round_mask = ~int32_t((1u << PREP_LIGHTMAP_SCALE_LOG2) - 1);
			d.lightmap_tc_shift[i] = uint32_t(sp.tc_min[i] - ((p.tex_coord_min[i] & round_mask) >> sp.mip));
		}
		// get_polygon_lightmap_size, lightmap.rs:11-27
		d.lightmap_size[0] = uint32_t(((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1);
		d.lightmap_size[1] = uint32_t(((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1);
		d.lightmap_scale_log2 = PREP_LIGHTMAP_SCALE_LOG2 - sp.mip;
		d.lightmap_offset = (directional || simple_lightmaps) ? p.lightmap_data_offset : SW_NO_LIGHTMAP;
	}
	if (emissive_texture != SW_NO_EMISSIVE)
	{
		d.emissive_mip = emissive_texture * PREP_NUM_MIPS + sp.mip;
		d.emissive_light[0] = emissive_light[0];
		d.emissive_light[1] = emissive_light[1];
		d.emissive_light[2] = emissive_light[2];
	}
}

// draw_polygon, partial_renderer.rs:4011-4142: projects and clips the transformed vertices against the
// leaf's draw bounds and selects the interpolation mode. Returns the vertex count (< 3: nothing drawn);
// fills `vertices` and every field of `d` but first_vertex.
SWH_HD inline uint32_t make_draw(const Vec3 clip_planes[8], const Vec3* vt, uint32_t num_vertices, const DepthEquation& depth,
	const TexCoordEquation& tc, uint32_t tex_w, uint32_t tex_h, uint64_t tex_offset, uint32_t tex_source, uint32_t blend,
	SwVertex16* vertices, SwDrawCmd& d)
{
	Vec2 v2d[PREP_MAX_VERTICES];
	const uint32_t count = project_and_clip_polygon(clip_planes, vt, num_vertices, v2d);
	if (count < 3) return count;
	float min_inv_z = 1e24f, max_inv_z = -1e24f, min_x = 1e24f, max_x = -1e24f;
	uint32_t min_i = 0, max_i = 0;
	for (uint32_t k = 0; k < count; ++k)
	{
		const float inv_z = depth.sample(v2d[k]);
		if (inv_z < min_inv_z)
		{
			min_inv_z = inv_z;
			min_i = k;
		}
		if (inv_z > max_inv_z)
		{
			max_inv_z = inv_z;
			max_i = k;
		}
		if (v2d[k].x < min_x) min_x = v2d[k].x;
		if (v2d[k].x > max_x) max_x = v2d[k].x;
	}
	d = SwDrawCmd{};
	d.vertex_count = count;
	for (uint32_t k = 0; k < count; ++k) // f32_to_fixed16_unchecked, fixed_math.rs:335-338
		vertices[k] = SwVertex16{as_i32(v2d[k].x * 65536.0f), as_i32(v2d[k].y * 65536.0f)};
	d.blend = blend;
	d.tex_size[0] = tex_w;
	d.tex_size[1] = tex_h;
	d.tex_source = tex_source;
	d.tex_offset = tex_offset;
	DepthEquation de = depth;
	TexCoordEquation te = tc;
	if (affine_may_be_used(depth, tc, v2d[min_i], v2d[max_i]))
		d.mode = SW_RASTER_AFFINE;
	else
	{
		const float z_scale = exp2_int(-5.0f - ceilf(log2_rn(fmaxf(max_inv_z, 1.0f / float(1 << 20)))));
		de = DepthEquation{de.d_inv_z_dx * z_scale, de.d_inv_z_dy * z_scale, de.k * z_scale};
		for (int i = 0; i < 2; ++i)
		{
			te.d_tc_dx[i] *= z_scale;
			te.d_tc_dy[i] *= z_scale;
			te.k[i] *= z_scale;
		}
		d.mode = line_z_may_be_used(depth, tc, v2d[max_i], min_x, max_x) ? SW_RASTER_LINE_Z_CORRECTED : SW_RASTER_FULL_PERSPECTIVE;
	}
	d.depth_eq[0] = de.d_inv_z_dx;
	d.depth_eq[1] = de.d_inv_z_dy;
	d.depth_eq[2] = de.k;
	for (int i = 0; i < 2; ++i)
	{
		d.tc_eq[i] = te.d_tc_dx[i];
		d.tc_eq[2 + i] = te.d_tc_dy[i];
		d.tc_eq[4 + i] = te.k[i];
	}
	return count;
}

} // namespace swhost
