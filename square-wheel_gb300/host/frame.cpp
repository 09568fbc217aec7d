// Per-frame host work (see frame.h). Compiled with -ffp-contract=off: every float expression is
// evaluated with the reference's operation order and rounding.
#include "frame.h"

#include <algorithm>
#include <cstring>

namespace swhost
{

namespace
{

constexpr uint32_t MAX_VERTICES = SW_MAX_POLYGON_VERTICES; // renderer_utils.rs:4
constexpr float Z_NEAR = 1.0f;                             // renderer_utils.rs:7
constexpr float TC_ERROR_THRESHOLD = 0.75f;                // renderer_utils.rs:199
constexpr uint32_t MAX_POLYGON_LIGHTS = SW_MAX_POLYGON_LIGHTS;
constexpr uint32_t MAX_BSP_TREE_DEPTH = 72;                // bsp_builder.rs:53
constexpr uint32_t MAX_MIP = 4;

// f32 -> integer `as` casts: truncating, saturating, NaN -> 0.
int32_t as_i32(float x)
{
	if (x != x) return 0;
	if (x >= 2147483648.0f) return INT32_MAX;
	if (x <= -2147483648.0f) return INT32_MIN;
	return int32_t(x);
}

// clip_3d_polygon_by_z_plane, clipping.rs:4-51
Vec3 line_z_intersection(Vec3 v0, Vec3 v1, float z)
{
	const float dist0 = v0.z - z, dist1 = v1.z - z, dist_sum = v1.z - v0.z;
	const float k0 = dist0 / dist_sum, k1 = dist1 / dist_sum;
	return v0 * k1 - v1 * k0;
}
uint32_t clip_3d_polygon_by_z_plane(const Vec3* polygon, uint32_t n, float z_dist, Vec3* out, uint32_t out_cap)
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
Vec2 line_line_intersection(Vec2 v0, Vec2 v1, Vec3 line)
{
	const float dist0 = dot(v0, v2(line.x, line.y)) - line.z;
	const float dist1 = dot(v1, v2(line.x, line.y)) - line.z;
	const float dist_sum = dist1 - dist0;
	const float k0 = dist0 / dist_sum, k1 = dist1 / dist_sum;
	return v0 * k1 - v1 * k0;
}
uint32_t clip_2d_polygon(const Vec2* polygon, uint32_t n, Vec3 line, Vec2* out, uint32_t out_cap)
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
uint32_t project_and_clip_polygon(const Vec3 clip_planes[8], const Vec3* vertices_transformed, uint32_t n, Vec2* out)
{
	uint32_t count = std::min(n, MAX_VERTICES);
	Vec3 z_clipped[MAX_VERTICES];
	count = clip_3d_polygon_by_z_plane(vertices_transformed, count, Z_NEAR, z_clipped, MAX_VERTICES);
	if (count < 3) return count;
	for (uint32_t i = 0; i < count; ++i) out[i] = v2(z_clipped[i].x, z_clipped[i].y) / z_clipped[i].z;
	Vec2 temp[MAX_VERTICES];
	for (uint32_t i = 0; i < 4; ++i)
	{
		count = clip_2d_polygon(out, count, clip_planes[i * 2], temp, MAX_VERTICES);
		if (count < 3) return count;
		count = clip_2d_polygon(temp, count, clip_planes[i * 2 + 1], out, MAX_VERTICES);
		if (count < 3) return count;
	}
	return count;
}

// affine_texture_coordinates_interpolation_may_be_used, renderer_utils.rs:60-132
bool affine_may_be_used(const DepthEquation& de, const TexCoordEquation& te, Vec2 min_p, Vec2 max_p)
{
	const Vec2 edge = max_p - min_p;
	const float edge_square_len = dot(edge, edge);
	if (edge_square_len == 0.0f) return true;
	const float edge_len = std::sqrt(edge_square_len);
	const Vec2 edge_vec_normalized = edge / edge_len;
	const float inv_z_clamp = 1.0f / float(1 << 20);
	const float min_point_inv_z = std::fmax(de.sample(min_p), inv_z_clamp);
	const float max_point_inv_z = std::fmax(de.sample(max_p), inv_z_clamp);
	(void)max_point_inv_z;
	const float a = dot(v2(de.d_inv_z_dx, de.d_inv_z_dy), edge_vec_normalized);
	const float b = min_point_inv_z;
	if (std::fabs(a) < 1.0e-10f) return true;
	const float b_div_a = b / a;
	const float max_diff_point = std::sqrt((0.0f + b_div_a) * (edge_len + b_div_a)) - b_div_a;
	const float max_diff_point_inv_z = a * max_diff_point + b;
	for (int i = 0; i < 2; ++i)
	{
		const float min_point_tc = te.d_tc_dx[i] * min_p.x + te.d_tc_dy[i] * min_p.y + te.k[i];
		const float max_point_tc = te.d_tc_dx[i] * max_p.x + te.d_tc_dy[i] * max_p.y + te.k[i];
		const float tc_a = dot(v2(te.d_tc_dx[i], te.d_tc_dy[i]), edge_vec_normalized);
		const float tc_b = min_point_tc;
		const float min_point_tc_z_mul = min_point_tc / min_point_inv_z;
		const float max_point_tc_z_mul = max_point_tc / std::fmax(de.sample(max_p), inv_z_clamp);
		const float real = (tc_a * max_diff_point + tc_b) / max_diff_point_inv_z;
		const float approx =
			min_point_tc_z_mul + (max_point_tc_z_mul - min_point_tc_z_mul) * (max_diff_point - 0.0f) / (edge_len - 0.0f);
		if (std::fabs(real - approx) > TC_ERROR_THRESHOLD) return false;
	}
	return true;
}

// line_z_corrected_texture_coordinates_interpolation_may_be_used, renderer_utils.rs:134-197
bool line_z_may_be_used(const DepthEquation& de, const TexCoordEquation& te, Vec2 max_p, float min_x, float max_x)
{
	if (max_x - min_x < 1.0f) return true;
	const float a = de.d_inv_z_dx;
	const float b = de.d_inv_z_dy * max_p.y + de.k;
	if (std::fabs(a) < 1.0e-10f) return true;
	const float b_div_a = b / a;
	const float max_diff_x = std::sqrt((min_x + b_div_a) * (max_x + b_div_a)) - b_div_a;
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
		if (std::fabs(real - approx) > TC_ERROR_THRESHOLD) return false;
	}
	return true;
}

// calculate_mip, renderer_utils.rs:201-242
uint32_t calculate_mip(const Vec2* points, uint32_t n, const DepthEquation& de, const TexCoordEquation& te, float mip_bias)
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
	const float max_d_tc_2 = std::fmax(d_tc_2[0], d_tc_2[1]);
	const float mip_f = std::log2(max_d_tc_2) * 0.5f + mip_bias;
	return uint32_t(std::max(0, std::min(as_i32(std::ceil(mip_f)), int32_t(MAX_MIP))));
}

struct Mat3
{
	Vec3 c[3];
};
// cgmath Matrix3::invert (cofactor form), then transpose; used by polygon_is_affected_by_light.
bool mat3_invert_transpose(Vec3 a, Vec3 b, Vec3 c, Mat3& out)
{
	const float det = dot(a, cross(b, c));
	if (det == 0.0f) return false;
	// inverse rows are cross products / det; transposed -> columns.
	out.c[0] = cross(b, c) / det;
	out.c[1] = cross(c, a) / det;
	out.c[2] = cross(a, b) / det;
	return true;
}

} // namespace

// ---- ClippingPolygon (clipping_polygon.rs) ----
ClippingPolygon ClippingPolygon::from_box(float min_x, float min_y, float max_x, float max_y)
{
	return ClippingPolygon{{min_x, max_x}, {min_y, max_y}, {min_x + min_y, max_x + max_y}, {min_x - max_y, max_x - min_y}};
}
ClippingPolygon ClippingPolygon::from_point(Vec2 p)
{
	return ClippingPolygon{{p.x, p.x}, {p.y, p.y}, {p.x + p.y, p.x + p.y}, {p.x - p.y, p.x - p.y}};
}
static bool axis_valid(const ClipAxis& a) { return a.min < a.max; }
bool ClippingPolygon::is_valid_and_non_empty() const
{
	return axis_valid(x) && axis_valid(y) && axis_valid(x_plus_y) && axis_valid(x_minus_y);
}
static bool axis_contains(const ClipAxis& a, const ClipAxis& o) { return o.min >= a.min && o.max <= a.max; }
bool ClippingPolygon::contains(const ClippingPolygon& o) const
{
	return axis_contains(x, o.x) && axis_contains(y, o.y) && axis_contains(x_plus_y, o.x_plus_y) &&
		axis_contains(x_minus_y, o.x_minus_y);
}
static void axis_extend(ClipAxis& a, const ClipAxis& o)
{
	if (o.min < a.min) a.min = o.min;
	if (o.max > a.max) a.max = o.max;
}
void ClippingPolygon::extend(const ClippingPolygon& o)
{
	axis_extend(x, o.x);
	axis_extend(y, o.y);
	axis_extend(x_plus_y, o.x_plus_y);
	axis_extend(x_minus_y, o.x_minus_y);
}
static void axis_point(ClipAxis& a, float p)
{
	if (p < a.min) a.min = p;
	if (p > a.max) a.max = p;
}
void ClippingPolygon::extend_with_point(Vec2 p)
{
	axis_point(x, p.x);
	axis_point(y, p.y);
	axis_point(x_plus_y, p.x + p.y);
	axis_point(x_minus_y, p.x - p.y);
}
static void axis_intersect(ClipAxis& a, const ClipAxis& o)
{
	if (o.min > a.min) a.min = o.min;
	if (o.max < a.max) a.max = o.max;
}
void ClippingPolygon::intersect(const ClippingPolygon& o)
{
	axis_intersect(x, o.x);
	axis_intersect(y, o.y);
	axis_intersect(x_plus_y, o.x_plus_y);
	axis_intersect(x_minus_y, o.x_minus_y);
}
void ClippingPolygon::get_clip_planes(Vec3 out[8]) const
{
	out[0] = v3(-1.0f, 0.0f, -x.max);
	out[1] = v3(1.0f, 0.0f, x.min);
	out[2] = v3(0.0f, -1.0f, -y.max);
	out[3] = v3(0.0f, 1.0f, y.min);
	out[4] = v3(-1.0f, -1.0f, -x_plus_y.max);
	out[5] = v3(1.0f, 1.0f, x_plus_y.min);
	out[6] = v3(-1.0f, 1.0f, -x_minus_y.max);
	out[7] = v3(1.0f, -1.0f, x_minus_y.min);
}

// ---- FramePrep ----
FramePrep::FramePrep(const Scene& scene) : sc(scene)
{
	leaf_data.resize(sc.leafs.size());
	portal_data.resize(sc.portals.size());
	poly.resize(sc.polygons.size());
	vertices_transformed.resize(sc.vertices.size());
	leaf_lights.resize(sc.leafs.size());
}

uint32_t FramePrep::find_current_leaf() const
{
	// map_visibility_calculator.rs:133-155
	uint32_t index = sc.root_node();
	const Vec4 w_row = cam.planes_matrix.row(3);
	for (uint32_t guard = 0; guard < 100000; ++guard)
	{
		if (index >= FIRST_LEAF_INDEX) return index - FIRST_LEAF_INDEX;
		const BspNode& node = sc.nodes[index];
		const float w = dot(w_row, extend(node.plane.vec, -node.plane.dist));
		index = w >= 0.0f ? node.children[0] : node.children[1];
	}
	return 0;
}

bool FramePrep::project_portal(const MapPortal& portal, ClippingPolygon& out) const
{
	// map_visibility_calculator.rs:286-326
	uint32_t count = std::min(portal.num_vertices, MAX_VERTICES);
	Vec3 transformed[MAX_VERTICES], clipped[MAX_VERTICES];
	for (uint32_t i = 0; i < count; ++i) transformed[i] = view_transform(cam.view_matrix, sc.vertices[portal.first_vertex + i]);
	count = clip_3d_polygon_by_z_plane(transformed, count, 1.0f / 4096.0f, clipped, MAX_VERTICES);
	if (count < 3) return false;
	out = ClippingPolygon::from_point(v2(clipped[0].x, clipped[0].y) / clipped[0].z);
	for (uint32_t i = 1; i < count; ++i) out.extend_with_point(v2(clipped[i].x, clipped[i].y) / clipped[i].z);
	return true;
}

void FramePrep::mark_reachable_leafs(const uint32_t* start, uint32_t n, const ClippingPolygon& start_bounds)
{
	// map_visibility_calculator.rs:157-267
	wave0.clear();
	wave1.clear();
	for (uint32_t i = 0; i < n; ++i)
	{
		wave0.push_back(start[i]);
		leaf_data[start[i]].bounds = start_bounds;
		leaf_data[start[i]].visible_frame = current_frame;
	}
	uint32_t depth = 0;
	while (!wave0.empty())
	{
		for (uint32_t leaf : wave0)
		{
			const ClippingPolygon leaf_bounds = leaf_data[leaf].bounds;
			const BspLeaf& lv = sc.leafs[leaf];
			for (uint32_t k = 0; k < lv.num_leaf_portals; ++k)
			{
				const uint32_t portal = sc.leafs_portals[lv.first_leaf_portal + k];
				const MapPortal& pv = sc.portals[portal];
				const float portal_plane_pos = (cam.planes_matrix * extend(pv.plane.vec, -pv.plane.dist)).w;
				uint32_t next_leaf;
				if (pv.leafs[0] == leaf)
				{
					if (portal_plane_pos <= 0.0f) continue;
					next_leaf = pv.leafs[1];
				}
				else
				{
					if (portal_plane_pos >= 0.0f) continue;
					next_leaf = pv.leafs[0];
				}
				PortalData& pd = portal_data[portal];
				if (pd.visible_frame != current_frame)
				{
					pd.visible_frame = current_frame;
					pd.has_projection = project_portal(pv, pd.projection);
				}
				if (!pd.has_projection) continue;
				ClippingPolygon b = pd.projection;
				b.intersect(leaf_bounds);
				if (!b.is_valid_and_non_empty()) continue;
				LeafData& nd = leaf_data[next_leaf];
				if (nd.visible_frame != current_frame)
				{
					nd.visible_frame = current_frame;
					nd.bounds = b;
				}
				else
				{
					if (nd.bounds.contains(b)) continue;
					nd.bounds.extend(b);
				}
				wave1.push_back(next_leaf);
			}
		}
		wave0.clear();
		std::swap(wave0, wave1);
		if (++depth > 1024) break;
	}
}

void FramePrep::update_visibility(const ClippingPolygon& frame_bounds)
{
	// map_visibility_calculator.rs:52-97
	const uint32_t current_leaf = find_current_leaf();
	stats.camera_leaf = current_leaf;
	uint32_t start[32];
	uint32_t n = 1;
	start[0] = current_leaf;
	const BspLeaf& lv = sc.leafs[current_leaf];
	for (uint32_t k = 0; k < lv.num_leaf_portals; ++k)
	{
		const MapPortal& pv = sc.portals[sc.leafs_portals[lv.first_leaf_portal + k]];
		const float scaled_dist = dot(pv.plane.vec, cam.position) - pv.plane.dist;
		const float eps = Z_NEAR * 2.0f;
		if (std::fabs(scaled_dist) <= eps * magnitude(pv.plane.vec))
		{
			start[n++] = pv.leafs[0] == current_leaf ? pv.leafs[1] : pv.leafs[0];
			if (n == 32) break;
		}
	}
	mark_reachable_leafs(start, n, frame_bounds);
}

void FramePrep::position_sphere(uint32_t id, Vec3 center, float radius, uint32_t node_index)
{
	// position_object_sphere_r, dynamic_objects_index.rs:206-241
	if (node_index >= FIRST_LEAF_INDEX)
	{
		leaf_lights[node_index - FIRST_LEAF_INDEX].push_back(id);
		return;
	}
	const BspNode& node = sc.nodes[node_index];
	const float scaled_radius = radius * magnitude(node.plane.vec);
	const float scaled_dist = dot(center, node.plane.vec);
	if (scaled_dist + scaled_radius >= node.plane.dist) position_sphere(id, center, radius, node.children[0]);
	if (scaled_dist - scaled_radius <= node.plane.dist) position_sphere(id, center, radius, node.children[1]);
}

void FramePrep::position_lights()
{
	for (auto& l : leaf_lights) l.clear();
	for (uint32_t i = 0; i < lights.size(); ++i)
		position_sphere(i, v3(lights[i].position[0], lights[i].position[1], lights[i].position[2]), lights[i].radius, sc.root_node());
}

void FramePrep::prepare_polygon_surface(const Vec3 clip_planes[8], uint64_t& offset, uint32_t polygon_index)
{
	// partial_renderer.rs:1464-1638
	PolyData& pd = poly[polygon_index];
	const MapPolygon& p = sc.polygons[polygon_index];
	const Vec4 plane_transformed = cam.planes_matrix * extend(p.plane.vec, -p.plane.dist);
	if (plane_transformed.w <= 0.0f) return;
	const Material& material = sc.materials[p.texture];
	if (!material.draw) return;
	for (uint32_t i = 0; i < p.num_vertices; ++i)
		vertices_transformed[p.first_vertex + i] = view_transform(cam.view_matrix, sc.vertices[p.first_vertex + i]);
	Vec2 v2d[MAX_VERTICES];
	const uint32_t count = project_and_clip_polygon(clip_planes, &vertices_transformed[p.first_vertex], p.num_vertices, v2d);
	if (count < 3) return;
	if (material.skybox)
	{
		// Sky polygons are not drawn; their screen bounds say where draw_skybox must draw (:1510-1528).
		ClippingPolygon b = ClippingPolygon::from_point(v2d[0]);
		for (uint32_t k = 1; k < count; ++k) b.extend_with_point(v2d[k]);
		if (has_sky)
			sky_bounds.extend(b);
		else
		{
			sky_bounds = b;
			has_sky = true;
		}
		return;
	}

	// DepthEquation::from_transformed_plane_equation, equations.rs:23-31
	const float pw = -plane_transformed.w;
	DepthEquation de{plane_transformed.x / pw, plane_transformed.y / pw, plane_transformed.z / pw};
	// tc equations, partial_renderer.rs:1536-1544, equations.rs:55-74
	const Vec4 tb[2] = {cam.planes_matrix * extend(p.tex_coord_equation[0].vec, p.tex_coord_equation[0].dist),
		cam.planes_matrix * extend(p.tex_coord_equation[1].vec, p.tex_coord_equation[1].dist)};
	TexCoordEquation te;
	for (int i = 0; i < 2; ++i)
	{
		te.d_tc_dx[i] = tb[i].x + tb[i].w * de.d_inv_z_dx;
		te.d_tc_dy[i] = tb[i].y + tb[i].w * de.d_inv_z_dy;
		te.k[i] = tb[i].z + tb[i].w * de.k;
	}
	const uint32_t mip = calculate_mip(v2d, count, de, te, opt.mip_bias);
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
		const float inv_z = std::fmax(de.sample(v2d[k]), 1.0f / max_z);
		const float z = 1.0f / inv_z;
		for (int i = 0; i < 2; ++i)
		{
			const float tc = z * (ts.d_tc_dx[i] * v2d[k].x + ts.d_tc_dy[i] * v2d[k].y + ts.k[i]);
			if (tc < tc_min[i]) tc_min[i] = tc;
			if (tc > tc_max[i]) tc_max[i] = tc;
		}
	}
	int32_t surface_tc_min[2];
	uint32_t surface_size[2];
	for (int i = 0; i < 2; ++i)
	{
		const float eps = 1.0f / 32.0f;
		tc_min[i] += eps;
		tc_max[i] -= eps;
		const int32_t round_mask = ~int32_t(LIGHTMAP_SCALE - 1);
		const int32_t min_down = (p.tex_coord_min[i] & round_mask) >> mip;
		const int32_t max_up = ((p.tex_coord_max[i] + int32_t(LIGHTMAP_SCALE) - 1) & round_mask) >> mip;
		int32_t tmin = std::max(as_i32(std::floor(std::fmax(tc_min[i], -inf))), min_down);
		int32_t tmax = std::min(as_i32(std::ceil(std::fmin(tc_max[i], inf))), max_up);
		if (tmin >= tmax)
		{
			tmin = std::min(tmin, max_up - 1);
			tmax = tmin + 1;
		}
		surface_tc_min[i] = tmin;
		surface_size[i] = uint32_t(tmax - tmin);
	}
	pd.visible_frame = current_frame;
	pd.depth = de;
	pd.tc = ts;
	pd.offset = offset;
	pd.size[0] = surface_size[0];
	pd.size[1] = surface_size[1];
	pd.mip = mip;
	pd.tc_min[0] = surface_tc_min[0];
	pd.tc_min[1] = surface_tc_min[1];
	offset += uint64_t(surface_size[0]) * surface_size[1];
	for (int i = 0; i < 2; ++i)
	{
		const float tmf = float(surface_tc_min[i]);
		pd.tc.d_tc_dx[i] -= tmf * de.d_inv_z_dx;
		pd.tc.d_tc_dy[i] -= tmf * de.d_inv_z_dy;
		pd.tc.k[i] -= tmf * de.k;
	}
	visible_polygons.push_back(polygon_index);
}

void FramePrep::prepare_polygons_surfaces()
{
	// partial_renderer.rs:1327-1359 (world leafs; no submodels in these maps)
	visible_polygons.clear();
	has_sky = false; // current_sky = None (:1336)
	uint64_t offset = 0;
	for (uint32_t i = 0; i < sc.leafs.size(); ++i)
	{
		if (leaf_data[i].visible_frame != current_frame) continue;
		Vec3 planes[8];
		leaf_data[i].bounds.get_clip_planes(planes);
		const BspLeaf& leaf = sc.leafs[i];
		for (uint32_t k = 0; k < leaf.num_polygons; ++k) prepare_polygon_surface(planes, offset, leaf.first_polygon + k);
	}
	total_texels = offset;
}

static bool polygon_is_affected_by_light(const MapPolygon& polygon, const PolygonBasisVecs& b, const SwLight& light)
{
	// partial_renderer.rs:3877-3985 (lights without a projector shadow map)
	const Vec3 lp = v3(light.position[0], light.position[1], light.position[2]);
	const Vec3 vec = lp - b.start;
	const float signed_distance = dot(vec, b.normal);
	if (signed_distance <= 0.0f) return false;
	const float square_radius = light.radius * light.radius - signed_distance * signed_distance;
	if (square_radius <= 0.0f) return false;
	Mat3 m;
	if (!mat3_invert_transpose(b.u, b.v, b.normal, m)) return false;
	const float tc0 = dot(vec, m.c[0]), tc1 = dot(vec, m.c[1]);
	const float radius = std::sqrt(square_radius);
	const float u_radius = radius * (1.0f / std::sqrt(magnitude2(b.u)));
	const float v_radius = radius * (1.0f / std::sqrt(magnitude2(b.v)));
	if (tc0 + u_radius < float(polygon.tex_coord_min[0]) || tc1 + v_radius < float(polygon.tex_coord_min[1]) ||
		tc0 - u_radius > float(polygon.tex_coord_max[0]) || tc1 - v_radius > float(polygon.tex_coord_max[1]))
		return false;
	return true;
}

void FramePrep::build_surface_descs()
{
	// partial_renderer.rs:1682-1819
	surfaces.resize(visible_polygons.size());
	const bool directional = opt.use_directional_lightmaps && sc.directional_lightmaps.size() > 1;
	for (size_t si = 0; si < visible_polygons.size(); ++si)
	{
		const uint32_t pi = visible_polygons[si];
		const MapPolygon& p = sc.polygons[pi];
		const PolyData& pd = poly[pi];
		const Material& mat = sc.materials[p.texture];
		SwSurfaceDesc& d = surfaces[si];
		std::memset(&d, 0, sizeof(d));
		const int32_t shift[2] = {0, 0}; // get_texture_shift: no scrolling materials in these maps
		const int32_t shift_mip[2] = {shift[0] >> pd.mip, shift[1] >> pd.mip};
		d.size[0] = pd.size[0];
		d.size[1] = pd.size[1];
		d.tc_start[0] = pd.tc_min[0] + shift_mip[0];
		d.tc_start[1] = pd.tc_min[1] + shift_mip[1];
		d.out_offset = pd.offset;
		d.emissive_mip = SW_NO_EMISSIVE;
		const bool diffuse_layer = mat.light && mat.has_diffuse;
		if (diffuse_layer)
		{
			d.flags = SW_SURF_DIFFUSE_LAYER;
			const uint32_t leaf = sc.polygon_leaf[pi];
			for (uint32_t li : leaf_lights[leaf])
			{
				if (polygon_is_affected_by_light(p, sc.basis[pi], lights[li]))
				{
					d.lights[d.num_lights++] = uint16_t(li);
					if (d.num_lights == MAX_POLYGON_LIGHTS) break;
				}
			}
			// get_basis_vecs_for_mip + texture shift correction (surfaces.rs:49-63, partial_renderer.rs:1736-1740)
			PolygonBasisVecs b = sc.basis[pi];
			if (pd.mip != 0)
			{
				const float scale = float(1u << pd.mip);
				b.u = b.u * scale;
				b.v = b.v * scale;
			}
			b.start = b.start - (float(shift_mip[0]) * b.u + float(shift_mip[1]) * b.v);
			const Vec3* vs[4] = {&b.u, &b.v, &b.start, &b.normal};
			float* ds[4] = {d.basis_u, d.basis_v, d.basis_start, d.basis_normal};
			for (int k = 0; k < 4; ++k)
			{
				ds[k][0] = vs[k]->x;
				ds[k][1] = vs[k]->y;
				ds[k][2] = vs[k]->z;
			}
			d.texture_mip = p.texture * NUM_MIPS + pd.mip;
			for (int i = 0; i < 2; ++i)
			{
				const int32_t round_mask = ~int32_t(LIGHTMAP_SCALE - 1);
				d.lightmap_tc_shift[i] = uint32_t(pd.tc_min[i] - ((p.tex_coord_min[i] & round_mask) >> pd.mip));
			}
			// get_polygon_lightmap_size, lightmap.rs:11-27
			d.lightmap_size[0] = uint32_t(((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1);
			d.lightmap_size[1] = uint32_t(((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1);
			d.lightmap_scale_log2 = LIGHTMAP_SCALE_LOG2 - pd.mip;
			d.lightmap_offset = (directional || sc.lightmaps.size() > 3) ? p.lightmap_data_offset : SW_NO_LIGHTMAP;
		}
		if (mat.emissive >= 0)
		{
			d.emissive_mip = uint32_t(mat.emissive) * NUM_MIPS + pd.mip;
			d.emissive_light[0] = mat.emissive_light[0];
			d.emissive_light[1] = mat.emissive_light[1];
			d.emissive_light[2] = mat.emissive_light[2];
		}
	}
}

void FramePrep::draw_polygon(const Vec3 clip_planes[8], uint32_t polygon_index)
{
	// draw_leaf's call of draw_polygon for a world polygon: its surface is the texture
	const MapPolygon& p = sc.polygons[polygon_index];
	const PolyData& pd = poly[polygon_index];
	if (p.num_vertices < 3) return;
	emit_draw(clip_planes, &vertices_transformed[p.first_vertex], p.num_vertices, pd.depth, pd.tc, pd.size[0], pd.size[1],
		pd.offset, SW_TEXSRC_SURFACE, sc.materials[p.texture].blending_mode);
}

void FramePrep::emit_draw(const Vec3 clip_planes[8], const Vec3* vt, uint32_t num_vertices, const DepthEquation& depth,
	const TexCoordEquation& tc, uint32_t tex_w, uint32_t tex_h, uint64_t tex_offset, uint32_t tex_source, uint32_t blend)
{
	// partial_renderer.rs:4011-4142
	Vec2 v2d[MAX_VERTICES];
	const uint32_t count = project_and_clip_polygon(clip_planes, vt, num_vertices, v2d);
	if (count < 3) return;
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
	SwDrawCmd d;
	std::memset(&d, 0, sizeof(d));
	d.first_vertex = uint32_t(vertices.size());
	d.vertex_count = count;
	for (uint32_t k = 0; k < count; ++k) // f32_to_fixed16_unchecked, fixed_math.rs:335-338
		vertices.push_back(SwVertex16{as_i32(v2d[k].x * 65536.0f), as_i32(v2d[k].y * 65536.0f)});
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
		const float z_scale = std::exp2(-5.0f - std::ceil(std::log2(std::fmax(max_inv_z, 1.0f / float(1 << 20)))));
		de = DepthEquation{de.d_inv_z_dx * z_scale, de.d_inv_z_dy * z_scale, de.k * z_scale};
		for (int i = 0; i < 2; ++i)
		{
			te.d_tc_dx[i] *= z_scale;
			te.d_tc_dy[i] *= z_scale;
			te.k[i] *= z_scale;
		}
		d.mode = line_z_may_be_used(depth, tc, v2d[max_i], min_x, max_x) ? SW_RASTER_LINE_Z_CORRECTED
																		 : SW_RASTER_FULL_PERSPECTIVE;
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
	draws.push_back(d);
}

void FramePrep::draw_leaf(const ClippingPolygon& bounds, uint32_t leaf_index)
{
	// partial_renderer.rs:2519-2559 (world polygons of the leaf in index order)
	Vec3 planes[8];
	bounds.get_clip_planes(planes);
	const BspLeaf& leaf = sc.leafs[leaf_index];
	for (uint32_t k = 0; k < leaf.num_polygons; ++k)
	{
		const uint32_t pi = leaf.first_polygon + k;
		if (poly[pi].visible_frame != current_frame) continue;
		draw_polygon(planes, pi);
	}
}

void FramePrep::draw_skybox(const ClippingPolygon& viewport)
{
	// partial_renderer.rs:2311-2448
	if (!has_sky || sc.sky_material < 0) return;
	ClippingPolygon bounds = sky_bounds;
	bounds.intersect(viewport);
	if (!bounds.is_valid_and_non_empty()) return;

	static const float BOX_VERTICES[8][3] = {{-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1},
		{1, 1, -1}, {1, 1, 1}};
	struct Side
	{
		uint32_t v[4];
		Vec3 normal, u, v_dir;
	};
	const Vec3 X = v3(1, 0, 0), Y = v3(0, 1, 0), Z = v3(0, 0, 1);
	const Side sides[6] = {
		{{0, 1, 3, 2}, X, Y, -Z},  // -X
		{{4, 6, 7, 5}, -X, -Y, -Z}, // +X
		{{0, 4, 5, 1}, Y, -X, -Z},  // -Y
		{{2, 3, 7, 6}, -Y, X, -Z},  // +Y
		{{0, 2, 6, 4}, Z, X, -Y},   // -Z
		{{1, 5, 7, 3}, -Z, X, Y},   // +Z
	};
	const float side_plane_dist = -1.0f, side_tc_shift = 1.0f;

	// get_object_matrix(position, rotation) = translate * rotate (src/common/matrix.rs:111-117)
	Mat4 translate = Mat4::identity();
	translate.c[3] = v4(cam.position.x, cam.position.y, cam.position.z, 1.0f);
	const Mat4 skybox_matrix = translate * mat4_from_quat(sky_rotation);
	Mat4 skybox_matrix_inverse;
	if (!invert(transpose(skybox_matrix), skybox_matrix_inverse)) return;
	const Mat4 skybox_view_matrix = cam.view_matrix * skybox_matrix;
	const Mat4 skybox_planes_matrix = cam.planes_matrix * skybox_matrix_inverse;

	const float SKY_SCALE = 16384.0f;
	Vec3 box[8];
	for (int i = 0; i < 8; ++i)
		box[i] = view_transform(skybox_view_matrix, v3(BOX_VERTICES[i][0], BOX_VERTICES[i][1], BOX_VERTICES[i][2]) * SKY_SCALE);
	Vec3 clip_planes[8];
	bounds.get_clip_planes(clip_planes);

	for (uint32_t side = 0; side < 6; ++side)
	{
		const SkyboxMip* mips = sc.skybox_mips[side];
		if (mips[0].size == 0) continue; // no texture for this side
		const Side& sd = sides[side];
		const Vec3 vt[4] = {box[sd.v[0]], box[sd.v[1]], box[sd.v[2]], box[sd.v[3]]};
		const Vec4 pt = skybox_planes_matrix * extend(sd.normal, -side_plane_dist);
		const float pw = -pt.w;
		const DepthEquation de{pt.x / pw, pt.y / pw, pt.z / pw};
		const float tc_equation_scale = float(mips[0].size) * 0.5f;
		const Vec4 tb[2] = {skybox_planes_matrix * (extend(sd.u, side_tc_shift) * tc_equation_scale),
			skybox_planes_matrix * (extend(sd.v_dir, side_tc_shift) * tc_equation_scale)};
		TexCoordEquation te;
		for (int i = 0; i < 2; ++i)
		{
			te.d_tc_dx[i] = tb[i].x + tb[i].w * de.d_inv_z_dx;
			te.d_tc_dy[i] = tb[i].y + tb[i].w * de.d_inv_z_dy;
			te.k[i] = tb[i].z + tb[i].w * de.k;
		}
		Vec2 v2d[MAX_VERTICES];
		const uint32_t count = project_and_clip_polygon(clip_planes, vt, 4, v2d);
		if (count < 3) continue;
		const uint32_t mip = calculate_mip(v2d, count, de, te, opt.mip_bias);
		const float mip_scale = 1.0f / float(1u << mip);
		TexCoordEquation ts;
		for (int i = 0; i < 2; ++i)
		{
			ts.d_tc_dx[i] = te.d_tc_dx[i] * mip_scale;
			ts.d_tc_dy[i] = te.d_tc_dy[i] * mip_scale;
			ts.k[i] = te.k[i] * mip_scale;
		}
		const SkyboxMip& t = mips[mip];
		if (t.size == 0) continue;
		const size_t before = draws.size();
		emit_draw(clip_planes, vt, 4, de, ts, t.size, t.size, t.offset, SW_TEXSRC_SKYBOX, SW_BLEND_NONE);
		stats.skybox_draws += uint32_t(draws.size() - before);
	}
}

void FramePrep::draw_tree()
{
	// partial_renderer.rs:2450-2517: back-to-front traversal with the camera-space w of node planes.
	const ClippingPolygon viewport = ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height));
	const Vec4 w_row = cam.planes_matrix.row(3);
	uint32_t stack[MAX_BSP_TREE_DEPTH];
	stack[0] = sc.root_node();
	uint32_t n = 1;
	while (n > 0)
	{
		const uint32_t node_index = stack[n - 1];
		if (node_index >= FIRST_LEAF_INDEX)
		{
			--n;
			const uint32_t leaf = node_index - FIRST_LEAF_INDEX;
			if (leaf_data[leaf].visible_frame != current_frame) continue;
			ClippingPolygon b = leaf_data[leaf].bounds;
			b.intersect(viewport);
			if (b.is_valid_and_non_empty())
			{
				++stats.visible_leafs;
				draw_leaf(b, leaf);
			}
		}
		else if (n < MAX_BSP_TREE_DEPTH)
		{
			const BspNode& node = sc.nodes[node_index];
			const float w = dot(w_row, extend(node.plane.vec, -node.plane.dist));
			const uint32_t mask = w >= 0.0f ? 1u : 0u;
			stack[n - 1] = node.children[1 ^ mask];
			stack[n] = node.children[mask];
			++n;
		}
		else
			--n; // deeper than the reference's stack: dropped as the reference does not push it
	}
}

void FramePrep::prepare_with_camera(const CameraMatrices& camera, const std::vector<SwLight>& frame_lights,
	const FrameOptions& options, Quat skybox_rotation)
{
	cam = camera;
	opt = options;
	sky_rotation = skybox_rotation;
	lights = frame_lights;
	stats = FrameStats();
	++current_frame;
	update_visibility(ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
	position_lights();
	prepare_polygons_surfaces();
	build_surface_descs();
	draws.clear();
	vertices.clear();
	// perform_rasterization_for_viewport_part (:1285-1325): skybox first, then the tree
	draw_skybox(ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
	draw_tree();
	std::memset(&params, 0, sizeof(params));
	params.pixel_format = opt.pixel_format;
	params.width = opt.width;
	params.height = opt.height;
	params.use_directional_lightmaps = (opt.use_directional_lightmaps && sc.directional_lightmaps.size() > 1) ? 1u : 0u;
	params.cam_pos[0] = cam.position.x;
	params.cam_pos[1] = cam.position.y;
	params.cam_pos[2] = cam.position.z;
	params.clear_background = opt.clear_background ? 1u : 0u;
	stats.visible_polygons = uint32_t(visible_polygons.size());
	stats.draws = uint32_t(draws.size());
	stats.surface_texels = total_texels;
}

void FramePrep::prepare(uint32_t frame_index, const FrameOptions& options)
{
	const CameraKey& k = sc.camera_path[frame_index % sc.camera_path.size()];
	const CameraMatrices camera =
		build_view_matrix(k.position, k.azimuth, k.elevation, options.fov, float(options.width), float(options.height));
	std::vector<SwLight> l;
	sc.frame_lights(frame_index % uint32_t(sc.camera_path.size()), l);
	prepare_with_camera(camera, l, options, quat_from_angle_z(float(frame_index) * sc.config.sky_rotation_speed));
}

} // namespace swhost
