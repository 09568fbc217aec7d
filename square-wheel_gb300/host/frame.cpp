// Per-frame host work (see frame.h). Compiled with -ffp-contract=off: every float expression is
// evaluated with the reference's operation order and rounding.
#include "frame.h"

#include <algorithm>
#include <cstring>

namespace swhost
{

namespace
{

constexpr uint32_t MAX_VERTICES = PREP_MAX_VERTICES;
constexpr float Z_NEAR = PREP_Z_NEAR;
constexpr uint32_t MAX_POLYGON_LIGHTS = SW_MAX_POLYGON_LIGHTS;
constexpr uint32_t MAX_BSP_TREE_DEPTH = 72; // bsp_builder.rs:53

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
	portals_depth = std::min(sc.config.portals_depth, 8u); // Renderer::new clamps it (renderer.rs:33)
	sc.map_polygons(map_polygons);
	map_polygons_base = map_polygons;
	// the polygons of every material with a framed animation (their material fields follow its frames)
	material_polygons.assign(sc.materials.size(), {});
	for (uint32_t pi = 0; pi < uint32_t(sc.polygons.size()); ++pi)
	{
		const uint32_t m = sc.polygons[pi].texture;
		if (m < sc.materials.size() && sc.materials[m].next_frame >= 0) material_polygons[m].push_back(pi);
	}
	leaf_sky_first.assign(sc.leafs.size() + 1, 0);
	for (uint32_t i = 0; i < sc.leafs.size(); ++i)
	{
		leaf_sky_first[i] = uint32_t(sky_polygons.size());
		for (uint32_t k = 0; k < sc.leafs[i].num_polygons; ++k)
			if (map_polygons[sc.leafs[i].first_polygon + k].flags & SW_POLY_SKY) sky_polygons.push_back(sc.leafs[i].first_polygon + k);
	}
	leaf_sky_first[sc.leafs.size()] = uint32_t(sky_polygons.size());
	leaf_view_index.resize(sc.leafs.size());
	poly.resize(sc.polygons.size());
	vertices_transformed.resize(sc.vertices.size());
	leaf_lights.resize(sc.leafs.size());
}

// ---- VisibilityCalculator (map_visibility_calculator.rs) ----
VisibilityCalculator::VisibilityCalculator(const Scene& scene) : sc(scene)
{
	leafs.resize(sc.leafs.size());
	portals.resize(sc.portals.size());
}

uint32_t VisibilityCalculator::find_current_leaf() const
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

bool VisibilityCalculator::project_portal(const MapPortal& portal, ClippingPolygon& out) const
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

void VisibilityCalculator::mark_reachable_leafs(const uint32_t* start, uint32_t n, const ClippingPolygon& start_bounds)
{
	// map_visibility_calculator.rs:157-267
	wave0.clear();
	wave1.clear();
	for (uint32_t i = 0; i < n; ++i)
	{
		wave0.push_back(start[i]);
		leafs[start[i]].bounds = start_bounds;
		leafs[start[i]].visible_frame = frame;
	}
	uint32_t depth = 0;
	while (!wave0.empty())
	{
		for (uint32_t leaf : wave0)
		{
			const ClippingPolygon leaf_bounds = leafs[leaf].bounds;
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
				Portal& pd = portals[portal];
				if (pd.visible_frame != frame)
				{
					pd.visible_frame = frame;
					pd.has_projection = project_portal(pv, pd.projection);
				}
				if (!pd.has_projection) continue;
				ClippingPolygon b = pd.projection;
				b.intersect(leaf_bounds);
				if (!b.is_valid_and_non_empty()) continue;
				Leaf& nd = leafs[next_leaf];
				if (nd.visible_frame != frame)
				{
					nd.visible_frame = frame;
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

void VisibilityCalculator::update(const CameraMatrices& camera, const ClippingPolygon& frame_bounds)
{
	// map_visibility_calculator.rs:52-97
	cam = camera;
	++frame;
	const uint32_t current_leaf = find_current_leaf();
	camera_leaf = current_leaf;
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

void VisibilityCalculator::update_with_start_leafs(const CameraMatrices& camera, const ClippingPolygon& frame_bounds,
	const uint32_t* start, uint32_t n)
{
	cam = camera;
	++frame;
	camera_leaf = n ? start[0] : 0;
	mark_reachable_leafs(start, n, frame_bounds);
}

void FramePrep::position_sphere(uint32_t id, Vec3 center, float radius, uint32_t node_index)
{
	// position_object_sphere_r, dynamic_objects_index.rs:206-241
	if (node_index >= FIRST_LEAF_INDEX)
	{
		leaf_lights[node_index - FIRST_LEAF_INDEX].push_back(id);
		light_leafs[id].push_back(node_index - FIRST_LEAF_INDEX);
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
	light_leafs.resize(lights.size());
	for (auto& l : light_leafs) l.clear();
	for (uint32_t i = 0; i < lights.size(); ++i)
		position_sphere(i, v3(lights[i].position[0], lights[i].position[1], lights[i].position[2]), lights[i].radius, sc.root_node());
}

void FramePrep::prepare_shadows()
{
	// prepare_dynamic_lights (partial_renderer.rs:398-515) for cube shadow maps: a shadowed light touching
	// a visible leaf gets six sides of 64..256 texels (by its distance from the camera), allocated in
	// light order; build_shadow_maps (:525-592) draws them with DepthRenderer::draw_map.
	depth_draws.clear();
	depth_vertices.clear();
	shadow_sides.clear();
	shadow_leafs.clear();
	SwLightShadow none;
	std::memset(&none, 0, sizeof(none));
	light_shadows.assign(lights.size(), none);
	uint64_t offset = 0;
	for (uint32_t li = 0; li < lights.size(); ++li)
	{
		if (sc.light_is_projector(li))
		{
			prepare_projector(li, offset);
			continue;
		}
		if (!sc.light_is_shadowed(li)) continue;
		bool visible = false;
		for (uint32_t leaf : light_leafs[li])
			if (vis.visible(leaf))
			{
				visible = true;
				break;
			}
		if (!visible) continue;
		const SwLight& light = lights[li];
		const Vec3 lp = v3(light.position[0], light.position[1], light.position[2]);
		const float dist_from_camera = magnitude(cam.position - lp);
		const float dist_to_closest_point = dist_from_camera - light.radius;
		const uint32_t min_size = 64, max_size = 256;
		uint32_t size = max_size;
		if (dist_to_closest_point > 0.0f)
		{
			const float target_size = 128.0f * light.radius / dist_to_closest_point;
			const float e = std::fmax(std::log2(target_size) + opt.shadows_quality, 0.0f); // f32 log2, `as u32`
			const uint32_t shift = e >= 31.0f ? 31u : uint32_t(e);
			size = std::max(std::min(1u << shift, max_size), min_size);
		}
		light_shadows[li] = none;
		light_shadows[li].kind = SW_SHADOW_CUBE;
		light_shadows[li].size = size;
		light_shadows[li].offset = offset;
		for (uint32_t side = 0; side < 6; ++side)
			draw_depth_map(cube_shadow_map_side_matrices(lp, float(size), side), size, offset + uint64_t(side) * size * size);
		offset += uint64_t(size) * size * 6;
	}
	shadow_texels = offset;
}

void FramePrep::prepare_projector(uint32_t li, uint64_t& offset)
{
	// prepare_dynamic_lights' projector branch (partial_renderer.rs:462-513): the map size from the
	// closest of the cone's five reference points, 32..1024 texels; build_shadow_maps (:565-590) draws it
	// with the light's matrices; its shadow map (renderer_structs.rs:288-308) carries the rotated axes.
	bool visible = false;
	for (uint32_t leaf : light_leafs[li])
		if (vis.visible(leaf))
		{
			visible = true;
			break;
		}
	if (!visible) return;
	const SwLight& light = lights[li];
	const Vec3 lp = v3(light.position[0], light.position[1], light.position[2]);
	Quat rotation;
	float fov;
	sc.projector_pose(li, frame_time_s, rotation, fov);
	const float hft = light.radius * std::tan(fov * 0.5f);
	Mat4 light_matrix = mat4_from_quat(rotation);
	light_matrix.c[3] = v4(lp.x, lp.y, lp.z, 1.0f);
	const Vec3 pts[5] = {v3(light.radius, 0, 0), v3(light.radius, hft, hft), v3(light.radius, hft, -hft),
		v3(light.radius, -hft, hft), v3(light.radius, -hft, -hft)};
	float closest_square = 1.0e24f;
	for (const Vec3& v : pts)
		closest_square = std::fmin(closest_square, magnitude2(cam.position - truncate(light_matrix * extend(v, 1.0f))));
	const float target_size = 1024.0f * hft / std::sqrt(closest_square);
	const float e = std::fmax(std::log2(target_size) + opt.shadows_quality, 0.0f);
	const uint32_t shift = e >= 31.0f ? 31u : uint32_t(e);
	const uint32_t size = std::max(std::min(1u << shift, 1024u), 32u);
	SwLightShadow& m = light_shadows[li];
	m.kind = SW_SHADOW_PROJECTOR;
	m.size = size;
	m.offset = offset;
	const float inv_half_fov_tan = 1.0f / std::tan(fov * 0.5f);
	const Vec3 bx = rotate_vector(rotation, v3(0, 1, 0)) * inv_half_fov_tan;
	const Vec3 by = rotate_vector(rotation, v3(0, 0, 1)) * inv_half_fov_tan;
	const Vec3 bz = rotate_vector(rotation, v3(-1, 0, 0));
	m.basis_x[0] = bx.x, m.basis_x[1] = bx.y, m.basis_x[2] = bx.z;
	m.basis_y[0] = by.x, m.basis_y[1] = by.y, m.basis_y[2] = by.z;
	m.basis_z[0] = bz.x, m.basis_z[1] = bz.y, m.basis_z[2] = bz.z;
	draw_depth_map(build_view_matrix_with_full_rotation(lp, rotation, fov, float(size), float(size)), size, offset);
	offset += uint64_t(size) * size;
}

template <class F>
void FramePrep::for_each_depth_leaf(const CameraMatrices& camera, uint32_t size, F&& leaf_fn)
{
	// DepthRenderer::draw_map / draw_tree / draw_leaf (depth_renderer.rs:45-197): the side camera's
	// visibility from the light, then the leafs it reaches, back to front
	const float fs = float(size);
	shadow_vis.update(camera, ClippingPolygon::from_box(0.0f, 0.0f, fs, fs));
	const Vec4 w_row = camera.planes_matrix.row(3);
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
			if (!shadow_vis.visible(leaf)) continue;
			Vec3 planes[8];
			shadow_vis.bounds(leaf).get_clip_planes(planes);
			leaf_fn(leaf, planes);
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
			--n;
	}
}

void FramePrep::draw_depth_map(const CameraMatrices& camera, uint32_t size, uint64_t map_offset)
{
	if (shadow_view)
	{
		// the GPU prepares the polygons (sw_build_shadow_maps_view): record the side and its leafs
		SwShadowSide sd;
		std::memset(&sd, 0, sizeof(sd));
		std::memcpy(sd.view_matrix, &camera.view_matrix, sizeof(sd.view_matrix));
		std::memcpy(sd.planes_matrix, &camera.planes_matrix, sizeof(sd.planes_matrix));
		sd.map_size = size;
		sd.map_offset = map_offset;
		const uint32_t side = uint32_t(shadow_sides.size());
		shadow_sides.push_back(sd);
		for_each_depth_leaf(camera, size, [this, side](uint32_t leaf, const Vec3 planes[8]) {
			const BspLeaf& lv = sc.leafs[leaf];
			SwShadowLeaf sl;
			std::memset(&sl, 0, sizeof(sl));
			sl.side = side;
			sl.first_polygon = lv.first_polygon;
			sl.num_polygons = lv.num_polygons;
			for (int k = 0; k < 8; ++k)
			{
				sl.clip_planes[k][0] = planes[k].x;
				sl.clip_planes[k][1] = planes[k].y;
				sl.clip_planes[k][2] = planes[k].z;
			}
			shadow_leafs.push_back(sl);
		});
		return;
	}
	for_each_depth_leaf(camera, size, [this, &camera, size, map_offset](uint32_t leaf, const Vec3 planes[8]) {
		const BspLeaf& lv = sc.leafs[leaf];
		for (uint32_t k = 0; k < lv.num_polygons; ++k) draw_depth_polygon(camera, planes, lv.first_polygon + k, size, map_offset);
	});
}

void FramePrep::draw_depth_polygon(const CameraMatrices& camera, const Vec3 clip_planes[8], uint32_t polygon_index, uint32_t size,
	uint64_t map_offset)
{
	// DepthRenderer::draw_polygon::<false> + draw_depth_polygon (depth_renderer.rs:199-287)
	const SwMapPolygon& p = map_polygons[polygon_index];
	SwDepthDraw d;
	std::memset(&d, 0, sizeof(d));
	if (!depth_map_equation(p, camera.planes_matrix, d.depth_eq)) return;
	const uint32_t nv = std::min(p.num_vertices, PREP_MAX_VERTICES);
	if (nv < 3) return;
	Vec3 vt[MAX_VERTICES];
	for (uint32_t i = 0; i < nv; ++i) vt[i] = view_transform(camera.view_matrix, sc.vertices[p.first_vertex + i]);
	Vec2 v2d[MAX_VERTICES];
	const uint32_t count = project_and_clip_polygon(clip_planes, vt, nv, v2d);
	if (count < 3) return;
	d.first_vertex = uint32_t(depth_vertices.size());
	d.vertex_count = count;
	d.map_size = size;
	d.map_offset = map_offset;
	for (uint32_t k = 0; k < count; ++k) // f32_to_fixed16 (fixed_math.rs:31-34): saturating `as`
		depth_vertices.push_back(SwVertex16{as_i32(v2d[k].x * 65536.0f), as_i32(v2d[k].y * 65536.0f)});
	depth_draws.push_back(d);
}

void FramePrep::prepare_polygon_surface(const Vec3 clip_planes[8], uint64_t& offset, uint32_t polygon_index)
{
	// partial_renderer.rs:1464-1638
	PolyData& pd = poly[polygon_index];
	const SwMapPolygon& p = map_polygons[polygon_index];
	Vec2 v2d[MAX_VERTICES];
	uint32_t count = 0;
	SurfacePrep sp;
	const PrepResult r = swhost::prepare_polygon_surface(p, sc.vertices.data(), cam.view_matrix, cam.planes_matrix, clip_planes,
		opt.mip_bias, &vertices_transformed[p.first_vertex], v2d, &count, sp);
	if (r == PREP_SKY)
	{
		// Sky polygons are not drawn; their screen bounds say where draw_skybox must draw (:1510-1528).
		extend_sky_bounds(v2d, count);
		return;
	}
	if (r != PREP_SURFACE) return;
	pd.visible_frame = current_frame;
	pd.depth = sp.depth;
	pd.tc = sp.tc;
	pd.offset = offset;
	pd.size[0] = sp.size[0];
	pd.size[1] = sp.size[1];
	pd.mip = sp.mip;
	pd.tc_min[0] = sp.tc_min[0];
	pd.tc_min[1] = sp.tc_min[1];
	offset += uint64_t(sp.size[0]) * sp.size[1];
	visible_polygons.push_back(polygon_index);
}

void FramePrep::extend_sky_bounds(const Vec2* v2d, uint32_t count)
{
	ClippingPolygon b = ClippingPolygon::from_point(v2d[0]);
	for (uint32_t k = 1; k < count; ++k) b.extend_with_point(v2d[k]);
	if (has_sky)
		sky_bounds.extend(b);
	else
	{
		sky_bounds = b;
		has_sky = true;
	}
}

void FramePrep::prepare_polygons_surfaces()
{
	// partial_renderer.rs:1327-1359 (world leafs; no submodels in these maps)
	visible_polygons.clear();
	has_sky = false; // current_sky = None (:1336)
	uint64_t offset = 0;
	for (uint32_t i = 0; i < sc.leafs.size(); ++i)
	{
		if (!vis.visible(i)) continue;
		Vec3 planes[8];
		vis.bounds(i).get_clip_planes(planes);
		const BspLeaf& leaf = sc.leafs[i];
		for (uint32_t k = 0; k < leaf.num_polygons; ++k) prepare_polygon_surface(planes, offset, leaf.first_polygon + k);
	}
	total_texels = offset;
}

void FramePrep::build_surface_descs()
{
	// partial_renderer.rs:1682-1819
	surfaces.resize(visible_polygons.size());
	const bool directional = opt.use_directional_lightmaps && sc.directional_lightmaps.size() > 1;
	const bool simple_lightmaps = sc.lightmaps.size() > 3;
	for (size_t si = 0; si < visible_polygons.size(); ++si)
	{
		const uint32_t pi = visible_polygons[si];
		const SwMapPolygon& p = map_polygons[pi];
		const PolyData& pd = poly[pi];
		SurfacePrep sp;
		sp.size[0] = pd.size[0];
		sp.size[1] = pd.size[1];
		sp.mip = pd.mip;
		sp.tc_min[0] = pd.tc_min[0];
		sp.tc_min[1] = pd.tc_min[1];
		SwSurfaceDesc& d = surfaces[si];
		const SwMaterialFrame& mf = material_frames[p.texture];
		make_surface_desc(p, sp, pd.offset, directional, simple_lightmaps, &mf, d);
		if (p.flags & SW_POLY_DIFFUSE_LAYER)
			for (uint32_t li : leaf_lights[sc.polygon_leaf[pi]])
				if (polygon_is_affected_by_light(p, lights[li], li < light_shadows.size() ? &light_shadows[li] : nullptr))
				{
					d.lights[d.num_lights++] = uint16_t(li);
					if (d.num_lights == MAX_POLYGON_LIGHTS) break;
				}
	}
}

void FramePrep::draw_polygon(const Vec3 clip_planes[8], uint32_t polygon_index)
{
	// draw_leaf's call of draw_polygon for a world polygon: its surface is the texture
	const SwMapPolygon& p = map_polygons[polygon_index];
	const PolyData& pd = poly[polygon_index];
	if (p.num_vertices < 3) return;
	emit_draw(clip_planes, &vertices_transformed[p.first_vertex], p.num_vertices, pd.depth, pd.tc, pd.size[0], pd.size[1],
		pd.offset, SW_TEXSRC_SURFACE, p.blending_mode);
}

void FramePrep::emit_draw(const Vec3 clip_planes[8], const Vec3* vt, uint32_t num_vertices, const DepthEquation& depth,
	const TexCoordEquation& tc, uint32_t tex_w, uint32_t tex_h, uint64_t tex_offset, uint32_t tex_source, uint32_t blend)
{
	SwVertex16 v[MAX_VERTICES];
	SwDrawCmd d;
	const uint32_t count = make_draw(clip_planes, vt, num_vertices, depth, tc, tex_w, tex_h, tex_offset, tex_source, blend, v, d);
	if (count < 3) return;
	d.first_vertex = uint32_t(vertices.size());
	vertices.insert(vertices.end(), v, v + count);
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
	// decals after all the leaf's polygons (partial_renderer.rs:2561-2575)
	if (leaf_index < sc.leaf_decals.size() && !sc.leaf_decals[leaf_index].empty())
		for (uint32_t k = 0; k < leaf.num_polygons; ++k) draw_polygon_decals(planes, leaf.first_polygon + k, sc.leaf_decals[leaf_index]);
	const bool models = leaf_index < sc.leaf_models.size() && !sc.leaf_models[leaf_index].empty();
	const bool sprites = leaf_index < sc.leaf_sprites.size() && !sc.leaf_sprites[leaf_index].empty();
	const bool portals = leaf_index < sc.leaf_view_portals.size() && !sc.leaf_view_portals[leaf_index].empty();
	if (models || sprites || portals) draw_leaf_models(bounds, leaf_index);
}

namespace
{
// get_light_cube_light, src/square_wheel/light.rs:296-340: the cube side facing each normal axis,
// weighted by that axis component.
void light_cube_light(const float cube[6][3], Vec3 n, float out[3])
{
	for (int i = 0; i < 3; ++i) out[i] = 0.0f;
	const float comps[3] = {n.x, n.y, n.z};
	for (int a = 0; a < 3; ++a)
	{
		const int side = comps[a] <= 0.0f ? 2 * a : 2 * a + 1;
		const float w = comps[a] <= 0.0f ? -comps[a] : comps[a];
		for (int i = 0; i < 3; ++i) out[i] += cube[side][i] * w;
	}
}

// Mat3 inverse (cgmath Matrix3::invert by cofactors): get_normals_matrix's inverse transpose of the
// model matrix's axes, triangle_models_rendering.rs:722-731 (identity if singular).
void normals_matrix(const Mat4& m, float out[3][3])
{
	const float a[3][3] = {{m.c[0].x, m.c[1].x, m.c[2].x}, {m.c[0].y, m.c[1].y, m.c[2].y}, {m.c[0].z, m.c[1].z, m.c[2].z}};
	// t = transpose(axes); out = inverse(t)
	float t[3][3];
	for (int r = 0; r < 3; ++r)
		for (int c = 0; c < 3; ++c) t[r][c] = a[c][r];
	const float det = t[0][0] * (t[1][1] * t[2][2] - t[1][2] * t[2][1]) - t[0][1] * (t[1][0] * t[2][2] - t[1][2] * t[2][0]) +
		t[0][2] * (t[1][0] * t[2][1] - t[1][1] * t[2][0]);
	if (det == 0.0f || !std::isfinite(det))
	{
		for (int r = 0; r < 3; ++r)
			for (int c = 0; c < 3; ++c) out[r][c] = r == c ? 1.0f : 0.0f;
		return;
	}
	const float id = 1.0f / det;
	out[0][0] = (t[1][1] * t[2][2] - t[1][2] * t[2][1]) * id;
	out[0][1] = (t[0][2] * t[2][1] - t[0][1] * t[2][2]) * id;
	out[0][2] = (t[0][1] * t[1][2] - t[0][2] * t[1][1]) * id;
	out[1][0] = (t[1][2] * t[2][0] - t[1][0] * t[2][2]) * id;
	out[1][1] = (t[0][0] * t[2][2] - t[0][2] * t[2][0]) * id;
	out[1][2] = (t[0][2] * t[1][0] - t[0][0] * t[1][2]) * id;
	out[2][0] = (t[1][0] * t[2][1] - t[1][1] * t[2][0]) * id;
	out[2][1] = (t[0][1] * t[2][0] - t[0][0] * t[2][1]) * id;
	out[2][2] = (t[0][0] * t[1][1] - t[0][1] * t[1][0]) * id;
}

// f32_to_fixed16, src/common/fixed_math.rs: (x * 65536) as i32, saturating.
int32_t to_fixed16(float x) { return as_i32(x * 65536.0f); }
} // namespace

// clip_3d_model_polygon_by_plane with the near plane z >= Z_NEAR (src/common/clipping.rs:259-310)
uint32_t FramePrep::clip_model_near(const ModelVertex3d* src, uint32_t n, ModelVertex3d* dst)
{
	uint32_t out = 0;
	const ModelVertex3d* prev = &src[n - 1];
	float prev_d = prev->pos.z;
	auto inter = [&](const ModelVertex3d& v0, const ModelVertex3d& v1) {
		const float d0 = v0.pos.z - PREP_Z_NEAR, d1 = v1.pos.z - PREP_Z_NEAR;
		const float sum = d1 - d0, k0 = d0 / sum, k1 = d1 / sum;
		ModelVertex3d r;
		r.pos = v0.pos * k1 - v1.pos * k0;
		for (int i = 0; i < 2; ++i) r.tc[i] = v0.tc[i] * k1 - v1.tc[i] * k0;
		for (int i = 0; i < 3; ++i) r.light[i] = v0.light[i] * k1 - v1.light[i] * k0;
		return r;
	};
	for (uint32_t i = 0; i < n && out < MAX_VERTICES; ++i)
	{
		const ModelVertex3d& v = src[i];
		const float d = v.pos.z;
		if (d > PREP_Z_NEAR)
		{
			if (prev_d < PREP_Z_NEAR && out < MAX_VERTICES) dst[out++] = inter(*prev, v);
			if (out < MAX_VERTICES) dst[out++] = v;
		}
		else if (d == PREP_Z_NEAR)
			dst[out++] = v;
		else if (prev_d > PREP_Z_NEAR)
			dst[out++] = inter(*prev, v);
		prev = &v;
		prev_d = d;
	}
	return out;
}

void FramePrep::draw_leaf_models(const ClippingPolygon& bounds, uint32_t leaf_index)
{
	// The leaf's models and sprites back to front: farther first by camera-space depth of the object's
	// origin, models before sprites at equal depth (the reference's LeafObjectsSorter, draw_ordering.rs,
	// orders the objects of a leaf by their projected boxes; objects here never leave their leaf).
	struct Obj
	{
		float z;
		uint32_t kind, index; // kind 0 model, 1 sprite
	};
	std::vector<Obj> order;
	if (leaf_index < sc.leaf_models.size())
		for (uint32_t m : sc.leaf_models[leaf_index]) order.push_back({view_transform(cam.view_matrix, sc.models[m].position).z, 0u, m});
	if (leaf_index < sc.leaf_sprites.size())
		for (uint32_t k : sc.leaf_sprites[leaf_index])
			order.push_back({view_transform(cam.view_matrix, sc.sprites[k].position).z, 1u, k});
	if (leaf_index < sc.leaf_view_portals.size())
		for (uint32_t k : sc.leaf_view_portals[leaf_index])
		{
			// a portal by its vertices' centre
			const ViewPortal& pt = sc.view_portals[k];
			Vec3 c = v3(0.0f, 0.0f, 0.0f);
			for (const Vec3& v : pt.vertices) c = c + v;
			c = c / float(pt.vertices.size());
			order.push_back({view_transform(cam.view_matrix, c).z, 2u, k});
		}
	std::stable_sort(order.begin(), order.end(), [](const Obj& a, const Obj& b) { return a.z > b.z; });
	Vec3 planes[8];
	bounds.get_clip_planes(planes);
	for (const Obj& o : order)
	{
		if (o.kind == 0)
			draw_model(bounds, o.index);
		else if (o.kind == 1)
			draw_sprite(bounds, o.index);
		else
			draw_view_portal(planes, o.index);
	}
}

void FramePrep::draw_sprite(const ClippingPolygon& bounds, uint32_t sprite_index)
{
	const SpriteEntity& sprite = sc.sprites[sprite_index];
	// prepare_sprites (partial_renderer.rs:740-991): the sprite's plane vectors from the camera basis
	Mat4 view_inverse;
	if (!invert(cam.view_matrix, view_inverse)) return;
	const Vec3 u_base_initial = truncate(view_inverse * v4(1, 0, 0, 0));
	const Vec3 u_base = u_base_initial / magnitude(u_base_initial);
	const Vec3 v_base_initial = truncate(view_inverse * v4(0, 1, 0, 0));
	const Vec3 v_base = v_base_initial / magnitude(v_base_initial);
	const Vec3 camera_direction = cross(u_base, v_base);
	Vec3 u_n = u_base, v_n = v_base;
	switch (sprite.orientation)
	{
	case SpriteEntity::PARALLEL_TO_CAMERA_PLANE:
		break;
	case SpriteEntity::FACING_TOWARDS_CAMERA:
	{
		const Vec3 to_camera = cam.position - sprite.position;
		const Vec3 plane_normal = to_camera / std::fmax(magnitude(to_camera), 0.001f);
		const Vec3 u_projected = u_base - plane_normal * dot(u_base, plane_normal);
		const float len = magnitude(u_projected);
		u_n = len < 0.0001f ? v3(1, 0, 0) : u_projected / len;
		v_n = cross(u_n, plane_normal);
		break;
	}
	case SpriteEntity::ALIGN_TO_Z_AXIS_PARALLEL_TO_CAMERA_PLANE:
	{
		v_n = v3(0, 0, -1);
		const Vec3 u = cross(v_n, camera_direction);
		const float len = magnitude(u);
		u_n = len < 0.0001f ? v3(1, 0, 0) : u / len;
		break;
	}
	default:
	{
		const Vec3 to_camera = cam.position - sprite.position;
		v_n = v3(0, 0, -1);
		const Vec3 u = cross(to_camera, v_n);
		const float len = magnitude(u);
		u_n = len < 0.0001f ? v3(1, 0, 0) : u / len;
		break;
	}
	}
	if (sprite.angle != 0.0f)
	{
		const float c = std::cos(sprite.angle), s = std::sin(sprite.angle);
		const Vec3 nu = u_n * c - v_n * s, nv = u_n * s + v_n * c;
		u_n = nu;
		v_n = nv;
	}
	const LiteMip& mip0 = sc.lite_mips[size_t(sprite.texture) * NUM_MIPS];
	const float ratio_h_w = float(mip0.height) / float(mip0.width);
	const float step_u = sprite.radius * (1.0f / std::sqrt(1.0f + ratio_h_w * ratio_h_w)); // inv_sqrt_fast, generic
	const float ratio_w_h = float(mip0.width) / float(mip0.height);
	const float step_v = sprite.radius * (1.0f / std::sqrt(1.0f + ratio_w_h * ratio_w_h));
	const Vec3 u_vec = u_n * step_u, v_vec = v_n * step_v;
	const Vec3 corners[4] = {sprite.position + u_vec + v_vec, sprite.position + u_vec - v_vec, sprite.position - u_vec - v_vec,
		sprite.position - u_vec + v_vec};
	Vec3 vp[4];
	for (int k = 0; k < 4; ++k) vp[k] = view_transform(cam.view_matrix, corners[k]);
	uint32_t mip = 0;
	if (vp[0].z > 0.0f && vp[1].z > 0.0f && vp[2].z > 0.0f && vp[3].z > 0.0f)
	{
		Vec2 pts[4];
		for (int k = 0; k < 4; ++k) pts[k] = v2(vp[k].x / vp[k].z, vp[k].y / vp[k].z);
		const Vec2 d0 = v2(pts[0].x - pts[2].x, pts[0].y - pts[2].y), d1 = v2(pts[1].x - pts[3].x, pts[1].y - pts[3].y);
		const float shortest = std::fmin(d0.x * d0.x + d0.y * d0.y, d1.x * d1.x + d1.y * d1.y);
		if (shortest <= 0.0f)
			mip = NUM_MIPS - 1;
		else
		{
			const float tc_diag = float(mip0.width) * float(mip0.width) + float(mip0.height) * float(mip0.height);
			const float mip_f = std::log2(tc_diag / shortest) * 0.5f + opt.mip_bias;
			mip = std::min<uint32_t>(uint32_t(as_i32(std::fmax(std::round(mip_f), 0.0f))), NUM_MIPS - 1);
		}
	}
	const float min_z = std::fmin(std::fmin(std::fmin(vp[0].z, vp[1].z), vp[2].z), vp[3].z);
	const float max_z = std::fmax(std::fmax(std::fmax(vp[0].z, vp[1].z), vp[2].z), vp[3].z);
	const uint32_t max_tess = 4; // MAX_SPRITE_TESSELATION_LEVEL, renderer_structs.rs:164
	const uint32_t tess = min_z <= 0.0f ? max_tess
										: std::min<uint32_t>(uint32_t(as_i32(std::fmax((max_z / min_z - 1.0f) * 4.0f, 1.0f))), max_tess);
	// the sprite's light: light_add, plus light_scale x (the light cube's mean, half the directional
	// component, half the visible unshadowed dynamic lights)
	float light[3] = {sprite.light_add[0], sprite.light_add[1], sprite.light_add[2]};
	if (sprite.light_scale > 0.0f)
	{
		const float side_scale = sprite.light_scale / 6.0f;
		for (int s6 = 0; s6 < 6; ++s6)
			for (int c = 0; c < 3; ++c) light[c] += sprite.light_cube[s6][c] * side_scale;
		const float dir_scale = sprite.light_scale * 0.5f * magnitude(sprite.light_dir_scaled);
		for (int c = 0; c < 3; ++c) light[c] += dir_scale * sprite.light_color[c];
		const float dyn_scale = sprite.light_scale * 0.5f;
		const float min_square_distance = sprite.radius * sprite.radius;
		for (size_t li = 0; li < lights.size(); ++li)
		{
			if (li < light_shadows.size() && light_shadows[li].kind != SW_SHADOW_NONE) continue;
			bool visible = false;
			if (li < light_leafs.size())
				for (uint32_t lf : light_leafs[li]) visible = visible || vis.visible(lf);
			if (!visible) continue;
			const SwLight& l = lights[li];
			const Vec3 to_light = v3(l.position[0], l.position[1], l.position[2]) - sprite.position;
			const float inv_square_dist = 1.0f / std::fmax(magnitude2(to_light), min_square_distance);
			const float light_inv_square_radius = 1.0f / (l.radius * l.radius);
			if (inv_square_dist < light_inv_square_radius) continue;
			const float scale = dyn_scale * 1.0f * (inv_square_dist - light_inv_square_radius);
			for (int c = 0; c < 3; ++c) light[c] += scale * l.color[c];
		}
	}

	// draw_sprite (partial_renderer.rs:3290-3523)
	const LiteMip& tex = sc.lite_mips[size_t(sprite.texture) * NUM_MIPS + mip];
	const float tw = float(tex.width), th = float(tex.height), tc_reduce = 1.0f / 16.0f;
	ModelVertex3d quad[4];
	const float tcs[4][2] = {{tw - tc_reduce, th - tc_reduce}, {tw - tc_reduce, tc_reduce}, {tc_reduce, tc_reduce}, {tc_reduce, th - tc_reduce}};
	for (int k = 0; k < 4; ++k)
	{
		quad[k].pos = vp[k];
		quad[k].tc[0] = tcs[k][0];
		quad[k].tc[1] = tcs[k][1];
		for (int c = 0; c < 3; ++c) quad[k].light[c] = light[c];
	}
	Vec3 planes[8];
	bounds.get_clip_planes(planes);
	ModelVertex3d clipped[MAX_VERTICES];
	if (tess <= 1)
	{
		const uint32_t n = clip_model_near(quad, 4, clipped);
		if (n < 3) return;
		stats.model_triangles += emit_model_polygon(clipped, n, planes, 8, tex, sprite.blending_mode, nullptr);
		return;
	}
	const uint32_t row = tess + 1;
	ModelVertex3d grid[(4 + 1) * (4 + 1)];
	const float inv_step = 1.0f / float(tess);
	for (uint32_t y = 0; y < row; ++y)
	{
		const float ym = float(y) * inv_step;
		for (uint32_t x = 0; x < row; ++x)
		{
			const float xm = float(x) * inv_step;
			const float w[4] = {xm * ym, (1.0f - xm) * ym, (1.0f - xm) * (1.0f - ym), xm * (1.0f - ym)};
			ModelVertex3d& g = grid[x + y * row];
			g.pos = quad[0].pos * w[0] + quad[1].pos * w[1] + quad[2].pos * w[2] + quad[3].pos * w[3];
			for (int i = 0; i < 2; ++i) g.tc[i] = w[0] * quad[0].tc[i] + w[1] * quad[1].tc[i] + w[2] * quad[2].tc[i] + w[3] * quad[3].tc[i];
			for (int c = 0; c < 3; ++c) g.light[c] = 0.0f;
		}
	}
	for (uint32_t x = 0; x < tess; ++x)
		for (uint32_t y = 0; y < tess; ++y)
		{
			ModelVertex3d sub[4] = {grid[x + y * row], grid[x + (y + 1) * row], grid[1 + x + (y + 1) * row], grid[1 + x + y * row]};
			const uint32_t n = clip_model_near(sub, 4, clipped);
			if (n < 3) continue;
			stats.model_triangles += emit_model_polygon(clipped, n, planes, 8, tex, sprite.blending_mode, light);
		}
}

void FramePrep::draw_model(const ClippingPolygon& bounds, uint32_t model_index)
{
	const ModelEntity& e = sc.models[model_index];
	const ModelMesh& mesh = sc.model_meshes[e.mesh];
	// AnimationPoint: frames f0, f1 and the weight of f0 at the frame's time
	const float t = frame_time_s * e.anim_speed + e.anim_phase;
	const float ft = std::floor(t);
	const uint32_t f0 = uint32_t(int64_t(ft) % int64_t(mesh.num_frames)), f1 = (f0 + 1) % mesh.num_frames;
	const float lerp0 = std::fmin(std::fmax(1.0f - (t - ft), 0.0f), 1.0f), lerp1 = 1.0f - lerp0;
	const bool perform_lerp = lerp0 > 0.01f && lerp0 < 0.99f;
	// get_object_matrix(position, rotation): translate * rotate (src/common/matrix.rs:111-117)
	Mat4 model_matrix = mat4_from_quat(quat_from_angle_z(e.yaw));
	model_matrix.c[3] = v4(e.position.x, e.position.y, e.position.z, 1.0f);
	const Mat4 model_view = cam.view_matrix * model_matrix;

	// calculate_triangle_model_texture_mip, triangle_models_rendering.rs:274-322 (bbox made a cube)
	uint32_t mip = 0;
	{
		const Vec3 c = (mesh.bbox_min + mesh.bbox_max) * 0.5f;
		const Vec3 hs = (mesh.bbox_max - mesh.bbox_min) * 0.5f;
		const float ch = (hs.x + hs.y + hs.z) / 3.0f;
		float min_x = 0, max_x = 0, min_y = 0, max_y = 0;
		bool behind = false;
		for (int k = 0; k < 8; ++k)
		{
			const Vec3 corner = v3(c.x + ((k & 1) ? ch : -ch), c.y + ((k & 2) ? ch : -ch), c.z + ((k & 4) ? ch : -ch));
			const Vec4 vp = model_view * extend(corner, 1.0f);
			if (vp.w <= 0.0f)
			{
				behind = true;
				break;
			}
			const float x = vp.x / vp.w, y = vp.y / vp.w;
			if (k == 0)
				min_x = max_x = x, min_y = max_y = y;
			min_x = std::fmin(min_x, x), max_x = std::fmax(max_x, x), min_y = std::fmin(min_y, y), max_y = std::fmax(max_y, y);
		}
		const LiteMip& m0 = sc.lite_mips[size_t(e.texture) * NUM_MIPS];
		const float max_dim = std::fmax(max_x - min_x, max_y - min_y);
		if (!behind)
		{
			if (max_dim <= 0.0f)
				mip = NUM_MIPS - 1;
			else
			{
				const float tpp = float(std::max(m0.width, m0.height)) / max_dim;
				mip = uint32_t(std::min<int32_t>(std::max<int32_t>(as_i32(std::floor(std::log2(tpp) + opt.mip_bias)), 0), NUM_MIPS - 1));
			}
		}
	}
	const LiteMip& tex = sc.lite_mips[size_t(e.texture) * NUM_MIPS + mip];

	// animate_and_transform_triangle_mesh_vertices (VertexAnimated), triangle_models_rendering.rs:7-95,
	// with get_vertex_light (:702-720): the light cube plus the directional component
	float nm[3][3];
	normals_matrix(model_matrix, nm);
	model_vertices.resize(mesh.num_vertices);
	const Vec3* p0 = &mesh.positions[size_t(f0) * mesh.num_vertices];
	const Vec3* p1 = &mesh.positions[size_t(f1) * mesh.num_vertices];
	const Vec3* n0 = &mesh.normals[size_t(f0) * mesh.num_vertices];
	const Vec3* n1 = &mesh.normals[size_t(f1) * mesh.num_vertices];
	const Vec3* ps = lerp0 > lerp1 ? p0 : p1;
	const Vec3* ns = lerp0 > lerp1 ? n0 : n1;
	for (uint32_t i = 0; i < mesh.num_vertices; ++i)
	{
		const Vec3 pos = perform_lerp ? p0[i] * lerp0 + p1[i] * lerp1 : ps[i];
		const Vec3 nrm = perform_lerp ? n0[i] * lerp0 + n1[i] * lerp1 : ns[i];
		const Vec3 nt = v3(nm[0][0] * nrm.x + nm[0][1] * nrm.y + nm[0][2] * nrm.z, nm[1][0] * nrm.x + nm[1][1] * nrm.y + nm[1][2] * nrm.z,
			nm[2][0] * nrm.x + nm[2][1] * nrm.y + nm[2][2] * nrm.z);
		const Vec3 nn = nt * (1.0f / std::sqrt(std::fmax(dot(nt, nt), 0.00000001f)));
		ModelVertex3d& v = model_vertices[i];
		v.pos = view_transform(model_view, pos);
		v.tc[0] = mesh.tex_coords[2 * i] * float(tex.width);
		v.tc[1] = mesh.tex_coords[2 * i + 1] * float(tex.height);
		light_cube_light(e.light_cube, nn, v.light);
		const float ld = std::fmax(dot(nn, e.light_dir_scaled), 0.0f);
		for (int c = 0; c < 3; ++c) v.light[c] += e.light_color[c] * ld;
	}
	// reject_triangle_model_back_faces and sort_model_triangles (:324-381): front faces, back to front by
	// each triangle's greatest z
	model_triangles.clear();
	for (size_t k = 0; k + 2 < mesh.triangles.size(); k += 3)
	{
		const Vec3 a = model_vertices[mesh.triangles[k]].pos, b = model_vertices[mesh.triangles[k + 1]].pos,
				   c = model_vertices[mesh.triangles[k + 2]].pos;
		if (dot(cross(b - a, c - b), a) > 0.0f) model_triangles.push_back(uint32_t(k));
	}
	auto max_z = [&](uint32_t k) {
		return std::fmax(std::fmax(model_vertices[mesh.triangles[k]].pos.z, model_vertices[mesh.triangles[k + 1]].pos.z),
			model_vertices[mesh.triangles[k + 2]].pos.z);
	};
	std::stable_sort(model_triangles.begin(), model_triangles.end(), [&](uint32_t a, uint32_t b) { return max_z(a) > max_z(b); });

	// draw_mesh (:3525-3718): the near plane when the bbox crosses it, the leaf's box planes that are
	// tighter than the model's screen box, then fill_triangle for every triangle of each clipped fan
	bool near_needed = false, all_behind = true;
	ClippingPolygon mesh_box = ClippingPolygon::from_box(1e30f, 1e30f, -1e30f, -1e30f);
	bool first_point = true;
	for (int k = 0; k < 8; ++k)
	{
		const Vec3 corner = v3((k & 1) ? mesh.bbox_max.x : mesh.bbox_min.x, (k & 2) ? mesh.bbox_max.y : mesh.bbox_min.y,
			(k & 4) ? mesh.bbox_max.z : mesh.bbox_min.z);
		const Vec3 v = view_transform(model_view, corner);
		if (v.z >= PREP_Z_NEAR)
		{
			all_behind = false;
			const Vec2 sp = v2(v.x / v.z, v.y / v.z);
			if (first_point)
				mesh_box = ClippingPolygon::from_point(sp), first_point = false;
			else
				mesh_box.extend_with_point(sp);
		}
		else
			near_needed = true;
	}
	if (all_behind) return;
	Vec3 box_planes[2][8];
	bounds.get_clip_planes(box_planes[0]);
	mesh_box.get_clip_planes(box_planes[1]);
	Vec3 planes_2d[4];
	uint32_t num_2d = 0;
	for (int k = 0; k < 4; ++k)
		if (near_needed || box_planes[0][k].z > box_planes[1][k].z) planes_2d[num_2d++] = box_planes[0][k];

	ModelVertex3d c3[2][MAX_VERTICES];
	for (uint32_t k : model_triangles)
	{
		for (int i = 0; i < 3; ++i) c3[0][i] = model_vertices[mesh.triangles[k + i]];
		uint32_t n = 3;
		int src3 = 0;
		if (near_needed)
		{
			n = clip_model_near(c3[0], n, c3[1]);
			if (n < 3) continue;
			src3 = 1;
		}
		stats.model_triangles += emit_model_polygon(c3[src3], n, planes_2d, num_2d, tex, e.blending_mode, nullptr);
	}
}

// draw_mesh's and draw_sprite's tail (partial_renderer.rs:3380-3418, 3640-3718): project the camera-space
// polygon, clip it by the given 2D planes (clip_2d_model_polygon, src/common/clipping.rs:203-257), convert
// to fixed point (f32_to_fixed16) and emit one fill_triangle draw per triangle of the fan. `light`, when
// given, replaces every vertex's light (the tessellated sprite path). Returns the triangles emitted.
uint32_t FramePrep::emit_model_polygon(const ModelVertex3d* verts, uint32_t n, const Vec3* planes_2d, uint32_t num_2d,
	const LiteMip& tex, uint32_t blend, const float* light)
{
	struct V2
	{
		Vec2 pos;
		float tc[2], light[3];
	};
	auto clip2 = [&](const V2* src, uint32_t count, const Vec3& line, V2* dst) {
		uint32_t out = 0;
		const V2* prev = &src[count - 1];
		float prev_d = prev->pos.x * line.x + prev->pos.y * line.y - line.z;
		auto inter = [&](const V2& v0, const V2& v1) {
			const float d0 = v0.pos.x * line.x + v0.pos.y * line.y - line.z, d1 = v1.pos.x * line.x + v1.pos.y * line.y - line.z;
			const float sum = d1 - d0, k0 = d0 / sum, k1 = d1 / sum;
			V2 r;
			r.pos = v2(v0.pos.x * k1 - v1.pos.x * k0, v0.pos.y * k1 - v1.pos.y * k0);
			for (int i = 0; i < 2; ++i) r.tc[i] = v0.tc[i] * k1 - v1.tc[i] * k0;
			for (int i = 0; i < 3; ++i) r.light[i] = v0.light[i] * k1 - v1.light[i] * k0;
			return r;
		};
		for (uint32_t i = 0; i < count && out < MAX_VERTICES; ++i)
		{
			const V2& v = src[i];
			const float d = v.pos.x * line.x + v.pos.y * line.y - line.z;
			if (d > 0.0f)
			{
				if (prev_d < 0.0f && out < MAX_VERTICES) dst[out++] = inter(*prev, v);
				if (out < MAX_VERTICES) dst[out++] = v;
			}
			else if (d == 0.0f)
				dst[out++] = v;
			else if (prev_d > 0.0f)
				dst[out++] = inter(*prev, v);
			prev = &v;
			prev_d = d;
		}
		return out;
	};
	V2 c2[2][MAX_VERTICES];
	for (uint32_t i = 0; i < n; ++i)
	{
		const ModelVertex3d& v = verts[i];
		c2[0][i].pos = v2(v.pos.x / v.pos.z, v.pos.y / v.pos.z);
		for (int j = 0; j < 2; ++j) c2[0][i].tc[j] = v.tc[j];
		for (int j = 0; j < 3; ++j) c2[0][i].light[j] = v.light[j];
	}
	int src2 = 0;
	for (uint32_t pl = 0; pl < num_2d; ++pl)
	{
		n = clip2(c2[src2], n, planes_2d[pl], c2[src2 ^ 1]);
		if (n < 3) return 0;
		src2 ^= 1;
	}
	SwTriVertex fixed[MAX_VERTICES];
	for (uint32_t i = 0; i < n; ++i)
	{
		const V2& v = c2[src2][i];
		const float* l = light ? light : v.light;
		fixed[i] = SwTriVertex{to_fixed16(v.pos.x), to_fixed16(v.pos.y), {to_fixed16(v.tc[0]), to_fixed16(v.tc[1])},
			{to_fixed16(l[0]), to_fixed16(l[1]), to_fixed16(l[2])}, 0};
	}
	uint32_t emitted = 0;
	for (uint32_t tri = 0; tri + 2 < n; ++tri)
	{
		SwDrawCmd d;
		std::memset(&d, 0, sizeof(d));
		d.first_vertex = uint32_t(tri_vertices.size());
		d.vertex_count = 3;
		d.mode = SW_RASTER_TRIANGLE;
		d.blend = blend;
		d.tex_size[0] = tex.width;
		d.tex_size[1] = tex.height;
		d.tex_source = SW_TEXSRC_LITE;
		d.tex_offset = tex.offset;
		tri_vertices.push_back(fixed[0]);
		tri_vertices.push_back(fixed[tri + 1]);
		tri_vertices.push_back(fixed[tri + 2]);
		draws.push_back(d);
		++emitted;
	}
	return emitted;
}

const FramePrep::DecalInfo& FramePrep::prepare_decal(uint32_t decal_index)
{
	if (decal_info.size() < sc.decals.size()) decal_info.resize(sc.decals.size());
	DecalInfo& info = decal_info[decal_index];
	if (info.frame == current_frame) return info;
	info.frame = current_frame;
	const DecalEntity& d = sc.decals[decal_index];
	// get_object_matrix_with_scale: translate * rotate * scale (src/common/matrix.rs:111-122)
	Mat4 m = mat4_from_quat(d.rotation);
	m.c[0] = m.c[0] * d.scale.x;
	m.c[1] = m.c[1] * d.scale.y;
	m.c[2] = m.c[2] * d.scale.z;
	m.c[3] = v4(d.position.x, d.position.y, d.position.z, 1.0f);
	Mat4 inv;
	if (!invert(transpose(m), inv)) inv = Mat4::identity();
	info.planes = cam.planes_matrix * inv;
	// the light cube of the dynamic lights at the decal's position (LightCube, src/common/light_cube.rs)
	float cube[6][3] = {};
	Vec3 sum_dirs[3] = {v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0)};
	const float min_vec_len = 0.00000001f;
	if (d.lightmap_light_scale > 0.0f)
	{
		const float min_square_distance = magnitude2(d.scale) * 0.25f;
		for (size_t li = 0; li < lights.size(); ++li)
		{
			if (li < light_shadows.size() && light_shadows[li].kind != SW_SHADOW_NONE) continue;
			bool visible = false;
			if (li < light_leafs.size())
				for (uint32_t lf : light_leafs[li]) visible = visible || vis.visible(lf);
			if (!visible) continue;
			const SwLight& l = lights[li];
			const Vec3 to_light = v3(l.position[0], l.position[1], l.position[2]) - d.position;
			const float inv_square_dist = 1.0f / std::fmax(magnitude2(to_light), min_square_distance);
			const float light_inv_square_radius = 1.0f / (l.radius * l.radius);
			if (inv_square_dist < light_inv_square_radius) continue;
			const float scale = 1.0f * (inv_square_dist - light_inv_square_radius);
			const float ls[3] = {l.color[0] * scale, l.color[1] * scale, l.color[2] * scale};
			// add_light_sample
			const Vec3 dn = to_light / std::fmax(magnitude(to_light), min_vec_len);
			const float comps[3] = {dn.x, dn.y, dn.z};
			for (int a = 0; a < 3; ++a)
				for (int c = 0; c < 3; ++c)
				{
					if (comps[a] <= 0.0f)
						cube[2 * a][c] += ls[c] * (-comps[a]);
					else
						cube[2 * a + 1][c] += ls[c] * comps[a];
				}
			for (int c = 0; c < 3; ++c) sum_dirs[c] = sum_dirs[c] + dn * ls[c];
		}
	}
	// convert_into_light_grid_sample
	const Vec3 dir = 0.33f * (sum_dirs[0] + sum_dirs[1] + sum_dirs[2]);
	const float len2 = std::fmax(magnitude2(dir), min_vec_len);
	for (int c = 0; c < 3; ++c) info.color[c] = std::fmax(dot(sum_dirs[c], dir), 0.0f) / len2;
	const float dcomps[3] = {dir.x, dir.y, dir.z};
	for (int c = 0; c < 3; ++c)
		for (int a = 0; a < 3; ++a)
		{
			if (dcomps[a] <= 0.0f)
				cube[2 * a][c] = std::fmax(cube[2 * a][c] - info.color[c] * (-dcomps[a]), 0.0f);
			else
				cube[2 * a + 1][c] = std::fmax(cube[2 * a + 1][c] - info.color[c] * dcomps[a], 0.0f);
		}
	std::memcpy(info.cube, cube, sizeof(cube));
	info.dir = dir;
	return info;
}

// draw_polygon_decals (partial_renderer.rs:2794-2957): the decals of the leaf cut out of one polygon
void FramePrep::draw_polygon_decals(const Vec3 clip_planes[8], uint32_t polygon_index, const std::vector<uint32_t>& leaf_decals)
{
	const PolyData& pd = poly[polygon_index];
	if (pd.visible_frame != current_frame) return;
	const MapPolygon& polygon = sc.polygons[polygon_index];
	const uint32_t cur_material = polygon.texture < mapping.size() ? mapping[polygon.texture] : polygon.texture;
	if (!sc.materials[cur_material].decals) return;
	const Vec3 normal = sc.basis[polygon_index].normal;
	static const float CUBE_SIDES[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
	for (uint32_t di : leaf_decals)
	{
		const DecalEntity& d = sc.decals[di];
		if (dot(normal, rotate_vector(d.rotation, v3(-1, 0, 0))) < 0.1f) continue; // MAX_ANGLE_COS
		const DecalInfo& info = prepare_decal(di);
		Vec3 vc[2][MAX_VERTICES];
		uint32_t n = std::min<uint32_t>(polygon.num_vertices, MAX_VERTICES);
		for (uint32_t i = 0; i < n; ++i) vc[0][i] = vertices_transformed[polygon.first_vertex + i];
		int src = 0;
		bool cut = false;
		for (const float* side : CUBE_SIDES)
		{
			const Vec4 pv = info.planes * v4(side[0], side[1], side[2], 1.0f);
			const Vec3 pn = truncate(pv);
			const float pdist = -pv.w;
			// clip_3d_polygon_by_plane (src/common/clipping.rs:53-105)
			uint32_t out = 0;
			const Vec3* prev = &vc[src][n - 1];
			float prev_dist = dot(pn, *prev);
			auto inter = [&](const Vec3& v0, const Vec3& v1) {
				const float d0 = dot(v0, pn) - pdist, d1 = dot(v1, pn) - pdist;
				const float sum = d1 - d0, k0 = d0 / sum, k1 = d1 / sum;
				return v0 * k1 - v1 * k0;
			};
			for (uint32_t i = 0; i < n; ++i)
			{
				const Vec3& v = vc[src][i];
				const float dist = dot(pn, v);
				if (dist > pdist)
				{
					if (prev_dist < pdist)
					{
						vc[src ^ 1][out++] = inter(*prev, v);
						if (out == MAX_VERTICES) break;
					}
					vc[src ^ 1][out++] = v;
					if (out == MAX_VERTICES) break;
				}
				else if (dist == pdist)
				{
					vc[src ^ 1][out++] = v;
					if (out == MAX_VERTICES) break;
				}
				else if (prev_dist > pdist)
				{
					vc[src ^ 1][out++] = inter(*prev, v);
					if (out == MAX_VERTICES) break;
				}
				prev = &v;
				prev_dist = dist;
			}
			n = out;
			if (n < 3)
			{
				cut = true;
				break;
			}
			src ^= 1;
		}
		if (cut) continue;
		Vec2 projected[MAX_VERTICES];
		n = project_and_clip_polygon(clip_planes, vc[src], n, projected);
		if (n < 3) continue;
		const LiteMip& tex0 = sc.lite_mips[size_t(d.texture) * NUM_MIPS];
		const Vec4 basis0 = info.planes * (v4(0.0f, -0.5f, 0.0f, 0.5f) * float(tex0.width));
		const Vec4 basis1 = info.planes * (v4(0.0f, 0.0f, -0.5f, 0.5f) * float(tex0.height));
		const DepthEquation& de = pd.depth;
		TexCoordEquation tc; // from_depth_equation_and_transformed_tex_coord_equations (equations.rs:55-74)
		tc.d_tc_dx[0] = basis0.x + basis0.w * de.d_inv_z_dx;
		tc.d_tc_dx[1] = basis1.x + basis1.w * de.d_inv_z_dx;
		tc.d_tc_dy[0] = basis0.y + basis0.w * de.d_inv_z_dy;
		tc.d_tc_dy[1] = basis1.y + basis1.w * de.d_inv_z_dy;
		tc.k[0] = basis0.z + basis0.w * de.k;
		tc.k[1] = basis1.z + basis1.w * de.k;
		const uint32_t mip = calculate_mip(projected, n, de, tc, opt.mip_bias);
		const LiteMip& tex = sc.lite_mips[size_t(d.texture) * NUM_MIPS + mip];
		const float ms = 1.0f / float(1 << mip);
		TexCoordEquation tcs;
		for (int i = 0; i < 2; ++i)
			tcs.d_tc_dx[i] = tc.d_tc_dx[i] * ms, tcs.d_tc_dy[i] = tc.d_tc_dy[i] * ms, tcs.k[i] = tc.k[i] * ms;
		// the polygon's surface coordinates give the lightmap coordinates of the decal's points
		const float lm_scale = float(1 << pd.mip) / float(LIGHTMAP_SCALE);
		const float lm_shift[2] = {float(pd.tc_min[0]) * lm_scale - float(polygon.tex_coord_min[0] >> LIGHTMAP_SCALE_LOG2),
			float(pd.tc_min[1]) * lm_scale - float(polygon.tex_coord_min[1] >> LIGHTMAP_SCALE_LOG2)};
		TexCoordEquation lm;
		for (int i = 0; i < 2; ++i)
			lm.d_tc_dx[i] = pd.tc.d_tc_dx[i] * lm_scale, lm.d_tc_dy[i] = pd.tc.d_tc_dy[i] * lm_scale, lm.k[i] = pd.tc.k[i] * lm_scale;
		float dyn[3];
		light_cube_light(info.cube, normal, dyn);
		const float dir_dot = std::fmax(dot(normal, info.dir), 0.0f);
		for (int c = 0; c < 3; ++c) dyn[c] += dir_dot * info.color[c];
		for (uint32_t t = 0; t + 2 < n; ++t)
		{
			const Vec2 tri[3] = {projected[0], projected[t + 1], projected[t + 2]};
			subdivide_decal_triangle(d, polygon, de, tcs, lm, lm_shift, tri, tex, dyn, 0);
		}
	}
}

namespace
{
// get_polygon_lightmap_light (partial_renderer.rs:3807-3875): the polygon's simple lightmap, bilinear,
// renormalised where samples fall outside it
void polygon_lightmap_light(const Scene& sc, const MapPolygon& p, Vec2 c, float out[3])
{
	out[0] = out[1] = out[2] = 0.0f;
	if (p.lightmap_data_offset == 0 || sc.lightmaps.empty()) return;
	const float* data = &sc.lightmaps[size_t(p.lightmap_data_offset) * 3];
	const int32_t ci[2] = {as_i32(std::floor(c.x)), as_i32(std::floor(c.y))};
	const int32_t lw = ((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1;
	const int32_t lh = ((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1;
	float total_factor = 0.0f;
	for (int dy = 0; dy <= 1; ++dy)
	{
		const int32_t y = ci[1] + dy;
		if (y < 0 || y >= lh) continue;
		const float fy = 1.0f - std::fabs(c.y - float(y));
		for (int dx = 0; dx <= 1; ++dx)
		{
			const int32_t x = ci[0] + dx;
			if (x < 0 || x >= lw) continue;
			const float fx = 1.0f - std::fabs(c.x - float(x));
			const float* l = data + size_t(x + y * lw) * 3;
			const float f = fx * fy;
			for (int i = 0; i < 3; ++i) out[i] += f * l[i];
			total_factor += f;
		}
	}
	if (total_factor < 1.0f)
	{
		const float inv = 1.0f / total_factor;
		for (int i = 0; i < 3; ++i) out[i] *= inv;
	}
}
} // namespace

// subdivide_and_draw_decal_triangle (partial_renderer.rs:2959-3080)
void FramePrep::subdivide_decal_triangle(const DecalEntity& d, const MapPolygon& polygon, const DepthEquation& de,
	const TexCoordEquation& tc, const TexCoordEquation& lm_eq, const float lm_shift[2], const Vec2 pts[3], const LiteMip& tex,
	const float dyn[3], int depth)
{
	const Vec2* min_p = &pts[0];
	const Vec2* max_p = &pts[0];
	float min_inv_z = de.sample(pts[0]), max_inv_z = min_inv_z;
	for (int k = 1; k < 3; ++k)
	{
		const float iz = de.sample(pts[k]);
		if (iz < min_inv_z) min_inv_z = iz, min_p = &pts[k];
		if (iz > max_inv_z) max_inv_z = iz, max_p = &pts[k];
	}
	if (depth >= 2 || affine_may_be_used(de, tc, *min_p, *max_p))
	{
		const float tc_eps = 1.0f / 32.0f;
		const float max_tc[2] = {float(tex.width) - tc_eps, float(tex.height) - tc_eps};
		SwTriVertex v[3];
		for (int k = 0; k < 3; ++k)
		{
			const Vec2& p = pts[k];
			const float z = 1.0f / de.sample(p);
			float light[3] = {d.light_add[0], d.light_add[1], d.light_add[2]};
			if (d.lightmap_light_scale > 0.0f)
			{
				const Vec2 lc = v2(z * (lm_eq.d_tc_dx[0] * p.x + lm_eq.d_tc_dy[0] * p.y + lm_eq.k[0]) + lm_shift[0],
					z * (lm_eq.d_tc_dx[1] * p.x + lm_eq.d_tc_dy[1] * p.y + lm_eq.k[1]) + lm_shift[1]);
				float lml[3];
				polygon_lightmap_light(sc, polygon, lc, lml);
				for (int i = 0; i < 3; ++i)
				{
					light[i] += lml[i] * d.lightmap_light_scale;
					light[i] += dyn[i];
				}
			}
			const float u = std::fmin(std::fmax(z * (tc.d_tc_dx[0] * p.x + tc.d_tc_dy[0] * p.y + tc.k[0]), tc_eps), max_tc[0]);
			const float w = std::fmin(std::fmax(z * (tc.d_tc_dx[1] * p.x + tc.d_tc_dy[1] * p.y + tc.k[1]), tc_eps), max_tc[1]);
			v[k] = SwTriVertex{to_fixed16(p.x), to_fixed16(p.y), {to_fixed16(u), to_fixed16(w)},
				{to_fixed16(light[0]), to_fixed16(light[1]), to_fixed16(light[2])}, 0};
		}
		SwDrawCmd c;
		std::memset(&c, 0, sizeof(c));
		c.first_vertex = uint32_t(tri_vertices.size());
		c.vertex_count = 3;
		c.mode = SW_RASTER_TRIANGLE;
		c.blend = d.blending_mode;
		c.tex_size[0] = tex.width;
		c.tex_size[1] = tex.height;
		c.tex_source = SW_TEXSRC_LITE;
		c.tex_offset = tex.offset;
		for (int k = 0; k < 3; ++k) tri_vertices.push_back(v[k]);
		draws.push_back(c);
		++stats.model_triangles;
		return;
	}
	const Vec2 c0 = (pts[0] + pts[1]) / 2.0f, c1 = (pts[1] + pts[2]) / 2.0f, c2 = (pts[2] + pts[0]) / 2.0f;
	const Vec2 subs[4][3] = {{pts[0], c0, c2}, {pts[1], c1, c0}, {pts[2], c2, c1}, {c0, c1, c2}};
	for (const auto& s : subs) subdivide_decal_triangle(d, polygon, de, tc, lm_eq, lm_shift, s, tex, dyn, depth + 1);
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

template <class F>
void FramePrep::for_each_drawn_leaf(F&& f)
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
			if (!vis.visible(leaf)) continue;
			ClippingPolygon b = vis.bounds(leaf);
			b.intersect(viewport);
			if (b.is_valid_and_non_empty())
			{
				++stats.visible_leafs;
				f(b, leaf);
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

void FramePrep::draw_tree()
{
	for_each_drawn_leaf([this](const ClippingPolygon& b, uint32_t leaf) { draw_leaf(b, leaf); });
}

void FramePrep::begin_frame(const CameraMatrices& camera, const std::vector<SwLight>& frame_lights, const FrameOptions& options,
	Quat skybox_rotation)
{
	cam = camera;
	opt = options;
	sky_rotation = skybox_rotation;
	lights = frame_lights;
	stats = FrameStats();
	++current_frame;
	vis.update(cam, ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
	stats.camera_leaf = vis.camera_leaf;
	position_lights();
	prepare_shadows();
	update_materials();
}

void FramePrep::update_materials()
{
	// MapMaterialsProcessor::update (map_materials_processor.rs:174-247) at the frame's time, once per
	// frame. Framed animations (:184-227): a mapping entry whose current frame has a next frame moves to
	// it once the time reaches its change point, which then advances by the new frame's duration (0.5 s
	// without one) and is not left behind the current time. Scrolling (:229-247): `(speed * t) as i32`
	// rem_euclid the mip-0 size. get_texture / get_texture_shift (:311-334) read both through the mapping.
	const uint32_t n = uint32_t(sc.materials.size());
	if (mapping.size() != n)
	{
		mapping.resize(n);
		change_time.assign(n, 0.0f);
		for (uint32_t m = 0; m < n; ++m) mapping[m] = m;
	}
	std::vector<int32_t> shift(2 * size_t(n), 0);
	animated = false;
	for (uint32_t m = 0; m < n; ++m)
	{
		const Material& mat = sc.materials[m];
		if (mat.next_frame >= 0) animated = true;
		for (int i = 0; i < 2; ++i)
			if (mat.scroll_speed[i] != 0.0f)
			{
				const int32_t size = int32_t(mat.texture_size);
				const int32_t s = as_i32(mat.scroll_speed[i] * frame_time_s) % size;
				shift[2 * m + i] = s < 0 ? s + size : s;
				animated = true;
			}
	}
	for (uint32_t m = 0; m < n; ++m)
	{
		const int32_t next = sc.materials[mapping[m]].next_frame;
		if (next < 0 || uint32_t(next) >= n || !(frame_time_s >= change_time[m])) continue;
		mapping[m] = uint32_t(next);
		const Material& cur = sc.materials[uint32_t(next)];
		change_time[m] += cur.next_frame >= 0 ? cur.frame_duration : 0.5f;
		if (change_time[m] < frame_time_s) change_time[m] = frame_time_s;
	}
	// update_animations (:249-303) runs after the framed animations and shifts, before anything reads the
	// textures
	update_texture_effects();
	update_simulations();
	material_frames.resize(n);
	for (uint32_t m = 0; m < n; ++m)
	{
		// get_texture (:311-327): the current frame's generated texture when it has a generative effect
		// (simulated ones once they have generated one); get_material and get_emissive_texture (:305-309,
		// 336-360): the current frame's properties
		const Material& cur = sc.materials[mapping[m]];
		const EffectSim* sim = effect_sim(mapping[m]);
		const bool generated = !sim || sim->generated();
		SwMaterialFrame& f = material_frames[m];
		f.shift[0] = shift[2 * mapping[m]];
		f.shift[1] = shift[2 * mapping[m] + 1];
		f.texture = (cur.effect_texture >= 0 && generated) ? uint32_t(cur.effect_texture) : mapping[m];
		f.flags = Scene::material_polygon_flags(cur);
		f.blending_mode = cur.blending_mode;
		f.emissive_texture = cur.emissive >= 0 ? uint32_t(cur.emissive) : SW_NO_EMISSIVE;
		if (cur.emissive >= 0 && cur.effect_emissive >= 0 && generated) f.emissive_texture = uint32_t(cur.effect_emissive);
		for (int c = 0; c < 3; ++c) f.emissive_light[c] = cur.emissive_light[c];
		f.reserved = 0;
		if (cur.effect != Material::NO_EFFECT) animated = true;
	}
	apply_material_frames();
}

void FramePrep::apply_material_frames()
{
	// the polygons the host prepares read the frame's material fields
	for (uint32_t m = 0; m < uint32_t(material_frames.size()) && m < uint32_t(material_polygons.size()); ++m)
	{
		const SwMaterialFrame& f = material_frames[m];
		for (uint32_t pi : material_polygons[m])
		{
			SwMapPolygon& p = map_polygons[pi];
			p.flags = f.flags;
			p.blending_mode = f.blending_mode;
			p.emissive_texture = f.emissive_texture;
			for (int c = 0; c < 3; ++c) p.emissive_light[c] = f.emissive_light[c];
		}
	}
}

void FramePrep::update_simulations()
{
	// the water and fire effects' GenerativeTextureEffect::update at the frame's time (their state persists
	// from frame to frame; each is created, running its equilibrium steps, on its first update)
	simulations.clear();
	sims.resize(sc.materials.size());
	for (uint32_t m = 0; m < uint32_t(sc.materials.size()); ++m)
	{
		const Material& mat = sc.materials[m];
		if (mat.effect != Material::WATER && mat.effect != Material::FIRE) continue;
		if (!sims[m]) sims[m].reset(new EffectSim(mat, mat.sim_state));
		SimTextures t;
		std::memset(&t, 0, sizeof(t));
		t.source_texture = m;
		t.output_texture = mat.effect_texture;
		t.output_emissive = mat.effect_emissive;
		t.source_emissive = mat.emissive;
		// the source's last mip's first texel (water.rs:280), Material::roughness clamped (:289)
		t.base_color = uint32_t(sc.texels[sc.texture_mips[size_t(m) * NUM_MIPS + NUM_MIPS - 1].offset]);
		t.roughness = std::fmin(std::fmax(mat.roughness, 1.0f / 126.0f), 1.0f);
		if (mat.emissive >= 0)
		{
			const SwEmissiveMip& em = sc.emissive_mips[size_t(mat.emissive) * NUM_MIPS];
			t.emissive_width = em.width * em.height ? em.width : 0;
			t.emissive_row = sc.emissive_pixels.data() + em.offset;
		}
		sims[m]->update(frame_time_s, t, simulations);
	}
	simulations.finish();
}

void FramePrep::update_texture_effects()
{
	// update_animations (map_materials_processor.rs:249-303) with the default update period of one frame:
	// every effect's GenerativeTextureEffect::update at the frame's time, as texture passes.
	const float tau = 6.28318530717958647692f;
	texture_passes.clear();
	texture_shifts.clear();
	turb_buffers.resize(sc.materials.size());
	for (uint32_t m = 0; m < uint32_t(sc.materials.size()); ++m)
	{
		const Material& mat = sc.materials[m];
		if (mat.effect == Material::NO_EFFECT) continue;
		for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
		{
			const uint32_t dst = uint32_t(mat.effect_texture) * NUM_MIPS + mip;
			if (mat.effect == Material::TURB)
			{
				// make_turb_distortion (generative_texture_effect_turb.rs:91-138): the shift table, kept in the
				// effect's buffer (resized to max(w, h), only the first w entries rewritten)
				const SwTextureMip& src = sc.texture_mips[m * NUM_MIPS + mip];
				std::vector<int32_t>& buf = turb_buffers[m];
				buf.resize(std::max(src.width, src.height), 0);
				const float mip_scale = 1.0f / float(1 << mip);
				const float amplitude = mip_scale * mat.turb_amplitude;
				const float frequency_scaled = tau / (mat.turb_wave_length * mip_scale);
				const float time_shift = frame_time_s * mat.turb_frequency * tau;
				for (uint32_t x = 0; x < src.width; ++x)
					buf[x] = as_i32(std::round(std::sin(float(x) * frequency_scaled + time_shift) * amplitude));
				SwTexturePass p;
				std::memset(&p, 0, sizeof(p));
				p.kind = SW_TEXPASS_TURB;
				p.dst_mip = dst;
				p.src_mip = m * NUM_MIPS + mip;
				p.shifts_offset = uint32_t(texture_shifts.size());
				texture_shifts.insert(texture_shifts.end(), buf.begin(), buf.end());
				texture_passes.push_back(p);
				continue;
			}
			// GenerativeTextureEffectLayered::update (generative_texture_effect_layered.rs:63-161)
			for (const EffectLayer& l : mat.layers)
			{
				SwTexturePass p;
				std::memset(&p, 0, sizeof(p));
				p.kind = SW_TEXPASS_LAYER;
				p.dst_mip = dst;
				for (int i = 0; i < 2; ++i) p.shift[i] = as_i32(l.tex_coord_shift[i].evaluate(frame_time_s)) >> mip;
				const float max_light = 127.0f;
				for (int c = 0; c < 3; ++c)
				{
					float v = 1.0f;
					if (l.has_modulate_color) v = l.modulate_color[c].evaluate(frame_time_s);
					else if (l.has_modulate) v = l.modulate.evaluate(frame_time_s);
					if (l.has_modulate_color || l.has_modulate) v = std::fmin(std::fmax(v, 0.0f), max_light);
					p.light[c] = v;
				}
				const uint32_t tex = l.follow_framed_animation ? mapping[l.material] : l.material;
				const Material& lm = sc.materials[tex];
				if (!lm.has_diffuse) continue;
				p.src_mip = tex * NUM_MIPS + mip;
				p.blending_mode = lm.blending_mode;
				texture_passes.push_back(p);
			}
		}
	}
}

void FramePrep::finish_params()
{
	std::memset(&params, 0, sizeof(params));
	params.pixel_format = opt.pixel_format;
	params.width = opt.width;
	params.height = opt.height;
	params.use_directional_lightmaps = (opt.use_directional_lightmaps && sc.directional_lightmaps.size() > 1) ? 1u : 0u;
	params.cam_pos[0] = cam.position.x;
	params.cam_pos[1] = cam.position.y;
	params.cam_pos[2] = cam.position.z;
	params.clear_background = opt.clear_background ? 1u : 0u;
}

void FramePrep::prepare_with_camera(const CameraMatrices& camera, const std::vector<SwLight>& frame_lights,
	const FrameOptions& options, Quat skybox_rotation)
{
	shadow_view = false;
	begin_frame(camera, frame_lights, options, skybox_rotation);
	prepare_polygons_surfaces();
	build_surface_descs();
	finish_view(ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
}

void FramePrep::prepare_view_with_camera(const CameraMatrices& camera, const std::vector<SwLight>& frame_lights,
	const FrameOptions& options, Quat skybox_rotation)
{
	shadow_view = true;
	begin_frame(camera, frame_lights, options, skybox_rotation);
	// The visible leafs in index order (prepare_polygons_surfaces' order, :1327-1359) with their bounds and
	// lights; the sky polygons' bounds are collected here, every other polygon is the GPU's.
	view_leafs.clear();
	view_leaf_lights.clear();
	surfaces.clear();
	visible_polygons.clear();
	total_texels = 0;
	has_sky = false;
	for (uint32_t i = 0; i < sc.leafs.size(); ++i)
	{
		if (!vis.visible(i)) continue;
		const BspLeaf& leaf = sc.leafs[i];
		leaf_view_index[i] = uint32_t(view_leafs.size());
		SwViewLeaf vl;
		std::memset(&vl, 0, sizeof(vl));
		vl.first_polygon = leaf.first_polygon;
		vl.num_polygons = leaf.num_polygons;
		vl.first_light = uint32_t(view_leaf_lights.size());
		vl.num_lights = uint32_t(leaf_lights[i].size());
		for (uint32_t li : leaf_lights[i]) view_leaf_lights.push_back(uint16_t(li));
		vl.draw_order = SW_LEAF_NOT_DRAWN;
		Vec3 planes[8];
		vis.bounds(i).get_clip_planes(planes);
		for (int k = 0; k < 8; ++k)
		{
			vl.clip_planes[k][0] = planes[k].x;
			vl.clip_planes[k][1] = planes[k].y;
			vl.clip_planes[k][2] = planes[k].z;
		}
		view_leafs.push_back(vl);
		for (uint32_t k = leaf_sky_first[i]; k < leaf_sky_first[i + 1]; ++k)
		{
			const SwMapPolygon& p = map_polygons[sky_polygons[k]];
			Vec3 vt[MAX_VERTICES];
			Vec2 v2d[MAX_VERTICES];
			uint32_t count = 0;
			SurfacePrep sp;
			if (swhost::prepare_polygon_surface(p, sc.vertices.data(), cam.view_matrix, cam.planes_matrix, planes, opt.mip_bias, vt,
					v2d, &count, sp) == PREP_SKY)
				extend_sky_bounds(v2d, count);
		}
	}
	draws.clear();
	vertices.clear();
	draw_skybox(ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
	uint32_t order = 0;
	for_each_drawn_leaf([this, &order](const ClippingPolygon& b, uint32_t leaf) {
		SwViewLeaf& vl = view_leafs[leaf_view_index[leaf]];
		vl.draw_order = order++;
		Vec3 planes[8];
		b.get_clip_planes(planes);
		for (int k = 0; k < 8; ++k)
		{
			vl.draw_clip_planes[k][0] = planes[k].x;
			vl.draw_clip_planes[k][1] = planes[k].y;
			vl.draw_clip_planes[k][2] = planes[k].z;
		}
	});
	finish_params();
	stats.draws = uint32_t(draws.size());
}

void FramePrep::camera_of_frame(uint32_t frame_index, const FrameOptions& options, CameraMatrices& camera,
	std::vector<SwLight>& frame_lights, Quat& skybox_rotation) const
{
	const CameraKey& k = sc.camera_path[frame_index % sc.camera_path.size()];
	camera = build_view_matrix(k.position, k.azimuth, k.elevation, options.fov, float(options.width), float(options.height));
	sc.frame_lights(frame_index % uint32_t(sc.camera_path.size()), frame_lights);
	skybox_rotation = quat_from_angle_z(float(frame_index) * sc.config.sky_rotation_speed);
}

void FramePrep::prepare(uint32_t frame_index, const FrameOptions& options)
{
	frame_time_s = float(frame_index) * (1.0f / 60.0f);
	CameraMatrices camera;
	std::vector<SwLight> l;
	Quat rotation;
	camera_of_frame(frame_index, options, camera, l, rotation);
	prepare_with_camera(camera, l, options, rotation);
}

void FramePrep::prepare_view(uint32_t frame_index, const FrameOptions& options)
{
	frame_time_s = float(frame_index) * (1.0f / 60.0f);
	CameraMatrices camera;
	std::vector<SwLight> l;
	Quat rotation;
	camera_of_frame(frame_index, options, camera, l, rotation);
	prepare_view_with_camera(camera, l, options, rotation);
}


// ---- portals (partial_renderer.rs:1834-2283, 3720-3772) --------------------------------------------

void FramePrep::ViewBlock::clear()
{
	surfaces.clear();
	lights.clear();
	light_shadows.clear();
	depth_draws.clear();
	depth_vertices.clear();
	shadow_texels = 0;
	draws.clear();
	vertices.clear();
	tri_vertices.clear();
	views.clear();
}

void FramePrep::prepare_portals()
{
	// prepare_view_portals_textures (:1834-1996): each portal seen through the visible leafs it lies in
	// gets a texture of its texture-coordinate extent at its mip, placed after this view's surfaces
	portal_infos.assign(sc.view_portals.size(), PortalInfo());
	for (uint32_t i = 0; i < uint32_t(sc.view_portals.size()); ++i)
	{
		const ViewPortal& portal = sc.view_portals[i];
		bool any = false;
		ClippingPolygon bounds{};
		for (uint32_t leaf : sc.view_portal_leafs[i])
			if (vis.visible(leaf))
			{
				if (any)
					bounds.extend(vis.bounds(leaf));
				else
					bounds = vis.bounds(leaf);
				any = true;
			}
		if (!any) continue; // in invisible leafs
		Vec3 clip_planes[8];
		bounds.get_clip_planes(clip_planes);
		const Vec4 plane_transformed = cam.planes_matrix * extend(portal.plane.vec, -portal.plane.dist);
		if (plane_transformed.w <= 0.0f) continue;
		const uint32_t nv = std::min(uint32_t(portal.vertices.size()), uint32_t(MAX_VERTICES));
		if (nv < 3) continue;
		Vec3 vt[MAX_VERTICES];
		for (uint32_t k = 0; k < nv; ++k) vt[k] = view_transform(cam.view_matrix, portal.vertices[k]);
		Vec2 v2d[MAX_VERTICES];
		const uint32_t count = project_and_clip_polygon(clip_planes, vt, nv, v2d);
		if (count < 3) continue; // fully clipped
		const float inf = float(1 << 29);
		float tc_min[2] = {inf, inf}, tc_max[2] = {-inf, -inf};
		for (const Vec3& v : portal.vertices)
			for (int c = 0; c < 2; ++c)
			{
				const float tc = dot(portal.tex_coord_equation[c].vec, v) + portal.tex_coord_equation[c].dist;
				if (tc < tc_min[c]) tc_min[c] = tc;
				if (tc > tc_max[c]) tc_max[c] = tc;
			}
		for (int c = 0; c < 2; ++c)
		{
			tc_min[c] += 1.0f / 32.0f;
			tc_max[c] -= 1.0f / 32.0f;
		}
		// DepthEquation::from_transformed_plane_equation and the tc equations projected onto the plane
		const float pw = -plane_transformed.w;
		const DepthEquation de{plane_transformed.x / pw, plane_transformed.y / pw, plane_transformed.z / pw};
		TexCoordEquation te;
		for (int c = 0; c < 2; ++c)
		{
			const Vec4 tb = cam.planes_matrix * extend(portal.tex_coord_equation[c].vec, portal.tex_coord_equation[c].dist);
			te.d_tc_dx[c] = tb.x + tb.w * de.d_inv_z_dx;
			te.d_tc_dy[c] = tb.y + tb.w * de.d_inv_z_dy;
			te.k[c] = tb.z + tb.w * de.k;
		}
		const uint32_t mip = calculate_mip(v2d, count, de, te, opt.mip_bias);
		const float mip_scale = 1.0f / float(1u << mip);
		PortalInfo& info = portal_infos[i];
		int32_t tmin[2], tmax[2];
		for (int c = 0; c < 2; ++c)
		{
			te.d_tc_dx[c] = te.d_tc_dx[c] * mip_scale;
			te.d_tc_dy[c] = te.d_tc_dy[c] * mip_scale;
			te.k[c] = te.k[c] * mip_scale;
			tmin[c] = as_i32(std::floor(tc_min[c]) * mip_scale);
			tmax[c] = std::max(as_i32(std::ceil(tc_max[c]) * mip_scale), tmin[c] + 1);
		}
		for (int c = 0; c < 2; ++c)
		{
			const float m = float(tmin[c]);
			te.d_tc_dx[c] -= m * de.d_inv_z_dx;
			te.d_tc_dy[c] -= m * de.d_inv_z_dy;
			te.k[c] -= m * de.k;
			info.resolution[c] = uint32_t(tmax[c] - tmin[c]);
			info.tc_min[c] = tmin[c];
		}
		info.pixels_offset = arena_end;
		info.depth = de;
		info.tc = te;
		info.mip = mip;
		arena_end += uint64_t(info.resolution[0]) * info.resolution[1];
	}

	// build_view_portals_textures (:2008-2283): each visible portal's view rendered by the nested renderer
	// (black without one: the depth limit), then mixed with the portal's texture
	for (uint32_t i = 0; i < uint32_t(sc.view_portals.size()); ++i)
	{
		const PortalInfo& info = portal_infos[i];
		const uint32_t w = info.resolution[0], h = info.resolution[1];
		if (uint64_t(w) * h == 0) continue;
		const ViewPortal& portal = sc.view_portals[i];
		if (portals_depth == 0)
		{
			gather_nested(nullptr, info.pixels_offset, w, h, portal, info);
			continue;
		}
		if (!portal_renderer)
		{
			portal_renderer.reset(new FramePrep(sc));
			portal_renderer->portals_depth = portals_depth - 1;
		}
		const float z_near = PREP_Z_NEAR;
		const float mip_scale = 1.0f / float(1u << info.mip);
		CameraMatrices pc;
		std::vector<uint32_t> start;
		const std::vector<uint32_t>* start_leafs = nullptr;
		// the tc-space basis of the portal plane: tc equations and the plane scaled to the mip (as rows)
		auto tex_coord_basis = [&](float normal_len) {
			Mat4 b;
			b.c[0] = extend(portal.tex_coord_equation[0].vec, portal.tex_coord_equation[0].dist) * mip_scale;
			b.c[1] = extend(portal.tex_coord_equation[1].vec, portal.tex_coord_equation[1].dist) * mip_scale;
			b.c[2] = extend(portal.plane.vec, -portal.plane.dist) * (mip_scale / normal_len);
			b.c[3] = v4(0.0f, 0.0f, 0.0f, 1.0f);
			return transpose(b);
		};
		auto view_of = [&](const Mat4& basis, Vec3 eye_tc, float dist_normalized) {
			Mat4 translate = Mat4::identity();
			translate.c[3] = v4(-eye_tc.x, -eye_tc.y, -eye_tc.z, 1.0f);
			Mat4 shift = Mat4::identity();
			shift.c[2].x = eye_tc.x - float(info.tc_min[0]);
			shift.c[2].y = eye_tc.y - float(info.tc_min[1]);
			// the portal plane becomes the near plane: what lies behind it is clipped
			Mat4 z_scale = Mat4::identity();
			z_scale.c[0].x = z_near;
			z_scale.c[1].y = z_near;
			z_scale.c[2].z = z_near / (dist_normalized * mip_scale);
			return shift * z_scale * translate * basis;
		};
		if (portal.kind == ViewPortal::CAMERA_AT_POSITION)
			pc = build_view_matrix_with_full_rotation(portal.position, portal.rotation, portal.fov, float(w), float(h));
		else if (portal.kind == ViewPortal::MIRROR)
		{
			const float normal_square_len = magnitude2(portal.plane.vec);
			const float normal_len = std::sqrt(normal_square_len);
			const float dist = dot(portal.plane.vec, cam.position) - portal.plane.dist;
			const Vec3 reflected = cam.position - portal.plane.vec * (2.0f * dist / normal_square_len);
			const float dist_normalized = dist / normal_len;
			const Mat4 basis = tex_coord_basis(normal_len);
			const Vec3 eye_tc = truncate(basis * extend(reflected, 1.0f));
			pc.position = reflected;
			pc.view_matrix = view_of(basis, eye_tc, dist_normalized);
			if (!invert(transpose(pc.view_matrix), pc.planes_matrix)) pc.planes_matrix = Mat4::identity();
			start_leafs = &sc.view_portal_leafs[i]; // the search starts in the mirror's leafs
		}
		else
		{
			// the portal's vertices moved by the transform: their leafs start the search
			std::vector<Vec3> moved(portal.vertices.size());
			for (size_t k = 0; k < moved.size(); ++k) moved[k] = truncate(portal.transform * extend(portal.vertices[k], 1.0f));
			sc.convex_hull_leafs(moved.data(), std::min(uint32_t(moved.size()), uint32_t(MAX_VERTICES)), start);
			start_leafs = &start;
			const float normal_len = magnitude(portal.plane.vec);
			const float dist_normalized = (portal.plane.dist - dot(portal.plane.vec, cam.position)) / normal_len;
			const Mat4 basis = tex_coord_basis(normal_len);
			const Vec3 eye_tc = truncate(basis * extend(cam.position, 1.0f));
			Mat4 inverse_transform;
			if (!invert(portal.transform, inverse_transform)) inverse_transform = Mat4::identity();
			pc.position = truncate(portal.transform * extend(cam.position, 1.0f));
			pc.view_matrix = view_of(basis, eye_tc, dist_normalized) * inverse_transform;
			if (!invert(transpose(pc.view_matrix), pc.planes_matrix)) pc.planes_matrix = Mat4::identity();
		}
		portal_renderer->prepare_nested(*this, pc, start_leafs, w, h);
		gather_nested(portal_renderer.get(), info.pixels_offset, w, h, portal, info);
	}
}

void FramePrep::prepare_nested(const FramePrep& parent, const CameraMatrices& camera, const std::vector<uint32_t>* start_leafs,
	uint32_t width, uint32_t height)
{
	// PartialRenderer::prepare_frame + draw_frame of the nested renderer (:156-258) for one portal: the
	// frame's lights, materials and time, the portal's camera and resolution
	shadow_view = false;
	cam = camera;
	opt = parent.opt;
	opt.width = width;
	opt.height = height;
	sky_rotation = parent.sky_rotation;
	lights = parent.lights; // the frame's lights (the parent's nested views are appended after its own draws)
	frame_time_s = parent.frame_time_s;
	stats = FrameStats();
	++current_frame;
	const ClippingPolygon frame_bounds = ClippingPolygon::from_box(0.0f, 0.0f, float(width), float(height));
	if (start_leafs)
		vis.update_with_start_leafs(cam, frame_bounds, start_leafs->data(), uint32_t(start_leafs->size()));
	else
		vis.update(cam, frame_bounds);
	stats.camera_leaf = vis.camera_leaf;
	position_lights();
	prepare_shadows();
	// the materials processor is the frame's: the parent's current frames and shifts
	mapping = parent.mapping;
	material_frames = parent.material_frames;
	animated = parent.animated;
	apply_material_frames();
	texture_passes.clear();
	texture_shifts.clear();
	simulations.clear();
	prepare_polygons_surfaces();
	build_surface_descs();
	finish_view(frame_bounds);
	// draw_frame's background: camera views as the root frame, mirrors and parallax portals never
	params.clear_background = (opt.clear_background && !start_leafs) ? 1u : 0u;
}

// The view's draws after its surfaces: its portals' textures (nested views), then skybox and tree, then
// the nested views' outputs appended behind its own.
void FramePrep::finish_view(const ClippingPolygon& viewport)
{
	surface_texels = total_texels;
	arena_end = total_texels;
	draws.clear();
	vertices.clear();
	tri_vertices.clear();
	views.clear();
	nested.clear();
	prepare_portals();
	// perform_rasterization_for_viewport_part (:1285-1325): skybox first, then the tree
	draw_skybox(viewport);
	draw_tree();
	main_draws = uint32_t(draws.size());
	finish_params();
	stats.visible_polygons = uint32_t(visible_polygons.size());
	stats.draws = uint32_t(draws.size());
	stats.surface_texels = surface_texels;
	append_nested();
}

void FramePrep::gather_nested(const FramePrep* n, uint64_t target_offset, uint32_t width, uint32_t height,
	const ViewPortal& portal, const PortalInfo& info)
{
	const uint64_t arena_base = arena_end;
	const uint32_t draw_base = uint32_t(nested.draws.size());
	if (n)
	{
		const uint32_t light_base = uint32_t(nested.lights.size());
		const uint64_t shadow_base = nested.shadow_texels;
		const uint32_t depth_vertex_base = uint32_t(nested.depth_vertices.size());
		const uint32_t vertex_base = uint32_t(nested.vertices.size()), tri_base = uint32_t(nested.tri_vertices.size());
		for (SwSurfaceDesc d : n->surfaces)
		{
			d.out_offset += arena_base;
			for (uint32_t k = 0; k < d.num_lights; ++k) d.lights[k] = uint16_t(d.lights[k] + light_base);
			nested.surfaces.push_back(d);
		}
		nested.lights.insert(nested.lights.end(), n->lights.begin(), n->lights.end());
		for (size_t l = 0; l < n->lights.size(); ++l)
		{
			SwLightShadow s;
			std::memset(&s, 0, sizeof(s));
			if (l < n->light_shadows.size()) s = n->light_shadows[l];
			if (s.kind != SW_SHADOW_NONE) s.offset += shadow_base;
			nested.light_shadows.push_back(s);
		}
		for (SwDepthDraw d : n->depth_draws)
		{
			d.map_offset += shadow_base;
			d.first_vertex += depth_vertex_base;
			nested.depth_draws.push_back(d);
		}
		nested.depth_vertices.insert(nested.depth_vertices.end(), n->depth_vertices.begin(), n->depth_vertices.end());
		nested.shadow_texels += n->shadow_texels;
		for (SwDrawCmd d : n->draws)
		{
			d.first_vertex += d.mode == SW_RASTER_TRIANGLE ? tri_base : vertex_base;
			if (d.tex_source == SW_TEXSRC_SURFACE) d.tex_offset += arena_base;
			nested.draws.push_back(d);
		}
		nested.vertices.insert(nested.vertices.end(), n->vertices.begin(), n->vertices.end());
		nested.tri_vertices.insert(nested.tri_vertices.end(), n->tri_vertices.begin(), n->tri_vertices.end());
		// the nested view's own nested views first (they render before it)
		for (SwView v : n->views)
		{
			v.target_offset += arena_base;
			v.first_draw += draw_base;
			nested.views.push_back(v);
		}
		arena_end += n->total_texels;
	}
	SwView v;
	std::memset(&v, 0, sizeof(v));
	v.target_offset = target_offset;
	v.width = width;
	v.height = height;
	v.first_draw = draw_base;
	v.num_draws = n ? n->main_draws : 0;
	v.clear_background = n ? n->params.clear_background : 0u;
	v.mix_blend = SW_VIEW_NO_MIX;
	if (portal.texture >= 0)
	{
		// mix_surface_with_texture with the texture's mip of the portal (:2230-2275); the light is
		// light_add, plus light_scale x the light grid's light at the portal polygon's centre (the cube
		// side facing the normal and the directional component) when light_scale > 0
		const LiteMip& m = sc.lite_mips[size_t(portal.texture) * NUM_MIPS + info.mip];
		float light[3] = {portal.light_add[0], portal.light_add[1], portal.light_add[2]};
		if (portal.light_scale > 0.0f)
		{
			const PolygonBasisVecs bv = form_plane_and_tex_coord_equation(portal.plane, portal.tex_coord_equation);
			const float scale = float(1u << info.mip);
			const Vec3 center = bv.start + (bv.u * scale) * (float(info.tc_min[0]) + float(width) * 0.5f) +
				(bv.v * scale) * (float(info.tc_min[1]) + float(height) * 0.5f);
			const LightGridElement g = sc.fetch_light_from_grid(center);
			float total[3];
			light_cube_light(g.light_cube, bv.normal, total);
			const float ld = std::fmax(dot(bv.normal, g.light_direction_vector_scaled), 0.0f);
			for (int c = 0; c < 3; ++c)
			{
				total[c] += g.directional_light_color[c] * ld;
				light[c] = total[c] * portal.light_scale + portal.light_add[c];
			}
		}
		v.mix_blend = portal.texture_blending_mode;
		v.mix_offset = m.offset;
		v.mix_size[0] = m.width;
		v.mix_size[1] = m.height;
		v.mix_tc_min[0] = info.tc_min[0];
		v.mix_tc_min[1] = info.tc_min[1];
		for (int c = 0; c < 3; ++c) v.mix_light[c] = light[c];
	}
	nested.views.push_back(v);
}

void FramePrep::append_nested()
{
	if (nested.views.empty())
	{
		total_texels = arena_end;
		return;
	}
	const uint32_t light_base = uint32_t(lights.size());
	const uint64_t shadow_base = shadow_texels;
	const uint32_t depth_vertex_base = uint32_t(depth_vertices.size());
	const uint32_t draw_base = uint32_t(draws.size()), vertex_base = uint32_t(vertices.size());
	const uint32_t tri_base = uint32_t(tri_vertices.size());
	// one shadow descriptor per light in the combined list (prepare_shadows keeps them parallel)
	SwLightShadow none;
	std::memset(&none, 0, sizeof(none));
	light_shadows.resize(lights.size(), none);
	for (SwSurfaceDesc d : nested.surfaces)
	{
		for (uint32_t k = 0; k < d.num_lights; ++k) d.lights[k] = uint16_t(d.lights[k] + light_base);
		surfaces.push_back(d);
	}
	lights.insert(lights.end(), nested.lights.begin(), nested.lights.end());
	for (SwLightShadow s : nested.light_shadows)
	{
		if (s.kind != SW_SHADOW_NONE) s.offset += shadow_base;
		light_shadows.push_back(s);
	}
	for (SwDepthDraw d : nested.depth_draws)
	{
		d.map_offset += shadow_base;
		d.first_vertex += depth_vertex_base;
		depth_draws.push_back(d);
	}
	depth_vertices.insert(depth_vertices.end(), nested.depth_vertices.begin(), nested.depth_vertices.end());
	shadow_texels += nested.shadow_texels;
	for (SwDrawCmd d : nested.draws)
	{
		d.first_vertex += d.mode == SW_RASTER_TRIANGLE ? tri_base : vertex_base;
		draws.push_back(d);
	}
	vertices.insert(vertices.end(), nested.vertices.begin(), nested.vertices.end());
	tri_vertices.insert(tri_vertices.end(), nested.tri_vertices.begin(), nested.tri_vertices.end());
	for (SwView v : nested.views)
	{
		v.first_draw += draw_base;
		views.push_back(v);
	}
	total_texels = arena_end;
	nested.clear();
}

void FramePrep::draw_view_portal(const Vec3 clip_planes[8], uint32_t portal_index)
{
	// draw_view_portal (:3720-3772): the portal polygon textured with its view. The leaf's 3D clip planes
	// cut nothing here: the generated portals lie inside their leaf.
	const PortalInfo& info = portal_infos[portal_index];
	if (uint64_t(info.resolution[0]) * info.resolution[1] == 0) return;
	const ViewPortal& portal = sc.view_portals[portal_index];
	const uint32_t nv = std::min(uint32_t(portal.vertices.size()), uint32_t(MAX_VERTICES));
	Vec3 vt[MAX_VERTICES];
	for (uint32_t k = 0; k < nv; ++k) vt[k] = view_transform(cam.view_matrix, portal.vertices[k]);
	emit_draw(clip_planes, vt, nv, info.depth, info.tc, info.resolution[0], info.resolution[1], info.pixels_offset,
		SW_TEXSRC_SURFACE, portal.blending_mode);
}

} // namespace swhost
