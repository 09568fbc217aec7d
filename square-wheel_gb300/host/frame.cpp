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
	sc.map_polygons(map_polygons);
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
	light_shadows.assign(lights.size(), SwLightShadow{SW_SHADOW_NONE, 0u, 0ull});
	uint64_t offset = 0;
	for (uint32_t li = 0; li < lights.size(); ++li)
	{
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
		light_shadows[li] = SwLightShadow{SW_SHADOW_CUBE, size, offset};
		for (uint32_t side = 0; side < 6; ++side)
			draw_depth_map(cube_shadow_map_side_matrices(lp, float(size), side), size, offset + uint64_t(side) * size * size);
		offset += uint64_t(size) * size * 6;
	}
	shadow_texels = offset;
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
		make_surface_desc(p, sp, pd.offset, directional, simple_lightmaps, mf.shift, mf.texture, d);
		if (p.flags & SW_POLY_DIFFUSE_LAYER)
			for (uint32_t li : leaf_lights[sc.polygon_leaf[pi]])
				if (polygon_is_affected_by_light(p, lights[li]))
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
	material_frames.resize(n);
	for (uint32_t m = 0; m < n; ++m)
	{
		material_frames[m].shift[0] = shift[2 * mapping[m]];
		material_frames[m].shift[1] = shift[2 * mapping[m] + 1];
		material_frames[m].texture = mapping[m];
		material_frames[m].reserved = 0;
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
	draws.clear();
	vertices.clear();
	// perform_rasterization_for_viewport_part (:1285-1325): skybox first, then the tree
	draw_skybox(ClippingPolygon::from_box(0.0f, 0.0f, float(opt.width), float(opt.height)));
	draw_tree();
	finish_params();
	stats.visible_polygons = uint32_t(visible_polygons.size());
	stats.draws = uint32_t(draws.size());
	stats.surface_texels = total_texels;
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

} // namespace swhost
