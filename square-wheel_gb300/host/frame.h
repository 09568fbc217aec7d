// Per-frame host work of the renderer: everything above the C ABI of the GPU path.
//
// Restates, for world polygons, the reference's host-side per-frame steps:
//   MapVisibilityCalculator::update_visibility (src/square_wheel/map_visibility_calculator.rs:52-326),
//   DynamicObjectsIndex::position_dynamic_lights (src/square_wheel/dynamic_objects_index.rs:108-241),
//   prepare_polygons_surfaces / prepare_polygon_surface (src/square_wheel/partial_renderer.rs:1327-1638),
//   the descriptor half of build_polygons_surfaces (partial_renderer.rs:1640-1819) with
//   polygon_is_affected_by_light (:3877-3985),
//   draw_skybox (:2311-2448) with the sky bounds collected in prepare_polygon_surface (:1510-1528),
//   draw_tree / draw_leaf / draw_polygon (:2450-2559, :4011-4142) with project_and_clip_polygon,
//   calculate_mip and the interpolation-mode tests (src/square_wheel/renderer_utils.rs), the clipping
//   helpers (src/common/clipping.rs:4-185) and ClippingPolygon (src/common/clipping_polygon.rs).
// Output: the SwSurfaceDesc list (in the reference's surface allocation order) and the SwDrawCmd list
// (in exact submission order) that the GPU path consumes.
#pragma once

#include <memory>
#include <vector>

#include "prep_math.h"
#include "scene.h"
#include "sims.h"

namespace swhost
{

struct ClipAxis
{
	float min, max;
};
struct ClippingPolygon
{
	ClipAxis x, y, x_plus_y, x_minus_y;
	static ClippingPolygon from_box(float min_x, float min_y, float max_x, float max_y);
	static ClippingPolygon from_point(Vec2 p);
	bool is_valid_and_non_empty() const;
	bool contains(const ClippingPolygon& o) const;
	void extend(const ClippingPolygon& o);
	void extend_with_point(Vec2 p);
	void intersect(const ClippingPolygon& o);
	void get_clip_planes(Vec3 out[8]) const;
};

// MapVisibilityCalculator (src/square_wheel/map_visibility_calculator.rs:52-326): the leafs reachable
// through portals from the camera's leaf, each with the screen bounds it is seen through.
class VisibilityCalculator
{
public:
	explicit VisibilityCalculator(const Scene& scene);
	void update(const CameraMatrices& cam, const ClippingPolygon& frame_bounds);
	// update_visibility_with_start_leafs (map_visibility_calculator.rs:99-113): portal and mirror views
	void update_with_start_leafs(const CameraMatrices& cam, const ClippingPolygon& frame_bounds, const uint32_t* start, uint32_t n);
	bool visible(uint32_t leaf) const { return leafs[leaf].visible_frame == frame; }
	const ClippingPolygon& bounds(uint32_t leaf) const { return leafs[leaf].bounds; }
	uint32_t camera_leaf = 0;

private:
	struct Leaf
	{
		uint32_t visible_frame = 0;
		ClippingPolygon bounds{};
	};
	struct Portal
	{
		uint32_t visible_frame = 0;
		bool has_projection = false;
		ClippingPolygon projection{};
	};
	const Scene& sc;
	CameraMatrices cam{};
	uint32_t frame = 0;
	std::vector<Leaf> leafs;
	std::vector<Portal> portals;
	std::vector<uint32_t> wave0, wave1;
	uint32_t find_current_leaf() const;
	bool project_portal(const MapPortal& p, ClippingPolygon& out) const;
	void mark_reachable_leafs(const uint32_t* start, uint32_t n, const ClippingPolygon& bounds);
};

struct FrameOptions
{
	uint32_t width = 640, height = 480;
	uint32_t pixel_format = SW_PIXEL_C32;
	bool use_directional_lightmaps = true;
	bool clear_background = false;
	float fov = 3.14159265358979323846f * 0.375f; // test game FOV, src/test_game/game_map.rs:865
	float mip_bias = 0.0f;                        // textures_mip_bias default, dynamic_mip_bias off
	float shadows_quality = 0.0f;                 // RendererConfig::shadows_quality default (clamped to [-1, 1])
};

struct FrameStats
{
	uint32_t visible_leafs = 0, visible_polygons = 0, draws = 0, camera_leaf = 0, skybox_draws = 0;
	uint32_t model_triangles = 0; // triangle draws of the visible models
	uint64_t surface_texels = 0;
};

class FramePrep
{
public:
	explicit FramePrep(const Scene& scene);
	// Camera, lights and skybox rotation of scene frame `frame_index` (camera path key, moving lights).
	void prepare(uint32_t frame_index, const FrameOptions& opt);
	// Same with an explicit camera, light list and skybox rotation (FrameWorldInfo::skybox_rotation).
	void prepare_with_camera(const CameraMatrices& cam, const std::vector<SwLight>& lights, const FrameOptions& opt,
		Quat skybox_rotation = Quat{1.0f, Vec3{0.0f, 0.0f, 0.0f}});
	// The host half of a frame whose surfaces and world draws are prepared on the GPU
	// (sw_draw_frame_view): visibility, light positioning, the skybox draws and the visible leafs with
	// their bounds, lights and back-to-front draw order (view_leafs, view_leaf_lights). surfaces stays
	// empty; draws / vertices hold the skybox's.
	void prepare_view(uint32_t frame_index, const FrameOptions& opt);
	void prepare_view_with_camera(const CameraMatrices& cam, const std::vector<SwLight>& lights, const FrameOptions& opt,
		Quat skybox_rotation = Quat{1.0f, Vec3{0.0f, 0.0f, 0.0f}});

	const CameraMatrices& camera() const { return cam; }

	// The map's polygons as the preparation reads them this frame (the material fields of animated
	// materials follow their current frame), and as the map holds them (uploaded by sw_set_map: the GPU
	// side applies the frame's SwMaterialFrame itself).
	std::vector<SwMapPolygon> map_polygons;
	std::vector<SwMapPolygon> map_polygons_base;
	std::vector<std::vector<uint32_t>> material_polygons;

	std::vector<SwSurfaceDesc> surfaces;
	uint64_t total_texels = 0;
	std::vector<SwDrawCmd> draws;
	std::vector<SwVertex16> vertices;
	std::vector<SwTriVertex> tri_vertices; // vertices of the triangle draws (the leafs' models)
	std::vector<SwLight> lights;
	SwFrameParams params{};
	FrameStats stats;
	std::vector<SwViewLeaf> view_leafs;
	std::vector<uint16_t> view_leaf_lights;
	// Cube shadow maps of the frame's shadowed visible lights: one SwLightShadow per light, the depth draws
	// of every side (side by side, light by light) and the storage they need.
	std::vector<SwLightShadow> light_shadows;
	std::vector<SwDepthDraw> depth_draws;
	std::vector<SwVertex16> depth_vertices;
	uint64_t shadow_texels = 0;
	// prepare_view: the depth draws are the GPU's (sw_build_shadow_maps_view); the host lists each side
	// and the leafs its visibility reaches, back to front (depth_draws / depth_vertices stay empty).
	std::vector<SwShadowSide> shadow_sides;
	std::vector<SwShadowLeaf> shadow_leafs;
	// Animated materials: per material its current frame's texture and scrolling shift; `animated` is
	// false when no material scrolls or has frames (the view input then passes no table).
	std::vector<SwMaterialFrame> material_frames;
	// the frame's generative texture effect passes (sw_update_textures) and their turbulence shifts
	std::vector<SwTexturePass> texture_passes;
	std::vector<int32_t> texture_shifts;
	// the frame's simulated effect work (sw_update_simulations): water and fire steps, textures, mips
	SimBatch simulations;
	// Portal views (prepare_view_portals_textures / build_view_portals_textures, partial_renderer.rs:
	// 1834-2283). Per scene portal its texture in the surface arena (resolution 0: not visible this frame);
	// the frame's nested views in render order (SwView: a portal texture region rendered from the view's
	// draws, then mixed with the portal's texture). Draws [0, main_draws) are this view's; the nested
	// views' draws, vertices, surfaces, lights and shadow maps follow this view's own. total_texels spans
	// this view's surfaces (surface_texels), its portal textures and the nested views' arenas.
	struct PortalInfo
	{
		uint32_t resolution[2] = {0, 0};
		uint64_t pixels_offset = 0;
		DepthEquation depth{};
		TexCoordEquation tc{};
		int32_t tc_min[2] = {0, 0};
		uint32_t mip = 0;
	};
	std::vector<PortalInfo> portal_infos;
	std::vector<SwView> views;
	uint32_t main_draws = 0;
	uint64_t surface_texels = 0;
	const EffectSim* effect_sim(uint32_t material) const
	{
		return material < sims.size() ? sims[material].get() : nullptr;
	}
	bool animated = false;
	// Game time of the frame (prepare / prepare_view: frame index / 60 s; the *_with_camera forms keep it).
	float frame_time_s = 0.0f;

private:
	struct PolyData
	{
		uint32_t visible_frame = 0;
		DepthEquation depth;
		TexCoordEquation tc;
		uint64_t offset = 0;
		uint32_t size[2] = {0, 0};
		uint32_t mip = 0;
		int32_t tc_min[2] = {0, 0};
	};

	const Scene& sc;
	uint32_t current_frame = 0;
	VisibilityCalculator vis{sc};        // the camera's
	VisibilityCalculator shadow_vis{sc}; // the shadow-map sides' (one after another)
	std::vector<std::vector<uint32_t>> light_leafs; // leafs each light's sphere touches
	std::vector<uint32_t> leaf_view_index; // position of a visible leaf in view_leafs (prepare_view)
	std::vector<PolyData> poly;
	std::vector<Vec3> vertices_transformed;
	std::vector<uint32_t> visible_polygons;
	std::vector<std::vector<uint32_t>> leaf_lights;
	CameraMatrices cam{};
	FrameOptions opt;
	Quat sky_rotation{1.0f, Vec3{0.0f, 0.0f, 0.0f}};
	bool shadow_view = false;    // prepare_view: list the shadow sides' leafs instead of depth draws
	bool has_sky = false;        // current_sky (partial_renderer.rs:35): a sky polygon is visible
	ClippingPolygon sky_bounds{}; // union of the visible sky polygons' screen bounds
	std::vector<uint32_t> sky_polygons;   // polygons of the sky material, grouped by leaf
	std::vector<uint32_t> leaf_sky_first; // leaf i's sky polygons: sky_polygons[leaf_sky_first[i] .. [i + 1])

	void position_lights();
	void position_sphere(uint32_t id, Vec3 center, float radius, uint32_t node);
	void prepare_polygons_surfaces();
	void prepare_polygon_surface(const Vec3 clip_planes[8], uint64_t& offset, uint32_t polygon_index);
	void extend_sky_bounds(const Vec2* v2d, uint32_t count);
	void prepare_shadows();
	template <class F>
	void for_each_depth_leaf(const CameraMatrices& camera, uint32_t size, F&& leaf_fn);
	void draw_depth_map(const CameraMatrices& camera, uint32_t size, uint64_t map_offset);
	void draw_depth_polygon(const CameraMatrices& camera, const Vec3 clip_planes[8], uint32_t polygon_index, uint32_t size,
		uint64_t map_offset);
	void update_materials();
	std::vector<uint32_t> mapping; // textures_mapping_table: current frame of each material (persists)
	std::vector<float> change_time; // its frame_change_time_point
	std::vector<std::vector<int32_t>> turb_buffers; // each turbulent material's temp_buffer (persists)
	void update_texture_effects();
	std::vector<std::unique_ptr<EffectSim>> sims; // each water / fire material's effect state (persists)
	void update_simulations();
	void apply_material_frames();
	// portals: the nested renderer (portals_depth - 1 levels below; none at depth 0), the view this one
	// renders a portal of, and the nested views' outputs gathered until this view's own draws are done
	struct ViewBlock
	{
		std::vector<SwSurfaceDesc> surfaces;
		std::vector<SwLight> lights;
		std::vector<SwLightShadow> light_shadows;
		std::vector<SwDepthDraw> depth_draws;
		std::vector<SwVertex16> depth_vertices;
		uint64_t shadow_texels = 0;
		std::vector<SwDrawCmd> draws;
		std::vector<SwVertex16> vertices;
		std::vector<SwTriVertex> tri_vertices;
		std::vector<SwView> views;
		void clear();
	};
	uint32_t portals_depth = 0;
	std::unique_ptr<FramePrep> portal_renderer;
	ViewBlock nested;
	uint64_t arena_end = 0;
	void prepare_portals();
	void finish_view(const ClippingPolygon& viewport);
	void prepare_nested(const FramePrep& parent, const CameraMatrices& camera, const std::vector<uint32_t>* start_leafs,
		uint32_t width, uint32_t height);
	void gather_nested(const FramePrep* n, uint64_t target_offset, uint32_t width, uint32_t height, const ViewPortal& portal,
		const PortalInfo& info);
	void append_nested();
	void draw_view_portal(const Vec3 clip_planes[8], uint32_t portal_index);
	void begin_frame(const CameraMatrices& cam, const std::vector<SwLight>& lights, const FrameOptions& opt, Quat skybox_rotation);
	void finish_params();
	void camera_of_frame(uint32_t frame_index, const FrameOptions& opt, CameraMatrices& cam, std::vector<SwLight>& lights,
		Quat& skybox_rotation) const;
	template <class F>
	void for_each_drawn_leaf(F&& f);
	void build_surface_descs();
	void draw_skybox(const ClippingPolygon& viewport);
	void draw_tree();
	void draw_leaf(const ClippingPolygon& bounds, uint32_t leaf_index);
	// A projector light's map (size, storage at `offset`, then advanced) and its depth draws.
	void prepare_projector(uint32_t light_index, uint64_t& offset);
	// The leaf's triangle models after its polygons (draw_leaf's dynamic models, partial_renderer.rs:
	// 2562-2792; build_dynamic_models_buffers :1122-1190; draw_mesh :3525-3718).
	void draw_leaf_models(const ClippingPolygon& bounds, uint32_t leaf_index);
	void draw_model(const ClippingPolygon& bounds, uint32_t model_index);
	void draw_sprite(const ClippingPolygon& bounds, uint32_t sprite_index);
	// prepare_decals (partial_renderer.rs:665-737) for one decal, once per frame: its camera-space
	// planes matrix and its light (a light cube of the visible unshadowed dynamic lights)
	struct DecalInfo
	{
		uint32_t frame = 0;
		Mat4 planes;
		float cube[6][3];
		Vec3 dir;
		float color[3];
	};
	std::vector<DecalInfo> decal_info;
	const DecalInfo& prepare_decal(uint32_t decal_index);
	void draw_polygon_decals(const Vec3 clip_planes[8], uint32_t polygon_index, const std::vector<uint32_t>& leaf_decals);
	void subdivide_decal_triangle(const DecalEntity& d, const MapPolygon& polygon, const DepthEquation& de,
		const TexCoordEquation& tc, const TexCoordEquation& lm_eq, const float lm_shift[2], const Vec2 pts[3],
		const LiteMip& tex, const float dyn[3], int depth);
	struct ModelVertex3d
	{
		Vec3 pos;
		float tc[2];
		float light[3];
	};
	std::vector<ModelVertex3d> model_vertices; // the current model's transformed vertices
	static uint32_t clip_model_near(const ModelVertex3d* src, uint32_t n, ModelVertex3d* dst);
	uint32_t emit_model_polygon(const ModelVertex3d* verts, uint32_t n, const Vec3* planes_2d, uint32_t num_2d,
		const LiteMip& tex, uint32_t blend, const float* light);
	std::vector<uint32_t> model_triangles;     // its visible triangles, back to front
	void draw_polygon(const Vec3 clip_planes[8], uint32_t polygon_index);
	// draw_polygon (partial_renderer.rs:4011-4142) of transformed vertices with their equations and texture.
	void emit_draw(const Vec3 clip_planes[8], const Vec3* vertices_transformed, uint32_t num_vertices,
		const DepthEquation& depth, const TexCoordEquation& tc, uint32_t tex_w, uint32_t tex_h, uint64_t tex_offset,
		uint32_t tex_source, uint32_t blend);
};

} // namespace swhost
