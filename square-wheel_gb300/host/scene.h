// Host-side map model and seeded synthetic scene generator.
//
// The map model is the subset of BSPMap (src/common/bsp_map_compact.rs:6-75) that world rendering
// reads: BSP nodes (last node is the root, children >= FIRST_LEAF_INDEX are leafs), leafs with their
// polygons and portals, polygons with plane, texture-coordinate equations, integer tc bounds and
// lightmap offset, portals, vertices, simple and directional lightmaps.
//
// The reference's map compiler and lightmapper (Rust executables) cannot run here and no compiled maps
// ship with it, so scenes are generated: a grid of axis-aligned box rooms (edges uniform in
// [room_min, room_max]) joined by 128x128 corridors, one convex BSP leaf per room and per corridor half,
// portals at the room walls and at the cell boundaries, faces cut around the corridor openings and
// tiled (tile_size) so every lightmap stays within the reference's size limit; lightmaps are lit by
// seeded point lights per room with a direct-light model; textures are procedural (value noise +
// checker, height-field normal maps) with full mip chains built as build_texture_mip does.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/swgpu.h"
#include "hmath.h"

namespace swhost
{

constexpr uint32_t FIRST_LEAF_INDEX = 1u << 31;
constexpr uint32_t LIGHTMAP_SCALE_LOG2 = 4;
constexpr uint32_t LIGHTMAP_SCALE = 1u << LIGHTMAP_SCALE_LOG2;
constexpr uint32_t NUM_MIPS = 5;

struct BspNode
{
	uint32_t children[2];
	Plane plane;
};
struct BspLeaf
{
	uint32_t first_polygon, num_polygons, first_leaf_portal, num_leaf_portals;
};
struct MapPolygon
{
	uint32_t first_vertex, num_vertices;
	Plane plane;
	Plane tex_coord_equation[2];
	int32_t tex_coord_min[2], tex_coord_max[2];
	uint32_t lightmap_data_offset;
	uint32_t texture; // material index
};
struct MapPortal
{
	uint32_t leafs[2];
	Plane plane;
	uint32_t first_vertex, num_vertices;
};

// SingleArgumentFunction (src/common/material_function.rs:5-140): a function of time.
struct TimeFunction
{
	enum Kind : uint32_t
	{
		CONSTANT = 0, // c
		LINEAR,       // x * scale + offset
		SIN_WAVE,     // amplitude * sin(2 pi (x * frequency) + phase) + offset
		TRIANGLE_WAVE,
		SAW_TOOTH_WAVE,
		STEP_WAVE,
	};
	uint32_t kind = CONSTANT;
	float a = 0.0f, b = 0.0f, c = 0.0f, d = 0.0f; // CONSTANT: a; LINEAR: scale a, offset b; waves: frequency a, phase b, amplitude c, offset d
	float evaluate(float x) const;
};

// LayeredAnimationLayer (src/common/material.rs:208-235)
struct EffectLayer
{
	uint32_t material = 0;
	bool follow_framed_animation = false;
	TimeFunction tex_coord_shift[2];
	bool has_modulate = false, has_modulate_color = false;
	TimeFunction modulate;
	TimeFunction modulate_color[3];
};

// WaterEffect (src/common/material_water.rs): a wave field simulated at update_frequency steps per second,
// disturbed by wave sources; its normals (and, per colour mode, a deformed copy of the material's colours)
// make the output texture.
struct WaveSource
{
	enum Kind : uint32_t
	{
		WAVY_SPOT = 0,        // sine at points[0] (+ offsets[0])
		WAVY_LINE = 1,        // sine along points[0] - points[1] (+ offsets)
		PERIODIC_DROPLET = 2, // `amplitude` at points[0] (+ offsets[0]) `frequency` times per second
		RAIN = 3,             // random droplets within `radius` of points[0] (anywhere for radius 0)
	};
	uint32_t kind = WAVY_SPOT;
	uint32_t points[2][2] = {{0, 0}, {0, 0}};
	TimeFunction offsets[2][2]; // center_offset = offsets[0], points_offset
	float frequency = 1.0f, phase = 0.0f, amplitude = 1.0f, offset = 0.0f, radius = 0.0f;
};
struct WaterEffect
{
	uint32_t resolution_log2[2] = {4, 4};
	float update_frequency = 30.0f, fluidity = 200.0f;
	uint32_t color_mode = 0; // ColorTextureApplyMode: single colour, source texture, deformed, deformed along x
	std::vector<WaveSource> sources;
};
// ValueWithRandomDeviation: value - deviation + uniform [0, 2 max(deviation, 0)]
struct RandomValue
{
	TimeFunction value, deviation;
};
// FireEffect (src/common/material_fire.rs): a heat map propagated upwards at update_frequency steps per
// second from heat sources; a palette maps it to the output emissive texture.
struct HeatSource
{
	enum Kind : uint32_t
	{
		POINT = 0,     // heat at points[0] + offset[0]
		LINE = 1,      // heat along points[0] - points[1]
		LIGHTNING = 2, // a jittered line between points (+ offset), heat optionally ramped
		FOUNTAIN = 3,  // particles emitted from points[0]
	};
	uint32_t kind = POINT;
	uint32_t points[2][2] = {{0, 0}, {0, 0}};
	RandomValue offset[2][2]; // POINT: offset[0]; LIGHTNING: per point and coordinate
	RandomValue heat;
	bool ramp = false;
	float frequency = 1.0f; // FOUNTAIN: particles per second
	RandomValue angle, speed, gravity, spawn_angle, spawn_distance, lifetime;
};
struct FireEffect
{
	uint32_t resolution_log2[2] = {4, 4};
	float update_frequency = 30.0f, heat_conductivity = 20.0f;
	bool slow = false;
	bool has_color = false;
	float color[3] = {1.0f, 1.0f, 1.0f};
	std::vector<HeatSource> sources;
};

// Material flags the renderer reads (src/common/material.rs): draw, light, diffuse layer, blending,
// optional emissive layer.
struct Material
{
	bool draw = true;
	bool light = true;
	bool has_diffuse = true;
	uint32_t blending_mode = SW_BLEND_NONE;
	int32_t emissive = -1; // emissive texture index or -1
	float emissive_light[3] = {1.0f, 1.0f, 1.0f};
	bool skybox = false; // SpecialMaterialEffect::Skybox: polygons only mark where the sky shows
	bool shadow = true;  // casts shadows (material.rs:50-53)
	bool decals = true;  // decals are drawn on its polygons (material.rs)
	float scroll_speed[2] = {0.0f, 0.0f}; // Material::scroll_speed, texels of mip 0 per second
	uint32_t texture_size = 0;            // mip-0 width = height
	int32_t next_frame = -1;              // framed_animation.next_material_name as a material index, -1: none
	float frame_duration = 0.5f;          // framed_animation.duration, seconds
	// Generative effect (SpecialMaterialEffect::Turb / LayeredAnimation, material.rs:146-160): its output
	// texture is the texture slot effect_texture (after the materials' own), rewritten every frame.
	enum Effect : uint32_t
	{
		NO_EFFECT = 0,
		TURB = 1,
		LAYERED = 2,
		WATER = 3, // output texture effect_texture (the field's size)
		FIRE = 4,  // output emissive texture effect_emissive (the heat map's size)
	};
	uint32_t effect = NO_EFFECT;
	int32_t effect_texture = -1;
	int32_t effect_emissive = -1;
	uint64_t sim_state = 0; // WATER / FIRE: word offset of its two fields / heat maps in the simulation state
	float roughness = 1.0f; // Material::roughness (WATER: the output's roughness)
	bool is_metal = false;
	WaterEffect water;
	FireEffect fire;
	float turb_amplitude = 0.0f, turb_wave_length = 1.0f, turb_frequency = 0.0f; // TurbParams
	std::vector<EffectLayer> layers;                                              // LayeredAnimation
};

// One mip of a skybox side (SkyboxSideTexture, src/square_wheel/textures.rs:83-87): size x size texels
// at `offset` in Scene::skybox32 / skybox64; size 0 = no texture.
struct SkyboxMip
{
	uint64_t offset = 0;
	uint32_t size = 0;
};

// PolygonBasisVecs, src/square_wheel/surfaces.rs:6-64
struct PolygonBasisVecs
{
	Vec3 u, v, start, normal;
};

struct DynamicLightSpec
{
	uint32_t path_offset; // frames ahead of the camera on its path
	Vec3 offset;          // displacement from the path point
	float orbit_radius;
	float radius;
	float color[3];
};

// A per-vertex animated triangle model mesh (TriangleModelMesh with VertexData::VertexAnimated,
// src/square_wheel/triangle_model.rs): frame f's vertex i at positions[f * num_vertices + i].
struct ModelMesh
{
	uint32_t num_vertices = 0, num_frames = 0;
	std::vector<Vec3> positions, normals; // num_frames x num_vertices
	std::vector<float> tex_coords;        // 2 per vertex, in units of the texture size
	std::vector<uint32_t> triangles;      // 3 vertex indices per triangle
	Vec3 bbox_min, bbox_max;              // over every frame
};

// A placed model (ModelEntity, src/square_wheel/frame_info.rs:44-78): its mesh, position, rotation about
// the vertical axis, animation (frames per second and phase), blending mode, skin (a TextureLite with
// NUM_MIPS mips) and the light it receives (LightGridElement, src/common/bsp_map_compact.rs: a light cube
// and a directional component).
struct ModelEntity
{
	uint32_t mesh, texture, leaf, blending_mode;
	Vec3 position;
	float yaw, anim_speed, anim_phase;
	float light_cube[6][3];
	Vec3 light_dir_scaled;
	float light_color[3];
};

// A sprite (Sprite, src/square_wheel/frame_info.rs:126-147): a textured quad of `radius` (half its
// diagonal) at `position`, turned by `angle` in its plane, oriented by one of the four SpriteOrientation
// rules, lit by light_add plus light_scale times its light (a light cube and directional component
// standing in for fetch_light_from_grid, and the frame's unshadowed dynamic lights), in one leaf.
struct SpriteEntity
{
	enum Orientation : uint32_t
	{
		PARALLEL_TO_CAMERA_PLANE = 0,
		FACING_TOWARDS_CAMERA,
		ALIGN_TO_Z_AXIS_PARALLEL_TO_CAMERA_PLANE,
		ALIGN_TO_Z_AXIS_FACING_TOWARDS_CAMERA,
	};
	Vec3 position;
	float angle, radius;
	uint32_t texture; // lite texture: mips at texture * NUM_MIPS in Scene::lite_mips
	uint32_t blending_mode, orientation, leaf;
	float light_scale;
	float light_add[3];
	float light_cube[6][3];
	Vec3 light_dir_scaled;
	float light_color[3];
};

// A decal (Decal, src/square_wheel/frame_info.rs): the cube [-1, 1]^3 of the object matrix
// (position, rotation, scale) projected along its -x axis onto the polygons it cuts, with a lite texture
// spanning its y and z extent, lit by light_add plus lightmap_light_scale times the polygon's lightmap
// and the dynamic light at its position; `leafs`: the leafs its cube reaches (position_object_bbox).
struct DecalEntity
{
	Vec3 position;
	Quat rotation;
	Vec3 scale;
	uint32_t texture, blending_mode;
	float lightmap_light_scale;
	float light_add[3];
};

// ViewPortal (src/square_wheel/frame_info.rs:171-205): a polygon showing another view of the world,
// rendered into a texture of its own every frame - a camera at a position, a mirror, or a parallax
// portal (the camera moved by `transform`) - optionally mixed with a texture.
struct ViewPortal
{
	enum Kind : uint32_t
	{
		CAMERA_AT_POSITION = 0,
		MIRROR = 1,
		PARALLAX = 2,
	};
	uint32_t kind = MIRROR;
	Vec3 position{0.0f, 0.0f, 0.0f}; // CAMERA_AT_POSITION
	Quat rotation{1.0f, Vec3{0.0f, 0.0f, 0.0f}};
	float fov = 1.5707964f;
	Mat4 transform = Mat4::identity(); // PARALLAX: camera position -> the portal's view point
	Plane plane{};
	Plane tex_coord_equation[2]{};
	std::vector<Vec3> vertices;
	uint32_t blending_mode = SW_BLEND_NONE;
	// ViewPortalTexture: a lite texture (Scene::lite_mips index / NUM_MIPS), its blending and light
	int32_t texture = -1;
	uint32_t texture_blending_mode = SW_BLEND_NONE;
	float light_scale = 0.0f;
	float light_add[3] = {1.0f, 1.0f, 1.0f};
};

// The map's light grid (bsp_map_compact.rs:162-188): columns of samples over a regular grid, each
// sample a light cube and one directional component; models, sprites and portal textures take their
// light from it (fetch_light_from_grid).
struct LightGridElement
{
	float light_cube[6][3];
	Vec3 light_direction_vector_scaled;
	float directional_light_color[3];
};
struct LightGridHeader
{
	float grid_cell_size[3];
	float grid_start[3];
	uint32_t grid_size[3];
};
struct LightGridColumn
{
	uint32_t start_z, first_sample, num_samples;
};

// One mip of a TextureLite (Color32 pixels, src/square_wheel/textures.rs:89-91) in Scene::lite_pixels.
struct LiteMip
{
	uint64_t offset;
	uint32_t width, height;
};

struct CameraKey
{
	Vec3 position;
	float azimuth, elevation;
};

struct SceneConfig
{
	uint64_t seed = 1;
	uint32_t grid_x = 4, grid_y = 2;
	float room_min = 256.0f, room_max = 1024.0f;
	float tile_size = 128.0f;
	uint32_t texture_size = 128;
	uint32_t num_materials = 16;
	float metal_frac = 0.0f, dielectric_frac = 0.0f;
	bool normal_maps = false;
	bool directional_lightmaps = false;
	uint32_t lights_per_room = 1;
	uint32_t num_dynamic_lights = 0;
	uint32_t num_frames = 64;
	float emissive_frac = 0.0f;
	uint32_t sky_rooms = 0;           // rooms whose ceiling is sky (a skybox material)
	uint32_t skybox_size = 128;       // skybox side texture size (power of two)
	float skybox_brightness = 1.0f;   // SkyboxParams::brightness
	int32_t skybox_missing_side = -1; // a side without texture (0..5), -1 = none
	float sky_rotation_speed = 0.01f; // skybox rotation about the vertical axis, radians per frame
	float camera_pitch = 0.0f;        // added to the camera path's elevation (radians, up > 0)
	uint32_t shadowed_lights = 0;     // the first this many dynamic lights cast cube shadows
	uint32_t projector_lights = 0;    // the next this many dynamic lights are shadowed projectors (cones)
	uint32_t scrolling_materials = 0; // the first this many materials scroll (Material::scroll_speed)
	uint32_t animated_materials = 0;  // the first this many materials cycle through 3 frames (framed_animation)
	uint32_t num_models = 0;          // per-vertex animated triangle models placed in the rooms
	uint32_t model_triangles = 2000;  // triangles per model mesh (about)
	uint32_t model_frames = 8;        // animation keyframes per mesh
	uint32_t num_sprites = 0;         // sprites in the rooms (all four orientations, several blending modes)
	uint32_t num_decals = 0;          // decals on the rooms' walls and floors
	uint32_t num_portals = 0;         // portals in the camera path's rooms: mirrors, cameras, parallax windows
	uint32_t light_grid = 0;          // a seeded light grid from the rooms' lights (models, sprites and portals lit from it)
	uint32_t portals_depth = 2;       // RendererConfig::portals_depth: nested portal views (at most 8)
	uint32_t turb_materials = 0;      // the last base materials but layered_materials have a turbulence effect
	uint32_t layered_materials = 0;   // the last this many base materials are layered animations
	uint32_t water_materials = 0;     // before the turbulence ones: water effects
	uint32_t fire_materials = 0;      // before the water ones: fire effects
};

struct Scene
{
	SceneConfig config;
	std::vector<BspNode> nodes;
	std::vector<BspLeaf> leafs;
	std::vector<MapPolygon> polygons;
	std::vector<MapPortal> portals;
	std::vector<uint32_t> leafs_portals;
	std::vector<Vec3> vertices;
	std::vector<float> lightmaps; // [f32; 3] elements, element 0 unused
	std::vector<SwDirectionalLightmapElement> directional_lightmaps;
	std::vector<Material> materials;
	uint64_t sim_state_words = 0; // the simulated effects' device state (sw_reserve_simulation_state)
	std::vector<uint64_t> texels; // TextureElement raw values of all materials' mips
	std::vector<SwTextureMip> texture_mips; // material * NUM_MIPS + mip
	std::vector<uint32_t> emissive_pixels;
	std::vector<SwEmissiveMip> emissive_mips; // emissive * NUM_MIPS + mip
	std::vector<PolygonBasisVecs> basis;      // per polygon, precomputed at load (partial_renderer.rs:63-78)
	std::vector<uint32_t> polygon_leaf;       // leaf of each polygon
	std::vector<CameraKey> camera_path;       // one key per frame
	std::vector<DynamicLightSpec> dynamic_lights;
	uint64_t lightmap_elements = 0;
	// Skybox of the sky material (SkyboxTextures<Color32> / <Color64>): sides in the reference's order
	// (-X, +X, -Y, +Y, -Z, +Z), NUM_MIPS mips each, the same layout in both formats.
	int32_t sky_material = -1;
	std::vector<uint32_t> skybox32;
	std::vector<uint64_t> skybox64;
	SkyboxMip skybox_mips[6][NUM_MIPS];
	// Triangle models: meshes, placed models, the models of each leaf, and their skins' mips
	// (texture * NUM_MIPS + mip) in one Color32 array (sw_set_lite_textures).
	std::vector<ModelMesh> model_meshes;
	std::vector<ModelEntity> models;
	std::vector<std::vector<uint32_t>> leaf_models;
	std::vector<uint32_t> lite_pixels;
	std::vector<LiteMip> lite_mips;
	// Sprites and the sprites of each leaf; their textures are lite textures after the model skins.
	std::vector<SpriteEntity> sprites;
	std::vector<std::vector<uint32_t>> leaf_sprites;
	// Decals and the decals of each leaf, in decal order; their textures are lite textures too.
	std::vector<DecalEntity> decals;
	std::vector<std::vector<uint32_t>> leaf_decals;
	// portals and the portals index (DynamicObjectsIndex::position_portals): each portal's leafs, each
	// leaf's portals in portal order
	LightGridHeader light_grid_header{};
	std::vector<LightGridColumn> light_grid_columns;
	std::vector<LightGridElement> light_grid_samples;
	// fetch_light_from_grid (triangle_models_rendering.rs:582-700): the trilinear mix of the up to 8
	// existing non-zero samples around `pos`, renormalised when some were missing; zero without a grid
	LightGridElement fetch_light_from_grid(Vec3 pos) const;
	std::vector<ViewPortal> view_portals;
	std::vector<std::vector<uint32_t>> view_portal_leafs;
	std::vector<std::vector<uint32_t>> leaf_view_portals;
	// get_convex_hull_bsp_leafs (src/common/bsp_map_compact.rs:294-338): the leafs a convex hull reaches,
	// front child first
	void convex_hull_leafs(const Vec3* vertices, uint32_t n, std::vector<uint32_t>& out) const;
	uint32_t leaf_of(Vec3 p) const; // the leaf holding a point (front of a node plane: the first child)
	// A scene loaded from a compiled map keeps its compressed lightmap lumps (4 bytes per simple
	// element, 13 per directional element, as the file holds them) for upload and decompression on the
	// GPU; empty for generated scenes.
	std::vector<uint8_t> lightmaps_compressed;
	std::vector<uint8_t> directional_lightmaps_compressed;

	uint32_t root_node() const { return nodes.empty() ? FIRST_LEAF_INDEX : uint32_t(nodes.size() - 1); }
	void frame_lights(uint32_t frame, std::vector<SwLight>& out) const;
	// DynamicLightShadowType::Cubemap for light `i` of frame_lights' list (the first shadowed_lights ones).
	bool light_is_shadowed(uint32_t i) const { return i < config.shadowed_lights; }
	// DynamicLightShadowType::Projector for the projector_lights lights after them.
	bool light_is_projector(uint32_t i) const
	{
		return i >= config.shadowed_lights && i < config.shadowed_lights + config.projector_lights;
	}
	// A projector light's rotation (yaw about the vertical axis, then pitch) and fov at time t (seconds).
	void projector_pose(uint32_t light, float t, Quat& rotation, float& fov) const;
	// The SW_POLY_* flags a material gives its polygons (draw, sky, diffuse layer, shadow).
	static uint32_t material_polygon_flags(const Material& m)
	{
		return (m.draw ? SW_POLY_DRAW : 0u) | (m.skybox ? SW_POLY_SKY : 0u) | ((m.light && m.has_diffuse) ? SW_POLY_DIFFUSE_LAYER : 0u) |
			(m.shadow ? SW_POLY_SHADOW : 0u);
	}
	// Polygons with their basis and material fields (SwMapPolygon), in polygon order.
	void map_polygons(std::vector<SwMapPolygon>& out) const;
	SwCreateInfo create_info(uint32_t device) const;
};

bool generate_scene(const SceneConfig& cfg, Scene& out, std::string& error);
// The config's generative texture effects on the base materials (and their layer materials and output
// texture slots); part of generate_scene.
void add_texture_effects(const SceneConfig& cfg, uint32_t n_metal, uint32_t n_diel, Scene& sc);

PolygonBasisVecs form_plane_and_tex_coord_equation(const Plane& plane, const Plane tc[2]);

} // namespace swhost
