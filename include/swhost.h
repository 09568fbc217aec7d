/*
 * swhost.h — C ABI of the host side of the GB300 renderer (libswhost.so).
 *
 * The reference keeps visibility, leaf ordering and per-polygon setup on the host in Rust; this library
 * is their C++ restatement (the Rust toolchain is not available to build the reference host), plus a
 * seeded synthetic scene generator that stands in for the map compiler and lightmapper. It produces the
 * SwSurfaceDesc / SwDrawCmd arrays of include/swgpu.h and can drive libswgpu.so itself:
 *   swh_renderer_prepare_frame  ~ Renderer::prepare_frame  (src/square_wheel/renderer.rs:61-104)
 *   swh_renderer_draw_frame     ~ Renderer::draw_frame     (src/square_wheel/renderer.rs:106-124)
 * Every function returns 0 or a negative SwStatus and never aborts.
 */
#ifndef SWHOST_H
#define SWHOST_H

#include "swgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct SwhSceneConfig {
	uint64_t seed;
	uint32_t grid_x, grid_y;      /* rooms in a grid_x x grid_y layout */
	float room_min, room_max;     /* room edge range, within [256, 1024] */
	float tile_size;              /* faces are cut into tiles of this size (16..256 units) */
	uint32_t texture_size;        /* material texture side (power of two) */
	uint32_t num_materials;
	float metal_frac, dielectric_frac; /* fractions of specular materials */
	uint32_t normal_maps;
	uint32_t directional_lightmaps;
	uint32_t lights_per_room;     /* static lights baked into the lightmaps */
	uint32_t num_dynamic_lights;  /* moving point lights */
	uint32_t num_frames;          /* camera path length */
	float emissive_frac;          /* fraction of materials with an emissive layer */
	uint32_t sky_rooms;           /* rooms whose ceiling is sky (0 = no sky material) */
	uint32_t skybox_size;         /* skybox side texture size (power of two, 16..2048) */
	float skybox_brightness;      /* skybox material brightness (SkyboxParams) */
	int32_t skybox_missing_side;  /* a side without texture (0..5: -X, +X, -Y, +Y, -Z, +Z), -1 = none */
	float sky_rotation_speed;     /* skybox rotation about the vertical axis, radians per frame */
	float camera_pitch;           /* added to the camera path's elevation (radians, up > 0) */
	uint32_t shadowed_lights;     /* the first this many dynamic lights cast cube shadows */
	uint32_t scrolling_materials; /* the first this many materials scroll (s and t speeds fixed per material) */
	uint32_t animated_materials;  /* the first this many materials cycle through 3 texture frames */
	uint32_t projector_lights;    /* the dynamic lights after the shadowed ones that are shadowed projectors */
	uint32_t num_models;          /* per-vertex animated triangle models on the rooms' floors (0 = none) */
	uint32_t model_triangles;     /* triangles per model mesh, about (0 = 2000) */
	uint32_t model_frames;        /* animation keyframes per mesh (0 = 8) */
	uint32_t turb_materials;      /* base materials with a turbulence effect (before the layered ones) */
	uint32_t layered_materials;   /* the last this many base materials are layered animations */
	uint32_t num_sprites;         /* sprites in the rooms (every orientation, alpha-family and additive blending) */
	uint32_t num_decals;          /* decals on the rooms' walls and floors (every blending mode) */
	uint32_t water_materials;     /* base materials with a water effect (before the turbulence ones) */
	uint32_t fire_materials;      /* base materials with a fire effect (before the water ones) */
	uint32_t num_portals;         /* portals (mirrors, cameras, parallax windows) in the camera path's rooms */
	uint32_t portals_depth;       /* RendererConfig::portals_depth: nested portal view levels (the reference's default is 2; at most 8; 0: portals show black mixed with their texture) */
	uint32_t light_grid;          /* nonzero: a seeded light grid over the rooms; models, sprites and portal textures take their light from it */
} SwhSceneConfig;

typedef struct SwhSceneInfo {
	uint32_t nodes, leafs, polygons, portals, materials, frames, dynamic_lights, reserved;
	uint64_t lightmap_elements, texels;
	uint64_t skybox_texels; /* texels of all skybox sides and mips (per format) */
} SwhSceneInfo;

typedef struct SwhScene SwhScene;

int swh_scene_create(const SwhSceneConfig* config, SwhScene** out_scene);
int swh_scene_destroy(SwhScene* scene);
int swh_scene_info(const SwhScene* scene, SwhSceneInfo* out_info);
/* Static data for sw_create; pointers stay valid while the scene lives. */
int swh_scene_create_info(const SwhScene* scene, uint32_t device, SwCreateInfo* out_info);
/* The models' Color32 skins with their mips for sw_set_lite_textures (pointer valid while the scene
 * lives; *out_count 0 without models). */
int swh_scene_lite_textures(const SwhScene* scene, const uint32_t** out_pixels, uint64_t* out_count);
/* Skybox texels for sw_set_skybox (Color32 and Color64 copies, the same layout) and, per side
 * (-X, +X, -Y, +Y, -Z, +Z) and mip, the first texel and size (0 = none): mip_offsets[side * 5 + mip].
 * Pointers stay valid while the scene lives; *out_count is 0 without a sky material. */
int swh_scene_skybox(const SwhScene* scene, const uint32_t** out_texels32, const uint64_t** out_texels64,
	uint64_t* out_count, uint64_t mip_offsets[30], uint32_t mip_sizes[30]);
/* A scene from a compiled map file (.sqwm, format version 11: load_map, src/common/bsp_map_save_load.rs:162-226,
 * lightmaps decompressed as lightmap_compression.rs does). The map's BSP tree, leafs, polygons, portals,
 * vertices and lightmaps are rendered as they are, after every index and range rendering follows is
 * checked; each texture name gets a procedural material (texture_size, normal_maps, metal_frac,
 * dielectric_frac and scrolling_materials apply; the image files the names refer to are not part of a
 * map); the camera path starts at the info_player_start entity (or leaf 0) and runs through leafs and
 * portals; num_dynamic_lights, shadowed_lights, projector_lights, num_frames, camera_pitch and
 * directional_lightmaps apply. grid_x, grid_y, room_min, room_max, tile_size and lights_per_room are
 * ignored; sky_rooms, num_models and animated_materials must be 0. A renderer created for such a scene
 * uploads the compressed lightmaps and decodes them on the GPU (sw_set_lightmaps_compressed).
 * Errors: SW_ERR_INVALID_ARGUMENT with swh_last_error() set (can't open, not a map, wrong version, a lump
 * past the end of the file, an index out of range). */
int swh_scene_load_map(const char* path, const SwhSceneConfig* config, SwhScene** out_scene);
int swh_scene_load_map_memory(const void* data, uint64_t size, const SwhSceneConfig* config, SwhScene** out_scene);
/* Write a scene's map data as a compiled map (save_map, bsp_map_save_load.rs:24-160): geometry as is, a
 * texture name per material, lightmaps compressed, a worldspawn entity and an info_player_start at the
 * camera path's first position. */
int swh_scene_save_map(const SwhScene* scene, const char* path);
/* A loaded map's compressed lightmap lumps as the file holds them (4-byte and 13-byte records; counts 0
 * for generated scenes). Pointers stay valid while the scene lives. */
int swh_scene_compressed_lightmaps(const SwhScene* scene, const void** out_lightmaps, uint64_t* out_count,
	const void** out_directional, uint64_t* out_directional_count);
/* A material's generative texture effect (SpecialMaterialEffect::Turb / LayeredAnimation, material.rs:146-197):
 * kind 0 none, 1 turbulence, 2 layered animation; the texture slot its output is written to; for
 * turbulence its TurbParams (amplitude, wave_length, frequency). */
typedef struct SwhTextureEffect {
	uint32_t kind;
	int32_t output_texture;
	uint32_t num_layers;
	float turb[3];
} SwhTextureEffect;
int swh_scene_texture_effect(const SwhScene* scene, uint32_t material, SwhTextureEffect* out_effect);
/* A material's simulated effect (SpecialMaterialEffect::Water / Fire, src/common/material_water.rs,
 * material_fire.rs), flattened: kind 3 water, 4 fire (0: none); its sources (WaveSource / HeatSource,
 * kinds in the order those enums list them), its output slot and its words of simulation state. A time
 * function is SingleArgumentFunction: kind 0 constant a, 1 linear (scale a, offset b), 2 sine, 3 triangle,
 * 4 saw-tooth, 5 step wave (frequency a, phase b, amplitude c, offset d); a random value is
 * ValueWithRandomDeviation (value, deviation). */
typedef struct SwhTimeFunction {
	uint32_t kind;
	float a, b, c, d;
} SwhTimeFunction;
typedef struct SwhRandomValue {
	SwhTimeFunction value, deviation;
} SwhRandomValue;
typedef struct SwhSimSource {
	uint32_t kind;
	uint32_t points[2][2];           /* a single-point source uses points[0] */
	SwhTimeFunction offsets[2][2];   /* water: center_offset (offsets[0]) / points_offset */
	float frequency, phase, amplitude, offset, radius; /* water; fire fountains: frequency */
	uint32_t ramp;                   /* fire lightning */
	SwhRandomValue fire_offsets[2][2]; /* fire: point offset (fire_offsets[0]) / lightning offsets */
	SwhRandomValue heat, angle, speed, gravity, spawn_angle, spawn_distance, lifetime;
} SwhSimSource;
#define SWH_MAX_SIM_SOURCES 8
typedef struct SwhSimEffect {
	uint32_t kind;
	uint32_t resolution_log2[2];
	float update_frequency;
	float attenuation_param; /* water: fluidity; fire: heat_conductivity */
	uint32_t color_mode;     /* water: ColorTextureApplyMode */
	uint32_t slow;           /* fire */
	uint32_t has_color;      /* fire: palette from `color` */
	float color[3];
	float roughness;         /* water: Material::roughness */
	int32_t output_texture;  /* water: texture slot written */
	int32_t output_emissive; /* fire: emissive slot written */
	int32_t source_emissive; /* fire: the material's emissive texture, -1 without */
	uint32_t num_sources;
	uint64_t state_offset;   /* word offset of its two fields / heat maps */
	SwhSimSource sources[SWH_MAX_SIM_SOURCES];
} SwhSimEffect;
int swh_scene_simulated_effect(const SwhScene* scene, uint32_t material, SwhSimEffect* out_effect);
/* Words of simulation state the scene's simulated effects use (sw_reserve_simulation_state). */
int swh_scene_simulation_words(const SwhScene* scene, uint64_t* out_words);
/* The scene's light grid (bsp_map_compact.rs:162-188): the header (cell size[3], start[3] as floats, then
   size[3] as u32: 36 bytes), columns (start_z, first_sample, num_samples as u32) and samples (light cube
   6x3, light_direction_vector_scaled 3, directional_light_color 3: 24 floats each). With null arrays only
   the counts are written; otherwise the arrays hold at least those counts. */
int swh_scene_light_grid(const SwhScene* scene, void* out_header, uint32_t* out_columns, float* out_samples,
	uint64_t* num_columns, uint64_t* num_samples);
/* fetch_light_from_grid (triangle_models_rendering.rs:582-700) at a position: 24 floats as one sample. */
int swh_scene_fetch_light(const SwhScene* scene, const float pos[3], float out_sample[24]);
const char* swh_last_error(void);

typedef struct SwhFrameOptions {
	uint32_t width, height, pixel_format;
	uint32_t use_directional_lightmaps;
	uint32_t clear_background;
	float fov;      /* radians; 0 = 0.375*pi */
	float mip_bias;
	float shadows_quality; /* RendererConfig::shadows_quality, -1..1 (shadow-map size scale, log2) */
} SwhFrameOptions;

typedef struct SwhFrameOutputs {
	const SwSurfaceDesc* surfaces;
	uint32_t num_surfaces;
	uint32_t num_draws;
	uint64_t total_texels;
	const SwDrawCmd* draws;
	const SwVertex16* vertices;
	uint32_t num_vertices;
	uint32_t num_lights;
	const SwLight* lights;
	SwFrameParams params;
	uint32_t visible_leafs, camera_leaf;
	uint32_t skybox_draws; /* draws of the skybox (the first ones) */
	/* cube shadow maps (sw_build_shadow_maps / sw_set_light_shadows): one SwLightShadow per light, the
	 * depth draws of every side and the storage size; num_depth_draws 0 and all kinds NONE without them */
	const SwLightShadow* light_shadows;
	const SwDepthDraw* depth_draws;
	uint32_t num_depth_draws;
	uint32_t num_depth_vertices;
	const SwVertex16* depth_vertices;
	uint64_t shadow_texels;
	/* swh_frame_prepare_view: the depth draws are prepared on the GPU (sw_build_shadow_maps_view) from
	 * the cube sides and the leafs each side's visibility reaches; num_depth_draws is 0 then */
	const SwShadowSide* shadow_sides;
	uint32_t num_shadow_sides;
	uint32_t num_shadow_leafs;
	const SwShadowLeaf* shadow_leafs;
	/* triangle draws of the visible models (SW_RASTER_TRIANGLE draws among `draws`): their vertices */
	const SwTriVertex* tri_vertices;
	uint32_t num_tri_vertices;
	uint32_t model_triangles;
	/* generative texture effects of the frame (sw_update_textures, before the frame's surfaces) */
	const SwTexturePass* texture_passes;
	uint32_t num_texture_passes;
	uint32_t num_texture_shifts;
	const int32_t* texture_shifts;
	/* simulated texture effects of the frame (sw_update_simulations, after the texture passes) */
	const SwSimPass* sim_passes;
	uint32_t num_sim_passes;
	uint32_t num_sim_points;
	const SwSimPoint* sim_points;
	/* portal views (SwFrameInput.views): rendered before the frame's own draws [0, main_draws); the
	 * draws after them are the views'; total_texels spans the surfaces (surface_texels), the portal
	 * textures and the nested views' arenas */
	const SwView* views;
	uint32_t num_views;
	uint32_t main_draws;
	uint64_t surface_texels;
} SwhFrameOutputs;

typedef struct SwhFrame SwhFrame;

/* Per-frame host state (visibility marks, per-polygon frame data, output arrays). */
int swh_frame_create(const SwhScene* scene, SwhFrame** out_frame);
int swh_frame_destroy(SwhFrame* frame);
/* The map's world polygons and vertices (xyz floats) as sw_set_map takes them; the pointers stay valid
 * while the frame lives. */
int swh_frame_map(const SwhFrame* frame, const SwMapPolygon** out_polygons, uint32_t* out_num_polygons,
	const float** out_vertices, uint32_t* out_num_vertices);
/* Host work of one frame of the scene's camera path: visibility, surface preparation, light
 * selection, back-to-front traversal and draw setup. */
int swh_frame_prepare(SwhFrame* frame, uint32_t frame_index, const SwhFrameOptions* options);
/* Pointers into the frame's arrays, valid until the next swh_frame_prepare. */
int swh_frame_outputs(const SwhFrame* frame, SwhFrameOutputs* out);
/* A simulated effect's host state after the last prepared frame: its update step, the state buffer (0 or
 * 1) holding its current field / heat map, whether it has generated its texture, its live particles. */
int swh_frame_effect_state(const SwhFrame* frame, uint32_t material, uint32_t* out_update_step,
	uint32_t* out_current_buffer, uint32_t* out_generated, uint32_t* out_particles);
/* The host half of a frame whose surfaces and world draws the GPU prepares (sw_draw_frame_view):
 * visibility, light positioning, the skybox draws and the visible leafs with their bounds, lights and
 * back-to-front order. swh_frame_view_input fills everything of SwViewFrameInput but mip_bias and the
 * postprocess / destination fields; its pointers stay valid until the next prepare call. */
int swh_frame_prepare_view(SwhFrame* frame, uint32_t frame_index, const SwhFrameOptions* options);
int swh_frame_view_input(const SwhFrame* frame, SwViewFrameInput* out);

typedef struct SwhRenderer SwhRenderer;

/* Renderer::new: upload the scene's static data to `device` (sw_create). */
int swh_renderer_create(const SwhScene* scene, uint32_t device, SwhRenderer** out_renderer);
int swh_renderer_destroy(SwhRenderer* renderer);
/* Renderer::prepare_frame: host work + sw_frame_begin + sw_submit_surfaces. */
int swh_renderer_prepare_frame(SwhRenderer* renderer, uint32_t frame_index, const SwhFrameOptions* options);
/* Renderer::draw_frame: sw_submit_draws + sw_render into dst (optional). */
int swh_renderer_draw_frame(SwhRenderer* renderer, void* dst, uint32_t pitch, int dst_is_device);
/* One whole frame as the host's frame loop runs it (host.rs:400-416: prepare_frame, draw_frame and,
 * when `post` is not NULL, perform_postprocessing): host work, then one CUDA graph (upload, surface and
 * draw preparation, surfaces, raster, postprocess) with the Color32 result (post) or the frame (no
 * post) in dst. */
int swh_renderer_render_frame(SwhRenderer* renderer, uint32_t frame_index, const SwhFrameOptions* options,
	const SwPostConfig* post, float frame_duration_s, const float color_modulate[3], void* dst, uint32_t pitch,
	int dst_is_device);
/* swh_renderer_render_frame's preparation: 1 (default) = the GPU prepares the surfaces and the world
 * draws (swh_frame_prepare_view + sw_draw_frame_view), 0 = the host does (swh_frame_prepare +
 * sw_draw_frame). Both give the same frame. */
int swh_renderer_set_gpu_prep(SwhRenderer* renderer, int enable);
/* Frames in flight of swh_renderer_render_frame (sw_set_frames_in_flight): with 2, a call returns once its
 * frame is enqueued and the previous frame is in its host buffer (registered buffers, alternated). */
int swh_renderer_set_frames_in_flight(SwhRenderer* renderer, uint32_t frames);
/* The GPU context and the frame used by the renderer. */
SwCtx* swh_renderer_context(SwhRenderer* renderer);
SwhFrame* swh_renderer_frame(SwhRenderer* renderer);

#ifdef __cplusplus
}
#endif

#endif /* SWHOST_H */
