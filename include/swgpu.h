/*
 * swgpu.h — C ABI of the GB300 world-rendering path of Square-Wheel.
 *
 * The Rust host (or any other host) keeps BSP/portal visibility, leaf ordering, per-polygon surface
 * preparation and per-polygon draw setup.  It hands the results to this library in two arrays:
 *   - SwSurfaceDesc: one per visible polygon surface, the arguments the reference passes to
 *     build_surface_{simple,directional}_lightmap and mix_surface_with_texture
 *     (src/square_wheel/partial_renderer.rs:1682-1819);
 *   - SwDrawCmd + SwVertex16: one per rasterised polygon in exact submission order, the arguments the
 *     reference passes to Rasterizer::fill_polygon (src/square_wheel/partial_renderer.rs:4084-4140).
 * The library builds the surfaces, rasterises them into a colour32/colour64 frame, and runs the HDR
 * postprocessor (bloom + tonemap + auto exposure) and the frame upscaler.
 *
 * Conventions
 *   - Every function returns SW_OK (0) or a negative SwStatus and never aborts; sw_last_error() gives text.
 *   - The context owns every device buffer; the caller owns host buffers.
 *   - One SwCtx is used by one caller thread; work is ordered on the context's CUDA stream and is
 *     asynchronous until sw_sync() unless a call reads results back into host memory.
 *   - Colour layouts are the reference's: Color32 = A<<24|R<<16|G<<8|B (src/common/color.rs:21-24),
 *     Color64 = A<<48|R<<32|G<<16|B (src/common/color.rs:144-147).
 *   - Arithmetic follows the reference's generic (non-SSE) fast_math semantics bit-exactly:
 *     exact 1/x and 1/sqrt(x), truncating float->int, unfused multiply-add
 *     (src/square_wheel/fast_math.rs:370-740).
 */
#ifndef SWGPU_H
#define SWGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWGPU_ABI_VERSION 2

typedef enum SwStatus {
	SW_OK = 0,
	SW_ERR_INVALID_ARGUMENT = -1,
	SW_ERR_OUT_OF_MEMORY = -2,
	SW_ERR_CUDA = -3,
	SW_ERR_LIMIT = -4,
	SW_ERR_NO_DEVICE = -5,
	SW_ERR_STATE = -6,
	SW_ERR_KERNEL = -7,
} SwStatus;

typedef enum SwPixelFormat {
	SW_PIXEL_C32 = 0, /* Color32, 4 bytes per pixel */
	SW_PIXEL_C64 = 1, /* Color64, 8 bytes per pixel (HDR) */
} SwPixelFormat;

/* BlendingMode, src/common/material.rs (None, Average, Additive, AlphaTest, AlphaBlend). */
typedef enum SwBlend {
	SW_BLEND_NONE = 0,
	SW_BLEND_AVERAGE = 1,
	SW_BLEND_ADDITIVE = 2,
	SW_BLEND_ALPHA_TEST = 3,
	SW_BLEND_ALPHA_BLEND = 4,
} SwBlend;

/* TetureCoordinatesInterpolationMode, src/square_wheel/rasterizer.rs:4-10, plus the triangle fill. */
typedef enum SwRasterMode {
	SW_RASTER_FULL_PERSPECTIVE = 0,
	SW_RASTER_LINE_Z_CORRECTED = 1,
	SW_RASTER_AFFINE = 2,
	/* Rasterizer::fill_triangle (src/square_wheel/rasterizer.rs:731-1292): a textured triangle with
	 * per-vertex light (models, decals, sprites); the draw's three vertices are SwTriVertex. */
	SW_RASTER_TRIANGLE = 3,
} SwRasterMode;

/* ---- static data, uploaded once (Renderer::new, src/square_wheel/renderer.rs:24-59) ---- */

/* Texture flags, src/square_wheel/textures.rs:11-18. */
#define SW_TEX_HAS_NORMAL_MAP 1u
#define SW_TEX_HAS_NON_ONE_ROUGHNESS 2u
#define SW_TEX_IS_METAL 4u

/* One mip level of a material texture. Texels are TextureElement (8 bytes: Color32 diffuse +
 * packed i8x4 normal/roughness, src/square_wheel/textures.rs:20-62), stored row-major. */
typedef struct SwTextureMip {
	uint64_t offset; /* in texels, into SwCreateInfo.texels */
	uint32_t width;
	uint32_t height;
	uint32_t flags; /* SW_TEX_* of the material */
	uint32_t reserved;
} SwTextureMip;

/* One mip level of an emissive texture (TextureLite = Color32 image, src/square_wheel/textures.rs:89-91). */
typedef struct SwEmissiveMip {
	uint64_t offset; /* in pixels, into SwCreateInfo.emissive_pixels */
	uint32_t width;
	uint32_t height;
} SwEmissiveMip;

/* DirectionalLightmapElement, src/common/bsp_map_compact.rs:144-156 (40 bytes). */
typedef struct SwDirectionalLightmapElement {
	float ambient_light[3];
	float light_direction_vector_scaled[3];
	float directional_light_deviation;
	float directional_light_color[3];
} SwDirectionalLightmapElement;

typedef struct SwCreateInfo {
	uint32_t abi_version; /* SWGPU_ABI_VERSION */
	uint32_t device;      /* CUDA device ordinal */
	const uint64_t* texels; /* TextureElement raw 8-byte values */
	uint64_t num_texels;
	const SwTextureMip* texture_mips;
	uint32_t num_texture_mips;
	uint32_t num_emissive_mips;
	const uint32_t* emissive_pixels; /* Color32 raw values */
	uint64_t num_emissive_pixels;
	const SwEmissiveMip* emissive_mips;
	/* LightmapElement = [f32;3] (src/common/bsp_map_compact.rs:142); element 0 is never used (offset 0 = no lightmap). */
	const float* lightmaps;
	uint64_t num_lightmap_elements;
	const SwDirectionalLightmapElement* directional_lightmaps;
	uint64_t num_directional_lightmap_elements;
	/* Capacity hints (0 = defaults). Exceeding them later grows the buffers. */
	uint64_t max_surface_texels;
	uint32_t max_surfaces;
	uint32_t max_draws;
} SwCreateInfo;

/* ---- per-frame data ---- */

/* DynamicLightWithShadow without a shadow map (shadow factor 1), src/square_wheel/light.rs:4-11,
 * created as in src/square_wheel/renderer_structs.rs:228-238. */
typedef struct SwLight {
	float position[3];
	float radius;
	float inv_square_radius; /* 1/(radius*radius), computed by the host */
	float color[3];
} SwLight;

#define SW_MAX_POLYGON_LIGHTS 6 /* MAX_POLYGON_LIGHTS, src/square_wheel/partial_renderer.rs:1666 */
#define SW_NO_LIGHTMAP 0u
#define SW_NO_EMISSIVE 0xFFFFFFFFu

/* Surface flags */
#define SW_SURF_DIFFUSE_LAYER 1u /* material.light && material.diffuse (partial_renderer.rs:1701) */

/* One visible polygon surface: the arguments of build_surface_impl_6_static_params
 * (src/square_wheel/surfaces.rs:433-451) plus the emissive layer of mix_surface_with_texture
 * (src/square_wheel/surfaces.rs:854-901), as computed in src/square_wheel/partial_renderer.rs:1682-1819. */
typedef struct SwSurfaceDesc {
	float basis_u[3];      /* PolygonBasisVecs scaled for the mip and shifted (partial_renderer.rs:1736-1740) */
	float basis_v[3];
	float basis_start[3];
	float basis_normal[3];
	uint32_t size[2];      /* surface_size */
	int32_t tc_start[2];   /* surface_tc_min + texture shift >> mip */
	uint32_t texture_mip;  /* index into SwCreateInfo.texture_mips */
	uint32_t emissive_mip; /* index into SwCreateInfo.emissive_mips, or SW_NO_EMISSIVE */
	uint32_t lightmap_offset; /* element offset, SW_NO_LIGHTMAP (0) if none */
	uint32_t lightmap_size[2];
	uint32_t lightmap_scale_log2; /* LIGHTMAP_SCALE_LOG2 - mip, 0..4 */
	uint32_t lightmap_tc_shift[2];
	uint32_t flags;        /* SW_SURF_* */
	uint32_t num_lights;   /* <= SW_MAX_POLYGON_LIGHTS */
	uint16_t lights[SW_MAX_POLYGON_LIGHTS]; /* indices into the frame's SwLight array */
	float emissive_light[3];
	uint64_t out_offset;   /* first texel of this surface in the frame's surface arena */
} SwSurfaceDesc;

/* A projected polygon vertex in 16.16 fixed point (PolygonPointProjected, rasterizer.rs:1484-1489). */
typedef struct SwVertex16 {
	int32_t x;
	int32_t y;
} SwVertex16;

/* A projected triangle vertex in 16.16 fixed point (TrianglePointProjected, rasterizer.rs:1492-1498):
 * screen position, texture coordinates in texels and light (1.0 = 65536, lanes r, g, b). */
typedef struct SwTriVertex {
	int32_t x, y;
	int32_t tc[2];
	int32_t light[3];
	int32_t reserved;
} SwTriVertex;

#define SW_MAX_POLYGON_VERTICES 24 /* MAX_VERTICES, src/square_wheel/renderer_utils.rs:4 */

/* Where a draw's texture lives. */
typedef enum SwTexSource {
	SW_TEXSRC_SURFACE = 0, /* a surface of the frame's surface arena (world polygons) */
	SW_TEXSRC_SKYBOX = 1,  /* a skybox side texture at one mip (draw_skybox, partial_renderer.rs:2311-2448),
	                       in the texels uploaded by sw_set_skybox */
	SW_TEXSRC_LITE = 2,    /* a Color32 texture (TextureLite, textures.rs:89-91: model skins, decals, sprites) in
	                       the pixels uploaded by sw_set_lite_textures; triangle draws only */
} SwTexSource;

/* One Rasterizer::fill_polygon call (src/square_wheel/rasterizer.rs:35-80) as emitted by
 * draw_polygon (src/square_wheel/partial_renderer.rs:4011-4142). Equations are the ones passed to
 * fill_polygon (already scaled by z_scale for the non-affine modes). With mode SW_RASTER_TRIANGLE it is
 * one Rasterizer::fill_triangle call instead (draw_view_models, draw_polygon_decals, draw_sprite,
 * partial_renderer.rs:2284, 2794, 3290): vertex_count 3, first_vertex indexes the SwTriVertex array,
 * tex_source SW_TEXSRC_LITE, the equations unused. */
typedef struct SwDrawCmd {
	uint32_t first_vertex; /* into the SwVertex16 array */
	uint32_t vertex_count; /* 3..SW_MAX_POLYGON_VERTICES, clockwise */
	uint32_t mode;         /* SwRasterMode */
	uint32_t blend;        /* SwBlend */
	float depth_eq[3];     /* d_inv_z_dx, d_inv_z_dy, k */
	float tc_eq[6];        /* d_tc_dx[2], d_tc_dy[2], k[2] */
	uint32_t tex_size[2];  /* texture size (surface, or skybox side mip: size x size) */
	uint32_t tex_source;   /* SwTexSource */
	uint64_t tex_offset;   /* texture's first texel in the surface arena or the skybox texels */
} SwDrawCmd;

typedef struct SwFrameParams {
	uint32_t pixel_format; /* SwPixelFormat of surfaces and framebuffer */
	uint32_t width;
	uint32_t height;
	uint32_t use_directional_lightmaps; /* RendererConfig::use_directional_lightmaps && data present */
	float cam_pos[3];
	uint32_t clear_background; /* draw_background before rasterisation (partial_renderer.rs:249-257) */
	uint32_t reserved;
} SwFrameParams;

/* PostprocessorConfig (src/square_wheel/postprocessor_config.rs). Every entry point clamps it first, as
 * Postprocessor::synchronize_config does before each frame (src/square_wheel/postprocessor.rs:958-977). */
typedef struct SwPostConfig {
	float exposure_update_speed;
	float base_brightness;
	float zero_level_brightness;
	float brightness_scale_power;
	float min_exposure;
	float max_exposure;
	float bloom_sigma;
	uint32_t bloom_buffer_scale_log2;
	float bloom_scale;
	uint32_t linear_bloom_filter;
} SwPostConfig;

typedef enum SwUpscaleMode {
	SW_UPSCALE_NEAREST = 0, /* FrameUpscaler::perform_upscale_impl::<SCALE> */
	SW_UPSCALE_AVG2X = 1,   /* FrameUpscaler::perform_upscale_2x_linear */
	SW_UPSCALE_LEARNED = 2, /* no reference counterpart: learned 2x upscaler (swlearn.h), scale must be 2 */
} SwUpscaleMode;

typedef struct SwCtx SwCtx;

/* Renderer::new (src/square_wheel/renderer.rs:24-59): upload static map data. */
int sw_create(const SwCreateInfo* info, SwCtx** out_ctx);
int sw_destroy(SwCtx* ctx);
const char* sw_last_error(const SwCtx* ctx);
int sw_sync(SwCtx* ctx);

/* Start a frame: camera, lights, pixel format and frame size (Renderer::prepare_frame, renderer.rs:61-104). */
int sw_frame_begin(SwCtx* ctx, const SwFrameParams* params, const SwLight* lights, uint32_t num_lights);

/* Surfaces of the frame's visible polygons, in any order; out_offset values must not overlap.
 * Builds them on the GPU (build_polygons_surfaces, partial_renderer.rs:1640-1832).
 * total_texels = size of the surface arena for this frame. */
int sw_submit_surfaces(SwCtx* ctx, const SwSurfaceDesc* surfaces, uint32_t num_surfaces, uint64_t total_texels);

/* Build the surfaces of the last sw_submit_surfaces again without re-uploading descriptors (after a
 * sw_frame_begin that changed only the camera position or the lights' parameters): one persistent
 * launch over all of them, replayed as a CUDA graph while the frame graph setting is on
 * (sw_set_frame_graph). */
int sw_rebuild_surfaces(SwCtx* ctx);
/* The same build as one kernel launch per surface, in descriptor order (the reference's per-polygon
 * tasks, partial_renderer.rs:1822-1831): the baseline the persistent launch is measured against. The
 * arena comes out identical. Needs descriptors from sw_submit_surfaces. */
int sw_rebuild_surfaces_per_surface(SwCtx* ctx);

/* Use a surface arena built elsewhere (host memory, pixel_format of sw_frame_begin) instead of
 * sw_submit_surfaces, e.g. textures the caller prepared itself. */
int sw_set_surfaces(SwCtx* ctx, const void* texels, uint64_t total_texels);

/* Skybox side textures of the map's sky material (SkyboxTextures<Color32> and <Color64>,
 * src/square_wheel/textures.rs:79-87, as MapMaterialsProcessor::get_skybox_textures returns them:
 * make_skybox_side_texture{,64} + make_skybox_side_texture_mips, textures.rs:183-290). Every side's mips
 * concatenated in the same order in both formats, so one texel offset (SwDrawCmd::tex_offset with
 * tex_source SW_TEXSRC_SKYBOX) addresses both; draws read the array of the frame's pixel format.
 * Synchronous upload; NULL / 0 texels removes the skybox. Load-time data like sw_create's. */
int sw_set_skybox(SwCtx* ctx, const uint32_t* texels32, const uint64_t* texels64, uint64_t num_texels);

/* Replace the lightmaps with a compiled map's compressed lightmap lumps, uploaded as the file holds them
 * and decoded on the GPU (LightmapElementCompressed::decompress and
 * DirectionalLightmapElementCompressed::decompress, src/common/lightmap_compression.rs:64-68, 88-130;
 * what load_map does on the host, bsp_map_save_load.rs:208-215): `lightmaps` holds num_elements 4-byte
 * CompressedColor records (r, g, b, scale: value = component * scale / 255), `directional` holds
 * num_directional_elements 13-byte records (ambient CompressedColor, direction CompressedVector - three
 * i8 and a scale, value = component * scale / 127 -, u8 deviation / 255, directional CompressedColor).
 * Fails if sw_set_map's polygons read past the new lightmaps. Load-time data like sw_create's;
 * synchronous (waits for frames in flight). */
#define SW_LIGHTMAP_COMPRESSED_BYTES 4
#define SW_DIR_LIGHTMAP_COMPRESSED_BYTES 13
int sw_set_lightmaps_compressed(SwCtx* ctx, const void* lightmaps, uint64_t num_elements, const void* directional,
	uint64_t num_directional_elements);

/* Generative texture effects (GenerativeTextureEffect::update, map_materials_processor.rs:249-303): each
 * frame the caller submits the passes that rewrite the effects' output textures, which are ordinary
 * texture slots (texture_mips entries, or emissive_mips entries) of the static data that surfaces then
 * read through SwMaterialFrame.texture / the surface descriptors. Passes run before the next frame's
 * surfaces, on the context's stream.
 *   SW_TEXPASS_TURB (make_turb_distortion, generative_texture_effect_turb.rs:91-138): dst texel (x, y) =
 *     src texel ((x + s[y]) & (w - 1), (y + s[x]) & (h - 1)), s = the pass's max(w, h) shifts starting at
 *     shifts_offset; src and dst the same power-of-two size; with SW_TEXPASS_EMISSIVE both are emissive
 *     (Color32) mips, else material mips.
 *   SW_TEXPASS_LAYER (apply_texture_layer, generative_texture_effect_layered.rs:163-381): the src mip,
 *     tiled over dst with offset `shift` (rem_euclid of the src size), modulated by `light` (applied when
 *     a component is outside [0.98, 1.02]) and blended into dst's current texels with blending_mode
 *     (SW_BLEND_*); an additive layer whose light is at most 1/128 in every component is skipped.
 *     Consecutive LAYER passes with the same dst form one group applied in order.
 * A pass's dst must not be another pass's src, and two groups must not share a dst. Validated before
 * anything is uploaded or launched. */
#define SW_TEXPASS_TURB 1u
#define SW_TEXPASS_LAYER 2u
#define SW_TEXPASS_EMISSIVE 0x100u
typedef struct SwTexturePass {
	uint32_t kind;          /* SW_TEXPASS_TURB or SW_TEXPASS_LAYER, | SW_TEXPASS_EMISSIVE (TURB only) */
	uint32_t dst_mip;       /* texture_mips (emissive_mips) index of the output mip */
	uint32_t src_mip;       /* texture_mips (emissive_mips) index of the source mip */
	uint32_t blending_mode; /* LAYER: SW_BLEND_* of the layer's material */
	int32_t shift[2];       /* LAYER: layer texture offset (tex_coord_shift evaluated, >> mip) */
	float light[3];         /* LAYER: modulate colour (r, g, b) */
	uint32_t shifts_offset; /* TURB: first of the mip's max(w, h) shifts in `shifts` */
} SwTexturePass;
int sw_update_textures(SwCtx* ctx, const SwTexturePass* passes, uint32_t num_passes, const int32_t* shifts,
	uint32_t num_shifts);

/* Simulated generative texture effects, water (GenerativeTextureEffectWater, generative_texture_effect_water.rs)
 * and fire (GenerativeTextureEffectFire, generative_texture_effect_fire.rs). Their fields live on the
 * device in the context's simulation state: sw_reserve_simulation_state allocates it (`words` 4-byte
 * words, zeroed; a second call with another size replaces it, zeroed). Each frame the caller submits the
 * passes of that frame's update steps and texture generation; the library runs them on the context's
 * stream, one kernel launch per distinct `launch` number, in increasing order (passes must be sorted by
 * it), every pass of a launch in parallel. Kinds (field and heat maps are 2^size_log2[0] x
 * 2^size_log2[1] words, row-major, both edges wrapping unless stated):
 *   SW_SIM_WATER_POINTS: the wave sources of one step (generative_texture_effect_water.rs:57-215): for each
 *     point in order, state_src[address] += value and state_dst[address] -= value (f32; value holds the
 *     f32's bits). Points with equal addresses must be consecutive (the host sorts them stably).
 *   SW_SIM_WATER_STEP (update_wave_field, :308-418): state_dst[x, y] = ((src[x-1, y] + src[x+1, y] +
 *     src[x, y-1] + src[x, y+1]) * 0.5 - state_dst[x, y]) * attenuation, src = state_src, attenuation =
 *     `param` as f32 bits.
 *   SW_SIM_FIRE_STEP (update_heat_map, generative_texture_effect_fire.rs:430-550): the heat map at state_src
 *     propagated upwards into state_dst (u32 words holding 0..255), attenuation_i = `param`; with
 *     SW_SIM_FIRE_SLOW in flags, the row-sequential slow form. The last row becomes 0.
 *   SW_SIM_FIRE_POINTS (the heat sources and particles of one step, :62-321): state_dst[address] =
 *     max(state_dst[address], value).
 *   SW_SIM_WATER_TEXTURE (make_wavy_texture, generative_texture_effect_water.rs:420-682): texture mip
 *     dst_mip (the field's size) gets the normals of the field at state_src with roughness `param` (f32
 *     bits); its diffuse per colour mode (flags >> SW_SIM_COLOR_MODE_SHIFT: 0 single colour, 1 source
 *     texture, 2 source deformed by the normal, 3 deformed along x only) from base_color or from mip
 *     src_mip (the material's mip 0, nearest-resized to the field's size); modes 0 and 1 write diffuse
 *     only with SW_SIM_WATER_INIT_DIFFUSE (the first generation) and keep it afterwards.
 *   SW_SIM_FIRE_TEXTURE (generate_emissive_texture_based_on_heat_map, :552-566): emissive mip dst_mip =
 *     palette[heat at state_src], the palette being the pass's 256 points (value = Color32).
 *   SW_SIM_TEXTURE_MIP / SW_SIM_EMISSIVE_MIP (build_texture_mip / build_texture_lite_mip, textures.rs:
 *     309-415): mip dst_mip (half of src_mip's size) rebuilt from mip src_mip.
 * Everything (kinds, offsets against the state, mips and sizes, point ranges and addresses) is validated
 * before anything is uploaded or launched. */
#define SW_SIM_WATER_POINTS 1u
#define SW_SIM_WATER_STEP 2u
#define SW_SIM_FIRE_STEP 3u
#define SW_SIM_FIRE_POINTS 4u
#define SW_SIM_WATER_TEXTURE 5u
#define SW_SIM_FIRE_TEXTURE 6u
#define SW_SIM_TEXTURE_MIP 7u
#define SW_SIM_EMISSIVE_MIP 8u
#define SW_SIM_FIRE_SLOW 1u
#define SW_SIM_WATER_INIT_DIFFUSE 2u
#define SW_SIM_COLOR_MODE_SHIFT 8u
typedef struct SwSimPoint {
	uint32_t address; /* word index within the pass's field / heat map (palette index for FIRE_TEXTURE) */
	uint32_t value;   /* f32 bits (water), heat 0..255 (fire), Color32 (palette) */
} SwSimPoint;
typedef struct SwSimPass {
	uint32_t kind;         /* SW_SIM_* */
	uint32_t launch;       /* launch number, non-decreasing over the pass list */
	uint32_t size_log2[2]; /* field / heat map size (all kinds but the MIP ones) */
	uint64_t state_src;    /* word offset of the field / heat map read */
	uint64_t state_dst;    /* word offset of the field / heat map written */
	uint32_t first_point;  /* POINTS and FIRE_TEXTURE: the pass's points */
	uint32_t num_points;
	uint32_t dst_mip;      /* TEXTURE and MIP passes: texture_mips (EMISSIVE: emissive_mips) index written */
	uint32_t src_mip;      /* WATER_TEXTURE: colour source mip; MIP passes: the mip read */
	uint32_t flags;        /* SW_SIM_FIRE_SLOW, SW_SIM_WATER_INIT_DIFFUSE, colour mode << SW_SIM_COLOR_MODE_SHIFT */
	uint32_t param;        /* see the kinds */
	uint32_t base_color;   /* WATER_TEXTURE colour mode 0: the Color32 */
	uint32_t reserved;
} SwSimPass;
int sw_reserve_simulation_state(SwCtx* ctx, uint64_t words);
int sw_update_simulations(SwCtx* ctx, const SwSimPass* passes, uint32_t num_passes, const SwSimPoint* points,
	uint32_t num_points);
/* Diagnostics: copy words [first, first + count) of the simulation state to host memory (synchronises). */
int sw_read_simulation_state(SwCtx* ctx, uint64_t first, uint64_t count, uint32_t* out);

/* Page-lock a host buffer the caller reuses for its frames (the window surface's pixels, say) with
 * cudaHostRegister (mapped), so that frames written to host memory inside it go straight from the
 * device into it instead of through the library's pinned staging buffer and a host copy (sw_draw_frame's
 * tonemap writes its rows there directly). Unregister it (or destroy the context) before freeing the
 * memory; registered buffers must not overlap. */
int sw_register_host_buffer(SwCtx* ctx, void* ptr, uint64_t bytes);
int sw_unregister_host_buffer(SwCtx* ctx, void* ptr);

/* Draw commands in exact submission order (draw_skybox, then draw_tree/draw_leaf/draw_polygon,
 * partial_renderer.rs:1285-1325, 2311-2559, 4011-4142). */
int sw_submit_draws(SwCtx* ctx, const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices);
/* The same with triangle draws among them (SW_RASTER_TRIANGLE: the leaf's decals after its polygons,
 * then its models and sprites, draw_leaf, partial_renderer.rs:2519-2792), their vertices in tri_vertices. */
int sw_submit_draws_ex(SwCtx* ctx, const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices, const SwTriVertex* tri_vertices, uint32_t num_tri_vertices);
/* The Color32 textures triangle draws read (SW_TEXSRC_LITE: model skins, decal and sprite textures with
 * their mips, TextureLite, textures.rs:89-91), all in one array; a draw's tex_offset is its first pixel.
 * Load-time data like sw_create's; synchronous. */
int sw_set_lite_textures(SwCtx* ctx, const uint32_t* pixels, uint64_t num_pixels);

/* Rasterise the submitted draws (Renderer::draw_frame, renderer.rs:106-124) into the context's
 * framebuffer. If dst != NULL the frame (pixel_format of sw_frame_begin) is also copied there:
 * dst_is_device != 0 means a device pointer, otherwise host memory; pitch is in pixels. */
int sw_render(SwCtx* ctx, void* dst, uint32_t pitch, int dst_is_device);

/* Postprocessor::perform_postprocessing (src/square_wheel/postprocessor.rs:68-204) on the context's
 * colour64 framebuffer, writing Color32 to dst (pitch in pixels). Exposure state lives in the context,
 * starting at 1.0; the frame's average colour updates it for the next frame. */
int sw_postprocess(SwCtx* ctx, const SwPostConfig* config, float frame_duration_s, const float color_modulate[3],
	void* dst, uint32_t pitch, int dst_is_device);

/* No counterpart in the reference. The postprocessor for callers that cannot allocate device memory
 * (engines that hand out all device memory from their own fixed pools, frame loops that cannot afford
 * cudaMalloc's implicit device synchronisation): no context, no allocation. hdr (width x height
 * Color64, tightly packed), dst (Color32, pitch in pixels) and average (4 floats, lanes b, g, r, a; may
 * be NULL) are device pointers; config and color_modulate are host memory; stream is a cudaStream_t
 * (NULL = default stream). The bloom buffers and per-line sums live in one static device array of
 * SW_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit, so frames are limited
 * to SW_NOALLOC_MAX_WIDTH x SW_NOALLOC_MAX_HEIGHT (SW_ERR_LIMIT beyond). The first call on a device
 * (with that device current) looks the array's address up once; make it before any stream capture.
 * cudaDeviceReset unloads the library's device code, so that address is stale afterwards: do not call
 * this entry point after a cudaDeviceReset in the same process. All calls share the array: calls that
 * overlap on the GPU race. The configuration is clamped as Postprocessor::synchronize_config clamps it.
 * The exposure is an input; the frame's average colour (postprocessor.rs:206-223 feeds it to
 * update_exposure) is written to `average`. */
#define SW_NOALLOC_MAX_WIDTH 1920u
#define SW_NOALLOC_MAX_HEIGHT 1080u
#define SW_NOALLOC_SCRATCH_BYTES 8320512u
int sw_postprocess_noalloc(const uint64_t* hdr, uint32_t width, uint32_t height, const SwPostConfig* config,
	float exposure, const float color_modulate[3], uint32_t* dst, uint32_t pitch, float* average, void* stream);

/* FrameUpscaler::perform_upscale (src/square_wheel/frame_upscaler.rs:42-70): src is a Color32 frame of
 * (dst_width/scale) x (dst_height/scale) pixels with pitch = its width; dst has dst_pitch pixels per row. */
int sw_upscale(SwCtx* ctx, uint32_t mode, uint32_t scale, const void* src, int src_is_device, void* dst,
	uint32_t dst_width, uint32_t dst_height, uint32_t dst_pitch, int dst_is_device);

/* Load a frame into the context's frame buffer (e.g. an HDR frame to postprocess that was rendered
 * elsewhere, Postprocessor::get_hdr_buffer, postprocessor.rs:56-66). Pixels are tightly packed. */
int sw_set_framebuffer(SwCtx* ctx, const void* src, uint32_t width, uint32_t height, uint32_t pixel_format,
	int src_is_device);

typedef struct SwStats {
	uint64_t surfaces;          /* surfaces built since sw_create */
	uint64_t surface_texels;    /* texels built since sw_create */
	uint64_t draws;             /* draw commands submitted since sw_create */
	uint64_t bad_texel_fetches; /* rasteriser fetches outside a surface (always 0 for well-formed draws) */
	uint64_t pixel_writes;      /* span pixels the rasteriser wrote (texel fetch + blend) since sw_create */
	uint64_t upload_bytes;      /* per-frame bytes copied from host to device memory since sw_create */
} SwStats;
int sw_get_stats(SwCtx* ctx, SwStats* out_stats);

/* Device-time measurement of the last call of each stage (CUDA events on the context's stream around
 * the stage's kernels only): [0] surface build, [1] rasterisation, [2] postprocess, [3] upscale, and
 * [4] the whole frame from sw_frame_begin to the end of sw_postprocess (both internal streams joined,
 * uploads and any idle time waiting for the host included), in ms. A stage not run since timing was
 * enabled reads 0. Timing is off by default; sw_enable_timing(ctx, 1) turns it on. sw_get_timings
 * synchronises. */
int sw_enable_timing(SwCtx* ctx, int enable);
int sw_get_timings(SwCtx* ctx, float out_ms[5]);

/* The context's CUDA stream (cudaStream_t) for callers that order their own work after the frame. */
int sw_get_stream(SwCtx* ctx, void** out_stream);

/* ---- whole frame in one call, as one CUDA graph (no reference counterpart) ----
 * Everything one frame of Renderer::prepare_frame + draw_frame + Postprocessor::perform_postprocessing
 * (renderer.rs:61-124, postprocessor.rs:68-204) hands to the GPU: sw_draw_frame is the same as
 * sw_frame_begin + sw_submit_surfaces + sw_submit_draws + sw_render (+ sw_postprocess), with the same
 * validation, results and exposure state, but the host prepares all of the frame's arrays first and the
 * device work (uploads, surface build, raster setup and tiles, postprocess, exposure readback) is
 * captured into one CUDA graph: the first frame instantiates it, later frames update it in place and
 * replay it, so the kernels run back to back without host submission gaps. */
/* A nested view of a whole frame (sw_draw_frame): a portal's texture (build_view_portals_textures,
 * partial_renderer.rs:2008-2283) rendered before the frame's own draws. Its render target is the
 * width x height region of the surface arena at target_offset (row pitch = width), cleared to black, then
 * drawn from draws [first_draw, first_draw + num_draws) (background first if clear_background) and
 * finally mixed with the portal's texture (mix_surface_with_texture, surfaces.rs:854-971): the lite
 * texture mip of mix_size pixels at mix_offset (SwCreateInfo lite pixels, sw_set_lite_textures),
 * tiled from mix_tc_min, modulated by mix_light, blended with mix_blend (SW_VIEW_NO_MIX: no texture).
 * A view may sample regions that earlier views rendered; views render in array order. */
#define SW_VIEW_NO_MIX 0xFFFFFFFFu
typedef struct SwView {
	uint64_t target_offset;
	uint32_t width, height;
	uint32_t first_draw, num_draws;
	uint32_t clear_background;
	uint32_t mix_blend;
	uint64_t mix_offset;
	uint32_t mix_size[2];
	int32_t mix_tc_min[2];
	float mix_light[3];
	uint32_t reserved;
} SwView;

typedef struct SwFrameInput {
	SwFrameParams params;
	uint32_t num_lights;
	const SwLight* lights;
	const SwSurfaceDesc* surfaces;
	uint64_t total_texels;
	uint32_t num_surfaces;
	uint32_t num_draws;
	const SwDrawCmd* draws;
	const SwVertex16* vertices;
	uint32_t num_vertices;
	uint32_t postprocess;      /* 1: postprocess the colour64 frame to Color32 into dst; 0: stop after rasterisation */
	SwPostConfig post;
	float frame_duration_s;
	float color_modulate[3];
	void* dst;                 /* postprocess: Color32 output; otherwise the frame (pixel_format); may be NULL */
	uint32_t dst_pitch;        /* pixels */
	int32_t dst_is_device;
	const SwTriVertex* tri_vertices; /* vertices of the SW_RASTER_TRIANGLE draws */
	uint32_t num_tri_vertices;
	uint32_t num_views;        /* nested views (portal textures), rendered first; 0: none */
	const SwView* views;
	uint32_t main_draws;       /* with views: the frame's own draws are [0, main_draws) */
	uint32_t reserved;
} SwFrameInput;
int sw_draw_frame(SwCtx* ctx, const SwFrameInput* frame);
/* Graph capture of sw_draw_frame: on (default) or off (the same work launched directly). */
int sw_set_frame_graph(SwCtx* ctx, int enable);
/* Frames in flight of the whole-frame calls (sw_draw_frame, sw_draw_frame_view). 1 (default): a call
 * returns when its frame is complete. 2: a postprocessed frame whose Color32 destination lies in a
 * registered host buffer (sw_register_host_buffer) returns once it is enqueued and the previous frame is
 * in its destination; its copy into host memory runs on a copy engine while the next frame computes,
 * as the reference overlaps the next frame's preparation with the previous frame's presentation
 * (host.rs:438-448). Give consecutive frames different destination buffers; sw_sync waits for both.
 * Frames and exposures are the same in either mode. */
int sw_set_frames_in_flight(SwCtx* ctx, uint32_t frames);

/* ---- GPU-side surface and draw preparation (no reference counterpart; the reference runs these steps
 * on the host in prepare_polygons_surfaces / build_polygons_surfaces / draw_tree, see below) ----
 *
 * The host keeps what is serial and tiny (visibility, light positioning, the BSP's back-to-front leaf
 * order, the skybox) and hands the GPU the visible leafs; the GPU runs, for every polygon of those
 * leafs, prepare_polygon_surface (partial_renderer.rs:1464-1638), the surface descriptor of
 * build_polygons_surfaces with polygon_is_affected_by_light (:1640-1819, :3877-3985) and draw_polygon
 * (:4011-4142), compacts surfaces in the reference's allocation order and draws in exact submission
 * order, and feeds the surface build and the rasteriser without a host round trip. Results equal the
 * host path's (sw_draw_frame with the host's SwSurfaceDesc / SwDrawCmd arrays) bit for bit. */

/* SwMapPolygon.flags */
#define SW_POLY_DRAW 1u          /* material.draw */
#define SW_POLY_SKY 2u           /* sky material: marks where the skybox shows, never a surface */
#define SW_POLY_DIFFUSE_LAYER 4u /* material.light && material has a diffuse layer */
#define SW_POLY_SHADOW 8u        /* material.shadow: casts shadows (materials_shadow_table, depth_renderer.rs:20-38) */

/* One world polygon of the map with the material fields its surface needs (bsp_map_compact::Polygon,
 * src/common/bsp_map_compact.rs:60-74, PolygonBasisVecs, src/square_wheel/surfaces.rs:7-47). */
typedef struct SwMapPolygon {
	float plane[4];                 /* vec.xyz, dist: points p of the plane have dot(vec, p) = dist */
	float tex_coord_equation[2][4]; /* tc_i(p) = dot(vec_i, p) + dist_i */
	float basis_u[3], basis_v[3], basis_start[3], basis_normal[3];
	int32_t tex_coord_min[2], tex_coord_max[2];
	uint32_t first_vertex, num_vertices; /* into sw_set_map's vertices */
	uint32_t texture;                    /* material texture: texture_mip = texture * 5 + mip */
	uint32_t lightmap_data_offset;
	uint32_t flags;                      /* SW_POLY_* */
	uint32_t blending_mode;              /* SwBlend of the material */
	uint32_t emissive_texture;           /* emissive_mip = emissive_texture * 5 + mip, or SW_NO_EMISSIVE */
	float emissive_light[3];
} SwMapPolygon;

/* Upload the world polygons and their vertices (xyz floats) for sw_draw_frame_view. Load-time data
 * like sw_create's; synchronous. */
int sw_set_map(SwCtx* ctx, const SwMapPolygon* polygons, uint32_t num_polygons, const float* vertices,
	uint32_t num_vertices);

/* One visible BSP leaf (MapVisibilityCalculator's leaf bounds, map_visibility_calculator.rs:157-267).
 * Clip planes are ClippingPolygon::get_clip_planes of the bounds (clipping_polygon.rs:140-152): 8 x
 * (a, b, c) with a*x + b*y >= c inside. */
typedef struct SwViewLeaf {
	uint32_t first_polygon, num_polygons; /* the leaf's polygons in SwMapPolygon order */
	uint32_t first_light, num_lights;     /* the leaf's lights (DynamicObjectsIndex order) in leaf_lights */
	uint32_t draw_order;                  /* position in draw_tree's back-to-front order, or SW_LEAF_NOT_DRAWN */
	uint32_t reserved;
	float clip_planes[8][3];              /* leaf bounds: surface preparation */
	float draw_clip_planes[8][3];         /* leaf bounds intersected with the viewport: draw_leaf */
} SwViewLeaf;
#define SW_LEAF_NOT_DRAWN 0xFFFFFFFFu

/* One material's state this frame (MapMaterialsProcessor, map_materials_processor.rs:174-247, 305-334):
 * the texture its polygons show (framed animation: textures_mapping_table's current frame; a generative
 * effect's output texture) and that frame's scrolling shift in texels of mip 0 (get_texture_shift), and
 * every other material property the renderer reads through the mapping table (get_material,
 * get_emissive_texture): the SW_POLY_* flags (draw, sky, diffuse layer, shadow) of the current frame's
 * material, its blending mode, and its emissive texture (SW_NO_EMISSIVE: none) with the light. These
 * replace the polygon's own (SwMapPolygon) for every polygon of the material. */
typedef struct SwMaterialFrame {
	int32_t shift[2];
	uint32_t texture; /* texture_mip = texture * 5 + mip */
	uint32_t flags;
	uint32_t blending_mode;
	uint32_t emissive_texture;
	float emissive_light[3];
	uint32_t reserved;
} SwMaterialFrame;

typedef struct SwViewFrameInput {
	SwFrameParams params;
	uint32_t num_lights;
	const SwLight* lights;
	float view_matrix[16];   /* CameraMatrices::view_matrix, column-major */
	float planes_matrix[16]; /* CameraMatrices::planes_matrix, column-major */
	float mip_bias;
	uint32_t num_leafs;       /* visible leafs in leaf index order */
	const SwViewLeaf* leafs;
	uint32_t num_leaf_lights;
	const uint16_t* leaf_lights;
	uint32_t num_draws;       /* draws before the leafs' (draw_skybox), in submission order */
	const SwDrawCmd* draws;
	const SwVertex16* vertices;
	uint32_t num_vertices;
	uint32_t postprocess;     /* as SwFrameInput */
	SwPostConfig post;
	float frame_duration_s;
	float color_modulate[3];
	void* dst;
	uint32_t dst_pitch;
	int32_t dst_is_device;
	/* animated materials, one SwMaterialFrame per material (SwMapPolygon.texture); materials at or past
	 * num_material_frames (or a NULL array) show their own texture unshifted */
	uint32_t num_material_frames;
	const struct SwMaterialFrame* material_frames;
} SwViewFrameInput;

/* One whole frame like sw_draw_frame, with the surfaces and the leafs' draws prepared on the GPU. */
int sw_draw_frame_view(SwCtx* ctx, const SwViewFrameInput* frame);

/* What the last sw_draw_frame_view prepared (diagnostics and tests; synchronises): the counts, and up
 * to the given capacities the surface descriptors, draw commands (the host's draws first) and vertices. */
typedef struct SwViewCounts {
	uint32_t num_surfaces, num_draws, num_vertices, error; /* error != 0: a capacity was exceeded */
	uint64_t total_texels, num_rows;
} SwViewCounts;
int sw_read_view_prep(SwCtx* ctx, SwViewCounts* out_counts, SwSurfaceDesc* surfaces, uint32_t max_surfaces,
	SwDrawCmd* draws, uint32_t max_draws, SwVertex16* vertices, uint32_t max_vertices);

/* ---- shadowed dynamic lights (cube shadow maps) ----
 * DynamicLightWithShadow with ShadowMap::Cube (src/square_wheel/light.rs:4-62): the renderer draws each
 * shadowed light's six depth maps (build_shadow_maps, partial_renderer.rs:525-592, DepthRenderer,
 * depth_renderer.rs, DepthRasterizer, rasterizer.rs:1295-1474) into one persistent f32 storage, and the
 * surface build multiplies the light's distance factor by cube_shadow_map_fetch (light.rs:196-258). */

#define SW_SHADOW_NONE 0u
#define SW_SHADOW_CUBE 1u
#define SW_SHADOW_PROJECTOR 2u /* ShadowMap::Projector (light.rs:53-60): one size x size map of a cone */

/* The shadow map of one of the frame's lights. */
typedef struct SwLightShadow {
	uint32_t kind;   /* SW_SHADOW_* */
	uint32_t size;   /* cube side size (or projector map size) in texels */
	uint64_t offset; /* cube: side s (light.rs:14-23 order: +X, -X, +Y, -Y, +Z, -Z) starts at offset + s * size * size;
	                  projector: the map */
	/* projector only (create_dynamic_light_projector_shadow_map, renderer_structs.rs:288-308): the
	 * light's rotated y and z axes scaled by 1/tan(fov/2), and its -x axis */
	float basis_x[3], basis_y[3], basis_z[3];
	uint32_t reserved;
} SwLightShadow;

/* One DepthRasterizer::fill_polygon call of DepthRenderer::draw_polygon (depth_renderer.rs:199-287):
 * the clipped polygon projected onto a cube side (f32_to_fixed16 vertices), its biased and scaled depth
 * equation, and the side it is drawn into. */
typedef struct SwDepthDraw {
	uint32_t first_vertex;   /* into the SwVertex16 array */
	uint32_t vertex_count;   /* 3..SW_MAX_POLYGON_VERTICES, clockwise */
	uint32_t map_size;       /* side width = height */
	uint32_t reserved;
	uint64_t map_offset;     /* the side's first texel in the shadow-map storage */
	float depth_eq[3];       /* d_inv_z_dx, d_inv_z_dy, k */
	uint32_t reserved2;
} SwDepthDraw;

/* Draw the depth draws, in array order, into the shadow-map storage (grown to total_texels f32 texels,
 * never cleared: a texel no polygon covers keeps its value, as the reference's storage does). Draws of
 * one side must be in the depth renderer's back-to-front order; the last draw covering a texel sets it. */
int sw_build_shadow_maps(SwCtx* ctx, const SwDepthDraw* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices, uint64_t total_texels);
/* Shadow maps of the next frame's lights (one per light, in the frame's SwLight order; num_lights 0 or a
 * NULL array = no shadows). Holds for the frames that follow until it is called again. Call it after the
 * frame's shadow-map builds: a projector map's corners outside its inscribed circle are then set to
 * 1e24 (make_shadow_map_circle, light.rs:135-156), after its depth draws. */
int sw_set_light_shadows(SwCtx* ctx, const SwLightShadow* shadows, uint32_t num_lights);
/* GPU-side depth-draw preparation (replaces the host's DepthRenderer::draw_polygon loop; needs sw_set_map):
 * one cube side as DepthRenderer::draw_map sees it (the side camera of light.rs:88-133) ... */
typedef struct SwShadowSide {
	float view_matrix[16];   /* CameraMatrices::view_matrix, column-major */
	float planes_matrix[16]; /* CameraMatrices::planes_matrix, column-major */
	uint32_t map_size;       /* side width = height, 1..SW_SHADOW_MAX_SIZE */
	uint32_t reserved;
	uint64_t map_offset;     /* the side's first texel in the shadow-map storage */
} SwShadowSide;
/* ... and one leaf that the side's visibility reaches, in DepthRenderer::draw_tree's back-to-front order
 * (depth_renderer.rs:96-136), sides one after another. */
typedef struct SwShadowLeaf {
	uint32_t side;                        /* index into the sides array */
	uint32_t first_polygon, num_polygons; /* the leaf's polygons in SwMapPolygon order */
	uint32_t reserved;
	float clip_planes[8][3];              /* the leaf's bounds in the side's visibility (clipping_polygon.rs:140-152) */
} SwShadowLeaf;
#define SW_SHADOW_MAX_SIZE 1024u
/* Prepare the depth draws of every listed leaf's polygons on the GPU (draw_polygon::<false> and
 * draw_depth_polygon, depth_renderer.rs:199-287: shadow-casting opaque polygons facing the light, the
 * biased depth equation, project_and_clip_polygon, f32_to_fixed16) and draw them as sw_build_shadow_maps
 * draws the same list prepared on the host: the same storage, texel for texel. */
int sw_build_shadow_maps_view(SwCtx* ctx, const SwShadowSide* sides, uint32_t num_sides, const SwShadowLeaf* leafs,
	uint32_t num_leafs, uint64_t total_texels);
/* Diagnostics: copy up to max_texels texels of the shadow-map storage to host memory (synchronises). */
int sw_read_shadow_maps(SwCtx* ctx, float* dst, uint64_t max_texels);

/* ---- launch configuration (no reference counterpart) ---- */
#define SW_RASTER_TILE_VARIANTS 5
typedef struct SwTuning {
	/* tile shape of the tile pass, 256 threads each: 0 = 64x16 pixels (4-pixel strips), 1 = 32x32 (4),
	 * 2 = 128x8 (4), 3 = 64x32 (8-pixel strips), 4 = 32x16 (2-pixel strips); all give the same frame */
	uint32_t raster_tile;
	/* persistent grid of the surface build: blocks per SM, 1..64 */
	uint32_t surface_blocks_per_sm;
	/* texels per surface-build thread: 1, or 4 consecutive texels sharing their lightmap line entries
	 * (0 = the default, 1) */
	uint32_t surface_texels_per_thread;
	uint32_t reserved;
} SwTuning;
int sw_set_tuning(SwCtx* ctx, const SwTuning* tuning);
int sw_get_tuning(SwCtx* ctx, SwTuning* out_tuning);
/* Autotuner: times `reps` replays of the sample frame (sw_draw_frame) for every raster tile shape and a
 * set of surface grid sizes (texels per surface thread kept as set), keeps the fastest configuration in
 * the context and returns it with its median device time per frame in ms. The exposure state is
 * restored afterwards. */
int sw_autotune(SwCtx* ctx, const SwFrameInput* sample, uint32_t reps, SwTuning* out_best, float* out_best_ms);

/* sizeof() of the ABI structs in this order: SwCreateInfo, SwTextureMip, SwEmissiveMip,
 * SwDirectionalLightmapElement, SwLight, SwSurfaceDesc, SwVertex16, SwDrawCmd, SwFrameParams,
 * SwPostConfig, SwStats, SwFrameInput, SwTuning, SwMapPolygon, SwViewLeaf, SwViewFrameInput,
 * SwViewCounts, SwLightShadow, SwDepthDraw, SwShadowSide, SwShadowLeaf, SwMaterialFrame, SwTriVertex.
 * Writes min(count, 23) values; returns the number of structs (23). Needs no GPU: bindings use it to
 * check their mirrored layouts. */
int sw_abi_layout(uint32_t* sizes, uint32_t count);

/* Diagnostics: copy the frame's surface arena (total_texels of sw_submit_surfaces, or of the surfaces a
 * sw_draw_frame_view prepared) to host memory (synchronises). */
int sw_read_surfaces(SwCtx* ctx, void* dst_host, uint64_t max_bytes);
/* Diagnostics: copy the context's frame buffer (the last frame rasterised, width x height pixels of its
 * pixel format, tightly packed; the HDR frame the postprocessor read) to host memory (synchronises). */
int sw_read_framebuffer(SwCtx* ctx, void* dst_host, uint64_t max_bytes);
/* Diagnostics: copy the context's material texels and emissive pixels (as texture effect passes left them)
 * to host memory (synchronises). */
int sw_read_texels(SwCtx* ctx, uint64_t* texels, uint64_t max_texels, uint32_t* emissive, uint64_t max_emissive);
/* Diagnostics: copy the context's decoded lightmaps (up to max_elements simple and max_directional_elements
 * directional elements) to host memory (synchronises). */
int sw_read_lightmaps(SwCtx* ctx, float* lightmaps, uint64_t max_elements, SwDirectionalLightmapElement* directional,
	uint64_t max_directional_elements);
/* Current exposure (Postprocessor::current_exposure). */
int sw_get_exposure(SwCtx* ctx, float* out_exposure);
int sw_set_exposure(SwCtx* ctx, float exposure);

#ifdef __cplusplus
}
#endif

#endif /* SWGPU_H */
