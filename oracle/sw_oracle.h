// Test infrastructure: C ABI of the CPU oracle for the GB300 rendering path.
//
// The oracle restates the reference's CPU renderer for the hot path (surface building, polygon
// rasterisation, HDR postprocessing, frame upscaling) in plain C++. Only the tests, the smoke check
// and the CPU-baseline leg of bench.py load it; the product never does. It consumes the same
// descriptors as the GPU library (include/swgpu.h), so both sides see identical inputs.
#pragma once

#include "../include/swgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* build_polygons_surfaces' per-polygon work (partial_renderer.rs:1682-1831): builds every surface of
 * `surfaces` into `arena` (pixel_format texels). num_threads 0/1 = sequential, N = N worker threads
 * with one task per surface (the reference's rayon par_iter). Returns 0 or a negative SwStatus. */
int orc_build_surfaces(const SwCreateInfo* data, const SwSurfaceDesc* surfaces, uint32_t num_surfaces,
	const SwLight* lights, uint32_t num_lights, const SwLightShadow* shadows, const float* shadow_texels,
	uint64_t shadow_texel_count, const SwFrameParams* frame, void* arena, uint64_t arena_texels, uint32_t num_threads);
/* (shadows: NULL, or one SwLightShadow per light with the cube maps in shadow_texels) */

/* DepthRasterizer::fill_polygon for every depth draw in order (DepthRenderer, depth_renderer.rs;
 * rasterizer.rs:1295-1474) into `storage` (f32 texels; draws overwrite, nothing is cleared). */
int orc_shadow_maps(const SwDepthDraw* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	float* storage, uint64_t total_texels);

/* make_shadow_map_circle (light.rs:135-156) on the projector map at `offset` (size x size texels). */
int orc_shadow_map_circle(float* storage, uint64_t total_texels, uint64_t offset, uint32_t size);

/* Rasterizer::fill_polygon for every draw in order (perform_rasterization, partial_renderer.rs:1192-1283)
 * into `framebuffer` (pixel_format of frame, pitch in pixels). num_threads 0/1 = the reference's
 * single-thread path (one full-screen ClipRect); N > 1 = split_rect into N regions with one ClipRect each.
 * Draws with tex_source SW_TEXSRC_SKYBOX read `skybox` (the frame's pixel format) instead of `arena`.
 * Out-of-range texel fetches (impossible for well-formed draws) read texel 0 and are counted in
 * *bad_fetches when the pointer is non-null. */
int orc_rasterize(const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	const void* arena, uint64_t arena_texels, const void* skybox, uint64_t skybox_texels, const SwFrameParams* frame,
	void* framebuffer, uint32_t pitch, uint32_t num_threads, uint64_t* bad_fetches);

/* orc_rasterize with triangle draws (SW_RASTER_TRIANGLE, Rasterizer::fill_triangle, rasterizer.rs:731-1292):
 * their vertices are in tri_vertices and their Color32 textures in `lite`. */
int orc_rasterize_ex(const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	const SwTriVertex* tri_vertices, uint32_t num_tri_vertices, const void* arena, uint64_t arena_texels,
	const void* skybox, uint64_t skybox_texels, const uint32_t* lite, uint64_t lite_texels, const SwFrameParams* frame,
	void* framebuffer, uint32_t pitch, uint32_t num_threads, uint64_t* bad_fetches);

/* draw_background, partial_renderer.rs:3987-4009, colour (32,16,8) via ColorVec. */
int orc_clear_background(const SwFrameParams* frame, void* framebuffer, uint32_t pitch);

/* Postprocessor::perform_postprocessing (postprocessor.rs:68-204) single-threaded: reads the HDR
 * Color64 frame (width*height, tightly packed), writes Color32 to dst (pitch in pixels) and updates
 * *exposure in place. If average_color is non-null it receives the frame's average colour (4 lanes). */
int orc_postprocess(const SwPostConfig* config, const uint64_t* hdr, uint32_t width, uint32_t height,
	float frame_duration_s, const float color_modulate[3], float* exposure, uint32_t* dst, uint32_t pitch,
	float* average_color);

/* FrameUpscaler::perform_upscale (frame_upscaler.rs:42-239). */
int orc_upscale(uint32_t mode, uint32_t scale, const uint32_t* src, uint32_t* dst, uint32_t dst_width,
	uint32_t dst_height, uint32_t dst_pitch);

/* Generative texture effects: make_turb_distortion's shift table (generative_texture_effect_turb.rs:100-113)
 * into `buffer` (persisting between calls like the effect's temp_buffer: entries below w rewritten), and
 * the passes of sw_update_textures applied in order to the texel and emissive arrays (turbulence gathers,
 * apply_texture_layer of generative_texture_effect_layered.rs:163-381). */
int orc_turb_shifts(float amplitude, float wave_length, float frequency, float time_s, uint32_t w, uint32_t h, uint32_t mip,
	int32_t* buffer, uint32_t buffer_len);
int orc_apply_texture_passes(const SwTexturePass* passes, uint32_t num_passes, const int32_t* shifts, uint32_t num_shifts,
	const SwTextureMip* mips, uint32_t num_mips, uint64_t* texels, const SwEmissiveMip* emissive_mips,
	uint32_t num_emissive_mips, uint32_t* emissive);

/* Lossy lightmap compression (src/common/lightmap_compression.rs:48-130): simple elements as 4-byte
 * CompressedColor records, directional elements as 13-byte records. */
int orc_compress_lightmaps(const float* rgb, uint64_t n, uint8_t* out);
int orc_decompress_lightmaps(const uint8_t* in, uint64_t n, float* rgb);
int orc_compress_directional_lightmaps(const SwDirectionalLightmapElement* in, uint64_t n, uint8_t* out);
int orc_decompress_directional_lightmaps(const uint8_t* in, uint64_t n, SwDirectionalLightmapElement* out);

/* compute_gaussian_kernel (postprocessor.rs:1026-1045) and the integer blur weights of
 * perform_blur_impl (postprocessor.rs:848-907); exported for known-answer tests. */
int orc_gaussian_kernel(float sigma, uint32_t radius, float* out33);

/* Simulated texture effects (generative_texture_effect_water.rs, generative_texture_effect_fire.rs), whole
 * on the CPU. The effect description: kind 3 water, 4 fire; a time function is SingleArgumentFunction
 * (kind 0 constant a, 1 linear a x + b, 2 sine, 3 triangle, 4 saw-tooth, 5 step: frequency a, phase b,
 * amplitude c, offset d), a random value is ValueWithRandomDeviation. */
typedef struct OrcTimeFunction {
	uint32_t kind;
	float a, b, c, d;
} OrcTimeFunction;
typedef struct OrcRandomValue {
	OrcTimeFunction value, deviation;
} OrcRandomValue;
typedef struct OrcSimSource {
	uint32_t kind; /* water: WavySpot, WavyLine, PeriodicDroplet, Rain; fire: Point, Line, Lightning, Fountain */
	uint32_t points[2][2];
	OrcTimeFunction offsets[2][2];
	float frequency, phase, amplitude, offset, radius;
	uint32_t ramp;
	OrcRandomValue fire_offsets[2][2];
	OrcRandomValue heat, angle, speed, gravity, spawn_angle, spawn_distance, lifetime;
} OrcSimSource;
#define ORC_MAX_SIM_SOURCES 8
typedef struct OrcSimEffect {
	uint32_t kind;
	uint32_t resolution_log2[2];
	float update_frequency;
	float attenuation_param; /* fluidity (water), heat_conductivity (fire) */
	uint32_t color_mode, slow, has_color;
	float color[3];
	float roughness;
	int32_t output_texture, output_emissive, source_emissive;
	uint32_t num_sources;
	uint64_t state_offset;
	OrcSimSource sources[ORC_MAX_SIM_SOURCES];
} OrcSimEffect;
uint32_t orc_sim_effect_size(void);
void* orc_sim_create(const OrcSimEffect* effect); /* runs the constructor's equilibrium steps; NULL if malformed */
void orc_sim_destroy(void* sim);
int orc_sim_update(void* sim, float current_time_s, const SwTextureMip* mips, uint32_t num_mips, uint64_t* texels,
	const SwEmissiveMip* emissive_mips, uint32_t num_emissive_mips, uint32_t* emissive, uint32_t source_texture);
int orc_sim_state(void* sim, uint32_t* out_words, uint64_t max_words, uint32_t* out_update_step, uint32_t* out_generated,
	uint32_t* out_particles);
void orc_xoshiro_outputs(const uint64_t state[4], uint64_t* out, uint32_t n);

/* A portal view's texture mix (partial_renderer.rs:2189-2280) over its rendered region. */
int orc_mix_view(const SwView* view, void* region, uint32_t pixel_format, const uint32_t* lite, uint64_t lite_pixels);
void orc_small_rng_state(uint64_t seed, uint64_t out_state[4]);

#ifdef __cplusplus
}
#endif
