// Kernel argument blocks and launch entry points of the GB300 rendering path.
#pragma once

#include "sw_device.cuh"

#include <algorithm>
#include <cmath>

namespace swgpu
{

// Per-surface record the surface kernel reads (built on the host from SwSurfaceDesc and the texture
// tables). Everything that is constant over a surface is evaluated once here, with the same IEEE f32
// operations and order as the reference's per-surface prologue (surfaces.rs:453-471), so the per-texel
// work in the kernel is only the reference's inner loop.
struct __align__(16) SurfaceGpu
{
	float start_pos[3]; // basis.start + u*(tc0 + 0.5) + v*(tc1 + 0.5)
	float u[3];
	float v[3];
	float normal[3];
	float u_norm[3];    // u * inv_sqrt_fast(max(|u|^2, MIN_POSITIVE_VALUE))
	float v_norm[3];
	float inv_scale;    // 1 / (1 << lightmap_scale_log2)
	float k_shift;      // 0.5 * inv_scale
	uint64_t tex_offset;
	uint32_t width;     // surface width in texels
	uint32_t tex_w, tex_h;
	uint32_t flags;     // SW_TEX_* in bits 0..2, SW_SURF_DIFFUSE_LAYER << 8, has lightmap << 9, emissive << 10
	int32_t tc0, tc1;
	uint32_t lm_offset, lm_width, lm_log2, lm_shift0, lm_shift1;
	uint32_t num_lights;
	uint16_t lights[SW_MAX_POLYGON_LIGHTS];
	uint64_t em_offset;
	uint32_t em_w, em_h;
	int32_t em_light[3]; // ColorVecI lanes [b, g, r] of the emissive light * 256 (truncated)
	uint64_t out_offset;
	// size - 1 of the texture (tex_mask) and emissive (em_mask) sides that are powers of two, whose
	// rem_euclid is then a mask; ~0u for other sizes
	uint32_t tex_mask[2], em_mask[2];
	float inv_width; // 1 / width: the row of a texel index by a float estimate and an exact correction
	uint32_t reserved;
};

#define SW_SG_DIFFUSE (1u << 8)
#define SW_SG_LIGHTMAP (1u << 9)
#define SW_SG_EMISSIVE (1u << 10)

struct SurfaceKernelArgs
{
	const SurfaceGpu* surfaces;
	const uint64_t* work_prefix; // num_surfaces + 1 entries, texel prefix sums in descriptor order
	uint32_t num_surfaces;
	uint32_t directional;
	uint64_t total_work;
	uint64_t work_begin; // first texel of the launch (0: all of [0, total_work)); one surface's range for per-surface launches
	const SwViewCounts* counts; // GPU-side preparation: num_surfaces / total_work from here (else NULL)
	const SwLightShadow* shadows; // per light (NULL: no shadows), maps in shadow_texels
	const unsigned long long* shadow_texels; // (sequence << 32 | f32 bits) per texel
	uint32_t num_shadows;
	const uint64_t* texels;
	const uint32_t* emissive_pixels;
	const float* lightmaps;
	const SwDirectionalLightmapElement* directional_lightmaps;
	const SwLight* lights;
	float cam_pos[3];
	const float* cam_pos_dev; // when set, the camera position is read here (a replayed frame graph)
	void* arena;
};

// f32 -> i32 `as` conversion: truncating, saturating, NaN -> 0.
__host__ __device__ inline int32_t f2i32_as(float x)
{
	if (x != x) return 0;
	if (x >= 2147483648.0f) return INT32_MAX;
	if (x <= -2147483648.0f) return INT32_MIN;
	return int32_t(x);
}

// One SurfaceGpu from its descriptor and texture tables (exact f32 arithmetic without FMA contraction;
// the host's sw_submit_surfaces and the GPU-side preparation both use it).
__host__ __device__ inline void make_surface_gpu(const SwSurfaceDesc& d, const SwTextureMip* tex, const SwEmissiveMip* em,
	SurfaceGpu& o)
{
	// surfaces.rs:456-462: start + u*(tc0+0.5) + v*(tc1+0.5); normalised basis vectors.
	const float a0 = float(d.tc_start[0]) + 0.5f, a1 = float(d.tc_start[1]) + 0.5f;
	for (int i = 0; i < 3; ++i)
	{
		o.start_pos[i] = (d.basis_start[i] + d.basis_u[i] * a0) + d.basis_v[i] * a1;
		o.u[i] = d.basis_u[i];
		o.v[i] = d.basis_v[i];
		o.normal[i] = d.basis_normal[i];
	}
	const float uu = d.basis_u[0] * d.basis_u[0] + (d.basis_u[1] * d.basis_u[1] + d.basis_u[2] * d.basis_u[2]);
	const float vv = d.basis_v[0] * d.basis_v[0] + (d.basis_v[1] * d.basis_v[1] + d.basis_v[2] * d.basis_v[2]);
	const float iu = 1.0f / sqrtf(fmaxf(uu, MIN_POSITIVE_VALUE));
	const float iv = 1.0f / sqrtf(fmaxf(vv, MIN_POSITIVE_VALUE));
	for (int i = 0; i < 3; ++i)
	{
		o.u_norm[i] = d.basis_u[i] * iu;
		o.v_norm[i] = d.basis_v[i] * iv;
	}
	const bool has_lm = d.lightmap_offset != SW_NO_LIGHTMAP;
	const uint32_t log2 = has_lm ? d.lightmap_scale_log2 : 0u;
	o.inv_scale = 1.0f / float(1u << log2);
	o.k_shift = 0.5f * o.inv_scale;
	o.width = d.size[0];
	o.flags = 0;
	if (d.flags & SW_SURF_DIFFUSE_LAYER)
	{
		o.tex_offset = tex->offset;
		o.tex_w = tex->width;
		o.tex_h = tex->height;
		o.flags |= (tex->flags & 7u) | SW_SG_DIFFUSE;
	}
	else
	{
		o.tex_offset = 0;
		o.tex_w = o.tex_h = 1;
	}
	if (has_lm) o.flags |= SW_SG_LIGHTMAP;
	o.tc0 = d.tc_start[0];
	o.tc1 = d.tc_start[1];
	o.lm_offset = d.lightmap_offset;
	o.lm_width = d.lightmap_size[0];
	o.lm_log2 = log2;
	o.lm_shift0 = d.lightmap_tc_shift[0];
	o.lm_shift1 = d.lightmap_tc_shift[1];
	o.num_lights = d.num_lights;
	for (int i = 0; i < SW_MAX_POLYGON_LIGHTS; ++i) o.lights[i] = d.lights[i];
	if (em)
	{
		o.flags |= SW_SG_EMISSIVE;
		o.em_offset = em->offset;
		o.em_w = em->width;
		o.em_h = em->height;
		// ColorVecI::from_color_f32x3([l0*256, l1*256, l2*256]) -> lanes [b, g, r] (surfaces.rs:911-914)
		o.em_light[0] = f2i32_as(d.emissive_light[2] * 256.0f);
		o.em_light[1] = f2i32_as(d.emissive_light[1] * 256.0f);
		o.em_light[2] = f2i32_as(d.emissive_light[0] * 256.0f);
	}
	else
	{
		o.em_offset = 0;
		o.em_w = o.em_h = 1;
		o.em_light[0] = o.em_light[1] = o.em_light[2] = 0;
	}
	o.out_offset = d.out_offset;
	auto pow2_mask = [](uint32_t n) { return (n != 0 && (n & (n - 1)) == 0) ? n - 1 : ~0u; };
	o.tex_mask[0] = pow2_mask(o.tex_w);
	o.tex_mask[1] = pow2_mask(o.tex_h);
	o.em_mask[0] = pow2_mask(o.em_w);
	o.em_mask[1] = pow2_mask(o.em_h);
	o.inv_width = 1.0f / float(d.size[0] ? d.size[0] : 1u);
	o.reserved = 0;
}

// Grid of at most num_sms * blocks_per_sm blocks of 256 threads that stride over the texels. With
// args.counts set the texel count is on the device: work_hint (an estimate) sizes the grid instead.
int launch_surface_build(const SurfaceKernelArgs& args, uint32_t pixel_format, int num_sms, int blocks_per_sm, cudaStream_t stream,
	uint64_t work_hint = 0, uint32_t texels_per_thread = 0);

// ---- rasteriser ----

// One polygon part of the edge walk (a draw_func call of fill_polygon_impl_2_static_params,
// src/square_wheel/rasterizer.rs:198-254), reduced to what a row needs to find its span.
struct RasterPart
{
	int32_t y_start_int; // first row, clipped to the frame
	int32_t y_end_int;   // one past the last row, clipped
	int32_t x_left0;     // x_left at row y_start_int (includes the +0.5 bias), 16.16
	int32_t x_right0;
	int32_t dx_dy_left;
	int32_t dx_dy_right;
	// Affine mode only (rasterizer.rs:616-682): per-edge texture coordinates at row y_start_int and
	// their per-row steps, 16.16.
	int32_t tc_left0[2];
	int32_t tc_right0[2];
	int32_t d_tc_left[2];
	int32_t d_tc_right[2];
	// Triangle parts (fill_triangle_part, rasterizer.rs:984-1292), after the reference's corrections:
	// the left edge's texture coordinates (tc_left0, per row d_tc_left) and light at row y_start_int and
	// their per-row steps, and the per-pixel steps d_tc_right (d_tc_dx) and d_light_dx; 16.16.
	int32_t light_left0[3];
	int32_t d_light_left[3];
	int32_t d_light_dx[3];
};

#define SW_RASTER_MAX_PARTS SW_MAX_POLYGON_VERTICES

// Rows a draw can cover, computed on the host from its vertices: [y0, y0 + nrows) contains every
// part's rows; row records of the draw start at row_base.
struct DrawRows
{
	uint32_t row_base;
	int32_t y0;
	uint32_t nrows;
	uint32_t reserved;
};

// One row of one draw after span setup (rasterizer.rs:329-422 / 513-556 / 686-703): the span
// [xs, xe) and, for pixel i = x - xs, the interpolants start + i * step of the draw's mode:
//   full perspective: (a0, b0) span inv_z, (a1, b1) and (a2, b2) span tc (i32, wrapping)
//   line-z corrected / affine: (a1, b1) and (a2, b2) the 16.16 texture coordinates.
//   triangle (rasterizer.rs:1188-1212): a0, b0 the first pixel's texture coordinates, a1, b1, a2 its
//   light (r, g, b), b2 the TriSteps index (draw * 2 + part) of the per-pixel steps.
// xs >= xe: the row holds no pixel.
struct RasterRow
{
	int32_t xs, xe;
	int32_t a0, b0, a1, b1, a2, b2;
};

// Per-pixel steps of one part of a triangle draw (fill_triangle_part's d_tc_dx and d_light_dx after
// its corrections, rasterizer.rs:1017-1186); the part's row records hold the row's first pixel's values.
struct TriSteps
{
	int32_t d_tc_dx[2];
	int32_t d_light_dx[3];
	int32_t reserved;
};

// Per-draw record of the tile kernel.
struct RasterDraw
{
	uint64_t tex_offset;
	uint32_t tex_w, tex_h;
	uint32_t row_base;
	int32_t y0;
	uint32_t mode;
	uint16_t blend, tex_source; // SwBlend, SwTexSource
};

// Pixel bounds of a draw: [x0, x1) x [y0, y1); empty when x0 >= x1 or y0 >= y1.
struct RasterBox
{
	int16_t x0, y0, x1, y1;
};

struct RasterArgs
{
	const SwDrawCmd* draws;
	const SwVertex16* vertices;
	const SwTriVertex* tri_vertices; // SW_RASTER_TRIANGLE draws' vertices
	const uint32_t* lite;            // Color32 textures of SW_TEXSRC_LITE draws
	uint64_t lite_texels;
	const DrawRows* draw_rows;
	uint32_t num_draws;
	const SwViewCounts* counts; // GPU-side preparation: num_draws from here (else NULL)
	uint32_t setup_blocks;      // with counts: raster setup CTAs, each striding over the draws
	uint32_t total_rows; // row records of all draws
	int32_t width, height;
	uint32_t clear_background;
	TriSteps* tri_steps;   // num_draws * 2: per-pixel steps of a triangle draw's two parts
	RasterDraw* rdraws;
	RasterRow* rows;
	RasterBox* boxes;
	const void* arena;
	uint64_t arena_texels;
	const void* skybox; // skybox texels of the frame's pixel format (SW_TEXSRC_SKYBOX draws)
	void* framebuffer;  // width * height pixels, tightly packed
	unsigned int* error_counter;
	// Bloom downscale fused into the tile pass (colour64 frames of a whole-frame graph): with
	// bloom_scale S != 0 each tile box-averages its final pixels into the bloom buffer (bloom_w x
	// bloom_h cells, downscale_hdr_buffer, postprocessor.rs:792-844) and adds its part of every bloom
	// line's exact integer lane sums to bloom_line_sums (zeroed before the pass).
	uint64_t* bloom_out;
	int32_t* bloom_line_sums;
	uint32_t bloom_scale, bloom_w, bloom_h;
	// Bins (raster_bin_kernel): the frame cut into RASTER_BIN_W x RASTER_BIN_H rectangles, each with the
	// draws whose box meets it in draw order (bin_lists[bin * bin_cap + i], bin_counts[bin] of them); a
	// tile scans its bin's list instead of every draw. NULL lists: every tile scans every draw.
	uint32_t* bin_lists;
	uint32_t* bin_counts;
	uint32_t bin_cap, bins_x, bins_y;
};

// Every tile shape divides the bin, so a tile lies in one bin.
constexpr int32_t RASTER_BIN_W = 128, RASTER_BIN_H = 64;
inline uint32_t raster_bins(int32_t extent, int32_t bin) { return uint32_t((extent + bin - 1) / bin); }

// Edge walk + row setup (raster_setup, one CTA per draw), the bins (raster_bins, one CTA per bin), then
// the tile pass (raster_tiles).
int launch_raster_setup(const RasterArgs& args, cudaStream_t stream);
// mix_surface_with_texture over a nested view's rendered region (surfaces.rs:854-971)
int launch_view_mix(const SwView& view, void* target, const uint32_t* lite, uint32_t pixel_format, cudaStream_t stream);
int launch_raster_bins(const RasterArgs& args, cudaStream_t stream);
// variant: tile shape index (< SW_RASTER_TILE_VARIANTS, see SwTuning); every variant gives the same frame.
int launch_raster_tiles(const RasterArgs& args, uint32_t pixel_format, uint32_t variant, cudaStream_t stream);

// Rows [y0, y0 + nrows) a draw can cover: [round(min_y), round(max_y)) of its vertices clipped to the
// frame (the edge walk's parts lie inside, rasterizer.rs:160-271 with fixed16_round_to_int; a triangle's
// two parts span its lowest to its highest vertex, :984-1004). Triangle draws take their vertices from tv.
__host__ __device__ inline void draw_row_range(const SwDrawCmd& d, const SwVertex16* v, int32_t height, int32_t& y0,
	uint32_t& nrows, const SwTriVertex* tv = nullptr)
{
	const bool tri = d.mode == SW_RASTER_TRIANGLE;
	auto vy = [&](uint32_t i) { return tri ? tv[d.first_vertex + i].y : v[d.first_vertex + i].y; };
	int32_t mn = vy(0), mx = mn;
	for (uint32_t i = 1; i < d.vertex_count; ++i)
	{
		const int32_t y = vy(i);
		mn = y < mn ? y : mn;
		mx = y > mx ? y : mx;
	}
	const int32_t a0 = int32_t(uint32_t(mn) + 0x8000u) >> 16; // + half, 16.16
	const int32_t b0 = int32_t(uint32_t(mx) + 0x8000u) >> 16;
	const int32_t a = a0 > 0 ? a0 : 0;
	const int32_t b = b0 < height ? b0 : height;
	y0 = a;
	nrows = b > a ? uint32_t(b - a) : 0u;
}

// ---- shadow maps ----


struct ShadowArgs
{
	const SwDepthDraw* draws;
	uint32_t num_draws;
	uint32_t seq_base;               // draw i writes sequence seq_base + i + 1 (< 2^32)
	const SwVertex16* vertices;
	unsigned long long* storage;     // the persistent storage: (sequence << 32 | f32 bits) per texel
};
// Draw every depth draw into the storage (last draw wins per texel).
int launch_shadow_maps(const ShadowArgs& args, cudaStream_t stream);

// GPU-side depth-draw preparation and drawing (sw_build_shadow_maps_view): candidate c is the c-th
// polygon of the listed leafs, drawn with sequence seq_base + c + 1.
struct ShadowViewArgs
{
	const SwShadowSide* sides;
	const SwShadowLeaf* leafs;
	const uint32_t* leaf_base; // first candidate of each leaf (exclusive prefix sum of num_polygons)
	uint32_t num_leafs, num_candidates;
	const SwMapPolygon* polygons;
	const float* map_vertices;
	unsigned long long* storage;
	uint32_t seq_base;
};
int launch_shadow_view(const ShadowViewArgs& args, cudaStream_t stream);
// make_shadow_map_circle on the size x size projector map at `map` with sequence `seq`.
int launch_shadow_circle(unsigned long long* map, uint32_t size, uint32_t seq, cudaStream_t stream);
// sw_update_textures (effects.cu): one group per output mip - a turbulence gather, or layers applied in
// order. Groups are in texel order (first_texel ascending).
struct TextureEffectGroup
{
	uint64_t first_texel;         // of the launch's flat texel space
	uint64_t dst_offset, src_offset; // texel (or emissive pixel) offsets; src for turbulence only
	uint32_t width, height;       // of the output mip
	uint32_t first_pass, num_passes;
};
struct TextureEffectLayer // per pass (LAYER passes only)
{
	uint64_t src_offset;
	uint32_t src_width, src_height;
	uint32_t modulate, skip;
	int32_t light[3]; // ColorVecI lanes b, g, r of light * 256
	uint32_t reserved;
};
struct TextureEffectArgs
{
	const TextureEffectGroup* groups;
	const TextureEffectLayer* layers;
	const SwTexturePass* passes;
	const int32_t* shifts;
	uint32_t num_groups;
	uint64_t total_texels;
	uint64_t* texels;
	uint32_t* emissive;
};
int launch_texture_effects(const TextureEffectArgs& a, cudaStream_t stream);
// sw_update_simulations (sims.cu): one group per pass of a launch, groups in item order (first_item
// ascending); an item is a point (POINTS), a word (STEP, TEXTURE), a row (slow FIRE_STEP) or a texel of
// the destination mip (MIP passes).
struct SimGroup
{
	uint64_t first_item;
	uint64_t dst_offset, src_offset; // TEXTURE / MIP passes: texel (emissive pixel) offsets of dst and src mips
	uint32_t pass;
	uint32_t src_width, src_height;  // WATER_TEXTURE: colour source mip; MIP passes: the source mip
	uint32_t reserved;
};
struct SimArgs
{
	const SimGroup* groups;
	const SwSimPass* passes;
	const SwSimPoint* points;
	uint32_t num_groups;
	uint64_t total_items;
	uint32_t* state;
	uint64_t* texels;
	uint32_t* emissive;
};
int launch_simulation(const SimArgs& a, cudaStream_t stream);

// Compressed lightmap lumps (4-byte simple, 13-byte directional elements, 16-byte aligned inputs) decoded
// into f32 lightmaps (lightmaps.cu).
int launch_lightmap_decompress(const void* simple_in, uint64_t num_simple, float* simple_out, const void* dir_in,
	uint64_t num_dir, SwDirectionalLightmapElement* dir_out, cudaStream_t stream);
// Sequences restart at 0: keep only the f32 bits of every texel.
int launch_shadow_rebase(unsigned long long* storage, uint64_t num_texels, cudaStream_t stream);

// ---- GPU-side surface and draw preparation (prep.cu) ----

// Per candidate polygon (every polygon of the visible leafs, in leaf index order): the surface
// descriptor and draw of prepare_polygon_surface / build_polygons_surfaces / draw_polygon, before
// compaction (out_offset, first_vertex and tex_offset are filled by the compaction).
struct PrepCand
{
	SurfaceGpu sgpu; // the surface build's record, out_offset 0
	SwSurfaceDesc desc;
	SwDrawCmd draw;
	uint64_t surface_offset;
	SwVertex16 v[SW_MAX_POLYGON_VERTICES];
};
// What the compaction scans, one compact record per candidate.
struct PrepKey
{
	uint64_t area;       // surface texels
	uint32_t state;      // 1: the polygon has a surface
	uint32_t draw_count; // vertices of its draw (0: not drawn)
	uint32_t row_n;      // rows of its draw, from row_y0
	int32_t row_y0;
};

// The per-frame values of the preparation, uploaded with the frame (a replayed graph's kernel
// arguments do not change between frames).
struct PrepFrame
{
	float view[16], planes[16]; // column-major
	float mip_bias;
	uint32_t num_leafs;
	uint32_t num_candidates;
	uint32_t num_draw_leafs;
	uint32_t num_host_draws, num_host_vertices;
	uint64_t num_host_rows;
	uint32_t num_material_frames; // materials with an entry in PrepArgs::material_frames
};

struct PrepArgs
{
	const PrepFrame* frame;
	const SwMaterialFrame* material_frames; // frame->num_material_frames of them
	const SwMapPolygon* polygons;
	const float* map_vertices; // xyz
	const SwViewLeaf* leafs;
	const uint32_t* leaf_cand_base; // num_leafs + 1: first candidate of each leaf
	const uint16_t* leaf_lights;
	const SwLight* lights;
	const uint32_t* draw_leaf;      // draw order -> leaf
	const uint32_t* draw_slot_base; // num_draw_leafs + 1: first draw slot of each drawn leaf
	uint32_t directional, simple_lightmaps;
	int32_t height;
	// draws prepared on the host (skybox), placed first
	const SwDrawCmd* host_draws;
	const SwVertex16* host_vertices;
	const DrawRows* host_rows;
	const SwTextureMip* texture_mips;
	const SwEmissiveMip* emissive_mips;
	const SwLightShadow* shadows; // the frame's lights' shadow maps (projector cones narrow the light lists)
	uint32_t num_shadows;
	PrepCand* cands;
	PrepKey* keys;
	// outputs and their capacities
	SwSurfaceDesc* descs;
	SurfaceGpu* surfaces;
	uint64_t* work_prefix; // cap_surfaces + 1
	SwDrawCmd* draws;
	SwVertex16* vertices;
	DrawRows* draw_rows;
	SwViewCounts* counts;
	uint32_t cap_candidates, cap_surfaces, cap_draws, cap_vertices;
	uint64_t cap_texels, cap_rows;
};

// Per-candidate preparation on `stream` (a grid for cap_candidates polygons; CTAs beyond the frame's
// candidates return at once), then the surface compaction on `stream` and the draw compaction on `aux`
// (after `candidates_done`, recorded here); the caller orders the raster setup after the draw compaction.
int launch_prep(const PrepArgs& args, cudaStream_t stream, cudaStream_t aux, cudaEvent_t candidates_done);

// ---- postprocessor / upscaler ----

struct PostArgs
{
	const uint64_t* hdr;
	uint32_t width, height;
	uint32_t scale; // bloom buffer scale S (2, 4 or 8)
	uint32_t bw, bh;
	uint64_t* bloom0;
	uint64_t* bloom1;
	int32_t* line_sums; // bh * 4 lanes (bloom) or unused
	float* line_sums_f; // height * 4 lanes (no bloom)
	float* average;     // 4 lanes
	uint32_t radius;
	int32_t kernel_h[33];
	int32_t kernel_v[33];
	float inv_scale[4]; // TonemappingFunction::inv_scale_vec lanes
	const float* inv_scale_dev; // when set, the four lanes are read here (a replayed frame graph)
	float inv_255[4];
	uint32_t linear_filter;
	uint32_t use_bloom;
	uint32_t downscaled; // bloom0 and line_sums were written by the raster tile pass (RasterArgs::bloom_*)
	uint32_t* dst;
	uint32_t dst_pitch;
};

// aux/fork/join (optional): run the exposure-average reduction on `aux`, joined back before returning.
// average_done (optional) is recorded as soon as the average is written (an external event record node
// when the launch is being captured).
int launch_postprocess(const PostArgs& args, int num_sms, cudaStream_t stream, cudaStream_t aux = nullptr,
	cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr, cudaEvent_t average_done = nullptr);

// PostprocessorConfig as Postprocessor::synchronize_config leaves it (postprocessor.rs:958-977), which
// the host calls before every frame: every field clamped to its range. fmax/fmin return the other
// operand for a NaN, as Rust's f32::max/min do.
inline SwPostConfig post_config_clamped(const SwPostConfig& in)
{
	SwPostConfig c = in;
	c.min_exposure = std::fmin(std::fmax(c.min_exposure, 1.0f / 65536.0f), 16.0f);
	c.max_exposure = std::fmin(std::fmax(c.max_exposure, 1.0f), 65536.0f);
	c.exposure_update_speed = std::fmin(std::fmax(c.exposure_update_speed, 0.5f), 16.0f);
	c.base_brightness = std::fmin(std::fmax(c.base_brightness, 0.5f), 2.0f);
	c.zero_level_brightness = std::fmin(std::fmax(c.zero_level_brightness, 1.0f / 16.0f), 16.0f);
	c.brightness_scale_power = std::fmin(std::fmax(c.brightness_scale_power, 0.01f), 0.5f);
	c.bloom_sigma = std::fmin(std::fmax(c.bloom_sigma, 0.0f), 40.0f);
	c.bloom_buffer_scale_log2 = c.bloom_buffer_scale_log2 < 1u ? 1u : (c.bloom_buffer_scale_log2 > 3u ? 3u : c.bloom_buffer_scale_log2);
	c.bloom_scale = std::fmin(std::fmax(c.bloom_scale, 1.0f / 16.0f), 0.5f);
	return c;
}

// Everything of PostArgs that comes from the (clamped) configuration, the exposure and the colour
// modulation, for a width x height frame: TonemappingFunction::new (postprocessor.rs:1005-1017, lanes
// [b, g, r, a]) and, with bloom, the buffer scale, bloom size, blur radius and the integer Gaussian
// weights of perform_bloom / compute_gaussian_kernel (postprocessor.rs:729-789, 1026-1045), evaluated
// on the host in f32 with the C library's exp and sqrt. Buffers and destination are the caller's.
// Returns false when the frame is too small for the bloom buffer (under 2 x 2 bloom pixels).
inline bool post_args_from_config(PostArgs& a, const SwPostConfig& c, float exposure, const float color_modulate[3],
	uint32_t width, uint32_t height)
{
	a.width = width;
	a.height = height;
	a.use_bloom = c.bloom_sigma > 0.0f ? 1u : 0u;
	a.linear_filter = c.linear_bloom_filter ? 1u : 0u;
	a.inv_scale[0] = 1.0f / (exposure * color_modulate[2]);
	a.inv_scale[1] = 1.0f / (exposure * color_modulate[1]);
	a.inv_scale[2] = 1.0f / (exposure * color_modulate[0]);
	a.inv_scale[3] = 0.0f;
	a.inv_255[0] = a.inv_255[1] = a.inv_255[2] = 1.0f / 255.0f;
	a.inv_255[3] = 0.0f;
	if (!a.use_bloom) return true;
	const int log2 = std::min(std::max(int(c.bloom_buffer_scale_log2), 1), 3);
	const uint32_t S = 1u << log2;
	a.scale = S;
	a.bw = width / S;
	a.bh = height / S;
	if (a.bw < 2 || a.bh < 2) return false;
	const float sigma = c.bloom_sigma / float(S);
	const float rf = std::ceil(3.0f * sigma - 0.5f);
	uint32_t radius = rf > 0.0f ? uint32_t(rf) : 0u;
	if (radius > 16) radius = 16;
	a.radius = radius;
	float kernel[33] = {0};
	const float samples[4] = {-0.375f, -0.125f, 0.125f, 0.375f};
	const float tau = 6.28318530717958647692f;
	for (int32_t x = -int32_t(radius); x <= int32_t(radius); ++x)
	{
		float val = 0.0f;
		for (float smp : samples)
		{
			const float coord = float(x) + smp;
			val += std::exp(-0.5f * (coord / sigma) * (coord / sigma)) / (sigma * std::sqrt(tau));
		}
		kernel[x + int32_t(radius)] = val / 4.0f;
	}
	for (int i = 0; i < 33; ++i)
	{
		a.kernel_h[i] = f2i32_as(kernel[i] * float(1 << 14));
		a.kernel_v[i] = f2i32_as(kernel[i] * c.bloom_scale * float(1 << 14));
	}
	return true;
}

int launch_upscale(uint32_t mode, uint32_t scale, const uint32_t* src, uint32_t* dst, uint32_t dst_width,
	uint32_t dst_height, uint32_t dst_pitch, cudaStream_t stream);

int launch_fill(void* dst, uint64_t count, uint64_t value, uint32_t bytes_per_pixel, cudaStream_t stream);

} // namespace swgpu
