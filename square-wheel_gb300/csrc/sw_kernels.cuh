// Kernel argument blocks and launch entry points of the GB300 rendering path.
#pragma once

#include "sw_device.cuh"

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
	const uint64_t* texels;
	const uint32_t* emissive_pixels;
	const float* lightmaps;
	const SwDirectionalLightmapElement* directional_lightmaps;
	const SwLight* lights;
	float cam_pos[3];
	void* arena;
};

// Host-side construction of one SurfaceGpu (exact f32 arithmetic; the file is compiled without FMA
// contraction).
void make_surface_gpu(const SwSurfaceDesc& d, const SwTextureMip* tex, const SwEmissiveMip* em, SurfaceGpu& out);

// Persistent grid of at most num_sms * blocks_per_sm blocks of 256 threads.
int launch_surface_build(const SurfaceKernelArgs& args, uint32_t pixel_format, int num_sms, int blocks_per_sm, cudaStream_t stream);

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
// xs >= xe: the row holds no pixel.
struct RasterRow
{
	int32_t xs, xe;
	int32_t a0, b0, a1, b1, a2, b2;
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
	const DrawRows* draw_rows;
	uint32_t num_draws;
	uint32_t total_rows; // row records of all draws
	int32_t width, height;
	uint32_t clear_background;
	RasterPart* parts;     // num_draws * SW_RASTER_MAX_PARTS
	uint32_t* part_counts; // num_draws
	RasterDraw* rdraws;
	RasterRow* rows;
	RasterBox* boxes;
	const void* arena;
	uint64_t arena_texels;
	const void* skybox; // skybox texels of the frame's pixel format (SW_TEXSRC_SKYBOX draws)
	void* framebuffer;  // width * height pixels, tightly packed
	unsigned int* error_counter;
};

// Edge walk + row setup (raster_setup, one CTA per draw), then the tile pass (raster_tiles).
int launch_raster_setup(const RasterArgs& args, cudaStream_t stream);
// variant: tile shape index (< SW_RASTER_TILE_VARIANTS, see SwTuning); every variant gives the same frame.
int launch_raster_tiles(const RasterArgs& args, uint32_t pixel_format, uint32_t variant, cudaStream_t stream);

// Host side: rows [y0, y0 + nrows) a draw can cover (from its vertices).
void draw_row_range(const SwDrawCmd& d, const SwVertex16* vertices, int32_t height, int32_t& y0, uint32_t& nrows);

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
	float inv_255[4];
	uint32_t linear_filter;
	uint32_t use_bloom;
	uint32_t* dst;
	uint32_t dst_pitch;
};

// aux/fork/join (optional): run the exposure-average reduction on `aux`, joined back before returning.
int launch_postprocess(const PostArgs& args, int num_sms, cudaStream_t stream, cudaStream_t aux = nullptr,
	cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);

int launch_upscale(uint32_t mode, uint32_t scale, const uint32_t* src, uint32_t* dst, uint32_t dst_width,
	uint32_t dst_height, uint32_t dst_pitch, cudaStream_t stream);

int launch_fill(void* dst, uint64_t count, uint64_t value, uint32_t bytes_per_pixel, cudaStream_t stream);

} // namespace swgpu
