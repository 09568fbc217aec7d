// C ABI of the GB300 rendering path (include/swgpu.h): context, device memory, uploads, launches.
//
// Device memory layout (HBM):
//   static, uploaded once by sw_create: all material texture mips as one TextureElement array, their
//   SwTextureMip table, emissive Color32 mips + table, simple (12 B) and directional (40 B) lightmap
//   element arrays;
//   per frame, grown on demand and reused: lights, surface descriptors + texel prefix sums, the surface
//   arena (one Color32/Color64 texel per surface texel, surfaces contiguous and row-major), draw
//   commands + vertices + per-draw row ranges, raster setup output (per-draw records, per-row span
//   records, pixel boxes), the frame buffer
//   (width*height pixels), bloom buffers and the exposure-average scratch.
// Host->device uploads go through pinned staging buffers on the context's stream. Every descriptor is
// validated on the host before launch so that no kernel can read outside its buffers.
#include "sw_kernels.cuh"
#include "../host/prep_math.h"

#include "../../include/swlearn.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace swgpu;

namespace
{

struct DevBuf
{
	void* ptr = nullptr;
	size_t bytes = 0;
};

struct Staging
{
	void* host = nullptr;
	size_t bytes = 0;
	cudaEvent_t done = nullptr;
	bool pending = false;
};

// Everything a view frame graph (sw_draw_frame_view) bakes in: when this differs from the graph's, it is
// captured again.
struct ViewGraphKey
{
	PrepArgs prep;
	SurfaceKernelArgs surf;
	RasterArgs raster;
	PostArgs post;
	const void* staging;
	size_t block_bytes;
	unsigned surface_blocks;
	int surface_blocks_per_sm;
	int surface_texels_per_thread;
	uint32_t raster_tile, pixel_format, postprocess, dst_pitch;
	void* dst;
	int32_t dst_is_device;
	uint32_t slot;
	uint32_t in_flight; // the frame runs in flight with the next one (average event in the graph)
};

} // namespace

struct SwCtx
{
	int device = 0;
	int num_sms = 0;
	cudaStream_t stream = nullptr;
	// Second stream: draw uploads + raster setup run beside the surface build; the exposure average
	// runs beside blur/tonemap. ev_setup / ev_tiles / ev_fork / ev_join order the two streams.
	cudaStream_t aux = nullptr;
	cudaEvent_t ev_setup = nullptr, ev_tiles = nullptr, ev_fork = nullptr, ev_join = nullptr;
	bool tiles_recorded = false;
	std::string last_error;

	// static
	DevBuf texels, texture_mips, emissive, emissive_mips, lightmaps, dir_lightmaps;
	DevBuf lm_compressed; // sw_set_lightmaps_compressed: the compressed lumps as uploaded
	// the tile pass's bins (raster_bin_kernel): bins_x * bins_y lists of bin_cap draw indices and counts
	DevBuf bin_lists, bin_counts;
	uint32_t bin_cap = 0, bins_x = 0, bins_y = 0;
	// the bins of a whole frame's nested views (portal textures), reused view after view
	DevBuf vbin_lists, vbin_counts;
	uint32_t vbin_cap = 0;
	uint64_t vbin_cells = 0;
	DevBuf skybox32, skybox64; // sw_set_skybox: the same texels in Color32 and Color64
	DevBuf frame_in;           // sw_draw_frame: all per-frame arrays of one frame, uploaded by one copy
	struct HostRange
	{
		char* ptr;
		size_t bytes;
	};
	std::vector<HostRange> registered; // sw_register_host_buffer
	uint64_t skybox_texels = 0;
	std::vector<SwTextureMip> h_texture_mips;
	std::vector<SwEmissiveMip> h_emissive_mips;
	uint64_t num_lightmap_elements = 0, num_dir_lightmap_elements = 0;
	uint64_t num_texels = 0, num_emissive_pixels = 0;

	// frame
	bool frame_open = false;
	SwFrameParams frame{};
	uint32_t num_lights = 0;
	DevBuf lights, surfaces, work_prefix, arena;
	uint64_t arena_texels = 0;
	uint32_t arena_format = SW_PIXEL_C32;
	bool arena_view = false; // the arena was sized by a view frame: its texels are in v_counts
	bool arena_valid = false;
	uint32_t last_num_surfaces = 0, last_surface_format = SW_PIXEL_C32, last_max_light = 0;
	uint64_t last_surface_work = 0;
	std::vector<uint64_t> h_prefix; // texel prefix sums of the last sw_submit_surfaces (per-surface launches)
	cudaGraphExec_t sexec = nullptr; // sw_rebuild_surfaces' graph: one persistent surface launch
	SurfaceKernelArgs skey{};        // ... and the arguments it was captured with
	unsigned sblocks = 0;
	bool last_surface_directional = false;
	DevBuf draws, vertices, tri_vertices, draw_rows, rdraws, rows, boxes, tri_steps;
	DevBuf lite; // sw_set_lite_textures: Color32 textures of triangle draws
	uint64_t lite_texels = 0;
	uint64_t num_rows = 0;
	uint32_t num_draws = 0;
	bool draws_valid = false;
	DevBuf framebuffer;
	uint32_t fb_width = 0, fb_height = 0, fb_format = SW_PIXEL_C32;
	bool fb_valid = false;

	// postprocessor
	DevBuf bloom0, bloom1, line_sums, line_sums_f, average, error_counter;
	float exposure = 1.0f;
	bool exposure_pending = false;
	SwPostConfig pending_config{};
	float pending_dt = 0.0f;
	float* h_average = nullptr; // pinned, 4 floats
	cudaEvent_t average_ready = nullptr;

	// Two frames in flight (sw_set_frames_in_flight): a whole-frame call returns once its frame is
	// enqueued and the previous frame is in its host destination. Each frame's Color32 result goes to a
	// device buffer of its slot and a copy engine moves it to the caller's registered host buffer on the
	// copy stream while the next frame computes; the frame's average colour is signalled by an event
	// recorded inside the graph, so the next frame's exposure is known before this frame's tonemap ends.
	uint32_t frames_in_flight = 1;
	cudaStream_t copy = nullptr;
	cudaEvent_t ev_graph_done[2] = {nullptr, nullptr}, ev_d2h[2] = {nullptr, nullptr};
	bool d2h_pending[2] = {false, false};
	DevBuf ldr[2];

	Staging stage_lights, stage_surfaces, stage_prefix, stage_draws, stage_vertices, stage_tri_vertices, stage_draw_rows, stage_io;

	// upscale scratch (src/dst copies for host buffers)
	DevBuf up_src, up_dst;
	SwUpscaler* learned = nullptr; // sw_set_learned_upscaler

	SwStats stats{};

	// Launch configuration (sw_set_tuning / sw_autotune).
	SwTuning tuning{0u, 24u, 0u, 0u};

	// Whole-frame CUDA graph (sw_draw_frame): double-buffered pinned staging of all per-frame arrays,
	// the instantiated graph, updated in place from each frame's capture.
	bool graph_enabled = true;
	bool capturing = false; // stage timing events are not recorded inside a capture
	cudaGraphExec_t gexec = nullptr;
	Staging gstage[2];
	uint32_t gset = 0;

	// GPU-side surface and draw preparation (sw_set_map, sw_draw_frame_view): the map's polygons and
	// vertices, per-polygon surface size bounds (prefix sums, for capacities), the candidates' scratch,
	// the prepared descriptors, the counts (device, and a pinned copy read back after each frame).
	DevBuf map_polygons, map_vertices, vslab;
	uint64_t vs_cands = 0, vs_draws = 0, vs_vertices = 0, vs_rows = 0; // the slab's capacities (only grow)
	SwViewCounts* v_counts = nullptr; // in the slab
	SwSurfaceDesc* v_descs = nullptr;
	SwDrawCmd* v_draws = nullptr;
	SwVertex16* v_vertices = nullptr;
	float* d_average_mapped = nullptr; // h_average as the device sees it
	uint32_t num_map_polygons = 0, num_map_vertices = 0;
	uint64_t map_lightmap_end = 0; // the largest lightmap end (offset + size) over sw_set_map's polygons
	std::vector<uint64_t> poly_bound_prefix;
	SwViewCounts* h_counts = nullptr; // pinned, one per staging set (frames alternate)
	cudaEvent_t ev_counts[2] = {nullptr, nullptr};
	bool counts_pending[2] = {false, false};
	uint64_t counts_seq[2] = {0, 0};
	uint64_t view_seq = 0, hint_seq = 0;
	uint64_t view_work_hint = 0; // texels of the latest frame read back (sizes the surface grid)
	uint32_t view_surfaces_cap = 0, view_draws_cap = 0, view_vertices_cap = 0;
	cudaGraphExec_t vexec[2] = {nullptr, nullptr}; // one per staging block, replayed while its key holds
	ViewGraphKey vkey[2];
	uint64_t vcap_lights = 0, vcap_leafs = 0, vcap_leaf_lights = 0, vcap_host_draws = 0, vcap_host_vertices = 0;
	uint64_t vcap_shifts = 0; // material frames in the view upload block
	unsigned view_surface_blocks = 0;
	uint64_t view_captures = 0;
	std::vector<uint32_t> v_draw_leaf;
	std::vector<DrawRows> v_host_rows;

	// Shadow maps (sw_build_shadow_maps / sw_set_light_shadows): the persistent f32 storage (grows, keeps
	// its contents), the packing scratch, and the frame's per-light descriptors on the device.
	DevBuf shadow_storage, shadow_descs;
	uint32_t shadow_seq = 0; // the next depth draw's sequence base (the storage's high words)
	uint64_t shadow_texels = 0;
	uint32_t num_shadow_descs = 0;
	Staging stage_shadow, stage_shadow_descs;
	// sw_update_textures: the groups, layers, passes and shifts of one call, uploaded together
	DevBuf effect_buf;
	Staging stage_effects;
	// sw_update_simulations: the fields / heat maps (sim_words 4-byte words) and one call's upload
	DevBuf sim_state, sim_buf;
	uint64_t sim_words = 0;
	Staging stage_sims;

	// Optional per-stage device timing (sw_enable_timing).
	bool timing = false;
	cudaEvent_t t_begin[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	cudaEvent_t t_end[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	bool t_valid[5] = {false, false, false, false, false};
};

namespace
{
enum Stage
{
	STAGE_SURFACES = 0,
	STAGE_RASTER = 1,
	STAGE_POST = 2,
	STAGE_UPSCALE = 3,
	STAGE_FRAME = 4, // sw_frame_begin .. end of sw_postprocess, both streams joined
	NUM_STAGES = 5
};

RasterArgs raster_args(SwCtx* ctx)
{
	RasterArgs a;
	std::memset(&a, 0, sizeof(a)); // padding included: view graph keys compare argument blocks bytewise
	a.draws = static_cast<const SwDrawCmd*>(ctx->draws.ptr);
	a.vertices = static_cast<const SwVertex16*>(ctx->vertices.ptr);
	a.num_draws = ctx->num_draws;
	a.counts = nullptr;
	a.setup_blocks = 0;
	a.width = int32_t(ctx->frame.width);
	a.height = int32_t(ctx->frame.height);
	a.clear_background = ctx->frame.clear_background;
	a.draw_rows = static_cast<const DrawRows*>(ctx->draw_rows.ptr);
	a.total_rows = uint32_t(ctx->num_rows);
	a.tri_vertices = static_cast<const SwTriVertex*>(ctx->tri_vertices.ptr);
	a.lite = static_cast<const uint32_t*>(ctx->lite.ptr);
	a.lite_texels = ctx->lite_texels;
	a.tri_steps = static_cast<TriSteps*>(ctx->tri_steps.ptr);
	a.rdraws = static_cast<RasterDraw*>(ctx->rdraws.ptr);
	a.rows = static_cast<RasterRow*>(ctx->rows.ptr);
	a.boxes = static_cast<RasterBox*>(ctx->boxes.ptr);
	a.arena = ctx->arena.ptr;
	a.arena_texels = ctx->arena_texels;
	a.skybox = ctx->frame.pixel_format == SW_PIXEL_C64 ? ctx->skybox64.ptr : ctx->skybox32.ptr;
	a.framebuffer = ctx->framebuffer.ptr;
	a.error_counter = static_cast<unsigned int*>(ctx->error_counter.ptr);
	a.bin_lists = static_cast<uint32_t*>(ctx->bin_lists.ptr);
	a.bin_counts = static_cast<uint32_t*>(ctx->bin_counts.ptr);
	a.bin_cap = ctx->bin_cap;
	a.bins_x = ctx->bins_x;
	a.bins_y = ctx->bins_y;
	return a;
}



void stage_begin(SwCtx* ctx, int s)
{
	if (ctx->timing && !ctx->capturing) cudaEventRecord(ctx->t_begin[s], ctx->stream);
}
void stage_end(SwCtx* ctx, int s)
{
	if (ctx->timing && !ctx->capturing)
	{
		cudaEventRecord(ctx->t_end[s], ctx->stream);
		ctx->t_valid[s] = true;
	}
}
} // namespace

namespace
{

int fail(SwCtx* ctx, int code, const char* fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	if (ctx) ctx->last_error = buf;
	return code;
}

int cuda_fail(SwCtx* ctx, cudaError_t e, const char* what)
{
	return fail(ctx, SW_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SW_CUDA(ctx, call)                                  \
	do                                                      \
	{                                                       \
		cudaError_t e_ = (call);                            \
		if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
	} while (0)

int ensure(SwCtx* ctx, DevBuf& b, size_t bytes)
{
	if (bytes <= b.bytes && b.ptr) return SW_OK;
	size_t want = std::max(bytes, b.bytes + b.bytes / 2);
	if (want == 0) want = 256;
	if (b.ptr)
	{
		cudaError_t e = cudaStreamSynchronize(ctx->stream);
		if (e == cudaSuccess && ctx->aux) e = cudaStreamSynchronize(ctx->aux);
		if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
		cudaFree(b.ptr);
		b.ptr = nullptr;
		b.bytes = 0;
	}
	cudaError_t e = cudaMalloc(&b.ptr, want);
	if (e != cudaSuccess)
	{
		cudaGetLastError();
		return fail(ctx, SW_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu bytes) failed: %s", want, cudaGetErrorString(e));
	}
	b.bytes = want;
	return SW_OK;
}

// The bins of a width x height frame for up to `draws` draws (capacities only grow, so replayed graphs
// keep their buffers).
int ensure_bins(SwCtx* ctx, uint32_t width, uint32_t height, uint64_t draws)
{
	const uint32_t bx = raster_bins(int32_t(width), RASTER_BIN_W), by = raster_bins(int32_t(height), RASTER_BIN_H);
	uint32_t cap = std::max<uint32_t>(ctx->bin_cap, 256);
	while (cap < draws) cap *= 2;
	int r;
	if ((r = ensure(ctx, ctx->bin_lists, size_t(bx) * by * cap * 4))) return r;
	if ((r = ensure(ctx, ctx->bin_counts, size_t(bx) * by * 4))) return r;
	ctx->bin_cap = cap;
	ctx->bins_x = bx;
	ctx->bins_y = by;
	return SW_OK;
}

// The bins of a frame's nested views: enough cells for the largest view and room for its draws.
int ensure_view_bins(SwCtx* ctx, const SwView* views, uint32_t num_views)
{
	uint64_t cells = 1;
	uint32_t draws = 1;
	for (uint32_t i = 0; i < num_views; ++i)
	{
		cells = std::max<uint64_t>(cells, uint64_t(raster_bins(int32_t(views[i].width), RASTER_BIN_W)) *
				raster_bins(int32_t(views[i].height), RASTER_BIN_H));
		draws = std::max(draws, views[i].num_draws);
	}
	uint32_t cap = std::max<uint32_t>(ctx->vbin_cap, 256);
	while (cap < draws) cap *= 2;
	cells = std::max(cells, ctx->vbin_cells);
	int r;
	if ((r = ensure(ctx, ctx->vbin_lists, size_t(cells) * cap * 4))) return r;
	if ((r = ensure(ctx, ctx->vbin_counts, size_t(cells) * 4))) return r;
	ctx->vbin_cap = cap;
	ctx->vbin_cells = cells;
	return SW_OK;
}

void release(DevBuf& b)
{
	if (b.ptr) cudaFree(b.ptr);
	b.ptr = nullptr;
	b.bytes = 0;
}

// Pinned staging: acquire() waits until the previous copy out of the buffer finished and grows it;
// the caller fills it; commit() enqueues the host-to-device copy on the context's stream.
int staging_acquire(SwCtx* ctx, Staging& st, size_t bytes, void** host)
{
	if (st.pending)
	{
		SW_CUDA(ctx, cudaEventSynchronize(st.done));
		st.pending = false;
	}
	if (st.bytes < bytes)
	{
		const size_t want = std::max(bytes, st.bytes * 2);
		if (st.host) cudaFreeHost(st.host);
		st.host = nullptr;
		st.bytes = 0;
		SW_CUDA(ctx, cudaMallocHost(&st.host, want));
		st.bytes = want;
	}
	if (!st.done) SW_CUDA(ctx, cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming));
	*host = st.host;
	return SW_OK;
}

int staging_commit(SwCtx* ctx, Staging& st, void* dst, size_t bytes, cudaStream_t stream = nullptr)
{
	if (bytes == 0) return SW_OK;
	if (!stream) stream = ctx->stream;
	SW_CUDA(ctx, cudaMemcpyAsync(dst, st.host, bytes, cudaMemcpyHostToDevice, stream));
	SW_CUDA(ctx, cudaEventRecord(st.done, stream));
	st.pending = true;
	ctx->stats.upload_bytes += bytes;
	return SW_OK;
}

// Copy `bytes` from host memory `src` into device buffer `dst` through a pinned staging buffer.
int upload(SwCtx* ctx, Staging& st, void* dst, const void* src, size_t bytes, cudaStream_t stream = nullptr)
{
	if (bytes == 0) return SW_OK;
	void* h = nullptr;
	int r = staging_acquire(ctx, st, bytes, &h);
	if (r) return r;
	std::memcpy(h, src, bytes);
	return staging_commit(ctx, st, dst, bytes, stream);
}

int upload_static(SwCtx* ctx, DevBuf& b, const void* src, size_t bytes)
{
	int r = ensure(ctx, b, bytes ? bytes : 16);
	if (r) return r;
	if (bytes) SW_CUDA(ctx, cudaMemcpy(b.ptr, src, bytes, cudaMemcpyHostToDevice));
	return SW_OK;
}

// Device -> user buffer copy of a width x height image with row pitches in pixels.
int copy_out(SwCtx* ctx, void* dst, uint32_t dst_pitch, int dst_is_device, const void* src, uint32_t src_pitch,
	uint32_t width, uint32_t height, uint32_t bpp)
{
	const size_t row = size_t(width) * bpp;
	if (dst_is_device)
	{
		SW_CUDA(ctx, cudaMemcpy2DAsync(dst, size_t(dst_pitch) * bpp, src, size_t(src_pitch) * bpp, row, height,
						 cudaMemcpyDeviceToDevice, ctx->stream));
		return SW_OK;
	}
	const size_t bytes = row * height;
	const size_t span = size_t(height - 1) * dst_pitch * bpp + row;
	for (const SwCtx::HostRange& hr : ctx->registered)
		if (static_cast<char*>(dst) >= hr.ptr && static_cast<char*>(dst) + span <= hr.ptr + hr.bytes)
		{
			// page-locked by sw_register_host_buffer: straight from the device into the caller's rows
			SW_CUDA(ctx, cudaMemcpy2DAsync(dst, size_t(dst_pitch) * bpp, src, size_t(src_pitch) * bpp, row, height,
							 cudaMemcpyDeviceToHost, ctx->stream));
			SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
			return SW_OK;
		}
	Staging& st = ctx->stage_io;
	if (st.pending)
	{
		SW_CUDA(ctx, cudaEventSynchronize(st.done));
		st.pending = false;
	}
	if (st.bytes < bytes)
	{
		if (st.host) cudaFreeHost(st.host);
		st.host = nullptr;
		SW_CUDA(ctx, cudaMallocHost(&st.host, bytes));
		st.bytes = bytes;
	}
	SW_CUDA(ctx, cudaMemcpy2DAsync(st.host, row, src, size_t(src_pitch) * bpp, row, height, cudaMemcpyDeviceToHost, ctx->stream));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	for (uint32_t y = 0; y < height; ++y)
		std::memcpy(static_cast<char*>(dst) + size_t(y) * dst_pitch * bpp, static_cast<const char*>(st.host) + y * row, row);
	return SW_OK;
}

// Device address of host memory [ptr, ptr + bytes) inside a buffer registered with
// sw_register_host_buffer (registered memory is mapped), or nullptr.
void* registered_device_pointer(SwCtx* ctx, void* ptr, size_t bytes)
{
	for (const SwCtx::HostRange& hr : ctx->registered)
		if (static_cast<char*>(ptr) >= hr.ptr && static_cast<char*>(ptr) + bytes <= hr.ptr + hr.bytes)
		{
			void* d = nullptr;
			if (cudaHostGetDevicePointer(&d, ptr, 0) != cudaSuccess)
			{
				cudaGetLastError();
				return nullptr;
			}
			return d;
		}
	return nullptr;
}

// The slot of a whole frame that runs in flight with the next one (sw_set_frames_in_flight(ctx, 2)): a
// postprocessed frame whose Color32 destination lies in a registered host buffer, so a copy engine can
// move it there asynchronously. -1: the frame completes within its call.
int frame_pipeline_slot(SwCtx* ctx, bool postprocess, const void* dst, uint32_t dst_pitch, const SwFrameParams& p,
	int dst_is_device, uint32_t slot)
{
	if (ctx->frames_in_flight < 2 || !postprocess || !dst || dst_is_device) return -1;
	const size_t span = (size_t(p.height) - 1) * dst_pitch * 4 + size_t(p.width) * 4;
	for (const SwCtx::HostRange& hr : ctx->registered)
		if (static_cast<const char*>(dst) >= hr.ptr && static_cast<const char*>(dst) + span <= hr.ptr + hr.bytes)
			return int(slot);
	return -1;
}

int check_kernel(SwCtx* ctx, int launch_result, const char* what)
{
	if (launch_result != 0)
		return fail(ctx, SW_ERR_CUDA, "%s launch failed: %s", what, cudaGetErrorString(cudaError_t(launch_result)));
	return SW_OK;
}

uint32_t bpp_of(uint32_t format) { return format == SW_PIXEL_C64 ? 8u : 4u; }

bool all_finite(const float* v, int n)
{
	for (int i = 0; i < n; ++i)
		if (!std::isfinite(v[i])) return false;
	return true;
}

// Camera position and lights of a frame: a NaN or an infinity there is a caller's error, rejected before
// anything is uploaded or launched.
int check_frame_inputs(SwCtx* ctx, const SwFrameParams& p, const SwLight* lights, uint32_t num_lights)
{
	if (!all_finite(p.cam_pos, 3)) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "non-finite camera position");
	for (uint32_t i = 0; i < num_lights; ++i)
	{
		const SwLight& l = lights[i];
		if (!all_finite(l.position, 3) || !all_finite(l.color, 3) || !std::isfinite(l.radius) ||
			!std::isfinite(l.inv_square_radius))
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "light %u: non-finite parameters", i);
	}
	return SW_OK;
}


// Apply the exposure update of the previous postprocessed frame (update_exposure,
// src/square_wheel/postprocessor.rs:206-223, with get_color_brightness :1047-1051), on the host in f32
// with the C library's expf/logf/powf exactly as the reference does.
int finalize_exposure(SwCtx* ctx)
{
	if (!ctx->exposure_pending) return SW_OK;
	SW_CUDA(ctx, cudaEventSynchronize(ctx->average_ready));
	ctx->exposure_pending = false;
	const SwPostConfig& c = ctx->pending_config;
	const float* avg = ctx->h_average;
	const float brightness_raw = (avg[0] + avg[1] + avg[2]) * 0.33f;
	const float brightness = std::fmin(std::fmax(brightness_raw, 1.0f / 1024.0f), 65536.0f) / 255.0f;
	const float target =
		std::pow(brightness / c.zero_level_brightness, c.brightness_scale_power) * 0.5f * c.base_brightness / brightness;
	const float clamped = std::fmin(std::fmax(target, c.min_exposure), c.max_exposure);
	const float mix = std::exp(-c.exposure_update_speed * ctx->pending_dt);
	ctx->exposure = std::exp(std::log(ctx->exposure) * mix + std::log(clamped) * (1.0f - mix));
	return SW_OK;
}

} // namespace

extern "C" {

int sw_create(const SwCreateInfo* info, SwCtx** out_ctx)
{
	if (!info || !out_ctx) return SW_ERR_INVALID_ARGUMENT;
	*out_ctx = nullptr;
	if (info->abi_version != SWGPU_ABI_VERSION) return SW_ERR_INVALID_ARGUMENT;
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
	{
		cudaGetLastError();
		return SW_ERR_NO_DEVICE;
	}
	if (int(info->device) >= count) return SW_ERR_INVALID_ARGUMENT;
	// Validate static tables.
	for (uint32_t i = 0; i < info->num_texture_mips; ++i)
	{
		const SwTextureMip& m = info->texture_mips[i];
		if (m.width == 0 || m.height == 0 || m.offset + uint64_t(m.width) * m.height > info->num_texels)
			return SW_ERR_INVALID_ARGUMENT;
	}
	for (uint32_t i = 0; i < info->num_emissive_mips; ++i)
	{
		const SwEmissiveMip& m = info->emissive_mips[i];
		if (m.width == 0 || m.height == 0 || m.offset + uint64_t(m.width) * m.height > info->num_emissive_pixels)
			return SW_ERR_INVALID_ARGUMENT;
	}

	SwCtx* ctx = new (std::nothrow) SwCtx();
	if (!ctx) return SW_ERR_OUT_OF_MEMORY;
	auto bail = [&](int r) {
		sw_destroy(ctx);
		return r;
	};
	ctx->device = int(info->device);
	if (cudaSetDevice(ctx->device) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess)
		return bail(SW_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess) return bail(SW_ERR_CUDA);
	for (cudaEvent_t* e : {&ctx->ev_setup, &ctx->ev_tiles, &ctx->ev_fork, &ctx->ev_join})
		if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaEventCreateWithFlags(&ctx->average_ready, cudaEventDisableTiming) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&ctx->copy, cudaStreamNonBlocking) != cudaSuccess) return bail(SW_ERR_CUDA);
	for (cudaEvent_t* e : {&ctx->ev_graph_done[0], &ctx->ev_graph_done[1], &ctx->ev_d2h[0], &ctx->ev_d2h[1]})
		if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaMallocHost(reinterpret_cast<void**>(&ctx->h_average), 4 * sizeof(float)) != cudaSuccess)
		return bail(SW_ERR_CUDA);
	if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->d_average_mapped), ctx->h_average, 0) != cudaSuccess)
		return bail(SW_ERR_CUDA);
	for (cudaEvent_t* e : {&ctx->ev_counts[0], &ctx->ev_counts[1]})
		if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaMallocHost(reinterpret_cast<void**>(&ctx->h_counts), 2 * sizeof(SwViewCounts)) != cudaSuccess) return bail(SW_ERR_CUDA);
	std::memset(ctx->h_counts, 0, 2 * sizeof(SwViewCounts));

	int r;
	if ((r = upload_static(ctx, ctx->texels, info->texels, info->num_texels * 8))) return bail(r);
	if ((r = upload_static(ctx, ctx->texture_mips, info->texture_mips, info->num_texture_mips * sizeof(SwTextureMip))))
		return bail(r);
	if ((r = upload_static(ctx, ctx->emissive, info->emissive_pixels, info->num_emissive_pixels * 4))) return bail(r);
	if ((r = upload_static(ctx, ctx->emissive_mips, info->emissive_mips, info->num_emissive_mips * sizeof(SwEmissiveMip))))
		return bail(r);
	if ((r = upload_static(ctx, ctx->lightmaps, info->lightmaps, info->num_lightmap_elements * 12))) return bail(r);
	if ((r = upload_static(ctx, ctx->dir_lightmaps, info->directional_lightmaps,
			 info->num_directional_lightmap_elements * sizeof(SwDirectionalLightmapElement))))
		return bail(r);
	ctx->h_texture_mips.assign(info->texture_mips, info->texture_mips + info->num_texture_mips);
	ctx->h_emissive_mips.assign(info->emissive_mips, info->emissive_mips + info->num_emissive_mips);
	ctx->num_texels = info->num_texels;
	ctx->num_emissive_pixels = info->num_emissive_pixels;
	ctx->num_lightmap_elements = info->num_lightmap_elements;
	ctx->num_dir_lightmap_elements = info->num_directional_lightmap_elements;
	if ((r = ensure(ctx, ctx->error_counter, 16))) return bail(r);
	if (cudaMemset(ctx->error_counter.ptr, 0, 16) != cudaSuccess) return bail(SW_ERR_CUDA);
	if ((r = ensure(ctx, ctx->average, 16))) return bail(r);
	if (info->max_surface_texels && (r = ensure(ctx, ctx->arena, info->max_surface_texels * 8))) return bail(r);
	*out_ctx = ctx;
	return SW_OK;
}

int sw_destroy(SwCtx* ctx)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	if (ctx->stream) cudaStreamSynchronize(ctx->stream);
	if (ctx->aux) cudaStreamSynchronize(ctx->aux);
	DevBuf* bufs[] = {&ctx->texels, &ctx->texture_mips, &ctx->emissive, &ctx->emissive_mips, &ctx->lightmaps, &ctx->lm_compressed, &ctx->bin_lists, &ctx->bin_counts, &ctx->skybox32,
		&ctx->skybox64, &ctx->frame_in,
		&ctx->dir_lightmaps, &ctx->lights, &ctx->surfaces, &ctx->work_prefix, &ctx->arena, &ctx->draws, &ctx->vertices,
		&ctx->draw_rows, &ctx->rdraws, &ctx->rows, &ctx->boxes, &ctx->tri_steps, &ctx->tri_vertices, &ctx->lite, &ctx->ldr[0], &ctx->ldr[1], &ctx->framebuffer, &ctx->bloom0, &ctx->bloom1, &ctx->line_sums,
		&ctx->line_sums_f, &ctx->average, &ctx->error_counter, &ctx->up_src, &ctx->up_dst, &ctx->map_polygons,
		&ctx->map_vertices, &ctx->vslab, &ctx->shadow_storage, &ctx->shadow_descs, &ctx->effect_buf, &ctx->sim_state, &ctx->sim_buf, &ctx->vbin_lists,
		&ctx->vbin_counts};
	for (DevBuf* b : bufs) release(*b);
	for (const SwCtx::HostRange& h : ctx->registered) cudaHostUnregister(h.ptr);
	if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
	if (ctx->sexec) cudaGraphExecDestroy(ctx->sexec);
	for (cudaGraphExec_t e : ctx->vexec)
		if (e) cudaGraphExecDestroy(e);
	if (ctx->h_counts) cudaFreeHost(ctx->h_counts);
	for (cudaEvent_t e : ctx->ev_counts)
		if (e) cudaEventDestroy(e);
	Staging* st[] = {&ctx->stage_lights, &ctx->stage_surfaces, &ctx->stage_prefix, &ctx->stage_draws,
		&ctx->stage_vertices, &ctx->stage_tri_vertices, &ctx->stage_draw_rows, &ctx->stage_io, &ctx->gstage[0], &ctx->gstage[1], &ctx->stage_shadow,
		&ctx->stage_shadow_descs, &ctx->stage_effects, &ctx->stage_sims};
	for (Staging* s : st)
	{
		if (s->host) cudaFreeHost(s->host);
		if (s->done) cudaEventDestroy(s->done);
	}
	if (ctx->h_average) cudaFreeHost(ctx->h_average);
	if (ctx->average_ready) cudaEventDestroy(ctx->average_ready);
	for (int i = 0; i < 5; ++i)
	{
		if (ctx->t_begin[i]) cudaEventDestroy(ctx->t_begin[i]);
		if (ctx->t_end[i]) cudaEventDestroy(ctx->t_end[i]);
	}
	if (ctx->stream) cudaStreamDestroy(ctx->stream);
	if (ctx->aux) cudaStreamDestroy(ctx->aux);
	if (ctx->copy) cudaStreamDestroy(ctx->copy);
	for (cudaEvent_t e : {ctx->ev_setup, ctx->ev_tiles, ctx->ev_fork, ctx->ev_join, ctx->ev_graph_done[0], ctx->ev_graph_done[1],
			 ctx->ev_d2h[0], ctx->ev_d2h[1]})
		if (e) cudaEventDestroy(e);
	delete ctx;
	return SW_OK;
}

const char* sw_last_error(const SwCtx* ctx)
{
	if (!ctx) return "null context";
	return ctx->last_error.c_str();
}

int sw_sync(SwCtx* ctx)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->copy));
	ctx->d2h_pending[0] = ctx->d2h_pending[1] = false;
	return SW_OK;
}

int sw_enable_timing(SwCtx* ctx, int enable)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	if (enable && !ctx->t_begin[0])
		for (int i = 0; i < 5; ++i)
		{
			SW_CUDA(ctx, cudaEventCreate(&ctx->t_begin[i]));
			SW_CUDA(ctx, cudaEventCreate(&ctx->t_end[i]));
		}
	ctx->timing = enable != 0;
	for (int i = 0; i < 5; ++i) ctx->t_valid[i] = false;
	return SW_OK;
}

int sw_get_timings(SwCtx* ctx, float out_ms[5])
{
	if (!ctx || !out_ms) return SW_ERR_INVALID_ARGUMENT;
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	for (int i = 0; i < 5; ++i)
	{
		out_ms[i] = 0.0f;
		if (ctx->t_valid[i]) SW_CUDA(ctx, cudaEventElapsedTime(&out_ms[i], ctx->t_begin[i], ctx->t_end[i]));
	}
	return SW_OK;
}

int sw_get_stream(SwCtx* ctx, void** out_stream)
{
	if (!ctx || !out_stream) return SW_ERR_INVALID_ARGUMENT;
	*out_stream = ctx->stream;
	return SW_OK;
}

int sw_frame_begin(SwCtx* ctx, const SwFrameParams* params, const SwLight* lights, uint32_t num_lights)
{
	if (!ctx || !params || (num_lights && !lights)) return SW_ERR_INVALID_ARGUMENT;
	if (params->pixel_format > SW_PIXEL_C64) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "bad pixel format");
	if (params->width == 0 || params->height == 0 || params->width > 16384 || params->height > 16384)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "bad frame size %ux%u", params->width, params->height);
	if (params->use_directional_lightmaps && ctx->num_dir_lightmap_elements == 0)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "directional lightmaps requested but none uploaded");
	if (num_lights > 65535) return fail(ctx, SW_ERR_LIMIT, "too many lights");
	int r = check_frame_inputs(ctx, *params, lights, num_lights);
	if (r) return r;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	ctx->frame = *params;
	ctx->num_lights = num_lights;
	stage_begin(ctx, STAGE_FRAME);
	if ((r = ensure(ctx, ctx->lights, std::max<size_t>(num_lights, 1) * sizeof(SwLight)))) return r;
	if ((r = upload(ctx, ctx->stage_lights, ctx->lights.ptr, lights, num_lights * sizeof(SwLight)))) return r;
	ctx->frame_open = true;
	ctx->arena_valid = false;
	ctx->draws_valid = false;
	return SW_OK;
}

// Surface build of the last submitted surfaces; `in` (optional) holds the lights, surface records and
// prefix sums instead of the context's own buffers.
struct SurfaceInputs
{
	const SwLight* lights;
	const SurfaceGpu* surfaces;
	const uint64_t* work_prefix;
};
static SurfaceKernelArgs surface_args(SwCtx* ctx, const SurfaceInputs* in = nullptr)
{
	SurfaceKernelArgs a;
	std::memset(&a, 0, sizeof(a)); // optional fields (counts, cam_pos_dev) stay unset on this path
	a.shadows = ctx->num_shadow_descs ? static_cast<const SwLightShadow*>(ctx->shadow_descs.ptr) : nullptr;
	a.shadow_texels = static_cast<const unsigned long long*>(ctx->shadow_storage.ptr);
	a.num_shadows = ctx->num_shadow_descs;
	a.surfaces = in ? in->surfaces : static_cast<const SurfaceGpu*>(ctx->surfaces.ptr);
	a.work_prefix = in ? in->work_prefix : static_cast<const uint64_t*>(ctx->work_prefix.ptr);
	a.num_surfaces = ctx->last_num_surfaces;
	a.counts = nullptr;
	a.directional = ctx->last_surface_directional ? 1u : 0u;
	a.total_work = ctx->last_surface_work;
	a.texels = static_cast<const uint64_t*>(ctx->texels.ptr);
	a.emissive_pixels = static_cast<const uint32_t*>(ctx->emissive.ptr);
	a.lightmaps = static_cast<const float*>(ctx->lightmaps.ptr);
	a.directional_lightmaps = static_cast<const SwDirectionalLightmapElement*>(ctx->dir_lightmaps.ptr);
	a.lights = in ? in->lights : static_cast<const SwLight*>(ctx->lights.ptr);
	for (int i = 0; i < 3; ++i) a.cam_pos[i] = ctx->frame.cam_pos[i];
	a.arena = ctx->arena.ptr;
	return a;
}

static int launch_surfaces(SwCtx* ctx, const SurfaceInputs* in = nullptr)
{
	const SurfaceKernelArgs a = surface_args(ctx, in);
	stage_begin(ctx, STAGE_SURFACES);
	int r = check_kernel(ctx,
		launch_surface_build(a, ctx->frame.pixel_format, ctx->num_sms, int(ctx->tuning.surface_blocks_per_sm), ctx->stream, 0,
			ctx->tuning.surface_texels_per_thread),
		"surface build");
	stage_end(ctx, STAGE_SURFACES);
	if (r) return r;
	ctx->arena_valid = true;
	ctx->stats.surfaces += ctx->last_num_surfaces;
	ctx->stats.surface_texels += ctx->last_surface_work;
	return SW_OK;
}

namespace
{
// Host side of sw_submit_surfaces: validate every descriptor against the static data and the frame's
// lights, and write the SurfaceGpu records and texel prefix sums (num_surfaces + 1 entries).
int prepare_surfaces(SwCtx* ctx, const SwSurfaceDesc* surfaces, uint32_t num_surfaces, uint64_t total_texels, SurfaceGpu* gs,
	uint64_t* prefix, uint64_t* out_work, uint32_t* out_max_light)
{
	const bool directional = ctx->frame.use_directional_lightmaps != 0;
	const uint64_t lm_elems = directional ? ctx->num_dir_lightmap_elements : ctx->num_lightmap_elements;
	uint64_t acc = 0;
	uint32_t max_light = 0;
	for (uint32_t i = 0; i < num_surfaces; ++i)
	{
		const SwSurfaceDesc& s = surfaces[i];
		prefix[i] = acc;
		const uint64_t area = uint64_t(s.size[0]) * s.size[1];
		if (s.size[0] == 0 || s.size[1] == 0 || s.size[0] > 65536 || s.size[1] > 65536)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: bad size", i);
		if (s.out_offset + area > total_texels) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: outside arena", i);
		if ((s.flags & SW_SURF_DIFFUSE_LAYER) && s.texture_mip >= ctx->h_texture_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: bad texture mip", i);
		if (s.emissive_mip != SW_NO_EMISSIVE && s.emissive_mip >= ctx->h_emissive_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: bad emissive mip", i);
		if (s.num_lights > SW_MAX_POLYGON_LIGHTS) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: too many lights", i);
		for (uint32_t l = 0; l < s.num_lights; ++l)
		{
			if (s.lights[l] >= ctx->num_lights) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: bad light index", i);
			max_light = std::max<uint32_t>(max_light, s.lights[l] + 1u);
		}
		if ((s.flags & SW_SURF_DIFFUSE_LAYER) && s.lightmap_offset != SW_NO_LIGHTMAP)
		{
			// Every texel reads lightmap rows lv, lv+1 and columns lu, lu+1 (surfaces.rs:479-543).
			if (s.lightmap_scale_log2 > 4) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: bad lightmap scale", i);
			const uint64_t lu_max = (uint64_t(s.size[0]) - 1 + s.lightmap_tc_shift[0]) >> s.lightmap_scale_log2;
			const uint64_t lv_max = (uint64_t(s.size[1]) - 1 + s.lightmap_tc_shift[1]) >> s.lightmap_scale_log2;
			if (lu_max + 1 >= s.lightmap_size[0] || lv_max + 1 >= s.lightmap_size[1] ||
				uint64_t(s.lightmap_offset) + uint64_t(s.lightmap_size[0]) * s.lightmap_size[1] > lm_elems)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "surface %u: lightmap reads out of range", i);
		}
		make_surface_gpu(s, (s.flags & SW_SURF_DIFFUSE_LAYER) ? &ctx->h_texture_mips[s.texture_mip] : nullptr,
			s.emissive_mip != SW_NO_EMISSIVE ? &ctx->h_emissive_mips[s.emissive_mip] : nullptr, gs[i]);
		acc += area;
	}
	prefix[num_surfaces] = acc;
	*out_work = acc;
	*out_max_light = max_light;
	return SW_OK;
}

// Records what the surface launch needs after the descriptors of this frame were prepared.
void note_surfaces(SwCtx* ctx, uint32_t num_surfaces, uint64_t total_texels, uint64_t work, uint32_t max_light)
{
	ctx->arena_texels = total_texels;
	ctx->arena_format = ctx->frame.pixel_format;
	ctx->arena_view = false;
	ctx->last_num_surfaces = num_surfaces;
	ctx->last_surface_work = work;
	ctx->last_surface_directional = ctx->frame.use_directional_lightmaps != 0;
	ctx->last_surface_format = ctx->frame.pixel_format;
	ctx->last_max_light = max_light;
}
} // namespace

int sw_submit_surfaces(SwCtx* ctx, const SwSurfaceDesc* surfaces, uint32_t num_surfaces, uint64_t total_texels)
{
	if (!ctx || (num_surfaces && !surfaces)) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open) return fail(ctx, SW_ERR_STATE, "sw_frame_begin must precede sw_submit_surfaces");
	int r;
	SurfaceGpu* gs = nullptr;
	uint64_t* prefix = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_surfaces, std::max<size_t>(num_surfaces, 1) * sizeof(SurfaceGpu),
			 reinterpret_cast<void**>(&gs))))
		return r;
	if ((r = staging_acquire(ctx, ctx->stage_prefix, (size_t(num_surfaces) + 1) * 8, reinterpret_cast<void**>(&prefix))))
		return r;
	uint64_t work = 0;
	uint32_t max_light = 0;
	if ((r = prepare_surfaces(ctx, surfaces, num_surfaces, total_texels, gs, prefix, &work, &max_light))) return r;
	ctx->h_prefix.assign(prefix, prefix + num_surfaces + 1);
	const uint32_t bpp = bpp_of(ctx->frame.pixel_format);
	if ((r = ensure(ctx, ctx->arena, std::max<uint64_t>(total_texels, 1) * bpp))) return r;
	if ((r = ensure(ctx, ctx->surfaces, std::max<size_t>(num_surfaces, 1) * sizeof(SurfaceGpu)))) return r;
	if ((r = ensure(ctx, ctx->work_prefix, (size_t(num_surfaces) + 1) * 8))) return r;
	if ((r = staging_commit(ctx, ctx->stage_surfaces, ctx->surfaces.ptr, num_surfaces * sizeof(SurfaceGpu)))) return r;
	if ((r = staging_commit(ctx, ctx->stage_prefix, ctx->work_prefix.ptr, (size_t(num_surfaces) + 1) * 8))) return r;
	note_surfaces(ctx, num_surfaces, total_texels, work, max_light);
	return launch_surfaces(ctx);
}

int sw_rebuild_surfaces(SwCtx* ctx)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open) return fail(ctx, SW_ERR_STATE, "sw_frame_begin must precede sw_rebuild_surfaces");
	if (ctx->last_surface_work == 0 && ctx->last_num_surfaces == 0) return fail(ctx, SW_ERR_STATE, "no surfaces submitted");
	if (ctx->frame.pixel_format != ctx->last_surface_format ||
		(ctx->frame.use_directional_lightmaps != 0) != ctx->last_surface_directional)
		return fail(ctx, SW_ERR_STATE, "frame format or lightmap kind changed since sw_submit_surfaces");
	if (ctx->last_max_light > ctx->num_lights) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "fewer lights than the surfaces use");
	if (!ctx->graph_enabled) return launch_surfaces(ctx);
	// the persistent launch as a CUDA graph, captured again only when its arguments change
	const SurfaceKernelArgs a = surface_args(ctx);
	const unsigned blocks = unsigned(ctx->tuning.surface_blocks_per_sm);
	if (!ctx->sexec || std::memcmp(&a, &ctx->skey, sizeof(a)) != 0 || blocks != ctx->sblocks)
	{
		if (ctx->sexec) cudaGraphExecDestroy(ctx->sexec);
		ctx->sexec = nullptr;
		SW_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
		const int lr = launch_surface_build(a, ctx->frame.pixel_format, ctx->num_sms, int(blocks), ctx->stream);
		cudaGraph_t g = nullptr;
		const cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
		if (lr || ee != cudaSuccess)
		{
			if (g) cudaGraphDestroy(g);
			cudaGetLastError();
			return lr ? check_kernel(ctx, lr, "surface build") : cuda_fail(ctx, ee, "cudaStreamEndCapture");
		}
		const cudaError_t ie = cudaGraphInstantiate(&ctx->sexec, g, 0);
		cudaGraphDestroy(g);
		if (ie != cudaSuccess)
		{
			ctx->sexec = nullptr;
			return cuda_fail(ctx, ie, "cudaGraphInstantiate");
		}
		ctx->skey = a;
		ctx->sblocks = blocks;
	}
	stage_begin(ctx, STAGE_SURFACES);
	SW_CUDA(ctx, cudaGraphLaunch(ctx->sexec, ctx->stream));
	stage_end(ctx, STAGE_SURFACES);
	ctx->arena_valid = true;
	ctx->stats.surfaces += ctx->last_num_surfaces;
	ctx->stats.surface_texels += ctx->last_surface_work;
	return SW_OK;
}

int sw_rebuild_surfaces_per_surface(SwCtx* ctx)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open) return fail(ctx, SW_ERR_STATE, "sw_frame_begin must precede sw_rebuild_surfaces_per_surface");
	if (ctx->h_prefix.size() != size_t(ctx->last_num_surfaces) + 1 || ctx->last_num_surfaces == 0)
		return fail(ctx, SW_ERR_STATE, "no surfaces submitted with sw_submit_surfaces");
	if (ctx->frame.pixel_format != ctx->last_surface_format ||
		(ctx->frame.use_directional_lightmaps != 0) != ctx->last_surface_directional)
		return fail(ctx, SW_ERR_STATE, "frame format or lightmap kind changed since sw_submit_surfaces");
	if (ctx->last_max_light > ctx->num_lights) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "fewer lights than the surfaces use");
	SurfaceKernelArgs a = surface_args(ctx);
	stage_begin(ctx, STAGE_SURFACES);
	for (uint32_t i = 0; i < ctx->last_num_surfaces; ++i)
	{
		// surface i's texels [prefix[i], prefix[i + 1]), a grid of its own
		a.work_begin = ctx->h_prefix[i];
		a.total_work = ctx->h_prefix[i + 1];
		const int lr = launch_surface_build(a, ctx->frame.pixel_format, ctx->num_sms, 1 << 20, ctx->stream);
		if (lr) return check_kernel(ctx, lr, "surface build");
	}
	stage_end(ctx, STAGE_SURFACES);
	ctx->arena_valid = true;
	ctx->stats.surfaces += ctx->last_num_surfaces;
	ctx->stats.surface_texels += ctx->last_surface_work;
	return SW_OK;
}

int sw_set_skybox(SwCtx* ctx, const uint32_t* texels32, const uint64_t* texels64, uint64_t num_texels)
{
	if (!ctx || (num_texels && (!texels32 || !texels64))) return SW_ERR_INVALID_ARGUMENT;
	if (num_texels > (uint64_t(1) << 32)) return fail(ctx, SW_ERR_LIMIT, "skybox too large");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	// frames in flight may read the old texels
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
	int r;
	if ((r = upload_static(ctx, ctx->skybox32, texels32, size_t(num_texels) * 4))) return r;
	if ((r = upload_static(ctx, ctx->skybox64, texels64, size_t(num_texels) * 8))) return r;
	ctx->skybox_texels = num_texels;
	return SW_OK;
}

int sw_register_host_buffer(SwCtx* ctx, void* ptr, uint64_t bytes)
{
	if (!ctx || !ptr || bytes == 0) return SW_ERR_INVALID_ARGUMENT;
	char* p = static_cast<char*>(ptr);
	for (const SwCtx::HostRange& h : ctx->registered)
		if (p < h.ptr + h.bytes && h.ptr < p + bytes) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "buffer overlaps a registered one");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaHostRegister(ptr, size_t(bytes), cudaHostRegisterMapped | cudaHostRegisterPortable));
	ctx->registered.push_back(SwCtx::HostRange{p, size_t(bytes)});
	return SW_OK;
}

int sw_unregister_host_buffer(SwCtx* ctx, void* ptr)
{
	if (!ctx || !ptr) return SW_ERR_INVALID_ARGUMENT;
	for (size_t i = 0; i < ctx->registered.size(); ++i)
		if (ctx->registered[i].ptr == ptr)
		{
			SW_CUDA(ctx, cudaSetDevice(ctx->device));
			// copies into it may still be in flight
			SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
			SW_CUDA(ctx, cudaHostUnregister(ptr));
			ctx->registered.erase(ctx->registered.begin() + long(i));
			return SW_OK;
		}
	return fail(ctx, SW_ERR_INVALID_ARGUMENT, "buffer not registered");
}

int sw_set_surfaces(SwCtx* ctx, const void* texels, uint64_t total_texels)
{
	if (!ctx || (total_texels && !texels)) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open) return fail(ctx, SW_ERR_STATE, "sw_frame_begin must precede sw_set_surfaces");
	const uint32_t bpp = bpp_of(ctx->frame.pixel_format);
	int r;
	if ((r = ensure(ctx, ctx->arena, std::max<uint64_t>(total_texels, 1) * bpp))) return r;
	if ((r = upload(ctx, ctx->stage_io, ctx->arena.ptr, texels, total_texels * bpp))) return r;
	ctx->arena_texels = total_texels;
	ctx->arena_format = ctx->frame.pixel_format;
	ctx->arena_view = false;
	ctx->arena_valid = true;
	return SW_OK;
}

namespace
{
// Host side of sw_submit_draws: validate every draw against its vertices and the surface arena, and
// compute the rows each draw can cover (row records are numbered in draw order).
int prepare_draws(SwCtx* ctx, const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	DrawRows* rows, uint64_t* out_rows, const SwTriVertex* tri_vertices = nullptr, uint32_t num_tri_vertices = 0,
	const SwView* views = nullptr, uint32_t num_views = 0)
{
	// rows are clipped to the height of the target a draw is rasterised into: the frame, or its view's
	std::vector<int32_t> view_height;
	if (num_views)
	{
		view_height.assign(num_draws, int32_t(ctx->frame.height));
		for (uint32_t v = 0; v < num_views; ++v)
			for (uint32_t i = views[v].first_draw; i < views[v].first_draw + views[v].num_draws && i < num_draws; ++i)
				view_height[i] = int32_t(views[v].height);
	}
	uint64_t row_acc = 0;
	for (uint32_t i = 0; i < num_draws; ++i)
	{
		const SwDrawCmd& d = draws[i];
		const int32_t clip_height = num_views ? view_height[i] : int32_t(ctx->frame.height);
		if (d.mode == SW_RASTER_TRIANGLE)
		{
			// Rasterizer::fill_triangle: three SwTriVertex, a Color32 texture of sw_set_lite_textures
			if (d.vertex_count != 3 || uint64_t(d.first_vertex) + 3 > num_tri_vertices)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: triangle vertices out of range", i);
			if (d.blend > SW_BLEND_ALPHA_BLEND) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: bad mode/blend", i);
			if (d.tex_source != SW_TEXSRC_LITE)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: a triangle needs a texture source of sw_set_lite_textures", i);
			const uint64_t area = uint64_t(d.tex_size[0]) * d.tex_size[1];
			if (d.tex_size[0] == 0 || d.tex_size[1] == 0 || d.tex_size[0] > 32768 || d.tex_size[1] > 32768 ||
				d.tex_offset > ctx->lite_texels || area > ctx->lite_texels - d.tex_offset)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: texture outside the lite textures", i);
			int32_t y0;
			uint32_t nrows;
			draw_row_range(d, vertices, clip_height, y0, nrows, tri_vertices);
			rows[i] = DrawRows{uint32_t(row_acc), y0, nrows, 0u};
			row_acc += nrows;
			if (row_acc > 0xFFFFFFFFull) return fail(ctx, SW_ERR_LIMIT, "too many draw rows in one frame");
			continue;
		}
		if (d.vertex_count < 3 || d.vertex_count > SW_MAX_POLYGON_VERTICES)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: bad vertex count", i);
		if (uint64_t(d.first_vertex) + d.vertex_count > num_vertices)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: vertices out of range", i);
		if (d.mode > SW_RASTER_AFFINE || d.blend > SW_BLEND_ALPHA_BLEND)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: bad mode/blend", i);
		if (d.tex_source > SW_TEXSRC_SKYBOX) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: bad texture source", i);
		const uint64_t limit = d.tex_source == SW_TEXSRC_SKYBOX ? ctx->skybox_texels : ctx->arena_texels;
		const uint64_t area = uint64_t(d.tex_size[0]) * d.tex_size[1];
		if (d.tex_size[0] == 0 || d.tex_size[1] == 0 || d.tex_offset > limit || area > limit - d.tex_offset)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: texture outside the %s", i,
				d.tex_source == SW_TEXSRC_SKYBOX ? "skybox texels" : "surface arena");
		int32_t y0;
		uint32_t nrows;
		draw_row_range(d, vertices, clip_height, y0, nrows);
		rows[i] = DrawRows{uint32_t(row_acc), y0, nrows, 0u};
		row_acc += nrows;
		if (row_acc > 0xFFFFFFFFull) return fail(ctx, SW_ERR_LIMIT, "too many draw rows in one frame");
	}
	*out_rows = row_acc;
	return SW_OK;
}

// Device buffers of the raster pass for num_draws draws, num_vertices vertices and `rows` row records.
int ensure_raster_buffers(SwCtx* ctx, uint32_t num_draws, uint32_t num_vertices, uint64_t rows, uint32_t num_tri_vertices = 0)
{
	int r;
	if ((r = ensure(ctx, ctx->draws, std::max<size_t>(num_draws, 1) * sizeof(SwDrawCmd)))) return r;
	if ((r = ensure(ctx, ctx->vertices, std::max<size_t>(num_vertices, 1) * sizeof(SwVertex16)))) return r;
	if ((r = ensure(ctx, ctx->tri_vertices, std::max<size_t>(num_tri_vertices, 1) * sizeof(SwTriVertex)))) return r;
	if ((r = ensure(ctx, ctx->draw_rows, std::max<size_t>(num_draws, 1) * sizeof(DrawRows)))) return r;
	if ((r = ensure(ctx, ctx->rdraws, std::max<size_t>(num_draws, 1) * sizeof(RasterDraw)))) return r;
	if ((r = ensure(ctx, ctx->rows, std::max<size_t>(rows, 1) * sizeof(RasterRow)))) return r;
	if ((r = ensure(ctx, ctx->boxes, std::max<size_t>(num_draws, 1) * sizeof(RasterBox)))) return r;
	if ((r = ensure(ctx, ctx->tri_steps, std::max<size_t>(num_draws, 1) * 2 * sizeof(TriSteps)))) return r;
	return SW_OK;
}
} // namespace

int sw_submit_draws(SwCtx* ctx, const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices)
{
	return sw_submit_draws_ex(ctx, draws, num_draws, vertices, num_vertices, nullptr, 0);
}

int sw_set_lite_textures(SwCtx* ctx, const uint32_t* pixels, uint64_t num_pixels)
{
	if (!ctx || (num_pixels && !pixels)) return SW_ERR_INVALID_ARGUMENT;
	if (num_pixels > (uint64_t(1) << 32)) return fail(ctx, SW_ERR_LIMIT, "lite textures too large");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	// frames in flight may read the old pixels
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
	int r;
	if ((r = upload_static(ctx, ctx->lite, pixels, num_pixels * 4))) return r;
	ctx->lite_texels = num_pixels;
	return SW_OK;
}

int sw_submit_draws_ex(SwCtx* ctx, const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	const SwTriVertex* tri_vertices, uint32_t num_tri_vertices)
{
	if (!ctx || (num_draws && !draws) || (num_vertices && !vertices) || (num_tri_vertices && !tri_vertices))
		return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open) return fail(ctx, SW_ERR_STATE, "sw_frame_begin must precede sw_submit_draws");
	if (!ctx->arena_valid && num_draws) return fail(ctx, SW_ERR_STATE, "sw_submit_surfaces must precede sw_submit_draws");
	int r;
	DrawRows* rows = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_draw_rows, std::max<size_t>(num_draws, 1) * sizeof(DrawRows),
			 reinterpret_cast<void**>(&rows))))
		return r;
	uint64_t row_acc = 0;
	if ((r = prepare_draws(ctx, draws, num_draws, vertices, num_vertices, rows, &row_acc, tri_vertices, num_tri_vertices)))
		return r;
	if ((r = ensure_raster_buffers(ctx, num_draws, num_vertices, row_acc, num_tri_vertices))) return r;
	if ((r = ensure_bins(ctx, ctx->frame.width, ctx->frame.height, num_draws))) return r;
	// The draw uploads and the raster setup run on the auxiliary stream, beside the surface build; they
	// first wait until the previous frame's tile pass has finished reading these buffers.
	if (ctx->tiles_recorded) SW_CUDA(ctx, cudaStreamWaitEvent(ctx->aux, ctx->ev_tiles, 0));
	if ((r = upload(ctx, ctx->stage_draws, ctx->draws.ptr, draws, num_draws * sizeof(SwDrawCmd), ctx->aux))) return r;
	if ((r = upload(ctx, ctx->stage_vertices, ctx->vertices.ptr, vertices, num_vertices * sizeof(SwVertex16), ctx->aux)))
		return r;
	if ((r = upload(ctx, ctx->stage_tri_vertices, ctx->tri_vertices.ptr, tri_vertices, num_tri_vertices * sizeof(SwTriVertex),
			 ctx->aux)))
		return r;
	if ((r = staging_commit(ctx, ctx->stage_draw_rows, ctx->draw_rows.ptr, num_draws * sizeof(DrawRows), ctx->aux))) return r;
	ctx->num_rows = row_acc;
	ctx->num_draws = num_draws;
	const RasterArgs a = raster_args(ctx);
	if ((r = check_kernel(ctx, launch_raster_setup(a, ctx->aux), "raster setup"))) return r;
	if ((r = check_kernel(ctx, launch_raster_bins(a, ctx->aux), "raster bins"))) return r;
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_setup, ctx->aux));
	ctx->draws_valid = true;
	ctx->stats.draws += num_draws;
	return SW_OK;
}

int sw_render(SwCtx* ctx, void* dst, uint32_t pitch, int dst_is_device)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->frame_open || !ctx->draws_valid) return fail(ctx, SW_ERR_STATE, "nothing submitted for this frame");
	if (ctx->num_draws && ctx->arena_format != ctx->frame.pixel_format)
		return fail(ctx, SW_ERR_STATE, "surface arena format differs from frame format");
	const uint32_t w = ctx->frame.width, h = ctx->frame.height, fmt = ctx->frame.pixel_format, bpp = bpp_of(fmt);
	if (dst && pitch < w) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "pitch < width");
	int r;
	if ((r = ensure(ctx, ctx->framebuffer, size_t(w) * h * bpp))) return r;
	if (!ctx->fb_valid || ctx->fb_width != w || ctx->fb_height != h || ctx->fb_format != fmt)
	{
		// A new frame buffer starts black, like a freshly allocated HDR buffer (postprocessor.rs:56-66).
		SW_CUDA(ctx, cudaMemsetAsync(ctx->framebuffer.ptr, 0, size_t(w) * h * bpp, ctx->stream));
		ctx->fb_width = w;
		ctx->fb_height = h;
		ctx->fb_format = fmt;
		ctx->fb_valid = true;
	}
	const RasterArgs a = raster_args(ctx);
	SW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_setup, 0));
	stage_begin(ctx, STAGE_RASTER);
	r = check_kernel(ctx, launch_raster_tiles(a, fmt, ctx->tuning.raster_tile, ctx->stream), "raster");
	stage_end(ctx, STAGE_RASTER);
	if (r) return r;
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_tiles, ctx->stream));
	ctx->tiles_recorded = true;
	ctx->frame_open = false;
	if (dst) return copy_out(ctx, dst, pitch, dst_is_device, ctx->framebuffer.ptr, w, w, h, bpp);
	return SW_OK;
}

int sw_set_framebuffer(SwCtx* ctx, const void* src, uint32_t width, uint32_t height, uint32_t pixel_format, int src_is_device)
{
	if (!ctx || !src || width == 0 || height == 0 || pixel_format > SW_PIXEL_C64) return SW_ERR_INVALID_ARGUMENT;
	const uint32_t bpp = bpp_of(pixel_format);
	const size_t bytes = size_t(width) * height * bpp;
	int r;
	if ((r = ensure(ctx, ctx->framebuffer, bytes))) return r;
	if (src_is_device)
		SW_CUDA(ctx, cudaMemcpyAsync(ctx->framebuffer.ptr, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
	else if ((r = upload(ctx, ctx->stage_io, ctx->framebuffer.ptr, src, bytes)))
		return r;
	ctx->fb_width = width;
	ctx->fb_height = height;
	ctx->fb_format = pixel_format;
	ctx->fb_valid = true;
	return SW_OK;
}

namespace
{
// Postprocessor arguments for the context's colour64 frame buffer (everything but the destination):
// tonemapping factors from the current exposure and colour modulation, bloom kernel weights, scratch
// buffers, from the configuration as synchronize_config clamps it. Runs finalize_exposure first (the
// previous frame's average updates the exposure).
int prepare_post(SwCtx* ctx, const SwPostConfig* config, const float color_modulate[3], PostArgs& a)
{
	const uint32_t w = ctx->fb_width, h = ctx->fb_height;
	int r;
	if ((r = finalize_exposure(ctx))) return r;

	std::memset(&a, 0, sizeof(a));
	a.hdr = static_cast<const uint64_t*>(ctx->framebuffer.ptr);
	a.average = static_cast<float*>(ctx->average.ptr);
	if (!post_args_from_config(a, post_config_clamped(*config), ctx->exposure, color_modulate, w, h))
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "frame too small for bloom");
	if (a.use_bloom)
	{
		if ((r = ensure(ctx, ctx->bloom0, size_t(a.bw) * a.bh * 8))) return r;
		if ((r = ensure(ctx, ctx->bloom1, size_t(a.bw) * a.bh * 8))) return r;
		if ((r = ensure(ctx, ctx->line_sums, size_t(a.bh) * 16))) return r;
		a.bloom0 = static_cast<uint64_t*>(ctx->bloom0.ptr);
		a.bloom1 = static_cast<uint64_t*>(ctx->bloom1.ptr);
		a.line_sums = static_cast<int32_t*>(ctx->line_sums.ptr);
	}
	else
	{
		if ((r = ensure(ctx, ctx->line_sums_f, size_t(h) * 16))) return r;
		a.line_sums_f = static_cast<float*>(ctx->line_sums_f.ptr);
	}
	return SW_OK;
}
} // namespace

int sw_postprocess(SwCtx* ctx, const SwPostConfig* config, float frame_duration_s, const float color_modulate[3], void* dst,
	uint32_t pitch, int dst_is_device)
{
	if (!ctx || !config || !color_modulate || !dst) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->fb_valid || ctx->fb_format != SW_PIXEL_C64)
		return fail(ctx, SW_ERR_STATE, "postprocessing needs a colour64 frame");
	const uint32_t w = ctx->fb_width, h = ctx->fb_height;
	if (pitch < w) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "pitch < width");
	int r;
	PostArgs a;
	if ((r = prepare_post(ctx, config, color_modulate, a))) return r;
	void* out = dst;
	uint32_t out_pitch = pitch;
	if (!dst_is_device)
	{
		if ((r = ensure(ctx, ctx->up_dst, size_t(w) * h * 4))) return r;
		out = ctx->up_dst.ptr;
		out_pitch = w;
	}
	a.dst = static_cast<uint32_t*>(out);
	a.dst_pitch = out_pitch;
	stage_begin(ctx, STAGE_POST);
	r = check_kernel(ctx, launch_postprocess(a, ctx->num_sms, ctx->stream, ctx->aux, ctx->ev_fork, ctx->ev_join),
		"postprocess");
	stage_end(ctx, STAGE_POST);
	if (r) return r;
	SW_CUDA(ctx, cudaMemcpyAsync(ctx->h_average, ctx->average.ptr, 16, cudaMemcpyDeviceToHost, ctx->stream));
	SW_CUDA(ctx, cudaEventRecord(ctx->average_ready, ctx->stream));
	stage_end(ctx, STAGE_FRAME);
	ctx->exposure_pending = true;
	ctx->pending_config = post_config_clamped(*config);
	ctx->pending_dt = frame_duration_s;
	if (!dst_is_device) return copy_out(ctx, dst, pitch, 0, out, w, w, h, 4);
	return SW_OK;
}

int sw_upscale(SwCtx* ctx, uint32_t mode, uint32_t scale, const void* src, int src_is_device, void* dst, uint32_t dst_width,
	uint32_t dst_height, uint32_t dst_pitch, int dst_is_device)
{
	if (!ctx || !src || !dst || dst_pitch < dst_width) return SW_ERR_INVALID_ARGUMENT;
	if (mode == SW_UPSCALE_LEARNED)
	{
		if (!ctx->learned) return fail(ctx, SW_ERR_STATE, "no learned upscaler attached (sw_set_learned_upscaler)");
		if (scale != 2 || (dst_width & 1) || (dst_height & 1))
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "the learned upscaler doubles both sides (scale 2, even size)");
	}
	if (mode == SW_UPSCALE_AVG2X || mode == SW_UPSCALE_LEARNED)
		scale = 2;
	else if (mode != SW_UPSCALE_NEAREST || scale < 1 || scale > 6)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "bad upscale mode/scale");
	const uint32_t sw = dst_width / scale, sh = dst_height / scale;
	if (sw < 1 || sh < 1 || (mode == SW_UPSCALE_AVG2X && (sw < 2 || sh < 2)))
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "frame too small");
	int r;
	const void* s = src;
	if (!src_is_device)
	{
		if ((r = ensure(ctx, ctx->up_src, size_t(sw) * sh * 4))) return r;
		if ((r = upload(ctx, ctx->stage_io, ctx->up_src.ptr, src, size_t(sw) * sh * 4))) return r;
		s = ctx->up_src.ptr;
	}
	void* d = dst;
	uint32_t dp = dst_pitch;
	if (!dst_is_device || (mode == SW_UPSCALE_LEARNED && ((dst_pitch & 1) || (reinterpret_cast<uintptr_t>(dst) & 7))))
	{
		if ((r = ensure(ctx, ctx->up_dst, size_t(dst_width) * dst_height * 4))) return r;
		d = ctx->up_dst.ptr;
		dp = dst_width;
	}
	stage_begin(ctx, STAGE_UPSCALE);
	if (mode == SW_UPSCALE_LEARNED)
	{
		r = sw_upscaler_infer(ctx->learned, static_cast<const uint32_t*>(s), sw, sh, sw, static_cast<uint32_t*>(d), dp, ctx->stream);
		if (r) r = fail(ctx, r, "learned upscale: %s", sw_upscaler_last_error(ctx->learned));
	}
	else
		r = check_kernel(ctx,
			launch_upscale(mode, scale, static_cast<const uint32_t*>(s), static_cast<uint32_t*>(d), dst_width, dst_height, dp,
				ctx->stream),
			"upscale");
	stage_end(ctx, STAGE_UPSCALE);
	if (!r && dst_is_device && d != dst)
		r = copy_out(ctx, dst, dst_pitch, 1, d, dp, dst_width, dst_height, 4);
	if (r) return r;
	if (!dst_is_device) return copy_out(ctx, dst, dst_pitch, 0, d, dp, dst_width, dst_height, 4);
	return SW_OK;
}

int sw_set_learned_upscaler(SwCtx* ctx, SwUpscaler* ups)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	ctx->learned = ups;
	return SW_OK;
}

int sw_read_surfaces(SwCtx* ctx, void* dst_host, uint64_t max_bytes)
{
	if (!ctx || !dst_host) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->arena_valid && ctx->arena_texels == 0) return fail(ctx, SW_ERR_STATE, "no surfaces built");
	uint64_t texels = ctx->arena_texels;
	if (ctx->arena_view && ctx->v_counts)
	{
		// a view frame's arena is sized by a bound: the frame's own texels are counted on the device
		SwViewCounts k;
		SW_CUDA(ctx, cudaMemcpyAsync(&k, ctx->v_counts, sizeof(k), cudaMemcpyDeviceToHost, ctx->stream));
		SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
		texels = std::min<uint64_t>(k.total_texels, ctx->arena_texels);
	}
	const uint64_t bytes = texels * bpp_of(ctx->arena_format);
	if (bytes > max_bytes) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "destination too small (%llu bytes needed)", (unsigned long long)bytes);
	SW_CUDA(ctx, cudaMemcpyAsync(dst_host, ctx->arena.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	return SW_OK;
}

int sw_read_framebuffer(SwCtx* ctx, void* dst_host, uint64_t max_bytes)
{
	if (!ctx || !dst_host) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->fb_valid) return fail(ctx, SW_ERR_STATE, "no frame rendered");
	const uint64_t bytes = uint64_t(ctx->fb_width) * ctx->fb_height * bpp_of(ctx->fb_format);
	if (bytes > max_bytes) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "destination too small (%llu bytes needed)", (unsigned long long)bytes);
	SW_CUDA(ctx, cudaMemcpyAsync(dst_host, ctx->framebuffer.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	return SW_OK;
}

int sw_update_textures(SwCtx* ctx, const SwTexturePass* passes, uint32_t num_passes, const int32_t* shifts,
	uint32_t num_shifts)
{
	if (!ctx || (num_passes && !passes) || (num_shifts && !shifts)) return SW_ERR_INVALID_ARGUMENT;
	if (num_passes == 0) return SW_OK;
	if (num_passes > (1u << 20) || num_shifts > (1u << 26)) return fail(ctx, SW_ERR_LIMIT, "too many texture passes or shifts");
	const std::vector<SwTextureMip>& tm = ctx->h_texture_mips;
	const std::vector<SwEmissiveMip>& em = ctx->h_emissive_mips;
	std::vector<TextureEffectGroup> groups;
	std::vector<TextureEffectLayer> layers(num_passes);
	// destinations (index | emissive bit 31) of the groups, and every source, for the race checks
	std::vector<uint32_t> dsts, srcs;
	uint64_t total = 0;
	for (uint32_t p = 0; p < num_passes;)
	{
		const SwTexturePass& a = passes[p];
		const bool emissive = (a.kind & SW_TEXPASS_EMISSIVE) != 0;
		const uint32_t kind = a.kind & ~SW_TEXPASS_EMISSIVE;
		TextureEffectGroup g;
		std::memset(&g, 0, sizeof(g));
		g.first_pass = p;
		g.first_texel = total;
		if (kind == SW_TEXPASS_TURB)
		{
			const size_t n = emissive ? em.size() : tm.size();
			if (a.dst_mip >= n || a.src_mip >= n || a.dst_mip == a.src_mip)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: bad mip", p);
			const uint32_t w = emissive ? em[a.dst_mip].width : tm[a.dst_mip].width;
			const uint32_t h = emissive ? em[a.dst_mip].height : tm[a.dst_mip].height;
			const uint32_t sw = emissive ? em[a.src_mip].width : tm[a.src_mip].width;
			const uint32_t sh = emissive ? em[a.src_mip].height : tm[a.src_mip].height;
			if (w == 0 || h == 0 || (w & (w - 1)) || (h & (h - 1)) || w != sw || h != sh)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: turbulence needs equal power-of-two sizes", p);
			if (uint64_t(a.shifts_offset) + std::max(w, h) > num_shifts)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: shifts out of range", p);
			g.width = w;
			g.height = h;
			g.dst_offset = emissive ? em[a.dst_mip].offset : tm[a.dst_mip].offset;
			g.src_offset = emissive ? em[a.src_mip].offset : tm[a.src_mip].offset;
			g.num_passes = 1;
			dsts.push_back(a.dst_mip | (emissive ? 0x80000000u : 0u));
			srcs.push_back(a.src_mip | (emissive ? 0x80000000u : 0u));
			++p;
		}
		else if (kind == SW_TEXPASS_LAYER && !emissive)
		{
			if (a.dst_mip >= tm.size()) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: bad mip", p);
			g.width = tm[a.dst_mip].width;
			g.height = tm[a.dst_mip].height;
			g.dst_offset = tm[a.dst_mip].offset;
			dsts.push_back(a.dst_mip);
			uint32_t q = p;
			for (; q < num_passes && passes[q].kind == SW_TEXPASS_LAYER && passes[q].dst_mip == a.dst_mip; ++q)
			{
				const SwTexturePass& l = passes[q];
				if (l.src_mip >= tm.size() || tm[l.src_mip].width == 0 || tm[l.src_mip].height == 0 ||
					tm[l.src_mip].width > (1u << 16) || tm[l.src_mip].height > (1u << 16))
					return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: bad layer mip", q);
				if (l.blending_mode > SW_BLEND_ALPHA_BLEND) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: bad blending mode", q);
				bool modulate = false, zero = true;
				for (int c = 0; c < 3; ++c)
				{
					const float v = l.light[c];
					if (!(v >= 0.0f && v <= 127.0f)) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: light outside [0, 127]", q);
					modulate |= v < 0.98f || v > 1.02f;
					zero &= v <= 1.0f / 128.0f;
				}
				TextureEffectLayer& L = layers[q];
				L.src_offset = tm[l.src_mip].offset;
				L.src_width = tm[l.src_mip].width;
				L.src_height = tm[l.src_mip].height;
				L.modulate = modulate ? 1u : 0u;
				L.skip = (l.blending_mode == SW_BLEND_ADDITIVE && zero) ? 1u : 0u;
				// ColorVecI::from_color_f32x3 of light * 256: lanes b, g, r (f32 -> i32 truncation)
				L.light[0] = int32_t(l.light[2] * 256.0f);
				L.light[1] = int32_t(l.light[1] * 256.0f);
				L.light[2] = int32_t(l.light[0] * 256.0f);
				srcs.push_back(l.src_mip);
			}
			g.num_passes = q - p;
			p = q;
		}
		else
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "texture pass %u: unknown kind", p);
		total += uint64_t(g.width) * g.height;
		groups.push_back(g);
	}
	std::vector<uint32_t> sorted = dsts;
	std::sort(sorted.begin(), sorted.end());
	if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "two texture pass groups write the same mip");
	for (uint32_t s : srcs)
		if (std::binary_search(sorted.begin(), sorted.end(), s))
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "a texture pass reads a mip that another pass writes");
	// one upload: groups | layers | passes | shifts
	auto up16 = [](size_t v) { return (v + 15) / 16 * 16; };
	const size_t o_layers = up16(groups.size() * sizeof(TextureEffectGroup));
	const size_t o_passes = o_layers + up16(layers.size() * sizeof(TextureEffectLayer));
	const size_t o_shifts = o_passes + up16(size_t(num_passes) * sizeof(SwTexturePass));
	const size_t bytes = o_shifts + up16(size_t(num_shifts) * 4 + 4);
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	int r;
	if ((r = ensure(ctx, ctx->effect_buf, bytes))) return r;
	void* h = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_effects, bytes, &h))) return r;
	unsigned char* hb = static_cast<unsigned char*>(h);
	std::memcpy(hb, groups.data(), groups.size() * sizeof(TextureEffectGroup));
	std::memcpy(hb + o_layers, layers.data(), layers.size() * sizeof(TextureEffectLayer));
	std::memcpy(hb + o_passes, passes, size_t(num_passes) * sizeof(SwTexturePass));
	if (num_shifts) std::memcpy(hb + o_shifts, shifts, size_t(num_shifts) * 4);
	if ((r = staging_commit(ctx, ctx->stage_effects, ctx->effect_buf.ptr, bytes))) return r;
	unsigned char* d = static_cast<unsigned char*>(ctx->effect_buf.ptr);
	TextureEffectArgs a;
	std::memset(&a, 0, sizeof(a));
	a.groups = reinterpret_cast<const TextureEffectGroup*>(d);
	a.layers = reinterpret_cast<const TextureEffectLayer*>(d + o_layers);
	a.passes = reinterpret_cast<const SwTexturePass*>(d + o_passes);
	a.shifts = reinterpret_cast<const int32_t*>(d + o_shifts);
	a.num_groups = uint32_t(groups.size());
	a.total_texels = total;
	a.texels = static_cast<uint64_t*>(ctx->texels.ptr);
	a.emissive = static_cast<uint32_t*>(ctx->emissive.ptr);
	return check_kernel(ctx, launch_texture_effects(a, ctx->stream), "texture effects");
}

int sw_reserve_simulation_state(SwCtx* ctx, uint64_t words)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	if (words > (1ull << 32)) return fail(ctx, SW_ERR_LIMIT, "simulation state above 2^32 words");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
	if (words * 4 > ctx->sim_state.bytes)
	{
		release(ctx->sim_state);
		int r = ensure(ctx, ctx->sim_state, size_t(words) * 4);
		if (r) return r;
	}
	ctx->sim_words = words;
	if (words) SW_CUDA(ctx, cudaMemsetAsync(ctx->sim_state.ptr, 0, size_t(words) * 4, ctx->stream));
	return SW_OK;
}

int sw_update_simulations(SwCtx* ctx, const SwSimPass* passes, uint32_t num_passes, const SwSimPoint* points,
	uint32_t num_points)
{
	if (!ctx || (num_passes && !passes) || (num_points && !points)) return SW_ERR_INVALID_ARGUMENT;
	if (num_passes == 0) return SW_OK;
	if (num_passes > (1u << 20) || num_points > (1u << 26)) return fail(ctx, SW_ERR_LIMIT, "too many simulation passes or points");
	const std::vector<SwTextureMip>& tm = ctx->h_texture_mips;
	const std::vector<SwEmissiveMip>& em = ctx->h_emissive_mips;
	std::vector<SimGroup> groups(num_passes);
	std::vector<uint32_t> launch_first; // first group of each launch
	std::vector<uint64_t> launch_items;
	uint64_t items = 0;
	for (uint32_t p = 0; p < num_passes; ++p)
	{
		const SwSimPass& a = passes[p];
		if (p > 0 && a.launch < passes[p - 1].launch) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: launches out of order", p);
		if (p == 0 || a.launch != passes[p - 1].launch)
		{
			if (p > 0) launch_items.push_back(items);
			launch_first.push_back(p);
			items = 0;
		}
		SimGroup& g = groups[p];
		std::memset(&g, 0, sizeof(g));
		g.pass = p;
		g.first_item = items;
		const bool mip_pass = a.kind == SW_SIM_TEXTURE_MIP || a.kind == SW_SIM_EMISSIVE_MIP;
		if (!mip_pass && (a.size_log2[0] < 2 || a.size_log2[1] < 2 || a.size_log2[0] + a.size_log2[1] > 24))
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: field size out of range", p);
		const uint64_t area = mip_pass ? 0 : (1ull << (a.size_log2[0] + a.size_log2[1]));
		auto in_state = [&](uint64_t off) { return off <= ctx->sim_words && area <= ctx->sim_words - off; };
		auto points_ok = [&](uint64_t need) {
			return uint64_t(a.first_point) + a.num_points <= num_points && (need == 0 || a.num_points == need);
		};
		uint64_t n = 0;
		switch (a.kind)
		{
		case SW_SIM_WATER_POINTS:
		case SW_SIM_FIRE_POINTS:
			if (!in_state(a.state_dst) || (a.kind == SW_SIM_WATER_POINTS && !in_state(a.state_src)) || !points_ok(0))
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: state or points out of range", p);
			for (uint32_t i = 0; i < a.num_points; ++i)
				if (points[a.first_point + i].address >= area)
					return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: point %u outside the field", p, i);
			n = a.num_points;
			break;
		case SW_SIM_WATER_STEP:
		case SW_SIM_FIRE_STEP:
			if (!in_state(a.state_src) || !in_state(a.state_dst) || a.state_src == a.state_dst)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: state out of range", p);
			if (a.kind == SW_SIM_FIRE_STEP && a.param > (1u << 18))
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: attenuation above 2^18", p);
			n = (a.kind == SW_SIM_FIRE_STEP && (a.flags & SW_SIM_FIRE_SLOW)) ? (1ull << a.size_log2[1]) : area;
			break;
		case SW_SIM_WATER_TEXTURE:
		case SW_SIM_FIRE_TEXTURE:
		{
			const bool water = a.kind == SW_SIM_WATER_TEXTURE;
			const size_t nm = water ? tm.size() : em.size();
			if (!in_state(a.state_src) || a.dst_mip >= nm || (water && (a.src_mip >= tm.size() || a.src_mip == a.dst_mip)) ||
				(!water && !points_ok(256)) || (water && (a.flags >> SW_SIM_COLOR_MODE_SHIFT) > 3))
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: state, mips, palette or colour mode out of range", p);
			const uint32_t w = water ? tm[a.dst_mip].width : em[a.dst_mip].width;
			const uint32_t h = water ? tm[a.dst_mip].height : em[a.dst_mip].height;
			if (w != (1u << a.size_log2[0]) || h != (1u << a.size_log2[1]))
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: output mip is not the field's size", p);
			g.dst_offset = water ? tm[a.dst_mip].offset : em[a.dst_mip].offset;
			if (water)
			{
				const SwTextureMip& s = tm[a.src_mip];
				if (s.width == 0 || s.height == 0 || s.width > (1u << 16) || s.height > (1u << 16))
					return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: bad colour source mip", p);
				g.src_offset = s.offset;
				g.src_width = s.width;
				g.src_height = s.height;
			}
			n = area;
			break;
		}
		case SW_SIM_TEXTURE_MIP:
		case SW_SIM_EMISSIVE_MIP:
		{
			const bool lite = a.kind == SW_SIM_EMISSIVE_MIP;
			const size_t nm = lite ? em.size() : tm.size();
			if (a.dst_mip >= nm || a.src_mip >= nm || a.dst_mip == a.src_mip)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: bad mip", p);
			const uint32_t sw = lite ? em[a.src_mip].width : tm[a.src_mip].width, sh = lite ? em[a.src_mip].height : tm[a.src_mip].height;
			const uint32_t dw = lite ? em[a.dst_mip].width : tm[a.dst_mip].width, dh = lite ? em[a.dst_mip].height : tm[a.dst_mip].height;
			if (dw != sw >> 1 || dh != sh >> 1 || dw == 0 || dh == 0)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: destination is not half the source", p);
			g.dst_offset = lite ? em[a.dst_mip].offset : tm[a.dst_mip].offset;
			g.src_offset = lite ? em[a.src_mip].offset : tm[a.src_mip].offset;
			g.src_width = sw;
			g.src_height = sh;
			n = uint64_t(dw) * dh;
			break;
		}
		default:
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "simulation pass %u: unknown kind", p);
		}
		items += n;
	}
	launch_items.push_back(items);
	// one upload: groups | passes | points
	auto up16 = [](size_t v) { return (v + 15) / 16 * 16; };
	const size_t o_passes = up16(groups.size() * sizeof(SimGroup));
	const size_t o_points = o_passes + up16(size_t(num_passes) * sizeof(SwSimPass));
	const size_t bytes = o_points + up16(size_t(num_points) * sizeof(SwSimPoint) + 8);
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	int r;
	if ((r = ensure(ctx, ctx->sim_buf, bytes))) return r;
	void* h = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_sims, bytes, &h))) return r;
	unsigned char* hb = static_cast<unsigned char*>(h);
	std::memcpy(hb, groups.data(), groups.size() * sizeof(SimGroup));
	std::memcpy(hb + o_passes, passes, size_t(num_passes) * sizeof(SwSimPass));
	if (num_points) std::memcpy(hb + o_points, points, size_t(num_points) * sizeof(SwSimPoint));
	if ((r = staging_commit(ctx, ctx->stage_sims, ctx->sim_buf.ptr, bytes))) return r;
	unsigned char* d = static_cast<unsigned char*>(ctx->sim_buf.ptr);
	for (size_t l = 0; l < launch_first.size(); ++l)
	{
		SimArgs a;
		std::memset(&a, 0, sizeof(a));
		const uint32_t first = launch_first[l];
		const uint32_t end = l + 1 < launch_first.size() ? launch_first[l + 1] : num_passes;
		a.groups = reinterpret_cast<const SimGroup*>(d) + first;
		a.passes = reinterpret_cast<const SwSimPass*>(d + o_passes);
		a.points = reinterpret_cast<const SwSimPoint*>(d + o_points);
		a.num_groups = end - first;
		a.total_items = launch_items[l];
		a.state = static_cast<uint32_t*>(ctx->sim_state.ptr);
		a.texels = static_cast<uint64_t*>(ctx->texels.ptr);
		a.emissive = static_cast<uint32_t*>(ctx->emissive.ptr);
		if ((r = check_kernel(ctx, launch_simulation(a, ctx->stream), "simulation"))) return r;
	}
	return SW_OK;
}

int sw_read_simulation_state(SwCtx* ctx, uint64_t first, uint64_t count, uint32_t* out)
{
	if (!ctx || (count && !out)) return SW_ERR_INVALID_ARGUMENT;
	if (first > ctx->sim_words || count > ctx->sim_words - first)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "range outside the simulation state (%llu words)", (unsigned long long)ctx->sim_words);
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (count) SW_CUDA(ctx, cudaMemcpy(out, static_cast<uint32_t*>(ctx->sim_state.ptr) + first, count * 4, cudaMemcpyDeviceToHost));
	return SW_OK;
}

int sw_set_lightmaps_compressed(SwCtx* ctx, const void* lightmaps, uint64_t num_elements, const void* directional,
	uint64_t num_directional_elements)
{
	if (!ctx || (num_elements && !lightmaps) || (num_directional_elements && !directional)) return SW_ERR_INVALID_ARGUMENT;
	if (num_elements > (1ull << 31) || num_directional_elements > (1ull << 31))
		return fail(ctx, SW_ERR_LIMIT, "too many lightmap elements");
	// the map's polygons (sw_set_map) must still read inside the lightmaps
	const uint64_t end = ctx->map_lightmap_end;
	if ((num_elements > 1 && num_elements < end) || (num_directional_elements > 1 && num_directional_elements < end))
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "lightmaps shorter than the map's polygons read (%llu elements)",
			(unsigned long long)end);
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	// frames in flight may still read the lightmaps being replaced
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
	if (ctx->copy) SW_CUDA(ctx, cudaStreamSynchronize(ctx->copy));
	const size_t simple_bytes = size_t(num_elements) * SW_LIGHTMAP_COMPRESSED_BYTES, dir_at = (simple_bytes + 255) / 256 * 256;
	const size_t dir_bytes = size_t(num_directional_elements) * SW_DIR_LIGHTMAP_COMPRESSED_BYTES;
	int r;
	if ((r = ensure(ctx, ctx->lm_compressed, dir_at + dir_bytes + 16))) return r;
	if ((r = ensure(ctx, ctx->lightmaps, std::max<size_t>(num_elements * 12, 16)))) return r;
	if ((r = ensure(ctx, ctx->dir_lightmaps, std::max<size_t>(num_directional_elements * sizeof(SwDirectionalLightmapElement), 16))))
		return r;
	unsigned char* staged = static_cast<unsigned char*>(ctx->lm_compressed.ptr);
	if (simple_bytes) SW_CUDA(ctx, cudaMemcpy(staged, lightmaps, simple_bytes, cudaMemcpyHostToDevice));
	if (dir_bytes) SW_CUDA(ctx, cudaMemcpy(staged + dir_at, directional, dir_bytes, cudaMemcpyHostToDevice));
	if ((r = check_kernel(ctx,
			 launch_lightmap_decompress(staged, num_elements, static_cast<float*>(ctx->lightmaps.ptr), staged + dir_at,
				 num_directional_elements, static_cast<SwDirectionalLightmapElement*>(ctx->dir_lightmaps.ptr), ctx->stream),
			 "lightmap decompression")))
		return r;
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	ctx->num_lightmap_elements = num_elements;
	ctx->num_dir_lightmap_elements = num_directional_elements;
	ctx->stats.upload_bytes += simple_bytes + dir_bytes;
	return SW_OK;
}

int sw_read_texels(SwCtx* ctx, uint64_t* texels, uint64_t max_texels, uint32_t* emissive, uint64_t max_emissive)
{
	if (!ctx || (max_texels && !texels) || (max_emissive && !emissive)) return SW_ERR_INVALID_ARGUMENT;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	const uint64_t n = std::min(max_texels, ctx->num_texels), ne = std::min(max_emissive, ctx->num_emissive_pixels);
	if (n) SW_CUDA(ctx, cudaMemcpy(texels, ctx->texels.ptr, n * 8, cudaMemcpyDeviceToHost));
	if (ne) SW_CUDA(ctx, cudaMemcpy(emissive, ctx->emissive.ptr, ne * 4, cudaMemcpyDeviceToHost));
	return SW_OK;
}

int sw_read_lightmaps(SwCtx* ctx, float* lightmaps, uint64_t max_elements, SwDirectionalLightmapElement* directional,
	uint64_t max_directional_elements)
{
	if (!ctx || (max_elements && !lightmaps) || (max_directional_elements && !directional)) return SW_ERR_INVALID_ARGUMENT;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	const uint64_t n = std::min(max_elements, ctx->num_lightmap_elements);
	const uint64_t nd = std::min(max_directional_elements, ctx->num_dir_lightmap_elements);
	if (n) SW_CUDA(ctx, cudaMemcpy(lightmaps, ctx->lightmaps.ptr, n * 12, cudaMemcpyDeviceToHost));
	if (nd) SW_CUDA(ctx, cudaMemcpy(directional, ctx->dir_lightmaps.ptr, nd * sizeof(SwDirectionalLightmapElement), cudaMemcpyDeviceToHost));
	return SW_OK;
}

int sw_get_exposure(SwCtx* ctx, float* out_exposure)
{
	if (!ctx || !out_exposure) return SW_ERR_INVALID_ARGUMENT;
	int r = finalize_exposure(ctx);
	if (r) return r;
	*out_exposure = ctx->exposure;
	return SW_OK;
}

int sw_set_exposure(SwCtx* ctx, float exposure)
{
	if (!ctx || !(exposure > 0.0f)) return SW_ERR_INVALID_ARGUMENT;
	int r = finalize_exposure(ctx);
	if (r) return r;
	ctx->exposure = exposure;
	return SW_OK;
}

namespace
{
size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// sw_draw_frame without a graph: the per-call API in order.
// Device work of one graph frame, issued on the context's streams while they are being captured.
// A graph frame with bloom: the raster tile pass writes the downscaled bloom buffer and the per-line
// sums (zeroed here, on the stream, before the pass), and the postprocess starts at the blur.
int fuse_bloom_downscale(SwCtx* ctx, RasterArgs& ra, PostArgs& pa, cudaStream_t s)
{
	if (!pa.use_bloom) return SW_OK;
	SW_CUDA(ctx, cudaMemsetAsync(pa.line_sums, 0, size_t(pa.bh) * 16, s));
	ra.bloom_out = pa.bloom0;
	ra.bloom_line_sums = pa.line_sums;
	ra.bloom_scale = pa.scale;
	ra.bloom_w = pa.bw;
	ra.bloom_h = pa.bh;
	pa.downscaled = 1;
	return SW_OK;
}

int enqueue_frame(SwCtx* ctx, const SwFrameInput& f, const unsigned char* h, const size_t* off, uint64_t rows,
	const PostArgs* post, cudaEvent_t average_done = nullptr)
{
	cudaStream_t s = ctx->stream, aux = ctx->aux;
	// every per-frame array in one copy: the device buffer has the staging block's layout
	unsigned char* d = static_cast<unsigned char*>(ctx->frame_in.ptr);
	SW_CUDA(ctx, cudaMemcpyAsync(d, h, off[7], cudaMemcpyHostToDevice, s));
	// raster setup on the auxiliary stream, beside the surface build
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_fork, s));
	SW_CUDA(ctx, cudaStreamWaitEvent(aux, ctx->ev_fork, 0));
	int r;
	RasterArgs ra = raster_args(ctx);
	ra.draws = reinterpret_cast<const SwDrawCmd*>(d + off[3]);
	ra.vertices = reinterpret_cast<const SwVertex16*>(d + off[4]);
	ra.draw_rows = reinterpret_cast<const DrawRows*>(d + off[5]);
	ra.tri_vertices = reinterpret_cast<const SwTriVertex*>(d + off[6]);
	ra.num_draws = f.num_views ? f.main_draws : f.num_draws; // the frame's own draws come first
	if ((r = check_kernel(ctx, launch_raster_setup(ra, aux), "raster setup"))) return r;
	if ((r = check_kernel(ctx, launch_raster_bins(ra, aux), "raster bins"))) return r;
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_setup, aux));
	const SurfaceInputs si{reinterpret_cast<const SwLight*>(d + off[0]), reinterpret_cast<const SurfaceGpu*>(d + off[1]),
		reinterpret_cast<const uint64_t*>(d + off[2])};
	if ((r = launch_surfaces(ctx, &si))) return r;
	// the nested views (portal textures), in order, into their arena regions: each cleared, rasterised
	// from its draws with its own setup, bins and tile pass, then mixed with its texture
	const uint32_t bpp = bpp_of(f.params.pixel_format);
	for (uint32_t i = 0; i < f.num_views; ++i)
	{
		const SwView& v = f.views[i];
		unsigned char* target = static_cast<unsigned char*>(ctx->arena.ptr) + v.target_offset * bpp;
		SW_CUDA(ctx, cudaMemsetAsync(target, 0, size_t(v.width) * v.height * bpp, s));
		if (v.num_draws || v.clear_background)
		{
			RasterArgs va = ra;
			va.draws = ra.draws + v.first_draw;
			va.draw_rows = ra.draw_rows + v.first_draw;
			va.rdraws = ra.rdraws + v.first_draw;
			va.boxes = ra.boxes + v.first_draw;
			va.tri_steps = ra.tri_steps + uint64_t(v.first_draw) * 2;
			va.num_draws = v.num_draws;
			va.width = int32_t(v.width);
			va.height = int32_t(v.height);
			va.clear_background = v.clear_background;
			va.framebuffer = target;
			va.bin_lists = static_cast<uint32_t*>(ctx->vbin_lists.ptr);
			va.bin_counts = static_cast<uint32_t*>(ctx->vbin_counts.ptr);
			va.bin_cap = ctx->vbin_cap;
			va.bins_x = raster_bins(int32_t(v.width), RASTER_BIN_W);
			va.bins_y = raster_bins(int32_t(v.height), RASTER_BIN_H);
			if (v.num_draws && (r = check_kernel(ctx, launch_raster_setup(va, s), "view raster setup"))) return r;
			if ((r = check_kernel(ctx, launch_raster_bins(va, s), "view raster bins"))) return r;
			if ((r = check_kernel(ctx, launch_raster_tiles(va, f.params.pixel_format, ctx->tuning.raster_tile, s), "view raster")))
				return r;
		}
		if (v.mix_blend != SW_VIEW_NO_MIX &&
			(r = check_kernel(ctx, launch_view_mix(v, target, static_cast<const uint32_t*>(ctx->lite.ptr), f.params.pixel_format, s),
				 "view texture mix")))
			return r;
	}
	SW_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_setup, 0));
	PostArgs pp;
	if (post)
	{
		pp = *post;
		if ((r = fuse_bloom_downscale(ctx, ra, pp, s))) return r;
	}
	stage_begin(ctx, STAGE_RASTER);
	r = check_kernel(ctx, launch_raster_tiles(ra, f.params.pixel_format, ctx->tuning.raster_tile, s), "raster");
	stage_end(ctx, STAGE_RASTER);
	if (r) return r;
	(void)rows;
	if (post)
	{
		stage_begin(ctx, STAGE_POST);
		r = check_kernel(ctx, launch_postprocess(pp, ctx->num_sms, s, aux, ctx->ev_fork, ctx->ev_join, average_done),
			"postprocess");
		stage_end(ctx, STAGE_POST);
		if (r) return r;
		if (!average_done) SW_CUDA(ctx, cudaMemcpyAsync(ctx->h_average, ctx->average.ptr, 16, cudaMemcpyDeviceToHost, s));
	}
	else if (f.dst && f.dst_is_device)
	{
		SW_CUDA(ctx, cudaMemcpy2DAsync(f.dst, size_t(f.dst_pitch) * bpp, ctx->framebuffer.ptr, size_t(f.params.width) * bpp,
						 size_t(f.params.width) * bpp, f.params.height, cudaMemcpyDeviceToDevice, s));
	}
	return SW_OK;
}
} // namespace

} // extern "C"

namespace
{
// The checks of sw_frame_begin for a whole-frame call.
int check_frame_params(SwCtx* ctx, const SwFrameParams& p, const SwLight* lights, uint32_t num_lights)
{
	if (p.pixel_format > SW_PIXEL_C64) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "bad pixel format");
	if (p.width == 0 || p.height == 0 || p.width > 16384 || p.height > 16384)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "bad frame size %ux%u", p.width, p.height);
	if (p.use_directional_lightmaps && ctx->num_dir_lightmap_elements == 0)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "directional lightmaps requested but none uploaded");
	if (num_lights > 65535) return fail(ctx, SW_ERR_LIMIT, "too many lights");
	return check_frame_inputs(ctx, p, lights, num_lights);
}

// The frame buffer of the frame's size and format; a new one starts black (postprocessor.rs:56-66),
// cleared before the graph.
int ensure_framebuffer(SwCtx* ctx, const SwFrameParams& p)
{
	const uint32_t bpp = bpp_of(p.pixel_format);
	int r;
	if ((r = ensure(ctx, ctx->framebuffer, size_t(p.width) * p.height * bpp))) return r;
	if (!ctx->fb_valid || ctx->fb_width != p.width || ctx->fb_height != p.height || ctx->fb_format != p.pixel_format)
	{
		SW_CUDA(ctx, cudaMemsetAsync(ctx->framebuffer.ptr, 0, size_t(p.width) * p.height * bpp, ctx->stream));
		ctx->fb_width = p.width;
		ctx->fb_height = p.height;
		ctx->fb_format = p.pixel_format;
		ctx->fb_valid = true;
	}
	return SW_OK;
}

// Postprocess arguments and destination of a graph frame. A registered host buffer is mapped into the
// device's address space: the tonemap writes the Color32 rows straight into it (*direct_host). Other
// host memory gets a device buffer copied out after the frame.
int frame_post_target(SwCtx* ctx, const SwFrameParams& p, const SwPostConfig& post, const float modulate[3], void* dst,
	uint32_t dst_pitch, int dst_is_device, PostArgs& pa, void** post_out, bool* direct_host, int pslot = -1)
{
	if (!dst) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "postprocess needs a destination");
	int r;
	if ((r = prepare_post(ctx, &post, modulate, pa))) return r;
	*post_out = dst;
	*direct_host = false;
	pa.dst_pitch = dst_pitch;
	if (pslot >= 0)
	{
		// a frame in flight: its slot's device buffer, copied out on the copy stream after the frame
		if ((r = ensure(ctx, ctx->ldr[pslot], size_t(p.width) * p.height * 4))) return r;
		*post_out = ctx->ldr[pslot].ptr;
		pa.dst_pitch = p.width;
	}
	else if (!dst_is_device)
	{
		void* mapped = registered_device_pointer(ctx, dst, (size_t(p.height) - 1) * dst_pitch * 4 + size_t(p.width) * 4);
		if (mapped)
		{
			*post_out = mapped;
			*direct_host = true;
		}
		else
		{
			if ((r = ensure(ctx, ctx->up_dst, size_t(p.width) * p.height * 4))) return r;
			*post_out = ctx->up_dst.ptr;
			pa.dst_pitch = p.width;
		}
	}
	pa.dst = static_cast<uint32_t*>(*post_out);
	return SW_OK;
}

// Capture the device work `enqueue` issues on the context's streams, update `exec` in place (or
// instantiate it when the topology changed) and launch it.
template <class F>
int capture_and_launch(SwCtx* ctx, cudaGraphExec_t& exec, F&& enqueue)
{
	SW_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
	ctx->capturing = true;
	const int er = enqueue();
	ctx->capturing = false;
	cudaGraph_t g = nullptr;
	const cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
	if (er || ee != cudaSuccess)
	{
		if (g) cudaGraphDestroy(g);
		cudaGetLastError();
		return er ? er : cuda_fail(ctx, ee, "cudaStreamEndCapture");
	}
	if (exec)
	{
		cudaGraphExecUpdateResultInfo info;
		if (cudaGraphExecUpdate(exec, g, &info) != cudaSuccess)
		{
			cudaGetLastError(); // the topology changed: instantiate anew
			cudaGraphExecDestroy(exec);
			exec = nullptr;
		}
	}
	if (!exec)
	{
		const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
		if (ie != cudaSuccess)
		{
			cudaGraphDestroy(g);
			exec = nullptr;
			return cuda_fail(ctx, ie, "cudaGraphInstantiate");
		}
	}
	cudaGraphDestroy(g);
	stage_begin(ctx, STAGE_FRAME);
	SW_CUDA(ctx, cudaGraphLaunch(exec, ctx->stream));
	stage_end(ctx, STAGE_FRAME);
	return SW_OK;
}

// After a graph frame was launched: staging and ordering events, exposure bookkeeping, and the frame
// into the caller's host memory (a direct-host frame only needs the stream to finish).
int finish_graph_frame(SwCtx* ctx, Staging& st, const SwFrameParams& p, bool postprocess, const SwPostConfig& post, float dt,
	void* dst, uint32_t dst_pitch, int dst_is_device, void* post_out, bool direct_host, int pslot = -1)
{
	SW_CUDA(ctx, cudaEventRecord(st.done, ctx->stream));
	st.pending = true;
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_tiles, ctx->stream));
	ctx->tiles_recorded = true;
	ctx->arena_valid = true;
	ctx->draws_valid = false;
	ctx->frame_open = false;
	if (postprocess && pslot >= 0)
	{
		// the graph recorded average_ready after the frame's average; the Color32 frame goes out on the
		// copy stream, and the call returns once the previous frame is in its destination
		ctx->exposure_pending = true;
		ctx->pending_config = post_config_clamped(post);
		ctx->pending_dt = dt;
		SW_CUDA(ctx, cudaEventRecord(ctx->ev_graph_done[pslot], ctx->stream));
		SW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy, ctx->ev_graph_done[pslot], 0));
		SW_CUDA(ctx, cudaMemcpy2DAsync(dst, size_t(dst_pitch) * 4, post_out, size_t(p.width) * 4, size_t(p.width) * 4, p.height,
						 cudaMemcpyDeviceToHost, ctx->copy));
		SW_CUDA(ctx, cudaEventRecord(ctx->ev_d2h[pslot], ctx->copy));
		ctx->d2h_pending[pslot] = true;
		const int other = pslot ^ 1;
		if (ctx->d2h_pending[other])
		{
			SW_CUDA(ctx, cudaEventSynchronize(ctx->ev_d2h[other]));
			ctx->d2h_pending[other] = false;
		}
		return SW_OK;
	}
	if (postprocess)
	{
		SW_CUDA(ctx, cudaEventRecord(ctx->average_ready, ctx->stream));
		ctx->exposure_pending = true;
		ctx->pending_config = post_config_clamped(post);
		ctx->pending_dt = dt;
		if (direct_host)
		{
			SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // the frame is in the caller's buffer on return
			return SW_OK;
		}
		if (!dst_is_device) return copy_out(ctx, dst, dst_pitch, 0, post_out, p.width, p.width, p.height, 4);
	}
	else if (dst && !dst_is_device)
		return copy_out(ctx, dst, dst_pitch, 0, ctx->framebuffer.ptr, p.width, p.width, p.height, bpp_of(p.pixel_format));
	return SW_OK;
}
} // namespace

extern "C" {

int sw_draw_frame(SwCtx* ctx, const SwFrameInput* in)
{
	if (!ctx || !in) return SW_ERR_INVALID_ARGUMENT;
	const SwFrameInput& f = *in;
	if ((f.num_lights && !f.lights) || (f.num_surfaces && !f.surfaces) || (f.num_draws && !f.draws) ||
		(f.num_vertices && !f.vertices) || (f.num_tri_vertices && !f.tri_vertices))
		return SW_ERR_INVALID_ARGUMENT;
	if (f.postprocess && f.params.pixel_format != SW_PIXEL_C64)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "postprocessing needs a colour64 frame");
	if (f.dst && f.dst_pitch < f.params.width) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "pitch < width");
	if (f.num_views)
	{
		// nested views: regions inside the arena, draws after the frame's own, textures inside the lite pixels
		if (!f.views) return SW_ERR_INVALID_ARGUMENT;
		if (f.num_views > 65536) return fail(ctx, SW_ERR_LIMIT, "too many views");
		if (f.main_draws > f.num_draws) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "main_draws > num_draws");
		for (uint32_t i = 0; i < f.num_views; ++i)
		{
			const SwView& v = f.views[i];
			if (v.width == 0 || v.height == 0 || v.width > 16384 || v.height > 16384)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: bad size %ux%u", i, v.width, v.height);
			const uint64_t area = uint64_t(v.width) * v.height;
			if (v.target_offset > f.total_texels || area > f.total_texels - v.target_offset)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: target outside the surface arena", i);
			if (v.first_draw < f.main_draws || uint64_t(v.first_draw) + v.num_draws > f.num_draws)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: draws outside [main_draws, num_draws)", i);
			if (v.clear_background > 1) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: bad clear_background", i);
			if (v.mix_blend != SW_VIEW_NO_MIX)
			{
				const uint64_t tex = uint64_t(v.mix_size[0]) * v.mix_size[1];
				if (v.mix_blend > SW_BLEND_ALPHA_BLEND || tex == 0 || v.mix_size[0] > 65536 || v.mix_size[1] > 65536 ||
					v.mix_offset > ctx->lite_texels || tex > ctx->lite_texels - v.mix_offset)
					return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: bad texture mix", i);
				for (int c = 0; c < 3; ++c)
					if (!(std::fabs(v.mix_light[c]) <= 65536.0f))
						return fail(ctx, SW_ERR_INVALID_ARGUMENT, "view %u: texture light not finite", i);
			}
		}
	}
	int r;
	const SwFrameParams& p = f.params;
	if ((r = check_frame_params(ctx, p, f.lights, f.num_lights))) return r;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	ctx->frame = p;
	ctx->num_lights = f.num_lights;

	// 1. every per-frame array into one pinned staging block (two blocks alternate between frames)
	const uint32_t slot = ctx->gset;
	Staging& st = ctx->gstage[slot];
	ctx->gset ^= 1u;
	size_t off[8];
	off[0] = 0;
	off[1] = align_up(off[0] + std::max<size_t>(f.num_lights, 1) * sizeof(SwLight), 256);
	off[2] = align_up(off[1] + std::max<size_t>(f.num_surfaces, 1) * sizeof(SurfaceGpu), 256);
	off[3] = align_up(off[2] + (size_t(f.num_surfaces) + 1) * 8, 256);
	off[4] = align_up(off[3] + std::max<size_t>(f.num_draws, 1) * sizeof(SwDrawCmd), 256);
	off[5] = align_up(off[4] + std::max<size_t>(f.num_vertices, 1) * sizeof(SwVertex16), 256);
	off[6] = align_up(off[5] + std::max<size_t>(f.num_draws, 1) * sizeof(DrawRows), 256);
	off[7] = align_up(off[6] + std::max<size_t>(f.num_tri_vertices, 1) * sizeof(SwTriVertex), 256);
	void* hv = nullptr;
	if ((r = staging_acquire(ctx, st, off[7], &hv))) return r;
	unsigned char* h = static_cast<unsigned char*>(hv);
	if (f.num_lights) std::memcpy(h + off[0], f.lights, f.num_lights * sizeof(SwLight));
	uint64_t work = 0;
	uint32_t max_light = 0;
	if ((r = prepare_surfaces(ctx, f.surfaces, f.num_surfaces, f.total_texels, reinterpret_cast<SurfaceGpu*>(h + off[1]),
			 reinterpret_cast<uint64_t*>(h + off[2]), &work, &max_light)))
		return r;
	note_surfaces(ctx, f.num_surfaces, f.total_texels, work, max_light);
	if (f.num_draws) std::memcpy(h + off[3], f.draws, f.num_draws * sizeof(SwDrawCmd));
	if (f.num_vertices) std::memcpy(h + off[4], f.vertices, f.num_vertices * sizeof(SwVertex16));
	if (f.num_tri_vertices) std::memcpy(h + off[6], f.tri_vertices, f.num_tri_vertices * sizeof(SwTriVertex));
	uint64_t rows = 0;
	if ((r = prepare_draws(ctx, f.draws, f.num_draws, f.vertices, f.num_vertices, reinterpret_cast<DrawRows*>(h + off[5]), &rows,
			 f.tri_vertices, f.num_tri_vertices, f.num_views ? f.views : nullptr, f.num_views)))
		return r;

	// 2. device buffers (growing them synchronises; the next capture picks up the new addresses)
	const uint32_t bpp = bpp_of(p.pixel_format);
	if ((r = ensure(ctx, ctx->frame_in, off[7]))) return r;
	if ((r = ensure(ctx, ctx->lights, std::max<size_t>(f.num_lights, 1) * sizeof(SwLight)))) return r;
	if ((r = ensure(ctx, ctx->arena, std::max<uint64_t>(f.total_texels, 1) * bpp))) return r;
	if ((r = ensure(ctx, ctx->surfaces, std::max<size_t>(f.num_surfaces, 1) * sizeof(SurfaceGpu)))) return r;
	if ((r = ensure(ctx, ctx->work_prefix, (size_t(f.num_surfaces) + 1) * 8))) return r;
	if ((r = ensure_raster_buffers(ctx, f.num_draws, f.num_vertices, rows))) return r;
	if ((r = ensure_bins(ctx, f.params.width, f.params.height, f.num_draws))) return r;
	if (f.num_views && (r = ensure_view_bins(ctx, f.views, f.num_views))) return r;
	if ((r = ensure_framebuffer(ctx, p))) return r;
	ctx->num_rows = rows;
	ctx->num_draws = f.num_draws;
	PostArgs pa;
	void* post_out = nullptr;
	bool direct_host = false;
	const int pslot = frame_pipeline_slot(ctx, f.postprocess != 0, f.dst, f.dst_pitch, p, f.dst_is_device, slot);
	if (f.postprocess && (r = frame_post_target(ctx, p, f.post, f.color_modulate, f.dst, f.dst_pitch, f.dst_is_device, pa,
							  &post_out, &direct_host, pslot)))
		return r;
	if (pslot >= 0)
	{
		// a frame in flight: the average kernel writes the average straight to host memory, where the next
		// frame's exposure update reads it once the graph's average event has fired; the slot's output
		// buffer is free once its previous copy-out has finished
		pa.average = ctx->d_average_mapped;
		if (ctx->d2h_pending[pslot]) SW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_d2h[pslot], 0));
	}

	// 3. capture the device work and update (or instantiate) the frame graph; with the graph off, the
	// same work is launched directly (with per-stage timing events when timing is on)
	auto enqueue = [&]() {
		return enqueue_frame(ctx, f, h, off, rows, f.postprocess ? &pa : nullptr, pslot >= 0 ? ctx->average_ready : nullptr);
	};
	if (ctx->graph_enabled)
	{
		if ((r = capture_and_launch(ctx, ctx->gexec, enqueue))) return r;
	}
	else
	{
		stage_begin(ctx, STAGE_FRAME);
		r = enqueue();
		stage_end(ctx, STAGE_FRAME);
		if (r) return r;
	}
	ctx->stats.draws += f.num_draws; // (surfaces are counted by launch_surfaces)
	ctx->stats.upload_bytes += off[7];
	return finish_graph_frame(ctx, st, p, f.postprocess != 0, f.post, f.frame_duration_s, f.dst, f.dst_pitch, f.dst_is_device,
		post_out, direct_host, pslot);
}

int sw_set_map(SwCtx* ctx, const SwMapPolygon* polygons, uint32_t num_polygons, const float* vertices, uint32_t num_vertices)
{
	if (!ctx || (num_polygons && !polygons) || (num_vertices && !vertices)) return SW_ERR_INVALID_ARGUMENT;
	const uint64_t simple = ctx->num_lightmap_elements, directional = ctx->num_dir_lightmap_elements;
	uint64_t lightmap_end = 0;
	std::vector<uint64_t> prefix(size_t(num_polygons) + 1, 0);
	for (uint32_t i = 0; i < num_polygons; ++i)
	{
		const SwMapPolygon& p = polygons[i];
		if (uint64_t(p.first_vertex) + p.num_vertices > num_vertices)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: vertices out of range", i);
		if (p.tex_coord_min[0] > p.tex_coord_max[0] || p.tex_coord_min[1] > p.tex_coord_max[1])
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: bad texture coordinate bounds", i);
		if ((p.flags & SW_POLY_DIFFUSE_LAYER) && uint64_t(p.texture) * 5 + 4 >= ctx->h_texture_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: bad texture", i);
		if (p.emissive_texture != SW_NO_EMISSIVE && uint64_t(p.emissive_texture) * 5 + 4 >= ctx->h_emissive_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: bad emissive texture", i);
		if (p.blending_mode > SW_BLEND_ALPHA_BLEND) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: bad blending mode", i);
		if ((p.flags & SW_POLY_DIFFUSE_LAYER) && p.lightmap_data_offset != SW_NO_LIGHTMAP)
		{
			// get_polygon_lightmap_size, lightmap.rs:11-27; every surface of the polygon reads inside it
			const uint64_t lw = uint64_t(int64_t((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1);
			const uint64_t lh = uint64_t(int64_t((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1);
			const uint64_t end = uint64_t(p.lightmap_data_offset) + lw * lh;
			if ((simple > 1 && end > simple) || (directional > 1 && end > directional))
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "polygon %u: lightmap out of range", i);
			lightmap_end = std::max(lightmap_end, end);
		}
		prefix[i + 1] = prefix[i] + swhost::max_surface_texels(p);
	}
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
	int r;
	if ((r = upload_static(ctx, ctx->map_polygons, polygons, size_t(num_polygons) * sizeof(SwMapPolygon)))) return r;
	if ((r = upload_static(ctx, ctx->map_vertices, vertices, size_t(num_vertices) * 12))) return r;
	ctx->num_map_polygons = num_polygons;
	ctx->num_map_vertices = num_vertices;
	ctx->map_lightmap_end = lightmap_end;
	ctx->poly_bound_prefix.swap(prefix);
	return SW_OK;
}

namespace
{
// Counts of a finished view frame (staging set `slot`): statistics and the surface grid size.
void consume_view_counts(SwCtx* ctx, uint32_t slot)
{
	const SwViewCounts& k = ctx->h_counts[slot];
	ctx->counts_pending[slot] = false;
	ctx->stats.surfaces += k.num_surfaces;
	ctx->stats.surface_texels += k.total_texels;
	ctx->stats.draws += k.num_draws;
	if (ctx->counts_seq[slot] > ctx->hint_seq)
	{
		ctx->view_work_hint = k.total_texels;
		ctx->hint_seq = ctx->counts_seq[slot];
	}
}
} // namespace

namespace
{
uint64_t pow2_at_least(uint64_t v, uint64_t floor_value)
{
	uint64_t c = floor_value;
	while (c < v) c <<= 1;
	return c;
}

// Fixed layout of a view frame's upload block for the current capacities (the replayed graph copies the
// whole block): per-frame header (PrepFrame, camera position, tonemap scale), then the arrays.
struct ViewBlock
{
	size_t frame, cam, inv_scale, lights, leafs, cand_base, leaf_lights, draw_leaf, slot_base, draws, vertices, rows, shifts, bytes;
};
ViewBlock view_block(const SwCtx* ctx)
{
	ViewBlock v;
	v.frame = 0;
	v.cam = align_up(v.frame + sizeof(PrepFrame), 16);
	v.inv_scale = v.cam + 16;
	v.lights = align_up(v.inv_scale + 16, 256);
	v.leafs = align_up(v.lights + ctx->vcap_lights * sizeof(SwLight), 256);
	v.cand_base = align_up(v.leafs + ctx->vcap_leafs * sizeof(SwViewLeaf), 256);
	v.leaf_lights = align_up(v.cand_base + (ctx->vcap_leafs + 1) * 4, 256);
	v.draw_leaf = align_up(v.leaf_lights + ctx->vcap_leaf_lights * 2, 256);
	v.slot_base = align_up(v.draw_leaf + ctx->vcap_leafs * 4, 256);
	v.draws = align_up(v.slot_base + (ctx->vcap_leafs + 1) * 4, 256);
	v.vertices = align_up(v.draws + ctx->vcap_host_draws * sizeof(SwDrawCmd), 256);
	v.rows = align_up(v.vertices + ctx->vcap_host_vertices * sizeof(SwVertex16), 256);
	v.shifts = align_up(v.rows + ctx->vcap_host_draws * sizeof(DrawRows), 256);
	v.bytes = align_up(v.shifts + ctx->vcap_shifts * sizeof(SwMaterialFrame), 256);
	return v;
}

// One device allocation for all of a view frame's small buffers (the upload block, the counts, the
// candidates, the compacted surfaces and draws, the raster setup's records): the preparation and setup
// kernels' dependent loads stay within a few pages.
struct ViewSlab
{
	size_t frame_in, counts, keys, cands, descs, surfaces, work_prefix, draws, draw_rows, rdraws, boxes, vertices, tri_steps,
		rows, bytes;
};
ViewSlab view_slab(size_t block_bytes, uint64_t cands, uint64_t draws, uint64_t vertices, uint64_t rows)
{
	ViewSlab v;
	size_t at = 0;
	auto take = [&](size_t bytes) {
		const size_t o = at;
		at = align_up(at + bytes, 256);
		return o;
	};
	v.frame_in = take(block_bytes);
	v.counts = take(sizeof(SwViewCounts));
	v.keys = take(cands * sizeof(PrepKey));
	v.cands = take(cands * sizeof(PrepCand));
	v.descs = take(cands * sizeof(SwSurfaceDesc));
	v.surfaces = take(cands * sizeof(SurfaceGpu));
	v.work_prefix = take((cands + 1) * 8);
	v.draws = take(draws * sizeof(SwDrawCmd));
	v.draw_rows = take(draws * sizeof(DrawRows));
	v.rdraws = take(draws * sizeof(RasterDraw));
	v.boxes = take(draws * sizeof(RasterBox));

	v.vertices = take(vertices * sizeof(SwVertex16));
	v.tri_steps = take(draws * 2 * sizeof(TriSteps));
	v.rows = take(rows * sizeof(RasterRow));
	v.bytes = at;
	return v;
}

} // namespace

int sw_draw_frame_view(SwCtx* ctx, const SwViewFrameInput* in)
{
	if (!ctx || !in) return SW_ERR_INVALID_ARGUMENT;
	const SwViewFrameInput& f = *in;
	if ((f.num_lights && !f.lights) || (f.num_leafs && !f.leafs) || (f.num_leaf_lights && !f.leaf_lights) ||
		(f.num_draws && (!f.draws || !f.vertices)) || (f.num_material_frames && !f.material_frames))
		return SW_ERR_INVALID_ARGUMENT;
	if (!all_finite(f.view_matrix, 16) || !all_finite(f.planes_matrix, 16))
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "non-finite camera matrices");
	if (f.num_material_frames > (1u << 20)) return fail(ctx, SW_ERR_LIMIT, "too many material frames");
	for (uint32_t i = 0; i < f.num_material_frames; ++i)
	{
		const SwMaterialFrame& m = f.material_frames[i];
		if (uint64_t(m.texture) * 5 + 4 >= ctx->h_texture_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "material %u: frame texture %u has no mips", i, m.texture);
		if (m.emissive_texture != SW_NO_EMISSIVE && uint64_t(m.emissive_texture) * 5 + 4 >= ctx->h_emissive_mips.size())
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "material %u: bad emissive texture", i);
		if (m.blending_mode > SW_BLEND_ALPHA_BLEND) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "material %u: bad blending mode", i);
		if (!all_finite(m.emissive_light, 3)) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "material %u: non-finite emissive light", i);
	}
	if (f.postprocess && f.params.pixel_format != SW_PIXEL_C64)
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "postprocessing needs a colour64 frame");
	if (f.dst && f.dst_pitch < f.params.width) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "pitch < width");
	int r;
	const SwFrameParams& p = f.params;
	if ((r = check_frame_params(ctx, p, f.lights, f.num_lights))) return r;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	for (uint32_t k = 0; k < 2; ++k)
		if (ctx->counts_pending[k] && cudaEventQuery(ctx->ev_counts[k]) == cudaSuccess) consume_view_counts(ctx, k);
	cudaGetLastError(); // a not-ready query is not an error

	// 1. validate the leafs and derive the candidate and draw-slot numbering and the capacity bounds
	const uint32_t nl = f.num_leafs;
	std::vector<uint32_t>& draw_leaf = ctx->v_draw_leaf;
	draw_leaf.assign(nl, 0xFFFFFFFFu);
	uint32_t num_draw_leafs = 0;
	uint64_t candidates = 0, slots = 0, texel_bound = 0, row_bound = 0;
	for (uint32_t i = 0; i < nl; ++i)
	{
		const SwViewLeaf& l = f.leafs[i];
		if (uint64_t(l.first_polygon) + l.num_polygons > ctx->num_map_polygons)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "leaf %u: polygons out of range (sw_set_map)", i);
		if (uint64_t(l.first_light) + l.num_lights > f.num_leaf_lights)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "leaf %u: lights out of range", i);
		candidates += l.num_polygons;
		texel_bound += ctx->poly_bound_prefix[l.first_polygon + l.num_polygons] - ctx->poly_bound_prefix[l.first_polygon];
		if (l.draw_order != SW_LEAF_NOT_DRAWN)
		{
			if (l.draw_order >= nl || draw_leaf[l.draw_order] != 0xFFFFFFFFu)
				return fail(ctx, SW_ERR_INVALID_ARGUMENT, "leaf %u: bad draw order", i);
			draw_leaf[l.draw_order] = i;
			++num_draw_leafs;
			slots += l.num_polygons;
			// rows of a draw lie in the leaf's draw bounds: y in [planes[3].c, -planes[2].c] (+ rounding)
			const float y_min = l.draw_clip_planes[3][2], y_max = -l.draw_clip_planes[2][2];
			uint64_t rows = p.height;
			if (y_min == y_min && y_max == y_max && y_max - y_min < float(p.height))
				rows = std::min<uint64_t>(p.height, uint64_t(std::max(0.0f, std::ceil(y_max - y_min))) + 2);
			row_bound += uint64_t(l.num_polygons) * rows;
		}
	}
	for (uint32_t j = 0; j < num_draw_leafs; ++j)
		if (draw_leaf[j] == 0xFFFFFFFFu) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw order has a gap at %u", j);
	for (uint32_t i = 0; i < f.num_leaf_lights; ++i)
		if (f.leaf_lights[i] >= f.num_lights) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "leaf light %u: bad light index", i);
	if (candidates > 0x7FFFFFFFull) return fail(ctx, SW_ERR_LIMIT, "too many polygons in the visible leafs");
	for (uint32_t i = 0; i < f.num_draws; ++i)
		if (f.draws[i].tex_source != SW_TEXSRC_SKYBOX)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "draw %u: host draws of a view frame read the skybox", i);
	std::vector<DrawRows>& host_draw_rows = ctx->v_host_rows;
	host_draw_rows.resize(std::max<size_t>(f.num_draws, 1));
	uint64_t host_rows = 0;
	ctx->frame = p; // prepare_draws checks the host draws against this frame's size
	if ((r = prepare_draws(ctx, f.draws, f.num_draws, f.vertices, f.num_vertices, host_draw_rows.data(), &host_rows))) return r;
	ctx->num_lights = f.num_lights;
	const uint64_t need_draws = uint64_t(f.num_draws) + slots;
	const uint64_t need_vertices = uint64_t(f.num_vertices) + slots * SW_MAX_POLYGON_VERTICES;
	const uint64_t need_rows = host_rows + row_bound;
	if (need_draws > 0x7FFFFFFFull || need_vertices > 0x7FFFFFFFull) return fail(ctx, SW_ERR_LIMIT, "too many draws");

	// 2. capacities only grow (power-of-two steps): the upload block's layout and the device buffers
	// stay the same from frame to frame, and so do the replayed graphs
	ctx->vcap_lights = pow2_at_least(f.num_lights, std::max<uint64_t>(ctx->vcap_lights, 16));
	ctx->vcap_leafs = pow2_at_least(nl, std::max<uint64_t>(ctx->vcap_leafs, 64));
	ctx->vcap_leaf_lights = pow2_at_least(f.num_leaf_lights, std::max<uint64_t>(ctx->vcap_leaf_lights, 256));
	ctx->vcap_host_draws = pow2_at_least(f.num_draws, std::max<uint64_t>(ctx->vcap_host_draws, 8));
	ctx->vcap_host_vertices = pow2_at_least(f.num_vertices, std::max<uint64_t>(ctx->vcap_host_vertices, 64));
	ctx->vcap_shifts = pow2_at_least(f.num_material_frames, std::max<uint64_t>(ctx->vcap_shifts, 16));
	const ViewBlock vb = view_block(ctx);
	const uint32_t bpp = bpp_of(p.pixel_format);
	ctx->vs_cands = pow2_at_least(candidates, std::max<uint64_t>(ctx->vs_cands, 1024));
	ctx->vs_draws = pow2_at_least(need_draws, std::max<uint64_t>(ctx->vs_draws, 1024));
	ctx->vs_vertices = pow2_at_least(need_vertices, std::max<uint64_t>(ctx->vs_vertices, 8192));
	ctx->vs_rows = pow2_at_least(need_rows, std::max<uint64_t>(ctx->vs_rows, uint64_t(1) << 16));
	const uint64_t texel_cap = pow2_at_least(texel_bound, 1u << 20);
	const ViewSlab vs = view_slab(vb.bytes, ctx->vs_cands, ctx->vs_draws, ctx->vs_vertices, ctx->vs_rows);
	if ((r = ensure(ctx, ctx->vslab, vs.bytes))) return r;
	if ((r = ensure(ctx, ctx->arena, texel_cap * bpp))) return r;
	if ((r = ensure_framebuffer(ctx, p))) return r;
	unsigned char* slab = static_cast<unsigned char*>(ctx->vslab.ptr);
	const uint64_t cap_candidates = ctx->vs_cands, cap_surfaces = ctx->vs_cands, cap_draws = ctx->vs_draws;
	const uint64_t cap_vertices = ctx->vs_vertices, cap_rows = ctx->vs_rows;
	const uint64_t cap_texels = uint64_t(ctx->arena.bytes / bpp);
	ctx->v_counts = reinterpret_cast<SwViewCounts*>(slab + vs.counts);
	ctx->v_descs = reinterpret_cast<SwSurfaceDesc*>(slab + vs.descs);
	ctx->v_draws = reinterpret_cast<SwDrawCmd*>(slab + vs.draws);
	ctx->v_vertices = reinterpret_cast<SwVertex16*>(slab + vs.vertices);
	ctx->arena_texels = cap_texels;
	ctx->arena_format = p.pixel_format;
	ctx->arena_view = true;
	ctx->view_surfaces_cap = uint32_t(cap_surfaces);
	ctx->view_draws_cap = uint32_t(std::min<uint64_t>(cap_draws, 0xFFFFFFFFu));
	ctx->view_vertices_cap = uint32_t(std::min<uint64_t>(cap_vertices, 0xFFFFFFFFu));
	PostArgs pa;
	void* post_out = nullptr;
	bool direct_host = false;
	const int pslot = frame_pipeline_slot(ctx, f.postprocess != 0, f.dst, f.dst_pitch, p, f.dst_is_device, ctx->gset);
	if (f.postprocess && (r = frame_post_target(ctx, p, f.post, f.color_modulate, f.dst, f.dst_pitch, f.dst_is_device, pa,
							  &post_out, &direct_host, pslot)))
		return r;
	// a frame in flight: its slot's output buffer is free once its previous copy-out has finished
	if (pslot >= 0 && ctx->d2h_pending[pslot]) SW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_d2h[pslot], 0));

	// 3. the upload block of this frame (two staging blocks alternate between frames)
	const uint32_t slot = ctx->gset;
	Staging& st = ctx->gstage[slot];
	ctx->gset ^= 1u;
	void* hv = nullptr;
	if ((r = staging_acquire(ctx, st, vb.bytes, &hv))) return r;
	if (ctx->counts_pending[slot])
	{
		// the frame that last used this staging set has finished (staging_acquire waited for it)
		SW_CUDA(ctx, cudaEventSynchronize(ctx->ev_counts[slot]));
		consume_view_counts(ctx, slot);
	}
	unsigned char* h = static_cast<unsigned char*>(hv);
	PrepFrame& pf = *reinterpret_cast<PrepFrame*>(h + vb.frame);
	std::memcpy(pf.view, f.view_matrix, sizeof(pf.view));
	std::memcpy(pf.planes, f.planes_matrix, sizeof(pf.planes));
	pf.mip_bias = f.mip_bias;
	pf.num_leafs = nl;
	pf.num_candidates = uint32_t(candidates);
	pf.num_draw_leafs = num_draw_leafs;
	pf.num_host_draws = f.num_draws;
	pf.num_host_vertices = f.num_vertices;
	pf.num_host_rows = host_rows;
	pf.num_material_frames = f.num_material_frames;
	float* cam = reinterpret_cast<float*>(h + vb.cam);
	cam[0] = p.cam_pos[0], cam[1] = p.cam_pos[1], cam[2] = p.cam_pos[2], cam[3] = 0.0f;
	float* isc = reinterpret_cast<float*>(h + vb.inv_scale);
	if (f.postprocess)
	{
		for (int k = 0; k < 4; ++k) isc[k] = pa.inv_scale[k];
		for (int k = 0; k < 4; ++k) pa.inv_scale[k] = 0.0f; // read from the block
	}
	if (f.num_lights) std::memcpy(h + vb.lights, f.lights, f.num_lights * sizeof(SwLight));
	if (nl) std::memcpy(h + vb.leafs, f.leafs, nl * sizeof(SwViewLeaf));
	uint32_t* cand_base = reinterpret_cast<uint32_t*>(h + vb.cand_base);
	cand_base[0] = 0;
	for (uint32_t i = 0; i < nl; ++i) cand_base[i + 1] = cand_base[i] + f.leafs[i].num_polygons;
	if (f.num_leaf_lights) std::memcpy(h + vb.leaf_lights, f.leaf_lights, f.num_leaf_lights * 2);
	uint32_t* dl = reinterpret_cast<uint32_t*>(h + vb.draw_leaf);
	uint32_t* slot_base = reinterpret_cast<uint32_t*>(h + vb.slot_base);
	slot_base[0] = 0;
	for (uint32_t j = 0; j < num_draw_leafs; ++j)
	{
		dl[j] = draw_leaf[j];
		slot_base[j + 1] = slot_base[j] + f.leafs[draw_leaf[j]].num_polygons;
	}
	if (f.num_draws)
	{
		std::memcpy(h + vb.draws, f.draws, f.num_draws * sizeof(SwDrawCmd));
		std::memcpy(h + vb.rows, host_draw_rows.data(), f.num_draws * sizeof(DrawRows));
	}
	if (f.num_vertices) std::memcpy(h + vb.vertices, f.vertices, f.num_vertices * sizeof(SwVertex16));
	if (f.num_material_frames)
		std::memcpy(h + vb.shifts, f.material_frames, size_t(f.num_material_frames) * sizeof(SwMaterialFrame));

	// 4. kernel arguments: buffers and capacities only (the per-frame values are in the block)
	unsigned char* d = slab + vs.frame_in;
	SwViewCounts* counts = ctx->v_counts;
	ViewGraphKey key;
	std::memset(&key, 0, sizeof(key)); // padding too: keys are compared bytewise
	PrepArgs& pr = key.prep;
	pr.frame = reinterpret_cast<const PrepFrame*>(d + vb.frame);
	pr.material_frames = reinterpret_cast<const SwMaterialFrame*>(d + vb.shifts);
	pr.polygons = static_cast<const SwMapPolygon*>(ctx->map_polygons.ptr);
	pr.map_vertices = static_cast<const float*>(ctx->map_vertices.ptr);
	pr.leafs = reinterpret_cast<const SwViewLeaf*>(d + vb.leafs);
	pr.leaf_cand_base = reinterpret_cast<const uint32_t*>(d + vb.cand_base);
	pr.leaf_lights = reinterpret_cast<const uint16_t*>(d + vb.leaf_lights);
	pr.lights = reinterpret_cast<const SwLight*>(d + vb.lights);
	pr.draw_leaf = reinterpret_cast<const uint32_t*>(d + vb.draw_leaf);
	pr.draw_slot_base = reinterpret_cast<const uint32_t*>(d + vb.slot_base);
	pr.directional = p.use_directional_lightmaps ? 1u : 0u;
	pr.simple_lightmaps = ctx->num_lightmap_elements > 1 ? 1u : 0u;
	pr.height = int32_t(p.height);
	pr.host_draws = reinterpret_cast<const SwDrawCmd*>(d + vb.draws);
	pr.host_vertices = reinterpret_cast<const SwVertex16*>(d + vb.vertices);
	pr.host_rows = reinterpret_cast<const DrawRows*>(d + vb.rows);
	pr.texture_mips = static_cast<const SwTextureMip*>(ctx->texture_mips.ptr);
	pr.emissive_mips = static_cast<const SwEmissiveMip*>(ctx->emissive_mips.ptr);
	pr.shadows = ctx->num_shadow_descs ? static_cast<const SwLightShadow*>(ctx->shadow_descs.ptr) : nullptr;
	pr.num_shadows = ctx->num_shadow_descs;
	pr.cands = reinterpret_cast<PrepCand*>(slab + vs.cands);
	pr.keys = reinterpret_cast<PrepKey*>(slab + vs.keys);
	pr.descs = ctx->v_descs;
	pr.surfaces = reinterpret_cast<SurfaceGpu*>(slab + vs.surfaces);
	pr.work_prefix = reinterpret_cast<uint64_t*>(slab + vs.work_prefix);
	pr.draws = ctx->v_draws;
	pr.vertices = ctx->v_vertices;
	pr.draw_rows = reinterpret_cast<DrawRows*>(slab + vs.draw_rows);
	pr.counts = counts;
	pr.cap_candidates = uint32_t(std::min<uint64_t>(cap_candidates, 0x7FFFFFFFu));
	pr.cap_surfaces = uint32_t(std::min<uint64_t>(cap_surfaces, 0x7FFFFFFFu));
	pr.cap_draws = uint32_t(std::min<uint64_t>(cap_draws, 0x7FFFFFFFu));
	pr.cap_vertices = uint32_t(std::min<uint64_t>(cap_vertices, 0x7FFFFFFFu));
	pr.cap_texels = cap_texels;
	pr.cap_rows = cap_rows;

	SurfaceKernelArgs& sa = key.surf;
	sa.surfaces = pr.surfaces;
	sa.work_prefix = pr.work_prefix;
	sa.directional = p.use_directional_lightmaps ? 1u : 0u;
	sa.counts = counts;
	sa.texels = static_cast<const uint64_t*>(ctx->texels.ptr);
	sa.emissive_pixels = static_cast<const uint32_t*>(ctx->emissive.ptr);
	sa.lightmaps = static_cast<const float*>(ctx->lightmaps.ptr);
	sa.directional_lightmaps = static_cast<const SwDirectionalLightmapElement*>(ctx->dir_lightmaps.ptr);
	sa.lights = pr.lights;
	sa.cam_pos_dev = reinterpret_cast<const float*>(d + vb.cam);
	sa.shadows = ctx->num_shadow_descs ? static_cast<const SwLightShadow*>(ctx->shadow_descs.ptr) : nullptr;
	sa.shadow_texels = static_cast<const unsigned long long*>(ctx->shadow_storage.ptr);
	sa.num_shadows = ctx->num_shadow_descs;
	sa.arena = ctx->arena.ptr;
	// surface grid: from the latest frame's texels with headroom; it changes (and the graphs are captured
	// again) only when the texel count leaves [grid/2, grid] blocks' worth
	{
		const uint64_t hint = ctx->view_work_hint ? ctx->view_work_hint + ctx->view_work_hint / 4 : (uint64_t(1) << 40);
		const uint64_t max_blocks = uint64_t(ctx->num_sms) * std::max<uint32_t>(ctx->tuning.surface_blocks_per_sm, 1);
		const uint64_t needed = std::min(std::max((hint + 255) / 256, uint64_t(ctx->num_sms)), max_blocks);
		if (ctx->view_surface_blocks == 0 || needed > ctx->view_surface_blocks || needed < ctx->view_surface_blocks / 2 ||
			ctx->view_surface_blocks > max_blocks)
			ctx->view_surface_blocks = unsigned(std::min(needed + needed / 4, max_blocks));
	}
	key.surface_blocks = ctx->view_surface_blocks;
	key.surface_blocks_per_sm = int(ctx->tuning.surface_blocks_per_sm);
	key.surface_texels_per_thread = int(ctx->tuning.surface_texels_per_thread);

	RasterArgs& ra = key.raster;
	if ((r = ensure_bins(ctx, p.width, p.height, cap_draws))) return r;
	ra = raster_args(ctx);
	ra.draws = pr.draws;
	ra.vertices = pr.vertices;
	ra.draw_rows = pr.draw_rows;
	ra.tri_steps = reinterpret_cast<TriSteps*>(slab + vs.tri_steps);
	ra.rdraws = reinterpret_cast<RasterDraw*>(slab + vs.rdraws);
	ra.rows = reinterpret_cast<RasterRow*>(slab + vs.rows);
	ra.boxes = reinterpret_cast<RasterBox*>(slab + vs.boxes);
	ra.counts = counts;
	ra.num_draws = 0;
	ra.setup_blocks = uint32_t(ctx->num_sms) * 2;
	ra.total_rows = 0;
	if (f.postprocess)
	{
		key.post = pa;
		key.post.inv_scale_dev = reinterpret_cast<const float*>(d + vb.inv_scale);
		key.post.average = ctx->d_average_mapped; // the frame's average colour goes straight to host memory
	}
	key.staging = st.host;
	key.block_bytes = vb.bytes;
	key.raster_tile = ctx->tuning.raster_tile;
	key.pixel_format = p.pixel_format;
	key.postprocess = f.postprocess ? 1u : 0u;
	key.dst = f.dst;
	key.dst_pitch = f.dst_pitch;
	key.dst_is_device = f.dst_is_device;
	key.slot = slot;
	key.in_flight = pslot >= 0 ? 1u : 0u;

	// 5. replay this staging block's graph; capture it again when its key changed
	cudaGraphExec_t& exec = ctx->vexec[slot];
	if (!exec || std::memcmp(&ctx->vkey[slot], &key, sizeof(key)) != 0)
	{
		auto enqueue = [&]() -> int {
			cudaStream_t s = ctx->stream, aux = ctx->aux;
			SW_CUDA(ctx, cudaMemcpyAsync(d, st.host, vb.bytes, cudaMemcpyHostToDevice, s));
			int rr;
			// per-candidate preparation, then the surface compaction here and the draw compaction on aux
			if ((rr = check_kernel(ctx, launch_prep(key.prep, s, aux, ctx->ev_fork), "surface and draw preparation"))) return rr;
			if ((rr = check_kernel(ctx, launch_raster_setup(key.raster, aux), "raster setup"))) return rr;
			if ((rr = check_kernel(ctx, launch_raster_bins(key.raster, aux), "raster bins"))) return rr;
			SW_CUDA(ctx, cudaEventRecord(ctx->ev_setup, aux));
			if ((rr = check_kernel(ctx,
					 launch_surface_build(key.surf, p.pixel_format, ctx->num_sms, int(ctx->tuning.surface_blocks_per_sm), s,
						 uint64_t(key.surface_blocks) * 256, uint32_t(key.surface_texels_per_thread)),
					 "surface build")))
				return rr;
			SW_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_setup, 0));
			RasterArgs ra2 = key.raster;
			PostArgs pp2 = key.post;
			if (f.postprocess && (rr = fuse_bloom_downscale(ctx, ra2, pp2, s))) return rr;
			if ((rr = check_kernel(ctx, launch_raster_tiles(ra2, p.pixel_format, ctx->tuning.raster_tile, s), "raster")))
				return rr;
			if (f.postprocess)
			{
				if ((rr = check_kernel(ctx, launch_postprocess(pp2, ctx->num_sms, s, aux, ctx->ev_fork, ctx->ev_join,
												key.in_flight ? ctx->average_ready : nullptr),
						 "postprocess")))
					return rr;
			}
			else if (f.dst && f.dst_is_device)
				SW_CUDA(ctx, cudaMemcpy2DAsync(f.dst, size_t(f.dst_pitch) * bpp, ctx->framebuffer.ptr, size_t(p.width) * bpp,
								 size_t(p.width) * bpp, p.height, cudaMemcpyDeviceToDevice, s));
			SW_CUDA(ctx, cudaMemcpyAsync(ctx->h_counts + slot, counts, sizeof(SwViewCounts), cudaMemcpyDeviceToHost, s));
			return SW_OK;
		};
		if ((r = capture_and_launch(ctx, exec, enqueue))) return r;
		ctx->vkey[slot] = key;
		++ctx->view_captures;
	}
	else
	{
		stage_begin(ctx, STAGE_FRAME);
		SW_CUDA(ctx, cudaGraphLaunch(exec, ctx->stream));
		stage_end(ctx, STAGE_FRAME);
	}
	SW_CUDA(ctx, cudaEventRecord(ctx->ev_counts[slot], ctx->stream));
	ctx->counts_pending[slot] = true;
	ctx->counts_seq[slot] = ++ctx->view_seq;
	ctx->stats.upload_bytes += vb.bytes;
	ctx->last_num_surfaces = 0; // sw_rebuild_surfaces has no host descriptors of this frame
	ctx->last_surface_work = 0;
	r = finish_graph_frame(ctx, st, p, f.postprocess != 0, f.post, f.frame_duration_s, f.dst, f.dst_pitch, f.dst_is_device,
		post_out, direct_host, pslot);
	if (r) return r;
	if (cudaEventQuery(ctx->ev_counts[slot]) == cudaSuccess)
	{
		consume_view_counts(ctx, slot);
		if (ctx->h_counts[slot].error) return fail(ctx, SW_ERR_LIMIT, "GPU-side preparation exceeded a capacity");
	}
	cudaGetLastError();
	return SW_OK;
}

int sw_read_view_prep(SwCtx* ctx, SwViewCounts* out_counts, SwSurfaceDesc* surfaces, uint32_t max_surfaces, SwDrawCmd* draws,
	uint32_t max_draws, SwVertex16* vertices, uint32_t max_vertices)
{
	if (!ctx || !out_counts) return SW_ERR_INVALID_ARGUMENT;
	if (!ctx->v_counts) return fail(ctx, SW_ERR_STATE, "no sw_draw_frame_view yet");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	for (uint32_t k = 0; k < 2; ++k)
		if (ctx->counts_pending[k]) consume_view_counts(ctx, k);
	SwViewCounts k;
	SW_CUDA(ctx, cudaMemcpy(&k, ctx->v_counts, sizeof(k), cudaMemcpyDeviceToHost));
	*out_counts = k;
	const uint32_t ns = std::min(std::min(max_surfaces, k.num_surfaces), ctx->view_surfaces_cap);
	const uint32_t nd = std::min(std::min(max_draws, k.num_draws), ctx->view_draws_cap);
	const uint32_t nv = std::min(std::min(max_vertices, k.num_vertices), ctx->view_vertices_cap);
	if (surfaces && ns) SW_CUDA(ctx, cudaMemcpy(surfaces, ctx->v_descs, size_t(ns) * sizeof(SwSurfaceDesc), cudaMemcpyDeviceToHost));
	if (draws && nd) SW_CUDA(ctx, cudaMemcpy(draws, ctx->v_draws, size_t(nd) * sizeof(SwDrawCmd), cudaMemcpyDeviceToHost));
	if (vertices && nv) SW_CUDA(ctx, cudaMemcpy(vertices, ctx->v_vertices, size_t(nv) * sizeof(SwVertex16), cudaMemcpyDeviceToHost));
	return SW_OK;
}

namespace
{
// Grow a device buffer keeping its contents (the new part zeroed).
int grow_preserve(SwCtx* ctx, DevBuf& b, size_t bytes)
{
	if (b.ptr && b.bytes >= bytes) return SW_OK;
	const size_t want = std::max(bytes, b.bytes + b.bytes / 2);
	void* p = nullptr;
	cudaError_t e = cudaMalloc(&p, want);
	if (e != cudaSuccess)
	{
		cudaGetLastError();
		return fail(ctx, SW_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu bytes) failed: %s", want, cudaGetErrorString(e));
	}
	SW_CUDA(ctx, cudaMemsetAsync(p, 0, want, ctx->stream));
	if (b.ptr)
	{
		SW_CUDA(ctx, cudaMemcpyAsync(p, b.ptr, b.bytes, cudaMemcpyDeviceToDevice, ctx->stream));
		SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
		if (ctx->aux) SW_CUDA(ctx, cudaStreamSynchronize(ctx->aux));
		cudaFree(b.ptr);
	}
	b.ptr = p;
	b.bytes = want;
	return SW_OK;
}
// The shadow-map storage: (sequence << 32 | f32 bits) per texel, grown with its contents kept (new
// texels read 0 with sequence 0).
int grow_shadow_storage(SwCtx* ctx, uint64_t total_texels)
{
	int r = grow_preserve(ctx, ctx->shadow_storage, std::max<uint64_t>(total_texels, 1) * 8);
	if (r) return r;
	ctx->shadow_texels = std::max(ctx->shadow_texels, total_texels);
	return SW_OK;
}

// Sequences of the next `count` depth draws: base + 1 .. base + count, above every sequence in the
// storage; when they would pass 2^32 - 1 the storage drops its sequences (keeping its depths) first.
int shadow_sequence(SwCtx* ctx, uint64_t count, uint32_t* base)
{
	if (uint64_t(ctx->shadow_seq) + count >= 0xFFFFFFFFull)
	{
		int r = check_kernel(ctx, launch_shadow_rebase(static_cast<unsigned long long*>(ctx->shadow_storage.ptr),
			ctx->shadow_texels, ctx->stream), "shadow-map rebase");
		if (r) return r;
		ctx->shadow_seq = 0;
	}
	*base = ctx->shadow_seq;
	ctx->shadow_seq += uint32_t(count);
	return SW_OK;
}
} // namespace

int sw_build_shadow_maps(SwCtx* ctx, const SwDepthDraw* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices, uint64_t total_texels)
{
	if (!ctx || (num_draws && (!draws || !vertices))) return SW_ERR_INVALID_ARGUMENT;
	if (total_texels > (uint64_t(1) << 34)) return fail(ctx, SW_ERR_LIMIT, "shadow-map storage too large");
	for (uint32_t i = 0; i < num_draws; ++i)
	{
		const SwDepthDraw& d = draws[i];
		if (d.vertex_count < 3 || d.vertex_count > SW_MAX_POLYGON_VERTICES || uint64_t(d.first_vertex) + d.vertex_count > num_vertices)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "depth draw %u: bad vertices", i);
		if (d.map_size == 0 || d.map_size > SW_SHADOW_MAX_SIZE || d.map_offset + uint64_t(d.map_size) * d.map_size > total_texels)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "depth draw %u: map outside the storage", i);
	}
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	int r;
	if ((r = grow_shadow_storage(ctx, total_texels))) return r;
	if (num_draws == 0) return SW_OK;
	// draws and vertices in one upload
	const size_t vo = align_up(size_t(num_draws) * sizeof(SwDepthDraw), 256);
	const size_t bytes = vo + size_t(num_vertices) * sizeof(SwVertex16);
	if ((r = ensure(ctx, ctx->up_src, bytes))) return r;
	void* h = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_shadow, bytes, &h))) return r;
	std::memcpy(h, draws, size_t(num_draws) * sizeof(SwDepthDraw));
	std::memcpy(static_cast<unsigned char*>(h) + vo, vertices, size_t(num_vertices) * sizeof(SwVertex16));
	if ((r = staging_commit(ctx, ctx->stage_shadow, ctx->up_src.ptr, bytes))) return r;
	ShadowArgs a;
	std::memset(&a, 0, sizeof(a));
	if ((r = shadow_sequence(ctx, num_draws, &a.seq_base))) return r;
	a.draws = static_cast<const SwDepthDraw*>(ctx->up_src.ptr);
	a.num_draws = num_draws;
	a.vertices = reinterpret_cast<const SwVertex16*>(static_cast<unsigned char*>(ctx->up_src.ptr) + vo);
	a.storage = static_cast<unsigned long long*>(ctx->shadow_storage.ptr);
	return check_kernel(ctx, launch_shadow_maps(a, ctx->stream), "shadow maps");
}

int sw_build_shadow_maps_view(SwCtx* ctx, const SwShadowSide* sides, uint32_t num_sides, const SwShadowLeaf* leafs,
	uint32_t num_leafs, uint64_t total_texels)
{
	if (!ctx || (num_sides && !sides) || (num_leafs && !leafs)) return SW_ERR_INVALID_ARGUMENT;
	if (total_texels > (uint64_t(1) << 34)) return fail(ctx, SW_ERR_LIMIT, "shadow-map storage too large");
	if (num_leafs && !ctx->num_map_polygons) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "no map: call sw_set_map first");
	for (uint32_t i = 0; i < num_sides; ++i)
	{
		const SwShadowSide& sd = sides[i];
		if (sd.map_size == 0 || sd.map_size > SW_SHADOW_MAX_SIZE || sd.map_offset + uint64_t(sd.map_size) * sd.map_size > total_texels)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "shadow side %u: map outside the storage", i);
	}
	uint64_t candidates = 0;
	for (uint32_t i = 0; i < num_leafs; ++i)
	{
		const SwShadowLeaf& l = leafs[i];
		if (l.side >= num_sides) return fail(ctx, SW_ERR_INVALID_ARGUMENT, "shadow leaf %u: no side %u", i, l.side);
		if (uint64_t(l.first_polygon) + l.num_polygons > ctx->num_map_polygons)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "shadow leaf %u: polygons outside the map", i);
		candidates += l.num_polygons;
	}
	if (candidates > (uint64_t(1) << 30)) return fail(ctx, SW_ERR_LIMIT, "too many shadow candidates");
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	int r;
	if ((r = grow_shadow_storage(ctx, total_texels))) return r;
	if (candidates == 0) return SW_OK;
	// sides, leafs and the leafs' first candidates in one upload
	const size_t lo = align_up(size_t(num_sides) * sizeof(SwShadowSide), 256);
	const size_t bo = align_up(lo + size_t(num_leafs) * sizeof(SwShadowLeaf), 256);
	const size_t bytes = bo + size_t(num_leafs) * 4;
	if ((r = ensure(ctx, ctx->up_src, bytes))) return r;
	void* h = nullptr;
	if ((r = staging_acquire(ctx, ctx->stage_shadow, bytes, &h))) return r;
	unsigned char* hb = static_cast<unsigned char*>(h);
	std::memcpy(hb, sides, size_t(num_sides) * sizeof(SwShadowSide));
	std::memcpy(hb + lo, leafs, size_t(num_leafs) * sizeof(SwShadowLeaf));
	uint32_t* base = reinterpret_cast<uint32_t*>(hb + bo);
	uint32_t c = 0;
	for (uint32_t i = 0; i < num_leafs; ++i)
	{
		base[i] = c;
		c += leafs[i].num_polygons;
	}
	if ((r = staging_commit(ctx, ctx->stage_shadow, ctx->up_src.ptr, bytes))) return r;
	unsigned char* db = static_cast<unsigned char*>(ctx->up_src.ptr);
	ShadowViewArgs a;
	std::memset(&a, 0, sizeof(a));
	if ((r = shadow_sequence(ctx, candidates, &a.seq_base))) return r;
	a.sides = reinterpret_cast<const SwShadowSide*>(db);
	a.leafs = reinterpret_cast<const SwShadowLeaf*>(db + lo);
	a.leaf_base = reinterpret_cast<const uint32_t*>(db + bo);
	a.num_leafs = num_leafs;
	a.num_candidates = uint32_t(candidates);
	a.polygons = static_cast<const SwMapPolygon*>(ctx->map_polygons.ptr);
	a.map_vertices = static_cast<const float*>(ctx->map_vertices.ptr);
	a.storage = static_cast<unsigned long long*>(ctx->shadow_storage.ptr);
	return check_kernel(ctx, launch_shadow_view(a, ctx->stream), "shadow maps");
}

int sw_set_light_shadows(SwCtx* ctx, const SwLightShadow* shadows, uint32_t num_lights)
{
	if (!ctx || (num_lights && !shadows)) return SW_ERR_INVALID_ARGUMENT;
	if (num_lights > 65535) return fail(ctx, SW_ERR_LIMIT, "too many lights");
	uint32_t used = 0;
	for (uint32_t i = 0; i < num_lights; ++i)
	{
		const SwLightShadow& m = shadows[i];
		if (m.kind == SW_SHADOW_NONE) continue;
		if (m.kind != SW_SHADOW_CUBE && m.kind != SW_SHADOW_PROJECTOR)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "light %u: unknown shadow kind", i);
		const uint64_t maps = m.kind == SW_SHADOW_CUBE ? 6u : 1u;
		if (m.size == 0 || m.size > SW_SHADOW_MAX_SIZE || m.offset + maps * uint64_t(m.size) * m.size > ctx->shadow_texels)
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "light %u: shadow map outside the shadow-map storage", i);
		if (m.kind == SW_SHADOW_PROJECTOR &&
			!(all_finite(m.basis_x, 3) && all_finite(m.basis_y, 3) && all_finite(m.basis_z, 3)))
			return fail(ctx, SW_ERR_INVALID_ARGUMENT, "light %u: non-finite projector basis", i);
		used = i + 1;
	}
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	ctx->num_shadow_descs = used; // lights past the last shadowed one need no descriptor
	if (!used) return SW_OK;
	int r;
	// projector maps: the corners outside the inscribed circle, after the frame's depth draws
	for (uint32_t i = 0; i < used; ++i)
		if (shadows[i].kind == SW_SHADOW_PROJECTOR)
		{
			uint32_t base = 0;
			if ((r = shadow_sequence(ctx, 1, &base))) return r;
			if ((r = check_kernel(ctx, launch_shadow_circle(static_cast<unsigned long long*>(ctx->shadow_storage.ptr) + shadows[i].offset,
									shadows[i].size, base + 1, ctx->stream),
					 "projector shadow-map circle")))
				return r;
		}
	if ((r = ensure(ctx, ctx->shadow_descs, size_t(used) * sizeof(SwLightShadow)))) return r;
	return upload(ctx, ctx->stage_shadow_descs, ctx->shadow_descs.ptr, shadows, size_t(used) * sizeof(SwLightShadow));
}

int sw_read_shadow_maps(SwCtx* ctx, float* dst, uint64_t max_texels)
{
	if (!ctx || (max_texels && !dst)) return SW_ERR_INVALID_ARGUMENT;
	SW_CUDA(ctx, cudaSetDevice(ctx->device));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	const uint64_t n = std::min(max_texels, ctx->shadow_texels);
	if (!n) return SW_OK;
	std::vector<unsigned long long> packed(n);
	SW_CUDA(ctx, cudaMemcpy(packed.data(), ctx->shadow_storage.ptr, n * 8, cudaMemcpyDeviceToHost));
	for (uint64_t i = 0; i < n; ++i)
	{
		const uint32_t bits = uint32_t(packed[i]);
		std::memcpy(dst + i, &bits, 4);
	}
	return SW_OK;
}

int sw_set_frames_in_flight(SwCtx* ctx, uint32_t frames)
{
	if (!ctx || frames < 1 || frames > 2) return SW_ERR_INVALID_ARGUMENT;
	if (frames == ctx->frames_in_flight) return SW_OK;
	int r;
	if ((r = sw_sync(ctx))) return r; // every frame in flight is in its destination
	ctx->frames_in_flight = frames;
	return SW_OK;
}

int sw_set_frame_graph(SwCtx* ctx, int enable)
{
	if (!ctx) return SW_ERR_INVALID_ARGUMENT;
	ctx->graph_enabled = enable != 0;
	return SW_OK;
}

int sw_set_tuning(SwCtx* ctx, const SwTuning* t)
{
	if (!ctx || !t) return SW_ERR_INVALID_ARGUMENT;
	if (t->raster_tile >= SW_RASTER_TILE_VARIANTS || t->surface_blocks_per_sm < 1 || t->surface_blocks_per_sm > 64 ||
		(t->surface_texels_per_thread != 0 && t->surface_texels_per_thread != 1 && t->surface_texels_per_thread != 4))
		return fail(ctx, SW_ERR_INVALID_ARGUMENT, "tuning out of range");
	if (t->raster_tile != ctx->tuning.raster_tile || t->surface_blocks_per_sm != ctx->tuning.surface_blocks_per_sm ||
		t->surface_texels_per_thread != ctx->tuning.surface_texels_per_thread)
	{
		// other kernels: the frame graph is instantiated anew
		SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
		if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
		ctx->gexec = nullptr;
	}
	ctx->tuning = *t;
	return SW_OK;
}

int sw_get_tuning(SwCtx* ctx, SwTuning* out)
{
	if (!ctx || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = ctx->tuning;
	return SW_OK;
}

int sw_autotune(SwCtx* ctx, const SwFrameInput* sample, uint32_t reps, SwTuning* out_best, float* out_best_ms)
{
	if (!ctx || !sample || reps == 0 || reps > 1000) return SW_ERR_INVALID_ARGUMENT;
	int r;
	if ((r = finalize_exposure(ctx))) return r;
	const float exposure = ctx->exposure;
	const bool timing = ctx->timing;
	const SwTuning start = ctx->tuning;
	if (!ctx->timing && (r = sw_enable_timing(ctx, 1))) return r;
	const uint32_t blocks[] = {8u, 16u, 24u, 32u, 48u};
	// texels per surface thread stay as set: 4 measured slower than 1 on frames (fewer resident warps)
	const uint32_t texels[] = {start.surface_texels_per_thread};
	SwTuning best = start;
	float best_ms = 1e30f;
	std::vector<float> ms(reps);
	for (uint32_t tile = 0; tile < SW_RASTER_TILE_VARIANTS && r == SW_OK; ++tile)
		for (uint32_t bi = 0; bi < sizeof(blocks) / sizeof(blocks[0]) && r == SW_OK; ++bi)
			for (uint32_t ki = 0; ki < sizeof(texels) / sizeof(texels[0]) && r == SW_OK; ++ki)
			{
				const uint32_t b = blocks[bi], k = texels[ki];
				const SwTuning t{tile, b, k, 0u};
				if ((r = sw_set_tuning(ctx, &t))) break;
				for (uint32_t i = 0; i < 2 + reps && r == SW_OK; ++i)
				{
					if ((r = sw_draw_frame(ctx, sample))) break;
					float t5[5];
					if ((r = sw_get_timings(ctx, t5))) break;
					if (i >= 2) ms[i - 2] = t5[STAGE_FRAME];
				}
				if (r) break;
				std::vector<float> sorted = ms;
				std::sort(sorted.begin(), sorted.end());
				const float med = sorted[sorted.size() / 2];
				if (med < best_ms)
				{
					best_ms = med;
					best = t;
				}
			}
	// restore the exposure state and the timing switch; keep the best configuration
	const int r2 = finalize_exposure(ctx);
	ctx->exposure = exposure;
	ctx->exposure_pending = false;
	if (!timing) sw_enable_timing(ctx, 0);
	if (r || r2) return r ? r : r2;
	if ((r = sw_set_tuning(ctx, &best))) return r;
	if (out_best) *out_best = best;
	if (out_best_ms) *out_best_ms = best_ms;
	return SW_OK;
}

int sw_abi_layout(uint32_t* sizes, uint32_t count)
{
	const uint32_t s[27] = {uint32_t(sizeof(SwCreateInfo)), uint32_t(sizeof(SwTextureMip)), uint32_t(sizeof(SwEmissiveMip)),
		uint32_t(sizeof(SwDirectionalLightmapElement)), uint32_t(sizeof(SwLight)), uint32_t(sizeof(SwSurfaceDesc)),
		uint32_t(sizeof(SwVertex16)), uint32_t(sizeof(SwDrawCmd)), uint32_t(sizeof(SwFrameParams)),
		uint32_t(sizeof(SwPostConfig)), uint32_t(sizeof(SwStats)), uint32_t(sizeof(SwFrameInput)), uint32_t(sizeof(SwTuning)),
		uint32_t(sizeof(SwMapPolygon)), uint32_t(sizeof(SwViewLeaf)), uint32_t(sizeof(SwViewFrameInput)),
		uint32_t(sizeof(SwViewCounts)), uint32_t(sizeof(SwLightShadow)), uint32_t(sizeof(SwDepthDraw)),
		uint32_t(sizeof(SwShadowSide)), uint32_t(sizeof(SwShadowLeaf)), uint32_t(sizeof(SwMaterialFrame)),
		uint32_t(sizeof(SwTriVertex)), uint32_t(sizeof(SwTexturePass)), uint32_t(sizeof(SwSimPass)), uint32_t(sizeof(SwSimPoint)),
		uint32_t(sizeof(SwView))};
	for (uint32_t i = 0; sizes && i < count && i < 27; ++i) sizes[i] = s[i];
	return 27;
}

int sw_get_stats(SwCtx* ctx, SwStats* out)
{
	if (!ctx || !out) return SW_ERR_INVALID_ARGUMENT;
	unsigned int errs[4] = {0, 0, 0, 0};
	SW_CUDA(ctx, cudaMemcpyAsync(errs, ctx->error_counter.ptr, 16, cudaMemcpyDeviceToHost, ctx->stream));
	SW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	*out = ctx->stats;
	out->bad_texel_fetches = errs[0];
	out->pixel_writes = uint64_t(errs[2]) | (uint64_t(errs[3]) << 32);
	return SW_OK;
}

} // extern "C"
