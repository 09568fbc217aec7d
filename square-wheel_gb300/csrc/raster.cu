// Tile-binned polygon rasteriser for the GB300 path.
//
// Replaces perform_rasterization's single-thread path (src/square_wheel/partial_renderer.rs:1207-1234)
// running Rasterizer::fill_polygon for each draw in submission order (src/square_wheel/rasterizer.rs:
// 137-729, write_into_framebuffer :1511-1536).
//
// Two launches:
//   raster_setup: one CTA per draw. Thread 0 runs the reference's edge walk (rasterizer.rs:160-270)
//     into the draw's parts and derives its tile-binning box; then the CTA's threads take the draw's
//     (row) records (row ranges and record offsets come from the host): the span [xs, xe) and the
//     start and step of the mode's interpolants (the span setup of rasterizer.rs:329-422 / 513-556 /
//     686-703), evaluated once per (draw, row) over the whole span with the frame as clip rectangle
//     (the reference's num_threads == 1 ClipRect).
//   raster_tiles: one 256-thread CTA per 64x16 tile, each thread a 1x4 pixel strip of one row (about
//     one wave of CTAs at 1080p). The CTA streams over the draws in submission order, 256 at a time;
//     each thread tests one draw's box against the tile and a ballot + prefix sum compacts the hits
//     (with their draw records) into shared memory in order. For batches of 32 hits the CTA stages
//     their 16 rows of this tile in shared memory with parallel loads; every thread then walks the
//     hits in order for its strip: for span pixel i it takes start + i*step (the reference's repeated
//     wrapping addition), the per-pixel z division and the texel address, issues its four texel loads
//     at once and blends them in submission order into registers. Blending order is the reference's,
//     the frame buffer is read and written once, and coverage and texel addresses are bit-exact.
#include "sw_kernels.cuh"
#include "warp_prep.cuh"

#include <algorithm>
#include <atomic>

namespace swgpu
{
namespace
{

typedef int32_t Fixed16;
constexpr Fixed16 FIXED16_ONE = 1 << 16;
constexpr Fixed16 FIXED16_HALF = FIXED16_ONE >> 1;
constexpr int TC_SHIFT = 24;
constexpr int INV_Z_SHIFT = 29;
constexpr int INV_Z_PRE_SHIFT = 8;
constexpr int Z_CALC_SHIFT = 31;
constexpr int TC_FINAL_SHIFT = TC_SHIFT + Z_CALC_SHIFT - INV_Z_SHIFT + INV_Z_PRE_SHIFT; // 34
constexpr float TC_SCALE = float(1 << TC_SHIFT);
constexpr float INV_Z_SCALE = float(1 << INV_Z_SHIFT);


__device__ __forceinline__ Fixed16 int_to_fixed16(int32_t x) { return int32_t(uint32_t(x) << 16); }
__device__ __forceinline__ int32_t round_to_int(Fixed16 x) { return wadd(x, FIXED16_HALF) >> 16; }
__device__ __forceinline__ Fixed16 fx_mul(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) * int64_t(y)) >> 16); }
__device__ __forceinline__ Fixed16 fx_div(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) << 16) / int64_t(y)); }
__device__ __forceinline__ Fixed16 fx_mul_div(Fixed16 x, Fixed16 y, Fixed16 z)
{
	return int32_t(int64_t(x) * int64_t(y) / int64_t(z));
}
__device__ __forceinline__ float fx_to_f32(Fixed16 x) { return __fdiv_rn(float(x), float(FIXED16_ONE)); }
__device__ __forceinline__ Fixed16 f32_to_fx(float x) { return __float2int_rz(fmul(x, float(FIXED16_ONE))); }
__device__ __forceinline__ int64_t f2i64(float x) { return __float2ll_rz(x); }
__device__ __forceinline__ int64_t w64add(int64_t a, int64_t b) { return int64_t(uint64_t(a) + uint64_t(b)); }
__device__ __forceinline__ int64_t w64mul(int64_t a, int64_t b) { return int64_t(uint64_t(a) * uint64_t(b)); }

// The draw_func body up to the row loop: first-row edge positions (rasterizer.rs:316-320) and, for
// the affine mode, the per-part texture coordinate edges (rasterizer.rs:597-682). False when the part
// has no row in the frame (the reference's loop runs no iteration).
__device__ bool make_part(const SwDrawCmd& d, int32_t height, Fixed16 y_start, Fixed16 y_end, Fixed16 xl_start, Fixed16 dxl,
	Fixed16 xr_start, Fixed16 dxr, RasterPart& p)
{
	const int32_t y_start_int = max(round_to_int(y_start), 0);
	const int32_t y_end_int = min(round_to_int(y_end), height);
	if (y_start_int >= y_end_int) return false;
	const Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
	p.y_start_int = y_start_int;
	p.y_end_int = y_end_int;
	p.x_left0 = wadd(wadd(xl_start, fx_mul(y_start_delta, dxl)), FIXED16_HALF);
	p.x_right0 = wadd(wadd(xr_start, fx_mul(y_start_delta, dxr)), FIXED16_HALF);
	p.dx_dy_left = dxl;
	p.dx_dy_right = dxr;
	p.tc_left0[0] = p.tc_left0[1] = p.tc_right0[0] = p.tc_right0[1] = 0;
	p.d_tc_left[0] = p.d_tc_left[1] = p.d_tc_right[0] = p.d_tc_right[1] = 0;
	if (d.mode == SW_RASTER_AFFINE)
	{
		const float* de = d.depth_eq;
		const float* te = d.tc_eq;
		const float y_start_f = fx_to_f32(y_start);
		const float y_end_f = fx_to_f32(y_end);
		const Fixed16 y_delta = wsub(y_end, y_start);
		const float x_start_left = fx_to_f32(xl_start);
		const float x_end_left = fx_to_f32(wadd(xl_start, fx_mul(y_delta, dxl)));
		const float x_start_right = fx_to_f32(xr_start);
		const float x_end_right = fx_to_f32(wadd(xr_start, fx_mul(y_delta, dxr)));
		auto inv_depth = [&](float x, float y) { return fadd(fadd(fmul(de[0], x), fmul(de[1], y)), de[2]); };
		const float z_sl = __fdiv_rn(1.0f, inv_depth(x_start_left, y_start_f));
		const float z_el = __fdiv_rn(1.0f, inv_depth(x_end_left, y_end_f));
		const float z_sr = __fdiv_rn(1.0f, inv_depth(x_start_right, y_start_f));
		const float z_er = __fdiv_rn(1.0f, inv_depth(x_end_right, y_end_f));
		const Fixed16 y_delta_tc = max(y_delta, FIXED16_ONE);
#pragma unroll
		for (int i = 0; i < 2; ++i)
		{
			const Fixed16 max_tc = wsub(int_to_fixed16(int32_t(i == 0 ? d.tex_size[0] : d.tex_size[1])), 1);
			auto tc_at = [&](float z, float x, float y) {
				return min(max(f32_to_fx(fmul(z, fadd(fadd(fmul(x, te[i]), fmul(y, te[2 + i])), te[4 + i]))), 0), max_tc);
			};
			const Fixed16 tsl = tc_at(z_sl, x_start_left, y_start_f);
			const Fixed16 tel = tc_at(z_el, x_end_left, y_end_f);
			const Fixed16 tsr = tc_at(z_sr, x_start_right, y_start_f);
			const Fixed16 ter = tc_at(z_er, x_end_right, y_end_f);
			p.d_tc_left[i] = fx_div(wsub(tel, tsl), y_delta_tc);
			p.d_tc_right[i] = fx_div(wsub(ter, tsr), y_delta_tc);
			p.tc_left0[i] = wadd(tsl, fx_mul(y_start_delta, p.d_tc_left[i]));
			p.tc_right0[i] = wadd(tsr, fx_mul(y_start_delta, p.d_tc_right[i]));
		}
	}
	return true;
}

// Edge walk of fill_polygon_impl_2_static_params (rasterizer.rs:160-270) for one draw, by one warp.
// The walk's control flow (which edges pair up between which y values) is cheap and sequential: lane 0
// records its steps. The costly part of every step - the 64-bit fixed-point divisions and, for affine
// draws, the texture-coordinate edges with their f32 divisions - is independent from step to step, so
// the lanes compute the steps' parts in parallel and an in-order compaction keeps the parts that have
// rows, at most SW_RASTER_MAX_PARTS of them, in the walk's order.
struct WalkStep
{
	Fixed16 cur_y, next_y;
	uint8_t li, nli, ri, nri;
	uint32_t kind; // 1: both edges taller than half a pixel, 2: a thin part
};
constexpr uint32_t MAX_WALK_STEPS = 2 * SW_MAX_POLYGON_VERTICES + 2;

template <class F>
__device__ __forceinline__ void walk(const SwVertex16* vtx, uint32_t n, F&& on_step)
{
	uint32_t lower = 0;
	Fixed16 min_y = vtx[0].y;
	for (uint32_t i = 0; i < n; ++i)
		if (vtx[i].y < min_y)
		{
			min_y = vtx[i].y;
			lower = i;
		}
	uint32_t li = lower, ri = lower;
	Fixed16 cur_y = min_y;
	for (uint32_t guard = 0; guard < MAX_WALK_STEPS; ++guard)
	{
		uint32_t nli = li + n - 1;
		if (nli >= n) nli -= n;
		uint32_t nri = ri + 1;
		if (nri >= n) nri -= n;
		const Fixed16 dy_left = wsub(vtx[nli].y, vtx[li].y);
		const Fixed16 dy_right = wsub(vtx[nri].y, vtx[ri].y);
		const Fixed16 next_y = min(vtx[nli].y, vtx[nri].y);
		uint32_t kind = 0;
		if (dy_left > FIXED16_HALF && dy_right > FIXED16_HALF)
			kind = 1;
		else if (dy_left > 0 && dy_right > 0 && round_to_int(cur_y) < round_to_int(next_y))
			kind = 2;
		if (kind) on_step(WalkStep{cur_y, next_y, uint8_t(li), uint8_t(nli), uint8_t(ri), uint8_t(nri), kind});
		if (nli == nri) break;
		if (vtx[nri].y < vtx[nli].y)
			ri = nri;
		else
			li = nli;
		cur_y = next_y;
	}
}

// A step's part (the divisions of the walk's loop body); false when it has no row in the frame.
__device__ __forceinline__ bool step_part(const SwDrawCmd& d, const SwVertex16* vtx, int32_t height, const WalkStep& st, RasterPart& p)
{
	const SwVertex16 lv = vtx[st.li], nlv = vtx[st.nli], rv = vtx[st.ri], nrv = vtx[st.nri];
	const Fixed16 dy_left = wsub(nlv.y, lv.y), dy_right = wsub(nrv.y, rv.y);
	if (st.kind == 1)
	{
		const Fixed16 dxl = fx_div(wsub(nlv.x, lv.x), dy_left);
		const Fixed16 dxr = fx_div(wsub(nrv.x, rv.x), dy_right);
		return make_part(d, height, st.cur_y, st.next_y, wadd(lv.x, fx_mul(dxl, wsub(st.cur_y, lv.y))), dxl,
			wadd(rv.x, fx_mul(dxr, wsub(st.cur_y, rv.y))), dxr, p);
	}
	const Fixed16 thin_y = wadd(int_to_fixed16(round_to_int(st.cur_y)), FIXED16_HALF);
	const Fixed16 xsl = wadd(lv.x, fx_mul_div(wsub(thin_y, lv.y), wsub(nlv.x, lv.x), dy_left));
	const Fixed16 xsr = wadd(rv.x, fx_mul_div(wsub(thin_y, rv.y), wsub(nrv.x, rv.x), dy_right));
	return make_part(d, height, st.cur_y, st.next_y, xsl, 0, xsr, 0, p);
}

// One warp: the draw's parts into `parts`; returns their count (to every lane).
__device__ uint32_t edge_walk_warp(const SwDrawCmd& d, const SwVertex16* vtx, int32_t height, RasterPart* parts, WalkStep* steps,
	uint32_t* s_count)
{
	const uint32_t lane = threadIdx.x & 31u;
	if (lane == 0)
	{
		uint32_t count = 0;
		walk(vtx, d.vertex_count, [&](const WalkStep& st) { steps[count++] = st; });
		*s_count = count;
	}
	__syncwarp();
	const uint32_t count = *s_count;
	uint32_t np = 0;
	for (uint32_t base = 0; base < count; base += 32)
	{
		const uint32_t k = base + lane;
		RasterPart p;
		const bool ok = k < count && step_part(d, vtx, height, steps[k], p);
		const unsigned mask = __ballot_sync(0xFFFFFFFFu, ok);
		const uint32_t pos = np + __popc(mask & ((1u << lane) - 1u));
		if (ok && pos < SW_RASTER_MAX_PARTS) parts[pos] = p;
		np += __popc(mask);
	}
	__syncwarp();
	return np < SW_RASTER_MAX_PARTS ? np : SW_RASTER_MAX_PARTS;
}

// The same walk by one thread (the shadow-map kernels draw one candidate per warp or per block and
// keep their shared memory small): the steps and their parts one after another.
__device__ uint32_t edge_walk(const SwDrawCmd& d, const SwVertex16* vtx, int32_t height, RasterPart* parts)
{
	uint32_t np = 0;
	walk(vtx, d.vertex_count, [&](const WalkStep& st) {
		if (np < SW_RASTER_MAX_PARTS && step_part(d, vtx, height, st, parts[np])) ++np;
	});
	return np;
}

// ---- triangles: Rasterizer::fill_triangle_impl / fill_triangle_part (rasterizer.rs:765-1292) ----

// fill_triangle_part's prologue (rasterizer.rs:984-1186): the part's rows clipped to the frame, its
// first-row edges and the texture-coordinate and light corrections, into one RasterPart (no part when
// it has no row).
__device__ void triangle_part(RasterPart* parts, uint32_t& np, int32_t height, Fixed16 y_start, Fixed16 y_end, Fixed16 xl_start,
	Fixed16 dxl, Fixed16 xr_start, Fixed16 dxr, const Fixed16* tc_start_left, const Fixed16* d_tc_dy_left_in,
	const Fixed16* d_tc_dx_in, const Fixed16* light_start_left, const Fixed16* d_light_left_in, const Fixed16* d_light_dx_in,
	int32_t tex_w, int32_t tex_h)
{
	const int32_t y_start_int = max(round_to_int(y_start), 0);
	const int32_t y_end_int = min(round_to_int(y_end), height);
	if (y_start_int >= y_end_int) return;
	Fixed16 d_tc_dy_left[2] = {d_tc_dy_left_in[0], d_tc_dy_left_in[1]};
	Fixed16 d_tc_dx[2] = {d_tc_dx_in[0], d_tc_dx_in[1]};
	Fixed16 d_light_left[3] = {d_light_left_in[0], d_light_left_in[1], d_light_left_in[2]};
	Fixed16 d_light_dx[3] = {d_light_dx_in[0], d_light_dx_in[1], d_light_dx_in[2]};
	const Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
	const Fixed16 x_left = wadd(wadd(xl_start, fx_mul(y_start_delta, dxl)), FIXED16_HALF);
	const Fixed16 x_right = wadd(wadd(xr_start, fx_mul(y_start_delta, dxr)), FIXED16_HALF);
	const Fixed16 y_end_delta = wsub(y_end, wadd(y_start, y_start_delta));
	const Fixed16 d_x_lower = max(wsub(x_right, x_left), 0);
	const Fixed16 x_upper_left = wadd(x_left, fx_mul(y_end_delta, dxl));
	const Fixed16 x_upper_right = wadd(x_right, fx_mul(y_end_delta, dxr));
	const Fixed16 d_x_upper = max(wsub(x_upper_right, x_upper_left), 0);

	Fixed16 tc_left[2];
	const int32_t tex_size[2] = {tex_w, tex_h};
#pragma unroll
	for (int i = 0; i < 2; ++i)
	{
		const Fixed16 max_tc = wsub(int_to_fixed16(tex_size[i]), 1);
		tc_left[i] = min(max(wadd(tc_start_left[i], fx_mul(y_start_delta, d_tc_dy_left[i])), 0), max_tc);
		const Fixed16 tc_lower_delta = fx_mul(d_tc_dx[i], d_x_lower);
		if (tc_lower_delta > max_tc)
		{
			tc_left[i] = 0;
			d_tc_dx[i] = fx_div(max_tc, d_x_lower);
		}
		else if (tc_lower_delta < -max_tc)
		{
			tc_left[i] = max_tc;
			d_tc_dx[i] = fx_div(-max_tc, d_x_lower);
		}
		else
		{
			const Fixed16 tc_lower_right = wadd(tc_left[i], tc_lower_delta);
			if (tc_lower_right > max_tc)
				tc_left[i] = wsub(tc_left[i], wsub(tc_lower_right, max_tc));
			else if (tc_lower_right < 0)
				tc_left[i] = wsub(tc_left[i], tc_lower_right);
		}
		Fixed16 tc_upper_left = min(max(wadd(tc_left[i], fx_mul(y_end_delta, d_tc_dy_left[i])), 0), max_tc);
		const Fixed16 tc_upper_delta = fx_mul(d_tc_dx[i], d_x_upper);
		if (tc_upper_delta > max_tc)
		{
			tc_upper_left = 0;
			d_tc_dx[i] = fx_div(max_tc, d_x_upper);
		}
		else if (tc_upper_delta < -max_tc)
		{
			tc_upper_left = max_tc;
			d_tc_dx[i] = fx_div(-max_tc, d_x_upper);
		}
		else
		{
			const Fixed16 tc_upper_right = wadd(tc_upper_left, tc_upper_delta);
			if (tc_upper_right > max_tc)
				tc_upper_left = wsub(tc_upper_left, wsub(tc_upper_right, max_tc));
			else if (tc_upper_right < 0)
				tc_upper_left = wsub(tc_upper_left, tc_upper_right);
		}
		d_tc_dy_left[i] = y_end_delta > 0 ? fx_div(wsub(tc_upper_left, tc_left[i]), y_end_delta) : 0;
		const Fixed16 tul = wadd(tc_left[i], fx_mul(y_end_delta, d_tc_dy_left[i]));
		const Fixed16 tur = wadd(tul, fx_mul(d_tc_dx[i], d_x_upper));
		if (tur < 0)
			d_tc_dx[i] = d_x_upper > 0 ? fx_div(-tul, d_x_upper) : 0;
		else if (tur > max_tc)
			d_tc_dx[i] = d_x_upper > 0 ? fx_div(wsub(max_tc, tul), d_x_upper) : 0;
	}
	Fixed16 light_left[3];
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		light_left[i] = max(wadd(light_start_left[i], fx_mul(y_start_delta, d_light_left[i])), 0);
		const Fixed16 llr = wadd(light_left[i], fx_mul(d_x_lower, d_light_dx[i]));
		if (llr < 0) light_left[i] = wsub(light_left[i], llr);
		Fixed16 lul = max(wadd(light_left[i], fx_mul(y_end_delta, d_light_left[i])), 0);
		const Fixed16 lur = wadd(lul, fx_mul(d_x_upper, d_light_dx[i]));
		if (lur < 0) lul = wsub(lul, lur);
		d_light_left[i] = y_end_delta > 0 ? fx_div(wsub(lul, light_left[i]), y_end_delta) : 0;
		const Fixed16 lul2 = wadd(light_left[i], fx_mul(y_end_delta, d_light_left[i]));
		const Fixed16 lur2 = wadd(lul2, fx_mul(d_x_upper, d_light_dx[i]));
		if (lur2 < 0) d_light_dx[i] = d_x_upper > 0 ? fx_div(-lul2, d_x_upper) : 0;
	}
	RasterPart p;
	p.y_start_int = y_start_int;
	p.y_end_int = y_end_int;
	p.x_left0 = x_left;
	p.x_right0 = x_right;
	p.dx_dy_left = dxl;
	p.dx_dy_right = dxr;
#pragma unroll
	for (int i = 0; i < 2; ++i)
	{
		p.tc_left0[i] = tc_left[i];
		p.d_tc_left[i] = d_tc_dy_left[i];
		p.tc_right0[i] = d_tc_dx[i]; // the per-pixel step
		p.d_tc_right[i] = 0;
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		p.light_left0[i] = light_left[i];
		p.d_light_left[i] = d_light_left[i];
		p.d_light_dx[i] = d_light_dx[i];
	}
	parts[np++] = p;
}

// fill_triangle_impl (rasterizer.rs:765-950): vertices sorted by y, the long edge, the interpolants'
// slopes, and the two parts on either side of the middle vertex.
__device__ uint32_t triangle_setup(const SwTriVertex* v, int32_t tex_w, int32_t tex_h, int32_t height, RasterPart* parts)
{
	int ui, li;
	if (v[0].y >= v[1].y && v[0].y >= v[2].y)
	{
		ui = 0;
		li = v[1].y < v[2].y ? 1 : 2;
	}
	else if (v[1].y >= v[0].y && v[1].y >= v[2].y)
	{
		ui = 1;
		li = v[0].y < v[2].y ? 0 : 2;
	}
	else
	{
		ui = 2;
		li = v[0].y < v[1].y ? 0 : 1;
	}
	const SwTriVertex up = v[ui], lo = v[li], mid = v[3 - ui - li];
	const Fixed16 long_dy = max(wsub(up.y, lo.y), FIXED16_HALF);
	const Fixed16 lower_dy = max(wsub(mid.y, lo.y), FIXED16_HALF);
	const Fixed16 upper_dy = max(wsub(up.y, mid.y), FIXED16_HALF);
	const Fixed16 long_dx_dy = fx_div(wsub(up.x, lo.x), long_dy);
	const Fixed16 long_x_mid = wadd(lo.x, fx_mul(long_dx_dy, wsub(mid.y, lo.y)));
	const Fixed16 lower_dx_dy = fx_div(wsub(mid.x, lo.x), lower_dy);
	const Fixed16 upper_dx_dy = fx_div(wsub(up.x, mid.x), upper_dy);
	Fixed16 long_d_tc[2], long_tc_mid[2], d_tc_lower[2], d_tc_upper[2];
#pragma unroll
	for (int i = 0; i < 2; ++i)
	{
		long_d_tc[i] = fx_div(wsub(up.tc[i], lo.tc[i]), long_dy);
		long_tc_mid[i] = wadd(lo.tc[i], fx_mul(long_d_tc[i], lower_dy));
		d_tc_lower[i] = fx_div(wsub(mid.tc[i], lo.tc[i]), lower_dy);
		d_tc_upper[i] = fx_div(wsub(up.tc[i], mid.tc[i]), upper_dy);
	}
	Fixed16 long_d_light[3], long_light_mid[3], d_light_lower[3], d_light_upper[3];
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		long_d_light[i] = fx_div(wsub(up.light[i], lo.light[i]), long_dy);
		long_light_mid[i] = wadd(lo.light[i], fx_mul(long_d_light[i], lower_dy));
		d_light_lower[i] = fx_div(wsub(mid.light[i], lo.light[i]), lower_dy);
		d_light_upper[i] = fx_div(wsub(up.light[i], mid.light[i]), upper_dy);
	}
	uint32_t np = 0;
	Fixed16 d_tc_dx[2], d_light_dx[3];
	if (long_x_mid >= mid.x)
	{
		const Fixed16 middle_dx = max(wsub(long_x_mid, mid.x), FIXED16_HALF);
#pragma unroll
		for (int i = 0; i < 2; ++i) d_tc_dx[i] = fx_div(wsub(long_tc_mid[i], mid.tc[i]), middle_dx);
#pragma unroll
		for (int i = 0; i < 3; ++i) d_light_dx[i] = fx_div(wsub(long_light_mid[i], mid.light[i]), middle_dx);
		triangle_part(parts, np, height, lo.y, mid.y, lo.x, lower_dx_dy, lo.x, long_dx_dy, lo.tc, d_tc_lower, d_tc_dx, lo.light,
			d_light_lower, d_light_dx, tex_w, tex_h);
		triangle_part(parts, np, height, mid.y, up.y, mid.x, upper_dx_dy, long_x_mid, long_dx_dy, mid.tc, d_tc_upper, d_tc_dx,
			mid.light, d_light_upper, d_light_dx, tex_w, tex_h);
	}
	else
	{
		const Fixed16 middle_dx = max(wsub(mid.x, long_x_mid), FIXED16_HALF);
#pragma unroll
		for (int i = 0; i < 2; ++i) d_tc_dx[i] = fx_div(wsub(mid.tc[i], long_tc_mid[i]), middle_dx);
#pragma unroll
		for (int i = 0; i < 3; ++i) d_light_dx[i] = fx_div(wsub(mid.light[i], long_light_mid[i]), middle_dx);
		triangle_part(parts, np, height, lo.y, mid.y, lo.x, long_dx_dy, lo.x, lower_dx_dy, lo.tc, long_d_tc, d_tc_dx, lo.light,
			long_d_light, d_light_dx, tex_w, tex_h);
		triangle_part(parts, np, height, mid.y, up.y, long_x_mid, long_dx_dy, mid.x, upper_dx_dy, long_tc_mid, long_d_tc,
			d_tc_dx, long_light_mid, long_d_light, d_light_dx, tex_w, tex_h);
	}
	return np;
}

// A triangle part's row (rasterizer.rs:1188-1212): the span and its first pixel's texture coordinates
// and light; the reference's per-row additions are start + k * step in wrapping i32 arithmetic.
__device__ RasterRow triangle_row(const RasterPart& p, int32_t y, int32_t width, uint32_t steps_index)
{
	RasterRow r;
	r.a0 = r.b0 = r.a1 = r.b1 = r.a2 = 0;
	r.b2 = int32_t(steps_index);
	const int32_t k = y - p.y_start_int;
	const Fixed16 x_left = wadd(p.x_left0, wmul(k, p.dx_dy_left));
	const Fixed16 x_right = wadd(p.x_right0, wmul(k, p.dx_dy_right));
	r.xs = max(x_left >> 16, 0);
	r.xe = min(x_right >> 16, width);
	if (r.xs >= r.xe) return r;
	const Fixed16 x_start_delta = wsub(wadd(int_to_fixed16(r.xs), FIXED16_ONE), x_left);
	r.a0 = wadd(wadd(p.tc_left0[0], wmul(k, p.d_tc_left[0])), fx_mul(x_start_delta, p.tc_right0[0]));
	r.b0 = wadd(wadd(p.tc_left0[1], wmul(k, p.d_tc_left[1])), fx_mul(x_start_delta, p.tc_right0[1]));
	r.a1 = wadd(wadd(p.light_left0[0], wmul(k, p.d_light_left[0])), fx_mul(x_start_delta, p.d_light_dx[0]));
	r.b1 = wadd(wadd(p.light_left0[1], wmul(k, p.d_light_left[1])), fx_mul(x_start_delta, p.d_light_dx[1]));
	r.a2 = wadd(wadd(p.light_left0[2], wmul(k, p.d_light_left[2])), fx_mul(x_start_delta, p.d_light_dx[2]));
	return r;
}

// Integer plane equations of fill_polygon_part* (rasterizer.rs:287-310).
struct DrawEq
{
	int64_t d_inv_z_dx, d_inv_z_dy, inv_z_k;
	int64_t d_tc_dx[2], d_tc_dy[2], tc_k[2];
};

__device__ __forceinline__ DrawEq draw_equations(const SwDrawCmd& d)
{
	DrawEq e;
	const float* de = d.depth_eq;
	const float* te = d.tc_eq;
	e.d_inv_z_dx = f2i64(fmul(INV_Z_SCALE, de[0]));
	e.d_inv_z_dy = f2i64(fmul(INV_Z_SCALE, de[1]));
	e.inv_z_k = f2i64(fmul(INV_Z_SCALE, fadd(de[2], fmul(fadd(de[0], de[1]), 0.5f))));
#pragma unroll
	for (int i = 0; i < 2; ++i)
	{
		e.d_tc_dx[i] = f2i64(fmul(TC_SCALE, te[i]));
		e.d_tc_dy[i] = f2i64(fmul(TC_SCALE, te[2 + i]));
		e.tc_k[i] = f2i64(fmul(TC_SCALE, fadd(te[4 + i], fmul(fadd(te[i], te[2 + i]), 0.5f))));
	}
	return e;
}

// Span setup of one row (rasterizer.rs:329-422 full perspective, :513-556 line-z, :686-703 affine),
// evaluated over the whole span with the frame as clip rectangle.
__device__ RasterRow row_setup(const SwDrawCmd& d, const DrawEq& e, const RasterPart& p, int32_t y, int32_t width)
{
	RasterRow r;
	r.a0 = r.b0 = r.a1 = r.b1 = r.a2 = r.b2 = 0;
	const int32_t k = y - p.y_start_int;
	const Fixed16 x_left = wadd(p.x_left0, wmul(k, p.dx_dy_left));
	const Fixed16 x_right = wadd(p.x_right0, wmul(k, p.dx_dy_right));
	const int32_t xs = max(x_left >> 16, 0);
	const int32_t xe = min(x_right >> 16, width);
	r.xs = xs;
	r.xe = xe;
	if (xs >= xe) return r;
	const int32_t len1 = (xe - 1) - xs;
	const int64_t span_start_x = xs, span_end_x = xe - 1;
	if (d.mode == SW_RASTER_AFFINE)
	{
		const Fixed16 x_delta = max(wsub(x_right, x_left), FIXED16_ONE);
		const int32_t tcl0 = wadd(p.tc_left0[0], wmul(k, p.d_tc_left[0]));
		const int32_t tcl1 = wadd(p.tc_left0[1], wmul(k, p.d_tc_left[1]));
		const int32_t tcr0 = wadd(p.tc_right0[0], wmul(k, p.d_tc_right[0]));
		const int32_t tcr1 = wadd(p.tc_right0[1], wmul(k, p.d_tc_right[1]));
		r.a1 = tcl0;
		r.b1 = fx_div(wsub(tcr0, tcl0), x_delta);
		r.a2 = tcl1;
		r.b2 = fx_div(wsub(tcr1, tcl1), x_delta);
		return r;
	}
	const int64_t line_inv_z = w64add(w64mul(int64_t(y), e.d_inv_z_dy), e.inv_z_k);
	const int64_t inv_z_min = 1 << INV_Z_PRE_SHIFT, inv_z_max = 1 << 29;
	if (d.mode == SW_RASTER_LINE_Z_CORRECTED)
	{
		const uint32_t izs = uint32_t(min(max(w64add(w64mul(span_start_x, e.d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
		const uint32_t ize = uint32_t(min(max(w64add(w64mul(span_end_x, e.d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
		const uint64_t zs = (1u << Z_CALC_SHIFT) / (izs >> INV_Z_PRE_SHIFT);
		const uint64_t ze = (1u << Z_CALC_SHIFT) / (ize >> INV_Z_PRE_SHIFT);
		int32_t start[2], step[2];
#pragma unroll
		for (int c = 0; c < 2; ++c)
		{
			const int64_t line_tc = w64add(w64mul(int64_t(y), e.d_tc_dy[c]), e.tc_k[c]);
			const uint64_t ts = uint64_t(max(w64add(line_tc, w64mul(span_start_x, e.d_tc_dx[c])), int64_t(0)));
			const uint64_t te = uint64_t(max(w64add(line_tc, w64mul(span_end_x, e.d_tc_dx[c])), int64_t(0)));
			const uint64_t max_tc = (uint64_t(d.tex_size[c]) << 16) - 1;
			const int32_t s0 = int32_t(min((zs * ts) >> (TC_FINAL_SHIFT - 16), max_tc));
			const int32_t s1 = int32_t(min((ze * te) >> (TC_FINAL_SHIFT - 16), max_tc));
			start[c] = s0;
			step[c] = len1 > 0 ? (s1 - s0) / len1 : 0;
		}
		r.a1 = start[0];
		r.b1 = step[0];
		r.a2 = start[1];
		r.b2 = step[1];
		return r;
	}
	// Full perspective.
	const int32_t izs = int32_t(max(inv_z_min, min(w64add(w64mul(span_start_x, e.d_inv_z_dx), line_inv_z), inv_z_max)));
	const int32_t ize = int32_t(max(inv_z_min, min(w64add(w64mul(span_end_x, e.d_inv_z_dx), line_inv_z), inv_z_max)));
	const int32_t d_inv_z = len1 > 0 ? (ize - izs) / len1 : 0;
	const int64_t izc = int64_t(izs - (1 << INV_Z_PRE_SHIFT));
	const int tc_max_shift = INV_Z_SHIFT - TC_SHIFT;
	const int64_t tc_max_max = 1 << 29;
	int32_t start[2], step[2];
#pragma unroll
	for (int c = 0; c < 2; ++c)
	{
		const int64_t size = int64_t(d.tex_size[c]);
		const int64_t line_tc = w64add(w64mul(int64_t(y), e.d_tc_dy[c]), e.tc_k[c]);
		const int64_t tc_max_start = max(int64_t(0), min((w64mul(izc, size) >> tc_max_shift) - 1, tc_max_max));
		const int32_t tcs = int32_t(max(int64_t(0), min(w64add(w64mul(span_start_x, e.d_tc_dx[c]), line_tc), tc_max_start)));
		int32_t s = tcs, st = 0;
		if (len1 > 0)
		{
			const int64_t tc_max_end =
				max(int64_t(0), min((w64mul(izc + int64_t(wmul(d_inv_z, len1)), size) >> tc_max_shift) - 1, tc_max_max));
			const int32_t tce = int32_t(max(int64_t(0), min(w64add(w64mul(span_end_x, e.d_tc_dx[c]), line_tc), tc_max_end)));
			st = (tce - tcs) / len1;
			s = tce > tcs ? tcs : wsub(tce, wmul(st, len1));
		}
		start[c] = s;
		step[c] = st;
	}
	r.a0 = izs;
	r.b0 = d_inv_z;
	r.a1 = start[0];
	r.b1 = step[0];
	r.a2 = start[1];
	r.b2 = step[1];
	return r;
}

// Raster setup of one draw per CTA. The draw and its vertices are staged in shared memory; thread 0
// runs the edge walk into shared memory (its loop reads vertices on the walk's dependency chain, which
// from shared memory costs a few cycles per step) and writes the draw's tile-binning box (conservative:
// x is linear in the row, so its extremes over a part are at the part's first and last rows) and the
// per-draw record of the tile kernel; then every thread sets up rows of the draw (its row records,
// numbered by the host in draw order) from those parts.
__global__ void __launch_bounds__(256) raster_setup_kernel(RasterArgs a)
{
	__shared__ __align__(8) SwDrawCmd s_d;
	__shared__ SwVertex16 s_v[SW_MAX_POLYGON_VERTICES];
	__shared__ SwTriVertex s_tv[3];
	__shared__ RasterPart s_parts[SW_RASTER_MAX_PARTS];
	__shared__ DrawRows s_dr;
	__shared__ uint32_t s_np, s_steps_count;
	__shared__ WalkStep s_steps[MAX_WALK_STEPS];
	// One draw per CTA; with the draw count on the device (GPU-side preparation) a fixed grid strides.
	const uint32_t num_draws = a.counts ? a.counts->num_draws : a.num_draws;
	for (uint32_t di = blockIdx.x; di < num_draws; di += gridDim.x)
	{
		static_assert(sizeof(SwDrawCmd) % 4 == 0 && sizeof(SwDrawCmd) / 4 <= 256, "draw record");
		if (threadIdx.x < sizeof(SwDrawCmd) / 4)
			reinterpret_cast<uint32_t*>(&s_d)[threadIdx.x] = reinterpret_cast<const uint32_t*>(a.draws + di)[threadIdx.x];
		if (threadIdx.x == 0) s_dr = a.draw_rows[di];
		__syncthreads();
		const bool tri = s_d.mode == SW_RASTER_TRIANGLE;
		if (tri)
		{
			if (threadIdx.x < 3) s_tv[threadIdx.x] = a.tri_vertices[s_d.first_vertex + threadIdx.x];
		}
		else if (threadIdx.x < s_d.vertex_count && threadIdx.x < SW_MAX_POLYGON_VERTICES)
			s_v[threadIdx.x] = a.vertices[s_d.first_vertex + threadIdx.x];
		__syncthreads();
		uint32_t walked = 0;
		if (!tri && threadIdx.x < 32) walked = edge_walk_warp(s_d, s_v, a.height, s_parts, s_steps, &s_steps_count);
		if (threadIdx.x == 0)
		{
			const SwDrawCmd& d = s_d;
			uint32_t np;
			if (tri)
			{
				np = triangle_setup(s_tv, int32_t(d.tex_size[0]), int32_t(d.tex_size[1]), a.height, s_parts);
				for (uint32_t pi = 0; pi < np; ++pi)
				{
					TriSteps ts;
					ts.d_tc_dx[0] = s_parts[pi].tc_right0[0];
					ts.d_tc_dx[1] = s_parts[pi].tc_right0[1];
					for (int i = 0; i < 3; ++i) ts.d_light_dx[i] = s_parts[pi].d_light_dx[i];
					ts.reserved = 0;
					a.tri_steps[uint64_t(di) * 2 + pi] = ts;
				}
			}
			else
				np = walked;
			s_np = np;
			int32_t bx0 = INT32_MAX, bx1 = INT32_MIN, by0 = INT32_MAX, by1 = INT32_MIN;
			for (uint32_t pi = 0; pi < np; ++pi)
			{
				const RasterPart& p = s_parts[pi];
				const int32_t last = p.y_end_int - 1 - p.y_start_int;
				bx0 = min(bx0, min(p.x_left0 >> 16, wadd(p.x_left0, wmul(last, p.dx_dy_left)) >> 16));
				bx1 = max(bx1, max(p.x_right0 >> 16, wadd(p.x_right0, wmul(last, p.dx_dy_right)) >> 16));
				by0 = min(by0, p.y_start_int);
				by1 = max(by1, p.y_end_int);
			}
			bx0 = max(bx0, 0);
			bx1 = min(bx1, a.width);
			const DrawRows dr = s_dr;
			// Rows outside the host's row range have no record; clamp the box to it.
			by0 = max(by0, dr.y0);
			by1 = min(by1, dr.y0 + int32_t(dr.nrows));
			a.boxes[di] = (np > 0 && bx0 < bx1 && by0 < by1) ? RasterBox{int16_t(bx0), int16_t(by0), int16_t(bx1), int16_t(by1)}
																: RasterBox{0, 0, 0, 0};
			RasterDraw rd;
			rd.tex_offset = d.tex_offset;
			rd.tex_w = d.tex_size[0];
			rd.tex_h = d.tex_size[1];
			rd.row_base = dr.row_base;
			rd.y0 = dr.y0;
			rd.mode = d.mode;
			rd.blend = uint16_t(d.blend);
			rd.tex_source = uint16_t(d.tex_source);
			a.rdraws[di] = rd;
		}
		__syncthreads();
		const uint32_t np = s_np;
		const DrawEq e = draw_equations(s_d);
		const DrawRows dr = s_dr;
		for (uint32_t k = threadIdx.x; k < dr.nrows; k += blockDim.x)
		{
			const int32_t y = dr.y0 + int32_t(k);
			RasterRow row;
			row.xs = row.xe = 0;
			row.a0 = row.b0 = row.a1 = row.b1 = row.a2 = row.b2 = 0;
			for (uint32_t pi = 0; pi < np; ++pi)
			{
				const RasterPart& p = s_parts[pi];
				if (y >= p.y_start_int && y < p.y_end_int)
				{
					row = s_d.mode == SW_RASTER_TRIANGLE ? triangle_row(p, y, a.width, di * 2 + pi) : row_setup(s_d, e, p, y, a.width);
					break;
				}
			}
			a.rows[dr.row_base + k] = row;
		}
		__syncthreads(); // the shared records are reused by the CTA's next draw
	}
}

template <class P>
__device__ __forceinline__ void blend_into(typename P::T& dst, typename P::T texel, uint32_t blend)
{
	switch (blend)
	{
	case SW_BLEND_NONE: dst = texel; break;
	case SW_BLEND_AVERAGE: dst = P::average(dst, texel); break;
	case SW_BLEND_ADDITIVE: dst = P::saturated_sum(dst, texel); break;
	case SW_BLEND_ALPHA_TEST:
		if (P::test_alpha(texel)) dst = texel;
		break;
	default: dst = alpha_blend<P>(dst, texel); break;
	}
}

// Texel address of span pixel i (rasterizer.rs:424-445, 558-572, 705-719): u32 arithmetic for the
// perspective modes, i32 for affine, then as usize.
__device__ __forceinline__ uint64_t pixel_address(const RasterRow& r, uint32_t mode, int32_t i, uint32_t tex_w)
{
	const int32_t t0 = wadd(r.a1, wmul(i, r.b1));
	const int32_t t1 = wadd(r.a2, wmul(i, r.b2));
	if (mode == SW_RASTER_FULL_PERSPECTIVE)
	{
		const int32_t inv_z = wadd(r.a0, wmul(i, r.b0));
		const uint32_t zdiv = uint32_t(inv_z) >> INV_Z_PRE_SHIFT;
		const uint32_t z = (1u << Z_CALC_SHIFT) / (zdiv ? zdiv : 1u);
		const uint32_t pu = uint32_t((uint64_t(z) * uint64_t(int64_t(t0))) >> TC_FINAL_SHIFT);
		const uint32_t pv = uint32_t((uint64_t(z) * uint64_t(int64_t(t1))) >> TC_FINAL_SHIFT);
		return uint32_t(pu + pv * tex_w);
	}
	if (mode == SW_RASTER_LINE_Z_CORRECTED) return uint32_t(t0 >> 16) + uint32_t(t1 >> 16) * tex_w;
	return uint64_t(int64_t(wadd(t0 >> 16, wmul(t1 >> 16, int32_t(tex_w)))));
}

constexpr int BATCH = 32; // draws whose tile rows are staged in shared memory at a time

// A thread's strip of one triangle row (fill_triangle_part's pixel loop, rasterizer.rs:1213-1279):
// texture coordinates and light of span pixel i are start + i * step (the reference's per-pixel
// additions), the Color32 texel is lit per lane ((texel * light) >> 16, the alpha lane by 0) and
// written with the draw's blend; alpha test and alpha blend use the unlit texel's alpha.
template <class P, int STRIP>
__device__ __forceinline__ void triangle_strip(const RasterArgs& a, const RasterDraw& d, const RasterRow& row, int xb,
	typename P::T* pix, unsigned int& errors, unsigned int& writes)
{
	const TriSteps ts = a.tri_steps[uint32_t(row.b2)];
	uint32_t tex[STRIP];
	bool ok[STRIP];
#pragma unroll
	for (int k = 0; k < STRIP; ++k)
	{
		const int x = xb + k;
		ok[k] = x >= row.xs && x < row.xe;
		tex[k] = 0;
		if (ok[k])
		{
			const int32_t i = x - row.xs;
			const int32_t u = wadd(row.a0, wmul(i, ts.d_tc_dx[0])) >> 16;
			const int32_t v = wadd(row.b0, wmul(i, ts.d_tc_dx[1])) >> 16;
			uint64_t ua = uint64_t(int64_t(wadd(u, wmul(v, int32_t(d.tex_w)))));
			if (ua >= uint64_t(d.tex_w) * d.tex_h)
			{
				++errors;
				ua = 0;
			}
			tex[k] = __ldg(a.lite + d.tex_offset + ua);
		}
	}
#pragma unroll
	for (int k = 0; k < STRIP; ++k)
		if (ok[k])
		{
			const int32_t i = xb + k - row.xs;
			const CI t = ci_from_c32(tex[k]);
			// line_light lanes [b, g, r, 0] = [light2, light1, light0, 0] (ColorVecI::from_color_i32x3)
			const CI lit{{wmul(t.v[0], wadd(row.a2, wmul(i, ts.d_light_dx[2]))) >> 16,
				wmul(t.v[1], wadd(row.b1, wmul(i, ts.d_light_dx[1]))) >> 16,
				wmul(t.v[2], wadd(row.a1, wmul(i, ts.d_light_dx[0]))) >> 16, 0}};
			typename P::T& dst = pix[k];
			switch (d.blend)
			{
			case SW_BLEND_NONE: dst = P::from_ci(lit); break;
			case SW_BLEND_AVERAGE: dst = P::average(dst, P::from_ci(lit)); break;
			case SW_BLEND_ADDITIVE: dst = P::saturated_sum(dst, P::from_ci(lit)); break;
			case SW_BLEND_ALPHA_TEST:
				if ((tex[k] & 0xFF000000u) > 0x7F000000u) dst = P::from_ci(lit);
				break;
			default:
			{
				const int32_t alpha = int32_t(tex[k] >> 24);
				const CI dv = P::to_ci(dst);
				CI r;
#pragma unroll
				for (int l = 0; l < 4; ++l) r.v[l] = wadd(wmul(dv.v[l], wsub(255, alpha)), wmul(lit.v[l], alpha)) >> 8;
				dst = P::from_ci(r);
			}
			}
			++writes;
		}
}

// The bloom downscale of a tile's final colour64 pixels (downscale_hdr_buffer, postprocessor.rs:792-844):
// the pixels go to shared memory (the row staging area, free once the draws are done), each bloom cell
// whose S x S source pixels lie in the tile gets their box average (i32 lanes, (sum * (256 / S^2)) >> 8),
// and the tile's part of each bloom line's lane sums is added to the line's global sums. The sums are
// wrapping i32 additions, associative and commutative, so the atomics keep them exact in any order.
// Every tile shape is a multiple of 8 pixels on both sides, so no cell straddles two tiles.
template <int TILE_W, int TILE_H, int STRIP>
__device__ __forceinline__ void bloom_epilogue(const RasterArgs& a, const uint64_t* pix, int tx0, int ty0, int tid, void* staging)
{
	constexpr int TPR = TILE_W / STRIP;
	static_assert(TILE_W % 8 == 0 && TILE_H % 8 == 0, "bloom cells must not straddle tiles");
	static_assert(size_t(TILE_W) * TILE_H * 8 <= sizeof(RasterRow) * BATCH * TILE_H, "tile pixels fit the row staging");
	__shared__ int32_t s_ls[TILE_H / 2][4];
	uint64_t* s_pix = static_cast<uint64_t*>(staging);
	__syncthreads(); // the row staging area is free
	{
		const int ly = tid / TPR, lx = (tid % TPR) * STRIP;
#pragma unroll
		for (int k = 0; k < STRIP; ++k) s_pix[ly * TILE_W + lx + k] = pix[k];
	}
	for (int i = tid; i < (TILE_H / 2) * 4; i += 256) (&s_ls[0][0])[i] = 0;
	__syncthreads();
	const int S = int(a.bloom_scale);
	const int cw = TILE_W / S, ch = TILE_H / S;
	const int32_t scaler = 256 / (S * S);
	const uint32_t bx0 = uint32_t(tx0 / S), by0 = uint32_t(ty0 / S);
	for (int i = tid; i < cw * ch; i += 256)
	{
		const int cx = i % cw, cy = i / cw;
		if (bx0 + cx >= a.bloom_w || by0 + cy >= a.bloom_h) continue;
		int32_t sum[4] = {0, 0, 0, 0};
		for (int dy = 0; dy < S; ++dy)
			for (int dx = 0; dx < S; ++dx)
			{
				const CI c = ci_from_c64(s_pix[(cy * S + dy) * TILE_W + cx * S + dx]);
#pragma unroll
				for (int l = 0; l < 4; ++l) sum[l] = wadd(sum[l], c.v[l]);
			}
		CI avg;
#pragma unroll
		for (int l = 0; l < 4; ++l)
		{
			avg.v[l] = wmul(sum[l], scaler) >> 8;
			atomicAdd(&s_ls[cy][l], avg.v[l]);
		}
		a.bloom_out[uint64_t(by0 + cy) * a.bloom_w + bx0 + cx] = ci_to_c64(avg);
	}
	__syncthreads();
	if (tid < ch * 4 && by0 + uint32_t(tid / 4) < a.bloom_h)
		atomicAdd(&a.bloom_line_sums[(by0 + tid / 4) * 4 + tid % 4], s_ls[tid / 4][tid % 4]);
}

// raster_bin_kernel: one CTA per bin. The draws whose box meets the bin, in draw order: chunks of 256
// draws, one box test per thread, an in-order ballot compaction, appended to the bin's list.
__global__ void __launch_bounds__(256) raster_bin_kernel(RasterArgs a)
{
	__shared__ uint32_t s_counts[8];
	const int32_t bx0 = int32_t(blockIdx.x % a.bins_x) * RASTER_BIN_W, by0 = int32_t(blockIdx.x / a.bins_x) * RASTER_BIN_H;
	const int32_t bx1 = min(bx0 + RASTER_BIN_W, a.width), by1 = min(by0 + RASTER_BIN_H, a.height);
	pdl_wait(); // the raster setup wrote the boxes
	const uint32_t num_draws = a.counts ? a.counts->num_draws : a.num_draws;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t* list = a.bin_lists + uint64_t(blockIdx.x) * a.bin_cap;
	uint32_t total = 0;
	for (uint32_t chunk = 0; chunk < num_draws; chunk += 256)
	{
		const uint32_t di = chunk + threadIdx.x;
		bool hit = false;
		if (di < num_draws)
		{
			const RasterBox b = a.boxes[di];
			hit = b.x0 < bx1 && b.x1 > bx0 && b.y0 < by1 && b.y1 > by0 && b.x0 < b.x1 && b.y0 < b.y1;
		}
		const unsigned mask = __ballot_sync(0xFFFFFFFFu, hit);
		if (lane == 0) s_counts[warp] = __popc(mask);
		__syncthreads();
		uint32_t base = total, sum = 0;
#pragma unroll
		for (int w = 0; w < 8; ++w)
		{
			if (w < warp) base += s_counts[w];
			sum += s_counts[w];
		}
		if (hit) list[base + __popc(mask & ((1u << lane) - 1u))] = di;
		total += sum;
		__syncthreads(); // s_counts is rewritten by the next chunk
	}
	if (threadIdx.x == 0) a.bin_counts[blockIdx.x] = total;
	pdl_trigger();
}

// The scale-2 bloom downscale without shared memory, when a tile row's threads share a warp with the
// next row's (TILE_W / STRIP <= 16): the thread of an even row takes the odd row's STRIP pixels from
// its partner by a shuffle, box-averages its STRIP / 2 cells and stores them; the line's lane sums of
// the row pair are reduced over its threads by shuffles and added to the global sums, one atomic per
// lane. Same integer arithmetic as bloom_epilogue, so the same values.
template <int TILE_W, int STRIP>
__device__ __forceinline__ void bloom_epilogue_s2(const RasterArgs& a, const uint64_t* pix, int tx0, int ty0, int tid)
{
	constexpr int TPR = TILE_W / STRIP;
	static_assert(TPR <= 16 && (TPR & (TPR - 1)) == 0 && STRIP % 2 == 0, "row pairs within a warp");
	const int ly = tid / TPR, lx = (tid % TPR) * STRIP;
	uint64_t other[STRIP];
#pragma unroll
	for (int k = 0; k < STRIP; ++k) other[k] = __shfl_xor_sync(0xFFFFFFFFu, pix[k], TPR);
	int32_t line[4] = {0, 0, 0, 0};
	const bool even = (ly & 1) == 0;
	const uint32_t by = uint32_t((ty0 + ly) / 2);
	if (even && by < a.bloom_h)
	{
#pragma unroll
		for (int c = 0; c < STRIP / 2; ++c)
		{
			const uint32_t bx = uint32_t((tx0 + lx) / 2 + c);
			if (bx >= a.bloom_w) continue;
			int32_t sum[4] = {0, 0, 0, 0};
			const uint64_t q[4] = {pix[2 * c], pix[2 * c + 1], other[2 * c], other[2 * c + 1]};
#pragma unroll
			for (int j = 0; j < 4; ++j)
			{
				const CI v = ci_from_c64(q[j]);
#pragma unroll
				for (int l = 0; l < 4; ++l) sum[l] = wadd(sum[l], v.v[l]);
			}
			CI avg;
#pragma unroll
			for (int l = 0; l < 4; ++l)
			{
				avg.v[l] = wmul(sum[l], 64) >> 8; // scaler 256 / (2 * 2)
				line[l] = wadd(line[l], avg.v[l]);
			}
			a.bloom_out[uint64_t(by) * a.bloom_w + bx] = ci_to_c64(avg);
		}
	}
	// the row pair's threads are TPR consecutive lanes (the odd row's add zeros)
#pragma unroll
	for (int l = 0; l < 4; ++l)
		for (int o = TPR / 2; o > 0; o >>= 1) line[l] = wadd(line[l], __shfl_xor_sync(0xFFFFFFFFu, line[l], o));
	if (even && (tid % TPR) == 0 && by < a.bloom_h)
	{
#pragma unroll
		for (int l = 0; l < 4; ++l) atomicAdd(&a.bloom_line_sums[by * 4 + l], line[l]);
	}
}

// Tile shapes of the tile pass (the autotuner's choice, SwTuning.raster_tile): TILE_W x TILE_H pixels,
// 256 threads, each thread a 1 x STRIP strip of one row. Every shape gives the same frame.
struct TileShape
{
	int w, h, strip;
};
constexpr TileShape TILE_SHAPES[SW_RASTER_TILE_VARIANTS] = {{64, 16, 4}, {32, 32, 4}, {128, 8, 4}, {64, 32, 8}, {32, 16, 2}};

template <class P, int TILE_W, int TILE_H, int STRIP>
__global__ void __launch_bounds__(256) raster_tiles_kernel(RasterArgs a)
{
	static_assert((TILE_W / STRIP) * TILE_H == 256, "256 threads per tile");
	constexpr int TPR = TILE_W / STRIP; // threads per tile row
	typedef typename P::T T;
	__shared__ uint32_t s_warp_counts[8];
	__shared__ RasterDraw s_rd[256];
	__shared__ RasterBox s_box[256];
	__shared__ __align__(16) RasterRow s_row[BATCH][TILE_H]; // also the bloom epilogue's pixel staging (8-byte lanes)

	const int tiles_x = (a.width + TILE_W - 1) / TILE_W;
	const int tx0 = int(blockIdx.x % tiles_x) * TILE_W;
	const int ty0 = int(blockIdx.x / tiles_x) * TILE_H;
	const int tid = threadIdx.x;
	const int ly = tid / TPR;
	pdl_wait(); // the surface build (launched before this kernel) has completed
	const uint32_t num_draws = a.counts ? a.counts->num_draws : a.num_draws;
	const int xb = tx0 + (tid % TPR) * STRIP; // first pixel of this thread's strip
	const int y = ty0 + ly;
	const bool row_valid = y < a.height;
	const int tx1 = min(tx0 + TILE_W, a.width), ty1 = min(ty0 + TILE_H, a.height);

	T* fb = static_cast<T*>(a.framebuffer);
	const T* arena = static_cast<const T*>(a.arena);
	const T* skybox = static_cast<const T*>(a.skybox);
	T pix[STRIP];
#pragma unroll
	for (int k = 0; k < STRIP; ++k)
	{
		pix[k] = T(0);
		const int x = xb + k;
		if (row_valid && x < a.width)
		{
			if (a.clear_background) // ColorVec::from_color_f32x3(&[32.0, 16.0, 8.0]).into(), partial_renderer.rs:255
				pix[k] = P::FORMAT == SW_PIXEL_C64 ? T(8ull | (16ull << 16) | (32ull << 32)) : T(0x00201008u);
			else
				pix[k] = fb[uint64_t(y) * a.width + x];
		}
	}
	unsigned int local_errors = 0, local_writes = 0;

	const int lane = tid & 31, warp = tid >> 5;
	// the draws to scan: the tile's bin's list (draw order), or every draw
	const uint32_t* list = nullptr;
	uint32_t list_len = num_draws;
	if (a.bin_lists)
	{
		const uint32_t bin = uint32_t(tx0 / RASTER_BIN_W) + uint32_t(ty0 / RASTER_BIN_H) * a.bins_x;
		list = a.bin_lists + uint64_t(bin) * a.bin_cap;
		list_len = a.bin_counts[bin];
	}
	for (uint32_t chunk = 0; chunk < list_len; chunk += 256)
	{
		// Ordered compaction of the chunk's draws whose box meets the tile; the hitting thread stages
		// the draw's record and box.
		const uint32_t k = chunk + tid;
		bool hit = false;
		RasterBox b{0, 0, 0, 0};
		RasterDraw rd{};
		if (k < list_len)
		{
			const uint32_t di = list ? list[k] : k;
			b = a.boxes[di];
			hit = b.x0 < tx1 && b.x1 > tx0 && b.y0 < ty1 && b.y1 > ty0 && b.x0 < b.x1 && b.y0 < b.y1;
			if (hit) rd = a.rdraws[di];
		}
		const unsigned mask = __ballot_sync(0xFFFFFFFFu, hit);
		if (lane == 0) s_warp_counts[warp] = __popc(mask);
		__syncthreads();
		uint32_t base = 0, total = 0;
#pragma unroll
		for (int w = 0; w < 8; ++w)
		{
			const uint32_t c = s_warp_counts[w];
			if (w < warp) base += c;
			total += c;
		}
		if (hit)
		{
			const uint32_t pos = base + __popc(mask & ((1u << lane) - 1u));
			s_rd[pos] = rd;
			s_box[pos] = b;
		}
		__syncthreads();

		for (uint32_t b0 = 0; b0 < total; b0 += BATCH)
		{
			const uint32_t n = min(uint32_t(BATCH), total - b0);
			// Stage the batch's rows of this tile (independent loads, one per thread).
			for (uint32_t k = tid; k < n * TILE_H; k += 256)
			{
				const uint32_t h = k / TILE_H, r = k % TILE_H;
				const RasterBox bx = s_box[b0 + h];
				const int32_t ry = ty0 + int32_t(r);
				RasterRow row;
				if (ry >= bx.y0 && ry < bx.y1)
				{
					const RasterDraw& d = s_rd[b0 + h];
					row = a.rows[d.row_base + uint32_t(ry - d.y0)];
				}
				else
					row.xs = row.xe = 0;
				s_row[h][r] = row;
			}
			__syncthreads();
			if (row_valid)
				for (uint32_t h = 0; h < n; ++h)
				{
					const RasterRow row = s_row[h][ly];
					if (xb + STRIP <= row.xs || xb >= row.xe) continue;
					const RasterDraw& d = s_rd[b0 + h];
					if (d.mode == SW_RASTER_TRIANGLE)
					{
						triangle_strip<P, STRIP>(a, d, row, xb, pix, local_errors, local_writes);
						continue;
					}
					// Up to four independent texel loads, then the blends in pixel order.
					T tex[STRIP];
					bool ok[STRIP];
#pragma unroll
					for (int k = 0; k < STRIP; ++k)
					{
						const int x = xb + k;
						ok[k] = x >= row.xs && x < row.xe;
						tex[k] = T(0);
						if (ok[k])
						{
							uint64_t ua = pixel_address(row, d.mode, x - row.xs, d.tex_w);
							if (ua >= uint64_t(d.tex_w) * d.tex_h)
							{
								++local_errors;
								ua = 0;
							}
							tex[k] = (d.tex_source == SW_TEXSRC_SKYBOX ? skybox : arena)[d.tex_offset + ua];
						}
					}
#pragma unroll
					for (int k = 0; k < STRIP; ++k)
						if (ok[k])
						{
							blend_into<P>(pix[k], tex[k], d.blend);
							++local_writes;
						}
				}
			__syncthreads();
		}
	}
	if (row_valid)
	{
#pragma unroll
		for (int k = 0; k < STRIP; ++k)
			if (xb + k < a.width) fb[uint64_t(y) * a.width + xb + k] = pix[k];
	}
	if constexpr (P::FORMAT == SW_PIXEL_C64)
	{
		if constexpr (TILE_W / STRIP <= 16)
		{
			if (a.bloom_scale == 2)
				bloom_epilogue_s2<TILE_W, STRIP>(a, reinterpret_cast<const uint64_t*>(pix), tx0, ty0, tid);
			else if (a.bloom_scale)
				bloom_epilogue<TILE_W, TILE_H, STRIP>(a, pix, tx0, ty0, tid, &s_row[0][0]);
		}
		else if (a.bloom_scale)
			bloom_epilogue<TILE_W, TILE_H, STRIP>(a, pix, tx0, ty0, tid, &s_row[0][0]);
	}
	if (local_errors) atomicAdd(a.error_counter, local_errors);
	// Pixel writes (span pixels processed) for the traffic accounting, one atomic per warp.
	for (int o = 16; o > 0; o >>= 1) local_writes += __shfl_xor_sync(0xFFFFFFFFu, local_writes, o);
	if (lane == 0 && local_writes)
		atomicAdd(reinterpret_cast<unsigned long long*>(a.error_counter + 2), (unsigned long long)local_writes);
	pdl_trigger();
}

} // namespace

// ---- shadow maps: DepthRasterizer (rasterizer.rs:1295-1474) over DepthRenderer's draws ----
//
// Painter's order with every draw in flight at once: the storage holds (sequence << 32 | f32 bits) per
// texel and every draw writes with atomicMax, so the last draw covering a texel wins, as the sequential
// overwrite does. Sequences keep growing from call to call (the caller passes each call's base), so a
// texel no draw of the current call covers keeps its value: the reference never clears its storage.

namespace
{

// One row of a part (fill_polygon_part's row loop, rasterizer.rs:1448-1470): `line` is the row's
// line_inv_z; inv_z is accumulated pixel by pixel as the reference does.
__device__ __forceinline__ void draw_depth_row(unsigned long long* map, int32_t size, const RasterPart& p, uint32_t r, float line,
	float dx, unsigned long long seq)
{
	const int32_t y = p.y_start_int + int32_t(r);
	const int32_t xs = max(wadd(p.x_left0, wmul(int32_t(r), p.dx_dy_left)) >> 16, 0);
	const int32_t xe = min(wadd(p.x_right0, wmul(int32_t(r), p.dx_dy_right)) >> 16, size);
	if (xs >= xe) return;
	float inv_z = fadd(line, fmul(float(xs), dx));
	unsigned long long* row = map + uint64_t(y) * uint32_t(size);
	for (int32_t x = xs; x < xe; ++x)
	{
		atomicMax(row + x, seq | __float_as_uint(inv_z));
		inv_z = fadd(inv_z, dx);
	}
}

// line_inv_z of the part's first row (rasterizer.rs:1442-1447); the next rows add dy one at a time.
__device__ __forceinline__ float depth_first_line(const RasterPart& p, float dx, float dy, float k)
{
	return fadd(fadd(fmul(float(p.y_start_int), dy), fmul(0.5f, fadd(dx, dy))), k);
}

} // namespace

__global__ void shadow_rebase_kernel(unsigned long long* storage, uint64_t n)
{
	for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
		storage[i] &= 0xFFFFFFFFull;
}

// Host-prepared depth draws (sw_build_shadow_maps), one per CTA: thread 0 walks the edges (the colour
// rasteriser's walk: the same parts and first-row edge positions) and accumulates each part's per-row
// inverse depth in the reference's sequential order; then one thread per row accumulates along its span.
__global__ void __launch_bounds__(256) shadow_draw_kernel(ShadowArgs a)
{
	__shared__ __align__(8) SwDrawCmd s_d;
	__shared__ SwVertex16 s_v[SW_MAX_POLYGON_VERTICES];
	__shared__ RasterPart s_parts[SW_RASTER_MAX_PARTS];
	__shared__ float s_line[SW_SHADOW_MAX_SIZE];
	__shared__ uint32_t s_np;
	for (uint32_t di = blockIdx.x; di < a.num_draws; di += gridDim.x)
	{
		const SwDepthDraw dd = a.draws[di];
		const int32_t size = int32_t(dd.map_size);
		if (threadIdx.x == 0)
		{
			s_d = SwDrawCmd{};
			s_d.vertex_count = dd.vertex_count;
			s_d.mode = SW_RASTER_FULL_PERSPECTIVE; // no texture-coordinate edges
		}
		if (threadIdx.x < dd.vertex_count) s_v[threadIdx.x] = a.vertices[dd.first_vertex + threadIdx.x];
		__syncthreads();
		if (threadIdx.x == 0) s_np = edge_walk(s_d, s_v, size, s_parts);
		__syncthreads();
		const float dx = dd.depth_eq[0], dy = dd.depth_eq[1], k = dd.depth_eq[2];
		const unsigned long long seq = (unsigned long long)(a.seq_base + di + 1u) << 32;
		unsigned long long* map = a.storage + dd.map_offset;
		for (uint32_t pi = 0; pi < s_np; ++pi)
		{
			const RasterPart p = s_parts[pi];
			const uint32_t rows = uint32_t(p.y_end_int - p.y_start_int); // <= size <= SW_SHADOW_MAX_SIZE
			if (threadIdx.x == 0)
			{
				float line = depth_first_line(p, dx, dy, k);
				for (uint32_t r = 0; r < rows; ++r)
				{
					s_line[r] = line;
					line = fadd(line, dy);
				}
			}
			__syncthreads();
			for (uint32_t r = threadIdx.x; r < rows; r += blockDim.x) draw_depth_row(map, size, p, r, s_line[r], dx, seq);
			__syncthreads(); // s_line is reused by the next part
		}
	}
}

// GPU-prepared depth draws (sw_build_shadow_maps_view): every polygon of every listed leaf is one warp,
// which prepares it (DepthRenderer::draw_polygon::<false> + draw_depth_polygon, depth_renderer.rs:
// 199-287: the shared depth_map_equation, the view transform, the warp-cooperative
// project_and_clip_polygon, f32_to_fixed16) and draws it at once. The candidate's index in the leaf
// list's polygon order is its painter's-order sequence, so nothing is compacted. Rows go to lanes 32 at
// a time: lane i takes the 32-row chunk's first line_inv_z and adds dy i times, which is the
// reference's sequential row accumulation; the next chunk starts from lane 31's value plus dy.
constexpr int SHADOW_VIEW_WARPS = 8;
constexpr uint32_t SHADOW_VIEW_SMEM_LEAFS = 8192; // leaf starts staged in shared memory up to this many

struct ShadowWarpShared
{
	WarpClipBuf clip;
	SwVertex16 v[SW_MAX_POLYGON_VERTICES];
	RasterPart parts[SW_RASTER_MAX_PARTS];
};

__global__ void __launch_bounds__(SHADOW_VIEW_WARPS * 32) shadow_view_kernel(ShadowViewArgs a)
{
	__shared__ ShadowWarpShared s_w[SHADOW_VIEW_WARPS];
	extern __shared__ uint32_t s_leaf_base[]; // the leafs' first candidates (dynamic: num_leafs when staged)
	// stage the leaf starts (one round of independent loads) so the search runs in shared memory
	const bool staged = a.num_leafs <= SHADOW_VIEW_SMEM_LEAFS;
	if (staged)
	{
		for (uint32_t i = threadIdx.x; i < a.num_leafs; i += blockDim.x) s_leaf_base[i] = a.leaf_base[i];
		__syncthreads();
	}
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	ShadowWarpShared& sw = s_w[warp];
	const uint32_t* leaf_base = staged ? s_leaf_base : a.leaf_base;
	// persistent: the grid is what fits on the GPU at once and each warp takes candidates in turn, so a
	// rejected candidate (facing away, clipped away: most of them) frees its warp at once
	for (uint32_t c = blockIdx.x * SHADOW_VIEW_WARPS + warp; c < a.num_candidates; c += gridDim.x * SHADOW_VIEW_WARPS)
	{
		__syncwarp(); // the previous candidate's reads of sw are done
		// every condition below is the warp's polygon's: the lanes stay together
		const uint32_t li = find_segment(leaf_base, a.num_leafs, c);
		const SwShadowLeaf& leaf = a.leafs[li];
		const SwShadowSide& side = a.sides[leaf.side];
		const SwMapPolygon& p = a.polygons[leaf.first_polygon + (c - leaf_base[li])];
		float eq[3];
		if (!swhost::depth_map_equation(p, load_mat4(side.planes_matrix), eq)) continue;
		const uint32_t nv = p.num_vertices < MAXV ? p.num_vertices : MAXV;
		if (nv < 3) continue;
		const Mat4 view = load_mat4(side.view_matrix);
		const Vec3* mv = reinterpret_cast<const Vec3*>(a.map_vertices);
		const Vec3 vt = lane < nv ? swhost::view_transform(view, mv[p.first_vertex + lane]) : swhost::v3(0.0f, 0.0f, 1.0f);
		Vec3 planes[8];
		load_planes(leaf.clip_planes, planes);
		Vec2 v2d = swhost::v2(0.0f, 0.0f);
		const uint32_t count = warp_project_and_clip(planes, vt, nv, v2d, sw.clip);
		if (count < 3) continue;
		if (lane < count) // f32_to_fixed16 (fixed_math.rs:31-34)
			sw.v[lane] = SwVertex16{swhost::as_i32(v2d.x * 65536.0f), swhost::as_i32(v2d.y * 65536.0f)};
		__syncwarp();
		const int32_t size = int32_t(side.map_size);
		uint32_t np = 0;
		if (lane == 0)
		{
			SwDrawCmd d{};
			d.vertex_count = count;
			d.mode = SW_RASTER_FULL_PERSPECTIVE; // no texture-coordinate edges
			np = edge_walk(d, sw.v, size, sw.parts);
		}
		np = __shfl_sync(FULL_MASK, np, 0);
		__syncwarp();
		const float dx = eq[0], dy = eq[1], k = eq[2];
		const unsigned long long seq = (unsigned long long)(a.seq_base + c + 1u) << 32;
		unsigned long long* map = a.storage + side.map_offset;
		for (uint32_t pi = 0; pi < np; ++pi)
		{
			const RasterPart pt = sw.parts[pi];
			const uint32_t rows = uint32_t(pt.y_end_int - pt.y_start_int);
			float chunk = depth_first_line(pt, dx, dy, k);
			for (uint32_t r0 = 0; r0 < rows; r0 += 32)
			{
				float line = chunk;
				for (uint32_t i = 0; i < lane; ++i) line = fadd(line, dy);
				if (r0 + lane < rows) draw_depth_row(map, size, pt, r0 + lane, line, dx, seq);
				chunk = fadd(__shfl_sync(FULL_MASK, line, 31), dy);
			}
		}
	}
}

int launch_shadow_maps(const ShadowArgs& args, cudaStream_t stream)
{
	if (args.num_draws > 0) shadow_draw_kernel<<<std::min(args.num_draws, 65535u), 256, 0, stream>>>(args);
	return int(cudaGetLastError());
}

int launch_shadow_view(const ShadowViewArgs& args, cudaStream_t stream)
{
	if (args.num_candidates == 0) return 0;
	const size_t smem = args.num_leafs <= SHADOW_VIEW_SMEM_LEAFS ? size_t(args.num_leafs) * 4 : 0; // + 16 KB static < 48 KB
	// resident CTAs of the largest staging (registers bound it first), once per device; concurrent first
	// calls compute the same value, so a relaxed atomic store is enough
	constexpr int MAX_DEVICES = 64;
	static std::atomic<int> resident_per_device[MAX_DEVICES];
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return int(e);
	int resident = dev >= 0 && dev < MAX_DEVICES ? resident_per_device[dev].load(std::memory_order_relaxed) : 0;
	if (resident == 0)
	{
		int sms = 0, per_sm = 0;
		e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (e == cudaSuccess)
			e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, shadow_view_kernel, SHADOW_VIEW_WARPS * 32,
				size_t(SHADOW_VIEW_SMEM_LEAFS) * 4);
		if (e != cudaSuccess) return int(e);
		resident = std::max(sms * per_sm, 1);
		if (dev >= 0 && dev < MAX_DEVICES) resident_per_device[dev].store(resident, std::memory_order_relaxed);
	}
	const uint32_t blocks = std::min<uint32_t>((args.num_candidates + SHADOW_VIEW_WARPS - 1) / SHADOW_VIEW_WARPS, uint32_t(resident));
	shadow_view_kernel<<<blocks, SHADOW_VIEW_WARPS * 32, smem, stream>>>(args);
	return int(cudaGetLastError());
}

namespace
{
// make_shadow_map_circle (light.rs:135-156) on one projector map: row y's first and last dx texels
// (outside the inscribed circle) become 1e24, written with sequence `seq` so that they replace every
// depth draw before them and give way to every later one.
__global__ void __launch_bounds__(256) shadow_circle_kernel(unsigned long long* map, uint32_t size, uint32_t seq)
{
	const int32_t s = int32_t(size), radius = s / 2, y = int32_t(blockIdx.x);
	const int32_t dy = y - radius;
	const int32_t rr = max(radius * radius - dy * dy, 0);
	const int32_t dx = radius - min(int32_t(ceilf(sqrtf(float(rr)))), radius);
	const unsigned long long v = (static_cast<unsigned long long>(seq) << 32) | __float_as_uint(1.0e24f);
	unsigned long long* line = map + uint64_t(y) * size;
	for (int32_t x = int32_t(threadIdx.x); x < dx; x += int32_t(blockDim.x))
	{
		line[x] = v;
		line[s - 1 - x] = v;
	}
}
} // namespace

int launch_shadow_circle(unsigned long long* map, uint32_t size, uint32_t seq, cudaStream_t stream)
{
	if (size == 0) return 0;
	shadow_circle_kernel<<<size, 256, 0, stream>>>(map, size, seq);
	return int(cudaGetLastError());
}

int launch_shadow_rebase(unsigned long long* storage, uint64_t num_texels, cudaStream_t stream)
{
	if (num_texels == 0) return 0;
	shadow_rebase_kernel<<<unsigned(std::min<uint64_t>((num_texels + 255) / 256, 4096)), 256, 0, stream>>>(storage, num_texels);
	return int(cudaGetLastError());
}

int launch_raster_setup(const RasterArgs& args, cudaStream_t stream)
{
	if (args.counts)
	{
		if (args.setup_blocks > 0) raster_setup_kernel<<<args.setup_blocks, 256, 0, stream>>>(args);
	}
	else if (args.num_draws > 0)
		raster_setup_kernel<<<args.num_draws, 256, 0, stream>>>(args);
	return int(cudaGetLastError());
}

namespace
{
template <int V>
void launch_tiles_variant(const RasterArgs& args, uint32_t pixel_format, cudaStream_t stream)
{
	constexpr TileShape t = TILE_SHAPES[V];
	const unsigned tiles = unsigned(((args.width + t.w - 1) / t.w) * ((args.height + t.h - 1) / t.h));
	if (tiles == 0) return;
	if (pixel_format == SW_PIXEL_C64)
		launch_dependent(raster_tiles_kernel<PixC64, t.w, t.h, t.strip>, dim3(tiles), dim3(256), 0, stream, args);
	else
		launch_dependent(raster_tiles_kernel<PixC32, t.w, t.h, t.strip>, dim3(tiles), dim3(256), 0, stream, args);
}
} // namespace

namespace
{
// mix_surface_with_texture_impl (surfaces.rs:903-971) on one pixel of a view's region: the texture texel
// at (tc_min + (x, y)) rem_euclid its size, modulated by the light (ColorVecI lanes * light * 256 >> 8),
// blended into the pixel with the view's blending mode.
template <class P>
__global__ void __launch_bounds__(256) view_mix_kernel(SwView v, typename P::T* target, const uint32_t* lite, CI light)
{
	const uint64_t total = uint64_t(v.width) * v.height;
	for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += uint64_t(gridDim.x) * blockDim.x)
	{
		const uint32_t x = uint32_t(i % v.width), y = uint32_t(i / v.width);
		int32_t su = (v.mix_tc_min[0] + int32_t(x)) % int32_t(v.mix_size[0]);
		int32_t sv = (v.mix_tc_min[1] + int32_t(y)) % int32_t(v.mix_size[1]);
		if (su < 0) su += int32_t(v.mix_size[0]);
		if (sv < 0) sv += int32_t(v.mix_size[1]);
		const uint32_t texel = lite[v.mix_offset + uint64_t(sv) * v.mix_size[0] + uint32_t(su)];
		const CI t = ci_from_c32(texel);
		CI m;
#pragma unroll
		for (int k = 0; k < 4; ++k) m.v[k] = wmul(t.v[k], light.v[k]) >> 8;
		typename P::T& dst = target[i];
		switch (v.mix_blend)
		{
		case SW_BLEND_NONE: dst = P::from_ci(m); break;
		case SW_BLEND_AVERAGE:
		{
			const CI d = P::to_ci(dst);
#pragma unroll
			for (int k = 0; k < 4; ++k) m.v[k] = wadd(m.v[k], d.v[k]) >> 1;
			dst = P::from_ci(m);
			break;
		}
		case SW_BLEND_ADDITIVE:
		{
			const CI d = P::to_ci(dst);
#pragma unroll
			for (int k = 0; k < 4; ++k) m.v[k] = wadd(m.v[k], d.v[k]);
			dst = P::from_ci(m);
			break;
		}
		case SW_BLEND_ALPHA_TEST:
			if ((texel & 0xFF000000u) > 0x7F000000u) dst = P::from_ci(m); // Color32::test_alpha
			break;
		default: // SW_BLEND_ALPHA_BLEND
		{
			const int32_t alpha = int32_t(texel >> 24);
			const CI d = P::to_ci(dst);
#pragma unroll
			for (int k = 0; k < 4; ++k) m.v[k] = wadd(wmul(m.v[k], alpha), wmul(d.v[k], 255 - alpha)) >> 8;
			dst = P::from_ci(m);
			break;
		}
		}
	}
}
} // namespace

int launch_view_mix(const SwView& view, void* target, const uint32_t* lite, uint32_t pixel_format, cudaStream_t stream)
{
	// ColorVecI::from_color_f32x3 of light * 256: lanes b, g, r (f32 -> i32 truncation), alpha 0
	const CI light{{int32_t(view.mix_light[2] * 256.0f), int32_t(view.mix_light[1] * 256.0f), int32_t(view.mix_light[0] * 256.0f), 0}};
	const uint64_t total = uint64_t(view.width) * view.height;
	const unsigned blocks = unsigned(std::min<uint64_t>((total + 255) / 256, 152 * 8));
	if (pixel_format == SW_PIXEL_C64)
		view_mix_kernel<PixC64><<<blocks, 256, 0, stream>>>(view, static_cast<uint64_t*>(target), lite, light);
	else
		view_mix_kernel<PixC32><<<blocks, 256, 0, stream>>>(view, static_cast<uint32_t*>(target), lite, light);
	return int(cudaGetLastError());
}

int launch_raster_bins(const RasterArgs& args, cudaStream_t stream)
{
	if (!args.bin_lists) return 0;
	return int(launch_dependent(raster_bin_kernel, dim3(args.bins_x * args.bins_y), dim3(256), 0, stream, args));
}

int launch_raster_tiles(const RasterArgs& args, uint32_t pixel_format, uint32_t variant, cudaStream_t stream)
{
	switch (variant)
	{
	case 0: launch_tiles_variant<0>(args, pixel_format, stream); break;
	case 1: launch_tiles_variant<1>(args, pixel_format, stream); break;
	case 2: launch_tiles_variant<2>(args, pixel_format, stream); break;
	case 3: launch_tiles_variant<3>(args, pixel_format, stream); break;
	case 4: launch_tiles_variant<4>(args, pixel_format, stream); break;
	default: return int(cudaErrorInvalidValue);
	}
	return int(cudaGetLastError());
}

} // namespace swgpu
