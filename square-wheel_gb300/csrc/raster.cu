// Tile-binned polygon rasteriser for the GB300 path.
//
// Replaces perform_rasterization's single-thread path (src/square_wheel/partial_renderer.rs:1207-1234)
// running Rasterizer::fill_polygon for each draw in submission order (src/square_wheel/rasterizer.rs:
// 137-729, write_into_framebuffer :1511-1536).
//
// Two launches:
//   raster_setup: one thread per draw runs the reference's edge walk (rasterizer.rs:160-270) and stores
//     each polygon part's first-row edge positions, the draw's integer plane equations
//     (rasterizer.rs:287-310) and a conservative pixel box.
//   raster_tiles: one 256-thread CTA per 16x16 tile, one thread per pixel. The CTA streams over the
//     draws in submission order, 256 at a time; each thread tests one draw's box against the tile and
//     a ballot + prefix sum compacts the hits into shared memory in order. Every thread then walks the
//     hits in order for its own pixel and keeps the pixel in a register, so blending order is the
//     reference's and the framebuffer is read and written once per frame.
// Span setup is evaluated over the whole span with the frame as clip rectangle (the reference's
// num_threads == 1 ClipRect); a pixel at span index i takes start + i*step, which is the reference's
// repeated wrapping addition. Coverage and texel addresses are therefore bit-exact.
#include "sw_kernels.cuh"

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
constexpr int TILE = 16;

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

struct SetupState
{
	const SwDrawCmd* d;
	int32_t width, height;
	RasterPart* parts;
	uint32_t num_parts;
	int32_t bx0, by0, bx1, by1;
};

// The draw_func body up to the row loop: first-row edge positions (rasterizer.rs:316-320) and, for
// the affine mode, the per-part texture coordinate edges (rasterizer.rs:597-682).
__device__ void emit_part(SetupState& st, Fixed16 y_start, Fixed16 y_end, Fixed16 xl_start, Fixed16 dxl,
	Fixed16 xr_start, Fixed16 dxr)
{
	const int32_t y_start_int = max(round_to_int(y_start), 0);
	const int32_t y_end_int = min(round_to_int(y_end), st.height);
	if (y_start_int >= y_end_int || st.num_parts >= SW_RASTER_MAX_PARTS) return;
	const Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
	RasterPart p;
	p.y_start_int = y_start_int;
	p.y_end_int = y_end_int;
	p.x_left0 = wadd(wadd(xl_start, fx_mul(y_start_delta, dxl)), FIXED16_HALF);
	p.x_right0 = wadd(wadd(xr_start, fx_mul(y_start_delta, dxr)), FIXED16_HALF);
	p.dx_dy_left = dxl;
	p.dx_dy_right = dxr;
	p.tc_left0[0] = p.tc_left0[1] = p.tc_right0[0] = p.tc_right0[1] = 0;
	p.d_tc_left[0] = p.d_tc_left[1] = p.d_tc_right[0] = p.d_tc_right[1] = 0;
	const SwDrawCmd& d = *st.d;
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
	st.parts[st.num_parts++] = p;
	// Box: x is linear in the row, so the extremes over the part are at its first and last rows.
	const int32_t last = y_end_int - 1 - y_start_int;
	const int32_t xl0 = p.x_left0 >> 16, xl1 = wadd(p.x_left0, wmul(last, dxl)) >> 16;
	const int32_t xr0 = p.x_right0 >> 16, xr1 = wadd(p.x_right0, wmul(last, dxr)) >> 16;
	st.bx0 = min(st.bx0, min(xl0, xl1));
	st.bx1 = max(st.bx1, max(xr0, xr1));
	st.by0 = min(st.by0, y_start_int);
	st.by1 = max(st.by1, y_end_int);
}

__global__ void __launch_bounds__(128) raster_setup_kernel(RasterArgs a)
{
	const uint32_t di = blockIdx.x * blockDim.x + threadIdx.x;
	if (di >= a.num_draws) return;
	const SwDrawCmd& d = a.draws[di];
	SetupState st;
	st.d = &d;
	st.width = a.width;
	st.height = a.height;
	st.parts = a.parts + uint64_t(di) * SW_RASTER_MAX_PARTS;
	st.num_parts = 0;
	st.bx0 = INT32_MAX;
	st.by0 = INT32_MAX;
	st.bx1 = INT32_MIN;
	st.by1 = INT32_MIN;

	const SwVertex16* vtx = a.vertices + d.first_vertex;
	const uint32_t n = d.vertex_count;
	// Edge walk, rasterizer.rs:160-270.
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
	for (uint32_t guard = 0; guard < 2 * SW_MAX_POLYGON_VERTICES + 2; ++guard)
	{
		uint32_t nli = li + n - 1;
		if (nli >= n) nli -= n;
		uint32_t nri = ri + 1;
		if (nri >= n) nri -= n;
		const SwVertex16 lv = vtx[li], nlv = vtx[nli], rv = vtx[ri], nrv = vtx[nri];
		const Fixed16 dy_left = wsub(nlv.y, lv.y);
		const Fixed16 dy_right = wsub(nrv.y, rv.y);
		const Fixed16 next_y = min(nlv.y, nrv.y);
		if (dy_left > FIXED16_HALF && dy_right > FIXED16_HALF)
		{
			const Fixed16 dxl = fx_div(wsub(nlv.x, lv.x), dy_left);
			const Fixed16 dxr = fx_div(wsub(nrv.x, rv.x), dy_right);
			emit_part(st, cur_y, next_y, wadd(lv.x, fx_mul(dxl, wsub(cur_y, lv.y))), dxl,
				wadd(rv.x, fx_mul(dxr, wsub(cur_y, rv.y))), dxr);
		}
		else if (dy_left > 0 && dy_right > 0)
		{
			const int32_t cur_y_int = round_to_int(cur_y);
			const int32_t next_y_int = round_to_int(next_y);
			if (cur_y_int < next_y_int)
			{
				const Fixed16 thin_y = wadd(int_to_fixed16(cur_y_int), FIXED16_HALF);
				const Fixed16 xsl = wadd(lv.x, fx_mul_div(wsub(thin_y, lv.y), wsub(nlv.x, lv.x), dy_left));
				const Fixed16 xsr = wadd(rv.x, fx_mul_div(wsub(thin_y, rv.y), wsub(nrv.x, rv.x), dy_right));
				emit_part(st, cur_y, next_y, xsl, 0, xsr, 0);
			}
		}
		if (nli == nri) break;
		if (nrv.y < nlv.y)
			ri = nri;
		else
			li = nli;
		cur_y = next_y;
	}

	RasterDraw rd;
	const float* de = d.depth_eq;
	const float* te = d.tc_eq;
	rd.d_inv_z_dx = f2i64(fmul(INV_Z_SCALE, de[0]));
	rd.d_inv_z_dy = f2i64(fmul(INV_Z_SCALE, de[1]));
	rd.inv_z_k = f2i64(fmul(INV_Z_SCALE, fadd(de[2], fmul(fadd(de[0], de[1]), 0.5f))));
#pragma unroll
	for (int i = 0; i < 2; ++i)
	{
		rd.d_tc_dx[i] = f2i64(fmul(TC_SCALE, te[i]));
		rd.d_tc_dy[i] = f2i64(fmul(TC_SCALE, te[2 + i]));
		rd.tc_k[i] = f2i64(fmul(TC_SCALE, fadd(te[4 + i], fmul(fadd(te[i], te[2 + i]), 0.5f))));
	}
	rd.tex_offset = d.tex_offset;
	rd.tex_w = d.tex_size[0];
	rd.tex_h = d.tex_size[1];
	rd.mode = d.mode;
	rd.blend = d.blend;
	rd.num_parts = st.num_parts;
	rd.reserved = 0;
	a.rdraws[di] = rd;

	RasterBox box;
	if (st.num_parts == 0 || st.bx0 >= a.width || st.bx1 <= 0)
		box = RasterBox{0, 0, 0, 0};
	else
		box = RasterBox{int16_t(max(st.bx0, 0)), int16_t(st.by0), int16_t(min(st.bx1, a.width)), int16_t(st.by1)};
	a.boxes[di] = box;
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

// Texel address of pixel (x, y) for one draw; returns false if the pixel is not covered. Addresses
// are the reference's (u32 arithmetic for the perspective modes, i32 for affine, then as usize).
__device__ __forceinline__ bool texel_address(const RasterDraw& rd, const RasterPart& p, int32_t x, int32_t y,
	int32_t width, uint64_t& address)
{
	const int32_t k = y - p.y_start_int;
	const Fixed16 x_left = wadd(p.x_left0, wmul(k, p.dx_dy_left));
	const Fixed16 x_right = wadd(p.x_right0, wmul(k, p.dx_dy_right));
	const int32_t xs = max(x_left >> 16, 0);
	const int32_t xe = min(x_right >> 16, width);
	if (x < xs || x >= xe) return false;
	const int32_t i = x - xs;
	const int32_t len1 = (xe - 1) - xs;
	const int64_t span_start_x = xs, span_end_x = xe - 1;

	if (rd.mode == SW_RASTER_AFFINE) // rasterizer.rs:684-719
	{
		int32_t tcl[2], tcr[2];
#pragma unroll
		for (int c = 0; c < 2; ++c)
		{
			tcl[c] = wadd(p.tc_left0[c], wmul(k, p.d_tc_left[c]));
			tcr[c] = wadd(p.tc_right0[c], wmul(k, p.d_tc_right[c]));
		}
		const Fixed16 x_delta = max(wsub(x_right, x_left), FIXED16_ONE);
		const int32_t tc0 = wadd(tcl[0], wmul(i, fx_div(wsub(tcr[0], tcl[0]), x_delta)));
		const int32_t tc1 = wadd(tcl[1], wmul(i, fx_div(wsub(tcr[1], tcl[1]), x_delta)));
		address = uint64_t(int64_t(wadd(tc0 >> 16, wmul(tc1 >> 16, int32_t(rd.tex_w)))));
		return true;
	}

	const int64_t line_inv_z = w64add(w64mul(int64_t(y), rd.d_inv_z_dy), rd.inv_z_k);
	const int64_t inv_z_min = 1 << INV_Z_PRE_SHIFT, inv_z_max = 1 << 29;
	if (rd.mode == SW_RASTER_LINE_Z_CORRECTED) // rasterizer.rs:528-572
	{
		const uint32_t izs = uint32_t(min(max(w64add(w64mul(span_start_x, rd.d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
		const uint32_t ize = uint32_t(min(max(w64add(w64mul(span_end_x, rd.d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
		const uint64_t zs = (1u << Z_CALC_SHIFT) / (izs >> INV_Z_PRE_SHIFT);
		const uint64_t ze = (1u << Z_CALC_SHIFT) / (ize >> INV_Z_PRE_SHIFT);
		int32_t tc[2];
#pragma unroll
		for (int c = 0; c < 2; ++c)
		{
			const int64_t line_tc = w64add(w64mul(int64_t(y), rd.d_tc_dy[c]), rd.tc_k[c]);
			const uint64_t ts = uint64_t(max(w64add(line_tc, w64mul(span_start_x, rd.d_tc_dx[c])), int64_t(0)));
			const uint64_t te = uint64_t(max(w64add(line_tc, w64mul(span_end_x, rd.d_tc_dx[c])), int64_t(0)));
			const uint64_t max_tc = (uint64_t(c == 0 ? rd.tex_w : rd.tex_h) << 16) - 1;
			const int32_t s0 = int32_t(min((zs * ts) >> (TC_FINAL_SHIFT - 16), max_tc));
			const int32_t s1 = int32_t(min((ze * te) >> (TC_FINAL_SHIFT - 16), max_tc));
			const int32_t step = len1 > 0 ? (s1 - s0) / len1 : 0;
			tc[c] = wadd(s0, wmul(i, step));
		}
		address = uint32_t(tc[0] >> 16) + uint32_t(tc[1] >> 16) * rd.tex_w;
		return true;
	}

	// Full perspective, rasterizer.rs:340-445.
	const int32_t izs = int32_t(max(inv_z_min, min(w64add(w64mul(span_start_x, rd.d_inv_z_dx), line_inv_z), inv_z_max)));
	const int32_t ize = int32_t(max(inv_z_min, min(w64add(w64mul(span_end_x, rd.d_inv_z_dx), line_inv_z), inv_z_max)));
	const int32_t d_inv_z = len1 > 0 ? (ize - izs) / len1 : 0;
	const int32_t inv_z = wadd(izs, wmul(i, d_inv_z));
	const int64_t izc = int64_t(izs - (1 << INV_Z_PRE_SHIFT));
	const int tc_max_shift = INV_Z_SHIFT - TC_SHIFT;
	const int64_t tc_max_max = 1 << 29;
	int32_t tc[2];
#pragma unroll
	for (int c = 0; c < 2; ++c)
	{
		const int64_t size = int64_t(c == 0 ? rd.tex_w : rd.tex_h);
		const int64_t line_tc = w64add(w64mul(int64_t(y), rd.d_tc_dy[c]), rd.tc_k[c]);
		const int64_t tc_max_start = max(int64_t(0), min((w64mul(izc, size) >> tc_max_shift) - 1, tc_max_max));
		const int32_t tcs = int32_t(max(int64_t(0), min(w64add(w64mul(span_start_x, rd.d_tc_dx[c]), line_tc), tc_max_start)));
		int32_t start = tcs, step = 0;
		if (len1 > 0)
		{
			const int64_t tc_max_end =
				max(int64_t(0), min((w64mul(izc + int64_t(wmul(d_inv_z, len1)), size) >> tc_max_shift) - 1, tc_max_max));
			const int32_t tce = int32_t(max(int64_t(0), min(w64add(w64mul(span_end_x, rd.d_tc_dx[c]), line_tc), tc_max_end)));
			step = (tce - tcs) / len1;
			start = tce > tcs ? tcs : wsub(tce, wmul(step, len1));
		}
		tc[c] = wadd(start, wmul(i, step));
	}
	const uint32_t zdiv = uint32_t(inv_z) >> INV_Z_PRE_SHIFT;
	const uint32_t z = (1u << Z_CALC_SHIFT) / (zdiv ? zdiv : 1u);
	const uint32_t pu = uint32_t((uint64_t(z) * uint64_t(int64_t(tc[0]))) >> TC_FINAL_SHIFT);
	const uint32_t pv = uint32_t((uint64_t(z) * uint64_t(int64_t(tc[1]))) >> TC_FINAL_SHIFT);
	address = uint32_t(pu + pv * rd.tex_w);
	return true;
}

template <class P>
__global__ void __launch_bounds__(256) raster_tiles_kernel(RasterArgs a)
{
	typedef typename P::T T;
	__shared__ uint32_t hits[256];
	__shared__ uint32_t warp_counts[8];

	const int tiles_x = (a.width + TILE - 1) / TILE;
	const int tx0 = int(blockIdx.x % tiles_x) * TILE;
	const int ty0 = int(blockIdx.x / tiles_x) * TILE;
	const int tid = threadIdx.x;
	const int x = tx0 + (tid & (TILE - 1));
	const int y = ty0 + (tid >> 4);
	const bool valid = x < a.width && y < a.height;
	const int tx1 = min(tx0 + TILE, a.width), ty1 = min(ty0 + TILE, a.height);

	T* fb = static_cast<T*>(a.framebuffer);
	const T* arena = static_cast<const T*>(a.arena);
	T pix = T(0);
	if (valid)
	{
		if (a.clear_background)
		{
			// ColorVec::from_color_f32x3(&[32.0, 16.0, 8.0]).into(), partial_renderer.rs:255
			pix = P::FORMAT == SW_PIXEL_C64 ? T(8ull | (16ull << 16) | (32ull << 32)) : T(0x00201008u);
		}
		else
			pix = fb[uint64_t(y) * a.width + x];
	}
	unsigned int local_errors = 0, local_writes = 0;

	const int lane = tid & 31, warp = tid >> 5;
	for (uint32_t chunk = 0; chunk < a.num_draws; chunk += 256)
	{
		const uint32_t di = chunk + tid;
		bool hit = false;
		if (di < a.num_draws)
		{
			const RasterBox b = a.boxes[di];
			hit = b.x0 < tx1 && b.x1 > tx0 && b.y0 < ty1 && b.y1 > ty0 && b.x0 < b.x1 && b.y0 < b.y1;
		}
		const unsigned mask = __ballot_sync(0xFFFFFFFFu, hit);
		if (lane == 0) warp_counts[warp] = __popc(mask);
		__syncthreads();
		uint32_t base = 0, total = 0;
#pragma unroll
		for (int w = 0; w < 8; ++w)
		{
			const uint32_t c = warp_counts[w];
			if (w < warp) base += c;
			total += c;
		}
		if (hit) hits[base + __popc(mask & ((1u << lane) - 1u))] = di;
		__syncthreads();

		if (valid)
			for (uint32_t h = 0; h < total; ++h)
			{
				const uint32_t d = hits[h];
				const RasterBox b = a.boxes[d];
				if (x < b.x0 || x >= b.x1 || y < b.y0 || y >= b.y1) continue;
				const RasterDraw rd = a.rdraws[d];
				const RasterPart* parts = a.parts + uint64_t(d) * SW_RASTER_MAX_PARTS;
				for (uint32_t pi = 0; pi < rd.num_parts; ++pi)
				{
					const RasterPart p = parts[pi];
					if (y < p.y_start_int || y >= p.y_end_int) continue;
					uint64_t ua;
					if (texel_address(rd, p, x, y, a.width, ua))
					{
						if (ua >= uint64_t(rd.tex_w) * rd.tex_h)
						{
							++local_errors;
							ua = 0;
						}
						const T texel = arena[rd.tex_offset + ua];
						blend_into<P>(pix, texel, rd.blend);
						++local_writes;
					}
					break;
				}
			}
		__syncthreads();
	}
	if (valid) fb[uint64_t(y) * a.width + x] = pix;
	if (local_errors) atomicAdd(a.error_counter, local_errors);
	// Pixel writes (span pixels processed) for the traffic accounting, one atomic per warp.
	for (int o = 16; o > 0; o >>= 1) local_writes += __shfl_xor_sync(0xFFFFFFFFu, local_writes, o);
	if ((tid & 31) == 0 && local_writes)
		atomicAdd(reinterpret_cast<unsigned long long*>(a.error_counter + 2), (unsigned long long)local_writes);
}

} // namespace

int launch_raster(const RasterArgs& args, uint32_t pixel_format, int num_sms, cudaStream_t stream)
{
	if (args.num_draws > 0)
		raster_setup_kernel<<<(args.num_draws + 127) / 128, 128, 0, stream>>>(args);
	const unsigned tiles = unsigned(((args.width + TILE - 1) / TILE) * ((args.height + TILE - 1) / TILE));
	if (tiles == 0) return 0;
	if (pixel_format == SW_PIXEL_C64)
		raster_tiles_kernel<PixC64><<<tiles, 256, 0, stream>>>(args);
	else
		raster_tiles_kernel<PixC32><<<tiles, 256, 0, stream>>>(args);
	(void)num_sms;
	return int(cudaGetLastError());
}

} // namespace swgpu
