// Test infrastructure (oracle): CPU restatement of the reference's polygon rasteriser.
//
// Follows src/square_wheel/rasterizer.rs:137-271 (edge walk of fill_polygon_impl_2_static_params),
// :273-454 (fill_polygon_part, full perspective), :456-581 (line-z corrected), :583-729 (affine),
// :765-1292 (fill_triangle_impl, fill_triangle_part: textured triangles with per-vertex light),
// :1511-1536 (write_into_framebuffer), :1573-1580 (fixed-point constants), src/common/fixed_math.rs,
// and its caller src/square_wheel/partial_renderer.rs:1192-1283 (perform_rasterization; N-thread mode
// uses src/square_wheel/rect_splitting.rs:23-78).
#include "sw_oracle.h"
#include "sw_oracle_math.h"

#include <thread>
#include <vector>

namespace sworacle
{
namespace
{

typedef int32_t Fixed16;
const Fixed16 FIXED16_ONE = 1 << 16;
const Fixed16 FIXED16_HALF = FIXED16_ONE >> 1;

inline Fixed16 int_to_fixed16(int32_t x) { return int32_t(uint32_t(x) << 16); }
inline int32_t fixed16_round_to_int(Fixed16 x) { return wadd(x, FIXED16_HALF) >> 16; }
inline int32_t fixed16_floor_to_int(Fixed16 x) { return x >> 16; }
inline float fixed16_to_f32(Fixed16 x) { return float(x) / float(FIXED16_ONE); }
inline Fixed16 f32_to_fixed16_unchecked(float x) { return f2i32(x * float(FIXED16_ONE)); }
inline Fixed16 fixed16_mul(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) * int64_t(y)) >> 16); }
inline Fixed16 fixed16_div(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) << 16) / int64_t(y)); }
inline Fixed16 fixed16_mul_div(Fixed16 x, Fixed16 y, Fixed16 z) { return int32_t(int64_t(x) * int64_t(y) / int64_t(z)); }

const int TC_SHIFT = 24;
const int INV_Z_SHIFT = 29;
const int INV_Z_PRE_SHIFT = 8;
const int Z_CALC_SHIFT = 31;
const int TC_FINAL_SHIFT = TC_SHIFT + Z_CALC_SHIFT - INV_Z_SHIFT + INV_Z_PRE_SHIFT; // 34
const float TC_SCALE = float(1 << TC_SHIFT);
const float INV_Z_SCALE = float(1 << INV_Z_SHIFT);

struct ClipRect
{
	int32_t min_x, min_y, max_x, max_y;
};
struct PolygonSide
{
	Fixed16 x_start;
	Fixed16 dx_dy;
};

template <class P>
struct Raster
{
	typedef typename P::T T;
	T* color_buffer;
	int32_t row_size;
	ClipRect clip_rect;
	const T* texture_data;
	uint64_t texture_len;
	uint64_t* bad_fetches;

	T fetch(uint64_t address) const
	{
		if (address >= texture_len)
		{
			if (bad_fetches) ++*bad_fetches;
			return texture_data[0];
		}
		return texture_data[address];
	}

	static void write(T& dst, T texel, uint32_t blend) // rasterizer.rs:1511-1536
	{
		switch (blend)
		{
		case SW_BLEND_NONE: dst = texel; break;
		case SW_BLEND_AVERAGE: dst = P::average(dst, texel); break;
		case SW_BLEND_ADDITIVE: dst = P::saturated_sum(dst, texel); break;
		case SW_BLEND_ALPHA_TEST:
			if (P::test_alpha(texel)) dst = texel;
			break;
		case SW_BLEND_ALPHA_BLEND: dst = alpha_blend<P>(dst, texel); break;
		}
	}

	// rasterizer.rs:273-454
	void part_full_perspective(Fixed16 y_start, Fixed16 y_end, PolygonSide left_side, PolygonSide right_side,
		const SwDrawCmd& d, uint32_t blend)
	{
		const float* de = d.depth_eq;
		const float* te = d.tc_eq;
		int64_t d_inv_z_dx = f2i64(INV_Z_SCALE * de[0]);
		int64_t d_inv_z_dy = f2i64(INV_Z_SCALE * de[1]);
		int64_t inv_z_k = f2i64(INV_Z_SCALE * (de[2] + (de[0] + de[1]) * 0.5f));
		int64_t d_tc_dx[2] = {f2i64(TC_SCALE * te[0]), f2i64(TC_SCALE * te[1])};
		int64_t d_tc_dy[2] = {f2i64(TC_SCALE * te[2]), f2i64(TC_SCALE * te[3])};
		int64_t tc_k[2] = {f2i64(TC_SCALE * (te[4] + (te[0] + te[2]) * 0.5f)), f2i64(TC_SCALE * (te[5] + (te[1] + te[3]) * 0.5f))};
		const int32_t tex_size[2] = {int32_t(d.tex_size[0]), int32_t(d.tex_size[1])};
		const uint32_t texture_width = uint32_t(tex_size[0]);

		int32_t y_start_int = std::max(fixed16_round_to_int(y_start), clip_rect.min_y);
		int32_t y_end_int = std::min(fixed16_round_to_int(y_end), clip_rect.max_y);
		Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
		Fixed16 x_left = wadd(wadd(left_side.x_start, fixed16_mul(y_start_delta, left_side.dx_dy)), FIXED16_HALF);
		Fixed16 x_right = wadd(wadd(right_side.x_start, fixed16_mul(y_start_delta, right_side.dx_dy)), FIXED16_HALF);
		int64_t line_inv_z = wadd64(wmul64(int64_t(y_start_int), d_inv_z_dy), inv_z_k);
		int64_t line_tc[2] = {wadd64(wmul64(int64_t(y_start_int), d_tc_dy[0]), tc_k[0]),
			wadd64(wmul64(int64_t(y_start_int), d_tc_dy[1]), tc_k[1])};

		for (int32_t y_int = y_start_int; y_int < y_end_int; ++y_int)
		{
			int32_t x_start_int = std::max(fixed16_floor_to_int(x_left), clip_rect.min_x);
			int32_t x_end_int = std::min(fixed16_floor_to_int(x_right), clip_rect.max_x);
			if (x_start_int < x_end_int)
			{
				T* line_dst = color_buffer + int64_t(y_int) * row_size;
				int64_t span_start_x = x_start_int;
				int64_t span_end_x = int64_t(x_end_int - 1);
				int32_t span_length_minus_one = (x_end_int - 1) - x_start_int;

				const int64_t inv_z_min = 1 << INV_Z_PRE_SHIFT;
				const int64_t inv_z_max = 1 << 29;
				int32_t span_inv_z_start = int32_t(
					std::max(inv_z_min, std::min(wadd64(wmul64(span_start_x, d_inv_z_dx), line_inv_z), inv_z_max)));
				int32_t span_inv_z_end =
					int32_t(std::max(inv_z_min, std::min(wadd64(wmul64(span_end_x, d_inv_z_dx), line_inv_z), inv_z_max)));
				int32_t span_d_inv_z = span_length_minus_one > 0 ? (span_inv_z_end - span_inv_z_start) / span_length_minus_one : 0;
				int32_t span_inv_z = span_inv_z_start;

				int32_t span_tc[2] = {0, 0};
				int32_t span_d_tc[2] = {0, 0};
				for (int i = 0; i < 2; ++i)
				{
					const int tc_max_shift = INV_Z_SHIFT - TC_SHIFT;
					const int64_t tc_max_max = 1 << 29;
					int64_t span_inv_z_corrected = int64_t(span_inv_z - (1 << INV_Z_PRE_SHIFT));
					int64_t tc_max_start = std::max(int64_t(0),
						std::min((wmul64(span_inv_z_corrected, int64_t(tex_size[i])) >> tc_max_shift) - 1, tc_max_max));
					int32_t span_tc_start = int32_t(std::max(
						int64_t(0), std::min(wadd64(wmul64(span_start_x, d_tc_dx[i]), line_tc[i]), tc_max_start)));
					if (span_length_minus_one > 0)
					{
						int64_t tc_max_end = std::max(int64_t(0),
							std::min((wmul64(span_inv_z_corrected + int64_t(wmul(span_d_inv_z, span_length_minus_one)),
										  int64_t(tex_size[i])) >>
										 tc_max_shift) -
									1,
								tc_max_max));
						int32_t span_tc_end = int32_t(std::max(
							int64_t(0), std::min(wadd64(wmul64(span_end_x, d_tc_dx[i]), line_tc[i]), tc_max_end)));
						span_d_tc[i] = (span_tc_end - span_tc_start) / span_length_minus_one;
						if (span_tc_end > span_tc_start)
							span_tc[i] = span_tc_start;
						else
							span_tc[i] = wsub(span_tc_end, wmul(span_d_tc[i], span_length_minus_one));
					}
					else
						span_tc[i] = span_tc_start;
				}

				for (int32_t x = x_start_int; x < x_end_int; ++x)
				{
					uint32_t z = (1u << Z_CALC_SHIFT) / (uint32_t(span_inv_z) >> INV_Z_PRE_SHIFT);
					uint32_t pix_tc0 = uint32_t((uint64_t(z) * uint64_t(int64_t(span_tc[0]))) >> TC_FINAL_SHIFT);
					uint32_t pix_tc1 = uint32_t((uint64_t(z) * uint64_t(int64_t(span_tc[1]))) >> TC_FINAL_SHIFT);
					uint32_t texel_address = pix_tc0 + pix_tc1 * texture_width;
					write(line_dst[x], fetch(texel_address), blend);
					span_inv_z = wadd(span_inv_z, span_d_inv_z);
					span_tc[0] = wadd(span_tc[0], span_d_tc[0]);
					span_tc[1] = wadd(span_tc[1], span_d_tc[1]);
				}
			}
			x_left = wadd(x_left, left_side.dx_dy);
			x_right = wadd(x_right, right_side.dx_dy);
			line_inv_z = wadd64(line_inv_z, d_inv_z_dy);
			line_tc[0] = wadd64(line_tc[0], d_tc_dy[0]);
			line_tc[1] = wadd64(line_tc[1], d_tc_dy[1]);
		}
	}

	// rasterizer.rs:456-581
	void part_line_z_corrected(Fixed16 y_start, Fixed16 y_end, PolygonSide left_side, PolygonSide right_side,
		const SwDrawCmd& d, uint32_t blend)
	{
		const int LINE_TC_SHIFT = 16;
		const float* de = d.depth_eq;
		const float* te = d.tc_eq;
		int64_t d_inv_z_dx = f2i64(INV_Z_SCALE * de[0]);
		int64_t d_inv_z_dy = f2i64(INV_Z_SCALE * de[1]);
		int64_t inv_z_k = f2i64(INV_Z_SCALE * (de[2] + (de[0] + de[1]) * 0.5f));
		int64_t d_tc_dx[2] = {f2i64(TC_SCALE * te[0]), f2i64(TC_SCALE * te[1])};
		int64_t d_tc_dy[2] = {f2i64(TC_SCALE * te[2]), f2i64(TC_SCALE * te[3])};
		int64_t tc_k[2] = {f2i64(TC_SCALE * (te[4] + (te[0] + te[2]) * 0.5f)), f2i64(TC_SCALE * (te[5] + (te[1] + te[3]) * 0.5f))};
		const uint32_t texture_width = d.tex_size[0];

		int32_t y_start_int = std::max(fixed16_round_to_int(y_start), clip_rect.min_y);
		int32_t y_end_int = std::min(fixed16_round_to_int(y_end), clip_rect.max_y);
		Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
		Fixed16 x_left = wadd(wadd(left_side.x_start, fixed16_mul(y_start_delta, left_side.dx_dy)), FIXED16_HALF);
		Fixed16 x_right = wadd(wadd(right_side.x_start, fixed16_mul(y_start_delta, right_side.dx_dy)), FIXED16_HALF);
		int64_t line_inv_z = wadd64(wmul64(int64_t(y_start_int), d_inv_z_dy), inv_z_k);
		int64_t line_tc[2] = {wadd64(wmul64(int64_t(y_start_int), d_tc_dy[0]), tc_k[0]),
			wadd64(wmul64(int64_t(y_start_int), d_tc_dy[1]), tc_k[1])};

		for (int32_t y_int = y_start_int; y_int < y_end_int; ++y_int)
		{
			int32_t x_start_int = std::max(fixed16_floor_to_int(x_left), clip_rect.min_x);
			int32_t x_end_int = std::min(fixed16_floor_to_int(x_right), clip_rect.max_x);
			if (x_start_int < x_end_int)
			{
				T* line_dst = color_buffer + int64_t(y_int) * row_size;
				int64_t span_start_x = x_start_int;
				int64_t span_end_x = int64_t(x_end_int - 1);
				int32_t span_length_minus_one = (x_end_int - 1) - x_start_int;
				const int64_t inv_z_min = 1 << INV_Z_PRE_SHIFT;
				const int64_t inv_z_max = 1 << 29;
				uint32_t span_inv_z_start =
					uint32_t(std::min(std::max(wadd64(wmul64(span_start_x, d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
				uint32_t span_inv_z_end =
					uint32_t(std::min(std::max(wadd64(wmul64(span_end_x, d_inv_z_dx), line_inv_z), inv_z_min), inv_z_max));
				uint64_t span_z_start = uint64_t((1u << Z_CALC_SHIFT) / (span_inv_z_start >> INV_Z_PRE_SHIFT));
				uint64_t span_z_end = uint64_t((1u << Z_CALC_SHIFT) / (span_inv_z_end >> INV_Z_PRE_SHIFT));

				int32_t span_tc[2] = {0, 0};
				int32_t span_d_tc[2] = {0, 0};
				for (int i = 0; i < 2; ++i)
				{
					uint64_t tc_start = uint64_t(std::max(wadd64(line_tc[i], wmul64(span_start_x, d_tc_dx[i])), int64_t(0)));
					uint64_t tc_end = uint64_t(std::max(wadd64(line_tc[i], wmul64(span_end_x, d_tc_dx[i])), int64_t(0)));
					uint64_t max_tc = (uint64_t(d.tex_size[i]) << LINE_TC_SHIFT) - 1;
					int32_t tc_mul_z_start = int32_t(std::min((span_z_start * tc_start) >> (TC_FINAL_SHIFT - LINE_TC_SHIFT), max_tc));
					int32_t tc_mul_z_end = int32_t(std::min((span_z_end * tc_end) >> (TC_FINAL_SHIFT - LINE_TC_SHIFT), max_tc));
					span_tc[i] = tc_mul_z_start;
					if (span_length_minus_one > 0) span_d_tc[i] = (tc_mul_z_end - tc_mul_z_start) / span_length_minus_one;
				}

				for (int32_t x = x_start_int; x < x_end_int; ++x)
				{
					int32_t tc_int0 = span_tc[0] >> LINE_TC_SHIFT;
					int32_t tc_int1 = span_tc[1] >> LINE_TC_SHIFT;
					uint32_t texel_address = uint32_t(tc_int0) + uint32_t(tc_int1) * texture_width;
					write(line_dst[x], fetch(texel_address), blend);
					span_tc[0] = wadd(span_tc[0], span_d_tc[0]);
					span_tc[1] = wadd(span_tc[1], span_d_tc[1]);
				}
			}
			x_left = wadd(x_left, left_side.dx_dy);
			x_right = wadd(x_right, right_side.dx_dy);
			line_inv_z = wadd64(line_inv_z, d_inv_z_dy);
			line_tc[0] = wadd64(line_tc[0], d_tc_dy[0]);
			line_tc[1] = wadd64(line_tc[1], d_tc_dy[1]);
		}
	}

	// rasterizer.rs:583-729
	void part_affine(Fixed16 y_start, Fixed16 y_end, PolygonSide left_side, PolygonSide right_side, const SwDrawCmd& d,
		uint32_t blend)
	{
		const float* de = d.depth_eq;
		const float* te = d.tc_eq;
		float y_start_f32 = fixed16_to_f32(y_start);
		float y_end_f32 = fixed16_to_f32(y_end);
		Fixed16 y_delta = wsub(y_end, y_start);
		float x_start_left = fixed16_to_f32(left_side.x_start);
		float x_end_left = fixed16_to_f32(wadd(left_side.x_start, fixed16_mul(y_delta, left_side.dx_dy)));
		float x_start_right = fixed16_to_f32(right_side.x_start);
		float x_end_right = fixed16_to_f32(wadd(right_side.x_start, fixed16_mul(y_delta, right_side.dx_dy)));
		float z_start_left = 1.0f / (de[0] * x_start_left + de[1] * y_start_f32 + de[2]);
		float z_end_left = 1.0f / (de[0] * x_end_left + de[1] * y_end_f32 + de[2]);
		float z_start_right = 1.0f / (de[0] * x_start_right + de[1] * y_start_f32 + de[2]);
		float z_end_right = 1.0f / (de[0] * x_end_right + de[1] * y_end_f32 + de[2]);

		Fixed16 y_delta_for_tc_interpolation = std::max(y_delta, FIXED16_ONE);
		Fixed16 tc_left[2], tc_right[2], d_tc_left[2], d_tc_right[2];
		for (int i = 0; i < 2; ++i)
		{
			const Fixed16 max_tc = wsub(int_to_fixed16(int32_t(d.tex_size[i])), 1);
			const float dtdx = te[i], dtdy = te[2 + i], tk = te[4 + i];
			Fixed16 tc_start_left =
				std::min(std::max(f32_to_fixed16_unchecked(z_start_left * (x_start_left * dtdx + y_start_f32 * dtdy + tk)), 0), max_tc);
			Fixed16 tc_end_left =
				std::min(std::max(f32_to_fixed16_unchecked(z_end_left * (x_end_left * dtdx + y_end_f32 * dtdy + tk)), 0), max_tc);
			Fixed16 tc_start_right = std::min(
				std::max(f32_to_fixed16_unchecked(z_start_right * (x_start_right * dtdx + y_start_f32 * dtdy + tk)), 0), max_tc);
			Fixed16 tc_end_right =
				std::min(std::max(f32_to_fixed16_unchecked(z_end_right * (x_end_right * dtdx + y_end_f32 * dtdy + tk)), 0), max_tc);
			d_tc_left[i] = fixed16_div(wsub(tc_end_left, tc_start_left), y_delta_for_tc_interpolation);
			d_tc_right[i] = fixed16_div(wsub(tc_end_right, tc_start_right), y_delta_for_tc_interpolation);
			tc_left[i] = tc_start_left;
			tc_right[i] = tc_start_right;
		}

		int32_t y_start_int = std::max(fixed16_round_to_int(y_start), clip_rect.min_y);
		int32_t y_end_int = std::min(fixed16_round_to_int(y_end), clip_rect.max_y);
		Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
		Fixed16 x_left = wadd(wadd(left_side.x_start, fixed16_mul(y_start_delta, left_side.dx_dy)), FIXED16_HALF);
		Fixed16 x_right = wadd(wadd(right_side.x_start, fixed16_mul(y_start_delta, right_side.dx_dy)), FIXED16_HALF);
		for (int i = 0; i < 2; ++i)
		{
			tc_left[i] = wadd(tc_left[i], fixed16_mul(y_start_delta, d_tc_left[i]));
			tc_right[i] = wadd(tc_right[i], fixed16_mul(y_start_delta, d_tc_right[i]));
		}

		for (int32_t y_int = y_start_int; y_int < y_end_int; ++y_int)
		{
			int32_t x_start_int = std::max(fixed16_floor_to_int(x_left), clip_rect.min_x);
			int32_t x_end_int = std::min(fixed16_floor_to_int(x_right), clip_rect.max_x);
			if (x_start_int < x_end_int)
			{
				T* line_dst = color_buffer + int64_t(y_int) * row_size;
				Fixed16 tc[2] = {tc_left[0], tc_left[1]};
				Fixed16 x_delta_for_tc_interpolation = std::max(wsub(x_right, x_left), FIXED16_ONE);
				Fixed16 d_tc[2] = {fixed16_div(wsub(tc_right[0], tc_left[0]), x_delta_for_tc_interpolation),
					fixed16_div(wsub(tc_right[1], tc_left[1]), x_delta_for_tc_interpolation)};
				for (int32_t x = x_start_int; x < x_end_int; ++x)
				{
					int32_t tc_int0 = fixed16_floor_to_int(tc[0]);
					int32_t tc_int1 = fixed16_floor_to_int(tc[1]);
					int32_t texel_address = wadd(tc_int0, wmul(tc_int1, int32_t(d.tex_size[0])));
					write(line_dst[x], fetch(uint64_t(int64_t(texel_address))), blend);
					tc[0] = wadd(tc[0], d_tc[0]);
					tc[1] = wadd(tc[1], d_tc[1]);
				}
			}
			x_left = wadd(x_left, left_side.dx_dy);
			x_right = wadd(x_right, right_side.dx_dy);
			tc_left[0] = wadd(tc_left[0], d_tc_left[0]);
			tc_left[1] = wadd(tc_left[1], d_tc_left[1]);
			tc_right[0] = wadd(tc_right[0], d_tc_right[0]);
			tc_right[1] = wadd(tc_right[1], d_tc_right[1]);
		}
	}

	void draw_part(Fixed16 y0, Fixed16 y1, PolygonSide l, PolygonSide r, const SwDrawCmd& d)
	{
		switch (d.mode)
		{
		case SW_RASTER_FULL_PERSPECTIVE: part_full_perspective(y0, y1, l, r, d, d.blend); break;
		case SW_RASTER_LINE_Z_CORRECTED: part_line_z_corrected(y0, y1, l, r, d, d.blend); break;
		default: part_affine(y0, y1, l, r, d, d.blend); break;
		}
	}

	// Edge walk, rasterizer.rs:160-270
	void fill_polygon(const SwVertex16* vertices, uint32_t n, const SwDrawCmd& d)
	{
		uint32_t lower_vertex_index = 0;
		Fixed16 min_y = vertices[0].y;
		for (uint32_t i = 0; i < n; ++i)
			if (vertices[i].y < min_y)
			{
				min_y = vertices[i].y;
				lower_vertex_index = i;
			}
		uint32_t left_index = lower_vertex_index, right_index = lower_vertex_index;
		Fixed16 cur_y = min_y;
		for (;;)
		{
			uint32_t next_left_index = left_index + n - 1;
			if (next_left_index >= n) next_left_index -= n;
			uint32_t next_right_index = right_index + 1;
			if (next_right_index >= n) next_right_index -= n;
			const SwVertex16& left_vertex = vertices[left_index];
			const SwVertex16& next_left_vertex = vertices[next_left_index];
			const SwVertex16& right_vertex = vertices[right_index];
			const SwVertex16& next_right_vertex = vertices[next_right_index];
			Fixed16 dy_left = wsub(next_left_vertex.y, left_vertex.y);
			Fixed16 dy_right = wsub(next_right_vertex.y, right_vertex.y);
			Fixed16 next_y = std::min(next_left_vertex.y, next_right_vertex.y);
			if (dy_left > FIXED16_HALF && dy_right > FIXED16_HALF)
			{
				Fixed16 dx_dy_left = fixed16_div(wsub(next_left_vertex.x, left_vertex.x), dy_left);
				Fixed16 dx_dy_right = fixed16_div(wsub(next_right_vertex.x, right_vertex.x), dy_right);
				draw_part(cur_y, next_y,
					PolygonSide{wadd(left_vertex.x, fixed16_mul(dx_dy_left, wsub(cur_y, left_vertex.y))), dx_dy_left},
					PolygonSide{wadd(right_vertex.x, fixed16_mul(dx_dy_right, wsub(cur_y, right_vertex.y))), dx_dy_right}, d);
			}
			else if (dy_left > 0 && dy_right > 0)
			{
				int32_t cur_y_int = fixed16_round_to_int(cur_y);
				int32_t next_y_int = fixed16_round_to_int(next_y);
				if (cur_y_int < next_y_int)
				{
					Fixed16 thin_line_y = wadd(int_to_fixed16(cur_y_int), FIXED16_HALF);
					Fixed16 x_start_left = wadd(left_vertex.x,
						fixed16_mul_div(wsub(thin_line_y, left_vertex.y), wsub(next_left_vertex.x, left_vertex.x), dy_left));
					Fixed16 x_start_right = wadd(right_vertex.x,
						fixed16_mul_div(wsub(thin_line_y, right_vertex.y), wsub(next_right_vertex.x, right_vertex.x), dy_right));
					draw_part(cur_y, next_y, PolygonSide{x_start_left, 0}, PolygonSide{x_start_right, 0}, d);
				}
			}
			if (next_left_index == next_right_index) break;
			if (next_right_vertex.y < next_left_vertex.y)
				right_index = next_right_index;
			else
				left_index = next_left_index;
			cur_y = next_y;
		}
	}

	// ---- triangles: Rasterizer::fill_triangle_impl / fill_triangle_part, rasterizer.rs:765-1292 ----

	const uint32_t* lite = nullptr; // the triangle's Color32 texture
	uint64_t lite_len = 0;

	uint32_t fetch_lite(uint64_t address) const
	{
		if (address >= lite_len)
		{
			if (bad_fetches) ++*bad_fetches;
			return lite[0];
		}
		return lite[address];
	}

	void fill_triangle(const SwTriVertex* vertices, int32_t tex_w, int32_t tex_h, uint32_t blend)
	{
		// sort by y: upper (max), lower (min), middle (rasterizer.rs:773-793)
		int upper_index, lower_index;
		if (vertices[0].y >= vertices[1].y && vertices[0].y >= vertices[2].y)
		{
			upper_index = 0;
			lower_index = vertices[1].y < vertices[2].y ? 1 : 2;
		}
		else if (vertices[1].y >= vertices[0].y && vertices[1].y >= vertices[2].y)
		{
			upper_index = 1;
			lower_index = vertices[0].y < vertices[2].y ? 0 : 2;
		}
		else
		{
			upper_index = 2;
			lower_index = vertices[0].y < vertices[1].y ? 0 : 1;
		}
		const int middle_index = 3 - upper_index - lower_index;
		const SwTriVertex& upper = vertices[upper_index];
		const SwTriVertex& lower = vertices[lower_index];
		const SwTriVertex& middle = vertices[middle_index];

		const Fixed16 long_edge_dy = std::max(wsub(upper.y, lower.y), FIXED16_HALF);
		const Fixed16 lower_part_dy = std::max(wsub(middle.y, lower.y), FIXED16_HALF);
		const Fixed16 upper_part_dy = std::max(wsub(upper.y, middle.y), FIXED16_HALF);

		const Fixed16 long_edge_dx_dy = fixed16_div(wsub(upper.x, lower.x), long_edge_dy);
		const Fixed16 long_edge_x_in_middle = wadd(lower.x, fixed16_mul(long_edge_dx_dy, wsub(middle.y, lower.y)));
		const Fixed16 lower_part_dx_dy = fixed16_div(wsub(middle.x, lower.x), lower_part_dy);
		const Fixed16 upper_part_dx_dy = fixed16_div(wsub(upper.x, middle.x), upper_part_dy);

		Fixed16 long_edge_d_tc_dy[2], long_edge_tc_in_middle[2], d_tc_dy_lower[2], d_tc_dy_upper[2];
		for (int i = 0; i < 2; ++i)
		{
			long_edge_d_tc_dy[i] = fixed16_div(wsub(upper.tc[i], lower.tc[i]), long_edge_dy);
			long_edge_tc_in_middle[i] = wadd(lower.tc[i], fixed16_mul(long_edge_d_tc_dy[i], lower_part_dy));
			d_tc_dy_lower[i] = fixed16_div(wsub(middle.tc[i], lower.tc[i]), lower_part_dy);
			d_tc_dy_upper[i] = fixed16_div(wsub(upper.tc[i], middle.tc[i]), upper_part_dy);
		}
		Fixed16 long_edge_d_light_dy[3], long_edge_light_in_middle[3], d_light_dy_lower[3], d_light_dy_upper[3];
		for (int i = 0; i < 3; ++i)
		{
			long_edge_d_light_dy[i] = fixed16_div(wsub(upper.light[i], lower.light[i]), long_edge_dy);
			long_edge_light_in_middle[i] = wadd(lower.light[i], fixed16_mul(long_edge_d_light_dy[i], lower_part_dy));
			d_light_dy_lower[i] = fixed16_div(wsub(middle.light[i], lower.light[i]), lower_part_dy);
			d_light_dy_upper[i] = fixed16_div(wsub(upper.light[i], middle.light[i]), upper_part_dy);
		}

		if (long_edge_x_in_middle >= middle.x)
		{
			// the middle vertex is on the left (rasterizer.rs:829-888)
			const Fixed16 middle_dx = std::max(wsub(long_edge_x_in_middle, middle.x), FIXED16_HALF);
			Fixed16 d_tc_dx[2], d_light_dx[3];
			for (int i = 0; i < 2; ++i) d_tc_dx[i] = fixed16_div(wsub(long_edge_tc_in_middle[i], middle.tc[i]), middle_dx);
			for (int i = 0; i < 3; ++i) d_light_dx[i] = fixed16_div(wsub(long_edge_light_in_middle[i], middle.light[i]), middle_dx);
			fill_triangle_part(lower.y, middle.y, PolygonSide{lower.x, lower_part_dx_dy}, PolygonSide{lower.x, long_edge_dx_dy},
				lower.tc, d_tc_dy_lower, d_tc_dx, lower.light, d_light_dy_lower, d_light_dx, tex_w, tex_h, blend);
			fill_triangle_part(middle.y, upper.y, PolygonSide{middle.x, upper_part_dx_dy},
				PolygonSide{long_edge_x_in_middle, long_edge_dx_dy}, middle.tc, d_tc_dy_upper, d_tc_dx, middle.light,
				d_light_dy_upper, d_light_dx, tex_w, tex_h, blend);
		}
		else
		{
			// the middle vertex is on the right (rasterizer.rs:889-950)
			const Fixed16 middle_dx = std::max(wsub(middle.x, long_edge_x_in_middle), FIXED16_HALF);
			Fixed16 d_tc_dx[2], d_light_dx[3];
			for (int i = 0; i < 2; ++i) d_tc_dx[i] = fixed16_div(wsub(middle.tc[i], long_edge_tc_in_middle[i]), middle_dx);
			for (int i = 0; i < 3; ++i) d_light_dx[i] = fixed16_div(wsub(middle.light[i], long_edge_light_in_middle[i]), middle_dx);
			fill_triangle_part(lower.y, middle.y, PolygonSide{lower.x, long_edge_dx_dy}, PolygonSide{lower.x, lower_part_dx_dy},
				lower.tc, long_edge_d_tc_dy, d_tc_dx, lower.light, long_edge_d_light_dy, d_light_dx, tex_w, tex_h, blend);
			fill_triangle_part(middle.y, upper.y, PolygonSide{long_edge_x_in_middle, long_edge_dx_dy},
				PolygonSide{middle.x, upper_part_dx_dy}, long_edge_tc_in_middle, long_edge_d_tc_dy, d_tc_dx,
				long_edge_light_in_middle, long_edge_d_light_dy, d_light_dx, tex_w, tex_h, blend);
		}
	}

	void fill_triangle_part(Fixed16 y_start, Fixed16 y_end, PolygonSide left_side, PolygonSide right_side,
		const Fixed16 tc_start_left[2], const Fixed16 d_tc_dy_left_in[2], const Fixed16 d_tc_dx_in[2],
		const Fixed16 light_start_left[3], const Fixed16 d_light_left_in[3], const Fixed16 d_light_dx_in[3], int32_t tex_w,
		int32_t tex_h, uint32_t blend)
	{
		Fixed16 d_tc_dy_left[2] = {d_tc_dy_left_in[0], d_tc_dy_left_in[1]};
		Fixed16 d_tc_dx[2] = {d_tc_dx_in[0], d_tc_dx_in[1]};
		Fixed16 d_light_left[3] = {d_light_left_in[0], d_light_left_in[1], d_light_left_in[2]};
		Fixed16 d_light_dx[3] = {d_light_dx_in[0], d_light_dx_in[1], d_light_dx_in[2]};
		const int32_t y_start_int = std::max(fixed16_round_to_int(y_start), clip_rect.min_y);
		const int32_t y_end_int = std::min(fixed16_round_to_int(y_end), clip_rect.max_y);
		if (y_start_int >= y_end_int) return;

		const Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
		Fixed16 x_left = wadd(wadd(left_side.x_start, fixed16_mul(y_start_delta, left_side.dx_dy)), FIXED16_HALF);
		Fixed16 x_right = wadd(wadd(right_side.x_start, fixed16_mul(y_start_delta, right_side.dx_dy)), FIXED16_HALF);

		const Fixed16 y_end_delta = wsub(y_end, wadd(y_start, y_start_delta));
		const Fixed16 d_x_lower = std::max(wsub(x_right, x_left), 0);
		const Fixed16 x_upper_left = wadd(x_left, fixed16_mul(y_end_delta, left_side.dx_dy));
		const Fixed16 x_upper_right = wadd(x_right, fixed16_mul(y_end_delta, right_side.dx_dy));
		const Fixed16 d_x_upper = std::max(wsub(x_upper_right, x_upper_left), 0);

		// texture coordinates kept inside the texture (rasterizer.rs:1017-1135)
		Fixed16 tc_left[2] = {0, 0};
		const int32_t tex_size[2] = {tex_w, tex_h};
		for (int i = 0; i < 2; ++i)
		{
			const Fixed16 max_tc = wsub(int_to_fixed16(tex_size[i]), 1);
			{
				tc_left[i] = std::min(std::max(wadd(tc_start_left[i], fixed16_mul(y_start_delta, d_tc_dy_left[i])), 0), max_tc);
				const Fixed16 tc_lower_delta = fixed16_mul(d_tc_dx[i], d_x_lower);
				if (tc_lower_delta > max_tc)
				{
					tc_left[i] = 0;
					d_tc_dx[i] = fixed16_div(max_tc, d_x_lower);
				}
				else if (tc_lower_delta < -max_tc)
				{
					tc_left[i] = max_tc;
					d_tc_dx[i] = fixed16_div(-max_tc, d_x_lower);
				}
				else
				{
					const Fixed16 tc_lower_right = wadd(tc_left[i], tc_lower_delta);
					if (tc_lower_right > max_tc)
						tc_left[i] = wsub(tc_left[i], wsub(tc_lower_right, max_tc));
					else if (tc_lower_right < 0)
						tc_left[i] = wsub(tc_left[i], tc_lower_right);
				}
			}
			{
				Fixed16 tc_upper_left = std::min(std::max(wadd(tc_left[i], fixed16_mul(y_end_delta, d_tc_dy_left[i])), 0), max_tc);
				const Fixed16 tc_upper_delta = fixed16_mul(d_tc_dx[i], d_x_upper);
				if (tc_upper_delta > max_tc)
				{
					tc_upper_left = 0;
					d_tc_dx[i] = fixed16_div(max_tc, d_x_upper);
				}
				else if (tc_upper_delta < -max_tc)
				{
					tc_upper_left = max_tc;
					d_tc_dx[i] = fixed16_div(-max_tc, d_x_upper);
				}
				else
				{
					const Fixed16 tc_upper_right = wadd(tc_upper_left, tc_upper_delta);
					if (tc_upper_right > max_tc)
						tc_upper_left = wsub(tc_upper_left, wsub(tc_upper_right, max_tc));
					else if (tc_upper_right < 0)
						tc_upper_left = wsub(tc_upper_left, tc_upper_right);
				}
				d_tc_dy_left[i] = y_end_delta > 0 ? fixed16_div(wsub(tc_upper_left, tc_left[i]), y_end_delta) : 0;

				const Fixed16 tc_upper_left2 = wadd(tc_left[i], fixed16_mul(y_end_delta, d_tc_dy_left[i]));
				const Fixed16 tc_upper_right = wadd(tc_upper_left2, fixed16_mul(d_tc_dx[i], d_x_upper));
				if (tc_upper_right < 0)
					d_tc_dx[i] = d_x_upper > 0 ? fixed16_div(-tc_upper_left2, d_x_upper) : 0;
				else if (tc_upper_right > max_tc)
					d_tc_dx[i] = d_x_upper > 0 ? fixed16_div(wsub(max_tc, tc_upper_left2), d_x_upper) : 0;
			}
		}

		// light kept non-negative (rasterizer.rs:1137-1186)
		Fixed16 light_left[3] = {0, 0, 0};
		for (int i = 0; i < 3; ++i)
		{
			light_left[i] = std::max(wadd(light_start_left[i], fixed16_mul(y_start_delta, d_light_left[i])), 0);
			const Fixed16 light_lower_right = wadd(light_left[i], fixed16_mul(d_x_lower, d_light_dx[i]));
			if (light_lower_right < 0) light_left[i] = wsub(light_left[i], light_lower_right);
			{
				Fixed16 light_upper_left = std::max(wadd(light_left[i], fixed16_mul(y_end_delta, d_light_left[i])), 0);
				const Fixed16 light_upper_right = wadd(light_upper_left, fixed16_mul(d_x_upper, d_light_dx[i]));
				if (light_upper_right < 0) light_upper_left = wsub(light_upper_left, light_upper_right);
				d_light_left[i] = y_end_delta > 0 ? fixed16_div(wsub(light_upper_left, light_left[i]), y_end_delta) : 0;

				const Fixed16 light_upper_left2 = wadd(light_left[i], fixed16_mul(y_end_delta, d_light_left[i]));
				const Fixed16 light_upper_right2 = wadd(light_upper_left2, fixed16_mul(d_x_upper, d_light_dx[i]));
				if (light_upper_right2 < 0) d_light_dx[i] = d_x_upper > 0 ? fixed16_div(-light_upper_left2, d_x_upper) : 0;
			}
		}

		// ColorVecI::from_color_i32x3: lanes [c2, c1, c0, 0]
		const ColorVecI d_light_dx_vec{{d_light_dx[2], d_light_dx[1], d_light_dx[0], 0}};
		for (int32_t y_int = y_start_int; y_int < y_end_int; ++y_int)
		{
			const int32_t x_start_int = std::max(fixed16_floor_to_int(x_left), clip_rect.min_x);
			const int32_t x_end_int = std::min(fixed16_floor_to_int(x_right), clip_rect.max_x);
			if (x_start_int < x_end_int)
			{
				const Fixed16 x_start_delta = wsub(wadd(int_to_fixed16(x_start_int), FIXED16_ONE), x_left);
				Fixed16 line_tc[2] = {wadd(tc_left[0], fixed16_mul(x_start_delta, d_tc_dx[0])),
					wadd(tc_left[1], fixed16_mul(x_start_delta, d_tc_dx[1]))};
				ColorVecI line_light{{wadd(light_left[2], fixed16_mul(x_start_delta, d_light_dx[2])),
					wadd(light_left[1], fixed16_mul(x_start_delta, d_light_dx[1])),
					wadd(light_left[0], fixed16_mul(x_start_delta, d_light_dx[0])), 0}};
				T* dst_line = color_buffer + int64_t(y_int) * row_size;
				for (int32_t x = x_start_int; x < x_end_int; ++x)
				{
					const int32_t u = fixed16_floor_to_int(line_tc[0]);
					const int32_t v = fixed16_floor_to_int(line_tc[1]);
					const uint64_t texel_address = uint64_t(int64_t(wadd(u, wmul(v, tex_w))));
					const uint32_t texel = fetch_lite(texel_address);
					const ColorVecI lighted = ci_shr(ci_mul(ci_from_c32(texel), line_light), 16);
					T& dst = dst_line[x];
					switch (blend) // rasterizer.rs:1233-1270
					{
					case SW_BLEND_NONE: dst = P::from_veci(lighted); break;
					case SW_BLEND_AVERAGE: dst = P::average(dst, P::from_veci(lighted)); break;
					case SW_BLEND_ADDITIVE: dst = P::saturated_sum(dst, P::from_veci(lighted)); break;
					case SW_BLEND_ALPHA_TEST:
						if (C32::test_alpha(texel)) dst = P::from_veci(lighted);
						break;
					case SW_BLEND_ALPHA_BLEND:
					{
						const int32_t alpha = C32::get_alpha(texel);
						dst = P::from_veci(ci_shr(
							ci_add(ci_mul_scalar(P::to_veci(dst), wsub(255, alpha)), ci_mul_scalar(lighted, alpha)), 8));
						break;
					}
					}
					for (int i = 0; i < 2; ++i) line_tc[i] = wadd(line_tc[i], d_tc_dx[i]);
					line_light = ci_add(line_light, d_light_dx_vec);
				}
			}
			x_left = wadd(x_left, left_side.dx_dy);
			x_right = wadd(x_right, right_side.dx_dy);
			for (int i = 0; i < 2; ++i) tc_left[i] = wadd(tc_left[i], d_tc_dy_left[i]);
			for (int i = 0; i < 3; ++i) light_left[i] = wadd(light_left[i], d_light_left[i]);
		}
	}
};

// rect_splitting.rs:29-78
struct RectF
{
	float min_x, min_y, max_x, max_y;
};
void split_rect_r(const RectF& r, uint32_t num_parts, std::vector<RectF>& out, size_t max_parts)
{
	if (num_parts <= 1)
	{
		if (out.size() < max_parts) out.push_back(r);
		return;
	}
	uint32_t num_parts0 = num_parts / 2;
	uint32_t num_parts1 = num_parts - num_parts0;
	float ratio0 = float(num_parts0) / float(num_parts);
	float ratio1 = float(num_parts1) / float(num_parts);
	RectF r0, r1;
	float width = r.max_x - r.min_x;
	float height = r.max_y - r.min_y;
	if (width >= height)
	{
		float middle = r.max_x * ratio0 + r.min_x * ratio1;
		r0 = RectF{r.min_x, r.min_y, middle, r.max_y};
		r1 = RectF{middle, r.min_y, r.max_x, r.max_y};
	}
	else
	{
		float middle = r.max_y * ratio0 + r.min_y * ratio1;
		r0 = RectF{r.min_x, r.min_y, r.max_x, middle};
		r1 = RectF{r.min_x, middle, r.max_x, r.max_y};
	}
	split_rect_r(r0, num_parts0, out, max_parts);
	split_rect_r(r1, num_parts1, out, max_parts);
}

template <class P>
void rasterize_all(const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices, const SwTriVertex* tri_vertices,
	const void* arena, uint64_t arena_texels, const void* skybox, uint64_t skybox_texels, const uint32_t* lite,
	uint64_t lite_texels, const SwFrameParams* frame, void* framebuffer, uint32_t pitch, uint32_t num_threads,
	uint64_t* bad_fetches)
{
	typedef typename P::T T;
	auto run = [&](ClipRect clip, uint64_t* bad) {
		Raster<P> r;
		r.color_buffer = static_cast<T*>(framebuffer);
		r.row_size = int32_t(pitch);
		r.clip_rect = clip;
		r.bad_fetches = bad;
		for (uint32_t i = 0; i < num_draws; ++i)
		{
			const SwDrawCmd& d = draws[i];
			if (d.mode == SW_RASTER_TRIANGLE)
			{
				// fill_triangle with a TextureLite (Color32) texture
				r.lite = lite + d.tex_offset;
				const uint64_t avail = lite_texels > d.tex_offset ? lite_texels - d.tex_offset : 0;
				const uint64_t want = uint64_t(d.tex_size[0]) * d.tex_size[1];
				r.lite_len = want < avail ? want : avail;
				if (r.lite_len == 0) continue;
				r.fill_triangle(tri_vertices + d.first_vertex, int32_t(d.tex_size[0]), int32_t(d.tex_size[1]), d.blend);
				continue;
			}
			// draw_polygon's texture: a surface, or a skybox side mip (draw_skybox, partial_renderer.rs:2434-2444)
			const bool sky = d.tex_source == SW_TEXSRC_SKYBOX;
			const uint64_t texels = sky ? skybox_texels : arena_texels;
			r.texture_data = static_cast<const T*>(sky ? skybox : arena) + d.tex_offset;
			uint64_t avail = texels > d.tex_offset ? texels - d.tex_offset : 0;
			uint64_t want = uint64_t(d.tex_size[0]) * d.tex_size[1];
			r.texture_len = want < avail ? want : avail;
			if (r.texture_len == 0) continue;
			r.fill_polygon(vertices + d.first_vertex, d.vertex_count, d);
		}
	};
	if (num_threads <= 1)
	{
		run(ClipRect{0, 0, int32_t(frame->width), int32_t(frame->height)}, bad_fetches);
		return;
	}
	std::vector<RectF> rects;
	split_rect_r(RectF{0.0f, 0.0f, float(frame->width), float(frame->height)}, num_threads, rects, 64);
	std::vector<uint64_t> bad(rects.size(), 0);
	std::vector<std::thread> pool;
	for (size_t t = 0; t < rects.size(); ++t)
		pool.emplace_back([&, t]() {
			const RectF& rc = rects[t];
			run(ClipRect{int32_t(rc.min_x), int32_t(rc.min_y), int32_t(rc.max_x), int32_t(rc.max_y)}, &bad[t]);
		});
	for (auto& th : pool) th.join();
	if (bad_fetches)
		for (uint64_t b : bad) *bad_fetches += b;
}

} // namespace
} // namespace sworacle

using namespace sworacle;

extern "C" int orc_rasterize(const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices, const void* arena, uint64_t arena_texels, const void* skybox, uint64_t skybox_texels,
	const SwFrameParams* frame, void* framebuffer, uint32_t pitch, uint32_t num_threads, uint64_t* bad_fetches)
{
	return orc_rasterize_ex(draws, num_draws, vertices, num_vertices, nullptr, 0, arena, arena_texels, skybox, skybox_texels,
		nullptr, 0, frame, framebuffer, pitch, num_threads, bad_fetches);
}

extern "C" int orc_rasterize_ex(const SwDrawCmd* draws, uint32_t num_draws, const SwVertex16* vertices,
	uint32_t num_vertices, const SwTriVertex* tri_vertices, uint32_t num_tri_vertices, const void* arena,
	uint64_t arena_texels, const void* skybox, uint64_t skybox_texels, const uint32_t* lite, uint64_t lite_texels,
	const SwFrameParams* frame, void* framebuffer, uint32_t pitch, uint32_t num_threads, uint64_t* bad_fetches)
{
	if (!frame || !framebuffer || (num_draws && !draws)) return SW_ERR_INVALID_ARGUMENT;
	if (pitch < frame->width) return SW_ERR_INVALID_ARGUMENT;
	for (uint32_t i = 0; i < num_draws; ++i)
	{
		const SwDrawCmd& d = draws[i];
		if (d.mode == SW_RASTER_TRIANGLE)
		{
			if (d.vertex_count != 3 || !tri_vertices || uint64_t(d.first_vertex) + 3 > num_tri_vertices) return SW_ERR_INVALID_ARGUMENT;
			if (d.tex_source != SW_TEXSRC_LITE || !lite || d.blend > SW_BLEND_ALPHA_BLEND) return SW_ERR_INVALID_ARGUMENT;
			if (d.tex_size[0] == 0 || d.tex_size[1] == 0) return SW_ERR_INVALID_ARGUMENT;
			continue;
		}
		if (!vertices || !arena) return SW_ERR_INVALID_ARGUMENT;
		if (d.vertex_count < 3 || d.vertex_count > SW_MAX_POLYGON_VERTICES) return SW_ERR_INVALID_ARGUMENT;
		if (uint64_t(d.first_vertex) + d.vertex_count > num_vertices) return SW_ERR_INVALID_ARGUMENT;
		if (d.mode > SW_RASTER_AFFINE || d.blend > SW_BLEND_ALPHA_BLEND) return SW_ERR_INVALID_ARGUMENT;
		if (d.tex_size[0] == 0 || d.tex_size[1] == 0) return SW_ERR_INVALID_ARGUMENT;
		if (d.tex_source > SW_TEXSRC_SKYBOX || (d.tex_source == SW_TEXSRC_SKYBOX && !skybox)) return SW_ERR_INVALID_ARGUMENT;
	}
	if (frame->pixel_format == SW_PIXEL_C64)
		rasterize_all<C64>(draws, num_draws, vertices, tri_vertices, arena, arena_texels, skybox, skybox_texels, lite,
			lite_texels, frame, framebuffer, pitch, num_threads, bad_fetches);
	else
		rasterize_all<C32>(draws, num_draws, vertices, tri_vertices, arena, arena_texels, skybox, skybox_texels, lite,
			lite_texels, frame, framebuffer, pitch, num_threads, bad_fetches);
	return SW_OK;
}

extern "C" int orc_clear_background(const SwFrameParams* frame, void* framebuffer, uint32_t pitch)
{
	if (!frame || !framebuffer) return SW_ERR_INVALID_ARGUMENT;
	const float c[3] = {32.0f, 16.0f, 8.0f};
	ColorVec v = cv_from_f32x3(c);
	for (uint32_t y = 0; y < frame->height; ++y)
		for (uint32_t x = 0; x < frame->width; ++x)
		{
			if (frame->pixel_format == SW_PIXEL_C64)
				static_cast<uint64_t*>(framebuffer)[uint64_t(y) * pitch + x] = cv_to_c64(v);
			else
				static_cast<uint32_t*>(framebuffer)[uint64_t(y) * pitch + x] = cv_to_c32(v);
		}
	return SW_OK;
}
