// Test infrastructure (oracle): CPU restatement of the reference's shadow-map drawing.
//
// DepthRasterizer::fill_polygon / fill_polygon_part (src/square_wheel/rasterizer.rs:1295-1474): the
// edge walk of the colour rasteriser without texture coordinates, and per row an f32 inverse depth
// accumulated sequentially (line_inv_z += d_inv_z_dy per row, inv_z += d_inv_z_dx per pixel), written
// without a depth test (DepthRenderer draws world polygons back to front, depth_renderer.rs:117-136),
// fixed-point helpers of src/common/fixed_math.rs.
#include "sw_oracle.h"
#include "sw_oracle_math.h"

#include <algorithm>
#include <cmath>

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
inline Fixed16 fixed16_mul(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) * int64_t(y)) >> 16); }
inline Fixed16 fixed16_div(Fixed16 x, Fixed16 y) { return int32_t((int64_t(x) << 16) / int64_t(y)); }
inline Fixed16 fixed16_mul_div(Fixed16 x, Fixed16 y, Fixed16 z) { return int32_t(int64_t(x) * int64_t(y) / int64_t(z)); }

struct DepthRaster
{
	float* depth;
	int32_t width, height;
	const float* eq; // d_inv_z_dx, d_inv_z_dy, k

	// rasterizer.rs:1432-1474
	void fill_part(Fixed16 y_start, Fixed16 y_end, Fixed16 left_x, Fixed16 left_dx_dy, Fixed16 right_x, Fixed16 right_dx_dy)
	{
		const int32_t y_start_int = std::max(fixed16_round_to_int(y_start), 0);
		const int32_t y_end_int = std::min(fixed16_round_to_int(y_end), height);
		const Fixed16 y_start_delta = wsub(wadd(int_to_fixed16(y_start_int), FIXED16_HALF), y_start);
		Fixed16 x_left = wadd(wadd(left_x, fixed16_mul(y_start_delta, left_dx_dy)), FIXED16_HALF);
		Fixed16 x_right = wadd(wadd(right_x, fixed16_mul(y_start_delta, right_dx_dy)), FIXED16_HALF);
		float line_inv_z = (float(y_start_int) * eq[1] + 0.5f * (eq[0] + eq[1])) + eq[2];
		for (int32_t y = y_start_int; y < y_end_int; ++y)
		{
			const int32_t x_start_int = std::max(fixed16_floor_to_int(x_left), 0);
			const int32_t x_end_int = std::min(fixed16_floor_to_int(x_right), width);
			if (x_start_int < x_end_int)
			{
				float* line = depth + int64_t(y) * width;
				float inv_z = line_inv_z + float(x_start_int) * eq[0];
				for (int32_t x = x_start_int; x < x_end_int; ++x)
				{
					line[x] = inv_z;
					inv_z += eq[0];
				}
			}
			x_left = wadd(x_left, left_dx_dy);
			x_right = wadd(x_right, right_dx_dy);
			line_inv_z += eq[1];
		}
	}

	// rasterizer.rs:1317-1430
	void fill_polygon(const SwVertex16* vertices, uint32_t n)
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
			const Fixed16 dy_left = wsub(next_left_vertex.y, left_vertex.y);
			const Fixed16 dy_right = wsub(next_right_vertex.y, right_vertex.y);
			const Fixed16 next_y = std::min(next_left_vertex.y, next_right_vertex.y);
			if (dy_left > FIXED16_HALF && dy_right > FIXED16_HALF)
			{
				const Fixed16 dx_dy_left = fixed16_div(wsub(next_left_vertex.x, left_vertex.x), dy_left);
				const Fixed16 dx_dy_right = fixed16_div(wsub(next_right_vertex.x, right_vertex.x), dy_right);
				fill_part(cur_y, next_y, wadd(left_vertex.x, fixed16_mul(dx_dy_left, wsub(cur_y, left_vertex.y))), dx_dy_left,
					wadd(right_vertex.x, fixed16_mul(dx_dy_right, wsub(cur_y, right_vertex.y))), dx_dy_right);
			}
			else if (dy_left > 0 && dy_right > 0)
			{
				const int32_t cur_y_int = fixed16_round_to_int(cur_y);
				const int32_t next_y_int = fixed16_round_to_int(next_y);
				if (cur_y_int < next_y_int)
				{
					// a single line
					const Fixed16 thin_line_y = wadd(int_to_fixed16(cur_y_int), FIXED16_HALF);
					const Fixed16 x_start_left = wadd(left_vertex.x,
						fixed16_mul_div(wsub(thin_line_y, left_vertex.y), wsub(next_left_vertex.x, left_vertex.x), dy_left));
					const Fixed16 x_start_right = wadd(right_vertex.x,
						fixed16_mul_div(wsub(thin_line_y, right_vertex.y), wsub(next_right_vertex.x, right_vertex.x), dy_right));
					fill_part(cur_y, next_y, x_start_left, 0, x_start_right, 0);
				}
			}
			if (next_left_index == next_right_index) break;
			if (vertices[next_right_index].y < vertices[next_left_index].y)
				right_index = next_right_index;
			else
				left_index = next_left_index;
			cur_y = next_y;
		}
	}
};

} // namespace
} // namespace sworacle

using namespace sworacle;

extern "C" int orc_shadow_maps(const SwDepthDraw* draws, uint32_t num_draws, const SwVertex16* vertices, uint32_t num_vertices,
	float* storage, uint64_t total_texels)
{
	if ((num_draws && (!draws || !vertices)) || (total_texels && !storage)) return SW_ERR_INVALID_ARGUMENT;
	for (uint32_t i = 0; i < num_draws; ++i)
	{
		const SwDepthDraw& d = draws[i];
		if (d.vertex_count < 3 || d.vertex_count > SW_MAX_POLYGON_VERTICES || uint64_t(d.first_vertex) + d.vertex_count > num_vertices)
			return SW_ERR_INVALID_ARGUMENT;
		if (d.map_size == 0 || d.map_offset + uint64_t(d.map_size) * d.map_size > total_texels) return SW_ERR_INVALID_ARGUMENT;
	}
	for (uint32_t i = 0; i < num_draws; ++i)
	{
		const SwDepthDraw& d = draws[i];
		DepthRaster r{storage + d.map_offset, int32_t(d.map_size), int32_t(d.map_size), d.depth_eq};
		r.fill_polygon(vertices + d.first_vertex, d.vertex_count);
	}
	return SW_OK;
}

// make_shadow_map_circle, light.rs:135-156: every texel of a projector map outside the circle inscribed
// in it becomes 1e24 (nothing behind it is lit).
extern "C" int orc_shadow_map_circle(float* storage, uint64_t total_texels, uint64_t offset, uint32_t size)
{
	if (!storage || size == 0 || offset + uint64_t(size) * size > total_texels) return SW_ERR_INVALID_ARGUMENT;
	const float inf = 1.0e24f;
	const int32_t size_signed = int32_t(size);
	const int32_t radius = size_signed / 2;
	for (int32_t y = 0; y < size_signed; ++y)
	{
		const int32_t dy = y - radius;
		const int32_t rr = std::max(radius * radius - dy * dy, 0);
		const int32_t dx = radius - std::min(int32_t(std::ceil(std::sqrt(float(rr)))), radius);
		float* line = storage + offset + uint64_t(y) * size;
		for (int32_t x = 0; x < dx; ++x) line[x] = inf;
		for (int32_t x = size_signed - dx; x < size_signed; ++x) line[x] = inf;
	}
	return SW_OK;
}
