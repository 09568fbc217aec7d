// Test infrastructure: restatement of the reference's lossy lightmap compression
// (src/common/lightmap_compression.rs) for checking the map reader/writer and the GPU decoder.
//
// Rust semantics restated: f32::max / f32::min return the other operand when one is NaN; `as u8` /
// `as i8` truncate toward zero after the explicit clamps (so NaN never reaches the cast: the clamp
// already turned it into the bound's other side); every expression is one IEEE f32 operation.
#include "sw_oracle.h"

#include <cmath>
#include <cstring>

namespace
{

// f32::max, f32::min (NaN-ignoring)
float rs_max(float a, float b)
{
	if (std::isnan(a)) return b;
	if (std::isnan(b)) return a;
	return a > b ? a : b;
}
float rs_min(float a, float b)
{
	if (std::isnan(a)) return b;
	if (std::isnan(b)) return a;
	return a < b ? a : b;
}

// CompressedColor::compress, lightmap_compression.rs:49-62: 255 / scale, scale = clamp(ceil(max), 1, 255)
void color_compress(const float* c, uint8_t* out)
{
	const float m = rs_max(rs_max(c[0], c[1]), c[2]);
	const float scale = rs_min(rs_max(std::ceil(m), 1.0f), 255.0f);
	const float mul = 255.0f / scale;
	for (int i = 0; i < 3; ++i)
	{
		const float v = rs_min(rs_max(c[i] * mul, 0.0f), 255.0f);
		out[i] = static_cast<uint8_t>(static_cast<int>(v));
	}
	out[3] = static_cast<uint8_t>(static_cast<int>(scale));
}

// CompressedColor::decompress, :64-68
void color_decompress(const uint8_t* in, float* out)
{
	const float mul = static_cast<float>(in[3]) / 255.0f;
	for (int i = 0; i < 3; ++i) out[i] = static_cast<float>(in[i]) * mul;
}

// CompressedVector::compress, :73-86
void vector_compress(const float* v, uint8_t* out)
{
	const float m = rs_max(rs_max(std::fabs(v[0]), std::fabs(v[1])), std::fabs(v[2]));
	const float scale = rs_min(rs_max(std::ceil(m), 1.0f), 255.0f);
	const float mul = 127.0f / scale;
	for (int i = 0; i < 3; ++i)
	{
		const float c = rs_min(rs_max(v[i] * mul, -127.0f), 127.0f);
		const int8_t q = static_cast<int8_t>(static_cast<int>(c));
		std::memcpy(out + i, &q, 1);
	}
	out[3] = static_cast<uint8_t>(static_cast<int>(scale));
}

// CompressedVector::decompress, :88-96
void vector_decompress(const uint8_t* in, float* out)
{
	const float mul = static_cast<float>(in[3]) / 127.0f;
	for (int i = 0; i < 3; ++i)
	{
		int8_t q;
		std::memcpy(&q, in + i, 1);
		out[i] = static_cast<float>(q) * mul;
	}
}

} // namespace

extern "C" int orc_compress_lightmaps(const float* rgb, uint64_t n, uint8_t* out)
{
	if (n && (!rgb || !out)) return SW_ERR_INVALID_ARGUMENT;
	for (uint64_t i = 0; i < n; ++i) color_compress(rgb + i * 3, out + i * 4);
	return 0;
}

extern "C" int orc_decompress_lightmaps(const uint8_t* in, uint64_t n, float* rgb)
{
	if (n && (!rgb || !in)) return SW_ERR_INVALID_ARGUMENT;
	for (uint64_t i = 0; i < n; ++i) color_decompress(in + i * 4, rgb + i * 3);
	return 0;
}

// DirectionalLightmapElementCompressed::compress, :101-112 (13 bytes: ambient, direction, deviation, colour)
extern "C" int orc_compress_directional_lightmaps(const SwDirectionalLightmapElement* in, uint64_t n, uint8_t* out)
{
	if (n && (!in || !out)) return SW_ERR_INVALID_ARGUMENT;
	for (uint64_t i = 0; i < n; ++i)
	{
		uint8_t* o = out + i * 13;
		color_compress(in[i].ambient_light, o);
		vector_compress(in[i].light_direction_vector_scaled, o + 4);
		const float d = rs_min(rs_max(in[i].directional_light_deviation * 255.0f, 0.0f), 255.0f);
		o[8] = static_cast<uint8_t>(static_cast<int>(d));
		color_compress(in[i].directional_light_color, o + 9);
	}
	return 0;
}

// DirectionalLightmapElementCompressed::decompress, :114-130 (a zero direction becomes (0, 0, 1/1024))
extern "C" int orc_decompress_directional_lightmaps(const uint8_t* in, uint64_t n, SwDirectionalLightmapElement* out)
{
	if (n && (!in || !out)) return SW_ERR_INVALID_ARGUMENT;
	for (uint64_t i = 0; i < n; ++i)
	{
		const uint8_t* e = in + i * 13;
		SwDirectionalLightmapElement& r = out[i];
		color_decompress(e, r.ambient_light);
		vector_decompress(e + 4, r.light_direction_vector_scaled);
		r.directional_light_deviation = static_cast<float>(e[8]) / 255.0f;
		color_decompress(e + 9, r.directional_light_color);
		const float* v = r.light_direction_vector_scaled;
		const float mag2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
		if (mag2 <= 0.0f)
		{
			r.light_direction_vector_scaled[0] = 0.0f;
			r.light_direction_vector_scaled[1] = 0.0f;
			r.light_direction_vector_scaled[2] = 1.0f / 1024.0f;
		}
	}
	return 0;
}
