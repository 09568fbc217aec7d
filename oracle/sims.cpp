// Test infrastructure: restatement of the simulated generative texture effects on the CPU, whole and in
// the reference's data flow (src/square_wheel/generative_texture_effect_water.rs:1-690,
// generative_texture_effect_fire.rs:1-566, generative_texture_effects_common.rs, textures.rs:164-181 and
// 309-415, src/common/material_function.rs:88-150), with rand 0.8.5's SmallRng (xoshiro256++ seeded by
// rand_core 0.6's default seed_from_u64) and its inclusive uniform samplers restated from their published
// algorithms. The wave fields swap after each step and the heat map is updated in place, row by row, as
// the reference does; the effect's output texture mips are written into the caller's texel / emissive
// arrays at the effect's output slot.
#include "sw_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace
{

constexpr float TAU = 6.28318530717958647692f;
constexpr uint32_t NUM_MIPS = 5;

int32_t f2i(float f) // `as i32`
{
	if (std::isnan(f)) return 0;
	if (f >= 2147483648.0f) return 2147483647;
	if (f < -2147483648.0f) return -2147483647 - 1;
	return static_cast<int32_t>(f);
}
uint8_t f2u8(float f) // `as u8`
{
	if (std::isnan(f) || f <= 0.0f) return 0;
	if (f >= 255.0f) return 255;
	return static_cast<uint8_t>(f);
}
float rmax(float a, float b) { return std::isnan(a) ? b : (std::isnan(b) ? a : (a > b ? a : b)); } // f32::max
float rmin(float a, float b) { return std::isnan(a) ? b : (std::isnan(b) ? a : (a < b ? a : b)); } // f32::min
int32_t add_w(int32_t a, int32_t b) { return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b)); }
int32_t sub_w(int32_t a, int32_t b) { return static_cast<int32_t>(static_cast<uint32_t>(a) - static_cast<uint32_t>(b)); }
int32_t to_fixed16(int32_t x) { return static_cast<int32_t>(static_cast<uint32_t>(x) << 16); }
int32_t fixed16_round(int32_t x) { return add_w(x, 1 << 15) >> 16; }
float bits_to_f32(uint32_t b)
{
	float f;
	std::memcpy(&f, &b, 4);
	return f;
}
uint32_t f32_to_bits(float f)
{
	uint32_t b;
	std::memcpy(&b, &f, 4);
	return b;
}

// SingleArgumentFunction::evaluate (material_function.rs:91-150)
float evaluate(const OrcTimeFunction& f, float x)
{
	switch (f.kind)
	{
	case 0: return f.a;
	case 1: return x * f.a + f.b;
	case 2: return std::sin(x * f.a * TAU + f.b) * f.c + f.d;
	default:
	{
		const float arg = x * f.a + f.b;
		const float fr = arg - std::floor(arg);
		float wave;
		if (f.kind == 3) wave = fr <= 0.25f ? 4.0f * fr : (fr <= 0.75f ? 2.0f - 4.0f * fr : -4.0f + 4.0f * fr);
		else if (f.kind == 4) wave = fr * 2.0f - 1.0f;
		else wave = fr <= 0.5f ? 1.0f : -1.0f;
		return wave * f.c + f.d;
	}
	}
}

// SmallRng: xoshiro256++ 1.0 with rand_core 0.6's PCG32-filled seed
struct Rand
{
	uint64_t s[4];
	explicit Rand(uint64_t seed)
	{
		uint32_t words[8];
		uint64_t st = seed;
		for (uint32_t& w : words)
		{
			st = st * 6364136223846793005ull + 11634580027462260723ull;
			const uint32_t xs = static_cast<uint32_t>(((st >> 18) ^ st) >> 27);
			const uint32_t rot = static_cast<uint32_t>(st >> 59);
			w = rot ? ((xs >> rot) | (xs << (32 - rot))) : xs;
		}
		for (int i = 0; i < 4; ++i) s[i] = uint64_t(words[2 * i]) | (uint64_t(words[2 * i + 1]) << 32);
		if ((s[0] | s[1] | s[2] | s[3]) == 0)
		{
			uint64_t x = 0;
			for (uint64_t& v : s)
			{
				x += 0x9e3779b97f4a7c15ull;
				uint64_t z = x;
				z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
				z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
				v = z ^ (z >> 31);
			}
		}
	}
	static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
	uint64_t next64()
	{
		const uint64_t out = rotl(s[0] + s[3], 23) + s[0];
		const uint64_t t = s[1] << 17;
		s[2] ^= s[0];
		s[3] ^= s[1];
		s[1] ^= s[2];
		s[0] ^= s[3];
		s[2] ^= t;
		s[3] = rotl(s[3], 45);
		return out;
	}
	uint32_t next32() { return static_cast<uint32_t>(next64() >> 32); }
	float uniform_inclusive(float low, float high) // UniformFloat::new_inclusive + UniformSampler::sample
	{
		const float max_rand = bits_to_f32(0x3F800000u | 0x7FFFFFu) - 1.0f;
		float scale = (high - low) / max_rand;
		while (std::isfinite(scale) && scale * max_rand + low > high) scale = bits_to_f32(f32_to_bits(scale) - 1u);
		const float v = bits_to_f32((next32() >> 9) | 0x3F800000u) - 1.0f;
		return v * scale + low;
	}
	int32_t uniform_inclusive(int32_t low, int32_t high) // UniformInt::sample_single_inclusive
	{
		const uint32_t range = static_cast<uint32_t>(sub_w(high, low)) + 1u;
		if (range == 0) return static_cast<int32_t>(next32());
		int lz = 0;
		while (!((range << lz) & 0x80000000u)) ++lz;
		const uint32_t zone = (range << lz) - 1u;
		while (true)
		{
			const uint64_t prod = static_cast<uint64_t>(next32()) * range;
			if (static_cast<uint32_t>(prod) <= zone) return add_w(low, static_cast<int32_t>(prod >> 32));
		}
	}
};
constexpr uint64_t RAND_SEED = 0b1001100000111010100101010101010111000111010110100101111001010101ull;

// ---- textures --------------------------------------------------------------------------------

uint32_t average_4(const uint32_t c[4]) // Color32::get_average_4
{
	uint32_t r = 0, g = 0, b = 0, a = 0;
	for (int i = 0; i < 4; ++i)
	{
		b += c[i] & 0xFFu;
		g += c[i] & 0xFF00u;
		r += c[i] & 0xFF0000u;
		a += (c[i] & 0xFF000000u) >> 2;
	}
	return (b >> 2) | ((g >> 2) & 0xFF00u) | ((r >> 2) & 0xFF0000u) | (a & 0xFF000000u);
}
uint32_t pack_normal(float x, float y, float z, float roughness) // PackedNormalRoughness::pack
{
	const float v[4] = {x, y, z, roughness};
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i) r |= (static_cast<uint32_t>(f2i(rmin(rmax(v[i] * 127.0f, -127.0f), 127.0f))) & 0xFFu) << (8 * i);
	return r;
}
void unpack_normal(uint32_t p, float out[4])
{
	const float scale[4] = {1.0f / 127.0f, 1.0f / 127.0f, 1.0f / 127.0f, 1.0f / 127.0f};
	for (int i = 0; i < 4; ++i) out[i] = static_cast<float>(static_cast<int32_t>(p << (24 - 8 * i)) >> 24) * scale[i];
}

struct Mip
{
	uint32_t w = 0, h = 0;
	std::vector<uint64_t> px; // TextureElement
};

void build_texture_mip(Mip& mip, const Mip& prev) // textures.rs:309-362
{
	mip.w = prev.w >> 1;
	mip.h = prev.h >> 1;
	mip.px.assign(size_t(mip.w) * mip.h, 0);
	for (uint32_t y = 0; y < mip.h; ++y)
		for (uint32_t x = 0; x < mip.w; ++x)
		{
			const uint64_t p00 = prev.px[size_t(2 * y) * prev.w + 2 * x], p01 = prev.px[size_t(2 * y + 1) * prev.w + 2 * x];
			const uint64_t p10 = prev.px[size_t(2 * y) * prev.w + 2 * x + 1], p11 = prev.px[size_t(2 * y + 1) * prev.w + 2 * x + 1];
			const uint32_t d[4] = {uint32_t(p00), uint32_t(p01), uint32_t(p10), uint32_t(p11)};
			float n[4][4];
			unpack_normal(uint32_t(p00 >> 32), n[0]);
			unpack_normal(uint32_t(p01 >> 32), n[1]);
			unpack_normal(uint32_t(p10 >> 32), n[2]);
			unpack_normal(uint32_t(p11 >> 32), n[3]);
			float sum[3];
			for (int c = 0; c < 3; ++c) sum[c] = n[0][c] + n[1][c] + n[2][c] + n[3][c];
			const float len = rmax(std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]), 0.000001f);
			const float deviation = (1.0f - len * 0.25f) / (1.0f - 0.5f);
			const float rough_sum = n[0][3] + n[1][3] + n[2][3] + n[3][3];
			const float rough = rmin(rmax(rough_sum * 0.25f + deviation, 1.0f / (127.0f - 1.0f)), 1.0f);
			mip.px[size_t(y) * mip.w + x] =
				uint64_t(average_4(d)) | (uint64_t(pack_normal(sum[0] / len, sum[1] / len, sum[2] / len, rough)) << 32);
		}
}

// ---- the effect -----------------------------------------------------------------------------

struct Particle
{
	float vx, vy, px, py;
	uint32_t despawn_time;
	float gravity;
	uint8_t heat;
};

struct Sim
{
	OrcSimEffect cfg;
	bool water;
	float update_frequency;
	uint32_t update_step = 0;
	float prev_update_time_s = 0.0f;
	Rand rand{RAND_SEED};
	// water
	std::vector<float> wave_field, wave_field_old;
	std::vector<uint32_t> color_image;
	// fire
	std::vector<uint8_t> heat_map;
	uint32_t palette[256];
	std::vector<Particle> particles;
	std::vector<int32_t> rand_buffer;
	// the generated texture (water: TextureElement mips; fire: Color32 mips)
	Mip tex[NUM_MIPS];
	std::vector<uint32_t> emissive[NUM_MIPS];
	bool generated = false;

	uint32_t w() const { return 1u << cfg.resolution_log2[0]; }
	uint32_t h() const { return 1u << cfg.resolution_log2[1]; }

	void water_step()
	{
		++update_step;
		const uint32_t mask[2] = {w() - 1, h() - 1};
		const uint32_t v_shift = cfg.resolution_log2[0];
		const float time_s = static_cast<float>(update_step) / update_frequency;
		auto add_point_value = [&](uint32_t x, uint32_t y, float value) {
			const size_t address = (x & mask[0]) + ((y & mask[1]) << v_shift);
			wave_field[address] += value;
			wave_field_old[address] -= value;
		};
		for (uint32_t si = 0; si < cfg.num_sources; ++si)
		{
			const OrcSimSource& s = cfg.sources[si];
			if (s.kind == 0) // WavySpot
			{
				const float field_value = std::sin(time_s * s.frequency * TAU + s.phase) * s.amplitude * s.frequency + s.offset;
				add_point_value(static_cast<uint32_t>(f2i(static_cast<float>(s.points[0][0]) + evaluate(s.offsets[0][0], time_s))),
					static_cast<uint32_t>(f2i(static_cast<float>(s.points[0][1]) + evaluate(s.offsets[0][1], time_s))), field_value);
			}
			else if (s.kind == 1) // WavyLine
			{
				int32_t pts[2][2];
				for (int i = 0; i < 2; ++i)
					for (int j = 0; j < 2; ++j) pts[i][j] = f2i(static_cast<float>(s.points[i][j]) + evaluate(s.offsets[i][j], time_s));
				const float field_value = std::sin(time_s * s.frequency * TAU + s.phase) * s.amplitude * s.frequency + s.offset;
				const int32_t abs_dx = std::abs(pts[0][0] - pts[1][0]), abs_dy = std::abs(pts[0][1] - pts[1][1]);
				if (abs_dx == 0 && abs_dy == 0)
					add_point_value(static_cast<uint32_t>(pts[0][0]), static_cast<uint32_t>(pts[0][1]), field_value);
				else if (abs_dx >= abs_dy)
				{
					if (pts[0][0] > pts[1][0]) std::swap(pts[0], pts[1]);
					const int32_t y_step = to_fixed16(pts[1][1] - pts[0][1]) / abs_dx;
					int32_t y_fract = to_fixed16(pts[0][1]);
					for (int32_t x_offset = 0; x_offset <= abs_dx; ++x_offset)
					{
						const int32_t x = pts[0][0] + x_offset;
						const int32_t y = fixed16_round(y_fract);
						y_fract = add_w(y_fract, y_step);
						add_point_value(static_cast<uint32_t>(x), static_cast<uint32_t>(y), field_value);
					}
				}
				else
				{
					if (pts[0][1] > pts[1][1]) std::swap(pts[0], pts[1]);
					const int32_t x_step = to_fixed16(pts[1][0] - pts[0][0]) / abs_dy;
					int32_t x_fract = to_fixed16(pts[0][0]);
					for (int32_t y_offset = 1; y_offset <= abs_dy; ++y_offset)
					{
						const int32_t y = pts[0][1] + y_offset;
						const int32_t x = fixed16_round(x_fract);
						x_fract = add_w(x_fract, x_step);
						add_point_value(static_cast<uint32_t>(x), static_cast<uint32_t>(y), field_value);
					}
				}
			}
			else if (s.kind == 2) // PeriodicDroplet
			{
				const float relative_frequency = s.frequency / update_frequency;
				const int32_t begin = f2i(static_cast<float>(update_step) * relative_frequency + s.phase);
				const int32_t end = f2i(static_cast<float>(update_step + 1) * relative_frequency + s.phase);
				if (begin < end)
				{
					const uint32_t x = static_cast<uint32_t>(f2i(static_cast<float>(s.points[0][0]) + evaluate(s.offsets[0][0], time_s)));
					const uint32_t y = static_cast<uint32_t>(f2i(static_cast<float>(s.points[0][1]) + evaluate(s.offsets[0][1], time_s)));
					for (int32_t i = begin; i < end; ++i) add_point_value(x, y, s.amplitude);
				}
			}
			else // Rain
			{
				if (rand.uniform_inclusive(0.0f, 1.0f) <= s.frequency / update_frequency)
				{
					uint32_t x, y;
					if (s.radius > 0.0f)
					{
						const float dist = rand.uniform_inclusive(0.0f, s.radius);
						const float angle = rand.uniform_inclusive(0.0f, TAU);
						const float dx = std::cos(angle) * dist, dy = std::sin(angle) * dist;
						x = static_cast<uint32_t>(add_w(static_cast<int32_t>(s.points[0][0]), f2i(dx)));
						y = static_cast<uint32_t>(add_w(static_cast<int32_t>(s.points[0][1]), f2i(dy)));
					}
					else
					{
						x = rand.next32();
						y = rand.next32();
					}
					add_point_value(x, y, s.amplitude);
				}
			}
		}
		const float attenuation = 1.0f - 1.0f / rmin(rmax(cfg.attenuation_param, 10.0f), 1000000.0f);
		update_wave_field(attenuation);
		std::swap(wave_field, wave_field_old);
	}

	// update_wave_field (water.rs:308-418): dst = old field, src = field, both edges wrapping
	void update_wave_field(float attenuation)
	{
		const uint32_t W = w(), H = h();
		std::vector<float>& dst = wave_field_old;
		const std::vector<float>& src = wave_field;
		for (uint32_t y = 0; y < H; ++y)
			for (uint32_t x = 0; x < W; ++x)
			{
				const size_t o = size_t(y) * W + x;
				const float sum = src[size_t(y) * W + (x + W - 1) % W] + src[size_t(y) * W + (x + 1) % W] +
					src[size_t((y + H - 1) % H) * W + x] + src[size_t((y + 1) % H) * W + x];
				dst[o] = (sum * 0.5f - dst[o]) * attenuation;
			}
	}

	float random_value(const OrcRandomValue& v, float time_s) // get_value_with_random_deviation
	{
		const float value = evaluate(v.value, time_s);
		const float deviation = evaluate(v.deviation, time_s);
		return value - deviation + rand.uniform_inclusive(0.0f, rmax(deviation, 0.0f) * 2.0f);
	}
	static uint8_t convert_heat(float heat) { return f2u8(rmin(rmax(heat * 255.0f, 0.0f), 255.0f)); }

	void fire_step()
	{
		++update_step;
		const float time_s = static_cast<float>(update_step) / update_frequency;
		const float attenuation = 1.0f - 1.0f / rmin(rmax(cfg.attenuation_param, 1.0f), 1000000.0f);
		update_heat_map(attenuation);
		const uint32_t mask[2] = {w() - 1, h() - 1};
		const uint32_t v_shift = cfg.resolution_log2[0];
		auto set_heat = [&](uint32_t x, uint32_t y, uint8_t heat) {
			uint8_t& v = heat_map[(x & mask[0]) + ((y & mask[1]) << v_shift)];
			v = std::max(v, heat);
		};
		for (uint32_t si = 0; si < cfg.num_sources; ++si)
		{
			const OrcSimSource& s = cfg.sources[si];
			if (s.kind == 0) // Point
			{
				const float offset_x = random_value(s.fire_offsets[0][0], time_s);
				const float offset_y = random_value(s.fire_offsets[0][1], time_s);
				const uint32_t x = static_cast<uint32_t>(f2i(std::floor(static_cast<float>(s.points[0][0]) + offset_x)));
				const uint32_t y = static_cast<uint32_t>(f2i(std::floor(static_cast<float>(s.points[0][1]) + offset_y)));
				set_heat(x, y, convert_heat(random_value(s.heat, time_s)));
			}
			else if (s.kind == 1) // Line
			{
				const uint8_t heat = convert_heat(random_value(s.heat, time_s));
				uint32_t pts[2][2] = {{s.points[0][0], s.points[0][1]}, {s.points[1][0], s.points[1][1]}};
				const int32_t abs_dx = std::abs(static_cast<int32_t>(pts[0][0]) - static_cast<int32_t>(pts[1][0]));
				const int32_t abs_dy = std::abs(static_cast<int32_t>(pts[0][1]) - static_cast<int32_t>(pts[1][1]));
				if (abs_dx >= abs_dy)
				{
					if (pts[0][0] > pts[1][0]) std::swap(pts[0], pts[1]);
					if (abs_dx == 0) // the reference divides by zero here
					{
						set_heat(pts[0][0], pts[0][1], heat);
						continue;
					}
					const int32_t y_step = to_fixed16(static_cast<int32_t>(pts[1][1]) - static_cast<int32_t>(pts[0][1])) / abs_dx;
					int32_t y_fract = to_fixed16(static_cast<int32_t>(pts[0][1]));
					for (int32_t x_offset = 0; x_offset <= abs_dx; ++x_offset)
					{
						const int32_t x = static_cast<int32_t>(pts[0][0]) + x_offset;
						const int32_t y = fixed16_round(y_fract);
						y_fract = add_w(y_fract, y_step);
						set_heat(static_cast<uint32_t>(x), static_cast<uint32_t>(y), heat);
					}
				}
				else
				{
					if (pts[0][1] > pts[1][1]) std::swap(pts[0], pts[1]);
					const int32_t x_step = to_fixed16(static_cast<int32_t>(pts[1][0]) - static_cast<int32_t>(pts[0][0])) / abs_dy;
					int32_t x_fract = to_fixed16(static_cast<int32_t>(pts[0][0]));
					for (int32_t y_offset = 1; y_offset <= abs_dy; ++y_offset)
					{
						const int32_t y = static_cast<int32_t>(pts[0][1]) + y_offset;
						const int32_t x = fixed16_round(x_fract);
						x_fract = add_w(x_fract, x_step);
						set_heat(static_cast<uint32_t>(x), static_cast<uint32_t>(y), heat);
					}
				}
			}
			else if (s.kind == 2) // Lightning
			{
				const uint8_t heat = convert_heat(random_value(s.heat, time_s));
				const int32_t head_fract = to_fixed16(static_cast<int32_t>(heat));
				int32_t heat_start = head_fract, heat_end = s.ramp ? 0 : head_fract;
				int32_t pts[2][2] = {{static_cast<int32_t>(s.points[0][0]), static_cast<int32_t>(s.points[0][1])},
					{static_cast<int32_t>(s.points[1][0]), static_cast<int32_t>(s.points[1][1])}};
				for (int i = 0; i < 2; ++i)
					for (int j = 0; j < 2; ++j) pts[i][j] = add_w(pts[i][j], f2i(random_value(s.fire_offsets[i][j], time_s)));
				const int32_t abs_dx = std::abs(pts[0][0] - pts[1][0]), abs_dy = std::abs(pts[0][1] - pts[1][1]);
				const int32_t max_delta = std::max(abs_dx, abs_dy);
				rand_buffer.resize(static_cast<size_t>(max_delta + 1), 0);
				int32_t rand_offset = 0;
				for (int32_t& rv : rand_buffer)
				{
					rv = add_w(rand_offset, rand.uniform_inclusive(-65536, 65536));
					rand_offset = rv;
				}
				if (max_delta == 0)
					set_heat(static_cast<uint32_t>(pts[0][0]), static_cast<uint32_t>(pts[0][1]), heat);
				else if (abs_dx >= abs_dy)
				{
					if (pts[0][0] > pts[1][0])
					{
						std::swap(pts[0], pts[1]);
						std::swap(heat_start, heat_end);
					}
					const int32_t y_step = sub_w(to_fixed16(pts[1][1] - pts[0][1]), rand_offset) / abs_dx;
					int32_t y_fract = to_fixed16(pts[0][1]);
					const int32_t heat_step = (heat_end - heat_start) / abs_dx;
					int32_t heat_cur = heat_start;
					for (int32_t x_offset = 0; x_offset <= abs_dx; ++x_offset)
					{
						const int32_t x = pts[0][0] + x_offset;
						const int32_t y = fixed16_round(add_w(y_fract, rand_buffer[static_cast<size_t>(x_offset)]));
						set_heat(static_cast<uint32_t>(x), static_cast<uint32_t>(y), static_cast<uint8_t>(heat_cur >> 16));
						y_fract = add_w(y_fract, y_step);
						heat_cur = add_w(heat_cur, heat_step);
					}
				}
				else
				{
					if (pts[0][1] > pts[1][1])
					{
						std::swap(pts[0], pts[1]);
						std::swap(heat_start, heat_end);
					}
					const int32_t x_step = sub_w(to_fixed16(pts[1][0] - pts[0][0]), rand_offset) / abs_dy;
					int32_t x_fract = to_fixed16(pts[0][0]);
					const int32_t heat_step = (heat_end - heat_start) / abs_dy;
					int32_t heat_cur = heat_start;
					for (int32_t y_offset = 0; y_offset <= abs_dy; ++y_offset)
					{
						const int32_t y = pts[0][1] + y_offset;
						const int32_t x = fixed16_round(add_w(x_fract, rand_buffer[static_cast<size_t>(y_offset)]));
						set_heat(static_cast<uint32_t>(x), static_cast<uint32_t>(y), static_cast<uint8_t>(heat_cur >> 16));
						x_fract = add_w(x_fract, x_step);
						heat_cur = add_w(heat_cur, heat_step);
					}
				}
			}
			else // Fountain
			{
				const float relative_frequency = s.frequency / update_frequency;
				const int32_t begin = f2i(static_cast<float>(update_step) * relative_frequency);
				const int32_t end = f2i(static_cast<float>(update_step + 1) * relative_frequency);
				for (int32_t i = begin; i < end; ++i)
				{
					if (particles.size() >= 256) continue;
					const float heat = random_value(s.heat, time_s);
					const float angle = random_value(s.angle, time_s);
					const float speed = random_value(s.speed, time_s);
					const float gravity = random_value(s.gravity, time_s);
					const float spawn_angle = random_value(s.spawn_angle, time_s);
					const float spawn_distance = random_value(s.spawn_distance, time_s);
					const float lifetime = random_value(s.lifetime, time_s);
					Particle p;
					const float vscale = speed / update_frequency;
					p.vx = std::cos(angle) * vscale;
					p.vy = std::sin(angle) * vscale;
					const float sx = std::cos(spawn_angle) * spawn_distance, sy = std::sin(spawn_angle) * spawn_distance;
					const uint32_t life = static_cast<uint32_t>(rmin(rmax(lifetime * update_frequency, 1.0f), 1024.0f));
					p.px = static_cast<float>(s.points[0][0]) + sx;
					p.py = static_cast<float>(s.points[0][1]) + sy;
					p.despawn_time = update_step + life;
					p.gravity = gravity / (update_frequency * update_frequency);
					p.heat = convert_heat(heat);
					particles.push_back(p);
				}
			}
		}
		size_t i = 0;
		while (i < particles.size())
		{
			Particle& p = particles[i];
			if (p.despawn_time <= update_step)
			{
				std::swap(particles[i], particles.back()); // swap_remove
				particles.pop_back();
				continue;
			}
			p.vy += p.gravity;
			p.px += p.vx;
			p.py += p.vy;
			set_heat(static_cast<uint32_t>(f2i(std::floor(p.px))), static_cast<uint32_t>(f2i(std::floor(p.py))), p.heat);
			++i;
		}
	}

	// update_heat_map (fire.rs:430-550), in place, rows top to bottom
	void update_heat_map(float attenuation)
	{
		const uint32_t W = w(), H = h();
		const uint32_t att = static_cast<uint32_t>(rmin(rmax(attenuation, 0.0f), 1.0f) * static_cast<float>(1 << 18));
		auto upd = [&](size_t o, size_t a, size_t b, size_t c, size_t d) {
			const uint32_t sum = uint32_t(heat_map[a]) + uint32_t(heat_map[b]) + uint32_t(heat_map[c]) + uint32_t(heat_map[d]);
			heat_map[o] = static_cast<uint8_t>((sum * att) >> 20);
		};
		if (cfg.slow)
			for (uint32_t y = 0; y + 1 < H; ++y)
			{
				const size_t s = size_t(y) * W, e = s + W - 1;
				upd(s, e, s, s + 1, s + W);
				for (size_t x = s + 1; x < e; ++x) upd(x, x - 1, x, x + 1, x + W);
				upd(e, e - 1, e, s, e + W);
			}
		else
		{
			for (uint32_t y = 0; y + 2 < H; ++y)
			{
				const size_t s = size_t(y) * W, e = s + W - 1;
				upd(s, e + W, s + W, s + 1 + W, s + 2 * W);
				for (size_t x = s + 1; x < e; ++x) upd(x, x - 1 + W, x + W, x + 1 + W, x + 2 * W);
				upd(e, e - 1 + W, e + W, s + W, e + 2 * W);
			}
			const size_t s = size_t(H - 2) * W, e = s + W - 1;
			upd(s, e + W, s + W, s + 1 + W, s + W);
			for (size_t x = s + 1; x < e; ++x) upd(x, x - 1 + W, x + W, x + 1 + W, x + W);
			upd(e, e - 1 + W, e + W, s + W, e + W);
		}
		std::fill(heat_map.begin() + size_t(H - 1) * W, heat_map.end(), uint8_t(0));
	}

	bool update(float current_time_s, const uint64_t* texels, const SwTextureMip* mips, uint32_t source_texture,
		const uint32_t* emissive_pixels, const SwEmissiveMip* emips)
	{
		const int32_t steps = std::min(std::max(sub_w(f2i(current_time_s * update_frequency), f2i(prev_update_time_s * update_frequency)), 0), 10);
		prev_update_time_s = current_time_s;
		if (steps == 0) return false;
		for (int32_t i = 0; i < steps; ++i)
		{
			if (water) water_step();
			else fire_step();
		}
		const uint32_t W = w(), H = h();
		if (water)
		{
			const SwTextureMip& src0 = mips[source_texture * NUM_MIPS];
			if (cfg.color_mode != 0 && color_image.empty())
			{
				// extract_color_image_from_texture + resize_image (textures.rs:164-181) when the sizes differ
				color_image.resize(size_t(W) * H);
				for (uint32_t y = 0; y < H; ++y)
					for (uint32_t x = 0; x < W; ++x)
					{
						const uint32_t sx = (src0.width == W) ? x : x * src0.width / W;
						const uint32_t sy = (src0.height == H) ? y : y * src0.height / H;
						color_image[size_t(y) * W + x] = uint32_t(texels[src0.offset + uint64_t(sy) * src0.width + sx]);
					}
			}
			const uint32_t base_color = uint32_t(texels[mips[source_texture * NUM_MIPS + NUM_MIPS - 1].offset]);
			const float roughness = rmin(rmax(cfg.roughness, 1.0f / (127.0f - 1.0f)), 1.0f);
			Mip& t = tex[0];
			if (t.px.empty())
			{
				t.w = W;
				t.h = H;
				t.px.assign(size_t(W) * H, 0);
				if (cfg.color_mode == 0)
					for (uint64_t& p : t.px) p = base_color;
				if (cfg.color_mode == 1)
					for (size_t i = 0; i < t.px.size(); ++i) t.px[i] = color_image[i];
			}
			// make_wavy_texture_impl (water.rs:497-682)
			for (uint32_t y = 0; y < H; ++y)
				for (uint32_t x = 0; x < W; ++x)
				{
					const float vxm = wave_field[size_t(y) * W + (x + W - 1) % W], vxp = wave_field[size_t(y) * W + (x + 1) % W];
					const float vym = wave_field[size_t((y + H - 1) % H) * W + x], vyp = wave_field[size_t((y + 1) % H) * W + x];
					const float dx = vxp - vxm, dy = vyp - vym;
					const float inv_len = 1.0f / std::sqrt(dx * dx + dy * dy + 1.0f * 1.0f);
					const float nx = dx * inv_len, ny = dy * inv_len, nz = 1.0f * inv_len;
					uint64_t& texel = t.px[size_t(y) * W + x];
					uint32_t diffuse = uint32_t(texel);
					if (cfg.color_mode == 2 || cfg.color_mode == 3)
					{
						const uint32_t u = static_cast<uint32_t>(static_cast<int32_t>(x) + f2i(nx * 16.0f)) & (W - 1);
						const uint32_t v = cfg.color_mode == 2 ? static_cast<uint32_t>(static_cast<int32_t>(y) + f2i(ny * 16.0f)) & (H - 1) : y;
						diffuse = color_image[size_t(v) * W + u];
					}
					texel = uint64_t(diffuse) | (uint64_t(pack_normal(nx, ny, nz, roughness)) << 32);
				}
			for (uint32_t m = 1; m < NUM_MIPS; ++m) build_texture_mip(tex[m], tex[m - 1]);
		}
		else
		{
			if (emissive[0].empty())
			{
				if (cfg.has_color)
					for (uint32_t i = 0; i < 256; ++i)
					{
						const float scale = static_cast<float>(i);
						palette[i] = (uint32_t(f2u8(rmin(rmax(cfg.color[0] * scale, 0.0f), 255.0f))) << 16) |
							(uint32_t(f2u8(rmin(rmax(cfg.color[1] * scale, 0.0f), 255.0f))) << 8) |
							uint32_t(f2u8(rmin(rmax(cfg.color[2] * scale, 0.0f), 255.0f)));
					}
				else if (cfg.source_emissive >= 0)
				{
					const SwEmissiveMip& e0 = emips[uint32_t(cfg.source_emissive) * NUM_MIPS];
					if (e0.width * e0.height != 0)
						for (uint32_t i = 0; i < 256; ++i) palette[i] = emissive_pixels[e0.offset + ((i * e0.width) >> 8)];
				}
			}
			emissive[0].resize(size_t(W) * H);
			for (size_t i = 0; i < emissive[0].size(); ++i) emissive[0][i] = palette[heat_map[i]];
			for (uint32_t m = 1; m < NUM_MIPS; ++m)
			{
				const uint32_t pw = W >> (m - 1), mw = W >> m, mh = H >> m;
				emissive[m].resize(size_t(mw) * mh);
				for (uint32_t y = 0; y < mh; ++y)
					for (uint32_t x = 0; x < mw; ++x)
					{
						const std::vector<uint32_t>& p = emissive[m - 1];
						const uint32_t c[4] = {p[size_t(2 * y) * pw + 2 * x], p[size_t(2 * y + 1) * pw + 2 * x],
							p[size_t(2 * y) * pw + 2 * x + 1], p[size_t(2 * y + 1) * pw + 2 * x + 1]};
						emissive[m][size_t(y) * mw + x] = average_4(c);
					}
			}
		}
		generated = true;
		return true;
	}
};

} // namespace

extern "C" uint32_t orc_sim_effect_size(void) { return uint32_t(sizeof(OrcSimEffect)); }

extern "C" void* orc_sim_create(const OrcSimEffect* cfg)
{
	if (!cfg || (cfg->kind != 3 && cfg->kind != 4) || cfg->num_sources > ORC_MAX_SIM_SOURCES ||
		cfg->resolution_log2[0] < 4 || cfg->resolution_log2[1] < 4 || cfg->resolution_log2[0] + cfg->resolution_log2[1] >= 22)
		return nullptr;
	Sim* s = new (std::nothrow) Sim();
	if (!s) return nullptr;
	s->cfg = *cfg;
	s->water = cfg->kind == 3;
	s->update_frequency = rmin(rmax(cfg->update_frequency, 1.0f), 200.0f);
	const size_t area = size_t(1) << (cfg->resolution_log2[0] + cfg->resolution_log2[1]);
	if (s->water)
	{
		s->wave_field.assign(area, 0.0f);
		s->wave_field_old.assign(area, 0.0f);
		const float diagonal_len = std::sqrt(static_cast<float>((1 << (cfg->resolution_log2[0] * 2)) + (1 << (cfg->resolution_log2[1] * 2))));
		const int32_t num_steps = std::min(f2i(diagonal_len), 512);
		for (int32_t i = 0; i < num_steps; ++i) s->water_step();
	}
	else
	{
		s->heat_map.assign(area, 0);
		for (uint32_t i = 0; i < 256; ++i) s->palette[i] = (i << 16) | (i << 8) | i;
		for (int i = 0; i < 16; ++i) s->fire_step();
	}
	return s;
}

extern "C" void orc_sim_destroy(void* h) { delete static_cast<Sim*>(h); }

// GenerativeTextureEffect::update at current_time_s; when the effect has generated its texture, its mips
// are written into the output slot (texels for water, emissive pixels for fire). Returns 1 if this
// update generated, 0 if not, < 0 on bad arguments.
extern "C" int orc_sim_update(void* h, float current_time_s, const SwTextureMip* mips, uint32_t num_mips, uint64_t* texels,
	const SwEmissiveMip* emips, uint32_t num_emips, uint32_t* emissive_pixels, uint32_t source_texture)
{
	Sim* s = static_cast<Sim*>(h);
	if (!s || !mips || !texels || (source_texture + 1) * NUM_MIPS > num_mips) return SW_ERR_INVALID_ARGUMENT;
	const int32_t out = s->water ? s->cfg.output_texture : s->cfg.output_emissive;
	if (out < 0 || (s->water ? uint64_t(out + 1) * NUM_MIPS > num_mips : uint64_t(out + 1) * NUM_MIPS > num_emips))
		return SW_ERR_INVALID_ARGUMENT;
	if (!s->water && s->cfg.source_emissive >= 0 && uint64_t(s->cfg.source_emissive + 1) * NUM_MIPS > num_emips)
		return SW_ERR_INVALID_ARGUMENT;
	const bool generated = s->update(current_time_s, texels, mips, source_texture, emissive_pixels, emips);
	if (s->generated)
		for (uint32_t m = 0; m < NUM_MIPS; ++m)
		{
			if (s->water)
			{
				const SwTextureMip& d = mips[uint32_t(out) * NUM_MIPS + m];
				if (size_t(d.width) * d.height != s->tex[m].px.size()) return SW_ERR_INVALID_ARGUMENT;
				std::copy(s->tex[m].px.begin(), s->tex[m].px.end(), texels + d.offset);
			}
			else
			{
				const SwEmissiveMip& d = emips[uint32_t(out) * NUM_MIPS + m];
				if (size_t(d.width) * d.height != s->emissive[m].size()) return SW_ERR_INVALID_ARGUMENT;
				std::copy(s->emissive[m].begin(), s->emissive[m].end(), emissive_pixels + d.offset);
			}
		}
	return generated ? 1 : 0;
}

// The current wave field (f32 bits) or heat map (one word per value), its update step and generation flag.
extern "C" int orc_sim_state(void* h, uint32_t* out_words, uint64_t max_words, uint32_t* out_update_step, uint32_t* out_generated,
	uint32_t* out_particles)
{
	Sim* s = static_cast<Sim*>(h);
	if (!s || !out_words) return SW_ERR_INVALID_ARGUMENT;
	const size_t area = size_t(s->w()) * s->h();
	if (max_words < area) return SW_ERR_INVALID_ARGUMENT;
	for (size_t i = 0; i < area; ++i) out_words[i] = s->water ? f32_to_bits(s->wave_field[i]) : uint32_t(s->heat_map[i]);
	if (out_update_step) *out_update_step = s->update_step;
	if (out_generated) *out_generated = s->generated ? 1u : 0u;
	if (out_particles) *out_particles = uint32_t(s->particles.size());
	return 0;
}

// The first n outputs of xoshiro256++ from an explicit state, and of SmallRng::seed_from_u64(seed)
// (known-answer checks of the random engine).
extern "C" void orc_xoshiro_outputs(const uint64_t state[4], uint64_t* out, uint32_t n)
{
	Rand r(1);
	for (int i = 0; i < 4; ++i) r.s[i] = state[i];
	for (uint32_t i = 0; i < n; ++i) out[i] = r.next64();
}
extern "C" void orc_small_rng_state(uint64_t seed, uint64_t out_state[4])
{
	Rand r(seed);
	for (int i = 0; i < 4; ++i) out_state[i] = r.s[i];
}
