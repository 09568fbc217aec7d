// Host side of the simulated water and fire texture effects (see sims.h).
#include "sims.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace swhost
{
namespace
{

constexpr float TAU = 6.28318530717958647692f;

// `f as i32`: truncation, saturating, NaN -> 0
int32_t as_i32(float f)
{
	if (std::isnan(f)) return 0;
	if (f >= 2147483647.0f) return 2147483647;
	if (f <= -2147483648.0f) return -2147483647 - 1;
	return int32_t(f);
}
// `f as u8`: truncation, saturating, NaN -> 0
uint32_t as_u8(float f)
{
	if (!(f > 0.0f)) return 0;
	if (f >= 255.0f) return 255;
	return uint32_t(f);
}
int32_t wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
int32_t wsub(int32_t a, int32_t b) { return int32_t(uint32_t(a) - uint32_t(b)); }
int32_t fx16(int32_t v) { return int32_t(uint32_t(v) << 16); }             // int_to_fixed16
int32_t fx16_round(int32_t v) { return wadd(v, 1 << 15) >> 16; }         // fixed16_round_to_int
int32_t iabs(int32_t v) { return v < 0 ? wsub(0, v) : v; }
uint32_t rotr32(uint32_t x, uint32_t r) { return (x >> (r & 31)) | (x << ((32 - r) & 31)); }
uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
uint32_t f32_bits(float f)
{
	uint32_t b;
	std::memcpy(&b, &f, 4);
	return b;
}
float from_bits(uint32_t b)
{
	float f;
	std::memcpy(&f, &b, 4);
	return f;
}

// convert_heat (generative_texture_effect_fire.rs:425-428): (heat * 255).max(0).min(255) as u8
uint32_t convert_heat(float heat) { return as_u8(std::fmin(std::fmax(heat * 255.0f, 0.0f), 255.0f)); }

// Color32::from_rgb (src/common/color.rs:16-19)
uint32_t from_rgb(uint32_t r, uint32_t g, uint32_t b) { return (r << 16) | (g << 8) | b; }

} // namespace

// ---- SmallRng ---------------------------------------------------------------------------------

SmallRng::SmallRng(uint64_t seed)
{
	// rand_core 0.6 SeedableRng::seed_from_u64: PCG32 (XSH RR) steps fill the seed four bytes at a time
	uint8_t bytes[32];
	uint64_t state = seed;
	for (int chunk = 0; chunk < 8; ++chunk)
	{
		state = state * 6364136223846793005ull + 11634580027462260723ull;
		const uint32_t xorshifted = uint32_t(((state >> 18) ^ state) >> 27);
		const uint32_t x = rotr32(xorshifted, uint32_t(state >> 59));
		for (int b = 0; b < 4; ++b) bytes[chunk * 4 + b] = uint8_t(x >> (8 * b));
	}
	bool zero = true;
	for (uint8_t b : bytes) zero = zero && b == 0;
	if (zero)
	{
		// Xoshiro256PlusPlus::from_seed of an all-zero seed falls back to its SplitMix64 seed_from_u64(0)
		uint64_t sm = 0;
		for (int i = 0; i < 4; ++i)
		{
			sm += 0x9e3779b97f4a7c15ull;
			uint64_t z = sm;
			z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
			z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
			s[i] = z ^ (z >> 31);
		}
		return;
	}
	for (int i = 0; i < 4; ++i)
	{
		uint64_t v = 0;
		for (int b = 0; b < 8; ++b) v |= uint64_t(bytes[i * 8 + b]) << (8 * b);
		s[i] = v;
	}
}

SmallRng SmallRng::from_state(const uint64_t st[4])
{
	SmallRng r;
	for (int i = 0; i < 4; ++i) r.s[i] = st[i];
	return r;
}

uint64_t SmallRng::next_u64()
{
	// xoshiro256++ 1.0
	const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
	const uint64_t t = s[1] << 17;
	s[2] ^= s[0];
	s[3] ^= s[1];
	s[1] ^= s[2];
	s[0] ^= s[3];
	s[2] ^= t;
	s[3] = rotl64(s[3], 45);
	return result;
}

float SmallRng::gen_f32_inclusive(float low, float high)
{
	// UniformFloat::new_inclusive: scale = (high - low) / max_rand, stepped down one ulp at a time until
	// scale * max_rand + low <= high; sample: a [1, 2) float from the top 23 bits of a u32, minus 1, times
	// scale plus low. (The reference asserts low <= high and a finite scale; both hold for its callers.)
	const float max_rand = from_bits(0x3FFFFFFFu) - 1.0f;
	float scale = (high - low) / max_rand;
	if (std::isfinite(scale))
		while (scale * max_rand + low > high) scale = from_bits(f32_bits(scale) - 1);
	const float value1_2 = from_bits((next_u32() >> 9) | 0x3F800000u);
	const float value0_1 = value1_2 - 1.0f;
	return value0_1 * scale + low;
}

int32_t SmallRng::gen_i32_inclusive(int32_t low, int32_t high)
{
	const uint32_t range = uint32_t(high) - uint32_t(low) + 1u;
	if (range == 0) return int32_t(next_u32());
	const uint32_t zone = (range << __builtin_clz(range)) - 1u;
	for (;;)
	{
		const uint64_t m = uint64_t(next_u32()) * range;
		if (uint32_t(m) <= zone) return wadd(low, int32_t(uint32_t(m >> 32)));
	}
}

// ---- SimBatch --------------------------------------------------------------------------------

void SimBatch::finish()
{
	uint32_t last = 0;
	bool any = false;
	for (const SwSimPass& p : passes)
		if (p.launch < TAIL)
		{
			last = std::max(last, p.launch);
			any = true;
		}
	const uint32_t base = any ? last + 1 : 0;
	for (SwSimPass& p : passes)
		if (p.launch >= TAIL) p.launch = base + (p.launch - TAIL);
	std::stable_sort(passes.begin(), passes.end(), [](const SwSimPass& a, const SwSimPass& b) { return a.launch < b.launch; });
}

// ---- EffectSim -------------------------------------------------------------------------------

uint64_t sim_state_words(const Material& m)
{
	if (m.effect == Material::WATER) return 2ull << (m.water.resolution_log2[0] + m.water.resolution_log2[1]);
	if (m.effect == Material::FIRE) return 2ull << (m.fire.resolution_log2[0] + m.fire.resolution_log2[1]);
	return 0;
}

EffectSim::EffectSim(const Material& m, uint64_t state_offset)
	: water_(m.effect == Material::WATER), water_cfg_(m.water), fire_cfg_(m.fire), state_offset_(state_offset),
	  rng_(EFFECT_RAND_SEED)
{
	if (water_)
	{
		// GenerativeTextureEffectWater::new (water.rs:21-55): a corrected frequency, then min(diagonal, 512)
		// steps towards equilibrium
		update_frequency_ = std::fmin(std::fmax(water_cfg_.update_frequency, 1.0f), 200.0f);
		lx_ = water_cfg_.resolution_log2[0];
		ly_ = water_cfg_.resolution_log2[1];
		const float diagonal = std::sqrt(float((1ull << (lx_ * 2)) + (1ull << (ly_ * 2))));
		const int32_t n = std::min(as_i32(diagonal), 512);
		for (int32_t i = 0; i < n; ++i)
		{
			pending_.emplace_back();
			water_step(pending_.back());
		}
	}
	else
	{
		// GenerativeTextureEffectFire::new (fire.rs:21-60): a grey palette, 16 steps towards equilibrium
		update_frequency_ = std::fmin(std::fmax(fire_cfg_.update_frequency, 1.0f), 200.0f);
		lx_ = fire_cfg_.resolution_log2[0];
		ly_ = fire_cfg_.resolution_log2[1];
		for (uint32_t i = 0; i < 256; ++i) palette_[i] = from_rgb(i, i, i);
		particles_.reserve(256);
		for (int i = 0; i < 16; ++i)
		{
			pending_.emplace_back();
			fire_step(pending_.back());
		}
	}
}

void EffectSim::water_step(std::vector<SwSimPoint>& pts)
{
	// step_update_wave_field (water.rs:57-225): the sources' points; the field step itself runs on the GPU
	++update_step_;
	const uint32_t mask[2] = {(1u << lx_) - 1u, (1u << ly_) - 1u};
	const float time_s = float(update_step_) / update_frequency_;
	auto add = [&](uint32_t x, uint32_t y, float v) {
		pts.push_back(SwSimPoint{(x & mask[0]) + ((y & mask[1]) << lx_), f32_bits(v)});
	};
	for (const WaveSource& src : water_cfg_.sources)
	{
		switch (src.kind)
		{
		case WaveSource::WAVY_SPOT:
		{
			const float value = std::sin(time_s * src.frequency * TAU + src.phase) * src.amplitude * src.frequency + src.offset;
			add(uint32_t(as_i32(float(src.points[0][0]) + src.offsets[0][0].evaluate(time_s))),
				uint32_t(as_i32(float(src.points[0][1]) + src.offsets[0][1].evaluate(time_s))), value);
			break;
		}
		case WaveSource::WAVY_LINE:
		{
			int32_t p[2][2];
			for (int i = 0; i < 2; ++i)
				for (int j = 0; j < 2; ++j) p[i][j] = as_i32(float(src.points[i][j]) + src.offsets[i][j].evaluate(time_s));
			const float value = std::sin(time_s * src.frequency * TAU + src.phase) * src.amplitude * src.frequency + src.offset;
			const int32_t adx = iabs(wsub(p[0][0], p[1][0])), ady = iabs(wsub(p[0][1], p[1][1]));
			if (adx == 0 && ady == 0)
				add(uint32_t(p[0][0]), uint32_t(p[0][1]), value);
			else if (adx >= ady)
			{
				if (p[0][0] > p[1][0]) std::swap(p[0], p[1]);
				const int32_t y_step = fx16(wsub(p[1][1], p[0][1])) / adx;
				int32_t y_fract = fx16(p[0][1]);
				for (int32_t xo = 0; xo <= adx; ++xo)
				{
					const int32_t y = fx16_round(y_fract);
					y_fract = wadd(y_fract, y_step);
					add(uint32_t(wadd(p[0][0], xo)), uint32_t(y), value);
				}
			}
			else
			{
				if (p[0][1] > p[1][1]) std::swap(p[0], p[1]);
				const int32_t x_step = fx16(wsub(p[1][0], p[0][0])) / ady;
				int32_t x_fract = fx16(p[0][0]);
				for (int32_t yo = 1; yo <= ady; ++yo)
				{
					const int32_t x = fx16_round(x_fract);
					x_fract = wadd(x_fract, x_step);
					add(uint32_t(x), uint32_t(wadd(p[0][1], yo)), value);
				}
			}
			break;
		}
		case WaveSource::PERIODIC_DROPLET:
		{
			const float rel = src.frequency / update_frequency_;
			const int32_t begin = as_i32(float(update_step_) * rel + src.phase);
			const int32_t end = as_i32(float(update_step_ + 1) * rel + src.phase);
			if (begin < end)
			{
				const uint32_t x = uint32_t(as_i32(float(src.points[0][0]) + src.offsets[0][0].evaluate(time_s)));
				const uint32_t y = uint32_t(as_i32(float(src.points[0][1]) + src.offsets[0][1].evaluate(time_s)));
				for (int32_t i = begin; i < end; ++i) add(x, y, src.amplitude);
			}
			break;
		}
		default: // RAIN
			if (rng_.gen_f32_inclusive(0.0f, 1.0f) <= src.frequency / update_frequency_)
			{
				uint32_t x, y;
				if (src.radius > 0.0f)
				{
					const float dist = rng_.gen_f32_inclusive(0.0f, src.radius);
					const float angle = rng_.gen_f32_inclusive(0.0f, TAU);
					const float dx = std::cos(angle) * dist, dy = std::sin(angle) * dist;
					x = uint32_t(wadd(int32_t(src.points[0][0]), as_i32(dx)));
					y = uint32_t(wadd(int32_t(src.points[0][1]), as_i32(dy)));
				}
				else
				{
					x = rng_.next_u32();
					y = rng_.next_u32();
				}
				add(x, y, src.amplitude);
			}
			break;
		}
	}
	// points on one address stay in order, the GPU applies each address's run in sequence
	std::stable_sort(pts.begin(), pts.end(), [](const SwSimPoint& a, const SwSimPoint& b) { return a.address < b.address; });
}

float EffectSim::random_value(const RandomValue& v, float time_s)
{
	// get_value_with_random_deviation (fire.rs:93-97)
	const float value = v.value.evaluate(time_s);
	const float deviation = v.deviation.evaluate(time_s);
	return value - deviation + rng_.gen_f32_inclusive(0.0f, std::fmax(deviation, 0.0f) * 2.0f);
}

void EffectSim::fire_step(std::vector<SwSimPoint>& pts)
{
	// step_update_heat_map (fire.rs:62-321): the heat map step runs on the GPU first, then these points
	// (sources, then particles) raise it to their heat (max: their order does not matter)
	++update_step_;
	const float time_s = float(update_step_) / update_frequency_;
	const uint32_t mask[2] = {(1u << lx_) - 1u, (1u << ly_) - 1u};
	auto set_heat = [&](uint32_t x, uint32_t y, uint32_t heat) {
		pts.push_back(SwSimPoint{(x & mask[0]) + ((y & mask[1]) << lx_), heat & 0xFFu});
	};
	for (const HeatSource& src : fire_cfg_.sources)
	{
		switch (src.kind)
		{
		case HeatSource::POINT:
		{
			const float ox = random_value(src.offset[0][0], time_s);
			const float oy = random_value(src.offset[0][1], time_s);
			const uint32_t x = uint32_t(as_i32(std::floor(float(src.points[0][0]) + ox)));
			const uint32_t y = uint32_t(as_i32(std::floor(float(src.points[0][1]) + oy)));
			set_heat(x, y, convert_heat(random_value(src.heat, time_s)));
			break;
		}
		case HeatSource::LINE:
		{
			const uint32_t heat = convert_heat(random_value(src.heat, time_s));
			int32_t p[2][2] = {{int32_t(src.points[0][0]), int32_t(src.points[0][1])}, {int32_t(src.points[1][0]), int32_t(src.points[1][1])}};
			const int32_t adx = iabs(wsub(p[0][0], p[1][0])), ady = iabs(wsub(p[0][1], p[1][1]));
			if (adx >= ady)
			{
				if (uint32_t(p[0][0]) > uint32_t(p[1][0])) std::swap(p[0], p[1]); // the u32 points compared
				// a zero-length line divides by zero in the reference (a panic); it sets the one point here
				const int32_t y_step = adx ? fx16(wsub(p[1][1], p[0][1])) / adx : 0;
				int32_t y_fract = fx16(p[0][1]);
				for (int32_t xo = 0; xo <= adx; ++xo)
				{
					const int32_t y = fx16_round(y_fract);
					y_fract = wadd(y_fract, y_step);
					set_heat(uint32_t(wadd(p[0][0], xo)), uint32_t(y), heat);
				}
			}
			else
			{
				if (uint32_t(p[0][1]) > uint32_t(p[1][1])) std::swap(p[0], p[1]);
				const int32_t x_step = fx16(wsub(p[1][0], p[0][0])) / ady;
				int32_t x_fract = fx16(p[0][0]);
				for (int32_t yo = 1; yo <= ady; ++yo)
				{
					const int32_t x = fx16_round(x_fract);
					x_fract = wadd(x_fract, x_step);
					set_heat(uint32_t(x), uint32_t(wadd(p[0][1], yo)), heat);
				}
			}
			break;
		}
		case HeatSource::LIGHTNING:
		{
			const uint32_t heat = convert_heat(random_value(src.heat, time_s));
			const int32_t head = fx16(int32_t(heat));
			int32_t heat_start = head, heat_end = src.ramp ? 0 : head;
			int32_t p[2][2] = {{int32_t(src.points[0][0]), int32_t(src.points[0][1])}, {int32_t(src.points[1][0]), int32_t(src.points[1][1])}};
			for (int i = 0; i < 2; ++i)
				for (int j = 0; j < 2; ++j) p[i][j] = wadd(p[i][j], as_i32(random_value(src.offset[i][j], time_s)));
			const int32_t adx = iabs(wsub(p[0][0], p[1][0])), ady = iabs(wsub(p[0][1], p[1][1]));
			const int32_t max_delta = std::max(adx, ady);
			rand_buffer_.resize(size_t(uint32_t(max_delta)) + 1, 0);
			int32_t rand_offset = 0;
			for (int32_t& r : rand_buffer_)
			{
				r = wadd(rand_offset, rng_.gen_i32_inclusive(-65536, 65536));
				rand_offset = r;
			}
			if (max_delta == 0)
				set_heat(uint32_t(p[0][0]), uint32_t(p[0][1]), heat);
			else if (adx >= ady)
			{
				if (p[0][0] > p[1][0])
				{
					std::swap(p[0], p[1]);
					std::swap(heat_start, heat_end);
				}
				const int32_t y_step = wsub(fx16(wsub(p[1][1], p[0][1])), rand_offset) / adx;
				int32_t y_fract = fx16(p[0][1]);
				const int32_t heat_step = wsub(heat_end, heat_start) / adx;
				int32_t heat_cur = heat_start;
				for (int32_t xo = 0; xo <= adx; ++xo)
				{
					const int32_t y = fx16_round(wadd(y_fract, rand_buffer_[size_t(xo)]));
					set_heat(uint32_t(wadd(p[0][0], xo)), uint32_t(y), uint32_t(heat_cur >> 16));
					y_fract = wadd(y_fract, y_step);
					heat_cur = wadd(heat_cur, heat_step);
				}
			}
			else
			{
				if (p[0][1] > p[1][1])
				{
					std::swap(p[0], p[1]);
					std::swap(heat_start, heat_end);
				}
				const int32_t x_step = wsub(fx16(wsub(p[1][0], p[0][0])), rand_offset) / ady;
				int32_t x_fract = fx16(p[0][0]);
				const int32_t heat_step = wsub(heat_end, heat_start) / ady;
				int32_t heat_cur = heat_start;
				for (int32_t yo = 0; yo <= ady; ++yo)
				{
					const int32_t x = fx16_round(wadd(x_fract, rand_buffer_[size_t(yo)]));
					set_heat(uint32_t(x), uint32_t(wadd(p[0][1], yo)), uint32_t(heat_cur >> 16));
					x_fract = wadd(x_fract, x_step);
					heat_cur = wadd(heat_cur, heat_step);
				}
			}
			break;
		}
		default: // FOUNTAIN
		{
			const float rel = src.frequency / update_frequency_;
			const int32_t begin = as_i32(float(update_step_) * rel), end = as_i32(float(update_step_ + 1) * rel);
			for (int32_t i = begin; i < end; ++i)
			{
				if (particles_.size() >= 256) continue;
				const float heat = random_value(src.heat, time_s);
				const float angle = random_value(src.angle, time_s);
				const float speed = random_value(src.speed, time_s);
				const float gravity = random_value(src.gravity, time_s);
				const float spawn_angle = random_value(src.spawn_angle, time_s);
				const float spawn_distance = random_value(src.spawn_distance, time_s);
				const float lifetime = random_value(src.lifetime, time_s);
				const float vs = speed / update_frequency_;
				Particle pt;
				pt.vx = std::cos(angle) * vs;
				pt.vy = std::sin(angle) * vs;
				pt.px = float(src.points[0][0]) + std::cos(spawn_angle) * spawn_distance;
				pt.py = float(src.points[0][1]) + std::sin(spawn_angle) * spawn_distance;
				const uint32_t life = uint32_t(std::fmin(std::fmax(lifetime * update_frequency_, 1.0f), 1024.0f));
				pt.despawn_time = update_step_ + life;
				pt.gravity = gravity / (update_frequency_ * update_frequency_);
				pt.heat = convert_heat(heat);
				particles_.push_back(pt);
			}
			break;
		}
		}
	}
	// particles: despawned ones swap-removed, the rest moved and heating their cell
	for (size_t i = 0; i < particles_.size();)
	{
		Particle& p = particles_[i];
		if (p.despawn_time <= update_step_)
		{
			p = particles_.back();
			particles_.pop_back();
			continue;
		}
		p.vy = p.vy + p.gravity;
		p.px = p.px + p.vx;
		p.py = p.py + p.vy;
		set_heat(uint32_t(as_i32(std::floor(p.px))), uint32_t(as_i32(std::floor(p.py))), p.heat);
		++i;
	}
}

void EffectSim::emit_step(const std::vector<SwSimPoint>& pts, SimBatch& out, uint32_t& k)
{
	const uint64_t area = 1ull << (lx_ + ly_);
	const uint64_t buf[2] = {state_offset_, state_offset_ + area};
	SwSimPass p;
	std::memset(&p, 0, sizeof(p));
	p.size_log2[0] = lx_;
	p.size_log2[1] = ly_;
	if (water_)
	{
		if (!pts.empty())
		{
			p.kind = SW_SIM_WATER_POINTS;
			p.launch = 2 * k;
			p.state_src = buf[cur_];
			p.state_dst = buf[1 - cur_];
			p.first_point = uint32_t(out.points.size());
			p.num_points = uint32_t(pts.size());
			out.points.insert(out.points.end(), pts.begin(), pts.end());
			out.passes.push_back(p);
		}
		// update_wave_field(attenuation, dst = old field, src = field), then the two swap
		const float attenuation = 1.0f - 1.0f / std::fmin(std::fmax(water_cfg_.fluidity, 10.0f), 1000000.0f);
		p.kind = SW_SIM_WATER_STEP;
		p.launch = 2 * k + 1;
		p.state_src = buf[cur_];
		p.state_dst = buf[1 - cur_];
		p.first_point = p.num_points = 0;
		p.param = f32_bits(attenuation);
		out.passes.push_back(p);
		cur_ = 1 - cur_;
	}
	else
	{
		const float attenuation = 1.0f - 1.0f / std::fmin(std::fmax(fire_cfg_.heat_conductivity, 1.0f), 1000000.0f);
		p.kind = SW_SIM_FIRE_STEP;
		p.launch = 2 * k + 1;
		p.state_src = buf[cur_];
		p.state_dst = buf[1 - cur_];
		p.flags = fire_cfg_.slow ? SW_SIM_FIRE_SLOW : 0u;
		p.param = uint32_t(std::fmin(std::fmax(attenuation, 0.0f), 1.0f) * float(1 << 18)); // attenuation_i
		out.passes.push_back(p);
		cur_ = 1 - cur_;
		if (!pts.empty())
		{
			p.kind = SW_SIM_FIRE_POINTS;
			p.launch = 2 * k + 2;
			p.state_src = p.state_dst = buf[cur_];
			p.flags = p.param = 0;
			p.first_point = uint32_t(out.points.size());
			p.num_points = uint32_t(pts.size());
			out.points.insert(out.points.end(), pts.begin(), pts.end());
			out.passes.push_back(p);
		}
	}
	++k;
}

void EffectSim::update(float current_time_s, const SimTextures& tex, SimBatch& out)
{
	uint32_t k = 0;
	// the constructor's steps first
	for (const std::vector<SwSimPoint>& pts : pending_) emit_step(pts, out, k);
	pending_.clear();
	// fixed steps: (t * f) as i32 - (prev * f) as i32, clamped to [0, 10] (water.rs:235-251, fire.rs:331-347)
	const int32_t steps = std::min(std::max(wsub(as_i32(current_time_s * update_frequency_),
		as_i32(prev_update_time_s_ * update_frequency_)), 0), 10);
	prev_update_time_s_ = current_time_s;
	if (steps == 0) return;
	std::vector<SwSimPoint> pts;
	for (int32_t i = 0; i < steps; ++i)
	{
		pts.clear();
		if (water_) water_step(pts);
		else fire_step(pts);
		emit_step(pts, out, k);
	}
	const uint64_t area = 1ull << (lx_ + ly_);
	SwSimPass p;
	std::memset(&p, 0, sizeof(p));
	p.size_log2[0] = lx_;
	p.size_log2[1] = ly_;
	p.state_src = state_offset_ + (cur_ ? area : 0);
	p.launch = SimBatch::TAIL;
	if (water_)
	{
		// make_wavy_texture into mip 0, then build_texture_mip for mips 1..4 (water.rs:253-305)
		p.kind = SW_SIM_WATER_TEXTURE;
		p.dst_mip = uint32_t(tex.output_texture) * NUM_MIPS;
		p.src_mip = tex.source_texture * NUM_MIPS;
		p.flags = (water_cfg_.color_mode << SW_SIM_COLOR_MODE_SHIFT) | (generated_ ? 0u : SW_SIM_WATER_INIT_DIFFUSE);
		p.param = f32_bits(tex.roughness);
		p.base_color = tex.base_color;
		out.passes.push_back(p);
		for (uint32_t mip = 1; mip < NUM_MIPS; ++mip)
		{
			SwSimPass m;
			std::memset(&m, 0, sizeof(m));
			m.kind = SW_SIM_TEXTURE_MIP;
			m.launch = SimBatch::TAIL + mip;
			m.dst_mip = uint32_t(tex.output_texture) * NUM_MIPS + mip;
			m.src_mip = m.dst_mip - 1;
			out.passes.push_back(m);
		}
	}
	else
	{
		if (!generated_)
		{
			// the first generation's palette (fire.rs:358-388): from the colour, else from the emissive
			// texture's first row, else the grey one
			if (fire_cfg_.has_color)
				for (uint32_t i = 0; i < 256; ++i)
				{
					const float scale = float(i);
					palette_[i] = from_rgb(as_u8(std::fmin(std::fmax(fire_cfg_.color[0] * scale, 0.0f), 255.0f)),
						as_u8(std::fmin(std::fmax(fire_cfg_.color[1] * scale, 0.0f), 255.0f)),
						as_u8(std::fmin(std::fmax(fire_cfg_.color[2] * scale, 0.0f), 255.0f)));
				}
			else if (tex.source_emissive >= 0 && tex.emissive_width > 0 && tex.emissive_row)
				for (uint32_t i = 0; i < 256; ++i) palette_[i] = tex.emissive_row[(i * tex.emissive_width) >> 8];
		}
		p.kind = SW_SIM_FIRE_TEXTURE;
		p.dst_mip = uint32_t(tex.output_emissive) * NUM_MIPS;
		p.first_point = uint32_t(out.points.size());
		p.num_points = 256;
		for (uint32_t i = 0; i < 256; ++i) out.points.push_back(SwSimPoint{i, palette_[i]});
		out.passes.push_back(p);
		for (uint32_t mip = 1; mip < NUM_MIPS; ++mip)
		{
			SwSimPass m;
			std::memset(&m, 0, sizeof(m));
			m.kind = SW_SIM_EMISSIVE_MIP;
			m.launch = SimBatch::TAIL + mip;
			m.dst_mip = uint32_t(tex.output_emissive) * NUM_MIPS + mip;
			m.src_mip = m.dst_mip - 1;
			out.passes.push_back(m);
		}
	}
	generated_ = true;
}

} // namespace swhost
