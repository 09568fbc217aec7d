// Host side of the simulated generative texture effects, water (GenerativeTextureEffectWater,
// src/square_wheel/generative_texture_effect_water.rs) and fire (GenerativeTextureEffectFire,
// generative_texture_effect_fire.rs): the scalar per-step work (time functions, the effects' random
// engine, line rasterisation of the sources, fire particles) done here, in the reference's order, and
// emitted as SwSimPass / SwSimPoint lists whose per-word work (field steps, textures, mips) the GPU runs
// on fields resident in the context's simulation state.
#pragma once

#include <cstdint>
#include <vector>

#include "scene.h"
#include "../../include/swgpu.h"

namespace swhost
{

// rand 0.8.5's SmallRng on 64-bit targets: xoshiro256++ (Blackman and Vigna), seeded through
// SeedableRng::seed_from_u64's default body in rand_core 0.6 (PCG32 outputs fill the 32-byte seed;
// SmallRng does not forward to xoshiro's own SplitMix64 seeding), with rand 0.8.5's uniform samplers.
class SmallRng
{
public:
	explicit SmallRng(uint64_t seed);
	static SmallRng from_state(const uint64_t s[4]);
	uint64_t next_u64();
	uint32_t next_u32() { return uint32_t(next_u64() >> 32); }
	// Rng::gen_range(low ..= high) for f32: UniformFloat::new_inclusive + sample (one u32 drawn)
	float gen_f32_inclusive(float low, float high);
	// Rng::gen_range(low ..= high) for i32: UniformInt::sample_single_inclusive (widening multiply, rejection)
	int32_t gen_i32_inclusive(int32_t low, int32_t high);
	uint64_t s[4];

private:
	SmallRng() = default;
};

// create_rand_engine's seed (generative_texture_effects_common.rs)
constexpr uint64_t EFFECT_RAND_SEED = 0b1001100000111010100101010101010111000111010110100101111001010101ull;

// One frame's simulation work: passes (sorted by launch once finished) and their points.
struct SimBatch
{
	std::vector<SwSimPass> passes;
	std::vector<SwSimPoint> points;
	// Launch numbers above TAIL are the texture / mip phases after every step: rewritten by finish().
	static constexpr uint32_t TAIL = 0x80000000u;
	void clear()
	{
		passes.clear();
		points.clear();
	}
	// Tail phases placed after the last step launch, passes stably sorted by launch.
	void finish();
};

// What an effect's texture generation reads from the static scene: its source and output slots.
struct SimTextures
{
	uint32_t source_texture;    // the material's own texture (colour source, base colour)
	int32_t output_texture;     // WATER: texture slot written
	int32_t output_emissive;    // FIRE: emissive slot written
	int32_t source_emissive;    // FIRE: the material's emissive texture (palette source), -1 without
	uint32_t base_color;        // WATER: the source's last mip's first texel's diffuse
	uint32_t emissive_width;    // FIRE: the source emissive mip 0's width (0: empty)
	const uint32_t* emissive_row; // FIRE: the source emissive mip 0's first row
	float roughness;            // WATER: Material::roughness clamped to [MIN_VALID_ROUGHNESS, 1]
};

// A water or fire effect's host state (update step, previous update time, random engine, particles),
// with the steps its constructor ran queued until the first update emits them.
class EffectSim
{
public:
	EffectSim(const Material& m, uint64_t state_offset);
	// GenerativeTextureEffect::update at current_time_s: 0..10 fixed steps, then (if any) the texture and
	// its mips. Appends to `out` with local launch numbers (2k: step k's water sources, 2k + 1: its field
	// step, 2k + 2: fire sources), tails for the texture phases.
	void update(float current_time_s, const SimTextures& tex, SimBatch& out);
	bool generated() const { return generated_; }
	uint32_t update_step() const { return update_step_; }
	uint32_t current_buffer() const { return cur_; }
	uint32_t num_particles() const { return uint32_t(particles_.size()); }

private:
	struct Particle
	{
		float vx, vy, px, py;
		uint32_t despawn_time;
		float gravity;
		uint32_t heat;
	};
	void water_step(std::vector<SwSimPoint>& pts);
	void fire_step(std::vector<SwSimPoint>& pts);
	float random_value(const RandomValue& v, float time_s);
	void emit_step(const std::vector<SwSimPoint>& pts, SimBatch& out, uint32_t& k);

	bool water_;
	WaterEffect water_cfg_;
	FireEffect fire_cfg_;
	float update_frequency_;
	uint64_t state_offset_;
	uint32_t lx_, ly_;
	SmallRng rng_;
	uint32_t update_step_ = 0;
	float prev_update_time_s_ = 0.0f;
	std::vector<Particle> particles_;
	std::vector<int32_t> rand_buffer_;
	uint32_t palette_[256];
	bool generated_ = false;
	uint32_t cur_ = 0; // which of the two buffers holds the current field / heat map on the device
	std::vector<std::vector<SwSimPoint>> pending_; // the constructor's steps, not yet emitted
};

// Words of simulation state a material's effect needs (two fields / heat maps), 0 for other materials.
uint64_t sim_state_words(const Material& m);

} // namespace swhost
