// Test infrastructure: restatement of the generative texture effects' per-frame work
// (src/square_wheel/generative_texture_effect_turb.rs:33-138, generative_texture_effect_layered.rs:63-381)
// on the CPU, for checking the host's pass lists and the GPU's output textures.
#include "sw_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace
{

constexpr float TAU = 6.28318530717958647692f;

// `f as i32` (saturating, NaN -> 0)
int32_t as_i32(float f)
{
	if (std::isnan(f)) return 0;
	if (f >= 2147483647.0f) return 2147483647;
	if (f <= -2147483648.0f) return -2147483647 - 1;
	return static_cast<int32_t>(f);
}

struct Lanes
{
	int32_t v[4];
};
Lanes lanes_of(uint32_t c)
{
	Lanes l;
	for (int i = 0; i < 4; ++i) l.v[i] = static_cast<int32_t>((c >> (8 * i)) & 0xFFu);
	return l;
}
uint32_t color_of(const Lanes& l)
{
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i) r |= std::min(static_cast<uint32_t>(l.v[i]), 255u) << (8 * i);
	return r;
}
int32_t wrap_add(int32_t a, int32_t b) { return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b)); }
int32_t wrap_mul(int32_t a, int32_t b) { return static_cast<int32_t>(static_cast<uint32_t>(a) * static_cast<uint32_t>(b)); }

// apply_texture_layer + apply_texture_layer_impl_1/2 over one destination mip
void apply_layer(uint64_t* dst, uint32_t dw, uint32_t dh, const uint64_t* src, uint32_t sw, uint32_t sh, const int32_t shift[2],
	const float light[3], uint32_t blend)
{
	bool modulate = false;
	for (int c = 0; c < 3; ++c) modulate = modulate || light[c] < 0.98f || light[c] > 1.02f;
	const float scale = 256.0f;
	const int32_t lv[4] = {as_i32(light[2] * scale), as_i32(light[1] * scale), as_i32(light[0] * scale), 0};
	for (uint32_t v = 0; v < dh; ++v)
	{
		int32_t sv = (shift[1] + static_cast<int32_t>(v)) % static_cast<int32_t>(sh);
		if (sv < 0) sv += static_cast<int32_t>(sh);
		int32_t su = shift[0] % static_cast<int32_t>(sw);
		if (su < 0) su += static_cast<int32_t>(sw);
		for (uint32_t u = 0; u < dw; ++u)
		{
			uint64_t& d = dst[uint64_t(v) * dw + u];
			const uint64_t t = src[uint64_t(sv) * sw + static_cast<uint32_t>(su)];
			const uint32_t td = static_cast<uint32_t>(t), dd = static_cast<uint32_t>(d);
			const uint64_t t_normal = t >> 32, d_normal = d >> 32;
			Lanes m = lanes_of(td);
			if (modulate)
				for (int i = 0; i < 4; ++i) m.v[i] = wrap_mul(m.v[i], lv[i]) >> 8;
			uint32_t out_diffuse = dd;
			uint64_t out_normal = d_normal;
			switch (blend)
			{
			case SW_BLEND_NONE:
				out_diffuse = modulate ? color_of(m) : td;
				out_normal = t_normal;
				break;
			case SW_BLEND_AVERAGE:
				if (modulate)
				{
					const Lanes dl = lanes_of(dd);
					Lanes s;
					for (int i = 0; i < 4; ++i) s.v[i] = wrap_add(m.v[i], dl.v[i]) >> 1;
					out_diffuse = color_of(s);
				}
				else
					out_diffuse = (((td ^ dd) & 0xFEFEFEFEu) >> 1) + (td & dd);
				break;
			case SW_BLEND_ADDITIVE:
			{
				const Lanes dl = lanes_of(dd);
				Lanes s;
				for (int i = 0; i < 4; ++i) s.v[i] = wrap_add(m.v[i], dl.v[i]);
				out_diffuse = color_of(s);
				break;
			}
			case SW_BLEND_ALPHA_TEST:
				if ((td & 0xFF000000u) > 0x7F000000u)
				{
					out_diffuse = modulate ? color_of(m) : td;
					out_normal = t_normal;
				}
				break;
			default:
			{
				const int32_t alpha = static_cast<int32_t>(td >> 24);
				const Lanes dl = lanes_of(dd);
				Lanes s;
				for (int i = 0; i < 4; ++i) s.v[i] = wrap_add(wrap_mul(m.v[i], alpha), wrap_mul(dl.v[i], 255 - alpha)) >> 8;
				out_diffuse = color_of(s);
				break;
			}
			}
			d = (out_normal << 32) | out_diffuse;
			if (++su == static_cast<int32_t>(sw)) su = 0;
		}
	}
}

} // namespace

// make_turb_distortion's shift table (turb.rs:100-113) into a buffer that persists between calls as the
// effect's temp_buffer does: resized to max(w, h) (new entries 0), entries below w rewritten.
extern "C" int orc_turb_shifts(float amplitude, float wave_length, float frequency, float time_s, uint32_t w, uint32_t h,
	uint32_t mip, int32_t* buffer, uint32_t buffer_len)
{
	if (!buffer || buffer_len < std::max(w, h)) return SW_ERR_INVALID_ARGUMENT;
	const float mip_scale = 1.0f / static_cast<float>(1 << mip);
	const float amplitude_corrected = mip_scale * amplitude;
	const float frequency_scaled = TAU / (wave_length * mip_scale);
	const float time_based_shift = time_s * frequency * TAU;
	for (uint32_t x = 0; x < w; ++x)
	{
		const float arg = static_cast<float>(x) * frequency_scaled + time_based_shift; // f32_mul_add, unfused
		buffer[x] = as_i32(std::round(std::sin(arg) * amplitude_corrected));
	}
	return 0;
}

// The passes of sw_update_textures applied in order to the texel / emissive arrays, in place.
extern "C" int orc_apply_texture_passes(const SwTexturePass* passes, uint32_t num_passes, const int32_t* shifts,
	uint32_t num_shifts, const SwTextureMip* mips, uint32_t num_mips, uint64_t* texels, const SwEmissiveMip* emissive_mips,
	uint32_t num_emissive_mips, uint32_t* emissive)
{
	for (uint32_t p = 0; p < num_passes; ++p)
	{
		const SwTexturePass& a = passes[p];
		if (a.kind & SW_TEXPASS_TURB)
		{
			const bool em = (a.kind & SW_TEXPASS_EMISSIVE) != 0;
			if (em ? (a.dst_mip >= num_emissive_mips || a.src_mip >= num_emissive_mips) : (a.dst_mip >= num_mips || a.src_mip >= num_mips))
				return SW_ERR_INVALID_ARGUMENT;
			const uint32_t w = em ? emissive_mips[a.dst_mip].width : mips[a.dst_mip].width;
			const uint32_t h = em ? emissive_mips[a.dst_mip].height : mips[a.dst_mip].height;
			if (a.shifts_offset + std::max(w, h) > num_shifts) return SW_ERR_INVALID_ARGUMENT;
			const int32_t* s = shifts + a.shifts_offset;
			const int32_t mask[2] = {static_cast<int32_t>(w) - 1, static_cast<int32_t>(h) - 1};
			for (uint32_t y = 0; y < h; ++y)
			{
				const int32_t row_shift = s[y];
				for (uint32_t x = 0; x < w; ++x)
				{
					const int32_t u = static_cast<int32_t>(x) + row_shift;
					const int32_t v = static_cast<int32_t>(y) + s[x];
					const uint64_t at = static_cast<uint64_t>((u & mask[0]) + (v & mask[1]) * static_cast<int32_t>(w));
					if (em)
						emissive[emissive_mips[a.dst_mip].offset + uint64_t(y) * w + x] = emissive[emissive_mips[a.src_mip].offset + at];
					else
						texels[mips[a.dst_mip].offset + uint64_t(y) * w + x] = texels[mips[a.src_mip].offset + at];
				}
			}
		}
		else
		{
			if (a.dst_mip >= num_mips || a.src_mip >= num_mips) return SW_ERR_INVALID_ARGUMENT;
			const bool zero = a.light[0] <= 1.0f / 128.0f && a.light[1] <= 1.0f / 128.0f && a.light[2] <= 1.0f / 128.0f;
			if (a.blending_mode == SW_BLEND_ADDITIVE && zero) continue; // adding zero
			const SwTextureMip& d = mips[a.dst_mip];
			const SwTextureMip& s = mips[a.src_mip];
			apply_layer(texels + d.offset, d.width, d.height, texels + s.offset, s.width, s.height, a.shift, a.light, a.blending_mode);
		}
	}
	return 0;
}
