// Test infrastructure: the texture mix of a portal's view (build_view_portals_textures' second loop,
// src/square_wheel/partial_renderer.rs:2189-2280, with mix_surface_with_texture_impl,
// src/square_wheel/surfaces.rs:903-971) on the CPU, over a rendered view region.
#include "sw_oracle.h"
#include "sw_oracle_math.h"

namespace
{
using namespace sworacle;

template <class T, ColorVecI (*FROM)(T), T (*TO)(const ColorVecI&)>
void mix_region(const SwView& v, T* region, const uint32_t* lite)
{
	const float scale = 256.0f;
	const float l[3] = {v.mix_light[0] * scale, v.mix_light[1] * scale, v.mix_light[2] * scale};
	const ColorVecI light = ci_from_f32x3(l);
	for (uint32_t dv = 0; dv < v.height; ++dv)
	{
		int32_t sv = (v.mix_tc_min[1] + static_cast<int32_t>(dv)) % static_cast<int32_t>(v.mix_size[1]);
		if (sv < 0) sv += static_cast<int32_t>(v.mix_size[1]);
		const uint32_t* src_line = lite + v.mix_offset + uint64_t(sv) * v.mix_size[0];
		int32_t su = v.mix_tc_min[0] % static_cast<int32_t>(v.mix_size[0]);
		if (su < 0) su += static_cast<int32_t>(v.mix_size[0]);
		for (uint32_t du = 0; du < v.width; ++du)
		{
			T& dst = region[uint64_t(dv) * v.width + du];
			const uint32_t texel = src_line[su];
			const ColorVecI modulated = ci_shr(ci_mul(ci_from_c32(texel), light), 8);
			switch (v.mix_blend)
			{
			case SW_BLEND_NONE: dst = TO(modulated); break;
			case SW_BLEND_AVERAGE: dst = TO(ci_shr(ci_add(modulated, FROM(dst)), 1)); break;
			case SW_BLEND_ADDITIVE: dst = TO(ci_add(modulated, FROM(dst))); break;
			case SW_BLEND_ALPHA_TEST:
				if ((texel & 0xFF000000u) > 0x7F000000u) dst = TO(modulated);
				break;
			default:
			{
				const int32_t alpha = static_cast<int32_t>(texel >> 24);
				dst = TO(ci_shr(ci_add(ci_mul_scalar(modulated, alpha), ci_mul_scalar(FROM(dst), 255 - alpha)), 8));
				break;
			}
			}
			if (++su == static_cast<int32_t>(v.mix_size[0])) su = 0;
		}
	}
}

ColorVecI from32(uint32_t c) { return ci_from_c32(c); }
ColorVecI from64(uint64_t c) { return ci_from_c64(c); }

} // namespace

// The view's texture mixed into its rendered region (width x height pixels of the pixel format).
extern "C" int orc_mix_view(const SwView* view, void* region, uint32_t pixel_format, const uint32_t* lite, uint64_t lite_pixels)
{
	if (!view || !region || !lite) return SW_ERR_INVALID_ARGUMENT;
	const SwView& v = *view;
	if (v.mix_blend == SW_VIEW_NO_MIX) return 0;
	if (v.mix_blend > SW_BLEND_ALPHA_BLEND || v.mix_size[0] == 0 || v.mix_size[1] == 0 ||
		v.mix_offset + uint64_t(v.mix_size[0]) * v.mix_size[1] > lite_pixels)
		return SW_ERR_INVALID_ARGUMENT;
	if (pixel_format == SW_PIXEL_C64)
		mix_region<uint64_t, from64, ci_to_c64>(v, static_cast<uint64_t*>(region), lite);
	else
		mix_region<uint32_t, from32, ci_to_c32>(v, static_cast<uint32_t*>(region), lite);
	return 0;
}
