// Generative texture effects on the GPU: the per-texel work of GenerativeTextureEffectTurb::update and
// GenerativeTextureEffectLayered::update (src/square_wheel/generative_texture_effect_turb.rs:33-138,
// generative_texture_effect_layered.rs:63-381), the per-frame rewrite of the effects' output textures.
//
// The host keeps the scalar per-frame work (the sine shift tables and the layer functions of time); the
// GPU runs every output texel of every group in one grid-stride launch. A group is one output mip and
// its passes: a turbulence gather, or the layers of a layered animation applied in layer order to the
// texel in registers (one read of each layer texel, one read and one write of the output texel).
// Integer colour arithmetic is ColorVecI's: wrapping i32 lanes, arithmetic shifts, (v as u32).min(255).
#include "sw_kernels.cuh"

namespace swgpu
{
namespace
{

__device__ __forceinline__ int32_t rem_euclid(int32_t a, int32_t m)
{
	const int32_t r = a % m;
	return r < 0 ? r + m : r;
}

// One layer applied to the output texel (apply_texture_layer_impl_2, layered.rs:258-381): texels are
// TextureElement, diffuse Color32 in the low half, packed normal/roughness in the high half.
__device__ __forceinline__ uint64_t apply_layer(uint64_t dst, uint64_t texel, uint32_t blend, bool modulate, const CI& light)
{
	const uint32_t td = uint32_t(texel), dd = uint32_t(dst);
	const uint64_t normal_of_texel = texel & 0xFFFFFFFF00000000ull;
	CI src;
	if (modulate)
	{
		const CI t = ci_from_c32(td);
#pragma unroll
		for (int i = 0; i < 4; ++i) src.v[i] = wmul(t.v[i], light.v[i]) >> 8;
	}
	else
		src = ci_from_c32(td);
	switch (blend)
	{
	case SW_BLEND_NONE:
		return modulate ? (normal_of_texel | ci_to_c32(src)) : texel;
	case SW_BLEND_AVERAGE:
	{
		uint32_t r;
		if (modulate)
		{
			const CI d = ci_from_c32(dd);
			CI s;
#pragma unroll
			for (int i = 0; i < 4; ++i) s.v[i] = wadd(src.v[i], d.v[i]) >> 1;
			r = ci_to_c32(s);
		}
		else
			r = (((dd ^ td) & 0xFEFEFEFEu) >> 1) + (dd & td); // Color32::get_average
		return (dst & 0xFFFFFFFF00000000ull) | r;
	}
	case SW_BLEND_ADDITIVE:
	{
		const CI d = ci_from_c32(dd);
		CI s;
#pragma unroll
		for (int i = 0; i < 4; ++i) s.v[i] = wadd(src.v[i], d.v[i]);
		return (dst & 0xFFFFFFFF00000000ull) | ci_to_c32(s);
	}
	case SW_BLEND_ALPHA_TEST:
		if ((td & 0xFF000000u) > 0x7F000000u) return modulate ? (normal_of_texel | ci_to_c32(src)) : texel;
		return dst;
	default: // SW_BLEND_ALPHA_BLEND
	{
		const int32_t alpha = int32_t(td >> 24);
		const CI d = ci_from_c32(dd);
		CI s;
#pragma unroll
		for (int i = 0; i < 4; ++i) s.v[i] = wadd(wmul(src.v[i], alpha), wmul(d.v[i], wsub(255, alpha))) >> 8;
		return (dst & 0xFFFFFFFF00000000ull) | ci_to_c32(s);
	}
	}
}

__global__ void __launch_bounds__(256) texture_effects_kernel(TextureEffectArgs a)
{
	const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
	for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < a.total_texels; t += stride)
	{
		// the group holding texel t (groups are few: a binary search over their first texels)
		uint32_t lo = 0, hi = a.num_groups - 1;
		while (lo < hi)
		{
			const uint32_t mid = (lo + hi + 1) >> 1;
			if (a.groups[mid].first_texel <= t) lo = mid;
			else hi = mid - 1;
		}
		const TextureEffectGroup& g = a.groups[lo];
		const uint32_t i = uint32_t(t - g.first_texel);
		const int32_t w = int32_t(g.width), x = int32_t(i % g.width), y = int32_t(i / g.width);
		const SwTexturePass& first = a.passes[g.first_pass];
		if (first.kind & SW_TEXPASS_TURB)
		{
			const int32_t* s = a.shifts + first.shifts_offset;
			const int32_t su = (x + __ldg(s + y)) & (w - 1);
			const int32_t sv = (y + __ldg(s + x)) & int32_t(g.height - 1);
			const uint64_t at = uint64_t(sv) * uint32_t(w) + uint32_t(su);
			if (first.kind & SW_TEXPASS_EMISSIVE)
				a.emissive[g.dst_offset + i] = __ldg(a.emissive + g.src_offset + at);
			else
				a.texels[g.dst_offset + i] = __ldg(reinterpret_cast<const unsigned long long*>(a.texels) + g.src_offset + at);
			continue;
		}
		uint64_t v = a.texels[g.dst_offset + i];
		for (uint32_t p = g.first_pass; p < g.first_pass + g.num_passes; ++p)
		{
			const SwTexturePass& pass = a.passes[p];
			const TextureEffectLayer& l = a.layers[p];
			if (l.skip) continue;
			const int32_t sv = rem_euclid(pass.shift[1] + y, int32_t(l.src_height));
			const int32_t su = rem_euclid(pass.shift[0] + x, int32_t(l.src_width));
			const uint64_t texel = __ldg(reinterpret_cast<const unsigned long long*>(a.texels) + l.src_offset +
				uint64_t(sv) * l.src_width + uint32_t(su));
			v = apply_layer(v, texel, pass.blending_mode, l.modulate != 0, CI{{l.light[0], l.light[1], l.light[2], 0}});
		}
		a.texels[g.dst_offset + i] = v;
	}
}

} // namespace

int launch_texture_effects(const TextureEffectArgs& a, cudaStream_t stream)
{
	if (a.total_texels == 0 || a.num_groups == 0) return 0;
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const uint64_t want = (a.total_texels + 255) / 256;
	const unsigned blocks = unsigned(std::min<uint64_t>(want, uint64_t(std::max(sms, 1)) * 8));
	texture_effects_kernel<<<blocks, 256, 0, stream>>>(a);
	return int(cudaGetLastError());
}

} // namespace swgpu
