// Surface builder for the GB300 path: every visible polygon surface of a frame in one persistent
// launch.
//
// Replaces build_polygons_surfaces' per-polygon work (src/square_wheel/partial_renderer.rs:1682-1831):
// build_surface_impl_6_static_params (src/square_wheel/surfaces.rs:433-852) followed by the emissive
// layer mix_surface_with_texture (src/square_wheel/surfaces.rs:903-971), fused in one pass.
//
// Work decomposition: the frame's surfaces form one flat texel index space (prefix sums of surface
// areas, in descriptor order). A grid of (#SMs x resident blocks) threads strides over it, so surfaces
// from 4x4 to 512x512 texels share one launch without tail effects. Each thread owns one output texel:
// it finds its surface by binary search over the prefix array (held in L1), rebuilds the reference's
// row-interpolated lightmap line entries it needs (the two vertical mixes of the line buffer and the
// horizontal mix, in the reference's operation order), evaluates lighting and stores the texel.
// Neighbouring threads read neighbouring TextureElements and share lightmap elements, so texture reads
// and surface writes are coalesced and lightmap reads are L1 broadcasts.
#include "sw_kernels.cuh"

namespace swgpu
{

namespace
{

const float NORMAL_UNPACK_SCALE = 1.0f / 127.0f;
constexpr float PI_F = 3.14159265358979323846f;
// Specular lobe constants, src/square_wheel/surfaces.rs:1108-1110 (f32 constant arithmetic).
constexpr float SPEC_A = 2.0f * PI_F / 2.645751311f;
constexpr float SPEC_B = PI_F * 2.645751311f / 2.0f;
constexpr float DIELECTRIC_ZERO_REFLECTIVITY = 0.04f;
constexpr float DIELECTRIC_AVERAGE_REFLECTIVITY = DIELECTRIC_ZERO_REFLECTIVITY * 3.0f;
constexpr float METAL_AVERAGE_SCHLICK_FACTOR = 0.5f;

__device__ __forceinline__ float specular_intensity(float angle_cos, float inv_roughness)
{
	float x = fmul(fsub(angle_cos, 1.0f), inv_roughness);
	return fmul(inv_fast(mad2(fmul(x, x), SPEC_B, SPEC_A)), inv_roughness);
}
__device__ __forceinline__ float fresnel_factor_base(float c)
{
	float omc = fmaxf(fsub(1.0f, c), 0.0f);
	float omc2 = fmul(omc, omc);
	return fmul(fmul(omc2, omc2), omc);
}
__device__ __forceinline__ float specular_k(int spec, float f, float roughness)
{
	if (spec == 1)
	{
		float fresnel = mad2(f, 1.0f - DIELECTRIC_ZERO_REFLECTIVITY, DIELECTRIC_ZERO_REFLECTIVITY);
		return mad2(fresnel, fsub(1.0f, roughness), fmul(DIELECTRIC_AVERAGE_REFLECTIVITY, roughness));
	}
	return mad2(f, fsub(1.0f, roughness), fmul(METAL_AVERAGE_SCHLICK_FACTOR, roughness));
}

struct Lm
{
	float amb[3];
	V3 dir;
	float dev;
	float col[3];
};

template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lm_load(const SurfaceKernelArgs& a, uint64_t index)
{
	Lm e;
	if (DIRECTIONAL)
	{
		const float* p = reinterpret_cast<const float*>(a.directional_lightmaps + index);
		e.amb[0] = __ldg(p + 0);
		e.amb[1] = __ldg(p + 1);
		e.amb[2] = __ldg(p + 2);
		e.dir = mkv3(__ldg(p + 3), __ldg(p + 4), __ldg(p + 5));
		e.dev = __ldg(p + 6);
		e.col[0] = __ldg(p + 7);
		e.col[1] = __ldg(p + 8);
		e.col[2] = __ldg(p + 9);
	}
	else
	{
		const float* p = a.lightmaps + index * 3;
		e.amb[0] = __ldg(p + 0);
		e.amb[1] = __ldg(p + 1);
		e.amb[2] = __ldg(p + 2);
	}
	return e;
}

// LightmapElementOps::mix(a, b, ratio) = a*ratio + b*(1-ratio), surfaces.rs:996-1071
template <bool DIRECTIONAL>
__device__ __forceinline__ Lm lm_mix(const Lm& a, const Lm& b, float ratio)
{
	const float omr = fsub(1.0f, ratio);
	Lm r;
#pragma unroll
	for (int i = 0; i < 3; ++i) r.amb[i] = mad2(a.amb[i], ratio, fmul(b.amb[i], omr));
	if (DIRECTIONAL)
	{
		r.dir = mkv3(mad2(a.dir.x, ratio, fmul(b.dir.x, omr)), mad2(a.dir.y, ratio, fmul(b.dir.y, omr)),
			mad2(a.dir.z, ratio, fmul(b.dir.z, omr)));
		r.dev = mad2(a.dev, ratio, fmul(b.dev, omr));
#pragma unroll
		for (int i = 0; i < 3; ++i) r.col[i] = mad2(a.col[i], ratio, fmul(b.col[i], omr));
	}
	return r;
}

__device__ __forceinline__ int32_t rem_euclid(int32_t a, int32_t b)
{
	int32_t r = a % b;
	return r < 0 ? r + b : r;
}

// Lighting of one texel for one lightmap kind; returns the ColorVec before conversion.
template <bool DIRECTIONAL>
__device__ __forceinline__ CV shade_texel(const SurfaceKernelArgs& a, const SwSurfaceDesc& s, uint32_t tex_flags,
	uint64_t texel, uint32_t u, uint32_t v)
{
	const bool use_normal_map = (tex_flags & SW_TEX_HAS_NORMAL_MAP) != 0;
	const int spec = (tex_flags & SW_TEX_HAS_NON_ONE_ROUGHNESS) ? ((tex_flags & SW_TEX_IS_METAL) ? 2 : 1) : 0;

	const V3 u_vec = mkv3(s.basis_u[0], s.basis_u[1], s.basis_u[2]);
	const V3 v_vec = mkv3(s.basis_v[0], s.basis_v[1], s.basis_v[2]);
	const V3 bnormal = mkv3(s.basis_normal[0], s.basis_normal[1], s.basis_normal[2]);
	// start_pos = start + u*(tc0+0.5) + v*(tc1+0.5), surfaces.rs:456-457
	const V3 start_pos = v3add(v3add(mkv3(s.basis_start[0], s.basis_start[1], s.basis_start[2]),
								   v3scale(u_vec, fadd(float(s.tc_start[0]), 0.5f))),
		v3scale(v_vec, fadd(float(s.tc_start[1]), 0.5f)));
	const V3 pos = v3sma(u_vec, float(u), v3sma(v_vec, float(v), start_pos));

	V3 tn = mkv3(0.0f, 0.0f, 1.0f);
	float rough = 0.0f;
	const int32_t packed = int32_t(uint32_t(texel >> 32));
	if (use_normal_map)
	{
		tn = mkv3(fmul(float(int32_t(uint32_t(packed) << 24) >> 24), NORMAL_UNPACK_SCALE),
			fmul(float(int32_t(uint32_t(packed) << 16) >> 24), NORMAL_UNPACK_SCALE),
			fmul(float(int32_t(uint32_t(packed) << 8) >> 24), NORMAL_UNPACK_SCALE));
		rough = fmul(float(packed >> 24), NORMAL_UNPACK_SCALE);
	}
	else if (spec != 0)
		rough = fmul(float(packed >> 24), NORMAL_UNPACK_SCALE);

	V3 u_norm = mkv3(0, 0, 0), v_norm = mkv3(0, 0, 0);
	if (spec != 0 || (use_normal_map && s.num_lights > 0))
	{
		u_norm = v3scale(u_vec, inv_sqrt_fast(fmaxf(v3dot(u_vec, u_vec), MIN_POSITIVE_VALUE)));
		v_norm = v3scale(v_vec, inv_sqrt_fast(fmaxf(v3dot(v_vec, v_vec), MIN_POSITIVE_VALUE)));
	}
	const V3 cam = mkv3(a.cam_pos[0], a.cam_pos[1], a.cam_pos[2]);

	CV albedo = cv_zero(); // total_light_albedo_modulated
	CV direct = cv_zero(); // total_light_direct
	if (s.lightmap_offset != SW_NO_LIGHTMAP)
	{
		const uint32_t log2 = s.lightmap_scale_log2;
		const float inv_scale = __fdiv_rn(1.0f, float(1u << log2));
		const float k_shift = fmul(0.5f, inv_scale);
		const uint32_t mask = (1u << log2) - 1u;
		const uint32_t base_v = v + s.lightmap_tc_shift[1];
		const uint32_t lv = base_v >> log2;
		const float kv = mad2(float(base_v & mask), inv_scale, k_shift);
		const uint32_t base_u = u + s.lightmap_tc_shift[0];
		const uint32_t lu = base_u >> log2;
		const float ku = mad2(float(base_u & mask), inv_scale, k_shift);
		const uint64_t row0 = uint64_t(s.lightmap_offset) + uint64_t(lv) * s.lightmap_size[0];
		const uint64_t row1 = row0 + s.lightmap_size[0];
		// line_lightmap[lu] and [lu + 1] of the reference's row buffer, then the horizontal mix.
		const Lm line0 = lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu), lm_load<DIRECTIONAL>(a, row0 + lu), kv);
		const Lm line1 =
			lm_mix<DIRECTIONAL>(lm_load<DIRECTIONAL>(a, row1 + lu + 1), lm_load<DIRECTIONAL>(a, row0 + lu + 1), kv);
		const Lm l = lm_mix<DIRECTIONAL>(line1, line0, ku);

		if (spec == 0)
		{
			albedo = cv_rgb(l.amb, 1.0f);
			if (DIRECTIONAL)
			{
				float dot = use_normal_map ? fmaxf(v3dot(l.dir, tn), 0.0f) : l.dir.z;
				albedo = cv_sma(cv_rgb(l.col, 0.0f), dot, albedo);
			}
		}
		else
		{
			const V3 normal = use_normal_map ? tn : mkv3(0.0f, 0.0f, 1.0f);
			const V3 to_cam = v3sub(cam, pos);
			const V3 to_cam_ts = mkv3(v3dot(to_cam, u_norm), v3dot(to_cam, v_norm), v3dot(to_cam, bnormal));
			const float ndot = v3dot(to_cam_ts, normal);
			const V3 refl = v3sub(v3scale(normal, fmul(2.0f, ndot)), to_cam_ts);
			const float refl_len2 = fmaxf(v3dot(refl, refl), MIN_POSITIVE_VALUE);
			const float angle_cos = fmaxf(fmul(ndot, inv_sqrt_fast(refl_len2)), 0.0f);
			const float sk = specular_k(spec, fresnel_factor_base(angle_cos), rough);
			const float omsk = fsub(1.0f, sk);
			const CV constant = cv_rgb(l.amb, 0.0f);
			albedo = cv_scale(constant, omsk);
			direct = cv_scale(constant, sk);
			albedo.a = 1.0f;
			if (DIRECTIONAL)
			{
				const float dir_len2 = v3dot(l.dir, l.dir);
				const float dir_len = fmul(dir_len2, inv_sqrt_fast(dir_len2));
				const float rl_cos = fmul(v3dot(refl, l.dir), inv_sqrt_fast(fmul(refl_len2, dir_len2)));
				const float inv_rc = fmaxf(inv_fast(fadd(rough, l.dev)), 0.75f);
				const float si = specular_intensity(rl_cos, inv_rc);
				const CV dcol = cv_rgb(l.col, 0.0f);
				if (spec == 1)
				{
					const float di = fmaxf(v3dot(l.dir, tn), 0.0f);
					albedo = cv_sma(dcol, fmul(di, omsk), albedo);
					direct = cv_sma(dcol, fmul(fmul(si, sk), dir_len), direct);
				}
				else
				{
					const float sf = fmul(si, dir_len);
					albedo = cv_sma(dcol, fmul(omsk, sf), albedo);
					direct = cv_sma(dcol, fmul(sk, sf), direct);
				}
			}
		}
	}

	if (s.num_lights > 0)
	{
		V3 normal = bnormal;
		if (use_normal_map)
			normal = mkv3(mad2(tn.x, u_norm.x, mad2(tn.y, v_norm.x, fmul(tn.z, bnormal.x))),
				mad2(tn.x, u_norm.y, mad2(tn.y, v_norm.y, fmul(tn.z, bnormal.y))),
				mad2(tn.x, u_norm.z, mad2(tn.y, v_norm.z, fmul(tn.z, bnormal.z))));
		V3 refl = mkv3(0.0f, 0.0f, 0.0f);
		float refl_len2 = MIN_POSITIVE_VALUE;
		float sk = 0.0f, inv_rough = 0.0f;
		if (spec != 0)
		{
			const V3 to_cam = v3sub(cam, pos);
			const float ndot = v3dot(to_cam, normal);
			refl = v3sub(v3scale(normal, fmul(2.0f, ndot)), to_cam);
			refl_len2 = fmaxf(v3dot(refl, refl), MIN_POSITIVE_VALUE);
			const float angle_cos = fmaxf(fmul(ndot, inv_sqrt_fast(refl_len2)), 0.0f);
			sk = specular_k(spec, fresnel_factor_base(angle_cos), rough);
			inv_rough = inv_fast(rough);
		}
		for (uint32_t li = 0; li < s.num_lights; ++li)
		{
			const SwLight& L = a.lights[s.lights[li]];
			const V3 to_light = v3sub(mkv3(L.position[0], L.position[1], L.position[2]), pos);
			const float tl_len2 = fmaxf(v3dot(to_light, to_light), MIN_POSITIVE_VALUE);
			const float sdf = fmul(1.0f, fmaxf(fsub(inv_fast(tl_len2), L.inv_square_radius), 0.0f));
			float di = 0.0f;
			if (spec != 2) di = fmaxf(fmul(v3dot(normal, to_light), inv_sqrt_fast(tl_len2)), 0.0f);
			float si = 0.0f;
			if (spec != 0)
				si = specular_intensity(fmul(v3dot(refl, to_light), inv_sqrt_fast(fmul(refl_len2, tl_len2))), inv_rough);
			const CV lc = cv_rgb(L.color, 0.0f);
			if (spec == 0)
				albedo = cv_sma(lc, fmul(di, sdf), albedo);
			else if (spec == 1)
			{
				albedo = cv_sma(lc, fmul(fmul(di, fsub(1.0f, sk)), sdf), albedo);
				direct = cv_sma(lc, fmul(fmul(si, sk), sdf), direct);
			}
			else
			{
				const float sisdf = fmul(si, sdf);
				albedo = cv_sma(lc, fmul(fsub(1.0f, sk), sisdf), albedo);
				direct = cv_sma(lc, fmul(sk, sisdf), direct);
			}
		}
	}

	CV result = cv_mul(cv_from_c32(uint32_t(texel)), albedo);
	if (spec != 0) result = cv_sma(direct, 255.0f, result);
	return result;
}

template <class P>
__device__ __forceinline__ typename P::T emissive_mix(const SurfaceKernelArgs& a, const SwSurfaceDesc& s, uint32_t u,
	uint32_t v, typename P::T dst, bool additive)
{
	const SwEmissiveMip em = a.emissive_mips[s.emissive_mip];
	const int32_t w = int32_t(em.width), h = int32_t(em.height);
	const int32_t sv = rem_euclid(s.tc_start[1] + int32_t(v), h);
	const int32_t su = rem_euclid(s.tc_start[0] + int32_t(u), w);
	const uint32_t texel = __ldg(a.emissive_pixels + em.offset + uint64_t(sv) * em.width + uint32_t(su));
	// ColorVecI::from_color_f32x3([l0*256, l1*256, l2*256]) -> [b, g, r, 0], truncating conversion.
	const int32_t lb = __float2int_rz(fmul(s.emissive_light[2], 256.0f));
	const int32_t lg = __float2int_rz(fmul(s.emissive_light[1], 256.0f));
	const int32_t lr = __float2int_rz(fmul(s.emissive_light[0], 256.0f));
	const CI t = ci_from_c32(texel);
	CI m{{wmul(t.v[0], lb) >> 8, wmul(t.v[1], lg) >> 8, wmul(t.v[2], lr) >> 8, 0}};
	if (!additive) return P::from_ci(m);
	const CI d = P::to_ci(dst);
#pragma unroll
	for (int i = 0; i < 4; ++i) m.v[i] = wadd(m.v[i], d.v[i]);
	return P::from_ci(m);
}

template <class P, bool DIRECTIONAL>
__global__ void __launch_bounds__(256) surf_build_kernel(SurfaceKernelArgs a)
{
	typedef typename P::T T;
	T* arena = static_cast<T*>(a.arena);
	const uint64_t total = a.total_work;
	const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
	for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += stride)
	{
		// Surface owning work item t: last s with prefix[s] <= t.
		uint32_t lo = 0, hi = a.num_surfaces; // invariant: prefix[lo] <= t < prefix[hi]
		while (hi - lo > 1)
		{
			uint32_t mid = (lo + hi) >> 1;
			if (__ldg(a.work_prefix + mid) <= t)
				lo = mid;
			else
				hi = mid;
		}
		const SwSurfaceDesc& s = a.surfaces[lo];
		const uint64_t local = t - __ldg(a.work_prefix + lo);
		const uint32_t w = s.size[0];
		const uint32_t v = uint32_t(local / w);
		const uint32_t u = uint32_t(local - uint64_t(v) * w);

		T out = T(0);
		const bool diffuse_layer = (s.flags & SW_SURF_DIFFUSE_LAYER) != 0;
		if (diffuse_layer)
		{
			const SwTextureMip tm = a.texture_mips[s.texture_mip];
			const int32_t sv = rem_euclid(s.tc_start[1] + int32_t(v), int32_t(tm.height));
			const int32_t su = rem_euclid(s.tc_start[0] + int32_t(u), int32_t(tm.width));
			const uint64_t texel = __ldg(reinterpret_cast<const unsigned long long*>(a.texels) + tm.offset +
				uint64_t(sv) * tm.width + uint32_t(su));
			out = P::from_cv(shade_texel<DIRECTIONAL>(a, s, tm.flags, texel, u, v));
		}
		if (s.emissive_mip != SW_NO_EMISSIVE) out = emissive_mix<P>(a, s, u, v, out, diffuse_layer);
		arena[s.out_offset + local] = out;
	}
}

} // namespace

int launch_surface_build(const SurfaceKernelArgs& args, uint32_t pixel_format, int num_sms, cudaStream_t stream)
{
	if (args.total_work == 0) return 0;
	const int threads = 256;
	uint64_t blocks_needed = (args.total_work + threads - 1) / threads;
	uint64_t blocks_max = uint64_t(num_sms) * 8;
	unsigned blocks = unsigned(blocks_needed < blocks_max ? blocks_needed : blocks_max);
	if (pixel_format == SW_PIXEL_C64)
	{
		if (args.directional)
			surf_build_kernel<PixC64, true><<<blocks, threads, 0, stream>>>(args);
		else
			surf_build_kernel<PixC64, false><<<blocks, threads, 0, stream>>>(args);
	}
	else
	{
		if (args.directional)
			surf_build_kernel<PixC32, true><<<blocks, threads, 0, stream>>>(args);
		else
			surf_build_kernel<PixC32, false><<<blocks, threads, 0, stream>>>(args);
	}
	return int(cudaGetLastError());
}

} // namespace swgpu
