// Simulated generative texture effects on the GPU: the per-word and per-texel work of
// GenerativeTextureEffectWater (src/square_wheel/generative_texture_effect_water.rs:57-682) and
// GenerativeTextureEffectFire (generative_texture_effect_fire.rs:62-566), and the run-time mip rebuilds
// (build_texture_mip / build_texture_lite_mip, textures.rs:309-415).
//
// The host keeps the scalar work of every step (time functions, the random engine, line rasterisation
// of the sources, particles) and hands over point lists; the wave fields and heat maps stay resident in
// the context's simulation state, ping-ponged between two buffers per effect. A launch runs one phase of
// every effect at once (sources, field step, texture, one mip level), grid-stride over the union of the
// passes' items with a binary search over the groups, as the texture-effect kernel does.
// Float arithmetic is plain IEEE single precision without contraction (the build's --fmad=false), in the
// reference's operation order.
#include "sw_kernels.cuh"

namespace swgpu
{
namespace
{

// PackedNormalRoughness::pack with the generic pack_f32x4_into_bytes (textures.rs:33-39,
// fast_math.rs:419-427): (v * 127).max(-127).min(127) as i32, low bytes.
__device__ __forceinline__ uint32_t pack_normal_roughness(float x, float y, float z, float r)
{
	const float v[4] = {x, y, z, r};
	uint32_t out = 0;
#pragma unroll
	for (int i = 0; i < 4; ++i)
	{
		const float s = fminf(fmaxf(__fmul_rn(v[i], 127.0f), -127.0f), 127.0f);
		out |= (uint32_t(__float2int_rz(s)) & 0xFFu) << (8 * i);
	}
	return out;
}

// upack_bytes_into_f32x4 (fast_math.rs:430-438) with scale 1 / 127
__device__ __forceinline__ float unpack_byte(uint32_t p, int i)
{
	return __fmul_rn(float(int32_t(p << (24 - 8 * i)) >> 24), 1.0f / 127.0f);
}

// Color32::get_average_4 (src/common/color.rs:51-71)
__device__ __forceinline__ uint32_t average4(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
	const uint32_t s0 = (a & 0xFFu) + (b & 0xFFu) + (c & 0xFFu) + (d & 0xFFu);
	const uint32_t s1 = (a & 0xFF00u) + (b & 0xFF00u) + (c & 0xFF00u) + (d & 0xFF00u);
	const uint32_t s2 = (a & 0xFF0000u) + (b & 0xFF0000u) + (c & 0xFF0000u) + (d & 0xFF0000u);
	const uint32_t s3 = ((a & 0xFF000000u) >> 2) + ((b & 0xFF000000u) >> 2) + ((c & 0xFF000000u) >> 2) + ((d & 0xFF000000u) >> 2);
	return (s0 >> 2) | ((s1 >> 2) & 0xFF00u) | ((s2 >> 2) & 0xFF0000u) | (s3 & 0xFF000000u);
}

// One heat map word of update_heat_map: ((sum * attenuation_i) >> 20) as u8
__device__ __forceinline__ uint32_t heat_of(uint32_t sum, uint32_t att) { return ((sum * att) >> 20) & 0xFFu; }

__device__ void water_points(const SimArgs& a, const SwSimPass& p, uint32_t i)
{
	const SwSimPoint* pts = a.points + p.first_point;
	const uint32_t addr = pts[i].address;
	if (i > 0 && pts[i - 1].address == addr) return; // a run of equal addresses is one thread's, in order
	float* cur = reinterpret_cast<float*>(a.state + p.state_src);
	float* old = reinterpret_cast<float*>(a.state + p.state_dst);
	float c = cur[addr], o = old[addr];
	for (uint32_t j = i; j < p.num_points && pts[j].address == addr; ++j)
	{
		const float v = __uint_as_float(pts[j].value);
		c = __fadd_rn(c, v);
		o = __fsub_rn(o, v);
	}
	cur[addr] = c;
	old[addr] = o;
}

__device__ void water_step(const SimArgs& a, const SwSimPass& p, uint32_t i)
{
	const uint32_t w = 1u << p.size_log2[0], h = 1u << p.size_log2[1];
	const uint32_t x = i & (w - 1), y = i >> p.size_log2[0];
	const float* src = reinterpret_cast<const float*>(a.state + p.state_src);
	float* dst = reinterpret_cast<float*>(a.state + p.state_dst);
	const uint32_t row = y << p.size_log2[0];
	const float xm = src[row + ((x - 1) & (w - 1))], xp = src[row + ((x + 1) & (w - 1))];
	const float ym = src[(((y - 1) & (h - 1)) << p.size_log2[0]) + x], yp = src[(((y + 1) & (h - 1)) << p.size_log2[0]) + x];
	const float sum = __fadd_rn(__fadd_rn(__fadd_rn(xm, xp), ym), yp);
	dst[i] = __fmul_rn(__fsub_rn(__fmul_rn(sum, 0.5f), dst[i]), __uint_as_float(p.param));
}

__device__ void fire_step_fast(const SimArgs& a, const SwSimPass& p, uint32_t i)
{
	const uint32_t w = 1u << p.size_log2[0], h = 1u << p.size_log2[1];
	const uint32_t x = i & (w - 1), y = i >> p.size_log2[0];
	const uint32_t* src = a.state + p.state_src;
	uint32_t* dst = a.state + p.state_dst;
	if (y == h - 1)
	{
		dst[i] = 0;
		return;
	}
	const uint32_t r1 = (y + 1) << p.size_log2[0];
	const uint32_t r2 = (y + 2 < h ? y + 2 : y + 1) << p.size_log2[0]; // the line before last reads y + 1 twice
	const uint32_t sum = src[r1 + ((x - 1) & (w - 1))] + src[r1 + x] + src[r1 + ((x + 1) & (w - 1))] + src[r2 + x];
	dst[i] = heat_of(sum, p.param);
}

// The slow form: each row left to right, reading the row's already-updated left neighbour (and, at the
// right border, its updated first word) - a sequential recurrence per row, one thread per row.
__device__ void fire_step_slow(const SimArgs& a, const SwSimPass& p, uint32_t y)
{
	const uint32_t w = 1u << p.size_log2[0], h = 1u << p.size_log2[1];
	const uint32_t* src = a.state + p.state_src + (uint64_t(y) << p.size_log2[0]);
	uint32_t* dst = a.state + p.state_dst + (uint64_t(y) << p.size_log2[0]);
	if (y == h - 1)
	{
		for (uint32_t x = 0; x < w; ++x) dst[x] = 0;
		return;
	}
	const uint32_t* below = src + w;
	const uint32_t first = heat_of(src[w - 1] + src[0] + src[1] + below[0], p.param);
	dst[0] = first;
	uint32_t prev = first;
	for (uint32_t x = 1; x + 1 < w; ++x)
	{
		prev = heat_of(prev + src[x] + src[x + 1] + below[x], p.param);
		dst[x] = prev;
	}
	dst[w - 1] = heat_of(prev + src[w - 1] + first + below[w - 1], p.param);
}

__device__ __forceinline__ uint32_t colour_image(const SimArgs& a, const SimGroup& g, uint32_t u, uint32_t v, uint32_t w, uint32_t h)
{
	// resize_image (textures.rs:164-181) of the source's diffuse: nearest, integer scaling
	const uint32_t sx = u * g.src_width / w, sy = v * g.src_height / h;
	return uint32_t(a.texels[g.src_offset + uint64_t(sy) * g.src_width + sx]);
}

__device__ void water_texture(const SimArgs& a, const SimGroup& g, const SwSimPass& p, uint32_t i)
{
	const uint32_t w = 1u << p.size_log2[0], h = 1u << p.size_log2[1];
	const uint32_t x = i & (w - 1), y = i >> p.size_log2[0];
	const float* f = reinterpret_cast<const float*>(a.state + p.state_src);
	const uint32_t row = y << p.size_log2[0];
	const float dx = __fsub_rn(f[row + ((x + 1) & (w - 1))], f[row + ((x - 1) & (w - 1))]);
	const float dy = __fsub_rn(f[(((y + 1) & (h - 1)) << p.size_log2[0]) + x], f[(((y - 1) & (h - 1)) << p.size_log2[0]) + x]);
	// Vec3f::new(dx, dy, 1).normalize(): v * (1 / sqrt((x * x + y * y) + z * z))
	const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), 1.0f));
	const float inv = __fdiv_rn(1.0f, len);
	const float nx = __fmul_rn(dx, inv), ny = __fmul_rn(dy, inv), nz = __fmul_rn(1.0f, inv);
	const uint32_t packed = pack_normal_roughness(nx, ny, nz, __uint_as_float(p.param));
	uint64_t* out = a.texels + g.dst_offset + i;
	const uint32_t mode = p.flags >> SW_SIM_COLOR_MODE_SHIFT;
	uint32_t diffuse;
	if (mode <= 1)
	{
		if (!(p.flags & SW_SIM_WATER_INIT_DIFFUSE))
		{
			// keep the diffuse written by the first generation: store the normal half alone
			reinterpret_cast<uint32_t*>(out)[1] = packed;
			return;
		}
		diffuse = mode == 0 ? p.base_color : colour_image(a, g, x, y, w, h);
	}
	else
	{
		const int32_t du = __float2int_rz(__fmul_rn(nx, 16.0f));
		const uint32_t u = uint32_t(int32_t(x) + du) & (w - 1);
		if (mode == 2)
		{
			const int32_t dv = __float2int_rz(__fmul_rn(ny, 16.0f));
			diffuse = colour_image(a, g, u, uint32_t(int32_t(y) + dv) & (h - 1), w, h);
		}
		else
			diffuse = colour_image(a, g, u, y, w, h);
	}
	*out = (uint64_t(packed) << 32) | diffuse;
}

__device__ void texture_mip(const SimArgs& a, const SimGroup& g, const SwSimPass& p, uint32_t i)
{
	const uint32_t dw = g.src_width >> 1;
	const uint32_t x = i % dw, y = i / dw;
	const uint64_t* s0 = a.texels + g.src_offset + uint64_t(2 * y) * g.src_width + 2 * x;
	const uint64_t* s1 = s0 + g.src_width;
	const uint64_t q[4] = {s0[0], s1[0], s0[1], s1[1]}; // p00, p01, p10, p11
	const uint32_t diffuse = average4(uint32_t(q[0]), uint32_t(q[1]), uint32_t(q[2]), uint32_t(q[3]));
	float nx = 0.0f, ny = 0.0f, nz = 0.0f, rs = 0.0f;
#pragma unroll
	for (int k = 0; k < 4; ++k)
	{
		const uint32_t pk = uint32_t(q[k] >> 32);
		if (k == 0)
		{
			nx = unpack_byte(pk, 0);
			ny = unpack_byte(pk, 1);
			nz = unpack_byte(pk, 2);
			rs = unpack_byte(pk, 3);
		}
		else
		{
			nx = __fadd_rn(nx, unpack_byte(pk, 0));
			ny = __fadd_rn(ny, unpack_byte(pk, 1));
			nz = __fadd_rn(nz, unpack_byte(pk, 2));
			rs = __fadd_rn(rs, unpack_byte(pk, 3));
		}
	}
	// textures.rs:342-360: normal = sum / max(|sum|, 1e-6); roughness grows with the normals' spread
	const float len = fmaxf(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz))), 0.000001f);
	const float deviation = __fdiv_rn(__fsub_rn(1.0f, __fmul_rn(len, 0.25f)), __fsub_rn(1.0f, 0.5f));
	const float rough = fminf(fmaxf(__fadd_rn(__fmul_rn(rs, 0.25f), deviation), 1.0f / 126.0f), 1.0f);
	const uint32_t packed = pack_normal_roughness(__fdiv_rn(nx, len), __fdiv_rn(ny, len), __fdiv_rn(nz, len), rough);
	a.texels[g.dst_offset + i] = (uint64_t(packed) << 32) | diffuse;
	(void)p;
}

__global__ void __launch_bounds__(256) simulation_kernel(SimArgs a)
{
	const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
	for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < a.total_items; t += stride)
	{
		uint32_t lo = 0, hi = a.num_groups - 1;
		while (lo < hi)
		{
			const uint32_t mid = (lo + hi + 1) >> 1;
			if (a.groups[mid].first_item <= t) lo = mid;
			else hi = mid - 1;
		}
		const SimGroup& g = a.groups[lo];
		const SwSimPass& p = a.passes[g.pass];
		const uint32_t i = uint32_t(t - g.first_item);
		switch (p.kind)
		{
		case SW_SIM_WATER_POINTS: water_points(a, p, i); break;
		case SW_SIM_WATER_STEP: water_step(a, p, i); break;
		case SW_SIM_FIRE_STEP:
			if (p.flags & SW_SIM_FIRE_SLOW) fire_step_slow(a, p, i);
			else fire_step_fast(a, p, i);
			break;
		case SW_SIM_FIRE_POINTS:
		{
			const SwSimPoint& q = a.points[p.first_point + i];
			atomicMax(a.state + p.state_dst + q.address, q.value);
			break;
		}
		case SW_SIM_WATER_TEXTURE: water_texture(a, g, p, i); break;
		case SW_SIM_FIRE_TEXTURE:
			a.emissive[g.dst_offset + i] = a.points[p.first_point + (a.state[p.state_src + i] & 0xFFu)].value;
			break;
		case SW_SIM_TEXTURE_MIP: texture_mip(a, g, p, i); break;
		default: // SW_SIM_EMISSIVE_MIP
		{
			const uint32_t dw = g.src_width >> 1;
			const uint32_t x = i % dw, y = i / dw;
			const uint32_t* s0 = a.emissive + g.src_offset + uint64_t(2 * y) * g.src_width + 2 * x;
			const uint32_t* s1 = s0 + g.src_width;
			a.emissive[g.dst_offset + i] = average4(s0[0], s1[0], s0[1], s1[1]);
			break;
		}
		}
	}
}

} // namespace

int launch_simulation(const SimArgs& a, cudaStream_t stream)
{
	if (a.total_items == 0 || a.num_groups == 0) return 0;
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const uint64_t want = (a.total_items + 255) / 256;
	const unsigned blocks = unsigned(std::min<uint64_t>(want, uint64_t(std::max(sms, 1)) * 8));
	simulation_kernel<<<blocks, 256, 0, stream>>>(a);
	return int(cudaGetLastError());
}

} // namespace swgpu
