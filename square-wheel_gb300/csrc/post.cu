// HDR postprocessor and frame upscaler for the GB300 path.
//
// Replaces Postprocessor::perform_postprocessing (src/square_wheel/postprocessor.rs:68-204): bloom
// downscale with exact per-line integer sums for the exposure average (:792-844), separable integer
// Gaussian blur (:846-956), Reinhard tonemapping with nearest or linear bloom (:226-726, :997-1024);
// and FrameUpscaler::perform_upscale (src/square_wheel/frame_upscaler.rs:42-239).
//
// With bloom the frame takes at most three launches: the downscale (one block per bloom line; in a
// whole-frame graph the raster tile pass does it instead), the blur of the downscaled cells (once per
// cell, both directions in shared memory) and the tonemap, a streaming pass over the HDR frame that
// samples the blurred cells from L2, plus the exposure average on the side.
// Integer sums use wrapping 32-bit adds, which are associative, so the per-line sums can be reduced in
// any order and remain bit-exact; the single float reduction over lines (sum of line sums, in line
// order) runs in one thread exactly as the reference's sequential loop does.
#include "sw_kernels.cuh"

namespace swgpu
{
namespace
{

// TonemappingFunction::inv_scale_vec lanes of the frame: from device memory when the frame's exposure
// is uploaded with it (a replayed frame graph), else from the arguments.
__device__ __forceinline__ float4 tonemap_scale(const PostArgs& a)
{
	if (a.inv_scale_dev) return make_float4(a.inv_scale_dev[0], a.inv_scale_dev[1], a.inv_scale_dev[2], a.inv_scale_dev[3]);
	return make_float4(a.inv_scale[0], a.inv_scale[1], a.inv_scale[2], a.inv_scale[3]);
}

__device__ __forceinline__ CV tonemap(CV c, const PostArgs& a, float4 isc)
{
	// TonemappingFunction::do_it: c / (c * inv_255 + inv_scale), unfused (postprocessor.rs:1019-1023).
	// The alpha lane of both vectors is 0 (from_color_f32x3), so for the non-negative alpha sums here it
	// divides by +0: +inf or NaN, which the Color32 conversion's min(255) turns into 255 either way.
	const float alpha = (a.inv_255[3] == 0.0f && isc.w == 0.0f) ? 255.0f : __fdiv_rn(c.a, mad2(c.a, a.inv_255[3], isc.w));
	return CV{__fdiv_rn(c.b, mad2(c.b, a.inv_255[0], isc.x)), __fdiv_rn(c.g, mad2(c.g, a.inv_255[1], isc.y)),
		__fdiv_rn(c.r, mad2(c.r, a.inv_255[2], isc.z)), alpha};
}

// Sequential f32 sum over `n` lines of 4-lane values, in line order, as the reference's loop does; the
// block stages chunks of lines in shared memory with coalesced loads and threads 0..3 (one per lane)
// run the ordered additions from shared memory.
template <class LoadT>
__device__ __forceinline__ void ordered_line_sum(uint32_t n, LoadT load, float inv, float* out)
{
	constexpr uint32_t CHUNK = 2048;
	constexpr int LOADS = 8; // global loads in flight per thread while staging
	__shared__ float s_lines[CHUNK * 4];
	float acc = 0.0f;
	for (uint32_t base = 0; base < n; base += CHUNK)
	{
		const uint32_t m = min(CHUNK, n - base);
		const uint32_t total = m * 4;
		for (uint32_t i0 = threadIdx.x; i0 < total; i0 += LOADS * blockDim.x)
		{
			float v[LOADS];
#pragma unroll
			for (int k = 0; k < LOADS; ++k)
			{
				const uint32_t i = i0 + k * blockDim.x;
				v[k] = i < total ? load(base * 4 + i) : 0.0f;
			}
#pragma unroll
			for (int k = 0; k < LOADS; ++k)
				if (i0 + k * blockDim.x < total) s_lines[i0 + k * blockDim.x] = v[k];
		}
		__syncthreads();
		if (threadIdx.x < 4)
		{
			// the additions stay in line order; only the shared-memory reads are batched ahead of them
			uint32_t y = 0;
			for (; y + 8 <= m; y += 8)
			{
				float t[8];
#pragma unroll
				for (int k = 0; k < 8; ++k) t[k] = s_lines[(y + k) * 4 + threadIdx.x];
#pragma unroll
				for (int k = 0; k < 8; ++k) acc = fadd(acc, t[k]);
			}
			for (; y < m; ++y) acc = fadd(acc, s_lines[y * 4 + threadIdx.x]);
		}
		__syncthreads();
	}
	if (threadIdx.x < 4) out[threadIdx.x] = fmul(acc, inv);
}

// Average colour: f32 sum of the line sums in line order, then scale (postprocessor.rs:835-843).
__global__ void __launch_bounds__(256) pp_average_bloom_kernel(PostArgs a)
{
	const int32_t* sums = a.line_sums;
	ordered_line_sum(a.bh, [&](uint32_t i) { return float(sums[i]); }, __fdiv_rn(1.0f, float(a.bw * a.bh)), a.average);
}

// HDR pixel (x, y) plus its bloom sample, nearest (postprocessor.rs:346-462) or linear (:464-726).
template <int S, bool LINEAR, class Bloom>
__device__ __forceinline__ CV bloom_sum(const PostArgs& a, const Bloom& bl, uint32_t x, uint32_t y, CV c)
{
	auto bloom_at = [&](const PostArgs&, uint32_t bx, uint32_t by) { return bl.at(bx, by); };
	CV sum;
	if (!LINEAR)
	{
		sum = cv_add(bloom_at(a, min(x / S, a.bw - 1), min(y / S, a.bh - 1)), c);
	}
	else
	{
		constexpr uint32_t half = S / 2;
		constexpr float sf = float(S);
		const uint32_t rbx = (a.bw - 1) * S + half; // right_border_begin_x
		const uint32_t uby = (a.bh - 1) * S + half; // upper_border_begin_y
		const bool x_inner = x >= half && x < rbx;
		const bool y_inner = y >= half && y < uby;
		auto mix_factor = [&](uint32_t i) { return fadd(__fdiv_rn(1.0f, fmul(2.0f, sf)), __fdiv_rn(float(i), sf)); };
		const uint32_t sx = x_inner ? (x - half) / S : (x < half ? 0u : a.bw - 1);
		const uint32_t sy = y_inner ? (y - half) / S : (y < half ? 0u : a.bh - 1);
		if (x_inner && y_inner)
		{
			const float xm = mix_factor((x - half) % S), ym = mix_factor((y - half) % S);
			const float oxm = fsub(1.0f, xm), oym = fsub(1.0f, ym);
			const CV left = cv_sma(bloom_at(a, sx, sy), oym, cv_scale(bloom_at(a, sx, sy + 1), ym));
			const CV right = cv_sma(bloom_at(a, sx + 1, sy), oym, cv_scale(bloom_at(a, sx + 1, sy + 1), ym));
			sum = cv_sma(left, oxm, cv_sma(right, xm, c));
		}
		else if (x_inner) // lower / upper border rows
		{
			const float xm = mix_factor((x - half) % S), oxm = fsub(1.0f, xm);
			sum = cv_sma(bloom_at(a, sx, sy), oxm, cv_sma(bloom_at(a, sx + 1, sy), xm, c));
		}
		else if (y_inner) // left / right border columns
		{
			const float ym = mix_factor((y - half) % S), oym = fsub(1.0f, ym);
			sum = cv_add(cv_sma(bloom_at(a, sx, sy), oym, cv_scale(bloom_at(a, sx, sy + 1), ym)), c);
		}
		else // corners
			sum = cv_add(bloom_at(a, sx, sy), c);
	}
	return sum;
}

// ---- bloom passes: downscale, then blur + tonemap ----
//
// In a whole-frame graph the raster tile pass writes the downscaled bloom buffer and the exact per-line
// sums itself (its epilogue box-averages the tile's final pixels), so the frame's postprocess is the
// blur of the bloom cells and one pass over the HDR frame (pp_blur_kernel, pp_tonemap_bloom_kernel).
// A frame that did not come from the tile pass
// (sw_set_framebuffer, the allocation-free entry point, per-call sw_render + sw_postprocess) gets
// pp_downscale_kernel first.
//
// pp_downscale_kernel: one block per bloom line. The S lines of HDR pixels are box-averaged into the
// line (downscale_hdr_buffer, postprocessor.rs:792-844), written to bloom0, and the line's exact integer
// lane sums are written for the exposure average (no atomics: the block owns the line).
template <int S>
__global__ void __launch_bounds__(256) pp_downscale_kernel(PostArgs a)
{
	__shared__ int32_t s_sum[8][4];
	const uint32_t by = blockIdx.x;
	pdl_wait(); // the frame's rasterisation has completed
	constexpr int32_t scaler = 256 / (S * S);
	// U bloom pixels per thread per pass, all their HDR loads issued before any is used
	constexpr int U = S == 2 ? 4 : S == 4 ? 2 : 1;
	const unsigned long long* hdr = reinterpret_cast<const unsigned long long*>(a.hdr);
	const bool vec = ((a.width & 1) == 0) && ((reinterpret_cast<uintptr_t>(a.hdr) & 15) == 0); // 16-byte pairs
	uint64_t* out = a.bloom0 + uint64_t(by) * a.bw;
	int32_t lsum[4] = {0, 0, 0, 0};
	for (uint32_t base = threadIdx.x; base < a.bw; base += blockDim.x * U)
	{
		unsigned long long q[U][S][S];
#pragma unroll
		for (int u = 0; u < U; ++u)
		{
			const uint32_t bx = base + u * blockDim.x;
			if (bx >= a.bw) break;
#pragma unroll
			for (int dy = 0; dy < S; ++dy)
			{
				const unsigned long long* row = hdr + uint64_t(by * S + dy) * a.width + uint64_t(bx) * S;
#pragma unroll
				for (int dx = 0; dx < S; dx += 2)
				{
					if (vec)
					{
						const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(row + dx));
						q[u][dy][dx] = v.x;
						q[u][dy][dx + 1] = v.y;
					}
					else
					{
						q[u][dy][dx] = __ldg(row + dx);
						q[u][dy][dx + 1] = __ldg(row + dx + 1);
					}
				}
			}
		}
#pragma unroll
		for (int u = 0; u < U; ++u)
		{
			const uint32_t bx = base + u * blockDim.x;
			if (bx >= a.bw) break;
			int32_t sum[4] = {0, 0, 0, 0};
#pragma unroll
			for (int dy = 0; dy < S; ++dy)
#pragma unroll
				for (int dx = 0; dx < S; ++dx)
				{
					const CI c = ci_from_c64(q[u][dy][dx]);
#pragma unroll
					for (int i = 0; i < 4; ++i) sum[i] = wadd(sum[i], c.v[i]);
				}
			CI avg;
#pragma unroll
			for (int i = 0; i < 4; ++i)
			{
				avg.v[i] = wmul(sum[i], scaler) >> 8;
				lsum[i] = wadd(lsum[i], avg.v[i]);
			}
			out[bx] = ci_to_c64(avg);
		}
	}
	// exact per-line sums of the averages (wrapping i32: order-independent)
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for (int i = 0; i < 4; ++i)
	{
		int32_t v = lsum[i];
		for (int o = 16; o > 0; o >>= 1) v = wadd(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
		if (lane == 0) s_sum[warp][i] = v;
	}
	__syncthreads();
	if (threadIdx.x < 4)
	{
		int32_t t = 0;
		for (int w = 0; w < int(blockDim.x >> 5); ++w) t = wadd(t, s_sum[w][threadIdx.x]);
		a.line_sums[by * 4 + threadIdx.x] = t;
	}
	pdl_trigger();
}

// pp_blur_kernel: the separable blur of the downscaled bloom buffer, once per cell (perform_blur_impl,
// postprocessor.rs:846-956): one block per BL_W x BL_H tile of cells stages its cells with a radius halo
// on every side (source indices clamped to the buffer as the reference's blur clamps them), runs the
// horizontal pass over every staged line and the vertical pass (bloom_scale folded into its weights)
// over the tile, and writes the blurred cells to bloom1.
constexpr uint32_t BL_W = 64, BL_H = 16;

__host__ __device__ __forceinline__ uint32_t blur_tile_smem(uint32_t radius)
{
	const uint32_t lines = BL_H + 2 * radius, cols = BL_W + 2 * radius;
	return (lines * cols + lines * BL_W) * 16u; // cells as four i32 lanes
}

// Colour64 cell -> its four u16 lanes as i32 (ColorVecI::from_color64).
__device__ __forceinline__ int4 lanes_of(unsigned long long c)
{
	return make_int4(int32_t(uint32_t(c) & 0xFFFFu), int32_t(uint32_t(c) >> 16), int32_t(uint32_t(c >> 32) & 0xFFFFu),
		int32_t(uint32_t(c >> 48)));
}
// A blur pass's result as the reference stores it: (sum >> 14) into a Colour64 lane, (v as u64).min(65535).
__device__ __forceinline__ int32_t pass_lane(int32_t sum) { return int32_t(min(uint32_t(sum >> 14), 65535u)); }

__global__ void __launch_bounds__(256) pp_blur_kernel(PostArgs a)
{
	extern __shared__ __align__(16) int4 s_cells[];
	const uint32_t cx0 = blockIdx.x * BL_W, cy0 = blockIdx.y * BL_H;
	pdl_wait(); // the downscale (the raster tile pass or pp_downscale_kernel) has completed
	const int32_t r = int32_t(a.radius);
	const uint32_t cols = min(BL_W, a.bw - cx0), lines = min(BL_H, a.bh - cy0);
	const uint32_t slines = lines + 2 * uint32_t(r), scols = cols + 2 * uint32_t(r);
	int4* s_b = s_cells;                  // slines x scols downscaled cells, unpacked once
	int4* s_h = s_b + slines * scols;     // slines x cols, horizontally blurred (already clamped lanes)
	{
		// four loads in flight per thread; staged cell (l, c) is cell (clamp(cy0 - r + l), clamp(cx0 - r + c))
		const uint32_t total = slines * scols;
		const unsigned long long* src = reinterpret_cast<const unsigned long long*>(a.bloom0);
		for (uint32_t i0 = threadIdx.x; i0 < total; i0 += 4 * blockDim.x)
		{
			unsigned long long v[4];
#pragma unroll
			for (int k = 0; k < 4; ++k)
			{
				const uint32_t i = i0 + k * blockDim.x;
				if (i < total)
				{
					const uint32_t l = i / scols, c = i % scols;
					const int32_t by = min(max(int32_t(cy0) - r + int32_t(l), 0), int32_t(a.bh) - 1);
					const int32_t bx = min(max(int32_t(cx0) - r + int32_t(c), 0), int32_t(a.bw) - 1);
					v[k] = __ldg(src + uint64_t(by) * a.bw + uint32_t(bx));
				}
			}
#pragma unroll
			for (int k = 0; k < 4; ++k)
				if (i0 + k * blockDim.x < total) s_b[i0 + k * blockDim.x] = lanes_of(v[k]);
		}
	}
	__syncthreads();
	// horizontal pass over every staged line: cell c of the tile sits at staged column c + r
	for (uint32_t i = threadIdx.x; i < slines * cols; i += blockDim.x)
	{
		const uint32_t l = i / cols, c = i % cols;
		const int4* line = s_b + l * scols + c + uint32_t(r);
		const int4 cc = line[0];
		const int32_t k0 = a.kernel_h[r];
		int32_t s0 = wmul(cc.x, k0), s1 = wmul(cc.y, k0), s2 = wmul(cc.z, k0), s3 = wmul(cc.w, k0);
		for (int32_t dx = 1; dx <= r; ++dx)
		{
			const int4 c0 = line[-dx], c1 = line[dx];
			const int32_t k = a.kernel_h[dx + r];
			s0 = wadd(s0, wmul(wadd(c0.x, c1.x), k));
			s1 = wadd(s1, wmul(wadd(c0.y, c1.y), k));
			s2 = wadd(s2, wmul(wadd(c0.z, c1.z), k));
			s3 = wadd(s3, wmul(wadd(c0.w, c1.w), k));
		}
		s_h[i] = make_int4(pass_lane(s0), pass_lane(s1), pass_lane(s2), pass_lane(s3));
	}
	__syncthreads();
	// vertical pass: line cy0 + l is staged at l + r
	for (uint32_t i = threadIdx.x; i < lines * cols; i += blockDim.x)
	{
		const uint32_t l = i / cols, c = i % cols;
		const int4 cc = s_h[(l + r) * cols + c];
		const int32_t k0 = a.kernel_v[r];
		int32_t s0 = wmul(cc.x, k0), s1 = wmul(cc.y, k0), s2 = wmul(cc.z, k0), s3 = wmul(cc.w, k0);
		for (int32_t dy = 1; dy <= r; ++dy)
		{
			const int4 c0 = s_h[(l + r - dy) * cols + c], c1 = s_h[(l + r + dy) * cols + c];
			const int32_t k = a.kernel_v[dy + r];
			s0 = wadd(s0, wmul(wadd(c0.x, c1.x), k));
			s1 = wadd(s1, wmul(wadd(c0.y, c1.y), k));
			s2 = wadd(s2, wmul(wadd(c0.z, c1.z), k));
			s3 = wadd(s3, wmul(wadd(c0.w, c1.w), k));
		}
		a.bloom1[uint64_t(cy0 + l) * a.bw + cx0 + c] = uint64_t(uint32_t(pass_lane(s0))) | (uint64_t(uint32_t(pass_lane(s1))) << 16) |
			(uint64_t(uint32_t(pass_lane(s2))) << 32) | (uint64_t(uint32_t(pass_lane(s3))) << 48);
	}
	pdl_trigger();
}

// Bloom cells read straight from the (blurred) bloom buffer in global memory (L2-resident).
struct BloomGlobal
{
	const unsigned long long* cells;
	uint32_t pitch;
	__device__ CV at(uint32_t x, uint32_t y) const { return cv_from_c64(__ldg(cells + uint64_t(y) * pitch + x)); }
};

// pp_tonemap_bloom_kernel: the HDR frame tonemapped with its nearest or linear bloom sample
// (postprocessor.rs:346-726, :997-1024), 4 horizontally adjacent pixels per thread over the flat pixel
// space (one 32-byte HDR load pair and one 16-byte store when the row width is a multiple of 4).
template <int S, bool LINEAR>
__global__ void __launch_bounds__(256) pp_tonemap_bloom_kernel(PostArgs a, const uint64_t* bloom)
{
	const uint64_t first = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
	pdl_wait(); // the blur (or the downscale) has completed
	const uint64_t total = uint64_t(a.width) * a.height;
	if (first >= total) return;
	const BloomGlobal bl{reinterpret_cast<const unsigned long long*>(bloom), a.bw};
	const float4 isc = tonemap_scale(a);
	const unsigned long long* hdr = reinterpret_cast<const unsigned long long*>(a.hdr);
	const bool vec = (a.width & 3) == 0 && (reinterpret_cast<uintptr_t>(a.hdr) & 15) == 0;
	if (vec)
	{
		// the 4 pixels share a row: x = first % width ... + 3
		const uint32_t y = uint32_t(first / a.width), x = uint32_t(first % a.width);
		const ulonglong2 v0 = __ldg(reinterpret_cast<const ulonglong2*>(hdr + first));
		const ulonglong2 v1 = __ldg(reinterpret_cast<const ulonglong2*>(hdr + first + 2));
		const unsigned long long p[4] = {v0.x, v0.y, v1.x, v1.y};
		uint32_t o[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) o[k] = cv_to_c32(tonemap(bloom_sum<S, LINEAR>(a, bl, x + k, y, cv_from_c64(p[k])), a, isc));
		const uint64_t dst = uint64_t(y) * a.dst_pitch + x;
		if ((dst & 3) == 0 && (reinterpret_cast<uintptr_t>(a.dst) & 15) == 0)
			*reinterpret_cast<uint4*>(a.dst + dst) = make_uint4(o[0], o[1], o[2], o[3]);
		else
		{
#pragma unroll
			for (int k = 0; k < 4; ++k) a.dst[dst + k] = o[k];
		}
		return;
	}
	for (uint64_t i = first; i < first + 4 && i < total; ++i)
	{
		const uint32_t y = uint32_t(i / a.width), x = uint32_t(i % a.width);
		a.dst[uint64_t(y) * a.dst_pitch + x] = cv_to_c32(tonemap(bloom_sum<S, LINEAR>(a, bl, x, y, cv_from_c64(__ldg(hdr + i))), a, isc));
	}
}

// Without bloom: sequential per-line f32 colour sums (postprocessor.rs:237-253), one thread per line.
__global__ void pp_line_sums_kernel(PostArgs a)
{
	const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
	if (y >= a.height) return;
	CV s = cv_zero();
	const unsigned long long* row = reinterpret_cast<const unsigned long long*>(a.hdr) + uint64_t(y) * a.width;
	for (uint32_t x = 0; x < a.width; ++x) s = cv_add(s, cv_from_c64(__ldg(row + x)));
	a.line_sums_f[y * 4 + 0] = s.b;
	a.line_sums_f[y * 4 + 1] = s.g;
	a.line_sums_f[y * 4 + 2] = s.r;
	a.line_sums_f[y * 4 + 3] = s.a;
}

__global__ void __launch_bounds__(256) pp_average_plain_kernel(PostArgs a)
{
	const float* sums = a.line_sums_f;
	ordered_line_sum(a.height, [&](uint32_t i) { return sums[i]; }, __fdiv_rn(1.0f, float(uint64_t(a.width) * a.height)),
		a.average);
}

__global__ void __launch_bounds__(256) pp_tonemap_plain_kernel(PostArgs a)
{
	const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t y = blockIdx.y;
	if (x >= a.width) return;
	const CV c = cv_from_c64(__ldg(reinterpret_cast<const unsigned long long*>(a.hdr) + uint64_t(y) * a.width + x));
	a.dst[uint64_t(y) * a.dst_pitch + x] = cv_to_c32(tonemap(c, a, tonemap_scale(a)));
}

__device__ __forceinline__ uint32_t avg32(uint32_t a, uint32_t b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); }

// FrameUpscaler nearest x S (frame_upscaler.rs:72-166)
__global__ void __launch_bounds__(256) up_nearest_kernel(const uint32_t* src, uint32_t* dst, uint32_t S, uint32_t dw,
	uint32_t dh, uint32_t pitch)
{
	const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t y = blockIdx.y;
	if (x >= dw) return;
	const uint32_t sw = dw / S, sh = dh / S;
	dst[uint64_t(y) * pitch + x] = __ldg(src + uint64_t(min(y / S, sh - 1)) * sw + min(x / S, sw - 1));
}

// FrameUpscaler 2x "linear" with Color32::get_average (frame_upscaler.rs:168-239)
__global__ void __launch_bounds__(256) up_avg2x_kernel(const uint32_t* src, uint32_t* dst, uint32_t dw, uint32_t dh,
	uint32_t pitch)
{
	const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t y = blockIdx.y;
	if (x >= dw) return;
	const uint32_t sw = dw / 2, sh = dh / 2;
	const bool x_main = x < (sw - 1) * 2, y_main = y < (sh - 1) * 2;
	uint32_t out;
	if (y_main)
	{
		const uint32_t sy = y >> 1;
		const uint32_t* l0 = src + uint64_t(sy) * sw;
		const uint32_t* l1 = l0 + sw;
		if (x_main)
		{
			const uint32_t sx = x >> 1;
			const uint32_t p00 = __ldg(l0 + sx), p10 = __ldg(l0 + sx + 1), p01 = __ldg(l1 + sx), p11 = __ldg(l1 + sx + 1);
			const uint32_t ox = x & 1, oy = y & 1;
			if (!ox && !oy)
				out = p00;
			else if (ox && !oy)
				out = avg32(p00, p10);
			else if (!ox && oy)
				out = avg32(p00, p01);
			else
				out = avg32(avg32(p00, p10), avg32(p01, p11));
		}
		else
			out = avg32(__ldg(l0 + sw - 1), __ldg(l1 + sw - 1));
	}
	else
	{
		const uint32_t* l = src + uint64_t(sh - 1) * sw;
		if (x_main)
		{
			const uint32_t sx = x >> 1;
			out = (x & 1) ? avg32(__ldg(l + sx), __ldg(l + sx + 1)) : __ldg(l + sx);
		}
		else
			out = __ldg(l + sw - 1);
	}
	dst[uint64_t(y) * pitch + x] = out;
}

__global__ void fill_kernel(void* dst, uint64_t count, uint64_t value, uint32_t bpp)
{
	for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += uint64_t(gridDim.x) * blockDim.x)
	{
		if (bpp == 8)
			static_cast<uint64_t*>(dst)[i] = value;
		else
			static_cast<uint32_t*>(dst)[i] = uint32_t(value);
	}
}

// Dynamic shared memory above the default 48 KB needs the kernel's opt-in (set once, before use).
template <class K>
int allow_smem(K kernel, uint32_t bytes)
{
	if (bytes <= 48 * 1024) return 0;
	if (bytes > 200 * 1024) return int(cudaErrorInvalidValue);
	return int(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

template <int S>
int launch_bloom_pass(const PostArgs& a, cudaStream_t stream, bool downscale)
{
	if (downscale) return int(launch_dependent(pp_downscale_kernel<S>, dim3(a.bh), dim3(256), 0, stream, a));
	// the blur (radius 0: the downscaled cells are sampled directly), then the tonemap
	const uint64_t* bloom = a.bloom0;
	if (a.radius)
	{
		const uint32_t smem = blur_tile_smem(a.radius);
		if (int e = allow_smem(pp_blur_kernel, smem)) return e;
		const dim3 grid((a.bw + BL_W - 1) / BL_W, (a.bh + BL_H - 1) / BL_H);
		if (int e = int(launch_dependent(pp_blur_kernel, grid, dim3(256), smem, stream, a))) return e;
		bloom = a.bloom1;
	}
	const dim3 grid(unsigned((uint64_t(a.width) * a.height + 1023) / 1024));
	if (a.linear_filter) return int(launch_dependent(pp_tonemap_bloom_kernel<S, true>, grid, dim3(256), 0, stream, a, bloom));
	return int(launch_dependent(pp_tonemap_bloom_kernel<S, false>, grid, dim3(256), 0, stream, a, bloom));
}

int launch_bloom(const PostArgs& a, cudaStream_t stream, bool downscale)
{
	return a.scale == 2 ? launch_bloom_pass<2>(a, stream, downscale)
		: a.scale == 4  ? launch_bloom_pass<4>(a, stream, downscale)
						: launch_bloom_pass<8>(a, stream, downscale);
}

} // namespace

int launch_postprocess(const PostArgs& a, int num_sms, cudaStream_t stream, cudaStream_t aux, cudaEvent_t fork,
	cudaEvent_t join, cudaEvent_t average_done)
{
	(void)num_sms;
	const dim3 block(256);
	if (a.use_bloom)
	{
		if (a.scale != 2 && a.scale != 4 && a.scale != 8) return int(cudaErrorInvalidValue);
		if (a.radius > 16 || a.bw == 0 || a.bh == 0) return int(cudaErrorInvalidValue);
		// the downscale (bloom0 and every line's exact lane sums), unless the raster tile pass wrote them
		if (!a.downscaled)
			if (int e = launch_bloom(a, stream, true)) return e;
		// The exposure average is consumed only after the frame: with an auxiliary stream it runs
		// beside the vertical blur and tonemap pass.
		const bool overlap = aux && fork && join;
		if (overlap)
		{
			cudaEventRecord(fork, stream);
			cudaStreamWaitEvent(aux, fork, 0);
		}
		pp_average_bloom_kernel<<<1, 256, 0, overlap ? aux : stream>>>(a);
		// the average is final here: inside a captured graph this is an event record node
		if (average_done) cudaEventRecordWithFlags(average_done, overlap ? aux : stream, cudaEventRecordExternal);
		if (overlap) cudaEventRecord(join, aux);
		// blur + tonemap with the bloom sample
		if (int e = launch_bloom(a, stream, false)) return e;
		if (overlap) cudaStreamWaitEvent(stream, join, 0);
	}
	else
	{
		pp_line_sums_kernel<<<(a.height + 127) / 128, 128, 0, stream>>>(a);
		pp_average_plain_kernel<<<1, 256, 0, stream>>>(a);
		if (average_done) cudaEventRecordWithFlags(average_done, stream, cudaEventRecordExternal);
		pp_tonemap_plain_kernel<<<dim3((a.width + 255) / 256, a.height), block, 0, stream>>>(a);
	}
	return int(cudaGetLastError());
}

int launch_upscale(uint32_t mode, uint32_t scale, const uint32_t* src, uint32_t* dst, uint32_t dw, uint32_t dh,
	uint32_t pitch, cudaStream_t stream)
{
	const dim3 grid((dw + 255) / 256, dh), block(256);
	if (mode == SW_UPSCALE_AVG2X)
		up_avg2x_kernel<<<grid, block, 0, stream>>>(src, dst, dw, dh, pitch);
	else
		up_nearest_kernel<<<grid, block, 0, stream>>>(src, dst, scale, dw, dh, pitch);
	return int(cudaGetLastError());
}

int launch_fill(void* dst, uint64_t count, uint64_t value, uint32_t bpp, cudaStream_t stream)
{
	if (count == 0) return 0;
	fill_kernel<<<1024, 256, 0, stream>>>(dst, count, value, bpp);
	return int(cudaGetLastError());
}

} // namespace swgpu
