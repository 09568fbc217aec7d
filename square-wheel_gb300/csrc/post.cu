// HDR postprocessor and frame upscaler for the GB300 path.
//
// Replaces Postprocessor::perform_postprocessing (src/square_wheel/postprocessor.rs:68-204): bloom
// downscale with exact per-line integer sums for the exposure average (:792-844), separable integer
// Gaussian blur (:846-956), Reinhard tonemapping with nearest or linear bloom (:226-726, :997-1024);
// and FrameUpscaler::perform_upscale (src/square_wheel/frame_upscaler.rs:42-239).
//
// All passes are HBM-bound streaming kernels with one thread per output pixel. Integer sums use
// wrapping 32-bit adds, which are associative, so the per-line sums can be reduced in any order and
// remain bit-exact; the single float reduction over lines (sum of line sums, in line order) runs in one
// thread exactly as the reference's sequential loop does.
#include "sw_kernels.cuh"

namespace swgpu
{
namespace
{

__device__ __forceinline__ CV tonemap(CV c, const PostArgs& a)
{
	// TonemappingFunction::do_it: c / (c * inv_255 + inv_scale), unfused (postprocessor.rs:1019-1023).
	// The alpha lane of both vectors is 0 (from_color_f32x3), so for the non-negative alpha sums here it
	// divides by +0: +inf or NaN, which the Color32 conversion's min(255) turns into 255 either way.
	const float alpha = (a.inv_255[3] == 0.0f && a.inv_scale[3] == 0.0f)
		? 255.0f
		: __fdiv_rn(c.a, mad2(c.a, a.inv_255[3], a.inv_scale[3]));
	return CV{__fdiv_rn(c.b, mad2(c.b, a.inv_255[0], a.inv_scale[0])), __fdiv_rn(c.g, mad2(c.g, a.inv_255[1], a.inv_scale[1])),
		__fdiv_rn(c.r, mad2(c.r, a.inv_255[2], a.inv_scale[2])), alpha};
}

// downscale_hdr_buffer::<S>, postprocessor.rs:792-844. Each thread computes two horizontally adjacent
// bloom pixels (all 2*S*S HDR pixels are loaded before any is used: S is a template parameter, so the
// loops unroll); a block covers 512 bloom pixels of one line and adds its lanes' exact integer line
// sums with one atomic per lane.
template <int S>
__global__ void __launch_bounds__(256) pp_downscale_kernel(PostArgs a)
{
	__shared__ int32_t s_sum[8][4];
	const uint32_t bx = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
	const uint32_t by = blockIdx.y;
	int32_t avg[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
	constexpr int32_t scaler = 256 / (S * S);
#pragma unroll
	for (int k = 0; k < 2; ++k)
	{
		if (bx + k >= a.bw) break;
		int32_t sum[4] = {0, 0, 0, 0};
		unsigned long long q[S][S];
#pragma unroll
		for (int dy = 0; dy < S; ++dy)
		{
			const uint64_t* row = a.hdr + uint64_t(by * S + dy) * a.width + (bx + k) * S;
			const bool aligned = (reinterpret_cast<uintptr_t>(row) & 15) == 0;
#pragma unroll
			for (int dx = 0; dx < S; dx += 2)
			{
				if (aligned)
				{
					const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(row + dx));
					q[dy][dx] = v.x;
					q[dy][dx + 1] = v.y;
				}
				else
				{
					q[dy][dx] = __ldg(reinterpret_cast<const unsigned long long*>(row) + dx);
					q[dy][dx + 1] = __ldg(reinterpret_cast<const unsigned long long*>(row) + dx + 1);
				}
			}
		}
#pragma unroll
		for (int dy = 0; dy < S; ++dy)
#pragma unroll
			for (int dx = 0; dx < S; ++dx)
			{
				const CI c = ci_from_c64(q[dy][dx]);
#pragma unroll
				for (int i = 0; i < 4; ++i) sum[i] = wadd(sum[i], c.v[i]);
			}
#pragma unroll
		for (int i = 0; i < 4; ++i) avg[k][i] = wmul(sum[i], scaler) >> 8;
	}
	if (bx < a.bw)
	{
		const uint64_t o = uint64_t(by) * a.bw + bx;
		const uint64_t v0 = ci_to_c64(CI{{avg[0][0], avg[0][1], avg[0][2], avg[0][3]}});
		if (bx + 1 < a.bw)
		{
			const uint64_t v1 = ci_to_c64(CI{{avg[1][0], avg[1][1], avg[1][2], avg[1][3]}});
			if ((o & 1) == 0)
				*reinterpret_cast<ulonglong2*>(a.bloom0 + o) = make_ulonglong2(v0, v1);
			else
			{
				a.bloom0[o] = v0;
				a.bloom0[o + 1] = v1;
			}
		}
		else
			a.bloom0[o] = v0;
	}
	// Exact per-line sums of the averages (wrapping i32: order-independent): warp, then block.
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for (int i = 0; i < 4; ++i)
	{
		int32_t v = wadd(avg[0][i], avg[1][i]);
		for (int o = 16; o > 0; o >>= 1) v = wadd(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
		if (lane == 0) s_sum[warp][i] = v;
	}
	__syncthreads();
	if (threadIdx.x < 4)
	{
		int32_t t = 0;
		for (int w = 0; w < 8; ++w) t = wadd(t, s_sum[w][threadIdx.x]);
		atomicAdd(a.line_sums + by * 4 + threadIdx.x, t);
	}
}

// Sequential f32 sum over `n` lines of 4-lane values, in line order, as the reference's loop does; the
// block stages chunks of lines in shared memory with coalesced loads and threads 0..3 (one per lane)
// run the ordered additions from shared memory.
template <class LoadT>
__device__ __forceinline__ void ordered_line_sum(uint32_t n, LoadT load, float inv, float* out)
{
	constexpr uint32_t CHUNK = 2048;
	__shared__ float s_lines[CHUNK * 4];
	float acc = 0.0f;
	for (uint32_t base = 0; base < n; base += CHUNK)
	{
		const uint32_t m = min(CHUNK, n - base);
		for (uint32_t i = threadIdx.x; i < m * 4; i += blockDim.x) s_lines[i] = load(base * 4 + i);
		__syncthreads();
		if (threadIdx.x < 4)
			for (uint32_t y = 0; y < m; ++y) acc = fadd(acc, s_lines[y * 4 + threadIdx.x]);
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

// perform_blur_impl, horizontal pass buf0 -> buf1 (postprocessor.rs:862-900)
__global__ void __launch_bounds__(256) pp_blur_h_kernel(PostArgs a)
{
	const int32_t x = int32_t(blockIdx.x * blockDim.x + threadIdx.x);
	const int32_t y = int32_t(blockIdx.y);
	if (x >= int32_t(a.bw)) return;
	const uint64_t* line = a.bloom0 + uint64_t(y) * a.bw;
	const int32_t r = int32_t(a.radius);
	const CI c = ci_from_c64(line[x]);
	int32_t sum[4];
#pragma unroll
	for (int i = 0; i < 4; ++i) sum[i] = wmul(c.v[i], a.kernel_h[r]);
	for (int32_t dx = 1; dx <= r; ++dx)
	{
		const CI c0 = ci_from_c64(line[max(x - dx, 0)]);
		const CI c1 = ci_from_c64(line[min(x + dx, int32_t(a.bw) - 1)]);
#pragma unroll
		for (int i = 0; i < 4; ++i) sum[i] = wadd(sum[i], wmul(wadd(c0.v[i], c1.v[i]), a.kernel_h[dx + r]));
	}
	a.bloom1[uint64_t(y) * a.bw + x] = ci_to_c64(CI{{sum[0] >> 14, sum[1] >> 14, sum[2] >> 14, sum[3] >> 14}});
}

// perform_blur_impl, vertical pass buf1 -> buf0 with bloom_scale folded into the weights (:902-955)
__global__ void __launch_bounds__(256) pp_blur_v_kernel(PostArgs a)
{
	const int32_t x = int32_t(blockIdx.x * blockDim.x + threadIdx.x);
	const int32_t y = int32_t(blockIdx.y);
	if (x >= int32_t(a.bw)) return;
	const int32_t r = int32_t(a.radius);
	const CI c = ci_from_c64(a.bloom1[uint64_t(y) * a.bw + x]);
	int32_t sum[4];
#pragma unroll
	for (int i = 0; i < 4; ++i) sum[i] = wmul(c.v[i], a.kernel_v[r]);
	for (int32_t dy = 1; dy <= r; ++dy)
	{
		const CI c0 = ci_from_c64(a.bloom1[uint64_t(max(y - dy, 0)) * a.bw + x]);
		const CI c1 = ci_from_c64(a.bloom1[uint64_t(min(y + dy, int32_t(a.bh) - 1)) * a.bw + x]);
#pragma unroll
		for (int i = 0; i < 4; ++i) sum[i] = wadd(sum[i], wmul(wadd(c0.v[i], c1.v[i]), a.kernel_v[dy + r]));
	}
	a.bloom0[uint64_t(y) * a.bw + x] = ci_to_c64(CI{{sum[0] >> 14, sum[1] >> 14, sum[2] >> 14, sum[3] >> 14}});
}

__device__ __forceinline__ CV bloom_at(const PostArgs& a, uint32_t x, uint32_t y)
{
	return cv_from_c64(__ldg(reinterpret_cast<const unsigned long long*>(a.bloom0) + uint64_t(y) * a.bw + x));
}

// HDR pixel (x, y) plus its bloom sample, nearest (postprocessor.rs:346-462) or linear (:464-726).
template <int S, bool LINEAR>
__device__ __forceinline__ CV bloom_sum(const PostArgs& a, uint32_t x, uint32_t y, CV c)
{
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

// Tonemapping with bloom: four horizontally adjacent pixels per thread (two 16-byte HDR loads issued
// together, one 16-byte store where aligned).
template <int S, bool LINEAR>
__global__ void __launch_bounds__(256) pp_tonemap_bloom_kernel(PostArgs a)
{
	const uint32_t x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
	const uint32_t y = blockIdx.y;
	if (x >= a.width) return;
	const uint64_t src = uint64_t(y) * a.width + x;
	const uint64_t dst = uint64_t(y) * a.dst_pitch + x;
	const uint32_t n = min(4u, a.width - x);
	unsigned long long p[4] = {0, 0, 0, 0};
	const unsigned long long* h = reinterpret_cast<const unsigned long long*>(a.hdr) + src;
	if (n == 4 && (src & 1) == 0)
	{
		const ulonglong2 v0 = __ldg(reinterpret_cast<const ulonglong2*>(h));
		const ulonglong2 v1 = __ldg(reinterpret_cast<const ulonglong2*>(h + 2));
		p[0] = v0.x;
		p[1] = v0.y;
		p[2] = v1.x;
		p[3] = v1.y;
	}
	else
	{
#pragma unroll
		for (int k = 0; k < 4; ++k)
			if (k < int(n)) p[k] = __ldg(h + k);
	}
	uint32_t o[4];
#pragma unroll
	for (int k = 0; k < 4; ++k)
		o[k] = k < int(n) ? cv_to_c32(tonemap(bloom_sum<S, LINEAR>(a, x + k, y, cv_from_c64(p[k])), a)) : 0u;
	if (n == 4 && (dst & 3) == 0)
		*reinterpret_cast<uint4*>(a.dst + dst) = make_uint4(o[0], o[1], o[2], o[3]);
	else
	{
#pragma unroll
		for (int k = 0; k < 4; ++k)
			if (k < int(n)) a.dst[dst + k] = o[k];
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
	a.dst[uint64_t(y) * a.dst_pitch + x] = cv_to_c32(tonemap(c, a));
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

template <int S>
void launch_bloom_passes(const PostArgs& a, cudaStream_t stream, bool downscale)
{
	const dim3 block(256);
	if (downscale)
	{
		pp_downscale_kernel<S><<<dim3((a.bw + 511) / 512, a.bh), block, 0, stream>>>(a);
		return;
	}
	const dim3 grid((a.width + 1023) / 1024, a.height);
	if (a.linear_filter)
		pp_tonemap_bloom_kernel<S, true><<<grid, block, 0, stream>>>(a);
	else
		pp_tonemap_bloom_kernel<S, false><<<grid, block, 0, stream>>>(a);
}

void launch_bloom(const PostArgs& a, cudaStream_t stream, bool downscale)
{
	if (a.scale == 2)
		launch_bloom_passes<2>(a, stream, downscale);
	else if (a.scale == 4)
		launch_bloom_passes<4>(a, stream, downscale);
	else
		launch_bloom_passes<8>(a, stream, downscale);
}

} // namespace

int launch_postprocess(const PostArgs& a, int num_sms, cudaStream_t stream, cudaStream_t aux, cudaEvent_t fork,
	cudaEvent_t join)
{
	(void)num_sms;
	const dim3 block(256);
	if (a.use_bloom)
	{
		cudaMemsetAsync(a.line_sums, 0, sizeof(int32_t) * 4 * a.bh, stream);
		if (a.scale != 2 && a.scale != 4 && a.scale != 8) return int(cudaErrorInvalidValue);
		launch_bloom(a, stream, true);
		// The exposure average is consumed only after the frame: with an auxiliary stream it runs
		// beside the blur and tonemap passes.
		const bool overlap = aux && fork && join;
		if (overlap)
		{
			cudaEventRecord(fork, stream);
			cudaStreamWaitEvent(aux, fork, 0);
		}
		pp_average_bloom_kernel<<<1, 256, 0, overlap ? aux : stream>>>(a);
		if (overlap) cudaEventRecord(join, aux);
		if (a.radius > 0)
		{
			pp_blur_h_kernel<<<dim3((a.bw + 255) / 256, a.bh), block, 0, stream>>>(a);
			pp_blur_v_kernel<<<dim3((a.bw + 255) / 256, a.bh), block, 0, stream>>>(a);
		}
		launch_bloom(a, stream, false);
		if (overlap) cudaStreamWaitEvent(stream, join, 0);
	}
	else
	{
		pp_line_sums_kernel<<<(a.height + 127) / 128, 128, 0, stream>>>(a);
		pp_average_plain_kernel<<<1, 256, 0, stream>>>(a);
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
