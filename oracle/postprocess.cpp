// Test infrastructure (oracle): CPU restatement of the reference's HDR postprocessor and frame
// upscaler.
//
// Follows src/square_wheel/postprocessor.rs:68-256 (perform_postprocessing single-thread path,
// update_exposure, perform_tonemapping), :346-726 (tonemapping with bloom, nearest and linear),
// :729-956 (perform_bloom, downscale_hdr_buffer, perform_blur_impl), :997-1051 (TonemappingFunction,
// compute_gaussian_kernel, get_color_brightness), and src/square_wheel/frame_upscaler.rs:42-239.
#include "sw_oracle.h"
#include "sw_oracle_math.h"

#include <vector>

namespace sworacle
{
namespace
{

const int MIN_BLOOM_BUFFER_SCALE_LOG2 = 1;
const int MAX_BLOOM_BUFFER_SCALE_LOG2 = 3;
const uint32_t MAX_GAUSSIAN_KERNEL_RADIUS = 16;
const uint32_t MAX_GAUSSIAN_KERNEL_SIZE = 1 + 2 * MAX_GAUSSIAN_KERNEL_RADIUS;

// postprocessor.rs:1026-1045
void compute_gaussian_kernel(float sigma, uint32_t radius, float* result)
{
	for (uint32_t i = 0; i < MAX_GAUSSIAN_KERNEL_SIZE; ++i) result[i] = 0.0f;
	const float samples[4] = {-0.375f, -0.125f, 0.125f, 0.375f};
	const float tau = 6.28318530717958647692f;
	for (int32_t x = -int32_t(radius); x <= int32_t(radius); ++x)
	{
		float val = 0.0f;
		for (float sample : samples)
		{
			float coord = float(x) + sample;
			val += std::exp(-0.5f * (coord / sigma) * (coord / sigma)) / (sigma * std::sqrt(tau));
		}
		result[x + int32_t(radius)] = val / 4.0f;
	}
}

// TonemappingFunction, postprocessor.rs:997-1024
struct Tonemap
{
	ColorVec inv_scale_vec, inv_255_vec;
	Tonemap(float exposure, const float m[3])
	{
		const float inv_255 = 1.0f / 255.0f;
		const float s[3] = {1.0f / (exposure * m[0]), 1.0f / (exposure * m[1]), 1.0f / (exposure * m[2])};
		const float i[3] = {inv_255, inv_255, inv_255};
		inv_scale_vec = cv_from_f32x3(s);
		inv_255_vec = cv_from_f32x3(i);
	}
	ColorVec operator()(const ColorVec& c) const { return cv_div(c, cv_mul_add(c, inv_255_vec, inv_scale_vec)); }
};

struct Post
{
	const SwPostConfig* cfg;
	const uint64_t* hdr;
	uint32_t w, h;
	uint32_t* dst;
	uint32_t pitch;
	uint32_t bw = 0, bh = 0;
	std::vector<uint64_t> bloom[2];

	// downscale_hdr_buffer, postprocessor.rs:792-844
	ColorVec downscale(uint32_t S)
	{
		const int COLOR_SHIFT = 8;
		int32_t average_scaler = (1 << COLOR_SHIFT) / int32_t(S * S);
		ColorVec colors_sum = cv_zero();
		for (uint32_t dst_y = 0; dst_y < bh; ++dst_y)
		{
			ColorVecI line_colors_sum = ci_zero();
			for (uint32_t dst_x = 0; dst_x < bw; ++dst_x)
			{
				ColorVecI sum = ci_zero();
				for (uint32_t dy = 0; dy < S; ++dy)
					for (uint32_t dx = 0; dx < S; ++dx)
						sum = ci_add(sum, ci_from_c64(hdr[uint64_t(dst_y * S + dy) * w + dst_x * S + dx]));
				ColorVecI average = ci_shr(ci_mul_scalar(sum, average_scaler), COLOR_SHIFT);
				bloom[0][uint64_t(dst_y) * bw + dst_x] = ci_to_c64(average);
				line_colors_sum = ci_add(line_colors_sum, average);
			}
			colors_sum = cv_add(colors_sum, ci_to_cv(line_colors_sum));
		}
		return cv_scalar_mul(colors_sum, 1.0f / float(bw * bh));
	}

	// perform_blur_impl, postprocessor.rs:846-956
	void blur(uint32_t radius, const float* kernel)
	{
		const int COLOR_SHIFT = 14;
		int32_t k[MAX_GAUSSIAN_KERNEL_SIZE];
		for (uint32_t i = 0; i < MAX_GAUSSIAN_KERNEL_SIZE; ++i) k[i] = f2i32(kernel[i] * float(1 << COLOR_SHIFT));
		const int32_t r = int32_t(radius);
		const int32_t max_x = int32_t(bw) - 1, max_y = int32_t(bh) - 1;
		for (uint32_t y = 0; y < bh; ++y)
			for (uint32_t x = 0; x < bw; ++x)
			{
				const uint64_t* line = bloom[0].data() + uint64_t(y) * bw;
				ColorVecI sum = ci_mul_scalar(ci_from_c64(line[x]), k[r]);
				for (int32_t dx = 1; dx <= r; ++dx)
				{
					int32_t x0 = std::max(int32_t(x) - dx, 0);
					int32_t x1 = std::min(int32_t(x) + dx, max_x);
					ColorVecI two = ci_add(ci_from_c64(line[x0]), ci_from_c64(line[x1]));
					sum = ci_add(sum, ci_mul_scalar(two, k[dx + r]));
				}
				bloom[1][uint64_t(y) * bw + x] = ci_to_c64(ci_shr(sum, COLOR_SHIFT));
			}
		for (uint32_t i = 0; i < MAX_GAUSSIAN_KERNEL_SIZE; ++i)
			k[i] = f2i32(kernel[i] * cfg->bloom_scale * float(1 << COLOR_SHIFT));
		for (uint32_t y = 0; y < bh; ++y)
			for (uint32_t x = 0; x < bw; ++x)
			{
				ColorVecI sum = ci_mul_scalar(ci_from_c64(bloom[1][uint64_t(y) * bw + x]), k[r]);
				for (int32_t dy = 1; dy <= r; ++dy)
				{
					int32_t y0 = std::max(int32_t(y) - dy, 0);
					int32_t y1 = std::min(int32_t(y) + dy, max_y);
					ColorVecI two = ci_add(ci_from_c64(bloom[1][uint64_t(y0) * bw + x]), ci_from_c64(bloom[1][uint64_t(y1) * bw + x]));
					sum = ci_add(sum, ci_mul_scalar(two, k[dy + r]));
				}
				bloom[0][uint64_t(y) * bw + x] = ci_to_c64(ci_shr(sum, COLOR_SHIFT));
			}
	}

	void put(uint32_t x, uint32_t y, const ColorVec& bloom_c, const Tonemap& tm)
	{
		ColorVec sum = cv_add(bloom_c, cv_from_c64(hdr[uint64_t(y) * w + x]));
		dst[uint64_t(y) * pitch + x] = cv_to_c32(tm(sum));
	}

	// perform_tonemapping_with_bloom_nearest, postprocessor.rs:346-462 (whole frame as one band)
	void tonemap_nearest(uint32_t S, const Tonemap& tm)
	{
		for (uint32_t y = 0; y < h; ++y)
			for (uint32_t x = 0; x < w; ++x)
			{
				uint32_t bx = std::min(x / S, bw - 1), by = std::min(y / S, bh - 1);
				put(x, y, cv_from_c64(bloom[0][uint64_t(by) * bw + bx]), tm);
			}
	}

	ColorVec bl(uint32_t x, uint32_t y) const { return cv_from_c64(bloom[0][uint64_t(y) * bw + x]); }

	// perform_tonemapping_with_bloom_linear, postprocessor.rs:464-726, restated loop for loop.
	void tonemap_linear(uint32_t S, const Tonemap& tm)
	{
		std::vector<float> mix_factors(S);
		const float sf = float(S);
		for (uint32_t i = 0; i < S; ++i) mix_factors[i] = float((S + 1) & 1) / (2.0f * sf) + float(i) / sf;
		const uint32_t half = S / 2;
		const uint32_t right_border_begin_x = (bw - 1) * S + half;
		const uint32_t right_border_size = w - right_border_begin_x;
		const uint32_t upper_border_begin_y = (bh - 1) * S + half;
		const uint32_t upper_border_size = h - upper_border_begin_y;

		// Lower border.
		{
			ColorVec b00 = bl(0, 0);
			for (uint32_t src_x = 0; src_x + 1 < bw; ++src_x)
			{
				uint32_t dst_x_base = src_x * S + half;
				ColorVec b10 = bl(src_x + 1, 0);
				for (uint32_t dy = 0; dy < half; ++dy)
					for (uint32_t dx = 0; dx < S; ++dx)
					{
						float xm = mix_factors[dx], oxm = 1.0f - xm;
						uint32_t x = dst_x_base + dx, y = dy;
						ColorVec sum = cv_mul_scalar_add(b00, oxm, cv_mul_scalar_add(b10, xm, cv_from_c64(hdr[uint64_t(y) * w + x])));
						dst[uint64_t(y) * pitch + x] = cv_to_c32(tm(sum));
					}
				b00 = b10;
			}
		}
		// Main image.
		for (uint32_t src_y = 0; src_y + 1 < bh; ++src_y)
		{
			uint32_t dst_y_base = src_y * S + half;
			ColorVec b00 = bl(0, src_y), b01 = bl(0, src_y + 1);
			for (uint32_t dy = 0; dy < S; ++dy) // left border
			{
				float ym = mix_factors[dy], oym = 1.0f - ym;
				ColorVec b = cv_mul_scalar_add(b00, oym, cv_scalar_mul(b01, ym));
				for (uint32_t dx = 0; dx < half; ++dx) put(dx, dst_y_base + dy, b, tm);
			}
			for (uint32_t src_x = 0; src_x + 1 < bw; ++src_x)
			{
				uint32_t dst_x_base = src_x * S + half;
				ColorVec b10 = bl(src_x + 1, src_y), b11 = bl(src_x + 1, src_y + 1);
				for (uint32_t dy = 0; dy < S; ++dy)
				{
					float ym = mix_factors[dy], oym = 1.0f - ym;
					ColorVec left = cv_mul_scalar_add(b00, oym, cv_scalar_mul(b01, ym));
					ColorVec right = cv_mul_scalar_add(b10, oym, cv_scalar_mul(b11, ym));
					for (uint32_t dx = 0; dx < S; ++dx)
					{
						float xm = mix_factors[dx], oxm = 1.0f - xm;
						uint32_t x = dst_x_base + dx, y = dst_y_base + dy;
						ColorVec sum = cv_mul_scalar_add(left, oxm, cv_mul_scalar_add(right, xm, cv_from_c64(hdr[uint64_t(y) * w + x])));
						dst[uint64_t(y) * pitch + x] = cv_to_c32(tm(sum));
					}
				}
				b00 = b10;
				b01 = b11;
			}
			for (uint32_t dy = 0; dy < S; ++dy) // right border
			{
				float ym = mix_factors[dy], oym = 1.0f - ym;
				ColorVec b = cv_mul_scalar_add(b00, oym, cv_scalar_mul(b01, ym));
				for (uint32_t dx = 0; dx < right_border_size; ++dx) put(right_border_begin_x + dx, dst_y_base + dy, b, tm);
			}
		}
		// Upper border.
		{
			uint32_t row = bh - 1;
			ColorVec b00 = bl(0, row);
			for (uint32_t src_x = 0; src_x + 1 < bw; ++src_x)
			{
				uint32_t dst_x_base = src_x * S + half;
				ColorVec b10 = bl(src_x + 1, row);
				for (uint32_t dy = 0; dy < upper_border_size; ++dy)
					for (uint32_t dx = 0; dx < S; ++dx)
					{
						float xm = mix_factors[dx], oxm = 1.0f - xm;
						uint32_t x = dst_x_base + dx, y = upper_border_begin_y + dy;
						ColorVec sum = cv_mul_scalar_add(b00, oxm, cv_mul_scalar_add(b10, xm, cv_from_c64(hdr[uint64_t(y) * w + x])));
						dst[uint64_t(y) * pitch + x] = cv_to_c32(tm(sum));
					}
				b00 = b10;
			}
		}
		// Corners.
		auto corner = [&](uint32_t x0, uint32_t x1, uint32_t y0, uint32_t y1, ColorVec b) {
			for (uint32_t y = y0; y < y1; ++y)
				for (uint32_t x = x0; x < x1; ++x) put(x, y, b, tm);
		};
		corner(0, half, 0, half, bl(0, 0));
		corner(right_border_begin_x, w, 0, half, bl(bw - 1, 0));
		corner(0, half, upper_border_begin_y, h, bl(0, bh - 1));
		corner(right_border_begin_x, w, upper_border_begin_y, h, bl(bw - 1, bh - 1));
	}

	// perform_tonemapping, postprocessor.rs:226-256: returns the sum of colours.
	ColorVec tonemap_plain(const Tonemap& tm)
	{
		ColorVec colors_sum = cv_zero();
		for (uint32_t y = 0; y < h; ++y)
		{
			ColorVec line_sum = cv_zero();
			for (uint32_t x = 0; x < w; ++x)
			{
				ColorVec c = cv_from_c64(hdr[uint64_t(y) * w + x]);
				line_sum = cv_add(line_sum, c);
				dst[uint64_t(y) * pitch + x] = cv_to_c32(tm(c));
			}
			colors_sum = cv_add(colors_sum, line_sum);
		}
		return colors_sum;
	}
};

// update_exposure + get_color_brightness, postprocessor.rs:206-223, 1047-1051
float update_exposure(const SwPostConfig* cfg, float current, const ColorVec& average, float dt)
{
	float brightness_raw = (average.v[0] + average.v[1] + average.v[2]) * 0.33f;
	float brightness = fminr(fmaxr(brightness_raw, 1.0f / 1024.0f), 65536.0f) / 255.0f;
	float target = std::pow(brightness / cfg->zero_level_brightness, cfg->brightness_scale_power) * 0.5f *
		cfg->base_brightness / brightness;
	float clamped = fminr(fmaxr(target, cfg->min_exposure), cfg->max_exposure);
	float mix = std::exp(-cfg->exposure_update_speed * dt);
	return std::exp(std::log(current) * mix + std::log(clamped) * (1.0f - mix));
}

// Postprocessor::synchronize_config, postprocessor.rs:958-977: the host clamps the configuration before
// every frame (host.rs:217-219, 274). f32::max / f32::min return the other operand for a NaN, as
// fmax / fmin do.
SwPostConfig synchronize_config(const SwPostConfig& in)
{
	SwPostConfig c = in;
	c.min_exposure = fminr(fmaxr(c.min_exposure, 1.0f / 65536.0f), 16.0f);
	c.max_exposure = fminr(fmaxr(c.max_exposure, 1.0f), 65536.0f);
	c.exposure_update_speed = fminr(fmaxr(c.exposure_update_speed, 0.5f), 16.0f);
	c.base_brightness = fminr(fmaxr(c.base_brightness, 0.5f), 2.0f);
	c.zero_level_brightness = fminr(fmaxr(c.zero_level_brightness, 1.0f / 16.0f), 16.0f);
	c.brightness_scale_power = fminr(fmaxr(c.brightness_scale_power, 0.01f), 0.5f);
	c.bloom_sigma = fminr(fmaxr(c.bloom_sigma, 0.0f), 40.0f);
	c.bloom_buffer_scale_log2 = std::min(std::max(c.bloom_buffer_scale_log2, uint32_t(MIN_BLOOM_BUFFER_SCALE_LOG2)),
		uint32_t(MAX_BLOOM_BUFFER_SCALE_LOG2));
	c.bloom_scale = fminr(fmaxr(c.bloom_scale, 1.0f / 16.0f), 1.0f / 2.0f);
	return c;
}

} // namespace
} // namespace sworacle

using namespace sworacle;

extern "C" int orc_gaussian_kernel(float sigma, uint32_t radius, float* out33)
{
	if (!out33 || radius > MAX_GAUSSIAN_KERNEL_RADIUS) return SW_ERR_INVALID_ARGUMENT;
	compute_gaussian_kernel(sigma, radius, out33);
	return SW_OK;
}

extern "C" int orc_postprocess(const SwPostConfig* config, const uint64_t* hdr, uint32_t width, uint32_t height,
	float frame_duration_s, const float color_modulate[3], float* exposure, uint32_t* dst, uint32_t pitch,
	float* average_color)
{
	if (!config || !hdr || !dst || !exposure || !color_modulate || pitch < width || width == 0 || height == 0)
		return SW_ERR_INVALID_ARGUMENT;
	const SwPostConfig synced = synchronize_config(*config);
	config = &synced;
	Post p;
	p.cfg = config;
	p.hdr = hdr;
	p.w = width;
	p.h = height;
	p.dst = dst;
	p.pitch = pitch;
	const bool use_bloom = config->bloom_sigma > 0.0f;
	ColorVec average = cv_zero();
	uint32_t S = 1;
	if (use_bloom) // perform_bloom, postprocessor.rs:729-789
	{
		int log2 = std::min(std::max(int(config->bloom_buffer_scale_log2), MIN_BLOOM_BUFFER_SCALE_LOG2), MAX_BLOOM_BUFFER_SCALE_LOG2);
		S = 1u << log2;
		p.bw = width / S;
		p.bh = height / S;
		if (p.bw < 2 || p.bh < 2) return SW_ERR_INVALID_ARGUMENT;
		p.bloom[0].assign(uint64_t(p.bw) * p.bh, 0);
		p.bloom[1].assign(uint64_t(p.bw) * p.bh, 0);
		average = p.downscale(S);
		float sigma_corrected = config->bloom_sigma / float(S);
		float rf = std::ceil(3.0f * sigma_corrected - 0.5f);
		uint32_t radius = f2u32(fmaxr(rf, 0.0f));
		if (radius > MAX_GAUSSIAN_KERNEL_RADIUS) radius = MAX_GAUSSIAN_KERNEL_RADIUS;
		float kernel[MAX_GAUSSIAN_KERNEL_SIZE];
		compute_gaussian_kernel(sigma_corrected, radius, kernel);
		if (radius > 0) p.blur(radius, kernel);
	}
	Tonemap tm(*exposure, color_modulate);
	if (use_bloom)
	{
		if (config->linear_bloom_filter)
			p.tonemap_linear(S, tm);
		else
			p.tonemap_nearest(S, tm);
	}
	else
	{
		ColorVec sum = p.tonemap_plain(tm);
		average = cv_scalar_mul(sum, 1.0f / float(uint64_t(width) * height));
	}
	if (average_color)
		for (int i = 0; i < 4; ++i) average_color[i] = average.v[i];
	*exposure = update_exposure(config, *exposure, average, frame_duration_s);
	return SW_OK;
}

// FrameUpscaler, frame_upscaler.rs:72-239
extern "C" int orc_upscale(uint32_t mode, uint32_t scale, const uint32_t* src, uint32_t* dst, uint32_t dst_width,
	uint32_t dst_height, uint32_t dst_pitch)
{
	if (!src || !dst || dst_pitch < dst_width) return SW_ERR_INVALID_ARGUMENT;
	if (mode == SW_UPSCALE_AVG2X)
	{
		const uint32_t sw = dst_width / 2, sh = dst_height / 2;
		if (sw < 1 || sh < 1) return SW_ERR_INVALID_ARGUMENT;
		auto avg = [](uint32_t a, uint32_t b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); };
		for (uint32_t src_y = 0; src_y + 1 < sh; ++src_y)
		{
			const uint32_t* sl = src + uint64_t(src_y) * sw;
			uint32_t* dl = dst + uint64_t(src_y) * 2 * dst_pitch;
			for (uint32_t src_x = 0; src_x + 1 < sw; ++src_x)
			{
				uint32_t p00 = sl[src_x], p10 = sl[src_x + 1], p01 = sl[sw + src_x], p11 = sl[sw + src_x + 1];
				uint32_t x_mix = avg(p00, p10), y_mix = avg(p00, p01);
				uint32_t corner_mix = avg(x_mix, avg(p01, p11));
				uint32_t dx = src_x * 2;
				dl[dx] = p00;
				dl[dx + 1] = x_mix;
				dl[dst_pitch + dx] = y_mix;
				dl[dst_pitch + dx + 1] = corner_mix;
			}
			uint32_t last_mix = avg(sl[sw - 1], sl[sw - 1 + sw]);
			for (uint32_t dx = (sw - 1) * 2; dx < dst_width; ++dx)
			{
				dl[dx] = last_mix;
				dl[dx + dst_pitch] = last_mix;
			}
		}
		const uint32_t src_y = sh - 1;
		const uint32_t y_left = dst_height - (sh - 1) * 2;
		const uint32_t* sl = src + uint64_t(src_y) * sw;
		uint32_t* dl = dst + uint64_t(src_y) * 2 * dst_pitch;
		for (uint32_t src_x = 0; src_x + 1 < sw; ++src_x)
		{
			uint32_t p0 = sl[src_x], p1 = sl[src_x + 1];
			uint32_t x_mix = avg(p0, p1);
			uint32_t dx = src_x * 2;
			for (uint32_t dy = 0; dy < y_left; ++dy)
			{
				dl[uint64_t(dy) * dst_pitch + dx] = p0;
				dl[uint64_t(dy) * dst_pitch + dx + 1] = x_mix;
			}
		}
		uint32_t last = sl[sw - 1];
		for (uint32_t dx = (sw - 1) * 2; dx < dst_width; ++dx)
			for (uint32_t dy = 0; dy < y_left; ++dy) dl[uint64_t(dy) * dst_pitch + dx] = last;
		return SW_OK;
	}
	if (mode != SW_UPSCALE_NEAREST || scale < 1 || scale > 6) return SW_ERR_INVALID_ARGUMENT;
	const uint32_t S = scale;
	const uint32_t sw = dst_width / S, sh = dst_height / S;
	if (sw < 1 || sh < 1) return SW_ERR_INVALID_ARGUMENT;
	for (uint32_t y = 0; y < dst_height; ++y)
		for (uint32_t x = 0; x < dst_width; ++x)
		{
			uint32_t sx = std::min(x / S, sw - 1), sy = std::min(y / S, sh - 1);
			dst[uint64_t(y) * dst_pitch + x] = src[uint64_t(sy) * sw + sx];
		}
	return SW_OK;
}
