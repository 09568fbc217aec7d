// Lightmap decompression on the GPU: the compressed lightmap lumps of a compiled map
// (src/common/lightmap_compression.rs), uploaded as the file holds them, are decoded in device memory
// into the f32 lightmaps the surface build reads.
//
// Simple element (CompressedColor, 4 bytes): rgb = component * (scale / 255).
// Directional element (DirectionalLightmapElementCompressed, 13 bytes, no padding): ambient colour,
// direction vector (i8 components, value = component * (scale / 127)), deviation (u8 / 255), directional
// colour; a direction that decodes to zero becomes (0, 0, 1/1024) as decompress does (:114-130).
//
// Byte work bound by HBM: the 13-byte directional records are read by each block as one aligned run of
// 16-byte words into shared memory (256 records = 208 words), decoded there, and the 40-byte outputs
// leave as 16-byte words from shared memory as well, so both directions of the copy are coalesced.
#include "sw_kernels.cuh"

namespace swgpu
{
namespace
{

constexpr uint32_t LM_BLOCK = 256;

__global__ void __launch_bounds__(LM_BLOCK) lightmap_simple_kernel(const uint32_t* __restrict__ in, uint64_t n, float* __restrict__ out)
{
	const uint64_t i = uint64_t(blockIdx.x) * LM_BLOCK + threadIdx.x;
	if (i >= n) return;
	const uint32_t v = __ldg(in + i); // components[0..3] in bytes 0..2, scale in byte 3
	const float m = __fdiv_rn(float(v >> 24), 255.0f);
	out[i * 3 + 0] = __fmul_rn(float(v & 0xFFu), m);
	out[i * 3 + 1] = __fmul_rn(float((v >> 8) & 0xFFu), m);
	out[i * 3 + 2] = __fmul_rn(float((v >> 16) & 0xFFu), m);
}

__global__ void __launch_bounds__(LM_BLOCK) lightmap_directional_kernel(const uint8_t* __restrict__ in, uint64_t n,
	SwDirectionalLightmapElement* __restrict__ out)
{
	constexpr uint32_t IN_BYTES = LM_BLOCK * 13;                                          // 3328 = 208 x 16
	constexpr uint32_t OUT_WORDS = LM_BLOCK * sizeof(SwDirectionalLightmapElement) / 16; // 640
	__shared__ __align__(16) uint8_t s_in[IN_BYTES];
	__shared__ __align__(16) float s_out[LM_BLOCK * 10];
	const uint64_t first = uint64_t(blockIdx.x) * LM_BLOCK;
	const uint32_t count = n - first < LM_BLOCK ? uint32_t(n - first) : LM_BLOCK;
	const uint8_t* src = in + first * 13;
	const uint32_t bytes = count * 13;
	if (count == LM_BLOCK) // whole block: 16-byte words (the input base is 16-byte aligned, 3328 = 208 x 16)
	{
		for (uint32_t w = threadIdx.x; w < IN_BYTES / 16; w += LM_BLOCK)
			reinterpret_cast<uint4*>(s_in)[w] = __ldg(reinterpret_cast<const uint4*>(src) + w);
	}
	else
	{
		for (uint32_t b = threadIdx.x; b < bytes; b += LM_BLOCK) s_in[b] = __ldg(src + b);
	}
	__syncthreads();
	if (threadIdx.x < count)
	{
		const uint8_t* e = s_in + threadIdx.x * 13;
		float* o = s_out + threadIdx.x * 10;
		const float ma = __fdiv_rn(float(e[3]), 255.0f);
		o[0] = __fmul_rn(float(e[0]), ma);
		o[1] = __fmul_rn(float(e[1]), ma);
		o[2] = __fmul_rn(float(e[2]), ma);
		const float mv = __fdiv_rn(float(e[7]), 127.0f);
		const float dx = __fmul_rn(float(int8_t(e[4])), mv);
		const float dy = __fmul_rn(float(int8_t(e[5])), mv);
		const float dz = __fmul_rn(float(int8_t(e[6])), mv);
		const bool zero = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) <= 0.0f;
		o[3] = zero ? 0.0f : dx;
		o[4] = zero ? 0.0f : dy;
		o[5] = zero ? 1.0f / 1024.0f : dz;
		o[6] = __fdiv_rn(float(e[8]), 255.0f);
		const float mc = __fdiv_rn(float(e[12]), 255.0f);
		o[7] = __fmul_rn(float(e[9]), mc);
		o[8] = __fmul_rn(float(e[10]), mc);
		o[9] = __fmul_rn(float(e[11]), mc);
	}
	__syncthreads();
	float* dst = reinterpret_cast<float*>(out + first);
	if (count == LM_BLOCK) // 40 x 256 bytes from a 16-byte aligned start (first x 40 is a multiple of 16 here)
	{
		for (uint32_t w = threadIdx.x; w < OUT_WORDS; w += LM_BLOCK)
			reinterpret_cast<uint4*>(dst)[w] = reinterpret_cast<const uint4*>(s_out)[w];
	}
	else
	{
		for (uint32_t f = threadIdx.x; f < count * 10; f += LM_BLOCK) dst[f] = s_out[f];
	}
}

} // namespace

int launch_lightmap_decompress(const void* simple_in, uint64_t num_simple, float* simple_out, const void* dir_in,
	uint64_t num_dir, SwDirectionalLightmapElement* dir_out, cudaStream_t stream)
{
	if (num_simple)
		lightmap_simple_kernel<<<unsigned((num_simple + LM_BLOCK - 1) / LM_BLOCK), LM_BLOCK, 0, stream>>>(
			static_cast<const uint32_t*>(simple_in), num_simple, simple_out);
	if (num_dir)
		lightmap_directional_kernel<<<unsigned((num_dir + LM_BLOCK - 1) / LM_BLOCK), LM_BLOCK, 0, stream>>>(
			static_cast<const uint8_t*>(dir_in), num_dir, dir_out);
	return int(cudaGetLastError());
}

} // namespace swgpu
