// sw_postprocess_noalloc: the HDR postprocessor for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: an engine that hands out all device memory
// from its own fixed-size pools (a direct cudaMalloc would bypass its budget), or a real-time frame
// loop where cudaMalloc's implicit device synchronisation would stall the frame. sw_postprocess
// needs a context, and a context allocates its bloom buffers; this entry point needs neither. The
// caller passes the HDR frame and the output frame in device memory; the bloom buffers, the per-line
// sums and the average colour live in one file-scope device array of fixed size, which every GPU that
// loads the library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the array's device address
// with cudaGetSymbolAddress and caches it for that device; a host-side symbol is not a device address,
// so kernels only ever receive the looked-up pointer. Make that first call on each device before any
// stream capture. cudaDeviceReset unloads the module and the cached address goes stale with it: the
// entry point is not for processes that reset a device and keep using the library.
// Sharing: every call on a device uses the same array and leaves its contents behind; the per-line
// sums that must start at zero are cleared by each call. Calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the array: serialise them.
#include "sw_kernels.cuh"

#include <cmath>
#include <cstring>
#include <mutex>

namespace
{

constexpr uint32_t MAX_W = SW_NOALLOC_MAX_WIDTH;
constexpr uint32_t MAX_H = SW_NOALLOC_MAX_HEIGHT;
constexpr size_t BLOOM_PIXELS = size_t(MAX_W / 2) * (MAX_H / 2); // the smallest bloom scale is 2
constexpr size_t OFF_BLOOM0 = 0;
constexpr size_t OFF_BLOOM1 = OFF_BLOOM0 + BLOOM_PIXELS * 8;
constexpr size_t OFF_LINE_SUMS = OFF_BLOOM1 + BLOOM_PIXELS * 8; // (MAX_H / 2) lines x 4 int32 lanes
constexpr size_t OFF_LINE_SUMS_F = OFF_LINE_SUMS + size_t(MAX_H / 2) * 16; // MAX_H lines x 4 f32 lanes
constexpr size_t OFF_AVERAGE = OFF_LINE_SUMS_F + size_t(MAX_H) * 16;
constexpr size_t SCRATCH_BYTES = (OFF_AVERAGE + 16 + 255) / 256 * 256;
static_assert(SCRATCH_BYTES == SW_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void* g_scratch[MAX_DEVICES] = {};

} // namespace

// The scratch array. In host code this name is only a host-side stand-in; kernels get the address
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_postprocess_scratch[SCRATCH_BYTES];

namespace
{

// Device address of the scratch array on the current device (looked up once per device).
int scratch_for_current_device(unsigned char** out)
{
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess)
	{
		cudaGetLastError();
		return SW_ERR_CUDA;
	}
	if (dev < 0 || dev >= MAX_DEVICES) return SW_ERR_LIMIT;
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	if (!g_scratch[dev])
	{
		void* p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_postprocess_scratch);
		if (e != cudaSuccess || !p)
		{
			cudaGetLastError();
			return SW_ERR_CUDA;
		}
		g_scratch[dev] = p;
	}
	*out = static_cast<unsigned char*>(g_scratch[dev]);
	return SW_OK;
}

} // namespace

extern "C" int sw_postprocess_noalloc(const uint64_t* hdr, uint32_t width, uint32_t height, const SwPostConfig* config,
	float exposure, const float color_modulate[3], uint32_t* dst, uint32_t pitch, float* average, void* stream)
{
	if (!hdr || !dst || !config || !color_modulate || !(exposure > 0.0f)) return SW_ERR_INVALID_ARGUMENT;
	if (width == 0 || height == 0 || pitch < width) return SW_ERR_INVALID_ARGUMENT;
	if (width > MAX_W || height > MAX_H) return SW_ERR_LIMIT; // the scratch array is sized for MAX_W x MAX_H
	unsigned char* scratch = nullptr;
	int r = scratch_for_current_device(&scratch);
	if (r) return r;

	swgpu::PostArgs a;
	std::memset(&a, 0, sizeof(a));
	a.hdr = hdr;
	a.bloom0 = reinterpret_cast<uint64_t*>(scratch + OFF_BLOOM0);
	a.bloom1 = reinterpret_cast<uint64_t*>(scratch + OFF_BLOOM1);
	a.line_sums = reinterpret_cast<int32_t*>(scratch + OFF_LINE_SUMS);
	a.line_sums_f = reinterpret_cast<float*>(scratch + OFF_LINE_SUMS_F);
	a.average = average ? average : reinterpret_cast<float*>(scratch + OFF_AVERAGE);
	// The same tonemapping factors and bloom weights as the context's postprocessor, from the
	// configuration as synchronize_config clamps it (bloom scales 2..8, so the bloom buffers fit).
	if (!swgpu::post_args_from_config(a, swgpu::post_config_clamped(*config), exposure, color_modulate, width, height))
		return SW_ERR_INVALID_ARGUMENT;
	a.dst = dst;
	a.dst_pitch = pitch;
	// launch_postprocess clears the per-line integer sums before accumulating into them.
	const int e = swgpu::launch_postprocess(a, 0, static_cast<cudaStream_t>(stream));
	return e == 0 ? SW_OK : SW_ERR_CUDA;
}
