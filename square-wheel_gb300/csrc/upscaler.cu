// Learned 2x upscaler (include/swlearn.h): tcgen05 implicit-GEMM 3x3 convolutions (forward, input
// gradient, weight gradient), the pixel-shuffle / bilinear-residual / loss epilogue, Adam, PSNR.
//
// Activation layout in HBM ("row planes"): per image, per row (one halo row above, zero rows below),
// per 8-channel chunk, per pixel (one halo pixel left, zero pixels right) 8 bf16 = 16 bytes:
//   element (img, y, chunk, x, e) at ((img * rows_alloc + y + 1) * chunks + chunk) * wp * 8 + (x + 1) * 8 + e
// A row of 128 pixels of one chunk is therefore 128 contiguous 16-byte rows, which is exactly a stack of
// 16 UMMA core matrices (8 pixels x 16 bytes): an M tile of the implicit GEMM is 128 consecutive pixels of
// one image row, and a tap (dy, dx) of the 3x3 kernel only moves the descriptor's start address. Halo and
// padding pixels are zeroed once at allocation and never written, which gives the zero padding of the
// convolution and of its transpose.
//
// conv_kernel: one CTA = 4 output rows x 128 pixels of one image. One thread bulk-copies (TMA, untiled)
// the 6 input rows x chunks x 130 pixels and the packed weights into shared memory, issues
// 4 rows x 9 taps x (chunks / 2) MMAs of 128 x N x 16 into TMEM (4 x N columns), and commits to an
// mbarrier; 4 warps then read the accumulators (warp w = TMEM lanes 32w.., i.e. pixels 32w..) and run
// the epilogue: bias + ReLU (forward), ReLU mask (input gradient), or the output stage (pixel shuffle +
// bilinear residual, written as Color32 for inference or as the loss gradient for training).
// wgrad_kernel: weight gradient dW[co][dy][dx][ci] = sum_p G[p][co] X[p + (dy, dx)][ci] with both operands
// MN-major: D rows = (dy, chunk, ci % 8) groups at a uniform shared-memory stride, D columns = co, one
// accumulator per dx, K = 16 pixels per MMA; per-CTA partial sums are reduced in a fixed order.
#include "sw_kernels.cuh"
#include "tc05.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "../../include/swlearn.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace swgpu;
using namespace swgpu::tc05;

namespace
{

constexpr int TILE_X = 128;            // pixels per M tile
constexpr int ROWS = 4;                // output rows per CTA
constexpr int XS = TILE_X + 2;         // staged pixels per row and chunk (one halo pixel each side)
constexpr uint32_t XS_BYTES = XS * 16; // 2080
constexpr uint32_t POLL_LIMIT = 1u << 21;
constexpr int NUM_LAYERS = 4;

// Layer shapes: real channel counts and the padded ones the MMAs use.
struct LayerShape
{
	int cin, cout;     // real
	int c8_in, n_out;  // input chunks (8 channels each), padded output channels
	int param_offset;  // weights, then bias at param_offset + cout*9*cin
};
constexpr LayerShape LAYERS[NUM_LAYERS] = {
	{3, 32, 2, 32, 0},
	{32, 32, 4, 32, 896},
	{32, 32, 4, 32, 896 + 9248},
	{32, 12, 4, 16, 896 + 2 * 9248},
};
static_assert(896 + 2 * 9248 + 3468 == SW_UPSCALER_NUM_PARAMS, "parameter count");
__constant__ LayerShape c_layers[NUM_LAYERS] = {
	{3, 32, 2, 32, 0},
	{32, 32, 4, 32, 896},
	{32, 32, 4, 32, 896 + 9248},
	{32, 12, 4, 16, 896 + 2 * 9248},
};

struct Planes
{
	uint16_t* data; // bf16 bits
	uint32_t images, height, width, chunks, wp, rows_alloc;
};

__host__ __device__ __forceinline__ size_t planes_index(const Planes& p, uint32_t img, int y, uint32_t chunk, int x)
{
	return ((size_t(img) * p.rows_alloc + size_t(y + 1)) * p.chunks + chunk) * p.wp * 8 + size_t(x + 1) * 8;
}

struct CropGpu
{
	const uint32_t* lo;
	const uint32_t* hi;
	uint32_t lo_w, lo_h, lo_pitch, hi_pitch;
	int32_t x, y;
};

enum Epi
{
	EPI_RELU = 0,  // out = bf16(max(acc + bias, 0))
	EPI_MASK = 1,  // out = bf16(acc * (mask > 0))
	EPI_INFER = 2, // Color32 output frame
	EPI_LOSS = 3,  // loss gradient planes + loss partial sums
};

struct ConvArgs
{
	CUtensorMap in_map; // rows of `in`: box = 8 channels x 130 pixels x all chunks x 1 row
	Planes in, out, mask;
	const uint16_t* wpack;
	const float* bias;
	const CropGpu* crops; // EPI_INFER / EPI_LOSS: one per image
	uint32_t* hi_out;     // EPI_INFER
	uint32_t hi_pitch;
	float* loss_partial; // EPI_LOSS: one per CTA
	uint32_t margin;
	int* error;
};

__device__ __forceinline__ uint16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float(uint32_t(h) << 16); }
__device__ __forceinline__ uint32_t pack2(float a, float b) { return uint32_t(f2bf(a)) | (uint32_t(f2bf(b)) << 16); }

__device__ __forceinline__ uint32_t to_byte(float v)
{
	const float s = rintf(v * 255.0f);
	return uint32_t(fminf(fmaxf(s, 0.0f), 255.0f));
}

constexpr int NSTAGE = 6;    // input rows staged in shared memory (ring)
constexpr int CONV_RING = 8; // TMEM output-row accumulators of the convolution

// Staged input row of the convolution: pixels x0 - 1 .. x0 + 134 of every chunk (17 groups of 8 pixels;
// pixel x0 - 1 starts a 128-byte group because of the layout's one-pixel halo offset), so the TMA box's
// innermost extent is a whole 128-byte group of 8 pixels x 8 channels.
constexpr int CXS = 136;
constexpr uint32_t CXS_BYTES = CXS * 16; // 2176: chunk stride of a staged row
// Ring slot of one staged input row: a tiled TMA destination must be 128-byte aligned.
template <int C8>
__host__ __device__ constexpr uint32_t conv_slot_bytes()
{
	return (C8 * CXS_BYTES + 127) / 128 * 128;
}
template <int C8, int N>
__host__ __device__ constexpr uint32_t conv_smem_bytes()
{
	return NSTAGE * conv_slot_bytes<C8>() + 9 * (C8 / 2) * 2 * N * 16 + 512;
}
template <int N>
__host__ __device__ constexpr uint32_t conv_tmem_cols()
{
	return CONV_RING * N <= 128 ? 128 : 256;
}

// Rows [begin, end) of the (strip, y) order a persistent CTA owns; strip = image * tiles_x + x tile.
struct RowRange
{
	uint32_t begin, end;
};
__device__ __forceinline__ RowRange cta_rows(uint32_t total)
{
	return RowRange{uint32_t(uint64_t(blockIdx.x) * total / gridDim.x), uint32_t(uint64_t(blockIdx.x + 1) * total / gridDim.x)};
}

// Epilogue of one output row for the 128 pixels of a tile: thread = pixel x, v = the row's N accumulators
// (all N loaded; `half` selects the work share of the two warps reading the same TMEM lane quadrant):
//   EPI_RELU / EPI_MASK: channels [half * N / 2, (half + 1) * N / 2);
//   EPI_INFER: output row 2y + half;  EPI_LOSS: half 0 only (the loss gradient planes need whole pixels).
template <int N, int EPI, int half>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, const float (&v)[N], const float (&bias)[N], uint32_t img,
	int x, int y, float& loss)
{
	if (x >= int(a.in.width) || y >= int(a.in.height)) return; // padding pixels stay zero
	if (EPI == EPI_RELU || EPI == EPI_MASK)
	{
		uint16_t* out = a.out.data + planes_index(a.out, img, y, 0, x);
		const size_t cstride = size_t(a.out.wp) * 8;
		const uint16_t* msk = EPI == EPI_MASK ? a.mask.data + planes_index(a.mask, img, y, 0, x) : nullptr;
#pragma unroll
		for (int cc = 0; cc < N / 16; ++cc)
		{
			const int c8 = half * (N / 16) + cc;
			uint32_t o[4];
			if (EPI == EPI_RELU)
			{
#pragma unroll
				for (int q = 0; q < 4; ++q)
					o[q] = pack2(fmaxf(v[c8 * 8 + 2 * q] + bias[c8 * 8 + 2 * q], 0.0f),
						fmaxf(v[c8 * 8 + 2 * q + 1] + bias[c8 * 8 + 2 * q + 1], 0.0f));
			}
			else
			{
				const uint4 m = *reinterpret_cast<const uint4*>(msk + c8 * cstride);
				const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
				for (int q = 0; q < 4; ++q)
				{
					// ReLU derivative: the stored activation is > 0 (sign clear, magnitude non-zero)
					const float g0 = (mw[q] & 0x7FFFu) && !(mw[q] & 0x8000u) ? v[c8 * 8 + 2 * q] : 0.0f;
					const float g1 = (mw[q] & 0x7FFF0000u) && !(mw[q] & 0x80000000u) ? v[c8 * 8 + 2 * q + 1] : 0.0f;
					o[q] = pack2(g0, g1);
				}
			}
			*reinterpret_cast<uint4*>(out + c8 * cstride) = make_uint4(o[0], o[1], o[2], o[3]);
		}
	}
	else
	{
		// Output stage: channel c*4 + sy*2 + sx is colour c of output pixel (2x + sx, 2y + sy), added to
		// the bilinear 2x upsample of the source (weights 3/4, 1/4; edges clamped).
		if (EPI == EPI_LOSS && half) return;
		const CropGpu c = a.crops[img];
		const int lx = c.x + x, ly = c.y + y;
		const int xs[3] = {max(lx - 1, 0), lx, min(lx + 1, int(c.lo_w) - 1)};
		const int ys[3] = {max(ly - 1, 0), ly, min(ly + 1, int(c.lo_h) - 1)};
		float g[16];
#pragma unroll
		for (int j = 0; j < 16; ++j) g[j] = 0.0f;
		const bool in_loss = EPI == EPI_LOSS && x >= int(a.margin) && x < int(a.in.width - a.margin) &&
			y >= int(a.margin) && y < int(a.in.height - a.margin);
#pragma unroll
		for (int sy = 0; sy < 2; ++sy)
		{
			if (EPI == EPI_INFER && sy != half) continue;
			const uint32_t* r1 = c.lo + size_t(ly) * c.lo_pitch;
			const uint32_t* r2 = c.lo + size_t(ys[sy ? 2 : 0]) * c.lo_pitch;
			const uint32_t p11 = r1[lx], p10 = r1[xs[0]], p12 = r1[xs[2]];
			const uint32_t p21 = r2[lx], p20 = r2[xs[0]], p22 = r2[xs[2]];
			uint32_t tp[2] = {0u, 0u};
			if (EPI == EPI_LOSS)
			{
				const uint2 t2 = *reinterpret_cast<const uint2*>(c.hi + size_t(2 * ly + sy) * c.hi_pitch + 2 * lx);
				tp[0] = t2.x;
				tp[1] = t2.y;
			}
			uint32_t px[2];
#pragma unroll
			for (int sx = 0; sx < 2; ++sx)
			{
				const int s = sy * 2 + sx;
				const uint32_t a01 = sx ? p12 : p10, a11 = sx ? p22 : p20;
				uint32_t bytes = p11 & 0xFF000000u; // alpha of the source pixel
#pragma unroll
				for (int ch = 0; ch < 3; ++ch)
				{
					const float top = 0.75f * float((p11 >> (8 * ch)) & 255u) + 0.25f * float((a01 >> (8 * ch)) & 255u);
					const float bot = 0.75f * float((p21 >> (8 * ch)) & 255u) + 0.25f * float((a11 >> (8 * ch)) & 255u);
					const float pred = (0.75f * top + 0.25f * bot) * (1.0f / 255.0f) + (v[ch * 4 + s] + bias[ch * 4 + s]);
					if (EPI == EPI_INFER)
						bytes |= to_byte(pred) << (8 * ch);
					else
					{
						const float d = in_loss ? pred - float((tp[sx] >> (8 * ch)) & 255u) * (1.0f / 255.0f) : 0.0f;
						g[ch * 4 + s] = d;
						loss += d * d;
					}
				}
				px[sx] = bytes;
			}
			if (EPI == EPI_INFER)
				*reinterpret_cast<uint2*>(a.hi_out + size_t(2 * ly + sy) * a.hi_pitch + 2 * lx) = make_uint2(px[0], px[1]);
		}
		if (EPI == EPI_LOSS)
		{
			uint16_t* out = a.out.data + planes_index(a.out, img, y, 0, x);
#pragma unroll
			for (int c8 = 0; c8 < 2; ++c8)
			{
				uint32_t o[4];
#pragma unroll
				for (int q = 0; q < 4; ++q) o[q] = pack2(g[c8 * 8 + 2 * q], g[c8 * 8 + 2 * q + 1]);
				*reinterpret_cast<uint4*>(out + c8 * size_t(a.out.wp) * 8) = make_uint4(o[0], o[1], o[2], o[3]);
			}
		}
	}
}

// Persistent, warp-specialised 3x3 convolution over row planes (CONV_THREADS = 320 threads). The three
// vertical taps are folded into the MMA's N dimension: input row y_in times the weights of all three ky
// gives, for output rows y_in + 1, y_in, y_in - 1, their ky = 0, 1, 2 contributions side by side
// (N = 3 x C_out), accumulated in place into a TMEM ring of R output-row accumulators (C_out columns
// each; the row with counter o sits at block (R - o % R) % R, so rows y_in + 1, y_in, y_in - 1 are
// consecutive blocks; a group that wraps the ring is split in two MMAs). Accumulators start at zero
// (the epilogue zeroes each one after reading it), so every MMA accumulates. One input row is read by
// 3 x (C8 / 2) MMAs of 128 x 3N x 16 and released; an output row is complete after input row y + 1.
//   warp 0 (one lane): bulk-copies the packed weights once, then loads input rows (all chunks, 136
//     pixels; one tiled TMA each) into a ring of NSTAGE shared-memory rows;
//   warp 1 (one lane; the warp owns the TMEM allocation): per input row waits for it (and, when it
//     starts a new output row, for that row's accumulator to be free), issues the MMAs and commits the
//     row to rowbar[k % NBAR]: that releases the input row's slot and completes output row y_in - 1;
//   warps 2..9: per output row: TMEM -> registers (warp w reads lanes 32*(w%4).., i.e. pixels), zero
//     the accumulator, release it, run the epilogue and store (the two warps of a lane quadrant split
//     the columns and the epilogue work).
// The issuing thread's own instruction latency bounds the MMA rate, so the common case (three
// contributions, no ring wrap) is straight-line code with compile-time descriptor offsets.
// Every wait is bounded: on expiry the role stops, the error flag is set, and the CTA still waits for
// its own MMAs and copies before freeing TMEM.
constexpr int CONV_THREADS = 320;
constexpr int CONV_EPI_WARPS = 8;
constexpr int NBAR = 16; // row-completion barriers (more than the rows the MMA issuer can run ahead)

// Named barrier 1 of the 8 epilogue warps; epi_any is the same barrier returning the OR of `v` over them
// (so all eight take the same branch).
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ bool epi_any(bool v)
{
	uint32_t r;
	asm volatile("{\n\t.reg .pred q, p;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, 256, q;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
				 : "=r"(r)
				 : "r"(v ? 1u : 0u)
				 : "memory");
	return r != 0;
}

template <int C8, int N, int EPI>
__global__ void __launch_bounds__(CONV_THREADS, 1) conv_kernel(const __grid_constant__ ConvArgs a)
{
	constexpr int KSTEPS = C8 / 2;      // 16-channel steps per horizontal tap
	constexpr int NB = 3 * N;           // MMA N for a whole input row
	constexpr int R = CONV_RING;        // TMEM output-row accumulators
	constexpr uint32_t ROW_BYTES = C8 * CXS_BYTES;       // bytes of one staged row (the TMA box)
	constexpr uint32_t SLOT_BYTES = conv_slot_bytes<C8>(); // ring stride (128-byte aligned)
	constexpr uint32_t W_BYTES = 3 * KSTEPS * 2 * NB * 16;
	constexpr uint32_t TMEM_COLS = conv_tmem_cols<N>();
	static_assert(C8 % 2 == 0 && N % 16 == 0 && N <= 32, "shape");
	extern __shared__ __align__(1024) unsigned char smem[];
	unsigned char* s_ring = smem;
	unsigned char* s_w = smem + NSTAGE * SLOT_BYTES;
	uint64_t* full = reinterpret_cast<uint64_t*>(s_w + W_BYTES);
	uint64_t* rowbar = full + NSTAGE;
	uint64_t* acce = rowbar + NBAR;
	uint64_t* wbar = acce + R;
	uint64_t* donebar = wbar + 1;
	uint32_t* s_tmem = reinterpret_cast<uint32_t*>(donebar + 1);
	float* s_red = reinterpret_cast<float*>(s_tmem + 4); // [CONV_EPI_WARPS]

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t H = a.in.height;
	const uint32_t tiles_x = (a.in.width + TILE_X - 1) / TILE_X;
	const RowRange rows = cta_rows(a.in.images * tiles_x * H);

	if (tid == 0)
	{
		for (int i = 0; i < NSTAGE; ++i) mbar_init(&full[i], 1);
		for (int i = 0; i < NBAR; ++i) mbar_init(&rowbar[i], 1);
		for (int i = 0; i < R; ++i) mbar_init(&acce[i], CONV_EPI_WARPS);
		mbar_init(wbar, 1);
		mbar_init(donebar, 1);
		fence_mbar_init();
	}
	if (warp == 1)
	{
		tmem_alloc(s_tmem, TMEM_COLS);
		tmem_relinquish();
	}
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	const uint32_t tmem = *s_tmem;
	if (warp >= 2)
	{
		// every accumulator starts at zero (the MMAs always accumulate)
		const uint32_t lane_base = uint32_t((warp & 3) * 32) << 16;
		const int half = (warp - 2) >> 2;
		for (int c = half * (R * N / 2); c < (half + 1) * (R * N / 2); c += 8) tmem_zero8(tmem + lane_base + c);
		tmem_st_wait();
	}
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	bool failed = false;

	if (warp == 0)
	{
		if (lane == 0)
		{
			mbar_expect_tx(wbar, W_BYTES);
			bulk_g2s(s_w, a.wpack, W_BYTES, wbar);
			uint32_t k = 0;
			for (uint32_t r = rows.begin; r < rows.end && !failed;)
			{
				const uint32_t strip = r / H, y_lo = r % H, y_hi = min(H, y_lo + (rows.end - r));
				r += y_hi - y_lo;
				const uint32_t img = strip / tiles_x;
				const int x0 = int(strip % tiles_x) * TILE_X;
				for (int yi = int(y_lo) - 1; yi <= int(y_hi); ++yi, ++k)
				{
					const uint32_t slot = k % NSTAGE;
					if (k >= NSTAGE)
					{
						// the slot's previous row (k - NSTAGE) has been consumed by its MMAs
						const uint32_t kp = k - NSTAGE;
						if (!mbar_wait_bounded(&rowbar[kp % NBAR], (kp / NBAR) & 1, POLL_LIMIT))
						{
							failed = true;
							break;
						}
					}
					mbar_expect_tx(&full[slot], ROW_BYTES);
					// one tiled TMA per input row: pixels x0 - 1 .. x0 + 134 of all chunks
					tma_load_4d(s_ring + slot * SLOT_BYTES, &a.in_map, 0, x0 / 8, 0, int(img * a.in.rows_alloc) + yi + 1, &full[slot]);
				}
			}
			// drain: the last fill of every slot has landed before the CTA can exit
			for (uint32_t kk = k > NSTAGE ? k - NSTAGE : 0; kk < k; ++kk)
				mbar_wait_bounded(&full[kk % NSTAGE], (kk / NSTAGE) & 1, POLL_LIMIT);
		}
	}
	else if (warp == 1)
	{
		if (lane == 0)
		{
			// Descriptors are precomputed: the start-address field is the low 14 bits (address >> 4), so a
			// descriptor of base + off is the base descriptor + (off >> 4) (shared addresses stay < 256 KB).
			const uint64_t a_base = make_sdesc(smem_addr(s_ring), CXS_BYTES, 128);
			const uint64_t b_base = make_sdesc(smem_addr(s_w), NB * 16, 128);
			constexpr uint32_t IDESC1 = make_idesc_bf16(128, N, 0, 0);
			constexpr uint32_t IDESC2 = make_idesc_bf16(128, 2 * N, 0, 0);
			constexpr uint32_t IDESC3 = make_idesc_bf16(128, 3 * N, 0, 0);
			failed = !mbar_wait_bounded(wbar, 0, POLL_LIMIT);
			uint32_t k = 0, o_base = 0;
			for (uint32_t r = rows.begin; r < rows.end && !failed;)
			{
				const uint32_t y_lo = r % H, y_hi = min(H, y_lo + (rows.end - r));
				r += y_hi - y_lo;
				for (int yi = int(y_lo) - 1; yi <= int(y_hi); ++yi, ++k)
				{
					failed = !mbar_wait_bounded(&full[k % NSTAGE], (k / NSTAGE) & 1, POLL_LIMIT);
					// contributions j = 0, 1, 2 go to output rows yi + 1 - j; keep those in [y_lo, y_hi)
					const int j_lo = max(0, yi + 2 - int(y_hi)), j_hi = min(2, yi + 1 - int(y_lo));
					const uint32_t o_first = o_base + uint32_t(yi + 1 - j_lo - int(y_lo)); // counter of row yi + 1 - j_lo
					const uint32_t b0 = (R - o_first % R) % R;
					if (!failed && j_lo == 0 && o_first >= R) // a new row's accumulator must have been drained
						failed = !mbar_wait_bounded(&acce[b0], ((o_first / R) - 1) & 1, POLL_LIMIT);
					if (failed) break;
					fence_after_sync();
					const uint64_t a_row = a_base + (((k % NSTAGE) * SLOT_BYTES) >> 4);
					if (j_lo == 0 && j_hi == 2 && b0 + 3 <= uint32_t(R))
					{
						// common case: one MMA per K step over the three blocks
						const uint32_t d = tmem + b0 * N;
#pragma unroll
						for (int dx = 0; dx < 3; ++dx)
#pragma unroll
							for (int ks = 0; ks < KSTEPS; ++ks)
								mma_bf16(d, a_row + ((2 * ks * CXS_BYTES + dx * 16) >> 4),
									b_base + (((dx * KSTEPS + ks) * (2 * NB * 16)) >> 4), IDESC3, 1u);
					}
					else
					{
						// segment edges (fewer contributions) and ring wraps: at most two pieces
						const int nj = j_hi - j_lo + 1;
						const int len0 = min(nj, int(R - b0));
						const uint32_t d0 = tmem + b0 * N, d1 = tmem;
						const uint32_t bo0 = uint32_t(j_lo * N * 16) >> 4, bo1 = uint32_t((j_lo + len0) * N * 16) >> 4;
						const uint32_t id0 = len0 == 1 ? IDESC1 : len0 == 2 ? IDESC2 : IDESC3;
						const uint32_t id1 = nj - len0 == 1 ? IDESC1 : IDESC2;
						const bool two = len0 < nj;
#pragma unroll
						for (int dx = 0; dx < 3; ++dx)
#pragma unroll
							for (int ks = 0; ks < KSTEPS; ++ks)
							{
								const uint64_t ad = a_row + ((2 * ks * CXS_BYTES + dx * 16) >> 4);
								const uint64_t bk = b_base + (((dx * KSTEPS + ks) * (2 * NB * 16)) >> 4);
								mma_bf16(d0, ad, bk + bo0, id0, 1u);
								if (two) mma_bf16(d1, ad, bk + bo1, id1, 1u);
							}
					}
					// one commit: the input row's slot is free and output row yi - 1 (if j_hi == 2) complete
					mma_commit(&rowbar[k % NBAR]);
				}
				if (failed) break;
				o_base += y_hi - y_lo;
			}
			mma_commit(donebar);
			if (!mbar_wait_bounded(donebar, 0, POLL_LIMIT)) failed = true;
		}
	}
	else
	{
		const int quad = warp & 3, half = (warp - 2) >> 2;
		const uint32_t lane_base = uint32_t(quad * 32) << 16;
		float bias[N];
#pragma unroll
		for (int c = 0; c < N; ++c) bias[c] = EPI == EPI_MASK ? 0.0f : a.bias[c];
		float loss = 0.0f;
		uint32_t o = 0, k_base = 0;
		for (uint32_t r = rows.begin; r < rows.end && !failed;)
		{
			const uint32_t strip = r / H, y_lo = r % H, y_hi = min(H, y_lo + (rows.end - r));
			r += y_hi - y_lo;
			const uint32_t img = strip / tiles_x;
			const int x = int(strip % tiles_x) * TILE_X + quad * 32 + lane;
			for (uint32_t y = y_lo; y < y_hi; ++y, ++o)
			{
				// output row y is complete once input row y + 1 (ring entry k_base + y - y_lo + 2) is committed
				const uint32_t kc = k_base + (y - y_lo) + 2;
				const bool ok = mbar_wait_bounded(&rowbar[kc % NBAR], (kc / NBAR) & 1, POLL_LIMIT);
				if (epi_any(!ok))
				{
					failed = true;
					break;
				}
				fence_after_sync();
				const uint32_t b = (R - o % R) % R;
				float v[N];
#pragma unroll
				for (int c8 = 0; c8 < N / 8; ++c8)
				{
					float t8[8];
					tmem_ld8(tmem + lane_base + b * N + c8 * 8, t8);
#pragma unroll
					for (int e = 0; e < 8; ++e) v[c8 * 8 + e] = t8[e];
				}
				tmem_ld_wait();
				epi_sync(); // both warps of the quadrant have read the accumulator
#pragma unroll
				for (int c8 = 0; c8 < N / 16; ++c8) tmem_zero8(tmem + lane_base + b * N + (half * (N / 16) + c8) * 8);
				tmem_st_wait();
				fence_before_sync();
				__syncwarp();
				if (lane == 0) mbar_arrive(&acce[b]);
				if (half)
					conv_epilogue<N, EPI, 1>(a, v, bias, img, x, int(y), loss);
				else
					conv_epilogue<N, EPI, 0>(a, v, bias, img, x, int(y), loss);
			}
			k_base += (y_hi - y_lo) + 2;
		}
		if (EPI == EPI_LOSS)
		{
			for (int o2 = 16; o2 > 0; o2 >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o2);
			if (lane == 0) s_red[warp - 2] = loss;
		}
	}
	if (failed) atomicExch(a.error, 1);
	fence_before_sync();
	__syncthreads();
	if (EPI == EPI_LOSS && tid == 0)
	{
		float t = 0.0f;
		for (int w = 0; w < CONV_EPI_WARPS; ++w) t += s_red[w];
		a.loss_partial[blockIdx.x] = t;
	}
	if (warp == 1)
	{
		fence_after_sync();
		tmem_dealloc(tmem, TMEM_COLS);
	}
}

// ---- fused inference: all four layers in one kernel ----
//
// One CTA owns a strip of 128 computed columns [c0, c0 + 128), c0 = 120 t - 4, and a segment of output
// rows [y_lo, y_hi). Every layer computes the strip's 128 columns; a column's value is exact while its
// receptive field lies inside the strip, so after four 3x3 layers the middle 120 columns are exact and
// are the strip's output (8 strips tile 960 columns). Layer l computes rows [y_lo - 3 + l, y_hi + 3 - l),
// reading rows one further up and down; rows or columns outside the frame are zero, exactly as the zero
// padding of the layer-by-layer convolution.
//
// Activations never leave the SM: layer l's input rows live in a shared-memory ring of FNS rows of
// C8_l chunks x 136 pixels (the layout conv_kernel stages from HBM), written by
//   warp 0 (all lanes) for layer 0: Color32 source -> (b, g, r) / 255 in bf16 (the input conversion),
//   the epilogue warps of layer l - 1 for layers 1..3: TMEM -> bias + ReLU -> bf16.
// MMAs are the dy-folded implicit GEMM of conv_kernel (128 pixels x 3 C_out x 16 per MMA, accumulated
// in place in a TMEM ring of 4 output rows per layer), issued by two threads: warp 1 for layers 0 and
// 2, warp 10 for layers 1 and 3 (in step s, layer l's input row s - FLAG l). Epilogue warps 2..5 drain
// layers 0 and 2, warps 6..9 layers 1 and 3 (the last one writes the Color32 output: pixel shuffle +
// bilinear residual); in step s they handle layer l's output row s - 2 - FLAG l. A layer's output row is
// complete two rows after its first input row, so FLAG - 2 steps of slack separate the epilogue that
// writes a row from the MMAs that read it: enough to cover the tensor pipe's queue and the epilogue
// itself, so that the roles run as a pipeline rather than a chain. The slot an epilogue writes was read
// about FNS + 2 - FLAG steps earlier.
constexpr int FNS = 5;          // input-row slots per layer
constexpr int FR = 4;           // TMEM output-row accumulators per layer
constexpr int FLAG = 5;         // rows of lag between layers
constexpr int F_THREADS = 352;  // 11 warps
constexpr int F_VALID = 120;    // output columns per strip
constexpr uint32_t F_TMEM_COLS = 512;

struct FusedArgs
{
	const uint32_t* lo;
	uint32_t lo_w, lo_h, lo_pitch;
	uint32_t* hi;
	uint32_t hi_pitch;
	const uint16_t* w[NUM_LAYERS]; // packed B operands (conv_kernel's forward layout)
	const float* bias[NUM_LAYERS];
	uint32_t strips, segments;     // grid = strips x segments
	int* error;
};

// Per-layer constants.
template <int L>
struct FL
{
	static constexpr int C8 = L == 0 ? 2 : 4;
	static constexpr int N = L == 3 ? 16 : 32;
	static constexpr int KSTEPS = C8 / 2;
	static constexpr int NB = 3 * N;
	static constexpr uint32_t SLOT = (C8 * CXS_BYTES + 127) / 128 * 128;
	static constexpr uint32_t WBYTES = 3 * KSTEPS * 2 * NB * 16;
	static constexpr uint32_t TCOL = L * 4 * 32; // TMEM column base (layers 0..2: 128 columns, 3: 64)
};

struct FusedSmem
{
	static constexpr uint32_t RING0 = 0;
	static constexpr uint32_t RING1 = RING0 + FNS * FL<0>::SLOT;
	static constexpr uint32_t RING2 = RING1 + FNS * FL<1>::SLOT;
	static constexpr uint32_t RING3 = RING2 + FNS * FL<2>::SLOT;
	static constexpr uint32_t W0 = RING3 + FNS * FL<3>::SLOT;
	static constexpr uint32_t W1 = W0 + FL<0>::WBYTES;
	static constexpr uint32_t W2 = W1 + FL<1>::WBYTES;
	static constexpr uint32_t W3 = W2 + FL<2>::WBYTES;
	static constexpr uint32_t BARS = W3 + FL<3>::WBYTES;
	// barriers: full[4][FNS], rowbar[4][NBAR], accfree[4][FR], wbar, done[2]
	static constexpr uint32_t NUM_BARS = 4 * FNS + 4 * NBAR + 4 * FR + 3;
	static constexpr uint32_t MISC = BARS + NUM_BARS * 8;
	static constexpr uint32_t TOTAL = MISC + 64;
};
static_assert(FusedSmem::TOTAL <= 227 * 1024, "fused kernel shared memory");

__device__ __forceinline__ uint32_t ring_base(int l)
{
	return l == 0 ? FusedSmem::RING0 : l == 1 ? FusedSmem::RING1 : l == 2 ? FusedSmem::RING2 : FusedSmem::RING3;
}

// Barriers of layer l: full[FNS] (input row written), rowbar[NBAR] (input row's MMAs done), accfree[FR]
// (output-row accumulator drained).
__device__ __forceinline__ uint64_t* f_full(unsigned char* smem, int l)
{
	return reinterpret_cast<uint64_t*>(smem + FusedSmem::BARS) + l * FNS;
}
__device__ __forceinline__ uint64_t* f_rowbar(unsigned char* smem, int l)
{
	return reinterpret_cast<uint64_t*>(smem + FusedSmem::BARS) + 4 * FNS + l * NBAR;
}
// Each MMA issuer commits once per step (issuer l & 1 serves layers l and l + 2; layer l's input row i
// is issued in step i + FLAG l), so "input row i of layer l consumed" is the completion of that step.
__device__ __forceinline__ bool f_wait_input_done(unsigned char* smem, int l, int i)
{
	const int s = i + FLAG * l;
	const bool ok = mbar_wait_bounded(&f_rowbar(smem, l & 1)[s % NBAR], (s / NBAR) & 1, POLL_LIMIT);
	return __all_sync(0xFFFFFFFFu, ok);
}
__device__ __forceinline__ uint64_t* f_accfree(unsigned char* smem, int l)
{
	return reinterpret_cast<uint64_t*>(smem + FusedSmem::BARS) + 4 * FNS + 4 * NBAR + l * FR;
}

// Rows of layer l of a segment: outputs [A, B), inputs [A - 1, B] (input index i <-> row A - 1 + i).
// Layer l + 1's input index i is layer l's output index i.
struct LayerRows
{
	int A, B;
	__device__ int inputs() const { return B - A + 2; }
	__device__ int outputs() const { return B - A; }
};
__device__ __forceinline__ LayerRows layer_rows(int l, int y_lo, int y_hi) { return LayerRows{y_lo - 3 + l, y_hi + 3 - l}; }

// Layer 0's source pixels of row y, columns c0 - 1 + j for j = lane + 32 k (the 136 staged pixels); 0
// outside the frame (converts to the zero padding) or when `valid` is false.
constexpr int F0_PX = (CXS + 31) / 32;
constexpr int F0_AHEAD = 3;
__device__ __forceinline__ void f0_load_row(const FusedArgs& a, int y, bool valid, int c0, int lane, uint32_t (&px)[F0_PX])
{
	const bool row_in = valid && y >= 0 && y < int(a.lo_h);
	const uint32_t* row = a.lo + size_t(row_in ? y : 0) * a.lo_pitch;
#pragma unroll
	for (int k = 0; k < F0_PX; ++k)
	{
		const int j = lane + 32 * k, x = c0 - 1 + j;
		px[k] = row_in && j < CXS && x >= 0 && x < int(a.lo_w) ? __ldg(row + x) : 0u;
	}
}

// MMA group of layer L for its input index i (row A - 1 + i): the dy-folded K steps into the TMEM ring.
// Returns false if a bounded wait expired.
template <int L>
__device__ __forceinline__ bool fused_mma(unsigned char* smem, uint32_t tmem, int y_lo, int y_hi, int i)
{
	using F = FL<L>;
	constexpr int N = F::N;
	const LayerRows lr = layer_rows(L, y_lo, y_hi);
	uint64_t* full = f_full(smem, L);
	uint64_t* accfree = f_accfree(smem, L);
	if (!mbar_wait_bounded(&full[i % FNS], (i / FNS) & 1, POLL_LIMIT)) return false;
	const int yi = lr.A - 1 + i;
	const int j_lo = max(0, yi + 2 - lr.B), j_hi = min(2, yi + 1 - lr.A);
	const uint32_t o_first = uint32_t(yi + 1 - j_lo - lr.A);
	const uint32_t b0 = (FR - o_first % FR) % FR;
	if (j_lo == 0 && o_first >= FR && !mbar_wait_bounded(&accfree[b0], ((o_first / FR) - 1) & 1, POLL_LIMIT)) return false;
	fence_after_sync();
	const uint64_t a_row = make_sdesc(smem_addr(smem + ring_base(L) + (i % FNS) * F::SLOT), CXS_BYTES, 128);
	const uint32_t wofs = L == 0 ? FusedSmem::W0 : L == 1 ? FusedSmem::W1 : L == 2 ? FusedSmem::W2 : FusedSmem::W3;
	const uint64_t b_base = make_sdesc(smem_addr(smem + wofs), F::NB * 16, 128);
	constexpr uint32_t ID1 = make_idesc_bf16(128, N, 0, 0), ID2 = make_idesc_bf16(128, 2 * N, 0, 0),
					   ID3 = make_idesc_bf16(128, 3 * N, 0, 0);
	const uint32_t tcol = tmem + F::TCOL;
	if (j_lo == 0 && j_hi == 2 && b0 + 3 <= uint32_t(FR))
	{
		const uint32_t d = tcol + b0 * N;
#pragma unroll
		for (int dx = 0; dx < 3; ++dx)
#pragma unroll
			for (int ks = 0; ks < F::KSTEPS; ++ks)
				mma_bf16(d, a_row + ((2 * ks * CXS_BYTES + dx * 16) >> 4), b_base + (((dx * F::KSTEPS + ks) * (2 * F::NB * 16)) >> 4),
					ID3, 1u);
	}
	else
	{
		const int nj = j_hi - j_lo + 1;
		const int len0 = min(nj, int(FR - b0));
		const uint32_t bo0 = uint32_t(j_lo * N * 16) >> 4, bo1 = uint32_t((j_lo + len0) * N * 16) >> 4;
		const uint32_t id0 = len0 == 1 ? ID1 : len0 == 2 ? ID2 : ID3;
		const uint32_t id1 = nj - len0 == 1 ? ID1 : ID2;
		const bool two = len0 < nj;
#pragma unroll
		for (int dx = 0; dx < 3; ++dx)
#pragma unroll
			for (int ks = 0; ks < F::KSTEPS; ++ks)
			{
				const uint64_t ad = a_row + ((2 * ks * CXS_BYTES + dx * 16) >> 4);
				const uint64_t bk = b_base + (((dx * F::KSTEPS + ks) * (2 * F::NB * 16)) >> 4);
				mma_bf16(tcol + b0 * N, ad, bk + bo0, id0, 1u);
				if (two) mma_bf16(tcol, ad, bk + bo1, id1, 1u);
			}
	}
	return true;
}

// Epilogue of layer L for its output index o (row A + o): accumulators -> registers, zero and release the
// accumulator, then the next layer's input row (layers 0..2) or the Color32 output (layer 3). The four
// warps of one group call this together (warp quad = lane quadrant = pixels quad*32..).
template <int L>
__device__ __forceinline__ bool fused_epilogue(const FusedArgs& a, unsigned char* smem, uint32_t tmem, int y_lo, int y_hi, int o, int c0,
	int quad, int lane, const float (&bias)[FL<L>::N])
{
	using F = FL<L>;
	constexpr int N = F::N;
	const LayerRows lr = layer_rows(L, y_lo, y_hi);
	uint64_t* accfree = f_accfree(smem, L);
	const int i = quad * 32 + lane; // pixel of the strip
	const int x = c0 + i;
	const int y = lr.A + o;
	// layer 3: the source pixels of the bilinear residual, loaded before the wait (rows y - 1, y, y + 1
	// and columns x - 1, x, x + 1, clamped to the frame)
	const bool out_px = L == 3 && i >= 4 && i < 4 + F_VALID && x < int(a.lo_w) && y < int(a.lo_h);
	uint32_t p[3][3];
	if constexpr (L == 3)
	{
		if (out_px)
		{
#pragma unroll
			for (int r = 0; r < 3; ++r)
			{
				const uint32_t* row = a.lo + size_t(min(max(y - 1 + r, 0), int(a.lo_h) - 1)) * a.lo_pitch;
				p[r][0] = __ldg(row + max(x - 1, 0));
				p[r][1] = __ldg(row + x);
				p[r][2] = __ldg(row + min(x + 1, int(a.lo_w) - 1));
			}
		}
	}
	const int kc = o + 2; // the layer's input index that completes output o
	if (!f_wait_input_done(smem, L, kc)) return false;
	fence_after_sync();
	const uint32_t b = (FR - uint32_t(o) % FR) % FR;
	const uint32_t taddr = tmem + (uint32_t(quad * 32) << 16) + F::TCOL + b * N;
	float v[N];
#pragma unroll
	for (int c8 = 0; c8 < N / 8; ++c8)
	{
		float t8[8];
		tmem_ld8(taddr + c8 * 8, t8);
#pragma unroll
		for (int e = 0; e < 8; ++e) v[c8 * 8 + e] = t8[e];
	}
	tmem_ld_wait();
#pragma unroll
	for (int c8 = 0; c8 < N / 8; ++c8) tmem_zero8(taddr + c8 * 8);
	tmem_st_wait();
	fence_before_sync();
	__syncwarp();
	if (lane == 0) mbar_arrive(&accfree[b]);
	if constexpr (L < 3)
	{
		uint64_t* next_full = f_full(smem, L + 1);
		// next layer's input index o: wait until its slot's previous row was consumed
		if (o >= FNS && !f_wait_input_done(smem, L + 1, o - FNS)) return false;
		const bool inside = x >= 0 && x < int(a.lo_w) && y >= 0 && y < int(a.lo_h);
		unsigned char* dst = smem + ring_base(L + 1) + (o % FNS) * FL<L + 1>::SLOT + (1 + i) * 16;
#pragma unroll
		for (int c8 = 0; c8 < N / 8; ++c8)
		{
			uint32_t w4[4];
#pragma unroll
			for (int q = 0; q < 4; ++q)
				w4[q] = inside ? pack2(fmaxf(v[c8 * 8 + 2 * q] + bias[c8 * 8 + 2 * q], 0.0f),
									 fmaxf(v[c8 * 8 + 2 * q + 1] + bias[c8 * 8 + 2 * q + 1], 0.0f))
							   : 0u;
			*reinterpret_cast<uint4*>(dst + c8 * CXS_BYTES) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
		}
		fence_proxy_async();
		__syncwarp();
		if (lane == 0) mbar_arrive(&next_full[o % FNS]);
	}
	else
	{
		// output stage: columns c0 + 4 .. c0 + 123 of the strip, inside the frame
		if (out_px)
		{
#pragma unroll
			for (int sy = 0; sy < 2; ++sy)
			{
				const uint32_t p11 = p[1][1], p10 = p[1][0], p12 = p[1][2];
				const uint32_t p21 = p[sy ? 2 : 0][1], p20 = p[sy ? 2 : 0][0], p22 = p[sy ? 2 : 0][2];
				uint32_t px[2];
#pragma unroll
				for (int sx = 0; sx < 2; ++sx)
				{
					const int s = sy * 2 + sx;
					const uint32_t a01 = sx ? p12 : p10, a11 = sx ? p22 : p20;
					uint32_t bytes = p11 & 0xFF000000u;
#pragma unroll
					for (int ch = 0; ch < 3; ++ch)
					{
						const float top = 0.75f * float((p11 >> (8 * ch)) & 255u) + 0.25f * float((a01 >> (8 * ch)) & 255u);
						const float bot = 0.75f * float((p21 >> (8 * ch)) & 255u) + 0.25f * float((a11 >> (8 * ch)) & 255u);
						const float pred = (0.75f * top + 0.25f * bot) * (1.0f / 255.0f) + (v[ch * 4 + s] + bias[ch * 4 + s]);
						bytes |= to_byte(pred) << (8 * ch);
					}
					px[sx] = bytes;
				}
				*reinterpret_cast<uint2*>(a.hi + size_t(2 * y + sy) * a.hi_pitch + 2 * x) = make_uint2(px[0], px[1]);
			}
		}
	}
	return true;
}

__global__ void __launch_bounds__(F_THREADS, 1) fused_upscale_kernel(const __grid_constant__ FusedArgs a)
{
	extern __shared__ __align__(1024) unsigned char smem[];
	uint64_t* wbar = reinterpret_cast<uint64_t*>(smem + FusedSmem::BARS) + 4 * FNS + 4 * NBAR + 4 * FR;
	uint64_t* done = wbar + 1; // [2]: one per MMA issuer
	uint32_t* s_tmem = reinterpret_cast<uint32_t*>(smem + FusedSmem::MISC);

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int strip = int(blockIdx.x % a.strips), seg = int(blockIdx.x / a.strips);
	const int H = int(a.lo_h);
	const int y_lo = int((int64_t(seg) * H) / int(a.segments)), y_hi = int((int64_t(seg + 1) * H) / int(a.segments));
	const int c0 = strip * F_VALID - 4;

	// zero every ring slot (halo pixels are never written; layer 0's second chunk stays zero)
	for (uint32_t off = tid * 16; off < FusedSmem::W0; off += F_THREADS * 16)
		*reinterpret_cast<uint4*>(smem + off) = make_uint4(0u, 0u, 0u, 0u);
	if (tid == 0)
	{
		for (int l = 0; l < 4; ++l)
		{
			for (int k = 0; k < FNS; ++k) mbar_init(&f_full(smem, l)[k], l == 0 ? 32 : 4);
			for (int k = 0; k < NBAR; ++k) mbar_init(&f_rowbar(smem, l)[k], 1);
			for (int k = 0; k < FR; ++k) mbar_init(&f_accfree(smem, l)[k], 4);
		}
		mbar_init(wbar, 1);
		mbar_init(&done[0], 1);
		mbar_init(&done[1], 1);
		fence_mbar_init();
	}
	if (warp == 1)
	{
		tmem_alloc(s_tmem, F_TMEM_COLS);
		tmem_relinquish();
	}
	fence_proxy_async();
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	const uint32_t tmem = *s_tmem;
	if (warp >= 2 && warp <= 9)
	{
		// every accumulator starts at zero (the MMAs always accumulate)
		const uint32_t lb = uint32_t((warp & 3) * 32) << 16;
		const uint32_t c_lo = warp <= 5 ? 0u : 256u, c_hi = warp <= 5 ? 256u : 448u; // halves of the 448 used columns
		for (uint32_t c = c_lo; c < c_hi; c += 8) tmem_zero8(tmem + lb + c);
		tmem_st_wait();
	}
	fence_before_sync();
	__syncthreads();
	fence_after_sync();

	const LayerRows lr0 = layer_rows(0, y_lo, y_hi);
	const int steps = lr0.inputs() + 3 * FLAG;
	bool failed = false;

	if (warp == 0)
	{
		// layer 0 input rows from the Color32 source. Lane t holds pixels t + 32 k (k < F0_PX) of a row;
		// the loads of a row are issued F0_AHEAD rows before it is stored, so their latency overlaps the
		// waits for ring slots instead of adding to every row.
		uint64_t* full0 = f_full(smem, 0);

		const int n0 = lr0.inputs();
		uint32_t pre[F0_AHEAD + 1][F0_PX];
#pragma unroll
		for (int r = 0; r < F0_AHEAD; ++r) f0_load_row(a, lr0.A - 1 + r, r < n0, c0, lane, pre[r]);
		for (int q = 0; q < n0 && !failed; ++q)
		{
			f0_load_row(a, lr0.A - 1 + q + F0_AHEAD, q + F0_AHEAD < n0, c0, lane, pre[F0_AHEAD]);
			if (q >= FNS && !f_wait_input_done(smem, 0, q - FNS))
			{
				failed = true;
				break;
			}
			unsigned char* dst = smem + FusedSmem::RING0 + (q % FNS) * FL<0>::SLOT;
#pragma unroll
			for (int k = 0; k < F0_PX; ++k)
			{
				const int j = lane + 32 * k;
				if (j < CXS)
				{
					const uint32_t px = pre[0][k];
					uint4 w4;
					w4.x = pack2(float(px & 255u) * (1.0f / 255.0f), float((px >> 8) & 255u) * (1.0f / 255.0f));
					w4.y = pack2(float((px >> 16) & 255u) * (1.0f / 255.0f), 0.0f);
					w4.z = 0u;
					w4.w = 0u;
					*reinterpret_cast<uint4*>(dst + j * 16) = w4;
				}
			}
			fence_proxy_async();
			mbar_arrive(&full0[q % FNS]);
#pragma unroll
			for (int r = 0; r < F0_AHEAD; ++r)
#pragma unroll
				for (int k = 0; k < F0_PX; ++k) pre[r][k] = pre[r + 1][k];
		}
	}
	else if (warp == 1 || warp == 10)
	{
		if (lane == 0)
		{
			if (warp == 1)
			{
				mbar_expect_tx(wbar, FL<0>::WBYTES + FL<1>::WBYTES + FL<2>::WBYTES + FL<3>::WBYTES);
				bulk_g2s(smem + FusedSmem::W0, a.w[0], FL<0>::WBYTES, wbar);
				bulk_g2s(smem + FusedSmem::W1, a.w[1], FL<1>::WBYTES, wbar);
				bulk_g2s(smem + FusedSmem::W2, a.w[2], FL<2>::WBYTES, wbar);
				bulk_g2s(smem + FusedSmem::W3, a.w[3], FL<3>::WBYTES, wbar);
			}
			failed = !mbar_wait_bounded(wbar, 0, POLL_LIMIT);
			const int la = warp == 1 ? 0 : 1; // this issuer's layers: la and la + 2
			const int n_a = layer_rows(la, y_lo, y_hi).inputs(), n_b = layer_rows(la + 2, y_lo, y_hi).inputs();
			for (int s = 0; s < steps && !failed; ++s)
			{
				const int i0 = s - FLAG * la, i1 = s - FLAG * (la + 2);
				if (i0 >= 0 && i0 < n_a)
					failed = !(la == 0 ? fused_mma<0>(smem, tmem, y_lo, y_hi, i0) : fused_mma<1>(smem, tmem, y_lo, y_hi, i0));
				if (!failed && i1 >= 0 && i1 < n_b)
					failed = !(la == 0 ? fused_mma<2>(smem, tmem, y_lo, y_hi, i1) : fused_mma<3>(smem, tmem, y_lo, y_hi, i1));
				if (!failed) mma_commit(&f_rowbar(smem, la)[s % NBAR]); // the step's rows are consumed
			}
			uint64_t* d = &done[warp == 1 ? 0 : 1];
			mma_commit(d);
			if (!mbar_wait_bounded(d, 0, POLL_LIMIT)) failed = true;
		}
	}
	else
	{
		const int quad = warp & 3;
		const bool group_a = warp <= 5; // layers 0 and 2; otherwise 1 and 3
		const int la = group_a ? 0 : 1, lb = la + 2;
		float bias_a[32], bias_b2[32], bias_b3[16];
#pragma unroll
		for (int c = 0; c < 32; ++c)
		{
			bias_a[c] = a.bias[la][c];
			bias_b2[c] = a.bias[2][c];
		}
#pragma unroll
		for (int c = 0; c < 16; ++c) bias_b3[c] = a.bias[3][c];
		const int n_a = layer_rows(la, y_lo, y_hi).outputs(), n_b = layer_rows(lb, y_lo, y_hi).outputs();
		for (int s = 0; s < steps && !failed; ++s)
		{
			// layer l's output o completes at its input o + 2, i.e. in step o + 2 + FLAG * l
			const int oa = s - 2 - FLAG * la, ob = s - 2 - FLAG * lb;
			if (oa >= 0 && oa < n_a)
			{
				const bool ok = group_a ? fused_epilogue<0>(a, smem, tmem, y_lo, y_hi, oa, c0, quad, lane, bias_a)
										: fused_epilogue<1>(a, smem, tmem, y_lo, y_hi, oa, c0, quad, lane, bias_a);
				if (!ok) failed = true;
			}
			if (!failed && ob >= 0 && ob < n_b)
			{
				const bool ok = group_a ? fused_epilogue<2>(a, smem, tmem, y_lo, y_hi, ob, c0, quad, lane, bias_b2)
										: fused_epilogue<3>(a, smem, tmem, y_lo, y_hi, ob, c0, quad, lane, bias_b3);
				if (!ok) failed = true;
			}
		}
	}
	if (failed) atomicExch(a.error, 1);
	fence_before_sync();
	__syncthreads();
	if (warp == 1)
	{
		fence_after_sync();
		tmem_dealloc(tmem, F_TMEM_COLS);
	}
}

// ---- weight gradient ----

struct WgradArgs
{
	Planes x; // layer input (C8X chunks)
	Planes g; // pre-activation gradient (NG / 8 chunks)
	float* partial;    // per CTA: [3 dx][128 rows][NG] then the bias partials [NG]
	uint32_t tiles_x, row_blocks;
	int* error;
};

template <int C8X, int NG>
__host__ __device__ constexpr uint32_t wgrad_partial_floats()
{
	return 3 * 128 * NG + NG;
}

template <int C8X, int NG>
__global__ void __launch_bounds__(128) wgrad_kernel(WgradArgs a)
{
	constexpr int DY = 16 / C8X;         // dy groups stacked in M (only the first 3 are taps)
	constexpr int XROWS = ROWS + DY - 1; // staged input rows
	constexpr int G8 = NG / 8;
	constexpr uint32_t X_BYTES = XROWS * C8X * XS_BYTES;
	constexpr uint32_t G_BYTES = ROWS * G8 * XS_BYTES;
	constexpr uint32_t TMEM_COLS = 3 * NG <= 64 ? 64 : 128;
	extern __shared__ __align__(1024) unsigned char smem[];
	unsigned char* s_x = smem;
	unsigned char* s_g = smem + X_BYTES;
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + X_BYTES + G_BYTES);
	uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + 2);
	float* s_bias = reinterpret_cast<float*>(bars + 4); // [128]

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	uint32_t bid = blockIdx.x;
	const uint32_t tx = bid % a.tiles_x;
	bid /= a.tiles_x;
	const uint32_t rb = bid % a.row_blocks;
	const uint32_t img = bid / a.row_blocks;
	const int x0 = int(tx) * TILE_X, y0 = int(rb) * ROWS;

	if (tid == 0)
	{
		mbar_init(&bars[0], 1);
		mbar_init(&bars[1], 1);
		fence_mbar_init();
	}
	if (warp == 0)
	{
		tmem_alloc(s_tmem, TMEM_COLS);
		tmem_relinquish();
	}
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	const uint32_t tmem = *s_tmem;

	if (tid == 0)
	{
		mbar_expect_tx(&bars[0], X_BYTES + G_BYTES);
		for (int r = 0; r < XROWS; ++r)
			for (int c = 0; c < C8X; ++c)
				bulk_g2s(s_x + (r * C8X + c) * XS_BYTES, a.x.data + planes_index(a.x, img, y0 - 1 + r, c, x0 - 1), XS_BYTES, &bars[0]);
		for (int r = 0; r < ROWS; ++r)
			for (int c = 0; c < G8; ++c)
				bulk_g2s(s_g + (r * G8 + c) * XS_BYTES, a.g.data + planes_index(a.g, img, y0 + r, c, x0 - 1), XS_BYTES, &bars[0]);
	}
	const bool loaded = mbar_wait_bounded(&bars[0], 0, POLL_LIMIT);
	if (__syncthreads_or(!loaded))
	{
		if (tid == 0) atomicExch(a.error, 3);
		mbar_wait_bounded(&bars[0], 0, POLL_LIMIT);
		__syncthreads();
		if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
		return;
	}
	if (tid == 0)
	{
		fence_after_sync();
		const uint32_t idesc = make_idesc_bf16(128, NG, 1, 1);
		const uint32_t xb = smem_addr(s_x), gb = smem_addr(s_g);
		bool first[3] = {true, true, true};
		for (int rr = 0; rr < ROWS; ++rr)
			for (int kc = 0; kc < TILE_X / 16; ++kc)
				for (int d = 0; d < 3; ++d)
				{
					// A = X^T: rows (dy, chunk, ci % 8), 8-row groups XS_BYTES apart; K = 16 pixels, LBO = 8 pixels.
					const uint32_t aaddr = xb + (rr * C8X) * XS_BYTES + (1 + (d - 1) + 16 * kc) * 16;
					// B = G^T: columns co, 8-column groups XS_BYTES apart; the same 16 pixels.
					const uint32_t baddr = gb + (rr * G8) * XS_BYTES + (1 + 16 * kc) * 16;
					mma_bf16(tmem + d * NG, make_sdesc(aaddr, 128, XS_BYTES), make_sdesc(baddr, 128, XS_BYTES), idesc,
						first[d] ? 0u : 1u);
					first[d] = false;
				}
		mma_commit(&bars[1]);
	}
	// Bias gradient partials from the staged gradient rows (pixels 0..127 of the tile).
	{
		constexpr int PARTS = 128 / NG;
		const int co = tid % NG, part = tid / NG;
		const int c8 = co / 8, e = co % 8;
		float s = 0.0f;
		for (int r = 0; r < ROWS; ++r)
			for (int p = part; p < TILE_X; p += PARTS)
				s += bf2f(*reinterpret_cast<const uint16_t*>(s_g + (r * G8 + c8) * XS_BYTES + (1 + p) * 16 + e * 2));
		s_bias[tid] = s;
	}
	const bool done = mbar_wait_bounded(&bars[1], 0, POLL_LIMIT);
	if (__syncthreads_or(!done))
	{
		if (tid == 0) atomicExch(a.error, 4);
		mbar_wait_bounded(&bars[1], 0, POLL_LIMIT);
		fence_before_sync();
		__syncthreads();
		fence_after_sync();
		if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
		return;
	}
	fence_after_sync();
	float* out = a.partial + size_t(blockIdx.x) * wgrad_partial_floats<C8X, NG>();
	const int m = warp * 32 + lane;
	const uint32_t lane_base = uint32_t(warp * 32) << 16;
	for (int d = 0; d < 3; ++d)
	{
#pragma unroll
		for (int c8 = 0; c8 < G8; ++c8)
		{
			float t8[8];
			tmem_ld8(tmem + lane_base + d * NG + c8 * 8, t8);
			tmem_ld_wait();
			float4* o = reinterpret_cast<float4*>(out + (size_t(d) * 128 + m) * NG + c8 * 8);
			o[0] = make_float4(t8[0], t8[1], t8[2], t8[3]);
			o[1] = make_float4(t8[4], t8[5], t8[6], t8[7]);
		}
	}
	if (tid < NG)
	{
		constexpr int PARTS = 128 / NG;
		float s = 0.0f;
		for (int q = 0; q < PARTS; ++q) s += s_bias[q * NG + tid];
		out[3 * 128 * NG + tid] = s;
	}
	fence_before_sync();
	__syncthreads();
	if (warp == 0)
	{
		fence_after_sync();
		tmem_dealloc(tmem, TMEM_COLS);
	}
}

template <int C8X, int NG>
__host__ __device__ constexpr uint32_t wgrad_smem_bytes()
{
	return (ROWS + 16 / C8X - 1) * C8X * XS_BYTES + ROWS * (NG / 8) * XS_BYTES + 32 + 512;
}

// Sum the per-CTA partials (fixed order) into canonical gradients of one layer, times `scale`.
__global__ void wgrad_reduce_kernel(const float* partial, uint32_t num_ctas, uint32_t partial_floats, int layer, int c8x, int ng,
	float scale, float* grads)
{
	const LayerShape L = c_layers[layer];
	const int nw = L.cout * 9 * L.cin;
	const int idx = blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= nw + L.cout) return;
	size_t off;
	if (idx < nw)
	{
		int r = idx;
		const int ci = r % L.cin;
		r /= L.cin;
		const int kx = r % 3;
		r /= 3;
		const int ky = r % 3;
		const int co = r / 3;
		const int m = (ky * c8x + ci / 8) * 8 + ci % 8;
		off = (size_t(kx) * 128 + m) * ng + co;
	}
	else
		off = size_t(3) * 128 * ng + (idx - nw);
	float s = 0.0f;
	for (uint32_t c = 0; c < num_ctas; ++c) s += partial[size_t(c) * partial_floats + off];
	grads[L.param_offset + idx] = s * scale;
}

// Input conversion: Color32 window of each crop -> chunk 0 of the row planes (b, g, r, 0...) / 255.
__global__ void convert_input_kernel(const CropGpu* crops, Planes p)
{
	const uint32_t img = blockIdx.y;
	const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= p.width * p.height) return;
	const int x = int(idx % p.width), y = int(idx / p.width);
	const CropGpu c = crops[img];
	const uint32_t px = c.lo[size_t(c.y + y) * c.lo_pitch + (c.x + x)];
	uint4 o;
	o.x = pack2(float(px & 255u) * (1.0f / 255.0f), float((px >> 8) & 255u) * (1.0f / 255.0f));
	o.y = pack2(float((px >> 16) & 255u) * (1.0f / 255.0f), 0.0f);
	o.z = 0u;
	o.w = 0u;
	*reinterpret_cast<uint4*>(p.data + planes_index(p, img, y, 0, x)) = o;
}

// Adam on the canonical parameters, then repack every weight into the forward and transposed
// (input-gradient) B-operand layouts as bf16 and every bias as f32.
struct AdamArgs
{
	float* params;
	float* m;
	float* v;
	const float* grads;
	float lr, beta1, beta2, eps, bc1, bc2; // bc = 1 - beta^t
	int update;
	uint16_t* wfwd[NUM_LAYERS];
	uint16_t* wbwd[NUM_LAYERS];
	float* bias[NUM_LAYERS];
};

__global__ void adam_pack_kernel(AdamArgs a)
{
	const int idx = blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= int(SW_UPSCALER_NUM_PARAMS)) return;
	float p = a.params[idx];
	if (a.update)
	{
		const float g = a.grads[idx];
		const float m = a.beta1 * a.m[idx] + (1.0f - a.beta1) * g;
		const float v = a.beta2 * a.v[idx] + (1.0f - a.beta2) * g * g;
		a.m[idx] = m;
		a.v[idx] = v;
		p -= a.lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
		a.params[idx] = p;
	}
	int l = NUM_LAYERS - 1;
	while (l > 0 && idx < c_layers[l].param_offset) --l;
	const LayerShape L = c_layers[l];
	const int local = idx - L.param_offset;
	const int nw = L.cout * 9 * L.cin;
	if (local >= nw)
	{
		a.bias[l][local - nw] = p;
		return;
	}
	int r = local;
	const int ci = r % L.cin;
	r /= L.cin;
	const int t = r % 9;
	const int co = r / 9;
	const uint16_t h = f2bf(p);
	const int ky = t / 3, kx = t % 3;
	{
		// B operand of conv_kernel: per (kx, 16-channel step ks, half hh): rows (ky, co) x 8 input channels
		const int ks = ci / 16, hh = (ci / 8) % 2, e = ci % 8;
		const int nb = 3 * L.n_out;
		a.wfwd[l][((kx * (L.c8_in / 2) + ks) * 2 + hh) * nb * 8 + (ky * L.n_out + co) * 8 + e] = h;
	}
	if (a.wbwd[l])
	{
		// input gradient = conv over the gradient (n_out / 8 chunks) producing c8_in * 8 channels with
		// the taps flipped: (ky, kx) -> (2 - ky, 2 - kx), input and output channels swapped
		const int no = L.c8_in * 8;
		const int ks = co / 16, hh = (co / 8) % 2, e = co % 8;
		a.wbwd[l][(((2 - kx) * (L.n_out / 16) + ks) * 2 + hh) * (3 * no) * 8 + ((2 - ky) * no + ci) * 8 + e] = h;
	}
}

__global__ void psnr_kernel(const uint32_t* a, uint32_t ap, const uint32_t* b, uint32_t bp, uint32_t w, uint32_t h,
	unsigned long long* sum)
{
	unsigned long long s = 0;
	for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < w * h; idx += gridDim.x * blockDim.x)
	{
		const uint32_t x = idx % w, y = idx / w;
		const uint32_t pa = a[size_t(y) * ap + x], pb = b[size_t(y) * bp + x];
		for (int ch = 0; ch < 3; ++ch)
		{
			const int d = int((pa >> (8 * ch)) & 255u) - int((pb >> (8 * ch)) & 255u);
			s += unsigned(d * d);
		}
	}
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
	if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

// ---- host side ----

struct DevMem
{
	void* ptr = nullptr;
	size_t bytes = 0;
};

uint64_t fnv1a(const void* data, size_t n, uint64_t h = 1469598103934665603ull)
{
	const unsigned char* p = static_cast<const unsigned char*>(data);
	for (size_t i = 0; i < n; ++i)
	{
		h ^= p[i];
		h *= 1099511628211ull;
	}
	return h;
}

uint64_t splitmix(uint64_t& s)
{
	uint64_t z = (s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

} // namespace

struct SwUpscaler
{
	int device = 0;
	cudaStream_t stream = nullptr;
	std::string last_error;
	uint64_t steps = 0;
	int num_sms = 1;
	uint32_t loss_ctas = 0; // CTAs of the last loss-epilogue launch
	// canonical parameters and Adam state (device, f32)
	DevMem params, adam_m, adam_v, grads;
	DevMem wfwd[NUM_LAYERS], wbwd[NUM_LAYERS], bias[NUM_LAYERS];
	DevMem error;
	// training workspace (SW_UPSCALER_MAX_CROPS crops)
	DevMem t_x0, t_a[3], t_g4, t_g[3], partial, loss_partial, crops;
	uint32_t crops_capacity = 0;
	DevMem h_stage; // pinned: crops + loss partials
	// inference workspace
	DevMem i_x0, i_p, i_q, i_crop;
	uint32_t i_w = 0, i_h = 0;
	CropGpu i_crop_host{};
	bool i_crop_valid = false;
	bool fused = true; // inference by fused_upscale_kernel (else the four layer launches)
	DevMem psnr_sum;
	unsigned long long* h_psnr = nullptr;
	cudaEvent_t ev = nullptr;
};

namespace
{

int fail(SwUpscaler* u, int code, const char* fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	if (u) u->last_error = buf;
	return code;
}

#define UP_CUDA(u, call)                                                                      \
	do                                                                                        \
	{                                                                                         \
		cudaError_t e_ = (call);                                                              \
		if (e_ != cudaSuccess) return fail(u, SW_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
	} while (0)

int dev_alloc(SwUpscaler* u, DevMem& m, size_t bytes, bool zero = true)
{
	if (m.ptr && m.bytes >= bytes) return SW_OK;
	if (m.ptr) cudaFree(m.ptr);
	m.ptr = nullptr;
	m.bytes = 0;
	cudaError_t e = cudaMalloc(&m.ptr, bytes);
	if (e != cudaSuccess)
	{
		cudaGetLastError();
		return fail(u, SW_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu) failed", bytes);
	}
	m.bytes = bytes;
	if (zero)
	{
		// Zeroed on the upscaler's stream and waited for here: a plain cudaMemset runs on the legacy
		// default stream, which the non-blocking streams the buffers are used on do not wait for.
		UP_CUDA(u, cudaMemsetAsync(m.ptr, 0, bytes, u->stream));
		UP_CUDA(u, cudaStreamSynchronize(u->stream));
	}
	return SW_OK;
}

void dev_free(DevMem& m)
{
	if (m.ptr) cudaFree(m.ptr);
	m.ptr = nullptr;
	m.bytes = 0;
}

Planes make_planes(void* data, uint32_t images, uint32_t width, uint32_t height, uint32_t chunks)
{
	Planes p;
	p.data = static_cast<uint16_t*>(data);
	p.images = images;
	p.width = width;
	p.height = height;
	p.chunks = chunks;
	p.wp = ((width + TILE_X - 1) / TILE_X) * TILE_X + 8;
	p.rows_alloc = ((height + ROWS - 1) / ROWS) * ROWS + 10;
	return p;
}

size_t planes_bytes(uint32_t images, uint32_t width, uint32_t height, uint32_t chunks)
{
	const Planes p = make_planes(nullptr, images, width, height, chunks);
	return size_t(images) * p.rows_alloc * chunks * p.wp * 16;
}

// Tensor map of the rows of a row-plane tensor as a 4-D bf16 array [images * rows_alloc][chunks][wp / 8][64]
// (innermost last; 64 elements = 8 pixels x 8 channels = 128 bytes): a box of 64 x 17 x chunks x 1 at
// group x0 / 8 is one input row of the 128-pixel tile starting at x0 with its halo (pixels x0 - 1 ..
// x0 + 134), landing in shared memory as [chunk][136 pixels][8 channels].
int make_row_map(SwUpscaler* u, const Planes& p, CUtensorMap* out)
{
	static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
	if (!encode)
	{
		cudaDriverEntryPointQueryResult q;
		void* fn = nullptr;
		UP_CUDA(u, cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
		if (q != cudaDriverEntryPointSuccess || !fn) return fail(u, SW_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
		encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
	}
	if (p.wp % 8) return fail(u, SW_ERR_KERNEL, "row planes: padded width %u not a multiple of 8", p.wp);
	const cuuint64_t dims[4] = {64, p.wp / 8, p.chunks, cuuint64_t(p.images) * p.rows_alloc};
	const cuuint64_t strides[3] = {128, cuuint64_t(p.wp) * 16, cuuint64_t(p.chunks) * p.wp * 16}; // bytes, dims 1..3
	const cuuint32_t box[4] = {64, CXS / 8, p.chunks, 1};
	const cuuint32_t estr[4] = {1, 1, 1, 1};
	const CUresult r = encode(out, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, p.data, dims, strides, box, estr,
		CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
		CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS) return fail(u, SW_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
	return SW_OK;
}

// Persistent grid: as many CTAs as fit on one SM at once (shared memory, and TMEM: 512 columns per SM)
// on every SM, at least 2 output rows each.
template <int C8, int N, int EPI>
int launch_conv(SwUpscaler* u, ConvArgs a, cudaStream_t s)
{
	a.error = static_cast<int*>(u->error.ptr);
	if (a.in.chunks != uint32_t(C8)) return fail(u, SW_ERR_KERNEL, "convolution input has %u chunks, kernel %d", a.in.chunks, C8);
	int r = make_row_map(u, a.in, &a.in_map);
	if (r) return r;
	constexpr uint32_t smem = conv_smem_bytes<C8, N>();
	constexpr int tmem_cols = int(conv_tmem_cols<N>());
	static int per_sm[64] = {};
	const int key = (C8 / 2) * 16 + (N / 16) * 4 + EPI;
	if (!per_sm[key])
	{
		UP_CUDA(u, cudaFuncSetAttribute(conv_kernel<C8, N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
		UP_CUDA(u, cudaFuncSetAttribute(conv_kernel<C8, N, EPI>, cudaFuncAttributePreferredSharedMemoryCarveout,
							 int(cudaSharedmemCarveoutMaxShared)));
		int smem_sm = 0;
		UP_CUDA(u, cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, u->device));
		const int by_smem = smem_sm / int(smem + 1024); // 1 KB reserved per CTA
		per_sm[key] = std::max(1, std::min(by_smem, 512 / tmem_cols));
	}
	const uint32_t rows = a.in.images * ((a.in.width + TILE_X - 1) / TILE_X) * a.in.height;
	const uint32_t blocks = std::max(1u, std::min(uint32_t(u->num_sms * per_sm[key]), (rows + 1) / 2));
	if (EPI == EPI_LOSS)
	{
		if (blocks * 4 > u->loss_partial.bytes) return fail(u, SW_ERR_LIMIT, "loss partial buffer too small");
		u->loss_ctas = blocks;
	}
	conv_kernel<C8, N, EPI><<<blocks, CONV_THREADS, smem, s>>>(a);
	UP_CUDA(u, cudaGetLastError());
	return SW_OK;
}

template <int C8X, int NG>
int launch_wgrad(SwUpscaler* u, const Planes& x, const Planes& g, int layer, float scale, cudaStream_t s)
{
	WgradArgs a;
	a.x = x;
	a.g = g;
	a.partial = static_cast<float*>(u->partial.ptr);
	a.tiles_x = (x.width + TILE_X - 1) / TILE_X;
	a.row_blocks = (x.height + ROWS - 1) / ROWS;
	a.error = static_cast<int*>(u->error.ptr);
	constexpr uint32_t smem = wgrad_smem_bytes<C8X, NG>();
	static bool configured[8] = {};
	const int key = (C8X / 2 - 1) * 2 + (NG / 16 - 1);
	if (!configured[key])
	{
		UP_CUDA(u, cudaFuncSetAttribute(wgrad_kernel<C8X, NG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
		configured[key] = true;
	}
	const uint32_t blocks = x.images * a.tiles_x * a.row_blocks;
	if (size_t(blocks) * wgrad_partial_floats<C8X, NG>() * 4 > u->partial.bytes)
		return fail(u, SW_ERR_LIMIT, "weight-gradient partial buffer too small");
	wgrad_kernel<C8X, NG><<<blocks, 128, smem, s>>>(a);
	UP_CUDA(u, cudaGetLastError());
	const LayerShape& L = LAYERS[layer];
	const int n = L.cout * 9 * L.cin + L.cout;
	wgrad_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(static_cast<const float*>(u->partial.ptr), blocks,
		wgrad_partial_floats<C8X, NG>(), layer, C8X, NG, scale, static_cast<float*>(u->grads.ptr));
	UP_CUDA(u, cudaGetLastError());
	return SW_OK;
}

int pack_weights(SwUpscaler* u, int update, float lr, cudaStream_t s)
{
	AdamArgs a;
	a.params = static_cast<float*>(u->params.ptr);
	a.m = static_cast<float*>(u->adam_m.ptr);
	a.v = static_cast<float*>(u->adam_v.ptr);
	a.grads = static_cast<const float*>(u->grads.ptr);
	a.lr = lr;
	a.beta1 = 0.9f;
	a.beta2 = 0.999f;
	a.eps = 1e-8f;
	const double t = double(u->steps + (update ? 1 : 0));
	a.bc1 = float(1.0 - std::pow(0.9, t));
	a.bc2 = float(1.0 - std::pow(0.999, t));
	a.update = update;
	for (int l = 0; l < NUM_LAYERS; ++l)
	{
		a.wfwd[l] = static_cast<uint16_t*>(u->wfwd[l].ptr);
		a.wbwd[l] = l > 0 ? static_cast<uint16_t*>(u->wbwd[l].ptr) : nullptr;
		a.bias[l] = static_cast<float*>(u->bias[l].ptr);
	}
	adam_pack_kernel<<<(SW_UPSCALER_NUM_PARAMS + 255) / 256, 256, 0, s>>>(a);
	UP_CUDA(u, cudaGetLastError());
	if (update) ++u->steps;
	return SW_OK;
}

// The failure path every upscaler kernel takes when a bounded mbarrier wait runs out, on a barrier
// that nothing completes: one CTA allocates TMEM as the kernels do, arms an mbarrier with one arrival
// and 16 transaction bytes that no copy will ever deliver (no copy or MMA is issued, so nothing is in
// flight), waits at most max_polls polls, then records code 5 in the error flag, frees the TMEM and
// returns - the recovery the real kernels run.
__global__ void __launch_bounds__(128) wait_probe_kernel(int* error, uint32_t max_polls)
{
	__shared__ __align__(8) uint64_t bar;
	__shared__ uint32_t s_tmem;
	if (threadIdx.x == 0)
	{
		mbar_init(&bar, 1);
		fence_mbar_init();
	}
	if (threadIdx.x < 32)
	{
		tmem_alloc(&s_tmem, 32);
		tmem_relinquish();
	}
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	const uint32_t tmem = s_tmem;
	if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);
	__syncthreads();
	const bool completed = mbar_wait_bounded(&bar, 0, max_polls);
	if (__syncthreads_or(!completed) && threadIdx.x == 0) atomicExch(error, 5);
	fence_before_sync();
	__syncthreads();
	fence_after_sync();
	if (threadIdx.x < 32) tmem_dealloc(tmem, 32);
}

int check_error_flag(SwUpscaler* u, cudaStream_t s)
{
	int h = 0;
	UP_CUDA(u, cudaMemcpyAsync(&h, u->error.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
	UP_CUDA(u, cudaStreamSynchronize(s));
	if (h) return fail(u, SW_ERR_KERNEL, "upscaler kernel gave up waiting (code %d)", h);
	return SW_OK;
}

int prepare_training(SwUpscaler* u, uint32_t n)
{
	if (n > u->crops_capacity)
	{
		const uint32_t W = SW_UPSCALER_CROP_W, H = SW_UPSCALER_CROP_H;
		const uint32_t cap = SW_UPSCALER_MAX_CROPS;
		int r;
		if ((r = dev_alloc(u, u->t_x0, planes_bytes(cap, W, H, 2)))) return r;
		for (int i = 0; i < 3; ++i)
		{
			if ((r = dev_alloc(u, u->t_a[i], planes_bytes(cap, W, H, 4)))) return r;
			if ((r = dev_alloc(u, u->t_g[i], planes_bytes(cap, W, H, 4)))) return r;
		}
		if ((r = dev_alloc(u, u->t_g4, planes_bytes(cap, W, H, 2)))) return r;
		const size_t ctas = size_t(cap) * (H / ROWS) * ((W + TILE_X - 1) / TILE_X);
		if ((r = dev_alloc(u, u->partial, ctas * wgrad_partial_floats<4, 32>() * 4, false))) return r;
		if ((r = dev_alloc(u, u->loss_partial, std::max<size_t>(ctas, 4096) * 4, false))) return r;
		if ((r = dev_alloc(u, u->crops, cap * sizeof(CropGpu), false))) return r;
		if (!u->h_stage.ptr)
		{
			const size_t hb = cap * sizeof(CropGpu) + std::max<size_t>(ctas, 4096) * 4;
			UP_CUDA(u, cudaMallocHost(&u->h_stage.ptr, hb));
			u->h_stage.bytes = hb;
		}
		u->crops_capacity = cap;
	}
	return SW_OK;
}

// Forward + backward of the crops; gradients (canonical, scaled by 1/n) end in u->grads.
int forward_backward(SwUpscaler* u, const SwUpscalerCrop* crops, uint32_t n, uint32_t* loss_count)
{
	if (!crops || n == 0 || n > SW_UPSCALER_MAX_CROPS) return fail(u, SW_ERR_INVALID_ARGUMENT, "bad crop list");
	const uint32_t W = SW_UPSCALER_CROP_W, H = SW_UPSCALER_CROP_H, M = SW_UPSCALER_CROP_MARGIN;
	for (uint32_t i = 0; i < n; ++i)
	{
		const SwUpscalerCrop& c = crops[i];
		if (!c.lo || !c.hi || c.lo_pitch < c.lo_width || c.hi_pitch < 2 * c.lo_width || (c.hi_pitch & 1) ||
			(reinterpret_cast<uintptr_t>(c.hi) & 7) || c.x < 0 || c.y < 0 ||
			uint64_t(c.x) + W > c.lo_width || uint64_t(c.y) + H > c.lo_height)
			return fail(u, SW_ERR_INVALID_ARGUMENT, "crop %u outside its frame", i);
	}
	int r = prepare_training(u, n);
	if (r) return r;
	cudaStream_t s = u->stream;
	// Crop table through pinned staging (wait for the previous step's use of it first).
	UP_CUDA(u, cudaEventSynchronize(u->ev));
	CropGpu* hc = static_cast<CropGpu*>(u->h_stage.ptr);
	for (uint32_t i = 0; i < n; ++i)
	{
		const SwUpscalerCrop& c = crops[i];
		hc[i] = CropGpu{c.lo, c.hi, c.lo_width, c.lo_height, c.lo_pitch, c.hi_pitch, c.x, c.y};
	}
	UP_CUDA(u, cudaMemcpyAsync(u->crops.ptr, hc, n * sizeof(CropGpu), cudaMemcpyHostToDevice, s));
	UP_CUDA(u, cudaEventRecord(u->ev, s));

	const Planes x0 = make_planes(u->t_x0.ptr, n, W, H, 2);
	Planes A[3], G[3];
	for (int i = 0; i < 3; ++i)
	{
		A[i] = make_planes(u->t_a[i].ptr, n, W, H, 4);
		G[i] = make_planes(u->t_g[i].ptr, n, W, H, 4);
	}
	const Planes g4 = make_planes(u->t_g4.ptr, n, W, H, 2);
	const CropGpu* dcrops = static_cast<const CropGpu*>(u->crops.ptr);

	convert_input_kernel<<<dim3((W * H + 255) / 256, n), 256, 0, s>>>(dcrops, x0);
	UP_CUDA(u, cudaGetLastError());
	ConvArgs a{};
	a.crops = dcrops;
	a.margin = M;
	// forward
	a.in = x0, a.out = A[0], a.wpack = static_cast<uint16_t*>(u->wfwd[0].ptr), a.bias = static_cast<float*>(u->bias[0].ptr);
	if ((r = launch_conv<2, 32, EPI_RELU>(u, a, s))) return r;
	a.in = A[0], a.out = A[1], a.wpack = static_cast<uint16_t*>(u->wfwd[1].ptr), a.bias = static_cast<float*>(u->bias[1].ptr);
	if ((r = launch_conv<4, 32, EPI_RELU>(u, a, s))) return r;
	a.in = A[1], a.out = A[2], a.wpack = static_cast<uint16_t*>(u->wfwd[2].ptr), a.bias = static_cast<float*>(u->bias[2].ptr);
	if ((r = launch_conv<4, 32, EPI_RELU>(u, a, s))) return r;
	a.in = A[2], a.out = g4, a.wpack = static_cast<uint16_t*>(u->wfwd[3].ptr), a.bias = static_cast<float*>(u->bias[3].ptr);
	a.loss_partial = static_cast<float*>(u->loss_partial.ptr);
	if ((r = launch_conv<4, 16, EPI_LOSS>(u, a, s))) return r;

	const uint32_t count = n * (W - 2 * M) * (H - 2 * M) * 4 * 3;
	*loss_count = count;
	const float scale = 1.0f / float(count);
	// layer 3 (32 -> 12): weight gradient, input gradient into G[2] masked by A[2]
	if ((r = launch_wgrad<4, 16>(u, A[2], g4, 3, scale, s))) return r;
	ConvArgs b{};
	b.in = g4, b.out = G[2], b.mask = A[2], b.wpack = static_cast<uint16_t*>(u->wbwd[3].ptr);
	if ((r = launch_conv<2, 32, EPI_MASK>(u, b, s))) return r;
	// layer 2
	if ((r = launch_wgrad<4, 32>(u, A[1], G[2], 2, scale, s))) return r;
	b.in = G[2], b.out = G[1], b.mask = A[1], b.wpack = static_cast<uint16_t*>(u->wbwd[2].ptr);
	if ((r = launch_conv<4, 32, EPI_MASK>(u, b, s))) return r;
	// layer 1
	if ((r = launch_wgrad<4, 32>(u, A[0], G[1], 1, scale, s))) return r;
	b.in = G[1], b.out = G[0], b.mask = A[0], b.wpack = static_cast<uint16_t*>(u->wbwd[1].ptr);
	if ((r = launch_conv<4, 32, EPI_MASK>(u, b, s))) return r;
	// layer 0 (3 -> 32): weight gradient only
	if ((r = launch_wgrad<2, 32>(u, x0, G[0], 0, scale, s))) return r;
	return SW_OK;
}

int read_loss(SwUpscaler* u, uint32_t count, float* out_mse)
{
	const uint32_t ctas = u->loss_ctas;
	float* h = reinterpret_cast<float*>(static_cast<unsigned char*>(u->h_stage.ptr) + SW_UPSCALER_MAX_CROPS * sizeof(CropGpu));
	UP_CUDA(u, cudaMemcpyAsync(h, u->loss_partial.ptr, ctas * 4, cudaMemcpyDeviceToHost, u->stream));
	int r = check_error_flag(u, u->stream);
	if (r) return r;
	double s = 0.0;
	for (uint32_t i = 0; i < ctas; ++i) s += h[i];
	*out_mse = float(s / double(count));
	return SW_OK;
}

} // namespace

extern "C" {

int sw_upscaler_create(int device, uint64_t seed, SwUpscaler** out)
{
	if (!out) return SW_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
	{
		cudaGetLastError();
		return SW_ERR_NO_DEVICE;
	}
	SwUpscaler* u = new (std::nothrow) SwUpscaler();
	if (!u) return SW_ERR_OUT_OF_MEMORY;
	u->device = device;
	int r = SW_OK;
	auto bail = [&](int code) {
		sw_upscaler_destroy(u);
		return code;
	};
	if (cudaSetDevice(device) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaDeviceGetAttribute(&u->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SW_ERR_CUDA); // before any dev_alloc
	if (cudaEventCreateWithFlags(&u->ev, cudaEventDisableTiming) != cudaSuccess) return bail(SW_ERR_CUDA);
	if (cudaEventRecord(u->ev, u->stream) != cudaSuccess) return bail(SW_ERR_CUDA);
	const size_t pb = SW_UPSCALER_NUM_PARAMS * sizeof(float);
	if ((r = dev_alloc(u, u->params, pb)) || (r = dev_alloc(u, u->adam_m, pb)) || (r = dev_alloc(u, u->adam_v, pb)) ||
		(r = dev_alloc(u, u->grads, pb)) || (r = dev_alloc(u, u->error, 16)) || (r = dev_alloc(u, u->psnr_sum, 16)))
		return bail(r);
	for (int l = 0; l < NUM_LAYERS; ++l)
	{
		const LayerShape& L = LAYERS[l];
		if ((r = dev_alloc(u, u->wfwd[l], size_t(9) * L.c8_in * 8 * L.n_out * 2))) return bail(r);
		if (l > 0 && (r = dev_alloc(u, u->wbwd[l], size_t(9) * L.n_out * L.c8_in * 8 * 2))) return bail(r);
		if ((r = dev_alloc(u, u->bias[l], size_t(L.n_out) * 4))) return bail(r);
	}
	if (cudaMallocHost(reinterpret_cast<void**>(&u->h_psnr), sizeof(unsigned long long)) != cudaSuccess) return bail(SW_ERR_CUDA);
	// Seeded He-normal initialisation (Box-Muller over splitmix64), zero biases, last layer / 10.
	std::vector<float> p(SW_UPSCALER_NUM_PARAMS, 0.0f);
	uint64_t st = seed;
	for (int l = 0; l < NUM_LAYERS; ++l)
	{
		const LayerShape& L = LAYERS[l];
		const float sd = std::sqrt(2.0f / float(9 * L.cin)) * (l == NUM_LAYERS - 1 ? 0.1f : 1.0f);
		const int nw = L.cout * 9 * L.cin;
		for (int i = 0; i < nw; ++i)
		{
			const double u1 = (double(splitmix(st) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
			const double u2 = double(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
			p[L.param_offset + i] = float(std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2)) * sd;
		}
	}
	if ((r = sw_upscaler_set_params(u, p.data(), SW_UPSCALER_NUM_PARAMS))) return bail(r);
	*out = u;
	return SW_OK;
}

int sw_upscaler_destroy(SwUpscaler* u)
{
	if (!u) return SW_ERR_INVALID_ARGUMENT;
	cudaSetDevice(u->device);
	if (u->stream) cudaStreamSynchronize(u->stream);
	DevMem* all[] = {&u->params, &u->adam_m, &u->adam_v, &u->grads, &u->error, &u->t_x0, &u->t_g4, &u->partial,
		&u->loss_partial, &u->crops, &u->i_x0, &u->i_p, &u->i_q, &u->i_crop, &u->psnr_sum};
	for (DevMem* m : all) dev_free(*m);
	for (int i = 0; i < 3; ++i)
	{
		dev_free(u->t_a[i]);
		dev_free(u->t_g[i]);
	}
	for (int l = 0; l < NUM_LAYERS; ++l)
	{
		dev_free(u->wfwd[l]);
		dev_free(u->wbwd[l]);
		dev_free(u->bias[l]);
	}
	if (u->h_stage.ptr) cudaFreeHost(u->h_stage.ptr);
	if (u->h_psnr) cudaFreeHost(u->h_psnr);
	if (u->ev) cudaEventDestroy(u->ev);
	if (u->stream) cudaStreamDestroy(u->stream);
	delete u;
	return SW_OK;
}

const char* sw_upscaler_last_error(const SwUpscaler* u) { return u ? u->last_error.c_str() : "null upscaler"; }

int sw_upscaler_get_params(SwUpscaler* u, float* params, uint32_t count)
{
	if (!u || !params || count != SW_UPSCALER_NUM_PARAMS) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	UP_CUDA(u, cudaMemcpyAsync(params, u->params.ptr, count * 4, cudaMemcpyDeviceToHost, u->stream));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	return SW_OK;
}

int sw_upscaler_set_params(SwUpscaler* u, const float* params, uint32_t count)
{
	if (!u || !params || count != SW_UPSCALER_NUM_PARAMS) return SW_ERR_INVALID_ARGUMENT;
	for (uint32_t i = 0; i < count; ++i)
		if (!std::isfinite(params[i])) return fail(u, SW_ERR_INVALID_ARGUMENT, "parameter %u is not finite", i);
	UP_CUDA(u, cudaSetDevice(u->device));
	UP_CUDA(u, cudaMemcpyAsync(u->params.ptr, params, count * 4, cudaMemcpyHostToDevice, u->stream));
	UP_CUDA(u, cudaMemsetAsync(u->adam_m.ptr, 0, count * 4, u->stream));
	UP_CUDA(u, cudaMemsetAsync(u->adam_v.ptr, 0, count * 4, u->stream));
	u->steps = 0;
	int r = pack_weights(u, 0, 0.0f, u->stream);
	if (r) return r;
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	return SW_OK;
}

int sw_upscaler_gradients(SwUpscaler* u, const SwUpscalerCrop* crops, uint32_t num_crops, float* grads, float* loss)
{
	if (!u || !grads) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	uint32_t count = 0;
	int r = forward_backward(u, crops, num_crops, &count);
	if (r) return r;
	UP_CUDA(u, cudaMemcpyAsync(grads, u->grads.ptr, SW_UPSCALER_NUM_PARAMS * 4, cudaMemcpyDeviceToHost, u->stream));
	float mse = 0.0f;
	if ((r = read_loss(u, count, &mse))) return r;
	if (loss) *loss = 0.5f * mse;
	return SW_OK;
}

int sw_upscaler_train_step(SwUpscaler* u, const SwUpscalerCrop* crops, uint32_t num_crops, float lr, float* mse)
{
	if (!u || !(lr >= 0.0f)) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	uint32_t count = 0;
	int r = forward_backward(u, crops, num_crops, &count);
	if (r) return r;
	if ((r = pack_weights(u, 1, lr, u->stream))) return r;
	if (mse) return read_loss(u, count, mse);
	return SW_OK;
}

int sw_upscaler_steps(SwUpscaler* u, uint64_t* out)
{
	if (!u || !out) return SW_ERR_INVALID_ARGUMENT;
	*out = u->steps;
	return SW_OK;
}

int sw_upscaler_infer(SwUpscaler* u, const uint32_t* lo, uint32_t lo_width, uint32_t lo_height, uint32_t lo_pitch, uint32_t* hi,
	uint32_t hi_pitch, void* stream)
{
	if (!u || !lo || !hi || lo_width == 0 || lo_height == 0 || lo_pitch < lo_width || hi_pitch < 2 * lo_width ||
		(hi_pitch & 1) || (reinterpret_cast<uintptr_t>(hi) & 7))
		return SW_ERR_INVALID_ARGUMENT; // output pixel pairs are stored as 8-byte words
	if (lo_width > 8192 || lo_height > 8192) return fail(u, SW_ERR_LIMIT, "frame too large");
	UP_CUDA(u, cudaSetDevice(u->device));
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : u->stream;
	int r;
	if (u->fused)
	{
		static bool configured = false;
		if (!configured)
		{
			UP_CUDA(u, cudaFuncSetAttribute(fused_upscale_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FusedSmem::TOTAL));
			configured = true;
		}
		FusedArgs f;
		f.lo = lo;
		f.lo_w = lo_width;
		f.lo_h = lo_height;
		f.lo_pitch = lo_pitch;
		f.hi = hi;
		f.hi_pitch = hi_pitch;
		for (int l = 0; l < NUM_LAYERS; ++l)
		{
			f.w[l] = static_cast<const uint16_t*>(u->wfwd[l].ptr);
			f.bias[l] = static_cast<const float*>(u->bias[l].ptr);
		}
		f.strips = (lo_width + F_VALID - 1) / F_VALID;
		f.segments = std::max(1u, std::min(lo_height, uint32_t(u->num_sms) / f.strips));
		f.error = static_cast<int*>(u->error.ptr);
		fused_upscale_kernel<<<f.strips * f.segments, F_THREADS, FusedSmem::TOTAL, s>>>(f);
		UP_CUDA(u, cudaGetLastError());
		return SW_OK;
	}
	if (lo_width != u->i_w || lo_height != u->i_h)
	{
		UP_CUDA(u, cudaStreamSynchronize(s));
		UP_CUDA(u, cudaStreamSynchronize(u->stream));
		dev_free(u->i_x0);
		dev_free(u->i_p);
		dev_free(u->i_q);
		if ((r = dev_alloc(u, u->i_x0, planes_bytes(1, lo_width, lo_height, 2)))) return r;
		if ((r = dev_alloc(u, u->i_p, planes_bytes(1, lo_width, lo_height, 4)))) return r;
		if ((r = dev_alloc(u, u->i_q, planes_bytes(1, lo_width, lo_height, 4)))) return r;
		if ((r = dev_alloc(u, u->i_crop, sizeof(CropGpu)))) return r;
		u->i_crop_valid = false;
		u->i_w = lo_width;
		u->i_h = lo_height;
	}
	// The frame record (source pointer, size, pitches) is re-uploaded only when it changes; the copy
	// from pageable memory is staged before cudaMemcpyAsync returns.
	const CropGpu c{lo, nullptr, lo_width, lo_height, lo_pitch, hi_pitch, 0, 0};
	if (!u->i_crop_valid || memcmp(&c, &u->i_crop_host, sizeof(c)) != 0)
	{
		UP_CUDA(u, cudaMemcpyAsync(u->i_crop.ptr, &c, sizeof(c), cudaMemcpyHostToDevice, s));
		u->i_crop_host = c;
		u->i_crop_valid = true;
	}
	const Planes x0 = make_planes(u->i_x0.ptr, 1, lo_width, lo_height, 2);
	const Planes P = make_planes(u->i_p.ptr, 1, lo_width, lo_height, 4);
	const Planes Q = make_planes(u->i_q.ptr, 1, lo_width, lo_height, 4);
	const CropGpu* dc = static_cast<const CropGpu*>(u->i_crop.ptr);
	convert_input_kernel<<<dim3((lo_width * lo_height + 255) / 256, 1), 256, 0, s>>>(dc, x0);
	UP_CUDA(u, cudaGetLastError());
	ConvArgs a{};
	a.crops = dc;
	a.hi_out = hi;
	a.hi_pitch = hi_pitch;
	a.in = x0, a.out = P, a.wpack = static_cast<uint16_t*>(u->wfwd[0].ptr), a.bias = static_cast<float*>(u->bias[0].ptr);
	if ((r = launch_conv<2, 32, EPI_RELU>(u, a, s))) return r;
	a.in = P, a.out = Q, a.wpack = static_cast<uint16_t*>(u->wfwd[1].ptr), a.bias = static_cast<float*>(u->bias[1].ptr);
	if ((r = launch_conv<4, 32, EPI_RELU>(u, a, s))) return r;
	a.in = Q, a.out = P, a.wpack = static_cast<uint16_t*>(u->wfwd[2].ptr), a.bias = static_cast<float*>(u->bias[2].ptr);
	if ((r = launch_conv<4, 32, EPI_RELU>(u, a, s))) return r;
	a.in = P, a.wpack = static_cast<uint16_t*>(u->wfwd[3].ptr), a.bias = static_cast<float*>(u->bias[3].ptr);
	if ((r = launch_conv<4, 16, EPI_INFER>(u, a, s))) return r;
	return SW_OK;
}

int sw_upscaler_set_fused(SwUpscaler* u, int enable)
{
	if (!u) return SW_ERR_INVALID_ARGUMENT;
	u->fused = enable != 0;
	return SW_OK;
}

int sw_upscaler_wait_probe(SwUpscaler* u, uint32_t max_polls, int* out_code)
{
	if (!u || !out_code || max_polls == 0 || max_polls > POLL_LIMIT) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	int prior = 0;
	UP_CUDA(u, cudaMemcpy(&prior, u->error.ptr, sizeof(int), cudaMemcpyDeviceToHost));
	if (prior) return fail(u, SW_ERR_STATE, "an earlier kernel already gave up (code %d)", prior);
	wait_probe_kernel<<<1, 128, 0, u->stream>>>(static_cast<int*>(u->error.ptr), max_polls);
	UP_CUDA(u, cudaGetLastError());
	UP_CUDA(u, cudaMemcpyAsync(out_code, u->error.ptr, sizeof(int), cudaMemcpyDeviceToHost, u->stream));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	// the probe's record is not a failure of the upscaler's work: clear it
	UP_CUDA(u, cudaMemsetAsync(u->error.ptr, 0, sizeof(int), u->stream));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	return SW_OK;
}

int sw_upscaler_check(SwUpscaler* u)
{
	if (!u) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	UP_CUDA(u, cudaDeviceSynchronize());
	return check_error_flag(u, u->stream);
}

int sw_upscaler_psnr(SwUpscaler* u, const uint32_t* a, uint32_t a_pitch, const uint32_t* b, uint32_t b_pitch, uint32_t width,
	uint32_t height, void* stream, double* out_psnr)
{
	if (!u || !a || !b || !out_psnr || width == 0 || height == 0 || a_pitch < width || b_pitch < width)
		return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : u->stream;
	UP_CUDA(u, cudaMemsetAsync(u->psnr_sum.ptr, 0, 8, s));
	psnr_kernel<<<1216, 256, 0, s>>>(a, a_pitch, b, b_pitch, width, height, static_cast<unsigned long long*>(u->psnr_sum.ptr));
	UP_CUDA(u, cudaGetLastError());
	UP_CUDA(u, cudaMemcpyAsync(u->h_psnr, u->psnr_sum.ptr, 8, cudaMemcpyDeviceToHost, s));
	UP_CUDA(u, cudaStreamSynchronize(s));
	const double mse = double(*u->h_psnr) / (3.0 * double(width) * double(height));
	*out_psnr = mse <= 0.0 ? 99.0 : std::min(99.0, 10.0 * std::log10(255.0 * 255.0 / mse));
	return SW_OK;
}

// Checkpoint file: magic "SWUPSCL1", u32 version, u32 num_params, u64 steps, params, m, v (f32 each),
// then the FNV-1a 64 hash of everything before it.
int sw_upscaler_save(SwUpscaler* u, const char* path)
{
	if (!u || !path) return SW_ERR_INVALID_ARGUMENT;
	UP_CUDA(u, cudaSetDevice(u->device));
	const size_t n = SW_UPSCALER_NUM_PARAMS;
	std::vector<unsigned char> buf(8 + 4 + 4 + 8 + 3 * n * 4);
	memcpy(buf.data(), "SWUPSCL1", 8);
	const uint32_t version = 1, np = uint32_t(n);
	memcpy(buf.data() + 8, &version, 4);
	memcpy(buf.data() + 12, &np, 4);
	memcpy(buf.data() + 16, &u->steps, 8);
	unsigned char* p = buf.data() + 24;
	UP_CUDA(u, cudaMemcpyAsync(p, u->params.ptr, n * 4, cudaMemcpyDeviceToHost, u->stream));
	UP_CUDA(u, cudaMemcpyAsync(p + n * 4, u->adam_m.ptr, n * 4, cudaMemcpyDeviceToHost, u->stream));
	UP_CUDA(u, cudaMemcpyAsync(p + 2 * n * 4, u->adam_v.ptr, n * 4, cudaMemcpyDeviceToHost, u->stream));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	const uint64_t h = fnv1a(buf.data(), buf.size());
	FILE* f = fopen(path, "wb");
	if (!f) return fail(u, SW_ERR_INVALID_ARGUMENT, "cannot open %s", path);
	const bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size() && fwrite(&h, 1, 8, f) == 8;
	fclose(f);
	return ok ? SW_OK : fail(u, SW_ERR_INVALID_ARGUMENT, "write to %s failed", path);
}

int sw_upscaler_load(SwUpscaler* u, const char* path)
{
	if (!u || !path) return SW_ERR_INVALID_ARGUMENT;
	const size_t n = SW_UPSCALER_NUM_PARAMS;
	std::vector<unsigned char> buf(8 + 4 + 4 + 8 + 3 * n * 4 + 8);
	FILE* f = fopen(path, "rb");
	if (!f) return fail(u, SW_ERR_INVALID_ARGUMENT, "cannot open %s", path);
	const size_t got = fread(buf.data(), 1, buf.size(), f);
	const int extra = fgetc(f);
	fclose(f);
	if (got != buf.size() || extra != EOF) return fail(u, SW_ERR_INVALID_ARGUMENT, "%s: wrong size", path);
	uint32_t version, np;
	memcpy(&version, buf.data() + 8, 4);
	memcpy(&np, buf.data() + 12, 4);
	if (memcmp(buf.data(), "SWUPSCL1", 8) != 0 || version != 1 || np != n)
		return fail(u, SW_ERR_INVALID_ARGUMENT, "%s: not an upscaler checkpoint of this version", path);
	uint64_t h;
	memcpy(&h, buf.data() + buf.size() - 8, 8);
	if (fnv1a(buf.data(), buf.size() - 8) != h) return fail(u, SW_ERR_INVALID_ARGUMENT, "%s: hash mismatch", path);
	uint64_t steps;
	memcpy(&steps, buf.data() + 16, 8);
	const float* p = reinterpret_cast<const float*>(buf.data() + 24);
	int r = sw_upscaler_set_params(u, p, uint32_t(n));
	if (r) return r;
	UP_CUDA(u, cudaMemcpyAsync(u->adam_m.ptr, p + n, n * 4, cudaMemcpyHostToDevice, u->stream));
	UP_CUDA(u, cudaMemcpyAsync(u->adam_v.ptr, p + 2 * n, n * 4, cudaMemcpyHostToDevice, u->stream));
	UP_CUDA(u, cudaStreamSynchronize(u->stream));
	u->steps = steps;
	return SW_OK;
}

int sw_monitor_init(SwMonitor* m, uint32_t check_interval, float threshold_db, uint32_t fallback_frames)
{
	if (!m || check_interval == 0 || fallback_frames == 0 || !std::isfinite(threshold_db)) return SW_ERR_INVALID_ARGUMENT;
	memset(m, 0, sizeof(*m));
	m->check_interval = check_interval;
	m->fallback_frames = fallback_frames;
	m->threshold_db = threshold_db;
	m->recheck = 1; // the first learned frame is checked
	return SW_OK;
}

int sw_monitor_plan(SwMonitor* m, uint32_t* out_plan)
{
	if (!m || !out_plan || m->check_interval == 0) return SW_ERR_INVALID_ARGUMENT;
	if (m->check_pending) return SW_ERR_STATE; // the last checked frame has no report yet
	++m->frames;
	if (m->plain_left > 0)
	{
		--m->plain_left;
		++m->plain_frames;
		*out_plan = SW_PLAN_PLAIN;
		return SW_OK;
	}
	++m->learned_frames;
	if (m->recheck || m->since_check + 1 >= m->check_interval)
	{
		m->recheck = 0;
		m->since_check = 0;
		m->check_pending = 1;
		++m->checks;
		*out_plan = SW_PLAN_LEARNED_CHECKED;
		return SW_OK;
	}
	++m->since_check;
	*out_plan = SW_PLAN_LEARNED;
	return SW_OK;
}

int sw_monitor_report(SwMonitor* m, double psnr_db)
{
	if (!m) return SW_ERR_INVALID_ARGUMENT;
	if (!m->check_pending) return SW_ERR_STATE;
	m->check_pending = 0;
	m->last_psnr_db = float(psnr_db);
	if (!(psnr_db >= double(m->threshold_db))) // NaN fails too
	{
		++m->failed_checks;
		++m->fallbacks;
		m->plain_left = m->fallback_frames;
		m->recheck = 1;
	}
	return SW_OK;
}

} // extern "C"
