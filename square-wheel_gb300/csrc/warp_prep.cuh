// Warp-cooperative pieces of the per-polygon preparation shared by the GPU-side surface and draw
// preparation (prep.cu) and the shadow-map sides' depth draws (raster.cu): one warp per polygon, one
// vertex per lane. The sequential loops of the host code (host/prep_math.h, compiled for the device
// without FMA contraction and with IEEE division and square root) become lane-parallel steps that
// reproduce them exactly: a clip pass classifies every vertex and its predecessor with the same
// comparisons, emits the same elements (computed by the same expressions: line_z_intersection /
// line_line_intersection of (previous, current)) at positions given by a prefix sum, and truncates at
// SW_MAX_POLYGON_VERTICES like the sequential `count == out_cap` break.
#pragma once

#include "sw_kernels.cuh"
#include "../host/prep_math.h"

namespace swgpu
{
namespace
{

using swhost::Mat4;
using swhost::Vec2;
using swhost::Vec3;
using swhost::Vec4;

// bar.sync on barrier `id` (1..15) for `threads` threads (whole warps).
__device__ __forceinline__ void named_barrier(uint32_t id, uint32_t threads)
{
	asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

__device__ inline Mat4 load_mat4(const float* m)
{
	Mat4 r;
	for (int c = 0; c < 4; ++c) r.c[c] = swhost::v4(m[c * 4 + 0], m[c * 4 + 1], m[c * 4 + 2], m[c * 4 + 3]);
	return r;
}

__device__ inline void load_planes(const float (*p)[3], Vec3 out[8])
{
	for (int k = 0; k < 8; ++k) out[k] = swhost::v3(p[k][0], p[k][1], p[k][2]);
}

// Largest i in [0, n) with base[i] <= x (base[0] == 0 <= x).
__device__ inline uint32_t find_segment(const uint32_t* base, uint32_t n, uint32_t x)
{
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1)
	{
		const uint32_t mid = (lo + hi) >> 1;
		if (base[mid] <= x)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}


constexpr uint32_t FULL_MASK = 0xFFFFFFFFu;
constexpr uint32_t MAXV = SW_MAX_POLYGON_VERTICES;

struct WarpClipBuf
{
	Vec3 v3[MAXV];
	Vec2 v2[MAXV];
};

__device__ inline Vec2 shfl(Vec2 v, int src) { return swhost::v2(__shfl_sync(FULL_MASK, v.x, src), __shfl_sync(FULL_MASK, v.y, src)); }
__device__ inline Vec3 shfl(Vec3 v, int src)
{
	return swhost::v3(__shfl_sync(FULL_MASK, v.x, src), __shfl_sync(FULL_MASK, v.y, src), __shfl_sync(FULL_MASK, v.z, src));
}

// Outcome of the sequential code's comparisons of a against b: 1 (a > b), 0 (a == b), -1 (a < b), 2 (NaN).
__device__ inline int cmp_class(float a, float b) { return a > b ? 1 : (a == b ? 0 : (a < b ? -1 : 2)); }

// One pass of clip_3d_polygon_by_z_plane / clip_2d_polygon (clipping.rs:4-51, 115-175). Lane i < n holds
// vertex i and the class of its test (c); returns the new count, lane k < count holding vertex k.
template <class T, class F>
__device__ inline uint32_t warp_clip_pass(T& v, int c, uint32_t n, T* buf, F isect)
{
	const uint32_t lane = threadIdx.x & 31u;
	// every vertex strictly inside: the sequential pass emits its input unchanged
	if (__all_sync(FULL_MASK, lane >= n || c == 1)) return n;
	const int prev = int(lane == 0 ? n - 1 : lane - 1);
	const T pv = shfl(v, prev);
	const int pc = __shfl_sync(FULL_MASK, c, prev);
	bool emit_i = false, emit_v = false;
	if (lane < n)
	{
		if (c == 1)
		{
			emit_i = pc == -1;
			emit_v = true;
		}
		else if (c == 0)
			emit_v = true;
		else if (pc == 1)
			emit_i = true;
	}
	// output position: elements emitted by the lanes before this one (each emits 0, 1 or 2)
	const uint32_t bi = __ballot_sync(FULL_MASK, emit_i), bv = __ballot_sync(FULL_MASK, emit_v);
	const uint32_t before = (1u << lane) - 1u;
	const uint32_t pos = uint32_t(__popc(bi & before) + __popc(bv & before));
	const uint32_t total = uint32_t(__popc(bi) + __popc(bv));
	if (emit_i && pos < MAXV) buf[pos] = isect(pv, v);
	if (emit_v && pos + uint32_t(emit_i) < MAXV) buf[pos + uint32_t(emit_i)] = v;
	__syncwarp();
	const uint32_t count = total < MAXV ? total : MAXV;
	if (lane < count) v = buf[lane];
	__syncwarp();
	return count;
}

// project_and_clip_polygon (renderer_utils.rs:10-58) of lane-held transformed vertices (lane < n).
__device__ inline uint32_t warp_project_and_clip(const Vec3 planes[8], Vec3 vt, uint32_t n, Vec2& out, WarpClipBuf& buf)
{
	const uint32_t lane = threadIdx.x & 31u;
	uint32_t count = n < MAXV ? n : MAXV;
	if (count == 0) return 0;
	Vec3 zv = vt;
	count = warp_clip_pass(zv, cmp_class(zv.z, swhost::PREP_Z_NEAR), count, buf.v3,
		[](Vec3 a, Vec3 b) { return swhost::line_z_intersection(a, b, swhost::PREP_Z_NEAR); });
	if (count < 3) return count;
	Vec2 p = lane < count ? swhost::v2(zv.x, zv.y) / zv.z : swhost::v2(0.0f, 0.0f);
	for (int i = 0; i < 8; ++i)
	{
		const Vec3 line = planes[i];
		const float dist = swhost::dot(p, swhost::v2(line.x, line.y)) - line.z;
		count = warp_clip_pass(p, cmp_class(dist, 0.0f), count, buf.v2,
			[line](Vec2 a, Vec2 b) { return swhost::line_line_intersection(a, b, line); });
		if (count < 3) return count;
	}
	out = p;
	return count;
}

} // namespace
} // namespace swgpu
