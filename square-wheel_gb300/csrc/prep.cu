// GPU-side surface and draw preparation (sw_draw_frame_view).
//
// The reference prepares surfaces and draws on the host, one polygon after another:
//   prepare_polygons_surfaces / prepare_polygon_surface (src/square_wheel/partial_renderer.rs:1327-1638)
//   allocates each visible polygon's surface in leaf index order; build_polygons_surfaces (:1640-1819)
//   fills its descriptor and light list; draw_tree / draw_leaf / draw_polygon (:2450-2559, :4011-4142)
//   emits the draws back to front.
// Here every polygon of the visible leafs is one warp of prep_polygons_kernel (a vertex per lane), which
// evaluates the host's per-polygon expressions (host/prep_math.h, compiled for the device without FMA
// contraction and with IEEE division and square root) with the sequential loops turned into exact
// lane-parallel equivalents. The serial parts of the reference - the running surface offset and the
// submission order - become prefix sums in prep_compact_kernel: one CTA scans the
// candidates in allocation order (surface index, texel offset) and the drawn leafs' polygons in draw
// order (draw index, first vertex, first row record), and writes the surface records, descriptors,
// draws, vertices and row ranges the surface build and the rasteriser read, plus the counts they
// take their sizes from. Everything stays on the device; the host only uploads the visible leafs.
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

constexpr int PREP_WARPS = 4;         // per-candidate kernel: one warp per polygon, 4 per CTA
constexpr int COMPACT_THREADS = 1024; // compaction: one CTA

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

// ---- warp-cooperative per-polygon preparation: one warp per polygon, one vertex per lane ----
//
// The sequential loops of the host code become lane-parallel steps that reproduce them exactly: a clip
// pass classifies every vertex and its predecessor with the same comparisons, emits the same elements
// (computed by the same expressions: line_z_intersection / line_line_intersection of (previous,
// current)) at positions given by a prefix sum, and truncates at SW_MAX_POLYGON_VERTICES like the
// sequential `count == out_cap` break; running "if (x < best) best = x" searches become the first lane
// attaining the extremum, whose value is taken as is (so even the sign of a zero matches).

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

// ceil(RN(log2(x)) * scale + bias) for the two ceil decisions of the preparation (calculate_mip:
// scale 0.5, bias mip_bias; the z scale of draw_polygon: scale 1, bias 0) - the value the host gets from
// log2_rn. The decision is monotone in the logarithm, so it is taken from log2f's result widened by a
// few representable steps on both sides (more than log2f's error); only when the two ends disagree is
// the correctly rounded logarithm evaluated in double precision.
__device__ inline float ceil_log2_decision(float x, float scale, float bias)
{
	const float lf = log2f(x);
	if (lf == lf && fabsf(lf) < 1.0e30f)
	{
		float lo = lf, hi = lf;
		for (int k = 0; k < 4; ++k)
		{
			lo = nextafterf(lo, -INFINITY);
			hi = nextafterf(hi, INFINITY);
		}
		const float c_lo = ceilf(lo * scale + bias), c_hi = ceilf(hi * scale + bias);
		if (c_lo == c_hi) return c_lo;
	}
	return ceilf(swhost::log2_rn(x) * scale + bias);
}

// Sequential `if (x < best) { best = x; at = i; }` over the valid lanes in lane order, from best = init:
// returns best, *at = its lane (or -1: init kept).
__device__ inline float warp_first_min(float x, bool valid, float init, int* at)
{
	const bool cand = valid && x < init;
	float m = cand ? x : __int_as_float(0x7F800000); // +inf
	for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(FULL_MASK, m, o));
	const uint32_t mask = __ballot_sync(FULL_MASK, cand && x == m);
	if (!mask)
	{
		*at = -1;
		return init;
	}
	*at = __ffs(mask) - 1;
	return __shfl_sync(FULL_MASK, x, *at);
}
// The same for `if (x > best)`.
__device__ inline float warp_first_max(float x, bool valid, float init, int* at)
{
	const bool cand = valid && x > init;
	float m = cand ? x : __int_as_float(0xFF800000); // -inf
	for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
	const uint32_t mask = __ballot_sync(FULL_MASK, cand && x == m);
	if (!mask)
	{
		*at = -1;
		return init;
	}
	*at = __ffs(mask) - 1;
	return __shfl_sync(FULL_MASK, x, *at);
}

constexpr uint32_t PREP_SMEM_LEAFS = 512; // leaf table staged per CTA up to this many leafs

__global__ void __launch_bounds__(PREP_WARPS * 32) prep_polygons_kernel(PrepArgs a)
{
	__shared__ WarpClipBuf s_buf[PREP_WARPS];
	__shared__ uint32_t s_base[PREP_SMEM_LEAFS + 1];
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	const uint32_t c = blockIdx.x * PREP_WARPS + warp;
	pdl_trigger(); // the compaction may be scheduled; it waits for this grid before reading
	const PrepFrame& frame = *a.frame;
	const uint32_t num_candidates = frame.num_candidates, num_leafs = frame.num_leafs;
	if (blockIdx.x * PREP_WARPS >= num_candidates) return; // the grid is sized for the capacity
	const bool staged = num_leafs <= PREP_SMEM_LEAFS;
	if (staged)
	{
		for (uint32_t i = threadIdx.x; i <= num_leafs; i += blockDim.x) s_base[i] = __ldg(a.leaf_cand_base + i);
		__syncthreads();
	}
	if (c >= num_candidates) return;
	WarpClipBuf& buf = s_buf[warp];
	const uint32_t* cand_base = staged ? s_base : a.leaf_cand_base;
	const uint32_t li = find_segment(cand_base, num_leafs, c);
	const SwViewLeaf& leaf = a.leafs[li];
	const uint32_t pi = leaf.first_polygon + (c - cand_base[li]);
	const SwMapPolygon& p = a.polygons[pi];
	// the leaf's first 32 lights, one per lane, loaded ahead of their use
	const uint32_t leaf_first_light = leaf.first_light, leaf_num_lights = leaf.num_lights;
	const uint32_t my_light = lane < leaf_num_lights ? uint32_t(a.leaf_lights[leaf_first_light + lane]) : 0u;
	const SwLight light0 = a.lights[lane < leaf_num_lights ? my_light : 0u];
	PrepCand& out = a.cands[c];
	PrepKey& key = a.keys[c];

	// prepare_polygon_surface (partial_renderer.rs:1464-1638)
	const Mat4 planes_matrix = load_mat4(frame.planes);
	const Vec4 plane_transformed = planes_matrix * swhost::extend(swhost::poly_vec3(p.plane), -p.plane[3]);
	const uint32_t flags = p.flags;
	if (plane_transformed.w <= 0.0f || !(flags & SW_POLY_DRAW))
	{
		if (lane == 0) key = PrepKey{0ull, 0u, 0u, 0u, 0};
		return;
	}
	const Mat4 view = load_mat4(frame.view);
	const uint32_t nv = p.num_vertices < MAXV ? p.num_vertices : MAXV;
	const Vec3* mv = reinterpret_cast<const Vec3*>(a.map_vertices);
	const Vec3 vt = lane < nv ? swhost::view_transform(view, mv[p.first_vertex + lane]) : swhost::v3(0.0f, 0.0f, 1.0f);
	Vec3 planes[8];
	load_planes(leaf.clip_planes, planes);
	Vec2 q;
	const uint32_t count = warp_project_and_clip(planes, vt, nv, q, buf);
	if (count < 3 || (flags & SW_POLY_SKY)) // hidden, or sky (its bounds are the host's)
	{
		if (lane == 0) key = PrepKey{0ull, 0u, 0u, 0u, 0};
		return;
	}
	const float pw = -plane_transformed.w;
	const swhost::DepthEquation de{plane_transformed.x / pw, plane_transformed.y / pw, plane_transformed.z / pw};
	const Vec4 tb[2] = {planes_matrix * swhost::extend(swhost::poly_vec3(p.tex_coord_equation[0]), p.tex_coord_equation[0][3]),
		planes_matrix * swhost::extend(swhost::poly_vec3(p.tex_coord_equation[1]), p.tex_coord_equation[1][3])};
	swhost::TexCoordEquation te;
	for (int i = 0; i < 2; ++i)
	{
		te.d_tc_dx[i] = tb[i].x + tb[i].w * de.d_inv_z_dx;
		te.d_tc_dy[i] = tb[i].y + tb[i].w * de.d_inv_z_dy;
		te.k[i] = tb[i].z + tb[i].w * de.k;
	}
	// calculate_mip (renderer_utils.rs:201-242): the first point of largest inv_z above 0, else point 0
	const bool in_poly = lane < count;
	int at;
	const float mip_point_inv_z = warp_first_max(de.sample(q), in_poly, 0.0f, &at);
	const Vec2 mip_point = shfl(q, at < 0 ? 0 : at);
	uint32_t mip;
	{
		const float z_2 = 1.0f / (mip_point_inv_z * mip_point_inv_z);
		const float z_4 = z_2 * z_2;
		float d_tc_2[2];
		for (int i = 0; i < 2; ++i)
		{
			const float d_tc_dx =
				te.d_tc_dx[i] * (de.k + de.d_inv_z_dy * mip_point.y) - (te.k[i] + te.d_tc_dy[i] * mip_point.y) * de.d_inv_z_dx;
			const float d_tc_dy =
				te.d_tc_dy[i] * (de.k + de.d_inv_z_dx * mip_point.x) - (te.k[i] + te.d_tc_dx[i] * mip_point.x) * de.d_inv_z_dy;
			d_tc_2[i] = (d_tc_dx * d_tc_dx + d_tc_dy * d_tc_dy) * z_4;
		}
		const int32_t m = swhost::as_i32(ceil_log2_decision(fmaxf(d_tc_2[0], d_tc_2[1]), 0.5f, frame.mip_bias));
		mip = uint32_t(m < 0 ? 0 : (m > int32_t(swhost::PREP_MAX_MIP) ? int32_t(swhost::PREP_MAX_MIP) : m));
	}
	const float mip_scale = 1.0f / float(1u << mip);
	swhost::TexCoordEquation ts;
	for (int i = 0; i < 2; ++i)
	{
		ts.d_tc_dx[i] = te.d_tc_dx[i] * mip_scale;
		ts.d_tc_dy[i] = te.d_tc_dy[i] * mip_scale;
		ts.k[i] = te.k[i] * mip_scale;
	}
	// surface rectangle: tc bounds over the clipped polygon, lightmap-aligned clamp
	swhost::SurfacePrep sp;
	{
		const float inf = float(1 << 29);
		const float max_z = float(1 << 16);
		const float inv_z = fmaxf(de.sample(q), 1.0f / max_z);
		const float z = 1.0f / inv_z;
		for (int i = 0; i < 2; ++i)
		{
			const float tc = z * (ts.d_tc_dx[i] * q.x + ts.d_tc_dy[i] * q.y + ts.k[i]);
			int unused;
			float tc_min = warp_first_min(tc, in_poly, inf, &unused);
			float tc_max = warp_first_max(tc, in_poly, -inf, &unused);
			const float eps = 1.0f / 32.0f;
			tc_min += eps;
			tc_max -= eps;
			const int32_t round_mask = ~int32_t((1u << swhost::PREP_LIGHTMAP_SCALE_LOG2) - 1);
			const int32_t min_down = (p.tex_coord_min[i] & round_mask) >> mip;
			const int32_t max_up = ((p.tex_coord_max[i] + int32_t(1u << swhost::PREP_LIGHTMAP_SCALE_LOG2) - 1) & round_mask) >> mip;
			int32_t tmin = swhost::as_i32(floorf(fmaxf(tc_min, -inf)));
			if (tmin < min_down) tmin = min_down;
			int32_t tmax = swhost::as_i32(ceilf(fminf(tc_max, inf)));
			if (tmax > max_up) tmax = max_up;
			if (tmin >= tmax)
			{
				if (tmin > max_up - 1) tmin = max_up - 1;
				tmax = tmin + 1;
			}
			sp.tc_min[i] = tmin;
			sp.size[i] = uint32_t(tmax - tmin);
		}
		sp.depth = de;
		sp.tc = ts;
		sp.mip = mip;
		for (int i = 0; i < 2; ++i)
		{
			const float tmf = float(sp.tc_min[i]);
			sp.tc.d_tc_dx[i] -= tmf * de.d_inv_z_dx;
			sp.tc.d_tc_dy[i] -= tmf * de.d_inv_z_dy;
			sp.tc.k[i] -= tmf * de.k;
		}
	}

	// build_polygons_surfaces: descriptor and the leaf's lights that reach the polygon, in order, up to 6
	SwSurfaceDesc d;
	swhost::make_surface_desc(p, sp, 0, a.directional != 0, a.simple_lightmaps != 0, d);
	if (flags & SW_POLY_DIFFUSE_LAYER)
		for (uint32_t base = 0; base < leaf_num_lights && d.num_lights < SW_MAX_POLYGON_LIGHTS; base += 32)
		{
			const uint32_t k = base + lane;
			bool hit = false;
			uint32_t light = my_light;
			if (k < leaf_num_lights)
			{
				if (base > 0) light = a.leaf_lights[leaf_first_light + k];
				hit = swhost::polygon_is_affected_by_light(p, base > 0 ? a.lights[light] : light0);
			}
			uint32_t mask = __ballot_sync(FULL_MASK, hit);
			while (mask && d.num_lights < SW_MAX_POLYGON_LIGHTS)
			{
				const uint32_t b = uint32_t(__ffs(mask) - 1);
				mask &= mask - 1;
				d.lights[d.num_lights++] = uint16_t(__shfl_sync(FULL_MASK, light, int(b)));
			}
		}
	if (lane == 0) out.desc = d;
	uint32_t draw_count = 0, row_n = 0;
	int32_t row_y0 = 0;

	// draw_leaf -> draw_polygon (partial_renderer.rs:4011-4142) with the leaf's draw bounds
	if (leaf.draw_order != SW_LEAF_NOT_DRAWN && p.num_vertices >= 3)
	{
		Vec3 draw_planes[8];
		load_planes(leaf.draw_clip_planes, draw_planes);
		Vec2 v;
		const uint32_t n = warp_project_and_clip(draw_planes, vt, nv, v, buf);
		if (n >= 3)
		{
			const bool in_draw = lane < n;
			const float inv_z = sp.depth.sample(v);
			int min_i, max_i, unused;
			warp_first_min(inv_z, in_draw, 1e24f, &min_i);
			const float max_inv_z = warp_first_max(inv_z, in_draw, -1e24f, &max_i);
			const float min_x = warp_first_min(v.x, in_draw, 1e24f, &unused);
			const float max_x = warp_first_max(v.x, in_draw, -1e24f, &unused);
			const Vec2 p_min = shfl(v, min_i < 0 ? 0 : min_i), p_max = shfl(v, max_i < 0 ? 0 : max_i);
			const SwVertex16 fv{swhost::as_i32(v.x * 65536.0f), swhost::as_i32(v.y * 65536.0f)};
			if (in_draw) out.v[lane] = fv;
			SwDrawCmd dc = SwDrawCmd{};
			dc.vertex_count = n;
			dc.blend = p.blending_mode;
			dc.tex_size[0] = sp.size[0];
			dc.tex_size[1] = sp.size[1];
			dc.tex_source = SW_TEXSRC_SURFACE;
			swhost::DepthEquation dd = sp.depth;
			swhost::TexCoordEquation dt = sp.tc;
			if (swhost::affine_may_be_used(sp.depth, sp.tc, p_min, p_max))
				dc.mode = SW_RASTER_AFFINE;
			else
			{
				const float z_scale = swhost::exp2_int(-5.0f - ceil_log2_decision(fmaxf(max_inv_z, 1.0f / float(1 << 20)), 1.0f, 0.0f));
				dd = swhost::DepthEquation{dd.d_inv_z_dx * z_scale, dd.d_inv_z_dy * z_scale, dd.k * z_scale};
				for (int i = 0; i < 2; ++i)
				{
					dt.d_tc_dx[i] *= z_scale;
					dt.d_tc_dy[i] *= z_scale;
					dt.k[i] *= z_scale;
				}
				dc.mode = swhost::line_z_may_be_used(sp.depth, sp.tc, p_max, min_x, max_x) ? SW_RASTER_LINE_Z_CORRECTED
																						  : SW_RASTER_FULL_PERSPECTIVE;
			}
			dc.depth_eq[0] = dd.d_inv_z_dx;
			dc.depth_eq[1] = dd.d_inv_z_dy;
			dc.depth_eq[2] = dd.k;
			for (int i = 0; i < 2; ++i)
			{
				dc.tc_eq[i] = dt.d_tc_dx[i];
				dc.tc_eq[2 + i] = dt.d_tc_dy[i];
				dc.tc_eq[4 + i] = dt.k[i];
			}
			if (lane == 0) out.draw = dc;
			// draw_row_range: [round(min y), round(max y)) clipped to the frame
			const int32_t y_lo = __reduce_min_sync(FULL_MASK, in_draw ? fv.y : INT32_MAX);
			const int32_t y_hi = __reduce_max_sync(FULL_MASK, in_draw ? fv.y : INT32_MIN);
			const int32_t r0 = int32_t(uint32_t(y_lo) + 0x8000u) >> 16, r1 = int32_t(uint32_t(y_hi) + 0x8000u) >> 16;
			const int32_t ra = r0 > 0 ? r0 : 0, rb = r1 < a.height ? r1 : a.height;
			row_y0 = ra;
			row_n = rb > ra ? uint32_t(rb - ra) : 0u;
			draw_count = n;
		}
	}
	if (lane == 0) key = PrepKey{uint64_t(sp.size[0]) * sp.size[1], 1u, draw_count, row_n, row_y0};
}

// Exclusive prefix sums of N values over the CTA (COMPACT_THREADS threads); `total` gets the sums.
template <int N>
__device__ inline void block_scan_exclusive(uint64_t (&x)[N], uint64_t (&total)[N])
{
	__shared__ uint64_t s_warp[COMPACT_THREADS / 32][N];
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint64_t inc[N];
	for (int i = 0; i < N; ++i) inc[i] = x[i];
	for (int o = 1; o < 32; o <<= 1)
		for (int i = 0; i < N; ++i)
		{
			const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, inc[i], o);
			if (lane >= uint32_t(o)) inc[i] += t;
		}
	if (lane == 31)
		for (int i = 0; i < N; ++i) s_warp[warp][i] = inc[i];
	__syncthreads();
	if (warp == 0)
		for (int i = 0; i < N; ++i)
		{
			uint64_t w = s_warp[lane][i];
			for (int o = 1; o < 32; o <<= 1)
			{
				const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, w, o);
				if (lane >= uint32_t(o)) w += t;
			}
			s_warp[lane][i] = w; // inclusive over warps
		}
	__syncthreads();
	for (int i = 0; i < N; ++i)
	{
		const uint64_t before = warp > 0 ? s_warp[warp - 1][i] : 0ull;
		x[i] = before + inc[i] - x[i];
		total[i] = s_warp[COMPACT_THREADS / 32 - 1][i];
	}
	__syncthreads(); // s_warp is reused by the next call
}

constexpr uint32_t SMEM_LEAFS = 2048; // index arrays staged in shared memory up to this many leafs

__global__ void __launch_bounds__(COMPACT_THREADS, 1) prep_compact_kernel(PrepArgs a)
{
	__shared__ uint32_t s_error;
	__shared__ uint32_t s_cand_base[SMEM_LEAFS + 1], s_slot_base[SMEM_LEAFS + 1], s_draw_leaf[SMEM_LEAFS];
	__shared__ uint32_t s_vcand[COMPACT_THREADS], s_vbase[COMPACT_THREADS + 1]; // the chunk's draws: vertex copy list
	const uint32_t tid = threadIdx.x;
	if (tid == 0) s_error = 0;
	// Before the per-candidate grid has finished: the uploaded index arrays and the host's draws
	// (draw_skybox: they come first, with their row records).
	const PrepFrame& frame = *a.frame;
	const uint32_t num_leafs = frame.num_leafs, num_candidates = frame.num_candidates, num_draw_leafs = frame.num_draw_leafs;
	const uint32_t num_host_draws = frame.num_host_draws, num_host_vertices = frame.num_host_vertices;
	const bool staged = num_leafs <= SMEM_LEAFS;
	if (staged)
	{
		for (uint32_t i = tid; i <= num_leafs; i += blockDim.x) s_cand_base[i] = __ldg(a.leaf_cand_base + i);
		for (uint32_t i = tid; i <= num_draw_leafs; i += blockDim.x) s_slot_base[i] = __ldg(a.draw_slot_base + i);
		for (uint32_t i = tid; i < num_draw_leafs; i += blockDim.x) s_draw_leaf[i] = __ldg(a.draw_leaf + i);
	}
	const uint32_t* cand_base = staged ? s_cand_base : a.leaf_cand_base;
	const uint32_t* slot_base = staged ? s_slot_base : a.draw_slot_base;
	const uint32_t* draw_leaf = staged ? s_draw_leaf : a.draw_leaf;
	for (uint32_t i = tid; i < num_host_draws && i < a.cap_draws; i += blockDim.x)
	{
		a.draws[i] = a.host_draws[i];
		a.draw_rows[i] = a.host_rows[i];
	}
	for (uint32_t i = tid; i < num_host_vertices && i < a.cap_vertices; i += blockDim.x) a.vertices[i] = a.host_vertices[i];
	pdl_wait(); // prep_polygons_kernel has completed
	__syncthreads();

	// Surfaces in allocation order: index and texel offset are prefix sums over the candidates.
	uint64_t num_surfaces = 0, total_texels = 0;
	for (uint32_t base = 0; base < num_candidates; base += blockDim.x)
	{
		const uint32_t c = base + tid;
		const PrepKey k = c < num_candidates ? a.keys[c] : PrepKey{0ull, 0u, 0u, 0u, 0};
		const bool vis = k.state == 1;
		const uint64_t area = vis ? k.area : 0ull;
		uint64_t x[2] = {vis ? 1ull : 0ull, area}, tot[2];
		block_scan_exclusive<2>(x, tot);
		if (vis)
		{
			const uint64_t s = num_surfaces + x[0], offset = total_texels + x[1];
			a.cands[c].surface_offset = offset;
			if (s < a.cap_surfaces && offset + area <= a.cap_texels)
			{
				SwSurfaceDesc d = a.cands[c].desc;
				d.out_offset = offset;
				a.descs[s] = d;
				SurfaceGpu g;
				make_surface_gpu(d, (d.flags & SW_SURF_DIFFUSE_LAYER) ? &a.texture_mips[d.texture_mip] : nullptr,
					d.emissive_mip != SW_NO_EMISSIVE ? &a.emissive_mips[d.emissive_mip] : nullptr, g);
				a.surfaces[s] = g;
				a.work_prefix[s] = offset;
			}
			else
				atomicOr(&s_error, 1u);
		}
		num_surfaces += tot[0];
		total_texels += tot[1];
	}
	if (tid == 0 && num_surfaces <= a.cap_surfaces) a.work_prefix[num_surfaces] = total_texels;
	__syncthreads(); // surface offsets of every candidate are visible to the CTA

	// Draws in submission order: drawn leafs back to front, each leaf's polygons in index order.
	const uint32_t slots = num_draw_leafs ? slot_base[num_draw_leafs] : 0u;
	uint64_t num_draws = num_host_draws, num_vertices = num_host_vertices, num_rows = frame.num_host_rows;
	for (uint32_t base = 0; base < slots; base += blockDim.x)
	{
		const uint32_t slot = base + tid;
		PrepKey k{0ull, 0u, 0u, 0u, 0};
		uint32_t c = 0;
		if (slot < slots)
		{
			const uint32_t j = find_segment(slot_base, num_draw_leafs, slot);
			c = cand_base[draw_leaf[j]] + (slot - slot_base[j]);
			k = a.keys[c];
		}
		const bool emit = k.state == 1 && k.draw_count >= 3;
		const uint32_t nv = emit ? k.draw_count : 0u;
		const uint32_t nr = emit ? k.row_n : 0u;
		uint64_t x[3] = {emit ? 1ull : 0ull, nv, nr}, tot[3];
		block_scan_exclusive<3>(x, tot);
		const bool fits = num_draws + tot[0] <= a.cap_draws && num_vertices + tot[1] <= a.cap_vertices &&
						  num_rows + tot[2] <= a.cap_rows;
		if (emit)
		{
			const uint64_t di = num_draws + x[0], vb = num_vertices + x[1], rb = num_rows + x[2];
			if (fits)
			{
				SwDrawCmd d = a.cands[c].draw;
				d.first_vertex = uint32_t(vb);
				d.tex_offset = a.cands[c].surface_offset;
				a.draws[di] = d;
				a.draw_rows[di] = DrawRows{uint32_t(rb), k.row_y0, nr, 0u};
			}
			else
				atomicOr(&s_error, 1u);
			s_vcand[x[0]] = c;
			s_vbase[x[0]] = uint32_t(x[1]);
		}
		if (tid == 0) s_vbase[tot[0]] = uint32_t(tot[1]);
		__syncthreads();
		// the chunk's vertices, copied by the whole CTA
		if (fits)
			for (uint32_t t = tid; t < uint32_t(tot[1]); t += blockDim.x)
			{
				const uint32_t j = find_segment(s_vbase, uint32_t(tot[0]), t);
				a.vertices[num_vertices + t] = a.cands[s_vcand[j]].v[t - s_vbase[j]];
			}
		__syncthreads();
		num_draws += tot[0];
		num_vertices += tot[1];
		num_rows += tot[2];
	}
	__syncthreads();
	if (tid == 0)
	{
		SwViewCounts k;
		const bool over = num_surfaces > a.cap_surfaces || total_texels > a.cap_texels || num_draws > a.cap_draws ||
						  num_vertices > a.cap_vertices || num_rows > a.cap_rows || num_rows > 0xFFFFFFFFull;
		if (s_error || over)
		{
			// Nothing downstream runs on an incomplete frame; the host reports the error.
			k.num_surfaces = k.num_draws = k.num_vertices = 0;
			k.total_texels = k.num_rows = 0;
			k.error = 1;
		}
		else
		{
			k.num_surfaces = uint32_t(num_surfaces);
			k.num_draws = uint32_t(num_draws);
			k.num_vertices = uint32_t(num_vertices);
			k.error = 0;
			k.total_texels = total_texels;
			k.num_rows = num_rows;
		}
		*a.counts = k;
	}
}

} // namespace

int launch_prep(const PrepArgs& args, cudaStream_t stream)
{
	if (args.cap_candidates > 0)
	{
		prep_polygons_kernel<<<(args.cap_candidates + PREP_WARPS - 1) / PREP_WARPS, PREP_WARPS * 32, 0, stream>>>(args);
		launch_dependent(prep_compact_kernel, dim3(1), dim3(COMPACT_THREADS), 0, stream, args);
	}
	else
		prep_compact_kernel<<<1, COMPACT_THREADS, 0, stream>>>(args);
	return int(cudaGetLastError());
}

} // namespace swgpu
