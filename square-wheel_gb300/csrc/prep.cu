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
#include <cstddef>

#include "sw_kernels.cuh"
#include "warp_prep.cuh"

namespace swgpu
{
namespace
{

using swhost::Mat4;
using swhost::Vec2;
using swhost::Vec3;
using swhost::Vec4;

constexpr int PREP_PAIRS = 4;         // per-candidate kernel: two warps per polygon, 4 polygons per CTA
constexpr int COMPACT_THREADS = 1024; // compaction: one CTA

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

// Exclusive prefix sums of N values over the CTA (THREADS threads); `total` gets the sums.
template <int THREADS, int N>
__device__ inline void block_scan_exclusive(uint64_t (&x)[N], uint64_t (&total)[N])
{
	__shared__ uint64_t s_warp[THREADS / 32][N];
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
			uint64_t w = lane < uint32_t(THREADS / 32) ? s_warp[lane][i] : 0ull;
			for (int o = 1; o < 32; o <<= 1)
			{
				const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, w, o);
				if (lane >= uint32_t(o)) w += t;
			}
			if (lane < uint32_t(THREADS / 32)) s_warp[lane][i] = w; // inclusive over warps
		}
	__syncthreads();
	for (int i = 0; i < N; ++i)
	{
		const uint64_t before = warp > 0 ? s_warp[warp - 1][i] : 0ull;
		x[i] = before + inc[i] - x[i];
		total[i] = s_warp[THREADS / 32 - 1][i];
	}
	__syncthreads(); // s_warp is reused by the next call
}

constexpr uint32_t PREP_SMEM_LEAFS = 512; // leaf table staged per CTA up to this many leafs

// What the surface warp of a candidate hands its draw warp (shared memory, one named barrier).
struct SurfaceHandoff
{
	swhost::SurfacePrep sp;
	uint32_t state; // 1: the polygon has a surface
};

// Two warps per candidate polygon: the surface warp runs prepare_polygon_surface and the descriptor
// half of build_polygons_surfaces; the draw warp runs draw_polygon's clipping against the leaf's draw
// bounds at the same time, then takes the surface's equations from the surface warp (named barrier) for
// the interpolation mode and the draw command.
// One candidate polygon on a warp pair (the kernel's body; returns early for hidden polygons).
__device__ void prep_pair(const PrepArgs& a, const PrepFrame& frame, uint32_t num_candidates, uint32_t num_leafs,
	const uint32_t* cand_base, WarpClipBuf* s_buf, SurfaceHandoff* s_hand)
{
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	const uint32_t pair = warp >> 1, role = warp & 1u; // role 0: surface, 1: draw
	const uint32_t c = blockIdx.x * PREP_PAIRS + pair;
	if (c >= num_candidates) return;
	WarpClipBuf& buf = s_buf[warp];
	SurfaceHandoff& hand = s_hand[pair];
	const uint32_t li = find_segment(cand_base, num_leafs, c);
	const SwViewLeaf& leaf = a.leafs[li];
	const uint32_t pi = leaf.first_polygon + (c - cand_base[li]);
	const SwMapPolygon& p = a.polygons[pi];
	PrepCand& out = a.cands[c];
	PrepKey& key = a.keys[c];

	// both warps: back-face and material test, the transformed vertices (one per lane)
	const Mat4 planes_matrix = load_mat4(frame.planes);
	const Vec4 plane_transformed = planes_matrix * swhost::extend(swhost::poly_vec3(p.plane), -p.plane[3]);
	// the material's state this frame: its current animation frame's texture, shift, flags, blending and
	// emissive layer (get_material / get_texture / get_emissive_texture through the mapping table)
	const bool animated = p.texture < frame.num_material_frames;
	const SwMaterialFrame* mf = animated ? a.material_frames + p.texture : nullptr;
	const uint32_t flags = animated ? mf->flags : p.flags;
	if (plane_transformed.w <= 0.0f || !(flags & SW_POLY_DRAW))
	{
		if (role == 1 && lane == 0) key = PrepKey{0ull, 0u, 0u, 0u, 0};
		return; // both warps leave before the handoff
	}
	const Mat4 view = load_mat4(frame.view);
	const uint32_t nv = p.num_vertices < MAXV ? p.num_vertices : MAXV;
	const Vec3* mv = reinterpret_cast<const Vec3*>(a.map_vertices);
	const Vec3 vt = lane < nv ? swhost::view_transform(view, mv[p.first_vertex + lane]) : swhost::v3(0.0f, 0.0f, 1.0f);
	// DepthEquation::from_transformed_plane_equation, equations.rs:23-31
	const float pw = -plane_transformed.w;
	const swhost::DepthEquation de{plane_transformed.x / pw, plane_transformed.y / pw, plane_transformed.z / pw};
	const uint32_t bar_id = 1u + pair;

	if (role == 0)
	{
		// ---- surface warp: prepare_polygon_surface (partial_renderer.rs:1464-1638) ----
		// lights of the leaf (first 32) and the polygon's texture mips, one per lane, loaded ahead
		const uint32_t leaf_first_light = leaf.first_light, leaf_num_lights = leaf.num_lights;
		const uint32_t my_light = lane < leaf_num_lights ? uint32_t(a.leaf_lights[leaf_first_light + lane]) : 0u;
		const SwLight light0 = a.lights[lane < leaf_num_lights ? my_light : 0u];
		const uint32_t emissive_texture = animated ? mf->emissive_texture : p.emissive_texture;
		const bool diffuse = (flags & SW_POLY_DIFFUSE_LAYER) != 0, emissive = emissive_texture != SW_NO_EMISSIVE;
		const uint32_t texture = animated ? mf->texture : p.texture;
		SwTextureMip tex_mip{};
		SwEmissiveMip em_mip{};
		if (lane < swhost::PREP_NUM_MIPS)
		{
			if (diffuse) tex_mip = a.texture_mips[texture * swhost::PREP_NUM_MIPS + lane];
			if (emissive) em_mip = a.emissive_mips[emissive_texture * swhost::PREP_NUM_MIPS + lane];
		}
		Vec3 planes[8];
		load_planes(leaf.clip_planes, planes);
		Vec2 q;
		const uint32_t count = warp_project_and_clip(planes, vt, nv, q, buf);
		if (count < 3 || (flags & SW_POLY_SKY)) // hidden, or sky (its bounds are the host's)
		{
			if (lane == 0) hand.state = 0;
			__syncwarp();
			named_barrier(bar_id, 64);
			return;
		}
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
		swhost::SurfacePrep sp;
		for (int i = 0; i < 2; ++i)
		{
			sp.tc.d_tc_dx[i] = te.d_tc_dx[i] * mip_scale;
			sp.tc.d_tc_dy[i] = te.d_tc_dy[i] * mip_scale;
			sp.tc.k[i] = te.k[i] * mip_scale;
		}
		// surface rectangle: tc bounds over the clipped polygon, lightmap-aligned clamp
		{
			const float inf = float(1 << 29);
			const float max_z = float(1 << 16);
			const float inv_z = fmaxf(de.sample(q), 1.0f / max_z);
			const float z = 1.0f / inv_z;
			for (int i = 0; i < 2; ++i)
			{
				const float tc = z * (sp.tc.d_tc_dx[i] * q.x + sp.tc.d_tc_dy[i] * q.y + sp.tc.k[i]);
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
		}
		sp.depth = de;
		sp.mip = mip;
		for (int i = 0; i < 2; ++i)
		{
			const float tmf = float(sp.tc_min[i]);
			sp.tc.d_tc_dx[i] -= tmf * de.d_inv_z_dx;
			sp.tc.d_tc_dy[i] -= tmf * de.d_inv_z_dy;
			sp.tc.k[i] -= tmf * de.k;
		}
		if (lane == 0)
		{
			hand.sp = sp;
			hand.state = 1;
		}
		__syncwarp();
		named_barrier(bar_id, 64); // the draw warp may take the equations

		// build_polygons_surfaces: descriptor, the leaf's lights that reach the polygon (in order, up to 6)
		// and the surface build's record (its texel offset is the compaction's)
		SwSurfaceDesc d;
		swhost::make_surface_desc(p, sp, 0, a.directional != 0, a.simple_lightmaps != 0, mf, d);
		if (diffuse)
			for (uint32_t base = 0; base < leaf_num_lights && d.num_lights < SW_MAX_POLYGON_LIGHTS; base += 32)
			{
				const uint32_t k = base + lane;
				bool hit = false;
				uint32_t light = my_light;
				if (k < leaf_num_lights)
				{
					if (base > 0) light = a.leaf_lights[leaf_first_light + k];
					hit = swhost::polygon_is_affected_by_light(p, base > 0 ? a.lights[light] : light0,
						light < a.num_shadows ? a.shadows + light : nullptr);
				}
				uint32_t mask = __ballot_sync(FULL_MASK, hit);
				while (mask && d.num_lights < SW_MAX_POLYGON_LIGHTS)
				{
					const uint32_t b = uint32_t(__ffs(mask) - 1);
					mask &= mask - 1;
					d.lights[d.num_lights++] = uint16_t(__shfl_sync(FULL_MASK, light, int(b)));
				}
			}
		SwTextureMip tm;
		tm.offset = __shfl_sync(FULL_MASK, (unsigned long long)tex_mip.offset, int(mip));
		tm.width = __shfl_sync(FULL_MASK, tex_mip.width, int(mip));
		tm.height = __shfl_sync(FULL_MASK, tex_mip.height, int(mip));
		tm.flags = __shfl_sync(FULL_MASK, tex_mip.flags, int(mip));
		tm.reserved = 0;
		SwEmissiveMip em;
		em.offset = __shfl_sync(FULL_MASK, (unsigned long long)em_mip.offset, int(mip));
		em.width = __shfl_sync(FULL_MASK, em_mip.width, int(mip));
		em.height = __shfl_sync(FULL_MASK, em_mip.height, int(mip));
		if (lane == 0)
		{
			out.desc = d;
			make_surface_gpu(d, diffuse ? &tm : nullptr, emissive ? &em : nullptr, out.sgpu);
		}
		return;
	}

	// ---- draw warp: draw_leaf -> draw_polygon (partial_renderer.rs:4011-4142) ----
	uint32_t n = 0;
	Vec2 v = swhost::v2(0.0f, 0.0f);
	SwVertex16 fv{0, 0};
	int min_i = -1, max_i = -1;
	float max_inv_z = -1e24f, min_x = 1e24f, max_x = -1e24f;
	int32_t row_y0 = 0;
	uint32_t row_n = 0;
	if (leaf.draw_order != SW_LEAF_NOT_DRAWN && p.num_vertices >= 3)
	{
		Vec3 draw_planes[8];
		load_planes(leaf.draw_clip_planes, draw_planes);
		n = warp_project_and_clip(draw_planes, vt, nv, v, buf);
		if (n >= 3)
		{
			const bool in_draw = lane < n;
			const float inv_z = de.sample(v);
			int unused;
			warp_first_min(inv_z, in_draw, 1e24f, &min_i);
			max_inv_z = warp_first_max(inv_z, in_draw, -1e24f, &max_i);
			min_x = warp_first_min(v.x, in_draw, 1e24f, &unused);
			max_x = warp_first_max(v.x, in_draw, -1e24f, &unused);
			fv = SwVertex16{swhost::as_i32(v.x * 65536.0f), swhost::as_i32(v.y * 65536.0f)};
			if (in_draw) out.v[lane] = fv;
			// draw_row_range: [round(min y), round(max y)) clipped to the frame
			const int32_t y_lo = __reduce_min_sync(FULL_MASK, in_draw ? fv.y : INT32_MAX);
			const int32_t y_hi = __reduce_max_sync(FULL_MASK, in_draw ? fv.y : INT32_MIN);
			const int32_t r0 = int32_t(uint32_t(y_lo) + 0x8000u) >> 16, r1 = int32_t(uint32_t(y_hi) + 0x8000u) >> 16;
			const int32_t ra = r0 > 0 ? r0 : 0, rb = r1 < a.height ? r1 : a.height;
			row_y0 = ra;
			row_n = rb > ra ? uint32_t(rb - ra) : 0u;
		}
	}
	named_barrier(bar_id, 64); // the surface warp's result is in shared memory
	const uint32_t state = hand.state;
	if (!state)
	{
		if (lane == 0) key = PrepKey{0ull, 0u, 0u, 0u, 0};
		return;
	}
	const swhost::SurfacePrep sp = hand.sp;
	uint32_t draw_count = 0;
	if (n >= 3)
	{
		const Vec2 p_min = shfl(v, min_i < 0 ? 0 : min_i), p_max = shfl(v, max_i < 0 ? 0 : max_i);
		SwDrawCmd dc = SwDrawCmd{};
		dc.vertex_count = n;
		dc.blend = animated ? mf->blending_mode : p.blending_mode;
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
		draw_count = n;
	}
	if (lane == 0) key = PrepKey{uint64_t(sp.size[0]) * sp.size[1], 1u, draw_count, draw_count ? row_n : 0u, row_y0};
}

constexpr uint32_t PREP_THREADS = PREP_PAIRS * 64;
constexpr uint32_t FAST_MAX = 2048; // candidates (and draw slots) the compactions keep in registers

// Record copies of the compactions in 8-byte chunks spread over the whole CTA (one chunk per thread and
// step) instead of one thread per record: one round trip for all of them.
constexpr uint32_t DESC_CHUNKS = sizeof(SwSurfaceDesc) / 8, SGPU_CHUNKS = sizeof(SurfaceGpu) / 8;
constexpr uint32_t DRAW_CHUNKS = sizeof(SwDrawCmd) / 8;
static_assert(sizeof(SwSurfaceDesc) % 8 == 0 && sizeof(SurfaceGpu) % 8 == 0 && sizeof(SwDrawCmd) % 8 == 0, "8-byte chunks");
static_assert(offsetof(SwSurfaceDesc, out_offset) % 8 == 0 && offsetof(SurfaceGpu, out_offset) % 8 == 0 &&
				  offsetof(SwDrawCmd, tex_offset) % 8 == 0 && offsetof(SwDrawCmd, first_vertex) == 0,
	"patched fields");

// Surfaces in allocation order: descriptors, the surface build's records, its texel prefix sums and the
// counts it reads (one CTA of THREADS threads).
template <uint32_t THREADS>
__device__ void compact_surfaces(const PrepArgs& a, uint32_t num_candidates)
{
	constexpr uint32_t ITEMS = FAST_MAX / THREADS;
	__shared__ uint32_t s_cand[FAST_MAX]; // surface -> candidate (fast path)
	__shared__ uint64_t s_off[FAST_MAX];  // surface -> texel offset
	__shared__ uint32_t s_error;
	const uint32_t tid = threadIdx.x;
	if (tid == 0) s_error = 0;
	__syncthreads();
	uint64_t num_surfaces = 0, total_texels = 0;
	bool fits = true;
	if (num_candidates <= FAST_MAX)
	{
		// thread t owns candidates ITEMS*t ..: one round trip for the keys, the scan, one for the copies
		PrepKey k[ITEMS];
		for (uint32_t i = 0; i < ITEMS; ++i)
		{
			const uint32_t c = tid * ITEMS + i;
			k[i] = c < num_candidates ? a.keys[c] : PrepKey{0ull, 0u, 0u, 0u, 0};
		}
		uint64_t x[2] = {0ull, 0ull}, tot[2];
		for (uint32_t i = 0; i < ITEMS; ++i)
			if (k[i].state == 1)
			{
				x[0] += 1;
				x[1] += k[i].area;
			}
		block_scan_exclusive<THREADS, 2>(x, tot);
		num_surfaces = tot[0];
		total_texels = tot[1];
		fits = num_surfaces <= a.cap_surfaces && total_texels <= a.cap_texels;
		if (fits)
		{
			for (uint32_t i = 0; i < ITEMS; ++i)
				if (k[i].state == 1)
				{
					s_cand[x[0]] = tid * ITEMS + i;
					s_off[x[0]] = x[1];
					a.work_prefix[x[0]] = x[1];
					x[0] += 1;
					x[1] += k[i].area;
				}
			__syncthreads();
			const uint32_t per = DESC_CHUNKS + SGPU_CHUNKS, chunks = uint32_t(num_surfaces) * per;
			for (uint32_t t = tid; t < chunks; t += THREADS)
			{
				const uint32_t sidx = t / per, q = t - sidx * per;
				const PrepCand& cand = a.cands[s_cand[sidx]];
				if (q < DESC_CHUNKS)
				{
					const uint64_t v = q == offsetof(SwSurfaceDesc, out_offset) / 8
						? s_off[sidx]
						: reinterpret_cast<const uint64_t*>(&cand.desc)[q];
					reinterpret_cast<uint64_t*>(a.descs + sidx)[q] = v;
				}
				else
				{
					const uint32_t r = q - DESC_CHUNKS;
					const uint64_t v = r == offsetof(SurfaceGpu, out_offset) / 8
						? s_off[sidx]
						: reinterpret_cast<const uint64_t*>(&cand.sgpu)[r];
					reinterpret_cast<uint64_t*>(a.surfaces + sidx)[r] = v;
				}
			}
		}
	}
	else
		for (uint32_t base = 0; base < num_candidates; base += THREADS)
		{
			const uint32_t c = base + tid;
			const PrepKey k = c < num_candidates ? a.keys[c] : PrepKey{0ull, 0u, 0u, 0u, 0};
			const bool vis = k.state == 1;
			const uint64_t area = vis ? k.area : 0ull;
			uint64_t x[2] = {vis ? 1ull : 0ull, area}, tot[2];
			block_scan_exclusive<THREADS, 2>(x, tot);
			if (vis)
			{
				const uint64_t s = num_surfaces + x[0], offset = total_texels + x[1];
				if (s < a.cap_surfaces && offset + area <= a.cap_texels)
				{
					SwSurfaceDesc d = a.cands[c].desc;
					SurfaceGpu g = a.cands[c].sgpu;
					d.out_offset = offset;
					g.out_offset = offset;
					a.descs[s] = d;
					a.surfaces[s] = g;
					a.work_prefix[s] = offset;
				}
				else
					atomicOr(&s_error, 1u);
			}
			num_surfaces += tot[0];
			total_texels += tot[1];
		}
	__syncthreads();
	if (tid == 0)
	{
		const bool error = !fits || s_error || num_surfaces > a.cap_surfaces || total_texels > a.cap_texels;
		if (!error) a.work_prefix[num_surfaces] = total_texels;
		a.counts->num_surfaces = error ? 0u : uint32_t(num_surfaces);
		a.counts->total_texels = error ? 0ull : total_texels;
		if (error) atomicOr(&a.counts->error, 1u);
	}
}

// Two warps per candidate polygon: the surface warp runs prepare_polygon_surface and the descriptor
// half of build_polygons_surfaces; the draw warp runs draw_polygon's clipping against the leaf's draw
// bounds at the same time, then takes the surface's equations from the surface warp (named barrier) for
// the interpolation mode and the draw command.
__global__ void __launch_bounds__(PREP_THREADS) prep_polygons_kernel(PrepArgs a)
{
	__shared__ WarpClipBuf s_buf[PREP_PAIRS * 2];
	__shared__ SurfaceHandoff s_hand[PREP_PAIRS];
	__shared__ uint32_t s_base[PREP_SMEM_LEAFS + 1];
	const PrepFrame& frame = *a.frame;
	const uint32_t num_candidates = min(frame.num_candidates, a.cap_candidates), num_leafs = frame.num_leafs;
	if (blockIdx.x == 0 && threadIdx.x == 0) a.counts->error = 0; // the compactions set their bits
	if (blockIdx.x * PREP_PAIRS >= num_candidates) return; // the grid is sized for the capacity
	const bool staged = num_leafs <= PREP_SMEM_LEAFS;
	if (staged)
	{
		for (uint32_t i = threadIdx.x; i <= num_leafs; i += blockDim.x) s_base[i] = __ldg(a.leaf_cand_base + i);
		__syncthreads();
	}
	prep_pair(a, frame, num_candidates, num_leafs, staged ? s_base : a.leaf_cand_base, s_buf, s_hand);
}

// The surface compaction: on the main stream, right before the surface build.
__global__ void __launch_bounds__(COMPACT_THREADS, 1) prep_surfaces_kernel(PrepArgs a)
{
	compact_surfaces<COMPACT_THREADS>(a, min(a.frame->num_candidates, a.cap_candidates));
}

constexpr uint32_t SMEM_LEAFS = 256; // index arrays staged in shared memory up to this many leafs
constexpr uint32_t FAST_ITEMS = FAST_MAX / COMPACT_THREADS; // draw compaction fast path: slots per thread
constexpr uint32_t ERROR_DRAWS = 2u; // SwViewCounts.error bit of the draw compaction (the surfaces' is 1)

struct DrawShared
{
	uint32_t error;
	uint32_t cand_base[SMEM_LEAFS + 1], slot_base[SMEM_LEAFS + 1], draw_leaf[SMEM_LEAFS];
	uint64_t surface_offset[FAST_MAX];             // fast path: per candidate
	uint32_t vcand[FAST_MAX], vbase[FAST_MAX + 1]; // draws' vertex copy list
};

// Candidate of draw slot `slot`: the drawn leafs' polygons in draw order.
__device__ inline uint32_t slot_candidate(const uint32_t* cand_base, const uint32_t* slot_base, const uint32_t* draw_leaf,
	uint32_t num_draw_leafs, uint32_t slot)
{
	const uint32_t j = find_segment(slot_base, num_draw_leafs, slot);
	return cand_base[draw_leaf[j]] + (slot - slot_base[j]);
}

// Draws in submission order: the host's (skybox) first, then the drawn leafs' polygons back to front,
// each with its surface's texel offset (the same scan as compact_surfaces', done again here so
// that this kernel runs on the auxiliary stream beside the surface compaction and build).
__global__ void __launch_bounds__(COMPACT_THREADS, 1) prep_draws_kernel(PrepArgs a)
{
	__shared__ DrawShared sh;
	const uint32_t tid = threadIdx.x;
	if (tid == 0) sh.error = 0;
	const PrepFrame& frame = *a.frame;
	const uint32_t num_leafs = frame.num_leafs, num_candidates = min(frame.num_candidates, a.cap_candidates);
	const uint32_t num_draw_leafs = frame.num_draw_leafs;
	const uint32_t num_host_draws = frame.num_host_draws, num_host_vertices = frame.num_host_vertices;
	const uint64_t num_host_rows = frame.num_host_rows;
	const bool staged = num_leafs <= SMEM_LEAFS;
	if (staged)
	{
		for (uint32_t i = tid; i <= num_leafs; i += blockDim.x) sh.cand_base[i] = __ldg(a.leaf_cand_base + i);
		for (uint32_t i = tid; i <= num_draw_leafs; i += blockDim.x) sh.slot_base[i] = __ldg(a.draw_slot_base + i);
		for (uint32_t i = tid; i < num_draw_leafs; i += blockDim.x) sh.draw_leaf[i] = __ldg(a.draw_leaf + i);
	}
	const uint32_t* cand_base = staged ? sh.cand_base : a.leaf_cand_base;
	const uint32_t* slot_base = staged ? sh.slot_base : a.draw_slot_base;
	const uint32_t* draw_leaf = staged ? sh.draw_leaf : a.draw_leaf;
	for (uint32_t i = tid; i < num_host_draws && i < a.cap_draws; i += blockDim.x)
	{
		a.draws[i] = a.host_draws[i];
		a.draw_rows[i] = a.host_rows[i];
	}
	for (uint32_t i = tid; i < num_host_vertices && i < a.cap_vertices; i += blockDim.x) a.vertices[i] = a.host_vertices[i];
	__syncthreads();
	const uint32_t slots = num_draw_leafs ? slot_base[num_draw_leafs] : 0u;
	uint64_t num_draws = num_host_draws, num_vertices = num_host_vertices, num_rows = num_host_rows;
	bool error = false;

	if (num_candidates <= FAST_MAX && slots <= FAST_MAX)
	{
		// one round trip for every key, the two scans, one round trip for every copy
		PrepKey sk[FAST_ITEMS], dk[FAST_ITEMS];
		uint32_t dc[FAST_ITEMS];
		for (uint32_t i = 0; i < FAST_ITEMS; ++i)
		{
			const uint32_t c = tid * FAST_ITEMS + i, slot = tid * FAST_ITEMS + i;
			dc[i] = slot < slots ? slot_candidate(cand_base, slot_base, draw_leaf, num_draw_leafs, slot) : 0u;
			sk[i] = c < num_candidates ? a.keys[c] : PrepKey{0ull, 0u, 0u, 0u, 0};
			dk[i] = slot < slots ? a.keys[dc[i]] : PrepKey{0ull, 0u, 0u, 0u, 0};
		}
		// the surfaces' texel offsets (allocation order)
		uint64_t off[1] = {0ull}, off_tot[1];
		for (uint32_t i = 0; i < FAST_ITEMS; ++i)
			if (sk[i].state == 1) off[0] += sk[i].area;
		block_scan_exclusive<COMPACT_THREADS, 1>(off, off_tot);
		const uint64_t total_texels = off_tot[0];
		for (uint32_t i = 0; i < FAST_ITEMS; ++i)
			if (sk[i].state == 1)
			{
				sh.surface_offset[tid * FAST_ITEMS + i] = off[0];
				off[0] += sk[i].area;
			}
		uint64_t y[3] = {0ull, 0ull, 0ull}, tot[3];
		for (uint32_t i = 0; i < FAST_ITEMS; ++i)
			if (dk[i].state == 1 && dk[i].draw_count >= 3)
			{
				y[0] += 1;
				y[1] += dk[i].draw_count;
				y[2] += dk[i].row_n;
			}
		block_scan_exclusive<COMPACT_THREADS, 3>(y, tot); // (its barriers also publish the surface offsets)
		num_draws += tot[0];
		num_vertices += tot[1];
		num_rows += tot[2];
		const bool fits = total_texels <= a.cap_texels && num_draws <= a.cap_draws && num_vertices <= a.cap_vertices &&
						  num_rows <= a.cap_rows;
		error = !fits;
		for (uint32_t i = 0; i < FAST_ITEMS; ++i)
			if (dk[i].state == 1 && dk[i].draw_count >= 3)
			{
				if (fits)
					a.draw_rows[num_host_draws + y[0]] = DrawRows{uint32_t(num_host_rows + y[2]), dk[i].row_y0, dk[i].row_n, 0u};
				sh.vcand[y[0]] = dc[i];
				sh.vbase[y[0]] = uint32_t(y[1]);
				y[0] += 1;
				y[1] += dk[i].draw_count;
				y[2] += dk[i].row_n;
			}
		if (tid == 0) sh.vbase[tot[0]] = uint32_t(tot[1]);
		__syncthreads();
		if (fits)
		{
			// draw records (first vertex and texture offset patched) and vertices, chunk by chunk
			const uint32_t ndraws = uint32_t(tot[0]), draw_chunks = ndraws * DRAW_CHUNKS;
			for (uint32_t t = tid; t < draw_chunks; t += blockDim.x)
			{
				const uint32_t j = t / DRAW_CHUNKS, q = t - j * DRAW_CHUNKS;
				const uint32_t c = sh.vcand[j];
				uint64_t v = reinterpret_cast<const uint64_t*>(&a.cands[c].draw)[q];
				if (q == 0) v = (v & 0xFFFFFFFF00000000ull) | uint64_t(num_host_vertices + sh.vbase[j]);
				if (q == offsetof(SwDrawCmd, tex_offset) / 8) v = sh.surface_offset[c];
				reinterpret_cast<uint64_t*>(a.draws + num_host_draws + j)[q] = v;
			}
			for (uint32_t t = tid; t < uint32_t(tot[1]); t += blockDim.x)
			{
				const uint32_t j = find_segment(sh.vbase, uint32_t(tot[0]), t);
				a.vertices[num_host_vertices + t] = a.cands[sh.vcand[j]].v[t - sh.vbase[j]];
			}
		}
	}
	else
	{
		// surface offsets of every candidate, chunk by chunk (kept with the candidates)
		uint64_t total_texels = 0;
		for (uint32_t base = 0; base < num_candidates; base += blockDim.x)
		{
			const uint32_t c = base + tid;
			const PrepKey k = c < num_candidates ? a.keys[c] : PrepKey{0ull, 0u, 0u, 0u, 0};
			const bool vis = k.state == 1;
			uint64_t x[1] = {vis ? k.area : 0ull}, tot[1];
			block_scan_exclusive<COMPACT_THREADS, 1>(x, tot);
			if (vis) a.cands[c].surface_offset = total_texels + x[0];
			total_texels += tot[0];
		}
		error = total_texels > a.cap_texels;
		__syncthreads(); // the offsets are visible to the CTA
		for (uint32_t base = 0; base < slots && !error; base += blockDim.x)
		{
			const uint32_t slot = base + tid;
			PrepKey k{0ull, 0u, 0u, 0u, 0};
			uint32_t c = 0;
			if (slot < slots)
			{
				c = slot_candidate(cand_base, slot_base, draw_leaf, num_draw_leafs, slot);
				k = a.keys[c];
			}
			const bool emit = k.state == 1 && k.draw_count >= 3;
			const uint32_t nv = emit ? k.draw_count : 0u;
			const uint32_t nr = emit ? k.row_n : 0u;
			uint64_t x[3] = {emit ? 1ull : 0ull, nv, nr}, tot[3];
			block_scan_exclusive<COMPACT_THREADS, 3>(x, tot);
			const bool fits = num_draws + tot[0] <= a.cap_draws && num_vertices + tot[1] <= a.cap_vertices &&
							  num_rows + tot[2] <= a.cap_rows;
			if (emit)
			{
				if (fits)
				{
					SwDrawCmd d = a.cands[c].draw;
					d.first_vertex = uint32_t(num_vertices + x[1]);
					d.tex_offset = a.cands[c].surface_offset;
					a.draws[num_draws + x[0]] = d;
					a.draw_rows[num_draws + x[0]] = DrawRows{uint32_t(num_rows + x[2]), k.row_y0, nr, 0u};
				}
				sh.vcand[x[0]] = c;
				sh.vbase[x[0]] = uint32_t(x[1]);
			}
			if (tid == 0) sh.vbase[tot[0]] = uint32_t(tot[1]);
			__syncthreads();
			if (fits)
				for (uint32_t t = tid; t < uint32_t(tot[1]); t += blockDim.x)
				{
					const uint32_t j = find_segment(sh.vbase, uint32_t(tot[0]), t);
					a.vertices[num_vertices + t] = a.cands[sh.vcand[j]].v[t - sh.vbase[j]];
				}
			__syncthreads();
			num_draws += tot[0];
			num_vertices += tot[1];
			num_rows += tot[2];
			error = error || !fits;
		}
	}
	__syncthreads();
	if (tid == 0)
	{
		error = error || num_draws > a.cap_draws || num_vertices > a.cap_vertices || num_rows > a.cap_rows ||
				num_rows > 0xFFFFFFFFull;
		a.counts->num_draws = error ? 0u : uint32_t(num_draws);
		a.counts->num_vertices = error ? 0u : uint32_t(num_vertices);
		a.counts->num_rows = error ? 0ull : num_rows;
		if (error) atomicOr(&a.counts->error, ERROR_DRAWS);
	}
}

} // namespace

int launch_prep(const PrepArgs& args, cudaStream_t stream, cudaStream_t aux, cudaEvent_t candidates_done)
{
	if (args.cap_candidates == 0) return int(cudaErrorInvalidValue);
	prep_polygons_kernel<<<(args.cap_candidates + PREP_PAIRS - 1) / PREP_PAIRS, PREP_THREADS, 0, stream>>>(args);
	cudaError_t e = cudaEventRecord(candidates_done, stream);
	if (e != cudaSuccess) return int(e);
	prep_surfaces_kernel<<<1, COMPACT_THREADS, 0, stream>>>(args);
	if ((e = cudaStreamWaitEvent(aux, candidates_done, 0)) != cudaSuccess) return int(e);
	prep_draws_kernel<<<1, COMPACT_THREADS, 0, aux>>>(args);
	return int(cudaGetLastError());
}

} // namespace swgpu
