// Seeded synthetic scene generator (see scene.h). Load-time work, not on the timed path.
#include "scene.h"
#include "sqwm.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>

namespace swhost
{

namespace
{

// Deterministic RNG (splitmix64): identical sequences on every platform.
struct Rng
{
	uint64_t s;
	explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
	uint64_t next()
	{
		uint64_t z = (s += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		return z ^ (z >> 31);
	}
	float uniform() { return float(next() >> 40) * (1.0f / 16777216.0f); } // [0, 1)
	float uniform(float a, float b) { return a + (b - a) * uniform(); }
	uint32_t below(uint32_t n) { return n ? uint32_t(next() % n) : 0u; }
};

constexpr float CELL_PITCH = 1280.0f;   // cell slot 1024 + 256 gap
constexpr float CELL_SLOT = 1024.0f;
constexpr float CORRIDOR_HALF = 64.0f;  // corridors are 128 wide and 128 high
constexpr float CORRIDOR_HEIGHT = 128.0f;

struct Room
{
	float x0, x1, y0, y1, h;
	float cx, cy; // corridor centre lines (cell centre lines)
	uint32_t mat_wall, mat_floor, mat_ceiling;
	uint32_t ceiling_first = 0, ceiling_end = 0; // the ceiling's polygons
	uint32_t leaf = 0;
	int32_t tc_shift[2];
	std::vector<Vec3> lights;
	std::vector<Vec3> light_colors;
};

float snap16(float v) { return std::floor(v / 16.0f) * 16.0f; }

// ---- textures -------------------------------------------------------------------------------

uint32_t pack_normal_roughness(Vec3 n, float roughness)
{
	// PackedNormalRoughness::pack with the generic pack_f32x4_into_bytes (truncating), textures.rs:33-39
	const float v[4] = {n.x, n.y, n.z, roughness};
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i)
	{
		float s = std::fmin(std::fmax(v[i] * 127.0f, -127.0f), 127.0f);
		r |= (uint32_t(int32_t(s)) & 0xFFu) << (i * 8);
	}
	return r;
}

void unpack_normal_roughness(uint32_t p, Vec3& n, float& r)
{
	float o[4];
	for (int i = 0; i < 4; ++i) o[i] = float(int32_t(p << (24 - i * 8)) >> 24) * (1.0f / 127.0f);
	n = v3(o[0], o[1], o[2]);
	r = o[3];
}

uint32_t average4(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
	// Color32::get_average_4, src/common/color.rs:51-71
	uint32_t s[4] = {0, 0, 0, 0};
	for (uint32_t x : {a, b, c, d})
	{
		s[0] += x & 0xFFu;
		s[1] += x & 0xFF00u;
		s[2] += x & 0xFF0000u;
		s[3] += (x & 0xFF000000u) >> 2;
	}
	return (s[0] >> 2) | ((s[1] >> 2) & 0xFF00u) | ((s[2] >> 2) & 0xFF0000u) | (s[3] & 0xFF000000u);
}

// build_texture_mip, src/square_wheel/textures.rs:309-362
void build_mip(const std::vector<uint64_t>& src, uint32_t sw, uint32_t sh, std::vector<uint64_t>& dst)
{
	const uint32_t w = sw >> 1, h = sh >> 1;
	dst.assign(size_t(w) * h, 0);
	for (uint32_t y = 0; y < h; ++y)
		for (uint32_t x = 0; x < w; ++x)
		{
			const uint64_t p00 = src[(2 * y) * sw + 2 * x], p01 = src[(2 * y + 1) * sw + 2 * x];
			const uint64_t p10 = src[(2 * y) * sw + 2 * x + 1], p11 = src[(2 * y + 1) * sw + 2 * x + 1];
			const uint32_t diffuse = average4(uint32_t(p00), uint32_t(p01), uint32_t(p10), uint32_t(p11));
			Vec3 n[4];
			float r[4];
			const uint64_t ps[4] = {p00, p01, p10, p11};
			for (int i = 0; i < 4; ++i) unpack_normal_roughness(uint32_t(ps[i] >> 32), n[i], r[i]);
			const Vec3 sum = n[0] + n[1] + n[2] + n[3];
			const float len = std::fmax(magnitude(sum), 0.000001f);
			const Vec3 nn = sum / len;
			const float deviation = (1.0f - len * 0.25f) / (1.0f - 0.5f);
			const float rs = r[0] + r[1] + r[2] + r[3];
			const float rough = std::fmin(std::fmax(rs * 0.25f + deviation, 1.0f / 126.0f), 1.0f);
			dst[size_t(y) * w + x] = uint64_t(diffuse) | (uint64_t(pack_normal_roughness(nn, rough)) << 32);
		}
}

std::vector<float> value_noise(Rng& rng, uint32_t size, uint32_t cells)
{
	std::vector<float> g((cells + 1) * (cells + 1));
	for (float& v : g) v = rng.uniform();
	for (uint32_t i = 0; i <= cells; ++i) g[cells * (cells + 1) + i] = g[i]; // tileable
	for (uint32_t j = 0; j <= cells; ++j) g[j * (cells + 1) + cells] = g[j * (cells + 1)];
	std::vector<float> out(size_t(size) * size);
	for (uint32_t y = 0; y < size; ++y)
		for (uint32_t x = 0; x < size; ++x)
		{
			float fx = float(x) * cells / size, fy = float(y) * cells / size;
			uint32_t ix = uint32_t(fx), iy = uint32_t(fy);
			float tx = fx - ix, ty = fy - iy;
			tx = tx * tx * (3 - 2 * tx);
			ty = ty * ty * (3 - 2 * ty);
			const float a = g[iy * (cells + 1) + ix], b = g[iy * (cells + 1) + ix + 1];
			const float c = g[(iy + 1) * (cells + 1) + ix], d = g[(iy + 1) * (cells + 1) + ix + 1];
			out[size_t(y) * size + x] = (a * (1 - tx) + b * tx) * (1 - ty) + (c * (1 - tx) + d * tx) * ty;
		}
	return out;
}

void make_material_texture(Rng& rng, uint32_t size, bool normal_map, float roughness, bool metal, Scene& sc)
{
	const std::vector<float> n1 = value_noise(rng, size, 8), n2 = value_noise(rng, size, 32);
	const float base[3] = {rng.uniform(0.3f, 0.9f), rng.uniform(0.3f, 0.9f), rng.uniform(0.3f, 0.9f)};
	const uint32_t check = std::max(size / 8, 1u);
	std::vector<float> height(size_t(size) * size);
	std::vector<uint64_t> level(size_t(size) * size);
	for (uint32_t y = 0; y < size; ++y)
		for (uint32_t x = 0; x < size; ++x)
		{
			const size_t i = size_t(y) * size + x;
			const float checker = float(((x / check) + (y / check)) & 1u);
			const float lum = 0.55f + 0.3f * n1[i] + 0.15f * n2[i] - 0.12f * checker;
			uint32_t c[3];
			for (int k = 0; k < 3; ++k) c[k] = uint32_t(std::fmin(std::fmax(lum * base[k] * 255.0f, 0.0f), 255.0f));
			level[i] = uint64_t((255u << 24) | (c[0] << 16) | (c[1] << 8) | c[2]);
			height[i] = n1[i] * 2.0f + n2[i] * 0.5f + checker * 0.5f;
		}
	for (uint32_t y = 0; y < size; ++y)
		for (uint32_t x = 0; x < size; ++x)
		{
			const size_t i = size_t(y) * size + x;
			Vec3 n = v3(0, 0, 1);
			if (normal_map)
			{
				const float gx = (height[y * size + (x + 1) % size] - height[y * size + (x + size - 1) % size]) * (size / 64.0f);
				const float gy = (height[((y + 1) % size) * size + x] - height[((y + size - 1) % size) * size + x]) * (size / 64.0f);
				n = v3(-gx, -gy, 1.0f);
				n = n / magnitude(n);
			}
			float r = 1.0f;
			if (roughness < 1.0f) r = std::fmin(std::fmax(roughness * (0.8f + 0.2f * n2[i]), 1.0f / 126.0f), 1.0f);
			level[i] |= uint64_t(pack_normal_roughness(n, r)) << 32;
		}
	uint32_t flags = 0;
	if (normal_map) flags |= SW_TEX_HAS_NORMAL_MAP;
	if (roughness < 1.0f) flags |= SW_TEX_HAS_NON_ONE_ROUGHNESS;
	if (metal) flags |= SW_TEX_IS_METAL;
	uint32_t w = size, h = size;
	for (uint32_t m = 0; m < NUM_MIPS; ++m)
	{
		SwTextureMip tm;
		tm.offset = sc.texels.size();
		tm.width = w;
		tm.height = h;
		tm.flags = flags;
		tm.reserved = 0;
		sc.texture_mips.push_back(tm);
		sc.texels.insert(sc.texels.end(), level.begin(), level.end());
		if (m + 1 < NUM_MIPS)
		{
			std::vector<uint64_t> next;
			build_mip(level, w, h, next);
			level.swap(next);
			w >>= 1;
			h >>= 1;
		}
	}
}

// ---- skybox ----------------------------------------------------------------------------------

// One procedural RGBA8 side image (the stand-in for the skybox image files): a vertical gradient from
// horizon haze to zenith blue on the four walls, the zenith colour on top, dark ground at the bottom,
// with value-noise clouds. Raw Color32 values (A << 24 | R << 16 | G << 8 | B).
std::vector<uint32_t> make_sky_image(Rng& rng, uint32_t size, uint32_t side)
{
	const std::vector<float> clouds = value_noise(rng, size, 8), detail = value_noise(rng, size, 32);
	std::vector<uint32_t> img(size_t(size) * size);
	for (uint32_t y = 0; y < size; ++y)
		for (uint32_t x = 0; x < size; ++x)
		{
			const size_t i = size_t(y) * size + x;
			// walls (sides 0..3): v runs from the zenith (y = 0) to the horizon; top (5) and bottom (4) flat
			const float t = side < 4 ? float(y) / float(size) : side == 5 ? 0.0f : 1.2f;
			float rgb[3] = {40.0f + 150.0f * t, 90.0f + 120.0f * t, 200.0f + 40.0f * std::fmin(t, 1.0f)};
			if (side == 4)
				for (float& c : rgb) c *= 0.3f;
			const float cloud = std::fmax(clouds[i] * 1.6f - 0.7f + 0.2f * detail[i], 0.0f);
			for (float& c : rgb) c = c + (250.0f - c) * std::fmin(cloud, 1.0f);
			uint32_t c8[3];
			for (int k = 0; k < 3; ++k) c8[k] = uint32_t(std::fmin(std::fmax(rgb[k], 0.0f), 255.0f));
			img[i] = (255u << 24) | (c8[0] << 16) | (c8[1] << 8) | c8[2];
		}
	return img;
}

// Lane helpers of the generic ColorVecI (src/square_wheel/fast_math.rs:600-720): lanes b, g, r, a.
struct Lanes
{
	int32_t v[4];
};
Lanes lanes32(uint32_t c)
{
	Lanes l;
	for (int i = 0; i < 4; ++i) l.v[i] = int32_t((c >> (i * 8)) & 0xFFu);
	return l;
}
Lanes lanes64(uint64_t c)
{
	Lanes l;
	for (int i = 0; i < 4; ++i) l.v[i] = int32_t((c >> (i * 16)) & 0xFFFFu);
	return l;
}
// into_color32 / into_color64: lane as unsigned, min(255) / min(65535)
uint32_t from_lanes32(const Lanes& l)
{
	uint32_t r = 0;
	for (int i = 0; i < 4; ++i) r |= std::min(uint32_t(l.v[i]), 255u) << (i * 8);
	return r;
}
uint64_t from_lanes64(const Lanes& l)
{
	uint64_t r = 0;
	for (int i = 0; i < 4; ++i) r |= uint64_t(std::min(uint32_t(l.v[i]), 65535u)) << (i * 16);
	return r;
}

// make_skybox_side_texture{,64} (textures.rs:183-229) + make_skybox_side_texture_mips (:231-290) of one
// side image, appended to the scene's skybox arrays. The 64-bit image of an 8-bit file holds the 8-bit
// values as 16-bit lanes (image::load64, src/common/image.rs:50-58).
void add_skybox_side(const std::vector<uint32_t>& img, uint32_t size, float brightness, uint32_t side, Scene& sc)
{
	const int32_t bi = int32_t(brightness * 256.0f); // (brightness * SCALE) as i32
	std::vector<uint32_t> l32(img.size());
	std::vector<uint64_t> l64(img.size());
	for (size_t i = 0; i < img.size(); ++i)
	{
		Lanes c = lanes32(img[i]);
		for (int k = 0; k < 3; ++k) c.v[k] = (c.v[k] * bi) >> 8;
		c.v[3] = 0; // brightness vector (b, b, b, 0)
		l32[i] = from_lanes32(c);
		l64[i] = from_lanes64(c); // the same lanes: 8-bit values * brightness, 16-bit range
	}
	uint32_t s = size;
	for (uint32_t m = 0; m < NUM_MIPS; ++m)
	{
		if (s == 0) break;
		sc.skybox_mips[side][m] = SkyboxMip{sc.skybox32.size(), s};
		sc.skybox32.insert(sc.skybox32.end(), l32.begin(), l32.end());
		sc.skybox64.insert(sc.skybox64.end(), l64.begin(), l64.end());
		const uint32_t n = s >> 1;
		if (m + 1 == NUM_MIPS || n == 0) break;
		std::vector<uint32_t> n32(size_t(n) * n);
		std::vector<uint64_t> n64(size_t(n) * n);
		for (uint32_t y = 0; y < n; ++y)
			for (uint32_t x = 0; x < n; ++x)
			{
				const size_t o0 = size_t(2 * y) * s + 2 * x, o1 = size_t(2 * y + 1) * s + 2 * x;
				Lanes a32 = lanes32(l32[o0]), b32 = lanes32(l32[o1]), c32 = lanes32(l32[o0 + 1]), d32 = lanes32(l32[o1 + 1]);
				Lanes a64 = lanes64(l64[o0]), b64 = lanes64(l64[o1]), c64 = lanes64(l64[o0 + 1]), d64 = lanes64(l64[o1 + 1]);
				Lanes r32, r64;
				for (int k = 0; k < 4; ++k)
				{
					// shift_right::<2>(add(add(p00, p01), add(p10, p11)))
					r32.v[k] = ((a32.v[k] + b32.v[k]) + (c32.v[k] + d32.v[k])) >> 2;
					r64.v[k] = ((a64.v[k] + b64.v[k]) + (c64.v[k] + d64.v[k])) >> 2;
				}
				n32[size_t(y) * n + x] = from_lanes32(r32);
				n64[size_t(y) * n + x] = from_lanes64(r64);
			}
		l32.swap(n32);
		l64.swap(n64);
		s = n;
	}
}

void make_emissive_texture(Rng& rng, uint32_t size, Scene& sc)
{
	std::vector<uint32_t> level(size_t(size) * size);
	const std::vector<float> n = value_noise(rng, size, 16);
	for (size_t i = 0; i < level.size(); ++i)
	{
		const uint32_t v = uint32_t(std::fmin(n[i] * n[i] * 400.0f, 255.0f));
		level[i] = (255u << 24) | (v << 16) | ((v * 3 / 4) << 8) | (v / 3);
	}
	uint32_t w = size, h = size;
	for (uint32_t m = 0; m < NUM_MIPS; ++m)
	{
		sc.emissive_mips.push_back(SwEmissiveMip{sc.emissive_pixels.size(), w, h});
		sc.emissive_pixels.insert(sc.emissive_pixels.end(), level.begin(), level.end());
		if (m + 1 < NUM_MIPS)
		{
			std::vector<uint32_t> next(size_t(w / 2) * (h / 2));
			for (uint32_t y = 0; y < h / 2; ++y)
				for (uint32_t x = 0; x < w / 2; ++x)
					next[y * (w / 2) + x] = average4(level[(2 * y) * w + 2 * x], level[(2 * y + 1) * w + 2 * x],
						level[(2 * y) * w + 2 * x + 1], level[(2 * y + 1) * w + 2 * x + 1]);
			level.swap(next);
			w >>= 1;
			h >>= 1;
		}
	}
}

// ---- geometry -------------------------------------------------------------------------------

// The config's moving point lights: each follows the camera path some frames ahead, orbiting a point
// displaced from it.
void add_dynamic_lights(const SceneConfig& cfg, Rng& rng, Scene& sc)
{
	for (uint32_t k = 0; k < cfg.num_dynamic_lights; ++k)
	{
		DynamicLightSpec d;
		d.path_offset = 8 + rng.below(48);
		d.offset = v3(rng.uniform(-24, 24), rng.uniform(-24, 24), rng.uniform(-16, 40));
		d.orbit_radius = rng.uniform(8, 40);
		d.radius = rng.uniform(192, 448);
		const float intensity = rng.uniform(4e4f, 1.2e5f);
		d.color[0] = intensity * rng.uniform(0.5f, 1.0f);
		d.color[1] = intensity * rng.uniform(0.5f, 1.0f);
		d.color[2] = intensity * rng.uniform(0.5f, 1.0f);
		sc.dynamic_lights.push_back(d);
	}
}

// The camera keys of a way-point polyline (densified as a Catmull-Rom spline when `smooth`): one key
// per frame, 6 units apart along the line, looking 6 dense points ahead.
void camera_path_from_way(const std::vector<Vec3>& way, bool smooth, const SceneConfig& cfg, Scene& sc)
{
	std::vector<Vec3> dense;
	if (smooth)
	{
		for (size_t k = 0; k + 1 < way.size(); ++k)
		{
			const Vec3 p0 = way[k == 0 ? 0 : k - 1], p1 = way[k], p2 = way[k + 1], p3 = way[std::min(k + 2, way.size() - 1)];
			for (int s = 0; s < 32; ++s)
			{
				const float t = s / 32.0f, t2 = t * t, t3 = t2 * t;
				dense.push_back((p1 * 2.0f + (p2 - p0) * t + (p0 * 2.0f - p1 * 5.0f + p2 * 4.0f - p3) * t2 +
					(p1 * 3.0f - p0 - p2 * 3.0f + p3) * t3) * 0.5f);
			}
		}
		dense.push_back(way.back());
	}
	else
	{
		// straight segments, 8 points each (so "6 points ahead" still looks ahead)
		for (size_t k = 0; k + 1 < way.size(); ++k)
			for (int s = 0; s < 8; ++s) dense.push_back(way[k] + (way[k + 1] - way[k]) * (float(s) / 8.0f));
		dense.push_back(way.back());
	}
	const float speed = 6.0f; // units per frame
	sc.camera_path.clear();
	size_t seg = 0;
	float along = 0.0f;
	Vec3 pos = dense[0];
	for (uint32_t f = 0; f < cfg.num_frames; ++f)
	{
		// Advance `speed` units along the polyline.
		float left = f == 0 ? 0.0f : speed;
		while (left > 0.0f && seg + 1 < dense.size())
		{
			const float seg_len = magnitude(dense[seg + 1] - dense[seg]);
			if (along + left < seg_len)
			{
				along += left;
				left = 0.0f;
			}
			else
			{
				left -= seg_len - along;
				along = 0.0f;
				++seg;
			}
		}
		const size_t s2 = std::min(seg + 1, dense.size() - 1);
		const float seg_len = std::fmax(magnitude(dense[s2] - dense[seg]), 1e-6f);
		pos = dense[seg] + (dense[s2] - dense[seg]) * (along / seg_len);
		const size_t ahead = std::min(seg + 6, dense.size() - 1);
		Vec3 dir = dense[ahead] - pos;
		if (magnitude2(dir) < 1e-6f) dir = v3(1, 0, 0);
		CameraKey k;
		k.position = pos;
		k.azimuth = std::atan2(dir.y, dir.x);
		k.elevation = 0.08f * std::sin(float(f) * 0.07f) + cfg.camera_pitch;
		sc.camera_path.push_back(k);
	}
}

struct Builder
{
	const SceneConfig& cfg;
	Scene& sc;
	Rng& rng;
	std::vector<Room> rooms;
	std::vector<uint8_t> edge_x, edge_y; // edge_x[i + j*gx]: (i,j)-(i+1,j); edge_y: (i,j)-(i,j+1)
	std::vector<int32_t> leaf_room;      // owner room of each leaf
	struct PendingPortal
	{
		uint32_t leafs[2];
		Plane plane;
		Vec3 v[4];
	};
	std::vector<PendingPortal> portals;

	Builder(const SceneConfig& c, Scene& s, Rng& r) : cfg(c), sc(s), rng(r) {}

	uint32_t gx() const { return cfg.grid_x; }
	uint32_t gy() const { return cfg.grid_y; }
	Room& room(uint32_t i, uint32_t j) { return rooms[j * gx() + i]; }
	bool has_x(uint32_t i, uint32_t j) const { return i + 1 < cfg.grid_x && edge_x[j * cfg.grid_x + i]; }
	bool has_y(uint32_t i, uint32_t j) const { return j + 1 < cfg.grid_y && edge_y[j * cfg.grid_x + i]; }

	void make_rooms()
	{
		rooms.resize(size_t(gx()) * gy());
		for (uint32_t j = 0; j < gy(); ++j)
			for (uint32_t i = 0; i < gx(); ++i)
			{
				Room& r = room(i, j);
				const float ox = i * CELL_PITCH, oy = j * CELL_PITCH;
				const float sx = snap16(rng.uniform(cfg.room_min, cfg.room_max + 1.0f));
				const float sy = snap16(rng.uniform(cfg.room_min, cfg.room_max + 1.0f));
				r.h = snap16(rng.uniform(std::max(cfg.room_min, 256.0f), cfg.room_max + 1.0f));
				// Each room covers the cell's centre band so corridors at the centre lines always fit.
				const float cx = ox + CELL_SLOT * 0.5f, cy = oy + CELL_SLOT * 0.5f;
				const float lo_x = std::max(ox, cx + CORRIDOR_HALF + 16.0f - sx), hi_x = std::min(cx - CORRIDOR_HALF - 16.0f, ox + CELL_SLOT - sx);
				const float lo_y = std::max(oy, cy + CORRIDOR_HALF + 16.0f - sy), hi_y = std::min(cy - CORRIDOR_HALF - 16.0f, oy + CELL_SLOT - sy);
				r.x0 = snap16(rng.uniform(lo_x, std::max(lo_x, hi_x)));
				r.y0 = snap16(rng.uniform(lo_y, std::max(lo_y, hi_y)));
				r.x1 = r.x0 + sx;
				r.y1 = r.y0 + sy;
				r.cx = cx;
				r.cy = cy;
				r.mat_wall = rng.below(cfg.num_materials);
				r.mat_floor = rng.below(cfg.num_materials);
				r.mat_ceiling = rng.below(cfg.num_materials);
				r.tc_shift[0] = int32_t(rng.below(256));
				r.tc_shift[1] = int32_t(rng.below(256));
				for (uint32_t l = 0; l < std::max(cfg.lights_per_room, 1u); ++l)
				{
					r.lights.push_back(v3(rng.uniform(r.x0 + 32, r.x1 - 32), rng.uniform(r.y0 + 32, r.y1 - 32), rng.uniform(96.0f, r.h - 32.0f)));
					const float intensity = rng.uniform(0.6e5f, 1.6e5f);
					r.light_colors.push_back(v3(intensity * rng.uniform(0.8f, 1.0f), intensity * rng.uniform(0.7f, 1.0f), intensity * rng.uniform(0.6f, 1.0f)));
				}
			}
		// Connectivity: random spanning tree over the grid plus extra edges.
		edge_x.assign(size_t(gx()) * gy(), 0);
		edge_y.assign(size_t(gx()) * gy(), 0);
		std::vector<uint8_t> seen(size_t(gx()) * gy(), 0);
		std::vector<uint32_t> stack{0};
		seen[0] = 1;
		while (!stack.empty())
		{
			const uint32_t c = stack.back();
			const uint32_t i = c % gx(), j = c / gx();
			uint32_t cand[4];
			int n = 0;
			if (i + 1 < gx() && !seen[c + 1]) cand[n++] = c + 1;
			if (i > 0 && !seen[c - 1]) cand[n++] = c - 1;
			if (j + 1 < gy() && !seen[c + gx()]) cand[n++] = c + gx();
			if (j > 0 && !seen[c - gx()]) cand[n++] = c - gx();
			if (n == 0)
			{
				stack.pop_back();
				continue;
			}
			const uint32_t d = cand[rng.below(uint32_t(n))];
			if (d == c + 1) edge_x[c] = 1;
			else if (d == c - 1) edge_x[c - 1] = 1;
			else if (d == c + gx()) edge_y[c] = 1;
			else edge_y[c - gx()] = 1;
			seen[d] = 1;
			stack.push_back(d);
		}
		for (uint32_t j = 0; j < gy(); ++j)
			for (uint32_t i = 0; i < gx(); ++i)
			{
				if (i + 1 < gx() && rng.uniform() < 0.35f) edge_x[j * gx() + i] = 1;
				if (j + 1 < gy() && rng.uniform() < 0.35f) edge_y[j * gx() + i] = 1;
			}
	}

	// Append one convex quad (clockwise seen from the front) with its tc equations.
	void add_quad(Vec3 p00, Vec3 p10, Vec3 p11, Vec3 p01, Vec3 normal, uint32_t material, const int32_t tc_shift[2])
	{
		// Clockwise on screen when seen from the front <=> cross(v1-v0, v2-v0) . normal < 0.
		Vec3 q[4] = {p00, p10, p11, p01};
		if (dot(cross(q[1] - q[0], q[2] - q[0]), normal) > 0.0f) std::swap(q[1], q[3]);
		MapPolygon p;
		p.first_vertex = uint32_t(sc.vertices.size());
		p.num_vertices = 4;
		for (const Vec3& v : q) sc.vertices.push_back(v);
		p.plane = Plane{normal, dot(normal, p00)};
		// Quake-style axis projection, one texel per unit.
		Vec3 ta, tb;
		if (std::fabs(normal.z) > 0.5f)
		{
			ta = v3(1, 0, 0);
			tb = v3(0, -1, 0);
		}
		else if (std::fabs(normal.x) > 0.5f)
		{
			ta = v3(0, 1, 0);
			tb = v3(0, 0, -1);
		}
		else
		{
			ta = v3(1, 0, 0);
			tb = v3(0, 0, -1);
		}
		p.tex_coord_equation[0] = Plane{ta, float(tc_shift[0])};
		p.tex_coord_equation[1] = Plane{tb, float(tc_shift[1])};
		// Integer tc bounds as the map compiler computes them (bsp_map_compact_conversion.rs:204-238).
		const float inf = float(1 << 29);
		float tmin[2] = {inf, inf}, tmax[2] = {-inf, -inf};
		for (const Vec3& v : q)
			for (int i = 0; i < 2; ++i)
			{
				const float tc = dot(p.tex_coord_equation[i].vec, v) + p.tex_coord_equation[i].dist;
				tmin[i] = std::fmin(tmin[i], tc);
				tmax[i] = std::fmax(tmax[i], tc);
			}
		for (int i = 0; i < 2; ++i)
		{
			p.tex_coord_min[i] = int32_t(std::floor(tmin[i] + 1.0f / 32.0f));
			p.tex_coord_max[i] = std::max(int32_t(std::ceil(tmax[i] - 1.0f / 32.0f)), p.tex_coord_min[i] + 1);
		}
		p.lightmap_data_offset = 0;
		p.texture = material;
		sc.polygons.push_back(p);
	}

	// Tile an axis-aligned rectangle of a face. axis = normal axis (0,1,2), w = coordinate on it,
	// (a0..a1) x (b0..b1) along the other two axes in increasing order.
	void add_face_rect(int axis, float w, float sign, float a0, float a1, float b0, float b1, uint32_t material,
		const int32_t tc_shift[2])
	{
		if (a1 - a0 < 0.5f || b1 - b0 < 0.5f) return;
		const float T = cfg.tile_size;
		auto cuts = [&](float lo, float hi) {
			std::vector<float> c{lo};
			for (float x = std::floor(lo / T) * T + T; x < hi - 0.5f; x += T)
				if (x > lo + 0.5f) c.push_back(x);
			c.push_back(hi);
			return c;
		};
		const std::vector<float> ca = cuts(a0, a1), cb = cuts(b0, b1);
		const Vec3 normal = axis == 0 ? v3(sign, 0, 0) : axis == 1 ? v3(0, sign, 0) : v3(0, 0, sign);
		auto P = [&](float a, float b) {
			return axis == 0 ? v3(w, a, b) : axis == 1 ? v3(a, w, b) : v3(a, b, w);
		};
		for (size_t ib = 0; ib + 1 < cb.size(); ++ib)
			for (size_t ia = 0; ia + 1 < ca.size(); ++ia)
				add_quad(P(ca[ia], cb[ib]), P(ca[ia + 1], cb[ib]), P(ca[ia + 1], cb[ib + 1]), P(ca[ia], cb[ib + 1]), normal, material,
					tc_shift);
	}

	// Wall with an optional opening at [o0, o1] x [0, CORRIDOR_HEIGHT] (the opening touches the floor).
	void add_wall(int axis, float w, float sign, float a0, float a1, float h, bool opening, float o0, float o1,
		uint32_t material, const int32_t tc_shift[2])
	{
		if (!opening)
		{
			add_face_rect(axis, w, sign, a0, a1, 0.0f, h, material, tc_shift);
			return;
		}
		add_face_rect(axis, w, sign, a0, o0, 0.0f, h, material, tc_shift);
		add_face_rect(axis, w, sign, o1, a1, 0.0f, h, material, tc_shift);
		add_face_rect(axis, w, sign, o0, o1, CORRIDOR_HEIGHT, h, material, tc_shift);
	}

	uint32_t begin_leaf(int32_t owner_room)
	{
		BspLeaf l;
		l.first_polygon = uint32_t(sc.polygons.size());
		l.num_polygons = 0;
		l.first_leaf_portal = 0;
		l.num_leaf_portals = 0;
		sc.leafs.push_back(l);
		leaf_room.push_back(owner_room);
		return uint32_t(sc.leafs.size() - 1);
	}
	void end_leaf(uint32_t leaf) { sc.leafs[leaf].num_polygons = uint32_t(sc.polygons.size()) - sc.leafs[leaf].first_polygon; }

	uint32_t add_node(Plane plane, uint32_t front, uint32_t back)
	{
		sc.nodes.push_back(BspNode{{front, back}, plane});
		return uint32_t(sc.nodes.size() - 1);
	}

	// Corridor-half leaf: axis 0 = corridor along x spanning [l0, l1], centre line y = c.
	uint32_t corridor_leaf(int axis, float l0, float l1, float c, uint32_t owner)
	{
		const Room& r = rooms[owner];
		const uint32_t leaf = begin_leaf(int32_t(owner));
		add_face_rect(2, 0.0f, 1.0f, axis == 0 ? l0 : c - CORRIDOR_HALF, axis == 0 ? l1 : c + CORRIDOR_HALF,
			axis == 0 ? c - CORRIDOR_HALF : l0, axis == 0 ? c + CORRIDOR_HALF : l1, r.mat_floor, r.tc_shift);
		add_face_rect(2, CORRIDOR_HEIGHT, -1.0f, axis == 0 ? l0 : c - CORRIDOR_HALF, axis == 0 ? l1 : c + CORRIDOR_HALF,
			axis == 0 ? c - CORRIDOR_HALF : l0, axis == 0 ? c + CORRIDOR_HALF : l1, r.mat_ceiling, r.tc_shift);
		const int side_axis = axis == 0 ? 1 : 0;
		add_face_rect(side_axis, c - CORRIDOR_HALF, 1.0f, l0, l1, 0.0f, CORRIDOR_HEIGHT, r.mat_wall, r.tc_shift);
		add_face_rect(side_axis, c + CORRIDOR_HALF, -1.0f, l0, l1, 0.0f, CORRIDOR_HEIGHT, r.mat_wall, r.tc_shift);
		end_leaf(leaf);
		return leaf;
	}

	void add_portal(uint32_t front_leaf, uint32_t back_leaf, int axis, float w, float sign, float a0, float a1, float b0, float b1)
	{
		PendingPortal p;
		p.leafs[0] = front_leaf;
		p.leafs[1] = back_leaf;
		const Vec3 n = axis == 0 ? v3(sign, 0, 0) : axis == 1 ? v3(0, sign, 0) : v3(0, 0, sign);
		p.plane = Plane{n, sign * w};
		auto P = [&](float a, float b) { return axis == 0 ? v3(w, a, b) : axis == 1 ? v3(a, w, b) : v3(a, b, w); };
		p.v[0] = P(a0, b0);
		p.v[1] = P(a1, b0);
		p.v[2] = P(a1, b1);
		p.v[3] = P(a0, b1);
		portals.push_back(p);
	}

	// Corridor halves of cell (i, j) towards its neighbours, created while building the cell subtree.
	struct CellLeafs
	{
		int32_t east = -1, west = -1, north = -1, south = -1;
	};
	std::vector<CellLeafs> cell_leafs;
	uint32_t path_start_room = 0; // room of the camera path's first key
	std::vector<uint32_t> path_rooms; // the rooms the camera path walks through, in order

	uint32_t build_cell(uint32_t i, uint32_t j)
	{
		const uint32_t ri = j * gx() + i;
		const Room& r = rooms[ri];
		const bool E = has_x(i, j), W = i > 0 && has_x(i - 1, j), N = has_y(i, j), S = j > 0 && has_y(i, j - 1);
		const float gap_e = (i + 1) * CELL_PITCH - 128.0f, gap_w = i * CELL_PITCH - 128.0f;
		const float gap_n = (j + 1) * CELL_PITCH - 128.0f, gap_s = j * CELL_PITCH - 128.0f;
		CellLeafs& cl = cell_leafs[ri];

		// Room leaf.
		const uint32_t room_leaf = begin_leaf(int32_t(ri));
		rooms[ri].leaf = room_leaf;
		add_face_rect(2, 0.0f, 1.0f, r.x0, r.x1, r.y0, r.y1, r.mat_floor, r.tc_shift);
		rooms[ri].ceiling_first = uint32_t(sc.polygons.size());
		add_face_rect(2, r.h, -1.0f, r.x0, r.x1, r.y0, r.y1, r.mat_ceiling, r.tc_shift);
		rooms[ri].ceiling_end = uint32_t(sc.polygons.size());
		add_wall(0, r.x1, -1.0f, r.y0, r.y1, r.h, E, r.cy - CORRIDOR_HALF, r.cy + CORRIDOR_HALF, r.mat_wall, r.tc_shift);
		add_wall(0, r.x0, 1.0f, r.y0, r.y1, r.h, W, r.cy - CORRIDOR_HALF, r.cy + CORRIDOR_HALF, r.mat_wall, r.tc_shift);
		add_wall(1, r.y1, -1.0f, r.x0, r.x1, r.h, N, r.cx - CORRIDOR_HALF, r.cx + CORRIDOR_HALF, r.mat_wall, r.tc_shift);
		add_wall(1, r.y0, 1.0f, r.x0, r.x1, r.h, S, r.cx - CORRIDOR_HALF, r.cx + CORRIDOR_HALF, r.mat_wall, r.tc_shift);
		end_leaf(room_leaf);

		uint32_t child = room_leaf + FIRST_LEAF_INDEX;
		if (S)
		{
			const uint32_t l = corridor_leaf(1, gap_s, r.y0, r.cx, ri);
			cl.south = int32_t(l);
			add_portal(l, room_leaf, 1, r.y0, -1.0f, r.cx - CORRIDOR_HALF, r.cx + CORRIDOR_HALF, 0.0f, CORRIDOR_HEIGHT);
			child = add_node(Plane{v3(0, -1, 0), -r.y0}, l + FIRST_LEAF_INDEX, child);
		}
		if (N)
		{
			const uint32_t l = corridor_leaf(1, r.y1, gap_n, r.cx, ri);
			cl.north = int32_t(l);
			add_portal(l, room_leaf, 1, r.y1, 1.0f, r.cx - CORRIDOR_HALF, r.cx + CORRIDOR_HALF, 0.0f, CORRIDOR_HEIGHT);
			child = add_node(Plane{v3(0, 1, 0), r.y1}, l + FIRST_LEAF_INDEX, child);
		}
		if (W)
		{
			const uint32_t l = corridor_leaf(0, gap_w, r.x0, r.cy, ri);
			cl.west = int32_t(l);
			add_portal(l, room_leaf, 0, r.x0, -1.0f, r.cy - CORRIDOR_HALF, r.cy + CORRIDOR_HALF, 0.0f, CORRIDOR_HEIGHT);
			child = add_node(Plane{v3(-1, 0, 0), -r.x0}, l + FIRST_LEAF_INDEX, child);
		}
		if (E)
		{
			const uint32_t l = corridor_leaf(0, r.x1, gap_e, r.cy, ri);
			cl.east = int32_t(l);
			add_portal(l, room_leaf, 0, r.x1, 1.0f, r.cy - CORRIDOR_HALF, r.cy + CORRIDOR_HALF, 0.0f, CORRIDOR_HEIGHT);
			child = add_node(Plane{v3(1, 0, 0), r.x1}, l + FIRST_LEAF_INDEX, child);
		}
		return child;
	}

	uint32_t build(uint32_t ix0, uint32_t ix1, uint32_t iy0, uint32_t iy1)
	{
		const uint32_t nx = ix1 - ix0, ny = iy1 - iy0;
		if (nx == 1 && ny == 1) return build_cell(ix0, iy0);
		if (nx >= ny)
		{
			const uint32_t mid = ix0 + nx / 2;
			const uint32_t back = build(ix0, mid, iy0, iy1);
			const uint32_t front = build(mid, ix1, iy0, iy1);
			return add_node(Plane{v3(1, 0, 0), mid * CELL_PITCH - 128.0f}, front, back);
		}
		const uint32_t mid = iy0 + ny / 2;
		const uint32_t back = build(ix0, ix1, iy0, mid);
		const uint32_t front = build(ix0, ix1, mid, iy1);
		return add_node(Plane{v3(0, 1, 0), mid * CELL_PITCH - 128.0f}, front, back);
	}

	void link_corridor_halves()
	{
		for (uint32_t j = 0; j < gy(); ++j)
			for (uint32_t i = 0; i < gx(); ++i)
			{
				const Room& r = room(i, j);
				if (has_x(i, j))
				{
					const uint32_t back = uint32_t(cell_leafs[j * gx() + i].east), front = uint32_t(cell_leafs[j * gx() + i + 1].west);
					add_portal(front, back, 0, (i + 1) * CELL_PITCH - 128.0f, 1.0f, r.cy - CORRIDOR_HALF, r.cy + CORRIDOR_HALF, 0.0f,
						CORRIDOR_HEIGHT);
				}
				if (has_y(i, j))
				{
					const uint32_t back = uint32_t(cell_leafs[j * gx() + i].north), front = uint32_t(cell_leafs[(j + 1) * gx() + i].south);
					add_portal(front, back, 1, (j + 1) * CELL_PITCH - 128.0f, 1.0f, r.cx - CORRIDOR_HALF, r.cx + CORRIDOR_HALF, 0.0f,
						CORRIDOR_HEIGHT);
				}
			}
		// Store portals and per-leaf portal lists.
		std::vector<std::vector<uint32_t>> per_leaf(sc.leafs.size());
		for (size_t k = 0; k < portals.size(); ++k)
		{
			const PendingPortal& p = portals[k];
			MapPortal mp;
			mp.leafs[0] = p.leafs[0];
			mp.leafs[1] = p.leafs[1];
			mp.plane = p.plane;
			mp.first_vertex = uint32_t(sc.vertices.size());
			mp.num_vertices = 4;
			for (const Vec3& v : p.v) sc.vertices.push_back(v);
			sc.portals.push_back(mp);
			per_leaf[p.leafs[0]].push_back(uint32_t(k));
			per_leaf[p.leafs[1]].push_back(uint32_t(k));
		}
		for (size_t l = 0; l < sc.leafs.size(); ++l)
		{
			sc.leafs[l].first_leaf_portal = uint32_t(sc.leafs_portals.size());
			sc.leafs[l].num_leaf_portals = uint32_t(per_leaf[l].size());
			sc.leafs_portals.insert(sc.leafs_portals.end(), per_leaf[l].begin(), per_leaf[l].end());
		}
	}

	// Lightmaps: direct light of the owner room's lights, simple (RGB) and directional (ambient +
	// dominant tangent-space direction, lightmaps_builder.rs:1076-1083 convention).
	void build_lightmaps()
	{
		sc.lightmaps.assign(3, 0.0f);
		sc.directional_lightmaps.assign(1, SwDirectionalLightmapElement{});
		uint64_t offset = 1;
		for (size_t pi = 0; pi < sc.polygons.size(); ++pi)
		{
			MapPolygon& p = sc.polygons[pi];
			const uint32_t lw = uint32_t(((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1);
			const uint32_t lh = uint32_t(((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1);
			p.lightmap_data_offset = uint32_t(offset);
			offset += uint64_t(lw) * lh;
			// calculate_lightmap_basis, src/common/lightmap.rs:36-62
			const float s = 1.0f / float(LIGHTMAP_SCALE);
			Mat4 m;
			m.c[0] = extend(p.tex_coord_equation[0].vec, p.tex_coord_equation[0].dist) * s;
			m.c[1] = extend(p.tex_coord_equation[1].vec, p.tex_coord_equation[1].dist) * s;
			m.c[2] = extend(p.plane.vec, -p.plane.dist);
			m.c[3] = v4(0, 0, 0, 1);
			Mat4 inv;
			invert(transpose(m), inv);
			const Vec3 u_vec = truncate(inv.c[0]), v_vec = truncate(inv.c[1]);
			const Vec3 pos0 = truncate(inv.c[3]) + u_vec * float(p.tex_coord_min[0] >> 4) + v_vec * float(p.tex_coord_min[1] >> 4);
			const Vec3 n = p.plane.vec / magnitude(p.plane.vec);
			const Vec3 un = u_vec / magnitude(u_vec), vn = v_vec / magnitude(v_vec);
			const Room& room_ = rooms[leaf_room[sc.polygon_leaf[pi]]];
			for (uint32_t y = 0; y < lh; ++y)
				for (uint32_t x = 0; x < lw; ++x)
				{
					const Vec3 tp = pos0 + u_vec * float(x) + v_vec * float(y) + n;
					float irr[3] = {0, 0, 0}, total[3] = {0, 0, 0};
					Vec3 dsum = v3(0, 0, 0);
					float lsum = 0.0f;
					for (size_t li = 0; li < room_.lights.size(); ++li)
					{
						const Vec3 d = room_.lights[li] - tp;
						const float nd = dot(n, d);
						if (nd <= 0.0f) continue;
						const float d2 = std::fmax(magnitude2(d), 1.0f);
						const float len = std::sqrt(d2);
						const float cosv = nd / len;
						const Vec3 c = room_.light_colors[li] / d2;
						irr[0] += c.x * cosv;
						irr[1] += c.y * cosv;
						irr[2] += c.z * cosv;
						total[0] += c.x;
						total[1] += c.y;
						total[2] += c.z;
						const float lum = (c.x + c.y + c.z) * (1.0f / 3.0f);
						dsum = dsum + v3(dot(d, un), dot(d, vn), nd) * (lum / len);
						lsum += lum;
					}
					const float ambient = 0.06f;
					sc.lightmaps.push_back(irr[0] + ambient);
					sc.lightmaps.push_back(irr[1] + ambient);
					sc.lightmaps.push_back(irr[2] + ambient);
					SwDirectionalLightmapElement de;
					const float dl = magnitude(dsum);
					const float deviation = lsum > 0.0f ? std::fmin(std::fmax(1.0f - dl / lsum, 0.0f), 1.0f) : 1.0f;
					for (int k = 0; k < 3; ++k) de.ambient_light[k] = ambient + total[k] * (0.25f + 0.5f * deviation);
					const Vec3 dir = dl > 0.0f ? dsum * ((1.0f - 0.5f * deviation)) : v3(0, 0, 0.001f);
					de.light_direction_vector_scaled[0] = dir.x;
					de.light_direction_vector_scaled[1] = dir.y;
					de.light_direction_vector_scaled[2] = std::fmax(dir.z, 0.001f);
					de.directional_light_deviation = deviation;
					const float mx = std::fmax(std::fmax(total[0], total[1]), std::fmax(total[2], 1e-6f));
					for (int k = 0; k < 3; ++k) de.directional_light_color[k] = lsum > 0.0f ? total[k] / mx : 1.0f;
					sc.directional_lightmaps.push_back(de);
				}
		}
		sc.lightmap_elements = offset;
	}

	// Camera path: a walk through connected rooms, Catmull-Rom through waypoints, resampled by arc length.
	void build_camera_path()
	{
		const float eye = 64.0f;
		std::vector<Vec3> way;
		uint32_t cur = rng.below(uint32_t(rooms.size()));
		path_start_room = cur;
		path_rooms.push_back(cur);
		uint32_t prev = ~0u;
		way.push_back(v3(rooms[cur].cx, rooms[cur].cy, eye));
		for (int step = 0; step < 64; ++step)
		{
			const uint32_t i = cur % gx(), j = cur / gx();
			uint32_t nb[4];
			int n = 0;
			if (has_x(i, j)) nb[n++] = cur + 1;
			if (i > 0 && has_x(i - 1, j)) nb[n++] = cur - 1;
			if (has_y(i, j)) nb[n++] = cur + gx();
			if (j > 0 && has_y(i, j - 1)) nb[n++] = cur - gx();
			if (n == 0) break;
			// Prefer not to turn straight back.
			uint32_t cand[4];
			int m = 0;
			for (int k = 0; k < n; ++k)
				if (nb[k] != prev) cand[m++] = nb[k];
			const uint32_t next = m > 0 ? cand[rng.below(uint32_t(m))] : nb[0];
			const Room& a = rooms[cur];
			const Room& b = rooms[next];
			if (next == cur + 1)
			{
				way.push_back(v3(a.x1 - 96, a.cy, eye));
				way.push_back(v3(a.x1, a.cy, eye));
				way.push_back(v3(b.x0, a.cy, eye));
				way.push_back(v3(b.x0 + 96, a.cy, eye));
			}
			else if (next + 1 == cur)
			{
				way.push_back(v3(a.x0 + 96, a.cy, eye));
				way.push_back(v3(a.x0, a.cy, eye));
				way.push_back(v3(b.x1, a.cy, eye));
				way.push_back(v3(b.x1 - 96, a.cy, eye));
			}
			else if (next == cur + gx())
			{
				way.push_back(v3(a.cx, a.y1 - 96, eye));
				way.push_back(v3(a.cx, a.y1, eye));
				way.push_back(v3(a.cx, b.y0, eye));
				way.push_back(v3(a.cx, b.y0 + 96, eye));
			}
			else
			{
				way.push_back(v3(a.cx, a.y0 + 96, eye));
				way.push_back(v3(a.cx, a.y0, eye));
				way.push_back(v3(a.cx, b.y1, eye));
				way.push_back(v3(a.cx, b.y1 - 96, eye));
			}
			way.push_back(v3(b.cx + rng.uniform(-64, 64), b.cy + rng.uniform(-64, 64), eye));
			prev = cur;
			cur = next;
			path_rooms.push_back(cur);
		}
		camera_path_from_way(way, true, cfg, sc);
	}
};

} // namespace

PolygonBasisVecs form_plane_and_tex_coord_equation(const Plane& plane, const Plane tc[2])
{
	// src/square_wheel/surfaces.rs:18-47
	Mat4 m;
	m.c[0] = extend(tc[0].vec, tc[0].dist);
	m.c[1] = extend(tc[1].vec, tc[1].dist);
	m.c[2] = extend(plane.vec, -plane.dist);
	m.c[3] = v4(0, 0, 0, 1);
	Mat4 inv;
	PolygonBasisVecs b;
	if (!invert(transpose(m), inv))
	{
		b.u = v3(1, 0, 0);
		b.v = v3(0, 1, 0);
		b.start = v3(0, 0, 0);
		b.normal = v3(0, 0, 1);
		return b;
	}
	b.u = truncate(inv.c[0]);
	b.v = truncate(inv.c[1]);
	b.start = truncate(inv.c[3]);
	b.normal = plane.vec / std::fmax(magnitude(plane.vec), 1.0f / float(1 << 30));
	return b;
}

void Scene::frame_lights(uint32_t frame, std::vector<SwLight>& out) const
{
	out.clear();
	if (camera_path.empty()) return;
	for (size_t k = 0; k < dynamic_lights.size(); ++k)
	{
		const DynamicLightSpec& d = dynamic_lights[k];
		const CameraKey& key = camera_path[std::min<size_t>(frame + d.path_offset, camera_path.size() - 1)];
		const float a = float(frame) * 0.05f + float(k);
		SwLight l;
		const Vec3 p = key.position + d.offset + v3(std::cos(a), std::sin(a), 0.0f) * d.orbit_radius;
		l.position[0] = p.x;
		l.position[1] = p.y;
		l.position[2] = p.z;
		l.radius = d.radius;
		l.inv_square_radius = 1.0f / (d.radius * d.radius); // renderer_structs.rs:237
		for (int i = 0; i < 3; ++i) l.color[i] = d.color[i];
		out.push_back(l);
	}
}

void Scene::projector_pose(uint32_t light, float t, Quat& rotation, float& fov) const
{
	// the cone sweeps around the vertical axis (1.2 rad/s) and looks 0.4 rad down; fov 60..94 degrees
	const float yaw = t * 1.2f + float(light) * 1.7f;
	rotation = quat_mul(quat_from_angle_z(yaw), quat_from_angle_y(0.4f));
	fov = 1.05f + 0.6f * float(light % 3) / 2.0f;
}

void Scene::map_polygons(std::vector<SwMapPolygon>& out) const
{
	out.resize(polygons.size());
	for (size_t i = 0; i < polygons.size(); ++i)
	{
		const MapPolygon& p = polygons[i];
		const Material& m = materials[p.texture];
		const PolygonBasisVecs& b = basis[i];
		SwMapPolygon& o = out[i];
		std::memset(&o, 0, sizeof(o));
		o.plane[0] = p.plane.vec.x, o.plane[1] = p.plane.vec.y, o.plane[2] = p.plane.vec.z, o.plane[3] = p.plane.dist;
		for (int k = 0; k < 2; ++k)
		{
			const Plane& t = p.tex_coord_equation[k];
			o.tex_coord_equation[k][0] = t.vec.x, o.tex_coord_equation[k][1] = t.vec.y;
			o.tex_coord_equation[k][2] = t.vec.z, o.tex_coord_equation[k][3] = t.dist;
			o.tex_coord_min[k] = p.tex_coord_min[k];
			o.tex_coord_max[k] = p.tex_coord_max[k];
		}
		const Vec3* vs[4] = {&b.u, &b.v, &b.start, &b.normal};
		float* ds[4] = {o.basis_u, o.basis_v, o.basis_start, o.basis_normal};
		for (int k = 0; k < 4; ++k) ds[k][0] = vs[k]->x, ds[k][1] = vs[k]->y, ds[k][2] = vs[k]->z;
		o.first_vertex = p.first_vertex;
		o.num_vertices = p.num_vertices;
		o.texture = p.texture;
		o.lightmap_data_offset = p.lightmap_data_offset;
		o.flags = material_polygon_flags(m);
		o.blending_mode = m.blending_mode;
		o.emissive_texture = m.emissive >= 0 ? uint32_t(m.emissive) : SW_NO_EMISSIVE;
		o.emissive_light[0] = m.emissive_light[0], o.emissive_light[1] = m.emissive_light[1], o.emissive_light[2] = m.emissive_light[2];
	}
}

SwCreateInfo Scene::create_info(uint32_t device) const
{
	SwCreateInfo ci;
	std::memset(&ci, 0, sizeof(ci));
	ci.abi_version = SWGPU_ABI_VERSION;
	ci.device = device;
	ci.texels = texels.data();
	ci.num_texels = texels.size();
	ci.texture_mips = texture_mips.data();
	ci.num_texture_mips = uint32_t(texture_mips.size());
	ci.emissive_pixels = emissive_pixels.data();
	ci.num_emissive_pixels = emissive_pixels.size();
	ci.emissive_mips = emissive_mips.data();
	ci.num_emissive_mips = uint32_t(emissive_mips.size());
	ci.lightmaps = lightmaps.data();
	ci.num_lightmap_elements = lightmaps.size() / 3;
	ci.directional_lightmaps = directional_lightmaps.data();
	ci.num_directional_lightmap_elements = directional_lightmaps.size();
	return ci;
}

// ---- triangle models ------------------------------------------------------------------------

// A blob mesh: a (stacks + 1) x (slices + 1) latitude-longitude grid (the seam duplicated for texture
// coordinates), 2 * slices * (stacks - 1) triangles, whose radius ripples over the animation's frames;
// normals are the ripple-free directions. Triangles wind so that the front side faces outwards.
ModelMesh make_model_mesh(Rng& rng, uint32_t triangles, uint32_t frames)
{
	const uint32_t n = std::max<uint32_t>(3, uint32_t(std::ceil(std::sqrt(float(triangles) * 0.5f))));
	const uint32_t stacks = n, slices = n;
	const float pi = 3.14159265358979323846f;
	const float radius = rng.uniform(18.0f, 36.0f);
	const float ripple = rng.uniform(0.08f, 0.22f);
	const float k0 = float(2 + rng.below(3)), k1 = float(1 + rng.below(3));
	ModelMesh m;
	m.num_frames = frames;
	m.num_vertices = (stacks + 1) * (slices + 1);
	m.positions.resize(size_t(frames) * m.num_vertices);
	m.normals.resize(size_t(frames) * m.num_vertices);
	m.tex_coords.resize(size_t(m.num_vertices) * 2);
	m.bbox_min = v3(1e30f, 1e30f, 1e30f);
	m.bbox_max = v3(-1e30f, -1e30f, -1e30f);
	for (uint32_t f = 0; f < frames; ++f)
		for (uint32_t i = 0; i <= stacks; ++i)
			for (uint32_t j = 0; j <= slices; ++j)
			{
				const float theta = pi * float(i) / float(stacks), phi = 2.0f * pi * float(j) / float(slices);
				const Vec3 dir = v3(std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta));
				const float r = radius * (1.0f + ripple * std::sin(k0 * phi + 2.0f * pi * float(f) / float(frames)) *
					std::sin(k1 * theta + pi * float(f) / float(frames)));
				const uint32_t v = i * (slices + 1) + j;
				const Vec3 p = dir * r;
				m.positions[size_t(f) * m.num_vertices + v] = p;
				m.normals[size_t(f) * m.num_vertices + v] = dir;
				m.bbox_min = v3(std::min(m.bbox_min.x, p.x), std::min(m.bbox_min.y, p.y), std::min(m.bbox_min.z, p.z));
				m.bbox_max = v3(std::max(m.bbox_max.x, p.x), std::max(m.bbox_max.y, p.y), std::max(m.bbox_max.z, p.z));
				if (f == 0)
				{
					m.tex_coords[2 * v + 0] = float(j) / float(slices);
					m.tex_coords[2 * v + 1] = float(i) / float(stacks);
				}
			}
	for (uint32_t i = 0; i < stacks; ++i)
		for (uint32_t j = 0; j < slices; ++j)
		{
			const uint32_t a = i * (slices + 1) + j, b = a + 1, c = a + slices + 1, d = c + 1;
			if (i != 0) m.triangles.insert(m.triangles.end(), {a, c, b});
			if (i != stacks - 1) m.triangles.insert(m.triangles.end(), {b, c, d});
		}
	return m;
}

// A model skin: a Color32 TextureLite with NUM_MIPS mips (each the 2x2 average of the one above, as
// Color32::get_average pairs average, color.rs:46-49), stripes over value noise; `cutout` skins get holes
// of zero alpha for alpha-tested models.
void make_model_skin(Rng& rng, uint32_t size, bool cutout, Scene& sc)
{
	std::vector<uint32_t> img(size_t(size) * size);
	const float base[3] = {rng.uniform(60, 230), rng.uniform(60, 230), rng.uniform(60, 230)};
	const float stripes = float(2 + rng.below(6));
	for (uint32_t y = 0; y < size; ++y)
		for (uint32_t x = 0; x < size; ++x)
		{
			const float s = 0.75f + 0.25f * std::sin(stripes * 6.2831853f * float(x + y) / float(size));
			const float noise = rng.uniform(0.85f, 1.0f);
			uint32_t c = 0;
			for (int k = 0; k < 3; ++k) c |= uint32_t(std::fmin(base[k] * s * noise, 255.0f)) << (8 * (2 - k));
			const bool hole = cutout && ((x / 4 + y / 4) % 5 == 0);
			c |= (hole ? 0u : 255u) << 24;
			img[size_t(y) * size + x] = c;
		}
	uint32_t w = size, h = size;
	for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
	{
		sc.lite_mips.push_back(LiteMip{uint64_t(sc.lite_pixels.size()), w, h});
		sc.lite_pixels.insert(sc.lite_pixels.end(), img.begin(), img.end());
		if (mip + 1 == NUM_MIPS) break;
		const uint32_t nw = std::max(w / 2, 1u), nh = std::max(h / 2, 1u);
		std::vector<uint32_t> next(size_t(nw) * nh);
		auto avg = [](uint32_t a, uint32_t b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); };
		for (uint32_t y = 0; y < nh; ++y)
			for (uint32_t x = 0; x < nw; ++x)
			{
				const uint32_t* r0 = &img[size_t(2 * y) * w + 2 * x];
				const uint32_t* r1 = r0 + w;
				next[size_t(y) * nw + x] = avg(avg(r0[0], r0[1]), avg(r1[0], r1[1]));
			}
		img.swap(next);
		w = nw;
		h = nh;
	}
}

// A sprite texture: a w x h Color32 TextureLite with NUM_MIPS mips (2x2 averages, as make_model_skin):
// a glowing blob whose alpha falls off from the centre (alpha-blended and additive sprites) or a hard
// disc (alpha-tested ones).
void make_sprite_texture(Rng& rng, uint32_t w, uint32_t h, bool hard, Scene& sc)
{
	std::vector<uint32_t> img(size_t(w) * h);
	const float base[3] = {rng.uniform(120, 255), rng.uniform(80, 255), rng.uniform(40, 255)};
	for (uint32_t y = 0; y < h; ++y)
		for (uint32_t x = 0; x < w; ++x)
		{
			const float dx = (float(x) + 0.5f) / float(w) * 2.0f - 1.0f, dy = (float(y) + 0.5f) / float(h) * 2.0f - 1.0f;
			const float r = std::sqrt(dx * dx + dy * dy);
			const float f = std::fmax(1.0f - r, 0.0f);
			uint32_t c = 0;
			for (int k = 0; k < 3; ++k) c |= uint32_t(std::fmin(base[k] * (0.4f + 0.6f * f) * rng.uniform(0.9f, 1.0f), 255.0f)) << (8 * (2 - k));
			const uint32_t alpha = hard ? (r < 0.8f ? 255u : 0u) : uint32_t(std::fmin(f * 1.5f, 1.0f) * 255.0f);
			img[size_t(y) * w + x] = c | (alpha << 24);
		}
	for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
	{
		sc.lite_mips.push_back(LiteMip{uint64_t(sc.lite_pixels.size()), w, h});
		sc.lite_pixels.insert(sc.lite_pixels.end(), img.begin(), img.end());
		if (mip + 1 == NUM_MIPS) break;
		const uint32_t nw = std::max(w / 2, 1u), nh = std::max(h / 2, 1u);
		std::vector<uint32_t> next(size_t(nw) * nh);
		auto avg = [](uint32_t a, uint32_t b) { return (((a ^ b) & 0xFEFEFEFEu) >> 1) + (a & b); };
		for (uint32_t y = 0; y < nh; ++y)
			for (uint32_t x = 0; x < nw; ++x)
			{
				const uint32_t* r0 = &img[size_t(std::min(2 * y, h - 1)) * w + std::min(2 * x, w - 1)];
				const uint32_t* r1 = &img[size_t(std::min(2 * y + 1, h - 1)) * w + std::min(2 * x, w - 1)];
				const uint32_t x1 = (2 * x + 1 < w) ? 1 : 0;
				next[size_t(y) * nw + x] = avg(avg(r0[0], r0[x1]), avg(r1[0], r1[x1]));
			}
		img.swap(next);
		w = nw;
		h = nh;
	}
}

float TimeFunction::evaluate(float x) const
{
	// SingleArgumentFunction::evaluate, material_function.rs:91-150
	const float tau = 6.28318530717958647692f;
	auto fract = [](float v) { return v - std::floor(v); };
	switch (kind)
	{
	case CONSTANT: return a;
	case LINEAR: return x * a + b;
	case SIN_WAVE: return std::sin(x * a * tau + b) * c + d;
	case TRIANGLE_WAVE:
	{
		const float f = fract(x * a + b);
		const float wave = f <= 0.25f ? 4.0f * f : f <= 0.75f ? 2.0f - 4.0f * f : -4.0f + 4.0f * f;
		return wave * c + d;
	}
	case SAW_TOOTH_WAVE: return (fract(x * a + b) * 2.0f - 1.0f) * c + d;
	default: return (fract(x * a + b) <= 0.5f ? 1.0f : -1.0f) * c + d;
	}
}

namespace
{

// Texture slots of the effects' outputs: for every effect material, NUM_MIPS mips appended after all
// materials' textures, initially a copy of the effect's source (turbulence: the material's texture;
// layered: the first layer's), flags the OR of what the layers carry (layered.rs:113-133).
void add_effect_outputs(Scene& sc)
{
	for (size_t m = 0; m < sc.materials.size(); ++m)
	{
		Material& mat = sc.materials[m];
		if (mat.effect == Material::NO_EFFECT) continue;
		if (mat.effect == Material::WATER || mat.effect == Material::FIRE)
		{
			// the simulation's output slot, the field's size, zero until the first generation (surfaces read
			// the material's own texture until then, as get_texture / get_emissive_texture do)
			const bool water = mat.effect == Material::WATER;
			const uint32_t* lg = water ? mat.water.resolution_log2 : mat.fire.resolution_log2;
			if (water) mat.effect_texture = int32_t(sc.texture_mips.size() / NUM_MIPS);
			else mat.effect_emissive = int32_t(sc.emissive_mips.size() / NUM_MIPS);
			for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
			{
				const uint32_t w = (1u << lg[0]) >> mip, h = (1u << lg[1]) >> mip;
				if (water)
				{
					SwTextureMip tm;
					std::memset(&tm, 0, sizeof(tm));
					tm.offset = sc.texels.size();
					tm.width = w;
					tm.height = h;
					// make_wavy_texture: a normal map, roughness below 1 when the material's is; is_metal the material's
					tm.flags = SW_TEX_HAS_NORMAL_MAP | (mat.roughness < 1.0f ? SW_TEX_HAS_NON_ONE_ROUGHNESS : 0u) |
						(mat.is_metal ? SW_TEX_IS_METAL : 0u);
					sc.texels.resize(sc.texels.size() + size_t(w) * h, 0);
					sc.texture_mips.push_back(tm);
				}
				else
				{
					sc.emissive_mips.push_back(SwEmissiveMip{sc.emissive_pixels.size(), w, h});
					sc.emissive_pixels.resize(sc.emissive_pixels.size() + size_t(w) * h, 0);
				}
			}
			mat.sim_state = sc.sim_state_words;
			sc.sim_state_words += 2ull << (lg[0] + lg[1]);
			continue;
		}
		const uint32_t src = mat.effect == Material::TURB ? uint32_t(m) : mat.layers[0].material;
		mat.effect_texture = int32_t(sc.texture_mips.size() / NUM_MIPS);
		for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
		{
			SwTextureMip tm = sc.texture_mips[src * NUM_MIPS + mip];
			const uint64_t n = uint64_t(tm.width) * tm.height;
			const uint64_t from = tm.offset;
			tm.offset = sc.texels.size();
			sc.texels.insert(sc.texels.end(), sc.texels.begin() + from, sc.texels.begin() + from + n);
			if (mat.effect == Material::LAYERED)
			{
				tm.flags = 0;
				for (const EffectLayer& l : mat.layers) tm.flags |= sc.texture_mips[l.material * NUM_MIPS + mip].flags;
			}
			sc.texture_mips.push_back(tm);
		}
	}
}

} // namespace

namespace
{

// Water and fire materials (their own generator): fire_materials materials from `first`, then
// water_materials, each with sources of every kind, over the material's own texture.
void add_simulated_effects(const SceneConfig& cfg, uint32_t first, Scene& sc)
{
	Rng r(cfg.seed ^ 0x5171u);
	uint32_t size_log2 = 0;
	while ((1u << size_log2) < cfg.texture_size) ++size_log2;
	auto sine = [&](float amplitude, float offset) {
		TimeFunction f;
		f.kind = TimeFunction::SIN_WAVE;
		f.a = r.uniform(0.1f, 0.8f);
		f.b = r.uniform(0.0f, 6.28f);
		f.c = amplitude;
		f.d = offset;
		return f;
	};
	auto constant = [](float c) {
		TimeFunction f;
		f.kind = TimeFunction::CONSTANT;
		f.a = c;
		return f;
	};
	auto deviated = [&](float value, float deviation) {
		RandomValue v;
		v.value = constant(value);
		v.deviation = constant(deviation);
		return v;
	};
	for (uint32_t i = 0; i < cfg.fire_materials; ++i)
	{
		Material& mat = sc.materials[first + i];
		FireEffect& f = mat.fire;
		f.resolution_log2[0] = std::max(4u, size_log2 - (i % 2));
		f.resolution_log2[1] = std::max(4u, size_log2 - ((i / 2) % 2));
		const uint32_t w = 1u << f.resolution_log2[0], h = 1u << f.resolution_log2[1];
		f.update_frequency = r.uniform(24.0f, 60.0f);
		f.heat_conductivity = r.uniform(8.0f, 30.0f);
		f.slow = (i % 2) == 1;
		f.has_color = (i % 3) == 0;
		f.color[0] = 1.0f, f.color[1] = r.uniform(0.3f, 0.7f), f.color[2] = r.uniform(0.0f, 0.3f);
		HeatSource point;
		point.kind = HeatSource::POINT;
		point.points[0][0] = w / 4, point.points[0][1] = h - 3;
		point.offset[0][0] = deviated(0.0f, 3.0f);
		point.offset[0][1] = deviated(0.0f, 1.0f);
		point.heat = deviated(0.9f, 0.1f);
		HeatSource line;
		line.kind = HeatSource::LINE;
		line.points[0][0] = 2, line.points[0][1] = h - 2, line.points[1][0] = w - 3, line.points[1][1] = h - 5;
		line.heat.value = sine(0.3f, 0.7f);
		HeatSource lightning;
		lightning.kind = HeatSource::LIGHTNING;
		lightning.points[0][0] = w / 2, lightning.points[0][1] = h - 4;
		lightning.points[1][0] = w / 2 + w / 8, lightning.points[1][1] = h / 4;
		lightning.offset[1][0] = deviated(0.0f, float(w) / 16.0f);
		lightning.heat = deviated(1.0f, 0.0f);
		lightning.ramp = (i % 2) == 0;
		HeatSource fountain;
		fountain.kind = HeatSource::FOUNTAIN;
		fountain.points[0][0] = 3 * w / 4, fountain.points[0][1] = h - 6;
		fountain.frequency = r.uniform(10.0f, 40.0f);
		fountain.heat = deviated(0.8f, 0.2f);
		fountain.angle = deviated(-1.5708f, 0.5f);
		fountain.speed = deviated(float(h) * 0.6f, float(h) * 0.2f);
		fountain.gravity = deviated(float(h) * 0.3f, 2.0f);
		fountain.spawn_angle = deviated(0.0f, 3.14159f);
		fountain.spawn_distance = deviated(2.0f, 2.0f);
		fountain.lifetime = deviated(1.0f, 0.5f);
		f.sources = {point, line, lightning, fountain};
		mat.effect = Material::FIRE;
		// the emissive layer the generated texture replaces (and, without a colour, the palette's source)
		mat.emissive = int32_t(sc.emissive_mips.size() / NUM_MIPS);
		make_emissive_texture(r, cfg.texture_size, sc);
		mat.emissive_light[0] = r.uniform(1.0f, 3.0f);
		mat.emissive_light[1] = r.uniform(0.5f, 2.0f);
		mat.emissive_light[2] = r.uniform(0.5f, 1.0f);
	}
	for (uint32_t i = 0; i < cfg.water_materials; ++i)
	{
		const uint32_t m = first + cfg.fire_materials + i;
		Material& mat = sc.materials[m];
		WaterEffect& wcfg = mat.water;
		// the second water material's field is narrower than its texture (the colour image is resized)
		wcfg.resolution_log2[0] = i == 1 ? std::max(4u, size_log2 - 1) : size_log2;
		wcfg.resolution_log2[1] = size_log2;
		const uint32_t w = 1u << wcfg.resolution_log2[0], h = 1u << wcfg.resolution_log2[1];
		wcfg.update_frequency = r.uniform(24.0f, 60.0f);
		wcfg.fluidity = r.uniform(40.0f, 300.0f);
		wcfg.color_mode = i % 4;
		WaveSource spot;
		spot.kind = WaveSource::WAVY_SPOT;
		spot.points[0][0] = w / 3, spot.points[0][1] = h / 3;
		spot.offsets[0][0] = sine(float(w) / 8.0f, 0.0f);
		spot.frequency = r.uniform(0.5f, 2.0f);
		spot.phase = r.uniform(0.0f, 6.0f);
		spot.amplitude = r.uniform(0.5f, 2.0f);
		WaveSource wline;
		wline.kind = WaveSource::WAVY_LINE;
		wline.points[0][0] = 1, wline.points[0][1] = h / 2, wline.points[1][0] = w / 2, wline.points[1][1] = h - 2;
		wline.offsets[1][1] = sine(float(h) / 6.0f, 0.0f);
		wline.frequency = r.uniform(0.5f, 2.0f);
		wline.amplitude = r.uniform(0.2f, 1.0f);
		wline.offset = r.uniform(-0.1f, 0.1f);
		WaveSource steep = wline; // more rows than columns: the other rasterisation branch
		steep.points[0][0] = w - 2, steep.points[0][1] = 1, steep.points[1][0] = w - 5, steep.points[1][1] = h / 2;
		steep.offsets[1][1] = TimeFunction();
		WaveSource drop;
		drop.kind = WaveSource::PERIODIC_DROPLET;
		drop.points[0][0] = 2 * w / 3, drop.points[0][1] = 2 * h / 3;
		drop.frequency = r.uniform(1.0f, 4.0f);
		drop.phase = 0.3f;
		drop.amplitude = r.uniform(2.0f, 6.0f);
		WaveSource rain;
		rain.kind = WaveSource::RAIN;
		rain.points[0][0] = w / 2, rain.points[0][1] = h / 2;
		rain.frequency = r.uniform(5.0f, 20.0f);
		rain.radius = (i % 2) ? 0.0f : float(w) / 4.0f;
		rain.amplitude = r.uniform(1.0f, 4.0f);
		wcfg.sources = {spot, wline, steep, drop, rain};
		mat.effect = Material::WATER;
		mat.roughness = r.uniform(0.2f, 0.6f);
		mat.is_metal = (sc.texture_mips[size_t(m) * NUM_MIPS].flags & SW_TEX_IS_METAL) != 0;
	}
}

} // namespace

void add_texture_effects(const SceneConfig& cfg, uint32_t n_metal, uint32_t n_diel, Scene& sc)
{
	Rng erng(cfg.seed ^ 0xEFFEC7u);
	const uint32_t nb = cfg.num_materials;
	const uint32_t first = nb - cfg.layered_materials - cfg.turb_materials;
	add_simulated_effects(cfg, first - cfg.water_materials - cfg.fire_materials, sc);
	auto wave = [&](uint32_t kind, float amplitude, float offset) {
		TimeFunction f;
		f.kind = kind;
		f.a = erng.uniform(0.2f, 1.5f);
		f.b = erng.uniform(0.0f, 6.28f);
		f.c = amplitude;
		f.d = offset;
		return f;
	};
	for (uint32_t m = first; m < nb; ++m)
	{
		sc.materials[m].emissive = -1;
		if (m < nb - cfg.layered_materials)
		{
			Material& mat = sc.materials[m];
			mat.effect = Material::TURB;
			mat.turb_amplitude = erng.uniform(2.0f, 8.0f);
			mat.turb_wave_length = erng.uniform(16.0f, 96.0f);
			mat.turb_frequency = erng.uniform(0.2f, 1.5f);
			continue;
		}
		// layer 0: the material's own texture scrolling along s; layers 1..3: additive (modulated by a sine),
		// alpha-blended (alpha ripples) and alpha-tested (per-component modulation) materials of their own
		std::vector<EffectLayer> layers(4);
		layers[0].material = m;
		layers[0].tex_coord_shift[0].kind = TimeFunction::LINEAR;
		layers[0].tex_coord_shift[0].a = erng.uniform(-40.0f, 40.0f);
		const uint32_t blends[3] = {SW_BLEND_ADDITIVE, SW_BLEND_ALPHA_BLEND, SW_BLEND_ALPHA_TEST};
		for (int k = 1; k < 4; ++k)
		{
			const bool metal = m < n_metal;
			const bool diel = !metal && m < n_metal + n_diel;
			make_material_texture(erng, cfg.texture_size, cfg.normal_maps, metal ? 0.35f : diel ? 0.5f : 1.0f, metal, sc);
			// alpha of the new texture's mips: a diagonal ripple over the whole 0..255 range
			for (uint32_t mip = 0; mip < NUM_MIPS; ++mip)
			{
				const SwTextureMip& tm = sc.texture_mips[sc.texture_mips.size() - NUM_MIPS + mip];
				for (uint32_t y = 0; y < tm.height; ++y)
					for (uint32_t x = 0; x < tm.width; ++x)
					{
						uint64_t& t = sc.texels[tm.offset + uint64_t(y) * tm.width + x];
						const uint64_t alpha = uint64_t(((x << mip) * 5 + (y << mip) * 3) & 255u);
						t = (t & ~0xFF000000ull) | (alpha << 24);
					}
			}
			Material lm;
			lm.texture_size = cfg.texture_size;
			lm.blending_mode = blends[k - 1];
			sc.materials.push_back(lm);
			EffectLayer& l = layers[k];
			l.material = uint32_t(sc.materials.size() - 1);
			l.tex_coord_shift[0] = wave(TimeFunction::SIN_WAVE, erng.uniform(4.0f, 24.0f), 0.0f);
			l.tex_coord_shift[1].kind = TimeFunction::LINEAR;
			l.tex_coord_shift[1].a = erng.uniform(-30.0f, 30.0f);
			l.tex_coord_shift[1].b = erng.uniform(-64.0f, 64.0f);
			if (k == 1)
			{
				l.has_modulate = true;
				l.modulate = wave(TimeFunction::SIN_WAVE, 0.6f, 0.4f); // below 1/128 for part of the period
			}
			else if (k == 3)
			{
				l.has_modulate_color = true;
				l.modulate_color[0] = wave(TimeFunction::TRIANGLE_WAVE, 0.5f, 1.0f);
				l.modulate_color[1] = wave(TimeFunction::SAW_TOOTH_WAVE, 0.3f, 0.8f);
				l.modulate_color[2] = wave(TimeFunction::STEP_WAVE, 0.02f, 1.0f); // stays within [0.98, 1.02]
			}
		}
		Material& mat = sc.materials[m];
		mat.effect = Material::LAYERED;
		mat.layers = layers;
	}
	add_effect_outputs(sc);
}

bool generate_scene(const SceneConfig& cfg, Scene& sc, std::string& error)
{
	if (cfg.grid_x == 0 || cfg.grid_y == 0 || cfg.grid_x * cfg.grid_y > 4096)
	{
		error = "bad grid size";
		return false;
	}
	if (cfg.room_min < 256.0f || cfg.room_max > 1024.0f || cfg.room_min > cfg.room_max)
	{
		error = "room edges must lie in [256, 1024]";
		return false;
	}
	if (cfg.tile_size < 16.0f || cfg.tile_size > 256.0f)
	{
		error = "tile_size must lie in [16, 256] (lightmaps stay within 17 texels)";
		return false;
	}
	if (uint64_t(cfg.turb_materials) + cfg.layered_materials + cfg.water_materials + cfg.fire_materials +
			std::max(cfg.animated_materials, cfg.scrolling_materials) >
		cfg.num_materials)
	{
		error = "fire, water, turb and layered materials + max(animated_materials, scrolling_materials) exceed num_materials";
		return false;
	}
	if (cfg.texture_size < 16 || (cfg.texture_size & (cfg.texture_size - 1)) || cfg.num_materials == 0)
	{
		error = "texture_size must be a power of two >= 16";
		return false;
	}
	if (cfg.sky_rooms && (cfg.skybox_size < 16 || cfg.skybox_size > 2048 || (cfg.skybox_size & (cfg.skybox_size - 1)) ||
							 !(cfg.skybox_brightness > 0.0f && cfg.skybox_brightness <= 64.0f) || cfg.skybox_missing_side > 5))
	{
		error = "skybox_size must be a power of two in [16, 2048], skybox_brightness in (0, 64]";
		return false;
	}
	sc = Scene();
	sc.config = cfg;
	Rng rng(cfg.seed);
	Builder b(cfg, sc, rng);
	b.make_rooms();
	b.cell_leafs.assign(b.rooms.size(), Builder::CellLeafs());
	b.build(0, cfg.grid_x, 0, cfg.grid_y);
	b.link_corridor_halves();
	sc.polygon_leaf.assign(sc.polygons.size(), 0);
	for (size_t l = 0; l < sc.leafs.size(); ++l)
		for (uint32_t p = 0; p < sc.leafs[l].num_polygons; ++p) sc.polygon_leaf[sc.leafs[l].first_polygon + p] = uint32_t(l);
	b.build_lightmaps();

	// Materials and textures.
	Rng trng(cfg.seed ^ 0x5EEDu);
	const uint32_t n_metal = uint32_t(cfg.metal_frac * cfg.num_materials + 0.5f);
	const uint32_t n_diel = uint32_t(cfg.dielectric_frac * cfg.num_materials + 0.5f);
	uint32_t n_emissive_tex = 0;
	for (uint32_t m = 0; m < cfg.num_materials; ++m)
	{
		const bool metal = m < n_metal;
		const bool diel = !metal && m < n_metal + n_diel;
		make_material_texture(trng, cfg.texture_size, cfg.normal_maps, metal ? 0.35f : diel ? 0.5f : 1.0f, metal, sc);
		Material mat;
		mat.texture_size = cfg.texture_size;
		if (m < cfg.scrolling_materials) // fixed speeds (no generator draws: the rest of the map is unchanged)
		{
			mat.scroll_speed[0] = 24.0f + 8.0f * float(m);
			mat.scroll_speed[1] = (m & 1) ? -13.5f : 6.25f;
		}
		if (trng.uniform() < cfg.emissive_frac)
		{
			mat.emissive = int32_t(n_emissive_tex++);
			make_emissive_texture(trng, cfg.texture_size, sc);
			mat.emissive_light[0] = trng.uniform(0.5f, 2.0f);
			mat.emissive_light[1] = trng.uniform(0.5f, 2.0f);
			mat.emissive_light[2] = trng.uniform(0.5f, 2.0f);
		}
		sc.materials.push_back(mat);
	}
	if (cfg.sky_rooms)
	{
		// The sky material (material index num_materials) with a stub regular texture, and its six side
		// textures (SpecialMaterialEffect::Skybox, src/common/material.rs; textures loaded as
		// resources_manager.rs:321-392 does).
		Rng krng(cfg.seed ^ 0x5CB0Bu);
		make_material_texture(krng, cfg.texture_size, false, 1.0f, false, sc);
		Material sky;
		sky.skybox = true;
		sky.light = false;
		sc.sky_material = int32_t(sc.materials.size());
		sc.materials.push_back(sky);
		for (uint32_t side = 0; side < 6; ++side)
		{
			const std::vector<uint32_t> img = make_sky_image(krng, cfg.skybox_size, side);
			if (int32_t(side) == cfg.skybox_missing_side) continue; // SkyboxSideTextureWithMips::default()
			add_skybox_side(img, cfg.skybox_size, cfg.skybox_brightness, side, sc);
		}
	}

	// Framed animations (framed_animation, material.rs:136-143): material m < animated_materials cycles
	// m -> a -> b -> m, the two extra frames appended after every other material (their own generator, so
	// the rest of the map is unchanged) as copies of m with their own textures.
	if (cfg.animated_materials)
	{
		Rng arng(cfg.seed ^ 0xF4A3Eu);
		const float durations[3] = {0.25f, 0.4f, 0.3f};
		for (uint32_t m = 0; m < std::min(cfg.animated_materials, cfg.num_materials); ++m)
		{
			const bool metal = m < n_metal;
			const bool diel = !metal && m < n_metal + n_diel;
			const int32_t first = int32_t(sc.materials.size());
			for (int k = 0; k < 2; ++k)
			{
				make_material_texture(arng, cfg.texture_size, cfg.normal_maps, metal ? 0.35f : diel ? 0.5f : 1.0f, metal, sc);
				Material f = sc.materials[m];
				f.next_frame = k == 0 ? first + 1 : int32_t(m);
				f.frame_duration = durations[k + 1];
				// every property can change from frame to frame: the first extra frame glows (an emissive
				// layer of its own), the second is averaged with what is behind it
				if (k == 0)
				{
					f.emissive = int32_t(sc.emissive_mips.size() / NUM_MIPS);
					make_emissive_texture(arng, cfg.texture_size, sc);
					f.emissive_light[0] = 1.5f, f.emissive_light[1] = 0.75f, f.emissive_light[2] = 0.25f;
				}
				else
					f.blending_mode = SW_BLEND_AVERAGE;
				sc.materials.push_back(f);
			}
			sc.materials[m].next_frame = first;
			sc.materials[m].frame_duration = durations[0];
		}
	}

	// Generative effects (their own generator: the rest of the scene is unchanged): the last
	// layered_materials base materials are layered animations over their own texture and three layer
	// materials (appended; no polygon uses them) with other blending modes; the turb_materials before
	// them are turbulent. Effect materials get no emissive layer.
	if (cfg.turb_materials || cfg.layered_materials || cfg.water_materials || cfg.fire_materials)
		add_texture_effects(cfg, n_metal, n_diel, sc);

	sc.basis.resize(sc.polygons.size());
	for (size_t p = 0; p < sc.polygons.size(); ++p)
		sc.basis[p] = form_plane_and_tex_coord_equation(sc.polygons[p].plane, sc.polygons[p].tex_coord_equation);

	b.build_camera_path();
	if (cfg.sky_rooms)
	{
		// Ceilings open to the sky: the room the camera path starts in and others drawn by their own
		// generator (the rest of the scene is the one without sky).
		Rng srng(cfg.seed ^ 0x5C1B0Bu);
		std::vector<uint8_t> sky(b.rooms.size(), 0);
		const uint32_t n = std::min<uint32_t>(cfg.sky_rooms, uint32_t(b.rooms.size()));
		sky[b.path_start_room] = 1;
		for (uint32_t k = 1; k < n;)
		{
			const uint32_t ri = srng.below(uint32_t(b.rooms.size()));
			if (sky[ri]) continue;
			sky[ri] = 1;
			++k;
		}
		for (size_t ri = 0; ri < b.rooms.size(); ++ri)
			if (sky[ri])
				for (uint32_t p = b.rooms[ri].ceiling_first; p < b.rooms[ri].ceiling_end; ++p)
					sc.polygons[p].texture = uint32_t(sc.sky_material);
	}
	if (cfg.num_models)
	{
		// Models: a few meshes and skins shared by num_models placements on the floors of the rooms (own
		// generator: the rest of the scene is unchanged), each inside one room leaf with its light.
		Rng mrng(cfg.seed ^ 0x30DE15u);
		const uint32_t num_meshes = 4;
		for (uint32_t k = 0; k < num_meshes; ++k)
		{
			sc.model_meshes.push_back(make_model_mesh(mrng, std::max(cfg.model_triangles, 8u), std::max(cfg.model_frames, 1u)));
			make_model_skin(mrng, 64, k == num_meshes - 1, sc);
		}
		sc.leaf_models.assign(sc.leafs.size(), {});
		const uint32_t blends[4] = {SW_BLEND_NONE, SW_BLEND_NONE, SW_BLEND_ALPHA_TEST, SW_BLEND_ADDITIVE};
		for (uint32_t i = 0; i < cfg.num_models; ++i)
		{
			const uint32_t ri = mrng.below(uint32_t(b.rooms.size()));
			const Room& r = b.rooms[ri];
			ModelEntity e;
			e.mesh = mrng.below(num_meshes);
			e.texture = e.mesh;
			e.leaf = r.leaf;
			e.blending_mode = e.mesh == num_meshes - 1 ? uint32_t(SW_BLEND_ALPHA_TEST) : blends[mrng.below(4)];
			const ModelMesh& mm = sc.model_meshes[e.mesh];
			const float margin = 48.0f;
			e.position = v3(mrng.uniform(r.x0 + margin, r.x1 - margin), mrng.uniform(r.y0 + margin, r.y1 - margin),
				-mm.bbox_min.z + 2.0f);
			e.yaw = mrng.uniform(0.0f, 6.2831853f);
			e.anim_speed = mrng.uniform(4.0f, 12.0f);
			e.anim_phase = mrng.uniform(0.0f, float(mm.num_frames));
			for (int s6 = 0; s6 < 6; ++s6)
				for (int c = 0; c < 3; ++c) e.light_cube[s6][c] = mrng.uniform(0.2f, 0.9f);
			e.light_dir_scaled = v3(mrng.uniform(-0.6f, 0.6f), mrng.uniform(-0.6f, 0.6f), mrng.uniform(0.2f, 1.0f));
			for (int c = 0; c < 3; ++c) e.light_color[c] = mrng.uniform(0.3f, 1.2f);
			sc.leaf_models[e.leaf].push_back(uint32_t(sc.models.size()));
			sc.models.push_back(e);
		}
	}
	if (cfg.num_sprites)
	{
		// Sprites (own generator): a few textures of other aspect ratios, placed inside the rooms' leafs
		// well away from their walls, every orientation, blending modes from the alpha family and additive.
		Rng prng(cfg.seed ^ 0x5B417E5u);
		const uint32_t first_texture = uint32_t(sc.lite_mips.size() / NUM_MIPS);
		const uint32_t sizes[4][2] = {{64, 64}, {32, 64}, {64, 32}, {128, 64}};
		for (int k = 0; k < 4; ++k) make_sprite_texture(prng, sizes[k][0], sizes[k][1], k == 3, sc);
		sc.leaf_sprites.assign(sc.leafs.size(), {});
		const uint32_t blends[3] = {SW_BLEND_ALPHA_BLEND, SW_BLEND_ADDITIVE, SW_BLEND_AVERAGE};
		for (uint32_t i = 0; i < cfg.num_sprites; ++i)
		{
			const Room& r = b.rooms[prng.below(uint32_t(b.rooms.size()))];
			SpriteEntity e;
			const uint32_t t = prng.below(4);
			e.texture = first_texture + t;
			e.blending_mode = t == 3 ? uint32_t(SW_BLEND_ALPHA_TEST) : blends[prng.below(3)];
			e.orientation = prng.below(4);
			e.radius = prng.uniform(12.0f, 48.0f);
			e.angle = prng.below(2) ? 0.0f : prng.uniform(-3.1f, 3.1f);
			const float margin = e.radius + 8.0f;
			e.position = v3(prng.uniform(r.x0 + margin, r.x1 - margin), prng.uniform(r.y0 + margin, r.y1 - margin),
				prng.uniform(margin, std::fmax(r.h - margin, margin + 1.0f)));
			e.leaf = r.leaf;
			e.light_scale = prng.below(4) ? prng.uniform(0.5f, 1.5f) : 0.0f;
			for (int c = 0; c < 3; ++c) e.light_add[c] = prng.uniform(0.0f, 0.6f);
			for (int s6 = 0; s6 < 6; ++s6)
				for (int c = 0; c < 3; ++c) e.light_cube[s6][c] = prng.uniform(0.2f, 0.9f);
			e.light_dir_scaled = v3(prng.uniform(-0.6f, 0.6f), prng.uniform(-0.6f, 0.6f), prng.uniform(0.2f, 1.0f));
			for (int c = 0; c < 3; ++c) e.light_color[c] = prng.uniform(0.3f, 1.2f);
			sc.leaf_sprites[e.leaf].push_back(uint32_t(sc.sprites.size()));
			sc.sprites.push_back(e);
		}
	}
	if (cfg.num_decals)
	{
		// Decals (own generator) on the walls and floors of the rooms, the cube's -x axis along the surface
		// normal: textures of their own, every blending mode, some lit by the lightmap.
		Rng drng(cfg.seed ^ 0xDECA1u);
		const uint32_t first_texture = uint32_t(sc.lite_mips.size() / NUM_MIPS);
		const uint32_t sizes[3][2] = {{64, 64}, {64, 32}, {32, 64}};
		for (int k = 0; k < 3; ++k) make_sprite_texture(drng, sizes[k][0], sizes[k][1], k == 2, sc);
		sc.leaf_decals.assign(sc.leafs.size(), {});
		const float pi = 3.14159265358979f;
		for (uint32_t i = 0; i < cfg.num_decals; ++i)
		{
			const Room& r = b.rooms[drng.below(uint32_t(b.rooms.size()))];
			DecalEntity d;
			const uint32_t t = drng.below(3);
			d.texture = first_texture + t;
			d.blending_mode = t == 2 ? uint32_t(SW_BLEND_ALPHA_TEST) : drng.below(5);
			d.scale = v3(drng.uniform(4.0f, 16.0f), drng.uniform(12.0f, 48.0f), drng.uniform(12.0f, 48.0f));
			const float ext = std::fmax(d.scale.y, d.scale.z) + 8.0f;
			// the surface: 0..3 the walls at x0, x1, y0, y1 (cube +x into the wall), 4 the floor
			const uint32_t side = drng.below(5);
			Quat facing;
			if (side == 0) facing = quat_from_angle_z(pi), d.position = v3(r.x0, drng.uniform(r.y0 + ext, r.y1 - ext), drng.uniform(ext, r.h - ext));
			else if (side == 1) facing = quat_from_angle_z(0.0f), d.position = v3(r.x1, drng.uniform(r.y0 + ext, r.y1 - ext), drng.uniform(ext, r.h - ext));
			else if (side == 2) facing = quat_from_angle_z(-0.5f * pi), d.position = v3(drng.uniform(r.x0 + ext, r.x1 - ext), r.y0, drng.uniform(ext, r.h - ext));
			else if (side == 3) facing = quat_from_angle_z(0.5f * pi), d.position = v3(drng.uniform(r.x0 + ext, r.x1 - ext), r.y1, drng.uniform(ext, r.h - ext));
			else facing = quat_from_angle_y(0.5f * pi), d.position = v3(drng.uniform(r.x0 + ext, r.x1 - ext), drng.uniform(r.y0 + ext, r.y1 - ext), 0.0f);
			// a turn of the texture about the cube's x axis
			const float roll = drng.uniform(-pi, pi);
			d.rotation = quat_mul(facing, Quat{std::cos(roll * 0.5f), v3(std::sin(roll * 0.5f), 0.0f, 0.0f)});
			d.lightmap_light_scale = drng.below(3) ? drng.uniform(0.5f, 1.5f) : 0.0f;
			for (int c = 0; c < 3; ++c) d.light_add[c] = drng.uniform(0.0f, 0.5f);
			// position_object_bbox (dynamic_objects_index.rs:159-205): the leafs the cube's convex hull reaches
			Mat4 m = mat4_from_quat(d.rotation);
			m.c[0] = m.c[0] * d.scale.x;
			m.c[1] = m.c[1] * d.scale.y;
			m.c[2] = m.c[2] * d.scale.z;
			m.c[3] = v4(d.position.x, d.position.y, d.position.z, 1.0f);
			Vec3 corners[8];
			for (int k = 0; k < 8; ++k)
				corners[k] = truncate(m * v4((k & 4) ? 1.0f : -1.0f, (k & 2) ? 1.0f : -1.0f, (k & 1) ? 1.0f : -1.0f, 1.0f));
			const uint32_t id = uint32_t(sc.decals.size());
			std::vector<uint32_t> stack{sc.root_node()};
			while (!stack.empty())
			{
				const uint32_t node = stack.back();
				stack.pop_back();
				if (node >= FIRST_LEAF_INDEX)
				{
					sc.leaf_decals[node - FIRST_LEAF_INDEX].push_back(id);
					continue;
				}
				const BspNode& nd = sc.nodes[node];
				uint32_t front = 0;
				for (const Vec3& v : corners)
					if (dot(nd.plane.vec, v) > nd.plane.dist) ++front;
				// the recursion's order (front child first): pushed back child first
				if (front < 8) stack.push_back(nd.children[1]);
				if (front > 0) stack.push_back(nd.children[0]);
			}
			sc.decals.push_back(d);
		}
	}
	if (cfg.num_portals)
	{
		// Portals (own generator): standing rectangles near a corner of the rooms the camera path walks
		// through, facing the room's centre - mirrors, screens showing a camera in another room of the path
		// (mixed with a scan-line texture), and parallax windows into another room.
		Rng qrng(cfg.seed ^ 0x9041A1u);
		std::vector<uint32_t> rooms_seen;
		for (uint32_t r : b.path_rooms)
			if (std::find(rooms_seen.begin(), rooms_seen.end(), r) == rooms_seen.end()) rooms_seen.push_back(r);
		const uint32_t screen_texture = uint32_t(sc.lite_mips.size() / NUM_MIPS);
		make_sprite_texture(qrng, 64, 64, false, sc);
		for (uint32_t m = 0; m < NUM_MIPS; ++m) // scan lines: every other row of each mip darker, alpha kept
		{
			const LiteMip& lm = sc.lite_mips[size_t(screen_texture) * NUM_MIPS + m];
			for (uint32_t y = 1; y < lm.height; y += 2)
				for (uint32_t x = 0; x < lm.width; ++x)
				{
					uint32_t& px = sc.lite_pixels[lm.offset + uint64_t(y) * lm.width + x];
					px = (px & 0xFF000000u) | ((px >> 1) & 0x7F7F7Fu);
				}
		}
		sc.leaf_view_portals.assign(sc.leafs.size(), {});
		for (uint32_t k = 0; k < cfg.num_portals; ++k)
		{
			// in view: ahead of a camera path key, facing it, inside the key's leaf
			const uint32_t nk = uint32_t(sc.camera_path.size());
			const uint32_t j = (k * 23u + 3u) % nk;
			const Vec3 eye = sc.camera_path[j].position;
			Vec3 dir = sc.camera_path[(j + 1) % nk].position - eye;
			dir.z = 0.0f;
			if (magnitude(dir) < 1e-3f) dir = v3(1.0f, 0.0f, 0.0f);
			dir = dir / magnitude(dir);
			const uint32_t eye_leaf = sc.leaf_of(eye);
			// the room of that leaf (else the path's first) and another room of the path
			uint32_t here = rooms_seen[0];
			for (uint32_t ri = 0; ri < uint32_t(b.rooms.size()); ++ri)
				if (b.rooms[ri].leaf == eye_leaf) here = ri;
			uint32_t there = rooms_seen[(k + 1) % rooms_seen.size()];
			if (there == here) there = rooms_seen[(k + 2) % rooms_seen.size()];
			const Room& r = b.rooms[here];
			const Room& other = b.rooms[there];
			ViewPortal pt;
			pt.kind = k % 3;
			const Vec3 n = -dir;
			const Vec3 t = v3(-n.y, n.x, 0.0f);
			const float hw = 40.0f + 8.0f * float(k % 3), z0 = 8.0f, z1 = 120.0f;
			Vec3 c{}, q[4];
			std::vector<uint32_t> leafs;
			bool placed = false;
			for (float dist : {220.0f, 160.0f, 110.0f, 70.0f})
			{
				c = eye + dir * dist;
				c.z = 0.0f;
				q[0] = c - t * hw + v3(0, 0, z0), q[1] = c + t * hw + v3(0, 0, z0);
				q[2] = c + t * hw + v3(0, 0, z1), q[3] = c - t * hw + v3(0, 0, z1);
				sc.convex_hull_leafs(q, 4, leafs);
				if (leafs.size() == 1 && leafs[0] == eye_leaf)
				{
					placed = true;
					break;
				}
			}
			if (!placed) continue;
			if (dot(cross(q[1] - q[0], q[2] - q[0]), n) > 0.0f) std::swap(q[1], q[3]); // clockwise seen from the front
			pt.vertices.assign(q, q + 4);
			pt.plane = Plane{n, dot(n, q[0])};
			pt.tex_coord_equation[0] = Plane{t, hw - dot(t, c)}; // one texel per unit, from the left edge
			pt.tex_coord_equation[1] = Plane{v3(0.0f, 0.0f, -1.0f), z1};
			if (pt.kind == ViewPortal::CAMERA_AT_POSITION)
			{
				pt.position = v3(other.cx, other.cy, 96.0f);
				pt.rotation = quat_from_angle_z(qrng.uniform(-3.1f, 3.1f));
				pt.fov = 1.5707964f;
				pt.texture = int32_t(screen_texture);
				pt.texture_blending_mode = SW_BLEND_AVERAGE;
				pt.light_add[0] = 1.0f, pt.light_add[1] = 0.9f, pt.light_add[2] = 0.8f;
			}
			else if (pt.kind == ViewPortal::PARALLAX)
			{
				pt.transform = Mat4::identity();
				pt.transform.c[3] = v4(other.cx - r.cx, other.cy - r.cy, 0.0f, 1.0f);
				pt.blending_mode = SW_BLEND_AVERAGE;
			}
			const uint32_t id = uint32_t(sc.view_portals.size());
			sc.convex_hull_leafs(pt.vertices.data(), uint32_t(pt.vertices.size()), leafs);
			for (uint32_t l : leafs) sc.leaf_view_portals[l].push_back(id);
			sc.view_portal_leafs.push_back(leafs);
			sc.view_portals.push_back(pt);
		}
	}
	if (cfg.light_grid)
	{
		// A seeded light grid (own generator): 64-unit cells over the rooms; a column inside a room holds
		// samples from the floor to one cell above its ceiling (the top one zero, as a lightmapper leaves
		// samples in solid space), each the room's static lights gathered into a light cube plus the
		// strongest as the directional component.
		Rng grng(cfg.seed ^ 0x6121Du);
		const float cell = 64.0f;
		float lo[2] = {1e30f, 1e30f}, hi[2] = {-1e30f, -1e30f}, top = 0.0f;
		for (const Room& r : b.rooms)
		{
			lo[0] = std::fmin(lo[0], r.x0), lo[1] = std::fmin(lo[1], r.y0);
			hi[0] = std::fmax(hi[0], r.x1), hi[1] = std::fmax(hi[1], r.y1);
			top = std::fmax(top, r.h);
		}
		LightGridHeader& hd = sc.light_grid_header;
		for (int i = 0; i < 3; ++i) hd.grid_cell_size[i] = cell;
		hd.grid_start[0] = lo[0], hd.grid_start[1] = lo[1], hd.grid_start[2] = 0.0f;
		hd.grid_size[0] = uint32_t(std::ceil((hi[0] - lo[0]) / cell)) + 1;
		hd.grid_size[1] = uint32_t(std::ceil((hi[1] - lo[1]) / cell)) + 1;
		hd.grid_size[2] = uint32_t(std::ceil(top / cell)) + 2;
		const Vec3 sides[6] = {v3(-1, 0, 0), v3(1, 0, 0), v3(0, -1, 0), v3(0, 1, 0), v3(0, 0, -1), v3(0, 0, 1)};
		const float ambient = grng.uniform(0.05f, 0.2f);
		for (uint32_t y = 0; y < hd.grid_size[1]; ++y)
			for (uint32_t x = 0; x < hd.grid_size[0]; ++x)
			{
				const float px = lo[0] + float(x) * cell, py = lo[1] + float(y) * cell;
				const Room* in = nullptr;
				for (const Room& r : b.rooms)
					if (px >= r.x0 && px <= r.x1 && py >= r.y0 && py <= r.y1) in = &r;
				LightGridColumn col{0, uint32_t(sc.light_grid_samples.size()), 0};
				if (in)
				{
					col.num_samples = uint32_t(std::floor(in->h / cell)) + 2;
					for (uint32_t z = 0; z < col.num_samples; ++z)
					{
						LightGridElement e;
						std::memset(&e, 0, sizeof(e));
						if (z + 1 < col.num_samples)
						{
							const Vec3 p = v3(px, py, float(z) * cell);
							float best = 0.0f;
							for (int s6 = 0; s6 < 6; ++s6)
								for (int c = 0; c < 3; ++c) e.light_cube[s6][c] = ambient;
							for (size_t li = 0; li < in->lights.size(); ++li)
							{
								// the light's intensity / distance^2 (the lightmaps' units), spread over the cube sides
								// facing it; the strongest also as the directional component
								const Vec3 to = in->lights[li] - p;
								const float d2 = std::fmax(dot(to, to), 32.0f * 32.0f);
								const Vec3 dir = to / std::sqrt(d2);
								const Vec3 c3 = in->light_colors[li] * (1.0f / d2);
								for (int s6 = 0; s6 < 6; ++s6)
								{
									const float f = std::fmax(dot(dir, sides[s6]), 0.0f) * 0.5f;
									e.light_cube[s6][0] += f * c3.x, e.light_cube[s6][1] += f * c3.y, e.light_cube[s6][2] += f * c3.z;
								}
								const float strength = c3.x + c3.y + c3.z;
								if (strength > best)
								{
									best = strength;
									e.light_direction_vector_scaled = dir * 0.5f;
									e.directional_light_color[0] = c3.x, e.directional_light_color[1] = c3.y, e.directional_light_color[2] = c3.z;
								}
							}
						}
						sc.light_grid_samples.push_back(e);
					}
				}
				sc.light_grid_columns.push_back(col);
			}
		// ModelLighting::Default (triangle_models_rendering.rs:541-546) and the sprites' grid fetch
		// (partial_renderer.rs:911-932): the static light at the (fixed) position, fetched from the grid
		for (ModelEntity& e : sc.models)
		{
			const LightGridElement g = sc.fetch_light_from_grid(e.position);
			std::memcpy(e.light_cube, g.light_cube, sizeof(e.light_cube));
			e.light_dir_scaled = g.light_direction_vector_scaled;
			std::memcpy(e.light_color, g.directional_light_color, sizeof(e.light_color));
		}
		for (SpriteEntity& e : sc.sprites)
		{
			const LightGridElement g = sc.fetch_light_from_grid(e.position);
			std::memcpy(e.light_cube, g.light_cube, sizeof(e.light_cube));
			e.light_dir_scaled = g.light_direction_vector_scaled;
			std::memcpy(e.light_color, g.directional_light_color, sizeof(e.light_color));
		}
		for (ViewPortal& vp : sc.view_portals)
			if (vp.texture >= 0) vp.light_scale = 1.0f;
	}
	add_dynamic_lights(cfg, rng, sc);
	return true;
}

LightGridElement Scene::fetch_light_from_grid(Vec3 pos) const
{
	// triangle_models_rendering.rs:582-700
	LightGridElement total;
	std::memset(&total, 0, sizeof(total));
	const LightGridHeader& h = light_grid_header;
	if (h.grid_size[0] == 0 || h.grid_size[1] == 0 || h.grid_size[2] == 0 || h.grid_cell_size[0] == 0.0f ||
		h.grid_cell_size[1] == 0.0f || h.grid_cell_size[2] == 0.0f || light_grid_samples.empty() || light_grid_columns.empty())
		return total;
	const float gp[3] = {(pos.x - h.grid_start[0]) / h.grid_cell_size[0], (pos.y - h.grid_start[1]) / h.grid_cell_size[1],
		(pos.z - h.grid_start[2]) / h.grid_cell_size[2]};
	int32_t gi[3];
	for (int i = 0; i < 3; ++i)
	{
		const float f = std::floor(gp[i]);
		gi[i] = std::isnan(f) ? 0 : (f >= 2147483647.0f ? 2147483647 : (f <= -2147483648.0f ? int32_t(-2147483647 - 1) : int32_t(f)));
	}
	float total_factor = 0.0f;
	for (int32_t dx = 0; dx <= 1; ++dx)
	{
		const int32_t x = gi[0] + dx;
		if (x < 0 || x >= int32_t(h.grid_size[0])) continue;
		const float fx = 1.0f - std::fabs(gp[0] - float(x));
		for (int32_t dy = 0; dy <= 1; ++dy)
		{
			const int32_t y = gi[1] + dy;
			if (y < 0 || y >= int32_t(h.grid_size[1])) continue;
			const LightGridColumn& column = light_grid_columns[uint32_t(x) + uint32_t(y) * h.grid_size[0]];
			if (column.num_samples == 0) continue;
			const float fy = 1.0f - std::fabs(gp[1] - float(y));
			for (int32_t dz = 0; dz <= 1; ++dz)
			{
				const int32_t z = gi[2] + dz;
				if (z < 0 || z >= int32_t(h.grid_size[2])) continue;
				if (uint32_t(z) < column.start_z || uint32_t(z) >= column.start_z + column.num_samples) continue;
				const LightGridElement& sample = light_grid_samples[column.first_sample + (uint32_t(z) - column.start_z)];
				bool zero = true;
				for (int s6 = 0; s6 < 6 && zero; ++s6)
					for (int c = 0; c < 3; ++c) zero = zero && sample.light_cube[s6][c] == 0.0f;
				for (int c = 0; c < 3; ++c) zero = zero && sample.directional_light_color[c] == 0.0f;
				zero = zero && sample.light_direction_vector_scaled.x == 0.0f && sample.light_direction_vector_scaled.y == 0.0f &&
					sample.light_direction_vector_scaled.z == 0.0f;
				if (zero) continue;
				const float fz = 1.0f - std::fabs(gp[2] - float(z));
				const float f = fx * fy * fz;
				for (int c = 0; c < 3; ++c)
				{
					for (int s6 = 0; s6 < 6; ++s6) total.light_cube[s6][c] += sample.light_cube[s6][c] * f;
					total.directional_light_color[c] += sample.directional_light_color[c] * f;
				}
				total.light_direction_vector_scaled = total.light_direction_vector_scaled + sample.light_direction_vector_scaled * f;
				total_factor += f;
			}
		}
	}
	if (total_factor <= 0.0f)
	{
		std::memset(&total, 0, sizeof(total));
		return total;
	}
	if (total_factor < 0.995f)
	{
		// renormalised when some of the 8 samples were missing
		const float inv = 1.0f / total_factor;
		for (int c = 0; c < 3; ++c)
		{
			for (int s6 = 0; s6 < 6; ++s6) total.light_cube[s6][c] *= inv;
			total.directional_light_color[c] *= inv;
		}
		total.light_direction_vector_scaled = total.light_direction_vector_scaled * inv;
	}
	return total;
}

uint32_t Scene::leaf_of(Vec3 p) const
{
	uint32_t node = root_node();
	while (node < FIRST_LEAF_INDEX)
	{
		const BspNode& nd = nodes[node];
		node = dot(nd.plane.vec, p) - nd.plane.dist >= 0.0f ? nd.children[0] : nd.children[1];
	}
	return node - FIRST_LEAF_INDEX;
}

void Scene::convex_hull_leafs(const Vec3* vertices, uint32_t n, std::vector<uint32_t>& out) const
{
	out.clear();
	std::vector<uint32_t> stack{root_node()};
	while (!stack.empty())
	{
		const uint32_t node = stack.back();
		stack.pop_back();
		if (node >= FIRST_LEAF_INDEX)
		{
			out.push_back(node - FIRST_LEAF_INDEX);
			continue;
		}
		const BspNode& nd = nodes[node];
		uint32_t front = 0;
		for (uint32_t i = 0; i < n; ++i)
			if (dot(nd.plane.vec, vertices[i]) > nd.plane.dist) ++front;
		if (front < n) stack.push_back(nd.children[1]); // the back child after the front one
		if (front > 0) stack.push_back(nd.children[0]);
	}
}

// ---- scenes from compiled maps ----------------------------------------------------------------

namespace
{

uint64_t fnv1a(const char* s, size_t n)
{
	uint64_t h = 1469598103934665603ull;
	for (size_t i = 0; i < n; ++i) h = (h ^ uint8_t(s[i])) * 1099511628211ull;
	return h;
}

// Every index and range of the map that rendering follows; false with a message on the first bad one.
bool check_map(const SqwmMap& m, bool directional, std::string& error)
{
	char buf[160];
	auto bad = [&](const char* fmt, uint64_t i) {
		std::snprintf(buf, sizeof(buf), fmt, (unsigned long long)i);
		error = buf;
		return false;
	};
	if (m.nodes.empty() || m.leafs.empty()) return bad("map has no BSP tree (%llu nodes)", m.nodes.size());
	if (m.textures.empty()) return bad("map has no textures (%llu)", 0);
	// children: leafs in range, nodes before their parent (the root is the last node), depth bounded
	std::vector<uint32_t> depth(m.nodes.size(), 0);
	for (size_t n = 0; n < m.nodes.size(); ++n)
		for (int c = 0; c < 2; ++c)
		{
			const uint32_t ch = m.nodes[n].children[c];
			if (ch >= FIRST_LEAF_INDEX)
			{
				if (ch - FIRST_LEAF_INDEX >= m.leafs.size()) return bad("node %llu: leaf child out of range", n);
			}
			else if (ch >= n)
				return bad("node %llu: child node not before its parent", n);
			else
				depth[n] = std::max(depth[n], depth[ch] + 1);
		}
	if (depth.back() + 1 >= 72) return bad("BSP tree deeper than 72 (%llu)", depth.back() + 1);
	std::vector<uint8_t> owned(m.polygons.size(), 0);
	for (size_t l = 0; l < m.leafs.size(); ++l)
	{
		const BspLeaf& f = m.leafs[l];
		if (uint64_t(f.first_polygon) + f.num_polygons > m.polygons.size()) return bad("leaf %llu: polygons out of range", l);
		if (uint64_t(f.first_leaf_portal) + f.num_leaf_portals > m.leafs_portals.size())
			return bad("leaf %llu: portals out of range", l);
		for (uint32_t p = 0; p < f.num_polygons; ++p)
			if (owned[f.first_polygon + p]++) return bad("polygon %llu in two leafs", f.first_polygon + p);
	}
	for (size_t i = 0; i < m.leafs_portals.size(); ++i)
		if (m.leafs_portals[i] >= m.portals.size()) return bad("leaf portal %llu out of range", i);
	for (size_t i = 0; i < m.portals.size(); ++i)
	{
		const MapPortal& p = m.portals[i];
		if (p.leafs[0] >= m.leafs.size() || p.leafs[1] >= m.leafs.size()) return bad("portal %llu: leaf out of range", i);
		if (p.num_vertices < 3 || uint64_t(p.first_vertex) + p.num_vertices > m.vertices.size())
			return bad("portal %llu: vertices out of range", i);
	}
	const uint64_t lm_elems = directional ? m.directional_lightmaps.size() : m.lightmaps.size() / 3;
	for (size_t i = 0; i < m.polygons.size(); ++i)
	{
		const MapPolygon& p = m.polygons[i];
		if (p.num_vertices < 3 || uint64_t(p.first_vertex) + p.num_vertices > m.vertices.size())
			return bad("polygon %llu: vertices out of range", i);
		if (p.texture >= m.textures.size()) return bad("polygon %llu: texture out of range", i);
		if (p.tex_coord_min[0] > p.tex_coord_max[0] || p.tex_coord_min[1] > p.tex_coord_max[1] ||
			int64_t(p.tex_coord_max[0]) - p.tex_coord_min[0] > 4096 || int64_t(p.tex_coord_max[1]) - p.tex_coord_min[1] > 4096)
			return bad("polygon %llu: bad texture coordinate bounds", i);
		if (p.lightmap_data_offset != 0)
		{
			// get_polygon_lightmap_size, lightmap.rs:11-27
			const uint64_t lw = uint64_t(((p.tex_coord_max[0] + 15) >> 4) - (p.tex_coord_min[0] >> 4) + 1);
			const uint64_t lh = uint64_t(((p.tex_coord_max[1] + 15) >> 4) - (p.tex_coord_min[1] >> 4) + 1);
			if (uint64_t(p.lightmap_data_offset) + lw * lh > lm_elems) return bad("polygon %llu: lightmap out of range", i);
		}
	}
	// the light grid: one column per (x, y) cell, each column's samples inside the sample list
	const LightGridHeader& g = m.light_grid_header;
	if (!m.light_grid_columns.empty() || !m.light_grid_samples.empty())
	{
		if (uint64_t(g.grid_size[0]) * g.grid_size[1] != m.light_grid_columns.size())
			return bad("light grid: %llu columns, not one per grid cell", m.light_grid_columns.size());
		for (size_t i = 0; i < m.light_grid_columns.size(); ++i)
		{
			const LightGridColumn& c = m.light_grid_columns[i];
			if (c.num_samples != 0 && uint64_t(c.first_sample) + c.num_samples > m.light_grid_samples.size())
				return bad("light grid column %llu: samples out of range", i);
		}
	}
	return true;
}

uint32_t leaf_of_point(const SqwmMap& m, const Vec3& p)
{
	// get_leaf_for_point, bsp_map_compact.rs:241-261
	uint32_t index = uint32_t(m.nodes.size() - 1);
	while (index < FIRST_LEAF_INDEX)
	{
		const BspNode& n = m.nodes[index];
		index = dot(n.plane.vec, p) > n.plane.dist ? n.children[0] : n.children[1];
	}
	return index - FIRST_LEAF_INDEX;
}

Vec3 sum_points(const std::vector<Vec3>& v, uint32_t first, uint32_t count, Vec3 sum, uint32_t& n)
{
	for (uint32_t i = 0; i < count; ++i) sum = sum + v[first + i];
	n += count;
	return sum;
}

} // namespace

bool scene_from_map(const SqwmMap& m, const SceneConfig& cfg, Scene& sc, std::string& error)
{
	if (cfg.texture_size < 16 || (cfg.texture_size & (cfg.texture_size - 1)))
	{
		error = "texture_size must be a power of two >= 16";
		return false;
	}
	if (cfg.directional_lightmaps && m.directional_lightmaps.empty())
	{
		error = "the map has no directional lightmaps";
		return false;
	}
	if (!cfg.directional_lightmaps && m.lightmaps.empty())
	{
		error = "the map has no lightmaps";
		return false;
	}
	if (cfg.sky_rooms || cfg.num_models || cfg.animated_materials)
	{
		error = "sky rooms, models and animated materials are options of generated scenes only";
		return false;
	}
	if (!check_map(m, cfg.directional_lightmaps, error)) return false;
	sc = Scene();
	sc.config = cfg;
	sc.config.num_materials = uint32_t(m.textures.size());
	sc.nodes = m.nodes;
	sc.leafs = m.leafs;
	sc.polygons = m.polygons;
	sc.portals = m.portals;
	sc.leafs_portals = m.leafs_portals;
	sc.vertices = m.vertices;
	sc.lightmaps = m.lightmaps;
	sc.directional_lightmaps = m.directional_lightmaps;
	sc.light_grid_header = m.light_grid_header;
	sc.light_grid_columns = m.light_grid_columns;
	sc.light_grid_samples = m.light_grid_samples;
	sc.lightmap_elements = cfg.directional_lightmaps ? m.directional_lightmaps.size() : m.lightmaps.size() / 3;
	sc.lightmaps_compressed.resize(m.lightmaps_compressed.size() * sizeof(CompressedColor));
	if (!sc.lightmaps_compressed.empty())
		std::memcpy(sc.lightmaps_compressed.data(), m.lightmaps_compressed.data(), sc.lightmaps_compressed.size());
	sc.directional_lightmaps_compressed.resize(m.directional_lightmaps_compressed.size() * sizeof(DirectionalLightmapElementCompressed));
	if (!sc.directional_lightmaps_compressed.empty())
		std::memcpy(sc.directional_lightmaps_compressed.data(), m.directional_lightmaps_compressed.data(),
			sc.directional_lightmaps_compressed.size());
	sc.polygon_leaf.assign(sc.polygons.size(), 0);
	for (size_t l = 0; l < sc.leafs.size(); ++l)
		for (uint32_t p = 0; p < sc.leafs[l].num_polygons; ++p) sc.polygon_leaf[sc.leafs[l].first_polygon + p] = uint32_t(l);

	// One material per texture name, its texture procedural (seeded by the name: the image files the
	// names refer to are not part of a compiled map).
	const uint32_t nm = uint32_t(m.textures.size());
	const uint32_t n_metal = uint32_t(cfg.metal_frac * nm + 0.5f);
	const uint32_t n_diel = uint32_t(cfg.dielectric_frac * nm + 0.5f);
	for (uint32_t t = 0; t < nm; ++t)
	{
		const char* name = m.textures[t].name;
		Rng trng(fnv1a(name, strnlen(name, sizeof(m.textures[t].name))) ^ cfg.seed);
		const bool metal = t < n_metal;
		const bool diel = !metal && t < n_metal + n_diel;
		make_material_texture(trng, cfg.texture_size, cfg.normal_maps, metal ? 0.35f : diel ? 0.5f : 1.0f, metal, sc);
		Material mat;
		mat.texture_size = cfg.texture_size;
		if (t < cfg.scrolling_materials)
		{
			mat.scroll_speed[0] = 24.0f + 8.0f * float(t);
			mat.scroll_speed[1] = (t & 1) ? -13.5f : 6.25f;
		}
		sc.materials.push_back(mat);
	}
	sc.basis.resize(sc.polygons.size());
	for (size_t p = 0; p < sc.polygons.size(); ++p)
		sc.basis[p] = form_plane_and_tex_coord_equation(sc.polygons[p].plane, sc.polygons[p].tex_coord_equation);

	// Camera path: from the player start (or leaf 0's centre) through leaf centres and the centres of
	// the portals between them, turning back only at dead ends.
	std::vector<Vec3> leaf_center(sc.leafs.size());
	for (size_t l = 0; l < sc.leafs.size(); ++l)
	{
		Vec3 sum = v3(0, 0, 0);
		uint32_t n = 0;
		const BspLeaf& f = sc.leafs[l];
		for (uint32_t p = 0; p < f.num_polygons; ++p)
		{
			const MapPolygon& poly = sc.polygons[f.first_polygon + p];
			sum = sum_points(sc.vertices, poly.first_vertex, poly.num_vertices, sum, n);
		}
		for (uint32_t k = 0; k < f.num_leaf_portals; ++k)
		{
			const MapPortal& portal = sc.portals[sc.leafs_portals[f.first_leaf_portal + k]];
			sum = sum_points(sc.vertices, portal.first_vertex, portal.num_vertices, sum, n);
		}
		leaf_center[l] = n ? sum * (1.0f / float(n)) : v3(0, 0, 0);
	}
	Rng rng(cfg.seed);
	std::vector<Vec3> way;
	uint32_t cur = 0;
	for (uint32_t e = 0; e < m.entities.size(); ++e)
		if (map_entity_value(m, e, "classname") == "info_player_start")
		{
			float x, y, z;
			if (std::sscanf(map_entity_value(m, e, "origin").c_str(), "%f %f %f", &x, &y, &z) == 3)
			{
				way.push_back(v3(x, y, z));
				cur = leaf_of_point(m, way.back());
			}
			break;
		}
	if (way.empty()) way.push_back(leaf_center[cur]);
	uint32_t prev = ~0u;
	for (int step = 0; step < 64; ++step)
	{
		const BspLeaf& f = sc.leafs[cur];
		std::vector<uint32_t> nb, fresh;
		for (uint32_t k = 0; k < f.num_leaf_portals; ++k)
		{
			const uint32_t pi = sc.leafs_portals[f.first_leaf_portal + k];
			const MapPortal& portal = sc.portals[pi];
			const uint32_t other = portal.leafs[0] == cur ? portal.leafs[1] : portal.leafs[0];
			if (other == cur) continue;
			nb.push_back(pi);
			if (other != prev) fresh.push_back(pi);
		}
		if (nb.empty()) break;
		const std::vector<uint32_t>& pick = fresh.empty() ? nb : fresh;
		const MapPortal& portal = sc.portals[pick[rng.below(uint32_t(pick.size()))]];
		const uint32_t next = portal.leafs[0] == cur ? portal.leafs[1] : portal.leafs[0];
		uint32_t n = 0;
		const Vec3 psum = sum_points(sc.vertices, portal.first_vertex, portal.num_vertices, v3(0, 0, 0), n);
		const Vec3 pc = psum * (1.0f / float(n));
		if (step > 0 || magnitude2(way.back() - leaf_center[cur]) > 1.0f) way.push_back(leaf_center[cur]);
		way.push_back(pc);
		prev = cur;
		cur = next;
	}
	way.push_back(leaf_center[cur]);
	camera_path_from_way(way, false, cfg, sc);
	add_dynamic_lights(cfg, rng, sc);
	return true;
}

} // namespace swhost
