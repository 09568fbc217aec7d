// Compiled-map files and lightmap compression (see sqwm.h). Load-time work, not on the timed path.
#include "sqwm.h"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace swhost
{

namespace
{

enum Lump : uint32_t
{
	LUMP_NODES = 0,
	LUMP_LEAFS,
	LUMP_POLYGONS,
	LUMP_PORTALS,
	LUMP_LEAFS_PORTALS,
	LUMP_VERTICES,
	LUMP_TEXTURES,
	LUMP_SUBMODELS,
	LUMP_SUBMODELS_BSP_NODES,
	LUMP_ENTITIES,
	LUMP_KEY_VALUE_PAIRS,
	LUMP_STRINGS_DATA,
	LUMP_LIGHTMAPS_DATA,
	LUMP_DIRECTIONAL_LIGHTMAPS_DATA,
	LUMP_LIGHT_GRID_HEADER,
	LUMP_LIGHT_GRID_COLUMNS,
	LUMP_LIGHT_GRID_SAMPLES,
};

const char* const LUMP_NAMES[] = {"nodes", "leafs", "polygons", "portals", "leafs_portals", "vertices", "textures",
	"submodels", "submodels_bsp_nodes", "entities", "key_value_pairs", "strings_data", "lightmaps_data",
	"directional_lightmaps_data", "light_grid_header", "light_grid_columns", "light_grid_samples"};

constexpr float COLOR_SCALE = 255.0f;
constexpr float VECTOR_SCALE = 127.0f;
constexpr float LIGHT_DEVIATION_SCALE = 255.0f;

struct LumpRec
{
	uint32_t offset, element_size, element_count;
};

uint32_t read_u32(const uint8_t* p)
{
	uint32_t v;
	std::memcpy(&v, p, 4);
	return v;
}

// f32::max / f32::min: a NaN operand yields the other one (as fmaxf / fminf).
float rmax(float a, float b) { return std::fmax(a, b); }
float rmin(float a, float b) { return std::fmin(a, b); }

class Reader
{
public:
	Reader(const uint8_t* d, size_t n, std::string* w) : data(d), size(n), warnings(w) {}

	bool header(std::string& error, SqwmStatus& st)
	{
		if (size < SQWM_HEADER_BYTES)
		{
			error = "can't read the map header";
			st = SQWM_NOT_A_MAP;
			return false;
		}
		if (std::memcmp(data, "SqwM", 4) != 0)
		{
			error = "not a compiled map (bad id)";
			st = SQWM_NOT_A_MAP;
			return false;
		}
		const uint32_t version = read_u32(data + 4);
		if (version != SQWM_VERSION)
		{
			char buf[96];
			std::snprintf(buf, sizeof(buf), "incompatible map version: %u, expected %u", version, SQWM_VERSION);
			error = buf;
			st = SQWM_BAD_VERSION;
			return false;
		}
		for (uint32_t i = 0; i < SQWM_MAX_LUMPS; ++i)
		{
			const uint8_t* l = data + 8 + i * 12;
			lumps[i] = {read_u32(l), read_u32(l + 4), read_u32(l + 8)};
		}
		return true;
	}

	// read_lump (bsp_map_save_load.rs:266-300)
	template <typename T>
	bool lump(uint32_t index, std::vector<T>& out, std::string& error)
	{
		out.clear();
		const LumpRec& l = lumps[index];
		if (l.element_size != sizeof(T))
		{
			wrong_size(index, l.element_size, sizeof(T));
			return true;
		}
		if (l.element_count == 0) return true;
		const uint64_t bytes = uint64_t(l.element_count) * sizeof(T);
		if (uint64_t(l.offset) + bytes > size)
		{
			error = std::string("lump ") + LUMP_NAMES[index] + " runs past the end of the file";
			return false;
		}
		out.resize(l.element_count);
		std::memcpy(out.data(), data + l.offset, size_t(bytes));
		return true;
	}

	// read_single_element_lump (:318-340)
	template <typename T>
	bool single(uint32_t index, T& out, std::string& error)
	{
		std::memset(&out, 0, sizeof(T));
		const LumpRec& l = lumps[index];
		if (l.element_size != sizeof(T))
		{
			wrong_size(index, l.element_size, sizeof(T));
			return true;
		}
		if (uint64_t(l.offset) + sizeof(T) > size)
		{
			error = std::string("lump ") + LUMP_NAMES[index] + " runs past the end of the file";
			return false;
		}
		std::memcpy(&out, data + l.offset, sizeof(T));
		return true;
	}

private:
	void wrong_size(uint32_t index, uint32_t got, size_t want)
	{
		if (!warnings) return;
		char buf[128];
		std::snprintf(buf, sizeof(buf), "lump %s: wrong element size %u, expected %zu\n", LUMP_NAMES[index], got, want);
		*warnings += buf;
	}

	const uint8_t* data;
	size_t size;
	std::string* warnings;
	LumpRec lumps[SQWM_MAX_LUMPS] = {};
};

// write_lump / write_single_element_lump (bsp_map_save_load.rs:232-264, 302-316)
template <typename T>
void put_lump(std::vector<uint8_t>& out, LumpRec* lumps, uint32_t index, const T* items, size_t count)
{
	lumps[index] = {uint32_t(out.size()), uint32_t(sizeof(T)), uint32_t(count)};
	if (count == 0) return;
	const size_t at = out.size();
	out.resize(at + count * sizeof(T));
	std::memcpy(out.data() + at, items, count * sizeof(T));
}

} // namespace

// CompressedColor::compress (lightmap_compression.rs:49-62)
CompressedColor compress_color(const float c[3])
{
	const float max_component = rmax(rmax(c[0], c[1]), c[2]);
	const float scale = rmin(rmax(std::ceil(max_component), 1.0f), 255.0f);
	const float multiplier = COLOR_SCALE / scale;
	CompressedColor r;
	for (int i = 0; i < 3; ++i) r.components[i] = uint8_t(rmin(rmax(c[i] * multiplier, 0.0f), 255.0f));
	r.scale = uint8_t(scale);
	return r;
}

// CompressedColor::decompress (:64-68)
void decompress_color(const CompressedColor& c, float out[3])
{
	const float multiplier = float(c.scale) / COLOR_SCALE;
	for (int i = 0; i < 3; ++i) out[i] = float(c.components[i]) * multiplier;
}

// CompressedVector::compress (:73-86)
CompressedVector compress_vector(const Vec3& v)
{
	const float max_component = rmax(rmax(std::fabs(v.x), std::fabs(v.y)), std::fabs(v.z));
	const float scale = rmin(rmax(std::ceil(max_component), 1.0f), 255.0f);
	const float multiplier = VECTOR_SCALE / scale;
	const float in[3] = {v.x, v.y, v.z};
	CompressedVector r;
	for (int i = 0; i < 3; ++i) r.components[i] = int8_t(rmin(rmax(in[i] * multiplier, -127.0f), 127.0f));
	r.scale = uint8_t(scale);
	return r;
}

// CompressedVector::decompress (:88-96)
Vec3 decompress_vector(const CompressedVector& v)
{
	const float multiplier = float(v.scale) / VECTOR_SCALE;
	return Vec3{float(v.components[0]) * multiplier, float(v.components[1]) * multiplier, float(v.components[2]) * multiplier};
}

// DirectionalLightmapElementCompressed::compress (:101-112)
DirectionalLightmapElementCompressed compress_directional(const SwDirectionalLightmapElement& e)
{
	DirectionalLightmapElementCompressed r;
	r.ambient_light = compress_color(e.ambient_light);
	r.light_direction_vector_scaled = compress_vector(
		Vec3{e.light_direction_vector_scaled[0], e.light_direction_vector_scaled[1], e.light_direction_vector_scaled[2]});
	r.directional_light_deviation = uint8_t(rmin(rmax(e.directional_light_deviation * LIGHT_DEVIATION_SCALE, 0.0f), 255.0f));
	r.directional_light_color = compress_color(e.directional_light_color);
	return r;
}

// DirectionalLightmapElementCompressed::decompress (:114-130), with its fix-up of a direction that
// quantised to zero.
SwDirectionalLightmapElement decompress_directional(const DirectionalLightmapElementCompressed& e)
{
	SwDirectionalLightmapElement r;
	decompress_color(e.ambient_light, r.ambient_light);
	const Vec3 d = decompress_vector(e.light_direction_vector_scaled);
	r.light_direction_vector_scaled[0] = d.x;
	r.light_direction_vector_scaled[1] = d.y;
	r.light_direction_vector_scaled[2] = d.z;
	r.directional_light_deviation = float(e.directional_light_deviation) / LIGHT_DEVIATION_SCALE;
	decompress_color(e.directional_light_color, r.directional_light_color);
	if (d.x * d.x + d.y * d.y + d.z * d.z <= 0.0f)
	{
		r.light_direction_vector_scaled[0] = 0.0f;
		r.light_direction_vector_scaled[1] = 0.0f;
		r.light_direction_vector_scaled[2] = 1.0f / 1024.0f;
	}
	return r;
}

// LightGridElementCompressed::compress / decompress (:133-149)
LightGridElementCompressed compress_light_grid(const LightGridElement& e)
{
	LightGridElementCompressed r;
	for (int s = 0; s < 6; ++s) r.light_cube[s] = compress_color(e.light_cube[s]);
	r.light_direction_vector_scaled = compress_vector(e.light_direction_vector_scaled);
	r.directional_light_color = compress_color(e.directional_light_color);
	return r;
}

LightGridElement decompress_light_grid(const LightGridElementCompressed& e)
{
	LightGridElement r;
	for (int s = 0; s < 6; ++s) decompress_color(e.light_cube[s], r.light_cube[s]);
	r.light_direction_vector_scaled = decompress_vector(e.light_direction_vector_scaled);
	decompress_color(e.directional_light_color, r.directional_light_color);
	return r;
}

// load_map (bsp_map_save_load.rs:162-226), from a file image
SqwmStatus sqwm_parse(const uint8_t* data, size_t size, SqwmMap& m, std::string& error, std::string* warnings)
{
	m = SqwmMap();
	Reader rd(data, size, warnings);
	SqwmStatus st = SQWM_OK;
	if (!rd.header(error, st)) return st;
	std::vector<LightGridElementCompressed> grid;
	const bool ok = rd.lump(LUMP_NODES, m.nodes, error) && rd.lump(LUMP_LEAFS, m.leafs, error) &&
		rd.lump(LUMP_POLYGONS, m.polygons, error) && rd.lump(LUMP_PORTALS, m.portals, error) &&
		rd.lump(LUMP_LEAFS_PORTALS, m.leafs_portals, error) && rd.lump(LUMP_VERTICES, m.vertices, error) &&
		rd.lump(LUMP_TEXTURES, m.textures, error) && rd.lump(LUMP_SUBMODELS, m.submodels, error) &&
		rd.lump(LUMP_SUBMODELS_BSP_NODES, m.submodels_bsp_nodes, error) && rd.lump(LUMP_ENTITIES, m.entities, error) &&
		rd.lump(LUMP_KEY_VALUE_PAIRS, m.key_value_pairs, error) && rd.lump(LUMP_STRINGS_DATA, m.strings_data, error) &&
		rd.lump(LUMP_LIGHTMAPS_DATA, m.lightmaps_compressed, error) &&
		rd.lump(LUMP_DIRECTIONAL_LIGHTMAPS_DATA, m.directional_lightmaps_compressed, error) &&
		rd.single(LUMP_LIGHT_GRID_HEADER, m.light_grid_header, error) &&
		rd.lump(LUMP_LIGHT_GRID_COLUMNS, m.light_grid_columns, error) && rd.lump(LUMP_LIGHT_GRID_SAMPLES, grid, error);
	if (!ok)
	{
		m = SqwmMap();
		return SQWM_TRUNCATED;
	}
	m.lightmaps.resize(m.lightmaps_compressed.size() * 3);
	for (size_t i = 0; i < m.lightmaps_compressed.size(); ++i) decompress_color(m.lightmaps_compressed[i], &m.lightmaps[i * 3]);
	m.directional_lightmaps.resize(m.directional_lightmaps_compressed.size());
	for (size_t i = 0; i < m.directional_lightmaps_compressed.size(); ++i)
		m.directional_lightmaps[i] = decompress_directional(m.directional_lightmaps_compressed[i]);
	m.light_grid_samples.resize(grid.size());
	for (size_t i = 0; i < grid.size(); ++i) m.light_grid_samples[i] = decompress_light_grid(grid[i]);
	return SQWM_OK;
}

// save_map (bsp_map_save_load.rs:24-160), into a file image
void sqwm_serialize(const SqwmMap& m, std::vector<uint8_t>& out)
{
	out.assign(SQWM_HEADER_BYTES, 0);
	LumpRec lumps[SQWM_MAX_LUMPS] = {};
	put_lump(out, lumps, LUMP_NODES, m.nodes.data(), m.nodes.size());
	put_lump(out, lumps, LUMP_LEAFS, m.leafs.data(), m.leafs.size());
	put_lump(out, lumps, LUMP_POLYGONS, m.polygons.data(), m.polygons.size());
	put_lump(out, lumps, LUMP_PORTALS, m.portals.data(), m.portals.size());
	put_lump(out, lumps, LUMP_LEAFS_PORTALS, m.leafs_portals.data(), m.leafs_portals.size());
	put_lump(out, lumps, LUMP_VERTICES, m.vertices.data(), m.vertices.size());
	put_lump(out, lumps, LUMP_TEXTURES, m.textures.data(), m.textures.size());
	put_lump(out, lumps, LUMP_SUBMODELS, m.submodels.data(), m.submodels.size());
	put_lump(out, lumps, LUMP_SUBMODELS_BSP_NODES, m.submodels_bsp_nodes.data(), m.submodels_bsp_nodes.size());
	put_lump(out, lumps, LUMP_ENTITIES, m.entities.data(), m.entities.size());
	put_lump(out, lumps, LUMP_KEY_VALUE_PAIRS, m.key_value_pairs.data(), m.key_value_pairs.size());
	put_lump(out, lumps, LUMP_STRINGS_DATA, m.strings_data.data(), m.strings_data.size());
	std::vector<CompressedColor> lm(m.lightmaps.size() / 3);
	for (size_t i = 0; i < lm.size(); ++i) lm[i] = compress_color(&m.lightmaps[i * 3]);
	put_lump(out, lumps, LUMP_LIGHTMAPS_DATA, lm.data(), lm.size());
	std::vector<DirectionalLightmapElementCompressed> dlm(m.directional_lightmaps.size());
	for (size_t i = 0; i < dlm.size(); ++i) dlm[i] = compress_directional(m.directional_lightmaps[i]);
	put_lump(out, lumps, LUMP_DIRECTIONAL_LIGHTMAPS_DATA, dlm.data(), dlm.size());
	put_lump(out, lumps, LUMP_LIGHT_GRID_HEADER, &m.light_grid_header, 1);
	put_lump(out, lumps, LUMP_LIGHT_GRID_COLUMNS, m.light_grid_columns.data(), m.light_grid_columns.size());
	std::vector<LightGridElementCompressed> grid(m.light_grid_samples.size());
	for (size_t i = 0; i < grid.size(); ++i) grid[i] = compress_light_grid(m.light_grid_samples[i]);
	put_lump(out, lumps, LUMP_LIGHT_GRID_SAMPLES, grid.data(), grid.size());
	std::memcpy(out.data(), "SqwM", 4);
	const uint32_t version = SQWM_VERSION;
	std::memcpy(out.data() + 4, &version, 4);
	std::memcpy(out.data() + 8, lumps, sizeof(lumps));
}

std::string map_entity_value(const SqwmMap& m, uint32_t entity, const char* key)
{
	if (entity >= m.entities.size()) return std::string();
	const MapEntity& e = m.entities[entity];
	auto str = [&](const MapStringRef& s) -> std::string {
		if (size_t(s.offset) + s.size > m.strings_data.size()) return std::string();
		return std::string(reinterpret_cast<const char*>(m.strings_data.data()) + s.offset, s.size);
	};
	for (uint64_t k = e.first_key_value_pair; k < uint64_t(e.first_key_value_pair) + e.num_key_value_pairs; ++k)
	{
		if (k >= m.key_value_pairs.size()) break;
		if (str(m.key_value_pairs[k].key) == key) return str(m.key_value_pairs[k].value);
	}
	return std::string();
}

void map_from_scene(const Scene& sc, SqwmMap& m)
{
	m = SqwmMap();
	m.nodes = sc.nodes;
	m.leafs = sc.leafs;
	m.polygons = sc.polygons;
	m.portals = sc.portals;
	m.leafs_portals = sc.leafs_portals;
	m.vertices = sc.vertices;
	m.textures.resize(sc.materials.size());
	for (size_t i = 0; i < sc.materials.size(); ++i)
	{
		std::memset(m.textures[i].name, 0, sizeof(m.textures[i].name));
		std::snprintf(m.textures[i].name, sizeof(m.textures[i].name), "generated/material_%zu", i);
	}
	m.lightmaps = sc.lightmaps;
	m.directional_lightmaps = sc.directional_lightmaps;
	m.light_grid_header = sc.light_grid_header;
	m.light_grid_columns = sc.light_grid_columns;
	m.light_grid_samples = sc.light_grid_samples;
	// Entities (deduplicated strings, StringRef offsets and sizes in u16): worldspawn and the player start.
	auto add_string = [&](const std::string& s) {
		for (size_t at = 0; at + s.size() <= m.strings_data.size(); ++at)
			if (std::memcmp(m.strings_data.data() + at, s.data(), s.size()) == 0) return MapStringRef{uint16_t(at), uint16_t(s.size())};
		const MapStringRef r{uint16_t(m.strings_data.size()), uint16_t(s.size())};
		m.strings_data.insert(m.strings_data.end(), s.begin(), s.end());
		return r;
	};
	auto add_entity = [&](const std::vector<std::pair<std::string, std::string>>& kv) {
		MapEntity e{uint32_t(m.key_value_pairs.size()), uint32_t(kv.size()), ~0u};
		for (const auto& p : kv) m.key_value_pairs.push_back(MapKeyValuePair{add_string(p.first), add_string(p.second)});
		m.entities.push_back(e);
	};
	add_entity({{"classname", "worldspawn"}});
	if (!sc.camera_path.empty())
	{
		const Vec3& p = sc.camera_path[0].position;
		char buf[96];
		std::snprintf(buf, sizeof(buf), "%.9g %.9g %.9g", double(p.x), double(p.y), double(p.z));
		char yaw[32];
		std::snprintf(yaw, sizeof(yaw), "%.9g", double(sc.camera_path[0].azimuth * 57.29577951308232f));
		add_entity({{"classname", "info_player_start"}, {"origin", buf}, {"angle", yaw}});
	}
}

} // namespace swhost
