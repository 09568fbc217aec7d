// Compiled-map files (.sqwm, format version 11) and the lossy lightmap compression they store.
//
// File format (src/common/bsp_map_save_load.rs:20-300): a 392-byte header - the id "SqwM", the version
// and 32 lumps of {offset, element_size, element_count} (u32 each) - followed by each lump's elements as
// the raw little-endian bytes of the reference's #[repr(C)] structs, in lump order. Lumps 12, 13 and 16
// (simple lightmaps, directional lightmaps, light-grid samples) hold compressed elements
// (src/common/lightmap_compression.rs): a colour as three u8 components and a u8 scale, a vector as three
// i8 components and a u8 scale.
//
// Reading follows load_map (bsp_map_save_load.rs:162-226): a short header, a wrong id or a wrong version
// is "not a map"; a lump whose element size differs from the struct's reads as empty (the light-grid
// header as zeroes), a lump that runs past the end of the data is an error. Writing follows save_map
// (:24-160): lumps back to back after the header, lightmaps compressed from their f32 values.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "scene.h"

namespace swhost
{

constexpr uint32_t SQWM_VERSION = 11;
constexpr uint32_t SQWM_MAX_LUMPS = 32;
constexpr size_t SQWM_HEADER_BYTES = 8 + SQWM_MAX_LUMPS * 12;

// CompressedColor (lightmap_compression.rs:25-34): value = component * scale / 255.
struct CompressedColor
{
	uint8_t components[3];
	uint8_t scale;
};
// CompressedVector (:36-45): value = component * scale / 127.
struct CompressedVector
{
	int8_t components[3];
	uint8_t scale;
};
// DirectionalLightmapElementCompressed (:5-12): 13 bytes, no padding.
struct DirectionalLightmapElementCompressed
{
	CompressedColor ambient_light;
	CompressedVector light_direction_vector_scaled;
	uint8_t directional_light_deviation;
	CompressedColor directional_light_color;
};
// LightGridElement (scene.h) in its compressed form (lightmap_compression.rs:14-20).
struct LightGridElementCompressed
{
	CompressedColor light_cube[6];
	CompressedVector light_direction_vector_scaled;
	CompressedColor directional_light_color;
};
struct MapSubmodel
{
	uint32_t root_node, first_polygon, num_polygons;
};
struct MapSubmodelBspNode
{
	Plane plane;
	uint32_t first_polygon, num_polygons;
	uint32_t children[2];
};
struct MapEntity
{
	uint32_t first_key_value_pair, num_key_value_pairs, submodel_index;
};
struct MapStringRef
{
	uint16_t offset, size;
};
struct MapKeyValuePair
{
	MapStringRef key, value;
};
// Texture name: UTF-8 bytes, the rest of the 64 filled with zeroes (bsp_map_compact.rs:133-135).
struct MapTextureName
{
	char name[64];
};

static_assert(sizeof(CompressedColor) == 4 && sizeof(CompressedVector) == 4, "compressed sizes");
static_assert(sizeof(DirectionalLightmapElementCompressed) == 13, "compressed directional element size");
static_assert(sizeof(LightGridElementCompressed) == 32 && sizeof(LightGridElement) == 96, "light grid sizes");
static_assert(sizeof(BspNode) == 24 && sizeof(BspLeaf) == 16 && sizeof(MapPolygon) == 80 && sizeof(MapPortal) == 32,
	"map struct sizes");
static_assert(sizeof(MapSubmodelBspNode) == 32 && sizeof(LightGridHeader) == 36, "map struct sizes");

// BSPMap (bsp_map_compact.rs:6-34) with its lightmaps decompressed, plus the compressed lightmap lumps
// exactly as the file holds them (for decompression on the GPU).
struct SqwmMap
{
	std::vector<BspNode> nodes;
	std::vector<BspLeaf> leafs;
	std::vector<MapPolygon> polygons;
	std::vector<MapPortal> portals;
	std::vector<uint32_t> leafs_portals;
	std::vector<Vec3> vertices;
	std::vector<MapTextureName> textures;
	std::vector<MapSubmodel> submodels;
	std::vector<MapSubmodelBspNode> submodels_bsp_nodes;
	std::vector<MapEntity> entities;
	std::vector<MapKeyValuePair> key_value_pairs;
	std::vector<uint8_t> strings_data;
	std::vector<float> lightmaps; // LightmapElement = [f32; 3], 3 floats per element
	std::vector<SwDirectionalLightmapElement> directional_lightmaps;
	LightGridHeader light_grid_header{};
	std::vector<LightGridColumn> light_grid_columns;
	std::vector<LightGridElement> light_grid_samples;

	std::vector<CompressedColor> lightmaps_compressed;
	std::vector<DirectionalLightmapElementCompressed> directional_lightmaps_compressed;
};

// lightmap_compression.rs:48-146
CompressedColor compress_color(const float c[3]);
void decompress_color(const CompressedColor& c, float out[3]);
CompressedVector compress_vector(const Vec3& v);
Vec3 decompress_vector(const CompressedVector& v);
DirectionalLightmapElementCompressed compress_directional(const SwDirectionalLightmapElement& e);
SwDirectionalLightmapElement decompress_directional(const DirectionalLightmapElementCompressed& e);
LightGridElementCompressed compress_light_grid(const LightGridElement& e);
LightGridElement decompress_light_grid(const LightGridElementCompressed& e);

enum SqwmStatus
{
	SQWM_OK = 0,
	SQWM_NOT_A_MAP = 1,   // short header or wrong id
	SQWM_BAD_VERSION = 2, // version other than 11
	SQWM_TRUNCATED = 3,   // a lump past the end of the data
};

// Parses a whole file image. `warnings` (optional) receives one line per lump read as empty because of
// a wrong element size.
SqwmStatus sqwm_parse(const uint8_t* data, size_t size, SqwmMap& out, std::string& error, std::string* warnings = nullptr);
// Serialises `map` (lightmaps and light-grid samples compressed from their f32 values).
void sqwm_serialize(const SqwmMap& map, std::vector<uint8_t>& out);

// The value of key `key` of entity `entity`, or "" (get_map_string, bsp_map_compact.rs:190-193).
std::string map_entity_value(const SqwmMap& map, uint32_t entity, const char* key);

// A scene's map data as a compiled map: geometry as is, one texture name per material, lightmaps, a
// worldspawn entity and an info_player_start at the camera path's first position.
void map_from_scene(const Scene& scene, SqwmMap& out);

// A renderable scene from a compiled map (scene.cpp): geometry and lightmaps from the map (after
// checking every index and range the renderer follows), one procedural material per texture name, a
// camera path through the leafs from the info_player_start entity (or leaf 0), and the config's dynamic
// lights along it. Keeps the compressed lightmaps for upload.
bool scene_from_map(const SqwmMap& map, const SceneConfig& cfg, Scene& out, std::string& error);

} // namespace swhost
